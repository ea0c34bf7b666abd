// Shared device helpers for the spinchem GB300 kernels.
//
// Complex numbers are double2 (x = re, y = im), the layout of complex(dp).
// The path is FP64-issue bound on GB300 (about 2 FP64 FMA lanes per clock per
// SM), so helpers are written to the minimum number of FP64 instructions:
// a complex multiply-accumulate is exactly 4 DFMA.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define SPC_WARPS 8           // warps per CTA of the row-pass kernels
#define SPC_LANES 32          // sample columns per CTA tile (one per lane)
#define SPC_MAX_M 64          // largest Krylov dimension supported

__device__ __forceinline__ double2 cz() { return make_double2(0.0, 0.0); }

// acc + a*b
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}
// acc + conj(a)*b
__device__ __forceinline__ double2 cjfma(double2 a, double2 b, double2 acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
  return acc;
}
// acc - a*b
__device__ __forceinline__ double2 cfms(double2 a, double2 b, double2 acc) {
  acc.x = fma(-a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(-a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
  return acc;
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) {
  return make_double2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ double2 cscale(double s, double2 a) {
  return make_double2(s * a.x, s * a.y);
}
// Smith's complex division a / d
__device__ __forceinline__ double2 cdiv(double2 a, double2 d) {
  if (fabs(d.x) >= fabs(d.y)) {
    double r = d.y / d.x, den = d.x + d.y * r;
    return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  }
  double r = d.x / d.y, den = d.x * r + d.y;
  return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}

__device__ __forceinline__ double2 shfl_xor2(double2 v, int mask) {
  v.x = __shfl_xor_sync(0xffffffffu, v.x, mask);
  v.y = __shfl_xor_sync(0xffffffffu, v.y, mask);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
