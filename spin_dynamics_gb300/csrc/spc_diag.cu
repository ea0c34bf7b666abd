// Diagnostics: per-kernel-class timing with CUDA events on the launching
// stream, and an FP64 FMA throughput probe (the roof of this FP64-bound path;
// the pool's measured-peaks file carries only HBM and bf16 tensor figures).
#include <vector>

#include "spc_common.cuh"
#include "spc_internal.h"

namespace spc {

static const char* kKindNames[PROF_KINDS] = {"spmm",   "mgs_dot",    "mgs_axpy_dot", "mgs_axpy_norm",
                                             "scale",  "expm",       "projectors",   "proj_reduce",
                                             "dtloop", "psi_update", "setup",        "contract",
                                             "costate", "sample_cta"};

const char* prof_kind_name(int k) { return (k >= 0 && k < PROF_KINDS) ? kKindNames[k] : ""; }

Prof::~Prof() {
  for (cudaEvent_t e : pool) cudaEventDestroy(e);
}

void Prof::reset() {
  for (int k = 0; k < PROF_KINDS; ++k) {
    ms[k] = 0.0;
    flops[k] = 0.0;
    bytes[k] = 0.0;
    launches[k] = 0;
  }
  pend.clear();
  used = 0;
}

int Prof::begin(cudaStream_t st) {
  if (!on) return -1;
  while ((int)pool.size() < used + 2) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return -1;
    pool.push_back(e);
  }
  int i = used;
  used += 2;
  cudaEventRecord(pool[i], st);
  return i;
}

void Prof::end(cudaStream_t st, int idx, int kind, double f, double b) {
  if (!on || idx < 0) return;
  cudaEventRecord(pool[idx + 1], st);
  pend.push_back({kind, f, b, idx});
}

void Prof::collect() {
  if (!on) return;
  for (const Pending& p : pend) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, pool[p.ev], pool[p.ev + 1]) == cudaSuccess) {
      ms[p.kind] += t;
      flops[p.kind] += p.flops;
      bytes[p.kind] += p.bytes;
      launches[p.kind] += 1;
    }
  }
  pend.clear();
  used = 0;
}

// Independent DFMA chains: 8 accumulators per thread, `iters` rounds.
__global__ void k_fp64_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-9, x2 = x0 + 2e-9, x3 = x0 + 3e-9;
  double x4 = x0 + 4e-9, x5 = x0 + 5e-9, x6 = x0 + 6e-9, x7 = x0 + 7e-9;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  const double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 1234.5) out[blockIdx.x] = s;  // keeps the chains live
}

}  // namespace spc

extern "C" {

int spc_set_profiling(spc_handle* hh, int enable);
int spc_get_profile(const spc_handle* hh, int kind, double* ms, int64_t* launches, double* flops,
                    double* bytes);
const char* spc_kernel_kind_name(int kind);
int spc_fp64_peak(int device, double* tflops);

const char* spc_kernel_kind_name(int kind) { return spc::prof_kind_name(kind); }

int spc_fp64_peak(int device, double* tflops) {
  if (!tflops) return spc::set_error(SPC_ERR_ARG, "null output");
  if (cudaSetDevice(device) != cudaSuccess) return spc::set_error(SPC_ERR_CUDA, "cudaSetDevice failed");
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * sms * 64) != cudaSuccess)
    return spc::set_error(SPC_ERR_ALLOC, "cudaMalloc failed");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  spc::k_fp64_probe<<<blocks, threads>>>(d, 64, 1.0000001, 1e-12);  // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    spc::k_fp64_probe<<<blocks, threads>>>(d, iters, 1.0000001, 1e-12);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    if (t < best) best = t;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (err != cudaSuccess) return spc::set_error(SPC_ERR_CUDA, "probe failed: %s", cudaGetErrorString(err));
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return SPC_OK;
}

}  // extern "C"
