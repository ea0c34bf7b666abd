// Batched trace-sampling propagation on the device.
//
// Restates trace_sampling_para (src/qm_dynamics.f90:257-384) for all M
// samples at once. Samples are the columns of every vector array, stored
// row-major with the sample index fastest: X[row * ld + w]. Each round, every
// sample that has not reached t_end builds a new Krylov basis (the reference
// rebuilds each sample independently; the build does not depend on t, so
// batching the builds of all unfinished samples is the same computation),
// then runs its own dt loop until its own rebuild test fires. Finished
// samples leave the batch (column map `map[w] -> sample`).
//
// Per round:
//   norm/scale passes      c = ||psi|| e1, Q0 = psi/||psi||      (get_krylov :445-449)
//   m x [ SpMM p = H Q_i ; MGS dot/axpy passes ; scale ]           (:451-465)
//   Pade-6 expm of -i dt A per sample, one CTA each               (matrix_exponential.f90)
//   Krylov projectors as Hermitian Grams per sample               (convert_to_krylov :469-498)
//   dt loop per sample, one warp each                             (:351-364)
//   psi = Q c                                                      (:365)
//
// All reductions are two-level and in a fixed order (per-CTA partials, then
// the last CTA of each sample tile sums them), so results do not depend on
// scheduling.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "spc_common.cuh"
#include "spc_internal.h"

namespace spc {

enum PassKind { PASS_NORM_GATHER = 0, PASS_DOT = 1, PASS_AXPY_DOT = 2, PASS_AXPY_NORM = 3 };

struct PassArgs {
  int64_t N;
  int ld, Ma, rpb, m, col_i, row_j;
  int lanczos;        // AXPY_NORM also seeds the next Lanczos coefficient
  const double2* X;   // NORM_GATHER: psi (ldp columns, gathered through map); DOT: Q_0
  double2* P;         // Arnoldi work vector
  const double2* Qj;  // AXPY_*: the basis vector removed from P
  const double2* Qn;  // AXPY_DOT: the next basis vector to project on
  const int* map;
  int ldp;
  double2* coef;      // current MGS coefficient per sample
  double* rbeta;      // 1/norm per sample
  double2* Ahess;     // Hessenberg matrices, m x m column-major per sample
  double2* cvec;      // Krylov coordinates per sample
  double2* partial;   // [row blocks][ld]
  unsigned* counters; // per sample tile
};

template <int KIND>
__device__ __forceinline__ void pass_finalize(const PassArgs& a, int w, double2 tot) {
  const size_t mm = (size_t)a.m * a.m;
  if (KIND == PASS_NORM_GATHER) {
    double b = sqrt(tot.x);
    double2* c = a.cvec + (size_t)w * a.m;
    c[0] = make_double2(b, 0.0);
    for (int j = 1; j < a.m; ++j) c[j] = cz();
    a.rbeta[w] = b > 0.0 ? 1.0 / b : 0.0;
  } else if (KIND == PASS_DOT || KIND == PASS_AXPY_DOT) {
    a.coef[w] = tot;
    a.Ahess[(size_t)w * mm + a.row_j + (size_t)a.col_i * a.m] = tot;
  } else {  // PASS_AXPY_NORM: A(i+1, i) = ||p||, and 1/||p|| for the scale
    double b = sqrt(tot.x);
    a.Ahess[(size_t)w * mm + a.row_j + (size_t)a.col_i * a.m] = make_double2(b, 0.0);
    // exact breakdown (p == 0): the next basis vector is 0 instead of 0/0
    a.rbeta[w] = b > 0.0 ? 1.0 / b : 0.0;
    if (a.lanczos) {
      // Hermitian tridiagonal: A(i, i+1) = beta_i, the coefficient of Q_i
      // in the next step's three-term recurrence
      a.Ahess[(size_t)w * mm + a.col_i + (size_t)a.row_j * a.m] = make_double2(b, 0.0);
      a.coef[w] = make_double2(b, 0.0);
    }
  }
}

// One pass over all rows for a tile of 32 samples: element update + per-sample
// reduction. Grid (sample tiles, row blocks), block (32, SPC_WARPS).
template <int KIND>
__global__ void __launch_bounds__(256) k_rowpass(PassArgs a) {
  __shared__ double2 red[SPC_WARPS][SPC_LANES];
  __shared__ bool am_last;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int w = blockIdx.x * SPC_LANES + tx;
  const bool act = w < a.Ma;
  const int64_t r0 = (int64_t)blockIdx.y * a.rpb;
  const int64_t r1 = min(a.N, r0 + a.rpb);
  double2 acc = cz();
  if (act) {
    if (KIND == PASS_NORM_GATHER) {
      const int src = a.map[w];
      for (int64_t r = r0 + ty; r < r1; r += SPC_WARPS) {
        double2 x = a.X[(size_t)r * a.ldp + src];
        acc.x = fma(x.x, x.x, acc.x);
        acc.x = fma(x.y, x.y, acc.x);
      }
    } else if (KIND == PASS_DOT) {
      for (int64_t r = r0 + ty; r < r1; r += SPC_WARPS) {
        size_t o = (size_t)r * a.ld + w;
        acc = cjfma(a.X[o], a.P[o], acc);
      }
    } else {
      const double2 cf = a.coef[w];
      for (int64_t r = r0 + ty; r < r1; r += SPC_WARPS) {
        size_t o = (size_t)r * a.ld + w;
        double2 p = cfms(cf, a.Qj[o], a.P[o]);
        a.P[o] = p;
        if (KIND == PASS_AXPY_DOT) {
          acc = cjfma(a.Qn[o], p, acc);
        } else {
          acc.x = fma(p.x, p.x, acc.x);
          acc.x = fma(p.y, p.y, acc.x);
        }
      }
    }
  }
  red[ty][tx] = acc;
  __syncthreads();
  if (ty == 0) {
    double2 s = red[0][tx];
#pragma unroll
    for (int y = 1; y < SPC_WARPS; ++y) s = cadd(s, red[y][tx]);
    a.partial[(size_t)blockIdx.y * a.ld + w] = s;
  }
  __threadfence();
  __syncthreads();
  if (tx == 0 && ty == 0) {
    unsigned t = atomicAdd(&a.counters[blockIdx.x], 1u);
    am_last = (t == gridDim.y - 1);
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  double2 s = cz();
  for (int b = ty; b < (int)gridDim.y; b += SPC_WARPS)
    s = cadd(s, __ldcg(&a.partial[(size_t)b * a.ld + w]));
  red[ty][tx] = s;
  __syncthreads();
  if (ty == 0) {
    double2 tot = red[0][tx];
#pragma unroll
    for (int y = 1; y < SPC_WARPS; ++y) tot = cadd(tot, red[y][tx]);
    if (act) pass_finalize<KIND>(a, w, tot);
    if (tx == 0) a.counters[blockIdx.x] = 0u;
  }
}

// Q_{i+1} = P / ||P||  (or Q_0 = psi[:, map] / ||psi|| when gather != 0)
__global__ void __launch_bounds__(256)
    k_scale(int64_t N, int ld, int Ma, int rpb, const double2* __restrict__ src, int ldp,
            const int* __restrict__ map, int gather, const double* __restrict__ rbeta,
            double2* __restrict__ dst) {
  const int w = blockIdx.x * SPC_LANES + threadIdx.x;
  if (w >= Ma) return;
  const double rb = rbeta[w];
  const int col = gather ? map[w] : w;
  const int lds = gather ? ldp : ld;
  const int64_t r0 = (int64_t)blockIdx.y * rpb;
  const int64_t r1 = min(N, r0 + rpb);
  for (int64_t r = r0 + threadIdx.y; r < r1; r += SPC_WARPS) {
    double2 x = src[(size_t)r * lds + col];
    dst[(size_t)r * ld + w] = make_double2(x.x * rb, x.y * rb);
  }
}

// Y = H X for a tile of 32 sample columns; one warp per row at a time, the
// row's (col, val) entries broadcast to all lanes. Rows are stored in the
// execution order of k_split_rows: entries with a nonzero imaginary part
// first (4 DFMA each), then real ones from split[r] on (2 DFMA each).
__global__ void __launch_bounds__(256)
    k_spmm(int64_t N, int ld, int Ma, int rpb, const int* __restrict__ rowptr,
           const int* __restrict__ split, const int* __restrict__ col,
           const double2* __restrict__ val, const double2* __restrict__ X,
           double2* __restrict__ Y) {
  const int w = blockIdx.x * SPC_LANES + threadIdx.x;
  const bool act = w < Ma;
  (void)rpb;
  // rows interleaved over the CTAs of a sample tile: balanced row lengths,
  // and all CTAs sweep X together (L2 reuse of the Kronecker neighbours)
  const int64_t stride = (int64_t)gridDim.y * SPC_WARPS;
  for (int64_t r = (int64_t)blockIdx.y * SPC_WARPS + threadIdx.y; r < N; r += stride) {
    const int k0 = __ldg(rowptr + r), ks = __ldg(split + r), k1 = __ldg(rowptr + r + 1);
    double2 a0 = cz(), a1 = cz();
    int k = k0;
    for (; k + 1 < ks; k += 2) {
      const int c0 = __ldg(col + k), c1 = __ldg(col + k + 1);
      const double2 v0 = __ldg(val + k), v1 = __ldg(val + k + 1);
      if (act) {
        const double2 x0 = X[(size_t)c0 * ld + w];
        const double2 x1 = X[(size_t)c1 * ld + w];
        a0 = cfma(v0, x0, a0);
        a1 = cfma(v1, x1, a1);
      }
    }
    if (k < ks) {
      const int c0 = __ldg(col + k);
      const double2 v0 = __ldg(val + k);
      if (act) a0 = cfma(v0, X[(size_t)c0 * ld + w], a0);
      k++;
    }
    for (; k + 1 < k1; k += 2) {
      const int c0 = __ldg(col + k), c1 = __ldg(col + k + 1);
      const double v0 = __ldg(&val[k].x), v1 = __ldg(&val[k + 1].x);
      if (act) {
        const double2 x0 = X[(size_t)c0 * ld + w];
        const double2 x1 = X[(size_t)c1 * ld + w];
        a0.x = fma(v0, x0.x, a0.x);
        a0.y = fma(v0, x0.y, a0.y);
        a1.x = fma(v1, x1.x, a1.x);
        a1.y = fma(v1, x1.y, a1.y);
      }
    }
    if (k < k1) {
      const int c0 = __ldg(col + k);
      const double v0 = __ldg(&val[k].x);
      if (act) {
        const double2 x0 = X[(size_t)c0 * ld + w];
        a0.x = fma(v0, x0.x, a0.x);
        a0.y = fma(v0, x0.y, a0.y);
      }
    }
    if (act) Y[(size_t)r * ld + w] = cadd(a0, a1);
  }
}

// Execution copy of a CSR for k_spmm: each row's entries reordered so that
// those with a nonzero imaginary part come first (original order kept within
// each class); split[r] is the index of the row's first real entry.
__global__ void k_split_rows(int64_t N, const int* __restrict__ rowptr, const int* __restrict__ col,
                             const double2* __restrict__ val, int* __restrict__ xcol,
                             double2* __restrict__ xval, int* __restrict__ split) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= N) return;
  const int k0 = rowptr[r], k1 = rowptr[r + 1];
  int o = k0;
  for (int k = k0; k < k1; ++k)
    if (val[k].y != 0.0) {
      xcol[o] = col[k];
      xval[o] = val[k];
      o++;
    }
  split[r] = o;
  for (int k = k0; k < k1; ++k)
    if (val[k].y == 0.0) {
      xcol[o] = col[k];
      xval[o] = val[k];
      o++;
    }
}

int prepare_spmm_rows(Handle* h) {
  const int64_t N = h->n, nnz = h->nnz;
  if (h->ensure(h->xcol, sizeof(int) * (nnz > 0 ? nnz : 1)) ||
      h->ensure(h->xval, sizeof(double2) * (nnz > 0 ? nnz : 1)) || h->ensure(h->xsplit, sizeof(int) * N))
    return SPC_ERR_ALLOC;
  k_split_rows<<<(int)((N + 255) / 256), 256, 0, h->stream>>>(
      N, h->d_rowptr, h->d_col, h->d_val, (int*)h->xcol.p, (double2*)h->xval.p, (int*)h->xsplit.p);
  h->count_launch();
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess)
    return set_error(SPC_ERR_CUDA, "row split of the Hamiltonian failed: %s", cudaGetErrorString(e));
  return SPC_OK;
}

// ---------------------------------------------------------------------------
// expm (src/matrix_exponential.f90:14-87) of -i dt A, one CTA per sample.
// Column-major m x m matrices in shared memory.
__device__ void smem_matmul(int m, const double2* A, const double2* B, double2* C) {
  const int mm = m * m;
  for (int idx = threadIdx.x; idx < mm; idx += blockDim.x) {
    const int i = idx % m, j = idx / m;
    double2 acc = cz();
    for (int k = 0; k < m; ++k) acc = cfma(A[i + k * m], B[k + j * m], acc);
    C[idx] = acc;
  }
}

__global__ void __launch_bounds__(128)
    k_expm(int m, int Ma, const double2* __restrict__ Ahess, double2* __restrict__ Aexp, double dt,
           int* __restrict__ err) {
  extern __shared__ double2 sm[];
  __shared__ double rowsum[SPC_MAX_M];
  __shared__ int piv[SPC_MAX_M];
  __shared__ int s_sh, p_sh;
  const int mm = m * m;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int w = blockIdx.x;
  if (w >= Ma) return;
  double2* A2 = sm;
  double2* X = A2 + mm;
  double2* E = X + mm;
  double2* D = E + mm;
  double2* T = D + mm;
  const double2* Ain = Ahess + (size_t)w * mm;
  // (0,-1)*dt*A
  for (int i = tid; i < mm; i += nt) {
    double2 a = Ain[i];
    A2[i] = make_double2(dt * a.y, -dt * a.x);
  }
  __syncthreads();
  // L-infinity norm (mat_norm_linf :89-104)
  for (int i = tid; i < m; i += nt) {
    double s = 0.0;
    for (int j = 0; j < m; ++j) s += hypot(A2[i + j * m].x, A2[i + j * m].y);
    rowsum[i] = s;
  }
  __syncthreads();
  if (tid == 0) {
    double an = 0.0;
    for (int i = 0; i < m; ++i) an = fmax(an, rowsum[i]);
    int s = 0;
    if (an > 0.0) {
      const double l2 = log(an) / log(2.0);  // log_2 (:106-117)
      const int ee = (int)l2 + 1;            // int() truncates toward zero
      s = max(0, ee + 1);
    }
    s_sh = s;
  }
  __syncthreads();
  const int s = s_sh;
  const double sc = ldexp(1.0, -s);  // A/2**s, exact
  for (int i = tid; i < mm; i += nt) {
    double2 a = make_double2(A2[i].x * sc, A2[i].y * sc);
    A2[i] = a;
    X[i] = a;
    const double id = (i % (m + 1) == 0) ? 1.0 : 0.0;
    E[i] = make_double2(id + 0.5 * a.x, 0.5 * a.y);
    D[i] = make_double2(id - 0.5 * a.x, -0.5 * a.y);
  }
  __syncthreads();
  // Pade(6,6) by the c_k recurrence (:54-77)
  const int q = 6;
  double c = 0.5;
  bool p = true;
  for (int k = 2; k <= q; ++k) {
    c = c * (double)(q - k + 1) / (double)(k * (2 * q - k + 1));
    smem_matmul(m, A2, X, T);
    __syncthreads();
    for (int i = tid; i < mm; i += nt) {
      const double2 x = T[i];
      X[i] = x;
      E[i] = make_double2(E[i].x + c * x.x, E[i].y + c * x.y);
      D[i] = p ? make_double2(D[i].x + c * x.x, D[i].y + c * x.y)
               : make_double2(D[i].x - c * x.x, D[i].y - c * x.y);
    }
    p = !p;
    __syncthreads();
  }
  // inv(D) by LU with partial pivoting (|re|+|im| pivot, as izamax), in place
  for (int k = 0; k < m; ++k) {
    if (tid < 32) {
      double best = -1.0;
      int bi = k;
      for (int i = k + tid; i < m; i += 32) {
        const double v = fabs(D[i + k * m].x) + fabs(D[i + k * m].y);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (tid == 0) {
        p_sh = bi;
        piv[k] = bi;
        if (best == 0.0) atomicExch(err, 2);
      }
    }
    __syncthreads();
    const int pr = p_sh;
    if (pr != k)
      for (int j = tid; j < m; j += nt) {
        const double2 t0 = D[k + j * m];
        D[k + j * m] = D[pr + j * m];
        D[pr + j * m] = t0;
      }
    __syncthreads();
    const double2 dkk = D[k + k * m];
    for (int i = k + 1 + tid; i < m; i += nt) D[i + k * m] = cdiv(D[i + k * m], dkk);
    __syncthreads();
    const int rem = m - k - 1;
    for (int idx = tid; idx < rem * rem; idx += nt) {
      const int i = k + 1 + idx % rem, j = k + 1 + idx / rem;
      D[i + j * m] = cfms(D[i + k * m], D[k + j * m], D[i + j * m]);
    }
    __syncthreads();
  }
  // T = inv(D): column j solves LU x = P e_j
  for (int j = tid; j < m; j += nt) {
    double2* x = T + j * m;
    for (int i = 0; i < m; ++i) x[i] = i == j ? make_double2(1.0, 0.0) : cz();
    for (int k = 0; k < m; ++k)
      if (piv[k] != k) {
        const double2 t0 = x[k];
        x[k] = x[piv[k]];
        x[piv[k]] = t0;
      }
    for (int i = 0; i < m; ++i) {
      double2 acc = x[i];
      for (int k = 0; k < i; ++k) acc = cfms(D[i + k * m], x[k], acc);
      x[i] = acc;
    }
    for (int i = m - 1; i >= 0; --i) {
      double2 acc = x[i];
      for (int k = i + 1; k < m; ++k) acc = cfms(D[i + k * m], x[k], acc);
      x[i] = cdiv(acc, D[i + i * m]);
    }
  }
  __syncthreads();
  // E = inv(D) E, then s squarings
  smem_matmul(m, T, E, X);
  __syncthreads();
  for (int i = tid; i < mm; i += nt) E[i] = X[i];
  __syncthreads();
  for (int k = 0; k < s; ++k) {
    smem_matmul(m, E, E, X);
    __syncthreads();
    for (int i = tid; i < mm; i += nt) E[i] = X[i];
    __syncthreads();
  }
  double2* out = Aexp + (size_t)w * mm;
  for (int i = tid; i < mm; i += nt) out[i] = E[i];
}

// ---------------------------------------------------------------------------
// Krylov-space projectors (convert_to_krylov :469-498) as Hermitian Grams:
//   Tp = Q_b1^H Q_b1, Tm = Q_b4^H Q_b4,
//   S  = 1/2 (Q_b2 - Q_b3)^H (Q_b2 - Q_b3),  T0 = 1/2 (Q_b2 + Q_b3)^H (Q_b2 + Q_b3)
// with b1..b4 the Z-row blocks |aa>, |ab>, |ba>, |bb>. S and T0 are the
// Hermitian parts of the reference's P_S, P_T0; Re(c^H P c) is unchanged.
// Grid (samples, Z splits); 256 threads each own up to MAXC (type, i<=j).
#define PROJ_NC 32
template <int MAXC>
__global__ void __launch_bounds__(256)
    k_proj(int64_t N, int64_t Z, int ld, int m, int ncombo, const unsigned* __restrict__ combos,
           const double2* __restrict__ Q, int nsplit, double2* __restrict__ part) {
  extern __shared__ double2 V[];  // [4][m][PROJ_NC]
  const int w = blockIdx.x;
  const int split = blockIdx.y;
  const int tid = threadIdx.x;
  const int64_t per = (Z + nsplit - 1) / nsplit;
  const int64_t n0 = (int64_t)split * per;
  const int64_t n1 = min(Z, n0 + per);
  double2 acc[MAXC];
  int oi[MAXC], oj[MAXC];
#pragma unroll
  for (int q = 0; q < MAXC; ++q) {
    acc[q] = cz();
    const int cid = tid + q * 256;
    if (cid < ncombo) {
      const unsigned cb = combos[cid];
      const int t = cb >> 16, i = (cb >> 8) & 255, j = cb & 255;
      oi[q] = (t * m + i) * PROJ_NC;
      oj[q] = (t * m + j) * PROJ_NC;
    } else {
      oi[q] = oj[q] = 0;
    }
  }
  const size_t qstride = (size_t)N * ld;
  for (int64_t c0 = n0; c0 < n1; c0 += PROJ_NC) {
    const int len = (int)min((int64_t)PROJ_NC, n1 - c0);
    for (int idx = tid; idx < m * PROJ_NC; idx += 256) {
      const int j = idx / PROJ_NC, nn = idx % PROJ_NC;
      double2 q1 = cz(), q2 = cz(), q3 = cz(), q4 = cz();
      if (nn < len) {
        const double2* base = Q + (size_t)j * qstride + w;
        const int64_t n = c0 + nn;
        q1 = base[(size_t)n * ld];
        q2 = base[(size_t)(Z + n) * ld];
        q3 = base[(size_t)(2 * Z + n) * ld];
        q4 = base[(size_t)(3 * Z + n) * ld];
      }
      V[(0 * m + j) * PROJ_NC + nn] = q1;
      V[(1 * m + j) * PROJ_NC + nn] = csub(q2, q3);
      V[(2 * m + j) * PROJ_NC + nn] = cadd(q2, q3);
      V[(3 * m + j) * PROJ_NC + nn] = q4;
    }
    __syncthreads();
#pragma unroll 4
    for (int nn = 0; nn < PROJ_NC; ++nn) {
#pragma unroll
      for (int q = 0; q < MAXC; ++q)
        if (tid + q * 256 < ncombo) acc[q] = cjfma(V[oi[q] + nn], V[oj[q] + nn], acc[q]);
    }
    __syncthreads();
  }
  double2* out = part + ((size_t)split * gridDim.x + w) * ncombo;
#pragma unroll
  for (int q = 0; q < MAXC; ++q) {
    const int cid = tid + q * 256;
    if (cid < ncombo) out[cid] = acc[q];
  }
}

__global__ void k_proj_reduce(int Ma, int m, int ncombo, int nsplit,
                              const unsigned* __restrict__ combos, const double2* __restrict__ part,
                              double2* __restrict__ proj) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)Ma * ncombo) return;
  const int w = (int)(idx / ncombo), cid = (int)(idx % ncombo);
  double2 s = cz();
  for (int sp = 0; sp < nsplit; ++sp) s = cadd(s, part[((size_t)sp * Ma + w) * ncombo + cid]);
  const unsigned cb = combos[cid];
  const int t = cb >> 16, i = (cb >> 8) & 255, j = cb & 255;
  if (t == 1 || t == 2) s = make_double2(0.5 * s.x, 0.5 * s.y);
  double2* P = proj + ((size_t)w * 4 + t) * m * m;
  P[i + j * m] = s;
  if (i != j) P[j + i * m] = make_double2(s.x, -s.y);
}

// Orthonormality of a Lanczos basis from the projector Grams:
// max_ij |(Tp + S + T0 + Tm)_ij - delta_ij| > tol flags the sample.
#define ORTHO_TOL 1e-12
__global__ void __launch_bounds__(128)
    k_ortho_check(int m, int Ma, const double2* __restrict__ proj, double tol, int* __restrict__ flag) {
  __shared__ double red[128];
  const int w = blockIdx.x;
  const size_t mm = (size_t)m * m;
  const double2* P = proj + (size_t)w * 4 * mm;
  double mx = 0.0;
  for (int idx = threadIdx.x; idx < (int)mm; idx += blockDim.x) {
    const double2 g = cadd(cadd(P[idx], P[mm + idx]), cadd(P[2 * mm + idx], P[3 * mm + idx]));
    const double d = (idx % (m + 1) == 0) ? 1.0 : 0.0;
    const double e = fmax(fabs(g.x - d), fabs(g.y));
    mx = (e > mx || e != e) ? e : mx;  // NaN flags too
  }
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int o = 64; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const double v = red[threadIdx.x + o];
      if (v > red[threadIdx.x] || v != v) red[threadIdx.x] = v;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) flag[w] = !(red[0] <= tol);
}

// ---------------------------------------------------------------------------
// dt loop (src/qm_dynamics.f90:348-364), one warp per sample. Projector types
// in `proj`: 0 Tp, 1 S, 2 T0, 3 Tm; obs slots per sample: 0 S, 1 T0, 2 Tp, 3 Tm.
__global__ void __launch_bounds__(128)
    k_dtloop(int m, int Ma, int T, const int* __restrict__ map, const int* __restrict__ skip,
             const double2* __restrict__ Aexp,
             const double2* __restrict__ proj, double2* __restrict__ cvec, double* __restrict__ tt,
             int* __restrict__ kk, int* __restrict__ done, double* __restrict__ obs, double dt,
             double t_end, double tol, long long* __restrict__ nsteps, int* __restrict__ err) {
  __shared__ double2 cs[4][SPC_MAX_M];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * 4 + warp;
  if (w >= Ma || skip[w]) return;
  const int s = map[w];
  const size_t mm = (size_t)m * m;
  const double2* E = Aexp + (size_t)w * mm;
  const double2* PX = proj + (size_t)w * 4 * mm;
  double2* c = cs[warp];
  const bool l0 = lane < m, l1 = lane + 32 < m;
  if (l0) c[lane] = cvec[(size_t)w * m + lane];
  if (l1) c[lane + 32] = cvec[(size_t)w * m + lane + 32];
  __syncwarp();
  double t = tt[s];
  int k = kk[s];
  double c2 = 1.0, cm2 = 0.0;
  double* o = obs + (size_t)s * 4 * T;
  const int slot[4] = {2, 0, 1, 3};  // proj type -> obs slot
  long long steps = 0;
  while (cm2 <= tol * c2 && t < t_end) {
    double2 n0 = cz(), n1 = cz();
    for (int j = 0; j < m; ++j) {
      const double2 cj = c[j];
      if (l0) n0 = cfma(E[lane + j * m], cj, n0);
      if (l1) n1 = cfma(E[lane + 32 + j * m], cj, n1);
    }
    __syncwarp();
    if (l0) c[lane] = n0;
    if (l1) c[lane + 32] = n1;
    __syncwarp();
    if (k >= T) {
      if (lane == 0) atomicExch(err, 1);
      break;
    }
    for (int ty = 0; ty < 4; ++ty) {
      const double2* P = PX + ty * mm;
      double2 v0 = cz(), v1 = cz();
      for (int j = 0; j < m; ++j) {
        const double2 cj = c[j];
        if (l0) v0 = cfma(P[lane + j * m], cj, v0);
        if (l1) v1 = cfma(P[lane + 32 + j * m], cj, v1);
      }
      double term = 0.0;
      if (l0) term = fma(n0.x, v0.x, n0.y * v0.y);
      if (l1) term += fma(n1.x, v1.x, n1.y * v1.y);
      term = warp_sum(term);
      if (lane == 0) o[slot[ty] * T + k] = term;
    }
    double nn = 0.0;
    if (l0) nn = fma(n0.x, n0.x, n0.y * n0.y);
    if (l1) nn += fma(n1.x, n1.x, n1.y * n1.y);
    c2 = warp_sum(nn);
    const double2 cmv = c[m - 1];
    cm2 = cmv.x * cmv.x + cmv.y * cmv.y;
    t = t + dt;
    k = k + 1;
    steps++;
  }
  __syncwarp();
  if (l0) cvec[(size_t)w * m + lane] = c[lane];
  if (l1) cvec[(size_t)w * m + lane + 32] = c[lane + 32];
  if (lane == 0) {
    tt[s] = t;
    kk[s] = k;
    done[s] = (t < t_end) ? 0 : 1;
    atomicAdd((unsigned long long*)nsteps, (unsigned long long)steps);
  }
}

// psi[:, map[w]] = Q c  (src/qm_dynamics.f90:365)
__global__ void __launch_bounds__(256)
    k_psi_update(int64_t N, int ld, int Ma, int rpb, int m, const int* __restrict__ map,
                 const int* __restrict__ skip, int ldp,
                 const double2* __restrict__ Q, const double2* __restrict__ cvec,
                 double2* __restrict__ psi) {
  __shared__ double2 cs[SPC_MAX_M][SPC_LANES];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int w = blockIdx.x * SPC_LANES + tx;
  const bool act = w < Ma;
  for (int j = ty; j < m; j += SPC_WARPS) cs[j][tx] = act ? cvec[(size_t)w * m + j] : cz();
  __syncthreads();
  if (!act || skip[w]) return;
  const int s = map[w];
  const size_t qstride = (size_t)N * ld;
  const int64_t r0 = (int64_t)blockIdx.y * rpb;
  const int64_t r1 = min(N, r0 + rpb);
  for (int64_t r = r0 + ty; r < r1; r += SPC_WARPS) {
    double2 acc = cz();
    const double2* q = Q + (size_t)r * ld + w;
    for (int j = 0; j < m; ++j) acc = cfma(q[(size_t)j * qstride], cs[j][tx], acc);
    psi[(size_t)r * ldp + s] = acc;
  }
}

// kron_vector(theta, Z_ket) for every sample (src/kroenecker.f90:85-97)
struct Theta {
  double2 v[4];
};
__global__ void k_kron_init(int64_t Z, int M, int ldp, Theta th, const double2* __restrict__ zk,
                            double2* __restrict__ psi) {
  const int64_t total = Z * (int64_t)M;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int s = (int)(idx % M);
    const int64_t n = idx / M;
    const double2 z = zk[(size_t)s * Z + n];
#pragma unroll
    for (int e = 0; e < 4; ++e) psi[(size_t)(e * Z + n) * ldp + s] = cmul(th.v[e], z);
  }
}

__global__ void k_obs_init(int M, int T, double p0, double p1, double p2, double p3,
                           double* __restrict__ obs, double* __restrict__ tt, int* __restrict__ kk,
                           int* __restrict__ done) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= M) return;
  double* o = obs + (size_t)s * 4 * T;
  o[0] = p0;
  o[T] = p1;
  o[2 * T] = p2;
  o[3 * T] = p3;
  tt[s] = 0.0;
  kk[s] = 1;
  done[s] = 0;
}

// res%update over samples in order, then res%scale(1/M)
__global__ void k_average(int M, int T, const double* __restrict__ obs, double* __restrict__ out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 4 * T) return;
  const int q = idx / T, t = idx % T;
  double acc = 0.0;
  for (int s = 0; s < M; ++s) acc = acc + obs[((size_t)s * 4 + q) * T + t];
  out[idx] = acc * (1.0 / (double)M);
}

// ---------------------------------------------------------------------------
// Row blocks per sample tile so that the grid fills one wave of resident
// CTAs (tiles x nrb <= resident), with at least 32 rows per block.
static void geometry(int64_t N, int tiles, int resident, int& nrb, int& rpb) {
  int64_t want = std::max<int64_t>(1, resident / tiles);
  const int64_t maxb = std::max<int64_t>(1, (N + 31) / 32);
  want = std::min(want, maxb);
  rpb = (int)((N + want - 1) / want);
  nrb = (int)((N + rpb - 1) / rpb);
}

int num_time_points(double dt, double t_end) {
  const double x = (t_end + dt) / dt;
  return (int)std::ceil(x) + 1;
}

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return set_error(SPC_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

int propagate(Handle* h, const double* theta, const double* init_pop, const double* zk_dev, int M,
              double dt, double t_end, int m, double tol, double* out_dev, int T) {
  auto t_start = std::chrono::steady_clock::now();
  const int64_t N = h->n, Z = N / 4;
  cudaStream_t st = h->stream;
  const int ldp = (M + SPC_LANES - 1) / SPC_LANES * SPC_LANES;
  const int ld = ldp;
  const size_t mm = (size_t)m * m;
  const int tiles_max = ld / SPC_LANES;
  const int64_t pmax = std::min<int64_t>(std::max<int64_t>(1, (N + 31) / 32), (int64_t)h->sm_count * 32);
  const int ncombo = 4 * m * (m + 1) / 2;
  // Z splits of the projector Grams (chosen per round, at most nsplit_max,
  // at least 64 rows each); the partial buffer is sized for nsplit_max
  const int nsplit_max = (int)std::max<int64_t>(1, std::min<int64_t>(16, (Z + 63) / 64));
  const int nsplit = nsplit_max;
  // buffers
  if (h->ensure(h->psi, sizeof(double2) * N * ldp) || h->ensure(h->Q, sizeof(double2) * m * N * ld) ||
      h->ensure(h->P, sizeof(double2) * N * ld) || h->ensure(h->partial, sizeof(double2) * pmax * ld) ||
      h->ensure(h->counters, sizeof(unsigned) * tiles_max) || h->ensure(h->coef, sizeof(double2) * ld) ||
      h->ensure(h->rbeta, sizeof(double) * ld) || h->ensure(h->Ahess, sizeof(double2) * mm * ld) ||
      h->ensure(h->Aexp, sizeof(double2) * mm * ld) || h->ensure(h->proj, sizeof(double2) * 4 * mm * ld) ||
      h->ensure(h->projpart, sizeof(double2) * (size_t)nsplit * ld * ncombo + sizeof(unsigned) * ncombo) ||
      h->ensure(h->cvec, sizeof(double2) * m * ld) || h->ensure(h->tt, sizeof(double) * M) ||
      h->ensure(h->kk, sizeof(int) * M) || h->ensure(h->done, sizeof(int) * M) ||
      h->ensure(h->map, sizeof(int) * ld) || h->ensure(h->obs, sizeof(double) * 4 * (size_t)T * M) ||
      h->ensure(h->err, 16) || h->ensure(h->flag, sizeof(int) * ld))
    return SPC_ERR_ALLOC;
  int* d_flag = (int*)h->flag.p;
  double2* d_psi = (double2*)h->psi.p;
  double2* d_Q = (double2*)h->Q.p;
  double2* d_P = (double2*)h->P.p;
  double2* d_part = (double2*)h->partial.p;
  unsigned* d_cnt = (unsigned*)h->counters.p;
  double2* d_coef = (double2*)h->coef.p;
  double* d_rb = (double*)h->rbeta.p;
  double2* d_A = (double2*)h->Ahess.p;
  double2* d_E = (double2*)h->Aexp.p;
  double2* d_proj = (double2*)h->proj.p;
  double2* d_ppart = (double2*)h->projpart.p;
  unsigned* d_combos = (unsigned*)((char*)h->projpart.p + sizeof(double2) * (size_t)nsplit * ld * ncombo);
  double2* d_c = (double2*)h->cvec.p;
  double* d_t = (double*)h->tt.p;
  int* d_k = (int*)h->kk.p;
  int* d_done = (int*)h->done.p;
  int* d_map = (int*)h->map.p;
  double* d_obs = (double*)h->obs.p;
  int* d_err = (int*)h->err.p;
  long long* d_nsteps = (long long*)((char*)h->err.p + 8);

  int64_t launches0 = h->launches;
  CK(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned) * tiles_max, st));
  CK(cudaMemsetAsync(h->err.p, 0, 16, st));
  CK(cudaMemsetAsync(d_obs, 0, sizeof(double) * 4 * (size_t)T * M, st));
  if (ldp != M) CK(cudaMemsetAsync(d_psi, 0, sizeof(double2) * N * ldp, st));
  {
    std::vector<unsigned> combos(ncombo);
    int id = 0;
    for (int t = 0; t < 4; ++t)
      for (int i = 0; i < m; ++i)
        for (int j = i; j < m; ++j) combos[id++] = ((unsigned)t << 16) | ((unsigned)i << 8) | (unsigned)j;
    CK(cudaMemcpyAsync(d_combos, combos.data(), sizeof(unsigned) * ncombo, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
  }
  Theta th;
  for (int e = 0; e < 4; ++e) th.v[e] = make_double2(theta[2 * e], theta[2 * e + 1]);
  {
    const int64_t tot = Z * (int64_t)M;
    const int blocks = (int)std::min<int64_t>((tot + 255) / 256, (int64_t)h->sm_count * 16);
    k_kron_init<<<std::max(blocks, 1), 256, 0, st>>>(Z, M, ldp, th, (const double2*)zk_dev, d_psi);
  }
  k_obs_init<<<(M + 127) / 128, 128, 0, st>>>(M, T, init_pop[0], init_pop[1], init_pop[2],
                                               init_pop[3], d_obs, d_t, d_k, d_done);
  h->count_launch(2);
  CK(cudaGetLastError());

  const size_t expm_smem = sizeof(double2) * 5 * mm;
  const size_t proj_smem = sizeof(double2) * 4 * m * PROJ_NC;
  CK(cudaFuncSetAttribute(k_expm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)expm_smem));
  const int maxc = (ncombo + 255) / 256;
  const void* proj_fn = maxc <= 8 ? (const void*)k_proj<8> : maxc <= 16 ? (const void*)k_proj<16>
                                                                         : (const void*)k_proj<24>;
  CK(cudaFuncSetAttribute(proj_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)proj_smem));
  // resident CTAs per kernel: grids are sized to whole waves
  auto resident = [&](const void* fn, int threads, size_t smem) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, threads, smem) != cudaSuccess) b = 1;
    return std::max(1, b) * h->sm_count;
  };
  const int res_spmm = resident((const void*)k_spmm, 256, 0);
  const int res_pass = std::min(resident((const void*)k_rowpass<PASS_AXPY_DOT>, 256, 0),
                                resident((const void*)k_rowpass<PASS_AXPY_NORM>, 256, 0));
  const int res_scale = resident((const void*)k_scale, 256, 0);
  const int res_psi = resident((const void*)k_psi_update, 256, 0);
  const int res_proj = resident(proj_fn, 256, proj_smem);

  std::vector<int> active;
  if (0.0 < t_end)
    for (int s = 0; s < M; ++s) active.push_back(s);
  std::vector<int> done_h(M, 0), flag_h(ld, 0);
  int64_t builds = 0, rounds = 0, fallbacks = 0;
  const dim3 blk(SPC_LANES, SPC_WARPS);
  const bool use_lanczos = h->lanczos_active();

  // One build round for the samples in `list`: Krylov basis (Lanczos or full
  // MGS), expm, projectors; then the dt loop and psi = Q c for every sample
  // whose basis passed the orthogonality check. Returns the samples that
  // failed it (Lanczos only); their state is left untouched.
  auto round = [&](const std::vector<int>& list, bool lanczos, std::vector<int>& failed) -> int {
    failed.clear();
    const int Ma = (int)list.size();
    const int tiles = (Ma + SPC_LANES - 1) / SPC_LANES;
    int nrb, rpb, nrb_s, rpb_s, nrb_c, rpb_c, nrb_u, rpb_u;
    geometry(N, tiles, res_pass, nrb, rpb);
    geometry(N, tiles, res_spmm, nrb_s, rpb_s);
    geometry(N, tiles, res_scale, nrb_c, rpb_c);
    geometry(N, tiles, res_psi, nrb_u, rpb_u);
    const dim3 grid(tiles, nrb), grid_s(tiles, nrb_s), grid_c(tiles, nrb_c), grid_u(tiles, nrb_u);
    // projector split: the count in [1, nsplit_max] whose grid wastes the
    // least of its last wave
    int ns = 1;
    {
      double best = 1e30;
      for (int c = 1; c <= nsplit_max; ++c) {
        const double waves = (double)Ma * c / res_proj;
        const double loss = std::ceil(waves) / waves - 1.0 + 0.002 * c;
        if (loss < best) {
          best = loss;
          ns = c;
        }
      }
    }
    CK(cudaMemcpyAsync(d_map, list.data(), sizeof(int) * Ma, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(d_A, 0, sizeof(double2) * mm * Ma, st));
    CK(cudaMemsetAsync(d_flag, 0, sizeof(int) * ld, st));
    PassArgs a{};
    a.N = N;
    a.ld = ld;
    a.Ma = Ma;
    a.rpb = rpb;
    a.m = m;
    a.map = d_map;
    a.ldp = ldp;
    a.coef = d_coef;
    a.rbeta = d_rb;
    a.Ahess = d_A;
    a.cvec = d_c;
    a.partial = d_part;
    a.counters = d_cnt;
    a.P = d_P;
    a.lanczos = lanczos ? 1 : 0;
    // c = ||psi|| e1 ; Q0 = psi/||psi||
    a.X = d_psi;
    const double elems = (double)N * Ma;
    int pe = h->prof.begin(st);
    k_rowpass<PASS_NORM_GATHER><<<grid, blk, 0, st>>>(a);
    h->prof.end(st, pe, PK_DOT, 4.0 * elems, 16.0 * elems);
    pe = h->prof.begin(st);
    k_scale<<<grid_c, blk, 0, st>>>(N, ld, Ma, rpb_c, d_psi, ldp, d_map, 1, d_rb, d_Q);
    h->prof.end(st, pe, PK_SCALE, 2.0 * elems, 32.0 * elems);
    h->count_launch(2);
    const size_t qs = (size_t)N * ld;
    for (int i = 0; i < m; ++i) {
      const double2* Qi = d_Q + (size_t)i * qs;
      pe = h->prof.begin(st);
      k_spmm<<<grid_s, blk, 0, st>>>(N, ld, Ma, rpb_s, h->d_rowptr, (const int*)h->xsplit.p,
                                     (const int*)h->xcol.p, (const double2*)h->xval.p, Qi, d_P);
      // algorithmic traffic: H once, X once, Y once
      h->prof.end(st, pe, PK_SPMM, 8.0 * (double)h->nnz * Ma,
                  20.0 * (double)h->nnz + 4.0 * (N + 1) + 32.0 * elems);
      h->count_launch();
      a.col_i = i;
      // MGS (get_krylov :453-456) projects p on Q_0..Q_i in order. Lanczos
      // (H_eff Hermitian up to -i*kappa) needs only Q_{i-1} (coefficient
      // beta_{i-1}, already in coef) and Q_i.
      int j0 = 0;
      if (lanczos && i > 0) {
        j0 = i - 1;
      } else {
        a.row_j = 0;
        a.X = d_Q;
        pe = h->prof.begin(st);
        k_rowpass<PASS_DOT><<<grid, blk, 0, st>>>(a);
        h->prof.end(st, pe, PK_DOT, 8.0 * elems, 32.0 * elems);
        h->count_launch();
      }
      for (int j = j0; j < i; ++j) {
        a.Qj = d_Q + (size_t)j * qs;
        a.Qn = d_Q + (size_t)(j + 1) * qs;
        a.row_j = j + 1;
        pe = h->prof.begin(st);
        k_rowpass<PASS_AXPY_DOT><<<grid, blk, 0, st>>>(a);
        h->prof.end(st, pe, PK_AXPY_DOT, 16.0 * elems, 64.0 * elems);
        h->count_launch();
      }
      if (i < m - 1) {
        a.Qj = Qi;
        a.row_j = i + 1;
        pe = h->prof.begin(st);
        k_rowpass<PASS_AXPY_NORM><<<grid, blk, 0, st>>>(a);
        h->prof.end(st, pe, PK_AXPY_NORM, 12.0 * elems, 48.0 * elems);
        pe = h->prof.begin(st);
        k_scale<<<grid_c, blk, 0, st>>>(N, ld, Ma, rpb_c, d_P, ldp, d_map, 0, d_rb,
                                          d_Q + (size_t)(i + 1) * qs);
        h->prof.end(st, pe, PK_SCALE, 2.0 * elems, 32.0 * elems);
        h->count_launch(2);
      }
    }
    pe = h->prof.begin(st);
    k_expm<<<Ma, 128, expm_smem, st>>>(m, Ma, d_A, d_E, dt, d_err);
    h->prof.end(st, pe, PK_EXPM, 8.0 * (double)mm * m * 9.0 * Ma, 32.0 * (double)mm * Ma);
    const dim3 pgrid(Ma, ns);
    pe = h->prof.begin(st);
    if (maxc <= 8)
      k_proj<8><<<pgrid, 256, proj_smem, st>>>(N, Z, ld, m, ncombo, d_combos, d_Q, ns, d_ppart);
    else if (maxc <= 16)
      k_proj<16><<<pgrid, 256, proj_smem, st>>>(N, Z, ld, m, ncombo, d_combos, d_Q, ns, d_ppart);
    else
      k_proj<24><<<pgrid, 256, proj_smem, st>>>(N, Z, ld, m, ncombo, d_combos, d_Q, ns, d_ppart);
    h->prof.end(st, pe, PK_PROJ, 8.0 * (double)ncombo * Z * Ma + 4.0 * (double)m * Z * Ma,
                16.0 * (double)m * N * Ma);
    {
      const int64_t tot = (int64_t)Ma * ncombo;
      pe = h->prof.begin(st);
      k_proj_reduce<<<(int)((tot + 255) / 256), 256, 0, st>>>(Ma, m, ncombo, ns, d_combos, d_ppart,
                                                             d_proj);
      h->prof.end(st, pe, PK_PROJ_REDUCE, 2.0 * tot * ns, 16.0 * tot * (ns + 1));
      h->count_launch(3);
    }
    if (lanczos) {
      // G = Q^H Q = Tp + S + T0 + Tm; a basis that drifted from orthonormal
      // beyond ORTHO_TOL is rebuilt with full MGS
      k_ortho_check<<<Ma, 128, 0, st>>>(m, Ma, d_proj, ORTHO_TOL, d_flag);
      h->count_launch();
      CK(cudaMemcpyAsync(flag_h.data(), d_flag, sizeof(int) * Ma, cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      for (int w = 0; w < Ma; ++w)
        if (flag_h[w]) failed.push_back(list[w]);
    }
    pe = h->prof.begin(st);
    k_dtloop<<<(Ma + 3) / 4, 128, 0, st>>>(m, Ma, T, d_map, d_flag, d_E, d_proj, d_c, d_t, d_k, d_done,
                                           d_obs, dt, t_end, tol, d_nsteps, d_err);
    h->prof.end(st, pe, PK_DTLOOP, 0.0, 0.0);
    pe = h->prof.begin(st);
    k_psi_update<<<grid_u, blk, 0, st>>>(N, ld, Ma, rpb_u, m, d_map, d_flag, ldp, d_Q, d_c, d_psi);
    h->prof.end(st, pe, PK_PSI, 8.0 * m * elems, 16.0 * (m + 1) * elems);
    h->count_launch(2);
    CK(cudaGetLastError());
    return SPC_OK;
  };

  std::vector<int> failed, failed2;
  while (!active.empty()) {
    int rc = round(active, use_lanczos, failed);
    if (rc) return rc;
    builds += (int64_t)active.size() - (int64_t)failed.size();
    if (!failed.empty()) {
      fallbacks += (int64_t)failed.size();
      rc = round(failed, false, failed2);
      if (rc) return rc;
      builds += (int64_t)failed.size();
    }
    CK(cudaMemcpyAsync(done_h.data(), d_done, sizeof(int) * M, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    h->prof.collect();
    rounds++;
    std::vector<int> next;
    next.reserve(active.size());
    for (int s : active)
      if (!done_h[s]) next.push_back(s);
    active.swap(next);
  }
  k_average<<<(4 * T + 255) / 256, 256, 0, st>>>(M, T, d_obs, out_dev);
  h->count_launch();
  CK(cudaGetLastError());
  int err_h[4] = {0, 0, 0, 0};
  CK(cudaMemcpyAsync(err_h, h->err.p, 16, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  long long nsteps = 0;
  std::memcpy(&nsteps, &err_h[2], 8);
  h->stats.krylov_builds = builds;
  h->stats.lanczos_fallbacks = fallbacks;
  h->stats.rounds = rounds;
  h->stats.sample_steps = nsteps;
  h->stats.kernel_launches = h->launches - launches0;
  h->stats.seconds =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  if (err_h[0] == 1)
    return set_error(SPC_ERR_NUMERIC, "time index overflow: the dt loop ran past %d output slots", T);
  if (err_h[0] == 2)
    return set_error(SPC_ERR_NUMERIC, "singular Pade denominator in expm");
  return SPC_OK;
}

}  // namespace spc
