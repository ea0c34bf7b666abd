// Batched trace-sampling propagation on the device.
//
// Restates trace_sampling_para (src/qm_dynamics.f90:257-384) for many samples
// of one or many independent systems ("jobs": radical pairs, field
// orientations, symmetry blocks) at once. Every job keeps its own
// Hamiltonian and dimension; its samples are grouped into tiles of 32, and a
// tile's vectors are stored as a self-contained [rows][32] block with the
// sample index fastest, so a warp reads 32 samples of one row as one 512-byte
// transaction and tiles of jobs of any size mix freely in one launch.
//
// Each round, every sample that has not reached t_end builds a new Krylov
// basis (the reference rebuilds each sample independently; the build does not
// depend on t, so batching the builds of all unfinished samples is the same
// computation), then runs its own dt loop until its own rebuild test fires.
// Finished samples leave the next round's tiles.
//
// Per round:
//   norm/scale passes      c = ||psi|| e1, Q0 = psi/||psi||      (get_krylov :445-449)
//   m x [ SpMM p = H Q_i ; MGS (or Lanczos) passes ; scale ]       (:451-465)
//   Pade-6 expm of -i dt A per sample, one CTA each               (matrix_exponential.f90)
//   Krylov projectors as Hermitian Grams per sample               (convert_to_krylov :469-498)
//   dt loop per sample, one warp each                             (:351-364)
//   psi = Q c                                                      (:365)
//
// Row kernels run over work items (tile, phase): an item takes every
// (items_of_tile * 8)-th row of its tile starting at phase*8 + warp, so row
// lengths balance and all items of a tile sweep its rows together. Item
// counts per tile are proportional to the tile's rows and sum to about one
// wave of resident CTAs. Reductions are two-level and in a fixed order
// (per-item partials, then the last item of each tile sums them), so results
// do not depend on scheduling.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <set>
#include <vector>

#include <cooperative_groups.h>

#include "spc_common.cuh"
#include "spc_internal.h"

namespace spc {

// Per-tile description (device copy built each round).
struct TileInfo {
  int job;           // job index
  int n;             // rows = Hilbert dimension of the job
  int ldp;           // leading dimension of the job's psi block
  int ip0, nip;      // first pass item, pass items of this tile
  int is0, nis;      // first SpMM item, SpMM items of this tile
  int m;             // Krylov dimension of this tile's job: min(m, n)
  int64_t q_off;     // Q_t[j] = Q + q_off + j * n * 32
  int64_t p_off;     // P_t = P + p_off
  int64_t psi_off;   // job psi block
  const int* rowptr;
  const int* split;
  const int* col;
  const double2* val;
  const double* vsum;  // Re + Im of every entry of the execution copy
  // non-null: the execution copy holds the Hermitian part A of
  // H_eff = A - i*kappa*1 (real diagonal) and *kappa the shift
  const double* kappa;
};

enum PassKind { PASS_NORM_GATHER = 0, PASS_DOT = 1, PASS_AXPY_DOT = 2, PASS_AXPY_NORM = 3 };

struct PassArgs {
  const TileInfo* tiles;
  const int2* items;  // pass items (tile, phase)
  int m, col_i, row_j;
  int lanczos;        // AXPY_NORM also seeds the next Lanczos coefficient
  int jx, jn;         // basis indices: DOT reads Q_jx; AXPY removes Q_jx, dots with Q_jn
  const double2* Q;
  double2* P;
  const double2* psi;
  const int* map;     // slot -> global sample (or -1)
  const int* scol;    // slot -> column in its job's psi
  double2* coef;      // current MGS coefficient per slot
  double* rbeta;      // 1/norm per slot
  double2* Ahess;     // Hessenberg matrices, m x m column-major per slot
  double2* cvec;      // Krylov coordinates per slot
  double2* partial;   // [items][32]
  unsigned* counters; // per tile
};

// REAL: the Hermitian Lanczos recurrence on A of H_eff = A - i*kappa*1
// (tile's kappa non-null): every coefficient is real, the dots keep their real
// part, and the tridiagonal's diagonal gets the shift: alpha - i*kappa.
template <int KIND, bool REAL>
__device__ __forceinline__ void pass_finalize(const PassArgs& a, int w, double2 tot, const double* kappa) {
  const size_t mm = (size_t)a.m * a.m;
  if (KIND == PASS_NORM_GATHER) {
    double b = sqrt(tot.x);
    double2* c = a.cvec + (size_t)w * a.m;
    c[0] = make_double2(b, 0.0);
    for (int j = 1; j < a.m; ++j) c[j] = cz();
    a.rbeta[w] = b > 0.0 ? 1.0 / b : 0.0;
  } else if (KIND == PASS_DOT || KIND == PASS_AXPY_DOT) {
    if (REAL) {
      a.coef[w] = make_double2(tot.x, 0.0);
      a.Ahess[(size_t)w * mm + a.row_j + (size_t)a.col_i * a.m] = make_double2(tot.x, -*kappa);
    } else {
      a.coef[w] = tot;
      a.Ahess[(size_t)w * mm + a.row_j + (size_t)a.col_i * a.m] = tot;
    }
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

// One pass over the rows of a work item: element update + per-slot
// reduction. Grid = pass items, block (32, SPC_WARPS). REAL (Lanczos on the
// Hermitian part): real coefficients (2 DFMA per axpy) and real dots.
template <int KIND, bool REAL = false>
__global__ void __launch_bounds__(256) k_rowpass(PassArgs a) {
  __shared__ double2 red[SPC_WARPS][SPC_LANES];
  __shared__ bool am_last;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int2 it = a.items[blockIdx.x];
  const TileInfo& T = a.tiles[it.x];
  // steps past this job's Krylov dimension (whole tile, so whole CTA)
  if (KIND != PASS_NORM_GATHER && (a.col_i >= T.m || (KIND == PASS_AXPY_NORM && a.col_i >= T.m - 1)))
    return;
  const int w = it.x * SPC_LANES + tx;
  const bool act = a.map[w] >= 0;
  const int n = T.n;
  const int stride = T.nip * SPC_WARPS;
  const size_t vs = (size_t)n * SPC_LANES;
  double2 acc = cz();
  if (act) {
    if (KIND == PASS_NORM_GATHER) {
      const double2* src = a.psi + T.psi_off + a.scol[w];
      for (int r = it.y * SPC_WARPS + ty; r < n; r += stride) {
        double2 x = src[(size_t)r * T.ldp];
        acc.x = fma(x.x, x.x, acc.x);
        acc.x = fma(x.y, x.y, acc.x);
      }
    } else if (KIND == PASS_DOT) {
      const double2* X = a.Q + T.q_off + a.jx * vs + tx;
      const double2* P = a.P + T.p_off + tx;
      for (int r = it.y * SPC_WARPS + ty; r < n; r += stride) {
        const size_t o = (size_t)r * SPC_LANES;
        if (REAL) {
          const double2 x = X[o], p = P[o];
          acc.x = fma(x.x, p.x, acc.x);
          acc.x = fma(x.y, p.y, acc.x);
        } else {
          acc = cjfma(X[o], P[o], acc);
        }
      }
    } else {
      const double2 cf = a.coef[w];
      const double2* Qj = a.Q + T.q_off + a.jx * vs + tx;
      const double2* Qn = a.Q + T.q_off + a.jn * vs + tx;
      double2* P = a.P + T.p_off + tx;
      for (int r = it.y * SPC_WARPS + ty; r < n; r += stride) {
        const size_t o = (size_t)r * SPC_LANES;
        double2 p;
        if (REAL) {
          const double2 q = Qj[o], p0 = P[o];
          p.x = fma(-cf.x, q.x, p0.x);
          p.y = fma(-cf.x, q.y, p0.y);
        } else {
          p = cfms(cf, Qj[o], P[o]);
        }
        P[o] = p;
        if (KIND == PASS_AXPY_DOT) {
          if (REAL) {
            const double2 q = Qn[o];
            acc.x = fma(q.x, p.x, acc.x);
            acc.x = fma(q.y, p.y, acc.x);
          } else {
            acc = cjfma(Qn[o], p, acc);
          }
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
    a.partial[(size_t)blockIdx.x * SPC_LANES + tx] = s;
  }
  __threadfence();
  __syncthreads();
  if (tx == 0 && ty == 0) {
    unsigned t = atomicAdd(&a.counters[it.x], 1u);
    am_last = (t == (unsigned)T.nip - 1);
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  double2 s = cz();
  for (int b = ty; b < T.nip; b += SPC_WARPS)
    s = cadd(s, __ldcg(&a.partial[(size_t)(T.ip0 + b) * SPC_LANES + tx]));
  red[ty][tx] = s;
  __syncthreads();
  if (ty == 0) {
    double2 tot = red[0][tx];
#pragma unroll
    for (int y = 1; y < SPC_WARPS; ++y) tot = cadd(tot, red[y][tx]);
    if (act) pass_finalize<KIND, REAL>(a, w, tot, T.kappa);
    if (tx == 0) a.counters[it.x] = 0u;
  }
}

// Q_{jd} = P / ||P||  (or Q_0 = psi[:, scol] / ||psi|| when gather != 0),
// and beside it XS = Re + Im of the stored Q_{jd} (the operand k_spmm's
// three-product form reads); grid = pass items. XS has P's layout (p_off).
__global__ void __launch_bounds__(256)
    k_scale(const TileInfo* __restrict__ tiles, const int2* __restrict__ items,
            const int* __restrict__ map, const int* __restrict__ scol,
            const double2* __restrict__ psi, const double2* __restrict__ P, int gather, int jd,
            const double* __restrict__ rbeta, double2* __restrict__ Q, double* __restrict__ XS) {
  const int2 it = items[blockIdx.x];
  const TileInfo& T = tiles[it.x];
  if (!gather && jd >= T.m) return;
  const int tx = threadIdx.x;
  const int w = it.x * SPC_LANES + tx;
  if (map[w] < 0) return;
  const double rb = rbeta[w];
  const int n = T.n;
  const int stride = T.nip * SPC_WARPS;
  double2* dst = Q + T.q_off + (size_t)jd * n * SPC_LANES + tx;
  double* xs = XS + T.p_off + tx;
  if (gather) {
    const double2* src = psi + T.psi_off + scol[w];
    for (int r = it.y * SPC_WARPS + threadIdx.y; r < n; r += stride) {
      const double2 x = src[(size_t)r * T.ldp];
      const double2 q = make_double2(x.x * rb, x.y * rb);
      dst[(size_t)r * SPC_LANES] = q;
      xs[(size_t)r * SPC_LANES] = q.x + q.y;
    }
  } else {
    const double2* src = P + T.p_off + tx;
    for (int r = it.y * SPC_WARPS + threadIdx.y; r < n; r += stride) {
      const double2 x = src[(size_t)r * SPC_LANES];
      const double2 q = make_double2(x.x * rb, x.y * rb);
      dst[(size_t)r * SPC_LANES] = q;
      xs[(size_t)r * SPC_LANES] = q.x + q.y;
    }
  }
}

// P_t = H Q_t[i] for the tile of a SpMM item; one warp per row at a time, the
// row's (col, val) entries broadcast to all lanes, one sample per lane.
// Complex products in the three-multiplication form (Gauss; Higham, SIAM J.
// Matrix Anal. Appl. 13 (1992) 681-687): with v = a + ib, x = c + id,
//   t1 += a c,  t2 += b d,  t3 += (a + b)(c + d);  y = (t1 - t2, t3 - t1 - t2)
// where a + b is stored with the execution copy (vsum) and c + d beside the
// basis vector (XS, written by k_scale): 3 DFMA per entry instead of 4 on
// GB300's narrow FP64 pipe. Rows are in the execution order of k_split_rows:
// entries with a nonzero imaginary part first, then real ones from split[r]
// on (b = 0: t1 and t3 only, 2 DFMA). A tile whose copy holds the Hermitian
// part A of A - i*kappa*1 gets A x, plus -i*kappa x when `shift` is set (full
// H_eff for MGS rounds; Lanczos rounds run on A). Five resident CTAs per SM
// (48 registers) instead of four keep more warps on each FP64 pipe: +2 % in
// this kernel's FP64 rate at dim 55296, M = 512.
__global__ void __launch_bounds__(256, 5)
    k_spmm(const TileInfo* __restrict__ tiles, const int2* __restrict__ items,
           const int* __restrict__ map, int i, const double2* __restrict__ Q,
           const double* __restrict__ XS, double2* __restrict__ Pout, int shift) {
  const int2 it = items[blockIdx.x];
  const TileInfo& T = tiles[it.x];
  if (i >= T.m) return;
  const bool sh = shift && T.kappa != nullptr;
  const double kp = sh ? __ldg(T.kappa) : 0.0;
  const int tx = threadIdx.x;
  const bool act = map[it.x * SPC_LANES + tx] >= 0;
  const int n = T.n;
  const int* __restrict__ rowptr = T.rowptr;
  const int* __restrict__ split = T.split;
  const int* __restrict__ col = T.col;
  const double2* __restrict__ val = T.val;
  const double* __restrict__ vsum = T.vsum;
  const double2* X = Q + T.q_off + (size_t)i * n * SPC_LANES + tx;
  const double* Xs = XS + T.p_off + tx;
  double2* Y = Pout + T.p_off + tx;
  const int stride = T.nis * SPC_WARPS;
  for (int r = it.y * SPC_WARPS + threadIdx.y; r < n; r += stride) {
    const int k0 = __ldg(rowptr + r), ks = __ldg(split + r), k1 = __ldg(rowptr + r + 1);
    double t1 = 0.0, t2 = 0.0, t3 = 0.0;
    int k = k0;
#pragma unroll 4
    for (; k < ks; ++k) {
      const int c = __ldg(col + k);
      const double2 v = __ldg(val + k);
      const double vs = __ldg(vsum + k);
      if (act) {
        const double2 x = X[(size_t)c * SPC_LANES];
        const double xs = Xs[(size_t)c * SPC_LANES];
        t1 = fma(v.x, x.x, t1);
        t2 = fma(v.y, x.y, t2);
        t3 = fma(vs, xs, t3);
      }
    }
#pragma unroll 4
    for (; k < k1; ++k) {
      const int c = __ldg(col + k);
      const double v = __ldg(&val[k].x);
      if (act) {
        const double xr = X[(size_t)c * SPC_LANES].x;
        const double xs = Xs[(size_t)c * SPC_LANES];
        t1 = fma(v, xr, t1);
        t3 = fma(v, xs, t3);
      }
    }
    if (act) {
      double2 y = make_double2(t1 - t2, t3 - t1 - t2);
      if (sh) {  // -i*kappa*x_r
        const double2 xr = X[(size_t)r * SPC_LANES];
        y.x = fma(kp, xr.y, y.x);
        y.y = fma(-kp, xr.x, y.y);
      }
      Y[(size_t)r * SPC_LANES] = y;
    }
  }
}

// Execution copy of a CSR for k_spmm: each row's entries reordered so that
// those with a nonzero imaginary part come first (original order kept within
// each class); split[r] is the index of the row's first real entry, and
// xvs[k] = Re + Im of entry k. herm (H = A - i*kappa*1, A Hermitian): diagonal
// entries are stored with their imaginary part removed (real class) and row
// 0's removed sum is kappa. meta->ncplx counts the copy's complex entries.
__global__ void k_split_rows(int64_t N, const int* __restrict__ rowptr, const int* __restrict__ col,
                             const double2* __restrict__ val, int* __restrict__ xcol,
                             double2* __restrict__ xval, double* __restrict__ xvs, int* __restrict__ split,
                             int herm, HMeta* __restrict__ meta) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long nc = 0;
  if (r < N) {
    const int k0 = rowptr[r], k1 = rowptr[r + 1];
    auto cplx = [&](int k) { return val[k].y != 0.0 && !(herm && col[k] == r); };
    int o = k0;
    for (int k = k0; k < k1; ++k)
      if (cplx(k)) {
        xcol[o] = col[k];
        xval[o] = val[k];
        xvs[o] = val[k].x + val[k].y;
        o++;
      }
    split[r] = o;
    nc = (unsigned long long)(o - k0);
    double shift = 0.0;
    for (int k = k0; k < k1; ++k)
      if (!cplx(k)) {
        xcol[o] = col[k];
        xval[o] = herm ? make_double2(val[k].x, 0.0) : val[k];
        xvs[o] = val[k].x;
        if (herm && col[k] == r) shift += val[k].y;
        o++;
      }
    if (herm && r == 0) meta->kappa = -shift;
  }
  for (int d = 16; d > 0; d >>= 1) nc += __shfl_down_sync(0xffffffffu, nc, d);
  if ((threadIdx.x & 31) == 0 && nc) atomicAdd(&meta->ncplx, nc);
}

void enqueue_split_rows(int64_t N, const int* rowptr, const int* col, const double2* val, int* xcol,
                        double2* xval, double* xvs, int* split, bool herm, HMeta* meta, cudaStream_t st) {
  if (N > 0)
    k_split_rows<<<(int)((N + 255) / 256), 256, 0, st>>>(N, rowptr, col, val, xcol, xval, xvs, split,
                                                          herm ? 1 : 0, meta);
}

int prepare_spmm_rows(Handle* h) {
  const int64_t N = h->n, nnz = h->nnz;
  if (h->ensure(h->xcol, sizeof(int) * (nnz > 0 ? nnz : 1)) ||
      h->ensure(h->xval, sizeof(double2) * (nnz > 0 ? nnz : 1)) ||
      h->ensure(h->xvs, sizeof(double) * (nnz > 0 ? nnz : 1)) || h->ensure(h->xsplit, sizeof(int) * N) ||
      h->ensure(h->hmeta, sizeof(HMeta)))
    return SPC_ERR_ALLOC;
  HMeta meta{};
  if (cudaMemsetAsync(h->hmeta.p, 0, sizeof(HMeta), h->stream) != cudaSuccess)
    return set_error(SPC_ERR_CUDA, "row split of the Hamiltonian failed");
  enqueue_split_rows(N, h->d_rowptr, h->d_col, h->d_val, (int*)h->xcol.p, (double2*)h->xval.p,
                     (double*)h->xvs.p, (int*)h->xsplit.p, h->herm_shift, (HMeta*)h->hmeta.p, h->stream);
  h->count_launch();
  cudaError_t e = cudaMemcpyAsync(&meta, h->hmeta.p, sizeof(HMeta), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess)
    return set_error(SPC_ERR_CUDA, "row split of the Hamiltonian failed: %s", cudaGetErrorString(e));
  h->nnz_cplx = (int64_t)meta.ncplx;
  return SPC_OK;
}

// ---------------------------------------------------------------------------
// expm (src/matrix_exponential.f90:14-87) of -i dt A per sample, column-major
// m x m matrices in shared memory. expm_one is run by nt threads (index tid)
// that synchronise as a whole CTA (one sample per CTA) or as one warp (k_expm
// packs four samples per 128-thread CTA for m <= 16); every element is
// computed by the same serial loop either way, so both give the same bits.
template <bool WARP>
__device__ __forceinline__ void expm_sync() {
  if (WARP)
    __syncwarp();
  else
    __syncthreads();
}

// C = A B; each dot in two interleaved partial sums (even and odd k) so that
// consecutive FMAs of a thread do not wait on each other.
__device__ void smem_matmul(int m, const double2* A, const double2* B, double2* C, int tid, int nt) {
  const int mm = m * m;
  for (int idx = tid; idx < mm; idx += nt) {
    const int i = idx % m, j = idx / m;
    double2 a0 = cz(), a1 = cz();
    int k = 0;
    for (; k + 1 < m; k += 2) {
      a0 = cfma(A[i + k * m], B[k + j * m], a0);
      a1 = cfma(A[i + (k + 1) * m], B[(k + 1) + j * m], a1);
    }
    if (k < m) a0 = cfma(A[i + k * m], B[k + j * m], a0);
    C[idx] = cadd(a0, a1);
  }
}

// C = A B for A with lower/upper bandwidths (la, ua) (A_ik = 0 when i - k > la
// or k - i > ua) and B with (lb, ub): only the k where both factors can be
// nonzero, in smem_matmul's even/odd partial sums and order. The skipped
// terms are exact zeros, so every element rounds as the full product does
// (finite inputs; at most the sign of a zero entry differs).
__device__ void smem_matmul_band(int m, const double2* A, int la, int ua, const double2* B, int lb, int ub,
                                 double2* C, int tid, int nt) {
  const int mm = m * m;
  for (int idx = tid; idx < mm; idx += nt) {
    const int i = idx % m, j = idx / m;
    const int k1 = min(min(i + ua, j + lb), m - 1);
    int k = max(max(i - la, j - ub), 0);
    double2 a0 = cz(), a1 = cz();
    if (k <= k1 && (k & 1)) {
      a1 = cfma(A[i + k * m], B[k + j * m], a1);
      ++k;
    }
    for (; k + 1 <= k1; k += 2) {
      a0 = cfma(A[i + k * m], B[k + j * m], a0);
      a1 = cfma(A[i + (k + 1) * m], B[(k + 1) + j * m], a1);
    }
    if (k <= k1) a0 = cfma(A[i + k * m], B[k + j * m], a0);
    C[idx] = cadd(a0, a1);
  }
}

// Padé(6,6) coefficient c_k by the reference's recurrence (:54-77),
// c_0 = 1, c_1 = 1/2, c_k = c_{k-1} (q - k + 1) / (k (2q - k + 1)), folded at
// compile time with the same IEEE double operations.
constexpr double pade6_coef(int k) {
  double c = 1.0;
  for (int j = 1; j <= k; ++j) c = j == 1 ? 0.5 : c * (double)(6 - j + 1) / (double)(j * (2 * 6 - j + 1));
  return c;
}

// Complex reciprocal 1/d = conj(d) / |d|^2, for the band path's pivots (the
// diagonal of a diagonally dominant denominator, |d| of order one).
__device__ __forceinline__ double2 crcp(double2 d) {
  const double s = 1.0 / fma(d.x, d.x, d.y * d.y);
  return make_double2(d.x * s, -d.y * s);
}

// Padé(6,6) with scaling and squaring, evaluated on the bands of the input:
// a Lanczos basis gives a tridiagonal matrix, MGS an upper Hessenberg one.
// The powers and the Padé sums (each element by the dense evaluation's
// operations in its order: the skipped terms are exact zeros), the LU
// factors (while partial pivoting keeps the diagonal, which the
// denominator's diagonal dominance at the scaled norm < 1/2 makes the rule)
// and the triangular solves then only touch their bands. On that path the
// multipliers and the upper solve use the pivots' reciprocals: a complex
// division is three IEEE divides on the serial path of every step. A pivot
// off the diagonal restarts the factorisation dense with Smith's division.
template <bool WARP>
__device__ void expm_one(int m, int mld, const double2* __restrict__ Ain, double2* __restrict__ out, double dt,
                         double2* sm, double* rowsum, int* piv, int* s_sh, int* p_sh, int tid, int nt,
                         int* __restrict__ err) {
  const int mm = m * m;
  double2* A2 = sm;
  double2* X = A2 + mm;
  double2* E = X + mm;
  double2* D = E + mm;
  double2* T = D + mm;
  // (0,-1)*dt*A and its bandwidths (held in piv[0], piv[1] until the LU)
  if (tid == 0) piv[0] = piv[1] = 0;
  expm_sync<WARP>();
  {
    int bl = 0, bu = 0;
    for (int i = tid; i < mm; i += nt) {
      const double2 a = Ain[(i % m) + (size_t)(i / m) * mld];
      const double2 v = make_double2(dt * a.y, -dt * a.x);
      A2[i] = v;
      if (v.x != 0.0 || v.y != 0.0) {
        bl = max(bl, i % m - i / m);
        bu = max(bu, i / m - i % m);
      }
    }
    if (bl) atomicMax(&piv[0], bl);
    if (bu) atomicMax(&piv[1], bu);
  }
  expm_sync<WARP>();
  const int l1 = piv[0], u1 = piv[1];
  const int l2 = min(2 * l1, m - 1), u2 = min(2 * u1, m - 1);
  const int l4 = min(2 * l2, m - 1), u4 = min(2 * u2, m - 1);
  const int l6 = min(l4 + l2, m - 1), u6 = min(u4 + u2, m - 1);
  const int lN = max(l6, min(l1 + l4, m - 1)), uN = max(u6, min(u1 + u4, m - 1));
  // L-infinity norm (mat_norm_linf :89-104): the row's band in column order
  // (the entries outside add exact zeros)
  for (int i = tid; i < m; i += nt) {
    double s = 0.0;
    for (int j = max(0, i - l1); j <= min(m - 1, i + u1); ++j) s += hypot(A2[i + j * m].x, A2[i + j * m].y);
    rowsum[i] = s;
  }
  expm_sync<WARP>();
  if (tid < 32) {
    // the largest row sum by a warp maximum (exact: the same value in any order)
    double an = 0.0;
    for (int i = tid; i < m; i += 32) an = fmax(an, rowsum[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) an = fmax(an, __shfl_xor_sync(0xffffffffu, an, o));
    if (tid == 0) {
      int s = 0;
      if (an > 0.0) {
        const double l2 = log(an) / log(2.0);  // log_2 (:106-117)
        const int ee = (int)l2 + 1;            // int() truncates toward zero
        s = max(0, ee + 1);
      }
      *s_sh = s;
    }
  }
  expm_sync<WARP>();
  const int s = *s_sh;
  const double sc = ldexp(1.0, -s);  // A/2**s, exact
  for (int i = tid; i < mm; i += nt) A2[i] = make_double2(A2[i].x * sc, A2[i].y * sc);
  expm_sync<WARP>();
  // Pade(6,6) numerator N = sum c_k a^k and denominator D = sum (-1)^k c_k a^k
  // with the reference's coefficient recurrence (:54-77), evaluated from the
  // even and odd parts (Paterson-Stockmeyer): a^2, a^4, a^6 and
  // a (c1 + c3 a^2 + c5 a^4), four products instead of five
  constexpr double ck[7] = {pade6_coef(0), pade6_coef(1), pade6_coef(2), pade6_coef(3),
                            pade6_coef(4), pade6_coef(5), pade6_coef(6)};
  smem_matmul_band(m, A2, l1, u1, A2, l1, u1, X, tid, nt);  // a^2
  expm_sync<WARP>();
  smem_matmul_band(m, X, l2, u2, X, l2, u2, T, tid, nt);    // a^4
  expm_sync<WARP>();
  smem_matmul_band(m, T, l4, u4, X, l2, u2, D, tid, nt);    // a^6
  expm_sync<WARP>();
  for (int i = tid; i < mm; i += nt) {
    const double id = (i % (m + 1) == 0) ? 1.0 : 0.0;
    const double2 x2 = X[i], x4 = T[i], x6 = D[i];
    E[i] = make_double2(id + ck[2] * x2.x + ck[4] * x4.x + ck[6] * x6.x, ck[2] * x2.y + ck[4] * x4.y + ck[6] * x6.y);
    D[i] = make_double2(id * ck[1] + ck[3] * x2.x + ck[5] * x4.x, ck[3] * x2.y + ck[5] * x4.y);
  }
  expm_sync<WARP>();
  smem_matmul_band(m, A2, l1, u1, D, l4, u4, X, tid, nt);   // odd part
  expm_sync<WARP>();
  for (int i = tid; i < mm; i += nt) {
    const double2 ev = E[i], od = X[i];
    T[i] = cadd(ev, od);  // N
    D[i] = csub(ev, od);  // D
    X[i] = D[i];          // kept for a dense restart of the LU
  }
  expm_sync<WARP>();
  // LU of D with partial pivoting (|re|+|im| pivot, as izamax), in place, on
  // the bands (lN, uN) while every pivot is the diagonal: then no row moves,
  // the unit-lower factor keeps bandwidth lN and the upper one uN. The
  // multipliers l_ik = D_ik / D_kk (formed with the pivot's reciprocal in the
  // same pass as the trailing update) go to the spent A2.
  bool swapped = false;
  for (int k = 0; k < m; ++k) {
    const int ie = min(k + lN, m - 1), je = min(k + uN, m - 1);
    if (tid < 32) {
      // non-negative doubles order as their bit patterns: integer compares
      long long best = -1;
      int bi = k;
      for (int i = k + tid; i <= ie; i += 32) {
        const long long v = __double_as_longlong(fabs(D[i + k * m].x) + fabs(D[i + k * m].y));
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const long long ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (tid == 0) {
        *p_sh = bi;
        piv[k] = bi;
        if (best == 0) atomicExch(err, 2);
      }
    }
    expm_sync<WARP>();
    if (*p_sh != k) {  // a row swap: the bands no longer hold
      swapped = true;
      break;
    }
    const int ri = ie - k, rj = je - k + 1;  // rows k+1..ie, columns k..je
    for (int idx = tid; idx < ri * rj; idx += nt) {
      const int i = k + 1 + idx % ri, j = k + idx / ri;
      const double2 l = cmul(D[i + k * m], crcp(D[k + k * m]));
      if (j == k)
        A2[i + k * m] = l;
      else
        D[i + j * m] = cfms(l, D[k + j * m], D[i + j * m]);
    }
    expm_sync<WARP>();
  }
  if (swapped) {
    // dense restart from the saved denominator
    for (int i = tid; i < mm; i += nt) D[i] = X[i];
    expm_sync<WARP>();
  }
  const int lL = swapped ? m - 1 : lN, uU = swapped ? m - 1 : uN;
  for (int k = 0; swapped && k < m; ++k) {
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
        *p_sh = bi;
        piv[k] = bi;
        if (best == 0.0) atomicExch(err, 2);
      }
    }
    expm_sync<WARP>();
    const int pr = *p_sh;
    if (pr != k)
      for (int j = tid; j < m; j += nt) {
        const double2 t0 = D[k + j * m];
        D[k + j * m] = D[pr + j * m];
        D[pr + j * m] = t0;
      }
    expm_sync<WARP>();
    const double2 dkk = D[k + k * m];
    for (int i = k + 1 + tid; i < m; i += nt) D[i + k * m] = cdiv(D[i + k * m], dkk);
    expm_sync<WARP>();
    const int rem = m - k - 1;
    for (int idx = tid; idx < rem * rem; idx += nt) {
      const int i = k + 1 + idx % rem, j = k + 1 + idx / rem;
      D[i + j * m] = cfms(D[i + k * m], D[k + j * m], D[i + j * m]);
    }
    expm_sync<WARP>();
  }
  // E = D^-1 N: the rows of N permuted as the LU's row swaps (P N), then the
  // unit-lower and the upper triangular solves of all m columns as rank-1
  // updates over every (row, column) at once, one sync per step
  int* perm = reinterpret_cast<int*>(rowsum);  // the row sums are spent
  if (tid == 0) {
    for (int i = 0; i < m; ++i) perm[i] = i;
    for (int k = 0; k < m; ++k) {
      const int a = perm[k];
      perm[k] = perm[piv[k]];
      perm[piv[k]] = a;
    }
  }
  expm_sync<WARP>();
  for (int idx = tid; idx < mm; idx += nt) E[idx] = T[perm[idx % m] + (idx / m) * m];
  expm_sync<WARP>();
  // (the factors' entries outside their bands are exact zeros; the band
  // path's multipliers are in A2, whose diagonal then takes the pivots'
  // reciprocals for the upper solve)
  const double2* Lf = swapped ? D : A2;
  for (int k = 0; k + 1 < m; ++k) {
    const int rem = min(lL, m - k - 1);
    for (int idx = tid; idx < rem * m; idx += nt) {
      const int i = k + 1 + idx % rem, j = idx / rem;
      E[i + j * m] = cfms(Lf[i + k * m], E[k + j * m], E[i + j * m]);
    }
    expm_sync<WARP>();
  }
  if (!swapped) {
    for (int k = tid; k < m; k += nt) A2[k + k * m] = crcp(D[k + k * m]);
    expm_sync<WARP>();
  }
  if (swapped) {
    for (int k = m - 1; k >= 0; --k) {
      for (int j = tid; j < m; j += nt) E[k + j * m] = cdiv(E[k + j * m], D[k + k * m]);
      expm_sync<WARP>();
      for (int idx = tid; idx < k * m; idx += nt) {
        const int i = idx % k, j = idx / k;
        E[i + j * m] = cfms(D[i + k * m], E[k + j * m], E[i + j * m]);
      }
      expm_sync<WARP>();
    }
  } else {
    // one sync per step: row k's solution, E_kj times the pivot's
    // reciprocal, goes to T (N is spent), and every thread that updates a
    // row above forms the same product itself
    for (int k = m - 1; k >= 0; --k) {
      const int i0 = max(0, k - uU), ri = k - i0 + 1;  // rows i0..k
      for (int idx = tid; idx < ri * m; idx += nt) {
        const int i = i0 + idx % ri, j = idx / ri;
        const double2 ek = cmul(E[k + j * m], A2[k + k * m]);
        if (i == k)
          T[k + j * m] = ek;
        else
          E[i + j * m] = cfms(D[i + k * m], ek, E[i + j * m]);
      }
      expm_sync<WARP>();
    }
    for (int i = tid; i < mm; i += nt) E[i] = T[i];
    expm_sync<WARP>();
  }
  // s squarings
  for (int k = 0; k < s; ++k) {
    smem_matmul(m, E, E, X, tid, nt);
    expm_sync<WARP>();
    for (int i = tid; i < mm; i += nt) E[i] = X[i];
    expm_sync<WARP>();
  }
  for (int i = tid; i < mm; i += nt) out[(i % m) + (size_t)(i / m) * mld] = E[i];
}

__global__ void __launch_bounds__(128)
    k_expm(int mld, int nslots, const TileInfo* __restrict__ tiles, const int* __restrict__ map,
           const double2* __restrict__ Ahess, double2* __restrict__ Aexp, double dt,
           int* __restrict__ err) {
  extern __shared__ double2 sm[];
  __shared__ double rowsum[SPC_MAX_M];
  __shared__ int piv[SPC_MAX_M];
  __shared__ int s_sh, p_sh;
  const int w = blockIdx.x;
  if (w >= nslots || map[w] < 0) return;
  // working dimension m <= mld (the storage leading dimension)
  const int m = tiles[w / SPC_LANES].m;
  expm_one<false>(m, mld, Ahess + (size_t)w * mld * mld, Aexp + (size_t)w * mld * mld, dt, sm, rowsum, piv,
                  &s_sh, &p_sh, threadIdx.x, blockDim.x, err);
}

// Four samples per 128-thread CTA, one warp each (m <= 16); dynamic shared
// memory 4 x 5 mld^2 complex.
__global__ void __launch_bounds__(128)
    k_expm_warp(int mld, int nslots, const TileInfo* __restrict__ tiles, const int* __restrict__ map,
                const double2* __restrict__ Ahess, double2* __restrict__ Aexp, double dt,
                int* __restrict__ err) {
  extern __shared__ double2 sm[];
  __shared__ double rowsum[4][SPC_MAX_M];
  __shared__ int piv[4][SPC_MAX_M];
  __shared__ int s_sh[4], p_sh[4];
  const int g = threadIdx.x >> 5;
  const int w = blockIdx.x * 4 + g;
  if (w >= nslots || map[w] < 0) return;
  const int m = tiles[w / SPC_LANES].m;
  expm_one<true>(m, mld, Ahess + (size_t)w * mld * mld, Aexp + (size_t)w * mld * mld, dt,
                 sm + (size_t)g * 5 * mld * mld, rowsum[g], piv[g], &s_sh[g], &p_sh[g], threadIdx.x & 31, 32,
                 err);
}

// Launch of the expm of every slot: packed warps for m <= 16.
static void launch_expm(int m, int nslots, const TileInfo* tiles, const int* map, const double2* Ahess,
                        double2* Aexp, double dt, int* err, cudaStream_t st) {
  const size_t mm = (size_t)m * m;
  if (m <= 16)
    k_expm_warp<<<(nslots + 3) / 4, 128, sizeof(double2) * 20 * mm, st>>>(m, nslots, tiles, map, Ahess, Aexp,
                                                                          dt, err);
  else
    k_expm<<<nslots, 128, sizeof(double2) * 5 * mm, st>>>(m, nslots, tiles, map, Ahess, Aexp, dt, err);
}

// Shared-memory limits of both expm kernels for Krylov dimension m.
static cudaError_t set_expm_smem(int m) {
  const size_t mm = (size_t)m * m;
  cudaError_t e = cudaFuncSetAttribute(k_expm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(sizeof(double2) * 5 * mm));
  if (e == cudaSuccess && m <= 16)
    e = cudaFuncSetAttribute(k_expm_warp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(double2) * 20 * mm));
  return e;
}

// ---------------------------------------------------------------------------
// Krylov-space projectors (convert_to_krylov :469-498) as Hermitian Grams:
//   Tp = Q_b1^H Q_b1, Tm = Q_b4^H Q_b4,
//   S  = 1/2 (Q_b2 - Q_b3)^H (Q_b2 - Q_b3),  T0 = 1/2 (Q_b2 + Q_b3)^H (Q_b2 + Q_b3)
// with b1..b4 the Z-row blocks |aa>, |ab>, |ba>, |bb>. S and T0 are the
// Hermitian parts of the reference's P_S, P_T0; Re(c^H P c) is unchanged.
// Grid (slots, splits); each of the CTA's threads owns MAXC (type, i<=j)
// combinations, MAXC = ceil(ncombo / 256) exactly and the block trimmed to
// ceil(ncombo / MAXC) threads: combination slots that no thread needs would
// still issue their (predicated-off) DFMAs and hold the FP64 pipe. A
// sample with Z nuclear rows uses min(nsplit, ceil(Z/rps)) splits of about
// rps rows (proj_splits), so CTAs of an uneven batch carry similar work.
//
// Each conj(a) b is formed with three products (Gauss; Higham 1992):
//   t1 += ar br,  t2 += ai bi,  t3 += (ar - ai)(br + bi)
//   Re = t1 + t2,  Im = t3 - t1 + t2
// with ar - ai and br + bi staged once per element beside the chunk, so a
// pair costs 3 DFMA instead of 4. Chunks of PROJ_NC rows; the staged rows
// are padded to PROJ_LD elements so that the eight lanes of a 16-byte
// shared load that read consecutive basis vectors hit distinct banks.
#define PROJ_NC 16
#define PROJ_LD (PROJ_NC + 1)
__host__ __device__ __forceinline__ int proj_splits(int nsplit, int64_t rps, int64_t Z) {
  const int64_t c = (Z + rps - 1) / rps;
  return (int)(c < 1 ? 1 : (c > nsplit ? nsplit : c));
}
// dynamic shared memory of k_proj at Krylov dimension m
__host__ __device__ __forceinline__ size_t proj_smem_bytes(int m) {
  return (sizeof(double2) + 2 * sizeof(double)) * 4 * (size_t)m * PROJ_LD;
}
template <int MAXC>
__global__ void __launch_bounds__(256)
    k_proj(const TileInfo* __restrict__ tiles, const int* __restrict__ map, int m, int ncombo,
           const unsigned* __restrict__ combos, const double2* __restrict__ Q, int nsplit, int64_t rps,
           double2* __restrict__ part) {
  extern __shared__ double2 V[];  // [4][m][PROJ_LD] complex, then Re - Im and Re + Im of each
  double* Vd = (double*)(V + 4 * m * PROJ_LD);
  double* Vs = Vd + 4 * m * PROJ_LD;
  const int w = blockIdx.x;
  if (map[w] < 0) return;
  const TileInfo& Ti = tiles[w / SPC_LANES];
  const int me = Ti.m;
  const int lane = w % SPC_LANES;
  const int split = blockIdx.y;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int64_t Z = Ti.n / 4;
  const int nsp = proj_splits(nsplit, rps, Z);
  if (split >= nsp) return;
  const int64_t per = (Z + nsp - 1) / nsp;
  const int64_t n0 = (int64_t)split * per;
  const int64_t n1 = min(Z, n0 + per);
  double t1[MAXC], t2[MAXC], t3[MAXC];
  int oi[MAXC], oj[MAXC];
#pragma unroll
  for (int q = 0; q < MAXC; ++q) {
    t1[q] = t2[q] = t3[q] = 0.0;
    const int cid = tid + q * nth;
    if (cid < ncombo) {
      const unsigned cb = combos[cid];
      const int t = cb >> 16, i = (cb >> 8) & 255, j = cb & 255;
      oi[q] = (t * m + i) * PROJ_LD;
      oj[q] = (t * m + j) * PROJ_LD;
    } else {
      oi[q] = oj[q] = 0;
    }
  }
  const size_t vs = (size_t)Ti.n * SPC_LANES;
  const double2* Qt = Q + Ti.q_off + lane;
  for (int64_t c0 = n0; c0 < n1; c0 += PROJ_NC) {
    const int len = (int)min((int64_t)PROJ_NC, n1 - c0);
    for (int idx = tid; idx < m * PROJ_NC; idx += nth) {
      const int j = idx / PROJ_NC, nn = idx % PROJ_NC;
      double2 q1 = cz(), q2 = cz(), q3 = cz(), q4 = cz();
      if (nn < len && j < me) {
        const double2* base = Qt + (size_t)j * vs;
        const int64_t n = c0 + nn;
        q1 = base[(size_t)n * SPC_LANES];
        q2 = base[(size_t)(Z + n) * SPC_LANES];
        q3 = base[(size_t)(2 * Z + n) * SPC_LANES];
        q4 = base[(size_t)(3 * Z + n) * SPC_LANES];
      }
      const double2 v[4] = {q1, csub(q2, q3), cadd(q2, q3), q4};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int o = (t * m + j) * PROJ_LD + nn;
        V[o] = v[t];
        Vd[o] = v[t].x - v[t].y;
        Vs[o] = v[t].x + v[t].y;
      }
    }
    __syncthreads();
#pragma unroll 4
    for (int nn = 0; nn < len; ++nn) {
#pragma unroll
      for (int q = 0; q < MAXC; ++q)
        if (tid + q * nth < ncombo) {
          const double2 a = V[oi[q] + nn], b = V[oj[q] + nn];
          t1[q] = fma(a.x, b.x, t1[q]);
          t2[q] = fma(a.y, b.y, t2[q]);
          t3[q] = fma(Vd[oi[q] + nn], Vs[oj[q] + nn], t3[q]);
        }
    }
    __syncthreads();
  }
  double2* out = part + ((size_t)split * gridDim.x + w) * ncombo;
#pragma unroll
  for (int q = 0; q < MAXC; ++q) {
    const int cid = tid + q * nth;
    if (cid < ncombo) out[cid] = make_double2(t1[q] + t2[q], t3[q] - t1[q] + t2[q]);
  }
}

__global__ void k_proj_reduce(const TileInfo* __restrict__ tiles, int nslots, const int* __restrict__ map,
                              int m, int ncombo, int nsplit, int64_t rps, const unsigned* __restrict__ combos,
                              const double2* __restrict__ part, double2* __restrict__ proj) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)nslots * ncombo) return;
  const int w = (int)(idx / ncombo), cid = (int)(idx % ncombo);
  if (map[w] < 0) return;
  const int nsp = proj_splits(nsplit, rps, tiles[w / SPC_LANES].n / 4);
  double2 s = cz();
  for (int sp = 0; sp < nsp; ++sp) s = cadd(s, part[((size_t)sp * nslots + w) * ncombo + cid]);
  const unsigned cb = combos[cid];
  const int t = cb >> 16, i = (cb >> 8) & 255, j = cb & 255;
  if (t == 1 || t == 2) s = make_double2(0.5 * s.x, 0.5 * s.y);
  if (i == j) s.y = 0.0;  // a Gram's diagonal is real; the three-product form leaves rounding there
  double2* P = proj + ((size_t)w * 4 + t) * m * m;
  P[i + j * m] = s;
  if (i != j) P[j + i * m] = make_double2(s.x, -s.y);
}

// Orthonormality of a Lanczos basis from the projector Grams:
// max_ij |(Tp + S + T0 + Tm)_ij - delta_ij| > tol flags the slot.
#define ORTHO_TOL 1e-12
__global__ void __launch_bounds__(128)
    k_ortho_check(int m, const TileInfo* __restrict__ tiles, const int* __restrict__ map,
                  const double2* __restrict__ proj, double tol, int* __restrict__ flag) {
  __shared__ double red[128];
  const int w = blockIdx.x;
  if (map[w] < 0) return;
  const size_t mm = (size_t)m * m;
  const double2* P = proj + (size_t)w * 4 * mm;
  const int me = tiles[w / SPC_LANES].m;
  double mx = 0.0;
  for (int id = threadIdx.x; id < me * me; id += blockDim.x) {
    const int i = id % me, j = id / me;
    const size_t idx = (size_t)i + (size_t)j * m;
    const double2 g = cadd(cadd(P[idx], P[mm + idx]), cadd(P[2 * mm + idx], P[3 * mm + idx]));
    const double d = (i == j) ? 1.0 : 0.0;
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
// dt loop (src/qm_dynamics.f90:348-364), one warp per slot. Projector types
// in `proj`: 0 Tp, 1 S, 2 T0, 3 Tm; obs slots per sample: 0 S, 1 T0, 2 Tp, 3 Tm.
__global__ void __launch_bounds__(128)
    k_dtloop(int m, int nslots, int T, const TileInfo* __restrict__ tiles,
             const int* __restrict__ map, const int* __restrict__ skip,
             const double2* __restrict__ Aexp, const double2* __restrict__ proj,
             double2* __restrict__ cvec, double* __restrict__ tt, int* __restrict__ kk,
             int* __restrict__ done, double* __restrict__ obs, double dt, double t_end, double tol,
             long long* __restrict__ nsteps, int* __restrict__ err) {
  __shared__ double2 cs[4][SPC_MAX_M];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * 4 + warp;
  if (w >= nslots || map[w] < 0 || skip[w]) return;
  const int s = map[w];
  const size_t mm = (size_t)m * m;
  const double2* E = Aexp + (size_t)w * mm;
  const double2* PX = proj + (size_t)w * 4 * mm;
  double2* c = cs[warp];
  const int me = tiles[w / SPC_LANES].m;  // this job's Krylov dimension
  const bool l0 = lane < me, l1 = lane + 32 < me;
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
    for (int j = 0; j < me; ++j) {
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
      for (int j = 0; j < me; ++j) {
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
    const double2 cmv = c[me - 1];
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

// The same dt loop with 32/LPS samples per warp, LPS lanes each, for Krylov
// dimensions m <= LPS (one row of c per lane). A warp instruction costs the
// same FP64 issue time however many lanes are active, so packing small bases
// raises throughput; the group sums add the same nonzero terms in the same
// tree order as the 32-lane sum (whose extra lanes add exact zeros), so the
// results are identical to k_dtloop's. Samples of one warp may stop after
// different steps: every sync and shuffle is masked to the sample's lanes.
template <int LPS>
__global__ void __launch_bounds__(128)
    k_dtloop_packed(int m, int nslots, int T, const TileInfo* __restrict__ tiles,
                    const int* __restrict__ map, const int* __restrict__ skip,
                    const double2* __restrict__ Aexp, const double2* __restrict__ proj,
                    double2* __restrict__ cvec, double* __restrict__ tt, int* __restrict__ kk,
                    int* __restrict__ done, double* __restrict__ obs, double dt, double t_end, double tol,
                    long long* __restrict__ nsteps, int* __restrict__ err) {
  constexpr int SPW = 32 / LPS;  // samples per warp
  __shared__ double2 cs[4 * SPW][LPS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int grp = lane / LPS, gl = lane % LPS;
  const unsigned gmask = ((1u << LPS) - 1u) << (grp * LPS);
  const int w = (blockIdx.x * 4 + warp) * SPW + grp;
  if (w >= nslots || map[w] < 0 || skip[w]) return;  // the sample's whole lane group leaves
  const int s = map[w];
  const size_t mm = (size_t)m * m;
  const double2* E = Aexp + (size_t)w * mm;
  const double2* PX = proj + (size_t)w * 4 * mm;
  double2* c = cs[warp * SPW + grp];
  const int me = tiles[w / SPC_LANES].m;
  const bool l0 = gl < me;
  if (l0) c[gl] = cvec[(size_t)w * m + gl];
  __syncwarp(gmask);
  auto gsum = [&](double v) {
#pragma unroll
    for (int o = LPS / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gmask, v, o);
    return v;
  };
  double t = tt[s];
  int k = kk[s];
  double c2 = 1.0, cm2 = 0.0;
  double* o = obs + (size_t)s * 4 * T;
  const int slot[4] = {2, 0, 1, 3};  // proj type -> obs slot
  long long steps = 0;
  while (cm2 <= tol * c2 && t < t_end) {
    double2 n0 = cz();
    for (int j = 0; j < me; ++j) {
      const double2 cj = c[j];
      if (l0) n0 = cfma(E[gl + j * m], cj, n0);
    }
    __syncwarp(gmask);
    if (l0) c[gl] = n0;
    __syncwarp(gmask);
    if (k >= T) {
      if (gl == 0) atomicExch(err, 1);
      break;
    }
    for (int ty = 0; ty < 4; ++ty) {
      const double2* P = PX + ty * mm;
      double2 v0 = cz();
      for (int j = 0; j < me; ++j) {
        const double2 cj = c[j];
        if (l0) v0 = cfma(P[gl + j * m], cj, v0);
      }
      double term = 0.0;
      if (l0) term = fma(n0.x, v0.x, n0.y * v0.y);
      term = gsum(term);
      if (gl == 0) o[slot[ty] * T + k] = term;
    }
    double nn = 0.0;
    if (l0) nn = fma(n0.x, n0.x, n0.y * n0.y);
    c2 = gsum(nn);
    const double2 cmv = c[me - 1];
    cm2 = cmv.x * cmv.x + cmv.y * cmv.y;
    t = t + dt;
    k = k + 1;
    steps++;
  }
  __syncwarp(gmask);
  if (l0) cvec[(size_t)w * m + gl] = c[gl];
  if (gl == 0) {
    tt[s] = t;
    kk[s] = k;
    done[s] = (t < t_end) ? 0 : 1;
    atomicAdd((unsigned long long*)nsteps, (unsigned long long)steps);
  }
}

// The same dt loop with one sample per 128-thread CTA (m <= 32), for rounds
// with few samples in flight: a warp-wide DFMA occupies one SM sub-partition
// for many cycles, so one warp per sample leaves three of an SM's four FP64
// units idle. Every product (E c and the four projector forms) is split over
// the four warps by column ranges; the partial sums are added in warp order
// through shared memory, and warp X finishes projector X.
__global__ void __launch_bounds__(128)
    k_dtloop_mw(int m, int nslots, int T, const TileInfo* __restrict__ tiles,
                const int* __restrict__ map, const int* __restrict__ skip,
                const double2* __restrict__ Aexp, const double2* __restrict__ proj,
                double2* __restrict__ cvec, double* __restrict__ tt, int* __restrict__ kk,
                int* __restrict__ done, double* __restrict__ obs, double dt, double t_end, double tol,
                long long* __restrict__ nsteps, int* __restrict__ err) {
  __shared__ double2 c[32];
  __shared__ double2 part[4][32];
  __shared__ double2 vpart[4][4][32];
  __shared__ double s_c2, s_cm2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x;
  if (w >= nslots || map[w] < 0 || skip[w]) return;  // whole CTA
  const int s = map[w];
  const size_t mm = (size_t)m * m;
  const double2* E = Aexp + (size_t)w * mm;
  const double2* PX = proj + (size_t)w * 4 * mm;
  const int me = tiles[w / SPC_LANES].m;
  const int j0 = (me * warp) / 4, j1 = (me * (warp + 1)) / 4;  // this warp's columns
  const bool l0 = lane < me;
  if (warp == 0) c[lane] = l0 ? cvec[(size_t)w * m + lane] : cz();
  __syncthreads();
  double t = tt[s];
  int k = kk[s];
  double c2 = 1.0, cm2 = 0.0;
  double* o = obs + (size_t)s * 4 * T;
  const int slot[4] = {2, 0, 1, 3};  // proj type -> obs slot
  long long steps = 0;
  while (cm2 <= tol * c2 && t < t_end) {
    // n = E c over this warp's columns
    double2 a = cz();
    if (l0)
      for (int j = j0; j < j1; ++j) a = cfma(E[lane + j * m], c[j], a);
    part[warp][lane] = a;
    __syncthreads();
    if (warp == 0) {
      double2 n = cadd(cadd(cadd(part[0][lane], part[1][lane]), part[2][lane]), part[3][lane]);
      if (!l0) n = cz();
      c[lane] = n;
      __syncwarp();
      const double nn = warp_sum(fma(n.x, n.x, n.y * n.y));
      if (lane == 0) {
        s_c2 = nn;
        const double2 cmv = c[me - 1];
        s_cm2 = cmv.x * cmv.x + cmv.y * cmv.y;
      }
    }
    __syncthreads();
    if (k >= T) {
      if (threadIdx.x == 0) atomicExch(err, 1);
      break;
    }
    // projector forms: partial P_X n over this warp's columns, all four types
    for (int ty = 0; ty < 4; ++ty) {
      const double2* P = PX + ty * mm;
      double2 v = cz();
      if (l0)
        for (int j = j0; j < j1; ++j) v = cfma(P[lane + j * m], c[j], v);
      vpart[warp][ty][lane] = v;
    }
    __syncthreads();
    {
      const int ty = warp;
      const double2 v = cadd(cadd(cadd(vpart[0][ty][lane], vpart[1][ty][lane]), vpart[2][ty][lane]),
                             vpart[3][ty][lane]);
      const double2 n = c[lane];
      double term = l0 ? fma(n.x, v.x, n.y * v.y) : 0.0;
      term = warp_sum(term);
      if (lane == 0) o[slot[ty] * T + k] = term;
    }
    c2 = s_c2;
    cm2 = s_cm2;
    t = t + dt;
    k = k + 1;
    steps++;
  }
  __syncthreads();
  if (warp == 0 && l0) cvec[(size_t)w * m + lane] = c[lane];
  if (threadIdx.x == 0) {
    tt[s] = t;
    kk[s] = k;
    done[s] = (t < t_end) ? 0 : 1;
    atomicAdd((unsigned long long*)nsteps, (unsigned long long)steps);
  }
}

// psi[:, scol] = Q c for the tile of a pass item (src/qm_dynamics.f90:365)
__global__ void __launch_bounds__(256)
    k_psi_update(const TileInfo* __restrict__ tiles, const int2* __restrict__ items, int m,
                 const int* __restrict__ map, const int* __restrict__ scol,
                 const int* __restrict__ skip, const double2* __restrict__ Q,
                 const double2* __restrict__ cvec, double2* __restrict__ psi) {
  __shared__ double2 cs[SPC_MAX_M][SPC_LANES];
  const int2 it = items[blockIdx.x];
  const TileInfo& T = tiles[it.x];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int w = it.x * SPC_LANES + tx;
  const bool act = map[w] >= 0 && !skip[w];
  const int me = T.m;
  for (int j = ty; j < me; j += SPC_WARPS) cs[j][tx] = act ? cvec[(size_t)w * m + j] : cz();
  __syncthreads();
  if (!act) return;
  const int n = T.n;
  const size_t vs = (size_t)n * SPC_LANES;
  const double2* q = Q + T.q_off + tx;
  double2* dst = psi + T.psi_off + scol[w];
  const int stride = T.nip * SPC_WARPS;
  for (int r = it.y * SPC_WARPS + ty; r < n; r += stride) {
    double2 acc = cz();
    const double2* qr = q + (size_t)r * SPC_LANES;
    for (int j = 0; j < me; ++j) acc = cfma(qr[(size_t)j * vs], cs[j][tx], acc);
    dst[(size_t)r * T.ldp] = acc;
  }
}

// kron_vector(theta, Z_ket) for every sample of every job (src/kroenecker.f90:85-97)
struct Theta {
  double2 v[4];
};
struct JobInit {
  int64_t Z, psi_off;
  int M, ldp;
  const double2* zk;  // M x Z, sample-major
};
__global__ void k_kron_init(const JobInit* __restrict__ jobs, int j0, Theta th,
                            double2* __restrict__ psi) {
  const JobInit J = jobs[j0 + blockIdx.y];
  const int64_t total = J.Z * (int64_t)J.M;
  double2* p = psi + J.psi_off;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int s = (int)(idx % J.M);
    const int64_t n = idx / J.M;
    const double2 z = J.zk[(size_t)s * J.Z + n];
#pragma unroll
    for (int e = 0; e < 4; ++e) p[(size_t)(e * J.Z + n) * J.ldp + s] = cmul(th.v[e], z);
  }
}

__global__ void k_obs_init(int G, int T, double p0, double p1, double p2, double p3,
                           double* __restrict__ obs, double* __restrict__ tt, int* __restrict__ kk,
                           int* __restrict__ done) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= G) return;
  double* o = obs + (size_t)s * 4 * T;
  o[0] = p0;
  o[T] = p1;
  o[2 * T] = p2;
  o[3 * T] = p3;
  tt[s] = 0.0;
  kk[s] = 1;
  done[s] = 0;
}

// res%update over a job's samples in order, then res%scale(1/M)
struct JobOut {
  int base, M;
  double* out;  // 4*T
};
__global__ void k_average(const JobOut* __restrict__ jobs, int j0, int T,
                          const double* __restrict__ obs) {
  const JobOut J = jobs[j0 + blockIdx.y];
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 4 * T) return;
  const int q = idx / T, t = idx % T;
  double acc = 0.0;
  for (int s = 0; s < J.M; ++s) acc = acc + obs[((size_t)(J.base + s) * 4 + q) * T + t];
  J.out[idx] = acc * (1.0 / (double)J.M);
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

// Work items per tile, proportional to the tile's rows and summing to about
// one wave of `resident` CTAs; at least 32 rows per item.
static void plan_items(const std::vector<int>& tile_n, int resident, std::vector<int>& first,
                       std::vector<int>& count, std::vector<int2>& items) {
  int64_t W = 0;
  for (int n : tile_n) W += n;
  first.resize(tile_n.size());
  count.resize(tile_n.size());
  items.clear();
  for (size_t t = 0; t < tile_n.size(); ++t) {
    const int n = tile_n[t];
    int64_t c = W > 0 ? (int64_t)n * resident / W : 1;
    c = std::max<int64_t>(1, std::min<int64_t>(c, (n + 31) / 32));
    first[t] = (int)items.size();
    count[t] = (int)c;
    for (int q = 0; q < c; ++q) items.push_back(make_int2((int)t, q));
  }
}

#include "spc_small.cuh"

int propagate_batch(Handle* h, const double* theta, const double* init_pop,
                    const std::vector<JobSpec>& jobs, double dt, double t_end, int m, double tol,
                    int T) {
  if (h->sample_path != SPC_SAMPLE_OFF) {
    size_t smem = 0;
    if (small_path_fits(h, jobs, m, T, smem))
      return propagate_small(h, theta, init_pop, jobs, dt, t_end, m, tol, T, smem);
  }
  auto t_start = std::chrono::steady_clock::now();
  cudaStream_t st = h->stream;
  const int nj = (int)jobs.size();
  const size_t mm = (size_t)m * m;
  const int ncombo = 4 * m * (m + 1) / 2;
  // job layout: psi blocks and global sample numbering
  std::vector<int64_t> psi_off(nj);
  std::vector<int> ldp(nj), base(nj);
  int64_t psi_total = 0, qcap = 0, pcap = 0;
  int G = 0, slots_cap = 0, tiles_cap = 0;
  int64_t Zmax = 1;
  for (int k = 0; k < nj; ++k) {
    ldp[k] = (jobs[k].M + SPC_LANES - 1) / SPC_LANES * SPC_LANES;
    psi_off[k] = psi_total;
    psi_total += (int64_t)jobs[k].n * ldp[k];
    qcap += (int64_t)m * jobs[k].n * ldp[k];
    pcap += (int64_t)jobs[k].n * ldp[k];
    base[k] = G;
    G += jobs[k].M;
    slots_cap += ldp[k];
    tiles_cap += ldp[k] / SPC_LANES;
    Zmax = std::max<int64_t>(Zmax, jobs[k].n / 4);
  }
  const int nsplit_max = (int)std::max<int64_t>(1, std::min<int64_t>(16, (Zmax + 63) / 64));
  int nmax = 1;
  for (const JobSpec& j : jobs) nmax = std::max(nmax, j.n);

  // Samples in flight per build round. All of them when their Krylov bases
  // and per-sample matrices fit the device (or the handle's memory limit);
  // otherwise every round runs over consecutive chunks of whole 32-sample
  // tiles, the capacities scaled down by one factor. States, populations and
  // clocks stay resident for every sample either way.
  const double slot_fixed = 16.0 * (6.0 * mm + m + 1 + (double)nsplit_max * ncombo) + 8.0 + 4.0 + 8.0;
  // basis + work vector (complex) + the current vector's Re + Im plane (XS)
  const double need_fl = 16.0 * (double)qcap + 24.0 * (double)pcap + slot_fixed * slots_cap +
                         (double)(sizeof(TileInfo) + sizeof(unsigned)) * tiles_cap;
  const double need_global = 16.0 * (double)psi_total + 8.0 * 4.0 * (double)T * G + 16.0 * G;
  double budget;
  {
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    // a held buffer is reused up to the size this call asks of it (buffers
    // only grow), so only that much of it counts toward the budget
    double held = 0.0;
    auto reuse = [&](const Handle::Buf& b, double bytes) { held += std::min((double)b.bytes, bytes); };
    reuse(h->Q, 16.0 * (double)qcap);
    reuse(h->P, 16.0 * (double)pcap);
    reuse(h->xsum, 8.0 * (double)pcap);
    reuse(h->psi, 16.0 * (double)psi_total);
    reuse(h->obs, 8.0 * 4.0 * (double)T * G);
    const double sl = (double)slots_cap;
    reuse(h->coef, 16.0 * sl);
    reuse(h->rbeta, 8.0 * sl);
    reuse(h->Ahess, 16.0 * (double)mm * sl);
    reuse(h->Aexp, 16.0 * (double)mm * sl);
    reuse(h->proj, 64.0 * (double)mm * sl);
    reuse(h->projpart, 16.0 * (double)nsplit_max * ncombo * sl);
    reuse(h->cvec, 16.0 * m * sl);
    reuse(h->flag, 4.0 * sl);
    reuse(h->tt, 8.0 * G);
    reuse(h->kk, 4.0 * G);
    reuse(h->done, 4.0 * G);
    budget = (double)free_b + held - need_global - (512.0 * (1 << 20) + 0.02 * (double)total_b);
    if (h->mem_limit) budget = std::min(budget, (double)h->mem_limit - need_global);
  }
  int64_t qfl = qcap, pfl = pcap;
  int slots_fl = slots_cap, tiles_fl = tiles_cap;
  const bool chunked = need_fl > budget;
  if (chunked) {
    const double f = std::max(0.0, budget) / need_fl;
    qfl = std::max<int64_t>((int64_t)(f * (double)qcap), (int64_t)m * nmax * SPC_LANES);
    pfl = std::max<int64_t>((int64_t)(f * (double)pcap), (int64_t)nmax * SPC_LANES);
    tiles_fl = std::max(1, (int)(f * tiles_cap));
    slots_fl = tiles_fl * SPC_LANES;
    const double fl = 16.0 * (double)qfl + 24.0 * (double)pfl + slot_fixed * slots_fl +
                      (double)(sizeof(TileInfo) + sizeof(unsigned)) * tiles_fl;
    if (fl > budget)
      return set_error(SPC_ERR_ALLOC,
                       "one 32-sample tile of dimension %d at Krylov dimension %d needs %.3g bytes; "
                       "%.3g are available",
                       nmax, m, fl, std::max(0.0, budget));
  }
  // upper bound on work items per round: one wave of the most resident kernel plus one per tile
  const int items_cap = h->sm_count * 32 + tiles_fl;
  if (h->ensure(h->psi, sizeof(double2) * psi_total) || h->ensure(h->Q, sizeof(double2) * qfl) ||
      h->ensure(h->P, sizeof(double2) * pfl) || h->ensure(h->xsum, sizeof(double) * pfl) ||
      h->ensure(h->partial, sizeof(double2) * (size_t)items_cap * SPC_LANES) ||
      h->ensure(h->counters, sizeof(unsigned) * tiles_fl) ||
      h->ensure(h->coef, sizeof(double2) * slots_fl) || h->ensure(h->rbeta, sizeof(double) * slots_fl) ||
      h->ensure(h->Ahess, sizeof(double2) * mm * slots_fl) ||
      h->ensure(h->Aexp, sizeof(double2) * mm * slots_fl) ||
      h->ensure(h->proj, sizeof(double2) * 4 * mm * slots_fl) ||
      h->ensure(h->projpart, sizeof(double2) * (size_t)nsplit_max * slots_fl * ncombo +
                                 sizeof(unsigned) * ncombo) ||
      h->ensure(h->cvec, sizeof(double2) * m * slots_fl) || h->ensure(h->tt, sizeof(double) * G) ||
      h->ensure(h->kk, sizeof(int) * G) || h->ensure(h->done, sizeof(int) * G) ||
      h->ensure(h->obs, sizeof(double) * 4 * (size_t)T * G) || h->ensure(h->err, 16) ||
      h->ensure(h->flag, sizeof(int) * slots_fl) ||
      h->ensure(h->plan, sizeof(TileInfo) * tiles_fl + sizeof(int2) * 2 * items_cap +
                             sizeof(int) * 2 * slots_fl + 256) ||
      h->ensure(h->jobtab, (sizeof(JobInit) + sizeof(JobOut)) * nj + 64))
    return SPC_ERR_ALLOC;
  double2* d_psi = (double2*)h->psi.p;
  double2* d_Q = (double2*)h->Q.p;
  double2* d_P = (double2*)h->P.p;
  double* d_xs = (double*)h->xsum.p;
  double2* d_part = (double2*)h->partial.p;
  unsigned* d_cnt = (unsigned*)h->counters.p;
  double2* d_coef = (double2*)h->coef.p;
  double* d_rb = (double*)h->rbeta.p;
  double2* d_A = (double2*)h->Ahess.p;
  double2* d_E = (double2*)h->Aexp.p;
  double2* d_proj = (double2*)h->proj.p;
  double2* d_ppart = (double2*)h->projpart.p;
  unsigned* d_combos =
      (unsigned*)((char*)h->projpart.p + sizeof(double2) * (size_t)nsplit_max * slots_fl * ncombo);
  double2* d_c = (double2*)h->cvec.p;
  double* d_t = (double*)h->tt.p;
  int* d_k = (int*)h->kk.p;
  int* d_done = (int*)h->done.p;
  double* d_obs = (double*)h->obs.p;
  int* d_err = (int*)h->err.p;
  long long* d_nsteps = (long long*)((char*)h->err.p + 8);
  int* d_flag = (int*)h->flag.p;
  // per-round plan: tiles | pass items | SpMM items | map | scol
  char* plan = (char*)h->plan.p;
  TileInfo* d_tiles = (TileInfo*)plan;
  int2* d_items_p = (int2*)(plan + sizeof(TileInfo) * tiles_fl);
  int2* d_items_s = d_items_p + items_cap;
  int* d_map = (int*)(d_items_s + items_cap);
  int* d_scol = d_map + slots_fl;
  JobInit* d_jinit = (JobInit*)h->jobtab.p;
  JobOut* d_jout = (JobOut*)((char*)h->jobtab.p + sizeof(JobInit) * nj);

  int64_t launches0 = h->launches;
  CK(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned) * tiles_fl, st));
  CK(cudaMemsetAsync(h->err.p, 0, 16, st));
  CK(cudaMemsetAsync(d_obs, 0, sizeof(double) * 4 * (size_t)T * G, st));
  CK(cudaMemsetAsync(d_flag, 0, sizeof(int) * slots_fl, st));
  CK(cudaMemsetAsync(d_psi, 0, sizeof(double2) * psi_total, st));
  {
    std::vector<unsigned> combos(ncombo);
    int id = 0;
    for (int t = 0; t < 4; ++t)
      for (int i = 0; i < m; ++i)
        for (int j = i; j < m; ++j) combos[id++] = ((unsigned)t << 16) | ((unsigned)i << 8) | (unsigned)j;
    std::vector<JobInit> ji(nj);
    std::vector<JobOut> jo(nj);
    for (int k = 0; k < nj; ++k) {
      ji[k] = JobInit{jobs[k].n / 4, psi_off[k], jobs[k].M, ldp[k], jobs[k].zk};
      jo[k] = JobOut{base[k], jobs[k].M, jobs[k].out};
    }
    CK(cudaMemcpyAsync(d_combos, combos.data(), sizeof(unsigned) * ncombo, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_jinit, ji.data(), sizeof(JobInit) * nj, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_jout, jo.data(), sizeof(JobOut) * nj, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
  }
  Theta th;
  for (int e = 0; e < 4; ++e) th.v[e] = make_double2(theta[2 * e], theta[2 * e + 1]);
  for (int j0 = 0; j0 < nj; j0 += 65535) {
    const int cnt = std::min(65535, nj - j0);
    k_kron_init<<<dim3(std::max(1, h->sm_count * 8 / std::max(1, cnt)), cnt), 256, 0, st>>>(
        d_jinit, j0, th, d_psi);
    h->count_launch();
  }
  k_obs_init<<<(G + 127) / 128, 128, 0, st>>>(G, T, init_pop[0], init_pop[1], init_pop[2],
                                               init_pop[3], d_obs, d_t, d_k, d_done);
  h->count_launch();
  CK(cudaGetLastError());

  const size_t proj_smem = proj_smem_bytes(m);
  CK(set_expm_smem(m));
  // combinations per thread (an instantiated count) and threads per CTA (a
  // multiple of 32, at most 256): the pair with the fewest padded slots, the
  // smaller count on a tie (every slot, used or not, issues its DFMAs)
  static const int kProjMaxc[] = {1, 2, 3, 4, 5, 6, 7, 8, 10, 12, 16, 20, 24};
  int maxc = 24, proj_threads = 256;
  {
    int64_t best = -1;
    for (int c : kProjMaxc) {
      const int th = ((ncombo + c - 1) / c + 31) / 32 * 32;
      if (th > 256) continue;
      const int64_t slots = (int64_t)c * th;
      if (best < 0 || slots < best) {
        best = slots;
        maxc = c;
        proj_threads = th;
      }
    }
  }
  const void* proj_fn = nullptr;
  switch (maxc) {
    case 1: proj_fn = (const void*)k_proj<1>; break;
    case 2: proj_fn = (const void*)k_proj<2>; break;
    case 3: proj_fn = (const void*)k_proj<3>; break;
    case 4: proj_fn = (const void*)k_proj<4>; break;
    case 5: proj_fn = (const void*)k_proj<5>; break;
    case 6: proj_fn = (const void*)k_proj<6>; break;
    case 7: proj_fn = (const void*)k_proj<7>; break;
    case 8: proj_fn = (const void*)k_proj<8>; break;
    case 10: proj_fn = (const void*)k_proj<10>; break;
    case 12: proj_fn = (const void*)k_proj<12>; break;
    case 16: proj_fn = (const void*)k_proj<16>; break;
    case 20: proj_fn = (const void*)k_proj<20>; break;
    default: proj_fn = (const void*)k_proj<24>; break;
  }
  CK(cudaFuncSetAttribute(proj_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)proj_smem));
  // resident CTAs per kernel: item lists are sized to whole waves
  auto resident = [&](const void* fn, int threads, size_t smem) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, threads, smem) != cudaSuccess) b = 1;
    return std::max(1, b) * h->sm_count;
  };
  const int res_spmm = resident((const void*)k_spmm, 256, 0);
  const int res_pass = std::min(resident((const void*)k_rowpass<PASS_AXPY_DOT>, 256, 0),
                                resident((const void*)k_rowpass<PASS_AXPY_NORM>, 256, 0));
  const int res_proj = resident(proj_fn, proj_threads, proj_smem);

  std::vector<int> active;
  if (0.0 < t_end)
    for (int g = 0; g < G; ++g) active.push_back(g);
  std::vector<int> job_of(G);
  for (int k = 0; k < nj; ++k)
    for (int s = 0; s < jobs[k].M; ++s) job_of[base[k] + s] = k;
  std::vector<int> done_h(G, 0), flag_h(slots_fl, 0);
  int64_t builds = 0, rounds = 0, fallbacks = 0;
  const dim3 blk(SPC_LANES, SPC_WARPS);
  bool lanczos_ok = h->krylov_method == 1 || h->krylov_method == 2;
  for (const JobSpec& j : jobs) lanczos_ok = lanczos_ok && j.herm_shift;
  std::vector<char> hplan;
  // round graphs of this call: plan shape -> (executable graph, launches in it)
  struct GraphCache : std::map<std::vector<int64_t>, std::pair<cudaGraphExec_t, int64_t>> {
    ~GraphCache() {
      for (auto& kv : *this) cudaGraphExecDestroy(kv.second.first);
    }
  } graph_cache;
  std::set<std::vector<int64_t>> shapes_seen;

  // One build round for the samples in `list` (global indices, job order):
  // Krylov basis (Lanczos or full MGS), expm, projectors; then the dt loop and
  // psi = Q c for every sample whose basis passed the orthogonality check.
  // Returns the samples that failed it (Lanczos only); their state is left
  // untouched.
  auto round = [&](const std::vector<int>& list, bool lanczos, std::vector<int>& failed) -> int {
    failed.clear();
    // tiles: each job's samples in this list, in groups of 32
    std::vector<TileInfo> tiles;
    std::vector<int> map, scol, tile_n;
    int64_t qo = 0, po = 0;
    size_t a = 0;
    double elems = 0.0;
    while (a < list.size()) {
      const int k = job_of[list[a]];
      size_t b = a;
      while (b < list.size() && job_of[list[b]] == k) ++b;
      for (size_t c = a; c < b; c += SPC_LANES) {
        TileInfo ti{};
        ti.job = k;
        ti.n = jobs[k].n;
        ti.ldp = ldp[k];
        ti.q_off = qo;
        ti.p_off = po;
        ti.psi_off = psi_off[k];
        ti.rowptr = jobs[k].rowptr;
        ti.split = jobs[k].split;
        ti.col = jobs[k].col;
        ti.val = jobs[k].val;
        ti.vsum = jobs[k].vsum;
        ti.kappa = jobs[k].herm_shift ? jobs[k].kappa : nullptr;
        ti.m = std::min(m, ti.n);
        qo += (int64_t)m * ti.n * SPC_LANES;
        po += (int64_t)ti.n * SPC_LANES;
        for (int l = 0; l < SPC_LANES; ++l) {
          if (c + l < b) {
            map.push_back(list[c + l]);
            scol.push_back(list[c + l] - base[k]);
          } else {
            map.push_back(-1);
            scol.push_back(-1);
          }
        }
        elems += (double)ti.n * (double)std::min<size_t>(SPC_LANES, b - c);
        tiles.push_back(ti);
        tile_n.push_back(ti.n);
      }
      a = b;
    }
    const int ntiles = (int)tiles.size();
    const int nslots = ntiles * SPC_LANES;
    std::vector<int> fp, cp, fs, cs;
    std::vector<int2> items_p, items_s;
    plan_items(tile_n, res_pass, fp, cp, items_p);
    plan_items(tile_n, res_spmm, fs, cs, items_s);
    for (int t = 0; t < ntiles; ++t) {
      tiles[t].ip0 = fp[t];
      tiles[t].nip = cp[t];
      tiles[t].is0 = fs[t];
      tiles[t].nis = cs[t];
    }
    const int nip = (int)items_p.size(), nis = (int)items_s.size();
    if (nip > items_cap || nis > items_cap || ntiles > tiles_fl || qo > qfl || po > pfl)
      return set_error(SPC_ERR_ARG, "internal: work plan exceeds its buffer");
    // one host->device copy of the plan
    const size_t off_items_p = sizeof(TileInfo) * tiles_fl;
    const size_t off_items_s = off_items_p + sizeof(int2) * items_cap;
    const size_t off_map = off_items_s + sizeof(int2) * items_cap;
    const size_t off_scol = off_map + sizeof(int) * slots_fl;
    const size_t plan_bytes = off_scol + sizeof(int) * nslots;
    hplan.resize(plan_bytes);
    std::memcpy(hplan.data(), tiles.data(), sizeof(TileInfo) * ntiles);
    std::memcpy(hplan.data() + off_items_p, items_p.data(), sizeof(int2) * nip);
    std::memcpy(hplan.data() + off_items_s, items_s.data(), sizeof(int2) * nis);
    std::memcpy(hplan.data() + off_map, map.data(), sizeof(int) * nslots);
    std::memcpy(hplan.data() + off_scol, scol.data(), sizeof(int) * nslots);
    CK(cudaMemcpyAsync(plan, hplan.data(), plan_bytes, cudaMemcpyHostToDevice, st));
    // projector splits: rows per split `rps` minimising the estimated time
    // (all rows plus a per-CTA overhead of 32 rows, over the resident CTAs,
    // plus the longest CTA); each sample takes ceil(Z/rps) splits, at most
    // nsplit_max
    int ns = 1;
    int64_t rps = 1;
    {
      int64_t zmax = 1;
      std::vector<int64_t> zact;  // Z of every active slot
      for (int t = 0; t < ntiles; ++t)
        for (int l = 0; l < SPC_LANES; ++l)
          if (map[t * SPC_LANES + l] >= 0) zact.push_back(tiles[t].n / 4);
      for (int64_t z : zact) zmax = std::max(zmax, z);
      double best = 1e300;
      for (int c = 1; c <= nsplit_max; ++c) {
        const int64_t r = (zmax + c - 1) / c;
        double rows = 0.0, ctas = 0.0;
        for (int64_t z : zact) {
          const int k = proj_splits(nsplit_max, r, z);
          ctas += k;
          rows += (double)z;
        }
        const double est = (rows + 32.0 * ctas) / res_proj + (double)r;
        if (est < best) {
          best = est;
          rps = r;
        }
      }
      for (int64_t z : zact) ns = std::max(ns, proj_splits(nsplit_max, rps, z));
    }
    // every launch of the round; captured as a CUDA graph per plan shape
    // within this call and replayed (the plan itself lives in device memory
    // and is copied before each round)
    auto enqueue = [&]() -> int {
      CK(cudaMemsetAsync(d_A, 0, sizeof(double2) * mm * nslots, st));
      CK(cudaMemsetAsync(d_flag, 0, sizeof(int) * nslots, st));
      PassArgs pa{};
      pa.tiles = d_tiles;
      pa.items = d_items_p;
      pa.m = m;
      pa.Q = d_Q;
      pa.P = d_P;
      pa.psi = d_psi;
      pa.map = d_map;
      pa.scol = d_scol;
      pa.coef = d_coef;
      pa.rbeta = d_rb;
      pa.Ahess = d_A;
      pa.cvec = d_c;
      pa.partial = d_part;
      pa.counters = d_cnt;
      pa.lanczos = lanczos ? 1 : 0;
      // SpMM work of the round: all entries (bytes) and the FP64 operations
      // issued (3 DFMA per complex entry, 2 per real one, 3 DADD per row to
      // close the three-product sums, 2 DFMA per row for the -i*kappa shift
      // of MGS rounds; a DFMA counts 2)
      int64_t nnz_work = 0;
      double spmm_flops = 0.0;
      for (const TileInfo& ti : tiles) {
        const JobSpec& J = jobs[ti.job];
        nnz_work += J.nnz;
        spmm_flops += 6.0 * (double)J.nnz_cplx + 4.0 * (double)(J.nnz - J.nnz_cplx) + 3.0 * ti.n +
                      (!lanczos && ti.kappa ? 4.0 * ti.n : 0.0);
      }
      int pe = h->prof.begin(st);
      k_rowpass<PASS_NORM_GATHER><<<nip, blk, 0, st>>>(pa);
      h->prof.end(st, pe, PK_DOT, 4.0 * elems, 16.0 * elems);
      pe = h->prof.begin(st);
      k_scale<<<nip, blk, 0, st>>>(d_tiles, d_items_p, d_map, d_scol, d_psi, d_P, 1, 0, d_rb, d_Q, d_xs);
      h->prof.end(st, pe, PK_SCALE, 2.0 * elems, 40.0 * elems);
      h->count_launch(2);
      for (int i = 0; i < m; ++i) {
        pe = h->prof.begin(st);
        k_spmm<<<nis, blk, 0, st>>>(d_tiles, d_items_s, d_map, i, d_Q, d_xs, d_P, lanczos ? 0 : 1);
        // algorithmic traffic: H (with its Re + Im) once per tile, X and its
        // Re + Im plane once, Y once
        h->prof.end(st, pe, PK_SPMM, spmm_flops * SPC_LANES, 28.0 * (double)nnz_work + 40.0 * elems);
        h->count_launch();
        pa.col_i = i;
        // MGS (get_krylov :453-456) projects p on Q_0..Q_i in order. Lanczos
        // (H_eff Hermitian up to -i*kappa) needs only Q_{i-1} (coefficient
        // beta_{i-1}, already in coef) and Q_i.
        int j0 = 0;
        if (lanczos && i > 0) {
          j0 = i - 1;
        } else {
          pa.row_j = 0;
          pa.jx = 0;
          pe = h->prof.begin(st);
          if (lanczos)
            k_rowpass<PASS_DOT, true><<<nip, blk, 0, st>>>(pa);
          else
            k_rowpass<PASS_DOT><<<nip, blk, 0, st>>>(pa);
          h->prof.end(st, pe, PK_DOT, (lanczos ? 4.0 : 8.0) * elems, 32.0 * elems);
          h->count_launch();
        }
        for (int j = j0; j < i; ++j) {
          pa.jx = j;
          pa.jn = j + 1;
          pa.row_j = j + 1;
          pe = h->prof.begin(st);
          if (lanczos)
            k_rowpass<PASS_AXPY_DOT, true><<<nip, blk, 0, st>>>(pa);
          else
            k_rowpass<PASS_AXPY_DOT><<<nip, blk, 0, st>>>(pa);
          h->prof.end(st, pe, PK_AXPY_DOT, (lanczos ? 8.0 : 16.0) * elems, 64.0 * elems);
          h->count_launch();
        }
        if (i < m - 1) {
          pa.jx = i;
          pa.row_j = i + 1;
          pe = h->prof.begin(st);
          if (lanczos)
            k_rowpass<PASS_AXPY_NORM, true><<<nip, blk, 0, st>>>(pa);
          else
            k_rowpass<PASS_AXPY_NORM><<<nip, blk, 0, st>>>(pa);
          h->prof.end(st, pe, PK_AXPY_NORM, (lanczos ? 8.0 : 12.0) * elems, 48.0 * elems);
          pe = h->prof.begin(st);
          k_scale<<<nip, blk, 0, st>>>(d_tiles, d_items_p, d_map, d_scol, d_psi, d_P, 0, i + 1, d_rb,
                                       d_Q, d_xs);
          h->prof.end(st, pe, PK_SCALE, 2.0 * elems, 40.0 * elems);
          h->count_launch(2);
        }
      }
      double zsum = 0.0;  // sum over active slots of Z
      for (size_t c = 0; c < map.size(); ++c)
        if (map[c] >= 0) zsum += tiles[c / SPC_LANES].n / 4;
      pe = h->prof.begin(st);
      launch_expm(m, nslots, d_tiles, d_map, d_A, d_E, dt, d_err, st);
      h->prof.end(st, pe, PK_EXPM, 8.0 * (double)mm * m * 9.0 * list.size(),
                  32.0 * (double)mm * list.size());
      const dim3 pgrid(nslots, ns);
      pe = h->prof.begin(st);
      {
        void* args[] = {(void*)&d_tiles, (void*)&d_map, (void*)&m, (void*)&ncombo, (void*)&d_combos,
                        (void*)&d_Q, (void*)&ns, (void*)&rps, (void*)&d_ppart};
        CK(cudaLaunchKernel(proj_fn, pgrid, dim3(proj_threads), args, proj_smem, st));
      }
      // 3 DFMA per (pair, row), 12 DADD per (vector, row) to stage the four
      // vector types with their Re - Im and Re + Im
      h->prof.end(st, pe, PK_PROJ, 6.0 * (double)ncombo * zsum + 12.0 * (double)m * zsum,
                  64.0 * (double)m * zsum);
      {
        const int64_t tot = (int64_t)nslots * ncombo;
        pe = h->prof.begin(st);
        k_proj_reduce<<<(int)((tot + 255) / 256), 256, 0, st>>>(d_tiles, nslots, d_map, m, ncombo, ns, rps, d_combos,
                                                               d_ppart, d_proj);
        h->prof.end(st, pe, PK_PROJ_REDUCE, 2.0 * tot * ns, 16.0 * tot * (ns + 1));
        h->count_launch(3);
      }
      if (lanczos) {
        // G = Q^H Q = Tp + S + T0 + Tm; a basis that drifted from orthonormal
        // beyond ORTHO_TOL is rebuilt with full MGS
        k_ortho_check<<<nslots, 128, 0, st>>>(m, d_tiles, d_map, d_proj, ORTHO_TOL, d_flag);
        h->count_launch();
      }
      pe = h->prof.begin(st);
      if (m <= 32 && (int64_t)list.size() * 2 <= (int64_t)h->sm_count * 4)
        k_dtloop_mw<<<nslots, 128, 0, st>>>(m, nslots, T, d_tiles, d_map, d_flag, d_E, d_proj, d_c, d_t, d_k,
                                            d_done, d_obs, dt, t_end, tol, d_nsteps, d_err);
      else if (m <= 8)
        k_dtloop_packed<8><<<(nslots + 15) / 16, 128, 0, st>>>(m, nslots, T, d_tiles, d_map, d_flag, d_E, d_proj,
                                                                d_c, d_t, d_k, d_done, d_obs, dt, t_end, tol,
                                                                d_nsteps, d_err);
      else if (m <= 16)
        k_dtloop_packed<16><<<(nslots + 7) / 8, 128, 0, st>>>(m, nslots, T, d_tiles, d_map, d_flag, d_E, d_proj,
                                                               d_c, d_t, d_k, d_done, d_obs, dt, t_end, tol,
                                                               d_nsteps, d_err);
      else
        k_dtloop<<<(nslots + 3) / 4, 128, 0, st>>>(m, nslots, T, d_tiles, d_map, d_flag, d_E, d_proj, d_c, d_t,
                                                   d_k, d_done, d_obs, dt, t_end, tol, d_nsteps, d_err);
      h->prof.end(st, pe, PK_DTLOOP, 0.0, 0.0);
      pe = h->prof.begin(st);
      k_psi_update<<<nip, blk, 0, st>>>(d_tiles, d_items_p, m, d_map, d_scol, d_flag, d_Q, d_c, d_psi);
      h->prof.end(st, pe, PK_PSI, 8.0 * m * elems, 16.0 * (m + 1) * elems);
      h->count_launch(2);
      CK(cudaGetLastError());
      return SPC_OK;
    };
    // a shape is captured the second time it occurs (calls whose rounds never
    // repeat a shape pay no capture)
    const std::vector<int64_t> key = {nip, nis, nslots, ns, rps, lanczos ? 1 : 0, (int64_t)list.size()};
    const bool graphs = h->use_graphs && !h->prof.on && !shapes_seen.insert(key).second;
    if (graphs) {
      auto itg = graph_cache.find(key);
      if (itg == graph_cache.end()) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int64_t l0 = h->launches;
        const int rc = enqueue();
        const cudaError_t ec = cudaStreamEndCapture(st, &g);
        if (rc) {
          if (g) cudaGraphDestroy(g);
          return rc;
        }
        if (ec != cudaSuccess) return set_error(SPC_ERR_CUDA, "round capture failed: %s", cudaGetErrorString(ec));
        const cudaError_t ei = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) return set_error(SPC_ERR_CUDA, "round graph instantiation failed: %s",
                                               cudaGetErrorString(ei));
        itg = graph_cache.emplace(key, std::make_pair(ge, h->launches - l0)).first;
        h->launches = l0;  // counted when the graph runs
      }
      CK(cudaGraphLaunch(itg->second.first, st));
      h->count_launch((int)itg->second.second);
    } else {
      const int rc = enqueue();
      if (rc) return rc;
    }
    if (lanczos) {
      CK(cudaMemcpyAsync(flag_h.data(), d_flag, sizeof(int) * nslots, cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      for (int w = 0; w < nslots; ++w)
        if (map[w] >= 0 && flag_h[w]) failed.push_back(map[w]);
    }
    return SPC_OK;
  };

  // end of the chunk of `list` starting at a: whole tiles (a job's run of
  // samples in groups of 32, as the round forms them) while the Krylov
  // bases, work vectors and tiles stay within the in-flight capacities
  auto chunk_end = [&](const std::vector<int>& list, size_t a) -> size_t {
    if (!chunked) return list.size();
    int64_t q = 0, p = 0;
    int nt = 0;
    size_t c = a;
    while (c < list.size()) {
      const int k = job_of[list[c]];
      size_t e = c;
      while (e < list.size() && job_of[list[e]] == k && e - c < (size_t)SPC_LANES) ++e;
      const int64_t dq = (int64_t)m * jobs[k].n * SPC_LANES, dp = (int64_t)jobs[k].n * SPC_LANES;
      if (nt > 0 && (q + dq > qfl || p + dp > pfl || nt + 1 > tiles_fl)) break;
      q += dq;
      p += dp;
      ++nt;
      c = e;
    }
    return c;
  };

  std::vector<int> failed, failed2, chunk;
  while (!active.empty()) {
    for (size_t a = 0; a < active.size();) {
      const size_t b = chunk_end(active, a);
      chunk.assign(active.begin() + a, active.begin() + b);
      a = b;
      int rc = round(chunk, lanczos_ok, failed);
      if (rc) return rc;
      builds += (int64_t)chunk.size() - (int64_t)failed.size();
      if (!failed.empty()) {
        fallbacks += (int64_t)failed.size();
        rc = round(failed, false, failed2);
        if (rc) return rc;
        builds += (int64_t)failed.size();
      }
    }
    CK(cudaMemcpyAsync(done_h.data(), d_done, sizeof(int) * G, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    h->prof.collect();
    rounds++;
    std::vector<int> next;
    next.reserve(active.size());
    for (int g : active)
      if (!done_h[g]) next.push_back(g);
    active.swap(next);
  }
  for (int j0 = 0; j0 < nj; j0 += 65535) {
    const int cnt = std::min(65535, nj - j0);
    k_average<<<dim3((4 * T + 255) / 256, cnt), 256, 0, st>>>(d_jout, j0, T, d_obs);
    h->count_launch();
  }
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

// The single-Hamiltonian call: one job on the handle's Hamiltonian.
int propagate(Handle* h, const double* theta, const double* init_pop, const double* zk_dev, int M,
              double dt, double t_end, int m, double tol, double* out_dev, int T) {
  JobSpec j{};
  j.n = h->n;
  j.nnz = h->nnz;
  j.M = M;
  j.rowptr = h->d_rowptr;
  j.split = (const int*)h->xsplit.p;
  j.col = (const int*)h->xcol.p;
  j.val = (const double2*)h->xval.p;
  j.vsum = (const double*)h->xvs.p;
  j.kappa = h->herm_shift ? &((const HMeta*)h->hmeta.p)->kappa : nullptr;
  j.nnz_cplx = h->nnz_cplx;
  j.zk = (const double2*)zk_dev;
  j.out = out_dev;
  j.herm_shift = h->herm_shift;
  return propagate_batch(h, theta, init_pop, std::vector<JobSpec>{j}, dt, t_end, m, tol, T);
}

#include "spc_adjoint.cuh"

}  // namespace spc
