// Device-side sparse Hamiltonian assembly.
//
// Both builders generate CSR rows directly from the Kronecker structure of
// the radical-pair basis (row = e*Z + n, electron state e = 2*s1 + s2 with
// s = 0 for m = +1/2, nuclear index n row-major over radical-1 then radical-2
// nuclei, each from m = +I down). A row's entries are computed by one thread;
// counts -> exclusive scan -> fill.
//
// SPC_H_REFERENCE reproduces getHiso_sp (src/hamiltonian.f90:17-205) followed
// by coo_to_csr (src/utils.f90:52-89): the same nonzeros (explicit zeros
// included), the same values rounded at the same points (no FMA contraction:
// __dmul_rn/__dadd_rn), and the same within-row order, which is the reverse
// of the order the COO blocks are appended in:
//   diag | S1+S2- | S1-S2+ | per radical-1 nucleus: S1+I-, S1-I+ | per
//   radical-2 nucleus: S2+I-, S2-I+
// SPC_H_GENERAL is the anisotropic extension (no sparse reference
// counterpart): every S_r I_c product of S.A.I, nuclear Zeeman along the
// field vector, the full electron-electron tensor; columns ascending, fixed
// structural pattern.
#include "spc_common.cuh"
#include "spc_internal.h"

namespace spc {

// ---- exact (uncontracted) complex arithmetic -------------------------------
__device__ __forceinline__ double2 xmul(double2 a, double2 b) {
  return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                      __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 xadd(double2 a, double2 b) {
  return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y));
}
__device__ __forceinline__ double2 xrscale(double s, double2 a) {
  return make_double2(__dmul_rn(s, a.x), __dmul_rn(s, a.y));
}

// nuclear state of nucleus j in nuclear index n
__device__ __forceinline__ int nuc_state(const NucInfo& q, int64_t n) {
  return (int)((n / q.stride) % q.g);
}

// Spin-I ladder element sqrt(S(S+1) - m_a m_b) as get_spinop_sp computes it
// (src/spinop.f90:88-92): m values S, S-1, ...; S(S+1) minus the complex
// product of the two Sz entries.
__device__ __forceinline__ double ladder(int g, int a, int b) {
  double S = ((double)g - 1.0) / 2.0;
  double ma = S - (double)a, mb = S - (double)b;
  return __dsqrt_rn(__dsub_rn(__dmul_rn(S, __dadd_rn(S, 1.0)), __dmul_rn(ma, mb)));
}

// ---------------------------------------------------------------------------
// reference builder
__device__ int ref_row_count(int64_t row, int64_t Z, int nn, const NucInfo* nuc) {
  int e = (int)(row / Z);
  int64_t n = row - (int64_t)e * Z;
  int s1 = e >> 1, s2 = e & 1;
  int cnt = 1 + (e == 1) + (e == 2);
  for (int j = 0; j < nn; ++j) {
    const NucInfo& q = nuc[j];
    int a = nuc_state(q, n);
    int s = q.owner == 0 ? s1 : s2;
    // S+ I- : electron up (s == 0), nucleus not at the top (a >= 1)
    if (s == 0 && a >= 1) cnt++;
    // S- I+ : electron down, nucleus not at the bottom
    if (s == 1 && a <= q.g - 2) cnt++;
  }
  return cnt;
}

__global__ void k_ref_count(int64_t N, int64_t Z, int nn, const NucInfo* __restrict__ nuc,
                            int* __restrict__ cnt) {
  int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= N) return;
  cnt[row] = ref_row_count(row, Z, nn, nuc);
}

__global__ void k_ref_fill(int64_t N, int64_t Z, int nn, const NucInfo* __restrict__ nuc,
                           RefElectron el, const int* __restrict__ rowptr, int* __restrict__ col,
                           double2* __restrict__ val) {
  int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= N) return;
  int e = (int)(row / Z);
  int64_t n = row - (int64_t)e * Z;
  int s1 = e >> 1, s2 = e & 1;
  int k = rowptr[row];
  // reverse COO block order: last nucleus of radical 2 first
  for (int j = nn - 1; j >= 0; --j) {
    const NucInfo& q = nuc[j];
    int a = nuc_state(q, n);
    int s = q.owner == 0 ? s1 : s2;
    int eflip = q.owner == 0 ? 2 : 1;  // electron-index offset of a spin flip
    // block S- I+ (appended after S+ I-, so it comes first here)
    if (s == 1 && a <= q.g - 2) {
      double2 v = xmul(make_double2(q.a_half, 0.0), make_double2(ladder(q.g, a, a + 1), 0.0));
      col[k] = (int)((int64_t)(e - eflip) * Z + n + q.stride);
      val[k] = v;
      k++;
    }
    if (s == 0 && a >= 1) {
      double2 v = xmul(make_double2(q.a_half, 0.0), make_double2(ladder(q.g, a, a - 1), 0.0));
      col[k] = (int)((int64_t)(e + eflip) * Z + n - q.stride);
      val[k] = v;
      k++;
    }
  }
  if (e == 2) {  // S1- S2+ : |ba> -> |ab>
    col[k] = (int)(1 * Z + n);
    val[k] = el.flip_ba;
    k++;
  }
  if (e == 1) {  // S1+ S2- : |ab> -> |ba>
    col[k] = (int)(2 * Z + n);
    val[k] = el.flip_ab;
    k++;
  }
  // diagonal: electronic part, then each nucleus in assembly order
  double2 d = el.diag[e];
  for (int j = 0; j < nn; ++j) {
    const NucInfo& q = nuc[j];
    int a = nuc_state(q, n);
    int s = q.owner == 0 ? s1 : s2;
    double sz = s == 0 ? 0.5 : -0.5;
    double2 x = xadd(xrscale(q.a_iso, make_double2(sz, 0.0)), xrscale(q.zf, make_double2(1.0, 0.0)));
    double S = ((double)q.g - 1.0) / 2.0;
    double m = S - (double)a;
    d = xadd(d, xmul(x, make_double2(m, 0.0)));
  }
  col[k] = (int)row;
  val[k] = d;
}

// ---------------------------------------------------------------------------
// general builder (mirrors the ascending-column generator of the oracle)
__device__ int gen_row_count(int64_t row, int64_t Z, int nn, const NucInfo* nuc) {
  int64_t n = row % Z;
  int cnt = 4;
  for (int j = 0; j < nn; ++j) {
    int a = nuc_state(nuc[j], n);
    int nb = (a > 0) + (a < nuc[j].g - 1);
    cnt += 2 * nb;
  }
  return cnt;
}

__global__ void k_gen_count(int64_t N, int64_t Z, int nn, const NucInfo* __restrict__ nuc,
                            int* __restrict__ cnt) {
  int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= N) return;
  cnt[row] = gen_row_count(row, Z, nn, nuc);
}

// One thread per row, every entry written straight to its place in the
// ascending-column row. Row (e, n) has, for each electron state ep, the block
// of columns ep*Z + n + delta: delta = -stride_j for the nuclei j (ascending)
// that S_k.A.I_j lowers, then delta = 0 (the electronic entry, plus every
// term that keeps the nuclear state, added in nucleus order), then
// delta = +stride_j for the nuclei (descending) that it raises. Strides of
// nuclei with multiplicity >= 2 are distinct and |delta| < Z, so this is the
// sorted order and no column repeats.
// Entry values come from the host-built tables (HostSystem::gen_tab), which
// hold every nucleus' matrix elements rounded as the per-row arithmetic would
// round them: a row does no FP64 work of its own, which would dominate a
// build on a part with a narrow FP64 pipe.
__global__ void k_gen_fill_tab(int64_t N, int64_t Z, int nn, const NucInfo* __restrict__ nuc,
                               GenElectron el, const double2* __restrict__ tab,
                               const int* __restrict__ rowptr, int* __restrict__ col,
                               double2* __restrict__ val) {
  int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= N) return;
  int e = (int)(row / Z);
  int64_t nidx = row - (int64_t)e * Z;
  int base = rowptr[row];
  auto couples = [&](int k, int ep) { return k == 0 ? ((e & 1) == (ep & 1)) : ((e >> 1) == (ep >> 1)); };
  int nminus[4] = {0, 0, 0, 0}, nplus[4] = {0, 0, 0, 0};
  for (int j = 0; j < nn; ++j) {
    const NucInfo& q = nuc[j];
    const int mj = nuc_state(q, nidx);
    for (int ep = 0; ep < 4; ++ep)
      if (couples(q.owner, ep)) {
        nminus[ep] += mj > 0;
        nplus[ep] += mj < q.g - 1;
      }
  }
  int off[4];
  off[0] = base;
  for (int ep = 1; ep < 4; ++ep) off[ep] = off[ep - 1] + nminus[ep - 1] + 1 + nplus[ep - 1];
  double2 d[4];
  for (int ep = 0; ep < 4; ++ep) d[ep] = el.H[e][ep];
  int seen_minus[4] = {0, 0, 0, 0}, seen_plus[4] = {0, 0, 0, 0};
  for (int j = 0; j < nn; ++j) {
    const NucInfo& q = nuc[j];
    const int g = q.g, k = q.owner;
    const int mj = nuc_state(q, nidx);
    for (int mp = mj - 1; mp <= mj + 1; ++mp) {
      if (mp < 0 || mp >= g) continue;
      const int64_t nc = nidx + (int64_t)(mp - mj) * q.stride;
      for (int ep = 0; ep < 4; ++ep) {
        if (!couples(k, ep)) continue;
        const double2 v = tab[q.tab_off + ((int64_t)(e * 4 + ep) * g + mj) * 3 + (mp - mj + 1)];
        int pos;
        if (mp == mj) {
          d[ep] = xadd(d[ep], v);
          continue;
        } else if (mp < mj) {
          pos = off[ep] + seen_minus[ep]++;
        } else {
          pos = off[ep] + nminus[ep] + 1 + (nplus[ep] - 1 - seen_plus[ep]++);
        }
        col[pos] = (int)((int64_t)ep * Z + nc);
        val[pos] = v;
      }
    }
  }
  for (int ep = 0; ep < 4; ++ep) {
    col[off[ep] + nminus[ep]] = (int)((int64_t)ep * Z + nidx);
    val[off[ep] + nminus[ep]] = d[ep];
  }
}

// Exclusive scan of per-row counts into rowptr (one CTA of 1024 threads).
__global__ void k_scan_rows(const int* __restrict__ cnt, int* __restrict__ rowptr, int64_t N,
                            long long* __restrict__ total) {
  __shared__ long long s[1024];
  long long carry = 0;
  for (int64_t base = 0; base < N; base += 1024) {
    int64_t i = base + threadIdx.x;
    long long v = i < N ? cnt[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      long long t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < N) rowptr[i] = (int)(carry + s[threadIdx.x] - v);
    long long blk = s[1023];
    __syncthreads();
    carry += blk;
  }
  if (threadIdx.x == 0) {
    rowptr[N] = (int)carry;
    *total = carry;
  }
}

// ---------------------------------------------------------------------------
// Builds of one or many systems into caller-placed CSR slices, in two phases
// with one synchronisation each: count + scan for every system, a check of
// every nonzero count against its closed form (so the fill never writes past
// the space reserved for it), then fill + row split for every system.
struct BuildSlice {
  const HostSystem* hs;
  const NucInfo* nuc;   // device nucleus table
  const double2* tab;   // device entry tables (general builder)
  int* cnt;             // N per-row counts (scratch)
  int* rowptr;          // N + 1
  int* col;             // fill target (nnz)
  double2* val;
  int* xcol;            // execution-order copy for k_spmm (nnz)
  double2* xval;
  double* xvs;          // Re + Im of every entry of the copy (nnz)
  int* split;           // N
  long long* total;     // 1
  bool herm;            // H = A - i*kappa*1: the execution copy holds A
  HMeta* meta;          // kappa and complex-entry count of the copy (zeroed)
};

static int build_slices(Handle* h, std::vector<BuildSlice>& sl, const std::vector<int64_t>& predicted,
                        int mode) {
  cudaStream_t st = h->stream;
  const int threads = 256;
  for (const BuildSlice& b : sl) {
    const int64_t N = b.hs->N, Z = b.hs->Z;
    const int nn = (int)b.hs->nuc.size();
    const int blocks = (int)((N + threads - 1) / threads);
    if (mode == SPC_H_REFERENCE)
      k_ref_count<<<blocks, threads, 0, st>>>(N, Z, nn, b.nuc, b.cnt);
    else
      k_gen_count<<<blocks, threads, 0, st>>>(N, Z, nn, b.nuc, b.cnt);
    k_scan_rows<<<1, 1024, 0, st>>>(b.cnt, b.rowptr, N, b.total);
    h->count_launch(2);
  }
  std::vector<long long> tot(sl.size());
  if (!sl.empty()) {
    // totals sit back to back (one slot per system)
    if (cudaMemcpyAsync(tot.data(), sl[0].total, sizeof(long long) * sl.size(), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return set_error(SPC_ERR_CUDA, "Hamiltonian count/scan failed: %s", cudaGetErrorString(cudaGetLastError()));
  }
  for (size_t k = 0; k < sl.size(); ++k)
    if (tot[k] != predicted[k])
      return set_error(SPC_ERR_STATE, "internal: system %zu has %lld nonzeros, %lld predicted", k, tot[k],
                       (long long)predicted[k]);
  for (const BuildSlice& b : sl) {
    const int64_t N = b.hs->N, Z = b.hs->Z;
    const int nn = (int)b.hs->nuc.size();
    const int blocks = (int)((N + threads - 1) / threads);
    if (mode == SPC_H_REFERENCE)
      k_ref_fill<<<blocks, threads, 0, st>>>(N, Z, nn, b.nuc, b.hs->ref, b.rowptr, b.col, b.val);
    else
      k_gen_fill_tab<<<blocks, threads, 0, st>>>(N, Z, nn, b.nuc, b.hs->gen, b.tab, b.rowptr, b.col, b.val);
    enqueue_split_rows(N, b.rowptr, b.col, b.val, b.xcol, b.xval, b.xvs, b.split, b.herm, b.meta, st);
    h->count_launch(2);
  }
  if (cudaStreamSynchronize(st) != cudaSuccess)
    return set_error(SPC_ERR_CUDA, "Hamiltonian fill failed: %s", cudaGetErrorString(cudaGetLastError()));
  return SPC_OK;
}

// Nucleus descriptions and entry tables of the systems back to back on the
// device (scratch in h): system k's nuclei from element off[k] of bnuc, their
// tab_off rebased onto the concatenated table in btab.
static int upload_nuclei(Handle* h, const std::vector<const HostSystem*>& hs, std::vector<size_t>& off) {
  std::vector<NucInfo> all;
  std::vector<double2> tab;
  off.resize(hs.size());
  for (size_t k = 0; k < hs.size(); ++k) {
    off[k] = all.size();
    const int64_t tb = (int64_t)tab.size();
    for (NucInfo q : hs[k]->nuc) {
      q.tab_off += tb;
      all.push_back(q);
    }
    tab.insert(tab.end(), hs[k]->gen_tab.begin(), hs[k]->gen_tab.end());
  }
  if (h->ensure(h->bnuc, sizeof(NucInfo) * std::max<size_t>(1, all.size())) ||
      h->ensure(h->btab, sizeof(double2) * std::max<size_t>(1, tab.size())))
    return SPC_ERR_ALLOC;
  if (!all.empty() &&
      cudaMemcpyAsync(h->bnuc.p, all.data(), sizeof(NucInfo) * all.size(), cudaMemcpyHostToDevice, h->stream) !=
          cudaSuccess)
    return set_error(SPC_ERR_CUDA, "nucleus table upload failed");
  if (!tab.empty() &&
      cudaMemcpyAsync(h->btab.p, tab.data(), sizeof(double2) * tab.size(), cudaMemcpyHostToDevice, h->stream) !=
          cudaSuccess)
    return set_error(SPC_ERR_CUDA, "entry table upload failed");
  // the host vectors are pageable: the copies have completed on return
  return SPC_OK;
}

int build_h_device(Handle* h, const HostSystem& hs, int mode) {
  const int64_t N = hs.N;
  const int64_t nnz = predict_nnz(hs, mode);
  if (nnz > INT32_MAX)
    return set_error(SPC_ERR_ARG, "Hamiltonian has %lld nonzeros, above the int32 CSR limit", (long long)nnz);
  std::vector<size_t> noff;
  int rc = upload_nuclei(h, {&hs}, noff);
  if (rc) return rc;
  if (h->ensure_rowptr(N + 1) || h->ensure_h_entries(nnz) || h->ensure(h->bcnt, sizeof(int) * N) ||
      h->ensure(h->btot, sizeof(long long)) || h->ensure(h->xcol, sizeof(int) * std::max<int64_t>(nnz, 1)) ||
      h->ensure(h->xval, sizeof(double2) * std::max<int64_t>(nnz, 1)) ||
      h->ensure(h->xvs, sizeof(double) * std::max<int64_t>(nnz, 1)) || h->ensure(h->xsplit, sizeof(int) * N) ||
      h->ensure(h->hmeta, sizeof(HMeta)))
    return SPC_ERR_ALLOC;
  if (cudaMemsetAsync(h->hmeta.p, 0, sizeof(HMeta), h->stream) != cudaSuccess)
    return set_error(SPC_ERR_CUDA, "Hamiltonian build failed");
  std::vector<BuildSlice> sl(1);
  sl[0] = BuildSlice{&hs, (const NucInfo*)h->bnuc.p, (const double2*)h->btab.p, (int*)h->bcnt.p, h->d_rowptr,
                     h->d_col, h->d_val,
                     (int*)h->xcol.p, (double2*)h->xval.p, (double*)h->xvs.p, (int*)h->xsplit.p,
                     (long long*)h->btot.p,
                     hs.herm_shift, (HMeta*)h->hmeta.p};
  rc = build_slices(h, sl, {nnz}, mode);
  if (rc) return rc;
  HMeta meta{};
  if (cudaMemcpy(&meta, h->hmeta.p, sizeof(HMeta), cudaMemcpyDeviceToHost) != cudaSuccess)
    return set_error(SPC_ERR_CUDA, "Hamiltonian build failed");
  h->n = (int)N;
  h->nnz = nnz;
  h->nnz_cplx = (int64_t)meta.ncplx;
  h->herm_shift = hs.herm_shift;
  return SPC_OK;
}

int build_h_batch_device(Handle* h, const std::vector<HostSystem>& hs, int mode) {
  auto& B = h->hb;
  const size_t ns = hs.size();
  B.n.assign(ns, 0);
  B.nnz.assign(ns, 0);
  B.rp_off.assign(ns, 0);
  B.nz_off.assign(ns, 0);
  B.herm.assign(ns, 0);
  int64_t rp_tot = 0, nz_tot = 0, n_tot = 0;
  std::vector<const HostSystem*> ptrs(ns);
  for (size_t k = 0; k < ns; ++k) {
    ptrs[k] = &hs[k];
    B.n[k] = (int)hs[k].N;
    B.nnz[k] = predict_nnz(hs[k], mode);
    if (B.nnz[k] > INT32_MAX)
      return set_error(SPC_ERR_ARG, "system %zu has %lld nonzeros, above the int32 CSR limit", k,
                       (long long)B.nnz[k]);
    B.rp_off[k] = rp_tot;
    B.nz_off[k] = nz_tot;
    B.herm[k] = hs[k].herm_shift;
    rp_tot += hs[k].N + 1;
    nz_tot += B.nnz[k];
    n_tot += hs[k].N;
  }
  std::vector<size_t> noff;
  int rc = upload_nuclei(h, ptrs, noff);
  if (rc) return rc;
  // fill into the unsplit scratch (xcol/xval), split into the store
  if (h->ensure(B.rowptr, sizeof(int) * rp_tot) || h->ensure(B.split, sizeof(int) * rp_tot) ||
      h->ensure(B.col, sizeof(int) * std::max<int64_t>(nz_tot, 1)) ||
      h->ensure(B.val, sizeof(double2) * std::max<int64_t>(nz_tot, 1)) ||
      h->ensure(B.vsum, sizeof(double) * std::max<int64_t>(nz_tot, 1)) ||
      h->ensure(h->xcol, sizeof(int) * std::max<int64_t>(nz_tot, 1)) ||
      h->ensure(h->xval, sizeof(double2) * std::max<int64_t>(nz_tot, 1)) ||
      h->ensure(h->bcnt, sizeof(int) * std::max<int64_t>(n_tot, 1)) || h->ensure(h->btot, sizeof(long long) * ns) ||
      h->ensure(B.meta, sizeof(HMeta) * std::max<size_t>(ns, 1)))
    return SPC_ERR_ALLOC;
  if (cudaMemsetAsync(B.meta.p, 0, sizeof(HMeta) * ns, h->stream) != cudaSuccess)
    return set_error(SPC_ERR_CUDA, "Hamiltonian build failed");
  std::vector<BuildSlice> sl(ns);
  int64_t coff = 0;
  for (size_t k = 0; k < ns; ++k) {
    sl[k] = BuildSlice{&hs[k], (const NucInfo*)h->bnuc.p + noff[k], (const double2*)h->btab.p, (int*)h->bcnt.p + coff,
                       (int*)B.rowptr.p + B.rp_off[k], (int*)h->xcol.p + B.nz_off[k],
                       (double2*)h->xval.p + B.nz_off[k], (int*)B.col.p + B.nz_off[k],
                       (double2*)B.val.p + B.nz_off[k], (double*)B.vsum.p + B.nz_off[k],
                       (int*)B.split.p + B.rp_off[k],
                       (long long*)h->btot.p + k, hs[k].herm_shift, (HMeta*)B.meta.p + k};
    coff += hs[k].N;
  }
  rc = build_slices(h, sl, B.nnz, mode);
  B.nnz_cplx.assign(ns, 0);
  if (!rc && ns) {
    std::vector<HMeta> meta(ns);
    if (cudaMemcpy(meta.data(), B.meta.p, sizeof(HMeta) * ns, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = set_error(SPC_ERR_CUDA, "Hamiltonian build failed");
    for (size_t k = 0; k < ns; ++k) B.nnz_cplx[k] = (int64_t)meta[k].ncplx;
  }
  // the single-Hamiltonian execution copy (xcol/xval) served as scratch
  h->n = 0;
  h->nnz = 0;
  return rc;
}

}  // namespace spc

// ===========================================================================
// Allocation-free Hamiltonian build (spc_build_h_noalloc).
//
// For callers that must not allocate device memory themselves or through
// the library: hosts that run inside a device-memory pool whose budget is
// fixed up front, or that only hand over buffers they own (Fortran programs,
// plugins). The caller passes the system and the CSR output buffers; the
// per-row counts, the nucleus table, the general builder's entry tables and
// the nonzero total live in the file-scope array below, which every GPU that
// loads the library holds until the process exits (about 5.2 MB).
//
// Limits: at most SPC_NOALLOC_MAX_ROWS rows (Hilbert dimension),
// SPC_NOALLOC_MAX_NUC nuclei and SPC_NOALLOC_MAX_TAB entry-table elements
// (48 per nucleus and unit of multiplicity); larger systems are rejected with
// SPC_ERR_ARG. Every call on a device shares the one array and it keeps the
// last call's contents (counts and tables are rewritten before use); calls
// that overlap on the GPU (different streams, or different host threads on
// one device) race on it and must be serialised by the caller. The call
// waits for its own stream twice (after the count and after the fill).
#include <cuda.h>

#include <mutex>

#define SPC_NOALLOC_MAX_ROWS (1 << 20)
#define SPC_NOALLOC_MAX_NUC 64
#define SPC_NOALLOC_MAX_TAB (1 << 16)
#define SPC_NOALLOC_MAX_DEVICES 64

namespace {
struct NoAllocScratch {
  int cnt[SPC_NOALLOC_MAX_ROWS];
  spc::NucInfo nuc[SPC_NOALLOC_MAX_NUC];
  double2 tab[SPC_NOALLOC_MAX_TAB];
  long long total;
};
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

// Set-up: the device address of g_noalloc_scratch, looked up with
// cudaGetSymbolAddress once per device context (with that device current)
// and kept with the context's unique id. The address belongs to the
// context: after cudaDeviceReset, or under another context of the device,
// the id differs and the address is looked up again. If the driver's
// context queries cannot be resolved, the address is looked up on every call.
typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);
static struct {
  unsigned long long ctx_id;
  void* ptr;
} g_noalloc_cache[SPC_NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mu;

static bool current_context_id(unsigned long long* id) {
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (PfnCtxGetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (PfnCtxGetId)f;
  });
  CUcontext ctx = nullptr;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}

static int noalloc_scratch(int device, NoAllocScratch** out) {
  if (device < 0 || device >= SPC_NOALLOC_MAX_DEVICES)
    return spc::set_error(SPC_ERR_ARG, "device %d above the supported range", device);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  unsigned long long id = 0;
  const bool have_id = current_context_id(&id);
  if (have_id && g_noalloc_cache[device].ptr && g_noalloc_cache[device].ctx_id == id) {
    *out = (NoAllocScratch*)g_noalloc_cache[device].ptr;
    return SPC_OK;
  }
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return spc::set_error(SPC_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed: %s",
                          cudaGetErrorString(e));
  // the lookup makes the device's primary context current if none was
  unsigned long long id2 = 0;
  if (current_context_id(&id2)) {
    g_noalloc_cache[device].ctx_id = id2;
    g_noalloc_cache[device].ptr = p;
  } else {
    g_noalloc_cache[device].ptr = nullptr;
  }
  *out = (NoAllocScratch*)p;
  return SPC_OK;
}

extern "C" int spc_build_h_noalloc(const spc_system* sys, int mode, int32_t* rowptr_dev,
                                   int32_t* col_dev, double* val_dev, int64_t cap_nnz,
                                   int32_t* n_out, int64_t* nnz_out, void* stream) {
  if (!rowptr_dev || !col_dev || !val_dev || !n_out || !nnz_out || cap_nnz < 0)
    return spc::set_error(SPC_ERR_ARG, "spc_build_h_noalloc: null output or negative capacity");
  spc::HostSystem hs;
  int rc = spc::make_host_system(sys, mode, hs);
  if (rc != SPC_OK) return rc;
  if (hs.N > SPC_NOALLOC_MAX_ROWS)
    return spc::set_error(SPC_ERR_ARG,
                          "spc_build_h_noalloc: dimension %lld above the %d rows of its scratch",
                          (long long)hs.N, SPC_NOALLOC_MAX_ROWS);
  if ((int)hs.nuc.size() > SPC_NOALLOC_MAX_NUC)
    return spc::set_error(SPC_ERR_ARG, "spc_build_h_noalloc: more than %d nuclei for its scratch",
                          SPC_NOALLOC_MAX_NUC);
  const size_t ntab = mode == SPC_H_REFERENCE ? 0 : hs.gen_tab.size();
  if (ntab > SPC_NOALLOC_MAX_TAB)
    return spc::set_error(SPC_ERR_ARG,
                          "spc_build_h_noalloc: entry tables of %zu elements above the %d of its scratch", ntab,
                          SPC_NOALLOC_MAX_TAB);
  // the closed-form count decides the size before anything is launched: a
  // capacity that is too small is refused with every output buffer untouched
  const int64_t predicted = spc::predict_nnz(hs, mode);
  if (predicted > INT32_MAX)
    return spc::set_error(SPC_ERR_ARG, "Hamiltonian has %lld nonzeros, above the int32 CSR limit",
                          (long long)predicted);
  *n_out = (int32_t)hs.N;
  *nnz_out = predicted;
  if (predicted > cap_nnz)
    return spc::set_error(SPC_ERR_ARG, "spc_build_h_noalloc: %lld nonzeros exceed the capacity %lld",
                          (long long)predicted, (long long)cap_nnz);
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess)
    return spc::set_error(SPC_ERR_CUDA, "cudaGetDevice failed");
  NoAllocScratch* scr = nullptr;
  rc = noalloc_scratch(device, &scr);
  if (rc != SPC_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t N = hs.N, Z = hs.Z;
  const int nn = (int)hs.nuc.size();
  // pageable host sources: each copy has left the host buffer on return
  if (nn > 0 && cudaMemcpyAsync(scr->nuc, hs.nuc.data(), sizeof(spc::NucInfo) * nn,
                                cudaMemcpyHostToDevice, st) != cudaSuccess)
    return spc::set_error(SPC_ERR_CUDA, "copy of the nucleus table failed");
  if (ntab > 0 && cudaMemcpyAsync(scr->tab, hs.gen_tab.data(), sizeof(double2) * ntab, cudaMemcpyHostToDevice,
                                  st) != cudaSuccess)
    return spc::set_error(SPC_ERR_CUDA, "copy of the entry tables failed");
  const int threads = 256;
  const int blocks = (int)((N + threads - 1) / threads);
  if (mode == SPC_H_REFERENCE)
    spc::k_ref_count<<<blocks, threads, 0, st>>>(N, Z, nn, scr->nuc, scr->cnt);
  else
    spc::k_gen_count<<<blocks, threads, 0, st>>>(N, Z, nn, scr->nuc, scr->cnt);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    spc::k_scan_rows<<<1, 1024, 0, st>>>(scr->cnt, rowptr_dev, N, &scr->total);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess)
    return spc::set_error(SPC_ERR_CUDA, "Hamiltonian count/scan launch failed: %s", cudaGetErrorString(e));
  // the scanned total must equal the closed form before the fill writes
  // through rowptr (it bounds every write to col/val by cap_nnz)
  long long total = -1;
  e = cudaMemcpyAsync(&total, &scr->total, sizeof(long long), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess)
    return spc::set_error(SPC_ERR_CUDA, "Hamiltonian count/scan failed: %s", cudaGetErrorString(e));
  if (total != predicted)
    return spc::set_error(SPC_ERR_STATE, "internal: %lld nonzeros counted, %lld predicted", total,
                          (long long)predicted);
  if (mode == SPC_H_REFERENCE)
    spc::k_ref_fill<<<blocks, threads, 0, st>>>(N, Z, nn, scr->nuc, hs.ref, rowptr_dev, col_dev,
                                                (double2*)val_dev);
  else
    spc::k_gen_fill_tab<<<blocks, threads, 0, st>>>(N, Z, nn, scr->nuc, hs.gen, scr->tab, rowptr_dev, col_dev,
                                                    (double2*)val_dev);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return spc::set_error(SPC_ERR_CUDA, "Hamiltonian fill launch failed: %s", cudaGetErrorString(e));
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess)
    return spc::set_error(SPC_ERR_CUDA, "Hamiltonian fill failed: %s", cudaGetErrorString(e));
  return SPC_OK;
}
