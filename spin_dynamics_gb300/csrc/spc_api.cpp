// extern "C" entry points of libspinchem_gpu (declared in include/spinchem_gpu.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "spc_internal.h"

struct spc_handle {
  spc::Handle h;
};

namespace spc {
const char* last_error();
void clear_error();
}  // namespace spc

#define CKR(call)                                                                             \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return spc::set_error(SPC_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));    \
  } while (0)

// True when H = A - i*kappa*1 with A exactly Hermitian (duplicates summed):
// every diagonal entry has the same imaginary part and H(c,r) = conj(H(r,c))
// for r != c, bit for bit.
static bool is_hermitian_plus_shift(int n, const std::vector<int>& rp, const std::vector<int>& cl,
                                    const double* val) {
  std::vector<std::pair<int64_t, std::pair<double, double>>> e;
  e.reserve(rp[n]);
  for (int r = 0; r < n; ++r)
    for (int k = rp[r]; k < rp[r + 1]; ++k)
      e.push_back({(int64_t)r * n + cl[k], {val[2 * (size_t)k], val[2 * (size_t)k + 1]}});
  std::sort(e.begin(), e.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  std::vector<std::pair<int64_t, std::pair<double, double>>> u;
  for (const auto& x : e) {
    if (!u.empty() && u.back().first == x.first) {
      u.back().second.first += x.second.first;
      u.back().second.second += x.second.second;
    } else {
      u.push_back(x);
    }
  }
  bool have_shift = false;
  double shift = 0.0;
  for (const auto& x : u) {
    const int r = (int)(x.first / n), c = (int)(x.first % n);
    if (r == c) {
      if (!have_shift) {
        shift = x.second.second;
        have_shift = true;
      } else if (x.second.second != shift) {
        return false;
      }
      continue;
    }
    const int64_t key = (int64_t)c * n + r;
    auto it = std::lower_bound(u.begin(), u.end(), key,
                               [](const auto& a, int64_t k) { return a.first < k; });
    const bool zero = x.second.first == 0.0 && x.second.second == 0.0;
    if (it == u.end() || it->first != key) {
      if (!zero) return false;
      continue;
    }
    if (it->second.first != x.second.first || it->second.second != -x.second.second) return false;
  }
  // rows without a stored diagonal have imaginary part 0 there
  for (int r = 0; r < n; ++r) {
    const int64_t key = (int64_t)r * n + r;
    auto it = std::lower_bound(u.begin(), u.end(), key,
                               [](const auto& a, int64_t k) { return a.first < k; });
    if ((it == u.end() || it->first != key) && have_shift && shift != 0.0) return false;
  }
  return true;
}

extern "C" {

int spc_set_krylov(spc_handle* h, int method) {
  if (!h) return spc::set_error(SPC_ERR_ARG, "null handle");
  if (method < SPC_KRYLOV_MGS || method > SPC_KRYLOV_AUTO)
    return spc::set_error(SPC_ERR_ARG, "unknown Krylov method %d", method);
  h->h.krylov_method = method;
  return SPC_OK;
}

int spc_create(int device, spc_handle** out) {
  if (!out) return spc::set_error(SPC_ERR_ARG, "null output pointer");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return spc::set_error(SPC_ERR_CUDA, "no CUDA device available (%s)",
                          e != cudaSuccess ? cudaGetErrorString(e) : "count = 0");
  if (device < 0 || device >= count)
    return spc::set_error(SPC_ERR_ARG, "device %d out of range (%d devices)", device, count);
  CKR(cudaSetDevice(device));
  spc_handle* hh = new (std::nothrow) spc_handle();
  if (!hh) return spc::set_error(SPC_ERR_ALLOC, "host allocation failed");
  hh->h.device = device;
  e = cudaStreamCreateWithFlags(&hh->h.own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete hh;
    return spc::set_error(SPC_ERR_CUDA, "cudaStreamCreate failed: %s", cudaGetErrorString(e));
  }
  hh->h.stream = hh->h.own_stream;
  cudaDeviceGetAttribute(&hh->h.sm_count, cudaDevAttrMultiProcessorCount, device);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  hh->h.smem_optin = (size_t)optin;
  *out = hh;
  spc::clear_error();
  return SPC_OK;
}

int spc_destroy(spc_handle* h) {
  if (!h) return SPC_OK;
  cudaSetDevice(h->h.device);
  if (h->h.stream) cudaStreamSynchronize(h->h.stream);
  delete h;
  return SPC_OK;
}

int spc_set_stream(spc_handle* h, void* stream) {
  if (!h) return spc::set_error(SPC_ERR_ARG, "null handle");
  h->h.stream = stream ? (cudaStream_t)stream : h->h.own_stream;
  return SPC_OK;
}

int spc_build_h(spc_handle* h, const spc_system* sys, int mode) {
  if (!h) return spc::set_error(SPC_ERR_ARG, "null handle");
  CKR(cudaSetDevice(h->h.device));
  spc::HostSystem hs;
  int rc = spc::make_host_system(sys, mode, hs);
  if (rc != SPC_OK) return rc;
  return spc::build_h_device(&h->h, hs, mode);
}

int spc_set_h(spc_handle* h, const spc_csr* H) {
  if (!h || !H || !H->rowptr || !H->col || !H->val || H->n < 4 || H->n % 4 != 0 || H->nnz < 0 ||
      (H->index_base != 0 && H->index_base != 1))
    return spc::set_error(SPC_ERR_ARG, "spc_set_h: bad argument (n must be a positive multiple of 4)");
  if (H->nnz > INT32_MAX) return spc::set_error(SPC_ERR_ARG, "nnz above the int32 CSR limit");
  const int n = H->n;
  const int64_t nnz = H->nnz;
  const int b = H->index_base;
  if ((int64_t)H->rowptr[0] != b || (int64_t)H->rowptr[n] - b != nnz)
    return spc::set_error(SPC_ERR_ARG, "row pointer does not match nnz");
  std::vector<int> rp(n + 1), cl(nnz > 0 ? nnz : 1);
  for (int i = 0; i <= n; ++i) {
    rp[i] = H->rowptr[i] - b;
    if (i > 0 && rp[i] < rp[i - 1]) return spc::set_error(SPC_ERR_ARG, "row pointer not monotone");
  }
  for (int64_t k = 0; k < nnz; ++k) {
    cl[k] = H->col[k] - b;
    if (cl[k] < 0 || cl[k] >= n) return spc::set_error(SPC_ERR_ARG, "column index out of range");
  }
  CKR(cudaSetDevice(h->h.device));
  if (h->h.ensure_rowptr(n + 1) || h->h.ensure_h_entries(nnz)) return SPC_ERR_ALLOC;
  CKR(cudaMemcpy(h->h.d_rowptr, rp.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
  if (nnz > 0) {
    CKR(cudaMemcpy(h->h.d_col, cl.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice));
    CKR(cudaMemcpy(h->h.d_val, H->val, sizeof(double2) * nnz, cudaMemcpyHostToDevice));
  }
  h->h.n = n;
  h->h.nnz = nnz;
  h->h.herm_shift = is_hermitian_plus_shift(n, rp, cl, H->val);
  return spc::prepare_spmm_rows(&h->h);
}

int spc_h_size(const spc_handle* h, int32_t* n, int64_t* nnz) {
  if (!h) return spc::set_error(SPC_ERR_ARG, "null handle");
  if (n) *n = h->h.n;
  if (nnz) *nnz = h->h.nnz;
  return SPC_OK;
}

int spc_get_h(spc_handle* h, int32_t* rowptr, int32_t* col, double* val) {
  if (!h || !rowptr || !col || !val) return spc::set_error(SPC_ERR_ARG, "null pointer");
  if (h->h.n == 0) return spc::set_error(SPC_ERR_STATE, "no Hamiltonian in the handle");
  CKR(cudaSetDevice(h->h.device));
  CKR(cudaStreamSynchronize(h->h.stream));
  CKR(cudaMemcpy(rowptr, h->h.d_rowptr, sizeof(int) * (h->h.n + 1), cudaMemcpyDeviceToHost));
  if (h->h.nnz > 0) {
    CKR(cudaMemcpy(col, h->h.d_col, sizeof(int) * h->h.nnz, cudaMemcpyDeviceToHost));
    CKR(cudaMemcpy(val, h->h.d_val, sizeof(double2) * h->h.nnz, cudaMemcpyDeviceToHost));
  }
  return SPC_OK;
}

int spc_num_time_points(double dt, double t_end) {
  if (!(dt > 0.0)) return -1;
  return spc::num_time_points(dt, t_end);
}

static int check_prop_args(spc_handle* h, const double* theta, const double* init_pop, int M,
                           double dt, int m, int T) {
  if (!h || !theta || !init_pop) return spc::set_error(SPC_ERR_ARG, "null pointer");
  if (h->h.n == 0) return spc::set_error(SPC_ERR_STATE, "no Hamiltonian: call spc_build_h or spc_set_h first");
  if (M < 1) return spc::set_error(SPC_ERR_ARG, "need at least one sample");
  if (!(dt > 0.0)) return spc::set_error(SPC_ERR_ARG, "dt must be positive");
  if (m < 1 || m > 48) return spc::set_error(SPC_ERR_ARG, "Krylov dimension %d outside [1, 48]", m);
  if (T < 1) return spc::set_error(SPC_ERR_ARG, "need at least one output slot");
  return SPC_OK;
}

int spc_trace_sampling_device(spc_handle* h, const double* theta, const double* init_pop,
                              const double* zkets_dev, int M, double dt, double t_end, int m,
                              double tol, double* out_dev, int T) {
  int rc = check_prop_args(h, theta, init_pop, M, dt, m, T);
  if (rc) return rc;
  if (!zkets_dev || !out_dev) return spc::set_error(SPC_ERR_ARG, "null device pointer");
  if (T != spc::num_time_points(dt, t_end))
    return spc::set_error(SPC_ERR_ARG, "T must be spc_num_time_points(dt, t_end) = %d",
                          spc::num_time_points(dt, t_end));
  CKR(cudaSetDevice(h->h.device));
  if (h->h.krylov_method == SPC_KRYLOV_LANCZOS && !h->h.herm_shift)
    return spc::set_error(SPC_ERR_ARG, "Lanczos needs H_eff = Hermitian - i*kappa (kS == kT)");
  return spc::propagate(&h->h, theta, init_pop, zkets_dev, M, dt, t_end, m, tol, out_dev, T);
}

int spc_trace_sampling(spc_handle* h, const double* theta, const double* init_pop,
                       const double* zkets, int M, double dt, double t_end, int m, double tol,
                       double* P_S, double* P_T0, double* P_Tp, double* P_Tm, int T) {
  int rc = check_prop_args(h, theta, init_pop, M, dt, m, T);
  if (rc) return rc;
  if (!zkets || !P_S || !P_T0 || !P_Tp || !P_Tm) return spc::set_error(SPC_ERR_ARG, "null pointer");
  if (T != spc::num_time_points(dt, t_end))
    return spc::set_error(SPC_ERR_ARG, "T must be spc_num_time_points(dt, t_end) = %d",
                          spc::num_time_points(dt, t_end));
  CKR(cudaSetDevice(h->h.device));
  if (h->h.krylov_method == SPC_KRYLOV_LANCZOS && !h->h.herm_shift)
    return spc::set_error(SPC_ERR_ARG, "Lanczos needs H_eff = Hermitian - i*kappa (kS == kT)");
  const int64_t Z = h->h.n / 4;
  spc::Handle& H = h->h;
  if (H.ensure(H.zk, sizeof(double) * 2 * Z * M) || H.ensure(H.out, sizeof(double) * 4 * T))
    return SPC_ERR_ALLOC;
  CKR(cudaMemcpyAsync(H.zk.p, zkets, sizeof(double) * 2 * Z * M, cudaMemcpyHostToDevice, H.stream));
  rc = spc::propagate(&H, theta, init_pop, (const double*)H.zk.p, M, dt, t_end, m, tol,
                      (double*)H.out.p, T);
  if (rc) return rc;
  double* outs[4] = {P_S, P_T0, P_Tp, P_Tm};
  for (int q = 0; q < 4; ++q)
    CKR(cudaMemcpyAsync(outs[q], (double*)H.out.p + (size_t)q * T, sizeof(double) * T,
                        cudaMemcpyDeviceToHost, H.stream));
  CKR(cudaStreamSynchronize(H.stream));
  return SPC_OK;
}

int spc_build_h_batch(spc_handle* h, int n_sys, const spc_system* systems, int mode) {
  if (!h || n_sys < 1 || !systems) return spc::set_error(SPC_ERR_ARG, "spc_build_h_batch: bad argument");
  CKR(cudaSetDevice(h->h.device));
  spc::Handle& H = h->h;
  std::vector<spc::HostSystem> hs(n_sys);
  auto& B = H.hb;
  B.n.assign(n_sys, 0);
  B.nnz.assign(n_sys, 0);
  B.rp_off.assign(n_sys, 0);
  B.nz_off.assign(n_sys, 0);
  B.herm.assign(n_sys, 0);
  int64_t rp_tot = 0, nz_tot = 0;
  for (int k = 0; k < n_sys; ++k) {
    int rc = spc::make_host_system(&systems[k], mode, hs[k]);
    if (rc != SPC_OK) return rc;
    B.n[k] = (int)hs[k].N;
    B.nnz[k] = spc::predict_nnz(hs[k], mode);
    B.rp_off[k] = rp_tot;
    B.nz_off[k] = nz_tot;
    B.herm[k] = hs[k].herm_shift;
    rp_tot += hs[k].N + 1;
    nz_tot += B.nnz[k];
  }
  if (H.ensure(B.rowptr, sizeof(int) * rp_tot) || H.ensure(B.split, sizeof(int) * rp_tot) ||
      H.ensure(B.col, sizeof(int) * nz_tot) || H.ensure(B.val, sizeof(double2) * nz_tot))
    return SPC_ERR_ALLOC;
  for (int k = 0; k < n_sys; ++k) {
    int rc = spc::build_h_device(&H, hs[k], mode);
    if (rc != SPC_OK) return rc;
    if (H.nnz != B.nnz[k]) return spc::set_error(SPC_ERR_STATE, "internal: nonzero count mismatch");
    cudaStream_t st = H.stream;
    CKR(cudaMemcpyAsync((int*)B.rowptr.p + B.rp_off[k], H.d_rowptr, sizeof(int) * (B.n[k] + 1),
                        cudaMemcpyDeviceToDevice, st));
    CKR(cudaMemcpyAsync((int*)B.split.p + B.rp_off[k], H.xsplit.p, sizeof(int) * B.n[k],
                        cudaMemcpyDeviceToDevice, st));
    CKR(cudaMemcpyAsync((int*)B.col.p + B.nz_off[k], H.xcol.p, sizeof(int) * B.nnz[k],
                        cudaMemcpyDeviceToDevice, st));
    CKR(cudaMemcpyAsync((double2*)B.val.p + B.nz_off[k], H.xval.p, sizeof(double2) * B.nnz[k],
                        cudaMemcpyDeviceToDevice, st));
  }
  CKR(cudaStreamSynchronize(H.stream));
  return SPC_OK;
}

static int batch_jobs(spc_handle* h, int n_jobs, const int* job_sys, const int* M,
                      const double2* zk_dev, double* out_dev, int T, std::vector<spc::JobSpec>& jobs) {
  const auto& B = h->h.hb;
  if (B.n.empty()) return spc::set_error(SPC_ERR_STATE, "no batch Hamiltonians: call spc_build_h_batch first");
  jobs.resize(n_jobs);
  int64_t zoff = 0;
  for (int k = 0; k < n_jobs; ++k) {
    const int s = job_sys ? job_sys[k] : k;
    if (s < 0 || s >= (int)B.n.size()) return spc::set_error(SPC_ERR_ARG, "job %d refers to system %d", k, s);
    if (M[k] < 1) return spc::set_error(SPC_ERR_ARG, "job %d has no samples", k);
    spc::JobSpec& j = jobs[k];
    j.n = B.n[s];
    j.nnz = B.nnz[s];
    j.M = M[k];
    j.rowptr = (const int*)B.rowptr.p + B.rp_off[s];
    j.split = (const int*)B.split.p + B.rp_off[s];
    j.col = (const int*)B.col.p + B.nz_off[s];
    j.val = (const double2*)B.val.p + B.nz_off[s];
    j.zk = zk_dev + zoff;
    j.out = out_dev + (size_t)k * 4 * T;
    j.herm_shift = B.herm[s] != 0;
    zoff += (int64_t)M[k] * (j.n / 4);
  }
  return SPC_OK;
}

int spc_trace_sampling_batch_device(spc_handle* h, int n_jobs, const int* job_sys, const int* M,
                                    const double* theta, const double* init_pop,
                                    const double* zkets_dev, double dt, double t_end, int m,
                                    double tol, double* out_dev, int T) {
  if (!h || n_jobs < 1 || !M || !theta || !init_pop || !zkets_dev || !out_dev)
    return spc::set_error(SPC_ERR_ARG, "spc_trace_sampling_batch: null argument");
  if (!(dt > 0.0)) return spc::set_error(SPC_ERR_ARG, "dt must be positive");
  if (m < 1 || m > 48) return spc::set_error(SPC_ERR_ARG, "Krylov dimension %d outside [1, 48]", m);
  if (T != spc::num_time_points(dt, t_end))
    return spc::set_error(SPC_ERR_ARG, "T must be spc_num_time_points(dt, t_end) = %d",
                          spc::num_time_points(dt, t_end));
  CKR(cudaSetDevice(h->h.device));
  std::vector<spc::JobSpec> jobs;
  int rc = batch_jobs(h, n_jobs, job_sys, M, (const double2*)zkets_dev, out_dev, T, jobs);
  if (rc) return rc;
  return spc::propagate_batch(&h->h, theta, init_pop, jobs, dt, t_end, m, tol, T);
}

int spc_trace_sampling_batch(spc_handle* h, int n_jobs, const int* job_sys, const int* M,
                             const double* theta, const double* init_pop, const double* zkets,
                             double dt, double t_end, int m, double tol, double* out, int T) {
  if (!h || n_jobs < 1 || !M || !zkets || !out)
    return spc::set_error(SPC_ERR_ARG, "spc_trace_sampling_batch: null argument");
  const auto& B = h->h.hb;
  int64_t ztot = 0;
  for (int k = 0; k < n_jobs; ++k) {
    const int s = job_sys ? job_sys[k] : k;
    if (s < 0 || s >= (int)B.n.size()) return spc::set_error(SPC_ERR_ARG, "job %d refers to system %d", k, s);
    ztot += (int64_t)M[k] * (B.n[s] / 4);
  }
  spc::Handle& H = h->h;
  CKR(cudaSetDevice(H.device));
  if (H.ensure(H.zk, sizeof(double) * 2 * ztot) || H.ensure(H.out, sizeof(double) * 4 * T * (size_t)n_jobs))
    return SPC_ERR_ALLOC;
  CKR(cudaMemcpyAsync(H.zk.p, zkets, sizeof(double) * 2 * ztot, cudaMemcpyHostToDevice, H.stream));
  int rc = spc_trace_sampling_batch_device(h, n_jobs, job_sys, M, theta, init_pop, (const double*)H.zk.p,
                                           dt, t_end, m, tol, (double*)H.out.p, T);
  if (rc) return rc;
  CKR(cudaMemcpyAsync(out, H.out.p, sizeof(double) * 4 * T * (size_t)n_jobs, cudaMemcpyDeviceToHost,
                      H.stream));
  CKR(cudaStreamSynchronize(H.stream));
  return SPC_OK;
}

int spc_set_profiling(spc_handle* h, int enable) {
  if (!h) return spc::set_error(SPC_ERR_ARG, "null handle");
  h->h.prof.on = enable != 0;
  h->h.prof.reset();
  return SPC_OK;
}

int spc_get_profile(const spc_handle* h, int kind, double* ms, int64_t* launches, double* flops,
                    double* bytes) {
  if (!h || kind < 0 || kind >= spc::PROF_KINDS) return spc::set_error(SPC_ERR_ARG, "bad argument");
  const spc::Prof& p = h->h.prof;
  if (ms) *ms = p.ms[kind];
  if (launches) *launches = p.launches[kind];
  if (flops) *flops = p.flops[kind];
  if (bytes) *bytes = p.bytes[kind];
  return SPC_OK;
}

int spc_get_stats(const spc_handle* h, spc_stats* out) {
  if (!h || !out) return spc::set_error(SPC_ERR_ARG, "null pointer");
  *out = h->h.stats;
  return SPC_OK;
}

}  // extern "C"
