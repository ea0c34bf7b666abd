// extern "C" entry points of libspinchem_gpu (declared in include/spinchem_gpu.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
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
  std::vector<spc::HostSystem> hs(n_sys);
  for (int k = 0; k < n_sys; ++k) {
    int rc = spc::make_host_system(&systems[k], mode, hs[k]);
    if (rc != SPC_OK) return rc;
  }
  return spc::build_h_batch_device(&h->h, hs, mode);
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
    j.vsum = (const double*)B.vsum.p + B.nz_off[s];
    j.zk = zk_dev + zoff;
    j.out = out_dev + (size_t)k * 4 * T;
    j.herm_shift = B.herm[s] != 0;
    j.kappa = j.herm_shift ? &((const spc::HMeta*)B.meta.p)[s].kappa : nullptr;
    j.nnz_cplx = B.nnz_cplx[s];
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

int spc_autotune_krylov(spc_handle* h, int n_jobs, const int* job_sys, const int* M, const double* theta,
                        const double* init_pop, const double* zkets, double dt, double t_window, double tol,
                        const int* candidates, int n_candidates, int* best_m, double* rates) {
  if (!h || n_jobs < 1 || !M || !theta || !init_pop || !zkets || !candidates || n_candidates < 1 || !best_m)
    return spc::set_error(SPC_ERR_ARG, "spc_autotune_krylov: null argument");
  if (!(dt > 0.0) || !(t_window > 0.0)) return spc::set_error(SPC_ERR_ARG, "dt and t_window must be positive");
  for (int c = 0; c < n_candidates; ++c)
    if (candidates[c] < 1 || candidates[c] > 48)
      return spc::set_error(SPC_ERR_ARG, "candidate Krylov dimension %d outside [1, 48]", candidates[c]);
  CKR(cudaSetDevice(h->h.device));
  spc::Handle& H = h->h;
  const auto& B = H.hb;
  if (B.n.empty()) return spc::set_error(SPC_ERR_STATE, "no batch Hamiltonians: call spc_build_h_batch first");
  // one tile (up to 32 samples) of every job, over a short window
  std::vector<int> Ms(n_jobs), sys(n_jobs);
  int64_t zsub = 0, ztot_src = 0;
  std::vector<int64_t> src_off(n_jobs);
  for (int k = 0; k < n_jobs; ++k) {
    sys[k] = job_sys ? job_sys[k] : k;
    if (sys[k] < 0 || sys[k] >= (int)B.n.size())
      return spc::set_error(SPC_ERR_ARG, "job %d refers to system %d", k, sys[k]);
    if (M[k] < 1) return spc::set_error(SPC_ERR_ARG, "job %d has no samples", k);
    Ms[k] = std::min(M[k], 32);
    src_off[k] = ztot_src;
    ztot_src += (int64_t)M[k] * (B.n[sys[k]] / 4);
    zsub += (int64_t)Ms[k] * (B.n[sys[k]] / 4);
  }
  const int T = spc::num_time_points(dt, t_window);
  if (H.ensure(H.tune_zk, sizeof(double2) * zsub) || H.ensure(H.tune_out, sizeof(double) * 4 * T * n_jobs))
    return SPC_ERR_ALLOC;
  {
    // the jobs' first Ms[k] sample vectors, back to back
    std::vector<double2> sub(zsub);
    int64_t o = 0;
    for (int k = 0; k < n_jobs; ++k) {
      const int64_t Z = B.n[sys[k]] / 4;
      std::memcpy(&sub[o], (const double2*)zkets + src_off[k], sizeof(double2) * Ms[k] * Z);
      o += Ms[k] * Z;
    }
    CKR(cudaMemcpyAsync(H.tune_zk.p, sub.data(), sizeof(double2) * zsub, cudaMemcpyHostToDevice, H.stream));
  }
  std::vector<spc::JobSpec> jobs;
  int rc = batch_jobs(h, n_jobs, sys.data(), Ms.data(), (const double2*)H.tune_zk.p, (double*)H.tune_out.p, T,
                      jobs);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  CKR(cudaEventCreate(&e0));
  CKR(cudaEventCreate(&e1));
  double best = -1.0;
  *best_m = candidates[0];
  for (int c = 0; c < n_candidates && rc == SPC_OK; ++c) {
    const int m = candidates[c];
    double secs = 0.0;
    for (int rep = 0; rep < 2 && rc == SPC_OK; ++rep) {  // the first run grows the buffers
      cudaEventRecord(e0, H.stream);
      rc = spc::propagate_batch(&H, theta, init_pop, jobs, dt, t_window, m, tol, T);
      cudaEventRecord(e1, H.stream);
      if (rc == SPC_OK && cudaEventSynchronize(e1) == cudaSuccess) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        secs = ms / 1e3;
      }
    }
    if (rc) break;
    const double rate = secs > 0.0 ? (double)H.stats.sample_steps / secs : 0.0;
    if (rates) rates[c] = rate;
    if (rate > best) {
      best = rate;
      *best_m = m;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int spc_mem_info(int device, int64_t* free_bytes, int64_t* total_bytes) {
  if (!free_bytes || !total_bytes) return spc::set_error(SPC_ERR_ARG, "spc_mem_info: null output");
  int cur = 0;
  CKR(cudaGetDevice(&cur));
  CKR(cudaSetDevice(device));
  size_t f = 0, t = 0;
  const cudaError_t e = cudaMemGetInfo(&f, &t);
  cudaSetDevice(cur);
  if (e != cudaSuccess) return spc::set_error(SPC_ERR_CUDA, "cudaMemGetInfo failed: %s", cudaGetErrorString(e));
  *free_bytes = (int64_t)f;
  *total_bytes = (int64_t)t;
  return SPC_OK;
}

int spc_set_graphs(spc_handle* h, int enable) {
  if (!h) return spc::set_error(SPC_ERR_ARG, "null handle");
  h->h.use_graphs = enable != 0;
  return SPC_OK;
}

int spc_set_sample_path(spc_handle* h, int mode) {
  if (!h) return spc::set_error(SPC_ERR_ARG, "null handle");
  if (mode < SPC_SAMPLE_AUTO || mode > SPC_SAMPLE_SINGLE) return spc::set_error(SPC_ERR_ARG, "unknown sample-path mode %d", mode);
  h->h.sample_path = mode;
  return SPC_OK;
}

int spc_set_memory_limit(spc_handle* h, int64_t bytes) {
  if (!h) return spc::set_error(SPC_ERR_ARG, "null handle");
  if (bytes < 0) return spc::set_error(SPC_ERR_ARG, "negative memory limit %lld", (long long)bytes);
  h->h.mem_limit = (size_t)bytes;
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

// ---------------------------------------------------------------------------
// yield gradient: host side (operators dH/dp and the contraction with the
// device's reduced matrices)
namespace {
using cplx = std::complex<double>;
using Mat = std::vector<cplx>;  // row-major square

// Sx, Sy, Sz of multiplicity g in the basis m = S, S-1, ..., -S
void spin_ops(int g, Mat out[3]) {
  const double S = 0.5 * (g - 1);
  for (int c = 0; c < 3; ++c) out[c].assign((size_t)g * g, 0.0);
  for (int i = 0; i < g; ++i) out[2][(size_t)i * g + i] = S - i;
  for (int i = 1; i < g; ++i) {
    const double sp = std::sqrt(S * (S + 1) - (S - i) * (S - i + 1));  // <m_{i-1}|S+|m_i>
    out[0][(size_t)(i - 1) * g + i] += 0.5 * sp;
    out[0][(size_t)i * g + i - 1] += 0.5 * sp;
    out[1][(size_t)(i - 1) * g + i] += cplx(0.0, -0.5 * sp);
    out[1][(size_t)i * g + i - 1] += cplx(0.0, 0.5 * sp);
  }
}
Mat kron(const Mat& A, int p, const Mat& B, int q) {
  Mat C((size_t)p * q * p * q);
  for (int i = 0; i < p; ++i)
    for (int j = 0; j < p; ++j)
      for (int k = 0; k < q; ++k)
        for (int l = 0; l < q; ++l) C[(size_t)(i * q + k) * p * q + j * q + l] = A[i * p + j] * B[k * q + l];
  return C;
}
Mat matmul(const Mat& A, const Mat& B, int n) {
  Mat C((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j) C[i * n + j] += A[i * n + k] * B[k * n + j];
  return C;
}
Mat eye(int n) {
  Mat I((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) I[i * n + i] = 1.0;
  return I;
}
// sum_ab O[a][b] R[a][b]
cplx contract_op(const Mat& O, const cplx* R, int G) {
  cplx s = 0.0;
  for (int i = 0; i < G * G; ++i) s += O[i] * R[i];
  return s;
}
}  // namespace

extern "C" {

int spc_yield_gradient_size(const spc_system* sys) {
  if (!sys || sys->n_nuc1 < 0 || sys->n_nuc2 < 0) return -1;
  return 15 + 9 * (sys->n_nuc1 + sys->n_nuc2);
}

// Upper bound on ||H_eff||_2 of the general builder's Hamiltonian:
// sqrt(max row sum * max column sum) of |H| (Holder), each sum bounded by the
// triangle inequality over the electronic 4x4 block and every nucleus' entry
// table (its largest row / column over the nuclear states).
static double h_norm_bound(const spc::HostSystem& hs) {
  double rmax = 0.0, cmax = 0.0;
  for (int e = 0; e < 4; ++e) {
    double r = 0.0, c = 0.0;
    for (int f = 0; f < 4; ++f) {
      r += std::hypot(hs.gen.H[e][f].x, hs.gen.H[e][f].y);
      c += std::hypot(hs.gen.H[f][e].x, hs.gen.H[f][e].y);
    }
    for (const spc::NucInfo& q : hs.nuc) {
      const int g = q.g;
      double rj = 0.0, cj = 0.0;
      // row (e, m): entries to (f, m + d - 1); column (e, m'): entries from
      // (f, m' - d + 1)
      for (int m = 0; m < g; ++m) {
        double rs = 0.0, cs = 0.0;
        for (int f = 0; f < 4; ++f)
          for (int d = 0; d < 3; ++d) {
            const double2 v = hs.gen_tab[q.tab_off + ((size_t)(e * 4 + f) * g + m) * 3 + d];
            rs += std::hypot(v.x, v.y);
            const int ms = m - d + 1;
            if (ms >= 0 && ms < g) {
              const double2 w = hs.gen_tab[q.tab_off + ((size_t)(f * 4 + e) * g + ms) * 3 + d];
              cs += std::hypot(w.x, w.y);
            }
          }
        rj = std::max(rj, rs);
        cj = std::max(cj, cs);
      }
      r += rj;
      c += cj;
    }
    rmax = std::max(rmax, r);
    cmax = std::max(cmax, c);
  }
  return std::sqrt(rmax * cmax);
}

// Gauss-Legendre nodes for the per-step derivative integral
// int_0^dt <exp(iH^H(dt-s)) lam| dH/dp |exp(-iHs) psi> ds. Its 2n-th
// derivative is at most (2||H|| )^(2n) times the integrand's scale, so the
// n-node rule's relative error is at most
//   (2||H|| dt)^(2n) (n!)^4 / ((2n+1) ((2n)!)^3)
// (the Gauss-Legendre remainder); the count is the smallest n with that
// below 1e-8, two orders under the 1e-6 agreement asked of the gradient.
static int nodes_for(double hnorm, double dt) {
  const double x = 2.0 * hnorm * dt;
  for (int n = 1; n <= 16; ++n) {
    double lf = 0.0;  // log of (n!)^4 / ((2n+1) ((2n)!)^3)
    for (int k = 2; k <= n; ++k) lf += 4.0 * std::log((double)k);
    for (int k = 2; k <= 2 * n; ++k) lf -= 3.0 * std::log((double)k);
    lf -= std::log(2.0 * n + 1.0);
    const double le = (x > 0.0 ? 2.0 * n * std::log(x) : -1e300) + lf;
    if (le <= std::log(1e-8)) return n;
  }
  return 16;
}

int spc_gradient_nodes(const spc_system* sys, double dt, int* n_quad) {
  if (!sys || !n_quad || !(dt > 0.0)) return spc::set_error(SPC_ERR_ARG, "spc_gradient_nodes: bad argument");
  spc::HostSystem hs;
  const int rc = spc::make_host_system(sys, SPC_H_GENERAL, hs);
  if (rc) return rc;
  *n_quad = nodes_for(h_norm_bound(hs), dt);
  return SPC_OK;
}

// Gradient of one job from its sample sums (pair slot first; then either
// (electron, nucleus) slots or nucleus-only slots per nucleus with g >= 2).
static void gradient_from_sums(const spc_system* sys, const spc::HostSystem& hs, int which, int M,
                               double wS, double wT, const std::vector<double2>& rs,
                               const std::vector<double2>& fs, double* yields, double* grad) {
  const int nn = (int)hs.nuc.size();
  const size_t con = 36;
  std::vector<cplx> R(rs.size()), F(con);
  for (size_t i = 0; i < rs.size(); ++i) R[i] = cplx(rs[i].x, rs[i].y);
  for (size_t i = 0; i < con; ++i) F[i] = cplx(fs[i].x, fs[i].y);
  Mat s2[3], I2 = eye(2), S1[3], S2[3];
  spin_ops(2, s2);
  for (int r = 0; r < 3; ++r) {
    S1[r] = kron(s2[r], 2, I2, 2);
    S2[r] = kron(I2, 2, s2[r], 2);
  }
  Mat S1S2(16, 0.0);
  for (int r = 0; r < 3; ++r) {
    const Mat p = matmul(S1[r], S2[r], 4);
    for (int i = 0; i < 16; ++i) S1S2[i] += p[i];
  }
  Mat PS(16), PT(16);
  for (int i = 0; i < 16; ++i) {
    const double d = (i % 5 == 0) ? 1.0 : 0.0;
    PS[i] = 0.25 * d - S1S2[i];
    PT[i] = 0.75 * d + S1S2[i];
  }
  const double inv_m = 1.0 / M;
  const double ps_int = contract_op(PS, F.data(), 4).real() * inv_m;
  const double pt_int = contract_op(PT, F.data(), 4).real() * inv_m;
  yields[0] = sys->kS * ps_int;
  yields[1] = sys->kT * pt_int;
  if (!grad) return;
  // d/dp = (2/M) Im(sum_ab O_p[a][b] R[a][b])
  auto dslot = [&](const Mat& O, int slot, int G) { return 2.0 * inv_m * contract_op(O, &R[slot * con], G).imag(); };
  // slot of nucleus j (its (electron, nucleus) or nucleus-only matrix)
  std::vector<int> slot_of(nn, -1);
  int next = 1;
  for (int j = 0; j < nn; ++j)
    if (hs.nuc[j].g >= 2) slot_of[j] = next++;
  for (int c = 0; c < 3; ++c) {
    Mat O(16);
    for (int i = 0; i < 16; ++i) O[i] = -(S1[c][i] + S2[c][i]);
    double g = dslot(O, 0, 4);
    for (int j = 0; j < nn; ++j) {
      if (slot_of[j] < 0) continue;
      const int gj = hs.nuc[j].g;
      Mat I[3];
      spin_ops(gj, I);
      if (which == SPC_GRAD_ALL)
        g += hs.nuc[j].gratio * dslot(kron(I2, 2, I[c], gj), slot_of[j], 2 * gj);
      else
        g += hs.nuc[j].gratio * dslot(I[c], slot_of[j], gj);
    }
    grad[c] = g;
  }
  {
    Mat O(16);
    for (int i = 0; i < 16; ++i) O[i] = 2.0 * S1S2[i];
    grad[3] = dslot(O, 0, 4);
  }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) grad[4 + r + 3 * c] = dslot(matmul(S1[r], S2[c], 4), 0, 4);
  {
    Mat OS(16), OT(16);
    for (int i = 0; i < 16; ++i) {
      OS[i] = cplx(0.0, -0.5) * PS[i];
      OT[i] = cplx(0.0, -0.5) * PT[i];
    }
    grad[13] = dslot(OS, 0, 4) + wS * ps_int;
    grad[14] = dslot(OT, 0, 4) + wT * pt_int;
  }
  if (which != SPC_GRAD_ALL) return;  // hyperfine entries stay 0
  for (int j = 0; j < nn; ++j) {
    if (slot_of[j] < 0) continue;
    const int gj = hs.nuc[j].g;
    Mat I[3];
    spin_ops(gj, I);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) grad[15 + 9 * j + r + 3 * c] = dslot(kron(s2[r], 2, I[c], gj), slot_of[j], 2 * gj);
  }
}

int spc_yield_gradient_batch(spc_handle* h, int n_jobs, const spc_system* systems, const int* M,
                             const double* theta, const double* zkets, double dt, double t_end, int m,
                             int n_quad, int checkpoint_every, double wS, double wT, int which,
                             double* yields, double* grad) {
  if (!h || n_jobs < 1 || !systems || !M || !theta || !zkets || !yields)
    return spc::set_error(SPC_ERR_ARG, "spc_yield_gradient_batch: null argument");
  if (!(dt > 0.0)) return spc::set_error(SPC_ERR_ARG, "dt must be positive");
  if (m < 1 || m > 48) return spc::set_error(SPC_ERR_ARG, "Krylov dimension %d outside [1, 48]", m);
  if (n_quad < 0 || n_quad > 16) return spc::set_error(SPC_ERR_ARG, "n_quad %d outside [0, 16]", n_quad);
  if (checkpoint_every < 0) return spc::set_error(SPC_ERR_ARG, "checkpoint_every must be >= 0");
  if (which != SPC_GRAD_ALL && which != SPC_GRAD_FIELD)
    return spc::set_error(SPC_ERR_ARG, "unknown gradient set %d", which);
  std::vector<spc::HostSystem> hs(n_jobs);
  int64_t ztot = 0, gtot = 0;
  for (int k = 0; k < n_jobs; ++k) {
    if (M[k] < 1) return spc::set_error(SPC_ERR_ARG, "job %d has no samples", k);
    int rc = spc::make_host_system(&systems[k], SPC_H_GENERAL, hs[k]);
    if (rc) return rc;
    if (h->h.krylov_method == SPC_KRYLOV_LANCZOS && !hs[k].herm_shift)
      return spc::set_error(SPC_ERR_ARG, "Lanczos needs H_eff = Hermitian - i*kappa (kS == kT)");
    for (const spc::NucInfo& q : hs[k].nuc) {
      if (which == SPC_GRAD_ALL && q.g > 3)
        return spc::set_error(SPC_ERR_UNSUPPORTED,
                              "hyperfine gradients take nuclei of multiplicity <= 3 (use SPC_GRAD_FIELD)");
      if (q.g > 6) return spc::set_error(SPC_ERR_UNSUPPORTED, "gradients take nuclei of multiplicity <= 6");
    }
    ztot += (int64_t)M[k] * hs[k].Z;
    gtot += 15 + 9 * (int64_t)hs[k].nuc.size();
  }
  if (n_quad == 0)  // the count the per-step bound asks for, the largest over the jobs
    for (int k = 0; k < n_jobs; ++k) n_quad = std::max(n_quad, nodes_for(h_norm_bound(hs[k]), dt));
  CKR(cudaSetDevice(h->h.device));
  spc::Handle& H = h->h;
  if (grad) std::fill(grad, grad + gtot, 0.0);
  std::fill(yields, yields + 2 * n_jobs, 0.0);
  const int T = spc::num_time_points(dt, t_end);
  const int nh = T / 2;
  if (nh < 2) return SPC_OK;  // get_kinetics adds no Simpson panel
  const int nsteps = 2 * nh - 2;
  std::vector<double> cw(nsteps + 1);
  for (int k = 0; k <= nsteps; ++k)
    cw[k] = (dt / 3.0) * ((k == 0 || k == nsteps) ? 1.0 : (k % 2 ? 4.0 : 2.0));
  // H_k and H_k^H = H_eff(-kS, -kT) as batch systems 2k and 2k + 1
  std::vector<spc_system> pairs(2 * (size_t)n_jobs);
  for (int k = 0; k < n_jobs; ++k) {
    pairs[2 * k] = pairs[2 * k + 1] = systems[k];
    pairs[2 * k + 1].kS = -systems[k].kS;
    pairs[2 * k + 1].kT = -systems[k].kT;
  }
  int rc = spc_build_h_batch(h, 2 * n_jobs, pairs.data(), SPC_H_GENERAL);
  if (rc) return rc;
  if (H.ensure(H.zk, sizeof(double) * 2 * ztot)) return SPC_ERR_ALLOC;
  CKR(cudaMemcpyAsync(H.zk.p, zkets, sizeof(double) * 2 * ztot, cudaMemcpyHostToDevice, H.stream));
  std::vector<spc::GradSlot> slots;
  std::vector<spc::GradJob> jobs(n_jobs);
  int64_t zoff = 0;
  for (int k = 0; k < n_jobs; ++k) {
    spc::GradJob& J = jobs[k];
    J.sys = 2 * k;
    J.M = M[k];
    J.slot0 = (int)slots.size();
    J.zk = (const double2*)H.zk.p + zoff;
    J.cI = wT * systems[k].kT;
    J.cP = wS * systems[k].kS - wT * systems[k].kT;
    zoff += (int64_t)M[k] * hs[k].Z;
    slots.push_back({4, -1, 1, 0, 1});
    if (grad)
      for (const spc::NucInfo& q : hs[k].nuc)
        if (q.g >= 2) {
          if (which == SPC_GRAD_ALL)
            slots.push_back({2 * q.g, q.owner, q.g, 0, q.stride});
          else
            slots.push_back({q.g, -2, q.g, 0, q.stride});
        }
    J.nslot = (int)slots.size() - J.slot0;
  }
  const int K = std::min(checkpoint_every, nsteps);  // 0: chosen by device memory
  std::vector<std::vector<double2>> rsum, fsum;
  rc = spc::yield_gradient_run(&H, theta, jobs, slots, dt, nsteps, cw, m, n_quad, K, grad != nullptr, rsum,
                               fsum);
  if (rc) return rc;
  int64_t goff = 0;
  for (int k = 0; k < n_jobs; ++k) {
    gradient_from_sums(&systems[k], hs[k], which, M[k], wS, wT, rsum[k], fsum[k], yields + 2 * k,
                       grad ? grad + goff : nullptr);
    goff += 15 + 9 * (int64_t)hs[k].nuc.size();
  }
  return SPC_OK;
}

int spc_yield_gradient(spc_handle* h, const spc_system* sys, const double* theta, const double* zkets,
                       int M, double dt, double t_end, int m, int n_quad, int checkpoint_every,
                       double wS, double wT, double* yields, double* grad) {
  if (!sys) return spc::set_error(SPC_ERR_ARG, "spc_yield_gradient: null argument");
  return spc_yield_gradient_batch(h, 1, sys, &M, theta, zkets, dt, t_end, m, n_quad, checkpoint_every, wS, wT,
                                  SPC_GRAD_ALL, yields, grad);
}

}  // extern "C"
