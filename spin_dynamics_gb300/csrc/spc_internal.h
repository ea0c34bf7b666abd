// Internal declarations shared by the translation units of libspinchem_gpu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/spinchem_gpu.h"

namespace spc {

// Per-nucleus description used by both device Hamiltonian builders.
struct NucInfo {
  int g;            // multiplicity
  int owner;        // 0 = radical 1, 1 = radical 2
  int64_t stride;   // stride of this nucleus in the nuclear index
  double a_iso;     // trace(A)/3 (reference builder)
  double a_half;    // 0.5 * a_iso (reference builder off-diagonals)
  double zf;        // nuclear Zeeman factor -w*gamma/gamma_e (reference builder)
  double A[9];      // full tensor, A[r*3+c] (general builder)
  double zeta[3];   // (gamma/gamma_e) * B_c (general builder)
  double gratio;    // gamma/gamma_e
  int64_t tab_off;  // general builder: offset of this nucleus' entry table (48 g complex)
};

// Electronic 4x4 pieces of getHiso_sp, rounded as the reference rounds them.
struct RefElectron {
  double2 diag[4];  // Hel_diag: Zeeman + (2J + 2i dk + D33) S1zS2z - i kbar/2
  double2 flip_ab;  // (J + i dk + D11/2) on S1+S2-
  double2 flip_ba;  // (J + i dk + D22/2) on S1-S2+
};
// Full 4x4 electronic Hamiltonian of the general builder.
struct GenElectron {
  double2 H[4][4];
};

struct HostSystem {
  int64_t Z = 1, N = 4;
  std::vector<NucInfo> nuc;
  RefElectron ref;
  GenElectron gen;
  bool herm_shift = false;  // kS == kT: H_eff is Hermitian minus i*kbar/2
  // general builder: per nucleus j, the matrix element of the Hamiltonian
  // terms of nucleus j between (e, m_j) and (ep, m_j + d - 1), d = 0..2, at
  // [tab_off + ((e * 4 + ep) * g + m_j) * 3 + d] (zero where S_k.A.I_j does
  // not couple e and ep)
  std::vector<double2> gen_tab;
};

// Builds the host-side description; returns SPC_OK or an error code with
// the message set.
int make_host_system(const spc_system* sys, int mode, HostSystem& out);

// Kernel classes timed by the optional profiler.
enum ProfKind {
  PK_SPMM = 0,
  PK_DOT,
  PK_AXPY_DOT,
  PK_AXPY_NORM,
  PK_SCALE,
  PK_EXPM,
  PK_PROJ,
  PK_PROJ_REDUCE,
  PK_DTLOOP,
  PK_PSI,
  PK_SETUP,
  PK_CONTRACT,
  PK_COSTATE,
  PK_SAMPLE,  // one CTA per sample (small systems)
  PROF_KINDS
};
const char* prof_kind_name(int k);

// CUDA-event timing of each launch on its own stream, with the algorithmic
// FLOPs and bytes of the launch, accumulated per kernel class.
struct Prof {
  struct Pending {
    int kind;
    double flops, bytes;
    int ev;
  };
  bool on = false;
  std::vector<cudaEvent_t> pool;
  int used = 0;
  std::vector<Pending> pend;
  double ms[PROF_KINDS] = {}, flops[PROF_KINDS] = {}, bytes[PROF_KINDS] = {};
  int64_t launches[PROF_KINDS] = {};
  int begin(cudaStream_t st);
  void end(cudaStream_t st, int idx, int kind, double f, double b);
  void collect();  // after a stream synchronize
  void reset();
  ~Prof();
};

// Per-system facts of a Hamiltonian's execution copy, written on the device
// by the row split.
struct HMeta {
  double kappa;              // H_eff = A - i*kappa*1 (systems with herm_shift)
  unsigned long long ncplx;  // entries with a nonzero imaginary part
};

struct Handle {
  Prof prof;
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // Hamiltonian (CSR, 0-based)
  int n = 0;
  int64_t nnz = 0;
  int* d_rowptr = nullptr;
  int* d_col = nullptr;
  double2* d_val = nullptr;
  size_t cap_rowptr = 0, cap_h = 0;
  // execution copy of the Hamiltonian: kappa and complex-entry count (HMeta)
  int64_t nnz_cplx = 0;
  // propagation workspace (grow-only)
  struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
  };
  Buf psi, Q, P, partial, counters, coef, rbeta, Ahess, Aexp, proj, projpart, cvec, tt, kk, done,
      map, obs, out, zk, err, nbuild, flag, xcol, xval, xsplit, plan, jobtab, hmeta;
  // execution copy: Re + Im of every entry (xvs, nnz doubles); Re + Im of
  // the current Krylov vector of every tile (xsum, beside P)
  Buf xvs, xsum;
  // Hamiltonian build scratch: row counts, nucleus tables, nonzero totals
  Buf bcnt, bnuc, btot, btab;
  // autotuner outputs and sample subsets
  Buf tune_out, tune_zk;
  // yield-gradient workspace: checkpoints, segment states, node states,
  // costate pair, second coordinate vector, slot table, accumulators
  Buf gck, gseg, gnu, gmu, glam, cvec2, gslots, gracc, gfacc;
  // Hamiltonians of a batch (spc_build_h_batch): execution-order CSRs back to back
  struct HBatch {
    std::vector<int> n;
    std::vector<int64_t> nnz, rp_off, nz_off;
    std::vector<char> herm;
    std::vector<int64_t> nnz_cplx;
    Buf rowptr, split, col, val, vsum, meta;  // meta: one HMeta per system; vsum: Re + Im per entry
  } hb;
  // Krylov method: 0 full MGS (the reference's get_krylov), 1 Lanczos, 2 auto
  int krylov_method = 0;
  // replay each build round's launches as a captured CUDA graph
  bool use_graphs = true;
  // cap on the device bytes one propagation call may hold (0: the device's
  // free memory decides)
  size_t mem_limit = 0;
  // one-CTA-per-sample kernel for small systems: 0 when it pays, 1 never,
  // 2 whenever the call fits it
  int sample_path = 0;
  // H_eff = (Hermitian) - i*kappa*1 for the current Hamiltonian: Lanczos applies
  bool herm_shift = false;
  bool lanczos_active() const {
    return herm_shift && (krylov_method == 1 || krylov_method == 2);
  }
  std::vector<void*> host_pinned;
  spc_stats stats{};
  int64_t launches = 0;
  int sm_count = 148;
  size_t smem_optin = 48 * 1024;

  int ensure_rowptr(size_t count);
  int ensure_h_entries(size_t count);
  int ensure(Buf& b, size_t bytes);
  void count_launch(int k = 1) { launches += k; }
  ~Handle();
};

// One job of a batched propagation: a Hamiltonian (execution-order CSR on the
// device), its sample vectors and its output.
struct JobSpec {
  int n = 0;               // Hilbert dimension
  int64_t nnz = 0;
  int M = 0;               // samples
  const int* rowptr = nullptr;
  const int* split = nullptr;
  const int* col = nullptr;
  const double2* val = nullptr;
  const double* vsum = nullptr;  // Re + Im of every entry of the execution copy
  const double2* zk = nullptr;  // device, M x n/4 complex, sample-major
  double* out = nullptr;        // device, 4*T
  bool herm_shift = false;
  // herm_shift: the execution copy holds the Hermitian part (real diagonal)
  // and kappa (device) the shift, H_eff = A - i*kappa*1
  const double* kappa = nullptr;
  int64_t nnz_cplx = 0;  // entries of the execution copy with a nonzero imaginary part
};

// One reduced-matrix slot of the yield gradient: the electron pair (G = 4,
// owner = -1), one nucleus alone (G = g, owner = -2), or (spin of electron
// `owner`, nucleus of multiplicity g) with G = 2g classes; stride is the
// nucleus' stride in the nuclear index.
struct GradSlot {
  int G;
  int owner;
  int g;
  int pad;
  int64_t stride;
};
// One job of the yield gradient: system `sys` of the batch store (its H^H at
// sys + 1), M samples (device, M x Z), slots [slot0, slot0 + nslot) of the
// slot table (slot0 is the electron pair).
struct GradJob {
  int sys;
  int M;
  int slot0, nslot;
  const double2* zk;
  double cI, cP;  // source of the costate: cI psi + cP Pi_S psi (times c_k)
};

int set_error(int code, const char* fmt, ...);
int build_h_device(Handle* h, const HostSystem& hs, int mode);
// Every system into the batch store (h->hb) with two synchronisations in all;
// the handle's single Hamiltonian is left unset.
int build_h_batch_device(Handle* h, const std::vector<HostSystem>& hs, int mode);
// Row split of a CSR for k_spmm (complex entries first), enqueued on st.
// herm: H = A - i*kappa*1 with A Hermitian; the copy then holds A (diagonal
// entries real) and meta->kappa the shift. meta->ncplx (zeroed by the caller)
// receives the copy's count of entries with a nonzero imaginary part. xvs[k]
// = Re + Im of the copy's entry k (the third product of k_spmm's 3M form).
void enqueue_split_rows(int64_t N, const int* rowptr, const int* col, const double2* val, int* xcol,
                        double2* xval, double* xvs, int* split, bool herm, HMeta* meta, cudaStream_t st);
int propagate(Handle* h, const double* theta, const double* init_pop, const double* zk_dev,
              int M, double dt, double t_end, int m, double tol, double* out_dev, int T);
int propagate_batch(Handle* h, const double* theta, const double* init_pop,
                    const std::vector<JobSpec>& jobs, double dt, double t_end, int m, double tol,
                    int T);
// Adjoint sweeps of spc_yield_gradient(_batch) over the batch store's
// Hamiltonians: per job, the sample sums of the reduced matrices of the
// gradient integrals (rsum[job]: nslot x 36 complex) and of
// sum_k cw[k] psi_k psi_k^H on the electron pair (fsum[job]: 36 complex).
// want_grad = false runs the forward sweep only.
int yield_gradient_run(Handle* h, const double* theta, const std::vector<GradJob>& jobs,
                       const std::vector<GradSlot>& cs, double dt, int nsteps,
                       const std::vector<double>& cw, int m, int nq, int K, bool want_grad,
                       std::vector<std::vector<double2>>& rsum, std::vector<std::vector<double2>>& fsum);
// Nonzero count spc_build_h produces for a system (closed form per mode).
int64_t predict_nnz(const HostSystem& hs, int mode);
int num_time_points(double dt, double t_end);
// Execution order of H's rows for k_spmm (complex entries first).
int prepare_spmm_rows(Handle* h);

}  // namespace spc
