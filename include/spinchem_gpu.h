/*
 * spinchem_gpu.h — C ABI of the GB300 trace-sampling library (libspinchem_gpu.so).
 *
 * Drop-in for the quantum hot path of KenHino/Spin_dynamics (`spinchem`):
 * the sparse spin Hamiltonian build and trace-sampling propagation behind
 * `trace_sampling_para` (src/qm_dynamics.f90:257-384). Every entry point is
 * plain C: integers, doubles and pointers, callable from Fortran through
 * iso_c_binding (bind(C)), from C/C++, and from Python through ctypes.
 *
 * Conventions
 *  - Status: every function returns 0 (SPC_OK) or a positive SPC_ERR_* code;
 *    spc_last_error() gives the message of the last failure on this thread.
 *    Where the reference stops the program (`stop 'Error: ...'`) the library
 *    returns SPC_ERR_UNSUPPORTED or SPC_ERR_ARG with the same message.
 *  - Complex numbers are complex(dp) / double _Complex: interleaved (re, im)
 *    pairs of doubles.
 *  - Units are the reference's internal units after read_inp
 *    (src/spinsys.f90:88-89,107-108): energies in mT, kS and kT in 1/us
 *    divided by gamma_e = 176.08596, dt and t_end in ns * gamma_e / 1000.
 *  - A handle owns one CUDA device, one stream and the device buffers; it is
 *    not thread-safe. Host pointers are caller-owned and only read/written
 *    during the call.
 *  - No CPU fallback: a handle cannot be created without a usable GPU.
 */
#ifndef SPINCHEM_GPU_H
#define SPINCHEM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPC_OK 0
#define SPC_ERR_ARG 1          /* bad argument (sizes, null pointers, unknown mode) */
#define SPC_ERR_CUDA 2         /* a CUDA runtime call failed */
#define SPC_ERR_ALLOC 3        /* device or host allocation failed */
#define SPC_ERR_UNSUPPORTED 4  /* a system the reference refuses (its `stop` conditions) */
#define SPC_ERR_NUMERIC 5      /* time-index overflow or non-finite result */
#define SPC_ERR_STATE 6        /* call order: e.g. propagation before a Hamiltonian exists */

typedef struct spc_handle spc_handle;

/* Spin system, host memory. Replaces the fields of `sys_param`/`electron`
 * (src/spinsys.f90:21-38) that getHiso_sp reads (src/hamiltonian.f90:17-205),
 * plus the field vector that app/main.f90:53-54 turns into the Larmor
 * frequencies w = -B. */
typedef struct {
  int n_nuc1, n_nuc2;      /* nuclei on radical 1 and radical 2 */
  const int* mult1;        /* nuclear multiplicities (2 = 1H, 3 = 14N, ...) */
  const int* mult2;
  const double* A1;        /* 9 doubles per nucleus: column-major 3x3 hyperfine tensor (mT),
                              the order of the A<i> keys in input.ini */
  const double* A2;
  const double* gamma1;    /* nuclear gyromagnetic ratios; NULL = by multiplicity as the
                              reference assigns them (src/hamiltonian.f90:132-138) */
  const double* gamma2;
  double B[3];             /* field vector (mT); the reference's scalar B is (0, 0, B) */
  double J;                /* exchange (mT) */
  double D[9];             /* dipolar tensor, column-major (mT) */
  double kS, kT;           /* Haberkorn rates, internal units */
} spc_system;

/* Compressed sparse row matrix in HOST memory (stdlib CSR_cdp_type layout:
 * rowptr(n+1), col(nnz), data(nnz) complex). index_base is 0 or 1. */
typedef struct {
  int32_t n;
  int64_t nnz;
  int32_t* rowptr;
  int32_t* col;
  double* val;       /* 2*nnz doubles */
  int32_t index_base;
} spc_csr;

/* Hamiltonian build modes for spc_build_h. */
#define SPC_H_REFERENCE 0  /* getHiso_sp + coo_to_csr: isotropic a = trace(A)/3, field along z
                              (B[0], B[1] must be 0), axial D; CSR rows in the reference's order */
#define SPC_H_GENERAL 1    /* anisotropic S.A.I, field vector, full D tensor; columns ascending */

/* Krylov methods for spc_set_krylov. */
#define SPC_KRYLOV_MGS 0      /* Arnoldi with full modified Gram-Schmidt, as get_krylov
                                 (src/qm_dynamics.f90:432-467); the default */
#define SPC_KRYLOV_LANCZOS 1  /* three-term recurrence; only for H_eff = Hermitian - i*kappa
                                 (kS == kT); a basis whose Gram matrix drifts from the identity
                                 by more than 1e-12 is rebuilt with full MGS */
#define SPC_KRYLOV_AUTO 2     /* Lanczos when H_eff is Hermitian - i*kappa, else MGS */

/* Counters of the last propagation call. */
typedef struct {
  int64_t krylov_builds;   /* sum over samples of Krylov subspaces built */
  int64_t lanczos_fallbacks; /* Lanczos bases rebuilt with full MGS */
  int64_t rounds;          /* batched build rounds (max builds of any sample) */
  int64_t sample_steps;    /* sum over samples of dt steps taken */
  int64_t kernel_launches; /* kernels launched by the library during the call */
  double seconds;          /* wall time of the call */
} spc_stats;

/* ---- library / handle ------------------------------------------------- */

/* Message of the last failure on the calling thread ("" if none). */
const char* spc_last_error(void);

/* Create a handle on CUDA device `device` (one stream, no buffers yet).
 * Returns SPC_ERR_CUDA when no usable GPU is present. */
int spc_create(int device, spc_handle** out);

/* Release every device buffer and the stream. */
int spc_destroy(spc_handle* h);

/* Use a caller-owned cudaStream_t (NULL = the handle's own stream). */
int spc_set_stream(spc_handle* h, void* cuda_stream);

/* ---- Hamiltonian ------------------------------------------------------ */

/* Build H_eff = H - iK/2 on the device and keep it in the handle.
 * SPC_H_REFERENCE replaces getHiso_sp (src/hamiltonian.f90:17-205) followed by
 * coo_to_csr (src/utils.f90:52-89): same nonzeros, same within-row order.
 * SPC_H_GENERAL is the anisotropic extension (no sparse reference counterpart;
 * hyperfine form of getH_dense, src/hamiltonian.f90:279-311). */
int spc_build_h(spc_handle* h, const spc_system* sys, int mode);

/* Upload a caller-built CSR (host memory, 0- or 1-based) as the Hamiltonian.
 * Replaces passing `type(CSR_cdp_type) :: H` into the propagation. */
int spc_set_h(spc_handle* h, const spc_csr* H);

/* Allocation-free Hamiltonian build (no counterpart in the reference). For
 * callers that cannot allocate device memory: hosts that run inside a
 * device-memory pool with a budget fixed up front, or plugins and Fortran
 * programs that only pass buffers they own. It builds the same CSR as
 * spc_build_h (same modes, bit-identical output) into caller-owned DEVICE
 * buffers rowptr_dev (n+1), col_dev and val_dev (cap_nnz entries) on `stream`
 * (a cudaStream_t, NULL = default stream) of the current device, without a
 * handle, and calls no cudaMalloc, cudaFree or allocating library routine.
 * Its scratch (per-row counts, nucleus table, entry tables) is a file-scope
 * device array of about 5.3 MB that every GPU loading the library holds until
 * exit; systems above 2^20 rows, 64 nuclei or 65536 entry-table elements are
 * rejected with SPC_ERR_ARG. The first call under a device's context looks up
 * that array's device address (again after cudaDeviceReset); make that first
 * call before any stream capture begins on the device. The size comes
 * from the closed-form nonzero count: *n_out and *nnz_out are set, and a
 * cap_nnz that is too small returns SPC_ERR_ARG before anything is launched
 * or written. The call waits for `stream` twice (after the count and after
 * the fill). All calls share the array: calls that overlap on the GPU race
 * and must be serialised by the caller. */
int spc_build_h_noalloc(const spc_system* sys, int mode, int32_t* rowptr_dev, int32_t* col_dev,
                        double* val_dev, int64_t cap_nnz, int32_t* n_out, int64_t* nnz_out,
                        void* stream);

/* Dimension and nonzero count of the handle's Hamiltonian. */
int spc_h_size(const spc_handle* h, int32_t* n, int64_t* nnz);

/* Copy the handle's Hamiltonian to caller buffers (rowptr n+1, col nnz,
 * val 2*nnz), 0-based indices. */
int spc_get_h(spc_handle* h, int32_t* rowptr, int32_t* col, double* val);

/* ---- propagation ------------------------------------------------------ */

/* Number of output time points: N_steps + 1 with
 * N_steps = ceiling((t_end + dt)/dt) (src/qm_dynamics.f90:305-306). */
int spc_num_time_points(double dt, double t_end);

/* Trace-sampling propagation of M caller-supplied nuclear sample vectors.
 * Replaces the body of trace_sampling_para from the OpenMP region to the
 * sample average (src/qm_dynamics.f90:322-378): for every sample, psi =
 * theta (x) z (kron_vector), Arnoldi/MGS Krylov bases of dimension m
 * (get_krylov :432-467), the Pade-6 exponential of -i dt A (expm,
 * src/matrix_exponential.f90:14-87), the Krylov-space projectors
 * (convert_to_krylov :469-498) and the Krylov-reuse dt loop (:340-366) with
 * the rebuild test |c_m|^2 <= tol |c|^2; then the sample average
 * (res%update, res%scale(1/M)).
 *   theta    4 complex, the electronic state (init_el_state :386-414)
 *   init_pop 4 doubles, populations at t = 0 in the order S, T0, Tp, Tm
 *   zkets    M x Z complex in host memory, sample-major (Z = n/4)
 *   outputs  P_S, P_T0, P_Tp, P_Tm: T doubles each, host memory,
 *            T = spc_num_time_points(dt, t_end); trailing slots the dt loop
 *            never reaches stay 0 as in the reference.
 * The host buffers are copied to and from the device inside the call. */
int spc_trace_sampling(spc_handle* h, const double* theta, const double* init_pop,
                       const double* zkets, int M, double dt, double t_end, int m, double tol,
                       double* P_S, double* P_T0, double* P_Tp, double* P_Tm, int T);

/* The same on device-resident buffers (no host copies, asynchronous apart
 * from one small flag read per build round): zkets_dev is M x Z complex,
 * out_dev receives 4*T doubles (P_S | P_T0 | P_Tp | P_Tm). */
int spc_trace_sampling_device(spc_handle* h, const double* theta, const double* init_pop,
                              const double* zkets_dev, int M, double dt, double t_end, int m,
                              double tol, double* out_dev, int T);

/* ---- batches: many independent systems in one propagation ------------ */

/* Build the Hamiltonians of n_sys systems (same mode) and keep them in the
 * handle as a batch; system k is addressed by index k below. Replaces the
 * per-block / per-field calls of getHiso_sp in symmetrised_dynamics
 * (src/symmetry.f90:102-110) and the field loop of app/main.f90:48-79 with
 * one device-resident set. All systems are built with two synchronisations
 * in total. The handle's single Hamiltonian is unset (spc_build_h or
 * spc_set_h sets it again). */
int spc_build_h_batch(spc_handle* h, int n_sys, const spc_system* systems, int mode);

/* Trace-sample n_jobs jobs together: job k propagates M[k] caller-supplied
 * vectors under system job_sys[k] (NULL: system k). Jobs may have different
 * dimensions; each job's samples are averaged separately. Every build round
 * batches the Krylov builds of all unfinished samples of all jobs in one set
 * of launches. zkets: the jobs' M[k] x Z_k complex blocks back to back (host
 * memory); out: n_jobs x (P_S | P_T0 | P_Tp | P_Tm), T doubles each.
 * dt, t_end, m, tol, theta and init_pop are shared by all jobs; Lanczos
 * applies only when every job's H_eff is Hermitian - i*kappa. */
int spc_trace_sampling_batch(spc_handle* h, int n_jobs, const int* job_sys, const int* M,
                             const double* theta, const double* init_pop, const double* zkets,
                             double dt, double t_end, int m, double tol, double* out, int T);

/* The same with device-resident zkets and out. */
int spc_trace_sampling_batch_device(spc_handle* h, int n_jobs, const int* job_sys, const int* M,
                                    const double* theta, const double* init_pop,
                                    const double* zkets_dev, double dt, double t_end, int m,
                                    double tol, double* out_dev, int T);

/* ---- yield gradient (no counterpart in the reference) ---------------- */

/* Entries of the gradient spc_yield_gradient writes for `sys`:
 * 15 + 9 * (n_nuc1 + n_nuc2), or -1 for a bad argument. */
int spc_yield_gradient_size(const spc_system* sys);

/* Gauss-Legendre node count (no counterpart in the reference) that
 * spc_yield_gradient uses with n_quad = 0 for `sys` at step dt: the smallest
 * n whose remainder bound (2 b dt)^(2n) (n!)^4 / ((2n+1) ((2n)!)^3) is at
 * most 1e-8, with b = sqrt(max row sum * max column sum) of |H_eff| >=
 * ||H_eff||_2. Host only. */
int spc_gradient_nodes(const spc_system* sys, double dt, int* n_quad);

/* Singlet and triplet yields and the gradient of wS*Phi_S + wT*Phi_T with
 * respect to every parameter of `sys`, by the discrete adjoint of a stepwise
 * propagation. The reference computes the yields only (get_kinetics,
 * src/observables.f90:74-101, on the populations of trace_sampling_para,
 * src/qm_dynamics.f90:257-384); it has no derivatives.
 * Model: every sample psi = theta (x) z is propagated by
 * psi_{k+1} = exp(-i H dt) psi_k with one Krylov basis of dimension m per
 * step (full MGS; the three-term recurrence only under SPC_KRYLOV_LANCZOS,
 * which needs kS == kT and is not Gram-checked here), the
 * Hamiltonian of SPC_H_GENERAL, populations averaged over the M samples, and
 * Phi_X = k_X * the Simpson sum of get_kinetics over the
 * spc_num_time_points(dt, t_end) grid (its last value).
 *   zkets            M x Z complex, host memory, sample-major
 *   n_quad           Gauss-Legendre nodes per step for the derivative of
 *                    exp(-i H dt) (1..16), or 0: the count
 *                    spc_gradient_nodes picks (largest over the jobs)
 *   checkpoint_every forward states kept every this many steps (0 = among
 *                    the spacings that fit in device memory, the one that
 *                    recomputes the fewest steps)
 *   yields           2 doubles: Phi_S, Phi_T
 *   grad             NULL: yields only (the forward sweep, one Krylov build
 *                    per sample and step); else spc_yield_gradient_size(sys) doubles:
 *                    dB[3], dJ, dD[9] (column-major as spc_system.D), dkS, dkT,
 *                    then 9 per nucleus (radical 1's, then radical 2's),
 *                    column-major as spc_system.A1/A2
 * Device memory: about (m + 6 + n_steps/K + (1 + n_quad) K) states of
 * 16 * n * ceil(M/32)*32 bytes, or (m + 6 + n_steps/K + K + n_quad) when that
 * does not fit (node states rebuilt per step); SPC_ERR_ALLOC when neither
 * fits. Nuclei of multiplicity above 3 return SPC_ERR_UNSUPPORTED. The
 * handle's batch is replaced by H and H^H (its single Hamiltonian unset). Cost: three
 * Krylov builds per sample and step (four when node states are rebuilt);
 * spc_get_stats reports rounds = 1 when node states were kept. */
int spc_yield_gradient(spc_handle* h, const spc_system* sys, const double* theta,
                       const double* zkets, int M, double dt, double t_end, int m, int n_quad,
                       int checkpoint_every, double wS, double wT, double* yields, double* grad);

/* Gradient sets for spc_yield_gradient_batch. */
#define SPC_GRAD_ALL 0    /* every parameter (nuclei of multiplicity <= 3) */
#define SPC_GRAD_FIELD 1  /* B, J, D, kS, kT; hyperfine entries left 0 (nuclei of
                             multiplicity <= 6, e.g. symmetry blocks) */

/* spc_yield_gradient for n_jobs systems of any dimensions in one sweep
 * (field orientations, radical pairs, symmetry blocks): job k propagates
 * M[k] vectors under systems[k]; zkets holds the jobs' M[k] x Z_k blocks back
 * to back. yields: n_jobs x (Phi_S, Phi_T); grad (NULL: yields only): the
 * jobs' spc_yield_gradient_size(systems[k]) blocks back to back. Every build,
 * contraction and costate step of all jobs shares one set of launches. The
 * handle's batch is replaced by H_k and H_k^H (its single Hamiltonian unset). */
int spc_yield_gradient_batch(spc_handle* h, int n_jobs, const spc_system* systems, const int* M,
                             const double* theta, const double* zkets, double dt, double t_end, int m,
                             int n_quad, int checkpoint_every, double wS, double wT, int which,
                             double* yields, double* grad);

/* Krylov-dimension autotuner (no counterpart in the reference): propagates
 * the first min(M[k], 32) vectors of every job of the batch store (as in
 * spc_trace_sampling_batch) over [0, t_window] once per candidate dimension,
 * times each run with CUDA events after a warm-up run, and returns the
 * candidate with the most sample-steps per second in *best_m (rates, if not
 * NULL, gets the rate of every candidate). The reference fixes N_krylov in
 * input.ini; results at any m are the reference's algorithm at that m. */
int spc_autotune_krylov(spc_handle* h, int n_jobs, const int* job_sys, const int* M, const double* theta,
                        const double* init_pop, const double* zkets, double dt, double t_window, double tol,
                        const int* candidates, int n_candidates, int* best_m, double* rates);

/* Select the Krylov orthogonalisation (SPC_KRYLOV_*). In exact arithmetic
 * Lanczos and MGS give the same basis when H_eff = Hermitian - i*kappa; the
 * Lanczos path skips the O(m^2 n) re-orthogonalisation and verifies the
 * basis through the projector Grams (their sum is Q^H Q). */
int spc_set_krylov(spc_handle* h, int method);

/* Free and total device memory of `device` in bytes (sizes batches of jobs
 * that do not fit one call). */
int spc_mem_info(int device, int64_t* free_bytes, int64_t* total_bytes);

/* Propagation of small systems with one CTA per sample carrying the
 * sample's whole run (every Krylov build, expm, projectors, dt loop) in one
 * launch: SPC_SAMPLE_AUTO (default) when every job has at most 2048 rows,
 * m <= 32, a build of about 2.5e6 FP64 FMAs or less and the samples fill at
 * most two waves of CTAs; SPC_SAMPLE_OFF never; SPC_SAMPLE_ON whenever the
 * call fits it (rows, m, shared and device memory). When the samples fill at
 * most half the SMs, each sample takes a cluster of two CTAs (the second
 * forms the projectors and the populations of every dt step beside the
 * first's serial path); SPC_SAMPLE_SINGLE is SPC_SAMPLE_ON with one CTA per
 * sample always. The tiled path serves every other call. Results agree with
 * the tiled path to rounding. */
#define SPC_SAMPLE_AUTO 0
#define SPC_SAMPLE_OFF 1
#define SPC_SAMPLE_ON 2
#define SPC_SAMPLE_SINGLE 3
int spc_set_sample_path(spc_handle* h, int mode);

/* Cap on the device memory one propagation call on this handle may hold
 * (0, the default: the device's free memory, less a reserve). A call whose
 * Krylov bases for every sample at once exceed it propagates its samples in
 * consecutive chunks of 32-sample tiles within each build round; results
 * agree with the unchunked call to rounding (per-sample reductions are
 * grouped differently). SPC_ERR_ALLOC when one tile of the largest job does
 * not fit. */
int spc_set_memory_limit(spc_handle* h, int64_t bytes);

/* Replay each build round of a propagation as a CUDA graph (1, the
 * default) or launch its kernels one by one (0). The launches of a round are
 * captured when a work-plan shape occurs for the second time within a call
 * and replayed while it repeats (small systems run hundreds of rounds of one
 * shape); results are identical either way. Not used while kernel profiling
 * is on. */
int spc_set_graphs(spc_handle* h, int enable);

/* Counters of the last propagation call on this handle. */
int spc_get_stats(const spc_handle* h, spc_stats* out);

/* ---- host helpers ----------------------------------------------------- */

/* Sample vectors exactly as the reference draws them: the master
 * xoroshiro128+ generator seeded with `seed` (app/main.f90:48,
 * src/m_random.f90:90-98); mode 0 = trace_sampling_para (two next() per
 * sample, then set_seed + sample_SUZ per sample, src/qm_dynamics.f90:315-327),
 * mode 1 = trace_sampling (one stream, :198-199). out: M x Z complex. */
int spc_seeded_samples(int64_t seed0, int64_t seed1, int Z, int M, int mode, double* out);

/* The raw next() stream of a generator seeded with `seed` (set_seed then
 * next(), src/m_random.f90:90-98,321-331): what the drivers draw per-sample
 * or per-block seeds from (src/qm_dynamics.f90:317-320,
 * src/symmetry.f90:76-79). */
int spc_rng_stream(int64_t seed0, int64_t seed1, int n, uint64_t* out);

/* Electronic initial state and populations (init_el_state,
 * src/qm_dynamics.f90:386-414): which = 0 singlet, 1 T0, 2 Tp, 3 Tm. */
int spc_init_el_state(int which, double* theta, double* init_pop);

/* Singlet/triplet yields by Simpson's rule (get_kinetics,
 * src/observables.f90:74-101). Inputs T each; Phi_S/Phi_T get T/2 entries,
 * iden T entries; any output may be NULL. */
int spc_kinetics(int T, const double* P_S, const double* P_T0, const double* P_Tp,
                 const double* P_Tm, double dt, double kS, double kT, double* Phi_S,
                 double* Phi_T, double* iden);

/* ---- diagnostics (no counterpart in the reference) ------------------- */

/* Time every kernel launch of later propagation calls with CUDA events on
 * the handle's stream, per kernel class (0 disables). */
int spc_set_profiling(spc_handle* h, int enable);

/* Accumulated time (ms), launches, and the algorithmic FLOPs and bytes of
 * kernel class `kind` (0 <= kind < SPC_KERNEL_KINDS) since profiling was
 * enabled. */
#define SPC_KERNEL_KINDS 14
int spc_get_profile(const spc_handle* h, int kind, double* ms, int64_t* launches, double* flops,
                    double* bytes);

/* Name of kernel class `kind` ("spmm", "mgs_axpy_dot", ...). */
const char* spc_kernel_kind_name(int kind);

/* FP64 FMA throughput of device `device` in TFLOP/s (a dependent-free DFMA
 * probe, best of 5), the roof of this FP64-bound path. */
int spc_fp64_peak(int device, double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* SPINCHEM_GPU_H */
