// Small systems: one CTA carries one sample's whole propagation -- every
// Krylov build, expm, projector Gram, dt loop and psi update until t_end --
// in a single launch (trace_sampling_para's per-sample loop,
// src/qm_dynamics.f90:322-378, with the CTA's threads over rows).
//
// Why: a system of a few hundred rows gives the tiled path (32 samples per
// tile, one launch per phase) kernels of microseconds, so a build round of
// ~90 launches is bound by launch and synchronisation latency, not by the
// FP64 pipe. Here a sample's build is ~1e6 DFMA on its own SM with
// block-level barriers only. Used (SPC_SAMPLE_AUTO) when every job has at
// most SMALL_NMAX rows, m <= 32, a small estimated build and the samples fill
// at most two waves of CTAs (small_path_fits).
//
// Calls with few samples give each sample a cluster of two CTAs instead
// (k_small_pair, below).
//
// Per sample the arithmetic is the tiled path's: the SpMM row loop of k_spmm,
// real-coefficient Lanczos on the Hermitian part (orthonormality checked from
// the projector Grams, MGS rebuild when it fails) or MGS, expm_one, the four
// Hermitian projector Grams, the reference's dt-loop semantics. Reductions
// are two-level and in a fixed order (a warp tree, then warp 0's tree over the
// warps' partials), so results repeat bit for bit; they differ from the tiled
// path's by rounding.
// Control flow is uniform across the CTA: every barrier is reached by all
// threads, and a sample leaves the loop only when the whole CTA does.
#define SMALL_THREADS 256
#define SMALL_WARPS (SMALL_THREADS / 32)
#define SMALL_NC 16      // projector staging: rows per chunk
#define SMALL_VS 17      // staging row stride (padded: rows of one chunk start in different banks)
#define SMALL_MAXC 9     // projector combinations per thread: 4 * 32 * 33 / 2 <= 9 * 256
#define SMALL_MAX_M 32
#define SMALL_ROUNDS 5   // dt-loop pair rounds over 128 threads: 32 * 33 / 2 <= 5 * 128
#define SMALL_NMAX 2048

struct SmallJob {
  int n, Z, me;            // rows, nuclear rows, Krylov dimension min(m, n)
  const int* rowptr;       // execution-order CSR (k_split_rows)
  const int* split;
  const int* col;
  const double2* val;
  const double* kappa;     // non-null: the copy holds A of A - i*kappa*1
  const double2* zk;       // M x Z sample vectors of the job
};

__device__ __forceinline__ double2 warp_sum2(double2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

// Barrier of warps 0-3 (the dt loop's warps; the others wait at the next
// __syncthreads).
__device__ __forceinline__ void small_bar4() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

// Sum over the CTA: warp trees, then warp 0 sums the warps' partials with the
// same tree; every thread gets the total (red holds SMALL_WARPS + 1). Only
// warp 0 spends FP64 adds on the second level. Called by all threads.
__device__ __forceinline__ double2 block_sum2(double2 v, double2* red) {
  v = warp_sum2(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double2 x = threadIdx.x < SMALL_WARPS ? red[threadIdx.x] : cz();
    x = warp_sum2(x);
    if (threadIdx.x == 0) red[SMALL_WARPS] = x;
  }
  __syncthreads();
  return red[SMALL_WARPS];
}

// Real sum over the CTA: warp trees (5 adds), then warp 0 adds the 8 warp
// sums in three shuffle levels. With norm, lane 0 of warp 0 also takes the
// square root and its reciprocal (0 for a zero norm) once for the CTA:
// every thread gets {sum or sqrt, reciprocal} (red holds SMALL_WARPS + 2).
// Called by all threads.
template <bool NORM>
__device__ __forceinline__ double2 block_sum1(double v, double* red) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double x = threadIdx.x < SMALL_WARPS ? red[threadIdx.x] : 0.0;
    x += __shfl_xor_sync(0xffffffffu, x, 4);
    x += __shfl_xor_sync(0xffffffffu, x, 2);
    x += __shfl_xor_sync(0xffffffffu, x, 1);
    if (threadIdx.x == 0) {
      if (NORM) {
        const double b = sqrt(x);
        red[SMALL_WARPS] = b;
        red[SMALL_WARPS + 1] = b > 0.0 ? 1.0 / b : 0.0;
      } else {
        red[SMALL_WARPS] = x;
      }
    }
  }
  __syncthreads();
  return make_double2(red[SMALL_WARPS], red[SMALL_WARPS + 1]);
}

// y = H x for the rows r = tid, tid + nt, ... (k_spmm's per-row order);
// shift adds -i*kappa*x_r.
__device__ __forceinline__ void small_spmm(const SmallJob& J, const double2* __restrict__ x, double2* __restrict__ y,
                                           bool shift, double kap) {
  for (int r = threadIdx.x; r < J.n; r += SMALL_THREADS) {
    const int k0 = __ldg(J.rowptr + r), ks = __ldg(J.split + r), k1 = __ldg(J.rowptr + r + 1);
    double2 a0 = cz(), a1 = cz();
    int k = k0;
    for (; k + 1 < ks; k += 2) {
      a0 = cfma(__ldg(J.val + k), x[__ldg(J.col + k)], a0);
      a1 = cfma(__ldg(J.val + k + 1), x[__ldg(J.col + k + 1)], a1);
    }
    if (k < ks) {
      a0 = cfma(__ldg(J.val + k), x[__ldg(J.col + k)], a0);
      k++;
    }
    for (; k + 1 < k1; k += 2) {
      const double v0 = __ldg(&J.val[k].x), v1 = __ldg(&J.val[k + 1].x);
      const double2 x0 = x[__ldg(J.col + k)], x1 = x[__ldg(J.col + k + 1)];
      a0.x = fma(v0, x0.x, a0.x);
      a0.y = fma(v0, x0.y, a0.y);
      a1.x = fma(v1, x1.x, a1.x);
      a1.y = fma(v1, x1.y, a1.y);
    }
    if (k < k1) {
      const double v0 = __ldg(&J.val[k].x);
      const double2 x0 = x[__ldg(J.col + k)];
      a0.x = fma(v0, x0.x, a0.x);
      a0.y = fma(v0, x0.y, a0.y);
    }
    double2 yv = cadd(a0, a1);
    if (shift) {
      const double2 xr = x[r];
      yv.x = fma(kap, xr.y, yv.x);
      yv.y = fma(-kap, xr.x, yv.y);
    }
    y[r] = yv;
  }
}

// The four projector Grams (k_proj + k_proj_reduce): P_t = V_t^H V_t over
// the Z nuclear rows, V_0 = Q_|aa>, V_1 = Q_|ab> - Q_|ba> (S, halved),
// V_2 = Q_|ab> + Q_|ba> (T0, halved), V_3 = Q_|bb>; staged SMALL_NC rows at
// a time in V (4 m SMALL_VS complex) with Re - Im (Vd) and Re + Im (Vs) of
// every element beside it, so that each conj(a) b takes three products as in
// k_proj: t1 += a_r b_r, t2 += a_i b_i, t3 += (a_r - a_i)(b_r + b_i),
// conj(a) b = (t1 + t2, t3 - t1 + t2). MAXC = ceil(combinations / threads)
// exactly: a combination slot that no thread needs still issues its
// (predicated-off) DFMAs. Ends with a barrier.
template <int MAXC>
__device__ void small_projectors(int m, int me, int n, int Z, const double2* __restrict__ Q, double2* P, double2* V) {
  const int tid = threadIdx.x;
  const size_t mm = (size_t)m * m;
  const int nc4 = me * (me + 1) / 2, ncombo = 4 * nc4;
  double* Vd = reinterpret_cast<double*>(V + 4 * m * SMALL_VS);
  double* Vs = Vd + 4 * m * SMALL_VS;
  // ceil(ncombo / MAXC) threads hold the combinations: the warps past them
  // skip the accumulation instead of issuing predicated-off FMAs
  const int nth = (ncombo + MAXC - 1) / MAXC;
  const bool on = tid < nth;
  double t1[MAXC], t2[MAXC], t3[MAXC];
  int oi[MAXC], oj[MAXC];
#pragma unroll
  for (int q = 0; q < MAXC; ++q) {
    t1[q] = t2[q] = t3[q] = 0.0;
    oi[q] = oj[q] = 0;
    const int cid = tid + q * nth;
    if (on && cid < ncombo) {
      const int t = cid / nc4;
      int rem = cid % nc4, i = 0;
      while (rem >= me - i) {  // (i, j >= i) in row order
        rem -= me - i;
        ++i;
      }
      oi[q] = (t * m + i) * SMALL_VS;
      oj[q] = (t * m + i + rem) * SMALL_VS;
    }
  }
  for (int c0 = 0; c0 < Z; c0 += SMALL_NC) {
    const int len = min(SMALL_NC, Z - c0);
    for (int idx = tid; idx < me * SMALL_NC; idx += SMALL_THREADS) {
      const int j = idx / SMALL_NC, nn = idx % SMALL_NC;
      double2 q1 = cz(), q2 = cz(), q3 = cz(), q4 = cz();
      if (nn < len) {
        const double2* base = Q + (size_t)j * n + c0 + nn;
        q1 = base[0];
        q2 = base[Z];
        q3 = base[2 * Z];
        q4 = base[3 * Z];
      }
      const double2 v[4] = {q1, csub(q2, q3), cadd(q2, q3), q4};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int o = (t * m + j) * SMALL_VS + nn;
        V[o] = v[t];
        Vd[o] = v[t].x - v[t].y;
        Vs[o] = v[t].x + v[t].y;
      }
    }
    __syncthreads();
    if (on)
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
#pragma unroll
  for (int q = 0; q < MAXC; ++q) {
    const int cid = tid + q * nth;
    if (on && cid < ncombo) {
      const int t = cid / nc4;
      int rem = cid % nc4, i = 0;
      while (rem >= me - i) {
        rem -= me - i;
        ++i;
      }
      const int j = i + rem;
      double2 s = make_double2(t1[q] + t2[q], t3[q] - t1[q] + t2[q]);
      if (t == 1 || t == 2) s = make_double2(0.5 * s.x, 0.5 * s.y);
      if (i == j) s.y = 0.0;  // a Gram's diagonal is real; the three-product form leaves rounding there
      double2* Pt = P + t * mm;
      Pt[i + j * m] = s;
      if (i != j) Pt[j + i * m] = make_double2(s.x, -s.y);
    }
  }
  __syncthreads();
}

__device__ void small_projectors_any(int m, int me, int n, int Z, const double2* Q, double2* P, double2* V) {
  const int ncombo = 2 * me * (me + 1);
  switch ((ncombo + SMALL_THREADS - 1) / SMALL_THREADS) {
    case 1: small_projectors<1>(m, me, n, Z, Q, P, V); break;
    case 2: small_projectors<2>(m, me, n, Z, Q, P, V); break;
    case 3: small_projectors<3>(m, me, n, Z, Q, P, V); break;
    case 4: small_projectors<4>(m, me, n, Z, Q, P, V); break;
    case 5: small_projectors<5>(m, me, n, Z, Q, P, V); break;
    case 6: small_projectors<6>(m, me, n, Z, Q, P, V); break;
    case 7: small_projectors<7>(m, me, n, Z, Q, P, V); break;
    case 8: small_projectors<8>(m, me, n, Z, Q, P, V); break;
    default: small_projectors<SMALL_MAXC>(m, me, n, Z, Q, P, V); break;
  }
}

// One Krylov basis of psi (get_krylov, src/qm_dynamics.f90:432-467): A (m x m,
// zeroed first) gets the tridiagonal (lz: Lanczos on the Hermitian part, real
// coefficients, alpha - i*kappa on the diagonal) or the Hessenberg (MGS),
// Q_0..Q_{me-1} the basis, cA = ||psi|| e_1; p is the work vector. Called by
// all SMALL_THREADS threads of the CTA; thread 0 writes A's last entries after
// the last barrier, so the caller synchronises before reading A.
__device__ __forceinline__ void small_krylov(const SmallJob& J, bool lz, bool herm, double kap, int m, double2* A,
                                             double2* cA, double2* Q, double2* p, const double2* psi,
                                             double2* red, double* redd) {
  const int n = J.n, me = J.me, tid = threadIdx.x;
  const size_t mm = (size_t)m * m;
  for (int i = tid; i < (int)mm; i += SMALL_THREADS) A[i] = cz();
  // c = ||psi|| e_1, Q_0 = psi / ||psi|| (get_krylov :440-447)
  double acc = 0.0;
  for (int r = tid; r < n; r += SMALL_THREADS) {
    const double2 x = psi[r];
    acc = fma(x.x, x.x, acc);
    acc = fma(x.y, x.y, acc);
  }
  const double2 bn0 = block_sum1<true>(acc, redd);
  const double b0 = bn0.x, rb0 = bn0.y;
  for (int r = tid; r < n; r += SMALL_THREADS) {
    const double2 x = psi[r];
    Q[r] = make_double2(x.x * rb0, x.y * rb0);
  }
  if (tid < m) cA[tid] = tid == 0 ? make_double2(b0, 0.0) : cz();
  __syncthreads();
  double beta = 0.0;
  for (int i = 0; i < me; ++i) {
    const double2* qi = Q + (size_t)i * n;
    // no barrier: the pass below reads only the rows this thread just wrote
    small_spmm(J, qi, p, !lz && herm, kap);
    if (lz) {
      // p -= beta_{i-1} Q_{i-1}; alpha_i = Re <Q_i, p>
      double a2 = 0.0;
      for (int r = tid; r < n; r += SMALL_THREADS) {
        double2 pv = p[r];
        if (i > 0) {
          const double2 q = qi[r - n];
          pv.x = fma(-beta, q.x, pv.x);
          pv.y = fma(-beta, q.y, pv.y);
          p[r] = pv;
        }
        const double2 x = qi[r];
        a2 = fma(x.x, pv.x, a2);
        a2 = fma(x.y, pv.y, a2);
      }
      const double alpha = block_sum1<false>(a2, redd).x;
      if (tid == 0) A[i + i * m] = make_double2(alpha, -kap);
      if (i < me - 1) {
        double nr = 0.0;
        for (int r = tid; r < n; r += SMALL_THREADS) {
          const double2 q = qi[r];
          double2 pv = p[r];
          pv.x = fma(-alpha, q.x, pv.x);
          pv.y = fma(-alpha, q.y, pv.y);
          p[r] = pv;
          nr = fma(pv.x, pv.x, nr);
          nr = fma(pv.y, pv.y, nr);
        }
        const double2 bn = block_sum1<true>(nr, redd);
        beta = bn.x;
        if (tid == 0) {
          A[(i + 1) + i * m] = make_double2(beta, 0.0);
          A[i + (i + 1) * m] = make_double2(beta, 0.0);
        }
        const double rb = bn.y;
        double2* qn = Q + (size_t)(i + 1) * n;
        for (int r = tid; r < n; r += SMALL_THREADS) {
          const double2 pv = p[r];
          qn[r] = make_double2(pv.x * rb, pv.y * rb);
        }
        __syncthreads();
      }
    } else {
      // MGS (get_krylov :453-456): h_0 = <Q_0, p>; then p -= h_j Q_j
      // fused with h_{j+1} = <Q_{j+1}, p>
      double2 a2 = cz();
      for (int r = tid; r < n; r += SMALL_THREADS) a2 = cjfma(Q[r], p[r], a2);
      double2 hc = block_sum2(a2, red);
      if (tid == 0) A[0 + i * m] = hc;
      for (int j = 0; j < i; ++j) {
        const double2* qj = Q + (size_t)j * n;
        a2 = cz();
        for (int r = tid; r < n; r += SMALL_THREADS) {
          const double2 pv = cfms(hc, qj[r], p[r]);
          p[r] = pv;
          a2 = cjfma(qj[r + n], pv, a2);
        }
        hc = block_sum2(a2, red);
        if (tid == 0) A[(j + 1) + i * m] = hc;
      }
      if (i < me - 1) {
        double nr = 0.0;
        for (int r = tid; r < n; r += SMALL_THREADS) {
          const double2 pv = cfms(hc, qi[r], p[r]);
          p[r] = pv;
          nr = fma(pv.x, pv.x, nr);
          nr = fma(pv.y, pv.y, nr);
        }
        const double2 bn = block_sum1<true>(nr, redd);
        if (tid == 0) A[(i + 1) + i * m] = make_double2(bn.x, 0.0);
        const double rb = bn.y;
        double2* qn = Q + (size_t)(i + 1) * n;
        for (int r = tid; r < n; r += SMALL_THREADS) {
          const double2 pv = p[r];
          qn[r] = make_double2(pv.x * rb, pv.y * rb);
        }
        __syncthreads();
      }
    }
  }
}

// max |sum_t P_t - I| over the me x me block of the four Grams (NaN wins):
// the orthonormality of a Lanczos basis (the Grams sum to Q^H Q). Called by
// all threads; every thread gets the maximum.
__device__ __forceinline__ double small_ortho_err(int me, int m, const double2* P, double* terms, double* cstat) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t mm = (size_t)m * m;
  double mx = 0.0;
  for (int id = tid; id < me * me; id += SMALL_THREADS) {
    const int i = id % me, j = id / me;
    const size_t x = (size_t)i + (size_t)j * m;
    const double2 g = cadd(cadd(P[x], P[mm + x]), cadd(P[2 * mm + x], P[3 * mm + x]));
    const double e = fmax(fabs(g.x - (i == j ? 1.0 : 0.0)), fabs(g.y));
    mx = (e > mx || e != e) ? e : mx;
  }
  for (int d = 16; d > 0; d >>= 1) {
    const double v = __shfl_xor_sync(0xffffffffu, mx, d);
    mx = (v > mx || v != v) ? v : mx;
  }
  if (lane == 0) terms[warp] = mx;
  __syncthreads();
  if (warp == 0) {
    double v = lane < SMALL_WARPS ? terms[lane] : 0.0;
    for (int d = 16; d > 0; d >>= 1) {
      const double u = __shfl_xor_sync(0xffffffffu, v, d);
      v = (u > v || u != u) ? u : v;
    }
    if (lane == 0) cstat[0] = v;
  }
  __syncthreads();
  const double mall = cstat[0];
  __syncthreads();
  return mall;
}

// Grid: one CTA of SMALL_THREADS per sample (global sample s = blockIdx.x).
// work + soff[s]: the sample's basis (m x n), work vector (n) and state (n);
// with vec_smem they live in shared memory instead (every job's (m+2) n
// complex fits there), which cuts the latency of the row sweeps.
// Dynamic shared memory: A, E (m^2 each), P (4 m^2), c and c' (m each),
// max(5 m^2, 8 m SMALL_VS) of expm / projector scratch, all complex, then
// the vectors when vec_smem.
__global__ void __launch_bounds__(SMALL_THREADS, 2)
    k_small_prop(const SmallJob* __restrict__ jobs, const int* __restrict__ sjob, const int* __restrict__ scol,
                 const int64_t* __restrict__ soff, double2* __restrict__ work, Theta th, int m, int T, double dt,
                 double t_end, double tol, int lanczos, int vec_smem, double* __restrict__ obs,
                 long long* __restrict__ nsteps, unsigned long long* __restrict__ counts, int* __restrict__ err) {
  extern __shared__ double2 smem[];
  __shared__ double rowsum[SPC_MAX_M];
  __shared__ int piv[SPC_MAX_M];
  __shared__ int s_sh, p_sh;
  __shared__ double2 red[SMALL_WARPS + 1];
  double* redd = reinterpret_cast<double*>(red);  // block_sum1's SMALL_WARPS + 2 doubles
  __shared__ double2 part[SMALL_WARPS][32];
  __shared__ double terms[16];
  __shared__ double cstat[2];
  __shared__ double loop_t;
  __shared__ int loop_k, loop_done;
  __shared__ long long loop_steps;

  const int s = blockIdx.x;
  const SmallJob J = jobs[sjob[s]];
  const int n = J.n, Z = J.Z, me = J.me;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t mm = (size_t)m * m;
  double2* A = smem;
  double2* E = A + mm;
  double2* P = E + mm;
  double2* cA = P + 4 * mm;
  double2* cB = cA + m;
  double2* X = cB + m;
  double2* Q = vec_smem ? X + std::max<size_t>(5 * mm, 8 * (size_t)m * SMALL_VS) : work + soff[s];
  double2* p = Q + (size_t)m * n;
  double2* psi = p + n;
  const bool herm = J.kappa != nullptr;
  const double kap = herm ? *J.kappa : 0.0;
  const double2* zk = J.zk + (size_t)scol[s] * Z;
  double* o = obs + (size_t)s * 4 * T;

  // psi_0 = theta (x) z (kron_vector)
  for (int r = tid; r < n; r += SMALL_THREADS) psi[r] = cmul(th.v[r / Z], zk[r % Z]);
  __syncthreads();
  double t = 0.0;
  int k = 1;  // outputs 0 hold the initial populations (k_obs_init)
  long long steps = 0;
  unsigned long long nb = 0, nf = 0;
  bool done = !(0.0 < t_end);
  while (!done) {
    bool lz = lanczos != 0 && herm;
    for (int attempt = 0; attempt < 2; ++attempt) {
      small_krylov(J, lz, herm, kap, m, A, cA, Q, p, psi, red, redd);
      small_projectors_any(m, me, n, Z, Q, P, X);
      if (!lz) break;
      // a Lanczos basis must be orthonormal: max |sum_t P_t - I| <= ORTHO_TOL
      const double mall = small_ortho_err(me, m, P, terms, cstat);
      if (mall <= ORTHO_TOL) break;
      nf++;
      lz = false;  // rebuild this basis with full MGS
    }
    nb++;
    expm_one<false>(me, m, A, E, dt, X, rowsum, piv, &s_sh, &p_sh, tid, SMALL_THREADS, err);
    __syncthreads();
    // dt loop (:348-364): c <- E c; P_X(t) = Re(c^H P_X c); stop when the
    // last Krylov coordinate grows past tol or the window ends. It runs on
    // warps 0-3, one per scheduler: GB300's FP64 pipe sits in each scheduler
    // and a warp instruction holds it for the same time whatever its active
    // lanes, so the step is laid out to issue few FP64 warp instructions:
    //  * c' = E c with lane = row and warp w over the columns j = w mod 4 (c_j
    //    by shuffle); every warp adds the four partials in warp order, so
    //    each holds c' in its lanes and no further barrier is needed;
    //  * the four forms over the pairs i <= j, with the Hermitian weights in
    //    W = (s Re P_ij, -s Im P_ij) (s = 1 on the diagonal, 2 above it) and
    //    g_ij = conj(c_i) c_j shared by the types: 12 FP64 operations a pair;
    //  * each warp's four sums by a reduce-scatter over its lanes (6 adds
    //    instead of 20), then the warps' sums added in warp order.
    // Warps 4-7 wait at the barrier after the loop.
    const int npair = me * (me + 1) / 2;
    double2* W = X;  // 4 x npair weights in the spent expm scratch
    for (int idx = tid; idx < 4 * npair; idx += SMALL_THREADS) {
      const int ty = idx / npair;
      int rem = idx % npair, i = 0;
      while (rem >= me - i) {
        rem -= me - i;
        ++i;
      }
      const double2 pv = P[ty * mm + i + (size_t)(i + rem) * m];
      const double sw = rem == 0 ? 1.0 : 2.0;
      W[idx] = make_double2(sw * pv.x, -sw * pv.y);
    }
    __syncthreads();
    if (warp < 4) {
      int pi[SMALL_ROUNDS], pj[SMALL_ROUNDS];
#pragma unroll
      for (int r = 0; r < SMALL_ROUNDS; ++r) {
        pi[r] = -1;
        pj[r] = 0;
        int rem = r * 128 + tid;
        if (rem < npair) {
          int i = 0;
          while (rem >= me - i) {
            rem -= me - i;
            ++i;
          }
          pi[r] = i;
          pj[r] = i + rem;
        }
      }
      double2 c = lane < me ? cA[lane] : cz();
      double c2 = 1.0, cm2 = 0.0;
      while (cm2 <= tol * c2 && t < t_end) {
        if (k >= T) {  // output full (guard; every thread takes it)
          if (tid == 0) atomicExch(err, 1);
          done = true;
          break;
        }
        double2 a = cz();
        for (int j = warp; j < me; j += 4) {
          const double2 cj = make_double2(__shfl_sync(0xffffffffu, c.x, j), __shfl_sync(0xffffffffu, c.y, j));
          if (lane < me) a = cfma(E[lane + j * m], cj, a);
        }
        part[warp][lane] = a;
        small_bar4();
        double2 cn = cz();
        if (lane < me) cn = cadd(cadd(cadd(part[0][lane], part[1][lane]), part[2][lane]), part[3][lane]);
        double f0 = 0.0, f1 = 0.0, f2 = 0.0, f3 = 0.0;
#pragma unroll
        for (int r = 0; r < SMALL_ROUNDS; ++r) {
          if (r * 128 + warp * 32 >= npair) break;  // no pair of this warp left
          const int i = max(pi[r], 0), j = pj[r];
          const double cix = __shfl_sync(0xffffffffu, cn.x, i), ciy = __shfl_sync(0xffffffffu, cn.y, i);
          const double cjx = __shfl_sync(0xffffffffu, cn.x, j), cjy = __shfl_sync(0xffffffffu, cn.y, j);
          if (pi[r] >= 0) {
            const double gx = fma(cix, cjx, ciy * cjy), gy = fma(cix, cjy, -ciy * cjx);
            const int pp = r * 128 + tid;
            const double2 w0 = W[pp], w1 = W[npair + pp], w2 = W[2 * npair + pp], w3 = W[3 * npair + pp];
            f0 = fma(w0.x, gx, fma(w0.y, gy, f0));
            f1 = fma(w1.x, gx, fma(w1.y, gy, f1));
            f2 = fma(w2.x, gx, fma(w2.y, gy, f2));
            f3 = fma(w3.x, gx, fma(w3.y, gy, f3));
          }
        }
        // reduce-scatter: lanes 8t..8t+7 end with the warp's sum of form t
        const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0;
        double ka = h16 ? f2 : f0, kb = h16 ? f3 : f1;
        ka += __shfl_xor_sync(0xffffffffu, h16 ? f0 : f2, 16);
        kb += __shfl_xor_sync(0xffffffffu, h16 ? f1 : f3, 16);
        double v = h8 ? kb : ka;
        v += __shfl_xor_sync(0xffffffffu, h8 ? ka : kb, 8);
        v += __shfl_xor_sync(0xffffffffu, v, 4);
        v += __shfl_xor_sync(0xffffffffu, v, 2);
        v += __shfl_xor_sync(0xffffffffu, v, 1);
        if ((lane & 7) == 0) terms[4 * warp + (lane >> 3)] = v;
        if (warp == 3) {  // the warp with the fewest pairs: |c'|^2, |c'_{m-1}|^2
          double nn = lane < me ? fma(cn.x, cn.x, cn.y * cn.y) : 0.0;
          nn = warp_sum(nn);
          if (lane == 0) cstat[0] = nn;
          if (lane == me - 1) cstat[1] = cn.x * cn.x + cn.y * cn.y;
        }
        small_bar4();
        if (tid < 4) {
          const int slot = tid == 0 ? 2 : (tid == 1 ? 0 : (tid == 2 ? 1 : 3));  // proj type -> obs slot
          o[slot * T + k] = ((terms[tid] + terms[4 + tid]) + terms[8 + tid]) + terms[12 + tid];
        }
        c2 = cstat[0];
        cm2 = cstat[1];
        c = cn;
        t = t + dt;
        k = k + 1;
        steps++;
      }
      if (warp == 0 && lane < me) cA[lane] = c;  // for psi = Q c
      if (tid == 0) {
        loop_t = t;
        loop_k = k;
        loop_steps = steps;
        loop_done = done ? 1 : 0;
      }
    }
    __syncthreads();
    t = loop_t;
    k = loop_k;
    steps = loop_steps;
    done = loop_done != 0;
    const double2* c = cA;
    if (!done) done = !(t < t_end);
    if (!done) {
      // psi = Q c (:365)
      for (int r = tid; r < n; r += SMALL_THREADS) {
        double2 acc3 = cz();
        for (int j = 0; j < me; ++j) acc3 = cfma(Q[(size_t)j * n + r], c[j], acc3);
        psi[r] = acc3;
      }
    }
    // c lives in cA; the next build rewrites it after a barrier
    __syncthreads();
  }
  if (tid == 0) {
    atomicAdd((unsigned long long*)nsteps, (unsigned long long)steps);
    atomicAdd(&counts[0], nb);
    atomicAdd(&counts[1], nf);
  }
}

// ---------------------------------------------------------------------------
// Pair form: a cluster of two CTAs per sample, for calls whose clusters are
// all resident at once (at most half as many samples as SMs: the dim-288
// workload runs 64 samples on 152 SMs, so one CTA per sample leaves 88 SMs
// idle). The main CTA (cluster rank 0) keeps
// the sample's serial path: the Krylov builds, the expm, the recurrence
// c <- E c of the dt loop with its stop test, and psi = Q c. The helper CTA
// (rank 1) takes the work off that path:
//  * the four projector Grams, staged from the main CTA's basis through
//    distributed shared memory, and the Lanczos orthonormality check, while
//    the main CTA runs the expm of the same basis;
//  * the populations Re(c^H P_X c) of every dt step, from the coordinates c
//    that the main CTA's dt loop stores into the helper's shared memory in
//    segments of at most hmax steps (two buffers): the helper evaluates a
//    segment while the main CTA runs the next one, psi = Q c and the next
//    Krylov build.
// The main CTA's dt step is then c' = E c on four warps (one barrier) and the
// stop test, which each of the four warps evaluates on its own copy of c'.
// Control flow is uniform across the cluster: a flag that ends a loop is
// written to both CTAs' shared memory before a cluster barrier and read after
// it, and every thread of both CTAs reaches every cluster barrier. The
// arithmetic is k_small_prop's except for the order in which the populations
// add their pair terms (each lane's pairs in order, then a shuffle tree), so
// populations agree with it to rounding and the rebuild schedule is the same.
struct PairCtrl {
  int ok;       // the basis passed the orthonormality check (written by the helper)
  int cnt[2];   // per history buffer (written by the main CTA): steps in the segment,
  int k0[2];    // output index of its first step,
  int more[2];  // whether the build continues past it,
  int done[2];  // whether the sample's propagation has ended
};

// Populations of cnt consecutive dt steps from their Krylov coordinates
// (hist[st * m + i]), with the build's Hermitian weights W (4 x npair) and
// pair table: step st on warp st mod SMALL_WARPS, the lanes over the pairs
// (each lane adds its pairs' terms in order), then k_small_prop's
// reduce-scatter; lanes 0, 8, 16, 24 write the four populations of output
// index k0 + st. Called by all threads of the helper CTA.
__device__ __forceinline__ void small_pair_forms(int cnt, int k0, int m, int npair, const double2* hist,
                                                 const double2* W, const int2* pij, double* o, int T) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int st = warp; st < cnt; st += SMALL_WARPS) {
    const double2* cv = hist + (size_t)st * m;
    double f0 = 0.0, f1 = 0.0, f2 = 0.0, f3 = 0.0;
    for (int pp = lane; pp < npair; pp += 32) {
      const int2 ij = pij[pp];
      const double2 ci = cv[ij.x], cj = cv[ij.y];
      const double gx = fma(ci.x, cj.x, ci.y * cj.y), gy = fma(ci.x, cj.y, -ci.y * cj.x);
      const double2 w0 = W[pp], w1 = W[npair + pp], w2 = W[2 * npair + pp], w3 = W[3 * npair + pp];
      f0 = fma(w0.x, gx, fma(w0.y, gy, f0));
      f1 = fma(w1.x, gx, fma(w1.y, gy, f1));
      f2 = fma(w2.x, gx, fma(w2.y, gy, f2));
      f3 = fma(w3.x, gx, fma(w3.y, gy, f3));
    }
    const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0;
    double ka = h16 ? f2 : f0, kb = h16 ? f3 : f1;
    ka += __shfl_xor_sync(0xffffffffu, h16 ? f0 : f2, 16);
    kb += __shfl_xor_sync(0xffffffffu, h16 ? f1 : f3, 16);
    double v = h8 ? kb : ka;
    v += __shfl_xor_sync(0xffffffffu, h8 ? ka : kb, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    if ((lane & 7) == 0) {
      const int ty = lane >> 3;
      const int slot = ty == 0 ? 2 : (ty == 1 ? 0 : (ty == 2 ? 1 : 3));  // proj type -> obs slot
      o[(size_t)slot * T + k0 + st] = v;
    }
  }
}

// Dynamic shared memory of k_small_pair (complex elements). Main CTA: A, E
// (m^2 each), c (m), expm scratch (5 m^2), then the vectors when vec_smem.
// Helper CTA: P (4 m^2), projector staging (8 m SMALL_VS), weights
// (4 m(m+1)/2), pair table (m(m+1)/2 int2), history (2 hmax m).
__host__ __device__ __forceinline__ size_t pair_main_elems(int m, int n, bool vec_smem) {
  const size_t mm = (size_t)m * m;
  return 7 * mm + (size_t)m + (vec_smem ? (size_t)(m + 2) * n : 0);
}
__host__ __device__ __forceinline__ size_t pair_help_elems(int m, int hmax) {
  const size_t mm = (size_t)m * m, np = (size_t)m * (m + 1) / 2;
  return 4 * mm + 8 * (size_t)m * SMALL_VS + 4 * np + (np + 1) / 2 + 2 * (size_t)hmax * m;
}

// Grid: two CTAs per sample (global sample s = blockIdx.x / 2), clusters of
// two; arguments as k_small_prop's, plus hmax (steps per history buffer).
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(SMALL_THREADS, 1)
    k_small_pair(const SmallJob* __restrict__ jobs, const int* __restrict__ sjob, const int* __restrict__ scol,
                 const int64_t* __restrict__ soff, double2* __restrict__ work, Theta th, int m, int T, double dt,
                 double t_end, double tol, int lanczos, int vec_smem, int hmax, double* __restrict__ obs,
                 long long* __restrict__ nsteps, unsigned long long* __restrict__ counts, int* __restrict__ err) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ double2 smem[];
  __shared__ double rowsum[SPC_MAX_M];
  __shared__ int piv[SPC_MAX_M];
  __shared__ int s_sh, p_sh;
  __shared__ double2 red[SMALL_WARPS + 1];
  double* redd = reinterpret_cast<double*>(red);
  __shared__ double2 part[2][4][32];
  __shared__ double terms[16];
  __shared__ double cstat[2];
  __shared__ PairCtrl ctrl;

  const int rank = (int)cluster.block_rank();
  const int s = blockIdx.x >> 1;
  const SmallJob J = jobs[sjob[s]];
  const int n = J.n, Z = J.Z, me = J.me;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t mm = (size_t)m * m;
  const int npair = me * (me + 1) / 2;
  // main CTA's layout
  double2* A = smem;
  double2* E = A + mm;
  double2* cA = E + mm;
  double2* X = cA + m;
  double2* Q = vec_smem ? X + 5 * mm : work + soff[s];
  double2* p = Q + (size_t)m * n;
  double2* psi = p + n;
  // helper CTA's layout
  const size_t np_max = (size_t)m * (m + 1) / 2;
  double2* P = smem;
  double2* V = P + 4 * mm;
  double2* W = V + 8 * (size_t)m * SMALL_VS;
  int2* pij = reinterpret_cast<int2*>(W + 4 * np_max);
  double2* H = W + 4 * np_max + (np_max + 1) / 2;
  // the other CTA's shared memory
  PairCtrl* ctrl_main = cluster.map_shared_rank(&ctrl, 0);
  PairCtrl* ctrl_help = cluster.map_shared_rank(&ctrl, 1);
  double2* H_help = cluster.map_shared_rank(H, 1);
  const double2* Q_main = vec_smem ? cluster.map_shared_rank(Q, 0) : Q;
  const bool herm = J.kappa != nullptr;
  const double kap = herm ? *J.kappa : 0.0;
  double* o = obs + (size_t)s * 4 * T;

  if (rank == 0) {
    // psi_0 = theta (x) z (kron_vector)
    const double2* zk = J.zk + (size_t)scol[s] * Z;
    for (int r = tid; r < n; r += SMALL_THREADS) psi[r] = cmul(th.v[r / Z], zk[r % Z]);
  }
  __syncthreads();
  double t = 0.0;
  int k = 1;  // outputs 0 hold the initial populations (k_obs_init)
  long long steps = 0;
  unsigned long long nb = 0, nf = 0;
  bool done = !(0.0 < t_end);
  while (!done) {
    bool lz = lanczos != 0 && herm;
    for (int attempt = 0; attempt < 2; ++attempt) {
      if (rank == 0) small_krylov(J, lz, herm, kap, m, A, cA, Q, p, psi, red, redd);
      cluster.sync();  // basis, A and c complete
      if (rank == 0) {
        expm_one<false>(me, m, A, E, dt, X, rowsum, piv, &s_sh, &p_sh, tid, SMALL_THREADS, err);
      } else {
        small_projectors_any(m, me, n, Z, Q_main, P, V);
        // a Lanczos basis must be orthonormal: max |sum_t P_t - I| <= ORTHO_TOL
        const bool okv = !lz || small_ortho_err(me, m, P, terms, cstat) <= ORTHO_TOL;
        if (tid == 0) {
          ctrl.ok = okv ? 1 : 0;
          ctrl_main->ok = okv ? 1 : 0;
        }
      }
      cluster.sync();  // Grams, check and exponential complete
      if (ctrl.ok) break;
      nf++;
      lz = false;  // rebuild this basis with full MGS
    }
    nb++;
    if (rank == 1) {
      // Hermitian weights W_t = (s Re P_t, -s Im P_t) of the pairs i <= j
      // (s = 1 on the diagonal, 2 above it) and the pair table
      for (int idx = tid; idx < 4 * npair; idx += SMALL_THREADS) {
        const int ty = idx / npair;
        int rem = idx % npair, i = 0;
        while (rem >= me - i) {
          rem -= me - i;
          ++i;
        }
        const double2 pv = P[ty * mm + i + (size_t)(i + rem) * m];
        const double sw = rem == 0 ? 1.0 : 2.0;
        W[idx] = make_double2(sw * pv.x, -sw * pv.y);
        if (ty == 0) pij[idx] = make_int2(i, i + rem);
      }
      __syncthreads();
    }
    // dt loop (:348-364) in segments of at most hmax steps. Main CTA, warps
    // 0-3: c' = E c with lane = row and warp w over the columns j = w mod 4
    // (c_j by shuffle), the four partials (double-buffered by step parity)
    // added in warp order by every warp, |c'|^2 and |c'_{me-1}|^2 by every
    // warp for the stop test; warp 0 stores c' into the helper's history.
    double2 c = (rank == 0 && lane < me) ? cA[lane] : cz();
    double c2 = 1.0, cm2 = 0.0;
    int buf = 0;
    for (;;) {
      if (rank == 0) {
        if (warp < 4) {
          double2* hist = H_help + (size_t)buf * hmax * m;
          const int k0 = k;
          int cnt = 0;
          bool overflow = false;
          while (cnt < hmax && cm2 <= tol * c2 && t < t_end) {
            if (k >= T) {  // output full (guard; every chain thread takes it)
              overflow = true;
              break;
            }
            double2 a = cz();
            for (int j = warp; j < me; j += 4) {
              const double2 cj = make_double2(__shfl_sync(0xffffffffu, c.x, j), __shfl_sync(0xffffffffu, c.y, j));
              if (lane < me) a = cfma(E[lane + j * m], cj, a);
            }
            part[cnt & 1][warp][lane] = a;
            small_bar4();
            double2 cn = cz();
            if (lane < me)
              cn = cadd(cadd(cadd(part[cnt & 1][0][lane], part[cnt & 1][1][lane]), part[cnt & 1][2][lane]),
                        part[cnt & 1][3][lane]);
            const double nn = lane < me ? fma(cn.x, cn.x, cn.y * cn.y) : 0.0;
            c2 = warp_sum(nn);
            cm2 = __shfl_sync(0xffffffffu, cn.x * cn.x + cn.y * cn.y, me - 1);
            if (warp == 0 && lane < me) hist[(size_t)cnt * m + lane] = cn;
            c = cn;
            t = t + dt;
            k = k + 1;
            steps++;
            cnt++;
          }
          const bool more = !overflow && cnt == hmax && cm2 <= tol * c2 && t < t_end;
          const bool dn = overflow || (!more && !(t < t_end));
          if (tid == 0) {
            if (overflow) atomicExch(err, 1);
            ctrl.more[buf] = more ? 1 : 0;
            ctrl.done[buf] = dn ? 1 : 0;
            ctrl_help->cnt[buf] = cnt;
            ctrl_help->k0[buf] = k0;
            ctrl_help->more[buf] = more ? 1 : 0;
            ctrl_help->done[buf] = dn ? 1 : 0;
          }
          if (!more && warp == 0 && lane < me) cA[lane] = c;  // for psi = Q c
        }
        __syncthreads();
      }
      // history segment and flags visible to the helper; the flags of buffer
      // buf are next written two segments on, after a cluster barrier that
      // every thread reaches only once it has read them here
      cluster.sync();
      const bool more = ctrl.more[buf] != 0;
      done = ctrl.done[buf] != 0;
      if (rank == 1)
        small_pair_forms(ctrl.cnt[buf], ctrl.k0[buf], m, npair, H + (size_t)buf * hmax * m, W, pij, o, T);
      if (!more) break;
      buf ^= 1;
    }
    if (rank == 0 && !done) {
      // psi = Q c (:365)
      for (int r = tid; r < n; r += SMALL_THREADS) {
        double2 acc3 = cz();
        for (int j = 0; j < me; ++j) acc3 = cfma(Q[(size_t)j * n + r], cA[j], acc3);
        psi[r] = acc3;
      }
    }
    __syncthreads();
  }
  // keep the helper's shared memory alive until the main CTA's last remote
  // access has completed
  cluster.sync();
  if (rank == 0 && tid == 0) {
    atomicAdd((unsigned long long*)nsteps, (unsigned long long)steps);
    atomicAdd(&counts[0], nb);
    atomicAdd(&counts[1], nf);
  }
}

// Dynamic shared memory of k_small_prop for Krylov dimension m (bytes),
// without the vectors.
static size_t small_smem_bytes(int m) {
  const size_t mm = (size_t)m * m;
  return sizeof(double2) * (6 * mm + 2 * (size_t)m + std::max<size_t>(5 * mm, 8 * (size_t)m * SMALL_VS));
}

// Whether a call runs on k_small_prop (sets smem). Rows, m, shared memory
// and device memory must fit; in SPC_SAMPLE_AUTO mode also every job's build
// must be small (an estimate of its FP64 FMAs: SpMM, passes, projectors,
// expm) and the samples at most two waves of resident CTAs.
static bool small_path_fits(Handle* h, const std::vector<JobSpec>& jobs, int m, int T, size_t& smem) {
  if (m > SMALL_MAX_M || jobs.empty()) return false;
  int64_t G = 0;
  double bytes = 0.0, wmax = 0.0;
  for (const JobSpec& j : jobs) {
    if (j.n > SMALL_NMAX || j.n < 4 || j.M < 1) return false;
    G += j.M;
    bytes += 16.0 * (double)(m + 2) * j.n * j.M;
    const double me = std::min(m, j.n), n = j.n;
    // MGS rounds (rates unequal, or MGS requested) add ~m^2 n/2 complex FMAs
    const bool mgs = !(h->krylov_method == 1 || h->krylov_method == 2) || !j.herm_shift;
    wmax = std::max(wmax, 4.0 * me * (double)j.nnz + 16.0 * me * n + 2.0 * n * me * me + 48.0 * me * me * me +
                              (mgs ? 2.0 * me * me * n : 0.0));
  }
  if (G > INT32_MAX) return false;
  bytes += 32.0 * T * (double)G + 16.0 * (double)G;
  smem = small_smem_bytes(m);
  if (smem > h->smem_optin) return false;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return false;
  double held = 0.0;
  for (const Handle::Buf* b : {&h->Q, &h->obs, &h->tt, &h->kk, &h->done}) held += (double)b->bytes;
  double budget = (double)free_b + held - (512.0 * (1 << 20) + 0.02 * (double)total_b);
  if (h->mem_limit) budget = std::min(budget, (double)h->mem_limit);
  if (bytes > budget) return false;
  if (h->sample_path == SPC_SAMPLE_ON || h->sample_path == SPC_SAMPLE_SINGLE) return true;
  if (cudaFuncSetAttribute(k_small_prop, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return false;
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_small_prop, SMALL_THREADS, smem) != cudaSuccess) return false;
  return wmax <= 2.5e6 && G <= 2LL * h->sm_count * std::max(1, b);
}

// propagate_batch on k_small_prop: one launch for every sample of every job,
// then the per-job average (k_average).
static int propagate_small(Handle* h, const double* theta, const double* init_pop, const std::vector<JobSpec>& jobs,
                           double dt, double t_end, int m, double tol, int T, size_t smem) {
  auto t_start = std::chrono::steady_clock::now();
  cudaStream_t st = h->stream;
  const int nj = (int)jobs.size();
  int G = 0;
  for (const JobSpec& j : jobs) G += j.M;
  std::vector<SmallJob> sj(nj);
  std::vector<JobOut> jo(nj);
  std::vector<int> sjob(G), scol(G);
  std::vector<int64_t> soff(G);
  bool lanczos = h->krylov_method == 1 || h->krylov_method == 2;
  int64_t wt = 0;
  for (int k = 0, g = 0; k < nj; ++k) {
    const JobSpec& j = jobs[k];
    lanczos = lanczos && j.herm_shift;
    sj[k] = SmallJob{j.n, j.n / 4, std::min(m, j.n), j.rowptr, j.split, j.col, j.val,
                     j.herm_shift ? j.kappa : nullptr, j.zk};
    jo[k] = JobOut{g, j.M, j.out};
    for (int s = 0; s < j.M; ++s, ++g) {
      sjob[g] = k;
      scol[g] = s;
      soff[g] = wt;
      wt += (int64_t)(m + 2) * j.n;
    }
  }
  // plan: jobs | sample -> job | sample -> column | sample -> work offset
  const size_t o_sjob = sizeof(SmallJob) * nj;
  const size_t o_scol = o_sjob + sizeof(int) * G;
  const size_t o_soff = (o_scol + sizeof(int) * G + 7) / 8 * 8;
  const size_t plan_bytes = o_soff + sizeof(int64_t) * G;
  if (h->ensure(h->Q, sizeof(double2) * wt) || h->ensure(h->obs, sizeof(double) * 4 * (size_t)T * G) ||
      h->ensure(h->tt, sizeof(double) * G) || h->ensure(h->kk, sizeof(int) * G) ||
      h->ensure(h->done, sizeof(int) * G) || h->ensure(h->err, 32) || h->ensure(h->plan, plan_bytes) ||
      h->ensure(h->jobtab, sizeof(JobOut) * nj + 64))
    return SPC_ERR_ALLOC;
  std::vector<char> hp(plan_bytes);
  std::memcpy(hp.data(), sj.data(), sizeof(SmallJob) * nj);
  std::memcpy(hp.data() + o_sjob, sjob.data(), sizeof(int) * G);
  std::memcpy(hp.data() + o_scol, scol.data(), sizeof(int) * G);
  std::memcpy(hp.data() + o_soff, soff.data(), sizeof(int64_t) * G);
  char* plan = (char*)h->plan.p;
  int64_t launches0 = h->launches;
  CK(cudaMemcpyAsync(plan, hp.data(), plan_bytes, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(h->jobtab.p, jo.data(), sizeof(JobOut) * nj, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(h->err.p, 0, 32, st));
  double* d_obs = (double*)h->obs.p;
  // slots past a sample's last step stay zero, as the reference's arrays
  CK(cudaMemsetAsync(d_obs, 0, sizeof(double) * 4 * (size_t)T * G, st));
  k_obs_init<<<(G + 127) / 128, 128, 0, st>>>(G, T, init_pop[0], init_pop[1], init_pop[2], init_pop[3], d_obs,
                                               (double*)h->tt.p, (int*)h->kk.p, (int*)h->done.p);
  h->count_launch();
  Theta th;
  for (int e = 0; e < 4; ++e) th.v[e] = make_double2(theta[2 * e], theta[2 * e + 1]);
  // the vectors in shared memory when every job's fit beside the matrices
  int nmax = 0;
  for (const JobSpec& j : jobs) nmax = std::max(nmax, j.n);
  const size_t budget = h->smem_optin > 8192 ? h->smem_optin - 8192 : 0;  // less the static shared memory
  int* d_err = (int*)h->err.p;
  long long* d_nsteps = (long long*)((char*)h->err.p + 8);
  unsigned long long* d_counts = (unsigned long long*)((char*)h->err.p + 16);
  // pair form (two CTAs per sample) when the samples fill at most half the
  // SMs and its shared memory fits: history buffers of up to 64 steps
  bool pair = h->sample_path != SPC_SAMPLE_SINGLE && 2 * (int64_t)G <= h->sm_count;
  CK(cudaGetLastError());  // a failed query below is cleared, not an earlier error
  int hmax = 64;
  size_t psmem = 0;
  bool pvec = false;
  if (pair) {
    while (hmax > 8 && sizeof(double2) * pair_help_elems(m, hmax) > budget) hmax /= 2;
    const size_t help = sizeof(double2) * pair_help_elems(m, hmax);
    pvec = sizeof(double2) * pair_main_elems(m, nmax, true) <= budget;
    psmem = std::max(help, sizeof(double2) * pair_main_elems(m, nmax, pvec));
    pair = psmem <= budget &&
           cudaFuncSetAttribute(k_small_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem) == cudaSuccess;
    if (pair) {
      // every cluster resident at once (SMs pair up within a GPC, so this can
      // be fewer than half the SMs)
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(2 * G);
      cfg.blockDim = dim3(SMALL_THREADS);
      cfg.dynamicSmemBytes = psmem;
      cfg.stream = st;
      int ncl = 0;
      pair = cudaOccupancyMaxActiveClusters(&ncl, k_small_pair, &cfg) == cudaSuccess && ncl >= G;
    }
    if (!pair) (void)cudaGetLastError();  // fall back to one CTA per sample
  }
  int pe = h->prof.begin(st);
  if (pair) {
    k_small_pair<<<2 * G, SMALL_THREADS, psmem, st>>>((const SmallJob*)plan, (const int*)(plan + o_sjob),
                                                      (const int*)(plan + o_scol), (const int64_t*)(plan + o_soff),
                                                      (double2*)h->Q.p, th, m, T, dt, t_end, tol, lanczos ? 1 : 0,
                                                      pvec ? 1 : 0, hmax, d_obs, d_nsteps, d_counts, d_err);
  } else {
    const size_t vbytes = sizeof(double2) * (size_t)(m + 2) * nmax;
    const bool vec_smem = smem + vbytes + 8192 <= h->smem_optin;
    if (vec_smem) smem += vbytes;
    CK(cudaFuncSetAttribute(k_small_prop, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_small_prop<<<G, SMALL_THREADS, smem, st>>>((const SmallJob*)plan, (const int*)(plan + o_sjob),
                                                 (const int*)(plan + o_scol), (const int64_t*)(plan + o_soff),
                                                 (double2*)h->Q.p, th, m, T, dt, t_end, tol, lanczos ? 1 : 0,
                                                 vec_smem ? 1 : 0, d_obs,
                                                 d_nsteps, d_counts, d_err);
  }
  h->prof.end(st, pe, PK_SAMPLE, 0.0, 0.0);
  h->count_launch();
  for (int j0 = 0; j0 < nj; j0 += 65535) {
    const int cnt = std::min(65535, nj - j0);
    k_average<<<dim3((4 * T + 255) / 256, cnt), 256, 0, st>>>((const JobOut*)h->jobtab.p, j0, T, d_obs);
    h->count_launch();
  }
  CK(cudaGetLastError());
  unsigned char eh[32];
  CK(cudaMemcpyAsync(eh, h->err.p, 32, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  h->prof.collect();
  int err0 = 0;
  long long nsteps = 0;
  unsigned long long counts[2] = {0, 0};
  std::memcpy(&err0, eh, 4);
  std::memcpy(&nsteps, eh + 8, 8);
  std::memcpy(counts, eh + 16, 16);
  h->stats.krylov_builds = (int64_t)counts[0];
  h->stats.lanczos_fallbacks = (int64_t)counts[1];
  h->stats.rounds = 1;
  h->stats.sample_steps = nsteps;
  h->stats.kernel_launches = h->launches - launches0;
  h->stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  if (err0 == 1) return set_error(SPC_ERR_NUMERIC, "time index overflow: the dt loop ran past %d output slots", T);
  if (err0 == 2) return set_error(SPC_ERR_NUMERIC, "singular Pade denominator in expm");
  return SPC_OK;
}
