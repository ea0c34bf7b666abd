// Adjoint gradient of the radical-pair yields (spc_yield_gradient and
// spc_yield_gradient_batch: many systems of uneven dimension in one sweep). Included
// at the end of spc_propagate.cu, inside namespace spc, so that it reuses the
// Krylov kernels defined there.
//
// Model: the stepwise propagation psi_{k+1} = exp(-i H dt) psi_k of every
// sample (a fresh Krylov basis each dt step, no data-dependent basis reuse,
// so the objective is a smooth function of the parameters), populations
// P_X(k) = <psi_k|Pi_X|psi_k> averaged over the samples, and the yields of
// get_kinetics (src/observables.f90:74-101): Phi_X = k_X sum_k c_k P_X(k)
// with Simpson weights c_k = dt/3 {1, 4, 2, ..., 4, 1} on the reference's time
// grid. The objective is wS Phi_S + wT Phi_T.
//
// Discrete adjoint with O = wS kS Pi_S + wT kT Pi_T:
//   lambda_N = c_N O psi_N,  lambda_k = c_k O psi_k + U^H lambda_{k+1},
//   dObj/dp = sum_k 2 Re <lambda_{k+1}| dU/dp |psi_k>  (+ explicit k_X terms)
//   <lambda| dU |psi> = -i int_0^dt <exp(i H^H (dt-tau)) lambda| dH/dp |exp(-i H tau) psi> dtau
// with the integral by Gauss-Legendre nodes. H^H = H_eff(-kS, -kT), so
// exp(i H^H s) lambda is a Krylov step of lambda under that Hamiltonian with a
// negative time step. Every dH/dp is an electron operator times at most one
// nuclear operator, so all of them are read off reduced matrices
// R[a][b] = sum_rest conj(mu_a) nu_b of the electron pair (4 x 4) and of each
// (electron spin, nucleus) pair (2g x 2g), accumulated on the device over the
// nodes and steps.
//
// Schedule: forward sweep with checkpoints every K steps; the backward sweep
// recomputes each segment from its checkpoint, and the Krylov basis built at
// psi_k for psi_{k+1} also gives the node states exp(-i H x_q dt) psi_k, kept
// for the segment. Per step: three Krylov builds (forward, recompute, costate)
// and 2*nq + 2 basis applications. When a segment's node states do not fit in
// device memory they are rebuilt per step instead (four builds per step).
// Without a gradient only the forward sweep runs (one build per step).

#define CON_MAXG 6

// One (tile, slot) of a contraction launch; roff is the accumulator offset
// (in 36-entry blocks) of the tile's lane 0, nsl its job's slot count.
struct ConPair {
  int t, js, jl, nsl;
  int64_t roff;
};

// Partial reduced matrices P[a][b] = sum_{o in chunk} conj(mu_row(a,o))
// nu_row(b,o) for the (tile, slot) pairs [p0, p0 + cnt), all of slot size G:
// CTA b = ((pair * nch) + chunk) * (G / RB) + row block; one warp per CTA,
// lanes = samples; rows a of the block [rb*RB, rb*RB + RB) against all G
// columns (RB x G accumulators keep the register footprint small enough for
// many resident warps). k_contract_close adds the chunks in order.
template <int G, int RB>
__global__ void __launch_bounds__(32, (RB * G > 20 ? 8 : 16))
    k_contract(const TileInfo* __restrict__ tiles, const int* __restrict__ map,
               const int* __restrict__ scol, const GradSlot* __restrict__ slots,
               const ConPair* __restrict__ pairs, int p0, int nch, const double2* __restrict__ mu,
               const double2* __restrict__ nu, double2* __restrict__ partial) {
  constexpr int NRB = G / RB;
  const int b = blockIdx.x;
  const int rb = b % NRB;
  const int pc = b / NRB;
  const int pl = pc / nch, ch = pc % nch;
  const ConPair PR = pairs[p0 + pl];
  const GradSlot S = slots[PR.js];
  const TileInfo& T = tiles[PR.t];
  const int lane = threadIdx.x;
  const int wslot = PR.t * SPC_LANES + lane;
  const bool act = map[wslot] >= 0;
  const int64_t Z = T.n / 4;
  const int64_t L = S.owner == -1 ? Z : (S.owner == -2 ? 4 * Z / S.g : 2 * Z / S.g);
  const int64_t per = (L + nch - 1) / nch;
  const int64_t o0 = (int64_t)ch * per, o1 = min(L, o0 + per);
  double2 acc[RB * G];
#pragma unroll
  for (int i = 0; i < RB * G; ++i) acc[i] = cz();
  if (act) {
    const int64_t ld = T.ldp;
    const double2* Mu = mu + T.psi_off + scol[wslot];
    const double2* Nu = nu + T.psi_off + scol[wslot];
    const int64_t zg = S.owner == -1 ? Z : Z / S.g;
    for (int64_t o = o0; o < o1; ++o) {
      // o = nuclear index (electron pair), else (electron state or spin of
      // the other electron, nuclear index without nucleus j)
      int so = 0;
      int64_t nbase = o;
      if (S.owner != -1) {
        so = (int)(o / zg);
        const int64_t rem = o - (int64_t)so * zg;
        const int64_t hi = rem / S.stride, lo = rem - hi * S.stride;
        nbase = hi * S.g * S.stride + lo;
      }
      auto row_of = [&](int c) -> int64_t {
        if (S.owner == -1) return (int64_t)c * Z + o;
        int e, mm;
        if (S.owner == -2) {
          e = so;
          mm = c;
        } else {
          const int sk = c / (G / 2);
          mm = c % (G / 2);
          e = S.owner == 0 ? (sk * 2 + so) : (so * 2 + sk);
        }
        return (int64_t)e * Z + nbase + (int64_t)mm * S.stride;
      };
      double2 a[RB], v[G];
#pragma unroll
      for (int i = 0; i < RB; ++i) a[i] = Mu[row_of(rb * RB + i) * ld];
#pragma unroll
      for (int c = 0; c < G; ++c) v[c] = Nu[row_of(c) * ld];
#pragma unroll
      for (int i = 0; i < RB; ++i)
#pragma unroll
        for (int j = 0; j < G; ++j) acc[i * G + j] = cjfma(a[i], v[j], acc[i * G + j]);
    }
  }
  // partial[(pair * nch + chunk)][entry][lane]
  double2* P = partial + ((size_t)pc * G * G + (size_t)rb * RB * G) * SPC_LANES + lane;
#pragma unroll
  for (int i = 0; i < RB * G; ++i) P[(size_t)i * SPC_LANES] = acc[i];
}

// R += w * sum over chunks (in chunk order) of the partials, one thread per
// (pair, entry, lane).
template <int G>
__global__ void __launch_bounds__(256)
    k_contract_close(const int* __restrict__ map, const ConPair* __restrict__ pairs, int p0, int cnt,
                     int nch, const double2* __restrict__ partial, double w, double2* __restrict__ racc) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)cnt * G * G * SPC_LANES) return;
  const int lane = (int)(idx % SPC_LANES);
  const int e = (int)((idx / SPC_LANES) % (G * G));
  const int pl = (int)(idx / ((int64_t)SPC_LANES * G * G));
  const ConPair PR = pairs[p0 + pl];
  if (map[PR.t * SPC_LANES + lane] < 0) return;
  double2 s = cz();
  const double2* src = partial + ((size_t)pl * nch * G * G + e) * SPC_LANES + lane;
  for (int c = 0; c < nch; ++c) s = cadd(s, src[(size_t)c * G * G * SPC_LANES]);
  double2* R = racc + ((size_t)PR.roff + (size_t)lane * PR.nsl + PR.jl) * CON_MAXG * CON_MAXG + e;
  *R = make_double2(fma(w, s.x, R->x), fma(w, s.y, R->y));
}

// Krylov coordinates of y = exp(-i tau A) (beta e1): beta * E[:, 0] per slot,
// beta = ||x|| as the norm pass left it in cvec[w][0].
__global__ void k_first_col(int nslots, const TileInfo* __restrict__ tiles, const int* __restrict__ map,
                            int m, const double2* __restrict__ Aexp, const double2* __restrict__ cvec,
                            double2* __restrict__ cout) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nslots || map[w] < 0) return;
  const int me = tiles[w / SPC_LANES].m;
  const double beta = cvec[(size_t)w * m].x;
  const double2* E = Aexp + (size_t)w * m * m;
  for (int j = 0; j < m; ++j) cout[(size_t)w * m + j] = j < me ? cscale(beta, E[j]) : cz();
}

// lam = ulam + c (cI psi + cP Pi_S psi) with (cI, cP) per tile, Pi_S = |S><S|
// on the electron pair, |S> = (|ab> - |ba>)/sqrt(2); grid (tiles, row
// blocks), block (32, SPC_WARPS).
__global__ void __launch_bounds__(256)
    k_costate(const TileInfo* __restrict__ tiles, const int* __restrict__ map,
              const int* __restrict__ scol, const double2* __restrict__ coefs, double c,
              const double2* __restrict__ psi, const double2* __restrict__ ulam,
              double2* __restrict__ lam) {
  const TileInfo& T = tiles[blockIdx.x];
  const int w = blockIdx.x * SPC_LANES + threadIdx.x;
  if (map[w] < 0) return;
  const double cI = c * coefs[blockIdx.x].x, cP = c * coefs[blockIdx.x].y;
  const int64_t Z = T.n / 4;
  const int64_t ld = T.ldp;
  const size_t base = T.psi_off + scol[w];
  for (int64_t r = (int64_t)blockIdx.y * SPC_WARPS + threadIdx.y; r < 4 * Z;
       r += (int64_t)gridDim.y * SPC_WARPS) {
    const int e = (int)(r / Z);
    const int64_t n = r - e * Z;
    double2 v = ulam[base + r * ld];
    const double2 x = psi[base + r * ld];
    v = make_double2(fma(cI, x.x, v.x), fma(cI, x.y, v.y));
    if (e == 1 || e == 2) {
      const double2 ab = psi[base + (Z + n) * ld], ba = psi[base + (2 * Z + n) * ld];
      const double2 d = cscale(e == 1 ? 0.5 * cP : -0.5 * cP, csub(ab, ba));
      v = cadd(v, d);
    }
    lam[base + r * ld] = v;
  }
}

// Gauss-Legendre nodes and weights on [0, 1] (Newton on P_n from the
// Tricomi initial guesses).
static void gauss_legendre01(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      // p1 = P_n(z), p0 = P_{n-1}(z)
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = 0.5 * (1.0 - z);
    w[i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
}

int yield_gradient_run(Handle* h, const double* theta, const std::vector<GradJob>& jobs,
                       const std::vector<GradSlot>& cs, double dt, int nsteps,
                       const std::vector<double>& cw, int m, int nq, int K, bool want_grad,
                       std::vector<std::vector<double2>>& rsum, std::vector<std::vector<double2>>& fsum) {
  auto t_start = std::chrono::steady_clock::now();
  cudaStream_t st = h->stream;
  const auto& HB = h->hb;
  const int nj = (int)jobs.size();
  // job layout: state blocks [rows][ldp] back to back, 32-sample tiles
  std::vector<int> ldp(nj), nrow(nj), tile0(nj);
  std::vector<int64_t> psi_off(nj);
  size_t S = 0;  // entries of one state of all samples of all jobs
  int ntiles = 0, Mtot = 0;
  for (int k = 0; k < nj; ++k) {
    nrow[k] = HB.n[jobs[k].sys];
    ldp[k] = (jobs[k].M + SPC_LANES - 1) / SPC_LANES * SPC_LANES;
    psi_off[k] = (int64_t)S;
    S += (size_t)nrow[k] * ldp[k];
    tile0[k] = ntiles;
    ntiles += ldp[k] / SPC_LANES;
    Mtot += jobs[k].M;
  }
  const int nslots = ntiles * SPC_LANES;
  const size_t mm = (size_t)m * m;
  const size_t con = (size_t)CON_MAXG * CON_MAXG;
  const double elems = [&] {
    double e = 0.0;
    for (int k = 0; k < nj; ++k) e += (double)nrow[k] * jobs[k].M;
    return e;
  }();
  const int items_cap = h->sm_count * 32 + ntiles;

  // tiles, slot maps, costate coefficients
  std::vector<TileInfo> tf(ntiles), tb(ntiles);
  std::vector<int> map(nslots), scol(nslots), tile_n(ntiles), tile_job(ntiles);
  std::vector<double2> coefs(ntiles);
  {
    int t = 0;
    int64_t qo = 0, po = 0;
    for (int k = 0; k < nj; ++k) {
      for (int c = 0; c < ldp[k] / SPC_LANES; ++c, ++t) {
        TileInfo ti{};
        ti.job = k;
        ti.n = nrow[k];
        ti.ldp = ldp[k];
        ti.m = std::min(m, nrow[k]);
        ti.q_off = qo;
        ti.p_off = po;
        ti.psi_off = psi_off[k];
        qo += (int64_t)m * nrow[k] * SPC_LANES;
        po += (int64_t)nrow[k] * SPC_LANES;
        tf[t] = tb[t] = ti;
        for (int e = 0; e < 2; ++e) {
          TileInfo& x = e == 0 ? tf[t] : tb[t];
          const int sy = jobs[k].sys + e;
          x.rowptr = (const int*)HB.rowptr.p + HB.rp_off[sy];
          x.split = (const int*)HB.split.p + HB.rp_off[sy];
          x.col = (const int*)HB.col.p + HB.nz_off[sy];
          x.val = (const double2*)HB.val.p + HB.nz_off[sy];
          x.vsum = (const double*)HB.vsum.p + HB.nz_off[sy];
          x.kappa = HB.herm[sy] ? &((const HMeta*)HB.meta.p)[sy].kappa : nullptr;
        }
        for (int l = 0; l < SPC_LANES; ++l) {
          const int s = c * SPC_LANES + l;
          map[t * SPC_LANES + l] = s < jobs[k].M ? tile0[k] * SPC_LANES + s : -1;
          scol[t * SPC_LANES + l] = s < jobs[k].M ? s : -1;
        }
        tile_n[t] = nrow[k];
        tile_job[t] = k;
        coefs[t] = make_double2(jobs[k].cI, jobs[k].cP);
      }
    }
  }
  // contraction pair tables: gradient pairs grouped by slot size, and the
  // electron-pair slot of every tile for the forward sum F
  std::vector<int64_t> roff(ntiles);
  int64_t rtot = 0;
  for (int t = 0; t < ntiles; ++t) {
    roff[t] = rtot;
    rtot += (int64_t)SPC_LANES * jobs[tile_job[t]].nslot;
  }
  std::vector<ConPair> pairs;
  std::vector<int> grp_G, grp_p0, grp_cnt;
  for (int Gv = 2; Gv <= CON_MAXG; ++Gv) {
    const int p0 = (int)pairs.size();
    for (int t = 0; t < ntiles; ++t) {
      const GradJob& J = jobs[tile_job[t]];
      for (int jl = 0; jl < J.nslot; ++jl)
        if (cs[J.slot0 + jl].G == Gv) pairs.push_back(ConPair{t, J.slot0 + jl, jl, J.nslot, roff[t]});
    }
    if ((int)pairs.size() > p0) {
      grp_G.push_back(Gv);
      grp_p0.push_back(p0);
      grp_cnt.push_back((int)pairs.size() - p0);
    }
  }
  const int pf0 = (int)pairs.size();
  for (int t = 0; t < ntiles; ++t)
    pairs.push_back(ConPair{t, jobs[tile_job[t]].slot0, 0, 1, (int64_t)t * SPC_LANES});
  const int npairs = (int)pairs.size();
  // chunks per pair: about two waves of one-warp CTAs over the group (row
  // blocks included), at least 32 rows of `o` each
  auto pair_len = [&](const ConPair& P) {
    const GradSlot& Sl = cs[P.js];
    const int64_t Z = tile_n[P.t] / 4;
    return Sl.owner == -1 ? Z : (Sl.owner == -2 ? 4 * Z / Sl.g : 2 * Z / Sl.g);
  };
  auto nrb_of = [](int G) { return G == 6 ? 2 : 1; };
  auto chunks_for = [&](int p0, int cnt, int G) {
    int64_t L = 1;
    for (int q = p0; q < p0 + cnt; ++q) L = std::max(L, pair_len(pairs[q]));
    const int64_t by_wave = (int64_t)h->sm_count * 64 / std::max(1, cnt * nrb_of(G));
    const int64_t by_len = (L + 31) / 32;
    return (int)std::max<int64_t>(1, std::min(by_wave, by_len));
  };
  const int nch_f = chunks_for(pf0, ntiles, 4);
  std::vector<int> grp_nch(grp_G.size());
  size_t part_need = (size_t)ntiles * nch_f * 16 * SPC_LANES;
  for (size_t gi = 0; gi < grp_G.size(); ++gi) {
    grp_nch[gi] = chunks_for(grp_p0[gi], grp_cnt[gi], grp_G[gi]);
    part_need = std::max(part_need, (size_t)grp_cnt[gi] * grp_nch[gi] * grp_G[gi] * grp_G[gi] * SPC_LANES);
  }
  const size_t part_cap = part_need;

  // checkpoint spacing K and whether a segment's node states are kept (one
  // Krylov build per step saved). K = 0 picks the largest spacing whose
  // states fit in device memory (fewest recomputed segments), else the
  // spacing of least memory with node states rebuilt per step.
  bool cache = false;
  if (want_grad) {
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const double avail = 0.85 * (double)free_b - (double)(1 << 28);
    const double sb = sizeof(double2) * (double)S;
    // bytes of every state buffer of the sweep, and the device memory they
    // take beyond what the handle already holds: a held buffer is reused up
    // to the size asked of it (buffers only grow), so its excess over that
    // size is no help
    auto need = [&](int k, bool keep) {
      return sb * ((double)m + 4.5 + (nsteps / k + 1) + k + 1.0 + (keep ? (double)k * nq : (double)nq));
    };
    auto extra = [&](int k, bool keep) {
      double x = 0.0;
      auto add = [&](const Handle::Buf& b, double bytes) { x += std::max(0.0, bytes - (double)b.bytes); };
      add(h->Q, sb * m);
      add(h->gmu, sb);
      add(h->glam, 2.0 * sb);
      add(h->P, sb);
      add(h->xsum, 0.5 * sb);  // the Re + Im plane of the current Krylov vector beside P
      add(h->gck, sb * (nsteps / k + 1));
      add(h->gseg, sb * (k + 1));
      add(h->gnu, sb * (keep ? (double)k * nq : (double)nq));
      return x;
    };
    if (K == 0) {
      // among the spacings whose states fit, the one that recomputes the
      // fewest steps (all but the last segment are recomputed), the larger
      // on a tie
      int64_t best = -1;
      for (int k = nsteps; k >= 1; --k) {
        if (extra(k, true) > avail) continue;
        const int64_t recomputed = (int64_t)((nsteps - 1) / k) * k;
        if (best < 0 || recomputed < best) {
          best = recomputed;
          K = k;
        }
      }
      if (K)
        cache = true;
      else
        K = std::max(1, (int)std::lround(std::sqrt((double)nsteps)));
    } else {
      cache = extra(K, true) <= avail;
    }
    if (!cache && extra(K, false) > avail)
      return set_error(SPC_ERR_ALLOC,
                       "yield gradient needs %.1f GB of device memory at checkpoint spacing %d (%.1f GB free)",
                       need(K, false) / 1e9, K, free_b / 1e9);
  }
  if (K < 1) K = 1;
  const int nck = nsteps / K + 1;
  const int a_last = ((nsteps - 1) / K) * K;  // first step of the last segment
  const size_t n_ck = want_grad ? nck : 0, n_seg = want_grad ? K + 1 : 0;
  const size_t n_nu = want_grad ? (cache ? (size_t)K * nq : (size_t)nq) : 0;
  const size_t plan_bytes = 2 * sizeof(TileInfo) * ntiles + sizeof(int2) * 2 * items_cap +
                            sizeof(int) * 2 * nslots + sizeof(double2) * ntiles + 64;
  if (h->ensure(h->gck, sizeof(double2) * S * n_ck) || h->ensure(h->gseg, sizeof(double2) * S * n_seg) ||
      h->ensure(h->gnu, sizeof(double2) * S * n_nu) || h->ensure(h->gmu, sizeof(double2) * S) ||
      h->ensure(h->glam, sizeof(double2) * S * 2) || h->ensure(h->Q, sizeof(double2) * m * S) ||
      h->ensure(h->P, sizeof(double2) * S) || h->ensure(h->xsum, sizeof(double) * S) ||
      h->ensure(h->partial, sizeof(double2) * std::max<size_t>((size_t)items_cap * SPC_LANES, part_cap)) ||
      h->ensure(h->counters, sizeof(unsigned) * std::max<size_t>(ntiles, npairs)) ||
      h->ensure(h->coef, sizeof(double2) * nslots) || h->ensure(h->rbeta, sizeof(double) * nslots) ||
      h->ensure(h->Ahess, sizeof(double2) * mm * nslots) || h->ensure(h->Aexp, sizeof(double2) * mm * nslots) ||
      h->ensure(h->cvec, sizeof(double2) * m * nslots) || h->ensure(h->cvec2, sizeof(double2) * m * nslots) ||
      h->ensure(h->flag, sizeof(int) * nslots) || h->ensure(h->err, 16) ||
      h->ensure(h->gslots, sizeof(GradSlot) * cs.size() + sizeof(ConPair) * npairs) ||
      h->ensure(h->gracc, sizeof(double2) * std::max<int64_t>(rtot, 1) * con) ||
      h->ensure(h->gfacc, sizeof(double2) * nslots * con) || h->ensure(h->plan, plan_bytes) ||
      h->ensure(h->jobtab, sizeof(JobInit) * nj))
    return SPC_ERR_ALLOC;
  double2 *ck = (double2*)h->gck.p, *seg = (double2*)h->gseg.p, *gnu = (double2*)h->gnu.p;
  double2 *gmu = (double2*)h->gmu.p, *lam = (double2*)h->glam.p, *ulam = lam + S;
  double2 *d_Q = (double2*)h->Q.p, *d_P = (double2*)h->P.p, *d_part = (double2*)h->partial.p;
  double* d_xs = (double*)h->xsum.p;
  unsigned* d_cnt = (unsigned*)h->counters.p;
  double2 *d_A = (double2*)h->Ahess.p, *d_E = (double2*)h->Aexp.p, *d_c = (double2*)h->cvec.p;
  double2* d_c2 = (double2*)h->cvec2.p;
  int* d_flag = (int*)h->flag.p;
  int* d_err = (int*)h->err.p;
  GradSlot* d_slots = (GradSlot*)h->gslots.p;
  ConPair* d_pairs = (ConPair*)((char*)h->gslots.p + sizeof(GradSlot) * cs.size());
  double2 *d_racc = (double2*)h->gracc.p, *d_facc = (double2*)h->gfacc.p;
  char* plan = (char*)h->plan.p;
  TileInfo* d_tf = (TileInfo*)plan;
  TileInfo* d_tb = d_tf + ntiles;
  int2* d_items = (int2*)(plan + 2 * sizeof(TileInfo) * ntiles);
  int2* d_items_s = d_items + items_cap;
  int* d_map = (int*)(d_items_s + items_cap);
  int* d_scol = d_map + nslots;
  double2* d_coefs = (double2*)(((uintptr_t)(d_scol + nslots) + 15) & ~(uintptr_t)15);
  int64_t launches0 = h->launches;

  auto resident = [&](const void* fn) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, 256, 0) != cudaSuccess) b = 1;
    return std::max(1, b) * h->sm_count;
  };
  std::vector<int> fp, cp, fs, csn;
  std::vector<int2> items_p, items_s;
  plan_items(tile_n, std::min(resident((const void*)k_rowpass<PASS_AXPY_DOT>),
                              resident((const void*)k_rowpass<PASS_AXPY_NORM>)), fp, cp, items_p);
  plan_items(tile_n, resident((const void*)k_spmm), fs, csn, items_s);
  const int nip = (int)items_p.size(), nis = (int)items_s.size();
  if (nip > items_cap || nis > items_cap) return set_error(SPC_ERR_ARG, "internal: work plan exceeds its buffer");
  // SpMM work per sample column: all entries (bytes); FP64 operations issued
  // 6 per complex entry, 4 per real one, 3 per row closing the three-product
  // sums (forward and adjoint Hamiltonians of a job share the pattern), plus
  // 4 per row for the -i*kappa shift outside Lanczos
  int64_t nnz_tiles = 0;
  double spmm_flops = 0.0, herm_rows = 0.0;
  for (int t = 0; t < ntiles; ++t) {
    tf[t].ip0 = tb[t].ip0 = fp[t];
    tf[t].nip = tb[t].nip = cp[t];
    tf[t].is0 = tb[t].is0 = fs[t];
    tf[t].nis = tb[t].nis = csn[t];
    const int sy = jobs[tile_job[t]].sys;
    nnz_tiles += HB.nnz[sy];
    spmm_flops += 6.0 * (double)HB.nnz_cplx[sy] + 4.0 * (double)(HB.nnz[sy] - HB.nnz_cplx[sy]) + 3.0 * tile_n[t];
    if (HB.herm[sy]) herm_rows += tile_n[t];
  }
  CK(cudaMemcpyAsync(d_tf, tf.data(), sizeof(TileInfo) * ntiles, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d_tb, tb.data(), sizeof(TileInfo) * ntiles, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d_items, items_p.data(), sizeof(int2) * nip, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d_items_s, items_s.data(), sizeof(int2) * nis, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d_map, map.data(), sizeof(int) * nslots, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d_scol, scol.data(), sizeof(int) * nslots, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d_coefs, coefs.data(), sizeof(double2) * ntiles, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d_slots, cs.data(), sizeof(GradSlot) * cs.size(), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d_pairs, pairs.data(), sizeof(ConPair) * npairs, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned) * std::max<size_t>(ntiles, npairs), st));
  CK(cudaMemsetAsync(d_racc, 0, sizeof(double2) * std::max<int64_t>(rtot, 1) * con, st));
  CK(cudaMemsetAsync(d_facc, 0, sizeof(double2) * nslots * con, st));
  CK(cudaMemsetAsync(d_flag, 0, sizeof(int) * nslots, st));
  CK(cudaMemsetAsync(h->err.p, 0, 16, st));
  // psi_0 = theta (x) z: into the last segment's buffer when it is the only one
  double2* psi0 = !want_grad ? lam : a_last == 0 ? seg : ck;
  CK(cudaMemsetAsync(psi0, 0, sizeof(double2) * S, st));
  {
    std::vector<JobInit> ji(nj);
    for (int k = 0; k < nj; ++k) ji[k] = JobInit{nrow[k] / 4, psi_off[k], jobs[k].M, ldp[k], jobs[k].zk};
    CK(cudaMemcpyAsync(h->jobtab.p, ji.data(), sizeof(JobInit) * nj, cudaMemcpyHostToDevice, st));
    Theta th;
    for (int e = 0; e < 4; ++e) th.v[e] = make_double2(theta[2 * e], theta[2 * e + 1]);
    for (int j0 = 0; j0 < nj; j0 += 65535) {
      const int cnt = std::min(65535, nj - j0);
      k_kron_init<<<dim3(std::max(1, h->sm_count * 8 / cnt), cnt), 256, 0, st>>>((const JobInit*)h->jobtab.p,
                                                                                 j0, th, psi0);
      h->count_launch();
    }
  }
  CK(set_expm_smem(m));
  const dim3 blk(SPC_LANES, SPC_WARPS);
  // the three-term recurrence only on explicit request: no projector Gram
  // verifies these bases (the trace-sampling path checks its own)
  bool lanczos = h->krylov_method == 1;
  for (const GradJob& J : jobs) lanczos = lanczos && HB.herm[J.sys] && HB.herm[J.sys + 1];
  std::vector<double> xq, wq;
  gauss_legendre01(nq, xq, wq);
  int64_t builds = 0;

  // Krylov basis of the states `x` (psi layout) under the tiles' Hamiltonians
  auto build = [&](const double2* x, const TileInfo* tiles) {
    CK(cudaMemsetAsync(d_A, 0, sizeof(double2) * mm * nslots, st));
    PassArgs pa{};
    pa.tiles = tiles;
    pa.items = d_items;
    pa.m = m;
    pa.Q = d_Q;
    pa.P = d_P;
    pa.psi = x;
    pa.map = d_map;
    pa.scol = d_scol;
    pa.coef = (double2*)h->coef.p;
    pa.rbeta = (double*)h->rbeta.p;
    pa.Ahess = d_A;
    pa.cvec = d_c;
    pa.partial = d_part;
    pa.counters = d_cnt;
    pa.lanczos = lanczos ? 1 : 0;
    int pe = h->prof.begin(st);
    k_rowpass<PASS_NORM_GATHER><<<nip, blk, 0, st>>>(pa);
    h->prof.end(st, pe, PK_DOT, 4.0 * elems, 16.0 * elems);
    pe = h->prof.begin(st);
    k_scale<<<nip, blk, 0, st>>>(tiles, d_items, d_map, d_scol, x, d_P, 1, 0, pa.rbeta, d_Q, d_xs);
    h->prof.end(st, pe, PK_SCALE, 2.0 * elems, 40.0 * elems);
    h->count_launch(2);
    for (int i = 0; i < m; ++i) {
      pe = h->prof.begin(st);
      k_spmm<<<nis, blk, 0, st>>>(tiles, d_items_s, d_map, i, d_Q, d_xs, d_P, lanczos ? 0 : 1);
      h->prof.end(st, pe, PK_SPMM, (spmm_flops + (lanczos ? 0.0 : 4.0 * herm_rows)) * SPC_LANES,
                  28.0 * (double)nnz_tiles + 40.0 * elems);
      h->count_launch();
      pa.col_i = i;
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
        k_scale<<<nip, blk, 0, st>>>(tiles, d_items, d_map, d_scol, x, d_P, 0, i + 1, pa.rbeta, d_Q, d_xs);
        h->prof.end(st, pe, PK_SCALE, 2.0 * elems, 40.0 * elems);
        h->count_launch(2);
      }
    }
    builds += Mtot;
    return SPC_OK;
  };
  // y = exp(-i tau H) x from the current bases (tau < 0 runs backwards)
  auto apply = [&](double tau, const TileInfo* tiles, double2* y) {
    int pe = h->prof.begin(st);
    launch_expm(m, nslots, tiles, d_map, d_A, d_E, tau, d_err, st);
    h->prof.end(st, pe, PK_EXPM, 8.0 * (double)mm * m * 9.0 * Mtot, 32.0 * (double)mm * Mtot);
    pe = h->prof.begin(st);
    k_first_col<<<(nslots + 127) / 128, 128, 0, st>>>(nslots, tiles, d_map, m, d_E, d_c, d_c2);
    h->prof.end(st, pe, PK_SETUP, 2.0 * m * Mtot, 32.0 * m * Mtot);
    pe = h->prof.begin(st);
    k_psi_update<<<nip, blk, 0, st>>>(tiles, d_items, m, d_map, d_scol, d_flag, d_Q, d_c2, y);
    h->prof.end(st, pe, PK_PSI, 8.0 * m * elems, 16.0 * (m + 1) * elems);
    h->count_launch(3);
  };
  // algorithmic FLOPs of a contraction over the gradient slots / the pair slot
  double con_fg = 0.0, con_ff = 0.0;
  for (const ConPair& P : pairs) {
    const GradSlot& Sl = cs[P.js];
    const double Z = tile_n[P.t] / 4;
    const double L = Sl.owner == -1 ? Z : (Sl.owner == -2 ? 4.0 * Z / Sl.g : 2.0 * Z / Sl.g);
    const double f = 8.0 * Sl.G * Sl.G * L * SPC_LANES;
    if (&P - pairs.data() < pf0)
      con_fg += f;
    else
      con_ff += f;
  }
  // acc += w * reduced matrices of (mu, nu): forward = the electron pair only
  auto launch_group = [&](int G, int p0, int cnt, int nc, const double2* mu, const double2* nu, double w,
                          double2* acc) {
    const int nb = cnt * nc * nrb_of(G);
    switch (G) {
      case 2:
        k_contract<2, 2><<<nb, 32, 0, st>>>(d_tf, d_map, d_scol, d_slots, d_pairs, p0, nc, mu, nu, d_part);
        break;
      case 3:
        k_contract<3, 3><<<nb, 32, 0, st>>>(d_tf, d_map, d_scol, d_slots, d_pairs, p0, nc, mu, nu, d_part);
        break;
      case 4:
        k_contract<4, 4><<<nb, 32, 0, st>>>(d_tf, d_map, d_scol, d_slots, d_pairs, p0, nc, mu, nu, d_part);
        break;
      case 5:
        k_contract<5, 5><<<nb, 32, 0, st>>>(d_tf, d_map, d_scol, d_slots, d_pairs, p0, nc, mu, nu, d_part);
        break;
      default:
        k_contract<6, 3><<<nb, 32, 0, st>>>(d_tf, d_map, d_scol, d_slots, d_pairs, p0, nc, mu, nu, d_part);
        break;
    }
    const int64_t nt = (int64_t)cnt * G * G * SPC_LANES;
    const int gb = (int)((nt + 255) / 256);
    switch (G) {
      case 2: k_contract_close<2><<<gb, 256, 0, st>>>(d_map, d_pairs, p0, cnt, nc, d_part, w, acc); break;
      case 3: k_contract_close<3><<<gb, 256, 0, st>>>(d_map, d_pairs, p0, cnt, nc, d_part, w, acc); break;
      case 4: k_contract_close<4><<<gb, 256, 0, st>>>(d_map, d_pairs, p0, cnt, nc, d_part, w, acc); break;
      case 5: k_contract_close<5><<<gb, 256, 0, st>>>(d_map, d_pairs, p0, cnt, nc, d_part, w, acc); break;
      default: k_contract_close<6><<<gb, 256, 0, st>>>(d_map, d_pairs, p0, cnt, nc, d_part, w, acc); break;
    }
    h->count_launch(2);
  };
  auto contract = [&](const double2* mu, const double2* nu, double w, bool forward, double2* acc) {
    int pe = h->prof.begin(st);
    if (forward) {
      launch_group(4, pf0, ntiles, nch_f, mu, nu, w, acc);
    } else {
      for (size_t gi = 0; gi < grp_G.size(); ++gi)
        launch_group(grp_G[gi], grp_p0[gi], grp_cnt[gi], grp_nch[gi], mu, nu, w, acc);
    }
    h->prof.end(st, pe, PK_CONTRACT, forward ? con_ff : con_fg, 32.0 * elems);
  };
  // basis at psi_k under H: node states nu_q and psi_{k+1}
  auto step_forward = [&](const double2* x, double2* nodes, double2* y) {
    int rc = build(x, d_tf);
    if (rc) return rc;
    if (nodes)
      for (int q = 0; q < nq; ++q) apply(dt * xq[q], d_tf, nodes + S * q);
    apply(dt, d_tf, y);
    return SPC_OK;
  };
  const dim3 lgrid(ntiles, std::max(1, h->sm_count * 4 / ntiles));
  auto costate = [&](double c, const double2* psi, const double2* u) {
    int pe = h->prof.begin(st);
    k_costate<<<lgrid, blk, 0, st>>>(d_tf, d_map, d_scol, d_coefs, c, psi, u, lam);
    h->prof.end(st, pe, PK_COSTATE, 6.0 * elems, 48.0 * elems);
    h->count_launch();
  };

  // forward sweep: checkpoints, the last segment's states and node states,
  // and F = sum_k c_k (electron-pair reduced matrix of psi_k)
  double2* cur = psi0;
  for (int k = 0; k < nsteps; ++k) {
    if (cw[k] != 0.0) contract(cur, cur, cw[k], true, d_facc);
    double2* nxt;
    if (want_grad && k + 1 >= a_last)
      nxt = seg + S * (k + 1 - a_last);
    else if (want_grad && (k + 1) % K == 0)
      nxt = ck + S * ((k + 1) / K);
    else
      nxt = cur == gmu ? ulam : gmu;
    int rc = step_forward(cur, want_grad && cache && k >= a_last ? gnu + S * nq * (k - a_last) : nullptr, nxt);
    if (rc) return rc;
    cur = nxt;
  }
  if (cw[nsteps] != 0.0) contract(cur, cur, cw[nsteps], true, d_facc);
  // backward sweep
  if (want_grad) {
    CK(cudaMemsetAsync(lam, 0, sizeof(double2) * S, st));
    costate(cw[nsteps], cur, lam);
  }
  for (int a = want_grad ? a_last : -1; a >= 0; a -= K) {
    const int b = std::min(nsteps, a + K);
    if (a != a_last) {
      CK(cudaMemcpyAsync(seg, ck + S * (a / K), sizeof(double2) * S, cudaMemcpyDeviceToDevice, st));
      for (int k = a; k < b; ++k) {
        int rc = step_forward(seg + S * (k - a), cache ? gnu + S * nq * (k - a) : nullptr, seg + S * (k - a + 1));
        if (rc) return rc;
      }
    }
    for (int k = b - 1; k >= a; --k) {
      double2* nodes = gnu + S * nq * (cache ? k - a : 0);
      if (!cache) {
        int rc = build(seg + S * (k - a), d_tf);
        if (rc) return rc;
        for (int q = 0; q < nq; ++q) apply(dt * xq[q], d_tf, nodes + S * q);
      }
      int rc = build(lam, d_tb);
      if (rc) return rc;
      for (int q = 0; q < nq; ++q) {
        apply(-dt * (1.0 - xq[q]), d_tb, gmu);
        contract(gmu, nodes + S * q, wq[q] * dt, false, d_racc);
      }
      apply(-dt, d_tb, ulam);
      costate(cw[k], seg + S * (k - a), ulam);
    }
  }
  CK(cudaGetLastError());
  std::vector<double2> racc_h((size_t)std::max<int64_t>(rtot, 1) * con), facc_h((size_t)nslots * con);
  CK(cudaMemcpyAsync(racc_h.data(), d_racc, sizeof(double2) * racc_h.size(), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(facc_h.data(), d_facc, sizeof(double2) * facc_h.size(), cudaMemcpyDeviceToHost, st));
  int err_h[4] = {0, 0, 0, 0};
  CK(cudaMemcpyAsync(err_h, h->err.p, 16, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  h->prof.collect();
  // per-job sample sums in sample order
  rsum.assign(nj, {});
  fsum.assign(nj, {});
  for (int k = 0; k < nj; ++k) {
    const int ns = jobs[k].nslot;
    rsum[k].assign((size_t)ns * con, double2{0.0, 0.0});
    fsum[k].assign(con, double2{0.0, 0.0});
    for (int s = 0; s < jobs[k].M; ++s) {
      const int t = tile0[k] + s / SPC_LANES, l = s % SPC_LANES;
      const double2* R = &racc_h[((size_t)roff[t] + (size_t)l * ns) * con];
      for (size_t i = 0; i < (size_t)ns * con; ++i) {
        rsum[k][i].x += R[i].x;
        rsum[k][i].y += R[i].y;
      }
      const double2* F = &facc_h[((size_t)t * SPC_LANES + l) * con];
      for (size_t i = 0; i < con; ++i) {
        fsum[k][i].x += F[i].x;
        fsum[k][i].y += F[i].y;
      }
    }
  }
  h->stats.krylov_builds = builds;
  h->stats.lanczos_fallbacks = 0;
  h->stats.rounds = cache ? 1 : 0;  // 1: node states kept per segment
  h->stats.sample_steps = (int64_t)nsteps * Mtot;
  h->stats.kernel_launches = h->launches - launches0;
  h->stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  if (err_h[0] == 2) return set_error(SPC_ERR_NUMERIC, "singular Pade denominator in expm");
  return SPC_OK;
}
