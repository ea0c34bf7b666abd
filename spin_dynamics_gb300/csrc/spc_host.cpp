// Host-side parts of libspinchem_gpu: error state, handle buffers, the spin
// system description handed to the device builders, the reference's sample
// generator (xoroshiro128+ / Marsaglia polar / sample_SUZ), init_el_state and
// get_kinetics.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "spc_internal.h"

namespace spc {

static thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}
const char* last_error() { return g_last_error.c_str(); }
void clear_error() { g_last_error.clear(); }

int Handle::ensure(Buf& b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (b.bytes >= bytes) return SPC_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  if (cudaMalloc(&b.p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return set_error(SPC_ERR_ALLOC, "cudaMalloc of %zu bytes failed", bytes);
  }
  b.bytes = bytes;
  return SPC_OK;
}
int Handle::ensure_rowptr(size_t count) {
  if (cap_rowptr >= count) return SPC_OK;
  if (d_rowptr) cudaFree(d_rowptr);
  d_rowptr = nullptr;
  cap_rowptr = 0;
  if (cudaMalloc(&d_rowptr, sizeof(int) * count) != cudaSuccess)
    return set_error(SPC_ERR_ALLOC, "cudaMalloc of the row pointer failed");
  cap_rowptr = count;
  return SPC_OK;
}
int Handle::ensure_h_entries(size_t count) {
  if (count == 0) count = 1;
  if (cap_h >= count) return SPC_OK;
  if (d_col) cudaFree(d_col);
  if (d_val) cudaFree(d_val);
  d_col = nullptr;
  d_val = nullptr;
  cap_h = 0;
  if (cudaMalloc(&d_col, sizeof(int) * count) != cudaSuccess ||
      cudaMalloc(&d_val, sizeof(double2) * count) != cudaSuccess)
    return set_error(SPC_ERR_ALLOC, "cudaMalloc of %zu Hamiltonian entries failed", count);
  cap_h = count;
  return SPC_OK;
}
Handle::~Handle() {
  Buf* all[] = {&psi, &Q,  &P,    &partial, &counters, &coef, &rbeta, &Ahess, &Aexp, &proj, &projpart,
                &cvec, &tt, &kk, &done, &map, &obs, &out, &zk, &err, &nbuild, &flag, &xcol, &xval, &xsplit, &plan, &jobtab,
                &hmeta, &xvs, &xsum, &hb.rowptr, &hb.split, &hb.col, &hb.val, &hb.vsum, &hb.meta, &gck, &gseg, &gnu, &gmu, &glam, &cvec2,
                &gslots, &gracc, &gfacc, &bcnt, &bnuc, &btot, &btab, &tune_out, &tune_zk};
  for (Buf* b : all)
    if (b->p) cudaFree(b->p);
  if (d_rowptr) cudaFree(d_rowptr);
  if (d_col) cudaFree(d_col);
  if (d_val) cudaFree(d_val);
  if (own_stream) cudaStreamDestroy(own_stream);
}

// ---------------------------------------------------------------------------
// uncontracted complex arithmetic (the reference's rounding points)
struct cd {
  double re, im;
};
static inline cd cadd(cd a, cd b) { return {a.re + b.re, a.im + b.im}; }
static inline cd csub(cd a, cd b) { return {a.re - b.re, a.im - b.im}; }
static inline cd cmulx(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
static inline cd rsc(double s, cd a) { return {s * a.re, s * a.im}; }

static const double GAMMA_E = 176.08596;
static const double GAMMA_1H = 0.26752218708;
static const double GAMMA_14N = 0.0193297792;

// <a|S_r|b> of a spin-1/2, states 0 = alpha, 1 = beta
static cd spin_half_el(int r, int a, int b) {
  if (r == 2) return a == b ? cd{a == 0 ? 0.5 : -0.5, 0.0} : cd{0.0, 0.0};
  if (a == b) return {0.0, 0.0};
  if (r == 0) return {0.5, 0.0};
  return a == 0 ? cd{0.0, -0.5} : cd{0.0, 0.5};
}
static cd pair_el(int k, int r, int e, int ep) {
  int s1 = e >> 1, s2 = e & 1, t1 = ep >> 1, t2 = ep & 1;
  if (k == 0) return s2 == t2 ? spin_half_el(r, s1, t1) : cd{0.0, 0.0};
  return s1 == t1 ? spin_half_el(r, s2, t2) : cd{0.0, 0.0};
}

// <a|I_c|b> for multiplicity g, states m = I, I-1, ...; ladder elements
// sqrt(I(I+1) - m_a m_b) as get_spinop_sp forms them (src/spinop.f90:88-92)
static cd nuc_el(int g, int c, int a, int b) {
  const double I = (g - 1) / 2.0;
  const double ma = I - a, mb = I - b;
  if (c == 2) return a == b ? cd{ma, 0.0} : cd{0.0, 0.0};
  if (!(a == b - 1 || a == b + 1)) return cd{0.0, 0.0};
  const double l = std::sqrt(I * (I + 1.0) - ma * mb);
  if (c == 0) return cd{0.5 * l, 0.0};
  return a == b - 1 ? cd{0.0, -0.5 * l} : cd{0.0, 0.5 * l};
}

// Entry tables of the general builder (see HostSystem::gen_tab): per
// nucleus, the matrix elements of its hyperfine and Zeeman terms between
// (e, m_j) and (ep, m_j + d - 1), in the operation order of
// getH_dense's S.A.I sum (src/hamiltonian.f90:279-311).
static void general_tables(HostSystem& hs) {
  hs.gen_tab.clear();
  for (NucInfo& q : hs.nuc) {
    q.tab_off = (int64_t)hs.gen_tab.size();
    const int g = q.g, k = q.owner;
    hs.gen_tab.resize(hs.gen_tab.size() + (size_t)48 * g, make_double2(0.0, 0.0));
    for (int e = 0; e < 4; ++e)
      for (int ep = 0; ep < 4; ++ep) {
        const bool couples = k == 0 ? ((e & 1) == (ep & 1)) : ((e >> 1) == (ep >> 1));
        if (!couples) continue;
        for (int mj = 0; mj < g; ++mj)
          for (int d = 0; d < 3; ++d) {
            const int mp = mj + d - 1;
            if (mp < 0 || mp >= g) continue;
            cd ie[3];
            for (int c = 0; c < 3; ++c) ie[c] = nuc_el(g, c, mj, mp);
            cd v{0.0, 0.0};
            for (int r = 0; r < 3; ++r) {
              const cd se = pair_el(k, r, e, ep);
              for (int c = 0; c < 3; ++c) v = cadd(v, rsc(q.A[r * 3 + c], cmulx(se, ie[c])));
            }
            if (ep == e)
              for (int c = 0; c < 3; ++c) v = cadd(v, rsc(q.zeta[c], ie[c]));
            hs.gen_tab[q.tab_off + ((size_t)(e * 4 + ep) * g + mj) * 3 + d] = make_double2(v.re, v.im);
          }
      }
  }
}

int make_host_system(const spc_system* sys, int mode, HostSystem& hs) {
  if (!sys) return set_error(SPC_ERR_ARG, "null system");
  if (mode != SPC_H_REFERENCE && mode != SPC_H_GENERAL)
    return set_error(SPC_ERR_ARG, "unknown Hamiltonian mode %d", mode);
  const int n1 = sys->n_nuc1, n2 = sys->n_nuc2;
  if (n1 < 0 || n2 < 0 || (n1 > 0 && (!sys->mult1 || !sys->A1)) ||
      (n2 > 0 && (!sys->mult2 || !sys->A2)))
    return set_error(SPC_ERR_ARG, "inconsistent nuclear arrays");
  hs.nuc.clear();
  int64_t Z = 1;
  for (int e = 0; e < 2; ++e) {
    const int n = e == 0 ? n1 : n2;
    for (int i = 0; i < n; ++i) {
      const int g = e == 0 ? sys->mult1[i] : sys->mult2[i];
      if (g < 1 || g > 64) return set_error(SPC_ERR_ARG, "nuclear multiplicity %d out of range", g);
      const double* A = (e == 0 ? sys->A1 : sys->A2) + 9 * i;  // column-major
      const double* gam = e == 0 ? sys->gamma1 : sys->gamma2;
      double gm;
      if (gam) {
        gm = gam[i];
      } else if (g == 3) {
        gm = GAMMA_14N;
      } else if (g == 2) {
        gm = GAMMA_1H;
      } else {
        // getHiso_sp's nuclear-Zeeman switch stops here (src/hamiltonian.f90:136-137)
        return set_error(SPC_ERR_UNSUPPORTED, "Error: sys%%e%d%%g_I(i) must be 3 or 2", e + 1);
      }
      NucInfo q{};
      q.g = g;
      q.owner = e;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) q.A[r * 3 + c] = A[c * 3 + r];
      // e%a_iso(i) = trace(e%A(i,:,:))/3 (src/spinsys.f90:232)
      q.a_iso = ((A[0] + A[4]) + A[8]) / 3.0;
      q.a_half = 0.5 * q.a_iso;
      // zeeman_factor = -w * gamma / gamma_e with w = -B (src/hamiltonian.f90:132-138)
      const double w = -sys->B[2];
      q.zf = -(w * gm / GAMMA_E);
      for (int c = 0; c < 3; ++c) q.zeta[c] = (gm / GAMMA_E) * sys->B[c];
      q.gratio = gm / GAMMA_E;
      hs.nuc.push_back(q);
      Z *= g;
      if (Z > (int64_t)1 << 29) return set_error(SPC_ERR_ARG, "nuclear space too large");
    }
  }
  hs.Z = Z;
  hs.N = 4 * Z;
  int64_t st = 1;
  for (int j = (int)hs.nuc.size() - 1; j >= 0; --j) {
    hs.nuc[j].stride = st;
    st *= hs.nuc[j].g;
  }
  const double kS = sys->kS, kT = sys->kT, J = sys->J;
  const double* D = sys->D;  // column-major
  const double k_bar = (kS + 3.0 * kT) / 4.0, dk = (kS - kT) / 4.0;
  // With kS == kT the Haberkorn term is the scalar -i*kbar/2 and H_eff is a
  // Hermitian matrix shifted by it (the reference builder additionally needs
  // D11 == D22 exactly for its two flip-flop entries to be equal).
  hs.herm_shift = (kS == kT) && (mode == SPC_H_GENERAL || D[0] == D[4]);
  if (mode == SPC_H_REFERENCE) {
    if (sys->B[0] != 0.0 || sys->B[1] != 0.0)
      return set_error(SPC_ERR_ARG, "the reference Hamiltonian takes a field along z only");
    for (const NucInfo& q : hs.nuc)
      if (q.A[0] != q.A[4])  // is_isotropic (src/spinsys.f90:251), stop at src/qm_dynamics.f90:300
        return set_error(SPC_ERR_UNSUPPORTED, "Anisotropic Hamiltoninans have not been implemented yet");
    const double D11 = D[0], D22 = D[4], D33 = D[8];
    if (std::fabs(D11 - D22) > 1.0e-12)
      return set_error(SPC_ERR_UNSUPPORTED,
                       "Error: sys%%D(1,1) must equal sys%%D(2,2) for isotropic conditions");
    if (std::fabs(D11 + 0.5 * D33) > 1.0e-12)
      return set_error(SPC_ERR_UNSUPPORTED,
                       "Error: sys%%D(1,1) must equal -0.5*sys%%D(3,3) for isotropic conditions");
    const double w1 = -sys->B[2], w2 = -sys->B[2];
    // Hel_diag (src/hamiltonian.f90:82-86), entry by entry in the same order
    cd cz{2.0 * J + 0.0, 0.0};
    cz = cadd(cz, cd{0.0 * dk, 2.0 * dk});
    cz = cadd(cz, cd{D33, 0.0});
    for (int e = 0; e < 4; ++e) {
      const double s1 = (e >> 1) ? -0.5 : 0.5, s2 = (e & 1) ? -0.5 : 0.5;
      const cd zz = cmulx(cd{s1, 0.0}, cd{s2, 0.0});
      cd v = cadd(cadd(rsc(w1, cd{s1, 0.0}), rsc(w2, cd{s2, 0.0})), cmulx(cz, zz));
      v = csub(v, cd{0.0 * k_bar, 0.5 * k_bar});
      hs.ref.diag[e] = make_double2(v.re, v.im);
    }
    const cd one = cmulx(cd{1.0, 0.0}, cd{1.0, 0.0});
    const cd cx1 = cadd(cadd(cd{J, 0.0}, cd{0.0 * dk, 1.0 * dk}), cd{0.5 * D11, 0.0});
    const cd cx2 = cadd(cadd(cd{J, 0.0}, cd{0.0 * dk, 1.0 * dk}), cd{0.5 * D22, 0.0});
    const cd f1 = cmulx(cx1, one), f2 = cmulx(cx2, one);
    hs.ref.flip_ab = make_double2(f1.re, f1.im);
    hs.ref.flip_ba = make_double2(f2.re, f2.im);
  } else {
    // H_el = -B.(S1+S2) + S1.(D + 2J).S2 - i kbar/2 + 2 i dk S1.S2
    for (int e = 0; e < 4; ++e)
      for (int ep = 0; ep < 4; ++ep) {
        cd hv{0.0, 0.0};
        for (int r = 0; r < 3; ++r) {
          hv = csub(hv, rsc(sys->B[r], pair_el(0, r, e, ep)));
          hv = csub(hv, rsc(sys->B[r], pair_el(1, r, e, ep)));
        }
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) {
            const double dd = D[c * 3 + r] + (r == c ? 2.0 * J : 0.0);
            cd ss{0.0, 0.0};
            for (int f = 0; f < 4; ++f) ss = cadd(ss, cmulx(pair_el(0, r, e, f), pair_el(1, c, f, ep)));
            hv = cadd(hv, rsc(dd, ss));
            if (r == c) hv = cadd(hv, cmulx(cd{0.0, 2.0 * dk}, ss));
          }
        if (e == ep) hv = csub(hv, cd{0.0, 0.5 * k_bar});
        hs.gen.H[e][ep] = make_double2(hv.re, hv.im);
      }
    general_tables(hs);
  }
  return SPC_OK;
}

int64_t predict_nnz(const HostSystem& hs, int mode) {
  // per nucleus of multiplicity g: the reference builder stores (g-1)/g of the
  // rows once (S+I- or S-I+), the general builder 4(g-1)/g (two electron
  // patterns times the m -> m+1 and m -> m-1 neighbours); src/hamiltonian.f90:62-73
  const int64_t N = hs.N;
  int64_t nnz = mode == SPC_H_REFERENCE ? N + N / 2 : 4 * N;
  for (const NucInfo& q : hs.nuc) nnz += (mode == SPC_H_REFERENCE ? 1 : 4) * (N / q.g) * (q.g - 1);
  return nnz;
}

}  // namespace spc

// ===========================================================================
// host helpers of the C ABI
namespace {

struct Rng {
  uint64_t s[2] = {123456789ull, 987654321ull};
  bool have = false;
  double stored = 0.0;
};
inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
// next(), src/m_random.f90:321-331
inline uint64_t rng_next(Rng& g) {
  const uint64_t t0 = g.s[0];
  uint64_t t1 = g.s[1];
  const uint64_t res = t0 + t1;
  t1 ^= t0;
  g.s[0] = rotl(t0, 55) ^ t1 ^ (t1 << 14);
  g.s[1] = rotl(t1, 36);
  return res;
}
// jump() then seed (src/m_random.f90:90-98,124-144)
void rng_seed(Rng& g, uint64_t a, uint64_t b) {
  g.s[0] = a;
  g.s[1] = b;
  static const uint64_t J[2] = {0xbeac0467eba5facbull, 0xd86b048b86aa9922ull};
  uint64_t t0 = 0, t1 = 0;
  for (int i = 0; i < 2; ++i)
    for (int bit = 0; bit < 64; ++bit) {
      if (J[i] & (1ull << bit)) {
        t0 ^= g.s[0];
        t1 ^= g.s[1];
      }
      rng_next(g);
    }
  g.s[0] = t0;
  g.s[1] = t1;
}
// unif_01 (:159-167), two_normals (:187-198), normal (:170-183)
inline double unif01(Rng& g) {
  uint64_t x = (1023ull << 52) | (rng_next(g) >> 12);
  double d;
  std::memcpy(&d, &x, 8);
  return d - 1.0;
}
double normal(Rng& g) {
  if (g.have) {
    g.have = false;
    return g.stored;
  }
  double r0, r1, ss;
  for (;;) {
    r0 = 2.0 * unif01(g) - 1.0;
    r1 = 2.0 * unif01(g) - 1.0;
    ss = r0 * r0 + r1 * r1;
    if (ss < 1.0 && ss > 0.0) break;
  }
  const double f = std::sqrt(-2.0 * std::log(ss) / ss);
  g.stored = r1 * f;
  g.have = true;
  return r0 * f;
}
// sample_SUZ (src/qm_dynamics.f90:416-430)
void sample_suz(Rng& g, double* z, int Z) {
  for (int i = 0; i < Z; ++i) {
    z[2 * i] = normal(g);
    z[2 * i + 1] = normal(g);
  }
  double re = 0.0, im = 0.0;
  for (int i = 0; i < Z; ++i) {
    const double a = z[2 * i], b = z[2 * i + 1];
    re = re + (a * a + b * b);
    im = im + (a * b - b * a);
  }
  const double s = std::sqrt(re);
  (void)im;
  for (int i = 0; i < 2 * Z; ++i) z[i] = z[i] / s;
}

}  // namespace

extern "C" {

const char* spc_last_error(void) { return spc::last_error(); }

int spc_seeded_samples(int64_t seed0, int64_t seed1, int Z, int M, int mode, double* out) {
  if (Z < 1 || M < 0 || !out || (mode != 0 && mode != 1))
    return spc::set_error(SPC_ERR_ARG, "spc_seeded_samples: bad argument");
  Rng master;
  rng_seed(master, (uint64_t)seed0, (uint64_t)seed1);
  if (mode == 1) {
    for (int i = 0; i < M; ++i) sample_suz(master, out + 2 * (size_t)i * Z, Z);
    return SPC_OK;
  }
  std::vector<uint64_t> seeds(2 * (size_t)M);
  for (int i = 0; i < M; ++i) {
    seeds[2 * i] = rng_next(master);
    seeds[2 * i + 1] = rng_next(master);
  }
  for (int i = 0; i < M; ++i) {
    Rng g;
    rng_seed(g, seeds[2 * i], seeds[2 * i + 1]);
    sample_suz(g, out + 2 * (size_t)i * Z, Z);
  }
  return SPC_OK;
}

int spc_rng_stream(int64_t seed0, int64_t seed1, int n, uint64_t* out) {
  if (n < 0 || (n > 0 && !out)) return spc::set_error(SPC_ERR_ARG, "spc_rng_stream: bad argument");
  Rng g;
  rng_seed(g, (uint64_t)seed0, (uint64_t)seed1);
  for (int i = 0; i < n; ++i) out[i] = rng_next(g);
  return SPC_OK;
}

int spc_init_el_state(int which, double* theta, double* init_pop) {
  if (!theta || !init_pop) return spc::set_error(SPC_ERR_ARG, "null pointer");
  const double h = 1.0 / std::sqrt(2.0);
  for (int i = 0; i < 8; ++i) theta[i] = 0.0;
  for (int i = 0; i < 4; ++i) init_pop[i] = 0.0;
  switch (which) {
    case 0: theta[2] = h; theta[4] = -h; init_pop[0] = 1.0; break;
    case 1: theta[2] = h; theta[4] = h; init_pop[1] = 1.0; break;
    case 2: theta[0] = 1.0; init_pop[2] = 1.0; break;
    case 3: theta[6] = 1.0; init_pop[3] = 1.0; break;
    default:
      return spc::set_error(SPC_ERR_ARG, "Error: Invalid initial radical pair state entered.");
  }
  return SPC_OK;
}

int spc_kinetics(int T, const double* P_S, const double* P_T0, const double* P_Tp,
                 const double* P_Tm, double dt, double kS, double kT, double* Phi_S,
                 double* Phi_T, double* iden) {
  if (T < 0 || !P_S || !P_T0 || !P_Tp || !P_Tm) return spc::set_error(SPC_ERR_ARG, "bad argument");
  std::vector<double> PT(T);
  for (int i = 0; i < T; ++i) PT[i] = (P_Tp[i] + P_T0[i]) + P_Tm[i];
  if (iden)
    for (int i = 0; i < T; ++i) iden[i] = P_S[i] + PT[i];
  const int nh = T / 2;
  if (nh < 1) return SPC_OK;
  const double fS = (1.0 / 3.0) * dt * kS, fT = (1.0 / 3.0) * dt * kT;
  double ps = 0.0, pt = 0.0;
  if (Phi_S) Phi_S[0] = 0.0;
  if (Phi_T) Phi_T[0] = 0.0;
  for (int i = 1; i <= nh - 1; ++i) {
    ps = ps + fS * ((P_S[2 * i - 2] + 4.0 * P_S[2 * i - 1]) + P_S[2 * i]);
    pt = pt + fT * ((PT[2 * i - 2] + 4.0 * PT[2 * i - 1]) + PT[2 * i]);
    if (Phi_S) Phi_S[i] = ps;
    if (Phi_T) Phi_T[i] = pt;
  }
  return SPC_OK;
}

}  // extern "C"
