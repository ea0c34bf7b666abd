// ORACLE — test infrastructure only.
//
// A plain C++ restatement of the reference (KenHino/Spin_dynamics, `spinchem`)
// trace-sampling path. It is the checker that the CUDA product is compared
// against, and the timed CPU baseline. Nothing in the product links, loads or
// calls this file: only tests/, __graft_entry__.smoke() and bench.py's CPU
// legs do.
//
// Parity status: the reference is Fortran (gfortran/fpm absent, its stdlib
// dependency un-vendored), so this restatement could not be compiled against
// or run beside the original. It is pinned instead by a dense FP64
// eigendecomposition oracle and analytic known answers (tests/). Every function
// cites the reference line it follows.
//
// Build flags: the parity build uses -ffp-contract=off so that every product
// and sum is rounded exactly where the Fortran source rounds it when compiled
// without FMA contraction (x86-64 default); results are then bit-identical on
// x86-64 and aarch64. The timed baseline build uses -O3 -ffp-contract=fast
// -mcpu/-march=native and OpenMP, the same source.

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// complex(dp) arithmetic written out so the rounding points are explicit
// (gfortran's complex multiply is (ac-bd, ad+bc); dot_product conjugates its
// first argument).
struct cd {
  double re, im;
};
inline cd cadd(cd a, cd b) { return {a.re + b.re, a.im + b.im}; }
inline cd csub(cd a, cd b) { return {a.re - b.re, a.im - b.im}; }
inline cd cmul(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
// conj(a) * b, the term of Fortran dot_product(a, b)
inline cd cjmul(cd a, cd b) { return {a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re}; }
inline cd rscale(double s, cd a) { return {s * a.re, s * a.im}; }
// Complex division by a value whose imaginary part is exactly zero: Smith's
// algorithm (gfortran) reduces to (a.re/s, a.im/s).
inline cd cdiv_real(cd a, cd s) {
  if (s.im == 0.0) return {a.re / s.re, a.im / s.re};
  // general Smith division (only reached when the imaginary part is nonzero)
  if (std::fabs(s.re) >= std::fabs(s.im)) {
    double r = s.im / s.re, den = s.re + s.im * r;
    return {(a.re + a.im * r) / den, (a.im - a.re * r) / den};
  }
  double r = s.re / s.im, den = s.re * r + s.im;
  return {(a.re * r + a.im) / den, (a.im * r - a.re) / den};
}
inline cd csqrt_(cd z) {
  if (z.im == 0.0 && z.re >= 0.0) return {std::sqrt(z.re), 0.0};
  double r = std::hypot(z.re, z.im);
  double a = std::sqrt(0.5 * (r + std::fabs(z.re)));
  if (z.re >= 0) return {a, z.im / (2 * a)};
  return {std::fabs(z.im) / (2 * a), z.im >= 0 ? a : -a};
}

// ---------------------------------------------------------------------------
// xoroshiro128+ (src/m_random.f90)
struct Rng {
  uint64_t s[2] = {123456789ull, 987654321ull};
  bool have_stored = false;
  double stored = 0.0;
};
inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
// next(): src/m_random.f90:321-331
inline uint64_t rng_next(Rng& g) {
  uint64_t t0 = g.s[0], t1 = g.s[1];
  uint64_t res = t0 + t1;
  t1 ^= t0;
  g.s[0] = rotl(t0, 55) ^ t1 ^ (t1 << 14);
  g.s[1] = rotl(t1, 36);
  return res;
}
// jump(): src/m_random.f90:124-144 (constants are the signed int64 literals)
void rng_jump(Rng& g) {
  const uint64_t jmp[2] = {(uint64_t)(-4707382666127344949LL), (uint64_t)(-2852180941702784734LL)};
  uint64_t t0 = 0, t1 = 0;
  for (int i = 0; i < 2; ++i)
    for (int b = 0; b < 64; ++b) {
      if (jmp[i] & (1ull << b)) {
        t0 ^= g.s[0];
        t1 ^= g.s[1];
      }
      rng_next(g);
    }
  g.s[0] = t0;
  g.s[1] = t1;
}
// set_seed(): src/m_random.f90:90-98 (the stored-normal flag is untouched)
void rng_set_seed(Rng& g, uint64_t a, uint64_t b) {
  g.s[0] = a;
  g.s[1] = b;
  rng_jump(g);
}
// unif_01(): src/m_random.f90:159-167
inline double rng_unif01(Rng& g) {
  uint64_t x = rng_next(g);
  x = (1023ull << 52) | (x >> 12);
  double d;
  std::memcpy(&d, &x, 8);
  return d - 1.0;
}
// two_normals(): src/m_random.f90:187-198 (Marsaglia polar)
void rng_two_normals(Rng& g, double out[2]) {
  double r0, r1, sum_sq;
  for (;;) {
    r0 = 2.0 * rng_unif01(g) - 1.0;
    r1 = 2.0 * rng_unif01(g) - 1.0;
    sum_sq = r0 * r0 + r1 * r1;
    if (sum_sq < 1.0 && sum_sq > 0.0) break;
  }
  double f = std::sqrt(-2.0 * std::log(sum_sq) / sum_sq);
  out[0] = r0 * f;
  out[1] = r1 * f;
}
// normal(): src/m_random.f90:170-183
inline double rng_normal(Rng& g) {
  if (g.have_stored) {
    g.have_stored = false;
    return g.stored;
  }
  double two[2];
  rng_two_normals(g, two);
  g.stored = two[1];
  g.have_stored = true;
  return two[0];
}
// sample_SUZ(): src/qm_dynamics.f90:416-430
void sample_suz(Rng& g, cd* z, int Z) {
  for (int i = 0; i < Z; ++i) {
    z[i].re = rng_normal(g);
    z[i].im = rng_normal(g);
  }
  cd nrm{0.0, 0.0};
  for (int i = 0; i < Z; ++i) nrm = cadd(nrm, cjmul(z[i], z[i]));
  cd s = csqrt_(nrm);
  for (int i = 0; i < Z; ++i) z[i] = cdiv_real(z[i], s);
}

// ---------------------------------------------------------------------------
// COO matrices and Kronecker products (src/kroenecker.f90, src/spinop.f90),
// 1-based indices as in the reference so that the COO order is reproduced.
struct Coo {
  int nrows = 0, ncols = 0;
  std::vector<int> r, c;
  std::vector<cd> v;
  size_t nnz() const { return v.size(); }
};
// get_spinop_sp(): src/spinop.f90:58-95
void get_spinop_sp(int mult, Coo& Sz, Coo& Sp, Coo& Sm) {
  double S = ((double)mult - 1.0) / 2.0;
  Sz = Coo();
  Sp = Coo();
  Sm = Coo();
  Sz.nrows = Sz.ncols = Sp.nrows = Sp.ncols = Sm.nrows = Sm.ncols = mult;
  Sz.r.push_back(1);
  Sz.c.push_back(1);
  Sz.v.push_back({S, 0.0});
  for (int i = 2; i <= mult; ++i) {
    cd zi = csub(Sz.v[i - 2], cd{1.0, 0.0});
    Sz.r.push_back(i);
    Sz.c.push_back(i);
    Sz.v.push_back(zi);
    // sqrt(S*(S+1) - Sz(i)*Sz(i-1)) evaluated in complex arithmetic
    cd prod = cmul(Sz.v[i - 1], Sz.v[i - 2]);
    cd val = csqrt_(cd{S * (S + 1.0) - prod.re, 0.0 - prod.im});
    Sp.r.push_back(i - 1);
    Sp.c.push_back(i);
    Sp.v.push_back(val);
    Sm.r.push_back(i);
    Sm.c.push_back(i - 1);
    Sm.v.push_back(val);
  }
}
// kron_iden_right_sp(): A (x) 1_N, src/kroenecker.f90:149-172
Coo kron_iden_right(const Coo& A, int N) {
  Coo B;
  B.nrows = A.nrows * N;
  B.ncols = A.ncols * N;
  for (size_t i = 0; i < A.nnz(); ++i)
    for (int j = 0; j < N; ++j) {
      B.r.push_back(1 + (A.r[i] - 1) * N + j);
      B.c.push_back(1 + (A.c[i] - 1) * N + j);
      B.v.push_back(A.v[i]);
    }
  return B;
}
// kron_iden_left_sp(): 1_A (x) Nm, src/kroenecker.f90:174-200
Coo kron_iden_left(int A, const Coo& Nm) {
  Coo B;
  B.nrows = A * Nm.nrows;
  B.ncols = A * Nm.ncols;
  for (int i = 1; i <= A; ++i)
    for (size_t k = 0; k < Nm.nnz(); ++k) {
      B.r.push_back(Nm.r[k] + (i - 1) * Nm.nrows);
      B.c.push_back(Nm.c[k] + (i - 1) * Nm.nrows);
      B.v.push_back(Nm.v[k]);
    }
  return B;
}
// kron_sp(): src/kroenecker.f90:56-83
Coo kron(const Coo& A, const Coo& B) {
  Coo C;
  C.nrows = A.nrows * B.nrows;
  C.ncols = A.ncols * B.ncols;
  for (size_t i = 0; i < A.nnz(); ++i)
    for (size_t j = 0; j < B.nnz(); ++j) {
      C.r.push_back(B.nrows * (A.r[i] - 1) + B.r[j]);
      C.c.push_back(B.ncols * (A.c[i] - 1) + B.c[j]);
      C.v.push_back(cmul(A.v[i], B.v[j]));
    }
  return C;
}
// operator(*) overloads, src/utils.f90:91-113
Coo scale(double s, const Coo& A) {
  Coo B = A;
  for (auto& x : B.v) x = rscale(s, x);
  return B;
}
Coo scale(cd s, const Coo& A) {
  Coo B = A;
  for (auto& x : B.v) x = cmul(s, x);
  return B;
}
// operator(+), src/utils.f90:116-129 (same index structure required)
Coo add(const Coo& A, const Coo& B) {
  Coo C = A;
  for (size_t i = 0; i < C.nnz(); ++i) C.v[i] = cadd(A.v[i], B.v[i]);
  return C;
}
// eye_cp_sparse(): src/utils.f90:147-160
Coo eye_sparse(int n) {
  Coo I;
  I.nrows = I.ncols = n;
  for (int i = 1; i <= n; ++i) {
    I.r.push_back(i);
    I.c.push_back(i);
    I.v.push_back({1.0, 0.0});
  }
  return I;
}

struct Csr {
  int n = 0;
  std::vector<int> rowptr, col;  // 0-based
  std::vector<cd> val;
};

// coo_to_csr(): src/utils.f90:52-89. Counting sort by row; inside a row the
// entries land in reverse COO order.
Csr coo_to_csr(const Coo& H) {
  Csr out;
  out.n = H.nrows;
  std::vector<int> row_elem(H.nrows, 0);
  for (size_t i = 0; i < H.nnz(); ++i) row_elem[H.r[i] - 1]++;
  out.rowptr.assign(H.nrows + 1, 0);
  for (int i = 0; i < H.nrows; ++i) out.rowptr[i + 1] = out.rowptr[i] + row_elem[i];
  out.col.resize(H.nnz());
  out.val.resize(H.nnz());
  for (size_t i = 0; i < H.nnz(); ++i) {
    int r = H.r[i] - 1;
    int idx = out.rowptr[r] + row_elem[r] - 1;
    row_elem[r]--;
    out.col[idx] = H.c[i] - 1;
    out.val[idx] = H.v[i];
  }
  return out;
}

const double GAMMA_E = 176.08596;        // src/spinsys.f90:17
const double GAMMA_1H = 0.26752218708;   // src/spinsys.f90:18
const double GAMMA_14N = 0.0193297792;   // src/spinsys.f90:19

// getHiso_sp(): src/hamiltonian.f90:17-205. w1 = w2 = -B (app/main.f90:53-54).
// Returns false (the reference's `stop`) for an unsupported multiplicity or a
// non-axial dipolar tensor.
bool get_hiso_sp(int n1, const int* g1, const double* a1, int n2, const int* g2, const double* a2,
                 double w1, double w2, double J, const double* D /*col-major 3x3*/, double kS,
                 double kT, Coo& H) {
  auto Dm = [&](int r, int c) { return D[(c - 1) * 3 + (r - 1)]; };
  long Z1 = 1, Z2 = 1;
  for (int i = 0; i < n1; ++i) Z1 *= g1[i];
  for (int i = 0; i < n2; ++i) Z2 *= g2[i];
  int N = (int)(4 * Z1 * Z2);
  Coo Sz, Sp, Sm;
  get_spinop_sp(2, Sz, Sp, Sm);
  Coo S1p = kron_iden_right(Sp, 2), S1m = kron_iden_right(Sm, 2), S1z = kron_iden_right(Sz, 2);
  Coo S2p = kron_iden_left(2, Sp), S2m = kron_iden_left(2, Sm), S2z = kron_iden_left(2, Sz);
  Coo S1pS2m = kron(Sp, Sm), S1mS2p = kron(Sm, Sp), S1zS2z = kron(Sz, Sz);
  Coo E = eye_sparse(4);
  double k_bar = (kS + 3.0 * kT) / 4.0;
  double delta_k = (kS - kT) / 4.0;

  H = Coo();
  H.nrows = H.ncols = N;
  // diagonal electronic part, src/hamiltonian.f90:82-90
  cd cz{2.0 * J + 0.0, 0.0};
  cz = cadd(cz, cd{0.0 * delta_k, 2.0 * delta_k});
  cz = cadd(cz, cd{Dm(3, 3), 0.0});
  Coo Hel = add(add(scale(w1, S1z), scale(w2, S2z)), scale(cz, S1zS2z));
  for (auto& x : Hel.v) x = csub(x, cd{0.0 * k_bar, 0.5 * k_bar});
  Coo T = kron_iden_right(Hel, (int)(Z1 * Z2));
  H.r = T.r;
  H.c = T.c;
  H.v = T.v;
  // off-diagonal electronic part, src/hamiltonian.f90:93-110
  if (std::fabs(Dm(1, 1) - Dm(2, 2)) > 1.0e-12) return false;
  if (std::fabs(Dm(1, 1) + 0.5 * Dm(3, 3)) > 1.0e-12) return false;
  auto append = [&](const Coo& X) {
    H.r.insert(H.r.end(), X.r.begin(), X.r.end());
    H.c.insert(H.c.end(), X.c.begin(), X.c.end());
    H.v.insert(H.v.end(), X.v.begin(), X.v.end());
  };
  cd cx1 = cadd(cadd(cd{J, 0.0}, cd{0.0 * delta_k, 1.0 * delta_k}), cd{0.5 * Dm(1, 1), 0.0});
  append(kron_iden_right(scale(cx1, S1pS2m), (int)(Z1 * Z2)));
  cd cx2 = cadd(cadd(cd{J, 0.0}, cd{0.0 * delta_k, 1.0 * delta_k}), cd{0.5 * Dm(2, 2), 0.0});
  append(kron_iden_right(scale(cx2, S1mS2p), (int)(Z1 * Z2)));

  // hyperfine + nuclear Zeeman for both electrons, src/hamiltonian.f90:112-203
  for (int e = 1; e <= 2; ++e) {
    int n = e == 1 ? n1 : n2;
    const int* g = e == 1 ? g1 : g2;
    const double* a = e == 1 ? a1 : a2;
    double w = e == 1 ? w1 : w2;
    const Coo& Sez = e == 1 ? S1z : S2z;
    const Coo& Sep = e == 1 ? S1p : S2p;
    const Coo& Sem = e == 1 ? S1m : S2m;
    Coo Iz, Ip, Im;
    if (n > 0) get_spinop_sp(g[0], Iz, Ip, Im);
    for (int i = 0; i < n; ++i) {
      if (i > 0 && g[i] != g[i - 1]) get_spinop_sp(g[i], Iz, Ip, Im);
      long Zl = 1, Zr = 1;
      if (e == 1) {
        for (int k = 0; k < i; ++k) Zl *= g[k];
        for (int k = i + 1; k < n; ++k) Zr *= g[k];
        Zr *= Z2;
      } else {
        Zl = Z1;
        for (int k = 0; k < i; ++k) Zl *= g[k];
        for (int k = i + 1; k < n; ++k) Zr *= g[k];
      }
      double zf;
      if (g[i] == 3)
        zf = -(w * GAMMA_14N / GAMMA_E);
      else if (g[i] == 2)
        zf = -(w * GAMMA_1H / GAMMA_E);
      else
        return false;
      Coo X = add(scale(a[i], Sez), scale(zf, E));
      Coo Td = kron(kron_iden_right(X, (int)Zl), kron_iden_right(Iz, (int)Zr));
      for (int k = 0; k < N; ++k) H.v[k] = cadd(H.v[k], Td.v[k]);
      append(kron(kron_iden_right(scale(0.5 * a[i], Sep), (int)Zl), kron_iden_right(Im, (int)Zr)));
      append(kron(kron_iden_right(scale(0.5 * a[i], Sem), (int)Zl), kron_iden_right(Ip, (int)Zr)));
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// General Hamiltonian (no sparse reference counterpart; the anisotropic
// hyperfine S.A.I form follows getH_dense, src/hamiltonian.f90:279-284,
// 306-311, while the Zeeman signs, nuclear Zeeman and Haberkorn term keep
// getHiso_sp's convention, src/hamiltonian.f90:82-110,132-139):
//   H = -B.(S1+S2) + sum_j (gamma_j/gamma_e) B.I_j + S1.(D + 2J 1).S2
//       + sum_j S_e(j).A_j.I_j - i kbar/2 + 2 i dk S1.S2
// Row entries are emitted in ascending column order; the structural pattern
// is fixed (explicit zeros are kept) so that it does not depend on values.
struct SpinHalf {
  // <a|S_r|b> for a,b in {0 (alpha), 1 (beta)}, r in {x,y,z}
  static cd el(int r, int a, int b) {
    if (r == 2) return a == b ? cd{a == 0 ? 0.5 : -0.5, 0.0} : cd{0.0, 0.0};
    if (a == b) return {0.0, 0.0};
    if (r == 0) return {0.5, 0.0};
    // Sy: <0|Sy|1> = -i/2, <1|Sy|0> = +i/2
    return a == 0 ? cd{0.0, -0.5} : cd{0.0, 0.5};
  }
};
// <m_a|I_c|m_b> for a nucleus of multiplicity g, states indexed 0..g-1 from m=+I.
cd nuc_el(int g, int c, int a, int b) {
  double I = (g - 1) / 2.0;
  double ma = I - a, mb = I - b;
  if (c == 2) return a == b ? cd{ma, 0.0} : cd{0.0, 0.0};
  double ladder = 0.0;  // I+ : a = b-1 ; I- : a = b+1
  if (a == b - 1) ladder = std::sqrt(I * (I + 1.0) - ma * mb);
  else if (a == b + 1) ladder = std::sqrt(I * (I + 1.0) - ma * mb);
  else return {0.0, 0.0};
  if (c == 0) return {0.5 * ladder, 0.0};
  // Iy = (I+ - I-)/(2i): <a|Iy|b> = -i/2 ladder for a=b-1 (I+), +i/2 for a=b+1
  return a == b - 1 ? cd{0.0, -0.5 * ladder} : cd{0.0, 0.5 * ladder};
}

struct GenSys {
  int nn;                     // total nuclei, radical-1 first
  std::vector<int> g, owner;  // multiplicity, electron (0 or 1)
  std::vector<double> A;      // nn x 9, A[j*9 + r*3 + c] = A_j(r,c)
  std::vector<double> zeta;   // nn x 3: (gamma_j/gamma_e) * B_c
  std::vector<long> stride;   // index stride of each nucleus in the nuclear index
  cd Hel[4][4];
  long Z;
};

// <e|S_{k,r}|e'> for electron k (0 or 1) in the 4-dim pair basis e = 2*s1+s2
cd pair_el(int k, int r, int e, int ep) {
  int s1 = e >> 1, s2 = e & 1, t1 = ep >> 1, t2 = ep & 1;
  if (k == 0) return s2 == t2 ? SpinHalf::el(r, s1, t1) : cd{0.0, 0.0};
  return s1 == t1 ? SpinHalf::el(r, s2, t2) : cd{0.0, 0.0};
}

void build_gen_sys(int n1, const int* g1, const double* A1, int n2, const int* g2,
                   const double* A2, const double* gam1, const double* gam2, const double* B,
                   double J, const double* D /*col-major*/, double kS, double kT, GenSys& s) {
  s.nn = n1 + n2;
  s.g.clear();
  s.owner.clear();
  s.A.clear();
  s.zeta.clear();
  for (int e = 0; e < 2; ++e) {
    int n = e == 0 ? n1 : n2;
    for (int i = 0; i < n; ++i) {
      int gi = e == 0 ? g1[i] : g2[i];
      const double* Ai = (e == 0 ? A1 : A2) + 9 * i;  // column-major 3x3 as in input.ini
      double gm = e == 0 ? gam1[i] : gam2[i];
      s.g.push_back(gi);
      s.owner.push_back(e);
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) s.A.push_back(Ai[c * 3 + r]);
      for (int c = 0; c < 3; ++c) s.zeta.push_back((gm / GAMMA_E) * B[c]);
    }
  }
  s.stride.assign(s.nn, 1);
  long st = 1;
  for (int j = s.nn - 1; j >= 0; --j) {
    s.stride[j] = st;
    st *= s.g[j];
  }
  s.Z = st;
  double k_bar = (kS + 3.0 * kT) / 4.0, dk = (kS - kT) / 4.0;
  for (int e = 0; e < 4; ++e)
    for (int ep = 0; ep < 4; ++ep) {
      cd h{0.0, 0.0};
      for (int r = 0; r < 3; ++r) {
        h = csub(h, rscale(B[r], pair_el(0, r, e, ep)));
        h = csub(h, rscale(B[r], pair_el(1, r, e, ep)));
      }
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          double dd = D[c * 3 + r] + (r == c ? 2.0 * J : 0.0);
          cd ss{0.0, 0.0};
          for (int f = 0; f < 4; ++f) ss = cadd(ss, cmul(pair_el(0, r, e, f), pair_el(1, c, f, ep)));
          h = cadd(h, rscale(dd, ss));
          if (r == c) h = cadd(h, cmul(cd{0.0, 2.0 * dk}, ss));
        }
      if (e == ep) h = csub(h, cd{0.0, 0.5 * k_bar});
      s.Hel[e][ep] = h;
    }
}

// Emit the entries of row `row` in ascending column order.
int gen_row(const GenSys& s, long row, long* cols, cd* vals) {
  int e = (int)(row / s.Z);
  long nidx = row % s.Z;
  int n_out = 0;
  // candidate list: (column, value) accumulated in a tiny map
  struct Ent {
    long c;
    cd v;
  };
  Ent ent[256];
  int ne = 0;
  auto put = [&](long c, cd v) {
    for (int k = 0; k < ne; ++k)
      if (ent[k].c == c) {
        ent[k].v = cadd(ent[k].v, v);
        return;
      }
    ent[ne].c = c;
    ent[ne].v = v;
    ne++;
  };
  // electron block: all four electron states, nuclear state unchanged
  for (int ep = 0; ep < 4; ++ep) put(ep * s.Z + nidx, s.Hel[e][ep]);
  for (int j = 0; j < s.nn; ++j) {
    int g = s.g[j], k = s.owner[j];
    int mj = (int)((nidx / s.stride[j]) % g);
    const double* A = &s.A[9 * j];
    const double* zt = &s.zeta[3 * j];
    for (int mp = mj - 1; mp <= mj + 1; ++mp) {
      if (mp < 0 || mp >= g) continue;
      long nc = nidx + (long)(mp - mj) * s.stride[j];
      for (int ep = 0; ep < 4; ++ep) {
        // only e' = e or e' = e with electron k flipped
        int other_same = k == 0 ? ((e & 1) == (ep & 1)) : ((e >> 1) == (ep >> 1));
        if (!other_same) continue;
        cd v{0.0, 0.0};
        for (int r = 0; r < 3; ++r) {
          cd se = pair_el(k, r, e, ep);
          for (int c = 0; c < 3; ++c) {
            cd ie = nuc_el(g, c, mj, mp);
            v = cadd(v, rscale(A[r * 3 + c], cmul(se, ie)));
          }
        }
        if (ep == e)
          for (int c = 0; c < 3; ++c) v = cadd(v, rscale(zt[c], nuc_el(g, c, mj, mp)));
        put(ep * s.Z + nc, v);
      }
    }
  }
  std::sort(ent, ent + ne, [](const Ent& a, const Ent& b) { return a.c < b.c; });
  for (int k = 0; k < ne; ++k) {
    cols[n_out] = ent[k].c;
    vals[n_out] = ent[k].v;
    n_out++;
  }
  return n_out;
}

// ---------------------------------------------------------------------------
// CSR spmv (stdlib spmv with alpha=1, beta=0, called at src/qm_dynamics.f90:452)
void spmv(const Csr& H, const cd* x, cd* y) {
  for (int i = 0; i < H.n; ++i) {
    cd acc{0.0, 0.0};
    for (int k = H.rowptr[i]; k < H.rowptr[i + 1]; ++k) acc = cadd(acc, cmul(H.val[k], x[H.col[k]]));
    y[i] = acc;
  }
}

inline cd dotc(const cd* a, const cd* b, long n) {
  cd acc{0.0, 0.0};
  for (long i = 0; i < n; ++i) acc = cadd(acc, cjmul(a[i], b[i]));
  return acc;
}

// get_krylov(): src/qm_dynamics.f90:432-467. Q is N x m column-major,
// A is m x m column-major (A[i + j*m] = A(i+1, j+1)).
void get_krylov(int N, const cd* psi, const Csr& H, int m, cd* Q, cd* c, cd* A, cd* p) {
  for (int i = 0; i < m; ++i) c[i] = {0.0, 0.0};
  c[0] = csqrt_(dotc(psi, psi, N));
  for (int i = 0; i < m * m; ++i) A[i] = {0.0, 0.0};
  for (int n = 0; n < N; ++n) Q[n] = cdiv_real(psi[n], c[0]);
  for (int i = 0; i < m - 1; ++i) {
    spmv(H, Q + (long)i * N, p);
    for (int j = 0; j <= i; ++j) {
      const cd* qj = Q + (long)j * N;
      cd a = dotc(qj, p, N);
      A[j + i * m] = a;
      for (int n = 0; n < N; ++n) p[n] = csub(p[n], cmul(a, qj[n]));
    }
    cd b = csqrt_(dotc(p, p, N));
    A[(i + 1) + i * m] = b;
    cd* qn = Q + (long)(i + 1) * N;
    for (int n = 0; n < N; ++n) qn[n] = cdiv_real(p[n], b);
  }
  spmv(H, Q + (long)(m - 1) * N, p);
  for (int j = 0; j < m; ++j) {
    const cd* qj = Q + (long)j * N;
    cd a = dotc(qj, p, N);
    A[j + (m - 1) * m] = a;
    for (int n = 0; n < N; ++n) p[n] = csub(p[n], cmul(a, qj[n]));
  }
}

// column-major n x n: C = A * B (Fortran matmul, k summed in order)
void matmul(int n, const cd* A, const cd* B, cd* C) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      cd acc{0.0, 0.0};
      for (int k = 0; k < n; ++k) acc = cadd(acc, cmul(A[i + k * n], B[k + j * n]));
      C[i + j * n] = acc;
    }
}

// inverse by LU with partial pivoting (stdlib `inv` -> LAPACK getrf/getri;
// pivot chosen by |re|+|im| as izamax does)
bool inv(int n, const cd* Ain, cd* X) {
  std::vector<cd> LU(Ain, Ain + (size_t)n * n);
  std::vector<int> piv(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = -1.0;
    for (int i = k; i < n; ++i) {
      double v = std::fabs(LU[i + k * n].re) + std::fabs(LU[i + k * n].im);
      if (v > best) {
        best = v;
        p = i;
      }
    }
    piv[k] = p;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(LU[k + j * n], LU[p + j * n]);
    cd d = LU[k + k * n];
    if (d.re == 0.0 && d.im == 0.0) return false;
    for (int i = k + 1; i < n; ++i) {
      // l = LU(i,k)/d (general complex division, Smith)
      cd a = LU[i + k * n];
      cd l;
      if (std::fabs(d.re) >= std::fabs(d.im)) {
        double r = d.im / d.re, den = d.re + d.im * r;
        l = {(a.re + a.im * r) / den, (a.im - a.re * r) / den};
      } else {
        double r = d.re / d.im, den = d.re * r + d.im;
        l = {(a.re * r + a.im) / den, (a.im * r - a.re) / den};
      }
      LU[i + k * n] = l;
      for (int j = k + 1; j < n; ++j) LU[i + j * n] = csub(LU[i + j * n], cmul(l, LU[k + j * n]));
    }
  }
  // solve LU X = P I column by column
  for (int j = 0; j < n; ++j) {
    std::vector<cd> b(n, cd{0.0, 0.0});
    b[j] = {1.0, 0.0};
    // apply the row interchanges to the unit column
    std::vector<cd> bb(n);
    for (int i = 0; i < n; ++i) bb[i] = i == j ? cd{1.0, 0.0} : cd{0.0, 0.0};
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) std::swap(bb[k], bb[piv[k]]);
    for (int i = 0; i < n; ++i) {
      cd acc = bb[i];
      for (int k = 0; k < i; ++k) acc = csub(acc, cmul(LU[i + k * n], bb[k]));
      bb[i] = acc;
    }
    for (int i = n - 1; i >= 0; --i) {
      cd acc = bb[i];
      for (int k = i + 1; k < n; ++k) acc = csub(acc, cmul(LU[i + k * n], bb[k]));
      cd d = LU[i + i * n];
      if (std::fabs(d.re) >= std::fabs(d.im)) {
        double r = d.im / d.re, den = d.re + d.im * r;
        bb[i] = {(acc.re + acc.im * r) / den, (acc.im - acc.re * r) / den};
      } else {
        double r = d.re / d.im, den = d.re * r + d.im;
        bb[i] = {(acc.re * r + acc.im) / den, (acc.im * r - acc.re) / den};
      }
    }
    for (int i = 0; i < n; ++i) X[i + j * n] = bb[i];
  }
  return true;
}

// expm(): src/matrix_exponential.f90:14-87 (Pade(6,6), scaling and squaring)
bool expm(int n, const cd* A, cd* E) {
  const int q = 6;
  std::vector<cd> A2(A, A + (size_t)n * n), D(n * n), X(n * n), T(n * n);
  // mat_norm_linf(): src/matrix_exponential.f90:89-104
  double a_norm = 0.0;
  for (int i = 0; i < n; ++i) {
    double row = 0.0;
    for (int j = 0; j < n; ++j) row += std::hypot(A2[i + j * n].re, A2[i + j * n].im);
    a_norm = std::max(a_norm, row);
  }
  int s;
  if (a_norm == 0.0) {
    s = 0;  // int(-huge) saturates to INT_MIN: s = max(0, ...) = 0
  } else {
    double l2 = std::log(std::fabs(a_norm)) / std::log(2.0);  // log_2(), :106-117
    int ee = (int)l2 + 1;                                      // int() truncates toward zero
    s = std::max(0, ee + 1);
  }
  double sc = std::pow(2.0, s);
  for (auto& x : A2) x = {x.re / sc, x.im / sc};
  X = A2;
  double c = 0.5;
  for (int i = 0; i < n * n; ++i) {
    cd id = (i % (n + 1) == 0) ? cd{1.0, 0.0} : cd{0.0, 0.0};
    E[i] = cadd(id, rscale(c, A2[i]));
    D[i] = csub(id, rscale(c, A2[i]));
  }
  bool p = true;
  for (int k = 2; k <= q; ++k) {
    c = c * (double)(q - k + 1) / (double)(k * (2 * q - k + 1));
    matmul(n, A2.data(), X.data(), T.data());
    X = T;
    for (int i = 0; i < n * n; ++i) {
      cd cx = rscale(c, X[i]);
      E[i] = cadd(E[i], cx);
      D[i] = p ? cadd(D[i], cx) : csub(D[i], cx);
    }
    p = !p;
  }
  std::vector<cd> Di(n * n);
  if (!inv(n, D.data(), Di.data())) return false;
  std::vector<cd> Ec(E, E + (size_t)n * n);
  matmul(n, Di.data(), Ec.data(), E);
  for (int k = 0; k < s; ++k) {
    Ec.assign(E, E + (size_t)n * n);
    matmul(n, Ec.data(), Ec.data(), E);
  }
  return true;
}

// convert_to_krylov(): src/qm_dynamics.f90:469-498 (full m x m, column-major)
void convert_to_krylov(int m, const cd* Q, int N, int Z, cd* PS, cd* PT0, cd* PTp, cd* PTm) {
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) {
      const cd* qi = Q + (long)i * N;
      const cd* qj = Q + (long)j * N;
      PTp[i + j * m] = dotc(qi, qj, Z);
      cd Pab = dotc(qi + Z, qj + Z, Z);
      cd Pba = dotc(qi + 2 * Z, qj + 2 * Z, Z);
      cd ZQC = dotc(qi + 2 * Z, qj + Z, Z);
      cd half = rscale(0.5, cadd(Pab, Pba));
      PT0[i + j * m] = cadd(half, ZQC);
      PS[i + j * m] = csub(half, ZQC);
      PTm[i + j * m] = dotc(qi + 3 * Z, qj + 3 * Z, Z);
    }
}

// column-major m x m times vector
inline void matvec(int m, const cd* A, const cd* x, cd* y) {
  for (int i = 0; i < m; ++i) {
    cd acc{0.0, 0.0};
    for (int j = 0; j < m; ++j) acc = cadd(acc, cmul(A[i + j * m], x[j]));
    y[i] = acc;
  }
}

}  // namespace

// ===========================================================================
// C ABI used by the tests and the CPU baseline (ctypes). All complex arrays
// are interleaved (re, im) doubles. CSR output is 0-based.
extern "C" {

int orc_version(void) { return 3; }

int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

// RNG pieces (src/m_random.f90), for unit tests of the restatement.
void orc_rng_stream(uint64_t s0, uint64_t s1, int do_seed, int n, uint64_t* out) {
  Rng g;
  g.s[0] = s0;
  g.s[1] = s1;
  if (do_seed) rng_set_seed(g, s0, s1);
  for (int i = 0; i < n; ++i) out[i] = rng_next(g);
}
void orc_rng_normals(uint64_t s0, uint64_t s1, int n, double* out) {
  Rng g;
  rng_set_seed(g, s0, s1);
  for (int i = 0; i < n; ++i) out[i] = rng_normal(g);
}

// Sample vectors exactly as trace_sampling_para draws them
// (app/main.f90:48 seeds the master generator; src/qm_dynamics.f90:315-327
// draws two next() per sample, then set_seed + sample_SUZ per sample).
// mode 0: trace_sampling_para (per-sample seeds); mode 1: trace_sampling
// (serial, src/qm_dynamics.f90:198-199, one stream across samples).
// out: M x Z complex, sample-major.
void orc_seeded_samples(uint64_t seed0, uint64_t seed1, int Z, int M, int mode, double* out) {
  Rng master;
  rng_set_seed(master, seed0, seed1);
  cd* z = reinterpret_cast<cd*>(out);
  if (mode == 1) {
    for (int i = 0; i < M; ++i) sample_suz(master, z + (size_t)i * Z, Z);
    return;
  }
  std::vector<uint64_t> seeds(2 * (size_t)M);
  for (int i = 0; i < M; ++i) {
    seeds[2 * i] = rng_next(master);
    seeds[2 * i + 1] = rng_next(master);
  }
  for (int i = 0; i < M; ++i) {
    Rng g;  // fresh private copy: the stored-normal flag starts false and an
            // even number (2Z) of normal() calls per sample leaves it false
    rng_set_seed(g, seeds[2 * i], seeds[2 * i + 1]);
    sample_suz(g, z + (size_t)i * Z, Z);
  }
}

// getHiso_sp + coo_to_csr. w = -B on both electrons. Returns nnz (>0), or a
// negative code: -1 unsupported multiplicity / non-axial D (the reference
// stops), -2 output buffer too small. With rowptr == NULL only nnz is
// returned.
long orc_build_h_iso(int n1, const int* g1, const double* a1, int n2, const int* g2,
                     const double* a2, double B, double J, const double* D9, double kS, double kT,
                     long cap, int* rowptr, int* col, double* val) {
  Coo H;
  if (!get_hiso_sp(n1, g1, a1, n2, g2, a2, -B, -B, J, D9, kS, kT, H)) return -1;
  if (!rowptr) return (long)H.nnz();
  if ((long)H.nnz() > cap) return -2;
  Csr C = coo_to_csr(H);
  std::memcpy(rowptr, C.rowptr.data(), sizeof(int) * (C.n + 1));
  std::memcpy(col, C.col.data(), sizeof(int) * C.col.size());
  std::memcpy(val, C.val.data(), sizeof(cd) * C.val.size());
  return (long)H.nnz();
}

// The raw COO (1-based), for checking the assembly order itself.
long orc_build_h_iso_coo(int n1, const int* g1, const double* a1, int n2, const int* g2,
                         const double* a2, double B, double J, const double* D9, double kS,
                         double kT, long cap, int* rows, int* cols, double* val) {
  Coo H;
  if (!get_hiso_sp(n1, g1, a1, n2, g2, a2, -B, -B, J, D9, kS, kT, H)) return -1;
  if (!rows) return (long)H.nnz();
  if ((long)H.nnz() > cap) return -2;
  std::memcpy(rows, H.r.data(), sizeof(int) * H.nnz());
  std::memcpy(cols, H.c.data(), sizeof(int) * H.nnz());
  std::memcpy(val, H.v.data(), sizeof(cd) * H.nnz());
  return (long)H.nnz();
}

// General anisotropic Hamiltonian. A1/A2: 9 doubles per nucleus, column-major
// 3x3 (input.ini order). gam1/gam2: gyromagnetic ratio per nucleus. B: field
// vector (mT). D9: column-major 3x3. Returns nnz or a negative code.
long orc_build_h_general(int n1, const int* g1, const double* A1, const double* gam1, int n2,
                         const int* g2, const double* A2, const double* gam2, const double* B,
                         double J, const double* D9, double kS, double kT, long cap, int* rowptr,
                         int* col, double* val) {
  GenSys s;
  build_gen_sys(n1, g1, A1, n2, g2, A2, gam1, gam2, B, J, D9, kS, kT, s);
  long N = 4 * s.Z;
  long cols[256];
  cd vals[256];
  long nnz = 0;
  for (long r = 0; r < N; ++r) {
    int k = gen_row(s, r, cols, vals);
    if (rowptr) {
      if (nnz + k > cap) return -2;
      rowptr[r] = (int)nnz;
      for (int i = 0; i < k; ++i) {
        col[nnz + i] = (int)cols[i];
        val[2 * (nnz + i)] = vals[i].re;
        val[2 * (nnz + i) + 1] = vals[i].im;
      }
    }
    nnz += k;
  }
  if (rowptr) rowptr[N] = (int)nnz;
  return nnz;
}

// expm of an n x n column-major complex matrix (for unit tests).
int orc_expm(int n, const double* A, double* E) {
  return expm(n, reinterpret_cast<const cd*>(A), reinterpret_cast<cd*>(E)) ? 0 : 1;
}

// Number of output time points: N_steps + 1, N_steps = ceiling((t_end+dt)/dt)
// (src/qm_dynamics.f90:305-306).
int orc_num_time_points(double dt, double t_end) {
  double x = (t_end + dt) / dt;
  double c = std::ceil(x);
  return (int)c + 1;
}

// init_el_state(): src/qm_dynamics.f90:386-414. which: 0 singlet, 1 T0, 2 Tp, 3 Tm.
int orc_init_el_state(int which, double* theta, double* init_pop) {
  double h = 1.0 / std::sqrt(2.0);
  for (int i = 0; i < 8; ++i) theta[i] = 0.0;
  for (int i = 0; i < 4; ++i) init_pop[i] = 0.0;
  switch (which) {
    case 0: theta[2] = h; theta[4] = -h; init_pop[0] = 1.0; break;
    case 1: theta[2] = h; theta[4] = h; init_pop[1] = 1.0; break;
    case 2: theta[0] = 1.0; init_pop[2] = 1.0; break;
    case 3: theta[6] = 1.0; init_pop[3] = 1.0; break;
    default: return 1;
  }
  return 0;
}

// trace_sampling_para(): src/qm_dynamics.f90:257-384, on caller-supplied
// sample vectors. CSR is 0-based; zkets: M x Z complex sample-major; theta:
// 4 complex; init_pop: 4. Outputs (length T each, T from
// orc_num_time_points): the sample-averaged populations, in the reference's
// order P_S, P_T0, P_Tp, P_Tm. per_sample (optional, M x 4 x T) keeps each
// sample's unaveraged arrays. n_builds (optional, M) counts Krylov builds
// per sample. Returns 0, or 1 on a bad argument / time index overflow.
int orc_trace_sampling(int N, const int* rowptr, const int* col, const double* val,
                       const double* theta, const double* init_pop, const double* zkets, int M,
                       double dt, double t_end, int m, double tol, double* P_S, double* P_T0,
                       double* P_Tp, double* P_Tm, int T, double* per_sample, long* n_builds) {
  if (N % 4 != 0 || m < 1 || M < 1) return 1;
  int Z = N / 4;
  Csr H;
  H.n = N;
  H.rowptr.assign(rowptr, rowptr + N + 1);
  H.col.assign(col, col + rowptr[N]);
  H.val.resize(rowptr[N]);
  std::memcpy(H.val.data(), val, sizeof(cd) * rowptr[N]);
  const cd* th = reinterpret_cast<const cd*>(theta);
  const cd* zk = reinterpret_cast<const cd*>(zkets);
  std::vector<double> obs((size_t)M * 4 * T, 0.0);
  int err = 0;

#pragma omp parallel
  {
    std::vector<cd> psi(N), Q((size_t)N * m), p(N), c(m), A(m * m), Ax(m * m), Aexp(m * m);
    std::vector<cd> PS(m * m), PT0(m * m), PTp(m * m), PTm(m * m), tmp(m), v(m);
#pragma omp for schedule(dynamic, 1)
    for (int s = 0; s < M; ++s) {
      double* o = &obs[(size_t)s * 4 * T];
      // kron_vector(theta, Z_ket), src/kroenecker.f90:85-97
      for (int e = 0; e < 4; ++e)
        for (int n = 0; n < Z; ++n) psi[(size_t)e * Z + n] = cmul(th[e], zk[(size_t)s * Z + n]);
      o[0 * T] = init_pop[0];
      o[1 * T] = init_pop[1];
      o[2 * T] = init_pop[2];
      o[3 * T] = init_pop[3];
      double t = 0.0;
      int k = 1;  // 0-based slot of the reference's k = 2
      long builds = 0;
      while (t < t_end) {
        get_krylov(N, psi.data(), H, m, Q.data(), c.data(), A.data(), p.data());
        builds++;
        // expm((0,-1)*dt*A): the scalar (0,-dt) times each entry
        for (int i = 0; i < m * m; ++i) Ax[i] = cmul(cd{0.0, -1.0 * dt}, A[i]);
        expm(m, Ax.data(), Aexp.data());
        convert_to_krylov(m, Q.data(), N, Z, PS.data(), PT0.data(), PTp.data(), PTm.data());
        double c2 = 1.0, cm2 = 0.0;
        while (cm2 <= tol * c2 && t < t_end) {
          matvec(m, Aexp.data(), c.data(), tmp.data());
          for (int i = 0; i < m; ++i) c[i] = tmp[i];
          if (k >= T) {
#pragma omp atomic write
            err = 1;
            break;
          }
          matvec(m, PS.data(), c.data(), v.data());
          o[0 * T + k] = dotc(c.data(), v.data(), m).re;
          matvec(m, PTp.data(), c.data(), v.data());
          o[2 * T + k] = dotc(c.data(), v.data(), m).re;
          matvec(m, PT0.data(), c.data(), v.data());
          o[1 * T + k] = dotc(c.data(), v.data(), m).re;
          matvec(m, PTm.data(), c.data(), v.data());
          o[3 * T + k] = dotc(c.data(), v.data(), m).re;
          c2 = dotc(c.data(), c.data(), m).re;
          cd cm = c[m - 1];
          cm2 = cmul(cm, cd{cm.re, -cm.im}).re;
          t = t + dt;
          k = k + 1;
        }
        // psi = matmul(Q, c)
        for (int n = 0; n < N; ++n) {
          cd acc{0.0, 0.0};
          for (int j = 0; j < m; ++j) acc = cadd(acc, cmul(Q[(size_t)j * N + n], c[j]));
          psi[n] = acc;
        }
        if (err) break;
      }
      if (n_builds) n_builds[s] = builds;
    }
  }
  if (err) return 1;
  // res%update in sample order, then res%scale(1/N_samples),
  // src/qm_dynamics.f90:373-378 and src/observables.f90:52-72
  double* outs[4] = {P_S, P_T0, P_Tp, P_Tm};
  double inv_m = 1.0 / (double)M;
  for (int q = 0; q < 4; ++q) {
    for (int i = 0; i < T; ++i) {
      double acc = 0.0;
      for (int s = 0; s < M; ++s) acc = acc + obs[(size_t)s * 4 * T + (size_t)q * T + i];
      outs[q][i] = acc * inv_m;
    }
  }
  if (per_sample) std::memcpy(per_sample, obs.data(), sizeof(double) * obs.size());
  return 0;
}

// get_kinetics(): src/observables.f90:74-101. Inputs length T; Phi_S and
// Phi_T get T/2 entries; iden gets T entries (any output may be NULL).
void orc_kinetics(int T, const double* P_S, const double* P_T0, const double* P_Tp,
                  const double* P_Tm, double dt, double kS, double kT, double* Phi_S,
                  double* Phi_T, double* iden) {
  std::vector<double> PT(T);
  for (int i = 0; i < T; ++i) PT[i] = (P_Tp[i] + P_T0[i]) + P_Tm[i];
  if (iden)
    for (int i = 0; i < T; ++i) iden[i] = P_S[i] + PT[i];
  int nh = T / 2;
  if (nh < 1) return;
  double fS = (1.0 / 3.0) * dt * kS, fT = (1.0 / 3.0) * dt * kT;
  double ps = 0.0, pt = 0.0;
  if (Phi_S) Phi_S[0] = 0.0;
  if (Phi_T) Phi_T[0] = 0.0;
  for (int i = 1; i <= nh - 1; ++i) {
    // 1-based P(2i-1), P(2i), P(2i+1)
    ps = ps + fS * ((P_S[2 * i - 2] + 4.0 * P_S[2 * i - 1]) + P_S[2 * i]);
    pt = pt + fT * ((PT[2 * i - 2] + 4.0 * PT[2 * i - 1]) + PT[2 * i]);
    if (Phi_S) Phi_S[i] = ps;
    if (Phi_T) Phi_T[i] = pt;
  }
}

}  // extern "C"
