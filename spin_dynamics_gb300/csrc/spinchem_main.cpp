// spinchem — command-line drop-in for the reference executable (app/main.f90):
//
//   spinchem input.ini
//
// reads the same input.ini keys with the same unit conversions and errors
// (read_inp / check_inp / electron_init, src/spinsys.f90:60-235), runs the
// selected simulation type for all the listed fields (app/main.f90:48-79)
// together through libspinchem_gpu's batch calls, and writes the same files
// into the same folders
// (<output_folder>/<B in F0.3>/S_prob.data, Tp_prob.data, T0_prob.data,
// Tm_prob.data; src/observables.f90:103-148). Where the reference stops with
// a message, this prints the same message and exits with status 1.
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/spinchem_gpu.h"

namespace {

const double GAMMA_E = 176.08596;  // src/spinsys.f90:17

[[noreturn]] void stop(const std::string& msg) {
  std::fprintf(stderr, "%s\n", msg.c_str());
  std::exit(1);
}

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? "" : s.substr(a, b - a + 1);
}

// Sections, "key = value" options, whitespace-separated lists (the subset of
// FiNeR's file_ini the reference uses).
struct Ini {
  std::map<std::string, std::map<std::string, std::string>> sec;
  std::vector<std::string> order;
  bool load(const std::string& path) {
    std::ifstream f(path);
    if (!f) return false;
    std::string line, cur;
    bool have = false;
    while (std::getline(f, line)) {
      line = trim(line);
      if (line.empty() || line[0] == ';' || line[0] == '#' || line[0] == '!') continue;
      if (line[0] == '[' && line.find(']') != std::string::npos) {
        cur = trim(line.substr(1, line.find(']') - 1));
        if (!sec.count(cur)) order.push_back(cur);
        sec[cur];
        have = true;
        continue;
      }
      size_t eq = line.find('=');
      if (eq == std::string::npos || !have) continue;
      sec[cur][trim(line.substr(0, eq))] = trim(line.substr(eq + 1));
    }
    return true;
  }
  const std::string* get(const std::string& s, const std::string& k) const {
    auto i = sec.find(s);
    if (i == sec.end()) return nullptr;
    auto j = i->second.find(k);
    return j == i->second.end() ? nullptr : &j->second;
  }
  std::vector<std::string> list(const std::string& s, const std::string& k) const {
    std::vector<std::string> out;
    const std::string* v = get(s, k);
    if (!v) return out;
    std::istringstream is(*v);
    std::string t;
    while (is >> t) out.push_back(t);
    return out;
  }
};

struct Electron {
  double g = 2.002319;
  std::vector<int> gI;
  std::vector<double> A;  // 9 per nucleus, column-major (input.ini order)
  bool isotropic() const {  // src/spinsys.f90:237-254
    for (size_t i = 0; i < gI.size(); ++i)
      if (A[9 * i + 0] != A[9 * i + 4]) return false;
    return true;
  }
  long Z() const {
    long z = 1;
    for (int g_ : gI) z *= g_;
    return z;
  }
};

struct Sys {
  Electron e1, e2;
  double J = 0, D[9] = {0}, kS = 0, kT = 0;
};

struct Sim {
  std::string type, init_state, output_folder;
  std::vector<double> B;
  int64_t seed[2] = {123456789, 987654321};
  int N_samples = 1, N_krylov = 7, M1 = 1, M2 = 1, restart = 0;
  double t_end = 0, dt = 0, tol = 1e-5, block_tol = 1e-5;
  bool isRestart = false;
};

double to_d(const std::string& s) { return std::strtod(s.c_str(), nullptr); }

// check_inp (src/spinsys.f90:137-163)
void check_inp(const Ini& ini) {
  const char* sections[4] = {"system variables", "simulation parameters", "electron 1", "electron 2"};
  if (ini.sec.size() < 4) stop("Error: Number of sections in input file is less than expected.");
  if (ini.sec.size() > 4) stop("Error: Number of sections in input file is more than expected.");
  for (const char* s : sections)
    if (!ini.sec.count(s)) stop(std::string("Error: Section \"") + s + "\" is missing from input file.");
}

// electron_init (src/spinsys.f90:165-235)
Electron electron_init(const Ini& ini, int n) {
  Electron e;
  const std::string sec = "electron " + std::to_string(n);
  if (const std::string* g = ini.get(sec, "g")) e.g = to_d(*g);
  std::vector<std::string> I = ini.list(sec, "I"), NI = ini.list(sec, "N_I");
  if (I.empty() || NI.empty()) {
    I.clear();
    NI.clear();
  }
  if (I.size() != NI.size()) stop("Sections N_I and I must have the sam length.");
  for (size_t i = 0; i < I.size(); ++i)
    for (int k = 0; k < std::atoi(NI[i].c_str()); ++k) e.gI.push_back(std::atoi(I[i].c_str()));
  for (size_t i = 0; i < e.gI.size(); ++i) {
    std::vector<std::string> a = ini.list(sec, "A" + std::to_string(i + 1));
    if (a.size() < 9) {
      char buf[128];
      std::snprintf(buf, sizeof(buf), "Error: Hyperfine copuling A%zu for electron %d is missing.", i + 1, n);
      stop(buf);
    }
    for (int k = 0; k < 9; ++k) e.A.push_back(to_d(a[k]));
  }
  return e;
}

// read_inp (src/spinsys.f90:60-135)
void read_inp(const std::string& file, Sys& sys, Sim& sim) {
  Ini ini;
  if (!ini.load(file)) stop("Error: Input file does not exist.");
  check_inp(ini);
  const std::string sv = "system variables", sp = "simulation parameters";
  auto need = [&](const std::string& s, const std::string& k, const char* msg) -> std::string {
    const std::string* v = ini.get(s, k);
    if (!v) stop(msg);
    return *v;
  };
  sys.J = to_d(need(sv, "J", "Error: Exchange coupling is missing"));
  std::vector<std::string> D = ini.list(sv, "D");
  if (D.size() < 9) stop("Error: Dipolar coupling is missing");
  for (int k = 0; k < 9; ++k) sys.D[k] = to_d(D[k]);
  sys.kS = to_d(need(sv, "kS", "Error: Singlet recombination rate is missing")) / GAMMA_E;
  sys.kT = to_d(need(sv, "kT", "Error: Triplet recombination rate is missing")) / GAMMA_E;
  sim.type = need(sp, "simulation_type", "Error: Simulation type is missing");
  std::vector<std::string> B = ini.list(sp, "B");
  if (B.empty()) stop("Error: List of experiment magnetic fields is missing");
  for (auto& b : B) sim.B.push_back(to_d(b));
  sim.init_state = need(sp, "initial_state", "Error: Initial state is missing");
  double dt = to_d(need(sp, "dt", "Error: Propagation timestep is missing"));
  std::vector<std::string> seed = ini.list(sp, "seed");
  if (seed.size() >= 2) {
    sim.seed[0] = std::strtoll(seed[0].c_str(), nullptr, 10);
    sim.seed[1] = std::strtoll(seed[1].c_str(), nullptr, 10);
  }
  if (const std::string* v = ini.get(sp, "N_samples")) sim.N_samples = std::atoi(v->c_str());
  double t_end = 0;
  if (const std::string* v = ini.get(sp, "simulation_time")) t_end = to_d(*v);
  sim.t_end = (t_end * GAMMA_E) / 1000.0;
  sim.dt = (dt * GAMMA_E) / 1000.0;
  if (const std::string* v = ini.get(sp, "block_tolerance")) sim.block_tol = to_d(*v);
  if (const std::string* v = ini.get(sp, "N_krylov")) sim.N_krylov = std::atoi(v->c_str());
  if (const std::string* v = ini.get(sp, "integrator_tolerance")) sim.tol = to_d(*v);
  if (const std::string* v = ini.get(sp, "M1")) sim.M1 = std::atoi(v->c_str());
  if (const std::string* v = ini.get(sp, "M2")) sim.M2 = std::atoi(v->c_str());
  if (const std::string* v = ini.get(sp, "restart")) {
    sim.restart = std::atoi(v->c_str());
    sim.isRestart = true;
  }
  if (const std::string* v = ini.get(sp, "output_folder")) sim.output_folder = *v;
  struct stat st;
  if (stat(sim.output_folder.c_str(), &st) != 0 || !S_ISDIR(st.st_mode))
    stop("Error: Output folder does not exist.");
  sys.e1 = electron_init(ini, 1);
  sys.e2 = electron_init(ini, 2);
}

// One REAL(8) as gfortran's list-directed WRITE prints it (17 significant
// digits, fixed for 0.1 <= |x| < 1e17, else d.dddE+xxx; width 26).
std::string list_directed(double x) {
  char body[64];
  if (x == 0.0) {
    std::snprintf(body, sizeof(body), "0.0000000000000000     ");
  } else if (!std::isfinite(x)) {
    std::snprintf(body, sizeof(body), "%23s", std::isnan(x) ? "NaN" : (x > 0 ? "Infinity" : "-Infinity"));
  } else {
    char m[64];
    std::snprintf(m, sizeof(m), "%.16e", x);
    int e = std::atoi(std::strchr(m, 'e') + 1);
    if (e >= -1 && e < 17) {
      std::snprintf(body, sizeof(body), "%.*f     ", e == -1 ? 17 : 16 - e, x);
    } else {
      *std::strchr(m, 'e') = '\0';
      std::snprintf(body, sizeof(body), "%sE%c%03d", m, e < 0 ? '-' : '+', std::abs(e));
    }
  }
  char out[64];
  std::snprintf(out, sizeof(out), " %25s", body);
  return out;
}

void write_data(const std::vector<double>& d, const std::string& path, const char* name) {
  FILE* f = std::fopen((path + "/" + name).c_str(), "w");
  if (!f) stop(std::string("Error: cannot write ") + path + "/" + name);
  for (double v : d) std::fprintf(f, "%s\n", list_directed(v).c_str());
  std::fclose(f);
}

// write(guz,'(F0.3)') B (app/main.f90:58)
std::string f0_3(double B) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%.3f", std::fabs(B));
  std::string s = buf;
  if (s.rfind("0.", 0) == 0) s = s.substr(1);
  if (B < 0 && std::strtod(buf, nullptr) != 0.0) s = "-" + s;
  return s;
}

void check(int rc) {
  if (rc != SPC_OK) stop(std::string("Error: ") + spc_last_error());
}

struct Result {
  std::vector<double> PS, PT0, PTp, PTm;
};

int init_state_index(const Sim& sim) {
  const int which = sim.init_state == "singlet" ? 0 : sim.init_state == "T0" ? 1 : sim.init_state == "Tp" ? 2
                  : sim.init_state == "Tm" ? 3 : -1;
  if (which < 0) stop("Error: Invalid initial radical pair state entered.");
  return which;
}

// Consecutive groups of jobs whose vector entries (rows x samples padded to
// tiles of 32) stay under a third of the device's free memory at m + 4
// complex states per entry; a job larger than that is a group of its own.
std::vector<std::vector<size_t>> batch_groups(const std::vector<double>& entries, int m) {
  int64_t free_b = 0, total_b = 0;
  check(spc_mem_info(0, &free_b, &total_b));
  const double budget = std::max(1.0, (double)free_b / 3.0 / (16.0 * (m + 4)));
  std::vector<std::vector<size_t>> out;
  std::vector<size_t> cur;
  double tot = 0.0;
  for (size_t i = 0; i < entries.size(); ++i) {
    if (!cur.empty() && tot + entries[i] > budget) {
      out.push_back(cur);
      cur.clear();
      tot = 0.0;
    }
    cur.push_back(i);
    tot += entries[i];
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

double padded(int M) { return (double)((M + 31) / 32 * 32); }

// trace_sampling_para / trace_sampling / exact_dynamics (src/qm_dynamics.f90)
// for every field of the list (app/main.f90:48-79) in one batch: main
// re-seeds the generator with sim%seed before each field (app/main.f90:50),
// so every field propagates the same vectors. Each field's Hamiltonian
// (getHiso_sp with w = -B) is one system of the batch store; groups of
// fields bounded by device memory share one build and one propagation.
std::vector<Result> run_fields(spc_handle* h, const Sys& sys, const Sim& sim) {
  if (!(sys.e1.isotropic() && sys.e2.isotropic()))
    stop("Anisotropic Hamiltoninans have not been implemented yet");
  std::vector<int> g1 = sys.e1.gI, g2 = sys.e2.gI;
  const long Z = sys.e1.Z() * sys.e2.Z();
  double theta[8], pop[4];
  check(spc_init_el_state(init_state_index(sim), theta, pop));
  std::vector<double> zk;
  int M;
  if (sim.type == "exact_dynamics") {
    M = (int)Z;
    zk.assign(2 * (size_t)Z * Z, 0.0);
    for (long i = 0; i < Z; ++i) zk[2 * ((size_t)i * Z + i)] = 1.0;
  } else {
    M = sim.N_samples;
    zk.resize(2 * (size_t)Z * M);
    check(spc_seeded_samples(sim.seed[0], sim.seed[1], (int)Z, M,
                             sim.type == "trace_sampling_serial" ? 1 : 0, zk.data()));
  }
  const int T = spc_num_time_points(sim.dt, sim.t_end);
  if (T < 1) stop("Error: Propagation timestep is missing");
  const size_t nB = sim.B.size();
  std::vector<Result> res(nB);
  const std::vector<double> entries(nB, 4.0 * (double)Z * padded(M));
  for (const std::vector<size_t>& grp : batch_groups(entries, sim.N_krylov)) {
    std::vector<spc_system> systems(grp.size());
    std::vector<double> zk_all;
    for (size_t j = 0; j < grp.size(); ++j) {
      spc_system& s = systems[j];
      s = spc_system{};
      s.n_nuc1 = (int)g1.size();
      s.n_nuc2 = (int)g2.size();
      s.mult1 = g1.data();
      s.mult2 = g2.data();
      s.A1 = sys.e1.A.data();
      s.A2 = sys.e2.A.data();
      s.B[2] = sim.B[grp[j]];
      s.J = sys.J;
      std::memcpy(s.D, sys.D, sizeof(s.D));
      s.kS = sys.kS;
      s.kT = sys.kT;
      zk_all.insert(zk_all.end(), zk.begin(), zk.end());
    }
    check(spc_build_h_batch(h, (int)systems.size(), systems.data(), SPC_H_REFERENCE));
    std::vector<int> Ms(grp.size(), M);
    std::vector<double> out(grp.size() * 4 * (size_t)T);
    check(spc_trace_sampling_batch(h, (int)grp.size(), nullptr, Ms.data(), theta, pop, zk_all.data(), sim.dt,
                                   sim.t_end, sim.N_krylov, sim.tol, out.data(), T));
    for (size_t j = 0; j < grp.size(); ++j) {
      const double* o = &out[j * 4 * (size_t)T];
      Result& r = res[grp[j]];
      r.PS.assign(o, o + T);
      r.PT0.assign(o + T, o + 2 * T);
      r.PTp.assign(o + 2 * T, o + 3 * T);
      r.PTm.assign(o + 3 * T, o + 4 * T);
    }
  }
  return res;
}

// ---------------------------------------------------------------------------
// symmetry_dynamics (src/symmetry.f90:16-139) with the moment matching of
// src/moments.f90:15-240: equivalent spin-1/2 nuclei (1H) of each radical form
// groups; every combination of the groups' total spins is a block (an
// ordinary radical pair whose "nuclei" are the groups, multiplicity 2I+1),
// propagated together through the batch ABI, weighted by
// prod C(n, (n+k-1)/2) 2k/(n+k+1) * Z_block / Z and summed.

const double GAMMA_1H = 0.26752218708;   // src/spinsys.f90:18
const double GAMMA_14N = 0.0193297792;   // src/spinsys.f90:19

// Eigenvalues (ascending) and eigenvectors (columns of V, row-major n x n) of
// a small symmetric matrix by cyclic Jacobi rotations.
void jacobi_eig(int n, std::vector<double> A, std::vector<double>& w, std::vector<double>& V) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        tot += A[i * n + j] * A[i * n + j];
        if (i != j) off += A[i * n + j] * A[i * n + j];
      }
    if (off <= 1e-32 * tot || off == 0.0) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p * n + q];
        if (apq == 0.0) continue;
        // rotation angle zeroing A[p][q]: tan(2 phi) = 2 apq / (aqq - app)
        const double tau = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t), sn = t * c;
        for (int k = 0; k < n; ++k) {  // A <- A R (columns p, q)
          const double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - sn * akq;
          A[k * n + q] = sn * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // A <- R^T A (rows p, q)
          const double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - sn * aqk;
          A[q * n + k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - sn * vkq;
          V[k * n + q] = sn * vkp + c * vkq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return A[a * n + a] < A[b * n + b]; });
  w.resize(n);
  std::vector<double> Vs((size_t)n * n);
  for (int c = 0; c < n; ++c) {
    w[c] = A[idx[c] * n + idx[c]];
    for (int r = 0; r < n; ++r) Vs[r * n + c] = V[r * n + idx[c]];
  }
  V.swap(Vs);
}

// quad_rule (src/moments.f90:97-158): the N-point Gauss rule of the discrete
// measure (W_init, X_init) by Stieltjes/Lanczos; nodes ascending.
void quad_rule(const std::vector<double>& Wi, const std::vector<double>& Xi, int N, std::vector<double>& W,
               std::vector<double>& X) {
  const size_t L = Xi.size();
  std::vector<double> q(L), P(L * N), w(N), x(N);
  for (size_t i = 0; i < L; ++i) q[i] = std::sqrt(Wi[i]);
  for (int k = 0; k < N; ++k) {
    double q2 = 0.0;
    for (double v : q) q2 += v * v;
    q2 = std::sqrt(q2);
    if (q2 == 0.0) stop("quad_rule 1");
    for (size_t i = 0; i < L; ++i) P[i * N + k] = q[i] / q2;
    for (size_t i = 0; i < L; ++i) q[i] = Xi[i] * P[i * N + k];
    for (int j = k; j >= 0; --j) {
      double pq = 0.0;
      for (size_t i = 0; i < L; ++i) pq += P[i * N + j] * q[i];
      if (j == k) {
        w[k] = q2;
        x[k] = pq;
      }
      for (size_t i = 0; i < L; ++i) q[i] -= pq * P[i * N + j];
    }
  }
  std::vector<double> T((size_t)N * N, 0.0), V;
  for (int i = 0; i < N; ++i) {
    T[i * N + i] = x[i];
    if (i + 1 < N) T[i * N + i + 1] = T[(i + 1) * N + i] = w[i + 1];  // cshift(W, 1)
  }
  jacobi_eig(N, T, X, V);
  W.resize(N);
  for (int k = 0; k < N; ++k) W[k] = (w[0] * V[k]) * (w[0] * V[k]);
}

// newton (src/moments.f90:182-240): sum_j n_j a_j^k = sum_j w_j aw_j^k, k = 1..M.
int newton(const std::vector<double>& aw, const std::vector<double>& wb, std::vector<double>& a,
           const std::vector<double>& nb, int M) {
  double dap = 0.0;
  for (int it = 1; it <= 30; ++it) {
    std::vector<double> f(M), g((size_t)M * M);
    for (int k = 1; k <= M; ++k) {
      double s1 = 0.0, s2 = 0.0;
      for (int j = 0; j < M; ++j) {
        s1 += nb[j] * std::pow(a[j], k);
        s2 += wb[j] * std::pow(aw[j], k);
      }
      f[k - 1] = s1 - s2;
      for (int j = 0; j < M; ++j) g[(k - 1) * M + j] = k * nb[j] * std::pow(a[j], k - 1);
    }
    // g q = f by Gaussian elimination with partial pivoting
    std::vector<double> qv = f;
    for (int c = 0; c < M; ++c) {
      int pr = c;
      for (int r = c + 1; r < M; ++r)
        if (std::fabs(g[r * M + c]) > std::fabs(g[pr * M + c])) pr = r;
      if (g[pr * M + c] == 0.0) return 1;
      if (pr != c) {
        for (int j = 0; j < M; ++j) std::swap(g[c * M + j], g[pr * M + j]);
        std::swap(qv[c], qv[pr]);
      }
      for (int r = c + 1; r < M; ++r) {
        const double l = g[r * M + c] / g[c * M + c];
        for (int j = c; j < M; ++j) g[r * M + j] -= l * g[c * M + j];
        qv[r] -= l * qv[c];
      }
    }
    for (int c = M - 1; c >= 0; --c) {
      double acc = qv[c];
      for (int j = c + 1; j < M; ++j) acc -= g[c * M + j] * qv[j];
      qv[c] = acc / g[c * M + c];
    }
    double a_abs = 0.0, d_abs = 0.0;
    for (int j = 0; j < M; ++j) {
      a_abs += std::fabs(a[j]);
      d_abs += std::fabs(qv[j]);
    }
    std::vector<double> a_old = a;
    for (int j = 0; j < M; ++j) a[j] -= qv[j];
    const double da = d_abs / a_abs;
    if (da > 1.0) return 1;
    if (1.0 + da == 1.0) return 0;
    if (it > 1 && da >= dap) {
      a = a_old;
      return 0;
    }
    dap = da;
  }
  return 2;
}

// shrink (src/moments.f90:15-95): M groups (couplings, sizes) matching the
// moments of the couplings a.
void shrink(const std::vector<double>& a, int M, std::vector<double>& a_bar, std::vector<int>& n_bar) {
  const int N = (int)a.size();
  if (M >= N) stop("Error: Symetry reduction requires M<N");
  std::vector<double> wb, aw;
  quad_rule(std::vector<double>(N, 1.0), a, M, wb, aw);
  std::vector<int> nfloor(M);
  int fsum = 0;
  for (int i = 0; i < M; ++i) {
    nfloor[i] = (int)wb[i];
    fsum += nfloor[i];
  }
  const int ndiff = N - fsum;
  double dmom = std::numeric_limits<double>::max();
  bool found = false;
  for (int ib = 0; ib < (1 << M); ++ib) {
    if (__builtin_popcount((unsigned)ib) != ndiff) continue;
    std::vector<double> nt(M), at = aw;
    for (int i = 0; i < M; ++i) nt[i] = nfloor[i] + ((ib >> i) & 1);
    if (newton(aw, wb, at, nt, M) != 0) continue;
    double emom = 0.0;
    for (int k = 1; k <= M + 1; ++k) {
      double s1 = 0.0, s2 = 0.0;
      for (double v : at) s1 += std::pow(v, k);
      for (double v : a) s2 += std::pow(v, k);
      emom += std::fabs(s1 - s2);
    }
    if (emom < dmom) {
      dmom = emom;
      a_bar = at;
      n_bar.assign(M, 0);
      for (int i = 0; i < M; ++i) n_bar[i] = (int)nt[i];
      found = true;
    }
  }
  if (!found) stop("Error: moment matching found no integer group sizes");
}

struct Groups {
  std::vector<double> a;  // group couplings
  std::vector<int> n;     // group sizes
  std::vector<int> other; // explicit nuclei (indices)
};

double a_iso(const Electron& e, int i) {
  const double* A = &e.A[9 * (size_t)i];
  return ((A[0] + A[4]) + A[8]) / 3.0;
}

Groups radical_groups(const Electron& e, int M) {
  Groups G;
  std::vector<double> a;
  for (size_t i = 0; i < e.gI.size(); ++i) {
    if (e.gI[i] == 2)
      a.push_back(a_iso(e, (int)i));
    else
      G.other.push_back((int)i);
  }
  if (a.empty() || M == 0) return G;
  std::vector<double> vals = a;
  std::sort(vals.begin(), vals.end());
  vals.erase(std::unique(vals.begin(), vals.end()), vals.end());
  if ((int)vals.size() == M) {  // exactly M distinct couplings: exact groups
    for (double v : vals) {
      G.a.push_back(v);
      G.n.push_back((int)std::count(a.begin(), a.end(), v));
    }
  } else {
    shrink(a, M, G.a, G.n);
  }
  return G;
}

int64_t n_choose_r(int64_t n, int64_t r) {
  if (r < 0 || r > n) return 0;
  int64_t c = 1;
  for (int64_t i = 1; i <= r; ++i) c = c * (n - r + i) / i;
  return c;
}

struct Block {
  double w;
  Electron e1, e2;          // the block's radicals: groups then explicit nuclei
  std::vector<double> gam1, gam2;
  long Z;
};

std::vector<Block> blocks(const Sys& sys, int M1, int M2) {
  const Groups G1 = radical_groups(sys.e1, M1), G2 = radical_groups(sys.e2, M2);
  std::vector<int> n = G1.n;
  n.insert(n.end(), G2.n.begin(), G2.n.end());
  // every combination of group multiplicities k = 2j + 1 + n mod 2, the
  // first group fastest (cartesian_product, src/symmetry.f90:171-208)
  std::vector<std::vector<int>> opts(n.size());
  for (size_t i = 0; i < n.size(); ++i)
    for (int j = 0; j <= n[i] / 2; ++j) opts[i].push_back(2 * j + 1 + n[i] % 2);
  std::vector<std::vector<int>> combos;
  std::vector<size_t> pos(n.size(), 0);
  while (true) {
    std::vector<int> c(n.size());
    for (size_t i = 0; i < n.size(); ++i) c[i] = opts[i][pos[i]];
    combos.push_back(c);
    size_t i = 0;
    while (i < n.size() && ++pos[i] == opts[i].size()) pos[i++] = 0;
    if (i == n.size()) break;
  }
  // stable order by block dimension (sort_col_prod, src/utils.f90:25-50)
  std::vector<int64_t> zc(combos.size(), 1);
  for (size_t c = 0; c < combos.size(); ++c)
    for (int k : combos[c]) zc[c] *= k;
  std::vector<size_t> order(combos.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return zc[a] < zc[b]; });
  int64_t z_expl = 1, z_full = sys.e1.Z() * sys.e2.Z();
  for (int i : G1.other) z_expl *= sys.e1.gI[i];
  for (int i : G2.other) z_expl *= sys.e2.gI[i];
  auto default_gamma = [](int g) { return g == 3 ? GAMMA_14N : GAMMA_1H; };
  std::vector<Block> out;
  for (size_t oi : order) {
    const std::vector<int>& K = combos[oi];
    int64_t w_ij = 1;
    for (size_t i = 0; i < n.size(); ++i) {
      const int64_t ni = n[i], ki = K[i];
      w_ij = w_ij * (n_choose_r(ni, (ni + ki - 1) / 2) * (2 * ki) / (ni + ki + 1));
    }
    Block b;
    const int64_t Zb = zc[oi] * z_expl;
    b.w = (double)(w_ij * Zb) / (double)z_full;
    b.Z = (long)Zb;
    auto radical = [&](const Electron& e, const Groups& G, size_t k0, Electron& re, std::vector<double>& gam) {
      re.g = e.g;
      for (size_t i = 0; i < G.a.size(); ++i) {
        re.gI.push_back(K[k0 + i]);
        const double a9[9] = {G.a[i], 0, 0, 0, G.a[i], 0, 0, 0, G.a[i]};
        re.A.insert(re.A.end(), a9, a9 + 9);
        gam.push_back(GAMMA_1H);
      }
      for (int i : G.other) {
        re.gI.push_back(e.gI[i]);
        re.A.insert(re.A.end(), e.A.begin() + 9 * (size_t)i, e.A.begin() + 9 * (size_t)i + 9);
        gam.push_back(default_gamma(e.gI[i]));
      }
    };
    radical(sys.e1, G1, 0, b.e1, b.gam1);
    radical(sys.e2, G2, G1.a.size(), b.e2, b.gam2);
    out.push_back(std::move(b));
  }
  return out;
}

// One block's populations as trace_sampling_para writes them into its
// folder (res%output(folder), src/qm_dynamics.f90:379-382), and read back.
const char* kBlockFiles[4] = {"S_prob.data", "T0_prob.data", "Tp_prob.data", "Tm_prob.data"};

std::string block_folder(const std::string& field_folder, size_t i) {
  return field_folder + "/hamiltonian_" + std::to_string(i + 1);
}

std::vector<double> read_data(const std::string& path, int T) {
  std::ifstream f(path);
  if (!f) stop("Error: restart: no saved block results in " + path);
  std::vector<double> v;
  std::string line;
  while (std::getline(f, line))
    if (!trim(line).empty()) v.push_back(std::strtod(line.c_str(), nullptr));
  if ((int)v.size() != T)
    stop("Error: restart: " + path + " holds " + std::to_string(v.size()) + " values, expected " +
         std::to_string(T));
  return v;
}

// symmetrised_dynamics (src/symmetry.f90:16-139) for every field of the list:
// every (field, block) job with weight >= block_tol, from the restart block
// on, in batches bounded by device memory. Each propagated block's
// populations go to <field folder>/hamiltonian_<i>/ (the reference writes
// them to <output_folder>/hamiltonian_<i>/, which every field overwrites);
// blocks before the restart block are read back from there, so a run that
// was stopped resumes where it left off (the reference leaves them
// unallocated). Weighted sum in block order, yields, the seven files.
void symmetrised_dynamics(spc_handle* h, const Sys& sys, const Sim& sim, const std::vector<std::string>& folders) {
  std::vector<Block> bl = blocks(sys, sim.M1, sim.M2);
  std::vector<uint64_t> seeds(std::max<size_t>(1, 2 * bl.size()));
  check(spc_rng_stream(sim.seed[0], sim.seed[1], (int)(2 * bl.size()), seeds.data()));
  const int start = sim.isRestart ? sim.restart : 1;
  std::vector<size_t> sel, run;  // blocks that count; of those, the ones to propagate
  for (size_t i = 0; i < bl.size(); ++i)
    if (bl[i].w >= sim.block_tol) {
      sel.push_back(i);
      if ((int)i + 1 >= start) run.push_back(i);
    }
  double theta[8], pop[4];
  check(spc_init_el_state(init_state_index(sim), theta, pop));
  const int T = spc_num_time_points(sim.dt, sim.t_end);
  if (T < 1) stop("Error: Propagation timestep is missing");
  // the block vectors (the same for every field: seeds per block from sim%seed)
  std::vector<std::vector<double>> zk(bl.size());
  for (size_t i : run) {
    zk[i].resize(2 * (size_t)bl[i].Z * sim.N_samples);
    check(spc_seeded_samples((int64_t)seeds[2 * i], (int64_t)seeds[2 * i + 1], (int)bl[i].Z, sim.N_samples, 0,
                             zk[i].data()));
  }
  // jobs block-major: a run stopped after some batches has finished every
  // field of its first blocks, so restart = the first unfinished block
  // resumes it
  const size_t nB = sim.B.size();
  std::vector<std::pair<size_t, size_t>> jobs;
  std::vector<double> entries;
  for (size_t i : run)
    for (size_t k = 0; k < nB; ++k) {
      jobs.push_back({k, i});
      entries.push_back(4.0 * (double)bl[i].Z * padded(sim.N_samples));
    }
  std::map<std::pair<size_t, size_t>, std::vector<double>> out;  // (field, block) -> S|T0|Tp|Tm
  for (const std::vector<size_t>& grp : batch_groups(entries, sim.N_krylov)) {
    std::vector<spc_system> systems(grp.size());
    std::vector<int> M(grp.size(), sim.N_samples);
    std::vector<double> zk_all;
    for (size_t j = 0; j < grp.size(); ++j) {
      const Block& b = bl[jobs[grp[j]].second];
      spc_system& s = systems[j];
      s = spc_system{};
      s.n_nuc1 = (int)b.e1.gI.size();
      s.n_nuc2 = (int)b.e2.gI.size();
      s.mult1 = b.e1.gI.data();
      s.mult2 = b.e2.gI.data();
      s.A1 = b.e1.A.data();
      s.A2 = b.e2.A.data();
      s.gamma1 = b.gam1.data();
      s.gamma2 = b.gam2.data();
      s.B[2] = sim.B[jobs[grp[j]].first];
      s.J = sys.J;
      std::memcpy(s.D, sys.D, sizeof(s.D));
      s.kS = sys.kS;
      s.kT = sys.kT;
      const std::vector<double>& z = zk[jobs[grp[j]].second];
      zk_all.insert(zk_all.end(), z.begin(), z.end());
    }
    check(spc_build_h_batch(h, (int)systems.size(), systems.data(), SPC_H_REFERENCE));
    std::vector<double> o(grp.size() * 4 * (size_t)T);
    check(spc_trace_sampling_batch(h, (int)grp.size(), nullptr, M.data(), theta, pop, zk_all.data(), sim.dt,
                                   sim.t_end, sim.N_krylov, sim.tol, o.data(), T));
    for (size_t j = 0; j < grp.size(); ++j) {  // block files as soon as the batch is done
      const size_t k = jobs[grp[j]].first, i = jobs[grp[j]].second;
      std::vector<double>& r = out[{k, i}];
      r.assign(o.begin() + j * 4 * T, o.begin() + (j + 1) * 4 * T);
      const std::string bf = block_folder(folders[k], i);
      mkdir(bf.c_str(), 0755);
      for (int c = 0; c < 4; ++c)
        write_data(std::vector<double>(r.begin() + c * T, r.begin() + (c + 1) * T), bf, kBlockFiles[c]);
    }
  }
  for (size_t k = 0; k < nB; ++k) {
    std::printf(" %g\n", sim.B[k]);
    std::vector<std::vector<double>> res(4, std::vector<double>(T, 0.0));  // S, T0, Tp, Tm
    for (size_t i : sel) {
      std::vector<std::vector<double>> P(4);
      if ((int)i + 1 >= start) {
        const std::vector<double>& o = out[{k, i}];
        for (int c = 0; c < 4; ++c) P[c].assign(o.begin() + c * T, o.begin() + (c + 1) * T);
      } else {
        for (int c = 0; c < 4; ++c) P[c] = read_data(block_folder(folders[k], i) + "/" + kBlockFiles[c], T);
      }
      const double w = bl[i].w;
      for (int c = 0; c < 4; ++c)  // res%scale(w) then res%update, block by block
        for (int t = 0; t < T; ++t) res[c][t] += P[c][t] * w;
    }
    std::vector<double> phiS(T / 2), phiT(T / 2), iden(T);
    check(spc_kinetics(T, res[0].data(), res[1].data(), res[2].data(), res[3].data(), sim.dt, sys.kS, sys.kT,
                       phiS.data(), phiT.data(), iden.data()));
    write_data(res[0], folders[k], "S_prob.data");
    write_data(res[2], folders[k], "Tp_prob.data");
    write_data(res[1], folders[k], "T0_prob.data");
    write_data(res[3], folders[k], "Tm_prob.data");
    write_data(iden, folders[k], "total_prob.data");
    write_data(phiS, folders[k], "S_yield.data");
    write_data(phiT, folders[k], "T_yield.data");
  }
}

}  // namespace

int main(int argc, char** argv) {
  auto t0 = std::chrono::steady_clock::now();
  std::printf(" Program initialised\n");
  if (argc < 2) stop("Error: Input file does not exist.");
  struct stat st;
  if (stat(argv[1], &st) != 0) stop("Error: Input file does not exist.");
  Sys sys;
  Sim sim;
  read_inp(argv[1], sys, sim);
  const char* dev = std::getenv("SPINCHEM_DEVICE");
  spc_handle* h = nullptr;
  check(spc_create(dev ? std::atoi(dev) : 0, &h));
  if (const char* km = std::getenv("SPINCHEM_KRYLOV"))  // mgs | lanczos | auto
    check(spc_set_krylov(h, std::strcmp(km, "lanczos") == 0 ? SPC_KRYLOV_LANCZOS
                            : std::strcmp(km, "auto") == 0  ? SPC_KRYLOV_AUTO
                                                            : SPC_KRYLOV_MGS));
  std::vector<std::string> folders;
  for (double B : sim.B) {
    folders.push_back(sim.output_folder + "/" + f0_3(B));
    mkdir(folders.back().c_str(), 0755);
  }
  if (sim.type == "trace_sampling" || sim.type == "trace_sampling_serial" || sim.type == "exact_dynamics") {
    const std::vector<Result> rs = run_fields(h, sys, sim);
    for (size_t k = 0; k < rs.size(); ++k) {
      write_data(rs[k].PS, folders[k], "S_prob.data");
      write_data(rs[k].PTp, folders[k], "Tp_prob.data");
      write_data(rs[k].PT0, folders[k], "T0_prob.data");
      write_data(rs[k].PTm, folders[k], "Tm_prob.data");
    }
  } else if (sim.type == "symmetry_dynamics") {
    symmetrised_dynamics(h, sys, sim, folders);
  } else if (sim.type == "semi_classical") {
    for (size_t k = 0; k < sim.B.size(); ++k) std::printf(" method not yet implemented\n");
  } else {
    stop("Error: Invalid simulation type entered.");
  }
  spc_destroy(h);
  const long secs =
      (long)std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (sim.type != "symmetry_dynamics")
    std::printf("Time elapsed:  %2ld:%2ld:%2ld\n", secs / 3600, (secs / 60) % 60, secs % 60);
  return 0;
}
