// spinchem — command-line drop-in for the reference executable (app/main.f90):
//
//   spinchem input.ini
//
// reads the same input.ini keys with the same unit conversions and errors
// (read_inp / check_inp / electron_init, src/spinsys.f90:60-235), loops over
// the listed fields (app/main.f90:48-79), runs the selected simulation type
// through libspinchem_gpu, and writes the same files into the same folders
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

// trace_sampling_para / trace_sampling / exact_dynamics (src/qm_dynamics.f90)
Result run_dynamics(spc_handle* h, const Sys& sys, const Sim& sim, double B) {
  if (!(sys.e1.isotropic() && sys.e2.isotropic()))
    stop("Anisotropic Hamiltoninans have not been implemented yet");
  std::vector<int> g1 = sys.e1.gI, g2 = sys.e2.gI;
  spc_system s{};
  s.n_nuc1 = (int)g1.size();
  s.n_nuc2 = (int)g2.size();
  s.mult1 = g1.data();
  s.mult2 = g2.data();
  s.A1 = sys.e1.A.data();
  s.A2 = sys.e2.A.data();
  s.B[2] = B;
  s.J = sys.J;
  std::memcpy(s.D, sys.D, sizeof(s.D));
  s.kS = sys.kS;
  s.kT = sys.kT;
  check(spc_build_h(h, &s, SPC_H_REFERENCE));
  const long Z = sys.e1.Z() * sys.e2.Z();
  int which = sim.init_state == "singlet" ? 0 : sim.init_state == "T0" ? 1 : sim.init_state == "Tp" ? 2
            : sim.init_state == "Tm" ? 3 : -1;
  if (which < 0) stop("Error: Invalid initial radical pair state entered.");
  double theta[8], pop[4];
  check(spc_init_el_state(which, theta, pop));
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
  Result r;
  r.PS.resize(T);
  r.PT0.resize(T);
  r.PTp.resize(T);
  r.PTm.resize(T);
  check(spc_trace_sampling(h, theta, pop, zk.data(), M, sim.dt, sim.t_end, sim.N_krylov, sim.tol,
                           r.PS.data(), r.PT0.data(), r.PTp.data(), r.PTm.data(), T));
  return r;
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
  for (double B : sim.B) {
    const std::string folder = sim.output_folder + "/" + f0_3(B);
    mkdir(folder.c_str(), 0755);
    if (sim.type == "trace_sampling" || sim.type == "trace_sampling_serial" ||
        sim.type == "exact_dynamics") {
      Result r = run_dynamics(h, sys, sim, B);
      write_data(r.PS, folder, "S_prob.data");
      write_data(r.PTp, folder, "Tp_prob.data");
      write_data(r.PT0, folder, "T0_prob.data");
      write_data(r.PTm, folder, "Tm_prob.data");
    } else if (sim.type == "symmetry_dynamics") {
      std::printf(" %g\n", B);
      stop("Error: symmetry_dynamics runs through the Python layer "
           "(python -m spin_dynamics_gb300 input.ini)");
    } else if (sim.type == "semi_classical") {
      std::printf(" method not yet implemented\n");
    } else {
      stop("Error: Invalid simulation type entered.");
    }
  }
  spc_destroy(h);
  const long secs =
      (long)std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (sim.type != "symmetry_dynamics")
    std::printf("Time elapsed:  %2ld:%2ld:%2ld\n", secs / 3600, (secs / 60) % 60, secs % 60);
  return 0;
}
