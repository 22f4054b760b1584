// rt_main.cpp -- the reference driver (for_src/main.f90) on top of the C ABI
// of libraytracer_gb300.so, for hosts without a Fortran toolchain.
//
// It follows main.f90:36-101 step by step: set_parameter and set_grid of an
// experiment, calc_grid (one rank), set_initial_conditions, calc_parameter
// (rt_calc_parameter), read_restart, the main loop of set_forcing +
// integrate (rt_integrate) with diagnose (rt_diagnose) every snapshot
// interval, write_restart, and the timing summary (rt_tic / rt_toc).  A
// failing library call prints rt_last_error and stops with exit code 99,
// as halt_stop's MPI_ABORT(99) does (parallel_mpi.f90:223-236).
//
//   rt_main <experiment> [--steps N] [--snap N] [--precision fp64|fp32]
//           [--schedule tma|split] [--restart DIR] [--dump DIR] [--dry]
//
// experiments: packet_small (8x8x16x16^3 Gaussian packet, CFL 0.4) and
// column_1d (the reference's test1D.f90 setup).  --dump writes the inputs
// and the final state as raw binary64 files with a text header (meta.txt);
// --dry builds the inputs and dumps them without touching the GPU.
//
// Build: g++ -O2 -ffp-contract=off -std=c++17 rt_main.cpp -I<repo>/include
//        -L<package> -lraytracer_gb300 -Wl,-rpath,<package>
// (no fused multiply-add: the host grid must equal the reference's bit for
// bit, as the Python host's and the oracle's do).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rt_gb300.h"

namespace {

constexpr int ONX = 2;
const double PI_F = (double)3.14159265358979323846f;   // main_module.f90:10, a default-real literal

double f32(double x) { return (double)(float)x; }         // a default-real literal widened

[[noreturn]] void halt_stop(const std::string& msg) {
  std::fprintf(stderr, " global pe #0 : %s\n global pe #0 aborting\n", msg.c_str());
  std::exit(99);
}

void rt_check(int rc, rt_handle* h, const char* what) {
  if (rc != RT_OK) halt_stop(std::string(what) + " failed: " + rt_last_error(h));
}

// ---- padded arrays (Fortran order, x fastest, onx ghosts per side) --------
struct Dims6 {
  int n[6];
  long long P(int a) const { return n[a] + 2 * ONX; }
  long long len6() const {
    long long l = 1;
    for (int a = 0; a < 6; a++) l *= P(a);
    return l;
  }
  long long len3() const { return P(0) * P(1) * P(2); }
  // padded position of Fortran indices (f = 1 - onx .. n + onx)
  long long i6(const int f[6]) const {
    long long p = 0, s = 1;
    for (int a = 0; a < 6; a++) {
      p += (long long)(f[a] + ONX - 1) * s;
      s *= P(a);
    }
    return p;
  }
  long long i3(int i, int j, int k) const {
    return (i + ONX - 1) + P(0) * ((j + ONX - 1) + P(1) * (long long)(k + ONX - 1));
  }
};

// ---- calc_grid.f90 on one rank: padded t, u, dt, du per axis -------------
struct Axis {
  std::vector<double> t, u, dt, du;
};

// u_centered_grid, calc_grid.f90:300-322 (0-based over the padded range)
void u_centered(const std::vector<double>& dyt, std::vector<double>& dyu, std::vector<double>& yt,
                std::vector<double>& yu) {
  const size_t n = dyt.size();
  yu.assign(n, 0.0);
  yt.assign(n, 0.0);
  dyu.assign(n, 0.0);
  for (size_t i = 1; i < n; i++) yu[i] = yu[i - 1] + dyt[i];
  yt[0] = yu[0] - dyt[0] * 0.5;
  for (size_t i = 1; i < n; i++) yt[i] = 2 * yu[i - 1] - yt[i - 1];
  for (size_t i = 0; i + 1 < n; i++) dyu[i] = yt[i + 1] - yt[i];
  const size_t j = (n - 1 > 1 ? n - 1 : 1) - 1;
  dyu[n - 1] = 2 * dyt[n - 1] - dyu[j];
}

// interior spacings -> padded grids (calc_grid.f90:104-177); fixed[] are
// k_fixed, l_fixed, m_fixed for collapsed spectral axes; checks :260-293
std::vector<Axis> calc_grid(const Dims6& D, const std::vector<double> dint[6], const double fixed[3]) {
  std::vector<Axis> g(6);
  auto P = [](int f) { return (size_t)(f + ONX - 1); };
  for (int a = 0; a < 6; a++) {
    const int na = D.n[a];
    Axis& A = g[a];
    A.dt.assign(na + 2 * ONX, 0.0);
    for (int i = 0; i < na; i++) A.dt[ONX + i] = dint[a][i];
    for (int i = 1; i <= ONX; i++) {
      A.dt[na + i + ONX - 1] = A.dt[na + ONX - 1];
      A.dt[1 - i + ONX - 1] = A.dt[ONX];
    }
    u_centered(A.dt, A.du, A.t, A.u);
    double sh;
    bool set_fixed = false;
    if (a < 2) {
      sh = A.du[P(1)];
    } else if (a == 2) {
      sh = A.u[P(na)];
    } else if (na > 1) {
      sh = A.u[P(na / 2)];
    } else {
      set_fixed = true;
      sh = 0.0;
    }
    if (set_fixed) {
      A.t.assign(A.t.size(), fixed[a - 3]);
      A.u.assign(A.u.size(), fixed[a - 3]);
    } else {
      for (auto& v : A.t) v = v - sh;
      for (auto& v : A.u) v = v - sh;
    }
  }
  const int axes[3] = {2, 5, 4};
  const int his[3] = {D.n[2], D.n[5] / 2, D.n[4] / 2};
  const char* names[3] = {"z", "m", "l"};
  for (int c = 0; c < 3; c++) {
    const Axis& A = g[axes[c]];
    for (int i = 2; i <= his[c]; i++)
      if (A.du[P(i)] - A.du[P(i - 1)] > 1e-12 || A.dt[P(i)] - A.dt[P(i - 1)] > 1e-12)
        halt_stop(std::string(" Error in ") + names[c] + " grid setup, spacings do not decrease monotonically");
  }
  return g;
}

// seeded uniform numbers in [0, 1) (splitmix64), for the packet's noise
struct Rng {
  uint64_t s;
  double next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  }
};

}  // namespace

namespace {

// ---- experiments: set_parameter, set_grid, set_initial_conditions --------
struct Experiment {
  std::string name;
  Dims6 D{};
  std::vector<double> dint[6];
  double f0 = 1e-4, sign = 1.0, dt = 0.0, cfl = 0.0;   // cfl > 0: dt = cfl / (max cell rate)
  bool upper = true, lower = true;
  double fixed[3] = {0.0, 0.0, 0.0};
  int steps = 10, snap = 5;
};

// the padded arrays of the module state the experiment fills
struct State {
  std::vector<double> N2, U, V, E;
};

// 8x8x16 x 16^3, f = 1e-4, N(z) = 5e-3 exp(z/1000 m) over 4000 m, no mean
// flow, Gaussian packet (widths 2 cells, amplitude 1e-3) at mid x, y, z and
// (k0,l0,m0) = (1e-3, 0, 1e-2) plus uniform noise of 1e-8, CFL 0.4
Experiment packet_small() {
  Experiment e;
  e.name = "packet_small";
  const int n[6] = {8, 8, 16, 16, 16, 16};
  for (int a = 0; a < 6; a++) e.D.n[a] = n[a];
  const double L[3] = {40e3, 40e3, 4000.0}, kmax = 2e-3, lmax = 2e-3, mmax = 5e-2;
  for (int a = 0; a < 3; a++) e.dint[a].assign(n[a], L[a] / n[a]);
  e.dint[3].assign(n[3], 2 * kmax / n[3]);
  e.dint[4].assign(n[4], 2 * lmax / n[4]);
  e.dint[5].assign(n[5], 2 * mmax / n[5]);
  e.f0 = 1e-4;
  e.cfl = 0.4;
  e.steps = 200;
  e.snap = 50;
  return e;
}

void packet_small_state(const Experiment& e, const std::vector<Axis>& g, State& s, uint64_t seed) {
  const Dims6& D = e.D;
  for (long long k = 0; k < D.P(2); k++)
    for (long long j = 0; j < D.P(1); j++)
      for (long long i = 0; i < D.P(0); i++) {
        const long long q = i + D.P(0) * (j + D.P(1) * k);
        const double N = 5e-3 * std::exp(g[2].t[k] / 1000.0);
        s.N2[q] = N * N;
        s.U[q] = 0.0;
        s.V[q] = 0.0;
      }
  const double c[6] = {40e3 / 2, 40e3 / 2, -4000.0 / 2, 1e-3, 0.0, 1e-2};
  std::vector<double> g1[6];
  for (int a = 0; a < 6; a++) {
    g1[a].assign(D.n[a], 1.0);
    if (D.n[a] == 1) continue;
    for (int i = 0; i < D.n[a]; i++) {
      const double r = (g[a].t[ONX + i] - c[a]) / (2.0 * g[a].dt[ONX + i]);
      g1[a][i] = std::exp(-0.5 * (r * r));
    }
  }
  Rng rng{seed};
  int f[6];
  for (f[5] = 1; f[5] <= D.n[5]; f[5]++)
    for (f[4] = 1; f[4] <= D.n[4]; f[4]++)
      for (f[3] = 1; f[3] <= D.n[3]; f[3]++)
        for (f[2] = 1; f[2] <= D.n[2]; f[2]++)
          for (f[1] = 1; f[1] <= D.n[1]; f[1]++)
            for (f[0] = 1; f[0] <= D.n[0]; f[0]++) {
              double v = 1e-3;
              for (int a = 0; a < 6; a++) v = v * g1[a][f[a] - 1];
              s.E[D.i6(f)] = v + 1e-8 * rng.next();
            }
}

// test1D.f90:3-78 with fac = 1: nz = 20, nm = 60, the other axes collapsed,
// k_fixed = 1e-3, dt = 5 s
Experiment column_1d() {
  Experiment e;
  e.name = "column_1d";
  const int n[6] = {1, 1, 20, 1, 1, 60};
  for (int a = 0; a < 6; a++) e.D.n[a] = n[a];
  const double Lx = f32(2000.0), Ly = f32(2000.0), Lz = f32(2000.0);
  e.dint[0].assign(1, Lx / 1);
  e.dint[1].assign(1, Ly / 1);
  e.dint[2].assign(n[2], Lz / n[2]);
  e.dint[3].assign(1, PI_F / Lx);
  e.dint[4].assign(1, PI_F / Ly);
  e.dint[5].assign(n[5], PI_F / Lz / 4.0);
  e.f0 = f32(1e-4);
  e.dt = 5.0;
  e.fixed[0] = f32(1e-3);
  e.steps = 20;
  e.snap = 10;
  return e;
}

void column_1d_state(const Experiment& e, const std::vector<Axis>& g, State& s) {
  const Dims6& D = e.D;
  const double Lz = f32(2000.0);
  for (long long k = 0; k < D.P(2); k++)
    for (long long j = 0; j < D.P(1); j++)
      for (long long i = 0; i < D.P(0); i++) {
        const long long q = i + D.P(0) * (j + D.P(1) * k);
        s.U[q] = 0.50 * (1 + std::tanh((g[2].t[k] + 750) / 150)) / 2.0;
        const double N = 30 * e.f0;
        s.N2[q] = N * N;
        s.V[q] = 0.0;
      }
  const int nz = D.n[2], nm = D.n[5];
  const double dmt1 = g[5].dt[ONX];
  for (int mm = 1; mm <= nm; mm++) {
    const double mt = g[5].t[mm + 1];
    if (!(mt < 0)) continue;
    for (int kk = 1; kk <= nz; kk++) {
      const int f[6] = {1, 1, kk, 1, 1, mm};
      s.E[D.i6(f)] = 1.0 + std::sin(mt * 2 * PI_F / (nm * dmt1 / 2 / 6.0)) *
                               std::sin(g[2].t[kk + 1] * 2 * PI_F / (Lz / 6.0));
    }
  }
}

}  // namespace

namespace {

// ---- restart files (restart.f90:2-93) in gfortran's sequential layout ----
// 4-byte length markers before and after each record; records longer than
// 2^31-9 bytes split into subrecords (leading marker negated while more
// follow, trailing marker negated after the first)
constexpr long long MAX_SUB = 2147483639LL;

void write_record(FILE* f, const void* data, long long n) {
  const char* p = static_cast<const char*>(data);
  long long pos = 0;
  do {
    const long long size = n - pos < MAX_SUB ? n - pos : MAX_SUB;
    const int32_t lead = (int32_t)(pos + size < n ? -size : size);
    const int32_t trail = (int32_t)(pos > 0 ? -size : size);
    std::fwrite(&lead, 4, 1, f);
    if (size) std::fwrite(p + pos, 1, (size_t)size, f);
    std::fwrite(&trail, 4, 1, f);
    pos += size;
  } while (pos < n);
}

bool read_record(FILE* f, std::vector<char>& out) {
  out.clear();
  bool first = true;
  for (;;) {
    int32_t lead = 0, trail = 0;
    if (std::fread(&lead, 4, 1, f) != 1) return false;
    const long long size = lead < 0 ? -(long long)lead : lead;
    const size_t at = out.size();
    out.resize(at + (size_t)size);
    if (size && std::fread(out.data() + at, 1, (size_t)size, f) != (size_t)size) return false;
    if (std::fread(&trail, 4, 1, f) != 1) return false;
    if ((trail < 0 ? -(long long)trail : trail) != size || (trail < 0) == first) return false;
    first = false;
    if (lead >= 0) return true;
  }
}

std::string restart_name(const std::string& dir) { return dir + "/restart_pe=000000000.dta"; }

void write_restart(const std::string& dir, const Dims6& D, int itt, const std::vector<double>& E,
                   const std::vector<double>& dE, const std::vector<double>& mf) {
  FILE* f = std::fopen(restart_name(dir).c_str(), "wb");
  if (!f) {
    std::printf(" Warning: error writing restart file\n");   // restart.f90:30-31
    return;
  }
  const int32_t r1[7] = {D.n[0], D.n[1], D.n[2], D.n[3], D.n[4], D.n[5], itt};
  const int32_t r2[6] = {1, D.n[0], 1, D.n[1], 1, D.n[2]};
  const int32_t r3[6] = {1, D.n[3], 1, D.n[4], 1, D.n[5]};
  write_record(f, r1, sizeof(r1));
  write_record(f, r2, sizeof(r2));
  write_record(f, r3, sizeof(r3));
  std::vector<double> all;
  all.reserve(3 * E.size());
  all.insert(all.end(), E.begin(), E.end());
  all.insert(all.end(), dE.begin(), dE.end());
  all.insert(all.end(), mf.begin(), mf.end());
  write_record(f, all.data(), (long long)(all.size() * sizeof(double)));
  std::fclose(f);
  FILE* r = std::fopen((dir + "/ritt").c_str(), "w");
  if (r) {
    std::fprintf(r, "%12d\n", itt);
    std::fclose(r);
  }
  std::printf(" writing to restart file %s\n at itt = %12d\n", restart_name(dir).c_str(), itt);
}

// read_restart: false when there is no file; a mismatch stops the run
bool read_restart(const std::string& dir, const Dims6& D, int& itt, std::vector<double>& E) {
  FILE* f = std::fopen(restart_name(dir).c_str(), "rb");
  if (!f) {
    std::printf(" found no restart file %s\n", restart_name(dir).c_str());
    return false;
  }
  std::vector<char> r1, r2, r3, r4;
  if (!read_record(f, r1) || !read_record(f, r2) || !read_record(f, r3) || !read_record(f, r4) ||
      r1.size() != 28 || r2.size() != 24 || r3.size() != 24) {
    std::fclose(f);
    halt_stop(" Warning: error reading restart file");
  }
  std::fclose(f);
  int32_t h1[7], h2[6], h3[6];
  std::memcpy(h1, r1.data(), 28);
  std::memcpy(h2, r2.data(), 24);
  std::memcpy(h3, r3.data(), 24);
  for (int a = 0; a < 6; a++)
    if (h1[a] != D.n[a]) halt_stop(" read from restart dimensions do not match dimensions");
  const int32_t want[12] = {1, D.n[0], 1, D.n[1], 1, D.n[2], 1, D.n[3], 1, D.n[4], 1, D.n[5]};
  for (int k = 0; k < 12; k++)
    if ((k < 6 ? h2[k] : h3[k - 6]) != want[k]) halt_stop(" read from restart PE boundaries do not match");
  if (r4.size() != 3 * E.size() * sizeof(double)) halt_stop(" Warning: error reading restart file");
  std::memcpy(E.data(), r4.data(), E.size() * sizeof(double));
  itt = h1[6];
  std::printf(" reading restart file %s\n  itt = %d\n", restart_name(dir).c_str(), itt);
  return true;
}

// ---- dump for the tests: raw binary64 arrays and a key = value header ----
void dump_array(const std::string& dir, const char* name, const std::vector<double>& v) {
  FILE* f = std::fopen((dir + "/" + name + ".bin").c_str(), "wb");
  if (!f) halt_stop(std::string("cannot write ") + dir + "/" + name + ".bin");
  std::fwrite(v.data(), sizeof(double), v.size(), f);
  std::fclose(f);
}

void dump_inputs(const std::string& dir, const std::vector<Axis>& g, const State& s, const char* ename) {
  const char* ax = "xyzklm";
  for (int a = 0; a < 6; a++) {
    const std::string b = std::string("grid_") + ax[a];
    dump_array(dir, (b + "_t").c_str(), g[a].t);
    dump_array(dir, (b + "_u").c_str(), g[a].u);
    dump_array(dir, (b + "_dt").c_str(), g[a].dt);
    dump_array(dir, (b + "_du").c_str(), g[a].du);
  }
  dump_array(dir, "Nsqr", s.N2);
  dump_array(dir, "U", s.U);
  dump_array(dir, "V", s.V);
  dump_array(dir, ename, s.E);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2 || !std::strcmp(argv[1], "--help")) {
    std::printf("usage: rt_main packet_small|column_1d [--steps N] [--snap N] [--precision fp64|fp32]\n"
                "       [--schedule tma|split] [--restart DIR] [--dump DIR] [--dry]\n");
    return argc < 2 ? 2 : 0;
  }
  const std::string which = argv[1];
  Experiment e;
  if (which == "packet_small") e = packet_small();
  else if (which == "column_1d") e = column_1d();
  else halt_stop("unknown experiment " + which);
  int precision = RT_FP64;
  bool dry = false, split = false;
  std::string restart_dir, dump_dir;
  for (int i = 2; i < argc; i++) {
    const std::string a = argv[i];
    const bool more = i + 1 < argc;
    if (a == "--steps" && more) e.steps = std::atoi(argv[++i]);
    else if (a == "--snap" && more) e.snap = std::atoi(argv[++i]);
    else if (a == "--precision" && more) precision = std::string(argv[++i]) == "fp32" ? RT_FP32 : RT_FP64;
    else if (a == "--schedule" && more) split = std::string(argv[++i]) == "split";
    else if (a == "--restart" && more) restart_dir = argv[++i];
    else if (a == "--dump" && more) dump_dir = argv[++i];
    else if (a == "--dry") dry = true;
    else halt_stop("unknown argument " + a);
  }
  if (e.snap < 1) e.snap = 1;
  const Dims6& D = e.D;

  // set_grid, calc_grid (main.f90:42-43)
  const std::vector<Axis> g = calc_grid(D, e.dint, e.fixed);
  // set_initial_conditions (main.f90:46)
  State s;
  s.N2.assign(D.len3(), 0.0);
  s.U.assign(D.len3(), 0.0);
  s.V.assign(D.len3(), 0.0);
  s.E.assign(D.len6(), 0.0);
  if (which == "packet_small") packet_small_state(e, g, s, 1234);
  else column_1d_state(e, g, s);
  if (!dump_dir.empty()) dump_inputs(dump_dir, g, s, "E0");
  if (dry) {
    if (!dump_dir.empty()) {
      FILE* m = std::fopen((dump_dir + "/meta.txt").c_str(), "w");
      std::fprintf(m, "name = %s\nn = %d %d %d %d %d %d\ndry = 1\n", e.name.c_str(), D.n[0], D.n[1], D.n[2],
                   D.n[3], D.n[4], D.n[5]);
      std::fclose(m);
    }
    return 0;
  }

  // allocate_main_module + calc_parameter (main.f90:39, :47) on the device
  const rt_dims dims{D.n[0], D.n[1], D.n[2], D.n[3], D.n[4], D.n[5], ONX};
  const rt_params par{e.dt > 0 ? e.dt : 1.0, e.f0, e.sign, e.upper ? 1 : 0, e.lower ? 1 : 0, precision};
  rt_handle* h = nullptr;
  rt_check(rt_create(&dims, &par, &h), nullptr, "rt_create");
  rt_check(rt_set_grid(h, g[0].dt.data(), g[1].dt.data(), g[2].dt.data(), g[3].dt.data(), g[4].dt.data(),
                       g[5].dt.data(), g[3].t.data(), g[4].t.data(), g[5].t.data()), h, "rt_set_grid");
  rt_check(rt_set_background(h, s.N2.data(), s.U.data(), s.V.data()), h, "rt_set_background");
  rt_check(rt_calc_parameter(h), h, "rt_calc_parameter");
  double dt = e.dt;
  if (e.cfl > 0) {   // dt from a CFL number through the largest cell rate
    double rate = 0.0;
    rt_check(rt_max_rate(h, &rate), h, "rt_max_rate");
    dt = e.cfl / rate;
    rt_check(rt_set_dt(h, dt), h, "rt_set_dt");
  }
  if (split && precision == RT_FP64) rt_check(rt_set_tuning(h, 15, 8, 256), h, "rt_set_tuning");

  // read_restart (main.f90:49)
  int itt = 0;
  if (!restart_dir.empty()) read_restart(restart_dir, D, itt, s.E);
  rt_check(rt_set_state(h, s.E.data()), h, "rt_set_state");
  const int enditt = itt + e.steps;
  std::printf("\n setup integration for %d steps of %.6g s\n from time step %10d to %10d\n"
              " snapshot interval is any %8d time steps\n\n", e.steps, dt, itt, enditt, e.snap);

  // main loop (main.f90:64-79)
  rt_budget b{};
  bool have_budget = false;
  std::vector<double> E_int(D.len3()), M_int(D.len3()), diss[6];
  for (auto& d : diss) d.assign(D.len3(), 0.0);
  while (itt < enditt) {
    rt_check(rt_tic(h, "main loop"), h, "rt_tic");
    rt_check(rt_tic(h, "integrate"), h, "rt_tic");
    rt_check(rt_integrate(h, 1), h, "rt_integrate");   // set_forcing + integrate
    rt_check(rt_toc(h, "integrate"), h, "rt_toc");
    if (itt % e.snap == 0) {   // diagnose (main.f90:74, diagnose.f90:295-329)
      rt_check(rt_tic(h, "diag"), h, "rt_tic");
      rt_check(rt_diagnose(h, &b, E_int.data(), M_int.data(), diss[0].data(), diss[1].data(), diss[2].data(),
                           diss[3].data(), diss[4].data(), diss[5].data()), h, "rt_diagnose");
      rt_check(rt_toc(h, "diag"), h, "rt_toc");
      have_budget = true;
      std::printf(" writing snapshot at %15.2f s\n", itt * dt);
      std::printf(" max CFL in x,y,z,k,l,m-dir = %8.2f%8.2f%8.2f%8.2f%8.2f%8.2f\n", b.cfl_x, b.cfl_y, b.cfl_z,
                  b.cfl_k, b.cfl_l, b.cfl_m);
      std::printf(" mean flow interaction scale %8.2f\n", b.mfl_max > 0 ? dt / b.mfl_max : 0.0);
      std::printf(" total dE          : %14.6e\n dE by mean-flow   : %14.6e\n", b.eint, b.mflint);
      std::printf(" by flux at min/max x  : %14.6e%14.6e\n", b.bfl_xs, b.bfl_xe);
      std::printf(" by flux at min/max y  : %14.6e%14.6e\n", b.bfl_ys, b.bfl_ye);
      std::printf(" by flux at min/max k  : %14.6e%14.6e\n", b.bfl_ks, b.bfl_ke);
      std::printf(" by flux at min/max l  : %14.6e%14.6e\n", b.bfl_ls, b.bfl_le);
      std::printf(" by flux at min/max m  : %14.6e%14.6e\n", b.bfl_ms, b.bfl_me);
      std::printf(" residual : %14.6e\n", b.residual);
    }
    itt += 1;
    rt_check(rt_toc(h, "main loop"), h, "rt_toc");
  }

  // write_restart (main.f90:81)
  rt_check(rt_get_state(h, s.E.data()), h, "rt_get_state");
  if (!restart_dir.empty()) {
    std::vector<double> dE(D.len6(), 0.0), mf(D.len6(), 0.0);
    if (e.steps > 0) rt_check(rt_get_tendency(h, dE.data(), mf.data()), h, "rt_get_tendency");
    write_restart(restart_dir, D, itt, s.E, dE, mf);
  }

  // timing summary (main.f90:86-101)
  const char* phases[3] = {"main loop", "integrate", "diag"};
  std::printf("\nTiming summary for PE #   0\n");
  for (const char* p : phases) {
    double secs = 0.0;
    long long calls = 0;
    rt_check(rt_timing_secs(h, p, &secs, &calls), h, "rt_timing_secs");
    std::printf(" %-24s = %12.4f s (%lld calls, device time)\n", p, secs, calls);
  }

  if (!dump_dir.empty()) {
    dump_array(dump_dir, "E", s.E);
    FILE* m = std::fopen((dump_dir + "/meta.txt").c_str(), "w");
    std::fprintf(m, "name = %s\nn = %d %d %d %d %d %d\ndt = %.17g\nf0 = %.17g\nsign = %.17g\n", e.name.c_str(),
                 D.n[0], D.n[1], D.n[2], D.n[3], D.n[4], D.n[5], dt, e.f0, e.sign);
    std::fprintf(m, "upper = %d\nlower = %d\nfixed = %.17g %.17g %.17g\nsteps = %d\nitt = %d\n", e.upper ? 1 : 0,
                 e.lower ? 1 : 0, e.fixed[0], e.fixed[1], e.fixed[2], e.steps, itt);
    std::fprintf(m, "precision = %s\nschedule = %s\n", precision == RT_FP64 ? "fp64" : "fp32",
                 split ? "split" : "tma");
    if (have_budget)
      std::fprintf(m, "eint = %.17g\nmflint = %.17g\nresidual = %.17g\n", b.eint, b.mflint, b.residual);
    std::fclose(m);
  }
  rt_check(rt_destroy(h), nullptr, "rt_destroy");
  return 0;
}
