// euler3d_gb300: command-line driver with the reference euler3d's interface
// (config.h:107-388, euler3d.cpp:69-826) on top of the C ABI.
//
//   euler3d_gb300 -i input.dat [-d dir] [-g cycles] [-o prefix] [-v] [-l] [-b]
//                 [-I interval] [-n] [-c config] [--output-variables]
//                 [--output-fluxes] [--output-step-factors]
//                 [--mach M] [--aoa DEG] [--precision fp64|mixed|dw]
//                 [--increment auto|atomic|gather|fused|coloured] [--accumulation fp64|pair32]
//
// Two ways to run the V-cycle:
//   * default: the device-resident solver (mgcfd_solver_*: renumbered, fused
//     kernels, one CUDA graph per V-cycle);
//   * --per-loop: the reference's main loop itself (euler3d.cpp:413-641) with
//     every op_par_loop replaced by the mgcfd_op_* entry point that binds it,
//     on device dats in OP2's layout and the mesh file's numbering -- what an
//     OP2 application bound to this library runs.  Like the reference it reads
//     its OP_MIN / OP_INC globals back after each loop that produces one, and
//     stops where the reference stops (min_dt < 0, NaN/Inf at level 0).
//
// Differences from the reference, all forced by running on one GPU:
//   * -m/-r (partitioner) and -p (PAPI) are accepted and ignored;
//   * -n selects reverse Cuthill-McKee renumbering instead of Scotch (with
//     --per-loop it has no effect: the loops' plans order the nodes);
//   * Mach and angle of attack are run-time options (defaults 1.2 and 0.0,
//     the values const.h:32-33 fixes at compile time).
#include <cuda_runtime.h>
#include <getopt.h>
#include <sys/time.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "mgcfd_gb300.h"

namespace {

struct Config {
  std::string input_file, input_dir, prefix;
  bool legacy = false, validate = false, mem_bound = false, renumber = false;
  bool out_variables = false, out_fluxes = false, out_step_factors = false;
  int cycles = 25;           // config.h:150
  int flow_interval = 0;
  double mach = 1.2, aoa = 0.0;
  int precision = MGCFD_PRECISION_FP64, increment = MGCFD_INCREMENT_AUTO, accumulation = MGCFD_ACCUM_FP64;
  bool per_loop = false;
};

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

bool yes(const std::string& v) { return v == "Y"; }

// config.h:167-265 keys.
void set_param(Config& c, const std::string& key, const std::string& value) {
  if (key == "input_file") c.input_file = value;
  else if (key == "input_file_directory") c.input_dir = value;
  else if (key == "output_file_prefix") c.prefix = value;
  else if (key == "validate_result") c.validate = c.validate || yes(value);
  else if (key == "measure_mem_bound") c.mem_bound = c.mem_bound || yes(value);
  else if (key == "cycles") c.cycles = std::atoi(value.c_str());
  else if (key == "renumber") c.renumber = c.renumber || yes(value);
  else if (key == "output_step_factors") c.out_step_factors = c.out_step_factors || yes(value);
  else if (key == "output_fluxes") c.out_fluxes = c.out_fluxes || yes(value);
  else if (key == "output_variables") c.out_variables = c.out_variables || yes(value);
  else if (key == "output_flow_interval") c.flow_interval = std::atoi(value.c_str());
  else if (key == "mach") c.mach = std::atof(value.c_str());
  else if (key == "aoa") c.aoa = std::atof(value.c_str());
  else if (key == "partitioner" || key == "partitioner-method" || key == "papi-config-file" || key == "config-filepath") {}
  else std::printf("WARNING: Unknown key '%s' encountered during parsing of config file.\n", key.c_str());
}

bool read_config(Config& c, const char* path) {
  if (access(path, F_OK) == -1) {
    std::fprintf(stderr, "ERROR: \"%s\" does not exist.\n", path);
    return false;
  }
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    if (!line.empty() && line[0] == '#') continue;
    size_t eq = line.find('=');
    if (eq == std::string::npos || eq + 1 >= line.size()) continue;
    set_param(c, trim(line.substr(0, eq)), trim(line.substr(eq + 1)));
  }
  return true;
}

void usage() {
  std::fprintf(stderr,
               "MG-CFD (GB300) instructions\n\n"
               "Usage: euler3d_gb300 [OPTIONS] -i input.dat\n"
               "       euler3d_gb300 [OPTIONS] -c conf.conf\n\n"
               "-i, --input-file=FILEPATH        multigrid input grid (.dat file)\n"
               "-c, --config-filepath=FILEPATH   config file\n"
               "-d, --input-directory=DIRPATH    directory path to input files\n"
               "-o, --output-file-prefix=STRING  string to prepend to output filenames\n"
               "-g, --num-cycles=INT             number of multigrid V-cycles to perform\n"
               "-l, --legacy-mode                read the legacy dataset names\n"
               "-n, --renumber                   renumber nodes by reverse Cuthill-McKee\n"
               "-b, --measure-mem-bound          also run unstructured_stream each RK stage\n"
               "-v, --validate-result            check final state against pre-calculated solution\n"
               "-I, --output-flow-interval=INT   cycles between writes of the level-0 flow\n"
               "--output-variables | --output-fluxes | --output-step-factors\n"
               "--mach=FLOAT (1.2)  --aoa=DEGREES (0.0)  --precision=fp64|mixed|dw\n"
               "--increment=auto|atomic|gather|fused|coloured  --accumulation=fp64|pair32\n"
               "--per-loop   run the reference's loop sequence through the per-loop entry points\n"
               "             (with --precision dw, the edge-flux calls in the DW form)\n"
               "-m, -r, -p are accepted for compatibility and ignored (one GPU, no PAPI).\n");
}

bool parse(int argc, char** argv, Config& c) {
  int out_vars = 0, out_flux = 0, out_sf = 0;
  static struct option opts[] = {
      {"help", no_argument, nullptr, 'h'},
      {"config-filepath", required_argument, nullptr, 'c'},
      {"legacy-mode", no_argument, nullptr, 'l'},
      {"input-file", required_argument, nullptr, 'i'},
      {"input-directory", required_argument, nullptr, 'd'},
      {"papi-config-file", required_argument, nullptr, 'p'},
      {"output-file-prefix", required_argument, nullptr, 'o'},
      {"num-cycles", required_argument, nullptr, 'g'},
      {"partitioner", required_argument, nullptr, 'm'},
      {"partitioner-method", required_argument, nullptr, 'r'},
      {"renumber", no_argument, nullptr, 'n'},
      {"validate", no_argument, nullptr, 'v'},
      {"measure-mem-bound", no_argument, nullptr, 'b'},
      {"output-variables", no_argument, &out_vars, 1},
      {"output-fluxes", no_argument, &out_flux, 1},
      {"output-step-factors", no_argument, &out_sf, 1},
      {"output-flow-interval", required_argument, nullptr, 'I'},
      {"mach", required_argument, nullptr, 1001},
      {"aoa", required_argument, nullptr, 1002},
      {"precision", required_argument, nullptr, 1003},
      {"increment", required_argument, nullptr, 1004},
      {"accumulation", required_argument, nullptr, 1005},
      {"per-loop", no_argument, nullptr, 1006},
      {nullptr, 0, nullptr, 0}};
  int o;
  while ((o = getopt_long(argc, argv, "hc:li:d:p:o:g:m:r:vbnI:", opts, nullptr)) != -1) {
    switch (o) {
      case 'h': usage(); return false;
      case 'c': if (!read_config(c, optarg)) std::exit(-1); break;
      case 'l': c.legacy = true; break;
      case 'i': c.input_file = optarg; break;
      case 'd': c.input_dir = optarg; break;
      case 'o': c.prefix = optarg; break;
      case 'g': c.cycles = std::atoi(optarg); break;
      case 'n': c.renumber = true; break;
      case 'v': c.validate = true; break;
      case 'b': c.mem_bound = true; break;
      case 'I': c.flow_interval = std::atoi(optarg); break;
      case 'm': case 'r': case 'p': break;
      case 1001: c.mach = std::atof(optarg); break;
      case 1002: c.aoa = std::atof(optarg); break;
      case 1003:
        c.precision = std::strcmp(optarg, "mixed") == 0 ? MGCFD_PRECISION_MIXED
                      : std::strcmp(optarg, "dw") == 0  ? MGCFD_PRECISION_DW
                                                        : MGCFD_PRECISION_FP64;
        break;
      case 1004:
        c.increment = std::strcmp(optarg, "gather") == 0   ? MGCFD_INCREMENT_GATHER
                      : std::strcmp(optarg, "atomic") == 0 ? MGCFD_INCREMENT_ATOMIC
                      : std::strcmp(optarg, "fused") == 0  ? MGCFD_INCREMENT_FUSED
                      : std::strcmp(optarg, "coloured") == 0 ? MGCFD_INCREMENT_COLOURED
                                                           : MGCFD_INCREMENT_AUTO;
        break;
      case 1005:
        c.accumulation = std::strcmp(optarg, "pair32") == 0 ? MGCFD_ACCUM_PAIR32 : MGCFD_ACCUM_FP64;
        break;
      case 1006: c.per_loop = true; break;
      case 0: break;
      default: std::printf("Unknown command line parameter '%c'\n", o);
    }
  }
  c.out_variables = c.out_variables || out_vars;
  c.out_fluxes = c.out_fluxes || out_flux;
  c.out_step_factors = c.out_step_factors || out_sf;
  return true;
}

double wall() {
  struct timeval t;
  gettimeofday(&t, nullptr);
  return (double)t.tv_sec + 1e-6 * (double)t.tv_usec;
}

int fail(int st) {
  std::printf("%s: %s\n", mgcfd_status_string(st), mgcfd_last_error());
  return 1;
}

std::string dir_join(const std::string& dir, const std::string& name) { return dir.empty() ? name : dir + "/" + name; }

// The run's results in the mesh file's numbering, per level.
struct Results {
  std::vector<std::vector<double>> vars, step_factors, fluxes;
};

// --per-loop: device dats of one level in OP2 layout ([set size][dim]).
struct LoopLevel {
  int32_t n = 0, ne = 0, nb = 0;
  bool legacy = false;
  double *coords = nullptr, *ewt = nullptr, *bwt = nullptr, *vol = nullptr, *var = nullptr, *old = nullptr;
  double *flux = nullptr, *res = nullptr, *sf = nullptr, *dummy = nullptr;
  int32_t *e2n = nullptr, *b2n = nullptr, *grp = nullptr, *n2mg = nullptr, *scratch = nullptr;
};

// Every device buffer of a --per-loop run, freed together (the role of
// OP2's own allocator for dats and maps).
class DeviceArena {
 public:
  ~DeviceArena() {
    for (void* q : ptrs_) cudaFree(q);
  }
  template <class T>
  bool alloc(T** out, size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return false;
    ptrs_.push_back(q);
    *out = static_cast<T*>(q);
    return true;
  }
  template <class T>
  bool upload(T** out, const T* src, size_t n) {
    if (!alloc(out, n)) return false;
    return n == 0 || cudaMemcpy(*out, src, n * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
  }
  template <class T>
  static bool download(std::vector<double>* out, const T* src, size_t n) {
    out->resize(n);
    return cudaMemcpy(out->data(), src, n * sizeof(T), cudaMemcpyDeviceToHost) == cudaSuccess;
  }

 private:
  std::vector<void*> ptrs_;
};

#define OPCALL(call)                    \
  do {                                  \
    const int st_ = (call);             \
    if (st_) return fail(st_);          \
  } while (0)

// The reference's main loop (euler3d.cpp:413-641), each op_par_loop one
// mgcfd_op_* call.  Returns 0, or 1 where the reference exits with an error.
int run_per_loop(const Config& c, const std::vector<mgcfd_level_view>& lv, Results* out) {
  const int levels = (int)lv.size();
  DeviceArena arena;
  std::vector<LoopLevel> L((size_t)levels);
  // The plans built for these maps go before the maps' memory does, on every
  // way out (declared after the arena, so destroyed before it).
  struct PlanRelease {
    const std::vector<LoopLevel>& L;
    ~PlanRelease() {
      for (const auto& d : L) {
        if (d.e2n) mgcfd_op_plan_release(d.e2n);
        if (d.n2mg) mgcfd_op_plan_release(d.n2mg);
      }
    }
  } release_plans{L};
  for (int l = 0; l < levels; l++) {
    const mgcfd_level_view& v = lv[(size_t)l];
    LoopLevel& d = L[(size_t)l];
    d.n = v.nnodes; d.ne = v.nedges; d.nb = v.nbnd;
    d.legacy = v.volumes != nullptr;
    const size_t n = (size_t)v.nnodes, ne = (size_t)v.nedges, nb = (size_t)v.nbnd;
    bool ok = arena.upload(&d.coords, v.coords, 3 * n) && arena.upload(&d.e2n, v.edge_to_nodes, 2 * ne) &&
              arena.upload(&d.b2n, v.bnd_to_node, nb) && arena.upload(&d.grp, v.bnd_group, nb) &&
              arena.upload(&d.ewt, v.edge_weights, 3 * ne) && arena.upload(&d.bwt, v.bnd_weights, 3 * nb) &&
              arena.alloc(&d.var, 5 * n) && arena.alloc(&d.old, 5 * n) && arena.alloc(&d.flux, 5 * n) &&
              arena.alloc(&d.res, 5 * n) && arena.alloc(&d.sf, n) && arena.alloc(&d.scratch, n) &&
              (d.legacy ? arena.upload(&d.vol, v.volumes, n) : arena.alloc(&d.vol, n)) &&
              (!v.node_to_mg || arena.upload(&d.n2mg, v.node_to_mg, n)) && (!c.mem_bound || arena.alloc(&d.dummy, 5 * n));
    if (!ok) {
      std::printf("Device allocation or upload failed: %s\n", cudaGetErrorString(cudaGetLastError()));
      return 1;
    }
  }
  double* d_min_dt = nullptr;
  double* d_rms = nullptr;
  int32_t* d_bad = nullptr;
  if (!arena.alloc(&d_min_dt, 1) || !arena.alloc(&d_rms, 1) || !arena.alloc(&d_bad, 1)) return fail(MGCFD_ERR_NOMEM);
  mgcfd_freestream ff;
  OPCALL(mgcfd_freestream_init(c.mach, c.aoa, &ff));

  // Initialise variables and geometry (euler3d.cpp:413-441).
  for (auto& d : L) {
    OPCALL(mgcfd_op_initialize_variables(d.n, &ff, d.var, nullptr));
    OPCALL(mgcfd_op_zero(d.n, 5, d.flux, nullptr));
    if (c.mem_bound) OPCALL(mgcfd_op_zero(d.n, 5, d.dummy, nullptr));
    if (!d.legacy) {
      OPCALL(mgcfd_op_zero(d.n, 1, d.vol, nullptr));
      OPCALL(mgcfd_op_calculate_cell_volumes(d.ne, d.n, d.e2n, d.coords, d.ewt, d.vol, nullptr));
    }
  }
  for (auto& d : L) {
    OPCALL(mgcfd_op_dampen_ewt(d.ne, d.ewt, nullptr));
    OPCALL(mgcfd_op_dampen_ewt(d.nb, d.bwt, nullptr));
  }

  std::printf("-----------------------------------------------------\nCompute beginning\n");
  const double t0 = wall();
  int level = 0, i = 0;
  bool up = true;
  while (i < c.cycles) {
    LoopLevel& d = L[(size_t)level];
    if (level == 0) std::printf("Performing MG cycle %d / %d\n", i + 1, c.cycles);
    OPCALL(mgcfd_op_copy_double(d.n, d.var, d.old, nullptr));
    OPCALL(mgcfd_op_calculate_dt(d.n, d.var, d.vol, d.sf, nullptr));
    OPCALL(mgcfd_op_get_min_dt(d.n, d.sf, d_min_dt, nullptr));
    double min_dt = 0.0;  // OP_MIN global, read back as OP2 returns it
    if (cudaMemcpy(&min_dt, d_min_dt, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return fail(MGCFD_ERR_CUDA);
    if (min_dt < 0.0) {
      std::printf("Fatal error during 'step factor' calculation, min_dt = %.5e\n", min_dt);
      return 1;
    }
    OPCALL(mgcfd_op_compute_step_factor(d.n, d.var, d.vol, d_min_dt, d.sf, nullptr));
    for (int rk = 0; rk < 3; rk++) {
      OPCALL(mgcfd_op_compute_flux_edge(d.ne, d.n, d.e2n, d.var, d.ewt, ff.smoothing_coefficient, d.flux, nullptr));
      OPCALL(mgcfd_op_compute_bnd_node_flux(d.nb, d.n, d.b2n, d.grp, d.bwt, d.var, &ff, d.flux, nullptr));
      OPCALL(mgcfd_op_time_step(d.n, rk, d.sf, d.flux, d.old, d.var, nullptr));
      if (c.mem_bound) OPCALL(mgcfd_op_unstructured_stream(d.ne, d.n, d.e2n, d.var, d.ewt, d.dummy, nullptr));
    }
    OPCALL(mgcfd_op_residual(d.n, d.old, d.var, d.res, nullptr));
    if (level == 0) {  // euler3d.cpp:533-548
      if (cudaMemset(d_rms, 0, sizeof(double)) != cudaSuccess || cudaMemset(d_bad, 0, sizeof(int32_t)) != cudaSuccess)
        return fail(MGCFD_ERR_CUDA);
      OPCALL(mgcfd_op_calc_rms(d.n, d.res, d_rms, nullptr));
      OPCALL(mgcfd_op_count_bad_vals(d.n, d.var, d_bad, nullptr));
      int32_t bad = 0;
      if (cudaMemcpy(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost) != cudaSuccess) return fail(MGCFD_ERR_CUDA);
      if (bad > 0) {
        std::printf("Bad variable values detected, aborting\n");
        return 1;
      }
      if (c.flow_interval > 0 && ((i + 1) % c.flow_interval) == 0) {  // euler3d.cpp:552-571
        std::vector<double> v;
        if (!DeviceArena::download(&v, d.var, 5 * (size_t)d.n)) return fail(MGCFD_ERR_CUDA);
        const std::string f = c.prefix + "variables.L0.cycle=" + std::to_string(i + 1) + ".h5";
        OPCALL(mgcfd_h5_write_f64(f.c_str(), "p_variables", v.data(), d.n, 5));
      }
    }
    if (levels <= 1) {
      i++;
    } else if (up) {  // euler3d.cpp:579-597
      level++;
      LoopLevel& f = L[(size_t)level - 1];
      LoopLevel& cl = L[(size_t)level];
      OPCALL(mgcfd_op_up_pre(f.n, cl.n, f.n2mg, cl.var, cl.scratch, nullptr));
      OPCALL(mgcfd_op_up(f.n, cl.n, f.n2mg, f.var, cl.var, cl.scratch, nullptr));
      OPCALL(mgcfd_op_up_post(cl.n, cl.var, cl.scratch, nullptr));
      if (level == levels - 1) up = false;
    } else {  // euler3d.cpp:598-639 (down_kernel: p_edge_to_mg_nodes is always NULL)
      level--;
      LoopLevel& f = L[(size_t)level];
      LoopLevel& cl = L[(size_t)level + 1];
      OPCALL(mgcfd_op_down(f.n, cl.n, f.n2mg, f.var, f.res, f.coords, cl.res, cl.coords, nullptr));
      if (level == 0) {
        up = true;
        i++;
      }
    }
  }
  if (cudaDeviceSynchronize() != cudaSuccess) return fail(MGCFD_ERR_CUDA);
  std::printf("\nCompute complete\n");
  std::printf("Max total runtime = %f\n", wall() - t0);

  out->vars.resize((size_t)levels);
  out->step_factors.resize((size_t)levels);
  out->fluxes.resize((size_t)levels);
  for (int l = 0; l < levels; l++) {
    const LoopLevel& d = L[(size_t)l];
    if (!DeviceArena::download(&out->vars[(size_t)l], d.var, 5 * (size_t)d.n) ||
        (c.out_step_factors && !DeviceArena::download(&out->step_factors[(size_t)l], d.sf, (size_t)d.n)) ||
        (c.out_fluxes && !DeviceArena::download(&out->fluxes[(size_t)l], d.flux, 5 * (size_t)d.n)))
      return fail(MGCFD_ERR_CUDA);
  }
  return 0;
}

// The default run: the device-resident solver.
int run_solver(const Config& c, const std::vector<mgcfd_level_view>& lv, Results* out) {
  const int levels = (int)lv.size();
  mgcfd_solver_options opt;
  mgcfd_solver_default_options(&opt);
  opt.precision = c.precision;
  opt.increment = c.increment;
  opt.accumulation = c.accumulation;
  opt.renumber = c.renumber ? MGCFD_RENUMBER_RCM : MGCFD_RENUMBER_SPATIAL;
  opt.measure_mem_bound = c.mem_bound ? 1 : 0;
  mgcfd_solver* s = nullptr;
  int st;
  if ((st = mgcfd_solver_create(levels, lv.data(), c.mach, c.aoa, &opt, nullptr, &s))) return fail(st);

  std::printf("-----------------------------------------------------\nCompute beginning\n");
  const double t0 = wall();
  if (c.flow_interval <= 0) {
    for (int i = 0; i < c.cycles && !st; i++) {
      std::printf("Performing MG cycle %d / %d\n", i + 1, c.cycles);
      st = mgcfd_solver_run(s, 1);
    }
  } else {
    int64_t done = 0;
    bool at_l0 = true;
    while (done < c.cycles && !st) {
      if (at_l0) std::printf("Performing MG cycle %d / %d\n", (int)done + 1, c.cycles);
      int32_t smoothed = 0;
      const int64_t before = done;
      if ((st = mgcfd_solver_step(s, &smoothed, &done))) break;
      at_l0 = done != before;
      if (smoothed == 0) {
        const int64_t i = levels <= 1 ? done - 1 : before;  // cycle whose level-0 smoothing this was
        if (((i + 1) % c.flow_interval) == 0) {
          std::vector<double> v((size_t)lv[0].nnodes * 5);
          if ((st = mgcfd_solver_fetch(s, 0, MGCFD_Q_VARIABLES, v.data()))) break;
          std::string f = c.prefix + "variables.L0.cycle=" + std::to_string(i + 1) + ".h5";
          if ((st = mgcfd_h5_write_f64(f.c_str(), "p_variables", v.data(), lv[0].nnodes, 5))) break;
        }
      }
    }
  }
  if (!st) st = mgcfd_solver_synchronize(s);
  if (st == MGCFD_ERR_NEGATIVE_DT || st == MGCFD_ERR_BAD_VALUES) {
    std::printf("%s\n", mgcfd_last_error());
    mgcfd_solver_destroy(s);
    return 1;
  }
  if (st) return fail(st);
  std::printf("\nCompute complete\n");
  std::printf("Max total runtime = %f\n", wall() - t0);

  out->vars.resize((size_t)levels);
  out->step_factors.resize((size_t)levels);
  out->fluxes.resize((size_t)levels);
  for (int l = 0; l < levels; l++) {
    const size_t n = (size_t)lv[(size_t)l].nnodes;
    out->vars[(size_t)l].resize(n * 5);
    if ((st = mgcfd_solver_fetch(s, l, MGCFD_Q_VARIABLES, out->vars[(size_t)l].data()))) return fail(st);
    if (c.out_step_factors) {
      out->step_factors[(size_t)l].resize(n);
      if ((st = mgcfd_solver_fetch(s, l, MGCFD_Q_STEP_FACTORS, out->step_factors[(size_t)l].data()))) return fail(st);
    }
    if (c.out_fluxes) {
      out->fluxes[(size_t)l].resize(n * 5);
      if ((st = mgcfd_solver_fetch(s, l, MGCFD_Q_FLUXES, out->fluxes[(size_t)l].data()))) return fail(st);
    }
  }
  mgcfd_solver_destroy(s);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  Config c;
  if (!parse(argc, argv, c)) return 1;
  if (c.input_file.empty()) {
    std::printf("ERROR: input_file not set\n");
    return 1;
  }
  std::printf("-----------------------------------------------------\nLoading from HDF5 files ...\n");
  mgcfd_host_mesh* mesh = nullptr;
  int st = mgcfd_host_mesh_load(c.input_file.c_str(), c.input_dir.c_str(), c.legacy ? 1 : 0, &mesh);
  if (st) {
    std::fprintf(stderr, "Error: %s\n", mgcfd_last_error());
    return 1;
  }
  const int levels = mgcfd_host_mesh_num_levels(mesh);
  std::vector<mgcfd_level_view> lv((size_t)levels);
  for (int l = 0; l < levels; l++) {
    mgcfd_host_mesh_level(mesh, l, &lv[(size_t)l]);
    std::printf("Loading level %d / %d\n", l + 1, levels);
  }
  // Solutions for -v (euler3d.cpp:314-335).
  std::vector<std::string> solution((size_t)levels);
  if (c.validate)
    for (int l = 0; l < levels; l++) {
      std::string p = dir_join(c.input_dir, "solution.variables.L" + std::to_string(l) + ".cycles=" +
                                                std::to_string(c.cycles) + ".h5");
      if (access(p.c_str(), R_OK) != -1) solution[(size_t)l] = p;
      else std::printf("Cannot find level %d solution file: %s\n", l, p.c_str());
    }

  if (c.per_loop && c.precision == MGCFD_PRECISION_MIXED) {
    std::printf("ERROR: --per-loop runs the reference's FP64 loops (the flux in the DW form with --precision dw); "
                "--precision mixed needs the solver\n");
    mgcfd_host_mesh_destroy(mesh);
    return 1;
  }
  // --per-loop --precision dw: the edge-flux calls in the DW form (through their plans).
  if (c.per_loop) mgcfd_op_flux_precision(c.precision == MGCFD_PRECISION_DW ? MGCFD_PRECISION_DW : MGCFD_PRECISION_FP64);
  if (c.per_loop && c.renumber) std::printf("Note: -n has no effect with --per-loop (the loops' plans order the nodes)\n");
  Results res;
  st = c.per_loop ? run_per_loop(c, lv, &res) : run_solver(c, lv, &res);
  if (st) {
    mgcfd_host_mesh_destroy(mesh);
    return 1;
  }
  std::vector<std::vector<double>>& vars = res.vars;

  if (c.validate) {  // euler3d.cpp:658-718, validation.h:46-115
    std::printf("-----------------------------------------------------\n");
    bool value_check_failed = false;
    std::printf("Looking for NaN and infinity values ...");
    for (int l = 0; l < levels && !value_check_failed; l++) {
      int bad = 0;
      for (double x : vars[(size_t)l]) bad += (std::isnan(x) || std::isinf(x)) ? 1 : 0;
      if (bad > 0) {
        value_check_failed = true;
        std::printf("\nValue check of MG level %d failed: %d bad values detected\n", l, bad);
      }
    }
    if (!value_check_failed) {
      std::printf(" None found\n");
      bool failed = false;
      std::printf("Validating result against solution ...");
      for (int l = 0; l < levels; l++) {
        if (solution[(size_t)l].empty()) {
          std::printf("\n- Do not have solution for level %d, cannot validate\n", l);
          failed = true;
          continue;
        }
        std::vector<double> ref(vars[(size_t)l].size());
        if (mgcfd_h5_read_f64(solution[(size_t)l].c_str(), ("p_variables_result_L" + std::to_string(l)).c_str(),
                              ref.data(), (int64_t)ref.size())) {
          std::printf("\n%s\n", mgcfd_last_error());
          failed = true;
          continue;
        }
        int count = 0;
        for (size_t k = 0; k < ref.size(); k++) {
          double acceptable = std::fabs(ref[k] * 10.0e-8);
          if (acceptable < 3.0e-19) acceptable = 3.0e-19;
          if (std::fabs(vars[(size_t)l][k] - ref[k]) > acceptable) count++;
        }
        if (count > lv[(size_t)l].nnodes / 5000) {
          failed = true;
          std::printf("\nValidation of MG level %d failed: %d incorrect values in 'variables' array\n", l, count);
          break;
        }
      }
      if (failed) std::printf("Validation failed\n");
      else std::printf(" Result correct\nValidation passed\n");
    }
  }

  if (c.out_variables || c.out_fluxes || c.out_step_factors) {  // euler3d.cpp:720-779
    std::printf("-----------------------------------------------------\nWriting out data...\n");
    for (int l = 0; l < levels; l++) {
      const std::string sfx = ".L" + std::to_string(l) + ".cycles=" + std::to_string(c.cycles) + ".h5";
      const int32_t n = lv[(size_t)l].nnodes;
      if (c.out_step_factors &&
          (st = mgcfd_h5_write_f64((c.prefix + "step_factors" + sfx).c_str(),
                                   ("p_step_factors_result_L" + std::to_string(l)).c_str(),
                                   res.step_factors[(size_t)l].data(), n, 1)))
        return fail(st);
      if (c.out_fluxes &&
          (st = mgcfd_h5_write_f64((c.prefix + "fluxes" + sfx).c_str(),
                                   ("p_fluxes_result_L" + std::to_string(l)).c_str(), res.fluxes[(size_t)l].data(),
                                   n, 5)))
        return fail(st);
      if (c.out_variables &&
          (st = mgcfd_h5_write_f64((c.prefix + "variables" + sfx).c_str(),
                                   ("p_variables_result_L" + std::to_string(l)).c_str(), vars[(size_t)l].data(), n, 5)))
        return fail(st);
    }
  }
  std::printf("-----------------------------------------------------\n");
  mgcfd_host_mesh_destroy(mesh);
  return 0;
}
