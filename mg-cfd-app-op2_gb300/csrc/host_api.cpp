// Host side of the C ABI: status strings, far-field state, host meshes
// (synthetic or read from an input.dat deck and its HDF5 level files) and the
// HDF5 helpers.
#include <cmath>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "common.h"
#include "h5lite.h"
#include "meshgen.h"
#include "mgcfd_gb300.h"

namespace mgcfd {

static thread_local std::string g_last_error;

int set_error(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}
void clear_error() { g_last_error.clear(); }

}  // namespace mgcfd


using mgcfd::set_error;

extern "C" int mgcfd_abi_version(void) { return MGCFD_ABI_VERSION; }

extern "C" const char* mgcfd_last_error(void) { return mgcfd::g_last_error.c_str(); }

extern "C" const char* mgcfd_status_string(int status) {
  switch (status) {
    case MGCFD_OK: return "ok";
    case MGCFD_ERR_INVALID: return "invalid argument";
    case MGCFD_ERR_CUDA: return "CUDA error";
    case MGCFD_ERR_NOMEM: return "out of memory";
    case MGCFD_ERR_IO: return "I/O error";
    case MGCFD_ERR_NEGATIVE_DT: return "negative time step (min_dt < 0)";
    case MGCFD_ERR_BAD_VALUES: return "bad variable values (NaN or Inf)";
    case MGCFD_ERR_TIMEOUT: return "device wait timed out";
    case MGCFD_ERR_BUDGET: return "request exceeds HBM budget";
    default: return "unknown status";
  }
}

// euler3d.cpp:157-189.  Same operation order as the reference, so the
// freestream bits match it for the same Mach and angle of attack.
extern "C" int mgcfd_freestream_init(double mach, double aoa_deg, mgcfd_freestream* ff) {
  if (!ff) return set_error(MGCFD_ERR_INVALID, "mgcfd_freestream_init: null output");
  const double angle = (3.1415926535897931 / 180.0) * aoa_deg;
  ff->smoothing_coefficient = (double)0.2f;
  double* v = ff->ff_variable;
  v[0] = 1.4;
  const double pressure = 1.0;
  const double sos = std::sqrt(mgcfd::kGamma * pressure / v[0]);
  const double speed = mach * sos;
  const double vel[3] = {speed * std::cos(angle), speed * std::sin(angle), 0.0};
  for (int d = 0; d < 3; d++) v[1 + d] = v[0] * vel[d];
  v[4] = v[0] * (0.5 * (speed * speed)) + (pressure / (mgcfd::kGamma - 1.0));
  // Momentum-flux tensor u_i m_j + p delta_ij and energy flux u_i (rhoE + p),
  // as inlined_funcs.h:70-96 evaluates them.
  double* fx = ff->ff_flux_contribution_momentum_x;
  double* fy = ff->ff_flux_contribution_momentum_y;
  double* fz = ff->ff_flux_contribution_momentum_z;
  double* fe = ff->ff_flux_contribution_density_energy;
  fx[0] = vel[0] * v[1] + pressure;
  fx[1] = vel[0] * v[2];
  fx[2] = vel[0] * v[3];
  fy[0] = fx[1];
  fy[1] = vel[1] * v[2] + pressure;
  fy[2] = vel[1] * v[3];
  fz[0] = fx[2];
  fz[1] = fy[2];
  fz[2] = vel[2] * v[3] + pressure;
  const double h = v[4] + pressure;
  for (int d = 0; d < 3; d++) fe[d] = vel[d] * h;
  return MGCFD_OK;
}

// ---------------------------------------------------------------------------
// Host meshes.

extern "C" int mgcfd_host_mesh_generate(int n, int nlevels, uint64_t seed, mgcfd_host_mesh** out) {
  if (!out) return set_error(MGCFD_ERR_INVALID, "mgcfd_host_mesh_generate: null output");
  *out = nullptr;
  std::unique_ptr<mgcfd_host_mesh> m(new (std::nothrow) mgcfd_host_mesh());
  if (!m) return set_error(MGCFD_ERR_NOMEM, "host allocation failed");
  std::string err;
  try {
    if (!mgcfd::generate_lattice_mesh(n, nlevels, seed, &m->mesh, &err)) return set_error(MGCFD_ERR_INVALID, err);
  } catch (const std::bad_alloc&) {
    return set_error(MGCFD_ERR_NOMEM, "host allocation failed while generating the mesh");
  }
  *out = m.release();
  return MGCFD_OK;
}

extern "C" int mgcfd_host_mesh_from_views(int32_t nlevels, const mgcfd_level_view* levels, mgcfd_host_mesh** out) {
  if (!out || !levels || nlevels < 1) return set_error(MGCFD_ERR_INVALID, "mgcfd_host_mesh_from_views: bad arguments");
  *out = nullptr;
  for (int l = 0; l < nlevels; l++) {
    const mgcfd_level_view& v = levels[l];
    if (v.nnodes < 1 || v.nedges < 0 || v.nbnd < 0 || !v.coords || (v.nedges && (!v.edge_to_nodes || !v.edge_weights)) ||
        (v.nbnd && (!v.bnd_to_node || !v.bnd_group || !v.bnd_weights)) || (l + 1 < nlevels && !v.node_to_mg))
      return set_error(MGCFD_ERR_INVALID, "mgcfd_host_mesh_from_views: level " + std::to_string(l) + " is incomplete");
  }
  try {
    std::unique_ptr<mgcfd_host_mesh> m(new mgcfd_host_mesh());
    m->mesh.levels.resize((size_t)nlevels);
    for (int l = 0; l < nlevels; l++) {
      const mgcfd_level_view& v = levels[l];
      mgcfd::HostLevel& L = m->mesh.levels[(size_t)l];
      const size_t n = (size_t)v.nnodes, ne = (size_t)v.nedges, nb = (size_t)v.nbnd;
      L.n_axis = v.n_axis;
      L.nnodes = v.nnodes; L.nedges = v.nedges; L.nbnd = v.nbnd;
      L.coords.assign(v.coords, v.coords + 3 * n);
      if (ne) {
        L.edge_to_nodes.assign(v.edge_to_nodes, v.edge_to_nodes + 2 * ne);
        L.edge_weights.assign(v.edge_weights, v.edge_weights + 3 * ne);
      }
      if (nb) {
        L.bnd_to_node.assign(v.bnd_to_node, v.bnd_to_node + nb);
        L.bnd_group.assign(v.bnd_group, v.bnd_group + nb);
        L.bnd_weights.assign(v.bnd_weights, v.bnd_weights + 3 * nb);
      }
      if (l + 1 < nlevels) L.node_to_mg.assign(v.node_to_mg, v.node_to_mg + n);
      if (v.volumes) L.volumes.assign(v.volumes, v.volumes + n);
    }
    *out = m.release();
  } catch (const std::bad_alloc&) {
    return set_error(MGCFD_ERR_NOMEM, "host allocation failed");
  }
  return MGCFD_OK;
}

namespace {

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) a++;
  while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
  return s.substr(a, b - a);
}

struct InputDeck {
  int size = 0, levels = 0, base_array_index = 1;
  std::vector<std::string> layers;
};

// io.h:28-205 (read_input_dat): key=value lines, '#' comments, a [levels]
// section of `num_levels` "i=file" lines and an optional [mg_mapping]
// section; size, num_levels, mesh_name and the level files are required.
int parse_input_dat(const std::string& path, InputDeck* deck) {
  std::ifstream f(path);
  if (!f.is_open()) return set_error(MGCFD_ERR_IO, "Could not open input file '" + path + "'");
  bool have_size = false, have_levels = false, have_name = false, have_files = false;
  std::string line;
  while (std::getline(f, line)) {
    if (!line.empty() && line[0] == '#') continue;
    if (!line.empty() && line[0] == '[') {
      bool is_levels = line == "[levels]", is_map = line == "[mg_mapping]";
      if (!is_levels && !is_map) continue;
      if (!have_levels)
        return set_error(MGCFD_ERR_IO, "Error parsing " + path + ": Need to know number of levels before parsing level filenames");
      int count = is_levels ? deck->levels : deck->levels - 1;
      if (is_levels) { have_files = true; deck->layers.assign((size_t)deck->levels, std::string()); }
      for (int i = 0; i < count; i++) {
        if (!std::getline(f, line))
          return set_error(MGCFD_ERR_IO, "Error parsing " + path + ": Have reached EOF before reading all mesh filenames");
        size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        std::string key = trim(line.substr(0, eq)), value = trim(line.substr(eq + 1));
        if (value.empty() && eq + 1 >= line.size()) continue;
        int idx = std::atoi(key.c_str());
        if (is_levels) {
          if (idx < 0 || idx >= deck->levels)
            return set_error(MGCFD_ERR_IO, "Error parsing " + path + ": level index " + key + " out of range");
          deck->layers[(size_t)idx] = value;
        }
      }
      continue;
    }
    size_t eq = line.find('=');
    if (eq == std::string::npos || eq + 1 > line.size()) continue;
    if (eq + 1 == line.size()) continue;  // no value after '='
    std::string key = trim(line.substr(0, eq)), value = trim(line.substr(eq + 1));
    if (key == "size") { deck->size = std::atoi(value.c_str()); have_size = true; }
    else if (key == "num_levels") { deck->levels = std::atoi(value.c_str()); have_levels = true; }
    else if (key == "base_array_index") { deck->base_array_index = std::atoi(value.c_str()); }
    else if (key == "mesh_name") {
      if (value == "la_cascade" || value == "rotor37" || value == "fvcorr" || value == "m6wing") have_name = true;
      else return set_error(MGCFD_ERR_IO, "Error parsing " + path + ": Unknown mesh_name '" + value + "'");
    }
  }
  if (!have_size) return set_error(MGCFD_ERR_IO, "Error parsing '" + path + "': size not present");
  if (!have_levels) return set_error(MGCFD_ERR_IO, "Error parsing '" + path + "': number of levels not present");
  if (!have_name) return set_error(MGCFD_ERR_IO, "Error parsing '" + path + "': mesh name not present");
  if (!have_files) return set_error(MGCFD_ERR_IO, "Error parsing '" + path + "': mesh filenames not present");
  if (deck->levels < 1) return set_error(MGCFD_ERR_IO, "Error parsing '" + path + "': num_levels must be >= 1");
  return MGCFD_OK;
}

int read_map(const h5lite::File& f, const std::string& file, const std::string& name, int64_t rows, int dim,
             int base, int64_t target_size, std::vector<int32_t>* out) {
  const h5lite::DatasetInfo* d = f.find(name);
  if (!d) return set_error(MGCFD_ERR_IO, "dataset '" + name + "' not found in " + file);
  if ((int64_t)d->dims[0] != rows || (int64_t)d->nelems() != rows * dim)
    return set_error(MGCFD_ERR_IO, "dataset '" + name + "' in " + file + " has the wrong shape");
  out->resize((size_t)(rows * dim));
  std::string err;
  if (!f.read_i32(name, out->data(), (uint64_t)(rows * dim), &err)) return set_error(MGCFD_ERR_IO, file + ": " + err);
  for (auto& v : *out) {
    v -= base;
    if (v < 0 || v >= target_size)
      return set_error(MGCFD_ERR_IO, "map '" + name + "' in " + file + " has an entry out of range");
  }
  return MGCFD_OK;
}

int read_dat(const h5lite::File& f, const std::string& file, const std::string& name, int64_t rows, int dim,
             std::vector<double>* out) {
  const h5lite::DatasetInfo* d = f.find(name);
  if (!d) return set_error(MGCFD_ERR_IO, "dataset '" + name + "' not found in " + file);
  if ((int64_t)d->dims[0] != rows || (int64_t)d->nelems() != rows * dim)
    return set_error(MGCFD_ERR_IO, "dataset '" + name + "' in " + file + " has the wrong shape");
  out->resize((size_t)(rows * dim));
  std::string err;
  if (!f.read_f64(name, out->data(), (uint64_t)(rows * dim), &err)) return set_error(MGCFD_ERR_IO, file + ": " + err);
  return MGCFD_OK;
}

}  // namespace

// euler3d.cpp:84-117 (paths, base_array_index) and :243-312 (per-level sets,
// maps and dats).
extern "C" int mgcfd_host_mesh_load(const char* input_file, const char* input_dir, int legacy_mode,
                                    mgcfd_host_mesh** out) {
  if (!input_file || !out) return set_error(MGCFD_ERR_INVALID, "mgcfd_host_mesh_load: null argument");
  *out = nullptr;
  std::string dir = input_dir ? input_dir : "";
  std::string path = dir.empty() ? std::string(input_file) : dir + "/" + input_file;
  InputDeck deck;
  int st = parse_input_dat(path, &deck);
  if (st) return st;
  const int base = (deck.base_array_index >= 1 && deck.base_array_index <= 9) ? deck.base_array_index : 0;
  const std::string sfx = legacy_mode ? ".renumbered" : "";
  std::unique_ptr<mgcfd_host_mesh> m(new (std::nothrow) mgcfd_host_mesh());
  if (!m) return set_error(MGCFD_ERR_NOMEM, "host allocation failed");
  m->mesh.levels.resize((size_t)deck.levels);
  std::vector<h5lite::File> files((size_t)deck.levels);
  std::vector<std::string> names((size_t)deck.levels);
  try {
    for (int l = 0; l < deck.levels; l++) {
      names[l] = dir.empty() ? deck.layers[l] : dir + "/" + deck.layers[l];
      std::string err;
      if (!files[l].open(names[l], &err)) return set_error(MGCFD_ERR_IO, err);
      const h5lite::File& f = files[l];
      auto rows_of = [&](const std::string& ds, int64_t* rows) -> int {
        const h5lite::DatasetInfo* d = f.find(ds);
        if (!d || d->rank < 1) return set_error(MGCFD_ERR_IO, "dataset '" + ds + "' not found in " + names[l]);
        if (d->dims[0] > 2147483647ull) return set_error(MGCFD_ERR_IO, "dataset '" + ds + "' too large");
        *rows = (int64_t)d->dims[0];
        return MGCFD_OK;
      };
      mgcfd::HostLevel& L = m->mesh.levels[l];
      int64_t N, E, B;
      if ((st = rows_of("node_coordinates" + sfx, &N)) || (st = rows_of("edge-->node" + sfx, &E)) ||
          (st = rows_of("bnd_node-->node" + sfx, &B)))
        return st;
      L.nnodes = (int32_t)N; L.nedges = (int32_t)E; L.nbnd = (int32_t)B; L.n_axis = 0;
      if ((st = read_map(f, names[l], "edge-->node" + sfx, E, 2, base, N, &L.edge_to_nodes)) ||
          (st = read_map(f, names[l], "bnd_node-->node" + sfx, B, 1, base, N, &L.bnd_to_node)))
        return st;
      // bnd_node-->group is a dat (no base subtraction), euler3d.cpp:279.
      {
        const h5lite::DatasetInfo* d = f.find("bnd_node-->group");
        if (!d || (int64_t)d->nelems() != B) return set_error(MGCFD_ERR_IO, "dataset 'bnd_node-->group' missing or wrong shape in " + names[l]);
        L.bnd_group.resize((size_t)B);
        if (!f.read_i32("bnd_node-->group", L.bnd_group.data(), (uint64_t)B, &err)) return set_error(MGCFD_ERR_IO, err);
      }
      if ((st = read_dat(f, names[l], legacy_mode ? "edge_weights.recalculated" : "edge_weights", E, 3, &L.edge_weights)) ||
          (st = read_dat(f, names[l], "bnd_node_weights", B, 3, &L.bnd_weights)) ||
          (st = read_dat(f, names[l], "node_coordinates" + sfx, N, 3, &L.coords)))
        return st;
      if (legacy_mode && (st = read_dat(f, names[l], "areas", N, 1, &L.volumes))) return st;
    }
    // node-->mg_node lives in level l's file and maps into level l+1 (euler3d.cpp:281-283).
    for (int l = 0; l + 1 < deck.levels; l++) {
      mgcfd::HostLevel& L = m->mesh.levels[l];
      if ((st = read_map(files[l], names[l], "node-->mg_node" + sfx, L.nnodes, 1, base,
                         m->mesh.levels[l + 1].nnodes, &L.node_to_mg)))
        return st;
    }
  } catch (const std::bad_alloc&) {
    return set_error(MGCFD_ERR_NOMEM, "host allocation failed while reading the mesh");
  }
  *out = m.release();
  return MGCFD_OK;
}

extern "C" int mgcfd_host_mesh_write(const mgcfd_host_mesh* mesh, const char* dir, const char* prefix,
                                     int32_t legacy_datasets) {
  if (!mesh || !dir) return set_error(MGCFD_ERR_INVALID, "mgcfd_host_mesh_write: null argument");
  std::string err;
  if (!mgcfd::write_mesh_files(mesh->mesh, dir, prefix ? prefix : "", legacy_datasets != 0, &err))
    return set_error(MGCFD_ERR_IO, err);
  return MGCFD_OK;
}

extern "C" int mgcfd_host_mesh_num_levels(const mgcfd_host_mesh* mesh) {
  return mesh ? (int)mesh->mesh.levels.size() : 0;
}

extern "C" int mgcfd_host_mesh_level(const mgcfd_host_mesh* mesh, int level, mgcfd_level_view* v) {
  if (!mesh || !v || level < 0 || level >= (int)mesh->mesh.levels.size())
    return set_error(MGCFD_ERR_INVALID, "mgcfd_host_mesh_level: bad arguments");
  const mgcfd::HostLevel& L = mesh->mesh.levels[(size_t)level];
  v->nnodes = L.nnodes; v->nedges = L.nedges; v->nbnd = L.nbnd; v->n_axis = L.n_axis;
  v->coords = L.coords.data();
  v->edge_to_nodes = L.edge_to_nodes.data();
  v->bnd_to_node = L.bnd_to_node.data();
  v->bnd_group = L.bnd_group.data();
  v->edge_weights = L.edge_weights.data();
  v->bnd_weights = L.bnd_weights.data();
  v->node_to_mg = L.node_to_mg.empty() ? nullptr : L.node_to_mg.data();
  v->volumes = L.volumes.empty() ? nullptr : L.volumes.data();
  return MGCFD_OK;
}

extern "C" void mgcfd_host_mesh_destroy(mgcfd_host_mesh* mesh) { delete mesh; }

// ---------------------------------------------------------------------------
// HDF5 helpers.

extern "C" int mgcfd_h5_dataset_shape(const char* path, const char* name, int64_t dims[2], int* rank) {
  if (!path || !name || !dims || !rank) return set_error(MGCFD_ERR_INVALID, "mgcfd_h5_dataset_shape: null argument");
  h5lite::File f;
  std::string err;
  if (!f.open(path, &err)) return set_error(MGCFD_ERR_IO, err);
  const h5lite::DatasetInfo* d = f.find(name);
  if (!d) return set_error(MGCFD_ERR_IO, std::string("dataset '") + name + "' not found in " + path);
  *rank = d->rank;
  dims[0] = d->rank > 0 ? (int64_t)d->dims[0] : 1;
  dims[1] = d->rank > 1 ? (int64_t)d->dims[1] : 0;
  return MGCFD_OK;
}

extern "C" int mgcfd_h5_read_f64(const char* path, const char* name, double* out, int64_t n) {
  if (!path || !name || (!out && n)) return set_error(MGCFD_ERR_INVALID, "mgcfd_h5_read_f64: null argument");
  h5lite::File f;
  std::string err;
  if (!f.open(path, &err) || !f.read_f64(name, out, (uint64_t)n, &err)) return set_error(MGCFD_ERR_IO, err);
  return MGCFD_OK;
}

extern "C" int mgcfd_h5_read_i32(const char* path, const char* name, int32_t* out, int64_t n) {
  if (!path || !name || (!out && n)) return set_error(MGCFD_ERR_INVALID, "mgcfd_h5_read_i32: null argument");
  h5lite::File f;
  std::string err;
  if (!f.open(path, &err) || !f.read_i32(name, out, (uint64_t)n, &err)) return set_error(MGCFD_ERR_IO, err);
  return MGCFD_OK;
}

extern "C" int mgcfd_h5_write_f64(const char* path, const char* name, const double* data, int64_t rows, int64_t cols) {
  if (!path || !name || (!data && rows) || rows < 0 || cols < 0)
    return set_error(MGCFD_ERR_INVALID, "mgcfd_h5_write_f64: bad argument");
  std::string err;
  h5lite::DatasetOut o{name, h5lite::F64, (uint64_t)rows, (uint64_t)cols, data, true};
  if (!h5lite::write_file(path, {o}, &err)) return set_error(MGCFD_ERR_IO, err);
  return MGCFD_OK;
}
