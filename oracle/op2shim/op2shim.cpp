// ORACLE TEST INFRASTRUCTURE -- not part of the product.
// Implementation of the sequential OP2 stand-in declared in op_seq.h/op_hdf5.h.
#include "op_hdf5.h"

#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>
#include <sys/time.h>

#include "h5lite.h"

static int g_map_base = 0;
static std::vector<void*> g_allocs;

static void shim_fail(const std::string& msg) {
  std::fprintf(stderr, "op2shim: %s\n", msg.c_str());
  std::fflush(stderr);
  std::exit(EXIT_FAILURE);
}

void op_init(int argc, char** argv, int) {
  const char* key = "OP_MAPS_BASE_INDEX=";
  for (int i = 0; i < argc; i++)
    if (std::strncmp(argv[i], key, std::strlen(key)) == 0) g_map_base = std::atoi(argv[i] + std::strlen(key));
}

void op_exit() {
  for (void* p : g_allocs) std::free(p);
  g_allocs.clear();
}

void op_printf(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vprintf(fmt, ap);
  va_end(ap);
}

void op_timers(double* cpu, double* wall) {
  *cpu = (double)std::clock() / CLOCKS_PER_SEC;
  struct timeval t;
  gettimeofday(&t, NULL);
  *wall = (double)t.tv_sec + 1.0e-6 * (double)t.tv_usec;
}

int op_get_size(op_set set) { return set->size; }
void op_rank(int* rank) { *rank = 0; }

static char* shim_calloc(size_t n) {
  void* p = std::calloc(n ? n : 1, 1);
  if (!p) shim_fail("out of memory");
  g_allocs.push_back(p);
  return static_cast<char*>(p);
}

op_set op_decl_set(int size, char const* name) {
  op_set s = new op_set_core;
  s->index = 0; s->size = size; s->name = name ? strdup(name) : "";
  return s;
}

op_map op_decl_map(op_set from, op_set to, int dim, int* imap, char const* name) {
  op_map m = new op_map_core;
  m->index = 0; m->from = from; m->to = to; m->dim = dim; m->map = imap; m->name = strdup(name);
  return m;
}

op_dat op_decl_dat_char(op_set set, int dim, char const* type, int size, char* data, char const* name) {
  op_dat d = new op_dat_core;
  d->index = 0; d->set = set; d->dim = dim; d->size = dim * size; d->data = data;
  d->name = strdup(name); d->type = strdup(type);
  return d;
}

op_dat op_decl_dat_temp_char(op_set set, int dim, char const* type, int size, char const* name) {
  char* data = shim_calloc((size_t)set->size * (size_t)dim * (size_t)size);
  return op_decl_dat_char(set, dim, type, size, data, name);
}

void op_partition(const char*, const char*, op_set, op_map, op_dat) {}
void op_renumber(op_map) {}

static const h5lite::DatasetInfo* open_info(h5lite::File& f, char const* file, char const* name) {
  std::string err;
  if (!f.open(file, &err)) shim_fail(err);
  const h5lite::DatasetInfo* d = f.find(name);
  if (!d) shim_fail(std::string("dataset '") + name + "' not found in " + file);
  return d;
}

op_set op_decl_set_hdf5_infer_size(char const* file, char const* name, char const* dataset_name) {
  h5lite::File f;
  const h5lite::DatasetInfo* d = open_info(f, file, dataset_name);
  if (d->rank < 1) shim_fail(std::string("dataset '") + dataset_name + "' has no dimensions");
  return op_decl_set((int)d->dims[0], name);
}

op_map op_decl_map_hdf5(op_set from, op_set to, int dim, char const* file, char const* name) {
  h5lite::File f;
  const h5lite::DatasetInfo* d = open_info(f, file, name);
  if ((int64_t)d->dims[0] != from->size) shim_fail(std::string("map '") + name + "' size mismatch");
  uint64_t n = (uint64_t)from->size * (uint64_t)dim;
  int* m = reinterpret_cast<int*>(shim_calloc(n * sizeof(int)));
  std::string err;
  if (!f.read_i32(name, m, n, &err)) shim_fail(err);
  for (uint64_t i = 0; i < n; i++) {
    m[i] -= g_map_base;
    if (m[i] < 0 || m[i] >= to->size) shim_fail(std::string("map '") + name + "' entry out of range");
  }
  return op_decl_map(from, to, dim, m, name);
}

op_dat op_decl_dat_hdf5(op_set set, int dim, char const* type, char const* file, char const* name) {
  h5lite::File f;
  open_info(f, file, name);
  uint64_t n = (uint64_t)set->size * (uint64_t)dim;
  std::string err;
  if (std::strcmp(type, "double") == 0) {
    double* p = reinterpret_cast<double*>(shim_calloc(n * sizeof(double)));
    if (!f.read_f64(name, p, n, &err)) shim_fail(err);
    return op_decl_dat_char(set, dim, type, sizeof(double), reinterpret_cast<char*>(p), name);
  }
  if (std::strcmp(type, "int") == 0) {
    int* p = reinterpret_cast<int*>(shim_calloc(n * sizeof(int)));
    if (!f.read_i32(name, p, n, &err)) shim_fail(err);
    return op_decl_dat_char(set, dim, type, sizeof(int), reinterpret_cast<char*>(p), name);
  }
  shim_fail(std::string("unsupported dat type ") + type);
  return NULL;
}

void op_fetch_data_hdf5_file(op_dat dat, char const* file_name) {
  bool is_double = std::strcmp(dat->type, "double") == 0;
  if (!is_double && std::strcmp(dat->type, "int") != 0) shim_fail("unsupported dat type in fetch");
  std::vector<uint8_t> buf((size_t)dat->set->size * (size_t)dat->dim * (is_double ? 8 : 4));
  size_t esz = is_double ? 8 : 4;
  for (int n = 0; n < dat->set->size; n++)
    std::memcpy(buf.data() + (size_t)n * dat->dim * esz, dat->data + (size_t)n * dat->size, (size_t)dat->dim * esz);
  h5lite::DatasetOut o{dat->name, is_double ? h5lite::F64 : h5lite::I32, (uint64_t)dat->set->size,
                       (uint64_t)dat->dim, buf.data(), true};
  std::string err;
  if (!h5lite::write_file(file_name, {o}, &err)) shim_fail(err);
}
