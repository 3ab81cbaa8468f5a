// ORACLE TEST INFRASTRUCTURE -- not part of the product.
//
// A sequential stand-in for the OP2 API that MG-CFD's euler3d.cpp uses, so
// that the reference driver and its elemental-kernel headers compile
// unmodified into the reference binary `oracle/_ref/euler3d_ref`.  OP2-Common
// (op_seq.h, op_hdf5.h and its runtime) is not part of the reference
// repository, so this header restates the *semantics* of OP2's sequential
// backend as euler3d.cpp relies on them:
//
//   * op_par_loop(kernel, name, set, args...) visits elements 0..size-1 in
//     order and calls kernel(ptr_0, ..., ptr_k) where ptr_i is
//       dat->data + n*dat->size                         for OP_ID arguments,
//       dat->data + map->map[n*map->dim + idx]*dat->size for mapped arguments,
//       the global's own address                         for op_arg_gbl;
//     OP_INC / OP_MIN globals are therefore updated in place in element
//     order, and indirect increments land in edge order (euler3d.cpp:498-503).
//   * dat->size is dim * (element size); op_decl_dat_temp_char allocates
//     zero-filled storage (euler3d.cpp:379-409 relies on p_up_scratch starting
//     at zero).
//   * maps are stored 0-based; OP_MAPS_BASE_INDEX=<b> on the command line
//     (appended by euler3d.cpp:104-117) makes map reads subtract b.
//   * op_partition / op_renumber are no-ops, as in a non-MPI sequential build.
//
// HDF5 access uses the project's own h5lite reader/writer.
#ifndef MGCFD_ORACLE_OP_SEQ_H
#define MGCFD_ORACLE_OP_SEQ_H

#include <cstddef>
#include <cstdio>
#include <cstdarg>
#include <utility>

typedef enum { OP_READ, OP_WRITE, OP_RW, OP_INC, OP_MIN, OP_MAX } op_access;

struct op_set_core {
  int index;
  int size;
  char const* name;
};
typedef op_set_core* op_set;

struct op_map_core {
  int index;
  op_set from;
  op_set to;
  int dim;
  int* map;
  char const* name;
};
typedef op_map_core* op_map;

struct op_dat_core {
  int index;
  op_set set;
  int dim;
  int size;       // bytes per element = dim * sizeof(type)
  char* data;
  char const* name;
  char const* type;
};
typedef op_dat_core* op_dat;

struct op_arg {
  op_dat dat;
  op_map map;
  int idx;
  char* gbl;
  int size;
  op_access acc;
  bool is_gbl;
};

#define OP_ID ((op_map)NULL)

void op_init(int argc, char** argv, int diags);
void op_exit();
void op_printf(const char* fmt, ...);
void op_timers(double* cpu, double* wall);
int op_get_size(op_set set);
void op_rank(int* rank);

op_set op_decl_set(int size, char const* name);
op_map op_decl_map(op_set from, op_set to, int dim, int* imap, char const* name);
op_dat op_decl_dat_char(op_set set, int dim, char const* type, int size, char* data, char const* name);
op_dat op_decl_dat_temp_char(op_set set, int dim, char const* type, int size, char const* name);

template <class T>
void op_decl_const(int, char const*, T*) {}

void op_partition(const char* lib, const char* method, op_set prime_set, op_map prime_map, op_dat coords);
void op_renumber(op_map base);

inline op_arg op_arg_dat(op_dat dat, int idx, op_map map, int dim, char const* type, op_access acc) {
  (void)dim; (void)type;
  op_arg a;
  a.dat = dat; a.map = map; a.idx = idx; a.gbl = NULL; a.size = dat ? dat->size : 0;
  a.acc = acc; a.is_gbl = false;
  return a;
}

template <class T>
op_arg op_arg_gbl(T* data, int dim, char const* type, op_access acc) {
  (void)type;
  op_arg a;
  a.dat = NULL; a.map = NULL; a.idx = -1; a.gbl = reinterpret_cast<char*>(data);
  a.size = dim * (int)sizeof(T); a.acc = acc; a.is_gbl = true;
  return a;
}

inline char* op_shim_elem_ptr(const op_arg& a, int n) {
  if (a.is_gbl) return a.gbl;
  if (a.map == NULL) return a.dat->data + (size_t)n * (size_t)a.dat->size;
  int target = a.map->map[(size_t)n * (size_t)a.map->dim + (size_t)a.idx];
  return a.dat->data + (size_t)target * (size_t)a.dat->size;
}

template <class... P, std::size_t... I>
inline void op_shim_call(void (*kernel)(P...), const op_arg* args, int n, std::index_sequence<I...>) {
  kernel(reinterpret_cast<P>(op_shim_elem_ptr(args[I], n))...);
}

template <class... P, class... A>
void op_par_loop(void (*kernel)(P...), char const* name, op_set set, A... args) {
  static_assert(sizeof...(P) == sizeof...(A), "op_par_loop: argument count does not match kernel");
  (void)name;
  const op_arg arr[] = {args...};
  for (int n = 0; n < set->size; n++) op_shim_call(kernel, arr, n, std::index_sequence_for<P...>{});
}

#endif
