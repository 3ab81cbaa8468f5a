// ORACLE TEST INFRASTRUCTURE -- not part of the product.
//
// HDF5 declarations of the sequential OP2 stand-in (see op_seq.h).  Semantics
// restated from how euler3d.cpp:243-336 and :552-571, :720-779 use them:
//   op_decl_set_hdf5_infer_size(file, set_name, dataset): set size = dim 0 of
//       the dataset;
//   op_decl_map_hdf5(from, to, dim, file, dataset): int map [from->size][dim],
//       minus the OP_MAPS_BASE_INDEX base;
//   op_decl_dat_hdf5(set, dim, type, file, dataset): "double" or "int" data
//       [set->size][dim];
//   op_fetch_data_hdf5_file(dat, file): writes [set->size][dim] under
//       dat->name into a new file, with OP2's "size"/"dim"/"type" attributes.
// Any failure prints the problem and exits, as OP2 does.
#ifndef MGCFD_ORACLE_OP_HDF5_H
#define MGCFD_ORACLE_OP_HDF5_H

#include "op_seq.h"

op_set op_decl_set_hdf5_infer_size(char const* file, char const* name, char const* dataset_name);
op_map op_decl_map_hdf5(op_set from, op_set to, int dim, char const* file, char const* name);
op_dat op_decl_dat_hdf5(op_set set, int dim, char const* type, char const* file, char const* name);
void op_fetch_data_hdf5_file(op_dat dat, char const* file_name);

#endif
