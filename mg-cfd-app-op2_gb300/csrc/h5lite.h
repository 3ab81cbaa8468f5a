// h5lite: a self-contained reader/writer for the subset of the HDF5 file
// format that MG-CFD's mesh and solution files use.
//
// MG-CFD (euler3d.cpp:243-336 for input, :552-571 and :720-779 for output)
// stores every mesh level and every solution as a flat HDF5 file whose root
// group holds contiguous, uncompressed 1-D or 2-D datasets of int32 or
// float64: "node_coordinates" [N][3], "edge-->node" [E][2],
// "bnd_node-->node" [B][1], "bnd_node-->group" [B][1], "edge_weights" [E][3],
// "bnd_node_weights" [B][3], "node-->mg_node" [N][1] and
// "p_variables_result_L<l>" [N][5].  libhdf5 is not available to this
// project, so this file implements the format directly:
//
//   writer: superblock version 0, a root group stored as a symbol table
//           (version-1 B-tree of group nodes, symbol-table nodes, local heap),
//           one version-1 object header per dataset with dataspace, datatype,
//           fill-value and version-3 contiguous layout messages, plus the
//           optional "size"/"dim"/"type" attributes that OP2 attaches to
//           datasets it writes.
//   reader: superblocks version 0 and 1, symbol-table root groups (any
//           B-tree depth), version-1 object headers with continuation
//           blocks, layout messages version 1-3 (compact or contiguous),
//           little-endian fixed-point (4/8 byte) and IEEE float (4/8 byte)
//           element types, converted on read to int32 or float64.
//
// Files produced by newer libhdf5 "latest format" settings (superblock v2/v3,
// object header v2, link messages, chunked layout) are rejected with a clear
// error message instead of being misread.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace h5lite {

enum DType : int { F64 = 1, I32 = 2 };

// One dataset to be written.  `data` points to rows*cols elements of `dtype`
// in row-major order.  rank is 1 when cols == 0, else 2.
struct DatasetOut {
  std::string name;
  DType dtype;
  uint64_t rows;
  uint64_t cols;          // 0 => 1-D dataset of `rows` elements
  const void* data;
  bool op2_attributes;    // attach OP2's "size", "dim", "type" attributes
};

// Write a new file (truncating any existing one) holding `sets` in its root
// group.  Returns false and fills *err on failure.
bool write_file(const std::string& path, const std::vector<DatasetOut>& sets,
                std::string* err);

struct DatasetInfo {
  std::string name;
  int rank = 0;
  uint64_t dims[4] = {0, 0, 0, 0};
  int type_class = -1;   // 0 fixed-point, 1 float, 3 string
  int type_size = 0;
  bool type_signed = true;
  uint64_t data_addr = 0;   // absolute file offset of contiguous data
  uint64_t data_size = 0;
  std::vector<uint8_t> compact;  // data for compact layout
  bool is_compact = false;
  uint64_t nelems() const {
    uint64_t n = 1;
    for (int i = 0; i < rank; i++) n *= dims[i];
    return rank == 0 ? 1 : n;
  }
};

class File {
 public:
  bool open(const std::string& path, std::string* err);
  const std::vector<DatasetInfo>& datasets() const { return sets_; }
  const DatasetInfo* find(const std::string& name) const;
  // Read a whole dataset, converting to float64 or int32.  `out` must hold
  // nelems() elements.  Returns false with *err on type or I/O error.
  bool read_f64(const std::string& name, double* out, uint64_t nelems, std::string* err) const;
  bool read_i32(const std::string& name, int32_t* out, uint64_t nelems, std::string* err) const;

 private:
  bool read_raw(const DatasetInfo& d, std::vector<uint8_t>* buf, std::string* err) const;
  std::vector<uint8_t> bytes_;
  uint64_t base_ = 0;
  std::vector<DatasetInfo> sets_;
};

}  // namespace h5lite
