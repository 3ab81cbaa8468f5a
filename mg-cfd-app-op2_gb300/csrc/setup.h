// Host-side preparation of a multigrid mesh for the device solver:
// geometry initialisation (euler3d.cpp:413-441), node renumbering for
// locality, edge orientation and ordering, boundary entries folded per node,
// and the multigrid transfer tables.  Everything here is integer work except
// the geometry initialisation, which follows the reference's sequential
// order exactly (so volumes and weights are bit-identical to the reference).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "mgcfd_gb300.h"

namespace mgcfd {

struct PreparedLevel {
  int32_t n = 0, ne = 0;
  std::vector<int32_t> perm;       // new id -> input id
  std::vector<int32_t> inv;        // input id -> new id
  std::vector<double> vol;         // [n] dual volumes (new order)
  std::vector<int32_t> e2n;        // [ne][2] new ids, a < b, sorted by (a, b)
  std::vector<double> w4;          // [ne][4] (-wx/2, -wy/2, -wz/2, -|w| * smoothing * 0.5), damped
  std::vector<int32_t> a_off;      // [n+1] edges with first node a occupy [a_off[a], a_off[a+1])
  std::vector<int32_t> b_off;      // [n+1] CSR of edges by second node
  std::vector<int32_t> b_list;     // [ne]
  std::vector<int32_t> bidx;       // [n] row in bdata or -1
  std::vector<double> bdata;       // [nb][12] far-field sum w (3), wall sum w (3), w.F_ff (5), pad
  std::vector<int32_t> n2mg;       // [n] new coarse id (empty on coarsest level)
  std::vector<double> dvec;        // [n][4] |dx|, |dy|, |dz|, dist to the coarse parent
  std::vector<int32_t> ch_off;     // [n+1] fine children of each node of this level (as coarse)
  std::vector<int32_t> ch_list;    // [n_fine]
  int32_t nb = 0;
};

// Sizes, null pointers and (when check_maps) every map entry of the views.
int validate_views(int32_t nlevels, const mgcfd_level_view* levels, bool check_maps);

// Returns MGCFD_OK or an error status (message via set_error).  With
// fp32_geometry (the mixed-precision form) the per-edge geometry -- volume
// contributions, damped weights and |w| -- is computed in FP32; volumes are
// still summed in FP64.
int prepare_mesh(int32_t nlevels, const mgcfd_level_view* levels, const mgcfd_freestream& ff, int renumber,
                 bool fp32_geometry, std::vector<PreparedLevel>* out);

// Node orderings (new id -> input id).
void spatial_order(const double* xyz, int32_t n, std::vector<int32_t>* perm);
void rcm_order(int32_t n, int32_t ne, const int32_t* e2n, std::vector<int32_t>* perm);

}  // namespace mgcfd
