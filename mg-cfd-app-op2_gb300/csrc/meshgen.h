// Synthetic multigrid meshes in MG-CFD's input layout.
//
// MG-CFD's published datasets (Onera M6, Rotor37) are distributed outside the
// reference repository, so workloads here are seeded jittered lattices with
// the same per-level structure the driver reads (euler3d.cpp:243-312):
//
//   * level 0 is an n x n x n lattice on [0,1]^3 with spacing h = 1/(n-1);
//     nodes that lie on no face of the cube are displaced by U(-0.2h, 0.2h)
//     per axis; nodes on a face are not displaced;
//   * level l+1 keeps every second lattice index of level l (same jittered
//     coordinates), so a level has ceil(n_l/2) nodes per axis;
//   * each level has its own lattice edges to the +x, +y and +z neighbours
//     (E = 3 n_l^2 (n_l - 1)); an edge's weight is h_l^2 * unit(x_b - x_a);
//   * boundary entries are one per (node, face): group 0 (solid wall,
//     flux_boundary.elem_func) on z = 0, group 3 (far field,
//     flux_wall.elem_func) on the other five faces; the weight is the
//     outward unit normal times h_l^2;
//   * node, edge and boundary-entry ids are randomly permuted per level
//     (Fisher-Yates driven by SplitMix64), so access is unstructured;
//   * node-->mg_node maps lattice index i to floor(i/2) per axis.
//
// All arithmetic is plain IEEE double without contraction, so the generator
// produces identical bits on every host.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace mgcfd {

struct HostLevel {
  int32_t n_axis = 0;
  int32_t nnodes = 0, nedges = 0, nbnd = 0;
  std::vector<double> coords;          // [N][3]
  std::vector<int32_t> edge_to_nodes;  // [E][2]
  std::vector<int32_t> bnd_to_node;    // [B]
  std::vector<int32_t> bnd_group;      // [B]
  std::vector<double> edge_weights;    // [E][3]
  std::vector<double> bnd_weights;     // [B][3]
  std::vector<int32_t> node_to_mg;     // [N] -> ids of level+1 (empty on the coarsest level)
  std::vector<double> volumes;         // [N] legacy-mode "areas" (empty: computed from edges)
};

struct HostMesh {
  std::vector<HostLevel> levels;
};

// Generate `nlevels` levels starting from an n^3 lattice.  Returns false
// (with *err) if the sizes are invalid (n < 2, a level shrinking below 2 nodes
// per axis, or more than 2^31-1 edges).
bool generate_lattice_mesh(int n, int nlevels, uint64_t seed, HostMesh* out, std::string* err);

// Write level files "<prefix>L<l>.h5" and "<dir>/input.dat" (base_array_index=0,
// mesh_name=fvcorr) in the layout euler3d.cpp reads.  With legacy_datasets the
// files also carry the legacy-mode datasets of euler3d.cpp:247-309
// ("*.renumbered" copies, "areas" = dual volumes and
// "edge_weights.recalculated" = re-oriented weights, both computed as
// misc.h:40-76 does in edge order).
bool write_mesh_files(const HostMesh& mesh, const std::string& dir, const std::string& prefix,
                      bool legacy_datasets, std::string* err);

}  // namespace mgcfd

// The opaque mgcfd_host_mesh handle of the C ABI.
struct mgcfd_host_mesh {
  mgcfd::HostMesh mesh;
};
