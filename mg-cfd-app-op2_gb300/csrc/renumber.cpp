// Mesh renumbering as a standalone step (the reference's -n option calls
// op_renumber(p_edge_to_nodes[0]) at euler3d.cpp:377, which reorders the
// level-0 node set with Scotch inside OP2).  Here every level is renumbered
// on the host with one of the solver's own orders (Morton curve or reverse
// Cuthill-McKee), and the result is an ordinary mesh that can be written in
// the reference's HDF5 layout for any consumer.
//
// For a node permutation P (P[new] = old) with inverse Q (Q[old] = new):
//   * node data moves: coords'[i] = coords[P[i]], volumes'[i] = volumes[P[i]];
//   * every edge keeps its direction (so its weight keeps its sign) and its
//     endpoints become (Q[a], Q[b]); edges are then ordered by
//     (min, max) of the new endpoints, ties kept in input order;
//   * boundary entries are ordered by Q[node], ties kept in input order;
//   * node-->mg_node of level l becomes Q_{l+1}[map[P_l[i]]].
// All of this is integer work: the output is a relabelling of the input, and
// a solve on it gives the input's solution up to the rounding of the changed
// edge order.
#include <algorithm>
#include <memory>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "common.h"
#include "meshgen.h"
#include "mgcfd_gb300.h"
#include "setup.h"

namespace mgcfd {
namespace {

bool node_order(int method, const HostLevel& L, std::vector<int32_t>* perm) {
  if (method == MGCFD_RENUMBER_SPATIAL) {
    spatial_order(L.coords.data(), L.nnodes, perm);
  } else if (method == MGCFD_RENUMBER_RCM) {
    rcm_order(L.nnodes, L.nedges, L.edge_to_nodes.data(), perm);
  } else if (method == MGCFD_RENUMBER_NONE) {
    perm->resize((size_t)L.nnodes);
    std::iota(perm->begin(), perm->end(), 0);
  } else {
    return false;
  }
  return true;
}

void relabel_level(const HostLevel& in, const std::vector<int32_t>& P, const std::vector<int32_t>& Q,
                   const std::vector<int32_t>* Q_next, HostLevel* out) {
  const size_t n = (size_t)in.nnodes, ne = (size_t)in.nedges, nb = (size_t)in.nbnd;
  out->n_axis = in.n_axis;
  out->nnodes = in.nnodes;
  out->nedges = in.nedges;
  out->nbnd = in.nbnd;
  out->coords.resize(3 * n);
  for (size_t i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) out->coords[3 * i + d] = in.coords[3 * (size_t)P[i] + d];
  if (!in.volumes.empty()) {
    out->volumes.resize(n);
    for (size_t i = 0; i < n; i++) out->volumes[i] = in.volumes[(size_t)P[i]];
  }
  // Edges: order by (min, max) of the new endpoints; a stable sort keeps
  // parallel edges (same endpoints) in input order.
  std::vector<int32_t> eorder(ne);
  std::iota(eorder.begin(), eorder.end(), 0);
  auto ekey = [&](int32_t e) {
    int32_t a = Q[(size_t)in.edge_to_nodes[2 * (size_t)e]], b = Q[(size_t)in.edge_to_nodes[2 * (size_t)e + 1]];
    return std::make_pair(std::min(a, b), std::max(a, b));
  };
  std::stable_sort(eorder.begin(), eorder.end(), [&](int32_t x, int32_t y) { return ekey(x) < ekey(y); });
  out->edge_to_nodes.resize(2 * ne);
  out->edge_weights.resize(3 * ne);
  for (size_t k = 0; k < ne; k++) {
    size_t e = (size_t)eorder[k];
    out->edge_to_nodes[2 * k] = Q[(size_t)in.edge_to_nodes[2 * e]];
    out->edge_to_nodes[2 * k + 1] = Q[(size_t)in.edge_to_nodes[2 * e + 1]];
    for (int d = 0; d < 3; d++) out->edge_weights[3 * k + d] = in.edge_weights[3 * e + d];
  }
  std::vector<int32_t> border(nb);
  std::iota(border.begin(), border.end(), 0);
  std::stable_sort(border.begin(), border.end(), [&](int32_t x, int32_t y) {
    return Q[(size_t)in.bnd_to_node[(size_t)x]] < Q[(size_t)in.bnd_to_node[(size_t)y]];
  });
  out->bnd_to_node.resize(nb);
  out->bnd_group.resize(nb);
  out->bnd_weights.resize(3 * nb);
  for (size_t k = 0; k < nb; k++) {
    size_t b = (size_t)border[k];
    out->bnd_to_node[k] = Q[(size_t)in.bnd_to_node[b]];
    out->bnd_group[k] = in.bnd_group[b];
    for (int d = 0; d < 3; d++) out->bnd_weights[3 * k + d] = in.bnd_weights[3 * b + d];
  }
  out->node_to_mg.clear();
  if (Q_next && !in.node_to_mg.empty()) {
    out->node_to_mg.resize(n);
    for (size_t i = 0; i < n; i++) out->node_to_mg[i] = (*Q_next)[(size_t)in.node_to_mg[(size_t)P[i]]];
  }
}

bool level_in_range(const HostLevel& L, int32_t next_nnodes, std::string* why) {
  auto bad = [&](const std::vector<int32_t>& v, int32_t lim) {
    for (int32_t x : v)
      if (x < 0 || x >= lim) return true;
    return false;
  };
  if ((int64_t)L.coords.size() != 3 * (int64_t)L.nnodes || (int64_t)L.edge_to_nodes.size() != 2 * (int64_t)L.nedges ||
      (int64_t)L.bnd_to_node.size() != (int64_t)L.nbnd) {
    *why = "inconsistent set sizes";
    return false;
  }
  if (bad(L.edge_to_nodes, L.nnodes) || bad(L.bnd_to_node, L.nnodes)) {
    *why = "map entry out of range";
    return false;
  }
  if (next_nnodes >= 0 && !L.node_to_mg.empty() && bad(L.node_to_mg, next_nnodes)) {
    *why = "node-->mg_node entry out of range";
    return false;
  }
  return true;
}

}  // namespace
}  // namespace mgcfd

extern "C" int mgcfd_renumber_nodes(int method, int32_t nnodes, const double* coords, int32_t nedges,
                                    const int32_t* edge_to_nodes, int32_t* perm_out) {
  if (nnodes < 1 || nedges < 0 || !perm_out || (method == MGCFD_RENUMBER_SPATIAL && !coords) ||
      (method == MGCFD_RENUMBER_RCM && nedges > 0 && !edge_to_nodes))
    return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_renumber_nodes: bad arguments");
  if (method == MGCFD_RENUMBER_RCM)
    for (int64_t k = 0; k < 2 * (int64_t)nedges; k++)
      if (edge_to_nodes[k] < 0 || edge_to_nodes[k] >= nnodes)
        return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_renumber_nodes: edge map entry out of range");
  std::vector<int32_t> perm;
  try {
    if (method == MGCFD_RENUMBER_SPATIAL) mgcfd::spatial_order(coords, nnodes, &perm);
    else if (method == MGCFD_RENUMBER_RCM) mgcfd::rcm_order(nnodes, nedges, edge_to_nodes, &perm);
    else if (method == MGCFD_RENUMBER_NONE) { perm.resize((size_t)nnodes); std::iota(perm.begin(), perm.end(), 0); }
    else return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_renumber_nodes: unknown method");
  } catch (const std::bad_alloc&) {
    return mgcfd::set_error(MGCFD_ERR_NOMEM, "host allocation failed");
  }
  std::copy(perm.begin(), perm.end(), perm_out);
  return MGCFD_OK;
}

extern "C" int mgcfd_host_mesh_renumber(const mgcfd_host_mesh* in, int method, mgcfd_host_mesh** out) {
  using namespace mgcfd;
  if (!in || !out) return set_error(MGCFD_ERR_INVALID, "mgcfd_host_mesh_renumber: null argument");
  *out = nullptr;
  if (method != MGCFD_RENUMBER_NONE && method != MGCFD_RENUMBER_SPATIAL && method != MGCFD_RENUMBER_RCM)
    return set_error(MGCFD_ERR_INVALID, "mgcfd_host_mesh_renumber: unknown method");
  const auto& lv = in->mesh.levels;
  const size_t nl = lv.size();
  for (size_t l = 0; l < nl; l++) {
    std::string why;
    if (!level_in_range(lv[l], l + 1 < nl ? lv[l + 1].nnodes : -1, &why))
      return set_error(MGCFD_ERR_INVALID, "mgcfd_host_mesh_renumber: level " + std::to_string(l) + ": " + why);
  }
  try {
    std::unique_ptr<mgcfd_host_mesh> m(new mgcfd_host_mesh());
    std::vector<std::vector<int32_t>> P(nl), Q(nl);
    for (size_t l = 0; l < nl; l++) {
      node_order(method, lv[l], &P[l]);
      Q[l].resize(P[l].size());
      for (size_t i = 0; i < P[l].size(); i++) Q[l][(size_t)P[l][i]] = (int32_t)i;
    }
    m->mesh.levels.resize(nl);
    for (size_t l = 0; l < nl; l++)
      relabel_level(lv[l], P[l], Q[l], l + 1 < nl ? &Q[l + 1] : nullptr, &m->mesh.levels[l]);
    *out = m.release();
  } catch (const std::bad_alloc&) {
    return set_error(MGCFD_ERR_NOMEM, "host allocation failed");
  }
  return MGCFD_OK;
}
