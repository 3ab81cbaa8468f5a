// Synthetic jittered-lattice multigrid meshes; the specification is in
// meshgen.h.  Output datasets and input.dat follow euler3d.cpp:243-312 and
// io.h:28-205 of the reference.
#include "meshgen.h"

#include <cmath>
#include <cstdio>

#include "h5lite.h"

namespace mgcfd {
namespace {

// SplitMix64 (Steele, Lea and Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014).
struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

uint64_t stream_seed(uint64_t seed, uint64_t tag) {
  SplitMix64 r(seed ^ (tag * 0xD1B54A32D192ED03ull));
  return r.next();
}

enum : uint64_t { kTagJitter = 1, kTagNodes = 0x100, kTagEdges = 0x200, kTagBnd = 0x300 };

// Fisher-Yates shuffle of the identity: result[i] is the new id of element i.
std::vector<int32_t> random_permutation(int64_t n, uint64_t seed) {
  std::vector<int32_t> p((size_t)n);
  for (int64_t i = 0; i < n; i++) p[(size_t)i] = (int32_t)i;
  SplitMix64 r(seed);
  for (int64_t i = n - 1; i > 0; i--) {
    int64_t j = (int64_t)(r.next() % (uint64_t)(i + 1));
    int32_t t = p[(size_t)i]; p[(size_t)i] = p[(size_t)j]; p[(size_t)j] = t;
  }
  return p;
}

}  // namespace

bool generate_lattice_mesh(int n, int nlevels, uint64_t seed, HostMesh* out, std::string* err) {
  if (n < 2) { *err = "lattice needs at least 2 nodes per axis"; return false; }
  if (nlevels < 1) { *err = "need at least one level"; return false; }
  std::vector<int> naxis(nlevels);
  naxis[0] = n;
  for (int l = 1; l < nlevels; l++) {
    naxis[l] = (naxis[l - 1] + 1) / 2;
    if (naxis[l] < 2) { *err = "level " + std::to_string(l) + " would have fewer than 2 nodes per axis"; return false; }
  }
  const int64_t n64 = n;
  if (3 * n64 * n64 * (n64 - 1) > 2147483647ll) { *err = "lattice too large for int32 ids"; return false; }

  // Level-0 coordinates in lattice order (i fastest), jittered in the interior.
  const double h = 1.0 / (double)(n - 1);
  std::vector<double> c0((size_t)(n64 * n64 * n64 * 3));
  {
    SplitMix64 rj(stream_seed(seed, kTagJitter));
    for (int64_t k = 0; k < n; k++)
      for (int64_t j = 0; j < n; j++)
        for (int64_t i = 0; i < n; i++) {
          size_t q = (size_t)(i + n64 * (j + n64 * k));
          double u0 = rj.uniform(), u1 = rj.uniform(), u2 = rj.uniform();
          double x = (double)i * h, y = (double)j * h, z = (double)k * h;
          bool interior = i > 0 && i < n - 1 && j > 0 && j < n - 1 && k > 0 && k < n - 1;
          if (interior) {
            x += (u0 * 0.4 - 0.2) * h;
            y += (u1 * 0.4 - 0.2) * h;
            z += (u2 * 0.4 - 0.2) * h;
          }
          c0[3 * q + 0] = x; c0[3 * q + 1] = y; c0[3 * q + 2] = z;
        }
  }

  out->levels.assign(nlevels, HostLevel());
  std::vector<std::vector<int32_t>> nperm(nlevels);
  for (int l = 0; l < nlevels; l++) {
    const int64_t m = naxis[l];
    const int64_t N = m * m * m;
    nperm[l] = random_permutation(N, stream_seed(seed, kTagNodes + l));
  }
  for (int l = 0; l < nlevels; l++) {
    HostLevel& L = out->levels[l];
    const int64_t m = naxis[l];
    const int64_t N = m * m * m;
    const int64_t stride = 1ll << l;
    const double hl = h * (double)stride;
    const double hl2 = hl * hl;
    const std::vector<int32_t>& np = nperm[l];
    L.n_axis = (int32_t)m;
    L.nnodes = (int32_t)N;
    L.coords.assign((size_t)N * 3, 0.0);
    for (int64_t k = 0; k < m; k++)
      for (int64_t j = 0; j < m; j++)
        for (int64_t i = 0; i < m; i++) {
          int64_t q = i + m * (j + m * k);
          size_t q0 = (size_t)(i * stride + n64 * (j * stride + n64 * (k * stride)));
          int32_t id = np[(size_t)q];
          for (int d = 0; d < 3; d++) L.coords[3 * (size_t)id + d] = c0[3 * q0 + d];
        }

    // Edges in lattice order, then permuted.
    const int64_t E = 3 * m * m * (m - 1);
    L.nedges = (int32_t)E;
    std::vector<int32_t> ep = random_permutation(E, stream_seed(seed, kTagEdges + l));
    L.edge_to_nodes.assign((size_t)E * 2, 0);
    L.edge_weights.assign((size_t)E * 3, 0.0);
    int64_t qe = 0;
    auto add_edge = [&](int64_t a, int64_t b) {
      int32_t pos = ep[(size_t)qe++];
      int32_t ia = np[(size_t)a], ib = np[(size_t)b];
      L.edge_to_nodes[2 * (size_t)pos + 0] = ia;
      L.edge_to_nodes[2 * (size_t)pos + 1] = ib;
      double d[3], len2 = 0.0;
      for (int c = 0; c < 3; c++) {
        d[c] = L.coords[3 * (size_t)ib + c] - L.coords[3 * (size_t)ia + c];
        len2 += d[c] * d[c];
      }
      double len = std::sqrt(len2);
      for (int c = 0; c < 3; c++) L.edge_weights[3 * (size_t)pos + c] = (d[c] / len) * hl2;
    };
    for (int64_t k = 0; k < m; k++)
      for (int64_t j = 0; j < m; j++)
        for (int64_t i = 0; i < m; i++) {
          int64_t q = i + m * (j + m * k);
          if (i + 1 < m) add_edge(q, q + 1);
          if (j + 1 < m) add_edge(q, q + m);
          if (k + 1 < m) add_edge(q, q + m * m);
        }

    // Boundary entries: one per (node, face), faces in order x-, x+, y-, y+, z-, z+.
    std::vector<int64_t> bn;
    std::vector<int32_t> bg;
    std::vector<double> bw;
    for (int64_t k = 0; k < m; k++)
      for (int64_t j = 0; j < m; j++)
        for (int64_t i = 0; i < m; i++) {
          int64_t q = i + m * (j + m * k);
          const int64_t idx[3] = {i, j, k};
          for (int ax = 0; ax < 3; ax++)
            for (int side = 0; side < 2; side++) {
              bool on = side == 0 ? idx[ax] == 0 : idx[ax] == m - 1;
              if (!on) continue;
              bn.push_back(q);
              bg.push_back((ax == 2 && side == 0) ? 0 : 3);
              double nrm[3] = {0.0, 0.0, 0.0};
              nrm[ax] = side == 0 ? -1.0 : 1.0;
              for (int c = 0; c < 3; c++) bw.push_back(nrm[c] * hl2);
            }
        }
    const int64_t B = (int64_t)bn.size();
    L.nbnd = (int32_t)B;
    std::vector<int32_t> bp = random_permutation(B, stream_seed(seed, kTagBnd + l));
    L.bnd_to_node.assign((size_t)B, 0);
    L.bnd_group.assign((size_t)B, 0);
    L.bnd_weights.assign((size_t)B * 3, 0.0);
    for (int64_t r = 0; r < B; r++) {
      int32_t pos = bp[(size_t)r];
      L.bnd_to_node[(size_t)pos] = np[(size_t)bn[(size_t)r]];
      L.bnd_group[(size_t)pos] = bg[(size_t)r];
      for (int c = 0; c < 3; c++) L.bnd_weights[3 * (size_t)pos + c] = bw[3 * (size_t)r + c];
    }

    // Fine -> coarse map.
    if (l + 1 < nlevels) {
      const int64_t mc = naxis[l + 1];
      const std::vector<int32_t>& npc = nperm[l + 1];
      L.node_to_mg.assign((size_t)N, 0);
      for (int64_t k = 0; k < m; k++)
        for (int64_t j = 0; j < m; j++)
          for (int64_t i = 0; i < m; i++) {
            int64_t q = i + m * (j + m * k);
            int64_t qc = (i >> 1) + mc * ((j >> 1) + mc * (k >> 1));
            L.node_to_mg[(size_t)np[(size_t)q]] = npc[(size_t)qc];
          }
    }
  }
  return true;
}

bool write_mesh_files(const HostMesh& mesh, const std::string& dir, const std::string& prefix,
                      bool legacy_datasets, std::string* err) {
  const int nl = (int)mesh.levels.size();
  for (int l = 0; l < nl; l++) {
    const HostLevel& L = mesh.levels[l];
    std::vector<double> areas, recalculated;
    if (legacy_datasets) {  // misc.h:40-76 in edge order
      areas.assign((size_t)L.nnodes, 0.0);
      recalculated = L.edge_weights;
      for (int32_t e = 0; e < L.nedges; e++) {
        const int32_t a = L.edge_to_nodes[2 * (size_t)e], b = L.edge_to_nodes[2 * (size_t)e + 1];
        double d[3], dist = 0.0, area = 0.0;
        for (int i = 0; i < 3; i++) {
          d[i] = L.coords[3 * (size_t)b + i] - L.coords[3 * (size_t)a + i];
          dist += d[i] * d[i];
        }
        dist = std::sqrt(dist);
        double* w = &recalculated[3 * (size_t)e];
        for (int i = 0; i < 3; i++) area += w[i] * w[i];
        area = std::sqrt(area);
        const double tv = (1.0 / 3.0) * 0.5 * dist * area;
        areas[(size_t)a] += tv;
        areas[(size_t)b] += tv;
        for (int i = 0; i < 3; i++) w[i] = (d[i] / dist) * area;
        for (int i = 0; i < 3; i++) w[i] /= dist;
      }
    }
    std::vector<h5lite::DatasetOut> sets = {
        {"node_coordinates", h5lite::F64, (uint64_t)L.nnodes, 3, L.coords.data(), false},
        {"edge-->node", h5lite::I32, (uint64_t)L.nedges, 2, L.edge_to_nodes.data(), false},
        {"bnd_node-->node", h5lite::I32, (uint64_t)L.nbnd, 1, L.bnd_to_node.data(), false},
        {"bnd_node-->group", h5lite::I32, (uint64_t)L.nbnd, 1, L.bnd_group.data(), false},
        {"edge_weights", h5lite::F64, (uint64_t)L.nedges, 3, L.edge_weights.data(), false},
        {"bnd_node_weights", h5lite::F64, (uint64_t)L.nbnd, 3, L.bnd_weights.data(), false},
    };
    if (!L.node_to_mg.empty())
      sets.push_back({"node-->mg_node", h5lite::I32, (uint64_t)L.nnodes, 1, L.node_to_mg.data(), false});
    if (legacy_datasets) {
      sets.push_back({"node_coordinates.renumbered", h5lite::F64, (uint64_t)L.nnodes, 3, L.coords.data(), false});
      sets.push_back({"edge-->node.renumbered", h5lite::I32, (uint64_t)L.nedges, 2, L.edge_to_nodes.data(), false});
      sets.push_back({"bnd_node-->node.renumbered", h5lite::I32, (uint64_t)L.nbnd, 1, L.bnd_to_node.data(), false});
      sets.push_back({"areas", h5lite::F64, (uint64_t)L.nnodes, 1, areas.data(), false});
      sets.push_back({"edge_weights.recalculated", h5lite::F64, (uint64_t)L.nedges, 3, recalculated.data(), false});
      if (!L.node_to_mg.empty())
        sets.push_back({"node-->mg_node.renumbered", h5lite::I32, (uint64_t)L.nnodes, 1, L.node_to_mg.data(), false});
    }
    std::string path = dir + "/" + prefix + "L" + std::to_string(l) + ".h5";
    if (!h5lite::write_file(path, sets, err)) return false;
  }
  std::string ip = dir + "/input.dat";
  FILE* f = std::fopen(ip.c_str(), "w");
  if (!f) { *err = "cannot create " + ip; return false; }
  std::fprintf(f, "size=%d\n", nl ? mesh.levels[0].nnodes : 0);
  std::fprintf(f, "num_levels=%d\n", nl);
  std::fprintf(f, "base_array_index=0\n");
  std::fprintf(f, "mesh_name=fvcorr\n");
  std::fprintf(f, "[levels]\n");
  for (int l = 0; l < nl; l++) std::fprintf(f, "%d=%sL%d.h5\n", l, prefix.c_str(), l);
  if (std::fclose(f) != 0) { *err = "write failed for " + ip; return false; }
  return true;
}

}  // namespace mgcfd
