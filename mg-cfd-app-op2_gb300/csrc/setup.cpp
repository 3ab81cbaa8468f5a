// Host-side mesh preparation for the device solver (see setup.h).
#include "setup.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <queue>

#include "common.h"

namespace mgcfd {
namespace {

// Stable LSD radix sort of (key, value) pairs by 64-bit key, 16 bits per pass.
void radix_sort_pairs(std::vector<uint64_t>& key, std::vector<int32_t>& val) {
  const size_t n = key.size();
  std::vector<uint64_t> k2(n);
  std::vector<int32_t> v2(n);
  std::vector<size_t> cnt(65536 + 1);
  for (int pass = 0; pass < 4; pass++) {
    const int shift = 16 * pass;
    std::fill(cnt.begin(), cnt.end(), 0);
    for (size_t i = 0; i < n; i++) cnt[((key[i] >> shift) & 0xffff) + 1]++;
    if (cnt[1] == n) continue;  // every key has the same digit
    for (size_t d = 0; d < 65536; d++) cnt[d + 1] += cnt[d];
    for (size_t i = 0; i < n; i++) {
      size_t pos = cnt[(key[i] >> shift) & 0xffff]++;
      k2[pos] = key[i];
      v2[pos] = val[i];
    }
    key.swap(k2);
    val.swap(v2);
  }
}

uint64_t spread3(uint64_t x) {  // 21 bits -> every third bit
  x &= 0x1fffff;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

}  // namespace

// Morton (Z-order) curve over coordinates quantised to 21 bits per axis in
// the bounding box; ties keep input order.
void spatial_order(const double* xyz, int32_t n, std::vector<int32_t>* perm) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int32_t i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      lo[d] = std::min(lo[d], xyz[3 * (size_t)i + d]);
      hi[d] = std::max(hi[d], xyz[3 * (size_t)i + d]);
    }
  double scale[3];
  for (int d = 0; d < 3; d++) scale[d] = (hi[d] > lo[d] && std::isfinite(hi[d] - lo[d])) ? 2097151.0 / (hi[d] - lo[d]) : 0.0;
  std::vector<uint64_t> key((size_t)n);
  std::vector<int32_t> val((size_t)n);
  for (int32_t i = 0; i < n; i++) {
    uint64_t q[3];
    for (int d = 0; d < 3; d++) {
      double t = (xyz[3 * (size_t)i + d] - lo[d]) * scale[d];
      if (!(t > 0.0)) t = 0.0;
      if (t > 2097151.0) t = 2097151.0;
      q[d] = (uint64_t)t;
    }
    key[(size_t)i] = (spread3(q[2]) << 2) | (spread3(q[1]) << 1) | spread3(q[0]);
    val[(size_t)i] = i;
  }
  radix_sort_pairs(key, val);
  perm->swap(val);
}

// Reverse Cuthill-McKee: breadth-first from a low-degree pseudo-peripheral
// node of each component, neighbours in ascending degree, then reversed.
void rcm_order(int32_t n, int32_t ne, const int32_t* e2n, std::vector<int32_t>* perm) {
  std::vector<int32_t> deg((size_t)n + 1, 0);
  for (int32_t e = 0; e < ne; e++) { deg[(size_t)e2n[2 * (size_t)e]]++; deg[(size_t)e2n[2 * (size_t)e + 1]]++; }
  std::vector<int64_t> off((size_t)n + 1, 0);
  for (int32_t i = 0; i < n; i++) off[(size_t)i + 1] = off[(size_t)i] + deg[(size_t)i];
  std::vector<int32_t> adj((size_t)off[(size_t)n]);
  std::vector<int64_t> fill(off.begin(), off.end() - 1);
  for (int32_t e = 0; e < ne; e++) {
    int32_t a = e2n[2 * (size_t)e], b = e2n[2 * (size_t)e + 1];
    adj[(size_t)fill[(size_t)a]++] = b;
    adj[(size_t)fill[(size_t)b]++] = a;
  }
  for (int32_t i = 0; i < n; i++)
    std::sort(adj.begin() + off[(size_t)i], adj.begin() + off[(size_t)i + 1], [&](int32_t x, int32_t y) {
      return deg[(size_t)x] != deg[(size_t)y] ? deg[(size_t)x] < deg[(size_t)y] : x < y;
    });
  std::vector<int32_t> order;
  order.reserve((size_t)n);
  std::vector<char> seen((size_t)n, 0);
  std::vector<int32_t> level((size_t)n, -1);
  auto bfs_last = [&](int32_t s) {  // farthest node from s (ties: lowest degree), for the start node
    std::vector<int32_t> q{s};
    level[(size_t)s] = 0;
    size_t h = 0;
    int32_t last = s;
    while (h < q.size()) {
      int32_t u = q[h++];
      if (level[(size_t)u] > level[(size_t)last] || (level[(size_t)u] == level[(size_t)last] && deg[(size_t)u] < deg[(size_t)last])) last = u;
      for (int64_t k = off[(size_t)u]; k < off[(size_t)u + 1]; k++) {
        int32_t v = adj[(size_t)k];
        if (level[(size_t)v] < 0) { level[(size_t)v] = level[(size_t)u] + 1; q.push_back(v); }
      }
    }
    for (int32_t u : q) level[(size_t)u] = -1;
    return last;
  };
  for (int32_t s0 = 0; s0 < n; s0++) {
    if (seen[(size_t)s0]) continue;
    int32_t s = bfs_last(bfs_last(s0));
    std::queue<int32_t> q;
    q.push(s);
    seen[(size_t)s] = 1;
    while (!q.empty()) {
      int32_t u = q.front();
      q.pop();
      order.push_back(u);
      for (int64_t k = off[(size_t)u]; k < off[(size_t)u + 1]; k++) {
        int32_t v = adj[(size_t)k];
        if (!seen[(size_t)v]) { seen[(size_t)v] = 1; q.push(v); }
      }
    }
  }
  std::reverse(order.begin(), order.end());
  perm->swap(order);
}

int validate_views(int32_t nlevels, const mgcfd_level_view* lv, bool check_maps) {
  if (nlevels < 1 || !lv) return set_error(MGCFD_ERR_INVALID, "need at least one level");
  for (int l = 0; l < nlevels; l++) {
    const mgcfd_level_view& v = lv[l];
    if (v.nnodes < 1 || v.nedges < 0 || v.nbnd < 0)
      return set_error(MGCFD_ERR_INVALID, "level " + std::to_string(l) + ": invalid set sizes");
    if (!v.coords || (v.nedges && (!v.edge_to_nodes || !v.edge_weights)) ||
        (v.nbnd && (!v.bnd_to_node || !v.bnd_group || !v.bnd_weights)))
      return set_error(MGCFD_ERR_INVALID, "level " + std::to_string(l) + ": null array");
    if (l + 1 < nlevels && !v.node_to_mg)
      return set_error(MGCFD_ERR_INVALID, "level " + std::to_string(l) + ": node_to_mg required above the coarsest level");
    if (!check_maps) continue;
    for (int64_t i = 0; i < 2 * (int64_t)v.nedges; i++)
      if (v.edge_to_nodes[i] < 0 || v.edge_to_nodes[i] >= v.nnodes)
        return set_error(MGCFD_ERR_INVALID, "level " + std::to_string(l) + ": edge-->node entry out of range");
    for (int32_t i = 0; i < v.nbnd; i++)
      if (v.bnd_to_node[i] < 0 || v.bnd_to_node[i] >= v.nnodes)
        return set_error(MGCFD_ERR_INVALID, "level " + std::to_string(l) + ": bnd_node-->node entry out of range");
    if (l + 1 < nlevels)
      for (int32_t i = 0; i < v.nnodes; i++)
        if (v.node_to_mg[i] < 0 || v.node_to_mg[i] >= lv[l + 1].nnodes)
          return set_error(MGCFD_ERR_INVALID, "level " + std::to_string(l) + ": node-->mg_node entry out of range");
  }
  return MGCFD_OK;
}

int prepare_mesh(int32_t nlevels, const mgcfd_level_view* lv, const mgcfd_freestream& ff, int renumber,
                 bool fp32_geometry, std::vector<PreparedLevel>* out) {
  int vr = validate_views(nlevels, lv, true);
  if (vr) return vr;
  out->assign((size_t)nlevels, PreparedLevel());
  const double sc = ff.smoothing_coefficient;
  for (int l = 0; l < nlevels; l++) {
    const mgcfd_level_view& v = lv[l];
    PreparedLevel& P = (*out)[(size_t)l];
    const int32_t n = v.nnodes, ne = v.nedges;
    P.n = n;
    P.ne = ne;
    // Node order.
    if (renumber == MGCFD_RENUMBER_SPATIAL) spatial_order(v.coords, n, &P.perm);
    else if (renumber == MGCFD_RENUMBER_RCM) rcm_order(n, ne, v.edge_to_nodes, &P.perm);
    else { P.perm.resize((size_t)n); for (int32_t i = 0; i < n; i++) P.perm[(size_t)i] = i; }
    P.inv.assign((size_t)n, 0);
    for (int32_t i = 0; i < n; i++) P.inv[(size_t)P.perm[(size_t)i]] = i;

    // Geometry: calculate_cell_volumes (misc.h:40-76) in input edge order,
    // then dampen_ewt (misc.h:78-84) -- the reference's sequential order.
    std::vector<double> vol_in((size_t)n, 0.0);
    std::vector<double> ewt((size_t)ne * 3);
    if (v.volumes) {  // legacy mode: volumes as read, weights not re-oriented
      for (int32_t i = 0; i < n; i++) vol_in[(size_t)i] = v.volumes[i];
      for (size_t k = 0; k < ewt.size(); k++) ewt[k] = v.edge_weights[k] * 1e-7;
    }
    for (int32_t e = 0; e < ne && !v.volumes && fp32_geometry; e++) {
      // The mixed-precision form's geometry: the same steps in FP32, from the
      // FP64 coordinate differences and input weights rounded once (the
      // device computes the same, device_setup.cu).
      const int32_t a = v.edge_to_nodes[2 * (size_t)e], b = v.edge_to_nodes[2 * (size_t)e + 1];
      float d[3], wf[3];
      for (int i = 0; i < 3; i++) {
        d[i] = (float)(v.coords[3 * (size_t)b + i] - v.coords[3 * (size_t)a + i]);
        wf[i] = (float)v.edge_weights[3 * (size_t)e + i];
      }
      const float dist = std::sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
      const float area = std::sqrt((wf[0] * wf[0] + wf[1] * wf[1]) + wf[2] * wf[2]);
      const float tv = ((float)((1.0 / 3.0) * 0.5) * dist) * area;
      vol_in[(size_t)a] += (double)tv;
      vol_in[(size_t)b] += (double)tv;
      for (int i = 0; i < 3; i++) ewt[3 * (size_t)e + i] = (double)((((d[i] / dist) * area) / dist) * 1e-7f);
    }
    for (int32_t e = 0; e < ne && !v.volumes && !fp32_geometry; e++) {
      const int32_t a = v.edge_to_nodes[2 * (size_t)e], b = v.edge_to_nodes[2 * (size_t)e + 1];
      double d[3], dist = 0.0, area = 0.0;
      for (int i = 0; i < 3; i++) {
        d[i] = v.coords[3 * (size_t)b + i] - v.coords[3 * (size_t)a + i];
        dist += d[i] * d[i];
      }
      dist = std::sqrt(dist);
      for (int i = 0; i < 3; i++) area += v.edge_weights[3 * (size_t)e + i] * v.edge_weights[3 * (size_t)e + i];
      area = std::sqrt(area);
      const double tv = (1.0 / 3.0) * 0.5 * dist * area;
      vol_in[(size_t)a] += tv;
      vol_in[(size_t)b] += tv;
      for (int i = 0; i < 3; i++) {
        double w = (d[i] / dist) * area;
        w /= dist;
        ewt[3 * (size_t)e + i] = w * 1e-7;
      }
    }
    P.vol.resize((size_t)n);
    for (int32_t i = 0; i < n; i++) P.vol[(size_t)i] = vol_in[(size_t)P.perm[(size_t)i]];

    // Edges: new ids, oriented a < b (weight negated on swap), counting sort by a, then b.
    std::vector<int32_t> na((size_t)ne), nb_((size_t)ne);
    std::vector<int32_t> cnt((size_t)n + 1, 0);
    for (int32_t e = 0; e < ne; e++) {
      int32_t a = P.inv[(size_t)v.edge_to_nodes[2 * (size_t)e]], b = P.inv[(size_t)v.edge_to_nodes[2 * (size_t)e + 1]];
      if (a > b) { std::swap(a, b); for (int i = 0; i < 3; i++) ewt[3 * (size_t)e + i] = -ewt[3 * (size_t)e + i]; }
      na[(size_t)e] = a; nb_[(size_t)e] = b;
      cnt[(size_t)a + 1]++;
    }
    for (int32_t i = 0; i < n; i++) cnt[(size_t)i + 1] += cnt[(size_t)i];
    P.a_off = cnt;
    std::vector<int32_t> order((size_t)ne);
    {
      std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
      for (int32_t e = 0; e < ne; e++) order[(size_t)fill[(size_t)na[(size_t)e]]++] = e;
    }
    for (int32_t a = 0; a < n; a++) {  // tiny buckets: insertion sort by b
      for (int32_t i = P.a_off[(size_t)a] + 1; i < P.a_off[(size_t)a + 1]; i++) {
        int32_t x = order[(size_t)i], j = i - 1;
        while (j >= P.a_off[(size_t)a] && nb_[(size_t)order[(size_t)j]] > nb_[(size_t)x]) { order[(size_t)j + 1] = order[(size_t)j]; j--; }
        order[(size_t)j + 1] = x;
      }
    }
    P.e2n.resize((size_t)ne * 2);
    P.w4.resize((size_t)ne * 4);
    for (int32_t k = 0; k < ne; k++) {
      const int32_t e = order[(size_t)k];
      P.e2n[2 * (size_t)k] = na[(size_t)e];
      P.e2n[2 * (size_t)k + 1] = nb_[(size_t)e];
      const double* w = &ewt[3 * (size_t)e];
      if (fp32_geometry) {
        const float x = (float)w[0], y = (float)w[1], z = (float)w[2];
        const float mag = std::sqrt((x * x + y * y) + z * z);
        P.w4[4 * (size_t)k + 0] = (double)(-0.5f * x);
        P.w4[4 * (size_t)k + 1] = (double)(-0.5f * y);
        P.w4[4 * (size_t)k + 2] = (double)(-0.5f * z);
        P.w4[4 * (size_t)k + 3] = (double)((-mag * (float)sc) * 0.5f);
        continue;
      }
      const double mag = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
      P.w4[4 * (size_t)k + 0] = -0.5 * w[0];  // flux.h:147 factor_x etc.
      P.w4[4 * (size_t)k + 1] = -0.5 * w[1];
      P.w4[4 * (size_t)k + 2] = -0.5 * w[2];
      P.w4[4 * (size_t)k + 3] = -mag * sc * 0.5;  // flux.h:139 factor without the speed sum
    }
    P.b_off.assign((size_t)n + 1, 0);
    for (int32_t k = 0; k < ne; k++) P.b_off[(size_t)P.e2n[2 * (size_t)k + 1] + 1]++;
    for (int32_t i = 0; i < n; i++) P.b_off[(size_t)i + 1] += P.b_off[(size_t)i];
    P.b_list.resize((size_t)ne);
    {
      std::vector<int32_t> fill(P.b_off.begin(), P.b_off.end() - 1);
      for (int32_t k = 0; k < ne; k++) P.b_list[(size_t)fill[(size_t)P.e2n[2 * (size_t)k + 1]]++] = k;
    }

    // Boundary entries folded per node: flux.h:14-39 is linear in the weight.
    std::vector<double> wff((size_t)n * 3, 0.0), wwall((size_t)n * 3, 0.0);
    std::vector<char> isb((size_t)n, 0);
    for (int32_t k = 0; k < v.nbnd; k++) {
      const int g = v.bnd_group[k];
      const int32_t node = P.inv[(size_t)v.bnd_to_node[k]];
      double* dst;
      if (g <= 2) dst = &wwall[3 * (size_t)node];
      else if (g == 3 || (g >= 4 && g <= 7)) dst = &wff[3 * (size_t)node];
      else continue;
      isb[(size_t)node] = 1;
      for (int i = 0; i < 3; i++) dst[i] += v.bnd_weights[3 * (size_t)k + i] * 1e-7;
    }
    P.bidx.assign((size_t)n, -1);
    P.nb = 0;
    for (int32_t i = 0; i < n; i++) {
      if (!isb[(size_t)i]) continue;
      P.bidx[(size_t)i] = P.nb++;
      const double* W = &wff[3 * (size_t)i];
      double row[12] = {W[0], W[1], W[2], wwall[3 * (size_t)i], wwall[3 * (size_t)i + 1], wwall[3 * (size_t)i + 2]};
      const double* fv = ff.ff_variable;
      row[6] = W[0] * fv[1] + W[1] * fv[2] + W[2] * fv[3];
      const double* rows[4] = {ff.ff_flux_contribution_momentum_x, ff.ff_flux_contribution_momentum_y,
                               ff.ff_flux_contribution_momentum_z, ff.ff_flux_contribution_density_energy};
      for (int r = 0; r < 4; r++) row[7 + r] = W[0] * rows[r][0] + W[1] * rows[r][1] + W[2] * rows[r][2];
      row[11] = 0.0;
      P.bdata.insert(P.bdata.end(), row, row + 12);
    }
  }

  // Multigrid tables (need both levels' orders).
  for (int l = 0; l + 1 < nlevels; l++) {
    PreparedLevel& F = (*out)[(size_t)l];
    PreparedLevel& Cl = (*out)[(size_t)l + 1];
    const mgcfd_level_view& vf = lv[l];
    const mgcfd_level_view& vc = lv[l + 1];
    F.n2mg.resize((size_t)F.n);
    F.dvec.resize((size_t)F.n * 4);
    Cl.ch_off.assign((size_t)Cl.n + 1, 0);
    for (int32_t f = 0; f < F.n; f++) {
      const int32_t fin = F.perm[(size_t)f];
      const int32_t cin = vf.node_to_mg[fin];
      const int32_t c = Cl.inv[(size_t)cin];
      F.n2mg[(size_t)f] = c;
      Cl.ch_off[(size_t)c + 1]++;
      const double* x = &vf.coords[3 * (size_t)fin];
      const double* xa = &vc.coords[3 * (size_t)cin];
      const double dx = std::fabs(x[0] - xa[0]), dy = std::fabs(x[1] - xa[1]), dz = std::fabs(x[2] - xa[2]);
      F.dvec[4 * (size_t)f + 0] = dx;
      F.dvec[4 * (size_t)f + 1] = dy;
      F.dvec[4 * (size_t)f + 2] = dz;
      F.dvec[4 * (size_t)f + 3] = std::sqrt(dx * dx + dy * dy + dz * dz);  // mg.h:76
    }
    for (int32_t c = 0; c < Cl.n; c++) Cl.ch_off[(size_t)c + 1] += Cl.ch_off[(size_t)c];
    Cl.ch_list.resize((size_t)F.n);
    std::vector<int32_t> fill(Cl.ch_off.begin(), Cl.ch_off.end() - 1);
    for (int32_t f = 0; f < F.n; f++) Cl.ch_list[(size_t)fill[(size_t)F.n2mg[(size_t)f]]++] = f;
  }
  return MGCFD_OK;
}

}  // namespace mgcfd
