// Host construction of the two-level preconditioner's coarse space: spatial
// clusters of rig instances, their coupling graph, a distance-2 colouring
// and the similarity modes (see coarse_space.h).
#include "coarse_space.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <numeric>
#include <thread>

namespace gbba {
namespace {

// Inverse of the left Jacobian of SO(3) at angle-axis phi (row-major 3 x 3):
// I - [phi]x / 2 + (1/t^2 - (1 + cos t) / (2 t sin t)) [phi]x^2, t = |phi|
// (the closed form of the Lie-group literature; the coefficient tends to
// 1/12 as t -> 0).
void left_jacobian_inverse(const double* phi, double* J) {
  const double t2 = phi[0] * phi[0] + phi[1] * phi[1] + phi[2] * phi[2];
  const double t = std::sqrt(t2);
  double c = 1.0 / 12.0;
  if (t > 1e-4) c = 1.0 / t2 - (1.0 + std::cos(t)) / (2.0 * t * std::sin(t));
  const double K[9] = {0.0, -phi[2], phi[1], phi[2], 0.0, -phi[0], -phi[1], phi[0], 0.0};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double k2 = 0.0;
      for (int m = 0; m < 3; ++m) k2 += K[3 * i + m] * K[3 * m + j];
      J[3 * i + j] = (i == j ? 1.0 : 0.0) - 0.5 * K[3 * i + j] + c * k2;
    }
}

// Recursive median splits along the widest axis of the centres until every
// part has at most `leaf` members; labels parts in split order (spatially
// coherent numbering).
void split(const std::vector<std::array<double, 3>>& c, std::vector<int>& idx, int lo, int hi, int leaf,
           std::vector<int>& label, int& next) {
  if (hi - lo <= leaf) {
    for (int i = lo; i < hi; ++i) label[idx[i]] = next;
    ++next;
    return;
  }
  double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
  for (int i = lo; i < hi; ++i)
    for (int k = 0; k < 3; ++k) {
      mn[k] = std::min(mn[k], c[idx[i]][k]);
      mx[k] = std::max(mx[k], c[idx[i]][k]);
    }
  int ax = 0;
  for (int k = 1; k < 3; ++k)
    if (mx[k] - mn[k] > mx[ax] - mn[ax]) ax = k;
  const int mid = lo + (hi - lo) / 2;
  std::nth_element(idx.begin() + lo, idx.begin() + mid, idx.begin() + hi, [&](int a, int b) {
    return c[a][ax] < c[b][ax] || (c[a][ax] == c[b][ax] && a < b);
  });
  split(c, idx, lo, mid, leaf, label, next);
  split(c, idx, mid, hi, leaf, label, next);
}

}  // namespace

CoarseSpace build_coarse_space(const Problem& P, const std::vector<uint8_t>& free_mask, int leaf,
                               const std::vector<int64_t>& point_major) {
  CoarseSpace cs;
  const int n_inst = int(P.instances.size());
  cs.cluster.assign(n_inst, -1);
  if (leaf < 1 || n_inst < 2) return cs;
  std::vector<int> active;
  std::vector<std::array<double, 3>> centre(n_inst);
  for (int i = 0; i < n_inst; ++i) {
    bool any = false;
    for (int k = 0; k < 6; ++k) any |= free_mask[6 * size_t(i) + k] != 0;
    bool finite = true;
    for (int k = 0; k < 6; ++k) finite &= std::isfinite(P.instances[i].value[k]);
    for (int k = 0; k < 3; ++k) centre[i][k] = P.instances[i].value[3 + k];
    // an instance without a free coordinate (or with a non-finite pose, which
    // the median splits could not order) joins no cluster
    if (any && finite) active.push_back(i);
  }
  const int na = int(active.size());
  if (na < 2) return cs;
  // clusters: grow the leaf until the coarse system fits the dense solver
  int L = std::max(leaf, (7 * na + kMaxCoarseDim - 1) / kMaxCoarseDim);
  std::vector<int> label(n_inst, -1);
  int nc = 0;
  for (;;) {
    std::vector<int> idx = active;
    nc = 0;
    split(centre, idx, 0, na, L, label, nc);
    if (7 * nc <= kMaxCoarseDim) break;
    L *= 2;
  }
  if (nc < 2) return cs;
  cs.leaf = L;
  cs.n_clusters = nc;
  for (int i : active) cs.cluster[i] = label[i];
  cs.member_start.assign(nc + 1, 0);
  for (int i : active) ++cs.member_start[cs.cluster[i] + 1];
  for (int c = 0; c < nc; ++c) cs.member_start[c + 1] += cs.member_start[c];
  cs.members.resize(active.size());
  {
    std::vector<int> fill(cs.member_start.begin(), cs.member_start.end() - 1);
    for (int i : active) cs.members[fill[cs.cluster[i]]++] = i;
  }

  // coupling graph: clusters that observe a common point, or whose
  // instances share a host term
  std::vector<std::vector<uint64_t>> adj(nc, std::vector<uint64_t>((nc + 63) / 64, 0));
  auto link = [&](int a, int b) {
    if (a < 0 || b < 0 || a == b) return;
    adj[a][b >> 6] |= uint64_t(1) << (b & 63);
    adj[b][a >> 6] |= uint64_t(1) << (a & 63);
  };
  auto cluster_of_obs = [&](const Observation& o) {
    const int inst = (o.shot >= 0 && size_t(o.shot) < P.shots.size()) ? P.shots[o.shot].instance : -1;
    return inst >= 0 ? cs.cluster[inst] : -1;
  };
  {
    // host threads over ranges of whole points, each with its own bitset
    const std::vector<int64_t>& pm = point_major;
    const size_t n_pm = pm.size();
    const int n_thr = int(std::max<size_t>(1, std::min<size_t>(16, std::min<size_t>(
                                                  std::thread::hardware_concurrency(), n_pm / 65536 + 1))));
    auto point_of = [&](size_t q) {
      const int64_t o = pm[q];
      return (o < 0 || size_t(o) >= P.observations.size()) ? -1 : P.observations[size_t(o)].point;
    };
    std::vector<size_t> cut(n_thr + 1, n_pm);
    cut[0] = 0;
    for (int k = 1; k < n_thr; ++k) {
      size_t q = std::max(cut[k - 1], n_pm * size_t(k) / size_t(n_thr));
      // advance to the first entry of a new point (entries without an
      // observation may sit inside a point's run)
      int prev = -2;
      for (size_t b = q; b > cut[k - 1]; --b)
        if (point_of(b - 1) >= 0) {
          prev = point_of(b - 1);
          break;
        }
      while (q < n_pm && (point_of(q) < 0 || point_of(q) == prev)) ++q;
      cut[k] = q;
    }
    const size_t words = (size_t(nc) + 63) / 64;
    std::vector<std::vector<uint64_t>> part(n_thr, std::vector<uint64_t>(size_t(nc) * words, 0));
    auto work = [&](int k) {
      std::vector<uint64_t>& a = part[k];
      std::vector<int> s;
      auto flush = [&]() {
        if (s.size() < 2) return;
        std::sort(s.begin(), s.end());
        s.erase(std::unique(s.begin(), s.end()), s.end());
        for (size_t x = 0; x < s.size(); ++x)
          for (size_t y = x + 1; y < s.size(); ++y) {
            a[size_t(s[x]) * words + (s[y] >> 6)] |= uint64_t(1) << (s[y] & 63);
            a[size_t(s[y]) * words + (s[x] >> 6)] |= uint64_t(1) << (s[x] & 63);
          }
      };
      int cur = -1;
      for (size_t q = cut[k]; q < cut[k + 1]; ++q) {
        const int64_t o = pm[q];
        if (o < 0 || size_t(o) >= P.observations.size()) continue;
        const Observation& ob = P.observations[size_t(o)];
        if (ob.point != cur) {
          flush();
          s.clear();
          cur = ob.point;
        }
        const int c = cluster_of_obs(ob);
        if (c >= 0) s.push_back(c);
      }
      flush();
    };
    std::vector<std::thread> pool;
    for (int k = 1; k < n_thr; ++k) pool.emplace_back(work, k);
    work(0);
    for (std::thread& th : pool) th.join();
    for (int k = 0; k < n_thr; ++k)
      for (int a = 0; a < nc; ++a)
        for (size_t w = 0; w < words; ++w) adj[a][w] |= part[k][size_t(a) * words + w];
  }
  for (const RelativeTerm& t : P.relative_terms)
    for (int a = 0; a < t.n_shots; ++a)
      for (int b = a + 1; b < t.n_shots; ++b) {
        const int ia = t.instance[a], ib = t.instance[b];
        if (ia >= 0 && ia < n_inst && ib >= 0 && ib < n_inst) link(cs.cluster[ia], cs.cluster[ib]);
      }
  cs.neighbours.assign(nc, {});
  for (int a = 0; a < nc; ++a)
    for (int b = 0; b < nc; ++b)
      if ((adj[a][b >> 6] >> (b & 63)) & 1) cs.neighbours[a].push_back(b);

  // greedy distance-2 colouring: a cluster takes the smallest colour not
  // used within two steps of it
  cs.colour.assign(nc, -1);
  for (int c = 0; c < nc; ++c) {
    std::vector<char> used(size_t(cs.n_colours) + 1, 0);
    auto mark = [&](int x) {
      if (cs.colour[x] >= 0) used[cs.colour[x]] = 1;
    };
    for (int a : cs.neighbours[c]) {
      mark(a);
      for (int b : cs.neighbours[a]) mark(b);
    }
    int k = 0;
    while (used[k]) ++k;
    cs.colour[c] = k;
    cs.n_colours = std::max(cs.n_colours, k + 1);
  }
  cs.partner.assign(size_t(nc) * cs.n_colours, -1);
  for (int c = 0; c < nc; ++c) {
    cs.partner[size_t(c) * cs.n_colours + cs.colour[c]] = c;
    for (int a : cs.neighbours[c]) cs.partner[size_t(c) * cs.n_colours + cs.colour[a]] = a;
  }

  // similarity modes about each cluster's centroid
  std::vector<std::array<double, 3>> g(nc, {0.0, 0.0, 0.0});
  std::vector<int> count(nc, 0);
  for (int i : active) {
    const int c = cs.cluster[i];
    for (int k = 0; k < 3; ++k) g[c][k] += centre[i][k];
    ++count[c];
  }
  for (int c = 0; c < nc; ++c)
    for (int k = 0; k < 3; ++k) g[c][k] /= double(count[c]);
  cs.basis.assign(size_t(n_inst) * 42, 0.0);
  for (int i : active) {
    const int c = cs.cluster[i];
    double* Z = cs.basis.data() + size_t(i) * 42;  // Z[a * 7 + j]
    double J[9];
    left_jacobian_inverse(P.instances[i].value, J);
    const double d[3] = {centre[i][0] - g[c][0], centre[i][1] - g[c][1], centre[i][2] - g[c][2]};
    for (int k = 0; k < 3; ++k) {
      Z[(3 + k) * 7 + k] = 1.0;  // translation
      for (int a = 0; a < 3; ++a) Z[a * 7 + 3 + k] = J[3 * a + k];
      // e_k x d
      const double e[3] = {k == 0 ? 1.0 : 0.0, k == 1 ? 1.0 : 0.0, k == 2 ? 1.0 : 0.0};
      const double x[3] = {e[1] * d[2] - e[2] * d[1], e[2] * d[0] - e[0] * d[2], e[0] * d[1] - e[1] * d[0]};
      for (int a = 0; a < 3; ++a) Z[(3 + a) * 7 + 3 + k] = x[a];
      Z[(3 + k) * 7 + 6] = d[k];  // scale
    }
    for (int a = 0; a < 6; ++a)
      if (!free_mask[6 * size_t(i) + a])
        for (int j = 0; j < 7; ++j) Z[a * 7 + j] = 0.0;
  }
  return cs;
}

std::vector<int64_t> point_major_order(const Problem& P) {
  const size_t n_pts = P.points.size();
  std::vector<int64_t> start(n_pts + 1, 0);
  for (const Observation& o : P.observations)
    if (o.point >= 0 && size_t(o.point) < n_pts) ++start[o.point + 1];
  for (size_t p = 0; p < n_pts; ++p) start[p + 1] += start[p];
  std::vector<int64_t> order(static_cast<size_t>(start[n_pts]));
  for (size_t i = 0; i < P.observations.size(); ++i) {
    const int p = P.observations[i].point;
    if (p >= 0 && size_t(p) < n_pts) order[size_t(start[p]++)] = int64_t(i);
  }
  return order;
}

}  // namespace gbba
