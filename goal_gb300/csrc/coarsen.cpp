// Coarsening of a tetrahedral mesh to a target size field by edge collapse,
// the coarsening half of goal's adaptation loop (src/main_nested.cpp:106-126,
// which calls SCOREC ma::adapt -- not part of the reference tree). An edge
// (a, b) shorter than ratio x (mean target size of its end points) is
// collapsed by moving b onto a. A collapse is taken only if it keeps the
// model: the node / side sets b belongs to (node_class bits) are a subset of
// a's, b is not on an element-set interface, a boundary b is on a flat part of
// the boundary and (a, b) is a boundary edge; and only if it keeps the mesh
// valid: the link condition (no fold-over of the topology), every remaining
// tet around b positively oriented with mean-ratio quality at least
// min(min_quality, the worst quality around b before), and no new edge longer
// than refine_ratio x its mean target size (the refinement would split it
// again). Candidates go shortest (relative to size) first, one independent set
// of collapses per pass; ties break on the end-point pair, so the result is
// deterministic.
//
// Host code: a sequence of local topological updates; the discretization built
// from its output goes back to the GPU.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <memory>
#include <vector>

#include "../../include/goal_gb300.h"
#include "common.cuh"

namespace goal {
namespace {

constexpr long long kBoundaryBit = 1ll << 62;

inline uint64_t ekey(int a, int b) {
  const uint64_t lo = (uint64_t)(unsigned)std::min(a, b), hi = (uint64_t)(unsigned)std::max(a, b);
  return (hi << 32) | lo;
}

struct Coarsener {
  int N = 0;
  std::vector<double> X;
  std::vector<long long> cls;
  std::vector<double> size;
  std::vector<char> valive;
  std::vector<std::array<int, 4>> T;
  std::vector<int> eset;
  std::vector<int> origin;  // original element of each tet (swaps make new ones)
  std::vector<char> talive;
  // quality of every live tet at the start of a coarsening pass: a collapse
  // changes only tets whose vertices it marks touched, so the tets around an
  // untouched vertex keep these values for the rest of the pass
  std::vector<double> tq;
  std::vector<std::vector<int>> vt;  // vertex -> tets (live ones; dead entries are filtered on use)
  // boundary faces (faces of exactly one tet) and side triangles
  std::vector<std::array<int, 3>> F;
  std::vector<char> falive;
  std::vector<std::vector<int>> vf;
  std::vector<std::array<int, 3>> S;
  std::vector<int> S_set;
  std::vector<char> salive;
  std::vector<std::vector<int>> vs;
  // nodal transfer of smoothing: a moved node's value is a combination of
  // original nodes' values (empty: the node itself)
  std::vector<std::vector<std::pair<int, double>>> W;

  double len2(int a, int b) const {
    const double dx = X[3 * a] - X[3 * b], dy = X[3 * a + 1] - X[3 * b + 1], dz = X[3 * a + 2] - X[3 * b + 2];
    return dx * dx + dy * dy + dz * dz;
  }
  // signed volume x 6 and mean-ratio quality 12 (3|V|)^(2/3) / sum l^2
  double vol6(const std::array<int, 4>& v) const {
    const double* p0 = &X[3 * v[0]];
    double e[3][3];
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) e[k][c] = X[3 * v[k + 1] + c] - p0[c];
    return e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) - e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
           e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
  }
  double quality(const std::array<int, 4>& v) const {
    const double V = vol6(v) / 6.0;
    double l2 = 0.0;
    for (int i = 0; i < 4; ++i)
      for (int j = i + 1; j < 4; ++j) l2 += len2(v[i], v[j]);
    if (!(V > 0.0) || !(l2 > 0.0)) return 0.0;
    return 12.0 * std::cbrt(9.0 * V * V) / l2;
  }
  static void compact(std::vector<int>& list, const std::vector<char>& alive) {
    list.erase(std::remove_if(list.begin(), list.end(), [&](int t) { return !alive[t]; }), list.end());
  }
  bool has(const std::array<int, 4>& v, int x) const { return v[0] == x || v[1] == x || v[2] == x || v[3] == x; }
  static bool has3(const std::array<int, 3>& v, int x) { return v[0] == x || v[1] == x || v[2] == x; }
  bool boundary(int v) const { return (cls[v] & kBoundaryBit) != 0; }

  void normal(const std::array<int, 3>& f, double n[3]) const {
    double u[3], w[3];
    for (int c = 0; c < 3; ++c) {
      u[c] = X[3 * f[1] + c] - X[3 * f[0] + c];
      w[c] = X[3 * f[2] + c] - X[3 * f[0] + c];
    }
    n[0] = u[1] * w[2] - u[2] * w[1];
    n[1] = u[2] * w[0] - u[0] * w[2];
    n[2] = u[0] * w[1] - u[1] * w[0];
    const double m = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int c = 0; c < 3; ++c) n[c] = m > 0.0 ? n[c] / m : 0.0;
  }

  // vertices sharing a live tet with v
  void adjacent(int v, std::vector<int>& out) const {
    out.clear();
    for (int t : vt[v])
      if (talive[t])
        for (int x : T[t])
          if (x != v) out.push_back(x);
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
  }

  // can b be moved onto a?
  bool can_collapse(int b, int a, double refine_ratio, double min_quality) const {
    if ((cls[b] & ~cls[a]) != 0) return false;
    // element sets: b inside one set
    int es = -1;
    for (int t : vt[b]) {
      if (!talive[t]) continue;
      if (es < 0) es = eset[t];
      else if (eset[t] != es) return false;
    }
    // boundary b: flat, and (a, b) a boundary edge
    if (boundary(b)) {
      bool edge_on_boundary = false;
      double n0[3] = {0, 0, 0};
      bool first = true;
      for (int f : vf[b]) {
        if (!falive[f]) continue;
        if (has3(F[f], a)) edge_on_boundary = true;
        double n[3];
        normal(F[f], n);
        if (first) {
          for (int c = 0; c < 3; ++c) n0[c] = n[c];
          first = false;
        } else if (std::fabs(n[0] * n0[0] + n[1] * n0[1] + n[2] * n0[2]) < 1.0 - 1e-10) {
          return false;
        }
      }
      if (!edge_on_boundary) return false;
    }
    thread_local std::vector<int> adj_a, adj_b, common, lab;
    thread_local std::vector<uint64_t> elab, ea, eb;
    adjacent(b, adj_b);
    if (!std::binary_search(adj_b.begin(), adj_b.end(), a)) return false;
    // no new edge too long (checked first: it needs no tet quality)
    for (int c : adj_b) {
      if (c == a) continue;
      const double s = refine_ratio * 0.5 * (size[a] + size[c]);
      if (len2(a, c) > s * s) return false;
    }
    // geometry: the tets that keep b (as a) stay valid and good enough
    double worst = 1.0;
    for (int t : vt[b])
      if (talive[t]) worst = std::min(worst, tq[t]);
    const double qmin = std::min(min_quality, worst);
    for (int t : vt[b]) {
      if (!talive[t] || has(T[t], a)) continue;
      std::array<int, 4> v = T[t];
      for (int& x : v)
        if (x == b) x = a;
      if (!(vol6(v) > 0.0) || quality(v) < qmin) return false;
    }
    // link condition: the vertices adjacent to both a and b are exactly the
    // vertices of the tets around edge ab; edges (c, d) seen from both a and b
    // must belong to a tet around ab
    adjacent(a, adj_a);
    common.clear();
    std::set_intersection(adj_a.begin(), adj_a.end(), adj_b.begin(), adj_b.end(), std::back_inserter(common));
    lab.clear();
    elab.clear();
    for (int t : vt[b]) {
      if (!talive[t] || !has(T[t], a)) continue;
      int cd[2], k = 0;
      for (int x : T[t])
        if (x != a && x != b) cd[k++] = x;
      lab.push_back(cd[0]);
      lab.push_back(cd[1]);
      elab.push_back(ekey(cd[0], cd[1]));
    }
    std::sort(lab.begin(), lab.end());
    lab.erase(std::unique(lab.begin(), lab.end()), lab.end());
    if (common != lab) return false;
    {
      std::sort(elab.begin(), elab.end());
      ea.clear();
      eb.clear();
      for (int t : vt[a]) {
        if (!talive[t] || has(T[t], b)) continue;
        int cd[3], k = 0;
        for (int x : T[t])
          if (x != a) cd[k++] = x;
        ea.push_back(ekey(cd[0], cd[1]));
        ea.push_back(ekey(cd[0], cd[2]));
        ea.push_back(ekey(cd[1], cd[2]));
      }
      for (int t : vt[b]) {
        if (!talive[t] || has(T[t], a)) continue;
        int cd[3], k = 0;
        for (int x : T[t])
          if (x != b) cd[k++] = x;
        eb.push_back(ekey(cd[0], cd[1]));
        eb.push_back(ekey(cd[0], cd[2]));
        eb.push_back(ekey(cd[1], cd[2]));
      }
      std::sort(ea.begin(), ea.end());
      std::sort(eb.begin(), eb.end());
      size_t i = 0, j = 0;
      while (i < ea.size() && j < eb.size()) {
        if (ea[i] < eb[j]) ++i;
        else if (eb[j] < ea[i]) ++j;
        else {
          if (!std::binary_search(elab.begin(), elab.end(), ea[i])) return false;
          ++i;
          ++j;
        }
      }
    }
    // the same on the boundary surface: a boundary vertex c joined to both a
    // and b by boundary edges must make a boundary face with them
    if (boundary(a) && boundary(b)) {
      std::vector<int> ca, cb, fab;
      for (int f : vf[a])
        if (falive[f] && !has3(F[f], b))
          for (int x : F[f])
            if (x != a) ca.push_back(x);
      for (int f : vf[b])
        if (falive[f]) {
          if (has3(F[f], a)) {
            for (int x : F[f])
              if (x != a && x != b) fab.push_back(x);
          } else {
            for (int x : F[f])
              if (x != b) cb.push_back(x);
          }
        }
      std::sort(ca.begin(), ca.end());
      std::sort(cb.begin(), cb.end());
      std::vector<int> both;
      std::set_intersection(ca.begin(), ca.end(), cb.begin(), cb.end(), std::back_inserter(both));
      for (int c : both)
        if (std::find(fab.begin(), fab.end(), c) == fab.end()) return false;
    }
    return true;
  }

  void collapse(int b, int a) {
    for (int t : vt[b]) {
      if (!talive[t]) continue;
      if (has(T[t], a)) {
        talive[t] = 0;
        continue;
      }
      for (int& x : T[t])
        if (x == b) x = a;
      vt[a].push_back(t);
    }
    vt[b].clear();
    for (int f : vf[b]) {
      if (!falive[f]) continue;
      if (has3(F[f], a)) {
        falive[f] = 0;
        continue;
      }
      for (int& x : F[f])
        if (x == b) x = a;
      vf[a].push_back(f);
    }
    vf[b].clear();
    for (int f : vs[b]) {
      if (!salive[f]) continue;
      if (has3(S[f], a)) {
        salive[f] = 0;
        continue;
      }
      for (int& x : S[f])
        if (x == b) x = a;
      vs[a].push_back(f);
    }
    vs[b].clear();
    valive[b] = 0;
    compact(vt[a], talive);
    compact(vf[a], falive);
    compact(vs[a], salive);
  }

  // ----- shape improvement by flips (nodes fixed) -----
  // tets around edge (d, e)
  void edge_tets(int d, int e, std::vector<int>& out) const {
    out.clear();
    for (int t : vt[d])
      if (talive[t] && has(T[t], e)) out.push_back(t);
  }
  bool boundary_edge(int d, int e) const {
    for (int f : vf[d])
      if (falive[f] && has3(F[f], e)) return true;
    return false;
  }
  bool side_edge(int d, int e) const {
    for (int f : vs[d])
      if (salive[f] && has3(S[f], e)) return true;
    return false;
  }
  bool side_face(int a, int b, int c) const {
    for (int f : vs[a])
      if (salive[f] && has3(S[f], b) && has3(S[f], c)) return true;
    return false;
  }
  // the tet across face (a, b, c) of t, or -1
  int across(int t, int a, int b, int c) const {
    for (int u : vt[a])
      if (u != t && talive[u] && has(T[u], b) && has(T[u], c)) return u;
    return -1;
  }
  std::array<int, 4> oriented(int a, int b, int c, int d) const {
    std::array<int, 4> v = {a, b, c, d};
    if (vol6(v) < 0.0) std::swap(v[2], v[3]);
    return v;
  }
  // the old tet (of ts) that contains the centroid of v best
  int donor(const std::array<int, 4>& v, const std::vector<int>& ts) const {
    double cen[3] = {0, 0, 0};
    for (int x : v)
      for (int c = 0; c < 3; ++c) cen[c] += 0.25 * X[3 * x + c];
    int best = ts[0];
    double best_b = -1e300;
    for (int t : ts) {
      // barycentric coordinates of cen in T[t]: the smallest one
      const auto& w = T[t];
      const double V = vol6(w);
      double bmin = 1e300;
      for (int k = 0; k < 4; ++k) {
        std::array<double, 12> P;
        for (int q = 0; q < 4; ++q)
          for (int c = 0; c < 3; ++c) P[3 * q + c] = (q == k) ? cen[c] : X[3 * w[q] + c];
        double e[3][3];
        for (int q = 0; q < 3; ++q)
          for (int c = 0; c < 3; ++c) e[q][c] = P[3 * (q + 1) + c] - P[c];
        const double vk = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) -
                          e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
                          e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
        bmin = std::min(bmin, vk / V);
      }
      if (bmin > best_b) { best_b = bmin; best = t; }
    }
    return best;
  }
  void replace(const std::vector<int>& old, const std::vector<std::array<int, 4>>& nu) {
    std::vector<int> org;
    for (const auto& v : nu) org.push_back(origin[donor(v, old)]);
    const int es = eset[old[0]];
    for (int t : old) talive[t] = 0;
    for (size_t k = 0; k < nu.size(); ++k) {
      const int id = (int)T.size();
      T.push_back(nu[k]);
      eset.push_back(es);
      origin.push_back(org[k]);
      talive.push_back(1);
      for (int x : nu[k]) vt[x].push_back(id);
    }
    for (const auto& v : nu)
      for (int x : v) compact(vt[x], talive);
  }
  // best flip touching tet t; returns the new min quality (0: none found)
  double best_flip(int t, std::vector<int>& old, std::vector<std::array<int, 4>>& nu) const {
    const double q0 = quality(T[t]);
    double best = q0 * (1.0 + 1e-3);
    bool found = false;
    std::vector<int> ring;
    const auto v = T[t];
    // 3-2: an interior edge with three tets around it
    for (int i = 0; i < 4; ++i)
      for (int j = i + 1; j < 4; ++j) {
        const int d = v[i], e = v[j];
        if (boundary_edge(d, e) || side_edge(d, e)) continue;
        edge_tets(d, e, ring);
        if (ring.size() != 3) continue;
        if (eset[ring[0]] != eset[ring[1]] || eset[ring[0]] != eset[ring[2]]) continue;
        std::vector<int> oth;
        double qold = 1.0;
        for (int u : ring) {
          qold = std::min(qold, quality(T[u]));
          for (int x : T[u])
            if (x != d && x != e) oth.push_back(x);
        }
        std::sort(oth.begin(), oth.end());
        oth.erase(std::unique(oth.begin(), oth.end()), oth.end());
        if (oth.size() != 3) continue;
        const int a = oth[0], b = oth[1], c = oth[2];
        // the new face must not exist already
        bool exists = false;
        for (int u : vt[a])
          if (talive[u] && has(T[u], b) && has(T[u], c) && std::find(ring.begin(), ring.end(), u) == ring.end())
            exists = true;
        if (exists) continue;
        // d-e must cross the triangle abc's interior (then the two new tets
        // fill exactly the three old ones)
        const std::array<int, 4> s1 = {a, b, d, e}, s2 = {b, c, d, e}, s3 = {c, a, d, e};
        const double v1 = vol6(s1), v2 = vol6(s2), v3 = vol6(s3);
        if (!((v1 > 0 && v2 > 0 && v3 > 0) || (v1 < 0 && v2 < 0 && v3 < 0))) continue;
        const auto n1 = oriented(a, b, c, d), n2 = oriented(a, b, c, e);
        if (!(vol6(n1) > 0.0) || !(vol6(n2) > 0.0)) continue;
        const double qn = std::min(quality(n1), quality(n2));
        if (qn > best && qn > qold) {
          best = qn;
          old = ring;
          nu = {n1, n2};
          found = true;
        }
      }
    // 2-3: an interior face shared with a tet of the same set
    static const int kF[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
    for (int k = 0; k < 4; ++k) {
      const int a = v[kF[k][0]], b = v[kF[k][1]], c = v[kF[k][2]], d = v[k];
      if (side_face(a, b, c)) continue;
      const int u = across(t, a, b, c);
      if (u < 0 || eset[u] != eset[t]) continue;
      int e = -1;
      for (int x : T[u])
        if (x != a && x != b && x != c) e = x;
      if (e < 0 || e == d) continue;
      // the new edge (d, e) must not exist already
      bool exists = false;
      for (int w : vt[d])
        if (talive[w] && has(T[w], e)) exists = true;
      if (exists) continue;
      const std::array<int, 4> s1 = {a, b, d, e}, s2 = {b, c, d, e}, s3 = {c, a, d, e};
      const double v1 = vol6(s1), v2 = vol6(s2), v3 = vol6(s3);
      // d-e crosses the face's interior: the three have one strict sign
      if (!((v1 > 0 && v2 > 0 && v3 > 0) || (v1 < 0 && v2 < 0 && v3 < 0))) continue;
      const auto n1 = oriented(a, b, d, e), n2 = oriented(b, c, d, e), n3 = oriented(c, a, d, e);
      const double qold = std::min(q0, quality(T[u]));
      const double qn = std::min(quality(n1), std::min(quality(n2), quality(n3)));
      if (qn > best && qn > qold) {
        best = qn;
        old = {t, u};
        nu = {n1, n2, n3};
        found = true;
      }
    }
    return found ? best : 0.0;
  }
  // ----- vertex smoothing (interior nodes of one element set) -----
  double star_quality(int v) const {
    double q = 1.0;
    for (int t : vt[v])
      if (talive[t]) q = std::min(q, quality(T[t]));
    return q;
  }
  std::vector<std::pair<int, double>> row(int v) const {
    if (W[v].empty()) return {{v, 1.0}};
    return W[v];
  }
  // moves v to p if every tet of its star stays positive and the star's
  // minimum quality rises; the value at v becomes the old field at p
  bool try_move(int v, const double p[3]) {
    const double keep[3] = {X[3 * v], X[3 * v + 1], X[3 * v + 2]};
    const double q0 = star_quality(v);
    // barycentric coordinates of p in the old star (before moving)
    int host = -1;
    double lam[4] = {0, 0, 0, 0};
    double best = -1e300;
    for (int t : vt[v]) {
      if (!talive[t]) continue;
      const auto& w = T[t];
      const double V = vol6(w);
      double l[4], lmin = 1e300;
      for (int k = 0; k < 4; ++k) {
        double e[3][3];
        double P[4][3];
        for (int q = 0; q < 4; ++q)
          for (int c = 0; c < 3; ++c) P[q][c] = (q == k) ? p[c] : X[3 * w[q] + c];
        for (int q = 0; q < 3; ++q)
          for (int c = 0; c < 3; ++c) e[q][c] = P[q + 1][c] - P[0][c];
        l[k] = (e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) - e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
                e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0])) / V;
        lmin = std::min(lmin, l[k]);
      }
      if (lmin > best) {
        best = lmin;
        host = t;
        for (int k = 0; k < 4; ++k) lam[k] = l[k];
      }
    }
    if (host < 0 || best < -1e-12) return false;
    for (int c = 0; c < 3; ++c) X[3 * v + c] = p[c];
    bool ok = true;
    double q1 = 1.0;
    for (int t : vt[v]) {
      if (!talive[t]) continue;
      if (!(vol6(T[t]) > 0.0)) { ok = false; break; }
      q1 = std::min(q1, quality(T[t]));
    }
    if (!ok || !(q1 > q0 * (1.0 + 1e-6))) {
      for (int c = 0; c < 3; ++c) X[3 * v + c] = keep[c];
      return false;
    }
    // compose the transfer rows (duplicates merged, order by node id)
    std::vector<std::pair<int, double>> acc;
    for (int k = 0; k < 4; ++k) {
      if (lam[k] == 0.0) continue;
      for (const auto& pr : row(T[host][k])) acc.push_back({pr.first, lam[k] * pr.second});
    }
    std::sort(acc.begin(), acc.end());
    std::vector<std::pair<int, double>> merged;
    for (const auto& pr : acc) {
      if (!merged.empty() && merged.back().first == pr.first) merged.back().second += pr.second;
      else merged.push_back(pr);
    }
    W[v] = merged;
    return true;
  }
  int smooth_pass(double target_quality) {
    std::vector<std::pair<double, int>> cand;
    for (int v = 0; v < N; ++v) {
      if (!valive[v] || cls[v] != 0) continue;  // interior, in no node or side set
      int es = -1;
      bool one = true;
      for (int t : vt[v]) {
        if (!talive[t]) continue;
        if (es < 0) es = eset[t];
        else if (eset[t] != es) one = false;
      }
      if (!one || es < 0) continue;
      const double q = star_quality(v);
      if (q < target_quality) cand.push_back({q, v});
    }
    std::sort(cand.begin(), cand.end());
    std::vector<char> touched(N, 0);
    std::vector<int> adj;
    int done = 0;
    for (const auto& qv : cand) {
      const int v = qv.second;
      if (touched[v]) continue;
      adjacent(v, adj);
      bool skip = false;
      for (int x : adj) skip |= touched[x] != 0;
      if (skip || adj.empty()) continue;
      double p[3] = {0, 0, 0};
      for (int x : adj)
        for (int c = 0; c < 3; ++c) p[c] += X[3 * x + c] / (double)adj.size();
      bool moved = try_move(v, p);
      if (!moved) {
        for (int c = 0; c < 3; ++c) p[c] = 0.5 * (p[c] + X[3 * v + c]);
        moved = try_move(v, p);
      }
      if (!moved) continue;
      touched[v] = 1;
      for (int x : adj) touched[x] = 1;
      ++done;
    }
    return done;
  }

  int swap_pass(double target_quality) {
    std::vector<std::pair<double, int>> bad;
    for (size_t t = 0; t < T.size(); ++t)
      if (talive[t]) {
        const double q = quality(T[t]);
        if (q < target_quality) bad.push_back({q, (int)t});
      }
    std::sort(bad.begin(), bad.end());
    std::vector<char> touched(N, 0);
    std::vector<int> old;
    std::vector<std::array<int, 4>> nu;
    int done = 0;
    for (const auto& qt : bad) {
      const int t = qt.second;
      if (!talive[t]) continue;
      bool skip = false;
      for (int x : T[t]) skip |= touched[x] != 0;
      if (skip) continue;
      if (best_flip(t, old, nu) <= 0.0) continue;
      for (int u : old)
        for (int x : T[u]) touched[x] = 1;
      replace(old, nu);
      ++done;
    }
    return done;
  }

  int pass(double ratio, double refine_ratio, double min_quality) {
    struct Cand {
      double r;
      uint64_t key;
    };
    std::vector<Cand> cand;
    // every edge once, from its lower end point: the higher neighbours of v
    // in v's live tets (a local sort per vertex instead of one of all edges)
    std::vector<int> nb;
    for (int lo = 0; lo < N; ++lo) {
      if (!valive[lo]) continue;
      nb.clear();
      for (int t : vt[lo]) {
        if (!talive[t]) continue;
        for (int x : T[t])
          if (x > lo) nb.push_back(x);
      }
      std::sort(nb.begin(), nb.end());
      nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
      for (int hi : nb) {
        const double s = 0.5 * (size[lo] + size[hi]);
        const double r = std::sqrt(len2(lo, hi)) / s;
        if (r < ratio) cand.push_back({r, ekey(lo, hi)});
      }
    }
    std::sort(cand.begin(), cand.end(), [](const Cand& x, const Cand& y) {
      return x.r != y.r ? x.r < y.r : x.key < y.key;
    });
    tq.assign(T.size(), 0.0);
    for (size_t t = 0; t < T.size(); ++t)
      if (talive[t]) tq[t] = quality(T[t]);
    std::vector<char> touched(N, 0);
    std::vector<int> adj;
    int done = 0;
    for (const Cand& c : cand) {
      const int lo = (int)(c.key & 0xffffffffu), hi = (int)(c.key >> 32);
      if (!valive[lo] || !valive[hi] || touched[lo] || touched[hi]) continue;
      int b = -1, a = -1;
      if (can_collapse(hi, lo, refine_ratio, min_quality)) { b = hi; a = lo; }
      else if (can_collapse(lo, hi, refine_ratio, min_quality)) { b = lo; a = hi; }
      if (b < 0) continue;
      adjacent(b, adj);
      touched[a] = touched[b] = 1;
      for (int x : adj) touched[x] = 1;
      collapse(b, a);
      ++done;
    }
    return done;
  }
};

}  // namespace
}  // namespace goal

struct goal_coarsener_s {
  goal::Coarsener c;
};

extern "C" {

int goal_coarsener_create(int num_nodes, const double* coords, int num_elems, const int* tets, const int* elem_set,
                          const long long* node_class, int num_sides, const int* tris, const int* tri_set,
                          goal_coarsener* out) {
  try {
    if (!out || !coords || !tets || !node_class || num_nodes <= 0 || num_elems <= 0 ||
        (num_sides > 0 && (!tris || !tri_set)))
      throw goal::Error(GOAL_ERR_ARG, "goal_coarsener_create: bad arguments");
    auto h = std::make_unique<goal_coarsener_s>();
    goal::Coarsener& c = h->c;
    c.N = num_nodes;
    c.X.assign(coords, coords + 3ll * num_nodes);
    c.cls.assign(node_class, node_class + num_nodes);
    for (long long& x : c.cls) x &= ~goal::kBoundaryBit;
    c.size.assign(num_nodes, 0.0);
    c.valive.assign(num_nodes, 1);
    c.T.resize(num_elems);
    c.eset.assign(num_elems, 0);
    c.talive.assign(num_elems, 1);
    c.vt.assign(num_nodes, {});
    c.vf.assign(num_nodes, {});
    c.vs.assign(num_nodes, {});
    c.W.assign(num_nodes, {});
    // boundary faces: the faces of exactly one tet (sorted vertex triples,
    // sorted, counted by runs)
    static const int kFaces[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
    for (int e = 0; e < num_elems; ++e) {
      for (int q = 0; q < 4; ++q) {
        const int v = tets[4ll * e + q];
        if (v < 0 || v >= num_nodes) throw goal::Error(GOAL_ERR_ARG, "goal_coarsener_create: node id out of range");
        c.T[e][q] = v;
        c.vt[v].push_back(e);
      }
      c.eset[e] = elem_set ? elem_set[e] : 0;
      c.origin.push_back(e);
    }
    // faces grouped by their smallest vertex (a counting sort over the
    // nodes), then matched within each group by the other two vertices
    struct FaceRec {
      uint64_t rest;  // (middle << 32) | largest vertex
      int tet, q;
    };
    std::vector<long long> start(num_nodes + 1, 0);
    auto face_key = [&](int e, int q, int& lo, uint64_t& rest) {
      int k[3] = {c.T[e][kFaces[q][0]], c.T[e][kFaces[q][1]], c.T[e][kFaces[q][2]]};
      std::sort(k, k + 3);
      lo = k[0];
      rest = ((uint64_t)(unsigned)k[1] << 32) | (uint64_t)(unsigned)k[2];
    };
    for (int e = 0; e < num_elems; ++e)
      for (int q = 0; q < 4; ++q) {
        int lo;
        uint64_t rest;
        face_key(e, q, lo, rest);
        ++start[lo + 1];
      }
    for (int n = 0; n < num_nodes; ++n) start[n + 1] += start[n];
    std::vector<FaceRec> all(4ull * num_elems);
    {
      std::vector<long long> fill(start.begin(), start.end() - 1);
      for (int e = 0; e < num_elems; ++e)
        for (int q = 0; q < 4; ++q) {
          int lo;
          uint64_t rest;
          face_key(e, q, lo, rest);
          all[fill[lo]++] = {rest, e, q};
        }
    }
    std::vector<std::array<int, 3>> bfaces;
    for (int n = 0; n < num_nodes; ++n) {
      auto b0 = all.begin() + start[n], b1 = all.begin() + start[n + 1];
      std::sort(b0, b1, [](const FaceRec& x, const FaceRec& y) { return x.rest < y.rest; });
      for (auto i = b0; i != b1;) {
        auto j = i + 1;
        while (j != b1 && j->rest == i->rest) ++j;
        if (j - i == 1) {
          const auto& fq = kFaces[i->q];
          bfaces.push_back({c.T[i->tet][fq[0]], c.T[i->tet][fq[1]], c.T[i->tet][fq[2]]});
        }
        i = j;
      }
    }
    std::sort(bfaces.begin(), bfaces.end());  // deterministic order
    for (const auto& f : bfaces) {
      const int id = (int)c.F.size();
      c.F.push_back(f);
      c.falive.push_back(1);
      for (int v : f) {
        c.vf[v].push_back(id);
        c.cls[v] |= goal::kBoundaryBit;
      }
    }
    for (int f = 0; f < num_sides; ++f) {
      std::array<int, 3> s = {tris[3ll * f], tris[3ll * f + 1], tris[3ll * f + 2]};
      for (int v : s)
        if (v < 0 || v >= num_nodes) throw goal::Error(GOAL_ERR_ARG, "goal_coarsener_create: side node out of range");
      c.S.push_back(s);
      c.S_set.push_back(tri_set[f]);
      c.salive.push_back(1);
      for (int v : s) c.vs[v].push_back(f);
    }
    *out = h.release();
  } catch (const goal::Error& e) {
    goal::set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    goal::set_last_error(e.what());
    return GOAL_ERR_STATE;
  }
  return GOAL_OK;
}

int goal_coarsener_coarsen(goal_coarsener h, const double* vtx_size, double ratio, double refine_ratio,
                           double min_quality, int max_passes, long long* sizes) {
  try {
    if (!h || !vtx_size || !sizes || !(ratio > 0.0) || !(refine_ratio > ratio) || !(min_quality >= 0.0))
      throw goal::Error(GOAL_ERR_ARG, "goal_coarsener_coarsen: bad arguments");
    goal::Coarsener& c = h->c;
    for (int n = 0; n < c.N; ++n) {
      if (!(vtx_size[n] > 0.0)) throw goal::Error(GOAL_ERR_ARG, "goal_coarsener_coarsen: sizes must be positive");
      c.size[n] = vtx_size[n];
    }
    for (int p = 0; p < max_passes; ++p)
      if (c.pass(ratio, refine_ratio, min_quality) == 0) break;
    long long nn = 0, ne = 0, ns = 0;
    for (char a : c.valive) nn += a ? 1 : 0;
    for (char a : c.talive) ne += a ? 1 : 0;
    for (char a : c.salive) ns += a ? 1 : 0;
    sizes[0] = nn;
    sizes[1] = ne;
    sizes[2] = ns;
  } catch (const goal::Error& e) {
    goal::set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    goal::set_last_error(e.what());
    return GOAL_ERR_STATE;
  }
  return GOAL_OK;
}

int goal_coarsener_swap(goal_coarsener h, double target_quality, int max_passes, long long* sizes) {
  try {
    if (!h || !sizes || !(target_quality > 0.0) || target_quality > 1.0)
      throw goal::Error(GOAL_ERR_ARG, "goal_coarsener_swap: bad arguments");
    goal::Coarsener& c = h->c;
    for (int p = 0; p < max_passes; ++p)
      if (c.swap_pass(target_quality) == 0) break;
    long long nn = 0, ne = 0, ns = 0;
    for (char a : c.valive) nn += a ? 1 : 0;
    for (char a : c.talive) ne += a ? 1 : 0;
    for (char a : c.salive) ns += a ? 1 : 0;
    sizes[0] = nn;
    sizes[1] = ne;
    sizes[2] = ns;
  } catch (const goal::Error& e) {
    goal::set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    goal::set_last_error(e.what());
    return GOAL_ERR_STATE;
  }
  return GOAL_OK;
}

int goal_coarsener_smooth(goal_coarsener h, double target_quality, int max_passes, long long* transfer_nnz) {
  try {
    if (!h || !transfer_nnz || !(target_quality > 0.0) || target_quality > 1.0)
      throw goal::Error(GOAL_ERR_ARG, "goal_coarsener_smooth: bad arguments");
    goal::Coarsener& c = h->c;
    for (int p = 0; p < max_passes; ++p)
      if (c.smooth_pass(target_quality) == 0) break;
    long long nnz = 0;
    for (int n = 0; n < c.N; ++n)
      if (c.valive[n]) nnz += c.W[n].empty() ? 1 : (long long)c.W[n].size();
    *transfer_nnz = nnz;
  } catch (const goal::Error& e) {
    goal::set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    goal::set_last_error(e.what());
    return GOAL_ERR_STATE;
  }
  return GOAL_OK;
}

int goal_coarsener_transfer(goal_coarsener h, int* ptr, int* ids, double* weights) {
  try {
    if (!h || !ptr || !ids || !weights) throw goal::Error(GOAL_ERR_ARG, "goal_coarsener_transfer: bad arguments");
    const goal::Coarsener& c = h->c;
    long long k = 0;
    int row = 0;
    ptr[0] = 0;
    for (int n = 0; n < c.N; ++n) {
      if (!c.valive[n]) continue;
      for (const auto& pr : c.row(n)) {
        ids[k] = pr.first;
        weights[k] = pr.second;
        ++k;
      }
      ptr[++row] = (int)k;
    }
  } catch (const goal::Error& e) {
    goal::set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    goal::set_last_error(e.what());
    return GOAL_ERR_STATE;
  }
  return GOAL_OK;
}

int goal_coarsener_get(goal_coarsener h, double* coords, int* node_origin, int* tets, int* elem_origin, int* tris,
                       int* tri_set) {
  try {
    if (!h || !coords || !node_origin || !tets || !elem_origin)
      throw goal::Error(GOAL_ERR_ARG, "goal_coarsener_get: bad arguments");
    const goal::Coarsener& c = h->c;
    std::vector<int> renum(c.N, -1);
    int k = 0;
    for (int n = 0; n < c.N; ++n)
      if (c.valive[n]) {
        renum[n] = k;
        node_origin[k] = n;
        for (int q = 0; q < 3; ++q) coords[3ll * k + q] = c.X[3ll * n + q];
        ++k;
      }
    long long e = 0;
    for (size_t t = 0; t < c.T.size(); ++t)
      if (c.talive[t]) {
        for (int q = 0; q < 4; ++q) tets[4 * e + q] = renum[c.T[t][q]];
        elem_origin[e] = c.origin[t];
        ++e;
      }
    if (tris && tri_set) {
      long long f = 0;
      for (size_t s = 0; s < c.S.size(); ++s)
        if (c.salive[s]) {
          for (int q = 0; q < 3; ++q) tris[3 * f + q] = renum[c.S[s][q]];
          tri_set[f] = c.S_set[s];
          ++f;
        }
    }
  } catch (const std::exception& e) {
    goal::set_last_error(e.what());
    return GOAL_ERR_STATE;
  }
  return GOAL_OK;
}

int goal_coarsener_destroy(goal_coarsener h) {
  delete h;
  return GOAL_OK;
}

}  // extern "C"
