// Conforming refinement of a tetrahedral mesh to a target size field, the
// refinement half of goal's adaptation loop (src/main_nested.cpp:106-126,
// which calls SCOREC ma::adapt -- not part of the reference tree). The
// algorithm is longest-edge propagation path (LEPP) bisection: a tet is
// refined by bisecting the "terminal" edge of its LEPP, the first edge along
// the path that is the longest edge of every tet around it, so the mesh stays
// conforming after every bisection. Edges are ordered by (squared length,
// end-point pair), a strict order, so paths end and results are deterministic.
//
// Host code: the refinement is a pointer-chasing sequence of local updates;
// the discretization built from its output goes back to the GPU.
#include <algorithm>
#include <array>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <vector>

#include "../../include/goal_gb300.h"
#include "common.cuh"

namespace goal {
namespace {

inline uint64_t edge_key(int a, int b) {
  const uint64_t lo = (uint64_t)(unsigned)std::min(a, b), hi = (uint64_t)(unsigned)std::max(a, b);
  return (hi << 32) | lo;
}

constexpr int kEdges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

// Open-addressing map from an edge key (never 0: the end points differ) to a
// dense id, with linear probing; keys are never removed.
struct EdgeIds {
  std::vector<uint64_t> keys;
  std::vector<int> ids;
  size_t count = 0;
  EdgeIds() { rehash(1 << 16); }
  static size_t hash(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    return (size_t)k;
  }
  void rehash(size_t cap) {
    std::vector<uint64_t> ok = std::move(keys);
    std::vector<int> oi = std::move(ids);
    keys.assign(cap, 0);
    ids.assign(cap, -1);
    for (size_t i = 0; i < ok.size(); ++i)
      if (ok[i]) {
        size_t h = hash(ok[i]) & (cap - 1);
        while (keys[h]) h = (h + 1) & (cap - 1);
        keys[h] = ok[i];
        ids[h] = oi[i];
      }
  }
  int find(uint64_t k) const {
    const size_t mask = keys.size() - 1;
    for (size_t h = hash(k) & mask;; h = (h + 1) & mask) {
      if (keys[h] == k) return ids[h];
      if (!keys[h]) return -1;
    }
  }
  // the id of k, inserting next_id when absent (inserted set accordingly)
  int get(uint64_t k, int next_id, bool& inserted) {
    if (2 * (count + 1) > keys.size()) rehash(2 * keys.size());
    const size_t mask = keys.size() - 1;
    for (size_t h = hash(k) & mask;; h = (h + 1) & mask) {
      if (keys[h] == k) {
        inserted = false;
        return ids[h];
      }
      if (!keys[h]) {
        keys[h] = k;
        ids[h] = next_id;
        ++count;
        inserted = true;
        return next_id;
      }
    }
  }
};

// An ordered list of element ids with inline room for eight (the tets around
// an edge of a tet mesh, or the triangles around a boundary edge)
struct IdList {
  int n = 0;
  int a[8];
  std::vector<int> more;
  int size() const { return n; }
  int operator[](int i) const { return i < 8 ? a[i] : more[i - 8]; }
  void push(int v) {
    if (n < 8) a[n] = v;
    else more.push_back(v);
    ++n;
  }
  void erase(int v) {
    int i = 0;
    while (i < n && (*this)[i] != v) ++i;
    if (i == n) return;
    for (int j = i; j + 1 < n; ++j) set(j, (*this)[j + 1]);
    --n;
    if (n >= 8) more.pop_back();
  }
  void set(int i, int v) {
    if (i < 8) a[i] = v;
    else more[i - 8] = v;
  }
  void clear() {
    n = 0;
    more.clear();
  }
  std::vector<int> copy() const {
    std::vector<int> out(n);
    for (int i = 0; i < n; ++i) out[i] = (*this)[i];
    return out;
  }
};

struct Refiner {
  std::vector<double> X;                      // 3 per node
  std::vector<double> size;                   // target size per node (new nodes: mean of the edge's)
  std::vector<int> pa, pb;                    // edge end points of new nodes (-1: original node)
  std::vector<std::array<int, 4>> T;          // all tets ever made
  std::vector<int> origin;                    // original element of each tet
  std::vector<char> alive;
  long long num_alive = 0;
  EdgeIds edge_id;              // edge key -> dense edge id
  std::vector<IdList> around;   // live tets around each edge (by edge id)
  std::vector<IdList> around_s; // live side triangles around each edge
  std::vector<int> mid;         // midpoint node of each bisected edge, -1 if none
  // side triangles (boundary faces), split with their edges
  std::vector<std::array<int, 3>> S;
  std::vector<int> S_set;
  std::vector<char> S_alive;

  int eid(uint64_t k) {
    bool ins;
    const int id = edge_id.get(k, (int)around.size(), ins);
    if (ins) {
      around.emplace_back();
      around_s.emplace_back();
      mid.push_back(-1);
    }
    return id;
  }

  double len2(int a, int b) const {
    const double dx = X[3 * a] - X[3 * b], dy = X[3 * a + 1] - X[3 * b + 1], dz = X[3 * a + 2] - X[3 * b + 2];
    return dx * dx + dy * dy + dz * dz;
  }
  // strict order on edges: length, then end-point pair
  bool longer(int a, int b, int c, int d) const {
    const double l1 = len2(a, b), l2 = len2(c, d);
    if (l1 != l2) return l1 > l2;
    return edge_key(a, b) > edge_key(c, d);
  }
  uint64_t longest(int t) const {
    const auto& v = T[t];
    int ba = v[0], bb = v[1];
    for (int q = 1; q < 6; ++q) {
      const int a = v[kEdges[q][0]], b = v[kEdges[q][1]];
      if (longer(a, b, ba, bb)) { ba = a; bb = b; }
    }
    return edge_key(ba, bb);
  }

  void link(int t) {
    const auto v = T[t];
    for (auto& e : kEdges) around[eid(edge_key(v[e[0]], v[e[1]]))].push(t);
  }
  void unlink(int t) {
    const auto v = T[t];
    for (auto& e : kEdges) around[eid(edge_key(v[e[0]], v[e[1]]))].erase(t);
  }
  void link_s(int f) {
    const auto v = S[f];
    for (int q = 0; q < 3; ++q) around_s[eid(edge_key(v[q], v[(q + 1) % 3]))].push(f);
  }
  void unlink_s(int f) {
    const auto v = S[f];
    for (int q = 0; q < 3; ++q) around_s[eid(edge_key(v[q], v[(q + 1) % 3]))].erase(f);
  }

  int midpoint(int a, int b) {
    const int e = eid(edge_key(a, b));
    if (mid[e] >= 0) return mid[e];
    const int m = (int)pa.size();
    for (int c = 0; c < 3; ++c) X.push_back(0.5 * (X[3 * a + c] + X[3 * b + c]));
    size.push_back(0.5 * (size[a] + size[b]));
    pa.push_back(a);
    pb.push_back(b);
    mid[e] = m;
    return m;
  }

  // bisects edge (a, b) in every live tet and side triangle around it
  void bisect(uint64_t k) {
    const int a = (int)(k & 0xffffffffu), b = (int)(k >> 32);
    const int m = midpoint(a, b);
    const int ke = eid(k);
    const std::vector<int> tets = around[ke].copy();
    for (int t : tets) {
      std::array<int, 4> v = T[t];
      int ia = -1, ib = -1;
      for (int q = 0; q < 4; ++q) {
        if (v[q] == a) ia = q;
        if (v[q] == b) ib = q;
      }
      unlink(t);
      alive[t] = 0;
      // replacing one end point by the midpoint keeps the orientation
      std::array<int, 4> c1 = v, c2 = v;
      c1[ib] = m;
      c2[ia] = m;
      for (const auto& c : {c1, c2}) {
        const int n = (int)T.size();
        T.push_back(c);
        origin.push_back(origin[t]);
        alive.push_back(1);
        link(n);
      }
      num_alive += 1;
    }
    around[ke].clear();
    if (around_s[ke].size() > 0) {
      const std::vector<int> tris = around_s[ke].copy();
      for (int f : tris) {
        std::array<int, 3> v = S[f];
        int ia = -1, ib = -1;
        for (int q = 0; q < 3; ++q) {
          if (v[q] == a) ia = q;
          if (v[q] == b) ib = q;
        }
        unlink_s(f);
        S_alive[f] = 0;
        std::array<int, 3> c1 = v, c2 = v;
        c1[ib] = m;
        c2[ia] = m;
        for (const auto& c : {c1, c2}) {
          const int n = (int)S.size();
          S.push_back(c);
          S_set.push_back(S_set[f]);
          S_alive.push_back(1);
          link_s(n);
        }
      }
      around_s[ke].clear();
    }
  }

  // refines tet t along its longest-edge propagation path until t is split
  void refine(int t, int depth) {
    if (depth > 1000) throw Error(GOAL_ERR_STATE, "refine: longest-edge path did not end");
    while (alive[t]) {
      const uint64_t e = longest(t);
      const IdList& ar = around[eid(e)];
      int other = -1;
      for (int i = 0; i < ar.size(); ++i)
        if (longest(ar[i]) != e) { other = ar[i]; break; }
      if (other < 0) {
        bisect(e);
        return;
      }
      refine(other, depth + 1);
    }
  }

  bool too_long(int t, double ratio) const {
    const auto& v = T[t];
    for (auto& e : kEdges) {
      const int a = v[e[0]], b = v[e[1]];
      const double s = ratio * 0.5 * (size[a] + size[b]);
      if (len2(a, b) > s * s) return true;
    }
    return false;
  }
};

}  // namespace
}  // namespace goal

struct goal_refiner_s {
  goal::Refiner r;
  int base_nodes = 0;
};

extern "C" {

int goal_refiner_create(int num_nodes, const double* coords, int num_elems, const int* tets, int num_sides,
                        const int* tris, const int* tri_set, goal_refiner* out) {
  try {
    if (!out || !coords || !tets || num_nodes <= 0 || num_elems <= 0 || (num_sides > 0 && (!tris || !tri_set)))
      throw goal::Error(GOAL_ERR_ARG, "goal_refiner_create: bad arguments");
    auto h = std::make_unique<goal_refiner_s>();
    goal::Refiner& r = h->r;
    r.X.assign(coords, coords + 3ll * num_nodes);
    r.size.assign(num_nodes, 0.0);
    r.pa.assign(num_nodes, -1);
    r.pb.assign(num_nodes, -1);
    r.T.resize(num_elems);
    r.origin.resize(num_elems);
    r.alive.assign(num_elems, 1);
    for (int e = 0; e < num_elems; ++e) {
      for (int q = 0; q < 4; ++q) {
        const int v = tets[4ll * e + q];
        if (v < 0 || v >= num_nodes) throw goal::Error(GOAL_ERR_ARG, "goal_refiner_create: node id out of range");
        r.T[e][q] = v;
      }
      r.origin[e] = e;
      r.link(e);
    }
    r.num_alive = num_elems;
    for (int f = 0; f < num_sides; ++f) {
      r.S.push_back({tris[3ll * f], tris[3ll * f + 1], tris[3ll * f + 2]});
      r.S_set.push_back(tri_set[f]);
      r.S_alive.push_back(1);
      r.link_s(f);
    }
    h->base_nodes = num_nodes;
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

int goal_refiner_refine(goal_refiner h, const double* vtx_size, double ratio, long long max_elems, int max_passes,
                        long long* sizes) {
  try {
    if (!h || !vtx_size || !sizes || !(ratio > 0.0))
      throw goal::Error(GOAL_ERR_ARG, "goal_refiner_refine: bad arguments");
    goal::Refiner& r = h->r;
    for (int n = 0; n < h->base_nodes; ++n) r.size[n] = vtx_size[n];
    for (int pass = 0; pass < max_passes; ++pass) {
      std::vector<int> marked;
      for (int t = 0; t < (int)r.T.size(); ++t)
        if (r.alive[t] && r.too_long(t, ratio)) marked.push_back(t);
      if (marked.empty()) break;
      for (int t : marked) {
        if (r.num_alive >= max_elems) break;
        if (r.alive[t] && r.too_long(t, ratio)) r.refine(t, 0);
      }
      if (r.num_alive >= max_elems) break;
    }
    long long ns = 0;
    for (char a : r.S_alive) ns += a ? 1 : 0;
    sizes[0] = (long long)r.pa.size();
    sizes[1] = r.num_alive;
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

int goal_refiner_get(goal_refiner h, double* coords, int* node_parents, int* tets, int* elem_origin, int* tris,
                     int* tri_set) {
  try {
    if (!h || !coords || !node_parents || !tets || !elem_origin)
      throw goal::Error(GOAL_ERR_ARG, "goal_refiner_get: bad arguments");
    const goal::Refiner& r = h->r;
    std::copy(r.X.begin(), r.X.end(), coords);
    for (size_t n = 0; n < r.pa.size(); ++n) {
      node_parents[2 * n] = r.pa[n];
      node_parents[2 * n + 1] = r.pb[n];
    }
    long long k = 0;
    for (size_t t = 0; t < r.T.size(); ++t)
      if (r.alive[t]) {
        for (int q = 0; q < 4; ++q) tets[4 * k + q] = r.T[t][q];
        elem_origin[k] = r.origin[t];
        ++k;
      }
    if (tris && tri_set) {
      long long f = 0;
      for (size_t s = 0; s < r.S.size(); ++s)
        if (r.S_alive[s]) {
          for (int q = 0; q < 3; ++q) tris[3 * f + q] = r.S[s][q];
          tri_set[f] = r.S_set[s];
          ++f;
        }
    }
  } catch (const std::exception& e) {
    goal::set_last_error(e.what());
    return GOAL_ERR_STATE;
  }
  return GOAL_OK;
}

int goal_refiner_destroy(goal_refiner h) {
  delete h;
  return GOAL_OK;
}

}  // extern "C"
