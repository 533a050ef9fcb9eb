// C++ through goal.hpp: refines a 2x2x2 Kuhn cube near one corner with
// goal::refine_to_size (the C ABI's host refiner) and checks that the refined
// tets tile the unit cube (total volume 1, every volume positive) and that
// every new node sits at the midpoint of its parent edge; then coarsens the
// result with goal::coarsen_to_size and checks the tiling again. Runs without
// a GPU.
#include <cmath>
#include <cstdio>
#include <vector>

#include "../../goal_gb300/host/goal.hpp"

int main() {
  const int n = 2, n1 = n + 1;
  std::vector<double> X;
  for (int k = 0; k < n1; ++k)
    for (int j = 0; j < n1; ++j)
      for (int i = 0; i < n1; ++i) {
        X.push_back(double(i) / n);
        X.push_back(double(j) / n);
        X.push_back(double(k) / n);
      }
  // Kuhn tets: paths through each hex along the 6 axis orders, oriented positively
  const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  const int step[3] = {1, n1, n1 * n1};
  std::vector<int> T;
  auto vol = [&](const int* t) {
    double a[3], b[3], c[3];
    for (int d = 0; d < 3; ++d) {
      a[d] = X[3 * t[1] + d] - X[3 * t[0] + d];
      b[d] = X[3 * t[2] + d] - X[3 * t[0] + d];
      c[d] = X[3 * t[3] + d] - X[3 * t[0] + d];
    }
    return (a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) + a[2] * (b[0] * c[1] - b[1] * c[0])) / 6.0;
  };
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        for (auto& p : perms) {
          int t[4];
          t[0] = i + n1 * (j + n1 * k);
          t[1] = t[0] + step[p[0]];
          t[2] = t[1] + step[p[1]];
          t[3] = t[2] + step[p[2]];
          if (vol(t) < 0) std::swap(t[2], t[3]);
          T.insert(T.end(), t, t + 4);
        }
  std::vector<double> size(X.size() / 3);
  for (size_t v = 0; v < size.size(); ++v)
    size[v] = 0.1 + 0.6 * std::sqrt(X[3 * v] * X[3 * v] + X[3 * v + 1] * X[3 * v + 1] + X[3 * v + 2] * X[3 * v + 2]);
  goal::RefinedMesh m = goal::refine_to_size(X, T, {}, {}, size);
  X = m.coords;
  double total = 0.0, vmin = 1.0;
  for (size_t e = 0; e < m.tets.size() / 4; ++e) {
    const double v = vol(&m.tets[4 * e]);
    total += v;
    vmin = std::fmin(vmin, v);
  }
  const int base = n1 * n1 * n1;
  double mid_err = 0.0;
  for (size_t v = base; v < X.size() / 3; ++v)
    for (int d = 0; d < 3; ++d)
      mid_err = std::fmax(mid_err, std::fabs(X[3 * v + d] - 0.5 * (X[3 * m.node_parents[2 * v] + d] +
                                                                   X[3 * m.node_parents[2 * v + 1] + d])));
  std::printf("refined %zu -> %zu tets, volume %.17g, min %.3g, midpoint error %.3g\n", T.size() / 4,
              m.tets.size() / 4, total, vmin, mid_err);
  const bool ok = m.tets.size() > T.size() && std::fabs(total - 1.0) < 1e-13 && vmin > 0.0 && mid_err == 0.0;
  // and back: goal::coarsen_to_size with a uniform size of half the cube (no
  // sets: the box's corners and edges are kept because their boundary faces
  // are not coplanar)
  std::vector<double> big(X.size() / 3, 0.5);
  std::vector<long long> cls(X.size() / 3, 0);
  goal::CoarsenedMesh c = goal::coarsen_to_size(X, m.tets, {}, cls, {}, {}, big);
  X = c.coords;
  double ctotal = 0.0, cmin = 1.0;
  for (size_t e = 0; e < c.tets.size() / 4; ++e) {
    const double v = vol(&c.tets[4 * e]);
    ctotal += v;
    cmin = std::fmin(cmin, v);
  }
  std::printf("coarsened %zu -> %zu tets, volume %.17g, min %.3g\n", m.tets.size() / 4, c.tets.size() / 4, ctotal,
              cmin);
  const bool ok2 = c.tets.size() < m.tets.size() && std::fabs(ctotal - 1.0) < 1e-13 && cmin > 0.0;
  return ok && ok2 ? 0 : 1;
}
