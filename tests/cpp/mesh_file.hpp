// Mesh file of the C++ tests (written by tests/test_gpu_cpp_shim.py):
// N E | coords (3N f64) | tets (4E i32) | node sets | side sets, each set as
// (name length, name, count, ids); side sets hold triangles (3 ids each).
#pragma once

#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "../../goal_gb300/host/goal.hpp"

struct MeshFile {
  int N = 0, E = 0;
  std::vector<double> coords;
  std::vector<int> tets;
  std::map<std::string, std::vector<int>> node_sets, side_sets;
};

// format: N E | coords | tets | nsets | (name len, name, n, ids)* | ssets | (name len, name, n, tris)*
inline MeshFile read_mesh(const char* path) {
  MeshFile m;
  std::ifstream f(path, std::ios::binary);
  if (!f) goal::fail("cannot open %s", path);
  auto rd = [&](void* p, size_t n) { f.read(reinterpret_cast<char*>(p), n); };
  rd(&m.N, 4);
  rd(&m.E, 4);
  m.coords.resize(3 * m.N);
  m.tets.resize(4 * m.E);
  rd(m.coords.data(), 8 * m.coords.size());
  rd(m.tets.data(), 4 * m.tets.size());
  for (int kind = 0; kind < 2; ++kind) {
    int ns = 0;
    rd(&ns, 4);
    for (int i = 0; i < ns; ++i) {
      int len = 0, n = 0;
      rd(&len, 4);
      std::string name(len, ' ');
      rd(&name[0], len);
      rd(&n, 4);
      std::vector<int> v(kind == 0 ? n : 3 * n);
      rd(v.data(), 4 * v.size());
      (kind == 0 ? m.node_sets : m.side_sets)[name] = v;
    }
  }
  return m;
}

