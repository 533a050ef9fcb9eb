// C++ driver through goal.hpp (the mirror of goal's host classes): runs the
// reference's neohookean_uniaxial_3D and J2_traction_3D cases on the
// reference's cube mesh (given as a flat binary file) and checks the final QoI
// against the reference's regression values (src/goal_regression.cpp:14-23),
// like goal's own GoalPrimal examples (src/main_primal.cpp:68-90).
#include <cmath>
#include <cstdio>
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
static MeshFile read_mesh(const char* path) {
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

static double run_case(const MeshFile& mf, const std::string& model, goal::Material mat, bool stretch) {
  std::vector<int> es(mf.E, 0);
  goal::Disc disc(mf.N, mf.E, mf.coords.data(), mf.tets.data(), es.data(), 1);
  for (auto& kv : mf.node_sets) disc.add_node_set(kv.first, kv.second);
  for (auto& kv : mf.side_sets) disc.add_side_set(kv.first, kv.second);
  disc.build_data();
  goal::Mechanics mech(disc, model, {mat});
  goal::BCs bcs(disc);
  bcs.add_dirichlet(0, "xmin", "0.0");
  bcs.add_dirichlet(1, "ymin", "0.0");
  bcs.add_dirichlet(2, "zmin", "0.0");
  if (stretch) bcs.add_dirichlet(0, "xmax", "0.01*t");
  else bcs.add_traction("ymax", "0.0", "1.0*t", "0.0");
  goal::LinearParams lp;
  goal::Primal primal(mech, bcs, lp);
  goal::Functional J(mech, "avg disp");
  double t_old = 0.0, t_now = 1.0;
  for (int step = 1; step <= 3; ++step) {
    goal::print("****** load step: %d", step);
    primal.solve(t_now, t_old);
    J.compute(t_now, t_old);
    J.print_value();
    mech.update_states();
    t_old = t_now;
    t_now += 1.0;
  }
  return J.get_value();
}

int main(int argc, char** argv) {
  if (argc != 2) goal::fail("usage: primal_kat mesh.bin");
  MeshFile mf = read_mesh(argv[1]);
  double v1 = run_case(mf, "neohookean", {1000.0, 0.25, 0.0, 0.0, 1.0}, true);
  double v2 = run_case(mf, "J2", {1000.0, 0.25, 100.0, 10.0, 1.0}, false);
  const double r1 = 2.541285341193943e-03, r2 = 2.512233163668167e-04;
  std::printf("neohookean_uniaxial_3D %.15e (regression %.15e)\n", v1, r1);
  std::printf("J2_traction_3D %.15e (regression %.15e)\n", v2, r2);
  if (std::fabs(v1 - r1) >= 1e-8 || std::fabs(v2 - r2) >= 1e-8) goal::fail("regression check failed");
  std::printf("OK\n");
  return 0;
}
