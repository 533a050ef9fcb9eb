// C++ driver through goal.hpp (the mirror of goal's host classes): runs the
// reference's neohookean_uniaxial_3D and J2_traction_3D cases on the
// reference's cube mesh (given as a flat binary file) and checks the final QoI
// against the reference's regression values (src/goal_regression.cpp:14-23),
// like goal's own GoalPrimal examples (src/main_primal.cpp:68-90).
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "../../goal_gb300/host/goal.hpp"
#include "mesh_file.hpp"

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
