// Device views of the linear objects through goal.hpp: the device graph, R,
// dMdu, the 4x4 blocks, the CSR values and the nodal solution must equal the
// host copies entry for entry, and a solve on device pointers
// (goal_solve_device with b = the SolInfo's own dMdu, x a caller buffer) must
// give the same iterate as the host solve. The system is goal's nested-adjoint
// shape on the reference cube: the transposed J2 Jacobian with avg disp's
// dM/du (src/goal_nested_adjoint.cpp:163-215), Dirichlet rows applied.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "mesh_file.hpp"

template <class T>
static std::vector<T> from_device(const T* p, size_t n) {
  std::vector<T> h(n);
  if (cudaMemcpy(h.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost) != cudaSuccess) goal::fail("cudaMemcpy failed");
  return h;
}

template <class T>
static void expect_equal(const char* what, const std::vector<T>& a, const std::vector<T>& b) {
  if (a.size() != b.size()) goal::fail("%s: sizes differ (%zu vs %zu)", what, a.size(), b.size());
  for (size_t i = 0; i < a.size(); ++i)
    if (!(a[i] == b[i])) goal::fail("%s: entry %zu differs", what, i);
  std::printf("%s: %zu entries equal\n", what, a.size());
}

int main(int argc, char** argv) {
  if (argc != 2) goal::fail("usage: device_views mesh.bin");
  MeshFile mf = read_mesh(argv[1]);
  std::vector<int> es(mf.E, 0);
  goal::Disc disc(mf.N, mf.E, mf.coords.data(), mf.tets.data(), es.data(), 1);
  for (auto& kv : mf.node_sets) disc.add_node_set(kv.first, kv.second);
  for (auto& kv : mf.side_sets) disc.add_side_set(kv.first, kv.second);
  disc.build_data();
  goal::Mechanics mech(disc, "J2", {{1000.0, 0.25, 100.0, 10.0, 1.0}});
  std::vector<double> U(disc.get_num_dofs());
  for (int n = 0; n < mf.N; ++n) {
    const double* x = &mf.coords[3 * n];
    U[4 * n + 0] = 0.01 * x[0] + 0.002 * x[1] * x[2];
    U[4 * n + 1] = -0.0025 * x[1] + 0.001 * x[0] * x[0];
    U[4 * n + 2] = -0.0025 * x[2];
    U[4 * n + 3] = 5.0 * x[0] - 1.0;
  }
  mech.set_solution(U);
  goal::BCs bcs(disc);
  bcs.add_dirichlet(0, "xmin", "0.0");
  bcs.add_dirichlet(1, "ymin", "0.0");
  bcs.add_dirichlet(2, "zmin", "0.0");
  bcs.add_dirichlet(0, "xmax", "0.01*t");
  goal::SolInfo si(disc);
  goal::assemble(mech, goal::Evaluators::adjoint(GOAL_QOI_AVG_DISP, 0.0), &si);
  goal::check(goal_set_jac_dbcs(mech.handle(), si.handle(), bcs.handle(), 1.0));

  const long long ndof = disc.get_num_dofs(), nnz = disc.get_nnz(), nnzb = nnz / 16;
  std::vector<int> row_ptr, col_idx;
  disc.get_owned_graph(row_ptr, col_idx);
  goal::Disc::DeviceGraph g = disc.device_graph();
  expect_equal("row_ptr", from_device(g.row_ptr, ndof + 1), row_ptr);
  expect_equal("col_idx", from_device(g.col_idx, nnz), col_idx);
  // the block graph expands to the scalar one: row 4n of the scalar graph has
  // 4 columns per block of block row n, in the block columns' order
  std::vector<int> brow = from_device(g.brow_ptr, ndof / 4 + 1), bcol = from_device(g.bcol, nnzb);
  for (long long n = 0; n < ndof / 4; ++n)
    for (int k = brow[n]; k < brow[n + 1]; ++k)
      if (col_idx[row_ptr[4 * n] + 4 * (k - brow[n])] != 4 * bcol[k]) goal::fail("block graph: node %lld", n);
  std::printf("block graph: %lld blocks consistent with the scalar graph\n", nnzb);

  goal::SolInfo::DeviceView v = si.device_view();
  expect_equal("R", from_device(v.R, ndof), si.R());
  expect_equal("dMdu", from_device(v.dMdu, ndof), si.dMdu());
  std::vector<double> bsr(16 * nnzb);
  goal::check(goal_sol_info_get_dRdu_bsr(si.handle(), bsr.data()));
  expect_equal("dRdu blocks", from_device(v.bsr, 16 * nnzb), bsr);
  expect_equal("dRdu csr", from_device(si.device_dRdu(), nnz), si.dRdu());
  expect_equal("U", from_device(mech.device_solution(), ndof), mech.get_solution());

  // dRdu^T z = dMdu, once on host arrays and once on device pointers
  goal_solve_params p{100, 2000, 1e-10, 0, 30, 0, 0};
  std::vector<double> b = si.dMdu(), x_host(ndof, 0.0);
  goal_solve_stats st_h, st_d;
  goal::check(goal_solve(si.handle(), &p, b.data(), x_host.data(), &st_h));
  double* x_dev = nullptr;
  if (cudaMalloc(&x_dev, ndof * sizeof(double)) != cudaSuccess) goal::fail("cudaMalloc failed");
  if (cudaMemset(x_dev, 0, ndof * sizeof(double)) != cudaSuccess) goal::fail("cudaMemset failed");
  goal::check(goal_solve_device(si.handle(), &p, v.dMdu, x_dev, &st_d));
  std::vector<double> x_d = from_device(x_dev, ndof);
  cudaFree(x_dev);
  if (!st_h.converged || !st_d.converged || st_h.iters != st_d.iters) goal::fail("solves differ in convergence");
  expect_equal("adjoint solution", x_d, x_host);
  std::printf("solve on device pointers: %d iterations, relative residual %.3e\n", st_d.iters, st_d.rel_res);
  std::printf("OK\n");
  return 0;
}
