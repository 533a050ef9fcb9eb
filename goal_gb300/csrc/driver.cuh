// Host drivers above the element kernels and the Krylov solver: Newton
// (Primal::solve), the nested adjoint + DWR error estimate (NestedAdjoint::run)
// and the helpers they need (solution update, prolongation, indicators).
#pragma once

#include <memory>

#include "krylov.cuh"
#include "mechanics.cuh"

namespace goal {

BsrView bsr_view(const Disc& d);

struct NewtonParams {
  int max_iters = 5;           // "nonlinear max iters"
  double tolerance = 1e-8;     // "nonlinear tolerance" (absolute ||R||_2)
  SolveParams lin;
  // 0: goal's full Newton steps. k > 0: backtracking on ||R||_2, the step
  // U += a du with the first a in 1, 1/2, ..., 2^-k whose residual norm is
  // below (1 - 1e-4 a) times the iteration's starting norm (else the smallest)
  int line_search = 0;
};

struct NewtonStats {
  int iters = 0;
  int converged = 0;
  double norms[32] = {0};
  int linear_iters = 0;
  int inner_iters = 0;
  int backtracks = 0;          // halvings of the step taken by the line search
  double seconds_assembly = 0.0;
  double seconds_solve = 0.0;
  SolveStats last;
};

// Primal::solve (src/goal_primal.cpp:111-137): Newton with the Jacobian and
// residual chains, traction then Dirichlet conditions, R *= -1, linear solve,
// U += du, absolute ||R||_2 convergence.
NewtonStats primal_solve(Mechanics& m, SolInfo& s, const std::vector<DBC>& dbcs, const std::vector<TBC>& tbcs,
                         double t_now, double t_old, const NewtonParams& p, Krylov& K);

// Linear solve on the SolInfo's matrix: block-Jacobi set-up (plus the FP32
// copy for the mixed solve) and FGMRES. dD (nullable) corrects the diagonal blocks.
SolveStats linear_solve(SolInfo& s, const SolveParams& p, const double* b, double* x, Krylov& K,
                        const double* dD = nullptr);

struct NestedAdjoint {
  Mechanics* base = nullptr;
  std::unique_ptr<Disc> disc;
  std::unique_ptr<Mechanics> mech;
  std::unique_ptr<SolInfo> si;
  DevBuf<double> z, zc, zd, err_nested, err_base, tmp;
  Krylov K;
  void build(Mechanics& base_mech);   // NestedAdjoint::build_data
  void refresh();                     // states (child = parent) and prolonged solution from the base
};

struct DwrResult {
  double eta = 0.0;        // -R.z  (z.R estimate, src/goal_nested_adjoint.cpp:213-214)
  double bound = 0.0;      // sum_contribs (src/goal_error.cpp:37-56)
  double qoi = 0.0;        // QoI on the nested mesh
  SolveStats solve;
  double seconds_adjoint = 0.0, seconds_solve = 0.0, seconds_localize = 0.0;
};

// NestedAdjoint::run (src/goal_nested_adjoint.cpp:163-257)
DwrResult nested_adjoint_run(NestedAdjoint& a, const std::vector<DBC>& dbcs, const std::vector<TBC>& tbcs, int qoi,
                             double rho, double t_now, double t_old, const SolveParams& p);

}  // namespace goal
