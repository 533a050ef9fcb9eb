// Dirichlet and traction boundary conditions on the device.
//
// set_resid_dbcs / set_jac_dbcs (src/goal_dbcs.cpp:39-99): for every node of
// the set, R[row] = u_eq - value(x, t); with the Jacobian the whole row becomes
// the identity row and dMdu[row] = 0. The rows are rows of whatever the matrix
// holds (dRdu in PRIMAL mode, dRdu^T in ADJOINT mode), as in the reference.
//
// set_tbcs (src/goal_tbcs.cpp:29-85): one point at the triangle centroid,
// R[node*4+d] -= T_d(x_c, t) w_n(d) ipw dv with ipw = 1/2, dv = 2 |area|,
// w_n = 1/3 (VectorWeight) or z_d(x_c)/3 (DisplacementAdjoint, error chain).
// The scatter is node-centric (each touched node sums its incident sides in a
// fixed order) so it is deterministic without atomics.
#include "mechanics.cuh"

namespace goal {

namespace {

__global__ void k_dbc(int n, const int* nodes, int eq, ExprCode code, double t, const double* X, const double* U,
                      double* R, int jac, double* A, const int* brow_ptr, const int* diag, double* dMdu) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    int node = nodes[k];
    int row = 4 * node + eq;
    double v = eval_expr(code, X[3 * node], X[3 * node + 1], X[3 * node + 2], t);
    R[row] = U[row] - v;
    if (jac) {
      if (dMdu) dMdu[row] = 0.0;
      for (int b = brow_ptr[node]; b < brow_ptr[node + 1]; ++b) {
        double* p = A + 16ll * b + 4 * eq;
        p[0] = 0.0; p[1] = 0.0; p[2] = 0.0; p[3] = 0.0;
      }
      A[16ll * diag[node] + 4 * eq + eq] = 1.0;
    }
  }
}

struct Tcodes {
  ExprCode c[3];
};

__global__ void k_traction(int nn, const int* nodes, const int* inc_ptr, const int* inc, const int* tris, Tcodes tc,
                           double t, const double* X, const double* Zd, double* R) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nn; j += gridDim.x * blockDim.x) {
    int node = nodes[j];
    double acc[3] = {0.0, 0.0, 0.0};
    for (int q = inc_ptr[j]; q < inc_ptr[j + 1]; ++q) {
      int side = inc[q] / 3;
      const int* tr = tris + 3 * side;
      const double* xa = X + 3 * tr[0];
      const double* xb = X + 3 * tr[1];
      const double* xc = X + 3 * tr[2];
      double e1[3] = {xb[0] - xa[0], xb[1] - xa[1], xb[2] - xa[2]};
      double e2[3] = {xc[0] - xa[0], xc[1] - xa[1], xc[2] - xa[2]};
      double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
      double dv = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
      const double BF = 1.0 / 3.0;
      double x[3];
      for (int d = 0; d < 3; ++d) x[d] = BF * xa[d] + BF * xb[d] + BF * xc[d];
      for (int d = 0; d < 3; ++d) {
        double T = eval_expr(tc.c[d], x[0], x[1], x[2], t);
        double w = BF;
        if (Zd) {
          double z = BF * Zd[4 * tr[0] + d] + BF * Zd[4 * tr[1] + d] + BF * Zd[4 * tr[2] + d];
          w = z * BF;
        }
        acc[d] += T * w * 0.5 * dv;
      }
    }
    for (int d = 0; d < 3; ++d) R[4 * node + d] -= acc[d];
  }
}

}  // namespace

void apply_dbcs(Mechanics& m, SolInfo& s, const std::vector<DBC>& bcs, double t, bool jac, cudaStream_t st) {
  const Disc& d = *m.disc;
  for (const DBC& bc : bcs) {
    int n = (int)bc.set->host.size();
    if (!n) continue;
    GOAL_REQUIRE(bc.eq >= 0 && bc.eq < 3, GOAL_ERR_ARG, "dirichlet bc: component must be 0, 1 or 2");
    k_dbc<<<grid_for(n, 128), 128, 0, st>>>(n, bc.set->dev.ptr, bc.eq, bc.code, t, d.coords.ptr, m.U.ptr, s.R.ptr,
                                             jac ? 1 : 0, s.A.ptr, d.brow_ptr.ptr, d.diag.ptr, s.dMdu.ptr);
    GOAL_CHECK_LAUNCH();
  }
}

void apply_tbcs(Mechanics& m, SolInfo& s, const std::vector<TBC>& bcs, double t, const double* Zd, cudaStream_t st) {
  const Disc& d = *m.disc;
  for (const TBC& bc : bcs) {
    SideSet& ss = *bc.set;
    int nn = (int)ss.nodes_h.size();
    if (!nn) continue;
    Tcodes tc;
    for (int k = 0; k < 3; ++k) tc.c[k] = bc.code[k];
    k_traction<<<grid_for(nn, 128), 128, 0, st>>>(nn, ss.nodes.ptr, ss.inc_ptr.ptr, ss.inc.ptr, ss.dtris.ptr, tc, t,
                                                   d.coords.ptr, Zd, s.R.ptr);
    GOAL_CHECK_LAUNCH();
  }
}

}  // namespace goal
