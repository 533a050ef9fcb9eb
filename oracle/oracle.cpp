// CPU restatement of goal's element hot path -- TEST INFRASTRUCTURE ONLY.
//
// This file is the oracle the CUDA path is checked against. It is built into
// oracle/_build/liboracle.so and loaded only by tests/, by the smoke check and
// by bench.py's CPU-baseline leg. Nothing in the product links or calls it.
//
// It restates, in plain C++ with its own 16-slot forward-mode dual number
// (the semantics of Sacado::Fad::SLFad<double,16>, src/goal_scalar_types.hpp:8-9),
// the evaluator chain that goal's assemble() drives for one integration point
// per linear tet (src/goal_assembly.cpp:65-88):
//   Displacement/Pressure gather+interp   src/goal_displacement.cpp:139-172, src/goal_pressure.cpp:136-165
//   Vector/Scalar weights                 src/goal_vector_weight.cpp:25-28, src/goal_scalar_weight.cpp:28-31
//   Kinematics                            src/goal_kinematics.cpp:18-25
//   Neohookean                            src/goal_neohookean.cpp:44-86
//   J2 (radial return, state update)      src/goal_J2.cpp:53-156
//   Mixed                                 src/goal_mixed.cpp:33-46
//   MResidual                             src/goal_mresidual.cpp:25-32
//   PResidual (large strain)              src/goal_presidual.cpp:42-59
//   Stabilization                         src/goal_stabilization.cpp:45-81
//   scatter NONE/PRIMAL/ADJOINT           src/goal_displacement.cpp:177-214, src/goal_pressure.cpp:170-203
//   QoI avg disp / KS max von Mises       src/goal_qoi.cpp:55-81, src/goal_avg_disp.cpp:16-21,
//                                         src/goal_ks_vm.cpp:36-105, src/goal_von_mises.cpp:6-17
//   DWR adjoint weights                   src/goal_displacement_adjoint.cpp:37-53,
//                                         src/goal_pressure_adjoint.cpp:38-49, src/goal_mechanics.cpp:169-218
//   Dirichlet / traction                  src/goal_dbcs.cpp:39-99, src/goal_tbcs.cpp:29-85
//   DOF numbering + CSR graph             src/goal_disc.cpp:195-222, 307-332
//   error indicators                      src/goal_error.cpp:7-56
//   nested uniform refinement rule        (declared rule; SCOREC ma is not part of the reference tree)
//
// Parity of this restatement is pinned end to end by the reference's own
// regression values on its own cube mesh (tests/test_oracle_kat.py).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace orc {

constexpr int ND = 16;  // GOAL_FAD_SIZE default (CMakeLists.txt:14)

// ---------------------------------------------------------------- dual number
struct Dual {
  double v;
  double d[ND];
  Dual() : v(0.0) { std::memset(d, 0, sizeof(d)); }
  Dual(double x) : v(x) { std::memset(d, 0, sizeof(d)); }  // NOLINT
  double val() const { return v; }
  void diff(int i) {
    std::memset(d, 0, sizeof(d));
    d[i] = 1.0;
  }
  Dual& operator+=(const Dual& b) { v += b.v; for (int i = 0; i < ND; ++i) d[i] += b.d[i]; return *this; }
  Dual& operator-=(const Dual& b) { v -= b.v; for (int i = 0; i < ND; ++i) d[i] -= b.d[i]; return *this; }
  Dual& operator*=(const Dual& b) {
    for (int i = 0; i < ND; ++i) d[i] = d[i] * b.v + v * b.d[i];
    v *= b.v;
    return *this;
  }
  Dual& operator/=(const Dual& b) {
    for (int i = 0; i < ND; ++i) d[i] = (d[i] * b.v - v * b.d[i]) / (b.v * b.v);
    v /= b.v;
    return *this;
  }
};
inline double val(double x) { return x; }
inline double val(const Dual& x) { return x.v; }
inline Dual operator+(Dual a, const Dual& b) { return a += b; }
inline Dual operator-(Dual a, const Dual& b) { return a -= b; }
inline Dual operator*(Dual a, const Dual& b) { return a *= b; }
inline Dual operator/(Dual a, const Dual& b) { return a /= b; }
inline Dual operator+(Dual a, double b) { a.v += b; return a; }
inline Dual operator+(double a, Dual b) { b.v += a; return b; }
inline Dual operator-(Dual a, double b) { a.v -= b; return a; }
inline Dual operator-(double a, const Dual& b) { Dual r; r.v = a - b.v; for (int i = 0; i < ND; ++i) r.d[i] = -b.d[i]; return r; }
inline Dual operator*(Dual a, double b) { a.v *= b; for (int i = 0; i < ND; ++i) a.d[i] *= b; return a; }
inline Dual operator*(double b, Dual a) { a.v = b * a.v; for (int i = 0; i < ND; ++i) a.d[i] = b * a.d[i]; return a; }
inline Dual operator/(Dual a, double b) { a.v /= b; for (int i = 0; i < ND; ++i) a.d[i] /= b; return a; }
inline Dual operator/(double a, const Dual& b) {
  Dual r;
  r.v = a / b.v;
  for (int i = 0; i < ND; ++i) r.d[i] = -a * b.d[i] / (b.v * b.v);
  return r;
}
inline Dual operator-(const Dual& a) { Dual r; r.v = -a.v; for (int i = 0; i < ND; ++i) r.d[i] = -a.d[i]; return r; }
inline bool operator>(const Dual& a, double b) { return a.v > b; }
inline bool operator<(const Dual& a, double b) { return a.v < b; }
inline Dual sqrt(const Dual& a) {
  Dual r;
  r.v = std::sqrt(a.v);
  for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] / (2.0 * r.v);
  return r;
}
inline Dual cbrt(const Dual& a) {
  Dual r;
  r.v = std::cbrt(a.v);
  for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] / (3.0 * r.v * r.v);
  return r;
}
inline Dual pow(const Dual& a, double e) {
  Dual r;
  r.v = std::pow(a.v, e);
  double dv = e * std::pow(a.v, e - 1.0);
  for (int i = 0; i < ND; ++i) r.d[i] = dv * a.d[i];
  return r;
}
inline Dual exp(const Dual& a) {
  Dual r;
  r.v = std::exp(a.v);
  for (int i = 0; i < ND; ++i) r.d[i] = r.v * a.d[i];
  return r;
}
inline Dual log(const Dual& a) {
  Dual r;
  r.v = std::log(a.v);
  for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] / a.v;
  return r;
}
inline double abs(const Dual& a) { return std::fabs(a.v); }

using std::cbrt;
using std::exp;
using std::log;
using std::pow;
using std::sqrt;
inline double abs(double a) { return std::fabs(a); }

// ---------------------------------------------------------------- 3x3 tensors
template <typename T>
struct Ten {
  T a[9];
  T& operator()(int i, int j) { return a[3 * i + j]; }
  const T& operator()(int i, int j) const { return a[3 * i + j]; }
};
template <typename T>
Ten<T> zeros() {
  Ten<T> r;
  for (int i = 0; i < 9; ++i) r.a[i] = T(0.0);
  return r;
}
template <typename T>
Ten<T> eye() {
  Ten<T> r = zeros<T>();
  r(0, 0) = T(1.0); r(1, 1) = T(1.0); r(2, 2) = T(1.0);
  return r;
}
template <typename T>
Ten<T> matmul(const Ten<T>& A, const Ten<T>& B) {
  Ten<T> r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      T s = A(i, 0) * B(0, j);
      s += A(i, 1) * B(1, j);
      s += A(i, 2) * B(2, j);
      r(i, j) = s;
    }
  return r;
}
template <typename T>
Ten<T> transpose(const Ten<T>& A) {
  Ten<T> r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r(i, j) = A(j, i);
  return r;
}
template <typename T>
T trace(const Ten<T>& A) { return A(0, 0) + A(1, 1) + A(2, 2); }
template <typename T>
T det(const Ten<T>& A) {
  return A(0, 0) * (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) -
         A(0, 1) * (A(1, 0) * A(2, 2) - A(1, 2) * A(2, 0)) +
         A(0, 2) * (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0));
}
template <typename T>
Ten<T> inverse(const Ten<T>& A) {
  Ten<T> r;
  T d = det(A);
  r(0, 0) = (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) / d;
  r(0, 1) = (A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2)) / d;
  r(0, 2) = (A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1)) / d;
  r(1, 0) = (A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2)) / d;
  r(1, 1) = (A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0)) / d;
  r(1, 2) = (A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2)) / d;
  r(2, 0) = (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0)) / d;
  r(2, 1) = (A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1)) / d;
  r(2, 2) = (A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0)) / d;
  return r;
}
template <typename T>
Ten<T> dev(const Ten<T>& A) {
  Ten<T> r = A;
  T t = trace(A) / 3.0;
  r(0, 0) -= t; r(1, 1) -= t; r(2, 2) -= t;
  return r;
}
template <typename T>
T norm(const Ten<T>& A) {
  T s = A.a[0] * A.a[0];
  for (int i = 1; i < 9; ++i) s += A.a[i] * A.a[i];
  return sqrt(s);
}
template <typename T, typename S>
Ten<T> scale(const S& s, const Ten<T>& A) {
  Ten<T> r;
  for (int i = 0; i < 9; ++i) r.a[i] = s * A.a[i];
  return r;
}

// Matrix exponential by scaling and squaring of a truncated Taylor series
// (terms added until they no longer change the sum). Used only for the
// plastic deformation-gradient state update Fp = exp(dgam N) Fp_old.
inline Ten<double> expm(const Ten<double>& A) {
  double nrm = 0.0;
  for (int i = 0; i < 9; ++i) nrm = std::max(nrm, std::fabs(A.a[i]));
  int sq = 0;
  while (nrm * 3.0 > 0.25) { nrm *= 0.5; ++sq; }
  Ten<double> B = scale(std::ldexp(1.0, -sq), A);
  Ten<double> R = eye<double>();
  Ten<double> term = eye<double>();
  for (int k = 1; k < 30; ++k) {
    term = scale(1.0 / k, matmul(term, B));
    double tn = 0.0;
    for (int i = 0; i < 9; ++i) { R.a[i] += term.a[i]; tn = std::max(tn, std::fabs(term.a[i])); }
    if (tn < 1e-20) break;
  }
  for (int s = 0; s < sq; ++s) R = matmul(R, R);
  return R;
}

// ---------------------------------------------------------------- geometry
struct Geom {
  double BF[4];
  double GBF[4][3];
  double wdv;  // integration weight x |det J| = signed volume
  double h;    // rms edge length (src/goal_stabilization.cpp:45-52)
};

inline Geom tet_geometry(const double* X, const int* v) {
  Geom g;
  const double* x0 = X + 3 * v[0];
  double Jm[3][3];  // columns: x1-x0, x2-x0, x3-x0
  for (int c = 0; c < 3; ++c) {
    const double* xc = X + 3 * v[c + 1];
    for (int r = 0; r < 3; ++r) Jm[r][c] = xc[r] - x0[r];
  }
  Ten<double> J;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) J(r, c) = Jm[r][c];
  double dJ = det(J);
  Ten<double> Ji = inverse(J);  // rows of Ji = gradients of xi, eta, zeta
  for (int a = 1; a < 4; ++a)
    for (int k = 0; k < 3; ++k) g.GBF[a][k] = Ji(a - 1, k);
  for (int k = 0; k < 3; ++k) g.GBF[0][k] = -(g.GBF[1][k] + g.GBF[2][k] + g.GBF[3][k]);
  for (int a = 0; a < 4; ++a) g.BF[a] = 0.25;
  g.wdv = dJ / 6.0;
  static const int E[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
  double h = 0.0;
  for (int e = 0; e < 6; ++e) {
    const double* a = X + 3 * v[E[e][0]];
    const double* b = X + 3 * v[E[e][1]];
    double l = std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
    h += l * l;
  }
  g.h = std::sqrt(h / 6.0);
  return g;
}

// ---------------------------------------------------------------- arguments
struct Mat {
  double E, nu, K, Y, c0;
};

struct Args {
  // mesh
  int num_nodes, num_elems;
  const double* coords;  // N x 3
  const int* tets;       // E x 4
  const int* elem_set;   // E (nullable -> set 0)
  const double* mats;    // per element set: E, nu, K, Y, c0
  int model;             // 0 neohookean, 1 J2
  int stabilization;
  // chain
  int mode;              // 0 NONE, 1 PRIMAL, 2 ADJOINT (src/goal_eval_modes.hpp:6)
  int fad;               // 1 = Jacobian chain (FADT), 0 = residual chain (ST)
  int save;              // save_state flag of the model evaluators
  int qoi;               // 0 none, 1 avg disp, 2 KS max von Mises
  double rho;            // KS parameter
  int error_chain;       // 1 = Mechanics::build_error weights
  const double* zu_diff; // N x 3  (u_z_diff)
  const double* zp_diff; // N      (p_z_diff)
  const double* zp_coarse; // N    (p_z_coarse)
  // fields
  const double* u;       // N x 3
  const double* p;       // N
  // states in
  const double* Fp_old;  // E x 9
  const double* eqps_old;// E
  const double* sigma_in;// E x 9 (stored Cauchy stress, KS pre-pass)
  // states out (nullable)
  double* sigma_out;     // E x 9
  double* Fp_out;        // E x 9
  double* eqps_out;      // E
  // outputs (nullable)
  double* R;             // 4N
  const int* row_ptr;    // 4N+1
  const int* col_idx;    // nnz
  double* vals;          // nnz
  double* dMdu;          // 4N
  double* qoi_value;     // 1
  int* num_plastic;      // 1
  int* status;           // 1: 0 ok, 1 return-map failure
  // 1 = also write Fp = Fp_old at elastic points. 0 is goal's behaviour
  // (src/goal_J2.cpp:97-136 writes Fp only where the point yields, so an
  // earlier Newton iterate's plastic Fp survives at points that end elastic
  // and States::update commits it); 1 is the option that makes the committed
  // state the converged iterate's.
  int fp_elastic_reset;
};

// ---------------------------------------------------------------- von Mises
template <typename T>
T von_mises(const Ten<T>& s) {
  T s1 = (s(0, 0) - s(1, 1)) * (s(0, 0) - s(1, 1));
  T s2 = (s(1, 1) - s(2, 2)) * (s(1, 1) - s(2, 2));
  T s3 = (s(2, 2) - s(0, 0)) * (s(2, 2) - s(0, 0));
  T s4 = s(0, 1) * s(0, 1);
  T s5 = s(1, 2) * s(1, 2);
  T s6 = s(2, 0) * s(2, 0);
  T s7 = 0.5 * (s1 + s2 + s3 + 6.0 * (s4 + s5 + s6));
  return sqrt(s7);
}

// ---------------------------------------------------------------- element
template <typename T>
struct ElemOut {
  T Ru[4][3];
  T Rp[4];
  T qoi;
};

// Evaluates the residual chain of one element in the order of
// Mechanics::build_resid (src/goal_mechanics.cpp:97-146), followed by an
// optional QoI evaluator (src/goal_mechanics.cpp:148-167).
template <typename T>
int eval_element(const Args& A, int e, double ks_max, double ks_scale, ElemOut<T>& out) {
  const int* v = A.tets + 4 * e;
  int es = A.elem_set ? A.elem_set[e] : 0;
  Mat m;
  m.E = A.mats[5 * es + 0]; m.nu = A.mats[5 * es + 1]; m.K = A.mats[5 * es + 2];
  m.Y = A.mats[5 * es + 3]; m.c0 = A.mats[5 * es + 4];
  const double kappa = m.E / (3.0 * (1.0 - 2.0 * m.nu));
  const double mu = m.E / (2.0 * (1.0 + m.nu));
  Geom g = tet_geometry(A.coords, v);
  const double ipw = 1.0 / 6.0;
  const double dv = g.wdv / ipw;

  // gather (Displacement<T>::gather, Pressure<T>::gather): dof n*4+d / n*4+3
  T un[4][3], pn[4];
  for (int n = 0; n < 4; ++n) {
    for (int d = 0; d < 3; ++d) {
      un[n][d] = T(A.u[3 * v[n] + d]);
      if constexpr (!std::is_same<T, double>::value) un[n][d].diff(n * 4 + d);
      out.Ru[n][d] = T(0.0);
    }
    pn[n] = T(A.p[v[n]]);
    if constexpr (!std::is_same<T, double>::value) pn[n].diff(n * 4 + 3);
    out.Rp[n] = T(0.0);
  }
  out.qoi = T(0.0);

  // interpolation at the point (Displacement::at_point, Pressure::at_point)
  T uval[3], ugrad[3][3], pval, pgrad[3];
  for (int i = 0; i < 3; ++i) {
    uval[i] = un[0][i] * g.BF[0];
    for (int n = 1; n < 4; ++n) uval[i] += un[n][i] * g.BF[n];
    for (int j = 0; j < 3; ++j) {
      ugrad[i][j] = un[0][i] * g.GBF[0][j];
      for (int n = 1; n < 4; ++n) ugrad[i][j] += un[n][i] * g.GBF[n][j];
    }
  }
  pval = pn[0] * g.BF[0];
  for (int n = 1; n < 4; ++n) pval += pn[n] * g.BF[n];
  for (int i = 0; i < 3; ++i) {
    pgrad[i] = pn[0] * g.GBF[0][i];
    for (int n = 1; n < 4; ++n) pgrad[i] += pn[n] * g.GBF[n][i];
  }

  // weights: VectorWeight/ScalarWeight (primal) or the DWR adjoint weights
  double wu_grad[4][3][3];  // w->grad(n,i,j) of the momentum weight
  double wp_val[4];         // pw->val(n)
  double ws_grad[4][3];     // weight used by Stabilization (pw or pwc) ->grad(n,j)
  if (!A.error_chain) {
    for (int n = 0; n < 4; ++n) {
      wp_val[n] = g.BF[n];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) wu_grad[n][i][j] = g.GBF[n][j];
      for (int j = 0; j < 3; ++j) ws_grad[n][j] = g.GBF[n][j];
    }
  } else {
    // DisplacementAdjoint::at_point with u_z_diff; PressureAdjoint with
    // p_z_diff ("pw") and p_z_coarse ("pwc", used by stabilization).
    double z[3] = {0, 0, 0}, gz[3][3] = {{0}}, zp = 0, gzp[3] = {0}, zc = 0, gzc[3] = {0};
    for (int n = 0; n < 4; ++n) {
      for (int i = 0; i < 3; ++i) {
        z[i] += g.BF[n] * A.zu_diff[3 * v[n] + i];
        for (int j = 0; j < 3; ++j) gz[i][j] += A.zu_diff[3 * v[n] + i] * g.GBF[n][j];
      }
      zp += g.BF[n] * A.zp_diff[v[n]];
      zc += g.BF[n] * A.zp_coarse[v[n]];
      for (int j = 0; j < 3; ++j) {
        gzp[j] += A.zp_diff[v[n]] * g.GBF[n][j];
        gzc[j] += A.zp_coarse[v[n]] * g.GBF[n][j];
      }
    }
    for (int n = 0; n < 4; ++n) {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) wu_grad[n][i][j] = gz[i][j] * g.BF[n] + z[i] * g.GBF[n][j];
      wp_val[n] = zp * g.BF[n];
      for (int j = 0; j < 3; ++j) ws_grad[n][j] = gzc[j] * g.BF[n] + zc * g.GBF[n][j];
    }
  }

  // Kinematics
  Ten<T> F;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) F(i, j) = ugrad[i][j];
  for (int i = 0; i < 3; ++i) F(i, i) += 1.0;
  T J = det(F);

  // Model
  Ten<T> sigma;
  Ten<T> I = eye<T>();
  int status = 0;
  bool plastic = false;
  if (A.model == 0) {
    T Jm13 = 1.0 / cbrt(J);
    T Jm23 = Jm13 * Jm13;
    T Jm53 = Jm23 * Jm23 * Jm13;
    Ten<T> b = matmul(F, transpose(F));
    T pm = 0.5 * kappa * (J - 1.0 / J);
    Ten<T> db = dev(b);
    for (int k = 0; k < 9; ++k) sigma.a[k] = mu * Jm53 * db.a[k] + pm * I.a[k];
  } else {
    const double sq23 = std::sqrt(2.0 / 3.0);
    T Jm23 = pow(J, -2.0 / 3.0);
    Ten<T> Fp;
    for (int k = 0; k < 9; ++k) Fp.a[k] = T(A.Fp_old[9 * e + k]);
    Ten<T> Fpinv = inverse(Fp);
    Ten<T> Cpinv = matmul(Fpinv, transpose(Fpinv));
    Ten<T> be = matmul(matmul(scale(Jm23, F), Cpinv), transpose(F));
    Ten<T> s = scale(mu, dev(be));
    T mubar = trace(be) * mu / 3.0;
    T smag = norm(s);
    T eqps = T(A.eqps_old[e]);
    T f = smag - sq23 * (m.Y + m.K * eqps);
    if (f > 1.0e-12) {
      plastic = true;
      int iter = 0;
      bool converged = false;
      T dgam = T(0.0);
      T H(0.0), dH(0.0), alpha(0.0), res(0.0);
      T X = T(0.0);
      T R = f;
      T dRdX = -2.0 * mubar * (1.0 + H / (3.0 * mubar));
      while ((!converged) && (iter < 30)) {
        iter++;
        X = X - R / dRdX;
        alpha = eqps + sq23 * X;
        H = m.K * alpha;
        dH = T(m.K);
        R = smag - (2.0 * mubar * X + sq23 * (m.Y + H));
        dRdX = -2.0 * mubar * (1.0 + dH / (3.0 * mubar));
        double rs = abs(R);
        if ((rs < 1.0e-11) || (rs / m.Y < 1.0e-11) || (rs / val(f) < 1.0e-11)) converged = true;
        if (iter == 30) status = 1;  // fail("J2: return mapping failed")
      }
      dgam = X;
      Ten<T> N = scale(1.0 / smag, s);
      for (int k = 0; k < 9; ++k) s.a[k] -= 2.0 * mubar * dgam * N.a[k];
      if (A.save && A.eqps_out) A.eqps_out[e] = val(alpha);
      if (A.save && A.Fp_out) {
        Ten<double> XN, Fpo;
        for (int k = 0; k < 9; ++k) { XN.a[k] = val(dgam) * val(N.a[k]); Fpo.a[k] = A.Fp_old[9 * e + k]; }
        Ten<double> Fpn = matmul(expm(XN), Fpo);
        for (int k = 0; k < 9; ++k) A.Fp_out[9 * e + k] = Fpn.a[k];
      }
    } else {
      if (A.save && A.eqps_out) A.eqps_out[e] = val(eqps);
      if (A.save && A.Fp_out && A.fp_elastic_reset)
        for (int k = 0; k < 9; ++k) A.Fp_out[9 * e + k] = A.Fp_old[9 * e + k];
    }
    T pm = 0.5 * kappa * (J - 1.0 / J);
    for (int k = 0; k < 9; ++k) sigma.a[k] = s.a[k] / J + pm * I.a[k];
  }
  if (A.save && A.sigma_out)
    for (int k = 0; k < 9; ++k) A.sigma_out[9 * e + k] = val(sigma.a[k]);

  // Mixed
  {
    T pbar = T(0.0);
    for (int i = 0; i < 3; ++i) pbar += sigma(i, i);
    pbar /= 3.0;
    for (int i = 0; i < 3; ++i) sigma(i, i) += pval - pbar;
    if (A.save && A.sigma_out)
      for (int k = 0; k < 9; ++k) A.sigma_out[9 * e + k] = val(sigma.a[k]);
  }

  // MResidual: P = J sigma F^{-T}
  {
    Ten<T> Finv = inverse(F);
    Ten<T> P = matmul(scale(J, sigma), transpose(Finv));
    for (int n = 0; n < 4; ++n)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out.Ru[n][i] += P(i, j) * wu_grad[n][i][j] * ipw * dv;
  }

  // PResidual (large strain)
  {
    T dUdJ = 0.5 * (J - 1.0 / J);
    for (int n = 0; n < 4; ++n) out.Rp[n] += ((pval / kappa) - dUdJ) * wp_val[n] * ipw * dv;
  }

  // Stabilization
  if (A.stabilization) {
    double h = g.h;
    double tau = 0.5 * m.c0 * h * h / mu;
    Ten<T> Cinv = inverse(matmul(transpose(F), F));
    for (int n = 0; n < 4; ++n)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out.Rp[n] += tau * J * Cinv(i, j) * pgrad[i] * ws_grad[n][j] * ipw * dv;
  }

  // QoI
  if (A.qoi == 1) {
    for (int i = 0; i < 3; ++i) out.qoi += uval[i] * ipw * dv;
    out.qoi /= 3.0;
  } else if (A.qoi == 2) {
    T vm = von_mises(sigma);
    out.qoi += (1.0 / (A.rho * ks_scale)) * exp(A.rho * (vm - ks_max)) * ipw * dv;
  }
  if (plastic && A.num_plastic) (*A.num_plastic)++;
  return status;
}

inline int find_col(const Args& A, int row, int col) {
  const int* b = A.col_idx + A.row_ptr[row];
  const int* e = A.col_idx + A.row_ptr[row + 1];
  const int* it = std::lower_bound(b, e, col);
  if (it == e || *it != col) return -1;
  return A.row_ptr[row] + (int)(it - b);
}

// The KS pre-pass over stored Cauchy stresses (src/goal_ks_vm.cpp:36-76).
inline void ks_prepass(const Args& A, double& mx, double& sc) {
  mx = 0.0;
  for (int e = 0; e < A.num_elems; ++e) {
    Ten<double> s;
    for (int k = 0; k < 9; ++k) s.a[k] = A.sigma_in[9 * e + k];
    mx = std::max(mx, von_mises(s));
  }
  sc = 0.0;
  for (int e = 0; e < A.num_elems; ++e) {
    Ten<double> s;
    for (int k = 0; k < 9; ++k) s.a[k] = A.sigma_in[9 * e + k];
    Geom g = tet_geometry(A.coords, A.tets + 4 * e);
    double vm = von_mises(s);
    sc += std::exp(A.rho * (vm - mx)) * (1.0 / 6.0) * (g.wdv * 6.0);
  }
}

}  // namespace orc

using namespace orc;

extern "C" {

// Node-adjacency CSR graph of the mesh expanded by num_eqs (src/goal_disc.cpp:307-332):
// row dof = node*neq+eq; columns = every dof of every element touching the row's
// node, sorted ascending. Call with row_ptr/col_idx null to get nnz.
long long orc_csr_graph(int num_nodes, int num_elems, const int* tets, int neq, int* row_ptr, int* col_idx) {
  std::vector<std::vector<int>> adj(num_nodes);
  for (int e = 0; e < num_elems; ++e)
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) adj[tets[4 * e + a]].push_back(tets[4 * e + b]);
  long long nnz = 0;
  for (int n = 0; n < num_nodes; ++n) {
    std::sort(adj[n].begin(), adj[n].end());
    adj[n].erase(std::unique(adj[n].begin(), adj[n].end()), adj[n].end());
    nnz += (long long)adj[n].size() * neq * neq;
  }
  if (!row_ptr) return nnz;
  long long k = 0;
  for (int n = 0; n < num_nodes; ++n) {
    for (int eq = 0; eq < neq; ++eq) {
      row_ptr[n * neq + eq] = (int)k;
      for (int m : adj[n])
        for (int l = 0; l < neq; ++l) col_idx[k++] = m * neq + l;
    }
  }
  row_ptr[num_nodes * neq] = (int)k;
  return nnz;
}

// assemble(E, SolInfo*) for one evaluator chain (src/goal_assembly.cpp:65-88).
// Outputs are accumulated (callers zero them, as SolInfo::zero_all does).
int orc_assemble(const Args* a) {
  const Args& A = *a;
  double ks_max = 0.0, ks_scale = 1.0;
  if (A.qoi == 2) ks_prepass(A, ks_max, ks_scale);
  int status = 0;
  double qoi = 0.0;
  if (A.num_plastic) *A.num_plastic = 0;
  for (int e = 0; e < A.num_elems; ++e) {
    const int* v = A.tets + 4 * e;
    int lids[16];
    for (int n = 0; n < 4; ++n)
      for (int q = 0; q < 4; ++q) lids[4 * n + q] = 4 * v[n] + q;
    if (A.fad) {
      ElemOut<Dual> o;
      status |= eval_element<Dual>(A, e, ks_max, ks_scale, o);
      for (int n = 0; n < 4; ++n) {
        for (int q = 0; q < 4; ++q) {
          const Dual& r = (q < 3) ? o.Ru[n][q] : o.Rp[n];
          int row = lids[4 * n + q];
          if (A.R && A.mode != 0) A.R[row] += r.v;
          if (A.vals && A.mode == 1) {
            for (int c = 0; c < 16; ++c) {
              int k = find_col(A, row, lids[c]);
              if (k >= 0) A.vals[k] += r.d[c];
            }
          } else if (A.vals && A.mode == 2) {
            for (int c = 0; c < 16; ++c) {
              int k = find_col(A, lids[c], row);
              if (k >= 0) A.vals[k] += r.d[c];
            }
          }
        }
      }
      if (A.qoi) {
        if (A.dMdu)
          for (int c = 0; c < 16; ++c) A.dMdu[lids[c]] += o.qoi.d[c];
        qoi += o.qoi.v;
      }
    } else {
      ElemOut<double> o;
      status |= eval_element<double>(A, e, ks_max, ks_scale, o);
      if (A.R && A.mode != 0) {
        for (int n = 0; n < 4; ++n) {
          for (int q = 0; q < 3; ++q) A.R[lids[4 * n + q]] += o.Ru[n][q];
          A.R[lids[4 * n + 3]] += o.Rp[n];
        }
      }
      if (A.qoi) qoi += o.qoi;
    }
  }
  if (A.qoi == 2) qoi = ks_max + (1.0 / A.rho) * std::log(ks_scale);
  if (A.qoi_value) *A.qoi_value = qoi;
  if (A.status) *A.status = status;
  return status;
}

// The same Jacobian chain evaluated with all host threads: elements are
// evaluated in parallel into per-element buffers, then scattered in element
// order (same sums as orc_assemble). Used as the timed CPU baseline.
int orc_assemble_parallel(const Args* a, int chunk) {
  const Args& A = *a;
  if (!A.fad || A.qoi != 0) return orc_assemble(a);
  int status = 0;
  std::vector<double> buf((size_t)chunk * 272);
  for (int e0 = 0; e0 < A.num_elems; e0 += chunk) {
    int ne = std::min(chunk, A.num_elems - e0);
#pragma omp parallel for schedule(dynamic, 64) reduction(| : status)
    for (int k = 0; k < ne; ++k) {
      ElemOut<Dual> o;
      status |= eval_element<Dual>(A, e0 + k, 0.0, 1.0, o);
      double* b = buf.data() + (size_t)k * 272;
      for (int n = 0; n < 4; ++n)
        for (int q = 0; q < 4; ++q) {
          const Dual& r = (q < 3) ? o.Ru[n][q] : o.Rp[n];
          b[4 * n + q] = r.v;
          for (int c = 0; c < 16; ++c) b[16 + 16 * (4 * n + q) + c] = r.d[c];
        }
    }
    for (int k = 0; k < ne; ++k) {
      const int* v = A.tets + 4 * (e0 + k);
      const double* b = buf.data() + (size_t)k * 272;
      int lids[16];
      for (int n = 0; n < 4; ++n)
        for (int q = 0; q < 4; ++q) lids[4 * n + q] = 4 * v[n] + q;
      for (int r = 0; r < 16; ++r) {
        if (A.R) A.R[lids[r]] += b[r];
        if (A.vals)
          for (int c = 0; c < 16; ++c) {
            int kk = (A.mode == 1) ? find_col(A, lids[r], lids[c]) : find_col(A, lids[c], lids[r]);
            if (kk >= 0) A.vals[kk] += b[16 + 16 * r + c];
          }
      }
    }
  }
  if (A.status) *A.status = status;
  return status;
}

// set_resid_dbcs / set_jac_dbcs for one boundary condition (src/goal_dbcs.cpp:39-99).
// rows are dofs node*4+eq, vals the prescribed values; jac != 0 also replaces
// the CSR row by the identity row and zeroes dMdu.
void orc_apply_dbc(int nrows, const int* rows, const double* values, const double* u, int jac,
                   double* R, const int* row_ptr, const int* col_idx, double* vals, double* dMdu) {
  for (int k = 0; k < nrows; ++k) {
    int row = rows[k];
    int node = row / 4, eq = row % 4;
    double sol = u[3 * node + eq];
    R[row] = sol - values[k];
    if (jac) {
      if (dMdu) dMdu[row] = 0.0;
      for (int j = row_ptr[row]; j < row_ptr[row + 1]; ++j) vals[j] = (col_idx[j] == row) ? 1.0 : 0.0;
    }
  }
}

// set_tbcs for one side set (src/goal_tbcs.cpp:29-85): one point at the
// triangle centroid, R[n*4+d] -= T_d w_n(d) |area|. traction holds T per side
// (S x 3, already evaluated at the centroid). zu (nullable) selects the DWR
// weight z_d(centroid) phi_n instead of phi_n.
void orc_apply_traction(int nsides, const int* tris, const double* coords, const double* traction,
                        const double* zu, double* R) {
  for (int s = 0; s < nsides; ++s) {
    const int* t = tris + 3 * s;
    const double* a = coords + 3 * t[0];
    const double* b = coords + 3 * t[1];
    const double* c = coords + 3 * t[2];
    double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    double e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    double dv = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    double ipw = 0.5;
    double BF = 1.0 / 3.0;
    double z[3] = {1.0, 1.0, 1.0};
    if (zu)
      for (int d = 0; d < 3; ++d) z[d] = BF * (zu[3 * t[0] + d] + zu[3 * t[1] + d] + zu[3 * t[2] + d]);
    for (int n = 0; n < 3; ++n)
      for (int d = 0; d < 3; ++d) {
        double w = zu ? z[d] * BF : BF;
        R[4 * t[n] + d] -= traction[3 * s + d] * w * ipw * dv;
      }
  }
}

// Per-element geometry (volume and stabilization size) for checks.
void orc_geometry(int num_elems, const double* coords, const int* tets, double* vol, double* h, double* grads) {
  for (int e = 0; e < num_elems; ++e) {
    Geom g = tet_geometry(coords, tets + 4 * e);
    if (vol) vol[e] = g.wdv;
    if (h) h[e] = g.h;
    if (grads)
      for (int a = 0; a < 4; ++a)
        for (int k = 0; k < 3; ++k) grads[12 * e + 3 * a + k] = g.GBF[a][k];
  }
}

// Element indicators |sum_d e_u,d + e_p| at the centroid (src/goal_error.cpp:7-35)
// and the bound sum over vertices (src/goal_error.cpp:37-56).
double orc_error(int num_nodes, int num_elems, const int* tets, const double* ue, const double* pe, double* elem_err) {
  for (int e = 0; e < num_elems; ++e) {
    const int* v = tets + 4 * e;
    double pu = 0.25 * pe[v[0]];
    for (int n = 1; n < 4; ++n) pu += 0.25 * pe[v[n]];
    double u[3];
    for (int d = 0; d < 3; ++d) {
      u[d] = 0.25 * ue[3 * v[0] + d];
      for (int n = 1; n < 4; ++n) u[d] += 0.25 * ue[3 * v[n] + d];
    }
    double total = 0.0;
    for (int d = 0; d < 3; ++d) total += u[d];
    total += pu;
    elem_err[e] = std::fabs(total);
  }
  double sum = 0.0;
  for (int n = 0; n < num_nodes; ++n) {
    double t = 0.0;
    for (int d = 0; d < 3; ++d) t += ue[3 * n + d];
    t += pe[n];
    sum += std::fabs(t);
  }
  return sum;
}

// Matrix exponential used for the Fp update (exposed for tests).
void orc_expm(const double* A, double* out) {
  Ten<double> a;
  for (int k = 0; k < 9; ++k) a.a[k] = A[k];
  Ten<double> r = expm(a);
  for (int k = 0; k < 9; ++k) out[k] = r.a[k];
}

}  // extern "C"
