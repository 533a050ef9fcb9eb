// Element kernels: residual, hand-derived tangent, QoI and DWR error chain of
// goal's stabilized mixed u-p mechanics on linear tets, one thread per element,
// elements of one colour per launch (no two of them share a node, so the
// scatter into the 4x4-block matrix needs no atomics and is deterministic).
//
// Reference chain (one integration point, src/goal_assembly.cpp:65-88):
//   Kinematics F = I + grad u, J = det F                   src/goal_kinematics.cpp:18-25
//   Neohookean sigma = mu J^-5/3 dev(F F^T) + k/2 (J-1/J) I  src/goal_neohookean.cpp:59-86
//   J2 trial be = J^-2/3 F Cp^-1 F^T, s = mu dev(be), radial return with linear
//      hardening, eqps/Fp/sigma state writes                src/goal_J2.cpp:71-156
//   Mixed sigma_ii += p - tr(sigma)/3                       src/goal_mixed.cpp:33-46
//   MResidual R^u_ai += P_ij dphi_a/dx_j w dv, P = J sigma F^-T   src/goal_mresidual.cpp:25-32
//   PResidual R^p_a += (p/kappa - (J-1/J)/2) phi_a w dv     src/goal_presidual.cpp:53-59
//   Stabilization R^p_a += tau J C^-1_ij dp/dx_i dphi_a/dx_j w dv, tau = c0 h^2/(2 mu)
//                                                            src/goal_stabilization.cpp:59-80
//   scatter PRIMAL (row-wise) / ADJOINT (transposed)        src/goal_displacement.cpp:177-214
//   QoI avg disp, KS max von Mises                          src/goal_avg_disp.cpp:16-21, src/goal_ks_vm.cpp:88-98
//   DWR weights z_diff phi_a, stabilization with z_coarse   src/goal_displacement_adjoint.cpp:37-53,
//                                                            src/goal_pressure_adjoint.cpp:38-49,
//                                                            src/goal_mechanics.cpp:169-218
//
// Tangent (replaces Sacado FAD). With G_a = grad phi_a, H = F^-T, h_a = H G_a,
// C = Cp^-1 (identity for neo-Hookean), B = F C F^T, Ic = tr B, m_a = F C G_a,
// q_a = m_a - Ic/3 h_a, alpha = mu J^-2/3, s = alpha dev B, the deviatoric
// Kirchhoff stress is S = gamma s (gamma = 1 when elastic) and
//   P G_a = S h_a + p J h_a.
// Its derivative in direction u_bk (dF = e_k (x) G_b) is
//   K^uu_{ai,bk} = V [ gamma alpha c_ab d_ik + h_ai X_bk + q_ai Y_bk + h_bi Z_ak ]
//   c_ab = G_a.C G_b,  X_b = -2/3 gamma alpha m_b + pJ h_b,
//   Y_b = -2/3 gamma alpha h_b + alpha dgamma_b,  Z_a = (gamma alpha Ic/3 - pJ) h_a,
// and for the plastic return (X = f / (2 mubar + kh), kh = 2K/3, or kh = 0 when
// goal's Newton loop stops after its first iterate)
//   dgamma_b = -A1 dmubar_b - A2 dsmag_b,  dmubar_b = 2 alpha/3 q_b,
//   dsmag_b = -2/3 smag h_b + 2 alpha/smag s m_b,
//   A1 = 2 f kh / (c^2 smag), A2 = 2 mubar k0 / (c smag^2).
// The pressure rows and columns:
//   K^up_{ai,b} = V J h_ai / 4
//   K^pu_{a,bk} = V [ h_bk (tau J w_a - (J+1/J)/8) - tau J e_ab v_k - tau J w_b h_ak ]
//   K^pp_{ab}   = V [ 1/(16 kappa) + tau J e_ab ]
// with v = H grad p, w_a = v.h_a, e_ab = h_a.h_b.
#include "mechanics.cuh"

namespace goal {

namespace {

struct ElemArgs {
  DiscView d;
  const double* mats;
  const double* U;
  const double* Fp_old;
  const double* eqps_old;
  const double* Cpinv;
  double* sigma;
  double* Fp;
  double* eqps;
  double* Apend;   // 6 x E deferred plastic increments (see StatesDev)
  int* pend;
  double* R;
  double* A;
  double* dMdu;
  double* qoi_elem;
  const double* Zd;
  const double* Zc;
  int* status;
  double* ebuf;    // two-phase mode: per element [R (16) | 16 blocks x 16] (stride estride)
  double* dbuf;    // two-phase mode: per element dM/du (16)
  int estride;
  int ebase;       // element slot of the buffers' first entry (a chunk's first element)
  int begin, end;
  int stab, save, overwrite, qoi;
  int fp_reset;    // also write Fp = Fp_old at elastic points (goal leaves Fp as it was)
  double rho, ks_max, ks_scale;
};

__device__ __forceinline__ void ld4(const double* p, double& a, double& b, double& c, double& d) {
  double4_32a v = *reinterpret_cast<const double4_32a*>(p);
  a = v.x; b = v.y; c = v.z; d = v.w;
}
__device__ __forceinline__ void st4(double* p, double a, double b, double c, double d) {
  double4_32a v;
  v.x = a; v.y = b; v.z = c; v.w = d;
  *reinterpret_cast<double4_32a*>(p) = v;
}
__device__ __forceinline__ void acc4(double* p, bool first, double a, double b, double c, double d) {
  if (!first) {
    double x, y, z, w;
    ld4(p, x, y, z, w);
    a += x; b += y; c += z; d += w;
  }
  st4(p, a, b, c, d);
}

constexpr int kMatStride = 8;  // kappa, mu, K, Y, c0, 1/kappa, c0/(2 mu), 1/(16 kappa)
constexpr double kThird = 1.0 / 3.0;

// 1/(k+1) for the exponential series
__constant__ double c_inv_k[80];

// exp(A) for a symmetric traceless 3x3 A (A = dgam N) by the power series
// reduced with Cayley-Hamilton: A^3 = I2 A + I3 I, I2 = tr(A^2)/2, I3 = det A.
// Returns false if the series did not settle in 80 terms.
__device__ bool exp_traceless_sym(const double A[3][3], double out[3][3]) {
  double A2[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A2[i][j] = A[i][0] * A[0][j] + A[i][1] * A[1][j] + A[i][2] * A[2][j];
  double I2 = 0.5 * (A2[0][0] + A2[1][1] + A2[2][2]);
  double I3 = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
              A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
  // term_k = A^k/k! = x I + y A + z A^2
  double x = 0.0, y = 0.0, z = 1.0 / 2.0;  // k = 2
  double s0 = 1.0, s1 = 1.0, s2 = 0.5;
  bool ok = false;
  for (int k = 2; k < 80; ++k) {
    double nx = z * I3, ny = x + z * I2, nz = y;
    const double inv = c_inv_k[k];
    x = nx * inv; y = ny * inv; z = nz * inv;
    s0 += x; s1 += y; s2 += z;
    double mag = fabs(x) + fabs(y) + fabs(z);
    if (mag < 1e-20 * (fabs(s0) + fabs(s1) + fabs(s2))) { ok = true; break; }
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) out[i][j] = s1 * A[i][j] + s2 * A2[i][j] + (i == j ? s0 : 0.0);
  return ok;
}

// BUF: element outputs go to the per-element buffer (phase 1 of the two-phase
// assembly) instead of being accumulated in place by one colour at a time.
// DSUM (with BUF): of the four diagonal element blocks (a, a) only column 3
// (K^up_a, K^pp_aa) is formed and stored, packed in the block's first four
// slots. The u columns of a matrix row sum to zero over the row's blocks (the
// gradients of a linear tet's shape functions sum to zero, and every u column
// of K^uu and K^pu is linear in them), so k_gather_diag forms the diagonal
// blocks' u columns as negated sums of the off-diagonal blocks.
template <int MODEL, int MODE, bool JAC, bool ERR, bool BUF, bool DSUM = false>
__global__ void __launch_bounds__(128) k_elem(const ElemArgs a) {
  const int s = a.begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.end) return;
  const int E = a.d.num_elems;

  int v[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) v[q] = __ldg(a.d.tets + q * E + s);
  double G[4][3];
#pragma unroll
  for (int q = 0; q < 12; ++q) G[q / 3][q % 3] = __ldg(a.d.grads + q * E + s);
  const double V = __ldg(a.d.vol + s);
  const int es = __ldg(a.d.elem_set + s);
  const double* mrow = a.mats + kMatStride * es;
  const double kappa = __ldg(mrow + 0);
  const double mu = __ldg(mrow + 1);
  const double Kh = __ldg(mrow + 2);
  const double Yld = __ldg(mrow + 3);
  const double inv_kappa = __ldg(mrow + 5);   // 1 / kappa
  const double tau_coef = __ldg(mrow + 6);    // c0 / (2 mu)
  const double pp_coef = __ldg(mrow + 7);     // 1 / (16 kappa)

  // gather + interpolation (Displacement/Pressure at_point)
  double un[4][3], pn[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) ld4(a.U + 4 * v[q], un[q][0], un[q][1], un[q][2], pn[q]);
  double F[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double t = un[0][i] * G[0][j];
      t += un[1][i] * G[1][j];
      t += un[2][i] * G[2][j];
      t += un[3][i] * G[3][j];
      F[i][j] = t;
    }
  F[0][0] += 1.0; F[1][1] += 1.0; F[2][2] += 1.0;
  const double pval = ((pn[0] * 0.25 + pn[1] * 0.25) + pn[2] * 0.25) + pn[3] * 0.25;
  double gp[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) gp[i] = ((pn[0] * G[0][i] + pn[1] * G[1][i]) + pn[2] * G[2][i]) + pn[3] * G[3][i];

  // kinematics: J and H = F^-T
  double cof[3][3];
  cof[0][0] = F[1][1] * F[2][2] - F[1][2] * F[2][1];
  cof[0][1] = F[1][2] * F[2][0] - F[1][0] * F[2][2];
  cof[0][2] = F[1][0] * F[2][1] - F[1][1] * F[2][0];
  cof[1][0] = F[0][2] * F[2][1] - F[0][1] * F[2][2];
  cof[1][1] = F[0][0] * F[2][2] - F[0][2] * F[2][0];
  cof[1][2] = F[0][1] * F[2][0] - F[0][0] * F[2][1];
  cof[2][0] = F[0][1] * F[1][2] - F[0][2] * F[1][1];
  cof[2][1] = F[0][2] * F[1][0] - F[0][0] * F[1][2];
  cof[2][2] = F[0][0] * F[1][1] - F[0][1] * F[1][0];
  const double J = F[0][0] * cof[0][0] + F[0][1] * cof[0][1] + F[0][2] * cof[0][2];
  const double Jinv = 1.0 / J;
  double H[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) H[i][j] = cof[i][j] * Jinv;

  // right Cauchy-Green of the plastic part (identity for neo-Hookean)
  double C[6] = {1.0, 1.0, 1.0, 0.0, 0.0, 0.0};  // xx yy zz xy yz xz
  double FC[3][3];  // F C
  if constexpr (MODEL == MODEL_J2) {
#pragma unroll
    for (int q = 0; q < 6; ++q) C[q] = __ldg(a.Cpinv + q * E + s);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      FC[i][0] = F[i][0] * C[0] + F[i][1] * C[3] + F[i][2] * C[5];
      FC[i][1] = F[i][0] * C[3] + F[i][1] * C[1] + F[i][2] * C[4];
      FC[i][2] = F[i][0] * C[5] + F[i][1] * C[4] + F[i][2] * C[2];
    }
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) FC[i][j] = F[i][j];
  }
  // B = F C F^T (symmetric)
  double B00 = FC[0][0] * F[0][0] + FC[0][1] * F[0][1] + FC[0][2] * F[0][2];
  double B11 = FC[1][0] * F[1][0] + FC[1][1] * F[1][1] + FC[1][2] * F[1][2];
  double B22 = FC[2][0] * F[2][0] + FC[2][1] * F[2][1] + FC[2][2] * F[2][2];
  double B01 = FC[0][0] * F[1][0] + FC[0][1] * F[1][1] + FC[0][2] * F[1][2];
  double B12 = FC[1][0] * F[2][0] + FC[1][1] * F[2][1] + FC[1][2] * F[2][2];
  double B02 = FC[0][0] * F[2][0] + FC[0][1] * F[2][1] + FC[0][2] * F[2][2];
  const double Ic = B00 + B11 + B22;
  const double Jm13 = rcbrt(J);
  const double alpha = mu * (Jm13 * Jm13);
  const double Ic3 = Ic * kThird;
  // trial deviatoric Kirchhoff stress s = alpha dev(B)
  const double s00 = alpha * (B00 - Ic3), s11 = alpha * (B11 - Ic3), s22 = alpha * (B22 - Ic3);
  const double s01 = alpha * B01, s12 = alpha * B12, s02 = alpha * B02;

  // J2 radial return (closed form of goal's scalar Newton loop)
  double gamma = 1.0;
  bool plastic = false;
  double smag = 0.0, mubar = 0.0, fyield = 0.0, k0 = 0.0, cc = 1.0, kh = 0.0, Xr = 0.0, rsmag = 0.0, rcc = 1.0;
  const double sq23 = 0.81649658092772603273;  // sqrt(2/3)
  if (MODEL == MODEL_J2 || (a.qoi == QOI_KS_VM)) {
    smag = sqrt(s00 * s00 + s11 * s11 + s22 * s22 + 2.0 * (s01 * s01 + s12 * s12 + s02 * s02));
  }
  if (MODEL == MODEL_J2) {
    mubar = alpha * Ic3;
    const double eq_old = __ldg(a.eqps_old + s);
    k0 = sq23 * (Yld + Kh * eq_old);
    fyield = smag - k0;
    if (fyield > 1.0e-12) {
      plastic = true;
      // reciprocals formed once (a division costs several FP64 instructions)
      rsmag = 1.0 / smag;
      const double r2mu = 1.0 / (2.0 * mubar);
      // first Newton iterate of src/goal_J2.cpp:101-121 (H = 0 in the first slope)
      double X1 = fyield * r2mu;
      double alpha1 = eq_old + sq23 * X1;
      double R1 = smag - (2.0 * mubar * X1 + sq23 * (Yld + Kh * alpha1));
      double r1 = fabs(R1);
      // goal's tests |R| < 1e-11, |R|/Y < 1e-11, |R|/f < 1e-11 (Y, f > 0)
      bool conv1 = (r1 < 1.0e-11) || (r1 < 1.0e-11 * Yld) || (r1 < 1.0e-11 * fyield);
      kh = conv1 ? 0.0 : (2.0 / 3.0) * Kh;
      cc = 2.0 * mubar + kh;
      if (!conv1) {
        rcc = 1.0 / cc;
        Xr = fyield * rcc;
      } else {
        rcc = r2mu;  // cc = 2 mubar
        Xr = X1;
      }
      gamma = 1.0 - 2.0 * mubar * Xr * rsmag;
      if (!(Xr >= 0.0) || !isfinite(Xr)) atomicOr(a.status, 1);
      if (a.save) {
        a.eqps[s] = eq_old + sq23 * Xr;
        // Fp = exp(dgam N) Fp_old (stored only at plastic points): the
        // increment dgam N is stored here, Fp formed when it is read
        const double is = Xr * rsmag;
        a.Apend[0 * E + s] = s00 * is;
        a.Apend[1 * E + s] = s11 * is;
        a.Apend[2 * E + s] = s22 * is;
        a.Apend[3 * E + s] = s01 * is;
        a.Apend[4 * E + s] = s12 * is;
        a.Apend[5 * E + s] = s02 * is;
        a.pend[s] = 1;
      }
    } else if (a.save) {
      a.eqps[s] = eq_old;
      if (a.fp_reset) {
        a.pend[s] = 0;
#pragma unroll
        for (int q = 0; q < 9; ++q) a.Fp[q * E + s] = __ldg(a.Fp_old + q * E + s);
      }
    }
  }

  // Cauchy stress of the model, then Mixed
  const double pm = 0.5 * kappa * (J - Jinv);
  const double gJ = gamma * Jinv;
  double sg[3][3];
  sg[0][0] = s00 * gJ + pm; sg[1][1] = s11 * gJ + pm; sg[2][2] = s22 * gJ + pm;
  sg[0][1] = sg[1][0] = s01 * gJ;
  sg[1][2] = sg[2][1] = s12 * gJ;
  sg[0][2] = sg[2][0] = s02 * gJ;
  {
    double pbar = ((sg[0][0] + sg[1][1]) + sg[2][2]) * kThird;
    double dp = pval - pbar;
    sg[0][0] += dp; sg[1][1] += dp; sg[2][2] += dp;
  }
  if (a.save) {
#pragma unroll
    for (int q = 0; q < 9; ++q) a.sigma[q * E + s] = sg[q / 3][q % 3];
  }

  // h_a = H G_a
  double hv[4][3];
#pragma unroll
  for (int n = 0; n < 4; ++n)
#pragma unroll
    for (int i = 0; i < 3; ++i) hv[n][i] = H[i][0] * G[n][0] + H[i][1] * G[n][1] + H[i][2] * G[n][2];
  // v = H grad p, w_a = v.h_a
  double vv[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) vv[i] = H[i][0] * gp[0] + H[i][1] * gp[1] + H[i][2] * gp[2];
  double wv[4];
#pragma unroll
  for (int n = 0; n < 4; ++n) wv[n] = vv[0] * hv[n][0] + vv[1] * hv[n][1] + vv[2] * hv[n][2];
  double tau = 0.0;
  if (a.stab) {
    const double hh = __ldg(a.d.h + s);
    tau = tau_coef * (hh * hh);
  }
  const double tauJ = tau * J;
  const double dUdJ = 0.5 * (J - Jinv);
  double T[3][3];  // J sigma
#pragma unroll
  for (int q = 0; q < 9; ++q) T[q / 3][q % 3] = J * sg[q / 3][q % 3];

  // ---------------------------------------------------------------- residual
  if (MODE != MODE_NONE) {
    double Ru[4][3], Rp[4];
    if (!ERR) {
      double TV[3][3];  // V J sigma
#pragma unroll
      for (int q = 0; q < 9; ++q) TV[q / 3][q % 3] = V * T[q / 3][q % 3];
      const double rp0 = ((pval * inv_kappa) - dUdJ) * 0.25 * V;
      const double rpw = a.stab ? tauJ * V : 0.0;
#pragma unroll
      for (int n = 0; n < 4; ++n) {
#pragma unroll
        for (int i = 0; i < 3; ++i) Ru[n][i] = fma(TV[i][0], hv[n][0], fma(TV[i][1], hv[n][1], TV[i][2] * hv[n][2]));
        Rp[n] = fma(rpw, wv[n], rp0);
      }
    } else {
      // DWR weights: z_diff phi_a (momentum, pressure), z_coarse phi_a (stabilization)
      double zn[4][4], zcn[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        ld4(a.Zd + 4 * v[q], zn[q][0], zn[q][1], zn[q][2], zn[q][3]);
        zcn[q] = __ldg(a.Zc + 4 * v[q] + 3);
      }
      double z[3], gz[3][3], zp, zc, gzc[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        z[i] = 0.25 * (zn[0][i] + zn[1][i] + zn[2][i] + zn[3][i]);
#pragma unroll
        for (int j = 0; j < 3; ++j)
          gz[i][j] = zn[0][i] * G[0][j] + zn[1][i] * G[1][j] + zn[2][i] * G[2][j] + zn[3][i] * G[3][j];
      }
      zp = 0.25 * (zn[0][3] + zn[1][3] + zn[2][3] + zn[3][3]);
      zc = 0.25 * (zcn[0] + zcn[1] + zcn[2] + zcn[3]);
#pragma unroll
      for (int j = 0; j < 3; ++j) gzc[j] = zcn[0] * G[0][j] + zcn[1] * G[1][j] + zcn[2] * G[2][j] + zcn[3] * G[3][j];
      double P[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) P[i][j] = T[i][0] * H[0][j] + T[i][1] * H[1][j] + T[i][2] * H[2][j];
      double Pg[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) Pg[i] = P[i][0] * gz[i][0] + P[i][1] * gz[i][1] + P[i][2] * gz[i][2];
      double hz[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) hz[i] = H[i][0] * gzc[0] + H[i][1] * gzc[1] + H[i][2] * gzc[2];
      const double vhz = vv[0] * hz[0] + vv[1] * hz[1] + vv[2] * hz[2];
#pragma unroll
      for (int n = 0; n < 4; ++n) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          double PGa = T[i][0] * hv[n][0] + T[i][1] * hv[n][1] + T[i][2] * hv[n][2];
          Ru[n][i] = V * (0.25 * Pg[i] + z[i] * PGa);
        }
        Rp[n] = ((pval * inv_kappa) - dUdJ) * (zp * 0.25) * V + (a.stab ? tauJ * (0.25 * vhz + zc * wv[n]) * V : 0.0);
      }
    }
    if constexpr (BUF) {
      double* eb = a.ebuf + (size_t)(s - a.ebase) * a.estride;
#pragma unroll
      for (int n = 0; n < 4; ++n) st4(eb + 4 * n, Ru[n][0], Ru[n][1], Ru[n][2], Rp[n]);
    } else {
      const unsigned fm = a.overwrite ? __ldg(a.d.first + s) : 0u;
#pragma unroll
      for (int n = 0; n < 4; ++n) acc4(a.R + 4 * v[n], (fm >> (16 + n)) & 1u, Ru[n][0], Ru[n][1], Ru[n][2], Rp[n]);
    }
  }

  // ---------------------------------------------------------------- QoI
  double ks_w = 0.0;
  if (a.qoi == QOI_AVG_DISP) {
    double uval[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) uval[i] = ((un[0][i] * 0.25 + un[1][i] * 0.25) + un[2][i] * 0.25) + un[3][i] * 0.25;
    double ev = 0.0;
    ev += uval[0] * V;
    ev += uval[1] * V;
    ev += uval[2] * V;
    a.qoi_elem[s] = ev * kThird;
  } else if (a.qoi == QOI_KS_VM) {
    double d1 = sg[0][0] - sg[1][1], d2 = sg[1][1] - sg[2][2], d3 = sg[2][2] - sg[0][0];
    double s7 = 0.5 * (d1 * d1 + d2 * d2 + d3 * d3 + 6.0 * (sg[0][1] * sg[0][1] + sg[1][2] * sg[1][2] + sg[2][0] * sg[2][0]));
    double vm = sqrt(s7);
    double ex = exp(a.rho * (vm - a.ks_max));
    a.qoi_elem[s] = (1.0 / (a.rho * a.ks_scale)) * ex * V;
    ks_w = (V / a.ks_scale) * ex;  // d(elem value)/d(vm)
  }

  if constexpr (JAC) {
  // ---------------------------------------------------------------- tangent
  // m_a = F C G_a, q_a = m_a - Ic/3 h_a
  double mv[4][3], qv[4][3];
#pragma unroll
  for (int n = 0; n < 4; ++n)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      mv[n][i] = FC[i][0] * G[n][0] + FC[i][1] * G[n][1] + FC[i][2] * G[n][2];
      qv[n][i] = mv[n][i] - Ic3 * hv[n][i];
    }
  const double pJ = pval * J;
  const double ga = gamma * alpha;
  // dgamma_b = yq q_b + yh h_b + yn (s m_b) ; Y_b = -2/3 ga h_b + alpha dgamma_b
  double yq = 0.0, yh = 0.0, yn = 0.0;
  // d(gamma smag) = dq q_b + dh h_b + dn (s m_b)   (KS derivative)
  double vq = 0.0, vh = 0.0, vn = 0.0;
  const bool need_n = plastic || (a.qoi == QOI_KS_VM);
  if (plastic) {
    const double A1 = 2.0 * fyield * kh * (rcc * rcc) * rsmag;
    const double A2 = 2.0 * mubar * k0 * rcc * (rsmag * rsmag);
    yq = -A1 * (2.0 * alpha / 3.0);
    yh = A2 * (2.0 / 3.0) * smag;
    yn = -A2 * (2.0 * alpha * rsmag);
  }
  if (a.qoi == QOI_KS_VM) {
    // dsmag_b = -2/3 smag h_b + 2 alpha/smag n_b ; dmubar_b = 2 alpha/3 q_b
    double fs = 1.0, fmu = 0.0;
    if (plastic) { fs = kh / cc; fmu = -2.0 * fyield * kh / (cc * cc); }
    vh = fs * (-(2.0 / 3.0) * smag);
    vn = fs * (2.0 * alpha / smag);
    vq = fmu * (2.0 * alpha / 3.0);
  }
  double Xp[4][3], Yp[4][3], nv[4][3];
  // X_b = V(-2/3 ga m_b + pJ h_b), Y_b = V(-2/3 ga h_b + alpha (yq q_b + yh h_b + yn n_b)),
  // with the coefficients folded once per element
  const double xm = V * (-(2.0 / 3.0) * ga), xh = V * pJ;
  const double yhc = V * (-(2.0 / 3.0) * ga + alpha * yh), yqc = V * (alpha * yq), ync = V * (alpha * yn);
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    if (need_n) {
      nv[b][0] = s00 * mv[b][0] + s01 * mv[b][1] + s02 * mv[b][2];
      nv[b][1] = s01 * mv[b][0] + s11 * mv[b][1] + s12 * mv[b][2];
      nv[b][2] = s02 * mv[b][0] + s12 * mv[b][1] + s22 * mv[b][2];
    } else {
      nv[b][0] = nv[b][1] = nv[b][2] = 0.0;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      Xp[b][k] = fma(xm, mv[b][k], xh * hv[b][k]);
      Yp[b][k] = need_n ? fma(yhc, hv[b][k], fma(yqc, qv[b][k], ync * nv[b][k])) : yhc * hv[b][k];
    }
  }
  // dM/du (QoI derivative) for the u dofs; pressure dofs do not enter the QoIs
  if (a.qoi != QOI_NONE) {
    const unsigned fm = (!BUF && a.overwrite) ? __ldg(a.d.first + s) : 0u;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      double d[3];
      if (a.qoi == QOI_AVG_DISP) {
        d[0] = d[1] = d[2] = V * (1.0 / 12.0);
      } else {
        const double c1 = ks_w * 1.22474487139158904909 * Jinv;  // sqrt(3/2)/J
        const double gs = gamma * smag;
#pragma unroll
        for (int k = 0; k < 3; ++k)
          d[k] = c1 * (vq * qv[b][k] + vh * hv[b][k] + vn * nv[b][k] - gs * hv[b][k]);
      }
      if constexpr (BUF) st4(a.dbuf + 16ll * (s - a.ebase) + 4 * b, d[0], d[1], d[2], 0.0);
      else acc4(a.dMdu + 4 * v[b], (fm >> (16 + b)) & 1u, d[0], d[1], d[2], 0.0);
    }
  }

  const double zs = V * (ga * Ic3 - pJ);
  const double gaV = ga * V;
  const double upf = V * J * 0.25;
  const double tJV = tauJ * V;
  const double ppc = V * pp_coef;
  const double pu0 = V * ((J + Jinv) * 0.125);
  // stabilization coefficients of the p-u rows, folded once per element
  double tvv[3], twv[4];
#pragma unroll
  for (int k = 0; k < 3; ++k) tvv[k] = a.stab ? tJV * vv[k] : 0.0;
#pragma unroll
  for (int b = 0; b < 4; ++b) twv[b] = a.stab ? tJV * wv[b] : 0.0;
  const double tJVs = a.stab ? tJV : 0.0;
  const unsigned fm = (!BUF && a.overwrite) ? __ldg(a.d.first + s) : 0u;
  // ga V C G_a and Z_a = zs h_a
  double CG[4][3], Zv[4][3];
#pragma unroll
  for (int ai = 0; ai < 4; ++ai) {
    if constexpr (MODEL == MODEL_J2) {
      CG[ai][0] = gaV * (C[0] * G[ai][0] + C[3] * G[ai][1] + C[5] * G[ai][2]);
      CG[ai][1] = gaV * (C[3] * G[ai][0] + C[1] * G[ai][1] + C[4] * G[ai][2]);
      CG[ai][2] = gaV * (C[5] * G[ai][0] + C[4] * G[ai][1] + C[2] * G[ai][2]);
    } else {
      CG[ai][0] = gaV * G[ai][0]; CG[ai][1] = gaV * G[ai][1]; CG[ai][2] = gaV * G[ai][2];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) Zv[ai][k] = zs * hv[ai][k];
  }
  // Element block (ai, b) from Pc[i][k] = h_bi Z_ak + c_ab d_ik (TP: Pc
  // transposed), written to the element buffer or accumulated into the matrix.
  auto block = [&](int ai, int b, const double (&Pc)[3][3], bool TP, double eab) {
    double K[4][4];
    const double pu1 = twv[ai] - pu0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int k = 0; k < 3; ++k) K[i][k] = fma(hv[ai][i], Xp[b][k], fma(qv[ai][i], Yp[b][k], TP ? Pc[k][i] : Pc[i][k]));
      K[i][3] = upf * hv[ai][i];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) K[3][k] = fma(pu1, hv[b][k], -fma(eab, tvv[k], twv[b] * hv[ai][k]));
    K[3][3] = fma(tJVs, eab, ppc);
    if constexpr (BUF) {
      double* eb = a.ebuf + (size_t)(s - a.ebase) * a.estride + 16 + 16 * (4 * ai + b);
#pragma unroll
      for (int r = 0; r < 4; ++r) st4(eb + 4 * r, K[r][0], K[r][1], K[r][2], K[r][3]);
    } else if (MODE == MODE_PRIMAL) {
      const int q = 4 * ai + b;
      double* blk = a.A + 16ll * __ldg(a.d.blk + q * E + s);
      const bool f1 = (fm >> q) & 1u;
#pragma unroll
      for (int r = 0; r < 4; ++r) acc4(blk + 4 * r, f1, K[r][0], K[r][1], K[r][2], K[r][3]);
    } else if (MODE == MODE_ADJOINT) {
      const int q = 4 * b + ai;
      double* blk = a.A + 16ll * __ldg(a.d.blk + q * E + s);
      const bool f1 = (fm >> q) & 1u;
#pragma unroll
      for (int r = 0; r < 4; ++r) acc4(blk + 4 * r, f1, K[0][r], K[1][r], K[2][r], K[3][r]);
    }
  };
  // The off-diagonal blocks in pairs: c_ab and e_ab are symmetric in (a, b)
  // and the term h_bi Z_ak = zs h_bi h_ak of block (a, b) is the term
  // (k, i) of block (b, a), so each pair forms them once.
#pragma unroll
  for (int ai = 0; ai < 4; ++ai) {
#pragma unroll
    for (int b = ai + 1; b < 4; ++b) {
      const double eab = hv[ai][0] * hv[b][0] + hv[ai][1] * hv[b][1] + hv[ai][2] * hv[b][2];
      const double cab = fma(CG[ai][0], G[b][0], fma(CG[ai][1], G[b][1], CG[ai][2] * G[b][2]));
      double Pc[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) Pc[i][k] = (i == k) ? fma(hv[b][i], Zv[ai][k], cab) : hv[b][i] * Zv[ai][k];
      block(ai, b, Pc, false, eab);
      block(b, ai, Pc, true, eab);
    }
  }
  // the diagonal blocks (a, a)
#pragma unroll
  for (int ai = 0; ai < 4; ++ai) {
    const double eaa = hv[ai][0] * hv[ai][0] + hv[ai][1] * hv[ai][1] + hv[ai][2] * hv[ai][2];
    if constexpr (DSUM) {
      // column 3 only: the u columns come from the row sums in the gather
      st4(a.ebuf + (size_t)(s - a.ebase) * a.estride + 16 + 16 * (5 * ai), upf * hv[ai][0], upf * hv[ai][1],
          upf * hv[ai][2], fma(tJVs, eaa, ppc));
    } else {
      const double caa = fma(CG[ai][0], G[ai][0], fma(CG[ai][1], G[ai][1], CG[ai][2] * G[ai][2]));
      double Pc[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) Pc[i][k] = (i == k) ? fma(hv[ai][i], Zv[ai][k], caa) : hv[ai][i] * Zv[ai][k];
      block(ai, ai, Pc, false, eaa);
    }
  }
  }  // JAC
}

// ------------------------------------------------------------------ reductions
__global__ void k_sum_partial(const double* x, int n, double* part) {
  KSum acc;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc.add(x[i]);
  acc = block_reduce(acc);
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = acc.s; part[2 * blockIdx.x + 1] = acc.c; }
}
__global__ void k_sum_final(const double* part, int nb, double* out) {
  KSum acc;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    KSum t;
    t.s = part[2 * i];
    t.c = part[2 * i + 1];
    acc.add(t);
  }
  acc = block_reduce(acc);
  if (threadIdx.x == 0) out[0] = acc.value();
}

__device__ __forceinline__ double vm_of(const double* sig, int E, int s) {
  double a00 = sig[0 * E + s], a11 = sig[4 * E + s], a22 = sig[8 * E + s];
  double a01 = sig[1 * E + s], a12 = sig[5 * E + s], a20 = sig[6 * E + s];
  double d1 = a00 - a11, d2 = a11 - a22, d3 = a22 - a00;
  return sqrt(0.5 * (d1 * d1 + d2 * d2 + d3 * d3 + 6.0 * (a01 * a01 + a12 * a12 + a20 * a20)));
}

__global__ void k_vm_max_partial(const double* sig, int E, double* part) {
  double m = 0.0;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) m = fmax(m, vm_of(sig, E, s));
  m = block_max(m);
  if (threadIdx.x == 0) part[blockIdx.x] = m;
}
__global__ void k_max_final(const double* part, int nb, double* out) {
  double m = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) m = fmax(m, part[i]);
  m = block_max(m);
  if (threadIdx.x == 0) out[0] = m;
}
__global__ void k_ks_terms(const double* sig, const double* vol, int E, double rho, const double* mx, double* out) {
  double m = mx[0];
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x)
    out[s] = exp(rho * (vm_of(sig, E, s) - m)) * vol[s];
}

__global__ void k_cpinv(int E, const double* Fp_old, double* Cpinv) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) {
    double A[3][3];
    for (int q = 0; q < 9; ++q) A[q / 3][q % 3] = Fp_old[q * E + s];
    double c00 = A[1][1] * A[2][2] - A[1][2] * A[2][1];
    double c01 = A[1][0] * A[2][2] - A[1][2] * A[2][0];
    double c02 = A[1][0] * A[2][1] - A[1][1] * A[2][0];
    double d = A[0][0] * c00 - A[0][1] * c01 + A[0][2] * c02;
    double I[3][3];
    I[0][0] = c00 / d;
    I[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / d;
    I[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / d;
    I[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / d;
    I[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / d;
    I[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / d;
    I[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) / d;
    I[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / d;
    I[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / d;
    // Cp^-1 = Fp^-1 Fp^-T
    auto cc = [&](int i, int j) { return I[i][0] * I[j][0] + I[i][1] * I[j][1] + I[i][2] * I[j][2]; };
    Cpinv[0 * E + s] = cc(0, 0);
    Cpinv[1 * E + s] = cc(1, 1);
    Cpinv[2 * E + s] = cc(2, 2);
    Cpinv[3 * E + s] = cc(0, 1);
    Cpinv[4 * E + s] = cc(1, 2);
    Cpinv[5 * E + s] = cc(0, 2);
  }
}

// Fp = exp(A) Fp_old at points with a pending plastic write (pend), then
// pend = 0. Bit 2 of status: the exponential series did not settle.
__global__ void k_materialize_fp(int E, const double* __restrict__ Apend, int* __restrict__ pend,
                                 const double* __restrict__ Fp_old, double* __restrict__ Fp, int* status) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) {
    if (!pend[s]) continue;
    const double a00 = Apend[0 * E + s], a11 = Apend[1 * E + s], a22 = Apend[2 * E + s];
    const double a01 = Apend[3 * E + s], a12 = Apend[4 * E + s], a02 = Apend[5 * E + s];
    const double Am[3][3] = {{a00, a01, a02}, {a01, a11, a12}, {a02, a12, a22}};
    double Ex[3][3];
    if (!exp_traceless_sym(Am, Ex)) atomicOr(status, 2);
    double Fo[3][3];
    for (int q = 0; q < 9; ++q) Fo[q / 3][q % 3] = Fp_old[q * E + s];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Fp[(3 * i + j) * E + s] = Ex[i][0] * Fo[0][j] + Ex[i][1] * Fo[1][j] + Ex[i][2] * Fo[2][j];
    pend[s] = 0;
  }
}

__global__ void k_fill_identity(int E, double* Fp) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x)
    for (int q = 0; q < 9; ++q) Fp[q * E + s] = (q % 4 == 0) ? 1.0 : 0.0;
}

template <int MODEL, int MODE, bool JAC, bool ERR>
void launch_colours(const Disc& d, ElemArgs args, cudaStream_t st, bool buffered, bool dsum = false) {
  const int block = 128;
  if (MODE == MODE_NONE || buffered) {
    // elements [args.begin, args.end) into the buffer (all of them, or a chunk)
    const int n = args.end - args.begin;
    if (n <= 0) return;
    if constexpr (JAC && MODE != MODE_NONE) {
      if (dsum) {
        k_elem<MODEL, MODE, JAC, ERR, true, true><<<(n + block - 1) / block, block, 0, st>>>(args);
        GOAL_CHECK_LAUNCH();
        return;
      }
    }
    k_elem<MODEL, MODE, JAC, ERR, true><<<(n + block - 1) / block, block, 0, st>>>(args);
    GOAL_CHECK_LAUNCH();
  } else {
  for (int c = 0; c < d.num_colors; ++c) {
    args.begin = d.color_ptr[c];
    args.end = d.color_ptr[c + 1];
    int n = args.end - args.begin;
    if (n <= 0) continue;
    k_elem<MODEL, MODE, JAC, ERR, false><<<(n + block - 1) / block, block, 0, st>>>(args);
    GOAL_CHECK_LAUNCH();
  }
  }
}

template <int MODEL>
void dispatch(const Disc& d, const Chain& c, const ElemArgs& args, cudaStream_t st, bool buf, bool dsum) {
  if (c.error_chain) {
    GOAL_REQUIRE(!c.jacobian && c.mode == MODE_PRIMAL, GOAL_ERR_ARG, "the error chain is a residual (PRIMAL) chain");
    launch_colours<MODEL, MODE_PRIMAL, false, true>(d, args, st, buf);
    return;
  }
  if (c.mode == MODE_NONE) {
    if (c.jacobian) launch_colours<MODEL, MODE_NONE, true, false>(d, args, st, true);
    else launch_colours<MODEL, MODE_NONE, false, false>(d, args, st, true);
  } else if (c.mode == MODE_PRIMAL) {
    if (c.jacobian) launch_colours<MODEL, MODE_PRIMAL, true, false>(d, args, st, buf, dsum);
    else launch_colours<MODEL, MODE_PRIMAL, false, false>(d, args, st, buf);
  } else {
    GOAL_REQUIRE(c.jacobian, GOAL_ERR_ARG, "ADJOINT mode is a Jacobian (FADT) chain");
    launch_colours<MODEL, MODE_ADJOINT, true, false>(d, args, st, buf, dsum);
  }
}

// Row r of contribution v (element slot v >> 4, element block v & 15) of the
// element buffer; TRANSPOSE reads column r of the transposed element block.
template <bool TRANSPOSE>
__device__ __forceinline__ void load_contrib(const double* __restrict__ ebuf, int estride, int v, int r, double& x0,
                                             double& x1, double& x2, double& x3, int lo = 0) {
  const int s = (v >> 4) - lo, lb = v & 15;
  if (TRANSPOSE) {
    const int lt = ((lb & 3) << 2) | (lb >> 2);
    const double* p = ebuf + (size_t)s * estride + 16 + 16 * lt + r;
    x0 = __ldg(p); x1 = __ldg(p + 4); x2 = __ldg(p + 8); x3 = __ldg(p + 12);
  } else {
    ld4(ebuf + (size_t)s * estride + 16 + 16 * lb + 4 * r, x0, x1, x2, x3);
  }
}

// Phase 2 of the two-phase assembly: every matrix block sums its element
// blocks in element order (4 threads per block, one per row); TRANSPOSE
// accumulates the element blocks transposed (ADJOINT mode stores dR/du^T).
// Contributions are fetched four at a time (independent loads in flight),
// then added in element order. The blocks come from a list (ks[0..count)):
// one launch for the off-diagonal blocks (a few contributions each) and one
// for the diagonal blocks (one per incident element), so that the threads of
// a warp do equal work.
template <bool TRANSPOSE>
__global__ void __launch_bounds__(256) k_gather_blocks(int count, const int* __restrict__ ks,
                                                       const int* __restrict__ bptr, const int* __restrict__ blist,
                                                       const double* __restrict__ ebuf, int estride,
                                                       double* __restrict__ A, int accumulate) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 4ll * count;
       t += (long long)gridDim.x * blockDim.x) {
    const int k = __ldg(ks + (t >> 2)), r = (int)(t & 3);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    if (accumulate) ld4(A + 16ll * k + 4 * r, a0, a1, a2, a3);
    const int c1 = __ldg(bptr + k + 1);
    int c = __ldg(bptr + k);
    for (; c + 4 <= c1; c += 4) {
      double x[4][4];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        load_contrib<TRANSPOSE>(ebuf, estride, __ldg(blist + c + q), r, x[q][0], x[q][1], x[q][2], x[q][3]);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a0 += x[q][0]; a1 += x[q][1]; a2 += x[q][2]; a3 += x[q][3];
      }
    }
    for (; c < c1; ++c) {
      double x0, x1, x2, x3;
      load_contrib<TRANSPOSE>(ebuf, estride, __ldg(blist + c), r, x0, x1, x2, x3);
      a0 += x0; a1 += x1; a2 += x2; a3 += x3;
    }
    st4(A + 16ll * k + 4 * r, a0, a1, a2, a3);
  }
}

// k_gather_blocks for one chunk of elements [lo, hi) (the element buffer
// holds that chunk only): the contributions of the chunk, in element order,
// are added to the block as it stands, so chunk after chunk the additions
// are the ones of the one-pass gather, in the same order.
template <bool TRANSPOSE>
__global__ void __launch_bounds__(256) k_gather_blocks_chunk(int count, const int* __restrict__ ks,
                                                             const int* __restrict__ bptr,
                                                             const int* __restrict__ blist,
                                                             const double* __restrict__ ebuf, int estride,
                                                             double* __restrict__ A, int accumulate, int lo, int hi) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 4ll * count;
       t += (long long)gridDim.x * blockDim.x) {
    const int k = __ldg(ks + (t >> 2)), r = (int)(t & 3);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    if (accumulate) ld4(A + 16ll * k + 4 * r, a0, a1, a2, a3);
    const int c1 = __ldg(bptr + k + 1);
    for (int c = __ldg(bptr + k); c < c1; ++c) {
      const int v = __ldg(blist + c), e = v >> 4;
      if (e < lo || e >= hi) continue;
      double x0, x1, x2, x3;
      load_contrib<TRANSPOSE>(ebuf, estride, v, r, x0, x1, x2, x3, lo);
      a0 += x0; a1 += x1; a2 += x2; a3 += x3;
    }
    st4(A + 16ll * k + 4 * r, a0, a1, a2, a3);
  }
}

// Phase 2 for the diagonal blocks after a DSUM element phase, once the
// off-diagonal blocks are gathered: thread (node n, row r). PRIMAL: the u
// columns of row r are the negated sum of row r of the row's off-diagonal
// blocks; column 3 sums the elements' packed column-3 contributions in element
// order. TRANSPOSE (ADJOINT mode stores dR/du^T): rows 0..2 are the negated
// sums of the same rows of the blocks (m, n) of the block column (btr), row 3
// sums the packed contributions. No atomics; fixed order.
template <bool TRANSPOSE>
__global__ void __launch_bounds__(256) k_gather_diag(int N, const int* __restrict__ brow_ptr,
                                                     const int* __restrict__ diag, const int* __restrict__ btr,
                                                     const int* __restrict__ bptr, const int* __restrict__ blist,
                                                     const double* __restrict__ ebuf, int estride,
                                                     double* __restrict__ A) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 4ll * N;
       t += (long long)gridDim.x * blockDim.x) {
    const int n = (int)(t >> 2), r = (int)(t & 3);
    const int kd = __ldg(diag + n), k0 = __ldg(brow_ptr + n), k1 = __ldg(brow_ptr + n + 1);
    const int c0 = __ldg(bptr + kd), c1 = __ldg(bptr + kd + 1);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    if (!TRANSPOSE || r < 3) {
      for (int k = k0; k < k1; ++k) {
        if (k == kd) continue;
        const int kk = TRANSPOSE ? __ldg(btr + k) : k;
        double x0, x1, x2, x3;
        ld4(A + 16ll * kk + 4 * r, x0, x1, x2, x3);
        a0 -= x0; a1 -= x1; a2 -= x2;
        if (TRANSPOSE) a3 -= x3;
      }
    }
    if (!TRANSPOSE) {
      for (int c = c0; c < c1; ++c) {
        const int v = __ldg(blist + c);
        a3 += __ldg(ebuf + (size_t)(v >> 4) * estride + 16 + 16 * (v & 15) + r);
      }
    } else if (r == 3) {
      for (int c = c0; c < c1; ++c) {
        const int v = __ldg(blist + c);
        double x0, x1, x2, x3;
        ld4(ebuf + (size_t)(v >> 4) * estride + 16 + 16 * (v & 15), x0, x1, x2, x3);
        a0 += x0; a1 += x1; a2 += x2; a3 += x3;
      }
    }
    st4(A + 16ll * kd + 4 * r, a0, a1, a2, a3);
  }
}

// Phase 2 for nodal vectors: node n, row q sums the element rows of its
// incident elements (entries 4*s + a of nlist) in element order.
// [lo, hi): the element slots the buffer holds (a chunk; the buffer's first
// entry is slot lo); the one-pass gather has lo = 0, hi = E.
__global__ void __launch_bounds__(256) k_gather_nodes(int N, const int* __restrict__ nptr,
                                                      const int* __restrict__ nlist, const double* __restrict__ ebuf,
                                                      int estride, double* __restrict__ out, int accumulate, int lo,
                                                      int hi) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 4ll * N;
       t += (long long)gridDim.x * blockDim.x) {
    const int n = (int)(t >> 2), q = (int)(t & 3);
    double acc = accumulate ? out[t] : 0.0;
    const int c1 = __ldg(nptr + n + 1);
    for (int c = __ldg(nptr + n); c < c1; ++c) {
      const int v = __ldg(nlist + c), e = v >> 2;
      if (e < lo || e >= hi) continue;
      acc += __ldg(ebuf + (size_t)(e - lo) * estride + 4 * (v & 3) + q);
    }
    out[t] = acc;
  }
}

double device_sum(const double* x, int n, DevBuf<double>& red, cudaStream_t st) {
  const int nb = std::min(grid_for(n, 256), 1024);
  if (red.n < 2 * (size_t)nb + 2) red.alloc(2 * nb + 2);
  k_sum_partial<<<nb, 256, 0, st>>>(x, n, red.ptr);
  GOAL_CHECK_LAUNCH();
  k_sum_final<<<1, 1024, 0, st>>>(red.ptr, nb, red.ptr + 2 * nb);
  GOAL_CHECK_LAUNCH();
  double out = 0.0;
  GOAL_CUDA(cudaMemcpyAsync(&out, red.ptr + 2 * nb, sizeof(double), cudaMemcpyDeviceToHost, st));
  GOAL_CUDA(cudaStreamSynchronize(st));
  return out;
}

}  // namespace

void Mechanics::init() {
  const int E = disc->num_elems, N = disc->num_nodes;
  std::vector<double> m;
  for (const MaterialRow& r : mats_h) {
    double kappa = r.E / (3.0 * (1.0 - 2.0 * r.nu));
    double mu = r.E / (2.0 * (1.0 + r.nu));
    m.insert(m.end(), {kappa, mu, r.K, r.Y, r.c0, 1.0 / kappa, 0.5 * r.c0 / mu, 1.0 / (16.0 * kappa)});
  }
  static bool table_ready = false;
  if (!table_ready) {
    double t[80];
    for (int k = 0; k < 80; ++k) t[k] = 1.0 / (k + 1);
    GOAL_CUDA(cudaMemcpyToSymbol(c_inv_k, t, sizeof(t)));
    table_ready = true;
  }
  mats.upload(m.data(), m.size(), disc->stream);
  U.alloc(4ll * N);
  U.zero(disc->stream);
  st.sigma.alloc(9ll * E);
  st.sigma.zero(disc->stream);
  st.eqps.alloc(E);
  st.eqps.zero(disc->stream);
  st.eqps_old.alloc(E);
  st.eqps_old.zero(disc->stream);
  st.Fp.alloc(9ll * E);
  st.Fp_old.alloc(9ll * E);
  st.Cpinv.alloc(6ll * E);
  st.Apend.alloc(6ll * E);
  st.pend.alloc(E);
  st.pend.zero(disc->stream);
  k_fill_identity<<<grid_for(E, 256), 256, 0, disc->stream>>>(E, st.Fp.ptr);
  k_fill_identity<<<grid_for(E, 256), 256, 0, disc->stream>>>(E, st.Fp_old.ptr);
  GOAL_CHECK_LAUNCH();
  refresh_cpinv();
  qoi_elem.alloc(E);
  status.alloc(1);
  status.zero(disc->stream);
}

void Mechanics::refresh_cpinv() {
  const int E = disc->num_elems;
  k_cpinv<<<grid_for(E, 256), 256, 0, disc->stream>>>(E, st.Fp_old.ptr, st.Cpinv.ptr);
  GOAL_CHECK_LAUNCH();
}

void Mechanics::materialize_fp() {
  const int E = disc->num_elems;
  GOAL_CUDA(cudaMemsetAsync(status.ptr, 0, sizeof(int), disc->stream));
  k_materialize_fp<<<grid_for(E, 256), 256, 0, disc->stream>>>(E, st.Apend.ptr, st.pend.ptr, st.Fp_old.ptr, st.Fp.ptr,
                                                               status.ptr);
  GOAL_CHECK_LAUNCH();
  int h = 0;
  GOAL_CUDA(cudaMemcpyAsync(&h, status.ptr, sizeof(int), cudaMemcpyDeviceToHost, disc->stream));
  GOAL_CUDA(cudaStreamSynchronize(disc->stream));
  GOAL_REQUIRE(h == 0, GOAL_ERR_RETURN_MAP, "J2: the exponential of the plastic increment did not converge");
}

void Mechanics::update_states() {
  const int E = disc->num_elems;
  materialize_fp();
  GOAL_CUDA(cudaMemcpyAsync(st.Fp_old.ptr, st.Fp.ptr, sizeof(double) * 9 * E, cudaMemcpyDeviceToDevice, disc->stream));
  GOAL_CUDA(cudaMemcpyAsync(st.eqps_old.ptr, st.eqps.ptr, sizeof(double) * E, cudaMemcpyDeviceToDevice, disc->stream));
  refresh_cpinv();
}

void SolInfo::init(Disc* d) {
  disc = d;
  R.alloc(4ll * d->num_nodes);
  dMdu.alloc(4ll * d->num_nodes);
  A.alloc(16ll * d->nnzb);
  R.zero(d->stream);
  dMdu.zero(d->stream);
  A.zero(d->stream);
}

void ks_prepass(Mechanics& m, double rho, double& max_vm, double& scale, cudaStream_t st) {
  const int E = m.disc->num_elems;
  const int nb = std::min(grid_for(E, 256), 1024);
  if (m.red.n < 2 * (size_t)nb + 2) m.red.alloc(2 * nb + 2);
  k_vm_max_partial<<<nb, 256, 0, st>>>(m.st.sigma.ptr, E, m.red.ptr);
  GOAL_CHECK_LAUNCH();
  k_max_final<<<1, 1024, 0, st>>>(m.red.ptr, nb, m.red.ptr + 2 * nb);
  GOAL_CHECK_LAUNCH();
  k_ks_terms<<<grid_for(E, 256), 256, 0, st>>>(m.st.sigma.ptr, m.disc->vol.ptr, E, rho, m.red.ptr + 2 * nb,
                                               m.qoi_elem.ptr);
  GOAL_CHECK_LAUNCH();
  GOAL_CUDA(cudaMemcpyAsync(&max_vm, m.red.ptr + 2 * nb, sizeof(double), cudaMemcpyDeviceToHost, st));
  GOAL_CUDA(cudaStreamSynchronize(st));
  scale = device_sum(m.qoi_elem.ptr, E, m.red, st);
}

namespace {
// Optional device timing of the two assembly phases (CUDA events on the
// assembly's stream, read after the stream synchronisation that ends every
// assembly). Off unless enabled.
struct PhaseTimer {
  bool on = false;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  double elem_ms = 0.0, gather_ms = 0.0;
  long long count = 0;
} g_phase;
}  // namespace

void assembly_timing(bool enable) {
  if (enable && !g_phase.ev[0])
    for (auto& e : g_phase.ev) GOAL_CUDA(cudaEventCreate(&e));
  g_phase.on = enable;
  if (enable) {
    g_phase.elem_ms = g_phase.gather_ms = 0.0;
    g_phase.count = 0;
  }
}

void assembly_timing_read(double* ms, long long* count) {
  ms[0] = g_phase.elem_ms;
  ms[1] = g_phase.gather_ms;
  *count = g_phase.count;
}

namespace {
long long g_ebuf_limit = 0;  // bytes; 0 = a quarter of the device's memory
}

void set_element_buffer_limit(long long bytes) { g_ebuf_limit = bytes < 0 ? 0 : bytes; }

long long element_buffer_limit() {
  if (g_ebuf_limit > 0) return g_ebuf_limit;
  // a quarter of the device's memory, looked up once per device (the query is
  // too slow to repeat in every assembly)
  constexpr int kDevs = 64;
  static long long total[kDevs] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevs) return 8ll << 30;
  if (total[dev] == 0) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || total_b == 0) return 8ll << 30;
    total[dev] = (long long)total_b;
  }
  return total[dev] / 4;
}

double assemble(Mechanics& m, SolInfo* s, const Chain& c, const ErrorWeights* w, cudaStream_t st) {
  const Disc& d = *m.disc;
  ElemArgs a;
  std::memset(&a, 0, sizeof(a));
  a.d = d.view();
  a.mats = m.mats.ptr;
  a.U = m.U.ptr;
  a.Fp_old = m.st.Fp_old.ptr;
  a.eqps_old = m.st.eqps_old.ptr;
  a.Cpinv = m.st.Cpinv.ptr;
  a.sigma = m.st.sigma.ptr;
  a.Fp = m.st.Fp.ptr;
  a.eqps = m.st.eqps.ptr;
  a.Apend = m.st.Apend.ptr;
  a.pend = m.st.pend.ptr;
  a.status = m.status.ptr;
  a.stab = m.stabilization ? 1 : 0;
  a.save = c.save_states;
  a.fp_reset = m.fp_reset ? 1 : 0;
  a.overwrite = c.overwrite;
  a.qoi = c.qoi;
  a.rho = c.rho;
  a.qoi_elem = m.qoi_elem.ptr;
  if (c.mode != MODE_NONE || c.jacobian) {
    GOAL_REQUIRE(s != nullptr, GOAL_ERR_ARG, "assemble: SolInfo required for this chain");
    a.R = s->R.ptr;
    a.A = s->A.ptr;
    a.dMdu = s->dMdu.ptr;
  }
  if (c.error_chain) {
    GOAL_REQUIRE(w && w->Zd && w->Zc, GOAL_ERR_ARG, "error chain needs z weights");
    a.Zd = w->Zd;
    a.Zc = w->Zc;
  }
  double ks_max = 0.0, ks_scale = 1.0;
  if (c.qoi == QOI_KS_VM) {
    GOAL_REQUIRE(c.rho > 0.0, GOAL_ERR_ARG, "KS functional needs rho > 0");
    ks_prepass(m, c.rho, ks_max, ks_scale, st);
    GOAL_REQUIRE(ks_max > 0.0 && ks_scale > 0.0, GOAL_ERR_STATE, "KS functional: stored stresses are zero");
  }
  a.ks_max = ks_max;
  a.ks_scale = ks_scale;
  GOAL_CUDA(cudaMemsetAsync(m.status.ptr, 0, sizeof(int), st));
  if (c.overwrite && c.jacobian && c.qoi == QOI_NONE && s) {  // zero_all also clears dMdu
    // dMdu is not written by a chain without QoI: SolInfo::zero_all semantics
    GOAL_CUDA(cudaMemsetAsync(s->dMdu.ptr, 0, sizeof(double) * s->dMdu.n, st));
  }
  const bool buf = !c.colored && (c.mode != MODE_NONE || c.jacobian);
  const bool scatter = c.mode != MODE_NONE;
  const int E = d.num_elems;
  int chunk = E;  // elements per pass of the two-phase assembly
  if (buf) {
    a.estride = c.jacobian ? 272 : 16;
    const size_t per_elem = sizeof(double) * (a.estride + ((c.jacobian && c.qoi != QOI_NONE) ? 16 : 0));
    chunk = (int)std::max<long long>(1, std::min<long long>(E, element_buffer_limit() / per_elem));
    size_t need = (size_t)chunk * a.estride;
    if (m.ebuf.n < need) m.ebuf.alloc(need);
    a.ebuf = m.ebuf.ptr;
    if (c.jacobian && c.qoi != QOI_NONE) {
      if (m.dbuf.n < 16ull * chunk) m.dbuf.alloc(16ull * chunk);
      a.dbuf = m.dbuf.ptr;
    }
  }
  // diagonal blocks from row sums: buffered Jacobian chains that overwrite, in one pass
  const bool dsum = buf && scatter && c.jacobian && c.overwrite && chunk == E;
  if (dsum && c.mode == MODE_ADJOINT) const_cast<Disc&>(d).block_transpose_map();
  const bool timed = g_phase.on;
  if (timed) GOAL_CUDA(cudaEventRecord(g_phase.ev[0], st));
  for (int e0 = 0; e0 < E; e0 += chunk) {
    const int e1 = buf ? std::min(E, e0 + chunk) : E;
    a.begin = e0;
    a.end = e1;
    a.ebase = e0;
    if (m.model == MODEL_J2) dispatch<MODEL_J2>(d, c, a, st, buf, dsum);
    else dispatch<MODEL_NEOHOOKEAN>(d, c, a, st, buf, dsum);
    if (timed && e0 == 0) GOAL_CUDA(cudaEventRecord(g_phase.ev[1], st));
    if (!buf) break;  // the coloured path covers every element itself
    const int acc = (c.overwrite && e0 == 0) ? 0 : 1;
    const bool chunked = chunk < E;
    if (scatter) {
      k_gather_nodes<<<grid_for(4ll * d.num_nodes, 256), 256, 0, st>>>(d.num_nodes, d.nptr.ptr, d.nlist.ptr,
                                                                          m.ebuf.ptr, a.estride, s->R.ptr, acc, e0, e1);
      GOAL_CHECK_LAUNCH();
      if (c.jacobian) {
        const int noff = d.nnzb - d.num_nodes;
        const int* lists[2] = {d.offd.ptr, d.diag.ptr};
        const int counts[2] = {noff, d.num_nodes};
        for (int q = 0; q < 2; ++q) {
          if (counts[q] <= 0) continue;
          const int g = grid_for(4ll * counts[q], 256);
          if (q == 1 && dsum) {  // the diagonal blocks, after the off-diagonal ones
            if (c.mode == MODE_ADJOINT)
              k_gather_diag<true><<<grid_for(4ll * d.num_nodes, 256), 256, 0, st>>>(
                  d.num_nodes, d.brow_ptr.ptr, d.diag.ptr, d.btr.ptr, d.bptr.ptr, d.blist.ptr, m.ebuf.ptr,
                  a.estride, s->A.ptr);
            else
              k_gather_diag<false><<<grid_for(4ll * d.num_nodes, 256), 256, 0, st>>>(
                  d.num_nodes, d.brow_ptr.ptr, d.diag.ptr, nullptr, d.bptr.ptr, d.blist.ptr, m.ebuf.ptr,
                  a.estride, s->A.ptr);
          } else if (chunked) {
            if (c.mode == MODE_ADJOINT)
              k_gather_blocks_chunk<true><<<g, 256, 0, st>>>(counts[q], lists[q], d.bptr.ptr, d.blist.ptr, m.ebuf.ptr,
                                                             a.estride, s->A.ptr, acc, e0, e1);
            else
              k_gather_blocks_chunk<false><<<g, 256, 0, st>>>(counts[q], lists[q], d.bptr.ptr, d.blist.ptr,
                                                              m.ebuf.ptr, a.estride, s->A.ptr, acc, e0, e1);
          } else if (c.mode == MODE_ADJOINT) {
            k_gather_blocks<true><<<g, 256, 0, st>>>(counts[q], lists[q], d.bptr.ptr, d.blist.ptr, m.ebuf.ptr,
                                                     a.estride, s->A.ptr, acc);
          } else {
            k_gather_blocks<false><<<g, 256, 0, st>>>(counts[q], lists[q], d.bptr.ptr, d.blist.ptr, m.ebuf.ptr,
                                                      a.estride, s->A.ptr, acc);
          }
          GOAL_CHECK_LAUNCH();
        }
      }
    }
    if (c.jacobian && c.qoi != QOI_NONE && s) {
      k_gather_nodes<<<grid_for(4ll * d.num_nodes, 256), 256, 0, st>>>(d.num_nodes, d.nptr.ptr, d.nlist.ptr,
                                                                          m.dbuf.ptr, 16, s->dMdu.ptr, acc, e0, e1);
      GOAL_CHECK_LAUNCH();
    }
  }
  if (timed) GOAL_CUDA(cudaEventRecord(g_phase.ev[2], st));
  int hstat = 0;
  GOAL_CUDA(cudaMemcpyAsync(&hstat, m.status.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  double q = 0.0;
  if (c.qoi != QOI_NONE) {
    q = device_sum(m.qoi_elem.ptr, d.num_elems, m.red, st);
    if (c.qoi == QOI_KS_VM) q = ks_max + (1.0 / c.rho) * std::log(ks_scale);
  } else {
    GOAL_CUDA(cudaStreamSynchronize(st));
  }
  if (timed) {
    float e = 0.0f, g = 0.0f;
    GOAL_CUDA(cudaEventElapsedTime(&e, g_phase.ev[0], g_phase.ev[1]));
    GOAL_CUDA(cudaEventElapsedTime(&g, g_phase.ev[1], g_phase.ev[2]));
    g_phase.elem_ms += e;
    g_phase.gather_ms += g;
    g_phase.count += 1;
  }
  GOAL_REQUIRE(hstat == 0, GOAL_ERR_RETURN_MAP, "J2: return mapping failed");
  return q;
}

}  // namespace goal
