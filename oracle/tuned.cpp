// "Tuned" CPU baseline of the element R+J assembly -- BASELINE / TEST
// INFRASTRUCTURE ONLY (timed beside the GPU path; never part of it).
//
// The same chain as oracle.cpp (Kinematics, Neohookean or J2 with goal's
// radial return, Mixed, MResidual, PResidual, Stabilization; src/goal_*.cpp as
// cited there) for the primal Jacobian chain with state writes, but written
// for speed on host cores instead of as a faithful restatement:
//   * the element tangent in closed form instead of forward-mode AD: with
//     G_a = grad phi_a, H = F^-T, h_a = H G_a, C = Cp^-1, m_a = F C G_a,
//     q_a = m_a - Ic/3 h_a, alpha = mu J^-2/3 and gamma the radial-return
//     factor, K^uu_{ai,bk} = V [gamma alpha c_ab d_ik + h_ai X_bk + q_ai Y_bk
//     + h_bi Z_ak] (c_ab = G_a.C G_b), plus the pressure rows and columns;
//   * per-mesh geometry (shape-function gradients, volumes, edge lengths,
//     Cp^-1, the 16 matrix block indices of each element) computed once;
//   * elements coloured so that no two of one colour share a node, each colour
//     assembled by all threads (OpenMP) straight into 4x4 blocks, no atomics.
// Its results agree with the dual-number oracle to rounding (checked by
// tests/test_tuned_cpu.py).
#include <cmath>
#include <cstring>
#include <vector>

namespace {

struct Geo {
  double G[4][3];
  double V;
  double h;
};

inline void geometry(const double* X, const int* t, Geo& g) {
  double J[3][3];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) J[r][c] = X[3 * t[c + 1] + r] - X[3 * t[0] + r];
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  // inverse of J (rows: d xi_r / d x)
  double Ji[3][3];
  Ji[0][0] = c00 / det;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  Ji[1][0] = c01 / det;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
  Ji[2][0] = c02 / det;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  for (int k = 0; k < 3; ++k) {
    g.G[1][k] = Ji[0][k];
    g.G[2][k] = Ji[1][k];
    g.G[3][k] = Ji[2][k];
    g.G[0][k] = -(Ji[0][k] + Ji[1][k] + Ji[2][k]);
  }
  g.V = det / 6.0;
  double s = 0.0;
  const int ed[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  for (auto& e : ed) {
    double l2 = 0.0;
    for (int d = 0; d < 3; ++d) {
      const double dx = X[3 * t[e[1]] + d] - X[3 * t[e[0]] + d];
      l2 += dx * dx;
    }
    s += l2;
  }
  g.h = std::sqrt(s / 6.0);
}

// exp(A) for a symmetric traceless 3x3 A by the power series reduced with
// Cayley-Hamilton (A^3 = I2 A + I3 I)
void expm_traceless(const double A[3][3], double out[3][3]) {
  double A2[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A2[i][j] = A[i][0] * A[0][j] + A[i][1] * A[1][j] + A[i][2] * A[2][j];
  const double I2 = 0.5 * (A2[0][0] + A2[1][1] + A2[2][2]);
  const double I3 = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
                    A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                    A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
  double x = 0.0, y = 0.0, z = 0.5, s0 = 1.0, s1 = 1.0, s2 = 0.5;
  for (int k = 2; k < 80; ++k) {
    const double nx = z * I3, ny = x + z * I2, nz = y;
    const double inv = 1.0 / (k + 1);
    x = nx * inv;
    y = ny * inv;
    z = nz * inv;
    s0 += x;
    s1 += y;
    s2 += z;
    if (std::fabs(x) + std::fabs(y) + std::fabs(z) < 1e-20 * (std::fabs(s0) + std::fabs(s1) + std::fabs(s2))) break;
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) out[i][j] = s1 * A[i][j] + s2 * A2[i][j] + (i == j ? s0 : 0.0);
}

}  // namespace

extern "C" {

// Per-mesh set-up: geometry (G 12, V, h per element) and Cp^-1 (6 per element:
// xx yy zz xy yz xz) of Fp_old.
void tuned_setup(int E, const double* X, const int* tets, const double* Fp_old, double* geo, double* cpinv) {
#pragma omp parallel for schedule(static)
  for (int e = 0; e < E; ++e) {
    Geo g;
    geometry(X, tets + 4 * e, g);
    double* o = geo + 14ll * e;
    for (int q = 0; q < 12; ++q) o[q] = g.G[q / 3][q % 3];
    o[12] = g.V;
    o[13] = g.h;
    if (Fp_old) {
      const double* A = Fp_old + 9ll * e;
      const double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[3] * A[8] - A[5] * A[6], c02 = A[3] * A[7] - A[4] * A[6];
      const double d = A[0] * c00 - A[1] * c01 + A[2] * c02;
      double I[9];
      I[0] = c00 / d;
      I[1] = (A[2] * A[7] - A[1] * A[8]) / d;
      I[2] = (A[1] * A[5] - A[2] * A[4]) / d;
      I[3] = -c01 / d;
      I[4] = (A[0] * A[8] - A[2] * A[6]) / d;
      I[5] = (A[2] * A[3] - A[0] * A[5]) / d;
      I[6] = c02 / d;
      I[7] = (A[1] * A[6] - A[0] * A[7]) / d;
      I[8] = (A[0] * A[4] - A[1] * A[3]) / d;
      auto cc = [&](int i, int j) { return I[3 * i] * I[3 * j] + I[3 * i + 1] * I[3 * j + 1] + I[3 * i + 2] * I[3 * j + 2]; };
      double* c = cpinv + 6ll * e;
      c[0] = cc(0, 0);
      c[1] = cc(1, 1);
      c[2] = cc(2, 2);
      c[3] = cc(0, 1);
      c[4] = cc(1, 2);
      c[5] = cc(0, 2);
    }
  }
}

// One primal Jacobian assembly with state writes (Primal::compute_jacob):
// R (4N) and the 4x4 blocks A (16 x nnzb, block blk[16 e + 4 a + b] for node
// pair (a, b) of element e) start from zero; elements are processed colour by
// colour (order[color_ptr[c] .. color_ptr[c+1])), each colour in parallel.
// mats per element set: E, nu, K, Y, c0. model 0 neo-Hookean, 1 J2. Returns the
// number of return-map failures.
int tuned_assemble(int N, int E, const int* tets, const int* elem_set, const double* mats, int model, int stab,
                   const double* geo, const double* cpinv, const double* U, const double* Fp_old,
                   const double* eqps_old, int ncolors, const int* color_ptr, const int* order, const int* blk,
                   long long nnzb, double* R, double* A, double* sigma_out, double* Fp_out, double* eqps_out) {
  std::memset(R, 0, sizeof(double) * 4ll * N);
  std::memset(A, 0, sizeof(double) * 16ll * nnzb);
  int failures = 0;
  const double sq23 = std::sqrt(2.0 / 3.0);
  for (int col = 0; col < ncolors; ++col) {
#pragma omp parallel for schedule(static) reduction(+ : failures)
    for (int i = color_ptr[col]; i < color_ptr[col + 1]; ++i) {
      const int e = order[i];
      const int* t = tets + 4 * e;
      const double* g = geo + 14ll * e;
      double G[4][3];
      for (int q = 0; q < 12; ++q) G[q / 3][q % 3] = g[q];
      const double V = g[12];
      const double* mr = mats + 5 * (elem_set ? elem_set[e] : 0);
      const double Em = mr[0], nu = mr[1], Kh = mr[2], Yld = mr[3], c0 = mr[4];
      const double kappa = Em / (3.0 * (1.0 - 2.0 * nu)), mu = Em / (2.0 * (1.0 + nu));
      double un[4][3], pn[4];
      for (int a = 0; a < 4; ++a) {
        for (int d = 0; d < 3; ++d) un[a][d] = U[4 * t[a] + d];
        pn[a] = U[4 * t[a] + 3];
      }
      double F[3][3];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          F[r][c] = (r == c ? 1.0 : 0.0) + un[0][r] * G[0][c] + un[1][r] * G[1][c] + un[2][r] * G[2][c] +
                    un[3][r] * G[3][c];
      const double pval = 0.25 * (pn[0] + pn[1] + pn[2] + pn[3]);
      double gp[3];
      for (int c = 0; c < 3; ++c) gp[c] = pn[0] * G[0][c] + pn[1] * G[1][c] + pn[2] * G[2][c] + pn[3] * G[3][c];
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
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) H[r][c] = cof[r][c] * Jinv;
      double C[6] = {1.0, 1.0, 1.0, 0.0, 0.0, 0.0};
      if (model == 1)
        for (int q = 0; q < 6; ++q) C[q] = cpinv[6ll * e + q];
      const double Cm[3][3] = {{C[0], C[3], C[5]}, {C[3], C[1], C[4]}, {C[5], C[4], C[2]}};
      double FC[3][3];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) FC[r][c] = F[r][0] * Cm[0][c] + F[r][1] * Cm[1][c] + F[r][2] * Cm[2][c];
      double B[3][3];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) B[r][c] = FC[r][0] * F[c][0] + FC[r][1] * F[c][1] + FC[r][2] * F[c][2];
      const double Ic = B[0][0] + B[1][1] + B[2][2], Ic3 = Ic / 3.0;
      const double alpha = mu * std::pow(J, -2.0 / 3.0);
      double sd[3][3];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) sd[r][c] = alpha * (B[r][c] - (r == c ? Ic3 : 0.0));
      double gamma = 1.0, smag = 0.0, mubar = 0.0, fyield = 0.0, k0 = 0.0, cc = 1.0, kh = 0.0, Xr = 0.0;
      bool plastic = false;
      if (model == 1) {
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) smag += sd[r][c] * sd[r][c];
        smag = std::sqrt(smag);
        mubar = alpha * Ic3;
        const double eq = eqps_old[e];
        k0 = sq23 * (Yld + Kh * eq);
        fyield = smag - k0;
        if (fyield > 1.0e-12) {
          plastic = true;
          // goal's return map: the first Newton iterate (slope -2 mubar), then
          // the closed form f / (2 mubar + 2K/3) unless the first converged
          const double X1 = fyield / (2.0 * mubar);
          const double R1 = smag - (2.0 * mubar * X1 + sq23 * (Yld + Kh * (eq + sq23 * X1)));
          const double r1 = std::fabs(R1);
          const bool conv1 = (r1 < 1.0e-11) || (r1 < 1.0e-11 * Yld) || (r1 < 1.0e-11 * fyield);
          kh = conv1 ? 0.0 : (2.0 / 3.0) * Kh;
          cc = 2.0 * mubar + kh;
          Xr = conv1 ? X1 : fyield / cc;
          if (!(Xr >= 0.0) || !std::isfinite(Xr)) failures += 1;
          gamma = 1.0 - 2.0 * mubar * Xr / smag;
          eqps_out[e] = eq + sq23 * Xr;
          double Am[3][3], Ex[3][3];
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) Am[r][c] = sd[r][c] * (Xr / smag);
          expm_traceless(Am, Ex);
          const double* Fo = Fp_old + 9ll * e;
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c)
              Fp_out[9ll * e + 3 * r + c] = Ex[r][0] * Fo[c] + Ex[r][1] * Fo[3 + c] + Ex[r][2] * Fo[6 + c];
        } else {
          eqps_out[e] = eq;  // Fp is left as it was (goal's state write)
        }
      }
      const double pm = 0.5 * kappa * (J - Jinv);
      double sg[3][3];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) sg[r][c] = sd[r][c] * gamma * Jinv + (r == c ? pm : 0.0);
      const double pbar = (sg[0][0] + sg[1][1] + sg[2][2]) / 3.0;
      for (int r = 0; r < 3; ++r) sg[r][r] += pval - pbar;
      for (int q = 0; q < 9; ++q) sigma_out[9ll * e + q] = sg[q / 3][q % 3];
      double hv[4][3], mv[4][3], qv[4][3], nv[4][3];
      for (int a = 0; a < 4; ++a)
        for (int r = 0; r < 3; ++r) {
          hv[a][r] = H[r][0] * G[a][0] + H[r][1] * G[a][1] + H[r][2] * G[a][2];
          mv[a][r] = FC[r][0] * G[a][0] + FC[r][1] * G[a][1] + FC[r][2] * G[a][2];
          qv[a][r] = mv[a][r] - Ic3 * hv[a][r];
        }
      for (int a = 0; a < 4; ++a)
        for (int r = 0; r < 3; ++r) nv[a][r] = sd[r][0] * mv[a][0] + sd[r][1] * mv[a][1] + sd[r][2] * mv[a][2];
      double vv[3], wv[4];
      for (int r = 0; r < 3; ++r) vv[r] = H[r][0] * gp[0] + H[r][1] * gp[1] + H[r][2] * gp[2];
      for (int a = 0; a < 4; ++a) wv[a] = vv[0] * hv[a][0] + vv[1] * hv[a][1] + vv[2] * hv[a][2];
      const double tau = stab ? 0.5 * c0 * g[13] * g[13] / mu : 0.0;
      const double tauJ = tau * J;
      // residual
      double* Rn[4];
      for (int a = 0; a < 4; ++a) Rn[a] = R + 4ll * t[a];
      for (int a = 0; a < 4; ++a) {
        for (int r = 0; r < 3; ++r)
          Rn[a][r] += V * J * (sg[r][0] * hv[a][0] + sg[r][1] * hv[a][1] + sg[r][2] * hv[a][2]);
        Rn[a][3] += ((pval / kappa) - 0.5 * (J - Jinv)) * 0.25 * V + tauJ * wv[a] * V;
      }
      // tangent
      const double ga = gamma * alpha, pJ = pval * J;
      double yq = 0.0, yh = 0.0, yn = 0.0;
      if (plastic) {
        const double A1 = 2.0 * fyield * kh / (cc * cc * smag);
        const double A2 = 2.0 * mubar * k0 / (cc * smag * smag);
        yq = -A1 * (2.0 * alpha / 3.0);
        yh = A2 * (2.0 / 3.0) * smag;
        yn = -A2 * (2.0 * alpha / smag);
      }
      double Xp[4][3], Yp[4][3];
      for (int b = 0; b < 4; ++b)
        for (int k = 0; k < 3; ++k) {
          Xp[b][k] = V * (-(2.0 / 3.0) * ga * mv[b][k] + pJ * hv[b][k]);
          Yp[b][k] = V * (-(2.0 / 3.0) * ga * hv[b][k] + alpha * (yq * qv[b][k] + yh * hv[b][k] + yn * nv[b][k]));
        }
      const double zs = V * (ga * Ic3 - pJ);
      // C G_b once per node; c_ab = ga V G_a.C G_b and e_ab = h_a.h_b are
      // symmetric in (a, b), and the term zs h_br h_ak of block (a, b) is the
      // term (k, r) of block (b, a): the blocks are formed in pairs
      double CGv[4][3];
      for (int b = 0; b < 4; ++b)
        for (int r = 0; r < 3; ++r) CGv[b][r] = Cm[r][0] * G[b][0] + Cm[r][1] * G[b][1] + Cm[r][2] * G[b][2];
      auto block = [&](int a, int b, const double (&P)[3][3], bool tp, double eab) {
        double* K = A + 16ll * blk[16ll * e + 4 * a + b];
        for (int r = 0; r < 3; ++r) {
          for (int k = 0; k < 3; ++k) K[4 * r + k] += hv[a][r] * Xp[b][k] + qv[a][r] * Yp[b][k] + (tp ? P[k][r] : P[r][k]);
          K[4 * r + 3] += V * J * hv[a][r] * 0.25;
        }
        for (int k = 0; k < 3; ++k)
          K[12 + k] += V * (hv[b][k] * (tauJ * wv[a] - (J + Jinv) * 0.125) - tauJ * eab * vv[k] - tauJ * wv[b] * hv[a][k]);
        K[15] += V * (1.0 / (16.0 * kappa) + tauJ * eab);
      };
      for (int a = 0; a < 4; ++a)
        for (int b = a; b < 4; ++b) {
          const double cab = ga * V * (G[a][0] * CGv[b][0] + G[a][1] * CGv[b][1] + G[a][2] * CGv[b][2]);
          const double eab = hv[a][0] * hv[b][0] + hv[a][1] * hv[b][1] + hv[a][2] * hv[b][2];
          double P[3][3];
          for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 3; ++k) P[r][k] = zs * hv[b][r] * hv[a][k] + (r == k ? cab : 0.0);
          block(a, b, P, false, eab);
          if (b != a) block(b, a, P, true, eab);
        }
    }
  }
  return failures;
}

}  // extern "C"

extern "C" {

// Greedy colouring: element e takes the smallest colour not yet taken by an
// element that shares a node with it (per-node bit masks of used colours,
// at most 128 colours). Returns the number of colours, or -1.
int tuned_color(int N, int E, const int* tets, int* color) {
  std::vector<unsigned long long> used(2ll * N, 0ull);
  int ncol = 0;
  for (int e = 0; e < E; ++e) {
    unsigned long long m0 = 0, m1 = 0;
    for (int a = 0; a < 4; ++a) {
      m0 |= used[2ll * tets[4 * e + a]];
      m1 |= used[2ll * tets[4 * e + a] + 1];
    }
    int c = 0;
    while (c < 128 && ((c < 64 ? (m0 >> c) : (m1 >> (c - 64))) & 1ull)) ++c;
    if (c >= 128) return -1;
    color[e] = c;
    for (int a = 0; a < 4; ++a) used[2ll * tets[4 * e + a] + (c >> 6)] |= 1ull << (c & 63);
    if (c + 1 > ncol) ncol = c + 1;
  }
  return ncol;
}

}  // extern "C"
