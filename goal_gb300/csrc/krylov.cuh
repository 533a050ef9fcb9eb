// Krylov solves on the 4x4-block matrix: the GB300 replacement of goal::solve
// (src/goal_linear_solve.cpp:53-90; Belos BlockGMRES + MueLu AMG there).
//
//   plain  : FGMRES(m) in FP64, right block-Jacobi preconditioner (4x4 node blocks)
//   nested : FGMRES(m) in FP64 whose preconditioner is a fixed number of inner
//            GMRES iterations on the dof-scaled matrix S A S with block-Jacobi;
//            the outer FP64 iteration refines to the requested tolerance. The
//            inner solve's storage and arithmetic:
//              PREC_MIXED      binary16 matrix and basis, FP32 arithmetic
//              PREC_MIXED_F32  FP32 matrix and basis, FP32 arithmetic
//              PREC_NESTED_F64 FP64 matrix and basis, FP64 arithmetic
//   learned: either of the above with the block-Jacobi blocks corrected by the
//            mesh-graph network (falls back to plain block-Jacobi when the
//            iteration count exceeds a cap)
// Convergence is on the true (unpreconditioned) residual ||b - A x|| / ||b||,
// which right preconditioning makes equal to the GMRES residual estimate.
// Every iteration runs on the device (Arnoldi, classical Gram-Schmidt with a
// conditional second pass, Givens rotations); the host reads one residual
// estimate per outer iteration.
#pragma once

#include <cuda_fp16.h>

#include "common.cuh"

namespace goal {

struct BsrView {
  int num_nodes;
  int nnzb;
  const int* brow_ptr;
  const int* bcol;
  const int* diag;
};

enum Precision : int { PREC_FP64 = 0, PREC_MIXED = 1, PREC_MIXED_F32 = 2, PREC_NESTED_F64 = 3 };
inline bool has_inner_solve(int precision) { return precision != PREC_FP64; }
enum Precond : int { PRECOND_BJ = 0, PRECOND_LEARNED = 1 };

struct SolveParams {
  int krylov_size = 100;      // outer restart length ("krylov size")
  int max_iters = 2000;       // outer iteration cap ("max iters")
  double tolerance = 1e-10;   // relative residual ("tolerance")
  int precision = PREC_FP64;
  int inner_iters = 30;       // inner GMRES iterations per outer iteration (nested precisions)
  int precond = PRECOND_BJ;
  int learned_cap = 0;        // fall back to plain block-Jacobi after this many outer iterations (0 = no cap)
};

struct SolveStats {
  int iters = 0;              // outer iterations
  int inner_iters = 0;        // total inner iterations
  double rel_res = 0.0;       // true relative residual at exit
  double seconds = 0.0;
  int converged = 0;
  int fell_back = 0;          // learned preconditioner replaced by plain block-Jacobi
  long long spmv64 = 0, spmv32 = 0;
};

// Device buffers of one solver instance (sized on first use).
struct Krylov {
  cudaStream_t stream = nullptr;
  int n = 0, m = 0, mi = 0;
  DevBuf<double> V, Z, w, r, H, cs, sn, g, y, red, scal, dots;
  DevBuf<double> Hi, csi, sni, gi, yi;   // inner (FP32 solve) Hessenberg and rotations
  // the inner solve of the nested precisions, on S A S with S = diag(|a_ii|^-1/2):
  // matrix and Krylov basis in binary16 (PREC_MIXED), FP32 (PREC_MIXED_F32) or
  // FP64 (PREC_NESTED_F64); work vectors and block-Jacobi blocks in the
  // arithmetic type (FP32, or FP64)
  DevBuf<float> w32, r32, t32;
  DevBuf<__half> V16, A16;
  DevBuf<float> V32, A32;
  DevBuf<double> w64, r64, t64, V64, A64;
  DevBuf<double> sd;
  DevBuf<double> Dinv;       // 16 x N inverse diagonal blocks (FP64)
  DevBuf<float> Dinv32;      // scaled blocks S^-1 D^-1 S^-1 of the inner solve
  DevBuf<double> Dinv64s;
  DevBuf<double> Bc64s;
  // learned two-sweep form: P r = z + B (r - A z), z = D^-1 r (B: 16 x N)
  bool two_sweep = false;
  DevBuf<double> Bc;
  DevBuf<float> Bc32;
  DevBuf<int> flag;
  double* h_scal = nullptr;  // pinned host mirror of a few scalars
  ~Krylov();
  void reserve(int n_, int m_, int mi_, int precision, int nnzb);
};

// Inverts the 4x4 diagonal blocks of A (optionally plus a correction dD,
// 16 x N, added before inversion) and selects plain block-Jacobi. Returns the
// number of singular blocks.
int block_jacobi_setup(const BsrView& A, const double* vals, const double* dD, Krylov& K);
// The inner solve's matrix: dof scales S and S A S in the storage type of the
// precision mode (binary16, FP32 or FP64).
void make_inner_copy(const BsrView& A, const double* vals, int precision, Krylov& K);

void spmv64(const BsrView& A, const double* vals, const double* x, double* y, cudaStream_t s);

// Solves A x = b (x holds the initial guess). All pointers are device pointers.
SolveStats fgmres(const BsrView& A, const double* vals, const double* b, double* x, const SolveParams& p, Krylov& K);

}  // namespace goal
