// Learned block-Jacobi correction: a 3-layer message-passing network on the
// node graph of the matrix, width 32, bfloat16 weights, float32 arithmetic,
// trained on the GPU with its own forward/backward kernels and Adam.
// It has no counterpart in the reference (goal preconditions with MueLu AMG,
// src/goal_linear_solve.cpp:59-65).
//
// The network sees the dof-scaled matrix A^ = S A S, S = diag(|a_ii|^-1/2),
// in which displacement and pressure rows are comparable:
//   x_n   = [D^_n, log10 max|D_n| - mean, offdiag/diag norm ratio of A^,
//            fraction of Dirichlet rows, (deg-1)/16]                (20 features)
//   e_nm  = A^_nm                                                   (16 features)
//   h0    = relu(W0 x + b0)
//   x3 layers: t_nm = We [e_nm; h_m] + be,  agg_n = mean_m relu(t_nm),
//              h_n += relu(Wu [h_n; agg_n] + bu)
//   W_n   = Wd h_n + bd, rows/columns of Dirichlet (identity) rows zeroed
// and weights the second of two block-Jacobi sweeps node by node:
//   z = D^-1 r,   P r = z + B (r - A z),   B_n = S_n W_n S_n^-1 D_n^-1.
// Training loss for probes w_i (scaled residual space): v_i = S^-1 w_i (even
// i) or A D^-1 S^-1 w_i (odd i), L = sum_i |S(v_i - A P v_i)|^2 / |S v_i|^2.
// Wd, bd start at zero, so the untrained network is plain block-Jacobi.
#pragma once

#include "common.cuh"
#include "krylov.cuh"

namespace goal {

constexpr int kMH = 32;   // hidden width
constexpr int kMF = 20;   // node features
constexpr int kME = 16;   // edge features
constexpr int kML = 3;    // message-passing layers

struct MpnnLayout {
  static constexpr int W0 = 0;
  static constexpr int b0 = W0 + kMH * kMF;
  static constexpr int L0 = b0 + kMH;
  static constexpr int We = 0;                          // offsets inside a layer
  static constexpr int be = We + kMH * (kME + kMH);
  static constexpr int Wu = be + kMH;
  static constexpr int bu = Wu + kMH * 2 * kMH;
  static constexpr int layer = bu + kMH;
  static constexpr int Wd = L0 + kML * layer;
  static constexpr int bd = Wd + 16 * kMH;
  static constexpr int total = bd + 16;
};

struct Mpnn {
  cudaStream_t stream = nullptr;
  std::vector<float> host_params;       // float32 master weights
  DevBuf<float> params, m1, m2;         // device master weights and Adam moments
  DevBuf<unsigned short> wbf;           // bfloat16 copy used by the kernels
  long long adam_t = 0;
  // per-graph work buffers
  DevBuf<float> x, h, t, u, agg, C, dC, dh, dh_acc, dagg, gbuf, grad, part;
  DevBuf<double> s, sd, Dinv, dP, y, r, gT, v, z, chat, red;
  DevBuf<int> tmap, deg, dmask;
  int cap_nodes = 0, cap_blocks = 0;
  void init(int seed);
  void upload();                        // host_params -> device (+ bfloat16 copy)
  void download();
  void reserve(int N, int nnzb);
};

struct BsrMatrix {
  BsrView v;
  const double* vals;
};

// Network outputs C (16 x N floats, node-major: W_n before masking) for matrix
// A; also leaves the dof scales S, D^-1 and the Dirichlet row masks in the
// network's buffers.
void mpnn_forward(Mpnn& net, const BsrMatrix& A, bool keep);
// Loss and parameter gradient (into net.grad) for the probe vectors (host or
// generated from seed when probes == nullptr).
double mpnn_loss_grad(Mpnn& net, const BsrMatrix& A, int num_probes, const double* probes_dev, unsigned seed);
// Adam step on net.params with net.grad.
void mpnn_adam(Mpnn& net, float lr, float beta1, float beta2, float eps);
// Writes the second-sweep blocks B (FP64) into the Krylov workspace
// and switches its preconditioner to the two-sweep form; the plain D^-1
// blocks must already be set up (block_jacobi_setup).
void mpnn_apply_to_block_jacobi(Mpnn& net, const BsrMatrix& A, Krylov& K);

}  // namespace goal
