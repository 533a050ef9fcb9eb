// Learned block-Jacobi correction: a 3-layer message-passing network on the
// node graph of the matrix, width 32, bfloat16 weights, float32 arithmetic,
// trained on the GPU with its own forward/backward kernels and Adam.
// It has no counterpart in the reference (goal preconditions with MueLu AMG,
// src/goal_linear_solve.cpp:59-65).
//
//   s_n   = max |D_n|,  x_n = [D_n/s_n, log10 s_n - mean, offdiag/diag norm ratio,
//                              Dirichlet flag, (deg-1)/16]               (20 features)
//   e_nm  = A_nm / sqrt(s_n s_m)                                           (16 features)
//   h0    = relu(W0 x + b0)
//   x3 layers: t_nm = We [e_nm; h_m] + be,  agg_n = mean_m relu(t_nm),
//              h_n += relu(Wu [h_n; agg_n] + bu)
//   C_n   = Wd h_n + bd;   preconditioner block P_n = D_n^-1 + C_n / s_n
// Training loss for probe vectors v: sum_v |v - A P v|^2 / |v|^2 (P acts as a
// right preconditioner). Wd, bd start at zero, so the untrained network is
// plain block-Jacobi.
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
  DevBuf<float> x, h, t, u, agg, C, dC, dh, dagg, gbuf, grad, part;
  DevBuf<double> s, Dinv, dP, y, r, gT, v, red;
  DevBuf<int> tmap, deg;
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

// Corrections C (16 x N floats, node-major) of the network for matrix A; also
// leaves the node scales s and D^-1 in the network's buffers.
void mpnn_forward(Mpnn& net, const BsrMatrix& A, bool keep);
// Loss and parameter gradient (into net.grad) for the probe vectors (host or
// generated from seed when probes == nullptr).
double mpnn_loss_grad(Mpnn& net, const BsrMatrix& A, int num_probes, const double* probes_dev, unsigned seed);
// Adam step on net.params with net.grad.
void mpnn_adam(Mpnn& net, float lr, float beta1, float beta2, float eps);
// Writes D^-1 + C/s into Krylov's block-Jacobi buffers (FP64 and FP32).
void mpnn_apply_to_block_jacobi(Mpnn& net, const BsrMatrix& A, Krylov& K);

}  // namespace goal
