// Isotropic target size field of goal's adaptation (get_iso_target_size,
// src/goal_size_field.cpp:39-151), from per-element error indicators:
//   G        = sum_e |theta_e|^(2d/(2p+d))                      (:39-52)
//   factor   = (G / target)^(1/d)                               (:54-59)
//   h_e      = sqrt(mean of the squared edge lengths)           (:61-68)
//   h_new_e  = factor |theta_e|^(-2/(2p+d)) h_e, clamped to [alpha h_e, beta h_e]
//              with alpha = 1/4, beta = 2                       (:70-81, :29-30)
//   size_v   = mean of h_new over the elements around vertex v  (:96-106)
// with d = 3 and p = 1 (linear tets). h_e is the per-element size the
// discretization already keeps for the stabilization (same formula).
#include "disc.cuh"
#include "size_field.cuh"

namespace goal {
namespace {

constexpr double kD = 3.0, kP = 1.0;

__global__ void k_err_pow_part(int E, const double* __restrict__ err, const int* __restrict__ orig,
                               double* __restrict__ part) {
  KSum acc;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x)
    acc.add(pow(fabs(err[orig[s]]), (2.0 * kD) / (2.0 * kP + kD)));
  acc = block_reduce(acc);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = acc.s;
    part[2 * blockIdx.x + 1] = acc.c;
  }
}

// factor = (G / target)^(1/d) into out[0]
__global__ void k_size_factor(const double* __restrict__ part, int nb, double target, double* out) {
  KSum acc;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    KSum t;
    t.s = part[2 * i];
    t.c = part[2 * i + 1];
    acc.add(t);
  }
  acc = block_reduce(acc);
  if (threadIdx.x == 0) out[0] = pow(acc.value() / target, 1.0 / kD);
}

__global__ void k_elem_size(int E, const double* __restrict__ err, const int* __restrict__ orig,
                            const double* __restrict__ h, const double* __restrict__ factor,
                            double* __restrict__ hnew) {
  const double f = factor[0];
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) {
    const double he = h[s];
    const double r = pow(fabs(err[orig[s]]), (-2.0) / (2.0 * kP + kD));
    double hn = f * r * he;
    if (hn < 0.25 * he) hn = 0.25 * he;
    if (hn > 2.0 * he) hn = 2.0 * he;
    hnew[s] = hn;
  }
}

// vertex size = mean of the incident elements' sizes (nlist entries 4*s + a)
__global__ void k_vertex_mean(int N, const int* __restrict__ nptr, const int* __restrict__ nlist,
                              const double* __restrict__ hnew, double* __restrict__ out) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    const int c0 = nptr[n], c1 = nptr[n + 1];
    double acc = 0.0;
    for (int c = c0; c < c1; ++c) acc += hnew[nlist[c] >> 2];
    out[n] = c1 > c0 ? acc / (c1 - c0) : 0.0;
  }
}

}  // namespace

void iso_target_size(const Disc& d, const double* err, int target, double* vtx_size, cudaStream_t st) {
  GOAL_REQUIRE(target > 0, GOAL_ERR_ARG, "size field: target elements must be positive");
  const int E = d.num_elems, N = d.num_nodes;
  const int nb = std::min(grid_for(E, 256), 1024);
  DevBuf<double> part, hnew;
  part.alloc(2ull * nb + 2);
  hnew.alloc(E);
  k_err_pow_part<<<nb, 256, 0, st>>>(E, err, d.elem_orig.ptr, part.ptr);
  GOAL_CHECK_LAUNCH();
  k_size_factor<<<1, 1024, 0, st>>>(part.ptr, nb, (double)target, part.ptr + 2 * nb);
  GOAL_CHECK_LAUNCH();
  k_elem_size<<<grid_for(E, 256), 256, 0, st>>>(E, err, d.elem_orig.ptr, d.h.ptr, part.ptr + 2 * nb, hnew.ptr);
  GOAL_CHECK_LAUNCH();
  k_vertex_mean<<<grid_for(N, 256), 256, 0, st>>>(N, d.nptr.ptr, d.nlist.ptr, hnew.ptr, vtx_size);
  GOAL_CHECK_LAUNCH();
  GOAL_CUDA(cudaStreamSynchronize(st));
}

}  // namespace goal
