// goal_avg_disp_noalloc: the "avg disp" functional of goal
// (AvgDisp::at_point, src/goal_avg_disp.cpp:17-21, summed over the mesh by
// Functional::compute, src/goal_functional.cpp) evaluated from caller-owned
// device arrays, without allocating device memory.
//
// The regular path (goal_assemble with GOAL_NONE and GOAL_QOI_AVG_DISP) writes
// one value per element into a buffer of the Mechanics and reduces it through a
// partial-sum buffer that grows on demand. This variant fuses the element
// values into the first reduction pass and keeps the per-block partial sums in
// a fixed file-scope device array, so a call performs kernel launches and
// nothing else: no cudaMalloc/cudaFree, no host synchronisation.
//
// Scratch: kMaxPartials compensated partial sums (two doubles each, 128 KiB).
// Every block of the first kernel owns a fixed chunk of kChunk elements, so
// the summation order depends on the element order only (not on the GPU), and
// at most kMaxPartials * kChunk = 16,777,216 elements fit; larger meshes are
// rejected with GOAL_ERR_CAPACITY. No scratch word has to start at zero: the
// second kernel reads only the partials the first one wrote in the same call.
// Calls that overlap in time (other streams, other host threads) share the
// scratch and race; callers order them (one stream, or events).
#include <mutex>

#include "common.cuh"

namespace goal {
namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 8;
constexpr int kChunk = kThreads * kPerThread;  // elements per block
constexpr int kMaxPartials = 8192;
constexpr long long kMaxElems = (long long)kMaxPartials * kChunk;
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_partials[2 * kMaxPartials];

double* g_scratch[kMaxDevices];  // address of g_partials per device (nullptr until set up)
std::mutex g_setup_mutex;

// Same element arithmetic as the QoI section of the element kernel: volume by
// the Jacobian determinant of the reference map, nodal average of u, the three
// components summed and divided by the dimension.
__global__ void __launch_bounds__(kThreads) k_avg_disp_partials(const double* __restrict__ X,
                                                                const int* __restrict__ tets,
                                                                const double* __restrict__ U, int num_nodes,
                                                                int num_elems, double* __restrict__ part) {
  constexpr double kThird = 1.0 / 3.0;
  KSum acc;
  const int base = blockIdx.x * kChunk + threadIdx.x;
#pragma unroll 2
  for (int j = 0; j < kPerThread; ++j) {
    const int e = base + j * kThreads;
    if (e >= num_elems) break;
    int v[4];
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      v[a] = tets[4 * (size_t)e + a];
      ok = ok && v[a] >= 0 && v[a] < num_nodes;
    }
    if (!ok) {  // a node id outside the mesh poisons the result
      acc.c = __longlong_as_double(0x7ff8000000000000ll);
      continue;
    }
    double J[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int r = 0; r < 3; ++r) J[r][c] = X[3 * (size_t)v[c + 1] + r] - X[3 * (size_t)v[0] + r];
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][0] * J[2][2] - J[1][2] * J[2][0];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const double V = (J[0][0] * c00 - J[0][1] * c01 + J[0][2] * c02) / 6.0;
    double ev = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double ui = ((U[4 * (size_t)v[0] + i] * 0.25 + U[4 * (size_t)v[1] + i] * 0.25) +
                         U[4 * (size_t)v[2] + i] * 0.25) +
                        U[4 * (size_t)v[3] + i] * 0.25;
      ev += ui * V;
    }
    acc.add(ev * kThird);
  }
  acc = block_reduce(acc);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = acc.s;
    part[2 * blockIdx.x + 1] = acc.c;
  }
}

__global__ void __launch_bounds__(1024) k_avg_disp_final(const double* __restrict__ part, int nb,
                                                         double* __restrict__ out) {
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

int fail(int code, const char* msg) {
  set_last_error(msg);
  return code;
}

}  // namespace
}  // namespace goal

extern "C" int goal_avg_disp_noalloc(const double* coords, const int* tets, const double* U, int num_nodes,
                                     int num_elems, double* J, void* stream) {
  using namespace goal;
  if (coords == nullptr || tets == nullptr || U == nullptr || J == nullptr)
    return fail(GOAL_ERR_ARG, "goal_avg_disp_noalloc: null pointer");
  if (num_nodes < 4 || num_elems < 1) return fail(GOAL_ERR_ARG, "goal_avg_disp_noalloc: empty mesh");
  if ((long long)num_elems > kMaxElems)
    return fail(GOAL_ERR_CAPACITY,
                "goal_avg_disp_noalloc: more than 16777216 elements (fixed scratch of 8192 partial sums)");
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(GOAL_ERR_CUDA, "goal_avg_disp_noalloc: no usable current device");
  double* scratch = nullptr;
  {
    // First call on a device, with that device current: look up the scratch
    // array's address once (a runtime query, made before the launches below).
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch[dev] == nullptr) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_partials);
      if (e != cudaSuccess || p == nullptr) {
        set_last_error(cudaGetErrorString(e));
        return GOAL_ERR_CUDA;
      }
      g_scratch[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nb = (num_elems + kChunk - 1) / kChunk;
  k_avg_disp_partials<<<nb, kThreads, 0, st>>>(coords, tets, U, num_nodes, num_elems, scratch);
  g_launches.fetch_add(1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return GOAL_ERR_CUDA;
  }
  k_avg_disp_final<<<1, 1024, 0, st>>>(scratch, nb, J);
  g_launches.fetch_add(1);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return GOAL_ERR_CUDA;
  }
  return GOAL_OK;
}
