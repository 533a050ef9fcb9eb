// Shared helpers of the GB300 element/solve library: error reporting, launch
// geometry, device buffers, compensated reductions.
#pragma once

#include <cuda_runtime.h>

#include "../../include/goal_gb300.h"

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace goal {

// Status codes of the C ABI (GOAL_OK = 0, GOAL_ERR_* nonzero) come from the
// public header. A nonzero status carries a message retrievable with
// goal_last_error(); the reference aborts instead (goal::fail,
// src/goal_control.cpp:91-99).
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

#define GOAL_CUDA(call)                                                                  \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      throw ::goal::Error(GOAL_ERR_CUDA,                                         \
                          std::string(#call) + ": " + cudaGetErrorString(e_) + " at " + \
                              __FILE__ + ":" + std::to_string(__LINE__));                \
  } while (0)

// Every kernel launch of this library is followed by GOAL_CHECK_LAUNCH(),
// which also counts it (goal_launch_count()).
extern std::atomic<long long> g_launches;
#define GOAL_CHECK_LAUNCH()                  \
  do {                                       \
    ::goal::g_launches.fetch_add(1);         \
    GOAL_CUDA(cudaGetLastError());           \
  } while (0)

#define GOAL_REQUIRE(cond, code, msg)                   \
  do {                                                  \
    if (!(cond)) throw ::goal::Error((code), (msg));    \
  } while (0)

constexpr int kSMs = 152;  // GB300: 2 dies x 76 SMs

inline int grid_for(long long n, int block, int max_blocks = kSMs * 32) {
  long long g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > max_blocks) g = max_blocks;
  return (int)g;
}

// Device allocation owned by a handle. Released with the owning object.
template <typename T>
struct DevBuf {
  T* ptr = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : ptr(o.ptr), n(o.n) { o.ptr = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); ptr = o.ptr; n = o.n; o.ptr = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count == n && ptr) return;
    release();
    if (count) GOAL_CUDA(cudaMalloc(&ptr, sizeof(T) * count));
    n = count;
  }
  void upload(const T* host, size_t count, cudaStream_t s = 0) {
    alloc(count);
    if (count) GOAL_CUDA(cudaMemcpyAsync(ptr, host, sizeof(T) * count, cudaMemcpyHostToDevice, s));
  }
  void download(T* host, cudaStream_t s = 0) const {
    if (n) GOAL_CUDA(cudaMemcpyAsync(host, ptr, sizeof(T) * n, cudaMemcpyDeviceToHost, s));
  }
  void zero(cudaStream_t s = 0) {
    if (n) GOAL_CUDA(cudaMemsetAsync(ptr, 0, sizeof(T) * n, s));
  }
  std::vector<T> to_host(cudaStream_t s = 0) const {
    std::vector<T> h(n);
    download(h.data(), s);
    GOAL_CUDA(cudaStreamSynchronize(s));
    return h;
  }
};

// grow-only: a buffer is reallocated only when it is smaller than required, so
// one workspace can serve problems of any size (kernels index with their own n)
template <typename T>
inline void need(DevBuf<T>& b, size_t count) {
  if (b.n < count || !b.ptr) b.alloc(count);
}

// ---------------------------------------------------------------- device side
#ifdef __CUDACC__
// Neumaier-compensated accumulator (sum + running correction).
struct KSum {
  double s, c;
  __device__ __forceinline__ KSum() : s(0.0), c(0.0) {}
  __device__ __forceinline__ void add(double x) {
    double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ void add(const KSum& o) {
    add(o.s);
    c += o.c;
  }
  __device__ __forceinline__ double value() const { return s + c; }
};

__device__ __forceinline__ KSum warp_reduce(KSum v) {
  for (int o = 16; o > 0; o >>= 1) {
    KSum w;
    w.s = __shfl_down_sync(0xffffffffu, v.s, o);
    w.c = __shfl_down_sync(0xffffffffu, v.c, o);
    v.add(w);
  }
  return v;
}

__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide compensated sum; result valid in thread 0. blockDim.x <= 1024.
__device__ __forceinline__ KSum block_reduce(KSum v) {
  __shared__ double ss[32], sc[32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_reduce(v);
  if (lane == 0) { ss[w] = v.s; sc[w] = v.c; }
  __syncthreads();
  KSum r;
  if (w == 0) {
    int nw = (blockDim.x + 31) >> 5;
    if (lane < nw) { r.s = ss[lane]; r.c = sc[lane]; }
    r = warp_reduce(r);
  }
  __syncthreads();
  return r;
}

__device__ __forceinline__ double block_max(double v) {
  __shared__ double sm[32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_max(v);
  if (lane == 0) sm[w] = v;
  __syncthreads();
  double r = -INFINITY;
  if (w == 0) {
    int nw = (blockDim.x + 31) >> 5;
    if (lane < nw) r = sm[lane];
    r = warp_max(r);
  }
  __syncthreads();
  return r;
}
#endif

}  // namespace goal
