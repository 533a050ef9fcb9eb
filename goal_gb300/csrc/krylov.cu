// Device-resident FGMRES on 4x4-block matrices (see krylov.cuh).
//
// Iteration state (column count j, done flag, reorthogonalization flag,
// residual estimate) lives in device memory, so one Arnoldi step is a fixed
// sequence of kernels that never waits for the host: the host enqueues steps
// and reads the residual estimate once per step.
#include <chrono>
#include <cmath>

#include "krylov.cuh"

#include <cuda_fp16.h>

#include <type_traits>

namespace goal {

namespace {

struct GState {
  int j;        // completed Arnoldi columns in this cycle
  int done;     // 1: converged, broke down or restart length reached
  int reorth;   // second Gram-Schmidt pass needed for the current column
  int pad;
  double wb2;   // |w|^2 before orthogonalization
  double res;   // |g[j]| residual estimate
  double beta;  // initial residual norm of the cycle
  double hnext; // |w| after a single-pass orthogonalization (read by the normalization)
  double inv;   // 1/|w| (or 1/beta) for the next normalization, 0 for a zero norm
  float inv32;  // the same in FP32, for the FP32 solve
  float pad2;
};

// On GB300 every FP64 instruction occupies the FP64 pipe for a whole warp
// (two lanes per clock per SM), so per-thread FP64 scalar work is costly: the
// reciprocals for the normalizations are formed once, by the thread that
// computed the norm, and the FP32 solve keeps its Hessenberg matrix, rotations
// and partial sums in FP32.
__device__ __forceinline__ void set_inv(GState* st, double h) {
  st->inv = h > 0.0 ? 1.0 / h : 0.0;
  st->inv32 = (float)st->inv;
}
__device__ __forceinline__ void set_inv(GState* st, float h) {
  st->inv32 = h > 0.0f ? 1.0f / h : 0.0f;
  st->inv = (double)st->inv32;
}
template <typename T>
__device__ __forceinline__ T state_inv(const GState* st);
template <>
__device__ __forceinline__ double state_inv<double>(const GState* st) {
  return st->inv;
}
template <>
__device__ __forceinline__ float state_inv<float>(const GState* st) {
  return st->inv32;
}
__device__ __forceinline__ double c_hypot(double a, double b) { return hypot(a, b); }

// This thread's share of a sum of n block partials (stride blockDim.x), four
// independent loads in flight: the sum of a few thousand partials is bound
// by memory latency, not by the adds.
template <typename C>
__device__ __forceinline__ C thread_partial_sum(const C* __restrict__ p, int n) {
  const int nt = blockDim.x;
  C a0 = C(0), a1 = C(0), a2 = C(0), a3 = C(0);
  int k = threadIdx.x;
  for (; k + 3 * nt < n; k += 4 * nt) {
    a0 += p[k];
    a1 += p[k + nt];
    a2 += p[k + 2 * nt];
    a3 += p[k + 3 * nt];
  }
  for (; k < n; k += nt) a0 += p[k];
  return (a0 + a1) + (a2 + a3);
}
__device__ __forceinline__ float c_hypot(float a, float b) { return hypotf(a, b); }

constexpr int kMaxM = 256;
constexpr int kDotChunk = 8;
// Gram-Schmidt passes: the FP64 outer basis gets the conditional second pass;
// the fixed-length FP32 inner solve is only a preconditioner of the flexible
// outer solve and takes one pass (measured on the nested adjoints: same outer
// iteration counts, 25% less inner time).
constexpr int kOuterPasses = 2, kInnerPasses = 1;
constexpr int kMaxRows = 8;  // rows per thread in the orthogonalization kernels: 1, 2, 4 or 8

template <typename T>
struct Vec4;
template <>
struct Vec4<double> {
  static __device__ __forceinline__ void load(const double* p, double& a, double& b, double& c, double& d) {
    double4_32a v = *reinterpret_cast<const double4_32a*>(p);
    a = v.x; b = v.y; c = v.z; d = v.w;
  }
};
template <>
struct Vec4<float> {
  static __device__ __forceinline__ void load(const float* p, float& a, float& b, float& c, float& d) {
    float4 v = *reinterpret_cast<const float4*>(p);
    a = v.x; b = v.y; c = v.z; d = v.w;
  }
};

// One row of a 4x4 matrix block in the arithmetic type T: same-type loads, or
// four binary16 values (the inner solve's matrix) widened to float.
template <typename T>
struct Vec4Store;
template <>
struct Vec4Store<double> {
  static __device__ __forceinline__ void store(double* p, double a, double b, double c, double d) {
    double4_32a v;
    v.x = a; v.y = b; v.z = c; v.w = d;
    *reinterpret_cast<double4_32a*>(p) = v;
  }
};
template <>
struct Vec4Store<float> {
  static __device__ __forceinline__ void store(float* p, float a, float b, float c, float d) {
    *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
  }
};
template <>
struct Vec4Store<__half> {
  static __device__ __forceinline__ void store(__half* p, float a, float b, float c, float d) {
    const __half2 h0 = __floats2half2_rn(a, b), h1 = __floats2half2_rn(c, d);
    uint2 u;
    u.x = *reinterpret_cast<const unsigned*>(&h0);
    u.y = *reinterpret_cast<const unsigned*>(&h1);
    *reinterpret_cast<uint2*>(p) = u;
  }
};

template <typename T, typename TA>
__device__ __forceinline__ void load_row(const TA* p, T& a, T& b, T& c, T& d) {
  Vec4<T>::load(p, a, b, c, d);
}
template <>
__device__ __forceinline__ void load_row<float, __half>(const __half* p, float& a, float& b, float& c, float& d) {
  const uint2 u = *reinterpret_cast<const uint2*>(p);
  const float2 f0 = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
  const float2 f1 = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
  a = f0.x; b = f0.y; c = f1.x; d = f1.y;
}

// Basis entries in their storage type (the inner solve keeps its basis in
// binary16), read and written in the arithmetic type.
template <typename T, typename TV>
__device__ __forceinline__ T ldv(const TV* p) {
  return (T)(*p);
}
template <>
__device__ __forceinline__ float ldv<float, __half>(const __half* p) {
  return __half2float(*p);
}
template <typename TV, typename T>
__device__ __forceinline__ void stv(TV* p, T v) {
  *p = (TV)v;
}
template <>
__device__ __forceinline__ void stv<__half, float>(__half* p, float v) {
  *p = __float2half_rn(v);
}

// Block-row product of node n, row r: sum_k A_k[r,:] . x_{bcol[k]}, one fused
// multiply-add per matrix entry (on GB300 the FP64 pipe, not HBM, bounds the
// FP64 kernels, so no operation is spent on reductions).
template <typename T, typename TA>
__device__ __forceinline__ T block_row_dot(const int* __restrict__ bcol, const TA* __restrict__ A,
                                           const T* __restrict__ x, int b0, int b1, int r) {
  T acc = T(0);
#pragma unroll 4
  for (int k = b0; k < b1; ++k) {
    const int c = __ldg(bcol + k);
    T a0, a1, a2, a3, x0, x1, x2, x3;
    load_row<T, TA>(A + 16ll * k + 4 * r, a0, a1, a2, a3);
    Vec4<T>::load(x + 4ll * c, x0, x1, x2, x3);
    acc = fma(a0, x0, acc);
    acc = fma(a1, x1, acc);
    acc = fma(a2, x2, acc);
    acc = fma(a3, x3, acc);
  }
  return acc;
}

// y = A x  (or y = b - A x). Four threads per block row (one per row of the
// node's 4x4 blocks), no cross-thread reduction.
template <typename T, typename TA, bool RESID>
__global__ void __launch_bounds__(256) k_spmv(int N, const int* __restrict__ brow_ptr, const int* __restrict__ bcol,
                                              const TA* __restrict__ A, const T* __restrict__ x,
                                              const T* __restrict__ b, T* __restrict__ y) {
  const int r = threadIdx.x & 3;
  const int nq = (gridDim.x * blockDim.x) >> 2;
  for (int n = (blockIdx.x * blockDim.x + threadIdx.x) >> 2; n < N; n += nq) {
    const T acc = block_row_dot<T, TA>(bcol, A, x, __ldg(brow_ptr + n), __ldg(brow_ptr + n + 1), r);
    if (RESID) y[4ll * n + r] = b[4ll * n + r] - acc;
    else y[4ll * n + r] = acc;
  }
}

// z = Dinv v for node blocks (one thread per row); column j of V/Z from the state.
template <typename T>
__global__ void k_bj_col(int N, const T* __restrict__ Dinv, const T* V, T* Z, long long ld, const GState* st) {
  if (st->done) return;
  const long long off = (long long)st->j * ld;
  const T* v = V + off;
  T* z = Z + off;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * N; i += gridDim.x * blockDim.x) {
    int n = i >> 2, r = i & 3;
    T d0, d1, d2, d3, x0, x1, x2, x3;
    Vec4<T>::load(Dinv + 16ll * n + 4 * r, d0, d1, d2, d3);
    Vec4<T>::load(v + 4ll * n, x0, x1, x2, x3);
    z[i] = d0 * x0 + d1 * x1 + d2 * x2 + d3 * x3;
  }
}

// out = Dinv v_j with v_j = column j of V
template <typename T, typename TV>
__global__ void k_bj_colin(int N, const T* __restrict__ Dinv, const TV* V, long long ld, const GState* st,
                           T* __restrict__ out) {
  if (st->done) return;
  const TV* v = V + (long long)st->j * ld;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * N; i += gridDim.x * blockDim.x) {
    int n = i >> 2, r = i & 3;
    T d0, d1, d2, d3, x0, x1, x2, x3;
    Vec4<T>::load(Dinv + 16ll * n + 4 * r, d0, d1, d2, d3);
    load_row<T, TV>(v + 4ll * n, x0, x1, x2, x3);
    out[i] = d0 * x0 + d1 * x1 + d2 * x2 + d3 * x3;
  }
}

template <typename T>
__global__ void k_bj(int N, const T* __restrict__ Dinv, const T* __restrict__ v, T* __restrict__ z) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * N; i += gridDim.x * blockDim.x) {
    int n = i >> 2, r = i & 3;
    T d0, d1, d2, d3, x0, x1, x2, x3;
    Vec4<T>::load(Dinv + 16ll * n + 4 * r, d0, d1, d2, d3);
    Vec4<T>::load(v + 4ll * n, x0, x1, x2, x3);
    z[i] = d0 * x0 + d1 * x1 + d2 * x2 + d3 * x3;
  }
}

// Second, weighted block-Jacobi sweep of the learned preconditioner:
// z += B (v - w) with w = A z, for column j of V and Z (state st; offset 0
// and no gate without a state).
template <typename T, typename TV>
__global__ void k_second_sweep_col(int N, const T* __restrict__ B, const TV* V, long long ldv, const T* __restrict__ w,
                                   T* Z, long long ldz, const GState* st) {
  if (st && st->done) return;
  const long long j = st ? st->j : 0;
  const TV* v = V + j * ldv;
  T* z = Z + j * ldz;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * N; i += gridDim.x * blockDim.x) {
    int n = i >> 2, r = i & 3;
    T b0, b1, b2, b3, v0, v1, v2, v3, w0, w1, w2, w3;
    Vec4<T>::load(B + 16ll * n + 4 * r, b0, b1, b2, b3);
    load_row<T, TV>(v + 4ll * n, v0, v1, v2, v3);
    Vec4<T>::load(w + 4ll * n, w0, w1, w2, w3);
    z[i] += b0 * (v0 - w0) + b1 * (v1 - w1) + b2 * (v2 - w2) + b3 * (v3 - w3);
  }
}

// w = A z_j with z_j = column j of Z
template <typename T, typename TA>
__global__ void __launch_bounds__(256) k_spmv_col(int N, const int* __restrict__ brow_ptr,
                                                  const int* __restrict__ bcol, const TA* __restrict__ A,
                                                  const T* Z, long long ld, const GState* st, T* __restrict__ y) {
  if (st->done) return;
  const T* x = Z + (long long)st->j * ld;
  const int r = threadIdx.x & 3;
  const int nq = (gridDim.x * blockDim.x) >> 2;
  for (int n = (blockIdx.x * blockDim.x + threadIdx.x) >> 2; n < N; n += nq)
    y[4ll * n + r] = block_row_dot<T, TA>(bcol, A, x, __ldg(brow_ptr + n), __ldg(brow_ptr + n + 1), r);
}

// First half of the learned preconditioner's step, fused: t = A z1 for the
// node (z1 = x, the block-Jacobi sweep of v_j), then z = z1 + B (v_j - t).
// The node's four rows are the four lanes of a quad, which exchange their t
// by shuffles. z goes to out, not over x: other quads still read z1. Same
// arithmetic as k_spmv_col followed by k_second_sweep_col.
template <typename T, typename TA, typename TV>
__global__ void __launch_bounds__(256, sizeof(T) == 8 ? 4 : 8) k_spmv_sweep(int N, const int* __restrict__ brow_ptr,
                                                    const int* __restrict__ bcol, const TA* __restrict__ A,
                                                    const T* __restrict__ x, const T* __restrict__ B, const TV* V,
                                                    long long ldv, const GState* st, T* __restrict__ out) {
  if (st->done) return;
  const TV* v = V + (long long)st->j * ldv;
  const int lane = threadIdx.x & 31, r = lane & 3, q0 = lane & ~3;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int nb = warp * 8; nb < N; nb += nwarps * 8) {
    const int n = nb + (lane >> 2);
    const bool live = n < N;
    const T t = live ? block_row_dot<T, TA>(bcol, A, x, __ldg(brow_ptr + n), __ldg(brow_ptr + n + 1), r) : T(0);
    const T w0 = __shfl_sync(0xffffffffu, t, q0), w1 = __shfl_sync(0xffffffffu, t, q0 + 1);
    const T w2 = __shfl_sync(0xffffffffu, t, q0 + 2), w3 = __shfl_sync(0xffffffffu, t, q0 + 3);
    if (live) {
      T b0, b1, b2, b3, v0, v1, v2, v3;
      Vec4<T>::load(B + 16ll * n + 4 * r, b0, b1, b2, b3);
      load_row<T, TV>(v + 4ll * n, v0, v1, v2, v3);
      T z = x[4ll * n + r];
      z += b0 * (v0 - w0) + b1 * (v1 - w1) + b2 * (v2 - w2) + b3 * (v3 - w3);
      out[4ll * n + r] = z;
    }
  }
}

// Orthogonalization kernels work on row slabs of 256 x R rows per block:
// every thread keeps its R entries of w in registers, and the
// columns of V are streamed slab by slab (long contiguous reads, w read once).

// Sums the kDotChunk per-thread values of a 256-thread block column by
// column (staged through shared memory, one warp per column; no FP64 work for
// float data); lane 0 of warp q returns column q's sum.
template <typename T>
__device__ __forceinline__ T chunk_reduce(const T (&acc)[kDotChunk], T (*sm)[257]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int cc = 0; cc < kDotChunk; ++cc) sm[cc][threadIdx.x] = acc[cc];
  __syncthreads();
  T v = T(0);
#pragma unroll
  for (int t = 0; t < 8; ++t) v += sm[wid][lane + 32 * t];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  return v;
}

// partial dot products of w with columns 0..j of V and with itself (column
// j+1); part[c * gridDim.x + block]
template <typename T, typename TV, int R>
__global__ void __launch_bounds__(256) k_multidot(long long n, const TV* V, long long ld, const T* __restrict__ w,
                                                  const GState* st, T* part, int pass) {
  if (st->done) return;
  if (pass == 1 && !st->reorth) return;
  const int j = st->j;
  const int ncols = j + 2;
  const long long base = (long long)blockIdx.x * (256ll * R) + threadIdx.x;
  T wr[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const long long i = base + 256ll * q;
    wr[q] = i < n ? w[i] : T(0);
  }
  __shared__ T sm[kDotChunk][257];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c0 = 0; c0 < ncols; c0 += kDotChunk) {
    T acc[kDotChunk];
#pragma unroll
    for (int cc = 0; cc < kDotChunk; ++cc) {
      const int c = c0 + cc;
      T a = T(0);
      if (c <= j) {
        const TV* v = V + (long long)c * ld;
#pragma unroll
        for (int q = 0; q < R; ++q) {
          const long long i = base + 256ll * q;
          if (i < n) a = fma(ldv<T, TV>(v + i), wr[q], a);
        }
      } else if (c == j + 1) {
#pragma unroll
        for (int q = 0; q < R; ++q) a = fma(wr[q], wr[q], a);
      }
      acc[cc] = a;
    }
    const T v = chunk_reduce<T>(acc, sm);
    const int c = c0 + wid;
    if (lane == 0 && c < ncols) part[(long long)c * gridDim.x + blockIdx.x] = v;
  }
}

template <typename C>
__global__ void k_dots_fin(int nbx, const C* part, GState* st, C* H, int ldh, C* dots, int pass) {
  if (st->done) return;
  if (pass == 1 && !st->reorth) return;
  const int j = st->j;
  const int c = blockIdx.x;
  if (c > j + 1) return;
  C v = thread_partial_sum<C>(part + (long long)c * nbx, nbx);
  __shared__ C sm[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    C s = C(0);
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sm[k];
    if (c <= j) {
      dots[c] = s;
      if (pass == 0) H[c + (long long)ldh * j] = s;
      else H[c + (long long)ldh * j] += s;
    } else if (pass == 0) {
      st->wb2 = s;
    }
  }
}

// w -= V dots ; partial |w|^2 per block
template <typename T, typename TV, int R>
__global__ void __launch_bounds__(256) k_update(long long n, const TV* V, long long ld, T* w, const T* dots,
                                                const GState* st, T* part, int pass) {
  if (st->done) return;
  if (pass == 1 && !st->reorth) return;
  const int j = st->j;
  __shared__ T sd[kMaxM + 1];
  for (int c = threadIdx.x; c <= j; c += blockDim.x) sd[c] = (T)dots[c];
  __syncthreads();
  const long long base = (long long)blockIdx.x * (256ll * R) + threadIdx.x;
  T wr[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const long long i = base + 256ll * q;
    wr[q] = i < n ? w[i] : T(0);
  }
  int c = 0;
  for (; c + 1 <= j; c += 2) {
    const T d0 = -sd[c], d1 = -sd[c + 1];
    const TV* v0 = V + (long long)c * ld;
    const TV* v1 = v0 + ld;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const long long i = base + 256ll * q;
      if (i < n) wr[q] = fma(d1, ldv<T, TV>(v1 + i), fma(d0, ldv<T, TV>(v0 + i), wr[q]));
    }
  }
  for (; c <= j; ++c) {
    const T d0 = -sd[c];
    const TV* v0 = V + (long long)c * ld;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const long long i = base + 256ll * q;
      if (i < n) wr[q] = fma(d0, ldv<T, TV>(v0 + i), wr[q]);
    }
  }
  T acc = T(0);
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const long long i = base + 256ll * q;
    if (i < n) {
      w[i] = wr[q];
      acc = fma(wr[q], wr[q], acc);
    }
  }
  __shared__ T sm[8];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    T s = T(0);
    for (int k = 0; k < 8; ++k) s += sm[k];
    part[blockIdx.x] = s;
  }
}

// Variants for a binary16 basis: every thread owns G groups of four
// consecutive rows (n = 4 x nodes, so a group is all in or all out), reads a
// group of w as one 16-byte load and a group of a basis column as one 8-byte
// load; a block covers 1024 G rows. Same sums as k_multidot / k_update.
template <typename T, typename TV, int G>
__global__ void __launch_bounds__(256) k_multidot_v(long long n, const TV* V, long long ld, const T* __restrict__ w,
                                                    const GState* st, T* part, int pass) {
  if (st->done) return;
  if (pass == 1 && !st->reorth) return;
  const int j = st->j;
  const int ncols = j + 2;
  const long long base = (long long)blockIdx.x * (1024ll * G) + 4 * threadIdx.x;
  T wr[G][4];
#pragma unroll
  for (int q = 0; q < G; ++q) {
    const long long i = base + 1024ll * q;
    if (i < n) Vec4<T>::load(w + i, wr[q][0], wr[q][1], wr[q][2], wr[q][3]);
    else wr[q][0] = wr[q][1] = wr[q][2] = wr[q][3] = T(0);
  }
  __shared__ T sm[kDotChunk][257];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c0 = 0; c0 < ncols; c0 += kDotChunk) {
    T acc[kDotChunk];
#pragma unroll
    for (int cc = 0; cc < kDotChunk; ++cc) {
      const int c = c0 + cc;
      T a = T(0);
      if (c <= j) {
        const TV* v = V + (long long)c * ld;
#pragma unroll
        for (int q = 0; q < G; ++q) {
          const long long i = base + 1024ll * q;
          if (i < n) {
            T x0, x1, x2, x3;
            load_row<T, TV>(v + i, x0, x1, x2, x3);
            a = fma(x0, wr[q][0], a);
            a = fma(x1, wr[q][1], a);
            a = fma(x2, wr[q][2], a);
            a = fma(x3, wr[q][3], a);
          }
        }
      } else if (c == j + 1) {
#pragma unroll
        for (int q = 0; q < G; ++q)
#pragma unroll
          for (int e = 0; e < 4; ++e) a = fma(wr[q][e], wr[q][e], a);
      }
      acc[cc] = a;
    }
    const T v = chunk_reduce<T>(acc, sm);
    const int c = c0 + wid;
    if (lane == 0 && c < ncols) part[(long long)c * gridDim.x + blockIdx.x] = v;
  }
}

template <typename T, typename TV, int G>
__global__ void __launch_bounds__(256) k_update_v(long long n, const TV* V, long long ld, T* w, const T* dots,
                                                  const GState* st, T* part, int pass) {
  if (st->done) return;
  if (pass == 1 && !st->reorth) return;
  const int j = st->j;
  __shared__ T sd[kMaxM + 1];
  for (int c = threadIdx.x; c <= j; c += blockDim.x) sd[c] = dots[c];
  __syncthreads();
  const long long base = (long long)blockIdx.x * (1024ll * G) + 4 * threadIdx.x;
  T wr[G][4];
#pragma unroll
  for (int q = 0; q < G; ++q) {
    const long long i = base + 1024ll * q;
    if (i < n) Vec4<T>::load(w + i, wr[q][0], wr[q][1], wr[q][2], wr[q][3]);
    else wr[q][0] = wr[q][1] = wr[q][2] = wr[q][3] = T(0);
  }
  for (int c = 0; c <= j; ++c) {
    const T d = -sd[c];
    const TV* v = V + (long long)c * ld;
#pragma unroll
    for (int q = 0; q < G; ++q) {
      const long long i = base + 1024ll * q;
      if (i < n) {
        T x0, x1, x2, x3;
        load_row<T, TV>(v + i, x0, x1, x2, x3);
        wr[q][0] = fma(d, x0, wr[q][0]);
        wr[q][1] = fma(d, x1, wr[q][1]);
        wr[q][2] = fma(d, x2, wr[q][2]);
        wr[q][3] = fma(d, x3, wr[q][3]);
      }
    }
  }
  T acc = T(0);
#pragma unroll
  for (int q = 0; q < G; ++q) {
    const long long i = base + 1024ll * q;
    if (i < n) {
      Vec4Store<T>::store(w + i, wr[q][0], wr[q][1], wr[q][2], wr[q][3]);
#pragma unroll
      for (int e = 0; e < 4; ++e) acc = fma(wr[q][e], wr[q][e], acc);
    }
  }
  __shared__ T sm[8];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    T s = T(0);
    for (int k = 0; k < 8; ++k) s += sm[k];
    part[blockIdx.x] = s;
  }
}

template <typename C>
__global__ void k_norm_fin(int nbx, const C* part, GState* st, C* H, int ldh, int pass) {
  if (st->done) return;
  if (pass == 1 && !st->reorth) return;
  C v = thread_partial_sum<C>(part, nbx);
  __shared__ C sm[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    C s = C(0);
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sm[k];
    const int j = st->j;
    if (pass == 0) st->reorth = (s < C(0.5) * (C)st->wb2) ? 1 : 0;
    const C h = sqrt(s);
    H[j + 1 + (long long)ldh * j] = h;
    set_inv(st, h);
  }
}


// V_{j+1} = w / H[j+1, j], four entries per thread (n = 4 x nodes; every
// column starts on a 32-byte boundary)
template <typename T, typename TV>
__global__ void k_normalize(long long n, TV* V, long long ld, const T* w, const GState* st) {
  if (st->done) return;
  const int j = st->j;
  const T inv = state_inv<T>(st);
  TV* v = V + (long long)(j + 1) * ld;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; 4 * q < n; q += (long long)gridDim.x * blockDim.x) {
    T a, b, c, d;
    Vec4<T>::load(w + 4 * q, a, b, c, d);
    Vec4Store<TV>::store(v + 4 * q, a * inv, b * inv, c * inv, d * inv);
  }
}

// Applies the previous rotations to the new Hessenberg column (staged in
// shared memory by the whole block), then forms rotation j (thread 0).
template <typename C>
__global__ void k_givens(GState* st, C* H, int ldh, C* cs, C* sn, C* g, int jmax, double tol_abs) {
  if (st->done) return;
  const int j = st->j;
  C* h = H + (long long)ldh * j;
  __shared__ C sh[kMaxM + 2], scs[kMaxM + 1], ssn[kMaxM + 1];
  for (int i = threadIdx.x; i <= j + 1; i += blockDim.x) sh[i] = h[i];
  for (int i = threadIdx.x; i < j; i += blockDim.x) {
    scs[i] = cs[i];
    ssn[i] = sn[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < j; ++i) {
      const C t = scs[i] * sh[i] + ssn[i] * sh[i + 1];
      sh[i + 1] = -ssn[i] * sh[i] + scs[i] * sh[i + 1];
      sh[i] = t;
    }
    const C a = sh[j], b = sh[j + 1];
    const C r = c_hypot(a, b);
    C c = C(1), s = C(0);
    if (r > C(0)) { c = a / r; s = b / r; }
    cs[j] = c;
    sn[j] = s;
    sh[j] = r;
    sh[j + 1] = C(0);
    g[j + 1] = -s * g[j];
    g[j] = c * g[j];
    st->res = (double)fabs(g[j + 1]);
    st->j = j + 1;
    if (st->res <= tol_abs || st->j >= jmax || b == C(0) || !(st->res == st->res)) st->done = 1;
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= j + 1; i += blockDim.x) h[i] = sh[i];
}

// Single-pass orthogonalization: |w| from the block partials (H[j+1, j] and
// hnext), then the Givens step, in one block.
template <typename C>
__global__ void k_norm_givens(int nbx, const C* part, GState* st, C* H, int ldh, C* cs, C* sn, C* g, int jmax,
                              double tol_abs) {
  if (st->done) return;
  const int j = st->j;
  C v = thread_partial_sum<C>(part, nbx);
  __shared__ C sm[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  C* h = H + (long long)ldh * j;
  __shared__ C sh[kMaxM + 2], scs[kMaxM + 1], ssn[kMaxM + 1];
  if (threadIdx.x == 0) {
    C s2 = C(0);
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s2 += sm[k];
    const C nrm = sqrt(s2);
    st->hnext = (double)nrm;
    set_inv(st, nrm);
    sh[j + 1] = nrm;
  }
  for (int i = threadIdx.x; i <= j; i += blockDim.x) sh[i] = h[i];
  for (int i = threadIdx.x; i < j; i += blockDim.x) {
    scs[i] = cs[i];
    ssn[i] = sn[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < j; ++i) {
      const C t = scs[i] * sh[i] + ssn[i] * sh[i + 1];
      sh[i + 1] = -ssn[i] * sh[i] + scs[i] * sh[i + 1];
      sh[i] = t;
    }
    const C a = sh[j], b = sh[j + 1];
    const C r = c_hypot(a, b);
    C c = C(1), s = C(0);
    if (r > C(0)) { c = a / r; s = b / r; }
    cs[j] = c;
    sn[j] = s;
    sh[j] = r;
    sh[j + 1] = C(0);
    g[j + 1] = -s * g[j];
    g[j] = c * g[j];
    st->res = (double)fabs(g[j + 1]);
    st->j = j + 1;
    if (st->res <= tol_abs || st->j >= jmax || b == C(0) || !(st->res == st->res)) st->done = 1;
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= j + 1; i += blockDim.x) h[i] = sh[i];
}

// V_j = w / hnext after k_norm_givens advanced j, and out = Dinv V_j (the
// block-Jacobi sweep of the next Arnoldi step, from the stored entries): one
// node (four rows) per thread
template <typename T, typename TV>
__global__ void k_normalize_next_bj(long long n, TV* V, long long ld, const T* w, const GState* st,
                                    const T* __restrict__ Dinv, T* __restrict__ out) {
  if (st->done) return;
  const T inv = state_inv<T>(st);
  TV* v = V + (long long)st->j * ld;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; 4 * q < n; q += (long long)gridDim.x * blockDim.x) {
    T a, b, c, d;
    Vec4<T>::load(w + 4 * q, a, b, c, d);
    Vec4Store<TV>::store(v + 4 * q, a * inv, b * inv, c * inv, d * inv);
    T x0, x1, x2, x3;
    load_row<T, TV>(v + 4 * q, x0, x1, x2, x3);
    T r[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      T d0, d1, d2, d3;
      Vec4<T>::load(Dinv + 16 * q + 4 * e, d0, d1, d2, d3);
      r[e] = d0 * x0 + d1 * x1 + d2 * x2 + d3 * x3;
    }
    Vec4Store<T>::store(out + 4 * q, r[0], r[1], r[2], r[3]);
  }
}

// V_j = w / hnext after k_norm_givens advanced j
template <typename T, typename TV>
__global__ void k_normalize_next(long long n, TV* V, long long ld, const T* w, const GState* st) {
  if (st->done) return;
  const T inv = state_inv<T>(st);
  TV* v = V + (long long)st->j * ld;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; 4 * q < n; q += (long long)gridDim.x * blockDim.x) {
    T a, b, c, d;
    Vec4<T>::load(w + 4 * q, a, b, c, d);
    Vec4Store<TV>::store(v + 4 * q, a * inv, b * inv, c * inv, d * inv);
  }
}

// y = R^-1 g for the k x k upper triangle R of the rotated Hessenberg matrix,
// one warp: reciprocals of the diagonal first (in parallel), then column by
// column, y_i = s_i / R_ii and s_r -= R_ri y_i for r < i across the lanes.
template <typename C>
__global__ void k_backsolve(const GState* st, const C* H, int ldh, const C* g, C* y) {
  const int k = st->j;
  const int lane = threadIdx.x;
  __shared__ C s[kMaxM + 1], dinv[kMaxM + 1];
  for (int r = lane; r < k; r += 32) {
    const C d = H[r + (long long)ldh * r];
    dinv[r] = d != C(0) ? C(1) / d : C(0);
    s[r] = g[r];
  }
  __syncwarp();
  for (int i = k - 1; i >= 0; --i) {
    const C yi = s[i] * dinv[i];
    if (lane == 0) y[i] = yi;
    const C* h = H + (long long)ldh * i;
    for (int r = lane; r < i; r += 32) s[r] -= h[r] * yi;
    __syncwarp();
  }
}

// x (+)= Z y; TX = float (the inner solve) works in FP32 throughout, with y
// in FP32, TX = double in FP64.
template <typename T, typename TX>
__global__ void k_combine(long long n, const T* Z, long long ld, const TX* y, const GState* st, TX* x, int zero_first) {
  const int k = st->j;
  __shared__ TX sy[kMaxM];
  for (int c = threadIdx.x; c < k; c += blockDim.x) sy[c] = y[c];
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    TX s = zero_first ? TX(0) : x[i];
    for (int c = 0; c < k; ++c) s = fma(sy[c], ldv<TX, T>(Z + c * ld + i), s);
    x[i] = s;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_norm2_part(long long n, const T* x, T* part) {
  T a = T(0);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a = fma(x[i], x[i], a);
  __shared__ T sm[32];
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    T s = T(0);
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sm[k];
    part[blockIdx.x] = s;
  }
}

// beta = |r| from partials; V_0 = r / beta; g = [beta, 0, ...]; state reset
template <typename C>
__global__ void k_cycle_fin(int nbx, const C* part, GState* st, C* g, int m, double* out_beta) {
  C v = thread_partial_sum<C>(part, nbx);
  __shared__ C sm[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    C s = C(0);
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sm[k];
    const C beta = sqrt(s);
    st->beta = (double)beta;
    set_inv(st, beta);
    st->j = 0;
    st->reorth = 0;
    st->res = (double)beta;
    st->done = (beta > C(0) && beta == beta) ? 0 : 1;
    g[0] = beta;
    for (int i = 1; i <= m; ++i) g[i] = C(0);
    if (out_beta) *out_beta = (double)beta;
  }
}

template <typename T, typename TR>
__global__ void k_scale_into(long long n, const TR* r, const GState* st, T* v0) {
  const TR inv = state_inv<TR>(st);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    stv<T, TR>(v0 + i, r[i] * inv);
}

// The inner solve works in the dof-scaled space: r^ = S r in, z = S z^ out.
template <typename T>
__global__ void k_col_to_inner(long long n, const double* V, long long ld, const GState* st, const double* sd,
                               T* out) {
  if (st->done) return;
  const double* v = V + (long long)st->j * ld;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (T)(v[i] * sd[i]);
}
template <typename T>
__global__ void k_inner_to_col(long long n, const T* in, const double* sd, double* Z, long long ld,
                               const GState* st) {
  if (st->done) return;
  double* z = Z + (long long)st->j * ld;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    z[i] = (double)in[i] * sd[i];
}
// inner solve runs only when the outer step is live
__global__ void k_gate(const GState* outer, GState* inner) {
  if (outer->done) inner->done = 1;
}

__global__ void k_bj_setup(int N, const int* diag, const double* A, const double* dD, double* Dinv, int* singular) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    double a[4][8];
    const double* blk = A + 16ll * diag[n];
    double scale = 0.0;
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) {
        double v = blk[4 * r + c];
        if (dD) v += dD[16ll * n + 4 * r + c];
        a[r][c] = v;
        a[r][4 + c] = (r == c) ? 1.0 : 0.0;
        scale = fmax(scale, fabs(v));
      }
    bool ok = scale > 0.0;
    for (int col = 0; col < 4 && ok; ++col) {
      int piv = col;
      for (int r = col + 1; r < 4; ++r)
        if (fabs(a[r][col]) > fabs(a[piv][col])) piv = r;
      if (!(fabs(a[piv][col]) > 1e-300 * scale + 0.0) || !(fabs(a[piv][col]) > 0.0)) { ok = false; break; }
      if (piv != col)
        for (int c = 0; c < 8; ++c) { double t = a[col][c]; a[col][c] = a[piv][c]; a[piv][c] = t; }
      double inv = 1.0 / a[col][col];
      for (int c = 0; c < 8; ++c) a[col][c] *= inv;
      for (int r = 0; r < 4; ++r) {
        if (r == col) continue;
        double f = a[r][col];
        if (f != 0.0)
          for (int c = 0; c < 8; ++c) a[r][c] -= f * a[col][c];
      }
    }
    if (!ok) atomicAdd(singular, 1);
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) {
        Dinv[16ll * n + 4 * r + c] = ok ? a[r][4 + c] : (r == c ? 1.0 : 0.0);
      }
  }
}

// Rows that are identity rows of the matrix (Dirichlet rows: the diagonal
// block's row r is e_r and every other block's row r is zero) take their value
// from b before the iteration starts. Block-Jacobi keeps those entries of every
// Krylov vector at zero, so GMRES then works on the interior problem only
// (without this the scale-1 Dirichlet rows of a Newton right-hand side stall
// right-preconditioned GMRES against the stiffness-scaled interior rows).
__global__ void k_lift_identity_rows(int N, const int* brow_ptr, const int* bcol, const int* diag, const double* A,
                                     const double* b, double* x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * N; i += gridDim.x * blockDim.x) {
    const int n = i >> 2, r = i & 3;
    bool ident = true;
    for (int k = brow_ptr[n]; k < brow_ptr[n + 1] && ident; ++k) {
      const double* row = A + 16ll * k + 4 * r;
      for (int c = 0; c < 4; ++c) {
        const double want = (k == diag[n] && c == r) ? 1.0 : 0.0;
        if (row[c] != want) { ident = false; break; }
      }
    }
    if (ident) x[i] = b[i];
  }
}

// dof scales S = diag(|a_ii|^-1/2) (1 for a zero diagonal)
__global__ void k_dof_scale(int N, const int* __restrict__ diag, const double* __restrict__ A, double* sd) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * N; i += gridDim.x * blockDim.x) {
    const double d = fabs(A[16ll * diag[i >> 2] + 5 * (i & 3)]);
    sd[i] = d > 0.0 ? 1.0 / sqrt(d) : 1.0;
  }
}
// A^ = S A S in the inner storage type (binary16 saturated to its finite
// range); thread = (node, row)
template <typename TA>
__device__ __forceinline__ TA to_storage(double v) {
  return (TA)v;
}
template <>
__device__ __forceinline__ __half to_storage<__half>(double v) {
  return __double2half(fmin(fmax(v, -65504.0), 65504.0));
}
template <typename TA>
__global__ void k_to_scaled(int N, const int* __restrict__ brow_ptr, const int* __restrict__ bcol,
                            const double* __restrict__ A, const double* __restrict__ sd, TA* As) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 4 * N; t += gridDim.x * blockDim.x) {
    const int n = t >> 2, r = t & 3;
    const double sr = sd[t];
    for (int k = brow_ptr[n]; k < brow_ptr[n + 1]; ++k) {
      const int m = bcol[k];
      for (int c = 0; c < 4; ++c) As[16ll * k + 4 * r + c] = to_storage<TA>(sr * A[16ll * k + 4 * r + c] * sd[4ll * m + c]);
    }
  }
}
// the preconditioner blocks in the scaled space: D^-1 -> S^-1 D^-1 S^-1 and
// (learned second sweep) B -> S^-1 B S^-1, in the inner arithmetic type
template <typename T>
__global__ void k_inner_blocks(int N, const double* __restrict__ Dinv, const double* __restrict__ Bc,
                               const double* __restrict__ sd, T* Dinv_s, T* Bc_s) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 16 * N; i += gridDim.x * blockDim.x) {
    const int n = i >> 4, r = (i >> 2) & 3, c = i & 3;
    const double s = sd[4ll * n + r] * sd[4ll * n + c];
    Dinv_s[i] = (T)(Dinv[i] / s);
    if (Bc) Bc_s[i] = (T)(Bc[i] / s);
  }
}

int spmv_grid(int N) { return grid_for((long long)N * 4, 256, kSMs * 16); }
int vec_grid(long long n) { return grid_for(n, 256, kSMs * 8); }
// Rows per thread of the orthogonalization kernels. FP64: always the longest
// slab, because the per-block reductions cost FP64 instructions (measured on
// the 530k-dof nested adjoint: 141 us per multidot pass with 2 rows per thread
// against 64 us with 8). FP32: enough blocks for about eight per SM, at least
// two and at most kMaxRows rows per thread.
template <typename T>
int slab_rows(long long n) {
  if (!std::is_same<T, float>::value) return kMaxRows;
  const long long target = 8ll * kSMs * 256;
  int r = 2;
  while (r < kMaxRows && n >= 2ll * r * target) r *= 2;
  return r;
}
int slab_grid(long long n, int rows) { return (int)std::max(1ll, (n + 256ll * rows - 1) / (256ll * rows)); }
// a binary16 basis is read in groups of four rows: 4 rows per thread, or 8
// once 4 would need more than one wave of eight 256-thread blocks per SM
template <typename T, typename TV>
int orth_rows(long long n) {
  if (!std::is_same<TV, __half>::value) return slab_rows<T>(n);
  return n > 1024ll * 8 * kSMs ? 8 : 4;
}

}  // namespace

Krylov::~Krylov() {
  if (h_scal) cudaFreeHost(h_scal);
}

void Krylov::reserve(int n_, int m_, int mi_, int precision, int nnzb) {
  (void)nnzb;
  GOAL_REQUIRE(m_ >= 1 && m_ < kMaxM && mi_ >= 1 && mi_ < kMaxM, GOAL_ERR_ARG, "krylov size must be in [1, 255]");
  if (!h_scal) GOAL_CUDA(cudaMallocHost(&h_scal, 64 * sizeof(double)));
  const size_t nn = (size_t)n_;
  need(V, nn * (m_ + 1));
  need(Z, nn * m_);
  need(w, nn);
  need(r, nn);
  need(H, (size_t)(m_ + 1) * m_);
  need(cs, m_ + 1);
  need(sn, m_ + 1);
  need(g, m_ + 2);
  need(y, m_ + 1);
  need(red, (size_t)(kMaxM + 4) * std::max(kSMs * 8, slab_grid(n_, 1)));
  need(scal, 64);
  need(flag, 8);
  need(dots, kMaxM + 2);
  if (has_inner_solve(precision)) {
    const size_t nb = nn * (mi_ + 1);
    if (precision == PREC_MIXED) need(V16, nb);
    if (precision == PREC_MIXED_F32) need(V32, nb);
    if (precision == PREC_NESTED_F64) {
      need(V64, nb);
      need(w64, nn);
      need(r64, nn);
      need(t64, nn);
    } else {
      need(w32, nn);
      need(r32, nn);
      need(t32, nn);
    }
    need(Hi, (size_t)(mi_ + 1) * mi_);
    need(csi, mi_ + 1);
    need(sni, mi_ + 1);
    need(gi, mi_ + 2);
    need(yi, mi_ + 1);
  }
  n = n_;
  m = m_;
  mi = mi_;
}

int block_jacobi_setup(const BsrView& A, const double* vals, const double* dD, Krylov& K) {
  const int N = A.num_nodes;
  need(K.Dinv, 16ull * N);
  need(K.flag, 8);
  K.two_sweep = false;
  GOAL_CUDA(cudaMemsetAsync(K.flag.ptr, 0, sizeof(int), K.stream));
  k_bj_setup<<<grid_for(N, 128), 128, 0, K.stream>>>(N, A.diag, vals, dD, K.Dinv.ptr, K.flag.ptr);
  GOAL_CHECK_LAUNCH();
  int sing = 0;
  GOAL_CUDA(cudaMemcpyAsync(&sing, K.flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, K.stream));
  GOAL_CUDA(cudaStreamSynchronize(K.stream));
  return sing;
}

void make_inner_copy(const BsrView& A, const double* vals, int precision, Krylov& K) {
  const int N = A.num_nodes;
  need(K.sd, 4ull * N);
  k_dof_scale<<<grid_for(4ll * N, 256), 256, 0, K.stream>>>(N, A.diag, vals, K.sd.ptr);
  GOAL_CHECK_LAUNCH();
  const int g = grid_for(4ll * N, 256);
  switch (precision) {
    case PREC_MIXED:
      need(K.A16, 16ull * A.nnzb);
      k_to_scaled<__half><<<g, 256, 0, K.stream>>>(N, A.brow_ptr, A.bcol, vals, K.sd.ptr, K.A16.ptr);
      break;
    case PREC_MIXED_F32:
      need(K.A32, 16ull * A.nnzb);
      k_to_scaled<float><<<g, 256, 0, K.stream>>>(N, A.brow_ptr, A.bcol, vals, K.sd.ptr, K.A32.ptr);
      break;
    case PREC_NESTED_F64:
      need(K.A64, 16ull * A.nnzb);
      k_to_scaled<double><<<g, 256, 0, K.stream>>>(N, A.brow_ptr, A.bcol, vals, K.sd.ptr, K.A64.ptr);
      break;
    default:
      throw Error(GOAL_ERR_ARG, "make_inner_copy: no inner solve in this precision mode");
  }
  GOAL_CHECK_LAUNCH();
}

void spmv64(const BsrView& A, const double* vals, const double* x, double* y, cudaStream_t s) {
  k_spmv<double, double, false><<<spmv_grid(A.num_nodes), 256, 0, s>>>(A.num_nodes, A.brow_ptr, A.bcol, vals, x, nullptr,
                                                                      y);
  GOAL_CHECK_LAUNCH();
}

namespace {

// Classical Gram-Schmidt of w against V_0..V_j, with a second pass when the
// first one removed more than half of |w|^2 (device-side decision).
template <typename T, typename TV, int R>
void orth_passes(long long n, TV* V, T* w, GState* st, T* H, int ldh, T* dots, T* red, int jmax, int passes,
                 cudaStream_t s) {
  const int nbx = slab_grid(n, R);
  T* part = red;
  T* npart = red + (size_t)(kMaxM + 2) * nbx;
  constexpr bool vec = std::is_same<TV, __half>::value && R >= 4;
  for (int pass = 0; pass < passes; ++pass) {
    if constexpr (vec) k_multidot_v<T, TV, R / 4><<<nbx, 256, 0, s>>>(n, V, n, w, st, part, pass);
    else k_multidot<T, TV, R><<<nbx, 256, 0, s>>>(n, V, n, w, st, part, pass);
    GOAL_CHECK_LAUNCH();
    k_dots_fin<T><<<jmax + 2, 256, 0, s>>>(nbx, part, st, H, ldh, dots, pass);
    GOAL_CHECK_LAUNCH();
    if constexpr (vec) k_update_v<T, TV, R / 4><<<nbx, 256, 0, s>>>(n, V, n, w, dots, st, npart, pass);
    else k_update<T, TV, R><<<nbx, 256, 0, s>>>(n, V, n, w, dots, st, npart, pass);
    GOAL_CHECK_LAUNCH();
    if (passes > 1) {
      k_norm_fin<T><<<1, 256, 0, s>>>(nbx, npart, st, H, ldh, pass);
      GOAL_CHECK_LAUNCH();
    }
  }
}

// One Arnoldi step's orthogonalization (CGS with a conditional second pass),
// normalization and Givens update, on state st.
// bj_D / bj_out (single pass only): also out = Dinv V_{j+1}, the first sweep
// of the next step's preconditioner.
template <typename T, typename TV>
void arnoldi_orth(long long n, TV* V, T* w, GState* st, T* H, int ldh, T* cs, T* sn, T* g, T* dots, T* red, int jmax,
                  double tol_abs, int passes, cudaStream_t s, const T* bj_D = nullptr, T* bj_out = nullptr) {
  switch (orth_rows<T, TV>(n)) {
    case 1: orth_passes<T, TV, 1>(n, V, w, st, H, ldh, dots, red, jmax, passes, s); break;
    case 2: orth_passes<T, TV, 2>(n, V, w, st, H, ldh, dots, red, jmax, passes, s); break;
    case 4: orth_passes<T, TV, 4>(n, V, w, st, H, ldh, dots, red, jmax, passes, s); break;
    default: orth_passes<T, TV, 8>(n, V, w, st, H, ldh, dots, red, jmax, passes, s); break;
  }
  if (passes > 1) {
    k_normalize<T, TV><<<vec_grid(n / 4), 256, 0, s>>>(n, V, n, w, st);
    GOAL_CHECK_LAUNCH();
    k_givens<T><<<1, 128, 0, s>>>(st, H, ldh, cs, sn, g, jmax, tol_abs);
    GOAL_CHECK_LAUNCH();
  } else {
    // one pass: norm and Givens in one block, then V_{j+1} = w / |w|
    const int nbx = slab_grid(n, orth_rows<T, TV>(n));
    k_norm_givens<T><<<1, 256, 0, s>>>(nbx, red + (size_t)(kMaxM + 2) * nbx, st, H, ldh, cs, sn, g, jmax, tol_abs);
    GOAL_CHECK_LAUNCH();
    if (bj_D) k_normalize_next_bj<T, TV><<<vec_grid(n / 4), 256, 0, s>>>(n, V, n, w, st, bj_D, bj_out);
    else k_normalize_next<T, TV><<<vec_grid(n / 4), 256, 0, s>>>(n, V, n, w, st);
    GOAL_CHECK_LAUNCH();
  }
}

double read_norm(long long n, const double* x, Krylov& K) {
  const int nbx = vec_grid(n);
  k_norm2_part<double><<<nbx, 256, 0, K.stream>>>(n, x, K.red.ptr);
  GOAL_CHECK_LAUNCH();
  k_cycle_fin<double><<<1, 256, 0, K.stream>>>(nbx, K.red.ptr, reinterpret_cast<GState*>(K.scal.ptr + 16),
                                               K.scal.ptr + 40, 0, K.scal.ptr + 8);
  GOAL_CHECK_LAUNCH();
  GOAL_CUDA(cudaMemcpyAsync(K.h_scal, K.scal.ptr + 8, sizeof(double), cudaMemcpyDeviceToHost, K.stream));
  GOAL_CUDA(cudaStreamSynchronize(K.stream));
  return K.h_scal[0];
}

}  // namespace

namespace {
// A captured CUDA graph, instantiated once and destroyed with its owner. The
// launch counter counts the captured kernels each time the graph runs.
struct StepGraph {
  cudaGraphExec_t exec = nullptr;
  long long kernels = 0;
  template <class F>
  void capture(cudaStream_t s, F&& issue) {
    cudaGraph_t g = nullptr;
    const long long before = g_launches.load();
    GOAL_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      issue();
    } catch (...) {
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    GOAL_CUDA(cudaStreamEndCapture(s, &g));
    kernels = g_launches.load() - before;
    g_launches.fetch_sub(kernels);
    cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    GOAL_CUDA(e);
  }
  void launch(cudaStream_t s) {
    GOAL_CUDA(cudaGraphLaunch(exec, s));
    g_launches.fetch_add(kernels);
  }
  ~StepGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};
}  // namespace

namespace {

// The inner solve's arrays for one storage / arithmetic combination: matrix
// (TA), basis (TV), work vectors, block-Jacobi blocks and the small Hessenberg
// state in the arithmetic type T (FP32 state lives in the FP64 buffers
// reserved for it).
template <typename T, typename TA, typename TV>
struct Inner {
  const TA* A;
  TV* V;
  T *r, *w, *t;
  const T *Dinv, *Bc;
  T *H, *cs, *sn, *g, *y, *dots, *red;
};

template <typename T>
T* as_t(double* p) {
  return reinterpret_cast<T*>(p);
}

Inner<float, __half, __half> inner_arrays(Krylov& K, __half*) {
  return {K.A16.ptr, K.V16.ptr, K.r32.ptr, K.w32.ptr, K.t32.ptr, K.Dinv32.ptr, K.Bc32.ptr, as_t<float>(K.Hi.ptr),
          as_t<float>(K.csi.ptr), as_t<float>(K.sni.ptr), as_t<float>(K.gi.ptr), as_t<float>(K.yi.ptr),
          as_t<float>(K.dots.ptr), as_t<float>(K.red.ptr)};
}
Inner<float, float, float> inner_arrays(Krylov& K, float*) {
  return {K.A32.ptr, K.V32.ptr, K.r32.ptr, K.w32.ptr, K.t32.ptr, K.Dinv32.ptr, K.Bc32.ptr, as_t<float>(K.Hi.ptr),
          as_t<float>(K.csi.ptr), as_t<float>(K.sni.ptr), as_t<float>(K.gi.ptr), as_t<float>(K.yi.ptr),
          as_t<float>(K.dots.ptr), as_t<float>(K.red.ptr)};
}
Inner<double, double, double> inner_arrays(Krylov& K, double*) {
  return {K.A64.ptr, K.V64.ptr, K.r64.ptr, K.w64.ptr, K.t64.ptr, K.Dinv64s.ptr, K.Bc64s.ptr, K.Hi.ptr, K.csi.ptr,
          K.sni.ptr, K.gi.ptr, K.yi.ptr, K.dots.ptr, K.red.ptr};
}

// The scaled block-Jacobi (and second-sweep) blocks of the inner solve.
void inner_blocks(int N, int precision, Krylov& K) {
  const bool two = K.two_sweep;
  if (precision == PREC_NESTED_F64) {
    need(K.Dinv64s, 16ull * N);
    if (two) need(K.Bc64s, 16ull * N);
    k_inner_blocks<double><<<grid_for(16ll * N, 256), 256, 0, K.stream>>>(N, K.Dinv.ptr, two ? K.Bc.ptr : nullptr,
                                                                          K.sd.ptr, K.Dinv64s.ptr, K.Bc64s.ptr);
  } else {
    need(K.Dinv32, 16ull * N);
    if (two) need(K.Bc32, 16ull * N);
    k_inner_blocks<float><<<grid_for(16ll * N, 256), 256, 0, K.stream>>>(N, K.Dinv.ptr, two ? K.Bc.ptr : nullptr,
                                                                         K.sd.ptr, K.Dinv32.ptr, K.Bc32.ptr);
  }
  GOAL_CHECK_LAUNCH();
}

// The outer step's preconditioner application Z_j = M^-1 V_j: mi inner GMRES
// iterations in the dof-scaled space with the right block-Jacobi (or learned
// two-sweep) preconditioner, Z_j = S M^-1 V_in y with V_in the inner basis
// started from S V_j. Every kernel is gated on the outer state st.
template <typename T, typename TA, typename TV>
void issue_inner(const BsrView& A, long long n, int mi, bool sweep2, GState* st, GState* sti, Krylov& K,
                 const Inner<T, TA, TV>& in) {
  const int N = A.num_nodes;
  const int nbx = vec_grid(n);
  cudaStream_t s = K.stream;
  k_col_to_inner<T><<<nbx, 256, 0, s>>>(n, K.V.ptr, n, st, K.sd.ptr, in.r);
  GOAL_CHECK_LAUNCH();
  k_norm2_part<T><<<nbx, 256, 0, s>>>(n, in.r, in.red);
  GOAL_CHECK_LAUNCH();
  k_cycle_fin<T><<<1, 256, 0, s>>>(nbx, in.red, sti, in.g, mi, nullptr);
  GOAL_CHECK_LAUNCH();
  k_gate<<<1, 1, 0, s>>>(st, sti);
  GOAL_CHECK_LAUNCH();
  k_scale_into<TV, T><<<nbx, 256, 0, s>>>(n, in.r, sti, in.V);
  GOAL_CHECK_LAUNCH();
  // r = D^-1 v_0; later steps get D^-1 v_it from the normalization
  k_bj_colin<T, TV><<<grid_for(n, 256), 256, 0, s>>>(N, in.Dinv, in.V, n, sti, in.r);
  GOAL_CHECK_LAUNCH();
  for (int it = 0; it < mi; ++it) {
    // z = M^-1 v_it (in t with the second sweep, else r); w = A^ z
    T* z = in.r;
    if (sweep2) {
      k_spmv_sweep<T, TA, TV><<<spmv_grid(N), 256, 0, s>>>(N, A.brow_ptr, A.bcol, in.A, in.r, in.Bc, in.V, n, sti,
                                                           in.t);
      GOAL_CHECK_LAUNCH();
      z = in.t;
    }
    k_spmv_col<T, TA><<<spmv_grid(N), 256, 0, s>>>(N, A.brow_ptr, A.bcol, in.A, z, 0, sti, in.w);
    GOAL_CHECK_LAUNCH();
    // orthogonalize, normalize into v_{it+1}, and r = D^-1 v_{it+1}
    arnoldi_orth<T, TV>(n, in.V, in.w, sti, in.H, mi + 1, in.cs, in.sn, in.g, in.dots, in.red, mi, 0.0, kInnerPasses,
                        s, in.Dinv, in.r);
  }
  k_backsolve<T><<<1, 32, 0, s>>>(sti, in.H, mi + 1, in.g, in.y);
  GOAL_CHECK_LAUNCH();
  k_combine<TV, T><<<nbx, 256, 0, s>>>(n, in.V, n, in.y, sti, in.w, 1);
  GOAL_CHECK_LAUNCH();
  k_bj<T><<<grid_for(n, 256), 256, 0, s>>>(N, in.Dinv, in.w, in.r);
  GOAL_CHECK_LAUNCH();
  if (sweep2) {
    k_spmv<T, TA, false><<<spmv_grid(N), 256, 0, s>>>(N, A.brow_ptr, A.bcol, in.A, in.r, nullptr, in.t);
    GOAL_CHECK_LAUNCH();
    k_second_sweep_col<T, T><<<grid_for(n, 256), 256, 0, s>>>(N, in.Bc, in.w, 0, in.t, in.r, 0, nullptr);
    GOAL_CHECK_LAUNCH();
  }
  k_inner_to_col<T><<<nbx, 256, 0, s>>>(n, in.r, K.sd.ptr, K.Z.ptr, n, st);
  GOAL_CHECK_LAUNCH();
}

}  // namespace

SolveStats fgmres(const BsrView& A, const double* vals, const double* b, double* x, const SolveParams& p, Krylov& K) {
  auto t0 = std::chrono::steady_clock::now();
  SolveStats out;
  const int N = A.num_nodes;
  const long long n = 4ll * N;
  const bool mixed = has_inner_solve(p.precision);
  const int m = p.krylov_size;
  const int mi = std::max(1, p.inner_iters);
  K.reserve((int)n, m, mi, p.precision, A.nnzb);
  cudaStream_t s = K.stream;
  GOAL_REQUIRE(K.Dinv.ptr, GOAL_ERR_STATE, "fgmres: block-Jacobi preconditioner not set up");
  if (mixed) {
    const bool have = K.sd.ptr && ((p.precision == PREC_MIXED && K.A16.ptr) ||
                                   (p.precision == PREC_MIXED_F32 && K.A32.ptr) ||
                                   (p.precision == PREC_NESTED_F64 && K.A64.ptr));
    GOAL_REQUIRE(have, GOAL_ERR_STATE, "fgmres: inner matrix copy missing");
    inner_blocks(N, p.precision, K);
  }

  GState* st = reinterpret_cast<GState*>(K.scal.ptr);         // outer state
  GState* sti = reinterpret_cast<GState*>(K.scal.ptr + 24);   // inner state
  double* dots = K.dots.ptr;

  const double bnorm = read_norm(n, b, K);
  const double tol_abs = p.tolerance * (bnorm > 0.0 ? bnorm : 1.0);
  k_lift_identity_rows<<<grid_for(n, 256), 256, 0, s>>>(N, A.brow_ptr, A.bcol, A.diag, vals, b, x);
  GOAL_CHECK_LAUNCH();
  // r = b - A x
  k_spmv<double, double, true><<<spmv_grid(N), 256, 0, s>>>(N, A.brow_ptr, A.bcol, vals, x, b, K.r.ptr);
  GOAL_CHECK_LAUNCH();
  out.spmv64++;
  double beta = read_norm(n, K.r.ptr, K);
  out.rel_res = bnorm > 0 ? beta / bnorm : beta;
  const int nbx = vec_grid(n);
  const bool sweep2 = K.two_sweep;

  // One outer Arnoldi step: Z_j = M^-1 V_j, w = A Z_j, orthogonalization and
  // Givens update. Every kernel is gated on the outer state.
  auto issue_step = [&]() {
    if (!mixed) {
      k_bj_col<double><<<grid_for(n, 256), 256, 0, s>>>(N, K.Dinv.ptr, K.V.ptr, K.Z.ptr, n, st);
      GOAL_CHECK_LAUNCH();
      if (sweep2) {
        k_spmv_col<double, double><<<spmv_grid(N), 256, 0, s>>>(N, A.brow_ptr, A.bcol, vals, K.Z.ptr, n, st, K.w.ptr);
        GOAL_CHECK_LAUNCH();
        k_second_sweep_col<double, double><<<grid_for(n, 256), 256, 0, s>>>(N, K.Bc.ptr, K.V.ptr, n, K.w.ptr, K.Z.ptr, n, st);
        GOAL_CHECK_LAUNCH();
      }
    } else if (p.precision == PREC_MIXED) {
      issue_inner(A, n, mi, sweep2, st, sti, K, inner_arrays(K, (__half*)nullptr));
    } else if (p.precision == PREC_MIXED_F32) {
      issue_inner(A, n, mi, sweep2, st, sti, K, inner_arrays(K, (float*)nullptr));
    } else {
      issue_inner(A, n, mi, sweep2, st, sti, K, inner_arrays(K, (double*)nullptr));
    }
    k_spmv_col<double, double><<<spmv_grid(N), 256, 0, s>>>(N, A.brow_ptr, A.bcol, vals, K.Z.ptr, n, st, K.w.ptr);
    GOAL_CHECK_LAUNCH();
    arnoldi_orth<double, double>(n, K.V.ptr, K.w.ptr, st, K.H.ptr, m + 1, K.cs.ptr, K.sn.ptr, K.g.ptr, dots, K.red.ptr, m,
                         tol_abs, kOuterPasses, s);
  };
  // one Arnoldi step as a CUDA graph, captured once per solve; its kernels are
  // gated on the device state, so steps launched past the end of a cycle are
  // no-ops, and the host reads the state every `batch` steps
  StepGraph step_graph;
  const int batch = mixed ? 1 : 4;

  while (beta > tol_abs && out.iters < p.max_iters) {
    // start a cycle: V_0 = r / beta
    k_norm2_part<double><<<nbx, 256, 0, s>>>(n, K.r.ptr, K.red.ptr);
    GOAL_CHECK_LAUNCH();
    k_cycle_fin<double><<<1, 256, 0, s>>>(nbx, K.red.ptr, st, K.g.ptr, m, nullptr);
    GOAL_CHECK_LAUNCH();
    k_scale_into<double, double><<<nbx, 256, 0, s>>>(n, K.r.ptr, st, K.V.ptr);
    GOAL_CHECK_LAUNCH();
    const int steps = std::min(m, p.max_iters - out.iters);
    if (!step_graph.exec) step_graph.capture(s, issue_step);
    int done_steps = 0;
    for (int step = 0; step < steps;) {
      const int k = std::min(batch, steps - step);
      for (int q = 0; q < k; ++q) step_graph.launch(s);
      step += k;
      GOAL_CUDA(cudaMemcpyAsync(K.h_scal, K.scal.ptr, sizeof(GState), cudaMemcpyDeviceToHost, s));
      GOAL_CUDA(cudaStreamSynchronize(s));
      const GState* hs = reinterpret_cast<const GState*>(K.h_scal);
      done_steps = hs->j;
      if (hs->done) break;
    }
    const long long extra = sweep2 ? 1 : 0;
    if (mixed) {
      out.inner_iters += (long long)mi * done_steps;
      out.spmv32 += (long long)done_steps * (mi * (1 + extra) + extra);
      out.spmv64 += done_steps;
    } else {
      out.spmv64 += (long long)done_steps * (1 + extra);
    }
    out.iters += done_steps;
    k_backsolve<double><<<1, 32, 0, s>>>(st, K.H.ptr, m + 1, K.g.ptr, K.y.ptr);
    GOAL_CHECK_LAUNCH();
    k_combine<double, double><<<nbx, 256, 0, s>>>(n, K.Z.ptr, n, K.y.ptr, st, x, 0);
    GOAL_CHECK_LAUNCH();
    k_spmv<double, double, true><<<spmv_grid(N), 256, 0, s>>>(N, A.brow_ptr, A.bcol, vals, x, b, K.r.ptr);
    GOAL_CHECK_LAUNCH();
    out.spmv64++;
    double nb = read_norm(n, K.r.ptr, K);
    if (!(nb == nb)) throw Error(GOAL_ERR_SOLVER, "fgmres: non-finite residual");
    if (done_steps == 0) { beta = nb; break; }  // breakdown without progress
    beta = nb;
  }
  out.rel_res = bnorm > 0 ? beta / bnorm : beta;
  out.converged = beta <= tol_abs ? 1 : 0;
  out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return out;
}

}  // namespace goal
