// Forward, backward and Adam kernels of the learned block-Jacobi correction
// (see mpnn.cuh). One warp per node; lane j owns hidden unit j. Layer weights
// are staged in shared memory (rows padded to avoid bank conflicts) from the
// bfloat16 copy; all arithmetic is float32. Weight gradients are summed per
// warp, then over warps in a fixed order, so training is deterministic.
#include <cuda_bf16.h>

#include <cmath>
#include <random>

#include "mpnn.cuh"

namespace goal {

namespace {

constexpr int kWarpsPerBlock = 8;
constexpr int kGridBlocks = kSMs;  // persistent grid for kernels with per-warp partials
constexpr int kTotalWarps = kGridBlocks * kWarpsPerBlock;

__device__ __forceinline__ float bf(unsigned short b) {
  return __uint_as_float(((unsigned)b) << 16);
}

__device__ __forceinline__ unsigned hash32(unsigned x) {
  x ^= x >> 16; x *= 0x7feb352du;
  x ^= x >> 15; x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__global__ void k_to_bf16(int n, const float* p, unsigned short* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    __nv_bfloat16 b = __float2bfloat16_rn(p[i]);
    out[i] = *reinterpret_cast<unsigned short*>(&b);
  }
}

__device__ __forceinline__ double dof_scale(double a) {
  const double d = fabs(a);
  return d > 0.0 ? 1.0 / sqrt(d) : 1.0;
}

// node features, dof scales, Dirichlet row masks and D^-1; x[16] holds
// log10 max|D_n| until the mean is removed
__global__ void k_features(int N, const int* brow_ptr, const int* bcol, const int* diag, const double* A, float* x,
                           double* s, double* sd, double* Dinv, int* deg, int* dmask) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    const double* D = A + 16ll * diag[n];
    double sn[4];
    for (int r = 0; r < 4; ++r) sn[r] = dof_scale(D[5 * r]);
    double smax = 0.0, dn = 0.0;
    for (int q = 0; q < 16; ++q) {
      smax = fmax(smax, fabs(D[q]));
      const double dh = sn[q >> 2] * D[q] * sn[q & 3];
      x[20ll * n + q] = (float)dh;
      dn += dh * dh;
    }
    const double sc = smax > 0.0 ? smax : 1.0;
    s[n] = sc;
    for (int r = 0; r < 4; ++r) sd[4ll * n + r] = sn[r];
    double offn = 0.0;
    double offr[4] = {0, 0, 0, 0};
    int nd = 0;
    for (int k = brow_ptr[n]; k < brow_ptr[n + 1]; ++k) {
      const int m = bcol[k];
      if (m == n) continue;
      ++nd;
      const double* Dm = A + 16ll * diag[m];
      double sm[4];
      for (int c = 0; c < 4; ++c) sm[c] = dof_scale(Dm[5 * c]);
      double f = 0.0;
      for (int q = 0; q < 16; ++q) {
        const double a = A[16ll * k + q];
        const double ah = sn[q >> 2] * a * sm[q & 3];
        f += ah * ah;
        offr[q >> 2] += fabs(a);
      }
      offn += sqrt(f);
    }
    deg[n] = nd > 0 ? nd : 1;
    dn = sqrt(dn);
    x[20ll * n + 16] = (float)log10(sc);
    x[20ll * n + 17] = (float)(offn / (dn > 0.0 ? dn : 1.0));
    int mask = 0;
    for (int r = 0; r < 4; ++r) {
      bool unit = true;
      for (int c = 0; c < 4; ++c) unit = unit && (D[4 * r + c] == (r == c ? 1.0 : 0.0));
      if (unit && offr[r] == 0.0) mask |= 1 << r;
    }
    dmask[n] = mask;
    x[20ll * n + 18] = (float)(__popc(mask) * 0.25);
    x[20ll * n + 19] = (float)((brow_ptr[n + 1] - brow_ptr[n] - 1) / 16.0);
    // D^-1 (Gauss-Jordan with partial pivoting; identity for a singular block)
    double a[4][8];
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) { a[r][c] = D[4 * r + c]; a[r][4 + c] = (r == c) ? 1.0 : 0.0; }
    bool ok = smax > 0.0;
    for (int col = 0; col < 4 && ok; ++col) {
      int piv = col;
      for (int r = col + 1; r < 4; ++r)
        if (fabs(a[r][col]) > fabs(a[piv][col])) piv = r;
      if (!(fabs(a[piv][col]) > 0.0)) { ok = false; break; }
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
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) Dinv[16ll * n + 4 * r + c] = ok ? a[r][4 + c] : (r == c ? 1.0 : 0.0);
  }
}

__global__ void k_sum_log(int N, const float* x, double* part) {
  KSum acc;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) acc.add((double)x[20ll * n + 16]);
  acc = block_reduce(acc);
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = acc.s; part[2 * blockIdx.x + 1] = acc.c; }
}
__global__ void k_sub_log_mean(int N, int nb, const double* part, float* x) {
  __shared__ double mean;
  KSum acc;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    KSum t;
    t.s = part[2 * i];
    t.c = part[2 * i + 1];
    acc.add(t);
  }
  acc = block_reduce(acc);
  if (threadIdx.x == 0) mean = acc.value() / N;
  __syncthreads();
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x)
    x[20ll * n + 16] = (float)((double)x[20ll * n + 16] - mean);
}

// index of block (m, n) for every block (n, m)
__global__ void k_tmap(int N, const int* brow_ptr, const int* bcol, int* tmap) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x)
    for (int k = brow_ptr[n]; k < brow_ptr[n + 1]; ++k) {
      int m = bcol[k];
      int lo = brow_ptr[m], hi = brow_ptr[m + 1];
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (bcol[mid] < n) lo = mid + 1;
        else hi = mid;
      }
      tmap[k] = lo;
    }
}

__global__ void __launch_bounds__(256) k_encoder(int N, const unsigned short* w, const float* x, float* h) {
  __shared__ float sW[kMH][kMF + 1];
  __shared__ float sb[kMH];
  for (int i = threadIdx.x; i < kMH * kMF; i += blockDim.x) sW[i / kMF][i % kMF] = bf(w[MpnnLayout::W0 + i]);
  for (int i = threadIdx.x; i < kMH; i += blockDim.x) sb[i] = bf(w[MpnnLayout::b0 + i]);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int n = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; n < N; n += (gridDim.x * blockDim.x) >> 5) {
    float z = sb[lane];
    for (int q = 0; q < kMF; ++q) z += sW[lane][q] * x[20ll * n + q];
    h[32ll * n + lane] = fmaxf(z, 0.0f);
  }
}

struct LayerSmem {
  float We[kMH][kME + kMH + 1];
  float be[kMH];
  float Wu[kMH][2 * kMH + 1];
  float bu[kMH];
  float in[kWarpsPerBlock][kME + kMH];
  float cat[kWarpsPerBlock][2 * kMH];
  float d[kWarpsPerBlock][kMH];
};

__device__ void load_layer(LayerSmem& sm, const unsigned short* wl) {
  for (int i = threadIdx.x; i < kMH * (kME + kMH); i += blockDim.x)
    sm.We[i / (kME + kMH)][i % (kME + kMH)] = bf(wl[MpnnLayout::We + i]);
  for (int i = threadIdx.x; i < kMH * 2 * kMH; i += blockDim.x) sm.Wu[i / (2 * kMH)][i % (2 * kMH)] = bf(wl[MpnnLayout::Wu + i]);
  for (int i = threadIdx.x; i < kMH; i += blockDim.x) {
    sm.be[i] = bf(wl[MpnnLayout::be + i]);
    sm.bu[i] = bf(wl[MpnnLayout::bu + i]);
  }
  __syncthreads();
}

// stage [e_nm; h_m] of edge k = (n, m) in sm.in[w]; e_nm = S_n A_nm S_m
__device__ __forceinline__ void stage_edge(LayerSmem& sm, int w, int lane, const double* A, long long k,
                                           const double* sd, int n, const float* h, int m) {
  if (lane < kME) sm.in[w][lane] = (float)(sd[4ll * n + (lane >> 2)] * A[16ll * k + lane] * sd[4ll * m + (lane & 3)]);
  sm.in[w][kME + lane] = h[32ll * m + lane];
  __syncwarp();
}

// ---------------------------------------------------------------- tensor cores
// mma.sync m16n8k16, bfloat16 operands, FP32 accumulation. Fragment layout
// (PTX ISA, m16n8k16 .bf16): g = lane / 4, q = lane % 4;
//   A (16 x 16, row major): a0 = A[g][2q..2q+1], a1 = A[g+8][2q..], a2 = A[g][2q+8..], a3 = A[g+8][2q+8..]
//   B (16 x 8, column major): b0 = B[2q..2q+1][g], b1 = B[2q+8..2q+9][g]
//   C (16 x 8): c0, c1 = C[g][2q..2q+1], c2, c3 = C[g+8][2q..2q+1]
// (each register holds two bfloat16, the lower column / row in the low half).
__device__ __forceinline__ void mma_bf16(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
// two FP32 values as a bfloat16 pair split in two terms, x = hi + lo with
// hi = rn(x), lo = rn(x - hi): the products with bfloat16 weights then carry
// about 16 mantissa bits of the activations instead of 8
__device__ __forceinline__ void split_bf16(float x0, float x1, unsigned& hi, unsigned& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
  hi = *reinterpret_cast<const unsigned*>(&h);
  lo = *reinterpret_cast<const unsigned*>(&l);
}

constexpr int kIn = kME + kMH;       // 48 inputs of an edge message
constexpr int kInStride = kIn + 4;   // staged row stride (floats)

// One message-passing layer, forward: per node n (one warp),
//   t_nm = We [e_nm; h_m] + be for its edges (m != n), agg = mean_m relu(t_nm),
//   h_n' = h_n + relu(Wu [h_n; agg] + bu).
// The edge messages are a (edges x 48) x (48 x 32) product: tiles of 16 edge
// rows staged in shared memory go through the tensor cores (mma.sync, the
// bfloat16 weights exact, the FP32 activations as two bfloat16 terms); the
// node update (64 x 32 per node) stays on the CUDA cores. tbuf, ubuf and aggbuf
// (training) keep t, the update's pre-activation and agg.
__global__ void __launch_bounds__(256) k_layer_fwd(int N, const int* brow_ptr, const int* bcol, const double* A,
                                                    const double* sd, const int* deg, const unsigned short* wl,
                                                    const float* h_in, float* h_out, float* tbuf, float* ubuf,
                                                    float* aggbuf) {
  __shared__ LayerSmem sm;
  __shared__ float sIn[kWarpsPerBlock][16][kInStride];
  load_layer(sm, wl);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane >> 2, q = lane & 3;
  // B = We^T (48 x 32) fragments, kept in registers: k-step ks, n-tile nt
  unsigned bfr[3][4][2];
#pragma unroll
  for (int ks = 0; ks < 3; ++ks)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const unsigned short* row = wl + MpnnLayout::We + (nt * 8 + g) * kIn + ks * 16 + 2 * q;
      bfr[ks][nt][0] = (unsigned)row[0] | ((unsigned)row[1] << 16);
      bfr[ks][nt][1] = (unsigned)row[8] | ((unsigned)row[9] << 16);
    }
  float bias[4][2];
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
    bias[nt][0] = sm.be[nt * 8 + 2 * q];
    bias[nt][1] = sm.be[nt * 8 + 2 * q + 1];
  }
  float (*tile)[kInStride] = sIn[w];
  for (int n = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; n < N; n += (gridDim.x * blockDim.x) >> 5) {
    const int k0 = brow_ptr[n], k1 = brow_ptr[n + 1];
    float aggp[4][2] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    for (int kk = k0; kk < k1; kk += 16) {
      // stage rows [e_nm (16); h_m (32)] of blocks kk .. kk+15 (zeros past the row's end)
      for (int idx = lane; idx < 16 * kIn; idx += 32) {
        const int r = idx / kIn, c = idx - r * kIn, k = kk + r;
        float v = 0.0f;
        if (k < k1) {
          const int m = bcol[k];
          v = c < kME ? (float)(sd[4ll * n + (c >> 2)] * A[16ll * k + c] * sd[4ll * m + (c & 3)])
                      : h_in[32ll * m + (c - kME)];
        }
        tile[r][c] = v;
      }
      __syncwarp();
      float acc[4][4];
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        acc[nt][0] = acc[nt][2] = bias[nt][0];
        acc[nt][1] = acc[nt][3] = bias[nt][1];
      }
#pragma unroll
      for (int ks = 0; ks < 3; ++ks) {
        const int c0 = ks * 16 + 2 * q;
        unsigned ahi[4], alo[4];
        split_bf16(tile[g][c0], tile[g][c0 + 1], ahi[0], alo[0]);
        split_bf16(tile[g + 8][c0], tile[g + 8][c0 + 1], ahi[1], alo[1]);
        split_bf16(tile[g][c0 + 8], tile[g][c0 + 9], ahi[2], alo[2]);
        split_bf16(tile[g + 8][c0 + 8], tile[g + 8][c0 + 9], ahi[3], alo[3]);
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
          mma_bf16(acc[nt], ahi, bfr[ks][nt][0], bfr[ks][nt][1]);
          mma_bf16(acc[nt], alo, bfr[ks][nt][0], bfr[ks][nt][1]);
        }
      }
      // rows g and g + 8 of the tile: edges kk + g, kk + g + 8 (the diagonal block excluded)
      const int ka = kk + g, kb = kk + g + 8;
      const bool va = ka < k1 && bcol[ka] != n, vb = kb < k1 && bcol[kb] != n;
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const int col = nt * 8 + 2 * q;
        if (va) {
          aggp[nt][0] += fmaxf(acc[nt][0], 0.0f);
          aggp[nt][1] += fmaxf(acc[nt][1], 0.0f);
          if (tbuf) *reinterpret_cast<float2*>(tbuf + 32ll * ka + col) = make_float2(acc[nt][0], acc[nt][1]);
        }
        if (vb) {
          aggp[nt][0] += fmaxf(acc[nt][2], 0.0f);
          aggp[nt][1] += fmaxf(acc[nt][3], 0.0f);
          if (tbuf) *reinterpret_cast<float2*>(tbuf + 32ll * kb + col) = make_float2(acc[nt][2], acc[nt][3]);
        }
      }
      __syncwarp();
    }
    // sum over the eight row groups (lanes with the same q), in a fixed order
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        float v = aggp[nt][e];
        v += __shfl_xor_sync(0xffffffffu, v, 4);
        v += __shfl_xor_sync(0xffffffffu, v, 8);
        v += __shfl_xor_sync(0xffffffffu, v, 16);
        aggp[nt][e] = v;
      }
    const float invdeg = 1.0f / (float)deg[n];
    if (g == 0) {
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        sm.cat[w][kMH + nt * 8 + 2 * q] = aggp[nt][0] * invdeg;
        sm.cat[w][kMH + nt * 8 + 2 * q + 1] = aggp[nt][1] * invdeg;
      }
    }
    const float hn = h_in[32ll * n + lane];
    sm.cat[w][lane] = hn;
    __syncwarp();
    const float agg = sm.cat[w][kMH + lane];
    float u = sm.bu[lane];
    for (int qq = 0; qq < 2 * kMH; ++qq) u += sm.Wu[lane][qq] * sm.cat[w][qq];
    if (ubuf) { ubuf[32ll * n + lane] = u; aggbuf[32ll * n + lane] = agg; }
    h_out[32ll * n + lane] = hn + fmaxf(u, 0.0f);
    __syncwarp();
  }
}

__global__ void __launch_bounds__(256) k_decoder(int N, const unsigned short* w, const float* h, float* C) {
  __shared__ float sW[16][kMH + 1];
  __shared__ float sb[16];
  for (int i = threadIdx.x; i < 16 * kMH; i += blockDim.x) sW[i / kMH][i % kMH] = bf(w[MpnnLayout::Wd + i]);
  for (int i = threadIdx.x; i < 16; i += blockDim.x) sb[i] = bf(w[MpnnLayout::bd + i]);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int n = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; n < N; n += (gridDim.x * blockDim.x) >> 5) {
    if (lane < 16) {
      float c = sb[lane];
      for (int q = 0; q < kMH; ++q) c += sW[lane][q] * h[32ll * n + q];
      C[16ll * n + lane] = c;
    }
  }
}

// ---------------------------------------------------------------- loss
__global__ void k_gauss(long long n, unsigned seed, double* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned a = hash32((unsigned)i * 2u + 1u + seed * 0x9e3779b9u);
    unsigned b = hash32(a ^ (unsigned)(i >> 31) ^ 0x85ebca6bu);
    double u1 = (a + 1.0) / 4294967297.0, u2 = b / 4294967296.0;
    out[i] = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
  }
}

__global__ void k_bsr_mv(int N, const int* brow_ptr, const int* bcol, const double* A, const double* x, double* y,
                         const double* sub) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * N; i += gridDim.x * blockDim.x) {
    int n = i >> 2, r = i & 3;
    double acc = 0.0;
    for (int k = brow_ptr[n]; k < brow_ptr[n + 1]; ++k) {
      const double* a = A + 16ll * k + 4 * r;
      const double* xx = x + 4ll * bcol[k];
      acc += a[0] * xx[0] + a[1] * xx[1] + a[2] * xx[2] + a[3] * xx[3];
    }
    y[i] = sub ? sub[i] - acc : acc;
  }
}
// y = A^T x using the transposed-block map
__global__ void k_bsr_mv_t(int N, const int* brow_ptr, const int* bcol, const int* tmap, const double* A,
                           const double* x, double* y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * N; i += gridDim.x * blockDim.x) {
    int n = i >> 2, c = i & 3;
    double acc = 0.0;
    for (int k = brow_ptr[n]; k < brow_ptr[n + 1]; ++k) {
      const double* a = A + 16ll * tmap[k];  // block (m, n); entry (r, c) multiplies x_m[r]
      const double* xx = x + 4ll * bcol[k];
      acc += a[c] * xx[0] + a[4 + c] * xx[1] + a[8 + c] * xx[2] + a[12 + c] * xx[3];
    }
    y[i] = acc;
  }
}
// y = D^-1 x
__global__ void k_bjn(int N, const double* Dinv, const double* x, double* y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * N; i += gridDim.x * blockDim.x) {
    int n = i >> 2, r = i & 3;
    double acc = 0.0;
    for (int c = 0; c < 4; ++c) acc += Dinv[16ll * n + 4 * r + c] * x[4ll * n + c];
    y[i] = acc;
  }
}
__device__ __forceinline__ bool kept(const int* dmask, int n, int r) { return ((dmask[n] >> r) & 1) == 0; }
// probe w (scaled residual space) -> residual-space q = S^-1 w on the non-Dirichlet rows
__global__ void k_probe(int N, const double* sd, const int* dmask, double* v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * N; i += gridDim.x * blockDim.x)
    v[i] = kept(dmask, i >> 2, i & 3) ? v[i] / sd[i] : 0.0;
}
// chat = (D^-1 t) / S ; y = z + S W chat   (W = C with Dirichlet rows/columns zeroed)
__global__ void k_second_sweep(int N, const double* Dinv, const double* sd, const int* dmask, const float* C,
                               const double* t, const double* z, double* chat, double* y) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    double ch[4];
    for (int r = 0; r < 4; ++r) {
      double acc = 0.0;
      for (int c = 0; c < 4; ++c) acc += Dinv[16ll * n + 4 * r + c] * t[4ll * n + c];
      ch[r] = acc / sd[4ll * n + r];
      chat[4ll * n + r] = ch[r];
    }
    for (int r = 0; r < 4; ++r) {
      double acc = 0.0;
      if (kept(dmask, n, r))
        for (int c = 0; c < 4; ++c)
          if (kept(dmask, n, c)) acc += (double)C[16ll * n + 4 * r + c] * ch[c];
      y[4ll * n + r] = z[4ll * n + r] + sd[4ll * n + r] * acc;
    }
  }
}
__global__ void k_scale_by(long long n, const double* sd, double* x) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] *= sd[i];
}
// sum of (w_i a_i)^2
__global__ void k_wnorm_part(long long n, const double* a, const double* w, double* part) {
  KSum acc;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double t = w[i] * a[i];
    acc.add(t * t);
  }
  acc = block_reduce(acc);
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = acc.s; part[2 * blockIdx.x + 1] = acc.c; }
}
__global__ void k_fin2(const double* part, int nb, double* out) {
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
// dW_n += (-2 / |S v|^2) (S g)_n chat_n^T on the kept rows/columns; g = A^T (S e)
__global__ void k_dW(int N, const double* g, const double* sd, const double* chat, const int* dmask,
                     const double* nv, double* dW) {
  const double coef = -2.0 / nv[0];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 16 * N; i += gridDim.x * blockDim.x) {
    int n = i >> 4, r = (i >> 2) & 3, c = i & 3;
    if (kept(dmask, n, r) && kept(dmask, n, c)) dW[i] += coef * sd[4ll * n + r] * g[4ll * n + r] * chat[4ll * n + c];
  }
}
// loss += |S e|^2 / |S v|^2 of one probe (kept on the device; read once per step)
__global__ void k_loss_acc(const double* scal, double* loss) {
  if (threadIdx.x == 0 && blockIdx.x == 0) loss[0] += scal[1] / scal[0];
}
__global__ void k_dC(int N, const double* dW, float* dC) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 16 * N; i += gridDim.x * blockDim.x) dC[i] = (float)dW[i];
}

// ---------------------------------------------------------------- backward
// decoder: dh = Wd^T dC ; partial dWd, dbd per warp
__global__ void __launch_bounds__(256) k_decoder_bwd(int N, const unsigned short* w, const float* h, const float* dC,
                                                      float* dh, float* part, int P) {
  __shared__ float sW[16][kMH + 1];
  for (int i = threadIdx.x; i < 16 * kMH; i += blockDim.x) sW[i / kMH][i % kMH] = bf(w[MpnnLayout::Wd + i]);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  float gW[16];
  for (int j = 0; j < 16; ++j) gW[j] = 0.0f;
  float gb = 0.0f;
  for (int n = gw; n < N; n += (gridDim.x * blockDim.x) >> 5) {
    const float hk = h[32ll * n + lane];
    float acc = 0.0f;
    for (int j = 0; j < 16; ++j) {
      const float dc = dC[16ll * n + j];
      acc += sW[j][lane] * dc;
      gW[j] += dc * hk;
    }
    if (lane < 16) gb += dC[16ll * n + lane];
    dh[32ll * n + lane] = acc;
  }
  float* p = part + (size_t)gw * P;
  for (int j = 0; j < 16; ++j) p[MpnnLayout::Wd + j * kMH + lane] = gW[j];
  if (lane < 16) p[MpnnLayout::bd + lane] = gb;
}

// node part of a layer's backward: du, dWu, dbu, dh_acc = dh + (Wu^T du)[:32], dagg = (Wu^T du)[32:]/deg
__global__ void __launch_bounds__(256) k_layer_bwd_node(int N, const unsigned short* wl, int woff, const float* h_in,
                                                         const float* ubuf, const float* aggbuf, const int* deg,
                                                         const float* dh, float* dh_acc, float* dagg, float* part,
                                                         int P) {
  __shared__ LayerSmem sm;
  load_layer(sm, wl);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  float gW[2 * kMH];
  for (int q = 0; q < 2 * kMH; ++q) gW[q] = 0.0f;
  float gb = 0.0f;
  for (int n = gw; n < N; n += (gridDim.x * blockDim.x) >> 5) {
    const float u = ubuf[32ll * n + lane];
    const float du = (u > 0.0f) ? dh[32ll * n + lane] : 0.0f;
    sm.cat[w][lane] = h_in[32ll * n + lane];
    sm.cat[w][kMH + lane] = aggbuf[32ll * n + lane];
    sm.d[w][lane] = du;
    __syncwarp();
    for (int q = 0; q < 2 * kMH; ++q) gW[q] += du * sm.cat[w][q];
    gb += du;
    float a0 = 0.0f, a1 = 0.0f;
    for (int j = 0; j < kMH; ++j) {
      a0 += sm.Wu[j][lane] * sm.d[w][j];
      a1 += sm.Wu[j][kMH + lane] * sm.d[w][j];
    }
    dh_acc[32ll * n + lane] = dh[32ll * n + lane] + a0;
    dagg[32ll * n + lane] = a1 / (float)deg[n];
    __syncwarp();
  }
  float* p = part + (size_t)gw * P + woff;
  for (int q = 0; q < 2 * kMH; ++q) p[MpnnLayout::Wu + lane * 2 * kMH + q] = gW[q];
  p[MpnnLayout::bu + lane] = gb;
}

// edge part: dt, dWe, dbe and g_k = (We^T dt)[16:] for every edge k = (n, m).
// Per tile of 16 edge rows of a node (one warp), on the tensor cores:
//   dWe (32 x 48) += dT^T (32 x 16) IN (16 x 48)   (both FP32 operands as two
//                    bfloat16 terms; hi*hi + hi*lo + lo*hi, the lo*lo term
//                    below FP32 rounding left out)
//   G (16 x 32)    = dT (16 x 32) We_h (32 x 32)   (We_h = the h columns of We,
//                    bfloat16 and exact; dT as two terms)
// with dT[r][j] = da_n[j] where t_kj > 0 (0 on the diagonal block and past the
// row's end). The dWe accumulators stay in registers for all of the warp's
// nodes; dbe sums dT's columns on the CUDA cores.
__global__ void __launch_bounds__(256) k_layer_bwd_edge(int N, const int* brow_ptr, const int* bcol, const double* A,
                                                         const double* sd, const unsigned short* wl, int woff,
                                                         const float* h_in, const float* tbuf, const float* dagg,
                                                         float* gbuf, float* part, int P) {
  __shared__ float sIn[kWarpsPerBlock][16][kInStride];
  __shared__ float sdT[kWarpsPerBlock][16][kMH + 4];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane >> 2, q = lane & 3;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  // B = We_h (32 x 32), B[j][c] = We[j][16 + c]: k-step ks (j), n-tile nt (c)
  unsigned bh[2][4][2];
#pragma unroll
  for (int ks = 0; ks < 2; ++ks)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const unsigned short* col = wl + MpnnLayout::We + kME + nt * 8 + g;
      const int j0 = ks * 16 + 2 * q;
      bh[ks][nt][0] = (unsigned)col[j0 * kIn] | ((unsigned)col[(j0 + 1) * kIn] << 16);
      bh[ks][nt][1] = (unsigned)col[(j0 + 8) * kIn] | ((unsigned)col[(j0 + 9) * kIn] << 16);
    }
  float gacc[2][6][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 6; ++nt) gacc[mt][nt][0] = gacc[mt][nt][1] = gacc[mt][nt][2] = gacc[mt][nt][3] = 0.0f;
  float gb = 0.0f;
  float (*tile)[kInStride] = sIn[w];
  float (*dT)[kMH + 4] = sdT[w];
  for (int n = gw; n < N; n += (gridDim.x * blockDim.x) >> 5) {
    const float da = dagg[32ll * n + lane];
    const int k0 = brow_ptr[n], k1 = brow_ptr[n + 1];
    for (int kk = k0; kk < k1; kk += 16) {
      for (int idx = lane; idx < 16 * kIn; idx += 32) {
        const int r = idx / kIn, c = idx - r * kIn, k = kk + r;
        float v = 0.0f;
        if (k < k1) {
          const int m = bcol[k];
          v = c < kME ? (float)(sd[4ll * n + (c >> 2)] * A[16ll * k + c] * sd[4ll * m + (c & 3)])
                      : h_in[32ll * m + (c - kME)];
        }
        tile[r][c] = v;
      }
      // lane = output unit j: column j of dT
      float colsum = 0.0f;
#pragma unroll 4
      for (int r = 0; r < 16; ++r) {
        const int k = kk + r;
        const bool live = k < k1 && bcol[k] != n;
        const float dt = (live && tbuf[32ll * k + lane] > 0.0f) ? da : 0.0f;
        dT[r][lane] = dt;
        colsum += dt;
      }
      gb += colsum;
      __syncwarp();
      // dWe += dT^T IN: A = dT^T (rows j: m-tile mt; columns: the 16 edges), B = IN (edges x 48)
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        unsigned ahi[4], alo[4];
        const int j = mt * 16 + g;
        split_bf16(dT[2 * q][j], dT[2 * q + 1][j], ahi[0], alo[0]);
        split_bf16(dT[2 * q][j + 8], dT[2 * q + 1][j + 8], ahi[1], alo[1]);
        split_bf16(dT[2 * q + 8][j], dT[2 * q + 9][j], ahi[2], alo[2]);
        split_bf16(dT[2 * q + 8][j + 8], dT[2 * q + 9][j + 8], ahi[3], alo[3]);
#pragma unroll
        for (int nt = 0; nt < 6; ++nt) {
          const int c = nt * 8 + g;
          unsigned bhi[2], blo[2];
          split_bf16(tile[2 * q][c], tile[2 * q + 1][c], bhi[0], blo[0]);
          split_bf16(tile[2 * q + 8][c], tile[2 * q + 9][c], bhi[1], blo[1]);
          mma_bf16(gacc[mt][nt], ahi, bhi[0], bhi[1]);
          mma_bf16(gacc[mt][nt], ahi, blo[0], blo[1]);
          mma_bf16(gacc[mt][nt], alo, bhi[0], bhi[1]);
        }
      }
      // G = dT We_h: A = dT (rows: edges; columns j), two k-steps of 16 j
      float gk[4][4];
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) gk[nt][0] = gk[nt][1] = gk[nt][2] = gk[nt][3] = 0.0f;
#pragma unroll
      for (int ks = 0; ks < 2; ++ks) {
        const int c0 = ks * 16 + 2 * q;
        unsigned ahi[4], alo[4];
        split_bf16(dT[g][c0], dT[g][c0 + 1], ahi[0], alo[0]);
        split_bf16(dT[g + 8][c0], dT[g + 8][c0 + 1], ahi[1], alo[1]);
        split_bf16(dT[g][c0 + 8], dT[g][c0 + 9], ahi[2], alo[2]);
        split_bf16(dT[g + 8][c0 + 8], dT[g + 8][c0 + 9], ahi[3], alo[3]);
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
          mma_bf16(gk[nt], ahi, bh[ks][nt][0], bh[ks][nt][1]);
          mma_bf16(gk[nt], alo, bh[ks][nt][0], bh[ks][nt][1]);
        }
      }
      const int ka = kk + g, kb = kk + g + 8;
      const bool va = ka < k1 && bcol[ka] != n, vb = kb < k1 && bcol[kb] != n;
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const int col = nt * 8 + 2 * q;
        if (va) *reinterpret_cast<float2*>(gbuf + 32ll * ka + col) = make_float2(gk[nt][0], gk[nt][1]);
        if (vb) *reinterpret_cast<float2*>(gbuf + 32ll * kb + col) = make_float2(gk[nt][2], gk[nt][3]);
      }
      __syncwarp();
    }
  }
  float* p = part + (size_t)gw * P + woff;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 6; ++nt) {
      const int j = mt * 16 + g, c = nt * 8 + 2 * q;
      p[MpnnLayout::We + j * kIn + c] = gacc[mt][nt][0];
      p[MpnnLayout::We + j * kIn + c + 1] = gacc[mt][nt][1];
      p[MpnnLayout::We + (j + 8) * kIn + c] = gacc[mt][nt][2];
      p[MpnnLayout::We + (j + 8) * kIn + c + 1] = gacc[mt][nt][3];
    }
  p[MpnnLayout::be + lane] = gb;
}

// dh_m = dh_acc_m + sum over edges (n, m) of g
__global__ void k_layer_bwd_gather(int N, const int* brow_ptr, const int* bcol, const int* tmap, const float* dh_acc,
                                   const float* gbuf, float* dh) {
  const int lane = threadIdx.x & 31;
  for (int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; m < N; m += (gridDim.x * blockDim.x) >> 5) {
    float acc = dh_acc[32ll * m + lane];
    for (int k = brow_ptr[m]; k < brow_ptr[m + 1]; ++k) {
      if (bcol[k] == m) continue;
      acc += gbuf[32ll * tmap[k] + lane];
    }
    dh[32ll * m + lane] = acc;
  }
}

__global__ void __launch_bounds__(256) k_encoder_bwd(int N, const float* x, const float* h0, const float* dh,
                                                      float* part, int P) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  float gW[kMF];
  for (int q = 0; q < kMF; ++q) gW[q] = 0.0f;
  float gb = 0.0f;
  for (int n = gw; n < N; n += (gridDim.x * blockDim.x) >> 5) {
    const float dz = (h0[32ll * n + lane] > 0.0f) ? dh[32ll * n + lane] : 0.0f;
    for (int q = 0; q < kMF; ++q) gW[q] += dz * x[20ll * n + q];
    gb += dz;
  }
  float* p = part + (size_t)gw * P;
  for (int q = 0; q < kMF; ++q) p[MpnnLayout::W0 + lane * kMF + q] = gW[q];
  p[MpnnLayout::b0 + lane] = gb;
}

__global__ void k_sum_parts(int P, int nw, const float* part, float* grad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
    float acc = 0.0f;
    for (int w = 0; w < nw; ++w) acc += part[(size_t)w * P + i];
    grad[i] = acc;
  }
}

__global__ void k_adam(int n, float* p, const float* g, float* m1, float* m2, float lr, float b1, float b2, float eps,
                       float c1, float c2, unsigned short* wbf) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float gi = g[i];
    if (!(gi == gi)) gi = 0.0f;
    m1[i] = b1 * m1[i] + (1.0f - b1) * gi;
    m2[i] = b2 * m2[i] + (1.0f - b2) * gi * gi;
    float mh = m1[i] / c1, vh = m2[i] / c2;
    p[i] -= lr * mh / (sqrtf(vh) + eps);
    __nv_bfloat16 b = __float2bfloat16_rn(p[i]);
    wbf[i] = *reinterpret_cast<unsigned short*>(&b);
  }
}

// B_n = S_n W_n S_n^-1 D_n^-1 (W = C with Dirichlet rows/columns zeroed)
__global__ void k_write_B(int N, const double* Dinv, const float* C, const double* sd, const int* dmask,
                          double* out64) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 16 * N; i += gridDim.x * blockDim.x) {
    int n = i >> 4, r = (i >> 2) & 3, c = i & 3;
    double acc = 0.0;
    if (kept(dmask, n, r))
      for (int k = 0; k < 4; ++k)
        if (kept(dmask, n, k))
          acc += (double)C[16ll * n + 4 * r + k] / sd[4ll * n + k] * Dinv[16ll * n + 4 * k + c];
    out64[i] = sd[4ll * n + r] * acc;
  }
}

}  // namespace

void Mpnn::init(int seed) {
  host_params.assign(MpnnLayout::total, 0.0f);
  std::mt19937_64 rng((unsigned long long)seed);
  std::normal_distribution<float> nd(0.0f, 1.0f);
  auto fill = [&](int off, int rows, int cols) {
    float sc = std::sqrt(2.0f / cols);
    for (int i = 0; i < rows * cols; ++i) host_params[off + i] = nd(rng) * sc;
  };
  fill(MpnnLayout::W0, kMH, kMF);
  for (int l = 0; l < kML; ++l) {
    int o = MpnnLayout::L0 + l * MpnnLayout::layer;
    fill(o + MpnnLayout::We, kMH, kME + kMH);
    fill(o + MpnnLayout::Wu, kMH, 2 * kMH);
  }
  // decoder starts at zero: the untrained network is plain block-Jacobi
  adam_t = 0;
  upload();
  m1.alloc(MpnnLayout::total);
  m2.alloc(MpnnLayout::total);
  m1.zero(stream);
  m2.zero(stream);
}

void Mpnn::upload() {
  params.upload(host_params.data(), host_params.size(), stream);
  wbf.alloc(MpnnLayout::total);
  k_to_bf16<<<grid_for(MpnnLayout::total, 256), 256, 0, stream>>>(MpnnLayout::total, params.ptr, wbf.ptr);
  GOAL_CHECK_LAUNCH();
  GOAL_CUDA(cudaStreamSynchronize(stream));
}

void Mpnn::download() {
  host_params.resize(MpnnLayout::total);
  params.download(host_params.data(), stream);
  GOAL_CUDA(cudaStreamSynchronize(stream));
}

void Mpnn::reserve(int N, int nnzb) {
  if (N > cap_nodes) {
    x.alloc(20ll * N);
    h.alloc(32ll * N * (kML + 1));
    u.alloc(32ll * N * kML);
    agg.alloc(32ll * N * kML);
    C.alloc(16ll * N);
    dC.alloc(16ll * N);
    dh.alloc(32ll * N);
    dh_acc.alloc(32ll * N);
    dagg.alloc(32ll * N);
    s.alloc(N);
    sd.alloc(4ll * N);
    Dinv.alloc(16ll * N);
    dP.alloc(16ll * N);
    y.alloc(4ll * N);
    r.alloc(4ll * N);
    gT.alloc(4ll * N);
    v.alloc(4ll * N);
    z.alloc(4ll * N);
    chat.alloc(4ll * N);
    deg.alloc(N);
    dmask.alloc(N);
    cap_nodes = N;
  }
  if (nnzb > cap_blocks) {
    t.alloc(32ll * nnzb * kML);
    gbuf.alloc(32ll * nnzb);
    tmap.alloc(nnzb);
    cap_blocks = nnzb;
  }
  grad.alloc(MpnnLayout::total);
  part.alloc((size_t)kTotalWarps * MpnnLayout::total);
  red.alloc(2 * 2048 + 8);
}

void mpnn_forward(Mpnn& net, const BsrMatrix& A, bool keep) {
  const int N = A.v.num_nodes;
  cudaStream_t st = net.stream;
  net.reserve(N, A.v.nnzb);
  k_features<<<grid_for(N, 128), 128, 0, st>>>(N, A.v.brow_ptr, A.v.bcol, A.v.diag, A.vals, net.x.ptr, net.s.ptr,
                                               net.sd.ptr, net.Dinv.ptr, net.deg.ptr, net.dmask.ptr);
  GOAL_CHECK_LAUNCH();
  const int nb = std::min(grid_for(N, 256), 1024);
  k_sum_log<<<nb, 256, 0, st>>>(N, net.x.ptr, net.red.ptr);
  GOAL_CHECK_LAUNCH();
  k_sub_log_mean<<<grid_for(N, 256), 256, 0, st>>>(N, nb, net.red.ptr, net.x.ptr);
  GOAL_CHECK_LAUNCH();
  const int wgrid = grid_for((long long)N * 32, 256, kSMs * 8);
  float* hbase = net.h.ptr;
  k_encoder<<<wgrid, 256, 0, st>>>(N, net.wbf.ptr, net.x.ptr, hbase);
  GOAL_CHECK_LAUNCH();
  for (int l = 0; l < kML; ++l) {
    const unsigned short* wl = net.wbf.ptr + MpnnLayout::L0 + l * MpnnLayout::layer;
    float* hin = hbase + 32ll * N * l;
    float* hout = hbase + 32ll * N * (l + 1);
    k_layer_fwd<<<wgrid, 256, 0, st>>>(N, A.v.brow_ptr, A.v.bcol, A.vals, net.sd.ptr, net.deg.ptr, wl, hin, hout,
                                       keep ? net.t.ptr + 32ll * A.v.nnzb * l : nullptr,
                                       keep ? net.u.ptr + 32ll * N * l : nullptr,
                                       keep ? net.agg.ptr + 32ll * N * l : nullptr);
    GOAL_CHECK_LAUNCH();
  }
  k_decoder<<<wgrid, 256, 0, st>>>(N, net.wbf.ptr, hbase + 32ll * N * kML, net.C.ptr);
  GOAL_CHECK_LAUNCH();
}

double mpnn_loss_grad(Mpnn& net, const BsrMatrix& A, int num_probes, const double* probes_dev, unsigned seed) {
  const int N = A.v.num_nodes;
  const long long n = 4ll * N;
  cudaStream_t st = net.stream;
  mpnn_forward(net, A, true);
  k_tmap<<<grid_for(N, 128), 128, 0, st>>>(N, A.v.brow_ptr, A.v.bcol, net.tmap.ptr);
  GOAL_CHECK_LAUNCH();
  net.dP.zero(st);
  const int vg = grid_for(n, 256);
  const int nb = std::min(grid_for(n, 256), 1024);
  double* scal = net.red.ptr + 2 * 1024 + 2;  // [|S v|^2, |S e|^2, loss]
  const int* bp = A.v.brow_ptr;
  const int* bc = A.v.bcol;
  GOAL_CUDA(cudaMemsetAsync(scal + 2, 0, sizeof(double), st));
  for (int p = 0; p < num_probes; ++p) {
    if (probes_dev) {
      GOAL_CUDA(cudaMemcpyAsync(net.v.ptr, probes_dev + (size_t)p * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    } else {
      k_gauss<<<vg, 256, 0, st>>>(n, seed + 7919u * (unsigned)p, net.v.ptr);
      GOAL_CHECK_LAUNCH();
    }
    k_probe<<<vg, 256, 0, st>>>(N, net.sd.ptr, net.dmask.ptr, net.v.ptr);
    GOAL_CHECK_LAUNCH();
    if (p & 1) {  // v = A D^-1 q
      k_bjn<<<vg, 256, 0, st>>>(N, net.Dinv.ptr, net.v.ptr, net.z.ptr);
      GOAL_CHECK_LAUNCH();
      k_bsr_mv<<<vg, 256, 0, st>>>(N, bp, bc, A.vals, net.z.ptr, net.v.ptr, nullptr);
      GOAL_CHECK_LAUNCH();
    }
    // z = D^-1 v ; r = v - A z ; y = z + S W chat with chat = D^-1 r / S
    k_bjn<<<vg, 256, 0, st>>>(N, net.Dinv.ptr, net.v.ptr, net.z.ptr);
    GOAL_CHECK_LAUNCH();
    k_bsr_mv<<<vg, 256, 0, st>>>(N, bp, bc, A.vals, net.z.ptr, net.r.ptr, net.v.ptr);
    GOAL_CHECK_LAUNCH();
    k_second_sweep<<<grid_for(N, 128), 128, 0, st>>>(N, net.Dinv.ptr, net.sd.ptr, net.dmask.ptr, net.C.ptr, net.r.ptr,
                                                     net.z.ptr, net.chat.ptr, net.y.ptr);
    GOAL_CHECK_LAUNCH();
    // e = S (v - A y) ; g = A^T (S e)
    k_bsr_mv<<<vg, 256, 0, st>>>(N, bp, bc, A.vals, net.y.ptr, net.r.ptr, net.v.ptr);
    GOAL_CHECK_LAUNCH();
    k_wnorm_part<<<nb, 256, 0, st>>>(n, net.v.ptr, net.sd.ptr, net.red.ptr);
    GOAL_CHECK_LAUNCH();
    k_fin2<<<1, 1024, 0, st>>>(net.red.ptr, nb, scal);
    GOAL_CHECK_LAUNCH();
    k_wnorm_part<<<nb, 256, 0, st>>>(n, net.r.ptr, net.sd.ptr, net.red.ptr);
    GOAL_CHECK_LAUNCH();
    k_fin2<<<1, 1024, 0, st>>>(net.red.ptr, nb, scal + 1);
    GOAL_CHECK_LAUNCH();
    k_scale_by<<<vg, 256, 0, st>>>(n, net.sd.ptr, net.r.ptr);
    GOAL_CHECK_LAUNCH();
    k_scale_by<<<vg, 256, 0, st>>>(n, net.sd.ptr, net.r.ptr);
    GOAL_CHECK_LAUNCH();
    k_bsr_mv_t<<<vg, 256, 0, st>>>(N, bp, bc, net.tmap.ptr, A.vals, net.r.ptr, net.gT.ptr);
    GOAL_CHECK_LAUNCH();
    k_dW<<<grid_for(16ll * N, 256), 256, 0, st>>>(N, net.gT.ptr, net.sd.ptr, net.chat.ptr, net.dmask.ptr, scal,
                                                  net.dP.ptr);
    GOAL_CHECK_LAUNCH();
    k_loss_acc<<<1, 32, 0, st>>>(scal, scal + 2);
    GOAL_CHECK_LAUNCH();
  }
  k_dC<<<grid_for(16ll * N, 256), 256, 0, st>>>(N, net.dP.ptr, net.dC.ptr);
  GOAL_CHECK_LAUNCH();
  // backward
  const int P = MpnnLayout::total;
  GOAL_CUDA(cudaMemsetAsync(net.part.ptr, 0, sizeof(float) * net.part.n, st));
  float* hbase = net.h.ptr;
  k_decoder_bwd<<<kGridBlocks, 256, 0, st>>>(N, net.wbf.ptr, hbase + 32ll * N * kML, net.dC.ptr, net.dh.ptr,
                                              net.part.ptr, P);
  GOAL_CHECK_LAUNCH();
  DevBuf<float>& dh_acc = net.dh_acc;
  for (int l = kML - 1; l >= 0; --l) {
    const int woff = MpnnLayout::L0 + l * MpnnLayout::layer;
    const unsigned short* wl = net.wbf.ptr + woff;
    const float* hin = hbase + 32ll * N * l;
    k_layer_bwd_node<<<kGridBlocks, 256, 0, st>>>(N, wl, woff, hin, net.u.ptr + 32ll * N * l,
                                                   net.agg.ptr + 32ll * N * l, net.deg.ptr, net.dh.ptr, dh_acc.ptr,
                                                   net.dagg.ptr, net.part.ptr, P);
    GOAL_CHECK_LAUNCH();
    k_layer_bwd_edge<<<kGridBlocks, 256, 0, st>>>(N, A.v.brow_ptr, A.v.bcol, A.vals, net.sd.ptr, wl, woff, hin,
                                                   net.t.ptr + 32ll * A.v.nnzb * l, net.dagg.ptr, net.gbuf.ptr,
                                                   net.part.ptr, P);
    GOAL_CHECK_LAUNCH();
    k_layer_bwd_gather<<<grid_for((long long)N * 32, 256, kSMs * 8), 256, 0, st>>>(
        N, A.v.brow_ptr, A.v.bcol, net.tmap.ptr, dh_acc.ptr, net.gbuf.ptr, net.dh.ptr);
    GOAL_CHECK_LAUNCH();
  }
  k_encoder_bwd<<<kGridBlocks, 256, 0, st>>>(N, net.x.ptr, hbase, net.dh.ptr, net.part.ptr, P);
  GOAL_CHECK_LAUNCH();
  k_sum_parts<<<grid_for(P, 256), 256, 0, st>>>(P, kTotalWarps, net.part.ptr, net.grad.ptr);
  GOAL_CHECK_LAUNCH();
  double loss = 0.0;
  GOAL_CUDA(cudaMemcpyAsync(&loss, scal + 2, sizeof(double), cudaMemcpyDeviceToHost, st));
  GOAL_CUDA(cudaStreamSynchronize(st));
  return loss;
}

void mpnn_adam(Mpnn& net, float lr, float beta1, float beta2, float eps) {
  net.adam_t += 1;
  float c1 = 1.0f - std::pow(beta1, (float)net.adam_t);
  float c2 = 1.0f - std::pow(beta2, (float)net.adam_t);
  k_adam<<<grid_for(MpnnLayout::total, 256), 256, 0, net.stream>>>(MpnnLayout::total, net.params.ptr, net.grad.ptr,
                                                                    net.m1.ptr, net.m2.ptr, lr, beta1, beta2, eps, c1,
                                                                    c2, net.wbf.ptr);
  GOAL_CHECK_LAUNCH();
}

void mpnn_apply_to_block_jacobi(Mpnn& net, const BsrMatrix& A, Krylov& K) {
  const int N = A.v.num_nodes;
  mpnn_forward(net, A, false);
  need(K.Bc, 16ull * N);
  k_write_B<<<grid_for(16ll * N, 256), 256, 0, net.stream>>>(N, net.Dinv.ptr, net.C.ptr, net.sd.ptr, net.dmask.ptr,
                                                             K.Bc.ptr);
  GOAL_CHECK_LAUNCH();
  K.two_sweep = true;
}

}  // namespace goal
