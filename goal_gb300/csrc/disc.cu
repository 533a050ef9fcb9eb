// Device-side discretization build: node->element incidence, block graph,
// element colouring, colour-major element layout and per-element geometry.
// All of it runs on the GPU; the host only sequences the passes.
//
// Reference behaviour followed (src/goal_disc.cpp):
//   DOF lid = node*num_eqs + eq                        (:195-201)
//   element lids node-major, 4 per node                (:214-222)
//   graph = union of element stencils, sorted columns  (:307-332; Tpetra fillComplete sorts)
//   geometry: one integration point per tet, weight 1/6 x detJ; stabilization
//   size = rms of the six edge lengths                 (src/goal_stabilization.cpp:45-52)
#include <cub/cub.cuh>

#include <algorithm>
#include <chrono>

#include "disc.cuh"

namespace goal {

namespace {

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16; x *= 0x7feb352du;
  x ^= x >> 15; x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__global__ void k_count_incidence(int n4, const int* tets, int* cnt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x)
    atomicAdd(&cnt[tets[i]], 1);
}

__global__ void k_iota(int n, int* a) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = i;
}

// One warp per node: sort-unique the nodes of all incident elements.
// pass 0 writes the unique count, pass 1 writes the sorted neighbour list.
constexpr int kCand = 4 * kMaxNodeElems;
__global__ void k_node_adjacency(int N, const int* tets, const int* ne_ptr, const int* ne_list,
                                 const int* brow_ptr, int* out_count, int* bcol, int* err) {
  extern __shared__ int sbuf[];
  int warps = blockDim.x >> 5;
  int lane = threadIdx.x & 31;
  int* buf = sbuf + (threadIdx.x >> 5) * kCand;
  for (int n = blockIdx.x * warps + (threadIdx.x >> 5); n < N; n += gridDim.x * warps) {
    int b = ne_ptr[n], m = ne_ptr[n + 1] - b;
    if (m > kMaxNodeElems) {
      if (lane == 0) atomicExch(err, 1);
      continue;
    }
    int cnt = 4 * m;
    int P = 32;
    while (P < cnt) P <<= 1;
    for (int i = lane; i < P; i += 32) {
      int v = 0x7fffffff;
      if (i < cnt) {
        int inc = ne_list[b + (i >> 2)];
        v = tets[4 * (inc >> 2) + (i & 3)];
      }
      buf[i] = v;
    }
    __syncwarp();
    for (int k = 2; k <= P; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = lane; i < P; i += 32) {
          int ixj = i ^ j;
          if (ixj > i) {
            int x = buf[i], y = buf[ixj];
            bool up = ((i & k) == 0);
            if ((x > y) == up) { buf[i] = y; buf[ixj] = x; }
          }
        }
        __syncwarp();
      }
    int base = brow_ptr ? brow_ptr[n] : 0;
    int total = 0;
    for (int i0 = 0; i0 < cnt; i0 += 32) {
      int i = i0 + lane;
      bool keep = (i < cnt) && (i == 0 || buf[i] != buf[i - 1]);
      unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (keep && bcol) bcol[base + total + __popc(bal & ((1u << lane) - 1u))] = buf[i];
      total += __popc(bal);
    }
    if (lane == 0 && out_count) out_count[n] = total;
    __syncwarp();
  }
}

__device__ __forceinline__ int lower_bound_dev(const int* a, int n, int key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// off-diagonal blocks in block order: block k of row n (k != diag[n]) goes to
// position k - n - (k > diag[n]) (one diagonal block per earlier row)
__global__ void k_offd(int N, const int* brow_ptr, const int* diag, int* offd) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    const int dn = diag[n];
    for (int k = brow_ptr[n]; k < brow_ptr[n + 1]; ++k)
      if (k != dn) offd[k - n - (k > dn ? 1 : 0)] = k;
  }
}

__global__ void k_diag(int N, const int* brow_ptr, const int* bcol, int* diag) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    int b = brow_ptr[n];
    diag[n] = b + lower_bound_dev(bcol + b, brow_ptr[n + 1] - b, n);
  }
}

// btr[k] = index of block (m, n) for block k = (n, m) of the symmetric block graph
__global__ void k_block_transpose(int N, const int* brow_ptr, const int* bcol, int* btr) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x)
    for (int k = brow_ptr[n]; k < brow_ptr[n + 1]; ++k) {
      const int m = bcol[k], b = brow_ptr[m];
      btr[k] = b + lower_bound_dev(bcol + b, brow_ptr[m + 1] - b, n);
    }
}

// Jones-Plassmann round with first-fit colours. Reads colours of the previous
// round only (cin), so the result does not depend on scheduling.
__global__ void k_color_round(int E, const int* tets, const int* ne_ptr, const int* ne_list,
                              const int* cin, int* cout, int* remaining, int* overflow) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
    int ce = cin[e];
    if (ce >= 0) { cout[e] = ce; continue; }
    uint32_t pe = mix32((uint32_t)e);
    unsigned long long m0 = 0ull, m1 = 0ull;
    bool ready = true;
    for (int a = 0; a < 4 && ready; ++a) {
      int n = tets[4 * e + a];
      for (int k = ne_ptr[n]; k < ne_ptr[n + 1]; ++k) {
        int f = ne_list[k] >> 2;
        if (f == e) continue;
        int cf = cin[f];
        if (cf >= 0) {
          if (cf < 64) m0 |= 1ull << cf;
          else m1 |= 1ull << (cf - 64);
        } else {
          uint32_t pf = mix32((uint32_t)f);
          if (pf > pe || (pf == pe && f > e)) { ready = false; break; }
        }
      }
    }
    if (ready) {
      int c;
      if (~m0) c = __ffsll((long long)~m0) - 1;
      else if (~m1) c = 64 + __ffsll((long long)~m1) - 1;
      else { c = 0; atomicExch(overflow, 1); }
      cout[e] = c;
    } else {
      cout[e] = -1;
      atomicAdd(remaining, 1);
    }
  }
}

__global__ void k_slots_and_min(int E, const int* tets, const int* brow_ptr, const int* bcol,
                                const int* color, int* blk_orig, int* bmin, int* nmin) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
    int c = color[e];
    int v[4];
    for (int a = 0; a < 4; ++a) v[a] = tets[4 * e + a];
    for (int a = 0; a < 4; ++a) {
      int b0 = brow_ptr[v[a]], len = brow_ptr[v[a] + 1] - b0;
      atomicMin(&nmin[v[a]], c);
      for (int b = 0; b < 4; ++b) {
        int k = b0 + lower_bound_dev(bcol + b0, len, v[b]);
        blk_orig[16 * e + 4 * a + b] = k;
        atomicMin(&bmin[k], c);
      }
    }
  }
}

// Writes the colour-major element arrays and the per-element geometry.
__global__ void k_permute(int E, const int* perm, const int* tets, const int* elem_set, const int* color,
                          const int* blk_orig, const int* bmin, const int* nmin, const double* X,
                          int* tets_s, int* es_s, int* orig, int* pos, int* blk_s, unsigned* first,
                          int* color_s, double* grads, double* vol, double* hh) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) {
    int e = perm[s];
    orig[s] = e;
    pos[e] = s;
    int c = color[e];
    color_s[s] = c;
    es_s[s] = elem_set[e];
    int v[4];
    for (int a = 0; a < 4; ++a) { v[a] = tets[4 * e + a]; tets_s[a * E + s] = v[a]; }
    unsigned mask = 0;
    for (int q = 0; q < 16; ++q) {
      int k = blk_orig[16 * e + q];
      blk_s[q * E + s] = k;
      if (bmin[k] == c) mask |= 1u << q;
    }
    for (int a = 0; a < 4; ++a)
      if (nmin[v[a]] == c) mask |= 1u << (16 + a);
    first[s] = mask;
    // geometry (same arithmetic as the oracle: inverse by cofactors / det)
    double J[3][3];
    for (int cc = 0; cc < 3; ++cc)
      for (int r = 0; r < 3; ++r) J[r][cc] = X[3 * v[cc + 1] + r] - X[3 * v[0] + r];
    double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    double c01 = J[1][0] * J[2][2] - J[1][2] * J[2][0];
    double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    double d = J[0][0] * c00 - J[0][1] * c01 + J[0][2] * c02;
    double Ji[3][3];
    Ji[0][0] = c00 / d;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / d;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / d;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / d;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / d;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / d;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / d;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / d;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / d;
    for (int a = 1; a < 4; ++a)
      for (int k = 0; k < 3; ++k) grads[(3 * a + k) * E + s] = Ji[a - 1][k];
    for (int k = 0; k < 3; ++k) grads[k * E + s] = -(Ji[0][k] + Ji[1][k] + Ji[2][k]);
    vol[s] = d / 6.0;
    const int ed[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
    double hs = 0.0;
    for (int q = 0; q < 6; ++q) {
      const double* pa = X + 3 * v[ed[q][0]];
      const double* pb = X + 3 * v[ed[q][1]];
      double dx = pa[0] - pb[0], dy = pa[1] - pb[1], dz = pa[2] - pb[2];
      double l = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
      hs = __dadd_rn(hs, __dmul_rn(l, l));
    }
    hh[s] = sqrt(hs / 6.0);
  }
}

__global__ void k_contrib_keys(int E, const int* blk_s, const int* tets_s, int* bkeys, int* bvals, int* nkeys,
                               int* nvals, int* bcnt, int* ncnt) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) {
    for (int q = 0; q < 16; ++q) {
      int k = blk_s[(long long)q * E + s];
      bkeys[16ll * s + q] = k;
      bvals[16ll * s + q] = 16 * s + q;
      atomicAdd(&bcnt[k], 1);
    }
    for (int a = 0; a < 4; ++a) {
      int n = tets_s[(long long)a * E + s];
      nkeys[4ll * s + a] = n;
      nvals[4ll * s + a] = 4 * s + a;
      atomicAdd(&ncnt[n], 1);
    }
  }
}

template <typename T>
void exclusive_scan(const T* in, T* out, int n, cudaStream_t s) {
  size_t bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, n, s);
  DevBuf<unsigned char> tmp;
  tmp.alloc(bytes ? bytes : 1);
  cub::DeviceScan::ExclusiveSum(tmp.ptr, bytes, in, out, n, s);
  GOAL_CHECK_LAUNCH();
  GOAL_CUDA(cudaStreamSynchronize(s));
}

void sort_pairs(const int* kin, int* kout, const int* vin, int* vout, int n, int end_bit, cudaStream_t s) {
  size_t bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, bytes, kin, kout, vin, vout, n, 0, end_bit, s);
  DevBuf<unsigned char> tmp;
  tmp.alloc(bytes ? bytes : 1);
  cub::DeviceRadixSort::SortPairs(tmp.ptr, bytes, kin, kout, vin, vout, n, 0, end_bit, s);
  GOAL_CHECK_LAUNCH();
  GOAL_CUDA(cudaStreamSynchronize(s));
}

int bits_for(int n) {
  int b = 1;
  while ((1ll << b) <= (long long)n) ++b;
  return b;
}

}  // namespace

void Disc::build() {
  GOAL_REQUIRE(num_nodes > 0 && num_elems > 0, GOAL_ERR_ARG, "empty mesh");
  cudaStream_t s = stream;
  const int N = num_nodes, E = num_elems;
  auto clock = [] { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
  double tp = clock();
  auto phase = [&](int k) {  // closes phase k at a stream synchronisation
    GOAL_CUDA(cudaStreamSynchronize(s));
    const double t = clock();
    build_seconds[k] = t - tp;
    tp = t;
  };
  coords.upload(coords_h.data(), coords_h.size(), s);
  DevBuf<int> tets_o, es_o;
  tets_o.upload(tets_h.data(), tets_h.size(), s);
  es_o.upload(elem_set_h.data(), elem_set_h.size(), s);

  // node -> element incidence (stable sort keeps element order within a node)
  DevBuf<int> cnt, ne_ptr, inc_idx, keys_sorted, ne_list;
  cnt.alloc(N + 1);
  cnt.zero(s);
  k_count_incidence<<<grid_for(4ll * E, 256), 256, 0, s>>>(4 * E, tets_o.ptr, cnt.ptr);
  GOAL_CHECK_LAUNCH();
  ne_ptr.alloc(N + 1);
  exclusive_scan(cnt.ptr, ne_ptr.ptr, N + 1, s);
  inc_idx.alloc(4 * E);
  k_iota<<<grid_for(4ll * E, 256), 256, 0, s>>>(4 * E, inc_idx.ptr);
  keys_sorted.alloc(4 * E);
  ne_list.alloc(4 * E);
  sort_pairs(tets_o.ptr, keys_sorted.ptr, inc_idx.ptr, ne_list.ptr, 4 * E, bits_for(N), s);

  // block graph
  DevBuf<int> err, deg;
  err.alloc(1);
  err.zero(s);
  deg.alloc(N + 1);
  deg.zero(s);
  const int warps = 8;
  size_t smem = (size_t)warps * kCand * sizeof(int);
  int gblocks = grid_for(N, warps, kSMs * 64);
  k_node_adjacency<<<gblocks, 32 * warps, smem, s>>>(N, tets_o.ptr, ne_ptr.ptr, ne_list.ptr, nullptr, deg.ptr,
                                                     nullptr, err.ptr);
  GOAL_CHECK_LAUNCH();
  int herr = 0;
  GOAL_CUDA(cudaMemcpyAsync(&herr, err.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  GOAL_CUDA(cudaStreamSynchronize(s));
  GOAL_REQUIRE(herr == 0, GOAL_ERR_CAPACITY, "a node has more than 128 incident elements");
  brow_ptr.alloc(N + 1);
  exclusive_scan(deg.ptr, brow_ptr.ptr, N + 1, s);
  GOAL_CUDA(cudaMemcpyAsync(&nnzb, brow_ptr.ptr + N, sizeof(int), cudaMemcpyDeviceToHost, s));
  GOAL_CUDA(cudaStreamSynchronize(s));
  nnz = 16ll * nnzb;
  bcol.alloc(nnzb);
  k_node_adjacency<<<gblocks, 32 * warps, smem, s>>>(N, tets_o.ptr, ne_ptr.ptr, ne_list.ptr, brow_ptr.ptr,
                                                     nullptr, bcol.ptr, err.ptr);
  GOAL_CHECK_LAUNCH();
  diag.alloc(N);
  k_diag<<<grid_for(N, 256), 256, 0, s>>>(N, brow_ptr.ptr, bcol.ptr, diag.ptr);
  GOAL_CHECK_LAUNCH();
  offd.alloc(nnzb - N);
  k_offd<<<grid_for(N, 256), 256, 0, s>>>(N, brow_ptr.ptr, diag.ptr, offd.ptr);
  GOAL_CHECK_LAUNCH();
  phase(0);

  // colouring
  DevBuf<int> ca, cb, rem, ovf;
  ca.alloc(E);
  cb.alloc(E);
  GOAL_CUDA(cudaMemsetAsync(ca.ptr, 0xff, sizeof(int) * E, s));
  rem.alloc(1);
  ovf.alloc(1);
  ovf.zero(s);
  int rounds = 0;
  for (;;) {
    rem.zero(s);
    k_color_round<<<grid_for(E, 256), 256, 0, s>>>(E, tets_o.ptr, ne_ptr.ptr, ne_list.ptr, ca.ptr, cb.ptr,
                                                    rem.ptr, ovf.ptr);
    GOAL_CHECK_LAUNCH();
    std::swap(ca.ptr, cb.ptr);
    int hrem = 0;
    GOAL_CUDA(cudaMemcpyAsync(&hrem, rem.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    GOAL_CUDA(cudaStreamSynchronize(s));
    ++rounds;
    if (hrem == 0) break;
    GOAL_REQUIRE(rounds < 100000, GOAL_ERR_STATE, "element colouring did not terminate");
  }
  int hovf = 0;
  GOAL_CUDA(cudaMemcpyAsync(&hovf, ovf.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  GOAL_CUDA(cudaStreamSynchronize(s));
  GOAL_REQUIRE(hovf == 0, GOAL_ERR_CAPACITY, "element colouring needs more than 128 colours");
  color_rounds = rounds;
  phase(1);

  // colour-major order (stable in element id)
  DevBuf<int> ids, csorted, perm;
  ids.alloc(E);
  k_iota<<<grid_for(E, 256), 256, 0, s>>>(E, ids.ptr);
  csorted.alloc(E);
  perm.alloc(E);
  sort_pairs(ca.ptr, csorted.ptr, ids.ptr, perm.ptr, E, 8, s);
  std::vector<int> cs = csorted.to_host(s);
  num_colors = cs.empty() ? 0 : cs.back() + 1;
  color_ptr.assign(num_colors + 1, 0);
  for (int c : cs) color_ptr[c + 1]++;
  for (int c = 0; c < num_colors; ++c) color_ptr[c + 1] += color_ptr[c];

  // block slots and first writers
  DevBuf<int> blk_orig, bmin, nmin;
  blk_orig.alloc(16ll * E);
  bmin.alloc(nnzb);
  nmin.alloc(N);
  GOAL_CUDA(cudaMemsetAsync(bmin.ptr, 0x7f, sizeof(int) * nnzb, s));
  GOAL_CUDA(cudaMemsetAsync(nmin.ptr, 0x7f, sizeof(int) * N, s));
  k_slots_and_min<<<grid_for(E, 256), 256, 0, s>>>(E, tets_o.ptr, brow_ptr.ptr, bcol.ptr, ca.ptr, blk_orig.ptr,
                                                    bmin.ptr, nmin.ptr);
  GOAL_CHECK_LAUNCH();

  tets.alloc(4ll * E);
  elem_set.alloc(E);
  elem_orig.alloc(E);
  elem_pos.alloc(E);
  blk.alloc(16ll * E);
  first.alloc(E);
  color.alloc(E);
  grads.alloc(12ll * E);
  vol.alloc(E);
  h.alloc(E);
  k_permute<<<grid_for(E, 256), 256, 0, s>>>(E, perm.ptr, tets_o.ptr, es_o.ptr, ca.ptr, blk_orig.ptr, bmin.ptr,
                                              nmin.ptr, coords.ptr, tets.ptr, elem_set.ptr, elem_orig.ptr,
                                              elem_pos.ptr, blk.ptr, first.ptr, color.ptr, grads.ptr, vol.ptr,
                                              h.ptr);
  GOAL_CHECK_LAUNCH();
  phase(2);
  {
    // contribution lists (stable sorts keep the element order within a block / node)
    DevBuf<int> bk, bv, nk, nv, bks, nks, bcnt, ncnt;
    bk.alloc(16ll * E);
    bv.alloc(16ll * E);
    nk.alloc(4ll * E);
    nv.alloc(4ll * E);
    bcnt.alloc(nnzb + 1);
    ncnt.alloc(N + 1);
    bcnt.zero(s);
    ncnt.zero(s);
    k_contrib_keys<<<grid_for(E, 256), 256, 0, s>>>(E, blk.ptr, tets.ptr, bk.ptr, bv.ptr, nk.ptr, nv.ptr, bcnt.ptr,
                                                     ncnt.ptr);
    GOAL_CHECK_LAUNCH();
    bptr.alloc(nnzb + 1);
    nptr.alloc(N + 1);
    exclusive_scan(bcnt.ptr, bptr.ptr, nnzb + 1, s);
    exclusive_scan(ncnt.ptr, nptr.ptr, N + 1, s);
    bks.alloc(16ll * E);
    blist.alloc(16ll * E);
    sort_pairs(bk.ptr, bks.ptr, bv.ptr, blist.ptr, 16 * E, bits_for(nnzb), s);
    nks.alloc(4ll * E);
    nlist.alloc(4ll * E);
    sort_pairs(nk.ptr, nks.ptr, nv.ptr, nlist.ptr, 4 * E, bits_for(N), s);
    phase(3);
  }

  // node sets / side sets to the device
  for (auto& kv : node_sets) kv.second->dev.upload(kv.second->host.data(), kv.second->host.size(), s);
  for (auto& kv : side_sets) {
    SideSet& ss = *kv.second;
    int S = (int)ss.tris.size() / 3;
    ss.dtris.upload(ss.tris.data(), ss.tris.size(), s);
    std::vector<std::pair<int, int>> incs;
    incs.reserve(3 * S);
    for (int k = 0; k < 3 * S; ++k) incs.emplace_back(ss.tris[k], k);
    std::sort(incs.begin(), incs.end());
    std::vector<int> nodes, ptr, inc;
    for (size_t k = 0; k < incs.size(); ++k) {
      if (k == 0 || incs[k].first != incs[k - 1].first) {
        nodes.push_back(incs[k].first);
        ptr.push_back((int)k);
      }
      inc.push_back(incs[k].second);
    }
    ptr.push_back((int)incs.size());
    ss.nodes_h = nodes;
    ss.nodes.upload(nodes.data(), nodes.size(), s);
    ss.inc_ptr.upload(ptr.data(), ptr.size(), s);
    ss.inc.upload(inc.data(), inc.size(), s);
  }
  phase(4);
  built = true;
}

DiscView Disc::view() const {
  DiscView v;
  v.num_nodes = num_nodes;
  v.num_elems = num_elems;
  v.nnzb = nnzb;
  v.coords = coords.ptr;
  v.tets = tets.ptr;
  v.grads = grads.ptr;
  v.vol = vol.ptr;
  v.h = h.ptr;
  v.blk = blk.ptr;
  v.first = first.ptr;
  v.brow_ptr = brow_ptr.ptr;
  v.bcol = bcol.ptr;
  v.diag = diag.ptr;
  v.elem_set = elem_set.ptr;
  v.elem_orig = elem_orig.ptr;
  return v;
}

namespace {
// Expands the block graph to the scalar CSR graph: row 4n+eq holds
// 4*deg(n) columns 4m+l for every neighbour m (sorted) and l = 0..3.
__global__ void k_csr_expand(int N, const int* brow_ptr, const int* bcol, int* row_ptr, int* col_idx) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    int b = brow_ptr[n], deg = brow_ptr[n + 1] - b;
    for (int eq = 0; eq < 4; ++eq) {
      int r0 = 16 * b + 4 * eq * deg;
      row_ptr[4 * n + eq] = r0;
      for (int j = 0; j < deg; ++j)
        for (int l = 0; l < 4; ++l) col_idx[r0 + 4 * j + l] = 4 * bcol[b + j] + l;
    }
    if (n == N - 1) row_ptr[4 * N] = 16 * brow_ptr[N];
  }
}
}  // namespace

void Disc::csr_graph(int* row_ptr_h, int* col_idx_h) const {
  DevBuf<int> rp, ci;
  rp.alloc(4ll * num_nodes + 1);
  ci.alloc(nnz);
  k_csr_expand<<<grid_for(num_nodes, 128), 128, 0, stream>>>(num_nodes, brow_ptr.ptr, bcol.ptr, rp.ptr, ci.ptr);
  GOAL_CHECK_LAUNCH();
  rp.download(row_ptr_h, stream);
  ci.download(col_idx_h, stream);
  GOAL_CUDA(cudaStreamSynchronize(stream));
}

void Disc::block_transpose_map() {
  if (btr.ptr) return;
  btr.alloc(nnzb);
  k_block_transpose<<<grid_for(num_nodes, 256), 256, 0, stream>>>(num_nodes, brow_ptr.ptr, bcol.ptr, btr.ptr);
  GOAL_CHECK_LAUNCH();
}

void Disc::csr_graph_device() {
  if (csr_row_ptr.ptr) return;
  GOAL_REQUIRE(nnz <= 2147483647ll, GOAL_ERR_CAPACITY, "scalar CSR graph: more than 2^31-1 nonzeros for int32 indices");
  csr_row_ptr.alloc(4ll * num_nodes + 1);
  csr_col_idx.alloc(nnz);
  k_csr_expand<<<grid_for(num_nodes, 128), 128, 0, stream>>>(num_nodes, brow_ptr.ptr, bcol.ptr, csr_row_ptr.ptr,
                                                             csr_col_idx.ptr);
  GOAL_CHECK_LAUNCH();
  GOAL_CUDA(cudaStreamSynchronize(stream));
}

// ------------------------------------------------------------------ nested
namespace {

__global__ void k_edge_count(int N, const int* brow_ptr, const int* diag, int* cnt) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x)
    cnt[n] = brow_ptr[n + 1] - diag[n] - 1;
}

__global__ void k_edges(int N, const int* brow_ptr, const int* bcol, const int* diag, const int* eptr,
                        const double* X, int* edges, double* Xn) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    int e0 = eptr[n];
    for (int k = diag[n] + 1; k < brow_ptr[n + 1]; ++k) {
      int id = e0 + (k - diag[n] - 1);
      int m = bcol[k];
      edges[2 * id] = n;
      edges[2 * id + 1] = m;
      for (int d = 0; d < 3; ++d) Xn[3 * (N + id) + d] = 0.5 * (X[3 * n + d] + X[3 * m + d]);
    }
    for (int d = 0; d < 3; ++d) Xn[3 * n + d] = X[3 * n + d];
  }
}

__device__ __forceinline__ double dot_rn(const double* v) {
  return __dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2]));
}

__device__ __forceinline__ void orient(const double* X, int* t) {
  double a[3], b[3], c[3];
  for (int d = 0; d < 3; ++d) {
    a[d] = X[3 * t[1] + d] - X[3 * t[0] + d];
    b[d] = X[3 * t[2] + d] - X[3 * t[0] + d];
    c[d] = X[3 * t[3] + d] - X[3 * t[0] + d];
  }
  double cr0 = b[1] * c[2] - b[2] * c[1];
  double cr1 = b[2] * c[0] - b[0] * c[2];
  double cr2 = b[0] * c[1] - b[1] * c[0];
  double v = a[0] * cr0 + a[1] * cr1 + a[2] * cr2;
  if (v < 0) { int tmp = t[2]; t[2] = t[3]; t[3] = tmp; }
}

__global__ void k_children(int E, int N, const int* tets, const int* blk, const int* diag, const int* eptr,
                           const int* orig, const int* es, const double* X, const double* Xn, int* ctets,
                           int* ces) {
  const int MID[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  const int OD[3][2] = {{0, 5}, {1, 4}, {2, 3}};
  const int OC[3][4] = {{1, 2, 4, 3}, {0, 2, 5, 3}, {0, 1, 5, 4}};
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) {
    int e = orig[s];
    int v[4];
    for (int a = 0; a < 4; ++a) v[a] = tets[a * E + s];
    int m[6];
    for (int q = 0; q < 6; ++q) {
      int a = MID[q][0], b = MID[q][1];
      if (v[a] > v[b]) { int t = a; a = b; b = t; }
      int k = blk[(4 * a + b) * E + s];
      m[q] = N + eptr[v[a]] + (k - diag[v[a]] - 1);
    }
    int ch[8][4] = {{v[0], m[0], m[1], m[2]}, {m[0], v[1], m[3], m[4]}, {m[1], m[3], v[2], m[5]},
                    {m[2], m[4], m[5], v[3]}};
    double d2[3];
    for (int k = 0; k < 3; ++k) {
      int a = MID[OD[k][0]][0], b = MID[OD[k][0]][1];
      int c = MID[OD[k][1]][0], d = MID[OD[k][1]][1];
      double vec[3];
      for (int x = 0; x < 3; ++x)
        vec[x] = __dsub_rn(__dsub_rn(__dadd_rn(X[3 * v[c] + x], X[3 * v[d] + x]), X[3 * v[a] + x]), X[3 * v[b] + x]);
      d2[k] = dot_rn(vec);
    }
    double dmin = fmin(d2[0], fmin(d2[1], d2[2]));
    double lim = __dmul_rn(dmin, 1.0 + 1e-12);
    int choice = (d2[0] <= lim) ? 0 : ((d2[1] <= lim) ? 1 : 2);
    for (int c = 0; c < 4; ++c) {
      ch[4 + c][0] = m[OD[choice][0]];
      ch[4 + c][1] = m[OD[choice][1]];
      ch[4 + c][2] = m[OC[choice][c]];
      ch[4 + c][3] = m[OC[choice][(c + 1) & 3]];
    }
    for (int c = 0; c < 8; ++c) {
      orient(Xn, ch[c]);
      for (int a = 0; a < 4; ++a) ctets[4 * (8 * e + c) + a] = ch[c][a];
      ces[8 * e + c] = es[s];
    }
  }
}

}  // namespace

std::unique_ptr<Disc> refine_uniform(const Disc& base) {
  GOAL_REQUIRE(base.built, GOAL_ERR_STATE, "base discretization not built");
  cudaStream_t s = base.stream;
  const int N = base.num_nodes, E = base.num_elems;
  DevBuf<int> cnt, eptr;
  cnt.alloc(N + 1);
  cnt.zero(s);
  k_edge_count<<<grid_for(N, 256), 256, 0, s>>>(N, base.brow_ptr.ptr, base.diag.ptr, cnt.ptr);
  GOAL_CHECK_LAUNCH();
  eptr.alloc(N + 1);
  exclusive_scan(cnt.ptr, eptr.ptr, N + 1, s);
  int Ne = 0;
  GOAL_CUDA(cudaMemcpyAsync(&Ne, eptr.ptr + N, sizeof(int), cudaMemcpyDeviceToHost, s));
  GOAL_CUDA(cudaStreamSynchronize(s));
  auto out = std::make_unique<Disc>();
  out->stream = s;
  out->num_nodes = N + Ne;
  out->num_elems = 8 * E;
  out->num_elem_sets = base.num_elem_sets;
  out->elem_set_names = base.elem_set_names;
  out->base_nodes = N;
  out->base_elems = E;
  out->parent_edges.alloc(2ll * Ne);
  DevBuf<double> Xn;
  Xn.alloc(3ll * (N + Ne));
  k_edges<<<grid_for(N, 256), 256, 0, s>>>(N, base.brow_ptr.ptr, base.bcol.ptr, base.diag.ptr, eptr.ptr,
                                            base.coords.ptr, out->parent_edges.ptr, Xn.ptr);
  GOAL_CHECK_LAUNCH();
  DevBuf<int> ctets, ces;
  ctets.alloc(32ll * E);
  ces.alloc(8ll * E);
  k_children<<<grid_for(E, 128), 128, 0, s>>>(E, N, base.tets.ptr, base.blk.ptr, base.diag.ptr, eptr.ptr,
                                               base.elem_orig.ptr, base.elem_set.ptr, base.coords.ptr, Xn.ptr,
                                               ctets.ptr, ces.ptr);
  GOAL_CHECK_LAUNCH();
  out->coords_h = Xn.to_host(s);
  out->tets_h = ctets.to_host(s);
  out->elem_set_h = ces.to_host(s);
  std::vector<int> edges = out->parent_edges.to_host(s);

  auto edge_of = [&](int a, int b) -> int {
    int lo = std::min(a, b), hi = std::max(a, b);
    // edges are sorted by (lo, hi)
    int l = 0, r = Ne;
    while (l < r) {
      int mid = (l + r) / 2;
      long long km = (long long)edges[2 * mid] * (N + 1) + edges[2 * mid + 1];
      long long kk = (long long)lo * (N + 1) + hi;
      if (km < kk) l = mid + 1;
      else r = mid;
    }
    GOAL_REQUIRE(l < Ne && edges[2 * l] == lo && edges[2 * l + 1] == hi, GOAL_ERR_STATE, "side edge not in mesh");
    return N + l;
  };
  for (auto& kv : base.node_sets) {
    auto ns = std::make_unique<NodeSet>();
    ns->name = kv.first;
    std::vector<char> in(N, 0);
    for (int n : kv.second->host) in[n] = 1;
    ns->host = kv.second->host;
    for (int k = 0; k < Ne; ++k)
      if (in[edges[2 * k]] && in[edges[2 * k + 1]]) ns->host.push_back(N + k);
    out->node_sets[kv.first] = std::move(ns);
  }
  for (auto& kv : base.side_sets) {
    auto ss = std::make_unique<SideSet>();
    ss->name = kv.first;
    const std::vector<int>& t = kv.second->tris;
    for (size_t k = 0; k + 2 < t.size(); k += 3) {
      int a = t[k], b = t[k + 1], c = t[k + 2];
      int mab = edge_of(a, b), mbc = edge_of(b, c), mca = edge_of(c, a);
      int sub[4][3] = {{a, mab, mca}, {mab, b, mbc}, {mca, mbc, c}, {mab, mbc, mca}};
      for (auto& q : sub) ss->tris.insert(ss->tris.end(), q, q + 3);
    }
    out->side_sets[kv.first] = std::move(ss);
  }
  out->build();
  return out;
}

}  // namespace goal
