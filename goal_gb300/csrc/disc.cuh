// Discretization on the device: mesh, DOF numbering, block graph, element
// colouring and per-element geometry (the GB300 counterpart of goal::Disc,
// src/goal_disc.hpp:26-98).
//
// Layout in HBM (E elements, N nodes, nnzb 4x4 blocks):
//   coords     N x 3 f64                      node coordinates
//   tets       4 x E i32 (SoA, colour order)  element nodes
//   grads      12 x E f64 (SoA, colour order) shape-function gradients dphi_a/dx_k
//   vol, h     E f64                          signed volume (weight x detJ), rms edge length
//   blk        16 x E i32 (SoA)               BSR block index of node pair (a,b) of the element
//   first      E u32                          bit 4a+b: element is the first writer of block (a,b)
//                                             in colour order; bit 16+a: first writer of node a
//   brow_ptr   N+1 i32, bcol nnzb i32         block graph (node adjacency incl. self, sorted)
//   color_ptr  num_colors+1                   elements of colour c are [color_ptr[c], color_ptr[c+1])
// DOF numbering is lid = node*4 + eq (src/goal_disc.cpp:195-201); the scalar
// CSR graph of the reference (src/goal_disc.cpp:307-332) is the block graph
// expanded by 4x4 and is produced on demand by csr_graph().
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "common.cuh"

namespace goal {

constexpr int kNeq = 4;        // num_eqs = num_dims + 1 (src/goal_disc.cpp:260)
constexpr int kMaxColors = 128;
constexpr int kMaxNodeElems = 128;  // incident elements per node supported by the graph build

struct DiscView {
  int num_nodes, num_elems, nnzb;
  const double* coords;
  const int* tets;
  const double* grads;
  const double* vol;
  const double* h;
  const int* blk;
  const unsigned* first;
  const int* brow_ptr;
  const int* bcol;
  const int* diag;
  const int* elem_set;   // colour order
  const int* elem_orig;  // colour order -> original element id
};

struct NodeSet {
  std::string name;
  std::vector<int> host;
  DevBuf<int> dev;
};

struct SideSet {
  std::string name;
  std::vector<int> tris;          // S x 3 (host)
  DevBuf<int> dtris;              // S x 3
  // node-centric incidence for a deterministic, atomic-free traction scatter
  std::vector<int> nodes_h;       // unique nodes touched
  DevBuf<int> nodes;
  DevBuf<int> inc_ptr;            // per touched node: range into inc
  DevBuf<int> inc;                // side id (S x 3 incidences, side*3 + local)
};

struct Disc {
  int num_nodes = 0, num_elems = 0, num_elem_sets = 1;
  long long nnz = 0;     // scalar nonzeros (16 x nnzb)
  int nnzb = 0, num_colors = 0;
  std::vector<int> color_ptr;  // host copy
  // wall seconds of build()'s phases: node graph (upload, incidence sort,
  // block graph), colouring (Jones-Plassmann rounds), layout (colour-major
  // order, block slots, geometry), contribution lists, node and side sets
  double build_seconds[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  int color_rounds = 0;
  cudaStream_t stream = nullptr;

  // host copies of the input (original element order)
  std::vector<double> coords_h;
  std::vector<int> tets_h, elem_set_h;

  DevBuf<double> coords;
  DevBuf<int> tets, elem_set, elem_orig, elem_pos;  // elem_pos: original -> colour order
  DevBuf<double> grads, vol, h;
  DevBuf<int> blk, brow_ptr, bcol, diag;
  DevBuf<unsigned> first;
  DevBuf<int> color;  // colour per element (colour order)
  // contribution lists of the two-phase (element buffer + gather) assembly:
  // block k of the matrix sums element blocks blist[bptr[k]..bptr[k+1]) with
  // entries 16*s + (4a+b); node n sums element rows nlist[nptr[n]..nptr[n+1])
  // with entries 4*s + a. Both are ordered by element, so sums are deterministic.
  DevBuf<int> bptr, blist, nptr, nlist;
  // off-diagonal block ids (nnzb - N), so that the gather can treat the
  // diagonal blocks (many contributions) apart from the others (few)
  DevBuf<int> offd;

  std::map<std::string, std::unique_ptr<NodeSet>> node_sets;
  std::map<std::string, std::unique_ptr<SideSet>> side_sets;
  std::vector<std::string> elem_set_names;
  bool built = false;

  // nested-mesh bookkeeping (Nested, src/goal_nested.hpp)
  int base_nodes = 0;          // nodes of the base mesh (new nodes follow)
  DevBuf<int> parent_edges;    // (num_nodes - base_nodes) x 2: edge end points of new nodes
  int base_elems = 0;          // children of base element e are 8e..8e+7 (original order)

  // the scalar CSR graph kept on the device (4N+1 row pointers, nnz columns),
  // built on the first request for device pointers
  DevBuf<int> csr_row_ptr, csr_col_idx;
  // btr[k]: index of block (m, n) for block k = (n, m); built by the first
  // transposed (ADJOINT) assembly
  DevBuf<int> btr;

  void build();                // Disc::build_data: graph, colouring, geometry
  DiscView view() const;
  void csr_graph(int* row_ptr, int* col_idx) const;  // host outputs
  void csr_graph_device();     // fills csr_row_ptr / csr_col_idx once
  void block_transpose_map();  // fills btr once
};

// Builds the uniformly refined nested mesh of ``base`` on the device
// (declared rule: new node N+k at the midpoint of edge k of the upper-triangular
// node graph; children 8e..8e+7 = four corner tets then the octahedron split on
// its shortest diagonal). Node sets and side sets are refined with it.
std::unique_ptr<Disc> refine_uniform(const Disc& base);

}  // namespace goal
