// Newton, nested adjoint and DWR drivers (see driver.cuh).
#include <chrono>

#include "driver.cuh"
#include "mpnn.cuh"

namespace goal {

namespace {

double now() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

__global__ void k_axpy_neg(long long n, double* R) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    R[i] = -R[i];
}
__global__ void k_add(long long n, double* U, const double* du) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    U[i] += du[i];
}
// U = U0 + a du (a line-search trial from the iteration's starting point)
__global__ void k_axpy_from(long long n, double* U, const double* U0, double a, const double* du) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    U[i] = fma(a, du[i], U0[i]);
}

// compensated dot product partials (also used for norms)
__global__ void k_dot_part(long long n, const double* a, const double* b, double* part) {
  KSum acc;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc.add(a[i] * b[i]);
  acc = block_reduce(acc);
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = acc.s; part[2 * blockIdx.x + 1] = acc.c; }
}
__global__ void k_ksum_fin(const double* part, int nb, double* out) {
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

// new node N0+k of the nested mesh = average of its edge's end points
// (Nested::set_coarse, src/goal_nested.cpp:369-393)
__global__ void k_prolong(int N0, int Ne, const int* edges, const double* src, double* dst, int copy_old) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * (N0 + Ne); i += gridDim.x * blockDim.x) {
    int n = i >> 2, q = i & 3;
    if (n < N0) {
      if (copy_old) dst[i] = src[i];
    } else {
      int k = n - N0;
      dst[i] = (src[4 * edges[2 * k] + q] + src[4 * edges[2 * k + 1] + q]) * 0.5;
    }
  }
}

// child = parent for every state field (SoA, colour order on both meshes)
__global__ void k_child_states(int Ec, int Eb, const int* c_orig, const int* b_pos, const double* bsig,
                               const double* bFp, const double* bFpo, const double* beq, const double* beqo,
                               const double* bC, double* sig, double* Fp, double* Fpo, double* eq, double* eqo,
                               double* C) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < Ec; s += gridDim.x * blockDim.x) {
    int sb = b_pos[c_orig[s] >> 3];
    for (int q = 0; q < 9; ++q) {
      sig[(long long)q * Ec + s] = bsig[(long long)q * Eb + sb];
      Fp[(long long)q * Ec + s] = bFp[(long long)q * Eb + sb];
      Fpo[(long long)q * Ec + s] = bFpo[(long long)q * Eb + sb];
    }
    for (int q = 0; q < 6; ++q) C[(long long)q * Ec + s] = bC[(long long)q * Eb + sb];
    eq[s] = beq[sb];
    eqo[s] = beqo[sb];
  }
}

__global__ void k_sub(long long n, const double* a, const double* b, double* c) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    c[i] = a[i] - b[i];
}

// |sum_d e_u,d + e_p| per vertex (for the bound) and per element at the centroid
// (compute_error, src/goal_error.cpp:7-35), element values in the original order.
__global__ void k_vertex_abs(int N, const double* Re, double* out) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    double t = 0.0;
    t += Re[4 * n];
    t += Re[4 * n + 1];
    t += Re[4 * n + 2];
    t += Re[4 * n + 3];
    out[n] = fabs(t);
  }
}
__global__ void k_elem_error(int E, const int* tets, const int* orig, const double* Re, double* err) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) {
    int v[4];
    for (int a = 0; a < 4; ++a) v[a] = tets[(long long)a * E + s];
    double pu = 0.25 * Re[4 * v[0] + 3];
    for (int a = 1; a < 4; ++a) pu += 0.25 * Re[4 * v[a] + 3];
    double total = 0.0;
    for (int d = 0; d < 3; ++d) {
      double u = 0.25 * Re[4 * v[0] + d];
      for (int a = 1; a < 4; ++a) u += 0.25 * Re[4 * v[a] + d];
      total += u;
    }
    total += pu;
    err[orig[s]] = fabs(total);
  }
}
// base element e = sum of its 8 children (Nested::set_error, src/goal_nested.cpp:395-412)
__global__ void k_children_sum(int Eb, const double* err_nested, double* err_base) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < Eb; e += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < 8; ++k) s += err_nested[8ll * e + k];
    err_base[e] = s;
  }
}

double device_dot(long long n, const double* a, const double* b, DevBuf<double>& red, cudaStream_t st) {
  const int nb = std::min(grid_for(n, 256), 1024);
  if (red.n < 2 * (size_t)nb + 2) red.alloc(2 * nb + 2);
  k_dot_part<<<nb, 256, 0, st>>>(n, a, b, red.ptr);
  GOAL_CHECK_LAUNCH();
  k_ksum_fin<<<1, 1024, 0, st>>>(red.ptr, nb, red.ptr + 2 * nb);
  GOAL_CHECK_LAUNCH();
  double out = 0.0;
  GOAL_CUDA(cudaMemcpyAsync(&out, red.ptr + 2 * nb, sizeof(double), cudaMemcpyDeviceToHost, st));
  GOAL_CUDA(cudaStreamSynchronize(st));
  return out;
}

}  // namespace

BsrView bsr_view(const Disc& d) {
  BsrView v;
  v.num_nodes = d.num_nodes;
  v.nnzb = d.nnzb;
  v.brow_ptr = d.brow_ptr.ptr;
  v.bcol = d.bcol.ptr;
  v.diag = d.diag.ptr;
  return v;
}

SolveStats linear_solve(SolInfo& s, const SolveParams& p, const double* b, double* x, Krylov& K, const double* dD) {
  K.stream = s.disc->stream;
  BsrView A = bsr_view(*s.disc);
  if (has_inner_solve(p.precision)) make_inner_copy(A, s.A.ptr, p.precision, K);
  if (p.precond == PRECOND_LEARNED) {
    GOAL_REQUIRE(s.learned, GOAL_ERR_STATE, "learned preconditioner requested but no network is attached");
    s.learned->stream = K.stream;
    BsrMatrix M{A, s.A.ptr};
    block_jacobi_setup(A, s.A.ptr, nullptr, K);
    mpnn_apply_to_block_jacobi(*s.learned, M, K);
    SolveParams q = p;
    if (p.learned_cap > 0) q.max_iters = std::min(p.max_iters, p.learned_cap);
    SolveStats r = fgmres(A, s.A.ptr, b, x, q, K);
    if (r.converged || p.learned_cap <= 0 || p.max_iters <= q.max_iters) return r;
    // fall back to plain block-Jacobi, continuing from the current iterate
    block_jacobi_setup(A, s.A.ptr, nullptr, K);
    SolveParams q2 = p;
    q2.max_iters = p.max_iters - r.iters;
    SolveStats r2 = fgmres(A, s.A.ptr, b, x, q2, K);
    r2.iters += r.iters;
    r2.inner_iters += r.inner_iters;
    r2.spmv64 += r.spmv64;
    r2.spmv32 += r.spmv32;
    r2.seconds += r.seconds;
    r2.fell_back = 1;
    return r2;
  }
  int sing = block_jacobi_setup(A, s.A.ptr, dD, K);
  (void)sing;  // singular blocks fall back to identity blocks
  return fgmres(A, s.A.ptr, b, x, p, K);
}

NewtonStats primal_solve(Mechanics& m, SolInfo& s, const std::vector<DBC>& dbcs, const std::vector<TBC>& tbcs,
                         double t_now, double t_old, const NewtonParams& p, Krylov& K) {
  (void)t_old;
  NewtonStats out;
  cudaStream_t st = m.disc->stream;
  K.stream = st;
  const long long n = 4ll * m.disc->num_nodes;
  DevBuf<double> du, U0;
  du.alloc(n);
  if (p.line_search > 0) U0.alloc(n);
  int iter = 1;
  bool converged = false;
  Chain cr;
  cr.mode = MODE_PRIMAL;
  cr.jacobian = 0;
  cr.save_states = 1;
  auto residual_norm = [&]() {
    assemble(m, &s, cr, nullptr, st);
    apply_tbcs(m, s, tbcs, t_now, nullptr, st);
    apply_dbcs(m, s, dbcs, t_now, false, st);
    return std::sqrt(device_dot(n, s.R.ptr, s.R.ptr, m.red, st));
  };
  while (iter <= p.max_iters && !converged) {
    double t0 = now();
    Chain cj;
    cj.mode = MODE_PRIMAL;
    cj.jacobian = 1;
    cj.save_states = 1;
    assemble(m, &s, cj, nullptr, st);
    apply_tbcs(m, s, tbcs, t_now, nullptr, st);
    apply_dbcs(m, s, dbcs, t_now, true, st);
    // ||R|| at the iteration's starting point (the line search's reference)
    const double norm0 = p.line_search > 0 ? std::sqrt(device_dot(n, s.R.ptr, s.R.ptr, m.red, st)) : 0.0;
    k_axpy_neg<<<grid_for(n, 256), 256, 0, st>>>(n, s.R.ptr);
    GOAL_CHECK_LAUNCH();
    du.zero(st);
    double t1 = now();
    SolveStats ls = linear_solve(s, p.lin, s.R.ptr, du.ptr, K);
    out.linear_iters += ls.iters;
    out.inner_iters += ls.inner_iters;
    out.last = ls;
    double t2 = now();
    double norm = 0.0;
    if (p.line_search > 0) {
      GOAL_CUDA(cudaMemcpyAsync(U0.ptr, m.U.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      double a = 1.0;
      for (int h = 0;; ++h) {
        k_axpy_from<<<grid_for(n, 256), 256, 0, st>>>(n, m.U.ptr, U0.ptr, a, du.ptr);
        GOAL_CHECK_LAUNCH();
        norm = residual_norm();
        if (norm < (1.0 - 1e-4 * a) * norm0 || h >= p.line_search) break;
        a *= 0.5;
        out.backtracks++;
      }
    } else {
      k_add<<<grid_for(n, 256), 256, 0, st>>>(n, m.U.ptr, du.ptr);
      GOAL_CHECK_LAUNCH();
      norm = residual_norm();
    }
    double t3 = now();
    out.seconds_assembly += (t1 - t0) + (t3 - t2);
    out.seconds_solve += t2 - t1;
    if (iter - 1 < 32) out.norms[iter - 1] = norm;
    out.iters = iter;
    if (norm < p.tolerance) converged = true;
    iter++;
  }
  out.converged = converged ? 1 : 0;
  return out;
}

void NestedAdjoint::build(Mechanics& base_mech) {
  base = &base_mech;
  disc = refine_uniform(*base_mech.disc);
  mech = std::make_unique<Mechanics>();
  mech->disc = disc.get();
  mech->model = base_mech.model;
  mech->stabilization = base_mech.stabilization;
  mech->fp_reset = base_mech.fp_reset;
  mech->mats_h = base_mech.mats_h;
  mech->init();
  si = std::make_unique<SolInfo>();
  si->init(disc.get());
  const long long n = 4ll * disc->num_nodes;
  z.alloc(n);
  zc.alloc(n);
  zd.alloc(n);
  err_nested.alloc(disc->num_elems);
  err_base.alloc(base_mech.disc->num_elems);
  tmp.alloc(std::max<long long>(n, disc->num_nodes));
  K.stream = disc->stream;
}

void NestedAdjoint::refresh() {
  base->materialize_fp();  // the children copy Fp
  const Disc& b = *base->disc;
  Disc& d = *disc;
  cudaStream_t st = d.stream;
  const int Ne = d.num_nodes - d.base_nodes;
  k_prolong<<<grid_for(4ll * d.num_nodes, 256), 256, 0, st>>>(d.base_nodes, Ne, d.parent_edges.ptr, base->U.ptr,
                                                               mech->U.ptr, 1);
  GOAL_CHECK_LAUNCH();
  k_child_states<<<grid_for(d.num_elems, 256), 256, 0, st>>>(
      d.num_elems, b.num_elems, d.elem_orig.ptr, b.elem_pos.ptr, base->st.sigma.ptr, base->st.Fp.ptr,
      base->st.Fp_old.ptr, base->st.eqps.ptr, base->st.eqps_old.ptr, base->st.Cpinv.ptr, mech->st.sigma.ptr,
      mech->st.Fp.ptr, mech->st.Fp_old.ptr, mech->st.eqps.ptr, mech->st.eqps_old.ptr, mech->st.Cpinv.ptr);
  GOAL_CHECK_LAUNCH();
}

DwrResult nested_adjoint_run(NestedAdjoint& a, const std::vector<DBC>& dbcs, const std::vector<TBC>& tbcs, int qoi,
                             double rho, double t_now, double t_old, const SolveParams& p) {
  (void)t_old;
  DwrResult out;
  Disc& d = *a.disc;
  Mechanics& m = *a.mech;
  SolInfo& s = *a.si;
  cudaStream_t st = d.stream;
  const long long n = 4ll * d.num_nodes;
  a.refresh();
  // compute_adjoint: transposed Jacobian, dMdu, R
  double t0 = now();
  Chain ca;
  ca.mode = MODE_ADJOINT;
  ca.jacobian = 1;
  ca.save_states = 0;
  ca.qoi = qoi;
  ca.rho = rho;
  out.qoi = assemble(m, &s, ca, nullptr, st);
  apply_tbcs(m, s, tbcs, t_now, nullptr, st);
  apply_dbcs(m, s, dbcs, t_now, true, st);
  GOAL_CUDA(cudaStreamSynchronize(st));
  double t1 = now();
  // solve dRdu^T z = dMdu
  a.z.zero(st);
  out.solve = linear_solve(s, p, s.dMdu.ptr, a.z.ptr, a.K);
  double t2 = now();
  // z_coarse: interpolant from the parent vertices; z_diff = z - z_coarse
  k_prolong<<<grid_for(n, 256), 256, 0, st>>>(d.base_nodes, d.num_nodes - d.base_nodes, d.parent_edges.ptr, a.z.ptr,
                                               a.zc.ptr, 1);
  GOAL_CHECK_LAUNCH();
  k_sub<<<grid_for(n, 256), 256, 0, st>>>(n, a.z.ptr, a.zc.ptr, a.zd.ptr);
  GOAL_CHECK_LAUNCH();
  out.eta = -device_dot(n, s.R.ptr, a.z.ptr, m.red, st);
  // localize: error chain with the DWR weights
  Chain ce;
  ce.mode = MODE_PRIMAL;
  ce.jacobian = 0;
  ce.save_states = 0;
  ce.error_chain = 1;
  ErrorWeights w;
  w.Zd = a.zd.ptr;
  w.Zc = a.zc.ptr;
  assemble(m, &s, ce, &w, st);
  apply_tbcs(m, s, tbcs, t_now, a.zd.ptr, st);
  apply_dbcs(m, s, dbcs, t_now, false, st);
  k_vertex_abs<<<grid_for(d.num_nodes, 256), 256, 0, st>>>(d.num_nodes, s.R.ptr, a.tmp.ptr);
  GOAL_CHECK_LAUNCH();
  DevBuf<double> ones;
  ones.alloc(d.num_nodes);
  std::vector<double> h1(d.num_nodes, 1.0);
  ones.upload(h1.data(), h1.size(), st);
  out.bound = device_dot(d.num_nodes, a.tmp.ptr, ones.ptr, m.red, st);
  k_elem_error<<<grid_for(d.num_elems, 256), 256, 0, st>>>(d.num_elems, d.tets.ptr, d.elem_orig.ptr, s.R.ptr,
                                                           a.err_nested.ptr);
  GOAL_CHECK_LAUNCH();
  k_children_sum<<<grid_for(d.base_elems, 256), 256, 0, st>>>(d.base_elems, a.err_nested.ptr, a.err_base.ptr);
  GOAL_CHECK_LAUNCH();
  GOAL_CUDA(cudaStreamSynchronize(st));
  double t3 = now();
  out.seconds_adjoint = t1 - t0;
  out.seconds_solve = t2 - t1;
  out.seconds_localize = t3 - t2;
  return out;
}

}  // namespace goal
