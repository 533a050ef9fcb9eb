// C ABI (include/goal_gb300.h): handles over Disc, Mechanics, SolInfo and the
// boundary conditions, with host<->device layout conversions.
#include <cstring>
#include <memory>
#include <string>

#include "../../include/goal_gb300.h"
#include "capi_internal.cuh"
#include "driver.cuh"
#include "mpnn.cuh"
#include "size_field.cuh"

namespace goal {

std::atomic<long long> g_launches{0};
static thread_local std::string t_last_error;
void set_last_error(const std::string& msg) { t_last_error = msg; }

namespace {

__global__ void k_soa_to_orig(int E, int nc, const double* soa, const int* orig, double* out) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) {
    int e = orig[s];
    for (int q = 0; q < nc; ++q) out[(size_t)e * nc + q] = soa[(size_t)q * E + s];
  }
}
__global__ void k_orig_to_soa(int E, int nc, const double* in, const int* orig, double* soa) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) {
    int e = orig[s];
    for (int q = 0; q < nc; ++q) soa[(size_t)q * E + s] = in[(size_t)e * nc + q];
  }
}
__global__ void k_bsr_to_csr(int N, const int* brow_ptr, const double* A, double* csr) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    int b0 = brow_ptr[n], deg = brow_ptr[n + 1] - b0;
    for (int k = b0; k < b0 + deg; ++k)
      for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) csr[16ll * b0 + 4ll * r * deg + 4ll * (k - b0) + c] = A[16ll * k + 4 * r + c];
  }
}
__global__ void k_colors_orig(int E, const int* color, const int* orig, int* out) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) out[orig[s]] = color[s];
}

}  // namespace

void states_to_host(Mechanics& m, int which, double* out) {
  const Disc& d = *m.disc;
  if (which == GOAL_STATE_FP) m.materialize_fp();
  const int E = d.num_elems;
  const double* src = nullptr;
  int nc = 9;
  switch (which) {
    case GOAL_STATE_SIGMA: src = m.st.sigma.ptr; break;
    case GOAL_STATE_FP: src = m.st.Fp.ptr; break;
    case GOAL_STATE_FP_OLD: src = m.st.Fp_old.ptr; break;
    case GOAL_STATE_EQPS: src = m.st.eqps.ptr; nc = 1; break;
    case GOAL_STATE_EQPS_OLD: src = m.st.eqps_old.ptr; nc = 1; break;
    default: throw Error(GOAL_ERR_ARG, "unknown state field");
  }
  DevBuf<double> tmp;
  tmp.alloc((size_t)nc * E);
  k_soa_to_orig<<<grid_for(E, 256), 256, 0, d.stream>>>(E, nc, src, d.elem_orig.ptr, tmp.ptr);
  GOAL_CHECK_LAUNCH();
  tmp.download(out, d.stream);
  GOAL_CUDA(cudaStreamSynchronize(d.stream));
}

void states_from_host(Mechanics& m, int which, const double* in) {
  const Disc& d = *m.disc;
  // pending plastic writes were formed with the current Fp_old: form them
  // before any state changes (a new Fp replaces them)
  m.materialize_fp();
  const int E = d.num_elems;
  double* dst = nullptr;
  int nc = 9;
  switch (which) {
    case GOAL_STATE_SIGMA: dst = m.st.sigma.ptr; break;
    case GOAL_STATE_FP: dst = m.st.Fp.ptr; break;
    case GOAL_STATE_FP_OLD: dst = m.st.Fp_old.ptr; break;
    case GOAL_STATE_EQPS: dst = m.st.eqps.ptr; nc = 1; break;
    case GOAL_STATE_EQPS_OLD: dst = m.st.eqps_old.ptr; nc = 1; break;
    default: throw Error(GOAL_ERR_ARG, "unknown state field");
  }
  DevBuf<double> tmp;
  tmp.upload(in, (size_t)nc * E, d.stream);
  k_orig_to_soa<<<grid_for(E, 256), 256, 0, d.stream>>>(E, nc, tmp.ptr, d.elem_orig.ptr, dst);
  GOAL_CHECK_LAUNCH();
  if (which == GOAL_STATE_FP_OLD) m.refresh_cpinv();
  GOAL_CUDA(cudaStreamSynchronize(d.stream));
}

void bsr_to_csr(const SolInfo& s, double* out_host) {
  const Disc& d = *s.disc;
  DevBuf<double> tmp;
  tmp.alloc(d.nnz);
  k_bsr_to_csr<<<grid_for(d.num_nodes, 128), 128, 0, d.stream>>>(d.num_nodes, d.brow_ptr.ptr, s.A.ptr, tmp.ptr);
  GOAL_CHECK_LAUNCH();
  tmp.download(out_host, d.stream);
  GOAL_CUDA(cudaStreamSynchronize(d.stream));
}

}  // namespace goal

using namespace goal;

struct goal_disc_s {
  std::unique_ptr<Disc> d;
  bool owns_stream = false;
  ~goal_disc_s() {
    cudaStream_t s = d ? d->stream : nullptr;
    d.reset();
    if (owns_stream && s) cudaStreamDestroy(s);
  }
};
struct goal_mechanics_s {
  std::unique_ptr<Mechanics> m;
  DevBuf<double> Zd, Zc;
};
struct goal_sol_info_s {
  std::unique_ptr<SolInfo> s;
};
struct goal_bcs_s {
  Disc* d = nullptr;
  std::vector<DBC> dbcs;
  std::vector<TBC> tbcs;
};
struct goal_learned_s {
  Mpnn net;
  cudaStream_t stream = nullptr;
  ~goal_learned_s() {
    if (stream) cudaStreamDestroy(stream);
  }
};
struct goal_nested_adjoint_s {
  NestedAdjoint a;
  goal_disc_s disc_view;      // non-owning views handed to goal_nested_adjoint_disc / _sol_info
  goal_sol_info_s si_view;
  ~goal_nested_adjoint_s() {
    disc_view.d.release();
    si_view.s.release();
  }
};

static SolveParams to_params(const goal_solve_params* p) {
  SolveParams q;
  if (p) {
    q.krylov_size = p->krylov_size;
    q.max_iters = p->max_iters;
    q.tolerance = p->tolerance;
    q.precision = p->precision;
    q.inner_iters = p->inner_iters;
    q.precond = p->precond;
    q.learned_cap = p->learned_cap;
  }
  GOAL_REQUIRE(q.krylov_size >= 1 && q.krylov_size < 256, GOAL_ERR_ARG, "krylov size must be in [1, 255]");
  GOAL_REQUIRE(q.max_iters >= 1, GOAL_ERR_ARG, "max iters must be >= 1");
  GOAL_REQUIRE(q.tolerance > 0.0, GOAL_ERR_ARG, "tolerance must be > 0");
  GOAL_REQUIRE(q.precision >= PREC_FP64 && q.precision <= PREC_NESTED_F64, GOAL_ERR_ARG, "unknown precision mode");
  GOAL_REQUIRE(!has_inner_solve(q.precision) || (q.inner_iters >= 1 && q.inner_iters < 256), GOAL_ERR_ARG,
               "inner iterations must be in [1, 255]");
  return q;
}

static void to_stats(const SolveStats& s, goal_solve_stats* o) {
  if (!o) return;
  o->iters = s.iters;
  o->inner_iters = s.inner_iters;
  o->converged = s.converged;
  o->fell_back = s.fell_back;
  o->rel_res = s.rel_res;
  o->seconds = s.seconds;
  o->spmv64 = s.spmv64;
  o->spmv32 = s.spmv32;
}

#define GOAL_API_BEGIN try {
#define GOAL_API_END                                      \
  }                                                       \
  catch (const goal::Error& e) {                          \
    goal::set_last_error(e.what());                       \
    return e.code;                                        \
  }                                                       \
  catch (const std::exception& e) {                       \
    goal::set_last_error(e.what());                       \
    return GOAL_ERR_STATE;                                \
  }                                                       \
  return GOAL_OK;

#define GOAL_ARG(cond, msg) GOAL_REQUIRE(cond, GOAL_ERR_ARG, msg)

extern "C" {

const char* goal_last_error(void) { return t_last_error.c_str(); }

int goal_assembly_timing(int enable) {
  GOAL_API_BEGIN
  goal::assembly_timing(enable != 0);
  GOAL_API_END
}

int goal_set_element_buffer_limit(long long bytes) {
  GOAL_API_BEGIN
  GOAL_ARG(bytes >= 0, "goal_set_element_buffer_limit: negative size");
  goal::set_element_buffer_limit(bytes);
  GOAL_API_END
}

int goal_assembly_timing_read(double* ms, long long* count) {
  GOAL_API_BEGIN
  GOAL_ARG(ms && count, "null argument");
  goal::assembly_timing_read(ms, count);
  GOAL_API_END
}

long long goal_launch_count(void) { return g_launches.load(); }

int goal_eval(const char* expr, double x, double y, double z, double t, double* out) {
  GOAL_API_BEGIN
  GOAL_ARG(expr && out, "goal_eval: null argument");
  ExprCode c;
  std::string err;
  GOAL_REQUIRE(compile_expr(expr, c, err), GOAL_ERR_ARG, err);
  *out = eval_expr(c, x, y, z, t);
  GOAL_API_END
}

int goal_disc_create(int num_nodes, int num_elems, const double* coords, const int* tets, const int* elem_set,
                     int num_elem_sets, goal_disc* out) {
  GOAL_API_BEGIN
  GOAL_ARG(out && coords && tets && num_nodes > 0 && num_elems > 0, "goal_disc_create: bad arguments");
  GOAL_ARG(num_elem_sets >= 1, "goal_disc_create: need at least one element set");
  for (long long i = 0; i < 4ll * num_elems; ++i)
    GOAL_ARG(tets[i] >= 0 && tets[i] < num_nodes, "goal_disc_create: tet node out of range");
  auto h = std::make_unique<goal_disc_s>();
  h->d = std::make_unique<Disc>();
  Disc& d = *h->d;
  GOAL_CUDA(cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking));
  h->owns_stream = true;
  d.num_nodes = num_nodes;
  d.num_elems = num_elems;
  d.num_elem_sets = num_elem_sets;
  d.coords_h.assign(coords, coords + 3ll * num_nodes);
  d.tets_h.assign(tets, tets + 4ll * num_elems);
  if (elem_set) {
    d.elem_set_h.assign(elem_set, elem_set + num_elems);
    for (int e : d.elem_set_h) GOAL_ARG(e >= 0 && e < num_elem_sets, "goal_disc_create: element set out of range");
  } else {
    d.elem_set_h.assign(num_elems, 0);
  }
  *out = h.release();
  GOAL_API_END
}

int goal_disc_add_node_set(goal_disc d, const char* name, int n, const int* nodes) {
  GOAL_API_BEGIN
  GOAL_ARG(d && name && (n == 0 || nodes), "goal_disc_add_node_set: bad arguments");
  auto ns = std::make_unique<NodeSet>();
  ns->name = name;
  ns->host.assign(nodes, nodes + n);
  for (int v : ns->host) GOAL_ARG(v >= 0 && v < d->d->num_nodes, "node set: node out of range");
  if (d->d->built) ns->dev.upload(ns->host.data(), ns->host.size(), d->d->stream);
  d->d->node_sets[name] = std::move(ns);
  GOAL_API_END
}

int goal_disc_add_side_set(goal_disc d, const char* name, int n, const int* tris) {
  GOAL_API_BEGIN
  GOAL_ARG(d && name && (n == 0 || tris) && !d->d->built, "goal_disc_add_side_set: bad arguments (add before build)");
  auto ss = std::make_unique<SideSet>();
  ss->name = name;
  ss->tris.assign(tris, tris + 3ll * n);
  for (int v : ss->tris) GOAL_ARG(v >= 0 && v < d->d->num_nodes, "side set: node out of range");
  d->d->side_sets[name] = std::move(ss);
  GOAL_API_END
}

int goal_disc_build_data(goal_disc d) {
  GOAL_API_BEGIN
  GOAL_ARG(d, "null disc");
  d->d->build();
  GOAL_API_END
}

int goal_disc_sizes(goal_disc d, long long* sizes) {
  GOAL_API_BEGIN
  GOAL_ARG(d && sizes, "null argument");
  const Disc& x = *d->d;
  sizes[0] = x.num_nodes;
  sizes[1] = x.num_elems;
  sizes[2] = 4ll * x.num_nodes;
  sizes[3] = x.nnz;
  sizes[4] = x.nnzb;
  sizes[5] = x.num_colors;
  GOAL_API_END
}

int goal_disc_build_times(goal_disc d, double* seconds, int* color_rounds) {
  GOAL_API_BEGIN
  GOAL_ARG(d && seconds && color_rounds && d->d->built, "goal_disc_build_times: disc not built");
  for (int k = 0; k < 5; ++k) seconds[k] = d->d->build_seconds[k];
  *color_rounds = d->d->color_rounds;
  GOAL_API_END
}

int goal_disc_get_graph(goal_disc d, int* row_ptr, int* col_idx) {
  GOAL_API_BEGIN
  GOAL_ARG(d && row_ptr && col_idx && d->d->built, "goal_disc_get_graph: disc not built");
  d->d->csr_graph(row_ptr, col_idx);
  GOAL_API_END
}

int goal_disc_get_mesh(goal_disc d, double* coords, int* tets, int* elem_set) {
  GOAL_API_BEGIN
  GOAL_ARG(d, "null disc");
  const Disc& x = *d->d;
  if (coords) std::memcpy(coords, x.coords_h.data(), sizeof(double) * x.coords_h.size());
  if (tets) std::memcpy(tets, x.tets_h.data(), sizeof(int) * x.tets_h.size());
  if (elem_set) std::memcpy(elem_set, x.elem_set_h.data(), sizeof(int) * x.elem_set_h.size());
  GOAL_API_END
}

int goal_disc_get_colors(goal_disc d, int* colors) {
  GOAL_API_BEGIN
  GOAL_ARG(d && colors && d->d->built, "goal_disc_get_colors: disc not built");
  const Disc& x = *d->d;
  DevBuf<int> tmp;
  tmp.alloc(x.num_elems);
  k_colors_orig<<<grid_for(x.num_elems, 256), 256, 0, x.stream>>>(x.num_elems, x.color.ptr, x.elem_orig.ptr, tmp.ptr);
  GOAL_CHECK_LAUNCH();
  tmp.download(colors, x.stream);
  GOAL_CUDA(cudaStreamSynchronize(x.stream));
  GOAL_API_END
}

int goal_disc_stream(goal_disc d, void** stream) {
  GOAL_API_BEGIN
  GOAL_ARG(d && stream, "null argument");
  *stream = (void*)d->d->stream;
  GOAL_API_END
}

int goal_disc_device_graph(goal_disc d, const int** brow_ptr, const int** bcol, const int** row_ptr,
                           const int** col_idx) {
  GOAL_API_BEGIN
  GOAL_ARG(d && d->d->built, "goal_disc_device_graph: disc not built");
  if (brow_ptr) *brow_ptr = d->d->brow_ptr.ptr;
  if (bcol) *bcol = d->d->bcol.ptr;
  if (row_ptr || col_idx) {
    d->d->csr_graph_device();
    if (row_ptr) *row_ptr = d->d->csr_row_ptr.ptr;
    if (col_idx) *col_idx = d->d->csr_col_idx.ptr;
  }
  GOAL_API_END
}

int goal_disc_destroy(goal_disc d) {
  GOAL_API_BEGIN
  delete d;
  GOAL_API_END
}

int goal_nested_create(goal_disc base, goal_disc* out) {
  GOAL_API_BEGIN
  GOAL_ARG(base && out && base->d->built, "goal_nested_create: base not built");
  auto h = std::make_unique<goal_disc_s>();
  h->d = refine_uniform(*base->d);
  h->owns_stream = false;
  *out = h.release();
  GOAL_API_END
}

int goal_size_field(goal_disc d, const double* elem_error, int target, double* vtx_size) {
  GOAL_API_BEGIN
  GOAL_ARG(d && elem_error && vtx_size && d->d->built, "goal_size_field: null argument or disc not built");
  GOAL_ARG(target > 0, "goal_size_field: target elements must be positive");
  Disc& D = *d->d;
  DevBuf<double> err, out;
  err.upload(elem_error, D.num_elems, D.stream);
  out.alloc(D.num_nodes);
  iso_target_size(D, err.ptr, target, out.ptr, D.stream);
  out.download(vtx_size, D.stream);
  GOAL_CUDA(cudaStreamSynchronize(D.stream));
  GOAL_API_END
}

int goal_nested_parent_edges(goal_disc nested, int* edges) {
  GOAL_API_BEGIN
  GOAL_ARG(nested && edges && nested->d->base_nodes > 0, "goal_nested_parent_edges: not a nested disc");
  nested->d->parent_edges.download(edges, nested->d->stream);
  GOAL_CUDA(cudaStreamSynchronize(nested->d->stream));
  GOAL_API_END
}

int goal_mechanics_create(goal_disc d, int model, const double* materials, int stabilization, goal_mechanics* out) {
  GOAL_API_BEGIN
  GOAL_ARG(d && materials && out && d->d->built, "goal_mechanics_create: bad arguments (disc must be built)");
  GOAL_ARG(model == GOAL_MODEL_NEOHOOKEAN || model == GOAL_MODEL_J2, "unknown model");
  auto h = std::make_unique<goal_mechanics_s>();
  h->m = std::make_unique<Mechanics>();
  Mechanics& m = *h->m;
  m.disc = d->d.get();
  m.model = model;
  m.stabilization = stabilization != 0;
  for (int k = 0; k < m.disc->num_elem_sets; ++k) {
    MaterialRow r{materials[5 * k], materials[5 * k + 1], materials[5 * k + 2], materials[5 * k + 3],
                  materials[5 * k + 4]};
    GOAL_ARG(r.E > 0 && r.nu > -1.0 && r.nu < 0.5, "material: need E > 0 and -1 < nu < 0.5");
    if (model == GOAL_MODEL_J2) GOAL_ARG(r.Y > 0, "J2 material: need Y > 0");
    m.mats_h.push_back(r);
  }
  m.init();
  GOAL_CUDA(cudaStreamSynchronize(m.disc->stream));
  *out = h.release();
  GOAL_API_END
}

int goal_mechanics_set_solution(goal_mechanics m, const double* U) {
  GOAL_API_BEGIN
  GOAL_ARG(m && U, "null argument");
  m->m->U.upload(U, 4ll * m->m->disc->num_nodes, m->m->disc->stream);
  GOAL_CUDA(cudaStreamSynchronize(m->m->disc->stream));
  GOAL_API_END
}

int goal_mechanics_get_solution(goal_mechanics m, double* U) {
  GOAL_API_BEGIN
  GOAL_ARG(m && U, "null argument");
  m->m->U.download(U, m->m->disc->stream);
  GOAL_CUDA(cudaStreamSynchronize(m->m->disc->stream));
  GOAL_API_END
}

int goal_mechanics_set_fp_reset(goal_mechanics m, int on) {
  GOAL_API_BEGIN
  GOAL_ARG(m, "goal_mechanics_set_fp_reset: null handle");
  m->m->fp_reset = on != 0;
  GOAL_API_END
}

int goal_mechanics_set_line_search(goal_mechanics m, int max_halvings) {
  GOAL_API_BEGIN
  GOAL_ARG(m && max_halvings >= 0 && max_halvings <= 30, "goal_mechanics_set_line_search: bad arguments");
  m->m->line_search = max_halvings;
  GOAL_API_END
}

int goal_mechanics_device_solution(goal_mechanics m, double** U) {
  GOAL_API_BEGIN
  GOAL_ARG(m && U, "goal_mechanics_device_solution: null argument");
  *U = m->m->U.ptr;
  GOAL_API_END
}

int goal_mechanics_set_weights(goal_mechanics m, const double* z_diff, const double* z_coarse) {
  GOAL_API_BEGIN
  GOAL_ARG(m && z_diff && z_coarse, "null argument");
  size_t n = 4ll * m->m->disc->num_nodes;
  m->Zd.upload(z_diff, n, m->m->disc->stream);
  m->Zc.upload(z_coarse, n, m->m->disc->stream);
  GOAL_CUDA(cudaStreamSynchronize(m->m->disc->stream));
  GOAL_API_END
}

int goal_states_set(goal_mechanics m, int which, const double* values) {
  GOAL_API_BEGIN
  GOAL_ARG(m && values, "null argument");
  states_from_host(*m->m, which, values);
  GOAL_API_END
}

int goal_states_get(goal_mechanics m, int which, double* values) {
  GOAL_API_BEGIN
  GOAL_ARG(m && values, "null argument");
  states_to_host(*m->m, which, values);
  GOAL_API_END
}

int goal_states_update(goal_mechanics m) {
  GOAL_API_BEGIN
  GOAL_ARG(m, "null argument");
  m->m->update_states();
  GOAL_CUDA(cudaStreamSynchronize(m->m->disc->stream));
  GOAL_API_END
}

int goal_mechanics_destroy(goal_mechanics m) {
  GOAL_API_BEGIN
  delete m;
  GOAL_API_END
}

int goal_sol_info_create(goal_disc d, goal_sol_info* out) {
  GOAL_API_BEGIN
  GOAL_ARG(d && out && d->d->built, "goal_sol_info_create: disc not built");
  auto h = std::make_unique<goal_sol_info_s>();
  h->s = std::make_unique<SolInfo>();
  h->s->init(d->d.get());
  GOAL_CUDA(cudaStreamSynchronize(d->d->stream));
  *out = h.release();
  GOAL_API_END
}

int goal_sol_info_zero_all(goal_sol_info s) {
  GOAL_API_BEGIN
  GOAL_ARG(s, "null argument");
  cudaStream_t st = s->s->disc->stream;
  s->s->R.zero(st);
  s->s->dMdu.zero(st);
  s->s->A.zero(st);
  GOAL_CUDA(cudaStreamSynchronize(st));
  GOAL_API_END
}

int goal_sol_info_get_vector(goal_sol_info s, int which, double* values) {
  GOAL_API_BEGIN
  GOAL_ARG(s && values && (which == GOAL_VEC_R || which == GOAL_VEC_DMDU), "bad arguments");
  cudaStream_t st = s->s->disc->stream;
  (which == GOAL_VEC_R ? s->s->R : s->s->dMdu).download(values, st);
  GOAL_CUDA(cudaStreamSynchronize(st));
  GOAL_API_END
}

int goal_sol_info_set_vector(goal_sol_info s, int which, const double* values) {
  GOAL_API_BEGIN
  GOAL_ARG(s && values && (which == GOAL_VEC_R || which == GOAL_VEC_DMDU), "bad arguments");
  cudaStream_t st = s->s->disc->stream;
  DevBuf<double>& b = (which == GOAL_VEC_R ? s->s->R : s->s->dMdu);
  b.upload(values, b.n, st);
  GOAL_CUDA(cudaStreamSynchronize(st));
  GOAL_API_END
}

int goal_sol_info_get_dRdu_csr(goal_sol_info s, double* values) {
  GOAL_API_BEGIN
  GOAL_ARG(s && values, "null argument");
  bsr_to_csr(*s->s, values);
  GOAL_API_END
}

int goal_sol_info_get_dRdu_bsr(goal_sol_info s, double* values) {
  GOAL_API_BEGIN
  GOAL_ARG(s && values, "null argument");
  cudaStream_t st = s->s->disc->stream;
  s->s->A.download(values, st);
  GOAL_CUDA(cudaStreamSynchronize(st));
  GOAL_API_END
}

int goal_sol_info_device_view(goal_sol_info s, double** R, double** dMdu, double** bsr_vals) {
  GOAL_API_BEGIN
  GOAL_ARG(s, "goal_sol_info_device_view: null handle");
  if (R) *R = s->s->R.ptr;
  if (dMdu) *dMdu = s->s->dMdu.ptr;
  if (bsr_vals) *bsr_vals = s->s->A.ptr;
  GOAL_API_END
}

int goal_sol_info_device_csr(goal_sol_info s, double** csr_vals) {
  GOAL_API_BEGIN
  GOAL_ARG(s && csr_vals, "goal_sol_info_device_csr: null argument");
  const Disc& d = *s->s->disc;
  GOAL_REQUIRE(d.nnz <= 2147483647ll, GOAL_ERR_CAPACITY,
               "goal_sol_info_device_csr: more than 2^31-1 nonzeros for int32 indices");
  s->s->csr.alloc(d.nnz);
  k_bsr_to_csr<<<grid_for(d.num_nodes, 128), 128, 0, d.stream>>>(d.num_nodes, d.brow_ptr.ptr, s->s->A.ptr,
                                                                 s->s->csr.ptr);
  GOAL_CHECK_LAUNCH();
  GOAL_CUDA(cudaStreamSynchronize(d.stream));
  *csr_vals = s->s->csr.ptr;
  GOAL_API_END
}

int goal_sol_info_destroy(goal_sol_info s) {
  GOAL_API_BEGIN
  delete s;
  GOAL_API_END
}

int goal_assemble(goal_mechanics m, goal_sol_info s, const goal_chain* chain, double* qoi_value) {
  GOAL_API_BEGIN
  GOAL_ARG(m && chain, "goal_assemble: null argument");
  GOAL_ARG(!s || s->s->disc == m->m->disc, "goal_assemble: SolInfo and Mechanics belong to different discs");
  Chain c;
  c.mode = chain->mode;
  c.jacobian = chain->jacobian;
  c.save_states = chain->save_states;
  c.qoi = chain->qoi;
  c.rho = chain->rho;
  c.error_chain = chain->error_chain;
  c.overwrite = chain->overwrite;
  c.colored = chain->colored;
  GOAL_ARG(c.mode >= 0 && c.mode <= 2 && c.qoi >= 0 && c.qoi <= 2, "goal_assemble: bad chain");
  ErrorWeights w;
  if (c.error_chain) {
    GOAL_ARG(m->Zd.ptr && m->Zc.ptr, "goal_assemble: error chain needs goal_mechanics_set_weights");
    w.Zd = m->Zd.ptr;
    w.Zc = m->Zc.ptr;
  }
  double q = assemble(*m->m, s ? s->s.get() : nullptr, c, &w, m->m->disc->stream);
  if (qoi_value) *qoi_value = q;
  GOAL_API_END
}

int goal_bcs_create(goal_disc d, goal_bcs* out) {
  GOAL_API_BEGIN
  GOAL_ARG(d && out, "null argument");
  auto b = std::make_unique<goal_bcs_s>();
  b->d = d->d.get();
  *out = b.release();
  GOAL_API_END
}

int goal_bcs_add_dirichlet(goal_bcs b, int eq, const char* node_set, const char* expr) {
  GOAL_API_BEGIN
  GOAL_ARG(b && node_set && expr, "null argument");
  GOAL_ARG(eq >= 0 && eq < 3, "dirichlet bc: component must be 0, 1 or 2");
  auto it = b->d->node_sets.find(node_set);
  GOAL_ARG(it != b->d->node_sets.end(), std::string("unknown node set: ") + node_set);
  DBC bc;
  bc.eq = eq;
  bc.set = it->second.get();
  std::string err;
  GOAL_REQUIRE(compile_expr(expr, bc.code, err), GOAL_ERR_ARG, err);
  b->dbcs.push_back(bc);
  GOAL_API_END
}

int goal_bcs_add_traction(goal_bcs b, const char* side_set, const char* tx, const char* ty, const char* tz) {
  GOAL_API_BEGIN
  GOAL_ARG(b && side_set && tx && ty && tz, "null argument");
  auto it = b->d->side_sets.find(side_set);
  GOAL_ARG(it != b->d->side_sets.end(), std::string("unknown side set: ") + side_set);
  TBC bc;
  bc.set = it->second.get();
  const char* e[3] = {tx, ty, tz};
  for (int k = 0; k < 3; ++k) {
    std::string err;
    GOAL_REQUIRE(compile_expr(e[k], bc.code[k], err), GOAL_ERR_ARG, err);
  }
  b->tbcs.push_back(bc);
  GOAL_API_END
}

int goal_bcs_destroy(goal_bcs b) {
  GOAL_API_BEGIN
  delete b;
  GOAL_API_END
}

int goal_set_resid_dbcs(goal_mechanics m, goal_sol_info s, goal_bcs b, double t) {
  GOAL_API_BEGIN
  GOAL_ARG(m && s && b && b->d == m->m->disc, "goal_set_resid_dbcs: bad arguments");
  apply_dbcs(*m->m, *s->s, b->dbcs, t, false, m->m->disc->stream);
  GOAL_CUDA(cudaStreamSynchronize(m->m->disc->stream));
  GOAL_API_END
}

int goal_set_jac_dbcs(goal_mechanics m, goal_sol_info s, goal_bcs b, double t) {
  GOAL_API_BEGIN
  GOAL_ARG(m && s && b && b->d == m->m->disc, "goal_set_jac_dbcs: bad arguments");
  apply_dbcs(*m->m, *s->s, b->dbcs, t, true, m->m->disc->stream);
  GOAL_CUDA(cudaStreamSynchronize(m->m->disc->stream));
  GOAL_API_END
}

int goal_set_tbcs(goal_mechanics m, goal_sol_info s, goal_bcs b, double t, int error_weights) {
  GOAL_API_BEGIN
  GOAL_ARG(m && s && b && b->d == m->m->disc, "goal_set_tbcs: bad arguments");
  const double* zd = nullptr;
  if (error_weights) {
    GOAL_ARG(m->Zd.ptr, "goal_set_tbcs: error weights not set");
    zd = m->Zd.ptr;
  }
  apply_tbcs(*m->m, *s->s, b->tbcs, t, zd, m->m->disc->stream);
  GOAL_CUDA(cudaStreamSynchronize(m->m->disc->stream));
  GOAL_API_END
}

int goal_solve_device(goal_sol_info s, const goal_solve_params* params, const double* b, double* x,
                      goal_solve_stats* stats) {
  GOAL_API_BEGIN
  GOAL_ARG(s && b && x, "goal_solve: null argument");
  SolveParams p = to_params(params);
  static thread_local Krylov K;
  SolveStats r = linear_solve(*s->s, p, b, x, K);
  to_stats(r, stats);
  GOAL_REQUIRE(r.rel_res == r.rel_res, GOAL_ERR_SOLVER, "linear solve produced a non-finite residual");
  GOAL_API_END
}

int goal_solve(goal_sol_info s, const goal_solve_params* params, const double* b, double* x, goal_solve_stats* stats) {
  GOAL_API_BEGIN
  GOAL_ARG(s && b && x, "goal_solve: null argument");
  cudaStream_t st = s->s->disc->stream;
  size_t n = 4ull * s->s->disc->num_nodes;
  DevBuf<double> db, dx;
  db.upload(b, n, st);
  dx.upload(x, n, st);
  int rc = goal_solve_device(s, params, db.ptr, dx.ptr, stats);
  if (rc) return rc;
  dx.download(x, st);
  GOAL_CUDA(cudaStreamSynchronize(st));
  GOAL_API_END
}

int goal_primal_solve(goal_mechanics m, goal_sol_info s, goal_bcs b, double t_now, double t_old, int max_iters,
                      double tolerance, const goal_solve_params* lin, goal_newton_stats* stats) {
  GOAL_API_BEGIN
  GOAL_ARG(m && s && b && b->d == m->m->disc && s->s->disc == m->m->disc, "goal_primal_solve: bad arguments");
  NewtonParams p;
  p.max_iters = max_iters;
  p.tolerance = tolerance;
  p.lin = to_params(lin);
  p.line_search = m->m->line_search;
  static thread_local Krylov K;
  NewtonStats r = primal_solve(*m->m, *s->s, b->dbcs, b->tbcs, t_now, t_old, p, K);
  if (stats) {
    stats->backtracks = r.backtracks;
    stats->iters = r.iters;
    stats->converged = r.converged;
    stats->linear_iters = r.linear_iters;
    stats->inner_iters = r.inner_iters;
    for (int i = 0; i < 32; ++i) stats->norms[i] = r.norms[i];
    stats->seconds_assembly = r.seconds_assembly;
    stats->seconds_solve = r.seconds_solve;
  }
  GOAL_REQUIRE(r.converged, GOAL_ERR_NEWTON,
               "newton's method failed in " + std::to_string(max_iters) + " iterations");
  GOAL_API_END
}

int goal_nested_adjoint_create(goal_mechanics base, goal_nested_adjoint* out) {
  GOAL_API_BEGIN
  GOAL_ARG(base && out, "null argument");
  auto h = std::make_unique<goal_nested_adjoint_s>();
  h->a.build(*base->m);
  h->disc_view.d.reset(h->a.disc.get());
  h->disc_view.owns_stream = false;
  h->si_view.s.reset(h->a.si.get());
  *out = h.release();
  GOAL_API_END
}

int goal_nested_adjoint_disc(goal_nested_adjoint a, goal_disc* nested) {
  GOAL_API_BEGIN
  GOAL_ARG(a && nested, "null argument");
  *nested = &a->disc_view;
  GOAL_API_END
}

int goal_nested_adjoint_sol_info(goal_nested_adjoint a, goal_sol_info* s) {
  GOAL_API_BEGIN
  GOAL_ARG(a && s, "null argument");
  *s = &a->si_view;
  GOAL_API_END
}

int goal_nested_adjoint_run(goal_nested_adjoint a, goal_bcs nested_bcs, int qoi, double rho, double t_now,
                            double t_old, const goal_solve_params* params, goal_dwr_result* result,
                            double* base_error, double* nested_error) {
  GOAL_API_BEGIN
  GOAL_ARG(a && nested_bcs && nested_bcs->d == a->a.disc.get(), "goal_nested_adjoint_run: bcs must be on the nested disc");
  GOAL_ARG(qoi == GOAL_QOI_AVG_DISP || qoi == GOAL_QOI_KS_VM, "goal_nested_adjoint_run: unknown functional");
  SolveParams p = to_params(params);
  DwrResult r = nested_adjoint_run(a->a, nested_bcs->dbcs, nested_bcs->tbcs, qoi, rho, t_now, t_old, p);
  if (result) {
    result->eta = r.eta;
    result->bound = r.bound;
    result->qoi = r.qoi;
    to_stats(r.solve, &result->solve);
    result->seconds_adjoint = r.seconds_adjoint;
    result->seconds_solve = r.seconds_solve;
    result->seconds_localize = r.seconds_localize;
  }
  cudaStream_t st = a->a.disc->stream;
  if (base_error) a->a.err_base.download(base_error, st);
  if (nested_error) a->a.err_nested.download(nested_error, st);
  GOAL_CUDA(cudaStreamSynchronize(st));
  GOAL_API_END
}

int goal_nested_adjoint_get_z(goal_nested_adjoint a, double* z) {
  GOAL_API_BEGIN
  GOAL_ARG(a && z, "null argument");
  a->a.z.download(z, a->a.disc->stream);
  GOAL_CUDA(cudaStreamSynchronize(a->a.disc->stream));
  GOAL_API_END
}

int goal_nested_adjoint_destroy(goal_nested_adjoint a) {
  GOAL_API_BEGIN
  delete a;
  GOAL_API_END
}

int goal_learned_create(int seed, goal_learned* out) {
  GOAL_API_BEGIN
  GOAL_ARG(out, "null argument");
  auto h = std::make_unique<goal_learned_s>();
  GOAL_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  h->net.stream = h->stream;
  h->net.init(seed);
  *out = h.release();
  GOAL_API_END
}

int goal_learned_num_params(goal_learned l, int* n) {
  GOAL_API_BEGIN
  GOAL_ARG(l && n, "null argument");
  *n = MpnnLayout::total;
  GOAL_API_END
}

int goal_learned_get_params(goal_learned l, float* params) {
  GOAL_API_BEGIN
  GOAL_ARG(l && params, "null argument");
  l->net.stream = l->stream;
  l->net.download();
  std::memcpy(params, l->net.host_params.data(), sizeof(float) * MpnnLayout::total);
  GOAL_API_END
}

int goal_learned_set_params(goal_learned l, const float* params) {
  GOAL_API_BEGIN
  GOAL_ARG(l && params, "null argument");
  l->net.stream = l->stream;
  l->net.host_params.assign(params, params + MpnnLayout::total);
  l->net.upload();
  GOAL_API_END
}

static BsrMatrix matrix_of(goal_sol_info s) {
  BsrMatrix M;
  M.v = bsr_view(*s->s->disc);
  M.vals = s->s->A.ptr;
  return M;
}

int goal_learned_loss_grad(goal_learned l, goal_sol_info s, int num_probes, const double* probes, int seed,
                           double* loss, float* grad) {
  GOAL_API_BEGIN
  GOAL_ARG(l && s && num_probes >= 1, "goal_learned_loss_grad: bad arguments");
  l->net.stream = s->s->disc->stream;
  DevBuf<double> pd;
  if (probes) pd.upload(probes, (size_t)num_probes * 4 * s->s->disc->num_nodes, l->net.stream);
  double L = mpnn_loss_grad(l->net, matrix_of(s), num_probes, probes ? pd.ptr : nullptr, (unsigned)seed);
  if (loss) *loss = L;
  if (grad) {
    l->net.grad.download(grad, l->net.stream);
    GOAL_CUDA(cudaStreamSynchronize(l->net.stream));
  }
  GOAL_API_END
}

int goal_learned_corrections(goal_learned l, goal_sol_info s, float* C) {
  GOAL_API_BEGIN
  GOAL_ARG(l && s && C, "null argument");
  l->net.stream = s->s->disc->stream;
  mpnn_forward(l->net, matrix_of(s), false);
  GOAL_CUDA(cudaMemcpyAsync(C, l->net.C.ptr, sizeof(float) * 16 * s->s->disc->num_nodes, cudaMemcpyDeviceToHost,
                            l->net.stream));
  GOAL_CUDA(cudaStreamSynchronize(l->net.stream));
  GOAL_API_END
}

int goal_learned_train(goal_learned l, const goal_sol_info* systems, int num_systems, int epochs, float lr,
                       int num_probes, int seed, double* losses) {
  GOAL_API_BEGIN
  GOAL_ARG(l && systems && num_systems >= 1 && epochs >= 1 && num_probes >= 1, "goal_learned_train: bad arguments");
  for (int e = 0; e < epochs; ++e) {
    double sum = 0.0;
    for (int k = 0; k < num_systems; ++k) {
      goal_sol_info s = systems[k];
      l->net.stream = s->s->disc->stream;
      sum += mpnn_loss_grad(l->net, matrix_of(s), num_probes, nullptr, (unsigned)(seed + 131 * (e * num_systems + k)));
      mpnn_adam(l->net, lr, 0.9f, 0.999f, 1e-8f);
    }
    if (losses) losses[e] = sum;
  }
  GOAL_CUDA(cudaStreamSynchronize(l->net.stream));
  GOAL_API_END
}

int goal_sol_info_set_learned(goal_sol_info s, goal_learned l) {
  GOAL_API_BEGIN
  GOAL_ARG(s, "null argument");
  s->s->learned = l ? &l->net : nullptr;
  GOAL_API_END
}

int goal_learned_destroy(goal_learned l) {
  GOAL_API_BEGIN
  delete l;
  GOAL_API_END
}

}  // extern "C"
