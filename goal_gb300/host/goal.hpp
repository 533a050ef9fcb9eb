// goal.hpp -- C++ mirror of goal's host interface on top of the C ABI.
//
// Same names and call order as the reference host code, so a driver written
// against goal's classes reads the same:
//   goal::Disc           src/goal_disc.hpp        (create_disc, build_data, get_num_eqs, graphs)
//   goal::Mechanics      src/goal_mechanics.hpp   (model, materials, states, fields u and p)
//   goal::SolInfo        src/goal_sol_info.hpp    (R, dMdu, dRdu; zero_all)
//   goal::EvalModes      src/goal_eval_modes.hpp  (NONE, PRIMAL, ADJOINT)
//   goal::assemble       src/goal_assembly.hpp    (one evaluator chain)
//   goal::solve          src/goal_linear_solve.hpp
//   goal::Primal         src/goal_primal.hpp      (Newton: compute_resid/compute_jacob/solve)
//   goal::Functional     src/goal_functional.hpp
//   goal::NestedAdjoint  src/goal_nested_adjoint.hpp
// A nonzero status from the library ends in goal::fail (print + abort), which
// is what the reference does on every error (src/goal_control.cpp:91-99).
#pragma once

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/goal_gb300.h"

namespace goal {

enum EvalModes { NONE = GOAL_NONE, PRIMAL = GOAL_PRIMAL, ADJOINT = GOAL_ADJOINT };

[[noreturn]] inline void fail(const char* why, ...) {
  va_list ap;
  va_start(ap, why);
  std::vfprintf(stderr, why, ap);
  va_end(ap);
  std::fprintf(stderr, "\n");
  std::abort();
}

inline void check(int rc) {
  if (rc != GOAL_OK) fail("goal: %s", goal_last_error());
}

inline void print(const char* msg, ...) {
  va_list ap;
  va_start(ap, msg);
  std::vfprintf(stdout, msg, ap);
  va_end(ap);
  std::printf("\n");
}

struct ElemSet {
  std::string name;
};

class Disc {
 public:
  // coords[3N], tets[4E] (positively oriented), elem_set[E] in [0, num_elem_sets)
  Disc(int num_nodes, int num_elems, const double* coords, const int* tets, const int* elem_set, int num_elem_sets) {
    check(goal_disc_create(num_nodes, num_elems, coords, tets, elem_set, num_elem_sets, &h_));
    owned_ = true;
  }
  explicit Disc(goal_disc borrowed) : h_(borrowed), owned_(false) { refresh(); }
  ~Disc() {
    if (owned_) goal_disc_destroy(h_);
  }
  Disc(const Disc&) = delete;
  Disc& operator=(const Disc&) = delete;
  void add_node_set(const std::string& name, const std::vector<int>& nodes) {
    check(goal_disc_add_node_set(h_, name.c_str(), (int)nodes.size(), nodes.data()));
  }
  void add_side_set(const std::string& name, const std::vector<int>& tris) {
    check(goal_disc_add_side_set(h_, name.c_str(), (int)tris.size() / 3, tris.data()));
  }
  void build_data() {
    check(goal_disc_build_data(h_));
    refresh();
  }
  int get_num_dims() const { return 3; }
  int get_num_eqs() const { return 4; }
  long long get_num_nodes() const { return sizes_[0]; }
  long long get_num_elems() const { return sizes_[1]; }
  long long get_num_dofs() const { return sizes_[2]; }
  long long get_nnz() const { return sizes_[3]; }
  // the owned CSR graph (row_ptr, col_idx) of dRdu
  void get_owned_graph(std::vector<int>& row_ptr, std::vector<int>& col_idx) const {
    row_ptr.resize(get_num_dofs() + 1);
    col_idx.resize(get_nnz());
    check(goal_disc_get_graph(h_, row_ptr.data(), col_idx.data()));
  }
  // the same graph as device pointers owned by the disc (plus the 4x4-block graph)
  struct DeviceGraph {
    const int* brow_ptr = nullptr;
    const int* bcol = nullptr;
    const int* row_ptr = nullptr;
    const int* col_idx = nullptr;
  };
  DeviceGraph device_graph() const {
    DeviceGraph g;
    check(goal_disc_device_graph(h_, &g.brow_ptr, &g.bcol, &g.row_ptr, &g.col_idx));
    return g;
  }
  // lid of equation eq of node n (src/goal_disc.cpp:195-201)
  static long long get_lid(long long node, int eq) { return node * 4 + eq; }
  goal_disc handle() const { return h_; }

 private:
  void refresh() { check(goal_disc_sizes(h_, sizes_)); }
  goal_disc h_ = nullptr;
  bool owned_ = true;
  long long sizes_[6] = {0, 0, 0, 0, 0, 0};
};

struct Material {
  double E, nu, K, Y, c0;
};

class Mechanics {
 public:
  // model: "neohookean" or "J2" (src/goal_mechanics.cpp:113-120); materials per element set
  Mechanics(Disc& d, const std::string& model, const std::vector<Material>& mats, bool stabilization = true)
      : disc_(d) {
    int m = (model == "J2") ? GOAL_MODEL_J2 : (model == "neohookean" ? GOAL_MODEL_NEOHOOKEAN : -1);
    if (m < 0) fail("unknown model: %s", model.c_str());
    std::vector<double> flat;
    for (const Material& x : mats) flat.insert(flat.end(), {x.E, x.nu, x.K, x.Y, x.c0});
    check(goal_mechanics_create(d.handle(), m, flat.data(), stabilization ? 1 : 0, &h_));
  }
  ~Mechanics() { goal_mechanics_destroy(h_); }
  Mechanics(const Mechanics&) = delete;
  Mechanics& operator=(const Mechanics&) = delete;
  Disc* get_disc() { return &disc_; }
  std::vector<double> get_solution() const {
    std::vector<double> U(disc_.get_num_dofs());
    check(goal_mechanics_get_solution(h_, U.data()));
    return U;
  }
  void set_solution(const std::vector<double>& U) { check(goal_mechanics_set_solution(h_, U.data())); }
  // the u and p fields on the device (4 per node)
  double* device_solution() const {
    double* U = nullptr;
    check(goal_mechanics_device_solution(h_, &U));
    return U;
  }
  void update_states() { check(goal_states_update(h_)); }  // States::update
  goal_mechanics handle() const { return h_; }

 private:
  Disc& disc_;
  goal_mechanics h_ = nullptr;
};

class SolInfo {
 public:
  explicit SolInfo(Disc& d) : disc_(d) { check(goal_sol_info_create(d.handle(), &h_)); }
  ~SolInfo() { goal_sol_info_destroy(h_); }
  SolInfo(const SolInfo&) = delete;
  SolInfo& operator=(const SolInfo&) = delete;
  Disc* get_disc() { return &disc_; }
  void zero_all() { check(goal_sol_info_zero_all(h_)); }
  std::vector<double> R() const { return vec(GOAL_VEC_R); }
  std::vector<double> dMdu() const { return vec(GOAL_VEC_DMDU); }
  std::vector<double> dRdu() const {  // CSR values in the order of Disc::get_owned_graph
    std::vector<double> v(disc_.get_nnz());
    check(goal_sol_info_get_dRdu_csr(h_, v.data()));
    return v;
  }
  // owned->R, owned->dMdu and dRdu (4x4 blocks) as device pointers owned by the SolInfo
  struct DeviceView {
    double* R = nullptr;
    double* dMdu = nullptr;
    double* bsr = nullptr;
  };
  DeviceView device_view() const {
    DeviceView v;
    check(goal_sol_info_device_view(h_, &v.R, &v.dMdu, &v.bsr));
    return v;
  }
  // dRdu in the order of Disc::device_graph().row_ptr/col_idx (device, refreshed by this call)
  double* device_dRdu() const {
    double* v = nullptr;
    check(goal_sol_info_device_csr(h_, &v));
    return v;
  }
  goal_sol_info handle() const { return h_; }

 private:
  std::vector<double> vec(int which) const {
    std::vector<double> v(disc_.get_num_dofs());
    check(goal_sol_info_get_vector(h_, which, v.data()));
    return v;
  }
  Disc& disc_;
  goal_sol_info h_ = nullptr;
};

// An evaluator chain as Mechanics::build_resid / build_functional / build_error build it.
struct Evaluators {
  goal_chain chain{GOAL_PRIMAL, 0, 0, GOAL_QOI_NONE, 0.0, 0, 1, 0};
  static Evaluators residual(bool save) { return Evaluators{{GOAL_PRIMAL, 0, save ? 1 : 0, GOAL_QOI_NONE, 0.0, 0, 1, 0}}; }
  static Evaluators jacobian(bool save) { return Evaluators{{GOAL_PRIMAL, 1, save ? 1 : 0, GOAL_QOI_NONE, 0.0, 0, 1, 0}}; }
  static Evaluators functional(int qoi, double rho) { return Evaluators{{GOAL_NONE, 0, 0, qoi, rho, 0, 1, 0}}; }
  static Evaluators adjoint(int qoi, double rho) { return Evaluators{{GOAL_ADJOINT, 1, 0, qoi, rho, 0, 1, 0}}; }
};

inline double assemble(Mechanics& m, const Evaluators& E, SolInfo* s) {
  double q = 0.0;
  check(goal_assemble(m.handle(), s ? s->handle() : nullptr, &E.chain, &q));
  return q;
}

class BCs {
 public:
  explicit BCs(Disc& d) { check(goal_bcs_create(d.handle(), &h_)); }
  ~BCs() { goal_bcs_destroy(h_); }
  BCs(const BCs&) = delete;
  BCs& operator=(const BCs&) = delete;
  // "dirichlet bcs: [eq, node set, expr]"
  void add_dirichlet(int eq, const std::string& set, const std::string& expr) {
    check(goal_bcs_add_dirichlet(h_, eq, set.c_str(), expr.c_str()));
  }
  // "traction bcs: [side set, Tx, Ty, Tz]"
  void add_traction(const std::string& set, const std::string& tx, const std::string& ty, const std::string& tz) {
    check(goal_bcs_add_traction(h_, set.c_str(), tx.c_str(), ty.c_str(), tz.c_str()));
  }
  goal_bcs handle() const { return h_; }

 private:
  goal_bcs h_ = nullptr;
};

struct LinearParams {  // "primal/adjoint linear algebra" (src/goal_linear_solve.cpp:22-32)
  int krylov_size = 100;
  int max_iters = 2000;
  double tolerance = 1e-10;
  int nonlinear_max_iters = 5;
  double nonlinear_tolerance = 1e-8;
  int precision = 0;
  int inner_iters = 30;
  goal_solve_params solve_params() const {
    return goal_solve_params{krylov_size, max_iters, tolerance, precision, inner_iters, 0, 0};
  }
};

// goal::solve (src/goal_linear_solve.cpp:72-90) on the SolInfo's dRdu
inline goal_solve_stats solve(const LinearParams& p, SolInfo& s, std::vector<double>& x, const std::vector<double>& b) {
  goal_solve_params q = p.solve_params();
  goal_solve_stats st;
  check(goal_solve(s.handle(), &q, b.data(), x.data(), &st));
  print(" > linear system: solved in %d iterations", st.iters);
  if (!st.converged) print(" >  but solve was incomplete! continuing anyway...");
  return st;
}

class Primal {
 public:
  Primal(Mechanics& m, BCs& bcs, const LinearParams& lp) : mech_(m), bcs_(bcs), lp_(lp), si_(*m.get_disc()) {}
  SolInfo* get_sol_info() { return &si_; }
  // Primal::solve (src/goal_primal.cpp:111-137)
  goal_newton_stats solve(double t_now, double t_old) {
    print("*** primal solve: %lld dofs", mech_.get_disc()->get_num_dofs());
    print("*** at time: %f", t_now);
    goal_solve_params q = lp_.solve_params();
    goal_newton_stats st;
    int rc = goal_primal_solve(mech_.handle(), si_.handle(), bcs_.handle(), t_now, t_old, lp_.nonlinear_max_iters,
                               lp_.nonlinear_tolerance, &q, &st);
    for (int i = 0; i < st.iters && i < 32; ++i) print(" > (%d) ||R|| = %e", i + 1, st.norms[i]);
    if (rc == GOAL_ERR_NEWTON) fail("newton's method failed in %d iterations", lp_.nonlinear_max_iters);
    check(rc);
    return st;
  }

 private:
  Mechanics& mech_;
  BCs& bcs_;
  LinearParams lp_;
  SolInfo si_;
};

class Functional {
 public:
  // type: "avg disp" or "max vm" (with rho) (src/goal_mechanics.cpp:148-167)
  Functional(Mechanics& m, const std::string& type, double rho = 0.0) : mech_(m), rho_(rho) {
    if (type == "avg disp") qoi_ = GOAL_QOI_AVG_DISP;
    else if (type == "max vm") qoi_ = GOAL_QOI_KS_VM;
    else fail("unknown functional type: %s", type.c_str());
    name_ = type;
  }
  void compute(double, double) { value_ = assemble(mech_, Evaluators::functional(qoi_, rho_), nullptr); }
  double get_value() const { return value_; }
  void print_value() const {
    print(" > functional : %s", name_.c_str());
    print(" > J(uH) = %.15e", value_);
  }
  int qoi() const { return qoi_; }
  double rho() const { return rho_; }

 private:
  Mechanics& mech_;
  int qoi_ = GOAL_QOI_AVG_DISP;
  double rho_ = 0.0, value_ = 0.0;
  std::string name_;
};

class NestedAdjoint {
 public:
  NestedAdjoint(Mechanics& base, const LinearParams& lp) : lp_(lp) {
    check(goal_nested_adjoint_create(base.handle(), &h_));
    goal_disc d = nullptr;
    check(goal_nested_adjoint_disc(h_, &d));
    disc_ = new Disc(d);
    bcs_ = new BCs(*disc_);
    base_elems_ = base.get_disc()->get_num_elems();
  }
  ~NestedAdjoint() {
    delete bcs_;
    delete disc_;
    goal_nested_adjoint_destroy(h_);
  }
  NestedAdjoint(const NestedAdjoint&) = delete;
  NestedAdjoint& operator=(const NestedAdjoint&) = delete;
  BCs& bcs() { return *bcs_; }  // boundary conditions on the nested discretization
  // NestedAdjoint::run: returns the error indicator of every base element
  std::vector<double> run(const Functional& J, double t_now, double t_old, goal_dwr_result* out = nullptr) {
    goal_solve_params q = lp_.solve_params();
    goal_dwr_result r;
    std::vector<double> err(base_elems_);
    check(goal_nested_adjoint_run(h_, bcs_->handle(), J.qoi(), J.rho(), t_now, t_old, &q, &r, err.data(), nullptr));
    print(" > z.R = %.15e", r.eta);
    print(" > |J(u)-J(uh)| < %.15e", r.bound);
    if (out) *out = r;
    return err;
  }

 private:
  LinearParams lp_;
  goal_nested_adjoint h_ = nullptr;
  Disc* disc_ = nullptr;
  BCs* bcs_ = nullptr;
  long long base_elems_ = 0;
};

// get_iso_target_size (src/goal_size_field.cpp:139-151): per-node target sizes
inline std::vector<double> get_iso_target_size(Disc& d, const std::vector<double>& elem_error, int target) {
  std::vector<double> size(d.get_num_nodes());
  check(goal_size_field(d.handle(), elem_error.data(), target, size.data()));
  return size;
}

// The refinement half of Solver::adapt (src/main_nested.cpp:106-126): the mesh
// refined until no edge is longer than ratio x its target size, with the node
// parents (new nodes at edge midpoints, after the old nodes) and the original
// element of every new element, for the field transfer.
struct RefinedMesh {
  std::vector<double> coords;
  std::vector<int> tets, elem_origin, node_parents, tris, tri_set;
};
inline RefinedMesh refine_to_size(const std::vector<double>& coords, const std::vector<int>& tets,
                                  const std::vector<int>& tris, const std::vector<int>& tri_set,
                                  const std::vector<double>& vtx_size, double ratio = 1.5,
                                  long long max_elems = 50000000, int max_passes = 64) {
  goal_refiner r = nullptr;
  check(goal_refiner_create((int)(coords.size() / 3), coords.data(), (int)(tets.size() / 4), tets.data(),
                            (int)tri_set.size(), tris.data(), tri_set.data(), &r));
  long long sizes[3];
  int rc = goal_refiner_refine(r, vtx_size.data(), ratio, max_elems, max_passes, sizes);
  if (rc != GOAL_OK) {
    goal_refiner_destroy(r);
    check(rc);
  }
  RefinedMesh m;
  m.coords.resize(3 * sizes[0]);
  m.node_parents.resize(2 * sizes[0]);
  m.tets.resize(4 * sizes[1]);
  m.elem_origin.resize(sizes[1]);
  m.tris.resize(3 * sizes[2]);
  m.tri_set.resize(sizes[2]);
  rc = goal_refiner_get(r, m.coords.data(), m.node_parents.data(), m.tets.data(), m.elem_origin.data(),
                        m.tris.data(), m.tri_set.data());
  goal_refiner_destroy(r);
  check(rc);
  return m;
}

// Coarsening to the target size (goal_coarsener_*): node_class holds the
// caller's set memberships per node (a collapsed node's sets must be a subset
// of its target's); elem_set may be empty (one set).
struct CoarsenedMesh {
  std::vector<double> coords;
  std::vector<int> tets, elem_origin, node_origin, tris, tri_set;
};
inline CoarsenedMesh coarsen_to_size(const std::vector<double>& coords, const std::vector<int>& tets,
                                     const std::vector<int>& elem_set, const std::vector<long long>& node_class,
                                     const std::vector<int>& tris, const std::vector<int>& tri_set,
                                     const std::vector<double>& vtx_size, double ratio = 0.5,
                                     double refine_ratio = 1.5, double min_quality = 0.2, int max_passes = 8,
                                     double improve_quality = 0.0) {
  goal_coarsener c = nullptr;
  check(goal_coarsener_create((int)(coords.size() / 3), coords.data(), (int)(tets.size() / 4), tets.data(),
                              elem_set.empty() ? nullptr : elem_set.data(), node_class.data(), (int)tri_set.size(),
                              tris.data(), tri_set.data(), &c));
  long long sizes[3];
  int rc = goal_coarsener_coarsen(c, vtx_size.data(), ratio, refine_ratio, min_quality, max_passes, sizes);
  // optional shape improvement: flips (vertex smoothing would move nodes and
  // needs the interpolating transfer of goal_coarsener_transfer)
  if (rc == GOAL_OK && improve_quality > 0.0) rc = goal_coarsener_swap(c, improve_quality, 4, sizes);
  if (rc != GOAL_OK) {
    goal_coarsener_destroy(c);
    check(rc);
  }
  CoarsenedMesh m;
  m.coords.resize(3 * sizes[0]);
  m.node_origin.resize(sizes[0]);
  m.tets.resize(4 * sizes[1]);
  m.elem_origin.resize(sizes[1]);
  m.tris.resize(3 * sizes[2]);
  m.tri_set.resize(sizes[2]);
  rc = goal_coarsener_get(c, m.coords.data(), m.node_origin.data(), m.tets.data(), m.elem_origin.data(),
                          m.tris.data(), m.tri_set.data());
  goal_coarsener_destroy(c);
  check(rc);
  return m;
}

}  // namespace goal
