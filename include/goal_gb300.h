/*
 * goal_gb300.h -- C ABI of the GB300 implementation of goal's element hot path
 * and its primal/adjoint solves.
 *
 * Plain pointers and sizes only. Every function returns 0 on success or a
 * nonzero status; goal_last_error() returns the message of the last failure
 * on the calling thread (the reference aborts through goal::fail,
 * src/goal_control.cpp:91-99). Handles are not thread-safe; each discretization
 * owns one CUDA stream that its mechanics, linear objects and solves use.
 *
 * Host arrays use goal's layouts: nodal DOF vectors are node-major with
 * num_eqs = 4 entries per node (u_x, u_y, u_z, p; lid = node*4 + eq,
 * src/goal_disc.cpp:195-201); element arrays are in the caller's element
 * order; tensors are row-major 3x3.
 */
#ifndef GOAL_GB300_H
#define GOAL_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GOAL_OK 0
#define GOAL_ERR_ARG 1
#define GOAL_ERR_CUDA 2
#define GOAL_ERR_STATE 3
#define GOAL_ERR_RETURN_MAP 4
#define GOAL_ERR_NEWTON 5
#define GOAL_ERR_CAPACITY 6
#define GOAL_ERR_SOLVER 7

/* goal::EvalModes (src/goal_eval_modes.hpp:6) */
#define GOAL_NONE 0
#define GOAL_PRIMAL 1
#define GOAL_ADJOINT 2

/* Mechanics "model" (src/goal_mechanics.cpp:113-120) */
#define GOAL_MODEL_NEOHOOKEAN 0
#define GOAL_MODEL_J2 1

/* functional "type" (src/goal_mechanics.cpp:148-167) */
#define GOAL_QOI_NONE 0
#define GOAL_QOI_AVG_DISP 1
#define GOAL_QOI_KS_VM 2 /* "max vm" with parameter rho */

/* state fields (src/goal_mechanics.cpp:87-95) */
#define GOAL_STATE_SIGMA 0
#define GOAL_STATE_FP 1
#define GOAL_STATE_FP_OLD 2
#define GOAL_STATE_EQPS 3
#define GOAL_STATE_EQPS_OLD 4

/* SolInfo vectors (src/goal_sol_info.hpp:12-16) */
#define GOAL_VEC_R 0
#define GOAL_VEC_DMDU 1

typedef struct goal_disc_s* goal_disc;
typedef struct goal_mechanics_s* goal_mechanics;
typedef struct goal_sol_info_s* goal_sol_info;
typedef struct goal_bcs_s* goal_bcs;

const char* goal_last_error(void);

/* Number of kernels this library has launched in the process. */
long long goal_launch_count(void);

/* goal::eval (src/goal_control.cpp:107-123): evaluates a boundary-condition
 * expression in x, y, z, t on the host with the same program the device runs. */
int goal_eval(const char* expr, double x, double y, double z, double t, double* out);

/* ---------------------------------------------------------------- Disc
 * goal::create_disc / Disc::build_data (src/goal_disc.hpp:95, :58;
 * src/goal_disc.cpp:224-235). tets are positively oriented linear tets.
 * build_data builds the node graph, the element colouring and the per-element
 * geometry on the GPU. */
int goal_disc_create(int num_nodes, int num_elems, const double* coords, const int* tets, const int* elem_set,
                     int num_elem_sets, goal_disc* out);
int goal_disc_add_node_set(goal_disc d, const char* name, int num_nodes, const int* nodes);
int goal_disc_add_side_set(goal_disc d, const char* name, int num_sides, const int* tris);
int goal_disc_build_data(goal_disc d);
/* sizes[0..5] = num_nodes, num_elems, num_dofs, nnz, nnzb (4x4 blocks), num_colors */
int goal_disc_sizes(goal_disc d, long long* sizes);
/* Wall seconds of the last build_data (Disc::compute_graphs and the element
 * layout, src/goal_disc.cpp:195-222, 307-332), by phase: seconds[0] node graph
 * (upload, node-element incidence sort, block graph), [1] element colouring
 * (Jones-Plassmann rounds; *color_rounds of them), [2] element layout
 * (colour-major order, block slots, geometry), [3] the sorted contribution
 * lists of the two-phase assembly, [4] node and side sets. */
int goal_disc_build_times(goal_disc d, double* seconds, int* color_rounds);
/* The owned CSR graph of dRdu (Disc::compute_graphs, src/goal_disc.cpp:307-332):
 * row_ptr[num_dofs+1], col_idx[nnz], columns sorted. */
int goal_disc_get_graph(goal_disc d, int* row_ptr, int* col_idx);
/* the mesh as stored (coords[3*num_nodes], tets[4*num_elems], elem_set[num_elems]);
 * for a nested discretization this is the refined mesh */
int goal_disc_get_mesh(goal_disc d, double* coords, int* tets, int* elem_set);
/* colour of every element (caller's element order) */
int goal_disc_get_colors(goal_disc d, int* colors);
/* cudaStream_t of the discretization (as void*) */
int goal_disc_stream(goal_disc d, void** stream);
int goal_disc_destroy(goal_disc d);

/* Nested(d, UNIFORM) (src/goal_nested.cpp:13-28, 144-154): uniformly refined
 * copy of a built discretization, built. New node num_nodes(base)+k sits at the
 * midpoint of edge k; edges are the upper triangle of the node graph in (i, j)
 * order. Children of base element e are 8e..8e+7. */
int goal_nested_create(goal_disc base, goal_disc* out);
/* end points of the edge of every new node: edges[2*(n - base_nodes) + {0,1}] */
int goal_nested_parent_edges(goal_disc nested, int* edges);

/* get_iso_target_size (src/goal_size_field.cpp:139-151): the isotropic target
 * size field that drives goal's mesh adaptation, from per-element error
 * indicators (elem_error[num_elems], caller's element order; e.g. the base
 * indicators of goal_nested_adjoint_run) and a target element count. Writes
 * one size per node (vtx_size[num_nodes]): the mean over the node's elements
 * of (G/target)^(1/3) |e|^(-2/5) h_e clamped to [h_e/4, 2 h_e], with
 * G = sum |e|^(6/5) and h_e the root mean square edge length. */
int goal_size_field(goal_disc d, const double* elem_error, int target, double* vtx_size);

/* Refinement to the target size, the refinement half of goal's adaptation
 * loop (src/main_nested.cpp:106-126, where SCOREC ma::adapt remeshes; that
 * library is not part of the reference). Conforming longest-edge-propagation
 * (LEPP) bisection on the host: every live tet with an edge longer than
 * ratio x (mean target size of its end points) is refined until none is left
 * (or max_elems / max_passes is reached). New nodes sit at edge midpoints and
 * take the mean target size of the edge's end points. Side triangles
 * (tris[3*num_sides], tri_set[num_sides]) are split with their edges.
 * create: the mesh; refine: vtx_size[num_nodes] -> sizes[0..2] = nodes,
 * elements, side triangles of the refined mesh; get: coords[3*nodes],
 * node_parents[2*nodes] (edge end points of new nodes, -1 -1 for original
 * nodes; new nodes follow the original ones in creation order),
 * tets[4*elements], elem_origin[elements] (original element of each tet),
 * tris/tri_set (may be NULL). */
typedef struct goal_refiner_s* goal_refiner;
int goal_refiner_create(int num_nodes, const double* coords, int num_elems, const int* tets, int num_sides,
                        const int* tris, const int* tri_set, goal_refiner* out);
int goal_refiner_refine(goal_refiner r, const double* vtx_size, double ratio, long long max_elems, int max_passes,
                        long long* sizes);
int goal_refiner_get(goal_refiner r, double* coords, int* node_parents, int* tets, int* elem_origin, int* tris,
                     int* tri_set);
int goal_refiner_destroy(goal_refiner r);

/* Coarsening to the target size by edge collapse, the other half of the
 * adaptation loop (same reference site; ma::adapt coarsens as well as
 * refines). An edge (a, b) shorter than ratio x (mean target size of its end
 * points) is collapsed by moving b onto a if node_class[b] has no bit that
 * node_class[a] lacks (the caller's node / side set memberships; the boundary
 * is added here), b is not on an element-set interface, a boundary b sits on a
 * flat part of the boundary and (a, b) is a boundary edge, the link condition
 * holds, every tet left around b stays positively oriented with mean-ratio
 * quality >= min(min_quality, the worst quality around b before), and no new
 * edge is longer than refine_ratio x its mean target size. Shortest (relative)
 * edges first, one independent set of collapses per pass, up to max_passes.
 * create: the mesh (elem_set may be NULL), node_class[num_nodes], side
 * triangles; coarsen: vtx_size[num_nodes] -> sizes[0..2] = nodes, elements,
 * side triangles left; get: coords[3*nodes], node_origin[nodes] (original node
 * of each kept node, in original order), tets[4*elements],
 * elem_origin[elements] (original element of each tet), tris/tri_set (may be
 * NULL). */
typedef struct goal_coarsener_s* goal_coarsener;
int goal_coarsener_create(int num_nodes, const double* coords, int num_elems, const int* tets, const int* elem_set,
                          const long long* node_class, int num_sides, const int* tris, const int* tri_set,
                          goal_coarsener* out);
int goal_coarsener_coarsen(goal_coarsener c, const double* vtx_size, double ratio, double refine_ratio,
                           double min_quality, int max_passes, long long* sizes);
/* Shape improvement by flips, nodes fixed (ma::adapt's shape correction in
 * part): tets with mean-ratio quality below target_quality, worst first, try
 * the 3-2 flip of each interior edge with three tets around it and the 2-3
 * flip of each interior face; the flip that raises the local minimum quality
 * most is taken. Flips stay inside one element set and do not cross side
 * triangles. A new tet takes the original element of the old tet that holds
 * its centroid. sizes as for coarsen. Callable with or without coarsen. */
int goal_coarsener_swap(goal_coarsener c, double target_quality, int max_passes, long long* sizes);
/* Vertex smoothing: interior nodes (in no node or side set, inside one
 * element set) whose surrounding tets have a quality below target_quality,
 * worst first and one independent set per pass, move to the mean of their
 * neighbours (or halfway there) when every tet around stays positive and the
 * worst quality around rises. A moved node's value becomes the old field at
 * its new position: transfer gives, per kept node (in the order of get), the
 * original nodes and weights (CSR: ptr[nodes + 1], ids/weights[nnz], nnz from
 * transfer_nnz); linear fields move exactly. */
int goal_coarsener_smooth(goal_coarsener c, double target_quality, int max_passes, long long* transfer_nnz);
int goal_coarsener_transfer(goal_coarsener c, int* ptr, int* ids, double* weights);
int goal_coarsener_get(goal_coarsener c, double* coords, int* node_origin, int* tets, int* elem_origin, int* tris,
                       int* tri_set);
int goal_coarsener_destroy(goal_coarsener c);

/* ---------------------------------------------------------------- Mechanics
 * goal::create_mechanics (src/goal_mechanics.hpp:50). materials holds, per
 * element set, E, nu, K, Y, c0 (K and Y are read by J2 only). States start as
 * sigma = 0, Fp = Fp_old = I, eqps = eqps_old = 0 (src/goal_states.cpp:99-128). */
int goal_mechanics_create(goal_disc d, int model, const double* materials, int stabilization, goal_mechanics* out);
int goal_mechanics_set_solution(goal_mechanics m, const double* U);  /* 4*num_nodes host values */
int goal_mechanics_get_solution(goal_mechanics m, double* U);
/* DWR weights for the error chain: z_diff and z_coarse, 4*num_nodes each
 * (u_z_diff/p_z_diff and p_z_coarse, src/goal_nested_adjoint.cpp:52-72) */
int goal_mechanics_set_weights(goal_mechanics m, const double* z_diff, const double* z_coarse);
/* J2 state writes at points that end a Newton solve elastic. 0 (default) is
 * goal's behaviour: J2::at_point writes Fp only where the point yields
 * (src/goal_J2.cpp:97-136), so the Fp of an earlier plastic Newton iterate
 * survives at a point that ends elastic and States::update commits it as
 * Fp_old. 1 also writes Fp = Fp_old at elastic points, so the committed state
 * is the converged iterate's. No counterpart in the reference: an option for
 * load paths on which goal's behaviour stops Newton from converging. */
int goal_mechanics_set_fp_reset(goal_mechanics m, int on);
/* state fields; sigma/Fp/Fp_old: 9*num_elems, eqps/eqps_old: num_elems */
int goal_states_set(goal_mechanics m, int which, const double* values);
int goal_states_get(goal_mechanics m, int which, double* values);
/* States::update: Fp_old = Fp, eqps_old = eqps (src/goal_states.cpp:130-141) */
int goal_states_update(goal_mechanics m);
int goal_mechanics_destroy(goal_mechanics m);

/* ---------------------------------------------------------------- SolInfo
 * goal::create_sol_info (src/goal_sol_info.hpp:41): R, dMdu and dRdu. dRdu is
 * stored as 4x4 blocks on the node graph; the CSR values in the order of
 * goal_disc_get_graph are produced on request. */
int goal_sol_info_create(goal_disc d, goal_sol_info* out);
int goal_sol_info_zero_all(goal_sol_info s);
int goal_sol_info_get_vector(goal_sol_info s, int which, double* values);
int goal_sol_info_set_vector(goal_sol_info s, int which, const double* values);
int goal_sol_info_get_dRdu_csr(goal_sol_info s, double* values);
int goal_sol_info_get_dRdu_bsr(goal_sol_info s, double* values);
int goal_sol_info_destroy(goal_sol_info s);

/* ---------------------------------------------------------------- device views
 * The linear objects as DEVICE pointers owned by the handles, for callers
 * whose own solver or vectors live on the GPU (goal's SolInfo hands out
 * owned->R, owned->dMdu and owned->dRdu, src/goal_sol_info.hpp:12-16,29; its
 * Tpetra objects are the ones Belos and MueLu read, src/goal_linear_solve.cpp:72-90).
 * No copies: the arrays are the ones goal_assemble, the boundary conditions
 * and goal_solve_device read and write, on the discretization's stream
 * (goal_disc_stream), so order other streams against it. They stay valid until
 * the handle is destroyed. Any output pointer may be NULL.
 *
 * goal_disc_device_graph: the block graph (brow_ptr[num_nodes+1],
 * bcol[nnzb], sorted; the matrix of 4x4 blocks, block k row-major at
 * bsr_vals + 16k) and goal's scalar CSR graph (row_ptr[num_dofs+1],
 * col_idx[nnz], the same arrays goal_disc_get_graph copies out; Disc's owned
 * graph, src/goal_disc.cpp:307-332). The scalar graph is built on the device
 * at the first request for it (one allocation, GOAL_ERR_CAPACITY beyond 2^31-1
 * nonzeros). */
int goal_disc_device_graph(goal_disc d, const int** brow_ptr, const int** bcol, const int** row_ptr,
                           const int** col_idx);
/* R[num_dofs], dMdu[num_dofs] and dRdu as 4x4 blocks (bsr_vals[16*nnzb]). */
int goal_sol_info_device_view(goal_sol_info s, double** R, double** dMdu, double** bsr_vals);
/* dRdu in the order of the scalar CSR graph (csr_vals[nnz]): written from the
 * blocks by this call (a snapshot of the current matrix; call it again after
 * the next assembly) into a buffer the SolInfo owns (allocated on the first
 * call). Returns when the values are written. */
int goal_sol_info_device_csr(goal_sol_info s, double** csr_vals);
/* the nodal solution U[num_dofs] (u_x, u_y, u_z, p per node) that every
 * assembly reads: the u and p fields of the mechanics, which Disc::add_soln
 * updates after a linear solve (src/goal_disc.cpp:398-422) */
int goal_mechanics_device_solution(goal_mechanics m, double** U);

/* ---------------------------------------------------------------- assemble
 * assemble(Evaluators, SolInfo*) (src/goal_assembly.cpp:65-88) for the chains
 * goal builds:
 *   Primal residual   {PRIMAL, jacobian 0, save 1}  (src/goal_primal.cpp:75-90)
 *   Primal jacobian   {PRIMAL, jacobian 1, save 1}  (src/goal_primal.cpp:92-109)
 *   Functional        {NONE, jacobian 0, save 0, qoi} (src/goal_functional.cpp:62-70)
 *   Nested adjoint    {ADJOINT, jacobian 1, save 0, qoi} (src/goal_nested_adjoint.cpp:163-180)
 *   Error             {PRIMAL, jacobian 0, save 0, error_chain 1} (src/goal_nested_adjoint.cpp:217-234)
 * overwrite = 1 makes the assembly start its outputs from zero (the zero_*
 * calls that precede every assembly in goal); 0 accumulates into them.
 * Both scatter strategies are deterministic and need no atomics: the default
 * evaluates every element in one launch into a per-element buffer and then
 * sums each matrix block / nodal row over its incident elements in element
 * order; colored = 1 evaluates one colour (no two elements sharing a node) per
 * launch and accumulates in place, without the buffer (2176 bytes per element). */
typedef struct {
  int mode;
  int jacobian;
  int save_states;
  int qoi;
  double rho;
  int error_chain;
  int overwrite;
  int colored; /* 0: element buffer + deterministic gather (default); 1: colour-by-colour in place */
} goal_chain;
int goal_assemble(goal_mechanics m, goal_sol_info s, const goal_chain* chain, double* qoi_value);
/* No counterpart in the reference. Size cap in bytes of the per-element buffer
 * of the default scatter (272 doubles per element for a Jacobian chain, 2176
 * bytes; 16 more with a QoI). A mesh whose buffer would be larger is
 * assembled in chunks of elements, each evaluated into the buffer and then
 * added to the matrix and vectors; the sums and their order are those of one
 * pass, so the results are the same bits. 0 (default) = a quarter of the
 * device's memory. Process-wide. */
int goal_set_element_buffer_limit(long long bytes);
/* No counterpart in the reference. Device time of goal_assemble's two phases,
 * measured with CUDA events on the discretization's stream: enable != 0 clears
 * the sums and starts measuring, 0 stops. ms[0] = element kernel(s), ms[1] =
 * gathers of R, dMdu and the matrix blocks; count = assemblies measured. */
int goal_assembly_timing(int enable);
int goal_assembly_timing_read(double* ms, long long* count);
/* No counterpart in the reference. Measured FP64 fused-multiply-add rate of
 * the current GPU in TFLOP/s (eight independent chains per thread, best of
 * five timed launches): the denominator of the element assembly's FP64
 * roofline. */
int goal_measure_fp64_peak(double* tflops);

/* ---------------------------------------------------------------- boundary conditions
 * "dirichlet bcs: [eq, node set, expr]" and "traction bcs: [side set, Tx, Ty, Tz]". */
int goal_bcs_create(goal_disc d, goal_bcs* out);
int goal_bcs_add_dirichlet(goal_bcs b, int eq, const char* node_set, const char* expr);
int goal_bcs_add_traction(goal_bcs b, const char* side_set, const char* tx, const char* ty, const char* tz);
int goal_bcs_destroy(goal_bcs b);
/* set_resid_dbcs / set_jac_dbcs (src/goal_dbcs.cpp:39-99) */
int goal_set_resid_dbcs(goal_mechanics m, goal_sol_info s, goal_bcs b, double t);
int goal_set_jac_dbcs(goal_mechanics m, goal_sol_info s, goal_bcs b, double t);
/* set_tbcs (src/goal_tbcs.cpp:29-85); error_weights = 1 uses the z_diff weights */
int goal_set_tbcs(goal_mechanics m, goal_sol_info s, goal_bcs b, double t, int error_weights);

/* ---------------------------------------------------------------- linear solve
 * goal::solve(params, A, x, b, disc) (src/goal_linear_solve.cpp:72-90) with
 * A = dRdu of the SolInfo. precision: 0 = FP64 FGMRES with block-Jacobi;
 * 1, 2, 3 = FP64 FGMRES (FP64 residual and update) whose preconditioner is
 * inner_iters GMRES iterations with block-Jacobi on the dof-scaled matrix
 * S A S, S = diag(|a_ii|^-1/2): 1 = matrix and Krylov basis stored in
 * binary16, FP32 arithmetic; 2 = stored in FP32, FP32 arithmetic; 3 = FP64
 * storage and arithmetic (nested FP64). precond: 0 = block-Jacobi, 1 = learned
 * block-Jacobi correction (see goal_learned_*), falling back to plain
 * block-Jacobi when the outer iterations exceed learned_cap.
 * Convergence: ||b - A x||_2 <= tolerance ||b||_2. */
typedef struct {
  int krylov_size;
  int max_iters;
  double tolerance;
  int precision;
  int inner_iters;
  int precond;
  int learned_cap;
} goal_solve_params;

typedef struct {
  int iters;
  int inner_iters;
  int converged;
  int fell_back;
  double rel_res;
  double seconds;
  long long spmv64;
  long long spmv32;
} goal_solve_stats;

/* b and x are host arrays of num_dofs values; x holds the initial guess. */
int goal_solve(goal_sol_info s, const goal_solve_params* params, const double* b, double* x, goal_solve_stats* stats);
/* the same with device pointers (no copies) */
int goal_solve_device(goal_sol_info s, const goal_solve_params* params, const double* b, double* x,
                      goal_solve_stats* stats);

/* ---------------------------------------------------------------- Newton
 * Primal::solve (src/goal_primal.cpp:111-137): per iteration the Jacobian chain,
 * traction and Dirichlet conditions, R *= -1, the linear solve, U += du, the
 * residual chain with its conditions, and ||R||_2 < tolerance (absolute).
 * Returns GOAL_ERR_NEWTON when max_iters is reached without convergence. */
typedef struct {
  int iters;
  int converged;
  int linear_iters;
  int inner_iters;
  double norms[32];
  double seconds_assembly;
  double seconds_solve;
  int backtracks; /* step halvings of the line search (goal_mechanics_set_line_search) */
} goal_newton_stats;
int goal_primal_solve(goal_mechanics m, goal_sol_info s, goal_bcs b, double t_now, double t_old, int max_iters,
                      double tolerance, const goal_solve_params* lin, goal_newton_stats* stats);
/* No counterpart in the reference (goal takes full Newton steps). max_halvings
 * > 0 makes goal_primal_solve backtrack: the step is U += a du with the first
 * a in 1, 1/2, ..., 2^-max_halvings whose residual norm is below
 * (1 - 1e-4 a) times the norm at the start of the iteration (else the
 * smallest a). 0 (default) is goal's full step. */
int goal_mechanics_set_line_search(goal_mechanics m, int max_halvings);

/* ---------------------------------------------------------------- nested adjoint + DWR
 * NestedAdjoint (src/goal_nested_adjoint.cpp): build_data creates the uniformly
 * refined discretization, its mechanics (child states = parent states) and
 * linear objects; run refreshes the prolonged solution and states, assembles the
 * transposed Jacobian and dM/du, solves dRdu^T z = dMdu, forms z_coarse (edge
 * midpoint interpolant) and z_diff, the estimate eta = -R.z, localizes the
 * error with the PU-DWR weights and returns the bound sum_v |e_u + e_p| and the
 * element indicators (base mesh: sum over the 8 children). Boundary conditions
 * are given on the nested discretization (goal_nested_adjoint_disc). */
typedef struct goal_nested_adjoint_s* goal_nested_adjoint;
typedef struct {
  double eta;
  double bound;
  double qoi;
  goal_solve_stats solve;
  double seconds_adjoint;
  double seconds_solve;
  double seconds_localize;
} goal_dwr_result;
int goal_nested_adjoint_create(goal_mechanics base, goal_nested_adjoint* out);
int goal_nested_adjoint_disc(goal_nested_adjoint a, goal_disc* nested);
/* the nested linear objects (dRdu^T after a run), e.g. to attach a learned preconditioner */
int goal_nested_adjoint_sol_info(goal_nested_adjoint a, goal_sol_info* s);
int goal_nested_adjoint_run(goal_nested_adjoint a, goal_bcs nested_bcs, int qoi, double rho, double t_now,
                            double t_old, const goal_solve_params* params, goal_dwr_result* result,
                            double* base_error, double* nested_error);
/* z (4*num_nodes of the nested mesh) of the last run */
int goal_nested_adjoint_get_z(goal_nested_adjoint a, double* z);
int goal_nested_adjoint_destroy(goal_nested_adjoint a);

/* ---------------------------------------------------------------- learned preconditioner
 * A mesh-graph network (3 message-passing layers, width 32, bfloat16 weights,
 * float32 arithmetic) on the matrix's node graph, in the dof-scaled space
 * S A S (S = diag(|a_ii|^-1/2)). It emits a 4x4 block W_n per node that
 * weights a second block-Jacobi sweep: z = D^-1 r, P r = z + B (r - A z),
 * B_n = S_n W_n S_n^-1 D_n^-1 (rows/columns of Dirichlet rows zeroed). It has
 * no counterpart in the reference (goal preconditions with MueLu AMG,
 * src/goal_linear_solve.cpp:59-65). Training minimizes
 * sum_i |S(v_i - A P v_i)|^2 / |S v_i|^2 over probes (v_i = S^-1 w_i or
 * A D^-1 S^-1 w_i) on the GPU with Adam; the untrained network (decoder at
 * zero) is plain block-Jacobi. A solve with precond = 1 uses the network
 * attached to the SolInfo. */
typedef struct goal_learned_s* goal_learned;
int goal_learned_create(int seed, goal_learned* out);
int goal_learned_num_params(goal_learned l, int* n);
int goal_learned_get_params(goal_learned l, float* params);
int goal_learned_set_params(goal_learned l, const float* params);
/* loss and gradient for the SolInfo's matrix; probes: num_probes x num_dofs host
 * values w_i (scaled residual space), or NULL to draw them from seed */
int goal_learned_loss_grad(goal_learned l, goal_sol_info s, int num_probes, const double* probes, int seed,
                           double* loss, float* grad);
/* network outputs W (16 per node, row-major 4x4, before the Dirichlet masking) for the SolInfo's matrix */
int goal_learned_corrections(goal_learned l, goal_sol_info s, float* C);
/* epochs x (one Adam step per system); losses[epochs] = summed loss per epoch */
int goal_learned_train(goal_learned l, const goal_sol_info* systems, int num_systems, int epochs, float lr,
                       int num_probes, int seed, double* losses);
int goal_sol_info_set_learned(goal_sol_info s, goal_learned l);
int goal_learned_destroy(goal_learned l);

/* ---------------------------------------------------------------- functional without allocation
 * No counterpart in the reference. The "avg disp" functional
 * (AvgDisp::at_point, src/goal_avg_disp.cpp:17-21) over a mesh given as the
 * caller's DEVICE arrays: coords (3 per node), tets (4 node ids per element),
 * U (4 per node: u_x, u_y, u_z, p). The value is written to the device double
 * *J on `stream` (a cudaStream_t; NULL = the default stream); the call does not
 * wait for it. It performs kernel launches only: no device allocation, no
 * free, no synchronisation. It is for callers that may not allocate device
 * memory: a framework that hands all free device memory to its own pool (a
 * cudaMalloc there fails or steals from that pool), or a time-critical loop
 * that must not pay for an allocation. The partial sums live in a fixed 128 KiB device array of this
 * library, which limits a call to 16,777,216 elements (GOAL_ERR_CAPACITY
 * beyond). The first call on each device, with that device current, looks up
 * that array's address. Nothing has to be zeroed beforehand; *J is
 * overwritten. Calls that overlap in time share the
 * array and race: issue them on one stream or order them with events. A node
 * id outside [0, num_nodes) makes *J NaN. Same value as goal_assemble with
 * GOAL_NONE and GOAL_QOI_AVG_DISP up to summation order. */
int goal_avg_disp_noalloc(const double* coords, const int* tets, const double* U, int num_nodes, int num_elems,
                          double* J, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GOAL_GB300_H */
