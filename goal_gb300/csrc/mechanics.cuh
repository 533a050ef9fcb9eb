// Mechanics on the device: material constants, integration-point states, the
// nodal solution and the linear objects of SolInfo (src/goal_sol_info.hpp).
#pragma once

#include "disc.cuh"
#include "expr.h"

namespace goal {

enum Model : int { MODEL_NEOHOOKEAN = 0, MODEL_J2 = 1 };
enum EvalMode : int { MODE_NONE = 0, MODE_PRIMAL = 1, MODE_ADJOINT = 2 };  // src/goal_eval_modes.hpp:6
enum QoIType : int { QOI_NONE = 0, QOI_AVG_DISP = 1, QOI_KS_VM = 2 };

// Per element set: E, nu, K, Y, c0 (src/goal_J2.cpp:53-64, src/goal_neohookean.cpp:44-52)
struct MaterialRow {
  double E, nu, K, Y, c0;
};

// States of one element, structure-of-arrays in colour order.
struct StatesDev {
  DevBuf<double> sigma;     // 9 x E  Cauchy stress after Mixed
  DevBuf<double> Fp, Fp_old;// 9 x E  plastic deformation gradient
  DevBuf<double> eqps, eqps_old;  // E
  DevBuf<double> Cpinv;     // 6 x E  Fp_old^{-1} Fp_old^{-T} (xx yy zz xy yz xz), refreshed with Fp_old
  // Deferred Fp writes: a plastic point's state write stores the plastic
  // increment A = dgam N (6 x E, xx yy zz xy yz xz) and sets pend; Fp =
  // exp(A) Fp_old is formed when Fp is read or committed (materialize_fp),
  // with the same arithmetic as an immediate write.
  DevBuf<double> Apend;
  DevBuf<int> pend;
};

struct Mechanics {
  Disc* disc = nullptr;
  int model = MODEL_NEOHOOKEAN;
  bool stabilization = true;
  // J2 state writes at elastic points: false is goal's behaviour
  // (src/goal_J2.cpp:97-136 writes Fp only where the point yields, so the Fp
  // of an earlier plastic Newton iterate survives at points that end elastic,
  // and States::update commits it); true writes Fp = Fp_old there.
  bool fp_reset = false;
  int line_search = 0;      // Newton backtracking halvings (0: goal's full Newton steps)
  std::vector<MaterialRow> mats_h;
  DevBuf<double> mats;      // per set: kappa, mu, K, Y, c0, 1/kappa, c0/(2 mu), 1/(16 kappa)
  DevBuf<double> U;         // 4N nodal solution: u_x u_y u_z p per node (the DOF layout)
  StatesDev st;
  DevBuf<double> qoi_elem;  // E   per-element QoI values (colour order)
  DevBuf<double> ebuf;      // two-phase assembly: per-element R and 16 4x4 blocks (272 doubles)
  DevBuf<double> dbuf;      // two-phase assembly: per-element dM/du (16 doubles)
  DevBuf<double> red;       // reduction scratch
  DevBuf<int> status;       // 1: return-map failures, non-finite etc.
  void init();
  void update_states();     // States::update (src/goal_states.cpp:130-141)
  void refresh_cpinv();
  void materialize_fp();    // Fp = exp(A) Fp_old at points with a pending plastic write
};

// Linear objects of one discretization (LinearObj, src/goal_sol_info.hpp:12-16).
// dRdu is stored as 4x4 blocks (BSR) on the disc's block graph.
struct Mpnn;

struct SolInfo {
  Disc* disc = nullptr;
  Mpnn* learned = nullptr;  // network used when a solve asks for the learned preconditioner
  DevBuf<double> R, dMdu;   // 4N
  DevBuf<double> A;         // 16 x nnzb, block (n,m) row-major
  DevBuf<double> csr;       // nnz: A in the order of the scalar CSR graph, written on request
  void init(Disc* d);
};

struct Chain {
  int mode = MODE_PRIMAL;
  int jacobian = 0;         // FADT chain (dRdu) when 1, residual (ST) chain when 0
  int save_states = 0;
  int qoi = QOI_NONE;
  double rho = 0.0;
  int error_chain = 0;      // Mechanics::build_error weights (src/goal_mechanics.cpp:169-218)
  int overwrite = 1;        // outputs start from zero (fuses SolInfo::zero_*)
  int colored = 0;          // 1: accumulate in place one colour at a time (no element buffer)
};

struct ErrorWeights {
  const double* Zd = nullptr;   // 4N z_fine - z_coarse (u_z_diff, p_z_diff)
  const double* Zc = nullptr;   // 4N z_coarse (p component used by stabilization)
};

// assemble(E, SolInfo*) (src/goal_assembly.cpp:65-88) for one chain.
// Returns the QoI value when chain.qoi != QOI_NONE.
double assemble(Mechanics& m, SolInfo* s, const Chain& c, const ErrorWeights* w, cudaStream_t stream);
// Size cap of the two-phase assembly's element buffer: a mesh whose buffer
// would be larger is assembled in chunks of elements (same sums, same order).
// 0 restores the default, a quarter of the device's memory.
void set_element_buffer_limit(long long bytes);
long long element_buffer_limit();
// Device time of the element-kernel phase and of the gather phase of every
// assemble() while enabled (enable clears the sums).
void assembly_timing(bool enable);
void assembly_timing_read(double* ms, long long* count);

// KS pre-pass over stored stresses (src/goal_ks_vm.cpp:36-76): max von Mises and scale.
void ks_prepass(Mechanics& m, double rho, double& max_vm, double& scale, cudaStream_t stream);

// Boundary conditions ----------------------------------------------------
struct DBC {
  int eq;
  NodeSet* set;
  ExprCode code;
};
struct TBC {
  SideSet* set;
  ExprCode code[3];
};

// set_resid_dbcs / set_jac_dbcs (src/goal_dbcs.cpp:39-99)
void apply_dbcs(Mechanics& m, SolInfo& s, const std::vector<DBC>& bcs, double t, bool jac, cudaStream_t stream);
// set_tbcs (src/goal_tbcs.cpp:29-85); Zd non-null selects the DWR weights
void apply_tbcs(Mechanics& m, SolInfo& s, const std::vector<TBC>& bcs, double t, const double* Zd,
                cudaStream_t stream);

}  // namespace goal
