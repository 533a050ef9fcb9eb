// Boundary-condition expressions in x, y, z, t.
//
// goal evaluates Dirichlet and traction values with a run-time compiled C
// expression (goal::eval, src/goal_control.cpp:107-123; used per node at
// src/goal_dbcs.cpp:26-37 and per side at src/goal_tbcs.cpp:59-60). Here the
// host parses the expression once into a small postfix program that both the
// host and the device interpret, so the per-node values are computed on the
// GPU inside the boundary-condition kernels.
#pragma once

#include <string>

#ifdef __CUDACC__
#define GOAL_HD __host__ __device__
#else
#define GOAL_HD
#endif

#include <cmath>

namespace goal {

enum ExprOp : unsigned char {
  EX_CONST = 0, EX_X, EX_Y, EX_Z, EX_T,
  EX_ADD, EX_SUB, EX_MUL, EX_DIV, EX_POW, EX_NEG,
  EX_SIN, EX_COS, EX_TAN, EX_ASIN, EX_ACOS, EX_ATAN, EX_EXP, EX_LOG, EX_LOG10,
  EX_SQRT, EX_FABS, EX_SINH, EX_COSH, EX_TANH, EX_FLOOR, EX_CEIL, EX_ATAN2, EX_FMOD,
};

struct ExprCode {
  static constexpr int kMaxOps = 64;
  static constexpr int kMaxConst = 24;
  static constexpr int kMaxStack = 16;
  int num_ops = 0;
  unsigned char op[kMaxOps];
  unsigned char arg[kMaxOps];  // constant index for EX_CONST
  double c[kMaxConst];
};

// Parses ``text`` into ``out``; returns false and fills ``err`` on failure.
bool compile_expr(const std::string& text, ExprCode& out, std::string& err);

GOAL_HD inline double eval_expr(const ExprCode& e, double x, double y, double z, double t) {
  double st[ExprCode::kMaxStack];
  int sp = 0;
  for (int i = 0; i < e.num_ops; ++i) {
    switch (e.op[i]) {
      case EX_CONST: st[sp++] = e.c[e.arg[i]]; break;
      case EX_X: st[sp++] = x; break;
      case EX_Y: st[sp++] = y; break;
      case EX_Z: st[sp++] = z; break;
      case EX_T: st[sp++] = t; break;
      case EX_ADD: --sp; st[sp - 1] = st[sp - 1] + st[sp]; break;
      case EX_SUB: --sp; st[sp - 1] = st[sp - 1] - st[sp]; break;
      case EX_MUL: --sp; st[sp - 1] = st[sp - 1] * st[sp]; break;
      case EX_DIV: --sp; st[sp - 1] = st[sp - 1] / st[sp]; break;
      case EX_POW: --sp; st[sp - 1] = pow(st[sp - 1], st[sp]); break;
      case EX_ATAN2: --sp; st[sp - 1] = atan2(st[sp - 1], st[sp]); break;
      case EX_FMOD: --sp; st[sp - 1] = fmod(st[sp - 1], st[sp]); break;
      case EX_NEG: st[sp - 1] = -st[sp - 1]; break;
      case EX_SIN: st[sp - 1] = sin(st[sp - 1]); break;
      case EX_COS: st[sp - 1] = cos(st[sp - 1]); break;
      case EX_TAN: st[sp - 1] = tan(st[sp - 1]); break;
      case EX_ASIN: st[sp - 1] = asin(st[sp - 1]); break;
      case EX_ACOS: st[sp - 1] = acos(st[sp - 1]); break;
      case EX_ATAN: st[sp - 1] = atan(st[sp - 1]); break;
      case EX_EXP: st[sp - 1] = exp(st[sp - 1]); break;
      case EX_LOG: st[sp - 1] = log(st[sp - 1]); break;
      case EX_LOG10: st[sp - 1] = log10(st[sp - 1]); break;
      case EX_SQRT: st[sp - 1] = sqrt(st[sp - 1]); break;
      case EX_FABS: st[sp - 1] = fabs(st[sp - 1]); break;
      case EX_SINH: st[sp - 1] = sinh(st[sp - 1]); break;
      case EX_COSH: st[sp - 1] = cosh(st[sp - 1]); break;
      case EX_TANH: st[sp - 1] = tanh(st[sp - 1]); break;
      case EX_FLOOR: st[sp - 1] = floor(st[sp - 1]); break;
      case EX_CEIL: st[sp - 1] = ceil(st[sp - 1]); break;
      default: break;
    }
  }
  return sp > 0 ? st[sp - 1] : 0.0;
}

}  // namespace goal
