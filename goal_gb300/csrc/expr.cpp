// Recursive-descent parser for boundary-condition expressions (see expr.h).
//   expr   := term (('+'|'-') term)*
//   term   := unary (('*'|'/') unary)*
//   unary  := ('-'|'+') unary | power
//   power  := atom ('^' unary)?
//   atom   := number | x | y | z | t | pi | name '(' expr (',' expr)? ')' | '(' expr ')'
#include "expr.h"

#include <cctype>
#include <cstdlib>
#include <cstring>

namespace goal {

namespace {

struct Parser {
  const std::string& s;
  size_t i = 0;
  ExprCode& out;
  std::string err;
  int depth = 0, max_depth = 0;
  Parser(const std::string& str, ExprCode& o) : s(str), out(o) {}

  void ws() { while (i < s.size() && std::isspace((unsigned char)s[i])) ++i; }
  bool emit(unsigned char op, unsigned char arg = 0, int push = 0) {
    if (out.num_ops >= ExprCode::kMaxOps) { err = "expression too long"; return false; }
    out.op[out.num_ops] = op;
    out.arg[out.num_ops] = arg;
    out.num_ops++;
    depth += push;
    if (depth > max_depth) max_depth = depth;
    if (max_depth > ExprCode::kMaxStack) { err = "expression nests too deeply"; return false; }
    return true;
  }
  bool constant(double v) {
    int n = 0;
    for (int k = 0; k < out.num_ops; ++k) if (out.op[k] == EX_CONST && out.arg[k] >= n) n = out.arg[k] + 1;
    if (n >= ExprCode::kMaxConst) { err = "too many constants"; return false; }
    out.c[n] = v;
    return emit(EX_CONST, (unsigned char)n, 1);
  }
  bool expr() {
    if (!term()) return false;
    for (;;) {
      ws();
      if (i < s.size() && (s[i] == '+' || s[i] == '-')) {
        char c = s[i++];
        if (!term()) return false;
        if (!emit(c == '+' ? EX_ADD : EX_SUB, 0, -1)) return false;
      } else {
        return true;
      }
    }
  }
  bool term() {
    if (!unary()) return false;
    for (;;) {
      ws();
      if (i < s.size() && (s[i] == '*' || s[i] == '/')) {
        char c = s[i++];
        if (!unary()) return false;
        if (!emit(c == '*' ? EX_MUL : EX_DIV, 0, -1)) return false;
      } else {
        return true;
      }
    }
  }
  bool unary() {
    ws();
    if (i < s.size() && s[i] == '-') { ++i; if (!unary()) return false; return emit(EX_NEG); }
    if (i < s.size() && s[i] == '+') { ++i; return unary(); }
    return power();
  }
  bool power() {
    if (!atom()) return false;
    ws();
    if (i < s.size() && s[i] == '^') {
      ++i;
      if (!unary()) return false;
      return emit(EX_POW, 0, -1);
    }
    return true;
  }
  bool atom() {
    ws();
    if (i >= s.size()) { err = "unexpected end of expression"; return false; }
    char c = s[i];
    if (c == '(') {
      ++i;
      if (!expr()) return false;
      ws();
      if (i >= s.size() || s[i] != ')') { err = "missing ')'"; return false; }
      ++i;
      return true;
    }
    if (std::isdigit((unsigned char)c) || c == '.') {
      const char* b = s.c_str() + i;
      char* e = nullptr;
      double v = std::strtod(b, &e);
      if (e == b) { err = "bad number"; return false; }
      i += (size_t)(e - b);
      return constant(v);
    }
    if (std::isalpha((unsigned char)c) || c == '_') {
      size_t b = i;
      while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '_')) ++i;
      std::string name = s.substr(b, i - b);
      ws();
      if (i < s.size() && s[i] == '(') {
        ++i;
        struct F { const char* n; unsigned char op; int args; };
        static const F fns[] = {
            {"sin", EX_SIN, 1}, {"cos", EX_COS, 1}, {"tan", EX_TAN, 1}, {"asin", EX_ASIN, 1},
            {"acos", EX_ACOS, 1}, {"atan", EX_ATAN, 1}, {"exp", EX_EXP, 1}, {"log", EX_LOG, 1},
            {"log10", EX_LOG10, 1}, {"sqrt", EX_SQRT, 1}, {"fabs", EX_FABS, 1}, {"abs", EX_FABS, 1},
            {"sinh", EX_SINH, 1}, {"cosh", EX_COSH, 1}, {"tanh", EX_TANH, 1}, {"floor", EX_FLOOR, 1},
            {"ceil", EX_CEIL, 1}, {"pow", EX_POW, 2}, {"atan2", EX_ATAN2, 2}, {"fmod", EX_FMOD, 2}};
        const F* f = nullptr;
        for (const F& g : fns) if (name == g.n) f = &g;
        if (!f) { err = "unknown function: " + name; return false; }
        if (!expr()) return false;
        if (f->args == 2) {
          ws();
          if (i >= s.size() || s[i] != ',') { err = "expected ',' in " + name; return false; }
          ++i;
          if (!expr()) return false;
        }
        ws();
        if (i >= s.size() || s[i] != ')') { err = "missing ')' after " + name; return false; }
        ++i;
        return emit(f->op, 0, f->args == 2 ? -1 : 0);
      }
      if (name == "x") return emit(EX_X, 0, 1);
      if (name == "y") return emit(EX_Y, 0, 1);
      if (name == "z") return emit(EX_Z, 0, 1);
      if (name == "t") return emit(EX_T, 0, 1);
      if (name == "pi") return constant(3.14159265358979323846);
      err = "unknown variable: " + name;
      return false;
    }
    err = std::string("unexpected character '") + c + "'";
    return false;
  }
};

}  // namespace

bool compile_expr(const std::string& text, ExprCode& out, std::string& err) {
  out = ExprCode();
  Parser p(text, out);
  bool ok = p.expr();
  if (ok) {
    p.ws();
    if (p.i != text.size()) { ok = false; p.err = "trailing characters in expression"; }
  }
  if (!ok) err = p.err + " in \"" + text + "\"";
  return ok;
}

}  // namespace goal
