// wg_ext.cuh -- host side of the registered external forces: the checks of
// an (id, parameters) pair from the C ABI, shared by every entry point.
//
// The reference hands any Python callable F(x, t) to its C step as a
// function pointer (wendy/wendy.py:389-418).  Here a force is a registered
// id with parameters: two closed forms (harmonic, pulsed tanh) and compiled
// expressions (WG_EXT_EXPR), whose parameters are the program that
// wendy_gb300/extforce.py compiles from a restricted F(x, t):
//
//   p[0] = number of ops (1 .. kExprMaxOps), p[1] = ops of the time phase,
//   then per op five numbers: code, dst, a, b, k (see ExprOp).
//
// The program is checked completely here: known codes, registers in range,
// every register read written by an earlier op, no x in the time phase.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstring>

#include "../../include/wendy_gb300.h"
#include "wg_common.cuh"

namespace wg {

// A force as the kernels see it plus, for an expression, its program on the
// host (ExtForce::prog points to a device copy once one is attached).
struct ExtSpec {
  ExtForce f{};
  ExprOp ops[kExprMaxOps];
};

inline bool integral_in(double v, int lo, int hi) {
  return std::isfinite(v) && v == std::floor(v) && v >= lo && v <= hi;
}

inline bool expr_reads_a(int code) { return code >= XOP_MOV; }
inline bool expr_reads_b(int code) {
  return code == XOP_ADD || code == XOP_SUB || code == XOP_MUL || code == XOP_DIV ||
         code == XOP_POW;
}

// Checks (kind, p[0 .. np)) and fills *spec.  Returns WG_OK, or WG_ERR_EXT
// with the reason in err.
inline int parse_ext(int kind, const double* p, int np, ExtSpec* spec, char* err,
                     size_t errlen) {
  ExtForce& f = spec->f;
  f = ExtForce{};
  f.kind = kind;
  if (kind == WG_EXT_NONE) return WG_OK;
  if (kind == WG_EXT_HARMONIC || kind == WG_EXT_PULSE_TANH) {
    const int need = kind == WG_EXT_HARMONIC ? 1 : 4;
    if (np < need || !p) {
      std::snprintf(err, errlen, "external force %d needs %d parameters, got %d", kind, need, np);
      return WG_ERR_EXT;
    }
    for (int i = 0; i < need; ++i) {
      if (!std::isfinite(p[i])) {
        std::snprintf(err, errlen, "external-force parameter %d is not finite", i);
        return WG_ERR_EXT;
      }
      f.p[i] = p[i];
    }
    if (kind == WG_EXT_PULSE_TANH && (p[2] == 0.0 || p[3] == 0.0)) {
      std::snprintf(err, errlen, "pulsed force needs tau != 0 and h != 0");
      return WG_ERR_EXT;
    }
    if (kind == WG_EXT_PULSE_TANH && !(f.ttab = tanh_table())) {
      std::snprintf(err, errlen, "the pulsed force's tanh table could not be set up on the device");
      return WG_ERR_CUDA;
    }
    return WG_OK;
  }
  if (kind != WG_EXT_EXPR) {
    std::snprintf(err, errlen, "unknown external-force id %d", kind);
    return WG_ERR_EXT;
  }
  if (!p || np < 2 || !integral_in(p[0], 1, kExprMaxOps) || !integral_in(p[1], 0, (int)p[0])) {
    std::snprintf(err, errlen, "expression force: bad program header (ops 1..%d)", kExprMaxOps);
    return WG_ERR_EXT;
  }
  const int n_ops = (int)p[0], n_time = (int)p[1];
  if (np < 2 + 5 * n_ops) {
    std::snprintf(err, errlen, "expression force: %d ops need %d parameters, got %d", n_ops,
                  2 + 5 * n_ops, np);
    return WG_ERR_EXT;
  }
  bool written[kExprRegs] = {};
  for (int i = 0; i < n_ops; ++i) {
    const double* q = p + 2 + 5 * i;
    if (!integral_in(q[0], 0, XOP_COUNT - 1) || !integral_in(q[1], 0, kExprRegs - 1) ||
        !integral_in(q[2], 0, kExprRegs - 1) || !integral_in(q[3], 0, kExprRegs - 1) ||
        !std::isfinite(q[4])) {
      std::snprintf(err, errlen, "expression force: op %d is malformed", i);
      return WG_ERR_EXT;
    }
    ExprOp& o = spec->ops[i];
    o.code = (int)q[0];
    o.dst = (int)q[1];
    o.a = (int)q[2];
    o.b = (int)q[3];
    o.k = q[4];
    if (i < n_time && o.code == XOP_X) {
      std::snprintf(err, errlen, "expression force: op %d reads x in the time phase", i);
      return WG_ERR_EXT;
    }
    if ((expr_reads_a(o.code) && !written[o.a]) || (expr_reads_b(o.code) && !written[o.b])) {
      std::snprintf(err, errlen, "expression force: op %d reads a register no op wrote", i);
      return WG_ERR_EXT;
    }
    // unary ops read b too (a register load the interpreter does for every
    // op): point it at a
    if (!expr_reads_b(o.code)) o.b = o.a;
    written[o.dst] = true;
  }
  f.n_ops = n_ops;
  f.n_time = n_time;
  return WG_OK;
}

// Copies an expression force's program to device memory *d_prog (allocated
// on first use, kExprMaxOps ops) and points the force at it.  A no-op for
// the closed forms.
inline cudaError_t attach_ext_program(ExtSpec* spec, ExprOp** d_prog, cudaStream_t s) {
  if (spec->f.kind != EXT_EXPR) {
    spec->f.prog = nullptr;
    return cudaSuccess;
  }
  if (!*d_prog) {
    const cudaError_t e = cudaMalloc(d_prog, sizeof(ExprOp) * kExprMaxOps);
    if (e != cudaSuccess) return e;
  }
  const cudaError_t e = cudaMemcpyAsync(*d_prog, spec->ops, sizeof(ExprOp) * spec->f.n_ops,
                                        cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  spec->f.prog = *d_prog;
  return cudaSuccess;
}

// Whether two forces are the same (the closed forms by their parameters,
// expressions by their programs).
inline bool same_ext(const ExtSpec& a, const ExtSpec& b) {
  if (a.f.kind != b.f.kind) return false;
  if (std::memcmp(a.f.p, b.f.p, sizeof(a.f.p)) != 0) return false;
  if (a.f.kind != EXT_EXPR) return true;
  if (a.f.n_ops != b.f.n_ops || a.f.n_time != b.f.n_time) return false;
  for (int i = 0; i < a.f.n_ops; ++i) {
    const ExprOp &x = a.ops[i], &y = b.ops[i];
    if (x.code != y.code || x.dst != y.dst || x.a != y.a || x.b != y.b ||
        std::memcmp(&x.k, &y.k, sizeof(double)) != 0)
      return false;
  }
  return true;
}

}  // namespace wg
