// wg_common.cuh -- shared device helpers of the GB300 approximate integrator.
//
// Order-preserving position keys, the exact fixed-point mass arithmetic the
// force kernel is built on, and the acquire/release primitives of the
// decoupled look-back scans.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "wg_tanh.cuh"

namespace wg {

typedef unsigned __int128 u128;
typedef __int128 i128;

// Device error word bits (read back by the host after every call).
enum : unsigned {
  DEV_ERR_LOOKBACK_TIMEOUT = 1u << 0,  // a look-back wait hit its iteration limit
  DEV_ERR_RADIX_TIMEOUT = 1u << 1,     // a radix-sort look-back wait hit its limit
  DEV_ERR_BUCKET_OVERFLOW = 1u << 2,   // a bucket received more sheets than its capacity
  DEV_ERR_FIXED_RANGE = 1u << 3,       // a mass outside the fixed-point range
  DEV_ERR_BAD_STATE = 1u << 4,         // an internal consistency check failed
  DEV_ERR_COPY_TIMEOUT = 1u << 5,      // a bulk copy into shared memory did not complete
};

// Upper bound on the iterations of any spin-wait on another CTA's flag.  Each
// iteration backs off with __nanosleep, so the bound is well above a second
// of wall time; after it the waiter records an error and stops waiting.
constexpr unsigned kSpinLimit = 1u << 22;

// ---------------------------------------------------------------------------
// Position keys.  key_of is strictly increasing in x over the non-NaN doubles
// except that -0.0 and +0.0 share a key (the reference's comparator treats
// them as equal, wendy/wendy.c:21).  Sorting by (key, original index) is the
// total order every path of this library uses.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t key_of(double x) {
  uint64_t b = (uint64_t)__double_as_longlong(x);
  if (b == 0x8000000000000000ull) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// ---------------------------------------------------------------------------
// Fixed-point masses.  A mass m >= 0 is represented by the integer
// round(m * 2^E) in 128 bits, where the host picks E so that
// 8 * totmass * 2^E < 2^127.  Prefix sums of these integers are exact and
// independent of association order, so the cumulative mass -- and with it the
// acceleration -- does not depend on tile size, look-back pattern or batching.
// The acceleration totmass - 2 C_i - m_i (wendy/wendy.c:375-383) is formed
// exactly in the integers and rounded to double once.
// ---------------------------------------------------------------------------
__device__ __forceinline__ u128 mass_to_fixed(double m, int E) {
  uint64_t b = (uint64_t)__double_as_longlong(m);
  int ex = (int)((b >> 52) & 0x7FF);
  uint64_t mant = b & 0xFFFFFFFFFFFFFull;
  if (ex == 0) {
    if (mant == 0) return 0;
    ex = 1;
  } else {
    mant |= 1ull << 52;
  }
  int s = ex - 1075 + E;  // m = mant * 2^(ex - 1075)
  if (s >= 0) return ((u128)mant) << s;
  int r = -s;
  if (r > 54) return 0;  // below half a unit
  return (u128)((mant + (1ull << (r - 1))) >> r);
}

// Signed 128-bit integer A times 2^-E, rounded to nearest even.  The normal
// range is handled with integer operations only (FP64 issue slots are the
// scarce resource on this part): the top 64 bits of |A| are normalised with
// one count-leading-zeros, the mantissa is their top 53 bits and the rest
// (plus a sticky bit for everything below) decides the rounding.  Values
// below 2^64 units or outside the normal exponent range take ldexp.
static __device__ __noinline__ double fixed_to_double_slow(i128 A, int E) {
  const bool neg = A < 0;
  const u128 u = neg ? (u128)(-A) : (u128)A;
  if (u == 0) return 0.0;
  const uint64_t hi = (uint64_t)(u >> 64), lo = (uint64_t)u;
  const int lz = hi ? __clzll((long long)hi) : 64 + __clzll((long long)lo);
  const int p = 127 - lz;
  uint64_t mant;
  int e2;
  if (p <= 52) {
    mant = lo << (52 - p);
    e2 = p - 52;
  } else {
    int sh = p - 52;
    mant = (uint64_t)(u >> sh);
    const u128 rem = u & ((((u128)1) << sh) - 1);
    const u128 half = ((u128)1) << (sh - 1);
    if (rem > half || (rem == half && (mant & 1ull))) {
      ++mant;
      if (mant == (1ull << 53)) {
        mant >>= 1;
        ++sh;
      }
    }
    e2 = sh;
  }
  const double r = ldexp((double)mant, e2 - E);
  return neg ? -r : r;
}

__device__ __forceinline__ double fixed_to_double(i128 A, int E) {
  const bool neg = A < 0;
  const u128 u = neg ? (u128)(-A) : (u128)A;
  const uint64_t hi = (uint64_t)(u >> 64), lo = (uint64_t)u;
  if (hi == 0) return fixed_to_double_slow(A, E);
  const int lz = __clzll((long long)hi);
  const uint64_t t = lz ? (hi << lz) | (lo >> (64 - lz)) : hi;  // top 64 bits
  const uint64_t rest = lo << lz;                                  // bits below t
  uint64_t mant = t >> 11;
  const uint64_t r = t & 0x7FFull;
  int bexp = 127 - lz - E + 1023;
  if (r > 0x400ull || (r == 0x400ull && (rest != 0 || (mant & 1ull)))) {
    ++mant;
    if (mant == (1ull << 53)) {
      mant >>= 1;
      ++bexp;
    }
  }
  if (bexp <= 0 || bexp >= 2047) return fixed_to_double_slow(A, E);
  const uint64_t bits = ((uint64_t)bexp << 52) | (mant & 0xFFFFFFFFFFFFFull) |
                        (neg ? 0x8000000000000000ull : 0ull);
  return __longlong_as_double((long long)bits);
}

// ---------------------------------------------------------------------------
// Memory-model helpers for flags that other CTAs spin on.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Relaxed (gpu scope) accesses for status words that carry their whole
// payload: never merged or hoisted out of a spin, free to overlap.
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ void st_relaxed_u32(unsigned* p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_cg_u64(const uint64_t* p) {
  return (uint64_t)__ldcg((const unsigned long long*)p);
}

// ---------------------------------------------------------------------------
// Bulk (TMA) copies global -> shared memory completed on an mbarrier.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
// Make generic-proxy shared-memory accesses visible to later async-proxy
// (bulk copy) accesses of the same CTA, and the mbarrier initialisation.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
// 16-byte aligned addresses, size a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// Bulk prefetch of global memory into L2 (16-byte aligned, size a multiple of 16).
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}
// Wait for the phase with the given parity; false if the bounded wait expired.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  for (unsigned it = 0; it < kSpinLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Warp-wide inclusive scan of a 128-bit unsigned value.
__device__ __forceinline__ u128 warp_inclusive_scan_u128(u128 v, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint64_t lo = __shfl_up_sync(0xffffffffu, (unsigned long long)(uint64_t)v, d);
    const uint64_t hi = __shfl_up_sync(0xffffffffu, (unsigned long long)(uint64_t)(v >> 64), d);
    if (lane >= d) v += (((u128)hi) << 64) | lo;
  }
  return v;
}

__device__ __forceinline__ u128 shfl_u128(u128 v, int src) {
  const uint64_t lo = __shfl_sync(0xffffffffu, (unsigned long long)(uint64_t)v, src);
  const uint64_t hi = __shfl_sync(0xffffffffu, (unsigned long long)(uint64_t)(v >> 64), src);
  return (((u128)hi) << 64) | lo;
}

__device__ __forceinline__ u128 warp_sum_u128(u128 v) {
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    const uint64_t lo = __shfl_xor_sync(0xffffffffu, (unsigned long long)(uint64_t)v, d);
    const uint64_t hi = __shfl_xor_sync(0xffffffffu, (unsigned long long)(uint64_t)(v >> 64), d);
    v += (((u128)hi) << 64) | lo;
  }
  return v;
}

// ---------------------------------------------------------------------------
// Registered external forces (closed forms replacing wendy's ext_force
// callables, wendy/wendy.py:389-418).
// ---------------------------------------------------------------------------
enum : int { EXT_NONE = 0, EXT_HARMONIC = 1, EXT_PULSE_TANH = 2, EXT_EXPR = 3, EXT_MAX = 3 };

// Compiled expression forces (EXT_EXPR).  wendy accepts any F(x, t) and
// compiles it with numba (wendy/wendy.py:389-404); here a restricted F is
// compiled on the host (wendy_gb300/extforce.py) into a short register
// program that the force kernels interpret.  The program has two phases:
// ops [0, n_time) use only t and constants and run once per force
// evaluation and thread; ops [n_time, n_ops) run per sheet with x.  The
// result is the register the last op writes.
constexpr int kExprMaxOps = 64;
constexpr int kExprRegs = 16;
enum : int {
  XOP_X = 0, XOP_T, XOP_K, XOP_MOV, XOP_ADD, XOP_SUB, XOP_MUL, XOP_DIV, XOP_NEG, XOP_POW,
  XOP_EXP, XOP_LOG, XOP_SQRT, XOP_SIN, XOP_COS, XOP_TAN, XOP_TANH, XOP_SINH, XOP_COSH,
  XOP_ATAN, XOP_ABS, XOP_COUNT
};
struct ExprOp {
  int code;
  int dst, a, b;  // registers
  double k;       // the constant of XOP_K
};

struct ExtForce {
  int kind;
  double p[4];
  const ExprOp* prog;  // EXT_EXPR: the program, in device memory
  int n_ops;
  int n_time;
  const long long* ttab;  // EXT_PULSE_TANH: the device's tanh table (wg_tanh.cuh)
};

// Runs ops [lo, hi) of an expression program on the registers r.
static __device__ __noinline__ void expr_run(const ExprOp* __restrict__ prog, int lo, int hi,
                                             double* r, double x, double t) {
  for (int i = lo; i < hi; ++i) {
    const ExprOp o = prog[i];  // the same op in every thread: a broadcast load
    const double va = r[o.a], vb = r[o.b];
    double y;
    switch (o.code) {
      case XOP_X: y = x; break;
      case XOP_T: y = t; break;
      case XOP_K: y = o.k; break;
      case XOP_MOV: y = va; break;
      case XOP_ADD: y = va + vb; break;
      case XOP_SUB: y = va - vb; break;
      case XOP_MUL: y = va * vb; break;
      case XOP_DIV: y = va / vb; break;
      case XOP_NEG: y = -va; break;
      case XOP_POW: y = pow(va, vb); break;
      case XOP_EXP: y = exp(va); break;
      case XOP_LOG: y = log(va); break;
      case XOP_SQRT: y = sqrt(va); break;
      case XOP_SIN: y = sin(va); break;
      case XOP_COS: y = cos(va); break;
      case XOP_TAN: y = tan(va); break;
      case XOP_TANH: y = tanh(va); break;
      case XOP_SINH: y = sinh(va); break;
      case XOP_COSH: y = cosh(va); break;
      case XOP_ATAN: y = atan(va); break;
      default: y = fabs(va); break;  // XOP_ABS
    }
    r[o.dst] = y;
  }
}

// The time phase of an expression force at time t (once per force
// evaluation; the registers then serve every sheet).
__device__ __forceinline__ void expr_time(const ExtForce& f, double t, double* r) {
  expr_run(f.prog, 0, f.n_time, r, 0.0, t);
}
// F(x) of an expression force after its time phase.
__device__ __forceinline__ double expr_space(const ExtForce& f, double* r, double x, double t) {
  expr_run(f.prog, f.n_time, f.n_ops, r, x, t);
  return r[f.prog[f.n_ops - 1].dst];
}

// Time factor of the pulsed force, A exp(-(t-t0)^2 / (2 tau^2)); evaluated
// once per force evaluation, with the numpy expression's operation order.
__device__ __forceinline__ double pulse_amplitude(const ExtForce& f, double t) {
  const double d = t - f.p[1];
  return f.p[0] * exp(-(d * d) / (2.0 * (f.p[2] * f.p[2])));
}

// F(x, t) given the per-evaluation amplitude `amp` and inv_h = 1 / h (pulse)
// -- harmonic: -p0 x; pulse: amp * tanh(x / h), as amp * tanh(x * inv_h) with
// the table-driven integer-pipe tanh (wg_tanh.cuh).
__device__ __forceinline__ double ext_force_at(const ExtForce& f, double amp, double inv_h,
                                               double x) {
  if (f.kind == EXT_HARMONIC) return -f.p[0] * x;
  if (f.kind == EXT_PULSE_TANH) return amp * tanh_tab(f.ttab, x * inv_h);
  return 0.0;
}

}  // namespace wg
