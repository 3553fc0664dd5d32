// wg_noalloc.cu -- a force evaluation that allocates nothing.
//
// Some callers cannot call cudaMalloc: a host application whose device memory
// is owned by another framework's allocator and budget, code that must not
// trigger the device-wide synchronisation cudaMalloc/cudaFree imply, or a
// latency-critical loop that may not allocate at all.  wg_accel_noalloc serves
// them: the caller passes device buffers for the inputs and outputs and a
// stream; every intermediate (the two sorted sheet sets, the radix-sort keys,
// slots, histograms and look-back words, the force kernel's tile records and
// the per-call flags) lives in one file-scope __device__ array of fixed size,
// which every GPU that loads this library holds until the process exits.
//
// The array's name in host code is only a host-side stand-in, not a device
// address; the device address is looked up once per device with
// cudaGetSymbolAddress (on that device's first call) and passed to the
// kernels.  The inputs are device memory, so they are checked on the device:
// a non-finite position or mass, or a negative mass, skips the sort and makes
// the call return WG_ERR_ARG once its launches have run.
// All calls share the array and it keeps the last call's contents:
// the counters, flags and error word that must start at zero are cleared at
// the start of every call, and two calls that overlap on the GPU (different
// streams, or different host threads) race on it.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/wendy_gb300.h"
#include "wg_internal.cuh"

using namespace wg;

namespace {

constexpr int64_t kMaxSheets = WG_NOALLOC_MAX_SHEETS;
constexpr size_t kScratchBytes = (size_t)8 << 20;  // 8 MiB

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
unsigned char* g_scratch_dev[kMaxDevices];  // device address of the array, per device
unsigned g_epoch[kMaxDevices];              // next look-back epoch, per device

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

struct Layout {
  StateTable* table;
  StateRef set[2];
  TileRec* recs;
  RadixWork radix;
  double* a_sorted;
  unsigned* err;
  StepFlags* flags;  // [2]
  unsigned* ticket;
  double* t_seq;
  unsigned* epoch;
  size_t used;
};

// The array is carved for kMaxSheets; a call with fewer sheets uses a prefix
// of every region.
Layout carve(unsigned char* base, int64_t n) {
  Layout L;
  unsigned char* p = base;
  L.table = reinterpret_cast<StateTable*>(p); p += al(sizeof(StateTable));
  L.err = reinterpret_cast<unsigned*>(p); p += al(4);
  L.flags = reinterpret_cast<StepFlags*>(p); p += al(2 * sizeof(StepFlags));
  L.ticket = reinterpret_cast<unsigned*>(p); p += al(4);
  L.t_seq = reinterpret_cast<double*>(p); p += al(8);
  L.epoch = reinterpret_cast<unsigned*>(p); p += al(4);
  const size_t nd = al((size_t)kMaxSheets * 8), ni = al((size_t)kMaxSheets * 4);
  for (int k = 0; k < 2; ++k) {
    L.set[k].x = reinterpret_cast<double*>(p); p += nd;
    L.set[k].v = reinterpret_cast<double*>(p); p += nd;
    L.set[k].m = reinterpret_cast<double*>(p); p += nd;
    L.set[k].idx = reinterpret_cast<int32_t*>(p); p += ni;
  }
  L.a_sorted = reinterpret_cast<double*>(p); p += nd;
  const int64_t max_tiles = (kMaxSheets + kForceTile - 1) / kForceTile;
  L.recs = reinterpret_cast<TileRec*>(p); p += al(sizeof(TileRec) * (size_t)max_tiles);
  radix_bind(&L.radix, p, n);
  p += radix_bytes(kMaxSheets);
  L.used = (size_t)(p - base);
  return L;
}

// Host copy of the fixed-point conversion of a mass, round(m * 2^E).
u128 fixed_of(double m, int E) {
  uint64_t b;
  std::memcpy(&b, &m, 8);
  int ex = (int)((b >> 52) & 0x7FF);
  uint64_t mant = b & 0xFFFFFFFFFFFFFull;
  if (ex == 0) {
    if (mant == 0) return 0;
    ex = 1;
  } else {
    mant |= 1ull << 52;
  }
  const int s = ex - 1075 + E;
  if (s >= 0) return ((u128)mant) << s;
  const int r = -s;
  if (r > 54) return 0;
  return (u128)((mant + (1ull << (r - 1))) >> r);
}

int fail(int code, const char* fmt, ...) {
  char msg[256];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  record_last_error(msg);
  return code;
}

// Per-call set-up: the table of sheet sets, the time and epoch of the single
// force evaluation, and the zeroing of everything a call must start from.
__global__ void k_noalloc_setup(Layout L, double t, unsigned epoch) {
  if (threadIdx.x == 0) {
    L.table->cur = L.set[0];
    L.table->other = L.set[1];
    *L.err = 0;
    *L.ticket = 0;
    L.flags[0] = StepFlags{1u, 0u, 0ull};  // the sheets arrive unsorted
    L.flags[1] = StepFlags{0u, 0u, 0ull};
    *L.t_seq = t;
    *L.epoch = epoch;
  }
}

// Copy the caller's positions and masses into the first set, checking them.
__global__ void k_noalloc_load(Layout L, int64_t n, const double* x, const double* m) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  bool bad = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const double xi = x[i], mi = m[i];
    if (!isfinite(xi) || !isfinite(mi) || !(mi >= 0.0)) bad = true;
    L.set[0].x[i] = xi;
    L.set[0].v[i] = 0.0;
    L.set[0].m[i] = mi;
    L.set[0].idx[i] = (int32_t)i;
  }
  if (bad) {
    // the sort is skipped (its flag cleared); the call reports WG_ERR_ARG
    atomicOr(L.err, DEV_ERR_BAD_STATE);
    L.flags[0].unsorted = 0u;
  }
}

__global__ void k_noalloc_store(Layout L, int64_t n, double* a, int32_t* perm) {
  const StateRef cur = L.table->cur;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int32_t j = cur.idx[i];
    if (a) a[j] = L.a_sorted[i];
    if (perm) perm[i] = j;
  }
}

}  // namespace

extern "C" int wg_accel_noalloc(int64_t n, const double* x, const double* m, double totmass,
                                double omega2, int ext_kind, const double* ext_params,
                                int n_ext_params, double t, double* a, int32_t* perm,
                                void* stream) {
  if (n < 1 || n > kMaxSheets)
    return fail(WG_ERR_ARG,
                "wg_accel_noalloc: n = %lld is outside [1, %lld], the size its fixed "
                "device scratch array was built for",
                (long long)n, (long long)kMaxSheets);
  if (!x || !m || (!a && !perm)) return fail(WG_ERR_ARG, "wg_accel_noalloc: null buffer");
  if (!std::isfinite(totmass) || totmass < 0 || !std::isfinite(omega2))
    return fail(WG_ERR_ARG, "wg_accel_noalloc: totmass must be finite and >= 0");
  ExtForce ext{};
  ext.kind = ext_kind;
  for (int i = 0; i < 4; ++i) ext.p[i] = 0.0;
  const int need = ext_kind == WG_EXT_NONE ? 0 : ext_kind == WG_EXT_HARMONIC ? 1
                 : ext_kind == WG_EXT_PULSE_TANH ? 4 : -1;
  if (ext_kind == WG_EXT_EXPR)
    return fail(WG_ERR_EXT, "wg_accel_noalloc: an expression force's program needs device "
                            "memory of its own; use wg_accel");
  if (need < 0 || n_ext_params < need || (need > 0 && !ext_params))
    return fail(WG_ERR_EXT, "wg_accel_noalloc: unknown external force %d or too few parameters",
                ext_kind);
  for (int i = 0; i < need; ++i) ext.p[i] = ext_params[i];
  if (ext_kind == WG_EXT_PULSE_TANH && (ext.p[2] == 0.0 || ext.p[3] == 0.0))
    return fail(WG_ERR_EXT, "wg_accel_noalloc: pulsed force needs tau != 0 and h != 0");
  // the pulsed force's tanh table is a __device__ array of the library, set
  // up on the device's first use (no allocation)
  if (ext_kind == WG_EXT_PULSE_TANH && !(ext.ttab = tanh_table()))
    return fail(WG_ERR_CUDA, "wg_accel_noalloc: the tanh table could not be set up");

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fail(WG_ERR_NODEV, "wg_accel_noalloc: no usable CUDA device");
  }
  unsigned char* base = nullptr;
  unsigned epoch = 0;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_dev[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return fail(WG_ERR_CUDA, "wg_accel_noalloc: cudaGetSymbolAddress failed: %s",
                    cudaGetErrorString(e));
      g_scratch_dev[dev] = static_cast<unsigned char*>(p);
      g_epoch[dev] = 1;
    }
    base = g_scratch_dev[dev];
    epoch = g_epoch[dev]++;
  }
  Layout L = carve(base, n);
  if (L.used > kScratchBytes)
    return fail(WG_ERR_ARG, "wg_accel_noalloc: internal layout exceeds the scratch array");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (epoch >= (1u << 29)) {
    // keep (epoch << 2) in 32 bits: forget old tile records and restart
    const int64_t max_tiles = (kMaxSheets + kForceTile - 1) / kForceTile;
    cudaMemsetAsync(L.recs, 0, sizeof(TileRec) * (size_t)max_tiles, s);
    std::lock_guard<std::mutex> lock(g_mu);
    g_epoch[dev] = 2;
    epoch = 1;
  }
  int eT = 0;
  int E = 0;
  if (totmass > 0) {
    std::frexp(totmass, &eT);
    E = 123 - eT;
  }
  const u128 T = fixed_of(totmass, E);

  k_noalloc_setup<<<1, 32, 0, s>>>(L, t, epoch);
  k_noalloc_load<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(L, n, x, m);
  radix_sort_state(L.table, n, &L.radix, &L.flags[0], L.err, s);
  ForceArgs f;
  f.table = L.table;
  f.n = n;
  f.T_lo = (uint64_t)T;
  f.T_hi = (uint64_t)(T >> 64);
  f.E = E;
  f.has_omega = omega2 >= 0;
  f.omega2 = omega2;
  f.ext = ext;
  f.t_seq = L.t_seq;
  f.epochs = L.epoch;
  f.sub = 0;
  f.a_out = L.a_sorted;
  f.recs = L.recs;
  f.ticket = L.ticket;
  f.flag_out = &L.flags[1];
  f.err = L.err;
  f.dt_kick = 0.0;
  f.dt_drift = 0.0;
  launch_force(f, (n + kForceTile - 1) / kForceTile, s);
  k_noalloc_store<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(L, n, a, perm);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(WG_ERR_CUDA, "wg_accel_noalloc: launch failed: %s",
                                    cudaGetErrorString(e));
  unsigned err = 0;
  e = cudaMemcpyAsync(&err, L.err, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
    return fail(WG_ERR_CUDA, "wg_accel_noalloc: %s", cudaGetErrorString(e));
  if (err & DEV_ERR_BAD_STATE)
    return fail(WG_ERR_ARG, "wg_accel_noalloc: a position or mass is not finite, or a mass is "
                            "negative");
  if (err) return fail(WG_ERR_DEVICE, "wg_accel_noalloc: device error word 0x%x", err);
  return WG_OK;
}
