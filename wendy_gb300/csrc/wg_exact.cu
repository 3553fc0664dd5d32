// wg_exact.cu -- wendy's exact event-driven solver (approx=False) on the GPU.
//
// Between collisions every sheet moves under a constant acceleration (or,
// with a harmonic external potential, on a shifted harmonic orbit), so the
// next crossing of two neighbours in position order is the root of a
// quadratic (or of a sinusoid).  The solver processes crossings one at a
// time in time order: advance the two sheets to the crossing, swap them,
// exchange their accelerations by the mass difference, and recompute the
// crossing times of the three neighbour pairs that changed.  The reference
// keeps the pair times in an unbalanced binary search tree
// (wendy/wendy.c:53-315, wendy/bst.c); here one warp owns the whole event
// loop and keeps them in a 32-ary tournament tree (each internal node holds
// the minimum of its 32 children and where it lies), so the next event is a
// read of the root and an update rewrites three leaves and their paths, each
// level one coalesced 32-wide load and a warp minimum.  The state lives in
// shared memory when it fits (a few thousand sheets), in global memory
// otherwise; the loop is a strict sequence of dependent steps, which is why
// this stays a cross-check at small N rather than a fast path.
//
// Arithmetic, operation order and the per-sheet clocks follow the
// reference (this file is compiled without FMA contraction, as the
// reference's C is), so trajectories agree to rounding; pair times that are NaN
// (pairs that never meet in the harmonic case) never come first, and among
// equal pair times the lowest pair index comes first.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/wendy_gb300.h"
#include "wg_internal.cuh"

using namespace wg;

namespace {

constexpr int kTreeFan = 32;
constexpr int kMaxLevels = 6;  // 32^6 pair times: more than any N this accepts

struct ExactState {
  double* x;
  double* v;
  double* a;
  double* m;
  double* t;      // each sheet's own clock within the output interval
  int32_t* sindx; // sheet at each position
  double* tcoll;  // crossing time of the pair at positions (i, i + 1)
};

struct ExactArgs {
  ExactState g;        // global memory copy of the state
  int n;
  double omega;        // > 0: harmonic external potential
  double dt;
  long long maxcoll;
  // internal levels of the tournament tree: the order key of the smallest
  // pair time below each node (see time_key) and that pair's index
  uint64_t* tree_key[kMaxLevels];
  int32_t* tree_idx[kMaxLevels];
  int levels;
  int level_n[kMaxLevels + 1];   // entries per level (level 0: the n - 1 pair times)
  int* cindx;          // in/out: pair of the next crossing
  double* next_tcoll;  // in/out: its time
  long long* ncoll;    // out: crossings processed
  int* err;            // out: -2 when maxcoll was reached
  int use_smem;        // the state is staged in shared memory (after the tree)
  size_t tree_bytes;   // shared memory of the tree's internal levels (16-byte multiple)
};

// The reference's root of the crossing quadratic c2 t^2 + c1 t + c0 = 0
// (wendy/wendy.c:33-38).
__device__ double solve_coll_quad(double c0, double c1, double c2) {
  const double mba = -c1 / c2;
  return 0.5 * (mba + sqrt(mba * mba - 4. * c0 / c2));
}

// The reference's first crossing under harmonic motion (wendy/wendy.c:39-52).
__device__ double solve_coll_harm(double c0, double c1, double c2, double omega) {
  const double A = c0 - c2, B = c1 / omega;
  double out = -asin(c2 / sqrt(B * B + A * A)) - atan2(A, B);
  if (out < 0) out = M_PI + asin(c2 / sqrt(B * B + A * A)) - atan2(A, B);
  return out / omega;
}

// Order key of a pair time: increasing in the time (integer compares, off
// the FP64 pipe), NaN after everything.
__device__ __forceinline__ uint64_t time_key(double t) {
  return isnan(t) ? ~0ull : key_of(t);
}

// The smallest (key, index) over the warp; ties to the lower index.
__device__ __forceinline__ void warp_min(uint64_t& k, int& i) {
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    const uint64_t ok = __shfl_xor_sync(0xffffffffu, k, d);
    const int oi = __shfl_xor_sync(0xffffffffu, i, d);
    if (ok < k || (ok == k && oi < i)) {
      k = ok;
      i = oi;
    }
  }
}

// Recomputes the tree path above pair time `leaf` (all lanes).
__device__ void tree_update(const ExactArgs& A, uint64_t* const* tkey, int32_t* const* tidx,
                            const double* tcoll, int leaf, int lane) {
  int g = leaf / kTreeFan;  // group at level 0
  for (int lv = 0; lv < A.levels; ++lv) {
    const int j = g * kTreeFan + lane;
    uint64_t k = ~0ull;
    int i = 0x7fffffff;
    if (j < A.level_n[lv]) {
      if (lv == 0) {
        k = time_key(tcoll[j]);
        i = j;
      } else {
        k = tkey[lv - 1][j];
        i = tidx[lv - 1][j];
      }
    }
    warp_min(k, i);
    if (lane == 0) {
      tkey[lv][g] = k;
      tidx[lv][g] = i;
    }
    __syncwarp();
    g /= kTreeFan;
  }
}

// Advance sheet s to time tn (reference operation order).
__device__ __forceinline__ void advance(const ExactState& S, int s, double tn, double omega) {
  const double tdt = tn - S.t[s];
  if (omega > 0) {
    const double sinot = sin(omega * tdt);
    const double cosot = sqrt(1. - sinot * sinot);
    const double tmpd = S.x[s] - S.a[s];
    S.x[s] = tmpd * cosot + S.v[s] / omega * sinot + S.a[s];
    S.v[s] = -tmpd * omega * sinot + S.v[s] * cosot;
  } else {
    const double dv = S.a[s] * tdt;
    S.x[s] += dv * tdt / 2. + S.v[s] * tdt;
    S.v[s] += dv;
  }
  S.t[s] = tn;
}

__global__ void __launch_bounds__(32, 1) k_exact_step(const ExactArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x;
  const int n = A.n;
  ExactState S = A.g;
  // the tree's internal levels: in shared memory always (n / 31 entries)
  uint64_t* tkey[kMaxLevels];
  int32_t* tidx[kMaxLevels];
  {
    unsigned char* p = smem;
    for (int lv = 0; lv < A.levels; ++lv) {
      tkey[lv] = reinterpret_cast<uint64_t*>(p);
      p += 8 * (size_t)A.level_n[lv + 1];
    }
    for (int lv = 0; lv < A.levels; ++lv) {
      tidx[lv] = reinterpret_cast<int32_t*>(p);
      p += 4 * (size_t)A.level_n[lv + 1];
    }
    for (int lv = 0; lv < A.levels; ++lv)
      for (int j = lane; j < A.level_n[lv + 1]; j += 32) {
        tkey[lv][j] = A.tree_key[lv][j];
        tidx[lv][j] = A.tree_idx[lv][j];
      }
    p = smem + A.tree_bytes;
    if (A.use_smem) {
      // stage the state in shared memory too: x v a m t tcoll, then sindx
      double* d = reinterpret_cast<double*>(p);
      S.x = d;
      S.v = d + n;
      S.a = d + 2 * n;
      S.m = d + 3 * n;
      S.t = d + 4 * n;
      S.tcoll = d + 5 * n;
      S.sindx = reinterpret_cast<int32_t*>(d + 6 * n);
      for (int i = lane; i < n; i += 32) {
        S.x[i] = A.g.x[i];
        S.v[i] = A.g.v[i];
        S.a[i] = A.g.a[i];
        S.m[i] = A.g.m[i];
        S.sindx[i] = A.g.sindx[i];
        if (i < n - 1) S.tcoll[i] = A.g.tcoll[i];
      }
    }
  }
  for (int i = lane; i < n; i += 32) S.t[i] = 0.;
  __syncwarp();
  const double omega = A.omega, dt = A.dt;
  int cindx = *A.cindx;
  double next = *A.next_tcoll;
  long long cnt = 0;
  while (next < dt && cnt < A.maxcoll) {
    ++cnt;
    if (lane == 0) {
      const int ci = cindx;
      int i1 = S.sindx[ci], i2 = S.sindx[ci + 1];
      advance(S, i1, next, omega);
      advance(S, i2, next, omega);
      S.sindx[ci] = i2;
      S.sindx[ci + 1] = i1;
      const double dm = S.m[i2] - S.m[i1];
      S.a[i1] -= dm;
      S.a[i2] -= dm;
      const double tmp = S.a[i1];
      S.a[i1] = S.a[i2];
      S.a[i2] = tmp;
      // the pair that just crossed (i1 still names the sheet now at ci + 1)
      double tn;
      if (omega > 0) {
        double q = (S.v[i1] - S.v[i2]) / (S.a[i2] - S.a[i1]) / omega;
        q *= q;
        q = (1. - q) / (1. + q);
        tn = acos(q) / omega;
      } else {
        tn = 2. * (S.v[i1] - S.v[i2]) / (S.a[i2] - S.a[i1]);
      }
      S.tcoll[ci] = next + tn;
      if (ci > 0) {
        const int j1 = S.sindx[ci - 1], j2 = S.sindx[ci];
        if (omega > 0) {
          advance(S, j1, next, omega);
          S.tcoll[ci - 1] = next + solve_coll_harm(S.x[j1] - S.x[j2], S.v[j1] - S.v[j2],
                                                   S.a[j1] - S.a[j2], omega);
        } else {
          const double tdt = S.t[j1] - next;
          S.tcoll[ci - 1] =
              next + solve_coll_quad(S.x[j1] + S.a[j1] * tdt * tdt / 2. - S.v[j1] * tdt - S.x[j2],
                                     S.v[j1] - S.a[j1] * tdt - S.v[j2],
                                     0.5 * (S.a[j1] - S.a[j2]));
        }
      }
      if (ci < n - 2) {
        const int j1 = S.sindx[ci + 2], j2 = S.sindx[ci + 1];
        if (omega > 0) {
          advance(S, j1, next, omega);
          S.tcoll[ci + 1] = next + solve_coll_harm(S.x[j1] - S.x[j2], S.v[j1] - S.v[j2],
                                                   S.a[j1] - S.a[j2], omega);
        } else {
          const double tdt = S.t[j1] - next;
          S.tcoll[ci + 1] =
              next + solve_coll_quad(S.x[j1] + S.a[j1] * tdt * tdt / 2. - S.v[j1] * tdt - S.x[j2],
                                     S.v[j1] - S.a[j1] * tdt - S.v[j2],
                                     0.5 * (S.a[j1] - S.a[j2]));
        }
      }
    }
    __syncwarp();
    // the three pair times that changed, and their paths up the tree
    const int ci = cindx;
    const int lo = ci > 0 ? ci - 1 : ci, hi = ci < n - 2 ? ci + 1 : ci;
    tree_update(A, tkey, tidx, S.tcoll, lo, lane);
    if (hi / kTreeFan != lo / kTreeFan) tree_update(A, tkey, tidx, S.tcoll, hi, lane);
    // the next crossing: the root
    const int i = tidx[A.levels - 1][0];
    const double v = S.tcoll[i];
    cindx = i;
    next = isnan(v) ? INFINITY : v;
  }
  // every sheet to the end of the interval, clocks and pending times shifted
  for (int s = lane; s < n; s += 32) advance(S, s, dt, omega);
  for (int i = lane; i < n - 1; i += 32) S.tcoll[i] -= dt;
  __syncwarp();
  if (A.use_smem) {
    for (int i = lane; i < n; i += 32) {
      A.g.x[i] = S.x[i];
      A.g.v[i] = S.v[i];
      A.g.a[i] = S.a[i];
      A.g.sindx[i] = S.sindx[i];
      if (i < n - 1) A.g.tcoll[i] = S.tcoll[i];
    }
  }
  // the tree holds absolute times of this interval: rebuilt by the host's
  // next call (k_exact_tree), like the reference rebuilds its BST per call
  if (lane == 0) {
    *A.cindx = cindx;
    *A.next_tcoll = next - dt;
    *A.ncoll = cnt;
    *A.err = cnt == A.maxcoll ? -2 : 0;
  }
}

// Builds the tree over the current pair times (one warp per level-0 group,
// then level by level).
__global__ void k_exact_tree_level(ExactArgs A, int lv) {
  const int lane = threadIdx.x & 31;
  const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int ng = (A.level_n[lv] + kTreeFan - 1) / kTreeFan;
  if (g >= ng) return;
  const int j = g * kTreeFan + lane;
  uint64_t k = ~0ull;
  int i = 0x7fffffff;
  if (j < A.level_n[lv]) {
    if (lv == 0) {
      k = time_key(A.g.tcoll[j]);
      i = j;
    } else {
      k = A.tree_key[lv - 1][j];
      i = A.tree_idx[lv - 1][j];
    }
  }
  warp_min(k, i);
  if (lane == 0) {
    A.tree_key[lv][g] = k;
    A.tree_idx[lv][g] = i;
  }
}

// Initial pair times from the sorted state (the reference computes them in
// Python with its C root finders, wendy/wendy.py:208-238).
__global__ void k_exact_pairs(ExactState S, int n, double omega) {
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += stride) {
    const int p = S.sindx[i], q = S.sindx[i + 1];
    S.tcoll[i] = omega > 0
                     ? solve_coll_harm(S.x[p] - S.x[q], S.v[p] - S.v[q], S.a[p] - S.a[q], omega)
                     : solve_coll_quad(S.x[p] - S.x[q], S.v[p] - S.v[q], (S.a[p] - S.a[q]) / 2.);
  }
}

thread_local char g_exact_error[256];

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_exact_error, sizeof(g_exact_error), fmt, ap);
  va_end(ap);
  record_last_error(g_exact_error);
  return code;
}

}  // namespace

struct wg_exact {
  int n = 0;
  double omega = 0;
  void* mem = nullptr;
  ExactArgs args{};
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  size_t smem = 0;
  int* h_ret = nullptr;  // page-locked: cindx, err, ncoll (as two ints), next (as two ints)
};

namespace {

void free_exact(wg_exact* e) {
  if (!e) return;
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->mem) cudaFree(e->mem);
  if (e->h_ret) cudaFreeHost(e->h_ret);
  if (e->ev0) cudaEventDestroy(e->ev0);
  if (e->ev1) cudaEventDestroy(e->ev1);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" {

int wg_exact_create(int64_t n, const double* x, const double* v, const double* a,
                    const double* m, const int32_t* sindx, double omega, wg_exact** out) {
  if (!out) return fail(WG_ERR_ARG, "null output handle");
  *out = nullptr;
  if (n < 2 || n > (1 << 24)) return fail(WG_ERR_ARG, "exact solver: n outside [2, 2^24]");
  if (!x || !v || !a || !m || !sindx) return fail(WG_ERR_ARG, "exact solver: null array");
  if (!std::isfinite(omega)) return fail(WG_ERR_ARG, "exact solver: omega not finite");
  for (int64_t i = 0; i < n; ++i) {
    if (!std::isfinite(x[i]) || !std::isfinite(v[i]) || !std::isfinite(a[i]) ||
        !std::isfinite(m[i]) || m[i] < 0)
      return fail(WG_ERR_ARG, "exact solver: sheet %lld has a non-finite value or a negative "
                              "mass", (long long)i);
    if (sindx[i] < 0 || sindx[i] >= n)
      return fail(WG_ERR_ARG, "exact solver: sindx[%lld] out of range", (long long)i);
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(WG_ERR_NODEV, "no CUDA device visible");
  }
  wg_exact* e = new wg_exact();
  e->n = (int)n;
  e->omega = omega > 0 ? omega : 0.0;
  ExactArgs& A = e->args;
  A.n = (int)n;
  A.omega = e->omega;
  // tree levels over the n - 1 pair times
  A.level_n[0] = (int)n - 1;
  A.levels = 0;
  while (true) {
    const int up = (A.level_n[A.levels] + kTreeFan - 1) / kTreeFan;
    A.level_n[A.levels + 1] = up;
    ++A.levels;
    if (up <= 1 || A.levels == kMaxLevels) break;
  }
  const size_t nd = al(8 * (size_t)n), ni = al(4 * (size_t)n);
  size_t tree_b = 0;
  for (int lv = 0; lv < A.levels; ++lv)
    tree_b += al(8 * (size_t)A.level_n[lv + 1]) + al(4 * (size_t)A.level_n[lv + 1]);
  const size_t total = 6 * nd + ni + tree_b + al(64);
  if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e->ev0) != cudaSuccess || cudaEventCreate(&e->ev1) != cudaSuccess ||
      cudaMallocHost(&e->h_ret, 64) != cudaSuccess) {
    cudaGetLastError();
    free_exact(e);
    return fail(WG_ERR_CUDA, "exact solver: stream set-up failed");
  }
  if (cudaMalloc(&e->mem, total) != cudaSuccess) {
    cudaGetLastError();
    free_exact(e);
    return fail(WG_ERR_NOMEM, "exact solver: cudaMalloc of %zu bytes failed", total);
  }
  char* p = static_cast<char*>(e->mem);
  A.g.x = reinterpret_cast<double*>(p); p += nd;
  A.g.v = reinterpret_cast<double*>(p); p += nd;
  A.g.a = reinterpret_cast<double*>(p); p += nd;
  A.g.m = reinterpret_cast<double*>(p); p += nd;
  A.g.t = reinterpret_cast<double*>(p); p += nd;
  A.g.tcoll = reinterpret_cast<double*>(p); p += nd;
  A.g.sindx = reinterpret_cast<int32_t*>(p); p += ni;
  A.tree_bytes = 0;
  for (int lv = 0; lv < A.levels; ++lv) {
    A.tree_key[lv] = reinterpret_cast<uint64_t*>(p); p += al(8 * (size_t)A.level_n[lv + 1]);
    A.tree_idx[lv] = reinterpret_cast<int32_t*>(p); p += al(4 * (size_t)A.level_n[lv + 1]);
    A.tree_bytes += 12 * (size_t)A.level_n[lv + 1];
  }
  A.tree_bytes = (A.tree_bytes + 15) & ~(size_t)15;
  A.cindx = reinterpret_cast<int*>(p);
  A.err = A.cindx + 1;
  A.ncoll = reinterpret_cast<long long*>(A.cindx + 2);
  A.next_tcoll = reinterpret_cast<double*>(A.cindx + 4);
  // the tree's internal levels always live in shared memory; the state too
  // when it fits (6 doubles and an index per sheet)
  const size_t smem = A.tree_bytes + 52 * (size_t)n + 64;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  A.use_smem = smem <= (size_t)optin;
  e->smem = A.use_smem ? smem : A.tree_bytes;
  if (e->smem > (size_t)optin ||
      cudaFuncSetAttribute(k_exact_step, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)e->smem) != cudaSuccess) {
    cudaGetLastError();
    free_exact(e);
    return fail(WG_ERR_ARG, "exact solver: %lld sheets need more shared memory for the pair-time "
                            "tree than a block has", (long long)n);
  }
  cudaStream_t s = e->stream;
  cudaError_t ce = cudaSuccess;
  auto up = [&](void* d, const void* h, size_t b) {
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d, h, b, cudaMemcpyHostToDevice, s);
  };
  up(A.g.x, x, 8 * n);
  up(A.g.v, v, 8 * n);
  up(A.g.a, a, 8 * n);
  up(A.g.m, m, 8 * n);
  up(A.g.sindx, sindx, 4 * n);
  if (ce == cudaSuccess) {
    k_exact_pairs<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(A.g, (int)n, A.omega);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) {
    free_exact(e);
    return fail(WG_ERR_CUDA, "exact solver: set-up failed: %s", cudaGetErrorString(ce));
  }
  // the first crossing, as the reference's argmin (lowest index on ties; a
  // NaN pair time never comes first)
  std::vector<double> tc((size_t)n - 1);
  cudaMemcpy(tc.data(), A.g.tcoll, 8 * (size_t)(n - 1), cudaMemcpyDeviceToHost);
  int ci = -1;
  for (int i = 0; i < (int)n - 1; ++i)
    if (!std::isnan(tc[(size_t)i]) && (ci < 0 || tc[(size_t)i] < tc[(size_t)ci])) ci = i;
  const double nxt = ci < 0 ? INFINITY : tc[(size_t)ci];
  if (ci < 0) ci = 0;
  int hret[2] = {ci, 0};
  cudaMemcpy(A.cindx, hret, 8, cudaMemcpyHostToDevice);
  cudaMemcpy(A.next_tcoll, &nxt, 8, cudaMemcpyHostToDevice);
  *out = e;
  return WG_OK;
}

int wg_exact_step(wg_exact* e, double dt, int64_t maxcoll, int64_t* ncoll,
                  double* time_elapsed) {
  if (!e || !(dt > 0) || !std::isfinite(dt) || maxcoll < 0)
    return fail(WG_ERR_ARG, "exact solver: needs a handle, dt > 0 and maxcoll >= 0");
  ExactArgs& A = e->args;
  A.dt = dt;
  A.maxcoll = (long long)maxcoll;
  cudaStream_t s = e->stream;
  // the tree over this interval's pair times
  for (int lv = 0; lv < A.levels; ++lv) {
    const int groups = (A.level_n[lv] + kTreeFan - 1) / kTreeFan;
    k_exact_tree_level<<<(unsigned)((groups + 7) / 8), 256, 0, s>>>(A, lv);
  }
  cudaEventRecord(e->ev0, s);
  k_exact_step<<<1, 32, e->smem, s>>>(A);
  cudaEventRecord(e->ev1, s);
  cudaMemcpyAsync(e->h_ret, A.cindx, 24, cudaMemcpyDeviceToHost, s);
  const cudaError_t ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return fail(WG_ERR_CUDA, "exact solver: %s", cudaGetErrorString(ce));
  long long nc = 0;
  std::memcpy(&nc, e->h_ret + 2, 8);
  if (ncoll) *ncoll = nc;
  float ms = 0;
  cudaEventElapsedTime(&ms, e->ev0, e->ev1);
  if (time_elapsed) *time_elapsed = ms * 1e-3;
  if (e->h_ret[1] == -2) return fail(WG_ERR_MAXCOLL, "Maximum number of collisions per time "
                                                     "step exceeded");
  return WG_OK;
}

int wg_exact_download(wg_exact* e, double* x, double* v, double* a, int32_t* sindx) {
  if (!e) return fail(WG_ERR_ARG, "null handle");
  const ExactArgs& A = e->args;
  cudaStream_t s = e->stream;
  cudaError_t ce = cudaSuccess;
  auto down = [&](void* h, const void* d, size_t b) {
    if (h && ce == cudaSuccess) ce = cudaMemcpyAsync(h, d, b, cudaMemcpyDeviceToHost, s);
  };
  down(x, A.g.x, 8 * (size_t)e->n);
  down(v, A.g.v, 8 * (size_t)e->n);
  down(a, A.g.a, 8 * (size_t)e->n);
  down(sindx, A.g.sindx, 4 * (size_t)e->n);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return fail(WG_ERR_CUDA, "exact solver: %s", cudaGetErrorString(ce));
  return WG_OK;
}

int wg_exact_destroy(wg_exact* e) {
  free_exact(e);
  return WG_OK;
}

}  // extern "C"
