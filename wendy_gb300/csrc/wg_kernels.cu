// wg_kernels.cu -- the fused force / kick / drift kernel and the small
// element-wise kernels around it.
//
// One sub-step of the reference (wendy/wendy.c:334-384 followed by
// leapfrog_leappq, wendy/wendy.c:324-333) on sheets that are already in
// sorted order is a single pass here:
//   exclusive prefix sum of the masses in sorted order (exact, 128-bit
//   fixed point, decoupled look-back across tiles)
//   a = [ext(x, t) +] (totmass - 2 C - m [- omega^2 x])
//   v += dt_kick a ;  x += dt_drift v
// with x, v updated in place.  The same pass records whether the new
// positions are still strictly increasing and the largest |v|, which is
// what decides how the next sub-step re-sorts.
#include <atomic>
#include <cstdint>
#include <mutex>

#include "wg_internal.cuh"

namespace wg {

namespace {

// Look-back over earlier tiles (called by all lanes of warp 0).  Returns the
// exclusive fixed-point prefix of `tile` and publishes the tile's inclusive
// prefix.  Every wait is bounded: on expiry DEV_ERR_LOOKBACK_TIMEOUT is
// raised and the missing predecessor counts as zero.
__device__ u128 force_lookback(const ForceArgs& a, int64_t tile, u128 total, int lane) {
  TileRec* recs = a.recs;
  const unsigned ep = a.epochs[a.sub];
  TileRec* me = recs + tile;
  // a withheld tile (test hook) publishes nothing: its successors' waits
  // on it run out after a.spin_limit iterations
  const bool publish = tile != a.withhold_tile;
  if (tile == 0) {
    if (lane == 0 && publish) {
      me->inc_lo = (uint64_t)total;
      me->inc_hi = (uint64_t)(total >> 64);
      st_release_u32(&me->flag, (ep << 2) | 2u);
    }
    return 0;
  }
  if (lane == 0 && publish) {
    me->agg_lo = (uint64_t)total;
    me->agg_hi = (uint64_t)(total >> 64);
    st_release_u32(&me->flag, (ep << 2) | 1u);
  }
  u128 prefix = 0;
  int64_t j = tile - 1;
  for (;;) {
    const int64_t jj = j - lane;
    unsigned status = 0;
    u128 val = 0;
    if (jj >= 0) {
      const TileRec* r = recs + jj;
      unsigned f = 0;
      unsigned spins = 0;
      for (;;) {
        f = ld_acquire_u32(&r->flag);
        if ((f >> 2) == ep && (f & 3u)) break;
        if (++spins > a.spin_limit) {
          atomicOr(a.err, DEV_ERR_LOOKBACK_TIMEOUT);
          f = 0;
          break;
        }
        __nanosleep(32);
      }
      status = ((f >> 2) == ep) ? (f & 3u) : 0u;
      if (status == 2u)
        val = (((u128)ld_cg_u64(&r->inc_hi)) << 64) | ld_cg_u64(&r->inc_lo);
      else if (status == 1u)
        val = (((u128)ld_cg_u64(&r->agg_hi)) << 64) | ld_cg_u64(&r->agg_lo);
    }
    const unsigned pmask = __ballot_sync(0xffffffffu, status == 2u);
    const int stop = pmask ? (__ffs(pmask) - 1) : 31;
    prefix += warp_sum_u128(lane <= stop ? val : (u128)0);
    if (pmask || j - 32 < 0) break;
    j -= 32;
  }
  if (lane == 0 && publish) {
    const u128 inc = prefix + total;
    me->inc_lo = (uint64_t)inc;
    me->inc_hi = (uint64_t)(inc >> 64);
    st_release_u32(&me->flag, (ep << 2) | 2u);
  }
  return prefix;
}

template <int THREADS, int ITEMS, bool EXPR>
__global__ void __launch_bounds__(THREADS, 2) k_force_kick_drift(const ForceArgs a) {
  constexpr int TILE = THREADS * ITEMS;
  constexpr int WARPS = THREADS / 32;
  static_assert(ITEMS % 2 == 0, "vector loads need an even item count");
  __shared__ unsigned s_tile;
  __shared__ u128 s_warp[WARPS];
  __shared__ u128 s_prefix;
  __shared__ double s_amp, s_inv_h;
  __shared__ uint64_t s_first[WARPS + 1];
  __shared__ unsigned s_unsorted;
  __shared__ unsigned long long s_maxv;
  __shared__ unsigned s_epoch;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    s_tile = atomicAdd(a.ticket, 1u);
    s_unsorted = 0;
    s_maxv = 0;
    s_epoch = a.epochs[a.sub];
    s_amp = (a.ext.kind == EXT_PULSE_TANH) ? pulse_amplitude(a.ext, a.t_seq[a.sub]) : 0.0;
    s_inv_h = (a.ext.kind == EXT_PULSE_TANH) ? 1.0 / a.ext.p[3] : 0.0;
  }
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t base = tile * TILE;
  const int64_t n = a.n;
  if (base >= n) {  // only with a ticket counter that was not reset: do nothing
    if (tid == 0) atomicOr(a.err, DEV_ERR_BAD_STATE);
    return;
  }
  const StateRef st = a.table->cur;
  const int64_t i0 = base + (int64_t)tid * ITEMS;
  const bool full = base + TILE <= n;

  double x[ITEMS], v[ITEMS], m[ITEMS];
  if (full) {
    const double2* px = reinterpret_cast<const double2*>(st.x + i0);
    const double2* pv = reinterpret_cast<const double2*>(st.v + i0);
    const double2* pm = reinterpret_cast<const double2*>(st.m + i0);
#pragma unroll
    for (int j = 0; j < ITEMS / 2; ++j) {
      const double2 tx = px[j], tv = pv[j], tm = __ldg(pm + j);
      x[2 * j] = tx.x; x[2 * j + 1] = tx.y;
      v[2 * j] = tv.x; v[2 * j + 1] = tv.y;
      m[2 * j] = tm.x; m[2 * j + 1] = tm.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      const int64_t e = i0 + i;
      const bool ok = e < n;
      x[i] = ok ? st.x[e] : 0.0;
      v[i] = ok ? st.v[e] : 0.0;
      m[i] = ok ? st.m[e] : 0.0;
    }
  }

  // Thread-local exclusive scan of the fixed-point masses.
  u128 cex[ITEMS];
  u128 run = 0;
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    cex[i] = run;
    run += mass_to_fixed(m[i], a.E);
  }
  const u128 tot = run;
  const u128 incl = warp_inclusive_scan_u128(tot, lane);
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const u128 wv = lane < WARPS ? s_warp[lane] : (u128)0;
    const u128 wincl = warp_inclusive_scan_u128(wv, lane);
    const u128 tile_total = shfl_u128(wincl, WARPS - 1);
    if (lane < WARPS) s_warp[lane] = wincl - wv;
    const u128 prefix = force_lookback(a, tile, tile_total, lane);
    if (lane == 0) s_prefix = prefix;
  }
  __syncthreads();
  const u128 tprefix = s_prefix + s_warp[warp] + (incl - tot);

  const i128 T = (i128)((((u128)a.T_hi) << 64) | a.T_lo);
  const double amp = s_amp, inv_h = s_inv_h;
  double xr[EXPR ? kExprRegs : 1];  // an expression force's registers
  double t_ev = 0.0;
  if constexpr (EXPR) {
    t_ev = a.t_seq[a.sub];
    expr_time(a.ext, t_ev, xr);
  }
  unsigned long long maxv = 0;
  bool unsorted = false;
  uint64_t first_key = ~0ull, last_key = 0, prev_key = 0;
  int nvalid = 0;
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    const bool ok = full || (i0 + i < n);
    const u128 M = (i + 1 < ITEMS ? cex[i + 1] : tot) - cex[i];
    const i128 C = (i128)(tprefix + cex[i]);
    const i128 A = T - 2 * C - (i128)M;
    double acc = fixed_to_double(A, a.E);
    if (a.has_omega) acc = fma(-a.omega2, x[i], acc);
    if constexpr (EXPR)
      acc = expr_space(a.ext, xr, x[i], t_ev) + acc;
    else if (a.ext.kind != EXT_NONE)
      acc = ext_force_at(a.ext, amp, inv_h, x[i]) + acc;
    const double vn = fma(a.dt_kick, acc, v[i]);
    const double xn = fma(a.dt_drift, vn, x[i]);
    v[i] = vn;
    x[i] = xn;
    if (a.a_out && ok) a.a_out[i0 + i] = acc;
    if (ok) {
      const unsigned long long av = (unsigned long long)__double_as_longlong(vn) & 0x7FFFFFFFFFFFFFFFull;
      maxv = av > maxv ? av : maxv;
      const uint64_t k = key_of(xn);
      if (nvalid == 0) first_key = k;
      else if (k <= prev_key) unsorted = true;
      prev_key = k;
      last_key = k;
      ++nvalid;
    }
  }

  if (full) {
    double2* px = reinterpret_cast<double2*>(st.x + i0);
    double2* pv = reinterpret_cast<double2*>(st.v + i0);
#pragma unroll
    for (int j = 0; j < ITEMS / 2; ++j) {
      px[j] = make_double2(x[2 * j], x[2 * j + 1]);
      pv[j] = make_double2(v[2 * j], v[2 * j + 1]);
    }
  } else {
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      const int64_t e = i0 + i;
      if (e < n) {
        st.x[e] = x[i];
        st.v[e] = v[i];
      }
    }
  }

  // Order checks across threads: thread t's last key against thread t+1's
  // first key (threads without sheets carry first_key = ~0).
  const uint64_t next_first = __shfl_down_sync(0xffffffffu, first_key, 1);
  if (lane == 0) s_first[warp] = first_key;
  if (tid == 0) s_first[WARPS] = ~0ull;
  __syncthreads();
  if (nvalid > 0) {
    const uint64_t nf = lane < 31 ? next_first : s_first[warp + 1];
    if (nf != ~0ull && last_key >= nf) unsorted = true;
  }
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, maxv, d);
    maxv = o > maxv ? o : maxv;
  }
  if (lane == 0 && maxv) atomicMax(&s_maxv, maxv);
  if (unsorted) s_unsorted = 1u;

  // Tile boundary: publish this tile's last key, then compare the first key
  // with the predecessor's last key (the predecessor never waits on us).
  const int last_tid = full ? THREADS - 1 : (int)((n - 1 - base) / ITEMS);
  if (tid == last_tid) {
    TileRec* me = a.recs + tile;
    me->last_key = last_key;
    st_release_u32(&me->last_flag, s_epoch);
  }
  if (tid == 0 && tile > 0) {
    const TileRec* prev = a.recs + tile - 1;
    unsigned spins = 0;
    bool ok = true;
    while (ld_acquire_u32(&prev->last_flag) != s_epoch) {
      if (++spins > a.spin_limit) {
        atomicOr(a.err, DEV_ERR_LOOKBACK_TIMEOUT);
        ok = false;
        break;
      }
      __nanosleep(32);
    }
    if (!ok || ld_cg_u64(&prev->last_key) >= first_key) s_unsorted = 1u;
  }
  __syncthreads();
  if (tid == 0) {
    StepFlags* f = a.flag_out;
    if (s_unsorted) atomicOr(&f->unsorted, 1u);
    if (s_maxv) atomicMax(&f->max_v, s_maxv);
  }
}

__global__ void k_drift(const StateTable* table, int64_t n, double dt, StepFlags* flag) {
  const StateRef st = table->cur;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    st.x[i] = fma(dt, st.v[i], st.x[i]);
  if (blockIdx.x == 0 && threadIdx.x == 0 && flag) atomicOr(&flag->unsorted, 1u);
}

__global__ void k_desort(const StateTable* table, int64_t n, double* x_out, double* v_out) {
  const StateRef st = table->cur;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int32_t j = st.idx[i];
    if (x_out) x_out[j] = st.x[i];
    if (v_out) v_out[j] = st.v[i];
  }
}

__global__ void k_scatter_accel(const StateTable* table, int64_t n, const double* a_sorted,
                                double* a_orig) {
  const StateRef st = table->cur;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    a_orig[st.idx[i]] = a_sorted[i];
}

__global__ void k_iota(const StateTable* table, int64_t n) {
  const StateRef st = table->cur;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    st.idx[i] = (int32_t)i;
}

int grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g > 152 * 16) g = 152 * 16;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

namespace {
std::atomic<unsigned> g_spin_limit{kSpinLimit};
std::atomic<int64_t> g_withhold_tile{-1};
}  // namespace

void set_wait_debug(unsigned spin_limit, int64_t withhold_tile) {
  g_spin_limit = spin_limit ? spin_limit : kSpinLimit;
  g_withhold_tile = withhold_tile;
}

void launch_force(const ForceArgs& a, int64_t n_tiles, cudaStream_t s) {
  ForceArgs b = a;
  b.spin_limit = g_spin_limit;
  b.withhold_tile = g_withhold_tile;
  if (b.ext.kind == EXT_EXPR)
    k_force_kick_drift<kForceThreads, kForceItems, true>
        <<<(unsigned)n_tiles, kForceThreads, 0, s>>>(b);
  else
    k_force_kick_drift<kForceThreads, kForceItems, false>
        <<<(unsigned)n_tiles, kForceThreads, 0, s>>>(b);
}

void launch_drift(const StateTable* table, int64_t n, double dt, StepFlags* flag,
                  cudaStream_t s) {
  k_drift<<<grid_for(n, 256), 256, 0, s>>>(table, n, dt, flag);
}

void launch_desort(const StateTable* table, int64_t n, double* x_out, double* v_out,
                   cudaStream_t s) {
  k_desort<<<grid_for(n, 256), 256, 0, s>>>(table, n, x_out, v_out);
}

void launch_scatter_accel(const StateTable* table, int64_t n, const double* a_sorted,
                          double* a_orig, cudaStream_t s) {
  k_scatter_accel<<<grid_for(n, 256), 256, 0, s>>>(table, n, a_sorted, a_orig);
}

// F(x_i, t) of a registered external force, with the force kernels' code:
// amplitude and 1 / h once per block, then ext_force_at per position.
__global__ void k_ext_eval(const ExtForce f, double t, const double* x, double* out, int64_t n) {
  __shared__ double s_amp, s_inv_h;
  if (threadIdx.x == 0) {
    s_amp = f.kind == EXT_PULSE_TANH ? pulse_amplitude(f, t) : 0.0;
    s_inv_h = f.kind == EXT_PULSE_TANH ? 1.0 / f.p[3] : 0.0;
  }
  __syncthreads();
  double xr[kExprRegs];
  if (f.kind == EXT_EXPR) expr_time(f, t, xr);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = f.kind == EXT_EXPR ? expr_space(f, xr, x[i], t)
                                : ext_force_at(f, s_amp, s_inv_h, x[i]);
}

void launch_ext_eval(const ExtForce& f, double t, const double* x, double* out, int64_t n,
                     cudaStream_t s) {
  k_ext_eval<<<grid_for(n, 256), 256, 0, s>>>(f, t, x, out, n);
}

// ---- the pulsed force's tanh table (wg_tanh.cuh): one per device, in a
// __device__ array of the library, computed by its first use on the device
namespace {
__device__ __align__(256) long long g_tanh_tab[kTanhCells * kTanhRow];

__global__ void k_tanh_table(long long* tab) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kTanhCells) tanh_table_row(i, tab + (size_t)kTanhRow * i);
}

std::once_flag g_tanh_once[kMaxDevices];
const long long* g_tanh_ptr[kMaxDevices];

const long long* tanh_table_setup() {
  long long* p = nullptr;
  if (cudaGetSymbolAddress((void**)&p, g_tanh_tab) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  k_tanh_table<<<(kTanhCells + 255) / 256, 256, 0, 0>>>(p);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(0) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}
}  // namespace

const long long* tanh_table() {
  const int dev = current_device();
  if (dev < 0) return nullptr;
  if (dev >= kMaxDevices) return tanh_table_setup();
  std::call_once(g_tanh_once[dev], [dev] { g_tanh_ptr[dev] = tanh_table_setup(); });
  return g_tanh_ptr[dev];
}

// Sums of the energy and momentum diagnostics over the sorted state, with
// the self-gravity accelerations a_sorted of that state:
//   part[0] = sum m v^2 / 2, part[1] = sum m x^2 / 2, part[2] = -sum m x a,
//   part[3] = sum m v.
// The pair sum of the reference's potential energy (wendy/wendy.py:467-475),
// sum_{x_j < x_i} m_i m_j (x_i - x_j), equals -sum_i m_i x_i a_i / 2piG for
// a_i = M - 2 C_i - m_i.  Each block writes its partial sums; the final
// kernel adds the partials in block order, so the result is deterministic.
constexpr int kEnergyThreads = 256;
__global__ void k_energy_partial(const StateTable* table, int64_t n, const double* a_sorted,
                                 double* part) {
  __shared__ double red[4][kEnergyThreads / 32];
  const StateRef st = table->cur;
  double k = 0.0, h = 0.0, w = 0.0, p = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const double m = st.m[i], x = st.x[i], v = st.v[i];
    k += m * v * v / 2.0;
    h += m * x * x / 2.0;
    w -= m * x * a_sorted[i];
    p += m * v;
  }
  double val[4] = {k, h, w, p};
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) val[q] += __shfl_down_sync(0xffffffffu, val[q], d);
    if (lane == 0) red[q][warp] = val[q];
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double t = 0.0;
    for (int j = 0; j < kEnergyThreads / 32; ++j) t += red[threadIdx.x][j];
    part[4 * blockIdx.x + threadIdx.x] = t;
  }
}

__global__ void k_energy_final(const double* part, int nblocks, double* out) {
  if (threadIdx.x < 4) {
    double t = 0.0;
    for (int j = 0; j < nblocks; ++j) t += part[4 * j + threadIdx.x];
    out[threadIdx.x] = t;
  }
}

void launch_energy(const StateTable* table, int64_t n, const double* a_sorted, double* scratch,
                   cudaStream_t s) {
  k_energy_partial<<<kEnergyBlocks, kEnergyThreads, 0, s>>>(table, n, a_sorted, scratch + 4);
  k_energy_final<<<1, 32, 0, s>>>(scratch + 4, kEnergyBlocks, scratch);
}

void launch_init_state(StateTable* table, int64_t n, cudaStream_t s) {
  k_iota<<<grid_for(n, 256), 256, 0, s>>>(table, n);
}

}  // namespace wg
