// wg_radix.cu -- full on-device re-sort of the sheets: a least-significant-
// digit radix sort of the 64-bit position keys with 8-bit digits, one pass
// per digit, each pass a single read and write of (key, slot) pairs whose
// tile offsets come from a decoupled look-back over per-tile digit counts
// ("onesweep").  It replaces the serial argsort of the reference
// (wendy/wendy.c:341-357) when the order cannot be repaired locally.
//
//   hist   one read of the positions: all eight digit histograms
//   plan   exclusive digit offsets; passes whose digit is the same for every
//          key are skipped (decided on the device)
//   pass   8x, persistent: bulk-copy the tile into shared memory (the next
//          tile's copy overlaps this one's write-out), rank within the tile
//          (bit-plane ballots + per-warp shared-memory counters, stable),
//          publish the tile's digit counts, stage in digit order, look back
//          for the tile's global digit offsets, write out
//   gather permute x, v, m, idx into the other state set
//   ties   equal keys are ordered by original index (rare; usually no-op):
//          short runs in place, long runs by one CTA each
//   flip   the other set becomes the current one
//
// Every kernel first reads the sub-step's `unsorted` flag and returns at once
// when the sheets are already in order, so the sequence can be captured in a
// CUDA graph and still cost nothing when no sort is needed.
#include <cstdint>
#include <functional>
#include <mutex>

#include "wg_internal.cuh"

namespace wg {

namespace {

constexpr int R = 256;
// Look-back status words: top two bits 0 = not yet published, kStatA = the
// tile's own count, kStatP = inclusive count, kStatX = poisoned (a wait of
// this tile or of one it depends on expired: its offsets are unknown).
constexpr unsigned kStatA = 1u << 30, kStatP = 2u << 30, kStatX = 3u << 30,
                   kCountMask = (1u << 30) - 1;

// plan layout (uint32 words)
constexpr int kPlanActive = 0;   // [8]
constexpr int kPlanSrc = 8;      // [8]
constexpr int kPlanDst = 16;     // [8]
constexpr int kPlanFinal = 24;   // [1]
constexpr int kPlanStarts = 32;  // [8 * 256]
constexpr int kPlanWords = kPlanStarts + 8 * R;

struct PassArgs {
  const StateTable* table;
  int64_t n;
  int pass;
  int64_t n_tiles;
  uint64_t* keys0;
  uint64_t* keys1;
  uint32_t* pos0;
  uint32_t* pos1;
  const uint32_t* plan;
  uint32_t* status;
  uint32_t* counters;
  const StepFlags* flag;
  unsigned* err;
};

__global__ void k_radix_hist(const StateTable* table, int64_t n, uint32_t* hist,
                             const StepFlags* flag) {
  if (!flag->unsorted) return;
  __shared__ uint32_t sh[8 * R];
  for (int i = threadIdx.x; i < 8 * R; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const double* x = table->cur.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t k = key_of(x[i]);
#pragma unroll
    for (int p = 0; p < 8; ++p) atomicAdd(&sh[p * R + ((k >> (8 * p)) & 255u)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 8 * R; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// One block of 256 threads.
__global__ void k_radix_plan(int64_t n, const uint32_t* hist, uint32_t* plan,
                             const StepFlags* flag) {
  if (!flag->unsorted) return;
  __shared__ uint32_t s_tmp[R / 32];
  __shared__ int s_trivial[8];
  const int d = threadIdx.x, lane = d & 31, warp = d >> 5;
  for (int p = 0; p < 8; ++p) {
    const uint32_t c = hist[p * R + d];
    const int triv = __syncthreads_or(c == (uint32_t)n);
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) s_tmp[warp] = incl;
    __syncthreads();
    uint32_t wpre = 0;
    for (int w = 0; w < warp; ++w) wpre += s_tmp[w];
    plan[kPlanStarts + p * R + d] = wpre + incl - c;
    if (d == 0) s_trivial[p] = triv;
    __syncthreads();
  }
  if (d == 0) {
    int cur = 0;
    plan[kPlanActive + 0] = 1;
    plan[kPlanSrc + 0] = 0;
    plan[kPlanDst + 0] = 0;
    for (int p = 1; p < 8; ++p) {
      const int act = !s_trivial[p];
      plan[kPlanActive + p] = act;
      plan[kPlanSrc + p] = cur;
      plan[kPlanDst + p] = act ? 1 - cur : cur;
      if (act) cur = 1 - cur;
    }
    plan[kPlanFinal] = cur;
  }
}

template <int THREADS, int ITEMS>
struct PassSmem {
  static constexpr int TILE = THREADS * ITEMS;
  static constexpr int WARPS = THREADS / 32;
  uint64_t keys[2][TILE];  // tile k lands in keys[k & 1] (positions on pass 0) ...
  uint32_t vals[2][TILE];  // ... and is staged in digit order in the same buffer
  uint32_t whist[WARPS][R];
  uint32_t tile_excl[R];
  uint32_t gbase[R];
  uint32_t tmp[WARPS];
  uint64_t mbar[2];
  int64_t tile[2];
  int64_t bad;  // 1 + the tile whose offsets are unknown (a bounded wait expired)
  int stop;     // a copy of this CTA never completed: claim no further tile
};

// Persistent: each CTA claims its next tile once the current one's global
// offsets are known and bulk-copies it into its other shared-memory buffer
// during the current write-out.  Claiming that late keeps claim order close
// to processing order, which keeps look-backs short; publishing the counts
// before staging, and looking back only after it, gives the tiles ahead the
// staging time to finish.  Claims are dynamic, so only running CTAs ever
// hold a tile and the look-back always progresses: the smallest tile in work
// has every predecessor finished.
template <int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS, 2) k_radix_pass(const PassArgs a) {
  using Smem = PassSmem<THREADS, ITEMS>;
  constexpr int TILE = Smem::TILE;
  constexpr int WARPS = Smem::WARPS;
  static_assert(THREADS == R, "one thread per digit");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>(smem_raw);

  if (!a.flag->unsorted) return;
  // an earlier pass gave up on a wait: its output is incomplete
  if (*a.err & DEV_ERR_RADIX_TIMEOUT) return;
  const int pass = a.pass;
  if (!a.plan[kPlanActive + pass]) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int shift = 8 * pass;
  const int srcb = (int)a.plan[kPlanSrc + pass], dstb = (int)a.plan[kPlanDst + pass];
  const uint64_t* ksrc = srcb ? a.keys1 : a.keys0;
  const uint32_t* psrc = srcb ? a.pos1 : a.pos0;
  uint64_t* kdst = dstb ? a.keys1 : a.keys0;
  uint32_t* pdst = dstb ? a.pos1 : a.pos0;
  const double* x = a.table->cur.x;
  const void* kfrom = pass == 0 ? (const void*)x : (const void*)ksrc;
  const bool bulk_ok = ((uintptr_t)kfrom & 15u) == 0 && (pass == 0 || ((uintptr_t)psrc & 15u) == 0);
  uint32_t* stat = a.status + ((int64_t)pass * a.n_tiles) * R;
  unsigned* claim = a.counters + pass;

  // thread 0: start the copy of tile t into buffer b; partial tiles (and
  // unaligned sources) are read with plain loads, their phase completes at once
  auto issue = [&](int64_t t, int b) {
    if (t >= a.n_tiles) return;
    const int64_t base = t * TILE;
    if (bulk_ok && a.n - base >= TILE) {
      const uint32_t kb = TILE * 8u, vb = pass ? TILE * 4u : 0u;
      mbar_expect_tx(&S.mbar[b], kb + vb);
      bulk_g2s(S.keys[b], static_cast<const char*>(kfrom) + base * 8, kb, &S.mbar[b]);
      if (pass) bulk_g2s(S.vals[b], psrc + base, vb, &S.mbar[b]);
    } else {
      mbar_expect_tx(&S.mbar[b], 0u);
    }
  };

  if (tid == 0) {
    S.bad = 0;
    S.stop = 0;
    mbar_init(&S.mbar[0], 1);
    mbar_init(&S.mbar[1], 1);
    fence_proxy_async_smem();
    const int64_t t0 = atomicAdd(claim, 1u);
    S.tile[0] = t0;
    issue(t0, 0);
  }
  for (int i = tid; i < WARPS * R; i += THREADS) (&S.whist[0][0])[i] = 0;
  __syncthreads();

  for (int k = 0;; ++k) {
    const int b = k & 1;
    const int64_t tile = S.tile[b];
    if (tile >= a.n_tiles) break;
    const int64_t base = tile * TILE;
    const int tile_n = (int)((a.n - base) < TILE ? (a.n - base) : TILE);
    const bool via_bulk = bulk_ok && tile_n == TILE;
    if (via_bulk && !mbar_wait(&S.mbar[b], (unsigned)(k >> 1) & 1u)) {
      // the tile never arrived: its keys, counts and offsets are unknown.  The
      // copy gets a second bounded wait; the tile is published as poisoned
      // and this CTA claims no further tile.
      if (lane == 0) atomicOr(a.err, DEV_ERR_RADIX_TIMEOUT);
      mbar_wait(&S.mbar[b], (unsigned)(k >> 1) & 1u);
      S.bad = tile + 1;
      S.stop = 1;
    }
    uint64_t key[ITEMS];
    uint32_t val[ITEMS];
    uint32_t rank[ITEMS];
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      const int local = warp * (32 * ITEMS) + i * 32 + lane;
      const int64_t e = base + local;
      if (local < tile_n) {
        if (via_bulk) {
          const uint64_t raw = S.keys[b][local];
          key[i] = pass == 0 ? key_of(__longlong_as_double((long long)raw)) : raw;
          val[i] = pass == 0 ? (uint32_t)e : S.vals[b][local];
        } else if (pass == 0) {
          key[i] = key_of(x[e]);
          val[i] = (uint32_t)e;
        } else {
          key[i] = ksrc[e];
          val[i] = psrc[e];
        }
      } else {
        key[i] = 0;
        val[i] = 0;
      }
    }
    // Stable ranking inside the warp: items in order, lanes in order.
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      const int local = warp * (32 * ITEMS) + i * 32 + lane;
      const bool ok = local < tile_n;
      const unsigned d = ok ? (unsigned)((key[i] >> shift) & 255u) : (0x100u + lane);
      // lanes holding the same digit, from its eight bit planes (one ballot
      // per bit: cheaper than a match instruction over 32 mostly distinct
      // digits)
      unsigned peers = __ballot_sync(0xffffffffu, ok);
      if (!ok) peers = ~peers;
#pragma unroll
      for (int bit = 0; bit < 8; ++bit) {
        const unsigned bal = __ballot_sync(0xffffffffu, (d >> bit) & 1u);
        peers &= ((d >> bit) & 1u) ? bal : ~bal;
      }
      uint32_t old = 0;
      if (ok) {
        old = S.whist[warp][d];
        rank[i] = old + __popc(peers & lanemask_lt());
      }
      __syncwarp();
      if (ok && lane == __ffs(peers) - 1) S.whist[warp][d] = old + __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    // Column of digit `tid`: exclusive offsets of the warps, tile count;
    // the count is published at once for the tiles behind this one.
    const int d = tid;
    uint32_t count = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      const uint32_t c = S.whist[w][d];
      S.whist[w][d] = count;
      count += c;
    }
    if (S.bad == tile + 1)
      st_relaxed_u32(&stat[tile * R + d], kStatX);
    else if (tile == 0)
      st_relaxed_u32(&stat[d], kStatP | count);
    else
      st_relaxed_u32(&stat[tile * R + d], kStatA | count);
    // Exclusive scan of the tile's counts over digits.
    uint32_t incl = count;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) S.tmp[warp] = incl;
    __syncthreads();
    uint32_t wpre = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) wpre += (w < warp) ? S.tmp[w] : 0u;
    const uint32_t tex = wpre + incl - count;
    S.tile_excl[d] = tex;
    __syncthreads();
    // Stage the tile in digit order (over the buffer it arrived in); this
    // needs only the tile's own offsets, and gives the tiles ahead time to
    // finish their look-back before this one starts its own.
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      const int local = warp * (32 * ITEMS) + i * 32 + lane;
      if (local < tile_n) {
        const unsigned dd = (unsigned)((key[i] >> shift) & 255u);
        const uint32_t p = S.tile_excl[dd] + S.whist[warp][dd] + rank[i];
        S.keys[b][p] = key[i];
        S.vals[b][p] = val[i];
      }
    }
    // Decoupled look-back over the same digit of earlier tiles.  Each status
    // word carries its count, so relaxed loads and stores suffice; LB
    // predecessors are read per round, their loads in flight together, and
    // summed in order up to the nearest inclusive one.
    uint32_t excl = 0;
    if (tile != 0 && S.bad != tile + 1) {
      constexpr int LB = 8;
      int64_t j = tile - 1;
      unsigned spins = 0;
      bool poisoned = false;
      for (;;) {
        uint32_t sv[LB];
#pragma unroll
        for (int w = 0; w < LB; ++w) sv[w] = (j - w >= 0) ? ld_relaxed_u32(&stat[(j - w) * R + d]) : 0u;
        bool done = false, blocked = false;
        int w = 0;
        for (; w < LB; ++w) {
          const uint32_t sw = sv[w];
          if ((sw >> 30) == 0u) {
            blocked = true;
            break;
          }
          if ((sw >> 30) == 3u) {  // a predecessor's offsets are unknown
            poisoned = done = true;
            break;
          }
          excl += sw & kCountMask;
          if ((sw >> 30) == 2u || j - w == 0) {
            done = true;
            break;
          }
        }
        if (done) break;
        if (blocked) {
          j -= w;  // resume at the tile that has not published yet
          if (++spins > kSpinLimit) {
            atomicOr(a.err, DEV_ERR_RADIX_TIMEOUT);
            poisoned = true;
            break;
          }
          __nanosleep(16);
          continue;
        }
        j -= LB;
      }
      if (poisoned) {
        // unknown offsets: publish the poison onward and write nothing
        atomicOr(a.err, DEV_ERR_RADIX_TIMEOUT);
        S.bad = tile + 1;
        st_relaxed_u32(&stat[tile * R + d], kStatX);
      } else {
        st_relaxed_u32(&stat[tile * R + d], kStatP | (excl + count));
      }
    }
    S.gbase[d] = a.plan[kPlanStarts + pass * R + d] + excl - tex;
    // claim the next tile once this one's offsets are known (claim order
    // then follows processing order) and start its copy into the other buffer
    if (tid == 0) {
      if (S.stop) {
        S.tile[b ^ 1] = a.n_tiles;  // ends the loop after this tile
      } else {
        const int64_t tn = atomicAdd(claim, 1u);
        S.tile[b ^ 1] = tn;
        fence_proxy_async_smem();
        issue(tn, b ^ 1);
      }
    }
    __syncthreads();
    for (int i = tid; i < WARPS * R; i += THREADS) (&S.whist[0][0])[i] = 0;
    const bool skip = S.bad == tile + 1;  // offsets unknown: no write may leave the tile
#pragma unroll
    for (int jj = 0; jj < ITEMS; ++jj) {
      const int p = jj * THREADS + tid;
      if (p < tile_n && !skip) {
        const uint64_t kk = S.keys[b][p];
        const unsigned dd = (unsigned)((kk >> shift) & 255u);
        const int64_t o = (int64_t)S.gbase[dd] + p;
        kdst[o] = kk;
        pdst[o] = S.vals[b][p];
      }
    }
    __syncthreads();
  }
}

// Permute x, v, m, idx into the other set; GU sheets per thread with their
// loads in flight together (the reads are random when the input was).
constexpr int kGatherThreads = 256, kGatherUnroll = 4;
__global__ void __launch_bounds__(kGatherThreads) k_radix_gather(
    StateTable* table, int64_t n, const uint64_t* keys0, const uint64_t* keys1,
    const uint32_t* pos0, const uint32_t* pos1, const uint32_t* plan, uint32_t* counters,
    const StepFlags* flag, const unsigned* err) {
  constexpr int GU = kGatherUnroll;
  // nothing after a pass that gave up on a wait: its slots are incomplete
  if (!flag->unsorted || (*err & DEV_ERR_RADIX_TIMEOUT)) return;
  const int fb = (int)plan[kPlanFinal];
  const uint64_t* __restrict__ keys = fb ? keys1 : keys0;
  const uint32_t* __restrict__ pos = fb ? pos1 : pos0;
  const StateRef cur = table->cur, oth = table->other;
  const int64_t chunk = (int64_t)gridDim.x * kGatherThreads * GU;
  bool tie = false;
  for (int64_t p0 = (int64_t)blockIdx.x * kGatherThreads * GU + threadIdx.x; p0 < n;
       p0 += chunk) {
    uint32_t q[GU];
#pragma unroll
    for (int u = 0; u < GU; ++u) {
      const int64_t p = p0 + (int64_t)u * kGatherThreads;
      q[u] = p < n ? __ldcs(pos + p) : 0u;
    }
    double xs[GU], vs[GU], ms[GU];
    int32_t is[GU];
#pragma unroll
    for (int u = 0; u < GU; ++u) {
      const int64_t p = p0 + (int64_t)u * kGatherThreads;
      if (p < n) {
        xs[u] = __ldg(cur.x + q[u]);
        vs[u] = __ldg(cur.v + q[u]);
        ms[u] = __ldg(cur.m + q[u]);
        is[u] = __ldg(cur.idx + q[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < GU; ++u) {
      const int64_t p = p0 + (int64_t)u * kGatherThreads;
      if (p < n) {
        oth.x[p] = xs[u];
        oth.v[p] = vs[u];
        oth.m[p] = ms[u];
        oth.idx[p] = is[u];
        if (p + 1 < n && keys[p] == keys[p + 1]) tie = true;
      }
    }
  }
  if (__syncthreads_or(tie) && threadIdx.x == 0) atomicOr(&counters[8], 1u);
}

// Equal keys: order each run by original index.  The thread at a run's
// first sheet finds its end by binary search over the sorted keys; runs of up
// to kShortRun sheets are insertion-sorted in place, longer ones are listed
// (start in list_start, length in list_len, count in counters[9]) for
// k_radix_long_ties, so no thread ever does work quadratic in a run.
constexpr int64_t kShortRun = 32;
__global__ void k_radix_ties(StateTable* table, int64_t n, const uint64_t* keys0,
                             const uint64_t* keys1, const uint32_t* plan, uint32_t* counters,
                             uint32_t* list_start, uint32_t* list_len, const StepFlags* flag,
                             const unsigned* err) {
  if (!flag->unsorted || !counters[8] || (*err & DEV_ERR_RADIX_TIMEOUT)) return;
  const int fb = (int)plan[kPlanFinal];
  const uint64_t* keys = fb ? keys1 : keys0;
  const StateRef oth = table->other;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p + 1 < n; p += stride) {
    const uint64_t kp = keys[p];
    if (kp != keys[p + 1] || (p > 0 && keys[p - 1] == kp)) continue;
    // last index e with keys[e] == kp: keys[p + 1] == kp, keys are sorted
    int64_t lo = p + 1, hi = n - 1;
    while (lo < hi) {
      const int64_t mid = lo + (hi - lo + 1) / 2;
      if (keys[mid] == kp) lo = mid; else hi = mid - 1;
    }
    const int64_t e = lo;
    if (e - p + 1 > kShortRun) {
      const unsigned slot = atomicAdd(&counters[9], 1u);
      list_start[slot] = (uint32_t)p;
      list_len[slot] = (uint32_t)(e - p + 1);
      continue;
    }
    for (int64_t i = p + 1; i <= e; ++i) {
      const double xi = oth.x[i], vi = oth.v[i], mi = oth.m[i];
      const int32_t ii = oth.idx[i];
      int64_t j = i - 1;
      while (j >= p && oth.idx[j] > ii) {
        oth.x[j + 1] = oth.x[j];
        oth.v[j + 1] = oth.v[j];
        oth.m[j + 1] = oth.m[j];
        oth.idx[j + 1] = oth.idx[j];
        --j;
      }
      oth.x[j + 1] = xi;
      oth.v[j + 1] = vi;
      oth.m[j + 1] = mi;
      oth.idx[j + 1] = ii;
    }
  }
}

// Long runs of equal keys, one CTA per run: a stable LSD radix sort (4-bit
// digits, each thread a contiguous chunk) of (index, place in run) pairs in
// the key buffers' slots of the run, then the run's sheets are permuted
// through the current set (free until the flip) and copied back.  Runs
// already in index order are left alone.  O(run length) work per digit.
constexpr int kLongTieThreads = 256;
__global__ void __launch_bounds__(kLongTieThreads) k_radix_long_ties(
    StateTable* table, int64_t n, uint64_t* bufa, uint64_t* bufb, const uint32_t* counters,
    const uint32_t* list_start, const uint32_t* list_len, const StepFlags* flag,
    const unsigned* err) {
  if (!flag->unsorted || !counters[9] || (*err & DEV_ERR_RADIX_TIMEOUT)) return;
  constexpr int T = kLongTieThreads;
  __shared__ uint32_t cnt[16][T + 1];
  __shared__ uint32_t tot[16];
  const int tid = threadIdx.x;
  const StateRef oth = table->other, cur = table->cur;
  int bits = 1;
  while (bits < 31 && ((int64_t)1 << bits) < n) ++bits;
  const int npass = (bits + 3) / 4;
  const unsigned nruns = counters[9];
  for (unsigned r = blockIdx.x; r < nruns; r += gridDim.x) {
    const int64_t s = list_start[r], L = list_len[r];
    bool unordered = false;
    for (int64_t j = tid; j + 1 < L; j += T) unordered |= oth.idx[s + j] > oth.idx[s + j + 1];
    if (!__syncthreads_or(unordered)) continue;
    uint64_t* src = bufa + s;
    uint64_t* dst = bufb + s;
    for (int64_t j = tid; j < L; j += T)
      src[j] = ((uint64_t)(uint32_t)oth.idx[s + j] << 32) | (uint64_t)j;
    const int64_t chunk = (L + T - 1) / T;
    const int64_t c_lo = (int64_t)tid * chunk < L ? (int64_t)tid * chunk : L;
    const int64_t c_hi = c_lo + chunk < L ? c_lo + chunk : L;
    __syncthreads();
    for (int ps = 0; ps < npass; ++ps) {
      const int shift = 32 + 4 * ps;
#pragma unroll
      for (int d = 0; d < 16; ++d) cnt[d][tid] = 0;
      for (int64_t j = c_lo; j < c_hi; ++j) ++cnt[(src[j] >> shift) & 15u][tid];
      __syncthreads();
      if (tid < 16) {  // digit-major exclusive offsets of each thread's chunk
        uint32_t run = 0;
        for (int t = 0; t < T; ++t) {
          const uint32_t c = cnt[tid][t];
          cnt[tid][t] = run;
          run += c;
        }
        tot[tid] = run;
      }
      __syncthreads();
      if (tid < 16) {
        uint32_t base = 0;
        for (int d = 0; d < tid; ++d) base += tot[d];
        for (int t = 0; t < T; ++t) cnt[tid][t] += base;
      }
      __syncthreads();
      for (int64_t j = c_lo; j < c_hi; ++j) {
        const uint64_t w = src[j];
        dst[cnt[(w >> shift) & 15u][tid]++] = w;
      }
      __syncthreads();
      uint64_t* t2 = src;
      src = dst;
      dst = t2;
    }
    for (int64_t j = tid; j < L; j += T) {
      const int64_t q = s + (int64_t)(uint32_t)src[j];
      cur.x[s + j] = oth.x[q];
      cur.v[s + j] = oth.v[q];
      cur.m[s + j] = oth.m[q];
      cur.idx[s + j] = oth.idx[q];
    }
    __syncthreads();
    for (int64_t j = tid; j < L; j += T) {
      oth.x[s + j] = cur.x[s + j];
      oth.v[s + j] = cur.v[s + j];
      oth.m[s + j] = cur.m[s + j];
      oth.idx[s + j] = cur.idx[s + j];
    }
    __syncthreads();
  }
}

__global__ void k_radix_flip(StateTable* table, const StepFlags* flag, const unsigned* err) {
  // after an expired wait the current set stays as it was (unsorted, intact)
  if (!flag->unsorted || (*err & DEV_ERR_RADIX_TIMEOUT)) return;
  const StateRef t = table->cur;
  table->cur = table->other;
  table->other = t;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Launch configuration of the radix passes on one device: its SM count and
// the resident pass CTAs per SM, after raising the pass kernel's dynamic
// shared-memory limit on that device.  Set up once per device (thread-safe).
struct RadixDevCfg {
  int sms = 1;
  int per_sm = 1;
};

void radix_cfg_init(RadixDevCfg& c, int dev) {
  constexpr size_t dyn = sizeof(PassSmem<kRadixThreads, kRadixItems>);
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(k_radix_pass<kRadixThreads, kRadixItems>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, k_radix_pass<kRadixThreads, kRadixItems>, kRadixThreads, dyn);
  c.sms = sms < 1 ? 1 : sms;
  c.per_sm = per_sm < 1 ? 1 : per_sm;
}

RadixDevCfg radix_cfg() {
  static std::once_flag once[kMaxDevices];
  static RadixDevCfg cfg[kMaxDevices];
  const int dev = current_device();
  if (dev < 0 || dev >= kMaxDevices) {
    RadixDevCfg c;
    radix_cfg_init(c, dev < 0 ? 0 : dev);
    return c;
  }
  std::call_once(once[dev], radix_cfg_init, std::ref(cfg[dev]), dev);
  return cfg[dev];
}

}  // namespace

size_t radix_bytes(int64_t n) {
  const int64_t tiles = (n + kRadixTile - 1) / kRadixTile;
  size_t b = 0;
  b += 2 * align256((size_t)n * 8);
  b += 2 * align256((size_t)n * 4);
  b += align256(8 * R * 4);
  b += align256(kPlanWords * 4);
  b += align256((size_t)8 * tiles * R * 4 + 16 * 4);
  return b;
}

void radix_bind(RadixWork* w, void* base, int64_t n) {
  char* p = static_cast<char*>(base);
  w->n_tiles = (n + kRadixTile - 1) / kRadixTile;
  w->keys[0] = reinterpret_cast<uint64_t*>(p); p += align256((size_t)n * 8);
  w->keys[1] = reinterpret_cast<uint64_t*>(p); p += align256((size_t)n * 8);
  w->pos[0] = reinterpret_cast<uint32_t*>(p); p += align256((size_t)n * 4);
  w->pos[1] = reinterpret_cast<uint32_t*>(p); p += align256((size_t)n * 4);
  w->hist = reinterpret_cast<uint32_t*>(p); p += align256(8 * R * 4);
  w->plan = reinterpret_cast<uint32_t*>(p); p += align256(kPlanWords * 4);
  w->status = reinterpret_cast<uint32_t*>(p);
  w->counters = w->status + (size_t)8 * w->n_tiles * R;
  w->scratch_bytes = (size_t)8 * w->n_tiles * R * 4 + 16 * 4;
}

void radix_sort_state(StateTable* table, int64_t n, RadixWork* w, const StepFlags* flag,
                      unsigned* err, cudaStream_t s) {
  constexpr size_t dyn = sizeof(PassSmem<kRadixThreads, kRadixItems>);
  static_assert(kRadixTile == PassSmem<kRadixThreads, kRadixItems>::TILE, "tile size");
  const RadixDevCfg cfg = radix_cfg();
  const int pass_grid_per_sm = cfg.per_sm, sms = cfg.sms;
  // the workspace may be bound for more sheets than this sort has: tiles,
  // look-back words and launches follow n
  const int64_t tiles = (n + kRadixTile - 1) / kRadixTile;
  cudaMemsetAsync(w->hist, 0, 8 * R * 4, s);
  cudaMemsetAsync(w->status, 0, (size_t)8 * tiles * R * 4, s);
  cudaMemsetAsync(w->counters, 0, 16 * 4, s);
  int hist_grid = (int)((n + 255) / 256);
  if (hist_grid > 152 * 8) hist_grid = 152 * 8;
  if (hist_grid < 1) hist_grid = 1;
  k_radix_hist<<<hist_grid, 256, 0, s>>>(table, n, w->hist, flag);
  k_radix_plan<<<1, R, 0, s>>>(n, w->hist, w->plan, flag);
  PassArgs a;
  a.table = table;
  a.n = n;
  a.n_tiles = tiles;
  a.keys0 = w->keys[0];
  a.keys1 = w->keys[1];
  a.pos0 = w->pos[0];
  a.pos1 = w->pos[1];
  a.plan = w->plan;
  a.status = w->status;
  a.counters = w->counters;
  a.flag = flag;
  a.err = err;
  int64_t pg = (int64_t)pass_grid_per_sm * sms;
  if (pg > tiles) pg = tiles;
  if (pg < 1) pg = 1;
  for (int p = 0; p < 8; ++p) {
    a.pass = p;
    k_radix_pass<kRadixThreads, kRadixItems><<<(unsigned)pg, kRadixThreads, dyn, s>>>(a);
  }
  int64_t gg = (n + kGatherThreads * kGatherUnroll - 1) / (kGatherThreads * kGatherUnroll);
  if (gg > (int64_t)sms * 8) gg = (int64_t)sms * 8;
  if (gg < 1) gg = 1;
  k_radix_gather<<<(unsigned)gg, kGatherThreads, 0, s>>>(table, n, w->keys[0], w->keys[1],
                                                          w->pos[0], w->pos[1], w->plan,
                                                          w->counters, flag, err);
  int g = (int)((n + 255) / 256);
  if (g > 152 * 16) g = 152 * 16;
  if (g < 1) g = 1;
  // pos[] is free once gathered: it holds the list of long runs
  k_radix_ties<<<g, 256, 0, s>>>(table, n, w->keys[0], w->keys[1], w->plan, w->counters,
                                 w->pos[0], w->pos[1], flag, err);
  // and, once the runs are listed, the key buffers are scratch for long ones
  k_radix_long_ties<<<sms, kLongTieThreads, 0, s>>>(table, n, w->keys[0], w->keys[1],
                                                    w->counters, w->pos[0], w->pos[1], flag,
                                                    err);
  k_radix_flip<<<1, 1, 0, s>>>(table, flag, err);
}

}  // namespace wg

