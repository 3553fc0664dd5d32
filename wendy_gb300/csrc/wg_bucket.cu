// wg_bucket.cu -- the fused sub-step on bucketed state.
//
// Between sub-steps the sheets of a simulation live in B buckets of fixed
// capacity; bucket b holds exactly the sheets whose (position key, index)
// lies in [Q_b, Q_{b+1}), in arbitrary order inside the bucket.  One kernel
// launch per sub-step then does, per bucket (one CTA, persistent over a list
// of (simulation, bucket) tasks):
//
//   claim the task one bucket ahead (warp 0, while the other warps write out
//     the previous bucket): the bucket's sheet count and exact fixed-point
//     mass were summed by the writers of the previous sub-step, so the
//     look-back over the earlier buckets of the same simulation for the
//     exclusive (mass, count) prefix never has to wait for a load
//   load the bucket into shared memory (optionally applying the half drift
//     a call starts with)
//   sort the bucket by (key, index) in shared memory: the bounded-window
//     fix-up, since a bucket only ever receives sheets from nearby buckets
//     (one counting-sort pass on a 12-bit order-preserving offset, equal
//     offsets ordered by the full key; a multi-pass radix sort when the keys
//     are too clustered for that)
//   exact prefix of the masses in sorted order, a = [ext(x,t) +]
//     (totmass - 2 C - m [- omega^2 x]); kick; drift
//   publish new splitters: the keys at global ranks j*T (quantiles)
//   route every sheet to the bucket of the next layout that covers its new
//     key (splitters computed by the previous sub-step), add the bucket's
//     count and mass to that layout's aggregates and append the sheet there
//     (the sheets of one warp bound for one bucket take consecutive slots)
//
// so a sub-step reads and writes each sheet once (28 B in, 28 B out).  A
// bucket that would overflow its capacity sends the sheet to an overflow
// list and flags the simulation, whose host side then re-sorts from scratch;
// no sheet is ever lost.  Simulations never interact: every sum, sort and
// splitter is per simulation, so a simulation gives the same bits alone and
// in an ensemble.
//
// Reference: _nbody_force and leapfrog_leappq, wendy/wendy.c:324-384; the
// argsort at wendy/wendy.c:341-357 is what the bucket sort replaces.
#include <cstdint>
#include <mutex>
#include <utility>
#include <vector>

#include "wg_bucket.cuh"

namespace wg {

namespace {

constexpr int BT = kBucketThreads;  // 256
constexpr int CAP = kBucketCap;     // 2048
constexpr int MAXI = CAP / BT;      // 8 sheets per thread at most
constexpr int WARPS = BT / 32;
constexpr int RWIN = kSplitterWindow;
constexpr int NBIN = 1 << kSortBitsMax;  // bins the shared memory is sized for
constexpr int MAXBIN = 48;          // a fuller bin sends the bucket to the radix sort
// Big buckets are cut into chunks of at most CAP sheets along 4096 key bins:
// a chunk starts at every bin whose exclusive count passes a multiple of
// CHUNK, so a chunk holds at most CHUNK + (its last bin) <= CAP sheets as long
// as no bin holds more than CAP - CHUNK.
constexpr int BIGBINS = 4096;
constexpr int CHUNK = CAP / 2;
constexpr int kMaxChunks = kBucketCapBig / CHUNK + 1;
// Two 16-bit bin counters (later offsets) per 32-bit word: bin b lives in the
// half (b & 1) of word b / 2.  Words are padded with one per 32 so that a
// thread scanning 16 consecutive words and its 31 neighbours hit 32
// different banks.
constexpr int NWORD = NBIN / 2;
constexpr int NBIN_PAD = NWORD + NWORD / 32 + 1;
__device__ __forceinline__ int binp(int w) { return w + (w >> 5); }
// Offset (or count) of bin b in the packed words.
__device__ __forceinline__ uint32_t bin_get(const uint32_t* bins, int b) {
  return (bins[binp(b >> 1)] >> ((b & 1) << 4)) & 0xffffu;
}

struct LsdSmem {
  uint32_t q[2][CAP];
  uint16_t p[2][CAP];
  uint32_t hist[WARPS][256];
};

// What the processing of one task needs, prepared by warp 0 one task ahead
// (while the other warps write out the current bucket), so that a bucket's
// load waits only for its bulk copies and not for a chain of dependent global
// reads, and its mass prefix is known before it starts.
struct TaskMeta {
  const double* x;
  const double* v;
  const double* m;
  const int32_t* idx;
  int64_t bucket;
  unsigned task;  // ticket; ntasks or more ends the launch
  int sim;
  int n;          // sheets in the bucket; -1: the simulation has aborted this call
  int lay;        // layout read by this sub-step
  uint32_t pcnt;  // sheets in the simulation's earlier buckets
  int wlo, whi;   // splitter window [wlo, whi] of the next layout ...
  int wbuf;       // ... in wkey[wbuf], widx[wbuf]
  double amp;     // time factor of a pulsed external force at this sub-step
  double inv_h;   // 1 / h of a pulsed external force
  uint64_t pm_lo, pm_hi;  // their fixed-point mass
};

struct StepSmem {
  double x[CAP];
  double v[CAP];
  double m[CAP];
  int32_t idx[CAP];
  uint16_t perm[CAP];  // sorted position -> slot
  union {
    struct {
      uint32_t bins[NBIN_PAD];
      uint64_t skey[CAP];  // key and index of each position in bin order
      int32_t sidx[CAP];
      uint32_t nlong;      // bins too full for one thread's insertion sort
    } srt;
    LsdSmem lsd;
    struct {
      u128 mfix[CAP];      // fixed-point mass of each sorted position
      uint16_t drk[CAP];   // rank of each sorted position among the sheets of its destination
      uint16_t order[CAP]; // sorted positions grouped by destination
      uint8_t dw[CAP];     // destination of each sorted position: window entry, or the
                           // window length for a bucket outside the window
    } pos;
  } u;
  // splitter windows of the next layout, double-buffered: the one of the
  // next task is read while the current task runs
  uint64_t wkey[2][2 * RWIN + 2];
  int32_t widx[2][2 * RWIN + 2];
  uint32_t dcount[2 * RWIN + 2];  // sheets bound for each window entry (+ outside the window)
  uint32_t dstart[2 * RWIN + 3];  // their exclusive prefix: segments of the grouped order
  uint32_t dbase[2 * RWIN + 2];   // first slot of each window bucket taken by this bucket
  unsigned next_ticket;              // the next task's ticket and entry, read ahead
  BucketTask next_tk;
  u128 warp_mass[WARPS];
  uint32_t warp_cnt[WARPS];
  uint32_t scan_tmp[WARPS];
  u128 prefix_mass;
  uint32_t prefix_cnt;
  uint64_t red_min[WARPS], red_max[WARPS];
  TaskMeta next;
  int win_lo, win_hi, cur_wbuf;
  double amp, inv_h;
  unsigned long long maxv;
  unsigned maxc;  // largest destination count this task saw after its reservations
  float vsum[WARPS];      // per warp: sum of the new velocities (predicted splitters)
  unsigned nsamp;         // splitter samples of this task (at most 3: n <= CAP < 3 target)
  double samp_x[4];
  int32_t samp_idx[4];
  uint32_t samp_q[4];
  uint64_t mbar;  // completion of the bucket's bulk copies
  // a big bucket (k_bucket_big): its chunks as ranges of key bins
  int chunk_lo[kMaxChunks + 1];
  int nchunks;
  unsigned load_cnt;  // sheets of the current chunk gathered so far
  unsigned splittable;
};

// Two CTAs per SM: 228 KiB of shared memory per SM, 1 KiB reserved per CTA.
static_assert(2 * (sizeof(StepSmem) + 1024) <= 228 * 1024, "StepSmem too large for 2 CTAs/SM");

__device__ __forceinline__ bool pair_less(uint64_t k1, int32_t i1, uint64_t k2, int32_t i2) {
  return k1 < k2 || (k1 == k2 && i1 < i2);
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and (through total) the block total.  Contains one barrier; the
// caller passes another before the next call (scan_tmp is reused).
__device__ __forceinline__ uint32_t block_excl_scan(StepSmem& S, uint32_t v, uint32_t& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) S.scan_tmp[warp] = incl;
  __syncthreads();
  uint32_t pre = 0;
  total = 0;
#pragma unroll
  for (int w = 0; w < WARPS; ++w) {
    const uint32_t t = S.scan_tmp[w];
    pre += (w < warp) ? t : 0u;
    total += t;
  }
  return pre + incl - v;
}

// Barrier of warps 1 .. WARPS-1 only (named barrier 1): warp 0 meanwhile
// prepares the next task.
__device__ __forceinline__ void bar_sync_workers() {
  asm volatile("bar.sync 1, %0;" ::"n"(BT - 32) : "memory");
}

// Multi-pass fallback: stable LSD radix sort of 32-bit order-preserving
// offsets, 8 bits per pass over the bits that differ, then exact tie order.
__device__ __forceinline__ void lsd_sort(StepSmem& S, int n, uint64_t kmin, uint64_t kmax) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t span = kmax - kmin;
  const int bits = span ? 64 - __clzll((long long)span) : 0;
  const int shift = bits > 32 ? bits - 32 : 0;
  const int passes = (bits - shift + 7) / 8;
  LsdSmem& L = S.u.lsd;
  __syncthreads();  // the union was just used as counting-sort bins
  for (int j = tid; j < n; j += BT) {
    L.q[0][j] = (uint32_t)((key_of(S.x[j]) - kmin) >> shift);
    L.p[0][j] = (uint16_t)j;
  }
  int cur = 0;
  __syncthreads();
  for (int pass = 0; pass < passes; ++pass) {
    const int ds = 8 * pass;
    for (int i = lane; i < 256; i += 32) L.hist[warp][i] = 0;
    __syncwarp();
    uint32_t rank[MAXI];
    unsigned dig[MAXI];
#pragma unroll
    for (int i = 0; i < MAXI; ++i) {
      const int j = warp * (32 * MAXI) + i * 32 + lane;
      const bool ok = j < n;
      const unsigned d = ok ? ((L.q[cur][j] >> ds) & 255u) : (256u + lane);
      dig[i] = d;
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      uint32_t old = 0;
      if (ok) {
        old = L.hist[warp][d];
        rank[i] = old + __popc(peers & lanemask_lt());
      }
      __syncwarp();
      if (ok && lane == __ffs(peers) - 1) L.hist[warp][d] = old + __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      const uint32_t c = L.hist[w][tid];
      L.hist[w][tid] = run;
      run += c;
    }
    uint32_t total;
    const uint32_t base = block_excl_scan(S, run, total);
#pragma unroll
    for (int w = 0; w < WARPS; ++w) L.hist[w][tid] += base;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < MAXI; ++i) {
      const int j = warp * (32 * MAXI) + i * 32 + lane;
      if (j < n) {
        const uint32_t dst = L.hist[warp][dig[i]] + rank[i];
        L.q[1 - cur][dst] = L.q[cur][j];
        L.p[1 - cur][dst] = L.p[cur][j];
      }
    }
    __syncthreads();
    cur = 1 - cur;
  }
  for (int j = tid; j < n; j += BT) S.perm[j] = L.p[cur][j];
  __syncthreads();
  // equal offsets: order by the full (key, idx)
  for (int j = tid; j + 1 < n; j += BT) {
    const uint32_t qj = L.q[cur][j];
    if (qj != L.q[cur][j + 1] || (j > 0 && L.q[cur][j - 1] == qj)) continue;
    int e = j + 1;
    while (e + 1 < n && L.q[cur][e + 1] == qj) ++e;
    for (int a = j + 1; a <= e; ++a) {
      const uint16_t s = S.perm[a];
      const uint64_t ks = key_of(S.x[s]);
      const int32_t is = S.idx[s];
      int b = a - 1;
      while (b >= j && pair_less(ks, is, key_of(S.x[S.perm[b]]), S.idx[S.perm[b]])) {
        S.perm[b + 1] = S.perm[b];
        --b;
      }
      S.perm[b + 1] = s;
    }
  }
  __syncthreads();
}

// Sort the n <= CAP sheets of the bucket by (key, idx) into S.perm, with
// 2^qb bins (9 <= qb <= 13).  The bin words are zero on entry (cleared while
// the bucket loads).
__device__ __forceinline__ void bucket_sort(StepSmem& S, int n, int ipt, uint64_t kmin,
                                            uint64_t kmax, int qb) {
  const int tid = threadIdx.x;
  const uint64_t span = kmax - kmin;
  const int nbin = 1 << qb;
  const int wpt = nbin / (2 * BT);  // bin words per thread in the scan (1..16)
  // Bin of a key: (key - kmin) * scale / 2^64, which is non-decreasing in the
  // key and spreads the bucket's key range over all nbin bins (a shift would
  // leave up to half of them empty).  The scale is a single-precision
  // reciprocal shrunk by 2^-20, so the largest key still lands below nbin;
  // a range narrower than nbin keys maps one key per bin.
  const bool narrow = span < (uint64_t)nbin;
  uint64_t scale = 0;
  if (!narrow) {
    const float f = (float)nbin / ((float)span + 1.0f) * 18446744073709551616.0f *
                    (1.0f - 9.5367431640625e-07f);
    scale = (uint64_t)f;
  }
  uint32_t* bins = S.u.srt.bins;
  uint64_t* skey = S.u.srt.skey;
  int32_t* sidx = S.u.srt.sidx;
  if (tid == 0) S.u.srt.nlong = 0;  // read after the barriers below
  uint16_t qv[MAXI], rk[MAXI];
#pragma unroll
  for (int i = 0; i < MAXI; ++i) {
    const int j = tid + i * BT;
    if (i < ipt && j < n) {
      const uint64_t dk = key_of(S.x[j]) - kmin;
      qv[i] = (uint16_t)(narrow ? dk : __umul64hi(dk, scale));
      const int sh = (qv[i] & 1) << 4;
      rk[i] = (uint16_t)(atomicAdd(&bins[binp(qv[i] >> 1)], 1u << sh) >> sh);
    }
  }
  __syncthreads();
  // exclusive scan of the bins: thread t owns words [wpt t, wpt t + wpt)
  constexpr int WMAX = NWORD / BT;
  uint32_t c[WMAX];
  uint32_t run = 0, mx = 0;
#pragma unroll
  for (int k = 0; k < WMAX; ++k) {
    c[k] = k < wpt ? bins[binp(tid * wpt + k)] : 0u;
    const uint32_t lo = c[k] & 0xffffu, hi = c[k] >> 16;
    mx = lo > mx ? lo : mx;
    mx = hi > mx ? hi : mx;
    run += lo + hi;
  }
  const int too_full = __syncthreads_or(mx > (uint32_t)MAXBIN);
  if (too_full) {
    lsd_sort(S, n, kmin, kmax);
    return;
  }
  uint32_t total;
  uint32_t off = block_excl_scan(S, run, total);
#pragma unroll
  for (int k = 0; k < WMAX; ++k) {
    const uint32_t lo = c[k] & 0xffffu, hi = c[k] >> 16;
    if (k < wpt) bins[binp(tid * wpt + k)] = off | ((off + lo) << 16);
    off += lo + hi;
  }
  if (tid == 0) bins[binp(nbin >> 1)] = (uint32_t)n;  // offset of bin nbin
  __syncthreads();
#pragma unroll
  for (int i = 0; i < MAXI; ++i) {
    const int j = tid + i * BT;
    if (i < ipt && j < n) {
      const uint32_t pos = bin_get(bins, qv[i]) + rk[i];
      S.perm[pos] = (uint16_t)j;
      skey[pos] = key_of(S.x[j]);
      sidx[pos] = S.idx[j];
    }
  }
  __syncthreads();
  // The order inside a bin came from atomics.  A bin holds two or more
  // sheets exactly when one of them took rank 1 in it: that sheet puts the
  // bin's few places in (key, idx) order, an insertion sort of their keys,
  // indices and slots in shared memory; every other sheet has nothing to do.
  // Bins of more than kOwnerSort sheets (rare) are counted and then ordered by
  // the whole block, each of their sheets counting the bin-mates that precede
  // it (owners never touch those bins).
  constexpr uint32_t kOwnerSort = 8;
#pragma unroll
  for (int i = 0; i < MAXI; ++i) {
    const int j = tid + i * BT;
    if (i < ipt && j < n && rk[i] == 1) {
      const uint32_t lo = bin_get(bins, qv[i]), hi = bin_get(bins, qv[i] + 1);
      if (hi - lo <= kOwnerSort) {
        for (uint32_t a = lo + 1; a < hi; ++a) {
          const uint64_t ka = skey[a];
          const int32_t ia = sidx[a];
          const uint16_t pa = S.perm[a];
          uint32_t b = a;
          while (b > lo && pair_less(ka, ia, skey[b - 1], sidx[b - 1])) {
            skey[b] = skey[b - 1];
            sidx[b] = sidx[b - 1];
            S.perm[b] = S.perm[b - 1];
            --b;
          }
          skey[b] = ka;
          sidx[b] = ia;
          S.perm[b] = pa;
        }
      } else {
        atomicAdd(&S.u.srt.nlong, 1u);
      }
    }
  }
  __syncthreads();
  if (S.u.srt.nlong == 0) return;
  // the full bins: each of their sheets counts the sheets of its bin that
  // precede it, then takes that place (keys and indices read-only here)
  uint32_t place[MAXI];
  uint16_t slot[MAXI];
#pragma unroll
  for (int i = 0; i < MAXI; ++i) {
    place[i] = 0xffffffffu;
    const int j = tid + i * BT;
    if (i < ipt && j < n) {
      const uint32_t lo = bin_get(bins, qv[i]), hi = bin_get(bins, qv[i] + 1);
      if (hi - lo > kOwnerSort) {
        const uint64_t kj = skey[lo + rk[i]];
        const int32_t ij = sidx[lo + rk[i]];
        uint32_t r = 0;
        for (uint32_t b = lo; b < hi; ++b) r += pair_less(skey[b], sidx[b], kj, ij) ? 1u : 0u;
        place[i] = lo + r;
        slot[i] = (uint16_t)j;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < MAXI; ++i)
    if (place[i] != 0xffffffffu) S.perm[place[i]] = slot[i];
  __syncthreads();
}

// Bucket of the next layout covering (k, i): the largest j with Q_j <= (k, i).
// (k, i) >= splitter j of the window (keys first; indices only on a tie)
__device__ __forceinline__ bool win_ge(const uint64_t* wk, const int32_t* wi, int j, uint64_t k,
                                       int32_t i) {
  const uint64_t K = wk[j];
  return k > K || (k == K && i >= wi[j]);
}

__device__ __forceinline__ int dest_bucket(const uint64_t* wk, const int32_t* wi, int lo, int w,
                                           const uint64_t* qk, const int32_t* qi, int64_t nb,
                                           uint64_t k, int32_t i) {
  if (win_ge(wk, wi, 0, k, i) && !win_ge(wk, wi, w, k, i)) {
    int l = 0, len = w;  // Q_{lo+l} <= (k,i) < Q_{lo+l+len}
    while (len > 1) {
      const int half = len >> 1;
      const bool ge = win_ge(wk, wi, l + half, k, i);
      l = ge ? l + half : l;
      len = ge ? len - half : half;
    }
    return lo + l;
  }
  int l = 0, h = (int)nb;  // Q_0 = -inf <= (k,i) < Q_nb = +inf
  while (h - l > 1) {
    const int mid = (l + h) >> 1;
    if (pair_less(k, i, __ldg(&qk[mid]), __ldg(&qi[mid])))
      h = mid;
    else
      l = mid;
  }
  return l;
}

__device__ __forceinline__ u128 mass_of_limbs(const unsigned long long* l) {
  return (u128)l[0] + ((u128)l[1] << 32) + ((u128)l[2] << 64) + ((u128)l[3] << 96);
}

// What the look-back reads of one earlier bucket.
struct PredLoad {
  unsigned c;          // its aggregate count ...
  u128 m;              // ... and mass
  ulonglong2 r0, r1;   // its look-back record
};

__device__ __forceinline__ PredLoad load_pred(const unsigned* cnt, const unsigned long long* mass,
                                              const BucketRec* recs, int64_t jj) {
  PredLoad p;
  if (jj >= 0) {
    p.c = cnt[jj];
    p.m = mass_of_limbs(mass + 4 * jj);
    const ulonglong2* r = reinterpret_cast<const ulonglong2*>(recs + jj);
    p.r0 = __ldcg(r);
    p.r1 = __ldcg(r + 1);
  } else {
    p.c = 0;
    p.m = 0;
    p.r0 = make_ulonglong2(0ull, 0ull);
    p.r1 = p.r0;
  }
  return p;
}

// Prepares task t (task-list entry tk) for processing; all lanes of one warp.
//
// Reads the simulation's abort word, its arrays for this sub-step, the
// bucket's aggregate and the splitter window of the next layout around the
// bucket, clears the bucket's aggregate slot two sub-steps on, and resolves
// the bucket's exclusive (mass, count) prefix by looking back over the
// earlier buckets of the simulation: a bucket whose inclusive prefix is
// published for this sub-step ends the walk, every other one contributes its
// aggregate.  Aggregates were completed by the previous launch, so the walk
// never waits; the bucket then publishes its own inclusive prefix.  The
// loads of the first look-back group are issued together with all the others.
__device__ __forceinline__ void prepare_task(const StepLaunch& L, int sub, unsigned ep, int lane,
                                             unsigned t, BucketTask tk, StepSmem& S, int wbuf) {
  TaskMeta& out = S.next;
  if (lane == 0) {
    out.task = t;
    out.wbuf = wbuf;
  }
  if (t >= (unsigned)L.ntasks) return;
  const SimDev& D = L.sims[tk.sim];
  const int64_t b = tk.bucket;
  const int cs = (D.cs0 + sub) % kAggSlots;
  const unsigned* cnt = D.bcnt[cs];
  const unsigned long long* mass = D.bmass[cs];
  const BucketRec* recs = D.recs;
  const int rw = D.window;
  const int64_t nbk = D.nb;
  const int wlo = (int)(b > rw ? b - rw : 0);
  const int whi = (int)((b + rw + 1) < nbk ? (b + rw + 1) : nbk);
  const int qs = (D.qsel0 + sub) & 1;
  const uint64_t* qdk = D.qk[qs];
  const int32_t* qdi = D.qi[qs];
  // ---- one round of loads
  const unsigned ab = __ldcg(D.ocount + 1);
  const unsigned own_c = cnt[b];
  const u128 own_m = mass_of_limbs(mass + 4 * b);
  constexpr int WQ = (2 * RWIN + 2 + 31) / 32;
  uint64_t wkr[WQ];
  int32_t wir[WQ];
#pragma unroll
  for (int q = 0; q < WQ; ++q) {
    const int j = lane + 32 * q;
    if (j <= whi - wlo) {
      wkr[q] = qdk[wlo + j];
      wir[q] = qdi[wlo + j];
    }
  }
  int64_t j = b - 1;
  PredLoad pl = load_pred(cnt, mass, recs, j - lane);
  double amp = 0.0, inv_h = 0.0;
  if (lane == 0 && D.ext.kind == EXT_PULSE_TANH) {
    amp = pulse_amplitude(D.ext, D.t_seq[sub]);
    inv_h = 1.0 / D.ext.p[3];
  }
  // an earlier sub-step of this call overflowed the simulation: its host
  // side finishes the call on the compact path
  if (ab != 0 && (int)ab <= sub) {
    if (lane == 0) out.n = -1;
    return;
  }
  const int capg = D.capg;
  const int n = own_c < (unsigned)capg ? (int)own_c : capg;
  const int lay = (D.lay0 + sub) & 1;
  if (lane == 0 && n > 0) {
    // the bucket is loaded after the current one: bring it into L2 now
    const uint32_t n4 = (uint32_t)((min(n, CAP) + 3) & ~3);
    const int64_t base = b * capg;
    bulk_prefetch_l2(D.bx[lay] + base, n4 * 8u);
    bulk_prefetch_l2(D.bv[lay] + base, n4 * 8u);
    bulk_prefetch_l2(D.bm[lay] + base, n4 * 8u);
    bulk_prefetch_l2(D.bi[lay] + base, n4 * 4u);
  }
#pragma unroll
  for (int q = 0; q < WQ; ++q) {
    const int jw = lane + 32 * q;
    if (jw <= whi - wlo) {
      S.wkey[wbuf][jw] = wkr[q];
      S.widx[wbuf][jw] = wir[q];
    }
  }
  {
    const int cz = (cs + 2) % kAggSlots;
    if (lane == 0) D.bcnt[cz][b] = 0u;
    if (lane < 4) D.bmass[cz][4 * b + lane] = 0ull;
  }
  // ---- look-back
  const uint64_t tag = (uint64_t)(ep & kEpochLimit) << 40;
  constexpr uint64_t PAY = (1ull << 40) - 1;
  u128 pm = 0;
  uint32_t pc = 0;
  while (j >= 0) {
    const bool inc = (j - lane >= 0) && ((pl.r0.x & ~PAY) == tag) &&
                     ((pl.r0.y & ~PAY) == tag) && ((pl.r1.x & ~PAY) == tag) &&
                     ((pl.r1.y & ~PAY) == tag);
    const u128 vm = inc ? ((u128)(pl.r0.x & PAY) | ((u128)(pl.r0.y & PAY) << 40) |
                           ((u128)(pl.r1.x & PAY) << 80) |
                           ((u128)((pl.r1.y >> 32) & 0x7Full) << 120))
                        : pl.m;
    const uint32_t vcl = inc ? (uint32_t)pl.r1.y : pl.c;
    const unsigned pmask = __ballot_sync(0xffffffffu, inc);
    const int stop = pmask ? (__ffs(pmask) - 1) : 31;
    const bool take = lane <= stop;
    pm += warp_sum_u128(take ? vm : (u128)0);
    uint32_t c = take ? vcl : 0u;
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) c += __shfl_xor_sync(0xffffffffu, c, d);
    pc += c;
    if (pmask) break;
    j -= 32;
    if (j >= 0) pl = load_pred(cnt, mass, recs, j - lane);
  }
  if (lane == 0) {
    const u128 im = pm + own_m;
    const uint32_t ic = pc + own_c;
    ulonglong2* r = reinterpret_cast<ulonglong2*>(D.recs + b);
    __stcg(r, make_ulonglong2(tag | ((uint64_t)im & PAY), tag | ((uint64_t)(im >> 40) & PAY)));
    __stcg(r + 1, make_ulonglong2(tag | ((uint64_t)(im >> 80) & PAY),
                                  tag | (((uint64_t)(im >> 120) & 0x7Full) << 32) | ic));
    out.sim = tk.sim;
    out.wlo = wlo;
    out.whi = whi;
    out.bucket = b;
    out.lay = lay;
    out.x = D.bx[lay];
    out.v = D.bv[lay];
    out.m = D.bm[lay];
    out.idx = D.bi[lay];
    out.n = n;
    out.amp = amp;
    out.inv_h = inv_h;
    out.pm_lo = (uint64_t)pm;
    out.pm_hi = (uint64_t)(pm >> 64);
    out.pcnt = pc;
  }
}

// Claims a ticket and prepares its task; all lanes of one warp.
__device__ __forceinline__ void claim_task(const StepLaunch& L, int sub, unsigned ep, int lane,
                                           StepSmem& S, int wbuf) {
  unsigned t = 0;
  if (lane == 0) t = atomicAdd(L.ticket, 1u);
  t = __shfl_sync(0xffffffffu, t, 0);
  BucketTask tk{0, 0};
  if (t < (unsigned)L.ntasks) tk = L.tasks[t];
  prepare_task(L, sub, ep, lane, t, tk, S, wbuf);
}

// Sort, scan, force, kick, drift, route and write out the n <= CAP sheets of
// a bucket (or of one chunk of a big bucket) that sit in shared memory, with
// their key range [kmin, kmax]; S.prefix_mass / S.prefix_cnt hold the
// exclusive (mass, count) prefix of the first of them and the splitter window
// of the next layout is in S.wkey[S.cur_wbuf].  PREP: warp 0 prepares the
// next task (S.next_ticket, ntk) during the grouping, as the main kernel's
// pipeline does; otherwise (chunks of a big bucket) the prefix base is
// advanced past these sheets at the end.
template <bool LAST, bool EXPR, bool PREP>
__device__ __forceinline__ void process_bucket(const StepLaunch& L, StepSmem& S, const SimDev& D,
                                               const int64_t b, const int lay, const int n,
                                               const int sub, const unsigned ep, uint64_t kmin,
                                               uint64_t kmax, const BucketTask ntk) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ipt = (n + BT - 1) / BT;
  const int E = D.E;
  const uint64_t* const wk = S.wkey[S.cur_wbuf];
  const int32_t* const wi = S.widx[S.cur_wbuf];
  // ---- sort the bucket
  if (n > 1) {
    bucket_sort(S, n, ipt, kmin, kmax, D.sort_bits);
  } else {
    if (tid == 0) S.perm[0] = 0;
    __syncthreads();
  }

  // ---- exact prefix of the masses in sorted order: thread tid holds the
  // sorted positions [tid * ipt, tid * ipt + ipt)
  if (PREP && tid == 0) S.next_tk = ntk;
  const int j0 = tid * ipt;
  const int nmine = (j0 < n) ? ((n - j0) < ipt ? (n - j0) : ipt) : 0;
  u128 tot = 0;
  for (int i = 0; i < nmine; ++i) {
    const u128 M = mass_to_fixed(S.m[S.perm[j0 + i]], E);
    S.u.pos.mfix[j0 + i] = M;
    tot += M;
  }
  const u128 incl = warp_inclusive_scan_u128(tot, lane);
  uint32_t cin = (uint32_t)nmine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, cin, o);
    if (lane >= o) cin += y;
  }
  if (lane == 31) {
    S.warp_mass[warp] = incl;
    S.warp_cnt[warp] = cin;
  }
  __syncthreads();
  u128 C = S.prefix_mass;
  uint32_t rank0 = S.prefix_cnt;
#pragma unroll
  for (int w = 0; w < WARPS; ++w) {
    if (w < warp) {
      C += S.warp_mass[w];
      rank0 += S.warp_cnt[w];
    }
  }
  C += incl - tot;
  rank0 += cin - (uint32_t)nmine;

  // ---- splitters of the layout after next: keys at global ranks j*T
  uint64_t* qnk = D.qk[1 - ((D.qsel0 + sub) & 1)];
  int32_t* qni = D.qi[1 - ((D.qsel0 + sub) & 1)];
  if (b == 0 && tid == 0) {
    qnk[0] = 0ull;
    qni[0] = (int32_t)0x80000000;
    qnk[D.nb] = ~0ull;
    qni[D.nb] = 0x7fffffff;
  }
  // descriptor fields used per sheet, held in registers (the descriptor is
  // in global memory and the compiler cannot prove the stores below leave it alone)
  const int has_omega = D.has_omega;
  const double omega2 = D.omega2;
  const ExtForce ext = D.ext;
  // an expression force: its time phase, once per task and thread
  double xr[EXPR ? kExprRegs : 1];
  double t_ev = 0.0;
  if constexpr (EXPR) {
    if (ext.kind == EXT_EXPR) {
      t_ev = D.t_seq[sub];
      expr_time(ext, t_ev, xr);
    }
  }
  const uint32_t target = (uint32_t)D.target;
  const int64_t nbk = D.nb;
  // ---- force, kick, drift, routing; new x, v go back to their slots and
  // the destination of every sorted position to the (now free) sort area
  const double dt = L.profile ? 0.0 : D.dt;
  const double dt_drift = LAST ? dt / 2. : dt;
  const double dest_dt = (LAST && !L.profile) ? dt / 2. : 0.0;
  const i128 T = (i128)((((u128)D.T_hi) << 64) | D.T_lo);
  unsigned long long maxv = 0;
  StateTable* const ptab = D.ptab;  // predicted splitters this sub-step

  // the first rank >= rank0 that is a positive multiple of the target
  // starts the next splitter (one per thread at most: ipt <= 8 < target)
  uint32_t qnext = (rank0 + target - 1) / target;
  qnext = qnext ? qnext : 1u;
  const uint32_t rnext = qnext * target;
  // two sheets at a time, interleaved, so that their shared-memory and
  // FP64 latencies overlap; the window searches run in lock-step
  const int wlen = S.win_hi - S.win_lo;
  int top = 1;
  while ((top << 1) < wlen) top <<= 1;
  for (int i0 = 0; i0 < nmine; i0 += 2) {
    const bool ok1 = i0 + 1 < nmine;
    int sl[2];
    uint64_t kd[2];
    int32_t idv[2];
    bool live[2] = {true, ok1};
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      sl[u] = S.perm[j0 + (live[u] ? i0 + u : i0)];
      idv[u] = S.idx[sl[u]];
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      if (!live[u]) {
        kd[u] = 0;
        continue;
      }
      const int sidx = sl[u];
      const uint32_t r = rank0 + (uint32_t)(i0 + u);
      const double x = S.x[sidx], v = S.v[sidx];
      if (r == rnext) {
        qnk[qnext] = key_of(x);
        qni[qnext] = idv[u];
        if (ptab) {
          const unsigned k = atomicAdd(&S.nsamp, 1u);
          if (k < 4u) {
            S.samp_x[k] = x;
            S.samp_idx[k] = idv[u];
            S.samp_q[k] = qnext;
          }
        }
      }
      const u128 M = S.u.pos.mfix[j0 + i0 + u];
      const i128 A = T - 2 * (i128)C - (i128)M;
      C += M;
      double acc = fixed_to_double(A, E);
      if (has_omega) acc = fma(-omega2, x, acc);
      if constexpr (EXPR) {
        if (ext.kind == EXT_EXPR)
          acc = expr_space(ext, xr, x, t_ev) + acc;
        else if (ext.kind != EXT_NONE)
          acc = ext_force_at(ext, S.amp, S.inv_h, x) + acc;
      } else if (ext.kind != EXT_NONE) {
        acc = ext_force_at(ext, S.amp, S.inv_h, x) + acc;
      }
      const double vn = fma(dt, acc, v);
      const double xn = fma(dt_drift, vn, x);
      S.x[sidx] = xn;
      S.v[sidx] = vn;

      const unsigned long long av =
          (unsigned long long)__double_as_longlong(vn) & 0x7FFFFFFFFFFFFFFFull;
      maxv = av > maxv ? av : maxv;
      if (LAST && !L.profile) {
        OutRec* const ro = D.rec_out;
        if (ro) {
          double2* const r2 = reinterpret_cast<double2*>(ro + idv[u]);
          r2[0] = make_double2(xn, vn);
          r2[1] = make_double2(acc, 0.0);
        } else {
          D.x_out[idv[u]] = xn;
          D.v_out[idv[u]] = vn;
          double* const a_out = D.a_out;
          if (a_out) a_out[idv[u]] = acc;
        }
        SheetRec* const xi_out = D.xi_out;
        if (xi_out) {
          SheetRec rec;
          rec.idx = idv[u];
          rec.pad = 0;
          rec.val = xn;
          xi_out[r] = rec;
        }
      }
      kd[u] = key_of(LAST && dest_dt != 0.0 ? fma(dest_dt, vn, xn) : xn);
    }
    // routing: binary lifting over the window, both sheets in lock-step
    int l[2] = {0, 0};
    bool inw[2];
#pragma unroll
    for (int u = 0; u < 2; ++u)
      inw[u] = live[u] && win_ge(wk, wi, 0, kd[u], idv[u]) && !win_ge(wk, wi, wlen, kd[u], idv[u]);
    // the largest l with key Q_l <= key, on keys alone; then splitters with
    // an equal key and a larger index step back (pair order)
    for (int step = top; step >= 1; step >>= 1) {
#pragma unroll
      for (int u = 0; u < 2; ++u)
        if (l[u] + step < wlen && wk[l[u] + step] <= kd[u]) l[u] += step;
    }
#pragma unroll
    for (int u = 0; u < 2; ++u)
      while (l[u] > 0 && wk[l[u]] == kd[u] && wi[l[u]] > idv[u]) --l[u];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      if (!live[u]) continue;
      // destination: window entry l, or wlen for a bucket outside the
      // window (found again, by a global search, where it is needed)
      const int w = inw[u] ? l[u] : wlen;
      const int pq = j0 + i0 + u;
      S.u.pos.dw[pq] = (uint8_t)w;
      S.u.pos.drk[pq] = (uint16_t)atomicAdd(&S.dcount[w], 1u);
    }
  }
  if (ptab) {
    // the new velocities of this thread's sheets (back from shared memory:
    // a register held across the force loop would spill)
    float vsum = 0.f;
    for (int i = 0; i < nmine; ++i) vsum += (float)S.v[S.perm[j0 + i]];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) vsum += __shfl_xor_sync(0xffffffffu, vsum, o);
    if (lane == 0) S.vsum[warp] = vsum;
  }
  __syncthreads();
  if (ptab && tid < (int)min(S.nsamp, 4u)) {
    // the sample's position moved on by two drifts at the bucket's mean
    // velocity: where the bucket is heading.  The mean, not the sample's
    // own velocity: in a warm region single velocities would scatter the
    // splitters by more than a bucket, while the mean follows the bulk flow
    // of a collapsing or breathing slab (single precision is plenty for a
    // splitter, which only has to be near the quantile)
    float vs = 0.f;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) vs += S.vsum[w];
    const StateRef c = ptab->cur;
    const uint32_t q = S.samp_q[tid];
    c.x[q - 1] = fma(2.0 * dt, (double)(vs / (float)n), S.samp_x[tid]);
    c.idx[q - 1] = S.samp_idx[tid];
  }
  // ---- the sheets grouped by destination bucket of the next layout.  Warp 0
  // prepares the next task meanwhile; the other warps synchronise among
  // themselves (named barrier 1) until the block-wide barrier below.
  const int cw = (D.cs0 + sub + 1) % kAggSlots;
  unsigned* const cnt_out = D.bcnt[cw];
  unsigned long long* const mass_out = D.bmass[cw];
  const uint64_t* const qfar = D.qk[(D.qsel0 + sub) & 1];
  const int32_t* const ifar = D.qi[(D.qsel0 + sub) & 1];
  uint32_t db = 0;
  if (warp == 0) {
    if constexpr (PREP) prepare_task(L, sub, ep, lane, S.next_ticket, S.next_tk, S, S.cur_wbuf ^ 1);
  } else {
    const int wt = tid - 32;  // 0 .. BT - 33
    // slots: one atomic per window bucket, its round trip overlapping the
    // grouping and the mass sums
    if (wt < wlen) {
      const uint32_t c = S.dcount[wt];
      if (c) {
        db = atomicAdd(&cnt_out[S.win_lo + wt], c);
        atomicMax(&S.maxc, db + c);
      }
    }
    if (warp == 1) {
      // segments: exclusive prefix of the counts of the wlen + 1 entries
      constexpr int E5 = (2 * RWIN + 2 + 31) / 32;
      uint32_t cv[E5];
      uint32_t sum = 0;
#pragma unroll
      for (int k = 0; k < E5; ++k) {
        const int j = lane * E5 + k;
        cv[k] = j <= wlen ? S.dcount[j] : 0u;
        sum += cv[k];
      }
      uint32_t incl = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      uint32_t ex = incl - sum;
#pragma unroll
      for (int k = 0; k < E5; ++k) {
        const int j = lane * E5 + k;
        if (j <= wlen) S.dstart[j] = ex;
        ex += cv[k];
      }
      if (lane == 31) S.dstart[wlen + 1] = incl;
    }
    bar_sync_workers();
    for (int pq = wt; pq < n; pq += BT - 32)
      S.u.pos.order[S.dstart[S.u.pos.dw[pq]] + S.u.pos.drk[pq]] = (uint16_t)pq;
    bar_sync_workers();
    // ---- masses of the next layout: a warp sums the fixed-point masses of
    // a window bucket's segment and adds them to that bucket's accumulators
    for (int w = warp - 1; w < wlen; w += WARPS - 1) {
      const int q0 = (int)S.dstart[w], q1 = (int)S.dstart[w + 1];
      if (q0 == q1) continue;
      u128 P = 0;
      for (int q = q0 + lane; q < q1; q += 32) P += S.u.pos.mfix[S.u.pos.order[q]];
      P = warp_sum_u128(P);
      if (lane < 4) {
        const unsigned long long limb = (unsigned long long)(uint32_t)(P >> (32 * lane));
        if (limb) atomicAdd(&mass_out[4 * (int64_t)(S.win_lo + w) + lane], limb);
      }
    }
    // sheets bound outside the window: one by one
    for (int q = (int)S.dstart[wlen] + wt; q < n; q += BT - 32) {
      const int pq = S.u.pos.order[q];
      const int sl = S.perm[pq];
      const double xn = S.x[sl];
      const uint64_t kf = key_of(LAST && dest_dt != 0.0 ? fma(dest_dt, S.v[sl], xn) : xn);
      const int d = dest_bucket(wk, wi, S.win_lo, wlen, qfar, ifar, nbk, kf, S.idx[sl]);
      const u128 M = S.u.pos.mfix[pq];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const unsigned long long limb = (unsigned long long)(uint32_t)(M >> (32 * k));
        if (limb) atomicAdd(&mass_out[4 * (int64_t)d + k], limb);
      }
    }
    if (wt < wlen) S.dbase[wt] = db;
  }
  __syncthreads();
  bool overflow = false;
  {
    // write-out grouped by destination: consecutive positions of a segment
    // take consecutive slots, so a warp's stores coalesce
    double* const xout = D.bx[1 - lay];
    double* const vout = D.bv[1 - lay];
    double* const mout = D.bm[1 - lay];
    int32_t* const iout = D.bi[1 - lay];
    for (int q = tid; q < n; q += BT) {
      const int pq = S.u.pos.order[q];
      const int w = S.u.pos.dw[pq];
      const int sl = S.perm[pq];
      int d;
      uint32_t slot;
      if (w < wlen) {
        d = S.win_lo + w;
        slot = S.dbase[w] + (uint32_t)q - S.dstart[w];
      } else {
        const double xn = S.x[sl];
        const uint64_t kf = key_of(LAST && dest_dt != 0.0 ? fma(dest_dt, S.v[sl], xn) : xn);
        d = dest_bucket(wk, wi, S.win_lo, wlen, qfar, ifar, nbk, kf, S.idx[sl]);
        slot = atomicAdd(&cnt_out[d], 1u);
        atomicMax(&S.maxc, slot + 1u);
      }
      if (slot < (uint32_t)D.capg) {
        const int64_t o = (int64_t)d * D.capg + slot;
        xout[o] = S.x[sl];
        vout[o] = S.v[sl];
        mout[o] = S.m[sl];
        iout[o] = S.idx[sl];
      } else {
        const uint32_t o = atomicAdd(D.ocount, 1u);
        D.ox[o] = S.x[sl];
        D.ov[o] = S.v[sl];
        D.om[o] = S.m[sl];
        D.oi[o] = S.idx[sl];
        overflow = true;
      }
    }
  }
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, maxv, d);
    maxv = o > maxv ? o : maxv;
  }
  if (lane == 0 && maxv) atomicMax(&S.maxv, maxv);
  if (overflow) atomicCAS(D.ocount + 1, 0u, (unsigned)(sub + 1));
  __syncthreads();
  if (tid == 0 && S.maxv) atomicMax(&D.flags[sub + 1].max_v, S.maxv);
  if (tid == 0 && S.maxc) atomicMax(&D.flags[sub + 1].max_cnt, S.maxc);
  if (!PREP && tid == 0) {
    // the next chunk of a big bucket starts where this one ended
    u128 tot_all = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) tot_all += S.warp_mass[w];
    S.prefix_mass += tot_all;
    S.prefix_cnt += (uint32_t)n;
  }
}

// Appends a big bucket's task to the list k_bucket_big works through (one
// thread).  Kept out of line: inlined, its fields stayed live across the
// bucket loop and pushed the kernel into register spills.
static __device__ __noinline__ void list_big(const TaskMeta* tm, unsigned* big_count,
                                             unsigned big_cap, BigTask* big_list,
                                             unsigned* err) {
  const unsigned slot = atomicAdd(big_count, 1u);
  if (slot >= big_cap) {
    atomicOr(err, DEV_ERR_BAD_STATE);
    return;
  }
  BigTask bt;
  bt.sim = tm->sim;
  bt.bucket = (int)tm->bucket;
  bt.n = tm->n;
  bt.lay = tm->lay;
  bt.wlo = tm->wlo;
  bt.whi = tm->whi;
  bt.pcnt = tm->pcnt;
  bt.pm_lo = tm->pm_lo;
  bt.pm_hi = tm->pm_hi;
  bt.amp = tm->amp;
  bt.inv_h = tm->inv_h;
  big_list[slot] = bt;
}

// The fused sub-step.  LAST: the call's last sub-step (half drift, outputs).
// EXPR: the launch has simulations with expression forces (the interpreter
// is compiled only into this instantiation).
template <bool LAST, bool EXPR>
__global__ void __launch_bounds__(BT, 2) k_bucket_step(const StepLaunch L) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  StepSmem& S = *reinterpret_cast<StepSmem*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int sub = L.sub;
  const unsigned ep = L.epochs[sub];
  if (tid == 0) {
    mbar_init(&S.mbar, 1);
    fence_proxy_async_smem();
  }
  if (warp == 0) claim_task(L, sub, ep, lane, S, 0);
  unsigned parity = 0;
  for (;;) {
    __syncthreads();
    const TaskMeta tm = S.next;  // claimed during the previous task
    if (tm.task >= (unsigned)L.ntasks) break;
    if (tm.n < 0 || tm.n > CAP) {
      // n < 0: the simulation has aborted this call.  n > CAP: more sheets
      // than shared memory holds (a simulation whose layout has room for
      // them): listed for k_bucket_big, which runs next on the stream and
      // takes the bucket in chunks; its prefix is known already.
      if (tm.n > CAP && tid == 0) list_big(&S.next, L.big_count, L.big_cap, L.big_list, L.err);
      __syncthreads();  // every thread has read S.next
      if (warp == 0) claim_task(L, sub, ep, lane, S, tm.wbuf);
      continue;
    }
    const SimDev& D = L.sims[tm.sim];
    const int64_t b = tm.bucket;
    const int lay = tm.lay;
    const int n = tm.n;
    const int64_t base = b * D.capg;
    // ---- load: the bucket's four arrays arrive by bulk copy (sizes rounded
    // up to 4 sheets, which stays inside the bucket's capacity), then its
    // keys and key range are formed from shared memory
    const int n4 = (n + 3) & ~3;
    if (n4 > 0 && tid == 0) {
      fence_proxy_async_smem();  // earlier generic accesses to these buffers are done
      mbar_expect_tx(&S.mbar, (uint32_t)n4 * 28u);
      bulk_g2s(S.x, tm.x + base, (uint32_t)n4 * 8u, &S.mbar);
      bulk_g2s(S.v, tm.v + base, (uint32_t)n4 * 8u, &S.mbar);
      bulk_g2s(S.m, tm.m + base, (uint32_t)n4 * 8u, &S.mbar);
      bulk_g2s(S.idx, tm.idx + base, (uint32_t)n4 * 4u, &S.mbar);
    }
    // the next task's ticket and task-list entry are read ahead (thread 0)
    // and the task is prepared by warp 0 during the write-out
    unsigned nt = 0;
    if (tid == 0) nt = atomicAdd(L.ticket, 1u);
    const double pre = sub == 0 ? D.pre_dt : 0.0;
    // the splitter window of the next layout around this bucket arrived with
    // the task; the per-destination counters are cleared here
    for (int j = tid; j <= tm.whi - tm.wlo; j += BT) S.dcount[j] = 0;  // wlen + 1 entries
    if (tid == 0) {
      S.win_lo = tm.wlo;
      S.win_hi = tm.whi;
      S.cur_wbuf = tm.wbuf;
      S.maxv = 0;
      S.maxc = 0;
      S.nsamp = 0;
      S.prefix_mass = (((u128)tm.pm_hi) << 64) | tm.pm_lo;
      S.prefix_cnt = tm.pcnt;
      S.amp = tm.amp;
      S.inv_h = tm.inv_h;
    }
    {
      // counting-sort bins, cleared while the copies are in flight
      for (int j = tid; j < NBIN_PAD; j += BT) S.u.srt.bins[j] = 0u;
    }
    // the copies' completion: a thread that did not see it within the bounded
    // wait leaves the data alone, and the barrier after the key range below
    // (which every thread reaches) decides for the whole CTA
    const bool arrived = n4 > 0 ? mbar_wait(&S.mbar, parity) : true;
    uint64_t kmin = ~0ull, kmax = 0;
    if (arrived) {
#pragma unroll 4
      for (int j = tid; j < n; j += BT) {
        double x = S.x[j];
        if (pre != 0.0) {
          x = fma(pre, S.v[j], x);
          S.x[j] = x;
        }
        const uint64_t k = key_of(x);
        kmin = k < kmin ? k : kmin;
        kmax = k > kmax ? k : kmax;
      }
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
      const uint64_t o1 = __shfl_xor_sync(0xffffffffu, kmin, d);
      const uint64_t o2 = __shfl_xor_sync(0xffffffffu, kmax, d);
      kmin = o1 < kmin ? o1 : kmin;
      kmax = o2 > kmax ? o2 : kmax;
    }
    if (lane == 0) {
      S.red_min[warp] = kmin;
      S.red_max[warp] = kmax;
    }
    if (__syncthreads_or(!arrived)) {
      // the bucket's copies did not complete within the bounded wait: its
      // contents are unknown, so this CTA writes nothing more.  It gives the
      // copies a second bounded wait and stops; the host sees the error word
      // (the call fails and the simulation is given up).
      if (tid == 0) atomicOr(L.err, DEV_ERR_COPY_TIMEOUT);
      mbar_wait(&S.mbar, parity);
      break;
    }
    if (n4 > 0) parity ^= 1u;
    BucketTask ntk{0, 0};
    if (tid == 0) {
      S.next_ticket = nt;
      if (nt < (unsigned)L.ntasks) ntk = L.tasks[nt];
    }
    kmin = ~0ull;
    kmax = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      kmin = S.red_min[w] < kmin ? S.red_min[w] : kmin;
      kmax = S.red_max[w] > kmax ? S.red_max[w] : kmax;
    }
    process_bucket<LAST, EXPR, true>(L, S, D, b, lay, n, sub, ep, kmin, kmax, ntk);
  }
}

// Bin of a key in [kmin, kmin + span] among BIGBINS (non-decreasing in the
// key; the same multiplicative map as the in-bucket counting sort).
__device__ __forceinline__ int big_bin(uint64_t k, uint64_t kmin, uint64_t span, uint64_t scale) {
  const uint64_t dk = k - kmin;
  return span < (uint64_t)BIGBINS ? (int)dk : (int)__umul64hi(dk, scale);
}

// Position (with the opening half drift of a call applied) of slot j.
__device__ __forceinline__ double big_pos(const double* gx, const double* gv, int j, double pre) {
  const double x = gx[j];
  return pre != 0.0 ? fma(pre, gv[j], x) : x;
}

// Block-wide minimum and maximum of per-thread key ranges (all threads).
__device__ __forceinline__ void block_range(StepSmem& S, uint64_t& kmin, uint64_t& kmax) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    const uint64_t o1 = __shfl_xor_sync(0xffffffffu, kmin, d);
    const uint64_t o2 = __shfl_xor_sync(0xffffffffu, kmax, d);
    kmin = o1 < kmin ? o1 : kmin;
    kmax = o2 > kmax ? o2 : kmax;
  }
  if (lane == 0) {
    S.red_min[warp] = kmin;
    S.red_max[warp] = kmax;
  }
  __syncthreads();
  kmin = ~0ull;
  kmax = 0;
#pragma unroll
  for (int w = 0; w < WARPS; ++w) {
    kmin = S.red_min[w] < kmin ? S.red_min[w] : kmin;
    kmax = S.red_max[w] > kmax ? S.red_max[w] : kmax;
  }
  __syncthreads();  // red_min / red_max are free again
}

// The big buckets k_bucket_step listed in this sub-step (kBucketCap < n <=
// capg sheets): each is cut by key into chunks that fit in shared memory --
// a histogram of its keys over BIGBINS bins, chunks along the bins -- and
// every chunk is gathered from the layout and processed like a bucket, the
// chunks in key order with the mass and rank prefix carried from one to the
// next.  A bucket whose keys crowd into one bin beyond CAP - CHUNK cannot be
// cut this way: the simulation is flagged (ocount[2]) and its host side
// re-sorts the layout this sub-step read, which the sub-step leaves intact.
template <bool LAST, bool EXPR>
__global__ void __launch_bounds__(BT, 2) k_bucket_big(const StepLaunch L) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  StepSmem& S = *reinterpret_cast<StepSmem*>(smem_raw);
  const int tid = threadIdx.x;
  const int sub = L.sub;
  const unsigned ep = L.epochs[sub];
  const unsigned total = *L.big_count;  // final: k_bucket_step ran before
  const unsigned ntask = total < L.big_cap ? total : L.big_cap;
  for (;;) {
    __syncthreads();
    if (tid == 0) S.next_ticket = atomicAdd(L.big_ticket, 1u);
    __syncthreads();
    const unsigned t = S.next_ticket;
    if (t >= ntask) break;
    const BigTask bt = L.big_list[t];
    const SimDev& D = L.sims[bt.sim];
    const int n = bt.n;
    const int64_t base = (int64_t)bt.bucket * D.capg;
    const double* gx = D.bx[bt.lay] + base;
    const double* gv = D.bv[bt.lay] + base;
    const double* gm = D.bm[bt.lay] + base;
    const int32_t* gi = D.bi[bt.lay] + base;
    const double pre = sub == 0 ? D.pre_dt : 0.0;
    // the splitter window of the next layout around the bucket
    {
      const int qs = (D.qsel0 + sub) & 1;
      for (int j = tid; j <= bt.whi - bt.wlo; j += BT) {
        S.wkey[0][j] = D.qk[qs][bt.wlo + j];
        S.widx[0][j] = D.qi[qs][bt.wlo + j];
      }
    }
    if (tid == 0) {
      S.win_lo = bt.wlo;
      S.win_hi = bt.whi;
      S.cur_wbuf = 0;
      S.maxv = 0;
      S.maxc = 0;
      S.nsamp = 0;
      S.prefix_mass = (((u128)bt.pm_hi) << 64) | bt.pm_lo;
      S.prefix_cnt = bt.pcnt;
      S.amp = bt.amp;
      S.inv_h = bt.inv_h;
      S.nchunks = 0;
      S.splittable = 1u;
      for (int c = 0; c <= kMaxChunks; ++c) S.chunk_lo[c] = BIGBINS;
    }
    // ---- the bucket's key range and the histogram of its keys
    uint64_t kmin = ~0ull, kmax = 0;
    for (int j = tid; j < n; j += BT) {
      const uint64_t k = key_of(big_pos(gx, gv, j, pre));
      kmin = k < kmin ? k : kmin;
      kmax = k > kmax ? k : kmax;
    }
    uint32_t* hist = S.u.srt.bins;  // BIGBINS 32-bit counters
    for (int j = tid; j < BIGBINS; j += BT) hist[j] = 0u;
    block_range(S, kmin, kmax);
    const uint64_t span = kmax - kmin;
    uint64_t scale = 0;
    if (span >= (uint64_t)BIGBINS)
      scale = (uint64_t)((float)BIGBINS / ((float)span + 1.0f) * 18446744073709551616.0f *
                         (1.0f - 9.5367431640625e-07f));
    for (int j = tid; j < n; j += BT) {
      const int bin = big_bin(key_of(big_pos(gx, gv, j, pre)), kmin, span, scale);
      atomicAdd(&hist[bin], 1u);
    }
    __syncthreads();
    // ---- chunks: thread tid owns bins [16 tid, 16 tid + 16)
    {
      constexpr int BPT = BIGBINS / BT;
      uint32_t c[BPT], sum = 0, mx = 0;
#pragma unroll
      for (int k = 0; k < BPT; ++k) {
        c[k] = hist[tid * BPT + k];
        sum += c[k];
        mx = c[k] > mx ? c[k] : mx;
      }
      uint32_t tot;
      uint32_t ex = block_excl_scan(S, sum, tot);
      if (mx > (uint32_t)(CAP - CHUNK)) atomicAnd(&S.splittable, 0u);
      // non-empty bin i belongs to chunk floor(ex_i / CHUNK), ex_i the
      // sheets in earlier bins; a chunk starts at its first bin.  With no
      // bin above CHUNK, consecutive non-empty bins differ by at most one
      // chunk, and a chunk holds fewer than 2 CHUNK = CAP sheets.
#pragma unroll
      for (int k = 0; k < BPT; ++k) {
        if (c[k]) {
          const uint32_t chunk = ex / CHUNK;
          if (chunk < (uint32_t)kMaxChunks) atomicMin(&S.chunk_lo[chunk], tid * BPT + k);
          atomicMax(&S.nchunks, (int)chunk + 1);
        }
        ex += c[k];
      }
    }
    __syncthreads();
    const int nchunks = S.nchunks;
    if (!S.splittable || nchunks > kMaxChunks) {
      // keys crowded into one bin: the host re-sorts the layout read here
      if (tid == 0) {
        atomicCAS(D.ocount + 2, 0u, (unsigned)(sub + 1));
        atomicCAS(D.ocount + 1, 0u, (unsigned)(sub + 1));
      }
      continue;
    }
    if (tid == 0) {
      S.chunk_lo[0] = 0;  // bins below the first non-empty one are empty
      S.chunk_lo[nchunks] = BIGBINS;
    }
    __syncthreads();
    // ---- the chunks in key order
    for (int ch = 0; ch < nchunks; ++ch) {
      const int blo = S.chunk_lo[ch], bhi = S.chunk_lo[ch + 1];
      for (int j = tid; j < NBIN_PAD; j += BT) S.u.srt.bins[j] = 0u;
      for (int j = tid; j <= S.win_hi - S.win_lo; j += BT) S.dcount[j] = 0;
      if (tid == 0) {
        S.load_cnt = 0;
        S.nsamp = 0;  // splitter samples of this chunk
      }
      __syncthreads();
      uint64_t cmin = ~0ull, cmax = 0;
      for (int j = tid; j < n; j += BT) {
        const double x = big_pos(gx, gv, j, pre);
        const uint64_t k = key_of(x);
        const int bin = big_bin(k, kmin, span, scale);
        if (bin >= blo && bin < bhi) {
          const unsigned slot = atomicAdd(&S.load_cnt, 1u);
          if (slot < (unsigned)CAP) {
            S.x[slot] = x;
            S.v[slot] = gv[j];
            S.m[slot] = gm[j];
            S.idx[slot] = gi[j];
            cmin = k < cmin ? k : cmin;
            cmax = k > cmax ? k : cmax;
          }
        }
      }
      block_range(S, cmin, cmax);
      const int nc = (int)S.load_cnt;
      if (nc > CAP) {  // cannot happen with the chunk rule; never write past the arrays
        if (tid == 0) atomicOr(L.err, DEV_ERR_BAD_STATE);
        break;
      }
      if (nc == 0) continue;
      process_bucket<LAST, EXPR, false>(L, S, D, bt.bucket, bt.lay, nc, sub, ep, cmin, cmax,
                                        BucketTask{0, 0});
    }
  }
}

// Compact sorted state -> bucket layout with exactly T sheets per bucket,
// the splitters Q_b = (key, idx) of the sheet at rank b*T, and the buckets'
// aggregates in slot 0 (slots 1 and 2 cleared).  One block per bucket.
__global__ void k_bucketize(const StateTable* table, int64_t n, int target, int64_t nb, int capg,
                            int E,
                            double* x, double* v, double* m, int32_t* idx, unsigned* cnt0,
                            unsigned* cnt1, unsigned* cnt2, unsigned long long* mass0,
                            unsigned long long* mass1, unsigned long long* mass2, uint64_t* qk,
                            int32_t* qi) {
  __shared__ u128 s_mass[32];
  const StateRef st = table->cur;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t b = blockIdx.x; b < nb; b += gridDim.x) {
    const int64_t r0 = b * target;
    const int c = (int)((n - r0) < target ? (n - r0) : target);
    u128 msum = 0;
    for (int j = threadIdx.x; j < c; j += blockDim.x) {
      const int64_t o = b * capg + j;
      const double mj = st.m[r0 + j];
      x[o] = st.x[r0 + j];
      v[o] = st.v[r0 + j];
      m[o] = mj;
      idx[o] = st.idx[r0 + j];
      msum += mass_to_fixed(mj, E);
    }
    msum = warp_sum_u128(msum);
    if (lane == 0) s_mass[warp] = msum;
    __syncthreads();
    if (warp == 0) {
      const u128 t = warp_sum_u128(lane < (int)(blockDim.x >> 5) ? s_mass[lane] : (u128)0);
      if (lane < 4) {
        mass0[4 * b + lane] = (uint32_t)(t >> (32 * lane));
        mass1[4 * b + lane] = 0ull;
        mass2[4 * b + lane] = 0ull;
      }
      if (lane == 0) {
        cnt0[b] = (unsigned)c;
        cnt1[b] = 0u;
        cnt2[b] = 0u;
        if (b > 0) {
          qk[b] = key_of(st.x[r0]);
          qi[b] = st.idx[r0];
        }
      }
    }
    __syncthreads();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    qk[0] = 0ull;
    qi[0] = (int32_t)0x80000000;
    qk[nb] = ~0ull;
    qi[nb] = 0x7fffffff;
  }
}

// Bucket layout (+ overflow list) -> compact arrays in table->cur, unsorted.
__global__ void k_compact(StateTable* table, int64_t nb, int capg, const double* x, const double* v,
                          const double* m, const int32_t* idx, const unsigned* cnt,
                          const unsigned* offs, const double* ox, const double* ov,
                          const double* om, const int32_t* oi, const unsigned* ocount,
                          int64_t n) {
  const StateRef st = table->cur;
  for (int64_t b = blockIdx.x; b < nb; b += gridDim.x) {
    const unsigned c = cnt[b] < (unsigned)capg ? cnt[b] : (unsigned)capg;
    const int64_t o = offs[b];
    for (unsigned j = threadIdx.x; j < c && o + j < n; j += blockDim.x) {
      const int64_t s = b * capg + j;
      st.x[o + j] = x[s];
      st.v[o + j] = v[s];
      st.m[o + j] = m[s];
      st.idx[o + j] = idx[s];
    }
  }
  const unsigned no = *ocount < (unsigned)n ? *ocount : (unsigned)n;
  const int64_t obase = n - no;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < no; k += stride) {
    st.x[obase + k] = ox[k];
    st.v[obase + k] = ov[k];
    st.m[obase + k] = om[k];
    st.idx[obase + k] = oi[k];
  }
}

// Exclusive scan of the clamped bucket counts (single block, any nb).
__global__ void k_count_offsets(const unsigned* cnt, int64_t nb, int capg, unsigned* offs) {
  __shared__ unsigned s_carry;
  __shared__ unsigned s_w[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < nb; base += blockDim.x) {
    const int64_t b = base + tid;
    const unsigned c = b < nb ? (cnt[b] < (unsigned)capg ? cnt[b] : (unsigned)capg) : 0u;
    unsigned incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    unsigned wpre = 0;
    for (int w = 0; w < warp; ++w) wpre += s_w[w];
    if (b < nb) offs[b] = s_carry + wpre + incl - c;
    __syncthreads();
    if (tid == (int)blockDim.x - 1) s_carry += wpre + incl;
    __syncthreads();
  }
}

}  // namespace

int bucket_step_grid(int sm_count) { return 2 * sm_count; }

namespace {
std::mutex g_tune_mu;
std::vector<std::pair<int64_t, BucketTuning>> g_tune;  // rows sorted by n_min
}  // namespace

BucketTuning tuning_for(int64_t n) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  BucketTuning t;
  for (const auto& row : g_tune)
    if (row.first <= n) t = row.second;
  return t;
}

void set_tuning(const std::vector<std::pair<int64_t, BucketTuning>>& rows) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune = rows;
}

// The sub-step kernel's dynamic shared-memory limit, raised once per device
// (function attributes belong to the device they were set on).
void bucket_attr_init() {
  cudaFuncSetAttribute(k_bucket_step<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(StepSmem));
  cudaFuncSetAttribute(k_bucket_step<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(StepSmem));
  cudaFuncSetAttribute(k_bucket_step<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(StepSmem));
  cudaFuncSetAttribute(k_bucket_step<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(StepSmem));
  cudaFuncSetAttribute(k_bucket_big<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(StepSmem));
  cudaFuncSetAttribute(k_bucket_big<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(StepSmem));
  cudaFuncSetAttribute(k_bucket_big<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(StepSmem));
  cudaFuncSetAttribute(k_bucket_big<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(StepSmem));
}

void bucket_step_prepare() {
  static std::once_flag once[kMaxDevices];
  const int dev = current_device();
  if (dev < 0 || dev >= kMaxDevices)
    bucket_attr_init();
  else
    std::call_once(once[dev], bucket_attr_init);
}

__global__ void __launch_bounds__(256) k_split_out(const OutRec* __restrict__ rec, int64_t n,
                                                   double* __restrict__ x_out,
                                                   double* __restrict__ v_out,
                                                   double* __restrict__ a_out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const double2* r2 = reinterpret_cast<const double2*>(rec + i);
    const double2 xv = __ldcs(r2);
    x_out[i] = xv.x;
    v_out[i] = xv.y;
    if (a_out) a_out[i] = __ldcs(r2 + 1).x;
  }
}

void launch_split_out(const OutRec* rec, int64_t n, double* x_out, double* v_out, double* a_out,
                      cudaStream_t s) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  if (g < 1) g = 1;
  k_split_out<<<(unsigned)g, 256, 0, s>>>(rec, n, x_out, v_out, a_out);
}

void launch_bucket_step(const StepLaunch& a, int grid, cudaStream_t s) {
  bucket_step_prepare();
  if (grid > a.ntasks) grid = a.ntasks;
  if (grid < 1) grid = 1;
  const bool last = a.sub == a.nleap - 1;
  if (a.any_expr) {
    if (last)
      k_bucket_step<true, true><<<grid, BT, sizeof(StepSmem), s>>>(a);
    else
      k_bucket_step<false, true><<<grid, BT, sizeof(StepSmem), s>>>(a);
  } else if (last) {
    k_bucket_step<true, false><<<grid, BT, sizeof(StepSmem), s>>>(a);
  } else {
    k_bucket_step<false, false><<<grid, BT, sizeof(StepSmem), s>>>(a);
  }
}

__global__ void __launch_bounds__(256) k_member_splitters(const SimDev* devs, const int* list,
                                                          int sub) {
  __shared__ uint64_t sk[kMemberSampleCap];
  __shared__ int32_t si[kMemberSampleCap];
  const SimDev& d = devs[list ? list[blockIdx.x] : (int)blockIdx.x];
  StateTable* const pt = d.ptab;
  if (!pt) return;
  const int64_t m64 = d.nb - 1;
  if (m64 < 1 || m64 > kMemberSampleCap) return;
  const int m = (int)m64;
  int P = 1;
  while (P < m) P <<= 1;
  const StateRef c = pt->cur;
  for (int j = threadIdx.x; j < P; j += blockDim.x) {
    sk[j] = j < m ? key_of(c.x[j]) : ~0ull;
    si[j] = j < m ? c.idx[j] : 0x7fffffff;
  }
  __syncthreads();
  // bitonic sort of (key, idx) pairs, ascending
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const bool up = (i & k) == 0;
          const bool gt = sk[i] > sk[l] || (sk[i] == sk[l] && si[i] > si[l]);
          if (gt == up) {
            const uint64_t tk = sk[i];
            sk[i] = sk[l];
            sk[l] = tk;
            const int32_t ti = si[i];
            si[i] = si[l];
            si[l] = ti;
          }
        }
      }
      __syncthreads();
    }
  }
  const int q = 1 - ((d.qsel0 + sub) & 1);
  uint64_t* const qk = d.qk[q];
  int32_t* const qi = d.qi[q];
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    qk[j + 1] = sk[j];
    qi[j + 1] = si[j];
  }
}

void launch_member_splitters(const SimDev* devs, const int* list, int count, int sub,
                             cudaStream_t s) {
  if (count > 0) k_member_splitters<<<(unsigned)count, 256, 0, s>>>(devs, list, sub);
}

__global__ void k_samples_to_splitters(const StateTable* table, int64_t m, uint64_t* qk,
                                       int32_t* qi) {
  const StateRef c = table->cur;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += stride) {
    qk[j + 1] = key_of(c.x[j]);
    qi[j + 1] = c.idx[j];
  }
}

// Exclusive scan of each batch member's clamped bucket counts (one block per
// member): offs[toff + b] = sheets of the member's buckets before b.
__global__ void k_batch_offsets(const SimDev* devs, const BatchSeg* segs, unsigned* offs) {
  __shared__ unsigned s_carry;
  __shared__ unsigned s_w[32];
  const BatchSeg g = segs[blockIdx.x];
  const SimDev& d = devs[g.k];
  const unsigned* cnt = d.bcnt[g.cslot];
  const int64_t nb = d.nb;
  const unsigned capg = (unsigned)d.capg;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < nb; base += blockDim.x) {
    const int64_t b = base + tid;
    const unsigned c = b < nb ? (cnt[b] < capg ? cnt[b] : capg) : 0u;
    unsigned incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    unsigned wpre = 0;
    for (int w = 0; w < warp; ++w) wpre += s_w[w];
    if (b < nb) offs[g.toff + b] = s_carry + wpre + incl - c;
    __syncthreads();
    if (tid == (int)blockDim.x - 1) s_carry += wpre + incl;
    __syncthreads();
  }
}

// One block per task: bucket b of batch member j into dst, or (b == nb) the
// member's overflow list after its buckets' sheets.
__global__ void k_batch_compact(const SimDev* devs, const BatchSeg* segs, const BucketTask* tasks,
                                StateRef dst, const unsigned* offs, int64_t total) {
  const BucketTask t = tasks[blockIdx.x];
  const BatchSeg g = segs[t.sim];
  const SimDev& d = devs[g.k];
  const int64_t b = t.bucket;
  if (b < d.nb) {
    const unsigned c0 = d.bcnt[g.cslot][b];
    const unsigned c = c0 < (unsigned)d.capg ? c0 : (unsigned)d.capg;
    const int64_t o = g.out + offs[g.toff + b];
    const int64_t base = b * d.capg;
    const double* x = d.bx[g.lay];
    const double* v = d.bv[g.lay];
    const double* m = d.bm[g.lay];
    const int32_t* idx = d.bi[g.lay];
    for (unsigned j = threadIdx.x; j < c && o + j < g.out + g.n && o + j < total;
         j += blockDim.x) {
      dst.x[o + j] = x[base + j];
      dst.v[o + j] = v[base + j];
      dst.m[o + j] = m[base + j];
      dst.idx[o + j] = idx[base + j];
    }
  } else {
    // the overflow list fills the member's last slots
    const unsigned no0 = d.ocount[0];
    const unsigned no = no0 < (unsigned)g.n ? no0 : (unsigned)g.n;
    const int64_t o = g.out + g.n - no;
    for (unsigned j = threadIdx.x; j < no && o + j < total; j += blockDim.x) {
      dst.x[o + j] = d.ox[j];
      dst.v[o + j] = d.ov[j];
      dst.m[o + j] = d.om[j];
      dst.idx[o + j] = d.oi[j];
    }
  }
}

void launch_batch_compact(const SimDev* devs, const BatchSeg* segs, int nseg,
                          const BucketTask* tasks, int64_t ntasks, StateRef dst, unsigned* offs,
                          int64_t total, cudaStream_t s) {
  if (nseg < 1 || ntasks < 1) return;
  k_batch_offsets<<<(unsigned)nseg, 1024, 0, s>>>(devs, segs, offs);
  k_batch_compact<<<(unsigned)ntasks, 256, 0, s>>>(devs, segs, tasks, dst, offs, total);
}

// One block per task: bucket b of batch member j from its sorted sheets into
// layout 0, its counts and fixed-point masses (slot 0; slots 1 and 2
// cleared) and splitter b (the first sheet's key and index).
__global__ void k_batch_bucketize(const SimDev* devs, const BatchSeg* segs,
                                  const BucketTask* tasks, StateRef src, int64_t total) {
  __shared__ u128 s_mass[32];
  const BucketTask t = tasks[blockIdx.x];
  const BatchSeg g = segs[t.sim];
  const SimDev& d = devs[g.k];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t b = t.bucket;
  const int64_t r0 = b * d.target;
  int c = (int)((g.n - r0) < d.target ? (g.n - r0) : d.target);
  if (g.out + r0 + c > total) c = (int)(total - g.out - r0 > 0 ? total - g.out - r0 : 0);
  u128 msum = 0;
  for (int j = threadIdx.x; j < c; j += blockDim.x) {
    const int64_t o = b * d.capg + j;
    const int64_t q = g.out + r0 + j;
    const double mj = src.m[q];
    d.bx[0][o] = src.x[q];
    d.bv[0][o] = src.v[q];
    d.bm[0][o] = mj;
    d.bi[0][o] = src.idx[q];
    msum += mass_to_fixed(mj, d.E);
  }
  msum = warp_sum_u128(msum);
  if (lane == 0) s_mass[warp] = msum;
  __syncthreads();
  if (warp == 0) {
    const u128 tm = warp_sum_u128(lane < (int)(blockDim.x >> 5) ? s_mass[lane] : (u128)0);
    if (lane < 4) {
      d.bmass[0][4 * b + lane] = (uint32_t)(tm >> (32 * lane));
      d.bmass[1][4 * b + lane] = 0ull;
      d.bmass[2][4 * b + lane] = 0ull;
    }
    if (lane == 0) {
      d.bcnt[0][b] = (unsigned)c;
      d.bcnt[1][b] = 0u;
      d.bcnt[2][b] = 0u;
      if (b > 0) {
        d.qk[0][b] = key_of(fma(g.pre, src.v[g.out + r0], src.x[g.out + r0]));
        d.qi[0][b] = src.idx[g.out + r0];
      } else {
        d.qk[0][0] = 0ull;
        d.qi[0][0] = (int32_t)0x80000000;
        d.qk[0][d.nb] = ~0ull;
        d.qi[0][d.nb] = 0x7fffffff;
      }
    }
  }
}

void launch_batch_bucketize(const SimDev* devs, const BatchSeg* segs, const BucketTask* tasks,
                            int64_t ntasks, StateRef src, int64_t total, cudaStream_t s) {
  if (ntasks > 0) k_batch_bucketize<<<(unsigned)ntasks, 256, 0, s>>>(devs, segs, tasks, src, total);
}

void launch_samples_to_splitters(const StateTable* table, int64_t m, uint64_t* qk, int32_t* qi,
                                 cudaStream_t s) {
  int64_t g = (m + 255) / 256;
  if (g > 1216) g = 1216;
  k_samples_to_splitters<<<(unsigned)(g < 1 ? 1 : g), 256, 0, s>>>(table, m, qk, qi);
}

void launch_bucket_big(const StepLaunch& a, int grid, cudaStream_t s) {
  bucket_step_prepare();
  if (grid < 1) grid = 1;
  const bool last = a.sub == a.nleap - 1;
  if (a.any_expr) {
    if (last)
      k_bucket_big<true, true><<<grid, BT, sizeof(StepSmem), s>>>(a);
    else
      k_bucket_big<false, true><<<grid, BT, sizeof(StepSmem), s>>>(a);
  } else if (last) {
    k_bucket_big<true, false><<<grid, BT, sizeof(StepSmem), s>>>(a);
  } else {
    k_bucket_big<false, false><<<grid, BT, sizeof(StepSmem), s>>>(a);
  }
}

void launch_bucketize(const StateTable* table, int64_t n, int target, int64_t nb, int capg, int E,
                      double* x, double* v, double* m, int32_t* idx,
                      unsigned* const cnt[kAggSlots], unsigned long long* const mass[kAggSlots],
                      uint64_t* qk, int32_t* qi, cudaStream_t s) {
  int64_t g = nb < 152 * 8 ? nb : 152 * 8;
  if (g < 1) g = 1;
  k_bucketize<<<(unsigned)g, 256, 0, s>>>(table, n, target, nb, capg, E, x, v, m, idx, cnt[0],
                                           cnt[1], cnt[2], mass[0], mass[1], mass[2], qk, qi);
}

void launch_compact(StateTable* table, int64_t nb, int capg, const double* x, const double* v,
                    const double* m, const int32_t* idx, const unsigned* cnt, unsigned* offs,
                    const double* ox, const double* ov, const double* om, const int32_t* oi,
                    const unsigned* ocount, int64_t n, cudaStream_t s) {
  k_count_offsets<<<1, 1024, 0, s>>>(cnt, nb, capg, offs);
  int64_t g = nb < 152 * 8 ? nb : 152 * 8;
  if (g < 1) g = 1;
  k_compact<<<(unsigned)g, 256, 0, s>>>(table, nb, capg, x, v, m, idx, cnt, offs, ox, ov, om,
                                         oi, ocount, n);
}

}  // namespace wg
