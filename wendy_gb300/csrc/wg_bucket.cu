// wg_bucket.cu -- the fused sub-step on bucketed state.
//
// Between sub-steps the sheets live in B buckets of fixed capacity; bucket b
// holds exactly the sheets whose (position key, index) lies in
// [Q_b, Q_{b+1}), in arbitrary order inside the bucket.  One kernel launch
// per sub-step then does, per bucket (one CTA, persistent over buckets):
//
//   load the bucket into shared memory (optionally applying the half drift
//     a call starts with)
//   sort it by (key, index) in shared memory: the bounded-window fix-up,
//     since a bucket only ever receives sheets from nearby buckets
//   exact fixed-point prefix sum of the masses plus a count prefix, with a
//     decoupled look-back across buckets (the count gives global ranks)
//   a = [ext(x,t) +] (totmass - 2 C - m [- omega^2 x]); kick; drift
//   publish new splitters: the keys at global ranks j*T (quantiles)
//   route every sheet to the bucket of the next layout that covers its new
//     key (splitters computed by the previous sub-step) and append it there
//
// so a sub-step reads and writes each sheet once (28 B in, 28 B out).  A
// bucket that would overflow its capacity, or a sheet that left the search
// window, is still placed (overflow list, global search) and the sub-step
// is flagged so that the host re-sorts from scratch; no sheet is ever lost.
//
// Reference: _nbody_force and leapfrog_leappq, wendy/wendy.c:324-384; the
// argsort at wendy/wendy.c:341-357 is what the bucket sort replaces.
#include <cstdint>

#include "wg_bucket.cuh"

namespace wg {

namespace {

constexpr int BT = kBucketThreads;  // 256
constexpr int CAP = kBucketCap;     // 2048
constexpr int ITEMS = CAP / BT;     // 8
constexpr int WARPS = BT / 32;
constexpr int RWIN = kSplitterWindow;  // splitters searched in shared memory on each side

struct SortSmem {
  uint32_t q[2][CAP];
  uint16_t p[2][CAP];
  uint32_t hist[WARPS][256];
};

struct StepSmem {
  double x[CAP];
  double v[CAP];
  double m[CAP];
  uint64_t key[CAP];
  int32_t idx[CAP];
  SortSmem sort;
  uint64_t wkey[2 * RWIN + 2];
  int32_t widx[2 * RWIN + 2];
  uint32_t dcount[2 * RWIN + 2];
  uint32_t dbase[2 * RWIN + 2];
  u128 warp_mass[WARPS];
  uint32_t warp_cnt[WARPS];
  u128 prefix_mass;
  uint32_t prefix_cnt;
  uint64_t red_min[WARPS], red_max[WARPS];
  unsigned bucket;
  int n;
  int win_lo, win_hi;
  int any_tie;
  int perm_buf;
  double amp;
  unsigned epoch;
  unsigned flags;
  unsigned long long maxv;
};

__device__ __forceinline__ bool pair_less(uint64_t k1, int32_t i1, uint64_t k2, int32_t i2) {
  return k1 < k2 || (k1 == k2 && i1 < i2);
}

// Sort the n <= CAP sheets of the bucket by (key, idx).  Keys are first
// mapped to 32-bit order-preserving offsets ((key - kmin) >> shift) and
// radix-sorted, stable, 8 bits per pass, only over the bits that differ;
// equal offsets are then ordered by the full (key, idx) pair.  Leaves the
// permutation (sorted position -> slot) in sort.p[*perm_buf].
__device__ void bucket_sort(StepSmem& S, int n, uint64_t kmin, uint64_t kmax) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t span = kmax - kmin;
  const int bits = span ? 64 - __clzll((long long)span) : 0;
  const int shift = bits > 32 ? bits - 32 : 0;
  const int passes = (bits - shift + 7) / 8;
  for (int j = tid; j < n; j += BT) {
    S.sort.q[0][j] = (uint32_t)((S.key[j] - kmin) >> shift);
    S.sort.p[0][j] = (uint16_t)j;
  }
  int cur = 0;
  __syncthreads();
  for (int pass = 0; pass < passes; ++pass) {
    const int ds = 8 * pass;
    for (int i = lane; i < 256; i += 32) S.sort.hist[warp][i] = 0;
    __syncwarp();
    uint32_t rank[ITEMS];
    unsigned dig[ITEMS];
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      const int j = warp * (32 * ITEMS) + i * 32 + lane;
      const bool ok = j < n;
      const unsigned d = ok ? ((S.sort.q[cur][j] >> ds) & 255u) : (256u + lane);
      dig[i] = d;
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      uint32_t old = 0;
      if (ok) {
        old = S.sort.hist[warp][d];
        rank[i] = old + __popc(peers & lanemask_lt());
      }
      __syncwarp();
      if (ok && lane == __ffs(peers) - 1) S.sort.hist[warp][d] = old + __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    {
      // thread tid owns digit tid: offsets of the warps inside the digit,
      // then an exclusive scan of the digit totals across threads
      uint32_t run = 0;
#pragma unroll
      for (int w = 0; w < WARPS; ++w) {
        const uint32_t c = S.sort.hist[w][tid];
        S.sort.hist[w][tid] = run;
        run += c;
      }
      uint32_t incl = run;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      __shared__ uint32_t s_wsum[WARPS];
      if (lane == 31) s_wsum[warp] = incl;
      __syncthreads();
      uint32_t base = incl - run;
      for (int w = 0; w < warp; ++w) base += s_wsum[w];
#pragma unroll
      for (int w = 0; w < WARPS; ++w) S.sort.hist[w][tid] += base;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      const int j = warp * (32 * ITEMS) + i * 32 + lane;
      if (j < n) {
        const uint32_t dst = S.sort.hist[warp][dig[i]] + rank[i];
        S.sort.q[1 - cur][dst] = S.sort.q[cur][j];
        S.sort.p[1 - cur][dst] = S.sort.p[cur][j];
      }
    }
    __syncthreads();
    cur = 1 - cur;
  }
  // equal 32-bit offsets: order by the full (key, idx)
  bool tie = false;
  for (int j = tid; j + 1 < n; j += BT)
    if (S.sort.q[cur][j] == S.sort.q[cur][j + 1]) tie = true;
  if (__syncthreads_or(tie)) {
    for (int j = tid; j + 1 < n; j += BT) {
      const uint32_t qj = S.sort.q[cur][j];
      if (qj != S.sort.q[cur][j + 1] || (j > 0 && S.sort.q[cur][j - 1] == qj)) continue;
      int e = j + 1;
      while (e + 1 < n && S.sort.q[cur][e + 1] == qj) ++e;
      uint16_t* p = S.sort.p[cur];
      for (int a = j + 1; a <= e; ++a) {
        const uint16_t s = p[a];
        const uint64_t ks = S.key[s];
        const int32_t is = S.idx[s];
        int b = a - 1;
        while (b >= j && pair_less(ks, is, S.key[p[b]], S.idx[p[b]])) {
          p[b + 1] = p[b];
          --b;
        }
        p[b + 1] = s;
      }
    }
    __syncthreads();
  }
  if (tid == 0) S.perm_buf = cur;
  __syncthreads();
}

// Look-back over earlier buckets of the same simulation for the exclusive
// (mass, count) prefix; all lanes of warp 0 call it.
__device__ void bucket_lookback(const BucketStepArgs& a, int64_t b, u128 mass, uint32_t cnt,
                                unsigned ep, int lane, u128& pmass, uint32_t& pcnt) {
  BucketRec* recs = a.recs;
  BucketRec* me = recs + b;
  pmass = 0;
  pcnt = 0;
  if (b == 0) {
    if (lane == 0) {
      me->inc_lo = (uint64_t)mass;
      me->inc_hi = (uint64_t)(mass >> 64);
      me->inc_cnt = cnt;
      st_release_u32(&me->flag, (ep << 2) | 2u);
    }
    return;
  }
  if (lane == 0) {
    me->agg_lo = (uint64_t)mass;
    me->agg_hi = (uint64_t)(mass >> 64);
    me->agg_cnt = cnt;
    st_release_u32(&me->flag, (ep << 2) | 1u);
  }
  int64_t j = b - 1;
  for (;;) {
    const int64_t jj = j - lane;
    unsigned status = 0;
    u128 vm = 0;
    uint32_t vc = 0;
    if (jj >= 0) {
      const BucketRec* r = recs + jj;
      unsigned f = 0, spins = 0;
      for (;;) {
        f = ld_acquire_u32(&r->flag);
        if ((f >> 2) == ep && (f & 3u)) break;
        if (++spins > kSpinLimit) {
          atomicOr(a.err, DEV_ERR_LOOKBACK_TIMEOUT);
          f = 0;
          break;
        }
        __nanosleep(32);
      }
      status = ((f >> 2) == ep) ? (f & 3u) : 0u;
      if (status == 2u) {
        vm = (((u128)ld_cg_u64(&r->inc_hi)) << 64) | ld_cg_u64(&r->inc_lo);
        vc = __ldcg(&r->inc_cnt);
      } else if (status == 1u) {
        vm = (((u128)ld_cg_u64(&r->agg_hi)) << 64) | ld_cg_u64(&r->agg_lo);
        vc = __ldcg(&r->agg_cnt);
      }
    }
    const unsigned pmask = __ballot_sync(0xffffffffu, status == 2u);
    const int stop = pmask ? (__ffs(pmask) - 1) : 31;
    const bool take = lane <= stop;
    pmass += warp_sum_u128(take ? vm : (u128)0);
    uint32_t c = take ? vc : 0u;
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) c += __shfl_xor_sync(0xffffffffu, c, d);
    pcnt += c;
    if (pmask || j - 32 < 0) break;
    j -= 32;
  }
  if (lane == 0) {
    const u128 im = pmass + mass;
    me->inc_lo = (uint64_t)im;
    me->inc_hi = (uint64_t)(im >> 64);
    me->inc_cnt = pcnt + cnt;
    st_release_u32(&me->flag, (ep << 2) | 2u);
  }
}

// Bucket of the next layout covering (k, i): the largest j with Q_j <= (k, i).
__device__ int dest_bucket(const BucketStepArgs& a, const StepSmem& S, uint64_t k, int32_t i,
                           bool& far) {
  // window [win_lo, win_hi] of splitter indices is in shared memory
  const int lo = S.win_lo, hi = S.win_hi;
  far = false;
  if (!pair_less(k, i, S.wkey[0], S.widx[0]) &&
      pair_less(k, i, S.wkey[hi - lo], S.widx[hi - lo])) {
    int l = 0, h = hi - lo;  // Q_{lo+l} <= (k,i) < Q_{lo+h}
    while (h - l > 1) {
      const int mid = (l + h) >> 1;
      if (pair_less(k, i, S.wkey[mid], S.widx[mid]))
        h = mid;
      else
        l = mid;
    }
    return lo + l;
  }
  far = true;
  int l = 0, h = (int)a.nb;  // Q_0 = -inf <= (k,i) < Q_nb = +inf
  while (h - l > 1) {
    const int mid = (l + h) >> 1;
    if (pair_less(k, i, __ldg(&a.q_dest_key[mid]), __ldg(&a.q_dest_idx[mid])))
      h = mid;
    else
      l = mid;
  }
  return l;
}

__global__ void __launch_bounds__(BT, 2) k_bucket_step(const BucketStepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  StepSmem& S = *reinterpret_cast<StepSmem*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  {
    const unsigned ab = *(volatile const unsigned*)a.abort;
    if (ab != 0 && (int)ab <= a.sub) return;  // an earlier sub-step of this call failed
  }
  if (tid == 0) {
    S.epoch = a.epochs[a.sub];
    S.amp = (a.ext.kind == EXT_PULSE_TANH) ? pulse_amplitude(a.ext, a.t_seq[a.sub]) : 0.0;
    S.maxv = 0;
    S.flags = 0;
  }
  const i128 T = (i128)((((u128)a.T_hi) << 64) | a.T_lo);
  for (;;) {
    __syncthreads();
    if (tid == 0) {
      S.bucket = atomicAdd(a.ticket, 1u);
      S.n = S.bucket < a.nb ? (int)a.cnt_in[S.bucket] : 0;
    }
    __syncthreads();
    const int64_t b = S.bucket;
    if (b >= a.nb) break;
    const int n = S.n < CAP ? S.n : CAP;
    const int64_t base = b * CAP;
    if (tid == 0) a.cnt_in[b] = 0;  // this count buffer is the target two sub-steps on
    // ---- load (applying the opening half drift of a call, if any)
    uint64_t kmin = ~0ull, kmax = 0;
    for (int j = tid; j < n; j += BT) {
      const double v = a.vin[base + j];
      double x = a.xin[base + j];
      if (a.pre_dt != 0.0) x = fma(a.pre_dt, v, x);
      const uint64_t k = key_of(x);
      S.x[j] = x;
      S.v[j] = v;
      S.m[j] = a.min[base + j];
      S.idx[j] = a.iin[base + j];
      S.key[j] = k;
      kmin = k < kmin ? k : kmin;
      kmax = k > kmax ? k : kmax;
    }
    // splitter window of the next layout around this bucket
    const int wlo = (int)(b > RWIN ? b - RWIN : 0);
    const int whi = (int)((b + RWIN + 1) < a.nb ? (b + RWIN + 1) : a.nb);
    for (int j = tid; j <= whi - wlo; j += BT) {
      S.wkey[j] = a.q_dest_key[wlo + j];
      S.widx[j] = a.q_dest_idx[wlo + j];
      S.dcount[j] = 0;
    }
    if (tid == 0) {
      S.win_lo = wlo;
      S.win_hi = whi;
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
    __syncthreads();
    kmin = ~0ull;
    kmax = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      kmin = S.red_min[w] < kmin ? S.red_min[w] : kmin;
      kmax = S.red_max[w] > kmax ? S.red_max[w] : kmax;
    }
    if (n > 1) {
      bucket_sort(S, n, kmin, kmax);
    } else {
      if (tid == 0) {
        S.sort.p[0][0] = 0;
        S.perm_buf = 0;
      }
      __syncthreads();
    }
    const uint16_t* perm = S.sort.p[S.perm_buf];

    // ---- exact prefix of the masses (blocked: ITEMS sorted positions per thread)
    const int j0 = tid * ITEMS;
    u128 cex[ITEMS];
    u128 run = 0;
    int nv = 0;
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      cex[i] = run;
      if (j0 + i < n) {
        run += mass_to_fixed(S.m[perm[j0 + i]], a.E);
        ++nv;
      }
    }
    const u128 tot = run;
    const u128 incl = warp_inclusive_scan_u128(tot, lane);
    uint32_t cin = (uint32_t)nv;
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
    if (warp == 0) {
      const u128 wm = lane < WARPS ? S.warp_mass[lane] : (u128)0;
      const uint32_t wc = lane < WARPS ? S.warp_cnt[lane] : 0u;
      const u128 wmi = warp_inclusive_scan_u128(wm, lane);
      uint32_t wci = wc;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, wci, o);
        if (lane >= o) wci += y;
      }
      const u128 bm = shfl_u128(wmi, WARPS - 1);
      const uint32_t bc = __shfl_sync(0xffffffffu, wci, WARPS - 1);
      if (lane < WARPS) {
        S.warp_mass[lane] = wmi - wm;
        S.warp_cnt[lane] = wci - wc;
      }
      u128 pm;
      uint32_t pc;
      bucket_lookback(a, b, bm, bc, S.epoch, lane, pm, pc);
      if (lane == 0) {
        S.prefix_mass = pm;
        S.prefix_cnt = pc;
      }
    }
    __syncthreads();
    const u128 tpm = S.prefix_mass + S.warp_mass[warp] + (incl - tot);
    const uint32_t rank0 = S.prefix_cnt + S.warp_cnt[warp] + (cin - (uint32_t)nv);

    // ---- splitters of the layout after next: keys at global ranks j*T
    if (b == 0 && tid == 0) {
      a.q_new_key[0] = 0ull;
      a.q_new_idx[0] = (int32_t)0x80000000;
      a.q_new_key[a.nb] = ~0ull;
      a.q_new_idx[a.nb] = 0x7fffffff;
    }
    // ---- force, kick, drift, routing
    unsigned long long maxv = 0;
    double xr[ITEMS], vr[ITEMS];
    int dst[ITEMS];
    uint32_t drank[ITEMS];
    bool dfar[ITEMS];
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      dst[i] = -1;
      if (j0 + i >= n) continue;
      const int s = perm[j0 + i];
      const uint32_t r = rank0 + (uint32_t)i;
      if (r != 0 && (r % (uint32_t)a.target) == 0) {
        a.q_new_key[r / a.target] = S.key[s];
        a.q_new_idx[r / a.target] = S.idx[s];
      }
      const double x = S.x[s], v = S.v[s];
      const u128 M = (i + 1 < ITEMS ? cex[i + 1] : tot) - cex[i];
      const i128 C = (i128)(tpm + cex[i]);
      const i128 A = T - 2 * C - (i128)M;
      double acc = fixed_to_double(A, a.E);
      if (a.has_omega) acc = fma(-a.omega2, x, acc);
      if (a.ext.kind != EXT_NONE) acc = ext_force_at(a.ext, S.amp, x) + acc;
      const double vn = fma(a.dt_kick, acc, v);
      const double xn = fma(a.dt_drift, vn, x);
      xr[i] = xn;
      vr[i] = vn;
      const unsigned long long av =
          (unsigned long long)__double_as_longlong(vn) & 0x7FFFFFFFFFFFFFFFull;
      maxv = av > maxv ? av : maxv;
      if (a.x_orig) {
        a.x_orig[S.idx[s]] = xn;
        a.v_orig[S.idx[s]] = vn;
      }
      const double xd = a.dest_dt != 0.0 ? fma(a.dest_dt, vn, xn) : xn;
      bool far;
      const int d = dest_bucket(a, S, key_of(xd), S.idx[s], far);
      dst[i] = d;
      dfar[i] = far;
      if (!far) drank[i] = atomicAdd(&S.dcount[d - S.win_lo], 1u);
    }
    __syncthreads();
    for (int j = tid; j <= S.win_hi - S.win_lo; j += BT) {
      const uint32_t c = S.dcount[j];
      S.dbase[j] = c ? atomicAdd(&a.cnt_out[S.win_lo + j], c) : 0u;
    }
    __syncthreads();
    unsigned fl = 0;
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      if (dst[i] < 0) continue;
      const int s = perm[j0 + i];
      const int d = dst[i];
      uint32_t slot;
      if (dfar[i]) {
        slot = atomicAdd(&a.cnt_out[d], 1u);
        fl |= 1u;
      } else {
        slot = S.dbase[d - S.win_lo] + drank[i];
      }
      if (slot < (uint32_t)CAP) {
        const int64_t o = (int64_t)d * CAP + slot;
        a.xout[o] = xr[i];
        a.vout[o] = vr[i];
        a.mout[o] = S.m[s];
        a.iout[o] = S.idx[s];
      } else {
        const uint32_t o = atomicAdd(a.ocount, 1u);
        a.ox[o] = xr[i];
        a.ov[o] = vr[i];
        a.om[o] = S.m[s];
        a.oi[o] = S.idx[s];
        fl |= 2u;
      }
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
      const unsigned long long o = __shfl_xor_sync(0xffffffffu, maxv, d);
      maxv = o > maxv ? o : maxv;
    }
    if (lane == 0 && maxv) atomicMax(&S.maxv, maxv);
    if (fl) atomicOr(&S.flags, fl);
  }
  __syncthreads();
  if (tid == 0) {
    if (S.maxv) atomicMax(&a.flag_out->max_v, S.maxv);
    if (S.flags & 1u) atomicAdd(&a.flag_out->pad, 1u);  // sheets found by the global search
    if (S.flags & 2u) atomicCAS(a.abort, 0u, (unsigned)(a.sub + 1));  // overflow: re-sort
  }
}

// Compact sorted state -> bucket layout with exactly T sheets per bucket and
// the splitters Q_b = (key, idx) of the sheet at rank b*T.
__global__ void k_bucketize(const StateTable* table, int64_t n, int target, int64_t nb,
                            double* x, double* v, double* m, int32_t* idx, unsigned* cnt,
                            uint64_t* qk, int32_t* qi, unsigned* cnt_other) {
  const StateRef st = table->cur;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += stride) {
    const int64_t b = r / target, j = r - b * target;
    const int64_t o = b * CAP + j;
    x[o] = st.x[r];
    v[o] = st.v[r];
    m[o] = st.m[r];
    idx[o] = st.idx[r];
    if (j == 0) {
      cnt[b] = (unsigned)((n - r) < target ? (n - r) : target);
      cnt_other[b] = 0;
      if (b > 0) {
        qk[b] = key_of(st.x[r]);
        qi[b] = st.idx[r];
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    qk[0] = 0ull;
    qi[0] = (int32_t)0x80000000;
    qk[nb] = ~0ull;
    qi[nb] = 0x7fffffff;
  }
}

// Bucket layout (+ overflow list) -> compact arrays in table->cur, unsorted.
__global__ void k_compact(StateTable* table, int64_t nb, const double* x, const double* v,
                          const double* m, const int32_t* idx, const unsigned* cnt,
                          const unsigned* offs, const double* ox, const double* ov,
                          const double* om, const int32_t* oi, const unsigned* ocount,
                          int64_t n) {
  const StateRef st = table->cur;
  for (int64_t b = blockIdx.x; b < nb; b += gridDim.x) {
    const unsigned c = cnt[b] < (unsigned)CAP ? cnt[b] : (unsigned)CAP;
    const int64_t o = offs[b];
    for (unsigned j = threadIdx.x; j < c && o + j < n; j += blockDim.x) {
      const int64_t s = b * CAP + j;
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
__global__ void k_count_offsets(const unsigned* cnt, int64_t nb, unsigned* offs) {
  __shared__ unsigned s_carry;
  __shared__ unsigned s_w[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < nb; base += blockDim.x) {
    const int64_t b = base + tid;
    const unsigned c = b < nb ? (cnt[b] < (unsigned)CAP ? cnt[b] : (unsigned)CAP) : 0u;
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

size_t bucket_step_smem() { return sizeof(StepSmem); }

void launch_bucket_step(const BucketStepArgs& a, int grid, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_bucket_step, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(StepSmem));
    attr = true;
  }
  k_bucket_step<<<grid, BT, sizeof(StepSmem), s>>>(a);
}

void launch_bucketize(const StateTable* table, int64_t n, int target, int64_t nb, double* x,
                      double* v, double* m, int32_t* idx, unsigned* cnt, uint64_t* qk,
                      int32_t* qi, unsigned* cnt_other, cudaStream_t s) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  k_bucketize<<<(unsigned)g, 256, 0, s>>>(table, n, target, nb, x, v, m, idx, cnt, qk, qi,
                                           cnt_other);
}

void launch_compact(StateTable* table, int64_t nb, const double* x, const double* v,
                    const double* m, const int32_t* idx, const unsigned* cnt, unsigned* offs,
                    const double* ox, const double* ov, const double* om, const int32_t* oi,
                    const unsigned* ocount, int64_t n, cudaStream_t s) {
  k_count_offsets<<<1, 1024, 0, s>>>(cnt, nb, offs);
  int64_t g = nb < 152 * 8 ? nb : 152 * 8;
  if (g < 1) g = 1;
  k_compact<<<(unsigned)g, 256, 0, s>>>(table, nb, x, v, m, idx, cnt, offs, ox, ov, om, oi,
                                         ocount, n);
}

}  // namespace wg
