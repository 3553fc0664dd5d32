// wg_pool.cu -- many simulations resident on one GPU, advanced together.
//
// A pool owns any number of simulations (each with its own bucket layouts,
// look-back records and splitters, allocated with the stream-ordered
// allocator) and one shared workspace (compact sheet sets, radix-sort
// buffers) sized for the largest of them.  wg_pool_step advances any subset
// of the simulations by one output interval with ONE launch of the fused
// bucket kernel per leapfrog sub-step: the launch walks the concatenated
// bucket lists of all chosen simulations, and every look-back, sort and
// splitter stays inside its own simulation, so each result is bit-identical
// to the same simulation run alone.  Simulations can be added and removed
// between steps, which is what continuous batching needs.
//
// Per simulation the arithmetic is that of wendy's approximate step
// (wendy/wendy.c:385-418); the reference has no ensemble API.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <unordered_set>
#include <vector>

#include "../../include/wendy_gb300.h"
#include "wg_bucket.cuh"
#include "wg_ext.cuh"
#include "wg_internal.cuh"

using namespace wg;

namespace {

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

int pool_fail(int code, const char* fmt, ...) {
  char msg[320];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  record_last_error(msg);
  return code;
}

#define PC(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return pool_fail(e_ == cudaErrorMemoryAllocation ? WG_ERR_NOMEM : WG_ERR_CUDA,    \
                       "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                       __LINE__);                                                       \
  } while (0)

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

// Persistent device memory of one simulation, in one allocation.
struct PoolSim {
  int64_t n = 0, nb = 0;
  void* mem = nullptr;
  size_t bytes = 0;
  double* bx[2];
  double* bv[2];
  double* bm[2];
  int32_t* bi[2];
  unsigned* bcnt[kAggSlots];
  unsigned long long* bmass[kAggSlots];
  uint64_t* qk[2];
  int32_t* qi[2];
  BucketRec* recs;
  double *ox, *ov, *om;  // overflow list; also the compact (unsorted) store in mode 0
  int32_t* oi;
  double *x_out, *v_out;     // output of the last step (during a step: being written)
  double *x_out2, *v_out2;   // the other pair; steps alternate between them
  double *done_x = nullptr, *done_v = nullptr;  // during a step: the output before it
  uint64_t T_lo = 0, T_hi = 0;
  int E = 0;
  double totmass = 0, omega2 = -1;
  ExtForce ext{};
  ExtSpec ext_spec{};         // the force with an expression's program on the host
  ExprOp* d_prog = nullptr;   // an expression force's program on the device
  int mode = 0;  // 0: sheets compact in ox..oi, half drift pending; 1: bucket layout
  int lay = 0, qsel = 0;
  int cslot = 0;  // aggregate slot describing layout `lay`
  double pending_dt = 0;
  bool fresh = false;      // just bucketized: the opening half drift is already applied
  bool out_valid = false;  // x_out / v_out hold the last output
  BucketTuning tune;
  // predicted splitters (members of at most kMaxMemberSamples + 1 buckets):
  // the sample set the sub-steps write (a StateTable whose current set holds
  // x and idx only) and the calls they are still on for
  StateTable* ptab = nullptr;
  int pred_calls = 0;
};

// A member's samples are sorted by one CTA in shared memory.
constexpr int kPredMemberCalls = 16;

size_t sim_bytes(int64_t n) {
  const BucketTuning t = tuning_for(n);
  const int64_t nb = (n + t.target - 1) / t.target;
  const size_t slots = (size_t)nb * kBucketCap;
  const size_t pred = (nb >= 3 && nb - 1 <= kMemberSampleCap)
                          ? al(sizeof(StateTable)) + al(8 * (size_t)nb) + al(4 * (size_t)nb)
                          : 0;
  return pred + 2 * (3 * al(slots * 8) + al(slots * 4)) +
         kAggSlots * (al(4 * (size_t)nb) + al(32 * (size_t)nb)) +
         2 * (al(8 * (size_t)(nb + 1)) + al(4 * (size_t)(nb + 1))) +
         al(sizeof(BucketRec) * (size_t)nb) + 3 * al(8 * (size_t)n) + al(4 * (size_t)n) +
         4 * al(8 * (size_t)n);
}

void carve(PoolSim* s) {
  const size_t slots = (size_t)s->nb * kBucketCap;
  char* p = static_cast<char*>(s->mem);
  for (int k = 0; k < 2; ++k) {
    s->bx[k] = reinterpret_cast<double*>(p); p += al(slots * 8);
    s->bv[k] = reinterpret_cast<double*>(p); p += al(slots * 8);
    s->bm[k] = reinterpret_cast<double*>(p); p += al(slots * 8);
    s->bi[k] = reinterpret_cast<int32_t*>(p); p += al(slots * 4);
  }
  for (int k = 0; k < kAggSlots; ++k) {
    s->bcnt[k] = reinterpret_cast<unsigned*>(p); p += al(4 * (size_t)s->nb);
    s->bmass[k] = reinterpret_cast<unsigned long long*>(p); p += al(32 * (size_t)s->nb);
  }
  for (int k = 0; k < 2; ++k) {
    s->qk[k] = reinterpret_cast<uint64_t*>(p); p += al(8 * (size_t)(s->nb + 1));
    s->qi[k] = reinterpret_cast<int32_t*>(p); p += al(4 * (size_t)(s->nb + 1));
  }
  s->recs = reinterpret_cast<BucketRec*>(p); p += al(sizeof(BucketRec) * (size_t)s->nb);
  s->ox = reinterpret_cast<double*>(p); p += al(8 * (size_t)s->n);
  s->ov = reinterpret_cast<double*>(p); p += al(8 * (size_t)s->n);
  s->om = reinterpret_cast<double*>(p); p += al(8 * (size_t)s->n);
  s->oi = reinterpret_cast<int32_t*>(p); p += al(4 * (size_t)s->n);
  s->x_out = reinterpret_cast<double*>(p); p += al(8 * (size_t)s->n);
  s->v_out = reinterpret_cast<double*>(p); p += al(8 * (size_t)s->n);
  s->x_out2 = reinterpret_cast<double*>(p); p += al(8 * (size_t)s->n);
  s->v_out2 = reinterpret_cast<double*>(p); p += al(8 * (size_t)s->n);
  s->ptab = nullptr;
  if (s->nb >= 3 && s->nb - 1 <= kMemberSampleCap) {
    s->ptab = reinterpret_cast<StateTable*>(p); p += al(sizeof(StateTable));
  }
}

// The sample set of a member with predicted splitters: x and idx of nb - 1
// samples right after the table (carve leaves the room).
StateTable member_sample_table(const PoolSim* s) {
  char* p = reinterpret_cast<char*>(s->ptab) + al(sizeof(StateTable));
  StateTable t{};
  t.cur.x = reinterpret_cast<double*>(p);
  t.cur.idx = reinterpret_cast<int32_t*>(p + al(8 * (size_t)s->nb));
  t.other = t.cur;
  return t;
}

__global__ void k_set_table(StateTable* t, StateRef cur, StateRef other) {
  t->cur = cur;
  t->other = other;
}

__global__ void k_iota_i32(int32_t* p, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    p[i] = (int32_t)i;
}

// Copy the current compact set into a simulation's compact store.
__global__ void k_store_compact(const StateTable* t, int64_t n, double* x, double* v,
                                double* m, int32_t* idx) {
  const StateRef c = t->cur;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    x[i] = c.x[i];
    v[i] = c.v[i];
    m[i] = c.m[i];
    idx[i] = c.idx[i];
  }
}

}  // namespace

struct wg_pool {
  cudaStream_t stream = nullptr;
  // a step's device time: ev0 -> ev_mid (the graph) plus ev_rec -> ev1 (the
  // recovery, which waits for the host's second half)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_mid = nullptr, ev_rec = nullptr;
  int sms = 152;
  int64_t budget = 0;  // bytes, 0 = no limit
  int64_t used = 0;
  std::vector<PoolSim*> sims;
  // shared workspace for the compact path, sized for ws_n sheets
  int64_t ws_n = 0;
  void* ws = nullptr;
  StateRef set[2];
  TileRec* trecs = nullptr;
  RadixWork radix;
  // Batch workspace: members restarted together are compacted into bW, sorted
  // by (member, key, index) with two radix sorts (sets bA, bB) and gathered
  // into bO, from which their fresh layouts are filled.
  void* bws = nullptr;
  int64_t bws_n = 0, bws_tasks = 0, bws_segs = 0;
  StateRef bW, bA[2], bB[2], bO;
  StateTable* btA = nullptr;
  StateTable* btB = nullptr;
  StepFlags* bflag = nullptr;
  RadixWork bradix{};
  unsigned* boffs = nullptr;
  BatchSeg* bsegs = nullptr;
  int64_t* bseg_out = nullptr;
  BucketTask* btasks = nullptr;
  // host staging of a chunk's tables: pageable, so each upload has copied
  // them out before it returns and the next chunk may refill them at once
  // (a page-locked buffer would be read when the copy runs, after the refill)
  std::vector<BatchSeg> h_bsegs;
  std::vector<int64_t> h_bseg_out;
  std::vector<BucketTask> h_btasks;
  unsigned* offs = nullptr;
  // small per-call arrays (device) and their pinned mirrors
  void* small = nullptr;
  int cap_sims = 0, cap_leap = 0;
  int64_t cap_tasks = 0;
  StateTable* table = nullptr;
  unsigned* err = nullptr;
  StepFlags* wflags = nullptr;    // [cap_leap + 1] for the compact path
  unsigned* tickets = nullptr;    // [cap_leap]
  unsigned* epochs = nullptr;     // [cap_leap]
  SimDev* d_dev = nullptr;        // [cap_sims]
  StepFlags* flags = nullptr;     // [cap_sims * (cap_leap + 1)]
  double* t_seq = nullptr;        // [cap_sims * cap_leap]
  unsigned* ocount = nullptr;     // [cap_sims * 2]
  BucketTask* tasks = nullptr;    // [cap_tasks]
  SimDev* h_dev = nullptr;
  double* h_t = nullptr;
  unsigned* h_ep = nullptr;
  unsigned* h_oc = nullptr;
  unsigned* d_oc = nullptr;        // h_oc as the device addresses it (mapped page-locked memory)
  BucketTask* rtasks = nullptr;    // [cap_tasks] tasks of the simulations restarted together
  int* rlist = nullptr;            // [cap_sims] their indices in this call
  BucketTask* h_rtasks = nullptr;
  int* h_rlist = nullptr;
  BucketTask* h_tasks = nullptr;
  unsigned epoch = 1;
  int64_t launches = 0;
  // the per-call device sequence (copies in, nleap sub-step launches, copy
  // back) captured once per (simulations, buckets, nleap) and replayed
  cudaGraphExec_t gexec = nullptr;
  int g_count = -1, g_nleap = -1;
  // a step begun (wg_pool_step_begin) and not yet completed
  bool pend_active = false;
  int pend_count = 0, pend_nleap = 0;
  std::vector<PoolSim*> pend_act;
  std::vector<double> pend_dt;
  cudaStream_t dl_stream = nullptr;  // downloads while a step runs
  int64_t g_ntasks = -1;
  void* g_small = nullptr;
  bool g_expr = false;   // the graph launches the expression-force instantiation
  int64_t graph_builds = 0;
  wg_pool_stats stats{};  // counters (launches and graph_builds are filled on read)
};

namespace {

void free_small(wg_pool* p) {
  if (p->small) cudaFree(p->small);
  if (p->h_dev) cudaFreeHost(p->h_dev);
  if (p->h_t) cudaFreeHost(p->h_t);
  if (p->h_ep) cudaFreeHost(p->h_ep);
  if (p->h_oc) cudaFreeHost(p->h_oc);
  if (p->h_tasks) cudaFreeHost(p->h_tasks);
  if (p->h_rtasks) cudaFreeHost(p->h_rtasks);
  if (p->h_rlist) cudaFreeHost(p->h_rlist);
  p->h_rtasks = nullptr;
  p->h_rlist = nullptr;
  p->small = nullptr;
  p->h_dev = nullptr;
  p->h_t = nullptr;
  p->h_ep = nullptr;
  p->h_oc = nullptr;
  p->d_oc = nullptr;
  p->h_tasks = nullptr;
}

int ensure_small(wg_pool* p, int nsims, int nleap, int64_t ntasks) {
  if (nsims <= p->cap_sims && nleap <= p->cap_leap && ntasks <= p->cap_tasks && p->small)
    return WG_OK;
  PC(cudaStreamSynchronize(p->stream));
  int cs = p->cap_sims > 16 ? p->cap_sims : 16, cl = p->cap_leap > 64 ? p->cap_leap : 64;
  int64_t ct = p->cap_tasks > 1024 ? p->cap_tasks : 1024;
  while (cs < nsims) cs *= 2;
  while (cl < nleap) cl *= 2;
  while (ct < ntasks) ct *= 2;
  free_small(p);
  const size_t b = al(sizeof(StateTable)) + al(64) + al(sizeof(StepFlags) * (cl + 1)) +
                   2 * al(4 * (size_t)cl) + al(sizeof(SimDev) * (size_t)cs) +
                   al(sizeof(StepFlags) * (size_t)cs * (cl + 1)) + al(8 * (size_t)cs * cl) +
                   al(8 * (size_t)cs) + al(sizeof(BucketTask) * (size_t)ct) +
                   al(sizeof(BucketTask) * (size_t)ct) + al(4 * (size_t)cs);
  PC(cudaMalloc(&p->small, b));
  char* q = static_cast<char*>(p->small);
  p->table = reinterpret_cast<StateTable*>(q); q += al(sizeof(StateTable));
  p->err = reinterpret_cast<unsigned*>(q); q += al(64);
  p->wflags = reinterpret_cast<StepFlags*>(q); q += al(sizeof(StepFlags) * (cl + 1));
  p->tickets = reinterpret_cast<unsigned*>(q); q += al(4 * (size_t)cl);
  p->epochs = reinterpret_cast<unsigned*>(q); q += al(4 * (size_t)cl);
  p->d_dev = reinterpret_cast<SimDev*>(q); q += al(sizeof(SimDev) * (size_t)cs);
  p->flags = reinterpret_cast<StepFlags*>(q); q += al(sizeof(StepFlags) * (size_t)cs * (cl + 1));
  p->t_seq = reinterpret_cast<double*>(q); q += al(8 * (size_t)cs * cl);
  p->ocount = reinterpret_cast<unsigned*>(q); q += al(8 * (size_t)cs);
  p->tasks = reinterpret_cast<BucketTask*>(q); q += al(sizeof(BucketTask) * (size_t)ct);
  p->rtasks = reinterpret_cast<BucketTask*>(q); q += al(sizeof(BucketTask) * (size_t)ct);
  p->rlist = reinterpret_cast<int*>(q); q += al(4 * (size_t)cs);
  PC(cudaMemsetAsync(p->small, 0, b, p->stream));
  PC(cudaMallocHost(&p->h_dev, sizeof(SimDev) * (size_t)cs));
  PC(cudaMallocHost(&p->h_t, 8 * (size_t)cs * cl));
  PC(cudaMallocHost(&p->h_ep, 4 * (size_t)cl));
  PC(cudaMallocHost(&p->h_oc, 8 * (size_t)cs));
  PC(cudaHostGetDevicePointer(reinterpret_cast<void**>(&p->d_oc), p->h_oc, 0));
  PC(cudaMallocHost(&p->h_tasks, sizeof(BucketTask) * (size_t)ct));
  PC(cudaMallocHost(&p->h_rtasks, sizeof(BucketTask) * (size_t)ct));
  PC(cudaMallocHost(&p->h_rlist, 4 * (size_t)cs));
  p->cap_sims = cs;
  p->cap_leap = cl;
  p->cap_tasks = ct;
  return WG_OK;
}

// Smallest power of two >= v (v >= 1).
static int64_t pow2_at_least(int64_t v) {
  int64_t r = 1;
  while (r < v) r <<= 1;
  return r;
}

int ensure_workspace(wg_pool* p, int64_t n) {
  if (n <= p->ws_n && p->ws) return WG_OK;
  n = pow2_at_least(n);  // fewer re-allocations (each waits for the device)
  PC(cudaStreamSynchronize(p->stream));
  if (p->ws) cudaFree(p->ws);
  p->ws = nullptr;
  const size_t nd = al((size_t)n * 8), ni = al((size_t)n * 4);
  const int64_t tiles = (n + kForceTile - 1) / kForceTile;
  const int64_t nb = n;  // compaction offsets: at most one bucket per sheet
  const size_t b = 2 * (3 * nd + ni) + al(sizeof(TileRec) * (size_t)tiles) + radix_bytes(n) +
                   al(4 * (size_t)nb);
  PC(cudaMalloc(&p->ws, b));
  char* q = static_cast<char*>(p->ws);
  for (int k = 0; k < 2; ++k) {
    p->set[k].x = reinterpret_cast<double*>(q); q += nd;
    p->set[k].v = reinterpret_cast<double*>(q); q += nd;
    p->set[k].m = reinterpret_cast<double*>(q); q += nd;
    p->set[k].idx = reinterpret_cast<int32_t*>(q); q += ni;
  }
  p->trecs = reinterpret_cast<TileRec*>(q); q += al(sizeof(TileRec) * (size_t)tiles);
  radix_bind(&p->radix, q, n);
  q += radix_bytes(n);
  p->offs = reinterpret_cast<unsigned*>(q);
  PC(cudaMemsetAsync(p->trecs, 0, sizeof(TileRec) * (size_t)tiles, p->stream));
  p->ws_n = n;
  return WG_OK;
}

// Sheets of one batch of members sorted together: keeps the workspace (about
// 210 B per sheet) to a few GB.  (The second sort's key, member and rank in
// rank_bits + member bits <= 50 bits, stays below the sign and exponent bits.)
constexpr int64_t kBatchSheets = 1ll << 25;

int ensure_batch(wg_pool* p, int64_t n, int64_t ntasks, int nsegs) {
  if (n <= p->bws_n && ntasks <= p->bws_tasks && nsegs <= p->bws_segs && p->bws) return WG_OK;
  // grown, never shrunk, in powers of two: batches of changing shape reuse it
  // (a re-allocation waits for the device)
  n = pow2_at_least(std::max<int64_t>(n, p->bws_n));
  ntasks = pow2_at_least(std::max<int64_t>(ntasks, p->bws_tasks));
  nsegs = (int)pow2_at_least(std::max<int64_t>(nsegs, p->bws_segs));
  PC(cudaStreamSynchronize(p->stream));
  if (p->bws) cudaFree(p->bws);
  p->bws = nullptr;
  p->bws_n = p->bws_tasks = p->bws_segs = 0;
  const size_t nd = al((size_t)n * 8), ni = al((size_t)n * 4);
  const size_t set = 3 * nd + ni;
  const size_t b = 6 * set + radix_bytes(n) + 2 * al(sizeof(StateTable)) + al(sizeof(StepFlags)) +
                   al(4 * (size_t)ntasks) + al(sizeof(BatchSeg) * (size_t)nsegs) +
                   al(8 * (size_t)(nsegs + 1)) + al(sizeof(BucketTask) * (size_t)ntasks);
  PC(cudaMalloc(&p->bws, b));
  char* q = static_cast<char*>(p->bws);
  StateRef* sets[6] = {&p->bW, &p->bA[0], &p->bA[1], &p->bB[0], &p->bB[1], &p->bO};
  for (StateRef* r : sets) {
    r->x = reinterpret_cast<double*>(q); q += nd;
    r->v = reinterpret_cast<double*>(q); q += nd;
    r->m = reinterpret_cast<double*>(q); q += nd;
    r->idx = reinterpret_cast<int32_t*>(q); q += ni;
  }
  radix_bind(&p->bradix, q, n);
  q += radix_bytes(n);
  p->btA = reinterpret_cast<StateTable*>(q); q += al(sizeof(StateTable));
  p->btB = reinterpret_cast<StateTable*>(q); q += al(sizeof(StateTable));
  p->bflag = reinterpret_cast<StepFlags*>(q); q += al(sizeof(StepFlags));
  p->boffs = reinterpret_cast<unsigned*>(q); q += al(4 * (size_t)ntasks);
  p->bsegs = reinterpret_cast<BatchSeg*>(q); q += al(sizeof(BatchSeg) * (size_t)nsegs);
  p->bseg_out = reinterpret_cast<int64_t*>(q); q += al(8 * (size_t)(nsegs + 1));
  p->btasks = reinterpret_cast<BucketTask*>(q);
  p->h_bsegs.resize((size_t)nsegs);
  p->h_bseg_out.resize((size_t)nsegs + 1);
  p->h_btasks.resize((size_t)ntasks);
  StepFlags f{};
  f.unsorted = 1u;
  PC(cudaMemcpy(p->bflag, &f, sizeof(f), cudaMemcpyHostToDevice));
  p->bws_n = n;
  p->bws_tasks = ntasks;
  p->bws_segs = nsegs;
  return WG_OK;
}

// Copy of the batch for the first sort: keys from x (moved on by the
// member's pending half drift, if any), ties by original index, and each
// sheet's place in the batch carried in v (as the bits of a double).
__global__ void k_seg_prep_a(StateRef w, StateRef a, const BatchSeg* segs, int nseg, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += stride) {
    int lo = 0, hi = nseg - 1;  // the member whose range holds q
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (segs[mid].out <= q) lo = mid; else hi = mid - 1;
    }
    // the key of the position the member's next sub-step will load it at
    // (the same fma as its load): x, or x + pre v after a last sub-step
    const double pre = segs[lo].pre;
    a.x[q] = pre != 0.0 ? fma(pre, w.v[q], w.x[q]) : w.x[q];
    a.v[q] = __longlong_as_double((long long)q);
    a.m[q] = 0.0;
    a.idx[q] = w.idx[q];
  }
}

// Second sort's keys: (member, rank in the first sort) packed into the bits
// of one double, so that sorting them groups the members and keeps the first
// order inside.
__global__ void k_seg_prep_b(const StateTable* ta, const int64_t* seg_out, int nseg, StateRef b,
                             int64_t n, int rank_bits) {
  const StateRef a = ta->cur;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += stride) {
    const int64_t g = (int64_t)__double_as_longlong(a.v[p]);
    int lo = 0, hi = nseg - 1;  // the member whose range holds g
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (seg_out[mid] <= g) lo = mid; else hi = mid - 1;
    }
    // the key as raw bits (a non-negative double whose order is that of its
    // bits): member above rank, so that the sort's passes over the bytes
    // above both are skipped as constant
    b.x[p] = __longlong_as_double(((long long)lo << rank_bits) | p);
    b.v[p] = 0.0;
    b.m[p] = 0.0;
    b.idx[p] = (int32_t)p;
  }
}

// The batch in (member, key, index) order: sheet q is the first sort's
// rank-p sheet, whose place in the compacted batch is g.
__global__ void k_seg_final(const StateTable* ta, const StateTable* tb, StateRef w, StateRef o,
                            int64_t n) {
  // tb null: a batch of one member, already in order after the first sort
  const StateRef a = ta->cur;
  const int32_t* bidx = tb ? tb->cur.idx : nullptr;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += stride) {
    const int64_t p = bidx ? (int64_t)bidx[q] : q;
    if (p < 0 || p >= n) continue;  // never, unless a sort gave up (the error word says so)
    const int64_t g = (int64_t)__double_as_longlong(a.v[p]);
    if (g < 0 || g >= n) continue;
    o.x[q] = w.x[g];
    o.v[q] = w.v[g];
    o.m[q] = w.m[g];
    o.idx[q] = w.idx[g];
  }
}

// n words device -> mapped host memory.
__global__ void k_read_back(const unsigned* src, unsigned* dst, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

int grid_1d(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  return (int)(g < 1 ? 1 : g);
}

// Bring a mode-0 simulation to its bucket layout: half drift of dt/2 on the
// compact store, full radix sort, bucketize.  Uses the shared workspace.
int to_buckets(wg_pool* p, PoolSim* s, double dt) {
  int rc = ensure_workspace(p, s->n);
  if (rc) return rc;
  StateRef own{s->ox, s->ov, s->om, s->oi};
  k_set_table<<<1, 1, 0, p->stream>>>(p->table, own, p->set[1]);
  launch_drift(p->table, s->n, dt / 2., &p->wflags[0], p->stream);  // also marks "unsorted"
  radix_sort_state(p->table, s->n, &p->radix, &p->wflags[0], p->err, p->stream);
  launch_bucketize(p->table, s->n, s->tune.target, s->nb, kBucketCap, s->E, s->bx[0], s->bv[0],
                   s->bm[0],
                   s->bi[0], s->bcnt, s->bmass, s->qk[0], s->qi[0], p->stream);
  p->launches += 3 + kRadixLaunches;
  s->lay = 0;
  s->qsel = 0;
  s->cslot = 0;
  s->mode = 1;
  s->pending_dt = dt;
  return WG_OK;
}

// Bucket layout `lay` of s with the counts of aggregate slot `cslot` (+ the
// overflow entries counted in oc) -> the workspace's first set, unsorted.
void buckets_to_workspace(wg_pool* p, PoolSim* s, int lay, int cslot, const unsigned* oc) {
  k_set_table<<<1, 1, 0, p->stream>>>(p->table, p->set[0], p->set[1]);
  launch_compact(p->table, s->nb, kBucketCap, s->bx[lay], s->bv[lay], s->bm[lay], s->bi[lay],
                 s->bcnt[cslot],
                 p->offs, s->ox, s->ov, s->om, s->oi, oc, s->n, p->stream);
  p->launches += 3;
}

void store_compact(wg_pool* p, PoolSim* s) {
  k_store_compact<<<grid_1d(s->n), 256, 0, p->stream>>>(p->table, s->n, s->ox, s->ov, s->om,
                                                          s->oi);
  p->launches += 1;
}

// Members of at least this many sheets that overflow again within two
// sub-steps of a re-sort finish the call on the compact path (below, one
// member at a time: for smaller members its launches cost more than the
// batched re-sorts it saves).
constexpr int64_t kCompactFinishSheets = 1ll << 20;

// Member k of the call overflowed in sub-step kk again right after a re-sort:
// it finishes the call on the compact path -- its layout `lay` (counts in
// aggregate slot `cslot`) and overflow list compacted into the workspace, then
// per remaining sub-step a full radix sort and the fused force kernel, the
// outputs de-sorted, the state stored compact (the next call re-sorts it).
int finish_compact(wg_pool* p, PoolSim* s, int k, int kk, int lay, int cslot, double dt,
                   int nleap) {
  int rc = ensure_workspace(p, s->n);
  if (rc) return rc;
  buckets_to_workspace(p, s, lay, cslot, p->ocount + 2 * k);
  ForceArgs f{};
  f.table = p->table;
  f.n = s->n;
  f.T_lo = s->T_lo;
  f.T_hi = s->T_hi;
  f.E = s->E;
  f.has_omega = s->omega2 >= 0;
  f.omega2 = s->omega2;
  f.ext = s->ext;
  f.t_seq = p->t_seq + (size_t)k * p->cap_leap;
  f.epochs = p->epochs;
  f.recs = p->trecs;
  f.err = p->err;
  f.a_out = nullptr;
  const int64_t tiles = (s->n + kForceTile - 1) / kForceTile;
  PC(cudaMemsetAsync(p->tickets, 0, 4 * (size_t)nleap, p->stream));
  // the tile records are shared by every member finished this way: cleared,
  // so that no tile takes another member's prefix
  PC(cudaMemsetAsync(p->trecs, 0, sizeof(TileRec) * (size_t)tiles, p->stream));
  for (int i = kk + 1; i < nleap; ++i) {
    PC(cudaMemsetAsync(&p->wflags[i].unsorted, 1, sizeof(unsigned), p->stream));
    radix_sort_state(p->table, s->n, &p->radix, &p->wflags[i], p->err, p->stream);
    f.sub = i;
    f.dt_kick = dt;
    f.dt_drift = (i == nleap - 1) ? dt / 2. : dt;
    f.ticket = p->tickets + i;
    f.flag_out = &p->wflags[i + 1];
    launch_force(f, tiles, p->stream);
  }
  launch_desort(p->table, s->n, s->x_out, s->v_out, p->stream);
  store_compact(p, s);
  p->launches += (int64_t)(nleap - kk - 1) * (1 + kRadixLaunches) + 1;
  s->mode = 0;
  return WG_OK;
}

}  // namespace

extern "C" {

int64_t wg_pool_sim_bytes(int64_t n) { return n < 1 ? 0 : (int64_t)sim_bytes(n); }

int wg_pool_create(int64_t budget_bytes, wg_pool** out) {
  if (!out) return pool_fail(WG_ERR_ARG, "null output handle");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return pool_fail(WG_ERR_NODEV, "no CUDA device visible");
  }
  wg_pool* p = new wg_pool();
  p->budget = budget_bytes > 0 ? budget_bytes : 0;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&p->dl_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&p->ev0) != cudaSuccess || cudaEventCreate(&p->ev1) != cudaSuccess ||
      cudaEventCreate(&p->ev_mid) != cudaSuccess || cudaEventCreate(&p->ev_rec) != cudaSuccess) {
    delete p;
    return pool_fail(WG_ERR_CUDA, "stream/event creation failed");
  }
  int rc = ensure_small(p, 16, 64, 1024);
  if (rc) {
    delete p;
    return rc;
  }
  bucket_step_prepare();
  *out = p;
  return WG_OK;
}

int wg_pool_add(wg_pool* p, int64_t n, const double* x, const double* v, const double* m,
                double totmass, double omega2, int ext_kind, const double* ext_params,
                int n_ext_params, int* sim_id) {
  if (p && p->pend_active)
    return pool_fail(WG_ERR_ARG, "a step is in flight: call wg_pool_step_end first");
  if (!p || !sim_id) return pool_fail(WG_ERR_ARG, "null argument");
  if (n < 1 || n >= (1ll << 30)) return pool_fail(WG_ERR_ARG, "n outside [1, 2^30)");
  if (!x || !v || !m) return pool_fail(WG_ERR_ARG, "null array");
  if (!std::isfinite(totmass) || totmass < 0 || !std::isfinite(omega2))
    return pool_fail(WG_ERR_ARG, "totmass must be finite and >= 0, omega2 finite");
  double mmax = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (!(m[i] >= 0) || !std::isfinite(m[i]) || !std::isfinite(x[i]) || !std::isfinite(v[i]))
      return pool_fail(WG_ERR_ARG, "sheet %lld: non-finite value or negative mass", (long long)i);
    if (m[i] > mmax) mmax = m[i];
  }
  if (mmax > 2 * totmass)
    return pool_fail(WG_ERR_ARG, "a single mass exceeds twice totmass");
  ExtSpec ext;
  {
    char msg[256];
    if (parse_ext(ext_kind, ext_params, n_ext_params, &ext, msg, sizeof(msg)) != WG_OK)
      return pool_fail(WG_ERR_EXT, "%s", msg);
  }
  const size_t bytes = sim_bytes(n);
  if (p->budget && p->used + (int64_t)bytes > p->budget)
    return pool_fail(WG_ERR_BUDGET, "simulation of %lld sheets needs %zu bytes; %lld of %lld in use",
                     (long long)n, bytes, (long long)p->used, (long long)p->budget);
  PoolSim* s = new PoolSim();
  s->n = n;
  s->tune = tuning_for(n);
  s->nb = (n + s->tune.target - 1) / s->tune.target;
  s->bytes = bytes;
  cudaError_t e = cudaMallocAsync(&s->mem, bytes, p->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete s;
    return pool_fail(WG_ERR_NOMEM, "allocation of %zu bytes failed: %s", bytes,
                     cudaGetErrorString(e));
  }
  carve(s);
  s->totmass = totmass;
  s->omega2 = omega2;
  s->ext_spec = ext;
  e = attach_ext_program(&s->ext_spec, &s->d_prog, p->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaFreeAsync(s->mem, p->stream);
    delete s;
    return pool_fail(WG_ERR_NOMEM, "upload of the external-force program failed: %s",
                     cudaGetErrorString(e));
  }
  s->ext = s->ext_spec.f;
  if (totmass > 0) {
    int eT = 0;
    std::frexp(totmass, &eT);
    s->E = 123 - eT;
  }
  const u128 T = fixed_of(totmass, s->E);
  s->T_lo = (uint64_t)T;
  s->T_hi = (uint64_t)(T >> 64);
  PC(cudaMemsetAsync(s->recs, 0, sizeof(BucketRec) * (size_t)s->nb, p->stream));
  if (s->ptab) {
    const StateTable t = member_sample_table(s);
    PC(cudaMemcpyAsync(s->ptab, &t, sizeof(t), cudaMemcpyHostToDevice, p->stream));
    PC(cudaStreamSynchronize(p->stream));  // t lives on this stack frame
  }
  PC(cudaMemcpyAsync(s->ox, x, 8 * (size_t)n, cudaMemcpyHostToDevice, p->stream));
  PC(cudaMemcpyAsync(s->ov, v, 8 * (size_t)n, cudaMemcpyHostToDevice, p->stream));
  PC(cudaMemcpyAsync(s->om, m, 8 * (size_t)n, cudaMemcpyHostToDevice, p->stream));
  k_iota_i32<<<grid_1d(n), 256, 0, p->stream>>>(s->oi, n);
  PC(cudaStreamSynchronize(p->stream));
  p->used += (int64_t)bytes;
  int id = -1;
  for (size_t i = 0; i < p->sims.size(); ++i)
    if (!p->sims[i]) {
      id = (int)i;
      break;
    }
  if (id < 0) {
    id = (int)p->sims.size();
    p->sims.push_back(nullptr);
  }
  p->sims[(size_t)id] = s;
  *sim_id = id;
  return WG_OK;
}

int wg_pool_remove(wg_pool* p, int sim_id) {
  if (!p || sim_id < 0 || (size_t)sim_id >= p->sims.size() || !p->sims[(size_t)sim_id])
    return pool_fail(WG_ERR_ARG, "no simulation %d in the pool", sim_id);
  if (p->pend_active) return pool_fail(WG_ERR_ARG, "a step is in flight: call wg_pool_step_end first");
  PoolSim* s = p->sims[(size_t)sim_id];
  cudaFreeAsync(s->mem, p->stream);
  if (s->d_prog) {
    cudaStreamSynchronize(p->stream);
    cudaFree(s->d_prog);
  }
  p->used -= (int64_t)s->bytes;
  delete s;
  p->sims[(size_t)sim_id] = nullptr;
  return WG_OK;
}

// The first half of a pool step: everything up to the launch of the
// sub-steps (or the replay of their graph); pool_step_end completes it.
static int pool_step_begin(wg_pool* p, int count, const int* ids, const double* dt, int nleap,
                           double* t0) {
  if (!p || count < 1 || !ids || !dt || nleap < 1 || nleap > kMaxLeap)
    return pool_fail(WG_ERR_ARG, "bad arguments to wg_pool_step");
  if (p->pend_active) return pool_fail(WG_ERR_ARG, "a step is in flight: call wg_pool_step_end first");
  std::vector<PoolSim*> act((size_t)count);
  int64_t ntasks = 0;
  for (int k = 0; k < count; ++k) {
    if (ids[k] < 0 || (size_t)ids[k] >= p->sims.size() || !p->sims[(size_t)ids[k]])
      return pool_fail(WG_ERR_ARG, "no simulation %d in the pool", ids[k]);
    if (!std::isfinite(dt[k])) return pool_fail(WG_ERR_ARG, "dt of simulation %d", ids[k]);
    for (int j = 0; j < k; ++j)
      if (ids[j] == ids[k]) return pool_fail(WG_ERR_ARG, "simulation %d listed twice", ids[k]);
    act[(size_t)k] = p->sims[(size_t)ids[k]];
    ntasks += act[(size_t)k]->nb;
  }
  if (ntasks >= (1ll << 31)) return pool_fail(WG_ERR_ARG, "too many buckets in one step");
  int rc = ensure_small(p, count, nleap, ntasks);
  if (rc) return rc;
  const int L1 = p->cap_leap;
  // times (the reference's lagged, repeatedly added t) and epochs
  for (int k = 0; k < count; ++k) {
    double t = t0 ? t0[k] : 0.0;
    for (int i = 0; i < nleap; ++i) {
      p->h_t[(size_t)k * L1 + i] = t;
      if (act[(size_t)k]->ext.kind != EXT_NONE) t += dt[k];
    }
    if (t0) t0[k] = t;
  }
  if (p->epoch + (unsigned)nleap > kEpochLimit) {
    // restart epochs: forget every look-back record
    for (PoolSim* s : p->sims)
      if (s) PC(cudaMemsetAsync(s->recs, 0, sizeof(BucketRec) * (size_t)s->nb, p->stream));
    if (p->ws)
      PC(cudaMemsetAsync(p->trecs, 0,
                         sizeof(TileRec) * (size_t)((p->ws_n + kForceTile - 1) / kForceTile),
                         p->stream));
    p->epoch = 1;
  }
  for (int i = 0; i < nleap; ++i) p->h_ep[i] = p->epoch + (unsigned)i;
  p->epoch += (unsigned)nleap;
  PC(cudaEventRecord(p->ev0, p->stream));
  PC(cudaMemsetAsync(p->ocount, 0, 8 * (size_t)count, p->stream));
  // simulations that are compact, or routed for another dt, re-sort first
  for (int k = 0; k < count; ++k) {
    PoolSim* s = act[(size_t)k];
    if (s->mode == 1 && dt[k] != s->pending_dt) {
      rc = ensure_workspace(p, s->n);
      if (rc) return rc;
      buckets_to_workspace(p, s, s->lay, s->cslot, p->ocount + 2 * k);
      store_compact(p, s);
      s->mode = 0;
    }
    if (s->mode == 0) {
      PC(cudaMemsetAsync(&p->wflags[0], 0, sizeof(StepFlags), p->stream));
      rc = to_buckets(p, s, dt[k]);
      ++p->stats.members_sorted;
      if (rc) return rc;
      s->fresh = true;
    }
  }
  // the output of each simulation's last step stays downloadable while this
  // one runs: the step writes the other pair of output buffers
  for (int k = 0; k < count; ++k) {
    PoolSim* s = act[(size_t)k];
    s->done_x = s->out_valid ? s->x_out : nullptr;
    s->done_v = s->out_valid ? s->v_out : nullptr;
    std::swap(s->x_out, s->x_out2);
    std::swap(s->v_out, s->v_out2);
  }
  // until the step is launched, an error return swaps the output buffers
  // back, so that wg_pool_download keeps returning the last completed output
  struct SwapBack {
    const std::vector<PoolSim*>& act;
    bool armed = true;
    ~SwapBack() {
      if (!armed) return;
      for (PoolSim* s : act) {
        std::swap(s->x_out, s->x_out2);
        std::swap(s->v_out, s->v_out2);
      }
    }
  } swap_back{act};
  // the kernel's view of every simulation, and the task list
  int64_t t = 0;
  for (int k = 0; k < count; ++k) {
    PoolSim* s = act[(size_t)k];
    SimDev& d = p->h_dev[k];
    d.rec_out = nullptr;  // members write x_out, v_out directly
    for (int j = 0; j < 2; ++j) {
      d.bx[j] = s->bx[j];
      d.bv[j] = s->bv[j];
      d.bm[j] = s->bm[j];
      d.bi[j] = s->bi[j];
      d.qk[j] = s->qk[j];
      d.qi[j] = s->qi[j];
    }
    for (int j = 0; j < kAggSlots; ++j) {
      d.bcnt[j] = s->bcnt[j];
      d.bmass[j] = s->bmass[j];
    }
    d.recs = s->recs;
    d.ox = s->ox;
    d.ov = s->ov;
    d.om = s->om;
    d.oi = s->oi;
    d.ocount = p->ocount + 2 * k;
    d.x_out = s->x_out;
    d.v_out = s->v_out;
    d.xi_out = nullptr;
    d.a_out = nullptr;
    d.flags = p->flags + (size_t)k * (L1 + 1);
    d.t_seq = p->t_seq + (size_t)k * L1;
    d.n = s->n;
    d.nb = s->nb;
    d.target = s->tune.target;
    d.window = s->tune.window;
    d.sort_bits = s->tune.sort_bits;
    d.capg = kBucketCap;  // members have no big buckets
    d.ptab = s->pred_calls > 0 ? s->ptab : nullptr;
    d.T_lo = s->T_lo;
    d.T_hi = s->T_hi;
    d.E = s->E;
    d.has_omega = s->omega2 >= 0;
    d.omega2 = s->omega2;
    d.ext = s->ext;
    d.dt = dt[k];
    d.pre_dt = s->fresh ? 0.0 : dt[k] / 2.;
    d.lay0 = s->lay;
    d.qsel0 = s->qsel;
    d.cs0 = s->cslot;
    for (int64_t b = 0; b < s->nb; ++b) p->h_tasks[t++] = BucketTask{k, (int)b};
  }
  // device sequence of the call, captured in a CUDA graph and replayed while
  // the number of simulations, buckets and sub-steps stays the same
  bool launch_expr = false;  // the graph's kernels carry the expression interpreter
  for (PoolSim* a : act) launch_expr |= a->ext.kind == EXT_EXPR;
  const bool rebuild = !p->gexec || p->g_count != count || p->g_nleap != nleap ||
                       p->g_ntasks != ntasks || p->g_small != p->small ||
                       p->g_expr != launch_expr;
  if (rebuild) {
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    p->gexec = nullptr;
    cudaGraph_t g = nullptr;
    PC(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
    cudaMemcpyAsync(p->t_seq, p->h_t, 8 * (size_t)count * L1, cudaMemcpyHostToDevice,
                    p->stream);
    cudaMemcpyAsync(p->epochs, p->h_ep, 4 * (size_t)nleap, cudaMemcpyHostToDevice, p->stream);
    cudaMemsetAsync(p->tickets, 0, 4 * (size_t)nleap, p->stream);
    cudaMemsetAsync(p->flags, 0, sizeof(StepFlags) * (size_t)count * (L1 + 1), p->stream);
    cudaMemcpyAsync(p->d_dev, p->h_dev, sizeof(SimDev) * (size_t)count, cudaMemcpyHostToDevice,
                    p->stream);
    cudaMemcpyAsync(p->tasks, p->h_tasks, sizeof(BucketTask) * (size_t)ntasks,
                    cudaMemcpyHostToDevice, p->stream);
    int cps = 1;
    int64_t nmax = 0;
    for (PoolSim* a : act)
      if (a->n > nmax) {
        nmax = a->n;
        cps = a->tune.ctas_per_sm;
      }
    const int grid = cps * p->sms;
    for (int i = 0; i < nleap; ++i) {
      StepLaunch L;
      L.sims = p->d_dev;
      L.tasks = p->tasks;
      L.ntasks = (int)ntasks;
      L.sub = i;
      L.nleap = nleap;
      L.epochs = p->epochs;
      L.ticket = p->tickets + i;
      L.err = p->err;
      L.profile = 0;
      L.any_expr = launch_expr;
      L.big_list = nullptr;
      L.big_count = nullptr;
      L.big_ticket = nullptr;
      L.big_cap = 0;
      launch_bucket_step(L, grid, p->stream);
      // members with predicted splitters: their samples, sorted, become the
      // splitters this sub-step published (one CTA per member; the others
      // return at once)
      launch_member_splitters(p->d_dev, nullptr, count, i, p->stream);
    }
    // the overflow counts to the host by a kernel's stores into mapped
    // page-locked memory, not a copy: a copy would queue on the copy engine
    // behind downloads running meanwhile, and the step would end with them
    k_read_back<<<1, 256, 0, p->stream>>>(p->ocount, p->d_oc, 2 * count);
    PC(cudaStreamEndCapture(p->stream, &g));
    const cudaError_t ie = cudaGraphInstantiate(&p->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      p->gexec = nullptr;
      return pool_fail(WG_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(ie));
    }
    p->g_count = count;
    p->g_nleap = nleap;
    p->g_ntasks = ntasks;
    p->g_small = p->small;
    p->g_expr = launch_expr;
    p->graph_builds++;
  }
  PC(cudaGraphLaunch(p->gexec, p->stream));
  PC(cudaEventRecord(p->ev_mid, p->stream));
  ++p->stats.steps;
  swap_back.armed = false;
  p->launches += 2 * nleap + 1;
  p->pend_active = true;
  p->pend_count = count;
  p->pend_nleap = nleap;
  p->pend_act = act;
  p->pend_dt.assign(dt, dt + count);
  return WG_OK;
}

// The second half: waits for the sub-steps, then the bookkeeping and the
// recovery of simulations that overflowed a bucket.
static int pool_step_end(wg_pool* p, double* time_elapsed) {
  if (!p || !p->pend_active) return pool_fail(WG_ERR_ARG, "no pool step in flight");
  p->pend_active = false;
  const int count = p->pend_count, nleap = p->pend_nleap;
  const std::vector<PoolSim*>& act = p->pend_act;
  const double* dt = p->pend_dt.data();
  int rc = WG_OK;
  PC(cudaStreamSynchronize(p->stream));
  // bookkeeping, and recovery of simulations that overflowed a bucket.  A
  // sub-step that overflowed a bucket left the sheets complete in the layout
  // it wrote plus the overflow list: re-sort them, lay out fresh buckets and
  // restart the remaining sub-steps on the bucket path (a last sub-step has
  // already written every output).  All simulations that overflowed are
  // handled together, in rounds: one segmented re-sort of all of them (in
  // chunks of at most kBatchSheets sheets), then one launch per sub-step over
  // all of them (each joining from the sub-step it restarts at) and one host
  // wait.  A simulation restarts past the sub-step that overflowed, so the
  // rounds end within nleap.
  std::vector<unsigned> ab((size_t)count);
  std::vector<int> l0((size_t)count), c0((size_t)count), q0((size_t)count);
  for (int k = 0; k < count; ++k) {
    PoolSim* s = act[(size_t)k];
    l0[(size_t)k] = s->lay;
    c0[(size_t)k] = s->cslot;
    s->lay = (s->lay + nleap) & 1;
    s->qsel = (s->qsel + nleap) & 1;
    s->cslot = (s->cslot + nleap) % kAggSlots;
    s->mode = 1;
    s->pending_dt = dt[k];
    s->fresh = false;
    s->out_valid = true;
    ab[(size_t)k] = p->h_oc[2 * k + 1];
    // predicted splitters for the next calls of a member that overflowed;
    // counted down by the calls that do not
    if (ab[(size_t)k] && s->ptab)
      s->pred_calls = kPredMemberCalls;
    else if (s->pred_calls > 0)
      --s->pred_calls;
  }
  const bool recovery = std::any_of(ab.begin(), ab.end(), [](unsigned a) { return a != 0; });
  if (recovery) PC(cudaEventRecord(p->ev_rec, p->stream));
  std::vector<int> restarted((size_t)count, -1);  // sub-step a member last restarted at
  for (;;) {
    std::vector<std::pair<int, int>> batch;   // (from, k)
    std::vector<std::pair<int, int>> finish;  // (kk, k): overflowed again right after a re-sort
    std::vector<int> lay_w((size_t)count), cs_w((size_t)count);
    for (int k = 0; k < count; ++k) {
      if (!ab[(size_t)k]) continue;
      const int kk = (int)ab[(size_t)k] - 1;
      ab[(size_t)k] = 0;
      lay_w[(size_t)k] = (l0[(size_t)k] + kk + 1) & 1;
      cs_w[(size_t)k] = (c0[(size_t)k] + kk + 1) % kAggSlots;
      // a large member that overflows again within two sub-steps of its
      // restart would keep overflowing: it finishes the call on the compact
      // path.  (An overflow in the call's last sub-step, whose outputs are
      // written, is re-sorted with the others and restarts nothing: from ==
      // nleap.)
      const int r = restarted[(size_t)k];
      if (r >= 0 && kk < r + 2 && kk < nleap - 1 && act[(size_t)k]->n >= kCompactFinishSheets)
        finish.emplace_back(kk, k);
      else
        batch.emplace_back(kk + 1, k);
    }
    if (batch.empty() && finish.empty()) break;
    ++p->stats.recovery_rounds;
    p->stats.overflows += (int64_t)(batch.size() + finish.size());
    for (const auto& e : batch) {
      p->stats.sheets_resorted += act[(size_t)e.second]->n;
      p->stats.substeps_relaunched += nleap - e.first;
      restarted[(size_t)e.second] = e.first;
    }
    for (const auto& e : finish) {
      const int kk = e.first, k = e.second;
      rc = finish_compact(p, act[(size_t)k], k, kk, lay_w[(size_t)k], cs_w[(size_t)k], dt[k],
                          nleap);
      if (rc) return rc;
      ++p->stats.members_compact;
      p->stats.substeps_compact += nleap - kk - 1;
    }
    if (batch.empty()) break;
    // the restarted members, re-sorted together in chunks of at most
    // kBatchSheets sheets: compaction of every layout and overflow list, one
    // sort by (member, key, index) as two radix sorts, fresh layouts
    // (a chunk of one member needs no grouping sort; sorting large members
    // alone that way measured slower than batching them, so members are
    // batched in their order and a chunk holds one only when it is that large)
    for (size_t j0 = 0; j0 < batch.size();) {
      size_t j1 = j0;
      int64_t sheets = 0, nbk = 0;
      while (j1 < batch.size()) {
        const PoolSim* s = act[(size_t)batch[j1].second];
        if (j1 > j0 && sheets + s->n > kBatchSheets) break;
        sheets += s->n;
        nbk += s->nb;
        ++j1;
      }
      const int nseg = (int)(j1 - j0);
      rc = ensure_batch(p, sheets, nbk + nseg, nseg);
      if (rc) return rc;
      int64_t out = 0, toff = 0, nt = 0;
      for (int j = 0; j < nseg; ++j) {
        const int k = batch[j0 + (size_t)j].second;
        const PoolSim* s = act[(size_t)k];
        BatchSeg g;
        g.k = k;
        g.lay = lay_w[(size_t)k];
        g.cslot = cs_w[(size_t)k];
        g.pad = 0;
        g.out = out;
        g.n = s->n;
        g.toff = toff;
        // after an overflow in the last sub-step the next call opens with a
        // half drift applied while loading: sort and bucket by where it puts
        // the sheets (a change of dt re-sorts them then)
        g.pre = batch[j0 + (size_t)j].first == nleap ? dt[k] / 2. : 0.0;
        p->h_bsegs[j] = g;
        p->h_bseg_out[j] = out;
        for (int64_t bb = 0; bb < s->nb; ++bb) p->h_btasks[nt++] = BucketTask{j, (int)bb};
        out += s->n;
        toff += s->nb;
      }
      p->h_bseg_out[nseg] = out;
      for (int j = 0; j < nseg; ++j)  // overflow lists, after every bucket task
        p->h_btasks[nt++] = BucketTask{j, (int)act[(size_t)batch[j0 + (size_t)j].second]->nb};
      PC(cudaMemcpyAsync(p->bsegs, p->h_bsegs.data(), sizeof(BatchSeg) * (size_t)nseg,
                         cudaMemcpyHostToDevice, p->stream));
      PC(cudaMemcpyAsync(p->bseg_out, p->h_bseg_out.data(), 8 * (size_t)(nseg + 1),
                         cudaMemcpyHostToDevice, p->stream));
      PC(cudaMemcpyAsync(p->btasks, p->h_btasks.data(), sizeof(BucketTask) * (size_t)nt,
                         cudaMemcpyHostToDevice, p->stream));
      launch_batch_compact(p->d_dev, p->bsegs, nseg, p->btasks, nt, p->bW, p->boffs, sheets,
                           p->stream);
      StateTable ta, tb;  // pageable: copied at once
      ta.cur = p->bA[0];
      ta.other = p->bA[1];
      tb.cur = p->bB[0];
      tb.other = p->bB[1];
      PC(cudaMemcpyAsync(p->btA, &ta, sizeof(ta), cudaMemcpyHostToDevice, p->stream));
      PC(cudaMemcpyAsync(p->btB, &tb, sizeof(tb), cudaMemcpyHostToDevice, p->stream));
      k_seg_prep_a<<<grid_1d(sheets), 256, 0, p->stream>>>(p->bW, p->bA[0], p->bsegs, nseg,
                                                           sheets);
      radix_sort_state(p->btA, sheets, &p->bradix, p->bflag, p->err, p->stream);
      if (nseg > 1) {
        int rank_bits = 1;  // bits of a rank in the batch; with the member's, at most 2 x 31
        while ((int64_t)1 << rank_bits < sheets) ++rank_bits;
        k_seg_prep_b<<<grid_1d(sheets), 256, 0, p->stream>>>(p->btA, p->bseg_out, nseg,
                                                             p->bB[0], sheets, rank_bits);
        radix_sort_state(p->btB, sheets, &p->bradix, p->bflag, p->err, p->stream);
        p->launches += 1 + kRadixLaunches;
      }
      k_seg_final<<<grid_1d(sheets), 256, 0, p->stream>>>(p->btA, nseg > 1 ? p->btB : nullptr,
                                                          p->bW, p->bO, sheets);
      launch_batch_bucketize(p->d_dev, p->bsegs, p->btasks, nbk, p->bO, sheets, p->stream);
      p->launches += 7 + kRadixLaunches;
      j0 = j1;
    }
    // their sub-steps from the restart on: `from` reads layout 0, aggregate
    // slot 0 and routes by splitter set 0
    for (const auto& e : batch) {
      const int from = e.first, k = e.second;
      PoolSim* s = act[(size_t)k];
      l0[(size_t)k] = from & 1;
      q0[(size_t)k] = from & 1;
      c0[(size_t)k] = (kAggSlots - from % kAggSlots) % kAggSlots;
      SimDev& d = p->h_dev[k];
      d.lay0 = l0[(size_t)k];
      d.qsel0 = q0[(size_t)k];
      d.cs0 = c0[(size_t)k];
      d.pre_dt = 0.0;
      d.ptab = s->ptab;  // the restarted sub-steps predict their splitters
      s->lay = (l0[(size_t)k] + nleap) & 1;
      s->qsel = (q0[(size_t)k] + nleap) & 1;
      s->cslot = (c0[(size_t)k] + nleap) % kAggSlots;
    }
    PC(cudaMemcpyAsync(p->d_dev, p->h_dev, sizeof(SimDev) * (size_t)count, cudaMemcpyHostToDevice,
                       p->stream));
    PC(cudaMemsetAsync(p->ocount, 0, 8 * (size_t)count, p->stream));
    if (batch.empty()) break;
    // the restarted simulations, earliest restart first: the launch of
    // sub-step i takes the prefix of them that restart at i or before
    std::sort(batch.begin(), batch.end());
    int64_t nt = 0;
    std::vector<int64_t> upto(batch.size());
    int cps = 1;
    bool any_expr = false;
    for (size_t j = 0; j < batch.size(); ++j) {
      const int k = batch[j].second;
      PoolSim* s = act[(size_t)k];
      for (int64_t b = 0; b < s->nb; ++b) p->h_rtasks[nt++] = BucketTask{k, (int)b};
      upto[j] = nt;
      p->h_rlist[j] = k;
      cps = s->tune.ctas_per_sm > cps ? s->tune.ctas_per_sm : cps;
      any_expr |= s->ext.kind == EXT_EXPR;
    }
    PC(cudaMemcpyAsync(p->rtasks, p->h_rtasks, sizeof(BucketTask) * (size_t)nt,
                       cudaMemcpyHostToDevice, p->stream));
    PC(cudaMemcpyAsync(p->rlist, p->h_rlist, 4 * batch.size(), cudaMemcpyHostToDevice,
                       p->stream));
    const int first = batch.front().first;
    // the launches of these sub-steps consumed their tickets
    if (first < nleap)
      PC(cudaMemsetAsync(p->tickets + first, 0, 4 * (size_t)(nleap - first), p->stream));
    size_t m = 0;
    for (int i = first; i < nleap; ++i) {
      while (m < batch.size() && batch[m].first <= i) ++m;
      StepLaunch L;
      L.sims = p->d_dev;
      L.tasks = p->rtasks;
      L.ntasks = (int)upto[m - 1];
      L.sub = i;
      L.nleap = nleap;
      L.epochs = p->epochs;
      L.ticket = p->tickets + i;
      L.err = p->err;
      L.profile = 0;
      L.any_expr = any_expr;
      L.big_list = nullptr;
      L.big_count = nullptr;
      L.big_ticket = nullptr;
      L.big_cap = 0;
      launch_bucket_step(L, cps * p->sms, p->stream);
      launch_member_splitters(p->d_dev, p->rlist, (int)m, i, p->stream);
      p->launches += 2;
    }
    k_read_back<<<1, 256, 0, p->stream>>>(p->ocount, p->d_oc, 2 * count);
    PC(cudaGetLastError());
    p->launches += 1;
    PC(cudaStreamSynchronize(p->stream));
    for (const auto& e : batch) ab[(size_t)e.second] = p->h_oc[2 * e.second + 1];
  }
  PC(cudaEventRecord(p->ev1, p->stream));
  unsigned err = 0;
  PC(cudaMemcpyAsync(&err, p->err, 4, cudaMemcpyDeviceToHost, p->stream));
  PC(cudaStreamSynchronize(p->stream));
  // the device's time: the graph, plus the recovery (not the wait for the
  // host between the two halves of the step)
  float ms = 0, ms_rec = 0;
  cudaEventElapsedTime(&ms, p->ev0, p->ev_mid);
  if (recovery) cudaEventElapsedTime(&ms_rec, p->ev_rec, p->ev1);
  if (time_elapsed) *time_elapsed = (ms + ms_rec) * 1e-3;
  p->stats.graph_seconds += ms * 1e-3;
  p->stats.recovery_seconds += ms_rec * 1e-3;
  if (err) {
    cudaMemsetAsync(p->err, 0, 4, p->stream);
    return pool_fail(WG_ERR_DEVICE, "device error word 0x%x", err);
  }
  return WG_OK;
}

int wg_pool_step(wg_pool* p, int count, const int* ids, const double* dt, int nleap, double* t0,
                 double* time_elapsed) {
  const int rc = pool_step_begin(p, count, ids, dt, nleap, t0);
  if (rc) return rc;
  return pool_step_end(p, time_elapsed);
}

int wg_pool_step_begin(wg_pool* p, int count, const int* ids, const double* dt, int nleap,
                       double* t0) {
  return pool_step_begin(p, count, ids, dt, nleap, t0);
}

int wg_pool_step_end(wg_pool* p, double* time_elapsed) { return pool_step_end(p, time_elapsed); }

// The device output a download of simulation sim_id reads: while a step is
// running, the output completed before it (the step writes the other pair),
// or the current one of a simulation it does not advance (stepping: the
// simulations of the running step, by id); else the last output.
static int download_source(wg_pool* p, int sim_id,
                           const std::unordered_set<const PoolSim*>* stepping,
                           const PoolSim** so, const double** sx, const double** sv) {
  if (sim_id < 0 || (size_t)sim_id >= p->sims.size() || !p->sims[(size_t)sim_id])
    return pool_fail(WG_ERR_ARG, "no simulation %d in the pool", sim_id);
  PoolSim* s = p->sims[(size_t)sim_id];
  *so = s;
  if (p->pend_active) {
    bool step = false;
    if (stepping) {
      step = stepping->count(s) != 0;
    } else {
      for (PoolSim* a : p->pend_act) step |= a == s;
    }
    *sx = step ? s->done_x : (s->out_valid ? s->x_out : nullptr);
    *sv = step ? s->done_v : (s->out_valid ? s->v_out : nullptr);
    if (!*sx) return pool_fail(WG_ERR_ARG, "simulation %d has no completed output", sim_id);
    return WG_OK;
  }
  if (!s->out_valid) return pool_fail(WG_ERR_ARG, "simulation %d has not been stepped", sim_id);
  *sx = s->x_out;
  *sv = s->v_out;
  return WG_OK;
}

int wg_pool_download(wg_pool* p, int sim_id, double* x, double* v) {
  if (!p) return pool_fail(WG_ERR_ARG, "null pool");
  const PoolSim* s = nullptr;
  const double *sx = nullptr, *sv = nullptr;
  const int rc = download_source(p, sim_id, nullptr, &s, &sx, &sv);
  if (rc) return rc;
  // during a step on a stream of its own
  cudaStream_t st = p->pend_active ? p->dl_stream : p->stream;
  if (x) host_pages_dirty(x, 8 * (size_t)s->n);
  if (v) host_pages_dirty(v, 8 * (size_t)s->n);
  if (x) PC(cudaMemcpyAsync(x, sx, 8 * (size_t)s->n, cudaMemcpyDeviceToHost, st));
  if (v) PC(cudaMemcpyAsync(v, sv, 8 * (size_t)s->n, cudaMemcpyDeviceToHost, st));
  PC(cudaStreamSynchronize(st));
  return WG_OK;
}

int wg_pool_download_many(wg_pool* p, int count, const int* ids, double* x, double* v) {
  if (!p || count < 0 || (count > 0 && !ids)) return pool_fail(WG_ERR_ARG, "bad arguments");
  std::unordered_set<const PoolSim*> stepping;
  if (p->pend_active) stepping.insert(p->pend_act.begin(), p->pend_act.end());
  std::vector<const double*> srcx((size_t)count), srcv((size_t)count);
  std::vector<int64_t> len((size_t)count);
  for (int k = 0; k < count; ++k) {  // every id checked before any copy
    const PoolSim* s = nullptr;
    const int rc = download_source(p, ids[k], p->pend_active ? &stepping : nullptr, &s,
                                   &srcx[(size_t)k], &srcv[(size_t)k]);
    if (rc) return rc;
    len[(size_t)k] = s->n;
  }
  // all copies enqueued back to back, one wait
  cudaStream_t st = p->pend_active ? p->dl_stream : p->stream;
  int64_t off = 0;
  for (int k = 0; k < count; ++k) {
    const size_t bytes = 8 * (size_t)len[(size_t)k];
    if (x) host_pages_dirty(x + off, bytes);
    if (v) host_pages_dirty(v + off, bytes);
    if (x) PC(cudaMemcpyAsync(x + off, srcx[(size_t)k], bytes, cudaMemcpyDeviceToHost, st));
    if (v) PC(cudaMemcpyAsync(v + off, srcv[(size_t)k], bytes, cudaMemcpyDeviceToHost, st));
    off += len[(size_t)k];
  }
  PC(cudaStreamSynchronize(st));
  return WG_OK;
}

int wg_pool_get_stats(wg_pool* p, wg_pool_stats* out) {
  if (!p || !out) return pool_fail(WG_ERR_ARG, "null pool or output");
  *out = p->stats;
  out->launches = p->launches;
  out->graph_builds = p->graph_builds;
  return WG_OK;
}

int wg_pool_info(wg_pool* p, int64_t* used_bytes, int64_t* budget_bytes, int* n_sims,
                 int64_t* launches) {
  if (!p) return pool_fail(WG_ERR_ARG, "null pool");
  int c = 0;
  for (PoolSim* s : p->sims) c += s ? 1 : 0;
  if (used_bytes) *used_bytes = p->used;
  if (budget_bytes) *budget_bytes = p->budget;
  if (n_sims) *n_sims = c;
  if (launches) *launches = p->launches;
  return WG_OK;
}

int wg_pool_destroy(wg_pool* p) {
  if (!p) return WG_OK;
  cudaStreamSynchronize(p->stream);
  for (PoolSim* s : p->sims)
    if (s) {
      cudaFreeAsync(s->mem, p->stream);
      if (s->d_prog) {
        cudaStreamSynchronize(p->stream);
        cudaFree(s->d_prog);
      }
      delete s;
    }
  cudaStreamSynchronize(p->stream);
  if (p->ws) cudaFree(p->ws);
  if (p->bws) cudaFree(p->bws);
  if (p->gexec) cudaGraphExecDestroy(p->gexec);
  free_small(p);
  if (p->ev0) cudaEventDestroy(p->ev0);
  if (p->ev1) cudaEventDestroy(p->ev1);
  if (p->ev_mid) cudaEventDestroy(p->ev_mid);
  if (p->ev_rec) cudaEventDestroy(p->ev_rec);
  if (p->stream) cudaStreamDestroy(p->stream);
  if (p->dl_stream) {
    cudaStreamSynchronize(p->dl_stream);
    cudaStreamDestroy(p->dl_stream);
  }
  delete p;
  return WG_OK;
}

}  // extern "C"
