// wg_api.cu -- the C ABI (include/wendy_gb300.h): simulation handles, the
// per-output step sequence, and the stateless entry points.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <unistd.h>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/wendy_gb300.h"
#include "wg_bucket.cuh"
#include "wg_ext.cuh"
#include "wg_internal.cuh"

using namespace wg;

namespace {

thread_local char g_last_error[512] = "";

}  // namespace

void wg::record_last_error(const char* msg) {
  std::snprintf(g_last_error, sizeof(g_last_error), "%s", msg);
}

namespace {

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

#define WG_CUDA(call)                                                              \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                __LINE__);                                                         \
      return e_ == cudaErrorMemoryAllocation ? WG_ERR_NOMEM : WG_ERR_CUDA;         \
    }                                                                              \
  } while (0)

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

// Most calls a violent overflow sends to the compact path before the bucket
// path is tried again.
constexpr int kMaxBackoff = 8;
constexpr int kPredCalls = 16;

// The bits of a device error word, by name.
std::string device_error_names(unsigned err) {
  static const struct {
    unsigned bit;
    const char* name;
  } names[] = {{DEV_ERR_LOOKBACK_TIMEOUT, "force look-back wait expired"},
               {DEV_ERR_RADIX_TIMEOUT, "radix-sort wait expired"},
               {DEV_ERR_BUCKET_OVERFLOW, "bucket overflow"},
               {DEV_ERR_FIXED_RANGE, "mass outside the fixed-point range"},
               {DEV_ERR_BAD_STATE, "internal check failed"},
               {DEV_ERR_COPY_TIMEOUT, "bulk-copy wait expired"}};
  std::string out;
  for (const auto& e : names)
    if (err & e.bit) {
      if (!out.empty()) out += ", ";
      out += e.name;
    }
  return out.empty() ? "unknown bits" : out;
}

// Host copy of the device conversion: round(m * 2^E) in 128 bits.
u128 host_mass_to_fixed(double m, int E) {
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

int check_ext(int kind, const double* p, int np, ExtSpec* out) {
  char msg[256];
  const int rc = parse_ext(kind, p, np, out, msg, sizeof(msg));
  if (rc) set_error("%s", msg);
  return rc;
}

}  // namespace

struct wg_sim {
  int64_t n = 0;
  int64_t n_tiles = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  void* big = nullptr;       // per-sheet arrays
  void* small = nullptr;     // tables, flags, per-call parameters
  size_t bytes = 0;
  StateTable* table = nullptr;  // device
  StateRef set[2];
  TileRec* recs = nullptr;
  RadixWork radix;
  double* x_out = nullptr;
  double* v_out = nullptr;
  double* a_sorted = nullptr;
  unsigned* err = nullptr;
  int cap = 0;                   // sub-steps the per-call arrays hold
  StepFlags* flags = nullptr;    // [cap + 1]
  unsigned* tickets = nullptr;   // [cap]
  double* t_seq = nullptr;       // [cap]
  unsigned* epochs = nullptr;    // [cap]
  // The reference-layout entry point (wg_nbody_approx_onestep): two output
  // sets (xi in the last sub-step's sorted order, x, v, a in original order)
  // used alternately, its inputs uploaded every call, and the masses of the
  // previous call.
  void* stage = nullptr;
  struct OutSet {
    wg_sheet* xi = nullptr;
    double *x = nullptr, *v = nullptr, *a = nullptr;
  } outs[2];
  int out_last = 0;              // the set returned by the previous call
  wg_sheet* in_xi = nullptr;
  double* in_v = nullptr;
  double* in_m = nullptr;
  double* prev_m = nullptr;
  unsigned* d_diff = nullptr;    // set when this call's inputs differ from those outputs
  cudaStream_t up_stream = nullptr;    // uploads and the comparison
  cudaStream_t down_stream = nullptr;  // downloads of the outputs
  cudaEvent_t ev_up = nullptr;
  // The previous call ended with the sheets in buckets routed for the next
  // opening half drift (resume_ok); a call handed back exactly its outputs
  // (and the same masses and total) continues from there.  After such a
  // call, the next one's sub-steps are enqueued at once (spec_*), assuming
  // the same scalars and the outputs as inputs; the next call checks both.
  bool resume_ok = false;
  double resume_totmass = 0;
  bool spec_enabled = true;
  bool spec_pending = false;
  int spec_set = 0, spec_nleap = 0;
  double spec_dt = 0, spec_t0_in = 0, spec_t0_out = 0, spec_totmass = 0, spec_omega2 = 0;
  ExtSpec spec_ext{};
  double* h_t = nullptr;         // pinned host mirrors
  unsigned* h_ep = nullptr;
  StepFlags* h_flags = nullptr;
  unsigned* h_ab = nullptr;      // page-locked copy of the overflow count and abort word
  // a call enqueued by wg_step_begin and not yet completed by wg_step_end
  bool pend_active = false;
  bool pend_compact = false;     // ... and it runs on the compact path
  double pend_dt = 0;
  int pend_nleap = 0, pend_lay0 = 0, pend_cs0 = 0;
  double pend_pre = 0;           // the opening half drift its first sub-step applies
  // bucketed layout (the fast path of wg_step)
  void* bk = nullptr;
  int64_t nb = 0;        // buckets: ceil(n / target)
  // Slots per bucket in the layouts: kBucketCapBig where the memory allows
  // (a bucket above kBucketCap sheets is then taken in chunks by
  // k_bucket_big), else kBucketCap (a fuller bucket overflows).
  int capg = kBucketCap;
  BigTask* big_list = nullptr;  // [nb]: big buckets of the sub-step in flight
  unsigned* big_counts = nullptr;  // [2 cap]: per sub-step, listed and taken
  double* bx[2] = {nullptr, nullptr};
  double* bv[2] = {nullptr, nullptr};
  double* bm[2] = {nullptr, nullptr};
  int32_t* bi[2] = {nullptr, nullptr};
  unsigned* bcnt[kAggSlots] = {nullptr, nullptr, nullptr};
  unsigned long long* bmass[kAggSlots] = {nullptr, nullptr, nullptr};
  uint64_t* qk[2] = {nullptr, nullptr};
  int32_t* qi[2] = {nullptr, nullptr};
  BucketRec* brecs = nullptr;
  double *ox = nullptr, *ov = nullptr, *om = nullptr;
  int32_t* oi = nullptr;
  unsigned* ocount = nullptr;
  unsigned* abort_word = nullptr;
  unsigned* offs = nullptr;
  double* diag = nullptr;        // energy / momentum sums and their block partials
  int mode = 0;          // 0: compact sorted sets (half drift pending), 1: buckets
  int lay = 0;           // layout holding the sheets in bucket mode
  int qsel = 0;          // splitter array defining the next layout
  int cslot = 0;         // aggregate slot describing layout `lay`
  // Calls a bucket overflow right after a re-sort sends to the compact path
  // (full re-sort + fused force kernel per sub-step), and the next such
  // penalty; the penalty halves after every call the bucket path completes.
  int compact_calls = 0;
  int backoff = 1;
  // Predicted splitters (single simulations with at least 3 buckets): a
  // sample per bucket, its position moved on by two drifts at its bucket's
  // mean velocity, sorted after every sub-step (a radix sort of nb - 1
  // entries) and taken as the splitters of the layout after next.  Turned on
  // for kPredCalls calls whenever a call sees a bucket receive more sheets
  // than one shared-memory pass sorts (flows that outrun the exact quantiles
  // of two sub-steps back: a collapsing cold slab); off otherwise, where the
  // exact quantiles already balance the buckets and the sort would be pure
  // cost.
  int pred_calls = 0;
  void* pmem = nullptr;
  StateTable* ptab = nullptr;   // device table of the two sample sets
  StepFlags* pflag = nullptr;   // device flags with `unsorted` set: the sort always runs
  RadixWork pradix{};
  double pending_dt = 0; // dt of the half drift the bucket layout was routed for
  bool out_valid = false;  // x_out / v_out hold the last call's output
  // Split steps (wg_step_begin): a second pair of output buffers, so that the
  // output completed before a step was begun can be downloaded (on its own
  // stream) while that step runs and writes the other pair.
  double* out2 = nullptr;        // [2n]: x, v of the second pair
  double* x_keep = nullptr;      // the first pair (x_out, v_out as allocated)
  double* v_keep = nullptr;
  double* done_x = nullptr;      // the completed output during a split step
  double* done_v = nullptr;
  cudaStream_t dl_stream = nullptr;
  cudaEvent_t ev_done = nullptr; // that output is materialised
  int grid_bucket = 0;
  BucketTuning tune;             // bucket size, window, sort bits, CTAs per SM
  SheetRec* call_xi = nullptr;    // extra outputs of the reference-shaped entry (this call)
  double* call_a = nullptr;
  SimDev dev{};                  // host copy of the kernel's view of this simulation
  SimDev* d_dev = nullptr;       // device copy (one entry)
  BucketTask* d_tasks = nullptr; // [nb]: (0, b)
  // physics
  uint64_t T_lo = 0, T_hi = 0;
  int E = 0;
  double totmass = 0, omega2 = -1;
  ExtForce ext{};        // the force as the kernels see it
  ExtSpec ext_spec{};    // ... with an expression force's program on the host
  ExprOp* d_prog = nullptr;  // an expression force's program on the device
  unsigned epoch = 1;
  wg_stats st{};
  // a kernel raised the device error word during a call: the state on the
  // device can no longer be trusted, and only wg_destroy is accepted
  bool broken = false;
};

namespace {

// The simulation's external force (an expression force's program is
// copied to the device on the simulation's stream).
int set_force(wg_sim* s, const ExtSpec& ext) {
  if (ext.f.kind == EXT_EXPR && s->d_prog && s->ext.kind == EXT_EXPR && same_ext(ext, s->ext_spec))
    return WG_OK;  // that program is on the device already
  s->ext_spec = ext;
  const cudaError_t e = attach_ext_program(&s->ext_spec, &s->d_prog, s->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("upload of the external-force program failed: %s", cudaGetErrorString(e));
    return WG_ERR_CUDA;
  }
  s->ext = s->ext_spec.f;
  return WG_OK;
}

int alloc_call_arrays(wg_sim* s, int nleap) {
  if (nleap <= s->cap) return WG_OK;
  int cap = 64;
  while (cap < nleap) cap *= 2;
  // Keep which sorted set is current across the re-allocation.
  StateTable t;
  t.cur = s->set[0];
  t.other = s->set[1];
  if (s->table) {
    WG_CUDA(cudaStreamSynchronize(s->stream));
    WG_CUDA(cudaMemcpy(&t, s->table, sizeof(t), cudaMemcpyDeviceToHost));
  }
  if (s->small) cudaFree(s->small);
  if (s->h_t) cudaFreeHost(s->h_t);
  if (s->h_ep) cudaFreeHost(s->h_ep);
  if (s->h_flags) cudaFreeHost(s->h_flags);
  s->small = nullptr;
  s->h_t = nullptr;
  s->h_ep = nullptr;
  s->h_flags = nullptr;
  const size_t b = al(sizeof(StateTable)) + al(64) + al(sizeof(StepFlags) * (cap + 1)) +
                   al(4 * (size_t)cap) + al(8 * (size_t)cap) + al(4 * (size_t)cap) +
                   al(8 * (size_t)cap);
  WG_CUDA(cudaMalloc(&s->small, b));
  char* p = static_cast<char*>(s->small);
  s->table = reinterpret_cast<StateTable*>(p); p += al(sizeof(StateTable));
  s->err = reinterpret_cast<unsigned*>(p); p += al(64);
  s->flags = reinterpret_cast<StepFlags*>(p); p += al(sizeof(StepFlags) * (cap + 1));
  s->tickets = reinterpret_cast<unsigned*>(p); p += al(4 * (size_t)cap);
  s->t_seq = reinterpret_cast<double*>(p); p += al(8 * (size_t)cap);
  s->epochs = reinterpret_cast<unsigned*>(p); p += al(4 * (size_t)cap);
  s->big_counts = reinterpret_cast<unsigned*>(p); p += al(8 * (size_t)cap);
  WG_CUDA(cudaMemsetAsync(s->small, 0, b, s->stream));
  WG_CUDA(cudaMemcpyAsync(s->table, &t, sizeof(t), cudaMemcpyHostToDevice, s->stream));
  WG_CUDA(cudaMallocHost(&s->h_t, 8 * (size_t)cap));
  WG_CUDA(cudaMallocHost(&s->h_ep, 4 * (size_t)cap));
  WG_CUDA(cudaMallocHost(&s->h_flags, sizeof(StepFlags) * (cap + 1)));
  if (!s->h_ab) WG_CUDA(cudaMallocHost(&s->h_ab, 64));
  WG_CUDA(cudaStreamSynchronize(s->stream));
  s->cap = cap;
  return WG_OK;
}

void free_sim(wg_sim* s) {
  if (!s) return;
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->big) cudaFree(s->big);
  if (s->bk) cudaFree(s->bk);
  if (s->pmem) cudaFree(s->pmem);
  if (s->small) cudaFree(s->small);
  if (s->stage) cudaFree(s->stage);
  if (s->h_t) cudaFreeHost(s->h_t);
  if (s->h_ep) cudaFreeHost(s->h_ep);
  if (s->h_flags) cudaFreeHost(s->h_flags);
  if (s->h_ab) cudaFreeHost(s->h_ab);
  if (s->up_stream) cudaStreamSynchronize(s->up_stream);
  if (s->down_stream) cudaStreamSynchronize(s->down_stream);
  if (s->dl_stream) cudaStreamSynchronize(s->dl_stream);
  if (s->out2) cudaFree(s->out2);
  if (s->d_prog) cudaFree(s->d_prog);
  if (s->ev_done) cudaEventDestroy(s->ev_done);
  if (s->dl_stream) cudaStreamDestroy(s->dl_stream);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->ev_up) cudaEventDestroy(s->ev_up);
  if (s->stream) cudaStreamDestroy(s->stream);
  if (s->up_stream) cudaStreamDestroy(s->up_stream);
  if (s->down_stream) cudaStreamDestroy(s->down_stream);
  delete s;
}

// Allocate a simulation for n sheets with the given physics; sheet data is
// uploaded by the caller.
int make_sim(int64_t n, double totmass, double omega2, const ExtSpec& ext, wg_sim** out,
             bool big_buckets = true) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    set_error("no CUDA device visible");
    return WG_ERR_NODEV;
  }
  wg_sim* s = new wg_sim();
  s->n = n;
  s->n_tiles = (n + kForceTile - 1) / kForceTile;
  s->totmass = totmass;
  s->omega2 = omega2;
  s->ext_spec = ext;
  // Fixed-point scale: totmass < 2^eT, so 8 * totmass * 2^E < 2^126.
  if (totmass > 0) {
    int eT = 0;
    std::frexp(totmass, &eT);
    s->E = 123 - eT;
  } else {
    s->E = 0;
  }
  const u128 T = host_mass_to_fixed(totmass, s->E);
  s->T_lo = (uint64_t)T;
  s->T_hi = (uint64_t)(T >> 64);
  int rc = WG_OK;
  auto fail = [&](int code) {
    free_sim(s);
    return code;
  };
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess) {
    set_error("stream/event creation failed: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(WG_ERR_CUDA);
  }
  const size_t nd = al((size_t)n * 8), ni = al((size_t)n * 4);
  const size_t set_b = 3 * nd + ni;
  const size_t recs_b = al(sizeof(TileRec) * (size_t)s->n_tiles);
  const size_t radix_b = radix_bytes(n);
  const size_t out_b = 3 * nd;  // x_out, v_out, a_sorted
  const size_t total = 2 * set_b + recs_b + radix_b + out_b;
  cudaError_t e = cudaMalloc(&s->big, total);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaMalloc of %zu bytes for %lld sheets failed: %s", total, (long long)n,
              cudaGetErrorString(e));
    return fail(WG_ERR_NOMEM);
  }
  s->bytes = total;
  char* p = static_cast<char*>(s->big);
  for (int k = 0; k < 2; ++k) {
    s->set[k].x = reinterpret_cast<double*>(p); p += nd;
    s->set[k].v = reinterpret_cast<double*>(p); p += nd;
    s->set[k].m = reinterpret_cast<double*>(p); p += nd;
    s->set[k].idx = reinterpret_cast<int32_t*>(p); p += ni;
  }
  s->recs = reinterpret_cast<TileRec*>(p); p += recs_b;
  radix_bind(&s->radix, p, n); p += radix_b;
  s->x_out = reinterpret_cast<double*>(p); p += nd;
  s->v_out = reinterpret_cast<double*>(p); p += nd;
  s->a_sorted = reinterpret_cast<double*>(p); p += nd;
  s->x_keep = s->x_out;
  s->v_keep = s->v_out;
  if (cudaMemsetAsync(s->recs, 0, recs_b, s->stream) != cudaSuccess) {
    set_error("memset failed");
    return fail(WG_ERR_CUDA);
  }
  // bucket layout: two layouts of nb buckets x capacity, counts, splitters,
  // look-back records, the overflow list
  s->tune = tuning_for(n);
  s->nb = (n + s->tune.target - 1) / s->tune.target;
  const int64_t nb = s->nb;
  // layouts with room for big buckets where asked for and where the memory
  // allows, else kBucketCap slots per bucket
  size_t slots = 0, bk_b = 0;
  auto bucket_bytes = [&](int capg) {
    slots = (size_t)nb * (size_t)capg;
    bk_b = 2 * (3 * al(slots * 8) + al(slots * 4)) +
           kAggSlots * (al(4 * (size_t)nb) + al(32 * (size_t)nb)) +
           2 * (al(8 * (size_t)(nb + 1)) + al(4 * (size_t)(nb + 1))) +
           al(sizeof(BucketRec) * (size_t)nb) + 3 * nd + ni + al(64) + al(4 * (size_t)nb) +
           al(sizeof(SimDev)) + al(sizeof(BucketTask) * (size_t)nb) +
           al(8 * 4 * (size_t)(kEnergyBlocks + 1)) +
           (capg > kBucketCap ? al(sizeof(BigTask) * (size_t)nb) : 0);
  };
  s->capg = big_buckets ? kBucketCapBig : kBucketCap;
  bucket_bytes(s->capg);
  e = cudaMalloc(&s->bk, bk_b);
  if (e != cudaSuccess && s->capg > kBucketCap) {
    cudaGetLastError();
    s->capg = kBucketCap;
    bucket_bytes(s->capg);
    e = cudaMalloc(&s->bk, bk_b);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaMalloc of %zu bytes for the bucket layout failed: %s", bk_b,
              cudaGetErrorString(e));
    return fail(WG_ERR_NOMEM);
  }
  p = static_cast<char*>(s->bk);
  for (int k = 0; k < 2; ++k) {
    s->bx[k] = reinterpret_cast<double*>(p); p += al(slots * 8);
    s->bv[k] = reinterpret_cast<double*>(p); p += al(slots * 8);
    s->bm[k] = reinterpret_cast<double*>(p); p += al(slots * 8);
    s->bi[k] = reinterpret_cast<int32_t*>(p); p += al(slots * 4);
  }
  for (int k = 0; k < kAggSlots; ++k) {
    s->bcnt[k] = reinterpret_cast<unsigned*>(p); p += al(4 * (size_t)nb);
    s->bmass[k] = reinterpret_cast<unsigned long long*>(p); p += al(32 * (size_t)nb);
  }
  for (int k = 0; k < 2; ++k) {
    s->qk[k] = reinterpret_cast<uint64_t*>(p); p += al(8 * (size_t)(nb + 1));
    s->qi[k] = reinterpret_cast<int32_t*>(p); p += al(4 * (size_t)(nb + 1));
  }
  s->brecs = reinterpret_cast<BucketRec*>(p); p += al(sizeof(BucketRec) * (size_t)nb);
  s->ox = reinterpret_cast<double*>(p); p += nd;
  s->ov = reinterpret_cast<double*>(p); p += nd;
  s->om = reinterpret_cast<double*>(p); p += nd;
  s->oi = reinterpret_cast<int32_t*>(p); p += ni;
  s->ocount = reinterpret_cast<unsigned*>(p);
  s->abort_word = s->ocount + 1;
  p += al(64);
  s->offs = reinterpret_cast<unsigned*>(p); p += al(4 * (size_t)nb);
  s->d_dev = reinterpret_cast<SimDev*>(p); p += al(sizeof(SimDev));
  s->d_tasks = reinterpret_cast<BucketTask*>(p); p += al(sizeof(BucketTask) * (size_t)nb);
  s->diag = reinterpret_cast<double*>(p); p += al(8 * 4 * (size_t)(kEnergyBlocks + 1));
  if (s->capg > kBucketCap) {
    s->big_list = reinterpret_cast<BigTask*>(p);
    p += al(sizeof(BigTask) * (size_t)nb);
  }
  {
    std::vector<BucketTask> tasks((size_t)nb);
    for (int64_t b = 0; b < nb; ++b) tasks[(size_t)b] = BucketTask{0, (int)b};
    if (cudaMemcpy(s->d_tasks, tasks.data(), sizeof(BucketTask) * (size_t)nb,
                   cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error("upload of the bucket task list failed");
      return fail(WG_ERR_CUDA);
    }
  }
  if (big_buckets && nb >= 3) {
    // predicted splitters: two sample sets of nb - 1 entries (SoA as the
    // radix sort wants them), their table, the sort's workspace and flags
    const int64_t m = nb - 1;
    const size_t nd = al(8 * (size_t)m), ni = al(4 * (size_t)m);
    const size_t pb = 2 * (3 * nd + ni) + al(sizeof(StateTable)) + al(sizeof(StepFlags)) +
                      radix_bytes(m);
    if (cudaMalloc(&s->pmem, pb) == cudaSuccess) {
      char* q = static_cast<char*>(s->pmem);
      StateRef set[2];
      for (int k = 0; k < 2; ++k) {
        set[k].x = reinterpret_cast<double*>(q); q += nd;
        set[k].v = reinterpret_cast<double*>(q); q += nd;
        set[k].m = reinterpret_cast<double*>(q); q += nd;
        set[k].idx = reinterpret_cast<int32_t*>(q); q += ni;
      }
      s->ptab = reinterpret_cast<StateTable*>(q); q += al(sizeof(StateTable));
      s->pflag = reinterpret_cast<StepFlags*>(q); q += al(sizeof(StepFlags));
      radix_bind(&s->pradix, q, m);
      StateTable t;
      t.cur = set[0];
      t.other = set[1];
      StepFlags f{};
      f.unsorted = 1u;
      if (cudaMemsetAsync(s->pmem, 0, 2 * (3 * nd + ni), s->stream) != cudaSuccess ||
          cudaMemcpyAsync(s->ptab, &t, sizeof(t), cudaMemcpyHostToDevice, s->stream) !=
              cudaSuccess ||
          cudaMemcpyAsync(s->pflag, &f, sizeof(f), cudaMemcpyHostToDevice, s->stream) !=
              cudaSuccess) {
        set_error("set-up of the predicted splitters failed");
        return fail(WG_ERR_CUDA);
      }
      s->st.device_bytes += (int64_t)pb;
    } else {
      cudaGetLastError();  // no room: the exact quantiles only
      s->pmem = nullptr;
    }
  }
  if (cudaMemsetAsync(s->brecs, 0, sizeof(BucketRec) * (size_t)nb, s->stream) != cudaSuccess ||
      cudaMemsetAsync(s->bcnt[0], 0,
                      static_cast<char*>(static_cast<void*>(s->bmass[kAggSlots - 1])) +
                          al(32 * (size_t)nb) - static_cast<char*>(static_cast<void*>(s->bcnt[0])),
                      s->stream) != cudaSuccess) {
    set_error("memset failed");
    return fail(WG_ERR_CUDA);
  }
  {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    s->grid_bucket = s->tune.ctas_per_sm * sms;
  }
  rc = alloc_call_arrays(s, 64);
  if (rc != WG_OK) return fail(rc);
  rc = set_force(s, ext);
  if (rc != WG_OK) return fail(rc);
  s->st.n = n;
  s->st.device_bytes += (int64_t)(total + bk_b);
  *out = s;
  return WG_OK;
}

int validate_sheets(int64_t n, const double* x, const double* v, const double* m,
                    double totmass) {
  if (n < 1 || n >= (1ll << 30)) {
    set_error("number of sheets %lld outside [1, 2^30)", (long long)n);
    return WG_ERR_ARG;
  }
  if (!x || !v || !m) {
    set_error("null array");
    return WG_ERR_ARG;
  }
  if (!std::isfinite(totmass) || totmass < 0) {
    set_error("totmass must be finite and >= 0");
    return WG_ERR_ARG;
  }
  double mmax = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (!(m[i] >= 0) || !std::isfinite(m[i])) {
      set_error("mass %lld is negative or not finite", (long long)i);
      return WG_ERR_ARG;
    }
    if (!std::isfinite(x[i]) || !std::isfinite(v[i])) {
      set_error("position or velocity %lld is not finite", (long long)i);
      return WG_ERR_ARG;
    }
    if (m[i] > mmax) mmax = m[i];
  }
  if (mmax > 2 * totmass) {
    set_error("a single mass exceeds twice totmass; totmass must be the sum of the masses");
    return WG_ERR_ARG;
  }
  return WG_OK;
}

// Read the device error word and the per-sub-step flags of the last call.
int finish_call(wg_sim* s, int nleap, bool count_sorts = true) {
  unsigned err = 0;
  WG_CUDA(cudaMemcpyAsync(&err, s->err, 4, cudaMemcpyDeviceToHost, s->stream));
  WG_CUDA(cudaMemcpyAsync(s->h_flags, s->flags, sizeof(StepFlags) * (nleap + 1),
                          cudaMemcpyDeviceToHost, s->stream));
  WG_CUDA(cudaStreamSynchronize(s->stream));
  for (int i = 0; i < nleap && count_sorts; ++i) {
    if (s->h_flags[i].unsorted)
      s->st.sorts_full++;
    else
      s->st.sorts_skipped++;
  }
  s->st.substeps += nleap;
  unsigned mc = 0;
  for (int i = 1; i <= nleap; ++i) mc = s->h_flags[i].max_cnt > mc ? s->h_flags[i].max_cnt : mc;
  s->st.last_max_count = mc;
  // predicted splitters for the next kPredCalls calls after a bucket outgrew
  // one shared-memory pass; counted down by the bucket-path calls that stay
  // within it (calls on the compact path see no buckets and count nothing)
  if (s->ptab && mc > (unsigned)kBucketCap)
    s->pred_calls = kPredCalls;
  else if (s->pred_calls > 0 && mc > 0)
    --s->pred_calls;
  if (s->big_list && nleap > 0) {
    // big buckets listed per sub-step (of the launches that ran last for each)
    std::vector<unsigned> bc(2 * (size_t)nleap);
    if (cudaMemcpy(bc.data(), s->big_counts, 8 * (size_t)nleap, cudaMemcpyDeviceToHost) ==
        cudaSuccess)
      for (int i = 0; i < nleap; ++i) s->st.big_buckets += bc[2 * (size_t)i];
    else
      cudaGetLastError();
  }
  if (err) {
    set_error("device error word 0x%x (%s); the simulation's state is lost, destroy it", err,
              device_error_names(err).c_str());
    cudaMemsetAsync(s->err, 0, 4, s->stream);
    s->broken = true;
    return WG_ERR_DEVICE;
  }
  return WG_OK;
}

static_assert(kMaxLeap == WG_MAX_LEAP, "sub-step limit of the C header");

// Epochs of the next `count` sub-steps into s->h_ep.  They stay within
// [1, kEpochLimit]: before passing it every look-back record is cleared and
// the epochs restart at 1.
int take_epochs(wg_sim* s, int count) {
  if (s->epoch + (unsigned)count > kEpochLimit) {
    WG_CUDA(cudaMemsetAsync(s->recs, 0, sizeof(TileRec) * (size_t)s->n_tiles, s->stream));
    WG_CUDA(cudaMemsetAsync(s->brecs, 0, sizeof(BucketRec) * (size_t)s->nb, s->stream));
    s->epoch = 1;
  }
  for (int i = 0; i < count; ++i) s->h_ep[i] = s->epoch + (unsigned)i;
  s->epoch += (unsigned)count;
  return WG_OK;
}

// Enqueue one output interval: half drift, nleap x [sort, force/kick/drift].
// The last force evaluation's accelerations go to s->a_sorted when
// want_accel is set.  t_seq must be in s->h_t already.
int enqueue_step(wg_sim* s, double dt, int nleap, bool want_accel, double dt_last_drift) {
  int rc = take_epochs(s, nleap);
  if (rc) return rc;
  WG_CUDA(cudaMemcpyAsync(s->t_seq, s->h_t, 8 * (size_t)nleap, cudaMemcpyHostToDevice, s->stream));
  WG_CUDA(cudaMemcpyAsync(s->epochs, s->h_ep, 4 * (size_t)nleap, cudaMemcpyHostToDevice, s->stream));
  WG_CUDA(cudaMemsetAsync(s->flags, 0, sizeof(StepFlags) * (nleap + 1), s->stream));
  WG_CUDA(cudaMemsetAsync(s->tickets, 0, 4 * (size_t)nleap, s->stream));
  launch_drift(s->table, s->n, dt / 2., &s->flags[0], s->stream);
  s->st.launches += 1 + (int64_t)nleap * (1 + kRadixLaunches);
  ForceArgs a;
  a.table = s->table;
  a.n = s->n;
  a.T_lo = s->T_lo;
  a.T_hi = s->T_hi;
  a.E = s->E;
  a.has_omega = s->omega2 >= 0;
  a.omega2 = s->omega2;
  a.ext = s->ext;
  a.t_seq = s->t_seq;
  a.epochs = s->epochs;
  a.recs = s->recs;
  a.err = s->err;
  for (int i = 0; i < nleap; ++i) {
    radix_sort_state(s->table, s->n, &s->radix, &s->flags[i], s->err, s->stream);
    a.sub = i;
    a.dt_kick = dt;
    a.dt_drift = (i == nleap - 1) ? dt_last_drift : dt;
    a.a_out = (want_accel && i == nleap - 1) ? s->a_sorted : nullptr;
    a.ticket = s->tickets + i;
    a.flag_out = &s->flags[i + 1];
    launch_force(a, s->n_tiles, s->stream);
  }
  WG_CUDA(cudaGetLastError());
  return WG_OK;
}

// Bucket layout `lay` with the counts of aggregate slot `cslot` (+ overflow
// list) -> compact, unsorted sheets in the current sorted-state set.
void bucket_to_compact(wg_sim* s, int lay, int cslot) {
  launch_compact(s->table, s->nb, s->capg, s->bx[lay], s->bv[lay], s->bm[lay], s->bi[lay],
                 s->bcnt[cslot],
                 s->offs, s->ox, s->ov, s->om, s->oi, s->ocount, s->n, s->stream);
  s->st.launches += 2;
}

// The kernel's view of this simulation for the coming call.
void fill_dev(wg_sim* s, double dt, double pre) {
  SimDev& d = s->dev;
  for (int k = 0; k < 2; ++k) {
    d.bx[k] = s->bx[k];
    d.bv[k] = s->bv[k];
    d.bm[k] = s->bm[k];
    d.bi[k] = s->bi[k];
    d.qk[k] = s->qk[k];
    d.qi[k] = s->qi[k];
  }
  for (int k = 0; k < kAggSlots; ++k) {
    d.bcnt[k] = s->bcnt[k];
    d.bmass[k] = s->bmass[k];
  }
  d.recs = s->brecs;
  d.ox = s->ox;
  d.ov = s->ov;
  d.om = s->om;
  d.oi = s->oi;
  d.ocount = s->ocount;
  d.x_out = s->x_out;
  d.v_out = s->v_out;
  d.xi_out = s->call_xi;
  d.a_out = s->call_a;
  // the compact sets are free while the sheets live in buckets: the last
  // sub-step's (x, v, a) records go there (56 B/sheet >= 32)
  d.rec_out = reinterpret_cast<OutRec*>(s->set[0].x);
  d.flags = s->flags;
  d.t_seq = s->t_seq;
  d.n = s->n;
  d.nb = s->nb;
  d.target = s->tune.target;
  d.capg = s->capg;
  d.window = s->tune.window;
  d.sort_bits = s->tune.sort_bits;
  d.T_lo = s->T_lo;
  d.T_hi = s->T_hi;
  d.E = s->E;
  d.has_omega = s->omega2 >= 0;
  d.omega2 = s->omega2;
  d.ext = s->ext;
  d.dt = dt;
  d.pre_dt = pre;
  d.lay0 = s->lay;
  d.qsel0 = s->qsel;
  d.cs0 = s->cslot;
  d.ptab = s->pred_calls > 0 ? s->ptab : nullptr;
}

StepLaunch step_launch(wg_sim* s, int i, int nleap, int profile) {
  StepLaunch L;
  L.sims = s->d_dev;
  L.tasks = s->d_tasks;
  L.ntasks = (int)s->nb;
  L.sub = i;
  L.nleap = nleap;
  L.epochs = s->epochs;
  L.ticket = s->tickets + i;
  L.err = s->err;
  L.profile = profile;
  L.any_expr = s->ext.kind == EXT_EXPR;
  L.big_list = s->big_list;
  L.big_count = s->big_counts + 2 * i;
  L.big_ticket = s->big_counts + 2 * i + 1;
  L.big_cap = s->big_list ? (unsigned)s->nb : 0u;
  return L;
}

// One sub-step on the bucket path: the fused kernel, then (simulations whose
// buckets can outgrow shared memory) the big buckets it listed.
void launch_substep(wg_sim* s, int i, int nleap, int profile) {
  const StepLaunch L = step_launch(s, i, nleap, profile);
  launch_bucket_step(L, s->grid_bucket, s->stream);
  if (s->big_list) launch_bucket_big(L, s->grid_bucket, s->stream);
  if (s->dev.ptab) {
    // the samples this sub-step wrote, sorted, become the splitters it
    // would have published (those of the layout after next)
    const int q = 1 - ((s->dev.qsel0 + i) & 1);
    radix_sort_state(s->ptab, s->nb - 1, &s->pradix, s->pflag, s->err, s->stream);
    launch_samples_to_splitters(s->ptab, s->nb - 1, s->qk[q], s->qi[q], s->stream);
    s->st.launches += kRadixLaunches + 1;
    if (!profile) s->st.substeps_predicted += 1;
  }
}

void fill_times(wg_sim* s, double dt, int nleap, double* t0) {
  double t = t0 ? *t0 : 0.0;
  for (int i = 0; i < nleap; ++i) {
    s->h_t[i] = t;
    if (s->ext.kind != EXT_NONE) t += dt;  // wendy/wendy.c:403-404,409-410
  }
  if (t0) *t0 = t;
}

// Cache of one simulation for the stateless reference-shaped entry point.
std::mutex g_cache_mu;
wg_sim* g_cache = nullptr;

// Whether the drop-in's inputs are, bit for bit, the previous call's
// outputs (xi, v) and masses: then the resident bucket state is the state
// they describe.
__global__ void k_inputs_differ(int64_t n, const wg_sheet* xi, const wg_sheet* xi_prev,
                                const double* v, const double* v_prev, const double* m,
                                const double* m_prev, unsigned* diff) {
  bool d = false;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    d |= xi[i].idx != xi_prev[i].idx ||
         __double_as_longlong(xi[i].val) != __double_as_longlong(xi_prev[i].val) ||
         __double_as_longlong(v[i]) != __double_as_longlong(v_prev[i]) ||
         __double_as_longlong(m[i]) != __double_as_longlong(m_prev[i]);
  }
  if (__syncthreads_or(d) && threadIdx.x == 0) atomicOr(diff, 1u);
}

__global__ void k_load_sheets(StateTable* table, int64_t n, const wg_sheet* xi, const double* v,
                              const double* m) {
  const StateRef st = table->cur;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int32_t j = xi[i].idx;
    st.idx[i] = j;
    st.x[i] = xi[i].val;
    st.v[i] = v[j];
    st.m[i] = m[j];
  }
}

__global__ void k_store_sheets(const StateTable* table, int64_t n, wg_sheet* xi) {
  const StateRef st = table->cur;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    wg_sheet r;
    r.idx = st.idx[i];
    r.val = st.x[i];
    xi[i] = r;
  }
}

// The sorted sheets as the reference's (idx, val) records, for the drop-in's xi.
void store_sheets(const StateTable* table, int64_t n, wg_sheet* xi, cudaStream_t st) {
  k_store_sheets<<<152 * 8, 256, 0, st>>>(table, n, xi);
}


}  // namespace

void wg::host_pages_dirty(void* p, size_t bytes) {
  static const size_t page = [] {
    const long ps = sysconf(_SC_PAGESIZE);
    return ps > 0 ? (size_t)ps : (size_t)4096;
  }();
  if (!p || !bytes) return;
  volatile char* c = static_cast<volatile char*>(p);
  c[0] = 0;
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  for (size_t o = (page - a % page) % page; o < bytes; o += page) c[o] = 0;
}

extern "C" {

int wg_version(void) { return 100; }

const char* wg_status_string(int status) {
  switch (status) {
    case WG_OK: return "ok";
    case WG_ERR_ARG: return "invalid argument";
    case WG_ERR_CUDA: return "CUDA runtime error";
    case WG_ERR_NOMEM: return "device memory allocation failed";
    case WG_ERR_DEVICE: return "device-side error (bounded wait expired or internal check)";
    case WG_ERR_EXT: return "unknown external force or bad parameters";
    case WG_ERR_BUDGET: return "memory budget exceeded";
    case WG_ERR_NODEV: return "no CUDA device";
    default: return "unknown status";
  }
}

const char* wg_last_error(void) { return g_last_error; }

int wg_device_info(int* sm_count, int64_t* free_bytes, int64_t* total_bytes) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    set_error("no CUDA device visible");
    return WG_ERR_NODEV;
  }
  int dev = 0;
  WG_CUDA(cudaGetDevice(&dev));
  if (sm_count) WG_CUDA(cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev));
  size_t fr = 0, tot = 0;
  WG_CUDA(cudaMemGetInfo(&fr, &tot));
  if (free_bytes) *free_bytes = (int64_t)fr;
  if (total_bytes) *total_bytes = (int64_t)tot;
  return WG_OK;
}

int wg_create(int64_t n, const double* x, const double* v, const double* m, double totmass,
              double omega2, int ext_kind, const double* ext_params, int n_ext_params,
              wg_sim** out) {
  if (!out) {
    set_error("null output handle");
    return WG_ERR_ARG;
  }
  *out = nullptr;
  int rc = validate_sheets(n, x, v, m, totmass);
  if (rc) return rc;
  if (!std::isfinite(omega2)) {
    set_error("omega2 must be finite");
    return WG_ERR_ARG;
  }
  ExtSpec ext;
  rc = check_ext(ext_kind, ext_params, n_ext_params, &ext);
  if (rc) return rc;
  wg_sim* s = nullptr;
  rc = make_sim(n, totmass, omega2, ext, &s);
  if (rc) return rc;
  const StateRef c = s->set[0];
  auto up = [&](void* d, const void* h, size_t b) {
    return cudaMemcpyAsync(d, h, b, cudaMemcpyHostToDevice, s->stream);
  };
  if (up(c.x, x, 8 * n) != cudaSuccess || up(c.v, v, 8 * n) != cudaSuccess ||
      up(c.m, m, 8 * n) != cudaSuccess) {
    set_error("upload failed: %s", cudaGetErrorString(cudaGetLastError()));
    free_sim(s);
    return WG_ERR_CUDA;
  }
  launch_init_state(s->table, n, s->stream);
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) {
    set_error("initialisation failed: %s", cudaGetErrorString(cudaGetLastError()));
    free_sim(s);
    return WG_ERR_CUDA;
  }
  *out = s;
  return WG_OK;
}

// Sub-steps from .. nleap - 1 of the current call on the compact path: the
// compact sets hold the sheets at the start of sub-step `from`; each sub-step
// re-sorts them in full and runs the fused force / kick / drift kernel.  The
// call's extra outputs (a, xi) come from the last one.  Waits.
static int compact_continue(wg_sim* s, double dt, int nleap, int from) {
  ForceArgs f;
  f.table = s->table;
  f.n = s->n;
  f.T_lo = s->T_lo;
  f.T_hi = s->T_hi;
  f.E = s->E;
  f.has_omega = s->omega2 >= 0;
  f.omega2 = s->omega2;
  f.ext = s->ext;
  f.t_seq = s->t_seq;
  f.epochs = s->epochs;
  f.recs = s->recs;
  f.err = s->err;
  // the bucket launches of these sub-steps consumed their tickets
  WG_CUDA(cudaMemsetAsync(s->tickets + from, 0, 4 * (size_t)(nleap - from), s->stream));
  for (int i = from; i < nleap; ++i) {
    WG_CUDA(cudaMemsetAsync(&s->flags[i].unsorted, 1, sizeof(unsigned), s->stream));
    radix_sort_state(s->table, s->n, &s->radix, &s->flags[i], s->err, s->stream);
    f.sub = i;
    f.dt_kick = dt;
    f.dt_drift = (i == nleap - 1) ? dt / 2. : dt;
    f.ticket = s->tickets + i;
    f.flag_out = &s->flags[i + 1];
    f.a_out = (i == nleap - 1 && s->call_a) ? s->a_sorted : nullptr;
    launch_force(f, s->n_tiles, s->stream);
  }
  if (s->call_a) launch_scatter_accel(s->table, s->n, s->a_sorted, s->call_a, s->stream);
  if (s->call_xi) store_sheets(s->table, s->n, reinterpret_cast<wg_sheet*>(s->call_xi), s->stream);
  s->st.launches += (int64_t)(nleap - from) * (1 + kRadixLaunches);
  s->st.substeps_compact += nleap - from;
  WG_CUDA(cudaStreamSynchronize(s->stream));
  return WG_OK;
}

// Enqueue one output interval on the simulation's stream (returns without
// waiting); run_call_end completes it.
static int run_call_begin(wg_sim* s, double dt, int nleap, double* t0, bool record_start) {
  int rc = alloc_call_arrays(s, nleap);
  if (rc) return rc;
  fill_times(s, dt, nleap, t0);
  if (s->compact_calls > 0) {
    // a recent overflow right after a re-sort: this call runs on the compact
    // path (full re-sort + fused force kernel per sub-step)
    if (record_start) WG_CUDA(cudaEventRecord(s->ev0, s->stream));
    if (s->mode == 1) {
      WG_CUDA(cudaMemsetAsync(s->ocount, 0, 16, s->stream));
      bucket_to_compact(s, s->lay, s->cslot);
      s->mode = 0;
    }
    rc = enqueue_step(s, dt, nleap, s->call_a != nullptr, dt / 2.);
    if (rc) return rc;
    WG_CUDA(cudaMemsetAsync(s->big_counts, 0, 8 * (size_t)nleap, s->stream));
    s->st.substeps_compact += nleap;
    if (s->call_a) launch_scatter_accel(s->table, s->n, s->a_sorted, s->call_a, s->stream);
    if (s->call_xi)
      store_sheets(s->table, s->n, reinterpret_cast<wg_sheet*>(s->call_xi), s->stream);
    s->compact_calls--;
    s->pend_active = true;
    s->pend_compact = true;
    s->pend_dt = dt;
    s->pend_nleap = nleap;
    return WG_OK;
  }
  rc = take_epochs(s, nleap);
  if (rc) return rc;
  if (record_start) WG_CUDA(cudaEventRecord(s->ev0, s->stream));
  WG_CUDA(cudaMemcpyAsync(s->t_seq, s->h_t, 8 * (size_t)nleap, cudaMemcpyHostToDevice, s->stream));
  WG_CUDA(cudaMemcpyAsync(s->epochs, s->h_ep, 4 * (size_t)nleap, cudaMemcpyHostToDevice, s->stream));
  WG_CUDA(cudaMemsetAsync(s->flags, 0, sizeof(StepFlags) * (nleap + 1), s->stream));
  WG_CUDA(cudaMemsetAsync(s->tickets, 0, 4 * (size_t)nleap, s->stream));
  WG_CUDA(cudaMemsetAsync(s->big_counts, 0, 8 * (size_t)nleap, s->stream));
  // overflow count, abort word and redo word
  WG_CUDA(cudaMemsetAsync(s->ocount, 0, 16, s->stream));
  if (s->mode == 1 && dt != s->pending_dt) {
    // routed for another dt: back to compact state, the half drift still pending
    bucket_to_compact(s, s->lay, s->cslot);
    s->mode = 0;
  }
  double pre = 0.0;
  if (s->mode == 0) {
    launch_drift(s->table, s->n, dt / 2., &s->flags[0], s->stream);
    radix_sort_state(s->table, s->n, &s->radix, &s->flags[0], s->err, s->stream);
    s->lay = 0;
    s->qsel = 0;
    s->cslot = 0;
    launch_bucketize(s->table, s->n, s->tune.target, s->nb, s->capg, s->E, s->bx[0], s->bv[0],
                     s->bm[0],
                     s->bi[0], s->bcnt, s->bmass, s->qk[0], s->qi[0], s->stream);
    s->st.launches += 2 + kRadixLaunches;
    s->st.sorts_full += 1;
  } else {
    pre = dt / 2.;
  }
  const int lay0 = s->lay, cs0 = s->cslot;
  s->pend_pre = pre;
  fill_dev(s, dt, pre);
  WG_CUDA(cudaMemcpyAsync(s->d_dev, &s->dev, sizeof(SimDev), cudaMemcpyHostToDevice, s->stream));
  for (int i = 0; i < nleap; ++i) launch_substep(s, i, nleap, 0);
  launch_split_out(s->dev.rec_out, s->n, s->x_out, s->v_out, s->call_a, s->stream);
  s->lay = (lay0 + nleap) & 1;
  s->qsel = (s->qsel + nleap) & 1;
  s->cslot = (cs0 + nleap) % kAggSlots;
  s->st.launches += nleap + 1;
  WG_CUDA(cudaGetLastError());
  WG_CUDA(cudaMemcpyAsync(s->h_ab, s->ocount, 16, cudaMemcpyDeviceToHost, s->stream));
  WG_CUDA(cudaMemcpyAsync(s->h_flags, s->flags, sizeof(StepFlags) * (nleap + 1),
                          cudaMemcpyDeviceToHost, s->stream));
  s->pend_active = true;
  s->pend_dt = dt;
  s->pend_nleap = nleap;
  s->pend_lay0 = lay0;
  s->pend_cs0 = cs0;
  return WG_OK;
}

// Wait for the enqueued call, finish it on the compact path if a sub-step
// overflowed a bucket, and report its device time.
static int run_call_end(wg_sim* s, double* time_elapsed) {
  if (!s->pend_active) {
    set_error("no step in flight");
    return WG_ERR_ARG;
  }
  s->pend_active = false;
  const double dt = s->pend_dt;
  const int nleap = s->pend_nleap;
  int rc = WG_OK;
  if (s->pend_compact) {
    s->pend_compact = false;
    WG_CUDA(cudaEventRecord(s->ev1, s->stream));
    rc = finish_call(s, nleap, true);  // waits
    s->out_valid = false;  // the sheets are sorted, x_out is stale
    s->mode = 0;
    s->pending_dt = dt;
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    if (time_elapsed) *time_elapsed = ms * 1e-3;
    double vmax;
    std::memcpy(&vmax, &s->h_flags[nleap].max_v, 8);
    s->st.last_max_disp = vmax * std::fabs(dt / 2.);
    return rc;
  }
  int lay0 = s->pend_lay0, cs0 = s->pend_cs0, qs0 = (s->qsel - nleap) & 1;
  WG_CUDA(cudaStreamSynchronize(s->stream));
  s->out_valid = true;
  s->mode = 1;
  s->pending_dt = dt;
  int64_t window_steps = 0;
  int from = 0;  // first sub-step of the current run of bucket launches
  bool clean = true;
  for (;;) {
    const unsigned ab = s->h_ab[1], redo = s->h_ab[2];
    if (ab == 0 && redo == 0) {
      window_steps += nleap - from;
      break;
    }
    clean = false;
    int k, resume;
    if (redo) {
      // sub-step k met a big bucket it could not cut into chunks: the layout
      // it read is intact, its own output is dropped.  Re-sort that layout
      // and run the sub-steps from k again.
      k = (int)redo - 1;
      window_steps += k - from;
      s->st.sorts_full += 1;
      WG_CUDA(cudaMemsetAsync(s->ocount, 0, 16, s->stream));
      bucket_to_compact(s, (lay0 + k) & 1, (cs0 + k) % kAggSlots);
      // a call's first sub-step applies the opening half drift while loading
      if (k == 0 && s->pend_pre != 0.0)
        launch_drift(s->table, s->n, s->pend_pre, nullptr, s->stream);
      resume = k;
    } else {
      // sub-step k overflowed a bucket: its sheets are complete in the layout
      // it wrote plus the overflow list.  Re-sort them once, lay out fresh
      // buckets (exact quantiles) and restart the remaining sub-steps on the
      // bucket path; a last sub-step has already written every output.
      k = (int)ab - 1;
      window_steps += k + 1 - from;
      s->st.sorts_full += 1;
      bucket_to_compact(s, (lay0 + k + 1) & 1, (cs0 + k + 1) % kAggSlots);
      if (k == nleap - 1) {
        s->mode = 0;  // the next call re-sorts
        break;
      }
      resume = k + 1;
    }
    if (from > 0 && k < from + 2) {
      // failed again right after a re-sort: the buckets cannot follow this
      // flow for now.  Finish the call on the compact path and keep the next
      // calls there (back-off doubling up to kMaxBackoff calls).
      compact_continue(s, dt, nleap, resume);
      s->mode = 0;
      s->out_valid = false;
      s->compact_calls = s->backoff;
      s->backoff = s->backoff < kMaxBackoff ? 2 * s->backoff : kMaxBackoff;
      break;
    }
    from = resume;
    // a bucket outgrew its layout: the restarted sub-steps predict their
    // splitters already (not only the calls after this one)
    if (s->ptab) s->pred_calls = kPredCalls;
    // fresh look-back epochs for the sub-steps that run again (a redone
    // sub-step published records under its old epoch)
    rc = take_epochs(s, nleap - from);
    if (rc) return rc;
    WG_CUDA(cudaMemcpyAsync(s->epochs + from, s->h_ep, 4 * (size_t)(nleap - from),
                            cudaMemcpyHostToDevice, s->stream));
    WG_CUDA(cudaMemsetAsync(&s->flags[from].unsorted, 1, sizeof(unsigned), s->stream));
    radix_sort_state(s->table, s->n, &s->radix, &s->flags[from], s->err, s->stream);
    launch_bucketize(s->table, s->n, s->tune.target, s->nb, s->capg, s->E, s->bx[0], s->bv[0],
                     s->bm[0],
                     s->bi[0], s->bcnt, s->bmass, s->qk[0], s->qi[0], s->stream);
    // sub-step `from` reads layout 0, aggregate slot 0 and routes by splitter set 0
    lay0 = from & 1;
    qs0 = from & 1;
    cs0 = (kAggSlots - from % kAggSlots) % kAggSlots;
    s->lay = lay0;
    s->qsel = qs0;
    s->cslot = cs0;
    fill_dev(s, dt, 0.0);
    WG_CUDA(cudaMemcpyAsync(s->d_dev, &s->dev, sizeof(SimDev), cudaMemcpyHostToDevice,
                            s->stream));
    WG_CUDA(cudaMemsetAsync(s->ocount, 0, 16, s->stream));
    // the skipped launches of these sub-steps consumed their tickets
    WG_CUDA(cudaMemsetAsync(s->tickets + from, 0, 4 * (size_t)(nleap - from), s->stream));
    WG_CUDA(cudaMemsetAsync(s->big_counts + 2 * from, 0, 8 * (size_t)(nleap - from),
                            s->stream));
    for (int i = from; i < nleap; ++i) launch_substep(s, i, nleap, 0);
    launch_split_out(s->dev.rec_out, s->n, s->x_out, s->v_out, s->call_a, s->stream);
    s->lay = (lay0 + nleap) & 1;
    s->qsel = (qs0 + nleap) & 1;
    s->cslot = (cs0 + nleap) % kAggSlots;
    s->st.launches += 4 + kRadixLaunches + (nleap - from);
    WG_CUDA(cudaGetLastError());
    WG_CUDA(cudaMemcpyAsync(s->h_ab, s->ocount, 16, cudaMemcpyDeviceToHost, s->stream));
    WG_CUDA(cudaMemcpyAsync(s->h_flags, s->flags, sizeof(StepFlags) * (nleap + 1),
                            cudaMemcpyDeviceToHost, s->stream));
    WG_CUDA(cudaStreamSynchronize(s->stream));
  }
  s->st.sorts_window += window_steps;
  if (clean && s->backoff > 1) s->backoff /= 2;
  WG_CUDA(cudaEventRecord(s->ev1, s->stream));
  rc = finish_call(s, nleap, false);
  float ms = 0;
  cudaEventElapsedTime(&ms, s->ev0, s->ev1);
  if (time_elapsed) *time_elapsed = ms * 1e-3;
  const double vmax = [&] {
    double d;
    unsigned long long b = s->h_flags[nleap].max_v;
    std::memcpy(&d, &b, 8);
    return d;
  }();
  s->st.last_max_disp = vmax * std::fabs(dt / 2.);
  return rc;
}

static int run_call(wg_sim* s, double dt, int nleap, double* t0, double* time_elapsed,
                    bool record_start) {
  const int rc = run_call_begin(s, dt, nleap, t0, record_start);
  if (rc) return rc;
  return run_call_end(s, time_elapsed);
}

// Entries other than wg_step_end and wg_destroy refuse a simulation with a
// step in flight.
static int check_idle(wg_sim* s) {
  if (!s) {
    set_error("null simulation");
    return WG_ERR_ARG;
  }
  if (s->pend_active) {
    set_error("a step is in flight: call wg_step_end first");
    return WG_ERR_ARG;
  }
  if (s->broken) {
    set_error("an earlier call on this simulation raised a device error; destroy it");
    return WG_ERR_DEVICE;
  }
  return WG_OK;
}

int wg_step(wg_sim* s, double dt, int nleap, double* t0, double* time_elapsed) {
  int rc = check_idle(s);
  if (rc) return rc;
  if (nleap < 1 || nleap > kMaxLeap || !std::isfinite(dt)) {
    set_error("nleap must be >= 1 and dt finite");
    return WG_ERR_ARG;
  }
  s->call_xi = nullptr;
  s->call_a = nullptr;
  return run_call(s, dt, nleap, t0, time_elapsed, true);
}

int wg_step_begin(wg_sim* s, double dt, int nleap, double* t0) {
  int rc = check_idle(s);
  if (rc) return rc;
  if (nleap < 1 || nleap > kMaxLeap || !std::isfinite(dt)) {
    set_error("nleap must be >= 1 and dt finite");
    return WG_ERR_ARG;
  }
  s->call_xi = nullptr;
  s->call_a = nullptr;
  if (!s->out2) {
    WG_CUDA(cudaMalloc(&s->out2, 16 * (size_t)s->n));
    WG_CUDA(cudaStreamCreateWithFlags(&s->dl_stream, cudaStreamNonBlocking));
    WG_CUDA(cudaEventCreateWithFlags(&s->ev_done, cudaEventDisableTiming));
    s->st.device_bytes += 16 * s->n;
  }
  // the output completed so far stays downloadable while this step runs:
  // materialised now if the last call left it in the sorted state, then the
  // step writes the other pair of buffers
  s->done_x = nullptr;
  s->done_v = nullptr;
  if (s->st.substeps > 0) {
    if (!s->out_valid) {
      launch_desort(s->table, s->n, s->x_out, s->v_out, s->stream);
      s->out_valid = true;
    }
    WG_CUDA(cudaEventRecord(s->ev_done, s->stream));
    s->done_x = s->x_out;
    s->done_v = s->v_out;
  }
  double* const other_x = s->x_out == s->out2 ? s->x_keep : s->out2;
  s->x_out = other_x;
  s->v_out = other_x == s->out2 ? s->out2 + s->n : s->v_keep;
  return run_call_begin(s, dt, nleap, t0, true);
}

int wg_step_end(wg_sim* s, double* time_elapsed) {
  if (!s) {
    set_error("null simulation");
    return WG_ERR_ARG;
  }
  return run_call_end(s, time_elapsed);
}

int wg_download(wg_sim* s, double* x, double* v) {
  if (s && s->pend_active && s->done_x) {
    // a split step is running: the output completed before it, on its own stream
    cudaStream_t d = s->dl_stream;
    if (x) host_pages_dirty(x, 8 * (size_t)s->n);
    if (v) host_pages_dirty(v, 8 * (size_t)s->n);
    WG_CUDA(cudaStreamWaitEvent(d, s->ev_done, 0));
    if (x) WG_CUDA(cudaMemcpyAsync(x, s->done_x, 8 * s->n, cudaMemcpyDeviceToHost, d));
    if (v) WG_CUDA(cudaMemcpyAsync(v, s->done_v, 8 * s->n, cudaMemcpyDeviceToHost, d));
    WG_CUDA(cudaStreamSynchronize(d));
    return WG_OK;
  }
  int rc = check_idle(s);
  if (rc) return rc;
  if (!s->out_valid) {
    launch_desort(s->table, s->n, s->x_out, s->v_out, s->stream);
    s->out_valid = true;
  }
  if (x) host_pages_dirty(x, 8 * (size_t)s->n);
  if (v) host_pages_dirty(v, 8 * (size_t)s->n);
  if (x) WG_CUDA(cudaMemcpyAsync(x, s->x_out, 8 * s->n, cudaMemcpyDeviceToHost, s->stream));
  if (v) WG_CUDA(cudaMemcpyAsync(v, s->v_out, 8 * s->n, cudaMemcpyDeviceToHost, s->stream));
  WG_CUDA(cudaStreamSynchronize(s->stream));
  return WG_OK;
}

int wg_get_stats(wg_sim* s, wg_stats* out) {
  if (!s || !out) {
    set_error("null argument");
    return WG_ERR_ARG;
  }
  *out = s->st;
  return WG_OK;
}

int wg_destroy(wg_sim* s) {
  free_sim(s);
  return WG_OK;
}

int wg_profile(wg_sim* s, int what, int reps, double* avg_seconds) {
  const int rc0 = check_idle(s);
  if (rc0) return rc0;
  if (reps < 1 || reps > kMaxLeap || !avg_seconds ||
      (what != WG_PROF_FORCE && what != WG_PROF_SORT && what != WG_PROF_BUCKET)) {
    set_error("bad arguments to wg_profile");
    return WG_ERR_ARG;
  }
  if (what == WG_PROF_BUCKET && s->mode != 1) {
    set_error("wg_profile(WG_PROF_BUCKET) needs the bucket layout: run wg_step first");
    return WG_ERR_ARG;
  }
  // the force and sort kernels run on the compact sets, which hold other
  // data while the sheets live in buckets: hand the current state back to
  // them first (the next wg_step re-sorts and re-buckets, as after wg_energy)
  if (what != WG_PROF_BUCKET && s->mode == 1) {
    bucket_to_compact(s, s->lay, s->cslot);
    s->mode = 0;
  }
  int rc = alloc_call_arrays(s, reps);
  if (rc) return rc;
  for (int i = 0; i < reps; ++i) s->h_t[i] = 0.0;
  rc = take_epochs(s, reps);
  if (rc) return rc;
  WG_CUDA(cudaMemcpyAsync(s->t_seq, s->h_t, 8 * (size_t)reps, cudaMemcpyHostToDevice, s->stream));
  WG_CUDA(cudaMemcpyAsync(s->epochs, s->h_ep, 4 * (size_t)reps, cudaMemcpyHostToDevice, s->stream));
  WG_CUDA(cudaMemsetAsync(s->tickets, 0, 4 * (size_t)reps, s->stream));
  WG_CUDA(cudaMemsetAsync(s->big_counts, 0, 8 * (size_t)reps, s->stream));
  // flags[i].unsorted = 1 forces every sort to run in full
  for (int i = 0; i < reps; ++i) s->h_flags[i] = StepFlags{1u, 0u, 0ull};
  WG_CUDA(cudaMemcpyAsync(s->flags, s->h_flags, sizeof(StepFlags) * (size_t)reps,
                          cudaMemcpyHostToDevice, s->stream));
  ForceArgs a;
  a.table = s->table;
  a.n = s->n;
  a.T_lo = s->T_lo;
  a.T_hi = s->T_hi;
  a.E = s->E;
  a.has_omega = s->omega2 >= 0;
  a.omega2 = s->omega2;
  a.ext = s->ext;
  a.t_seq = s->t_seq;
  a.epochs = s->epochs;
  a.recs = s->recs;
  a.err = s->err;
  a.a_out = nullptr;
  a.dt_kick = 0.0;
  a.dt_drift = 0.0;
  a.flag_out = &s->flags[s->cap];  // scratch slot
  WG_CUDA(cudaMemsetAsync(s->ocount, 0, 16, s->stream));
  WG_CUDA(cudaStreamSynchronize(s->stream));
  const int lay_start = s->lay, cs_start = s->cslot;
  if (what == WG_PROF_BUCKET) {
    fill_dev(s, 0.0, 0.0);
    WG_CUDA(cudaMemcpyAsync(s->d_dev, &s->dev, sizeof(SimDev), cudaMemcpyHostToDevice,
                            s->stream));
  }
  WG_CUDA(cudaEventRecord(s->ev0, s->stream));
  for (int i = 0; i < reps; ++i) {
    if (what == WG_PROF_BUCKET) {
      launch_substep(s, i, reps, 1);
    } else if (what == WG_PROF_FORCE) {
      a.sub = i;
      a.ticket = s->tickets + i;
      launch_force(a, s->n_tiles, s->stream);
    } else {
      radix_sort_state(s->table, s->n, &s->radix, &s->flags[i], s->err, s->stream);
    }
  }
  WG_CUDA(cudaEventRecord(s->ev1, s->stream));
  WG_CUDA(cudaStreamSynchronize(s->stream));
  WG_CUDA(cudaGetLastError());
  float ms = 0;
  WG_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
  *avg_seconds = ms * 1e-3 / reps;
  s->st.launches += what == WG_PROF_SORT ? (int64_t)reps * kRadixLaunches : reps;
  if (what == WG_PROF_BUCKET) {
    // dt = 0 kept every sheet in place, but the layout is now routed by the
    // stored positions rather than by the pending half drift: hand the
    // sheets back to the compact state so the next wg_step re-sorts them
    unsigned ab[2] = {0, 0};
    WG_CUDA(cudaMemcpy(ab, s->ocount, 8, cudaMemcpyDeviceToHost));
    const int lay_end = ab[1] ? (((ab[1] - 1) % 2 == 0) ? 1 - lay_start : lay_start)
                              : ((lay_start + reps) & 1);
    const int cs_end = (cs_start + (ab[1] ? (int)ab[1] : reps)) % kAggSlots;
    bucket_to_compact(s, lay_end, cs_end);
    s->lay = lay_end;
    s->qsel = (s->qsel + reps) & 1;
    s->cslot = cs_end;
    s->mode = 0;
    WG_CUDA(cudaStreamSynchronize(s->stream));
  }
  unsigned err = 0;
  WG_CUDA(cudaMemcpy(&err, s->err, 4, cudaMemcpyDeviceToHost));
  if (err) {
    set_error("device error word 0x%x during profiling", err);
    cudaMemset(s->err, 0, 4);
    return WG_ERR_DEVICE;
  }
  return WG_OK;
}

int wg_set_tuning(const wg_tuning* rows, int nrows) {
  if (nrows < 0 || (nrows > 0 && !rows)) {
    set_error("bad tuning table");
    return WG_ERR_ARG;
  }
  std::vector<std::pair<int64_t, BucketTuning>> t;
  for (int i = 0; i < nrows; ++i) {
    const wg_tuning& r = rows[i];
    if (r.target < 64 || r.target > kMaxTarget || r.window < 1 ||
        r.window > kSplitterWindow || r.sort_bits < kSortBitsMin || r.sort_bits > kSortBitsMax ||
        r.ctas_per_sm < 1 || r.ctas_per_sm > 2 || (i > 0 && r.n_min < rows[i - 1].n_min)) {
      set_error("tuning row %d out of range (target 64..%d, window 1..%d, sort_bits %d..%d, "
                "ctas_per_sm 1..2, n_min ascending)", i, kMaxTarget, kSplitterWindow,
                kSortBitsMin, kSortBitsMax);
      return WG_ERR_ARG;
    }
    BucketTuning b;
    b.target = r.target;
    b.window = r.window;
    b.sort_bits = r.sort_bits;
    b.ctas_per_sm = r.ctas_per_sm;
    t.emplace_back(r.n_min, b);
  }
  set_tuning(t);
  return WG_OK;
}

int wg_get_tuning(int64_t n, wg_tuning* out) {
  if (!out) {
    set_error("null output");
    return WG_ERR_ARG;
  }
  const BucketTuning b = tuning_for(n);
  out->n_min = 0;
  out->target = b.target;
  out->window = b.window;
  out->sort_bits = b.sort_bits;
  out->ctas_per_sm = b.ctas_per_sm;
  return WG_OK;
}

int wg_host_register(void* ptr, int64_t bytes) {
  if (!ptr || bytes <= 0) {
    set_error("bad arguments to wg_host_register");
    return WG_ERR_ARG;
  }
  WG_CUDA(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault));
  return WG_OK;
}

int wg_host_unregister(void* ptr) {
  WG_CUDA(cudaHostUnregister(ptr));
  return WG_OK;
}

int wg_host_alloc(int64_t bytes, void** ptr) {
  if (!ptr || bytes <= 0) {
    set_error("bad arguments to wg_host_alloc");
    return WG_ERR_ARG;
  }
  *ptr = nullptr;
  WG_CUDA(cudaHostAlloc(ptr, (size_t)bytes, cudaHostAllocDefault));
  return WG_OK;
}

int wg_host_free(void* ptr) {
  if (!ptr) return WG_OK;
  WG_CUDA(cudaFreeHost(ptr));
  return WG_OK;
}

int wg_energy(wg_sim* s, double twopiG, double omega2, double* energy, double* momentum) {
  const int rc0 = check_idle(s);
  if (rc0) return rc0;
  if (!(twopiG > 0.0) || !std::isfinite(twopiG) || !std::isfinite(omega2)) {
    set_error("wg_energy needs a simulation, a positive finite twopiG and a finite omega2");
    return WG_ERR_ARG;
  }
  // the current state in sorted order: the bucket layout (if any) goes back
  // to the compact sets, which the next wg_step re-sorts and re-buckets
  if (s->mode == 1) {
    bucket_to_compact(s, s->lay, s->cslot);
    s->mode = 0;
  }
  int rc = alloc_call_arrays(s, 1);
  if (rc) return rc;
  s->h_t[0] = 0.0;
  // one self-gravity force evaluation (no harmonic or external term), dt = 0
  const double om = s->omega2;
  const ExtForce ext = s->ext;
  s->omega2 = -1.0;
  s->ext.kind = EXT_NONE;
  rc = enqueue_step(s, 0.0, 1, true, 0.0);
  s->omega2 = om;
  s->ext = ext;
  if (rc) return rc;
  launch_energy(s->table, s->n, s->a_sorted, s->diag, s->stream);
  s->st.launches += 3 + kRadixLaunches;
  double sums[4];
  WG_CUDA(cudaMemcpyAsync(sums, s->diag, sizeof(sums), cudaMemcpyDeviceToHost, s->stream));
  rc = finish_call(s, 0, false);  // synchronises and checks the device error word
  if (rc) return rc;
  // masses on the device are m twopiG (wendy/wendy.py:373)
  const double e = sums[0] + (omega2 >= 0.0 ? omega2 * sums[1] : 0.0) + sums[2];
  if (energy) *energy = e / twopiG;
  if (momentum) *momentum = sums[3] / twopiG;
  return WG_OK;
}

int wg_ext_force_eval(int64_t n, const double* x, double t, int ext_kind,
                      const double* ext_params, int n_ext_params, double* out) {
  if (n < 1 || !x || !out || !std::isfinite(t)) {
    set_error("wg_ext_force_eval needs n >= 1, x, out and a finite t");
    return WG_ERR_ARG;
  }
  ExtSpec ext;
  int rc = check_ext(ext_kind, ext_params, n_ext_params, &ext);
  if (rc) return rc;
  double* d = nullptr;
  ExprOp* d_prog = nullptr;
  cudaError_t e = cudaMalloc(&d, 16 * (size_t)n);
  if (e == cudaSuccess) e = attach_ext_program(&ext, &d_prog, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (d) cudaFree(d);
    if (d_prog) cudaFree(d_prog);
    set_error("device buffers of %zu bytes failed: %s", 16 * (size_t)n, cudaGetErrorString(e));
    return WG_ERR_NOMEM;
  }
  e = cudaMemcpy(d, x, 8 * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    launch_ext_eval(ext.f, t, d, d + n, n, 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d + n, 8 * (size_t)n, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (d_prog) cudaFree(d_prog);
  if (e != cudaSuccess) {
    set_error("wg_ext_force_eval failed: %s", cudaGetErrorString(e));
    return WG_ERR_CUDA;
  }
  return WG_OK;
}

int wg_accel(int64_t n, const double* x, const double* m, double totmass, double omega2,
             int ext_kind, const double* ext_params, int n_ext_params, double t, double* a,
             int32_t* perm) {
  std::vector<double> zero((size_t)(n > 0 ? n : 1), 0.0);
  int rc = validate_sheets(n, x, zero.data(), m, totmass);
  if (rc) return rc;
  ExtSpec ext;
  rc = check_ext(ext_kind, ext_params, n_ext_params, &ext);
  if (rc) return rc;
  wg_sim* s = nullptr;
  rc = make_sim(n, totmass, omega2, ext, &s, false);
  if (rc) return rc;
  const StateRef c = s->set[0];
  cudaMemcpyAsync(c.x, x, 8 * n, cudaMemcpyHostToDevice, s->stream);
  cudaMemsetAsync(c.v, 0, 8 * n, s->stream);
  cudaMemcpyAsync(c.m, m, 8 * n, cudaMemcpyHostToDevice, s->stream);
  launch_init_state(s->table, n, s->stream);
  s->h_t[0] = t;
  // One force evaluation: a zero-length drift (v = 0) leaves x as given and
  // marks the order for sorting, then sort and one force kernel with
  // dt_kick = dt_drift = 0.
  rc = enqueue_step(s, 0.0, 1, true, 0.0);
  if (rc == WG_OK) {
    StateTable tab;
    launch_scatter_accel(s->table, n, s->a_sorted, s->x_out, s->stream);
    cudaMemcpyAsync(&tab, s->table, sizeof(tab), cudaMemcpyDeviceToHost, s->stream);
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) {
      set_error("accel failed: %s", cudaGetErrorString(cudaGetLastError()));
      rc = WG_ERR_CUDA;
    } else {
      if (a) cudaMemcpy(a, s->x_out, 8 * n, cudaMemcpyDeviceToHost);
      if (perm) cudaMemcpy(perm, tab.cur.idx, 4 * n, cudaMemcpyDeviceToHost);
      rc = finish_call(s, 1);
    }
  }
  free_sim(s);
  return rc;
}

int wg_set_debug_wait(unsigned spin_limit, int64_t withhold_tile) {
  set_wait_debug(spin_limit, withhold_tile);
  return WG_OK;
}

int wg_nbody_approx_stats(wg_stats* out) {
  if (!out) {
    set_error("null output");
    return WG_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_cache_mu);
  *out = wg_stats{};
  if (g_cache) *out = g_cache->st;
  return WG_OK;
}

int wg_nbody_approx_onestep(int n, wg_sheet* xi, double* x, double* v, const double* m,
                            double* a, double totmass, double dt, int nleap, double* t0,
                            double omega2, int ext_kind, const double* ext_params,
                            int n_ext_params, int* err, double* time_elapsed) {
  if (err) *err = 0;
  if (!xi || !x || !v || !m || !a || nleap < 1 || nleap > kMaxLeap || n < 1) {
    set_error("null buffer, n < 1, nleap < 1 or nleap > %d", kMaxLeap);
    return WG_ERR_ARG;
  }
  ExtSpec ext;
  int rc = check_ext(ext_kind, ext_params, n_ext_params, &ext);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_cache_mu);
  wg_sim* s = g_cache;
  // (a cached state that a device error left untrustworthy is rebuilt: every
  // call of this entry hands over its complete inputs)
  if (!s || s->n != n || s->broken) {
    free_sim(s);
    g_cache = nullptr;
    rc = make_sim(n, totmass, omega2, ext, &s);
    if (rc) return rc;
    g_cache = s;
  }
  auto bits_eq = [](double p, double q) { return std::memcmp(&p, &q, sizeof(double)) == 0; };
  auto point_at = [&](int set) {
    wg_sim::OutSet& o = s->outs[set];
    s->x_out = o.x;
    s->v_out = o.v;
    s->call_xi = reinterpret_cast<SheetRec*>(o.xi);
    s->call_a = o.a;
  };
  auto clear_call = [&]() {
    s->call_xi = nullptr;
    s->call_a = nullptr;
  };
  // The sub-steps the previous call enqueued for this one are usable only
  // with this call's scalars; otherwise they are completed and dropped first
  // (they hold the per-call arrays and the physics).  They advanced the
  // resident state past the previous call's outputs, so this call cannot
  // continue from it: it loads its inputs.
  auto drop_spec = [&]() {
    point_at(s->spec_set);
    double ignored = 0;
    run_call_end(s, &ignored);
    clear_call();
    s->spec_pending = false;
    s->spec_enabled = false;
    s->resume_ok = false;
  };
  bool spec = s->spec_pending;
  if (spec) {
    const bool same = t0 && bits_eq(dt, s->spec_dt) && nleap == s->spec_nleap &&
                      bits_eq(*t0, s->spec_t0_in) && bits_eq(totmass, s->spec_totmass) &&
                      bits_eq(omega2, s->spec_omega2) && same_ext(ext, s->spec_ext);
    if (!same) {
      drop_spec();
      spec = false;
    }
  }
  // physics of this call
  s->totmass = totmass;
  s->omega2 = omega2;
  rc = set_force(s, ext);
  if (rc) return rc;
  if (totmass > 0) {
    int eT = 0;
    std::frexp(totmass, &eT);
    s->E = 123 - eT;
  } else {
    s->E = 0;
  }
  const u128 T = host_mass_to_fixed(totmass, s->E);
  s->T_lo = (uint64_t)T;
  s->T_hi = (uint64_t)(T >> 64);
  rc = alloc_call_arrays(s, nleap);
  if (rc) return rc;
  if (!s->stage) {
    const size_t bx = al(sizeof(wg_sheet) * (size_t)n), bd = al(8 * (size_t)n);
    const size_t b = 3 * bx + 9 * bd + al(16);
    WG_CUDA(cudaMalloc(&s->stage, b));
    char* q = static_cast<char*>(s->stage);
    for (int k = 0; k < 2; ++k) {
      s->outs[k].xi = reinterpret_cast<wg_sheet*>(q); q += bx;
      s->outs[k].x = reinterpret_cast<double*>(q); q += bd;
      s->outs[k].v = reinterpret_cast<double*>(q); q += bd;
      s->outs[k].a = reinterpret_cast<double*>(q); q += bd;
    }
    s->in_xi = reinterpret_cast<wg_sheet*>(q); q += bx;
    s->in_v = reinterpret_cast<double*>(q); q += bd;
    s->in_m = reinterpret_cast<double*>(q); q += bd;
    s->prev_m = reinterpret_cast<double*>(q); q += bd;
    s->d_diff = reinterpret_cast<unsigned*>(q);
    s->st.device_bytes += (int64_t)b;
    WG_CUDA(cudaStreamCreateWithFlags(&s->up_stream, cudaStreamNonBlocking));
    WG_CUDA(cudaStreamCreateWithFlags(&s->down_stream, cudaStreamNonBlocking));
    WG_CUDA(cudaEventCreateWithFlags(&s->ev_up, cudaEventDisableTiming));
    s->resume_ok = false;
  }
  // This call's inputs are uploaded on their own stream and compared bit for
  // bit with the previous call's outputs and masses.  The previous call left
  // the sheets in buckets routed for this call's opening half drift: when
  // the inputs are exactly its outputs, the call continues from there (the
  // same arithmetic as loading, re-sorting and re-bucketing them), and its
  // sub-steps may already have run (enqueued by the previous call).
  // Otherwise the sheets are loaded in xi's order and sorted.
  const bool candidate = s->resume_ok && bits_eq(totmass, s->resume_totmass);
  unsigned* const h_diff = s->h_ab + 8;
  cudaStream_t up = s->up_stream;
  const int prev = s->out_last;
  WG_CUDA(cudaMemcpyAsync(s->in_xi, xi, sizeof(wg_sheet) * (size_t)n, cudaMemcpyHostToDevice, up));
  WG_CUDA(cudaMemcpyAsync(s->in_v, v, 8 * (size_t)n, cudaMemcpyHostToDevice, up));
  WG_CUDA(cudaMemcpyAsync(s->in_m, m, 8 * (size_t)n, cudaMemcpyHostToDevice, up));
  if (candidate) {
    WG_CUDA(cudaMemsetAsync(s->d_diff, 0, 4, up));
    k_inputs_differ<<<152 * 8, 256, 0, up>>>(n, s->in_xi, s->outs[prev].xi, s->in_v,
                                             s->outs[prev].v, s->in_m, s->prev_m, s->d_diff);
    WG_CUDA(cudaGetLastError());
    WG_CUDA(cudaMemcpyAsync(h_diff, s->d_diff, 4, cudaMemcpyDeviceToHost, up));
  }
  WG_CUDA(cudaEventRecord(s->ev_up, up));
  int out = prev ^ 1;  // the set this call's outputs go to
  bool resumed = false;
  if (spec) {
    WG_CUDA(cudaEventSynchronize(s->ev_up));
    if (candidate && *h_diff == 0) {
      point_at(s->spec_set);
      rc = run_call_end(s, time_elapsed);
      s->spec_pending = false;
      if (rc == WG_OK && !s->out_valid) {
        launch_desort(s->table, n, s->x_out, s->v_out, s->stream);
        s->out_valid = true;
      }
      clear_call();
      if (rc) {
        if (err) *err = rc;
        return rc;
      }
      *t0 = s->spec_t0_out;
      out = s->spec_set;
      resumed = true;
    } else {
      drop_spec();
    }
  } else if (candidate && s->mode == 1) {
    WG_CUDA(cudaEventSynchronize(s->ev_up));
    if (*h_diff == 0) {
      point_at(out);
      rc = run_call(s, dt, nleap, t0, time_elapsed, true);
      if (rc == WG_OK && !s->out_valid) {
        launch_desort(s->table, n, s->x_out, s->v_out, s->stream);
        s->out_valid = true;
      }
      clear_call();
      if (rc) {
        if (err) *err = rc;
        return rc;
      }
      resumed = true;
      s->spec_enabled = true;
    }
  }
  if (!resumed) {
    WG_CUDA(cudaStreamWaitEvent(s->stream, s->ev_up, 0));
    StateTable t0tab;
    t0tab.cur = s->set[0];
    t0tab.other = s->set[1];
    WG_CUDA(cudaMemcpyAsync(s->table, &t0tab, sizeof(t0tab), cudaMemcpyHostToDevice, s->stream));
    k_load_sheets<<<152 * 8, 256, 0, s->stream>>>(s->table, n, s->in_xi, s->in_v, s->in_m);
    // the sheets are compact with the opening half drift pending: the call
    // sorts them and runs on the bucket path
    s->mode = 0;
    point_at(out);
    rc = run_call(s, dt, nleap, t0, time_elapsed, true);
    if (rc == WG_OK && !s->out_valid) {
      launch_desort(s->table, n, s->x_out, s->v_out, s->stream);
      s->out_valid = true;
    }
    clear_call();
    if (rc) {
      if (err) *err = rc;
      return rc;
    }
  }
  // desorts above ran on the main stream: done before the downloads
  WG_CUDA(cudaStreamSynchronize(s->stream));
  s->resume_ok = s->mode == 1;
  s->resume_totmass = totmass;
  // the next call's sub-steps, enqueued now on the main stream: they run
  // while this call's outputs download and the caller works on them
  if (s->spec_enabled && s->resume_ok && s->compact_calls == 0 && t0) {
    s->spec_set = out ^ 1;
    point_at(s->spec_set);
    double t_spec = *t0;
    const int rs = run_call_begin(s, dt, nleap, &t_spec, true);
    clear_call();
    if (rs == WG_OK) {
      s->spec_pending = true;
      s->spec_dt = dt;
      s->spec_nleap = nleap;
      s->spec_t0_in = *t0;
      s->spec_t0_out = t_spec;
      s->spec_totmass = totmass;
      s->spec_omega2 = omega2;
      s->spec_ext = ext;
    }
  }
  // the caller's buffers were read by the uploads before they are written here
  cudaStream_t down = s->down_stream;
  const wg_sim::OutSet& o = s->outs[out];
  WG_CUDA(cudaStreamWaitEvent(down, s->ev_up, 0));
  // (the uploads have read x, v and xi before the host writes into them)
  WG_CUDA(cudaEventSynchronize(s->ev_up));
  host_pages_dirty(xi, sizeof(wg_sheet) * (size_t)n);
  host_pages_dirty(x, 8 * (size_t)n);
  host_pages_dirty(v, 8 * (size_t)n);
  host_pages_dirty(a, 8 * (size_t)n);
  WG_CUDA(cudaMemcpyAsync(xi, o.xi, sizeof(wg_sheet) * (size_t)n, cudaMemcpyDeviceToHost, down));
  WG_CUDA(cudaMemcpyAsync(x, o.x, 8 * (size_t)n, cudaMemcpyDeviceToHost, down));
  WG_CUDA(cudaMemcpyAsync(v, o.v, 8 * (size_t)n, cudaMemcpyDeviceToHost, down));
  WG_CUDA(cudaMemcpyAsync(a, o.a, 8 * (size_t)n, cudaMemcpyDeviceToHost, down));
  WG_CUDA(cudaStreamSynchronize(down));
  // this call's masses are the next call's reference
  std::swap(s->in_m, s->prev_m);
  s->out_last = out;
  return WG_OK;
}

}  // extern "C"
