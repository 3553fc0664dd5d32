// wg_bucket.cuh -- bucketed sheet layout and the fused sub-step kernel.
//
// A launch of the sub-step kernel serves any number of simulations at once:
// each simulation has its own arrays (described by a SimDev entry) and the
// launch walks a list of (simulation, bucket) tasks in order, so one launch
// per sub-step advances a whole ensemble.  A single simulation is an ensemble
// of one.
#pragma once
#include <cstdint>

#include "wg_internal.cuh"

namespace wg {

constexpr int kBucketThreads = 256;
constexpr int kBucketCap = 2048;      // sheets a bucket's shared-memory pass can hold
constexpr int kBucketCapBig = 3 * kBucketCap;  // sheets a bucket of a single simulation
                                               // can hold (taken in chunks above kBucketCap)
constexpr int kSplitterWindow = 64;   // largest splitter window (buckets on each side)
constexpr int kMemberSampleCap = 4096; // most splitter samples a pool member sorts in one CTA
constexpr int kSortBitsMin = 9;       // smallest counting-sort offset (bits)
constexpr int kSortBitsMax = 13;      // largest counting-sort offset (bits)
constexpr int kMaxTarget = kBucketCap * 3 / 4;  // largest bucket target

// Tunables of the fused sub-step, chosen per simulation size by the
// autotuner (wendy_gb300/autotune.py) or left at their defaults.
struct BucketTuning {
  int target = 1536;      // sheets per bucket right after a re-sort (<= kMaxTarget)
  int window = 64;        // splitters searched in shared memory on each side
  int sort_bits = 12;     // counting-sort bins = 2^sort_bits (9..13)
  int ctas_per_sm = 2;    // persistent CTAs per SM (1 or 2)
};
BucketTuning tuning_for(int64_t n);
}  // namespace wg
#include <utility>
#include <vector>
namespace wg {
void set_tuning(const std::vector<std::pair<int64_t, BucketTuning>>& rows);

// Epochs tag the records of one sub-step; they run from 1 to kEpochLimit,
// after which the host clears every record and starts again at 1.
constexpr unsigned kEpochLimit = (1u << 24) - 1;
constexpr int kMaxLeap = 1 << 22;  // sub-steps in one call (WG_MAX_LEAP)

// Look-back record of one bucket: its inclusive (mass, count) prefix in four
// 64-bit words, each carrying the 24-bit epoch of the sub-step that wrote it
// in its top bits and 40 payload bits below: mass bits [0,40), [40,80),
// [80,120), and mass bits [120,127) << 32 | count.  Each word is stored and
// loaded whole, so a reader that finds the current epoch in all four has the
// complete prefix without any flag or fence; a cleared record (epoch 0) never
// matches.
struct __align__(32) BucketRec {
  uint64_t w[4];
};

// Per-bucket aggregates (sheet count and fixed-point mass) rotate over three
// slots: sub-step g reads slot g % 3 (filled by the writers of sub-step g - 1),
// its writers fill slot (g + 1) % 3, and it clears slot (g + 2) % 3 for the
// sub-step after.  The mass is kept as four 32-bit limbs in 64-bit
// accumulators, mass = sum_k limb[k] << 32 k, so that writers can add to it
// with plain 64-bit atomics.
constexpr int kAggSlots = 3;

// Same layout as wendy's struct array_w_index (int idx; double val).
struct SheetRec {
  int32_t idx;
  int32_t pad;
  double val;
};

// One simulation as the sub-step kernel sees it.  Arrays are the
// simulation's own; layouts, counts and splitters come in pairs used
// alternately from sub-step to sub-step, starting at lay0 / qsel0.
// One sheet's output in original order: a whole 32-byte sector, so that the
// random write of the last sub-step needs no read-modify-write of the
// memory line it lands in (three 8-byte writes to x, v and a each did).
struct alignas(32) OutRec {
  double x, v, a, pad;
};

struct SimDev {
  double* bx[2];
  double* bv[2];
  double* bm[2];
  int32_t* bi[2];
  unsigned* bcnt[kAggSlots];         // per-bucket sheet counts
  unsigned long long* bmass[kAggSlots];  // per-bucket mass limbs [4 * nb]
  uint64_t* qk[2];       // [nb + 1] splitter keys (Q_0 = -inf, Q_nb = +inf)
  int32_t* qi[2];        // [nb + 1] splitter indices
  BucketRec* recs;       // [nb]
  double* ox;            // overflow list
  double* ov;
  double* om;
  int32_t* oi;
  unsigned* ocount;      // [0] sheets in the overflow list, [1] 1 + sub-step that overflowed,
                         // [2] 1 + sub-step that could not take a big bucket (its input
                         // layout is intact and is re-sorted by the host)
  double* x_out;         // output of the call's last sub-step, original order
  double* v_out;
  SheetRec* xi_out;      // optional: (idx, x) in the last sub-step's sorted order
  double* a_out;         // optional: accelerations of the last force evaluation, original order
  OutRec* rec_out;       // optional: if set, the last sub-step writes (x, v, a) records
                         // here in original order instead, for launch_split_out
  StepFlags* flags;      // [nleap + 1] of this call
  const double* t_seq;   // [nleap] times of this call's force evaluations
  int64_t n;
  int64_t nb;
  int target;            // sheets per bucket at a re-sort (splitters at ranks j * target)
  int window;            // splitter window half-width (<= kSplitterWindow)
  int sort_bits;         // counting-sort offset bits (9..13)
  int capg;              // slots per bucket in the layouts (kBucketCap .. kBucketCapBig)
  uint64_t T_lo, T_hi;   // totmass in fixed point
  int E;
  int has_omega;
  double omega2;
  ExtForce ext;
  double dt;             // leapfrog step of this call
  double pre_dt;         // half drift applied while loading the first sub-step (or 0)
  int lay0;              // layout read by the call's first sub-step
  int qsel0;             // splitter array defining the layout the first sub-step writes
  int cs0;               // aggregate slot read by the call's first sub-step
  int pad1;
  // predicted splitters (or null): the sheet at global rank j * target writes
  // its position moved on by two drifts at its bucket's mean velocity into
  // entry j - 1 of this table's current set; the host sorts the set after the
  // sub-step and takes it as the splitters of the layout after next
  StateTable* ptab;
};

struct BucketTask {
  int sim;
  int bucket;
};

// A bucket with more sheets than shared memory holds (kBucketCap < n <=
// capg), listed by k_bucket_step for k_bucket_big with what its preparation
// found: its exclusive (mass, count) prefix, splitter window and force
// factors.
struct BigTask {
  int sim;
  int bucket;
  int n;
  int lay;
  int wlo, whi;
  uint32_t pcnt;
  uint32_t pad;
  uint64_t pm_lo, pm_hi;
  double amp, inv_h;
};

struct StepLaunch {
  const SimDev* sims;
  const BucketTask* tasks;
  int ntasks;
  int sub;               // sub-step index within the call
  int nleap;
  const unsigned* epochs;
  unsigned* ticket;      // zero before the launch
  unsigned* err;
  int profile;           // 1: dt = 0 and no outputs (timing harness)
  int any_expr;          // some simulation of the launch has an expression force
  // big buckets of this sub-step (simulations with capg > kBucketCap only):
  // the list k_bucket_step fills and k_bucket_big takes in ticket order
  BigTask* big_list;
  unsigned* big_count;   // zero before the launch
  unsigned* big_ticket;  // zero before the launch
  unsigned big_cap;      // entries of big_list
};

void launch_bucket_step(const StepLaunch& a, int grid, cudaStream_t s);
// The big buckets k_bucket_step listed (launch right after it, same arguments).
void launch_bucket_big(const StepLaunch& a, int grid, cudaStream_t s);
// Pool members with predicted splitters (SimDev::ptab set): block k sorts the
// nb - 1 samples member list[k] (k itself without a list) wrote in sub-step
// `sub` in shared memory and writes them as the splitters that sub-step
// published.  Other blocks return.
void launch_member_splitters(const SimDev* devs, const int* list, int count, int sub,
                             cudaStream_t s);
// ---- pool members re-sorted together after bucket overflows ------------
// One member of such a batch: where its sheets are and where they go.
struct BatchSeg {
  int k;          // index of the member in the call's SimDev array
  int lay;        // layout holding its sheets (plus its overflow list)
  int cslot;      // aggregate slot holding that layout's counts
  int pad;
  int64_t out;    // its first sheet in the batch arrays
  int64_t n;      // its sheets
  int64_t toff;   // its first bucket in the per-bucket offsets
  double pre;     // the half drift its next call opens with, when it overflowed in the
                  // call's last sub-step (else 0): it is sorted and bucketed by
                  // x + pre v, as that sub-step would have routed it
};
// Every batch member's layout and overflow list -> dst[out, out + n),
// unsorted.  tasks: (batch index, bucket) for every bucket of every member
// plus one (batch index, nb) per member for its overflow list; offs: one
// entry per bucket (toff + b).
void launch_batch_compact(const SimDev* devs, const BatchSeg* segs, int nseg,
                          const BucketTask* tasks, int64_t ntasks, StateRef dst, unsigned* offs,
                          int64_t total, cudaStream_t s);
// The members' sorted sheets src[out, out + n) -> fresh bucket layouts 0 with
// exact quantile splitters of x + pre v (tasks: (batch index, bucket) for
// every bucket).
void launch_batch_bucketize(const SimDev* devs, const BatchSeg* segs, const BucketTask* tasks,
                            int64_t ntasks, StateRef src, int64_t total, cudaStream_t s);
// Splitters 1 .. m of a layout from the m sorted samples in table->cur
// (predicted splitters): keys of their positions, and their indices.
void launch_samples_to_splitters(const StateTable* table, int64_t m, uint64_t* qk, int32_t* qi,
                                 cudaStream_t s);
// x_out, v_out (and a_out when not null) from the records of rec_out.
void launch_split_out(const OutRec* rec, int64_t n, double* x_out, double* v_out, double* a_out,
                      cudaStream_t s);
// One-time kernel attribute set-up; call before any stream capture.
void bucket_step_prepare();
int bucket_step_grid(int sm_count);
// Compact sorted state -> layout 0 with `target` sheets per bucket; fills
// aggregate slot 0 and clears the other two.
void launch_bucketize(const StateTable* table, int64_t n, int target, int64_t nb, int capg, int E,
                      double* x, double* v, double* m, int32_t* idx,
                      unsigned* const cnt[kAggSlots], unsigned long long* const mass[kAggSlots],
                      uint64_t* qk, int32_t* qi, cudaStream_t s);
void launch_compact(StateTable* table, int64_t nb, int capg, const double* x, const double* v,
                    const double* m, const int32_t* idx, const unsigned* cnt, unsigned* offs,
                    const double* ox, const double* ov, const double* om, const int32_t* oi,
                    const unsigned* ocount, int64_t n, cudaStream_t s);

}  // namespace wg
