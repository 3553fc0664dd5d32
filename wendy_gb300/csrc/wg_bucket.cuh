// wg_bucket.cuh -- bucketed sheet layout and the fused sub-step kernel.
#pragma once
#include <cstdint>

#include "wg_internal.cuh"

namespace wg {

constexpr int kBucketThreads = 256;
constexpr int kBucketCap = 2048;      // sheets a bucket can hold
constexpr int kBucketTarget = 1024;   // sheets per bucket right after a re-sort
constexpr int kSplitterWindow = 64;   // buckets searched in shared memory on each side

// Decoupled look-back record of one bucket (48 bytes).
struct __align__(16) BucketRec {
  uint64_t agg_lo, agg_hi;  // bucket's fixed-point mass
  uint64_t inc_lo, inc_hi;  // inclusive mass prefix
  uint32_t agg_cnt, inc_cnt;  // sheet count, inclusive count prefix
  unsigned flag;              // (epoch << 2) | {1: aggregate, 2: inclusive}
  unsigned pad;
};

struct BucketStepArgs {
  // layout read by this sub-step (bucket b = slots [b*cap, b*cap + cnt_in[b]))
  const double* xin;
  const double* vin;
  const double* min;
  const int32_t* iin;
  unsigned* cnt_in;        // zeroed after reading (reused two sub-steps later)
  // layout written by this sub-step
  double* xout;
  double* vout;
  double* mout;
  int32_t* iout;
  unsigned* cnt_out;       // zero on entry, appended to
  const uint64_t* q_dest_key;  // [nb + 1] splitters of the written layout
  const int32_t* q_dest_idx;
  uint64_t* q_new_key;     // [nb + 1] quantiles of this sub-step's sorted keys
  int32_t* q_new_idx;
  int64_t n;
  int64_t nb;
  int target;
  BucketRec* recs;
  const unsigned* epochs;
  int sub;
  unsigned* ticket;
  // physics
  uint64_t T_lo, T_hi;
  int E;
  int has_omega;
  double omega2;
  ExtForce ext;
  const double* t_seq;
  double pre_dt;    // drift applied on load (a call's opening half drift) or 0
  double dt_kick;
  double dt_drift;
  double dest_dt;   // routing uses x + dest_dt v (the next call's opening half drift) or 0
  double* x_orig;   // if set: new x, v written in original order (the call's output)
  double* v_orig;
  // overflow list (sheets that found their bucket full)
  double* ox;
  double* ov;
  double* om;
  int32_t* oi;
  unsigned* ocount;
  unsigned* abort;  // 1 + first sub-step of the call that overflowed, or 0
  unsigned* err;
  StepFlags* flag_out;
};

size_t bucket_step_smem();
void launch_bucket_step(const BucketStepArgs& a, int grid, cudaStream_t s);
void launch_bucketize(const StateTable* table, int64_t n, int target, int64_t nb, double* x,
                      double* v, double* m, int32_t* idx, unsigned* cnt, uint64_t* qk,
                      int32_t* qi, unsigned* cnt_other, cudaStream_t s);
void launch_compact(StateTable* table, int64_t nb, const double* x, const double* v,
                    const double* m, const int32_t* idx, const unsigned* cnt, unsigned* offs,
                    const double* ox, const double* ov, const double* om, const int32_t* oi,
                    const unsigned* ocount, int64_t n, cudaStream_t s);

}  // namespace wg
