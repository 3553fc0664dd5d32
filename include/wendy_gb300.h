/*
  wendy_gb300.h -- C ABI of the GB300-native approximate integrator.

  One shared library (wendy_gb300/_wendy_gb300.so) exposes plain-C entry
  points with pointers and sizes only, loaded from Python through ctypes the
  way wendy loads its own C extension (wendy/wendy.py:13-37).  Every entry
  returns an int status (WG_OK or a negative WG_ERR_* code); nothing throws
  across the boundary and nothing calls back into the host.

  Physics and argument meaning follow the reference's approximate path:
  masses are already multiplied by 2 pi G, `totmass` is their sum as the
  caller computed it, `omega2` is omega^2 or a negative number for "no
  harmonic term", and the time of a time-dependent external force lags the
  positions and advances by dt per force evaluation
  (wendy/wendy.c:385-418, wendy/wendy.py:363-383).

  External forces are registered closed forms (WG_EXT_*) rather than host
  callbacks: the force is evaluated inside the fused device kernel.
*/
#ifndef WENDY_GB300_H
#define WENDY_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define WG_OK 0
#define WG_ERR_ARG (-1)      /* invalid argument (sizes, non-finite or negative masses, ...) */
#define WG_ERR_CUDA (-2)     /* a CUDA runtime call failed; see wg_last_error() */
#define WG_ERR_NOMEM (-3)    /* device allocation failed */
#define WG_ERR_DEVICE (-4)   /* a kernel raised its error word (e.g. a bounded wait expired);
                                the simulation it ran on is unusable afterwards */
#define WG_ERR_EXT (-5)      /* unknown external-force id or bad parameter count */
#define WG_ERR_BUDGET (-6)   /* request exceeds the memory budget it was admitted under */
#define WG_ERR_NODEV (-7)    /* no CUDA device */
#define WG_ERR_MAXCOLL (-8)  /* the exact solver reached maxcoll crossings in one output */

/* ---- registered external forces ---------------------------------------- */
#define WG_EXT_NONE 0
#define WG_EXT_HARMONIC 1    /* F = -p[0] x                                  (1 param)  */
#define WG_EXT_PULSE_TANH 2  /* F = p[0] exp(-(t-p[1])^2/(2 p[2]^2)) tanh(x/p[3]) (4 params) */
/* A compiled expression F(x, t): the parameters are a register program
   (at most WG_EXPR_MAX_OPS ops on WG_EXPR_REGS registers) that
   wendy_gb300/extforce.py compiles from a restricted Python function or
   string -- arithmetic, integer and real powers, exp, log, sqrt, sin, cos,
   tan, tanh, sinh, cosh, arctan, abs of x, t and constants:
     p[0] = number of ops, p[1] = ops of the time phase (t and constants
     only, run once per force evaluation), then five numbers per op:
     code, destination register, operand registers a and b, constant.
   Codes: 0 x, 1 t, 2 constant, 3 copy a, 4 a+b, 5 a-b, 6 a*b, 7 a/b, 8 -a,
   9 pow(a, b), 10 exp, 11 log, 12 sqrt, 13 sin, 14 cos, 15 tan, 16 tanh,
   17 sinh, 18 cosh, 19 atan, 20 abs (of a).  F is the register the last op
   writes.  Malformed programs (unknown codes, registers out of range or read
   before written, x in the time phase) return WG_ERR_EXT.  Replaces the
   numba-compiled callables of wendy/wendy.py:389-404. */
#define WG_EXT_EXPR 3
#define WG_EXPR_MAX_OPS 64
#define WG_EXPR_REGS 16

/* Same layout as wendy's `struct array_w_index` (wendy/wendy.h:12-16). */
typedef struct wg_sheet {
  int idx;
  double val;
} wg_sheet;

typedef struct wg_sim wg_sim; /* opaque: one simulation resident on the device */

typedef struct wg_stats {
  int64_t n;                 /* sheets */
  int64_t substeps;          /* force evaluations run so far */
  int64_t sorts_full;        /* sub-steps that needed a full radix sort */
  int64_t sorts_skipped;     /* sub-steps whose order was already sorted */
  int64_t sorts_window;      /* sub-steps repaired by the bounded-window fix-up */
  double last_max_disp;      /* largest |dx| of the last drift */
  int64_t device_bytes;      /* device memory held by the simulation */
  int64_t launches;          /* kernels this handle has launched */
  int64_t last_max_count;    /* most sheets any bucket received during the last call */
  int64_t substeps_compact;  /* sub-steps run on the compact path (full re-sort + force) */
  int64_t big_buckets;       /* buckets taken in chunks (more sheets than one pass holds) */
  int64_t substeps_predicted; /* bucket sub-steps whose splitters were predicted from velocities */
} wg_stats;

/* Library and device information. */
int wg_version(void);
const char *wg_status_string(int status);
const char *wg_last_error(void); /* detail of the last failure on this thread */
int wg_device_info(int *sm_count, int64_t *free_bytes, int64_t *total_bytes);

/* ---- the stateful path behind nbody(..., approx=True, sort='cuda') ------
   Replaces the per-output ctypes call to _wendy_nbody_approx_onestep
   (wendy/wendy.py:425-433, wendy/wendy.c:385-418) with a handle that keeps
   the sheets on the device, in sorted order, between outputs. */

/* Copy n sheets to the device (original order) and validate them.
   Reference: the set-up half of _nbody_approx, wendy/wendy.py:363-387. */
int wg_create(int64_t n, const double *x, const double *v, const double *m, double totmass,
              double omega2, int ext_kind, const double *ext_params, int n_ext_params,
              wg_sim **out);

/* Advance by one output interval: nleap leapfrog sub-steps of dt each
   (dt here is the reference's dt_leap = dt_output / nleap).  *t0 is updated
   exactly as the reference does (repeated += dt, only with an external
   force); *time_elapsed receives the device time of the call in seconds.
   nleap is limited to WG_MAX_LEAP sub-steps per call (WG_ERR_ARG beyond).
   Reference: _wendy_nbody_approx_onestep, wendy/wendy.c:385-418. */
#define WG_MAX_LEAP 4194304
int wg_step(wg_sim *s, double dt, int nleap, double *t0, double *time_elapsed);

/* wg_step in two halves: wg_step_begin enqueues the output interval on the
   simulation's stream and returns at once (*t0 is advanced immediately);
   wg_step_end waits for it, completes it (a sub-step that overflowed a
   bucket is finished on the full re-sort path here) and reports its device
   time.  Between the two, wg_download returns the output completed before
   wg_step_begin (the step writes a second pair of output buffers), copied on
   a stream of its own while the step runs; every other entry on the
   simulation except wg_destroy returns WG_ERR_ARG.  Lets a caller overlap its
   own work on the previous output, and its download, with the device
   computing the next one.
   Reference: _wendy_nbody_approx_onestep, wendy/wendy.c:385-418. */
int wg_step_begin(wg_sim *s, double dt, int nleap, double *t0);
int wg_step_end(wg_sim *s, double *time_elapsed);

/* Copy positions and velocities back in original particle order (during a
   split step: those of the output completed before it).
   Reference: the de-sort at wendy/wendy.c:413-415 and the in-place yield
   of wendy/wendy.py:434-437. */
int wg_download(wg_sim *s, double *x, double *v);

/* Total energy and momentum of the simulation's current state (the last
   output), computed on the device: sorted order, one self-gravity force
   evaluation, and sums in a fixed order.  twopiG and omega2 (< 0: no
   harmonic term) have the meaning of the reference's energy(); the masses
   the simulation holds are already times twopiG.  The potential term uses
   sum_{x_j<x_i} m_i m_j (x_i - x_j) = -sum_i m_i x_i a_i / twopiG.  Leaves the
   simulation compact (the next wg_step re-sorts once).
   Reference: energy and momentum, wendy/wendy.py:439-491. */
int wg_energy(wg_sim *s, double twopiG, double omega2, double *energy, double *momentum);
int wg_get_stats(wg_sim *s, wg_stats *out);
int wg_destroy(wg_sim *s);

/* Average device time (seconds, CUDA events on the handle's stream) of one
   component over `reps` back-to-back launches on the resident sheets,
   without changing them: what = WG_PROF_FORCE (the fused force / kick /
   drift kernel on sorted sets, dt = 0), WG_PROF_SORT (a full re-sort),
   WG_PROF_BUCKET (the fused bucket sub-step, dt = 0; needs one wg_step
   first).  For the measurement harness; no reference counterpart. */
#define WG_PROF_FORCE 0
#define WG_PROF_SORT 1
#define WG_PROF_BUCKET 2
int wg_profile(wg_sim *s, int what, int reps, double *avg_seconds);

/* Tuning of the fused bucket sub-step by simulation size.  Row i applies to
   simulations of n >= n_min[i] sheets (rows ascending in n_min) created after
   the call: sheets per bucket after a re-sort (64..1024), splitter window
   (1..64 buckets each side), counting-sort bits (8..12), persistent CTAs per
   SM (1..2).  Written by the autotuner (wendy_gb300/autotune.py); no
   reference counterpart. */
typedef struct wg_tuning {
  int64_t n_min;
  int target;
  int window;
  int sort_bits;
  int ctas_per_sm;
} wg_tuning;
int wg_set_tuning(const wg_tuning *rows, int nrows);
int wg_get_tuning(int64_t n, wg_tuning *out);

/* Test hook for the bounded waits (no reference counterpart).  The force
   kernel of the compact path finds each tile's mass prefix by looking back
   over earlier tiles; spin_limit bounds each of its waits (0 = the production
   limit, well above a second) and withhold_tile names a tile whose look-back
   record is never published (-1 = none), so that the waits on it run out.
   A call whose waits ran out returns WG_ERR_DEVICE (its message names the
   expired wait) and leaves its simulation unusable: every later call on it
   except wg_destroy returns WG_ERR_DEVICE.  The setting is process-wide and
   applies to launches made after the call. */
int wg_set_debug_wait(unsigned spin_limit, int64_t withhold_tile);

/* Page-lock (or release) caller memory so that downloads and uploads run
   at full link speed.  No reference counterpart (wendy's buffers are plain
   numpy arrays).  On the measured GB300 hosts a registered range loses most
   of its copy rate after tens of seconds of sustained device load (about
   190 -> 5 GB/s for downloads into it); memory from wg_host_alloc kept its
   rate in the same test.  Every download entry of this library also writes
   one byte per page of its destination before the copy: a page-locked
   buffer that only copies write falls to about 20 GB/s within a minute of
   repeated downloads, and a host write per page restores the full rate. */
int wg_host_register(void *ptr, int64_t bytes);
int wg_host_unregister(void *ptr);
/* Page-locked host memory (cudaHostAlloc) and its release; wg_host_free of
   NULL does nothing.  No reference counterpart. */
int wg_host_alloc(int64_t bytes, void **ptr);
int wg_host_free(void *ptr);

/* ---- stateless entry points ------------------------------------------- */

/* One force evaluation at positions x (original order): accelerations in
   original order and the sort permutation used (perm[i] = original index of
   the sheet at sorted slot i).  Either output may be NULL.
   Reference: _nbody_force, wendy/wendy.c:334-384. */
int wg_accel(int64_t n, const double *x, const double *m, double totmass, double omega2,
             int ext_kind, const double *ext_params, int n_ext_params, double t, double *a,
             int32_t *perm);

/* out[i] = F(x[i], t) of a registered external force, evaluated on the device
   by the force kernels' own code (for the pulsed force: the amplitude once,
   then amp * tanh(x / h) with the integer-pipe tanh).  The device side of the
   reference's ext_force(x, t) callables, wendy/wendy.py:389-418. */
int wg_ext_force_eval(int64_t n, const double *x, double t, int ext_kind,
                      const double *ext_params, int n_ext_params, double *out);

/* Counters of the state behind wg_nbody_approx_onestep (all zero before its
   first call).  A call handed back exactly the previous call's outputs, with
   the same masses and total, resumes from the resident sorted state and adds
   no full sort; any other call loads, sorts and lays out the sheets anew. */
int wg_nbody_approx_stats(wg_stats *out);

/* Drop-in shape of the reference's step function: same buffers, same
   in/out meaning (xi updated to the new sorted order and positions, x
   de-sorted, v updated, a = accelerations of the last force evaluation in
   original order, *t0 advanced), with the external force given as a
   registered id instead of a function pointer.  Every call uploads its
   inputs and downloads its outputs; a call whose inputs are bit for bit the
   previous call's outputs (the reference's generator loop) continues from
   the resident state instead of re-sorting it, and after such a call the
   next one's sub-steps are enqueued before returning (kept if the next
   call's scalars and inputs match, dropped otherwise): identical results,
   with the transfers under the sub-steps.
   Reference: _wendy_nbody_approx_onestep, wendy/wendy.c:385-418 and its
   argtypes at wendy/wendy.py:76-93. */
int wg_nbody_approx_onestep(int n, wg_sheet *xi, double *x, double *v, const double *m,
                            double *a, double totmass, double dt, int nleap, double *t0,
                            double omega2, int ext_kind, const double *ext_params,
                            int n_ext_params, int *err, double *time_elapsed);

/* ---- ensembles: many simulations resident on one GPU -------------------
   A pool holds any number of simulations (sheets, bucket layouts and
   look-back state of each in its own device allocation) and advances any
   subset of them by one output interval with one launch of the fused
   sub-step kernel per leapfrog sub-step.  Each simulation's arithmetic is
   that of _wendy_nbody_approx_onestep (wendy/wendy.c:385-418) and its result
   is bit-identical to running it alone; the reference itself has no
   ensemble API.  Simulations can be added and removed between steps
   (continuous batching). */
typedef struct wg_pool wg_pool;

/* Device bytes a simulation of n sheets holds in a pool (admission control). */
int64_t wg_pool_sim_bytes(int64_t n);
/* budget_bytes > 0 caps the bytes of all simulations (wg_pool_add returns
   WG_ERR_BUDGET beyond it); 0 = no cap. */
int wg_pool_create(int64_t budget_bytes, wg_pool **out);
/* Same inputs as wg_create; returns the simulation's id. */
int wg_pool_add(wg_pool *p, int64_t n, const double *x, const double *v, const double *m,
                double totmass, double omega2, int ext_kind, const double *ext_params,
                int n_ext_params, int *sim_id);
int wg_pool_remove(wg_pool *p, int sim_id);
/* Advance the `count` simulations ids[] by nleap sub-steps each (dt[k] is
   simulation k's dt_leap; t0[k] advances as in wg_step; t0 may be NULL). */
int wg_pool_step(wg_pool *p, int count, const int *ids, const double *dt, int nleap, double *t0,
                 double *time_elapsed);
/* wg_pool_step in two halves (enqueue, then wait and complete), as
   wg_step_begin / wg_step_end.  While a step is in flight, wg_pool_download
   returns each simulation's output completed before it (the step writes a
   second pair of output buffers), on a stream of its own, and wg_pool_add,
   wg_pool_remove and wg_pool_step return WG_ERR_ARG. */
int wg_pool_step_begin(wg_pool *p, int count, const int *ids, const double *dt, int nleap,
                       double *t0);
int wg_pool_step_end(wg_pool *p, double *time_elapsed);
/* (time_elapsed of a pool step: the device time of its launches, and of the
   recovery of simulations that overflowed a bucket, which runs in
   wg_pool_step_end -- not the time its stream waits for that call.) */
/* Positions and velocities of the last step, original order (during a step:
   of the last step completed before it). */
int wg_pool_download(wg_pool *p, int sim_id, double *x, double *v);
/* wg_pool_download of `count` simulations ids[] at once, their outputs one
   after another in x and v (each simulation's sheets in original order):
   every id is checked before anything is copied, the copies run back to back
   and the call returns when all have landed. */
int wg_pool_download_many(wg_pool *p, int count, const int *ids, double *x, double *v);
/* Counters of a pool since its creation.  No reference counterpart. */
typedef struct wg_pool_stats {
  int64_t steps;              /* pool steps (one per wg_pool_step or step_begin/step_end) */
  int64_t launches;           /* kernels the pool has launched */
  int64_t graph_builds;       /* captures of the per-step CUDA graph */
  int64_t members_sorted;     /* members sorted from scratch (joined, dt changed, compact) */
  int64_t overflows;          /* member sub-steps that overflowed a bucket */
  int64_t recovery_rounds;    /* rounds of recovery (segmented re-sort + relaunch) */
  int64_t sheets_resorted;    /* sheets those rounds re-sorted */
  int64_t substeps_relaunched; /* member sub-steps run again after a recovery */
  double graph_seconds;       /* device time of the steps' launches (CUDA events) */
  double recovery_seconds;    /* device time of their recoveries */
  int64_t members_compact;    /* members (of 2^20 sheets or more) that finished a step on the
                                 compact path, having overflowed again within two sub-steps
                                 of a re-sort */
  int64_t substeps_compact;   /* sub-steps they ran there (full re-sort + force kernel) */
} wg_pool_stats;
int wg_pool_get_stats(wg_pool *p, wg_pool_stats *out);
int wg_pool_info(wg_pool *p, int64_t *used_bytes, int64_t *budget_bytes, int *n_sims,
                 int64_t *launches);
int wg_pool_destroy(wg_pool *p);

/* ---- the exact event-driven solver (nbody(..., approx=False)) ----------
   wendy's exact path: every crossing of two neighbouring sheets is found
   and processed in time order (wendy/wendy.c:53-315, its Python set-up
   wendy/wendy.py:158-238).  One warp runs the event loop, with the state in
   shared memory when it fits.  A cross-check for small N, not a fast path:
   the events are a strict sequence.  The caller sets up the arrays as the
   reference's _setup_arrays does: x, v, masses m (times twopiG, and divided
   by omega^2 when omega > 0), accelerations a (mass above minus mass below;
   with omega, the equilibrium offset of the same formula) and the sort order
   sindx of x; the pair crossing times are computed on the device.
   omega <= 0: no harmonic potential.  n from 2 to what the pair-time tree's
   shared memory allows (about 600,000 sheets; WG_ERR_ARG beyond). */
typedef struct wg_exact wg_exact;
int wg_exact_create(int64_t n, const double *x, const double *v, const double *a,
                    const double *m, const int32_t *sindx, double omega, wg_exact **out);
/* One output interval dt: crossings until the next one lies beyond dt, at
   most maxcoll of them (then WG_ERR_MAXCOLL, with the state advanced as the
   reference's _wendy_nbody_onestep leaves it); *ncoll receives the number
   processed, *time_elapsed the device time of the event loop.
   Reference: _wendy_nbody_onestep and _wendy_nbody_harm_onestep,
   wendy/wendy.c:53-315. */
int wg_exact_step(wg_exact *e, double dt, int64_t maxcoll, int64_t *ncoll,
                  double *time_elapsed);
/* x, v, a in original order and the position order sindx (any may be NULL). */
int wg_exact_download(wg_exact *e, double *x, double *v, double *a, int32_t *sindx);
int wg_exact_destroy(wg_exact *e);

/* Allocation-free force evaluation (no counterpart in the reference).
   For callers that cannot call cudaMalloc themselves or let this library do
   so: an application whose device memory belongs to another framework's
   allocator and budget, code that must not trigger the device-wide
   synchronisation cudaMalloc and cudaFree imply, or a latency-critical loop
   that may not allocate.  Same result as wg_accel, but x, m, a and perm are
   DEVICE pointers the caller owns (a or perm may be NULL), the work runs on
   `stream` (a cudaStream_t; NULL = legacy default stream), and the call
   returns after that stream has finished it.  All intermediates live in one
   fixed __device__ array of this library (8 MiB, held by every GPU that loads
   the library until the process exits), so n is limited to
   WG_NOALLOC_MAX_SHEETS; larger n returns WG_ERR_ARG.  The first call on a
   device looks up the array's device address (cudaGetSymbolAddress): make
   that first call before any stream capture.  All calls share the array:
   calls that overlap on the GPU (other streams or host threads) race.  The
   inputs are checked on the device (they are device memory): a non-finite
   position or mass, or a negative mass, returns WG_ERR_ARG after the call's
   launches have run (the sort is skipped, `a` and `perm` are then undefined). */
#define WG_NOALLOC_MAX_SHEETS 65536
int wg_accel_noalloc(int64_t n, const double *x, const double *m, double totmass,
                     double omega2, int ext_kind, const double *ext_params, int n_ext_params,
                     double t, double *a, int32_t *perm, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* WENDY_GB300_H */
