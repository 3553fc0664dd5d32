// wg_internal.cuh -- data layout and kernel launchers shared by the
// translation units of the library (not part of the C ABI).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "wg_common.cuh"

namespace wg {

// Sorted structure-of-arrays record of the sheets, FP64 throughout:
// position, velocity, mass (already times 2 pi G) and the original index.
// The library keeps two such sets and flips between them when a sort
// permutes the sheets; kernels reach the current set through a small
// device-resident table so that a device-side decision (skip the sort or
// not) needs no host round trip and the sequence can live in a CUDA graph.
struct StateRef {
  double* x;
  double* v;
  double* m;
  int32_t* idx;
};

struct StateTable {
  StateRef cur;    // sorted set the next force kernel reads
  StateRef other;  // the other set (gather target)
};

// Decoupled look-back record of one force-kernel tile (48 bytes).
struct __align__(16) TileRec {
  uint64_t agg_lo, agg_hi;  // tile's own fixed-point mass sum
  uint64_t inc_lo, inc_hi;  // inclusive prefix through this tile
  uint64_t last_key;        // post-drift key of the tile's last sheet
  unsigned flag;            // (epoch << 2) | {1: aggregate, 2: inclusive}
  unsigned last_flag;       // epoch once last_key is valid
};

// Per-sub-step bookkeeping written by the device (one slot per sub-step).
struct StepFlags {
  unsigned unsorted;         // nonzero: the order after this drift is not strictly increasing
  unsigned max_cnt;          // largest bucket count of the layout this sub-step wrote
  unsigned long long max_v;  // largest |v| after the kick (bit pattern of a non-negative double)
};

struct ForceArgs {
  const StateTable* table;
  int64_t n;
  uint64_t T_lo, T_hi;  // totmass in fixed point
  int E;                // fixed-point scale exponent
  int has_omega;
  double omega2;
  double dt_kick, dt_drift;
  ExtForce ext;
  const double* t_seq;       // time of each force evaluation of this call
  const unsigned* epochs;    // look-back epoch of each force evaluation of this call
  int sub;                   // index of this sub-step within the call
  double* a_out;             // optional: accelerations in sorted order
  TileRec* recs;
  unsigned* ticket;          // tile ticket counter, zero before the launch
  StepFlags* flag_out;       // order / speed record of the positions this drift produces
  unsigned* err;
  // filled in by launch_force from the wait settings (set_wait_debug): the
  // look-back's iteration limit and a tile that leaves its record unpublished
  unsigned spin_limit;
  int64_t withhold_tile;     // -1: none
};

// Radix-sort workspace (one set per simulation).
struct RadixWork {
  uint64_t* keys[2];
  uint32_t* pos[2];
  uint32_t* hist;       // 8 x 256 digit counts
  uint32_t* plan;       // per-pass: active, src, dst; final buffer; digit starts
  uint32_t* status;     // 8 passes x tiles x 256 look-back words
  uint32_t* counters;   // 8 tile tickets + tie flag
  int64_t n_tiles;
  size_t scratch_bytes; // bytes of status + counters (cleared before each sort)
};

// Devices whose one-time kernel set-up (attributes, occupancy) is cached;
// launchers on a device beyond this redo the set-up on every call.
constexpr int kMaxDevices = 64;
// The calling thread's current device, or -1 when none can be had.
inline int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return d;
}

// The tanh table of the pulsed force (wg_tanh.cuh) on the current device,
// computed there by its first call (a kernel on the legacy stream, waited
// for; no allocation: the table is a __device__ array of the library), or
// nullptr when the device cannot be reached.  Call it before any stream
// capture, as every entry point does when it parses a force.
const long long* tanh_table();

constexpr int kForceThreads = 256;
constexpr int kForceItems = 8;
constexpr int kForceTile = kForceThreads * kForceItems;

constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 16;
constexpr int kRadixTile = kRadixThreads * kRadixItems;

// --- launchers (wg_kernels.cu) ---
void launch_force(const ForceArgs& a, int64_t n_tiles, cudaStream_t s);
// Wait settings of the force kernel's look-back (a test hook behind
// wg_set_debug_wait): the iteration limit of its waits, and a tile whose
// look-back record is never published (-1: none), so that the waits on it
// run out.  Defaults kSpinLimit and -1.
void set_wait_debug(unsigned spin_limit, int64_t withhold_tile);
void launch_drift(const StateTable* table, int64_t n, double dt, StepFlags* flag, cudaStream_t s);
void launch_desort(const StateTable* table, int64_t n, double* x_out, double* v_out,
                   cudaStream_t s);
void launch_scatter_accel(const StateTable* table, int64_t n, const double* a_sorted,
                          double* a_orig, cudaStream_t s);
void launch_init_state(StateTable* table, int64_t n, cudaStream_t s);
// Energy / momentum sums of the sorted state (deterministic): scratch[0..3]
// receives sum m v^2/2, sum m x^2/2, -sum m x a, sum m v; scratch holds
// 4 (kEnergyBlocks + 1) doubles.
constexpr int kEnergyBlocks = 152 * 4;
void launch_ext_eval(const ExtForce& f, double t, const double* x, double* out, int64_t n,
                     cudaStream_t s);
void launch_energy(const StateTable* table, int64_t n, const double* a_sorted, double* scratch,
                   cudaStream_t s);

// Record a message for wg_last_error() (wg_api.cu).
void record_last_error(const char* msg);
// Writes one byte in every memory page of the host range [p, p + bytes),
// which a device-to-host copy is about to overwrite.  On the measured GB300
// hosts the copy engine's writes into page-locked pages that the host has not
// written for some seconds run at a fraction of the link's rate (about 20
// instead of 145 GB/s for a 9.9 GB download into a buffer written only by
// copies); a host write to each page first restores the full rate.
void host_pages_dirty(void* p, size_t bytes);

// --- launchers (wg_radix.cu) ---
constexpr int kRadixLaunches = 14;  // kernels radix_sort_state enqueues (hist, plan, 8 passes,
                                    // gather, ties, long ties, flip)
size_t radix_bytes(int64_t n);
void radix_bind(RadixWork* w, void* base, int64_t n);
// Sort table->cur by (position key, original index) unless flags->unsorted
// is zero; the sorted sheets end in table->cur (the sets are swapped on the
// device).  err receives DEV_ERR_RADIX_TIMEOUT if a wait expired.
void radix_sort_state(StateTable* table, int64_t n, RadixWork* w, const StepFlags* flag,
                      unsigned* err, cudaStream_t s);

}  // namespace wg
