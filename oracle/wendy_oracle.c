/*
  wendy_oracle.c -- TEST INFRASTRUCTURE ONLY.

  A plain-C restatement of wendy's approximate leapfrog integrator
  (wendy/wendy.c:317-418) and of the two CPU sorts it is timed with
  (the quick sort instantiated from wendy/sort.h:651-763 and the OpenMP
  task-parallel merge sort of wendy/parallel_sort.c:9-137).  It exists so
  that the CUDA implementation in wendy_gb300/ can be checked on machines
  where the reference itself is not present, and so that the reference's
  CPU path can be timed on the same host cores as the GPU.

  Only tests/, __graft_entry__.smoke() and bench.py (its CPU-baseline and
  reference legs) may load this library.  Nothing in the product links it.

  Parity of this restatement is pinned against the reference compiled from
  its own sources (oracle/Makefile, target `ref`) and against golden vectors
  produced by the reference (tests/golden/make_golden.py): for the same
  inputs and sort type the outputs are bit-identical (tests/test_oracle.py).

  Build flags: -O2 -fopenmp -ffp-contract=off, so that x86-64 and aarch64
  builds perform the same IEEE operations in the same order.
*/
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#else
#include <time.h>
static double omp_get_wtime(void) { return (double)clock() / CLOCKS_PER_SEC; }
#endif

/* Same memory layout as `struct array_w_index` (wendy/wendy.h:12-16):
   int idx, 4 bytes of padding, double val -> 16 bytes. */
typedef struct {
  int idx;
  double val;
} wo_sheet;

/* Chunk size of the reference's OpenMP loops (wendy/wendy.h:6-8). */
#define WO_CHUNK 1000
/* Below this N the reference evaluates ext_force one sheet at a time
   (wendy/wendy.h:9-11, wendy/wendy.c:362-370). */
#define WO_EXTERNAL_SWITCH 10

/* Three-way comparison on positions, as SORT_CMP at wendy/wendy.c:21. */
static inline int wo_cmp(const wo_sheet *a, const wo_sheet *b) {
  return (a->val < b->val) ? -1 : ((a->val > b->val) ? 1 : 0);
}
static int wo_cmp_void(const void *a, const void *b) {
  return wo_cmp((const wo_sheet *)a, (const wo_sheet *)b);
}
static inline void wo_swap(wo_sheet *a, wo_sheet *b) {
  wo_sheet t = *a;
  *a = *b;
  *b = t;
}

/* ---------------------------------------------------------------------
   Quick sort, restating the algorithm wendy instantiates from sort.h:
   middle-element pivot moved to the right end, Lomuto partition that
   records whether every key equals the pivot (sort.h:651-680), binary
   insertion sort for ranges shorter than 16 (sort.h:733-739, 290-367).
   The tie order it produces is the reference's, which keeps the oracle
   bit-identical to the reference even for coincident positions.
   --------------------------------------------------------------------- */

/* Insertion point of x in sorted a[0..n) (n >= 1), favouring the right
   among equal keys (sort.h:290-327).  Only called when x < a[n-1]. */
static size_t wo_insert_pos(const wo_sheet *a, const wo_sheet *x, size_t n) {
  size_t lo = 0, hi = n - 1, mid;
  if (wo_cmp(x, &a[0]) < 0) return 0;
  if (wo_cmp(x, &a[hi]) > 0) return hi;
  mid = hi >> 1;
  for (;;) {
    if (wo_cmp(x, &a[mid]) < 0) {
      if (mid - lo <= 1) return mid;
      hi = mid;
    } else {
      if (hi - mid <= 1) return mid + 1;
      lo = mid;
    }
    mid = lo + ((hi - lo) >> 1);
  }
}

static void wo_binary_insertion_sort(wo_sheet *a, size_t n) {
  size_t i, j, at;
  wo_sheet x;
  for (i = 1; i < n; i++) {
    if (wo_cmp(&a[i - 1], &a[i]) <= 0) continue;
    x = a[i];
    at = wo_insert_pos(a, &x, i);
    for (j = i; j > at; j--) a[j] = a[j - 1];
    a[at] = x;
  }
}

/* Returns the final pivot slot, or SIZE_MAX when every key in [lo,hi]
   compared equal to the pivot (sort.h:651-680). */
static size_t wo_partition(wo_sheet *a, size_t lo, size_t hi, size_t p) {
  wo_sheet pivot = a[p];
  size_t store = lo, i;
  int differs = 0;
  wo_swap(&a[p], &a[hi]);
  for (i = lo; i < hi; i++) {
    int c = wo_cmp(&a[i], &pivot);
    differs |= c;
    if (c < 0) {
      wo_swap(&a[i], &a[store]);
      store++;
    }
  }
  wo_swap(&a[hi], &a[store]);
  return differs ? store : SIZE_MAX;
}

static void wo_quick_rec(wo_sheet *a, size_t lo, size_t hi) {
  size_t p;
  if (hi <= lo) return;
  if (hi - lo + 1 < 16) {
    wo_binary_insertion_sort(a + lo, hi - lo + 1);
    return;
  }
  p = wo_partition(a, lo, hi, lo + ((hi - lo) >> 1));
  if (p == SIZE_MAX) return;
  if (p > lo) wo_quick_rec(a, lo, p - 1);
  wo_quick_rec(a, p + 1, hi);
}

void wo_quick_sort(wo_sheet *a, size_t n) {
  if (n > 1) wo_quick_rec(a, 0, n - 1);
}

/* ---------------------------------------------------------------------
   Task-parallel merge sort restating wendy/parallel_sort.c.  The thread
   count and the two serial switches are compile-time macros in the
   reference (parallel_sort.h:7-15); here they are runtime settings so one
   build can be timed with the host's core count.
   --------------------------------------------------------------------- */
static int wo_par_threads = 32;
static size_t wo_par_sort_switch = 10000;
static size_t wo_par_merge_switch = 50000;

void wo_set_parallel_sort(int nthreads, long sort_switch, long merge_switch) {
  if (nthreads > 0) wo_par_threads = nthreads;
  if (sort_switch > 0) wo_par_sort_switch = (size_t)sort_switch;
  if (merge_switch > 0) wo_par_merge_switch = (size_t)merge_switch;
}

/* parallel_sort.c:9-46 */
static void wo_merge_serial(const wo_sheet *l, const wo_sheet *r, wo_sheet *out,
                            size_t nl, size_t nr) {
  const wo_sheet *le = l + nl, *re = r + nr;
  if (wo_cmp(le - 1, r) < 0) {
    memcpy(out, l, nl * sizeof(wo_sheet));
    memcpy(out + nl, r, nr * sizeof(wo_sheet));
    return;
  }
  if (wo_cmp(re - 1, l) < 0) {
    memcpy(out, r, nr * sizeof(wo_sheet));
    memcpy(out + nr, l, nl * sizeof(wo_sheet));
    return;
  }
  while (l < le && r < re) *out++ = (wo_cmp(r, l) < 0) ? *r++ : *l++;
  if (l < le)
    memcpy(out, l, (size_t)(le - l) * sizeof(wo_sheet));
  else if (r < re)
    memcpy(out, r, (size_t)(re - r) * sizeof(wo_sheet));
}

/* parallel_sort.c:47-67: first slot of a[0..n) whose key is >= *x. */
static size_t wo_lower_slot(const wo_sheet *a, const wo_sheet *x, size_t n) {
  size_t lo, hi, mid;
  if (wo_cmp(x, a) < 0) return 0;
  if (wo_cmp(x, a + (n - 1)) > 0) return n;
  lo = 0;
  hi = n - 1;
  while (wo_cmp(a + lo, a + hi) < 0) {
    mid = lo + (hi - lo) / 2;
    if (wo_cmp(x, a + mid) <= 0)
      hi = mid;
    else
      lo = mid + 1;
  }
  return lo;
}

/* parallel_sort.c:68-94 */
static void wo_merge_par(const wo_sheet *s1, const wo_sheet *s2, wo_sheet *out,
                         size_t n1, size_t n2) {
  size_t half, cut;
  if (n1 + n2 < wo_par_merge_switch) {
    wo_merge_serial(s1, s2, out, n1, n2);
    return;
  }
  if (n1 < n2) {
    wo_merge_par(s2, s1, out, n2, n1);
    return;
  }
  half = n1 / 2;
  cut = wo_lower_slot(s2, s1 + half, n2);
  out[half + cut] = s1[half];
#pragma omp task
  wo_merge_par(s1, s2, out, half, cut);
#pragma omp task
  wo_merge_par(s1 + half + 1, s2 + cut, out + half + 1 + cut, n1 - half - 1,
               n2 - cut);
#pragma omp taskwait
}

/* parallel_sort.c:95-127 */
static void wo_mergesort_par(wo_sheet *src, wo_sheet *dst, size_t n, int to_dst) {
  size_t h = n / 2;
  if (n < wo_par_sort_switch) {
    if (to_dst) {
      qsort(src, n, sizeof(wo_sheet), wo_cmp_void);
      memcpy(dst, src, n * sizeof(wo_sheet));
    } else {
      qsort(dst, n, sizeof(wo_sheet), wo_cmp_void);
      memcpy(src, dst, n * sizeof(wo_sheet));
    }
    return;
  }
#pragma omp task
  wo_mergesort_par(src, dst, h, !to_dst);
#pragma omp task
  wo_mergesort_par(src + h, dst + h, n - h, !to_dst);
#pragma omp taskwait
  if (to_dst)
    wo_merge_par(src, src + h, dst, h, n - h);
  else
    wo_merge_par(dst, dst + h, src, h, n - h);
}

/* parallel_sort.c:128-137 */
void wo_parallel_sort(wo_sheet *a, size_t n) {
  wo_sheet *aux = (wo_sheet *)malloc(n * sizeof(wo_sheet));
  memcpy(aux, a, n * sizeof(wo_sheet));
#pragma omp parallel num_threads(wo_par_threads)
#pragma omp single
  wo_mergesort_par(aux, a, n, 1);
  free(aux);
}

/* ---------------------------------------------------------------------
   External forces.  The reference takes an arbitrary callback with the
   signature double f(int N, double *x, double t, double *a)
   (wendy/wendy.py:389-418).  The rebuild replaces callables by registered
   closed forms; the oracle evaluates the same closed forms in C.
     kind 0: none
     kind 1: harmonic,     F = -p[0] * x                (p[0] = omega^2)
     kind 2: pulsed tanh,  F = p[0]*exp(-(t-p[1])^2/(2 p[2]^2))*tanh(x/p[3])
     kind 3: a compiled expression (below)
   The expression order matches the numpy expression
   A*numpy.exp(-(t-t0)**2/(2*tau**2))*numpy.tanh(x/h).
   --------------------------------------------------------------------- */
#define WO_EXT_NONE 0
#define WO_EXT_HARMONIC 1
#define WO_EXT_PULSE_TANH 2
#define WO_EXT_EXPR 3

/* kind 3: a compiled expression F(x, t), the register program of the
   library's WG_EXT_EXPR (wendy_gb300/extforce.py writes it): p[0] ops,
   p[1] of them free of x, then (code, dst, a, b, constant) per op; F is the
   register the last op writes.  Evaluated here op by op in libm double
   arithmetic, the way the reference evaluates a numba-compiled callable. */
static double wo_expr_eval(const double *p, double x, double t) {
  double r[16] = {0};
  int i, n = (int)p[0];
  for (i = 0; i < n; i++) {
    const double *q = p + 2 + 5 * i;
    int code = (int)q[0], dst = (int)q[1], a = (int)q[2], b = (int)q[3];
    double va = r[a], vb = r[b], y;
    switch (code) {
      case 0: y = x; break;
      case 1: y = t; break;
      case 2: y = q[4]; break;
      case 3: y = va; break;
      case 4: y = va + vb; break;
      case 5: y = va - vb; break;
      case 6: y = va * vb; break;
      case 7: y = va / vb; break;
      case 8: y = -va; break;
      case 9: y = pow(va, vb); break;
      case 10: y = exp(va); break;
      case 11: y = log(va); break;
      case 12: y = sqrt(va); break;
      case 13: y = sin(va); break;
      case 14: y = cos(va); break;
      case 15: y = tan(va); break;
      case 16: y = tanh(va); break;
      case 17: y = sinh(va); break;
      case 18: y = cosh(va); break;
      case 19: y = atan(va); break;
      default: y = fabs(va); break;
    }
    r[dst] = y;
  }
  return r[(int)p[2 + 5 * (n - 1) + 1]];
}

static double wo_ext_eval(int kind, const double *p, double x, double t) {
  if (kind == WO_EXT_HARMONIC) return -p[0] * x;
  if (kind == WO_EXT_PULSE_TANH) {
    double dt = t - p[1];
    double amp = p[0] * exp(-(dt * dt) / (2. * (p[2] * p[2])));
    return amp * tanh(x / p[3]);
  }
  if (kind == WO_EXT_EXPR) return wo_expr_eval(p, x, t);
  return 0.;
}

/* A C callback with the reference's ext_force signature, so that the
   reference library built from its own sources can be driven with the same
   registered force (the reference passes `a` in original order for N > 10
   and asks for one scalar when N == 1, wendy/wendy.py:397-403). */
#define WO_MAX_PARAMS (2 + 5 * 64)
static int wo_cb_kind = WO_EXT_NONE;
static double wo_cb_params[WO_MAX_PARAMS];
void wo_set_callback_force(int kind, const double *params, int nparams) {
  int i;
  wo_cb_kind = kind;
  for (i = 0; i < nparams && i < WO_MAX_PARAMS; i++) wo_cb_params[i] = params[i];
}
double wo_callback_force(int n, double *x, double t, double *a) {
  int i;
  if (n == 1) return wo_ext_eval(wo_cb_kind, wo_cb_params, x[0], t);
  for (i = 0; i < n; i++) a[i] = wo_ext_eval(wo_cb_kind, wo_cb_params, x[i], t);
  return 0.;
}

/* ---------------------------------------------------------------------
   The integrator.
   --------------------------------------------------------------------- */
#define WO_SORT_QUICK 0
#define WO_SORT_QSORT 3
#define WO_SORT_PARALLEL 4

static void wo_sort(wo_sheet *xi, int n, int sort_kind) {
  if (sort_kind == WO_SORT_QSORT)
    qsort(xi, (size_t)n, sizeof(wo_sheet), wo_cmp_void);
  else if (sort_kind == WO_SORT_PARALLEL)
    wo_parallel_sort(xi, (size_t)n);
  else
    wo_quick_sort(xi, (size_t)n);
}

/* Position update of every sheet, reached through its index
   (wendy/wendy.c:318-323). */
static void wo_drift(int n, wo_sheet *xi, const double *v, double dt) {
  int i;
#pragma omp parallel for schedule(static, WO_CHUNK) private(i)
  for (i = 0; i < n; i++) xi[i].val += dt * v[xi[i].idx];
}

/* Kick then drift (wendy/wendy.c:324-333). */
static void wo_kick_drift(int n, wo_sheet *xi, double *v, const double *a,
                          double dt_kick, double dt_drift) {
  int i;
#pragma omp parallel for schedule(static, WO_CHUNK) private(i)
  for (i = 0; i < n; i++) {
    v[xi[i].idx] += dt_kick * a[xi[i].idx];
    xi[i].val += dt_drift * v[xi[i].idx];
  }
}

/* Sort, serial exclusive prefix sum of the masses in sorted order, then
   a = ext + (M - 2 C_i - m_i [- omega2 x_i]) scattered to original order
   (wendy/wendy.c:334-384).  Masses are already multiplied by 2 pi G. */
static void wo_force(int n, int sort_kind, wo_sheet *xi, double *x, const double *m,
                     double *a, double t, double totmass, double omega2,
                     int ext_kind, const double *ext_params, double *cumulmass) {
  int i;
  wo_sort(xi, n, sort_kind);
  for (i = 0; i < n - 1; i++) cumulmass[i + 1] = cumulmass[i] + m[xi[i].idx];
  if (ext_kind != WO_EXT_NONE && n > WO_EXTERNAL_SWITCH) {
#pragma omp parallel for schedule(static, WO_CHUNK) private(i)
    for (i = 0; i < n; i++) x[xi[i].idx] = xi[i].val;
#pragma omp parallel for schedule(static, WO_CHUNK) private(i)
    for (i = 0; i < n; i++) a[i] = wo_ext_eval(ext_kind, ext_params, x[i], t);
  } else if (ext_kind != WO_EXT_NONE) {
    for (i = 0; i < n; i++)
      a[xi[i].idx] = wo_ext_eval(ext_kind, ext_params, xi[i].val, t);
  } else {
#pragma omp parallel for schedule(static, WO_CHUNK) private(i)
    for (i = 0; i < n; i++) a[i] = 0.;
  }
  if (omega2 < 0) {
#pragma omp parallel for schedule(static, WO_CHUNK) private(i)
    for (i = 0; i < n; i++)
      a[xi[i].idx] += totmass - 2 * cumulmass[i] - m[xi[i].idx];
  } else {
#pragma omp parallel for schedule(static, WO_CHUNK) private(i)
    for (i = 0; i < n; i++)
      a[xi[i].idx] += totmass - 2 * cumulmass[i] - m[xi[i].idx] - omega2 * xi[i].val;
  }
}

/* One output interval of nleap leapfrog sub-steps (wendy/wendy.c:385-418):
   half drift, (nleap-1) x [force, kick, drift], force, kick, half drift,
   then the positions are written back in original order.  *t0 advances by
   dt per force evaluation, by repeated addition, only when an external
   force is set (wendy/wendy.c:403-404,409-410).  cumulmass[0] must be 0 on
   entry and is never written (wendy/wendy.py:372). */
void wo_approx_onestep(int n, wo_sheet *xi, double *x, double *v, const double *m,
                       double *a, double totmass, double dt, int nleap, double *t0,
                       double omega2, int ext_kind, const double *ext_params,
                       int sort_kind, double *time_elapsed, double *cumulmass) {
  int i;
  double t_begin = omp_get_wtime();
  wo_drift(n, xi, v, dt / 2.);
  for (i = 0; i < nleap - 1; i++) {
    wo_force(n, sort_kind, xi, x, m, a, *t0, totmass, omega2, ext_kind, ext_params,
             cumulmass);
    if (ext_kind != WO_EXT_NONE) *t0 += dt;
    wo_kick_drift(n, xi, v, a, dt, dt);
  }
  wo_force(n, sort_kind, xi, x, m, a, *t0, totmass, omega2, ext_kind, ext_params,
           cumulmass);
  if (ext_kind != WO_EXT_NONE) *t0 += dt;
  wo_kick_drift(n, xi, v, a, dt, dt / 2.);
#pragma omp parallel for schedule(static, WO_CHUNK) private(i)
  for (i = 0; i < n; i++) x[xi[i].idx] = xi[i].val;
  *time_elapsed = omp_get_wtime() - t_begin;
}

/* Accelerations of one force evaluation on a given (unsorted) state, in
   original order, with the sort permutation it used: the quantity the
   GPU's fused kernel is checked against.  perm[i] is the original index
   of the sheet at sorted slot i. */
void wo_accel(int n, const double *x, const double *m, double totmass, double omega2,
              int ext_kind, const double *ext_params, double t, double *a, int *perm,
              int sort_type) {
  int i;
  wo_sheet *xi = (wo_sheet *)malloc((size_t)n * sizeof(wo_sheet));
  double *xs = (double *)malloc((size_t)n * sizeof(double));
  double *cm = (double *)calloc((size_t)n, sizeof(double));
  for (i = 0; i < n; i++) {
    xi[i].idx = i;
    xi[i].val = x[i];
    xs[i] = x[i];
  }
  wo_force(n, sort_type, xi, xs, m, a, t, totmass, omega2, ext_kind, ext_params, cm);
  if (perm)
    for (i = 0; i < n; i++) perm[i] = xi[i].idx;
  free(xi);
  free(xs);
  free(cm);
}

int wo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
