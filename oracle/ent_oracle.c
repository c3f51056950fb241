/*
 * ent_oracle.c -- CPU oracle for the entropical density hot path.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the CPU
 * baseline leg of bench.py as the checker, never by the product. See
 * ent_oracle.h for what each function restates and how parity is pinned.
 *
 * Compiled with -ffp-contract=off so that no a*b+c is fused on either host
 * architecture; float expressions follow the reference's C++ promotion rules
 * (float op double -> double, assigned back to float where the reference
 * stores into a float).
 */
#include "ent_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ sorting */

typedef struct {
  double v;
  uint32_t i;
} kv_t;

static int kv_cmp(const void* a, const void* b) {
  const kv_t* x = (const kv_t*)a;
  const kv_t* y = (const kv_t*)b;
  if (x->v < y->v) return -1;
  if (x->v > y->v) return 1;
  return (x->i > y->i) - (x->i < y->i);
}

static uint32_t* sorted_perm(const float* x, size_t n) {
  kv_t* kv = (kv_t*)malloc(n * sizeof(kv_t));
  uint32_t* p = (uint32_t*)malloc(n * sizeof(uint32_t));
  for (size_t i = 0; i < n; ++i) {
    kv[i].v = x[i];
    kv[i].i = (uint32_t)i;
  }
  qsort(kv, n, sizeof(kv_t), kv_cmp);
  for (size_t i = 0; i < n; ++i) p[i] = kv[i].i;
  free(kv);
  return p;
}

static int f32_cmp(const void* a, const void* b) {
  float x = *(const float*)a, y = *(const float*)b;
  return (x > y) - (x < y);
}

/* first index k in sorted s[0..n) with s[k] >= v (double compare) */
static size_t lower_bound_d(const double* s, size_t n, double v) {
  size_t lo = 0, hi = n;
  while (lo < hi) {
    size_t m = lo + (hi - lo) / 2;
    if (s[m] < v) lo = m + 1; else hi = m;
  }
  return lo;
}
static size_t upper_bound_d(const double* s, size_t n, double v) {
  size_t lo = 0, hi = n;
  while (lo < hi) {
    size_t m = lo + (hi - lo) / 2;
    if (s[m] <= v) lo = m + 1; else hi = m;
  }
  return lo;
}

/* ------------------------------------------------------ FP64 brute force */

int orc_density_fp64_at(const float* sel, size_t n, int d, const double* h,
                        double norm, const uint32_t* targets, size_t n_targets,
                        double* out) {
  if (d < 1 || d > 3 || n == 0) return 1;
  uint32_t* p = sorted_perm(sel, n);
  double* s = (double*)malloc(n * sizeof(double) * (size_t)d);
  for (size_t k = 0; k < n; ++k)
    for (int j = 0; j < d; ++j) s[(size_t)j * n + k] = sel[(size_t)j * n + p[k]];
  free(p);
#pragma omp parallel for schedule(dynamic, 64)
  for (size_t t = 0; t < n_targets; ++t) {
    size_t i = targets ? targets[t] : t;
    double x[3];
    for (int j = 0; j < d; ++j) x[j] = sel[(size_t)j * n + i];
    size_t lo = lower_bound_d(s, n, x[0] - h[0]);
    size_t hi = upper_bound_d(s, n, x[0] + h[0]);
    double acc = 0.0;
    for (size_t k = lo; k < hi; ++k) {
      double w = 1.0;
      for (int j = 0; j < d; ++j) {
        double u = (x[j] - s[(size_t)j * n + k]) / h[j];
        double u2 = u * u;
        if (u2 > 1.0) { w = 0.0; break; }
        w *= 0.75 * (1.0 - u2) / h[j];
      }
      acc += w;
    }
    out[t] = acc / norm;
  }
  free(s);
  return 0;
}

int orc_density_fp64(const float* sel, size_t n, int d, const double* h,
                     double norm, double* out) {
  return orc_density_fp64_at(sel, n, d, h, norm, NULL, n, out);
}

uint64_t orc_support_count_fp64(const float* sel, size_t n, int d,
                                const double* h) {
  if (d < 1 || d > 3 || n == 0) return 0;
  uint32_t* p = sorted_perm(sel, n);
  double* s = (double*)malloc(n * sizeof(double) * (size_t)d);
  for (size_t k = 0; k < n; ++k)
    for (int j = 0; j < d; ++j) s[(size_t)j * n + k] = sel[(size_t)j * n + p[k]];
  free(p);
  uint64_t tot = 0;
#pragma omp parallel for reduction(+ : tot) schedule(dynamic, 64)
  for (size_t i = 0; i < n; ++i) {
    double x[3];
    for (int j = 0; j < d; ++j) x[j] = s[(size_t)j * n + i];
    size_t lo = lower_bound_d(s, n, x[0] - h[0]);
    size_t hi = upper_bound_d(s, n, x[0] + h[0]);
    for (size_t k = lo; k < hi; ++k) {
      int in = 1;
      for (int j = 1; j < d && in; ++j) in = fabs(x[j] - s[(size_t)j * n + k]) <= h[j];
      tot += (uint64_t)in;
    }
  }
  free(s);
  return tot;
}

/* ------------------------------------------- reference float restatement */

/* Densities::OMP::epanechnikov::operator() (densities_omp.cpp:19-26):
 * u = (ref - val)/h in float, squared in float; the kept branch is
 * 0.75 * (1.0f - u^2) in double, divided by h in double, returned as float. */
static float epa_ref(float ref, float val, float h) {
  float u2 = (ref - val) / h;
  u2 *= u2;
  double k = (u2 <= 1.0f ? 0.75 * (double)(1.0f - u2) : 0.0) / (double)h;
  return (float)k;
}

/* boxes() (densities_omp.cpp:33-65). The two linear scans search monotone
 * predicates (float subtraction is monotone), so the first/last hits are
 * found by bisection with the identical float compares. */
static void boxes_of(const float* sorted, size_t n, float ref, float h,
                     size_t* lo_out, size_t* hi_out) {
  size_t lo = 0, hi = n; /* first k with ref - s[k] < h */
  while (lo < hi) {
    size_t m = lo + (hi - lo) / 2;
    if (ref - sorted[m] < h) hi = m; else lo = m + 1;
  }
  *lo_out = lo;
  lo = 0; hi = n; /* last k with s[k] - ref < h: first k failing, minus one */
  while (lo < hi) {
    size_t m = lo + (hi - lo) / 2;
    if (sorted[m] - ref < h) lo = m + 1; else hi = m;
  }
  *hi_out = lo - 1;
}

void orc_boxes(const float* col, size_t n, float h, uint64_t* lo, uint64_t* hi) {
  float* s = (float*)malloc(n * sizeof(float));
  memcpy(s, col, n * sizeof(float));
  qsort(s, n, sizeof(float), f32_cmp);
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < n; ++i) {
    size_t a, b;
    boxes_of(s, n, col[i], h, &a, &b);
    lo[i] = a;
    hi[i] = b;
  }
  free(s);
}

/* The reference's own scans (densities_omp.cpp:49-62): from the front for
 * the first hit, from the back for the last. Same result as boxes_of(), at
 * the reference's O(n) cost per point; used to time the CPU baseline. */
static void boxes_linear(const float* sorted, size_t n, float ref, float h,
                         size_t* lo_out, size_t* hi_out) {
  size_t k;
  for (k = 0; k < n; ++k)
    if (ref - sorted[k] < h) { *lo_out = k; break; }
  for (k = n; k > 0; --k)
    if (sorted[k - 1] - ref < h) { *hi_out = k - 1; break; }
}

static int density_ref_f32_impl(const float* sel, size_t n, int d,
                                const float* h, float* out, int linear);

int orc_density_ref_f32(const float* sel, size_t n, int d, const float* h,
                        float* out) {
  return density_ref_f32_impl(sel, n, d, h, out, 0);
}

int orc_density_ref_f32_linear(const float* sel, size_t n, int d,
                               const float* h, float* out) {
  return density_ref_f32_impl(sel, n, d, h, out, 1);
}

static int density_ref_f32_impl(const float* sel, size_t n, int d,
                                const float* h, float* out, int linear) {
  if (d < 1 || d > 3 || n == 0) return 1;
  /* dim1_sorted_coords (tools.hxx:113-150): rows sorted on column 0 */
  uint32_t* p = sorted_perm(sel, n);
  float* s = (float*)malloc(n * sizeof(float) * (size_t)d);
  for (size_t k = 0; k < n; ++k)
    for (int j = 0; j < d; ++j) s[(size_t)j * n + k] = sel[(size_t)j * n + p[k]];
  free(p);
  float fn = (float)n;
#pragma omp parallel for schedule(dynamic, 16)
  for (size_t i = 0; i < n; ++i) {
    size_t lo = 0, hi = 0;
    if (linear) boxes_linear(s, n, sel[i], h[0], &lo, &hi);
    else boxes_of(s, n, sel[i], h[0], &lo, &hi);
    float acc = 0.0f;
    for (size_t k = lo; k <= hi && k < n; ++k) {
      float e = epa_ref(sel[i], s[k], h[0]);
      if (d >= 2) e = e * epa_ref(sel[n + i], s[n + k], h[1]);
      if (d >= 3) e = e * epa_ref(sel[2 * n + i], s[2 * n + k], h[2]);
      acc = acc + e;
    }
    out[i] = acc / fn;
  }
  free(s);
  return 0;
}

/* ------------------------------------------------------- boxed search */

uint64_t orc_boxedsearch(const float* col, size_t n, float box_size,
                         uint64_t* box_of_state, uint64_t* n_neighbors) {
  float mn = FLT_MAX, mx = -FLT_MAX;
  for (size_t i = 0; i < n; ++i) {
    mn = col[i] < mn ? col[i] : mn;
    mx = col[i] > mx ? col[i] : mx;
  }
  /* boxedsearch.cpp:27 */
  uint64_t nb = (uint64_t)ceil((double)((mx - mn) / box_size));
  if (nb == 0) nb = 1;
  uint64_t* cnt = (uint64_t*)calloc(nb, sizeof(uint64_t));
  for (size_t i = 0; i < n; ++i) {
    /* boxedsearch.cpp:31 */
    uint64_t b = (uint64_t)floor((double)((col[i] - mn) / box_size));
    if (b >= nb) b = nb - 1;
    box_of_state[i] = b;
    cnt[b]++;
  }
  /* neighbour list = own box and the adjacent boxes (boxedsearch.cpp:35-57) */
  for (size_t i = 0; i < n; ++i) {
    uint64_t b = box_of_state[i];
    uint64_t c = cnt[b];
    if (b > 0) c += cnt[b - 1];
    if (b + 1 < nb) c += cnt[b + 1];
    n_neighbors[i] = c;
  }
  free(cnt);
  return nb;
}

/* ------------------------------------------------ AMISE / hestimate */

typedef struct {
  float s, c;
} kahan_t;
static void kahan_add(kahan_t* k, float x) {
  volatile float y = x - k->c;
  volatile float t = k->s + y;
  volatile float tm = t - k->s;
  k->c = tm - y;
  k->s = t;
}

float orc_epa_conv_ref(const float* sorted, size_t n, float h) {
  float* outer = (float*)malloc(n * sizeof(float));
#pragma omp parallel for schedule(dynamic, 8)
  for (size_t i = 0; i < n; ++i) {
    kahan_t k = {0.0f, 0.0f};
    float ci = sorted[i];
    for (size_t j = 0; j < n; ++j) {
      float dd = fabsf(ci - sorted[j]) / h;
      float term = 0.0f;
      if (dd <= 2) term = (float)fma((double)dd, -2.25, 4.5);
      kahan_add(&k, term);
    }
    outer[i] = k.s;
  }
  kahan_t k = {0.0f, 0.0f};
  for (size_t i = 0; i < n; ++i) kahan_add(&k, outer[i]);
  free(outer);
  return k.s / (float)(n * n);
}

double orc_epa_conv_fp64(const float* sorted, size_t n, double h) {
  double* s = (double*)malloc(n * sizeof(double));
  for (size_t i = 0; i < n; ++i) s[i] = sorted[i];
  double tot = 0.0;
#pragma omp parallel for reduction(+ : tot) schedule(dynamic, 64)
  for (size_t i = 0; i < n; ++i) {
    size_t lo = lower_bound_d(s, n, s[i] - 2.0 * h);
    size_t hi = upper_bound_d(s, n, s[i] + 2.0 * h);
    double a = 0.0;
    for (size_t j = lo; j < hi; ++j) {
      double u = fabs(s[i] - s[j]) / h;
      if (u <= 2.0) a += 4.5 - 2.25 * u;
    }
    tot += a;
  }
  free(s);
  return tot / ((double)n * (double)n);
}

float orc_thumb_ref(const float* col, size_t n) {
  float sum = 0.0f, sum2 = 0.0f;
  for (size_t i = 0; i < n; ++i) {
    sum += col[i];
    sum2 += col[i] * col[i];
  }
  float m2 = sum2 / (float)n;
  float m = sum / (float)n;
  float var = m2 - m * m;
  return (float)(pow((double)n, -1.0 / 7.0) * sqrt((double)var));
}

float orc_amise_from_conv(float conv, float h, size_t n) {
  float a = (float)(0.04 * 1 / pow((double)h, 5.0) * (double)conv);
  a = (float)pow((double)a, 0.2);
  a = (float)((double)a * 1.25 * pow(0.6, 0.8) / pow((double)(float)n, 0.8));
  return a;
}

typedef struct {
  const float* sorted;
  size_t n;
  int exact;
  int calls;
} amise_ctx;

static float amise_at(amise_ctx* c, float h) {
  float conv = c->exact ? orc_epa_conv_ref(c->sorted, c->n, h)
                        : (float)orc_epa_conv_fp64(c->sorted, c->n, (double)h);
  c->calls++;
  return orc_amise_from_conv(conv, h, c->n);
}

/* AmiseMin::_interval_optimized_h (hestimate.cpp:55-86) */
static float interval_h(amise_ctx* c, float prec, float lo, float hi,
                        unsigned iter_max) {
  float delta = hi - lo;
  float pivot = (float)((double)lo + 0.5 * (double)delta);
  if (iter_max == 0 || delta <= prec) return pivot;
  float pl = (float)((double)pivot - 0.25 * (double)delta);
  float ph = (float)((double)pivot + 0.25 * (double)delta);
  float al = amise_at(c, pl);
  float ah = amise_at(c, ph);
  if (al < ah) return interval_h(c, prec, lo, pivot, iter_max - 1);
  return interval_h(c, prec, pivot, hi, iter_max - 1);
}

float orc_hestimate_amise(const float* col, size_t n, int exact_conv,
                          int* n_conv) {
  float* s = (float*)malloc(n * sizeof(float));
  memcpy(s, col, n * sizeof(float));
  qsort(s, n, sizeof(float), f32_cmp);
  float h0 = orc_thumb_ref(col, n);
  amise_ctx c = {s, n, exact_conv, 0};
  float h = interval_h(&c, (float)(0.01 * (double)h0), (float)(0.1 * (double)h0),
                       2 * h0, 20);
  if (n_conv) *n_conv = c.calls;
  free(s);
  return h;
}
