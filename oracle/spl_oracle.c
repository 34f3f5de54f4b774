/*
 * spl_oracle.c -- CPU oracle for the Splotch particle-render path.
 *
 * TEST INFRASTRUCTURE ONLY (see spl_oracle.h).  A plain-C restatement of the
 * reference host renderer, written to reproduce its float/double arithmetic
 * operation by operation.  Build with -ffp-contract=off and without
 * -ffast-math: the reference is only reproducible without fused multiply-add.
 *
 * Integer conversion: the reference truncates with int(float).  For NaN and
 * out-of-range values that is undefined in C++; this restatement (like the CUDA
 * cvt.rzi.s32.f32 instruction and AArch64 fcvtzs) maps NaN to 0 and saturates.
 */
#include "spl_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* cxxsupport/lsconstants.h:35,51 */
static const double SPO_PI = 3.141592653589793238462643383279502884197;
#define SPO_DEGR2RAD (SPO_PI / 180.0)

static int g_threads = 0;

void spo_set_threads(int n) { g_threads = n; }

int spo_get_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

static inline int f2i(float v) {
  if (v != v) return 0;
  if (v >= 2147483648.0f) return INT_MAX;
  if (v <= -2147483904.0f) return INT_MIN;
  return (int)v;
}
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int imin(int a, int b) { return a < b ? a : b; }

/* splotch/splotch_host.cc:44-49 (SPLOTCH_CLASSIC) */
static float h2sigma_f(void) { return (float)(0.5 * pow(SPO_PI, -1. / 6.)); }
static float bfak_f(void) { return (float)(0.5 * pow(SPO_PI, -5. / 6.)); }
static const float RFAC = 0.75f;

/* ---------------------------------------------------------------------- */
/* vec3 (double) and TRANSMAT (float) -- cxxsupport/vec3.h, kernel/transform.cxx */

typedef struct { double x, y, z; } v3;

static v3 v3_sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static v3 v3_normed(v3 a) { /* vec3.h:72-83 */
  double l = 1.0 / sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  v3 r = {a.x * l, a.y * l, a.z * l};
  return r;
}
static double v3_len(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static v3 v3_cross(v3 a, v3 b) { /* vec3.h:129-131 */
  v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
  return r;
}

typedef struct { float e[3][4]; } tmat;

static void tmat_identity(tmat *m) {
  memset(m, 0, sizeof(*m));
  m->e[0][0] = m->e[1][1] = m->e[2][2] = 1.f;
}

/* TRANSMAT::Inverse, kernel/transform.cxx:64-112 */
static int tmat_inverse(const tmat *a, tmat *t) {
  const float (*e)[4] = a->e;
  t->e[0][0] = e[1][1] * e[2][2] - e[2][1] * e[1][2];
  t->e[0][1] = e[0][1] * e[2][2] - e[2][1] * e[0][2];
  t->e[0][2] = e[0][1] * e[1][2] - e[1][1] * e[0][2];
  t->e[1][0] = e[1][0] * e[2][2] - e[2][0] * e[1][2];
  t->e[1][1] = e[0][0] * e[2][2] - e[2][0] * e[0][2];
  t->e[1][2] = e[0][0] * e[1][2] - e[1][0] * e[0][2];
  t->e[2][0] = e[1][0] * e[2][1] - e[2][0] * e[1][1];
  t->e[2][1] = e[0][0] * e[2][1] - e[2][0] * e[0][1];
  t->e[2][2] = e[0][0] * e[1][1] - e[1][0] * e[0][1];
  float df = e[0][0] * t->e[0][0] - e[1][0] * t->e[0][1] + e[2][0] * t->e[0][2];
  double d = (double)df;
  if (!(fabs(d) > 1e-10)) return -1;
  d = 1. / d;
  t->e[0][0] = (float)(t->e[0][0] * d);
  t->e[2][0] = (float)(t->e[2][0] * d);
  t->e[1][1] = (float)(t->e[1][1] * d);
  t->e[0][2] = (float)(t->e[0][2] * d);
  t->e[2][2] = (float)(t->e[2][2] * d);
  d = -d;
  t->e[1][0] = (float)(t->e[1][0] * d);
  t->e[0][1] = (float)(t->e[0][1] * d);
  t->e[2][1] = (float)(t->e[2][1] * d);
  t->e[1][2] = (float)(t->e[1][2] * d);
  for (int j = 0; j < 3; ++j)
    t->e[j][3] = -(t->e[j][0] * e[0][3] + t->e[j][1] * e[1][3] + t->e[j][2] * e[2][3]);
  return 0;
}

/* TRANSMAT::operator*=, kernel/transform.cxx:50-62 */
static void tmat_mul_inplace(tmat *self, const tmat *b) {
  tmat a = *self;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 3; ++j)
      self->e[j][i] = a.e[0][i] * b->e[j][0] + a.e[1][i] * b->e[j][1] + a.e[2][i] * b->e[j][2];
  self->e[0][3] += b->e[0][3];
  self->e[1][3] += b->e[1][3];
  self->e[2][3] += b->e[2][3];
}

/* camera set-up of particle_project, splotch/splotch_host.cc:62-110 */
int spo_camera_setup(const spo_params *prm, spo_camera *cam) {
  int xres = prm->xres, yres = prm->yres;
  cam->ycorr = .5f * (yres - xres);
  cam->res2 = 0.5f * xres;
  cam->fovfct = (float)tan((double)(prm->fov * 0.5f) * SPO_DEGR2RAD);

  v3 campos = {prm->campos[0], prm->campos[1], prm->campos[2]};
  v3 lookat = {prm->lookat[0], prm->lookat[1], prm->lookat[2]};
  v3 sky = {prm->sky[0], prm->sky[1], prm->sky[2]};
  v3 centerpos = {prm->centerpos[0], prm->centerpos[1], prm->centerpos[2]};

  sky = v3_normed(sky);
  v3 zaxis = v3_normed(v3_sub(centerpos, lookat));
  v3 xaxis = v3_normed(v3_cross(sky, zaxis));
  v3 yaxis = v3_cross(zaxis, xaxis);

  /* TRANSMAT ctor stores its 12 arguments transposed (transform.cxx:28-48) */
  tmat gen;
  gen.e[0][0] = (float)xaxis.x; gen.e[1][0] = (float)xaxis.y; gen.e[2][0] = (float)xaxis.z;
  gen.e[0][1] = (float)yaxis.x; gen.e[1][1] = (float)yaxis.y; gen.e[2][1] = (float)yaxis.z;
  gen.e[0][2] = (float)zaxis.x; gen.e[1][2] = (float)zaxis.y; gen.e[2][2] = (float)zaxis.z;
  gen.e[0][3] = 0.f; gen.e[1][3] = 0.f; gen.e[2][3] = 0.f;
  tmat gen_inv;
  if (tmat_inverse(&gen, &gen_inv)) return -1;
  /* trans.Invert() swaps matrix and inverse: matrix = gen_inv */
  tmat trans_matrix = gen_inv;

  /* trans2 = translation(-campos); trans2.Add_Transform(trans) */
  tmat t2;
  tmat_identity(&t2);
  t2.e[0][3] = (float)(-campos.x);
  t2.e[1][3] = (float)(-campos.y);
  t2.e[2][3] = (float)(-campos.z);
  tmat_mul_inplace(&t2, &trans_matrix);
  memcpy(cam->mat, t2.e, sizeof(cam->mat));

  const float *p = cam->mat; /* TRANSFORM::TransPoint, transform.cxx:212-219 */
  double tcx = centerpos.x * p[0] + centerpos.y * p[1] + centerpos.z * p[2] + p[3];
  double tcy = centerpos.x * p[4] + centerpos.y * p[5] + centerpos.z * p[6] + p[7];

  float dist = (float)v3_len(v3_sub(centerpos, lookat));
  cam->xfac = cam->res2 / (cam->fovfct * dist);
  cam->xshift = -cam->xfac * tcx;
  cam->yshift = -cam->xfac * tcy;
  return 0;
}

/* per-particle loop of particle_project, splotch/splotch_host.cc:111-178 */
void spo_project(const spo_params *prm, const spo_camera *cam, spo_particle *pp,
                 int64_t n) {
  const int xres = prm->xres, yres = prm->yres;
  const float zmax = prm->zmax;
  const float zmin = prm->zmin > 0.f ? prm->zmin : 0.f;
  const float res2 = cam->res2, ycorr = cam->ycorr, fovfct = cam->fovfct;
  const double xshift = cam->xshift, yshift = cam->yshift;
  const float *m = cam->mat;
  const float bfak = bfak_f();
  const float minrad = prm->minrad_pix;
  const int projection = prm->projection;

#pragma omp parallel for schedule(guided, 1000) num_threads(spo_get_threads())
  for (int64_t i = 0; i < n; ++i) {
    spo_particle *p = &pp[i];
    double vx = p->x, vy = p->y, vz = p->z;
    double tx = vx * m[0] + vy * m[1] + vz * m[2] + m[3];
    double ty = vx * m[4] + vy * m[5] + vz * m[6] + m[7];
    double tz = vx * m[8] + vy * m[9] + vz * m[10] + m[11];
    p->x = (float)tx; p->y = (float)ty; p->z = (float)tz;
    p->active = 0;
    if (-p->z <= zmin) continue;
    if (-p->z >= zmax) continue;
    float xfac2 = cam->xfac;
    if (!projection) {
      p->x = res2 + p->x * xfac2;
      p->y = res2 + ycorr + p->y * xfac2;
    } else {
      xfac2 = -res2 / (fovfct * p->z);
      float px = p->x * xfac2, py = p->y * xfac2;
      p->x = (float)((double)res2 + xshift + (double)px);
      p->y = (float)((double)res2 + yshift + (double)ycorr + (double)py);
    }
    p->I *= 0.5f * bfak / p->r;
    p->r *= 2;
    p->r *= xfac2 * prm->smooth_factor[p->type];
    float rcorr = sqrtf(p->r * p->r + minrad * minrad) / p->r;
    p->r *= rcorr;
    p->I /= rcorr;

    float posx = p->x, posy = p->y;
    float rfacr = RFAC * p->r;
    int minx = f2i(posx - rfacr + 1);
    if (minx >= xres) continue;
    minx = imax(minx, 0);
    int maxx = f2i(posx + rfacr + 1);
    if (maxx <= 0) continue;
    maxx = imin(maxx, xres);
    if (minx >= maxx) continue;
    int miny = f2i(posy - rfacr + 1);
    if (miny >= yres) continue;
    miny = imax(miny, 0);
    int maxy = f2i(posy + rfacr + 1);
    if (maxy <= 0) continue;
    maxy = imin(maxy, yres);
    if (miny >= maxy) continue;
    p->active = 1;
  }
}

/* linearMap<COLOUR>::getVal_const, cxxsupport/linear_map.h:71-84, with
   interpol_helper, cxxsupport/math_utils.h:186-196 */
static void palette_lookup(int n, const double *x, const float *rgb, double xv,
                           float out[3]) {
  int idx;
  if (n == 1 || xv <= x[0]) { idx = 0; goto ends; }
  if (xv >= x[n - 1]) { idx = n - 1; goto ends; }
  {
    int lo = 0, hi = n; /* lower_bound: first x[i] >= xv */
    while (lo < hi) {
      int mid = lo + (hi - lo) / 2;
      if (x[mid] < xv) lo = mid + 1; else hi = mid;
    }
    idx = lo;
    if (idx > 0) --idx;
    if (idx > n - 2) idx = n - 2;
    double frac = (xv - x[idx]) / (x[idx + 1] - x[idx]);
    for (int c = 0; c < 3; ++c) {
      float a = (float)(rgb[3 * idx + c] * (1. - frac));
      float b = (float)(rgb[3 * (idx + 1) + c] * frac);
      out[c] = a + b;
    }
    return;
  }
ends:
  out[0] = rgb[3 * idx]; out[1] = rgb[3 * idx + 1]; out[2] = rgb[3 * idx + 2];
}

/* particle_colorize, splotch/splotch_host.cc:252-287 */
void spo_colorize(const spo_params *prm, spo_particle *pp, int64_t n) {
  float bright[SPO_MAX_TYPES];
  for (int t = 0; t < prm->ptypes && t < SPO_MAX_TYPES; ++t)
    bright[t] = prm->brightness[t] * prm->b_brightness;
#pragma omp parallel for schedule(guided, 1000) num_threads(spo_get_threads())
  for (int64_t i = 0; i < n; ++i) {
    spo_particle *p = &pp[i];
    if (!p->active) continue;
    int t = p->type;
    if (!prm->color_is_vector[t]) {
      float c[3];
      palette_lookup(prm->pal_n[t], prm->pal_x[t], prm->pal_rgb[t], (double)p->er, c);
      p->er = c[0]; p->eg = c[1]; p->eb = c[2];
    }
    float fac = p->I * bright[t];
    p->er *= fac; p->eg *= fac; p->eb *= fac;
  }
}

/* ---------------------------------------------------------------------- */
/* stable sort, splotch/splotch_host.cc:289-321 with the comparators of
   splotch/splotchutils.h:74-96 (stable, i.e. ties keep the original order) */

typedef struct {
  float key;
  uint32_t idx;
} kv;

/* a goes strictly before b under the comparator (ties: not before) */
static inline int kv_before(const kv *a, const kv *b, int desc) {
  return desc ? a->key > b->key : a->key < b->key;
}

int spo_sort_perm(const spo_particle *p, int64_t n, int sort_type, uint32_t *perm) {
  for (int64_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
  if (sort_type == 0 || n < 2) return 0;
  if (sort_type < 0 || sort_type > 4) return -1;
  kv *a = (kv *)malloc((size_t)n * sizeof(kv)), *b = (kv *)malloc((size_t)n * sizeof(kv));
  if (!a || !b) { free(a); free(b); return -2; }
  const int desc = sort_type == 2 || sort_type == 4;
  for (int64_t i = 0; i < n; ++i) {
    a[i].idx = (uint32_t)i;
    a[i].key = sort_type == 1 ? p[i].z : (sort_type == 4 ? p[i].r : p[i].er);
  }
  /* bottom-up merge sort (serial, stable): runs of 16 by insertion first */
  for (int64_t lo = 0; lo < n; lo += 16) {
    int64_t hi = lo + 16 < n ? lo + 16 : n;
    for (int64_t i = lo + 1; i < hi; ++i) {
      kv t = a[i];
      int64_t j = i;
      while (j > lo && kv_before(&t, &a[j - 1], desc)) { a[j] = a[j - 1]; --j; }
      a[j] = t;
    }
  }
  kv *src = a, *dst = b;
  for (int64_t w = 16; w < n; w *= 2) {
    for (int64_t lo = 0; lo < n; lo += 2 * w) {
      int64_t mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
      int64_t i = lo, j = mid, k = lo;
      while (i < mid && j < hi) dst[k++] = kv_before(&src[j], &src[i], desc) ? src[j++] : src[i++];
      while (i < mid) dst[k++] = src[i++];
      while (j < hi) dst[k++] = src[j++];
    }
    kv *s = src; src = dst; dst = s;
  }
  for (int64_t i = 0; i < n; ++i) perm[i] = src[i].idx;
  free(a);
  free(b);
  return 0;
}

void spo_apply_perm(const spo_particle *in, const uint32_t *perm, int64_t n,
                    spo_particle *out) {
#pragma omp parallel for num_threads(spo_get_threads())
  for (int64_t i = 0; i < n; ++i) out[i] = in[perm[i]];
}

/* ---------------------------------------------------------------------- */
/* binning, render_new region A, splotch/splotch_host.cc:339-406 */

typedef struct {
  int T, ncx, ncy;
  float rcell, cmid0;
} tiling;

static tiling make_tiling(int xres, int yres, int T) {
  tiling g;
  g.T = T;
  g.ncx = (xres + T - 1) / T;
  g.ncy = (yres + T - 1) / T;
  g.rcell = sqrtf(2.f) * (T * 0.5f - 0.5f);
  g.cmid0 = 0.5f * (T - 1);
  return g;
}

/* visits the tiles of one particle; returns count, optionally writes ids */
static int particle_tiles(const spo_particle *pp, const tiling *g, uint32_t *ids) {
  if (!pp->active) return 0;
  const int T = g->T;
  float rfacr = RFAC * pp->r;
  int minx = imax(0, f2i(pp->x - rfacr + 1) / T);
  int maxx = imin(g->ncx - 1, f2i(pp->x + rfacr) / T);
  int miny = imax(0, f2i(pp->y - rfacr + 1) / T);
  int maxy = imin(g->ncy - 1, f2i(pp->y + rfacr) / T);
  float sumsq = (g->rcell + rfacr) * (g->rcell + rfacr);
  int cnt = 0;
  for (int ix = minx; ix <= maxx; ++ix) {
    float cx = g->cmid0 + ix * T;
    for (int iy = miny; iy <= maxy; ++iy) {
      float cy = g->cmid0 + iy * T;
      float rtot2 = (pp->x - cx) * (pp->x - cx) + (pp->y - cy) * (pp->y - cy);
      if (rtot2 < sumsq) {
        if (ids) ids[cnt] = (uint32_t)(iy * g->ncx + ix);
        ++cnt;
      }
    }
  }
  return cnt;
}

int64_t spo_bin(const spo_particle *p, const uint32_t *order, int64_t n, int xres,
                int yres, int T, int64_t *tile_start, uint32_t *entries) {
  tiling g = make_tiling(xres, yres, T);
  const int64_t ntiles = (int64_t)g.ncx * g.ncy;
  const int nth = spo_get_threads();
  int64_t *cnt = (int64_t *)calloc((size_t)(nth * ntiles), sizeof(int64_t));
  if (!cnt) return -1;
  /* pass 1: per-thread per-tile counts over contiguous shares (like the
     per-thread lists of the reference, concatenated in thread order) */
#pragma omp parallel num_threads(nth)
  {
    int th = 0;
#ifdef _OPENMP
    th = omp_get_thread_num();
#endif
    int64_t lo = n * th / nth, hi = n * (th + 1) / nth;
    int64_t *c = cnt + (int64_t)th * ntiles;
    uint32_t ids[4096];
    for (int64_t s = lo; s < hi; ++s) {
      const spo_particle *pp = &p[order ? order[s] : s];
      int k = particle_tiles(pp, &g, NULL);
      if (k <= 4096) {
        particle_tiles(pp, &g, ids);
        for (int j = 0; j < k; ++j) c[ids[j]]++;
      } else {
        uint32_t *big = (uint32_t *)malloc((size_t)k * sizeof(uint32_t));
        particle_tiles(pp, &g, big);
        for (int j = 0; j < k; ++j) c[big[j]]++;
        free(big);
      }
    }
  }
  /* exclusive scan, tile-major then thread order */
  int64_t run = 0;
  for (int64_t t = 0; t < ntiles; ++t) {
    if (tile_start) tile_start[t] = run;
    for (int th = 0; th < nth; ++th) {
      int64_t v = cnt[(int64_t)th * ntiles + t];
      cnt[(int64_t)th * ntiles + t] = run;
      run += v;
    }
  }
  if (tile_start) tile_start[ntiles] = run;
  if (entries) {
#pragma omp parallel num_threads(nth)
    {
      int th = 0;
#ifdef _OPENMP
      th = omp_get_thread_num();
#endif
      int64_t lo = n * th / nth, hi = n * (th + 1) / nth;
      int64_t *c = cnt + (int64_t)th * ntiles;
      uint32_t ids[4096];
      for (int64_t s = lo; s < hi; ++s) {
        uint32_t i = (uint32_t)(order ? order[s] : s);
        int k = particle_tiles(&p[i], &g, NULL);
        uint32_t *buf = k <= 4096 ? ids : (uint32_t *)malloc((size_t)k * sizeof(uint32_t));
        particle_tiles(&p[i], &g, buf);
        for (int j = 0; j < k; ++j) entries[c[buf[j]]++] = i;
        if (buf != ids) free(buf);
      }
    }
  }
  free(cnt);
  return run;
}

/* ---------------------------------------------------------------------- */
/* exptable<float32>(-20), splotch/splotchutils.h:174-215 */

typedef struct {
  float expfac, taylorlimit;
  float tab1[1024], tab2[1024];
} exptab;

static void exptab_init(exptab *t, float maxexp) {
  t->expfac = 1048576 / maxexp;
  for (int m = 0; m < 1024; ++m) {
    t->tab1[m] = expf(m * 1024 / t->expfac);
    t->tab2[m] = expf(m / t->expfac);
  }
  t->taylorlimit = sqrtf(2.f * fabsf(maxexp) / 1048576);
}

static inline float exptab_exp(const exptab *t, float arg) {
  int iarg = f2i(arg * t->expfac);
  if (iarg & ~((1 << 20) - 1)) return (iarg < 0) ? 1.f : 0.f;
  return t->tab1[iarg >> 10] * t->tab2[iarg & 1023];
}

static inline float exptab_expm1(const exptab *t, float arg) {
  if (fabsf(arg) < t->taylorlimit) return arg;
  return exptab_exp(t, arg) - 1.f;
}

/* tile lists for the splat: built with spo_bin */
typedef struct {
  tiling g;
  int64_t ntiles;
  int64_t *start;
  uint32_t *ent;
} bins;

static int make_bins(const spo_particle *p, const uint32_t *order, int64_t n, int xres,
                     int yres, int T, bins *b) {
  b->g = make_tiling(xres, yres, T);
  b->ntiles = (int64_t)b->g.ncx * b->g.ncy;
  b->start = (int64_t *)malloc((size_t)(b->ntiles + 1) * sizeof(int64_t));
  int64_t tot = spo_bin(p, order, n, xres, yres, T, b->start, NULL);
  if (tot < 0) return -1;
  b->ent = (uint32_t *)malloc((size_t)(tot > 0 ? tot : 1) * sizeof(uint32_t));
  spo_bin(p, order, n, xres, yres, T, b->start, b->ent);
  return 0;
}
static void free_bins(bins *b) { free(b->start); free(b->ent); }

/* per-particle, per-tile coverage of render_new (splotch_host.cc:461-476) */
typedef struct {
  float posx, posy, rfacr, radsq, stp;
  int minx, maxx, miny, maxy;
} pcov;

static inline void particle_cover(const spo_particle *pp, int x0s, int y0s, int x1, int y1,
                                  float h2sigma, pcov *c) {
  c->rfacr = pp->r * RFAC;
  c->posx = pp->x - x0s;
  c->posy = pp->y - y0s;
  c->minx = imax(f2i(c->posx - c->rfacr + 1), 0);
  c->maxx = imin(f2i(c->posx + c->rfacr + 1), x1);
  c->miny = imax(f2i(c->posy - c->rfacr + 1), 0);
  c->maxy = imin(f2i(c->posy + c->rfacr + 1), y1);
  c->radsq = c->rfacr * c->rfacr;
  float sigma = h2sigma * pp->r;
  c->stp = -1.f / (sigma * sigma);
}

/* column run of render_new (splotch_host.cc:603-606) */
static inline void column_run(const pcov *c, int x, int *lo, int *hi, float *dxsq) {
  float dx = x - c->posx;
  *dxsq = dx * dx;
  float dy = sqrtf(c->radsq - *dxsq);
  *lo = imax(c->miny, f2i(c->posy - dy + 1));
  *hi = imin(c->maxy, f2i(c->posy + dy + 1));
}

int64_t spo_render_fp32(const spo_particle *p, const uint32_t *order, int64_t n,
                        int xres, int yres, int T, int a_eq_e, float gray,
                        int simd_branch, float *pic) {
  bins b;
  if (make_bins(p, order, n, xres, yres, T, &b)) return -1;
  exptab xexp;
  exptab_init(&xexp, -20.f);
  const float taylorlimit = xexp.taylorlimit;
  const float h2sigma = h2sigma_f();
  int64_t frags = 0;

#pragma omp parallel num_threads(spo_get_threads()) reduction(+ : frags)
  {
    float *lpic = (float *)malloc((size_t)T * T * 3 * sizeof(float));
    float *pre1 = (float *)malloc((size_t)T * sizeof(float));
#pragma omp for schedule(dynamic, 1)
    for (int64_t chunk = 0; chunk < b.ntiles; ++chunk) {
      int ix = (int)(chunk % b.g.ncx), iy = (int)(chunk / b.g.ncx);
      int x0s = ix * T, y0s = iy * T;
      int x1 = imin(x0s + T, xres) - x0s, y1 = imin(y0s + T, yres) - y0s;
      memset(lpic, 0, (size_t)x1 * y1 * 3 * sizeof(float));
      for (int64_t k = b.start[chunk]; k < b.start[chunk + 1]; ++k) {
        const spo_particle *pp = &p[b.ent[k]];
        pcov c;
        particle_cover(pp, x0s, y0s, x1, y1, h2sigma, &c);
        float ar = -pp->er, ag = -pp->eg, ab = -pp->eb;
        for (int y = c.miny; y < c.maxy; ++y) {
          float t = y - c.posy;
          pre1[y] = exptab_exp(&xexp, c.stp * t * t);
        }
        if (a_eq_e) {
          for (int x = c.minx; x < c.maxx; ++x) {
            int lo, hi; float dxsq;
            column_run(&c, x, &lo, &hi, &dxsq);
            float pre2 = exptab_exp(&xexp, c.stp * dxsq);
            float *col = lpic + (size_t)x * y1 * 3;
            for (int y = lo; y < hi; ++y) {
              float att = pre1[y] * pre2;
              col[3 * y] += att * ar;
              col[3 * y + 1] += att * ag;
              col[3 * y + 2] += att * ab;
            }
            if (hi > lo) frags += hi - lo;
          }
        } else {
          float qr = pp->er / (pp->er + gray), qg = pp->eg / (pp->eg + gray),
                qb = pp->eb / (pp->eb + gray);
          float maxa = fabsf(ar);
          if (fabsf(ag) > maxa) maxa = fabsf(ag);
          if (fabsf(ab) > maxa) maxa = fabsf(ab);
          for (int x = c.minx; x < c.maxx; ++x) {
            int lo, hi; float dxsq;
            column_run(&c, x, &lo, &hi, &dxsq);
            float pre2 = exptab_exp(&xexp, c.stp * dxsq);
            float *col = lpic + (size_t)x * y1 * 3;
            for (int y = lo; y < hi; ++y) {
              float att = pre1[y] * pre2;
              float *v = col + 3 * y;
              if (simd_branch && (maxa * att) < taylorlimit) {
                v[0] += ((v[0] - qr) * ar) * att;
                v[1] += ((v[1] - qg) * ag) * att;
                v[2] += ((v[2] - qb) * ab) * att;
              } else {
                v[0] += exptab_expm1(&xexp, att * ar) * (v[0] - qr);
                v[1] += exptab_expm1(&xexp, att * ag) * (v[1] - qg);
                v[2] += exptab_expm1(&xexp, att * ab) * (v[2] - qb);
              }
            }
            if (hi > lo) frags += hi - lo;
          }
        }
      }
      for (int x = 0; x < x1; ++x)
        memcpy(pic + ((size_t)(x + x0s) * yres + y0s) * 3, lpic + (size_t)x * y1 * 3,
               (size_t)y1 * 3 * sizeof(float));
    }
    free(lpic);
    free(pre1);
  }
  free_bins(&b);
  return frags;
}

int64_t spo_render_fp64(const spo_particle *p, const uint32_t *order, int64_t n,
                        int xres, int yres, int T, int a_eq_e, double gray,
                        double *pic) {
  bins b;
  if (make_bins(p, order, n, xres, yres, T, &b)) return -1;
  const float h2sigma = h2sigma_f();
  int64_t frags = 0;
#pragma omp parallel num_threads(spo_get_threads()) reduction(+ : frags)
  {
    double *lpic = (double *)malloc((size_t)T * T * 3 * sizeof(double));
    double *pre1 = (double *)malloc((size_t)T * sizeof(double));
#pragma omp for schedule(dynamic, 1)
    for (int64_t chunk = 0; chunk < b.ntiles; ++chunk) {
      int ix = (int)(chunk % b.g.ncx), iy = (int)(chunk / b.g.ncx);
      int x0s = ix * T, y0s = iy * T;
      int x1 = imin(x0s + T, xres) - x0s, y1 = imin(y0s + T, yres) - y0s;
      memset(lpic, 0, (size_t)x1 * y1 * 3 * sizeof(double));
      for (int64_t k = b.start[chunk]; k < b.start[chunk + 1]; ++k) {
        const spo_particle *pp = &p[b.ent[k]];
        pcov c;
        particle_cover(pp, x0s, y0s, x1, y1, h2sigma, &c);
        double sigma = (double)h2sigma * pp->r;
        double stp = -1.0 / (sigma * sigma);
        double px = (double)pp->x - x0s, py = (double)pp->y - y0s;
        double e[3] = {pp->er, pp->eg, pp->eb};
        double q[3];
        for (int ch = 0; ch < 3; ++ch) q[ch] = e[ch] / (e[ch] + gray);
        for (int y = c.miny; y < c.maxy; ++y) pre1[y] = exp(stp * (y - py) * (y - py));
        for (int x = c.minx; x < c.maxx; ++x) {
          int lo, hi; float dxsq;
          column_run(&c, x, &lo, &hi, &dxsq);
          double pre2 = exp(stp * (x - px) * (x - px));
          double *col = lpic + (size_t)x * y1 * 3;
          for (int y = lo; y < hi; ++y) {
            double att = pre1[y] * pre2;
            double *v = col + 3 * y;
            if (a_eq_e) {
              for (int ch = 0; ch < 3; ++ch) v[ch] += -e[ch] * att;
            } else {
              for (int ch = 0; ch < 3; ++ch) v[ch] += expm1(-e[ch] * att) * (v[ch] - q[ch]);
            }
          }
          if (hi > lo) frags += hi - lo;
        }
      }
      for (int x = 0; x < x1; ++x)
        memcpy(pic + ((size_t)(x + x0s) * yres + y0s) * 3, lpic + (size_t)x * y1 * 3,
               (size_t)y1 * 3 * sizeof(double));
    }
    free(lpic);
    free(pre1);
  }
  free_bins(&b);
  return frags;
}

/* ---------------------------------------------------------------------- */
/* FP64 adjoint of the splat.  Per tile and pixel: replay the ordered layer
   list forward (storing every intermediate value), then walk it backwards. */

int spo_splat_adjoint_fp64(const spo_particle *p, const uint32_t *order, int64_t n,
                           int xres, int yres, int T, int a_eq_e, double gray,
                           const double *gpic, double *gx, double *gy, double *gr,
                           double *ge) {
  bins b;
  if (make_bins(p, order, n, xres, yres, T, &b)) return -1;
  const float h2sigma = h2sigma_f();
  memset(gx, 0, (size_t)n * sizeof(double));
  memset(gy, 0, (size_t)n * sizeof(double));
  memset(gr, 0, (size_t)n * sizeof(double));
  memset(ge, 0, (size_t)n * 3 * sizeof(double));
  /* serial over tiles keeps the per-particle accumulation deterministic */
  for (int64_t chunk = 0; chunk < b.ntiles; ++chunk) {
    int ix = (int)(chunk % b.g.ncx), iy = (int)(chunk / b.g.ncx);
    int x0s = ix * T, y0s = iy * T;
    int x1 = imin(x0s + T, xres) - x0s, y1 = imin(y0s + T, yres) - y0s;
    int64_t k0 = b.start[chunk], k1 = b.start[chunk + 1];
    int64_t L = k1 - k0;
    if (L == 0) continue;
    double *att = (double *)malloc((size_t)L * sizeof(double));
    double *hist = (double *)malloc((size_t)(L + 1) * 3 * sizeof(double));
    pcov *cv = (pcov *)malloc((size_t)L * sizeof(pcov));
    for (int64_t k = 0; k < L; ++k)
      particle_cover(&p[b.ent[k0 + k]], x0s, y0s, x1, y1, h2sigma, &cv[k]);
    for (int x = 0; x < x1; ++x)
      for (int y = 0; y < y1; ++y) {
        const double *G = gpic + ((size_t)(x + x0s) * yres + (y + y0s)) * 3;
        /* forward replay */
        hist[0] = hist[1] = hist[2] = 0.0;
        for (int64_t k = 0; k < L; ++k) {
          const spo_particle *pp = &p[b.ent[k0 + k]];
          const pcov *c = &cv[k];
          double *h0 = hist + 3 * k, *h1 = hist + 3 * (k + 1);
          att[k] = 0.0;
          int inside = 0;
          if (x >= c->minx && x < c->maxx) {
            int lo, hi; float dxsq;
            column_run(c, x, &lo, &hi, &dxsq);
            inside = (y >= lo && y < hi);
          }
          if (inside) {
            double sigma = (double)h2sigma * pp->r;
            double stp = -1.0 / (sigma * sigma);
            double dx = (double)(x + x0s) - pp->x, dy = (double)(y + y0s) - pp->y;
            att[k] = exp(stp * dy * dy) * exp(stp * dx * dx);
          }
          double e[3] = {pp->er, pp->eg, pp->eb};
          for (int ch = 0; ch < 3; ++ch) {
            if (!inside) { h1[ch] = h0[ch]; continue; }
            if (a_eq_e) h1[ch] = h0[ch] - e[ch] * att[k];
            else {
              double q = e[ch] / (e[ch] + gray);
              h1[ch] = h0[ch] + expm1(-e[ch] * att[k]) * (h0[ch] - q);
            }
          }
        }
        /* reverse sweep */
        double lam[3] = {G[0], G[1], G[2]};
        for (int64_t k = L - 1; k >= 0; --k) {
          if (att[k] == 0.0) continue;
          uint32_t i = b.ent[k0 + k];
          const spo_particle *pp = &p[i];
          double sigma = (double)h2sigma * pp->r;
          double stp = -1.0 / (sigma * sigma);
          double dx = (double)(x + x0s) - pp->x, dy = (double)(y + y0s) - pp->y;
          double e[3] = {pp->er, pp->eg, pp->eb};
          double gatt = 0.0;
          for (int ch = 0; ch < 3; ++ch) {
            if (a_eq_e) {
              ge[3 * (size_t)i + ch] += -lam[ch] * att[k];
              gatt += -lam[ch] * e[ch];
            } else {
              double Cprev = hist[3 * k + ch];
              double q = e[ch] / (e[ch] + gray);
              double Tk = exp(-e[ch] * att[k]);
              double dT = lam[ch] * (Cprev - q);
              double dq = lam[ch] * (1.0 - Tk);
              ge[3 * (size_t)i + ch] += dT * (-att[k] * Tk) + dq * gray / ((e[ch] + gray) * (e[ch] + gray));
              gatt += dT * (-e[ch] * Tk);
              lam[ch] *= Tk;
            }
          }
          double a = att[k];
          gx[i] += gatt * a * (-2.0 * stp) * dx;
          gy[i] += gatt * a * (-2.0 * stp) * dy;
          gr[i] += gatt * a * (dx * dx + dy * dy) * (-2.0 * stp / pp->r);
        }
      }
    free(att);
    free(hist);
    free(cv);
  }
  free_bins(&b);
  return 0;
}

/* ---------------------------------------------------------------------- */
/* host_rendering, splotch/splotch_host.cc:711-834 (non-MPI, classic path) */
int spo_host_rendering(const spo_params *prm, spo_particle *p, int64_t n,
                       int simd_branch, float *pic) {
  spo_camera cam;
  if (spo_camera_setup(prm, &cam)) return -1;
  spo_project(prm, &cam, p, n);
  spo_colorize(prm, p, n);
  if (!prm->a_eq_e && prm->sort_type != 0) {
    uint32_t *perm = (uint32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(uint32_t));
    spo_particle *tmp = (spo_particle *)malloc((size_t)(n > 0 ? n : 1) * sizeof(spo_particle));
    if (!perm || !tmp) { free(perm); free(tmp); return -2; }
    if (spo_sort_perm(p, n, prm->sort_type, perm)) { free(perm); free(tmp); return -3; }
    spo_apply_perm(p, perm, n, tmp);
    memcpy(p, tmp, (size_t)n * sizeof(spo_particle));
    free(perm);
    free(tmp);
  }
  int64_t r = spo_render_fp32(p, NULL, n, prm->xres, prm->yres, prm->tile_size,
                              prm->a_eq_e, prm->gray_absorption, simd_branch, pic);
  return r < 0 ? -4 : 0;
}

/* ====================================================================== */
/* Differentiable FP64 model -- the checker of the adjoint (gradient) path.
   particle_project + particle_colorize (splotch_host.cc:111-153, 270-284) as
   a smooth double-precision function of one particle's inputs and of the
   camera position; the splat as a function of (X, Y, R, E) with coverage,
   tile lists and order held at the reference's float decisions. */

static spo_model_in model_in_of(const spo_particle *p) {
  spo_model_in q;
  q.I = p->I; q.e[0] = p->er; q.e[1] = p->eg; q.e[2] = p->eb;
  q.x = p->x; q.y = p->y; q.z = p->z; q.r = p->r;
  q.type = p->type;
  return q;
}

static void model_colour(const spo_model *m, const spo_model_in *p, double col[3],
                         double dcol[3], int *seg) {
  const int t = p->type;
  *seg = -3;
  if (m->colvec[t]) {
    col[0] = p->e[0]; col[1] = p->e[1]; col[2] = p->e[2];
    dcol[0] = dcol[1] = dcol[2] = 0.0;
    return;
  }
  /* linearMap::getVal_const in double (linear_map.h:71-84), plus its slope */
  const int n = m->pal_n[t];
  const double *x = m->pal_x[t];
  const float *rgb = m->pal_rgb[t];
  const double v = p->e[0];
  int idx;
  if (n == 1 || v <= x[0]) { idx = 0; *seg = -1; goto ends; }
  if (v >= x[n - 1]) { idx = n - 1; *seg = -2; goto ends; }
  {
    int lo = 0, hi = n;
    while (lo < hi) {
      int mid = lo + (hi - lo) / 2;
      if (x[mid] < v) lo = mid + 1; else hi = mid;
    }
    idx = lo > 0 ? lo - 1 : 0;
    if (idx > n - 2) idx = n - 2;
    const double dx = x[idx + 1] - x[idx], frac = (v - x[idx]) / dx;
    for (int c = 0; c < 3; ++c) {
      col[c] = rgb[3 * idx + c] * (1. - frac) + rgb[3 * (idx + 1) + c] * frac;
      dcol[c] = (rgb[3 * (idx + 1) + c] - (double)rgb[3 * idx + c]) / dx;
    }
    *seg = idx;
    return;
  }
ends:
  for (int c = 0; c < 3; ++c) { col[c] = rgb[3 * idx + c]; dcol[c] = 0.0; }
}

int spo_model_setup(const spo_params *prm, spo_model *m) {
  spo_camera cam;
  if (spo_camera_setup(prm, &cam)) return -1;
  memset(m, 0, sizeof(*m));
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) m->A[i][j] = cam.mat[4 * i + j];
    m->campos[i] = prm->campos[i];
    m->centerpos[i] = prm->centerpos[i];
  }
  m->res2 = cam.res2; m->ycorr = cam.ycorr; m->fovfct = cam.fovfct; m->xfac = cam.xfac;
  m->projection = prm->projection;
  m->minrad = prm->minrad_pix;
  m->bfak = bfak_f();
  m->h2sigma = h2sigma_f();
  for (int t = 0; t < prm->ptypes && t < SPO_MAX_TYPES; ++t) {
    m->smooth[t] = prm->smooth_factor[t];
    m->bright[t] = (float)(prm->brightness[t] * prm->b_brightness);
    m->colvec[t] = prm->color_is_vector[t];
    m->pal_n[t] = prm->pal_n[t];
    m->pal_x[t] = prm->pal_x[t];
    m->pal_rgb[t] = prm->pal_rgb[t];
  }
  return 0;
}

typedef struct {
  double xc, yc, zc, f, r2, R, K, col[3], dcol[3];
  int seg;
} model_fwd;

static void model_eval(const spo_model *m, const spo_model_in *p, model_fwd *s, double w[6]) {
  double d[3] = {p->x - m->campos[0], p->y - m->campos[1], p->z - m->campos[2]};
  s->xc = m->A[0][0] * d[0] + m->A[0][1] * d[1] + m->A[0][2] * d[2];
  s->yc = m->A[1][0] * d[0] + m->A[1][1] * d[1] + m->A[1][2] * d[2];
  s->zc = m->A[2][0] * d[0] + m->A[2][1] * d[1] + m->A[2][2] * d[2];
  if (m->projection) {
    double dc[3] = {m->centerpos[0] - m->campos[0], m->centerpos[1] - m->campos[1],
                    m->centerpos[2] - m->campos[2]};
    double xs = -m->xfac * (m->A[0][0] * dc[0] + m->A[0][1] * dc[1] + m->A[0][2] * dc[2]);
    double ys = -m->xfac * (m->A[1][0] * dc[0] + m->A[1][1] * dc[1] + m->A[1][2] * dc[2]);
    s->f = -m->res2 / (m->fovfct * s->zc);
    w[0] = m->res2 + xs + s->xc * s->f;
    w[1] = m->res2 + ys + m->ycorr + s->yc * s->f;
  } else {
    s->f = m->xfac;
    w[0] = m->res2 + s->xc * s->f;
    w[1] = m->res2 + m->ycorr + s->yc * s->f;
  }
  const int t = p->type;
  s->r2 = 2.0 * p->r * s->f * m->smooth[t];
  s->R = sqrt(s->r2 * s->r2 + m->minrad * m->minrad);
  s->K = m->bfak * m->bright[t] * s->f * m->smooth[t] / s->R;
  model_colour(m, p, s->col, s->dcol, &s->seg);
  w[2] = s->R;
  for (int c = 0; c < 3; ++c) w[3 + c] = s->col[c] * p->I * s->K;
}

void spo_model_project(const spo_model *m, const spo_model_in *p, double w[6]) {
  model_fwd s;
  model_eval(m, p, &s, w);
}

void spo_model_vjp(const spo_model *m, const spo_model_in *p, const double gin[6],
                   double gout[8], double gcampos[3]) {
  model_fwd s;
  double w[6];
  model_eval(m, p, &s, w);
  const int t = p->type;
  const double sm = m->smooth[t];
  const double gX = gin[0], gY = gin[1], gR = gin[2];
  double gK = 0.0, gI = 0.0, gcol[3];
  for (int c = 0; c < 3; ++c) {
    gK += gin[3 + c] * s.col[c] * p->I;
    gI += gin[3 + c] * s.col[c] * s.K;
    gcol[c] = gin[3 + c] * p->I * s.K;
  }
  /* K = bfak*bright*f*s/R */
  const double gRt = gR - gK * s.K / s.R;
  double gf = gK * s.K / s.f;
  /* R = sqrt(r2^2 + minrad^2), r2 = 2*h*f*s */
  const double gr2 = gRt * s.r2 / s.R;
  const double gh = gr2 * 2.0 * s.f * sm;
  gf += gr2 * 2.0 * p->r * sm;
  /* X = res2 (+ xshift) + xc*f */
  gf += gX * s.xc + gY * s.yc;
  double gcam[3] = {gX * s.f, gY * s.f, 0.0};
  if (m->projection) {
    gcam[2] = gf * (-s.f / s.zc);  /* f = -res2/(fovfct*zc) */
    for (int j = 0; j < 3; ++j)  /* xshift = -xfac*A0.(centerpos-campos) */
      gcampos[j] += m->xfac * (gX * m->A[0][j] + gY * m->A[1][j]);
  }
  double gp[3];
  for (int j = 0; j < 3; ++j) {
    gp[j] = m->A[0][j] * gcam[0] + m->A[1][j] * gcam[1] + m->A[2][j] * gcam[2];
    gcampos[j] -= gp[j];
  }
  gout[0] = gI;
  if (m->colvec[t]) {
    gout[1] = gcol[0]; gout[2] = gcol[1]; gout[3] = gcol[2];
  } else {
    gout[1] = gcol[0] * s.dcol[0] + gcol[1] * s.dcol[1] + gcol[2] * s.dcol[2];
    gout[2] = gout[3] = 0.0;
  }
  gout[4] = gp[0]; gout[5] = gp[1]; gout[6] = gp[2];
  gout[7] = gh;
}

/* The model is anchored at the render's own values.  The render projects in
   double and stores float (splotch_host.cc:134), so its X, Y, R, E sit up to
   half a float ulp (1.2e-4 px at X ~ 2048) from the smooth model's; for a
   particle whose Gaussian is under a pixel wide that moves weights and their
   derivatives by ~1e-3.  Per particle, a constant off = float value - model
   value at the base camera carries the model onto the render's values there;
   derivatives are the smooth model's (the float rounding's own derivative is
   zero almost everywhere), and the splat -- adjoint and finite differences
   alike -- is evaluated where the render evaluated it. */
static void model_offsets(const spo_model *m0, const spo_particle *raw, const spo_particle *cov,
                          int64_t n, double *off) {
#pragma omp parallel for schedule(static) num_threads(spo_get_threads())
  for (int64_t i = 0; i < n; ++i) {
    double *o = off + 6 * i;
    if (!cov[i].active) { memset(o, 0, 6 * sizeof(double)); continue; }
    const spo_model_in q = model_in_of(&raw[i]);
    double wd[6];
    spo_model_project(m0, &q, wd);
    const double f[6] = {cov[i].x, cov[i].y, cov[i].r, cov[i].er, cov[i].eg, cov[i].eb};
    for (int j = 0; j < 6; ++j) o[j] = f[j] - wd[j];
  }
}

static void model_all(const spo_model *m, const spo_particle *raw, const spo_particle *cov,
                      int64_t n, const double *off, double *w) {
#pragma omp parallel for schedule(static) num_threads(spo_get_threads())
  for (int64_t i = 0; i < n; ++i) {
    if (cov[i].active) {
      const spo_model_in q = model_in_of(&raw[i]);
      spo_model_project(m, &q, w + 6 * i);
      for (int j = 0; j < 6; ++j) w[6 * i + j] += off[6 * i + j];
    } else {
      memset(w + 6 * i, 0, 6 * sizeof(double));
    }
  }
}

/* one pixel's fragment weight: exp(stp*d^2) with the model's X, Y, R */
static inline double frag_att(const double *wi, double h2sigma, double px, double py) {
  const double sigma = h2sigma * wi[2];
  const double stp = -1.0 / (sigma * sigma);
  const double dx = px - wi[0], dy = py - wi[1];
  return exp(stp * (dx * dx + dy * dy));
}

static inline int covers_pixel(const pcov *c, int x, int y) {
  if (x < c->minx || x >= c->maxx || y < c->miny || y >= c->maxy) return 0;
  int lo, hi;
  float dxsq;
  column_run(c, x, &lo, &hi, &dxsq);
  return y >= lo && y < hi;
}

static inline void frag_apply(int a_eq_e, double gray, const double *E, double att,
                              double *v) {
  for (int ch = 0; ch < 3; ++ch) {
    if (a_eq_e) v[ch] += -E[ch] * att;
    else v[ch] += expm1(-E[ch] * att) * (v[ch] - E[ch] / (E[ch] + gray));
  }
}

int64_t spo_render_frozen_fp64(const spo_particle *cov, const double *w, const uint32_t *order,
                               int64_t n, int xres, int yres, int T, int a_eq_e, double gray,
                               double *pic) {
  bins b;
  if (make_bins(cov, order, n, xres, yres, T, &b)) return -1;
  const double h2s = h2sigma_f();
  const float h2sf = h2sigma_f();
  int64_t frags = 0;
#pragma omp parallel num_threads(spo_get_threads()) reduction(+ : frags)
  {
    double *lpic = (double *)malloc((size_t)T * T * 3 * sizeof(double));
#pragma omp for schedule(dynamic, 1)
    for (int64_t chunk = 0; chunk < b.ntiles; ++chunk) {
      int ix = (int)(chunk % b.g.ncx), iy = (int)(chunk / b.g.ncx);
      int x0s = ix * T, y0s = iy * T;
      int x1 = imin(x0s + T, xres) - x0s, y1 = imin(y0s + T, yres) - y0s;
      memset(lpic, 0, (size_t)x1 * y1 * 3 * sizeof(double));
      for (int64_t k = b.start[chunk]; k < b.start[chunk + 1]; ++k) {
        const uint32_t i = b.ent[k];
        pcov c;
        particle_cover(&cov[i], x0s, y0s, x1, y1, h2sf, &c);
        const double *wi = w + 6 * (size_t)i;
        for (int x = c.minx; x < c.maxx; ++x) {
          int lo, hi;
          float dxsq;
          column_run(&c, x, &lo, &hi, &dxsq);
          for (int y = lo; y < hi; ++y) {
            double att = frag_att(wi, h2s, (double)(x + x0s), (double)(y + y0s));
            frag_apply(a_eq_e, gray, wi + 3, att, lpic + ((size_t)x * y1 + y) * 3);
          }
          if (hi > lo) frags += hi - lo;
        }
      }
      for (int x = 0; x < x1; ++x)
        memcpy(pic + ((size_t)(x + x0s) * yres + y0s) * 3, lpic + (size_t)x * y1 * 3,
               (size_t)y1 * 3 * sizeof(double));
    }
    free(lpic);
  }
  free_bins(&b);
  return frags;
}

/* Exact reverse mode of the frozen render: per pixel, replay the ordered list
   storing every intermediate, then sweep it backwards.  gw (n x 6) receives
   dL/d(X, Y, R, E.r, E.g, E.b) for L = sum(gpic * pic). */
int spo_render_frozen_vjp_fp64(const spo_particle *cov, const double *w, const uint32_t *order,
                               int64_t n, int xres, int yres, int T, int a_eq_e, double gray,
                               const double *gpic, double *gw) {
  bins b;
  if (make_bins(cov, order, n, xres, yres, T, &b)) return -1;
  const double h2s = h2sigma_f();
  const float h2sf = h2sigma_f();
  memset(gw, 0, (size_t)n * 6 * sizeof(double));
#pragma omp parallel num_threads(spo_get_threads())
  {
    int64_t cap = 0;
    double *att = NULL, *hist = NULL;
    pcov *cv = NULL;
#pragma omp for schedule(dynamic, 1)
    for (int64_t chunk = 0; chunk < b.ntiles; ++chunk) {
      int ix = (int)(chunk % b.g.ncx), iy = (int)(chunk / b.g.ncx);
      int x0s = ix * T, y0s = iy * T;
      int x1 = imin(x0s + T, xres) - x0s, y1 = imin(y0s + T, yres) - y0s;
      int64_t k0 = b.start[chunk], L = b.start[chunk + 1] - k0;
      if (L == 0) continue;
      if (L > cap) {
        cap = L;
        free(att); free(hist); free(cv);
        att = (double *)malloc((size_t)L * sizeof(double));
        hist = (double *)malloc((size_t)(L + 1) * 3 * sizeof(double));
        cv = (pcov *)malloc((size_t)L * sizeof(pcov));
      }
      for (int64_t k = 0; k < L; ++k)
        particle_cover(&cov[b.ent[k0 + k]], x0s, y0s, x1, y1, h2sf, &cv[k]);
      for (int x = 0; x < x1; ++x)
        for (int y = 0; y < y1; ++y) {
          const double *G = gpic + ((size_t)(x + x0s) * yres + (y + y0s)) * 3;
          const double px = x + x0s, py = y + y0s;
          hist[0] = hist[1] = hist[2] = 0.0;
          for (int64_t k = 0; k < L; ++k) {
            const double *wi = w + 6 * (size_t)b.ent[k0 + k];
            memcpy(hist + 3 * (k + 1), hist + 3 * k, 3 * sizeof(double));
            att[k] = 0.0;
            if (!covers_pixel(&cv[k], x, y)) continue;
            att[k] = frag_att(wi, h2s, px, py);
            frag_apply(a_eq_e, gray, wi + 3, att[k], hist + 3 * (k + 1));
          }
          double lam[3] = {G[0], G[1], G[2]};
          for (int64_t k = L - 1; k >= 0; --k) {
            if (!covers_pixel(&cv[k], x, y)) continue;
            const uint32_t i = b.ent[k0 + k];
            const double *wi = w + 6 * (size_t)i;
            const double a = att[k];
            double ge[3], gatt = 0.0;
            for (int ch = 0; ch < 3; ++ch) {
              const double E = wi[3 + ch];
              if (a_eq_e) {
                ge[ch] = -lam[ch] * a;
                gatt += -lam[ch] * E;
              } else {
                const double Cp = hist[3 * k + ch], q = E / (E + gray), Tk = exp(-E * a);
                const double dT = lam[ch] * (Cp - q), dq = lam[ch] * (1.0 - Tk);
                ge[ch] = dT * (-a * Tk) + dq * gray / ((E + gray) * (E + gray));
                gatt += dT * (-E * Tk);
                lam[ch] *= Tk;
              }
            }
            const double sigma = h2s * wi[2], stp = -1.0 / (sigma * sigma);
            const double dx = px - wi[0], dy = py - wi[1];
            const double gg[6] = {gatt * a * (-2.0 * stp) * dx, gatt * a * (-2.0 * stp) * dy,
                                  gatt * a * (dx * dx + dy * dy) * (-2.0 * stp / wi[2]),
                                  ge[0], ge[1], ge[2]};
            for (int j = 0; j < 6; ++j) {
#pragma omp atomic
              gw[6 * (size_t)i + j] += gg[j];
            }
          }
        }
    }
    free(att); free(hist); free(cv);
  }
  free_bins(&b);
  return 0;
}

int spo_grad_fp64(const spo_params *prm, const spo_particle *raw, const spo_particle *cov,
                  const uint32_t *order, int64_t n, int T, const double *gpic, double *grad,
                  double gcampos[3]) {
  spo_model m;
  if (spo_model_setup(prm, &m)) return -1;
  double *w = (double *)malloc((size_t)(n > 0 ? n : 1) * 6 * sizeof(double));
  double *gw = (double *)malloc((size_t)(n > 0 ? n : 1) * 6 * sizeof(double));
  double *off = (double *)malloc((size_t)(n > 0 ? n : 1) * 6 * sizeof(double));
  if (!w || !gw || !off) { free(w); free(gw); free(off); return -2; }
  model_offsets(&m, raw, cov, n, off);
  model_all(&m, raw, cov, n, off, w);
  free(off);
  int rc = spo_render_frozen_vjp_fp64(cov, w, order, n, prm->xres, prm->yres, T, prm->a_eq_e,
                                      (double)prm->gray_absorption, gpic, gw);
  gcampos[0] = gcampos[1] = gcampos[2] = 0.0;
  for (int64_t i = 0; i < n && rc == 0; ++i) {
    if (!cov[i].active) { memset(grad + 8 * i, 0, 8 * sizeof(double)); continue; }
    const spo_model_in q = model_in_of(&raw[i]);
    spo_model_vjp(&m, &q, gw + 6 * i, grad + 8 * i, gcampos);
  }
  free(w);
  free(gw);
  return rc;
}

/* Central differences of L = sum((pic - target)^2) of the model with frozen
   coverage.  Per selected particle and input (I, e.r, e.g, e.b, x, y, z, r):
   only the pixels the particle covers change, and each of them is the affine
   image of the particle's own update -- C_final = C_i * Tsuffix + Dsuffix
   (C_i + Dsuffix in additive mode) with C_i computed from the state Cprefix
   that the earlier list entries leave -- so each evaluation costs one pass
   over the covered pixels.  excluded[j] = 1 where the +-h pair lands on
   different palette segments (a kink of the piecewise-linear colour map). */
int spo_fd_particles(const spo_params *prm, const spo_particle *raw, const spo_particle *cov,
                     const uint32_t *order, int64_t n, int T, const float *target,
                     const int64_t *sel, int nsel, double h, double *fd, uint8_t *excluded) {
  spo_model m;
  if (spo_model_setup(prm, &m)) return -1;
  const int xres = prm->xres, yres = prm->yres, a_eq_e = prm->a_eq_e;
  const double gray = prm->gray_absorption;
  double *w = (double *)malloc((size_t)(n > 0 ? n : 1) * 6 * sizeof(double));
  double *off = (double *)malloc((size_t)(n > 0 ? n : 1) * 6 * sizeof(double));
  if (!w || !off) { free(w); free(off); return -2; }
  model_offsets(&m, raw, cov, n, off);
  model_all(&m, raw, cov, n, off, w);
  bins b;
  if (make_bins(cov, order, n, xres, yres, T, &b)) { free(w); return -1; }
  const double h2s = h2sigma_f();
  const float h2sf = h2sigma_f();
  int err = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(spo_get_threads())
  for (int s = 0; s < nsel; ++s) {
    const int64_t i = sel[s];
    memset(fd + 8 * (size_t)s, 0, 8 * sizeof(double));
    memset(excluded + 8 * (size_t)s, 0, 8);
    if (i < 0 || i >= n || !cov[i].active) continue;
    /* pixels covered by i with their prefix state and suffix map */
    int64_t np = 0, capp = 64;
    double *px = (double *)malloc((size_t)capp * 14 * sizeof(double));
    uint32_t ids[4096];
    int nt = particle_tiles(&cov[i], &b.g, NULL);
    if (nt > 4096) { err = 1; free(px); continue; }
    particle_tiles(&cov[i], &b.g, ids);
    for (int tt = 0; tt < nt; ++tt) {
      const int64_t chunk = ids[tt];
      int ix = (int)(chunk % b.g.ncx), iy = (int)(chunk / b.g.ncx);
      int x0s = ix * T, y0s = iy * T;
      int x1 = imin(x0s + T, xres) - x0s, y1 = imin(y0s + T, yres) - y0s;
      int64_t k0 = b.start[chunk], k1 = b.start[chunk + 1], ki = -1;
      for (int64_t k = k0; k < k1; ++k)
        if (b.ent[k] == (uint32_t)i) { ki = k; break; }
      if (ki < 0) continue;
      pcov ci;
      particle_cover(&cov[i], x0s, y0s, x1, y1, h2sf, &ci);
      for (int x = ci.minx; x < ci.maxx; ++x)
        for (int y = ci.miny; y < ci.maxy; ++y) {
          if (!covers_pixel(&ci, x, y)) continue;
          double C[3] = {0, 0, 0}, Tp[3] = {1, 1, 1}, D[3] = {0, 0, 0};
          const double gx = x + x0s, gy = y + y0s;
          for (int64_t k = k0; k < k1; ++k) {
            if (k == ki) continue;
            const uint32_t j = b.ent[k];
            pcov cj;
            particle_cover(&cov[j], x0s, y0s, x1, y1, h2sf, &cj);
            if (!covers_pixel(&cj, x, y)) continue;
            const double *wj = w + 6 * (size_t)j;
            const double att = frag_att(wj, h2s, gx, gy);
            if (k < ki) {
              frag_apply(a_eq_e, gray, wj + 3, att, C);
            } else {
              for (int ch = 0; ch < 3; ++ch) {
                const double E = wj[3 + ch];
                if (a_eq_e) D[ch] += -E * att;
                else {
                  const double Tj = exp(-E * att), q = E / (E + gray);
                  Tp[ch] *= Tj;
                  D[ch] = D[ch] * Tj + q * (1.0 - Tj);
                }
              }
            }
          }
          if (np == capp) {
            capp *= 2;
            px = (double *)realloc(px, (size_t)capp * 14 * sizeof(double));
          }
          double *r = px + 14 * np++;
          r[0] = gx; r[1] = gy;
          const float *tg = target + ((size_t)(x + x0s) * yres + (y + y0s)) * 3;
          for (int ch = 0; ch < 3; ++ch) {
            r[2 + ch] = C[ch]; r[5 + ch] = Tp[ch]; r[8 + ch] = D[ch]; r[11 + ch] = tg[ch];
          }
        }
    }
    for (int j = 0; j < 8; ++j) {
      double L[2];
      int segs[2];
      for (int sg = 0; sg < 2; ++sg) {
        spo_model_in q = model_in_of(&raw[i]);
        double *fld[8] = {&q.I, &q.e[0], &q.e[1], &q.e[2], &q.x, &q.y, &q.z, &q.r};
        *fld[j] += sg ? -h : h;
        double wq[6];
        model_fwd st;
        model_eval(&m, &q, &st, wq);
        for (int jj = 0; jj < 6; ++jj) wq[jj] += off[6 * (size_t)i + jj];
        segs[sg] = st.seg;
        double acc = 0.0;
        for (int64_t k = 0; k < np; ++k) {
          const double *r = px + 14 * k;
          const double att = frag_att(wq, h2s, r[0], r[1]);
          double Ci[3] = {r[2], r[3], r[4]};
          frag_apply(a_eq_e, gray, wq + 3, att, Ci);
          for (int ch = 0; ch < 3; ++ch) {
            const double Cf = a_eq_e ? Ci[ch] + r[8 + ch] : Ci[ch] * r[5 + ch] + r[8 + ch];
            const double dlt = Cf - r[11 + ch];
            acc += dlt * dlt;
          }
        }
        L[sg] = acc;
      }
      fd[8 * (size_t)s + j] = (L[0] - L[1]) / (2.0 * h);
      if (j == 1 && segs[0] != segs[1]) excluded[8 * (size_t)s + j] = 1;
    }
    free(px);
  }
  free_bins(&b);
  free(w);
  free(off);
  return err ? -3 : 0;
}

/* Central differences of the same loss with respect to the camera position
   (centerpos, lookat and sky held): two frozen renders per component. */
int spo_fd_campos(const spo_params *prm, const spo_particle *raw, const spo_particle *cov,
                  const uint32_t *order, int64_t n, int T, const float *target, double h,
                  double fd[3]) {
  const size_t npix = (size_t)prm->xres * prm->yres * 3;
  double *w = (double *)malloc((size_t)(n > 0 ? n : 1) * 6 * sizeof(double));
  double *off = (double *)malloc((size_t)(n > 0 ? n : 1) * 6 * sizeof(double));
  double *pp = (double *)malloc(npix * sizeof(double));
  double *pm = (double *)malloc(npix * sizeof(double));
  if (!w || !off || !pp || !pm) { free(w); free(off); free(pp); free(pm); return -2; }
  int rc = 0;
  {
    spo_model m0;
    if (spo_model_setup(prm, &m0)) rc = -1;
    else model_offsets(&m0, raw, cov, n, off);  /* anchored at the base camera */
  }
  for (int k = 0; k < 3 && rc == 0; ++k) {
    for (int sg = 0; sg < 2 && rc == 0; ++sg) {
      spo_model m;
      if (spo_model_setup(prm, &m)) { rc = -1; break; }
      m.campos[k] += sg ? -h : h;
      model_all(&m, raw, cov, n, off, w);
      if (spo_render_frozen_fp64(cov, w, order, n, prm->xres, prm->yres, T, prm->a_eq_e,
                                 (double)prm->gray_absorption, sg ? pm : pp) < 0)
        rc = -1;
    }
    double acc = 0.0;
    for (size_t j = 0; j < npix && rc == 0; ++j)
      acc += (pp[j] - pm[j]) * (pp[j] + pm[j] - 2.0 * (double)target[j]);
    fd[k] = acc / (2.0 * h);
  }
  free(w); free(off); free(pp); free(pm);
  return rc;
}

/* The smooth model's X, Y, R, E for every active particle (zeros elsewhere),
   without the anchoring offsets. */
int spo_model_project_all(const spo_params *prm, const spo_particle *raw,
                          const spo_particle *cov, int64_t n, double *w) {
  spo_model m;
  if (spo_model_setup(prm, &m)) return -1;
  double *zero = (double *)calloc((size_t)(n > 0 ? n : 1) * 6, sizeof(double));
  if (!zero) return -2;
  model_all(&m, raw, cov, n, zero, w);
  free(zero);
  return 0;
}

/* Per-particle chain rule alone: gw (n x 6, d/d(X,Y,R,E)) -> grad (n x 8). */
int spo_model_vjp_all(const spo_params *prm, const spo_particle *raw, const spo_particle *cov,
                      int64_t n, const double *gw, double *grad, double gcampos[3]) {
  spo_model m;
  if (spo_model_setup(prm, &m)) return -1;
  gcampos[0] = gcampos[1] = gcampos[2] = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    if (!cov[i].active) { memset(grad + 8 * i, 0, 8 * sizeof(double)); continue; }
    const spo_model_in q = model_in_of(&raw[i]);
    spo_model_vjp(&m, &q, gw + 6 * i, grad + 8 * i, gcampos);
  }
  return 0;
}

/* ====================================================================== */
/* Post-processing and image output after host_rendering
   (splotch/splotch.cc:272-323). */

/* pic = -expm1(pic) with exptable<float32>(-20) when a_eq_e
   (splotch.cc:272-281); colour_adjust (splotchutils.cc:230-250); add_colorbar
   (splotchutils.cc:35-58).  Colour-bar rows that would fall below row 0 (more
   than yres/10 palette types) are skipped. */
int spo_postprocess(const spo_params *prm, const spo_post *post, float *pic, int xres,
                    int yres) {
  const size_t nv = (size_t)xres * yres * 3;
  if (post->a_eq_e) {
    exptab t;
    exptab_init(&t, -20.f);
    for (size_t k = 0; k < nv; ++k) pic[k] = -exptab_expm1(&t, pic[k]);
  }
  const double g = post->gamma, h = post->brightness, c = post->contrast;
  if (g != 1.0 || h != 0.0 || c != 1.0)
    for (size_t k = 0; k < nv; ++k) pic[k] = (float)(c * pow((double)pic[k], g) + h);
  if (post->colorbar) {
    int offset = 0;
    for (int t = 0; t < prm->ptypes && t < SPO_MAX_TYPES; ++t) {
      if (prm->color_is_vector[t]) continue;
      for (int x = 0; x < xres; ++x) {
        float e[3];
        palette_lookup(prm->pal_n[t], prm->pal_x[t], prm->pal_rgb[t], x / (double)xres, e);
        for (int y = 0; y < 10; ++y) {
          const int row = yres - offset - 1 - y;
          if (row < 0) continue;
          float *o = pic + ((size_t)x * yres + row) * 3;
          o[0] = e[0]; o[1] = e[1]; o[2] = e[2];
        }
      }
      offset += 10;
    }
  }
  return 0;
}

/* Colour8 (cxxsupport/ls_image.h:65-75) */
static inline uint8_t to8(float v) {
  int i = f2i(v * 256);
  return (uint8_t)(i < 0 ? 0 : (i > 255 ? 255 : i));
}

static void put(uint8_t *out, int64_t cap, int64_t *len, uint8_t v) {
  if (*len < cap) out[*len] = v;
  ++*len;
}

/* The bytes LS_Image writes (cxxsupport/ls_image.cc:178-314) for pictype 0
   (TGA), 2 (PPM) or 3 (run-length TGA).  Returns the length (bytes beyond cap
   are counted, not stored); -1 for another pictype. */
int64_t spo_image_bytes(const float *pic, int xres, int yres, int pictype, uint8_t *out,
                        int64_t cap) {
  int64_t len = 0;
  if (pictype == 0 || pictype == 3) {
    const uint8_t hdr[18] = {0, 0, (uint8_t)(pictype == 0 ? 2 : 10), 0, 0, 0, 0, 0, 0, 0, 0,
                             0, (uint8_t)(xres % 256), (uint8_t)(xres / 256),
                             (uint8_t)(yres % 256), (uint8_t)(yres / 256), 24, 32};
    for (int k = 0; k < 18; ++k) put(out, cap, &len, hdr[k]);
  } else if (pictype == 2) {
    char hdr[64];
    int n = snprintf(hdr, sizeof hdr, "P6\n%d\n%d\n255\n", xres, yres);
    for (int k = 0; k < n; ++k) put(out, cap, &len, (uint8_t)hdr[k]);
  } else {
    return -1;
  }
  uint8_t *row = (uint8_t *)malloc((size_t)xres * 3 + 3);
  for (int j = 0; j < yres; ++j) {
    for (int i = 0; i < xres; ++i) {
      const float *s = pic + ((size_t)i * yres + j) * 3;
      row[3 * i] = to8(s[0]); row[3 * i + 1] = to8(s[1]); row[3 * i + 2] = to8(s[2]);
    }
    if (pictype != 3) {
      for (int i = 0; i < xres; ++i) {
        const uint8_t *p = row + 3 * i;
        if (pictype == 0) { put(out, cap, &len, p[2]); put(out, cap, &len, p[1]); put(out, cap, &len, p[0]); }
        else { put(out, cap, &len, p[0]); put(out, cap, &len, p[1]); put(out, cap, &len, p[2]); }
      }
      continue;
    }
    /* run-length encoding of one row (ls_image.cc:206-286): runs of equal
       pixels and of pairwise-different pixels, each cut into chunks of 128 */
#define SAME(a, b) (row[3 * (a)] == row[3 * (b)] && row[3 * (a) + 1] == row[3 * (b) + 1] && \
                    row[3 * (a) + 2] == row[3 * (b) + 2])
    int xs = 0;
    while (xs < xres) {
      int xe;
      int equal;
      if (xs == xres - 1) { xe = xres; equal = 0; }
      else if (SAME(xs + 1, xs)) {
        xe = xs + 2;
        while (xe < xres && SAME(xe, xs)) ++xe;
        equal = 1;
      } else {
        xe = xs + 2;
        while (xe < xres && !SAME(xe, xe - 1)) ++xe;
        equal = 0;
      }
      for (int cb = xs; cb < xe; cb += 128) {
        const int csz = (xe - cb) < 128 ? (xe - cb) : 128;
        if (equal) {
          put(out, cap, &len, (uint8_t)(csz - 1 + 128));
          put(out, cap, &len, row[3 * xs + 2]); put(out, cap, &len, row[3 * xs + 1]);
          put(out, cap, &len, row[3 * xs]);
        } else {
          put(out, cap, &len, (uint8_t)(csz - 1));
          for (int k = cb; k < cb + csz; ++k) {
            put(out, cap, &len, row[3 * k + 2]); put(out, cap, &len, row[3 * k + 1]);
            put(out, cap, &len, row[3 * k]);
          }
        }
      }
      xs = xe;
    }
#undef SAME
  }
  free(row);
  return len;
}

/* ====================================================================== */
/* sceneMaker::particle_normalize, host branch (splotch/scenemaker.cc:40-296),
   with Normalizer (splotch/splotchutils.h:139-172) and my_asinh
   (splotch/splotchutils.cc:31-32). */

typedef struct { float minv, maxv; } spo_normalizer;

static inline void nz_collect(spo_normalizer *z, float v) {
  /* std::min(minv, v) / std::max(maxv, v): a NaN v leaves both unchanged */
  z->minv = (v < z->minv) ? v : z->minv;
  z->maxv = (z->maxv < v) ? v : z->maxv;
}

static inline float nz_clamp(const spo_normalizer *z, float v) {
  if (z->maxv == z->minv) return 1.f;
  float lo = (v < z->maxv) ? v : z->maxv;  /* min(maxv, v) */
  lo = (z->minv < lo) ? lo : z->minv;      /* max(minv, .) */
  return (lo - z->minv) / (z->maxv - z->minv);
}

static inline float my_asinh_f(float v) {
  const double d = v;
  return (float)log(d + sqrt(1. + d * d));
}

int spo_particle_normalize(const spo_norm_params *np, spo_particle *p, int64_t n,
                           spo_norm_out *out) {
  const int nt = np->ptypes;
  if (nt < 1 || nt > SPO_MAX_TYPES) return -1;
  spo_normalizer in[SPO_MAX_TYPES], cn[SPO_MAX_TYPES], rn[SPO_MAX_TYPES];
  for (int t = 0; t < nt; ++t) {
    in[t].minv = cn[t].minv = rn[t].minv = 1e37f;
    in[t].maxv = cn[t].maxv = rn[t].maxv = -1e37f;
  }
  for (int64_t m = 0; m < n; ++m) {
    spo_particle *q = &p[m];
    const int t = q->type;
    if (t < 0 || t >= nt) return -2;
    nz_collect(&rn[t], q->r);
    if (np->intensity_log[t]) {
      if (q->I > 0) { q->I = log10f(q->I); nz_collect(&in[t], q->I); }
      else q->I = -38;
    } else {
      nz_collect(&in[t], q->I);
    }
    if (np->color_log[t]) {
      if (q->er > 0) { q->er = log10f(q->er); nz_collect(&cn[t], q->er); }
      else q->er = -38;
    } else {
      if (np->color_asinh[t]) q->er = my_asinh_f(q->er);
      nz_collect(&cn[t], q->er);
    }
    if (np->color_is_vector[t]) {
      if (np->color_log[t]) { q->eg = log10f(q->eg); q->eb = log10f(q->eb); }
      if (np->color_asinh[t]) { q->eg = my_asinh_f(q->eg); q->eb = my_asinh_f(q->eb); }
      nz_collect(&cn[t], q->eg);
      nz_collect(&cn[t], q->eb);
    }
  }
  for (int t = 0; t < nt; ++t) {
    out->range_min[t] = cn[t].minv;
    out->range_max[t] = cn[t].maxv;
    if (np->has_intensity_min[t]) in[t].minv = np->intensity_min[t];
    if (np->has_intensity_max[t]) in[t].maxv = np->intensity_max[t];
    if (np->has_color_min[t]) cn[t].minv = np->color_min[t];
    if (np->has_color_max[t]) cn[t].maxv = np->color_max[t];
    out->clamp_min[t] = cn[t].minv;
    out->clamp_max[t] = cn[t].maxv;
    out->intensity_min[t] = in[t].minv;
    out->intensity_max[t] = in[t].maxv;
    out->size_min[t] = rn[t].minv;
    out->size_max[t] = rn[t].maxv;
  }
  for (int64_t m = 0; m < n; ++m) {
    spo_particle *q = &p[m];
    const int t = q->type;
    q->I = nz_clamp(&in[t], q->I);
    q->er = nz_clamp(&cn[t], q->er);
    if (np->color_is_vector[t]) {
      q->eg = nz_clamp(&cn[t], q->eg);
      q->eb = nz_clamp(&cn[t], q->eb);
    }
  }
  return 0;
}
