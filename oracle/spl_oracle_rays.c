/*
 * spl_oracle_rays.c -- CPU oracle of the ray-sphere renderer, TEST
 * INFRASTRUCTURE ONLY (the checker of the CUDA path; the product never links
 * it).
 *
 * Restates host_rendering_new (splotch/new_renderer.cc:522-641), the
 * renderer that host_rendering selects with new_renderer=true
 * (splotch/splotch_host.cc:714-723): every particle is a sphere seen from
 * campos; a pixel ray collects -e*exp(-sin^2(angle)/(r*h2sigma)^2) from each
 * sphere it meets (additive only).  Particles are rendered on a pyramid of
 * pixel grids chosen by their angular radius, each grid by a recursive
 * subdivision of the image with per-region culling, and the grids are summed
 * by bilinear upsampling.
 *
 * Two arithmetic modes with the same decisions (culling, coverage):
 *   exact = 0: the reference's arithmetic -- exptable<double>(-20) weights,
 *              COLOUR (float) sums -- pinned bit-for-bit against the
 *              reference's own compiled renderer;
 *   exact = 1: FP64 truth -- exact exp, double sums (pic64).
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "spl_oracle.h"

#define R_PI 3.141592653589793238462643383279502884197
#define R_HALFPI 1.570796326794896619231321691639751442099

typedef struct { double x, y, z; } rv3;

static rv3 rv(double x, double y, double z) { rv3 r = {x, y, z}; return r; }
static rv3 radd(rv3 a, rv3 b) { return rv(a.x + b.x, a.y + b.y, a.z + b.z); }
static rv3 rsub(rv3 a, rv3 b) { return rv(a.x - b.x, a.y - b.y, a.z - b.z); }
static rv3 rscale(rv3 a, double f) { return rv(a.x * f, a.y * f, a.z * f); }
static double rdot(rv3 a, rv3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static double rlen(rv3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static rv3 rcross(rv3 a, rv3 b) { /* cxxsupport/vec3.h:129-131 */
  return rv(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static rv3 rnorm(rv3 a) { /* vec3.h:72-83: scale by 1/length */
  double l = 1. / sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return rv(a.x * l, a.y * l, a.z * l);
}

/* ---- exptable<double>(-20) (splotch/splotchutils.h:174-215) ---------- */
static double g_tab1[1024], g_tab2[1024], g_expfac;
static int g_tab_ready;
static void rtab_init(void) {
  if (g_tab_ready) return;
  g_expfac = (double)(1 << 20) / -20.;
  for (int m = 0; m < 1024; ++m) {
    g_tab1[m] = exp((double)(m * 1024) / g_expfac);
    g_tab2[m] = exp((double)m / g_expfac);
  }
  g_tab_ready = 1;
}
static double rtab_exp(double arg) {
  /* int(NaN) is INT_MIN on x86-64 and 0 on AArch64: both give 1 below */
  double v = arg * g_expfac;
  int iarg = (v != v) ? 0 : (int)v;
  if (iarg & ~((1 << 20) - 1)) return iarg < 0 ? 1. : 0.;
  return g_tab1[iarg >> 10] * g_tab2[iarg & 1023];
}
/* exact weight; NaN arguments give 1, as the table does */
static double exact_exp(double arg) { return arg != arg ? 1. : exp(arg); }

/* ---- projectors (new_renderer.cc:51-241) ------------------------------ */
typedef struct {
  int dome;
  rv3 p0, dpx, dpy;     /* PlaneProjector */
  rv3 zen, ex, ey;      /* DomeProjector: zenith, x, y */
  double dp;
} rproj;

static rv3 pix_dir(const rproj *P, int ix, int iy) {
  if (!P->dome) /* (p0+dpx*ix+dpy*iy).Norm() */
    return rnorm(radd(radd(P->p0, rscale(P->dpx, (double)ix)), rscale(P->dpy, (double)iy)));
  double px = 2. * P->dp * (ix + .5) - 1., py = 2. * P->dp * (iy + .5) - 1.;
  double r = sqrt(px * px + py * py), xr = 1. / r;
  double theta = R_HALFPI * r;
  double sthxr = sin(theta) * xr;
  return radd(radd(rscale(P->ex, sthxr * px), rscale(P->ey, sthxr * py)),
              rscale(P->zen, cos(theta)));
}

static double pix_rad(const rproj *P) {
  if (P->dome) return P->dp * R_PI;
  double screendist = fabs(rdot(P->p0, rnorm(rcross(P->dpx, P->dpy))));
  double a = rlen(P->dpx), b = rlen(P->dpy);
  return (a < b ? a : b) / screendist;
}

typedef struct { rv3 c; double r; } rpart;

/* Region test of reduceList for pixel columns [ix0,ix1), rows [iy0,iy1). */
typedef struct {
  rv3 n[4];               /* plane: the four side normals */
  int centered;           /* dome */
  rv3 nx0, nx1;
  double thetamin, thetamax, cthetamin, cthetamax;
} rregion;

static void region_setup(const rproj *P, int ix0, int ix1, int iy0, int iy1, rregion *g) {
  if (!P->dome) { /* new_renderer.cc:77-101 */
    double x0 = ix0, x1 = ix1, y0 = iy0, y1 = iy1;
    if (ix1 == ix0 + 1) x1 += 0.001;
    if (iy1 == iy0 + 1) y1 += 0.001;
    rv3 corner[4];
    corner[0] = radd(radd(P->p0, rscale(P->dpx, x0)), rscale(P->dpy, y0));
    corner[1] = radd(radd(P->p0, rscale(P->dpx, x1 - 1)), rscale(P->dpy, y0));
    corner[2] = radd(radd(P->p0, rscale(P->dpx, x1 - 1)), rscale(P->dpy, y1 - 1));
    corner[3] = radd(radd(P->p0, rscale(P->dpx, x0)), rscale(P->dpy, y1 - 1));
    for (int k = 0; k < 4; ++k) g->n[k] = rnorm(rcross(corner[k], corner[(k + 1) & 3]));
    return;
  }
  /* new_renderer.cc:164-213 */
  double dp = P->dp;
  double x0 = 2. * dp * (ix0 + .5) - 1., x1 = 2. * dp * (ix1 - .5) - 1.;
  double y0 = 2. * dp * (iy0 + .5) - 1., y1 = 2. * dp * (iy1 - .5) - 1.;
  if (ix1 == ix0 + 1) x1 += 0.001 * dp;
  if (iy1 == iy0 + 1) y1 += 0.001 * dp;
  g->centered = ((x0 * x1) <= 0) && ((y0 * y1) <= 0);
  double amaxx = fmax(fabs(x0), fabs(x1)), amaxy = fmax(fabs(y0), fabs(y1));
  double aminx = fmin(fabs(x0), fabs(x1)), aminy = fmin(fabs(y0), fabs(y1));
  g->thetamax = R_HALFPI * sqrt(amaxx * amaxx + amaxy * amaxy);
  g->thetamin = 0;
  if (!g->centered) {
    if (x0 * x1 <= 0) g->thetamin = R_HALFPI * aminy;
    else if (y0 * y1 <= 0) g->thetamin = R_HALFPI * aminx;
    else g->thetamin = R_HALFPI * sqrt(aminx * aminx + aminy * aminy);
  }
  g->cthetamin = cos(g->thetamin);
  g->cthetamax = cos(g->thetamax);
  rv3 c = radd(rscale(P->ex, (x0 + x1) * .5), rscale(P->ey, (y0 + y1) * .5));
  rv3 n[4];
  n[0] = rnorm(rsub(rscale(P->ex, y0), rscale(P->ey, x0)));
  n[1] = rnorm(rsub(rscale(P->ex, y1), rscale(P->ey, x0)));
  n[2] = rnorm(rsub(rscale(P->ex, y0), rscale(P->ey, x1)));
  n[3] = rnorm(rsub(rscale(P->ex, y1), rscale(P->ey, x1)));
  rv3 nx0 = n[0], nx1 = n[1];
  double curmin = 1.5;
  for (int i = 0; i < 4; ++i)
    for (int j = i + 1; j < 4; ++j)
      if (rdot(n[i], n[j]) < curmin) {
        curmin = rdot(n[i], n[j]);
        nx0 = n[i];
        nx1 = n[j];
      }
  if (rdot(c, nx0) > 0) nx0 = rscale(nx0, -1.); /* Flip: negation */
  if (rdot(c, nx1) > 0) nx1 = rscale(nx1, -1.);
  g->nx0 = nx0;
  g->nx1 = nx1;
}

static int region_keeps(const rproj *P, const rregion *g, const rpart *pg) {
  if (!P->dome)
    return (pg->r > rdot(pg->c, g->n[0])) && (pg->r > rdot(pg->c, g->n[1])) &&
           (pg->r > rdot(pg->c, g->n[2])) && (pg->r > rdot(pg->c, g->n[3]));
  if (pg->r < -rdot(P->zen, pg->c)) return 0;
  if (!g->centered)
    if ((pg->r < rdot(pg->c, g->nx0)) || (pg->r < rdot(pg->c, g->nx1))) return 0;
  double cpthetac = rdot(P->zen, pg->c);
  if ((cpthetac > g->cthetamin) || (cpthetac < g->cthetamax)) {
    double pthetac = atan2(rlen(rcross(P->zen, pg->c)), rdot(P->zen, pg->c));
    double dptheta = atan2(pg->r, sqrt((1. + pg->r) * (1. - pg->r)));
    if ((pthetac + dptheta < g->thetamin) || (pthetac - dptheta > g->thetamax)) return 0;
  }
  return 1;
}

static int64_t reduce(const rproj *P, int ix0, int ix1, int iy0, int iy1, const rpart *p,
                      const uint32_t *in, int64_t nin, uint32_t *out) {
  rregion g;
  region_setup(P, ix0, ix1, iy0, iy1, &g);
  int64_t k = 0;
  for (int64_t i = 0; i < nin; ++i)
    if (region_keeps(P, &g, &p[in[i]])) out[k++] = in[i];
  return k;
}

/* ---- one pixel grid (subrender4, new_renderer.cc:247-364) ------------- */
typedef struct {
  const rproj *P;
  int fact, xdim, ydim, exact;
  const rpart *p;
  const float *pod;     /* 3 per particle */
  float *pic;           /* x-major xdim*ydim*3 (exact == 0) */
  double *pic64;        /* (exact == 1) */
  double h2;            /* h2sigma */
  int64_t frags;
} grid;

static void render_leaf(grid *G, int x0, int x1, int y0, int y1, const uint32_t *l, int64_t nl) {
  int64_t frags = 0;
  for (int ix = x0; ix < x1; ++ix)
    for (int iy = y0; iy < y1; ++iy) {
      rv3 dir = pix_dir(G->P, ix * G->fact, iy * G->fact);
      float od[3] = {0.f, 0.f, 0.f};
      double od64[3] = {0., 0., 0.};
      for (int64_t k = 0; k < nl; ++k) {
        const rpart *q = &G->p[l[k]];
        double r = q->r;
        double cosang = rdot(dir, q->c);
        if (cosang < 0) continue;
        double casq = cosang * cosang;
        double crsq = (1. - r) * (1. + r);
        if (casq < crsq) continue; /* no intersection */
        double sasq = (1. - cosang) * (1. + cosang);
        double fract = sasq / (r * r * G->h2 * G->h2);
        const float *e = G->pod + 3 * (size_t)l[k];
        ++frags;
        if (G->exact) {
          double w = -exact_exp(-fract);
          for (int ch = 0; ch < 3; ++ch) od64[ch] += (double)e[ch] * w;
        } else {
          double w = -rtab_exp(-fract);
          for (int ch = 0; ch < 3; ++ch) od[ch] += (float)(e[ch] * w);
        }
      }
      size_t px = ((size_t)ix * G->ydim + iy) * 3;
      for (int ch = 0; ch < 3; ++ch) {
        if (G->exact) G->pic64[px + ch] = od64[ch];
        else G->pic[px + ch] = od[ch];
      }
    }
#pragma omp atomic
  G->frags += frags;
}

static void zero_region(grid *G, int x0, int x1, int y0, int y1) {
  for (int ix = x0; ix < x1; ++ix)
    for (int iy = y0; iy < y1; ++iy)
      for (int ch = 0; ch < 3; ++ch) {
        size_t px = ((size_t)ix * G->ydim + iy) * 3 + ch;
        if (G->exact) G->pic64[px] = 0.;
        else G->pic[px] = 0.f;
      }
}

/* One job of subrender4: list = the parent's reduced list. */
static void job(grid *G, int x0, int x1, int y0, int y1, const uint32_t *list, int64_t nlist) {
  const uint32_t *l2 = list;
  uint32_t *own = NULL;
  int64_t n2 = nlist;
  if (!(x0 == 0 && x1 == G->xdim && y0 == 0 && y1 == G->ydim)) {
    own = (uint32_t *)malloc((nlist ? nlist : 1) * sizeof(uint32_t));
    n2 = reduce(G->P, x0 * G->fact, (x1 - 1) * G->fact + 1, y0 * G->fact,
                (y1 - 1) * G->fact + 1, G->p, list, nlist, own);
    l2 = own;
  }
  int nx = x1 - x0, ny = y1 - y0;
  if (n2 == 0) {
    zero_region(G, x0, x1, y0, y1);
  } else if (nx < 10 && ny < 10) {
    render_leaf(G, x0, x1, y0, y1, l2, n2);
  } else {
    int xm = (x0 + x1) >> 1, ym = (y0 + y1) >> 1;
    const int big = n2 > 4096;
    if (nx > sqrt(2.) * ny) {
#pragma omp task if (big)
      job(G, x0, xm, y0, y1, l2, n2);
      job(G, xm, x1, y0, y1, l2, n2);
    } else if (ny > sqrt(2.) * nx) {
#pragma omp task if (big)
      job(G, x0, x1, y0, ym, l2, n2);
      job(G, x0, x1, ym, y1, l2, n2);
    } else {
#pragma omp task if (big)
      job(G, x0, xm, y0, ym, l2, n2);
#pragma omp task if (big)
      job(G, x0, xm, ym, y1, l2, n2);
#pragma omp task if (big)
      job(G, xm, x1, y0, ym, l2, n2);
      job(G, xm, x1, ym, y1, l2, n2);
    }
#pragma omp taskwait
  }
  free(own);
}

/* add_overlap2 (new_renderer.cc:367-393): spheres that contain the camera. */
static void add_overlap(grid *G, const rpart *po, const float *podo, int64_t npo) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(spo_get_threads())
  for (int ix = 0; ix < G->xdim; ++ix)
    for (int iy = 0; iy < G->ydim; ++iy) {
      rv3 dir = pix_dir(G->P, ix * G->fact, iy * G->fact);
      float od[3] = {0.f, 0.f, 0.f};
      double od64[3] = {0., 0., 0.};
      for (int64_t i = 0; i < npo; ++i) {
        double r = po[i].r;
        double cosang = rdot(dir, po[i].c);
        double sasq = (1. - cosang) * (1. + cosang);
        double fract = sasq / (r * r * G->h2 * G->h2);
        double er = 0.5 * (erfc(-cosang / (r * G->h2)));
        const float *e = podo + 3 * (size_t)i;
        if (G->exact) {
          double w = -exact_exp(-fract);
          for (int ch = 0; ch < 3; ++ch) od64[ch] += er * (double)e[ch] * w;
        } else {
          double w = -rtab_exp(-fract);
          for (int ch = 0; ch < 3; ++ch) od[ch] += (float)((float)(e[ch] * er) * w);
        }
      }
      size_t px = ((size_t)ix * G->ydim + iy) * 3;
      for (int ch = 0; ch < 3; ++ch) {
        if (G->exact) G->pic64[px + ch] += od64[ch];
        else G->pic[px + ch] += od[ch];
      }
    }
}

/* ---- host_rendering_new ------------------------------------------------ */
int spo_render_rays(const spo_params *prm, const spo_rays_params *rp, spo_particle *pp,
                    int64_t n, int exact, float *pic_out, double *pic64_out, int64_t *stats) {
  const double h2sigma = 0.5 * pow(R_PI, -1. / 6.);
  const double bfak = 0.5 * pow(R_PI, -5. / 6.);
  if (!prm->a_eq_e) return -1; /* planck_assert(a_eq_e, "inconsistent") */
  const int xres = prm->xres, yres = prm->yres;
  if (rp->dome && xres != yres) return -2;
  rtab_init();
  const int nthr = spo_get_threads();

  /* classic intensity and radius scaling, distance cut (new_renderer.cc:530-561) */
  const rv3 campos = rv(prm->campos[0], prm->campos[1], prm->campos[2]);
  const rv3 centerpos = rv(prm->centerpos[0], prm->centerpos[1], prm->centerpos[2]);
  const rv3 lookat = rv(prm->lookat[0], prm->lookat[1], prm->lookat[2]);
  rv3 sky = rv(prm->sky[0], prm->sky[1], prm->sky[2]);
#pragma omp parallel for num_threads(nthr)
  for (int64_t m = 0; m < n; ++m) {
    pp[m].I = (float)(pp[m].I * (0.5f * bfak / pp[m].r));
    pp[m].r *= 2;
    rv3 pos = rv(pp[m].x, pp[m].y, pp[m].z);
    float dist = (float)rlen(rsub(centerpos, pos));
    pp[m].active = dist < prm->zmax;
  }
  spo_colorize(prm, pp, n);

  int64_t nuse = 0;
  for (int64_t i = 0; i < n; ++i) nuse += pp[i].active != 0;
  rpart *p = (rpart *)malloc((nuse ? nuse : 1) * sizeof(rpart));
  float *pod = (float *)malloc((nuse ? nuse : 1) * 3 * sizeof(float));
  {
    int64_t j = 0;
    for (int64_t i = 0; i < n; ++i)
      if (pp[i].active) {
        p[j].c = rsub(rv(pp[i].x, pp[i].y, pp[i].z), campos);
        p[j].r = pp[i].r;
        pod[3 * j] = pp[i].er;
        pod[3 * j + 1] = pp[i].eg;
        pod[3 * j + 2] = pp[i].eb;
        ++j;
      }
  }

  /* projector (new_renderer.cc:588-612) */
  rproj P;
  memset(&P, 0, sizeof(P));
  P.dome = rp->dome;
  if (rp->dome) {
    P.dp = 1. / xres;
    P.zen = rnorm(rsub(lookat, campos));
    P.ey = rnorm(rcross(P.zen, sky));
    P.ex = rnorm(rcross(P.ey, P.zen));
  } else {
    double fovfct = tan(rp->fov * 0.5f * (R_PI / 180.0));
    sky = rnorm(sky);
    rv3 zaxis = rnorm(rsub(centerpos, lookat));
    rv3 xaxis = rnorm(rcross(sky, zaxis));
    rv3 yaxis = rnorm(rcross(zaxis, xaxis));
    P.dpx = rscale(xaxis, fovfct / (0.5 * xres));
    P.dpy = rscale(yaxis, fovfct / (0.5 * xres));
    rv3 newcenter = rscale(rsub(centerpos, campos), 1. / rlen(rsub(centerpos, lookat)));
    rv3 corner = rsub(rsub(rsub(newcenter, zaxis), rscale(P.dpx, 0.5 * xres)),
                      rscale(P.dpy, 0.5 * yres));
    P.p0 = radd(radd(corner, rscale(P.dpx, .5)), rscale(P.dpy, .5));
  }

  /* real_host_rendering (new_renderer.cc:395-519) */
  const double pixrad = pix_rad(&P);
  const double mr = rp->minrad_pix;
#pragma omp parallel for num_threads(nthr)
  for (int64_t i = 0; i < nuse; ++i) {
    double xl = 1. / rlen(p[i].c);
    p[i].c = rscale(p[i].c, xl);
    p[i].r *= xl;
    double rcorr = sqrt(p[i].r * p[i].r + mr * mr * pixrad * pixrad) / p[i].r;
    p[i].r *= rcorr;
    float fac = (float)(1. / (rcorr * rcorr));
    for (int ch = 0; ch < 3; ++ch) pod[3 * i + ch] *= fac;
  }
  /* screen cull; spheres around the camera (r > 1) go to the overlap list */
  int64_t nkeep = 0, npo = 0, np = 0;
  uint32_t *all = (uint32_t *)malloc((nuse ? nuse : 1) * sizeof(uint32_t));
  uint32_t *kept = (uint32_t *)malloc((nuse ? nuse : 1) * sizeof(uint32_t));
  for (int64_t i = 0; i < nuse; ++i) all[i] = (uint32_t)i;
  nkeep = reduce(&P, 0, xres, 0, yres, p, all, nuse, kept);
  rpart *po = (rpart *)malloc((nkeep ? nkeep : 1) * sizeof(rpart));
  float *podo = (float *)malloc((nkeep ? nkeep : 1) * 3 * sizeof(float));
  for (int64_t k = 0; k < nkeep; ++k) {
    uint32_t i = kept[k];
    if (p[i].r > 1) {
      po[npo] = p[i];
      memcpy(podo + 3 * npo, pod + 3 * (size_t)i, 12);
      ++npo;
    } else {
      p[np] = p[i];
      memmove(pod + 3 * np, pod + 3 * (size_t)i, 12);
      ++np;
    }
  }

  const double minpixperrad = 15;
  double maxfac = 1. / (minpixperrad * pixrad);
  double mres = (xres < yres ? xres : yres) / 10.;
  if (mres < maxfac) maxfac = mres;
  int nsteps = 0;
  while ((1 << nsteps) < maxfac) ++nsteps;
  nsteps = nsteps - 1 > 0 ? nsteps - 1 : 0;

  float *pic = NULL;
  double *pic64 = NULL;
  int pdx = 0, pdy = 0;
  int64_t frags = 0;
  uint32_t *lst = (uint32_t *)malloc((np ? np : 1) * sizeof(uint32_t));
  for (int fact = 1 << nsteps; fact > 0; fact >>= 1) {
    int xdim = xres, ydim = yres;
    for (int f2 = fact; f2 > 1; f2 >>= 1) {
      xdim = (xdim >> 1) + 1;
      ydim = (ydim >> 1) + 1;
    }
    size_t npx = (size_t)xdim * ydim * 3;
    float *xpic = exact ? NULL : (float *)calloc(npx, sizeof(float));
    double *xpic64 = exact ? (double *)calloc(npx, sizeof(double)) : NULL;
    double minrad = minpixperrad * pixrad * fact;
    double maxrad = 2 * minrad < 1. ? 2 * minrad : 1.;
    if (fact == 1) minrad = 0.;
    if (fact == 1 << nsteps) maxrad = 1;
    int64_t nl = 0;
    for (int64_t i = 0; i < np; ++i)
      if ((p[i].r > minrad) && (p[i].r <= maxrad)) lst[nl++] = (uint32_t)i;
    grid G = {&P, fact, xdim, ydim, exact, p, pod, xpic, xpic64, h2sigma, 0};
#pragma omp parallel num_threads(nthr)
#pragma omp single
    job(&G, 0, xdim, 0, ydim, lst, nl);
    frags += G.frags;
    if (fact == 1 << nsteps) add_overlap(&G, po, podo, npo);
    if (fact != 1 << nsteps) { /* add the coarser grid, upsampled */
#pragma omp parallel for num_threads(nthr)
      for (int ix = 0; ix < xdim; ++ix)
        for (int iy = 0; iy < ydim; ++iy)
          for (int ch = 0; ch < 3; ++ch) {
            size_t a = ((size_t)(ix >> 1) * pdy + (iy >> 1)) * 3 + ch;
            size_t b = ((size_t)((ix + 1) >> 1) * pdy + (iy >> 1)) * 3 + ch;
            size_t c = ((size_t)(ix >> 1) * pdy + ((iy + 1) >> 1)) * 3 + ch;
            size_t d = ((size_t)((ix + 1) >> 1) * pdy + ((iy + 1) >> 1)) * 3 + ch;
            size_t o = ((size_t)ix * ydim + iy) * 3 + ch;
            if (exact)
              xpic64[o] += (((pic64[a] + pic64[b]) + pic64[c]) + pic64[d]) * 0.25;
            else
              xpic[o] += (float)((((pic[a] + pic[b]) + pic[c]) + pic[d]) * 0.25);
          }
    }
    free(pic);
    free(pic64);
    pic = xpic;
    pic64 = xpic64;
    pdx = xdim;
    pdy = ydim;
  }
  (void)pdx;

  if (rp->dome) { /* corners outside the fisheye circle (new_renderer.cc:619-639) */
    int res = xres;
    double xf = 1. / (res - 1);
    for (int i = 0; i <= res / 2; ++i) {
      double x = (i + 0.5) * xf;
      x = 2 * x - 1;
      for (int j = 0; j < res; ++j) {
        double y = (j + 0.5) * xf;
        y = 2 * y - 1;
        if (x * x + y * y > 1.) {
          int q[4][2] = {{i, j}, {i, res - 1 - j}, {res - 1 - i, res - 1 - j}, {res - 1 - i, j}};
          for (int k = 0; k < 4; ++k)
            for (int ch = 0; ch < 3; ++ch) {
              size_t o = ((size_t)q[k][0] * res + q[k][1]) * 3 + ch;
              if (exact) pic64[o] = 0.;
              else pic[o] = 0.f;
            }
        } else {
          break;
        }
      }
    }
  }
  size_t npx = (size_t)xres * yres * 3;
  if (exact) memcpy(pic64_out, pic64, npx * sizeof(double));
  else memcpy(pic_out, pic, npx * sizeof(float));
  if (stats) {
    stats[0] = nuse;
    stats[1] = np;
    stats[2] = npo;
    stats[3] = nsteps + 1;
    stats[4] = frags;
  }
  free(pic);
  free(pic64);
  free(lst);
  free(p);
  free(pod);
  free(all);
  free(kept);
  free(po);
  free(podo);
  return 0;
}
