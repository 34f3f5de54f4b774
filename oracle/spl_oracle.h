/*
 * spl_oracle.h -- CPU oracle for the Splotch particle-render path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the
 * reference's host renderer (splotch/splotch_host.cc, splotch/splotchutils.h,
 * kernel/transform.cxx, cxxsupport/linear_map.h).  It is the checker for the
 * CUDA path: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it.  The product library never links or calls it.
 *
 * Parity pin: every stage is checked bit-for-bit against the reference's own
 * compiled code (oracle/_ref, built from the reference sources by
 * oracle/build_ref.sh) through the golden fixtures in tests/golden/.
 */
#ifndef SPL_ORACLE_H
#define SPL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Byte layout of particle_sim (splotch/splotchutils.h:52-72, non-MPI build):
   COLOUR e (3 floats), x, y, z, r, I, unsigned short type, bool active. */
typedef struct {
  float er, eg, eb;
  float x, y, z, r, I;
  uint16_t type;
  uint8_t active;
  uint8_t pad;
} spo_particle;

#define SPO_MAX_TYPES 8

/* Everything host_rendering() reads from the paramfile and render_context. */
typedef struct {
  int xres, yres;
  float fov, zmin, zmax, minrad_pix;
  int projection;
  int ptypes;
  float smooth_factor[SPO_MAX_TYPES];
  float brightness[SPO_MAX_TYPES];
  int color_is_vector[SPO_MAX_TYPES];
  float b_brightness;
  int pal_n[SPO_MAX_TYPES];
  const double *pal_x[SPO_MAX_TYPES];
  const float *pal_rgb[SPO_MAX_TYPES]; /* 3*n floats, r,g,b interleaved */
  int a_eq_e;
  float gray_absorption;
  int sort_type;
  int tile_size;
  double campos[3], lookat[3], sky[3], centerpos[3];
} spo_params;

/* Camera quantities of particle_project (splotch/splotch_host.cc:62-110). */
typedef struct {
  float mat[12]; /* TRANSFORM matrix, TRANSMAT::p layout */
  float res2, ycorr, fovfct, xfac;
  double xshift, yshift;
} spo_camera;

void spo_set_threads(int n);
int spo_get_threads(void);

int spo_camera_setup(const spo_params *prm, spo_camera *cam);
void spo_project(const spo_params *prm, const spo_camera *cam, spo_particle *p,
                 int64_t n);
void spo_colorize(const spo_params *prm, spo_particle *p, int64_t n);

/* Stable sort by the sort_type comparator; perm[i] = original index. */
int spo_sort_perm(const spo_particle *p, int64_t n, int sort_type,
                  uint32_t *perm);
void spo_apply_perm(const spo_particle *in, const uint32_t *perm, int64_t n,
                    spo_particle *out);

/* Binning loop of render_new (splotch_host.cc:356-406) at tile size T.
   Particles are visited in sequence order (order==NULL: 0..n-1); entries hold
   original particle indices.  tile_start has ntiles+1 slots. */
int64_t spo_bin(const spo_particle *p, const uint32_t *order, int64_t n,
                int xres, int yres, int T, int64_t *tile_start,
                uint32_t *entries);

/* Splat of render_new (splotch_host.cc:434-692).  pic is x-major
   [xres][yres][3].  simd_branch selects the __SSE2__ absorption branch
   (splotch_host.cc:647-658) instead of the scalar one (:663-665).
   Returns the exact fragment count of the reference loop. */
int64_t spo_render_fp32(const spo_particle *p, const uint32_t *order,
                        int64_t n, int xres, int yres, int T, int a_eq_e,
                        float gray, int simd_branch, float *pic);

/* Same coverage decisions as the FP32 loop, Gaussian weights and
   compositing in double with exact exp/expm1. */
int64_t spo_render_fp64(const spo_particle *p, const uint32_t *order,
                        int64_t n, int xres, int yres, int T, int a_eq_e,
                        double gray, double *pic);

/* Whole host_rendering(): camera, project, colourise, stable sort when
   !a_eq_e (p is permuted in place), binning and FP32 splat. */
int spo_host_rendering(const spo_params *prm, spo_particle *p, int64_t n,
                       int simd_branch, float *pic);

/* FP64 adjoint of the splat for the L2-type loss sum(gpic * pic).
   Inputs: projected+colourised particles (x,y,r,e), the visiting order,
   the upstream gradient gpic (x-major, 3 channels).  Outputs per particle:
   d/dx, d/dy, d/dr, d/de (3).  Coverage decisions are held fixed. */
int spo_splat_adjoint_fp64(const spo_particle *p, const uint32_t *order,
                           int64_t n, int xres, int yres, int T, int a_eq_e,
                           double gray, const double *gpic, double *gx,
                           double *gy, double *gr, double *ge);

/* ---- differentiable FP64 model: checker of the adjoint path ------------
   particle_project + particle_colorize (splotch_host.cc:111-153, 270-284)
   as a smooth double-precision function of a particle's inputs and of the
   camera position (centerpos, lookat, sky held); coverage, tile lists and
   order stay at the reference's float decisions ("frozen").  Loss
   L = sum over pixels and channels of (pic - target)^2 for the FD routines. */
typedef struct {
  double A[3][3]; /* camera rotation: the float TRANSMAT entries */
  double campos[3], centerpos[3];
  double res2, ycorr, fovfct, xfac;
  int projection;
  double minrad, bfak, h2sigma;
  double smooth[SPO_MAX_TYPES], bright[SPO_MAX_TYPES]; /* bright*b_brightness */
  int colvec[SPO_MAX_TYPES];
  int pal_n[SPO_MAX_TYPES];
  const double *pal_x[SPO_MAX_TYPES];
  const float *pal_rgb[SPO_MAX_TYPES];
} spo_model;

/* One particle's inputs in double: I, colour (palette value in e[0], or
   RGB), world position, hsml, type. */
typedef struct {
  double I, e[3], x, y, z, r;
  int type;
} spo_model_in;

int spo_model_setup(const spo_params *prm, spo_model *m);
/* w = X, Y, R (pixels), E.r, E.g, E.b */
void spo_model_project(const spo_model *m, const spo_model_in *p, double w[6]);
/* gin = dL/d(X, Y, R, E); gout = dL/d(I, e.r, e.g, e.b, x, y, z, r);
   gcampos += dL/dcampos of this particle */
void spo_model_vjp(const spo_model *m, const spo_model_in *p, const double gin[6],
                   double gout[8], double gcampos[3]);
int spo_model_project_all(const spo_params *prm, const spo_particle *raw,
                          const spo_particle *cov, int64_t n, double *w);
int spo_model_vjp_all(const spo_params *prm, const spo_particle *raw,
                      const spo_particle *cov, int64_t n, const double *gw,
                      double *grad, double gcampos[3]);
/* Splat with coverage from cov (projected particles) and weights w (n x 6). */
int64_t spo_render_frozen_fp64(const spo_particle *cov, const double *w,
                               const uint32_t *order, int64_t n, int xres,
                               int yres, int T, int a_eq_e, double gray,
                               double *pic);
/* Its exact reverse mode: gw = dL/dw for L = sum(gpic * pic). */
int spo_render_frozen_vjp_fp64(const spo_particle *cov, const double *w,
                               const uint32_t *order, int64_t n, int xres,
                               int yres, int T, int a_eq_e, double gray,
                               const double *gpic, double *gw);
/* Full FP64 gradient: grad (n x 8, the gout layout) and dL/dcampos. */
int spo_grad_fp64(const spo_params *prm, const spo_particle *raw,
                  const spo_particle *cov, const uint32_t *order, int64_t n, int T,
                  const double *gpic, double *grad, double gcampos[3]);
/* Central finite differences (step h) of L for selected particles
   (fd: nsel x 8, excluded: nsel x 8 palette-kink flags) and for campos. */
int spo_fd_particles(const spo_params *prm, const spo_particle *raw,
                     const spo_particle *cov, const uint32_t *order, int64_t n,
                     int T, const float *target, const int64_t *sel, int nsel,
                     double h, double *fd, uint8_t *excluded);
int spo_fd_campos(const spo_params *prm, const spo_particle *raw,
                  const spo_particle *cov, const uint32_t *order, int64_t n,
                  int T, const float *target, double h, double fd[3]);

/* ---- after host_rendering: post-processing and image output -------------
   splotch/splotch.cc:272-323, splotchutils.cc:35-58,230-250,
   cxxsupport/ls_image.cc:178-314. */
typedef struct {
  int a_eq_e;        /* pic = -expm1(pic) with exptable<float32>(-20) */
  double gamma, brightness, contrast; /* pic_gamma, pic_brightness, pic_contrast */
  int colorbar;
} spo_post;
/* in place on an x-major image; palettes and types from prm */
int spo_postprocess(const spo_params *prm, const spo_post *post, float *pic, int xres,
                    int yres);
/* the file bytes of pictype 0 (TGA), 2 (PPM), 3 (run-length TGA) */
int64_t spo_image_bytes(const float *pic, int xres, int yres, int pictype, uint8_t *out,
                        int64_t cap);

/* ---- before host_rendering: sceneMaker::particle_normalize ---------------
   splotch/scenemaker.cc:40-296 (host branch): per type optional log10 of I,
   log10 or asinh of the colour, min/max of size, intensity and colour,
   optional intensity_min/max and color_min/max overrides, then
   Normalizer::normAndClamp of I and colour. */
typedef struct {
  int ptypes;
  int intensity_log[SPO_MAX_TYPES], color_log[SPO_MAX_TYPES];
  int color_asinh[SPO_MAX_TYPES], color_is_vector[SPO_MAX_TYPES];
  int has_intensity_min[SPO_MAX_TYPES], has_intensity_max[SPO_MAX_TYPES];
  int has_color_min[SPO_MAX_TYPES], has_color_max[SPO_MAX_TYPES];
  float intensity_min[SPO_MAX_TYPES], intensity_max[SPO_MAX_TYPES];
  float color_min[SPO_MAX_TYPES], color_max[SPO_MAX_TYPES];
} spo_norm_params;
typedef struct {
  /* range_*: colour range of the data (the range_min/max keys it sets);
     clamp_*: the colour range used, after overrides (clamp_min/max keys) */
  double range_min[SPO_MAX_TYPES], range_max[SPO_MAX_TYPES];
  double clamp_min[SPO_MAX_TYPES], clamp_max[SPO_MAX_TYPES];
  double intensity_min[SPO_MAX_TYPES], intensity_max[SPO_MAX_TYPES];
  double size_min[SPO_MAX_TYPES], size_max[SPO_MAX_TYPES];
} spo_norm_out;
int spo_particle_normalize(const spo_norm_params *np, spo_particle *p, int64_t n,
                           spo_norm_out *out);

/* ---- host_rendering_new: the ray-sphere renderer -------------------------
   splotch/new_renderer.cc:522-641, selected by new_renderer=true
   (splotch/splotch_host.cc:714-723).  Reads xres, yres, zmax, ptypes,
   brightness, color_is_vector, palettes, b_brightness and the camera vectors
   from prm; fov and minrad_pix come from rp because this renderer reads them
   as double.  p is changed as the reference changes it before emptying its
   vector (I, r, active, e).  exact = 0: the reference's arithmetic into pic
   (float); exact = 1: exact exp and double sums into pic64.  stats (may be
   NULL): particles used, particles on the level grids, spheres around the
   camera, levels, covered (pixel, particle) pairs.  Returns -1 when !a_eq_e,
   -2 for a dome with xres != yres. */
typedef struct {
  int dome;          /* "dome" (false) */
  double fov;        /* "fov" (45) */
  double minrad_pix; /* "minrad_pix" (1) */
} spo_rays_params;
int spo_render_rays(const spo_params *prm, const spo_rays_params *rp, spo_particle *p,
                    int64_t n, int exact, float *pic, double *pic64, int64_t *stats);

#ifdef __cplusplus
}
#endif
#endif
