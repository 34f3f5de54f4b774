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

#ifdef __cplusplus
}
#endif
#endif
