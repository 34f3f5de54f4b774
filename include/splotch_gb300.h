/*
 * splotch_gb300.h -- C ABI of the GB300 particle renderer (libsplgpu.so).
 *
 * Drop-in boundary for Splotch's host renderer.  The C++ shim in
 * splotch_gb300/shim/ implements
 *     void host_rendering(paramfile&, std::vector<particle_sim>&, render_context&)
 * (splotch/splotch_host.h:43, defined at splotch/splotch_host.cc:711) on top
 * of these entry points; ctypes / cgo-style callers bind them directly.
 *
 * Conventions: every entry point returns spl_status (0 = success), never
 * throws and never traps the GPU; on failure spl_last_error_string() holds a
 * one-line reason.  Plain pointers and sizes only.  Images are x-major like
 * the reference's arr2<COLOUR> (cxxsupport/arr.h:429): pixel (x,y) channel c
 * lives at pic[(x*yres + y)*3 + c].
 */
#ifndef SPLOTCH_GB300_H
#define SPLOTCH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPL_MAX_TYPES 8

typedef int spl_status;
enum {
  SPL_OK = 0,
  SPL_ERR_INVALID = 1,     /* bad argument (planck_fail in the reference) */
  SPL_ERR_CUDA = 2,        /* CUDA runtime error */
  SPL_ERR_ALLOC = 3,       /* device or pinned allocation failed */
  SPL_ERR_CAPACITY = 4,    /* a fixed-capacity buffer overflowed */
  SPL_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
  SPL_ERR_UNSUPPORTED = 6, /* option not implemented on this path */
  SPL_ERR_INTERNAL = 7     /* an internal consistency check failed */
};

/* Memory space of a caller buffer. */
enum { SPL_MEM_HOST = 0, SPL_MEM_DEVICE = 1 };
/* Particle layout: AoS = particle_sim records (splotch/splotchutils.h:52-72,
   36-byte stride); SoA = one array per field. */
enum { SPL_LAYOUT_AOS = 0, SPL_LAYOUT_SOA = 1 };
/* What spl_render writes back into an AoS input.  FULL reproduces the
   reference's in-place side effects (projected x,y,z,r,I, colourised e,
   active, z-sorted order when a_eq_e is false); NONE leaves it untouched. */
enum { SPL_WRITEBACK_NONE = 0, SPL_WRITEBACK_FULL = 1 };
/* Compositing order for the ordered (a_eq_e=false) splat.  BACK_TO_FRONT
   applies particles in list order exactly like render_new; FRONT_TO_BACK
   (the default) evaluates the same sum, term for term, in reverse and stops
   a pixel once every channel's transmittance is below spl_frame_desc.
   ftb_epsilon (1e-9: what lies behind then adds less than 1e-9 of its colour)
   or below ftb_relative (1e-5) times the colour the channel has composited
   (what lies behind then adds at most 1e-5 of the pixel).  Both orders are
   within 1e-4 of the FP64 oracle; front-to-back skips the opaque depths of
   dense tiles, which back-to-front must walk in full. */
enum { SPL_ORDER_BACK_TO_FRONT = 0, SPL_ORDER_FRONT_TO_BACK = 1 };

typedef struct spl_context spl_context;

/* Camera quantities of particle_project's set-up (splotch_host.cc:62-110),
   computed on the host bit-for-bit like the reference. */
typedef struct {
  float mat[12]; /* TRANSFORM matrix in TRANSMAT::p order */
  float res2, ycorr, fovfct, xfac;
  double xshift, yshift;
} spl_camera;

/* Everything host_rendering() reads from the paramfile and render_context.
   Fill with spl_frame_desc_defaults() (the reference defaults), then set. */
typedef struct {
  int xres, yres;           /* "xres" (800), "yres" (=xres) */
  float fov;                /* "fov" (45), degrees */
  float zmin, zmax;         /* "zmin" (0), "zmax" (1e23) */
  float minrad_pix;         /* "minrad_pix" (1) */
  int projection;           /* "projection" (true) */
  int ptypes;               /* "ptypes" (1) */
  float smooth_factor[SPL_MAX_TYPES];  /* "smooth_factor{t}" (1) */
  float brightness[SPL_MAX_TYPES];     /* "brightness{t}" (1) */
  int color_is_vector[SPL_MAX_TYPES];  /* "color_is_vector{t}" (false) */
  float b_brightness;       /* render_context::b_brightness */
  int pal_n[SPL_MAX_TYPES];            /* palette of type t (rc.amap[t]) */
  const double *pal_x[SPL_MAX_TYPES];  /* host: n knot positions, ascending */
  const float *pal_rgb[SPL_MAX_TYPES]; /* host: 3n floats, r,g,b per knot */
  int a_eq_e;               /* "a_eq_e" (true) */
  float gray_absorption;    /* "gray_absorption" (0.2) */
  int sort_type;            /* "sort_type" (1) */
  int tile_size;            /* "tile_size_cpu" (50); 1..64 on the GPU */
  double campos[3], lookat[3], sky[3], centerpos[3]; /* render_context */
  /* GPU-only knobs (no reference counterpart) */
  int order_mode;           /* SPL_ORDER_* (default FRONT_TO_BACK) */
  float ftb_epsilon;        /* transmittance cut for FRONT_TO_BACK (1e-9) */
  int splat_config;         /* splat launch configuration, -1 = default for the
                               tile size (see spl_splat_config_valid) */
  float ftb_relative;       /* FRONT_TO_BACK also stops a pixel once each channel's
                               transmittance is below ftb_relative times the colour
                               it has composited (1e-5): all that lies behind adds
                               at most that fraction of the pixel (q <= 1).  Frames
                               kept for spl_render_backward stop the same way; the
                               backward differentiates what they composited. */
} spl_frame_desc;

/* Particle input.  AoS: aos points at n particle_sim records.  SoA: x..I,
   cr/cg/cb (e.r/e.g/e.b) are float arrays; type may be NULL (all type 0).
   Any alignment of the element type works; x, y, z, r 16-byte aligned and type
   8-byte aligned (as allocations are) let the activity pass read four
   particles per 16-byte load. */
typedef struct {
  int64_t n;
  int layout;   /* SPL_LAYOUT_* */
  int memspace; /* SPL_MEM_* */
  void *aos;
  const float *x, *y, *z, *r, *I, *cr, *cg, *cb;
  const uint16_t *type;
} spl_particles;

typedef struct {
  float *pic;   /* x-major xres*yres*3 floats */
  int memspace; /* SPL_MEM_* */
} spl_image;

/* Per-stage device times of the last spl_render call (CUDA events). */
typedef struct {
  float h2d_ms, project_ms, sort_ms, bin_ms, splat_ms, d2h_ms, total_ms;
  int64_t n_active;
  int64_t n_entries;   /* (particle, tile) bin entries */
  int64_t n_tiles;
  int kernel_launches; /* kernels launched by the call */
  int64_t n_fallback;  /* particles projected through the exact FP64 fallback */
  int64_t n_wide;      /* particles binned by the wide (many-tile) path */
  /* last spl_render_backward: adjoint splat, chain rule, whole call */
  float bwd_splat_ms, bwd_project_ms, bwd_total_ms;
} spl_stats;

/* ---- context ---------------------------------------------------------- */
spl_status spl_context_create(spl_context **ctx, int device);
spl_status spl_context_destroy(spl_context *ctx);
/* Bind the context to a CUDA stream (cudaStream_t as void*; NULL = legacy). */
spl_status spl_context_set_stream(spl_context *ctx, void *stream);
const char *spl_last_error_string(void);
const char *spl_version(void);

/* ---- frame set-up ----------------------------------------------------- */
void spl_frame_desc_defaults(spl_frame_desc *d);
/* The camera set-up of particle_project (splotch/splotch_host.cc:62-110). */
spl_status spl_camera_setup(const spl_frame_desc *d, spl_camera *cam);

/* Splat launch configurations (threads per tile x pixels per lane); the
   autotuner picks one per (tile size, workload).  Returns the number of
   configurations / whether cfg can cover a tile_size x tile_size tile. */
int spl_splat_config_count(void);
int spl_splat_config_valid(int cfg, int tile_size);

/* ---- plain render: replaces host_rendering (splotch_host.cc:711-834) --- */
spl_status spl_render(spl_context *ctx, const spl_frame_desc *d,
                      const spl_particles *p, spl_image *out, int writeback);

/* Copy ahead the host particle arrays of a later spl_render on this context
   (no counterpart in the reference, whose frames are rendered one call at a
   time): the copy runs on a stream of its own while the current frame
   renders, and the spl_render whose view names the same host arrays and count
   waits for it instead of copying.  Up to two prefetches may be pending; they
   are consumed in order, and a render of other arrays drops them.  The host
   arrays must not change between the prefetch and that render; pinned memory
   lets the copy overlap.  Device-memory views need no copy (no-op). */
spl_status spl_prefetch(spl_context *ctx, const spl_particles *p);

/* Cut heavy tiles into list segments in later spl_render calls (no
   counterpart in the reference, whose tiles are dynamically scheduled CPU
   work items): one GPU block per segment instead of per tile, so that a few
   dense tiles do not keep most of the GPU idle; the segments' results are
   then folded per pixel in list order.  Each pixel's sums are then grouped by
   segment, which changes float rounding within the usual tolerance (the
   image stays deterministic), so a split frame is not bit-equal to the same
   frame of spl_batch_render.
     SPL_SPLIT_ADDITIVE (default): additive frames only.  Their segments add
       up exactly the work of the whole tile.
     SPL_SPLIT_ON: also front-to-back frames, whose tiles are cut only when
       their list is at least 8x the frame's mean; a segment behind the front
       one cannot stop early until the front one is opaque, so dense ordered
       frames may render slower.
     SPL_SPLIT_OFF: never.
   Ordered frames kept for spl_render_backward are never split. */
#define SPL_SPLIT_OFF 0
#define SPL_SPLIT_ON 1
#define SPL_SPLIT_ADDITIVE 2
spl_status spl_context_set_split_tiles(spl_context *ctx, int mode);
spl_status spl_get_stats(const spl_context *ctx, spl_stats *s);

/* ---- test hooks: state of the last spl_render (host destinations) ----- */
/* Projected + colourised particles in original order (particle_sim layout):
   the reference's particle_project + particle_colorize side effects. */
spl_status spl_debug_get_projected(spl_context *ctx, void *aos_out, int64_t n);
/* Visiting order of the active particles (particle indices, *n_out of them):
   ascending index when a_eq_e, else the stable sort order -- the order in
   which the reference's stably sorted array meets its active particles. */
spl_status spl_debug_get_order(spl_context *ctx, uint32_t *order_out, int64_t cap,
                               int64_t *n_out);
/* Tile bins: tile_start has ntiles+1 entries; entries hold particle indices. */
spl_status spl_debug_get_bins(spl_context *ctx, int64_t *tile_start_out,
                              int64_t ntiles_plus_one, uint32_t *entries_out,
                              int64_t cap);

/* Exact fragment count of the reference splat loop for the last frame: the
   number of (pixel, particle) pairs render_new visits (splotch_host.cc:601-622).
   The algorithmic work behind the splat's roofline figure. */
spl_status spl_debug_count_fragments(spl_context *ctx, int64_t *frags_out);

/* Debug options for later spl_render calls.  Bit 0: project through the
   exact FP64 arithmetic only (no float-float fast path); the two must agree
   bit for bit.  Bit 1: radix sorts in the reduce-then-scan form instead of
   onesweep (no inter-block waits); results are identical.  Bit 2 (failure
   test): the depth sort's first scatter pass never takes its first tile, so
   the next tile's look-back finds that status unpublished and gives up after
   a short bounded spin; spl_render then returns SPL_ERR_TIMEOUT before the
   invalid permutation is used, and the context stays usable.  Bit 4 (failure
   test): the first active particle's tile count is stored one short (when it
   covers 2 to 64 tiles), so bin emission finds one passing tile more than
   counted; it stores nothing outside the particle's slots and spl_render
   returns SPL_ERR_CAPACITY. */
#define SPL_DEBUG_EXACT_FP64 1
#define SPL_DEBUG_RADIX_REDUCE_SCAN 2
#define SPL_DEBUG_LOOKBACK_STALL 4
#define SPL_DEBUG_SHORT_COUNT 16
spl_status spl_debug_set_options(spl_context *ctx, int flags);

/* Failure test of device allocation (process-wide): the nth device buffer
   allocation the library makes from now on -- a spl_context growing a
   buffer, or a batch's buffers -- fails once with SPL_ERR_ALLOC without
   calling cudaMalloc; nth = 0 cancels.  The reference's analogue is the
   abort on a device allocation error (cuda/cuda_splotch.cc:105). */
spl_status spl_debug_fail_alloc(int64_t nth);

/* ---- ray-sphere render: host_rendering with new_renderer=true ---------- */
/* The second renderer behind host_rendering (splotch/splotch_host.cc:714-723
   -> host_rendering_new, splotch/new_renderer.cc:522-641): every particle is
   a sphere seen from campos, every pixel a ray that collects
   -e*exp(-sin^2(angle)/(r*h2sigma)^2) from the spheres it meets; additive
   only.  Keys of this renderer that spl_frame_desc does not hold, or holds
   at another precision (it reads fov and minrad_pix as double): */
typedef struct {
  int dome;          /* "dome" (false): fisheye projector; needs xres == yres */
  double fov;        /* "fov" (45), degrees */
  double minrad_pix; /* "minrad_pix" (1) */
} spl_rays_desc;
void spl_rays_desc_defaults(spl_rays_desc *r);
/* Reads from d: xres, yres, zmax, ptypes, brightness, color_is_vector,
   palettes, b_brightness, a_eq_e (must be true: SPL_ERR_INVALID otherwise, the
   reference's planck_assert) and campos, centerpos, lookat, sky.  out gets
   the x-major xres*yres*3 image.  The reference empties the particle vector
   afterwards (new_renderer.cc:584); the particle view is not written. */
spl_status spl_render_rays(spl_context *ctx, const spl_frame_desc *d, const spl_rays_desc *r,
                           const spl_particles *p, spl_image *out);

/* ---- gradients ---------------------------------------------------------- */
/* Per-particle gradient arrays (n floats each, by particle index, in
   memspace; NULL = not wanted) and the camera-position gradient.  Colour:
   for palette types d/d(colour value) lands in cr (cg, cb stay 0); for
   color_is_vector types cr, cg, cb get d/d(r, g, b).  x, y, z are world
   positions, r is the smoothing length (hsml) as read. */
typedef struct {
  int memspace; /* SPL_MEM_* */
  float *I, *cr, *cg, *cb, *x, *y, *z, *r;
  double campos[3]; /* out: d/dcampos (centerpos, lookat, sky held) */
} spl_grads;

/* No counterpart in the reference, which has no derivative of its renderer.
   Gradients of a scalar loss L with respect to the inputs of the last frame
   spl_render drew on ctx, given grad_pic = dL/dpic (the image's layout).
   Coverage, tile lists and order are held at the forward's decisions (their
   derivative is zero almost everywhere).  Needs that frame's inputs and, for
   a device image, its output unchanged, and a forward without writeback.
   Ordered absorption frames need spl_context_set_differentiable: the adjoint
   walks each pixel's composited fragments back to front from the optical
   depth and stop position the forward kept (no per-particle intermediates). */
spl_status spl_render_backward(spl_context *ctx, const spl_image *grad_pic, spl_grads *g);
/* Ordered (a_eq_e = false) frames can only be differentiated when they were
   rendered with this switch on: the forward then also keeps, per pixel, the
   optical depth it composited and where its front-to-back pass stopped
   (16 bytes per pixel, a few adds per fragment).  Off by default. */
spl_status spl_context_set_differentiable(spl_context *ctx, int enable);

/* ---- before host_rendering: particle normalisation --------------------- */
/* sceneMaker::particle_normalize (splotch/scenemaker.cc:40-296, host branch)
   on the device: per type, optional log10 of I (intensity_log{t}) and of the
   colour (color_log{t}) or asinh of the colour (color_asinh{t}); the ranges of
   size, intensity and colour; intensity_min/max{t} and color_min/max{t}
   overrides; then every I and colour mapped to [0,1] by Normalizer::
   normAndClamp.  The particles (AoS or SoA, host or device) change in place;
   log10f/log come from CUDA's math library (an ulp from the host's). */
typedef struct {
  int ptypes;
  int intensity_log[SPL_MAX_TYPES], color_log[SPL_MAX_TYPES];
  int color_asinh[SPL_MAX_TYPES], color_is_vector[SPL_MAX_TYPES];
  int has_intensity_min[SPL_MAX_TYPES], has_intensity_max[SPL_MAX_TYPES];
  int has_color_min[SPL_MAX_TYPES], has_color_max[SPL_MAX_TYPES];
  float intensity_min[SPL_MAX_TYPES], intensity_max[SPL_MAX_TYPES];
  float color_min[SPL_MAX_TYPES], color_max[SPL_MAX_TYPES];
} spl_normalize_desc;
typedef struct {
  /* range_*: colour range of the data (the range_min/max{t} keys the
     reference sets); clamp_*: the colour range applied (clamp_min/max{t}) */
  float range_min[SPL_MAX_TYPES], range_max[SPL_MAX_TYPES];
  float clamp_min[SPL_MAX_TYPES], clamp_max[SPL_MAX_TYPES];
  float intensity_min[SPL_MAX_TYPES], intensity_max[SPL_MAX_TYPES];
  float size_min[SPL_MAX_TYPES], size_max[SPL_MAX_TYPES];
} spl_normalize_result;
spl_status spl_particle_normalize(spl_context *ctx, const spl_normalize_desc *d,
                                  spl_particles *p, spl_normalize_result *res);

/* ---- after host_rendering: post-processing and image output ------------ */
/* What splotch/splotch.cc:272-323 does with the image once host_rendering has
   returned, on the device. */
typedef struct {
  int a_eq_e;        /* additive frame: pic = -expm1(pic) with exptable<float32>(-20) */
  double gamma;      /* colour_adjust (splotchutils.cc:230-250): pic_gamma (1) */
  double brightness; /* pic_brightness (0) */
  double contrast;   /* pic_contrast (1) */
  int colorbar;      /* add_colorbar (splotchutils.cc:35-58): colorbar (F) */
} spl_post_desc;
void spl_post_desc_defaults(spl_post_desc *p);
/* In place on an x-major image (host or device) of d->xres x d->yres; the
   colour bars use d's palettes and types. */
spl_status spl_postprocess(spl_context *ctx, const spl_frame_desc *d, const spl_post_desc *p,
                           spl_image *img);
/* LS_Image's file bytes (cxxsupport/ls_image.cc:178-314) for pictype 0 (TGA),
   2 (PPM) or 3 (run-length TGA): Colour8 conversion and the x-major to row
   transpose on the device.  *len = full length; at most cap bytes are stored
   (out may be NULL to query the length). */
spl_status spl_image_encode(spl_context *ctx, const spl_image *img, int xres, int yres,
                            int pictype, uint8_t *out, int64_t cap, int64_t *len);
/* The same bytes written to path (splotch.cc:299-323). */
spl_status spl_write_image(spl_context *ctx, const spl_image *img, int xres, int yres,
                           int pictype, const char *path);

/* ---- batched rendering ------------------------------------------------- */
/* No counterpart in the reference, which renders one frame per
   host_rendering call.  Many frames -- camera poses, resolutions, additive or
   ordered modes, particle sets of uneven size -- are rendered by one launch of
   a captured CUDA graph: projection of every frame, one stable depth sort and
   one tile binning over all frames' active particles, and persistent splat
   kernels that take (frame, tile) items from a work queue ordered
   longest-list-first across all frames.  Buffer sizes come from a measured
   plan (one plain render of every frame at create); a render whose counts
   outgrow the plan re-plans and renders again.  Each frame's image equals the
   image spl_render gives for that frame at the same tile size and launch
   configuration, bit for bit. */
typedef struct {
  int set;              /* index into the particle sets */
  spl_frame_desc desc;  /* the frame's keys; tile_size and splat_config are the batch's */
  float *pic;           /* device image, x-major xres*yres*3 floats */
} spl_batch_frame;

typedef struct {
  int tile_size;                /* 0: chosen by the autotuner among 8, 16, 32 */
  int splat_config_additive;    /* -1: chosen by the autotuner */
  int splat_config_absorption;  /* -1: chosen by the autotuner */
  float capacity_margin;        /* buffer headroom over the measured counts (1.1);
                                   below 1 forces a re-plan (test hook) */
  int use_graph;                /* 1: capture and replay a CUDA graph; 0: launch eagerly */
  int tune_cache;               /* 1 (default): the autotuner's choice is kept per batch
                                   shape for the life of the process, and a later batch
                                   of the same shape takes it without timing anything;
                                   0: always search */
} spl_batch_options;

typedef struct {
  int tile_size, splat_config_additive, splat_config_absorption;
  int graph;                    /* 1 when renders replay a captured graph */
  int64_t cap_active, cap_entries, total_tiles;
  int64_t n_active, n_entries;  /* last render */
  float render_ms;              /* last spl_batch_render, launch to completion */
  float tune_ms;                /* spl_batch_create's search: timed candidate tile sizes
                                   and launch configurations (0 when the choice came
                                   from the tuning cache) */
  int kernel_launches;          /* kernels per render */
  int replans;                  /* capacity re-plans so far */
  int tune_cached;              /* 1 when the choice came from the tuning cache */
  float plan_ms;                /* spl_batch_create's measured plan at the chosen tile
                                   size (one plain render of every frame) */
} spl_batch_info;

typedef struct spl_batch spl_batch;

void spl_batch_options_defaults(spl_batch_options *o);
/* Sets must be device-resident (AoS or SoA) and stay unchanged while the batch
   lives; frame palettes are copied at create.  The batch uses its own stream. */
spl_status spl_batch_create(spl_context *ctx, const spl_particles *sets, int nsets,
                            const spl_batch_frame *frames, int nframes,
                            const spl_batch_options *opt, spl_batch **out);
/* Render every frame into its image; returns once they are complete. */
spl_status spl_batch_render(spl_batch *b);
spl_status spl_batch_get_info(const spl_batch *b, spl_batch_info *info);
spl_status spl_batch_destroy(spl_batch *b);

/* ---- depth sort without allocation ------------------------------------ */
/* No counterpart in the reference, which sorts the particle array on the host
   with std::sort (splotch/splotch_host.cc:289-321).

   Stable LSD radix sort of n (key, value) uint32 pairs in device memory,
   ascending in the low key_bits bits of the key; equal keys keep their input
   order.  It is the sort spl_render applies to the active particles' depth
   keys, with all of its scratch in one fixed array inside the library, so the
   call allocates nothing: for callers that must not allocate device memory
   while they run (a render loop whose memory is all reserved up front, a
   process whose device memory belongs to another allocator, code under a
   fixed device-memory budget).  spl_render grows its buffers on demand and
   does not suit them.

   keys_in   device, 16-byte aligned, n keys
   vals_in   device, n values; NULL sorts the indices 0..n-1
   keys_out  device, 16-byte aligned, n entries
   vals_out  device, n entries; neither output overlaps the other or an input
   key_bits  1..32
   stream    cudaStream_t as void*, NULL = legacy default stream
   The call only enqueues work on the stream.  n > SPL_NOALLOC_MAX_PAIRS
   returns SPL_ERR_CAPACITY before anything is launched.  The scratch array
   (about 19 MB per device) is shared by all calls on a device: calls that may
   run at the same time, on different streams or host threads, race and
   corrupt each other's results; serialise them.  The first call on a device
   (n == 0 is enough) loads the library's device code there and checks the
   array's capacity; make it before any stream capture begins.  Every call
   looks up the array's address on the current device, so a
   cudaDeviceReset between calls is harmless.  A CUDA error already pending on
   the calling thread is reported (SPL_ERR_CUDA), not cleared, and nothing is
   launched. */
#define SPL_NOALLOC_MAX_PAIRS (1 << 21)
spl_status spl_sort_pairs_noalloc(const uint32_t *keys_in, const uint32_t *vals_in,
                                  uint32_t *keys_out, uint32_t *vals_out, int64_t n,
                                  int key_bits, void *stream);

#ifdef __cplusplus
}
#endif
#endif
