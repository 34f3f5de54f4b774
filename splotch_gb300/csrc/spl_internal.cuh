// spl_internal.cuh -- device helpers and launch interfaces shared by the
// kernels of libsplgpu.so (sm_103a).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define SPL_MAXT 8  // particle types (SPL_MAX_TYPES)

namespace spl {

// ---------------------------------------------------------------------------
// IEEE-exact scalar arithmetic.  The reference's projection, binning and
// coverage decisions are reproduced bit-for-bit only if no multiply-add is
// contracted: these intrinsics are never fused by nvcc.
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// int(float) of the reference: truncation toward zero.  cvt.rzi.s32.f32
// saturates out-of-range values and maps NaN to 0.
__device__ __forceinline__ int f2i(float v) { return __float2int_rz(v); }

// 2^x on the MUFU unit (hand-written PTX; relative error ~2^-22).
__device__ __forceinline__ float ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

constexpr float kLog2e = 1.4426950408889634f;

// expm1(x) for x <= 0 in float, branch-free: the Taylor polynomial of degree
// 4 for -0.05 < x (truncation below 5e-8 relative) where exp(x)-1 would
// cancel, and ex2(x*log2e)-1 elsewhere (relative error below 4e-6 there,
// from the ~2^-22.5 error of ex2.approx).
__device__ __forceinline__ float expm1_neg(float x) {
  float p = fmaf(x, 1.f / 24.f, 1.f / 6.f);
  p = fmaf(p, x, 0.5f);
  p = fmaf(p, x, 1.f);
  p *= x;
  const float e = ex2(x * kLog2e) - 1.f;
  return x > -0.05f ? p : e;
}

// ---------------------------------------------------------------------------
// Packed float pairs: two FP32 values in one 64-bit register pair, operated on
// by the .f32x2 forms of add/sub/mul/fma (sm_100 and later).  Each lane of a
// pair is rounded exactly as the scalar instruction would round it, so a
// packed computation gives the scalar computation's bits; it takes half the
// issue slots.
struct F2 {
  unsigned long long v;
};

__device__ __forceinline__ F2 f2(float lo, float hi) {
  F2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ F2 f2(float x) { return f2(x, x); }
__device__ __forceinline__ float f2lo(F2 a) {
  float lo;
  asm("{\n .reg .f32 t;\n mov.b64 {%0, t}, %1;\n}" : "=f"(lo) : "l"(a.v));
  return lo;
}
__device__ __forceinline__ float f2hi(F2 a) {
  float hi;
  asm("{\n .reg .f32 t;\n mov.b64 {t, %0}, %1;\n}" : "=f"(hi) : "l"(a.v));
  return hi;
}
__device__ __forceinline__ F2 add2(F2 a, F2 b) {
  F2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 sub2(F2 a, F2 b) {
  F2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 mul2(F2 a, F2 b) {
  F2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
  F2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}

// expm1(-u) for u >= 0 on a pair, lane for lane the value of expm1_neg(-u):
// the same Taylor polynomial (its coefficients negated with u) below 0.05 and
// ex2(-u*log2e)-1 above.
// The Taylor form of expm1_neg2 alone (u < 0.05 in every component).
__device__ __forceinline__ F2 expm1_neg2_poly(F2 u) {
  F2 p = fma2(u, f2(1.f / 24.f), f2(-1.f / 6.f));
  p = fma2(p, u, f2(0.5f));
  p = fma2(p, u, f2(-1.f));
  return mul2(p, u);
}
constexpr float kExpm1TaylorCut = 0.05f;

__device__ __forceinline__ F2 expm1_neg2(F2 u) {
  F2 p = fma2(u, f2(1.f / 24.f), f2(-1.f / 6.f));
  p = fma2(p, u, f2(0.5f));
  p = fma2(p, u, f2(-1.f));
  p = mul2(p, u);
  const F2 a = mul2(u, f2(-kLog2e));
  const F2 t = add2(f2(ex2(f2lo(a)), ex2(f2hi(a))), f2(-1.f));
  return f2(f2lo(u) < 0.05f ? f2lo(p) : f2lo(t), f2hi(u) < 0.05f ? f2hi(p) : f2hi(t));
}

// ---------------------------------------------------------------------------
// Float-float ("double-float") arithmetic for reproducing double results.
// GB300's FP64 rate is a small fraction of its FP32 rate, so the reference's
// double-precision steps (transform, screen shift, palette interpolation) are
// evaluated in float-float with a rigorous error bound; when the bound cannot
// decide the final float rounding, the caller redoes the particle in FP64.
// Algorithms: TwoSum / Fast2Sum (Knuth, Dekker), TwoProd via FMA, and
// AccurateDWPlusDW (Joldes, Muller, Popescu, ACM TOMS 2017, relative error
// <= 3u^2 with u = 2^-24).
struct ff {
  float h, l;
};
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const ff s = two_sum(a.h, b.h);
  const ff t = two_sum(a.l, b.l);
  const ff v = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
  return fast_two_sum(v.h, __fadd_rn(t.l, v.l));
}
// a + b with an absolute error of at most 3u^2 (|a.h| + |b.h|) (u = 2^-24):
// TwoSum of the high parts, the low parts added in float, and a final TwoSum
// (exact, whatever the magnitudes).  No bound relative to the result under
// cancellation: callers bound the error by the operands' magnitudes.
__device__ __forceinline__ ff ff_add_abs(ff a, ff b) {
  const ff s = two_sum(a.h, b.h);
  const float w = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
  return two_sum(s.h, w);
}
// (a.h + a.l) * (b.h + b.l), relative error about 2^-45
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  ff p = two_prod(a.h, b.h);
  const float c = __fmaf_rn(a.h, b.l, __fmul_rn(a.l, b.h));
  return fast_two_sum(p.h, __fadd_rn(p.l, c));
}

// True when every real number within `delta` of v.h + v.l rounds to v.h in
// float round-to-nearest-even, i.e. the float result is decided.
__device__ __forceinline__ bool rn24_decided(ff v, float delta) {
  const uint32_t b = __float_as_uint(v.h) & 0x7fffffffu;
  const uint32_t E = b >> 23;
  if (E < 30u || E > 250u) return false;  // tiny, huge, inf or nan: no fast verdict
  const float ulp = __uint_as_float((E - 23u) << 23);
  const bool toward_zero = v.l != 0.f && ((__float_as_uint(v.l) ^ __float_as_uint(v.h)) >> 31);
  const float half = (toward_zero && (b & 0x7fffffu) == 0) ? 0.25f * ulp : 0.5f * ulp;
  return fabsf(v.l) + delta < half;
}

// Canonical radix keys: ascending unsigned order == ascending float order,
// with -0 == +0 (the comparators of splotch/splotchutils.h:74-96 treat them
// as equal, so the stable order keeps the original index order).
__device__ __forceinline__ uint32_t fkey_asc(float f) {
  uint32_t b = __float_as_uint(f);
  if ((b << 1) == 0) b = 0;  // -0 -> +0
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// ---------------------------------------------------------------------------
// Frame constants passed by value to the project kernel.
struct ProjConst {
  float mat[12];
  float res2, ycorr, fovfct, xfac;
  double xsum;  // (double)res2 + xshift                (splotch_host.cc:134)
  double ysum;  // ((double)res2 + yshift) + ycorr       (splotch_host.cc:135)
  ff xsum_ff, ysum_ff;  // the same as float-float pairs
  int exact_fp64;       // 1: skip the float-float fast path (test hook)
  uint32_t *n_fallback; // particles that took the FP64 path (may be null)
  // palette acceleration, per knot k: thr_gt[k] = least float > x[k];
  // x_ff[k] = x[k] as float-float; per segment k: inv_ff[k] = 1/(x[k+1]-x[k]);
  // per palette: lo_f = largest float <= x[0], hi_f = least float >= x[n-1]
  const float *pal_thr;
  const float2 *pal_xff;
  const float2 *pal_invff;
  float pal_lo_f[SPL_MAXT], pal_hi_f[SPL_MAXT];
  float zmin, zmax, minrad2, half_bfak;
  int xres, yres, projection, ptypes;
  float smooth[SPL_MAXT];
  float bright[SPL_MAXT];  // brightness{t} * b_brightness
  int colvec[SPL_MAXT];
  int pal_off[SPL_MAXT];   // knot offset of palette t in pal_x / pal_rgb
  int pal_n[SPL_MAXT];
  const double *pal_x;     // device
  const float *pal_rgb;    // device, 3 per knot
  // tiling of render_new (splotch_host.cc:337-343)
  int T, ncx, ncy;
  float rcell, cmid0;
  int sort_type;           // 0 = no key
  // per particle of the set, the palette colour of palette types (computed
  // once for frames sharing the set and its palettes), or null
  const float4 *pal_cache;
  // failure test (spl_debug_set_options): the first compact record's tile count
  // is stored one short when it is 2..64, so the emission finds a tile more
  int debug_short_count;
};

struct Tiling {
  int T, ncx, ncy;
  float rcell, cmid0;
};

// Circle-vs-tile test of render_new's binning (splotch_host.cc:367-386).
// Visits every passing tile id in reference loop order.
template <typename F>
__device__ __forceinline__ int for_each_tile(float x, float y, float r, const Tiling &g,
                                             F &&f) {
  const int T = g.T;
  const float rfacr = fmul(0.75f, r);
  int minx = max(0, f2i(fadd(fsub(x, rfacr), 1.f)) / T);
  int maxx = min(g.ncx - 1, f2i(fadd(x, rfacr)) / T);
  int miny = max(0, f2i(fadd(fsub(y, rfacr), 1.f)) / T);
  int maxy = min(g.ncy - 1, f2i(fadd(y, rfacr)) / T);
  const float rs = fadd(g.rcell, rfacr);
  const float sumsq = fmul(rs, rs);
  int cnt = 0;
  for (int ix = minx; ix <= maxx; ++ix) {
    const float cx = fadd(g.cmid0, (float)(ix * T));
    const float dx = fsub(x, cx);
    const float dx2 = fmul(dx, dx);
    for (int iy = miny; iy <= maxy; ++iy) {
      const float cy = fadd(g.cmid0, (float)(iy * T));
      const float dy = fsub(y, cy);
      if (fadd(dx2, fmul(dy, dy)) < sumsq) {
        f(iy * g.ncx + ix, cnt);
        ++cnt;
      }
    }
  }
  return cnt;
}

// The number of tiles for_each_tile visits, without visiting each one.  In a
// column the passing rows are one interval around the row nearest y (cy rises
// with iy, |dy| has one minimum, and every rounded step of the test is
// monotone), found by binary search with the same test; rectangles of up to 64
// cells are walked as for_each_tile walks them.
__device__ __forceinline__ int count_tiles(float x, float y, float r, const Tiling &g) {
  const int T = g.T;
  const float rfacr = fmul(0.75f, r);
  const int minx = max(0, f2i(fadd(fsub(x, rfacr), 1.f)) / T);
  const int maxx = min(g.ncx - 1, f2i(fadd(x, rfacr)) / T);
  const int miny = max(0, f2i(fadd(fsub(y, rfacr), 1.f)) / T);
  const int maxy = min(g.ncy - 1, f2i(fadd(y, rfacr)) / T);
  if (maxx < minx || maxy < miny) return 0;
  if ((maxx - minx + 1) * (maxy - miny + 1) <= 64) return for_each_tile(x, y, r, g, [](int, int) {});
  const float rs = fadd(g.rcell, rfacr);
  const float sumsq = fmul(rs, rs);
  auto dy2 = [&](int iy) {
    const float dy = fsub(y, fadd(g.cmid0, (float)(iy * T)));
    return fmul(dy, dy);
  };
  // the row nearest y: an estimate, then the smaller of its two candidates' dy^2
  const int t = (int)floorf((y - g.cmid0) / (float)T);
  const int ra = min(max(t, miny), maxy), rb = min(max(t + 1, miny), maxy);
  const int c0 = dy2(rb) < dy2(ra) ? rb : ra;
  const float d0 = dy2(c0);
  int cnt = 0;
  for (int ix = minx; ix <= maxx; ++ix) {
    const float dx = fsub(x, fadd(g.cmid0, (float)(ix * T)));
    const float dx2 = fmul(dx, dx);
    if (!(fadd(dx2, d0) < sumsq)) continue;
    int lo = miny, hi = c0;  // first passing row
    while (lo < hi) {
      const int m = (lo + hi) >> 1;
      if (fadd(dx2, dy2(m)) < sumsq) hi = m; else lo = m + 1;
    }
    const int first = lo;
    lo = c0;
    hi = maxy;  // last passing row
    while (lo < hi) {
      const int m = (lo + hi + 1) >> 1;
      if (fadd(dx2, dy2(m)) < sumsq) lo = m; else hi = m - 1;
    }
    cnt += lo - first + 1;
  }
  return cnt;
}

// ---------------------------------------------------------------------------
// Launch wrappers (defined in the .cu files).
struct ProjectOut {
  // full form, indexed by particle
  float4 *pos;      // x, y, r, z   (projected)
  float4 *col;      // e.r, e.g, e.b, I (colourised)
  uint8_t *active;
  uint32_t *count;  // tiles per particle (binning circle test), may be null
  uint32_t *key;    // sort key (when sort_type != 0), may be null
  // compact form, indexed by rank among active particles (ascending index)
  float4 *pos_c, *col_c;
  uint32_t *idx_c;    // particle index of each active particle
  uint32_t *count_c;
  uint32_t *key_c;    // may be null
  uint32_t cap_c;        // capacity of the compact arrays: records at or beyond
                         // it are dropped and bit 3 (8) of *err is set
  uint32_t *n_act;       // number of active particles
  uint32_t *flags;       // activity bits, (n+31)/32 words
  uint32_t *word_off;    // exclusive scan of the words' popcounts
  void *scan_scratch;    // scan_scratch_bytes((n+31)/32)
  uint32_t *err;    // device error word
};

struct SoAIn {
  const float *x, *y, *z, *r, *I, *cr, *cg, *cb;
  const uint16_t *type;
};

// aos non-null: particle_sim records; otherwise soa.  compact selects the
// active-only form (the render path) over the full form.
void launch_project(const void *aos, const SoAIn *soa, int64_t n, const ProjConst &c,
                    ProjectOut o, bool compact, cudaStream_t s, int *launches);
// Palette colour of each particle of a set (types with a palette) into out
// (n entries), for ProjConst::pal_cache of the frames that share the set.
void launch_palette_cache(const void *aos, const SoAIn *soa, int64_t n, const ProjConst &c,
                          float4 *out, cudaStream_t s);
// The two passes of the compact form on their own (the batch runs the
// popcount scan once over every frame's activity words): o.flags and
// o.word_off point at this frame's words, o.pos_c etc. at the arrays shared
// by all frames (records land at the scanned global positions).
void launch_project_flags(const void *aos, const SoAIn *soa, int64_t n, const ProjConst &c,
                          const ProjectOut &o, cudaStream_t s);
void launch_project_dense(const void *aos, const SoAIn *soa, int64_t n, const ProjConst &c,
                          const ProjectOut &o, cudaStream_t s);

// Both passes for many frames in one launch each: a device table of frames
// (ascending fblock0 / dblock0), each with its constants, inputs and outputs
// (flags / word_off at the frame's words; pos_c etc. at its record segment,
// cap_c that segment's capacity).  A flags block covers kFlagWordsPerBlock
// activity words, a dense block kDenseWordsPerBlock.
constexpr int kFlagWordsPerBlock = 8;
constexpr int kDenseWordsPerBlock = 64;
struct FrameProj {
  ProjConst c;
  const void *aos;  // particle_sim records, or null: soa
  SoAIn soa;
  int64_t n;
  ProjectOut o;
  uint32_t fblock0, dblock0;
};
void launch_project_flags_multi(const FrameProj *tab, int nf, uint32_t nblocks, cudaStream_t s);
void launch_project_dense_multi(const FrameProj *tab, int nf, uint32_t nblocks, cudaStream_t s);

// Exclusive scan of popcount(words[i]) into out (nwords entries); the total
// goes to *total.
void scan_popc(const uint32_t *words, int64_t nwords, uint32_t *out, uint32_t *total,
               void *scratch, cudaStream_t s, int *launches);
// AoS writeback (particle_sim records) in visiting order (perm may be null).
void launch_writeback_aos(const float4 *pos, const float4 *col, const uint8_t *active,
                          const void *type_src, int type_src_kind, const uint32_t *perm,
                          int64_t n, void *aos_out, cudaStream_t s);

// Radix sort of (key, value) pairs over bits [bit0, bit1); values == null on
// input means the identity 0..n-1.  Stable.  Scratch must hold
// radix_scratch_bytes(n).  Result lands in keys_out/vals_out (all four
// buffers distinct from keys_in/vals_in); sorted keys are written only when
// keys_needed.
size_t radix_scratch_bytes(int64_t n);
// onesweep: one histogram pass then one decoupled-look-back pass per digit
// (bounded waits; a wait that gives up sets bit 1 of *err); otherwise the
// reduce-then-scan form (no inter-block waits).
// stall_test (onesweep, a debug option of spl_render): the first scatter pass
// never takes tile 0, so tile 1's look-back finds its status unpublished and
// gives up after a short spin limit; every write stays in bounds, the
// permutation is invalid and bit 1 of *err is set.
int radix_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_tmp,
                     uint32_t *vals_tmp, uint32_t *keys_out, uint32_t *vals_out, int64_t n,
                     int bit0, int bit1, bool keys_needed, void *scratch, cudaStream_t s,
                     int *launches, uint32_t *err, bool onesweep, bool stall_test = false);

// Message returned by spl_last_error_string() on this host thread.
void set_last_error(const char *msg);

// The allocation failure test (spl_debug_fail_alloc): true when the device
// allocation about to be made is the one chosen to fail.
bool alloc_failure_due();

// Post-processing and output (spl_post.cu).  exptable_tables builds the two
// 1024-entry tables, expfac and taylorlimit of exptable<float32>(maxexp) on the
// host; launch_post applies -expm1 and/or colour_adjust to nfloats floats;
// launch_colorbar writes 10 rows ending at rows[k] (top) with colours[k]
// (xres rgb each); launch_encode writes Colour8 rows (row-major, BGR if bgr).
void exptable_tables(float maxexp, float *tab1, float *tab2, float *expfac,
                     float *taylorlimit);
void launch_post(float *pic, int64_t nfloats, bool do_expm1, bool do_adjust, float expfac,
                 float taylorlimit, const float *tab1, const float *tab2, double gamma,
                 double bright, double contrast, cudaStream_t s);
void launch_colorbar(float *pic, int xres, int yres, const float *colours, const int *rows,
                     int nbars, cudaStream_t s);
void launch_encode(const float *pic, int xres, int yres, bool bgr, uint8_t *out,
                   cudaStream_t s);

// particle_normalize (spl_normalize.cu).  Particles as particle_sim records
// (aos) or SoA arrays, in place.  stats: SPL_MAXT x 6 ints (per type: size,
// intensity, colour min/max as order-preserving ints), set by norm_stats_init
// before launch_norm_collect; norm_stat_value turns one back into a float.
struct NormConst {
  int ptypes;
  int intensity_log[SPL_MAXT], color_log[SPL_MAXT], color_asinh[SPL_MAXT];
  int color_is_vector[SPL_MAXT];
};
struct NormRanges {
  float imin[SPL_MAXT], imax[SPL_MAXT], cmin[SPL_MAXT], cmax[SPL_MAXT];
};
struct NormView {
  void *aos;
  float *I, *cr, *cg, *cb;
  const float *r;
  const uint16_t *type;
};
void norm_stats_init(int *h_stats);
float norm_stat_value(int i);
void launch_norm_collect(const NormView &v, int64_t n, const NormConst &c, int *stats,
                         uint32_t *err, cudaStream_t s);
void launch_norm_clamp(const NormView &v, int64_t n, const NormConst &c, const NormRanges &r,
                       cudaStream_t s);

// Exclusive scan of count[order[s]] (order may be null) into off (n+1 slots;
// off[n] = total).
size_t scan_scratch_bytes(int64_t n);
void scan_counts(const uint32_t *count, const uint32_t *order, int64_t n, uint64_t *off,
                 void *scratch, cudaStream_t s, int *launches);

// Bin emission and tile ranges.
// count[s] is the tile count of the s-th particle in visiting order (order[s]
// its index; order null = identity).  wide_list must hold n entries, wide_n
// one counter (particles with more than 64 tiles go to the warp-per-particle
// emitter through this list).
// out[i] = src[perm[i]]; with nsrc > 0, a perm value >= nsrc reads nothing,
// gives 0 and sets bit 1 of *err (a permutation left invalid by a look-back
// that gave up).
void launch_gather_u32(const uint32_t *src, const uint32_t *perm, int64_t n, uint32_t *out,
                       cudaStream_t s, int64_t nsrc = 0, uint32_t *err = nullptr);
void launch_emit(const float4 *pos, const uint32_t *count, const uint32_t *order,
                 const uint64_t *off, int64_t n, Tiling g, uint32_t *tkey, uint32_t *tval,
                 uint32_t *wide_list, uint32_t *wide_n, uint32_t *err, cudaStream_t s);
void launch_tile_ranges(const uint32_t *sorted_tkey, int64_t ne, int64_t ntiles,
                        uint32_t *tile_start, cudaStream_t s);
// 8-bit longest-first scheduling key per tile (sort ascending with
// radix_sort_pairs over bits [0,8) to get the launch order).
void launch_tile_cost(const uint32_t *tile_start, int64_t ntiles, uint32_t *key,
                      cudaStream_t s);

// Splat.
struct SplatArgs {
  const float4 *pos;
  const float4 *col;
  const uint32_t *entries;     // particle index per bin entry, tile-major
  const uint32_t *tile_start;  // ntiles+1
  const uint32_t *tile_order;  // launch order of the tiles (null: row order)
  int T, ncx, ncy, xres, yres;
  float gray;
  float h2sigma;
  int a_eq_e;
  int order_mode;
  float ftb_eps;
  float ftb_rel;               // relative transmittance cut (front-to-back)
  int config;                  // launch configuration (-1: default for T)
  float *pic;                  // device, x-major xres*yres*3
  // ordered frames kept for the adjoint (null: not kept): per pixel, x-major,
  // the optical depth sum(E*att) over the fragments composited (rgb) and, in
  // w (as uint bits), the tile-list position below which nothing was
  // composited (front-to-back early stop; 0 when the whole list was used)
  float4 *aux;
};
int launch_splat(const SplatArgs &a, cudaStream_t s);
// Heavy tiles cut into list segments of seg_len entries (additive and
// front-to-back frames without the adjoint's aux): seg_off (ntiles + 1, tile
// order) numbers the segments; partial holds two float4 per tile pixel for
// every segment of a split tile.  grid >= seg_off[ntiles].
struct SplatSegs {
  const uint64_t *seg_off;
  int64_t ntiles;
  uint32_t seg_len;
  float4 *partial;
  uint32_t *opaque;  // per tile (tile order), zero before the launch
};
int launch_splat_split(const SplatArgs &a, const SplatSegs &g, uint32_t grid, cudaStream_t s);
int splat_batch_size(const SplatArgs &a);  // list entries staged per batch
// Segments per tile of the forward split: ceil(len / seg_len), 1 for an empty
// tile (its segment writes the tile's zeros) or one shorter than split_min.
void launch_seg_count(const uint32_t *tile_start, int64_t ntiles, uint32_t seg_len,
                      uint32_t split_min, uint32_t *cnt, cudaStream_t s);
int splat_config_count();
bool splat_config_valid(int cfg, int T);
int splat_default_config(int T, bool additive);
void launch_count_fragments(const SplatArgs &a, unsigned long long *total, cudaStream_t s);

// Persistent splat over a (frame, tile) work queue: item i of this launch is
// global tile work[work_begin + i]; its frame f = frame_of_tile[tile] and its
// local tile = tile - tile_base[f]; frames[f] holds the frame's arguments with
// tile_start pointing at the frame's slice of the global tile ranges.  One
// launch configuration (cfg) and tile size T for every item of the launch.
struct BatchSplatArgs {
  const SplatArgs *frames;
  const uint32_t *tile_base;
  const uint32_t *frame_of_tile;
  const uint32_t *work;
  uint32_t work_begin, nwork;
  uint32_t *counter;  // zero before the launch
  int T;
  // the frames of the queue's items: 0 all additive, 1 all ordered
  // front-to-back, 2 any (the kernel chooses per item); a single-mode kernel
  // holds one splat form and fewer registers
  int mode;
};
int launch_splat_queue(const BatchSplatArgs &q, int cfg, cudaStream_t s);

// Adjoint of the splat: per active particle, sums of dL/dE (gcol.xyz) and of
// gatt*att*(dx, dy, dx^2+dy^2) (gpos.xyz), accumulated with atomics (zero them
// first).  f is the forward's argument set, f.pic its final image.
// The adjoint runs one CTA per segment of a tile's list, seg_len entries each:
// additive segments are independent (their per-particle sums do not depend on
// list order); an ordered segment after the first starts from state that a
// first pass computes for the segments behind it.  seg_cnt (ntiles) and
// seg_off (ntiles + 1) are scratch for the launch; scan_scratch holds
// scan_scratch_bytes(ntiles + 1) bytes.
struct AdjArgs {
  SplatArgs f;
  const float *gpic;  // dL/dpic, x-major
  float4 *gpos;
  float4 *gcol;
  int64_t n_entries;  // bin entries of the frame
  uint32_t *seg_cnt;
  uint64_t *seg_off;  // exclusive scan of segments per tile, in tile order
  void *scan_scratch;
  int64_t ntiles;     // set by the launch
  uint32_t seg_len;   // set by the launch
  // split ordered tiles: per segment and tile pixel (x*T + y) the pair
  // (U, V) of k_adj_ordered_state; seg_state_cap float4 entries available
  float4 *seg_state;
  size_t seg_state_cap;
};
// The list-segment length the adjoint uses for frame f with n_entries bin
// entries (a multiple of the launch's batch size).
uint32_t adjoint_seg_len(const SplatArgs &f, int64_t n_entries);
int launch_splat_adjoint(const AdjArgs &a, cudaStream_t s);

// Chain rule from the splat sums to the inputs (written by particle index;
// inactive particles are not touched) and block sums for the camera
// position: cam_sums = sum d/d(xc, yc, zc), sum dL/dX, sum dL/dY (zero it).
struct ProjAdjArgs {
  ProjConst c;
  const void *aos;  // particle_sim records, or null: soa
  SoAIn soa;
  const float4 *pos_c;
  const uint32_t *idx_c;
  const float4 *gpos, *gcol;
  int64_t na;
  float h2sigma;
  float *gI, *gcr, *gcg, *gcb, *gx, *gy, *gz, *gr;
  double *cam_sums;
};
int launch_project_adjoint(const ProjAdjArgs &a, cudaStream_t s);

// ---------------------------------------------------------------------------
// Ray-sphere renderer: host_rendering_new (splotch/new_renderer.cc:522-641),
// which host_rendering selects with new_renderer=true.  Every particle is a
// sphere of angular radius r around the unit direction c from campos; a pixel
// ray d collects -e*exp(-sin^2(d,c)/(r*h2sigma)^2) from every sphere it meets.
// Particles go to a pyramid of pixel grids by angular radius; each grid is a
// tree of image regions (the reference's recursive subdivision) whose
// culling test (reduceList) decides which particles a leaf region lists.
constexpr int kRayMaxLevels = 16;
constexpr int kRayLeafWarps = 4;  // leaf regions per CTA, one warp each
constexpr int kRayWalkSlots = 8;   // leaves a particle's first walk keeps

// reduceList parameters of one region (new_renderer.cc:77-101, 164-213),
// computed on the host in double exactly as the reference computes them.
struct RayRegion {
  float nf[4][3];      // n rounded to float (screening)
  double n[4][3];      // plane: side normals; dome: n[0] = nx0, n[1] = nx1
  double cthetamin, cthetamax, thetamin, thetamax;  // dome
  int centered;        // dome
  int pad;
};
// One region of a level's tree as the walk reads it (64 bytes): the float
// test vectors and the links of a depth-first walk without a stack.
struct RayNode {
  float4 f[3];      // RayRegion::nf
  int first_child;  // -1 for a leaf
  int skip;         // the next node after this subtree in depth-first order (-1: none)
  int leaf;         // global leaf id, or -1
  int centered;     // dome: RayRegion::centered
};
struct RayLevel {
  int fact, xdim, ydim;
  int root;          // node of the whole grid (never tested: the reference
                     // skips reduceList for the whole image)
  int leaf0, nleaves;
  double minrad, maxrad;  // radius range (minrad, maxrad] of the level's particles
};
struct RayConst {
  int dome, nlev;      // level 0 is the coarsest grid
  double p0[3], dpx[3], dpy[3];    // PlaneProjector
  float p0f[3], dpxf[3], dpyf[3];  // the same rounded to float
  double zen[3], ex[3], ey[3], dp; // DomeProjector (zenith, x, y, 1/res)
  double campos[3], centerpos[3];
  float zmax;
  double half_bfak;    // 0.5*bfak
  double mr2pr2;       // minrad_pix^2 * pixrad^2
  double h2sigma;
  RayLevel lev[kRayMaxLevels];
  RayRegion screen;    // reduceList(0, xres, 0, yres): the screen cut
};
// Per particle: key = code << kRayCodeShift | a Morton code of c (27 bits),
// code = level (0..nlev-1), nlev for a sphere around the camera (r > 1),
// nlev+1 for a particle not rendered.  Sorting by key groups the particles
// by level and, within a level, by direction: neighbouring threads of the
// walk then follow neighbouring paths, and a leaf's list is close in memory.
constexpr int kRayCodeShift = 27;
struct RayParts {
  double4_16a *rc;  // unit direction c and angular radius r, as the reference has them
  float4 *cf;      // the same rounded to float
  float4 *clo;     // c - cf (float), the low parts of c as a float-float pair
  float4 *pod;     // colour after the radius correction
  float2 *cov;     // per sphere: chord^2 limit 2r^2/(1+sqrt(1-r^2)) (-1: always decide in
                   // double), 1/(r*h2sigma)^2
  uint32_t *key;
  uint32_t *err;   // bit 0: type outside [0, ptypes); bit 5: two levels claim a particle
};
void launch_rays_prep(const void *aos, const SoAIn *soa, int64_t n, const ProjConst &pc,
                      const RayConst &k, const RayParts &o, cudaStream_t s);
// Level ranges of the sorted keys (lev_start: nlev + 3 entries) and the
// records of every rendered particle gathered into key order (dst indexed
// by sorted position).
void launch_rays_sorted(const uint32_t *key_s, const uint32_t *order, int64_t n, int nlev,
                        uint32_t *lev_start, const RayParts &src, const RayParts &dst,
                        cudaStream_t s);
// Walk of every particle of the level grids (key_s: the sorted keys, p: the
// records in that order, n entries) through its level's region tree.  Count pass (emit
// false): leaves reached per sorted position into count, the first
// kRayWalkSlots of them into slots (n * kRayWalkSlots).  Emit pass: (leaf id,
// particle) pairs at off[s], copied from the slots, or walked again for a
// particle that reached more leaves.
void launch_rays_walk(bool emit, const RayConst &k, const RayNode *nodes, const RayRegion *regs,
                      const uint32_t *key_s, int64_t n, const RayParts &p, uint32_t *count,
                      uint32_t *slots, const uint64_t *off, uint32_t *keys, uint32_t *vals,
                      cudaStream_t s);
// One pyramid level: every leaf region of level L (leaf ranges in leaf_start,
// entries' particles in vals).  A leaf's list is cut into segments of
// kRaySegLen entries, one warp each (seg_off: exclusive scan of the segments
// per leaf, item_leaf: the leaf of each segment); a leaf of one segment is
// finished by its warp, the segments of a longer one leave partial sums that
// a second kernel folds in segment order.  Finishing adds the spheres around
// the camera (order[lev_start[nlev] .. lev_start[nlev+1]]) on the coarsest
// level, the coarser level's grid (coarse, cdim_y rows per column) upsampled
// on the others.  out: x-major xdim*ydim*3.
constexpr uint32_t kRaySegLen = 256;
constexpr int kRayLeafPixels = 81;  // a leaf region holds at most 9 x 9 pixels
struct RayLeafArgs {
  const RayConst *kd;        // the frame's constants in device memory
  const ushort4 *leaf_box;   // x0, x1, y0, y1 in level pixels
  const uint32_t *leaf_start;
  const uint64_t *seg_off;   // nleaves + 1
  const uint32_t *item_leaf;
  const uint32_t *vals;      // sorted positions of the entries' particles
  const uint32_t *lev_start; // code ranges in the sorted order (nlev + 3)
  float *partial;            // per segment item, kRayLeafPixels * 3 floats
  const float *coarse;
  int cdim_y;
  float *out;
};
// Segments per leaf (every leaf, at least one) and the item -> leaf table.
void launch_rays_segments(const uint32_t *leaf_start, int64_t nleaves, uint32_t *cnt,
                          cudaStream_t s);
void launch_rays_items(const uint64_t *seg_off, int64_t nleaves, uint32_t *item_leaf,
                       cudaStream_t s);
void launch_rays_leaves(const RayConst &k, int L, const RayParts &p, const RayLeafArgs &a,
                        cudaStream_t s);
// The dome's post step (new_renderer.cc:619-639): pixels outside the fisheye
// circle are zeroed, in the reference's row order.  jstop: res/2 + 1 ints.
void launch_rays_dome_mask(float *pic, int res, int *jstop, cudaStream_t s);

}  // namespace spl
