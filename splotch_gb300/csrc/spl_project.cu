// spl_project.cu -- fused camera transform, perspective projection,
// hsml->pixel radius, palette colourisation, tile-count and sort-key
// generation (particle_project + particle_colorize of
// splotch/splotch_host.cc:58-287, plus the counting half of render_new's
// binning, splotch_host.cc:356-387).
//
// Arithmetic follows the reference operation by operation: the transform and
// the screen shift in double (vec3 is double, cxxsupport/vec3.h:143; xshift is
// double, splotch_host.cc:103), everything else in float, with no contracted
// multiply-adds.  The outputs x, y, z, r, I and active are therefore
// bit-identical to the reference's.
#include "spl_internal.cuh"
#include "spl_rays.cuh"

namespace spl {

namespace {

struct PIn {
  float er, eg, eb, x, y, z, r, I;
  int type;
};

// ---- exact FP64 forms (the reference's arithmetic; fallback and test path) ----

// TRANSFORM::TransPoint (kernel/transform.cxx:212-219) in double.
__device__ __forceinline__ float transpoint_fp64(const float *m, float x, float y, float z) {
  const double vx = x, vy = y, vz = z;
  return __double2float_rn(
      dadd(dadd(dadd(dmul(vx, m[0]), dmul(vy, m[1])), dmul(vz, m[2])), (double)m[3]));
}

// ---- float-float fast forms ----------------------------------------------------

// One row of the transform; false when the float rounding is undecided.
__device__ __forceinline__ bool transpoint_fast(const float *m, float x, float y, float z,
                                                float &out) {
  const ff a = two_prod(x, m[0]), b = two_prod(y, m[1]), c = two_prod(z, m[2]);
  if (a.l == 0.f && b.l == 0.f && c.l == 0.f) {
    // Products and the first two partial sums exact in float (axis-aligned
    // cameras): the double sum is then exactly representable up to the last
    // add, whose single rounding to float -- ties included -- is one float add.
    const ff t1 = two_sum(a.h, b.h);
    const ff t2 = two_sum(t1.h, c.h);
    if (t1.l == 0.f && t2.l == 0.f) {
      out = fadd(t2.h, m[3]);
      return true;
    }
  }
  const ff s1 = ff_add_abs(a, b);
  const ff s2 = ff_add_abs(s1, c);
  const ff s3 = ff_add_abs(s2, ff{m[3], 0.f});
  // reference rounding (2^-53 per double add, relative to each partial sum) +
  // float-float error (3*2^-48 per add, relative to its operands), with a
  // margin of at least 5
  const float delta = 0x1p-44f * (fabsf(a.h) + fabsf(b.h) + fabsf(c.h) + fabsf(m[3]) +
                                  fabsf(s1.h) + fabsf(s2.h) + fabsf(s3.h));
  out = s3.h;
  return rn24_decided(s3, delta);
}

// (float)(A + (double)p) for a double A given as float-float.
__device__ __forceinline__ bool shift_fast(ff A, float p, float &out) {
  if (A.l == 0.f) {
    // A is a float: A + p is exact in double unless p is far below A's last
    // bit, where it cannot move the float rounding; one float add is exact.
    out = fadd(A.h, p);
    return true;
  }
  const ff s = ff_add_abs(A, ff{p, 0.f});
  const float delta = 0x1p-44f * (fabsf(A.h) + fabsf(p) + fabsf(s.h));
  out = s.h;
  return s.h != 0.f && rn24_decided(s, delta);
}

// One channel of (1-frac)*y0 + frac*y1 with the reference's roundings:
// RN24(RN53(y0*RN53(1-frac))) + RN24(RN53(y1*frac)) in float.
__device__ __forceinline__ bool lerp_channel_fast(float y0, float y1, ff omf, ff frac,
                                                  float efrac, float &out) {
  float p0 = 0.f, p1 = 0.f;
  if (y0 != 0.f) {
    const ff P = ff_mul(ff{y0, 0.f}, omf);
    if (!rn24_decided(P, fabsf(y0) * efrac + 0x1p-42f * fabsf(P.h))) return false;
    p0 = P.h;
  }
  if (y1 != 0.f) {
    const ff P = ff_mul(ff{y1, 0.f}, frac);
    if (!rn24_decided(P, fabsf(y1) * efrac + 0x1p-42f * fabsf(P.h))) return false;
    p1 = P.h;
  }
  out = fadd(p0, p1);
  return true;
}

// linearMap<COLOUR>::getVal_const (cxxsupport/linear_map.h:71-84) with
// interpol_helper (cxxsupport/math_utils.h:186-196), float-float form.
// Knot comparisons use precomputed float thresholds, which is exact for a
// float argument; the interpolation is decided or reported undecided.
__device__ __forceinline__ bool palette_fast(const ProjConst &c, int t, float v, float &r,
                                             float &g, float &b) {
  const int n = c.pal_n[t];
  const int off = c.pal_off[t];
  const float *rgb = c.pal_rgb + 3 * off;
  int idx;
  if (n == 1 || v <= c.pal_lo_f[t]) {
    idx = 0;
  } else if (v >= c.pal_hi_f[t]) {
    idx = n - 1;
  } else {
    const float *thr = c.pal_thr + off;
    int lo = 0, hi = n;
    while (lo < hi) {  // lower_bound: first knot with !(x[k] < v)
      const int mid = (lo + hi) >> 1;
      if (v >= __ldg(thr + mid)) lo = mid + 1; else hi = mid;
    }
    idx = lo > 0 ? lo - 1 : 0;
    if (idx > n - 2) idx = n - 2;
    const float2 xk = __ldg(c.pal_xff + off + idx);
    const float2 ik = __ldg(c.pal_invff + off + idx);
    const ff num = ff_add(ff{v, 0.f}, ff{-xk.x, -xk.y});
    const ff frac = ff_mul(num, ff{ik.x, ik.y});
    const ff omf = ff_add(ff{1.f, 0.f}, ff{-frac.h, -frac.l});
    // |frac - reference frac|: float-float and double roundings of the
    // quotient plus the float-float representation error of x[k]
    const float efrac = 0x1p-43f * fabsf(frac.h) + 0x1p-46f * fabsf(xk.x) * fabsf(ik.x);
    const float *y0 = rgb + 3 * idx;
    return lerp_channel_fast(__ldg(y0), __ldg(y0 + 3), omf, frac, efrac, r) &&
           lerp_channel_fast(__ldg(y0 + 1), __ldg(y0 + 4), omf, frac, efrac, g) &&
           lerp_channel_fast(__ldg(y0 + 2), __ldg(y0 + 5), omf, frac, efrac, b);
  }
  r = __ldg(rgb + 3 * idx);
  g = __ldg(rgb + 3 * idx + 1);
  b = __ldg(rgb + 3 * idx + 2);
  return true;
}

// linearMap<COLOUR>::getVal_const (cxxsupport/linear_map.h:71-84) with
// interpol_helper (cxxsupport/math_utils.h:186-196), in double like the
// reference.
__device__ __forceinline__ void palette(const ProjConst &c, int t, float v, float &r,
                                       float &g, float &b) {
  const int n = c.pal_n[t];
  const double *x = c.pal_x + c.pal_off[t];
  const float *rgb = c.pal_rgb + 3 * c.pal_off[t];
  const double xv = (double)v;
  int idx;
  if (n == 1 || xv <= x[0]) {
    idx = 0;
  } else if (xv >= x[n - 1]) {
    idx = n - 1;
  } else {
    int lo = 0, hi = n;
    while (lo < hi) {  // lower_bound
      int mid = (lo + hi) >> 1;
      if (x[mid] < xv) lo = mid + 1; else hi = mid;
    }
    idx = lo > 0 ? lo - 1 : 0;
    if (idx > n - 2) idx = n - 2;
    const double frac = ddiv(dsub(xv, x[idx]), dsub(x[idx + 1], x[idx]));
    const double omf = dsub(1.0, frac);
    r = fadd(__double2float_rn(dmul((double)rgb[3 * idx], omf)),
             __double2float_rn(dmul((double)rgb[3 * idx + 3], frac)));
    g = fadd(__double2float_rn(dmul((double)rgb[3 * idx + 1], omf)),
             __double2float_rn(dmul((double)rgb[3 * idx + 4], frac)));
    b = fadd(__double2float_rn(dmul((double)rgb[3 * idx + 2], omf)),
             __double2float_rn(dmul((double)rgb[3 * idx + 5], frac)));
    return;
  }
  r = rgb[3 * idx];
  g = rgb[3 * idx + 1];
  b = rgb[3 * idx + 2];
}

struct POut {
  float4 pos, col;
  bool active;
  uint32_t count, key;
};

// Geometry of particle_project (splotch_host.cc:118-176): camera transform,
// z cut, perspective, radius and intensity scaling, footprint test.  Returns
// `active`; x,y,z,r,I hold what the reference leaves in the particle.
__device__ __forceinline__ bool project_geom(const ProjConst &c, const PIn &in, float &x,
                                             float &y, float &z, float &r, float &I,
                                             bool &fell_back, uint32_t *err) {
  const float *m = c.mat;
  const bool fast = !c.exact_fp64;
  // TRANSFORM::TransPoint (kernel/transform.cxx:212-219), double in the reference
  if (!(fast && transpoint_fast(m, in.x, in.y, in.z, x) &&
        transpoint_fast(m + 4, in.x, in.y, in.z, y) &&
        transpoint_fast(m + 8, in.x, in.y, in.z, z))) {
    fell_back = fast;
    x = transpoint_fp64(m, in.x, in.y, in.z);
    y = transpoint_fp64(m + 4, in.x, in.y, in.z);
    z = transpoint_fp64(m + 8, in.x, in.y, in.z);
  }
  r = in.r;
  I = in.I;
  const int t = in.type;
  if (t < 0 || t >= c.ptypes) {
    atomicOr(err, 1u);  // type outside [0, ptypes): planck_fail in spirit
    return false;
  }
  if (-z <= c.zmin || -z >= c.zmax) return false;
  float xfac2 = c.xfac;
  if (!c.projection) {
    x = fadd(c.res2, fmul(x, xfac2));
    y = fadd(fadd(c.res2, c.ycorr), fmul(y, xfac2));
  } else {
    xfac2 = fdiv(-c.res2, fmul(c.fovfct, z));
    const float px = fmul(x, xfac2), py = fmul(y, xfac2);
    // res2 + xshift + x*xfac2 in double, stored to float (splotch_host.cc:134-135)
    if (!(fast && shift_fast(c.xsum_ff, px, x) && shift_fast(c.ysum_ff, py, y))) {
      fell_back = fell_back || fast;
      x = __double2float_rn(dadd(c.xsum, (double)px));
      y = __double2float_rn(dadd(c.ysum, (double)py));
    }
  }
  I = fmul(I, fdiv(c.half_bfak, r));
  r = fmul(r, 2.f);
  r = fmul(r, fmul(xfac2, c.smooth[t]));
  const float rcorr = fdiv(fsqrt(fadd(fmul(r, r), c.minrad2)), r);
  r = fmul(r, rcorr);
  I = fdiv(I, rcorr);
  const float rfacr = fmul(0.75f, r);
  const int minx = f2i(fadd(fsub(x, rfacr), 1.f));
  const int maxx = f2i(fadd(fadd(x, rfacr), 1.f));
  const int miny = f2i(fadd(fsub(y, rfacr), 1.f));
  const int maxy = f2i(fadd(fadd(y, rfacr), 1.f));
  return !(minx >= c.xres) && !(maxx <= 0) && max(minx, 0) < min(maxx, c.xres) &&
         !(miny >= c.yres) && !(maxy <= 0) && max(miny, 0) < min(maxy, c.yres);
}

// linearMap colour of a palette particle (colour value v, type t): the
// float-float form, or the double form when it cannot decide a rounding.
__device__ __forceinline__ void palette_colour(const ProjConst &c, int t, float v, float &r,
                                               float &g, float &b, bool &fell_back) {
  const bool fast = !c.exact_fp64;
  if (fast && palette_fast(c, t, v, r, g, b)) return;
  fell_back = fell_back || fast;
  palette(c, t, v, r, g, b);
}

// i: the particle's index in its set (for the palette cache).
__device__ __forceinline__ POut project_core(const ProjConst &c, const PIn &in, int64_t i,
                                             uint32_t *err) {
  bool fell_back = false;
  float x, y, z, r, I;
  float er = in.er, eg = in.eg, eb = in.eb;
  const int t = in.type;
  const bool active = project_geom(c, in, x, y, z, r, I, fell_back, err);
  {
    if (active) {  // particle_colorize (splotch_host.cc:276-282)
      if (!c.colvec[t]) {
        if (c.pal_cache) {  // computed once for the particle set (batched frames)
          const float4 pc = __ldg(c.pal_cache + i);
          er = pc.x;
          eg = pc.y;
          eb = pc.z;
        } else {
          float pr, pg, pb;
          palette_colour(c, t, er, pr, pg, pb, fell_back);
          er = pr;
          eg = pg;
          eb = pb;
        }
      }
      const float fac = fmul(I, c.bright[t]);
      er = fmul(er, fac);
      eg = fmul(eg, fac);
      eb = fmul(eb, fac);
    }
  }
  if (c.n_fallback) {
    const uint32_t am = __activemask();
    const uint32_t fb = __ballot_sync(am, fell_back);
    if (fb && (int)(threadIdx.x & 31) == __ffs(am) - 1) atomicAdd(c.n_fallback, __popc(fb));
  }
  POut o;
  o.pos = make_float4(x, y, r, z);
  o.col = make_float4(er, eg, eb, I);
  o.active = active;
  o.count = 0;
  if (active) {
    Tiling g{c.T, c.ncx, c.ncy, c.rcell, c.cmid0};
    o.count = (uint32_t)count_tiles(x, y, r, g);
  }
  switch (c.sort_type) {
    case 1: o.key = fkey_asc(z); break;    // zcmp: z ascending
    case 2: o.key = ~fkey_asc(er); break;  // vcmp1: e.r descending
    case 3: o.key = fkey_asc(er); break;   // vcmp2: e.r ascending
    case 4: o.key = ~fkey_asc(r); break;   // hcmp: r descending
    default: o.key = 0u; break;
  }
  return o;
}

struct LoadAoS {
  const uint8_t *aos;
  __device__ __forceinline__ PIn operator()(int64_t i) const {
    const float *f = reinterpret_cast<const float *>(aos + i * 36);
    PIn in;
    in.er = __ldg(f + 0); in.eg = __ldg(f + 1); in.eb = __ldg(f + 2);
    in.x = __ldg(f + 3); in.y = __ldg(f + 4); in.z = __ldg(f + 5);
    in.r = __ldg(f + 6); in.I = __ldg(f + 7);
    in.type = __ldg(reinterpret_cast<const unsigned short *>(aos + i * 36 + 32));
    return in;
  }
};

struct LoadSoA {
  const float *x, *y, *z, *r, *I, *cr, *cg, *cb;
  const uint16_t *type;
  __device__ __forceinline__ PIn operator()(int64_t i) const {
    PIn in;
    in.x = __ldg(x + i); in.y = __ldg(y + i); in.z = __ldg(z + i);
    in.r = __ldg(r + i); in.I = __ldg(I + i);
    in.er = __ldg(cr + i);
    in.eg = cg ? __ldg(cg + i) : 0.f;
    in.eb = cb ? __ldg(cb + i) : 0.f;
    in.type = type ? (int)__ldg(type + i) : 0;
    return in;
  }
};

// Every particle's projected state, indexed by particle (writeback, test hooks,
// and the full-array depth sort that the reference's in-place sort implies).
template <class L>
__global__ void __launch_bounds__(256) k_project_full(L load, int64_t n, ProjConst c,
                                                      ProjectOut o) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const POut p = project_core(c, load(i), i, o.err);
    o.pos[i] = p.pos;
    o.col[i] = p.col;
    o.active[i] = p.active ? 1 : 0;
    if (o.count) o.count[i] = p.count;
    if (o.key) o.key[i] = p.key;
  }
}

// Active particles only, compacted in ascending particle order, in three
// deterministic kernels (no inter-block waits):
//   k_project_flags  : activity of every particle, one bit each, 32 per word
//   (scan)           : exclusive scan of the words' population counts
//   k_project_dense  : each block expands its words into a dense list of
//                      active particles, projects and colourises them with
//                      all lanes busy, and writes the compact records
// A float screen of project_geom's activity decision (perspective frames):
// 1 when the particle is active and 0 when it is inactive whatever the
// roundings of the exact computation, -1 when it cannot decide (near a z
// plane or an image edge; a NaN, infinite or non-positive radius; a type
// outside [0, ptypes); orthographic or exact-FP64 frames), which leaves the
// particle to project_geom.  The camera transform is evaluated with fused
// multiply-adds, within 2^-20 of a bound on its terms' magnitude (the row's
// absolute sum times max(|x|, |y|, |z|), plus the translation); the
// projection factor's relative error is then below ek = ez/(nz - ez) + 2^-18
// (the factor and ek use the fast division, within 2 ulp), and screen
// position and radius are within (4 ek + 2^-16) of their magnitudes plus
// 2^-6 pixel, bounds far above the float errors of both computations.  The
// footprint test holds, or fails, for every value inside those bounds.
__device__ __forceinline__ int screen_activity(const ProjConst &c, const PIn &in) {
  if (c.exact_fp64 || !c.projection) return -1;
  const int t = in.type;
  if (t < 0 || t >= c.ptypes) return -1;
  const float *m = c.mat;
  const float am = fmaxf(fmaxf(fabsf(in.x), fabsf(in.y)), fabsf(in.z));
  const float zf = fmaf(m[10], in.z, fmaf(m[9], in.y, fmaf(m[8], in.x, m[11])));
  const float ez =
      0x1p-20f * fmaf(fabsf(m[8]) + fabsf(m[9]) + fabsf(m[10]), am, fabsf(m[11]));
  const float nz = -zf;  // the z cut keeps zmin < -z < zmax
  if (nz + ez <= c.zmin || nz - ez >= c.zmax) return 0;
  // (the fast division's bound holds for denominators in [2^-126, 2^126])
  if (!(nz - ez > c.zmin && nz - ez > 1e-30f && nz + ez < c.zmax && nz + ez < 1e30f))
    return -1;
  const float den = c.fovfct * nz;
  if (!(den > 1e-30f && den < 1e30f)) return -1;
  const float xc = fmaf(m[2], in.z, fmaf(m[1], in.y, fmaf(m[0], in.x, m[3])));
  const float yc = fmaf(m[6], in.z, fmaf(m[5], in.y, fmaf(m[4], in.x, m[7])));
  const float sx = fmaf(fabsf(m[0]) + fabsf(m[1]) + fabsf(m[2]), am, fabsf(m[3]));
  const float sy = fmaf(fabsf(m[4]) + fabsf(m[5]) + fabsf(m[6]), am, fabsf(m[7]));
  const float k = __fdividef(c.res2, den);                // the projection factor xfac2
  const float ek = __fdividef(ez, nz - ez) + 0x1p-18f;  // its relative error, with margin
  const float xs = (float)c.xsum, ys = (float)c.ysum;
  const float X = xs + xc * k, Y = ys + yc * k;
  const float r2 = 2.f * in.r * k * c.smooth[t];
  const float R = sqrtf(r2 * r2 + c.minrad2);  // the radius after the minrad correction
  const float e = 4.f * ek + 0x1p-16f;
  const float mX = (fabsf(xs) + fabsf(xc * k) + R) * e + sx * k * 0x1p-19f + 0x1p-6f;
  const float mY = (fabsf(ys) + fabsf(yc * k) + R) * e + sy * k * 0x1p-19f + 0x1p-6f;
  const float ext = 0.75f * R;
  if (!(fabsf(X) < 1e30f && fabsf(Y) < 1e30f && mX < 1e30f && mY < 1e30f && ext < 1e30f))
    return -1;
  // maxx <= 0 needs x + 0.75r + 1 < 1; minx >= xres needs x - 0.75r + 1 >= xres
  if (X + ext + mX < 0.f || X - ext - mX + 1.f >= (float)c.xres || Y + ext + mY < 0.f ||
      Y - ext - mY + 1.f >= (float)c.yres)
    return 0;
  if (!(in.r > 1e-30f && in.r < 1e30f && r2 > 1e-20f && c.smooth[t] > 0.f)) return -1;
  // active: max(int(x - 0.75r + 1), 0) < min(int(x + 0.75r + 1), xres), and in y
  const float ax = fmaxf(floorf(X - ext + 1.f + mX), 0.f);
  const float bx = fminf(floorf(X + ext + 1.f - mX), (float)c.xres);
  const float ay = fmaxf(floorf(Y - ext + 1.f + mY), 0.f);
  const float by = fminf(floorf(Y + ext + 1.f - mY), (float)c.yres);
  return (ax < bx && ay < by) ? 1 : -1;
}

// One warp: the activity bits of word w (particles 32w .. 32w+31).  The float
// screen decides nearly every particle; the few it cannot go through
// project_geom.
template <class L>
__device__ __forceinline__ void flags_word(const L &load, int64_t n, const ProjConst &c,
                                           uint32_t *__restrict__ flags, uint32_t *err,
                                           int64_t w, int lane) {
  const int64_t i = w * 32 + lane;
  int dec = 0;
  PIn in{};
  if (i < n) {
    in = load(i);
    dec = screen_activity(c, in);
  }
  bool active = dec == 1;
  if (__any_sync(0xffffffffu, dec < 0) && dec < 0) {
    float x, y, z, r, I;
    bool fb = false;
    active = project_geom(c, in, x, y, z, r, I, fb, err);
  }
  const uint32_t bits = __ballot_sync(0xffffffffu, active);
  if (lane == 0) flags[w] = bits;
}

template <class L>
__global__ void __launch_bounds__(256, 5) k_project_flags(L load, int64_t n, ProjConst c,
                                                       uint32_t *__restrict__ flags,
                                                       uint32_t *err) {
  const int lane = threadIdx.x & 31;
  const int64_t nwords = (n + 31) / 32;
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < nwords;
       w += ((int64_t)gridDim.x * blockDim.x) >> 5)
    flags_word(load, n, c, flags, err, w, lane);
}

// SoA activity flags, four particles per lane: a warp step takes 128
// particles (four flag words) with 16-byte loads of x, y, z, r and an 8-byte
// load of the types, so each warp keeps four times the bytes in flight of the
// one-particle-per-lane form (which the latency of its loads bounded, not its
// arithmetic).  Needs x, y, z, r 16-byte and type 8-byte aligned.
__global__ void __launch_bounds__(256) k_project_flags_soa4(SoAIn soa, int64_t n, ProjConst c,
                                                            uint32_t *__restrict__ flags,
                                                            uint32_t *err) {
  const int lane = threadIdx.x & 31;
  const int64_t nwords = (n + 31) / 32;
  const int64_t nsteps = (n + 127) / 128;
  for (int64_t st = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; st < nsteps;
       st += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t i0 = st * 128 + lane * 4;
    float xs[4], ys[4], zs[4], rs[4];
    int ts[4] = {0, 0, 0, 0};
    if (i0 + 4 <= n) {
      const float4 X = __ldg(reinterpret_cast<const float4 *>(soa.x + i0));
      const float4 Y = __ldg(reinterpret_cast<const float4 *>(soa.y + i0));
      const float4 Z = __ldg(reinterpret_cast<const float4 *>(soa.z + i0));
      const float4 R = __ldg(reinterpret_cast<const float4 *>(soa.r + i0));
      xs[0] = X.x; xs[1] = X.y; xs[2] = X.z; xs[3] = X.w;
      ys[0] = Y.x; ys[1] = Y.y; ys[2] = Y.z; ys[3] = Y.w;
      zs[0] = Z.x; zs[1] = Z.y; zs[2] = Z.z; zs[3] = Z.w;
      rs[0] = R.x; rs[1] = R.y; rs[2] = R.z; rs[3] = R.w;
      if (soa.type) {
        const ushort4 T = __ldg(reinterpret_cast<const ushort4 *>(soa.type + i0));
        ts[0] = T.x; ts[1] = T.y; ts[2] = T.z; ts[3] = T.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t i = i0 + j;
        xs[j] = i < n ? __ldg(soa.x + i) : 0.f;
        ys[j] = i < n ? __ldg(soa.y + i) : 0.f;
        zs[j] = i < n ? __ldg(soa.z + i) : 0.f;
        rs[j] = i < n ? __ldg(soa.r + i) : 0.f;
        ts[j] = (i < n && soa.type) ? (int)__ldg(soa.type + i) : 0;
      }
    }
    uint32_t nib = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      PIn in{};
      in.x = xs[j];
      in.y = ys[j];
      in.z = zs[j];
      in.r = rs[j];
      in.I = 1.f;  // activity does not depend on the intensity or the colour
      in.type = ts[j];
      const bool here = i0 + j < n;
      const int dec = here ? screen_activity(c, in) : 0;
      bool active = dec == 1;
      if (__any_sync(0xffffffffu, dec < 0) && dec < 0) {
        float x, y, z, r, I;
        bool fb = false;
        active = project_geom(c, in, x, y, z, r, I, fb, err);
      }
      nib |= (active ? 1u : 0u) << j;
    }
    // word q of the step holds lanes 8q .. 8q+7, four bits each
    uint32_t v = nib << (4 * (lane & 7));
    v |= __shfl_xor_sync(0xffffffffu, v, 1);
    v |= __shfl_xor_sync(0xffffffffu, v, 2);
    v |= __shfl_xor_sync(0xffffffffu, v, 4);
    const int64_t w = st * 4 + (lane >> 3);
    if ((lane & 7) == 0 && w < nwords) flags[w] = v;
  }
}

bool soa4_ok(const SoAIn *soa) {
  auto a16 = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
  return soa && a16(soa->x) && a16(soa->y) && a16(soa->z) && a16(soa->r) &&
         (!soa->type || (reinterpret_cast<uintptr_t>(soa->type) & 7u) == 0);
}

int soa4_grid(int64_t n) {
  const int64_t nsteps = (n + 127) / 128;
  const int64_t b = (nsteps + 7) / 8;
  return (int)(b < 152 * 16 ? b : 152 * 16);
}

constexpr int DW = kDenseWordsPerBlock;  // flag words per dense block (2048 particles)

template <class L>
__device__ __forceinline__ void dense_block(const L &load, int64_t n, const ProjConst &c,
                                            const uint32_t *__restrict__ flags,
                                            const uint32_t *__restrict__ word_off,
                                            const ProjectOut &o, int64_t w0,
                                            uint32_t *s_list, uint32_t *s_cnt);

template <class L>
__global__ void __launch_bounds__(256, 4) k_project_dense(L load, int64_t n, ProjConst c,
                                                       const uint32_t *__restrict__ flags,
                                                       const uint32_t *__restrict__ word_off,
                                                       ProjectOut o) {
  __shared__ uint32_t s_list[DW * 32];
  __shared__ uint32_t s_cnt[DW];
  dense_block(load, n, c, flags, word_off, o, (int64_t)blockIdx.x * DW, s_list, s_cnt);
}

// One block: the active particles of words [w0, w0 + DW), expanded into a
// dense list in shared memory, projected and colourised with all lanes busy.
template <class L>
__device__ __forceinline__ void dense_block(const L &load, int64_t n, const ProjConst &c,
                                            const uint32_t *__restrict__ flags,
                                            const uint32_t *__restrict__ word_off,
                                            const ProjectOut &o, int64_t w0,
                                            uint32_t *s_list, uint32_t *s_cnt) {
  const int64_t nwords = (n + 31) / 32;
  const int nw = (int)min((int64_t)DW, nwords - w0);
  if ((int)threadIdx.x < nw) {  // expand word t's set bits at its local offset
    uint32_t f = __ldg(flags + w0 + threadIdx.x);
    uint32_t pos = __ldg(word_off + w0 + threadIdx.x) - __ldg(word_off + w0);
    if ((int)threadIdx.x == nw - 1) s_cnt[0] = pos + (uint32_t)__popc(f);  // the block's count
    const int64_t ibase = (w0 + threadIdx.x) * 32;
    while (f) {
      const int b = __ffs(f) - 1;
      f &= f - 1;
      s_list[pos++] = (uint32_t)(ibase + b);
    }
  }
  __syncthreads();
  const uint32_t nloc = nw > 0 ? s_cnt[0] : 0u;
  const uint32_t base = nw > 0 ? __ldg(word_off + w0) : 0u;
  for (uint32_t k = threadIdx.x; k < nloc; k += blockDim.x) {
    const uint32_t i = s_list[k];
    const POut p = project_core(c, load(i), i, o.err);
    if (!p.active) atomicOr(o.err, 32u);  // the activity pass and this one disagree
    const uint32_t dst = base + k;
    if (dst >= o.cap_c) {
      atomicOr(o.err, 8u);
      continue;
    }
    o.pos_c[dst] = p.pos;
    o.col_c[dst] = p.col;
    o.idx_c[dst] = i;
    const bool shorten = c.debug_short_count && dst == 0 && p.count >= 2 && p.count <= 64;
    o.count_c[dst] = p.count - (shorten ? 1u : 0u);
    if (o.key_c) o.key_c[dst] = p.key;
  }
}

// ---- many frames in one launch (batched rendering) ---------------------------
// Each block belongs to one frame of the table: the frame whose first block
// (fblock0 / dblock0, ascending in table order) is the last one <= blockIdx.x.
__device__ __forceinline__ int table_row(const FrameProj *tab, int nf, uint32_t b, bool dense) {
  int lo = 0, hi = nf;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if ((dense ? tab[mid].dblock0 : tab[mid].fblock0) <= b) lo = mid; else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(256) k_project_flags_multi(const FrameProj *__restrict__ tab,
                                                             int nf) {
  const FrameProj &fp = tab[table_row(tab, nf, blockIdx.x, false)];
  const int64_t nwords = (fp.n + 31) / 32;
  const int64_t w = (int64_t)(blockIdx.x - fp.fblock0) * kFlagWordsPerBlock + (threadIdx.x >> 5);
  if (w >= nwords) return;  // whole warps
  const int lane = threadIdx.x & 31;
  if (fp.aos)
    flags_word(LoadAoS{static_cast<const uint8_t *>(fp.aos)}, fp.n, fp.c, fp.o.flags, fp.o.err,
               w, lane);
  else
    flags_word(LoadSoA{fp.soa.x, fp.soa.y, fp.soa.z, fp.soa.r, fp.soa.I, fp.soa.cr, fp.soa.cg,
                       fp.soa.cb, fp.soa.type},
               fp.n, fp.c, fp.o.flags, fp.o.err, w, lane);
}

__global__ void __launch_bounds__(256) k_project_dense_multi(const FrameProj *__restrict__ tab,
                                                             int nf) {
  __shared__ uint32_t s_list[DW * 32];
  __shared__ uint32_t s_cnt[DW];
  const FrameProj &fp = tab[table_row(tab, nf, blockIdx.x, true)];
  const int64_t w0 = (int64_t)(blockIdx.x - fp.dblock0) * DW;
  if (fp.aos)
    dense_block(LoadAoS{static_cast<const uint8_t *>(fp.aos)}, fp.n, fp.c, fp.o.flags,
                fp.o.word_off, fp.o, w0, s_list, s_cnt);
  else
    dense_block(LoadSoA{fp.soa.x, fp.soa.y, fp.soa.z, fp.soa.r, fp.soa.I, fp.soa.cr, fp.soa.cg,
                        fp.soa.cb, fp.soa.type},
                fp.n, fp.c, fp.o.flags, fp.o.word_off, fp.o, w0, s_list, s_cnt);
}

// Palette colour of every particle of a set whose type has a palette (the
// colourisation that does not depend on the camera), for frames that share
// the set and its palettes; other particles' slots are left as they are.
template <class L>
__global__ void __launch_bounds__(256) k_palette_cache(L load, int64_t n, ProjConst c,
                                                       float4 *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const PIn in = load(i);
    const int t = in.type;
    if (t < 0 || t >= c.ptypes || c.colvec[t]) continue;
    float r, g, b;
    bool fb = false;
    palette_colour(c, t, in.er, r, g, b, fb);
    out[i] = make_float4(r, g, b, 0.f);
  }
}

// ---- ray-sphere renderer: the per-particle pass ----------------------------
// host_rendering_new's particle loop and colourisation
// (splotch/new_renderer.cc:530-582), real_host_rendering's normalisation
// (:402-415) and screen cut (:418-446), and each particle's pyramid level
// (:488-501).  What decides which particles reach which pixels -- the
// distance cut, the unit direction c and the radius r -- follows the
// reference's double operations in order, none fused (the distance cut is
// first screened in float with a bound on its rounding); the intensity and
// colour, which only scale a particle's contribution, are computed in float.

// 9-bit-per-axis Morton code of a unit direction (a sort key for locality).
__device__ __forceinline__ uint32_t morton27(float x, float y, float z) {
  auto q = [](float v) {
    const int t = (int)((v + 1.f) * 256.f);
    uint32_t u = (uint32_t)min(max(t, 0), 511);
    u = (u | (u << 16)) & 0x030000FFu;
    u = (u | (u << 8)) & 0x0300F00Fu;
    u = (u | (u << 4)) & 0x030C30C3u;
    u = (u | (u << 2)) & 0x09249249u;
    return u;
  };
  return q(x) | (q(y) << 1) | (q(z) << 2);
}

template <class L>
__global__ void __launch_bounds__(256) k_rays_prep(L load, int64_t n, ProjConst c, RayConst k,
                                                   RayParts o) {
  const uint32_t none = (uint32_t)(k.nlev + 1) << kRayCodeShift;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const PIn in = load(i);
    const int t = in.type;
    if (t < 0 || t >= c.ptypes) {
      atomicOr(o.err, 1u);
      o.key[i] = none;
      continue;
    }
    // SPLOTCH_CLASSIC: I *= 0.5f*bfak/r, r *= 2
    const float I = in.I * ((float)k.half_bfak / in.r);
    const float r2 = fmul(in.r, 2.f);
    // the distance cut: float(|centerpos - x|) < zmax
    bool active;
    {
      const float fx = (float)k.centerpos[0] - in.x, fy = (float)k.centerpos[1] - in.y;
      const float fz = (float)k.centerpos[2] - in.z;
      const float d2 = fmaf(fz, fz, fmaf(fy, fy, fx * fx));
      // roundings of centerpos, the differences and the sum of squares
      const float E = 2.5e-7f * (fabsf((float)k.centerpos[0]) + fabsf(in.x) +
                                 fabsf((float)k.centerpos[1]) + fabsf(in.y) +
                                 fabsf((float)k.centerpos[2]) + fabsf(in.z));
      const float bound = 2.f * sqrtf(d2) * E + E * E + 5e-7f * d2;
      const float z2 = k.zmax * k.zmax;
      if (d2 + bound < z2 * 0.9999f) {
        active = true;
      } else if (d2 - bound > z2 * 1.0001f && z2 < INFINITY) {
        active = false;
      } else {
        const double dx = dsub(k.centerpos[0], (double)in.x);
        const double dy = dsub(k.centerpos[1], (double)in.y);
        const double dz = dsub(k.centerpos[2], (double)in.z);
        const float dist =
            __double2float_rn(__dsqrt_rn(dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz))));
        active = dist < k.zmax;
      }
    }
    if (!active) {
      o.key[i] = none;
      continue;
    }
    float er = in.er, eg = in.eg, eb = in.eb;
    if (!c.colvec[t]) {  // particle_colorize (splotch_host.cc:276-282)
      bool fb = false;
      float pr, pg, pb;
      palette_colour(c, t, er, pr, pg, pb, fb);
      er = pr;
      eg = pg;
      eb = pb;
    }
    const float fac = I * c.bright[t];
    double cc[3] = {dsub((double)in.x, k.campos[0]), dsub((double)in.y, k.campos[1]),
                    dsub((double)in.z, k.campos[2])};
    const double xl = ddiv(
        1.0, __dsqrt_rn(dadd(dadd(dmul(cc[0], cc[0]), dmul(cc[1], cc[1])), dmul(cc[2], cc[2]))));
    for (int a = 0; a < 3; ++a) cc[a] = dmul(cc[a], xl);
    double r = dmul((double)r2, xl);
    const double rcorr = ddiv(__dsqrt_rn(dadd(dmul(r, r), k.mr2pr2)), r);
    r = dmul(r, rcorr);
    const float rc1 = (float)rcorr;
    const float f2 = fac / (rc1 * rc1);  // brightness / rcorr^2
    const double4_16a rc = make_double4_16a(cc[0], cc[1], cc[2], r);
    const float4 cf = make_float4(__double2float_rn(cc[0]), __double2float_rn(cc[1]),
                                  __double2float_rn(cc[2]), __double2float_rn(r));
    uint32_t code = (uint32_t)k.nlev + 1;
    RayPart part = ray_part(k, rc, cf);
    if (ray_keeps(k, &k.screen.nf[0][0], k.screen.centered, k.screen, part, true)) {
      if (r > 1) {
        code = (uint32_t)k.nlev;  // a sphere around the camera
      } else {
        int hits = 0;
        for (int lv = 0; lv < k.nlev; ++lv)
          if ((r > k.lev[lv].minrad) && (r <= k.lev[lv].maxrad)) {
            code = (uint32_t)lv;
            ++hits;
          }
        if (hits > 1) atomicOr(o.err, 32u);
      }
    }
    o.key[i] = (code << kRayCodeShift) | morton27(cf.x, cf.y, cf.z);
    o.rc[i] = rc;
    o.cf[i] = cf;
    o.clo[i] = make_float4(__double2float_rn(dsub(cc[0], (double)cf.x)),
                           __double2float_rn(dsub(cc[1], (double)cf.y)),
                           __double2float_rn(dsub(cc[2], (double)cf.z)), 0.f);
    o.pod[i] = make_float4(er * f2, eg * f2, eb * f2, 0.f);
    // a ray meets the sphere iff |d - c|^2 <= 2 - 2 sqrt(1 - r^2) = 2r^2/(1 + sqrt(1 - r^2));
    // in float within 1e-7 of that for r <= 0.9; beyond, the limit is
    // ill-conditioned and every pixel is decided in double
    const float rf = cf.w;
    const float cm = rf <= 0.9f ? 2.f * rf * rf / (1.f + sqrtf(1.f - rf * rf)) : -1.f;
    const float h2 = (float)k.h2sigma;
    o.cov[i] = make_float2(cm, 1.f / (rf * rf * h2 * h2));
  }
}

// particle_sim writeback: e, x, y, z, r, I, type, active (36 bytes).
__global__ void __launch_bounds__(256) k_writeback_aos(
    const float4 *__restrict__ pos, const float4 *__restrict__ col,
    const uint8_t *__restrict__ active, const void *type_src, int type_src_kind,
    const uint32_t *__restrict__ perm, int64_t n, uint8_t *__restrict__ out) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm ? perm[s] : s;
    const float4 p = pos[i], c = col[i];
    uint16_t t = 0;
    if (type_src_kind == 1)  // AoS source: type at byte 32 of the record
      t = reinterpret_cast<const uint16_t *>(static_cast<const uint8_t *>(type_src) + i * 36 + 32)[0];
    else if (type_src_kind == 2)
      t = static_cast<const uint16_t *>(type_src)[i];
    float *f = reinterpret_cast<float *>(out + s * 36);
    f[0] = c.x; f[1] = c.y; f[2] = c.z;
    f[3] = p.x; f[4] = p.y; f[5] = p.w; f[6] = p.z; f[7] = c.w;
    uint16_t *u = reinterpret_cast<uint16_t *>(out + s * 36 + 32);
    u[0] = t;
    out[s * 36 + 34] = active[i];
    out[s * 36 + 35] = 0;
  }
}

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  const int64_t cap = 152LL * 8 * 16;  // enough resident blocks, grid-stride beyond
  if (b > cap) b = cap;
  return (int)(b > 0 ? b : 1);
}

}  // namespace

void launch_project(const void *aos, const SoAIn *soa, int64_t n, const ProjConst &c,
                    ProjectOut o, bool compact, cudaStream_t s, int *launches) {
  if (n <= 0) {
    if (compact) cudaMemsetAsync(o.n_act, 0, 4, s);
    return;
  }
  const LoadAoS la{static_cast<const uint8_t *>(aos)};
  const LoadSoA ls{soa->x, soa->y, soa->z, soa->r, soa->I, soa->cr, soa->cg, soa->cb, soa->type};
  if (compact) {
    const int64_t nwords = (n + 31) / 32;
    int fb = (int)((nwords * 32 + 255) / 256);
    if (fb > 152 * 16) fb = 152 * 16;
    const unsigned db = (unsigned)((nwords + DW - 1) / DW);
    if (aos) {
      k_project_flags<<<fb, 256, 0, s>>>(la, n, c, o.flags, o.err);
      scan_popc(o.flags, nwords, o.word_off, o.n_act, o.scan_scratch, s, launches);
      k_project_dense<<<db, 256, 0, s>>>(la, n, c, o.flags, o.word_off, o);
    } else {
      if (soa4_ok(soa))
        k_project_flags_soa4<<<soa4_grid(n), 256, 0, s>>>(*soa, n, c, o.flags, o.err);
      else
        k_project_flags<<<fb, 256, 0, s>>>(ls, n, c, o.flags, o.err);
      scan_popc(o.flags, nwords, o.word_off, o.n_act, o.scan_scratch, s, launches);
      k_project_dense<<<db, 256, 0, s>>>(ls, n, c, o.flags, o.word_off, o);
    }
    if (launches) *launches += 2;
  } else {
    if (aos)
      k_project_full<<<grid_for(n), 256, 0, s>>>(la, n, c, o);
    else
      k_project_full<<<grid_for(n), 256, 0, s>>>(ls, n, c, o);
    if (launches) *launches += 1;
  }
}

void launch_project_flags(const void *aos, const SoAIn *soa, int64_t n, const ProjConst &c,
                          const ProjectOut &o, cudaStream_t s) {
  if (n <= 0) return;
  const int64_t nwords = (n + 31) / 32;
  int fb = (int)((nwords * 32 + 255) / 256);
  if (fb > 152 * 16) fb = 152 * 16;
  if (aos)
    k_project_flags<<<fb, 256, 0, s>>>(LoadAoS{static_cast<const uint8_t *>(aos)}, n, c,
                                       o.flags, o.err);
  else if (soa4_ok(soa))
    k_project_flags_soa4<<<soa4_grid(n), 256, 0, s>>>(*soa, n, c, o.flags, o.err);
  else
    k_project_flags<<<fb, 256, 0, s>>>(
        LoadSoA{soa->x, soa->y, soa->z, soa->r, soa->I, soa->cr, soa->cg, soa->cb, soa->type},
        n, c, o.flags, o.err);
}

void launch_project_dense(const void *aos, const SoAIn *soa, int64_t n, const ProjConst &c,
                          const ProjectOut &o, cudaStream_t s) {
  if (n <= 0) return;
  const int64_t nwords = (n + 31) / 32;
  const unsigned db = (unsigned)((nwords + DW - 1) / DW);
  if (aos)
    k_project_dense<<<db, 256, 0, s>>>(LoadAoS{static_cast<const uint8_t *>(aos)}, n, c, o.flags,
                                       o.word_off, o);
  else
    k_project_dense<<<db, 256, 0, s>>>(
        LoadSoA{soa->x, soa->y, soa->z, soa->r, soa->I, soa->cr, soa->cg, soa->cb, soa->type},
        n, c, o.flags, o.word_off, o);
}

void launch_project_flags_multi(const FrameProj *tab, int nf, uint32_t nblocks,
                                cudaStream_t s) {
  if (nf > 0 && nblocks > 0) k_project_flags_multi<<<nblocks, 256, 0, s>>>(tab, nf);
}

void launch_project_dense_multi(const FrameProj *tab, int nf, uint32_t nblocks,
                                cudaStream_t s) {
  if (nf > 0 && nblocks > 0) k_project_dense_multi<<<nblocks, 256, 0, s>>>(tab, nf);
}

void launch_palette_cache(const void *aos, const SoAIn *soa, int64_t n, const ProjConst &c,
                          float4 *out, cudaStream_t s) {
  if (n <= 0) return;
  ProjConst cc = c;
  cc.pal_cache = nullptr;
  if (aos)
    k_palette_cache<<<grid_for(n), 256, 0, s>>>(LoadAoS{static_cast<const uint8_t *>(aos)}, n,
                                                cc, out);
  else
    k_palette_cache<<<grid_for(n), 256, 0, s>>>(
        LoadSoA{soa->x, soa->y, soa->z, soa->r, soa->I, soa->cr, soa->cg, soa->cb, soa->type}, n,
        cc, out);
}

void launch_rays_prep(const void *aos, const SoAIn *soa, int64_t n, const ProjConst &pc,
                      const RayConst &k, const RayParts &o, cudaStream_t s) {
  if (n <= 0) return;
  ProjConst cc = pc;
  cc.pal_cache = nullptr;
  if (aos)
    k_rays_prep<<<grid_for(n), 256, 0, s>>>(LoadAoS{static_cast<const uint8_t *>(aos)}, n, cc,
                                            k, o);
  else
    k_rays_prep<<<grid_for(n), 256, 0, s>>>(
        LoadSoA{soa->x, soa->y, soa->z, soa->r, soa->I, soa->cr, soa->cg, soa->cb, soa->type}, n,
        cc, k, o);
}

void launch_writeback_aos(const float4 *pos, const float4 *col, const uint8_t *active,
                          const void *type_src, int type_src_kind, const uint32_t *perm,
                          int64_t n, void *aos_out, cudaStream_t s) {
  if (n <= 0) return;
  k_writeback_aos<<<grid_for(n), 256, 0, s>>>(pos, col, active, type_src, type_src_kind, perm,
                                             n, static_cast<uint8_t *>(aos_out));
}

}  // namespace spl
