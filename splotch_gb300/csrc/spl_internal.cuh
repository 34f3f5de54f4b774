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

// expm1(x) for x <= 0 in float with ~1e-7 relative error everywhere:
// Taylor series (degree 7, Horner form) near zero where exp(x)-1 cancels,
// ex2-based exp(x)-1 elsewhere.
__device__ __forceinline__ float expm1_neg(float x) {
  if (x > -0.25f) {
    float p = 1.f / 5040.f;
    p = fmaf(p, x, 1.f / 720.f);
    p = fmaf(p, x, 1.f / 120.f);
    p = fmaf(p, x, 1.f / 24.f);
    p = fmaf(p, x, 1.f / 6.f);
    p = fmaf(p, x, 0.5f);
    p = fmaf(p, x, 1.f);
    return p * x;
  }
  return ex2(x * kLog2e) - 1.f;
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

// ---------------------------------------------------------------------------
// Launch wrappers (defined in the .cu files).
struct ProjectOut {
  float4 *pos;      // x, y, r, z   (projected)
  float4 *col;      // e.r, e.g, e.b, I (colourised)
  uint8_t *active;
  uint32_t *count;  // tiles per particle (binning circle test)
  uint32_t *key;    // sort key (when sort_type != 0)
  uint32_t *err;    // device error word
};

void launch_project_aos(const void *aos, int64_t n, const ProjConst &c, ProjectOut o,
                        cudaStream_t s);
void launch_project_soa(const float *x, const float *y, const float *z, const float *r,
                        const float *I, const float *cr, const float *cg, const float *cb,
                        const uint16_t *type, int64_t n, const ProjConst &c, ProjectOut o,
                        cudaStream_t s);
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
int radix_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_tmp,
                     uint32_t *vals_tmp, uint32_t *keys_out, uint32_t *vals_out, int64_t n,
                     int bit0, int bit1, bool keys_needed, void *scratch, cudaStream_t s,
                     int *launches);

// Exclusive scan of count[order[s]] (order may be null) into off (n+1 slots;
// off[n] = total).
size_t scan_scratch_bytes(int64_t n);
void scan_counts(const uint32_t *count, const uint32_t *order, int64_t n, uint64_t *off,
                 void *scratch, cudaStream_t s, int *launches);

// Bin emission and tile ranges.
// wide_list must hold n entries, wide_n one counter (particles with more than
// 64 tiles go to the warp-per-particle emitter through this list).
void launch_emit(const float4 *pos, const uint32_t *count, const uint32_t *order,
                 const uint64_t *off, int64_t n, Tiling g, uint32_t *tkey, uint32_t *tval,
                 uint32_t *wide_list, uint32_t *wide_n, cudaStream_t s);
void launch_tile_ranges(const uint32_t *sorted_tkey, int64_t ne, int64_t ntiles,
                        uint32_t *tile_start, cudaStream_t s);

// Splat.
struct SplatArgs {
  const float4 *pos;
  const float4 *col;
  const uint32_t *entries;     // particle index per bin entry, tile-major
  const uint32_t *tile_start;  // ntiles+1
  int T, ncx, ncy, xres, yres;
  float gray;
  float h2sigma;
  int a_eq_e;
  int order_mode;
  float ftb_eps;
  float *pic;                  // device, x-major xres*yres*3
};
int launch_splat(const SplatArgs &a, cudaStream_t s);
void launch_count_fragments(const SplatArgs &a, unsigned long long *total, cudaStream_t s);

}  // namespace spl
