// spl_tile.cuh -- the per-tile particle staging shared by the forward splat
// (spl_splat.cu) and its adjoint (spl_backward.cu).
//
// A tile's particle list is streamed through shared memory B entries at a
// time.  Each entry is staged once per tile: tile-local position, Gaussian
// width, colour, the exact column runs of the footprint inside the tile and
// the rows they cover, decided as the reference decides coverage
// (splotch/splotch_host.cc:580-606: tile-local coordinates, truncating int
// conversion, the column run y in [int(py-dy+1), int(py+dy+1)) with
// dy = sqrt(r^2 - dx^2)), in non-contracted float arithmetic.
#pragma once

#include "spl_internal.cuh"

namespace spl {

constexpr int IW = 8, IH = 4;  // item: 8 columns x 4 rows, one pixel per lane

// Staged particles, one entry per list slot.  Each value a pixel pair shares
// is held twice, so one 128-bit load gives packed (F2) operands.
template <int B>
struct Stage {
  float4 pxy[B];   // posx, posx, posy, posy (tile-local)
  float4 es[B];    // e0, e0, stp*log2e, stp*log2e (e negated when additive)
  float4 e12[B];   // e1, e1, e2, e2                (negated when additive)
  float4 q01[B];   // q0, q0, q1, q1 (q = e/(e+grayabsorb); negated on request)
  float2 q2[B];    // q2, q2
  uint32_t bb[B];  // minx | maxx<<8 | miny<<16 | maxy<<24: the clipped bounding box's
                   // columns, the covered rows (0: none covered)
};

// Run-table row length: T rounded up to whole 8-pixel items, so that every
// column an item can address lies in the row and rows stay 16-byte aligned.
// Per column the covered rows [lo, hi): as lo | (hi-lo)<<8, or (tiles of 9
// to 16 pixels, MK) as the row mask with bits lo..hi-1 set, column c at slot
// mask_slot(c) so that columns c and c + 8 share one 32-bit word; zero
// outside the bounding box.
__host__ __device__ constexpr int run_stride(int T) { return (T + 7) & ~7; }
__host__ __device__ constexpr int mask_slot(int c) { return (c & 7) * 2 + (c >> 3); }

// Stage list entry jj of the tile at (x0s, y0s), tw x th pixels, into slot;
// an entry past the list end stages an empty box.  Returns the particle index
// (0xffffffff past the end); *colour receives the particle's colour.
template <int B, bool ADD, bool NEGQ, bool MK = false>
__device__ __forceinline__ uint32_t stage_entry(Stage<B> &S, uint16_t *srun, int RS, int slot,
                                                const SplatArgs &a, uint32_t jj, uint32_t end,
                                                int x0s, int y0s, int tw, int th,
                                                float4 *colour = nullptr) {
  uint32_t bb = 0, idx = 0xffffffffu;
  if (jj < end) {
    idx = __ldg(a.entries + jj);
    const float4 p = __ldg(a.pos + idx);
    const float4 c = __ldg(a.col + idx);
    if (colour) *colour = c;
    const float rfacr = fmul(p.z, 0.75f);
    const float posx = fsub(p.x, (float)x0s), posy = fsub(p.y, (float)y0s);
    const int minx = max(f2i(fadd(fsub(posx, rfacr), 1.f)), 0);
    const int maxx = min(f2i(fadd(fadd(posx, rfacr), 1.f)), tw);
    const int miny = max(f2i(fadd(fsub(posy, rfacr), 1.f)), 0);
    const int maxy = min(f2i(fadd(fadd(posy, rfacr), 1.f)), th);
    const float radsq = fmul(rfacr, rfacr);
    const float sigma = fmul(a.h2sigma, p.z);
    const float stp = fdiv(-1.f, fmul(sigma, sigma));
    if (minx < maxx && miny < maxy) {
      uint16_t *run = srun + slot * RS;
      uint4 *row16 = reinterpret_cast<uint4 *>(run);
      for (int i = 0; i < RS / 8; ++i) row16[i] = make_uint4(0u, 0u, 0u, 0u);
      for (int x = minx; x < maxx; ++x) {  // splotch_host.cc:603-606
        const float dx = fsub((float)x, posx);
        const float dxsq = fmul(dx, dx);
        const float dy = fsqrt(fsub(radsq, dxsq));
        const int lo = max(miny, f2i(fadd(fsub(posy, dy), 1.f)));
        const int hi = min(maxy, f2i(fadd(fadd(posy, dy), 1.f)));
        if (MK)  // 0 <= lo < hi <= th <= 16 when the run is not empty
          run[mask_slot(x)] =
              hi > lo ? (uint16_t)(((1u << hi) - 1u) & ~((1u << lo) - 1u)) : (uint16_t)0;
        else
          run[x] = (uint16_t)(lo | (max(hi - lo, 0) << 8));
      }
      // The rows the particle covers.  Every step from |dx| to the run is
      // monotone, so a column nearer the centre holds the runs of the columns
      // beyond it: the union of all runs is the longer run of the two columns
      // next to posx (clamped to the box).  A warp whose rows it misses gets
      // no hit; the columns stay those of the bounding box.
      const int xa = min(max(f2i(floorf(posx)), minx), maxx - 1);
      const int xb = min(xa + 1, maxx - 1);
      const uint32_t ra = run[MK ? mask_slot(xa) : xa], rb = run[MK ? mask_slot(xb) : xb];
      if (MK) {
        const uint32_t rc = ra | rb;  // nested runs: the union is the longer
        if (rc)
          bb = (uint32_t)minx | ((uint32_t)maxx << 8) | ((uint32_t)(__ffs(rc) - 1) << 16) |
               ((uint32_t)(32 - __clz(rc)) << 24);
      } else {
        const uint32_t rc = (rb >> 8) > (ra >> 8) ? rb : ra;
        if ((rc >> 8) > 0u)
          bb = (uint32_t)minx | ((uint32_t)maxx << 8) | ((rc & 255u) << 16) |
               (((rc & 255u) + (rc >> 8)) << 24);
      }
    }
    const float s2 = stp * kLog2e;
    S.pxy[slot] = make_float4(posx, posx, posy, posy);
    if (ADD) {
      S.es[slot] = make_float4(-c.x, -c.x, s2, s2);
      S.e12[slot] = make_float4(-c.y, -c.y, -c.z, -c.z);
    } else {
      // q = e/(e+grayabsorb), splotch_host.cc:626-628
      const float sq = NEGQ ? -1.f : 1.f;
      const float q0 = sq * fdiv(c.x, fadd(c.x, a.gray));
      const float q1 = sq * fdiv(c.y, fadd(c.y, a.gray));
      const float q2 = sq * fdiv(c.z, fadd(c.z, a.gray));
      S.es[slot] = make_float4(c.x, c.x, s2, s2);
      S.e12[slot] = make_float4(c.y, c.y, c.z, c.z);
      S.q01[slot] = make_float4(q0, q0, q1, q1);
      S.q2[slot] = make_float2(q2, q2);
    }
  }
  S.bb[slot] = bb;
  return idx;
}

// Exact coverage of a lane's pixel by a staged particle: the pixel's row
// inside its column's run (a pixel outside the tile has row 255).
__device__ __forceinline__ bool covered(const uint16_t *run, int col, int row) {
  const uint32_t r = run[col];
  return (uint32_t)(row - (int)(r & 255)) < (r >> 8);
}

// The same test on a row-mask table: bit is the pixel's row bit (0 outside
// the tile).
__device__ __forceinline__ bool covered_mask(const uint16_t *run, int col, uint32_t bit) {
  return (run[mask_slot(col)] & bit) != 0u;
}

// Coverage of a lane's pixel pair: pixel 0 at column c0, row r0 (row bit b0),
// pixel 1 (when has1) at c1, r1, b1.  Row masks (MK): the pair's columns are
// c0 < 8 and c0 + 8, whose masks share the 32-bit word at c0.
template <bool MK>
__device__ __forceinline__ void covered_pair(const uint16_t *run, int c0, int r0, uint32_t b0,
                                             bool has1, int c1, int r1, uint32_t b1, bool &in0,
                                             bool &in1) {
  if (MK && has1) {
    const uint32_t w2 = reinterpret_cast<const uint32_t *>(run)[c0 & 7];
    in0 = (w2 & b0) != 0u;
    in1 = ((w2 >> 16) & b1) != 0u;
  } else if (MK) {
    in0 = covered_mask(run, c0, b0);
    in1 = false;
  } else {
    in0 = covered(run, c0, r0);
    in1 = has1 && covered(run, c1, r1);
  }
}

// Does a bounding box reach the 16x4 pixels of the pair whose left item
// starts at (ix0, iy0)?
__device__ __forceinline__ bool box_meets_pair(uint32_t bb, int ix0, int iy0) {
  const int mnx = bb & 255, mxx = (bb >> 8) & 255, mny = (bb >> 16) & 255, mxy = bb >> 24;
  return mnx < ix0 + 2 * IW && mxx > ix0 && mny < iy0 + IH && mxy > iy0;
}

// Does a bounding box (non-empty) reach the warp's box [x0, x1) x [y0, y1)?
__device__ __forceinline__ bool box_meets_warp(uint32_t bb, int x0, int x1, int y0, int y1) {
  const int mnx = bb & 255, mxx = (bb >> 8) & 255, mny = (bb >> 16) & 255, mxy = bb >> 24;
  return (mnx < mxx) && (mnx < x1) && (mxx > x0) && (mny < y1) && (mxy > y0);
}

}  // namespace spl
