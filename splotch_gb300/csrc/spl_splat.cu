// spl_splat.cu -- tiled Gaussian splat (render_new region B,
// splotch/splotch_host.cc:434-692), additive and ordered emission-absorption.
//
// One CTA per tile.  The tile is cut into 8x4-pixel items; lane l of an item
// owns pixel (l%8, l/8) of it and keeps its three channels in registers for
// the whole tile.  Each warp owns a WX x WY group of items (K = WX*WY pixels
// per lane), so one particle's per-warp cost (parameter loads, bounding-box
// tests) is shared by up to 32*K pixels and an item the particle misses costs
// one uniform branch.
//
// The tile's particle list is streamed through shared memory B entries at a
// time: each thread stages particles (tile-local position, Gaussian width,
// clipped bounding box, colour) and the exact column runs of their footprint
// inside the tile.  Each warp ballots the staged particles against its own
// bounding box and walks only the hits, in list order (or reverse list order
// front-to-back).
//
// A lane's pixels are processed in pairs (items 2p and 2p+1, side by side) with
// packed .f32x2 arithmetic: the pair's three channels take three packed
// operations per step where two pixels took six.  A pixel of the pair that the
// particle does not cover gets weight 0, which leaves its state unchanged.
//
// Coverage is decided exactly as the reference decides it (tile-local
// coordinates, truncating int conversion, the column run
// y in [int(py-dy+1), int(py+dy+1)) with dy = sqrt(r^2 - dx^2)), in
// non-contracted float arithmetic, so every pixel receives exactly the
// reference's fragments.  The Gaussian weight exp(stp*dx^2)*exp(stp*dy^2) is
// evaluated as one ex2(stp*log2e*(dx^2+dy^2)) instead of the reference's
// exptable<float> (splotch/splotchutils.h:174-215), closer to the exact weight.
//
// Absorption: back-to-front applies C += expm1(-e*att)*(C - q) in list order
// (splotch_host.cc:663-665).  Front-to-back visits the list in reverse and
// accumulates C += Tr*q*(1-T), Tr *= T -- the same sum term by term -- and stops
// a warp once every pixel's transmittance in all channels is below epsilon or
// below ftb_rel times the colour it has composited, and the tile once every
// warp has stopped.  expm1(-u) is a Taylor polynomial below u = 0.05 and the
// exponential form above; a warp evaluates only the polynomial when all its
// fragments of a hit are below the cut (one vote per hit).
#include "spl_tile.cuh"

namespace spl {

namespace {

template <int B>
using Smem = Stage<B>;  // followed by uint16_t run[B][run_stride(T)]

template <int B>
size_t smem_bytes(int T) {
  return sizeof(Smem<B>) + (size_t)B * run_stride(T) * 2;
}

// One tile of one frame, by the whole CTA (shared by the per-frame launch and
// the persistent batch kernel).
// AUX (ordered frames only): also accumulate each pixel's optical depth and
// record where the warp stopped, for the adjoint (SplatArgs::aux).
// MK: the run table holds row masks (tiles of 9 to 16 pixels).
template <int NT, int WX, int WY, int B, bool ADD, bool FTB, bool AUX = false, bool MK = false>
// [start, end): the part of the tile's list to composite (the whole list, or
// one segment of a heavy tile).  partial: null to write the tile into the
// image, else the segment's own result per tile pixel (x*T + y): its
// composite and its transmittance, two float4.  opaque (front-to-back
// segments, may be null): a per-tile flag that the tile's front segment sets
// once all its pixels are opaque, after which the segments behind it stop.
__device__ __forceinline__ void splat_tile(const SplatArgs &a, const int tile,
                                           uint8_t *smem_raw, const uint32_t start,
                                           const uint32_t end, float4 *partial,
                                           uint32_t *opaque = nullptr, bool front = false) {
  __shared__ uint32_t s_opaque;
  constexpr int K = WX * WY;
  constexpr int NP = (K + 1) / 2;  // pixel pairs per lane: items (2p, 2p+1)
  static_assert(!(AUX && ADD), "optical depth is kept for ordered frames only");
  static_assert(K == 1 || WX % 2 == 0, "the items of a pair share one row");
  Smem<B> &S = *reinterpret_cast<Smem<B> *>(smem_raw);
  uint16_t *srun = reinterpret_cast<uint16_t *>(smem_raw + sizeof(Smem<B>));

  const int T = a.T;
  const int RS = run_stride(T);
  const int ix = tile % a.ncx, iy = tile / a.ncx;
  const int x0s = ix * T, y0s = iy * T;
  const int tw = min(x0s + T, a.xres) - x0s;
  const int th = min(y0s + T, a.yres) - y0s;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;

  // ---- this warp's items ------------------------------------------------
  const int nbx = (tw + IW - 1) / IW, nby = (th + IH - 1) / IH;
  const int nwx = (nbx + WX - 1) / WX, nwy = (nby + WY - 1) / WY;
  const int wx = w % nwx, wy = w / nwx;
  const bool warp_has_pixels = wy < nwy;
  const int wbx0 = wx * WX * IW, wby0 = wy * WY * IH;  // warp box, tile-local
  const int wbx1 = min(wbx0 + WX * IW, tw), wby1 = min(wby0 + WY * IH, th);

  // Pixel (k) of this lane: run-table column and row (MK: the row's bit); a
  // pixel outside the tile reads column 0 with row 255 (bit 0), which no run
  // contains.
  int col[K], row[K];
  uint32_t rbit[K];
  F2 px2[NP], py2[NP];                   // pixel coordinates of each pair
  F2 acc[NP][3], tr[NP][3];              // per channel: (pixel 2p, pixel 2p+1)
  F2 od[AUX ? NP : 1][3];                // optical depth (AUX)
  uint32_t stop = 0;  // list position below which this warp composited nothing
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int x = wbx0 + (k % WX) * IW + (lane & 7);
    const int y = wby0 + (k / WX) * IH + (lane >> 3);
    const bool valid = warp_has_pixels && x < tw && y < th;
    col[k] = valid ? x : 0;
    row[k] = valid ? y : 255;
    rbit[k] = valid ? 1u << y : 0u;
  }
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    const int x = wbx0 + ((2 * p) % WX) * IW + (lane & 7);
    const int y = wby0 + ((2 * p) / WX) * IH + (lane >> 3);
    px2[p] = f2((float)x, (float)(x + IW));
    py2[p] = f2((float)y);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (AUX) od[AUX ? p : 0][c] = f2(0.f);
      acc[p][c] = f2(0.f);
      tr[p][c] = f2(1.f);
    }
  }

  const int nbatch = (int)((end - start + B - 1) / B);
  bool warp_done = !warp_has_pixels;

  for (int b = 0; b < nbatch; ++b) {
    const int bi = FTB ? nbatch - 1 - b : b;
    // ---- stage B particles ------------------------------------------------
#pragma unroll 1
    for (int slot = threadIdx.x; slot < B; slot += NT)
      stage_entry<B, ADD, FTB, MK>(S, srun, RS, slot, a, start + (uint32_t)bi * B + slot, end,
                                   x0s, y0s, tw, th);
    if (FTB && opaque && threadIdx.x == 0)
      s_opaque = *reinterpret_cast<volatile uint32_t *>(opaque);
    __syncthreads();
    // the segment in front made every pixel opaque: what lies behind is
    // weighted below ftb_eps (this segment's partial is folded behind it)
    if (FTB && opaque && !front && s_opaque) break;
    // ---- accumulate ---------------------------------------------------------
    if (!warp_done) {
#pragma unroll 1
      for (int cc = 0; cc < B / 32; ++cc) {
        const int ch = FTB ? B / 32 - 1 - cc : cc;
        const bool hit = box_meets_warp(S.bb[ch * 32 + lane], wbx0, wbx1, wby0, wby1);
        uint32_t mask = __ballot_sync(0xffffffffu, hit);
        while (mask) {
          const int bit = FTB ? 31 - __clz(mask) : __ffs(mask) - 1;
          mask &= ~(1u << bit);
          const int j = ch * 32 + bit;
          const float4 pxy = S.pxy[j];
          const float4 es = S.es[j];
          const float4 e12 = S.e12[j];
          float4 q01 = make_float4(0.f, 0.f, 0.f, 0.f);
          float2 q2 = make_float2(0.f, 0.f);
          if (!ADD) {
            q01 = S.q01[j];
            q2 = S.q2[j];
          }
          uint32_t bbj = 0;
          if (NP > 1) bbj = S.bb[j];
          const uint16_t *run = srun + j * RS;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            // does the particle's box reach this pair's 16x4 pixels (uniform)?
            if (NP > 1 && !box_meets_pair(bbj, wbx0 + ((2 * p) % WX) * IW,
                                          wby0 + ((2 * p) / WX) * IH))
              continue;
            const int k1 = 2 * p + 1 < K ? 2 * p + 1 : 0;
            bool in0, in1;
            covered_pair<MK>(run, col[2 * p], row[2 * p], rbit[2 * p], 2 * p + 1 < K, col[k1],
                             row[k1], rbit[k1], in0, in1);
            // a pixel the particle does not cover gets att = 0: its update is
            // the identity in every mode
            if (ADD) {
              if (in0 || in1) {
                const F2 dx = sub2(px2[p], f2(pxy.x, pxy.y));
                const F2 dy = sub2(py2[p], f2(pxy.z, pxy.w));
                const F2 arg = mul2(f2(es.z, es.w), fma2(dy, dy, mul2(dx, dx)));
                const F2 att = f2(in0 ? ex2(f2lo(arg)) : 0.f, in1 ? ex2(f2hi(arg)) : 0.f);
                acc[p][0] = fma2(f2(es.x, es.y), att, acc[p][0]);  // e negated
                acc[p][1] = fma2(f2(e12.x, e12.y), att, acc[p][1]);
                acc[p][2] = fma2(f2(e12.z, e12.w), att, acc[p][2]);
              }
            } else {
              // every lane updates (uncovered pixels with att = 0), so that the
              // warp can vote: when all its optical depths e*att are below the
              // Taylor cut, expm1 takes the polynomial alone (the same values
              // the per-component choice gives)
              const F2 dx = sub2(px2[p], f2(pxy.x, pxy.y));
              const F2 dy = sub2(py2[p], f2(pxy.z, pxy.w));
              const F2 arg = mul2(f2(es.z, es.w), fma2(dy, dy, mul2(dx, dx)));
              const F2 att = f2(in0 ? ex2(f2lo(arg)) : 0.f, in1 ? ex2(f2hi(arg)) : 0.f);
              const F2 e[3] = {f2(es.x, es.y), f2(e12.x, e12.y), f2(e12.z, e12.w)};
              const F2 q[3] = {f2(q01.x, q01.y), f2(q01.z, q01.w), f2(q2.x, q2.y)};
              F2 u[3];
#pragma unroll
              for (int c = 0; c < 3; ++c) u[c] = mul2(e[c], att);
              const float um = fmaxf(fmaxf(fmaxf(f2lo(u[0]), f2hi(u[0])), fmaxf(f2lo(u[1]), f2hi(u[1]))),
                                     fmaxf(f2lo(u[2]), f2hi(u[2])));
              const bool poly = __all_sync(0xffffffffu, um < kExpm1TaylorCut);
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                if (AUX) od[AUX ? p : 0][c] = add2(od[AUX ? p : 0][c], u[c]);
                const F2 m = poly ? expm1_neg2_poly(u[c]) : expm1_neg2(u[c]);
                if (!FTB) {
                  acc[p][c] = fma2(m, sub2(acc[p][c], q[c]), acc[p][c]);
                } else {
                  // -w = Tr*expm1(-e*att); C += w*q (q negated); Tr -= w
                  const F2 nw = mul2(tr[p][c], m);
                  acc[p][c] = fma2(nw, q[c], acc[p][c]);
                  tr[p][c] = add2(tr[p][c], nw);
                }
              }
            }
          }
        }
      }
      if (FTB) {
        // a pixel is done once each channel's transmittance is below the
        // absolute cut or below ftb_rel times the colour it has composited
        // (acc).  Frames kept for the adjoint stop the same way: the list
        // position where a warp stopped is kept, and the adjoint walks exactly
        // the fragments composited before it.
        const float rel = a.ftb_rel;
        bool mine_done = true;
#pragma unroll
        for (int k = 0; k < K; ++k) {
          if (MK ? rbit[k] != 0u : row[k] != 255) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const float t = (k & 1) ? f2hi(tr[k / 2][c]) : f2lo(tr[k / 2][c]);
              const float v = (k & 1) ? f2hi(acc[k / 2][c]) : f2lo(acc[k / 2][c]);
              mine_done = mine_done && (t < a.ftb_eps || t < rel * v);
            }
          }
        }
        warp_done = __all_sync(0xffffffffu, mine_done);
        if (AUX && warp_done) stop = (uint32_t)bi * B;
      }
    }
    if (FTB) {
      if (__syncthreads_and(warp_done ? 1 : 0)) {
        if (front && opaque && threadIdx.x == 0) *reinterpret_cast<volatile uint32_t *>(opaque) = 1u;
        break;
      }
    } else {
      __syncthreads();
    }
  }

  // ---- write the tile (pic is x-major: pixel (x,y) at (x*yres + y)*3) ----
  if (MK) {
#pragma unroll
    for (int k = 0; k < K; ++k) row[k] = rbit[k] ? __ffs(rbit[k]) - 1 : 255;
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (row[k] != 255 && partial) {
      float v[3], t[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        v[c] = (k & 1) ? f2hi(acc[k / 2][c]) : f2lo(acc[k / 2][c]);
        t[c] = (k & 1) ? f2hi(tr[k / 2][c]) : f2lo(tr[k / 2][c]);
      }
      const int px = (col[k] * T + row[k]) * 2;
      partial[px] = make_float4(v[0], v[1], v[2], 0.f);
      partial[px + 1] = make_float4(t[0], t[1], t[2], 0.f);
    } else if (row[k] != 255) {
      const size_t pix = (size_t)(x0s + col[k]) * a.yres + (y0s + row[k]);
      float v[3], d[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        v[c] = (k & 1) ? f2hi(acc[k / 2][c]) : f2lo(acc[k / 2][c]);
        if (AUX) d[c] = (k & 1) ? f2hi(od[AUX ? k / 2 : 0][c]) : f2lo(od[AUX ? k / 2 : 0][c]);
      }
      float *o = a.pic + pix * 3;
      o[0] = v[0];
      o[1] = v[1];
      o[2] = v[2];
      if (AUX) a.aux[pix] = make_float4(d[0], d[1], d[2], __uint_as_float(stop));
    }
  }
}

template <int NT, int WX, int WY, int B, bool ADD, bool FTB, bool AUX, bool MK>
__global__ void __launch_bounds__(NT) k_splat(SplatArgs a) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  const int tile = a.tile_order ? (int)__ldg(a.tile_order + blockIdx.x) : (int)blockIdx.x;
  splat_tile<NT, WX, WY, B, ADD, FTB, AUX, MK>(a, tile, smem_raw, a.tile_start[tile],
                                           a.tile_start[tile + 1], nullptr);
}

// Persistent splat over a queue of (frame, tile) items: each CTA takes the
// next item from an atomic counter until the queue is empty.  The queue is in
// longest-list-first order across all frames; every frame's own arguments
// (image, tiling, mode, tile-range slice) come from a per-frame table.  MODE
// 0 / 1: every item is additive / front-to-back (one splat form compiled in);
// 2: the form is chosen per item.  MK: row-mask coverage (the batch's tile
// size is 9 to 16 pixels).  The 128-thread forms are held to 64 registers (8
// CTAs per SM, as the per-frame splat runs): measured on the 96-frame batch,
// 215.2 -> 210.5 ms.
template <int NT, int WX, int WY, int B, int MODE, bool MK>
__global__ void __launch_bounds__(NT, NT == 128 ? 8 : 0) k_splat_queue(BatchSplatArgs q) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  __shared__ uint32_t s_item;
  __shared__ SplatArgs s_args;  // the item's frame arguments, read from shared memory
  for (;;) {
    if (threadIdx.x == 0) {
      const uint32_t item = atomicAdd(q.counter, 1u);
      s_item = item;
      if (item < q.nwork) s_args = q.frames[__ldg(q.frame_of_tile + __ldg(q.work + q.work_begin + item))];
    }
    __syncthreads();
    const uint32_t item = s_item;
    if (item >= q.nwork) break;
    const uint32_t gt = __ldg(q.work + q.work_begin + item);
    const uint32_t f = __ldg(q.frame_of_tile + gt);
    const SplatArgs &a = s_args;
    const int tile = (int)(gt - q.tile_base[f]);
    const uint32_t t0 = a.tile_start[tile], t1 = a.tile_start[tile + 1];
    if (MODE == 0)
      splat_tile<NT, WX, WY, B, true, false, false, MK>(a, tile, smem_raw, t0, t1, nullptr);
    else if (MODE == 1)
      splat_tile<NT, WX, WY, B, false, true, false, MK>(a, tile, smem_raw, t0, t1, nullptr);
    else if (a.a_eq_e)
      splat_tile<NT, WX, WY, B, true, false, false, MK>(a, tile, smem_raw, t0, t1, nullptr);
    else if (a.order_mode == 1)
      splat_tile<NT, WX, WY, B, false, true, false, MK>(a, tile, smem_raw, t0, t1, nullptr);
    else
      splat_tile<NT, WX, WY, B, false, false, false, MK>(a, tile, smem_raw, t0, t1, nullptr);
    __syncthreads();  // s_item and the staging buffers are reused
  }
}

// Heavy tiles cut into list segments (spl_context_set_split_tiles): CTA i of
// the launch takes segment i, numbered in tile order (SplatSegs::seg_off).  A
// tile of one segment is rendered into the image directly; each segment of a
// longer tile writes its own composite and transmittance, and
// k_splat_combine folds them.
template <int NT, int WX, int WY, int B, bool ADD, bool FTB, bool MK>
__global__ void __launch_bounds__(NT) k_splat_seg(SplatArgs a, SplatSegs g) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  const uint64_t item = blockIdx.x;
  if (item >= g.seg_off[g.ntiles]) return;
  int o = 0, ohi = (int)g.ntiles;  // seg_off[o] <= item < seg_off[ohi]
  while (ohi - o > 1) {
    const int mid = (o + ohi) >> 1;
    if (g.seg_off[mid] <= item) o = mid; else ohi = mid;
  }
  const int tile = a.tile_order ? (int)__ldg(a.tile_order + o) : o;
  const uint32_t nseg = (uint32_t)(g.seg_off[o + 1] - g.seg_off[o]);
  const uint32_t k = (uint32_t)(item - g.seg_off[o]);
  // front-to-back: the front segment (last in list order) takes the first
  // item of its tile, so that it starts first and can stop the others early
  const uint32_t ls = (FTB && nseg > 1) ? nseg - 1 - k : k;  // segment in list order
  const uint32_t t1 = a.tile_start[tile + 1];
  const uint32_t s0 = a.tile_start[tile] + ls * g.seg_len;
  // a tile of one segment is its whole list (it may be longer than seg_len)
  const uint32_t s1 = nseg == 1 ? t1 : (uint32_t)min((uint64_t)t1, (uint64_t)s0 + g.seg_len);
  float4 *part =
      nseg > 1 ? g.partial + (g.seg_off[o] + ls) * (size_t)(a.T * a.T) * 2 : nullptr;
  uint32_t *opq = (FTB && nseg > 1) ? g.opaque + o : nullptr;
  splat_tile<NT, WX, WY, B, ADD, FTB, false, MK>(a, tile, smem_raw, s0, s1, part, opq,
                                                ls == nseg - 1);
}

// One CTA per tile (tile order): a tile of several segments gets, per pixel,
// the segments' results folded in list order (back to front): additive
// C = the parts' sum in order; front-to-back C <- acc_k + tr_k * C.
template <bool ADD>
__global__ void __launch_bounds__(256) k_splat_combine(SplatArgs a, SplatSegs g) {
  const int o = blockIdx.x;
  const uint32_t nseg = (uint32_t)(g.seg_off[o + 1] - g.seg_off[o]);
  if (nseg <= 1) return;
  const int tile = a.tile_order ? (int)__ldg(a.tile_order + o) : o;
  const int T = a.T;
  const int ix = tile % a.ncx, iy = tile / a.ncx;
  const int x0s = ix * T, y0s = iy * T;
  const int tw = min(x0s + T, a.xres) - x0s;
  const int th = min(y0s + T, a.yres) - y0s;
  const float4 *part = g.partial + g.seg_off[o] * (size_t)(T * T) * 2;
  for (int px = threadIdx.x; px < tw * th; px += blockDim.x) {
    const int x = px / th, y = px - (px / th) * th;
    const int lp = (x * T + y) * 2;
    float c0 = 0.f, c1 = 0.f, c2 = 0.f;
    for (uint32_t k = 0; k < nseg; ++k) {
      const float4 v = __ldg(part + (size_t)k * (T * T) * 2 + lp);
      if (ADD) {
        c0 += v.x;
        c1 += v.y;
        c2 += v.z;
      } else {
        const float4 t = __ldg(part + (size_t)k * (T * T) * 2 + lp + 1);
        c0 = fmaf(t.x, c0, v.x);
        c1 = fmaf(t.y, c1, v.y);
        c2 = fmaf(t.z, c2, v.z);
      }
    }
    float *out = a.pic + ((size_t)(x0s + x) * a.yres + (y0s + y)) * 3;
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
  }
}

// Exact fragment count of the reference loop (sum over tile entries of the
// column runs, splotch_host.cc:601-606): the algorithmic work of the splat.
__global__ void __launch_bounds__(256) k_count_fragments(SplatArgs a,
                                                         unsigned long long *total) {
  const int T = a.T;
  const int tile = blockIdx.x;
  const int ix = tile % a.ncx, iy = tile / a.ncx;
  const int x0s = ix * T, y0s = iy * T;
  const int tw = min(x0s + T, a.xres) - x0s;
  const int th = min(y0s + T, a.yres) - y0s;
  const uint32_t start = a.tile_start[tile], end = a.tile_start[tile + 1];
  unsigned long long cnt = 0;
  for (uint32_t jj = start + threadIdx.x; jj < end; jj += blockDim.x) {
    const float4 p = __ldg(a.pos + __ldg(a.entries + jj));
    const float rfacr = fmul(p.z, 0.75f);
    const float posx = fsub(p.x, (float)x0s), posy = fsub(p.y, (float)y0s);
    const int minx = max(f2i(fadd(fsub(posx, rfacr), 1.f)), 0);
    const int maxx = min(f2i(fadd(fadd(posx, rfacr), 1.f)), tw);
    const int miny = max(f2i(fadd(fsub(posy, rfacr), 1.f)), 0);
    const int maxy = min(f2i(fadd(fadd(posy, rfacr), 1.f)), th);
    const float radsq = fmul(rfacr, rfacr);
    for (int x = minx; x < maxx; ++x) {
      const float dx = fsub((float)x, posx);
      const float dy = fsqrt(fsub(radsq, fmul(dx, dx)));
      const int lo = max(miny, f2i(fadd(fsub(posy, dy), 1.f)));
      const int hi = min(maxy, f2i(fadd(fadd(posy, dy), 1.f)));
      if (hi > lo) cnt += (unsigned long long)(hi - lo);
    }
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(total, cnt);
}

template <int NT, int WX, int WY, int B, bool ADD, bool FTB, bool AUX, bool MK>
void launch_one(const SplatArgs &a, size_t sm, cudaStream_t s) {
  auto k = k_splat<NT, WX, WY, B, ADD, FTB, AUX, MK>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<a.ncx * a.ncy, NT, sm, s>>>(a);
}

template <int NT, int WX, int WY, int B, bool MK>
void launch_form(const SplatArgs &a, size_t sm, cudaStream_t s) {
  const bool aux = a.aux != nullptr;
  if (a.a_eq_e)
    launch_one<NT, WX, WY, B, true, false, false, MK>(a, sm, s);
  else if (a.order_mode == 1)
    aux ? launch_one<NT, WX, WY, B, false, true, true, MK>(a, sm, s)
        : launch_one<NT, WX, WY, B, false, true, false, MK>(a, sm, s);
  else
    aux ? launch_one<NT, WX, WY, B, false, false, true, MK>(a, sm, s)
        : launch_one<NT, WX, WY, B, false, false, false, MK>(a, sm, s);
}

// MKOK: tiles of 9 to 16 pixels take the row-mask form of the run table in
// this configuration (its warp boxes start at column 0 or 8, and a pixel
// pair's columns are x < 8 and x + 8).
template <int NT, int WX, int WY, int B, bool MKOK>
int launch_cfg(const SplatArgs &a, cudaStream_t s) {
  const size_t sm = smem_bytes<B>(a.T);
  if (MKOK && a.T > 8 && a.T <= 16)
    launch_form<NT, WX, WY, B, MKOK>(a, sm, s);
  else
    launch_form<NT, WX, WY, B, false>(a, sm, s);
  return 1;
}

// Does a (threads, WX, WY) configuration cover a T x T tile?
bool covers(int T, int nt, int wxi, int wyi) {
  const int nbx = (T + IW - 1) / IW, nby = (T + IH - 1) / IH;
  const int nwx = (nbx + wxi - 1) / wxi, nwy = (nby + wyi - 1) / wyi;
  return nwx * nwy <= nt / 32;
}

}  // namespace

void launch_count_fragments(const SplatArgs &a, unsigned long long *total, cudaStream_t s) {
  cudaMemsetAsync(total, 0, sizeof(unsigned long long), s);
  if (a.ncx * a.ncy > 0) k_count_fragments<<<a.ncx * a.ncy, 256, 0, s>>>(a, total);
}

// Launch configurations (threads per tile, items per warp): the autotuner
// chooses among those that cover the tile size.
int splat_config_count() { return 5; }

bool splat_config_valid(int cfg, int T) {
  switch (cfg) {
    case 0: return covers(T, 256, 1, 1);  // 8 warps x (8x4)
    case 1: return covers(T, 64, 2, 2);   // 2 warps x (16x8)
    case 2: return covers(T, 128, 2, 1);  // 4 warps x (16x4)
    case 3: return covers(T, 256, 2, 2);  // 8 warps x (16x8)
    case 4: return covers(T, 256, 4, 4);  // 8 warps x (32x16)
  }
  return false;
}

// Measured on GB300 (50M-particle absorption frame and 1M additive frame at
// T=16): 4 warps x 16x4 is fastest for both splats (absorption 4.34 ms against
// 5.33 for 2 warps x 16x8 and 7.08 for 8 warps x 8x4; additive 0.30 ms against
// 0.34 for both); larger tiles need the wider configurations.
int splat_default_config(int T, bool /*additive*/) {
  if (splat_config_valid(2, T)) return 2;
  if (splat_config_valid(0, T)) return 0;
  if (splat_config_valid(3, T)) return 3;
  return 4;
}

int launch_splat(const SplatArgs &a, cudaStream_t s) {
  if (a.ncx * a.ncy <= 0) return 0;
  int cfg = a.config >= 0 && splat_config_valid(a.config, a.T)
                ? a.config
                : splat_default_config(a.T, a.a_eq_e != 0);
  switch (cfg) {
    case 0: return launch_cfg<256, 1, 1, 256, true>(a, s);
    case 1: return launch_cfg<64, 2, 2, 128, true>(a, s);
    case 2: return launch_cfg<128, 2, 1, 128, true>(a, s);
    case 3: return launch_cfg<256, 2, 2, 256, false>(a, s);
    default: return launch_cfg<256, 4, 4, 256, false>(a, s);
  }
}

namespace {

template <int NT, int WX, int WY, int B, bool ADD, bool FTB, bool MK>
void launch_seg_one(const SplatArgs &a, const SplatSegs &g, uint32_t grid, cudaStream_t s) {
  const size_t sm = smem_bytes<B>(a.T);
  auto k = k_splat_seg<NT, WX, WY, B, ADD, FTB, MK>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<grid, NT, sm, s>>>(a, g);
}

template <int NT, int WX, int WY, int B, bool MKOK>
void launch_seg_cfg(const SplatArgs &a, const SplatSegs &g, uint32_t grid, cudaStream_t s) {
  const bool mk = MKOK && a.T > 8 && a.T <= 16;
  if (a.a_eq_e)
    mk ? launch_seg_one<NT, WX, WY, B, true, false, MKOK>(a, g, grid, s)
       : launch_seg_one<NT, WX, WY, B, true, false, false>(a, g, grid, s);
  else
    mk ? launch_seg_one<NT, WX, WY, B, false, true, MKOK>(a, g, grid, s)
       : launch_seg_one<NT, WX, WY, B, false, true, false>(a, g, grid, s);
}

}  // namespace

int splat_batch_size(const SplatArgs &a) {
  const int cfg = a.config >= 0 && splat_config_valid(a.config, a.T)
                      ? a.config
                      : splat_default_config(a.T, a.a_eq_e != 0);
  return (cfg == 1 || cfg == 2) ? 128 : 256;
}

int launch_splat_split(const SplatArgs &a, const SplatSegs &g, uint32_t grid, cudaStream_t s) {
  if (a.ncx * a.ncy <= 0) return 0;
  const int cfg = a.config >= 0 && splat_config_valid(a.config, a.T)
                      ? a.config
                      : splat_default_config(a.T, a.a_eq_e != 0);
  switch (cfg) {
    case 0: launch_seg_cfg<256, 1, 1, 256, true>(a, g, grid, s); break;
    case 1: launch_seg_cfg<64, 2, 2, 128, true>(a, g, grid, s); break;
    case 2: launch_seg_cfg<128, 2, 1, 128, true>(a, g, grid, s); break;
    case 3: launch_seg_cfg<256, 2, 2, 256, false>(a, g, grid, s); break;
    default: launch_seg_cfg<256, 4, 4, 256, false>(a, g, grid, s); break;
  }
  if (a.a_eq_e)
    k_splat_combine<true><<<a.ncx * a.ncy, 256, 0, s>>>(a, g);
  else
    k_splat_combine<false><<<a.ncx * a.ncy, 256, 0, s>>>(a, g);
  return 2;
}

namespace {

template <int NT, int WX, int WY, int B, int MODE, bool MK>
int launch_queue_mode(const BatchSplatArgs &q, cudaStream_t s) {
  const size_t sm = smem_bytes<B>(q.T);
  auto k = k_splat_queue<NT, WX, WY, B, MODE, MK>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  int per_sm = 0, dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, NT, sm);
  if (per_sm < 1) per_sm = 1;
  int grid = nsm * per_sm;
  if ((uint32_t)grid > q.nwork) grid = (int)q.nwork;
  if (grid < 1) return 0;
  k<<<grid, NT, sm, s>>>(q);
  return 1;
}

template <int NT, int WX, int WY, int B, bool MK>
int launch_queue_form(const BatchSplatArgs &q, cudaStream_t s) {
  switch (q.mode) {
    case 0: return launch_queue_mode<NT, WX, WY, B, 0, MK>(q, s);
    case 1: return launch_queue_mode<NT, WX, WY, B, 1, MK>(q, s);
    default: return launch_queue_mode<NT, WX, WY, B, 2, MK>(q, s);
  }
}

template <int NT, int WX, int WY, int B, bool MKOK>
int launch_queue_cfg(const BatchSplatArgs &q, cudaStream_t s) {
  return MKOK && q.T > 8 && q.T <= 16 ? launch_queue_form<NT, WX, WY, B, MKOK>(q, s)
                                      : launch_queue_form<NT, WX, WY, B, false>(q, s);
}

}  // namespace

int launch_splat_queue(const BatchSplatArgs &q, int cfg, cudaStream_t s) {
  if (q.nwork == 0) return 0;
  switch (cfg) {
    case 0: return launch_queue_cfg<256, 1, 1, 256, true>(q, s);
    case 1: return launch_queue_cfg<64, 2, 2, 128, true>(q, s);
    case 2: return launch_queue_cfg<128, 2, 1, 128, true>(q, s);
    case 3: return launch_queue_cfg<256, 2, 2, 256, false>(q, s);
    default: return launch_queue_cfg<256, 4, 4, 256, false>(q, s);
  }
}

}  // namespace spl
