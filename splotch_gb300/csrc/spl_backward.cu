// spl_backward.cu -- adjoint of the render path: gradients of a scalar loss L
// with respect to every particle's inputs (I, colour, position, hsml) and the
// camera position, given dL/dpic of a frame rendered by spl_render.  Coverage,
// tile lists and order are those of the forward (their derivative is zero
// almost everywhere).
//
// k_splat_adj -- one CTA per tile with the forward splat's pixel layout (8x4
//   items, one pixel per lane, WX x WY items per warp).  For each fragment a
//   lane forms its pixel's share of six per-particle sums
//     S_E[c] = dL/dE_c,   S_X = sum gatt*att*dx,  S_Y = sum gatt*att*dy,
//     S_D2 = sum gatt*att*(dx^2+dy^2)           (gatt = dL/datt)
//   a warp reduce-scatter adds them over the lanes in eight shuffles, warps
//   add their totals into shared memory, and one vector atomic per (particle,
//   tile) publishes them.  dL/dX = -2*stp*S_X etc. follow in k_project_adj.
//
//   Additive: pic = -sum E*att, so dL/dE_c = -sum g_c*att, gatt = -g.E.
//   Ordered absorption: the list is walked back to front (list order) over
//   exactly the fragments the forward composited -- from the position where
//   the forward's front-to-back pass stopped, stored per pixel with the
//   pixel's optical depth od = sum u by the forward (SplatArgs::aux).  With
//   u = E*att, T = exp(-u), q = E/(E+gray), Tr the transmittance in front of
//   the particle and Tr' = Tr*T behind it, the pixel is
//     C = A_front + Tr*(q*(1-T) + T*Cb)  =>  dC/du = q*Tr' - B,  dC/dq = Tr - Tr'
//   where B = Tr'*Cb is the composite of everything behind.  The lane sums B
//   from the back (small terms first, no cancellation against the image) and
//   the optical depth sb behind and at the particle, and recomputes
//   Tr = exp(-(od - sb)) -- no per-particle intermediate is stored.
//
// k_project_adj -- per active particle, the chain rule through
//   particle_colorize and particle_project (splotch_host.cc:111-153, 270-284):
//     E = col(e) * I * K,  K = bfak*bright*f*s/R,  R = sqrt(r2^2 + minrad^2),
//     r2 = 2*h*f*s,  X = res2 (+xshift) + xc*f,  f = -res2/(fovfct*zc) or xfac,
//     (xc, yc, zc) = A*(p - campos)
//   and block sums of dL/d(xc, yc, zc) and dL/d(X, Y) for the camera position.
#include <algorithm>

#include "spl_tile.cuh"

namespace spl {

namespace {

template <int B>
struct AdjSmem {
  Stage<B> st;
  float4 nw01[B];       // -dq/dE doubled: -w0, -w0, -w1, -w1 (w = gray/(E+gray)^2)
  float2 nw2[B];        // -w2, -w2
  uint32_t idx[B];      // particle index of each slot
  float acc[6][B + 4];  // the batch's per-particle sums; the row pad puts one
                        // particle's six sums in six different banks
  // followed by uint16_t run[B][run_stride(T)]
};

template <int B>
size_t adj_smem_bytes(int T) {
  return sizeof(AdjSmem<B>) + (size_t)B * run_stride(T) * 2;
}

// Warp sum of six values in eight shuffles (reduce-scatter): afterwards lane l
// with (l & 3) == 0 holds the warp total of value j = 3*b4 + 2*b3 + b2 (bits
// 4, 3, 2 of l); j is a pad slot when b3 and b2 are both set.
__device__ __forceinline__ float warp_sum6(const float v[6], int lane, int &j, bool &ok) {
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  float a[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float keep = b4 ? v[i + 3] : v[i];
    const float send = b4 ? v[i] : v[i + 3];
    a[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
  const float k0 = b3 ? a[2] : a[0], k1 = b3 ? 0.f : a[1];
  const float s0 = b3 ? a[0] : a[2], s1 = b3 ? a[1] : 0.f;
  const float c0 = k0 + __shfl_xor_sync(0xffffffffu, s0, 8);
  const float c1 = k1 + __shfl_xor_sync(0xffffffffu, s1, 8);
  float c = (b2 ? c1 : c0) + __shfl_xor_sync(0xffffffffu, b2 ? c0 : c1, 4);
  c += __shfl_xor_sync(0xffffffffu, c, 2);
  c += __shfl_xor_sync(0xffffffffu, c, 1);
  j = (b4 ? 3 : 0) + (b3 ? 2 : 0) + (b2 ? 1 : 0);
  ok = !(b3 && b2);
  return c;
}

// Segments of each tile's list for the adjoint: ceil(len / seg_len), 0 for an
// empty tile.
// (split_min: a tile shorter than this stays one segment.)
// Segments per tile: an empty list has empty_cnt (the adjoint skips it; the
// forward still writes the tile's pixels from one empty segment).
__global__ void k_adj_seg_count(const uint32_t *__restrict__ tile_start, int64_t ntiles,
                                uint32_t seg_len, uint32_t split_min, uint32_t empty_cnt,
                                uint32_t *__restrict__ cnt) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntiles;
       t += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t len = tile_start[t + 1] - tile_start[t];
    cnt[t] = len == 0 ? empty_cnt : len < split_min ? 1u : 1u + (len - 1u) / seg_len;
  }
}

// One CTA per segment of a tile's list (segments numbered in tile order,
// AdjArgs::seg_off); the forward's pixel layout: 8x4 items, WX x WY items per
// warp, pixels processed in pairs (items 2p, 2p+1) with packed arithmetic.
// The ordered 128-thread form is held to 6 CTAs per SM (80 registers): with
// heavy tiles cut into segments it is throughput-bound, and more resident
// warps pay for the few spilled values.  Other forms choose their registers.
// MK: the staged coverage is held as row masks (tiles of 9 to 16 pixels).
template <int NT, int WX, int WY, int B, bool ADD, bool MK>
__global__ void __launch_bounds__(NT, (NT == 128 && !ADD) ? 6 : 0) k_splat_adj(AdjArgs a) {
  constexpr int K = WX * WY;
  constexpr int NP = (K + 1) / 2;
  constexpr int NO = ADD ? 1 : NP;  // ordered-only state
  static_assert(K == 1 || WX % 2 == 0, "the items of a pair share one row");
  extern __shared__ __align__(16) uint8_t smem_raw[];
  AdjSmem<B> &S = *reinterpret_cast<AdjSmem<B> *>(smem_raw);
  Stage<B> &St = S.st;
  uint16_t *srun = reinterpret_cast<uint16_t *>(smem_raw + sizeof(AdjSmem<B>));
  const SplatArgs &f = a.f;
  const int T = f.T, RS = run_stride(T);

  // ---- work item: segment blockIdx.x -> (tile, list range) ----------------
  const uint64_t item = blockIdx.x;
  if (item >= a.seg_off[a.ntiles]) return;
  int o = 0, ohi = (int)a.ntiles;  // seg_off[o] <= item < seg_off[ohi]
  while (ohi - o > 1) {
    const int mid = (o + ohi) >> 1;
    if (a.seg_off[mid] <= item) o = mid; else ohi = mid;
  }
  const int tile = f.tile_order ? (int)__ldg(f.tile_order + o) : o;
  const uint32_t tile_end = f.tile_start[tile + 1];
  const uint32_t kseg = (uint32_t)(item - a.seg_off[o]);  // segment within the tile
  const uint32_t rel0 = kseg * a.seg_len;                  // its first list position
  const uint32_t start = f.tile_start[tile] + rel0;
  const uint32_t end = (uint32_t)min((uint64_t)tile_end, (uint64_t)start + a.seg_len);

  const int ix = tile % f.ncx, iy = tile / f.ncx;
  const int x0s = ix * T, y0s = iy * T;
  const int tw = min(x0s + T, f.xres) - x0s;
  const int th = min(y0s + T, f.yres) - y0s;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;

  const int nbx = (tw + IW - 1) / IW, nby = (th + IH - 1) / IH;
  const int nwx = (nbx + WX - 1) / WX, nwy = (nby + WY - 1) / WY;
  const int wx = w % nwx, wy = w / nwx;
  const bool warp_has_pixels = wy < nwy;
  const int wbx0 = wx * WX * IW, wby0 = wy * WY * IH;
  const int wbx1 = min(wbx0 + WX * IW, tw), wby1 = min(wby0 + WY * IH, th);

  // g: dL/dpic; od: the forward's optical depth; sb: optical depth behind
  // and at the current particle; nbg: minus the composite behind it
  int col[K], row[K];
  uint32_t rbit[K];  // the row's bit (0 outside the tile)
  F2 px2[NP], py2[NP];
  F2 g[NP][3], od[NO][3], sb[NO][3], nbg[NO][3];
  uint32_t mystop = 0xffffffffu;
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
    float gv[2][3], ov[2][3];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = 2 * p + h;
      const bool valid = k < K && row[k < K ? k : 0] != 255;
      const size_t pix = (size_t)(x0s + x + h * IW) * f.yres + (y0s + y);
      float4 ax = make_float4(0.f, 0.f, 0.f, 0.f);
      if (!ADD && valid) {
        ax = __ldg(f.aux + pix);
        mystop = min(mystop, __float_as_uint(ax.w));
      }
      ov[h][0] = ax.x;
      ov[h][1] = ax.y;
      ov[h][2] = ax.z;
#pragma unroll
      for (int c = 0; c < 3; ++c) gv[h][c] = valid ? __ldg(a.gpic + pix * 3 + c) : 0.f;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      g[p][c] = f2(gv[0][c], gv[1][c]);
      if (!ADD) {
        od[ADD ? 0 : p][c] = f2(ov[0][c], ov[1][c]);
        sb[ADD ? 0 : p][c] = f2(0.f);
        nbg[ADD ? 0 : p][c] = f2(0.f);
      }
    }
  }

  // A later segment of a split ordered tile starts from the state the walk
  // would have reached: per earlier segment i (back to front) its optical depth
  // U_i and its own back-to-front composite V_i (k_adj_ordered_state), so
  // sb = sum U_i and bg = sum Tr_i*V_i with Tr_i = exp(-(od - sb after i)).
  if (!ADD && kseg > 0) {
    const float4 *st = a.seg_state + (size_t)a.seg_off[o] * (size_t)(T * T) * 2;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      float sbv[2][3] = {}, nbv[2][3] = {};
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int k = 2 * p + h;
        if (k >= K || row[k < K ? k : 0] == 255) continue;
        const int px = (col[k] * T + row[k]) * 2;
        const float odv[3] = {h ? f2hi(od[ADD ? 0 : p][0]) : f2lo(od[ADD ? 0 : p][0]),
                              h ? f2hi(od[ADD ? 0 : p][1]) : f2lo(od[ADD ? 0 : p][1]),
                              h ? f2hi(od[ADD ? 0 : p][2]) : f2lo(od[ADD ? 0 : p][2])};
        for (uint32_t i = 0; i < kseg; ++i) {
          const float4 U = __ldg(st + (size_t)i * (T * T) * 2 + px);
          const float4 V = __ldg(st + (size_t)i * (T * T) * 2 + px + 1);
          const float u3[3] = {U.x, U.y, U.z}, v3[3] = {V.x, V.y, V.z};
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            sbv[h][c] += u3[c];
            nbv[h][c] = fmaf(-ex2((sbv[h][c] - odv[c]) * kLog2e), v3[c], nbv[h][c]);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sb[ADD ? 0 : p][c] = f2(sbv[0][c], sbv[1][c]);
        nbg[ADD ? 0 : p][c] = f2(nbv[0][c], nbv[1][c]);
      }
    }
  }

  const int nbatch = (int)((end - start + B - 1) / B);
  // Ordered frames: the forward composited, per warp, list positions
  // [stop, end) of the tile (stop a multiple of B); walk exactly those, in list
  // order (back to front).  Positions are compared relative to the tile's
  // list start (the segment starts at rel0).
  __shared__ uint32_t s_first;
  uint32_t wstop = 0;
  if (!ADD) {
    wstop = __reduce_min_sync(0xffffffffu, mystop);
    if (threadIdx.x == 0) s_first = 0xffffffffu;
    __syncthreads();
    if (lane == 0 && warp_has_pixels) atomicMin(&s_first, wstop);
    __syncthreads();
  }
  const int b_first =
      ADD ? 0 : (int)min((uint32_t)nbatch, s_first > rel0 ? (s_first - rel0) / (uint32_t)B : 0u);
  const bool warp_idle = !warp_has_pixels;

  for (int bi = b_first; bi < nbatch; ++bi) {
    // ---- stage B particles (as the forward, plus dq/dE and the index) ----
#pragma unroll 1
    for (int slot = threadIdx.x; slot < B; slot += NT) {
      float4 c;
      const uint32_t idx = stage_entry<B, ADD, false, MK>(St, srun, RS, slot, f,
                                                          start + (uint32_t)bi * B + slot, end,
                                                          x0s, y0s, tw, th, &c);
      if (!ADD && idx != 0xffffffffu) {
        const float d0 = fadd(c.x, f.gray), d1 = fadd(c.y, f.gray), d2 = fadd(c.z, f.gray);
        const float w0 = -(f.gray / (d0 * d0)), w1 = -(f.gray / (d1 * d1));
        const float w2 = -(f.gray / (d2 * d2));
        S.nw01[slot] = make_float4(w0, w0, w1, w1);
        S.nw2[slot] = make_float2(w2, w2);
      }
      S.idx[slot] = idx;
#pragma unroll
      for (int j = 0; j < 6; ++j) S.acc[j][slot] = 0.f;
    }
    __syncthreads();
    // ---- per-fragment adjoint ----------------------------------------------
    if (!warp_idle && (ADD || rel0 + (uint32_t)bi * B >= wstop)) {
#pragma unroll 1
      for (int ch = 0; ch < B / 32; ++ch) {
        const bool hit = box_meets_warp(St.bb[ch * 32 + lane], wbx0, wbx1, wby0, wby1);
        uint32_t mask = __ballot_sync(0xffffffffu, hit);
        while (mask) {
          const int bit = __ffs(mask) - 1;
          mask &= ~(1u << bit);
          const int j = ch * 32 + bit;
          const float4 pxy = St.pxy[j];
          const float4 es = St.es[j];
          const float4 e12 = St.e12[j];
          float4 q01 = make_float4(0.f, 0.f, 0.f, 0.f), nw01 = q01;
          float2 q2 = make_float2(0.f, 0.f), nw2 = q2;
          if (!ADD) {
            q01 = St.q01[j];
            q2 = St.q2[j];
            nw01 = S.nw01[j];
            nw2 = S.nw2[j];
          }
          uint32_t bbj = 0;
          if (NP > 1) bbj = St.bb[j];
          const uint16_t *run = srun + j * RS;
          F2 sm[6];
#pragma unroll
          for (int i = 0; i < 6; ++i) sm[i] = f2(0.f);
          bool any = false;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            if (NP > 1 && !box_meets_pair(bbj, wbx0 + ((2 * p) % WX) * IW,
                                          wby0 + ((2 * p) / WX) * IH))
              continue;
            const int k1 = 2 * p + 1 < K ? 2 * p + 1 : 0;
            bool in0, in1;
            covered_pair<MK>(run, col[2 * p], row[2 * p], rbit[2 * p], 2 * p + 1 < K, col[k1],
                             row[k1], rbit[k1], in0, in1);
            // additive: lanes without a covered pixel skip; ordered: every lane
            // runs the terms (they vanish), so that the warp can vote on the
            // Taylor range of expm1 below
            if (ADD && !(in0 || in1)) continue;
            any = any || in0 || in1;
            // an uncovered pixel of the pair gets att = 0 (and g = 0 outside
            // the tile): its terms vanish
            const F2 dx = sub2(px2[p], f2(pxy.x, pxy.y));
            const F2 dy = sub2(py2[p], f2(pxy.z, pxy.w));
            const F2 d2 = fma2(dy, dy, mul2(dx, dx));
            const F2 arg = mul2(f2(es.z, es.w), d2);
            const F2 att = f2(in0 ? ex2(f2lo(arg)) : 0.f, in1 ? ex2(f2hi(arg)) : 0.f);
            const F2 e[3] = {f2(es.x, es.y), f2(e12.x, e12.y), f2(e12.z, e12.w)};
            F2 gatt;
            if (ADD) {
              // pic = -sum E*att (e staged negated): dL/dE_c = -sum g_c*att
              // (negated at the reduction), gatt = -g.E
#pragma unroll
              for (int c = 0; c < 3; ++c) sm[c] = fma2(g[p][c], att, sm[c]);
              gatt = fma2(g[p][0], e[0], fma2(g[p][1], e[1], mul2(g[p][2], e[2])));
            } else {
              const F2 q[3] = {f2(q01.x, q01.y), f2(q01.z, q01.w), f2(q2.x, q2.y)};
              const F2 nw[3] = {f2(nw01.x, nw01.y), f2(nw01.z, nw01.w), f2(nw2.x, nw2.y)};
              gatt = f2(0.f);
              F2 u[3];
#pragma unroll
              for (int c = 0; c < 3; ++c) u[c] = mul2(e[c], att);  // u as the forward forms it
              const float um =
                  fmaxf(fmaxf(fmaxf(f2lo(u[0]), f2hi(u[0])), fmaxf(f2lo(u[1]), f2hi(u[1]))),
                        fmaxf(f2lo(u[2]), f2hi(u[2])));
              const bool poly = __all_sync(0xffffffffu, um < kExpm1TaylorCut);
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                F2 &sbc = sb[ADD ? 0 : p][c], &nbgc = nbg[ADD ? 0 : p][c];
                // transmittance in front of the particle from the stored
                // optical depth, Tr = exp(-(od - sb))
                sbc = add2(sbc, u[c]);
                const F2 ta = mul2(sub2(sbc, od[ADD ? 0 : p][c]), f2(kLog2e));
                const F2 trm = f2(ex2(f2lo(ta)), ex2(f2hi(ta)));
                const F2 nwt =
                    mul2(trm, poly ? expm1_neg2_poly(u[c]) : expm1_neg2(u[c]));  // -(Tr - Tr')
                const F2 trn = add2(trm, nwt);            // Tr' = Tr*T
                // dC/du = q*Tr' - B, dC/dq = Tr - Tr'  (B: composite behind)
                const F2 ga = mul2(g[p][c], fma2(q[c], trn, nbgc));
                sm[c] = fma2(ga, att, fma2(mul2(g[p][c], nwt), nw[c], sm[c]));
                gatt = fma2(ga, e[c], gatt);
                nbgc = fma2(nwt, q[c], nbgc);
              }
            }
            const F2 ga2 = mul2(gatt, att);
            sm[3] = fma2(ga2, dx, sm[3]);
            sm[4] = fma2(ga2, dy, sm[4]);
            sm[5] = fma2(ga2, d2, sm[5]);
          }
          if (__any_sync(0xffffffffu, any)) {
            float v[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) {
              v[i] = f2lo(sm[i]) + f2hi(sm[i]);
              if (ADD && i < 3) v[i] = -v[i];
            }
            int jj;
            bool ok;
            const float tot = warp_sum6(v, lane, jj, ok);
            if ((lane & 3) == 0 && ok) atomicAdd(&S.acc[jj][j], tot);
          }
        }
      }
    }
    __syncthreads();
    // ---- publish this batch's sums (each slot by the thread that staged it)
#pragma unroll 1
    for (int slot = threadIdx.x; slot < B; slot += NT) {
      const uint32_t idx = S.idx[slot];
      if (idx == 0xffffffffu) continue;
      const float4 ge = make_float4(S.acc[0][slot], S.acc[1][slot], S.acc[2][slot], 0.f);
      const float4 gp = make_float4(S.acc[3][slot], S.acc[4][slot], S.acc[5][slot], 0.f);
      if (ge.x != 0.f || ge.y != 0.f || ge.z != 0.f) atomicAdd(a.gcol + idx, ge);
      if (gp.x != 0.f || gp.y != 0.f || gp.z != 0.f) atomicAdd(a.gpos + idx, gp);
    }
  }
}

// Pass 1 for split ordered tiles: for every segment but a tile's last, per
// pixel, the optical depth U of the fragments the forward composited in it
// and their own back-to-front composite V (V <- V*T + q*(1-T), from 0), into
// seg_state[segment][pixel] = (U, V).  Same item mapping and pixel layout as
// k_splat_adj.
template <int NT, int WX, int WY, int B, bool MK>
__global__ void __launch_bounds__(NT) k_adj_ordered_state(AdjArgs a) {
  constexpr int K = WX * WY;
  constexpr int NP = (K + 1) / 2;
  extern __shared__ __align__(16) uint8_t smem_raw[];
  Stage<B> &St = *reinterpret_cast<Stage<B> *>(smem_raw);
  uint16_t *srun = reinterpret_cast<uint16_t *>(smem_raw + sizeof(Stage<B>));
  const SplatArgs &f = a.f;
  const int T = f.T, RS = run_stride(T);
  const uint64_t item = blockIdx.x;
  if (item >= a.seg_off[a.ntiles]) return;
  int o = 0, ohi = (int)a.ntiles;
  while (ohi - o > 1) {
    const int mid = (o + ohi) >> 1;
    if (a.seg_off[mid] <= item) o = mid; else ohi = mid;
  }
  const uint32_t kseg = (uint32_t)(item - a.seg_off[o]);
  if (kseg + 1 >= (uint32_t)(a.seg_off[o + 1] - a.seg_off[o])) return;  // last: not needed
  const int tile = f.tile_order ? (int)__ldg(f.tile_order + o) : o;
  const uint32_t rel0 = kseg * a.seg_len;
  const uint32_t start = f.tile_start[tile] + rel0;
  const uint32_t end = (uint32_t)min((uint64_t)f.tile_start[tile + 1], (uint64_t)start + a.seg_len);
  const int ix = tile % f.ncx, iy = tile / f.ncx;
  const int x0s = ix * T, y0s = iy * T;
  const int tw = min(x0s + T, f.xres) - x0s;
  const int th = min(y0s + T, f.yres) - y0s;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nbx = (tw + IW - 1) / IW, nby = (th + IH - 1) / IH;
  const int nwx = (nbx + WX - 1) / WX, nwy = (nby + WY - 1) / WY;
  const int wx = w % nwx, wy = w / nwx;
  const bool warp_has_pixels = wy < nwy;
  const int wbx0 = wx * WX * IW, wby0 = wy * WY * IH;
  const int wbx1 = min(wbx0 + WX * IW, tw), wby1 = min(wby0 + WY * IH, th);

  int col[K], row[K];
  uint32_t rbit[K];
  F2 px2[NP], py2[NP], U[NP][3], V[NP][3];
  uint32_t mystop = 0xffffffffu;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int x = wbx0 + (k % WX) * IW + (lane & 7);
    const int y = wby0 + (k / WX) * IH + (lane >> 3);
    const bool valid = warp_has_pixels && x < tw && y < th;
    col[k] = valid ? x : 0;
    row[k] = valid ? y : 255;
    rbit[k] = valid ? 1u << y : 0u;
    if (valid)
      mystop = min(mystop, __float_as_uint(
                               __ldg(f.aux + (size_t)(x0s + x) * f.yres + (y0s + y)).w));
  }
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    const int x = wbx0 + ((2 * p) % WX) * IW + (lane & 7);
    const int y = wby0 + ((2 * p) / WX) * IH + (lane >> 3);
    px2[p] = f2((float)x, (float)(x + IW));
    py2[p] = f2((float)y);
#pragma unroll
    for (int c = 0; c < 3; ++c) U[p][c] = V[p][c] = f2(0.f);
  }
  const uint32_t wstop = __reduce_min_sync(0xffffffffu, mystop);
  const int nbatch = (int)((end - start + B - 1) / B);
  for (int bi = 0; bi < nbatch; ++bi) {
#pragma unroll 1
    for (int slot = threadIdx.x; slot < B; slot += NT)
      stage_entry<B, false, false, MK>(St, srun, RS, slot, f, start + (uint32_t)bi * B + slot,
                                       end, x0s, y0s, tw, th);
    __syncthreads();
    if (warp_has_pixels && rel0 + (uint32_t)bi * B >= wstop) {
#pragma unroll 1
      for (int ch = 0; ch < B / 32; ++ch) {
        const bool hit = box_meets_warp(St.bb[ch * 32 + lane], wbx0, wbx1, wby0, wby1);
        uint32_t mask = __ballot_sync(0xffffffffu, hit);
        while (mask) {
          const int bit = __ffs(mask) - 1;
          mask &= ~(1u << bit);
          const int j = ch * 32 + bit;
          const float4 pxy = St.pxy[j], es = St.es[j], e12 = St.e12[j];
          const float4 q01 = St.q01[j];
          const float2 q2 = St.q2[j];
          uint32_t bbj = 0;
          if (NP > 1) bbj = St.bb[j];
          const uint16_t *run = srun + j * RS;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            if (NP > 1 && !box_meets_pair(bbj, wbx0 + ((2 * p) % WX) * IW,
                                          wby0 + ((2 * p) / WX) * IH))
              continue;
            const int k1 = 2 * p + 1 < K ? 2 * p + 1 : 0;
            bool in0, in1;
            covered_pair<MK>(run, col[2 * p], row[2 * p], rbit[2 * p], 2 * p + 1 < K, col[k1],
                             row[k1], rbit[k1], in0, in1);
            if (!(in0 || in1)) continue;
            const F2 dx = sub2(px2[p], f2(pxy.x, pxy.y));
            const F2 dy = sub2(py2[p], f2(pxy.z, pxy.w));
            const F2 arg = mul2(f2(es.z, es.w), fma2(dy, dy, mul2(dx, dx)));
            const F2 att = f2(in0 ? ex2(f2lo(arg)) : 0.f, in1 ? ex2(f2hi(arg)) : 0.f);
            const F2 e[3] = {f2(es.x, es.y), f2(e12.x, e12.y), f2(e12.z, e12.w)};
            const F2 q[3] = {f2(q01.x, q01.y), f2(q01.z, q01.w), f2(q2.x, q2.y)};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const F2 u = mul2(e[c], att);
              U[p][c] = add2(U[p][c], u);
              V[p][c] = fma2(expm1_neg2(u), sub2(V[p][c], q[c]), V[p][c]);
            }
          }
        }
      }
    }
    __syncthreads();
  }
  float4 *st = a.seg_state + (size_t)item * (size_t)(T * T) * 2;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (row[k] == 255) continue;
    float u3[3], v3[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      u3[c] = (k & 1) ? f2hi(U[k / 2][c]) : f2lo(U[k / 2][c]);
      v3[c] = (k & 1) ? f2hi(V[k / 2][c]) : f2lo(V[k / 2][c]);
    }
    const int px = (col[k] * T + row[k]) * 2;
    st[px] = make_float4(u3[0], u3[1], u3[2], 0.f);
    st[px + 1] = make_float4(v3[0], v3[1], v3[2], 0.f);
  }
}

template <int NT, int WX, int WY, int B, bool MK>
void launch_adj_form(const AdjArgs &a, uint32_t grid, cudaStream_t s) {
  const size_t sm = adj_smem_bytes<B>(a.f.T);
  if (a.f.a_eq_e) {
    auto k = k_splat_adj<NT, WX, WY, B, true, MK>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k<<<grid, NT, sm, s>>>(a);
  } else {
    if (a.seg_len != 0xffffffffu) {  // split ordered tiles: the state pass first
      auto k1 = k_adj_ordered_state<NT, WX, WY, B, MK>;
      const size_t sm1 = sizeof(Stage<B>) + (size_t)B * run_stride(a.f.T) * 2;
      cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
      k1<<<grid, NT, sm1, s>>>(a);
    }
    auto k = k_splat_adj<NT, WX, WY, B, false, MK>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k<<<grid, NT, sm, s>>>(a);
  }
}

// MKOK: tiles of 9 to 16 pixels take row masks in this configuration (warp
// boxes at column 0 or 8).
template <int NT, int WX, int WY, int B, bool MKOK>
void launch_adj_cfg(const AdjArgs &a, uint32_t grid, cudaStream_t s) {
  if (MKOK && a.f.T > 8 && a.f.T <= 16)
    launch_adj_form<NT, WX, WY, B, MKOK>(a, grid, s);
  else
    launch_adj_form<NT, WX, WY, B, false>(a, grid, s);
}

// ---- chain rule through colourisation and projection ------------------------

struct RawIn {
  float er, eg, eb, x, y, z, r, I;
  int type;
};

__device__ __forceinline__ RawIn load_raw(const ProjAdjArgs &a, int64_t i) {
  RawIn in;
  if (a.aos) {
    const uint8_t *rec = static_cast<const uint8_t *>(a.aos) + i * 36;
    const float *f = reinterpret_cast<const float *>(rec);
    in.er = __ldg(f + 0); in.eg = __ldg(f + 1); in.eb = __ldg(f + 2);
    in.x = __ldg(f + 3); in.y = __ldg(f + 4); in.z = __ldg(f + 5);
    in.r = __ldg(f + 6); in.I = __ldg(f + 7);
    in.type = __ldg(reinterpret_cast<const unsigned short *>(rec + 32));
  } else {
    const SoAIn &s = a.soa;
    in.x = __ldg(s.x + i); in.y = __ldg(s.y + i); in.z = __ldg(s.z + i);
    in.r = __ldg(s.r + i); in.I = __ldg(s.I + i);
    in.er = __ldg(s.cr + i);
    in.eg = s.cg ? __ldg(s.cg + i) : 0.f;
    in.eb = s.cb ? __ldg(s.cb + i) : 0.f;
    in.type = s.type ? (int)__ldg(s.type + i) : 0;
  }
  return in;
}

// piecewise-linear colour map and its slope (linear_map.h:71-84)
__device__ __forceinline__ void palette_slope(const ProjConst &c, int t, float v, float col[3],
                                              float dcol[3]) {
  const int n = c.pal_n[t];
  const double *x = c.pal_x + c.pal_off[t];
  const float *rgb = c.pal_rgb + 3 * c.pal_off[t];
  const double vd = v;
  int idx;
  if (n == 1 || vd <= x[0] || vd >= x[n - 1]) {
    idx = (n == 1 || vd <= x[0]) ? 0 : n - 1;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      col[k] = rgb[3 * idx + k];
      dcol[k] = 0.f;
    }
    return;
  }
  int lo = 0, hi = n;  // lower_bound
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (x[mid] < vd) lo = mid + 1; else hi = mid;
  }
  idx = lo > 0 ? lo - 1 : 0;
  if (idx > n - 2) idx = n - 2;
  const double span = x[idx + 1] - x[idx];
  const float frac = (float)((vd - x[idx]) / span);
  const float inv = (float)(1.0 / span);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float r0 = rgb[3 * idx + k], r1 = rgb[3 * (idx + 1) + k];
    col[k] = r0 + (r1 - r0) * frac;
    dcol[k] = (r1 - r0) * inv;
  }
}

__global__ void __launch_bounds__(256) k_project_adj(ProjAdjArgs a) {
  const ProjConst &c = a.c;
  double part[5] = {0., 0., 0., 0., 0.};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.na;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t idx = __ldg(a.idx_c + i);
    const RawIn in = load_raw(a, idx);
    const float4 pp = __ldg(a.pos_c + i);
    const float4 gp = a.gpos[i], ge = a.gcol[i];
    const int t = min(max(in.type, 0), SPL_MAXT - 1);
    // camera-space position (the forward's transform, in double)
    const double px = in.x, py = in.y, pz = in.z;
    const float *m = c.mat;
    const float xc = (float)(px * m[0] + py * m[1] + pz * m[2] + m[3]);
    const float yc = (float)(px * m[4] + py * m[5] + pz * m[6] + m[7]);
    const float zc = (float)(px * m[8] + py * m[9] + pz * m[10] + m[11]);
    const float fz = c.projection ? -c.res2 / (c.fovfct * zc) : c.xfac;
    const float sm = c.smooth[t];
    const float r2 = 2.f * in.r * fz * sm;
    const float R = sqrtf(r2 * r2 + c.minrad2);
    const float K = 2.f * c.half_bfak * c.bright[t] * fz * sm / R;
    float col[3], dcol[3];
    if (c.colvec[t]) {
      col[0] = in.er; col[1] = in.eg; col[2] = in.eb;
      dcol[0] = dcol[1] = dcol[2] = 0.f;
    } else {
      palette_slope(c, t, in.er, col, dcol);
    }
    // splat sums -> d/d(X, Y, R) with the forward's Gaussian width
    const float sig = a.h2sigma * pp.z;
    const float m2stp = 2.f / (sig * sig);  // -2*stp
    const float gX = m2stp * gp.x, gY = m2stp * gp.y, gR = m2stp * gp.z / pp.z;
    const float gE[3] = {ge.x, ge.y, ge.z};
    float gK = 0.f, gI = 0.f, gcol[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      gK = fmaf(gE[k] * col[k], in.I, gK);
      gI = fmaf(gE[k] * col[k], K, gI);
      gcol[k] = gE[k] * in.I * K;
    }
    const float gRt = gR - gK * K / R;
    float gf = gK * K / fz;
    const float gr2 = gRt * r2 / R;
    const float gh = gr2 * 2.f * fz * sm;
    gf = fmaf(gr2 * 2.f * in.r, sm, gf);
    gf = fmaf(gX, xc, fmaf(gY, yc, gf));
    const float gxc = gX * fz, gyc = gY * fz;
    const float gzc = c.projection ? gf * (-fz / zc) : 0.f;
    const float gwx = m[0] * gxc + m[4] * gyc + m[8] * gzc;
    const float gwy = m[1] * gxc + m[5] * gyc + m[9] * gzc;
    const float gwz = m[2] * gxc + m[6] * gyc + m[10] * gzc;
    if (a.gI) a.gI[idx] = gI;
    if (c.colvec[t]) {
      if (a.gcr) a.gcr[idx] = gcol[0];
      if (a.gcg) a.gcg[idx] = gcol[1];
      if (a.gcb) a.gcb[idx] = gcol[2];
    } else if (a.gcr) {
      a.gcr[idx] = gcol[0] * dcol[0] + gcol[1] * dcol[1] + gcol[2] * dcol[2];
    }
    if (a.gx) a.gx[idx] = gwx;
    if (a.gy) a.gy[idx] = gwy;
    if (a.gz) a.gz[idx] = gwz;
    if (a.gr) a.gr[idx] = gh;
    part[0] += gxc;
    part[1] += gyc;
    part[2] += gzc;
    part[3] += gX;
    part[4] += gY;
  }
  // block sums for the camera position
  __shared__ double red[5][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    double v = part[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[k][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    double v = 0.;
    for (int ww = 0; ww < (int)(blockDim.x >> 5); ++ww) v += red[threadIdx.x][ww];
    atomicAdd(a.cam_sums + threadIdx.x, v);
  }
}

}  // namespace

namespace {

// The ordered adjoint walks the forward's warps (it reads where each warp
// stopped); the additive one takes its own layout, four warps of 16x4
// pixels, which shares each hit's reduction among 64 pixels.
int adjoint_cfg(const SplatArgs &f) {
  const bool add = f.a_eq_e != 0;
  const int fwd_cfg = f.config >= 0 && splat_config_valid(f.config, f.T)
                          ? f.config
                          : splat_default_config(f.T, add);
  return add && splat_config_valid(2, f.T) ? 2 : fwd_cfg;
}

}  // namespace

// Segments of about 1/16 of an SM's share of the frame's entries (at least
// four batches), so that the heaviest tiles spread over many SMs.
uint32_t adjoint_seg_len(const SplatArgs &f, int64_t n_entries) {
  const int cfg = adjoint_cfg(f);
  const int64_t B = (cfg == 1 || cfg == 2) ? 128 : 256;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int64_t per = (n_entries + (int64_t)nsm * 16 - 1) / ((int64_t)nsm * 16);
  int64_t L = (per + B - 1) / B * B;
  if (L < 4 * B) L = 4 * B;
  if (L > 0x40000000) L = 0x40000000;
  return (uint32_t)L;
}

int launch_splat_adjoint(const AdjArgs &a0, cudaStream_t s) {
  const int64_t ntiles = (int64_t)a0.f.ncx * a0.f.ncy;
  if (ntiles <= 0) return 0;
  AdjArgs a = a0;
  const bool add = a.f.a_eq_e != 0;
  const int T = a.f.T;
  const int cfg = adjoint_cfg(a.f);
  uint32_t seg_len = adjoint_seg_len(a.f, a.n_entries);
  // segments <= sum over tiles of (len / seg_len + 1)
  int64_t grid64 = ntiles + a.n_entries / seg_len + 1;
  // ordered tiles split only with room for the state of every segment
  if (!add && (!a.seg_state || (size_t)grid64 * (size_t)(T * T) * 2 > a.seg_state_cap)) {
    seg_len = 0xffffffffu;
    grid64 = ntiles + 1;
  }
  a.ntiles = ntiles;
  a.seg_len = seg_len;
  int launches = 1;
  int cb = (int)std::min<int64_t>((ntiles + 255) / 256, 152 * 8);
  k_adj_seg_count<<<cb, 256, 0, s>>>(a.f.tile_start, ntiles, seg_len, 0u, 0u, a.seg_cnt);
  scan_counts(a.seg_cnt, a.f.tile_order, ntiles, a.seg_off, a.scan_scratch, s, &launches);
  const uint32_t grid = (uint32_t)std::min<int64_t>(grid64, 0x7fffffff);
  switch (cfg) {
    case 0: launch_adj_cfg<256, 1, 1, 256, true>(a, grid, s); break;
    case 1: launch_adj_cfg<64, 2, 2, 128, true>(a, grid, s); break;
    case 2: launch_adj_cfg<128, 2, 1, 128, true>(a, grid, s); break;
    case 3: launch_adj_cfg<256, 2, 2, 256, false>(a, grid, s); break;
    default: launch_adj_cfg<256, 4, 4, 256, false>(a, grid, s); break;
  }
  return launches + (!add && seg_len != 0xffffffffu ? 2 : 1);
}

void launch_seg_count(const uint32_t *tile_start, int64_t ntiles, uint32_t seg_len,
                      uint32_t split_min, uint32_t *cnt, cudaStream_t s) {
  if (ntiles <= 0) return;
  const int cb = (int)std::min<int64_t>((ntiles + 255) / 256, 152 * 8);
  // every tile of the forward has a segment: an empty one writes zeros
  k_adj_seg_count<<<cb, 256, 0, s>>>(tile_start, ntiles, seg_len, split_min, 1u, cnt);
}

int launch_project_adjoint(const ProjAdjArgs &a, cudaStream_t s) {
  if (a.na <= 0) return 0;
  int blocks = (int)((a.na + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_project_adj<<<blocks, 256, 0, s>>>(a);
  return 1;
}

}  // namespace spl
