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
#include "spl_internal.cuh"

namespace spl {

namespace {

constexpr int IW = 8, IH = 4;

template <int B>
struct AdjSmem {
  float4 p0[B];   // posx, posy, stp*log2e, bbox bits
  float4 e[B];    // E.r, E.g, E.b, q.r
  float2 q[B];    // q.g, q.b
  float4 wq[B];   // dq/dE per channel: gray/(E+gray)^2
  float acc[6][B];
  uint32_t idx[B];
  // followed by uint16_t run[B*T]
};

template <int B>
size_t adj_smem_bytes(int T) {
  return sizeof(AdjSmem<B>) + (size_t)B * T * 2;
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

template <int NT, int WX, int WY, int B, bool ADD>
__global__ void __launch_bounds__(NT) k_splat_adj(AdjArgs a) {
  constexpr int K = WX * WY;
  extern __shared__ __align__(16) uint8_t smem_raw[];
  AdjSmem<B> &S = *reinterpret_cast<AdjSmem<B> *>(smem_raw);
  uint16_t *srun = reinterpret_cast<uint16_t *>(smem_raw + sizeof(AdjSmem<B>));
  const SplatArgs &f = a.f;

  const int T = f.T;
  const int tile = f.tile_order ? (int)__ldg(f.tile_order + blockIdx.x) : (int)blockIdx.x;
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

  float pxf[K], pyf[K];
  int pxi[K], pyi[K];
  bool valid[K];
  // g: dL/dpic; od: the forward's optical depth; sb: optical depth behind
  // and at the current particle; bg: composite contribution behind it
  float g[K][3], od[K][3], sb[K][3], bg[K][3];
  uint32_t mystop = 0xffffffffu;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int x = wbx0 + (k % WX) * IW + (lane & 7);
    const int y = wby0 + (k / WX) * IH + (lane >> 3);
    valid[k] = warp_has_pixels && x < tw && y < th;
    pxi[k] = x;
    pyi[k] = y;
    pxf[k] = (float)x;
    pyf[k] = (float)y;
    const size_t pix = (size_t)(x0s + x) * f.yres + (y0s + y);
    float4 ax = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!ADD && valid[k]) {
      ax = __ldg(f.aux + pix);
      mystop = min(mystop, __float_as_uint(ax.w));
    }
    od[k][0] = ax.x;
    od[k][1] = ax.y;
    od[k][2] = ax.z;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      g[k][c] = valid[k] ? __ldg(a.gpic + pix * 3 + c) : 0.f;
      sb[k][c] = 0.f;
      bg[k][c] = 0.f;
    }
  }

  const uint32_t start = f.tile_start[tile], end = f.tile_start[tile + 1];
  const int nbatch = (int)((end - start + B - 1) / B);
  // Ordered frames: the forward composited, per warp, list positions
  // [stop, end) (a multiple of B); walk exactly those, in list order (back to
  // front).  Additive frames: the whole list.
  __shared__ uint32_t s_first;
  uint32_t wstop = 0;
  if (!ADD) {
    wstop = __reduce_min_sync(0xffffffffu, mystop);
    if (threadIdx.x == 0) s_first = 0xffffffffu;
    __syncthreads();
    if (lane == 0 && warp_has_pixels) atomicMin(&s_first, wstop);
    __syncthreads();
  }
  const int b_first = ADD ? 0 : (int)min((uint32_t)nbatch, s_first / (uint32_t)B);
  const bool warp_idle = !warp_has_pixels;

  for (int bi = b_first; bi < nbatch; ++bi) {
    // ---- stage B particles (as the forward, plus dq/dE and the index) ----
#pragma unroll 1
    for (int slot = threadIdx.x; slot < B; slot += NT) {
      const uint32_t jj = start + (uint32_t)bi * B + slot;
      uint32_t bb = 0, idx = 0xffffffffu;
      float4 p0 = make_float4(0.f, 0.f, 0.f, 0.f);
      if (jj < end) {
        idx = __ldg(f.entries + jj);
        const float4 p = __ldg(f.pos + idx);
        const float4 c = __ldg(f.col + idx);
        const float rfacr = fmul(p.z, 0.75f);
        const float posx = fsub(p.x, (float)x0s), posy = fsub(p.y, (float)y0s);
        const int minx = max(f2i(fadd(fsub(posx, rfacr), 1.f)), 0);
        const int maxx = min(f2i(fadd(fadd(posx, rfacr), 1.f)), tw);
        const int miny = max(f2i(fadd(fsub(posy, rfacr), 1.f)), 0);
        const int maxy = min(f2i(fadd(fadd(posy, rfacr), 1.f)), th);
        const float radsq = fmul(rfacr, rfacr);
        const float sigma = fmul(f.h2sigma, p.z);
        const float stp = fdiv(-1.f, fmul(sigma, sigma));
        if (minx < maxx && miny < maxy) {
          bb = (uint32_t)minx | ((uint32_t)maxx << 8) | ((uint32_t)miny << 16) |
               ((uint32_t)maxy << 24);
          uint16_t *run = srun + slot * T;
          for (int x = minx; x < maxx; ++x) {
            const float dx = fsub((float)x, posx);
            const float dy = fsqrt(fsub(radsq, fmul(dx, dx)));
            const int lo = max(miny, f2i(fadd(fsub(posy, dy), 1.f)));
            int hi = min(maxy, f2i(fadd(fadd(posy, dy), 1.f)));
            if (hi < lo) hi = lo;
            run[x] = (uint16_t)(lo | (hi << 8));
          }
        }
        p0 = make_float4(posx, posy, stp * kLog2e, 0.f);
        if (ADD) {
          S.e[slot] = make_float4(c.x, c.y, c.z, 0.f);
        } else {
          const float d0 = fadd(c.x, f.gray), d1 = fadd(c.y, f.gray), d2 = fadd(c.z, f.gray);
          S.e[slot] = make_float4(c.x, c.y, c.z, fdiv(c.x, d0));
          S.q[slot] = make_float2(fdiv(c.y, d1), fdiv(c.z, d2));
          S.wq[slot] = make_float4(f.gray / (d0 * d0), f.gray / (d1 * d1), f.gray / (d2 * d2), 0.f);
        }
      }
      p0.w = __uint_as_float(bb);
      S.p0[slot] = p0;
      S.idx[slot] = idx;
#pragma unroll
      for (int j = 0; j < 6; ++j) S.acc[j][slot] = 0.f;
    }
    __syncthreads();
    // ---- per-fragment adjoint ----------------------------------------------
    if (!warp_idle && (ADD || (uint32_t)bi * B >= wstop)) {
#pragma unroll 1
      for (int ch = 0; ch < B / 32; ++ch) {
        const uint32_t bbl = __float_as_uint(S.p0[ch * 32 + lane].w);
        const int mnx = bbl & 255, mxx = (bbl >> 8) & 255;
        const int mny = (bbl >> 16) & 255, mxy = bbl >> 24;
        const bool hit = (mnx < mxx) && (mnx < wbx1) && (mxx > wbx0) && (mny < wby1) &&
                         (mxy > wby0);
        uint32_t mask = __ballot_sync(0xffffffffu, hit);
        while (mask) {
          const int bit = __ffs(mask) - 1;
          mask &= ~(1u << bit);
          const int j = ch * 32 + bit;
          const float4 p0 = S.p0[j];
          const uint32_t bbj = __float_as_uint(p0.w);
          const int jmnx = bbj & 255, jmxx = (bbj >> 8) & 255;
          const int jmny = (bbj >> 16) & 255, jmxy = bbj >> 24;
          const float4 e = S.e[j];
          float2 q2 = make_float2(0.f, 0.f);
          float4 wq = make_float4(0.f, 0.f, 0.f, 0.f);
          if (!ADD) {
            q2 = S.q[j];
            wq = S.wq[j];
          }
          const uint16_t *run = srun + j * T;
          float sm[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
          bool any = false;
#pragma unroll
          for (int k = 0; k < K; ++k) {
            const int ix0 = wbx0 + (k % WX) * IW, iy0 = wby0 + (k / WX) * IH;
            if (jmnx < ix0 + IW && jmxx > ix0 && jmny < iy0 + IH && jmxy > iy0) {  // uniform
              bool in = valid[k] && pxi[k] >= jmnx && pxi[k] < jmxx;
              if (in) {
                const uint32_t rr = run[pxi[k]];
                in = pyi[k] >= (int)(rr & 255) && pyi[k] < (int)(rr >> 8);
              }
              if (in) {
                any = true;
                const float dx = pxf[k] - p0.x, dy = pyf[k] - p0.y;
                const float d2 = fmaf(dy, dy, dx * dx);
                const float att = ex2(p0.z * d2);
                float gatt;
                if (ADD) {
                  sm[0] = fmaf(-g[k][0], att, sm[0]);
                  sm[1] = fmaf(-g[k][1], att, sm[1]);
                  sm[2] = fmaf(-g[k][2], att, sm[2]);
                  gatt = -fmaf(g[k][0], e.x, fmaf(g[k][1], e.y, g[k][2] * e.z));
                } else {
                  const float E[3] = {e.x, e.y, e.z}, Q[3] = {e.w, q2.x, q2.y};
                  const float W[3] = {wq.x, wq.y, wq.z};
                  gatt = 0.f;
#pragma unroll
                  for (int c = 0; c < 3; ++c) {
                    // u as the forward forms it; transmittance in front of the
                    // particle from the stored optical depth, Tr = exp(-(od - sb))
                    const float u = E[c] * att;
                    sb[k][c] += u;
                    const float trm = ex2((sb[k][c] - od[k][c]) * kLog2e);
                    const float wt = -trm * expm1_neg(-u);  // Tr - Tr'
                    const float trn = trm - wt;            // Tr' = Tr*T
                    // dC/du = q*Tr' - B, dC/dq = Tr - Tr'  (B: composite behind)
                    const float ga = g[k][c] * fmaf(Q[c], trn, -bg[k][c]);
                    sm[c] = fmaf(ga, att, fmaf(g[k][c] * wt, W[c], sm[c]));
                    gatt = fmaf(ga, E[c], gatt);
                    bg[k][c] = fmaf(wt, Q[c], bg[k][c]);
                  }
                }
                const float ga2 = gatt * att;
                sm[3] = fmaf(ga2, dx, sm[3]);
                sm[4] = fmaf(ga2, dy, sm[4]);
                sm[5] = fmaf(ga2, d2, sm[5]);
              }
            }
          }
          if (__any_sync(0xffffffffu, any)) {
            int jj;
            bool ok;
            const float tot = warp_sum6(sm, lane, jj, ok);
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

template <int NT, int WX, int WY, int B>
void launch_adj_cfg(const AdjArgs &a, cudaStream_t s) {
  const int ntiles = a.f.ncx * a.f.ncy;
  const size_t sm = adj_smem_bytes<B>(a.f.T);
  if (a.f.a_eq_e) {
    auto k = k_splat_adj<NT, WX, WY, B, true>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k<<<ntiles, NT, sm, s>>>(a);
  } else {
    auto k = k_splat_adj<NT, WX, WY, B, false>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k<<<ntiles, NT, sm, s>>>(a);
  }
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

int launch_splat_adjoint(const AdjArgs &a, cudaStream_t s) {
  if (a.f.ncx * a.f.ncy <= 0) return 0;
  const int cfg = a.f.config >= 0 && splat_config_valid(a.f.config, a.f.T)
                      ? a.f.config
                      : splat_default_config(a.f.T, a.f.a_eq_e != 0);
  switch (cfg) {
    case 0: launch_adj_cfg<256, 1, 1, 256>(a, s); break;
    case 1: launch_adj_cfg<64, 2, 2, 128>(a, s); break;
    case 2: launch_adj_cfg<128, 2, 1, 128>(a, s); break;
    case 3: launch_adj_cfg<256, 2, 2, 256>(a, s); break;
    default: launch_adj_cfg<256, 4, 4, 256>(a, s); break;
  }
  return 1;
}

int launch_project_adjoint(const ProjAdjArgs &a, cudaStream_t s) {
  if (a.na <= 0) return 0;
  int blocks = (int)((a.na + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_project_adj<<<blocks, 256, 0, s>>>(a);
  return 1;
}

}  // namespace spl
