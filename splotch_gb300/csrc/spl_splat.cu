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
// a warp once every pixel's transmittance in all channels is below epsilon,
// and the tile once every warp has stopped.
#include "spl_internal.cuh"

namespace spl {

namespace {

constexpr int IW = 8, IH = 4;  // item: 8 columns x 4 rows, one pixel per lane

template <int B>
struct Smem {
  float4 p0[B];  // posx, posy, stp*log2e, bbox bits
  float4 e[B];   // e.r, e.g, e.b, q.r
  float2 q[B];   // q.g, q.b
  // followed by uint16_t run[B*T]: column runs lo | hi<<8
};

template <int B>
size_t smem_bytes(int T) {
  return sizeof(Smem<B>) + (size_t)B * T * 2;
}

// One tile of one frame, by the whole CTA (shared by the per-frame launch and
// the persistent batch kernel).
// AUX (ordered frames only): also accumulate each pixel's optical depth and
// record where the warp stopped, for the adjoint (SplatArgs::aux).
template <int NT, int WX, int WY, int B, bool ADD, bool FTB, bool AUX = false>
__device__ __forceinline__ void splat_tile(const SplatArgs &a, const int tile,
                                           uint8_t *smem_raw) {
  constexpr int K = WX * WY;
  static_assert(!(AUX && ADD), "optical depth is kept for ordered frames only");
  Smem<B> &S = *reinterpret_cast<Smem<B> *>(smem_raw);
  uint16_t *srun = reinterpret_cast<uint16_t *>(smem_raw + sizeof(Smem<B>));

  const int T = a.T;
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

  float pxf[K], pyf[K];
  int pxi[K], pyi[K];
  bool valid[K];
  float acc[K][3], tr[K][3];
  float od[AUX ? K : 1][3];  // optical depth (AUX)
  uint32_t stop = 0;         // list position below which this warp composited nothing
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int x = wbx0 + (k % WX) * IW + (lane & 7);
    const int y = wby0 + (k / WX) * IH + (lane >> 3);
    valid[k] = warp_has_pixels && x < tw && y < th;
    pxi[k] = x;
    pyi[k] = y;
    pxf[k] = (float)x;
    pyf[k] = (float)y;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (AUX) od[AUX ? k : 0][c] = 0.f;
      acc[k][c] = 0.f;
      tr[k][c] = 1.f;
    }
  }

  const uint32_t start = a.tile_start[tile], end = a.tile_start[tile + 1];
  const int nbatch = (int)((end - start + B - 1) / B);
  bool warp_done = !warp_has_pixels;

  for (int b = 0; b < nbatch; ++b) {
    const int bi = FTB ? nbatch - 1 - b : b;
    // ---- stage B particles ------------------------------------------------
#pragma unroll 1
    for (int slot = threadIdx.x; slot < B; slot += NT) {
      const uint32_t jj = start + (uint32_t)bi * B + slot;
      uint32_t bb = 0;
      float4 p0 = make_float4(0.f, 0.f, 0.f, 0.f);
      if (jj < end) {
        const uint32_t idx = __ldg(a.entries + jj);
        const float4 p = __ldg(a.pos + idx);
        const float4 c = __ldg(a.col + idx);
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
          bb = (uint32_t)minx | ((uint32_t)maxx << 8) | ((uint32_t)miny << 16) |
               ((uint32_t)maxy << 24);
          uint16_t *run = srun + slot * T;
          for (int x = minx; x < maxx; ++x) {  // splotch_host.cc:603-606
            const float dx = fsub((float)x, posx);
            const float dxsq = fmul(dx, dx);
            const float dy = fsqrt(fsub(radsq, dxsq));
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
          // q = e/(e+grayabsorb), splotch_host.cc:626-628
          S.e[slot] = make_float4(c.x, c.y, c.z, fdiv(c.x, fadd(c.x, a.gray)));
          S.q[slot] = make_float2(fdiv(c.y, fadd(c.y, a.gray)), fdiv(c.z, fadd(c.z, a.gray)));
        }
      }
      p0.w = __uint_as_float(bb);
      S.p0[slot] = p0;
    }
    __syncthreads();
    // ---- accumulate ---------------------------------------------------------
    if (!warp_done) {
#pragma unroll 1
      for (int cc = 0; cc < B / 32; ++cc) {
        const int ch = FTB ? B / 32 - 1 - cc : cc;
        const uint32_t bbl = __float_as_uint(S.p0[ch * 32 + lane].w);
        const int mnx = bbl & 255, mxx = (bbl >> 8) & 255;
        const int mny = (bbl >> 16) & 255, mxy = bbl >> 24;
        const bool hit = (mnx < mxx) && (mnx < wbx1) && (mxx > wbx0) && (mny < wby1) &&
                         (mxy > wby0);
        uint32_t mask = __ballot_sync(0xffffffffu, hit);
        while (mask) {
          const int bit = FTB ? 31 - __clz(mask) : __ffs(mask) - 1;
          mask &= ~(1u << bit);
          const int j = ch * 32 + bit;
          const float4 p0 = S.p0[j];
          const uint32_t bbj = __float_as_uint(p0.w);
          const int jmnx = bbj & 255, jmxx = (bbj >> 8) & 255;
          const int jmny = (bbj >> 16) & 255, jmxy = bbj >> 24;
          const float4 e = S.e[j];
          float2 q2 = make_float2(0.f, 0.f);
          if (!ADD) q2 = S.q[j];
          const uint16_t *run = srun + j * T;
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
                const float dx = pxf[k] - p0.x, dy = pyf[k] - p0.y;
                const float att = ex2(p0.z * fmaf(dy, dy, dx * dx));
                if (ADD) {
                  acc[k][0] = fmaf(-e.x, att, acc[k][0]);
                  acc[k][1] = fmaf(-e.y, att, acc[k][1]);
                  acc[k][2] = fmaf(-e.z, att, acc[k][2]);
                } else if (!FTB) {
                  const float u0 = e.x * att, u1 = e.y * att, u2 = e.z * att;
                  if (AUX) {
                    od[AUX ? k : 0][0] += u0;
                    od[AUX ? k : 0][1] += u1;
                    od[AUX ? k : 0][2] += u2;
                  }
                  const float m0 = expm1_neg(-u0);
                  const float m1 = expm1_neg(-u1);
                  const float m2 = expm1_neg(-u2);
                  acc[k][0] = fmaf(m0, acc[k][0] - e.w, acc[k][0]);
                  acc[k][1] = fmaf(m1, acc[k][1] - q2.x, acc[k][1]);
                  acc[k][2] = fmaf(m2, acc[k][2] - q2.y, acc[k][2]);
                } else {
                  // w = Tr*(1-T) = -Tr*expm1(-e*att); C += w*q; Tr -= w
                  const float u0 = e.x * att, u1 = e.y * att, u2 = e.z * att;
                  if (AUX) {
                    od[AUX ? k : 0][0] += u0;
                    od[AUX ? k : 0][1] += u1;
                    od[AUX ? k : 0][2] += u2;
                  }
                  const float w0 = -tr[k][0] * expm1_neg(-u0);
                  const float w1 = -tr[k][1] * expm1_neg(-u1);
                  const float w2 = -tr[k][2] * expm1_neg(-u2);
                  acc[k][0] = fmaf(w0, e.w, acc[k][0]);
                  acc[k][1] = fmaf(w1, q2.x, acc[k][1]);
                  acc[k][2] = fmaf(w2, q2.y, acc[k][2]);
                  tr[k][0] -= w0;
                  tr[k][1] -= w1;
                  tr[k][2] -= w2;
                }
              }
            }
          }
        }
      }
      if (FTB) {
        bool mine_done = true;
#pragma unroll
        for (int k = 0; k < K; ++k)
          if (valid[k])
            mine_done = mine_done && tr[k][0] < a.ftb_eps && tr[k][1] < a.ftb_eps &&
                        tr[k][2] < a.ftb_eps;
        warp_done = __all_sync(0xffffffffu, mine_done);
        if (AUX && warp_done) stop = (uint32_t)bi * B;
      }
    }
    if (FTB) {
      if (__syncthreads_and(warp_done ? 1 : 0)) break;
    } else {
      __syncthreads();
    }
  }

  // ---- write the tile (pic is x-major: pixel (x,y) at (x*yres + y)*3) ----
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (valid[k]) {
      float *o = a.pic + ((size_t)(x0s + pxi[k]) * a.yres + (y0s + pyi[k])) * 3;
      o[0] = acc[k][0];
      o[1] = acc[k][1];
      o[2] = acc[k][2];
      if (AUX)
        a.aux[(size_t)(x0s + pxi[k]) * a.yres + (y0s + pyi[k])] =
            make_float4(od[AUX ? k : 0][0], od[AUX ? k : 0][1], od[AUX ? k : 0][2],
                        __uint_as_float(stop));
    }
  }
}

template <int NT, int WX, int WY, int B, bool ADD, bool FTB, bool AUX>
__global__ void __launch_bounds__(NT) k_splat(SplatArgs a) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  const int tile = a.tile_order ? (int)__ldg(a.tile_order + blockIdx.x) : (int)blockIdx.x;
  splat_tile<NT, WX, WY, B, ADD, FTB, AUX>(a, tile, smem_raw);
}

// Persistent splat over a queue of (frame, tile) items: each CTA takes the
// next item from an atomic counter until the queue is empty.  The queue is in
// longest-list-first order across all frames; every frame's own arguments
// (image, tiling, mode, tile-range slice) come from a per-frame table.
template <int NT, int WX, int WY, int B>
__global__ void __launch_bounds__(NT) k_splat_queue(BatchSplatArgs q) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  __shared__ uint32_t s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(q.counter, 1u);
    __syncthreads();
    const uint32_t item = s_item;
    if (item >= q.nwork) break;
    const uint32_t gt = __ldg(q.work + q.work_begin + item);
    const uint32_t f = __ldg(q.frame_of_tile + gt);
    const SplatArgs a = q.frames[f];
    const int tile = (int)(gt - q.tile_base[f]);
    if (a.a_eq_e)
      splat_tile<NT, WX, WY, B, true, false>(a, tile, smem_raw);
    else if (a.order_mode == 1)
      splat_tile<NT, WX, WY, B, false, true>(a, tile, smem_raw);
    else
      splat_tile<NT, WX, WY, B, false, false>(a, tile, smem_raw);
    __syncthreads();  // s_item and the staging buffers are reused
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

template <int NT, int WX, int WY, int B, bool ADD, bool FTB, bool AUX>
void launch_one(const SplatArgs &a, size_t sm, cudaStream_t s) {
  auto k = k_splat<NT, WX, WY, B, ADD, FTB, AUX>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<a.ncx * a.ncy, NT, sm, s>>>(a);
}

template <int NT, int WX, int WY, int B>
int launch_cfg(const SplatArgs &a, cudaStream_t s) {
  const size_t sm = smem_bytes<B>(a.T);
  const bool aux = a.aux != nullptr;
  if (a.a_eq_e)
    launch_one<NT, WX, WY, B, true, false, false>(a, sm, s);
  else if (a.order_mode == 1)
    aux ? launch_one<NT, WX, WY, B, false, true, true>(a, sm, s)
        : launch_one<NT, WX, WY, B, false, true, false>(a, sm, s);
  else
    aux ? launch_one<NT, WX, WY, B, false, false, true>(a, sm, s)
        : launch_one<NT, WX, WY, B, false, false, false>(a, sm, s);
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
// T=16): 4 warps x 16x4 is fastest for the absorption splat, 8 warps x 8x4 for
// the additive one; larger tiles need the wider configurations.
int splat_default_config(int T, bool additive) {
  if (!additive && splat_config_valid(2, T)) return 2;
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
    case 0: return launch_cfg<256, 1, 1, 256>(a, s);
    case 1: return launch_cfg<64, 2, 2, 128>(a, s);
    case 2: return launch_cfg<128, 2, 1, 128>(a, s);
    case 3: return launch_cfg<256, 2, 2, 256>(a, s);
    default: return launch_cfg<256, 4, 4, 256>(a, s);
  }
}

namespace {

template <int NT, int WX, int WY, int B>
int launch_queue_cfg(const BatchSplatArgs &q, cudaStream_t s) {
  const size_t sm = smem_bytes<B>(q.T);
  auto k = k_splat_queue<NT, WX, WY, B>;
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

}  // namespace

int launch_splat_queue(const BatchSplatArgs &q, int cfg, cudaStream_t s) {
  if (q.nwork == 0) return 0;
  switch (cfg) {
    case 0: return launch_queue_cfg<256, 1, 1, 256>(q, s);
    case 1: return launch_queue_cfg<64, 2, 2, 128>(q, s);
    case 2: return launch_queue_cfg<128, 2, 1, 128>(q, s);
    case 3: return launch_queue_cfg<256, 2, 2, 256>(q, s);
    default: return launch_queue_cfg<256, 4, 4, 256>(q, s);
  }
}

}  // namespace spl
