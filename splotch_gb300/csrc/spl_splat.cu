// spl_splat.cu -- tiled Gaussian splat (render_new region B,
// splotch/splotch_host.cc:434-692), additive and ordered emission-absorption.
//
// One CTA (256 threads, 8 warps) per tile.  The tile's pixels are numbered
// column-major (p = x*th + y, tile-local) and dealt out in contiguous spans:
// warp w owns pixels [w*32K, (w+1)*32K), lane l of item k owns pixel
// w*32K + 32k + l, and keeps its three channels in registers for the whole
// tile.  The tile's particle list is streamed through shared memory 256
// entries at a time: each thread stages one particle (tile-local position,
// Gaussian width, clipped bounding box) and the exact column runs of its
// footprint inside the tile.  Each warp then ballots the 256 staged particles
// against its own column range and walks only the hits, in list order.
//
// Coverage is decided exactly as the reference decides it (tile-local
// coordinates, truncating int conversion, the column run
// y in [int(py-dy+1), int(py+dy+1)) with dy = sqrt(r^2 - dx^2)), in
// non-contracted float arithmetic, so every pixel receives exactly the
// reference's fragments.  The Gaussian weight exp(stp*dx^2)*exp(stp*dy^2) is
// evaluated as one ex2(stp*log2e*(dx^2+dy^2)) instead of the reference's
// exptable<float> (splotch/splotchutils.h:174-215), which is closer to the
// exact weight than the table.
//
// Absorption: back-to-front applies C += expm1(-e*att)*(C - q) in list order
// (splotch_host.cc:663-665).  Front-to-back visits the list in reverse and
// accumulates C += Tr*q*(1-T), Tr *= T, the same sum term by term, and stops a
// tile once every pixel's transmittance in all channels is below epsilon.
#include "spl_internal.cuh"

namespace spl {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kBatch = kThreads;

struct SmemLayout {
  float *px, *py, *stp;
  uint32_t *bb;
  float4 *e, *q;
  uint16_t *run;
};

__device__ __forceinline__ SmemLayout smem_layout(uint8_t *base) {
  SmemLayout L;
  L.e = reinterpret_cast<float4 *>(base);
  L.q = L.e + kBatch;
  L.px = reinterpret_cast<float *>(L.q + kBatch);
  L.py = L.px + kBatch;
  L.stp = L.py + kBatch;
  L.bb = reinterpret_cast<uint32_t *>(L.stp + kBatch);
  L.run = reinterpret_cast<uint16_t *>(L.bb + kBatch);
  return L;
}

size_t smem_bytes(int T) {
  return (size_t)kBatch * (16 + 16 + 4 + 4 + 4 + 4) + (size_t)kBatch * T * 2;
}

template <int K, bool ADD, bool FTB>
__global__ void __launch_bounds__(kThreads) k_splat(SplatArgs a) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  const SmemLayout L = smem_layout(smem_raw);
  const int T = a.T;
  const int tile = a.tile_order ? (int)__ldg(a.tile_order + blockIdx.x) : (int)blockIdx.x;
  const int ix = tile % a.ncx, iy = tile / a.ncx;
  const int x0s = ix * T, y0s = iy * T;
  const int tw = min(x0s + T, a.xres) - x0s;
  const int th = min(y0s + T, a.yres) - y0s;
  const int P = tw * th;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int wbase = w * 32 * K;
  const bool warp_has_pixels = wbase < P;
  const int wc0 = warp_has_pixels ? wbase / th : 0;
  const int wc1 = warp_has_pixels ? (min(wbase + 32 * K, P) - 1) / th : -1;

  int pxy[K];
  float pxf[K], pyf[K];  // tile-local pixel coordinates as floats
  int ic0[K], ic1[K];
  float acc[K][3];
  float tr[K][3];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int p0 = wbase + k * 32;
    const int p = p0 + lane;
    pxy[k] = p < P ? (((p / th) << 8) | (p % th)) : -1;
    pxf[k] = (float)(pxy[k] >> 8);
    pyf[k] = (float)(pxy[k] & 255);
    ic0[k] = p0 < P ? p0 / th : 1 << 20;
    ic1[k] = p0 < P ? (min(p0 + 31, P - 1)) / th : -1;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      acc[k][c] = 0.f;
      tr[k][c] = 1.f;
    }
  }

  const uint32_t start = a.tile_start[tile], end = a.tile_start[tile + 1];
  const int nbatch = (int)((end - start + kBatch - 1) / kBatch);
  bool warp_done = !warp_has_pixels;

  for (int b = 0; b < nbatch; ++b) {
    const int bi = FTB ? nbatch - 1 - b : b;
    // ---- stage one particle per thread ---------------------------------
    {
      const uint32_t jj = start + (uint32_t)bi * kBatch + threadIdx.x;
      uint32_t bb = 0;
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
          uint16_t *run = L.run + threadIdx.x * T;
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
        L.px[threadIdx.x] = posx;
        L.py[threadIdx.x] = posy;
        L.stp[threadIdx.x] = stp * kLog2e;
        L.e[threadIdx.x] = make_float4(c.x, c.y, c.z, 0.f);
        if (!ADD) {
          // q = e/(e+grayabsorb), splotch_host.cc:626-628
          L.q[threadIdx.x] = make_float4(fdiv(c.x, fadd(c.x, a.gray)),
                                         fdiv(c.y, fadd(c.y, a.gray)),
                                         fdiv(c.z, fadd(c.z, a.gray)), 0.f);
        }
      }
      L.bb[threadIdx.x] = bb;
    }
    __syncthreads();
    // ---- accumulate ------------------------------------------------------
    if (!warp_done) {
#pragma unroll 1
      for (int cc = 0; cc < kBatch / 32; ++cc) {
        const int ch = FTB ? kBatch / 32 - 1 - cc : cc;
        const uint32_t bbl = L.bb[ch * 32 + lane];
        const int mnx = bbl & 255, mxx = (bbl >> 8) & 255;
        const bool hit = (mnx < mxx) && (mxx > wc0) && (mnx <= wc1);
        uint32_t mask = __ballot_sync(0xffffffffu, hit);
        while (mask) {
          const int bit = FTB ? 31 - __clz(mask) : __ffs(mask) - 1;
          mask &= ~(1u << bit);
          const int j = ch * 32 + bit;
          const uint32_t bbj = L.bb[j];
          const int jmnx = bbj & 255, jmxx = (bbj >> 8) & 255;
          const float posx = L.px[j], posy = L.py[j], stp2 = L.stp[j];
          const float4 e = L.e[j];
          float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
          if (!ADD) q = L.q[j];
          const uint16_t *run = L.run + j * T;
#pragma unroll
          for (int k = 0; k < K; ++k) {
            if (ic1[k] >= jmnx && ic0[k] < jmxx) {  // warp-uniform
              const int x = pxy[k] >> 8, y = pxy[k] & 255;
              bool in = pxy[k] >= 0 && x >= jmnx && x < jmxx;
              if (in) {
                const uint32_t rr = run[x];
                in = y >= (int)(rr & 255) && y < (int)(rr >> 8);
              }
              if (in) {
                const float dx = pxf[k] - posx, dy = pyf[k] - posy;
                const float s2 = fmaf(dy, dy, dx * dx);
                const float att = ex2(stp2 * s2);
                if (ADD) {
                  acc[k][0] = fmaf(-e.x, att, acc[k][0]);
                  acc[k][1] = fmaf(-e.y, att, acc[k][1]);
                  acc[k][2] = fmaf(-e.z, att, acc[k][2]);
                } else if (!FTB) {
                  const float m0 = expm1_neg(-e.x * att);
                  const float m1 = expm1_neg(-e.y * att);
                  const float m2 = expm1_neg(-e.z * att);
                  acc[k][0] = fmaf(m0, acc[k][0] - q.x, acc[k][0]);
                  acc[k][1] = fmaf(m1, acc[k][1] - q.y, acc[k][1]);
                  acc[k][2] = fmaf(m2, acc[k][2] - q.z, acc[k][2]);
                } else {
                  const float m0 = expm1_neg(-e.x * att);
                  const float m1 = expm1_neg(-e.y * att);
                  const float m2 = expm1_neg(-e.z * att);
                  acc[k][0] = fmaf(-tr[k][0] * q.x, m0, acc[k][0]);
                  acc[k][1] = fmaf(-tr[k][1] * q.y, m1, acc[k][1]);
                  acc[k][2] = fmaf(-tr[k][2] * q.z, m2, acc[k][2]);
                  tr[k][0] = fmaf(tr[k][0], m0, tr[k][0]);
                  tr[k][1] = fmaf(tr[k][1], m1, tr[k][1]);
                  tr[k][2] = fmaf(tr[k][2], m2, tr[k][2]);
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
          if (pxy[k] >= 0)
            mine_done = mine_done && tr[k][0] < a.ftb_eps && tr[k][1] < a.ftb_eps &&
                        tr[k][2] < a.ftb_eps;
        warp_done = __all_sync(0xffffffffu, mine_done);
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
    if (pxy[k] >= 0) {
      const int x = pxy[k] >> 8, y = pxy[k] & 255;
      float *o = a.pic + ((size_t)(x0s + x) * a.yres + (y0s + y)) * 3;
      o[0] = acc[k][0];
      o[1] = acc[k][1];
      o[2] = acc[k][2];
    }
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

template <int K>
int launch_k(const SplatArgs &a, cudaStream_t s) {
  const int ntiles = a.ncx * a.ncy;
  const size_t sm = smem_bytes(a.T);
  if (a.a_eq_e) {
    k_splat<K, true, false><<<ntiles, kThreads, sm, s>>>(a);
  } else if (a.order_mode == 1) {
    k_splat<K, false, true><<<ntiles, kThreads, sm, s>>>(a);
  } else {
    k_splat<K, false, false><<<ntiles, kThreads, sm, s>>>(a);
  }
  return 1;
}

}  // namespace

void launch_count_fragments(const SplatArgs &a, unsigned long long *total, cudaStream_t s) {
  cudaMemsetAsync(total, 0, sizeof(unsigned long long), s);
  if (a.ncx * a.ncy > 0) k_count_fragments<<<a.ncx * a.ncy, 256, 0, s>>>(a, total);
}

int launch_splat(const SplatArgs &a, cudaStream_t s) {
  const int need = (a.T * a.T + kThreads - 1) / kThreads;  // pixels per lane
  if (a.ncx * a.ncy <= 0) return 0;
  if (need <= 1) return launch_k<1>(a, s);
  if (need <= 2) return launch_k<2>(a, s);
  if (need <= 4) return launch_k<4>(a, s);
  if (need <= 8) return launch_k<8>(a, s);
  if (need <= 10) return launch_k<10>(a, s);
  return launch_k<16>(a, s);
}

}  // namespace spl
