// spl_bin.cu -- particle-to-tile binning (render_new region A,
// splotch/splotch_host.cc:339-406) as count -> exclusive scan -> emit ->
// stable sort by tile id.
//
// The reference builds one list per tile; because each OpenMP thread scans a
// contiguous, ascending share of the particle array and the lists are read in
// thread order (splotch_host.cc:455), every tile's list is in ascending array
// position.  Here entries are emitted in visiting order (scan offsets) and a
// stable radix sort by tile id groups them without reordering, which gives the
// same per-tile order bit-for-bit.
//
// Two emission paths: footprints of up to kWideTiles tiles are dealt across
// the lanes of a warp (the candidate tiles of its 32 particles laid end to
// end), and a wide particle gets a warp of its own (rows of its tile rectangle
// spread over the lanes), so a particle covering thousands of tiles does not
// hold up the particles beside it.
#include "spl_internal.cuh"

namespace spl {

namespace {

constexpr int kWideTiles = 64;

// One warp per 32 consecutive visiting positions.  The candidate cells of the
// warp's narrow particles (each particle's tile rectangle, column-major like
// the reference loop) are laid end to end and dealt to the lanes 32 at a
// time: a lane finds its cell's particle by binary search over the warp's
// cell prefix, runs the circle test, and the passing cells take consecutive
// slots in visiting order (a ballot prefix).  Every lane does useful work,
// whatever the mix of footprints, and a warp's stores are contiguous.
//
// A particle's passing cells fill exactly its slots [off, off + count): the
// count came from the same test in the same arithmetic; a store is also
// checked against the particle's count before it is made (one past it sets
// bit 4 (16) of *err instead).
__global__ void __launch_bounds__(256) k_emit_narrow(const float4 *__restrict__ pos,
                                                     const uint32_t *__restrict__ count,
                                                     const uint32_t *__restrict__ order,
                                                     const uint64_t *__restrict__ off,
                                                     int64_t n, Tiling g,
                                                     uint32_t *__restrict__ tkey,
                                                     uint32_t *__restrict__ tval,
                                                     uint32_t *__restrict__ wide_list,
                                                     uint32_t *__restrict__ wide_n,
                                                     uint32_t *err) {
  __shared__ uint32_t cpre[256 / 32][33];  // per warp: exclusive cell prefix of its lanes
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const int T = g.T;
  const int64_t nchunk = (n + 31) / 32;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t ch = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; ch < nchunk;
       ch += nwarp) {
    const int64_t s = ch * 32 + lane;
    const uint32_t c = s < n ? __ldg(count + s) : 0u;  // counts are in visiting order
    const uint32_t i = s < n ? (order ? __ldg(order + s) : (uint32_t)s) : 0u;
    const bool narrow = c > 0u && c <= (uint32_t)kWideTiles;
    if (c > (uint32_t)kWideTiles)  // handed to the warp-per-particle path
      wide_list[atomicAdd(wide_n, 1u)] = (uint32_t)s;
    float px = 0.f, py = 0.f, sumsq = 0.f;
    int minx = 0, miny = 0, wy = 1;
    uint32_t cells = 0, magic = 0, olo = 0, ohi = 0;
    if (narrow) {
      const float4 p = __ldg(pos + i);
      px = p.x;
      py = p.y;
      const float rfacr = fmul(0.75f, p.z);
      minx = max(0, f2i(fadd(fsub(px, rfacr), 1.f)) / T);
      const int maxx = min(g.ncx - 1, f2i(fadd(px, rfacr)) / T);
      miny = max(0, f2i(fadd(fsub(py, rfacr), 1.f)) / T);
      const int maxy = min(g.ncy - 1, f2i(fadd(py, rfacr)) / T);
      const float rs = fadd(g.rcell, rfacr);
      sumsq = fmul(rs, rs);
      wy = maxy - miny + 1;
      cells = (uint32_t)((maxx - minx + 1) * wy);
      // q / wy = umulhi(q, ceil(2^32 / wy)), exact for q, wy < 2^16
      magic = wy > 1 ? 0xffffffffu / (uint32_t)wy + 1u : 0u;
      const uint64_t o = __ldg(off + s);
      olo = (uint32_t)o;
      ohi = (uint32_t)(o >> 32);
    }
    // inclusive warp scans: candidate cells, and the narrow particles' counts
    uint32_t cin = cells, nin = narrow ? c : 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t0 = __shfl_up_sync(0xffffffffu, cin, d);
      const uint32_t t1 = __shfl_up_sync(0xffffffffu, nin, d);
      if (lane >= d) {
        cin += t0;
        nin += t1;
      }
    }
    const uint32_t total = __shfl_sync(0xffffffffu, cin, 31);
    const uint32_t nexcl = nin - (narrow ? c : 0u);  // passing cells before this lane's particle
    __syncwarp();  // the previous chunk's readers of cpre are done
    cpre[w][lane] = cin - cells;
    __syncwarp();
    uint32_t carry = 0;  // passing cells dealt so far in this chunk
    for (uint32_t k0 = 0; k0 < total; k0 += 32) {
      const uint32_t k = k0 + (uint32_t)lane;
      int l = 0;  // the last lane whose cells start at or before k
#pragma unroll
      for (int step = 16; step > 0; step >>= 1)
        if (cpre[w][l + step] <= k) l += step;
      const int lminx = __shfl_sync(0xffffffffu, minx, l);
      const int lminy = __shfl_sync(0xffffffffu, miny, l);
      const int lwy = __shfl_sync(0xffffffffu, wy, l);
      const uint32_t lmag = __shfl_sync(0xffffffffu, magic, l);
      const float lpx = __shfl_sync(0xffffffffu, px, l);
      const float lpy = __shfl_sync(0xffffffffu, py, l);
      const float lsq = __shfl_sync(0xffffffffu, sumsq, l);
      const uint32_t lc = __shfl_sync(0xffffffffu, c, l);
      const uint32_t lnex = __shfl_sync(0xffffffffu, nexcl, l);
      const uint32_t li = __shfl_sync(0xffffffffu, i, l);
      const uint32_t lolo = __shfl_sync(0xffffffffu, olo, l);
      const uint32_t lohi = __shfl_sync(0xffffffffu, ohi, l);
      const uint32_t q = k - cpre[w][l];
      const uint32_t qx = lwy > 1 ? __umulhi(q, lmag) : q;
      const int ix = lminx + (int)qx;
      const int iy = lminy + (int)(q - qx * (uint32_t)lwy);
      bool pass = false;
      if (k < total) {  // the test of for_each_tile, operation for operation
        const float cx = fadd(g.cmid0, (float)(ix * T));
        const float dx = fsub(lpx, cx);
        const float dx2 = fmul(dx, dx);
        const float cy = fadd(g.cmid0, (float)(iy * T));
        const float dy = fsub(lpy, cy);
        pass = fadd(dx2, fmul(dy, dy)) < lsq;
      }
      const uint32_t b = __ballot_sync(0xffffffffu, pass);
      const uint32_t j = carry + __popc(b & lt) - lnex;  // rank among the particle's tiles
      if (pass && j < lc) {
        const uint64_t slot = (((uint64_t)lohi << 32) | lolo) + j;
        tkey[slot] = (uint32_t)(iy * g.ncx + ix);
        tval[slot] = li;
      } else if (pass) {
        atomicOr(err, 16u);  // more passing tiles than counted: reported, not stored
      }
      carry += __popc(b);
    }
  }
}

// One warp per wide particle.  Lane l takes tile rows iy = miny + l, +32, ...;
// each row's passing tiles are counted first, a warp scan gives each row its
// slot, then the row is written.  The order of a particle's entries inside its
// slot range does not matter: the stable tile sort only orders entries of the
// same tile, and a particle contributes at most one entry per tile.
__global__ void __launch_bounds__(256) k_emit_wide(const float4 *__restrict__ pos,
                                                   const uint32_t *__restrict__ count,
                                                   const uint32_t *__restrict__ order,
                                                   const uint64_t *__restrict__ off,
                                                   const uint32_t *__restrict__ wide_list,
                                                   const uint32_t *__restrict__ wide_n,
                                                   Tiling g, uint32_t *__restrict__ tkey,
                                                   uint32_t *__restrict__ tval, uint32_t *err) {
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t nw = *wide_n;
  for (int64_t w = warp0; w < nw; w += nwarps) {
    const uint32_t s = wide_list[w];
    const uint32_t i = order ? __ldg(order + s) : s;
    const uint64_t o = __ldg(off + s);
    const uint64_t oend = o + __ldg(count + s);  // the particle's slots end here
    const float4 p = __ldg(pos + i);
    const int T = g.T;
    const float rfacr = fmul(0.75f, p.z);
    const int minx = max(0, f2i(fadd(fsub(p.x, rfacr), 1.f)) / T);
    const int maxx = min(g.ncx - 1, f2i(fadd(p.x, rfacr)) / T);
    const int miny = max(0, f2i(fadd(fsub(p.y, rfacr), 1.f)) / T);
    const int maxy = min(g.ncy - 1, f2i(fadd(p.y, rfacr)) / T);
    const float rs = fadd(g.rcell, rfacr);
    const float sumsq = fmul(rs, rs);
    uint64_t base = o;
    for (int iy0 = miny; iy0 <= maxy; iy0 += 32) {
      const int iy = iy0 + lane;
      int rc = 0;
      float dy2 = 0.f;
      if (iy <= maxy) {
        const float cy = fadd(g.cmid0, (float)(iy * T));
        const float dy = fsub(p.y, cy);
        dy2 = fmul(dy, dy);
        for (int ix = minx; ix <= maxx; ++ix) {
          const float cx = fadd(g.cmid0, (float)(ix * T));
          const float dx = fsub(p.x, cx);
          if (fadd(fmul(dx, dx), dy2) < sumsq) ++rc;
        }
      }
      // exclusive warp scan of row counts
      int incl = rc;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += t;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      uint64_t slot = base + (uint64_t)(incl - rc);
      if (iy <= maxy && rc > 0) {
        for (int ix = minx; ix <= maxx; ++ix) {
          const float cx = fadd(g.cmid0, (float)(ix * T));
          const float dx = fsub(p.x, cx);
          if (fadd(fmul(dx, dx), dy2) < sumsq) {
            if (slot < oend) {
              tkey[slot] = (uint32_t)(iy * g.ncx + ix);
              tval[slot] = i;
            } else {
              atomicOr(err, 16u);  // more passing tiles than counted: reported, not stored
            }
            ++slot;
          }
        }
      }
      base += (uint64_t)total;
    }
  }
}

// tile_start[t] = first sorted position whose key is >= t.  A thread takes
// four consecutive positions 4q..4q+3 (one 16-byte load when the keys are
// 16-byte aligned and all four exist) and the key before them; positions run
// to ne inclusive, where the key is taken as ntiles.
__global__ void __launch_bounds__(256) k_tile_ranges(const uint32_t *__restrict__ key,
                                                     int64_t ne, int64_t ntiles,
                                                     uint32_t *__restrict__ tile_start) {
  const bool vec = (reinterpret_cast<uintptr_t>(key) & 15u) == 0;
  const int64_t nq = ne / 4 + 1;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nq;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p0 = q * 4;
    uint32_t k4[4];
    if (vec && p0 + 4 <= ne) {
      const uint4 v = __ldg(reinterpret_cast<const uint4 *>(key + p0));
      k4[0] = v.x;
      k4[1] = v.y;
      k4[2] = v.z;
      k4[3] = v.w;
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) k4[i] = p0 + i < ne ? __ldg(key + p0 + i) : 0u;
    }
    int64_t kprev = p0 > 0 ? (int64_t)__ldg(key + p0 - 1) : -1;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t p = p0 + i;
      if (p > ne) break;
      const int64_t kcur = p < ne ? (int64_t)k4[i] : ntiles;
      for (int64_t t = kprev + 1; t <= kcur; ++t) tile_start[t] = (uint32_t)p;
      kprev = kcur;
    }
  }
}

// Scheduling key per tile: 8-bit log-scale of the list length, inverted so an
// ascending sort puts the longest lists first (longest-processing-time order).
__global__ void __launch_bounds__(256) k_tile_cost(const uint32_t *__restrict__ tile_start,
                                                   int64_t ntiles, uint32_t *__restrict__ key) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntiles;
       t += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t cnt = tile_start[t + 1] - tile_start[t];
    const int lg = (int)(8.f * __log2f((float)cnt + 1.f));
    key[t] = 255u - (uint32_t)min(lg, 255);
  }
}

int grid_for(int64_t n, int per_block) {
  int64_t b = (n + per_block - 1) / per_block;
  const int64_t cap = 152LL * 16;
  if (b > cap) b = cap;
  return (int)(b > 0 ? b : 1);
}

}  // namespace

void launch_emit(const float4 *pos, const uint32_t *count, const uint32_t *order,
                 const uint64_t *off, int64_t n, Tiling g, uint32_t *tkey, uint32_t *tval,
                 uint32_t *wide_list, uint32_t *wide_n, uint32_t *err, cudaStream_t s) {
  if (n <= 0) return;
  cudaMemsetAsync(wide_n, 0, sizeof(uint32_t), s);
  k_emit_narrow<<<grid_for(n, 256), 256, 0, s>>>(pos, count, order, off, n, g, tkey, tval,
                                                 wide_list, wide_n, err);
  k_emit_wide<<<152 * 4, 256, 0, s>>>(pos, count, order, off, wide_list, wide_n, g, tkey, tval,
                                      err);
}

void launch_tile_ranges(const uint32_t *sorted_tkey, int64_t ne, int64_t ntiles,
                        uint32_t *tile_start, cudaStream_t s) {
  k_tile_ranges<<<grid_for(ne / 4 + 1, 256), 256, 0, s>>>(sorted_tkey, ne, ntiles, tile_start);
}

__global__ void __launch_bounds__(256) k_gather_u32(const uint32_t *__restrict__ src,
                                                    const uint32_t *__restrict__ perm,
                                                    int64_t n, uint32_t *__restrict__ out,
                                                    uint64_t nsrc, uint32_t *err) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t v = __ldg(perm + s);
    if (v < nsrc) {
      out[s] = __ldg(src + v);
    } else {
      out[s] = 0u;
      if (err) atomicOr(err, 2u);
    }
  }
}

void launch_gather_u32(const uint32_t *src, const uint32_t *perm, int64_t n, uint32_t *out,
                       cudaStream_t s, int64_t nsrc, uint32_t *err) {
  const uint64_t lim = nsrc > 0 ? (uint64_t)nsrc : ~0ull;
  if (n > 0) k_gather_u32<<<grid_for(n, 256), 256, 0, s>>>(src, perm, n, out, lim, err);
}

void launch_tile_cost(const uint32_t *tile_start, int64_t ntiles, uint32_t *key,
                      cudaStream_t s) {
  if (ntiles > 0) k_tile_cost<<<grid_for(ntiles, 256), 256, 0, s>>>(tile_start, ntiles, key);
}

}  // namespace spl
