// spl_batch.cu -- batched rendering: many frames (camera poses, resolutions,
// additive or ordered modes, particle sets of uneven size) in one launch of a
// captured CUDA graph.
//
// Per render, with no host round trip between stages (frames are kept
// additive first, then ordered):
//   per set     : the palette colour of each particle, when several frames
//                 share the set and its palettes (it does not depend on the
//                 camera); their projection reads it instead of interpolating
//   all frames  : one activity-flag launch over every frame's particle set
//                 (projection test; a per-frame table of projection constants
//                 and inputs)
//   per class   : one popcount scan over the class's flag words -> the class's
//                 active particles get consecutive record numbers, frame after
//                 frame, in the class's own segment (additive [0, cap_add),
//                 ordered [cap_add, cap_add + cap_ord)); record starts per frame
//   all frames  : one dense projection + colourisation launch into the records
//   ordered     : stable depth sort of the ordered segment by key, then stable
//                 sort by frame id (each frame in its own order, frame-major);
//                 additive records keep their record order, as a per-frame
//                 additive render does
//   all frames  : tile counts in visiting order, one scan, one emission of
//                 (global tile id, record) pairs, one stable sort by tile id;
//                 tile ranges; work queue = every (frame, tile) item, additive
//                 frames first, each class longest list first
//   splat       : one persistent kernel per class (additive / ordered) that
//                 takes items from the queue; each item renders one tile of
//                 one frame straight into that frame's image.
// Sizes that depend on the data (active records, bin entries) are capacities
// taken from a measured plan; the arrays past the live counts hold sentinel
// keys that sort last, and a render whose counts outgrow the plan sets a
// status bit, re-plans from new measurements and renders again.
//
// The autotuner picks the tile size and a launch configuration per class by
// timing the pipeline (tile sizes 8, 16, 32) and the persistent splat (every
// configuration that covers the tile size) on the batch itself.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "spl_host.h"

namespace spl {
namespace {

struct FrameTile {
  Tiling g;
  uint32_t tile_base;
};

constexpr int kWide = 64;  // tiles above which a record goes to the warp path

// Record start of each frame of one class (rows j0 .. j0+m-1 of the projection
// order, word bases wbase relative to the class's first word; word_off is the
// class's own exclusive scan) and the class's live count at [m].
__global__ void k_frame_bounds(const uint32_t *__restrict__ word_off,
                               const uint32_t *__restrict__ wbase, int j0, int m,
                               int64_t nwords, const uint32_t *__restrict__ total,
                               uint32_t *__restrict__ actv_start) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= m; k += gridDim.x * blockDim.x) {
    const int64_t w = k < m ? (int64_t)wbase[j0 + k] : nwords;
    actv_start[k] = (k == m || w >= nwords) ? *total : word_off[w];
  }
}

// Frame of every live record of one class segment (binary search over the
// class's record starts, frame ids from fmap); sentinels past the live count:
// key all ones, frame nf, no tiles.
__global__ void k_batch_records(const uint32_t *__restrict__ actv_start, int m,
                                const uint32_t *__restrict__ fmap, int nf, uint32_t cap,
                                uint32_t *__restrict__ key, uint32_t *__restrict__ count,
                                uint32_t *__restrict__ frame, uint32_t *status) {
  const uint32_t live = actv_start[m];
  if (blockIdx.x == 0 && threadIdx.x == 0 && live > cap) atomicOr(status, 1u);
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < cap;
       r += (int64_t)gridDim.x * blockDim.x) {
    if (r < live) {
      int lo = 0, hi = m;  // last k with actv_start[k] <= r
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (actv_start[mid] <= (uint32_t)r) lo = mid; else hi = mid;
      }
      frame[r] = fmap[lo];
    } else {
      frame[r] = (uint32_t)nf;
      key[r] = 0xffffffffu;
      count[r] = 0u;
    }
  }
}

// Visiting order of all records: additive records in place, then the ordered
// segment in its sorted order.
__global__ void k_compose_order(const uint32_t *__restrict__ perm_ord, uint32_t cap_add,
                                uint32_t cap_ord, uint32_t *__restrict__ order) {
  const int64_t total = (int64_t)cap_add + cap_ord;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < total;
       s += (int64_t)gridDim.x * blockDim.x)
    order[s] = s < cap_add ? (uint32_t)s : cap_add + perm_ord[s - cap_add];
}

// One warp per 32 consecutive visiting positions, the cells of its narrow
// records dealt to the lanes 32 at a time, as k_emit_narrow does for one
// frame; each record brings its frame's tiling and global tile base.  A
// record whose slots pass the capacity is not dealt: it raises the status bit
// and turns its slots below the capacity into sentinels (the render is redone
// after a re-plan).
__global__ void __launch_bounds__(256) k_emit_batch_narrow(
    const float4 *__restrict__ pos, const uint32_t *__restrict__ count,
    const uint32_t *__restrict__ order, const uint64_t *__restrict__ off, int64_t n,
    const uint32_t *__restrict__ frame, const FrameTile *__restrict__ ft, uint64_t cap,
    uint32_t *__restrict__ tkey, uint32_t *__restrict__ tval, uint32_t *__restrict__ wide_list,
    uint32_t *__restrict__ wide_n, uint32_t *status) {
  __shared__ uint32_t cpre[256 / 32][32];  // per warp: exclusive cell prefix of its lanes
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const int64_t nchunk = (n + 31) / 32;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t ch = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; ch < nchunk;
       ch += nwarp) {
    const int64_t s = ch * 32 + lane;
    const uint32_t c = s < n ? __ldg(count + s) : 0u;
    const uint64_t o = s < n ? __ldg(off + s) : 0u;
    const uint32_t i = s < n ? (order ? __ldg(order + s) : (uint32_t)s) : 0u;
    bool narrow = false;
    if (c > 0u) {
      if (o + c > cap) {
        atomicOr(status, 2u);
        for (uint64_t q = o; q < cap && q < o + c; ++q) {
          tkey[q] = 0xffffffffu;
          tval[q] = 0u;
        }
      } else if (c > (uint32_t)kWide) {
        wide_list[atomicAdd(wide_n, 1u)] = (uint32_t)s;
      } else {
        narrow = true;
      }
    }
    float px = 0.f, py = 0.f, sumsq = 0.f, cmid0 = 0.f;
    int minx = 0, miny = 0, wy = 1, T = 1, ncx = 0;
    uint32_t cells = 0, magic = 0, base = 0;
    if (narrow) {
      const float4 p = __ldg(pos + i);
      const FrameTile t = ft[__ldg(frame + i)];
      px = p.x;
      py = p.y;
      T = t.g.T;
      ncx = t.g.ncx;
      cmid0 = t.g.cmid0;
      base = t.tile_base;
      const float rfacr = fmul(0.75f, p.z);
      minx = max(0, f2i(fadd(fsub(px, rfacr), 1.f)) / T);
      const int maxx = min(t.g.ncx - 1, f2i(fadd(px, rfacr)) / T);
      miny = max(0, f2i(fadd(fsub(py, rfacr), 1.f)) / T);
      const int maxy = min(t.g.ncy - 1, f2i(fadd(py, rfacr)) / T);
      const float rs = fadd(t.g.rcell, rfacr);
      sumsq = fmul(rs, rs);
      wy = maxy - miny + 1;
      cells = (uint32_t)((maxx - minx + 1) * wy);
      magic = wy > 1 ? 0xffffffffu / (uint32_t)wy + 1u : 0u;  // q / wy = umulhi(q, magic)
    }
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
    const uint32_t nexcl = nin - (narrow ? c : 0u);
    __syncwarp();
    cpre[w][lane] = cin - cells;
    __syncwarp();
    uint32_t carry = 0;
    for (uint32_t k0 = 0; k0 < total; k0 += 32) {
      const uint32_t k = k0 + (uint32_t)lane;
      int l = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1)
        if (cpre[w][l + step] <= k) l += step;
      const int lminx = __shfl_sync(0xffffffffu, minx, l);
      const int lminy = __shfl_sync(0xffffffffu, miny, l);
      const int lwy = __shfl_sync(0xffffffffu, wy, l);
      const int lT = __shfl_sync(0xffffffffu, T, l);
      const int lncx = __shfl_sync(0xffffffffu, ncx, l);
      const uint32_t lmag = __shfl_sync(0xffffffffu, magic, l);
      const float lpx = __shfl_sync(0xffffffffu, px, l);
      const float lpy = __shfl_sync(0xffffffffu, py, l);
      const float lsq = __shfl_sync(0xffffffffu, sumsq, l);
      const float lcm = __shfl_sync(0xffffffffu, cmid0, l);
      const uint32_t lbase = __shfl_sync(0xffffffffu, base, l);
      const uint32_t lc = __shfl_sync(0xffffffffu, c, l);
      const uint32_t lnex = __shfl_sync(0xffffffffu, nexcl, l);
      const uint32_t li = __shfl_sync(0xffffffffu, i, l);
      const uint32_t lolo = __shfl_sync(0xffffffffu, (uint32_t)o, l);
      const uint32_t lohi = __shfl_sync(0xffffffffu, (uint32_t)(o >> 32), l);
      const uint32_t q = k - cpre[w][l];
      const uint32_t qx = lwy > 1 ? __umulhi(q, lmag) : q;
      const int ix = lminx + (int)qx;
      const int iy = lminy + (int)(q - qx * (uint32_t)lwy);
      bool pass = false;
      if (k < total) {  // the test of for_each_tile, operation for operation
        const float cx = fadd(lcm, (float)(ix * lT));
        const float dx = fsub(lpx, cx);
        const float dx2 = fmul(dx, dx);
        const float cy = fadd(lcm, (float)(iy * lT));
        const float dy = fsub(lpy, cy);
        pass = fadd(dx2, fmul(dy, dy)) < lsq;
      }
      const uint32_t b = __ballot_sync(0xffffffffu, pass);
      const uint32_t j = carry + __popc(b & lt) - lnex;
      if (pass && j < lc) {
        const uint64_t slot = (((uint64_t)lohi << 32) | lolo) + j;
        tkey[slot] = lbase + (uint32_t)(iy * lncx + ix);
        tval[slot] = li;
      } else if (pass) {
        atomicOr(status, 4u);  // more passing tiles than counted: reported, not stored
      }
      carry += __popc(b);
    }
  }
}

// One warp per wide record: lane l takes tile rows miny + l, +32, ...
__global__ void __launch_bounds__(256) k_emit_batch_wide(
    const float4 *__restrict__ pos, const uint32_t *__restrict__ count,
    const uint32_t *__restrict__ order, const uint64_t *__restrict__ off,
    const uint32_t *__restrict__ wide_list, const uint32_t *__restrict__ wide_n,
    const uint32_t *__restrict__ frame, const FrameTile *__restrict__ ft,
    uint32_t *__restrict__ tkey, uint32_t *__restrict__ tval, uint32_t *status) {
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t nw = *wide_n;
  for (int64_t w = warp0; w < nw; w += nwarps) {
    const uint32_t s = wide_list[w];
    const uint32_t i = order ? __ldg(order + s) : s;
    const FrameTile t = ft[__ldg(frame + i)];
    const Tiling &g = t.g;
    const uint64_t o = __ldg(off + s);
    const uint64_t oend = o + __ldg(count + s);  // the record's slots end here
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
        const float dy = fsub(p.y, fadd(g.cmid0, (float)(iy * T)));
        dy2 = fmul(dy, dy);
        for (int ix = minx; ix <= maxx; ++ix) {
          const float dx = fsub(p.x, fadd(g.cmid0, (float)(ix * T)));
          if (fadd(fmul(dx, dx), dy2) < sumsq) ++rc;
        }
      }
      int incl = rc;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      uint64_t slot = base + (uint64_t)(incl - rc);
      if (iy <= maxy && rc > 0) {
        for (int ix = minx; ix <= maxx; ++ix) {
          const float dx = fsub(p.x, fadd(g.cmid0, (float)(ix * T)));
          if (fadd(fmul(dx, dx), dy2) < sumsq) {
            if (slot < oend) {
              tkey[slot] = t.tile_base + (uint32_t)(iy * g.ncx + ix);
              tval[slot] = i;
            } else {
              atomicOr(status, 4u);  // more passing tiles than counted: reported, not stored
            }
            ++slot;
          }
        }
      }
      base += (uint64_t)total;
    }
  }
}

__global__ void k_fill_tail(uint32_t *__restrict__ key, const uint64_t *__restrict__ live,
                            uint64_t cap) {
  const uint64_t from = min(*live, cap);
  for (uint64_t p = from + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < cap;
       p += (uint64_t)gridDim.x * blockDim.x)
    key[p] = 0xffffffffu;
}

// tile_start[t] = first sorted position whose key is >= t; sentinel keys
// (past every real tile) count as ntiles.
__global__ void k_tile_ranges_clamped(const uint32_t *__restrict__ key, int64_t ne,
                                      int64_t ntiles, uint32_t *__restrict__ tile_start) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p <= ne;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t kprev = p > 0 ? min((int64_t)key[p - 1], ntiles) : -1;
    const int64_t kcur = p < ne ? min((int64_t)key[p], ntiles) : ntiles;
    for (int64_t t = kprev + 1; t <= kcur; ++t) tile_start[t] = (uint32_t)p;
  }
}

// Queue key: class (0 additive, 1 ordered) above an inverted 8-bit log of the
// list length, so one ascending sort gives each class longest-first.
__global__ void k_tile_cost_class(const uint32_t *__restrict__ tile_start, int64_t ntiles,
                                  const uint32_t *__restrict__ frame_of_tile,
                                  const uint8_t *__restrict__ frame_ordered,
                                  uint32_t *__restrict__ key) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntiles;
       t += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t cnt = tile_start[t + 1] - tile_start[t];
    const int lg = (int)(8.f * __log2f((float)cnt + 1.f));
    key[t] = ((uint32_t)frame_ordered[frame_of_tile[t]] << 8) | (255u - (uint32_t)min(lg, 255));
  }
}

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b > 0 ? b : 1);
}

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

}  // namespace
}  // namespace spl

using spl::DevBuf;

struct spl_batch {
  spl_context *ctx = nullptr;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t stream2 = nullptr;              // the ordered class's splat queue
  cudaEvent_t fork = nullptr, join = nullptr;  // stream <-> stream2 (no timing)
  std::vector<spl_particles> sets;
  std::vector<spl_batch_frame> frames;  // descs point at the palette copies below
  std::vector<std::vector<double>> pal_x_copy;
  std::vector<std::vector<float>> pal_rgb_copy;
  spl_batch_options opt{};
  int T = 16, cfg_add = 0, cfg_abs = 2;
  bool ord_all_ftb = true;  // every ordered frame composites front-to-back
  // palette cache: per set, the frame whose constants colourise the set once
  // per render for all its frames (-1: not cached), and its offset in pal_cache
  std::vector<int> cache_frame;
  std::vector<int64_t> cache_off;
  // plan.  Projection order: additive frames, then ordered ones; records of
  // the two classes live in separate segments, [0, cap_add) and
  // [cap_add, cap_add + cap_ord), so that only ordered records are sorted.
  std::vector<spl::FrameSetup> fs;
  std::vector<spl::ProjConst> pc;      // device palette pointers filled in
  std::vector<int> proj;               // projection order -> frame
  int n_add_frames = 0;
  std::vector<uint32_t> wbase;         // activity-word base per projection row,
                                       // relative to its class's first word
  std::vector<uint32_t> tbase;         // global tile base per frame (+ total)
  int64_t nwords = 0, nw_add = 0, ntiles = 0, n_add_tiles = 0;
  int64_t cap_add = 0, cap_ord = 0, cap_a = 0, cap_e = 0;
  uint32_t fblocks = 0, dblocks = 0;
  int frame_bits = 1, tile_bits = 1;
  std::vector<DevBuf *> owned;
  DevBuf pal_x, pal_rgb, pal_thr, pal_xff, pal_invff;
  DevBuf flags, word_off, d_wbase, pal_cache, d_tbase, ftab, actv_add, actv_ord, fmap_add, fmap_ord;
  DevBuf pos_c, col_c, idx_c, count_c, key_c, frame_c;
  DevBuf ktmp, vtmp, kout, perm1, fkey, perm, order, count_seq, off, wide_list, radix_scr;
  DevBuf tkey, tval, tkey2, tval2, tkey_s, tval_s;
  DevBuf tile_start, tcost, tcost_s, work, work_tmp, frame_of_tile, frame_ord, ft, splat_args;
  DevBuf status;  // [0] overflow bits, [1] wide count, [2],[3] queue counters,
                  // [4] error word, [5] live additive records, [6] live ordered
  uint32_t *h_status = nullptr;  // pinned copy of the first 8 status words
  uint64_t *h_entries = nullptr; // pinned copy of the live entry count
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int launches = 0;
  spl_batch_info info{};
};

namespace {

spl_status fail(spl_status code, const std::string &msg) { return spl::host_fail(code, msg); }

#define BCK(call)                                                                       \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      cudaGetLastError();                                                               \
      return fail(SPL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
    }                                                                                   \
  } while (0)

spl_status dev_alloc(spl_batch *b, DevBuf &d, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (d.bytes >= bytes) return SPL_OK;
  if (d.p) cudaFree(d.p);
  d.p = nullptr;
  d.bytes = 0;
  if (spl::alloc_failure_due())
    return fail(SPL_ERR_ALLOC, "batch: cudaMalloc(" + std::to_string(bytes) +
                                   "): failure injected by spl_debug_fail_alloc");
  cudaError_t e = cudaMalloc(&d.p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SPL_ERR_ALLOC, "batch: cudaMalloc(" + std::to_string(bytes) + "): " +
                                   cudaGetErrorString(e));
  }
  d.bytes = bytes;
  if (std::find(b->owned.begin(), b->owned.end(), &d) == b->owned.end()) b->owned.push_back(&d);
  return SPL_OK;
}

template <typename T>
T *as(DevBuf &d) {
  return static_cast<T *>(d.p);
}

void drop_graph(spl_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

const void *set_aos(const spl_particles &p) {
  return p.layout == SPL_LAYOUT_AOS ? p.aos : nullptr;
}

spl::SoAIn set_soa(const spl_particles &p) {
  return spl::SoAIn{p.x, p.y, p.z, p.r, p.I, p.cr, p.cg, p.cb, p.type};
}

// Measured sizes at tile size T: one plain render of every frame on the
// context (its image lands in the frame's buffer and is redrawn by the batch).
spl_status measure(spl_batch *b, int T, int64_t &acts_add, int64_t &acts_ord, int64_t &ents) {
  acts_add = acts_ord = ents = 0;
  for (const auto &fr : b->frames) {
    spl_frame_desc d = fr.desc;
    d.tile_size = T;
    d.splat_config = -1;
    spl_image img{fr.pic, SPL_MEM_DEVICE};
    spl_status st = spl_render(b->ctx, &d, &b->sets[fr.set], &img, SPL_WRITEBACK_NONE);
    if (st) return st;
    spl_stats s;
    spl_get_stats(b->ctx, &s);
    (fr.desc.a_eq_e ? acts_add : acts_ord) += s.n_active;
    ents += s.n_entries;
  }
  return SPL_OK;
}

// Buffers, per-frame constants and the static tables for tile size T and the
// given capacities.
spl_status plan(spl_batch *b, int T, int64_t cap_add, int64_t cap_ord, int64_t cap_e) {
  drop_graph(b);
  const int nf = (int)b->frames.size();
  b->T = T;
  b->fs.assign(nf, spl::FrameSetup());
  b->pc.assign(nf, spl::ProjConst());
  b->tbase.assign(nf + 1, 0);
  int64_t npal = 0, tiles = 0, add_tiles = 0;
  std::vector<uint8_t> ordered(nf, 0);
  spl_status st;
  b->proj.clear();
  for (int f = 0; f < nf; ++f) {
    const spl_batch_frame &fr = b->frames[f];
    if ((st = spl::frame_setup(&fr.desc, T, false, b->fs[f]))) return st;
    b->tbase[f] = (uint32_t)tiles;
    tiles += b->fs[f].ntiles;
    npal += b->fs[f].npal + 1;
    ordered[f] = fr.desc.a_eq_e ? 0 : 1;
    if (fr.desc.a_eq_e) {
      add_tiles += b->fs[f].ntiles;
      b->proj.push_back(f);
    }
  }
  b->n_add_frames = (int)b->proj.size();
  // palette cache: a set is colourised once per render when it has two or
  // more frames and they all use the same palettes and colour-vector flags
  const int ns = (int)b->sets.size();
  b->cache_frame.assign(ns, -1);
  b->cache_off.assign(ns, 0);
  int64_t cache_n = 0;
  {
    std::vector<int> nfr(ns, 0);
    for (int f = 0; f < nf; ++f) {
      const int si = b->frames[f].set;
      const spl::FrameSetup &a = b->fs[f];
      if (nfr[si]++ == 0) {
        b->cache_frame[si] = f;
        continue;
      }
      const int f0 = b->cache_frame[si];
      if (f0 < 0) continue;
      const spl::FrameSetup &z = b->fs[f0];
      bool same = a.pal_x == z.pal_x && a.pal_rgb == z.pal_rgb && a.pc.ptypes == z.pc.ptypes &&
                  a.pc.exact_fp64 == z.pc.exact_fp64;
      for (int t = 0; same && t < a.pc.ptypes; ++t)
        same = a.pc.colvec[t] == z.pc.colvec[t] && a.pc.pal_off[t] == z.pc.pal_off[t] &&
               a.pc.pal_n[t] == z.pc.pal_n[t];
      if (!same) b->cache_frame[si] = -1;
    }
    for (int si = 0; si < ns; ++si) {
      const int f0 = b->cache_frame[si];
      bool any_palette = false;
      if (f0 >= 0)
        for (int t = 0; t < b->fs[f0].pc.ptypes; ++t) any_palette |= !b->fs[f0].pc.colvec[t];
      if (f0 < 0 || nfr[si] < 2 || !any_palette) {
        b->cache_frame[si] = -1;
        continue;
      }
      b->cache_off[si] = cache_n;
      cache_n += b->sets[si].n;
    }
  }
  for (int f = 0; f < nf; ++f)
    if (ordered[f]) b->proj.push_back(f);
  // activity words in projection order, based per class
  b->wbase.assign(nf + 1, 0);
  int64_t words = 0, nw_add = 0, fblocks = 0, dblocks = 0;
  std::vector<uint32_t> fb0(nf), db0(nf);
  for (int j = 0; j < nf; ++j) {
    if (j == b->n_add_frames) nw_add = words;
    b->wbase[j] = (uint32_t)(words - (j >= b->n_add_frames ? nw_add : 0));
    const int64_t w = (b->sets[b->frames[b->proj[j]].set].n + 31) / 32;
    fb0[j] = (uint32_t)fblocks;
    db0[j] = (uint32_t)dblocks;
    fblocks += (w + spl::kFlagWordsPerBlock - 1) / spl::kFlagWordsPerBlock;
    dblocks += (w + spl::kDenseWordsPerBlock - 1) / spl::kDenseWordsPerBlock;
    words += w;
  }
  if (b->n_add_frames == nf) nw_add = words;
  if (tiles >= 0x7fffffffLL || words >= 0xffffffffLL || cap_add + cap_ord >= 0xffffffffLL ||
      cap_e >= 0xffffffffLL || fblocks >= 0x7fffffffLL)
    return fail(SPL_ERR_CAPACITY, "batch: more than 2^31 tiles or 2^32 records/entries");
  b->tbase[nf] = (uint32_t)tiles;
  b->nwords = words;
  b->nw_add = nw_add;
  b->fblocks = (uint32_t)fblocks;
  b->dblocks = (uint32_t)dblocks;
  b->ntiles = tiles;
  b->n_add_tiles = add_tiles;
  b->cap_add = cap_add;
  b->cap_ord = cap_ord;
  b->cap_a = std::max<int64_t>(cap_add + cap_ord, 1);
  b->cap_e = std::max<int64_t>(cap_e, 1);
  b->frame_bits = spl::bits_for(nf + 1);
  b->tile_bits = spl::bits_for(tiles + 1);
  const int64_t A = b->cap_a, E = b->cap_e, O = std::max<int64_t>(cap_ord, 1);

  // ---- buffers -------------------------------------------------------------
  size_t scan_b = spl::scan_scratch_bytes(std::max<int64_t>(words, A + 1));
  size_t radix_b = std::max(spl::radix_scratch_bytes(A), spl::radix_scratch_bytes(E));
  radix_b = std::max(radix_b, spl::radix_scratch_bytes(tiles));
  radix_b = std::max(radix_b, scan_b);
  if ((st = dev_alloc(b, b->pal_x, npal * 8)) || (st = dev_alloc(b, b->pal_rgb, npal * 12)) ||
      (st = dev_alloc(b, b->pal_thr, npal * 4)) || (st = dev_alloc(b, b->pal_xff, npal * 8)) ||
      (st = dev_alloc(b, b->pal_invff, npal * 8)) ||
      (st = dev_alloc(b, b->flags, words * 4)) || (st = dev_alloc(b, b->word_off, words * 4)) ||
      (st = dev_alloc(b, b->d_wbase, (nf + 1) * 4)) ||
      (st = dev_alloc(b, b->d_tbase, (nf + 1) * 4)) ||
      (st = dev_alloc(b, b->ftab, nf * sizeof(spl::FrameProj))) ||
      (st = dev_alloc(b, b->pal_cache, cache_n * 16)) ||
      (st = dev_alloc(b, b->actv_add, (nf + 1) * 4)) ||
      (st = dev_alloc(b, b->actv_ord, (nf + 1) * 4)) ||
      (st = dev_alloc(b, b->fmap_add, (nf + 1) * 4)) ||
      (st = dev_alloc(b, b->fmap_ord, (nf + 1) * 4)) ||
      (st = dev_alloc(b, b->pos_c, A * 16)) || (st = dev_alloc(b, b->col_c, A * 16)) ||
      (st = dev_alloc(b, b->idx_c, A * 4)) || (st = dev_alloc(b, b->count_c, A * 4)) ||
      (st = dev_alloc(b, b->key_c, A * 4)) || (st = dev_alloc(b, b->frame_c, A * 4)) ||
      (st = dev_alloc(b, b->ktmp, O * 4)) || (st = dev_alloc(b, b->vtmp, O * 4)) ||
      (st = dev_alloc(b, b->kout, O * 4)) || (st = dev_alloc(b, b->perm1, O * 4)) ||
      (st = dev_alloc(b, b->fkey, O * 4)) || (st = dev_alloc(b, b->perm, O * 4)) ||
      (st = dev_alloc(b, b->order, A * 4)) ||
      (st = dev_alloc(b, b->count_seq, A * 4)) || (st = dev_alloc(b, b->off, (A + 1) * 8)) ||
      (st = dev_alloc(b, b->wide_list, A * 4)) || (st = dev_alloc(b, b->radix_scr, radix_b)) ||
      (st = dev_alloc(b, b->tkey, E * 4)) || (st = dev_alloc(b, b->tval, E * 4)) ||
      (st = dev_alloc(b, b->tkey2, E * 4)) || (st = dev_alloc(b, b->tval2, E * 4)) ||
      (st = dev_alloc(b, b->tkey_s, E * 4)) || (st = dev_alloc(b, b->tval_s, E * 4)) ||
      (st = dev_alloc(b, b->tile_start, (tiles + 1) * 4)) ||
      (st = dev_alloc(b, b->tcost, tiles * 4)) || (st = dev_alloc(b, b->tcost_s, tiles * 4)) ||
      (st = dev_alloc(b, b->work, tiles * 4)) || (st = dev_alloc(b, b->work_tmp, tiles * 4)) ||
      (st = dev_alloc(b, b->frame_of_tile, tiles * 4)) ||
      (st = dev_alloc(b, b->frame_ord, nf)) ||
      (st = dev_alloc(b, b->ft, nf * sizeof(spl::FrameTile))) ||
      (st = dev_alloc(b, b->splat_args, nf * sizeof(spl::SplatArgs))) ||
      (st = dev_alloc(b, b->status, 64)))
    return st;

  // ---- static tables ---------------------------------------------------------
  std::vector<double> px;
  std::vector<float> prgb, pthr;
  std::vector<float2> pxff, pinvff;
  std::vector<uint32_t> fot((size_t)tiles);
  std::vector<spl::FrameTile> fts(nf);
  std::vector<spl::SplatArgs> sas(nf);
  b->ord_all_ftb = true;
  const float h2sigma =
      (float)(0.5 * std::pow(3.141592653589793238462643383279502884197, -1. / 6.));
  for (int f = 0; f < nf; ++f) {
    const spl::FrameSetup &s = b->fs[f];
    const size_t o = px.size();
    px.insert(px.end(), s.pal_x.begin(), s.pal_x.end());
    prgb.insert(prgb.end(), s.pal_rgb.begin(), s.pal_rgb.end());
    pthr.insert(pthr.end(), s.thr.begin(), s.thr.end());
    pxff.insert(pxff.end(), s.xff.begin(), s.xff.end());
    pinvff.insert(pinvff.end(), s.invff.begin(), s.invff.end());
    spl::ProjConst c = s.pc;
    c.pal_x = as<double>(b->pal_x) + o;
    c.pal_rgb = as<float>(b->pal_rgb) + 3 * o;
    c.pal_thr = as<float>(b->pal_thr) + o;
    c.pal_xff = as<float2>(b->pal_xff) + o;
    c.pal_invff = as<float2>(b->pal_invff) + o;
    c.n_fallback = nullptr;
    const int si = b->frames[f].set;
    c.pal_cache = b->cache_frame[si] >= 0 ? as<float4>(b->pal_cache) + b->cache_off[si] : nullptr;
    b->pc[f] = c;
    for (int64_t t = 0; t < s.ntiles; ++t) fot[b->tbase[f] + t] = (uint32_t)f;
    fts[f].g = s.g;
    fts[f].tile_base = b->tbase[f];
    const spl_frame_desc &d = b->frames[f].desc;
    spl::SplatArgs &a = sas[f];
    std::memset(&a, 0, sizeof(a));
    a.pos = as<float4>(b->pos_c);
    a.col = as<float4>(b->col_c);
    a.entries = as<uint32_t>(b->tval_s);
    a.tile_start = as<uint32_t>(b->tile_start) + b->tbase[f];
    a.tile_order = nullptr;
    a.T = T;
    a.ncx = s.g.ncx;
    a.ncy = s.g.ncy;
    a.xres = d.xres;
    a.yres = d.yres;
    a.gray = d.gray_absorption;
    a.h2sigma = h2sigma;
    a.a_eq_e = d.a_eq_e ? 1 : 0;
    a.order_mode = d.order_mode;
    if (!d.a_eq_e && d.order_mode != 1) b->ord_all_ftb = false;
    a.ftb_eps = d.ftb_epsilon;
    a.ftb_rel = d.ftb_relative;
    a.config = -1;
    a.pic = b->frames[f].pic;
  }
  // projection table (projection order) and the frame ids of each class
  std::vector<spl::FrameProj> ftab(nf);
  std::vector<uint32_t> fmap_add, fmap_ord;
  for (int j = 0; j < nf; ++j) {
    const int f = b->proj[j];
    const bool add = j < b->n_add_frames;
    const spl_particles &p = b->sets[b->frames[f].set];
    spl::FrameProj &t = ftab[j];
    std::memset(&t, 0, sizeof(t));
    t.c = b->pc[f];
    t.aos = set_aos(p);
    t.soa = set_soa(p);
    t.n = p.n;
    const int64_t seg = add ? 0 : b->cap_add;          // first record of the class
    const int64_t w = b->wbase[j] + (add ? 0 : nw_add);  // first word, absolute
    t.o.flags = as<uint32_t>(b->flags) + w;
    t.o.word_off = as<uint32_t>(b->word_off) + w;
    t.o.pos_c = as<float4>(b->pos_c) + seg;
    t.o.col_c = as<float4>(b->col_c) + seg;
    t.o.idx_c = as<uint32_t>(b->idx_c) + seg;
    t.o.count_c = as<uint32_t>(b->count_c) + seg;
    t.o.key_c = as<uint32_t>(b->key_c) + seg;
    t.o.cap_c = (uint32_t)(add ? b->cap_add : b->cap_ord);
    t.o.err = as<uint32_t>(b->status) + 4;
    t.fblock0 = fb0[j];
    t.dblock0 = db0[j];
    (add ? fmap_add : fmap_ord).push_back((uint32_t)f);
  }
  fmap_add.push_back(0);
  fmap_ord.push_back(0);
  cudaStream_t s = b->stream;
  BCK(cudaMemcpyAsync(b->ftab.p, ftab.data(), nf * sizeof(spl::FrameProj),
                      cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->fmap_add.p, fmap_add.data(), fmap_add.size() * 4,
                      cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->fmap_ord.p, fmap_ord.data(), fmap_ord.size() * 4,
                      cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->pal_x.p, px.data(), px.size() * 8, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->pal_rgb.p, prgb.data(), prgb.size() * 4, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->pal_thr.p, pthr.data(), pthr.size() * 4, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->pal_xff.p, pxff.data(), pxff.size() * 8, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->pal_invff.p, pinvff.data(), pinvff.size() * 8, cudaMemcpyHostToDevice,
                      s));
  BCK(cudaMemcpyAsync(b->d_wbase.p, b->wbase.data(), (nf + 1) * 4, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->d_tbase.p, b->tbase.data(), (nf + 1) * 4, cudaMemcpyHostToDevice, s));
  if (tiles)
    BCK(cudaMemcpyAsync(b->frame_of_tile.p, fot.data(), tiles * 4, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->frame_ord.p, ordered.data(), nf, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->ft.p, fts.data(), nf * sizeof(spl::FrameTile), cudaMemcpyHostToDevice,
                      s));
  BCK(cudaMemcpyAsync(b->splat_args.p, sas.data(), nf * sizeof(spl::SplatArgs),
                      cudaMemcpyHostToDevice, s));
  BCK(cudaStreamSynchronize(s));
  b->info.cap_active = b->cap_a;
  b->info.cap_entries = b->cap_e;
  b->info.total_tiles = tiles;
  b->info.tile_size = T;
  return SPL_OK;
}

// The work queue of one class: 0 additive frames (the first n_add_tiles
// items), 1 ordered frames (the rest); counter in status word 2 + cls.
spl::BatchSplatArgs queue_args(spl_batch *b, int cls) {
  spl::BatchSplatArgs q;
  q.frames = as<spl::SplatArgs>(b->splat_args);
  q.tile_base = as<uint32_t>(b->d_tbase);
  q.frame_of_tile = as<uint32_t>(b->frame_of_tile);
  q.work = as<uint32_t>(b->work);
  q.T = b->T;
  q.work_begin = cls == 0 ? 0u : (uint32_t)b->n_add_tiles;
  q.nwork = cls == 0 ? (uint32_t)b->n_add_tiles : (uint32_t)(b->ntiles - b->n_add_tiles);
  q.counter = as<uint32_t>(b->status) + 2 + cls;
  q.mode = cls == 0 ? 0 : (b->ord_all_ftb ? 1 : 2);
  return q;
}

// Every kernel of one batch render, in stream order (eager or under capture).
// splat_class: -1 both queues, 0 additive only, 1 ordered only, 2 none.
spl_status enqueue(spl_batch *b, cudaStream_t s, int splat_class = -1) {
  const int nf = (int)b->frames.size();
  int launches = 0;
  uint32_t *status = as<uint32_t>(b->status);
  uint32_t *err = status + 4;
  const uint32_t capA = (uint32_t)b->cap_a;
  const uint64_t capE = (uint64_t)b->cap_e;
  BCK(cudaMemsetAsync(status, 0, 64, s));
  // ---- projection: one flags launch, one scan per class, one dense launch -------
  const int n_add = b->n_add_frames, n_ord = nf - n_add;
  const int64_t nw_ord = b->nwords - b->nw_add;
  const spl::FrameProj *tab = as<spl::FrameProj>(b->ftab);
  // palette colours of the sets that several frames share, once per render
  for (int si = 0; si < (int)b->sets.size(); ++si) {
    const int f0 = b->cache_frame[si];
    if (f0 < 0) continue;
    const spl_particles &p = b->sets[si];
    const spl::SoAIn soa = set_soa(p);
    spl::launch_palette_cache(set_aos(p), &soa, p.n, b->pc[f0],
                              as<float4>(b->pal_cache) + b->cache_off[si], s);
    ++launches;
  }
  spl::launch_project_flags_multi(tab, nf, b->fblocks, s);
  ++launches;
  uint32_t *flags = as<uint32_t>(b->flags), *woff = as<uint32_t>(b->word_off);
  if (n_add > 0) {
    spl::scan_popc(flags, b->nw_add, woff, status + 5, b->radix_scr.p, s, &launches);
    spl::k_frame_bounds<<<1, 256, 0, s>>>(woff, as<uint32_t>(b->d_wbase), 0, n_add, b->nw_add,
                                          status + 5, as<uint32_t>(b->actv_add));
    ++launches;
  }
  if (n_ord > 0) {
    spl::scan_popc(flags + b->nw_add, nw_ord, woff + b->nw_add, status + 6, b->radix_scr.p, s,
                   &launches);
    spl::k_frame_bounds<<<1, 256, 0, s>>>(woff + b->nw_add, as<uint32_t>(b->d_wbase), n_add,
                                          n_ord, nw_ord, status + 6, as<uint32_t>(b->actv_ord));
    ++launches;
  }
  spl::launch_project_dense_multi(tab, nf, b->dblocks, s);
  ++launches;
  if (n_add > 0 && b->cap_add > 0) {
    spl::k_batch_records<<<spl::grid_for(b->cap_add), 256, 0, s>>>(
        as<uint32_t>(b->actv_add), n_add, as<uint32_t>(b->fmap_add), nf, (uint32_t)b->cap_add,
        as<uint32_t>(b->key_c), as<uint32_t>(b->count_c), as<uint32_t>(b->frame_c), status);
    ++launches;
  }
  const int64_t seg = b->cap_add;
  if (n_ord > 0 && b->cap_ord > 0) {
    spl::k_batch_records<<<spl::grid_for(b->cap_ord), 256, 0, s>>>(
        as<uint32_t>(b->actv_ord), n_ord, as<uint32_t>(b->fmap_ord), nf, (uint32_t)b->cap_ord,
        as<uint32_t>(b->key_c) + seg, as<uint32_t>(b->count_c) + seg,
        as<uint32_t>(b->frame_c) + seg, status);
    ++launches;
  }
  // ---- visiting order: additive records as they are; the ordered segment
  //      stable by depth key, then stable by frame ------------------------------------
  const uint32_t *order = nullptr;
  if (n_ord > 0 && b->cap_ord > 0) {
    const int64_t O = b->cap_ord;
    spl::radix_sort_pairs(as<uint32_t>(b->key_c) + seg, nullptr, as<uint32_t>(b->ktmp),
                          as<uint32_t>(b->vtmp), as<uint32_t>(b->kout), as<uint32_t>(b->perm1),
                          O, 0, 32, false, b->radix_scr.p, s, &launches, err, true);
    spl::launch_gather_u32(as<uint32_t>(b->frame_c) + seg, as<uint32_t>(b->perm1), O,
                           as<uint32_t>(b->fkey), s);
    ++launches;
    spl::radix_sort_pairs(as<uint32_t>(b->fkey), as<uint32_t>(b->perm1), as<uint32_t>(b->ktmp),
                          as<uint32_t>(b->vtmp), as<uint32_t>(b->kout), as<uint32_t>(b->perm),
                          O, 0, b->frame_bits, false, b->radix_scr.p, s, &launches, err, true);
    spl::k_compose_order<<<spl::grid_for(capA), 256, 0, s>>>(
        as<uint32_t>(b->perm), (uint32_t)seg, (uint32_t)O, as<uint32_t>(b->order));
    ++launches;
    order = as<uint32_t>(b->order);
  }
  // ---- binning over all frames ------------------------------------------------------
  const uint32_t *count_seq = as<uint32_t>(b->count_c);
  if (order) {
    spl::launch_gather_u32(as<uint32_t>(b->count_c), order, capA, as<uint32_t>(b->count_seq), s);
    ++launches;
    count_seq = as<uint32_t>(b->count_seq);
  }
  uint64_t *off = as<uint64_t>(b->off);
  spl::scan_counts(count_seq, nullptr, capA, off, b->radix_scr.p, s, &launches);
  spl::k_emit_batch_narrow<<<spl::grid_for(capA), 256, 0, s>>>(
      as<float4>(b->pos_c), count_seq, order, off, capA, as<uint32_t>(b->frame_c),
      as<spl::FrameTile>(b->ft), capE, as<uint32_t>(b->tkey), as<uint32_t>(b->tval),
      as<uint32_t>(b->wide_list), status + 1, status);
  spl::k_emit_batch_wide<<<152 * 4, 256, 0, s>>>(
      as<float4>(b->pos_c), count_seq, order, off, as<uint32_t>(b->wide_list), status + 1,
      as<uint32_t>(b->frame_c), as<spl::FrameTile>(b->ft), as<uint32_t>(b->tkey),
      as<uint32_t>(b->tval), status);
  spl::k_fill_tail<<<spl::grid_for(capE), 256, 0, s>>>(as<uint32_t>(b->tkey), off + capA, capE);
  launches += 3;
  spl::radix_sort_pairs(as<uint32_t>(b->tkey), as<uint32_t>(b->tval), as<uint32_t>(b->tkey2),
                        as<uint32_t>(b->tval2), as<uint32_t>(b->tkey_s), as<uint32_t>(b->tval_s),
                        (int64_t)capE, 0, b->tile_bits, true, b->radix_scr.p, s, &launches, err,
                        true);
  spl::k_tile_ranges_clamped<<<spl::grid_for((int64_t)capE + 1), 256, 0, s>>>(
      as<uint32_t>(b->tkey_s), (int64_t)capE, b->ntiles, as<uint32_t>(b->tile_start));
  spl::k_tile_cost_class<<<spl::grid_for(b->ntiles), 256, 0, s>>>(
      as<uint32_t>(b->tile_start), b->ntiles, as<uint32_t>(b->frame_of_tile),
      as<uint8_t>(b->frame_ord), as<uint32_t>(b->tcost));
  launches += 2;
  spl::radix_sort_pairs(as<uint32_t>(b->tcost), nullptr, as<uint32_t>(b->tcost_s),
                        as<uint32_t>(b->work_tmp), as<uint32_t>(b->tcost_s),
                        as<uint32_t>(b->work), b->ntiles, 0, 9, false, b->radix_scr.p, s,
                        &launches, err, true);
  // ---- splat: one persistent launch per class; with both classes the ordered
  //      queue runs on a second stream, so that its CTAs start on the SMs the
  //      additive queue's CTAs leave as that queue drains -------------------------
  const bool both = splat_class == -1 && b->n_add_tiles > 0 && b->ntiles > b->n_add_tiles;
  if (both) {
    BCK(cudaEventRecord(b->fork, s));
    BCK(cudaStreamWaitEvent(b->stream2, b->fork, 0));
    launches += spl::launch_splat_queue(queue_args(b, 0), b->cfg_add, s);
    launches += spl::launch_splat_queue(queue_args(b, 1), b->cfg_abs, b->stream2);
    BCK(cudaEventRecord(b->join, b->stream2));
    BCK(cudaStreamWaitEvent(s, b->join, 0));
  } else {
    if (splat_class == -1 || splat_class == 0)
      launches += spl::launch_splat_queue(queue_args(b, 0), b->cfg_add, s);
    if (splat_class == -1 || splat_class == 1)
      launches += spl::launch_splat_queue(queue_args(b, 1), b->cfg_abs, s);
  }
  BCK(cudaMemcpyAsync(b->h_status, status, 32, cudaMemcpyDeviceToHost, s));
  BCK(cudaMemcpyAsync(b->h_entries, off + capA, 8, cudaMemcpyDeviceToHost, s));
  b->launches = launches;
  return SPL_OK;
}

spl_status capture(spl_batch *b) {
  drop_graph(b);
  cudaStream_t s = b->stream;
  BCK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  spl_status st = enqueue(b, s);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (st) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SPL_ERR_CUDA, std::string("batch: graph capture failed: ") + cudaGetErrorString(e));
  }
  e = cudaGraphInstantiate(&b->exec, g, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaGraphDestroy(g);
    return fail(SPL_ERR_CUDA, std::string("batch: graph instantiation failed: ") +
                                  cudaGetErrorString(e));
  }
  b->graph = g;
  return SPL_OK;
}

// One render (graph or eager), waiting for completion; returns the status
// words through the pinned copies.
spl_status run_once(spl_batch *b, float *ms) {
  cudaStream_t s = b->stream;
  BCK(cudaEventRecord(b->ev0, s));
  if (b->exec) {
    BCK(cudaGraphLaunch(b->exec, s));
  } else {
    spl_status st = enqueue(b, s);
    if (st) return st;
  }
  BCK(cudaEventRecord(b->ev1, s));
  BCK(cudaStreamSynchronize(s));
  BCK(cudaGetLastError());
  if (ms) cudaEventElapsedTime(ms, b->ev0, b->ev1);
  return SPL_OK;
}

spl_status check_status(spl_batch *b, bool &overflow) {
  const uint32_t *h = b->h_status;
  overflow = (h[0] & 3u) != 0 || (h[4] & 8u) != 0;
  if (h[4] & 1u) return fail(SPL_ERR_INVALID, "particle type outside [0, ptypes)");
  if (h[4] & 2u) return fail(SPL_ERR_TIMEOUT, "a look-back wait gave up");
  if (h[4] & 32u)
    return fail(SPL_ERR_INTERNAL, "the activity screen kept a particle the projection culls");
  if (h[0] & 4u)
    return fail(SPL_ERR_CAPACITY, "bin emission found more tiles than a record's count");
  return SPL_OK;
}

int64_t with_margin(int64_t v, float margin) {
  return (int64_t)std::ceil((double)v * (double)margin) + 1024;
}

spl_status build(spl_batch *b, int T) {
  int64_t acts_add, acts_ord, ents;
  spl_status st;
  if ((st = measure(b, T, acts_add, acts_ord, ents))) return st;
  const float m = b->opt.capacity_margin;
  return plan(b, T, acts_add ? with_margin(acts_add, m) : 0,
              acts_ord ? with_margin(acts_ord, m) : 0, with_margin(ents, m));
}

// Autotuner: for each tile size, the fastest splat configuration per class
// (persistent launch timed alone on this batch's bins), then the fastest tile
// size by timing the whole pipeline.
// The tuning cache: the autotuner's choice per batch shape, for the life of
// the process.  A shape is the device, the tile-size and configuration
// options, and per frame (sorted) its resolution, mode class and the size
// bucket of its particle set (floor(log2 n)): batches of the same shape take
// the cached choice and time nothing.
struct TuneChoice {
  int T, cfg_add, cfg_abs;
};
std::mutex g_tune_mu;
std::map<std::string, TuneChoice> g_tune_cache;

std::string tune_key(const spl_batch *b) {
  std::vector<std::string> fr;
  fr.reserve(b->frames.size());
  for (const auto &f : b->frames) {
    const int64_t n = b->sets[f.set].n;
    int lg = 0;
    while (lg < 62 && (int64_t(1) << (lg + 1)) <= n) ++lg;
    const spl_frame_desc &d = f.desc;
    fr.push_back(std::to_string(d.xres) + "x" + std::to_string(d.yres) + ":" +
                 (d.a_eq_e ? "add" : (d.order_mode == 1 ? "ftb" : "btf")) + ":" +
                 std::to_string(lg));
  }
  std::sort(fr.begin(), fr.end());
  std::string k = "dev" + std::to_string(b->device) + "/T" + std::to_string(b->opt.tile_size) +
                  "/a" + std::to_string(b->opt.splat_config_additive) + "/o" +
                  std::to_string(b->opt.splat_config_absorption);
  for (const auto &x : fr) k += "/" + x;
  return k;
}

spl_status autotune(spl_batch *b) {
  const auto t0 = std::chrono::steady_clock::now();
  const auto since = [](std::chrono::steady_clock::time_point t) {
    return std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t)
        .count();
  };
  spl_status st;
  const std::string key = b->opt.tune_cache ? tune_key(b) : std::string();
  if (b->opt.tune_cache) {
    TuneChoice c{};
    bool hit = false;
    {
      std::lock_guard<std::mutex> lock(g_tune_mu);
      auto it = g_tune_cache.find(key);
      if (it != g_tune_cache.end()) {
        c = it->second;
        hit = true;
      }
    }
    if (hit) {  // the measured plan at the cached tile size; nothing is timed
      b->cfg_add = c.cfg_add;
      b->cfg_abs = c.cfg_abs;
      if ((st = build(b, c.T))) return st;
      b->info.tune_ms = 0.f;
      b->info.tune_cached = 1;
      b->info.plan_ms = since(t0);
      return SPL_OK;
    }
  }
  std::vector<int> sizes;
  if (b->opt.tile_size > 0) sizes.push_back(b->opt.tile_size);
  else sizes = {8, 16, 32};
  bool has_add = false, has_ord = false;
  for (const auto &fr : b->frames) (fr.desc.a_eq_e ? has_add : has_ord) = true;
  float best_ms = 1e30f;
  int best_T = sizes[0], best_add = 0, best_abs = 0;
  for (int T : sizes) {
    if ((st = build(b, T))) return st;
    int cands[8], nc = 0;
    for (int c = 0; c < spl::splat_config_count(); ++c)
      if (spl::splat_config_valid(c, T)) cands[nc++] = c;
    if (nc == 0) continue;
    // bins of this tile size once; then each class's splat timed alone per
    // configuration (second of two launches)
    if ((st = enqueue(b, b->stream, 2))) return st;
    BCK(cudaStreamSynchronize(b->stream));
    bool overflow = false;
    if ((st = check_status(b, overflow))) return st;
    for (int cls = 0; cls < 2; ++cls) {
      const bool present = cls == 0 ? has_add : has_ord;
      const int fixed = cls == 0 ? b->opt.splat_config_additive : b->opt.splat_config_absorption;
      const bool is_fixed = fixed >= 0 && spl::splat_config_valid(fixed, T);
      int pick = is_fixed ? fixed : spl::splat_default_config(T, cls == 0);
      if (present && !is_fixed) {
        float bms = 1e30f;
        for (int k = 0; k < nc; ++k) {
          float ms = 0.f;
          for (int rep = 0; rep < 2; ++rep) {
            BCK(cudaMemsetAsync(as<uint32_t>(b->status) + 2 + cls, 0, 4, b->stream));
            BCK(cudaEventRecord(b->ev0, b->stream));
            spl::launch_splat_queue(queue_args(b, cls), cands[k], b->stream);
            BCK(cudaEventRecord(b->ev1, b->stream));
            BCK(cudaStreamSynchronize(b->stream));
            BCK(cudaGetLastError());
            cudaEventElapsedTime(&ms, b->ev0, b->ev1);
          }
          if (ms < bms) {
            bms = ms;
            pick = cands[k];
          }
        }
      }
      (cls == 0 ? b->cfg_add : b->cfg_abs) = pick;
    }
    float tot = 0.f;
    for (int rep = 0; rep < 2; ++rep) {
      if ((st = run_once(b, &tot))) return st;
    }
    if ((st = check_status(b, overflow))) return st;
    if (tot < best_ms && !overflow) {
      best_ms = tot;
      best_T = T;
      best_add = b->cfg_add;
      best_abs = b->cfg_abs;
    }
  }
  b->cfg_add = best_add;
  b->cfg_abs = best_abs;
  b->info.tune_ms = since(t0);
  b->info.tune_cached = 0;
  const auto tp = std::chrono::steady_clock::now();
  if (b->T != best_T || sizes.size() > 1) {
    if ((st = build(b, best_T))) return st;
  }
  b->info.plan_ms = since(tp);
  if (b->opt.tune_cache) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache[key] = TuneChoice{best_T, best_add, best_abs};
  }
  return SPL_OK;
}

void free_batch(spl_batch *b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  for (DevBuf *d : b->owned)
    if (d->p) cudaFree(d->p);
  if (b->h_status) cudaFreeHost(b->h_status);
  if (b->h_entries) cudaFreeHost(b->h_entries);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  if (b->stream2) cudaStreamDestroy(b->stream2);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

}  // namespace

extern "C" {

void spl_batch_options_defaults(spl_batch_options *o) {
  if (!o) return;
  o->tile_size = 0;
  o->splat_config_additive = -1;
  o->splat_config_absorption = -1;
  o->capacity_margin = 1.1f;
  o->use_graph = 1;
  o->tune_cache = 1;
}

spl_status spl_batch_create(spl_context *ctx, const spl_particles *sets, int nsets,
                            const spl_batch_frame *frames, int nframes,
                            const spl_batch_options *opt, spl_batch **out) {
  if (!ctx || !out || (nsets > 0 && !sets) || nframes < 1 || !frames)
    return fail(SPL_ERR_INVALID, "batch: null argument or no frames");
  *out = nullptr;
  spl_batch_options o;
  spl_batch_options_defaults(&o);
  if (opt) o = *opt;
  if (o.tile_size < 0 || o.tile_size > 64 || !(o.capacity_margin > 0.f))
    return fail(SPL_ERR_INVALID, "batch: bad options");
  for (int k = 0; k < nsets; ++k) {
    const spl_particles &p = sets[k];
    if (p.memspace != SPL_MEM_DEVICE)
      return fail(SPL_ERR_UNSUPPORTED, "batch: particle sets must be device-resident");
  }
  for (int f = 0; f < nframes; ++f) {
    const spl_batch_frame &fr = frames[f];
    if (fr.set < 0 || fr.set >= nsets)
      return fail(SPL_ERR_INVALID, "batch: frame " + std::to_string(f) + " names no set");
    spl_image img{fr.pic, SPL_MEM_DEVICE};
    spl_frame_desc d = fr.desc;
    d.tile_size = o.tile_size > 0 ? o.tile_size : 16;
    spl_status st = spl::validate_frame(&d, &sets[fr.set], &img);
    if (st) return st;
  }
  spl_batch *b = new spl_batch();
  b->ctx = ctx;
  b->device = spl::context_device(ctx);
  b->sets.assign(sets, sets + nsets);
  b->frames.assign(frames, frames + nframes);
  b->opt = o;
  cudaSetDevice(b->device);
  spl_status st = SPL_OK;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
      cudaMallocHost((void **)&b->h_status, 64) != cudaSuccess ||
      cudaMallocHost((void **)&b->h_entries, 8) != cudaSuccess) {
    cudaGetLastError();
    free_batch(b);
    return fail(SPL_ERR_CUDA, "batch: stream, event or pinned-memory creation failed");
  }
  // private copies of the frames' palettes: re-plans read them after create
  b->pal_x_copy.reserve((size_t)nframes * SPL_MAX_TYPES);
  b->pal_rgb_copy.reserve((size_t)nframes * SPL_MAX_TYPES);
  for (auto &fr : b->frames) {
    for (int t = 0; t < fr.desc.ptypes; ++t) {
      if (fr.desc.color_is_vector[t] || fr.desc.pal_n[t] < 1) continue;
      const int nk = fr.desc.pal_n[t];
      b->pal_x_copy.emplace_back(fr.desc.pal_x[t], fr.desc.pal_x[t] + nk);
      b->pal_rgb_copy.emplace_back(fr.desc.pal_rgb[t], fr.desc.pal_rgb[t] + 3 * nk);
      fr.desc.pal_x[t] = b->pal_x_copy.back().data();
      fr.desc.pal_rgb[t] = b->pal_rgb_copy.back().data();
    }
  }
  if ((st = autotune(b))) {
    free_batch(b);
    return st;
  }
  b->info.splat_config_additive = b->cfg_add;
  b->info.splat_config_absorption = b->cfg_abs;
  if (o.use_graph && (st = capture(b))) {
    free_batch(b);
    return st;
  }
  b->info.graph = b->exec ? 1 : 0;
  b->info.replans = 0;
  *out = b;
  return SPL_OK;
}

spl_status spl_batch_render(spl_batch *b) {
  if (!b) return fail(SPL_ERR_INVALID, "null batch");
  BCK(cudaSetDevice(b->device));
  spl_status st;
  for (int attempt = 0; attempt < 3; ++attempt) {
    float ms = 0.f;
    if ((st = run_once(b, &ms))) return st;
    bool overflow = false;
    if ((st = check_status(b, overflow))) return st;
    b->info.render_ms = ms;
    b->info.n_active = (int64_t)b->h_status[5] + b->h_status[6];
    b->info.n_entries = (int64_t)*b->h_entries;
    b->info.kernel_launches = b->launches;
    if (!overflow) return SPL_OK;
    // counts outgrew the plan: measure again with a margin of at least 1.1
    b->opt.capacity_margin = std::max(b->opt.capacity_margin, 1.1f);
    ++b->info.replans;
    if ((st = build(b, b->T))) return st;
    if (b->opt.use_graph && (st = capture(b))) return st;
  }
  return fail(SPL_ERR_CAPACITY, "batch: capacities still exceeded after re-planning");
}

spl_status spl_batch_get_info(const spl_batch *b, spl_batch_info *info) {
  if (!b || !info) return fail(SPL_ERR_INVALID, "null argument");
  *info = b->info;
  info->tile_size = b->T;
  info->splat_config_additive = b->cfg_add;
  info->splat_config_absorption = b->cfg_abs;
  info->graph = b->exec ? 1 : 0;
  info->cap_active = b->cap_a;
  info->cap_entries = b->cap_e;
  info->total_tiles = b->ntiles;
  return SPL_OK;
}

spl_status spl_batch_destroy(spl_batch *b) {
  free_batch(b);
  return SPL_OK;
}

}  // extern "C"
