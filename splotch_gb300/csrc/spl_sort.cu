// spl_sort.cu -- stable LSD radix sort of (uint32 key, uint32 value) pairs
// and the exclusive scans used by binning.
//
// The depth sort replaces particle_sort (splotch/splotch_host.cc:289-321).
// The reference calls std::sort, which is not stable; this sort is stable, so
// equal keys keep ascending particle index (= std::stable_sort with the same
// comparator), the tie-break the renderer specifies.
//
// Structure per 8-bit digit pass (reduce-then-scan, no inter-block waits):
//   upsweep   : per-block digit histogram -> counts[digit][block]
//   scan      : exclusive scan over the digit-major counts array
//   downsweep : stable in-block ranking with warp match/ballot, then scatter
#include "spl_internal.cuh"

namespace spl {

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;  // keys per block
constexpr int RS_BINS = 256;

constexpr int SC_THREADS = 256;
constexpr int SC_ITEMS = 16;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_upsweep(const uint32_t *__restrict__ keys,
                                                           int64_t n, int shift, int nbits,
                                                           uint32_t *__restrict__ counts,
                                                           int nblocks) {
  __shared__ uint32_t whist[RS_WARPS][RS_BINS];  // per-warp privatised histograms
  for (int i = threadIdx.x; i < RS_WARPS * RS_BINS; i += RS_THREADS) (&whist[0][0])[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t mask = (1u << nbits) - 1u;
  const int64_t base = (int64_t)blockIdx.x * RS_TILE + (int64_t)w * 32 * RS_ITEMS;
  if (base + 32 * RS_ITEMS <= n) {
    const uint4 *k4 = reinterpret_cast<const uint4 *>(keys + base);
#pragma unroll
    for (int j = 0; j < RS_ITEMS / 4; ++j) {
      const uint4 v = __ldg(k4 + j * 32 + lane);
      atomicAdd(&whist[w][(v.x >> shift) & mask], 1u);
      atomicAdd(&whist[w][(v.y >> shift) & mask], 1u);
      atomicAdd(&whist[w][(v.z >> shift) & mask], 1u);
      atomicAdd(&whist[w][(v.w >> shift) & mask], 1u);
    }
  } else {
    for (int j = 0; j < RS_ITEMS; ++j) {
      const int64_t idx = base + j * 32 + lane;
      if (idx < n) atomicAdd(&whist[w][(__ldg(keys + idx) >> shift) & mask], 1u);
    }
  }
  __syncthreads();
  uint32_t tot = 0;
#pragma unroll
  for (int ww = 0; ww < RS_WARPS; ++ww) tot += whist[ww][threadIdx.x];
  counts[(int64_t)threadIdx.x * nblocks + blockIdx.x] = tot;
}

// Look-back state word (one per tile and digit): epoch (8 bits) | kind (2 bits)
// | count (54 bits).  kind 1 = this tile's own count, 2 = inclusive prefix.
constexpr int OS_EPOCH_SHIFT = 56, OS_KIND_SHIFT = 54;
constexpr unsigned long long OS_VALUE_MASK = (1ull << OS_KIND_SHIFT) - 1ull;
constexpr uint32_t OS_SPIN_LIMIT = 1u << 22;  // bounded wait, then error flag
constexpr uint32_t OS_SPIN_LIMIT_TEST = 4096u;  // the stall test's limit (~1 ms)

__device__ __forceinline__ unsigned long long os_word(uint32_t epoch, uint32_t kind,
                                                      unsigned long long v) {
  return ((unsigned long long)epoch << OS_EPOCH_SHIFT) |
         ((unsigned long long)kind << OS_KIND_SHIFT) | v;
}

// Scatter pass.  OS=false: reduce-then-scan (offsets from the upsweep and a
// scan).  OS=true: onesweep -- tiles are taken in launch order from a counter
// and each digit's global offset comes from the global digit base plus a
// decoupled look-back over earlier tiles' published counts.  A tile only ever
// waits on tiles that started before it, and every wait is bounded.
//
// Per tile: load the keys; rank each key among the equal digits before it
// (stable); publish the tile's digit counts at once (onesweep); sort the tile
// into shared memory by digit; look back (by then the keys' registers are
// dead, and the tiles in front have had the ranking's time to publish their
// own prefixes); write each digit's run to its global offset.
//
// Ranking: the lanes of a warp holding the same digit find each other
// through a per-warp table of 256 lane masks in shared memory (each lane ORs
// its bit into its digit's slot, then reads the slot back); the group's
// lowest lane claims the group's slots in the warp's digit count and clears
// the slot.  Items are ranked in order, so equal digits keep input order.
// (A warp match instruction gives the same masks, at several times the cost
// per item with the ~30 distinct digits a warp of 32 keys usually holds.)
constexpr int OS_WINDOW = 8;  // look-back: predecessor states read per round

template <bool OS>
__global__ void __launch_bounds__(RS_THREADS, 3) k_rs_downsweep(
    const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
    uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, int64_t n, int shift,
    int nbits, const uint32_t *__restrict__ offsets, int nblocks,
    const unsigned long long *__restrict__ digit_base, unsigned long long *state,
    uint32_t *tile_ctr, uint32_t *err, uint32_t epoch, uint32_t spin_limit) {
  __shared__ uint32_t whist[RS_WARPS][RS_BINS];
  __shared__ uint32_t boff[RS_BINS];
  __shared__ uint32_t lstart[RS_BINS];
  __shared__ uint32_t wtot[RS_WARPS];
  __shared__ uint32_t skey[RS_TILE];
  __shared__ uint32_t sval[RS_TILE];
  __shared__ uint32_t tile_sh;
  // the ranking's lane-mask table lives in skey, which is written only after
  // the ranking (behind a barrier)
  static_assert(RS_TILE >= RS_WARPS * RS_BINS, "the mask table fits in skey");
  uint32_t(*mtab)[RS_BINS] = reinterpret_cast<uint32_t(*)[RS_BINS]>(skey);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < RS_WARPS * RS_BINS; i += RS_THREADS) {
    (&whist[0][0])[i] = 0;
    skey[i] = 0;
  }
  if (OS && threadIdx.x == 0) tile_sh = atomicAdd(tile_ctr, 1u);
  __syncthreads();
  const int blk = OS ? (int)tile_sh : (int)blockIdx.x;
  const uint32_t mask = (1u << nbits) - 1u;
  const int64_t base = (int64_t)blk * RS_TILE + (int64_t)w * 32 * RS_ITEMS;
  uint32_t key[RS_ITEMS], val[RS_ITEMS], rank[RS_ITEMS];
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    const int64_t idx = base + j * 32 + lane;
    const bool valid = idx < n;
    key[j] = valid ? __ldg(keys_in + idx) : 0xffffffffu;
    val[j] = valid ? (vals_in ? __ldg(vals_in + idx) : (uint32_t)idx) : 0u;
  }
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    const bool valid = base + j * 32 + lane < n;
    const uint32_t d = (key[j] >> shift) & mask;
    uint32_t *slot = &mtab[w][d];
    __syncwarp();  // the previous item's slot clears are visible
    if (valid) atomicOr(slot, 1u << lane);
    __syncwarp();
    const uint32_t peers = valid ? *slot : 0u;
    const int leader = __ffs(peers) - 1;
    uint32_t prior = 0;
    if (valid && lane == leader) prior = atomicAdd(&whist[w][d], (uint32_t)__popc(peers));
    __syncwarp();  // every peer has read the slot
    if (valid && lane == leader) *slot = 0u;
    prior = __shfl_sync(0xffffffffu, prior, leader & 31);
    rank[j] = prior + __popc(peers & lanemask_lt());
  }
  __syncthreads();
  const int d = threadIdx.x;
  unsigned long long *st = OS ? state + (size_t)blk * RS_BINS + d : nullptr;
  uint32_t run = 0;
  {  // per digit: exclusive prefix over warps, then over digits (block-local)
#pragma unroll
    for (int ww = 0; ww < RS_WARPS; ++ww) {
      const uint32_t t = whist[ww][d];
      whist[ww][d] = run;
      run += t;
    }
    // onesweep: publish this tile's count of digit d (tile 0: its prefix)
    if (OS)
      *reinterpret_cast<volatile unsigned long long *>(st) = os_word(epoch, blk == 0 ? 2u : 1u, run);
    uint32_t inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) wtot[w] = inc;
    __syncthreads();
    uint32_t wpre = 0;
    for (int ww = 0; ww < w; ++ww) wpre += wtot[ww];
    lstart[d] = wpre + inc - run;
  }
  __syncthreads();
  // stable local sort into shared memory ...
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    if (base + j * 32 + lane < n) {
      const uint32_t dd = (key[j] >> shift) & mask;
      const uint32_t lpos = lstart[dd] + whist[w][dd] + rank[j];
      skey[lpos] = key[j];
      sval[lpos] = val[j];
    }
  }
  // ... the digit's global offset ...
  unsigned long long excl = 0;
  if (OS) {
    if (blk > 0) {  // decoupled look-back, OS_WINDOW tiles per round
      int t = blk - 1;
      uint32_t spins = 0;
      while (t >= 0) {
        unsigned long long v[OS_WINDOW];
#pragma unroll
        for (int i = 0; i < OS_WINDOW; ++i)  // before tile 0: an inclusive zero
          v[i] = t - i >= 0 ? *reinterpret_cast<const volatile unsigned long long *>(
                                  state + (size_t)(t - i) * RS_BINS + d)
                            : os_word(epoch, 2u, 0ull);
        bool go = true, found = false;
        int used = 0;
#pragma unroll
        for (int i = 0; i < OS_WINDOW; ++i) {
          if (go) {
            const uint32_t kind = (uint32_t)(v[i] >> OS_KIND_SHIFT) & 3u;
            if ((uint32_t)(v[i] >> OS_EPOCH_SHIFT) != epoch || kind == 0u) {
              go = false;  // not published yet: read again from here
            } else {
              excl += v[i] & OS_VALUE_MASK;
              used = i + 1;
              if (kind == 2u) {
                found = true;
                go = false;
              }
            }
          }
        }
        if (found) break;
        t -= used;
        if (used < OS_WINDOW && t >= 0) {
          // give up: this tile's offsets come from a partial prefix (never
          // above the true one, so its writes stay inside [0, n)); the
          // results are invalid and the host reports it
          if (++spins > spin_limit) {
            atomicOr(err, 2u);
            break;
          }
          if (spins > 64) __nanosleep(64);
        }
      }
      *reinterpret_cast<volatile unsigned long long *>(st) = os_word(epoch, 2u, excl + run);
    }
    boff[d] = (uint32_t)(digit_base[d] + excl) - lstart[d];
  } else {
    boff[d] = offsets[(int64_t)d * nblocks + blk] - lstart[d];
  }
  __syncthreads();
  // ... then consecutive threads write consecutive slots of each digit run
  const int nloc = (int)min((int64_t)RS_TILE, n - (int64_t)blk * RS_TILE);
  for (int i = threadIdx.x; i < nloc; i += RS_THREADS) {
    const uint32_t k = skey[i];
    const uint32_t dst = boff[(k >> shift) & mask] + (uint32_t)i;
    if (keys_out) keys_out[dst] = k;
    vals_out[dst] = sval[i];
  }
}

__global__ void k_set_u32(uint32_t *p, uint32_t v) { *p = v; }

// All digit histograms of the onesweep passes in one read of the keys.
constexpr int OS_MAX_PASS = 4;
__global__ void __launch_bounds__(RS_THREADS) k_os_hist(const uint32_t *__restrict__ keys,
                                                        int64_t n, int bit0, int bit1,
                                                        unsigned long long *hist) {
  __shared__ uint32_t h[OS_MAX_PASS][RS_BINS];
  for (int i = threadIdx.x; i < OS_MAX_PASS * RS_BINS; i += RS_THREADS) (&h[0][0])[i] = 0;
  __syncthreads();
  const int npass = (bit1 - bit0 + 7) / 8;
  auto count = [&](uint32_t k) {
    for (int p = 0; p < npass; ++p) {
      const int sh = bit0 + 8 * p;
      const int nb = min(8, bit1 - sh);
      atomicAdd(&h[p][(k >> sh) & ((1u << nb) - 1u)], 1u);
    }
  };
  // four keys per 16-byte load when the keys are 16-byte aligned, the
  // remainder one at a time
  const int64_t nq = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0 ? n / 4 : 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nq; q += stride) {
    const uint4 v = __ldg(reinterpret_cast<const uint4 *>(keys) + q);
    count(v.x);
    count(v.y);
    count(v.z);
    count(v.w);
  }
  for (int64_t i = nq * 4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    count(__ldg(keys + i));
  __syncthreads();
  for (int p = 0; p < npass; ++p)
    if (h[p][threadIdx.x]) atomicAdd(hist + p * RS_BINS + threadIdx.x, (unsigned long long)h[p][threadIdx.x]);
}

// Exclusive scan of each pass's 256 digit counts (one block).
__global__ void __launch_bounds__(RS_THREADS) k_os_prefix(unsigned long long *hist, int npass) {
  __shared__ unsigned long long sm[33];
  for (int p = 0; p < npass; ++p) {
    const unsigned long long v = hist[p * RS_BINS + threadIdx.x];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) sm[w] = inc;
    __syncthreads();
    unsigned long long pre = 0;
    for (int ww = 0; ww < w; ++ww) pre += sm[ww];
    __syncthreads();
    hist[p * RS_BINS + threadIdx.x] = pre + inc - v;
    __syncthreads();
  }
}

// ---- generic exclusive scan (three kernels) ------------------------------

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// block-wide exclusive scan of one value per thread; returns exclusive
// prefix and writes the block total
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T *sm_warp, T &total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T inc = warp_incl_scan(v, lane);
  if (lane == 31) sm_warp[w] = inc;
  __syncthreads();
  if (w == 0) {
    T x = lane < (int)(blockDim.x >> 5) ? sm_warp[lane] : T(0);
    T xi = warp_incl_scan(x, lane);
    if (lane < (int)(blockDim.x >> 5)) sm_warp[lane] = xi - x;
    if (lane == 31) sm_warp[32] = xi;
  }
  __syncthreads();
  total = sm_warp[32];
  T r = sm_warp[w] + inc - v;
  __syncthreads();
  return r;
}

template <typename T, typename L>
__global__ void __launch_bounds__(SC_THREADS) k_scan_reduce(L load, int64_t n, T *partials) {
  __shared__ T sm[33];
  const int64_t base = (int64_t)blockIdx.x * SC_TILE;
  T s = 0;
  for (int j = 0; j < SC_ITEMS; ++j) {
    const int64_t i = base + j * SC_THREADS + threadIdx.x;
    if (i < n) s += load(i);
  }
  T total;
  block_excl_scan<T>(s, sm, total);
  if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

// single block: exclusive scan of m partials in place; total to *total_out
template <typename T>
__global__ void __launch_bounds__(SC_THREADS) k_scan_partials(T *partials, int64_t m,
                                                              T *total_out) {
  __shared__ T sm[33];
  T carry = 0;
  for (int64_t b = 0; b < m; b += SC_THREADS) {
    const int64_t i = b + threadIdx.x;
    T v = i < m ? partials[i] : T(0);
    T tot;
    T ex = block_excl_scan<T>(v, sm, tot);
    if (i < m) partials[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0 && total_out) *total_out = carry;
}

template <typename T, typename L>
__global__ void __launch_bounds__(SC_THREADS) k_scan_apply(L load, int64_t n,
                                                           const T *partials, T *out) {
  __shared__ T sm[33];
  // the tile passes through shared memory both ways, so that a warp's loads
  // and stores are consecutive elements while each thread scans SC_ITEMS
  // consecutive ones (rows padded by one element against bank conflicts)
  __shared__ T stage[SC_THREADS * (SC_ITEMS + 1)];
  const int64_t base = (int64_t)blockIdx.x * SC_TILE;
#pragma unroll 4
  for (int r = 0; r < SC_ITEMS; ++r) {
    const int e = r * SC_THREADS + threadIdx.x;
    const int64_t i = base + e;
    stage[(e / SC_ITEMS) * (SC_ITEMS + 1) + e % SC_ITEMS] = i < n ? load(i) : T(0);
  }
  __syncthreads();
  T v[SC_ITEMS];
  T s = 0;
#pragma unroll
  for (int j = 0; j < SC_ITEMS; ++j) {
    v[j] = stage[threadIdx.x * (SC_ITEMS + 1) + j];
    s += v[j];
  }
  T tot;  // (the scan's barriers also order the reads above before the writes below)
  T ex = block_excl_scan<T>(s, sm, tot) + partials[blockIdx.x];
#pragma unroll
  for (int j = 0; j < SC_ITEMS; ++j) {
    stage[threadIdx.x * (SC_ITEMS + 1) + j] = ex;
    ex += v[j];
  }
  __syncthreads();
#pragma unroll 4
  for (int r = 0; r < SC_ITEMS; ++r) {
    const int e = r * SC_THREADS + threadIdx.x;
    const int64_t i = base + e;
    if (i < n) out[i] = stage[(e / SC_ITEMS) * (SC_ITEMS + 1) + e % SC_ITEMS];
  }
}

struct LoadU32 {
  const uint32_t *p;
  __device__ __forceinline__ uint32_t operator()(int64_t i) const { return __ldg(p + i); }
};
struct LoadPopc {
  const uint32_t *w;
  __device__ __forceinline__ uint32_t operator()(int64_t i) const { return __popc(__ldg(w + i)); }
};
struct LoadCountOrdered {
  const uint32_t *count;
  const uint32_t *order;
  __device__ __forceinline__ uint64_t operator()(int64_t i) const {
    return (uint64_t)__ldg(count + (order ? __ldg(order + i) : (uint32_t)i));
  }
};

template <typename T, typename L>
void exclusive_scan(L load, int64_t n, T *out, T *total_out, void *scratch, cudaStream_t s,
                    int *launches) {
  const int64_t nb = (n + SC_TILE - 1) / SC_TILE;
  T *partials = static_cast<T *>(scratch);
  if (nb > 0) {
    k_scan_reduce<T, L><<<(unsigned)nb, SC_THREADS, 0, s>>>(load, n, partials);
    k_scan_partials<T><<<1, SC_THREADS, 0, s>>>(partials, nb, total_out);
    k_scan_apply<T, L><<<(unsigned)nb, SC_THREADS, 0, s>>>(load, n, partials, out);
    if (launches) *launches += 3;
  } else if (total_out) {
    cudaMemsetAsync(total_out, 0, sizeof(T), s);
  }
}

}  // namespace

size_t radix_scratch_bytes(int64_t n) {
  const int64_t nb = (n + RS_TILE - 1) / RS_TILE;
  const int64_t m = nb * RS_BINS;
  const int64_t np = (m + SC_TILE - 1) / SC_TILE;
  const size_t rts = (size_t)(2 * m + np + 64) * sizeof(uint32_t);
  const size_t os = (size_t)OS_MAX_PASS * RS_BINS * 8 + 256 + (size_t)m * 8;
  return (rts > os ? rts : os) + 256;
}

int radix_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_tmp,
                     uint32_t *vals_tmp, uint32_t *keys_out, uint32_t *vals_out, int64_t n,
                     int bit0, int bit1, bool keys_needed, void *scratch, cudaStream_t s,
                     int *launches, uint32_t *err, bool onesweep, bool stall_test) {
  if (n <= 0) return 0;
  const int nblocks = (int)((n + RS_TILE - 1) / RS_TILE);
  const int64_t m = (int64_t)nblocks * RS_BINS;
  int npass = 0;
  for (int b = bit0; b < bit1; b += 8) ++npass;
  if (npass > OS_MAX_PASS) onesweep = false;
  // onesweep scratch: digit bases, per-pass tile counters, look-back state
  unsigned long long *hist = static_cast<unsigned long long *>(scratch);
  uint32_t *tile_ctr = reinterpret_cast<uint32_t *>(hist + OS_MAX_PASS * RS_BINS);
  unsigned long long *state = reinterpret_cast<unsigned long long *>(
      reinterpret_cast<uint8_t *>(tile_ctr) + 256);
  // reduce-then-scan scratch
  uint32_t *counts = static_cast<uint32_t *>(scratch);
  uint32_t *offsets = counts + m;
  uint32_t *sc = offsets + m;
  if (onesweep) {
    cudaMemsetAsync(scratch, 0, (size_t)OS_MAX_PASS * RS_BINS * 8 + 256 + (size_t)m * 8, s);
    int hb = (int)((n + RS_THREADS * 16 - 1) / (RS_THREADS * 16));
    if (hb > 152 * 8) hb = 152 * 8;
    k_os_hist<<<hb, RS_THREADS, 0, s>>>(keys_in, n, bit0, bit1, hist);
    k_os_prefix<<<1, RS_THREADS, 0, s>>>(hist, npass);
    if (launches) *launches += 2;
  }
  // ping-pong so that the last pass lands in (keys_out, vals_out)
  const uint32_t *kin = keys_in;
  const uint32_t *vin = vals_in;
  int pass = 0;
  for (int b = bit0; b < bit1; b += 8, ++pass) {
    const int nbits = (bit1 - b) < 8 ? (bit1 - b) : 8;
    const bool last = pass == npass - 1;
    const bool to_out = ((npass - 1 - pass) % 2) == 0;
    uint32_t *ko = to_out ? keys_out : keys_tmp;
    uint32_t *vo = to_out ? vals_out : vals_tmp;
    uint32_t *kout = (last && !keys_needed) ? nullptr : ko;
    if (onesweep) {
      // the stall test: the pass's tile counter starts at 1, so tiles
      // 1..nblocks-1 run (one block each) and tile 0 never publishes
      const bool stall = stall_test && pass == 0 && nblocks >= 2;
      if (stall) k_set_u32<<<1, 1, 0, s>>>(tile_ctr + pass, 1u);
      k_rs_downsweep<true><<<stall ? nblocks - 1 : nblocks, RS_THREADS, 0, s>>>(
          kin, vin, kout, vo, n, b, nbits, nullptr, nblocks, hist + pass * RS_BINS, state,
          tile_ctr + pass, err, (uint32_t)(pass + 1),
          stall_test ? OS_SPIN_LIMIT_TEST : OS_SPIN_LIMIT);
      if (launches) *launches += stall ? 2 : 1;
    } else {
      k_rs_upsweep<<<nblocks, RS_THREADS, 0, s>>>(kin, n, b, nbits, counts, nblocks);
      exclusive_scan<uint32_t>(LoadU32{counts}, m, offsets, (uint32_t *)nullptr, sc, s,
                               launches);
      k_rs_downsweep<false><<<nblocks, RS_THREADS, 0, s>>>(
          kin, vin, kout, vo, n, b, nbits, offsets, nblocks, nullptr, nullptr, nullptr, nullptr, 0,
          0u);
      if (launches) *launches += 2;
    }
    kin = ko;
    vin = vo;
  }
  return npass;
}

size_t scan_scratch_bytes(int64_t n) {
  return (size_t)((n + SC_TILE - 1) / SC_TILE + 64) * sizeof(uint64_t);
}

void scan_popc(const uint32_t *words, int64_t nwords, uint32_t *out, uint32_t *total,
               void *scratch, cudaStream_t s, int *launches) {
  exclusive_scan<uint32_t>(LoadPopc{words}, nwords, out, total, scratch, s, launches);
}

void scan_counts(const uint32_t *count, const uint32_t *order, int64_t n, uint64_t *off,
                 void *scratch, cudaStream_t s, int *launches) {
  exclusive_scan<uint64_t>(LoadCountOrdered{count, order}, n, off, off + n, scratch, s,
                           launches);
}

}  // namespace spl
