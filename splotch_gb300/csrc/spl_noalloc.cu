// spl_noalloc.cu -- spl_sort_pairs_noalloc: the stable (key, value) radix sort
// of the depth-sort stage with every scratch buffer in one static device array
// of this file, so that a call allocates no memory at all.
//
// Who needs it: a caller that may not allocate device memory while it runs --
// a render loop that reserves all of its memory up front, a process whose
// device memory is owned by another allocator, code held to a fixed
// device-memory budget.  The context of spl_render grows its buffers with
// cudaMalloc on demand, which such callers cannot accept.
//
// Layout of the array (each piece 256-byte aligned):
//   [0, P)      key ping-pong buffer   (SPL_NOALLOC_MAX_PAIRS keys)
//   [P, 2P)     value ping-pong buffer (SPL_NOALLOC_MAX_PAIRS values)
//   [2P, end)   per-block digit counts, their scanned offsets, scan partials
// The digit passes use the reduce-then-scan form: every word of the array is
// written before it is read within a call, so nothing has to be cleared first,
// and no block ever waits on another.
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/splotch_gb300.h"
#include "spl_internal.cuh"

namespace {

constexpr int64_t kMaxPairs = SPL_NOALLOC_MAX_PAIRS;
constexpr size_t kPairBytes = (size_t)kMaxPairs * sizeof(uint32_t);
// 2 x 256 counts per 4096-pair block plus the scan partials need about
// kMaxPairs / 2 bytes; the set-up checks the exact figure against this.
constexpr size_t kRadixBytes = (size_t)kMaxPairs + (1u << 16);
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_sort_scratch[2 * kPairBytes + kRadixBytes];

std::mutex g_mu;
bool g_checked[kMaxDevices];  // capacity checked on this device

spl_status fail(spl_status code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  spl::set_last_error(buf);
  return code;
}

spl_status cuda_fail(const char *what, cudaError_t e) {
  cudaGetLastError();
  return fail(SPL_ERR_CUDA, "spl_sort_pairs_noalloc: %s: %s", what, cudaGetErrorString(e));
}

// Set-up: the capacity check, once per device, and the scratch array's
// address on the current device.  The first call on a device also loads the
// library's device code there (lazy module loading).  The address is looked
// up again on every call -- a host-side table lookup that allocates nothing --
// so that a cudaDeviceReset or another context on the device between calls
// never leaves a stale address behind.
spl_status scratch_base(int *dev_out, unsigned char **base_out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail("cudaGetDevice", e);
  if (dev < 0 || dev >= kMaxDevices)
    return fail(SPL_ERR_UNSUPPORTED, "spl_sort_pairs_noalloc: device %d is beyond the %d supported",
                dev, kMaxDevices);
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_checked[dev]) {
      const size_t need = spl::radix_scratch_bytes(kMaxPairs);
      if (need > kRadixBytes)
        return fail(SPL_ERR_CAPACITY,
                    "spl_sort_pairs_noalloc: digit-count scratch of %zu bytes exceeds the %zu "
                    "reserved", need, kRadixBytes);
      g_checked[dev] = true;
    }
  }
  void *p = nullptr;
  e = cudaGetSymbolAddress(&p, g_sort_scratch);
  if (e != cudaSuccess) return cuda_fail("cudaGetSymbolAddress", e);
  *dev_out = dev;
  *base_out = static_cast<unsigned char *>(p);
  return SPL_OK;
}

spl_status check_device_ptr(const void *p, int dev, const char *name) {
  cudaPointerAttributes a{};
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SPL_ERR_INVALID, "spl_sort_pairs_noalloc: %s is not a device pointer", name);
  }
  if ((a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) || a.device != dev)
    return fail(SPL_ERR_INVALID,
                "spl_sort_pairs_noalloc: %s is not device memory of the current device %d", name,
                dev);
  return SPL_OK;
}

bool overlap(const void *a, const void *b, size_t bytes) {
  const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
  return x < y + bytes && y < x + bytes;
}

}  // namespace

extern "C" spl_status spl_sort_pairs_noalloc(const uint32_t *keys_in, const uint32_t *vals_in,
                                             uint32_t *keys_out, uint32_t *vals_out, int64_t n,
                                             int key_bits, void *stream) {
  if (n < 0)
    return fail(SPL_ERR_INVALID, "spl_sort_pairs_noalloc: n = %lld is negative", (long long)n);
  if (key_bits < 1 || key_bits > 32)
    return fail(SPL_ERR_INVALID, "spl_sort_pairs_noalloc: key_bits = %d is outside 1..32",
                key_bits);
  int dev = -1;
  unsigned char *base = nullptr;
  spl_status st = scratch_base(&dev, &base);
  if (st != SPL_OK) return st;
  if (n == 0) return SPL_OK;
  if (n > kMaxPairs)
    return fail(SPL_ERR_CAPACITY,
                "spl_sort_pairs_noalloc: n = %lld pairs exceeds its fixed capacity of %lld "
                "(SPL_NOALLOC_MAX_PAIRS)",
                (long long)n, (long long)kMaxPairs);
  if (!keys_in || !keys_out || !vals_out)
    return fail(SPL_ERR_INVALID, "spl_sort_pairs_noalloc: keys_in, keys_out and vals_out are "
                                 "required");
  // the digit-count pass reads its keys 16 bytes at a time, and with three or
  // four digit passes one of them reads keys_out
  if (reinterpret_cast<uintptr_t>(keys_in) & 15u)
    return fail(SPL_ERR_INVALID, "spl_sort_pairs_noalloc: keys_in must be 16-byte aligned");
  if (reinterpret_cast<uintptr_t>(keys_out) & 15u)
    return fail(SPL_ERR_INVALID, "spl_sort_pairs_noalloc: keys_out must be 16-byte aligned");
  if ((st = check_device_ptr(keys_in, dev, "keys_in")) != SPL_OK) return st;
  if (vals_in && (st = check_device_ptr(vals_in, dev, "vals_in")) != SPL_OK) return st;
  if ((st = check_device_ptr(keys_out, dev, "keys_out")) != SPL_OK) return st;
  if ((st = check_device_ptr(vals_out, dev, "vals_out")) != SPL_OK) return st;
  const size_t bytes = (size_t)n * sizeof(uint32_t);
  if (overlap(keys_out, vals_out, bytes) || overlap(keys_out, keys_in, bytes) ||
      overlap(vals_out, keys_in, bytes) ||
      (vals_in && (overlap(keys_out, vals_in, bytes) || overlap(vals_out, vals_in, bytes))))
    return fail(SPL_ERR_INVALID, "spl_sort_pairs_noalloc: output buffers overlap each other "
                                 "or an input");
  uint32_t *keys_tmp = reinterpret_cast<uint32_t *>(base);
  uint32_t *vals_tmp = reinterpret_cast<uint32_t *>(base + kPairBytes);
  void *digit_scratch = base + 2 * kPairBytes;
  // an error that the caller's earlier work left pending is reported, not
  // cleared, and nothing is launched
  const cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess)
    return fail(SPL_ERR_CUDA, "spl_sort_pairs_noalloc: a CUDA error is already pending on this "
                              "thread (%s); nothing was launched", cudaGetErrorString(pending));
  spl::radix_sort_pairs(keys_in, vals_in, keys_tmp, vals_tmp, keys_out, vals_out, n, 0, key_bits,
                        true, digit_scratch, static_cast<cudaStream_t>(stream), nullptr, nullptr,
                        false);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail("radix sort launch", e);
  return SPL_OK;
}
