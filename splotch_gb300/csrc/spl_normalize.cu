// spl_normalize.cu -- sceneMaker::particle_normalize (splotch/scenemaker.cc:
// 40-296, host branch) on the device, the step right before host_rendering:
//
//   pass 1 (k_norm_collect): per particle, the optional log10 of I and of the
//     colour (values <= 0 become -38 and are not collected; the vector-colour
//     channels take log10 unconditionally) or asinh of the colour, written
//     back; per type min/max of hsml, intensity and colour (NaN never wins,
//     as with std::min/std::max), reduced in shared memory per block and
//     published with one global atomic per (type, statistic) per block;
//   host: intensity_min/max and color_min/max overrides;
//   pass 2 (k_norm_clamp): Normalizer::normAndClamp of I and colour
//     (splotch/splotchutils.h:158-165).
// Both passes are HBM-bound: 20 B read + 16 B written, then 18 B read + 16 B
// written per particle.  log10f and log/sqrt come from CUDA's math library, so
// a transformed value can differ from the host's by an ulp.
#include <cstring>

#include "spl_internal.cuh"

namespace spl {
namespace {

constexpr int kStats = 6;  // size min/max, intensity min/max, colour min/max

// Order-preserving int image of a float for atomic min/max (-0 maps to +0).
__device__ __forceinline__ int ord(float f) {
  int i = __float_as_int(f);
  if (i == (int)0x80000000) i = 0;
  return i >= 0 ? i : i ^ 0x7fffffff;
}

__device__ __forceinline__ float my_asinh_dev(float v) {
  const double d = v;
  return (float)log(d + sqrt(1. + d * d));  // splotch/splotchutils.cc:31-32
}

struct Fields {
  float *I, *er, *eg, *eb;
  const float *r;
  const uint16_t *type;
  int64_t stride;  // in floats: 9 for particle_sim records, 1 for SoA arrays
  int64_t tstride; // in uint16: 18 for records, 1 for SoA
};

__global__ void __launch_bounds__(256) k_norm_collect(Fields f, int64_t n, NormConst c,
                                                      int *__restrict__ stats,
                                                      uint32_t *err) {
  __shared__ int s[SPL_MAXT * kStats];
  for (int k = threadIdx.x; k < SPL_MAXT * kStats; k += blockDim.x)
    s[k] = (k & 1) ? ord(-1e37f) : ord(1e37f);  // even: min, odd: max
  __syncthreads();
  auto collect = [&](int t, int which, float v) {
    if (v != v) return;  // NaN never replaces a bound
    atomicMin(&s[t * kStats + 2 * which], ord(v));
    atomicMax(&s[t * kStats + 2 * which + 1], ord(v));
  };
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int t = f.type ? (int)f.type[i * f.tstride] : 0;
    if (t >= c.ptypes) {
      atomicOr(err, 1u);
      continue;
    }
    const int64_t o = i * f.stride;
    collect(t, 0, f.r[o]);
    float I = f.I[o];
    if (c.intensity_log[t]) {
      if (I > 0.f) {
        I = log10f(I);
        collect(t, 1, I);
      } else {
        I = -38.f;
      }
      f.I[o] = I;
    } else {
      collect(t, 1, I);
    }
    float er = f.er[o];
    if (c.color_log[t]) {
      if (er > 0.f) {
        er = log10f(er);
        collect(t, 2, er);
      } else {
        er = -38.f;
      }
      f.er[o] = er;
    } else {
      if (c.color_asinh[t]) {
        er = my_asinh_dev(er);
        f.er[o] = er;
      }
      collect(t, 2, er);
    }
    if (c.color_is_vector[t]) {
      float eg = f.eg[o], eb = f.eb[o];
      if (c.color_log[t]) {
        eg = log10f(eg);
        eb = log10f(eb);
      }
      if (c.color_asinh[t]) {
        eg = my_asinh_dev(eg);
        eb = my_asinh_dev(eb);
      }
      if (c.color_log[t] || c.color_asinh[t]) {
        f.eg[o] = eg;
        f.eb[o] = eb;
      }
      collect(t, 2, eg);
      collect(t, 2, eb);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < c.ptypes * kStats; k += blockDim.x) {
    const int init = (k & 1) ? ord(-1e37f) : ord(1e37f);
    if (s[k] == init) continue;
    if (k & 1) atomicMax(&stats[k], s[k]); else atomicMin(&stats[k], s[k]);
  }
}

// Normalizer::normAndClamp (splotch/splotchutils.h:158-165)
__device__ __forceinline__ float norm_clamp(float v, float lo, float hi) {
  if (hi == lo) return 1.f;
  float m = (v < hi) ? v : hi;  // min(maxv, v)
  m = (lo < m) ? m : lo;        // max(minv, .)
  return fdiv(fsub(m, lo), fsub(hi, lo));
}

__global__ void __launch_bounds__(256) k_norm_clamp(Fields f, int64_t n, NormConst c,
                                                    NormRanges rg) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int t = f.type ? (int)f.type[i * f.tstride] : 0;
    if (t >= c.ptypes) continue;
    const int64_t o = i * f.stride;
    f.I[o] = norm_clamp(f.I[o], rg.imin[t], rg.imax[t]);
    f.er[o] = norm_clamp(f.er[o], rg.cmin[t], rg.cmax[t]);
    if (c.color_is_vector[t]) {
      f.eg[o] = norm_clamp(f.eg[o], rg.cmin[t], rg.cmax[t]);
      f.eb[o] = norm_clamp(f.eb[o], rg.cmin[t], rg.cmax[t]);
    }
  }
}

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b > 0 ? b : 1);
}

Fields fields(const NormView &v) {
  Fields f;
  if (v.aos) {
    float *base = static_cast<float *>(v.aos);
    f.er = base + 0;
    f.eg = base + 1;
    f.eb = base + 2;
    f.r = base + 6;
    f.I = base + 7;
    f.type = reinterpret_cast<const uint16_t *>(static_cast<uint8_t *>(v.aos) + 32);
    f.stride = 9;
    f.tstride = 18;
  } else {
    f.I = v.I;
    f.er = v.cr;
    f.eg = v.cg;
    f.eb = v.cb;
    f.r = v.r;
    f.type = v.type;
    f.stride = 1;
    f.tstride = 1;
  }
  return f;
}

}  // namespace

void norm_stats_init(int *h_stats) {
  for (int k = 0; k < SPL_MAXT * kStats; ++k) {
    const float v = (k & 1) ? -1e37f : 1e37f;
    int i;
    std::memcpy(&i, &v, 4);
    h_stats[k] = i >= 0 ? i : i ^ 0x7fffffff;
  }
}

float norm_stat_value(int i) {
  const int b = i >= 0 ? i : i ^ 0x7fffffff;
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}

void launch_norm_collect(const NormView &v, int64_t n, const NormConst &c, int *stats,
                         uint32_t *err, cudaStream_t s) {
  if (n <= 0) return;
  k_norm_collect<<<grid_for(n), 256, 0, s>>>(fields(v), n, c, stats, err);
}

void launch_norm_clamp(const NormView &v, int64_t n, const NormConst &c, const NormRanges &r,
                       cudaStream_t s) {
  if (n <= 0) return;
  k_norm_clamp<<<grid_for(n), 256, 0, s>>>(fields(v), n, c, r);
}

}  // namespace spl
