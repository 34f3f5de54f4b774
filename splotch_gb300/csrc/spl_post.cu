// spl_post.cu -- what Splotch's main does with the image after host_rendering
// (splotch/splotch.cc:272-323), on the device:
//   * additive frames: pic = -expm1(pic) with exptable<float32>(-20)
//     (splotch/splotchutils.h:174-215), tables built on the host exactly as the
//     reference builds them;
//   * colour_adjust (splotch/splotchutils.cc:230-250): kontrast*pow(v, gamma)
//     + helligkeit in double;
//   * add_colorbar (splotch/splotchutils.cc:35-58): 10 rows per palette type;
//   * LS_Image output (cxxsupport/ls_image.cc:178-314): Colour8 conversion
//     int(v*256) clamped to [0,255], transposed from the x-major image to the
//     file's row order (BGR for TGA, RGB for PPM).  The run-length TGA form is
//     encoded on the host from these rows.
// The image pass is HBM-bound: 12 B read + 12 B written per pixel for the
// elementwise step, 12 B read + 3 B written for the byte conversion.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "spl_host.h"

namespace spl {
namespace {

struct ExpTable {
  float expfac, taylorlimit;
};

// exptable<float32>::expm1 (splotchutils.h:203-214) with the tables in
// shared memory.
__device__ __forceinline__ float table_expm1(float arg, const ExpTable &t, const float *tab1,
                                             const float *tab2) {
  if (fabsf(arg) < t.taylorlimit) return arg;
  const int iarg = f2i(fmul(arg, t.expfac));
  float e;
  if (iarg & ~((1 << 20) - 1))
    e = iarg < 0 ? 1.f : 0.f;
  else
    e = fmul(tab1[iarg >> 10], tab2[iarg & 1023]);
  return fsub(e, 1.f);
}

__device__ __forceinline__ float post_one(float v, bool do_expm1, bool do_adjust,
                                          const ExpTable &t, const float *tab1,
                                          const float *tab2, double gamma, double bright,
                                          double contrast) {
  if (do_expm1) v = -table_expm1(v, t, tab1, tab2);
  if (do_adjust) v = (float)dadd(dmul(contrast, pow((double)v, gamma)), bright);
  return v;
}

__global__ void __launch_bounds__(256) k_post(float *__restrict__ pic, int64_t n, bool do_expm1,
                                              bool do_adjust, ExpTable t,
                                              const float *__restrict__ g_tab1,
                                              const float *__restrict__ g_tab2, double gamma,
                                              double bright, double contrast) {
  __shared__ float tab1[1024], tab2[1024];
  if (do_expm1)
    for (int k = threadIdx.x; k < 1024; k += blockDim.x) {
      tab1[k] = g_tab1[k];
      tab2[k] = g_tab2[k];
    }
  __syncthreads();
  // float4 body when the image is 16-byte aligned, scalar otherwise
  const bool vec = (reinterpret_cast<uintptr_t>(pic) & 15u) == 0;
  const int64_t n4 = vec ? n / 4 : 0;
  float4 *p4 = reinterpret_cast<float4 *>(pic);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += stride) {
    float4 v = p4[i];
    v.x = post_one(v.x, do_expm1, do_adjust, t, tab1, tab2, gamma, bright, contrast);
    v.y = post_one(v.y, do_expm1, do_adjust, t, tab1, tab2, gamma, bright, contrast);
    v.z = post_one(v.z, do_expm1, do_adjust, t, tab1, tab2, gamma, bright, contrast);
    v.w = post_one(v.w, do_expm1, do_adjust, t, tab1, tab2, gamma, bright, contrast);
    p4[i] = v;
  }
  for (int64_t i = n4 * 4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    pic[i] = post_one(pic[i], do_expm1, do_adjust, t, tab1, tab2, gamma, bright, contrast);
}

// rows[k] = first image row of colour bar k; colours: xres rgb per bar
__global__ void k_colorbar(float *__restrict__ pic, int xres, int yres,
                           const float *__restrict__ colours, const int *__restrict__ rows,
                           int nbars) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= xres) return;
  for (int k = 0; k < nbars; ++k) {
    const float *c = colours + ((size_t)k * xres + x) * 3;
    for (int y = 0; y < 10; ++y) {
      const int row = rows[k] - y;
      if (row < 0 || row >= yres) continue;
      float *o = pic + ((size_t)x * yres + row) * 3;
      o[0] = c[0];
      o[1] = c[1];
      o[2] = c[2];
    }
  }
}

// Colour8 of every pixel, transposed from x-major to rows of the file: a
// 32x32-pixel tile per block, read along y (contiguous in the x-major image)
// and written along x (contiguous in a row).  bgr: TGA channel order.
__global__ void __launch_bounds__(256) k_encode(const float *__restrict__ pic, int xres, int yres,
                                                bool bgr, uint8_t *__restrict__ out) {
  __shared__ uint8_t tile[32][32 * 3 + 1];
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 rows of 32
  for (int dx = ty; dx < 32; dx += 8) {  // read: lanes along y
    const int x = x0 + dx, y = y0 + tx;
    if (x < xres && y < yres) {
      const float *s = pic + ((size_t)x * yres + y) * 3;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int v = f2i(fmul(s[c], 256.f));
        tile[tx][dx * 3 + (bgr ? 2 - c : c)] = (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
      }
    }
  }
  __syncthreads();
  for (int dy = ty; dy < 32; dy += 8) {  // write: lanes along x
    const int y = y0 + dy, x = x0 + tx;
    if (x < xres && y < yres) {
      uint8_t *o = out + ((size_t)y * xres + x) * 3;
      o[0] = tile[dy][tx * 3];
      o[1] = tile[dy][tx * 3 + 1];
      o[2] = tile[dy][tx * 3 + 2];
    }
  }
}

}  // namespace

void exptable_tables(float maxexp, float *tab1, float *tab2, float *expfac,
                     float *taylorlimit) {
  // exptable<float32>(maxexp) (splotchutils.h:186-196): float arithmetic,
  // std::exp of a float
  const int dim1 = 1 << 10, dim2 = 1 << 20;
  const float ef = dim2 / maxexp;
  for (int m = 0; m < dim1; ++m) {
    tab1[m] = std::exp(m * dim1 / ef);
    tab2[m] = std::exp(m / ef);
  }
  *expfac = ef;
  *taylorlimit = std::sqrt(float(2) * std::abs(maxexp) / dim2);
}

void launch_post(float *pic, int64_t nfloats, bool do_expm1, bool do_adjust, float expfac,
                 float taylorlimit, const float *tab1, const float *tab2, double gamma,
                 double bright, double contrast, cudaStream_t s) {
  if (nfloats <= 0 || (!do_expm1 && !do_adjust)) return;
  int64_t blocks = (nfloats / 4 + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  k_post<<<(unsigned)blocks, 256, 0, s>>>(pic, nfloats, do_expm1, do_adjust,
                                          ExpTable{expfac, taylorlimit}, tab1, tab2, gamma,
                                          bright, contrast);
}

void launch_colorbar(float *pic, int xres, int yres, const float *colours, const int *rows,
                     int nbars, cudaStream_t s) {
  if (nbars <= 0 || xres <= 0) return;
  k_colorbar<<<(xres + 255) / 256, 256, 0, s>>>(pic, xres, yres, colours, rows, nbars);
}

void launch_encode(const float *pic, int xres, int yres, bool bgr, uint8_t *out,
                   cudaStream_t s) {
  if (xres <= 0 || yres <= 0) return;
  dim3 grid((xres + 31) / 32, (yres + 31) / 32);
  k_encode<<<grid, 256, 0, s>>>(pic, xres, yres, bgr, out);
}

}  // namespace spl
