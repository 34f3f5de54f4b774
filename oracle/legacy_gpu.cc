// legacy_gpu.cc -- TEST INFRASTRUCTURE ONLY: a host driver for the
// reference's own legacy GPU kernels (cuda/cuda_kernel.cu: k_range,
// k_process, k_render), compiled from the reference sources to PTX by
// oracle/build_ref.sh.  It is the GPU floor the benchmark reports beside the
// CPU baseline; nothing in the product path loads it.
//
// What it does per frame follows cuda_rendering with one chunk
// (cuda/cuda_splotch.cc:121-183) and cu_draw_chunk's full-atomics branch
// (cuda/cuda_render.cu:236-262): clear the device image, copy the particle_sim
// records host -> device, k_range, k_process and k_render with 512-thread
// blocks (cuda/cuda_policy.cu:38,82-89) and a device synchronisation after
// each, then copy the image back.  The constant-memory parameter block is
// filled as cu_get_trans_params / cu_init_transform fill it
// (cuda/cuda_utils.cu:46-246), from camera quantities the caller computes with
// the oracle's restatement of the reference camera; the colour map as
// setup_colormap lays it out (cuda/cuda_splotch.cc:186-233).
//
// The parameter block's layout is the reference's cu_param
// (cuda/cuda_utils.h:83-108), restated member for member: the kernels read it
// from constant memory by offset, so it has to be alike.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace {

struct LegacyParam {  // cu_param, cuda/cuda_utils.h:83-108
  float p[12];
  bool projection;
  int xres, yres;
  float fovfct, dist, xfac;
  float minrad_pix;
  double xshift, yshift;
  int ptypes;
  float zmaxval, zminval;
  bool col_vector[8];
  float brightness[8];
  float smooth_fac[8];
  bool log_int[8];
  bool log_col[8];
  bool asinh_col[8];
  float inorm_mins[8];
  float inorm_maxs[8];
  float cnorm_mins[8];
  float cnorm_maxs[8];
  bool do_logs;
  float bfak, h2sigma, rfac;
};

struct LegacyMapEntry {  // cu_color_map_entry
  float val, r, g, b;
};

struct State {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t k_range = nullptr, k_process = nullptr, k_render = nullptr;
  void *d_params = nullptr, *d_map = nullptr, *d_points = nullptr;
  size_t params_bytes = 0, map_bytes = 0, points_bytes = 0;
  void *d_particles = nullptr;
  size_t particles_cap = 0;
  float *d_pic = nullptr;
  size_t pic_cap = 0;
};
State g;

int check(cudaError_t e) { return e == cudaSuccess ? 0 : (int)e; }

}  // namespace

extern "C" {

// The inputs of one frame.  Camera quantities as the reference computes them
// (TRANSFORM matrix, fovfct, dist, xfac, xshift, yshift).
typedef struct {
  float mat[12];
  int projection, xres, yres;
  float fovfct, dist, xfac, minrad_pix;
  double xshift, yshift;
  int ptypes;
  int col_vector[8];
  float brightness[8], smooth_fac[8];
  float inorm_min[8], inorm_max[8], cnorm_min[8], cnorm_max[8];
} leg_frame;

// Load the PTX module once per process.  Returns 0 or a CUDA error code.
int leg_open(const char *ptx_path) {
  if (g.lib) return 0;
  int e;
  if ((e = check(cudaLibraryLoadFromFile(&g.lib, ptx_path, nullptr, nullptr, 0, nullptr, nullptr,
                                         0))))
    return e;
  // the kernels' names are those of their C++ signatures
  if ((e = check(cudaLibraryGetKernel(&g.k_range, g.lib, "_Z7k_rangeiP15cu_particle_sim"))) ||
      (e = check(cudaLibraryGetKernel(&g.k_process, g.lib,
                                      "_Z9k_processP15cu_particle_simiii"))) ||
      (e = check(cudaLibraryGetKernel(&g.k_render, g.lib,
                                      "_Z8k_renderiP15cu_particle_simP8cu_color"))) ||
      (e = check(cudaLibraryGetGlobal(&g.d_params, &g.params_bytes, g.lib, "dparams"))) ||
      (e = check(cudaLibraryGetGlobal(&g.d_map, &g.map_bytes, g.lib, "dmap"))) ||
      (e = check(cudaLibraryGetGlobal(&g.d_points, &g.points_bytes, g.lib, "ptype_points"))))
    return e;
  if (g.params_bytes != sizeof(LegacyParam)) return -100;  // layout mismatch
  return 0;
}

// Render one frame.  particles: n particle_sim records (36 bytes) in host
// memory; map: map_size entries (val, r, g, b) of all types, points: the first
// entry of each type; pic: xres*yres*3 floats (x-major) out.  ms[6]: host wall
// time of clear+copy-in, k_range, k_process, k_render, copy-out, and total.
int leg_render(const leg_frame *f, const void *particles, int64_t n, const float *map,
               int map_size, const int *points, float *pic, double *ms) {
  if (!g.lib) return -101;
  if (map_size < 1 || (size_t)map_size * sizeof(LegacyMapEntry) > g.map_bytes) return -102;
  if (f->ptypes < 1 || f->ptypes > 8 || (size_t)f->ptypes * 4 > g.points_bytes) return -103;
  if (n < 0 || n > 0x7fffffffLL) return -104;
  int e;
  LegacyParam prm;
  std::memset(&prm, 0, sizeof prm);
  std::memcpy(prm.p, f->mat, sizeof prm.p);
  prm.projection = f->projection != 0;
  prm.xres = f->xres;
  prm.yres = f->yres;
  prm.fovfct = f->fovfct;
  prm.dist = f->dist;
  prm.xfac = f->xfac;
  prm.minrad_pix = f->minrad_pix;
  prm.xshift = f->xshift;
  prm.yshift = f->yshift;
  prm.ptypes = f->ptypes;
  prm.zmaxval = 1e23f;
  prm.zminval = 0.f;
  for (int t = 0; t < f->ptypes; ++t) {
    prm.col_vector[t] = f->col_vector[t] != 0;
    prm.brightness[t] = f->brightness[t];
    prm.smooth_fac[t] = f->smooth_fac[t];
    prm.inorm_mins[t] = f->inorm_min[t];
    prm.inorm_maxs[t] = f->inorm_max[t];
    prm.cnorm_mins[t] = f->cnorm_min[t];
    prm.cnorm_maxs[t] = f->cnorm_max[t];
  }
  prm.do_logs = true;
  const double pi = 3.141592653589793238462643383279502884197;
  prm.h2sigma = (float)(0.5 * std::pow(pi, -1. / 6.));  // cuda/cuda_utils.cu:103
  prm.bfak = (float)(0.5 * std::pow(pi, -5. / 6.));     // SPLOTCH_CLASSIC, :106
  prm.rfac = 0.75f;
  const size_t pbytes = (size_t)n * 36, picn = (size_t)f->xres * f->yres * 3;
  if (pbytes > g.particles_cap) {
    if (g.d_particles) cudaFree(g.d_particles);
    g.d_particles = nullptr;
    if ((e = check(cudaMalloc(&g.d_particles, pbytes ? pbytes : 36)))) return e;
    g.particles_cap = pbytes;
  }
  if (picn * 4 > g.pic_cap) {
    if (g.d_pic) cudaFree(g.d_pic);
    g.d_pic = nullptr;
    if ((e = check(cudaMalloc(&g.d_pic, picn * 4)))) return e;
    g.pic_cap = picn * 4;
  }
  if ((e = check(cudaMemcpy(g.d_params, &prm, sizeof prm, cudaMemcpyHostToDevice))) ||
      (e = check(cudaMemcpy(g.d_map, map, (size_t)map_size * 16, cudaMemcpyHostToDevice))) ||
      (e = check(cudaMemcpy(g.d_points, points, (size_t)f->ptypes * 4, cudaMemcpyHostToDevice))))
    return e;
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  if ((e = check(cudaMemset(g.d_pic, 0, picn * 4))) ||
      (e = check(cudaMemcpy(g.d_particles, particles, pbytes, cudaMemcpyHostToDevice))))
    return e;
  const auto t1 = clk::now();
  const int nP = (int)n;
  const dim3 block(512), grid((unsigned)((nP + 511) / 512));
  int msize = map_size, ptypes = f->ptypes;
  void *args_range[] = {(void *)&nP, (void *)&g.d_particles};
  void *args_process[] = {(void *)&g.d_particles, (void *)&nP, (void *)&msize, (void *)&ptypes};
  void *args_render[] = {(void *)&nP, (void *)&g.d_particles, (void *)&g.d_pic};
  if (nP > 0) {
    if ((e = check(cudaLaunchKernel((const void *)g.k_range, grid, block, args_range, 0,
                                    nullptr))) ||
        (e = check(cudaDeviceSynchronize())))
      return e;
  }
  const auto t2 = clk::now();
  if (nP > 0) {
    if ((e = check(cudaLaunchKernel((const void *)g.k_process, grid, block, args_process, 0,
                                    nullptr))) ||
        (e = check(cudaDeviceSynchronize())))
      return e;
  }
  const auto t3 = clk::now();
  if (nP > 0) {
    if ((e = check(cudaLaunchKernel((const void *)g.k_render, grid, block, args_render, 0,
                                    nullptr))) ||
        (e = check(cudaDeviceSynchronize())))
      return e;
  }
  const auto t4 = clk::now();
  if ((e = check(cudaMemcpy(pic, g.d_pic, picn * 4, cudaMemcpyDeviceToHost)))) return e;
  const auto t5 = clk::now();
  const auto d = [](clk::time_point a, clk::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
  };
  if (ms) {
    ms[0] = d(t0, t1);
    ms[1] = d(t1, t2);
    ms[2] = d(t2, t3);
    ms[3] = d(t3, t4);
    ms[4] = d(t4, t5);
    ms[5] = d(t0, t5);
  }
  return 0;
}

void leg_close(void) {
  if (g.d_particles) cudaFree(g.d_particles);
  if (g.d_pic) cudaFree(g.d_pic);
  if (g.lib) cudaLibraryUnload(g.lib);
  g = State();
}

}  // extern "C"
