// spl_api.cu -- the C ABI of libsplgpu.so: context, buffer pool and the
// plain-render pipeline that replaces host_rendering()
// (splotch/splotch_host.cc:711-834):
//
//   H2D (host inputs) -> project+colourise -> [stable depth sort] ->
//   count scan -> bin emission -> stable tile sort -> tile ranges ->
//   tiled splat -> D2H (host outputs) [-> particle writeback]
//
// All device memory is owned by the context and grows on demand; a frame that
// fits the current capacity allocates nothing.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/splotch_gb300.h"
#include "spl_host.h"
#include "spl_internal.cuh"

struct spl_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  struct Buf {
    void *p = nullptr;
    size_t cap = 0;
  };
  Buf aos_in, soa_in[9], pos, col, active, count, key, perm, ktmp, vtmp, off, scratch, tkey,
      tval, tkey2, tval2, tkey_s, tval_s, tile_start, wide_list, small, pic, pal_x, pal_rgb,
      aos_out, pal_thr, pal_xff, pal_invff, tcost, tcost_s, tord, pos_c, col_c, idx_c, pstate,
      poff, gpic, gpos_c, gcol_c, camsum, gout[8], aux, post_tab, post_bar, post_img, post_bytes,
      seg_cnt, seg_off, seg_state, ray_rc, ray_cf, ray_pod, ray_cov, ray_code, ray_lev, ray_slots,
      ray_rc2, ray_cf2, ray_pod2, ray_cov2, ray_clo, ray_clo2,
      ray_kd, ray_segcnt, ray_segoff, ray_items, ray_partial,
      ray_nodes, ray_regs, ray_box, ray_leaf_start, ray_img[2], ray_jstop;
  // spl_render_rays: the host-built region trees of the last geometry
  struct RayKey {
    int xres, yres, dome;
    double fov, minrad_pix, v[12];  // campos, centerpos, lookat, sky
  };
  RayKey ray_key{};
  spl::RayFrame *rays = nullptr;
  int debug_flags = 0;  // SPL_DEBUG_* bits
  bool differentiable = false;  // ordered forwards keep SplatArgs::aux
  int split_mode = SPL_SPLIT_ADDITIVE;  // which frames have heavy tiles cut into segments
  // state of the last frame (for the debug getters)
  int64_t n = 0, na = 0, ne = 0, ntiles = 0;
  bool has_order = false, writeback_done = false;
  int last_T = 0;
  spl::SplatArgs last_splat{};
  spl::ProjConst last_pc{};
  const void *last_aos = nullptr;
  spl::SoAIn last_soa{};
  spl_stats stats{};
  cudaEvent_t ev[8]{};
  // spl_prefetch: host inputs copied ahead on copy_stream into a ring of
  // slots.  A slot is queued from its prefetch until the spl_render that
  // reads it, then in use until the next spl_render (spl_render_backward
  // reads the inputs again); `freed` is recorded on the render stream after
  // the last kernel that read it, and a new prefetch into the slot waits on it.
  struct InSlot {
    Buf aos, soa[9];
    const void *host[10] = {};  // aos, x, y, z, r, I, cr, cg, cb, type
    int64_t n = 0;
    int layout = -1;
    cudaEvent_t ready = nullptr, freed = nullptr;
    bool queued = false;
  };
  InSlot pf[3];
  int pf_fifo[3] = {-1, -1, -1};  // queued slots, oldest first
  int pf_len = 0;
  int pf_in_use = -1;             // slot read by the last render
  cudaStream_t copy_stream = nullptr;
};

namespace {

thread_local std::string g_err;

spl_status fail(spl_status code, const std::string &msg) {
  g_err = msg;
  return code;
}

#define SPL_CK(call)                                                                    \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(SPL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
  } while (0)

std::atomic<int64_t> g_alloc_countdown{0};  // spl_debug_fail_alloc

spl_status ensure(spl_context::Buf &b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (b.cap >= bytes) return SPL_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  size_t want = bytes + bytes / 8;  // headroom for slowly growing frames
  if (spl::alloc_failure_due())
    return fail(SPL_ERR_ALLOC, "cudaMalloc(" + std::to_string(want) +
                                   "): failure injected by spl_debug_fail_alloc");
  cudaError_t e = cudaMalloc(&b.p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SPL_ERR_ALLOC, "cudaMalloc(" + std::to_string(want) + "): " +
                                   cudaGetErrorString(e));
  }
  b.cap = want;
  return SPL_OK;
}

template <typename T>
T *as(spl_context::Buf &b) {
  return static_cast<T *>(b.p);
}

int is_device_ptr(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

spl_status validate(const spl_frame_desc *d, const spl_particles *p, const spl_image *o) {
  if (!d || !p || !o) return fail(SPL_ERR_INVALID, "null argument");
  if (d->xres <= 0 || d->yres <= 0 || d->xres > 65536 || d->yres > 65536)
    return fail(SPL_ERR_INVALID, "xres/yres out of range");
  if (d->tile_size < 1 || d->tile_size > 64)
    return fail(SPL_ERR_UNSUPPORTED, "tile size must be in [1,64] on the GPU path");
  if (d->ptypes < 1 || d->ptypes > SPL_MAX_TYPES)
    return fail(SPL_ERR_INVALID, "ptypes must be in [1,8]");
  if (d->sort_type < 0 || d->sort_type > 4)
    return fail(SPL_ERR_INVALID, "unknown sorting chosen ...");  // splotch_host.cc:318
  for (int t = 0; t < d->ptypes; ++t)
    if (!d->color_is_vector[t] && (d->pal_n[t] < 1 || !d->pal_x[t] || !d->pal_rgb[t]))
      return fail(SPL_ERR_INVALID, "trying to access an empty map (palette of type " +
                                       std::to_string(t) + ")");
  if (p->n < 0 || p->n > 0xffffffffLL) return fail(SPL_ERR_INVALID, "particle count out of range");
  if (p->layout == SPL_LAYOUT_AOS) {
    if (p->n > 0 && !p->aos) return fail(SPL_ERR_INVALID, "null AoS pointer");
  } else if (p->layout == SPL_LAYOUT_SOA) {
    if (p->n > 0 && (!p->x || !p->y || !p->z || !p->r || !p->I || !p->cr))
      return fail(SPL_ERR_INVALID, "null SoA pointer");
  } else {
    return fail(SPL_ERR_INVALID, "unknown layout");
  }
  if (!o->pic) return fail(SPL_ERR_INVALID, "null image pointer");
  if (o->memspace == SPL_MEM_DEVICE && !is_device_ptr(o->pic))
    return fail(SPL_ERR_INVALID, "image marked device but pointer is not device memory");
  if (p->memspace == SPL_MEM_DEVICE && p->n > 0) {
    const void *probe = p->layout == SPL_LAYOUT_AOS ? p->aos : (const void *)p->x;
    if (!is_device_ptr(probe))
      return fail(SPL_ERR_INVALID, "particles marked device but pointer is not device memory");
  }
  return SPL_OK;
}

float2 split_ff(double v) {  // v as a float-float pair (hi, lo)
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

float least_float_above(double v) {  // least float f with f > v
  float f = (float)v;
  if ((double)f <= v) f = std::nextafter(f, INFINITY);
  return f;
}

float least_float_not_below(double v) {  // least float f with f >= v
  float f = (float)v;
  if ((double)f < v) f = std::nextafter(f, INFINITY);
  return f;
}

float greatest_float_not_above(double v) {  // greatest float f with f <= v
  float f = (float)v;
  if ((double)f > v) f = std::nextafter(f, -INFINITY);
  return f;
}

// Every particle's projected state (indexed by particle) from the last
// frame's inputs and constants: the writeback and the projection test hook.
spl_status project_full(spl_context *c, int64_t n, bool with_key, int *launches) {
  spl_status st;
  if ((st = ensure(c->pos, n * sizeof(float4))) || (st = ensure(c->col, n * sizeof(float4))) ||
      (st = ensure(c->active, n)) || (with_key && (st = ensure(c->key, n * 4))))
    return st;
  spl::ProjectOut po;
  std::memset(&po, 0, sizeof(po));
  po.pos = as<float4>(c->pos);
  po.col = as<float4>(c->col);
  po.active = as<uint8_t>(c->active);
  po.key = with_key ? as<uint32_t>(c->key) : nullptr;
  po.err = as<uint32_t>(c->small);
  spl::ProjConst pc = c->last_pc;
  pc.n_fallback = nullptr;
  spl::launch_project(c->last_aos, &c->last_soa, n, pc, po, false, c->stream, launches);
  return SPL_OK;
}

}  // namespace

void spl::set_last_error(const char *msg) { g_err = msg; }

bool spl::alloc_failure_due() {
  int64_t v = g_alloc_countdown.load();
  while (v > 0) {  // count this allocation; the one that reaches zero fails
    if (g_alloc_countdown.compare_exchange_weak(v, v - 1)) return v == 1;
  }
  return false;
}

spl_status spl::host_fail(spl_status code, const std::string &msg) { return fail(code, msg); }

// The host arrays of a particle view, in a fixed order (aos, x, y, z, r, I,
// cr, cg, cb, type), for matching a render to a prefetch.
static void host_keys(const spl_particles *p, const void *k[10]) {
  const void *v[10] = {p->aos, p->x, p->y, p->z, p->r, p->I, p->cr, p->cg, p->cb, p->type};
  for (int i = 0; i < 10; ++i) k[i] = p->layout == SPL_LAYOUT_AOS ? (i == 0 ? v[0] : nullptr)
                                                                  : (i == 0 ? nullptr : v[i]);
}

// The oldest queued prefetch if it holds this view's host arrays (it leaves
// the queue), else -1 and the queue is dropped (stale or out of order).
static int take_prefetch(spl_context *c, const spl_particles *p) {
  if (c->pf_len == 0) return -1;
  const int slot = c->pf_fifo[0];
  const spl_context::InSlot &q = c->pf[slot];
  const void *k[10];
  host_keys(p, k);
  bool match = q.layout == p->layout && q.n == p->n;
  for (int i = 0; match && i < 10; ++i) match = k[i] == q.host[i];
  if (!match) {
    for (int i = 0; i < c->pf_len; ++i) c->pf[c->pf_fifo[i]].queued = false;
    c->pf_len = 0;
    return -1;
  }
  c->pf[slot].queued = false;
  for (int i = 1; i < c->pf_len; ++i) c->pf_fifo[i - 1] = c->pf_fifo[i];
  --c->pf_len;
  return slot;
}

spl_status spl::validate_frame(const spl_frame_desc *d, const spl_particles *p,
                               const spl_image *o) {
  return validate(d, p, o);
}

int spl::context_device(const spl_context *c) { return c->device; }

int spl::bits_for(int64_t v) {
  int b = 0;
  while (b < 32 && ((int64_t)1 << b) < v) ++b;
  return b;
}

spl_status spl::frame_setup(const spl_frame_desc *d, int T, bool exact_fp64, FrameSetup &fs,
                            bool camera) {
  spl_camera cam;
  std::memset(&cam, 0, sizeof(cam));
  if (camera && spl_camera_setup(d, &cam))
    return fail(SPL_ERR_INVALID, "degenerate matrix in TRANSMAT::Inverse()");
  const int xres = d->xres, yres = d->yres;
  ProjConst &pc = fs.pc;
  std::memset(&pc, 0, sizeof(pc));
  std::memcpy(pc.mat, cam.mat, sizeof(pc.mat));
  pc.res2 = cam.res2;
  pc.ycorr = cam.ycorr;
  pc.fovfct = cam.fovfct;
  pc.xfac = cam.xfac;
  pc.xsum = (double)cam.res2 + cam.xshift;
  pc.ysum = (double)cam.res2 + cam.yshift + (double)cam.ycorr;
  {
    const float2 xs = split_ff(pc.xsum), ys = split_ff(pc.ysum);
    pc.xsum_ff = ff{xs.x, xs.y};
    pc.ysum_ff = ff{ys.x, ys.y};
  }
  pc.exact_fp64 = exact_fp64 ? 1 : 0;
  pc.zmin = d->zmin > 0.f ? d->zmin : 0.f;
  pc.zmax = d->zmax;
  pc.minrad2 = d->minrad_pix * d->minrad_pix;
  const float bfak = (float)(0.5 * std::pow(3.141592653589793238462643383279502884197, -5. / 6.));
  pc.half_bfak = 0.5f * bfak;
  pc.xres = xres;
  pc.yres = yres;
  pc.projection = d->projection ? 1 : 0;
  pc.ptypes = d->ptypes;
  int npal = 0;
  for (int t = 0; t < d->ptypes; ++t) {
    pc.smooth[t] = d->smooth_factor[t];
    pc.bright[t] = d->brightness[t] * d->b_brightness;
    pc.colvec[t] = d->color_is_vector[t] ? 1 : 0;
    pc.pal_off[t] = npal;
    pc.pal_n[t] = d->color_is_vector[t] ? 0 : d->pal_n[t];
    npal += pc.pal_n[t];
  }
  Tiling &g = fs.g;
  g.T = T;
  g.ncx = (xres + T - 1) / T;
  g.ncy = (yres + T - 1) / T;
  g.rcell = std::sqrt(2.f) * (T * 0.5f - 0.5f);
  g.cmid0 = 0.5f * (T - 1);
  pc.T = g.T;
  pc.ncx = g.ncx;
  pc.ncy = g.ncy;
  pc.rcell = g.rcell;
  pc.cmid0 = g.cmid0;
  fs.do_sort = !d->a_eq_e && d->sort_type != 0;
  pc.sort_type = fs.do_sort ? d->sort_type : 0;
  pc.pal_cache = nullptr;
  fs.ntiles = (int64_t)g.ncx * g.ncy;
  if (fs.ntiles >= 0xffffffffLL) return fail(SPL_ERR_INVALID, "too many tiles");
  fs.npal = npal;
  fs.pal_x.assign(npal + 1, 0.0);
  fs.pal_rgb.assign(3 * (size_t)(npal + 1), 0.f);
  fs.thr.assign(npal + 1, 0.f);
  fs.xff.assign(npal + 1, make_float2(0.f, 0.f));
  fs.invff.assign(npal + 1, make_float2(0.f, 0.f));
  for (int t = 0; t < d->ptypes; ++t) {
    const int nk = pc.pal_n[t], o = pc.pal_off[t];
    if (!nk) continue;
    const double *x = d->pal_x[t];
    for (int k = 0; k < nk; ++k) {
      fs.pal_x[o + k] = x[k];
      for (int ch = 0; ch < 3; ++ch) fs.pal_rgb[3 * (o + k) + ch] = d->pal_rgb[t][3 * k + ch];
      fs.thr[o + k] = least_float_above(x[k]);
      fs.xff[o + k] = split_ff(x[k]);
      fs.invff[o + k] = k + 1 < nk ? split_ff(1.0 / (x[k + 1] - x[k])) : make_float2(0.f, 0.f);
    }
    pc.pal_lo_f[t] = greatest_float_not_above(x[0]);
    pc.pal_hi_f[t] = least_float_not_below(x[nk - 1]);
  }
  return SPL_OK;
}

extern "C" {

const char *spl_last_error_string(void) { return g_err.c_str(); }

const char *spl_version(void) { return "splotch_gb300 0.1 (sm_103a)"; }

spl_status spl_context_create(spl_context **ctx, int device) {
  if (!ctx) return fail(SPL_ERR_INVALID, "null ctx");
  *ctx = nullptr;
  int ndev = 0;
  SPL_CK(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return fail(SPL_ERR_INVALID, "no such device");
  SPL_CK(cudaSetDevice(device));
  spl_context *c = new spl_context();
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return fail(SPL_ERR_CUDA, "cudaStreamCreate failed");
  }
  c->own_stream = true;
  for (auto &e : c->ev) cudaEventCreate(&e);
  *ctx = c;
  return SPL_OK;
}

spl_status spl_context_destroy(spl_context *c) {
  if (!c) return SPL_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  spl_context::Buf *bufs[] = {&c->aos_in, &c->pos, &c->col, &c->active, &c->count, &c->key,
                              &c->perm, &c->ktmp, &c->vtmp, &c->off, &c->scratch, &c->tkey,
                              &c->tval, &c->tkey2, &c->tval2, &c->tkey_s, &c->tval_s,
                              &c->tile_start, &c->wide_list, &c->small, &c->pic, &c->pal_x,
                              &c->pal_rgb, &c->aos_out, &c->pal_thr, &c->pal_xff,
                              &c->pal_invff, &c->tcost, &c->tcost_s, &c->tord, &c->pos_c,
                              &c->col_c, &c->idx_c, &c->pstate, &c->poff, &c->gpic,
                              &c->gpos_c, &c->gcol_c, &c->camsum, &c->aux, &c->post_tab,
                              &c->post_bar, &c->post_img, &c->post_bytes, &c->seg_cnt,
                              &c->seg_off, &c->seg_state, &c->ray_rc, &c->ray_cf,
                              &c->ray_pod, &c->ray_cov, &c->ray_code, &c->ray_lev,
                              &c->ray_nodes, &c->ray_regs, &c->ray_box, &c->ray_leaf_start,
                              &c->ray_img[0], &c->ray_img[1], &c->ray_jstop, &c->ray_slots,
                              &c->ray_kd, &c->ray_segcnt, &c->ray_segoff, &c->ray_items,
                              &c->ray_partial, &c->ray_rc2, &c->ray_cf2, &c->ray_pod2,
                              &c->ray_cov2, &c->ray_clo, &c->ray_clo2};
  for (auto *b : bufs)
    if (b->p) cudaFree(b->p);
  delete c->rays;
  for (auto &b : c->soa_in)
    if (b.p) cudaFree(b.p);
  for (auto &b : c->gout)
    if (b.p) cudaFree(b.p);
  for (auto &e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
  for (auto &q : c->pf) {
    if (q.aos.p) cudaFree(q.aos.p);
    for (auto &b : q.soa)
      if (b.p) cudaFree(b.p);
    if (q.ready) cudaEventDestroy(q.ready);
    if (q.freed) cudaEventDestroy(q.freed);
  }
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return SPL_OK;
}

spl_status spl_context_set_stream(spl_context *c, void *stream) {
  if (!c) return fail(SPL_ERR_INVALID, "null ctx");
  SPL_CK(cudaSetDevice(c->device));
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  c->stream = static_cast<cudaStream_t>(stream);
  c->own_stream = false;
  return SPL_OK;
}

spl_status spl_get_stats(const spl_context *c, spl_stats *s) {
  if (!c || !s) return fail(SPL_ERR_INVALID, "null argument");
  *s = c->stats;
  return SPL_OK;
}

spl_status spl_render(spl_context *c, const spl_frame_desc *d, const spl_particles *p,
                      spl_image *out, int writeback) {
  if (!c) return fail(SPL_ERR_INVALID, "null ctx");
  SPL_CK(cudaSetDevice(c->device));
  spl_status st = validate(d, p, out);
  if (st) return st;
  if (writeback == SPL_WRITEBACK_FULL && p->layout != SPL_LAYOUT_AOS)
    return fail(SPL_ERR_UNSUPPORTED, "writeback needs the AoS (particle_sim) layout");
  cudaStream_t s = c->stream;
  const int64_t n = p->n;
  const int xres = d->xres, yres = d->yres, T = d->tile_size;
  int launches = 0;

  // ---- frame constants ---------------------------------------------------
  spl::FrameSetup fs;
  if ((st = spl::frame_setup(d, T, (c->debug_flags & 1) != 0, fs))) return st;
  spl::ProjConst pc = fs.pc;
  pc.debug_short_count = (c->debug_flags & SPL_DEBUG_SHORT_COUNT) != 0;
  const spl::Tiling g = fs.g;
  const bool onesweep = (c->debug_flags & 2) == 0;
  const int npal = fs.npal;
  const bool do_sort = fs.do_sort;
  const int64_t ntiles = fs.ntiles;

  // ---- buffers -------------------------------------------------------------
  // compact (active-only) arrays are sized for n: the active count is known
  // only after projection
  const int64_t nprojtiles = (n + 255) / 256;
  if ((st = ensure(c->pos_c, n * sizeof(float4))) || (st = ensure(c->col_c, n * sizeof(float4))) ||
      (st = ensure(c->idx_c, n * 4)) || (st = ensure(c->count, n * 4)) ||
      (st = ensure(c->off, (n + 1) * 8)) || (st = ensure(c->wide_list, n * 4)) ||
      (st = ensure(c->small, 256)) || (st = ensure(c->tile_start, (ntiles + 1) * 4)) ||
      (st = ensure(c->pstate, (nprojtiles * 8 + 1) * 4)) ||
      (st = ensure(c->poff, (nprojtiles * 8 + 1) * 4)) ||
      (st = ensure(c->pic, (size_t)xres * yres * 3 * 4)) ||
      (st = ensure(c->pal_x, (npal + 1) * 8)) || (st = ensure(c->pal_rgb, (npal + 1) * 12)))
    return st;
  if ((st = ensure(c->key, n * 4)) || (st = ensure(c->perm, n * 4)) ||
      (st = ensure(c->ktmp, n * 4)) || (st = ensure(c->vtmp, n * 4)))
    return st;
  size_t scr = spl::scan_scratch_bytes(n + 1);
  size_t rs = spl::radix_scratch_bytes(n);
  if (rs > scr) scr = rs;
  if ((st = ensure(c->scratch, scr))) return st;
  // small words: 0 error, 1 wide-particle count, 2 FP64 fallbacks, 3 active
  // count, 4 projection tile counter
  uint32_t *d_err = as<uint32_t>(c->small);
  uint32_t *d_wide_n = d_err + 1;
  uint32_t *d_nact = d_err + 3;

  // palettes (a few KB): exact knots and the float-float tables of the fast
  // colourisation path
  if ((st = ensure(c->pal_thr, (npal + 1) * 4)) || (st = ensure(c->pal_xff, (npal + 1) * 8)) ||
      (st = ensure(c->pal_invff, (npal + 1) * 8)))
    return st;
  // small copies from pageable memory: they travel in the command stream, not
  // behind a large copy-engine transfer (a next frame's prefetch) as copies
  // from pinned memory would
  SPL_CK(cudaMemcpyAsync(c->pal_x.p, fs.pal_x.data(), (npal + 1) * 8, cudaMemcpyHostToDevice, s));
  SPL_CK(cudaMemcpyAsync(c->pal_rgb.p, fs.pal_rgb.data(), (npal + 1) * 12, cudaMemcpyHostToDevice,
                         s));
  SPL_CK(cudaMemcpyAsync(c->pal_thr.p, fs.thr.data(), (npal + 1) * 4, cudaMemcpyHostToDevice, s));
  SPL_CK(cudaMemcpyAsync(c->pal_xff.p, fs.xff.data(), (npal + 1) * 8, cudaMemcpyHostToDevice, s));
  SPL_CK(cudaMemcpyAsync(c->pal_invff.p, fs.invff.data(), (npal + 1) * 8, cudaMemcpyHostToDevice,
                         s));
  // the host tables live in fs: wait for the copies before anything else
  SPL_CK(cudaStreamSynchronize(s));
  pc.pal_x = as<double>(c->pal_x);
  pc.pal_rgb = as<float>(c->pal_rgb);
  pc.pal_thr = as<float>(c->pal_thr);
  pc.pal_xff = as<float2>(c->pal_xff);
  pc.pal_invff = as<float2>(c->pal_invff);
  SPL_CK(cudaMemsetAsync(d_err, 0, 32, s));
  pc.n_fallback = d_err + 2;

  cudaEventRecord(c->ev[0], s);
  // ---- inputs --------------------------------------------------------------
  const void *aos_dev = nullptr;
  spl::SoAIn soa{p->x, p->y, p->z, p->r, p->I, p->cr, p->cg, p->cb, p->type};
  const int slot = p->memspace == SPL_MEM_HOST ? take_prefetch(c, p) : -1;
  c->pf_in_use = slot;
  if (slot >= 0) {  // copied ahead by spl_prefetch: wait for that copy
    spl_context::InSlot &q = c->pf[slot];
    SPL_CK(cudaStreamWaitEvent(s, q.ready, 0));
    if (p->layout == SPL_LAYOUT_AOS) {
      aos_dev = q.aos.p;
    } else {
      const float **f[8] = {&soa.x, &soa.y, &soa.z, &soa.r, &soa.I, &soa.cr, &soa.cg, &soa.cb};
      for (int k = 0; k < 8; ++k)
        if (*f[k]) *f[k] = as<float>(q.soa[k]);
      if (p->type) soa.type = as<uint16_t>(q.soa[8]);
    }
  } else if (p->layout == SPL_LAYOUT_AOS) {
    if (p->memspace == SPL_MEM_HOST) {
      if ((st = ensure(c->aos_in, n * 36))) return st;
      SPL_CK(cudaMemcpyAsync(c->aos_in.p, p->aos, n * 36, cudaMemcpyHostToDevice, s));
      aos_dev = c->aos_in.p;
    } else {
      aos_dev = p->aos;
    }
  } else if (p->memspace == SPL_MEM_HOST) {
    const float **f[8] = {&soa.x, &soa.y, &soa.z, &soa.r, &soa.I, &soa.cr, &soa.cg, &soa.cb};
    for (int k = 0; k < 8; ++k) {
      if (!*f[k]) continue;
      if ((st = ensure(c->soa_in[k], n * 4))) return st;
      SPL_CK(cudaMemcpyAsync(c->soa_in[k].p, *f[k], n * 4, cudaMemcpyHostToDevice, s));
      *f[k] = as<float>(c->soa_in[k]);
    }
    if (p->type) {
      if ((st = ensure(c->soa_in[8], n * 2))) return st;
      SPL_CK(cudaMemcpyAsync(c->soa_in[8].p, p->type, n * 2, cudaMemcpyHostToDevice, s));
      soa.type = as<uint16_t>(c->soa_in[8]);
    }
  }
  cudaEventRecord(c->ev[1], s);

  // ---- project + colourise, active particles compacted -----------------------
  spl::ProjectOut po;
  std::memset(&po, 0, sizeof(po));
  po.pos_c = as<float4>(c->pos_c);
  po.col_c = as<float4>(c->col_c);
  po.idx_c = as<uint32_t>(c->idx_c);
  po.count_c = as<uint32_t>(c->count);
  po.key_c = do_sort ? as<uint32_t>(c->key) : nullptr;
  po.n_act = d_nact;
  po.flags = as<uint32_t>(c->pstate);
  po.word_off = as<uint32_t>(c->poff);
  po.scan_scratch = c->scratch.p;
  po.err = d_err;
  po.cap_c = (uint32_t)n;  // compact arrays hold every particle
  spl::launch_project(aos_dev, &soa, n, pc, po, true, s, &launches);
  uint32_t nact_h = 0;
  SPL_CK(cudaMemcpyAsync(&nact_h, d_nact, 4, cudaMemcpyDeviceToHost, s));
  cudaEventRecord(c->ev[2], s);
  SPL_CK(cudaStreamSynchronize(s));
  const int64_t na = nact_h;

  // ---- depth sort of the active particles (a_eq_e=false), splotch_host.cc:805-815
  // The reference sorts every particle; a stable sort of all of them visits the
  // active ones in exactly the order of this stable sort of the active subset.
  const uint32_t *order = nullptr;
  if (do_sort && na > 0) {
    spl::radix_sort_pairs(as<uint32_t>(c->key), nullptr, as<uint32_t>(c->ktmp),
                          as<uint32_t>(c->vtmp), as<uint32_t>(c->key) /*unused out*/,
                          as<uint32_t>(c->perm), na, 0, 32, false, c->scratch.p, s, &launches,
                          d_err, onesweep, (c->debug_flags & SPL_DEBUG_LOOKBACK_STALL) != 0);
    order = as<uint32_t>(c->perm);
  }
  cudaEventRecord(c->ev[3], s);

  // ---- binning ---------------------------------------------------------------
  // tile counts in visiting order (one gather; the sort's key scratch is free)
  const uint32_t *count_seq = as<uint32_t>(c->count);
  if (order) {
    // a permutation that a look-back left invalid reads nothing out of range
    spl::launch_gather_u32(as<uint32_t>(c->count), order, na, as<uint32_t>(c->ktmp), s, na,
                           d_err);
    ++launches;
    count_seq = as<uint32_t>(c->ktmp);
  }
  uint64_t *off = as<uint64_t>(c->off);
  spl::scan_counts(count_seq, nullptr, na, off, c->scratch.p, s, &launches);
  uint64_t ne = 0;
  uint32_t err_mid = 0;
  SPL_CK(cudaMemcpyAsync(&ne, off + na, 8, cudaMemcpyDeviceToHost, s));
  SPL_CK(cudaMemcpyAsync(&err_mid, d_err, 4, cudaMemcpyDeviceToHost, s));
  SPL_CK(cudaStreamSynchronize(s));
  // the depth sort's permutation is consumed from here on: stop if it is invalid
  if (err_mid & 2u) {
    c->has_order = false;
    return fail(SPL_ERR_TIMEOUT, "a look-back wait of the depth sort gave up");
  }
  if (ne >= 0xffffffffULL) return fail(SPL_ERR_CAPACITY, "more than 2^32-1 bin entries");
  if ((st = ensure(c->tkey, ne * 4)) || (st = ensure(c->tval, ne * 4)) ||
      (st = ensure(c->tkey2, ne * 4)) || (st = ensure(c->tval2, ne * 4)) ||
      (st = ensure(c->tkey_s, ne * 4)) || (st = ensure(c->tval_s, ne * 4)))
    return st;
  size_t rs2 = spl::radix_scratch_bytes((int64_t)ne);
  if ((st = ensure(c->scratch, rs2))) return st;
  if (ne > 0) {
    spl::launch_emit(as<float4>(c->pos_c), count_seq, order, off, na, g,
                     as<uint32_t>(c->tkey), as<uint32_t>(c->tval), as<uint32_t>(c->wide_list),
                     d_wide_n, d_err, s);
    launches += 2;
    const int tb = spl::bits_for(ntiles);
    if (tb > 0) {
      spl::radix_sort_pairs(as<uint32_t>(c->tkey), as<uint32_t>(c->tval),
                            as<uint32_t>(c->tkey2), as<uint32_t>(c->tval2),
                            as<uint32_t>(c->tkey_s), as<uint32_t>(c->tval_s), (int64_t)ne, 0,
                            tb, true, c->scratch.p, s, &launches, d_err, onesweep);
    } else {
      SPL_CK(cudaMemcpyAsync(c->tkey_s.p, c->tkey.p, ne * 4, cudaMemcpyDeviceToDevice, s));
      SPL_CK(cudaMemcpyAsync(c->tval_s.p, c->tval.p, ne * 4, cudaMemcpyDeviceToDevice, s));
    }
  }
  spl::launch_tile_ranges(as<uint32_t>(c->tkey_s), (int64_t)ne, ntiles,
                          as<uint32_t>(c->tile_start), s);
  ++launches;
  // longest lists first: the splat's tail is set by its heaviest tiles
  if ((st = ensure(c->tcost, ntiles * 4)) || (st = ensure(c->tcost_s, ntiles * 4)) ||
      (st = ensure(c->tord, ntiles * 4)) ||
      (st = ensure(c->scratch, spl::radix_scratch_bytes(ntiles))))
    return st;
  spl::launch_tile_cost(as<uint32_t>(c->tile_start), ntiles, as<uint32_t>(c->tcost), s);
  spl::radix_sort_pairs(as<uint32_t>(c->tcost), nullptr, as<uint32_t>(c->tcost_s),
                        as<uint32_t>(c->tord), as<uint32_t>(c->tcost_s), as<uint32_t>(c->tord),
                        ntiles, 0, 8, false, c->scratch.p, s, &launches, d_err, onesweep);
  ++launches;
  cudaEventRecord(c->ev[4], s);

  // ---- splat ---------------------------------------------------------------------
  spl::SplatArgs sa;
  sa.pos = as<float4>(c->pos_c);
  sa.col = as<float4>(c->col_c);
  sa.entries = as<uint32_t>(c->tval_s);
  sa.tile_start = as<uint32_t>(c->tile_start);
  sa.tile_order = as<uint32_t>(c->tord);
  sa.T = T;
  sa.ncx = g.ncx;
  sa.ncy = g.ncy;
  sa.xres = xres;
  sa.yres = yres;
  sa.gray = d->gray_absorption;
  sa.h2sigma = (float)(0.5 * std::pow(3.141592653589793238462643383279502884197, -1. / 6.));
  sa.a_eq_e = d->a_eq_e ? 1 : 0;
  sa.order_mode = d->order_mode;
  sa.ftb_eps = d->ftb_epsilon;
  sa.ftb_rel = d->ftb_relative;
  sa.config = d->splat_config;
  sa.pic = out->memspace == SPL_MEM_DEVICE ? out->pic : as<float>(c->pic);
  sa.aux = nullptr;
  if (c->differentiable && !d->a_eq_e) {
    if ((st = ensure(c->aux, (size_t)xres * yres * 16))) return st;
    sa.aux = as<float4>(c->aux);
  }
  // Heavy tiles cut into list segments when asked (additive and front-to-back
  // frames whose per-pixel data the adjoint does not need)
  const bool split = !sa.aux && ntiles > 0 &&
                     ((sa.a_eq_e && c->split_mode != SPL_SPLIT_OFF) ||
                      (!sa.a_eq_e && sa.order_mode == 1 && c->split_mode == SPL_SPLIT_ON));
  if (split) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t B = spl::splat_batch_size(sa);
    // segments of about 1/16 of an SM's share of the entries, at least 4 batches
    int64_t L = ((int64_t)ne + (int64_t)nsm * 16 - 1) / ((int64_t)nsm * 16);
    L = std::max<int64_t>((L + B - 1) / B * B, 4 * B);
    L = std::min<int64_t>(L, 0x40000000);
    const int64_t nseg_max = ntiles + (int64_t)ne / L + 1;
    if ((st = ensure(c->seg_cnt, ntiles * 4 + 4)) || (st = ensure(c->seg_off, (ntiles + 1) * 8)) ||
        (st = ensure(c->scratch, spl::scan_scratch_bytes(ntiles + 1))) ||
        (st = ensure(c->seg_state, (size_t)nseg_max * T * T * 32)))
      return st;
    spl::SplatSegs sg;
    sg.seg_off = as<uint64_t>(c->seg_off);
    sg.ntiles = ntiles;
    sg.seg_len = (uint32_t)L;
    sg.partial = as<float4>(c->seg_state);
    // a front-to-back tile is split only when it dominates the frame (8x the
    // mean list): its segments lose early termination across segment bounds
    const int64_t split_min = sa.a_eq_e ? L : std::max<int64_t>(L, 8 * ((int64_t)ne / ntiles));
    spl::launch_seg_count(sa.tile_start, ntiles, (uint32_t)L,
                          (uint32_t)std::min<int64_t>(split_min, 0xffffffffLL),
                          as<uint32_t>(c->seg_cnt), s);
    spl::scan_counts(as<uint32_t>(c->seg_cnt), sa.tile_order, ntiles, as<uint64_t>(c->seg_off),
                     c->scratch.p, s, &launches);
    // the counts are consumed: the same words become the per-tile opaque flags
    sg.opaque = as<uint32_t>(c->seg_cnt);
    SPL_CK(cudaMemsetAsync(c->seg_cnt.p, 0, ntiles * 4, s));
    launches += 1 + spl::launch_splat_split(sa, sg, (uint32_t)std::min<int64_t>(nseg_max, 0x7fffffff), s);
  } else {
    launches += spl::launch_splat(sa, s);
  }
  SPL_CK(cudaGetLastError());
  c->last_splat = sa;
  cudaEventRecord(c->ev[5], s);

  // ---- outputs -------------------------------------------------------------------
  if (out->memspace == SPL_MEM_HOST)
    SPL_CK(cudaMemcpyAsync(out->pic, c->pic.p, (size_t)xres * yres * 12, cudaMemcpyDeviceToHost,
                           s));
  // remembered for the test hooks (full-form projection on demand)
  c->last_pc = pc;
  c->last_aos = aos_dev;
  c->last_soa = soa;
  if (writeback == SPL_WRITEBACK_FULL && n > 0) {
    // the reference's side effects: every particle projected and colourised,
    // the whole array stably sorted when a_eq_e is false
    if ((st = project_full(c, n, do_sort, &launches))) return st;
    const uint32_t *perm_all = nullptr;
    if (do_sort) {
      spl::radix_sort_pairs(as<uint32_t>(c->key), nullptr, as<uint32_t>(c->ktmp),
                            as<uint32_t>(c->vtmp), as<uint32_t>(c->key), as<uint32_t>(c->perm),
                            n, 0, 32, false, c->scratch.p, s, &launches, d_err, onesweep);
      perm_all = as<uint32_t>(c->perm);
    }
    if ((st = ensure(c->aos_out, n * 36))) return st;
    spl::launch_writeback_aos(as<float4>(c->pos), as<float4>(c->col), as<uint8_t>(c->active),
                              aos_dev ? aos_dev : (const void *)soa.type,
                              aos_dev ? 1 : (soa.type ? 2 : 0), perm_all, n, c->aos_out.p, s);
    ++launches;
    SPL_CK(cudaMemcpyAsync(p->aos, c->aos_out.p, n * 36,
                           p->memspace == SPL_MEM_DEVICE ? cudaMemcpyDeviceToDevice
                                                         : cudaMemcpyDeviceToHost,
                           s));
    c->has_order = false;  // the compact order buffers were reused
  } else {
    c->has_order = order != nullptr;
  }
  cudaEventRecord(c->ev[6], s);
  uint32_t words[3] = {0, 0, 0};  // error word, wide-particle count, FP64 fallbacks
  SPL_CK(cudaMemcpyAsync(words, d_err, 12, cudaMemcpyDeviceToHost, s));
  SPL_CK(cudaStreamSynchronize(s));
  SPL_CK(cudaGetLastError());
  const uint32_t err = words[0];
  if (err & 1u) return fail(SPL_ERR_INVALID, "particle type outside [0, ptypes)");
  if (err & 2u) return fail(SPL_ERR_TIMEOUT, "a look-back wait gave up");
  if (err & 8u) return fail(SPL_ERR_CAPACITY, "the compacted particle arrays overflowed");
  if (err & 16u)
    return fail(SPL_ERR_CAPACITY, "bin emission found more tiles than a particle's count");
  if (err & 32u)
    return fail(SPL_ERR_INTERNAL, "the activity screen kept a particle the projection culls");
  c->stats.n_fallback = words[2];
  c->stats.n_wide = words[1];

  c->n = n;
  c->na = na;
  c->ne = (int64_t)ne;
  c->ntiles = ntiles;
  c->last_T = T;
  c->writeback_done = writeback == SPL_WRITEBACK_FULL;
  spl_stats &S = c->stats;
  cudaEventElapsedTime(&S.h2d_ms, c->ev[0], c->ev[1]);
  cudaEventElapsedTime(&S.project_ms, c->ev[1], c->ev[2]);
  cudaEventElapsedTime(&S.sort_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&S.bin_ms, c->ev[3], c->ev[4]);
  cudaEventElapsedTime(&S.splat_ms, c->ev[4], c->ev[5]);
  cudaEventElapsedTime(&S.d2h_ms, c->ev[5], c->ev[6]);
  cudaEventElapsedTime(&S.total_ms, c->ev[0], c->ev[6]);
  S.n_entries = (int64_t)ne;
  S.n_tiles = ntiles;
  S.kernel_launches = launches;
  S.n_active = na;
  if (c->pf_in_use >= 0) cudaEventRecord(c->pf[c->pf_in_use].freed, s);
  return SPL_OK;
}

spl_status spl_prefetch(spl_context *c, const spl_particles *p) {
  if (!c || !p) return fail(SPL_ERR_INVALID, "null argument");
  if (p->memspace != SPL_MEM_HOST) return SPL_OK;  // device inputs are not copied
  if (p->n < 0 || p->n > 0xffffffffLL) return fail(SPL_ERR_INVALID, "particle count out of range");
  const int64_t n = p->n;
  if (p->layout == SPL_LAYOUT_AOS) {
    if (n > 0 && !p->aos) return fail(SPL_ERR_INVALID, "null AoS pointer");
  } else if (p->layout == SPL_LAYOUT_SOA) {
    if (n > 0 && (!p->x || !p->y || !p->z || !p->r || !p->I || !p->cr))
      return fail(SPL_ERR_INVALID, "null SoA pointer");
  } else {
    return fail(SPL_ERR_INVALID, "bad layout");
  }
  SPL_CK(cudaSetDevice(c->device));
  if (c->pf_len >= 2)
    return fail(SPL_ERR_INVALID, "spl_prefetch: two prefetches are already pending");
  int slot = -1;  // not queued, and not the inputs of the last render
  for (int k = 0; k < 3 && slot < 0; ++k)
    if (!c->pf[k].queued && k != c->pf_in_use) slot = k;
  if (slot < 0)
    return fail(SPL_ERR_INVALID, "spl_prefetch: two prefetches are already pending");
  if (!c->copy_stream) SPL_CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  spl_context::InSlot &q = c->pf[slot];
  if (!q.ready) SPL_CK(cudaEventCreateWithFlags(&q.ready, cudaEventDisableTiming));
  if (!q.freed) SPL_CK(cudaEventCreateWithFlags(&q.freed, cudaEventDisableTiming));
  spl_status st;
  SPL_CK(cudaStreamWaitEvent(c->copy_stream, q.freed, 0));
  cudaStream_t cs = c->copy_stream;
  if (p->layout == SPL_LAYOUT_AOS) {
    if ((st = ensure(q.aos, n * 36))) return st;
    if (n > 0) SPL_CK(cudaMemcpyAsync(q.aos.p, p->aos, n * 36, cudaMemcpyHostToDevice, cs));
  } else {
    const float *f[8] = {p->x, p->y, p->z, p->r, p->I, p->cr, p->cg, p->cb};
    for (int k = 0; k < 8; ++k) {
      if (!f[k]) continue;
      if ((st = ensure(q.soa[k], n * 4))) return st;
      if (n > 0) SPL_CK(cudaMemcpyAsync(q.soa[k].p, f[k], n * 4, cudaMemcpyHostToDevice, cs));
    }
    if (p->type) {
      if ((st = ensure(q.soa[8], n * 2))) return st;
      if (n > 0) SPL_CK(cudaMemcpyAsync(q.soa[8].p, p->type, n * 2, cudaMemcpyHostToDevice, cs));
    }
  }
  SPL_CK(cudaEventRecord(q.ready, cs));
  host_keys(p, q.host);
  q.n = n;
  q.layout = p->layout;
  q.queued = true;
  c->pf_fifo[c->pf_len++] = slot;
  return SPL_OK;
}

spl_status spl_context_set_split_tiles(spl_context *c, int mode) {
  if (!c) return fail(SPL_ERR_INVALID, "null ctx");
  if (mode != SPL_SPLIT_OFF && mode != SPL_SPLIT_ON && mode != SPL_SPLIT_ADDITIVE)
    return fail(SPL_ERR_INVALID, "spl_context_set_split_tiles: unknown mode " +
                                     std::to_string(mode));
  c->split_mode = mode;
  return SPL_OK;
}

spl_status spl_context_set_differentiable(spl_context *c, int enable) {
  if (!c) return fail(SPL_ERR_INVALID, "null ctx");
  c->differentiable = enable != 0;
  return SPL_OK;
}

spl_status spl_render_backward(spl_context *c, const spl_image *gp, spl_grads *g) {
  if (!c || !gp || !g || !gp->pic) return fail(SPL_ERR_INVALID, "null argument");
  if (c->last_T <= 0)
    return fail(SPL_ERR_INVALID, "spl_render_backward: no frame was rendered on this context");
  if (c->writeback_done)
    return fail(SPL_ERR_UNSUPPORTED,
                "spl_render_backward: the last frame wrote its particles back; render it "
                "with writeback none to differentiate it");
  if ((gp->memspace != SPL_MEM_HOST && gp->memspace != SPL_MEM_DEVICE) ||
      (g->memspace != SPL_MEM_HOST && g->memspace != SPL_MEM_DEVICE))
    return fail(SPL_ERR_INVALID, "spl_render_backward: bad memspace");
  if (!c->last_splat.a_eq_e && !c->last_splat.aux)
    return fail(SPL_ERR_INVALID,
                "spl_render_backward: the ordered frame was rendered without "
                "spl_context_set_differentiable(ctx, 1)");
  SPL_CK(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  const int64_t n = c->n, na = c->na;
  const spl::SplatArgs &f = c->last_splat;
  const size_t npix = (size_t)f.xres * f.yres * 3;
  spl_status st;
  float *outs[8] = {g->I, g->cr, g->cg, g->cb, g->x, g->y, g->z, g->r};
  float *dev[8];
  for (int k = 0; k < 8; ++k) {
    dev[k] = nullptr;
    if (!outs[k]) continue;
    if (g->memspace == SPL_MEM_DEVICE) {
      dev[k] = outs[k];
    } else {
      if ((st = ensure(c->gout[k], n * 4))) return st;
      dev[k] = as<float>(c->gout[k]);
    }
  }
  // split ordered tiles: (U, V) per segment and tile pixel, 32 B
  size_t seg_state_bytes = 16;
  if (!f.a_eq_e)
    seg_state_bytes = (size_t)(c->ntiles + c->ne / spl::adjoint_seg_len(f, c->ne) + 1) *
                      (size_t)(f.T * f.T) * 32;
  if ((st = ensure(c->gpos_c, na * 16)) || (st = ensure(c->gcol_c, na * 16)) ||
      (st = ensure(c->camsum, 5 * 8)) || (st = ensure(c->seg_cnt, c->ntiles * 4 + 4)) ||
      (st = ensure(c->seg_off, (c->ntiles + 1) * 8)) ||
      (st = ensure(c->seg_state, seg_state_bytes)) ||
      (st = ensure(c->scratch, spl::scan_scratch_bytes(c->ntiles + 1))))
    return st;
  const float *gpic_d = gp->pic;
  cudaEventRecord(c->ev[0], s);
  if (gp->memspace == SPL_MEM_HOST) {
    if ((st = ensure(c->gpic, npix * 4))) return st;
    SPL_CK(cudaMemcpyAsync(c->gpic.p, gp->pic, npix * 4, cudaMemcpyHostToDevice, s));
    gpic_d = as<float>(c->gpic);
  }
  SPL_CK(cudaMemsetAsync(c->camsum.p, 0, 5 * 8, s));
  for (int k = 0; k < 8; ++k)
    if (dev[k] && n > 0) SPL_CK(cudaMemsetAsync(dev[k], 0, n * 4, s));
  cudaEventRecord(c->ev[1], s);
  if (na > 0) {
    SPL_CK(cudaMemsetAsync(c->gpos_c.p, 0, na * 16, s));
    SPL_CK(cudaMemsetAsync(c->gcol_c.p, 0, na * 16, s));
    spl::AdjArgs aa;
    aa.f = f;
    aa.gpic = gpic_d;
    aa.gpos = as<float4>(c->gpos_c);
    aa.gcol = as<float4>(c->gcol_c);
    aa.n_entries = c->ne;
    aa.seg_cnt = as<uint32_t>(c->seg_cnt);
    aa.seg_off = as<uint64_t>(c->seg_off);
    aa.scan_scratch = c->scratch.p;
    aa.seg_state = as<float4>(c->seg_state);
    aa.seg_state_cap = c->seg_state.cap / 16;
    spl::launch_splat_adjoint(aa, s);
  }
  cudaEventRecord(c->ev[2], s);
  spl::ProjAdjArgs pa;
  pa.c = c->last_pc;
  pa.aos = c->last_aos;
  pa.soa = c->last_soa;
  pa.pos_c = as<float4>(c->pos_c);
  pa.idx_c = as<uint32_t>(c->idx_c);
  pa.gpos = as<float4>(c->gpos_c);
  pa.gcol = as<float4>(c->gcol_c);
  pa.na = na;
  pa.h2sigma = f.h2sigma;
  pa.gI = dev[0]; pa.gcr = dev[1]; pa.gcg = dev[2]; pa.gcb = dev[3];
  pa.gx = dev[4]; pa.gy = dev[5]; pa.gz = dev[6]; pa.gr = dev[7];
  pa.cam_sums = as<double>(c->camsum);
  spl::launch_project_adjoint(pa, s);
  SPL_CK(cudaGetLastError());
  cudaEventRecord(c->ev[3], s);
  if (g->memspace == SPL_MEM_HOST)
    for (int k = 0; k < 8; ++k)
      if (dev[k] && n > 0)
        SPL_CK(cudaMemcpyAsync(outs[k], dev[k], n * 4, cudaMemcpyDeviceToHost, s));
  double cs[5];
  SPL_CK(cudaMemcpyAsync(cs, c->camsum.p, 5 * 8, cudaMemcpyDeviceToHost, s));
  cudaEventRecord(c->ev[4], s);
  SPL_CK(cudaStreamSynchronize(s));
  SPL_CK(cudaGetLastError());
  // campos: cam = A*(p - campos) and, in perspective, xshift/yshift =
  // -xfac*A[0|1]*(centerpos - campos)
  const float *m = c->last_pc.mat;
  for (int j = 0; j < 3; ++j) {
    double v = -(m[j] * cs[0] + m[4 + j] * cs[1] + m[8 + j] * cs[2]);
    if (c->last_pc.projection) v += (double)c->last_pc.xfac * (m[j] * cs[3] + m[4 + j] * cs[4]);
    g->campos[j] = v;
  }
  spl_stats &S = c->stats;
  cudaEventElapsedTime(&S.bwd_splat_ms, c->ev[1], c->ev[2]);
  cudaEventElapsedTime(&S.bwd_project_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&S.bwd_total_ms, c->ev[0], c->ev[4]);
  if (c->pf_in_use >= 0) cudaEventRecord(c->pf[c->pf_in_use].freed, c->stream);
  return SPL_OK;
}

// ---- particle normalisation ---------------------------------------------------
void spl_rays_desc_defaults(spl_rays_desc *r) {
  if (!r) return;
  r->dome = 0;
  r->fov = 45.0;
  r->minrad_pix = 1.0;
}

// host_rendering_new (splotch/new_renderer.cc:522-641): particle pass, level
// sort, region-tree walk, leaf sort, per-level leaf rendering, dome mask.
spl_status spl_render_rays(spl_context *c, const spl_frame_desc *d, const spl_rays_desc *r,
                           const spl_particles *p, spl_image *out) {
  if (!c || !r) return fail(SPL_ERR_INVALID, "null argument");
  SPL_CK(cudaSetDevice(c->device));
  spl_status st = validate(d, p, out);
  if (st) return st;
  if (!d->a_eq_e)
    return fail(SPL_ERR_INVALID, "inconsistent: the ray-sphere renderer needs a_eq_e=true");
  cudaStream_t s = c->stream;
  const int64_t n = p->n;
  const int xres = d->xres, yres = d->yres;
  int launches = 0;
  // spl_render_backward and the debug getters describe a spl_render frame
  c->last_T = 0;
  c->has_order = false;
  c->pf_in_use = -1;

  spl::FrameSetup fs;
  if ((st = spl::frame_setup(d, 16, (c->debug_flags & 1) != 0, fs, false))) return st;
  spl::ProjConst pc = fs.pc;
  const int npal = fs.npal;

  // ---- projector, levels and region trees (kept while the geometry holds) --
  spl_context::RayKey key;
  std::memset(&key, 0, sizeof(key));  // compared byte for byte, padding included
  key.xres = xres;
  key.yres = yres;
  key.dome = r->dome ? 1 : 0;
  key.fov = r->fov;
  key.minrad_pix = r->minrad_pix;
  for (int a = 0; a < 3; ++a) {
    key.v[a] = d->campos[a];
    key.v[3 + a] = d->centerpos[a];
    key.v[6 + a] = d->lookat[a];
    key.v[9 + a] = d->sky[a];
  }
  const bool rebuild = !c->rays || std::memcmp(&key, &c->ray_key, sizeof(key)) != 0;
  if (rebuild) {
    delete c->rays;
    c->rays = new spl::RayFrame;
    if ((st = spl::rays_setup(d, r, *c->rays))) {
      delete c->rays;
      c->rays = nullptr;
      return st;
    }
    c->ray_key = key;
  }
  spl::RayFrame &F = *c->rays;
  spl::RayConst k = F.k;
  k.zmax = d->zmax;
  const int nlev = k.nlev;
  const int64_t nnodes = (int64_t)F.nodes.size(), nleaves = (int64_t)F.leaf_box.size();

  // ---- buffers ---------------------------------------------------------------
  size_t img_floats = 1;
  for (int L = 0; L + 1 < nlev; ++L)
    img_floats = std::max(img_floats, (size_t)k.lev[L].xdim * k.lev[L].ydim * 3);
  const size_t pic_bytes = (size_t)xres * yres * 3 * 4;
  if ((st = ensure(c->ray_rc, n * 32)) || (st = ensure(c->ray_cf, n * 16)) ||
      (st = ensure(c->ray_pod, n * 16)) || (st = ensure(c->ray_cov, n * 8)) ||
      (st = ensure(c->ray_code, n * 4)) || (st = ensure(c->ray_lev, (nlev + 3) * 4)) ||
      (st = ensure(c->ray_slots, n * 4 * spl::kRayWalkSlots)) ||
      (st = ensure(c->ray_rc2, n * 32)) || (st = ensure(c->ray_cf2, n * 16)) ||
      (st = ensure(c->ray_pod2, n * 16)) || (st = ensure(c->ray_cov2, n * 8)) ||
      (st = ensure(c->ray_clo, n * 16)) || (st = ensure(c->ray_clo2, n * 16)) ||
      (st = ensure(c->key, n * 4)) || (st = ensure(c->perm, n * 4)) ||
      (st = ensure(c->ktmp, n * 4)) || (st = ensure(c->vtmp, n * 4)) ||
      (st = ensure(c->count, n * 4)) || (st = ensure(c->off, (n + 1) * 8)) ||
      (st = ensure(c->small, 256)) || (st = ensure(c->ray_leaf_start, (nleaves + 1) * 4)) ||
      (st = ensure(c->ray_img[0], img_floats * 4)) || (st = ensure(c->ray_img[1], img_floats * 4)) ||
      (st = ensure(c->ray_jstop, (xres / 2 + 1) * 4)) ||
      (out->memspace == SPL_MEM_HOST && (st = ensure(c->pic, pic_bytes))) ||
      (st = ensure(c->pal_x, (npal + 1) * 8)) || (st = ensure(c->pal_rgb, (npal + 1) * 12)) ||
      (st = ensure(c->pal_thr, (npal + 1) * 4)) || (st = ensure(c->pal_xff, (npal + 1) * 8)) ||
      (st = ensure(c->pal_invff, (npal + 1) * 8)))
    return st;
  size_t scr = std::max(spl::scan_scratch_bytes(n + 1), spl::radix_scratch_bytes(n));
  if ((st = ensure(c->scratch, scr))) return st;
  if (rebuild) {
    if ((st = ensure(c->ray_nodes, nnodes * sizeof(spl::RayNode))) ||
        (st = ensure(c->ray_regs, nnodes * sizeof(spl::RayRegion))) ||
        (st = ensure(c->ray_box, nleaves * sizeof(ushort4))))
      return st;
    SPL_CK(cudaMemcpyAsync(c->ray_nodes.p, F.nodes.data(), nnodes * sizeof(spl::RayNode),
                           cudaMemcpyHostToDevice, s));
    SPL_CK(cudaMemcpyAsync(c->ray_regs.p, F.regs.data(), nnodes * sizeof(spl::RayRegion),
                           cudaMemcpyHostToDevice, s));
    SPL_CK(cudaMemcpyAsync(c->ray_box.p, F.leaf_box.data(), nleaves * sizeof(ushort4),
                           cudaMemcpyHostToDevice, s));
  }
  SPL_CK(cudaMemcpyAsync(c->pal_x.p, fs.pal_x.data(), (npal + 1) * 8, cudaMemcpyHostToDevice, s));
  SPL_CK(cudaMemcpyAsync(c->pal_rgb.p, fs.pal_rgb.data(), (npal + 1) * 12, cudaMemcpyHostToDevice,
                         s));
  SPL_CK(cudaMemcpyAsync(c->pal_thr.p, fs.thr.data(), (npal + 1) * 4, cudaMemcpyHostToDevice, s));
  SPL_CK(cudaMemcpyAsync(c->pal_xff.p, fs.xff.data(), (npal + 1) * 8, cudaMemcpyHostToDevice, s));
  SPL_CK(cudaMemcpyAsync(c->pal_invff.p, fs.invff.data(), (npal + 1) * 8, cudaMemcpyHostToDevice,
                         s));
  SPL_CK(cudaStreamSynchronize(s));  // the host tables live in fs and F
  pc.pal_x = as<double>(c->pal_x);
  pc.pal_rgb = as<float>(c->pal_rgb);
  pc.pal_thr = as<float>(c->pal_thr);
  pc.pal_xff = as<float2>(c->pal_xff);
  pc.pal_invff = as<float2>(c->pal_invff);
  uint32_t *d_err = as<uint32_t>(c->small);
  SPL_CK(cudaMemsetAsync(d_err, 0, 32, s));

  cudaEventRecord(c->ev[0], s);
  // ---- inputs ------------------------------------------------------------------
  const void *aos_dev = nullptr;
  spl::SoAIn soa{p->x, p->y, p->z, p->r, p->I, p->cr, p->cg, p->cb, p->type};
  if (p->layout == SPL_LAYOUT_AOS) {
    if (p->memspace == SPL_MEM_HOST) {
      if ((st = ensure(c->aos_in, n * 36))) return st;
      if (n > 0) SPL_CK(cudaMemcpyAsync(c->aos_in.p, p->aos, n * 36, cudaMemcpyHostToDevice, s));
      aos_dev = c->aos_in.p;
    } else {
      aos_dev = p->aos;
    }
  } else if (p->memspace == SPL_MEM_HOST) {
    const float **f[8] = {&soa.x, &soa.y, &soa.z, &soa.r, &soa.I, &soa.cr, &soa.cg, &soa.cb};
    for (int a = 0; a < 8; ++a) {
      if (!*f[a]) continue;
      if ((st = ensure(c->soa_in[a], n * 4))) return st;
      if (n > 0) SPL_CK(cudaMemcpyAsync(c->soa_in[a].p, *f[a], n * 4, cudaMemcpyHostToDevice, s));
      *f[a] = as<float>(c->soa_in[a]);
    }
    if (p->type) {
      if ((st = ensure(c->soa_in[8], n * 2))) return st;
      if (n > 0) SPL_CK(cudaMemcpyAsync(c->soa_in[8].p, p->type, n * 2, cudaMemcpyHostToDevice, s));
      soa.type = as<uint16_t>(c->soa_in[8]);
    }
  }
  cudaEventRecord(c->ev[1], s);

  // ---- particle pass, then the particles sorted by level and direction -------
  spl::RayParts rp{as<double4_16a>(c->ray_rc), as<float4>(c->ray_cf), as<float4>(c->ray_clo),
                   as<float4>(c->ray_pod), as<float2>(c->ray_cov), as<uint32_t>(c->ray_code),
                   d_err};
  spl::launch_rays_prep(aos_dev, &soa, n, pc, k, rp, s);
  ++launches;
  cudaEventRecord(c->ev[2], s);
  uint32_t *key_s = as<uint32_t>(c->key), *order = as<uint32_t>(c->perm);
  uint32_t *lev_start = as<uint32_t>(c->ray_lev);
  if (n > 0) {
    spl::radix_sort_pairs(rp.key, nullptr, as<uint32_t>(c->ktmp), as<uint32_t>(c->vtmp), key_s,
                          order, n, 0, 32, true, c->scratch.p, s, &launches, d_err,
                          (c->debug_flags & 2) == 0);
  }
  spl::RayParts rs{as<double4_16a>(c->ray_rc2), as<float4>(c->ray_cf2), as<float4>(c->ray_clo2),
                   as<float4>(c->ray_pod2), as<float2>(c->ray_cov2), key_s, d_err};
  spl::launch_rays_sorted(key_s, order, n, nlev, lev_start, rp, rs, s);
  launches += 2;
  cudaEventRecord(c->ev[3], s);

  // ---- region-tree walk: (leaf, particle) pairs, grouped by leaf (stable) -----
  const spl::RayNode *d_nodes = as<spl::RayNode>(c->ray_nodes);
  const spl::RayRegion *d_regs = as<spl::RayRegion>(c->ray_regs);
  spl::launch_rays_walk(false, k, d_nodes, d_regs, key_s, n, rs, as<uint32_t>(c->count),
                        as<uint32_t>(c->ray_slots), nullptr, nullptr, nullptr, s);
  ++launches;
  spl::scan_counts(as<uint32_t>(c->count), nullptr, n, as<uint64_t>(c->off), c->scratch.p, s,
                   &launches);
  uint64_t ne64 = 0;
  std::vector<uint32_t> hlev(nlev + 3, 0);
  SPL_CK(cudaMemcpyAsync(&ne64, as<uint64_t>(c->off) + n, 8, cudaMemcpyDeviceToHost, s));
  SPL_CK(cudaMemcpyAsync(hlev.data(), lev_start, (nlev + 3) * 4, cudaMemcpyDeviceToHost, s));
  SPL_CK(cudaStreamSynchronize(s));
  if (ne64 > 0xffffffffULL) return fail(SPL_ERR_CAPACITY, "more than 2^32 leaf-list entries");
  const int64_t ne = (int64_t)ne64;
  if ((st = ensure(c->tkey, ne * 4)) || (st = ensure(c->tval, ne * 4)) ||
      (st = ensure(c->tkey2, ne * 4)) || (st = ensure(c->tval2, ne * 4)) ||
      (st = ensure(c->tkey_s, ne * 4)) || (st = ensure(c->tval_s, ne * 4)) ||
      (st = ensure(c->scratch, std::max(scr, spl::radix_scratch_bytes(ne)))))
    return st;
  spl::launch_rays_walk(true, k, d_nodes, d_regs, key_s, n, rs, as<uint32_t>(c->count),
                        as<uint32_t>(c->ray_slots), as<uint64_t>(c->off), as<uint32_t>(c->tkey),
                        as<uint32_t>(c->tval), s);
  ++launches;
  if (ne > 0)
    spl::radix_sort_pairs(as<uint32_t>(c->tkey), as<uint32_t>(c->tval), as<uint32_t>(c->tkey2),
                          as<uint32_t>(c->tval2), as<uint32_t>(c->tkey_s), as<uint32_t>(c->tval_s),
                          ne, 0, std::max(1, spl::bits_for(nleaves)), true, c->scratch.p, s,
                          &launches, d_err,
                          (c->debug_flags & 2) == 0);
  spl::launch_tile_ranges(as<uint32_t>(c->tkey_s), ne, nleaves, as<uint32_t>(c->ray_leaf_start),
                          s);
  ++launches;
  // leaf lists cut into segments of kRaySegLen entries, one warp each
  const int64_t max_items = nleaves + ne / spl::kRaySegLen + 1;
  if ((st = ensure(c->ray_kd, sizeof(spl::RayConst))) ||
      (st = ensure(c->ray_segcnt, nleaves * 4)) || (st = ensure(c->ray_segoff, (nleaves + 1) * 8)) ||
      (st = ensure(c->ray_items, max_items * 4)) ||
      (st = ensure(c->ray_partial, (size_t)max_items * spl::kRayLeafPixels * 3 * 4)) ||
      (st = ensure(c->scratch, std::max(c->scratch.cap, spl::scan_scratch_bytes(nleaves + 1)))))
    return st;
  SPL_CK(cudaMemcpyAsync(c->ray_kd.p, &k, sizeof(k), cudaMemcpyHostToDevice, s));
  spl::launch_rays_segments(as<uint32_t>(c->ray_leaf_start), nleaves, as<uint32_t>(c->ray_segcnt),
                            s);
  spl::scan_counts(as<uint32_t>(c->ray_segcnt), nullptr, nleaves, as<uint64_t>(c->ray_segoff),
                   c->scratch.p, s, &launches);
  spl::launch_rays_items(as<uint64_t>(c->ray_segoff), nleaves, as<uint32_t>(c->ray_items), s);
  launches += 2;
  cudaEventRecord(c->ev[4], s);

  // ---- the pyramid, coarsest level first -----------------------------------------
  float *final_pic = out->memspace == SPL_MEM_HOST ? as<float>(c->pic) : out->pic;
  spl::RayLeafArgs la{};
  la.kd = as<spl::RayConst>(c->ray_kd);
  la.leaf_box = as<ushort4>(c->ray_box);
  la.leaf_start = as<uint32_t>(c->ray_leaf_start);
  la.seg_off = as<uint64_t>(c->ray_segoff);
  la.item_leaf = as<uint32_t>(c->ray_items);
  la.partial = as<float>(c->ray_partial);
  la.vals = as<uint32_t>(c->tval_s);
  la.lev_start = lev_start;
  for (int L = 0; L < nlev; ++L) {
    la.out = L == nlev - 1 ? final_pic : as<float>(c->ray_img[L & 1]);
    la.coarse = L > 0 ? as<float>(c->ray_img[(L - 1) & 1]) : nullptr;
    la.cdim_y = L > 0 ? k.lev[L - 1].ydim : 0;
    spl::launch_rays_leaves(k, L, rs, la, s);
    launches += 2;
  }
  if (k.dome) {
    spl::launch_rays_dome_mask(final_pic, xres, as<int>(c->ray_jstop), s);
    launches += 2;
  }
  cudaEventRecord(c->ev[5], s);
  if (out->memspace == SPL_MEM_HOST)
    SPL_CK(cudaMemcpyAsync(out->pic, final_pic, pic_bytes, cudaMemcpyDeviceToHost, s));
  cudaEventRecord(c->ev[6], s);
  uint32_t err = 0;
  SPL_CK(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, s));
  SPL_CK(cudaStreamSynchronize(s));
  SPL_CK(cudaGetLastError());
  if (err & 1u) return fail(SPL_ERR_INVALID, "particle type outside [0, ptypes)");
  if (err & 2u) return fail(SPL_ERR_TIMEOUT, "a look-back wait gave up");
  if (err & 32u) return fail(SPL_ERR_INVALID, "a particle fell in two pyramid levels");

  spl_stats &S = c->stats;
  S = spl_stats{};
  cudaEventElapsedTime(&S.h2d_ms, c->ev[0], c->ev[1]);
  cudaEventElapsedTime(&S.project_ms, c->ev[1], c->ev[2]);
  cudaEventElapsedTime(&S.sort_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&S.bin_ms, c->ev[3], c->ev[4]);
  cudaEventElapsedTime(&S.splat_ms, c->ev[4], c->ev[5]);
  cudaEventElapsedTime(&S.d2h_ms, c->ev[5], c->ev[6]);
  cudaEventElapsedTime(&S.total_ms, c->ev[0], c->ev[6]);
  S.n_active = hlev[nlev + 1];  // spheres rendered: level grids and around the camera
  S.n_entries = ne;
  S.n_tiles = nleaves;
  S.kernel_launches = launches;
  return SPL_OK;
}


spl_status spl_particle_normalize(spl_context *c, const spl_normalize_desc *d,
                                  spl_particles *p, spl_normalize_result *res) {
  if (!c || !d || !p || !res) return fail(SPL_ERR_INVALID, "null argument");
  if (d->ptypes < 1 || d->ptypes > SPL_MAX_TYPES)
    return fail(SPL_ERR_INVALID, "ptypes must be in [1,8]");
  const int64_t n = p->n;
  if (n < 0 || n > 0xffffffffLL) return fail(SPL_ERR_INVALID, "particle count out of range");
  bool any_vec = false;
  for (int t = 0; t < d->ptypes; ++t) any_vec = any_vec || d->color_is_vector[t];
  if (p->layout == SPL_LAYOUT_SOA) {
    if (n > 0 && (!p->r || !p->I || !p->cr || (any_vec && (!p->cg || !p->cb))))
      return fail(SPL_ERR_INVALID, "null SoA pointer");
  } else if (p->layout != SPL_LAYOUT_AOS || (n > 0 && !p->aos)) {
    return fail(SPL_ERR_INVALID, "bad particle view");
  }
  SPL_CK(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  spl_status st;
  spl::NormView v{};
  // device view of the particles (host inputs are staged and copied back); the
  // view's fields are declared read-only for rendering, normalisation writes
  // them in place
  float *soa_host[5] = {const_cast<float *>(p->I), const_cast<float *>(p->cr),
                        const_cast<float *>(p->cg), const_cast<float *>(p->cb),
                        const_cast<float *>(p->r)};
  if (p->layout == SPL_LAYOUT_AOS) {
    if (p->memspace == SPL_MEM_HOST) {
      if ((st = ensure(c->aos_in, n * 36))) return st;
      SPL_CK(cudaMemcpyAsync(c->aos_in.p, p->aos, n * 36, cudaMemcpyHostToDevice, s));
      v.aos = c->aos_in.p;
    } else {
      v.aos = p->aos;
    }
  } else if (p->memspace == SPL_MEM_HOST) {
    float **dst[5] = {&v.I, &v.cr, &v.cg, &v.cb, const_cast<float **>(&v.r)};
    for (int k = 0; k < 5; ++k) {
      if (!soa_host[k]) continue;
      if ((st = ensure(c->soa_in[k], n * 4))) return st;
      SPL_CK(cudaMemcpyAsync(c->soa_in[k].p, soa_host[k], n * 4, cudaMemcpyHostToDevice, s));
      *dst[k] = as<float>(c->soa_in[k]);
    }
    if (p->type) {
      if ((st = ensure(c->soa_in[8], n * 2))) return st;
      SPL_CK(cudaMemcpyAsync(c->soa_in[8].p, p->type, n * 2, cudaMemcpyHostToDevice, s));
      v.type = as<uint16_t>(c->soa_in[8]);
    }
  } else {
    v.I = soa_host[0];
    v.cr = soa_host[1];
    v.cg = soa_host[2];
    v.cb = soa_host[3];
    v.r = p->r;
    v.type = p->type;
  }
  spl::NormConst nc{};
  nc.ptypes = d->ptypes;
  for (int t = 0; t < d->ptypes; ++t) {
    nc.intensity_log[t] = d->intensity_log[t] != 0;
    nc.color_log[t] = d->color_log[t] != 0;
    nc.color_asinh[t] = d->color_asinh[t] != 0;
    nc.color_is_vector[t] = d->color_is_vector[t] != 0;
  }
  // pass 1: transforms and per-type ranges
  int h_stats[SPL_MAXT * 6];
  spl::norm_stats_init(h_stats);
  if ((st = ensure(c->small, 256)) || (st = ensure(c->post_tab, sizeof h_stats))) return st;
  uint32_t *d_err = as<uint32_t>(c->small);
  SPL_CK(cudaMemsetAsync(d_err, 0, 4, s));
  SPL_CK(cudaMemcpyAsync(c->post_tab.p, h_stats, sizeof h_stats, cudaMemcpyHostToDevice, s));
  spl::launch_norm_collect(v, n, nc, as<int>(c->post_tab), d_err, s);
  uint32_t err = 0;
  SPL_CK(cudaMemcpyAsync(h_stats, c->post_tab.p, sizeof h_stats, cudaMemcpyDeviceToHost, s));
  SPL_CK(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, s));
  SPL_CK(cudaStreamSynchronize(s));
  if (err & 1u) return fail(SPL_ERR_INVALID, "particle type outside [0, ptypes)");
  // overrides (scenemaker.cc:222-232) and pass 2: normAndClamp
  spl::NormRanges rg{};
  for (int t = 0; t < d->ptypes; ++t) {
    const int *st6 = h_stats + 6 * t;
    res->size_min[t] = spl::norm_stat_value(st6[0]);
    res->size_max[t] = spl::norm_stat_value(st6[1]);
    float imin = spl::norm_stat_value(st6[2]), imax = spl::norm_stat_value(st6[3]);
    float cmin = spl::norm_stat_value(st6[4]), cmax = spl::norm_stat_value(st6[5]);
    res->range_min[t] = cmin;
    res->range_max[t] = cmax;
    if (d->has_intensity_min[t]) imin = d->intensity_min[t];
    if (d->has_intensity_max[t]) imax = d->intensity_max[t];
    if (d->has_color_min[t]) cmin = d->color_min[t];
    if (d->has_color_max[t]) cmax = d->color_max[t];
    res->clamp_min[t] = cmin;
    res->clamp_max[t] = cmax;
    res->intensity_min[t] = imin;
    res->intensity_max[t] = imax;
    rg.imin[t] = imin;
    rg.imax[t] = imax;
    rg.cmin[t] = cmin;
    rg.cmax[t] = cmax;
  }
  spl::launch_norm_clamp(v, n, nc, rg, s);
  if (p->memspace == SPL_MEM_HOST && n > 0) {
    if (p->layout == SPL_LAYOUT_AOS) {
      SPL_CK(cudaMemcpyAsync(p->aos, v.aos, n * 36, cudaMemcpyDeviceToHost, s));
    } else {
      float *dev[4] = {v.I, v.cr, v.cg, v.cb};
      for (int k = 0; k < 4; ++k)
        if (soa_host[k] && dev[k])
          SPL_CK(cudaMemcpyAsync(soa_host[k], dev[k], n * 4, cudaMemcpyDeviceToHost, s));
    }
  }
  SPL_CK(cudaStreamSynchronize(s));
  SPL_CK(cudaGetLastError());
  return SPL_OK;
}

// ---- post-processing and image output ---------------------------------------

void spl_post_desc_defaults(spl_post_desc *p) {
  if (!p) return;
  p->a_eq_e = 0;
  p->gamma = 1.0;
  p->brightness = 0.0;
  p->contrast = 1.0;
  p->colorbar = 0;
}

namespace {

// linearMap<COLOUR>::getVal_const (cxxsupport/linear_map.h:71-84) on the host:
// lower_bound in double, interpolated per channel in double, rounded to float
// per term, summed in float.
void palette_host(int n, const double *x, const float *rgb, double v, float out[3]) {
  int idx;
  if (n == 1 || v <= x[0]) {
    idx = 0;
  } else if (v >= x[n - 1]) {
    idx = n - 1;
  } else {
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = lo + (hi - lo) / 2;
      if (x[mid] < v) lo = mid + 1; else hi = mid;
    }
    idx = lo > 0 ? lo - 1 : 0;
    if (idx > n - 2) idx = n - 2;
    const double frac = (v - x[idx]) / (x[idx + 1] - x[idx]);
    for (int c = 0; c < 3; ++c) {
      const float a = (float)(rgb[3 * idx + c] * (1. - frac));
      const float b = (float)(rgb[3 * (idx + 1) + c] * frac);
      out[c] = a + b;
    }
    return;
  }
  for (int c = 0; c < 3; ++c) out[c] = rgb[3 * idx + c];
}

}  // namespace

spl_status spl_postprocess(spl_context *c, const spl_frame_desc *d, const spl_post_desc *p,
                           spl_image *img) {
  if (!c || !d || !p || !img || !img->pic) return fail(SPL_ERR_INVALID, "null argument");
  if (d->xres <= 0 || d->yres <= 0) return fail(SPL_ERR_INVALID, "xres/yres out of range");
  SPL_CK(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  const int xres = d->xres, yres = d->yres;
  const size_t nf = (size_t)xres * yres * 3;
  spl_status st;
  float *pic = img->pic;
  if (img->memspace == SPL_MEM_HOST) {
    if ((st = ensure(c->post_img, nf * 4))) return st;
    SPL_CK(cudaMemcpyAsync(c->post_img.p, img->pic, nf * 4, cudaMemcpyHostToDevice, s));
    pic = as<float>(c->post_img);
  }
  const bool adjust = p->gamma != 1.0 || p->brightness != 0.0 || p->contrast != 1.0;
  std::vector<float> tabs(2048);
  float expfac = 0.f, taylor = 0.f;
  if (p->a_eq_e) {
    spl::exptable_tables(-20.f, tabs.data(), tabs.data() + 1024, &expfac, &taylor);
    if ((st = ensure(c->post_tab, 2048 * 4))) return st;
    SPL_CK(cudaMemcpyAsync(c->post_tab.p, tabs.data(), 2048 * 4, cudaMemcpyHostToDevice, s));
  }
  spl::launch_post(pic, (int64_t)nf, p->a_eq_e != 0, adjust, expfac, taylor,
                   as<float>(c->post_tab), as<float>(c->post_tab) + 1024, p->gamma,
                   p->brightness, p->contrast, s);
  std::vector<float> bars;
  std::vector<int> rows;
  if (p->colorbar) {
    int offset = 0;
    for (int t = 0; t < d->ptypes && t < SPL_MAX_TYPES; ++t) {
      if (d->color_is_vector[t]) continue;  // "adding no color bar for type t"
      if (d->pal_n[t] < 1 || !d->pal_x[t] || !d->pal_rgb[t])
        return fail(SPL_ERR_INVALID, "trying to access an empty map");
      const size_t o = bars.size();
      bars.resize(o + (size_t)xres * 3);
      for (int x = 0; x < xres; ++x)
        palette_host(d->pal_n[t], d->pal_x[t], d->pal_rgb[t], x / (double)xres,
                     bars.data() + o + 3 * (size_t)x);
      rows.push_back(yres - offset - 1);
      offset += 10;
    }
    if (!rows.empty()) {
      const size_t nb = bars.size() * 4, nr = rows.size() * 4;
      if ((st = ensure(c->post_bar, nb + nr + 16))) return st;
      SPL_CK(cudaMemcpyAsync(c->post_bar.p, bars.data(), nb, cudaMemcpyHostToDevice, s));
      int *drows = reinterpret_cast<int *>(static_cast<uint8_t *>(c->post_bar.p) + nb);
      SPL_CK(cudaMemcpyAsync(drows, rows.data(), nr, cudaMemcpyHostToDevice, s));
      spl::launch_colorbar(pic, xres, yres, as<float>(c->post_bar), drows, (int)rows.size(), s);
    }
  }
  if (img->memspace == SPL_MEM_HOST)
    SPL_CK(cudaMemcpyAsync(img->pic, pic, nf * 4, cudaMemcpyDeviceToHost, s));
  SPL_CK(cudaStreamSynchronize(s));  // the host tables above die here
  SPL_CK(cudaGetLastError());
  return SPL_OK;
}

namespace {

// One row of the run-length TGA body (cxxsupport/ls_image.cc:206-286): runs of
// equal pixels and of pairwise-different pixels, each cut into chunks of 128.
void rle_row(const uint8_t *bgr, int xres, std::vector<uint8_t> &buf) {
  auto same = [&](int a, int b) {
    return bgr[3 * a] == bgr[3 * b] && bgr[3 * a + 1] == bgr[3 * b + 1] &&
           bgr[3 * a + 2] == bgr[3 * b + 2];
  };
  int xs = 0;
  while (xs < xres) {
    int xe;
    bool equal;
    if (xs == xres - 1) {
      xe = xres;
      equal = false;
    } else if (same(xs + 1, xs)) {
      xe = xs + 2;
      while (xe < xres && same(xe, xs)) ++xe;
      equal = true;
    } else {
      xe = xs + 2;
      while (xe < xres && !same(xe, xe - 1)) ++xe;
      equal = false;
    }
    for (int cb = xs; cb < xe; cb += 128) {
      const int csz = std::min(xe - cb, 128);
      if (equal) {
        buf.push_back((uint8_t)(csz - 1 + 128));
        buf.insert(buf.end(), bgr + 3 * xs, bgr + 3 * xs + 3);
      } else {
        buf.push_back((uint8_t)(csz - 1));
        buf.insert(buf.end(), bgr + 3 * cb, bgr + 3 * (cb + csz));
      }
    }
    xs = xe;
  }
}

spl_status encode_image(spl_context *c, const spl_image *img, int xres, int yres, int pictype,
                        std::vector<uint8_t> &file) {
  if (!img || !img->pic) return fail(SPL_ERR_INVALID, "null image");
  if (xres <= 0 || yres <= 0) return fail(SPL_ERR_INVALID, "xres/yres out of range");
  if (pictype == 1) return fail(SPL_ERR_UNSUPPORTED, "ASCII PPM no longer supported");
  if (pictype != 0 && pictype != 2 && pictype != 3)
    return fail(SPL_ERR_INVALID, "No valid image file type given ...");
  SPL_CK(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  const size_t np = (size_t)xres * yres;
  spl_status st;
  const float *pic = img->pic;
  if (img->memspace == SPL_MEM_HOST) {
    if ((st = ensure(c->post_img, np * 12))) return st;
    SPL_CK(cudaMemcpyAsync(c->post_img.p, img->pic, np * 12, cudaMemcpyHostToDevice, s));
    pic = as<float>(c->post_img);
  }
  if ((st = ensure(c->post_bytes, np * 3))) return st;
  spl::launch_encode(pic, xres, yres, pictype != 2, as<uint8_t>(c->post_bytes), s);
  std::vector<uint8_t> body(np * 3);
  SPL_CK(cudaMemcpyAsync(body.data(), c->post_bytes.p, np * 3, cudaMemcpyDeviceToHost, s));
  SPL_CK(cudaStreamSynchronize(s));
  SPL_CK(cudaGetLastError());
  file.clear();
  if (pictype == 2) {
    char hdr[64];
    const int n = std::snprintf(hdr, sizeof hdr, "P6\n%d\n%d\n255\n", xres, yres);
    file.insert(file.end(), hdr, hdr + n);
    file.insert(file.end(), body.begin(), body.end());
    return SPL_OK;
  }
  const uint8_t hdr[18] = {0, 0, (uint8_t)(pictype == 0 ? 2 : 10), 0, 0, 0, 0, 0, 0, 0, 0, 0,
                           (uint8_t)(xres % 256), (uint8_t)(xres / 256),
                           (uint8_t)(yres % 256), (uint8_t)(yres / 256), 24, 32};
  file.insert(file.end(), hdr, hdr + 18);
  if (pictype == 0) {
    file.insert(file.end(), body.begin(), body.end());
  } else {
    for (int y = 0; y < yres; ++y) rle_row(body.data() + (size_t)y * xres * 3, xres, file);
  }
  return SPL_OK;
}

}  // namespace

spl_status spl_image_encode(spl_context *c, const spl_image *img, int xres, int yres,
                            int pictype, uint8_t *out, int64_t cap, int64_t *len) {
  if (!c || !len) return fail(SPL_ERR_INVALID, "null argument");
  std::vector<uint8_t> file;
  spl_status st = encode_image(c, img, xres, yres, pictype, file);
  if (st) return st;
  *len = (int64_t)file.size();
  if (out && cap > 0) std::memcpy(out, file.data(), std::min<size_t>((size_t)cap, file.size()));
  return SPL_OK;
}

spl_status spl_write_image(spl_context *c, const spl_image *img, int xres, int yres,
                           int pictype, const char *path) {
  if (!c || !path) return fail(SPL_ERR_INVALID, "null argument");
  std::vector<uint8_t> file;
  spl_status st = encode_image(c, img, xres, yres, pictype, file);
  if (st) return st;
  FILE *f = std::fopen(path, "wb");
  if (!f) return fail(SPL_ERR_INVALID, std::string("could not create file '") + path + "'");
  const size_t w = std::fwrite(file.data(), 1, file.size(), f);
  const int cl = std::fclose(f);
  if (w != file.size() || cl != 0)
    return fail(SPL_ERR_INVALID, std::string("error writing output file '") + path + "'");
  return SPL_OK;
}

spl_status spl_debug_get_projected(spl_context *c, void *aos_out, int64_t n) {
  if (!c || !aos_out || n != c->n) return fail(SPL_ERR_INVALID, "bad arguments");
  SPL_CK(cudaSetDevice(c->device));
  spl_status st;
  int launches = 0;
  if ((st = project_full(c, n, false, &launches))) return st;
  if ((st = ensure(c->aos_out, n * 36))) return st;
  const void *tsrc = c->last_aos ? c->last_aos : (const void *)c->last_soa.type;
  const int kind = c->last_aos ? 1 : (c->last_soa.type ? 2 : 0);
  spl::launch_writeback_aos(as<float4>(c->pos), as<float4>(c->col), as<uint8_t>(c->active),
                            tsrc, kind, nullptr, n, c->aos_out.p, c->stream);
  SPL_CK(cudaMemcpyAsync(aos_out, c->aos_out.p, n * 36, cudaMemcpyDeviceToHost, c->stream));
  SPL_CK(cudaStreamSynchronize(c->stream));
  return SPL_OK;
}

int spl_splat_config_count(void) { return spl::splat_config_count(); }

int spl_splat_config_valid(int cfg, int tile_size) {
  return (cfg >= 0 && cfg < spl::splat_config_count() && tile_size >= 1 && tile_size <= 64 &&
          spl::splat_config_valid(cfg, tile_size))
             ? 1
             : 0;
}

spl_status spl_debug_set_options(spl_context *c, int flags) {
  if (!c) return fail(SPL_ERR_INVALID, "null ctx");
  c->debug_flags = flags;
  return SPL_OK;
}

spl_status spl_debug_fail_alloc(int64_t nth) {
  if (nth < 0) return fail(SPL_ERR_INVALID, "spl_debug_fail_alloc: nth must be >= 0");
  g_alloc_countdown.store(nth);
  return SPL_OK;
}

spl_status spl_debug_count_fragments(spl_context *c, int64_t *frags_out) {
  if (!c || !frags_out) return fail(SPL_ERR_INVALID, "bad arguments");
  SPL_CK(cudaSetDevice(c->device));
  spl_status st;
  if ((st = ensure(c->small, 256))) return st;
  unsigned long long *d = reinterpret_cast<unsigned long long *>(as<uint8_t>(c->small) + 64);
  spl::launch_count_fragments(c->last_splat, d, c->stream);
  unsigned long long h = 0;
  SPL_CK(cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, c->stream));
  SPL_CK(cudaStreamSynchronize(c->stream));
  *frags_out = (int64_t)h;
  return SPL_OK;
}

spl_status spl_debug_get_order(spl_context *c, uint32_t *order_out, int64_t cap,
                               int64_t *n_out) {
  if (!c || !n_out) return fail(SPL_ERR_INVALID, "bad arguments");
  SPL_CK(cudaSetDevice(c->device));
  *n_out = c->na;
  if (c->na == 0) return SPL_OK;
  if (!order_out || cap < c->na) return fail(SPL_ERR_CAPACITY, "order buffer too small");
  if (c->writeback_done) return fail(SPL_ERR_UNSUPPORTED, "order not kept after a writeback");
  std::vector<uint32_t> idx(c->na), perm;
  SPL_CK(cudaMemcpy(idx.data(), c->idx_c.p, c->na * 4, cudaMemcpyDeviceToHost));
  if (c->has_order) {
    perm.resize(c->na);
    SPL_CK(cudaMemcpy(perm.data(), c->perm.p, c->na * 4, cudaMemcpyDeviceToHost));
  }
  for (int64_t s = 0; s < c->na; ++s) order_out[s] = idx[c->has_order ? perm[s] : s];
  return SPL_OK;
}

spl_status spl_debug_get_bins(spl_context *c, int64_t *tile_start_out, int64_t ntp1,
                              uint32_t *entries_out, int64_t cap) {
  if (!c || !tile_start_out || ntp1 != c->ntiles + 1)
    return fail(SPL_ERR_INVALID, "bad arguments (need ntiles+1 tile starts)");
  if (cap < c->ne || (c->ne > 0 && !entries_out))
    return fail(SPL_ERR_CAPACITY, "entries buffer too small: need " + std::to_string(c->ne));
  SPL_CK(cudaSetDevice(c->device));
  std::vector<uint32_t> ts(ntp1);
  SPL_CK(cudaMemcpy(ts.data(), c->tile_start.p, ntp1 * 4, cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < ntp1; ++i) tile_start_out[i] = ts[i];
  if (c->ne > 0) {
    // entries hold ranks among active particles; report particle indices
    std::vector<uint32_t> idx(c->na);
    SPL_CK(cudaMemcpy(idx.data(), c->idx_c.p, c->na * 4, cudaMemcpyDeviceToHost));
    SPL_CK(cudaMemcpy(entries_out, c->tval_s.p, c->ne * 4, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < c->ne; ++i) entries_out[i] = idx[entries_out[i]];
  }
  return SPL_OK;
}

}  // extern "C"
