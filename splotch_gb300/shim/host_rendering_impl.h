// host_rendering_impl.h -- the logic of the host_rendering() drop-in, written
// once over the caller's types so that it builds both inside the Splotch tree
// (host_rendering_gb300.cc, with Splotch's paramfile, render_context and
// particle_sim) and without it.
//
// Env supplies the types and the few Splotch services the renderer calls:
//   Env::Params    find<T>(key, default) inserting the default like
//                  paramfile::find, find<T>(key), param_present(key)
//   Env::Particle  the 36-byte particle_sim record
//   Env::Context   render_context: campos, lookat, sky, centerpos (x, y, z),
//                  b_brightness, npart, amap[t] (size, getX, getY -> r, g, b),
//                  pic (size1, size2, alloc, pic[0][0])
//   Env::fail(msg)                         planck_fail (throws)
//   Env::timer_push(name), timer_pop(name) tstack
//   Env::checkbbox(particles, params), Env::checkrth(r_th, npart, particles,
//   params)                                splotchutils.cc helpers
//
// Behaviour kept from the reference (splotch/splotch_host.cc:711-834):
//   * the same paramfile keys with the same defaults (find() inserts them);
//   * rc.pic is overwritten (x-major arr2<COLOUR>);
//   * the particle vector is modified in place -- projected x,y,z,r,I,
//     colourised e, active flags, and the z-sorted order when a_eq_e=false
//     (sorted stably: equal depths keep their original order);
//   * errors go through planck_fail;
//   * new_renderer=true runs the ray-sphere renderer (spl_render_rays) and
//     empties the particle vector, as host_rendering_new does
//     (splotch_host.cc:714-723, new_renderer.cc:584).
// GPU-only keys (all optional): gpu_device (0), gpu_writeback (true),
// gpu_order ("ftb" | "btf"; default ftb), gpu_ftb_epsilon (1e-9),
// gpu_ftb_relative (1e-5), gpu_splat_config (-1).
#pragma once

#include <string>
#include <vector>

#include "splotch_gb300.h"

namespace spl_shim {

template <class Env>
spl_context *gpu_context(int device) {
  static spl_context *ctx = nullptr;
  static int ctx_device = -1;
  if (ctx && ctx_device != device) {
    spl_context_destroy(ctx);
    ctx = nullptr;
  }
  if (!ctx) {
    if (spl_context_create(&ctx, device) != SPL_OK)
      Env::fail(std::string("GB300 renderer: ") + spl_last_error_string());
    ctx_device = device;
  }
  return ctx;
}

template <class V>
void put3(double *dst, const V &v) {
  dst[0] = v.x;
  dst[1] = v.y;
  dst[2] = v.z;
}

// Camera vectors and b_brightness of the render context.
template <class Env>
void copy_context(const typename Env::Context &rc, spl_frame_desc &d) {
  d.b_brightness = rc.b_brightness;
  put3(d.campos, rc.campos);
  put3(d.lookat, rc.lookat);
  put3(d.sky, rc.sky);
  put3(d.centerpos, rc.centerpos);
}

// palettes: rc.amap[t] knots (get_colourmaps, splotch/splotchutils.cc:63-125)
template <class Env>
void copy_palettes(typename Env::Context &rc, spl_frame_desc &d,
                   std::vector<std::vector<double>> &px, std::vector<std::vector<float>> &prgb) {
  px.assign(d.ptypes, {});
  prgb.assign(d.ptypes, {});
  for (int t = 0; t < d.ptypes; ++t) {
    if (d.color_is_vector[t]) continue;
    if (t >= (int)rc.amap.size() || rc.amap[t].size() == 0)
      Env::fail("trying to access an empty map");
    auto &m = rc.amap[t];
    for (size_t k = 0; k < m.size(); ++k) {
      px[t].push_back(m.getX(k));
      const auto c = m.getY(k);
      prgb[t].push_back(c.r);
      prgb[t].push_back(c.g);
      prgb[t].push_back(c.b);
    }
    d.pal_n[t] = (int)px[t].size();
    d.pal_x[t] = px[t].data();
    d.pal_rgb[t] = prgb[t].data();
  }
}

// new_renderer=true (splotch_host.cc:714-723): host_rendering_new
// (splotch/new_renderer.cc:522-641) through spl_render_rays, reading the keys
// that renderer reads, and emptying the particle vector afterwards as it does.
template <class Env>
void host_rendering_rays(typename Env::Params &params,
                         std::vector<typename Env::Particle> &particles,
                         typename Env::Context &rc) {
  spl_frame_desc d;
  spl_frame_desc_defaults(&d);
  spl_rays_desc r;
  spl_rays_desc_defaults(&r);
  d.zmax = params.template find<float>("zmax", 1.e23f);
  d.ptypes = params.template find<int>("ptypes", 1);  // particle_colorize (:256-265)
  if (d.ptypes < 1 || d.ptypes > SPL_MAX_TYPES) Env::fail("ptypes must be in [1,8]");
  for (int t = 0; t < d.ptypes; ++t) {
    d.brightness[t] = params.template find<float>("brightness" + std::to_string(t), 1.f);
    d.color_is_vector[t] =
        params.template find<bool>("color_is_vector" + std::to_string(t), false);
  }
  d.a_eq_e = params.template find<bool>("a_eq_e", true);
  r.dome = params.template find<bool>("dome", false);
  d.xres = params.template find<int>("xres", 800);
  if (r.dome) {
    d.yres = d.xres;
  } else {
    d.yres = params.template find<int>("yres", d.xres);
    r.fov = params.template find<double>("fov", 45);
  }
  r.minrad_pix = params.template find<double>("minrad_pix", 1.);
  const int device = params.template find<int>("gpu_device", 0);
  copy_context<Env>(rc, d);
  std::vector<std::vector<double>> px;
  std::vector<std::vector<float>> prgb;
  copy_palettes<Env>(rc, d, px, prgb);
  if ((int)rc.pic.size1() != d.xres || (int)rc.pic.size2() != d.yres) {
    if (r.dome) Env::fail("inconsistency");  // new_renderer.cc:593-594
    rc.pic.alloc(d.xres, d.yres);
  }
  spl_particles p = {};
  p.n = (int64_t)particles.size();
  p.layout = SPL_LAYOUT_AOS;
  p.memspace = SPL_MEM_HOST;
  p.aos = p.n ? &particles[0] : nullptr;
  spl_image img = {};
  img.pic = reinterpret_cast<float *>(&rc.pic[0][0]);
  img.memspace = SPL_MEM_HOST;
  Env::timer_push("GB300 rendering");
  const spl_status st = spl_render_rays(gpu_context<Env>(device), &d, &r, &p, &img);
  Env::timer_pop("GB300 rendering");
  if (st != SPL_OK) Env::fail(std::string("GB300 renderer: ") + spl_last_error_string());
  particles.resize(0);
  particles.shrink_to_fit();
}

template <class Env>
void host_rendering(typename Env::Params &params, std::vector<typename Env::Particle> &particles,
                    typename Env::Context &rc) {
  static_assert(sizeof(typename Env::Particle) == 36, "particle_sim layout");
  if (params.template find<bool>("new_renderer", false)) {
    host_rendering_rays<Env>(params, particles, rc);
    return;
  }
  if (params.template find<bool>("bbox", false)) Env::checkbbox(particles, params);

  spl_frame_desc d;
  spl_frame_desc_defaults(&d);
  // splotch_host.cc:62-109
  d.xres = params.template find<int>("xres", 800);
  d.yres = params.template find<int>("yres", d.xres);
  d.zmax = params.template find<float>("zmax", 1.e23f);
  d.zmin = params.template find<float>("zmin", 0.f);
  d.fov = params.template find<float>("fov", 45.f);
  d.ptypes = params.template find<int>("ptypes", 1);
  if (d.ptypes < 1 || d.ptypes > SPL_MAX_TYPES) Env::fail("ptypes must be in [1,8]");
  for (int t = 0; t < d.ptypes; ++t)
    d.smooth_factor[t] = params.template find<float>("smooth_factor" + std::to_string(t), 1.f);
  d.projection = params.template find<bool>("projection", true);
  d.minrad_pix = params.template find<float>("minrad_pix", 1.f);
  // splotch_host.cc:256-265
  for (int t = 0; t < d.ptypes; ++t) {
    d.brightness[t] = params.template find<float>("brightness" + std::to_string(t), 1.f);
    d.color_is_vector[t] =
        params.template find<bool>("color_is_vector" + std::to_string(t), false);
  }
  // splotch_host.cc:806, 812, 823-825
  d.a_eq_e = params.template find<bool>("a_eq_e", true);
  d.sort_type = params.template find<int>("sort_type", 1);
  d.gray_absorption = params.template find<float>("gray_absorption", 0.2f);
  d.tile_size = (int)params.template find<float>("tile_size_cpu", 50.f);
  // GPU-only knobs
  const int device = params.template find<int>("gpu_device", 0);
  const bool writeback = params.template find<bool>("gpu_writeback", true);
  if (params.param_present("gpu_order"))
    d.order_mode = params.template find<std::string>("gpu_order") == "btf"
                       ? SPL_ORDER_BACK_TO_FRONT
                       : SPL_ORDER_FRONT_TO_BACK;
  if (params.param_present("gpu_ftb_epsilon"))
    d.ftb_epsilon = params.template find<float>("gpu_ftb_epsilon");
  if (params.param_present("gpu_ftb_relative"))
    d.ftb_relative = params.template find<float>("gpu_ftb_relative");
  if (params.param_present("gpu_splat_config"))
    d.splat_config = params.template find<int>("gpu_splat_config");

  copy_context<Env>(rc, d);
  std::vector<std::vector<double>> px;
  std::vector<std::vector<float>> prgb;
  copy_palettes<Env>(rc, d, px, prgb);

  if ((int)rc.pic.size1() != d.xres || (int)rc.pic.size2() != d.yres)
    rc.pic.alloc(d.xres, d.yres);

  spl_particles p = {};
  p.n = (int64_t)rc.npart;
  p.layout = SPL_LAYOUT_AOS;
  p.memspace = SPL_MEM_HOST;
  p.aos = p.n ? &particles[0] : nullptr;
  spl_image img = {};
  img.pic = reinterpret_cast<float *>(&rc.pic[0][0]);
  img.memspace = SPL_MEM_HOST;

  Env::timer_push("GB300 rendering");
  const spl_status st = spl_render(gpu_context<Env>(device), &d, &p, &img,
                                   writeback ? SPL_WRITEBACK_FULL : SPL_WRITEBACK_NONE);
  Env::timer_pop("GB300 rendering");
  if (st != SPL_OK) Env::fail(std::string("GB300 renderer: ") + spl_last_error_string());

  const float r_th = params.template find<float>("rth", 0.f);  // splotch_host.cc:769-775
  if (r_th != 0.f && writeback) Env::checkrth(r_th, rc.npart, particles, params);
}

}  // namespace spl_shim
