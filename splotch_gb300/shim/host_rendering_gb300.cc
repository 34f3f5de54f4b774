// host_rendering_gb300.cc -- drop-in replacement for Splotch's host renderer.
//
// Defines the same symbol as splotch/splotch_host.cc:711,
//     void host_rendering(paramfile&, std::vector<particle_sim>&, render_context&)
// (declared at splotch/splotch_host.h:43) and runs the whole frame -- project,
// colourise, depth sort, binning, splat -- through libsplgpu.so's C ABI
// (include/splotch_gb300.h).  It is compiled inside the Splotch tree against the
// Splotch headers and linked instead of splotch_host.o (and new_renderer.o).
//
// Behaviour kept from the reference:
//   * the same paramfile keys with the same defaults (find() inserts them);
//   * rc.pic is overwritten (x-major arr2<COLOUR>);
//   * the particle vector is modified in place -- projected x,y,z,r,I,
//     colourised e, active flags, and the z-sorted order when a_eq_e=false
//     (sorted stably: equal depths keep their original order);
//   * errors raise PlanckError through planck_fail;
//   * new_renderer=true runs the ray-sphere renderer (spl_render_rays) and
//     empties the particle vector, as host_rendering_new does.
// GPU-only keys (all optional): gpu_device (0), gpu_writeback (true),
// gpu_order ("ftb" | "btf"; default ftb), gpu_ftb_epsilon (1e-9), gpu_ftb_relative
// (1e-5), gpu_splat_config (-1).
#include <string>
#include <vector>

#include "splotch/splotch_host.h"
#include "splotch_gb300.h"

namespace {

spl_context *gpu_context(int device) {
  static spl_context *ctx = nullptr;
  static int ctx_device = -1;
  if (ctx && ctx_device != device) {
    spl_context_destroy(ctx);
    ctx = nullptr;
  }
  if (!ctx) {
    if (spl_context_create(&ctx, device) != SPL_OK)
      planck_fail(std::string("GB300 renderer: ") + spl_last_error_string());
    ctx_device = device;
  }
  return ctx;
}

// Camera vectors and b_brightness of the render context.
void copy_context(const render_context &rc, spl_frame_desc &d) {
  d.b_brightness = rc.b_brightness;
  const vec3 *cams[4] = {&rc.campos, &rc.lookat, &rc.sky, &rc.centerpos};
  double *dst[4] = {d.campos, d.lookat, d.sky, d.centerpos};
  for (int k = 0; k < 4; ++k) {
    dst[k][0] = cams[k]->x;
    dst[k][1] = cams[k]->y;
    dst[k][2] = cams[k]->z;
  }
}

// palettes: rc.amap[t] knots (get_colourmaps, splotch/splotchutils.cc:63-125)
void copy_palettes(render_context &rc, spl_frame_desc &d, std::vector<std::vector<double>> &px,
                   std::vector<std::vector<float>> &prgb) {
  px.assign(d.ptypes, {});
  prgb.assign(d.ptypes, {});
  for (int t = 0; t < d.ptypes; ++t) {
    if (d.color_is_vector[t]) continue;
    if (t >= (int)rc.amap.size() || rc.amap[t].size() == 0)
      planck_fail("trying to access an empty map");
    COLOURMAP &m = rc.amap[t];
    for (size_t k = 0; k < m.size(); ++k) {
      px[t].push_back(m.getX(k));
      const COLOUR c = m.getY(k);
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
void host_rendering_rays(paramfile &params, std::vector<particle_sim> &particles,
                         render_context &rc) {
  spl_frame_desc d;
  spl_frame_desc_defaults(&d);
  spl_rays_desc r;
  spl_rays_desc_defaults(&r);
  d.zmax = params.find<float32>("zmax", 1.e23);
  d.ptypes = params.find<int>("ptypes", 1);  // particle_colorize (splotch_host.cc:256-265)
  if (d.ptypes < 1 || d.ptypes > SPL_MAX_TYPES) planck_fail("ptypes must be in [1,8]");
  for (int t = 0; t < d.ptypes; ++t) {
    d.brightness[t] = params.find<float32>("brightness" + dataToString(t), 1.f);
    d.color_is_vector[t] = params.find<bool>("color_is_vector" + dataToString(t), false);
  }
  d.a_eq_e = params.find<bool>("a_eq_e", true);
  r.dome = params.find<bool>("dome", false);
  d.xres = params.find<int>("xres", 800);
  if (r.dome) {
    d.yres = d.xres;
  } else {
    d.yres = params.find<int>("yres", d.xres);
    r.fov = params.find<double>("fov", 45);
  }
  r.minrad_pix = params.find<double>("minrad_pix", 1.);
  const int device = params.find<int>("gpu_device", 0);
  copy_context(rc, d);
  std::vector<std::vector<double>> px;
  std::vector<std::vector<float>> prgb;
  copy_palettes(rc, d, px, prgb);
  if ((int)rc.pic.size1() != d.xres || (int)rc.pic.size2() != d.yres) {
    if (r.dome) planck_fail("inconsistency");  // new_renderer.cc:593-594
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
  tstack_push("GB300 rendering");
  const spl_status st = spl_render_rays(gpu_context(device), &d, &r, &p, &img);
  tstack_pop("GB300 rendering");
  if (st != SPL_OK) planck_fail(std::string("GB300 renderer: ") + spl_last_error_string());
  particles.resize(0);
  particles.shrink_to_fit();
}

}  // namespace

void host_rendering(paramfile &params, std::vector<particle_sim> &particles,
                    render_context &rc) {
  if (params.find<bool>("new_renderer", false)) {
    host_rendering_rays(params, particles, rc);
    return;
  }
  if (params.find<bool>("bbox", false)) checkbbox(particles, params);

  spl_frame_desc d;
  spl_frame_desc_defaults(&d);
  // splotch_host.cc:62-109
  d.xres = params.find<int>("xres", 800);
  d.yres = params.find<int>("yres", d.xres);
  d.zmax = params.find<float32>("zmax", 1.e23);
  d.zmin = params.find<float32>("zmin", 0.0);
  d.fov = params.find<float32>("fov", 45);
  d.ptypes = params.find<int>("ptypes", 1);
  if (d.ptypes < 1 || d.ptypes > SPL_MAX_TYPES) planck_fail("ptypes must be in [1,8]");
  for (int t = 0; t < d.ptypes; ++t)
    d.smooth_factor[t] = params.find<float32>("smooth_factor" + dataToString(t), 1.f);
  d.projection = params.find<bool>("projection", true);
  d.minrad_pix = params.find<float32>("minrad_pix", 1.);
  // splotch_host.cc:256-265
  for (int t = 0; t < d.ptypes; ++t) {
    d.brightness[t] = params.find<float32>("brightness" + dataToString(t), 1.f);
    d.color_is_vector[t] = params.find<bool>("color_is_vector" + dataToString(t), false);
  }
  // splotch_host.cc:806, 812, 823-825
  d.a_eq_e = params.find<bool>("a_eq_e", true);
  d.sort_type = params.find<int>("sort_type", 1);
  d.gray_absorption = params.find<float32>("gray_absorption", 0.2);
  d.tile_size = params.find<float32>("tile_size_cpu", 50);
  // GPU-only knobs
  const int device = params.find<int>("gpu_device", 0);
  const bool writeback = params.find<bool>("gpu_writeback", true);
  if (params.param_present("gpu_order"))
    d.order_mode = params.find<std::string>("gpu_order") == "ftb" ? SPL_ORDER_FRONT_TO_BACK
                                                                 : SPL_ORDER_BACK_TO_FRONT;
  if (params.param_present("gpu_ftb_epsilon"))
    d.ftb_epsilon = params.find<float32>("gpu_ftb_epsilon");
  if (params.param_present("gpu_ftb_relative"))
    d.ftb_relative = params.find<float32>("gpu_ftb_relative");
  if (params.param_present("gpu_splat_config"))
    d.splat_config = params.find<int>("gpu_splat_config");

  copy_context(rc, d);
  std::vector<std::vector<double>> px;
  std::vector<std::vector<float>> prgb;
  copy_palettes(rc, d, px, prgb);

  if ((int)rc.pic.size1() != d.xres || (int)rc.pic.size2() != d.yres)
    rc.pic.alloc(d.xres, d.yres);
  static_assert(sizeof(particle_sim) == 36, "particle_sim layout");
  static_assert(sizeof(COLOUR) == 12, "COLOUR layout");

  spl_particles p = {};
  p.n = (int64_t)rc.npart;
  p.layout = SPL_LAYOUT_AOS;
  p.memspace = SPL_MEM_HOST;
  p.aos = p.n ? &particles[0] : nullptr;
  spl_image img = {};
  img.pic = reinterpret_cast<float *>(&rc.pic[0][0]);
  img.memspace = SPL_MEM_HOST;

  tstack_push("GB300 rendering");
  const spl_status st = spl_render(gpu_context(device), &d, &p, &img,
                                   writeback ? SPL_WRITEBACK_FULL : SPL_WRITEBACK_NONE);
  tstack_pop("GB300 rendering");
  if (st != SPL_OK) planck_fail(std::string("GB300 renderer: ") + spl_last_error_string());

  const float r_th = params.find<float>("rth", 0.0);  // splotch_host.cc:769-775
  if (r_th != 0.0 && writeback) checkrth(r_th, rc.npart, particles, params);
}
