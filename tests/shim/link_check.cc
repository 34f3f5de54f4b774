// link_check.cc -- a minimal Splotch-side caller of host_rendering(), linked
// with host_rendering_gb300.cc in place of splotch/splotch_host.cc.  It shows
// that the shim is a drop-in at the link level: built against the Splotch
// headers, resolved against libsplgpu.so.  Prints "rendered" after a frame, or
// the PlanckError text when no GPU is present (exit code 3).  With the
// argument "rays" the frame goes through the ray-sphere renderer
// (new_renderer=true), after which the particle vector is empty.
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "splotch/splotch_host.h"

int main(int argc, char **argv) {
  const bool rays = argc > 1 && std::string(argv[1]) == "rays";
  std::map<std::string, std::string> kv = {
      {"xres", "48"}, {"yres", "40"}, {"fov", "45"}, {"tile_size_cpu", "16"}};
  if (rays) kv["new_renderer"] = "T";
  paramfile params(kv, false);
  render_context rc;
  rc.campos = vec3(0, 0, 100);
  rc.centerpos = rc.campos;
  rc.lookat = vec3(0, 0, 0);
  rc.sky = vec3(0, 1, 0);
  rc.amap.resize(1);
  rc.amap[0].addVal(0.0, COLOUR(0, 0, 1));
  rc.amap[0].addVal(1.0, COLOUR(1, 1, 1));
  rc.amap[0].sortMap();
  rc.xres = 48;
  rc.yres = 40;
  rc.pic.alloc(48, 40);
  rc.b_brightness = 1;
  std::vector<particle_sim> p;
  for (int i = 0; i < 64; ++i)
    p.push_back(particle_sim(COLOUR(i / 64.f, 0, 0), (i % 8) - 4.f, (i / 8) - 4.f, 0.f, 0.6f,
                             1.f, 0, false));
  rc.npart = rc.npart_all = p.size();
  try {
    host_rendering(params, p, rc);
  } catch (PlanckError &e) {
    std::printf("planck: %s\n", e.what());
    return 3;
  }
  if (rays) {
    std::printf("rendered rays, %d particles left, pic[24][20].b = %g\n", (int)p.size(),
                rc.pic[24][20].b);
    return p.empty() ? 0 : 4;
  }
  int active = 0;
  for (const auto &q : p) active += q.active;
  std::printf("rendered %d active, pic[24][20].b = %g\n", active, rc.pic[24][20].b);
  return 0;
}
