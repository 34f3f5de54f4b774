// host_rendering_gb300.cc -- drop-in replacement for Splotch's host renderer.
//
// Defines the same symbol as splotch/splotch_host.cc:711,
//     void host_rendering(paramfile&, std::vector<particle_sim>&, render_context&)
// (declared at splotch/splotch_host.h:43) and runs the whole frame -- project,
// colourise, depth sort, binning, splat -- through libsplgpu.so's C ABI
// (include/splotch_gb300.h).  It is compiled inside the Splotch tree against the
// Splotch headers and linked instead of splotch_host.o (and new_renderer.o).
//
// The renderer's logic (keys, defaults, side effects, errors) is
// host_rendering_impl.h; this file binds it to Splotch's types and services:
// paramfile, render_context, particle_sim, planck_fail, tstack, and the
// checkbbox / checkrth helpers of splotch/splotchutils.h:260-261.
#include <string>
#include <vector>

#include "splotch/splotch_host.h"
#include "host_rendering_impl.h"

namespace {

struct SplotchEnv {
  using Params = paramfile;
  using Particle = particle_sim;
  using Context = render_context;
  [[noreturn]] static void fail(const std::string &msg) { planck_fail(msg); }  // throws
  static void timer_push(const char *name) { tstack_push(name); }
  static void timer_pop(const char *name) { tstack_pop(name); }
  static void checkbbox(std::vector<particle_sim> &p, paramfile &params) {
    ::checkbbox(p, params);
  }
  static void checkrth(float r_th, int npart, std::vector<particle_sim> &p,
                       paramfile &params) {
    ::checkrth(r_th, npart, p, params);
  }
};

static_assert(sizeof(COLOUR) == 12, "COLOUR layout");

}  // namespace

void host_rendering(paramfile &params, std::vector<particle_sim> &particles,
                    render_context &rc) {
  spl_shim::host_rendering<SplotchEnv>(params, particles, rc);
}
