// spl_host.h -- host-side helpers shared by the C-ABI translation units
// (spl_api.cu, spl_batch.cu).
#pragma once

#include <string>
#include <vector>

#include "../../include/splotch_gb300.h"
#include "spl_internal.cuh"

namespace spl {

// Sets the message of spl_last_error_string() and returns code.
spl_status host_fail(spl_status code, const std::string &msg);

// Argument checks of spl_render (frame keys, particle view, image view).
spl_status validate_frame(const spl_frame_desc *d, const spl_particles *p, const spl_image *o);

// Bits needed to represent 0..v-1.
int bits_for(int64_t v);

// The CUDA device of a context.
int context_device(const spl_context *c);

// Everything a frame's kernels need that the host derives from its keys:
// projection constants (device pointers left null), tiling at tile size T,
// and the palette tables -- exact knots and the float-float acceleration
// tables -- concatenated over the particle types at pc.pal_off[t].
struct FrameSetup {
  ProjConst pc;
  Tiling g;
  int64_t ntiles = 0;
  bool do_sort = false;
  int npal = 0;
  std::vector<double> pal_x;
  std::vector<float> pal_rgb, thr;
  std::vector<float2> xff, invff;
};
// camera false: the main path's camera (spl_camera_setup) is not needed and
// not checked (the ray-sphere renderer has its own projector).
spl_status frame_setup(const spl_frame_desc *d, int T, bool exact_fp64, FrameSetup &fs,
                       bool camera = true);

// The ray-sphere renderer's frame on the host: projector, pyramid levels and
// every level's region tree (nodes and their reduceList constants, leaf
// regions), in the reference's double arithmetic.
struct RayFrame {
  RayConst k;
  std::vector<RayNode> nodes;
  std::vector<RayRegion> regs;
  std::vector<ushort4> leaf_box;
};
spl_status rays_setup(const spl_frame_desc *d, const spl_rays_desc *r, RayFrame &f);

}  // namespace spl
