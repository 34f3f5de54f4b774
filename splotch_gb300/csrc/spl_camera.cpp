// spl_camera.cpp -- host-side frame set-up of the C ABI: reference defaults
// and the camera quantities of particle_project (splotch/splotch_host.cc:62-110).
//
// Compiled with -ffp-contract=off: the camera matrix, xfac and the screen
// shifts must come out bit-identical to the reference's, because every
// projected coordinate depends on them.
#include <cmath>
#include <cstring>

#include "../../include/splotch_gb300.h"

namespace {

// cxxsupport/lsconstants.h:35,51
const double kPi = 3.141592653589793238462643383279502884197;
const double kDegr2rad = kPi / 180.0;

struct V3 {
  double x, y, z;
};
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 normed(V3 a) {  // vec3_t::Norm (cxxsupport/vec3.h:72-83)
  const double l = 1.0 / std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return {a.x * l, a.y * l, a.z * l};
}
double length(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
V3 cross(V3 a, V3 b) {  // crossprod (cxxsupport/vec3.h:129-131)
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// TRANSMAT (kernel/transform.h:33-67): 3 rows of 4 floats.
struct M34 {
  float e[3][4];
};

// TRANSMAT::Inverse (kernel/transform.cxx:64-112)
bool inverse(const M34 &a, M34 &t) {
  const float(*e)[4] = a.e;
  t.e[0][0] = e[1][1] * e[2][2] - e[2][1] * e[1][2];
  t.e[0][1] = e[0][1] * e[2][2] - e[2][1] * e[0][2];
  t.e[0][2] = e[0][1] * e[1][2] - e[1][1] * e[0][2];
  t.e[1][0] = e[1][0] * e[2][2] - e[2][0] * e[1][2];
  t.e[1][1] = e[0][0] * e[2][2] - e[2][0] * e[0][2];
  t.e[1][2] = e[0][0] * e[1][2] - e[1][0] * e[0][2];
  t.e[2][0] = e[1][0] * e[2][1] - e[2][0] * e[1][1];
  t.e[2][1] = e[0][0] * e[2][1] - e[2][0] * e[0][1];
  t.e[2][2] = e[0][0] * e[1][1] - e[1][0] * e[0][1];
  const float det = e[0][0] * t.e[0][0] - e[1][0] * t.e[0][1] + e[2][0] * t.e[0][2];
  double d = det;
  if (!(std::fabs(d) > 1e-10)) return false;  // "degenerate matrix"
  d = 1. / d;
  t.e[0][0] = (float)(t.e[0][0] * d);
  t.e[2][0] = (float)(t.e[2][0] * d);
  t.e[1][1] = (float)(t.e[1][1] * d);
  t.e[0][2] = (float)(t.e[0][2] * d);
  t.e[2][2] = (float)(t.e[2][2] * d);
  d = -d;
  t.e[1][0] = (float)(t.e[1][0] * d);
  t.e[0][1] = (float)(t.e[0][1] * d);
  t.e[2][1] = (float)(t.e[2][1] * d);
  t.e[1][2] = (float)(t.e[1][2] * d);
  for (int j = 0; j < 3; ++j)
    t.e[j][3] = -(t.e[j][0] * e[0][3] + t.e[j][1] * e[1][3] + t.e[j][2] * e[2][3]);
  return true;
}

// TRANSMAT::operator*= (kernel/transform.cxx:50-62)
void mul_inplace(M34 &self, const M34 &b) {
  const M34 a = self;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 3; ++j)
      self.e[j][i] = a.e[0][i] * b.e[j][0] + a.e[1][i] * b.e[j][1] + a.e[2][i] * b.e[j][2];
  for (int j = 0; j < 3; ++j) self.e[j][3] += b.e[j][3];
}

}  // namespace

extern "C" void spl_frame_desc_defaults(spl_frame_desc *d) {
  std::memset(d, 0, sizeof(*d));
  d->xres = 800;
  d->yres = 800;
  d->fov = 45.f;
  d->zmin = 0.f;
  d->zmax = 1.e23f;
  d->minrad_pix = 1.f;
  d->projection = 1;
  d->ptypes = 1;
  for (int t = 0; t < SPL_MAX_TYPES; ++t) {
    d->smooth_factor[t] = 1.f;
    d->brightness[t] = 1.f;
  }
  d->b_brightness = 1.f;
  d->a_eq_e = 1;
  d->gray_absorption = 0.2f;
  d->sort_type = 1;
  d->tile_size = 50;
  d->sky[1] = 1.0;
  d->order_mode = SPL_ORDER_FRONT_TO_BACK;
  d->ftb_epsilon = 1e-9f;
  d->ftb_relative = 1e-5f;
  d->splat_config = -1;
}

extern "C" spl_status spl_camera_setup(const spl_frame_desc *d, spl_camera *cam) {
  if (!d || !cam) return SPL_ERR_INVALID;
  const int xres = d->xres, yres = d->yres;
  cam->ycorr = .5f * (yres - xres);
  cam->res2 = 0.5f * xres;
  cam->fovfct = (float)std::tan((double)(d->fov * 0.5f) * kDegr2rad);

  const V3 campos{d->campos[0], d->campos[1], d->campos[2]};
  const V3 lookat{d->lookat[0], d->lookat[1], d->lookat[2]};
  const V3 centerpos{d->centerpos[0], d->centerpos[1], d->centerpos[2]};
  const V3 sky = normed(V3{d->sky[0], d->sky[1], d->sky[2]});
  const V3 zaxis = normed(sub(centerpos, lookat));
  const V3 xaxis = normed(cross(sky, zaxis));
  const V3 yaxis = cross(zaxis, xaxis);

  // TRANSMAT's constructor stores its arguments transposed
  // (kernel/transform.cxx:28-48): row j = (xaxis[j], yaxis[j], zaxis[j], 0).
  M34 gen;
  gen.e[0][0] = (float)xaxis.x; gen.e[1][0] = (float)xaxis.y; gen.e[2][0] = (float)xaxis.z;
  gen.e[0][1] = (float)yaxis.x; gen.e[1][1] = (float)yaxis.y; gen.e[2][1] = (float)yaxis.z;
  gen.e[0][2] = (float)zaxis.x; gen.e[1][2] = (float)zaxis.y; gen.e[2][2] = (float)zaxis.z;
  gen.e[0][3] = gen.e[1][3] = gen.e[2][3] = 0.f;
  M34 rot;  // Make_General_Transform + Invert: the matrix becomes gen^-1
  if (!inverse(gen, rot)) return SPL_ERR_INVALID;
  M34 t2;  // Make_Translation_Transform(-campos), then Add_Transform(rot)
  std::memset(&t2, 0, sizeof(t2));
  t2.e[0][0] = t2.e[1][1] = t2.e[2][2] = 1.f;
  t2.e[0][3] = (float)(-campos.x);
  t2.e[1][3] = (float)(-campos.y);
  t2.e[2][3] = (float)(-campos.z);
  mul_inplace(t2, rot);
  std::memcpy(cam->mat, t2.e, sizeof(cam->mat));

  const float *p = cam->mat;  // TRANSFORM::TransPoint (kernel/transform.cxx:212-219)
  const double tcx = centerpos.x * p[0] + centerpos.y * p[1] + centerpos.z * p[2] + p[3];
  const double tcy = centerpos.x * p[4] + centerpos.y * p[5] + centerpos.z * p[6] + p[7];
  const float dist = (float)length(sub(centerpos, lookat));
  cam->xfac = cam->res2 / (cam->fovfct * dist);
  cam->xshift = -cam->xfac * tcx;
  cam->yshift = -cam->xfac * tcy;
  return SPL_OK;
}
