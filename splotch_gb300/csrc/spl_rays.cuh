// spl_rays.cuh -- device helpers of the ray-sphere renderer
// (host_rendering_new, splotch/new_renderer.cc:522-641), shared by the
// particle pass (spl_project.cu) and the walk / leaf kernels (spl_rays.cu).
//
// Every decision the reference makes in double -- the screen and region
// culls (reduceList) and the sphere-vs-ray test -- is made here with the
// same double operations in the same order, none of them fused, so that the
// same particles reach the same pixels.  Where a float computation with a
// proven error bound already decides a test, the double one is skipped.
#pragma once

#include "spl_internal.cuh"

namespace spl {

constexpr double kRayHalfPi = 1.570796326794896619231321691639751442099;

__device__ __forceinline__ double ddot3(const double a[3], const double b[3]) {
  return dadd(dadd(dmul(a[0], b[0]), dmul(a[1], b[1])), dmul(a[2], b[2]));
}

// One particle as the region tests see it: c, r in double (the reference's
// values), the float copies, and for the dome the zenith terms of
// new_renderer.cc:203-211.
struct RayPart {
  double c[3], r;
  float cf[3], rf;
  double zdot, th_hi, th_lo;
  bool th_ready;  // th_hi, th_lo computed (on first use)
};

__device__ __forceinline__ RayPart ray_part(const RayConst &k, double4_16a rc, float4 cf) {
  RayPart p;
  p.c[0] = rc.x;
  p.c[1] = rc.y;
  p.c[2] = rc.z;
  p.r = rc.w;
  p.cf[0] = cf.x;
  p.cf[1] = cf.y;
  p.cf[2] = cf.z;
  p.rf = cf.w;
  p.zdot = p.th_hi = p.th_lo = 0.0;
  p.th_ready = false;
  if (k.dome) p.zdot = ddot3(k.zen, p.c);
  return p;
}

// The angle of c from the zenith plus and minus the sphere's angular
// half-width (new_renderer.cc:207-209), computed when a theta check first
// needs them.
__device__ __forceinline__ void ray_part_theta(const RayConst &k, RayPart &p) {
  const double cx = dsub(dmul(k.zen[1], p.c[2]), dmul(k.zen[2], p.c[1]));
  const double cy = dsub(dmul(k.zen[2], p.c[0]), dmul(k.zen[0], p.c[2]));
  const double cz = dsub(dmul(k.zen[0], p.c[1]), dmul(k.zen[1], p.c[0]));
  const double cl = __dsqrt_rn(dadd(dadd(dmul(cx, cx), dmul(cy, cy)), dmul(cz, cz)));
  const double pth = atan2(cl, p.zdot);  // v_angle (cxxsupport/geom_utils.h:59-63)
  const double dpth = atan2(p.r, __dsqrt_rn(dmul(dadd(1.0, p.r), dsub(1.0, p.r))));
  p.th_hi = dadd(pth, dpth);
  p.th_lo = dsub(pth, dpth);
  p.th_ready = true;
}

// Sign of r - dot(c, n): +1, -1, or 0 (equal, or a NaN).  The float dot
// product is within 4e-7 of the double one (unit vectors, float copies within
// 2^-24 per component) and the float radius within 6e-8 of the double
// radius, so a float difference beyond 1e-6 has the double difference's
// sign; otherwise n (double) is read and the reference's comparison made.
__device__ __forceinline__ int ray_side(const float *nf, const double *n, const RayPart &p) {
  const float s = p.rf - fmaf(p.cf[2], nf[2], fmaf(p.cf[1], nf[1], p.cf[0] * nf[0]));
  if (s > 1e-6f) return 1;
  if (s < -1e-6f) return -1;
  const double dt = ddot3(p.c, n);
  return p.r > dt ? 1 : (p.r < dt ? -1 : 0);
}

// reduceList's per-particle test (new_renderer.cc:95-100, 195-212) for the
// region g with float test vectors nf (12 floats) and the dome's centered
// flag.  The dome's halfspace check depends on the particle alone: made at
// the screen cut (halfspace true), it holds for every region after it.
__device__ __forceinline__ bool ray_keeps(const RayConst &k, const float *nf, int centered,
                                          const RayRegion &g, RayPart &p, bool halfspace) {
  if (!k.dome)
    return ray_side(nf, g.n[0], p) > 0 && ray_side(nf + 3, g.n[1], p) > 0 &&
           ray_side(nf + 6, g.n[2], p) > 0 && ray_side(nf + 9, g.n[3], p) > 0;
  if (halfspace && p.r < -p.zdot) return false;
  if (!centered && (ray_side(nf, g.n[0], p) < 0 || ray_side(nf + 3, g.n[1], p) < 0))
    return false;  // phi check
  if ((p.zdot > g.cthetamin) || (p.zdot < g.cthetamax)) {  // theta check
    if (!p.th_ready) ray_part_theta(k, p);
    if ((p.th_hi < g.thetamin) || (p.th_lo > g.thetamax)) return false;
  }
  return true;
}

// PlaneProjector::getPixDir: (p0 + dpx*ix + dpy*iy).Norm() (new_renderer.cc:71-72).
__device__ __forceinline__ void ray_pix_dir_plane(const RayConst &k, int ix, int iy, double d[3]) {
  const double X = (double)ix, Y = (double)iy;
  double t[3];
  for (int c = 0; c < 3; ++c) t[c] = dadd(dadd(k.p0[c], dmul(k.dpx[c], X)), dmul(k.dpy[c], Y));
  const double l =
      ddiv(1.0, __dsqrt_rn(dadd(dadd(dmul(t[0], t[0]), dmul(t[1], t[1])), dmul(t[2], t[2]))));
  for (int c = 0; c < 3; ++c) d[c] = dmul(t[c], l);
}

// Projector::getPixDir at full-resolution pixel (ix, iy).
__device__ __forceinline__ void ray_pix_dir(const RayConst &k, int ix, int iy, double d[3]) {
  if (!k.dome) {
    ray_pix_dir_plane(k, ix, iy, d);
    return;
  }
  // DomeProjector::getPixDir / igetPixDir (new_renderer.cc:126-138)
  const double px = dsub(dmul(dmul(2.0, k.dp), dadd((double)ix, 0.5)), 1.0);
  const double py = dsub(dmul(dmul(2.0, k.dp), dadd((double)iy, 0.5)), 1.0);
  const double r = __dsqrt_rn(dadd(dmul(px, px), dmul(py, py)));
  const double xr = ddiv(1.0, r);
  const double theta = dmul(kRayHalfPi, r);
  const double sthxr = dmul(sin(theta), xr);
  const double ct = cos(theta);
  const double a = dmul(sthxr, px), b = dmul(sthxr, py);
  for (int c = 0; c < 3; ++c) d[c] = dadd(dadd(dmul(k.ex[c], a), dmul(k.ey[c], b)), dmul(k.zen[c], ct));
}

// The sphere-vs-ray test of subrender4 (new_renderer.cc:303-312) in double;
// on a hit, w = exp(-sin^2/(r*h2sigma)^2) (1 for a NaN argument, which is
// what the reference's exptable returns for it).
__device__ __forceinline__ bool ray_exact_hit(const double d[3], double4_16a rc, double h2sigma,
                                              float &w) {
  const double c[3] = {rc.x, rc.y, rc.z};
  const double r = rc.w;
  const double cosang = ddot3(d, c);
  if (cosang < 0) return false;
  const double casq = dmul(cosang, cosang);
  const double crsq = dmul(dsub(1.0, r), dadd(1.0, r));
  if (casq < crsq) return false;  // no intersection
  const double sasq = dmul(dsub(1.0, cosang), dadd(1.0, cosang));
  const double fract = ddiv(sasq, dmul(dmul(dmul(r, r), h2sigma), h2sigma));
  w = fract != fract ? 1.f : (float)exp(-fract);
  return true;
}

}  // namespace spl
