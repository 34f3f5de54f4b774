// spl_rays.cu -- the ray-sphere renderer (host_rendering_new,
// splotch/new_renderer.cc:522-641), selected in the reference by
// new_renderer=true (splotch/splotch_host.cc:714-723).
//
//   particle pass (spl_project.cu: k_rays_prep) -> radix sort by pyramid
//   level and direction, records gathered into that order -> per particle, a
//   walk of its level's region tree (count, scan, emit (leaf, particle)
//   pairs) -> stable sort by leaf -> leaf ranges -> leaf lists cut into
//   segments -> per level, coarsest first: one warp per segment
//   (k_rays_leaf), segment sums folded per pixel (k_rays_fold), plus the
//   spheres around the camera (coarsest level) or the coarser level
//   upsampled -> dome mask.
//
// The reference renders each level by recursive subdivision of the image:
// a region's list is its parent's list culled by the region's reduceList
// test, and a region smaller than 10x10 pixels is rendered by testing every
// pixel against every listed sphere.  Here the region tree is built on the
// host once per camera and level (it depends on nothing else), and each
// particle walks it on the GPU, emitting the leaf regions it survives to.  A
// leaf's list therefore holds exactly the reference's particles for that
// region (ordered by direction rather than by index: the sums differ from
// the reference's by rounding only).
//
// The pixel-vs-sphere test is screened in float: with d and c expressed
// relative to a direction u of the leaf, the chord |d - c|^2 is known to
// float precision relative to its own size, so it is compared with the
// sphere's chord limit with a margin that bounds every rounding; only a
// chord inside the margin is decided by the reference's double test.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "spl_host.h"
#include "spl_rays.cuh"

namespace spl {

namespace {

int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  return (int)std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 64);
}

// ---------------------------------------------------------------------------
// Host side: projector, pyramid levels and region trees, in double with the
// reference's operation order (this file's host code is built without fused
// multiply-adds).
struct V3 {
  double x, y, z;
};
V3 v3(double x, double y, double z) { return V3{x, y, z}; }
V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
V3 operator*(V3 a, double f) { return v3(a.x * f, a.y * f, a.z * f); }
double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
double length(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
V3 norm(V3 a) {  // vec3_t::Normalize: scale by 1/length
  const double l = 1. / std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return v3(a.x * l, a.y * l, a.z * l);
}
V3 from(const double *p) { return v3(p[0], p[1], p[2]); }
void put(double *p, V3 a) {
  p[0] = a.x;
  p[1] = a.y;
  p[2] = a.z;
}

constexpr double kPi = 3.141592653589793238462643383279502884197;

// reduceList's region constants for full-resolution pixel columns [ix0,ix1)
// and rows [iy0,iy1) (new_renderer.cc:77-94, 164-194).
RayRegion region_setup(const RayConst &k, int ix0, int ix1, int iy0, int iy1) {
  RayRegion g;
  std::memset(&g, 0, sizeof(g));
  if (!k.dome) {
    double x0 = ix0, x1 = ix1, y0 = iy0, y1 = iy1;
    if (ix1 == ix0 + 1) x1 += 0.001;
    if (iy1 == iy0 + 1) y1 += 0.001;
    const V3 p0 = from(k.p0), dpx = from(k.dpx), dpy = from(k.dpy);
    V3 corner[4];
    corner[0] = p0 + dpx * x0 + dpy * y0;
    corner[1] = p0 + dpx * (x1 - 1) + dpy * y0;
    corner[2] = p0 + dpx * (x1 - 1) + dpy * (y1 - 1);
    corner[3] = p0 + dpx * x0 + dpy * (y1 - 1);
    for (int i = 0; i < 4; ++i) {
      const V3 n = norm(cross(corner[i], corner[(i + 1) & 3]));
      put(g.n[i], n);
      g.nf[i][0] = (float)n.x;
      g.nf[i][1] = (float)n.y;
      g.nf[i][2] = (float)n.z;
    }
    return g;
  }
  const double dp = k.dp, halfpi = kRayHalfPi;
  double x0 = 2. * dp * (ix0 + .5) - 1., x1 = 2. * dp * (ix1 - .5) - 1.;
  double y0 = 2. * dp * (iy0 + .5) - 1., y1 = 2. * dp * (iy1 - .5) - 1.;
  if (ix1 == ix0 + 1) x1 += 0.001 * dp;
  if (iy1 == iy0 + 1) y1 += 0.001 * dp;
  const bool centered = ((x0 * x1) <= 0) && ((y0 * y1) <= 0);
  const double amaxx = std::max(std::abs(x0), std::abs(x1));
  const double amaxy = std::max(std::abs(y0), std::abs(y1));
  const double aminx = std::min(std::abs(x0), std::abs(x1));
  const double aminy = std::min(std::abs(y0), std::abs(y1));
  const double thetamax = halfpi * std::sqrt(amaxx * amaxx + amaxy * amaxy);
  double thetamin = 0;
  if (!centered) {
    if (x0 * x1 <= 0) thetamin = halfpi * aminy;
    else if (y0 * y1 <= 0) thetamin = halfpi * aminx;
    else thetamin = halfpi * std::sqrt(aminx * aminx + aminy * aminy);
  }
  const V3 ex = from(k.ex), ey = from(k.ey);
  const V3 c = ex * ((x0 + x1) * .5) + ey * ((y0 + y1) * .5);
  V3 n[4];
  n[0] = norm(ex * y0 - ey * x0);
  n[1] = norm(ex * y1 - ey * x0);
  n[2] = norm(ex * y0 - ey * x1);
  n[3] = norm(ex * y1 - ey * x1);
  V3 nx0 = n[0], nx1 = n[1];
  double curmin = 1.5;
  for (int i = 0; i < 4; ++i)
    for (int j = i + 1; j < 4; ++j)
      if (dot(n[i], n[j]) < curmin) {
        curmin = dot(n[i], n[j]);
        nx0 = n[i];
        nx1 = n[j];
      }
  if (dot(c, nx0) > 0) nx0 = v3(-nx0.x, -nx0.y, -nx0.z);
  if (dot(c, nx1) > 0) nx1 = v3(-nx1.x, -nx1.y, -nx1.z);
  put(g.n[0], nx0);
  put(g.n[1], nx1);
  for (int i = 0; i < 2; ++i)
    for (int a = 0; a < 3; ++a) g.nf[i][a] = (float)g.n[i][a];
  g.centered = centered ? 1 : 0;
  g.thetamin = thetamin;
  g.thetamax = thetamax;
  g.cthetamin = std::cos(thetamin);
  g.cthetamax = std::cos(thetamax);
  return g;
}

// subrender4's subdivision of one level's grid (new_renderer.cc:280-360):
// a region of 10 or more pixels in either direction splits in two along a
// direction more than sqrt(2) times longer than the other, else in four.
// Children are stored together; skip links give the depth-first order.
RayNode node_of(const RayRegion &g) {
  RayNode nd;
  std::memset(&nd, 0, sizeof(nd));
  const float *f = &g.nf[0][0];
  for (int i = 0; i < 3; ++i) nd.f[i] = make_float4(f[4 * i], f[4 * i + 1], f[4 * i + 2], f[4 * i + 3]);
  nd.first_child = -1;
  nd.skip = -1;
  nd.leaf = -1;
  nd.centered = g.centered;
  return nd;
}

void build_tree(RayConst &k, int L, RayFrame &f) {
  RayLevel &lv = k.lev[L];
  std::vector<int4> box;  // x0, x1, y0, y1 of each node of this level
  const int base = (int)f.nodes.size();
  lv.root = base;
  lv.leaf0 = (int)f.leaf_box.size();
  f.regs.push_back(RayRegion{});
  f.nodes.push_back(node_of(f.regs.back()));
  box.push_back(make_int4(0, lv.xdim, 0, lv.ydim));
  const int fact = lv.fact;
  for (size_t q = 0; q < box.size(); ++q) {
    const int4 b = box[q];
    const int nx = b.y - b.x, ny = b.w - b.z;
    if (nx < 10 && ny < 10) {
      f.nodes[base + q].leaf = (int)f.leaf_box.size();
      f.leaf_box.push_back(make_ushort4((unsigned short)b.x, (unsigned short)b.y,
                                        (unsigned short)b.z, (unsigned short)b.w));
      continue;
    }
    const int xm = (b.x + b.y) >> 1, ym = (b.z + b.w) >> 1;
    int4 ch[4];
    int nch;
    if (nx > std::sqrt(2.) * ny) {
      ch[0] = make_int4(b.x, xm, b.z, b.w);
      ch[1] = make_int4(xm, b.y, b.z, b.w);
      nch = 2;
    } else if (ny > std::sqrt(2.) * nx) {
      ch[0] = make_int4(b.x, b.y, b.z, ym);
      ch[1] = make_int4(b.x, b.y, ym, b.w);
      nch = 2;
    } else {
      ch[0] = make_int4(b.x, xm, b.z, ym);
      ch[1] = make_int4(b.x, xm, ym, b.w);
      ch[2] = make_int4(xm, b.y, b.z, ym);
      ch[3] = make_int4(xm, b.y, ym, b.w);
      nch = 4;
    }
    const int first = (int)f.nodes.size();
    const int parent_skip = f.nodes[base + q].skip;
    f.nodes[base + q].first_child = first;
    for (int i = 0; i < nch; ++i) {
      const int4 c = ch[i];
      f.regs.push_back(region_setup(k, c.x * fact, (c.y - 1) * fact + 1, c.z * fact,
                                    (c.w - 1) * fact + 1));
      RayNode nd = node_of(f.regs.back());
      nd.skip = i + 1 < nch ? first + i + 1 : parent_skip;
      f.nodes.push_back(nd);
      box.push_back(c);
    }
  }
  lv.nleaves = (int)f.leaf_box.size() - lv.leaf0;
}

}  // namespace

spl_status rays_setup(const spl_frame_desc *d, const spl_rays_desc *r, RayFrame &f) {
  RayConst &k = f.k;
  std::memset(&k, 0, sizeof(k));
  f.nodes.clear();
  f.regs.clear();
  f.leaf_box.clear();
  const int xres = d->xres, yres = d->yres;
  if (xres > 65535 || yres > 65535)  // leaf regions hold 16-bit pixel bounds
    return host_fail(SPL_ERR_UNSUPPORTED, "the ray-sphere renderer takes up to 65535 pixels a side");
  if (r->dome && xres != yres)
    return host_fail(SPL_ERR_INVALID, "inconsistency: a dome needs xres == yres");
  const V3 campos = from(d->campos), centerpos = from(d->centerpos), lookat = from(d->lookat);
  V3 sky = from(d->sky);
  k.dome = r->dome ? 1 : 0;
  // projector (new_renderer.cc:588-612)
  if (k.dome) {
    k.dp = 1. / xres;
    const V3 zen = norm(lookat - campos);
    const V3 y = norm(cross(zen, sky));
    const V3 x = norm(cross(y, zen));
    put(k.zen, zen);
    put(k.ex, x);
    put(k.ey, y);
  } else {
    const double fovfct = std::tan(r->fov * 0.5f * (kPi / 180.0));
    sky = norm(sky);
    const V3 zaxis = norm(centerpos - lookat);
    const V3 xaxis = norm(cross(sky, zaxis));
    const V3 yaxis = norm(cross(zaxis, xaxis));
    const V3 dpx = xaxis * (fovfct / (0.5 * xres));
    const V3 dpy = yaxis * (fovfct / (0.5 * xres));
    const V3 newcenter = (centerpos - campos) * (1. / length(centerpos - lookat));
    const V3 corner = newcenter - zaxis - dpx * (0.5 * xres) - dpy * (0.5 * yres);
    put(k.p0, corner + dpx * .5 + dpy * .5);
    put(k.dpx, dpx);
    put(k.dpy, dpy);
    for (int a = 0; a < 3; ++a) {
      k.p0f[a] = (float)k.p0[a];
      k.dpxf[a] = (float)k.dpx[a];
      k.dpyf[a] = (float)k.dpy[a];
    }
  }
  put(k.campos, campos);
  put(k.centerpos, centerpos);
  k.zmax = d->zmax;
  k.half_bfak = 0.5f * (0.5 * std::pow(kPi, -5. / 6.));
  k.h2sigma = 0.5 * std::pow(kPi, -1. / 6.);
  // real_host_rendering (new_renderer.cc:398-501)
  double pixrad;
  if (k.dome) {
    pixrad = k.dp * kPi;
  } else {
    const V3 p0 = from(k.p0), dpx = from(k.dpx), dpy = from(k.dpy);
    const double screendist = std::abs(dot(p0, norm(cross(dpx, dpy))));
    pixrad = std::min(length(dpx), length(dpy)) / screendist;
  }
  const double mr = r->minrad_pix;
  k.mr2pr2 = mr * mr * pixrad * pixrad;
  k.screen = region_setup(k, 0, xres, 0, yres);
  const double minpixperrad = 15;
  double maxfac = 1. / (minpixperrad * pixrad);
  maxfac = std::min(maxfac, std::min(xres, yres) / 10.);
  int nsteps = 0;
  while ((1 << nsteps) < maxfac) ++nsteps;
  nsteps = std::max(nsteps - 1, 0);
  if (nsteps + 1 > kRayMaxLevels)
    return host_fail(SPL_ERR_UNSUPPORTED, "too many pyramid levels");
  k.nlev = nsteps + 1;
  for (int L = 0; L < k.nlev; ++L) {
    const int fact = 1 << (nsteps - L);
    RayLevel &lv = k.lev[L];
    lv.fact = fact;
    lv.xdim = xres;
    lv.ydim = yres;
    for (int f2 = fact; f2 > 1; f2 >>= 1) {
      lv.xdim = (lv.xdim >> 1) + 1;
      lv.ydim = (lv.ydim >> 1) + 1;
    }
    double minrad = minpixperrad * pixrad * fact;
    double maxrad = std::min(1., 2 * minrad);
    if (fact == 1) minrad = 0.;
    if (fact == 1 << nsteps) maxrad = 1;
    lv.minrad = minrad;
    lv.maxrad = maxrad;
    build_tree(k, L, f);
  }
  return SPL_OK;
}

namespace {

// ---------------------------------------------------------------------------
// Device side.

// Each particle of a level grid walks its level's region tree depth first,
// without a stack: a region it passes is entered (its first child next), a
// region it fails is stepped over (its skip link next).
template <bool EMIT>
__global__ void __launch_bounds__(128) k_rays_walk(
    RayConst k, const RayNode *__restrict__ nodes, const RayRegion *__restrict__ regs,
    const uint32_t *__restrict__ key_s, int64_t n, RayParts p, uint32_t *__restrict__ count,
    uint32_t *__restrict__ slots, const uint64_t *__restrict__ off, uint32_t *__restrict__ keys,
    uint32_t *__restrict__ vals) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t L = key_s[s] >> kRayCodeShift;
    if (L >= (uint32_t)k.nlev) {
      if (!EMIT) count[s] = 0;
      continue;
    }
    const uint32_t i = (uint32_t)s;  // records are in sorted order
    uint64_t o = 0;
    if (EMIT) {
      const uint32_t c = count[s];
      o = off[s];
      if (c <= (uint32_t)kRayWalkSlots) {  // the first walk kept them all
        for (uint32_t j = 0; j < c; ++j) {
          keys[o + j] = slots[(size_t)s * kRayWalkSlots + j];
          vals[o + j] = i;
        }
        continue;
      }
    }
    RayPart part = ray_part(k, p.rc[i], p.cf[i]);
    uint32_t cnt = 0;
    auto emit = [&](int leaf) {
      if (EMIT) {
        keys[o + cnt] = (uint32_t)leaf;
        vals[o + cnt] = i;
      } else if (cnt < (uint32_t)kRayWalkSlots) {
        slots[(size_t)s * kRayWalkSlots + cnt] = (uint32_t)leaf;
      }
      ++cnt;
    };
    const RayNode root = nodes[k.lev[L].root];
    if (root.leaf >= 0) {  // the whole grid is one leaf region: no test
      emit(root.leaf);
    } else {
      int nd = root.first_child;
      while (nd >= 0) {
        const RayNode node = nodes[nd];
        if (ray_keeps(k, &node.f[0].x, node.centered, regs[nd], part, false)) {
          if (node.leaf >= 0) {
            emit(node.leaf);
            nd = node.skip;
          } else {
            nd = node.first_child;
          }
        } else {
          nd = node.skip;
        }
      }
    }
    if (!EMIT) count[s] = cnt;
  }
}

// Level ranges of the sorted keys: lev_start[c] = first sorted position of
// code c (c = 0 .. nlev + 2).
__global__ void __launch_bounds__(256) k_rays_level_ranges(const uint32_t *__restrict__ key_s,
                                                           int64_t n, int ncodes,
                                                           uint32_t *__restrict__ lev_start) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q <= n;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cprev = q > 0 ? (int64_t)(key_s[q - 1] >> kRayCodeShift) : -1;
    const int64_t ccur = q < n ? (int64_t)(key_s[q] >> kRayCodeShift) : ncodes;
    for (int64_t c = cprev + 1; c <= ccur; ++c) lev_start[c] = (uint32_t)q;
  }
}

// Records of the rendered particles (levels and spheres around the camera)
// gathered into sorted order.
__global__ void __launch_bounds__(256) k_rays_gather(const uint32_t *__restrict__ key_s,
                                                     const uint32_t *__restrict__ order, int64_t n,
                                                     int nlev, RayParts src, RayParts dst) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    if ((key_s[q] >> kRayCodeShift) > (uint32_t)nlev) continue;
    const uint32_t i = order[q];
    dst.rc[q] = src.rc[i];
    dst.cf[q] = src.cf[i];
    dst.clo[q] = src.clo[i];
    dst.pod[q] = src.pod[i];
    dst.cov[q] = src.cov[i];
  }
}

// Direction of full-resolution pixel (X, Y) in double, out of line (once
// per pixel and leaf segment).
__device__ __noinline__ double3 ray_dir3(const RayConst *__restrict__ kd, int X, int Y) {
  double d[3];
  ray_pix_dir(*kd, X, Y, d);
  return make_double3(d[0], d[1], d[2]);
}

// The plane projector's sphere-vs-ray test in double at full-resolution
// pixel (X, Y), out of line (a chord within the float screen's margin): the
// weight on a hit, -1 on a miss.
__device__ __noinline__ float ray_plane_exact(const RayConst *__restrict__ kd, int X, int Y,
                                              double4_16a rc) {
  double d[3];
  ray_pix_dir_plane(*kd, X, Y, d);
  float w;
  return ray_exact_hit(d, rc, kd->h2sigma, w) ? w : -1.f;
}

// add_overlap2 (new_renderer.cc:367-393) at full-resolution pixel (X, Y):
// the spheres around the camera (sorted positions s0 .. s1), each weighted by the erfc
// of its near half (no coverage test).
__device__ __noinline__ float4 ray_overlap(const RayConst *__restrict__ kd, int X, int Y,
                                           uint32_t s0, uint32_t s1,
                                           const double4_16a *__restrict__ rcs,
                                           const float4 *__restrict__ pods) {
  double d[3];
  ray_pix_dir(*kd, X, Y, d);
  const double h2 = kd->h2sigma;
  float o0 = 0.f, o1 = 0.f, o2 = 0.f;
  for (uint32_t i = s0; i < s1; ++i) {
    const double4_16a rc = rcs[i];
    const double c[3] = {rc.x, rc.y, rc.z};
    const double cosang = ddot3(d, c);
    const double sasq = dmul(dsub(1.0, cosang), dadd(1.0, cosang));
    const double fract = ddiv(sasq, dmul(dmul(dmul(rc.w, rc.w), h2), h2));
    const double er = dmul(0.5, erfc(ddiv(-cosang, dmul(rc.w, h2))));
    const float w = fract != fract ? 1.f : (float)exp(-fract);
    const float ew = __double2float_rn(er) * w;
    const float4 e = pods[i];
    o0 = fmaf(-e.x, ew, o0);
    o1 = fmaf(-e.y, ew, o1);
    o2 = fmaf(-e.z, ew, o2);
  }
  return make_float4(o0, o1, o2, 0.f);
}

// A leaf pixel's final value: its sum over the leaf's list plus the spheres
// around the camera (coarsest level) or the coarser grid upsampled
// (new_renderer.cc:509-515).
template <bool TOP>
__device__ __forceinline__ void ray_finish(const RayConst &k, const RayLevel &lv,
                                           const RayLeafArgs &a, const RayParts &p, int x, int y,
                                           float od0, float od1, float od2) {
  if (TOP) {
    const float4 o = ray_overlap(a.kd, x * lv.fact, y * lv.fact, a.lev_start[k.nlev],
                                 a.lev_start[k.nlev + 1], p.rc, p.pod);
    od0 = fadd(od0, o.x);
    od1 = fadd(od1, o.y);
    od2 = fadd(od2, o.z);
  } else {
    const float *C = a.coarse;
    const size_t cy = (size_t)a.cdim_y;
    const size_t pa = ((size_t)(x >> 1) * cy + (y >> 1)) * 3;
    const size_t pb = ((size_t)((x + 1) >> 1) * cy + (y >> 1)) * 3;
    const size_t pc = ((size_t)(x >> 1) * cy + ((y + 1) >> 1)) * 3;
    const size_t pd = ((size_t)((x + 1) >> 1) * cy + ((y + 1) >> 1)) * 3;
    od0 = fadd(od0, fmul(fadd(fadd(fadd(C[pa], C[pb]), C[pc]), C[pd]), 0.25f));
    od1 = fadd(od1, fmul(fadd(fadd(fadd(C[pa + 1], C[pb + 1]), C[pc + 1]), C[pd + 1]), 0.25f));
    od2 = fadd(od2, fmul(fadd(fadd(fadd(C[pa + 2], C[pb + 2]), C[pc + 2]), C[pd + 2]), 0.25f));
  }
  float *o = a.out + ((size_t)x * lv.ydim + y) * 3;
  o[0] = od0;
  o[1] = od1;
  o[2] = od2;
}

// One segment (kRaySegLen list entries) of one leaf region per warp, over
// every segment of level L (persistent warps).  Lane l owns pixels l, l+32,
// l+64 of the leaf (column-major within it).  The segment is staged through
// the warp's shared slice 32 entries at a time, in list order; each pixel
// accumulates -e*w over the spheres its ray meets.
//
// The float screen works with directions relative to u, the leaf's first
// pixel's direction: c - u from the float-float pair of c, and d - u for a
// plane projector from the float pixel grid (d - u = dt/|t| - t_u g with
// t = t_u + dt and g = (2 t_u.dt + dt.dt) / (|t| |t_u| (|t| + |t_u|)), which
// loses nothing to cancellation), for the dome from the double directions.
template <bool TOP, bool DOME>
__global__ void __launch_bounds__(32 * kRayLeafWarps, 6) k_rays_leaf(RayConst k, int L, RayParts p,
                                                                  RayLeafArgs a) {
  const RayLevel &lv = k.lev[L];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ float4 s_a[kRayLeafWarps][32], s_b[kRayLeafWarps][32];
  __shared__ float s_inv[kRayLeafWarps][32];
  __shared__ uint32_t s_idx[kRayLeafWarps][32];
  __shared__ double s_d[kRayLeafWarps][3][DOME ? 96 : 1];  // dome: the pixels' directions
  const uint64_t it0 = a.seg_off[lv.leaf0], it1 = a.seg_off[lv.leaf0 + lv.nleaves];
  const int fact = lv.fact;
  for (uint64_t item = it0 + (uint64_t)blockIdx.x * kRayLeafWarps + warp; item < it1;
       item += (uint64_t)gridDim.x * kRayLeafWarps) {
    const uint32_t leaf = a.item_leaf[item];
    const uint64_t first = a.seg_off[leaf];
    const uint32_t nseg = (uint32_t)(a.seg_off[leaf + 1] - first);
    const uint32_t sidx = (uint32_t)(item - first);
    const ushort4 box = a.leaf_box[leaf];
    const int nx = box.y - box.x, ny = box.w - box.z;
    const int npx = nx * ny;
    const int npl = (npx + 31) >> 5;  // pixels per lane, warp-uniform

    // u: the leaf's first pixel's direction, in double and as a float-float pair
    const int X0 = box.x * fact, Y0 = box.z * fact;
    const double3 ud = ray_dir3(a.kd, X0, Y0);
    const float uh0 = __double2float_rn(ud.x), uh1 = __double2float_rn(ud.y);
    const float uh2 = __double2float_rn(ud.z);
    const float ul0 = __double2float_rn(dsub(ud.x, (double)uh0));
    const float ul1 = __double2float_rn(dsub(ud.y, (double)uh1));
    const float ul2 = __double2float_rn(dsub(ud.z, (double)uh2));
    float tu0 = 0.f, tu1 = 0.f, tu2 = 0.f, ntu = 1.f;
    if (!DOME) {
      tu0 = fmaf((float)Y0, k.dpyf[0], fmaf((float)X0, k.dpxf[0], k.p0f[0]));
      tu1 = fmaf((float)Y0, k.dpyf[1], fmaf((float)X0, k.dpxf[1], k.p0f[1]));
      tu2 = fmaf((float)Y0, k.dpyf[2], fmaf((float)X0, k.dpxf[2], k.p0f[2]));
      ntu = sqrtf(fmaf(tu2, tu2, fmaf(tu1, tu1, tu0 * tu0)));
    }
    float dd[3][3], od[3][3];
    bool has[3];
    float l1max = 0.f;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const int q = lane + 32 * m;
      has[m] = q < npx;
      const int ixm = box.x + (has[m] ? q / ny : 0), iym = box.z + (has[m] ? q % ny : 0);
      od[m][0] = od[m][1] = od[m][2] = 0.f;
      dd[m][0] = dd[m][1] = dd[m][2] = 0.f;
      if (m < npl) {
        if (DOME) {
          const double3 d = ray_dir3(a.kd, ixm * fact, iym * fact);
          s_d[warp][0][q] = d.x;
          s_d[warp][1][q] = d.y;
          s_d[warp][2][q] = d.z;
          dd[m][0] = __double2float_rn(dsub(d.x, ud.x));
          dd[m][1] = __double2float_rn(dsub(d.y, ud.y));
          dd[m][2] = __double2float_rn(dsub(d.z, ud.z));
        } else {
          const float gx = (float)(ixm * fact - X0), gy = (float)(iym * fact - Y0);
          const float t0 = gx * k.dpxf[0] + gy * k.dpyf[0];
          const float t1 = gx * k.dpxf[1] + gy * k.dpyf[1];
          const float t2 = gx * k.dpxf[2] + gy * k.dpyf[2];
          const float a0 = tu0 + t0, a1 = tu1 + t1, a2 = tu2 + t2;
          const float nt = sqrtf(fmaf(a2, a2, fmaf(a1, a1, a0 * a0)));
          const float num = fmaf(t2, fmaf(2.f, tu2, t2), fmaf(t1, fmaf(2.f, tu1, t1),
                                                              t0 * fmaf(2.f, tu0, t0)));
          const float g = num / (nt * ntu * (nt + ntu));
          const float it = 1.f / nt;
          dd[m][0] = fmaf(t0, it, -tu0 * g);
          dd[m][1] = fmaf(t1, it, -tu1 * g);
          dd[m][2] = fmaf(t2, it, -tu2 * g);
        }
        const float l1 = fabsf(dd[m][0]) + fabsf(dd[m][1]) + fabsf(dd[m][2]);
        if (has[m]) l1max = l1 == l1 ? fmaxf(l1max, l1) : INFINITY;  // NaN: a NaN direction
      }
    }
    // largest |d - u|_1 of the leaf (non-negative floats order as their bits)
    const float rd1 = __uint_as_float(
        __reduce_max_sync(0xffffffffu, __float_as_uint(l1max * 1.0001f)));

    const uint32_t l0 = a.leaf_start[leaf];
    const uint32_t e0 = l0 + sidx * kRaySegLen;
    const uint32_t e1 = min(a.leaf_start[leaf + 1], e0 + kRaySegLen);
    for (uint32_t b0 = e0; b0 < e1; b0 += 32) {
      const uint32_t cnt = min(32u, e1 - b0);
      if ((uint32_t)lane < cnt) {
        const uint32_t i = a.vals[b0 + lane];
        const float4 cf = p.cf[i];
        const float4 cl = p.clo[i];
        const float2 cv = p.cov[i];
        const float4 e = p.pod[i];
        const float c0 = (cf.x - uh0) + (cl.x - ul0);
        const float c1 = (cf.y - uh1) + (cl.y - ul1);
        const float c2 = (cf.z - uh2) + (cl.z - ul2);
        // |q - |d - c|^2| <= 2|d - c| E + E^2 + 3 ulp(q) with E bounding the
        // error of d - c: 4 ulp of d - u (the float grid form) and 2 ulp of
        // c - u plus the float-float pairs' 2^-48, 1e-13 in all; the margin
        // doubles that at the limit cm and adds the rounding of cm itself.
        // No limit (cm < 0), or a NaN direction in the leaf (rd1 infinite):
        // every pixel is decided in double.
        float lo = -1.f, hi = INFINITY;
        if (cv.x >= 0.f && rd1 < INFINITY) {
          const float E = 6e-7f * (rd1 + fabsf(c0) + fabsf(c1) + fabsf(c2)) + 1e-13f;
          const float mg = 4.f * sqrtf(cv.x) * E + 2.f * E * E + 1e-6f * cv.x + 1e-13f;
          lo = cv.x - mg;
          hi = cv.x + mg;
        }
        s_a[warp][lane] = make_float4(c0, c1, c2, lo);
        s_b[warp][lane] = make_float4(-e.x, -e.y, -e.z, hi);
        s_inv[warp][lane] = cv.y * kLog2e;
        s_idx[warp][lane] = i;
      }
      __syncwarp();
      // entries whose chord falls within the screen's margin, per pixel:
      // decided after the batch (out of the inner loop, which keeps its
      // register footprint small); only the order of those few additions moves
      uint32_t und[3] = {0u, 0u, 0u};
      for (uint32_t j = 0; j < cnt; ++j) {
        const float4 A = s_a[warp][j];
        const float4 B = s_b[warp][j];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          if (m >= npl) break;
          const float x0 = dd[m][0] - A.x, x1 = dd[m][1] - A.y, x2 = dd[m][2] - A.z;
          const float q = fmaf(x2, x2, fmaf(x1, x1, x0 * x0));
          if (!has[m] || q > B.w) continue;  // the ray misses the sphere
          if (q < A.w) {  // it meets it: sin^2 = q (1 - q/4)
            const float sasq = q * fmaf(-0.25f, q, 1.f);
            const float w = ex2(-sasq * s_inv[warp][j]);
            od[m][0] = fmaf(B.x, w, od[m][0]);
            od[m][1] = fmaf(B.y, w, od[m][1]);
            od[m][2] = fmaf(B.z, w, od[m][2]);
          } else {
            und[m] |= 1u << j;
          }
        }
      }
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        while (und[m]) {  // the reference's double test
          const int j = __ffs(und[m]) - 1;
          und[m] &= und[m] - 1;
          float w;
          if (DOME) {
            const int qq = lane + 32 * m;
            const double d[3] = {s_d[warp][0][DOME ? qq : 0], s_d[warp][1][DOME ? qq : 0],
                                 s_d[warp][2][DOME ? qq : 0]};
            if (!ray_exact_hit(d, p.rc[s_idx[warp][j]], k.h2sigma, w)) continue;
          } else {
            w = ray_plane_exact(a.kd, (box.x + (lane + 32 * m) / ny) * fact,
                                (box.z + (lane + 32 * m) % ny) * fact, p.rc[s_idx[warp][j]]);
            if (w < 0.f) continue;
          }
          const float4 B = s_b[warp][j];
          od[m][0] = fmaf(B.x, w, od[m][0]);
          od[m][1] = fmaf(B.y, w, od[m][1]);
          od[m][2] = fmaf(B.z, w, od[m][2]);
        }
      }
      __syncwarp();
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (!has[m]) continue;
      if (nseg == 1) {
        const int q = lane + 32 * m;
        ray_finish<TOP>(k, lv, a, p, box.x + q / ny, box.z + q % ny, od[m][0], od[m][1],
                        od[m][2]);
      } else {  // this segment's sums, folded by k_rays_fold
        float *pp = a.partial + (size_t)item * (kRayLeafPixels * 3) + (lane + 32 * m) * 3;
        pp[0] = od[m][0];
        pp[1] = od[m][1];
        pp[2] = od[m][2];
      }
    }
  }
}

// Leaves of level L cut into several segments: each pixel's segment sums
// added in segment order (list order), then finished.  One warp per leaf.
template <bool TOP>
__global__ void __launch_bounds__(32 * kRayLeafWarps) k_rays_fold(RayConst k, int L, RayParts p,
                                                                  RayLeafArgs a) {
  const RayLevel &lv = k.lev[L];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int li = blockIdx.x * kRayLeafWarps + warp; li < lv.nleaves;
       li += gridDim.x * kRayLeafWarps) {
    const uint32_t leaf = lv.leaf0 + li;
    const uint64_t first = a.seg_off[leaf];
    const uint32_t nseg = (uint32_t)(a.seg_off[leaf + 1] - first);
    if (nseg < 2) continue;
    const ushort4 box = a.leaf_box[leaf];
    const int ny = box.w - box.z;
    const int npx = (box.y - box.x) * ny;
    for (int q = lane; q < npx; q += 32) {
      float v0 = 0.f, v1 = 0.f, v2 = 0.f;
      for (uint32_t sg = 0; sg < nseg; ++sg) {
        const float *pp = a.partial + (size_t)(first + sg) * (kRayLeafPixels * 3) + q * 3;
        v0 = fadd(v0, pp[0]);
        v1 = fadd(v1, pp[1]);
        v2 = fadd(v2, pp[2]);
      }
      ray_finish<TOP>(k, lv, a, p, box.x + q / ny, box.z + q % ny, v0, v1, v2);
    }
  }
}

__global__ void k_rays_segments(const uint32_t *__restrict__ leaf_start, int64_t nleaves,
                                uint32_t *__restrict__ cnt) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < nleaves;
       l += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t len = leaf_start[l + 1] - leaf_start[l];
    cnt[l] = max(1u, (len + kRaySegLen - 1) / kRaySegLen);
  }
}

__global__ void k_rays_items(const uint64_t *__restrict__ seg_off, int64_t nleaves,
                             uint32_t *__restrict__ item_leaf) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < nleaves;
       l += (int64_t)gridDim.x * blockDim.x)
    for (uint64_t it = seg_off[l]; it < seg_off[l + 1]; ++it) item_leaf[it] = (uint32_t)l;
}

// First column j of each row i <= res/2 inside the fisheye circle, with the
// reference's double arithmetic (new_renderer.cc:622-637): the least j whose
// point is inside (jstop starts above any column: a row with none keeps it).
__global__ void k_dome_rows(int res, int *jstop) {
  const int64_t np = (int64_t)(res / 2 + 1) * res;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < np;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q / res), j = (int)(q % res);
    const double xf = ddiv(1.0, (double)(res - 1));
    double x = dmul(dadd((double)i, 0.5), xf);
    x = dsub(dmul(2.0, x), 1.0);
    double y = dmul(dadd((double)j, 0.5), xf);
    y = dsub(dmul(2.0, y), 1.0);
    if (!(dadd(dmul(x, x), dmul(y, y)) > 1.)) atomicMin(jstop + i, j);
  }
}

// The reference zeroes (i, j), (i, res-1-j), (res-1-i, res-1-j), (res-1-i, j)
// for every i <= res/2 and j < jstop[i].
__global__ void k_dome_mask(float *pic, int res, const int *__restrict__ jstop) {
  const int64_t np = (int64_t)res * res;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < np;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(q / res), b = (int)(q % res);
    const int is[2] = {a, res - 1 - a}, js[2] = {b, res - 1 - b};
    bool zero = false;
    for (int u = 0; u < 2; ++u)
      if (is[u] <= res / 2)
        for (int v = 0; v < 2; ++v) zero = zero || js[v] < jstop[is[u]];
    if (zero) {
      pic[q * 3] = 0.f;
      pic[q * 3 + 1] = 0.f;
      pic[q * 3 + 2] = 0.f;
    }
  }
}

}  // namespace

void launch_rays_walk(bool emit, const RayConst &k, const RayNode *nodes, const RayRegion *regs,
                      const uint32_t *key_s, int64_t n, const RayParts &p, uint32_t *count,
                      uint32_t *slots, const uint64_t *off, uint32_t *keys, uint32_t *vals,
                      cudaStream_t s) {
  if (n <= 0) return;
  if (emit)
    k_rays_walk<true><<<grid_for(n, 128), 128, 0, s>>>(k, nodes, regs, key_s, n, p, count, slots,
                                                        off, keys, vals);
  else
    k_rays_walk<false><<<grid_for(n, 128), 128, 0, s>>>(k, nodes, regs, key_s, n, p, count, slots,
                                                         off, keys, vals);
}

void launch_rays_sorted(const uint32_t *key_s, const uint32_t *order, int64_t n, int nlev,
                        uint32_t *lev_start, const RayParts &src, const RayParts &dst,
                        cudaStream_t s) {
  k_rays_level_ranges<<<grid_for(n + 1, 256), 256, 0, s>>>(key_s, n, nlev + 2, lev_start);
  if (n > 0) k_rays_gather<<<grid_for(n, 256), 256, 0, s>>>(key_s, order, n, nlev, src, dst);
}

void launch_rays_segments(const uint32_t *leaf_start, int64_t nleaves, uint32_t *cnt,
                          cudaStream_t s) {
  if (nleaves > 0) k_rays_segments<<<grid_for(nleaves, 256), 256, 0, s>>>(leaf_start, nleaves, cnt);
}

void launch_rays_items(const uint64_t *seg_off, int64_t nleaves, uint32_t *item_leaf,
                       cudaStream_t s) {
  if (nleaves > 0)
    k_rays_items<<<grid_for(nleaves, 256), 256, 0, s>>>(seg_off, nleaves, item_leaf);
}

void launch_rays_leaves(const RayConst &k, int L, const RayParts &p, const RayLeafArgs &a,
                        cudaStream_t s) {
  const int nl = k.lev[L].nleaves;
  if (nl <= 0) return;
  // persistent warps over the level's segments (their count stays on the device)
  const int grid = 152 * 16;
  const int fgrid = std::min((nl + kRayLeafWarps - 1) / kRayLeafWarps, 152 * 8);
  if (L == 0) {
    if (k.dome)
      k_rays_leaf<true, true><<<grid, 32 * kRayLeafWarps, 0, s>>>(k, L, p, a);
    else
      k_rays_leaf<true, false><<<grid, 32 * kRayLeafWarps, 0, s>>>(k, L, p, a);
    k_rays_fold<true><<<fgrid, 32 * kRayLeafWarps, 0, s>>>(k, L, p, a);
  } else {
    if (k.dome)
      k_rays_leaf<false, true><<<grid, 32 * kRayLeafWarps, 0, s>>>(k, L, p, a);
    else
      k_rays_leaf<false, false><<<grid, 32 * kRayLeafWarps, 0, s>>>(k, L, p, a);
    k_rays_fold<false><<<fgrid, 32 * kRayLeafWarps, 0, s>>>(k, L, p, a);
  }
}

void launch_rays_dome_mask(float *pic, int res, int *jstop, cudaStream_t s) {
  if (res <= 0) return;
  cudaMemsetAsync(jstop, 0x7f, (size_t)(res / 2 + 1) * sizeof(int), s);
  k_dome_rows<<<grid_for((int64_t)(res / 2 + 1) * res, 256), 256, 0, s>>>(res, jstop);
  k_dome_mask<<<grid_for((int64_t)res * res, 256), 256, 0, s>>>(pic, res, jstop);
}

}  // namespace spl
