// spl_project.cu -- fused camera transform, perspective projection,
// hsml->pixel radius, palette colourisation, tile-count and sort-key
// generation (particle_project + particle_colorize of
// splotch/splotch_host.cc:58-287, plus the counting half of render_new's
// binning, splotch_host.cc:356-387).
//
// Arithmetic follows the reference operation by operation: the transform and
// the screen shift in double (vec3 is double, cxxsupport/vec3.h:143; xshift is
// double, splotch_host.cc:103), everything else in float, with no contracted
// multiply-adds.  The outputs x, y, z, r, I and active are therefore
// bit-identical to the reference's.
#include "spl_internal.cuh"

namespace spl {

namespace {

struct PIn {
  float er, eg, eb, x, y, z, r, I;
  int type;
};

// linearMap<COLOUR>::getVal_const (cxxsupport/linear_map.h:71-84) with
// interpol_helper (cxxsupport/math_utils.h:186-196), in double like the
// reference.
__device__ __forceinline__ void palette(const ProjConst &c, int t, float v, float &r,
                                       float &g, float &b) {
  const int n = c.pal_n[t];
  const double *x = c.pal_x + c.pal_off[t];
  const float *rgb = c.pal_rgb + 3 * c.pal_off[t];
  const double xv = (double)v;
  int idx;
  if (n == 1 || xv <= x[0]) {
    idx = 0;
  } else if (xv >= x[n - 1]) {
    idx = n - 1;
  } else {
    int lo = 0, hi = n;
    while (lo < hi) {  // lower_bound
      int mid = (lo + hi) >> 1;
      if (x[mid] < xv) lo = mid + 1; else hi = mid;
    }
    idx = lo > 0 ? lo - 1 : 0;
    if (idx > n - 2) idx = n - 2;
    const double frac = ddiv(dsub(xv, x[idx]), dsub(x[idx + 1], x[idx]));
    const double omf = dsub(1.0, frac);
    r = fadd(__double2float_rn(dmul((double)rgb[3 * idx], omf)),
             __double2float_rn(dmul((double)rgb[3 * idx + 3], frac)));
    g = fadd(__double2float_rn(dmul((double)rgb[3 * idx + 1], omf)),
             __double2float_rn(dmul((double)rgb[3 * idx + 4], frac)));
    b = fadd(__double2float_rn(dmul((double)rgb[3 * idx + 2], omf)),
             __double2float_rn(dmul((double)rgb[3 * idx + 5], frac)));
    return;
  }
  r = rgb[3 * idx];
  g = rgb[3 * idx + 1];
  b = rgb[3 * idx + 2];
}

__device__ __forceinline__ void project_one(const ProjConst &c, const PIn &in, int64_t i,
                                            const ProjectOut &o) {
  const float *m = c.mat;
  const double vx = in.x, vy = in.y, vz = in.z;
  // TRANSFORM::TransPoint (kernel/transform.cxx:212-219)
  double tx = dadd(dadd(dadd(dmul(vx, m[0]), dmul(vy, m[1])), dmul(vz, m[2])), (double)m[3]);
  double ty = dadd(dadd(dadd(dmul(vx, m[4]), dmul(vy, m[5])), dmul(vz, m[6])), (double)m[7]);
  double tz = dadd(dadd(dadd(dmul(vx, m[8]), dmul(vy, m[9])), dmul(vz, m[10])), (double)m[11]);
  float x = __double2float_rn(tx), y = __double2float_rn(ty), z = __double2float_rn(tz);
  float r = in.r, I = in.I;
  float er = in.er, eg = in.eg, eb = in.eb;
  bool active = false;
  const int t = in.type;
  if (t < 0 || t >= c.ptypes) {
    atomicOr(o.err, 1u);  // type outside [0, ptypes): planck_fail in spirit
  } else if (!(-z <= c.zmin) && !(-z >= c.zmax)) {
    float xfac2 = c.xfac;
    if (!c.projection) {
      x = fadd(c.res2, fmul(x, xfac2));
      y = fadd(fadd(c.res2, c.ycorr), fmul(y, xfac2));
    } else {
      xfac2 = fdiv(-c.res2, fmul(c.fovfct, z));
      x = __double2float_rn(dadd(c.xsum, (double)fmul(x, xfac2)));
      y = __double2float_rn(dadd(c.ysum, (double)fmul(y, xfac2)));
    }
    I = fmul(I, fdiv(c.half_bfak, r));
    r = fmul(r, 2.f);
    r = fmul(r, fmul(xfac2, c.smooth[t]));
    const float rcorr = fdiv(fsqrt(fadd(fmul(r, r), c.minrad2)), r);
    r = fmul(r, rcorr);
    I = fdiv(I, rcorr);
    const float rfacr = fmul(0.75f, r);
    int minx = f2i(fadd(fsub(x, rfacr), 1.f));
    int maxx = f2i(fadd(fadd(x, rfacr), 1.f));
    int miny = f2i(fadd(fsub(y, rfacr), 1.f));
    int maxy = f2i(fadd(fadd(y, rfacr), 1.f));
    active = !(minx >= c.xres) && !(maxx <= 0) && max(minx, 0) < min(maxx, c.xres) &&
             !(miny >= c.yres) && !(maxy <= 0) && max(miny, 0) < min(maxy, c.yres);
    if (active) {  // particle_colorize (splotch_host.cc:276-282)
      if (!c.colvec[t]) palette(c, t, er, er, eg, eb);
      const float fac = fmul(I, c.bright[t]);
      er = fmul(er, fac);
      eg = fmul(eg, fac);
      eb = fmul(eb, fac);
    }
  }
  o.pos[i] = make_float4(x, y, r, z);
  o.col[i] = make_float4(er, eg, eb, I);
  o.active[i] = active ? 1 : 0;
  if (o.count) {
    uint32_t cnt = 0;
    if (active) {
      Tiling g{c.T, c.ncx, c.ncy, c.rcell, c.cmid0};
      cnt = (uint32_t)for_each_tile(x, y, r, g, [](int, int) {});
    }
    o.count[i] = cnt;
  }
  if (o.key) {
    uint32_t k;
    switch (c.sort_type) {
      case 1: k = fkey_asc(z); break;             // zcmp: z ascending
      case 2: k = ~fkey_asc(er); break;           // vcmp1: e.r descending
      case 3: k = fkey_asc(er); break;            // vcmp2: e.r ascending
      default: k = ~fkey_asc(r); break;           // hcmp: r descending
    }
    o.key[i] = k;
  }
}

__global__ void __launch_bounds__(256) k_project_aos(const uint8_t *__restrict__ aos,
                                                     int64_t n, ProjConst c, ProjectOut o) {
  // 4 particles = 144 bytes = 9 aligned float4 per thread group step when the
  // base is 16-byte aligned; the simple strided form below lets L1 merge the
  // 36-byte records of a warp into full sectors.
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float *f = reinterpret_cast<const float *>(aos + i * 36);
    PIn in;
    in.er = __ldg(f + 0); in.eg = __ldg(f + 1); in.eb = __ldg(f + 2);
    in.x = __ldg(f + 3); in.y = __ldg(f + 4); in.z = __ldg(f + 5);
    in.r = __ldg(f + 6); in.I = __ldg(f + 7);
    in.type = __ldg(reinterpret_cast<const unsigned short *>(aos + i * 36 + 32));
    project_one(c, in, i, o);
  }
}

__global__ void __launch_bounds__(256) k_project_soa(
    const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
    const float *__restrict__ r, const float *__restrict__ I, const float *__restrict__ cr,
    const float *__restrict__ cg, const float *__restrict__ cb,
    const uint16_t *__restrict__ type, int64_t n, ProjConst c, ProjectOut o) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    PIn in;
    in.x = __ldg(x + i); in.y = __ldg(y + i); in.z = __ldg(z + i);
    in.r = __ldg(r + i); in.I = __ldg(I + i);
    in.er = __ldg(cr + i);
    in.eg = cg ? __ldg(cg + i) : 0.f;
    in.eb = cb ? __ldg(cb + i) : 0.f;
    in.type = type ? (int)__ldg(type + i) : 0;
    project_one(c, in, i, o);
  }
}

// particle_sim writeback: e, x, y, z, r, I, type, active (36 bytes).
__global__ void __launch_bounds__(256) k_writeback_aos(
    const float4 *__restrict__ pos, const float4 *__restrict__ col,
    const uint8_t *__restrict__ active, const void *type_src, int type_src_kind,
    const uint32_t *__restrict__ perm, int64_t n, uint8_t *__restrict__ out) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm ? perm[s] : s;
    const float4 p = pos[i], c = col[i];
    uint16_t t = 0;
    if (type_src_kind == 1)  // AoS source: type at byte 32 of the record
      t = reinterpret_cast<const uint16_t *>(static_cast<const uint8_t *>(type_src) + i * 36 + 32)[0];
    else if (type_src_kind == 2)
      t = static_cast<const uint16_t *>(type_src)[i];
    float *f = reinterpret_cast<float *>(out + s * 36);
    f[0] = c.x; f[1] = c.y; f[2] = c.z;
    f[3] = p.x; f[4] = p.y; f[5] = p.w; f[6] = p.z; f[7] = c.w;
    uint16_t *u = reinterpret_cast<uint16_t *>(out + s * 36 + 32);
    u[0] = t;
    out[s * 36 + 34] = active[i];
    out[s * 36 + 35] = 0;
  }
}

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  const int64_t cap = 152LL * 8 * 16;  // enough resident blocks, grid-stride beyond
  if (b > cap) b = cap;
  return (int)(b > 0 ? b : 1);
}

}  // namespace

void launch_project_aos(const void *aos, int64_t n, const ProjConst &c, ProjectOut o,
                        cudaStream_t s) {
  if (n <= 0) return;
  k_project_aos<<<grid_for(n), 256, 0, s>>>(static_cast<const uint8_t *>(aos), n, c, o);
}

void launch_project_soa(const float *x, const float *y, const float *z, const float *r,
                        const float *I, const float *cr, const float *cg, const float *cb,
                        const uint16_t *type, int64_t n, const ProjConst &c, ProjectOut o,
                        cudaStream_t s) {
  if (n <= 0) return;
  k_project_soa<<<grid_for(n), 256, 0, s>>>(x, y, z, r, I, cr, cg, cb, type, n, c, o);
}

void launch_writeback_aos(const float4 *pos, const float4 *col, const uint8_t *active,
                          const void *type_src, int type_src_kind, const uint32_t *perm,
                          int64_t n, void *aos_out, cudaStream_t s) {
  if (n <= 0) return;
  k_writeback_aos<<<grid_for(n), 256, 0, s>>>(pos, col, active, type_src, type_src_kind, perm,
                                             n, static_cast<uint8_t *>(aos_out));
}

}  // namespace spl
