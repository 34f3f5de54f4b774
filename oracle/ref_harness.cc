// ref_harness.cc -- C-ABI harness around the reference's own host renderer.
//
// TEST INFRASTRUCTURE ONLY.  Compiled together with the reference sources
// (splotch/splotch_host.cc and friends, read in place) by oracle/build_ref.sh
// into oracle/_ref/libsplotch_ref.so.  It lets the tests run the reference's
// particle_project / particle_colorize / render_new / host_rendering on the
// same seeded inputs as the CUDA path, to pin the oracle restatement and to
// make golden fixtures.  Nothing in the product links it.
#include <algorithm>
#include <cstdlib>
#include <map>
#include <string>
#include <vector>

#include "cxxsupport/ls_image.h"
#include "splotch/scenemaker.h"
#include "splotch/splotch_host.h"
#include "splotch/splotchutils.h"

namespace host_funct {
// The definitions in splotch/splotch_host.cc:289,330 differ from the header
// declarations (splotch/splotch_host.h:32-35); declare what is defined.
void particle_sort(particle_sim *p, int npart, int sort_type, bool verbose);
void render_new(particle_sim *p, int npart, arr2<COLOUR> &pic, bool a_eq_e,
                float32 grayabsorb, int tile_size);
}  // namespace host_funct

static_assert(sizeof(particle_sim) == 36, "particle_sim must be 36 bytes");

// sceneMaker::particle_normalize (splotch/scenemaker.cc:40-296) is private: its
// address is taken through an explicit template instantiation, where access
// checking does not apply ([temp.explicit]).
namespace {
struct NormalizeTag {
  typedef void (sceneMaker::*type)(std::vector<particle_sim> &, bool) const;
  friend type member(NormalizeTag);
};
template <typename Tag, typename Tag::type M>
struct Expose {
  friend typename Tag::type member(Tag) { return M; }
};
template struct Expose<NormalizeTag, &sceneMaker::particle_normalize>;
}  // namespace

namespace {

paramfile make_params(const char *const *keys, const char *const *vals, int nkv) {
  std::map<std::string, std::string> m;
  for (int i = 0; i < nkv; ++i) m[keys[i]] = vals[i];
  return paramfile(m, false);
}

void make_amap(std::vector<COLOURMAP> &amap, int ntypes, const int *pal_n,
               const double *const *pal_x, const float *const *pal_rgb) {
  amap.resize(ntypes);
  for (int t = 0; t < ntypes; ++t) {
    if (pal_n[t] <= 0) continue;
    for (int i = 0; i < pal_n[t]; ++i)
      amap[t].addVal(pal_x[t][i], COLOUR(pal_rgb[t][3 * i], pal_rgb[t][3 * i + 1],
                                         pal_rgb[t][3 * i + 2]));
    amap[t].sortMap();
  }
}

void pic_out(const arr2<COLOUR> &pic, float *out) {
  const tsize nx = pic.size1(), ny = pic.size2();
  for (tsize x = 0; x < nx; ++x)
    for (tsize y = 0; y < ny; ++y) {
      const COLOUR &c = pic[x][y];
      float *o = out + (x * ny + y) * 3;
      o[0] = c.r; o[1] = c.g; o[2] = c.b;
    }
}

}  // namespace

extern "C" {

int ref_simd_branch(void) {
#ifdef __SSE2__
  return 1;
#else
  return 0;
#endif
}

// particle_project (+ particle_colorize when colorize != 0), in place.
int ref_project_colorize(const char *const *keys, const char *const *vals, int nkv,
                         void *particles, long n, const double *campos,
                         const double *lookat, const double *sky,
                         const double *centerpos, int ntypes, const int *pal_n,
                         const double *const *pal_x, const float *const *pal_rgb,
                         float b_brightness, int colorize) {
  try {
    paramfile params = make_params(keys, vals, nkv);
    particle_sim *p = static_cast<particle_sim *>(particles);
    std::vector<particle_sim> v(p, p + n);
    vec3 cp(campos[0], campos[1], campos[2]), la(lookat[0], lookat[1], lookat[2]),
        sk(sky[0], sky[1], sky[2]), ce(centerpos[0], centerpos[1], centerpos[2]);
    host_funct::particle_project(params, v, cp, la, sk, ce);
    if (colorize) {
      std::vector<COLOURMAP> amap;
      make_amap(amap, ntypes, pal_n, pal_x, pal_rgb);
      host_funct::particle_colorize(params, v, amap, b_brightness);
    }
    std::copy(v.begin(), v.end(), p);
    return 0;
  } catch (...) {
    return -1;
  }
}

// render_new over particles already projected and colourised (and ordered).
int ref_render_new(void *particles, int n, int xres, int yres, int a_eq_e,
                   float gray, int tile, float *pic) {
  try {
    arr2<COLOUR> img(xres, yres);
    host_funct::render_new(static_cast<particle_sim *>(particles), n, img, a_eq_e != 0,
                           gray, tile);
    pic_out(img, pic);
    return 0;
  } catch (...) {
    return -1;
  }
}

// The reference's own (unstable) particle_sort.
int ref_particle_sort(void *particles, int n, int sort_type) {
  try {
    host_funct::particle_sort(static_cast<particle_sim *>(particles), n, sort_type, false);
    return 0;
  } catch (...) {
    return -1;
  }
}

// The whole host_rendering() call.
int ref_host_rendering(const char *const *keys, const char *const *vals, int nkv,
                       void *particles, long n, const double *campos,
                       const double *lookat, const double *sky, const double *centerpos,
                       int ntypes, const int *pal_n, const double *const *pal_x,
                       const float *const *pal_rgb, float b_brightness, int xres,
                       int yres, float *pic) {
  try {
    paramfile params = make_params(keys, vals, nkv);
    particle_sim *p = static_cast<particle_sim *>(particles);
    std::vector<particle_sim> v(p, p + n);
    render_context rc;
    rc.campos = vec3(campos[0], campos[1], campos[2]);
    rc.lookat = vec3(lookat[0], lookat[1], lookat[2]);
    rc.sky = vec3(sky[0], sky[1], sky[2]);
    rc.centerpos = vec3(centerpos[0], centerpos[1], centerpos[2]);
    make_amap(rc.amap, ntypes, pal_n, pal_x, pal_rgb);
    rc.xres = xres;
    rc.yres = yres;
    rc.pic.alloc(xres, yres);
    rc.npart = n;
    rc.npart_all = n;
    rc.b_brightness = b_brightness;
    host_rendering(params, v, rc);
    std::copy(v.begin(), v.end(), p);
    pic_out(rc.pic, pic);
    return 0;
  } catch (...) {
    return -1;
  }
}

// The master's post-processing of splotch/splotch.cc:272-291 on an x-major
// image, in place: pic = -expm1(pic) with exptable<float32>(-20) when a_eq_e,
// then colour_adjust, then add_colorbar when the colorbar key is set.
int ref_postprocess(const char *const *keys, const char *const *vals, int nkv, float *pic,
                    int xres, int yres, int a_eq_e, int ntypes, const int *pal_n,
                    const double *const *pal_x, const float *const *pal_rgb) {
  try {
    paramfile params = make_params(keys, vals, nkv);
    render_context rc;
    make_amap(rc.amap, ntypes, pal_n, pal_x, pal_rgb);
    rc.xres = xres;
    rc.yres = yres;
    rc.pic.alloc(xres, yres);
    for (int x = 0; x < xres; ++x)
      for (int y = 0; y < yres; ++y) {
        const float *s = pic + ((size_t)x * yres + y) * 3;
        rc.pic[x][y] = COLOUR(s[0], s[1], s[2]);
      }
    exptable<float32> xexp(-20.0);
    if (a_eq_e)
      for (int ix = 0; ix < rc.xres; ix++)
        for (int iy = 0; iy < rc.yres; iy++) {
          rc.pic[ix][iy].r = -xexp.expm1(rc.pic[ix][iy].r);
          rc.pic[ix][iy].g = -xexp.expm1(rc.pic[ix][iy].g);
          rc.pic[ix][iy].b = -xexp.expm1(rc.pic[ix][iy].b);
        }
    colour_adjust(params, rc);
    if (params.find<bool>("colorbar", false)) add_colorbar(params, rc.pic, rc.amap);
    pic_out(rc.pic, pic);
    return 0;
  } catch (...) {
    return -1;
  }
}

// sceneMaker::particle_normalize on particle_sim records, in place.  out
// receives, per type, the values it leaves in the paramfile: range_min,
// range_max, clamp_min, clamp_max (4 doubles per type).
int ref_particle_normalize(const char *const *keys, const char *const *vals, int nkv,
                           void *particles, long n, int ntypes, double *out) {
  try {
    paramfile params = make_params(keys, vals, nkv);
    if (!params.param_present("outfile")) params.setParam("outfile", std::string("ref"));
    sceneMaker sm(params);
    particle_sim *p = static_cast<particle_sim *>(particles);
    std::vector<particle_sim> v(p, p + n);
    (sm.*member(NormalizeTag()))(v, false);
    std::copy(v.begin(), v.end(), p);
    // read back as text: the values may be infinite, which stringToData<double>
    // does not parse
    auto num = [&](const std::string &k) {
      return std::strtod(params.find<std::string>(k).c_str(), nullptr);
    };
    for (int t = 0; t < ntypes; ++t) {
      const std::string s = dataToString(t);
      out[4 * t + 0] = num("range_min" + s);
      out[4 * t + 1] = num("range_max" + s);
      out[4 * t + 2] = num("clamp_min" + s);
      out[4 * t + 3] = num("clamp_max" + s);
    }
    return 0;
  } catch (...) {
    return -1;
  }
}

// The output step of splotch/splotch.cc:295-323: LS_Image from an x-major
// image, written as pictype 0 (TGA), 2 (PPM) or 3 (run-length TGA).
int ref_write_image(const float *pic, int xres, int yres, int pictype, const char *path) {
  try {
    LS_Image img(xres, yres);
    for (int i = 0; i < xres; ++i)
      for (int j = 0; j < yres; ++j) {
        const float *s = pic + ((size_t)i * yres + j) * 3;
        img.put_pixel(i, j, Colour(s[0], s[1], s[2]));
      }
    switch (pictype) {
      case 0: img.write_TGA(path); break;
      case 2: img.write_PPM(path); break;
      case 3: img.write_TGA_rle(path); break;
      default: return -2;
    }
    return 0;
  } catch (...) {
    return -1;
  }
}

}  // extern "C"
