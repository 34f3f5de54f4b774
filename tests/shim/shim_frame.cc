// shim_frame.cc -- runs the host_rendering() drop-in's logic
// (splotch_gb300/shim/host_rendering_impl.h) on the GPU without the Splotch
// tree: minimal stand-ins for paramfile, render_context, the colour maps, the
// image and particle_sim, read from files the test writes.
//
//   shim_frame <dir>
//     <dir>/params.txt     key=value lines (the paramfile)
//     <dir>/context.bin    campos, lookat, sky, centerpos (3 doubles each),
//                          b_brightness (float), npal (int32), then per
//                          palette n (int32), n doubles (x), 3n floats (rgb)
//     <dir>/particles.bin  n (int64), n particle_sim records (36 bytes)
//   writes <dir>/pic.bin (x-major xres*yres*3 floats), <dir>/particles_out.bin
//   (the caller's vector after the call: int64 n, records) and
//   <dir>/params_out.txt (the paramfile after the call: defaults inserted).
// Exit status 0, or 3 with the error's message on stdout.
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "host_rendering_impl.h"

namespace {

struct Vec {
  double x, y, z;
};
struct Col {
  float r, g, b;
};
struct Particle {  // particle_sim's 36-byte layout
  Col e;
  float x, y, z, r, I;
  unsigned short type;
  bool active;
};

struct Palette {
  std::vector<double> x;
  std::vector<Col> c;
  size_t size() const { return x.size(); }
  double getX(size_t k) const { return x[k]; }
  Col getY(size_t k) const { return c[k]; }
};

struct Pic {
  std::vector<Col> d;
  size_t n1 = 0, n2 = 0;
  size_t size1() const { return n1; }
  size_t size2() const { return n2; }
  void alloc(size_t a, size_t b) {
    n1 = a;
    n2 = b;
    d.assign(a * b, Col{0.f, 0.f, 0.f});
  }
  Col *operator[](size_t i) { return &d[i * n2]; }
};

struct Context {
  Vec campos, lookat, sky, centerpos;
  float b_brightness = 1.f;
  long npart = 0;
  std::vector<Palette> amap;
  Pic pic;
};

// paramfile::find semantics: a missing key with a default is inserted.
struct Params {
  std::map<std::string, std::string> kv;
  bool param_present(const std::string &k) const { return kv.count(k) != 0; }
  template <class T>
  static T conv(const std::string &s);
  template <class T>
  static std::string str(const T &v) {
    std::ostringstream o;
    o << v;
    return o.str();
  }
  template <class T>
  T find(const std::string &k) const {
    auto it = kv.find(k);
    if (it == kv.end()) throw std::runtime_error("Cannot find the key '" + k + "'.");
    return conv<T>(it->second);
  }
  template <class T>
  T find(const std::string &k, const T &def) {
    auto it = kv.find(k);
    if (it == kv.end()) {
      kv[k] = str(def);
      return def;
    }
    return conv<T>(it->second);
  }
};
template <>
int Params::conv<int>(const std::string &s) { return std::stoi(s); }
template <>
float Params::conv<float>(const std::string &s) { return std::stof(s); }
template <>
double Params::conv<double>(const std::string &s) { return std::stod(s); }
template <>
std::string Params::conv<std::string>(const std::string &s) { return s; }
template <>
bool Params::conv<bool>(const std::string &s) {
  if (s == "T" || s == "t" || s == "true" || s == "y" || s == ".true.") return true;
  if (s == "F" || s == "f" || s == "false" || s == "n" || s == ".false.") return false;
  throw std::runtime_error("conversion error in stringToData<bool>(\"" + s + "\")");
}
template <>
std::string Params::str<bool>(const bool &v) { return v ? "T" : "F"; }

struct TestEnv {
  using Params = ::Params;
  using Particle = ::Particle;
  using Context = ::Context;
  [[noreturn]] static void fail(const std::string &msg) { throw std::runtime_error(msg); }
  static void timer_push(const char *) {}
  static void timer_pop(const char *) {}
  static void checkbbox(std::vector<Particle> &, Params &) { fail("bbox is not supported here"); }
  static void checkrth(float, int, std::vector<Particle> &, Params &) {
    fail("rth is not supported here");
  }
};

template <class T>
void get(std::ifstream &f, T &v) {
  f.read(reinterpret_cast<char *>(&v), sizeof(T));
  if (!f) throw std::runtime_error("short input file");
}

}  // namespace

int main(int argc, char **argv) {
  static_assert(sizeof(Particle) == 36, "particle_sim layout");
  if (argc != 2) {
    std::printf("usage: shim_frame <dir>\n");
    return 2;
  }
  const std::string dir = argv[1];
  try {
    Params params;
    {
      std::ifstream f(dir + "/params.txt");
      std::string line;
      while (std::getline(f, line)) {
        const size_t eq = line.find('=');
        if (eq != std::string::npos) params.kv[line.substr(0, eq)] = line.substr(eq + 1);
      }
    }
    Context rc;
    {
      std::ifstream f(dir + "/context.bin", std::ios::binary);
      Vec *v[4] = {&rc.campos, &rc.lookat, &rc.sky, &rc.centerpos};
      for (Vec *p : v) {
        get(f, p->x);
        get(f, p->y);
        get(f, p->z);
      }
      get(f, rc.b_brightness);
      int32_t npal = 0;
      get(f, npal);
      rc.amap.resize(npal);
      for (Palette &pal : rc.amap) {
        int32_t n = 0;
        get(f, n);
        pal.x.resize(n);
        pal.c.resize(n);
        for (auto &x : pal.x) get(f, x);
        for (auto &c : pal.c) {
          get(f, c.r);
          get(f, c.g);
          get(f, c.b);
        }
      }
    }
    std::vector<Particle> particles;
    {
      std::ifstream f(dir + "/particles.bin", std::ios::binary);
      int64_t n = 0;
      get(f, n);
      particles.resize(n);
      if (n) f.read(reinterpret_cast<char *>(particles.data()), n * sizeof(Particle));
      if (!f) throw std::runtime_error("short particle file");
    }
    rc.npart = (long)particles.size();
    spl_shim::host_rendering<TestEnv>(params, particles, rc);
    {
      std::ofstream f(dir + "/pic.bin", std::ios::binary);
      f.write(reinterpret_cast<const char *>(rc.pic.d.data()), rc.pic.d.size() * sizeof(Col));
    }
    {
      std::ofstream f(dir + "/particles_out.bin", std::ios::binary);
      const int64_t n = (int64_t)particles.size();
      f.write(reinterpret_cast<const char *>(&n), 8);
      if (n) f.write(reinterpret_cast<const char *>(particles.data()), n * sizeof(Particle));
    }
    {
      std::ofstream f(dir + "/params_out.txt");
      for (const auto &kv : params.kv) f << kv.first << "=" << kv.second << "\n";
    }
  } catch (const std::exception &e) {
    std::printf("%s\n", e.what());
    return 3;
  }
  std::printf("rendered\n");
  return 0;
}
