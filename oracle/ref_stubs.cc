// ref_stubs.cc -- TEST INFRASTRUCTURE ONLY.  splotch/scenemaker.cc (compiled
// into oracle/_ref for sceneMaker::particle_normalize) also references the
// snapshot readers and the mesh "booster"; the harness never reads files or
// builds meshes, so those symbols are defined here as functions that fail.
#include "booster/mesh_vis.h"
#include "cxxsupport/error_handling.h"
#include "reader/reader.h"

namespace {
[[noreturn]] void absent(const char *what) {
  planck_fail(std::string(what) + " is not part of the oracle harness");
}
}  // namespace

void gadget_reader(paramfile &, int, std::vector<particle_sim> &, std::vector<MyIDType> &,
                   std::vector<vec3f> &, int, double &, double &) {
  absent("gadget_reader");
}
void gadget_millenium_reader(paramfile &, std::vector<particle_sim> &, int, double *) {
  absent("gadget_millenium_reader");
}
void bin_reader_tab(paramfile &, std::vector<particle_sim> &) { absent("bin_reader_tab"); }
void bin_reader_block(paramfile &, std::vector<particle_sim> &) { absent("bin_reader_block"); }
void mesh_reader(paramfile &, std::vector<particle_sim> &) { absent("mesh_reader"); }
void tipsy_reader(paramfile &, std::vector<particle_sim> &, std::vector<MyIDType> &, int) {
  absent("tipsy_reader");
}
void ramses_reader(paramfile &, std::vector<particle_sim> &) { absent("ramses_reader"); }
void ascii_reader(paramfile &, std::vector<particle_sim> &) { absent("ascii_reader"); }
void mesh_creator(std::vector<particle_sim> &, Mesh_vis **, Mesh_dim *) {
  absent("mesh_creator");
}
void p_selector(std::vector<particle_sim> &, Mesh_vis *, Mesh_dim, std::vector<particle_sim> &) {
  absent("p_selector");
}
void randomizer(std::vector<particle_sim> &, Mesh_vis *, Mesh_dim) { absent("randomizer"); }
void m_rotation(paramfile &, Mesh_vis **, Mesh_dim, const vec3 &, const vec3 &, vec3) {
  absent("m_rotation");
}
