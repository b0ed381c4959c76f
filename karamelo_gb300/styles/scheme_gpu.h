/* scheme_gpu.h -- the scheme that runs whole Karamelo time steps on the GPU.
 *
 * SchemeGPU replaces USL::run / MUSL::run / USF::run (src/usl.cpp:34-94,
 * src/musl.cpp:34-95, src/usf.cpp:34-95).  On its first run it uploads the
 * state that Karamelo's host classes built (Domain, Grid::init,
 * Solid::populate, Material, Group, Fix) into a libkmpm context, then runs the
 * steps on the GPU in batches that end at the output steps; before each
 * Output::write it downloads the particle fields the dumps, computes and
 * logs read and sets the time variables.  The method styles tlmpm/gpu and
 * ulmpm/gpu install it with the scheme current at their setup; the styles
 * usl/gpu, musl/gpu and usf/gpu select it explicitly for scripts that set the
 * scheme after the method.
 *
 * Fixes lowered to the device: velocity_nodes (values c0 + c1 time, checked
 * at five times), body_force (constant), initial_velocity_particles (applied
 * to the particles on the host before the upload, as its step-1
 * initial_integrate would), the two contact fixes, and the kinetic / strain
 * energy fixes (their *_s variables from kmpm_energy).  Any other fix stops
 * the run with an error: there is no CPU fallback. */
#ifdef SCHEME_CLASS

SchemeStyle(usl/gpu, SchemeGPUUSL)
SchemeStyle(musl/gpu, SchemeGPUMUSL)
SchemeStyle(usf/gpu, SchemeGPUUSF)

#else

#ifndef KMPM_STYLE_SCHEME_GPU_H
#define KMPM_STYLE_SCHEME_GPU_H

#include <map>
#include <string>
#include <vector>

#include "scheme.h"

struct kmpm_ctx;

class SchemeGPU : public Scheme {
 public:
  SchemeGPU(class MPM *mpm, const std::string &scheme);
  ~SchemeGPU();
  void setup() override;
  void run(class Var) override;

  // installs a SchemeGPU in place of update->scheme, for the scheme style
  // current at the call (usl, musl or usf)
  static void install(class MPM *mpm);

 private:
  void upload();
  void lower_fixes(bool check_only);
  void download();
  void check(int rc, const char *what);
  int material_id(const class Mat *m);
  int grid_id(class Grid *g);
  double eval_at(const std::string &expr, double t);

  std::string scheme_;
  kmpm_ctx *ctx_ = nullptr;
  std::vector<int> mat_ids_;
  std::map<class Grid *, int> grid_ids_;
  std::vector<int> solid_ids_;
  std::vector<std::string> lowered_;     // fixes already on the device
  std::vector<std::string> energy_fix_;  // ids of kinetic / strain energy fixes, with their style
  std::vector<int> energy_kind_;
};

class SchemeGPUUSL : public SchemeGPU {
 public:
  SchemeGPUUSL(class MPM *mpm) : SchemeGPU(mpm, "usl") {}
};
class SchemeGPUMUSL : public SchemeGPU {
 public:
  SchemeGPUMUSL(class MPM *mpm) : SchemeGPU(mpm, "musl") {}
};
class SchemeGPUUSF : public SchemeGPU {
 public:
  SchemeGPUUSF(class MPM *mpm) : SchemeGPU(mpm, "usf") {}
};

#endif
#endif
