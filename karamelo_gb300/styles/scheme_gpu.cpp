// scheme_gpu.cpp -- SchemeGPU and the setup of the tlmpm/gpu and ulmpm/gpu
// method styles: Karamelo's run loop over the C ABI of libkmpm.so.
//
// Built against Karamelo's own headers with the styles registered in its
// style_method.h / style_scheme.h registries (karamelo_gb300/styles/Makefile).
#include "scheme_gpu.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <unistd.h>
#include <vector>

#include "damage.h"
#include "domain.h"
#include "eos.h"
#include "error.h"
#include "fix.h"
#include "grid.h"
#include "group.h"
#include "input.h"
#include "kmpm.h"
#include "material.h"
#include "method.h"
#include "modify.h"
#include "mpm.h"
#include "output.h"
#include "solid.h"
#include "strength.h"
#include "temperature.h"
#include "tlmpm_gpu.h"
#include "ulmpm_gpu.h"
#include "update.h"
#include "var.h"

using namespace std;

namespace {

// The parameters a law serialises through its public write_restart()
// (Material::write_restart, src/material.cpp:384-496), read back as doubles.
template <typename Law> vector<double> law_params(Law *law) {
  char path[] = "/tmp/kmpm_law_XXXXXX";
  const int fd = mkstemp(path);
  if (fd < 0) return {};
  close(fd);
  {
    ofstream of(path, ios::binary);
    law->write_restart(&of);
  }
  vector<double> p;
  ifstream in(path, ios::binary);
  double v;
  while (in.read(reinterpret_cast<char *>(&v), sizeof(double))) p.push_back(v);
  unlink(path);
  return p;
}

const char *GPU_SCHEME_MISSING =
    "A tlmpm/gpu or ulmpm/gpu method runs its steps in the GPU scheme, but a scheme() command given after "
    "method() installed a CPU scheme: use scheme(usl/gpu), scheme(musl/gpu) or scheme(usf/gpu), or give "
    "scheme() before method().\n";

}  // namespace

// ---------------------------------------------------------------- methods
void TLMPMGPU::setup(vector<string> args) {
  TLMPM::setup(args);
  // the reference's dumps, grids and solids test the method's name
  // (e.g. src/dump_particle.cpp:98): the GPU style answers to "tlmpm"
  update->method_type = "tlmpm";
  SchemeGPU::install(mpm);
}

void TLMPMGPU::compute_grid_weight_functions_and_gradients() { error->all(FLERR, GPU_SCHEME_MISSING); }

void ULMPMGPU::setup(vector<string> args) {
  ULMPM::setup(args);
  update->method_type = "ulmpm";
  SchemeGPU::install(mpm);
}

void ULMPMGPU::compute_grid_weight_functions_and_gradients() { error->all(FLERR, GPU_SCHEME_MISSING); }

// ---------------------------------------------------------------- scheme
SchemeGPU::SchemeGPU(MPM *mpm, const string &scheme) : Scheme(mpm), scheme_(scheme) {}

SchemeGPU::~SchemeGPU() {
  if (ctx_) kmpm_destroy(ctx_);
}

void SchemeGPU::install(MPM *mpm) {
  Update *u = mpm->update;
  string base = u->scheme_style;
  if (base.size() > 4 && base.compare(base.size() - 4, 4, "/gpu") == 0) base.resize(base.size() - 4);
  if (base != "usl" && base != "musl" && base != "usf")
    mpm->error->all(FLERR, "The GPU method runs the usl, musl or usf scheme, not " + u->scheme_style + ".\n");
  u->scheme = new SchemeGPU(mpm, base);
}

void SchemeGPU::setup() { output->setup(); }

void SchemeGPU::check(int rc, const char *what) {
  if (rc >= 0) return;
  string msg = ctx_ ? kmpm_last_error(ctx_) : "";
  if (msg.empty()) {  // before a context exists: the status code's meaning (include/kmpm.h)
    msg = rc == KMPM_ERR_ARG ? "bad argument or unsupported combination"
          : rc == KMPM_ERR_CUDA ? "CUDA runtime failure or no CUDA device"
          : "status " + to_string(rc);
  }
  error->one(FLERR, string(what) + ": " + msg + "\n");
}

int SchemeGPU::material_id(const Mat *m) {
  const int k = (int)(m - material->materials.data());
  if (k < 0 || k >= (int)mat_ids_.size()) error->all(FLERR, "GPU scheme: a solid's material is unknown.\n");
  return mat_ids_[k];
}

int SchemeGPU::grid_id(Grid *g) {
  auto it = grid_ids_.find(g);
  if (it != grid_ids_.end()) return it->second;
  if (g->x0.empty()) error->all(FLERR, "GPU scheme: a grid has no nodes.\n");
  const double lo[3] = {g->x0[0][0], g->x0[0][1], g->x0[0][2]};
  const int n[3] = {g->nx, g->ny, g->nz}, ng[3] = {g->nx_global, g->ny_global, g->nz_global};
  const int id = kmpm_add_grid(ctx_, lo, g->cellsize, n, ng);
  check(id, "kmpm_add_grid");
  grid_ids_[g] = id;
  return id;
}

// The value of a fix's expression at time t (the reference evaluates it with
// the `time` variable, src/fix_velocity_nodes.cpp:66-108).
double SchemeGPU::eval_at(const string &expr, double t) {
  Var saved = (*input->vars)["time"];
  (*input->vars)["time"] = Var("time", t);
  const double v = input->parsev(expr).result(mpm);
  (*input->vars)["time"] = saved;
  return v;
}

void SchemeGPU::upload() {
  if (domain->solids.empty()) error->all(FLERR, "GPU scheme: no solid was defined.\n");
  kmpm_params p{};
  p.method = update->method->is_TL ? KMPM_TLMPM : KMPM_ULMPM;
  p.scheme = scheme_ == "usl" ? KMPM_USL : (scheme_ == "usf" ? KMPM_USF : KMPM_MUSL);
  switch (update->shape_function) {
    case Update::ShapeFunctions::LINEAR: p.basis = KMPM_BASIS_LINEAR; break;
    case Update::ShapeFunctions::CUBIC_SPLINE: p.basis = KMPM_BASIS_CUBIC; break;
    case Update::ShapeFunctions::QUADRATIC_SPLINE: p.basis = KMPM_BASIS_QUADRATIC; break;
    default: p.basis = KMPM_BASIS_BERNSTEIN; break;
  }
  switch (update->sub_method_type) {
    case Update::SubMethodType::APIC: p.transfer = KMPM_TRANSFER_APIC; break;
    case Update::SubMethodType::AFLIP: p.transfer = KMPM_TRANSFER_AFLIP; break;
    case Update::SubMethodType::ASFLIP: p.transfer = KMPM_TRANSFER_ASFLIP; break;
    case Update::SubMethodType::MLS: p.transfer = KMPM_TRANSFER_MLS; break;
    default: p.transfer = KMPM_TRANSFER_FLIP; break;
  }
  p.dim = domain->dimension;
  p.pic_flip = update->PIC_FLIP;
  p.thermal = update->method->temp ? 1 : 0;
  p.dt = update->dt;
  p.dt_factor = update->dt_factor;
  p.dt_constant = update->dt_constant ? 1 : 0;
  for (int d = 0; d < 3; d++) {
    p.boxlo[d] = domain->boxlo[d];
    p.boxhi[d] = domain->boxhi[d];
  }
  p.precision = KMPM_PREC_FP32;
  p.track_strain = 1;  // Solid::strain_el, for the strain-energy fix and the dumps
  p.autotune = 1;
  p.axisymmetric = domain->axisymmetric ? 1 : 0;

  // everything is checked before the device is touched: unsupported
  // materials, laws and fixes stop the run here
  vector<kmpm_material> mats;
  // materials (Material::add_material, src/material.cpp:249-380): the laws'
  // parameters in the C ABI's order, from their restart serialisation
  for (Mat &m : material->materials) {
    kmpm_material km{};
    km.damage = -1;
    km.temp = -1;
    km.rho0 = m.rho0;
    km.E = m.E;
    km.nu = m.nu;
    km.cp = m.cp;
    km.kappa = m.kappa;
    if (m.rigid || m.type == Material::RIGID) error->all(FLERR, "GPU scheme: rigid materials are not supported.\n");
    if (m.type == Material::LINEAR) km.type = KMPM_MAT_LINEAR;
    else if (m.type == Material::NEO_HOOKEAN) km.type = KMPM_MAT_NEO_HOOKEAN;
    else {
      km.type = KMPM_MAT_EOS_STRENGTH;
      const vector<double> e = law_params(m.eos);
      const string es = m.eos->style;
      if (es == "linear" && e.size() >= 2) {
        km.eos = 0;
        km.eos_p[0] = e[0]; km.eos_p[1] = e[1];
      } else if (es == "shock" && e.size() >= 9) {  // serialised rho0 K c0 S Gamma Tr cv Q1 Q2
        km.eos = 1;
        const int order[9] = {0, 1, 2, 3, 4, 6, 5, 7, 8};  // -> rho0 K c0 S Gamma cv Tr Q1 Q2
        for (int k = 0; k < 9; k++) km.eos_p[k] = e[order[k]];
      } else if (es == "fluid" && e.size() >= 3) {
        km.eos = 2;
        for (int k = 0; k < 3; k++) km.eos_p[k] = e[k];
      } else {
        error->all(FLERR, "GPU scheme: EOS style " + es + " is not supported.\n");
      }
      const vector<double> s = law_params(m.strength);
      const string ss = m.strength->style;
      if (ss == "linear" && s.size() >= 1) {
        km.strength = 0;
        km.str_p[0] = s[0];
      } else if (ss == "plastic" && s.size() >= 2) {
        km.strength = 1;
        km.str_p[0] = s[0]; km.str_p[1] = s[1];
      } else if (ss == "johnson_cook" && s.size() >= 9) {  // serialised G A B n m epsdot0 C Tr Tm
        km.strength = 2;
        const int order[9] = {0, 1, 2, 3, 5, 6, 4, 7, 8};   // -> G A B n epsdot0 C m Tr Tm
        for (int k = 0; k < 9; k++) km.str_p[k] = s[order[k]];
      } else if (ss == "swift" && s.size() >= 5) {
        km.strength = 3;
        for (int k = 0; k < 5; k++) km.str_p[k] = s[k];
      } else if (ss == "fluid" && s.size() >= 1) {
        km.strength = 4;
        km.str_p[0] = s[0];
      } else {
        error->all(FLERR, "GPU scheme: strength style " + ss + " is not supported.\n");
      }
      if (m.damage) {
        const vector<double> dm = law_params(m.damage);
        if (m.damage->style != "damage_johnson_cook" || dm.size() < 8)
          error->all(FLERR, "GPU scheme: damage style " + m.damage->style + " is not supported.\n");
        km.damage = 0;
        for (int k = 0; k < 8; k++) km.dam_p[k] = dm[k];
      }
      if (m.temp) {
        const vector<double> t = law_params(m.temp);  // serialised chi kappa cp alpha T0 Tm
        if (m.temp->style != "plastic_work" || t.size() < 6)
          error->all(FLERR, "GPU scheme: temperature style " + m.temp->style + " is not supported.\n");
        km.temp = 0;
        const int order[6] = {0, 2, 1, 3, 4, 5};  // -> chi cp kappa alpha T0 Tm
        for (int k = 0; k < 6; k++) km.temp_p[k] = t[order[k]];
      }
    }
    mats.push_back(km);
  }
  lower_fixes(true);

  check(kmpm_create(&p, &ctx_), "kmpm_create");
  for (const kmpm_material &km : mats) {
    const int id = kmpm_add_material(ctx_, &km);
    check(id, "kmpm_add_material");
    mat_ids_.push_back(id);
  }

  // initial_velocity_particles: its step-1 initial_integrate
  // (src/fix_initial_velocity_particles.cpp:99-163) on the host particles,
  // before they are uploaded
  for (Fix *f : modify->fix) {
    if (f->style != "initial_velocity_particles") continue;
    const int gb = f->groupbit, gs = group->solid[f->igroup];
    for (size_t k = 0; k < 3 && 3 + k < f->args.size(); k++) {
      if (f->args[3 + k] == "NULL") continue;
      const double val = input->parsev(f->args[3 + k]).result(mpm);
      for (int is = 0; is < (int)domain->solids.size(); is++) {
        if (gs != -1 && gs != is) continue;
        Solid *s = domain->solids[is];
        for (int i = 0; i < s->np_local; i++)
          if (s->mask[i] & gb) s->v[i][k] = val;
      }
    }
    lowered_.push_back(f->id);
  }

  // grids and solids (Grid::init, Solid::populate): Eigen::Vector3d arrays
  // are three contiguous doubles per particle
  for (Solid *s : domain->solids) {
    const int gid = grid_id(update->method->is_TL ? s->grid : domain->grid);
    const double T0 = s->T.empty() ? 0.0 : s->T[0];
    const int sid = kmpm_add_solid(ctx_, gid, material_id(s->mat), s->np_local, s->x0[0].data(), s->x[0].data(),
                                   s->v[0].data(), s->mass.data(), s->vol0.data(), T0);
    check(sid, "kmpm_add_solid");
    check(kmpm_set_np_per_cell(ctx_, sid, s->np_per_cell), "kmpm_set_np_per_cell");
    solid_ids_.push_back(sid);
  }
  lower_fixes(false);
}

// The fixes not yet on the device (a script may add fixes between runs, as
// the Taylor-bar script adds its wall after run(1)).  check_only: validate
// the styles and value expressions without a device context.
void SchemeGPU::lower_fixes(bool check_only) {
  for (Fix *f : modify->fix) {
    if (find(lowered_.begin(), lowered_.end(), f->id) != lowered_.end()) continue;
    const string &st = f->style;
    const int gb = f->groupbit, gs = group->solid[f->igroup];
    if (st == "velocity_nodes" || st == "body_force") {
      int set[3] = {0, 0, 0};
      double coef[12] = {0};
      for (int k = 0; k < 3; k++) {
        if (3 + k >= (int)f->args.size() || f->args[3 + k] == "NULL" || k >= domain->dimension) continue;
        set[k] = 1;
        const string &ex = f->args[3 + k];
        // c0 + c1 time: fitted at t = 0 and 1, checked at three more times
        const double v0 = eval_at(ex, 0.0), v1 = eval_at(ex, 1.0);
        coef[4 * k] = v0;
        coef[4 * k + 1] = st == "velocity_nodes" ? v1 - v0 : 0.0;
        for (double t : {0.25, 2.5, 7.0}) {
          const double want = eval_at(ex, t), got = v0 + coef[4 * k + 1] * t;
          if (std::fabs(want - got) > 1e-12 * std::max(1.0, std::fabs(want)))
            error->all(FLERR, "GPU scheme: fix " + f->id + ": the value " + ex +
                                  (st == "body_force" ? " must be constant.\n" : " must be constant or linear in time.\n"));
        }
      }
      if (check_only) continue;
      const int kind = st == "velocity_nodes" ? KMPM_FIX_VELOCITY_NODES : KMPM_FIX_BODY_FORCE;
      // the group's node mask on every grid it covers (one per solid for
      // TLMPM; the shared grid once per solid for ULMPM, as
      // FixBodyforce applies it, src/fix_body_force.cpp:118-140)
      for (int is = 0; is < (int)domain->solids.size(); is++) {
        if (gs != -1 && gs != is) continue;
        Grid *g = update->method->is_TL ? domain->solids[is]->grid : domain->grid;
        vector<unsigned char> mask(g->mask.size());
        for (size_t n = 0; n < mask.size(); n++) mask[n] = (g->mask[n] & gb) ? 1 : 0;
        check(kmpm_add_fix(ctx_, kind, grid_id(g), mask.data(), set, coef), "kmpm_add_fix");
        if (!update->method->is_TL && kind == KMPM_FIX_VELOCITY_NODES) break;  // one shared grid
      }
    } else if (st == "kinetic_energy" || st == "strain_energy") {
      if (check_only) continue;
      energy_fix_.push_back(f->id);
      energy_kind_.push_back(st == "kinetic_energy" ? 0 : 1);
    } else if (st == "contact/minimize_penetration" || st == "contact/hertz") {
      if (f->args.size() < 4) error->all(FLERR, "GPU scheme: fix " + f->id + " needs two solids.\n");
      if (check_only) continue;
      const int s1 = domain->find_solid(f->args[2]), s2 = domain->find_solid(f->args[3]);
      const double mu = st == "contact/minimize_penetration" && f->args.size() > 4
                            ? input->parsev(f->args[4]).result(mpm) : 0.0;
      check(kmpm_add_contact(ctx_, st == "contact/hertz" ? KMPM_CONTACT_HERTZ : KMPM_CONTACT_MIN_PENETRATION,
                             solid_ids_[s1], solid_ids_[s2], mu),
            "kmpm_add_contact");
    } else if (st != "initial_velocity_particles") {
      error->all(FLERR, "GPU scheme: fix style " + st + " is not supported on the GPU (no CPU fallback).\n");
    }
    if (!check_only) lowered_.push_back(f->id);
  }
}

// The particle fields Output::write may read (dumps, computes, logs), into
// the host solids.  For TLMPM the stress arrives rotated (R sigma R^T) with
// R set to the identity, so the dump's R sigma R^T (src/dump_particle.cpp:98-102)
// writes it unchanged.
void SchemeGPU::download() {
  const bool tl = update->method->is_TL;
  for (size_t is = 0; is < domain->solids.size(); is++) {
    Solid *s = domain->solids[is];
    const int sid = solid_ids_[is], n = s->np_local;
    vector<double> buf((size_t)n * 9);
    check(kmpm_download_particles(ctx_, sid, KMPM_P_X, s->x[0].data()), "kmpm_download_particles");
    check(kmpm_download_particles(ctx_, sid, KMPM_P_V, s->v[0].data()), "kmpm_download_particles");
    auto mat9 = [&](int field, vector<Eigen::Matrix3d> &dst) {
      if (dst.size() < (size_t)n) return;
      check(kmpm_download_particles(ctx_, sid, field, buf.data()), "kmpm_download_particles");
      for (int i = 0; i < n; i++)
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++) dst[i](a, b) = buf[9 * i + 3 * a + b];  // row-major in the ABI
    };
    auto vec1 = [&](int field, vector<double> &dst) {
      if (dst.size() < (size_t)n) return;
      check(kmpm_download_particles(ctx_, sid, field, dst.data()), "kmpm_download_particles");
    };
    mat9(tl ? KMPM_P_SIGMA_ROT : KMPM_P_SIGMA, s->sigma);
    if (tl)
      for (int i = 0; i < n && i < (int)s->R.size(); i++) s->R[i].setIdentity();
    mat9(KMPM_P_F, s->F);
    mat9(KMPM_P_STRAIN_EL, s->strain_el);
    vec1(KMPM_P_EPS_P, s->eff_plastic_strain);
    vec1(KMPM_P_EPSDOT_P, s->eff_plastic_strain_rate);
    vec1(KMPM_P_DAMAGE, s->damage);
    vec1(KMPM_P_DAMAGE_INIT, s->damage_init);
    vec1(KMPM_P_J, s->J);
    vec1(KMPM_P_VOL, s->vol);
    if (update->method->temp) vec1(KMPM_P_T, s->T);
  }
}

// Scheme::run: the steps between output steps run on the GPU in one call
// each; the run's condition, the output schedule and the time variables are
// Karamelo's own (Run::command, RunTime::command, Output::write).
void SchemeGPU::run(Var condition) {
  if (!dynamic_cast<TLMPMGPU *>(update->method) && !dynamic_cast<ULMPMGPU *>(update->method))
    error->all(FLERR, "Scheme " + scheme_ + "/gpu needs the tlmpm/gpu or ulmpm/gpu method.\n");
  if (!ctx_) upload();
  else lower_fixes(false);
  output->write(update->ntimestep);
  while ((bool)condition.result(mpm)) {
    bigint until = output->next;
    if (update->maxtime == -1) until = std::min<bigint>(until, update->laststep);
    const int n = (int)std::max<bigint>(1, until - update->ntimestep);
    if (update->maxtime == -1) check(kmpm_run(ctx_, n), "kmpm_run");
    else check(kmpm_run_until(ctx_, n, update->maxtime, nullptr), "kmpm_run_until");  // run_time
    double t = 0, dt = 0;
    long long step = 0;
    check(kmpm_scalars(ctx_, &t, &dt, &step), "kmpm_scalars");
    update->atime = t;
    update->atimestep = step;
    update->dt = dt;
    update->ntimestep = step;
    (*input->vars)["time"] = Var("time", t);
    (*input->vars)["timestep"] = Var("timestep", (double)step);
    (*input->vars)["dt"] = Var("dt", dt);
    const bool out = step == output->next || step == update->laststep ||
                     (update->maxtime != -1 && t >= update->maxtime);
    if (out) {
      download();
      if (!energy_fix_.empty()) {
        double e[2];
        check(kmpm_energy(ctx_, e), "kmpm_energy");
        for (size_t k = 0; k < energy_fix_.size(); k++)
          (*input->vars)[energy_fix_[k] + "_s"] = Var(energy_fix_[k] + "_s", e[energy_kind_[k]]);
      }
      output->write(step);
    }
    if (update->maxtime != -1 && t >= update->maxtime) {
      update->nsteps = (int)step;
      break;
    }
  }
}
