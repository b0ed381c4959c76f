// ref_harness.cpp -- drives the reference's own MPM object (every src/*.cpp
// of the Karamelo tree but main.cpp, compiled unmodified; oracle/Makefile)
// through an input script, and writes the particle state and chosen
// variables at full FP64 precision.  Test infrastructure: it makes the golden
// fixtures of the parity tests (tests/golden/make_ref_golden.py); nothing in
// the product runs it.
//
//   ref_harness <script> <out.bin>
//
// The script is Karamelo's input language, executed line by line through the
// reference's own Input::parsev (as Input::file does: text after '#' is
// dropped).  Two harness directives, written as comments so that the same
// script also runs in the plain reference, append records to out.bin:
//   #@state <label>          every solid's particles
//   #@vars <label> v1 v2 ... the named input variables (Var::result)
// Record layout (little-endian): char label[32], int64 step, double time, dt;
// then for a state record int32 nsolid and per solid int64 np followed by np
// rows of STATE_COLS doubles; for a vars record int32 nvar and nvar doubles.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include <mpi.h>

#include "domain.h"
#include "input.h"
#include "mpm.h"
#include "solid.h"
#include "update.h"
#include "var.h"

namespace {

// ptag, x0 (3), x (3), v (3), the dumped stress (9: R sigma R^T for TLMPM,
// sigma for ULMPM, as Dump particle writes it, src/dump_particle.cpp:93-102),
// F (9), eps_p, eps_p rate, damage, damage_init, T, J, vol, mass
constexpr int STATE_COLS = 1 + 3 + 3 + 3 + 9 + 9 + 8;

void put_header(std::ofstream &o, const std::string &label, MPM *mpm) {
  char lab[32] = {0};
  std::strncpy(lab, label.c_str(), 31);
  o.write(lab, 32);
  const int64_t step = (int64_t)mpm->update->ntimestep;
  const double time = mpm->update->atime, dt = mpm->update->dt;
  o.write((const char *)&step, 8);
  o.write((const char *)&time, 8);
  o.write((const char *)&dt, 8);
}

void write_state(std::ofstream &o, const std::string &label, MPM *mpm) {
  put_header(o, label, mpm);
  const int32_t ns = (int32_t)mpm->domain->solids.size();
  o.write((const char *)&ns, 4);
  const bool tl = mpm->update->method_type == "tlmpm";
  for (Solid *s : mpm->domain->solids) {
    const int64_t np = (int64_t)s->np_local;
    o.write((const char *)&np, 8);
    std::vector<double> row(STATE_COLS);
    for (int64_t i = 0; i < np; i++) {
      int k = 0;
      row[k++] = (double)s->ptag[i];
      for (int d = 0; d < 3; d++) row[k++] = s->x0[i][d];
      for (int d = 0; d < 3; d++) row[k++] = s->x[i][d];
      for (int d = 0; d < 3; d++) row[k++] = s->v[i][d];
      const Eigen::Matrix3d sg = tl ? Eigen::Matrix3d(s->R[i] * s->sigma[i] * s->R[i].transpose()) : s->sigma[i];
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) row[k++] = sg(a, b);
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) row[k++] = s->F[i](a, b);
      // the reference allocates some fields only when a law uses them (T only
      // for thermo-mechanical runs): an absent field is written as 0
      auto at = [i](const std::vector<double> &f) { return (size_t)i < f.size() ? f[i] : 0.0; };
      row[k++] = at(s->eff_plastic_strain);
      row[k++] = at(s->eff_plastic_strain_rate);
      row[k++] = at(s->damage);
      row[k++] = at(s->damage_init);
      row[k++] = at(s->T);
      row[k++] = at(s->J);
      row[k++] = at(s->vol);
      row[k++] = at(s->mass);
      o.write((const char *)row.data(), sizeof(double) * STATE_COLS);
    }
  }
}

void write_vars(std::ofstream &o, const std::string &label, const std::vector<std::string> &names, MPM *mpm) {
  put_header(o, label, mpm);
  const int32_t nv = (int32_t)names.size();
  o.write((const char *)&nv, 4);
  for (const auto &n : names) {
    double v = 0.0;
    auto it = mpm->input->vars->find(n);
    if (it != mpm->input->vars->end()) v = it->second.result();
    else std::fprintf(stderr, "ref_harness: no variable %s\n", n.c_str());
    o.write((const char *)&v, 8);
  }
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: ref_harness <script> <out.bin>\n");
    return 2;
  }
  std::ifstream in(argv[1]);
  if (!in) {
    std::fprintf(stderr, "ref_harness: cannot open %s\n", argv[1]);
    return 2;
  }
  std::ofstream out(argv[2], std::ios::binary);
  // the MPM constructor wants "-i <script>" and opens it (src/mpm.cpp:59-93);
  // the lines are then fed to Input::parsev here instead of Input::file
  char prog[] = "ref_harness", flag[] = "-i";
  char *mpm_argv[] = {prog, flag, argv[1], nullptr};
  int mpm_argc = 3;
  MPI_Init(&argc, &argv);
  MPM *mpm = new MPM(mpm_argc, mpm_argv, MPI_COMM_WORLD);
  std::string line;
  while (std::getline(in, line)) {
    if (line.rfind("#@", 0) == 0) {
      std::istringstream ss(line.substr(2));
      std::string cmd, label;
      ss >> cmd >> label;
      if (cmd == "state") {
        write_state(out, label, mpm);
      } else if (cmd == "vars") {
        std::vector<std::string> names;
        std::string n;
        while (ss >> n) names.push_back(n);
        write_vars(out, label, names, mpm);
      }
      continue;
    }
    const size_t hash = line.find('#');
    if (hash != std::string::npos) line.erase(hash);
    if (line.find_first_not_of(" \t\r") == std::string::npos) continue;
    mpm->input->parsev(line).result();
  }
  out.close();
  delete mpm;
  MPI_Finalize();
  return 0;
}
