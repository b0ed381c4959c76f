// mpm_oracle.cpp -- FP64 CPU restatement of Karamelo's explicit MPM time step.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
// smoke check and the CPU-baseline leg of the benchmark call it; the product
// (karamelo_gb300/) never links, imports or executes it.
//
// Parity status: partially pinned.
//   - The 1-D basis functions below are checked against the reference's own
//     header (src/basis_functions.h, compiled by oracle/Makefile into
//     oracle/_ref/ and stored as golden vectors in tests/golden/).
//   - The whole TLMPM MUSL step with a neo-Hookean material, a body force
//     and a velocity fix follows the reference's published runs of
//     examples/Vertical_bar (their logged tip displacement,
//     tests/golden/vertical_bar_golden.npz): FLIP with the cubic spline to
//     8e-6 relative over 100 steps; FLIP with the linear basis and APIC with
//     either basis to 4e-6 over 50 steps.
//   - The reference itself cannot be built here (it needs Eigen 3 and MPI),
//     so the other laws and transfers rest on this line-by-line restatement
//     of the cited reference functions: double precision, with the
//     reference's loop and summation order.
//
// All citations are paths inside the Karamelo source tree.
//
// Layout: row-major 3x3 matrices (M[3*i+j] = M(i,j)), vectors of 3 doubles.
// Scatter (P2G) is a node-centric gather over per-node particle lists in
// particle-index order, exactly as src/solid.cpp:317-522 does, so the sums
// are deterministic.  Loops over nodes and over particles are OpenMP-parallel;
// no reduction crosses threads except min/max, which are order-free.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// src/solid.cpp:39-40 (the reference's truncated constants; kept alike so that
// the oracle reproduces the reference's rounding of the von Mises factor).
constexpr double SQRT_3_OVER_2 = 1.224744871;
constexpr double FOUR_THIRD = 1.333333333333333333333333333333333333333;

// ---------------------------------------------------------------- 3x3 algebra
struct M3 {
  double a[9];
  double &operator()(int i, int j) { return a[3 * i + j]; }
  double operator()(int i, int j) const { return a[3 * i + j]; }
};
inline M3 zero3() { M3 m; for (double &x : m.a) x = 0; return m; }
inline M3 eye3() { M3 m = zero3(); m.a[0] = m.a[4] = m.a[8] = 1; return m; }
inline M3 mul(const M3 &A, const M3 &B) {
  M3 C;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      C(i, j) = A(i, 0) * B(0, j) + A(i, 1) * B(1, j) + A(i, 2) * B(2, j);
  return C;
}
inline M3 tr(const M3 &A) { M3 C; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) C(i, j) = A(j, i); return C; }
inline M3 add(const M3 &A, const M3 &B) { M3 C; for (int k = 0; k < 9; k++) C.a[k] = A.a[k] + B.a[k]; return C; }
inline M3 sub(const M3 &A, const M3 &B) { M3 C; for (int k = 0; k < 9; k++) C.a[k] = A.a[k] - B.a[k]; return C; }
inline M3 scale(double s, const M3 &A) { M3 C; for (int k = 0; k < 9; k++) C.a[k] = s * A.a[k]; return C; }
inline double trace(const M3 &A) { return A.a[0] + A.a[4] + A.a[8]; }
inline double fnorm(const M3 &A) { double s = 0; for (double x : A.a) s += x * x; return std::sqrt(s); }
inline double det(const M3 &A) {
  return A(0, 0) * (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) -
         A(0, 1) * (A(1, 0) * A(2, 2) - A(1, 2) * A(2, 0)) +
         A(0, 2) * (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0));
}
inline M3 inv(const M3 &A) {
  M3 C;
  double d = det(A);
  C(0, 0) = (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) / d;
  C(0, 1) = (A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2)) / d;
  C(0, 2) = (A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1)) / d;
  C(1, 0) = (A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2)) / d;
  C(1, 1) = (A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0)) / d;
  C(1, 2) = (A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2)) / d;
  C(2, 0) = (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0)) / d;
  C(2, 1) = (A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1)) / d;
  C(2, 2) = (A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0)) / d;
  return C;
}
// MPM_Math::Deviator, src/mpm_math.h:28-33
inline M3 deviator(const M3 &M) {
  M3 C = M;
  double t = trace(M) / 3.0;
  C.a[0] -= t; C.a[4] -= t; C.a[8] -= t;
  return C;
}

// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (Golub & Van
// Loan, "Matrix Computations", sec. 8.5).  A = V diag(w) V^T.
void sym_eig(const M3 &Ain, double w[3], M3 &V) {
  M3 A = Ain;
  V = eye3();
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = A(0, 1) * A(0, 1) + A(0, 2) * A(0, 2) + A(1, 2) * A(1, 2);
    double dia = A(0, 0) * A(0, 0) + A(1, 1) * A(1, 1) + A(2, 2) * A(2, 2);
    if (off <= 1e-34 * dia || off == 0) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        double apq = A(p, q);
        if (apq == 0) continue;
        double theta = (A(q, q) - A(p, p)) / (2 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < 3; k++) {  // A <- J^T A J
          double akp = A(k, p), akq = A(k, q);
          A(k, p) = c * akp - s * akq;
          A(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < 3; k++) {
          double apk = A(p, k), aqk = A(q, k);
          A(p, k) = c * apk - s * aqk;
          A(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; k++) {
          double vkp = V(k, p), vkq = V(k, q);
          V(k, p) = c * vkp - s * vkq;
          V(k, q) = s * vkp + c * vkq;
        }
      }
  }
  w[0] = A(0, 0); w[1] = A(1, 1); w[2] = A(2, 2);
}

// MPM_Math::PolDec(M, R), src/mpm_math.h:104-133: R = U V^T from the SVD
// M = U S V^T; if det R < 0 the smallest singular value is flipped and
// R = M V S^-1 V^T.  The SVD is obtained from the eigen-decomposition of
// M^T M (V, S^2), which gives the same R: for S > 0, U = M V S^-1, so
// U V^T = M V S^-1 V^T.
bool poldec(const M3 &M, M3 &R) {
  double w[3];
  M3 V;
  sym_eig(mul(tr(M), M), w, V);
  double s[3];
  for (int i = 0; i < 3; i++) s[i] = std::sqrt(std::max(w[i], 0.0));
  auto build = [&](const double *sv) {
    M3 Sinv = zero3();
    for (int i = 0; i < 3; i++) Sinv(i, i) = 1.0 / sv[i];
    return mul(mul(mul(M, V), Sinv), tr(V));
  };
  R = build(s);
  if (det(R) < 0.0) {
    int imin = 0;
    for (int i = 1; i < 3; i++) if (s[i] < s[imin]) imin = i;
    double sf[3] = {s[0], s[1], s[2]};
    sf[imin] *= -1.0;
    R = build(sf);
  }
  return det(R) > 0.0;
}

// Real parts of the eigenvalues of a general 3x3 matrix (the reference calls
// Eigen::EigenSolver<Matrix3d>, src/solid.cpp:1401-1409).  F is written as
// I + H and the characteristic cubic of H, mu^3 - c2 mu^2 + c1 mu - c0, is
// solved in closed form (trigonometric form for three real roots, Cardano
// otherwise); lambda = 1 + mu.  Working with H keeps the near-identity
// deformation gradients of the MPM step free of cancellation.  Real roots are
// polished by guarded Newton steps.
void eig_real_parts(const M3 &F, double re[3]) {
  M3 H = F;
  H.a[0] -= 1; H.a[4] -= 1; H.a[8] -= 1;
  double c2 = trace(H);
  double c1 = H(0, 0) * H(1, 1) - H(0, 1) * H(1, 0) + H(0, 0) * H(2, 2) - H(0, 2) * H(2, 0) +
              H(1, 1) * H(2, 2) - H(1, 2) * H(2, 1);
  double c0 = det(H);
  // depressed cubic t^3 + p t + q with mu = t + c2/3
  double a = -c2, b = c1, c = -c0;
  double p = b - a * a / 3.0;
  double q = 2.0 * a * a * a / 27.0 - a * b / 3.0 + c;
  double shift = -a / 3.0;
  double disc = q * q / 4.0 + p * p * p / 27.0;
  // Newton steps are kept only when they reduce the residual: at a (near-)
  // multiple root the derivative vanishes and an unguarded step diverges.
  auto polish = [&](double x) {
    for (int it = 0; it < 2; it++) {
      double f = ((x - c2) * x + c1) * x - c0;
      double df = (3 * x - 2 * c2) * x + c1;
      if (df == 0) break;
      double xn = x - f / df;
      double fn = ((xn - c2) * xn + c1) * xn - c0;
      if (std::fabs(fn) >= std::fabs(f)) break;
      x = xn;
    }
    return x;
  };
  if (disc <= 0) {
    double r = std::sqrt(std::max(-p / 3.0, 0.0));
    double arg = (r > 0) ? (-q / 2.0) / (r * r * r) : 0.0;
    arg = std::max(-1.0, std::min(1.0, arg));
    double phi = std::acos(arg);
    for (int k = 0; k < 3; k++)
      re[k] = 1.0 + polish(2 * r * std::cos((phi + 2 * M_PI * k) / 3.0) + shift);
  } else {
    double sd = std::sqrt(disc);
    double u = std::cbrt(-q / 2.0 + sd), v = std::cbrt(-q / 2.0 - sd);
    double x = polish(u + v + shift);
    re[0] = 1.0 + x;
    re[1] = re[2] = 1.0 + (c2 - x) / 2.0;  // real part of the complex pair
  }
}

// ---------------------------------------------------------------- basis
// BasisFunction::*, src/basis_functions.h:21-138 (restated).
double bf_linear(double r_, int) {
  double r = std::fabs(r_);
  return r >= 1.0 ? 0.0 : 1.0 - r;
}
double dbf_linear(double r, int, double ih) {
  if (r >= 1.0 || r <= -1.0 || r == 0) return 0.0;
  return r > 0.0 ? -ih : ih;
}
double bf_cubic(double r, int nt) {
  if (r >= 1 && r < 2) return nt == 1 ? 0 : ((-1.0 / 6.0 * r + 1) * r - 2) * r + 4.0 / 3.0;
  if (r >= 0 && r < 1) {
    if (nt == -2) return (1.0 / 6.0 * r * r - 1) * r + 1;
    if (nt == 2) return 1;
    if (nt == 1) return (1.0 / 3.0 * r - 1) * r * r + 2.0 / 3.0;
    return (0.5 * r - 1) * r * r + 2.0 / 3.0;
  }
  if (r >= -1 && r < 0) {
    if (nt == 2) return (-1.0 / 6.0 * r * r + 1) * r + 1;
    if (nt == -1) return (-1.0 / 3.0 * r - 1) * r * r + 2.0 / 3.0;
    return (-0.5 * r - 1) * r * r + 2.0 / 3.0;
  }
  if (r >= -2 && r < -1) return ((1.0 / 6.0 * r + 1) * r + 2) * r + 4.0 / 3.0;
  return 0;
}
double dbf_cubic(double r, int nt, double ih) {
  if (r >= 1 && r < 2) return nt == 1 ? -ih : ih * ((-0.5 * r + 2) * r - 2);
  if (r >= 0 && r < 1) {
    if (nt == -2) return ih * (0.5 * r * r - 1);
    if (nt == 2) return ih;
    if (nt == 1) return ih * r * (r - 2);
    return ih * (3.0 / 2.0 * r - 2) * r;
  }
  if (r >= -1 && r < 0) {
    if (nt == 2) return ih * (-0.5 * r * r + 1);
    if (nt == -1) return ih * (-r - 2) * r;
    return ih * (-3.0 / 2.0 * r - 2) * r;
  }
  if (r >= -2 && r < -1) return ih * ((0.5 * r + 2) * r + 2);
  return 0;
}
// BasisFunction::quadratic_spline / derivative_quadratic_spline,
// src/basis_functions.h:140-241 (ranges restated as in the reference)
double bf_quad(double r, int nt) {
  if (nt == 0) {
    if (r >= 0.5 && r < 1.5) return (0.5 * r - 1.5) * r + 1.125;
    if (r >= -0.5 && r < 0.5) return -r * r + 0.75;
    if (r >= -1.5 && r < 0.5) return (0.5 * r + 1.5) * r + 1.125;
    return 0;
  }
  if (nt == -2) {
    if (r >= 0. && r < 0.5) return 1 - r;
    if (r >= 0.5 && r < 1.5) return (0.5 * r - 1.5) * r + 1.125;
    return 0;
  }
  if (nt == -1) {
    if (r >= -1. && r < -0.5) return 1 + r;
    if (r >= -0.5 && r < 0.5) return -r * r + 0.75;
    if (r >= 0.5 && r < 1.5) return (0.5 * r - 1.5) * r + 1.125;
    return 0;
  }
  if (nt == 1) {
    if (r >= -1.5 && r < -0.5) return (0.5 * r + 1.5) * r + 1.125;
    if (r >= -0.5 && r < 0.5) return -r * r + 0.75;
    if (r >= 0.5 && r < 1.) return 1 - r;
    return 0;
  }
  if (r >= -1.5 && r < -0.5) return (0.5 * r + 1.5) * r + 1.125;
  if (r >= -0.5 && r <= 0.) return 1 + r;
  return 0;
}
double dbf_quad(double r, int nt, double ih) {
  if (nt == 0) {
    if (r >= 0.5 && r < 1.5) return ih * (r - 1.5);
    if (r >= -0.5 && r < 0.5) return -2 * ih * r;
    if (r >= -1.5 && r < 0.5) return ih * (r + 1.5);
    return 0;
  }
  if (nt == -2) {
    if (r >= 0. && r < 0.5) return -ih;
    if (r >= 0.5 && r < 1.5) return ih * (r - 1.5);
    return 0;
  }
  if (nt == -1) {
    if (r >= -1. && r < -0.5) return ih;
    if (r >= -0.5 && r < 0.5) return -2 * ih * r;
    if (r >= 0.5 && r < 1.5) return ih * (r - 1.5);
    return 0;
  }
  if (nt == 1) {
    if (r >= -1.5 && r < -0.5) return ih * (r + 1.5);
    if (r >= -0.5 && r < 0.5) return -2 * ih * r;
    if (r >= 0.5 && r < 1.) return -ih;
    return 0;
  }
  if (r >= -1.5 && r < -0.5) return ih * (r + 1.5);
  if (r >= -0.5 && r <= 0.) return ih;
  return 0;
}

double bf_bern(double r_, int nt) {
  double r = std::fabs(r_);
  if (r >= 1.0) return 0;
  if (nt == 1) return r >= 0.5 ? 0 : 0.5 - 2 * r * r;
  return (1 - r) * (1 - r);
}
double dbf_bern(double rs, int nt, double ih) {
  double r = std::fabs(rs);
  if (r >= 1.0) return 0;
  if (nt == 1) return r > 0.5 ? 0 : -4 * rs * ih;
  return rs > 0 ? -2 * (1 - rs) * ih : 2 * (1 + rs) * ih;
}

// ---------------------------------------------------------------- model
enum { TLMPM = 0, ULMPM = 1 };
enum { USL = 0, MUSL = 1, USF = 2 };
enum { LINEAR = 0, CUBIC = 1, BERNSTEIN = 2, QUADRATIC = 3 };
enum { MAT_LINEAR = 0, MAT_NEO_HOOKEAN = 1, MAT_EOS_STRENGTH = 2 };
enum { EOS_LINEAR = 0, EOS_SHOCK = 1, EOS_FLUID = 2 };
enum { STR_LINEAR = 0, STR_PLASTIC = 1, STR_JC = 2, STR_SWIFT = 3, STR_FLUID = 4 };

}  // namespace

extern "C" {
// Material description shared with the Python side (same field order as the
// ctypes Structure in oracle/oracle.py).
typedef struct {
  int type;                 // MAT_*
  double rho0, E, nu, cp, kappa;  // linear / neo-Hookean (src/material.cpp:749-769)
  int eos;                  // EOS_*
  double eos_p[12];         // linear: rho0 K; shock: rho0 K c0 S Gamma cv Tr Q1 Q2; fluid: rho0 K Gamma
  int strength;             // STR_*
  double str_p[12];         // linear: G; plastic: G sy; jc: G A B n epsdot0 C m Tr Tm; swift: G A B C n; fluid: mu
  int damage;               // -1 none, 0 johnson_cook
  double dam_p[8];          // d1 d2 d3 d4 d5 epsdot0 Tr Tm
  int temp;                 // -1 none, 0 plastic_work
  double temp_p[6];         // chi cp kappa alpha T0 Tm
} om_material;
}

namespace {

struct Mat {
  om_material d;
  int type;
  double rho0, K, G, lambda, signal_velocity, cp, invcp, kappa;
  double E, nu;  // Young's modulus and Poisson ratio (derived from K and G for EOS materials)
  // Mat::Mat, src/material.cpp:720-778
  explicit Mat(const om_material &m) : d(m), type(m.type) {
    if (type == MAT_EOS_STRENGTH) {
      rho0 = m.eos_p[0];
      K = m.eos_p[1];
      G = m.str_p[0];
      E = 9 * K * G / (3 * K + G);
      nu = (3 * K - 2 * G) / (2 * (3 * K + G));
      lambda = K - 2 * G / 3;
      signal_velocity = std::sqrt((lambda + 2 * G) / rho0);
      if (m.temp >= 0) {
        cp = m.temp_p[1];
        invcp = 1.0 / cp;
        kappa = m.temp_p[2];
      } else {
        cp = invcp = kappa = 0;
      }
    } else {
      rho0 = m.rho0;
      E = m.E;
      nu = m.nu;
      G = E / (2 * (1 + nu));
      lambda = E * nu / ((1 + nu) * (1 - 2 * nu));
      K = E / (3 * (1 - 2 * nu));
      signal_velocity = std::sqrt(K / rho0);
      cp = m.cp;
      invcp = cp != 0 ? 1.0 / cp : 0;
      kappa = m.kappa;
    }
  }
};

struct Grid {
  int nx, ny, nz, nxg, nyg, nzg, nn;
  double h;         // node spacing (cellsize/2 for Bernstein)
  double cellsize;  // Grid::cellsize (used for weights and dtCFL)
  double lo[3];
  std::vector<double> x0, x, v, vu, f, mb, mass, T, Tu, Qext, Qint;
  std::vector<int> ntype;
  std::vector<int> map_ntag;  // global tag -> local index
};

struct Solid {
  int grid, mat, np;
  double T0;
  std::vector<double> x0, x, v, vu, a, mbp, f, q;          // 3 per particle
  std::vector<M3> sigma, strain_el, vol0PK1, L, F, R, D, Finv, Fdot;
  std::vector<double> vol0, vol, rho0, rho, mass, epsp, epsdot, damage, damage_init, ienergy, J, T, gamma;
  // neighbour lists (src/solid.h: numneigh_pn, neigh_pn, wf_pn, wfd_pn, *_np)
  std::vector<std::vector<int>> neigh_pn, neigh_np;
  std::vector<std::vector<double>> wf_pn, wf_np;
  std::vector<std::vector<double>> wfd_pn, wfd_np;  // 3 per entry
  double dtCFL;
  double Di[3] = {1, 1, 1};  // APIC inertia tensor inverse (diagonal), Solid::compute_inertia_tensor
  int np_per_cell = 0;       // Solid::np_per_cell (src/solid.cpp:2027)
};

enum { FIX_VEL_NODES = 0, FIX_BODY_FORCE = 1 };
struct Fix {
  int kind, grid;
  std::vector<uint8_t> mask;
  int set[3];
  double c[3][4];  // velocity: v(t) = c0 + c1 t + c2 exp(c3 t); body force: c0
};

// contact fix between two solids (FixContactMinPenetration, FixContactHertz)
enum { CONTACT_MIN_PENETRATION = 0, CONTACT_HERTZ = 1 };
struct Contact {
  int kind, s1, s2;
  double mu;
  double ftot[3] = {0, 0, 0};  // the fix's <id>_x, _y, _z
};

struct Sim {
  int method, scheme, basis, dim;
  double pic_flip;
  bool apic = false;  // affine transfers: APIC, and for ULMPM AFLIP / ASFLIP / MLS (src/ulmpm.cpp:79-85)
  bool asflip = false;  // ULMPM ASFLIP: positions move with the blended velocity (src/ulmpm.cpp:453-473)
  bool mls = false;     // ULMPM MLS: internal forces from moments (src/solid.cpp:524-574)
  bool axisym = false;  // Domain::axisymmetric: 2-D with x = r, y = z (src/domain.cpp:554-570)
  bool thermal;
  double dt, dt_factor;
  bool dt_constant;
  double boxlo[3], boxhi[3];
  double time = 0;
  long ntimestep = 0;
  bool update_wf = true, update_mass_nodes = true;
  std::vector<Mat> mats;
  std::vector<Grid> grids;
  std::vector<Solid> solids;
  std::vector<Fix> fixes;
  std::vector<Contact> contacts;
  std::string err;
  double (*bf)(double, int) = bf_linear;
  double (*dbf)(double, int, double) = dbf_linear;
};

double fix_value(const double *c, double t) { return c[0] + c[1] * t + c[2] * std::exp(c[3] * t); }

// Grid::init, src/grid.cpp:68-413 for one process (sublo = boxlo, subhi =
// boxhi, no neighbouring process).
void grid_init(Sim &s, Grid &g, const double *boundlo, const double *boundhi, double cellsize) {
  double h = cellsize;
  if (s.basis == BERNSTEIN) h /= 2;
  g.h = h;
  g.cellsize = cellsize;
  double L[3], Lhi[3];
  for (int d = 0; d < 3; d++) {
    L[d] = std::max(0.0, std::min(s.boxhi[d], boundhi[d]) - boundlo[d]);
    Lhi[d] = L[d];
  }
  int noffhi[3];
  for (int d = 0; d < 3; d++) noffhi[d] = (int)std::ceil(Lhi[d] / h);
  double Lg[3] = {boundhi[0] - boundlo[0], boundhi[1] - boundlo[1], boundhi[2] - boundlo[2]};
  g.nxg = ((int)(Lg[0] / h)) + 1;
  while (g.nxg * h <= Lg[0] + 0.5 * h) g.nxg++;
  if (s.dim >= 2) {
    g.nyg = (int)(((int)Lg[1]) / h) + 1;  // src/grid.cpp:143 casts before dividing
    while (g.nyg * h <= Lg[1] + 0.5 * h) g.nyg++;
  } else g.nyg = 1;
  if (s.dim == 3) {
    g.nzg = (int)(((int)Lg[2]) / h) + 1;
    while (g.nzg * h <= Lg[2] + 0.5 * h) g.nzg++;
  } else g.nzg = 1;
  g.nx = std::max(0, noffhi[0]);
  g.ny = s.dim >= 2 ? std::max(0, noffhi[1]) : 1;
  g.nz = s.dim >= 3 ? std::max(0, noffhi[2]) : 1;
  while (boundlo[0] + h * (g.nx - 0.5) < std::min(s.boxhi[0], boundhi[0])) g.nx++;
  while (boundlo[1] + h * (g.ny - 0.5) < std::min(s.boxhi[1], boundhi[1])) g.ny++;
  while (boundlo[2] + h * (g.nz - 0.5) < std::min(s.boxhi[2], boundhi[2])) g.nz++;
  g.nn = g.nx * g.ny * g.nz;
  for (int d = 0; d < 3; d++) g.lo[d] = boundlo[d];
  g.x0.assign(3 * g.nn, 0);
  g.ntype.assign(3 * g.nn, 0);
  g.map_ntag.assign((size_t)g.nxg * g.nyg * g.nzg, -1);
  int l = 0;
  for (int i = 0; i < g.nx; i++)
    for (int j = 0; j < g.ny; j++)
      for (int k = 0; k < g.nz; k++) {
        g.x0[3 * l + 0] = boundlo[0] + i * h;
        g.x0[3 * l + 1] = s.dim >= 2 ? boundlo[1] + j * h : 0;
        g.x0[3 * l + 2] = s.dim == 3 ? boundlo[2] + k * h : 0;
        if (s.basis == BERNSTEIN) {
          g.ntype[3 * l + 0] = i % 2;
          g.ntype[3 * l + 1] = j % 2;
          g.ntype[3 * l + 2] = k % 2;
        } else if (s.basis == CUBIC || s.basis == QUADRATIC) {
          g.ntype[3 * l + 0] = std::min(2, i) - std::min(g.nxg - 1 - i, 2);
          g.ntype[3 * l + 1] = std::min(2, j) - std::min(g.nyg - 1 - j, 2);
          g.ntype[3 * l + 2] = std::min(2, k) - std::min(g.nzg - 1 - k, 2);
        }
        long tag = (long)g.nzg * g.nyg * i + (long)g.nzg * j + k;
        if (tag < (long)g.map_ntag.size()) g.map_ntag[tag] = l;
        l++;
      }
  g.x = g.x0;
  g.v.assign(3 * g.nn, 0); g.vu.assign(3 * g.nn, 0); g.f.assign(3 * g.nn, 0); g.mb.assign(3 * g.nn, 0);
  g.mass.assign(g.nn, 0);
  g.T.assign(g.nn, 0); g.Tu.assign(g.nn, 0); g.Qext.assign(g.nn, 0); g.Qint.assign(g.nn, 0);
}

// TLMPM/ULMPM::compute_grid_weight_functions_and_gradients,
// src/tlmpm.cpp:87-340 and src/ulmpm.cpp:88-337.  TL uses x0 relative to the
// solid's lower bound, UL uses x relative to the box.
// Solid::compute_inertia_tensor, src/solid.cpp:1440-1478: Di = 3 / cellsize^2
// (cubic) or 4 / cellsize^2 (quadratic) on the active dimensions, 1 on the others
void compute_inertia_tensor(const Sim &s, Solid &S) {
  const double c = s.grids[S.grid].cellsize;
  // linear: 16/4 (one particle per cell per direction) or 16/3 (two), src/solid.cpp:1447-1462
  const double k = s.basis == QUADRATIC ? 4.0 : s.basis == LINEAR ? (S.np_per_cell == 1 ? 16.0 / 4.0 : 16.0 / 3.0) : 3.0;
  for (int d = 0; d < 3; d++) S.Di[d] = d < s.dim ? k / (c * c) : 1.0;
}

void build_neighbours(Sim &s, Solid &S) {
  Grid &g = s.grids[S.grid];
  if (s.apic) compute_inertia_tensor(s, S);
  const std::vector<double> &xp = (s.method == TLMPM) ? S.x0 : S.x;
  const double *lo = (s.method == TLMPM) ? g.lo : s.boxlo;
  double ih = 1.0 / g.cellsize;
  long nnodes = (long)g.nxg * g.nyg * g.nzg;
  int ny = g.nyg, nz = g.nzg;
  for (int in = 0; in < g.nn; in++) {
    S.neigh_np[in].clear(); S.wf_np[in].clear(); S.wfd_np[in].clear();
  }
#pragma omp parallel for schedule(static)
  for (int ip = 0; ip < S.np; ip++) {
    S.neigh_pn[ip].clear(); S.wf_pn[ip].clear(); S.wfd_pn[ip].clear();
    int i0, j0, k0, w;
    double t[3] = {(xp[3 * ip] - lo[0]) * ih, (xp[3 * ip + 1] - lo[1]) * ih, (xp[3 * ip + 2] - lo[2]) * ih};
    if (s.basis == LINEAR) {
      i0 = (int)t[0]; j0 = (int)t[1]; k0 = (int)t[2]; w = 2;
    } else if (s.basis == BERNSTEIN) {
      i0 = 2 * (int)t[0]; j0 = 2 * (int)t[1]; k0 = 2 * (int)t[2]; w = 3;
    } else {
      i0 = (int)(t[0] - 1); j0 = (int)(t[1] - 1); k0 = (int)(t[2] - 1); w = 4;
    }
    std::vector<int> cand;
    for (int i = i0; i < i0 + w; i++) {
      if (ny > 1) {
        for (int j = j0; j < j0 + w; j++) {
          if (nz > 1) {
            for (int k = k0; k < k0 + w; k++) {
              long tag = (long)nz * ny * i + (long)nz * j + k;
              if (tag >= 0 && tag < nnodes && g.map_ntag[tag] != -1) cand.push_back(g.map_ntag[tag]);
            }
          } else {
            long tag = (long)ny * i + j;
            if (tag >= 0 && tag < nnodes && g.map_ntag[tag] != -1) cand.push_back(g.map_ntag[tag]);
          }
        }
      } else if (i >= 0 && i < g.nn) cand.push_back(i);
    }
    for (int in : cand) {
      double r[3], sv[3], sd[3] = {0, 0, 0};
      for (int d = 0; d < 3; d++) r[d] = (xp[3 * ip + d] - g.x0[3 * in + d]) * ih;
      sv[0] = s.bf(r[0], g.ntype[3 * in]);
      sv[1] = s.dim >= 2 ? s.bf(r[1], g.ntype[3 * in + 1]) : 1;
      sv[2] = s.dim == 3 ? s.bf(r[2], g.ntype[3 * in + 2]) : 1;
      if (sv[0] != 0 && sv[1] != 0 && sv[2] != 0) {
        sd[0] = s.dbf(r[0], g.ntype[3 * in], ih);
        if (s.dim >= 2) sd[1] = s.dbf(r[1], g.ntype[3 * in + 1], ih);
        if (s.dim == 3) sd[2] = s.dbf(r[2], g.ntype[3 * in + 2], ih);
        double wf, wfd[3];
        if (s.dim == 1) { wf = sv[0]; wfd[0] = sd[0]; wfd[1] = wfd[2] = 0; }
        else if (s.dim == 2) { wf = sv[0] * sv[1]; wfd[0] = sd[0] * sv[1]; wfd[1] = sv[0] * sd[1]; wfd[2] = 0; }
        else { wf = sv[0] * sv[1] * sv[2]; wfd[0] = sd[0] * sv[1] * sv[2]; wfd[1] = sv[0] * sd[1] * sv[2]; wfd[2] = sv[0] * sv[1] * sd[2]; }
        S.neigh_pn[ip].push_back(in);
        S.wf_pn[ip].push_back(wf);
        for (int d = 0; d < 3; d++) S.wfd_pn[ip].push_back(wfd[d]);
      }
    }
  }
  // node lists in particle-index order (the reference pushes to neigh_np
  // inside the same particle loop)
  for (int ip = 0; ip < S.np; ip++)
    for (size_t j = 0; j < S.neigh_pn[ip].size(); j++) {
      int in = S.neigh_pn[ip][j];
      S.neigh_np[in].push_back(ip);
      S.wf_np[in].push_back(S.wf_pn[ip][j]);
      for (int d = 0; d < 3; d++) S.wfd_np[in].push_back(S.wfd_pn[ip][3 * j + d]);
    }
}

// Solid::compute_mass_nodes, src/solid.cpp:317-335
void compute_mass_nodes(Solid &S, Grid &g, bool reset) {
#pragma omp parallel for schedule(static)
  for (int in = 0; in < g.nn; in++) {
    if (reset) g.mass[in] = 0;
    for (size_t j = 0; j < S.neigh_np[in].size(); j++) g.mass[in] += S.wf_np[in][j] * S.mass[S.neigh_np[in][j]];
  }
}

// Solid::compute_velocity_nodes, src/solid.cpp:337-390, and with APIC
// Solid::compute_velocity_nodes_APIC, src/solid.cpp:392-426: the particle
// velocity plus C (x0_node - x_p), C = Fdot (TL) or L (UL), x_p = x0 (TL) or x (UL)
void compute_velocity_nodes(const Sim &s, Solid &S, Grid &g, bool reset) {
  const bool TL = s.method == TLMPM;
  const std::vector<double> &pos = TL ? S.x0 : S.x;
  const std::vector<M3> &C = TL ? S.Fdot : S.L;
#pragma omp parallel for schedule(static)
  for (int in = 0; in < g.nn; in++) {
    if (reset) for (int d = 0; d < 3; d++) g.v[3 * in + d] = 0;
    if (g.mass[in] > 0) {
      double vt[3] = {0, 0, 0};
      for (size_t j = 0; j < S.neigh_np[in].size(); j++) {
        int ip = S.neigh_np[in][j];
        double wm = S.wf_np[in][j] * S.mass[ip];
        double vp[3] = {S.v[3 * ip], S.v[3 * ip + 1], S.v[3 * ip + 2]};
        if (s.apic) {
          double dx[3];
          for (int d = 0; d < 3; d++) dx[d] = g.x0[3 * in + d] - pos[3 * ip + d];
          for (int d = 0; d < 3; d++) vp[d] += C[ip](d, 0) * dx[0] + C[ip](d, 1) * dx[1] + C[ip](d, 2) * dx[2];
        }
        for (int d = 0; d < 3; d++) vt[d] += wm * vp[d];
      }
      for (int d = 0; d < 3; d++) g.v[3 * in + d] += vt[d] / g.mass[in];
    }
  }
}

// Solid::compute_external_forces_nodes, src/solid.cpp:428-450 (TL)
void compute_external_forces_nodes(Solid &S, Grid &g, bool reset) {
#pragma omp parallel for schedule(static)
  for (int in = 0; in < g.nn; in++) {
    if (reset) for (int d = 0; d < 3; d++) g.mb[3 * in + d] = 0;
    if (g.mass[in] > 0)
      for (size_t j = 0; j < S.neigh_np[in].size(); j++) {
        int ip = S.neigh_np[in][j];
        for (int d = 0; d < 3; d++) g.mb[3 * in + d] += S.wf_np[in][j] * S.mbp[3 * ip + d];
      }
  }
}

// Solid::compute_internal_forces_nodes_TL, src/solid.cpp:452-480 (axisymmetric:
// the hoop term -vol0PK1(2,2) w / r, r = x0_r, in the same loop)
void compute_internal_forces_nodes_TL(const Sim &s, Solid &S, Grid &g) {
#pragma omp parallel for schedule(static)
  for (int in = 0; in < g.nn; in++) {
    double ft[3] = {0, 0, 0};
    for (size_t j = 0; j < S.neigh_np[in].size(); j++) {
      int ip = S.neigh_np[in][j];
      const M3 &P = S.vol0PK1[ip];
      const double *gw = &S.wfd_np[in][3 * j];
      for (int d = 0; d < 3; d++) ft[d] -= P(d, 0) * gw[0] + P(d, 1) * gw[1] + P(d, 2) * gw[2];
      if (s.axisym) ft[0] -= P(2, 2) * S.wf_np[in][j] / S.x0[3 * ip];
    }
    for (int d = 0; d < 3; d++) g.f[3 * in + d] = ft[d];
  }
}

// Solid::compute_external_and_internal_forces_nodes_UL, src/solid.cpp:482-522
void compute_forces_nodes_UL(const Sim &s, Solid &S, Grid &g, bool reset) {
#pragma omp parallel for schedule(static)
  for (int in = 0; in < g.nn; in++) {
    if (reset) for (int d = 0; d < 3; d++) { g.f[3 * in + d] = 0; g.mb[3 * in + d] = 0; }
    for (size_t j = 0; j < S.neigh_np[in].size(); j++) {
      int ip = S.neigh_np[in][j];
      const M3 &sg = S.sigma[ip];
      double gw[3];
      if (s.mls) {
        // compute_external_and_internal_forces_nodes_UL_MLS, src/solid.cpp:524-574:
        // w Di (x0_node - x_p) in place of grad w
        for (int d = 0; d < 3; d++) gw[d] = S.wf_np[in][j] * S.Di[d] * (g.x0[3 * in + d] - S.x[3 * ip + d]);
      } else {
        for (int d = 0; d < 3; d++) gw[d] = S.wfd_np[in][3 * j + d];
      }
      for (int d = 0; d < 3; d++) {
        g.f[3 * in + d] -= S.vol[ip] * (sg(d, 0) * gw[0] + sg(d, 1) * gw[1] + sg(d, 2) * gw[2]);
        g.mb[3 * in + d] += S.wf_np[in][j] * S.mbp[3 * ip + d];
      }
    }
    // axisymmetric hoop term, in a second loop as the reference writes it
    // (src/solid.cpp:513-519, 565-571): -vol sigma(2,2) w / r, r = x_r
    if (s.axisym)
      for (size_t j = 0; j < S.neigh_np[in].size(); j++) {
        int ip = S.neigh_np[in][j];
        g.f[3 * in] -= S.vol[ip] * (S.sigma[ip](2, 2) * S.wf_np[in][j] / S.x[3 * ip]);
      }
  }
}

// thermal P2G, src/solid.cpp:2743-2800
void compute_temperature_nodes(Solid &S, Grid &g, bool reset) {
#pragma omp parallel for schedule(static)
  for (int in = 0; in < g.nn; in++) {
    if (reset) g.T[in] = 0;
    if (g.mass[in] > 0) {
      double tt = 0;
      for (size_t j = 0; j < S.neigh_np[in].size(); j++) {
        int ip = S.neigh_np[in][j];
        tt += S.wf_np[in][j] * S.mass[ip] * S.T[ip];
      }
      g.T[in] += tt / g.mass[in];
    }
  }
}
void compute_temperature_forces(Solid &S, Grid &g, bool reset) {
#pragma omp parallel for schedule(static)
  for (int in = 0; in < g.nn; in++) {
    if (reset) g.Qext[in] = 0;
    if (g.mass[in] > 0)
      for (size_t j = 0; j < S.neigh_np[in].size(); j++) g.Qext[in] += S.wf_np[in][j] * S.gamma[S.neigh_np[in][j]];
    g.Qint[in] = 0;
    for (size_t j = 0; j < S.neigh_np[in].size(); j++) {
      int ip = S.neigh_np[in][j];
      const double *gw = &S.wfd_np[in][3 * j];
      g.Qint[in] += gw[0] * S.q[3 * ip] + gw[1] * S.q[3 * ip + 1] + gw[2] * S.q[3 * ip + 2];
    }
  }
}

// EOS::compute_pressure: src/eos_linear.cpp:71-74, src/eos_shock.cpp:99-133,
// src/eos_fluid.cpp:68-73
double eos_pressure(const Mat &m, double &e, double J, double rho, double damage, const M3 &D, double cellsize, double T) {
  const double *p = m.d.eos_p;
  if (m.d.eos == EOS_LINEAR) {
    e = 0;
    return p[1] * (1 - J) * (1 - damage);
  }
  if (m.d.eos == EOS_FLUID) {
    double mu = rho / p[0];
    e = 0;
    return p[1] * (std::pow(mu, p[2]) - 1.0);
  }
  // shock: rho0 K c0 S Gamma cv Tr Q1 Q2
  double rho0 = p[0], c0 = p[2], S = p[3], Gamma = p[4], cv = p[5], Tr = p[6], Q1 = p[7], Q2 = p[8];
  double alpha = cv * rho0, e0 = 0;
  double mu = rho / rho0 - 1.0;
  double dd = 1.0 - (S - 1.0) * mu;
  double pH = rho0 * c0 * c0 * mu * (1.0 + mu) / (dd * dd);
  e = (T > Tr) ? alpha * (T - Tr) : 0;
  double pF = pH + Gamma * (e - e0);
  if (damage > 0.0 && pF < 0.0) {
    if (damage >= 1.0) pF = 0;
    else pF *= 1.0 - damage;
  }
  if (Q1 != 0 || Q2 != 0) {
    double tre = trace(D);
    if (tre < 0) pF += rho * cellsize * (Q1 * cellsize * tre * tre - Q2 * c0 * std::sqrt(J) * tre);
  }
  return pF;
}

// Strength::update_deviatoric_stress: src/strength_linear.cpp:59-71,
// src/strength_plastic.cpp:62-115, src/strength_jc.cpp:100-184,
// src/strength_swift.cpp:77-147, src/strength_fluid.cpp:46-58
M3 strength_update(const Mat &m, double dt, const M3 &sigma, const M3 &D, double &dep, double epsp, double epsdot,
                   double damage, double T) {
  const double *p = m.d.str_p;
  switch (m.d.strength) {
    case STR_LINEAR:
      return add(deviator(sigma), scale(dt, scale(2.0 * p[0] * (1 - damage), deviator(D))));
    case STR_FLUID:
      return scale(2.0 * p[0], deviator(D));
    case STR_PLASTIC: {
      double Gd = p[0] * (1 - damage), syD = p[1] * (1 - damage);
      M3 tr_dev = add(deviator(sigma), scale(dt, scale(2.0 * Gd, deviator(D))));
      double J2 = std::sqrt(3. / 2.) * fnorm(tr_dev);
      if (J2 < syD) { dep = 0.0; return tr_dev; }
      dep = (J2 - syD) / (3.0 * Gd);
      return scale(syD / J2, tr_dev);
    }
    case STR_JC:
    case STR_SWIFT: {
      if (damage >= 1.0) return zero3();
      double G = p[0], ys;
      if (m.d.strength == STR_JC) {
        double A = p[1], B = p[2], n = p[3], epsdot0 = p[4], C = p[5], mm = p[6], Tr = p[7], Tm = p[8];
        double ratio = std::max(epsdot / epsdot0, 1.0);
        ys = (epsp < 1.0e-10) ? A : A + B * std::pow(epsp, n);
        if (C != 0) ys *= std::pow(1.0 + ratio, C);
        if (T < Tm) {
          if (mm != 0 && T >= Tr) ys *= 1.0 - std::pow((T - Tr) / (Tm - Tr), mm);
        } else ys = 0;
      } else {
        double A = p[1], B = p[2], C = p[3], n = p[4];
        ys = (epsp > 1.0e-10 && epsp > C) ? A + B * std::pow(epsp - C, n) : A;
      }
      double Gd = G;
      if (damage > 0) { Gd *= (1 - damage); ys *= (1 - damage); }
      M3 trial_dev = deviator(add(sigma, scale(dt * 2.0 * Gd, D)));
      double J2 = SQRT_3_OVER_2 * fnorm(trial_dev);
      if (J2 < ys) { dep = 0.0; return trial_dev; }
      dep = (J2 - ys) / (3.0 * Gd);
      return scale(ys / J2, trial_dev);
    }
  }
  return zero3();
}

// DamageJohnsonCook::compute_damage, src/damage_jc.cpp:91-143
void damage_update(const Mat &m, double &dinit, double &damage, double pH, const M3 &Sdev, double epsdot, double dep,
                   double T) {
  const double *p = m.d.dam_p;
  double d1 = p[0], d2 = p[1], d3 = p[2], d4 = p[3], d5 = p[4], epsdot0 = p[5], Tr = p[6], Tm = p[7];
  if (dep == 0 && damage >= 1.0) return;
  double vm = SQRT_3_OVER_2 * fnorm(Sdev);
  double triax = 0.0;
  if (pH != 0.0 && vm != 0.0) triax = -pH / (vm + 0.001 * std::fabs(pH));
  if (triax <= -3) { dinit = 0; return; }
  double ef = d1 + d2 * std::exp(d3 * triax);
  if (d4 > 0.0 && epsdot > epsdot0) ef *= (1.0 + d4 * std::log(epsdot / epsdot0));
  if (d5 > 0.0 && T >= Tr) ef *= 1 + d5 * (T - Tr) / (Tm - Tr);
  dinit += dep / ef;
  if (dinit >= 1.0) damage = std::min((dinit - 1.0) * 10, 1.0);
}

bool fail(Sim &s, const std::string &msg) {
  if (s.err.empty()) s.err = msg;
  return false;
}

// Solid::update_deformation_gradient, src/solid.cpp:1155-1244
bool update_deformation_gradient(Sim &s, Solid &S) {
  const Mat &m = s.mats[S.mat];
  bool nh = m.type == MAT_NEO_HOOKEAN;
  bool TL = s.method == TLMPM;
  int bad = -1;
#pragma omp parallel for schedule(static)
  for (int ip = 0; ip < S.np; ip++) {
    if (TL) S.F[ip] = add(S.F[ip], scale(s.dt, S.Fdot[ip]));
    else S.F[ip] = mul(add(eye3(), scale(s.dt, S.L[ip])), S.F[ip]);
    S.Finv[ip] = inv(S.F[ip]);
    S.J[ip] = det(S.F[ip]);
    S.vol[ip] = S.J[ip] * S.vol0[ip];
    if (S.J[ip] <= 0.0 && S.damage[ip] < 1.0) {
#pragma omp critical
      bad = ip;
    }
    S.rho[ip] = S.rho0[ip] / S.J[ip];
    if (!nh) {
      if (TL) {
        bool ok = poldec(S.F[ip], S.R[ip]);
        S.L[ip] = mul(S.Fdot[ip], S.Finv[ip]);
        S.D[ip] = scale(0.5, mul(mul(tr(S.R[ip]), add(S.L[ip], tr(S.L[ip]))), S.R[ip]));
        if (!ok) {
#pragma omp critical
          bad = ip;
        }
      } else {
        S.D[ip] = scale(0.5, add(S.L[ip], tr(S.L[ip])));
      }
    }
  }
  if (bad >= 0) return fail(s, "J<=0 or polar decomposition failed for particle " + std::to_string(bad));
  return true;
}

// Solid::update_stress, src/solid.cpp:1246-1438
bool update_stress(Sim &s, Solid &S) {
  const Mat &m = s.mats[S.mat];
  Grid &g = s.grids[S.grid];
  bool TL = s.method == TLMPM;
  double dt = s.dt;
  M3 eye = eye3();
  if (m.type == MAT_LINEAR) {
#pragma omp parallel for schedule(static)
    for (int ip = 0; ip < S.np; ip++) {
      M3 inc = scale(dt, S.D[ip]);
      S.strain_el[ip] = add(S.strain_el[ip], inc);
      S.sigma[ip] = add(S.sigma[ip], add(scale(2 * m.G, inc), scale(m.lambda * trace(inc), eye)));
      if (TL)
        S.vol0PK1[ip] = scale(S.vol0[ip] * S.J[ip], mul(mul(mul(S.R[ip], S.sigma[ip]), tr(S.R[ip])), tr(S.Finv[ip])));
    }
  } else if (m.type == MAT_NEO_HOOKEAN) {
#pragma omp parallel for schedule(static)
    for (int ip = 0; ip < S.np; ip++) {
      M3 FinvT = tr(S.Finv[ip]);
      M3 PK1 = add(scale(m.G, sub(S.F[ip], FinvT)), scale(m.lambda * std::log(S.J[ip]), FinvT));
      S.vol0PK1[ip] = scale(S.vol0[ip], PK1);
      S.sigma[ip] = scale(1.0 / S.J[ip], mul(S.F[ip], tr(PK1)));
      S.strain_el[ip] = scale(0.5, sub(mul(tr(S.F[ip]), S.F[ip]), eye));
    }
  } else {
    bool has_T = m.cp != 0;
    double tav = 1000 * g.cellsize / m.signal_velocity;
#pragma omp parallel for schedule(static)
    for (int ip = 0; ip < S.np; ip++) {
      double pH = 0, dep = 0;
      double T = has_T ? S.T[ip] : 0.0;
      pH = eos_pressure(m, S.ienergy[ip], S.J[ip], S.rho[ip], S.damage[ip], S.D[ip], g.cellsize, T);
      if (has_T) pH += m.d.temp_p[3] * (m.d.temp_p[4] - T);  // TemperaturePlasticWork::compute_thermal_pressure
      M3 sdev = strength_update(m, dt, S.sigma[ip], S.D[ip], dep, S.epsp[ip], S.epsdot[ip], S.damage[ip], T);
      S.epsp[ip] += dep;
      S.epsdot[ip] -= S.epsdot[ip] * dt / tav;
      S.epsdot[ip] += dep / tav;
      S.epsdot[ip] = std::max(0.0, S.epsdot[ip]);
      if (m.d.damage >= 0)
        damage_update(m, S.damage_init[ip], S.damage[ip], pH, sdev, S.epsdot[ip], dep, s.thermal ? S.T[ip] : 0.0);
      if (has_T) {
        double flow = SQRT_3_OVER_2 * fnorm(sdev);
        // TemperaturePlasticWork::compute_heat_source, src/temperature_plastic_work.cpp:59-65
        S.gamma[ip] = (S.T[ip] < m.d.temp_p[5]) ? m.d.temp_p[0] * flow * S.epsdot[ip] : 0;
        S.gamma[ip] *= (TL ? S.vol0[ip] : S.vol[ip]) * m.invcp;
      }
      if (S.damage[ip] == 0 || pH >= 0) S.sigma[ip] = add(scale(-pH, eye), sdev);
      else S.sigma[ip] = add(scale(-pH * (1.0 - S.damage[ip]), eye), sdev);
      double trD = s.dt * trace(S.D[ip]) + trace(S.strain_el[ip]);
      if (S.damage[ip] > 1e-10)
        S.strain_el[ip] = add(scale(trD / 3.0, eye), scale(1.0 / (m.G * (1 - S.damage[ip])), sdev));
      else
        S.strain_el[ip] = add(scale(trD / 3.0, eye), scale(1.0 / m.G, sdev));
      if (TL)
        S.vol0PK1[ip] = scale(S.vol0[ip] * S.J[ip], mul(mul(mul(S.R[ip], S.sigma[ip]), tr(S.R[ip])), tr(S.Finv[ip])));
    }
  }
  // wave speed and dtCFL, src/solid.cpp:1376-1437
  double maxc = 0, min_h_ratio = 1.0;
  bool nan = false;
#pragma omp parallel for schedule(static) reduction(max : maxc) reduction(min : min_h_ratio) reduction(|| : nan)
  for (int ip = 0; ip < S.np; ip++) {
    if (S.damage[ip] >= 1.0) continue;
    double c = std::sqrt((m.K + FOUR_THIRD * m.G) / S.rho[ip]) +
               std::max(std::max(std::fabs(S.v[3 * ip]), std::fabs(S.v[3 * ip + 1])), std::fabs(S.v[3 * ip + 2]));
    if (std::isnan(c)) nan = true;
    maxc = std::max(maxc, c);
    if (TL) {
      double re[3];
      eig_real_parts(S.F[ip], re);
      for (int k = 0; k < 3; k++) min_h_ratio = std::min(min_h_ratio, std::fabs(re[k]));
    }
  }
  if (nan) return fail(s, "max_p_wave_speed is nan");
  if (min_h_ratio == 0) return fail(s, "min_h_ratio == 0");
  S.dtCFL = std::min(S.dtCFL, g.cellsize * min_h_ratio / maxc);
  if (std::isnan(S.dtCFL)) return fail(s, "dtCFL is nan");
  return true;
}

// Solid::update_heat_flux, src/solid.cpp:2812-2839
void update_heat_flux(Sim &s, Solid &S, bool doublemapping) {
  Grid &g = s.grids[S.grid];
  const Mat &m = s.mats[S.mat];
  const std::vector<double> &Tn = doublemapping ? g.T : g.Tu;
  bool TL = s.method == TLMPM;
#pragma omp parallel for schedule(static)
  for (int ip = 0; ip < S.np; ip++) {
    double q[3] = {0, 0, 0};
    for (size_t j = 0; j < S.neigh_pn[ip].size(); j++) {
      int in = S.neigh_pn[ip][j];
      for (int d = 0; d < 3; d++) q[d] -= S.wfd_pn[ip][3 * j + d] * Tn[in];
    }
    double f = (TL ? S.vol0[ip] : S.vol[ip]) * m.invcp * m.kappa;
    for (int d = 0; d < 3; d++) S.q[3 * ip + d] = q[d] * f;
  }
}

// one time step, src/usl.cpp:43-92 and src/musl.cpp:43-93
// Contact fixes, initial_integrate: every pair (ip1 of solid1, ip2 of
// solid2) in the reference's loop order, so that each particle's mbp sums its
// pairs in the same order (FixContactMinPenetration::initial_integrate,
// src/fix_contact_min_penetration.cpp:83-235; FixContactHertz::initial_integrate,
// src/fix_contact_hertz.cpp:82-197).  Only 2-D and 3-D runs take a contact.
void contact_forces(Sim &s, Contact &C) {
  Solid &A = s.solids[C.s1], &B = s.solids[C.s2];
  const Mat &ma = s.mats[A.mat], &mb = s.mats[B.mat];
  const double Estar = 1.0 / ((1 - ma.nu * ma.nu) / ma.E + (1 - mb.nu * mb.nu) / mb.E);
  const double alpha = ma.kappa / (ma.kappa + mb.kappa);
  const double cmax = std::max(s.grids[A.grid].cellsize, s.grids[B.grid].cellsize);
  const bool hertz = C.kind == CONTACT_HERTZ;
  // the reference's own constant for 4/3 in both fixes (#define four_thirds)
  const double hertz_coef = s.dim == 3 ? 1.333333333 : 0.25 * M_PI;
  const int dim = s.dim;
  double ft[3] = {0, 0, 0};
  // Rp; the 2-D min-penetration fix divides the volume by r in axisymmetric runs
  auto radius = [&](double vol, double r) {
    if (dim == 3) return hertz ? 0.5 * std::pow(vol, 0.333333333) : 0.5 * std::cbrt(vol);
    if (s.axisym && !hertz) return 0.5 * std::sqrt(vol / r);
    return 0.5 * std::sqrt(vol);
  };
  if (dim == 2 || dim == 3) {
    for (int i = 0; i < A.np; i++) {
      for (int j = 0; j < B.np; j++) {
        double dx[3];
        for (int d = 0; d < 3; d++) dx[d] = B.x[3 * j + d] - A.x[3 * i + d];
        // per-axis screen on the larger cellsize (the 2-D min-penetration fix
        // screens x and y only; z differences are zero in 2-D runs)
        bool near = true;
        const int ns = (dim == 2 && !hertz) ? 2 : 3;
        for (int d = 0; d < ns; d++) near = near && dx[d] < cmax && dx[d] > -cmax;
        if (!near) continue;
        const double R1 = radius(A.vol[i], A.x[3 * i]), R2 = radius(B.vol[j], B.x[3 * j]), Rp = R1 + R2;
        for (int d = 0; d < ns; d++) near = near && dx[d] < Rp && dx[d] > -Rp;
        if (!near) continue;
        const double r = std::sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
        if (!(r < Rp)) continue;
        double f[3];
        if (hertz) {
          const double p = Rp - r;  // penetration
          const double fmag = hertz_coef * Estar * std::sqrt(R1 * R2 / (R1 + R2) * p * p * p);
          for (int d = 0; d < 3; d++) f[d] = fmag * dx[d] / r;
          for (int d = 0; d < 3; d++) {
            A.mbp[3 * i + d] -= f[d];
            B.mbp[3 * j + d] += f[d];
            ft[d] += f[d];
          }
          continue;
        }
        const double ir = 1.0 / r;
        const double fmag = A.mass[i] * B.mass[j] / ((A.mass[i] + B.mass[j]) * s.dt * s.dt) * (1 - Rp * ir);
        for (int d = 0; d < 3; d++) f[d] = fmag * dx[d];
        if (C.mu != 0) {
          double dv[3], vt[3];
          for (int d = 0; d < 3; d++) dv[d] = B.v[3 * j + d] - A.v[3 * i + d];
          const double dvn = (dv[0] * dx[0] + dv[1] * dx[1] + dv[2] * dx[2]) * ir * ir;
          for (int d = 0; d < 3; d++) vt[d] = dv[d] - dvn * dx[d];
          const double vtn = std::sqrt(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
          if (vtn != 0) {
            const double ffric = C.mu * fmag * r;
            for (int d = 0; d < 3; d++) f[d] -= ffric * (vt[d] / vtn);
            if (s.thermal) {
              // frictional heat: split alpha / (1 - alpha) in 2-D; in 3-D the
              // reference gives both solids the share alpha
              if (dim == 2) {
                const double g = ffric * vtn * s.dt;
                A.gamma[i] += alpha * A.vol0[i] * ma.invcp * g;
                B.gamma[j] += (1.0 - alpha) * B.vol0[j] * mb.invcp * g;
              } else {
                const double g = alpha * ffric * vtn * s.dt;
                A.gamma[i] += A.vol0[i] * ma.invcp * g;
                B.gamma[j] += B.vol0[j] * mb.invcp * g;
              }
            }
          }
        }
        for (int d = 0; d < 3; d++) {
          A.mbp[3 * i + d] += f[d];
          B.mbp[3 * j + d] -= f[d];
          ft[d] += f[d];
        }
      }
    }
  }
  for (int d = 0; d < 3; d++) C.ftot[d] = ft[d];
}

bool step(Sim &s) {
  bool TL = s.method == TLMPM;
  bool musl = s.scheme == MUSL;
  s.ntimestep++;
  // compute_grid_weight_functions_and_gradients
  if (!TL || s.update_wf) {
    for (auto &S : s.solids) build_neighbours(s, S);
    s.update_wf = false;
  }
  // reset(): src/tlmpm.cpp:516-525, src/ulmpm.cpp:553-563
  for (auto &S : s.solids) {
    S.dtCFL = 1.0e22;
    std::fill(S.mbp.begin(), S.mbp.end(), 0.0);
  }
  // initial_integrate: the contact fixes (src/musl.cpp:49, src/usl.cpp:49, src/usf.cpp:49)
  for (auto &C : s.contacts) contact_forces(s, C);
  // particles_to_grid (src/tlmpm.cpp:342-366, src/ulmpm.cpp:338-378), body
  // forces, update_grid_state and the velocity fixes
  auto p2g_grid = [&]() {
  if (TL) {
    if (s.update_mass_nodes) {
      for (auto &S : s.solids) compute_mass_nodes(S, s.grids[S.grid], true);
      s.update_mass_nodes = false;
    }
    for (auto &S : s.solids) {
      Grid &g = s.grids[S.grid];
      compute_velocity_nodes(s, S, g, true);
      compute_external_forces_nodes(S, g, true);
      compute_internal_forces_nodes_TL(s, S, g);
      if (s.thermal) {
        compute_temperature_nodes(S, g, true);
        compute_temperature_forces(S, g, true);
      }
    }
  } else {
    Grid &g = s.grids[0];
    for (size_t i = 0; i < s.solids.size(); i++) compute_mass_nodes(s.solids[i], g, i == 0);
    for (size_t i = 0; i < s.solids.size(); i++) {
      compute_velocity_nodes(s, s.solids[i], g, i == 0);
      compute_forces_nodes_UL(s, s.solids[i], g, i == 0);
      if (s.thermal) {
        compute_temperature_nodes(s.solids[i], g, i == 0);
        compute_temperature_forces(s.solids[i], g, i == 0);
      }
    }
  }
  // post_particles_to_grid: FixBodyforce, src/fix_body_force.cpp:106-179
  for (auto &fx : s.fixes) {
    if (fx.kind != FIX_BODY_FORCE) continue;
    Grid &g = s.grids[fx.grid];
    for (int in = 0; in < g.nn; in++)
      if (g.mass[in] > 0 && fx.mask[in])
        for (int d = 0; d < 3; d++)
          if (fx.set[d]) g.mb[3 * in + d] += fx.c[d][0] * g.mass[in];
  }
  // update_grid_state: Grid::update_grid_velocities src/grid.cpp:448-466,
  // Grid::update_grid_temperature src/grid.cpp:1354-1361
  for (auto &g : s.grids) {
#pragma omp parallel for schedule(static)
    for (int in = 0; in < g.nn; in++) {
      for (int d = 0; d < 3; d++)
        g.vu[3 * in + d] = (g.mass[in] != 0) ? g.v[3 * in + d] + s.dt * (g.f[3 * in + d] + g.mb[3 * in + d]) / g.mass[in]
                                             : g.v[3 * in + d];
      if (s.thermal)
        g.Tu[in] = (g.mass[in] != 0) ? g.T[in] + s.dt * (g.Qint[in] + g.Qext[in]) / g.mass[in] : g.T[in];
    }
  }
  // post_update_grid_state: FixVelocityNodes, src/fix_velocity_nodes.cpp:130-225
  for (auto &fx : s.fixes) {
    if (fx.kind != FIX_VEL_NODES) continue;
    Grid &g = s.grids[fx.grid];
    double vnow[3], vold[3];
    for (int d = 0; d < 3; d++) {
      vnow[d] = fix_value(fx.c[d], s.time);
      vold[d] = fix_value(fx.c[d], s.time - s.dt);
    }
    for (int in = 0; in < g.nn; in++)
      if (fx.mask[in])
        for (int d = 0; d < 3; d++)
          if (fx.set[d]) { g.vu[3 * in + d] = vnow[d]; g.v[3 * in + d] = vold[d]; }
  }
  };
  // USL: compute_rate_deformation_gradient(false) before grid_to_points
  auto rate = [&](Solid &S, bool doublemapping) {
    Grid &g = s.grids[S.grid];
    const std::vector<double> &vn = doublemapping ? g.v : g.vu;
    const std::vector<double> &pos = TL ? S.x0 : S.x;
#pragma omp parallel for schedule(static)
    for (int ip = 0; ip < S.np; ip++) {
      M3 G = zero3();
      if (s.apic) {
        // compute_rate_deformation_gradient_{TL,UL}_APIC, src/solid.cpp:1006-1153:
        // sum w v_node (x0_node - x_p)^T, times Di
        for (size_t j = 0; j < S.neigh_pn[ip].size(); j++) {
          int in = S.neigh_pn[ip][j];
          const double w = S.wf_pn[ip][j];
          for (int a = 0; a < s.dim; a++)
            for (int b = 0; b < s.dim; b++) G(a, b) += vn[3 * in + a] * (g.x0[3 * in + b] - pos[3 * ip + b]) * w;
          // axisymmetric: v_r w / r (src/solid.cpp:1046-1058, 1120-1132); Di(2,2) = 1 in 2-D
          if (s.axisym) G(2, 2) += vn[3 * in] * w / pos[3 * ip];
        }
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++) G(a, b) *= S.Di[b];
      } else {
        for (size_t j = 0; j < S.neigh_pn[ip].size(); j++) {
          int in = S.neigh_pn[ip][j];
          const double *gw = &S.wfd_pn[ip][3 * j];
          for (int a = 0; a < s.dim; a++)
            for (int b = 0; b < s.dim; b++) G(a, b) += vn[3 * in + a] * gw[b];
          // axisymmetric: Fdot(2,2) / L(2,2) += v_r w / r (src/solid.cpp:818-829, 900-913)
          if (s.axisym) G(2, 2) += vn[3 * in] * S.wf_pn[ip][j] / pos[3 * ip];
        }
      }
      if (TL) S.Fdot[ip] = G;  // src/solid.cpp:798-858
      else S.L[ip] = G;        // src/solid.cpp:860-936
    }
  };
  // grid_to_points and advance_particles
  auto g2p = [&]() -> bool {
  // grid_to_points: Solid::compute_particle_accelerations_velocities_and_positions src/solid.cpp:576-635
  int left = -1;
  for (auto &S : s.solids) {
    Grid &g = s.grids[S.grid];
    double inv_dt = 1.0 / s.dt;
#pragma omp parallel for schedule(static)
    for (int ip = 0; ip < S.np; ip++) {
      double vu[3] = {0, 0, 0}, a[3] = {0, 0, 0};
      for (size_t j = 0; j < S.neigh_pn[ip].size(); j++) {
        int in = S.neigh_pn[ip][j];
        double w = S.wf_pn[ip][j];
        for (int d = 0; d < 3; d++) {
          vu[d] += w * g.vu[3 * in + d];
          a[d] += w * (g.vu[3 * in + d] - g.v[3 * in + d]);
        }
      }
      for (int d = 0; d < 3; d++) {
        S.vu[3 * ip + d] = vu[d];
        S.a[3 * ip + d] = a[d] * inv_dt;
        S.f[3 * ip + d] = S.a[3 * ip + d] * S.mass[ip];
        // ASFLIP: Solid::compute_particle_accelerations_velocities leaves x
        if (!s.asflip) S.x[3 * ip + d] += s.dt * vu[d];
      }
      if (!TL) {
        const double *x = &S.x[3 * ip];
        if (!(x[0] >= s.boxlo[0] && x[0] <= s.boxhi[0] && x[1] >= s.boxlo[1] && x[1] <= s.boxhi[1] &&
              x[2] >= s.boxlo[2] && x[2] <= s.boxhi[2])) {
#pragma omp critical
          left = ip;
        }
      }
      if (s.thermal) {  // Solid::update_particle_temperature src/solid.cpp:2802-2810
        double T = 0;
        for (size_t j = 0; j < S.neigh_pn[ip].size(); j++) T += S.wf_pn[ip][j] * g.Tu[S.neigh_pn[ip][j]];
        S.T[ip] = T;
      }
    }
  }
  if (left >= 0) return fail(s, "particle " + std::to_string(left) + " left the domain");
  // advance_particles: Solid::update_particle_velocities src/solid.cpp:786-790
  for (auto &S : s.solids)
#pragma omp parallel for schedule(static)
    for (int ip = 0; ip < S.np; ip++)
      for (int d = 0; d < 3; d++) {
        S.v[3 * ip + d] = (1 - s.pic_flip) * S.vu[3 * ip + d] + s.pic_flip * (S.v[3 * ip + d] + s.dt * S.a[3 * ip + d]);
        // ASFLIP: Solid::update_particle_velocities_and_positions, src/solid.cpp:791-796
        if (s.asflip) S.x[3 * ip + d] += s.dt * S.v[3 * ip + d];
      }
    return true;
  };
  // update_time and adjust_dt
  auto finish = [&]() -> bool {
    // update_time: src/update.cpp:201-206
    s.time += s.dt;
    // adjust_dt: src/tlmpm.cpp:489-514, src/ulmpm.cpp:525-551
    if (!s.dt_constant) {
      double dtCFL = 1.0e22;
      for (auto &S : s.solids) {
        dtCFL = std::min(dtCFL, S.dtCFL);
        if (dtCFL == 0 || std::isnan(dtCFL)) return fail(s, "dtCFL == 0 or nan");
      }
      s.dt = dtCFL * s.dt_factor;
    }
    return true;
  };
  if (s.scheme == USF) {
    // USF::run, src/usf.cpp:43-86: velocities to the grid, stress from the
    // grid velocities, then the forces of the new stress
    p2g_grid();
    for (auto &S : s.solids) rate(S, true);
    for (auto &S : s.solids)
      if (!update_deformation_gradient(s, S)) return false;
    for (auto &S : s.solids)
      if (!update_stress(s, S)) return false;
    p2g_grid();
    if (!g2p()) return false;
    if (TL)
      for (auto &g : s.grids)
        for (int q = 0; q < 3 * g.nn; q++) g.x[q] += s.dt * g.v[q];
    return finish();
  }
  p2g_grid();
  if (!musl)
    for (auto &S : s.solids) rate(S, false);
  if (!g2p()) return false;
  if (musl) {
    // velocities_to_grid: src/tlmpm.cpp:440-452, src/ulmpm.cpp:476-496
    if (TL) {
      for (auto &S : s.solids) {
        compute_velocity_nodes(s, S, s.grids[S.grid], true);
        if (s.thermal) compute_temperature_nodes(S, s.grids[S.grid], true);
      }
    } else {
      for (size_t i = 0; i < s.solids.size(); i++) {
        compute_velocity_nodes(s, s.solids[i], s.grids[0], i == 0);
        if (s.thermal) compute_temperature_nodes(s.solids[i], s.grids[0], i == 0);
      }
    }
    // post_velocities_to_grid: src/fix_velocity_nodes.cpp:227-271
    for (auto &fx : s.fixes) {
      if (fx.kind != FIX_VEL_NODES) continue;
      Grid &g = s.grids[fx.grid];
      for (int in = 0; in < g.nn; in++)
        if (fx.mask[in])
          for (int d = 0; d < 3; d++)
            if (fx.set[d]) g.v[3 * in + d] = fix_value(fx.c[d], s.time);
    }
  }
  // update_grid_positions: Grid::update_grid_positions src/grid.cpp:468-474 (TL only)
  if (TL)
    for (auto &g : s.grids)
      for (int k = 0; k < 3 * g.nn; k++) g.x[k] += s.dt * g.v[k];
  if (musl)
    for (auto &S : s.solids) rate(S, true);
  for (auto &S : s.solids)
    if (!update_deformation_gradient(s, S)) return false;
  for (auto &S : s.solids) {
    if (!update_stress(s, S)) return false;
    if (s.thermal) update_heat_flux(s, S, musl);
  }
  return finish();
}

}  // namespace

// ---------------------------------------------------------------- C ABI
extern "C" {

void *om_create(int method, int scheme, int basis, int dim, double pic_flip, int thermal, double dt, double dt_factor,
                int dt_constant, const double *boxlo, const double *boxhi) {
  Sim *s = new Sim();
  s->method = method; s->scheme = scheme; s->basis = basis; s->dim = dim;
  s->pic_flip = pic_flip; s->thermal = thermal != 0;
  s->dt = dt; s->dt_factor = dt_factor; s->dt_constant = dt_constant != 0;
  for (int d = 0; d < 3; d++) { s->boxlo[d] = boxlo[d]; s->boxhi[d] = boxhi[d]; }
  if (basis == CUBIC) { s->bf = bf_cubic; s->dbf = dbf_cubic; }
  else if (basis == BERNSTEIN) { s->bf = bf_bern; s->dbf = dbf_bern; }
  else if (basis == QUADRATIC) { s->bf = bf_quad; s->dbf = dbf_quad; }
  return s;
}
void om_destroy(void *h) { delete (Sim *)h; }
// sub-method APIC: PIC velocity update (PIC_FLIP = 0) and affine transfers;
// the reference supports it with the cubic spline (and linear TLMPM)
// kind: 0 PIC/FLIP, 1 APIC, 2 AFLIP, 3 ASFLIP, 4 MLS (Update::create_method,
// src/update.cpp:129-149).  TLMPM takes the affine path for APIC only
// (src/tlmpm.cpp:82-84, 354); ULMPM for all four (src/ulmpm.cpp:79-85).
int om_set_transfer(void *h, int kind) {
  Sim *s = (Sim *)h;
  const bool TL = s->method == TLMPM;
  if (kind < 0 || kind > 4 || (kind == 4 && TL)) { s->err = "unsupported sub-method"; return -1; }
  const bool affine = kind == 1 || (!TL && kind >= 2);
  if (affine && s->basis != CUBIC && s->basis != QUADRATIC && !(s->basis == LINEAR && TL)) {
    s->err = "affine transfers are restated for the cubic and quadratic splines, and the linear basis in TLMPM";
    return -1;
  }
  s->apic = affine;
  s->asflip = !TL && kind == 3;
  s->mls = !TL && kind == 4;
  if (kind == 1 || kind == 4) s->pic_flip = 0;
  return 0;
}
// Domain::set_axisymmetric (src/domain.cpp:558-570): 2-D only; the reference
// stops thermo-mechanical axisymmetric runs (src/solid.cpp:2789-2792)
int om_set_axisymmetric(void *h, int on) {
  Sim *s = (Sim *)h;
  if (on && (s->dim != 2 || s->thermal)) { s->err = "axisymmetric runs are 2-D and mechanical"; return -1; }
  s->axisym = on != 0;
  return 0;
}
const char *om_error(void *h) { return ((Sim *)h)->err.c_str(); }

int om_add_material(void *h, const om_material *m) {
  Sim *s = (Sim *)h;
  s->mats.emplace_back(*m);
  return (int)s->mats.size() - 1;
}
int om_add_grid(void *h, const double *boundlo, const double *boundhi, double cellsize) {
  Sim *s = (Sim *)h;
  s->grids.emplace_back();
  grid_init(*s, s->grids.back(), boundlo, boundhi, cellsize);
  return (int)s->grids.size() - 1;
}
// dims[0..5] = nx ny nz nx_global ny_global nz_global; returns number of nodes
int om_grid_info(void *h, int gi, int *dims, double *lo_h) {
  Grid &g = ((Sim *)h)->grids[gi];
  dims[0] = g.nx; dims[1] = g.ny; dims[2] = g.nz; dims[3] = g.nxg; dims[4] = g.nyg; dims[5] = g.nzg;
  lo_h[0] = g.lo[0]; lo_h[1] = g.lo[1]; lo_h[2] = g.lo[2]; lo_h[3] = g.h;
  return g.nn;
}
int om_grid_ntype(void *h, int gi, int *out) {
  Grid &g = ((Sim *)h)->grids[gi];
  std::memcpy(out, g.ntype.data(), sizeof(int) * 3 * g.nn);
  return g.nn;
}
int om_add_solid(void *h, int grid, int mat, int np, const double *x0, const double *v, const double *mass,
                 const double *vol0, double T0) {
  Sim *s = (Sim *)h;
  s->solids.emplace_back();
  Solid &S = s->solids.back();
  const Mat &m = s->mats[mat];
  S.grid = grid; S.mat = mat; S.np = np; S.T0 = T0;
  S.x0.assign(x0, x0 + 3 * np); S.x = S.x0;
  S.v.assign(v, v + 3 * np);
  auto z3 = [&](std::vector<double> &a) { a.assign(3 * np, 0.0); };
  z3(S.vu); z3(S.a); z3(S.mbp); z3(S.f); z3(S.q);
  M3 Z = zero3(), I = eye3();
  S.sigma.assign(np, Z); S.strain_el.assign(np, Z); S.vol0PK1.assign(np, Z); S.L.assign(np, Z);
  S.F.assign(np, I); S.R.assign(np, I); S.D.assign(np, Z); S.Finv.assign(np, Z); S.Fdot.assign(np, Z);
  S.mass.assign(mass, mass + np);
  S.vol0.assign(vol0, vol0 + np); S.vol = S.vol0;
  S.rho0.assign(np, m.rho0); S.rho = S.rho0;
  S.epsp.assign(np, 0); S.epsdot.assign(np, 0); S.damage.assign(np, 0); S.damage_init.assign(np, 0);
  S.ienergy.assign(np, 0); S.J.assign(np, 1.0); S.gamma.assign(np, 0);
  // src/solid.cpp:2297-2306: T = T0 only for thermo-mechanical runs (value-initialised otherwise)
  S.T.assign(np, s->thermal ? T0 : 0.0);
  Grid &g = s->grids[grid];
  S.neigh_pn.resize(np); S.wf_pn.resize(np); S.wfd_pn.resize(np);
  S.neigh_np.resize(g.nn); S.wf_np.resize(g.nn); S.wfd_np.resize(g.nn);
  S.dtCFL = 1e22;
  return (int)s->solids.size() - 1;
}
int om_add_fix(void *h, int kind, int grid, const uint8_t *mask, const int *set, const double *coef) {
  Sim *s = (Sim *)h;
  Fix f;
  f.kind = kind; f.grid = grid;
  f.mask.assign(mask, mask + s->grids[grid].nn);
  for (int d = 0; d < 3; d++) {
    f.set[d] = set[d];
    for (int k = 0; k < 4; k++) f.c[d][k] = coef[4 * d + k];
  }
  s->fixes.push_back(f);
  return (int)s->fixes.size() - 1;
}
// Solid::np_per_cell; linear APIC accepts 1 or 2 (src/solid.cpp:1453-1462)
int om_set_np_per_cell(void *h, int si, int n) {
  Sim *s = (Sim *)h;
  if (s->apic && s->basis == LINEAR && n != 1 && n != 2) {
    s->err = "Number of particle per cell not supported with linear shape functions and APIC";
    return -1;
  }
  s->solids[si].np_per_cell = n;
  return 0;
}
// contact fix: kind 0 contact/minimize_penetration, 1 contact/hertz
int om_add_contact(void *h, int kind, int s1, int s2, double mu) {
  Sim *s = (Sim *)h;
  Contact C;
  C.kind = kind; C.s1 = s1; C.s2 = s2; C.mu = mu;
  s->contacts.push_back(C);
  return (int)s->contacts.size() - 1;
}
void om_contact_force(void *h, int k, double *out) {
  Sim *s = (Sim *)h;
  for (int d = 0; d < 3; d++) out[d] = s->contacts[k].ftot[d];
}
int om_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}
// returns 0 on success, -1 on a reference error (message via om_error)
int om_run(void *h, int nsteps) {
  Sim *s = (Sim *)h;
  for (int i = 0; i < nsteps; i++)
    if (!step(*s)) return -1;
  return 0;
}
// run until time >= maxtime (RunTime::command, src/run_time.cpp); returns steps done or -1
int om_run_time(void *h, double maxtime) {
  Sim *s = (Sim *)h;
  int n = 0;
  while (s->time < maxtime) {
    if (!step(*s)) return -1;
    n++;
    if (s->time > maxtime) break;
  }
  return n;
}
void om_scalars(void *h, double *out) {
  Sim *s = (Sim *)h;
  out[0] = s->time; out[1] = s->dt; out[2] = (double)s->ntimestep;
}
// the clock, as a restart sets it (Update::read_restart, src/update.cpp:363-393):
// the next step runs with this dt, and adjust_dt sets the one after
void om_set_scalars(void *h, double time, double dt) {
  Sim *s = (Sim *)h;
  s->time = time; s->dt = dt;
}
// Particle fields: 0 x, 1 x0, 2 v, 3 sigma (as stored), 4 sigma rotated (R sigma R^T for TL dumps,
// src/dump_particle.cpp:98-102), 5 F, 6 eps_p, 7 epsdot_p, 8 damage, 9 damage_init, 10 T, 11 J, 12 vol,
// 13 strain_el, 14 vol0PK1, 15 mass
int om_get_particles(void *h, int si, int field, double *out) {
  Sim *s = (Sim *)h;
  Solid &S = s->solids[si];
  auto cpm = [&](const std::vector<M3> &A) { for (int i = 0; i < S.np; i++) std::memcpy(out + 9 * i, A[i].a, 72); };
  auto cps = [&](const std::vector<double> &A) { std::memcpy(out, A.data(), sizeof(double) * A.size()); };
  switch (field) {
    case 0: cps(S.x); break;
    case 1: cps(S.x0); break;
    case 2: cps(S.v); break;
    case 3: cpm(S.sigma); break;
    case 4:
      for (int i = 0; i < S.np; i++) {
        M3 r = s->method == TLMPM ? mul(mul(S.R[i], S.sigma[i]), tr(S.R[i])) : S.sigma[i];
        std::memcpy(out + 9 * i, r.a, 72);
      }
      break;
    case 5: cpm(S.F); break;
    case 6: cps(S.epsp); break;
    case 7: cps(S.epsdot); break;
    case 8: cps(S.damage); break;
    case 9: cps(S.damage_init); break;
    case 10: cps(S.T); break;
    case 11: cps(S.J); break;
    case 12: cps(S.vol); break;
    case 13: cpm(S.strain_el); break;
    case 14: cpm(S.vol0PK1); break;
    case 15: cps(S.mass); break;
    default: return -1;
  }
  return S.np;
}
// Rounds every particle state field to single precision in place: the
// sensitivity-floor protocol of the parity tests runs the oracle with this
// applied after each step, to bound how far an FP32 computation of the same
// run may legitimately stray from the FP64 one.
void om_round_state_f32(void *h) {
  Sim *s = (Sim *)h;
  auto rv = [](std::vector<double> &A) { for (double &x : A) x = (double)(float)x; };
  auto rm = [](std::vector<M3> &A) { for (M3 &m : A) for (double &x : m.a) x = (double)(float)x; };
  for (auto &S : s->solids) {
    rv(S.x); rv(S.v); rv(S.epsp); rv(S.epsdot); rv(S.damage); rv(S.damage_init); rv(S.T); rv(S.J); rv(S.vol);
    rm(S.sigma); rm(S.F); rm(S.strain_el); rm(S.vol0PK1);
  }
}
// Grid fields: 0 mass, 1 v, 2 v_update, 3 x, 4 f, 5 mb, 6 T
int om_get_grid(void *h, int gi, int field, double *out) {
  Grid &g = ((Sim *)h)->grids[gi];
  const std::vector<double> *src[] = {&g.mass, &g.v, &g.vu, &g.x, &g.f, &g.mb, &g.T};
  if (field < 0 || field > 6) return -1;
  std::memcpy(out, src[field]->data(), sizeof(double) * src[field]->size());
  return g.nn;
}
// FixKineticEnergy (src/fix_kinetic_energy.cpp:78-118) and ComputeStrainEnergy
// (src/compute_strain_energy.cpp:64-117) over all solids.
void om_energy(void *h, double *out) {
  Sim *s = (Sim *)h;
  double Ek = 0, Es = 0;
  for (auto &S : s->solids)
    for (int i = 0; i < S.np; i++) {
      double v2 = S.v[3 * i] * S.v[3 * i] + S.v[3 * i + 1] * S.v[3 * i + 1] + S.v[3 * i + 2] * S.v[3 * i + 2];
      Ek += 0.5 * S.mass[i] * v2;
      double e = 0;
      for (int k = 0; k < 9; k++) e += S.sigma[i].a[k] * S.strain_el[i].a[k];
      Es += 0.5 * S.vol[i] * e;
    }
  out[0] = Ek; out[1] = Es;
}
// 1-D basis evaluation (for the golden-vector pin): kind 0 value, 1 derivative
double om_basis(int basis, int kind, double r, int ntype, double icellsize) {
  if (basis == LINEAR) return kind ? dbf_linear(r, ntype, icellsize) : bf_linear(r, ntype);
  if (basis == CUBIC) return kind ? dbf_cubic(r, ntype, icellsize) : bf_cubic(r, ntype);
  if (basis == QUADRATIC) return kind ? dbf_quad(r, ntype, icellsize) : bf_quad(r, ntype);
  return kind ? dbf_bern(r, ntype, icellsize) : bf_bern(r, ntype);
}
// Constitutive kernels exposed for unit checks (strength + EOS on one state).
// in: sigma[9], D[9], scalars {dt, epsp, epsdot, damage, T, J, rho, cellsize}
// out: sdev[9], {dep, pH}
void om_constitutive(void *h, int mat, const double *sigma, const double *D, const double *sc, double *out) {
  Sim *s = (Sim *)h;
  const Mat &m = s->mats[mat];
  M3 sg, d;
  std::memcpy(sg.a, sigma, 72); std::memcpy(d.a, D, 72);
  double dep = 0, e = 0;
  double pH = eos_pressure(m, e, sc[5], sc[6], sc[3], d, sc[7], sc[4]);
  M3 sdev = strength_update(m, sc[0], sg, d, dep, sc[1], sc[2], sc[3], sc[4]);
  std::memcpy(out, sdev.a, 72);
  out[9] = dep; out[10] = pH;
}
// polar decomposition + eigenvalue helpers exposed for unit checks
int om_poldec(const double *F, double *R) {
  M3 f, r;
  std::memcpy(f.a, F, 72);
  bool ok = poldec(f, r);
  std::memcpy(R, r.a, 72);
  return ok ? 1 : 0;
}
void om_eig_real(const double *F, double *re) {
  M3 f;
  std::memcpy(f.a, F, 72);
  eig_real_parts(f, re);
}

}  // extern "C"
