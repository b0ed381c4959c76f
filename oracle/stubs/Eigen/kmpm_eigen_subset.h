/* A small subset of the Eigen 3 C++ API, written for this project from the
 * mathematics (no Eigen source was used), so that the reference's sources
 * compile and run as the test oracle without an Eigen installation.  It is
 * test infrastructure: the checker's build of the reference
 * (oracle/Makefile) is its only user.
 *
 * Covered: fixed-size dense matrices and vectors of double (Matrix2d/3d/4d,
 * Vector2d/3d/4d) with eager arithmetic, the comma initialiser, transpose,
 * trace, norm, dot, cross, determinant, inverse, asDiagonal, min/maxCoeff,
 * col, data, noalias, setZero/setIdentity, Zero/Identity; JacobiSVD (one-sided
 * Jacobi, Hestenes 1958), EigenSolver of a real 3x3 matrix (characteristic
 * cubic of the shifted matrix with Newton refinement) and
 * SelfAdjointEigenSolver (cyclic Jacobi rotations).
 *
 * Storage is column-major, as Eigen's default.  Everything evaluates
 * eagerly, so aliasing (a = a * b) is always safe.  Round-off differs from
 * Eigen's algorithms; the results the reference's step depends on are unique
 * (the rotation of the polar decomposition of a matrix with positive
 * determinant, the eigenvalues of F), so they agree to round-off. */
#ifndef KMPM_EIGEN_SUBSET_H
#define KMPM_EIGEN_SUBSET_H

// standard headers the full Eigen headers bring in, on which code written
// against Eigen may rely (INT_MAX, CHAR_BIT, ...)
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <vector>
#include <complex>
#include <cstddef>
#include <initializer_list>
#include <ostream>

namespace Eigen {

typedef std::ptrdiff_t Index;

enum DecompositionOptions { ComputeFullU = 0x04, ComputeThinU = 0x08, ComputeFullV = 0x10, ComputeThinV = 0x20 };
enum ComputationInfo { Success = 0, NumericalIssue = 1, NoConvergence = 2, InvalidInput = 3 };

template <typename S, int R, int C> class Matrix;

template <typename M> class CommaInit {
 public:
  CommaInit(M &m, typename M::Scalar v) : m_(m), k_(0) { put(v); }
  CommaInit &operator,(typename M::Scalar v) {
    put(v);
    return *this;
  }

 private:
  void put(typename M::Scalar v) {  // row-major fill order, as Eigen's
    const int r = k_ / M::ColsAtCompileTime, c = k_ % M::ColsAtCompileTime;
    if (r < M::RowsAtCompileTime) m_(r, c) = v;
    k_++;
  }
  M &m_;
  int k_;
};

template <typename S, int R, int C> class Matrix {
 public:
  typedef S Scalar;
  enum { RowsAtCompileTime = R, ColsAtCompileTime = C, SizeAtCompileTime = R * C };

  Matrix() { setZero(); }
  Matrix(S x, S y) {
    static_assert(R * C == 2, "two-coefficient constructor");
    v_[0] = x; v_[1] = y;
  }
  Matrix(S x, S y, S z) {
    static_assert(R * C == 3, "three-coefficient constructor");
    v_[0] = x; v_[1] = y; v_[2] = z;
  }
  Matrix(S x, S y, S z, S w) {
    static_assert(R * C == 4, "four-coefficient constructor");
    v_[0] = x; v_[1] = y; v_[2] = z; v_[3] = w;
  }

  static Matrix Zero() { return Matrix(); }
  static Matrix Identity() {
    Matrix m;
    m.setIdentity();
    return m;
  }
  static Matrix Constant(S c) {
    Matrix m;
    for (int k = 0; k < R * C; k++) m.v_[k] = c;
    return m;
  }
  static Matrix Ones() { return Constant(S(1)); }

  Index rows() const { return R; }
  Index cols() const { return C; }
  Index size() const { return R * C; }

  S &operator()(Index i, Index j) { return v_[j * R + i]; }
  const S &operator()(Index i, Index j) const { return v_[j * R + i]; }
  S &operator()(Index k) { return v_[k]; }
  const S &operator()(Index k) const { return v_[k]; }
  S &operator[](Index k) { return v_[k]; }
  const S &operator[](Index k) const { return v_[k]; }
  S &x() { return v_[0]; }
  S &y() { return v_[1]; }
  S &z() { return v_[2]; }
  S &w() { return v_[3]; }
  const S &x() const { return v_[0]; }
  const S &y() const { return v_[1]; }
  const S &z() const { return v_[2]; }
  const S &w() const { return v_[3]; }
  S *data() { return v_; }
  const S *data() const { return v_; }

  Matrix &setZero() {
    for (int k = 0; k < R * C; k++) v_[k] = S(0);
    return *this;
  }
  Matrix &setIdentity() {
    for (int j = 0; j < C; j++)
      for (int i = 0; i < R; i++) (*this)(i, j) = i == j ? S(1) : S(0);
    return *this;
  }
  Matrix &setConstant(S c) {
    for (int k = 0; k < R * C; k++) v_[k] = c;
    return *this;
  }
  Matrix &noalias() { return *this; }
  CommaInit<Matrix> operator<<(S v) { return CommaInit<Matrix>(*this, v); }

  Matrix<S, C, R> transpose() const {
    Matrix<S, C, R> t;
    for (int j = 0; j < C; j++)
      for (int i = 0; i < R; i++) t(j, i) = (*this)(i, j);
    return t;
  }
  Matrix<S, R, 1> col(Index j) const {
    Matrix<S, R, 1> c;
    for (int i = 0; i < R; i++) c(i) = (*this)(i, j);
    return c;
  }
  Matrix<S, 1, C> row(Index i) const {
    Matrix<S, 1, C> r;
    for (int j = 0; j < C; j++) r(j) = (*this)(i, j);
    return r;
  }
  S trace() const {
    S t = 0;
    for (int i = 0; i < (R < C ? R : C); i++) t += (*this)(i, i);
    return t;
  }
  S squaredNorm() const {
    S s = 0;
    for (int k = 0; k < R * C; k++) s += v_[k] * v_[k];
    return s;
  }
  S norm() const { return std::sqrt(squaredNorm()); }
  S sum() const {
    S s = 0;
    for (int k = 0; k < R * C; k++) s += v_[k];
    return s;
  }
  Matrix normalized() const { return *this / norm(); }
  void normalize() { *this = normalized(); }
  S dot(const Matrix &o) const {
    S s = 0;
    for (int k = 0; k < R * C; k++) s += v_[k] * o.v_[k];
    return s;
  }
  Matrix cross(const Matrix &o) const {
    static_assert(R * C == 3, "cross product of 3-vectors");
    return Matrix(v_[1] * o.v_[2] - v_[2] * o.v_[1], v_[2] * o.v_[0] - v_[0] * o.v_[2],
                  v_[0] * o.v_[1] - v_[1] * o.v_[0]);
  }
  Matrix cwiseAbs() const {
    Matrix m;
    for (int k = 0; k < R * C; k++) m.v_[k] = std::fabs(v_[k]);
    return m;
  }
  template <typename I> S minCoeff(I *at = nullptr) const {
    int b = 0;
    for (int k = 1; k < R * C; k++)
      if (v_[k] < v_[b]) b = k;
    if (at) *at = (I)b;
    return v_[b];
  }
  S minCoeff() const { return minCoeff<int>(nullptr); }
  template <typename I> S maxCoeff(I *at = nullptr) const {
    int b = 0;
    for (int k = 1; k < R * C; k++)
      if (v_[k] > v_[b]) b = k;
    if (at) *at = (I)b;
    return v_[b];
  }
  S maxCoeff() const { return maxCoeff<int>(nullptr); }
  Matrix<S, R * C, R * C> asDiagonal() const {
    static_assert(R == 1 || C == 1, "asDiagonal of a vector");
    Matrix<S, R * C, R * C> d;
    for (int k = 0; k < R * C; k++) d(k, k) = v_[k];
    return d;
  }

  S determinant() const;
  Matrix inverse() const;

  Matrix &operator+=(const Matrix &o) {
    for (int k = 0; k < R * C; k++) v_[k] += o.v_[k];
    return *this;
  }
  Matrix &operator-=(const Matrix &o) {
    for (int k = 0; k < R * C; k++) v_[k] -= o.v_[k];
    return *this;
  }
  Matrix &operator*=(S s) {
    for (int k = 0; k < R * C; k++) v_[k] *= s;
    return *this;
  }
  Matrix &operator/=(S s) {
    for (int k = 0; k < R * C; k++) v_[k] /= s;
    return *this;
  }
  Matrix &operator*=(const Matrix &o);
  Matrix operator-() const {
    Matrix m;
    for (int k = 0; k < R * C; k++) m.v_[k] = -v_[k];
    return m;
  }
  Matrix operator+(const Matrix &o) const {
    Matrix m = *this;
    return m += o;
  }
  Matrix operator-(const Matrix &o) const {
    Matrix m = *this;
    return m -= o;
  }
  Matrix operator*(S s) const {
    Matrix m = *this;
    return m *= s;
  }
  Matrix operator/(S s) const {
    Matrix m = *this;
    return m /= s;
  }
  bool operator==(const Matrix &o) const {
    for (int k = 0; k < R * C; k++)
      if (v_[k] != o.v_[k]) return false;
    return true;
  }
  bool operator!=(const Matrix &o) const { return !(*this == o); }

 private:
  S v_[R * C];
};

template <typename S, int R, int C> Matrix<S, R, C> operator*(S s, const Matrix<S, R, C> &m) { return m * s; }
template <typename S, int R, int C> Matrix<S, R, C> operator*(int s, const Matrix<S, R, C> &m) { return m * S(s); }

template <typename S, int R, int K, int C>
Matrix<S, R, C> operator*(const Matrix<S, R, K> &a, const Matrix<S, K, C> &b) {
  Matrix<S, R, C> m;
  for (int j = 0; j < C; j++)
    for (int i = 0; i < R; i++) {
      S s = 0;
      for (int k = 0; k < K; k++) s += a(i, k) * b(k, j);
      m(i, j) = s;
    }
  return m;
}

template <typename S, int R, int C> Matrix<S, R, C> &Matrix<S, R, C>::operator*=(const Matrix &o) {
  *this = (*this) * o;
  return *this;
}

namespace detail {
template <typename S, int N> S det(const Matrix<S, N, N> &m) {
  // Gaussian elimination with partial pivoting
  Matrix<S, N, N> a = m;
  S d = 1;
  for (int c = 0; c < N; c++) {
    int p = c;
    for (int r = c + 1; r < N; r++)
      if (std::fabs(a(r, c)) > std::fabs(a(p, c))) p = r;
    if (a(p, c) == S(0)) return S(0);
    if (p != c) {
      for (int k = 0; k < N; k++) std::swap(a(p, k), a(c, k));
      d = -d;
    }
    d *= a(c, c);
    for (int r = c + 1; r < N; r++) {
      const S f = a(r, c) / a(c, c);
      for (int k = c; k < N; k++) a(r, k) -= f * a(c, k);
    }
  }
  return d;
}
template <typename S> S det(const Matrix<S, 1, 1> &m) { return m(0, 0); }
template <typename S> S det(const Matrix<S, 2, 2> &m) { return m(0, 0) * m(1, 1) - m(0, 1) * m(1, 0); }
template <typename S> S det(const Matrix<S, 3, 3> &m) {
  return m(0, 0) * (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) - m(0, 1) * (m(1, 0) * m(2, 2) - m(1, 2) * m(2, 0)) +
         m(0, 2) * (m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0));
}
template <typename S, int N> Matrix<S, N, N> inv(const Matrix<S, N, N> &m) {
  // Gauss-Jordan elimination with partial pivoting
  Matrix<S, N, N> a = m, b = Matrix<S, N, N>::Identity();
  for (int c = 0; c < N; c++) {
    int p = c;
    for (int r = c + 1; r < N; r++)
      if (std::fabs(a(r, c)) > std::fabs(a(p, c))) p = r;
    for (int k = 0; k < N; k++) {
      std::swap(a(p, k), a(c, k));
      std::swap(b(p, k), b(c, k));
    }
    const S piv = a(c, c);
    for (int k = 0; k < N; k++) {
      a(c, k) /= piv;
      b(c, k) /= piv;
    }
    for (int r = 0; r < N; r++) {
      if (r == c) continue;
      const S f = a(r, c);
      for (int k = 0; k < N; k++) {
        a(r, k) -= f * a(c, k);
        b(r, k) -= f * b(c, k);
      }
    }
  }
  return b;
}
template <typename S> Matrix<S, 2, 2> inv(const Matrix<S, 2, 2> &m) {
  const S d = det(m);
  Matrix<S, 2, 2> r;
  r(0, 0) = m(1, 1) / d; r(0, 1) = -m(0, 1) / d;
  r(1, 0) = -m(1, 0) / d; r(1, 1) = m(0, 0) / d;
  return r;
}
template <typename S> Matrix<S, 3, 3> inv(const Matrix<S, 3, 3> &m) {
  // adjugate over determinant
  Matrix<S, 3, 3> c;
  c(0, 0) = m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1);
  c(0, 1) = m(0, 2) * m(2, 1) - m(0, 1) * m(2, 2);
  c(0, 2) = m(0, 1) * m(1, 2) - m(0, 2) * m(1, 1);
  c(1, 0) = m(1, 2) * m(2, 0) - m(1, 0) * m(2, 2);
  c(1, 1) = m(0, 0) * m(2, 2) - m(0, 2) * m(2, 0);
  c(1, 2) = m(0, 2) * m(1, 0) - m(0, 0) * m(1, 2);
  c(2, 0) = m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0);
  c(2, 1) = m(0, 1) * m(2, 0) - m(0, 0) * m(2, 1);
  c(2, 2) = m(0, 0) * m(1, 1) - m(0, 1) * m(1, 0);
  const S d = m(0, 0) * c(0, 0) + m(0, 1) * c(1, 0) + m(0, 2) * c(2, 0);
  return c / d;
}
}  // namespace detail

template <typename S, int R, int C> S Matrix<S, R, C>::determinant() const {
  static_assert(R == C, "determinant of a square matrix");
  return detail::det(*this);
}
template <typename S, int R, int C> Matrix<S, R, C> Matrix<S, R, C>::inverse() const {
  static_assert(R == C, "inverse of a square matrix");
  return detail::inv(*this);
}

template <typename S, int R, int C> std::ostream &operator<<(std::ostream &os, const Matrix<S, R, C> &m) {
  for (int i = 0; i < R; i++) {
    for (int j = 0; j < C; j++) os << (j ? " " : "") << m(i, j);
    if (i + 1 < R) os << "\n";
  }
  return os;
}

typedef Matrix<double, 2, 2> Matrix2d;
typedef Matrix<double, 3, 3> Matrix3d;
typedef Matrix<double, 4, 4> Matrix4d;
typedef Matrix<double, 2, 1> Vector2d;
typedef Matrix<double, 3, 1> Vector3d;
typedef Matrix<double, 4, 1> Vector4d;
typedef Matrix<int, 3, 1> Vector3i;

/* Singular value decomposition M = U diag(s) V^T of a square matrix by the
 * one-sided Jacobi method (M. R. Hestenes, J. SIAM 6, 1958): plane rotations
 * applied to the columns of M (and accumulated in V) until every pair of
 * columns is orthogonal; the column norms are then the singular values and
 * the normalised columns U.  Singular values are non-negative and sorted in
 * decreasing order. */
template <typename M> class JacobiSVD {
 public:
  typedef typename M::Scalar S;
  enum { N = M::RowsAtCompileTime };
  typedef Matrix<S, N, 1> SingularValuesType;

  JacobiSVD() {}
  explicit JacobiSVD(const M &m, unsigned int = 0) { compute(m); }

  JacobiSVD &compute(const M &m, unsigned int = 0) {
    static_assert(M::RowsAtCompileTime == M::ColsAtCompileTime, "square matrices only");
    M a = m, v = M::Identity();
    for (int sweep = 0; sweep < 80; sweep++) {
      bool rotated = false;
      for (int p = 0; p < N - 1; p++)
        for (int q = p + 1; q < N; q++) {
          S alpha = 0, beta = 0, gamma = 0;
          for (int i = 0; i < N; i++) {
            alpha += a(i, p) * a(i, p);
            beta += a(i, q) * a(i, q);
            gamma += a(i, p) * a(i, q);
          }
          if (gamma == S(0) || std::fabs(gamma) <= S(1e-17) * std::sqrt(alpha * beta)) continue;
          rotated = true;
          const S zeta = (beta - alpha) / (S(2) * gamma);
          const S t = (zeta >= 0 ? S(1) : S(-1)) / (std::fabs(zeta) + std::sqrt(S(1) + zeta * zeta));
          const S c = S(1) / std::sqrt(S(1) + t * t), s = c * t;
          for (int i = 0; i < N; i++) {
            const S ap = a(i, p), aq = a(i, q);
            a(i, p) = c * ap - s * aq;
            a(i, q) = s * ap + c * aq;
            const S vp = v(i, p), vq = v(i, q);
            v(i, p) = c * vp - s * vq;
            v(i, q) = s * vp + c * vq;
          }
        }
      if (!rotated) break;
    }
    // singular values and left vectors, sorted by decreasing value
    S sv[N];
    int order[N];
    for (int j = 0; j < N; j++) {
      sv[j] = a.col(j).norm();
      order[j] = j;
    }
    std::stable_sort(order, order + N, [&](int x, int y) { return sv[x] > sv[y]; });
    const S scale = sv[order[0]];
    for (int k = 0; k < N; k++) {
      const int j = order[k];
      s_(k) = sv[j];
      for (int i = 0; i < N; i++) v_(i, k) = v(i, j);
      const bool zero = !(sv[j] > scale * S(1e-300)) || sv[j] == S(0);
      for (int i = 0; i < N; i++) u_(i, k) = zero ? S(0) : a(i, j) / sv[j];
    }
    // complete U where a singular value vanished: Gram-Schmidt on unit vectors
    for (int k = 0; k < N; k++) {
      if (u_.col(k).norm() > S(0.5)) continue;
      for (int e = 0; e < N; e++) {
        Matrix<S, N, 1> c;
        c(e) = S(1);
        for (int j = 0; j < N; j++)
          if (j != k && u_.col(j).norm() > S(0.5)) {
            const S d = u_.col(j).dot(c);
            for (int i = 0; i < N; i++) c(i) -= d * u_(i, j);
          }
        const S nc = c.norm();
        if (nc > S(0.1)) {
          for (int i = 0; i < N; i++) u_(i, k) = c(i) / nc;
          break;
        }
      }
    }
    return *this;
  }
  const SingularValuesType &singularValues() const { return s_; }
  const M &matrixU() const { return u_; }
  const M &matrixV() const { return v_; }

 private:
  M u_, v_;
  SingularValuesType s_;
};

/* Eigenvalues of a real 3x3 (or 2x2) matrix.  With m = I c + H (c the mean of
 * the diagonal), the eigenvalues are c + mu, mu the roots of the
 * characteristic polynomial of H, which are found by the trigonometric or
 * Cardano form and refined by Newton steps on that polynomial.  Only the
 * eigenvalues are computed. */
template <typename M> class EigenSolver {
 public:
  typedef typename M::Scalar S;
  enum { N = M::RowsAtCompileTime };
  typedef Matrix<std::complex<S>, N, 1> EigenvalueType;

  EigenSolver() {}
  explicit EigenSolver(const M &m, bool = true) { compute(m); }

  EigenSolver &compute(const M &m, bool = true) {
    static_assert(N == 2 || N == 3, "EigenSolver subset: 2x2 and 3x3");
    info_ = Success;
    for (int k = 0; k < N * N; k++)
      if (!std::isfinite(m(k))) {
        info_ = NoConvergence;
        return *this;
      }
    const S c = m.trace() / S(N);
    M h = m;
    for (int i = 0; i < N; i++) h(i, i) -= c;
    if (N == 2) {
      // mu^2 + det(h) = 0 (trace 0)
      const S d = h(0, 0) * h(1, 1) - h(0, 1) * h(1, 0);
      if (d <= 0) {
        const S r = std::sqrt(-d);
        ev_(0) = std::complex<S>(c + r, 0);
        ev_(1) = std::complex<S>(c - r, 0);
      } else {
        const S r = std::sqrt(d);
        ev_(0) = std::complex<S>(c, r);
        ev_(1) = std::complex<S>(c, -r);
      }
      return *this;
    }
    // mu^3 + p mu + q = 0 (h has trace 0): p = sum of principal minors, q = -det h
    const S p = h(0, 0) * h(1, 1) - h(0, 1) * h(1, 0) + h(0, 0) * h(2, 2) - h(0, 2) * h(2, 0) +
                h(1, 1) * h(2, 2) - h(1, 2) * h(2, 1);
    const S q = -detail::det(h);
    auto f = [&](S x) { return (x * x + p) * x + q; };
    auto df = [&](S x) { return S(3) * x * x + p; };
    auto polish = [&](S x) {
      for (int it = 0; it < 4; it++) {
        const S d = df(x);
        if (d == S(0)) break;
        const S nx = x - f(x) / d;
        if (!(std::fabs(f(nx)) < std::fabs(f(x)))) break;
        x = nx;
      }
      return x;
    };
    const S disc = q * q / S(4) + p * p * p / S(27);
    if (disc <= 0) {
      // three real roots: mu = 2 sqrt(-p/3) cos(phi/3 - 2 pi k / 3)
      const S r = std::sqrt(std::max(-p / S(3), S(0)));
      S arg = r > 0 ? (-q / S(2)) / (r * r * r) : S(0);
      arg = std::min(S(1), std::max(S(-1), arg));
      const S phi = std::acos(arg);
      const S pi = std::acos(S(-1));
      for (int k = 0; k < 3; k++) ev_(k) = std::complex<S>(c + polish(S(2) * r * std::cos((phi - S(2) * pi * k) / S(3))), 0);
    } else {
      // one real root (Cardano) and a complex pair from the deflated quadratic
      const S sd = std::sqrt(disc);
      const S mu = polish(std::cbrt(-q / S(2) + sd) + std::cbrt(-q / S(2) - sd));
      // mu^3 + p mu + q = (mu - mu0)(mu^2 + mu0 mu + mu0^2 + p)
      const S re = -mu / S(2), im2 = mu * mu + p - re * re;
      const S im = std::sqrt(std::max(im2, S(0)));
      ev_(0) = std::complex<S>(c + mu, 0);
      ev_(1) = std::complex<S>(c + re, im);
      ev_(2) = std::complex<S>(c + re, -im);
    }
    return *this;
  }
  const EigenvalueType &eigenvalues() const { return ev_; }
  ComputationInfo info() const { return info_; }

 private:
  EigenvalueType ev_;
  ComputationInfo info_ = Success;
};

/* Eigen-decomposition of a symmetric matrix by cyclic Jacobi rotations
 * (C. G. J. Jacobi, 1846; Golub and Van Loan, Matrix Computations, sec. 8.5):
 * eigenvalues in increasing order, eigenvectors as the matching columns. */
template <typename M> class SelfAdjointEigenSolver {
 public:
  typedef typename M::Scalar S;
  enum { N = M::RowsAtCompileTime };
  typedef Matrix<S, N, 1> RealVectorType;

  SelfAdjointEigenSolver() {}
  explicit SelfAdjointEigenSolver(const M &m, int = 0) { compute(m); }

  SelfAdjointEigenSolver &compute(const M &m, int = 0) {
    M a = m, v = M::Identity();
    for (int sweep = 0; sweep < 60; sweep++) {
      S off = 0;
      for (int p = 0; p < N; p++)
        for (int q = p + 1; q < N; q++) off += a(p, q) * a(p, q);
      if (off == S(0)) break;
      for (int p = 0; p < N - 1; p++)
        for (int q = p + 1; q < N; q++) {
          if (a(p, q) == S(0)) continue;
          const S theta = (a(q, q) - a(p, p)) / (S(2) * a(p, q));
          const S t = (theta >= 0 ? S(1) : S(-1)) / (std::fabs(theta) + std::sqrt(theta * theta + S(1)));
          const S c = S(1) / std::sqrt(t * t + S(1)), s = t * c;
          for (int k = 0; k < N; k++) {  // a <- J^T a J
            const S akp = a(k, p), akq = a(k, q);
            a(k, p) = c * akp - s * akq;
            a(k, q) = s * akp + c * akq;
          }
          for (int k = 0; k < N; k++) {
            const S apk = a(p, k), aqk = a(q, k);
            a(p, k) = c * apk - s * aqk;
            a(q, k) = s * apk + c * aqk;
          }
          for (int k = 0; k < N; k++) {
            const S vkp = v(k, p), vkq = v(k, q);
            v(k, p) = c * vkp - s * vkq;
            v(k, q) = s * vkp + c * vkq;
          }
        }
    }
    int order[N];
    for (int k = 0; k < N; k++) order[k] = k;
    std::stable_sort(order, order + N, [&](int x, int y) { return a(x, x) < a(y, y); });
    for (int k = 0; k < N; k++) {
      ev_(k) = a(order[k], order[k]);
      for (int i = 0; i < N; i++) vec_(i, k) = v(i, order[k]);
    }
    return *this;
  }
  const RealVectorType &eigenvalues() const { return ev_; }
  const M &eigenvectors() const { return vec_; }
  ComputationInfo info() const { return Success; }

 private:
  RealVectorType ev_;
  M vec_;
};

}  // namespace Eigen

#endif
