// Symmetric eigen-solvers for LMOD (csrc/lmod.cpp).
//
// The reference takes LMOD's low modes from ARPACK (src/arpack/dsarpack.f:
// dsaupd/dseupd in regular mode, which = "SM", tol 1e-4, src/sff/
// lmodC.c:1094-1230), a Fortran 77 library.  This file is this library's own
// replacement, with the same reverse-communication contract: the caller
// supplies products y = A x of a symmetric operator (LMOD's finite-difference
// Hessian) and gets back the nev eigenpairs of smallest magnitude, eigenvalues
// in ascending algebraic order and orthonormal eigenvectors, as dseupd
// returns them.  The method is a thick-restart Lanczos iteration with full
// re-orthogonalisation (Wu and Simon, SIAM J. Matrix Anal. Appl. 22 (2000)
// 602-616) and ARPACK's convergence test (Ritz residual <= tol *
// max(eps^(2/3), |theta|)).  With ncv = n, LMOD's default, one sweep spans the
// whole space and the result is exact to rounding.
//
// sym_eigen is the dense solver underneath (Householder reduction to
// tridiagonal form, then implicit symmetric QR steps with Wilkinson shifts;
// Golub and Van Loan, Matrix Computations, 4th ed., algorithms 8.3.1 and
// 8.3.3); LMOD's all-atom superposition (rmsfit) uses it on 3 x 3 too.
//
// The arithmetic is plain IEEE double (+, -, *, /, sqrt) in a fixed order and
// this file is compiled without floating-point contraction, so every host
// computes the same bits.
#pragma once

#include <vector>

namespace sffg {

// All eigenpairs of the symmetric n x n matrix a (row-major; destroyed):
// eigenvalues in descending order in d[n], eigenvector j in column j of z
// (z[i * n + j]).  Returns 0, or -1 if the QR sweeps did not converge.
int sym_eigen(int n, double *a, double *d, double *z);

// Thick-restart Lanczos for the nev eigenpairs of smallest magnitude.
class LowModes {
 public:
  // n: dimension; nev < ncv <= n Ritz vectors requested / kept in the
  // basis; tol: relative residual bound; max_restarts: restarts allowed.
  // Returns 0, or -1 for inconsistent sizes.
  int init(int n, int nev, int ncv, double tol, int max_restarts);
  // 1: a product is wanted -- read x from in(), store A x in out(), call
  // again; 0: finished (nconv() pairs available); -1: no pair converged or
  // the projected eigenproblem failed.
  int iterate();
  const double *in() const { return x_.data(); }
  double *out() { return y_.data(); }
  int nconv() const { return nconv_; }
  int restarts() const { return restarts_; }
  int products() const { return products_; }
  // eigenvalues ascending, vector k at vectors() + k * n
  const double *values() const { return val_.data(); }
  const double *vectors() const { return vec_.data(); }

 private:
  void orthogonalise(double *w, int ncols, double *h);
  void random_unit(double *v);
  int finish_sweep();

  int n_ = 0, nev_ = 0, ncv_ = 0, max_restarts_ = 0;
  double tol_ = 0.0;
  std::vector<double> V_, H_, x_, y_, r_, h_, val_, vec_;
  int j_ = 0, restarts_ = 0, products_ = 0, nconv_ = 0, state_ = 0;
  unsigned long long rng_ = 0;
};

}  // namespace sffg
