// Test infrastructure only: the reference's LMOD (src/sff/lmodC.c) takes
// its low modes from ARPACK's driver dsarpack (src/arpack/dsarpack.f), which
// is Fortran 77 and cannot be compiled here.  This stands in for it with the
// same argument list and reverse-communication protocol (label 0 starts,
// label 1 resumes after an evaluation; hessvec_ -- the reference's own
// finite-difference Hessian product in lmodC.c -- supplies the operator),
// computing the modes with libsffg's LowModes solver
// (nabc_gb300/csrc/lowmodes.cpp, compiled into the same binary), so that the
// reference's search logic can be compared with libsffg's bit for bit.
// Output as dseupd leaves it: n_eig_out converged pairs, eigenvalues
// ascending, eigenvectors one after another.  The ARPACK debug printout is
// not reproduced.
#include <cstring>

#include "lowmodes.h"

extern "C" int hessvec_(int *ndim, double *vec_in, double *vec_out, double *xyz, double *grad, int *return_flag,
                        int *label);

namespace {
sffg::LowModes g_modes;
int g_status = 0;
}  // namespace

extern "C" int dsarpack_(int *n_dim, int *n_eig_in, int *n_eig_out, int *ncv_in, int *itr_in, double *eigval_tol,
                         double *eigvals, double *eigvecs, int *spectrum, int *need_eigvecs, int *ierr,
                         int *debug_arpack, double *v, double *workl, double *workd, double *d, double *resid,
                         double *ax, int *select, double *xyz, double *grad, int *return_flag, int *label) {
  (void)spectrum; (void)need_eigvecs; (void)ierr; (void)debug_arpack; (void)v; (void)workl;
  (void)workd; (void)d; (void)resid; (void)ax; (void)select;
  const int kArpackError = -2;
  if (*label == 0) {
    if (g_modes.init(*n_dim, *n_eig_in, *ncv_in, *eigval_tol, *itr_in)) {
      *label = kArpackError;
      return 0;
    }
  } else {
    // the evaluation for the pending product is done: finish it
    hessvec_(n_dim, const_cast<double *>(g_modes.in()), g_modes.out(), xyz, grad, return_flag, &g_status);
    if (g_status < 0) {
      *label = g_status;
      return 0;
    }
  }
  int r;
  while ((r = g_modes.iterate()) == 1) {
    g_status = 0;
    hessvec_(n_dim, const_cast<double *>(g_modes.in()), g_modes.out(), xyz, grad, return_flag, &g_status);
    if (g_status > 0) {
      *label = 1;
      return 0;
    }
    if (g_status < 0) {
      *label = g_status;
      return 0;
    }
  }
  if (r < 0) {
    *label = kArpackError;
    return 0;
  }
  *n_eig_out = g_modes.nconv();
  std::memcpy(eigvals, g_modes.values(), sizeof(double) * g_modes.nconv());
  std::memcpy(eigvecs, g_modes.vectors(), sizeof(double) * g_modes.nconv() * static_cast<size_t>(*n_dim));
  *label = 0;
  return 0;
}
