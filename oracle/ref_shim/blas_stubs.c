/*
 * Test infrastructure only.  The reference's src/sff/newton.c (included into
 * sff.c at sff.c:850) references six Fortran BLAS/LAPACK symbols for the
 * Newton-Raphson minimiser, which is not on the GB energy/gradient path.
 * They are never called by mme/md/conjgrad; these stubs only satisfy the
 * linker and abort loudly if anything does reach them.
 */
#include <stdio.h>
#include <stdlib.h>

static void blas_stub_abort(const char *name)
{
  fprintf(stderr, "oracle/_ref: BLAS/LAPACK routine %s is not available\n", name);
  abort();
}

void daxpy_(void) { blas_stub_abort("daxpy_"); }
void dcopy_(void) { blas_stub_abort("dcopy_"); }
double ddot_(void) { blas_stub_abort("ddot_"); return 0.0; }
void dgemm_(void) { blas_stub_abort("dgemm_"); }
double dnrm2_(void) { blas_stub_abort("dnrm2_"); return 0.0; }
void dposv_(void) { blas_stub_abort("dposv_"); }
