/* A C caller of the drop-in boundary, compiled by tests/test_c_abi.py with a
 * plain C compiler against include/ddcsvd.h and linked to libddcsvd.so.
 *
 * The function-pointer assignments make the compiler check the drop-ins'
 * signatures against the reference's declarations (svd_gpu.h:5,
 * bidiag_par.h:30, :33-34).  At run time it calls svd_gpu on a 3 x 2 matrix
 * (the reference's calling pattern, test-whole-svd.c:75) and the host-only
 * planning calls, and prints what it got for the test to check: with a GPU,
 * the singular values; without one, NaN (the library has no CPU path). */
#include <stdio.h>

#include "ddcsvd.h"

typedef void (*svd_gpu_fn)(int, int, double *, double *, double *, double *);
typedef void (*bidiag_par_fn)(int, int, double *, double *, double *);
typedef void (*form_fn)(int, int, const double *, double *);

int main(void) {
  svd_gpu_fn f_svd = svd_gpu;
  bidiag_par_fn f_bidiag = bidiag_par;
  form_fn f_u = form_u_par, f_v = form_v_par;
  (void)f_bidiag;
  (void)f_u;
  (void)f_v;

  double A[6] = {3.0, 0.0, 0.0, 0.0, 2.0, 0.0}; /* 3 x 2, column-major: diag(3, 2) */
  double sigma[2] = {0.0, 0.0}, U[9], V[4];
  f_svd(3, 2, A, sigma, U, V);
  printf("sigma %.17g %.17g\n", sigma[0], sigma[1]);

  double a[6] = {1.0, 2.0, 3.0, 4.0, 5.0, 6.0}, b[6] = {1.0, 0.0, 1e-30, 1.0, 1.0, 0.0};
  int starts[7], nstarts = 0;
  int rc = ddcsvd_split_plan(6, a, b, 2.220446049250313e-16, starts, &nstarts);
  printf("split %d %d", rc, nstarts);
  for (int i = 0; i < nstarts; i++) printf(" %d", starts[i]);
  printf("\n");

  int meta[8], table[4096];
  rc = ddcsvd_dc_plan(6, nstarts, starts, 8, table, 4096, meta);
  printf("plan %d nodes %d trees %d\n", rc, meta[0], meta[3]);
  printf("status %s\n", ddcsvd_status_string(0));
  return 0;
}
