/* A host program in plain C against include/tlq.h: the caller a compiled
 * driver (the Fortran main loop, or a C/C++ code) would be.  It builds the
 * Sod shock tube of the tests (256 x 4 x 4, gamma 1.4, HLL, outflow) in the
 * reference layout U(5, -1:nx+2, -1:ny+2, -1:nz+2), fills the ghosts with
 * tlq_borders, uploads, runs to t = 0.2 (tlq_run_until) and prints t, it and
 * the sums of each conserved variable over the interior as one line. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "tlq.h"

#define CHECK(call)                                                                      \
  do {                                                                                   \
    int rc_ = (call);                                                                    \
    if (rc_ != TLQ_OK) {                                                                 \
      fprintf(stderr, "%s: %s (%s)\n", #call, tlq_status_string(rc_), tlq_last_error(ctx)); \
      return 1;                                                                          \
    }                                                                                    \
  } while (0)

int main(void) {
  tlq_config cfg;
  tlq_config_default(&cfg);
  cfg.nx = 256; cfg.ny = 4; cfg.nz = 4;
  const double dx = 1.0 / cfg.nx;
  cfg.xl = 0.0; cfg.xr = 1.0; cfg.yl = 0.0; cfg.yr = 4 * dx; cfg.zl = 0.0; cfg.zr = 4 * dx;
  cfg.gamma = 1.4; cfg.cfl = 0.4; cfg.eta = 0.5e-2;
  cfg.limiter = TLQ_LIMITER_VANLEER; cfg.solver = TLQ_SOLVER_HLL;
  for (int q = 0; q < 6; ++q) cfg.bc[q] = TLQ_BC_OUTFLOW;
  tlq_ctx* ctx = NULL;
  CHECK(tlq_create(&cfg, &ctx));
  const long nxg = cfg.nx + 4, nyg = cfg.ny + 4, nzg = cfg.nz + 4;
  double* U = (double*)calloc((size_t)(5 * nxg * nyg * nzg), sizeof(double));
  for (long k = 0; k < nzg; ++k)
    for (long j = 0; j < nyg; ++j)
      for (long i = 0; i < nxg; ++i) {
        const double x = (cfg.xl + dx * (double)(i - 1)) - dx / 2.0; /* cell -1 .. nx+2 */
        const int left = x < 0.5;
        double* u = U + 5 * (i + nxg * (j + nyg * k));
        u[0] = left ? 1.0 : 0.125;
        u[4] = (left ? 1.0 : 0.1) / (cfg.gamma - 1.0);
      }
  CHECK(tlq_borders(ctx, U, 1));
  CHECK(tlq_upload(ctx, U));
  double t = 0.0, dt = 0.0;
  int it = 0;
  CHECK(tlq_run_until(ctx, 0.2, 1 << 20, &t, &it, &dt));
  CHECK(tlq_download(ctx, U, NULL));
  double s[5] = {0, 0, 0, 0, 0};
  for (long k = 2; k < nzg - 2; ++k)
    for (long j = 2; j < nyg - 2; ++j)
      for (long i = 2; i < nxg - 2; ++i)
        for (int e = 0; e < 5; ++e) s[e] += U[e + 5 * (i + nxg * (j + nyg * k))];
  printf("t %.17g it %d sums %.17g %.17g %.17g %.17g %.17g\n", t, it, s[0], s[1], s[2], s[3], s[4]);
  free(U);
  CHECK(tlq_destroy(ctx));
  return 0;
}
