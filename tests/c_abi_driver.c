/* Plain C99 client of the C ABI (include/gbilu.h), as the reference's host
 * code or an FFI binding would call it: no C++ and no CUDA headers.
 *
 * usage: c_abi_driver DEVICE OUT
 * DEVICE -1: host-only handle (analysis, ordering, host factorization,
 * schedule, error reporting); DEVICE >= 0 also solves on that GPU. The
 * system is a chain of nb 3x3 block rows (blocks i-1, i, i+1) with a
 * diagonally dominant diagonal; b_k = 1 + k % 7. OUT receives, as text:
 * ncolors, the host status of each call, and for a device the solve's
 * status, half-iterations, relative residual and x.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gbilu.h"

#define NB 50

static int fail(const char *what, int rc, void *h) {
  fprintf(stderr, "%s: %d (%s) %s\n", what, rc, gbilu_status_string(rc),
          h ? gbilu_last_error(h) : "");
  return 1;
}

int main(int argc, char **argv) {
  int device, nnzb = 0, i, k, rc, ncolors = 0, nsteps = 0;
  int rowptr[NB + 1], colind[3 * NB], color[NB], perm[NB], color_ptr[NB + 1];
  double vals[9 * 3 * NB], b[3 * NB], x[3 * NB];
  int steps[13 * 64];
  gbilu_options opt;
  gbilu_stats st;
  void *h = NULL;
  FILE *out;
  if (argc < 3) return 2;
  device = atoi(argv[1]);
  out = fopen(argv[2], "w");
  if (!out) return 2;

  /* the pattern and values */
  rowptr[0] = 0;
  for (i = 0; i < NB; ++i) {
    for (k = i - 1; k <= i + 1; ++k) {
      int e;
      if (k < 0 || k >= NB) continue;
      colind[nnzb] = k;
      for (e = 0; e < 9; ++e) {
        const int r = e / 3, c = e % 3;
        double v = (r == c) ? -1.0 : 0.1 * (double)((r + 2 * c + i) % 3 - 1);
        if (k == i) v = (r == c) ? 4.0 + 0.01 * (double)(i % 5) : 0.2;
        vals[9 * nnzb + e] = v;
      }
      ++nnzb;
    }
    rowptr[i + 1] = nnzb;
  }
  for (i = 0; i < 3 * NB; ++i) b[i] = 1.0 + (double)(i % 7);

  if ((rc = gbilu_default_options(&opt)) != GBILU_OK) return fail("default_options", rc, NULL);
  opt.device = device;
  if ((rc = gbilu_create(&opt, &h)) != GBILU_OK) return fail("create", rc, h);

  /* bad input first: a status and a message, the handle stays usable */
  rc = gbilu_analyze(h, NB, rowptr, NULL);
  fprintf(out, "bad_analyze %d %d\n", rc, (int)(strlen(gbilu_last_error(h)) > 0));

  if ((rc = gbilu_analyze(h, NB, rowptr, colind)) != GBILU_OK) return fail("analyze", rc, h);
  if ((rc = gbilu_get_ordering(h, &ncolors, color, perm, color_ptr)) != GBILU_OK)
    return fail("get_ordering", rc, h);
  fprintf(out, "ncolors %d\n", ncolors);
  for (i = 0; i + 1 < NB; ++i)
    if (color[i] == color[i + 1]) return fail("coloring couples a chain link", -1, h);
  if ((rc = gbilu_schedule(h, 0, 64, &nsteps, steps)) != GBILU_OK) return fail("schedule", rc, h);
  fprintf(out, "steps %d\n", nsteps);
  if ((rc = gbilu_factor(h, vals)) != GBILU_OK) return fail("factor", rc, h);
  if ((rc = gbilu_get_stats(h, &st)) != GBILU_OK) return fail("get_stats", rc, h);
  fprintf(out, "stats %d %d %d\n", st.nb, st.nnzb, st.ncolors);

  if (device >= 0) {
    gbilu_result res;
    memset(x, 0, sizeof x);
    if ((rc = gbilu_solve(h, b, x, 1e-8, 200, &res)) != GBILU_OK) return fail("solve", rc, h);
    fprintf(out, "solve %d %d %.17g\n", res.status, res.half_iters, res.relres);
    for (i = 0; i < 3 * NB; ++i) fprintf(out, "%.17g\n", x[i]);
  } else {
    gbilu_result res;
    rc = gbilu_solve(h, b, x, 1e-8, 200, &res);
    fprintf(out, "host_solve %d\n", rc);   /* a host-only handle cannot solve */
  }
  if ((rc = gbilu_destroy(h)) != GBILU_OK) return fail("destroy", rc, NULL);
  fclose(out);
  return 0;
}
