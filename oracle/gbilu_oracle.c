/*
 * CPU oracle for the ILU0-BiCGSTAB path -- TEST INFRASTRUCTURE ONLY.
 * See gbilu_oracle.h for scope and parity status. Reference paths below are
 * relative to linearalgebra/ilu0bicgstab/xilinx/ in the OPM/FPGA tree.
 */
#include "gbilu_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* "already solved" bound on ||r0|| in relative mode:
 * alveo_u280/rtl/pkg/constants.vhd:59 (ALREADY_SOLVED_THRESHOLD = 1e-30),
 * selected in src/rtl/bicgstab_solver_2r-3r3w/solver.vhd:636-641. */
#define ORC_ALREADY_SOLVED 1e-30

/* ------------------------------------------------------------------ */
/* coloring and ordering (opm-simulators side, defined here)            */
/* ------------------------------------------------------------------ */

int orc_color_greedy(int nb, const int *rowptr, const int *colind, int *color) {
  int ncolors = 0;
  /* mark[c] == i+1 when color c is taken by a neighbour of row i */
  int *mark = (int *)calloc((size_t)nb + 1, sizeof(int));
  for (int i = 0; i < nb; ++i) color[i] = -1;
  for (int i = 0; i < nb; ++i) {
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      int j = colind[k];
      if (j != i && color[j] >= 0) mark[color[j]] = i + 1;
    }
    int c = 0;
    while (mark[c] == i + 1) ++c;
    color[i] = c;
    if (c + 1 > ncolors) ncolors = c + 1;
  }
  free(mark);
  return ncolors;
}

/* 1 when the sorted column lists of rows a and v share a row other than
 * the excluded ones (x1, x2, a and v themselves) */
static int shares_other(const int *rowptr, const int *colind, int a, int v, int x1, int x2) {
  int p = rowptr[a], q = rowptr[v];
  while (p < rowptr[a + 1] && q < rowptr[v + 1]) {
    int ca = colind[p], cv = colind[q];
    if (ca < cv) { ++p; continue; }
    if (cv < ca) { ++q; continue; }
    if (ca != x1 && ca != x2 && ca != a && ca != v) return 1;
    ++p; ++q;
  }
  return 0;
}

int orc_color_parity(int nb, const int *rowptr, const int *colind, int *color) {
  size_t nnzb = (size_t)rowptr[nb];
  /* (1) face[k]: block k = (u, v) lies on a 4-cycle u - a - b - v - u with
   * a, b outside {u, v}: some a in N(u) shares a neighbour b != u with v */
  char *face = (char *)calloc(nnzb + 1, 1);
  for (int u = 0; u < nb; ++u)
    for (int k = rowptr[u]; k < rowptr[u + 1]; ++k) {
      int v = colind[k];
      if (v == u) continue;
      for (int ka = rowptr[u]; ka < rowptr[u + 1] && !face[k]; ++ka) {
        int a = colind[ka];
        if (a == u || a == v) continue;
        if (shares_other(rowptr, colind, a, v, u, v)) face[k] = 1;
      }
    }
  /* (2) distance parity over face blocks from the lowest-numbered row of
   * each connected part, level by level */
  int *dist = (int *)malloc(sizeof(int) * (size_t)(nb > 0 ? nb : 1));
  int *cur = (int *)malloc(sizeof(int) * (size_t)(nb > 0 ? nb : 1));
  int *nxt = (int *)malloc(sizeof(int) * (size_t)(nb > 0 ? nb : 1));
  for (int i = 0; i < nb; ++i) dist[i] = -1;
  for (int root = 0; root < nb; ++root) {
    if (dist[root] >= 0) continue;
    int ncur = 1, level = 0;
    cur[0] = root;
    dist[root] = 0;
    while (ncur > 0) {
      int nn = 0;
      ++level;
      for (int t = 0; t < ncur; ++t) {
        int u = cur[t];
        for (int k = rowptr[u]; k < rowptr[u + 1]; ++k)
          if (face[k] && dist[colind[k]] < 0) {
            dist[colind[k]] = level;
            nxt[nn++] = colind[k];
          }
      }
      int *tmp = cur; cur = nxt; nxt = tmp;
      ncur = nn;
    }
  }
  /* (3) blocks (u, v), u < v, of equal parity, in row-major order: unless
   * an end is already moved, move v -- or u when v has a moved neighbour
   * and u has none */
  char *moved = (char *)calloc((size_t)nb + 1, 1);
  for (int u = 0; u < nb; ++u)
    for (int k = rowptr[u]; k < rowptr[u + 1]; ++k) {
      int v = colind[k];
      if (v <= u || (dist[u] & 1) != (dist[v] & 1) || moved[u] || moved[v]) continue;
      int vm = 0, um = 0;
      for (int q = rowptr[v]; q < rowptr[v + 1]; ++q) vm |= moved[colind[q]];
      for (int q = rowptr[u]; q < rowptr[u + 1]; ++q) um |= moved[colind[q]];
      if (vm && !um) moved[u] = 1; else moved[v] = 1;
    }
  /* (4) first-fit greedy over rows ordered (parity 0, parity 1, moved),
   * natural order inside each class */
  int *mark = (int *)calloc((size_t)nb + 2, sizeof(int));
  int ncolors = 0, step = 0;
  for (int i = 0; i < nb; ++i) color[i] = -1;
  for (int cls = 0; cls < 3; ++cls)
    for (int i = 0; i < nb; ++i) {
      int ci = moved[i] ? 2 : (dist[i] & 1);
      if (ci != cls) continue;
      ++step;
      for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
        int j = colind[k];
        if (j != i && color[j] >= 0) mark[color[j]] = step;
      }
      int c = 0;
      while (mark[c] == step) ++c;
      color[i] = c;
      if (c + 1 > ncolors) ncolors = c + 1;
    }
  free(face); free(dist); free(cur); free(nxt); free(moved); free(mark);
  return ncolors;
}

void orc_color_order(int nb, const int *rowptr, const int *colind,
                     const int *color, int ncolors, int *perm, int *color_ptr,
                     int *split) {
  /* higher[i] = 1: row i shares a block with a row of a higher color */
  char *higher = (char *)calloc((size_t)nb + 1, 1);
  for (int i = 0; i < nb; ++i)
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      int j = colind[k];
      if (color[j] > color[i]) higher[i] = 1;
      if (color[i] > color[j]) higher[j] = 1;
    }
  for (int c = 0; c <= ncolors; ++c) color_ptr[c] = 0;
  for (int c = 0; c < ncolors; ++c) split[c] = 0;
  for (int i = 0; i < nb; ++i) {
    color_ptr[color[i] + 1]++;
    if (higher[i]) split[color[i]]++;
  }
  for (int c = 0; c < ncolors; ++c) color_ptr[c + 1] += color_ptr[c];
  int *first = (int *)malloc(sizeof(int) * (size_t)(ncolors > 0 ? ncolors : 1));
  int *second = (int *)malloc(sizeof(int) * (size_t)(ncolors > 0 ? ncolors : 1));
  for (int c = 0; c < ncolors; ++c) {
    first[c] = color_ptr[c];
    second[c] = color_ptr[c] + split[c];
  }
  for (int i = 0; i < nb; ++i) perm[higher[i] ? first[color[i]]++ : second[color[i]]++] = i;
  free(first);
  free(second);
  free(higher);
}

void orc_permute_bsr(int nb, const int *rowptr, const int *colind,
                     const double *vals, const int *perm, int *prowptr,
                     int *pcolind, double *pvals, int *src) {
  int *iperm = (int *)malloc(sizeof(int) * (size_t)nb);
  for (int i = 0; i < nb; ++i) iperm[perm[i]] = i;
  prowptr[0] = 0;
  for (int i = 0; i < nb; ++i) {
    int o = perm[i];
    prowptr[i + 1] = prowptr[i] + (rowptr[o + 1] - rowptr[o]);
  }
  for (int i = 0; i < nb; ++i) {
    int o = perm[i], base = prowptr[i], len = rowptr[o + 1] - rowptr[o];
    /* insertion sort of (new column, source block) */
    for (int t = 0; t < len; ++t) {
      int k = rowptr[o] + t, c = iperm[colind[k]], p = base + t;
      while (p > base && pcolind[p - 1] > c) {
        pcolind[p] = pcolind[p - 1];
        src[p] = src[p - 1];
        --p;
      }
      pcolind[p] = c;
      src[p] = k;
    }
    if (vals && pvals)
      for (int t = 0; t < len; ++t)
        memcpy(pvals + (size_t)(base + t) * 9, vals + (size_t)src[base + t] * 9,
               9 * sizeof(double));
  }
  free(iperm);
}

/* ------------------------------------------------------------------ */
/* 3x3 block helpers                                                     */
/* ------------------------------------------------------------------ */

int orc_inv3(const double *a, double *o) {
  double c00 = a[4] * a[8] - a[5] * a[7];
  double c01 = a[5] * a[6] - a[3] * a[8];
  double c02 = a[3] * a[7] - a[4] * a[6];
  double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  if (det == 0.0 || !isfinite(det)) return 1;
  double id = 1.0 / det;
  o[0] = c00 * id;
  o[1] = (a[2] * a[7] - a[1] * a[8]) * id;
  o[2] = (a[1] * a[5] - a[2] * a[4]) * id;
  o[3] = c01 * id;
  o[4] = (a[0] * a[8] - a[2] * a[6]) * id;
  o[5] = (a[2] * a[3] - a[0] * a[5]) * id;
  o[6] = c02 * id;
  o[7] = (a[1] * a[6] - a[0] * a[7]) * id;
  o[8] = (a[0] * a[4] - a[1] * a[3]) * id;
  return 0;
}

static void mm3(const double *a, const double *b, double *o) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      o[r * 3 + c] = a[r * 3 + 0] * b[0 * 3 + c] + a[r * 3 + 1] * b[1 * 3 + c] +
                     a[r * 3 + 2] * b[2 * 3 + c];
}

/* ------------------------------------------------------------------ */
/* block ILU(0)                                                          */
/* ------------------------------------------------------------------ */

int orc_bilu0(int nb, const int *rowptr, const int *colind, double *vals,
              double *dinv) {
  int *diag = (int *)malloc(sizeof(int) * (size_t)nb);
  int *pos = (int *)malloc(sizeof(int) * (size_t)nb);
  for (int i = 0; i < nb; ++i) pos[i] = -1;
  int ret = 0;
  for (int i = 0; i < nb; ++i) {
    diag[i] = -1;
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (colind[k] == i) diag[i] = k;
    if (diag[i] < 0) { ret = -(i + 1); goto done; }
  }
  for (int i = 0; i < nb; ++i) {
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) pos[colind[k]] = k;
    for (int kk = rowptr[i]; kk < rowptr[i + 1]; ++kk) {
      int k = colind[kk];
      if (k >= i) break;
      double l[9];
      mm3(vals + (size_t)kk * 9, dinv + (size_t)k * 9, l);   /* L_ik = A_ik U_kk^-1 */
      memcpy(vals + (size_t)kk * 9, l, sizeof l);
      for (int jj = diag[k] + 1; jj < rowptr[k + 1]; ++jj) {  /* j > k in row k */
        int p = pos[colind[jj]];
        if (p < 0) continue;
        double t[9];
        mm3(l, vals + (size_t)jj * 9, t);
        for (int e = 0; e < 9; ++e) vals[(size_t)p * 9 + e] -= t[e];
      }
    }
    if (orc_inv3(vals + (size_t)diag[i] * 9, dinv + (size_t)i * 9)) {
      ret = -(i + 1);
      goto done;
    }
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) pos[colind[k]] = -1;
  }
done:
  free(diag);
  free(pos);
  return ret;
}

/* ------------------------------------------------------------------ */
/* kernels of the PROGRAM: SpMV, L/U sweeps, vector ops                 */
/* ------------------------------------------------------------------ */

void orc_spmv(int nb, const int *rowptr, const int *colind, const double *vals,
              const double *x, double *y) {
  for (int i = 0; i < nb; ++i) {
    double a0 = 0, a1 = 0, a2 = 0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const double *b = vals + (size_t)k * 9, *xj = x + 3 * (size_t)colind[k];
      a0 += b[0] * xj[0] + b[1] * xj[1] + b[2] * xj[2];
      a1 += b[3] * xj[0] + b[4] * xj[1] + b[5] * xj[2];
      a2 += b[6] * xj[0] + b[7] * xj[1] + b[8] * xj[2];
    }
    y[3 * i] = a0; y[3 * i + 1] = a1; y[3 * i + 2] = a2;
  }
}

void orc_spmv_t(int nb, const int *rowptr, const int *colind,
                const double *vals, const double *x, double *y) {
  memset(y, 0, sizeof(double) * 3 * (size_t)nb);
  for (int i = 0; i < nb; ++i)
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const double *b = vals + (size_t)k * 9, *xi = x + 3 * (size_t)i;
      double *yj = y + 3 * (size_t)colind[k];
      for (int c = 0; c < 3; ++c)
        yj[c] += b[c] * xi[0] + b[3 + c] * xi[1] + b[6 + c] * xi[2];
    }
}

/* L sweep (src/rtl/bicgstab_solver_2r-3r3w/ilu0.vhd:406-417, colors in
 * forward order, sparstition.vhd:751-756): y_i = p_i - sum_{j<i} L_ij y_j.
 * U sweep (ilu0.vhd:293-323,380-411, colors and rows in reverse,
 * sparstition.vhd:860-872): z_i = Dinv_i (y_i - sum_{j>i} U_ij z_j).
 * Rows of one color are never coupled, so the row-sequential loops below
 * give the same values as the per-color order of the reference. */
void orc_ilu_apply(int nb, const int *rowptr, const int *colind,
                   const double *lu, const double *dinv, const double *p,
                   double *z) {
  if (z != p) memcpy(z, p, sizeof(double) * 3 * (size_t)nb);
  for (int i = 0; i < nb; ++i) {
    double a[3] = {z[3 * i], z[3 * i + 1], z[3 * i + 2]};
    for (int k = rowptr[i]; k < rowptr[i + 1] && colind[k] < i; ++k) {
      const double *b = lu + (size_t)k * 9, *yj = z + 3 * (size_t)colind[k];
      for (int r = 0; r < 3; ++r)
        a[r] -= b[r * 3] * yj[0] + b[r * 3 + 1] * yj[1] + b[r * 3 + 2] * yj[2];
    }
    z[3 * i] = a[0]; z[3 * i + 1] = a[1]; z[3 * i + 2] = a[2];
  }
  for (int i = nb - 1; i >= 0; --i) {
    double a[3] = {z[3 * i], z[3 * i + 1], z[3 * i + 2]};
    for (int k = rowptr[i + 1] - 1; k >= rowptr[i] && colind[k] > i; --k) {
      const double *b = lu + (size_t)k * 9, *zj = z + 3 * (size_t)colind[k];
      for (int r = 0; r < 3; ++r)
        a[r] -= b[r * 3] * zj[0] + b[r * 3 + 1] * zj[1] + b[r * 3 + 2] * zj[2];
    }
    const double *d = dinv + (size_t)i * 9;
    for (int r = 0; r < 3; ++r)
      z[3 * i + r] = d[r * 3] * a[0] + d[r * 3 + 1] * a[1] + d[r * 3 + 2] * a[2];
  }
}

/* (LU)^-T = L^-T U^-T. U^T is block lower triangular with diagonal
 * blocks U_ii^T: w_i = Dinv_i^T (q_i - sum_{j<i} U_ji^T w_j), forward.
 * L^T is unit upper triangular: z_i = w_i - sum_{j>i} L_ji^T z_j, backward.
 * The transposed contributions are scattered from the rows of L and U, so
 * the loops visit rows j and push into later/earlier rows. */
void orc_ilu_apply_t(int nb, const int *rowptr, const int *colind,
                     const double *lu, const double *dinv, const double *p,
                     double *z) {
  double *acc = (double *)malloc(sizeof(double) * 3 * (size_t)nb);
  memcpy(acc, p, sizeof(double) * 3 * (size_t)nb);
  for (int i = 0; i < nb; ++i) {
    const double *d = dinv + (size_t)i * 9, *a = acc + 3 * (size_t)i;
    double w[3];
    for (int c = 0; c < 3; ++c) w[c] = d[c] * a[0] + d[3 + c] * a[1] + d[6 + c] * a[2];
    z[3 * i] = w[0]; z[3 * i + 1] = w[1]; z[3 * i + 2] = w[2];
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      int j = colind[k];
      if (j <= i) continue;          /* U_ij, j > i contributes to row j of U^T */
      const double *b = lu + (size_t)k * 9;
      for (int c = 0; c < 3; ++c)
        acc[3 * (size_t)j + c] -= b[c] * w[0] + b[3 + c] * w[1] + b[6 + c] * w[2];
    }
  }
  memcpy(acc, z, sizeof(double) * 3 * (size_t)nb);
  for (int i = nb - 1; i >= 0; --i) {
    double w[3] = {acc[3 * i], acc[3 * i + 1], acc[3 * i + 2]};
    z[3 * i] = w[0]; z[3 * i + 1] = w[1]; z[3 * i + 2] = w[2];
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      int j = colind[k];
      if (j >= i) break;             /* L_ij, j < i contributes to row j of L^T */
      const double *b = lu + (size_t)k * 9;
      for (int c = 0; c < 3; ++c)
        acc[3 * (size_t)j + c] -= b[c] * w[0] + b[3 + c] * w[1] + b[6 + c] * w[2];
    }
  }
  free(acc);
}

static double dot(size_t n, const double *a, const double *b) {
  double s = 0;
  for (size_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* record the m-th norm after the initial one in the reference's ring:
 * solver.vhd:913-918 (index 0 once, then 1,2,3,1,2,3...) */
static void push_norm(orc_result *res, double nrm, int half) {
  res->norm = nrm;
  int idx = (half % 3) + 1;
  res->norms[idx] = nrm;
  res->last_norm_idx = idx;
}

/* ------------------------------------------------------------------ */
/* BiCGSTAB in PROGRAM order                                             */
/* ------------------------------------------------------------------ */

/*
 * src/rtl/bicgstab_solver_2r-3r3w/pkg/solver_pkg.vhd:120-141 (PROGRAM) and
 * solver.vhd:552-558 (criteria), 785-936 (scalar units, stop rule):
 *   step 0/1   v = A x0; rt = r = b - v; rho = ||r||^2; stop if ||r|| <= 1e-30
 *              (relative) or <= tol (absolute); bound = tol*||r|| (relative)
 *   steps 2-8  p^ = M^-1 p (p = rt in the first iteration); v = A p^;
 *              alpha = rho/(v,rt); x += alpha p^; s = r - alpha v; stop if
 *              ||s|| <= bound; also stop after this half when the full
 *              iteration count equals maxit (is_final_iter)
 *   steps 2-12 s^ = M^-1 s; t = A s^; omega = (t,s)/(t,t); x += omega s^;
 *              r = s - omega t; stop if ||r|| <= bound
 *   13-17      rho' = (r,rt); beta = (rho'/rho)(alpha/omega); rho = rho';
 *              p = r + beta (p - omega v)
 * The half-iteration counter starts at -1, becomes 0 after step 1, and
 * increments after every half that does not end the solve.
 */
int orc_bicgstab(int nb, const int *rowptr, const int *colind,
                 const double *avals, const double *lu, const double *dinv,
                 const double *b, double *x, double tol, int absolute,
                 int maxit, int transpose, orc_result *res, double *hist,
                 int hist_cap) {
  size_t n = 3 * (size_t)nb;
  double *r = (double *)malloc(8 * n), *rt = (double *)malloc(8 * n);
  double *p = (double *)malloc(8 * n), *v = (double *)malloc(8 * n);
  double *ph = (double *)malloc(8 * n), *s = (double *)malloc(8 * n);
  double *t = (double *)malloc(8 * n);
  memset(res, 0, sizeof *res);
  res->nhist = 0;
#define SPMV(xx, yy) (transpose ? orc_spmv_t(nb, rowptr, colind, avals, xx, yy) \
                                : orc_spmv(nb, rowptr, colind, avals, xx, yy))
#define PREC(in, out) (transpose ? orc_ilu_apply_t(nb, rowptr, colind, lu, dinv, in, out) \
                                 : orc_ilu_apply(nb, rowptr, colind, lu, dinv, in, out))
#define HIST(vv) do { if (hist && res->nhist < hist_cap) hist[res->nhist] = (vv); res->nhist++; } while (0)
  SPMV(x, v);
  for (size_t i = 0; i < n; ++i) { r[i] = b[i] - v[i]; rt[i] = r[i]; p[i] = r[i]; }
  double rho = dot(n, r, r), norm0 = sqrt(rho);
  res->norm0 = norm0; res->norm = norm0; res->norms[0] = norm0; res->last_norm_idx = 0;
  HIST(norm0);
  double bound = absolute ? tol : ORC_ALREADY_SOLVED;
  int status = ORC_MAXIT, half = 0;
  if (!isfinite(norm0)) { status = ORC_NONFINITE; half = -1; goto out; }
  if (!(norm0 > bound)) { status = ORC_ALREADY_CONVERGED; half = -1; goto out; }
  if (!absolute) bound = tol * norm0;
  for (int k = 0;; ++k) {
    half = 2 * k;
    PREC(p, ph);
    SPMV(ph, v);
    double vr = dot(n, v, rt);
    double alpha = rho / vr;
    if (vr == 0.0 || !isfinite(alpha)) { status = ORC_BREAKDOWN; break; }
    for (size_t i = 0; i < n; ++i) { x[i] += alpha * ph[i]; s[i] = r[i] - alpha * v[i]; }
    double ns = sqrt(dot(n, s, s));
    push_norm(res, ns, half); HIST(ns);
    if (!isfinite(ns)) { status = ORC_NONFINITE; break; }
    if (!(ns > bound)) { status = ORC_OK; break; }
    if (k == maxit) { status = ORC_MAXIT; break; }
    half = 2 * k + 1;
    PREC(s, ph);
    SPMV(ph, t);
    double ts = dot(n, t, s), tt = dot(n, t, t);
    double omega = ts / tt;
    if (tt == 0.0 || !isfinite(omega)) { status = ORC_BREAKDOWN; break; }
    for (size_t i = 0; i < n; ++i) { x[i] += omega * ph[i]; r[i] = s[i] - omega * t[i]; }
    double nr = sqrt(dot(n, r, r));
    push_norm(res, nr, half); HIST(nr);
    if (!isfinite(nr)) { status = ORC_NONFINITE; break; }
    if (!(nr > bound)) { status = ORC_OK; break; }
    double rho_new = dot(n, r, rt);
    double beta = (rho_new / rho) * (alpha / omega);
    rho = rho_new;
    if (omega == 0.0 || !isfinite(beta)) { status = ORC_BREAKDOWN; break; }
    for (size_t i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
  }
out:
  res->status = status;
  res->half_iters = half;
  res->relres = norm0 > 0 ? res->norm / norm0 : 0.0;
#undef SPMV
#undef PREC
#undef HIST
  free(r); free(rt); free(p); free(v); free(ph); free(s); free(t);
  return status;
}

void orc_grad_a(int nb, const int *rowptr, const int *colind,
                const double *lambda, const double *x, double *dA) {
  for (int i = 0; i < nb; ++i)
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      int j = colind[k];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          dA[(size_t)k * 9 + r * 3 + c] = -lambda[3 * (size_t)i + r] * x[3 * (size_t)j + c];
    }
}

/* ------------------------------------------------------------------ */
/* threaded variant (CPU baseline timing)                               */
/* ------------------------------------------------------------------ */

static void spmv_omp(int nb, const int *rowptr, const int *colind,
                     const double *vals, const double *x, double *y) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nb; ++i) {
    double a0 = 0, a1 = 0, a2 = 0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const double *b = vals + (size_t)k * 9, *xj = x + 3 * (size_t)colind[k];
      a0 += b[0] * xj[0] + b[1] * xj[1] + b[2] * xj[2];
      a1 += b[3] * xj[0] + b[4] * xj[1] + b[5] * xj[2];
      a2 += b[6] * xj[0] + b[7] * xj[1] + b[8] * xj[2];
    }
    y[3 * i] = a0; y[3 * i + 1] = a1; y[3 * i + 2] = a2;
  }
}

static void ilu_omp(int ncolors, const int *color_ptr, const int *rowptr,
                    const int *colind, const double *lu, const double *dinv,
                    const double *p, double *z) {
  for (int c = 0; c < ncolors; ++c) {
#pragma omp parallel for schedule(static)
    for (int i = color_ptr[c]; i < color_ptr[c + 1]; ++i) {
      double a[3] = {p[3 * i], p[3 * i + 1], p[3 * i + 2]};
      for (int k = rowptr[i]; k < rowptr[i + 1] && colind[k] < i; ++k) {
        const double *b = lu + (size_t)k * 9, *yj = z + 3 * (size_t)colind[k];
        for (int r = 0; r < 3; ++r)
          a[r] -= b[r * 3] * yj[0] + b[r * 3 + 1] * yj[1] + b[r * 3 + 2] * yj[2];
      }
      z[3 * i] = a[0]; z[3 * i + 1] = a[1]; z[3 * i + 2] = a[2];
    }
  }
  for (int c = ncolors - 1; c >= 0; --c) {
#pragma omp parallel for schedule(static)
    for (int i = color_ptr[c]; i < color_ptr[c + 1]; ++i) {
      double a[3] = {z[3 * i], z[3 * i + 1], z[3 * i + 2]};
      for (int k = rowptr[i + 1] - 1; k >= rowptr[i] && colind[k] > i; --k) {
        const double *b = lu + (size_t)k * 9, *zj = z + 3 * (size_t)colind[k];
        for (int r = 0; r < 3; ++r)
          a[r] -= b[r * 3] * zj[0] + b[r * 3 + 1] * zj[1] + b[r * 3 + 2] * zj[2];
      }
      const double *d = dinv + (size_t)i * 9;
      for (int r = 0; r < 3; ++r)
        z[3 * i + r] = d[r * 3] * a[0] + d[r * 3 + 1] * a[1] + d[r * 3 + 2] * a[2];
    }
  }
}

/* z = (LU)^-T p with the explicit transpose T of the factored matrix
 * (blocks transposed): T's strictly lower blocks are U^T, its strictly
 * upper ones L^T. Forward over colors with the transposed inverse diagonal
 * blocks (U^T y = p), then backward with the unit diagonal (L^T z = y);
 * the rows of one color are independent (structurally symmetric pattern). */
static void ilu_t_omp(int ncolors, const int *color_ptr, const int *trowptr,
                      const int *tcolind, const double *tlu, const double *dinv,
                      const double *p, double *z) {
  for (int c = 0; c < ncolors; ++c) {
#pragma omp parallel for schedule(static)
    for (int i = color_ptr[c]; i < color_ptr[c + 1]; ++i) {
      double a[3] = {p[3 * i], p[3 * i + 1], p[3 * i + 2]};
      for (int k = trowptr[i]; k < trowptr[i + 1] && tcolind[k] < i; ++k) {
        const double *b = tlu + (size_t)k * 9, *yj = z + 3 * (size_t)tcolind[k];
        for (int r = 0; r < 3; ++r)
          a[r] -= b[r * 3] * yj[0] + b[r * 3 + 1] * yj[1] + b[r * 3 + 2] * yj[2];
      }
      const double *d = dinv + (size_t)i * 9;   /* (D^-1)^T: column r of d */
      for (int r = 0; r < 3; ++r)
        z[3 * i + r] = d[r] * a[0] + d[3 + r] * a[1] + d[6 + r] * a[2];
    }
  }
  for (int c = ncolors - 1; c >= 0; --c) {
#pragma omp parallel for schedule(static)
    for (int i = color_ptr[c]; i < color_ptr[c + 1]; ++i) {
      double a[3] = {z[3 * i], z[3 * i + 1], z[3 * i + 2]};
      for (int k = trowptr[i + 1] - 1; k >= trowptr[i] && tcolind[k] > i; --k) {
        const double *b = tlu + (size_t)k * 9, *zj = z + 3 * (size_t)tcolind[k];
        for (int r = 0; r < 3; ++r)
          a[r] -= b[r * 3] * zj[0] + b[r * 3 + 1] * zj[1] + b[r * 3 + 2] * zj[2];
      }
      z[3 * i] = a[0]; z[3 * i + 1] = a[1]; z[3 * i + 2] = a[2];
    }
  }
}

void orc_transpose_bsr(int nb, const int *rowptr, const int *colind, const double *vals,
                       int *trowptr, int *tcolind, double *tvals) {
  int *fill = (int *)calloc((size_t)nb + 1, sizeof(int));
  for (int i = 0; i <= nb; ++i) trowptr[i] = 0;
  for (int k = 0; k < rowptr[nb]; ++k) trowptr[colind[k] + 1]++;
  for (int i = 0; i < nb; ++i) trowptr[i + 1] += trowptr[i];
  for (int i = 0; i < nb; ++i) fill[i] = trowptr[i];
  for (int i = 0; i < nb; ++i)             /* rows ascending: columns sorted */
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int p = fill[colind[k]]++;
      tcolind[p] = i;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) tvals[(size_t)p * 9 + r * 3 + c] = vals[(size_t)k * 9 + c * 3 + r];
    }
  free(fill);
}

static double dot_omp(size_t n, const double *a, const double *b) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (long i = 0; i < (long)n; ++i) s += a[i] * b[i];
  return s;
}

static int bicgstab_omp_core(int nb, int ncolors, const int *color_ptr,
                             const int *rowptr, const int *colind, const double *avals,
                             const double *lu, const double *dinv, const double *b,
                             double *x, double tol, int absolute, int maxit,
                             int nthreads, orc_result *res, int transpose);

int orc_bicgstab_omp(int nb, int ncolors, const int *color_ptr,
                     const int *rowptr, const int *colind, const double *avals,
                     const double *lu, const double *dinv, const double *b,
                     double *x, double tol, int absolute, int maxit,
                     int nthreads, orc_result *res) {
  return bicgstab_omp_core(nb, ncolors, color_ptr, rowptr, colind, avals, lu, dinv, b, x, tol,
                           absolute, maxit, nthreads, res, 0);
}

int orc_bicgstab_omp_t(int nb, int ncolors, const int *color_ptr,
                       const int *trowptr, const int *tcolind, const double *tavals,
                       const double *tlu, const double *dinv, const double *b,
                       double *x, double tol, int absolute, int maxit,
                       int nthreads, orc_result *res) {
  return bicgstab_omp_core(nb, ncolors, color_ptr, trowptr, tcolind, tavals, tlu, dinv, b, x,
                           tol, absolute, maxit, nthreads, res, 1);
}

static int bicgstab_omp_core(int nb, int ncolors, const int *color_ptr,
                             const int *rowptr, const int *colind, const double *avals,
                             const double *lu, const double *dinv, const double *b,
                             double *x, double tol, int absolute, int maxit,
                             int nthreads, orc_result *res, int transpose) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  size_t n = 3 * (size_t)nb;
  long ln = (long)n;
  double *r = (double *)malloc(8 * n), *rt = (double *)malloc(8 * n);
  double *p = (double *)malloc(8 * n), *v = (double *)malloc(8 * n);
  double *ph = (double *)malloc(8 * n), *s = (double *)malloc(8 * n);
  double *t = (double *)malloc(8 * n);
  memset(res, 0, sizeof *res);
  spmv_omp(nb, rowptr, colind, avals, x, v);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < ln; ++i) { r[i] = b[i] - v[i]; rt[i] = r[i]; p[i] = r[i]; }
  double rho = dot_omp(n, r, r), norm0 = sqrt(rho);
  res->norm0 = norm0; res->norm = norm0; res->norms[0] = norm0;
  double bound = absolute ? tol : ORC_ALREADY_SOLVED;
  int status = ORC_MAXIT, half = 0;
  if (!isfinite(norm0)) { status = ORC_NONFINITE; half = -1; goto out; }
  if (!(norm0 > bound)) { status = ORC_ALREADY_CONVERGED; half = -1; goto out; }
  if (!absolute) bound = tol * norm0;
  for (int k = 0;; ++k) {
    half = 2 * k;
    (transpose ? ilu_t_omp : ilu_omp)(ncolors, color_ptr, rowptr, colind, lu, dinv, p, ph);
    spmv_omp(nb, rowptr, colind, avals, ph, v);
    double vr = dot_omp(n, v, rt), alpha = rho / vr;
    if (vr == 0.0 || !isfinite(alpha)) { status = ORC_BREAKDOWN; break; }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < ln; ++i) { x[i] += alpha * ph[i]; s[i] = r[i] - alpha * v[i]; }
    double ns = sqrt(dot_omp(n, s, s));
    push_norm(res, ns, half);
    if (!isfinite(ns)) { status = ORC_NONFINITE; break; }
    if (!(ns > bound)) { status = ORC_OK; break; }
    if (k == maxit) { status = ORC_MAXIT; break; }
    half = 2 * k + 1;
    (transpose ? ilu_t_omp : ilu_omp)(ncolors, color_ptr, rowptr, colind, lu, dinv, s, ph);
    spmv_omp(nb, rowptr, colind, avals, ph, t);
    double ts = dot_omp(n, t, s), tt = dot_omp(n, t, t), omega = ts / tt;
    if (tt == 0.0 || !isfinite(omega)) { status = ORC_BREAKDOWN; break; }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < ln; ++i) { x[i] += omega * ph[i]; r[i] = s[i] - omega * t[i]; }
    double nr = sqrt(dot_omp(n, r, r));
    push_norm(res, nr, half);
    if (!isfinite(nr)) { status = ORC_NONFINITE; break; }
    if (!(nr > bound)) { status = ORC_OK; break; }
    double rho_new = dot_omp(n, r, rt), beta = (rho_new / rho) * (alpha / omega);
    rho = rho_new;
    if (omega == 0.0 || !isfinite(beta)) { status = ORC_BREAKDOWN; break; }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < ln; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
  }
out:
  res->status = status;
  res->half_iters = half;
  res->relres = norm0 > 0 ? res->norm / norm0 : 0.0;
  free(r); free(rt); free(p); free(v); free(ph); free(s); free(t);
  return status;
}

/* ------------------------------------------------------------------ */
/* mixed precision: float storage, float vectors, double dots, double IR */
/* ------------------------------------------------------------------ */

static void spmv_f(int nb, const int *rowptr, const int *colind,
                   const float *vals, const float *x, float *y) {
  for (int i = 0; i < nb; ++i) {
    float a0 = 0, a1 = 0, a2 = 0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const float *b = vals + (size_t)k * 9, *xj = x + 3 * (size_t)colind[k];
      a0 += b[0] * xj[0] + b[1] * xj[1] + b[2] * xj[2];
      a1 += b[3] * xj[0] + b[4] * xj[1] + b[5] * xj[2];
      a2 += b[6] * xj[0] + b[7] * xj[1] + b[8] * xj[2];
    }
    y[3 * i] = a0; y[3 * i + 1] = a1; y[3 * i + 2] = a2;
  }
}

static void ilu_f(int nb, const int *rowptr, const int *colind, const float *lu,
                  const float *dinv, const float *p, float *z) {
  if (z != p) memcpy(z, p, sizeof(float) * 3 * (size_t)nb);
  for (int i = 0; i < nb; ++i) {
    float a[3] = {z[3 * i], z[3 * i + 1], z[3 * i + 2]};
    for (int k = rowptr[i]; k < rowptr[i + 1] && colind[k] < i; ++k) {
      const float *b = lu + (size_t)k * 9, *yj = z + 3 * (size_t)colind[k];
      for (int r = 0; r < 3; ++r)
        a[r] -= b[r * 3] * yj[0] + b[r * 3 + 1] * yj[1] + b[r * 3 + 2] * yj[2];
    }
    z[3 * i] = a[0]; z[3 * i + 1] = a[1]; z[3 * i + 2] = a[2];
  }
  for (int i = nb - 1; i >= 0; --i) {
    float a[3] = {z[3 * i], z[3 * i + 1], z[3 * i + 2]};
    for (int k = rowptr[i + 1] - 1; k >= rowptr[i] && colind[k] > i; --k) {
      const float *b = lu + (size_t)k * 9, *zj = z + 3 * (size_t)colind[k];
      for (int r = 0; r < 3; ++r)
        a[r] -= b[r * 3] * zj[0] + b[r * 3 + 1] * zj[1] + b[r * 3 + 2] * zj[2];
    }
    const float *d = dinv + (size_t)i * 9;
    for (int r = 0; r < 3; ++r)
      z[3 * i + r] = d[r * 3] * a[0] + d[r * 3 + 1] * a[1] + d[r * 3 + 2] * a[2];
  }
}

static double dot_f(size_t n, const float *a, const float *b) {
  double s = 0;
  for (size_t i = 0; i < n; ++i) s += (double)a[i] * (double)b[i];
  return s;
}

/* one inner solve A d = r (float), d starts at 0, BiCGSTAB in PROGRAM order */
static int inner_solve_f(int nb, const int *rowptr, const int *colind,
                         const float *a, const float *lu, const float *dinv,
                         const float *rhs, float *d, double tol, int maxit,
                         int *half_out) {
  size_t n = 3 * (size_t)nb;
  float *r = (float *)malloc(4 * n), *rt = (float *)malloc(4 * n);
  float *p = (float *)malloc(4 * n), *v = (float *)malloc(4 * n);
  float *ph = (float *)malloc(4 * n), *s = (float *)malloc(4 * n);
  float *t = (float *)malloc(4 * n);
  for (size_t i = 0; i < n; ++i) { d[i] = 0; r[i] = rhs[i]; rt[i] = r[i]; p[i] = r[i]; }
  double rho = dot_f(n, r, r), bound = tol * sqrt(rho);
  int status = ORC_MAXIT, half = 0;
  for (int k = 0;; ++k) {
    half = 2 * k;
    ilu_f(nb, rowptr, colind, lu, dinv, p, ph);
    spmv_f(nb, rowptr, colind, a, ph, v);
    double vr = dot_f(n, v, rt), alpha = rho / vr;
    if (vr == 0.0 || !isfinite(alpha)) { status = ORC_BREAKDOWN; break; }
    float fa = (float)alpha;
    for (size_t i = 0; i < n; ++i) { d[i] += fa * ph[i]; s[i] = r[i] - fa * v[i]; }
    double ns = sqrt(dot_f(n, s, s));
    if (!(ns > bound)) { status = ORC_OK; break; }
    if (k == maxit) break;
    half = 2 * k + 1;
    ilu_f(nb, rowptr, colind, lu, dinv, s, ph);
    spmv_f(nb, rowptr, colind, a, ph, t);
    double ts = dot_f(n, t, s), tt = dot_f(n, t, t), omega = ts / tt;
    if (tt == 0.0 || !isfinite(omega)) { status = ORC_BREAKDOWN; break; }
    float fo = (float)omega;
    for (size_t i = 0; i < n; ++i) { d[i] += fo * ph[i]; r[i] = s[i] - fo * t[i]; }
    double nr = sqrt(dot_f(n, r, r));
    if (!(nr > bound)) { status = ORC_OK; break; }
    double rho_new = dot_f(n, r, rt), beta = (rho_new / rho) * (alpha / omega);
    rho = rho_new;
    float fb = (float)beta;
    for (size_t i = 0; i < n; ++i) p[i] = r[i] + fb * (p[i] - fo * v[i]);
  }
  *half_out = half;
  free(r); free(rt); free(p); free(v); free(ph); free(s); free(t);
  return status;
}

int orc_mixed_ir(int nb, const int *rowptr, const int *colind,
                 const double *avals, const double *lu, const double *dinv,
                 const double *b, double *x, double tol, double inner_tol,
                 int inner_maxit, int max_outer, orc_result *res, int *outer,
                 int *inner_half) {
  size_t n = 3 * (size_t)nb, nnz9 = (size_t)rowptr[nb] * 9, nd = (size_t)nb * 9;
  float *af = (float *)malloc(4 * nnz9), *luf = (float *)malloc(4 * nnz9);
  float *df = (float *)malloc(4 * nd);
  for (size_t i = 0; i < nnz9; ++i) { af[i] = (float)avals[i]; luf[i] = (float)lu[i]; }
  for (size_t i = 0; i < nd; ++i) df[i] = (float)dinv[i];
  double *r = (double *)malloc(8 * n), *ax = (double *)malloc(8 * n);
  float *rf = (float *)malloc(4 * n), *df_ = (float *)malloc(4 * n);
  memset(res, 0, sizeof *res);
  orc_spmv(nb, rowptr, colind, avals, x, ax);
  for (size_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
  double norm0 = sqrt(dot(n, r, r)), nr = norm0;
  res->norm0 = norm0;
  int status = ORC_MAXIT, o = 0, tot = 0;
  if (!(norm0 > ORC_ALREADY_SOLVED)) { status = ORC_ALREADY_CONVERGED; goto out; }
  for (o = 0; o < max_outer && nr > tol * norm0; ++o) {
    double scale = 1.0 / nr;
    for (size_t i = 0; i < n; ++i) rf[i] = (float)(r[i] * scale);
    int h = 0;
    int st = inner_solve_f(nb, rowptr, colind, af, luf, df, rf, df_, inner_tol,
                           inner_maxit, &h);
    tot += h + 1;
    if (st == ORC_BREAKDOWN) { status = ORC_BREAKDOWN; break; }
    for (size_t i = 0; i < n; ++i) x[i] += nr * (double)df_[i];
    orc_spmv(nb, rowptr, colind, avals, x, ax);
    for (size_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
    nr = sqrt(dot(n, r, r));
    if (!isfinite(nr)) { status = ORC_NONFINITE; break; }
  }
  if (nr <= tol * norm0) status = ORC_OK;
out:
  res->status = status;
  res->norm = nr;
  res->relres = norm0 > 0 ? nr / norm0 : 0.0;
  *outer = o;
  *inner_half = tot;
  free(af); free(luf); free(df); free(r); free(ax); free(rf); free(df_);
  return status;
}
