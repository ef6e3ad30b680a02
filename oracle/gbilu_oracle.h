/*
 * CPU oracle for the ILU0-BiCGSTAB path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the algorithm the OPM/FPGA Alveo kernel computes,
 * used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the
 * checker. Nothing in the product library links or calls this code.
 *
 * Parity status: the solver itself is only VHDL in the reference (there is
 * no CPU implementation, no golden vector and no known-answer test of the
 * solver in the reference tree), so the numeric part of this oracle is
 * "parity unpinned" against reference outputs; it is pinned by structural
 * identities instead (L*U == A on the pattern, dense LU on small grids, a
 * scipy cross-check). The host-side packed-buffer layout and the status-line
 * decoding are pinned against the reference's own host library compiled
 * under oracle/_ref (see oracle/ref/Makefile).
 *
 * The coloring, permutation and ILU0 factorization live in opm-simulators in
 * the reference setup (not vendored, no pinned version); the reference only
 * consumes their output (linearalgebra/ilu0bicgstab/xilinx/src/sda_app/
 * common/fpga_functions_bicgstab.cpp:506-629). Those three steps are defined
 * here as documented deterministic algorithms.
 *
 * Layout conventions: block sparse row (BSR) with 3x3 blocks stored
 * row-major, vals[k*9 + r*3 + c]; vectors hold 3*nb doubles, unknown 3*i+r
 * belongs to block row i.
 */
#ifndef GBILU_ORACLE_H
#define GBILU_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes, same values as include/gbilu.h */
enum {
  ORC_OK = 0, ORC_MAXIT = 1, ORC_ALREADY_CONVERGED = 2, ORC_BREAKDOWN = 3,
  ORC_NONFINITE = 4, ORC_BAD_INPUT = 6, ORC_SINGULAR = 7
};

/* Greedy first-fit coloring of the block graph, rows visited in natural
 * order: color[i] = smallest color not taken by an already colored
 * neighbour. Returns the number of colors. */
int orc_color_greedy(int nb, const int *rowptr, const int *colind, int *color);

/* Greedy first-fit coloring in the grid's parity order (the default of the
 * product): (1) a block (u, v) is a face when it lies on a 4-cycle
 * u - a - b - v - u of the block graph with a, b outside {u, v}; (2) every
 * row gets the parity of its breadth-first distance over face blocks from
 * the lowest-numbered row of its connected part; (3) the off-diagonal
 * blocks (u, v), u < v, whose ends have equal parity are visited in
 * row-major order: if neither end is moved yet, v is moved -- except that
 * u is moved when v has a moved neighbour and u has none; (4) rows are
 * colored first-fit in the order: parity-0 rows, parity-1 rows, moved rows,
 * natural order inside each class. Returns the number of colors. */
int orc_color_parity(int nb, const int *rowptr, const int *colind, int *color);

/* perm[new] = old: rows ordered by color; inside a color, the rows that
 * share a block with a row of a higher color (as either end) come first,
 * then the others, each group in natural order. color_ptr[c]..color_ptr[c+1]
 * is the new-index range of color c and split[c] the size of its first
 * group. (The rows of one color are never coupled, so this order inside a
 * color does not change the ILU0 factors.) */
void orc_color_order(int nb, const int *rowptr, const int *colind,
                     const int *color, int ncolors, int *perm, int *color_ptr,
                     int *split);

/* Permuted copy P A P^T with columns sorted inside each row.
 * prowptr[nb+1], pcolind[nnzb], pvals[nnzb*9]; src[k] = input block index. */
void orc_permute_bsr(int nb, const int *rowptr, const int *colind,
                     const double *vals, const int *perm, int *prowptr,
                     int *pcolind, double *pvals, int *src);

/* 3x3 inverse by cofactors; returns 0, or 1 when the block is singular or
 * the determinant is not finite. */
int orc_inv3(const double *a, double *out);

/* In-place block ILU(0) (IKJ order) of a BSR matrix with sorted columns.
 * On return blocks with col < row hold L (unit block diagonal implied),
 * blocks with col >= row hold U; dinv[i*9..] = inverse of U's diagonal block.
 * Returns 0, or -(i+1) when the pivot of row i is singular. */
int orc_bilu0(int nb, const int *rowptr, const int *colind, double *vals,
              double *dinv);

/* Explicit transpose of a BSR matrix with sorted columns: the pattern
 * transposed, each 3x3 block transposed; trowptr[nb+1], tcolind and
 * tvals[9*nnzb] sized like the input. */
void orc_transpose_bsr(int nb, const int *rowptr, const int *colind, const double *vals,
                       int *trowptr, int *tcolind, double *tvals);

/* y = A x */
void orc_spmv(int nb, const int *rowptr, const int *colind, const double *vals,
              const double *x, double *y);
/* y = A^T x */
void orc_spmv_t(int nb, const int *rowptr, const int *colind,
                const double *vals, const double *x, double *y);

/* z = (LU)^-1 p on the factored matrix (L forward, then U backward with
 * dinv); z may alias p. */
void orc_ilu_apply(int nb, const int *rowptr, const int *colind,
                   const double *lu, const double *dinv, const double *p,
                   double *z);
/* z = (LU)^-T p: U^T forward (with dinv^T), then L^T backward. */
void orc_ilu_apply_t(int nb, const int *rowptr, const int *colind,
                     const double *lu, const double *dinv, const double *p,
                     double *z);

typedef struct {
  int status;        /* ORC_* */
  int half_iters;    /* the reference's half-iteration counter at the stop;
                        -1 when the initial residual already met the bound */
  double norm0;      /* ||b - A x0|| */
  double norm;       /* last computed residual norm (s or r) */
  double relres;     /* norm / norm0 */
  double norms[4];   /* norms[0] = initial norm, [1..3] ring of the latest */
  int last_norm_idx; /* index in norms of the newest entry */
  int nhist;         /* entries written to hist */
} orc_result;

/* Right-preconditioned ILU0-BiCGSTAB in the reference's PROGRAM order.
 * A and the factors are given in the (same) permuted numbering; b, x in
 * that numbering too. x holds x0 on entry and the solution on return.
 * transpose != 0 solves A^T x = b with the transposed operators.
 * hist (may be NULL) receives up to hist_cap residual norms, one per
 * half-iteration, starting with the initial norm. */
int orc_bicgstab(int nb, const int *rowptr, const int *colind,
                 const double *avals, const double *lu, const double *dinv,
                 const double *b, double *x, double tol, int absolute,
                 int maxit, int transpose, orc_result *res, double *hist,
                 int hist_cap);

/* dA[k] = -lambda_i x_j^T for every block k = (i, j) of the pattern. */
void orc_grad_a(int nb, const int *rowptr, const int *colind,
                const double *lambda, const double *x, double *dA);

/* Threaded variants of the hot loop for the timed CPU baseline (OpenMP over
 * rows of one color / rows of the matrix / vector chunks). Same results as
 * the sequential versions up to the order of floating-point reductions. */
int orc_bicgstab_omp(int nb, int ncolors, const int *color_ptr,
                     const int *rowptr, const int *colind, const double *avals,
                     const double *lu, const double *dinv, const double *b,
                     double *x, double tol, int absolute, int maxit,
                     int nthreads, orc_result *res);

/* The same for the transposed system A^T x = b (the adjoint), on the
 * explicit transposes of A and of the factored matrix (orc_transpose_bsr):
 * the preconditioner is (LU)^-T, U^T with the transposed inverse diagonal
 * blocks forward over the colors, then L^T backward. */
int orc_bicgstab_omp_t(int nb, int ncolors, const int *color_ptr,
                       const int *trowptr, const int *tcolind, const double *tavals,
                       const double *tlu, const double *dinv, const double *b,
                       double *x, double tol, int absolute, int maxit,
                       int nthreads, orc_result *res);

/* Mixed-precision restatement: A, L, U and dinv rounded to float, inner
 * BiCGSTAB on float vectors with double dot accumulation, outer iterative
 * refinement with the double residual b - A x until relres <= tol.
 * inner_tol is the inner relative tolerance. Returns the number of outer
 * steps in *outer and the total inner half-iterations in *inner_half. */
int orc_mixed_ir(int nb, const int *rowptr, const int *colind,
                 const double *avals, const double *lu, const double *dinv,
                 const double *b, double *x, double tol, double inner_tol,
                 int inner_maxit, int max_outer, orc_result *res, int *outer,
                 int *inner_half);

#ifdef __cplusplus
}
#endif
#endif
