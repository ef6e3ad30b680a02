/*
 * gbilu -- GB300-native ILU0-preconditioned BiCGSTAB for 3x3-block BSR
 * systems. C ABI of libgbilu.so: plain pointers and sizes, int status
 * returns, caller-owned host arrays, device memory owned by the handle.
 *
 * It replaces the host library that drives the OPM/FPGA Alveo kernel
 * (linearalgebra/ilu0bicgstab/xilinx/src/sda_app/common/
 * fpga_functions_bicgstab.hpp:30-136). That library consumes a matrix that
 * the Flow backend has already colored, ILU0-factored and packed; here the
 * library does those steps itself from plain BSR arrays:
 *
 *   fpga_setup_host_datamem (fpga_functions_bicgstab.hpp:33-47)
 *   + the coloring/packing that fills vectorPointers   -> gbilu_analyze
 *   fpga_copy_host_datamem (:49-61)
 *   + fpga_copy_to_device_datamem (:77-78)
 *   + the ILU0 factorization feeding vectorPointers[18] -> gbilu_factor
 *   fpga_set_kernel_parameters (:119-122)
 *   + fpga_kernel_run (:124)
 *   + fpga_copy_from_device_debugbuf (:84-92)
 *   + fpga_map_results / fpga_unmap_results (:105-113)  -> gbilu_solve
 *
 * Conventions (same as the reference host library):
 *  - every function returns int, 0 (GBILU_OK) on success; on failure a
 *    GBILU_* code and a message retrievable with gbilu_last_error();
 *  - single-threaded use per handle; calls block until the device is done;
 *  - block values are 3x3 row-major, vals[k*9 + r*3 + c]; vectors hold
 *    3*nb doubles with unknown 3*i+r belonging to block row i.
 */
#ifndef GBILU_H
#define GBILU_H

#ifdef __cplusplus
extern "C" {
#endif

#define GBILU_ABI_VERSION 1

/* return / solve status codes */
enum {
  GBILU_OK = 0,                /* converged (solve) or call succeeded */
  GBILU_MAXIT = 1,             /* stopped at the iteration limit */
  GBILU_ALREADY_CONVERGED = 2, /* ||b - A x0|| met the bound before any
                                  iteration; x untouched ("no results",
                                  bicgstab_utils.cpp:133) */
  GBILU_BREAKDOWN = 3,         /* (v,rt) == 0, (t,t) == 0 or omega == 0 */
  GBILU_NONFINITE = 4,         /* NaN or Inf in a residual norm */
  GBILU_TIMEOUT = 5,           /* device time budget exceeded (the
                                  reference's abort_cycles,
                                  fpga_functions_bicgstab.cpp:1254) */
  GBILU_BAD_INPUT = 6,         /* invalid arguments or sparsity pattern */
  GBILU_SINGULAR = 7,          /* singular diagonal block in ILU0 */
  GBILU_CUDA_ERROR = 8,        /* a CUDA call failed */
  GBILU_NOT_READY = 9,         /* wrong call order (e.g. solve before factor) */
  GBILU_NO_DEVICE = 10         /* handle created host-only (device = -1) */
};

/* precision modes */
enum {
  GBILU_FP64 = 0,   /* FP64 storage and arithmetic (the reference's mode) */
  GBILU_MIXED = 1   /* FP32 storage/sweeps inside FP64 iterative refinement */
};

typedef struct {
  int precision;      /* GBILU_FP64 or GBILU_MIXED */
  int absolute_tol;   /* 0: stop when ||r|| <= tol*||r0|| (relative);
                         1: stop when ||r|| <= tol. Setup-array config bit 1
                         (fpga_functions_bicgstab.cpp:423, solver.vhd:587) */
  int device;         /* CUDA device ordinal; -1 = host-only handle that
                         can analyze and factor but not solve */
  int use_graph;      /* 1: iteration loop as a CUDA graph with a device-
                         side while loop; 0: host-driven launches */
  double timeout_ms;  /* 0 = none; else a solve that exceeds this device
                         time stops with GBILU_TIMEOUT */
  double inner_tol;   /* mixed: relative tolerance of each inner solve */
  int inner_maxit;    /* mixed: iteration limit of each inner solve */
  int max_outer;      /* mixed: refinement step limit */
  int verbose;        /* 0 quiet, 1 INFO lines on stdout */
  int sweep_mode;     /* 1: the whole ILU0 apply is one cooperative launch
                         (default): grid barriers around the large
                         colors, the small ones ordered by their data;
                         0: one launch per color */
  int factor_on_device; /* 1: gbilu_factor permutes and ILU0-factors on the
                         GPU (color-parallel, bit-identical to the host
                         factorization); 0: on the host (default) */
  int mixed_scheme;   /* mixed mode: 0 (default) iterative refinement: FP64
                         b - Ax, FP32 inner solves of A d = r to inner_tol,
                         x += d in FP64; 1 one FP32 BiCGSTAB run whose residual
                         is replaced by the FP64 b - Ax whenever it dropped by
                         ru_delta, x accumulated in FP64, stop on the FP64
                         residual */
  double ru_delta;    /* mixed scheme 1: replacement threshold (default 0.1) */
  int stage_small_steps; /* 1 (default): the single-launch apply copies the
                         small color steps' matrix slices into shared memory
                         when it starts and orders those steps by their data;
                         0: they read global memory and are separated by grid
                         barriers, like the large steps (same results) */
  int coloring;       /* 0 (default): first-fit greedy in the grid's parity
                         order -- rows two-colored by the parity of their
                         distance over blocks that lie on a 4-cycle (grid
                         faces), one end of each equal-parity block (a fault
                         connection) moved to the end of the order -- which
                         leaves one small color on a grid with faults;
                         1: first-fit greedy in natural row order */
  int stream_large_steps; /* 1: in the single-launch apply one warp per CTA
                         streams the large color steps' matrix slices into a
                         shared-memory ring with bulk copies (running ahead
                         across barriers) and the others compute from it;
                         0 (default): every warp loads its own rows (same
                         results) */
  int color_on_device; /* 1: gbilu_analyze computes the parity-order coloring
                         (coloring = 0) on the GPU, the same colors bit for
                         bit; 0 (default): on the host */
} gbilu_options;

typedef struct {
  int status;           /* GBILU_OK, _MAXIT, _ALREADY_CONVERGED, ... */
  int half_iters;       /* the reference's half-iteration counter at the
                           stop (bicgstab_utils.cpp:223): 2k after the first
                           half of iteration k, 2k+1 after the second;
                           -1 when no iteration ran */
  double iterations;    /* half_iters/2 + 0.5 (fpga_functions_bicgstab.cpp:926) */
  double norm0;         /* ||b - A x0|| */
  double norm;          /* last residual norm the solver computed */
  double relres;        /* norm / norm0 */
  double norms[4];      /* norms[0] initial norm, [1..3] ring of the three
                           latest (bicgstab_utils.cpp:248-258) */
  int last_norm_idx;    /* index of the newest entry in norms */
  int outer_iters;      /* mixed: refinement steps (scheme 0) or residual
                           replacements (scheme 1) */
  int inner_half_iters; /* mixed: inner half-iterations over all steps */
  double true_relres;   /* mixed: ||b - A x|| / ||b - A x0|| in FP64 */
  double device_ms;     /* device time of the solve (CUDA events) */
  double total_ms;      /* host wall time including host<->device copies */
} gbilu_result;

typedef struct {
  int nb;               /* block rows */
  int nnzb;             /* blocks of A */
  int ncolors;          /* colors of the greedy coloring */
  int nnzb_lower;       /* blocks of L (strictly lower) */
  int nnzb_upper;       /* blocks of U (strictly upper) */
  int slices;           /* 32-row slices of the device layout */
  long long slots_a;    /* padded block slots of A (x32 lanes) */
  long long slots_l;
  long long slots_u;
  long long device_bytes;   /* device memory held by the handle */
  int launches_per_iter;    /* kernels one BiCGSTAB iteration launches */
  long long last_launches;  /* kernels launched by the last solve */
  double factor_ms;         /* host ILU0 + upload time of the last factor */
  double analyze_ms;
  /* algorithmic bytes (every operand read or written once, x gathers
   * counted once) of one SpMV, one ILU apply and one full iteration:
   * [0] FP64 storage and vectors, [1] FP32 storage and vectors */
  double alg_bytes_spmv[2];
  double alg_bytes_ilu[2];
  double alg_bytes_iter[2];
  /* the forward single-launch apply, [0] FP64 / [1] FP32 (0 when that
   * precision is not set up): stages and bytes per stage of the ring that
   * streams the large color steps, dynamic shared memory per CTA */
  int ring_stages[2];
  int ring_stage_bytes[2];
  int apply_smem_bytes[2];
  double color_ms;          /* the coloring inside the last gbilu_analyze */
  int color_on_device;      /* 1: it ran on the GPU */
} gbilu_stats;

/* fill *opt with defaults: FP64, relative tolerance, device 0, graph on,
 * no timeout, inner_tol 1e-1, inner_maxit 500, max_outer 30, single-launch
 * sweeps, host factorization, mixed scheme 0, ru_delta 0.1, small steps
 * staged, parity-order coloring */
int gbilu_default_options(gbilu_options *opt);

int gbilu_create(const gbilu_options *opt, void **handle);
int gbilu_destroy(void *handle);

/* Sparsity analysis: greedy block coloring, color-ordered permutation,
 * L/U split and the device layout. rowptr[nb+1], colind[nnzb] 0-based,
 * columns sorted and unique per row, diagonal block present, the pattern
 * structurally symmetric (block (i, j) present iff (j, i) is, as in the
 * simulator's matrices; values need not be symmetric).
 * Structure of fpga_setup_host_datamem's sizes (fpga_functions_bicgstab.cpp
 * :84-131) and of the coloring that fills vectorPointers (:608-629). */
int gbilu_analyze(void *handle, int nb, const int *rowptr, const int *colind);

/* Coloring and ordering chosen by gbilu_analyze; pointers may be NULL.
 * color[nb], perm[nb] (perm[new] = old), color_ptr[ncolors+1]. */
int gbilu_get_ordering(void *handle, int *ncolors, int *color, int *perm,
                       int *color_ptr);

/* Self-test of the device waits' bounds (failure detection without a GPU
 * fault): mode 0 runs a grid barrier that one of its two CTAs never reaches,
 * mode 1 a data-ordered load of a word that stays the sentinel. The wait
 * runs out after its poll limit (about a second or two), and the probe
 * reports what the solve kernels would report: *bar_fail (1: barrier, 3:
 * data wait), *status (GBILU_TIMEOUT) and the device time in *ms. The
 * handle's solve state is untouched and stays usable. Counterpart of the
 * reference's kernel watchdog (abort_cycles, reported as kernel_aborted by
 * bicgstab_utils.cpp:93-129). */
int gbilu_wait_probe(void *handle, int mode, int *bar_fail, int *status, double *ms);

/* Diagnostic of the mixed mode's dot products: (x, y) of two FP32 host
 * vectors of length n (n <= 3*nb) computed on the device as the FP32
 * kernels of a mixed solve accumulate their dots (*dot_df: an error-free
 * double-float sum per thread on the FP32 pipe, FP64 across threads) and
 * with FP64 sums per thread (*dot_fp64). Needs GBILU_MIXED. No counterpart
 * in the reference, whose dots are FP64. */
int gbilu_dot_check(void *handle, int n, const float *x, const float *y, double *dot_df,
                    double *dot_fp64);

/* The numbering of the device vectors and sliced layouts: order[d] = input
 * row held at device row d. It keeps perm's color ranges and each color's
 * leading rows with a higher-colored neighbour, and inside each of these
 * runs sorts the rows by descending block count so that the 32 rows of a
 * slice carry nearly equal numbers of blocks (no padding slots). Row
 * results are unchanged by it: every row keeps its blocks in the order of
 * the permuted numbering. A diagnostic; the solve functions take and return
 * vectors in input order. */
int gbilu_device_order(void *handle, int *order);

/* Block ILU0 of A (values in the order of the analyzed colind, nnzb*9
 * doubles) in the color-permuted order, FP64 3x3 inversions, and upload of
 * A, L, U and the inverted diagonal blocks to the device (the arrays
 * fpga_copy_host_datamem copies, fpga_functions_bicgstab.cpp:606-629).
 * Can be called again with new values after one gbilu_analyze. */
int gbilu_factor(void *handle, const double *vals);

/* The factors computed by gbilu_factor, in the permuted BSR order with
 * sorted columns (blocks with col < row: L; col >= row: U), and the
 * inverted diagonal blocks; lu[nnzb*9], dinv[nb*9]; either may be NULL. */
int gbilu_get_factors(void *handle, double *lu, double *dinv);

/* Solve A x = b. b[3*nb] and x[3*nb] are HOST arrays in the original
 * numbering; x holds x0 on entry and the solution on return. tol and maxit
 * follow the reference: maxit full iterations plus the first half of one
 * more (solver.vhd:557, solver_pkg.vhd:127-128). res may be NULL.
 * In GBILU_MIXED mode maxit caps the FP32 inner half-iterations of all
 * refinement steps together at 2*maxit + 1 (scheme 0: each inner solve is
 * also capped by inner_maxit and the steps by max_outer; scheme 1: the one
 * FP32 run), and a solve stopped by the cap returns GBILU_MAXIT; res->
 * half_iters is then the total inner half-iterations minus one, the value
 * the reference's counter would show had all inner halves been one run
 * (2*maxit at the cap), and res->inner_half_iters the total itself.
 * When both arrays are page-locked (cudaHostAlloc / cudaHostRegister), x0
 * and x move over the CPU-GPU link in place and b by the copy engine while
 * A x0 is computed; other host memory goes through staging copies. Both
 * give the same bits. */
int gbilu_solve(void *handle, const double *b, double *x, double tol,
                int maxit, gbilu_result *res);

/* As gbilu_solve with DEVICE pointers (original numbering). */
int gbilu_solve_device(void *handle, const double *d_b, double *d_x,
                       double tol, int maxit, gbilu_result *res);

/* Single operator applications in FP64, host arrays, original numbering:
 * y = A x (transpose: y = A^T x) -- the SpMV steps 0/4/9 of the PROGRAM
 * (solver_pkg.vhd:122,126,131); z = (LU)^-1 p (transpose: (LU)^-T p) --
 * the ILU0 L/U sweeps of steps 2/3 (solver_pkg.vhd:124-125). */
int gbilu_apply_spmv(void *handle, const double *x, double *y, int transpose);
int gbilu_apply_ilu(void *handle, const double *p, double *z, int transpose);

/* Adjoint of x = A^-1 b for a loss L(x): given g = dL/dx at the solution
 * x (host arrays, original numbering), solves A^T lambda = g with the
 * transposed SpMV and U^T/L^T sweeps reusing the forward factors, and
 * forms dL/db = lambda and dL/dA = -lambda_i x_j^T on the pattern
 * (dA[nnzb*9] in the analyzed input block order; may be NULL). lambda
 * stays on the device between the solve and the gradient; res->device_ms
 * covers the whole backward pass (transposed solve and dL/dA). No
 * counterpart in the reference, which has no gradient path. */
int gbilu_adjoint(void *handle, const double *g, const double *x,
                  double *lambda, double *dA, double tol, int maxit,
                  gbilu_result *res);

/* As gbilu_adjoint with DEVICE pointers (original numbering): d_g[3*nb],
 * d_x[3*nb] in, d_lambda[3*nb] out (x0 = 0), d_dA[nnzb*9] out or NULL. */
int gbilu_adjoint_device(void *handle, const double *d_g, const double *d_x,
                         double *d_lambda, double *d_dA, double tol, int maxit,
                         gbilu_result *res);

int gbilu_get_stats(void *handle, gbilu_stats *stats);

/* Times one kernel family on the handle's stream with CUDA events, reps
 * applications back to back on the factored system: which = 0 SpMV FP64,
 * 1 ILU apply FP64 (all colors), 2 SpMV FP32, 3 ILU apply FP32; the other
 * kernels of one iteration, 4-8 in FP64 and 9-13 in FP32: SpMV with the
 * alpha dot, SpMV with the omega dots, update_s, update_r, update_p (FP32
 * ids need GBILU_MIXED). Returns the average device ms per application, its
 * algorithmic bytes and the kernel launches per application. The
 * counterpart of the reference's kernel timing around clEnqueueTask
 * (fpga_functions_bicgstab.cpp:1305-1325), per kernel instead of per run. */
int gbilu_bench_kernel(void *handle, int which, int reps, double *avg_ms,
                       double *alg_bytes, int *launches);

/* Traced ILU apply: runs the single-launch preconditioner apply (FP64, or
 * FP32 with GBILU_MIXED; forward or transposed) with device timestamps at
 * every color step and returns each step's duration in microseconds (the
 * step plus the grid barrier after it, as CTA 0 sees it; inside a run of
 * small steps ordered by their data, CTA 0's own progress) and its row
 * count. The GB300
 * counterpart of the reference's periodic debug lines (solver.vhd:1106-1133),
 * per color step instead of per sampling interval. */
/* The step list of the single-launch ILU apply (forward or transposed) for
 * the analyzed pattern, a diagnostic of its schedule: per step 13 ints
 * {row0, nrows, slice0, lane0 (lane of row0 in its slice), matrix (0: first
 * sweep, 1: second), has_d, own_y, nbr_hat, src_rows, to_y, final0,
 * final_d, barrier_after (1: a grid barrier ends the step; 2: a CTA barrier
 * only -- the step and the next have one slice each and run on the same
 * CTA; 3: no barrier -- both steps are small, staged in shared memory, and
 * the next one waits for each value it reads)}. Up to cap steps
 * are written; *nsteps gets the count. Works on host-only handles.
 * Counterpart of the reference's per-color processing order
 * (sparstition.vhd:751-756, ilu0.vhd:293-323,406-417). */
int gbilu_schedule(void *handle, int transpose, int cap, int *nsteps, int *steps);

int gbilu_ilu_trace(void *handle, int fp32, int transpose, double *us, int *rows,
                    int cap, int *nphases);

const char *gbilu_status_string(int status);
const char *gbilu_last_error(void *handle);

/* --- interchange with the Alveo kernel's host-side formats (host only) --- */

/* Bank layout of the five data buffers and the 40-word (5-cacheline) setup
 * array, as fpga_setup_host_datamem builds them
 * (fpga_functions_bicgstab.cpp:84-496, port configuration 2r_3r3w).
 * processed_sizes[18] as there (row, val, colors, columns, new-row, block-diag
 * sizes of A, then of L, then of U), nnz_sizes[3] = value counts of A, L, U.
 * Outputs: setup[40], totals[5] (bytes per bank), offsets[23] (byte offset of
 * setup, nnz, L/U nnz, color sizes, L/U color sizes, block diag | P indices,
 * L/U P indices, col indices, L/U col indices, NRs, L/U NRs | X2, R1 | X1, R2
 * | L res, U res inside their bank; may be NULL) and result_offsets[6] (X
 * even, R even, X odd, R odd, L res, U res; may be NULL). debug_bytes must be
 * a whole number of 64-byte lines, else GBILU_BAD_INPUT. */
int gbilu_fpga_layout(unsigned int config_bits, const int *processed_sizes,
                      const int *nnz_sizes, unsigned int debug_bytes,
                      unsigned long long *setup, unsigned int *totals,
                      long long *offsets, unsigned int *result_offsets);

/* Packs the backend's vectorPointers (indices as in
 * fpga_functions_bicgstab.cpp:606-629) into the five banks exactly as
 * fpga_copy_host_datamem does after a reset: setup array first, color sizes
 * past their 8-int header, results sentinels in the padding of X2/R2 when
 * fill_results is set. banks[b] must hold totals[b] bytes of
 * gbilu_fpga_layout. */
int gbilu_fpga_pack(unsigned int config_bits, const int *processed_sizes,
                    const int *nnz_sizes, void *const *vector_pointers,
                    const int *vector_sizes, int fill_results,
                    unsigned char *const *banks);

/* Exports the analyzed and factored system as the backend's vectorPointers
 * that fpga_copy_host_datamem packs for the Alveo kernel
 * (fpga_functions_bicgstab.cpp:528-545 sizes, :606-629 arrays): scalar rows
 * in the color-permuted order, every color cut into parts ("colors" of the
 * kernel) within the kernel's limits (2048 rows, 8192 vector-copy entries
 * and 32768 values a part, 256 parts, 163840 unknowns, 2^21 values:
 * alveo_u280/rtl/pkg/constants.vhd:76-105; larger systems ->
 * GBILU_BAD_INPUT naming the limit). With vp == NULL it fills
 * vector_sizes[18] (rows, values, colors, vector-copy entries, new-row
 * offsets, block diagonal; for A, L, U) and nnz_sizes[3]; then the caller
 * allocates vp[0,6,12] color sizes (8 + 4*colors words), vp[1,7,13] P
 * indices (uint32), vp[2,8,14] a double* to the values, vp[3,9,15] column
 * indices (uint16), vp[4,10,16] new-row offsets (uint8), vp[18] the block
 * diagonal, vp[19] rhs and vp[20] x0 (3*nb doubles, permuted; b and x0 may
 * be NULL for zeros) and calls again with vp. The same arrays then go to
 * gbilu_fpga_pack. The format follows the kernel's RTL; gbilu_fpga_export.cpp
 * states it and the RTL lines it rests on. */
int gbilu_fpga_export(void *handle, const double *b, const double *x0, int *vector_sizes,
                      int *nnz_sizes, void *const *vector_pointers);

/* Writes a solve's outcome as the kernel's debug buffer (lines x 8 words):
 * line 0 = general status (signature, aborted / no-results flags, run length
 * in ns), line 1 = final status line (half-iteration counter, four-norm ring),
 * the rest the "unwritten" marker, so decode_debuginfo_bicgstab
 * (bicgstab_utils.cpp:90-280) reads GB300 runs. lines >= 2. */
int gbilu_status_lines(const gbilu_result *res, unsigned long long *buf, int lines);

/* Allocation-free y = A x and *d_dot = (y, w) on plain BSR device arrays
 * (rowptr[nb+1], colind, vals[nnzb*9], x, y, w[3*nb], one double for the
 * dot), enqueued on `stream` (a cudaStream_t, NULL = default stream). No
 * counterpart in the reference. For callers that cannot allocate device
 * memory or create a handle (a host framework that hands out a fixed
 * device arena, a callback in which cudaMalloc's implicit synchronisation
 * is not allowed): it calls no cudaMalloc/cudaFree; its reduction scratch
 * is a fixed ~32 KiB device array inside the library, which limits nb to
 * 1,048,576 block rows (larger nb -> GBILU_BAD_INPUT). y must not alias x
 * or w (w may alias x). The first call on a device looks the array's
 * address up in the device's primary context (the CUDA runtime's) and
 * keeps it for the life of the process: make that first call before any
 * stream capture, call it with the primary context current, and not
 * across a cudaDeviceReset. Calls that overlap on the GPU share the array
 * and race. */
int gbilu_bsr_spmv_dot_noalloc(int nb, const int *d_rowptr, const int *d_colind,
                               const double *d_vals, const double *d_x, double *d_y,
                               const double *d_w, double *d_dot, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GBILU_H */
