// gbilu_bridge.hpp -- C++ adapter between a simulator's linear-solver
// backend and libgbilu.so (header-only; only the C ABI of gbilu.h crosses
// the library boundary).
//
// In the reference setup the Flow simulator hands each Newton step's
// Jacobian (a Dune BCRSMatrix of 3x3 blocks) to an accelerator backend
// through a bridge that extracts the block row pointers, column indices and
// contiguous block values, and the backend then colors, factors, packs and
// calls the FPGA host library (fpga_functions_bicgstab.hpp:30-136: setup,
// copy, set parameters, run, read the debug buffer, map results). This
// adapter is the GB300 end of that bridge:
//
//   update_matrix(nb, rowptr, colind, vals)  -> gbilu_analyze when the
//       pattern changed (a new well, a changed grid), gbilu_factor always
//       (new values every Newton step): the coloring, permutation and device
//       layout survive across solves on one pattern;
//   solve(b, res) / get_result(x)            -> gbilu_solve from x0 = 0;
//   solve_system(...)                        -> both, with the status
//       classes a backend reports (analysis failed, preconditioner failed,
//       other failure) and a result record with the fields of Dune's
//       InverseOperatorResult (iterations, reduction, converged, elapsed).
//
// One bridge per thread (a handle is single-threaded), as in the reference.
#pragma once

#include "gbilu.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

namespace gbilu {

// How a solve_system call ended. A solve that stops at the iteration limit
// is Success with converged = false (the caller decides), as with the
// reference's kernel that simply reports its half-iteration count.
enum class SolverStatus { Success, AnalysisFailed, CreatePreconditionerFailed, UnknownError };

struct SolveResult {
  int iterations = 0;       // full iterations: ceil(half_iters / 2)
  int half_iters = -1;      // the reference's half-iteration counter
  double reduction = 0.0;   // ||r|| / ||r0|| (mixed: in FP64)
  bool converged = false;
  double elapsed = 0.0;     // seconds, host wall time of the solve call
  int status = GBILU_OK;    // GBILU_* status of the solve
};

class BsrBridge {
 public:
  // tol: relative tolerance, maxit: iteration limit (reference semantics);
  // opt: handle options (precision, device, ...). Without opt the library's
  // defaults, except that the refactorization of every Newton step and the
  // coloring of a new pattern run on the GPU (the same factors and colors
  // bit for bit; on the 500k-cell system 2.6 ms instead of 383 ms for the
  // factorization, 3.8 ms instead of 45 ms for the coloring).
  BsrBridge(double tol, int maxit, const gbilu_options *opt = nullptr) : tol_(tol), maxit_(maxit) {
    gbilu_options o;
    gbilu_default_options(&o);
    o.factor_on_device = 1;
    o.color_on_device = 1;
    if (opt) o = *opt;
    ok_ = gbilu_create(&o, &h_) == GBILU_OK;
    if (!ok_) err_ = h_ ? gbilu_last_error(h_) : "gbilu_create failed";
  }
  ~BsrBridge() {
    if (h_) gbilu_destroy(h_);
  }
  BsrBridge(const BsrBridge &) = delete;
  BsrBridge &operator=(const BsrBridge &) = delete;

  // New Jacobian values, possibly on a new pattern. rowptr[nb+1],
  // colind[nnzb] (sorted, diagonal present), vals[nnzb*9] row-major blocks.
  SolverStatus update_matrix(int nb, const int *rowptr, const int *colind, const double *vals) {
    if (!ok_) return SolverStatus::UnknownError;
    const int nnzb = nb >= 0 && rowptr ? rowptr[nb] : -1;
    const bool same = nb == nb_ && nnzb == (int)colind_.size() &&
                      std::equal(rowptr, rowptr + nb + 1, rowptr_.begin()) &&
                      std::equal(colind, colind + nnzb, colind_.begin());
    if (!same) {
      factored_ = false;
      nb_ = -1;
      if (gbilu_analyze(h_, nb, rowptr, colind) != GBILU_OK) {
        err_ = gbilu_last_error(h_);
        return SolverStatus::AnalysisFailed;
      }
      rowptr_.assign(rowptr, rowptr + nb + 1);
      colind_.assign(colind, colind + nnzb);
      nb_ = nb;
      ++analyses_;
      x_.assign(3 * (size_t)nb, 0.0);
    }
    if (gbilu_factor(h_, vals) != GBILU_OK) {
      factored_ = false;
      err_ = gbilu_last_error(h_);
      return SolverStatus::CreatePreconditionerFailed;
    }
    factored_ = true;
    ++factorizations_;
    return SolverStatus::Success;
  }

  // Solves with the last matrix from x0 = 0; b[3*nb] in the caller's numbering.
  SolverStatus solve(const double *b, SolveResult &res) {
    res = SolveResult();
    if (!ok_ || !factored_) {
      if (ok_) err_ = "solve before update_matrix";
      return SolverStatus::UnknownError;
    }
    std::fill(x_.begin(), x_.end(), 0.0);
    gbilu_result r;
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = gbilu_solve(h_, b, x_.data(), tol_, maxit_, &r);
    res.elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc != GBILU_OK) {
      err_ = gbilu_last_error(h_);
      res.status = rc;
      return SolverStatus::UnknownError;
    }
    res.status = r.status;
    res.half_iters = r.half_iters;
    res.iterations = r.half_iters < 0 ? 0 : (r.half_iters + 1) / 2;
    res.reduction = r.true_relres > 0.0 ? r.true_relres : r.relres;
    res.converged = r.status == GBILU_OK || r.status == GBILU_ALREADY_CONVERGED;
    if (r.status == GBILU_BREAKDOWN || r.status == GBILU_NONFINITE || r.status == GBILU_TIMEOUT)
      return SolverStatus::UnknownError;
    return SolverStatus::Success;
  }

  SolverStatus solve_system(int nb, const int *rowptr, const int *colind, const double *vals,
                            const double *b, SolveResult &res) {
    const SolverStatus st = update_matrix(nb, rowptr, colind, vals);
    if (st != SolverStatus::Success) {
      res = SolveResult();
      return st;
    }
    return solve(b, res);
  }

  // The last solution, x[3*nb] in the caller's numbering.
  void get_result(double *x) const { std::copy(x_.begin(), x_.end(), x); }

  int analyses() const { return analyses_; }
  int factorizations() const { return factorizations_; }
  const std::string &last_error() const { return err_; }
  void *handle() const { return h_; }

 private:
  void *h_ = nullptr;
  bool ok_ = false, factored_ = false;
  double tol_;
  int maxit_;
  int nb_ = -1;
  std::vector<int> rowptr_, colind_;
  std::vector<double> x_;
  int analyses_ = 0, factorizations_ = 0;
  std::string err_;
};

}  // namespace gbilu
