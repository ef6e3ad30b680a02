// Test driver of include/gbilu_bridge.hpp: plays the simulator side of the
// bridge (two Newton steps on one pattern, then a new pattern) and writes
// what the bridge returned.
//
//   bridge_driver <in> <out> <device>
//
// in:  int32 nb, nnzb, precision; rowptr[nb+1], colind[nnzb] (int32);
//      vals[9 nnzb], b[3 nb] (float64); float64 tol; int32 maxit
// out: int32 st1, st2, st3, analyses_after_2, factorizations_after_2,
//      analyses_after_3; per solve (1, 2): int32 iterations, half_iters,
//      converged, status and float64 reduction; then x1[3 nb], x2[3 nb]
//
// Step 2 uses the values scaled by 1.5 (same pattern: no new analysis);
// step 3 drops the off-diagonal blocks of the last block row and column (new
// pattern). With
// device = -1 (host-only handle) only update_matrix runs.
#include "gbilu_bridge.hpp"

#include <cstdio>
#include <cstdlib>
#include <vector>

template <typename T> static bool rd(FILE *f, T *p, size_t n) { return fread(p, sizeof(T), n, f) == n; }
template <typename T> static void wr(FILE *f, const T *p, size_t n) { fwrite(p, sizeof(T), n, f); }

int main(int argc, char **argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: %s <in> <out> <device>\n", argv[0]);
    return 2;
  }
  FILE *in = fopen(argv[1], "rb");
  if (!in) return 2;
  int hdr[3];
  if (!rd(in, hdr, 3)) return 2;
  const int nb = hdr[0], nnzb = hdr[1], precision = hdr[2];
  std::vector<int> rowptr(nb + 1), colind(nnzb);
  std::vector<double> vals(9 * (size_t)nnzb), b(3 * (size_t)nb);
  double tol;
  int maxit;
  if (!rd(in, rowptr.data(), nb + 1) || !rd(in, colind.data(), nnzb) || !rd(in, vals.data(), vals.size()) ||
      !rd(in, b.data(), b.size()) || !rd(in, &tol, 1) || !rd(in, &maxit, 1))
    return 2;
  fclose(in);

  gbilu_options opt;
  gbilu_default_options(&opt);
  opt.device = atoi(argv[3]);
  opt.precision = precision;
  // as a simulator backend would run it: refactorization and coloring on
  // the GPU (no effect on a host-only handle)
  opt.factor_on_device = 1;
  opt.color_on_device = 1;
  gbilu::BsrBridge bridge(tol, maxit, &opt);
  const bool dev = opt.device >= 0;

  gbilu::SolveResult r1, r2;
  std::vector<double> x1(b.size()), x2(b.size());
  gbilu::SolverStatus s1, s2, s3;
  if (dev) {
    s1 = bridge.solve_system(nb, rowptr.data(), colind.data(), vals.data(), b.data(), r1);
    bridge.get_result(x1.data());
  } else {
    s1 = bridge.update_matrix(nb, rowptr.data(), colind.data(), vals.data());
  }
  std::vector<double> v2(vals);
  for (double &v : v2) v *= 1.5;
  if (dev) {
    s2 = bridge.solve_system(nb, rowptr.data(), colind.data(), v2.data(), b.data(), r2);
    bridge.get_result(x2.data());
  } else {
    s2 = bridge.update_matrix(nb, rowptr.data(), colind.data(), v2.data());
  }
  const int an2 = bridge.analyses(), fa2 = bridge.factorizations();
  // new pattern: the last block row and column lose their off-diagonal
  // blocks (the pattern stays symmetric)
  std::vector<int> rp3(rowptr), ci3;
  std::vector<double> v3;
  for (int i = 0; i < nb; ++i) {
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      if ((i == nb - 1 || colind[k] == nb - 1) && colind[k] != i) continue;
      ci3.push_back(colind[k]);
      v3.insert(v3.end(), vals.begin() + 9 * (size_t)k, vals.begin() + 9 * (size_t)k + 9);
    }
    rp3[i + 1] = (int)ci3.size();
  }
  s3 = bridge.update_matrix(nb, rp3.data(), ci3.data(), v3.data());
  if (s1 != gbilu::SolverStatus::Success || s2 != gbilu::SolverStatus::Success ||
      s3 != gbilu::SolverStatus::Success)
    fprintf(stderr, "bridge: %s\n", bridge.last_error().c_str());

  FILE *out = fopen(argv[2], "wb");
  if (!out) return 2;
  const int head[6] = {(int)s1, (int)s2, (int)s3, an2, fa2, bridge.analyses()};
  wr(out, head, 6);
  for (const auto *p : {&r1, &r2}) {
    const int iv[4] = {p->iterations, p->half_iters, p->converged ? 1 : 0, p->status};
    wr(out, iv, 4);
    wr(out, &p->reduction, 1);
  }
  wr(out, x1.data(), x1.size());
  wr(out, x2.data(), x2.size());
  fclose(out);
  return 0;
}
