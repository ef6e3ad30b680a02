// Checker-side C entry points over the reference's own host library
// (src/sda_app/common/fpga_functions_bicgstab.cpp, bicgstab_utils.cpp,
// bda_utils.cpp, compiled unmodified from the reference tree by
// oracle/ref/Makefile). TEST INFRASTRUCTURE ONLY: the product never links it.
#include <CL/opencl.h>
#include <cstdlib>
#include <cstring>

#include "bicgstab_utils.hpp"
#include "fpga_functions_bicgstab.hpp"

namespace {
struct Arrays {
  long unsigned int *setup = nullptr;
  double **nnz = nullptr, **lnnz = nullptr, **unnz = nullptr;
  short unsigned int *ci = nullptr, *lci = nullptr, *uci = nullptr;
  unsigned char *nr = nullptr, *lnr = nullptr, *unr = nullptr;
  unsigned int *pi = nullptr, *lpi = nullptr, *upi = nullptr;
  unsigned int *cs = nullptr, *lcs = nullptr, *ucs = nullptr;
  double *blkd = nullptr, *x1 = nullptr, *r1 = nullptr, *x2 = nullptr, *r2 = nullptr;
  double *lres = nullptr, *ures = nullptr;
  unsigned int *total = nullptr;
  unsigned char *buf[RW_BUF] = {};
  unsigned int result_offsets[6] = {};
};

int setup(Arrays &a, int level_scheduling, unsigned config_bits, const int *sizes,
          const int *nnz_sizes, unsigned dbg_bytes) {
  int s[18];
  memcpy(s, sizes, sizeof s);
  int nz[1] = {nnz_sizes[0]}, lnz[1] = {nnz_sizes[1]}, unz[1] = {nnz_sizes[2]};
  return fpga_setup_host_datamem(level_scheduling != 0, config_bits, s, &a.setup, &a.nnz, nz,
                                 &a.ci, &a.nr, &a.pi, &a.cs, &a.lnnz, lnz, &a.lci, &a.lnr,
                                 &a.lpi, &a.lcs, &a.unnz, unz, &a.uci, &a.unr, &a.upi, &a.ucs,
                                 &a.blkd, &a.x1, &a.r1, &a.x2, &a.r2, &a.lres, &a.ures,
                                 &a.total, a.buf, a.result_offsets, 1, true, dbg_bytes);
}

void release(Arrays &a) {
  for (int b = 0; b < RW_BUF; ++b) free(a.buf[b]);
  free(a.total);
  free(a.nnz);
  free(a.lnnz);
  free(a.unnz);
}

long long off(const Arrays &a, int bank, const void *p) {
  return (long long)((const unsigned char *)p - a.buf[bank]);
}
}  // namespace

// Byte offsets of the 22 arrays inside their banks, in the order
// setup, nnz, L nnz, U nnz, color sizes, L/U color sizes, block diag (bank 0);
// P idx, L/U P idx, col idx, L/U col idx, NRs, L/U NRs (bank 1);
// X2, R1 (bank 2); X1, R2 (bank 3); Lres, Ures (bank 4).
extern "C" int ref_setup_layout(int level_scheduling, unsigned config_bits, const int *sizes,
                                const int *nnz_sizes, unsigned dbg_bytes,
                                unsigned long long *setup_out, unsigned *total_out,
                                long long *offsets_out, unsigned *result_offsets_out) {
  Arrays a;
  int rc = setup(a, level_scheduling, config_bits, sizes, nnz_sizes, dbg_bytes);
  if (rc) return rc;
  memcpy(setup_out, a.setup, 40 * sizeof(unsigned long long));
  memcpy(total_out, a.total, RW_BUF * sizeof(unsigned));
  memcpy(result_offsets_out, a.result_offsets, sizeof a.result_offsets);
  const void *p[22] = {a.setup, a.nnz[0], a.lnnz[0], a.unnz[0], a.cs, a.lcs, a.ucs, a.blkd,
                       a.pi, a.lpi, a.upi, a.ci, a.lci, a.uci, a.nr, a.lnr, a.unr,
                       a.x2, a.r1, a.x1, a.r2, a.lres};
  const int bank[22] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 3, 3, 4};
  for (int i = 0; i < 22; ++i) offsets_out[i] = off(a, bank[i], p[i]);
  offsets_out[22] = off(a, 4, a.ures);
  release(a);
  return 0;
}

// Packs the vectorPointers arrays into the 5 data buffers exactly as
// fpga_copy_host_datamem does (reset, result sentinels, copies); out[b]
// receives total[b] bytes of bank b.
extern "C" int ref_pack(unsigned config_bits, const int *sizes, const int *nnz_sizes,
                        void **vector_pointers, const int *vector_sizes, int fill_results,
                        unsigned char **out) {
  Arrays a;
  int rc = setup(a, 0, config_bits, sizes, nnz_sizes, 64 * 8);
  if (rc) return rc;
  int nz[1] = {nnz_sizes[0]}, lnz[1] = {nnz_sizes[1]}, unz[1] = {nnz_sizes[2]};
  int vs[18];
  memcpy(vs, vector_sizes, sizeof vs);
  rc = fpga_copy_host_datamem(vector_pointers, vs, a.setup, a.nnz, nz, a.ci, a.nr, a.pi, a.cs,
                              a.lnnz, lnz, a.lci, a.lnr, a.lpi, a.lcs, a.unnz, unz, a.uci,
                              a.unr, a.upi, a.ucs, a.blkd, a.x1, a.r1, a.x2, a.r2,
                              false, a.lres, a.ures, a.total, a.buf, 1, true,
                              fill_results != 0, 0, 0);
  if (!rc)
    for (int b = 0; b < RW_BUF; ++b) memcpy(out[b], a.buf[b], a.total[b]);
  release(a);
  return rc;
}

// decode_debuginfo_bicgstab (bicgstab_utils.cpp:90) on a debug buffer.
extern "C" int ref_decode(unsigned long long *dbg, unsigned lines, unsigned *cycles,
                          unsigned *iters, double *norms, unsigned char *last_idx, int *flags) {
  bool f[6] = {};
  int rc = decode_debuginfo_bicgstab(true, false, (unsigned long int *)dbg, lines, 8, 0, cycles,
                                     iters, norms, last_idx, &f[0], &f[1], &f[2], &f[3], &f[4],
                                     &f[5]);
  for (int i = 0; i < 6; ++i) flags[i] = f[i];
  return rc;
}
