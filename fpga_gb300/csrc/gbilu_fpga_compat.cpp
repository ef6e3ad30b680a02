// Interchange with the Alveo kernel's host-side formats: the five-bank
// buffer layout with its 5-cacheline setup array, the packing of the
// backend's vectorPointers into those banks, and the debug/status lines the
// reference's decoder reads. Plain C++ (no CUDA); see include/gbilu.h.
#include "gbilu.h"

#include <cstdint>
#include <cstring>
#include <initializer_list>

namespace {

constexpr int kLine = 64;          // cacheline bytes (bicgstab_solver_config.hpp:53)
constexpr int kSetupLines = 5;     // setup cachelines (bicgstab_solver_config.hpp:38)

inline long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

// Array order of gbilu_fpga_layout's offsets (bank in brackets):
enum {
  SETUP, NNZ, L_NNZ, U_NNZ, CSIZE, L_CSIZE, U_CSIZE, BLKD,  // [0]
  PIDX, L_PIDX, U_PIDX, COLS, L_COLS, U_COLS, NRS, L_NRS, U_NRS,  // [1]
  X2, R1,                                                    // [2]
  X1, R2, P1, P2, RT,                                        // [3]
  T, V, LRES, URES,                                          // [4]
  NARR
};

struct Layout {
  long long off[NARR];
  int bank[NARR];
  long long total[5];
};

// Bank layout (which array goes where, in which order, padded to whole
// cachelines) as the reference's host library lays it out for the 2r_3r3w
// port configuration: fpga_functions_bicgstab.cpp:176-238 (lengths) and
// :246-305 (positions).
Layout layout(const int *ps, const int *nnz) {
  const long long vec = 8 * round_up(ps[0], 8);
  long long len[NARR];
  len[SETUP] = kLine * kSetupLines;
  len[NNZ] = 8 * round_up(nnz[0], 8);
  len[L_NNZ] = 8 * round_up(nnz[1], 8);
  len[U_NNZ] = 8 * round_up(nnz[2], 8);
  len[CSIZE] = 4 * round_up(4LL * ps[2], 16);
  len[L_CSIZE] = 4 * round_up(4LL * ps[8], 16);
  len[U_CSIZE] = 4 * round_up(4LL * ps[14], 16);
  len[BLKD] = 8 * round_up(ps[5], 8);
  len[PIDX] = 4 * round_up(ps[3], 16);
  len[L_PIDX] = 4 * round_up(ps[9], 16);
  len[U_PIDX] = 4 * round_up(ps[15], 16);
  len[COLS] = 2 * round_up(ps[1], 32);
  len[L_COLS] = 2 * round_up(ps[7], 32);
  len[U_COLS] = 2 * round_up(ps[13], 32);
  len[NRS] = round_up(ps[4], 64);
  len[L_NRS] = round_up(ps[10], 64);
  len[U_NRS] = round_up(ps[16], 64);
  for (int a : {X2, R1, X1, R2, P1, P2, RT, T, V, LRES, URES}) len[a] = vec;
  static const int order[5][9] = {
      {SETUP, NNZ, L_NNZ, U_NNZ, CSIZE, L_CSIZE, U_CSIZE, BLKD, -1},
      {PIDX, L_PIDX, U_PIDX, COLS, L_COLS, U_COLS, NRS, L_NRS, U_NRS},
      {X2, R1, -1, -1, -1, -1, -1, -1, -1},
      {X1, R2, P1, P2, RT, -1, -1, -1, -1},
      {T, V, LRES, URES, -1, -1, -1, -1, -1}};
  Layout L;
  for (int b = 0; b < 5; ++b) {
    long long pos = 0;
    for (int i = 0; i < 9 && order[b][i] >= 0; ++i) {
      L.off[order[b][i]] = pos;
      L.bank[order[b][i]] = b;
      pos += len[order[b][i]];
    }
    L.total[b] = pos;
  }
  return L;
}

inline unsigned long long cl(const Layout &L, int a) { return (unsigned long long)(L.off[a] / kLine); }

}  // namespace

extern "C" int gbilu_fpga_layout(unsigned int config_bits, const int *processed_sizes,
                                 const int *nnz_sizes, unsigned int debug_bytes,
                                 unsigned long long *setup, unsigned int *totals,
                                 long long *offsets, unsigned int *result_offsets) {
  if (!processed_sizes || !nnz_sizes || !setup || !totals) return GBILU_BAD_INPUT;
  if (debug_bytes % kLine != 0) return GBILU_BAD_INPUT;   // :182-193
  const int *ps = processed_sizes;
  for (int i = 0; i < 18; ++i)
    if (ps[i] < 0) return GBILU_BAD_INPUT;
  const Layout L = layout(ps, nnz_sizes);
  for (int b = 0; b < 5; ++b) totals[b] = (unsigned int)L.total[b];
  if (offsets) {
    // same order as the arrays of the reference's setup (see the enum)
    static const int pub[23] = {SETUP, NNZ, L_NNZ, U_NNZ, CSIZE, L_CSIZE, U_CSIZE, BLKD,
                                PIDX, L_PIDX, U_PIDX, COLS, L_COLS, U_COLS, NRS, L_NRS, U_NRS,
                                X2, R1, X1, R2, LRES, URES};
    for (int i = 0; i < 23; ++i) offsets[i] = L.off[pub[i]];
  }
  if (result_offsets) {      // X even, R even, X odd, R odd, L res, U res (:274-298)
    result_offsets[0] = (unsigned int)L.off[X2];
    result_offsets[1] = (unsigned int)L.off[R2];
    result_offsets[2] = (unsigned int)L.off[X1];
    result_offsets[3] = (unsigned int)L.off[R1];
    result_offsets[4] = (unsigned int)L.off[LRES];
    result_offsets[5] = (unsigned int)L.off[URES];
  }
  // setup array: 40 words, unused ones hold a filler pattern (:415-477)
  for (int i = 0; i < kSetupLines * 8; ++i) setup[i] = 0xDEADC0DEDEADC0DEULL;
  auto pack2 = [](long long hi, long long lo) {
    return ((unsigned long long)(uint32_t)hi << 32) + (unsigned long long)(uint32_t)lo;
  };
  setup[0] = pack2(ps[1], ps[0]);
  setup[1] = pack2(config_bits, ps[2]);
  setup[2] = cl(L, R1);
  setup[3] = cl(L, R2);
  setup[4] = cl(L, X1);
  setup[5] = cl(L, X2);
  setup[6] = cl(L, P1);
  setup[7] = cl(L, P2);
  setup[8] = pack2(ps[7], ps[6]);
  setup[9] = (unsigned long long)(uint32_t)ps[8];
  setup[10] = cl(L, CSIZE);
  setup[11] = cl(L, PIDX);
  setup[12] = cl(L, NNZ);
  setup[13] = cl(L, COLS);
  setup[14] = cl(L, NRS);
  setup[15] = cl(L, RT);
  setup[16] = pack2(ps[13], ps[12]);
  setup[17] = (unsigned long long)(uint32_t)ps[14];
  setup[18] = cl(L, L_CSIZE);
  setup[19] = cl(L, L_PIDX);
  setup[20] = cl(L, L_NNZ);
  setup[21] = cl(L, L_COLS);
  setup[22] = cl(L, L_NRS);
  setup[23] = cl(L, BLKD);
  setup[24] = cl(L, U_CSIZE);
  setup[25] = cl(L, U_PIDX);
  setup[26] = cl(L, U_NNZ);
  setup[27] = cl(L, U_COLS);
  setup[28] = cl(L, U_NRS);
  setup[29] = cl(L, T);
  setup[30] = cl(L, V);
  return GBILU_OK;
}

extern "C" int gbilu_fpga_pack(unsigned int config_bits, const int *processed_sizes,
                               const int *nnz_sizes, void *const *vector_pointers,
                               const int *vector_sizes, int fill_results,
                               unsigned char *const *banks) {
  if (!processed_sizes || !nnz_sizes || !vector_pointers || !vector_sizes || !banks)
    return GBILU_BAD_INPUT;
  unsigned long long setup[40];
  unsigned int totals[5];
  int rc = gbilu_fpga_layout(config_bits, processed_sizes, nnz_sizes, 64, setup, totals, nullptr,
                             nullptr);
  if (rc) return rc;
  const Layout L = layout(processed_sizes, nnz_sizes);
  const int *vs = vector_sizes;
  // banks start cleared; the setup array (with the actual sizes) leads bank 0
  for (int b = 0; b < 5; ++b) std::memset(banks[b], 0, totals[b]);
  setup[0] = ((unsigned long long)(uint32_t)vs[1] << 32) + (uint32_t)vs[0];
  setup[8] = ((unsigned long long)(uint32_t)vs[7] << 32) + (uint32_t)vs[6];
  setup[16] = ((unsigned long long)(uint32_t)vs[13] << 32) + (uint32_t)vs[12];
  std::memcpy(banks[0], setup, sizeof setup);
  auto put = [&](int arr, const void *src, size_t bytes) {
    std::memcpy(banks[L.bank[arr]] + L.off[arr], src, bytes);
  };
  const int rows = vs[0];
  if (fill_results) {
    // output regions start as 0x9696...96xx | index (fpga_functions_bicgstab.cpp:572-592)
    for (long long d = 0; d < round_up(rows, 8); ++d) {
      unsigned long long v = 0;
      for (int j = 15; j >= 8; --j) v |= (unsigned long long)((j % 2 == 0) ? 0x9 : 0x6) << (4 * j);
      v |= (unsigned long long)d;
      for (int a : {X2, R2}) std::memcpy(banks[L.bank[a]] + L.off[a] + 8 * d, &v, 8);
    }
  }
  // color sizes skip an 8-int header; the other arrays are copied as given
  put(CSIZE, (const int *)vector_pointers[0] + 8, sizeof(int) * 4 * (size_t)vs[2]);
  put(L_CSIZE, (const int *)vector_pointers[6] + 8, sizeof(int) * 4 * (size_t)vs[8]);
  put(U_CSIZE, (const int *)vector_pointers[12] + 8, sizeof(int) * 4 * (size_t)vs[14]);
  put(PIDX, vector_pointers[1], sizeof(int) * (size_t)vs[3]);
  put(L_PIDX, vector_pointers[7], sizeof(int) * (size_t)vs[9]);
  put(U_PIDX, vector_pointers[13], sizeof(int) * (size_t)vs[15]);
  put(NNZ, ((double *const *)vector_pointers[2])[0], sizeof(double) * (size_t)nnz_sizes[0]);
  put(L_NNZ, ((double *const *)vector_pointers[8])[0], sizeof(double) * (size_t)nnz_sizes[1]);
  put(U_NNZ, ((double *const *)vector_pointers[14])[0], sizeof(double) * (size_t)nnz_sizes[2]);
  put(COLS, vector_pointers[3], sizeof(short) * (size_t)vs[1]);
  put(L_COLS, vector_pointers[9], sizeof(short) * (size_t)vs[7]);
  put(U_COLS, vector_pointers[15], sizeof(short) * (size_t)vs[13]);
  put(NRS, vector_pointers[4], (size_t)vs[4]);
  put(L_NRS, vector_pointers[10], (size_t)vs[10]);
  put(U_NRS, vector_pointers[16], (size_t)vs[16]);
  put(R1, vector_pointers[19], sizeof(double) * (size_t)rows);
  std::memset(banks[L.bank[R2]] + L.off[R2], 0, sizeof(double) * (size_t)rows);
  put(X1, vector_pointers[20], sizeof(double) * (size_t)rows);
  std::memset(banks[L.bank[X2]] + L.off[X2], 0, sizeof(double) * (size_t)rows);
  put(BLKD, vector_pointers[18], sizeof(double) * (size_t)vs[5]);
  return GBILU_OK;
}

extern "C" int gbilu_status_lines(const gbilu_result *res, unsigned long long *buf, int lines) {
  if (!res || !buf || lines < 2) return GBILU_BAD_INPUT;
  // unwritten lines hold the 0x5a5a... marker (fpga_functions_bicgstab.cpp:697-719)
  for (int i = 0; i < lines * 8; ++i) buf[i] = 0x5a5a5a5a5a5a5a5aULL;
  // line 0: general status (bicgstab_utils.cpp:114-137): flags in word 0
  // (bit 0 aborted, bit 1 no results), run length in word 1, signature
  // "BDA" in word 7 bits 40..63. The run length is the solve's device time
  // in nanoseconds.
  unsigned long long *l0 = buf;
  for (int i = 0; i < 8; ++i) l0[i] = 0;
  l0[0] = (res->status == GBILU_TIMEOUT ? 1ULL : 0ULL) |
          (res->status == GBILU_ALREADY_CONVERGED ? 2ULL : 0ULL);
  const double ns = res->device_ms * 1e6;
  l0[1] = (unsigned long long)(ns > 4294967295.0 ? 4294967295.0 : (ns < 0 ? 0 : ns));
  l0[7] = 0x414442ULL << 40;
  // line 1: the final kernel-status line (bicgstab_utils.cpp:139-262): no
  // overflow flags, debug-line count 1, the half-iteration counter (16 bits)
  // and the four-norm ring
  unsigned long long *l1 = buf + 8;
  for (int i = 0; i < 8; ++i) l1[i] = 0;
  const unsigned int itr = (unsigned int)res->half_iters & 0xFFFFu;
  l1[3] = (1ULL << 16) | ((unsigned long long)itr << 32);
  for (int i = 0; i < 4; ++i) std::memcpy(&l1[4 + i], &res->norms[i], 8);
  return GBILU_OK;
}
