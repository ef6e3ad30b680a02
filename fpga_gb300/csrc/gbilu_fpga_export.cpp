// Export of an analyzed and factored system as the input arrays of the
// OPM/FPGA Alveo kernel: the backend's vectorPointers that
// fpga_copy_host_datamem packs into the kernel's buffers
// (linearalgebra/ilu0bicgstab/xilinx/src/sda_app/common/
// fpga_functions_bicgstab.cpp:528-545 for the sizes, :606-629 for the
// arrays). The backend code that produces them in the reference setup lives
// in opm-simulators and is not part of the reference; this restates the
// format from the kernel's RTL (linearalgebra/ilu0bicgstab/xilinx/src/rtl/
// bicgstab_solver_2r-3r3w/ and alveo_u280/rtl/pkg/constants.vhd):
//
//  - the kernel works on scalar rows (3 per block row) in the color order;
//    every color is cut into parts ("colors" of the kernel) that fit its
//    limits: at most 2048 rows (ROW_INDEX_WIDTH 11), 8192 entries of the
//    part's vector copy (COL_INDEX_WIDTH 13), 32768 values
//    (MAT_PART_ADDR_WIDTH 15), at most 256 parts (MAX_COLORS_DEPTH 8),
//    163840 unknowns (VECTOR_SIZE_ELEM) and 2^21 values in all
//    (MATRIX_ADDR_WIDTH 21) (constants.vhd:76-105);
//  - per part 4 words {row, arow, col, val} (rw_pkg.vhd:79-84): its rows,
//    the rows it writes (the RTL reads arow, col and val: ext_read_unit.vhd
//    :98-152, int_read_unit.vhd:281-299), the entries of its vector copy
//    and its values;
//  - the vector copy of a part (P indices, global scalar indices) lists the
//    columns its values read, ascending; in the L and U matrices the part's
//    own rows follow at the end, where the ILU0 unit's results go
//    (int_read_unit.vhd:281-284: the results start at col - arow);
//  - the values of a part run row by row; the column index of a value (16
//    bits) addresses the vector copy; its new-row offset (8 bits) is the
//    number of rows the value moves on from the previous value's row, the
//    row before the first being -1 (NR2offset.vhd:32-42: a value starts a
//    new row iff its offset is not zero, and the offsets of a cycle add
//    up); a gap of more than 255 rows is bridged by zero values;
//  - each part's values are padded to a multiple of 8, its column indices
//    to 32, its new-row offsets to 64 and its vector copy to 16 entries
//    (the line reads of ext_read_unit.vhd:104,135,141), with zeros;
//  - the L and A parts are listed in color order, rows ascending; the U
//    sweep runs backwards (sparstition.vhd:751-756, int_read_unit.vhd:
//    296-299, ilu0.vhd:375-379: rows stream in reverse), so the U parts are
//    listed last part first with their rows descending;
//  - the block diagonal holds, per scalar row, the three values of that row
//    of the inverted diagonal block and one zero (the "4 values per element"
//    of ilu0.vhd:360-362), in the U sweep's order (the kernel reads it in
//    U_bs, ext_read_unit.vhd:111-121), each part padded to 8 doubles.
//
// The color-sizes arrays carry an 8-word header that fpga_copy_host_datamem
// skips (fpga_functions_bicgstab.cpp:608-610); this writes {parts, rows,
// values, vector-copy entries, 0, 0, 0, 0} there.
#include "gbilu_fpga_export.hpp"

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace gbilu {
namespace {

constexpr int kMaxPartRows = 2048;
constexpr int kMaxPartCols = 8192;
constexpr int kMaxPartVals = 32768;
constexpr int kMaxParts = 256;
constexpr long long kMaxVector = 163840;
constexpr long long kMaxValues = 1LL << 21;
constexpr int kMaxNR = 255;

inline long long up(long long v, long long m) { return (v + m - 1) / m * m; }

// The scalar rows of block rows [b0, b1) of the permuted matrix, one sweep:
// which = 0 A (all blocks), 1 L (columns before the row), 2 U (after).
struct Part {
  int b0, b1;   // block rows
};

struct MatOut {
  std::vector<unsigned int> sizes;   // 8-word header + 4 per part
  std::vector<unsigned int> pidx;
  std::vector<double> vals;
  std::vector<unsigned short> cols;
  std::vector<unsigned char> nrs;
  int parts = 0;
};

bool in_sweep(int which, int i, int j) { return which == 0 || (which == 1 ? j < i : j > i); }

// Column set of a part of one matrix (sorted global scalar columns it
// reads), plus its own rows for L and U.
void part_columns(const Analysis &an, int which, const Part &p, std::vector<int> &cols) {
  cols.clear();
  for (int i = p.b0; i < p.b1; ++i)
    for (int k = an.prowptr[i]; k < an.prowptr[i + 1]; ++k) {
      const int j = an.pcolind[k];
      if (!in_sweep(which, i, j)) continue;
      for (int c = 0; c < 3; ++c) cols.push_back(3 * j + c);
    }
  std::sort(cols.begin(), cols.end());
  cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
}

long long part_values(const Analysis &an, int which, const Part &p) {
  long long v = 0;
  for (int i = p.b0; i < p.b1; ++i)
    for (int k = an.prowptr[i]; k < an.prowptr[i + 1]; ++k)
      if (in_sweep(which, i, an.pcolind[k])) v += 9;
  return v;
}

// Whether block rows [b0, b1) fit one part in all three matrices.
bool fits(const Analysis &an, const Part &p, std::vector<int> &tmp) {
  const int rows = 3 * (p.b1 - p.b0);
  if (rows > kMaxPartRows) return false;
  for (int which = 0; which < 3; ++which) {
    part_columns(an, which, p, tmp);
    const long long cols = (long long)tmp.size() + (which ? rows : 0);
    if (cols > kMaxPartCols) return false;
    // values plus the zero values that bridge long gaps (at most one per
    // 255 rows)
    if (part_values(an, which, p) + rows / kMaxNR + 1 > kMaxPartVals) return false;
  }
  return true;
}

// Emits one part of one matrix. rev: rows descending (U).
void emit(const Analysis &an, int which, const Part &p, bool rev, const double *vals,
          MatOut &m) {
  std::vector<int> cols;
  part_columns(an, which, p, cols);
  const int arow = 3 * (p.b1 - p.b0);
  std::vector<unsigned int> pidx(cols.begin(), cols.end());
  if (which)   // own rows at the end of the vector copy
    for (int r = 0; r < arow; ++r) pidx.push_back((unsigned int)(3 * p.b0 + r));
  const size_t v0 = m.vals.size();
  int prev = -1;   // stream row of the previous value
  for (int t = 0; t < arow; ++t) {
    const int R = rev ? 3 * p.b1 - 1 - t : 3 * p.b0 + t;   // scalar row
    const int i = R / 3, r = R % 3;
    bool first = true;
    for (int k = an.prowptr[i]; k < an.prowptr[i + 1]; ++k) {
      const int j = an.pcolind[k];
      if (!in_sweep(which, i, j)) continue;
      for (int c = 0; c < 3; ++c) {
        int nr = 0;
        if (first) {
          int gap = t - prev;
          while (gap > kMaxNR) {   // zero values bridge a long run of empty rows
            m.vals.push_back(0.0);
            m.cols.push_back(0);
            m.nrs.push_back((unsigned char)kMaxNR);
            gap -= kMaxNR;
          }
          nr = gap;
          prev = t;
          first = false;
        }
        const int col = (int)(std::lower_bound(cols.begin(), cols.end(), 3 * j + c) - cols.begin());
        m.vals.push_back(vals[(size_t)k * 9 + r * 3 + c]);
        m.cols.push_back((unsigned short)col);
        m.nrs.push_back((unsigned char)nr);
      }
    }
  }
  const long long nval = (long long)(m.vals.size() - v0);
  // per-part padding of the line reads; the column indices and offsets of
  // the value padding stay zero (the values add nothing)
  const size_t c0 = m.cols.size() - (size_t)nval, n0 = m.nrs.size() - (size_t)nval;
  m.vals.resize(v0 + (size_t)up(nval, 8), 0.0);
  m.cols.resize(c0 + (size_t)up(nval, 32), 0);
  m.nrs.resize(n0 + (size_t)up(nval, 64), 0);
  const unsigned int colsz = (unsigned int)pidx.size();
  pidx.resize((size_t)up((long long)pidx.size(), 16), 0u);
  m.pidx.insert(m.pidx.end(), pidx.begin(), pidx.end());
  for (unsigned int w : {(unsigned int)arow, (unsigned int)arow, colsz, (unsigned int)nval})
    m.sizes.push_back(w);
  ++m.parts;
}

}  // namespace

std::string fpga_export(const Analysis &an, const double *pvals, const double *lu,
                        const double *dinv, FpgaExport &out) {
  out = FpgaExport();
  const long long n = 3LL * an.nb;
  if (n > kMaxVector)
    return "the system has " + std::to_string(n) + " unknowns; the kernel's vector holds " +
           std::to_string(kMaxVector) + " (VECTOR_SIZE_ELEM)";
  // parts: each color cut greedily, whole block rows, all three matrices
  // within the limits
  std::vector<Part> parts;
  std::vector<int> tmp;
  for (int c = 0; c < an.ncolors; ++c) {
    int b = an.color_ptr[c];
    const int e = an.color_ptr[c + 1];
    while (b < e) {
      int lo = b + 1, hi = std::min(e, b + kMaxPartRows / 3);
      if (!fits(an, Part{b, lo}, tmp))
        return "block row " + std::to_string(b) + " alone exceeds a part's limits";
      while (lo < hi) {   // the largest end that still fits (fits is monotone)
        const int mid = (lo + hi + 1) / 2;
        if (fits(an, Part{b, mid}, tmp)) lo = mid; else hi = mid - 1;
      }
      parts.push_back(Part{b, lo});
      b = lo;
    }
  }
  if ((int)parts.size() > kMaxParts)
    return std::to_string(parts.size()) + " parts; the kernel takes " + std::to_string(kMaxParts) +
           " colors (MAX_COLORS_DEPTH)";
  MatOut mats[3];
  for (MatOut &m : mats) m.sizes.assign(8, 0u);
  for (const Part &p : parts) {
    emit(an, 0, p, false, pvals, mats[0]);
    emit(an, 1, p, false, lu, mats[1]);
  }
  for (size_t q = parts.size(); q-- > 0;) emit(an, 2, parts[q], true, lu, mats[2]);
  // block diagonal in the U sweep's order
  for (size_t q = parts.size(); q-- > 0;) {
    const Part &p = parts[q];
    const size_t d0 = out.blkdiag.size();
    for (int i = p.b1 - 1; i >= p.b0; --i)
      for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) out.blkdiag.push_back(dinv[(size_t)i * 9 + r * 3 + c]);
        out.blkdiag.push_back(0.0);
      }
    out.blkdiag.resize(d0 + (size_t)up((long long)(out.blkdiag.size() - d0), 8), 0.0);
  }
  for (int m = 0; m < 3; ++m) {
    MatOut &M = mats[m];
    if ((long long)M.vals.size() > kMaxValues)
      return "the " + std::string(m == 0 ? "A" : m == 1 ? "L" : "U") + " matrix has " +
             std::to_string(M.vals.size()) + " values; the kernel takes " +
             std::to_string(kMaxValues) + " (MATRIX_ADDR_WIDTH)";
    M.sizes[0] = (unsigned int)M.parts;
    M.sizes[1] = (unsigned int)n;
    M.sizes[2] = (unsigned int)M.vals.size();
    M.sizes[3] = (unsigned int)M.pidx.size();
    // vectorSizes (fpga_functions_bicgstab.cpp:528-545): rows, values (the
    // column-index array), colors, vector-copy entries, new-row offsets,
    // block diagonal
    int *vs = out.vector_sizes + 6 * m;
    vs[0] = (int)n;
    vs[1] = (int)M.cols.size();
    vs[2] = M.parts;
    vs[3] = (int)M.pidx.size();
    vs[4] = (int)M.nrs.size();
    vs[5] = (int)out.blkdiag.size();
    out.nnz_sizes[m] = (int)M.vals.size();
    out.sizes[m] = std::move(M.sizes);
    out.pidx[m] = std::move(M.pidx);
    out.vals[m] = std::move(M.vals);
    out.cols[m] = std::move(M.cols);
    out.nrs[m] = std::move(M.nrs);
  }
  return "";
}

}  // namespace gbilu
