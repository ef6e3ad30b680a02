// Export of an analyzed and factored system in the Alveo kernel's input
// format (see gbilu_fpga_export.cpp). Plain C++.
#pragma once

#include <string>
#include <vector>

#include "gbilu_host.hpp"

namespace gbilu {

struct FpgaExport {
  int vector_sizes[18] = {};   // rows, values, colors, vector copy, new-row, block diag; A, L, U
  int nnz_sizes[3] = {};       // value counts of A, L, U (with padding)
  std::vector<unsigned int> sizes[3];      // 8-word header + {row, arow, col, val} per part
  std::vector<unsigned int> pidx[3];       // vector copies (global scalar indices)
  std::vector<double> vals[3];
  std::vector<unsigned short> cols[3];
  std::vector<unsigned char> nrs[3];
  std::vector<double> blkdiag;             // 4 per scalar row, U sweep order
};

// pvals: A in the permuted block order, lu: its ILU0 factors there, dinv:
// the inverted diagonal blocks. Returns "" or the limit that was exceeded.
std::string fpga_export(const Analysis &an, const double *pvals, const double *lu,
                        const double *dinv, FpgaExport &out);

}  // namespace gbilu
