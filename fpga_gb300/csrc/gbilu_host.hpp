// Host-side analysis for the GB300 ILU0-BiCGSTAB path: greedy block coloring,
// color-ordered permutation, block ILU0 factorization and the sliced device
// layout. Plain C++ (no CUDA): the same code runs in host-only handles.
//
// In the reference these steps happen in the Flow backend before the FPGA
// host library is called; the library only receives their output through
// vectorPointers (linearalgebra/ilu0bicgstab/xilinx/src/sda_app/common/
// fpga_functions_bicgstab.cpp:506-629).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace gbilu {

constexpr int kSliceRows = 32;  // block rows per slice = one warp

// One matrix (A, L, U or a transpose) in the sliced layout shared by all
// matrices of a handle. Slice s covers device rows slice_row0[s] ..
// slice_row0[s] + slice_len[s] - 1 of one color; row lane l of slice s keeps
// its k-th block in slot off[s] + k: column col[slot*32 + l] (a device row;
// -1 = padding, always after the row's last block) and value entry e at
// val[(slot*9 + e)*32 + l] in FP64 (FP32 copies: entries 0-3 and 4-7 as 4
// consecutive floats per lane, entry 8 one float per lane, within the same
// 288 values of the slot). Blocks of a row are in ascending column order of
// the permuted numbering.
struct SlicedMatrix {
  std::vector<int> off;   // [S+1]
  std::vector<int> col;   // [slots*32]
  std::vector<int> vsrc;  // [slots*32] source block in the value array, -1 pad
  bool transpose_blocks = false;  // fill with the transposed 3x3 block
  long long slots() const { return off.empty() ? 0 : off.back(); }
};

struct Analysis {
  int nb = 0, nnzb = 0, ncolors = 0;
  std::vector<int> rowptr, colind;        // input pattern
  std::vector<int> color;                 // [nb] color of input row
  std::vector<int> perm, iperm;           // perm[new] = old
  std::vector<int> color_ptr;             // [C+1] new-index range per color
  std::vector<int> split;                 // [C] leading rows of a color with a
                                          // higher-colored neighbour
  std::vector<int> prowptr, pcolind;      // permuted pattern, sorted columns
  std::vector<int> psrc;                  // permuted block -> input block
  std::vector<int> pdiag;                 // position of the diagonal block
  // Device numbering: inside each run of a color's split rows and of its
  // other rows, the rows by descending block count (stable), so that the 32
  // rows of a slice have nearly equal widths and a slice carries almost no
  // padding slots (a padded slot still costs the warp its FMA
  // instructions). dperm[device row] = permuted row; idperm is its inverse.
  // Only the sliced layouts and the device vectors use this numbering: the
  // factorization, the factors and every row's block order stay those of
  // the permuted numbering, so each row's arithmetic is unchanged.
  std::vector<int> dperm, idperm;
  int nnzb_l = 0, nnzb_u = 0;
  // slices
  int S = 0;
  std::vector<int> slice_color_ptr;       // [C+1]
  std::vector<int> slice_row0, slice_len; // [S]
  SlicedMatrix A, L, U;                   // forward operators
  SlicedMatrix At, Ut, Lt;                // transposed operators (adjoint)
};

// Greedy first-fit coloring in natural row order; returns the color count.
int color_greedy(int nb, const int *rowptr, const int *colind, int *color);

// Greedy first-fit coloring in an order that follows the grid's two-color
// parity (the default): blocks on a 4-cycle of the block graph are grid
// faces; the parity of the breadth-first distance over them from the
// lowest-numbered row of each connected part two-colors the grid; of each
// block whose ends have equal parity (a fault connection), one end is
// moved; rows are then colored first-fit, parity-0 rows first, then
// parity-1 rows, then the moved rows, each in natural order. On a
// structured grid with fault connections this gives two large colors and
// one small one (the moved rows), where natural order cascades into more
// and larger small colors. Returns the color count.
int color_parity_greedy(int nb, const int *rowptr, const int *colind, int *color);

// Validates the pattern (sorted unique columns, diagonal present, indices in
// range, structurally symmetric); returns an empty string when it is fine.
std::string check_pattern(int nb, const int *rowptr, const int *colind);

// Builds everything above from an input pattern. Returns "" or an error.
// coloring: 0 color_parity_greedy (default), 1 color_greedy; colors: a
// coloring computed elsewhere (color_parity_device), or null. *color_ms gets
// the time of the host coloring when it ran.
std::string analyze(int nb, const int *rowptr, const int *colind, Analysis &an,
                    bool with_transposes, int coloring = 0, const int *colors = nullptr,
                    double *color_ms = nullptr);

// color_parity_greedy on the GPU (gbilu_color.cu): the same colors; *ms
// gets its device time (uploads, kernels, download).
std::string color_parity_device(int nb, const int *rowptr, const int *colind, int device,
                                int *color, int *ncolors, double *ms);

// Block ILU(0) (IKJ) of the permuted matrix. pvals (nnzb*9, permuted order)
// is overwritten with L (col < row) and U (col >= row); dinv[nb*9] gets the
// inverses of U's diagonal blocks. Returns -1 or the first singular row.
int bilu0(const Analysis &an, double *pvals, double *dinv);

// Gathers input-order values into the permuted order.
void permute_values(const Analysis &an, const double *vals, double *pvals);

// Fills an FP64 sliced value array (slots*9*32 entries, the FP64 layout
// [(slot*9 + e)*32 + l]) from a value source array (9 doubles per block);
// padding entries become 0. The FP32 copies on the device use the FP32
// layout of the kernels (two 16-byte groups and one float per lane and
// slot), converted from this one.
template <typename V>
void fill_sliced(const SlicedMatrix &m, const double *src, V *out);

// Sliced copy of per-row 3x3 blocks (nb*9 doubles in permuted row order),
// optionally transposed, laid out [(slice*9 + e)*32 + lane] by device row
// (FP64 layout, as fill_sliced).
template <typename V>
void fill_sliced_diag(const Analysis &an, const double *dinv, bool transpose,
                      V *out);

}  // namespace gbilu
