// Host-side analysis, block ILU0 and sliced layout (see gbilu_host.hpp).
#include "gbilu_host.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>

namespace gbilu {

int color_greedy(int nb, const int *rowptr, const int *colind, int *color) {
  // First-fit greedy in natural order: a row takes the smallest color that no
  // already colored neighbour holds. stamp[c] == i+1 marks color c as taken
  // for row i.
  if (nb <= 0) return 0;
  std::vector<int> stamp(static_cast<size_t>(nb) + 1, 0);
  int ncolors = 0;
  std::fill(color, color + nb, -1);
  for (int i = 0; i < nb; ++i) {
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = colind[k];
      if (j != i && color[j] >= 0) stamp[color[j]] = i + 1;
    }
    int c = 0;
    while (stamp[c] == i + 1) ++c;
    color[i] = c;
    ncolors = std::max(ncolors, c + 1);
  }
  return ncolors;
}

int color_parity_greedy(int nb, const int *rowptr, const int *colind, int *color) {
  if (nb <= 0) return 0;
  // 1. Grid edges: an off-diagonal block (u, v) lies on a 4-cycle u-a-b-v
  //    of the block graph (a != v, b != u). A structured grid's faces all
  //    do; a non-neighbour connection between distant cells (a fault)
  //    almost never does.
  std::vector<char> grid(static_cast<size_t>(rowptr[nb]), 0);
  std::vector<int> mark(nb, -1);
  for (int u = 0; u < nb; ++u) {
    for (int k = rowptr[u]; k < rowptr[u + 1]; ++k) mark[colind[k]] = u;
    for (int k = rowptr[u]; k < rowptr[u + 1]; ++k) {
      const int v = colind[k];
      if (v == u) continue;
      bool found = false;
      // b in N(v) \ {u, v}, then a in N(b) \ {b} with a in N(u) \ {u, v}
      for (int kb = rowptr[v]; kb < rowptr[v + 1] && !found; ++kb) {
        const int b = colind[kb];
        if (b == v || b == u) continue;
        for (int ka = rowptr[b]; ka < rowptr[b + 1]; ++ka) {
          const int a = colind[ka];
          if (a != b && a != u && a != v && mark[a] == u) { found = true; break; }
        }
      }
      grid[k] = found;
    }
  }
  // 2. Distance parity from the lowest-numbered row of each connected part
  //    of the grid-edge graph (breadth-first; distances do not depend on
  //    the visiting order).
  std::vector<int> dist(nb, -1), queue(nb);
  for (int r = 0; r < nb; ++r) {
    if (dist[r] >= 0) continue;
    int head = 0, tail = 0;
    dist[r] = 0;
    queue[tail++] = r;
    while (head < tail) {
      const int u = queue[head++];
      for (int k = rowptr[u]; k < rowptr[u + 1]; ++k) {
        const int v = colind[k];
        if (grid[k] && dist[v] < 0) {
          dist[v] = dist[u] + 1;
          queue[tail++] = v;
        }
      }
    }
  }
  // 3. Every block (u, v), u < v, whose ends have the same parity needs one
  //    end moved off the two parity colors. Blocks in row-major order: an
  //    end already moved covers it; else move v unless v touches a moved
  //    row and u does not (moved rows that touch get a fourth color).
  std::vector<char> moved(nb, 0);
  auto touches_moved = [&](int x) {
    for (int k = rowptr[x]; k < rowptr[x + 1]; ++k)
      if (moved[colind[k]]) return true;
    return false;
  };
  for (int u = 0; u < nb; ++u)
    for (int k = rowptr[u]; k < rowptr[u + 1]; ++k) {
      const int v = colind[k];
      if (v <= u || ((dist[u] ^ dist[v]) & 1)) continue;
      if (moved[u] || moved[v]) continue;
      if (!touches_moved(v)) moved[v] = 1;
      else if (!touches_moved(u)) moved[u] = 1;
      else moved[v] = 1;
    }
  // 4. First-fit greedy visiting rows by class (parity 0, parity 1, moved),
  //    each class in natural order.
  std::vector<int> order;
  order.reserve(nb);
  for (int cls = 0; cls < 3; ++cls)
    for (int i = 0; i < nb; ++i)
      if ((moved[i] ? 2 : (dist[i] & 1)) == cls) order.push_back(i);
  std::vector<int> stamp(static_cast<size_t>(nb) + 1, 0);
  std::fill(color, color + nb, -1);
  int ncolors = 0;
  for (int t = 0; t < nb; ++t) {
    const int i = order[t];
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = colind[k];
      if (j != i && color[j] >= 0) stamp[color[j]] = t + 1;
    }
    int c = 0;
    while (stamp[c] == t + 1) ++c;
    color[i] = c;
    ncolors = std::max(ncolors, c + 1);
  }
  return ncolors;
}

std::string check_pattern(int nb, const int *rowptr, const int *colind) {
  if (nb <= 0) return "nb must be positive";
  // vector entries are indexed with int (3 per block row, 9 per block in
  // per-row scratch)
  if (nb > std::numeric_limits<int>::max() / 9) return "nb too large";
  if (!rowptr || !colind) return "rowptr/colind must not be NULL";
  if (rowptr[0] != 0) return "rowptr[0] must be 0";
  for (int i = 0; i < nb; ++i) {
    if (rowptr[i + 1] < rowptr[i]) return "rowptr must be non-decreasing";
    bool diag = false;
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = colind[k];
      if (j < 0 || j >= nb) return "column index out of range in row " + std::to_string(i);
      if (k > rowptr[i] && colind[k - 1] >= j)
        return "columns must be sorted and unique in row " + std::to_string(i);
      diag |= (j == i);
    }
    if (!diag) return "missing diagonal block in row " + std::to_string(i);
  }
  // Structural symmetry (block (i, j) present iff (j, i) is), as in the
  // simulator's matrices: rows of one color must not be coupled in either
  // direction, and the coloring only sees each row's own columns.
  for (int i = 0; i < nb; ++i)
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = colind[k];
      if (j == i) continue;
      if (!std::binary_search(colind + rowptr[j], colind + rowptr[j + 1], i))
        return "pattern must be structurally symmetric: block (" + std::to_string(i) + ", " +
               std::to_string(j) + ") has no transpose (" + std::to_string(j) + ", " +
               std::to_string(i) + ")";
    }
  return "";
}

namespace {

struct Csr {
  std::vector<int> rowptr, col, src;
};

// Builds the sliced layout of a CSR matrix given in the permuted numbering:
// lane l of slice s holds device row slice_row0[s] + l, i.e. permuted row
// dperm[...], with its blocks in their CSR order and columns renumbered to
// device rows.
void slice_matrix(const Analysis &an, const Csr &m, bool transpose_blocks,
                  SlicedMatrix &out) {
  out.transpose_blocks = transpose_blocks;
  out.off.assign(static_cast<size_t>(an.S) + 1, 0);
  for (int s = 0; s < an.S; ++s) {
    int w = 0;
    for (int l = 0; l < an.slice_len[s]; ++l) {
      const int r = an.dperm[an.slice_row0[s] + l];
      w = std::max(w, m.rowptr[r + 1] - m.rowptr[r]);
    }
    out.off[s + 1] = out.off[s] + w;
  }
  const size_t n = static_cast<size_t>(out.off[an.S]) * kSliceRows;
  out.col.assign(n, -1);
  out.vsrc.assign(n, -1);
  for (int s = 0; s < an.S; ++s) {
    for (int l = 0; l < an.slice_len[s]; ++l) {
      const int r = an.dperm[an.slice_row0[s] + l];
      for (int k = m.rowptr[r]; k < m.rowptr[r + 1]; ++k) {
        const size_t slot = static_cast<size_t>(out.off[s]) + (k - m.rowptr[r]);
        out.col[slot * kSliceRows + l] = an.idperm[m.col[k]];
        out.vsrc[slot * kSliceRows + l] = m.src[k];
      }
    }
  }
}

// Transpose of a CSR pattern selection: entries (i -> j, src) become (j -> i).
Csr transpose_csr(int nb, const Csr &m) {
  Csr t;
  t.rowptr.assign(static_cast<size_t>(nb) + 1, 0);
  for (int c : m.col) t.rowptr[c + 1]++;
  for (int i = 0; i < nb; ++i) t.rowptr[i + 1] += t.rowptr[i];
  t.col.resize(m.col.size());
  t.src.resize(m.col.size());
  std::vector<int> fill(t.rowptr.begin(), t.rowptr.end() - 1);
  for (int i = 0; i < nb; ++i)            // rows ascending -> columns sorted
    for (int k = m.rowptr[i]; k < m.rowptr[i + 1]; ++k) {
      const int p = fill[m.col[k]]++;
      t.col[p] = i;
      t.src[p] = m.src[k];
    }
  return t;
}

}  // namespace

std::string analyze(int nb, const int *rowptr, const int *colind, Analysis &an,
                    bool with_transposes, int coloring, const int *colors, double *color_ms) {
  std::string err = check_pattern(nb, rowptr, colind);
  if (!err.empty()) return err;
  an = Analysis();
  an.nb = nb;
  an.nnzb = rowptr[nb];
  an.rowptr.assign(rowptr, rowptr + nb + 1);
  an.colind.assign(colind, colind + an.nnzb);
  an.color.resize(nb);
  if (colors) {
    std::copy(colors, colors + nb, an.color.begin());
    an.ncolors = 1 + *std::max_element(colors, colors + nb);
  } else {
    const auto t0 = std::chrono::steady_clock::now();
    an.ncolors = coloring == 1 ? color_greedy(nb, rowptr, colind, an.color.data())
                               : color_parity_greedy(nb, rowptr, colind, an.color.data());
    if (color_ms)
      *color_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                      .count();
  }
  const int C = an.ncolors;

  // Color-ordered permutation (counting sort). Inside a color, the rows that
  // share a block with a row of a higher color (either end) come first: the
  // others have empty U and L^T rows, so their value is final right after
  // the first sweep and the second sweep of the color only covers the
  // leading split[c] rows. Rows of one color are never coupled, so this
  // order does not change the ILU0 factors.
  std::vector<char> higher(nb, 0);
  for (int i = 0; i < nb; ++i)
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = colind[k];
      if (an.color[j] > an.color[i]) higher[i] = 1;
      if (an.color[i] > an.color[j]) higher[j] = 1;
    }
  an.color_ptr.assign(C + 1, 0);
  an.split.assign(C, 0);
  for (int i = 0; i < nb; ++i) {
    an.color_ptr[an.color[i] + 1]++;
    if (higher[i]) an.split[an.color[i]]++;
  }
  for (int c = 0; c < C; ++c) an.color_ptr[c + 1] += an.color_ptr[c];
  an.perm.resize(nb);
  an.iperm.resize(nb);
  {
    std::vector<int> first(C), second(C);
    for (int c = 0; c < C; ++c) {
      first[c] = an.color_ptr[c];
      second[c] = an.color_ptr[c] + an.split[c];
    }
    for (int i = 0; i < nb; ++i)
      an.perm[higher[i] ? first[an.color[i]]++ : second[an.color[i]]++] = i;
  }
  for (int i = 0; i < nb; ++i) an.iperm[an.perm[i]] = i;

  // permuted pattern with sorted columns
  an.prowptr.assign(static_cast<size_t>(nb) + 1, 0);
  for (int i = 0; i < nb; ++i)
    an.prowptr[i + 1] = an.prowptr[i] + (rowptr[an.perm[i] + 1] - rowptr[an.perm[i]]);
  an.pcolind.resize(an.nnzb);
  an.psrc.resize(an.nnzb);
  an.pdiag.resize(nb);
  std::vector<std::pair<int, int>> tmp;
  for (int i = 0; i < nb; ++i) {
    const int o = an.perm[i];
    tmp.clear();
    for (int k = rowptr[o]; k < rowptr[o + 1]; ++k) tmp.emplace_back(an.iperm[colind[k]], k);
    std::sort(tmp.begin(), tmp.end());
    for (size_t t = 0; t < tmp.size(); ++t) {
      const int p = an.prowptr[i] + static_cast<int>(t);
      an.pcolind[p] = tmp[t].first;
      an.psrc[p] = tmp[t].second;
      if (tmp[t].first == i) an.pdiag[i] = p;
    }
  }

  // L / U / A row selections (src = permuted block index)
  Csr a, l, u;
  a.rowptr.assign(static_cast<size_t>(nb) + 1, 0);
  l.rowptr = a.rowptr;
  u.rowptr = a.rowptr;
  for (int i = 0; i < nb; ++i) {
    for (int k = an.prowptr[i]; k < an.prowptr[i + 1]; ++k) {
      const int j = an.pcolind[k];
      a.col.push_back(j); a.src.push_back(k);
      if (j < i) { l.col.push_back(j); l.src.push_back(k); }
      if (j > i) { u.col.push_back(j); u.src.push_back(k); }
    }
    a.rowptr[i + 1] = static_cast<int>(a.col.size());
    l.rowptr[i + 1] = static_cast<int>(l.col.size());
    u.rowptr[i + 1] = static_cast<int>(u.col.size());
  }
  an.nnzb_l = static_cast<int>(l.col.size());
  an.nnzb_u = static_cast<int>(u.col.size());

  // slices: 32 consecutive rows of one color
  an.slice_color_ptr.assign(C + 1, 0);
  for (int c = 0; c < C; ++c) {
    const int rows = an.color_ptr[c + 1] - an.color_ptr[c];
    const int ns = (rows + kSliceRows - 1) / kSliceRows;
    an.slice_color_ptr[c + 1] = an.slice_color_ptr[c] + ns;
    for (int s = 0; s < ns; ++s) {
      an.slice_row0.push_back(an.color_ptr[c] + s * kSliceRows);
      an.slice_len.push_back(std::min(kSliceRows, rows - s * kSliceRows));
    }
  }
  an.S = an.slice_color_ptr[C];

  // device numbering: each color's split run and its other run, rows by
  // descending block count (stable)
  an.dperm.resize(nb);
  an.idperm.resize(nb);
  std::iota(an.dperm.begin(), an.dperm.end(), 0);
  for (int c = 0; c < C; ++c) {
    const int bounds[3] = {an.color_ptr[c], an.color_ptr[c] + an.split[c], an.color_ptr[c + 1]};
    for (int g = 0; g < 2; ++g)
      std::stable_sort(an.dperm.begin() + bounds[g], an.dperm.begin() + bounds[g + 1],
                       [&](int x, int y) {
                         return an.prowptr[x + 1] - an.prowptr[x] > an.prowptr[y + 1] - an.prowptr[y];
                       });
  }
  for (int d = 0; d < nb; ++d) an.idperm[an.dperm[d]] = d;

  slice_matrix(an, a, false, an.A);
  slice_matrix(an, l, false, an.L);
  slice_matrix(an, u, false, an.U);
  if (with_transposes) {
    slice_matrix(an, transpose_csr(nb, a), true, an.At);
    // rows of U^T hold U_ij^T (i < j): lower part; rows of L^T: upper part
    slice_matrix(an, transpose_csr(nb, u), true, an.Ut);
    slice_matrix(an, transpose_csr(nb, l), true, an.Lt);
  }
  return "";
}

void permute_values(const Analysis &an, const double *vals, double *pvals) {
  for (int k = 0; k < an.nnzb; ++k)
    std::memcpy(pvals + static_cast<size_t>(k) * 9,
                vals + static_cast<size_t>(an.psrc[k]) * 9, 9 * sizeof(double));
}

namespace {

// 3x3 inverse via cofactors; false when singular or not finite.
bool inv3(const double *a, double *o) {
  const double c00 = a[4] * a[8] - a[5] * a[7];
  const double c01 = a[5] * a[6] - a[3] * a[8];
  const double c02 = a[3] * a[7] - a[4] * a[6];
  const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  if (det == 0.0 || !std::isfinite(det)) return false;
  const double id = 1.0 / det;
  o[0] = c00 * id;
  o[1] = (a[2] * a[7] - a[1] * a[8]) * id;
  o[2] = (a[1] * a[5] - a[2] * a[4]) * id;
  o[3] = c01 * id;
  o[4] = (a[0] * a[8] - a[2] * a[6]) * id;
  o[5] = (a[2] * a[3] - a[0] * a[5]) * id;
  o[6] = c02 * id;
  o[7] = (a[1] * a[6] - a[0] * a[7]) * id;
  o[8] = (a[0] * a[4] - a[1] * a[3]) * id;
  return true;
}

inline void mul3(const double *a, const double *b, double *o) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      o[r * 3 + c] = a[r * 3] * b[c] + a[r * 3 + 1] * b[3 + c] + a[r * 3 + 2] * b[6 + c];
}

}  // namespace

int bilu0(const Analysis &an, double *v, double *dinv) {
  // IKJ block ILU(0): for row i and each k < i in row i, L_ik = A_ik U_kk^-1,
  // then A_ij -= L_ik U_kj for every j > k present in both rows i and k.
  const int nb = an.nb;
  std::vector<int> pos(nb, -1);
  for (int i = 0; i < nb; ++i) {
    for (int k = an.prowptr[i]; k < an.prowptr[i + 1]; ++k) pos[an.pcolind[k]] = k;
    for (int kk = an.prowptr[i]; kk < an.pdiag[i]; ++kk) {
      const int k = an.pcolind[kk];
      double l[9];
      mul3(v + static_cast<size_t>(kk) * 9, dinv + static_cast<size_t>(k) * 9, l);
      std::memcpy(v + static_cast<size_t>(kk) * 9, l, sizeof l);
      for (int jj = an.pdiag[k] + 1; jj < an.prowptr[k + 1]; ++jj) {
        const int p = pos[an.pcolind[jj]];
        if (p < 0) continue;
        double t[9];
        mul3(l, v + static_cast<size_t>(jj) * 9, t);
        double *dst = v + static_cast<size_t>(p) * 9;
        for (int e = 0; e < 9; ++e) dst[e] -= t[e];
      }
    }
    if (!inv3(v + static_cast<size_t>(an.pdiag[i]) * 9, dinv + static_cast<size_t>(i) * 9))
      return i;
    for (int k = an.prowptr[i]; k < an.prowptr[i + 1]; ++k) pos[an.pcolind[k]] = -1;
  }
  return -1;
}

template <typename V>
void fill_sliced(const SlicedMatrix &m, const double *src, V *out) {
  const size_t slots = static_cast<size_t>(m.slots());
  for (size_t slot = 0; slot < slots; ++slot)
    for (int l = 0; l < kSliceRows; ++l) {
      const int s = m.vsrc[slot * kSliceRows + l];
      for (int e = 0; e < 9; ++e) {
        double x = 0.0;
        if (s >= 0) {
          const int ee = m.transpose_blocks ? (e % 3) * 3 + e / 3 : e;
          x = src[static_cast<size_t>(s) * 9 + ee];
        }
        out[(slot * 9 + e) * kSliceRows + l] = static_cast<V>(x);
      }
    }
}

template <typename V>
void fill_sliced_diag(const Analysis &an, const double *d, bool transpose, V *out) {
  for (int s = 0; s < an.S; ++s)
    for (int l = 0; l < kSliceRows; ++l) {
      const int r = l < an.slice_len[s] ? an.dperm[an.slice_row0[s] + l] : 0;
      for (int e = 0; e < 9; ++e) {
        double x = 0.0;
        if (l < an.slice_len[s]) {
          const int ee = transpose ? (e % 3) * 3 + e / 3 : e;
          x = d[static_cast<size_t>(r) * 9 + ee];
        }
        out[(static_cast<size_t>(s) * 9 + e) * kSliceRows + l] = static_cast<V>(x);
      }
    }
}

template void fill_sliced<double>(const SlicedMatrix &, const double *, double *);
template void fill_sliced_diag<double>(const Analysis &, const double *, bool, double *);

}  // namespace gbilu
