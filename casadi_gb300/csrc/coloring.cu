// Graph colourings for compressed Jacobians and Hessians (host code).
//
// Restatements of the reference's colourings, step by step, so the seed matrices match:
//   uni_coloring   SparsityInternal::uni_coloring   (casadi/core/sparsity_internal.cpp:2959-3045)
//   largest_first  SparsityInternal::largest_first  (:3511-3545)
//   star_coloring  SparsityInternal::star_coloring  (:3398-3509), largest-first ordering by
//                  default as Sparsity::star_coloring (casadi/core/sparsity.hpp:1120)
// Patterns are compressed-column arrays with sorted rows (CasADi's Sparsity layout).
#include <algorithm>
#include <cstdint>
#include <vector>

#include "coloring.cuh"

namespace cgb {

namespace {

// Column colouring of A (nrow x ncol) given A and its transpose AT: columns of one colour
// share no row. Returns the number of colours.
int uni_coloring(int ncol, const int* colind, const int* row, const int* at_colind,
                 const int* at_row, int* color) {
  std::vector<int> forbidden;
  for (int i = 0; i < ncol; ++i) {
    for (int el = colind[i]; el < colind[i + 1]; ++el) {
      const int c = row[el];
      // previous columns with an element in row c
      for (int el_prev = at_colind[c]; el_prev < at_colind[c + 1]; ++el_prev) {
        const int i_prev = at_row[el_prev];
        if (i_prev >= i) break;
        forbidden[color[i_prev]] = i;
      }
    }
    int ci = 0;
    while (ci < static_cast<int>(forbidden.size()) && forbidden[ci] == i) ++ci;
    color[i] = ci;
    if (ci == static_cast<int>(forbidden.size())) forbidden.push_back(-1);
  }
  return static_cast<int>(forbidden.size());
}

std::vector<int> largest_first(int n, const int* colind) {
  std::vector<int> degree(n);
  int max_degree = 0;
  for (int k = 0; k < n; ++k) {
    degree[k] = colind[k + 1] - colind[k];
    max_degree = std::max(max_degree, 1 + degree[k]);
  }
  std::vector<int> count(max_degree + 1, 0);
  for (int d : degree) count[d + 1]++;
  for (int d = 0; d < max_degree; ++d) count[d + 1] += count[d];
  std::vector<int> ordering(n);
  for (int k = n - 1; k >= 0; --k) ordering[count[degree[k]]++] = k;
  std::reverse(ordering.begin(), ordering.end());
  return ordering;
}

// Star colouring (Gebremedhin, Manne, Pothen, Algorithm 4.1 as the reference states it) of
// a symmetric pattern, vertices in index order.
int star_coloring0(int n, const int* colind, const int* row, int* color) {
  std::vector<int> forbidden;
  std::fill(color, color + n, -1);
  for (int i = 0; i < n; ++i) {
    for (int w_el = colind[i]; w_el < colind[i + 1]; ++w_el) {
      const int w = row[w_el];
      if (color[w] != -1) forbidden[color[w]] = i;
      for (int x_el = colind[w]; x_el < colind[w + 1]; ++x_el) {
        const int x = row[x_el];
        if (color[x] == -1) continue;
        if (color[w] == -1) {
          forbidden[color[x]] = i;
        } else {
          for (int y_el = colind[x]; y_el < colind[x + 1]; ++y_el) {
            const int y = row[y_el];
            if (color[y] == -1 || y == w) continue;
            if (color[y] == color[w]) {
              forbidden[color[x]] = i;
              break;
            }
          }
        }
      }
    }
    bool fresh = true;
    for (int ci = 0; ci < static_cast<int>(forbidden.size()); ++ci) {
      if (forbidden[ci] != i) {
        color[i] = ci;
        fresh = false;
        break;
      }
    }
    if (fresh) {
      color[i] = static_cast<int>(forbidden.size());
      forbidden.push_back(-1);
    }
  }
  return static_cast<int>(forbidden.size());
}

}  // namespace

int uni_coloring_ccs(int nrow, int ncol, const int* colind, const int* row, int* color) {
  const int nnz = colind[ncol];
  // transpose (rows sorted by construction)
  std::vector<int> at_colind(nrow + 1, 0), at_row(nnz);
  for (int k = 0; k < nnz; ++k) at_colind[row[k] + 1]++;
  for (int r = 0; r < nrow; ++r) at_colind[r + 1] += at_colind[r];
  std::vector<int> fill(at_colind.begin(), at_colind.end() - 1);
  for (int j = 0; j < ncol; ++j)
    for (int el = colind[j]; el < colind[j + 1]; ++el) at_row[fill[row[el]]++] = j;
  return uni_coloring(ncol, colind, row, at_colind.data(), at_row.data(), color);
}

int star_coloring_ccs(int n, const int* colind, const int* row, int ordering, int* color) {
  if (ordering == 0) return star_coloring0(n, colind, row, color);
  // vertex ord[k] becomes k (rows and columns), colour, map the colours back
  const int nnz = colind[n];
  const std::vector<int> ord = largest_first(n, colind);
  std::vector<int> inv(n);
  for (int k = 0; k < n; ++k) inv[ord[k]] = k;
  std::vector<std::vector<int>> cols(n);
  for (int j = 0; j < n; ++j)
    for (int el = colind[j]; el < colind[j + 1]; ++el) cols[inv[j]].push_back(inv[row[el]]);
  std::vector<int> pc(n + 1, 0), pr;
  pr.reserve(nnz);
  for (int j = 0; j < n; ++j) {
    std::sort(cols[j].begin(), cols[j].end());
    pr.insert(pr.end(), cols[j].begin(), cols[j].end());
    pc[j + 1] = static_cast<int>(pr.size());
  }
  std::vector<int> cp(n);
  const int nc = star_coloring0(n, pc.data(), pr.data(), cp.data());
  for (int k = 0; k < n; ++k) color[ord[k]] = cp[k];
  return nc;
}

}  // namespace cgb
