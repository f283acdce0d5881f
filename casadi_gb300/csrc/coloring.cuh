// Graph colourings for compressed Jacobians and Hessians (host code, see coloring.cu).
#pragma once

namespace cgb {

// Column colouring of a CCS pattern (nrow x ncol, sorted rows): columns of one colour share no
// row. Writes color[ncol]; returns the number of colours.
int uni_coloring_ccs(int nrow, int ncol, const int* colind, const int* row, int* color);

// Star colouring of a symmetric CCS pattern (n x n); ordering 1 = largest-first, 0 = index
// order. Writes color[n]; returns the number of colours.
int star_coloring_ccs(int n, const int* colind, const int* row, int ordering, int* color);

}  // namespace cgb
