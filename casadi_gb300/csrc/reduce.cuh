// Reductions over instances for MapSum (casadi/core/mapsum.cpp:153-181, :196-232).
//
// A block of `rows` rows, row r holding the values of one output nonzero (of one direction)
// for n instances at src + r*ld. Sums are either
//   kOrderInstance  in instance order from +0: ((0 + x0) + x1) + ... -- MapSum's own order
//                   (casadi_clear, then casadi_add per instance), identical bits; a chain of
//                   n dependent adds per row
//   kOrderTree      a fixed blocked tree: per level, 256-instance blocks; lane l of a warp
//                   adds x[b*256 + m*32 + l] for m = 0..7 in order starting from +0, then a
//                   butterfly over lanes (xor 16, 8, 4, 2, 1); the block sums form the next
//                   level's row until one value remains. The bits do not depend on the grid.
// bvec_t rows OR-reduce (order does not matter).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace cgb {

constexpr int kOrderInstance = 0;
constexpr int kOrderTree = 1;
constexpr int kTreeBlock = 256;

// Device scratch (bytes) kOrderTree needs for `rows` rows of n instances (0 for
// kOrderInstance and n <= kTreeBlock).
size_t reduce_scratch_bytes(long long rows, long long n, int order);

// dst[r] (= or +=, see `accumulate`) the sum of row r. `scratch` as reduce_scratch_bytes.
cudaError_t reduce_sum(long long rows, long long n, const double* src, long long ld, double* dst,
                       int order, double* scratch, cudaStream_t s);
// Several blocks of rows summed in instance order (kOrderInstance) by one launch, one thread
// per row: the rows' chains of n dependent adds run concurrently instead of one block after
// the other (each add waits for the previous one, ~85 cycles on GB300's FP64 pipe, so a chain
// costs ~40 ns per instance whatever else runs beside it). Same bits as reduce_sum.
struct SumRows {
  const double* src;  // rows of n values, row r at src + r*ld
  long long ld;
  double* dst;        // dst[r] = the sum of row r
  long long rows;
};
constexpr int kMaxSumGroups = 120;  // groups per launch: the parameter block stays under 4 KB
cudaError_t reduce_sum_instance_multi(const SumRows* groups, int count, long long n,
                                      cudaStream_t s);

// dst[r] |= OR of row r (accumulate) or dst[r] = OR of row r.
cudaError_t reduce_or(long long rows, long long n, const unsigned long long* src, long long ld,
                      unsigned long long* dst, bool accumulate, cudaStream_t s);
// dst + r*ld holds n copies of src[r] (8-byte elements).
cudaError_t broadcast_rows(long long rows, long long n, const unsigned long long* src,
                           unsigned long long* dst, long long ld, cudaStream_t s);

// dst[(d*nnz + k)*n + i] = a[d*a_dir + k*a_nz + i] + b[(d*nnz + k)*n + i] over ndir x nnz x n;
// a null operand contributes nothing (the other is copied), both null give zeros.
cudaError_t add_blocks(long long ndir, long long nnz, long long n, const double* a, long long a_nz,
                       long long a_dir, const double* b, double* dst, cudaStream_t s);

}  // namespace cgb
