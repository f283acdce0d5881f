// Reductions over instances (MapSum). See reduce.cuh for the two summation orders.
//
// Both sum kernels run one warp per work item with coalesced loads along the instance axis
// (rows are instance-minor). The instance-order kernel broadcasts each 32-instance segment
// with shuffles and adds it lane by lane in order: its time is the dependent FP64 add chain,
// n adds per row, rows in parallel. The tree kernel is bound by HBM (one read of the block).
#include <algorithm>

#include "reduce.cuh"

namespace cgb {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarpsPerCta = 8;

__global__ void __launch_bounds__(kWarpsPerCta * 32)
    k_sum_instance_order(long long rows, long long n, const double* __restrict__ src,
                         long long ld, double* __restrict__ dst) {
  const int lane = threadIdx.x & 31;
  const long long r = static_cast<long long>(blockIdx.x) * kWarpsPerCta + (threadIdx.x >> 5);
  if (r >= rows) return;
  const double* row = src + r * ld;
  // one lane runs the chain: no shuffle between two dependent adds, and the FP64 pipe takes
  // one active lane per add instead of a full warp; the loads are independent of the chain
  // and run ahead of it (unrolled)
  if (lane != 0) return;
  double acc = 0.0;
  long long i = 0;
  for (; i + 8 <= n; i += 8) {
    double v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = __ldg(row + i + k);
#pragma unroll
    for (int k = 0; k < 8; ++k) acc = __dadd_rn(acc, v[k]);
  }
  for (; i < n; ++i) acc = __dadd_rn(acc, __ldg(row + i));
  dst[r] = acc;
}

struct SumRowsArgs {
  SumRows g[kMaxSumGroups];
  int count;
};

__global__ void __launch_bounds__(128)
    k_sum_instance_multi(const __grid_constant__ SumRowsArgs a, long long n) {
  long long r = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  int k = 0;
  while (k < a.count && r >= a.g[k].rows) r -= a.g[k++].rows;
  if (k >= a.count) return;
  const double* row = a.g[k].src + r * a.g[k].ld;
  double acc = 0.0;
  long long i = 0;
  for (; i + 8 <= n; i += 8) {
    double v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __ldg(row + i + j);
#pragma unroll
    for (int j = 0; j < 8; ++j) acc = __dadd_rn(acc, v[j]);
  }
  for (; i < n; ++i) acc = __dadd_rn(acc, __ldg(row + i));
  a.g[k].dst[r] = acc;
}

// One level of the blocked tree: item (r, b) sums x[r][b*256 .. b*256+255] into y[r][b].
__global__ void __launch_bounds__(kWarpsPerCta * 32)
    k_sum_tree_level(long long rows, long long m, const double* __restrict__ src, long long ld,
                     double* __restrict__ dst, long long dst_ld) {
  const int lane = threadIdx.x & 31;
  const long long nb = (m + kTreeBlock - 1) / kTreeBlock;
  const long long item = static_cast<long long>(blockIdx.x) * kWarpsPerCta + (threadIdx.x >> 5);
  if (item >= rows * nb) return;
  const long long r = item / nb, b = item - r * nb;
  const double* x = src + r * ld + b * kTreeBlock;
  const long long left = m - b * kTreeBlock;
  double acc = 0.0;
#pragma unroll
  for (int k = 0; k < kTreeBlock / 32; ++k) {
    const int i = k * 32 + lane;
    if (i < left) acc = __dadd_rn(acc, __ldg(x + i));
  }
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) acc = __dadd_rn(acc, __shfl_xor_sync(kFull, acc, s));
  if (lane == 0) dst[r * dst_ld + b] = acc;
}

__global__ void __launch_bounds__(kWarpsPerCta * 32)
    k_or_rows(long long rows, long long n, const unsigned long long* __restrict__ src,
              long long ld, unsigned long long* __restrict__ dst, bool accumulate) {
  const int lane = threadIdx.x & 31;
  const long long r = static_cast<long long>(blockIdx.x) * kWarpsPerCta + (threadIdx.x >> 5);
  if (r >= rows) return;
  const unsigned long long* row = src + r * ld;
  unsigned long long acc = 0;
  for (long long i = lane; i < n; i += 32) acc |= __ldg(row + i);
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) acc |= __shfl_xor_sync(kFull, acc, s);
  if (lane == 0) dst[r] = accumulate ? (dst[r] | acc) : acc;
}

__global__ void k_broadcast_rows(long long rows, long long n,
                                 const unsigned long long* __restrict__ src,
                                 unsigned long long* __restrict__ dst, long long ld) {
  const long long total = rows * n;
  for (long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; k < total;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long r = k / n, i = k - r * n;
    dst[r * ld + i] = __ldg(src + r);
  }
}

__global__ void k_add_blocks(long long ndir, long long nnz, long long n,
                             const double* __restrict__ a, long long a_nz, long long a_dir,
                             const double* __restrict__ b, double* __restrict__ dst) {
  const long long total = ndir * nnz * n;
  for (long long q = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; q < total;
       q += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long i = q % n, r = q / n, k = r % nnz, d = r / nnz;
    const double* pa = a ? a + d * a_dir + k * a_nz + i : nullptr;
    double v;
    if (pa && b) v = __dadd_rn(__ldg(pa), __ldg(b + q));
    else if (pa) v = __ldg(pa);
    else if (b) v = __ldg(b + q);
    else v = 0.0;
    dst[q] = v;
  }
}

unsigned blocks_for(long long items) {
  const long long b = (items + kWarpsPerCta - 1) / kWarpsPerCta;
  return static_cast<unsigned>(std::max<long long>(1, b));
}

}  // namespace

size_t reduce_scratch_bytes(long long rows, long long n, int order) {
  if (order != kOrderTree) return 0;
  // two ping-pong level buffers; the first level's output is the largest
  const long long nb = (n + kTreeBlock - 1) / kTreeBlock;
  if (nb <= 1) return 0;
  const long long nb2 = (nb + kTreeBlock - 1) / kTreeBlock;
  return static_cast<size_t>(rows) * static_cast<size_t>(nb + nb2) * sizeof(double);
}

cudaError_t reduce_sum(long long rows, long long n, const double* src, long long ld, double* dst,
                       int order, double* scratch, cudaStream_t s) {
  if (rows <= 0) return cudaSuccess;
  if (order == kOrderInstance || n == 0) {  // no instances: +0, as the instance-order sum
    k_sum_instance_order<<<blocks_for(rows), kWarpsPerCta * 32, 0, s>>>(rows, n, src, ld, dst);
    return cudaGetLastError();
  }
  // tree: levels until one value per row; at least one level (n <= 256 included)
  long long m = n;
  const double* x = src;
  long long x_ld = ld;
  const long long nb1 = (n + kTreeBlock - 1) / kTreeBlock;
  double* buf[2] = {scratch, scratch ? scratch + rows * nb1 : nullptr};
  int which = 0;
  for (;;) {
    const long long nb = (m + kTreeBlock - 1) / kTreeBlock;
    const bool last = nb <= 1;
    double* y = last ? dst : buf[which];
    const long long y_ld = last ? 1 : nb;
    if (!y) return cudaErrorInvalidValue;
    k_sum_tree_level<<<blocks_for(rows * std::max<long long>(nb, 1)), kWarpsPerCta * 32, 0, s>>>(
        rows, m, x, x_ld, y, y_ld);
    if (cudaError_t e = cudaGetLastError()) return e;
    if (last) return cudaSuccess;
    x = y;
    x_ld = y_ld;
    m = nb;
    which ^= 1;
  }
}

cudaError_t reduce_sum_instance_multi(const SumRows* groups, int count, long long n,
                                      cudaStream_t s) {
  // at most kMaxSumGroups groups per launch (the launch's parameter block holds them); more
  // groups take more launches, each row's chain being the same
  for (int k0 = 0; k0 < count; k0 += kMaxSumGroups) {
    const int c = std::min(kMaxSumGroups, count - k0);
    SumRowsArgs a;
    long long total = 0;
    for (int k = 0; k < c; ++k) {
      a.g[k] = groups[k0 + k];
      total += groups[k0 + k].rows;
    }
    a.count = c;
    if (total == 0) continue;
    const long long blocks = (total + 127) / 128;
    k_sum_instance_multi<<<static_cast<unsigned>(blocks), 128, 0, s>>>(a, n);
    if (cudaError_t e = cudaGetLastError()) return e;
  }
  return cudaSuccess;
}

cudaError_t reduce_or(long long rows, long long n, const unsigned long long* src, long long ld,
                      unsigned long long* dst, bool accumulate, cudaStream_t s) {
  if (rows <= 0) return cudaSuccess;
  k_or_rows<<<blocks_for(rows), kWarpsPerCta * 32, 0, s>>>(rows, n, src, ld, dst, accumulate);
  return cudaGetLastError();
}

cudaError_t broadcast_rows(long long rows, long long n, const unsigned long long* src,
                           unsigned long long* dst, long long ld, cudaStream_t s) {
  if (rows <= 0 || n <= 0) return cudaSuccess;
  const long long total = rows * n;
  const unsigned grid = static_cast<unsigned>(std::min<long long>((total + 255) / 256, 4096));
  k_broadcast_rows<<<grid, 256, 0, s>>>(rows, n, src, dst, ld);
  return cudaGetLastError();
}

cudaError_t add_blocks(long long ndir, long long nnz, long long n, const double* a, long long a_nz,
                       long long a_dir, const double* b, double* dst, cudaStream_t s) {
  const long long total = ndir * nnz * n;
  if (total <= 0) return cudaSuccess;
  const unsigned grid = static_cast<unsigned>(std::min<long long>((total + 255) / 256, 8192));
  k_add_blocks<<<grid, 256, 0, s>>>(ndir, nnz, n, a, a_nz, a_dir, b, dst);
  return cudaGetLastError();
}

}  // namespace cgb
