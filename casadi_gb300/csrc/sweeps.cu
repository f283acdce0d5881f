// Tape-sweep kernels for sm_103a.
//
// Every kernel interprets the same instruction stream. It is staged chunk by chunk
// (kChunk 8-byte words) from global memory into a two-slot shared-memory ring with TMA bulk
// copies (cp.async.bulk ... mbarrier::complete_tx), while the previous chunk is being
// interpreted. Every thread of a CTA runs the same instruction on a different instance
// (or instance/direction pair), so the opcode dispatch is warp-uniform and never diverges.
// The work vector lives in shared memory in slot-major order, w[slot*BS + thread]:
// consecutive lanes hit consecutive 8-byte words, so every work-vector access is
// bank-conflict free. Instance data in global memory is read and written through IoDesc
// strides, which covers both the instance-minor layout (coalesced) and the instance-major
// layout of CasADi's Map (casadi/core/map.cpp:150-153) without a separate transpose pass.
//
// Kernels:
//   k_primal<BS,false>  forward value sweep           SXFunction::eval (sx_function.cpp:110-124)
//   k_primal<BS,true>   values + recorded partials    (first half of the AD sweeps)
//   k_tangent<DW>       forward-mode directions       ad_forward, numeric (sx_function.cpp:1318-1364)
//   k_adjoint<DW>       adjoint directions            ad_reverse, numeric (sx_function.cpp:1454-1560)
//   k_sp_forward<BS>    bvec_t OR-propagation         sp_forward (sx_function.cpp:1657-1682)
//   k_sp_reverse<BS>    bvec_t reverse propagation    sp_reverse (sx_function.cpp:1742-1782)
//
// Waits on the staging barriers are bounded: after ~1 s without completion a kernel sets
// kErrWaitTimeout in the tape's error word, waits (again bounded) for its own copies in
// flight and returns. No kernel traps.
#include "sweeps.cuh"

namespace cgb {

constexpr long long kWaitCycles = 2000000000ll;  // ~1 s at GB300 clocks
constexpr size_t kRingBytes = 2 * kChunk * sizeof(u64);
constexpr size_t kHeaderBytes = kRingBytes + 2 * sizeof(u64);  // ring + two mbarriers

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void stage_init(u64* bars) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[0])) : "memory");
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[1])) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Issue the copy of chunk `chunk` into ring slot (seq & 1). Called by one thread.
__device__ __forceinline__ void stage_issue(u64* ring, u64* bars, const u64* code,
                                            unsigned seq, int chunk) {
  u64* dst = ring + (seq & 1u) * kChunk;
  u64* bar = bars + (seq & 1u);
  const unsigned bytes = kChunk * sizeof(u64);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(code + static_cast<size_t>(chunk) * kChunk), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait for the copy of sequence number `seq` (k-th use of a slot has parity k&1).
__device__ __forceinline__ bool stage_wait(u64* bars, unsigned seq) {
  const unsigned addr = smem_u32(bars + (seq & 1u));
  const unsigned parity = (seq >> 1) & 1u;
  const long long t0 = clock64();
  for (unsigned it = 0;; ++it) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 31u) == 31u && clock64() - t0 > kWaitCycles) return false;
  }
}

// Timeout path: flag the error and give copies still in flight a bounded chance to land
// before the CTA's shared memory is released.
__device__ __noinline__ void stage_abort(const TapeView& t, u64* bars, unsigned seq,
                                         bool next_issued) {
  if (threadIdx.x == 0) {
    atomicOr(t.err, kErrWaitTimeout);
    stage_wait(bars, seq);
    if (next_issued) stage_wait(bars, seq + 1);
  }
}

// Run f(instruction) over the whole tape in order. Returns false (for every thread of the
// CTA) if a staged chunk did not arrive in time.
template <class F>
__device__ __forceinline__ bool sweep_forward(const TapeView& t, u64* ring, u64* bars,
                                              unsigned& seq, F&& f) {
  const int nch = t.n_chunks;
  if (threadIdx.x == 0) stage_issue(ring, bars, t.code, seq, 0);
#pragma unroll 1
  for (int ch = 0; ch < nch; ++ch) {
    const bool more = ch + 1 < nch;
    if (threadIdx.x == 0 && more) stage_issue(ring, bars, t.code, seq + 1, ch + 1);
    const bool ok = stage_wait(bars, seq);
    if (!__syncthreads_and(ok)) {
      stage_abort(t, bars, seq, more);
      return false;
    }
    const u64* code = ring + (seq & 1u) * kChunk;
#pragma unroll 1
    for (int k = 0; k < kChunk; ++k) f(code[k]);
    __syncthreads();
    ++seq;
  }
  return true;
}

// Same, last instruction first.
template <class F>
__device__ __forceinline__ bool sweep_reverse(const TapeView& t, u64* ring, u64* bars,
                                              unsigned& seq, F&& f) {
  const int nch = t.n_chunks;
  if (threadIdx.x == 0) stage_issue(ring, bars, t.code, seq, nch - 1);
#pragma unroll 1
  for (int ch = nch - 1; ch >= 0; --ch) {
    const bool more = ch > 0;
    if (threadIdx.x == 0 && more) stage_issue(ring, bars, t.code, seq + 1, ch - 1);
    const bool ok = stage_wait(bars, seq);
    if (!__syncthreads_and(ok)) {
      stage_abort(t, bars, seq, more);
      return false;
    }
    const u64* code = ring + (seq & 1u) * kChunk;
#pragma unroll 1
    for (int k = kChunk - 1; k >= 0; --k) f(code[k]);
    __syncthreads();
    ++seq;
  }
  return true;
}

__device__ __forceinline__ long long io_off(const IoDesc& d, long long dir, long long nz,
                                            long long inst) {
  return dir * d.dir_stride + nz * d.nz_stride + inst * d.inst_stride;
}

// ---------------------------------------------------------------------------------------------
// Forward value sweep (RECORD=false) and value + partials sweep (RECORD=true).
// One thread per instance; BS instances per tile; persistent over tiles.
// ---------------------------------------------------------------------------------------------
template <int BS, bool RECORD>
__global__ void __launch_bounds__(BS) k_primal(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  u64* ring = reinterpret_cast<u64*>(smem);
  u64* bars = ring + 2 * kChunk;
  double* w = reinterpret_cast<double*>(smem + kHeaderBytes);
  const int tid = threadIdx.x;
  if (tid == 0) stage_init(bars);
  __syncthreads();
  unsigned seq = 0;
  const long long ntiles = (a.n + BS - 1) / BS;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long il = tile * BS + tid;
    const bool active = il < a.n;
    const long long ig = a.i_begin + il;
    long long pidx = 0;
    const bool ok = sweep_forward(a.t, ring, bars, seq, [&](u64 ins) {
      const unsigned op = dec_op(ins), A = dec_a(ins), B = dec_b(ins), C = dec_c(ins);
      switch (op) {
        case D_NOP:
          break;
        case D_CONST:
          w[A * BS + tid] = __ldg(a.t.consts + B);
          break;
        case D_INPUT: {
          const IoDesc& d = a.in[B];
          double v = 0.0;
          if (active && d.ptr) v = __ldg(static_cast<const double*>(d.ptr) + io_off(d, 0, C, ig));
          w[A * BS + tid] = v;
        } break;
        case D_OUTPUT: {
          const IoDesc& d = a.out[A];
          if (active && d.ptr) static_cast<double*>(d.ptr)[io_off(d, 0, C, ig)] = w[B * BS + tid];
        } break;
        default: {
          const double x = w[B * BS + tid], y = w[C * BS + tid];
          if (RECORD) {
            const unsigned m = partial_mask(op);
            double d0 = 0.0, d1 = 0.0;
            const double f = dev_fun_der(op, x, y, d0, d1);
            if (m & 1u) {
              if (active) a.partials[pidx * a.pt_stride + il] = d0;
              ++pidx;
            }
            if (m & 2u) {
              if (active) a.partials[pidx * a.pt_stride + il] = d1;
              ++pidx;
            }
            w[A * BS + tid] = f;
          } else {
            w[A * BS + tid] = dev_fun(op, x, y);
          }
        }
      }
    });
    if (!ok) return;
  }
}

// ---------------------------------------------------------------------------------------------
// Forward-mode directions from recorded partials. CTA = 32 instances x DW directions
// (warp = direction), so each recorded partial is fetched by DW warps of one CTA.
// w'[i0] = d0*w'[i1] + d1*w'[i2] (binary), d0*w'[i1] (unary),
// if_else_zero(d1, w'[i2]) (IF_ELSE_ZERO): sx_function.cpp:1280-1363.
// ---------------------------------------------------------------------------------------------
template <int DW>
__global__ void __launch_bounds__(32 * DW) k_tangent(const __grid_constant__ SweepArgs a) {
  constexpr int BS = 32 * DW;
  extern __shared__ __align__(128) unsigned char smem[];
  u64* ring = reinterpret_cast<u64*>(smem);
  u64* bars = ring + 2 * kChunk;
  double* wd = reinterpret_cast<double*>(smem + kHeaderBytes);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) stage_init(bars);
  __syncthreads();
  const long long dir = static_cast<long long>(blockIdx.y) * DW + warp;
  const bool dir_ok = dir < a.ndir;
  unsigned seq = 0;
  const long long ntiles = (a.n + 31) / 32;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long il = tile * 32 + lane;
    const bool inst_ok = il < a.n;
    const bool active = inst_ok && dir_ok;
    const long long ig = a.i_begin + il;
    long long pidx = 0;
    const bool ok = sweep_forward(a.t, ring, bars, seq, [&](u64 ins) {
      const unsigned op = dec_op(ins), A = dec_a(ins), B = dec_b(ins), C = dec_c(ins);
      // operand slots are read only by the ops whose b/c fields are slots
      double* wa = wd + A * BS + tid;
      switch (op) {
        case D_NOP:
          break;
        case D_CONST:
          *wa = 0.0;
          break;
        case D_INPUT: {
          double v = 0.0;
          if (a.identity_seed) {
            v = (a.in_off[B] + static_cast<int>(C) == a.dir0 + dir) ? 1.0 : 0.0;
          } else {
            const IoDesc& d = a.seed[B];
            if (active && d.ptr)
              v = __ldg(static_cast<const double*>(d.ptr) + io_off(d, dir, C, ig));
          }
          *wa = v;
        } break;
        case D_OUTPUT: {
          const IoDesc& d = a.sens[A];
          if (active && d.ptr) static_cast<double*>(d.ptr)[io_off(d, dir, C, ig)] = wd[B * BS + tid];
        } break;
        case D_ADD: *wa = __dadd_rn(wd[B * BS + tid], wd[C * BS + tid]); break;
        case D_SUB: *wa = __dsub_rn(wd[B * BS + tid], wd[C * BS + tid]); break;
        case D_NEG: *wa = d_neg(wd[B * BS + tid]); break;
        case D_TWICE: { const double xb = wd[B * BS + tid]; *wa = __dadd_rn(xb, xb); } break;
        case D_ASSIGN: *wa = wd[B * BS + tid]; break;
        default: {
          const double xb = wd[B * BS + tid];
          const unsigned m = partial_mask(op);
          double d0 = const_d0(op), d1 = const_d1(op);
          if (m & 1u) {
            if (inst_ok) d0 = __ldg(a.partials + pidx * a.pt_stride + il);
            ++pidx;
          }
          if (m & 2u) {
            if (inst_ok) d1 = __ldg(a.partials + pidx * a.pt_stride + il);
            ++pidx;
          }
          if (op == D_IF_ELSE_ZERO) {
            *wa = d1 == 0.0 ? 0.0 : wd[C * BS + tid];
          } else if (is_binary(op)) {
            *wa = __dadd_rn(__dmul_rn(d0, xb), __dmul_rn(d1, wd[C * BS + tid]));
          } else {
            *wa = __dmul_rn(d0, xb);
          }
        }
      }
    });
    if (!ok) return;
  }
}

// ---------------------------------------------------------------------------------------------
// Adjoint directions from recorded partials, last instruction first.
// seed = w'[i0]; w'[i0] = 0; w'[i1] += d0*seed; w'[i2] += d1*seed (sx_function.cpp:1454-1560).
// ---------------------------------------------------------------------------------------------
template <int DW>
__global__ void __launch_bounds__(32 * DW) k_adjoint(const __grid_constant__ SweepArgs a) {
  constexpr int BS = 32 * DW;
  extern __shared__ __align__(128) unsigned char smem[];
  u64* ring = reinterpret_cast<u64*>(smem);
  u64* bars = ring + 2 * kChunk;
  double* wb = reinterpret_cast<double*>(smem + kHeaderBytes);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) stage_init(bars);
  __syncthreads();
  const long long dir = static_cast<long long>(blockIdx.y) * DW + warp;
  const bool dir_ok = dir < a.ndir;
  unsigned seq = 0;
  const long long ntiles = (a.n + 31) / 32;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long il = tile * 32 + lane;
    const bool inst_ok = il < a.n;
    const bool active = inst_ok && dir_ok;
    const long long ig = a.i_begin + il;
    for (int s = 0; s < a.t.sz_w; ++s) wb[s * BS + tid] = 0.0;
    if (active) {
      // input nonzeros the tape never reads have a zero sensitivity
      for (int k = 0; k < a.t.n_absent_in; ++k) {
        const int2 jk = a.t.absent_in[k];
        const IoDesc& d = a.sens[jk.x];
        if (d.ptr) static_cast<double*>(d.ptr)[io_off(d, dir, jk.y, ig)] = 0.0;
      }
    }
    long long pidx = a.t.n_partials;
    const bool ok = sweep_reverse(a.t, ring, bars, seq, [&](u64 ins) {
      const unsigned op = dec_op(ins), A = dec_a(ins), B = dec_b(ins), C = dec_c(ins);
      switch (op) {
        case D_NOP:
          break;
        case D_CONST:
          wb[A * BS + tid] = 0.0;
          break;
        case D_INPUT: {
          const IoDesc& d = a.sens[B];
          if (active && d.ptr) static_cast<double*>(d.ptr)[io_off(d, dir, C, ig)] = wb[A * BS + tid];
          wb[A * BS + tid] = 0.0;
        } break;
        case D_OUTPUT: {
          const IoDesc& d = a.seed[A];
          if (active && d.ptr) {
            const double s = __ldg(static_cast<const double*>(d.ptr) + io_off(d, dir, C, ig));
            wb[B * BS + tid] = __dadd_rn(wb[B * BS + tid], s);
          }
        } break;
        default: {
          const double seed = wb[A * BS + tid];
          wb[A * BS + tid] = 0.0;
          double* w1 = wb + B * BS + tid;
          double* w2 = wb + C * BS + tid;
          switch (op) {
            case D_ADD: *w1 = __dadd_rn(*w1, seed); *w2 = __dadd_rn(*w2, seed); break;
            case D_SUB: *w1 = __dadd_rn(*w1, seed); *w2 = __dadd_rn(*w2, d_neg(seed)); break;
            case D_NEG: *w1 = __dadd_rn(*w1, d_neg(seed)); break;
            case D_TWICE: *w1 = __dadd_rn(*w1, __dadd_rn(seed, seed)); break;
            case D_ASSIGN: *w1 = __dadd_rn(*w1, seed); break;
            default: {
              const unsigned m = partial_mask(op);
              double d0 = const_d0(op), d1 = const_d1(op);
              if (m & 2u) {
                --pidx;
                if (inst_ok) d1 = __ldg(a.partials + pidx * a.pt_stride + il);
              }
              if (m & 1u) {
                --pidx;
                if (inst_ok) d0 = __ldg(a.partials + pidx * a.pt_stride + il);
              }
              if (op == D_IF_ELSE_ZERO) {
                *w2 = __dadd_rn(*w2, d1 == 0.0 ? 0.0 : seed);
              } else if (is_binary(op)) {
                *w1 = __dadd_rn(*w1, __dmul_rn(d0, seed));
                *w2 = __dadd_rn(*w2, __dmul_rn(d1, seed));
              } else {
                *w1 = __dadd_rn(*w1, __dmul_rn(d0, seed));
              }
            }
          }
        }
      }
    });
    if (!ok) return;
  }
}

// ---------------------------------------------------------------------------------------------
// bvec_t sparsity sweeps (uint64 bit sets, 64 directions at once).
// ---------------------------------------------------------------------------------------------
template <int BS>
__global__ void __launch_bounds__(BS) k_sp_forward(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  u64* ring = reinterpret_cast<u64*>(smem);
  u64* bars = ring + 2 * kChunk;
  u64* w = reinterpret_cast<u64*>(smem + kHeaderBytes);
  const int tid = threadIdx.x;
  if (tid == 0) stage_init(bars);
  __syncthreads();
  unsigned seq = 0;
  const long long ntiles = (a.n + BS - 1) / BS;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long il = tile * BS + tid;
    const bool active = il < a.n;
    const long long ig = a.i_begin + il;
    const bool ok = sweep_forward(a.t, ring, bars, seq, [&](u64 ins) {
      const unsigned op = dec_op(ins), A = dec_a(ins), B = dec_b(ins), C = dec_c(ins);
      switch (op) {
        case D_NOP:
          break;
        case D_CONST:
          w[A * BS + tid] = 0;
          break;
        case D_INPUT: {
          const IoDesc& d = a.in[B];
          u64 v = 0;
          if (active && d.ptr) v = __ldg(static_cast<const u64*>(d.ptr) + io_off(d, 0, C, ig));
          w[A * BS + tid] = v;
        } break;
        case D_OUTPUT: {
          const IoDesc& d = a.out[A];
          if (active && d.ptr) static_cast<u64*>(d.ptr)[io_off(d, 0, C, ig)] = w[B * BS + tid];
        } break;
        default:
          w[A * BS + tid] = w[B * BS + tid] | w[C * BS + tid];
      }
    });
    if (!ok) return;
  }
}

template <int BS>
__global__ void __launch_bounds__(BS) k_sp_reverse(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  u64* ring = reinterpret_cast<u64*>(smem);
  u64* bars = ring + 2 * kChunk;
  u64* w = reinterpret_cast<u64*>(smem + kHeaderBytes);
  const int tid = threadIdx.x;
  if (tid == 0) stage_init(bars);
  __syncthreads();
  unsigned seq = 0;
  const long long ntiles = (a.n + BS - 1) / BS;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long il = tile * BS + tid;
    const bool active = il < a.n;
    const long long ig = a.i_begin + il;
    for (int s = 0; s < a.t.sz_w; ++s) w[s * BS + tid] = 0;
    const bool ok = sweep_reverse(a.t, ring, bars, seq, [&](u64 ins) {
      const unsigned op = dec_op(ins), A = dec_a(ins), B = dec_b(ins), C = dec_c(ins);
      switch (op) {
        case D_NOP:
          break;
        case D_CONST:
          w[A * BS + tid] = 0;
          break;
        case D_INPUT: {
          const IoDesc& d = a.in[B];
          if (active && d.ptr) static_cast<u64*>(d.ptr)[io_off(d, 0, C, ig)] |= w[A * BS + tid];
          w[A * BS + tid] = 0;
        } break;
        case D_OUTPUT: {
          const IoDesc& d = a.out[A];
          if (active && d.ptr) {
            u64* p = static_cast<u64*>(d.ptr) + io_off(d, 0, C, ig);
            w[B * BS + tid] |= *p;
            *p = 0;
          }
        } break;
        default: {
          const u64 seed = w[A * BS + tid];
          w[A * BS + tid] = 0;
          w[B * BS + tid] |= seed;
          w[C * BS + tid] |= seed;
        }
      }
    });
    if (!ok) return;
  }
}

// ---------------------------------------------------------------------------------------------
// Host-side launchers
// ---------------------------------------------------------------------------------------------
size_t smem_primal(int sz_w, int block) {
  return kHeaderBytes + static_cast<size_t>(sz_w > 0 ? sz_w : 1) * block * 8;
}
size_t smem_dir(int sz_w, int dir_warps) {
  return kHeaderBytes + static_cast<size_t>(sz_w > 0 ? sz_w : 1) * 32 * dir_warps * 8;
}

int max_smem_optin() {
  static int v = -1;
  if (v < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
      v = 48 * 1024;
  }
  return v;
}

template <class K>
static cudaError_t launch_k(K kernel, dim3 grid, int block, size_t smem, const SweepArgs& a,
                            cudaStream_t s) {
  cudaError_t e =
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kernel<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

#define CGB_DISPATCH_BS(KT, ...)                                                        \
  switch (a.block) {                                                                    \
    case 32: return launch_k(KT<32 __VA_ARGS__>, grid, 32, smem, a, s);                 \
    case 64: return launch_k(KT<64 __VA_ARGS__>, grid, 64, smem, a, s);                 \
    case 128: return launch_k(KT<128 __VA_ARGS__>, grid, 128, smem, a, s);              \
    case 256: return launch_k(KT<256 __VA_ARGS__>, grid, 256, smem, a, s);              \
    default: return cudaErrorInvalidValue;                                              \
  }

cudaError_t launch_eval(const SweepArgs& a, int grid, cudaStream_t s) {
  const size_t smem = smem_primal(a.t.sz_w, a.block);
  CGB_DISPATCH_BS(k_primal, , false)
}

cudaError_t launch_record(const SweepArgs& a, int grid, cudaStream_t s) {
  const size_t smem = smem_primal(a.t.sz_w, a.block);
  CGB_DISPATCH_BS(k_primal, , true)
}

cudaError_t launch_sp_forward(const SweepArgs& a, int grid, cudaStream_t s) {
  const size_t smem = smem_primal(a.t.sz_w, a.block);
  CGB_DISPATCH_BS(k_sp_forward)
}

cudaError_t launch_sp_reverse(const SweepArgs& a, int grid, cudaStream_t s) {
  const size_t smem = smem_primal(a.t.sz_w, a.block);
  CGB_DISPATCH_BS(k_sp_reverse)
}

cudaError_t launch_tangent(const SweepArgs& a, int grid_x, int grid_y, cudaStream_t s) {
  const int dw = a.block / 32;
  const size_t smem = smem_dir(a.t.sz_w, dw);
  const dim3 grid(grid_x, grid_y);
  switch (dw) {
    case 1: return launch_k(k_tangent<1>, grid, 32, smem, a, s);
    case 2: return launch_k(k_tangent<2>, grid, 64, smem, a, s);
    case 4: return launch_k(k_tangent<4>, grid, 128, smem, a, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_adjoint(const SweepArgs& a, int grid_x, int grid_y, cudaStream_t s) {
  const int dw = a.block / 32;
  const size_t smem = smem_dir(a.t.sz_w, dw);
  const dim3 grid(grid_x, grid_y);
  switch (dw) {
    case 1: return launch_k(k_adjoint<1>, grid, 32, smem, a, s);
    case 2: return launch_k(k_adjoint<2>, grid, 64, smem, a, s);
    case 4: return launch_k(k_adjoint<4>, grid, 128, smem, a, s);
    default: return cudaErrorInvalidValue;
  }
}

int occupancy_primal(int block, size_t smem) {
  int n = 0;
  cudaError_t e = cudaErrorInvalidValue;
  switch (block) {
    case 32:
      cudaFuncSetAttribute(k_primal<32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_primal<32, true>, 32, smem);
      break;
    case 64:
      cudaFuncSetAttribute(k_primal<64, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_primal<64, true>, 64, smem);
      break;
    case 128:
      cudaFuncSetAttribute(k_primal<128, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_primal<128, true>, 128, smem);
      break;
    case 256:
      cudaFuncSetAttribute(k_primal<256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_primal<256, true>, 256, smem);
      break;
  }
  return (e == cudaSuccess && n > 0) ? n : 1;
}

int occupancy_dir(size_t smem) {
  int n = 0;
  cudaFuncSetAttribute(k_adjoint<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adjoint<4>, 128, smem);
  return (e == cudaSuccess && n > 0) ? n : 1;
}

}  // namespace cgb
