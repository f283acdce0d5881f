// Tape-sweep kernels for sm_103a.
//
// The value and sparsity sweeps interpret the instruction stream, staged chunk by chunk
// (kChunk 8-byte words) from global memory into a two-slot shared-memory ring with TMA bulk
// copies (cp.async.bulk ... mbarrier::complete_tx) while the previous chunk is being
// interpreted; the warp-level derivative sweeps walk host-compiled keyed entry streams over the
// recorded partials (see "Derivative sweeps, warp-independent" below). Every thread of a CTA
// runs the same instruction on a different instance (or instance/direction pair), so the
// dispatch is warp-uniform and never diverges.
// The work vector lives in shared memory in slot-major order, w[slot*BS + thread]:
// consecutive lanes hit consecutive 8-byte words, so every work-vector access is
// bank-conflict free. Instance data in global memory is read and written through IoDesc
// strides, which covers both the instance-minor layout (coalesced) and the instance-major
// layout of CasADi's Map (casadi/core/map.cpp:150-153) without a separate transpose pass.
//
// Kernels:
//   k_primal<BS,false>  forward value sweep           SXFunction::eval (sx_function.cpp:110-124)
//   k_primal<BS,true>   values + recorded partials    (first half of the AD sweeps)
//   k_tangent<G,MB,IPT,K>  forward-mode directions    ad_forward, numeric
//                                                     (sx_function.cpp:1318-1364)
//   k_adjoint<G,MB,IPT>    adjoint directions         ad_reverse, numeric
//                                                     (sx_function.cpp:1454-1560)
//   k_sp_forward<BS>    bvec_t OR-propagation         sp_forward (sx_function.cpp:1657-1682)
//   k_sp_forward<BS,GW,true>  activity propagation    eval_activity (sx_function.cpp:1684-1718)
//   k_sp_reverse<BS>    bvec_t reverse propagation    sp_reverse (sx_function.cpp:1742-1782)
//
// Waits on the staging barriers are bounded: after ~1 s without completion a kernel sets
// kErrWaitTimeout in the tape's error word, waits (again bounded) for its own copies in
// flight and returns. No kernel traps.
#include <algorithm>

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
// GW: the work vector lives in global memory (a per-CTA block of a.wglob, L1/L2-cached)
// instead of shared memory, for tapes whose work vector does not fit or is worth trading for
// residency.
// The last sin/cos pair of a value or record sweep (dev_fun_pair, dev_fun_der_pair).
struct PairState {
  double s = 0.0, c = 0.0;
};

template <int BS, bool RECORD, bool GW = false>
__global__ void __launch_bounds__(BS) k_primal(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  u64* ring = reinterpret_cast<u64*>(smem);
  u64* bars = ring + 2 * kChunk;
  double* w = GW ? reinterpret_cast<double*>(a.wglob + blockIdx.x * a.wglob_stride)
                 : reinterpret_cast<double*>(smem + kHeaderBytes);
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
    PairState pair;
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
          if constexpr (RECORD) {
            const unsigned m = partial_mask(op);
            double d0 = 0.0, d1 = 0.0;
            const double f = dev_fun_der_pair(op, x, y, d0, d1, ins, pair.s, pair.c);
            if (m & 1u) {
              if (active) a.partials[((il >> 5) * a.t.n_partials + pidx) * 32 + (il & 31)] = d0;
              ++pidx;
            }
            if (m & 2u) {
              if (active) a.partials[((il >> 5) * a.t.n_partials + pidx) * 32 + (il & 31)] = d1;
              ++pidx;
            }
            w[A * BS + tid] = f;
          } else {
            w[A * BS + tid] = dev_fun_pair(op, x, y, ins, pair.s, pair.c);
          }
        }
      }
    });
    if (!ok) return;
  }
}

#include "sweeps_coop.cuh"

// ---------------------------------------------------------------------------------------------
// Plan-free adjoint sweep (the allocation-free entry point).
//
// The record sweep stores partials tile-major: for the 32-instance tile T of a wave,
// partial p of lane l is at partials[(T*P + p)*32 + l]. The partials an instruction chunk
// consumes for one tile are therefore one contiguous block. This CTA-level adjoint sweep
// stages each chunk, last first, with TMA bulk copies on one mbarrier (instruction words and
// partial block) and treats every instruction as active, so it needs no host-built plan and
// no plan memory. The regular derivative sweeps (warp-independent entry streams) follow
// further below.
// ---------------------------------------------------------------------------------------------
struct DirSmem {
  u64* ring;      // 2 x chunk instruction words
  double* pbuf;   // 2 x (2*chunk partials x 32 lanes)
  u64* bars;      // 2 mbarriers
  double* wd;     // sz_w x (32*DW) adjoints
};

__host__ __device__ __forceinline__ size_t dir_header_bytes(int ch) {
  return static_cast<size_t>(2 * ch) * sizeof(u64) + static_cast<size_t>(4 * ch * 32) * 8 +
         2 * sizeof(u64);
}

__device__ __forceinline__ DirSmem dir_smem(unsigned char* smem, int ch) {
  DirSmem s;
  s.ring = reinterpret_cast<u64*>(smem);
  s.pbuf = reinterpret_cast<double*>(smem + 2 * ch * sizeof(u64));
  s.bars = reinterpret_cast<u64*>(s.pbuf + 2 * (2 * ch * 32));
  s.wd = reinterpret_cast<double*>(s.bars + 2);
  return s;
}

__device__ __forceinline__ int chunk_p0(const SweepArgs& a, int c) {
  return __ldg(a.pofs + c * (a.chunk / kPofsGran));
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, u64* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Stage chunk c (instructions and the partial block of wave-local tile tl) into slot seq&1.
__device__ __forceinline__ void stage_dir(const SweepArgs& a, const DirSmem& s, unsigned seq,
                                          int c, long long tl) {
  const int ch = a.chunk;
  const int p0 = chunk_p0(a, c), p1 = chunk_p0(a, c + 1);
  const unsigned ibytes = ch * sizeof(u64);
  const unsigned pbytes = static_cast<unsigned>(p1 - p0) * 32u * sizeof(double);
  const unsigned slot = seq & 1u;
  u64* bar = s.bars + slot;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(ibytes + pbytes)
               : "memory");
  bulk_g2s(s.ring + slot * ch, a.t.code + static_cast<size_t>(c) * ch, ibytes, bar);
  if (pbytes)
    bulk_g2s(s.pbuf + slot * (2 * ch * 32), a.partials + (tl * a.t.n_partials + p0) * 32, pbytes,
             bar);
}

// Adjoint sweep over the 8-byte instruction stream (seed = w'[i0]; w'[i0] = 0;
// w'[i1] += d0*seed; w'[i2] += d1*seed, sx_function.cpp:1454-1560): every chunk, every
// instruction active, contributions always added to a zeroed adjoint; DW directions per CTA.
template <int DW>
__global__ void __launch_bounds__(32 * DW) k_adjoint_tape(const __grid_constant__ SweepArgs a) {
  constexpr int BS = 32 * DW;
  extern __shared__ __align__(128) unsigned char smem[];
  const DirSmem s = dir_smem(smem, a.chunk);
  double* wb = s.wd;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) stage_init(s.bars);
  __syncthreads();
  const int ngroups = (a.ndir + DW - 1) / DW;
  const int group = blockIdx.x % ngroups;
  const long long dir = static_cast<long long>(group) * DW + warp;
  const bool dir_ok = dir < a.ndir;
  const int ch = a.chunk;
  const int nlist = a.n_code / ch;
  const long long ntiles = (a.n + 31) / 32;
  const long long tstride = gridDim.x / ngroups;
  unsigned seq = 0;
  for (int q = 0; q < a.t.sz_w; ++q) wb[q * BS + tid] = 0.0;
  for (long long tile = blockIdx.x / ngroups; tile < ntiles; tile += tstride) {
    const long long il = tile * 32 + lane;
    const bool active = il < a.n && dir_ok;
    const long long ig = a.i_begin + il;
    if (active) {
      // input nonzeros whose adjoint is structurally zero (or never read) get a zero
      const int nz = a.t.n_absent_in;
      const int2* zl = a.t.absent_in;
      for (int k = 0; k < nz; ++k) {
        const int2 jk = __ldg(zl + k);
        const IoDesc& d = a.sens[jk.x];
        if (d.ptr) static_cast<double*>(d.ptr)[io_off(d, dir, jk.y, ig)] = 0.0;
      }
    }
    if (nlist == 0) continue;
    if (tid == 0) stage_dir(a, s, seq, nlist - 1, tile);
#pragma unroll 1
    for (int idx = nlist - 1; idx >= 0; --idx) {
      const bool more = idx > 0;
      if (tid == 0 && more) stage_dir(a, s, seq + 1, idx - 1, tile);
      const bool ok = stage_wait(s.bars, seq);
      if (!__syncthreads_and(ok)) {
        stage_abort(a.t, s.bars, seq, more);
        return;
      }
      const int c = idx;
      const u64* code = s.ring + (seq & 1u) * ch;
      const double* pb = s.pbuf + (seq & 1u) * (2 * ch * 32) + lane;
      int pl = chunk_p0(a, c + 1) - chunk_p0(a, c);
#pragma unroll 1
      for (int k = ch - 1; k >= 0; --k) {
        const u64 ins = code[k];
        const unsigned op = dec_op(ins), A = dec_a(ins), B = dec_b(ins), C = dec_c(ins);
        const unsigned m = dec_pmask(ins);
        const unsigned f = op == D_OUTPUT ? 32u
                           : (op == D_NOP ? 0u
                                          : 1u | (carries_d0(op) ? 2u : 0u) |
                                                (carries_d1(op) ? 4u : 0u));
        double d0 = 1.0, d1 = 0.0;
        if (m & 2u) d1 = pb[32 * --pl];
        if (m & 1u) d0 = pb[32 * --pl];
        if (op == D_OUTPUT) {
          const IoDesc& d = a.seed[A];
          if (d.ptr) {
            const double sd =
                active ? __ldg(static_cast<const double*>(d.ptr) + io_off(d, dir, C, ig)) : 0.0;
            wb[B * BS + tid] = (f & 8u) ? sd : __dadd_rn(wb[B * BS + tid], sd);
          }
          continue;
        }
        if (!(f & 1u)) continue;  // structurally zero adjoint
        if (op == D_INPUT) {
          const IoDesc& d = a.sens[B];
          if (active && d.ptr) static_cast<double*>(d.ptr)[io_off(d, dir, C, ig)] = wb[A * BS + tid];
          wb[A * BS + tid] = 0.0;
          continue;
        }
        if (op == D_CONST) {
          wb[A * BS + tid] = 0.0;
          continue;
        }
        const double seed = wb[A * BS + tid];
        wb[A * BS + tid] = 0.0;
        // a contribution d*seed is added with one fused multiply-add (one rounding)
        if (f & 2u) {
          double* w1 = wb + B * BS + tid;
          switch (op) {
            case D_ADD: case D_SUB: case D_ASSIGN: *w1 = __dadd_rn(*w1, seed); break;
            case D_NEG: *w1 = __dsub_rn(*w1, seed); break;
            case D_TWICE: *w1 = __dadd_rn(*w1, d_twice(seed)); break;
            default: *w1 = __fma_rn(d0, seed, *w1);
          }
        }
        if (f & 4u) {
          double* w2 = wb + C * BS + tid;
          switch (op) {
            case D_ADD: *w2 = __dadd_rn(*w2, seed); break;
            case D_SUB: *w2 = __dsub_rn(*w2, seed); break;
            case D_IF_ELSE_ZERO: *w2 = __dadd_rn(*w2, d1 == 0.0 ? 0.0 : seed); break;
            default: *w2 = __fma_rn(d1, seed, *w2);
          }
        }
      }
      __syncthreads();
      ++seq;
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Derivative sweeps, warp-independent.
//
// Each warp owns one (32-instance tile, direction) work item at a time and walks its own
// host-compiled entry stream: for the tangent sweep the stream of its direction (only the
// instructions whose derivative is structurally nonzero for that direction, plus outputs),
// for the adjoint sweep the one stream of instructions with a nonzero adjoint, last
// instruction first. Warps never wait for each other, so a sparse direction finishes early
// instead of waiting for a dense one. Entries and recorded partials are loaded straight from
// global memory (L2-resident, one coalesced 256-byte request per partial) and
// software-pipelined through registers: while group g computes, the entries of group g+1 and
// the partials they use (described by group g's entries, see the keyed streams in sweeps.cuh)
// are in flight. Two groups are unrolled per iteration, so the pipeline needs no register
// moves. Each entry is one jump-table dispatch on its key, whose case holds only the FP64
// operations and work-vector accesses that entry needs. Shared memory holds only the work
// vector, w[slot][lane], so as many warps fit as the work vector allows.
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ double& wreg(unsigned char* base, unsigned off) {
  return *reinterpret_cast<double*>(base + off);
}

// Meta word of the windowed tangent sweep's entries (k_tangent_win): bits 0-4 flags (1/2
// operand b/c carries a derivative), 5-8 kind, 9-10 recorded-partial mask, 11-31 index of the
// instruction's first recorded partial.
__host__ __device__ __forceinline__ unsigned ent_flags(unsigned m) { return m & 31u; }
__host__ __device__ __forceinline__ unsigned ent_kind(unsigned m) { return (m >> 5) & 15u; }
__host__ __device__ __forceinline__ unsigned ent_pmask(unsigned m) { return (m >> 9) & 3u; }
__host__ __device__ __forceinline__ unsigned ent_pk(unsigned m) { return m >> 11; }

// kNC: read-only path (partials written by an earlier launch); otherwise L2 loads that see the
// same kernel's stores.
template <bool kNC>
__device__ __forceinline__ double ld_partial(const double* p) {
  return kNC ? __ldg(p) : __ldcg(p);
}

// G: entries per software-pipeline group; MB: minimum resident CTAs per SM the register
// allocation must allow (1: unconstrained); IPT: 32-instance tiles per warp (each lane
// carries IPT instances of the same direction, whose FP64 chains are independent). The work
// vector is w[slot][j][lane]: byte offset slot*256*IPT + j*256 + lane*8.
template <int IPT>
__device__ __forceinline__ double& wj(unsigned char* wb, unsigned off, int j) {
  return wreg(wb, off * IPT + j * 256);
}

// Group gi of a keyed stream (0: the header, g+1: body group g).
template <int G>
__device__ __forceinline__ void load_grp(const uint4* st, int gi, uint4 (&E)[G]) {
  const uint4* p = st + gi * G;
#pragma unroll
  for (int i = 0; i < G; ++i) E[i] = __ldg(p + i);
}

// The partials group E describes (those of the next group) for IPT tiles, tile j's block at
// pt + j*tstride; tiles past the wave's end are not read. Registers of partials not loaded
// keep stale values that the entries' cases do not read.
template <bool kNC, int G, int IPT>
__device__ __forceinline__ void issue_partials(const uint4 (&E)[G], const double* pt,
                                               size_t tstride, const bool (&tok)[IPT],
                                               double (&P)[G][IPT], double (&Q)[G][IPT]) {
#pragma unroll
  for (int i = 0; i < G; ++i) {
    const unsigned w = E[i].w;
    const double* pp = pt + static_cast<size_t>(w >> kPiIndexShift) * 32;
    // Q's row: P's, or the next one (32 doubles on) when kPiQNext is set; the shift moves that
    // bit (bit 8 of w) onto the value 32 (bit 5)
    static_assert(kPiQNext << kPiShift == (32u << 3), "kPiQNext sits at bit 8 of the key word");
    const double* pq = pp + ((w >> 3) & 32u);
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
      if ((w & (kPiP << kPiShift)) && tok[j]) P[i][j] = ld_partial<kNC>(pp + j * tstride);
      if ((w & (kPiQ << kPiShift)) && tok[j]) Q[i][j] = ld_partial<kNC>(pq + j * tstride);
    }
  }
}

// Tangent of form F from the operand tangents a, b and the partials p, q.
template <int F>
__device__ __forceinline__ double tf_eval(double p, double q, double a, double b) {
  if constexpr (F == TF_PY) return __dmul_rn(p, a);
  else if constexpr (F == TF_QZ) return __dmul_rn(q, b);
  else if constexpr (F == TF_PYQZ) return __fma_rn(p, a, __dmul_rn(q, b));
  else if constexpr (F == TF_Y) return a;
  else if constexpr (F == TF_Z) return b;
  else if constexpr (F == TF_YQZ) return __dadd_rn(a, __dmul_rn(q, b));
  else if constexpr (F == TF_YZ) return __dadd_rn(a, b);
  else if constexpr (F == TF_NZ) return d_neg(b);
  else if constexpr (F == TF_YMZ) return __dsub_rn(a, b);
  else if constexpr (F == TF_NY) return d_neg(a);
  else if constexpr (F == TF_2Y) return d_twice(a);
  else return d_iszero(q) ? 0.0 : b;  // TF_IFZ
}

// Tangent of one direction of a mixed union-stream entry: instruction kind rk, flags fk
// (1/2: operand b/c carries a derivative), partials p (1 when d0 is not recorded) and q.
__device__ __forceinline__ double tan_mixed(unsigned rk, unsigned fk, double p, double q,
                                            double a, double b) {
  switch ((rk << 2) | fk) {
    case (LK_GEN << 2) | 1u: return __dmul_rn(p, a);
    case (LK_GEN << 2) | 2u: return __dmul_rn(q, b);
    case (LK_GEN << 2) | 3u: return __fma_rn(p, a, __dmul_rn(q, b));
    case (LK_ADD << 2) | 1u: case (LK_SUB << 2) | 1u: case (LK_ASSIGN << 2) | 1u: return a;
    case (LK_ADD << 2) | 2u: return b;
    case (LK_ADD << 2) | 3u: return __dadd_rn(a, b);
    case (LK_SUB << 2) | 2u: return d_neg(b);
    case (LK_SUB << 2) | 3u: return __dsub_rn(a, b);
    case (LK_NEG << 2) | 1u: return d_neg(a);
    case (LK_TWICE << 2) | 1u: return d_twice(a);
    case (LK_IFZ << 2) | 2u: return d_iszero(q) ? 0.0 : b;
    default: return 0.0;
  }
}

// Tangent entries of K > 1 directions: x bits 0-18 hold the destination (see k_tangent).
constexpr unsigned kTanXMask = (1u << 19) - 1;

// One group of tangent entries (IPT tiles, K directions dir0..): their keys in E, their
// partials in P/Q.
template <int G, int IPT, int K>
__device__ __forceinline__ void tan_group(const uint4 (&E)[G], const double (&P)[G][IPT],
                                          const double (&Q)[G][IPT], unsigned char* wb,
                                          const IoDesc* seed, const IoDesc* sens, bool identity,
                                          const bool (&active)[IPT], int dir0, int ndir,
                                          const long long (&ig)[IPT]) {
#define CGB_W(off, j, k) wj<IPT * K>(wb, (off), (j) * K + (k))
#define CGB_JK _Pragma("unroll") for (int j = 0; j < IPT; ++j) _Pragma("unroll") for (int k = 0; k < K; ++k)
#pragma unroll
  for (int i = 0; i < G; ++i) {
    const uint4 cur = E[i];
    const unsigned key = ent_key(cur.w);
    const unsigned xo = K > 1 ? (cur.x & kTanXMask) : cur.x;
    double r[IPT][K];
    switch (key) {
      case TK_OUT0:
      case TK_OUT: {
        const IoDesc& d = sens[xo];
        CGB_JK {
          if (dir0 + k < ndir && active[j] && d.ptr)
            static_cast<double*>(d.ptr)[io_off(d, dir0 + k, cur.z, ig[j])] =
                key == TK_OUT ? CGB_W(cur.y, j, k) : 0.0;
        }
        continue;
      }
      case TK_IN:
        if (identity) {
          CGB_JK r[j][k] = 1.0;
        } else {
          const IoDesc& d = seed[cur.y];
          CGB_JK r[j][k] = (active[j] && dir0 + k < ndir)
              ? __ldg(static_cast<const double*>(d.ptr) + io_off(d, dir0 + k, cur.z, ig[j]))
              : 0.0;
        }
        break;
#define CGB_TK_CASE(KEY, F)                                              \
  case KEY:                                                              \
    CGB_JK {                                                             \
      const double av = tf_uses_y(F) ? CGB_W(cur.y, j, k) : 0.0;         \
      const double bv = tf_uses_z(F) ? CGB_W(cur.z, j, k) : 0.0;         \
      r[j][k] = tf_eval<F>(P[i][j], Q[i][j], av, bv);                    \
    }                                                                    \
    break;
      CGB_TK_ARITH(CGB_TK_CASE)
#undef CGB_TK_CASE
      case TK_MIXED:
      case TK_MIXED + 1:
      case TK_MIXED + 2:
      case TK_MIXED + 3: {
        if (K == 1) continue;
        // directions of the group differ: one dispatch per direction
        const unsigned pm = key - TK_MIXED;
        const unsigned rk = (cur.x >> 19) & 15u;
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const unsigned fk = (cur.x >> (24 + 2 * k)) & 3u;
          if (rk == LK_OUTPUT) {
            const IoDesc& d = sens[xo];
#pragma unroll
            for (int j = 0; j < IPT; ++j)
              if (dir0 + k < ndir && active[j] && d.ptr)
                static_cast<double*>(d.ptr)[io_off(d, dir0 + k, cur.z, ig[j])] =
                    (fk & 1u) ? CGB_W(cur.y, j, k) : 0.0;
            continue;
          }
          if (!fk) continue;
          if (rk == LK_INPUT) {
#pragma unroll
            for (int j = 0; j < IPT; ++j) {
              double v = 1.0;
              if (!identity) {
                const IoDesc& d = seed[cur.y];
                v = (active[j] && dir0 + k < ndir)
                    ? __ldg(static_cast<const double*>(d.ptr) + io_off(d, dir0 + k, cur.z, ig[j]))
                    : 0.0;
              }
              CGB_W(xo, j, k) = v;
            }
            continue;
          }
#pragma unroll
          for (int j = 0; j < IPT; ++j) {
            const double a = (fk & 1u) ? CGB_W(cur.y, j, k) : 0.0;
            const double b = (fk & 2u) ? CGB_W(cur.z, j, k) : 0.0;
            CGB_W(xo, j, k) = tan_mixed(rk, fk, (pm & 1u) ? P[i][j] : 1.0,
                                        (pm & 2u) ? Q[i][j] : 0.0, a, b);
          }
        }
        continue;
      }
      default:
        continue;  // NOP padding
    }
    CGB_JK CGB_W(xo, j, k) = r[j][k];
  }
#undef CGB_JK
#undef CGB_W
}

// One tangent sweep by one warp over its keyed stream st (body of ngr groups of G, ngr even):
// IPT tiles (tile j's partials at pt + j*tstride), K directions dir0.. (the union stream of
// the K directions).
template <bool kNC, int G, int IPT, int K>
__device__ __forceinline__ void tangent_walk(const uint4* st, int ngr, const double* pt,
                                             size_t tstride, const bool (&tok)[IPT],
                                             unsigned char* wb, const IoDesc* seed,
                                             const IoDesc* sens, bool identity,
                                             const bool (&active)[IPT], int dir0, int ndir,
                                             const long long (&ig)[IPT]) {
  uint4 Ea[G], Eb[G];
  double Pa[G][IPT], Qa[G][IPT], Pb[G][IPT], Qb[G][IPT];
#pragma unroll
  for (int i = 0; i < G; ++i)
#pragma unroll
    for (int j = 0; j < IPT; ++j) Pa[i][j] = Qa[i][j] = Pb[i][j] = Qb[i][j] = 0.0;
  load_grp<G>(st, 0, Eb);  // the header: the first group's partials
  issue_partials<kNC, G, IPT>(Eb, pt, tstride, tok, Pa, Qa);
  load_grp<G>(st, 1, Ea);
#pragma unroll 1
  for (int g = 0; g < ngr; g += 2) {
    load_grp<G>(st, g + 2, Eb);
    issue_partials<kNC, G, IPT>(Ea, pt, tstride, tok, Pb, Qb);
    tan_group<G, IPT, K>(Ea, Pa, Qa, wb, seed, sens, identity, active, dir0, ndir, ig);
    load_grp<G>(st, g + 3, Ea);
    issue_partials<kNC, G, IPT>(Eb, pt, tstride, tok, Pa, Qa);
    tan_group<G, IPT, K>(Eb, Pb, Qb, wb, seed, sens, identity, active, dir0, ndir, ig);
  }
}

// Tangent sweep. A warp takes one work item (IPT tiles, K directions): the work vector holds
// IPT*K values per slot and lane, w[slot][j*K + k][lane]. With K > 1 the warp walks the
// union stream of its K directions: recorded partials and entries are loaded once for all K,
// and the K directions give independent FP64 chains. An entry whose flags are the same for
// every direction of the group is dispatched once ("uniform"); otherwise its kind is
// LK_MIXED and x carries the real kind (bits 19-22) and the flags of direction k (bits
// 24+2k, 25+2k), handled one direction at a time.

template <int G, int MB, int IPT, int K, bool GW = false>
__global__ void __launch_bounds__(32, MB) k_tangent(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  unsigned char* wb = (GW ? a.wglob + blockIdx.x * a.wglob_stride : smem) + lane * 8;
  const long long ntiles = (a.n + 31) / 32;
  const int ngroups = (a.ndir + K - 1) / K;
  const long long nwork = (ntiles + IPT - 1) / IPT * ngroups;
  const size_t tstride = static_cast<size_t>(a.t.n_partials) * 32;
  // Direction streams differ in length (a direction seeded late in the tape has little
  // work), so a fixed stride over the items leaves some CTAs with several times the work of
  // others. With a queue, a CTA takes its first item by index and every later one from the
  // counter, claimed before the current walk so the atomic's latency is hidden.
  long long work = blockIdx.x;
  while (work < nwork) {
    long long next = work + gridDim.x;
    if (a.queue) {
      unsigned long long q = 0;
      if (lane == 0) q = atomicAdd(a.queue, 1ull);
      next = static_cast<long long>(gridDim.x) +
             static_cast<long long>(__shfl_sync(0xffffffffu, q, 0));
    }
    const long long tg = work / ngroups;
    const int pos = static_cast<int>(work % ngroups);
    const int grp = a.gorder ? __ldg(a.gorder + pos) : pos;
    const int dir0 = grp * K;
    bool active[IPT], tok[IPT];
    long long ig[IPT];
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
      const long long tile = tg * IPT + j;
      const long long il = tile * 32 + lane;
      tok[j] = tile < ntiles;
      active[j] = il < a.n;
      ig[j] = a.i_begin + il;
    }
    const int2 se = __ldg(a.dchunks + grp);  // (first entry, entry count) of this group
    const uint4* st = a.dstream + se.x;
    const int ngr = se.y / G;
    const double* pt = a.partials + static_cast<size_t>(tg * IPT) * tstride + lane;
    tangent_walk<true, G, IPT, K>(st, ngr, pt, tstride, tok, wb, a.seed, a.sens,
                                  a.identity_seed != 0, active, dir0, a.ndir, ig);
    work = next;
  }
}

#include "sweeps_win.cuh"

#define CGB_J _Pragma("unroll") for (int j = 0; j < IPT; ++j)

// Adjoint contribution of form F into a slot holding w, from the entry's adjoint s and the
// operand's partial m.
template <int F>
__device__ __forceinline__ double cf_eval(double w, double m, double s) {
  if constexpr (F == CF_RF) return __dmul_rn(m, s);
  else if constexpr (F == CF_RA) return __fma_rn(m, s, w);
  else if constexpr (F == CF_UF) return s;
  else if constexpr (F == CF_UA) return __dadd_rn(w, s);
  else if constexpr (F == CF_MF) return d_neg(s);
  else if constexpr (F == CF_MA) return __dsub_rn(w, s);
  else if constexpr (F == CF_TF) return d_twice(s);
  else if constexpr (F == CF_TA) return __dadd_rn(w, d_twice(s));
  else if constexpr (F == CF_IF) return d_iszero(m) ? 0.0 : s;
  else return __dadd_rn(w, d_iszero(m) ? 0.0 : s);  // CF_IA
}

// One group of adjoint entries (IPT tiles, direction dir): keys in E, partials in P/Q. Every
// slot's first contribution (in sweep order) is assigned, so a slot is never read before it
// is written and the adjoint read by an entry needs no reset afterwards.
template <int G, int IPT>
__device__ __forceinline__ void adj_group(const uint4 (&E)[G], const double (&P)[G][IPT],
                                          const double (&Q)[G][IPT], unsigned char* wb,
                                          const IoDesc* seed, const IoDesc* sens,
                                          const bool (&active)[IPT], long long dir,
                                          const long long (&ig)[IPT]) {
#pragma unroll
  for (int i = 0; i < G; ++i) {
    const uint4 cur = E[i];
    switch (ent_key(cur.w)) {
      case AK_OUT_SET:
      case AK_OUT_ADD: {
        const IoDesc& d = seed[cur.x];
        CGB_J {
          const double sd = active[j]
              ? __ldg(static_cast<const double*>(d.ptr) + io_off(d, dir, cur.z, ig[j])) : 0.0;
          double& w = wj<IPT>(wb, cur.y, j);
          w = ent_key(cur.w) == AK_OUT_SET ? sd : __dadd_rn(w, sd);
        }
      } break;
      case AK_IN: {
        const IoDesc& d = sens[cur.y];
        CGB_J {
          if (active[j] && d.ptr)
            static_cast<double*>(d.ptr)[io_off(d, dir, cur.z, ig[j])] = wj<IPT>(wb, cur.x, j);
        }
      } break;
#define CGB_AK_CASE(KEY, BF, CF)                                     \
  case KEY:                                                          \
    CGB_J {                                                          \
      const double sd = wj<IPT>(wb, cur.x, j);                       \
      if constexpr (BF != CF_N) {                                    \
        double& w1 = wj<IPT>(wb, cur.y, j);                          \
        w1 = cf_eval<BF>(cf_reads(BF) ? w1 : 0.0, P[i][j], sd);      \
      }                                                              \
      if constexpr (CF != CF_N) {                                    \
        double& w2 = wj<IPT>(wb, cur.z, j);                          \
        w2 = cf_eval<CF>(cf_reads(CF) ? w2 : 0.0, Q[i][j], sd);      \
      }                                                              \
    }                                                                \
    break;
      CGB_AK_ARITH(CGB_AK_CASE)
#undef CGB_AK_CASE
      default:
        break;  // NOP padding
    }
  }
}

// One adjoint sweep of IPT 32-instance tiles by one warp: keyed stream st (body of ngr groups,
// ngr even, last instruction first), recorded partials at pt (lane-offset, first tile; tile j
// at pt + j*tstride), work vector at wb (lane-offset, w[slot][j][lane]).
template <bool kNC, int G, int IPT>
__device__ __forceinline__ void adjoint_walk(const uint4* st, int ngr, const double* pt,
                                             size_t tstride, const bool (&tok)[IPT],
                                             unsigned char* wb, const IoDesc* seed,
                                             const IoDesc* sens, const bool (&active)[IPT],
                                             long long dir, const long long (&ig)[IPT]) {
  uint4 Ea[G], Eb[G];
  double Pa[G][IPT], Qa[G][IPT], Pb[G][IPT], Qb[G][IPT];
#pragma unroll
  for (int i = 0; i < G; ++i)
#pragma unroll
    for (int j = 0; j < IPT; ++j) Pa[i][j] = Qa[i][j] = Pb[i][j] = Qb[i][j] = 0.0;
  load_grp<G>(st, 0, Eb);  // the header: the first group's partials
  issue_partials<kNC, G, IPT>(Eb, pt, tstride, tok, Pa, Qa);
  load_grp<G>(st, 1, Ea);
#pragma unroll 1
  for (int g = 0; g < ngr; g += 2) {
    load_grp<G>(st, g + 2, Eb);
    issue_partials<kNC, G, IPT>(Ea, pt, tstride, tok, Pb, Qb);
    adj_group<G, IPT>(Ea, Pa, Qa, wb, seed, sens, active, dir, ig);
    load_grp<G>(st, g + 3, Ea);
    issue_partials<kNC, G, IPT>(Eb, pt, tstride, tok, Pa, Qa);
    adj_group<G, IPT>(Eb, Pb, Qb, wb, seed, sens, active, dir, ig);
  }
}

// Adjoint sweep: a warp takes one work item (IPT tiles, one direction) at a time and walks the
// keyed adjoint stream over the tiles' recorded partials.
template <int G, int MB, int IPT, bool GW = false>
__global__ void __launch_bounds__(32, MB) k_adjoint(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  unsigned char* wb = (GW ? a.wglob + blockIdx.x * a.wglob_stride : smem) + lane * 8;
  const long long ntiles = (a.n + 31) / 32;
  const long long nwork = (ntiles + IPT - 1) / IPT * a.ndir;
  const size_t tstride = static_cast<size_t>(a.t.n_partials) * 32;
  const int2 se = __ldg(a.dchunks);
  const int ngr = se.y / G;
  const uint4* st = a.dstream + se.x;
  for (int q = 0; q < a.t.sz_w * IPT; ++q) wreg(wb, q * 256) = 0.0;
  for (long long work = blockIdx.x; work < nwork; work += gridDim.x) {
    const long long tg = work / a.ndir;
    const int dir = static_cast<int>(work % a.ndir);
    bool active[IPT], tok[IPT];
    long long ig[IPT];
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
      const long long tile = tg * IPT + j;
      const long long il = tile * 32 + lane;
      tok[j] = tile < ntiles;
      active[j] = il < a.n;
      ig[j] = a.i_begin + il;
      if (active[j]) {
        // input nonzeros whose adjoint is structurally zero (or never read) get a zero
        for (int k = 0; k < a.n_zero; ++k) {
          const int2 jk = __ldg(a.zero_in + k);
          const IoDesc& d = a.sens[jk.x];
          if (d.ptr) static_cast<double*>(d.ptr)[io_off(d, dir, jk.y, ig[j])] = 0.0;
        }
      }
    }
    const double* pt = a.partials + static_cast<size_t>(tg * IPT) * tstride + lane;
    adjoint_walk<true, G, IPT>(st, ngr, pt, tstride, tok, wb, a.seed, a.sens, active, dir, ig);
  }
}
#undef CGB_J

#include "sweeps_batch.cuh"

// ---------------------------------------------------------------------------------------------
// bvec_t sparsity sweeps (uint64 bit sets, 64 directions at once).
// ---------------------------------------------------------------------------------------------
// ACT: the activity sweep (SXFunction::eval_activity, sx_function.cpp:1684-1718) on the same
// walk: constants are active when nonzero, arithmetic results follow activity_of.
template <int BS, bool GW = false, bool ACT = false>
__global__ void __launch_bounds__(BS) k_sp_forward(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  u64* ring = reinterpret_cast<u64*>(smem);
  u64* bars = ring + 2 * kChunk;
  u64* w = GW ? reinterpret_cast<u64*>(a.wglob + blockIdx.x * a.wglob_stride)
              : reinterpret_cast<u64*>(smem + kHeaderBytes);
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
          w[A * BS + tid] = ACT && __ldg(a.t.consts + B) != 0.0 ? ~0ull : 0ull;
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
          if (ACT)
            w[A * BS + tid] = activity_of(op, is_binary(op), w[B * BS + tid], w[C * BS + tid]);
          else
            w[A * BS + tid] = w[B * BS + tid] | w[C * BS + tid];
      }
    });
    if (!ok) return;
  }
}

template <int BS, bool GW = false>
__global__ void __launch_bounds__(BS) k_sp_reverse(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  u64* ring = reinterpret_cast<u64*>(smem);
  u64* bars = ring + 2 * kChunk;
  u64* w = GW ? reinterpret_cast<u64*>(a.wglob + blockIdx.x * a.wglob_stride)
              : reinterpret_cast<u64*>(smem + kHeaderBytes);
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
size_t smem_lean(int sz_w, int dir_warps, int chunk) {
  (void)chunk;
  return static_cast<size_t>(sz_w > 0 ? sz_w : 1) * 32 * dir_warps * 8;
}

size_t smem_dir(int sz_w, int dir_warps, int chunk) {
  return dir_header_bytes(chunk) + static_cast<size_t>(sz_w > 0 ? sz_w : 1) * 32 * dir_warps * 8;
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
static int occ_of_k(K kernel, int block, size_t smem) {
  int n = 0;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, block, smem) != cudaSuccess)
    return 0;
  return n;
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

// With a.wglob set the global-work-vector instance runs (block kGwBlock, ring header only).
cudaError_t launch_eval(const SweepArgs& a, int grid, cudaStream_t s) {
  if (a.wglob) return launch_k(k_primal<kGwBlock, false, true>, grid, kGwBlock, kHeaderBytes, a, s);
  const size_t smem = smem_primal(a.t.sz_w, a.block);
  CGB_DISPATCH_BS(k_primal, , false)
}

cudaError_t launch_record(const SweepArgs& a, int grid, cudaStream_t s) {
  if (a.wglob) return launch_k(k_primal<kGwBlock, true, true>, grid, kGwBlock, kHeaderBytes, a, s);
  const size_t smem = smem_primal(a.t.sz_w, a.block);
  CGB_DISPATCH_BS(k_primal, , true)
}

cudaError_t launch_sp_forward(const SweepArgs& a, int grid, cudaStream_t s) {
  if (a.wglob) return launch_k(k_sp_forward<kGwBlock, true>, grid, kGwBlock, kHeaderBytes, a, s);
  const size_t smem = smem_primal(a.t.sz_w, a.block);
  CGB_DISPATCH_BS(k_sp_forward)
}

cudaError_t launch_activity(const SweepArgs& a, int grid, cudaStream_t s) {
  if (a.wglob)
    return launch_k(k_sp_forward<kGwBlock, true, true>, grid, kGwBlock, kHeaderBytes, a, s);
  const size_t smem = smem_primal(a.t.sz_w, a.block);
  CGB_DISPATCH_BS(k_sp_forward, , false, true)
}

size_t smem_coop(int lv_sz_w) { return static_cast<size_t>(lv_sz_w > 0 ? lv_sz_w : 1) * 32 * 8; }

cudaError_t launch_coop(const SweepArgs& a, bool record, int grid, cudaStream_t s) {
  if (a.block < 32 || a.block > kCoopMaxThreads || a.block % 32) return cudaErrorInvalidValue;
  if (a.wglob)
    return record ? launch_k(k_coop<true, true>, grid, a.block, 0, a, s)
                  : launch_k(k_coop<false, true>, grid, a.block, 0, a, s);
  const size_t smem = smem_coop(a.t.lv_sz_w);
  return record ? launch_k(k_coop<true, false>, grid, a.block, smem, a, s)
                : launch_k(k_coop<false, false>, grid, a.block, smem, a, s);
}

size_t smem_tangent_coop(int lv_sz_w, bool global) {
  const size_t slots = static_cast<size_t>(lv_sz_w > 0 ? lv_sz_w : 1);
  return (global ? 0 : slots * 256) + ((slots + 15) / 16) * 16;
}

cudaError_t launch_tangent_coop(const SweepArgs& a, int grid, cudaStream_t s) {
  if (a.block != kCoopTanThreads) return cudaErrorInvalidValue;
  const size_t smem = smem_tangent_coop(a.t.lv_sz_w, a.wglob != nullptr);
  return a.wglob ? launch_k(k_tangent_coop<kCoopTanQ, true>, grid, a.block, smem, a, s)
                 : launch_k(k_tangent_coop<kCoopTanQ, false>, grid, a.block, smem, a, s);
}

int occupancy_tangent_coop(size_t smem, bool global) {
  return global ? occ_of_k(k_tangent_coop<kCoopTanQ, true>, kCoopTanThreads, smem)
                : occ_of_k(k_tangent_coop<kCoopTanQ, false>, kCoopTanThreads, smem);
}

cudaError_t launch_coop_sp(const SweepArgs& a, bool reverse, int grid, cudaStream_t s) {
  if (a.block < 32 || a.block > kCoopMaxThreads || a.block % 32) return cudaErrorInvalidValue;
  const size_t smem = smem_coop(reverse ? a.t.rlv_sz_w : a.t.lv_sz_w);
  return reverse ? launch_k(k_coop_sp<true>, grid, a.block, smem, a, s)
                 : launch_k(k_coop_sp<false>, grid, a.block, smem, a, s);
}

int occupancy_coop_sp(int threads, size_t smem) {
  return occ_of_k(k_coop_sp<false>, threads, smem);
}

cudaError_t launch_adjoint_coop(const SweepArgs& a, int grid, cudaStream_t s) {
  if (a.block != kCoopTanThreads) return cudaErrorInvalidValue;
  return launch_k(k_adjoint_coop<kCoopTanQ>, grid, a.block,
                  smem_tangent_coop(a.t.rlv_sz_w, false), a, s);
}

int occupancy_adjoint_coop(size_t smem) {
  return occ_of_k(k_adjoint_coop<kCoopTanQ>, kCoopTanThreads, smem);
}

int occupancy_coop(int threads, size_t smem, bool global) {
  return global ? occ_of_k(k_coop<true, true>, threads, 0)
                : occ_of_k(k_coop<true, false>, threads, smem);
}

cudaError_t launch_sp_reverse(const SweepArgs& a, int grid, cudaStream_t s) {
  if (a.wglob) return launch_k(k_sp_reverse<kGwBlock, true>, grid, kGwBlock, kHeaderBytes, a, s);
  const size_t smem = smem_primal(a.t.sz_w, a.block);
  CGB_DISPATCH_BS(k_sp_reverse)
}

int occupancy_gw_primal(bool record) {
  return record ? occ_of_k(k_primal<kGwBlock, true, true>, kGwBlock, kHeaderBytes)
                : occ_of_k(k_primal<kGwBlock, false, true>, kGwBlock, kHeaderBytes);
}
int occupancy_gw_sp() { return occ_of_k(k_sp_reverse<kGwBlock, true>, kGwBlock, kHeaderBytes); }

// Derivative-sweep variants: G entries per software-pipeline group, MB minimum CTAs per SM
// (register cap), IPT tiles per warp and, for the tangent sweep, K directions per warp.
// CGB_TAN_VARIANTS(X) lists X(variant, G, MB, IPT, K); CGB_ADJ_VARIANTS(X) X(variant, G, MB, IPT).
#define CGB_TAN_VARIANTS(X)    \
  X(TV_G2_R80, 2, 24, 1, 1)    \
  X(TV_G2_R64, 2, 32, 1, 1)    \
  X(TV_G1_R64, 1, 32, 1, 1)    \
  X(TV_G2_K2, 2, 16, 1, 2)     \
  X(TV_G2_K4, 2, 8, 1, 4)      \
  X(TV_G4_R128, 4, 16, 1, 1)   \
  X(TV_G8_R256, 8, 8, 1, 1)
#define CGB_ADJ_VARIANTS(X)    \
  X(AV_G2_R80, 2, 24, 1)       \
  X(AV_G1_R64, 1, 32, 1)       \
  X(AV_G2_R64, 2, 32, 1)       \
  X(AV_G2_I2_R128, 2, 16, 2)   \
  X(AV_G4_R128, 4, 16, 1)      \
  X(AV_G8_R256, 8, 8, 1)

void tan_variant_shape(int variant, int* ipt, int* k) {
  *ipt = 1;
  *k = 1;
  switch (variant) {
#define CGB_SHAPE(V, G, MB, IPT, K) \
  case V: *ipt = IPT; *k = K; break;
    CGB_TAN_VARIANTS(CGB_SHAPE)
#undef CGB_SHAPE
    default: break;
  }
}

int adj_variant_ipt(int variant) {
  switch (variant) {
#define CGB_IPT(V, G, MB, IPT) case V: return IPT;
    CGB_ADJ_VARIANTS(CGB_IPT)
#undef CGB_IPT
    default: return 1;
  }
}

// The launch's arguments with the keyed streams laid out for group size G.
SweepArgs with_group(const SweepArgs& a, int g) {
  SweepArgs b = a;
  b.dstream = a.dstreams[group_slot(g)];
  b.dchunks = a.dchunkss[group_slot(g)];
  return b;
}

int tan_variant_group(int variant) {
  switch (variant) {
#define CGB_G(V, G, MB, IPT, K) case V: return G;
    CGB_TAN_VARIANTS(CGB_G)
#undef CGB_G
    default: return 2;
  }
}

int adj_variant_group(int variant) {
  switch (variant) {
#define CGB_G(V, G, MB, IPT) case V: return G;
    CGB_ADJ_VARIANTS(CGB_G)
#undef CGB_G
    default: return 2;
  }
}

cudaError_t launch_tangent(const SweepArgs& a, int grid, int variant, cudaStream_t s) {
  if (a.wglob)
    return launch_k(k_tangent<2, 32, 1, 1, true>, dim3(grid), 32, 0, with_group(a, 2), s);
  switch (variant) {
#define CGB_LAUNCH(V, G, MB, IPT, K)                                                          \
  case V:                                                                                     \
    return launch_k(k_tangent<G, MB, IPT, K>, dim3(grid), 32, smem_lean(a.t.sz_w, IPT * K, 0), \
                    with_group(a, G), s);
    CGB_TAN_VARIANTS(CGB_LAUNCH)
#undef CGB_LAUNCH
    default: return cudaErrorInvalidValue;
  }
}

size_t smem_tangent_win(int sz_w, int dirs, int stages, int rows, int ents) {
  return kWinBarBytes + static_cast<size_t>(stages) * (static_cast<size_t>(rows) * 256 +
                                                       static_cast<size_t>(ents) * 16) +
         static_cast<size_t>(dirs) * (sz_w > 0 ? sz_w : 1) * 256;
}

cudaError_t launch_tangent_win(const SweepArgs& a, int grid, cudaStream_t s) {
  if (a.win_dirs < 1 || a.win_dirs > kWinMaxDirs || a.win_stages < 2 ||
      a.win_stages > kWinBarBytes / 16 || a.win_n < 1)
    return cudaErrorInvalidValue;
  const size_t smem =
      smem_tangent_win(a.t.sz_w, a.win_dirs, a.win_stages, a.win_rows, a.win_ents);
  return launch_k(k_tangent_win, dim3(grid), (a.win_dirs + 1) * 32, smem, a, s);
}

cudaError_t launch_adjoint(const SweepArgs& a, int grid, int variant, cudaStream_t s) {
  if (a.wglob)
    return launch_k(k_adjoint<2, 32, 1, true>, dim3(grid), 32, 0, with_group(a, 2), s);
  switch (variant) {
#define CGB_LAUNCH(V, G, MB, IPT)                                                       \
  case V:                                                                               \
    return launch_k(k_adjoint<G, MB, IPT>, dim3(grid), 32, smem_lean(a.t.sz_w, IPT, 0), \
                    with_group(a, G), s);
    CGB_ADJ_VARIANTS(CGB_LAUNCH)
#undef CGB_LAUNCH
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_adjoint_dense(const SweepArgs& a, int grid, cudaStream_t s) {
  const size_t smem = smem_dir(a.t.sz_w, a.block / 32, a.chunk);
  switch (a.block / 32) {
    case 1: return launch_k(k_adjoint_tape<1>, dim3(grid), 32, smem, a, s);
    case 2: return launch_k(k_adjoint_tape<2>, dim3(grid), 64, smem, a, s);
    case 4: return launch_k(k_adjoint_tape<4>, dim3(grid), 128, smem, a, s);
    case 6: return launch_k(k_adjoint_tape<6>, dim3(grid), 192, smem, a, s);
    case 8: return launch_k(k_adjoint_tape<8>, dim3(grid), 256, smem, a, s);
    default: return cudaErrorInvalidValue;
  }
}

// Gather of rows: dst[e*ld + i] = src[src_row[e]*ld + i] (recovery of sparse Jacobian and
// Hessian nonzeros from colour-compressed products; HBM-bound, coalesced over instances).
__global__ void __launch_bounds__(256) k_gather(long long n, long long ld, int count,
                                                const long long* __restrict__ src_row,
                                                const double* __restrict__ src,
                                                double* __restrict__ dst) {
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int e = blockIdx.y; e < count; e += gridDim.y)
    dst[static_cast<long long>(e) * ld + i] = __ldg(src + __ldg(src_row + e) * ld + i);
}

cudaError_t launch_gather(long long n, long long ld, int count, const long long* src_row,
                          const double* src, double* dst, cudaStream_t s) {
  const long long bx = (n + 255) / 256;
  if (bx > 0x7fffffffll) return cudaErrorInvalidValue;
  dim3 grid(static_cast<unsigned>(bx), static_cast<unsigned>(std::min(count, 65535)));
  k_gather<<<grid, 256, 0, s>>>(n, ld, count, src_row, src, dst);
  return cudaGetLastError();
}

cudaError_t launch_batch(const BatchArgs& b, int grid, size_t smem, bool split, bool gw,
                         cudaStream_t s) {
  // the attribute is raised once to the device maximum, so a captured graph never depends on
  // a later call lowering it
  static const cudaError_t set0 = cudaFuncSetAttribute(
      k_batch<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_optin());
  static const cudaError_t set1 = cudaFuncSetAttribute(
      k_batch<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_optin());
  if (set0 != cudaSuccess) return set0;
  if (set1 != cudaSuccess) return set1;
  if (smem > static_cast<size_t>(max_smem_optin())) return cudaErrorInvalidValue;
  if (gw) {
    if (split)
      k_batch<true, true><<<grid, 32, 0, s>>>(b);
    else
      k_batch<false, true><<<grid, 32, 0, s>>>(b);
  } else if (split) {
    k_batch<true, false><<<grid, 32, smem, s>>>(b);
  } else {
    k_batch<false, false><<<grid, 32, smem, s>>>(b);
  }
  return cudaGetLastError();
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

template <class K>
static int occ_of(K kernel, int block, size_t smem) {
  int n = 0;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, block, smem) != cudaSuccess)
    return 0;
  return n;
}

int occupancy_batch(size_t smem, bool split, bool gw) {
  if (gw) return split ? occ_of(k_batch<true, true>, 32, 0) : occ_of(k_batch<false, true>, 32, 0);
  int n = 0;
  if (split) {
    if (cudaFuncSetAttribute(k_batch<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             max_smem_optin()) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<true, false>, 32, smem) !=
            cudaSuccess)
      return 0;
  } else {
    if (cudaFuncSetAttribute(k_batch<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             max_smem_optin()) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<false, false>, 32, smem) !=
            cudaSuccess)
      return 0;
  }
  return n;
}

int occupancy_dense(int dir_warps, size_t smem) {
  switch (dir_warps) {
    case 1: return occ_of(k_adjoint_tape<1>, 32, smem);
    case 2: return occ_of(k_adjoint_tape<2>, 64, smem);
    case 4: return occ_of(k_adjoint_tape<4>, 128, smem);
    case 6: return occ_of(k_adjoint_tape<6>, 192, smem);
    case 8: return occ_of(k_adjoint_tape<8>, 256, smem);
    default: return 0;
  }
}

int occupancy_gw_dir(bool adjoint) {
  return adjoint ? occ_of(k_adjoint<2, 32, 1, true>, 32, 0) : occ_of(k_tangent<2, 32, 1, 1, true>, 32, 0);
}

int occupancy_dir(int variant, bool adjoint, size_t smem) {
  if (adjoint) {
    switch (variant) {
#define CGB_OCC(V, G, MB, IPT) \
  case V: return occ_of(k_adjoint<G, MB, IPT>, 32, smem);
      CGB_ADJ_VARIANTS(CGB_OCC)
#undef CGB_OCC
      default: return 0;
    }
  }
  switch (variant) {
#define CGB_OCC(V, G, MB, IPT, K) \
  case V: return occ_of(k_tangent<G, MB, IPT, K>, 32, smem);
    CGB_TAN_VARIANTS(CGB_OCC)
#undef CGB_OCC
    default: return 0;
  }
}

}  // namespace cgb
