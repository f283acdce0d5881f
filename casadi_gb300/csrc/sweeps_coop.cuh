// Cooperative (level-scheduled) sweeps.
//
// Part of the sweeps.cu translation unit (included where it stands): it uses that file's
// staging, decoding and I/O helpers and is not compiled on its own.
#pragma once

// ---------------------------------------------------------------------------------------------
// Cooperative value / record sweep for launches with few instances.
//
// One 32-instance tile per CTA (lane = instance) and several warps per CTA: the host's level
// schedule groups the tape into levels of independent instructions; the warps of the CTA split
// each level between them and meet at a barrier before the next, so a tile's sweep advances
// by a whole level of independent instructions per step instead of one instruction. Each
// instruction is the same operation on the same operand values as in the sequential sweep
// (identical bits), and writes its partials at its index of the sequential order.
// ---------------------------------------------------------------------------------------------
template <bool RECORD, bool GW>
__global__ void __launch_bounds__(kCoopMaxThreads) k_coop(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  double* w = GW ? reinterpret_cast<double*>(a.wglob + blockIdx.x * a.wglob_stride)
                 : reinterpret_cast<double*>(smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const long long ntiles = (a.n + 31) / 32;
  const int nl = a.t.n_levels;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long il = tile * 32 + lane;
    const bool active = il < a.n;
    const long long ig = a.i_begin + il;
    double* pt = RECORD ? a.partials + static_cast<size_t>(tile) * a.t.n_partials * 32 + lane
                        : nullptr;
    int end = __ldg(a.t.lbegin);
    for (int l = 0; l < nl; ++l) {
      const int beg = end;
      end = __ldg(a.t.lbegin + l + 1);
      for (int i = beg + warp; i < end; i += nw) {
        const u64 ins = __ldg(a.t.lcode + i);
        const unsigned op = dec_op(ins), A = dec_a(ins), B = dec_b(ins), C = dec_c(ins);
        switch (op) {
          case D_CONST:
            w[A * 32 + lane] = __ldg(a.t.consts + B);
            break;
          case D_INPUT: {
            const IoDesc& d = a.in[B];
            double v = 0.0;
            if (active && d.ptr) v = __ldg(static_cast<const double*>(d.ptr) + io_off(d, 0, C, ig));
            w[A * 32 + lane] = v;
          } break;
          case D_OUTPUT: {
            const IoDesc& d = a.out[A];
            if (active && d.ptr) static_cast<double*>(d.ptr)[io_off(d, 0, C, ig)] = w[B * 32 + lane];
          } break;
          default: {
            const double x = w[B * 32 + lane], y = w[C * 32 + lane];
            if (RECORD) {
              const unsigned m = partial_mask(op);
              double d0 = 0.0, d1 = 0.0;
              const double f = dev_fun_der(op, x, y, d0, d1);
              if (m && active) {
                const size_t p = static_cast<size_t>(__ldg(a.t.lpidx + i));
                if (m & 1u) pt[p * 32] = d0;
                if (m & 2u) pt[(p + (m & 1u)) * 32] = d1;
              }
              w[A * 32 + lane] = f;
            } else {
              w[A * 32 + lane] = dev_fun(op, x, y);
            }
          }
        }
      }
      __syncthreads();
    }
  }
}

// Cooperative bvec_t sparsity sweeps (SXFunction::sp_forward / sp_reverse): the value
// sweep's level walk with OR instead of arithmetic; the reverse sweep walks the reverse level
// schedule last level first (no two users of a value in one level, so no two instructions of
// a level OR into one slot). OR does not depend on order: the same bits as the sequential
// sweeps.
template <bool REV>
__global__ void __launch_bounds__(kCoopMaxThreads) k_coop_sp(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  u64* w = reinterpret_cast<u64*>(smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const long long ntiles = (a.n + 31) / 32;
  const int nl = REV ? a.t.n_rlevels : a.t.n_levels;
  const u64* code = REV ? a.t.rcode : a.t.lcode;
  const int* lb = REV ? a.t.rbegin : a.t.lbegin;
  const int lv = REV ? a.t.rlv_sz_w : a.t.lv_sz_w;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long il = tile * 32 + lane;
    const bool active = il < a.n;
    const long long ig = a.i_begin + il;
    if (REV) {
      for (int k = warp; k < lv; k += nw) w[k * 32 + lane] = 0;
      __syncthreads();
    }
    for (int step = 0; step < nl; ++step) {
      const int l = REV ? nl - 1 - step : step;
      const int beg = __ldg(lb + l), end = __ldg(lb + l + 1);
      for (int i = beg + warp; i < end; i += nw) {
        const u64 ins = __ldg(code + i);
        const unsigned op = dec_op(ins), A = dec_a(ins), B = dec_b(ins), C = dec_c(ins);
        switch (op) {
          case D_CONST:
            w[A * 32 + lane] = 0;
            break;
          case D_INPUT: {
            const IoDesc& d = a.in[B];
            if (REV) {
              if (active && d.ptr) static_cast<u64*>(d.ptr)[io_off(d, 0, C, ig)] |= w[A * 32 + lane];
              w[A * 32 + lane] = 0;
            } else {
              u64 v = 0;
              if (active && d.ptr) v = __ldg(static_cast<const u64*>(d.ptr) + io_off(d, 0, C, ig));
              w[A * 32 + lane] = v;
            }
          } break;
          case D_OUTPUT: {
            const IoDesc& d = a.out[A];
            if (REV) {
              if (active && d.ptr) {
                u64* p = static_cast<u64*>(d.ptr) + io_off(d, 0, C, ig);
                w[B * 32 + lane] |= *p;
                *p = 0;
              }
            } else if (active && d.ptr) {
              static_cast<u64*>(d.ptr)[io_off(d, 0, C, ig)] = w[B * 32 + lane];
            }
          } break;
          default:
            if (REV) {
              const u64 seed = w[A * 32 + lane];
              w[A * 32 + lane] = 0;
              w[B * 32 + lane] |= seed;
              w[C * 32 + lane] |= seed;
            } else {
              w[A * 32 + lane] = w[B * 32 + lane] | w[C * 32 + lane];
            }
        }
      }
      __syncthreads();
    }
  }
}

// Cooperative tangent sweep: one CTA per (tile, direction) item runs the level schedule of
// the forward-mode sweep over the partials the record sweep stored. Activity is structural
// (the same for every lane), so it is kept per slot in shared memory (act) and an instruction
// whose operands carry no derivative is skipped exactly where the sequential sweep's entry
// stream has no entry; the arithmetic of every case is the sequential sweep's (same
// operations, same order), so the sensitivities are the same bits. Each warp takes up to Q
// instructions of a level at a time, loading all their operands and partials before any
// arithmetic so the loads overlap.
__device__ __forceinline__ bool is_arith(unsigned op) {
  return op < D_CONST || (op >= D_ERFINV && op != D_NOP);
}

template <int Q, bool GW>
__global__ void __launch_bounds__(kCoopTanThreads)
    k_tangent_coop(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int lv = a.t.lv_sz_w;
  double* wd = GW ? reinterpret_cast<double*>(a.wglob + blockIdx.x * a.wglob_stride)
                  : reinterpret_cast<double*>(smem);
  unsigned char* act = GW ? smem : smem + static_cast<size_t>(lv) * 256;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const long long ntiles = (a.n + 31) / 32;
  const long long items = ntiles * a.ndir;
  const int nl = a.t.n_levels;
  const u64 nop = static_cast<u64>(D_NOP);
  for (long long item = blockIdx.x; item < items; item += gridDim.x) {
    const long long tile = item / a.ndir;
    const int dir = static_cast<int>(item - tile * a.ndir);
    const long long il = tile * 32 + lane;
    const bool active = il < a.n;
    const long long ig = a.i_begin + il;
    const double* pt = a.partials + static_cast<size_t>(tile) * a.t.n_partials * 32 + lane;
    int end = __ldg(a.t.lbegin);
    for (int l = 0; l < nl; ++l) {
      const int beg = end;
      end = __ldg(a.t.lbegin + l + 1);
      for (int base = beg + warp; base < end; base += Q * nw) {
        u64 ins[Q];
        unsigned fl[Q];
        double p0[Q], p1[Q], xb[Q], xc[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int i = base + q * nw;
          ins[q] = i < end ? __ldg(a.t.lcode + i) : nop;
          fl[q] = 0;
          p0[q] = 1.0;
          p1[q] = 0.0;
          xb[q] = 0.0;
          xc[q] = 0.0;
          const unsigned op = dec_op(ins[q]), B = dec_b(ins[q]), C = dec_c(ins[q]);
          if (is_arith(op)) {
            const bool fb = act[B] && carries_d0(op);
            const bool fc = act[C] && carries_d1(op);
            fl[q] = (fb ? 1u : 0u) | (fc ? 2u : 0u);
            const unsigned m = partial_mask(op);
            if (m & fl[q]) {
              const size_t pk = static_cast<size_t>(__ldg(a.t.lpidx + i));
              if (m & fl[q] & 1u) p0[q] = __ldg(pt + pk * 32);
              if (m & fl[q] & 2u) p1[q] = __ldg(pt + (pk + (m & 1u)) * 32);
            }
            if (fb) xb[q] = wd[B * 32 + lane];
            if (fc) xc[q] = wd[C * 32 + lane];
          } else if (op == D_OUTPUT) {
            fl[q] = act[B] ? 1u : 0u;
            if (fl[q]) xb[q] = wd[B * 32 + lane];
          }
        }
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const unsigned op = dec_op(ins[q]), A = dec_a(ins[q]), B = dec_b(ins[q]),
                         C = dec_c(ins[q]);
          const unsigned f = fl[q];
          if (op == D_NOP) continue;
          if (op == D_CONST) {
            if (lane == 0) act[A] = 0;
            continue;
          }
          if (op == D_INPUT) {
            bool on;
            double v = 0.0;
            if (a.identity_seed) {
              const int flat = a.in_off[B] + static_cast<int>(C);
              on = (a.dirmap ? __ldg(a.dirmap + flat) : flat) == dir;
              v = 1.0;
            } else {
              const IoDesc& d = a.seed[B];
              on = d.ptr != nullptr;
              if (on && active)
                v = __ldg(static_cast<const double*>(d.ptr) + io_off(d, dir, C, ig));
            }
            if (on) wd[A * 32 + lane] = v;
            if (lane == 0) act[A] = on ? 1 : 0;
            continue;
          }
          if (op == D_OUTPUT) {
            const IoDesc& d = a.sens[A];
            if (active && d.ptr)
              static_cast<double*>(d.ptr)[io_off(d, dir, C, ig)] = f ? xb[q] : 0.0;
            continue;
          }
          if (!f) {
            if (lane == 0) act[A] = 0;
            continue;
          }
          double r;
          switch (op) {
            case D_ADD:
              r = f == 3u ? __dadd_rn(xb[q], xc[q]) : (f == 1u ? xb[q] : xc[q]);
              break;
            case D_SUB:
              r = f == 3u ? __dsub_rn(xb[q], xc[q]) : (f == 1u ? xb[q] : d_neg(xc[q]));
              break;
            case D_NEG:
              r = d_neg(xb[q]);
              break;
            case D_TWICE:
              r = d_twice(xb[q]);
              break;
            case D_ASSIGN:
              r = xb[q];
              break;
            case D_IF_ELSE_ZERO:
              r = d_iszero(p1[q]) ? 0.0 : xc[q];
              break;
            default:
              r = f == 3u ? __fma_rn(p0[q], xb[q], __dmul_rn(p1[q], xc[q]))
                          : (f == 1u ? __dmul_rn(p0[q], xb[q]) : __dmul_rn(p1[q], xc[q]));
          }
          wd[A * 32 + lane] = r;
          if (lane == 0) act[A] = 1;
        }
      }
      __syncthreads();
    }
  }
}

// Cooperative adjoint sweep: one CTA per (tile, direction) item walks the reverse level
// schedule (whose levels also keep the users of every value in order, so each adjoint
// receives its contributions in the order of the sequential sweep, last user first). The
// activity of each slot's adjoint lives in shared memory (act) and decides, like the
// sequential sweep's plan, whether a contribution is the first (assigned) or added; the
// arithmetic of every case is the sequential sweep's, so the sensitivities are the same bits.
template <int Q>
__global__ void __launch_bounds__(kCoopTanThreads)
    k_adjoint_coop(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int lv = a.t.rlv_sz_w;
  double* wd = reinterpret_cast<double*>(smem);
  unsigned char* act = smem + static_cast<size_t>(lv) * 256;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const long long ntiles = (a.n + 31) / 32;
  const long long items = ntiles * a.ndir;
  const int nl = a.t.n_rlevels;
  const u64 nop = static_cast<u64>(D_NOP);
  for (long long item = blockIdx.x; item < items; item += gridDim.x) {
    const long long tile = item / a.ndir;
    const int dir = static_cast<int>(item - tile * a.ndir);
    const long long il = tile * 32 + lane;
    const bool active = il < a.n;
    const long long ig = a.i_begin + il;
    const double* pt = a.partials + static_cast<size_t>(tile) * a.t.n_partials * 32 + lane;
    for (int k = threadIdx.x; k < lv; k += blockDim.x) act[k] = 0;
    for (int k = warp; k < a.n_zero; k += nw) {
      const int2 jk = __ldg(a.zero_in + k);
      const IoDesc& d = a.sens[jk.x];
      if (active && d.ptr) static_cast<double*>(d.ptr)[io_off(d, dir, jk.y, ig)] = 0.0;
    }
    __syncthreads();
    int beg = __ldg(a.t.rbegin + nl);
    for (int l = nl - 1; l >= 0; --l) {
      const int end = beg;
      beg = __ldg(a.t.rbegin + l);
      for (int base = beg + warp; base < end; base += Q * nw) {
        u64 ins[Q];
        unsigned fl[Q];  // 1 result active, 2/4 b/c receives, 8/16 first to b/c
        double sd[Q], p0[Q], p1[Q], ob[Q], oc[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int i = base + q * nw;
          ins[q] = i < end ? __ldg(a.t.rcode + i) : nop;
          fl[q] = 0;
          sd[q] = 0.0;
          p0[q] = 1.0;
          p1[q] = 0.0;
          ob[q] = 0.0;
          oc[q] = 0.0;
          const unsigned op = dec_op(ins[q]), A = dec_a(ins[q]), B = dec_b(ins[q]),
                         C = dec_c(ins[q]);
          if (op == D_OUTPUT) {
            const IoDesc& d = a.seed[A];
            if (d.ptr) {
              fl[q] = act[B] ? 1u : 9u;
              if (active) sd[q] = __ldg(static_cast<const double*>(d.ptr) + io_off(d, dir, C, ig));
              if (!(fl[q] & 8u)) ob[q] = wd[B * 32 + lane];
            }
          } else if (op == D_INPUT || op == D_CONST) {
            if (act[A]) {
              fl[q] = 1u;
              if (op == D_INPUT) sd[q] = wd[A * 32 + lane];
            }
          } else if (op != D_NOP && act[A]) {
            unsigned f = 1u;
            sd[q] = wd[A * 32 + lane];
            const bool cb = carries_d0(op), cc = carries_d1(op);
            if (cb) {
              f |= 2u | (act[B] ? 0u : 8u);
              if (!(f & 8u)) ob[q] = wd[B * 32 + lane];
            }
            if (cc) {
              // c == b: c's contribution follows b's, which has just activated the slot
              const bool first_c = (cb && C == B) ? false : !act[C];
              f |= 4u | (first_c ? 16u : 0u);
              if (!first_c && !(cb && C == B)) oc[q] = wd[C * 32 + lane];
            }
            fl[q] = f;
            const unsigned m = partial_mask(op);
            const unsigned use = (f >> 1) & 3u;
            if (m & use) {
              const size_t pk = static_cast<size_t>(__ldg(a.t.rpidx + i));
              if (m & use & 1u) p0[q] = __ldg(pt + pk * 32);
              if (m & use & 2u) p1[q] = __ldg(pt + (pk + (m & 1u)) * 32);
            }
          }
        }
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const unsigned op = dec_op(ins[q]), A = dec_a(ins[q]), B = dec_b(ins[q]),
                         C = dec_c(ins[q]);
          const unsigned f = fl[q];
          if (!f) continue;
          if (op == D_OUTPUT) {
            wd[B * 32 + lane] = (f & 8u) ? sd[q] : __dadd_rn(ob[q], sd[q]);
            if (lane == 0) act[B] = 1;
            continue;
          }
          if (op == D_INPUT) {
            const IoDesc& d = a.sens[B];
            if (active && d.ptr) static_cast<double*>(d.ptr)[io_off(d, dir, C, ig)] = sd[q];
            if (lane == 0) act[A] = 0;
            continue;
          }
          if (lane == 0) act[A] = 0;
          if (op == D_CONST) continue;
          const double s = sd[q];
          double nb = ob[q];
          if (f & 2u) {
            const bool first = f & 8u;
            switch (op) {
              case D_ADD: case D_SUB: case D_ASSIGN:
                nb = first ? s : __dadd_rn(ob[q], s);
                break;
              case D_NEG:
                nb = first ? d_neg(s) : __dsub_rn(ob[q], s);
                break;
              case D_TWICE:
                nb = first ? d_twice(s) : __dadd_rn(ob[q], d_twice(s));
                break;
              default:
                nb = first ? __dmul_rn(p0[q], s) : __fma_rn(p0[q], s, ob[q]);
            }
            wd[B * 32 + lane] = nb;
            if (lane == 0) act[B] = 1;
          }
          if (f & 4u) {
            const bool first = f & 16u;
            const double old = (f & 2u) && C == B ? nb : oc[q];
            double nc;
            switch (op) {
              case D_ADD:
                nc = first ? s : __dadd_rn(old, s);
                break;
              case D_SUB:
                nc = first ? d_neg(s) : __dsub_rn(old, s);
                break;
              case D_IF_ELSE_ZERO:
                nc = first ? (d_iszero(p1[q]) ? 0.0 : s)
                           : (d_iszero(p1[q]) ? __dadd_rn(old, 0.0) : __dadd_rn(old, s));
                break;
              default:
                nc = first ? __dmul_rn(p1[q], s) : __fma_rn(p1[q], s, old);
            }
            wd[C * 32 + lane] = nc;
            if (lane == 0) act[C] = 1;
          }
        }
      }
      __syncthreads();
    }
  }
}
