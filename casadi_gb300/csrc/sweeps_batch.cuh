// The persistent multi-tape batch kernel.
//
// Part of the sweeps.cu translation unit (included where it stands): it uses that file's
// staging, decoding and I/O helpers and is not compiled on its own.
#pragma once

// ---------------------------------------------------------------------------------------------
// Persistent multi-tape batch: one launch drains a host-built list of work units
// (item, 32-instance tile), longest first, through an atomic counter. An item is one tape over
// its own instance range: a value sweep, a value + adjoint sweep, or a value + tangent sweep
// with identity (or colour-compressed) seeds. Each one-warp CTA grabs a unit, runs the
// warp-level value (or record) walk for its tile and then the adjoint or tangent walk of every
// direction, then grabs the next unit. Tapes of any length and
// instance count share the GPU in one launch instead of one underfilled launch per tape.
// ---------------------------------------------------------------------------------------------
// Warp-level value sweep of one tile; instruction words are read straight from the tape
// (uniform across the warp, cached) with the next word prefetched. RECORD writes partials to
// pt (lane-offset, tile-local [partial][lane]).
template <bool RECORD>
__device__ __forceinline__ void primal_walk(const TapeView& t, int n_code, double* pt,
                                            unsigned char* wb, const IoDesc* in,
                                            const IoDesc* out, bool active, long long ig) {
  const u64* code = t.code;
  int pidx = 0;
  PairState pair;  // the last sin/cos pair
  u64 nxt = __ldg(code);
#pragma unroll 1
  for (int k = 0; k < n_code; ++k) {
    const u64 ins = nxt;
    if (k + 1 < n_code) nxt = __ldg(code + k + 1);
    const unsigned op = dec_op(ins), A = dec_a(ins), B = dec_b(ins), C = dec_c(ins);
    switch (op) {
      case D_NOP:
        break;
      case D_CONST:
        wreg(wb, A * 256u) = __ldg(t.consts + B);
        break;
      case D_INPUT: {
        const IoDesc& d = in[B];
        double v = 0.0;
        if (active && d.ptr) v = __ldg(static_cast<const double*>(d.ptr) + io_off(d, 0, C, ig));
        wreg(wb, A * 256u) = v;
      } break;
      case D_OUTPUT: {
        const IoDesc& d = out[A];
        if (active && d.ptr) static_cast<double*>(d.ptr)[io_off(d, 0, C, ig)] = wreg(wb, B * 256u);
      } break;
      default: {
        const double x = wreg(wb, B * 256u), y = wreg(wb, C * 256u);
        if constexpr (RECORD) {
          const unsigned m = dec_pmask(ins);
          double d0 = 0.0, d1 = 0.0;
          const double f = dev_fun_der_pair(op, x, y, d0, d1, ins, pair.s, pair.c);
          if (m & 1u) pt[32 * pidx++] = d0;
          if (m & 2u) pt[32 * pidx++] = d1;
          wreg(wb, A * 256u) = f;
        } else {
          wreg(wb, A * 256u) = dev_fun_pair(op, x, y, ins, pair.s, pair.c);
        }
      }
    }
  }
}

// Bounded wait (lane 0, then shared with the warp) for a split item's tile flag. Every record
// unit precedes every direction unit in the list, so the unit that sets the flag was taken by
// a CTA that is already running and waits on nothing: the wait ends unless that CTA faults.
__device__ __forceinline__ bool wait_tile(const unsigned* flag, unsigned* err) {
  bool ok = true;
  if ((threadIdx.x & 31) == 0) {
    const long long t0 = clock64();
    for (unsigned k = 0;; ++k) {
      if (*reinterpret_cast<const volatile unsigned*>(flag)) break;
      if ((k & 63u) == 63u && clock64() - t0 > kWaitCycles) {
        ok = false;
        atomicOr(err, kErrWaitTimeout);
        break;
      }
      __nanosleep(128);
    }
  }
  ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
  __threadfence();  // the partials written before the flag are visible from here on
  return ok;
}

// One warp waiting, with the batch's bounded wait, on a flag that nothing sets: the wait runs
// out after kWaitCycles, records kErrWaitTimeout in *err and the kernel returns.
__global__ void k_wait_probe(const unsigned* flag, unsigned* err) { wait_tile(flag, err); }

cudaError_t launch_wait_probe(const unsigned* flag, unsigned* err, cudaStream_t s) {
  k_wait_probe<<<1, 32, 0, s>>>(flag, err);
  return cudaGetLastError();
}

// kSplit: the batch has split items (per-tile record units and per-direction units); batches
// without any run the instance that holds only the whole-unit path. GW: the work vector lives
// in global memory (per-CTA blocks) instead of shared memory, so residency is not capped by
// the longest tape's work vector.
template <bool kSplit, bool GW>
__global__ void __launch_bounds__(32, 16) k_batch(const __grid_constant__ BatchArgs b) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int lane = threadIdx.x;
  unsigned char* wb = (GW ? b.wglob + blockIdx.x * b.wglob_stride : smem) + lane * 8;
  double* const pcta = b.scratch + static_cast<size_t>(blockIdx.x) * b.scratch_stride + lane;
  for (;;) {
    unsigned u = 0;
    if (lane == 0) u = atomicAdd(b.counter, 1u);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= static_cast<unsigned>(b.n_units)) break;
    const int4 unit = __ldg(b.units + u);
    const BatchItem& it = b.items[unit.x];
    const long long il = static_cast<long long>(unit.y) * 32 + lane;
    const bool active = il < it.n;
    const IoDesc* io = it.io;
    // partials: the item's per-tile buffer (split items) or this CTA's scratch (whole units)
    double* pt = (kSplit && it.tile_partials)
                     ? it.tile_partials + static_cast<size_t>(unit.y) * it.t.n_partials * 32 + lane
                     : pcta;
    int d0 = 0, d1 = it.ndir;
    if (!kSplit || unit.z < 0) {
      // record (or value) unit
      if (it.ndir == 0) {
        primal_walk<false>(it.t, it.n_code, pt, wb, io, io + kMaxIo, active, il);
        continue;
      }
      primal_walk<true>(it.t, it.n_code, pt, wb, io, io + kMaxIo, active, il);
      if (kSplit && it.tile_partials) {
        // split item: publish the tile's partials; its directions are separate units
        __threadfence();
        __syncwarp();
        if (lane == 0) atomicExch(it.ready + unit.y, 1u);
        continue;
      }
      // whole unit: the warp's own partial stores must be visible to its loads below
      __syncwarp();
    } else {
      // one direction of a split item, after its tile's record unit
      if (!wait_tile(it.ready + unit.y, b.err)) continue;
      d0 = unit.z;
      d1 = unit.z + 1;
    }
    const bool act1[1] = {active}, tok1[1] = {true};
    const long long ig1[1] = {il};
    for (int dir = d0; dir < d1; ++dir) {
      if (it.forward) {
        const int2 se = __ldg(it.tan_chunks + dir);
        tangent_walk<false, kBatchTanGroup, 1, 1>(it.tan_stream + se.x, se.y / kBatchTanGroup,
                                                  pt, 0, tok1, wb, io + 2 * kMaxIo,
                                                  io + 3 * kMaxIo, true, act1, dir, it.ndir, ig1);
        continue;
      }
      // (the work vector needs no clearing: the adjoint walk assigns every slot before reading)
      if (active) {
        for (int k = 0; k < it.n_zero; ++k) {
          const int2 jk = __ldg(it.zero_in + k);
          const IoDesc& d = io[3 * kMaxIo + jk.x];
          if (d.ptr) static_cast<double*>(d.ptr)[io_off(d, dir, jk.y, il)] = 0.0;
        }
      }
      adjoint_walk<false, kBatchAdjGroup, 1>(it.adj_stream, it.adj_ngr, pt, 0, tok1, wb,
                                             io + 2 * kMaxIo, io + 3 * kMaxIo, act1, dir, ig1);
    }
  }
}
