// Windowed tangent sweep: the directions of one 32-instance tile walk the tape together.
//
// Part of the sweeps.cu translation unit (included after k_tangent, whose entry format, case
// arithmetic and helpers -- bulk_g2s, smem_u32, wreg, io_off -- it shares); not compiled on
// its own.
//
// The warp-independent tangent sweep (k_tangent) gives each (tile, direction) item to its own
// warp; the 24 directions of a tile then walk the tape at unrelated positions, so every
// direction fetches the tile's recorded partials from L2/HBM on its own (on the 20-step
// rollout 5x the partial bytes come from HBM, and the walks stall on those loads). Here one CTA
// per SM takes a (tile, direction group) item and the host has cut the tape into windows of a
// few dozen instructions. Warp 0 stages each window into a shared-memory ring with two bulk
// copies completing on the stage's mbarrier: the tile's partial rows of the window (contiguous
// in the tile-major layout) and the window's entry block (a header with the window's first
// partial row and per-direction entry offsets, then every direction's entries). Warps 1..D each
// walk one direction's entries of the window with partials and entries read from shared
// memory, then release the stage. The arithmetic of every entry is k_tangent's, so results are
// the same bits. Measured on the 20-step rollout (262144 instances, 24 directions): 29.9 ms
// against 24.1 ms for k_tangent. With one tile in flight per SM the densest direction's chain
// of dependent entries (2976 of the tape's 3057 instructions) gates every window of the tile,
// where k_tangent overlaps such chains of many tiles; the autotuner keeps it for tapes where it
// wins. Waits are bounded (~1 s): a wait that runs out sets kErrWaitTimeout, the other
// warps see the abort flag and leave, and warp 0 waits (bounded) for its copies in flight.
#pragma once

constexpr int kWinMaxThreads = (kWinMaxDirs + 1) * 32;

__device__ __forceinline__ void mbar_init(u64* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(u64* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(u64* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Bounded wait for the completion of the phase of `bar` with the given parity. False when
// about 1 s passes, or when another warp has set *abort (if given). A waiting warp backs off
// with a short sleep between tests, so it leaves the issue slots of its SM sub-partition to
// the warps that are still walking the window.
__device__ __forceinline__ bool mbar_wait(u64* bar, unsigned parity, volatile int* abort) {
  const unsigned addr = smem_u32(bar);
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
    __nanosleep(it < 4 ? 32 : 256);
    if ((it & 31u) == 31u) {
      if (abort && *abort) return false;
      if (clock64() - t0 > kWaitCycles) return false;
    }
  }
}

// One direction's entries of one window (k_tangent's K = 1 cases). pw: the window's partial
// rows in shared memory, lane-offset (row r at pw + r*32), p0 the window's first partial row;
// wb the warp's work vector w[slot][lane], lane-offset; last the value the previous entry of
// the direction wrote (operand forwarding carries across windows). Only the partials and
// operands an entry uses are read. (Loading the next entry's partials and operands before the
// current one computes made the sweep slower on the rollout, 29.9 -> 41.0 ms.)
__device__ __forceinline__ void win_walk(const uint4* ents, int cnt, const double* pw,
                                         unsigned p0, unsigned char* wb, double& last,
                                         const SweepArgs& a, int dir, bool active,
                                         long long ig) {
#define CGB_WOP(off) (((off) & 0x80000000u) ? last : wreg(wb, (off) & 0x7fffffffu))
#pragma unroll 1
  for (int e = 0; e < cnt; ++e) {
    const uint4 cur = ents[e];
    const unsigned meta = cur.w;
    const unsigned key = (ent_kind(meta) << 2) | (ent_flags(meta) & 3u);
    const unsigned m = ent_pmask(meta);
    const unsigned r0 = ent_pk(meta) - p0;
    const unsigned r1 = r0 + (m & 1u);
    double r;
    switch (key) {
      case (LK_OUTPUT << 2) | 0u:
      case (LK_OUTPUT << 2) | 1u: {
        const IoDesc& d = a.sens[cur.x];
        if (active && d.ptr)
          static_cast<double*>(d.ptr)[io_off(d, dir, cur.z, ig)] =
              (meta & 1u) ? CGB_WOP(cur.y) : 0.0;
        continue;
      }
      case (LK_INPUT << 2) | 1u:
        if (a.identity_seed) {
          r = 1.0;
        } else {
          const IoDesc& d = a.seed[cur.y];
          r = active ? __ldg(static_cast<const double*>(d.ptr) + io_off(d, dir, cur.z, ig))
                     : 0.0;
        }
        break;
      case (LK_GEN << 2) | 1u:
        r = __dmul_rn((m & 1u) ? pw[r0 * 32] : 1.0, CGB_WOP(cur.y));
        break;
      case (LK_GEN << 2) | 2u:
        r = __dmul_rn((m & 2u) ? pw[r1 * 32] : 0.0, CGB_WOP(cur.z));
        break;
      case (LK_GEN << 2) | 3u:
        r = __fma_rn((m & 1u) ? pw[r0 * 32] : 1.0, CGB_WOP(cur.y),
                     __dmul_rn((m & 2u) ? pw[r1 * 32] : 0.0, CGB_WOP(cur.z)));
        break;
      case (LK_ADD << 2) | 1u: r = CGB_WOP(cur.y); break;
      case (LK_ADD << 2) | 2u: r = CGB_WOP(cur.z); break;
      case (LK_ADD << 2) | 3u: r = __dadd_rn(CGB_WOP(cur.y), CGB_WOP(cur.z)); break;
      case (LK_SUB << 2) | 1u: r = CGB_WOP(cur.y); break;
      case (LK_SUB << 2) | 2u: r = d_neg(CGB_WOP(cur.z)); break;
      case (LK_SUB << 2) | 3u: r = __dsub_rn(CGB_WOP(cur.y), CGB_WOP(cur.z)); break;
      case (LK_NEG << 2) | 1u: r = d_neg(CGB_WOP(cur.y)); break;
      case (LK_TWICE << 2) | 1u: r = d_twice(CGB_WOP(cur.y)); break;
      case (LK_ASSIGN << 2) | 1u: r = CGB_WOP(cur.y); break;
      case (LK_IFZ << 2) | 2u:
        r = d_iszero((m & 2u) ? pw[r1 * 32] : 0.0) ? 0.0 : CGB_WOP(cur.z);
        break;
      default:
        continue;  // NOP padding
    }
    wreg(wb, cur.x) = r;
    last = r;
  }
#undef CGB_WOP
}

__global__ void __launch_bounds__(kWinMaxThreads, 1)
    k_tangent_win(const __grid_constant__ SweepArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int D = a.win_dirs, S = a.win_stages;
  u64* full = reinterpret_cast<u64*>(smem);
  u64* empty = full + S;
  const size_t stage_bytes =
      static_cast<size_t>(a.win_rows) * 256 + static_cast<size_t>(a.win_ents) * 16;
  unsigned char* stage0 = smem + kWinBarBytes;
  unsigned char* wv = stage0 + S * stage_bytes;
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, static_cast<unsigned>(D));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  __syncthreads();
  const long long ntiles = (a.n + 31) / 32;
  const int groups = (a.ndir + D - 1) / D;
  const long long nitems = ntiles * groups;
  const int nwin = a.win_n;
  volatile int* abort = &abort_flag;

  if (warp == 0) {
    // producer: one thread issues both copies of every window, a stage at a time
    if (lane != 0) return;
    unsigned seq = 0;
    bool ok = true;
    for (long long item = blockIdx.x; ok && item < nitems; item += gridDim.x) {
      const long long tile = item / groups;
      const int g = static_cast<int>(item % groups);
      const double* tp = a.partials + static_cast<size_t>(tile) * a.t.n_partials * 32;
      for (int w = 0; w < nwin; ++w, ++seq) {
        const int s = static_cast<int>(seq % S);
        const unsigned use = seq / S;
        // the stage's previous contents must have been released by every consumer warp
        if (use > 0 && !mbar_wait(empty + s, (use - 1) & 1u, abort)) {
          ok = false;
          break;
        }
        const int4 mw = __ldg(a.win_meta + static_cast<size_t>(g) * nwin + w);
        unsigned char* st = stage0 + s * stage_bytes;
        mbar_expect_tx(full + s, static_cast<unsigned>(mw.y) * 256u +
                                     static_cast<unsigned>(mw.w) * 16u);
        if (mw.y > 0)
          bulk_g2s(st, tp + static_cast<size_t>(mw.x) * 32, static_cast<unsigned>(mw.y) * 256u,
                   full + s);
        bulk_g2s(st + static_cast<size_t>(a.win_rows) * 256, a.win_blocks + mw.z,
                 static_cast<unsigned>(mw.w) * 16u, full + s);
      }
    }
    if (!ok) {
      atomicOr(a.t.err, kErrWaitTimeout);
      *abort = 1;
      // copies issued but not yet seen complete: a bounded chance to land before the CTA's
      // shared memory is released
      for (unsigned q = seq > static_cast<unsigned>(S) ? seq - S : 0u; q < seq; ++q)
        mbar_wait(full + q % S, (q / S) & 1u, nullptr);
    }
    return;
  }

  // consumers: warp j walks direction g*D + j of each item
  const int j = warp - 1;
  unsigned char* wb = wv + static_cast<size_t>(j) * a.t.sz_w * 256 + lane * 8;
  const int hw = win_header_words(D);
  const int sj = a.identity_seed ? j : 0;  // general seeds: one stream serves every direction
  unsigned seq = 0;
  for (long long item = blockIdx.x; item < nitems; item += gridDim.x) {
    const long long tile = item / groups;
    const int g = static_cast<int>(item % groups);
    const int dir = g * D + j;
    const bool dir_ok = dir < a.ndir;
    const long long il = tile * 32 + lane;
    const bool active = il < a.n;
    const long long ig = a.i_begin + il;
    double last = 0.0;
    for (int w = 0; w < nwin; ++w, ++seq) {
      const int s = static_cast<int>(seq % S);
      // one verdict for the whole warp, so no lane leaves while the others go on
      if (!__all_sync(0xffffffffu, mbar_wait(full + s, (seq / S) & 1u, abort))) {
        if (lane == 0) {
          atomicOr(a.t.err, kErrWaitTimeout);
          *abort = 1;
        }
        return;
      }
      const unsigned char* st = stage0 + s * stage_bytes;
      const unsigned* hdr =
          reinterpret_cast<const unsigned*>(st + static_cast<size_t>(a.win_rows) * 256);
      if (dir_ok) {
        const unsigned e0 = hdr[2 + sj], e1 = hdr[3 + sj];
        win_walk(reinterpret_cast<const uint4*>(hdr + hw) + e0, static_cast<int>(e1 - e0),
                 reinterpret_cast<const double*>(st) + lane, hdr[0], wb, last, a, dir, active,
                 ig);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(empty + s);
    }
  }
}
