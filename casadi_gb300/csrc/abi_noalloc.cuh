// C ABI: the allocation-free adjoint entry point.
//
// Part of the abi.cu translation unit (included at its end): it uses that file's internal
// registry, plans and launch helpers and is not compiled on its own.
#pragma once

// ---------------------------------------------------------------------------------------------
// Allocation-free adjoint sweep.
//
// Some callers cannot allocate device memory at the point where they need derivatives: a
// real-time control loop that forbids allocation after start-up, or a plugin hosted by a
// framework that owns the device allocator. casadi_gb300_reverse_noalloc serves them: its partials scratch is the file-scope
// device array below, a fixed 64 MiB that every GPU which loads this library holds until the
// process exits. It runs the record sweep and the plan-free adjoint variant, so it makes no
// device allocation of any kind, and it needs no host allocation either.
// ---------------------------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;
constexpr int kNoAllocMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mtx;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device. In host code the symbol's name
// is only a handle, so the address is looked up once per device, with that device current.
int noalloc_scratch(void** ptr) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return fail(CASADI_GB300_ERR_UNSUPPORTED, "device %d is beyond the %d supported", dev,
                kNoAllocMaxDevices);
  std::lock_guard<std::mutex> lk(g_noalloc_mtx);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
    g_noalloc_ptr[dev] = p;
  }
  *ptr = g_noalloc_ptr[dev];
  return 0;
}

// Launch shape of the plan-free adjoint: the most resident warps that fit, as dir_shape
// chooses, computed without touching the tape's shape cache. dw = 0: no shape fits (the
// work vector is too long for shared memory).
DirShape noalloc_shape(const Tape& t, int ndir) {
  const int max_smem = max_smem_optin();
  DirShape best;
  best.dw = 0;
  double best_score = -1;
  for (int ch : {64, 32, 16}) {
    for (int dw : {8, 6, 4, 2, 1}) {
      if (dw > 1 && dw >= 2 * ndir) continue;
      const size_t sm = smem_dir(t.sz_w, dw, ch);
      if (sm > static_cast<size_t>(max_smem)) continue;
      const int occ = occupancy_dense(dw, sm);
      if (occ <= 0) continue;
      const int groups = (ndir + dw - 1) / dw;
      const double used = static_cast<double>(ndir) / (groups * dw);
      const double score = std::min(occ * dw, 8) * used * (1.0 + 0.01 * ch);
      if (score > best_score) {
        best_score = score;
        best.dw = dw;
        best.ch = ch;
        best.blocks_per_sm = occ;
      }
    }
  }
  return best;
}

}  // namespace

extern "C" {

int casadi_gb300_reverse_noalloc(int id, int64_t n, int64_t ld, int nadj,
                                 const double* const* arg, double* const* res,
                                 const double* const* aseed, double* const* asens, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (nadj < 0 || nadj > 65535) return fail(CASADI_GB300_ERR_ARG, "bad direction count %d", nadj);
  if (n == 0) return 0;
  // both sweeps keep the work vector in shared memory (the global-memory form would need
  // device buffers of its own): find the record sweep's block size and the adjoint's shape
  int block = 0;
  for (int bs : {t->primal_block, 128, 64, 32})
    if (bs >= 32 && smem_primal(t->sz_w, bs) <= static_cast<size_t>(max_smem_optin())) {
      block = bs;
      break;
    }
  const DirShape ds = noalloc_shape(*t, std::max(nadj, 1));
  if (block == 0 || (nadj > 0 && ds.dw == 0))
    return fail(CASADI_GB300_ERR_UNSUPPORTED,
                "allocation-free adjoint: the tape's work vector (%d slots, %zu bytes per "
                "32-instance tile) does not fit in shared memory, where this entry point keeps "
                "it; use casadi_gb300_reverse",
                t->sz_w, static_cast<size_t>(t->sz_w) * 256);
  const unsigned long long need =
      8ull * 32ull * static_cast<unsigned long long>(t->n_partials) *
      static_cast<unsigned long long>((n + 31) / 32);
  if (need > kNoAllocScratchBytes)
    return fail(CASADI_GB300_ERR_SCRATCH,
                "allocation-free adjoint: %lld instances need %llu bytes of scratch, above its "
                "fixed %zu bytes; split the call or use casadi_gb300_reverse",
                static_cast<long long>(n), need, kNoAllocScratchBytes);
  void* scratch = nullptr;
  if (int rc = noalloc_scratch(&scratch)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  SweepArgs a = base_args(*t, n, 0);
  a.partials = static_cast<double*>(scratch);
  a.pofs = t->d_pofs;
  a.n_code = t->n_chunks * kChunk;
  a.ndir = nadj;
  fill_io(a.in, t->n_in, vptrs(arg), t->nnz_in, ld, false);
  fill_io(a.out, t->n_out, vptrs(res), t->nnz_out, ld, false);
  a.block = block;
  const int rgrid = grid_for((n + a.block - 1) / a.block,
                             sm_count() * std::max(1, occupancy_primal(
                                                          block, smem_primal(t->sz_w, block))));
  cudaError_t e = timed(F_RECORD, s, [&] { return launch_record(a, rgrid, s); });
  if (e != cudaSuccess) return cuda_fail(e, "record sweep launch");
  if (nadj == 0) return 0;
  fill_io(a.seed, t->n_out, vptrs(aseed), t->nnz_out, ld, true);
  fill_io(a.sens, t->n_in, vptrs(asens), t->nnz_in, ld, true);
  const int groups = (nadj + ds.dw - 1) / ds.dw;
  a.block = 32 * ds.dw;
  a.chunk = ds.ch;
  const long long tiles = (n + 31) / 32;
  const long long per_group = std::max<long long>(
      1, std::min<long long>(tiles, static_cast<long long>(sm_count()) * ds.blocks_per_sm / groups));
  e = timed(F_ADJOINT, s,
            [&] { return launch_adjoint_dense(a, static_cast<int>(per_group * groups), s); });
  if (e != cudaSuccess) return cuda_fail(e, "adjoint launch");
  return 0;
}

}  // extern "C"
