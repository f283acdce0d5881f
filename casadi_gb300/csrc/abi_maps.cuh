// C ABI: MapSum, Mapaccum and the self-check of the bounded waits.
//
// Part of the abi.cu translation unit (included at its end): it uses that file's internal
// registry, plans and launch helpers and is not compiled on its own.
#pragma once

// A MapSum call sums at most two row groups per output (values and their directions) in
// forward mode and one per output and per shared input in reverse mode; the instance-order
// reduction takes them in launches of up to kMaxSumGroups groups.

// ---- MapSum: shared inputs and instance-summed outputs (casadi/core/mapsum.cpp) -------------
namespace {

// Bump allocator over the caller's scratch (256-byte aligned regions).
struct Arena {
  char* p = nullptr;
  size_t left = 0;
  Arena(void* base, size_t bytes) {
    const uintptr_t b = reinterpret_cast<uintptr_t>(base);
    const uintptr_t a = (b + 255) & ~static_cast<uintptr_t>(255);
    if (base && bytes >= a - b) {
      p = reinterpret_cast<char*>(a);
      left = bytes - (a - b);
    }
  }
  void* take(size_t bytes) {
    const size_t b = (bytes + 255) & ~static_cast<size_t>(255);
    if (!p || b > left) return nullptr;
    void* r = p;
    p += b;
    left -= b;
    return r;
  }
};

struct SumFlags {
  bool shared[kMaxIo] = {};
  bool summed[kMaxIo] = {};
  int order = 0;
};

int sum_flags(const Tape& t, const casadi_gb300_mapsum_spec* spec, SumFlags* f) {
  if (!spec) return fail(CASADI_GB300_ERR_ARG, "missing MapSum spec");
  if (spec->order != 0 && spec->order != 1)
    return fail(CASADI_GB300_ERR_ARG, "MapSum order must be 0 (instance order) or 1 (tree)");
  for (int j = 0; j < t.n_in; ++j) f->shared[j] = spec->reduce_in && spec->reduce_in[j] != 0;
  for (int j = 0; j < t.n_out; ++j) f->summed[j] = spec->reduce_out && spec->reduce_out[j] != 0;
  f->order = spec->order;
  return 0;
}

// An input (or seed) shared by every instance: ptr[d*nnz + k].
IoDesc shared_io(const void* ptr, int nnz) {
  return IoDesc{const_cast<void*>(ptr), 1, 0, static_cast<long long>(nnz)};
}
// Rows of n instances: ptr[(d*nnz + k)*n + i] (the per-instance values of a summed output).
IoDesc rows_io(void* ptr, int nnz, long long n) {
  return IoDesc{ptr, n, 1, static_cast<long long>(nnz) * n};
}
// The ordinary instance-minor layout with leading dimension ld.
IoDesc plain_io(const void* ptr, int nnz, long long ld, bool dir_major) {
  return IoDesc{const_cast<void*>(ptr), ld, 1, dir_major ? static_cast<long long>(nnz) * ld : 0};
}

template <class T>
const void* at(T* const* p, int j) {
  return p ? static_cast<const void*>(p[j]) : nullptr;
}

// Scratch the reductions of one call need besides the derivative sweeps: the per-instance rows
// of every summed output (values and ndir directions) and shared input (ndir sensitivity
// directions, or the sparsity bits), and the tree's level buffers.
size_t sum_bytes(const Tape& t, long long n, int ndir, const SumFlags& f) {
  const long long nd = std::max(1, ndir);
  size_t bytes = 0;
  long long max_rows = 0;
  for (int j = 0; j < t.n_out; ++j) {
    if (!f.summed[j]) continue;
    const long long k = t.nnz_out[j];
    bytes += ((8 * k * n + 255) / 256) * 256 + ((8 * k * nd * n + 255) / 256) * 256;
    max_rows = std::max(max_rows, k * nd);
  }
  for (int j = 0; j < t.n_in; ++j) {
    if (!f.shared[j]) continue;
    const long long k = t.nnz_in[j];
    bytes += ((8 * k * nd * n + 255) / 256) * 256;
    max_rows = std::max(max_rows, k * nd);
  }
  return bytes + ((reduce_scratch_bytes(max_rows, n, f.order) + 255) / 256) * 256 + 256;
}

// Largest row count one reduction of the call handles (its tree buffers are reused).
long long max_sum_rows(const Tape& t, int ndir, const SumFlags& f) {
  const long long nd = std::max(1, ndir);
  long long m = 0;
  for (int j = 0; j < t.n_out; ++j)
    if (f.summed[j]) m = std::max(m, static_cast<long long>(t.nnz_out[j]) * nd);
  for (int j = 0; j < t.n_in; ++j)
    if (f.shared[j]) m = std::max(m, static_cast<long long>(t.nnz_in[j]) * nd);
  return m;
}

int scratch_short(const char* what) {
  return fail(CASADI_GB300_ERR_SCRATCH,
              "MapSum scratch too small for the %s (see casadi_gb300_mapsum_scratch_size)", what);
}

int take_tree(Arena& ar, const Tape& t, long long n, int ndir, const SumFlags& f, double** tree) {
  const size_t b = reduce_scratch_bytes(max_sum_rows(t, ndir, f), n, f.order);
  *tree = nullptr;
  if (b == 0) return 0;
  *tree = static_cast<double*>(ar.take(b));
  return *tree ? 0 : scratch_short("summation tree");
}

int sum_rows(long long rows, long long n, const double* src, double* dst, int order,
             double* tree, cudaStream_t s) {
  cudaError_t e = reduce_sum(rows, n, src, n, dst, order, tree, s);
  return e == cudaSuccess ? 0 : cuda_fail(e, "MapSum reduction");
}

// The row sums of one call: instance-order sums are collected and run by one launch, since
// their chains are independent; tree sums run as they come.
struct RowSums {
  int order;
  double* tree;
  std::vector<SumRows> g;
  int add(long long rows, long long n, const double* src, double* dst, cudaStream_t s) {
    if (order != kOrderInstance) return sum_rows(rows, n, src, dst, order, tree, s);
    g.push_back({src, n, dst, rows});
    return 0;
  }
  int flush(long long n, cudaStream_t s) {
    cudaError_t e = reduce_sum_instance_multi(g.data(), static_cast<int>(g.size()), n, s);
    g.clear();
    return e == cudaSuccess ? 0 : cuda_fail(e, "MapSum reduction");
  }
};

}  // namespace

extern "C" {

int casadi_gb300_mapsum_scratch_size(int id, int64_t n, int ndir,
                                     const casadi_gb300_mapsum_spec* spec, size_t* bytes) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (!bytes || n < 0 || ndir < 0) return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  SumFlags f;
  if (int rc = sum_flags(*t, spec, &f)) return rc;
  const size_t sweep =
      ndir > 0 ? static_cast<size_t>(8) * t->n_partials * static_cast<size_t>(((n + 31) / 32) * 32)
               : 0;
  *bytes = sum_bytes(*t, n, ndir, f) + sweep + 256 + kQueueSlack;
  return 0;
}

int casadi_gb300_mapsum_eval(int id, int64_t n, int64_t ld, const casadi_gb300_mapsum_spec* spec,
                             const double* const* arg, double* const* res, void* scratch,
                             size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  SumFlags f;
  if (int rc = sum_flags(*t, spec, &f)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Arena ar(scratch, scratch_bytes);
  SweepArgs a = base_args(*t, n, 0);
  double* rows[kMaxIo] = {};
  for (int j = 0; j < t->n_in; ++j)
    a.in[j] = f.shared[j] ? shared_io(at(arg, j), t->nnz_in[j])
                          : plain_io(at(arg, j), t->nnz_in[j], ld, false);
  for (int j = 0; j < t->n_out; ++j) {
    if (f.summed[j] && at(res, j)) {
      rows[j] = static_cast<double*>(ar.take(8 * static_cast<size_t>(t->nnz_out[j]) * n));
      if (!rows[j]) return scratch_short("summed outputs");
      a.out[j] = rows_io(rows[j], t->nnz_out[j], n);
    } else {
      a.out[j] = plain_io(at(res, j), t->nnz_out[j], ld, false);
    }
  }
  double* tree = nullptr;
  if (int rc = take_tree(ar, *t, n, 0, f, &tree)) return rc;
  if (n > 0)
    if (int rc = primal_launch(*t, a, n, PK_EVAL, s)) return rc;
  RowSums sums{f.order, tree, {}};
  for (int j = 0; j < t->n_out; ++j)
    if (rows[j])
      if (int rc = sums.add(t->nnz_out[j], n, rows[j], res[j], s)) return rc;
  return sums.flush(n, s);
}

int casadi_gb300_mapsum_forward(int id, int64_t n, int64_t ld,
                                const casadi_gb300_mapsum_spec* spec, int nfwd,
                                const double* const* arg, double* const* res,
                                const double* const* fseed, double* const* fsens, void* scratch,
                                size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (nfwd < 0 || nfwd > 65535) return fail(CASADI_GB300_ERR_ARG, "bad direction count %d", nfwd);
  SumFlags f;
  if (int rc = sum_flags(*t, spec, &f)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Arena ar(scratch, scratch_bytes);
  IoDesc in[kMaxIo], out[kMaxIo], seed[kMaxIo], sens[kMaxIo];
  double* rows[kMaxIo] = {};
  double* srows[kMaxIo] = {};
  for (int j = 0; j < t->n_in; ++j) {
    const int k = t->nnz_in[j];
    in[j] = f.shared[j] ? shared_io(at(arg, j), k) : plain_io(at(arg, j), k, ld, false);
    seed[j] = f.shared[j] ? shared_io(at(fseed, j), k) : plain_io(at(fseed, j), k, ld, true);
  }
  for (int j = 0; j < t->n_out; ++j) {
    const int k = t->nnz_out[j];
    out[j] = plain_io(at(res, j), k, ld, false);
    sens[j] = plain_io(at(fsens, j), k, ld, true);
    if (!f.summed[j]) continue;
    if (at(res, j)) {
      rows[j] = static_cast<double*>(ar.take(8 * static_cast<size_t>(k) * n));
      if (!rows[j]) return scratch_short("summed outputs");
      out[j] = rows_io(rows[j], k, n);
    }
    if (at(fsens, j) && nfwd > 0) {
      srows[j] = static_cast<double*>(ar.take(8 * static_cast<size_t>(k) * nfwd * n));
      if (!srows[j]) return scratch_short("summed sensitivities");
      sens[j] = rows_io(srows[j], k, n);
    }
  }
  double* tree = nullptr;
  if (int rc = take_tree(ar, *t, n, nfwd, f, &tree)) return rc;
  if (int rc = run_ad(*t, n, in, out, seed, sens, nfwd, false, false, ar.p, ar.left, s))
    return rc;
  RowSums sums{f.order, tree, {}};
  for (int j = 0; j < t->n_out; ++j) {
    if (rows[j])
      if (int rc = sums.add(t->nnz_out[j], n, rows[j], res[j], s)) return rc;
    if (srows[j])
      if (int rc = sums.add(static_cast<long long>(t->nnz_out[j]) * nfwd, n, srows[j],
                            fsens[j], s))
        return rc;
  }
  return sums.flush(n, s);
}

int casadi_gb300_mapsum_reverse(int id, int64_t n, int64_t ld,
                                const casadi_gb300_mapsum_spec* spec, int nadj,
                                const double* const* arg, double* const* res,
                                const double* const* aseed, double* const* asens, void* scratch,
                                size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (nadj < 0 || nadj > 65535) return fail(CASADI_GB300_ERR_ARG, "bad direction count %d", nadj);
  SumFlags f;
  if (int rc = sum_flags(*t, spec, &f)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Arena ar(scratch, scratch_bytes);
  IoDesc in[kMaxIo], out[kMaxIo], seed[kMaxIo], sens[kMaxIo];
  double* rows[kMaxIo] = {};
  double* srows[kMaxIo] = {};
  for (int j = 0; j < t->n_out; ++j) {
    const int k = t->nnz_out[j];
    out[j] = plain_io(at(res, j), k, ld, false);
    seed[j] = f.summed[j] ? shared_io(at(aseed, j), k) : plain_io(at(aseed, j), k, ld, true);
    if (f.summed[j] && at(res, j)) {
      rows[j] = static_cast<double*>(ar.take(8 * static_cast<size_t>(k) * n));
      if (!rows[j]) return scratch_short("summed outputs");
      out[j] = rows_io(rows[j], k, n);
    }
  }
  for (int j = 0; j < t->n_in; ++j) {
    const int k = t->nnz_in[j];
    in[j] = f.shared[j] ? shared_io(at(arg, j), k) : plain_io(at(arg, j), k, ld, false);
    sens[j] = plain_io(at(asens, j), k, ld, true);
    if (f.shared[j] && at(asens, j) && nadj > 0) {
      srows[j] = static_cast<double*>(ar.take(8 * static_cast<size_t>(k) * nadj * n));
      if (!srows[j]) return scratch_short("summed sensitivities");
      sens[j] = rows_io(srows[j], k, n);
    }
  }
  double* tree = nullptr;
  if (int rc = take_tree(ar, *t, n, nadj, f, &tree)) return rc;
  if (int rc = run_ad(*t, n, in, out, seed, sens, nadj, true, false, ar.p, ar.left, s)) return rc;
  RowSums sums{f.order, tree, {}};
  for (int j = 0; j < t->n_out; ++j)
    if (rows[j])
      if (int rc = sums.add(t->nnz_out[j], n, rows[j], res[j], s)) return rc;
  for (int j = 0; j < t->n_in; ++j)
    if (srows[j])
      if (int rc = sums.add(static_cast<long long>(t->nnz_in[j]) * nadj, n, srows[j],
                            asens[j], s))
        return rc;
  return sums.flush(n, s);
}

int casadi_gb300_mapsum_sp_forward(int id, int64_t n, int64_t ld,
                                   const casadi_gb300_mapsum_spec* spec,
                                   const uint64_t* const* arg, uint64_t* const* res,
                                   void* scratch, size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  SumFlags f;
  if (int rc = sum_flags(*t, spec, &f)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Arena ar(scratch, scratch_bytes);
  SweepArgs a = base_args(*t, n, 0);
  u64* rows[kMaxIo] = {};
  for (int j = 0; j < t->n_in; ++j)
    a.in[j] = f.shared[j] ? shared_io(at(arg, j), t->nnz_in[j])
                          : plain_io(at(arg, j), t->nnz_in[j], ld, false);
  for (int j = 0; j < t->n_out; ++j) {
    if (f.summed[j] && at(res, j)) {
      rows[j] = static_cast<u64*>(ar.take(8 * static_cast<size_t>(t->nnz_out[j]) * n));
      if (!rows[j]) return scratch_short("summed outputs");
      a.out[j] = rows_io(rows[j], t->nnz_out[j], n);
    } else {
      a.out[j] = plain_io(at(res, j), t->nnz_out[j], ld, false);
    }
  }
  if (n > 0)
    if (int rc = primal_launch(*t, a, n, PK_SP_FORWARD, s)) return rc;
  for (int j = 0; j < t->n_out; ++j) {
    if (!rows[j]) continue;
    cudaError_t e = reduce_or(t->nnz_out[j], n, rows[j], n, reinterpret_cast<u64*>(res[j]), false, s);
    if (e != cudaSuccess) return cuda_fail(e, "MapSum OR reduction");
  }
  return 0;
}

int casadi_gb300_mapsum_sp_reverse(int id, int64_t n, int64_t ld,
                                   const casadi_gb300_mapsum_spec* spec, uint64_t* const* arg,
                                   uint64_t* const* res, void* scratch, size_t scratch_bytes,
                                   void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  SumFlags f;
  if (int rc = sum_flags(*t, spec, &f)) return rc;
  if (n == 0) return 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Arena ar(scratch, scratch_bytes);
  SweepArgs a = base_args(*t, n, 0);
  u64* arows[kMaxIo] = {};
  u64* srows[kMaxIo] = {};
  cudaError_t e = cudaSuccess;
  for (int j = 0; j < t->n_in; ++j) {
    const int k = t->nnz_in[j];
    a.in[j] = plain_io(at(arg, j), k, ld, false);
    if (f.shared[j] && at(arg, j)) {
      // every instance ORs its bits into its own row; the rows are OR-ed into arg[j] after
      arows[j] = static_cast<u64*>(ar.take(8 * static_cast<size_t>(k) * n));
      if (!arows[j]) return scratch_short("shared inputs");
      if ((e = cudaMemsetAsync(arows[j], 0, 8 * static_cast<size_t>(k) * n, s)) != cudaSuccess)
        return cuda_fail(e, "MapSum clear");
      a.in[j] = rows_io(arows[j], k, n);
    }
  }
  for (int j = 0; j < t->n_out; ++j) {
    const int k = t->nnz_out[j];
    a.out[j] = plain_io(at(res, j), k, ld, false);
    if (f.summed[j] && at(res, j)) {
      // the summed output's seed reaches every instance (MapSum restores it before each one)
      srows[j] = static_cast<u64*>(ar.take(8 * static_cast<size_t>(k) * n));
      if (!srows[j]) return scratch_short("summed outputs");
      if ((e = broadcast_rows(k, n, reinterpret_cast<const u64*>(res[j]), srows[j], n, s)) !=
          cudaSuccess)
        return cuda_fail(e, "MapSum seed broadcast");
      a.out[j] = rows_io(srows[j], k, n);
    }
  }
  if (int rc = primal_launch(*t, a, n, PK_SP_REVERSE, s)) return rc;
  for (int j = 0; j < t->n_in; ++j)
    if (arows[j] && (e = reduce_or(t->nnz_in[j], n, arows[j], n,
                                   reinterpret_cast<u64*>(arg[j]), true, s)) != cudaSuccess)
      return cuda_fail(e, "MapSum OR reduction");
  for (int j = 0; j < t->n_out; ++j)
    if (srows[j] &&
        (e = cudaMemsetAsync(res[j], 0, 8 * static_cast<size_t>(t->nnz_out[j]), s)) != cudaSuccess)
      return cuda_fail(e, "MapSum clear");
  return 0;
}

}  // extern "C"

// ---- Mapaccum: N chained calls of one tape (Function::mapaccum, casadi/core/function.cpp) ----
namespace {

int accum_check(const Tape& t, int N, int n_accum) {
  if (N < 1) return fail(CASADI_GB300_ERR_ARG, "mapaccum: N must be positive");
  if (n_accum < 0 || n_accum > std::min(t.n_in, t.n_out))
    return fail(CASADI_GB300_ERR_ARG, "mapaccum: %d accumulators for %d inputs and %d outputs",
                n_accum, t.n_in, t.n_out);
  for (int i = 0; i < n_accum; ++i)
    if (t.nnz_in[i] != t.nnz_out[i])
      return fail(CASADI_GB300_ERR_ARG,
                  "mapaccum: accumulator %d has %d input but %d output nonzeros", i,
                  t.nnz_in[i], t.nnz_out[i]);
  return 0;
}

// Block k of a stacked input/output: nonzeros [k*nnz, (k+1)*nnz) of an (nnz*N, ld) array, and
// of each direction of an (ndir, nnz*N, ld) one.
IoDesc step_io(const void* base, int nnz, int N, int k, long long ld) {
  if (!base) return IoDesc{nullptr, ld, 1, 0};
  return IoDesc{const_cast<char*>(static_cast<const char*>(base)) +
                    static_cast<size_t>(k) * nnz * ld * sizeof(double),
                ld, 1, static_cast<long long>(nnz) * N * ld};
}
// A contiguous (ndir, nnz, n) block of the scratch.
IoDesc block_io(void* p, int nnz, long long n) {
  return IoDesc{p, n, 1, static_cast<long long>(nnz) * n};
}

size_t bytes_of(long long count) { return ((static_cast<size_t>(count) * 8 + 255) / 256) * 256; }

// Accumulator values of step k-1 (the input of step k > 0): the caller's output block, or the
// scratch copy (history: every step kept, for the reverse sweep; else two alternating blocks).
struct AccumValues {
  const double* const* res;
  double* keep[kMaxIo] = {};
  bool history = false;
  IoDesc value(int i, int nnz, int N, int k, long long n, long long ld) const {
    if (res && res[i]) return step_io(res[i], nnz, N, k, ld);
    double* p = keep[i] + static_cast<size_t>(history ? k : (k & 1)) * nnz * n;
    return IoDesc{p, n, 1, 0};
  }
};

int accum_values(const Tape& t, int N, int n_accum, long long n, const double* const* res,
                 bool history, Arena& ar, AccumValues* v) {
  v->res = res;
  v->history = history;
  for (int i = 0; i < n_accum; ++i) {
    if (res && res[i]) continue;
    v->keep[i] = static_cast<double*>(
        ar.take(bytes_of(static_cast<long long>(t.nnz_out[i]) * n * (history ? N : 2))));
    if (!v->keep[i])
      return fail(CASADI_GB300_ERR_SCRATCH,
                  "mapaccum scratch too small (see casadi_gb300_mapaccum_scratch_size)");
  }
  return 0;
}

// The value sweep of every step: inputs of step k from arg / the previous step's outputs.
// Partials scratch of one call over n instances (tile-major, as run_ad_multi lays it out).
size_t accum_call_partials(const Tape& t, long long n) {
  return static_cast<size_t>(8) * t.n_partials * static_cast<size_t>(((n + 31) / 32) * 32);
}

// The N calls forward. With `partials`, each call is a record sweep that leaves its partials at
// partials + k * accum_call_partials (the reverse sweep then needs no record of its own);
// otherwise a value sweep.
int accum_forward_values(Tape& t, int N, int n_accum, long long n, long long ld,
                         const double* const* arg, double* const* res, const AccumValues& v,
                         cudaStream_t s, char* partials = nullptr) {
  for (int k = 0; k < N; ++k) {
    SweepArgs a = base_args(t, n, 0);
    if (partials) {
      a.partials = reinterpret_cast<double*>(partials + k * accum_call_partials(t, n));
      a.pofs = t.d_pofs;
      a.n_code = t.n_chunks * kChunk;
      for (int j = 0, off = 0; j < t.n_in; off += t.nnz_in[j], ++j) a.in_off[j] = off;
    }
    for (int j = 0; j < t.n_in; ++j) {
      const int nz = t.nnz_in[j];
      if (j < n_accum)
        a.in[j] = k == 0 ? plain_io(at(arg, j), nz, ld, false) : v.value(j, nz, N, k - 1, n, ld);
      else
        a.in[j] = step_io(at(arg, j), nz, N, k, ld);
    }
    for (int j = 0; j < t.n_out; ++j)
      a.out[j] = j < n_accum ? v.value(j, t.nnz_out[j], N, k, n, ld)
                             : step_io(res ? res[j] : nullptr, t.nnz_out[j], N, k, ld);
    if (int rc = primal_launch(t, a, n, partials ? PK_RECORD : PK_EVAL, s)) return rc;
  }
  return 0;
}

}  // namespace

extern "C" {

int casadi_gb300_mapaccum_scratch_size(int id, int N, int n_accum, int64_t n, int ndir,
                                       size_t* bytes) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (!bytes || n < 0 || ndir < 0) return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  if (int rc = accum_check(*t, N, n_accum)) return rc;
  size_t b = 512;
  for (int i = 0; i < n_accum; ++i) {
    const long long nz = t->nnz_out[i];
    b += bytes_of(nz * n * std::max(N, 2));                // accumulator values
    b += 3 * bytes_of(static_cast<long long>(std::max(ndir, 1)) * nz * n);  // tangents/adjoints
  }
  b += static_cast<size_t>(8) * t->n_partials * static_cast<size_t>(((n + 31) / 32) * 32);
  *bytes = b + kQueueSlack;
  return 0;
}

int casadi_gb300_mapaccum_eval(int id, int N, int n_accum, int64_t n, int64_t ld,
                               const double* const* arg, double* const* res, void* scratch,
                               size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (int rc = accum_check(*t, N, n_accum)) return rc;
  if (n == 0) return 0;
  Arena ar(scratch, scratch_bytes);
  AccumValues v;
  if (int rc = accum_values(*t, N, n_accum, n, res, false, ar, &v)) return rc;
  return accum_forward_values(*t, N, n_accum, n, ld, arg, res, v,
                              static_cast<cudaStream_t>(stream));
}

int casadi_gb300_mapaccum_forward(int id, int N, int n_accum, int64_t n, int64_t ld, int nfwd,
                                  const double* const* arg, double* const* res,
                                  const double* const* fseed, double* const* fsens,
                                  void* scratch, size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (int rc = accum_check(*t, N, n_accum)) return rc;
  if (nfwd < 1 || nfwd > 65535) return fail(CASADI_GB300_ERR_ARG, "bad direction count %d", nfwd);
  if (n == 0) return 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Arena ar(scratch, scratch_bytes);
  AccumValues v;
  if (int rc = accum_values(*t, N, n_accum, n, res, false, ar, &v)) return rc;
  // accumulator tangents the caller does not keep: two alternating blocks
  double* ttmp[kMaxIo] = {};
  for (int i = 0; i < n_accum; ++i) {
    if (fsens && fsens[i]) continue;
    ttmp[i] = static_cast<double*>(ar.take(bytes_of(2ll * nfwd * t->nnz_out[i] * n)));
    if (!ttmp[i])
      return fail(CASADI_GB300_ERR_SCRATCH,
                  "mapaccum scratch too small (see casadi_gb300_mapaccum_scratch_size)");
  }
  auto tangent = [&](int i, int k) -> IoDesc {
    const int nz = t->nnz_out[i];
    if (fsens && fsens[i]) return step_io(fsens[i], nz, N, k, ld);
    return block_io(ttmp[i] + static_cast<size_t>(k & 1) * nfwd * nz * n, nz, n);
  };
  for (int k = 0; k < N; ++k) {
    IoDesc in[kMaxIo], out[kMaxIo], seed[kMaxIo], sens[kMaxIo];
    for (int j = 0; j < t->n_in; ++j) {
      const int nz = t->nnz_in[j];
      if (j < n_accum) {
        in[j] = k == 0 ? plain_io(at(arg, j), nz, ld, false) : v.value(j, nz, N, k - 1, n, ld);
        seed[j] = k == 0 ? plain_io(at(fseed, j), nz, ld, true) : tangent(j, k - 1);
      } else {
        in[j] = step_io(at(arg, j), nz, N, k, ld);
        seed[j] = step_io(at(fseed, j), nz, N, k, ld);
      }
    }
    for (int j = 0; j < t->n_out; ++j) {
      const int nz = t->nnz_out[j];
      out[j] = j < n_accum ? v.value(j, nz, N, k, n, ld)
                           : step_io(res ? res[j] : nullptr, nz, N, k, ld);
      sens[j] = j < n_accum ? tangent(j, k) : step_io(fsens ? fsens[j] : nullptr, nz, N, k, ld);
    }
    if (int rc = run_ad(*t, n, in, out, seed, sens, nfwd, false, false, ar.p, ar.left, s))
      return rc;
  }
  return 0;
}

int casadi_gb300_mapaccum_reverse(int id, int N, int n_accum, int64_t n, int64_t ld, int nadj,
                                  const double* const* arg, double* const* res,
                                  const double* const* aseed, double* const* asens,
                                  void* scratch, size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (int rc = accum_check(*t, N, n_accum)) return rc;
  if (nadj < 1 || nadj > 65535) return fail(CASADI_GB300_ERR_ARG, "bad direction count %d", nadj);
  if (n == 0) return 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Arena ar(scratch, scratch_bytes);
  // every step's accumulator values are kept (the caller's outputs or a scratch history): the
  // reverse sweep of step k records it again from its inputs
  AccumValues v;
  if (int rc = accum_values(*t, N, n_accum, n, res, true, ar, &v)) return rc;
  // adjoints of the accumulator inputs, carried from step k+1 to step k, and the combined
  // seeds of the accumulator outputs
  double* carry[kMaxIo] = {};
  double* cseed[kMaxIo] = {};
  for (int i = 0; i < n_accum; ++i) {
    const long long blk = static_cast<long long>(nadj) * t->nnz_out[i] * n;
    carry[i] = static_cast<double*>(ar.take(bytes_of(2 * blk)));
    cseed[i] = static_cast<double*>(ar.take(bytes_of(blk)));
    if (!carry[i] || !cseed[i])
      return fail(CASADI_GB300_ERR_SCRATCH,
                  "mapaccum scratch too small (see casadi_gb300_mapaccum_scratch_size)");
  }
  // with room for every call's partials (casadi_gb300_mapaccum_reverse_scratch_size), the
  // forward pass records them and the reverse pass runs adjoint sweeps only; otherwise each
  // call is recorded again from its checkpointed inputs on the way back
  const size_t per_call = accum_call_partials(*t, n);
  char* recorded = nullptr;
  if (t->n_partials > 0 && ar.left >= per_call * static_cast<size_t>(N) + kQueueSlack)
    recorded = static_cast<char*>(ar.take(per_call * static_cast<size_t>(N)));
  if (int rc = accum_forward_values(*t, N, n_accum, n, ld, arg, res, v, s, recorded)) return rc;
  for (int k = N - 1; k >= 0; --k) {
    IoDesc in[kMaxIo], out[kMaxIo], seed[kMaxIo], sens[kMaxIo];
    for (int j = 0; j < t->n_out; ++j) {
      const int nz = t->nnz_out[j];
      out[j] = IoDesc{nullptr, ld, 1, 0};  // the values were written by the value sweeps
      if (j < n_accum) {
        // seed of x_{k+1}: its own adjoint seed plus what step k+1 passed back
        const double* a_blk = aseed && aseed[j] ? aseed[j] + static_cast<size_t>(k) * nz * ld
                                                : nullptr;
        const double* prev = k < N - 1 ? carry[j] + static_cast<size_t>((k + 1) & 1) * nadj * nz * n
                                       : nullptr;
        cudaError_t e = add_blocks(nadj, nz, n, a_blk, ld, static_cast<long long>(nz) * N * ld,
                                   prev, cseed[j], s);
        if (e != cudaSuccess) return cuda_fail(e, "mapaccum seeds");
        seed[j] = block_io(cseed[j], nz, n);
      } else {
        seed[j] = step_io(at(aseed, j), nz, N, k, ld);
      }
    }
    for (int j = 0; j < t->n_in; ++j) {
      const int nz = t->nnz_in[j];
      if (j < n_accum) {
        in[j] = k == 0 ? plain_io(at(arg, j), nz, ld, false) : v.value(j, nz, N, k - 1, n, ld);
        sens[j] = k == 0 ? plain_io(asens ? asens[j] : nullptr, nz, ld, true)
                         : block_io(carry[j] + static_cast<size_t>(k & 1) * nadj * nz * n, nz, n);
      } else {
        in[j] = step_io(at(arg, j), nz, N, k, ld);
        sens[j] = step_io(asens ? asens[j] : nullptr, nz, N, k, ld);
      }
    }
    if (recorded) {
      if (int rc = run_ad(*t, n, in, out, seed, sens, nadj, true, false,
                          recorded + static_cast<size_t>(k) * per_call, per_call, s, true))
        return rc;
    } else if (int rc = run_ad(*t, n, in, out, seed, sens, nadj, true, false, ar.p, ar.left, s)) {
      return rc;
    }
  }
  return 0;
}

// Scratch for the mapaccum reverse sweep that records every call's partials on the way
// forward: casadi_gb300_mapaccum_scratch_size plus N calls' partials.
int casadi_gb300_mapaccum_reverse_scratch_size(int id, int N, int n_accum, int64_t n, int nadj,
                                               size_t* bytes) {
  if (int rc = casadi_gb300_mapaccum_scratch_size(id, N, n_accum, n, nadj, bytes)) return rc;
  const Tape* t = get_tape(id);
  *bytes += accum_call_partials(*t, n) * static_cast<size_t>(std::max(N, 0)) + 256;
  return 0;
}

}  // extern "C"

// ---- Self-check of the bounded waits ------------------------------------------------------
extern "C" {

int casadi_gb300_check_wait_timeout(void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned* words = nullptr;  // [0] a flag nothing sets, [1] the error word
  cudaError_t e = cudaMalloc(&words, 2 * sizeof(unsigned));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(wait probe)");
  unsigned host[2] = {0, 0};
  if ((e = cudaMemsetAsync(words, 0, 2 * sizeof(unsigned), s)) == cudaSuccess &&
      (e = launch_wait_probe(words, words + 1, s)) == cudaSuccess &&
      (e = cudaMemcpyAsync(host, words, sizeof(host), cudaMemcpyDeviceToHost, s)) == cudaSuccess)
    e = cudaStreamSynchronize(s);
  cudaFree(words);
  if (e != cudaSuccess) return cuda_fail(e, "wait probe");
  if (host[1] & kErrWaitTimeout)
    return fail(CASADI_GB300_ERR_DEVICE, "bounded wait ran out (flag never set)");
  return fail(CASADI_GB300_ERR_CUDA, "bounded wait did not report its timeout");
}

}  // extern "C"
