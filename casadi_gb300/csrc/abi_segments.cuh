// C ABI: the adjoint with segment checkpointing.
//
// Part of the abi.cu translation unit (included at its end): it uses that file's internal
// registry, encoder and launch helpers and is not compiled on its own.
#pragma once

// ---------------------------------------------------------------------------------------------
// Segment checkpointing of the adjoint sweep.
//
// The plain adjoint records every instruction's partials for all instances before the reverse
// walk (8 bytes x partials x instances; instance waves bound it). With checkpointing the
// scheduled tape is cut into K runs of consecutive instructions. A cut is placed near an equal
// share of the recorded partials, where the fewest work-vector slots are live (read later
// before being overwritten). Each run becomes an ordinary tape of this library: its inputs are
// the tape's inputs plus one more, the slots live at its first cut; its outputs are the tape's
// outputs (those its instructions write) plus one more, the slots live at its last cut.
//
//   forward:  segments 0 .. K-2 evaluated in order; the live slots at every cut are kept
//             (the checkpoints: every k-th work vector, restricted to what is still read);
//   backward: segments K-1 .. 0, each re-recorded from its checkpoint and swept in reverse,
//             seeded with the adjoints of the slots live at its end, giving those of the slots
//             live at its start.
//
// Partials are held for one segment at a time, so the scratch shrinks by about K while the
// values are computed twice. This is the numeric counterpart of the reference's reverse sweep
// (SXFunction::ad_reverse, casadi/core/sx_function.cpp:1454-1560) over a stored work vector,
// with the storage traded for recomputation. The adjoint sums of a slot may associate
// differently across a cut (each segment tape is scheduled on its own), so results equal the
// unsegmented sweep up to rounding; values are identical.
// ---------------------------------------------------------------------------------------------
namespace {

struct SegmentPlan {
  std::vector<int> cut;                              // K + 1 positions in the instruction list
  std::vector<std::vector<int>> live;                // live slots at each cut
  std::vector<std::vector<casadi_gb300_atomic>> alg;  // the segment tapes, reference format
};

// Slots an instruction reads (count returned) and the slot it writes (-1: none).
int seg_reads(u64 w, int r[2]) {
  const unsigned op = dec_op(w);
  if (op == D_NOP || op == D_CONST || op == D_INPUT) return 0;
  r[0] = static_cast<int>(dec_b(w));
  if (op == D_OUTPUT || !is_binary(op)) return 1;
  r[1] = static_cast<int>(dec_c(w));
  return 2;
}

int seg_writes(u64 w) {
  const unsigned op = dec_op(w);
  return (op == D_NOP || op == D_OUTPUT) ? -1 : static_cast<int>(dec_a(w));
}

// Plans K segments of the encoded (scheduled) instruction list `code`. The segment tapes keep
// the tape's slot numbering (sz_w slots) and its input and output indices; the live slots enter
// as input n_in and leave as output n_out.
int plan_segments(const std::vector<u64>& code_in, const std::vector<double>& consts, int n_in,
                  int n_out, int sz_w, int k, SegmentPlan& p) {
  if (k < 1) return fail(CASADI_GB300_ERR_ARG, "segment count %d < 1", k);
  if (n_in + 1 > kMaxIo || n_out + 1 > kMaxIo)
    return fail(CASADI_GB300_ERR_UNSUPPORTED,
                "checkpointing needs one input and one output beyond the tape's (max %d)", kMaxIo);
  std::vector<u64> code;
  code.reserve(code_in.size());
  for (u64 w : code_in)
    if (dec_op(w) != D_NOP) code.push_back(w);
  const int L = static_cast<int>(code.size());
  k = std::max(1, std::min(k, L));
  // live slot count before each position, from a backward pass
  std::vector<int> nlive(L + 1, 0);
  std::vector<char> live(std::max(1, sz_w), 0);
  int cnt = 0;
  auto step = [&](u64 w) {
    const int d = seg_writes(w);
    if (d >= 0 && live[d]) {
      live[d] = 0;
      --cnt;
    }
    int r[2];
    const int nr = seg_reads(w, r);
    for (int i = 0; i < nr; ++i)
      if (!live[r[i]]) {
        live[r[i]] = 1;
        ++cnt;
      }
  };
  for (int q = L - 1; q >= 0; --q) {
    step(code[q]);
    nlive[q] = cnt;
  }
  if (L > 0 && nlive[0] != 0)
    return fail(CASADI_GB300_ERR_ARG, "the tape reads %d slots before writing them", nlive[0]);
  // work of each instruction: one, plus its recorded partials
  std::vector<long long> acc(L + 1, 0);
  for (int q = 0; q < L; ++q) {
    const unsigned op = dec_op(code[q]);
    long long wq = 1;
    if (op != D_CONST && op != D_INPUT && op != D_OUTPUT)
      wq += __builtin_popcount(partial_mask(op));
    acc[q + 1] = acc[q] + wq;
  }
  p.cut.assign(k + 1, 0);
  p.cut[k] = L;
  const int win = std::max(1, L / (8 * k));
  for (int s = 1; s < k; ++s) {
    const long long target = acc[L] * s / k;
    const int c0 =
        static_cast<int>(std::lower_bound(acc.begin(), acc.end(), target) - acc.begin());
    const int lo = p.cut[s - 1] + 1, hi = L - (k - s);
    auto dist = [c0](int c) { return c > c0 ? c - c0 : c0 - c; };
    int best = std::min(std::max(c0, lo), hi);
    for (int c = std::max(lo, c0 - win); c <= std::min(hi, c0 + win); ++c)
      if (nlive[c] < nlive[best] || (nlive[c] == nlive[best] && dist(c) < dist(best)))
        best = c;
    p.cut[s] = best;
  }
  // the live sets at the cuts
  p.live.assign(k + 1, {});
  std::fill(live.begin(), live.end(), 0);
  cnt = 0;
  for (int q = L - 1, s = k - 1; q >= 0; --q) {
    step(code[q]);
    for (; s >= 0 && p.cut[s] == q; --s)
      for (int v = 0; v < sz_w; ++v)
        if (live[v]) p.live[s].push_back(v);
  }
  // the segment tapes
  p.alg.assign(k, {});
  for (int s = 0; s < k; ++s) {
    std::vector<casadi_gb300_atomic>& a = p.alg[s];
    a.reserve(p.live[s].size() + (p.cut[s + 1] - p.cut[s]) + p.live[s + 1].size());
    for (size_t i = 0; i < p.live[s].size(); ++i) {
      casadi_gb300_atomic e;
      std::memset(&e, 0, sizeof(e));
      e.op = kOpInput;
      e.i0 = p.live[s][i];
      e.a.i[0] = n_in;
      e.a.i[1] = static_cast<int>(i);
      a.push_back(e);
    }
    for (int q = p.cut[s]; q < p.cut[s + 1]; ++q) a.push_back(decode_atomic(code[q], consts));
    for (size_t i = 0; i < p.live[s + 1].size(); ++i) {
      casadi_gb300_atomic e;
      std::memset(&e, 0, sizeof(e));
      e.op = kOpOutput;
      e.i0 = n_out;
      e.a.i[0] = p.live[s + 1][i];
      e.a.i[1] = static_cast<int>(i);
      a.push_back(e);
    }
  }
  return k;
}

// Builds the segment tapes of `t` for `k` segments (caller holds t.seg_mtx).
int ensure_segments(Tape& t, int k) {
  if (t.seg_req == k && !t.seg.empty()) return 0;
  SegmentPlan p;
  const int kk = plan_segments(t.h_code, t.h_consts, t.n_in, t.n_out, t.sz_w, k, p);
  if (kk < 0) return kk;
  std::vector<std::unique_ptr<Tape>> seg(kk);
  std::vector<int> nnz_in(t.nnz_in), nnz_out(t.nnz_out);
  nnz_in.push_back(0);
  nnz_out.push_back(0);
  // the tape's never-read inputs get their zero sensitivities from the first segment; in the
  // others an input nonzero that is not read belongs to another segment and is left alone
  const std::vector<int2> none;
  for (int s = 0; s < kk; ++s) {
    nnz_in.back() = static_cast<int>(p.live[s].size());
    nnz_out.back() = static_cast<int>(p.live[s + 1].size());
    if (int rc = make_tape(p.alg[s].data(), static_cast<int>(p.alg[s].size()), t.n_in + 1,
                           nnz_in.data(), t.n_out + 1, nnz_out.data(), t.sz_w, false,
                           s == 0 ? &t.absent_in : &none, seg[s]))
      return rc;
  }
  t.seg.swap(seg);
  t.seg_live.swap(p.live);
  t.seg_count = kk;
  t.seg_req = k;
  return 0;
}

size_t seg_align(size_t b) { return (b + 255) & ~static_cast<size_t>(255); }

// Scratch layout of a checkpointed call: checkpoints of cuts 1 .. K-1, then two adjoint
// buffers of the largest live set, then the partials of one segment.
struct SegLayout {
  std::vector<size_t> ckpt;  // offset of each cut's checkpoint (K + 1 entries)
  size_t adj[2] = {0, 0};
  size_t partials = 0;       // offset of the partials scratch
  size_t partials_full = 0;  // its size for one wave of all instances
  size_t partials_min = 0;   // its minimum (one warp of instances)
};

SegLayout seg_layout(const Tape& t, long long n, int nadj) {
  SegLayout l;
  const int k = t.seg_count;
  size_t off = 0;
  l.ckpt.assign(k + 1, 0);
  size_t maxlive = 0;
  for (int s = 0; s <= k; ++s) {
    l.ckpt[s] = off;
    if (s > 0 && s < k) off += seg_align(8ull * t.seg_live[s].size() * n);
    maxlive = std::max(maxlive, t.seg_live[s].size());
  }
  for (int b = 0; b < 2; ++b) {
    l.adj[b] = off;
    off += seg_align(8ull * maxlive * static_cast<size_t>(std::max(nadj, 0)) * n);
  }
  l.partials = off;
  long long most = 0;
  for (const auto& g : t.seg) most = std::max<long long>(most, g->n_partials);
  l.partials_full = 8ull * most * static_cast<size_t>(((n + 31) / 32) * 32) + kQueueSlack;
  l.partials_min = 8ull * most * 32 + kQueueSlack;
  return l;
}

}  // namespace

extern "C" {

int casadi_gb300_tape_segments(const casadi_gb300_atomic* alg, int n_instr, int n_in,
                               const int* nnz_in, int n_out, const int* nnz_out, int sz_w,
                               int segments, int* cut, int* live_count, int* seg_len,
                               casadi_gb300_atomic* seg_alg, int capacity, int* sz_w_out) {
  if (!cut || !live_count || !seg_len || !sz_w_out || capacity < 0 || (capacity > 0 && !seg_alg))
    return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  Encoded en;
  const int wlen = encode_and_schedule(alg, n_instr, n_in, nnz_in, n_out, nnz_out, sz_w, en);
  if (wlen < 0) return wlen;
  SegmentPlan p;
  const int k = plan_segments(en.code, en.consts, n_in, n_out, wlen, segments, p);
  if (k < 0) return k;
  size_t total = 0;
  for (const auto& a : p.alg) total += a.size();
  if (total > static_cast<size_t>(capacity))
    return fail(CASADI_GB300_ERR_ARG, "segment tapes need %zu instructions, capacity %d", total,
                capacity);
  for (int s = 0; s <= k; ++s) {
    cut[s] = p.cut[s];
    live_count[s] = static_cast<int>(p.live[s].size());
  }
  size_t off = 0;
  for (int s = 0; s < k; ++s) {
    seg_len[s] = static_cast<int>(p.alg[s].size());
    std::memcpy(seg_alg + off, p.alg[s].data(), p.alg[s].size() * sizeof(casadi_gb300_atomic));
    off += p.alg[s].size();
  }
  *sz_w_out = wlen;
  return k;
}

int casadi_gb300_checkpoint_scratch_size(int id, int segments, int nadj, int64_t n,
                                         size_t* bytes, size_t* min_bytes) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (n < 0 || nadj < 0 || nadj > 65535 || (!bytes && !min_bytes))
    return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  if (int rc = check_device(*t)) return rc;
  std::lock_guard<std::mutex> lk(t->seg_mtx);
  if (int rc = ensure_segments(*t, segments)) return rc;
  const SegLayout l = seg_layout(*t, n, nadj);
  if (bytes) *bytes = l.partials + l.partials_full;
  if (min_bytes) *min_bytes = l.partials + l.partials_min;
  return t->seg_count;
}

int casadi_gb300_reverse_checkpointed(int id, int64_t n, int64_t ld, int nadj, int segments,
                                      const double* const* arg, double* const* res,
                                      const double* const* aseed, double* const* asens,
                                      void* scratch, size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (nadj < 0 || nadj > 65535) return fail(CASADI_GB300_ERR_ARG, "bad direction count %d", nadj);
  std::lock_guard<std::mutex> lk(t->seg_mtx);
  if (int rc = ensure_segments(*t, segments)) return rc;
  if (n == 0) return 0;
  const int k = t->seg_count;
  const SegLayout l = seg_layout(*t, n, nadj);
  if (!scratch || scratch_bytes < l.partials + l.partials_min)
    return fail(CASADI_GB300_ERR_SCRATCH,
                "scratch of %zu bytes is below the minimum of %zu bytes for %d segments",
                scratch_bytes, l.partials + l.partials_min, k);
  unsigned char* base = static_cast<unsigned char*>(scratch);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  IoDesc in[kMaxIo], out[kMaxIo], seed[kMaxIo], sens[kMaxIo];
  fill_io(in, t->n_in, vptrs(arg), t->nnz_in, ld, false);
  fill_io(out, t->n_out, vptrs(res), t->nnz_out, ld, false);
  fill_io(seed, t->n_out, vptrs(aseed), t->nnz_out, ld, true);
  fill_io(sens, t->n_in, vptrs(asens), t->nnz_in, ld, true);
  // the live slots at cut s (none at the tape's ends): values, instance-minor, leading dim n
  auto ckpt = [&](int s) {
    IoDesc d;
    std::memset(&d, 0, sizeof(d));
    if (s > 0 && s < k && !t->seg_live[s].empty()) d.ptr = base + l.ckpt[s];
    d.nz_stride = n;
    d.inst_stride = 1;
    return d;
  };
  // their adjoints, direction-major; cut s uses buffer s % 2
  auto adj = [&](int s) {
    IoDesc d;
    std::memset(&d, 0, sizeof(d));
    if (s > 0 && s < k && !t->seg_live[s].empty()) d.ptr = base + l.adj[s & 1];
    d.nz_stride = n;
    d.inst_stride = 1;
    d.dir_stride = static_cast<long long>(t->seg_live[s].size()) * n;
    return d;
  };
  const int nfwd_segs = nadj > 0 ? k - 1 : k;
  for (int s = 0; s < nfwd_segs; ++s) {
    Tape& g = *t->seg[s];
    SweepArgs a = base_args(g, n, 0);
    std::memcpy(a.in, in, sizeof(IoDesc) * t->n_in);
    a.in[t->n_in] = ckpt(s);
    std::memcpy(a.out, out, sizeof(IoDesc) * t->n_out);
    a.out[t->n_out] = ckpt(s + 1);
    if (int rc = primal_launch(g, a, n, PK_EVAL, st)) return rc;
  }
  if (nadj == 0) return 0;
  IoDesc null_io;
  std::memset(&null_io, 0, sizeof(null_io));
  for (int s = k - 1; s >= 0; --s) {
    Tape& g = *t->seg[s];
    IoDesc gin[kMaxIo], gout[kMaxIo], gseed[kMaxIo], gsens[kMaxIo];
    std::memcpy(gin, in, sizeof(IoDesc) * t->n_in);
    gin[t->n_in] = ckpt(s);
    // the last segment's record sweep writes its values; the others' went out going forward
    for (int j = 0; j < t->n_out; ++j) gout[j] = s == k - 1 ? out[j] : null_io;
    gout[t->n_out] = null_io;
    std::memcpy(gseed, seed, sizeof(IoDesc) * t->n_out);
    gseed[t->n_out] = adj(s + 1);
    std::memcpy(gsens, sens, sizeof(IoDesc) * t->n_in);
    gsens[t->n_in] = adj(s);
    if (int rc = run_ad(g, n, gin, gout, gseed, gsens, nadj, true, false, base + l.partials,
                        scratch_bytes - l.partials, st))
      return rc;
  }
  return 0;
}

}  // extern "C"
