// C ABI of the GB300 SX-tape evaluator (declared in include/casadi_gb300.h).
//
// Host side: tape registry (int ids, as casadi/core/casadi_c.cpp:73-110 keeps Functions),
// host validation of every tape index before anything reaches the GPU, instruction encoding,
// launch-shape selection from the shared-memory footprint, and the wave loop that bounds
// the AD scratch. No exception crosses the ABI: every entry point returns a status and
// records a message for casadi_gb300_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/casadi_gb300.h"
#include "coloring.cuh"
#include "schedule.cuh"
#include "reduce.cuh"
#include "serial.cuh"
#include "sweeps.cuh"

using namespace cgb;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(CASADI_GB300_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// CasADi operation ids (casadi/core/calculus.hpp:60-218) of the scalar ops numbered above
// OP_CALL, and their device opcodes.
constexpr int kOpConst = 44, kOpInput = 45, kOpOutput = 46, kOpParameter = 47, kOpCall = 48;

int device_opcode(int op) {
  if (op >= 0 && op <= 43) return op;  // ASSIGN .. ATAN2 keep their ids
  switch (op) {
    case kOpConst: return D_CONST;
    case kOpInput: return D_INPUT;
    case kOpOutput: return D_OUTPUT;
    case 86: return D_ERFINV;
    case 87: return D_PRINTME;
    case 88: return D_LIFT;
    case 93: return D_LOG1P;
    case 94: return D_EXPM1;
    case 95: return D_HYPOT;
    case 97: return D_REMAINDER;
    default: return -1;
  }
}

int reference_opcode(unsigned dop) {
  if (dop <= 43) return static_cast<int>(dop);
  switch (dop) {
    case D_CONST: return kOpConst;
    case D_INPUT: return kOpInput;
    case D_OUTPUT: return kOpOutput;
    case D_ERFINV: return 86;
    case D_PRINTME: return 87;
    case D_LIFT: return 88;
    case D_LOG1P: return 93;
    case D_EXPM1: return 94;
    case D_HYPOT: return 95;
    case D_REMAINDER: return 97;
    default: return -1;
  }
}

// Activity plan of the tangent sweep for one seed pattern and launch shape.
struct TanPlan {
  int ndir = 0, dw = 0, ch = 0;
  bool identity = false;
  std::vector<int> dirmap;   // identity mode: direction seeded by each flat input nonzero
                             // (empty: nonzero k seeds direction k; -1: not seeded)
  std::vector<char> seeded;  // per input: seed pointer given (general seeds)
  std::vector<char> wanted;  // per output: sensitivities requested (others are pruned)
  int groups = 0;
  // keyed entry streams of all direction groups, one layout per group size (group_slot)
  uint4* d_stream[kNumGroupSizes] = {};
  int2* d_chunks[kNumGroupSizes] = {};  // per direction group: (first entry, body entries)
  std::vector<int2> h_chunks[kNumGroupSizes];
  int* d_dirmap = nullptr;    // identity mode with a dirmap: its device copy
  int* d_order = nullptr;     // groups in work order, longest stream first (null: natural)
  ~TanPlan() {
    for (int g = 0; g < kNumGroupSizes; ++g) {
      cudaFree(d_stream[g]);
      cudaFree(d_chunks[g]);
    }
    cudaFree(d_dirmap);
    cudaFree(d_order);
  }
};

// Window plan of the windowed tangent sweep (k_tangent_win) for one seed pattern: the tape cut
// into windows, each window's entry block per direction group, and the launch shape.
struct WinPlan {
  int ndir = 0;
  bool identity = false;
  std::vector<int> dirmap;
  std::vector<char> seeded;
  std::vector<char> wanted;
  bool usable = false;  // false: the sweep does not fit (or has too few directions to pay)
  int dirs = 0, groups = 0, stages = 0, rows = 0, ents = 0, nwin = 0;
  uint4* d_blocks = nullptr;
  int4* d_meta = nullptr;
  ~WinPlan() {
    cudaFree(d_blocks);
    cudaFree(d_meta);
  }
};

// Activity plan of the adjoint sweep for one pattern of seeded outputs and chunk size.
struct AdjPlan {
  int ch = 0;
  std::vector<char> seeded;  // per output: seed pointer given
  int dw = 0;
  // keyed entry stream, one layout per group size (group_slot)
  uint4* d_stream[kNumGroupSizes] = {};
  int2* d_chunks[kNumGroupSizes] = {};  // (first entry, body entries)
  int2 h_chunks[kNumGroupSizes] = {};
  int2* d_zero = nullptr;
  int n_zero = 0;
  ~AdjPlan() {
    for (int g = 0; g < kNumGroupSizes; ++g) {
      cudaFree(d_stream[g]);
      cudaFree(d_chunks[g]);
    }
    cudaFree(d_zero);
  }
};

struct Tape {
  int device = 0;
  int n_instr = 0, n_in = 0, n_out = 0, sz_w = 0, n_partials = 0, n_chunks = 0;
  int ref_sz_w = 0;  // the work-vector length the tape came with (sz_w: after scheduling)
  int residence = 0;  // work vector: 0 auto (shared memory when it fits, value sweeps tuned),
                      // 1 global memory, 2 shared memory whenever it fits
  // per PrimalKind and launch size class (0: at most 16 tiles per SM): 0 shared, 1 global,
  // 2 cooperative level sweep (autotuned)
  std::atomic<int> primal_tuned[5][2];
  // level schedule of the cooperative value/record sweeps, built on first use
  int lv_state = 0;  // 0 not built, 1 built, -1 unavailable
  u64* d_lcode = nullptr;
  int* d_lbegin = nullptr;
  int* d_lpidx = nullptr;
  int n_levels = 0, lv_sz_w = 0;
  // the reverse sweep's level schedule (users of each value in order), built on first use
  int rlv_state = 0;
  u64* d_rcode = nullptr;
  int* d_rbegin = nullptr;
  int* d_rpidx = nullptr;
  int n_rlevels = 0, rlv_sz_w = 0;
  // global work vector: per-CTA blocks, grown on demand; uses on different streams are
  // ordered by gw_event
  std::mutex gw_mtx;
  unsigned char* d_gw = nullptr;
  size_t gw_cap = 0;
  cudaEvent_t gw_event = nullptr;
  bool gw_recorded = false;
  std::vector<int> nnz_in, nnz_out;
  std::vector<int2> absent_in;
  std::vector<int> pofs;    // partials recorded before instruction k*kPofsGran
  u64* d_code = nullptr;
  int* d_pofs = nullptr;
  double* d_consts = nullptr;
  int2* d_absent = nullptr;
  int* d_err = nullptr;
  // launch shapes
  int primal_block = 128, primal_grid_cap = 1;
  std::mutex shape_mtx;
  // derivative-sweep variant per kind (seeded/identity tangent, adjoint) and launch size class
  // (0: at most 16 tiles per SM); tangent kinds may keep the cooperative sweep (TV_COUNT)
  std::atomic<int> tuned[3][2];
  // one thread tunes a tape at a time; others meanwhile run the untuned defaults
  std::mutex tune_mtx;
  Tape() {
    for (auto& k : primal_tuned) k[0] = k[1] = -1;
    for (auto& k : tuned) k[0] = k[1] = -1;
  }
  std::vector<double> h_consts;  // constant pool (host copy, for inlining into callers)
  std::vector<u64> h_code;                            // padded instruction stream
  std::vector<std::unique_ptr<TanPlan>> tan_plans;
  std::vector<std::unique_ptr<WinPlan>> win_plans;
  std::vector<std::unique_ptr<AdjPlan>> adj_plans;
  // the checkpointed adjoint's segment tapes, for one segment count at a time (seg_count 0:
  // none yet); calls on this tape's checkpointed entry point are serialised by seg_mtx
  std::mutex seg_mtx;
  int seg_count = 0, seg_req = 0;                 // segments made, segments asked for
  std::vector<std::vector<int>> seg_live;         // live slots at each cut (seg_count + 1)
  std::vector<std::unique_ptr<Tape>> seg;         // segment tapes, in tape order

  ~Tape() {
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != device) cudaSetDevice(device);
    tan_plans.clear();
    win_plans.clear();
    adj_plans.clear();
    seg.clear();
    cudaFree(d_code);
    cudaFree(d_pofs);
    cudaFree(d_consts);
    cudaFree(d_absent);
    cudaFree(d_err);
    cudaFree(d_lcode);
    cudaFree(d_lbegin);
    cudaFree(d_lpidx);
    cudaFree(d_rcode);
    cudaFree(d_rbegin);
    cudaFree(d_rpidx);
    if (gw_event) cudaEventSynchronize(gw_event);
    cudaFree(d_gw);
    if (gw_event) cudaEventDestroy(gw_event);
    if (cur != device) cudaSetDevice(cur);
  }

  TapeView view() const {
    TapeView v;
    v.code = d_code;
    v.pofs = d_pofs;
    v.consts = d_consts;
    v.absent_in = d_absent;
    v.n_chunks = n_chunks;
    v.n_absent_in = static_cast<int>(absent_in.size());
    v.sz_w = sz_w;
    v.n_partials = n_partials;
    v.err = d_err;
    v.lcode = d_lcode;
    v.lbegin = d_lbegin;
    v.lpidx = d_lpidx;
    v.n_levels = n_levels;
    v.lv_sz_w = lv_sz_w;
    v.rcode = d_rcode;
    v.rbegin = d_rbegin;
    v.rpidx = d_rpidx;
    v.n_rlevels = n_rlevels;
    v.rlv_sz_w = rlv_sz_w;
    return v;
  }
};

constexpr int kMaxChunks = 4;  // host-buffer calls: instance chunks pipelined over copy engines

struct Mem {
  cudaStream_t stream = nullptr;
  // copy streams and events of the pipelined host-buffer calls (created on first use)
  cudaStream_t s_in = nullptr, s_out = nullptr;
  cudaEvent_t ev_in[kMaxChunks] = {}, ev_done[kMaxChunks] = {}, ev_out = nullptr;
  // per chunk: the outputs a call finishes before its last sweep (the Jacobian of a Jacobian +
  // adjoint call) can be downloaded from here on
  cudaEvent_t ev_early[kMaxChunks] = {};
  std::vector<void*> bufs;   // device staging buffers, grown on demand
  std::vector<size_t> caps;
  ~Mem() {
    for (void* p : bufs) cudaFree(p);
    for (int k = 0; k < kMaxChunks; ++k) {
      if (ev_in[k]) cudaEventDestroy(ev_in[k]);
      if (ev_done[k]) cudaEventDestroy(ev_done[k]);
      if (ev_early[k]) cudaEventDestroy(ev_early[k]);
    }
    if (ev_out) cudaEventDestroy(ev_out);
    if (s_in) cudaStreamDestroy(s_in);
    if (s_out) cudaStreamDestroy(s_out);
    if (stream) cudaStreamDestroy(stream);
  }
  cudaError_t pipe() {
    if (s_in) return cudaSuccess;
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&s_in, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&s_out, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming)) != cudaSuccess)
      return e;
    for (int k = 0; k < kMaxChunks; ++k)
      if ((e = cudaEventCreateWithFlags(&ev_in[k], cudaEventDisableTiming)) != cudaSuccess ||
          (e = cudaEventCreateWithFlags(&ev_done[k], cudaEventDisableTiming)) != cudaSuccess ||
          (e = cudaEventCreateWithFlags(&ev_early[k], cudaEventDisableTiming)) != cudaSuccess)
        return e;
    return cudaSuccess;
  }
  // device buffer k of at least `bytes`
  void* buf(size_t k, size_t bytes, cudaError_t* e) {
    if (bufs.size() <= k) {
      bufs.resize(k + 1, nullptr);
      caps.resize(k + 1, 0);
    }
    if (caps[k] < bytes) {
      cudaFree(bufs[k]);
      bufs[k] = nullptr;
      caps[k] = 0;
      *e = cudaMalloc(&bufs[k], bytes);
      if (*e != cudaSuccess) return nullptr;
      caps[k] = bytes;
    }
    return bufs[k];
  }
};

std::mutex g_mtx;
std::vector<std::unique_ptr<Tape>> g_tapes;
std::vector<std::unique_ptr<Mem>> g_mems;

// ---- optional per-launch timing (CUDA events on the launch stream) -------------------------
enum Family { F_EVAL = 0, F_RECORD, F_TANGENT, F_ADJOINT, F_SP_FORWARD, F_SP_REVERSE, F_BATCH,
              F_ACTIVITY, F_COUNT };
struct ProfEntry {
  int family;
  cudaEvent_t start, stop;
};
bool g_prof = false;
std::vector<ProfEntry> g_prof_live;
std::vector<cudaEvent_t> g_prof_pool;
std::mutex g_prof_mtx;

cudaEvent_t prof_event() {
  if (!g_prof_pool.empty()) {
    cudaEvent_t e = g_prof_pool.back();
    g_prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Launch `fn` (returning cudaError_t) on stream s, bracketed by events when profiling is on.
template <class Fn>
cudaError_t timed(int family, cudaStream_t s, Fn&& fn) {
  if (!g_prof) return fn();
  std::lock_guard<std::mutex> lk(g_prof_mtx);
  ProfEntry p{family, prof_event(), prof_event()};
  cudaEventRecord(p.start, s);
  cudaError_t e = fn();
  cudaEventRecord(p.stop, s);
  g_prof_live.push_back(p);
  return e;
}

Tape* get_tape(int id) {
  std::lock_guard<std::mutex> lk(g_mtx);
  if (id < 0 || id >= static_cast<int>(g_tapes.size()) || !g_tapes[id]) return nullptr;
  return g_tapes[id].get();
}

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
    n = 1;
  return n;
}

// Pick the CTA shapes that keep the most threads resident given the shared-memory footprint.
void choose_shapes(Tape& t) {
  const int max_smem = max_smem_optin();
  const int sms = sm_count();
  int best_threads = -1;
  for (int bs : {256, 128, 64, 32}) {
    const size_t sm = smem_primal(t.sz_w, bs);
    if (sm > static_cast<size_t>(max_smem)) continue;
    const int occ = occupancy_primal(bs, sm);
    if (occ * bs > best_threads) {
      best_threads = occ * bs;
      t.primal_block = bs;
      t.primal_grid_cap = occ * sms;
    }
  }
}

// Shape of a derivative-sweep launch: DW warps (one direction each) per CTA on one 32-instance
// tile, `ch` instructions per staged chunk. Prefers the configuration with the most resident
// warps per SM (enough to keep every sub-partition's FP64 unit busy), then the fewest idle
// direction slots, then the longest chunk.
struct DirShape {
  int dw = 1, ch = 16, blocks_per_sm = 1;
};

// Autotuning of the derivative sweeps: the first large enough call of each kind on a tape
// runs every variant once on its first wave (same arithmetic, same results), times them with
// CUDA events and keeps the fastest for the tape. It synchronizes the stream once; it is
// skipped while the stream is being captured into a graph, and can be switched off.
bool g_autotune = true;


bool fits_smem(int sz_w) {
  return smem_primal(sz_w, 32) <= static_cast<size_t>(max_smem_optin());
}

// Work-vector residence: global memory when asked for or when shared memory cannot hold it.
bool primal_global(const Tape& t) {
  return t.residence == 1 || !fits_smem(t.sz_w);
}
bool dir_global(const Tape& t) {
  return t.residence == 1 || smem_lean(t.sz_w, 1, 0) > static_cast<size_t>(max_smem_optin());
}

constexpr size_t kGwMaxBytes = 4ull << 30;  // global work vectors of one launch

bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cs);
  return cs != cudaStreamCaptureStatusNone;
}

// Points a.wglob at a per-CTA block of per_cta bytes for *grid CTAs (grid capped to the
// byte budget), growing the tape's buffer if needed; orders the launch after the buffer's
// last use on another stream.
int gw_prepare(Tape& t, SweepArgs& a, int* grid, size_t per_cta, cudaStream_t s) {
  const long long max_grid = std::max<long long>(1, static_cast<long long>(kGwMaxBytes / per_cta));
  *grid = static_cast<int>(std::min<long long>(*grid, max_grid));
  const size_t need = per_cta * static_cast<size_t>(*grid);
  std::lock_guard<std::mutex> lk(t.gw_mtx);
  cudaError_t e;
  if (!t.gw_event && (e = cudaEventCreateWithFlags(&t.gw_event, cudaEventDisableTiming)) != cudaSuccess)
    return cuda_fail(e, "work-vector event");
  if (t.gw_cap < need) {
    if (capturing(s))
      return fail(CASADI_GB300_ERR_ARG,
                  "global work vector must grow (%zu bytes): call once before graph capture", need);
    if (t.gw_recorded && (e = cudaEventSynchronize(t.gw_event)) != cudaSuccess)
      return cuda_fail(e, "work-vector wait");
    cudaFree(t.d_gw);
    t.d_gw = nullptr;
    t.gw_cap = 0;
    if ((e = cudaMalloc(&t.d_gw, need)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(work vectors)");
    t.gw_cap = need;
  } else if (t.gw_recorded && !capturing(s)) {
    if ((e = cudaStreamWaitEvent(s, t.gw_event, 0)) != cudaSuccess)
      return cuda_fail(e, "work-vector ordering");
  }
  a.wglob = t.d_gw;
  a.wglob_stride = static_cast<long long>(per_cta);
  return 0;
}

int gw_done(Tape& t, cudaStream_t s) {
  if (capturing(s)) return 0;
  std::lock_guard<std::mutex> lk(t.gw_mtx);
  cudaError_t e = cudaEventRecord(t.gw_event, s);
  if (e != cudaSuccess) return cuda_fail(e, "work-vector event record");
  t.gw_recorded = true;
  return 0;
}

int check_device(const Tape& t) {
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (cur != t.device)
    return fail(CASADI_GB300_ERR_ARG, "tape lives on device %d, current device is %d", t.device,
                cur);
  return 0;
}

void fill_io(IoDesc* dst, int count, void* const* ptrs, const std::vector<int>& nnz,
             long long ld, bool dir_major) {
  for (int j = 0; j < count; ++j) {
    dst[j].ptr = ptrs ? ptrs[j] : nullptr;
    dst[j].nz_stride = ld;
    dst[j].inst_stride = 1;
    dst[j].dir_stride = dir_major ? static_cast<long long>(nnz[j]) * ld : 0;
  }
}

SweepArgs base_args(const Tape& t, long long n, long long i_begin) {
  SweepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.t = t.view();
  a.n = n;
  a.i_begin = i_begin;
  a.n_in = t.n_in;
  a.n_out = t.n_out;
  return a;
}

int grid_for(long long tiles, int cap) {
  long long g = std::min<long long>(tiles, cap);
  return static_cast<int>(std::max<long long>(g, 1));
}

// Room the reported scratch sizes leave past the partials for the tangent sweep's work
// counter.
constexpr size_t kQueueSlack = 256;

// Instances per AD wave that fit in `bytes` of scratch (multiple of 32).
long long wave_capacity(const Tape& t, long long n, size_t bytes) {
  if (t.n_partials == 0) return n;
  long long per = 8ll * t.n_partials;
  long long w = static_cast<long long>(bytes / per);
  w = (w / 32) * 32;
  return std::min<long long>(w, ((n + 31) / 32) * 32);
}

template <class T>
cudaError_t upload(T** dst, const std::vector<T>& v) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(dst), std::max<size_t>(1, v.size()) * sizeof(T));
  if (e != cudaSuccess) return e;
  if (v.empty()) return cudaSuccess;
  return cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

unsigned lean_kind(unsigned op) {
  switch (op) {
    case D_ADD: return LK_ADD;
    case D_SUB: return LK_SUB;
    case D_NEG: return LK_NEG;
    case D_TWICE: return LK_TWICE;
    case D_ASSIGN: return LK_ASSIGN;
    case D_IF_ELSE_ZERO: return LK_IFZ;
    case D_INPUT: return LK_INPUT;
    case D_OUTPUT: return LK_OUTPUT;
    case D_CONST: return LK_CONST;
    case D_NOP: return LK_NOP;
    default: return LK_GEN;
  }
}

// Entry of the windowed tangent sweep (k_tangent_win) for instruction word w (flags: 1/2
// operand b/c carries a derivative); slot fields become byte offsets into the warp's work
// vector w[slot][lane] (slot * 256).
uint4 dir_entry(u64 w, unsigned flags, int pk) {
  const unsigned op = dec_op(w), A = dec_a(w), B = dec_b(w), C = dec_c(w);
  uint4 e;
  if (op == D_INPUT) {
    e = make_uint4(A * 256u, B, C, 0);
  } else if (op == D_OUTPUT) {
    e = make_uint4(A, B * 256u, C, 0);
  } else {
    e = make_uint4(A * 256u, B * 256u, C * 256u, 0);
  }
  e.w = (flags & 31u) | (lean_kind(op) << 5) | (dec_pmask(w) << 9) |
        (static_cast<unsigned>(pk) << 11);
  return e;
}

// Operand forwarding in the windowed sweep's entries: an operand that is the value the
// previous value-writing entry just computed is marked (bit 31 of its slot offset) and the
// sweep takes it from a register instead of reading it back from shared memory.
constexpr unsigned kFwdBit = 1u << 31;
void forward_operands(std::vector<uint4>& ents) {
  bool have = false;
  unsigned last = 0;  // slot byte offset the previous value-writing entry wrote
  for (uint4& e : ents) {
    const unsigned kind = (e.w >> 5) & 15u, f = e.w & 3u;
    if (kind == LK_OUTPUT) {
      if (have && (f & 1u) && e.y == last) e.y |= kFwdBit;
      continue;
    }
    if (kind == LK_INPUT) {
      if (f & 1u) {
        have = true;
        last = e.x;
      }
      continue;
    }
    if (kind == LK_NOP || kind == LK_CONST || !f) continue;
    if (have && (f & 1u) && e.y == last) e.y |= kFwdBit;
    if (have && (f & 2u) && e.z == last) e.z |= kFwdBit;
    have = true;
    last = e.x;
  }
}

// One entry of a keyed stream before layout (see the keyed streams in sweeps.cuh).
struct KEnt {
  unsigned x = 0, y = 0, z = 0;
  unsigned key = 0;    // TK_* or AK_*
  unsigned pinfo = 0;  // what the walk loads for this entry: kPiP, kPiQ, kPiQNext, index << 3
};

// The partial loads of an entry: P (its d0) and/or Q (its d1) of an instruction with
// recorded-partial mask pm whose first recorded partial is pk.
unsigned pinfo_of(bool lp, bool lq, unsigned pm, int pk) {
  if (!lp && !lq) return 0;
  return (lp ? kPiP : 0u) | (lq ? kPiQ : 0u) | ((pm & 1u) ? kPiQNext : 0u) |
         (static_cast<unsigned>(pk) << (kPiIndexShift - kPiShift));
}

// Lays out one keyed stream for group size gsz at the end of `all`: a header group, the body
// padded to an even number of groups, one trailing group; entry p carries the partial loads of
// entry p + gsz. Returns (first entry, body entries).
int2 lay_out(std::vector<uint4>& all, const std::vector<KEnt>& ents, int gsz) {
  const long long n = static_cast<long long>(ents.size());
  long long ngr = (n + gsz - 1) / gsz;
  if (ngr & 1) ++ngr;
  const long long body = ngr * gsz;
  const int first = static_cast<int>(all.size());
  for (long long p = -gsz; p < body + gsz; ++p) {
    uint4 u = make_uint4(0, 0, 0, 0);
    if (p >= 0 && p < n) u = make_uint4(ents[p].x, ents[p].y, ents[p].z, ents[p].key);
    const long long q = p + gsz;
    if (q >= 0 && q < n) u.w |= ents[q].pinfo << kPiShift;
    all.push_back(u);
  }
  return make_int2(first, static_cast<int>(body));
}

constexpr int kGroupSizeOf[kNumGroupSizes] = {1, 2, 4, 8};

// Tangent entry before keying: fields as the walks read them, the instruction's kind, flags
// (1/2: operand b/c carries a derivative; inputs/outputs: 1 active), recorded-partial mask and
// first partial.
struct TanRaw {
  unsigned x = 0, y = 0, z = 0;
  unsigned op = 0, kind = 0, f = 0, pm = 0;
  int pk = 0;
  bool mixed = false;
};

TanRaw tan_raw(u64 w, unsigned flags, int pk) {
  const unsigned op = dec_op(w), A = dec_a(w), B = dec_b(w), C = dec_c(w);
  TanRaw e;
  if (op == D_INPUT) {
    e.x = A * 256u, e.y = B, e.z = C;
  } else if (op == D_OUTPUT) {
    e.x = A, e.y = B * 256u, e.z = C;
  } else {
    e.x = A * 256u, e.y = B * 256u, e.z = C * 256u;
  }
  e.op = op;
  e.kind = lean_kind(op);
  e.f = flags & 3u;
  e.pm = dec_pmask(w);
  e.pk = pk;
  return e;
}

// Tangent form of an arithmetic entry (-1: none). GEN ops whose d0 is a constant 1 and not
// recorded (FMOD, REMAINDER, PRINTME, LIFT) take the unit forms: 1*a + q*b and 1*a are a + q*b
// and a, bit for bit.
int tan_form(const TanRaw& e) {
  const unsigned f = e.f;
  switch (e.kind) {
    case LK_GEN: {
      const bool p = e.pm & 1u, q = e.pm & 2u, unit = !p && const_d0(e.op) == 1.0;
      if (f == 1u) return p ? TF_PY : unit ? TF_Y : -1;
      if (f == 2u) return q ? TF_QZ : -1;
      if (f == 3u) return !q ? -1 : p ? TF_PYQZ : unit ? TF_YQZ : -1;
      return -1;
    }
    case LK_ADD: return f == 1u ? TF_Y : f == 2u ? TF_Z : f == 3u ? TF_YZ : -1;
    case LK_SUB: return f == 1u ? TF_Y : f == 2u ? TF_NZ : f == 3u ? TF_YMZ : -1;
    case LK_NEG: return f == 1u ? TF_NY : -1;
    case LK_TWICE: return f == 1u ? TF_2Y : -1;
    case LK_ASSIGN: return f == 1u ? TF_Y : -1;
    case LK_IFZ: return f == 2u ? TF_IFZ : -1;
    default: return -1;
  }
}

unsigned tan_key_of(int form) {
#define CGB_FIND(KEY, F) \
  if (form == (F)) return KEY;
  CGB_TK_ARITH(CGB_FIND)
#undef CGB_FIND
  return ~0u;
}

// Keyed tangent entry; false when the instruction has no tangent form (not expected).
bool tan_keyed(const TanRaw& e, KEnt* k) {
  k->x = e.x, k->y = e.y, k->z = e.z;
  k->pinfo = 0;
  if (e.mixed) {
    k->key = TK_MIXED + e.pm;
    k->pinfo = pinfo_of(e.pm & 1u, e.pm & 2u, e.pm, e.pk);
    return true;
  }
  if (e.kind == LK_OUTPUT) {
    k->key = (e.f & 1u) ? TK_OUT : TK_OUT0;
    return true;
  }
  if (e.kind == LK_INPUT) {
    k->key = TK_IN;
    return true;
  }
  const int form = tan_form(e);
  if (form < 0) return false;
  k->key = tan_key_of(form);
  k->pinfo = pinfo_of(tf_uses_p(form), tf_uses_q(form), e.pm, e.pk);
  return k->key != ~0u;
}

// Adjoint contribution forms of an arithmetic instruction (op, kind, recorded-partial mask pm)
// with adjoint-plan flags f (2/4: operand b/c receives, 8/16: its first contribution); -1:
// none. GEN ops with an unrecorded unit d0 take the unit forms (1*s and fma(1, s, w) are s
// and w + s, bit for bit).
int adj_bform(unsigned op, unsigned kind, unsigned pm, unsigned f) {
  if (!(f & 2u)) return CF_N;
  const bool first = f & 8u;
  switch (kind) {
    case LK_GEN:
      if (pm & 1u) return first ? CF_RF : CF_RA;
      return const_d0(op) == 1.0 ? (first ? CF_UF : CF_UA) : -1;
    case LK_ADD: case LK_SUB: case LK_ASSIGN: return first ? CF_UF : CF_UA;
    case LK_NEG: return first ? CF_MF : CF_MA;
    case LK_TWICE: return first ? CF_TF : CF_TA;
    default: return -1;
  }
}
int adj_cform(unsigned kind, unsigned pm, unsigned f) {
  if (!(f & 4u)) return CF_N;
  const bool first = f & 16u;
  switch (kind) {
    case LK_GEN: return (pm & 2u) ? (first ? CF_RF : CF_RA) : -1;
    case LK_ADD: return first ? CF_UF : CF_UA;
    case LK_SUB: return first ? CF_MF : CF_MA;
    case LK_IFZ: return first ? CF_IF : CF_IA;
    default: return -1;
  }
}
unsigned adj_key_of(int bf, int cf) {
#define CGB_FIND(KEY, BF, CF) \
  if (bf == (BF) && cf == (CF)) return KEY;
  CGB_AK_ARITH(CGB_FIND)
#undef CGB_FIND
  return ~0u;
}

std::vector<int> partial_starts(const Tape& t) {
  std::vector<int> pk(t.h_code.size());
  int acc = 0;
  for (size_t k = 0; k < t.h_code.size(); ++k) {
    pk[k] = acc;
    const unsigned op = dec_op(t.h_code[k]);
    if (op != D_CONST && op != D_INPUT && op != D_OUTPUT && op != D_NOP)
      acc += __builtin_popcount(partial_mask(op));
  }
  return pk;
}

// Structural activity of the tangent sweep, per direction: an input slot is active when it is
// seeded (unit seeds: when it is the direction's own input nonzero), an arithmetic result
// when an operand that carries a derivative is active (the reference's 0*x -> 0, x+0 -> x).
// Returns, per group of dw directions and instruction, 2 bits per direction (operand b / c
// carries a derivative; an input or output: bit 0 when active). Instructions whose result
// reaches no output in `wanted` (outputs whose sensitivities were requested; empty: all) get
// no bits: their tangents would feed nothing that is written. Activity itself is propagated
// over every instruction, so the entries kept are the same as without pruning.
std::vector<unsigned short> tan_activity(const Tape& t, int ndir, int dw, bool identity,
                                         const std::vector<char>& seeded,
                                         const std::vector<int>& dirmap,
                                         const std::vector<char>& wanted) {
  const int groups = (ndir + dw - 1) / dw;
  const size_t nc = t.h_code.size();
  // instructions a wanted output depends on: a backward pass over the slots read later
  std::vector<char> need(nc, 1);
  bool all = true;
  for (char c : wanted) all = all && c;
  if (!all) {
    std::vector<char> live(std::max(1, t.sz_w), 0);
    for (size_t kk = nc; kk-- > 0;) {
      const u64 w = t.h_code[kk];
      const unsigned op = dec_op(w), A = dec_a(w), B = dec_b(w), C = dec_c(w);
      need[kk] = 0;
      if (op == D_NOP) continue;
      if (op == D_OUTPUT) {
        need[kk] = wanted[A];
        if (wanted[A]) live[B] = 1;
        continue;
      }
      if (!live[A]) continue;
      need[kk] = 1;
      live[A] = 0;
      if (op == D_CONST || op == D_INPUT) continue;
      live[B] = 1;
      if (is_binary(op)) live[C] = 1;
    }
  }
  std::vector<int> off(t.n_in + 1, 0);
  for (int j = 0; j < t.n_in; ++j) off[j + 1] = off[j] + t.nnz_in[j];
  std::vector<unsigned short> bits(static_cast<size_t>(groups) * nc, 0);
  std::vector<char> act(std::max(1, t.sz_w));
  const int ncomp = identity ? ndir : 1;  // general seeds: every direction has the same pattern
  for (int d = 0; d < ncomp; ++d) {
    std::fill(act.begin(), act.end(), 0);
    for (size_t k = 0; k < nc; ++k) {
      const u64 w = t.h_code[k];
      const unsigned op = dec_op(w), A = dec_a(w), B = dec_b(w), C = dec_c(w);
      unsigned b = 0;
      if (op == D_NOP) continue;
      if (op == D_CONST) {
        act[A] = 0;
        continue;
      }
      if (op == D_INPUT) {
        const int flat = off[B] + static_cast<int>(C);
        const bool on = identity ? ((dirmap.empty() ? flat : dirmap[flat]) == d)
                                 : seeded[B] != 0;
        act[A] = on;
        b = on ? 1u : 0u;
      } else if (op == D_OUTPUT) {
        b = act[B] ? 1u : 0u;
      } else {
        const bool cb = act[B] && carries_d0(op);
        const bool cc = act[C] && carries_d1(op);
        act[A] = cb || cc;
        b = (cb ? 1u : 0u) | (cc ? 2u : 0u);
      }
      if (!b || !need[k]) continue;
      for (int dd = identity ? d : 0; dd < (identity ? d + 1 : ndir); ++dd)
        bits[static_cast<size_t>(dd / dw) * nc + k] |=
            static_cast<unsigned short>(b << (2 * (dd % dw)));
    }
  }
  return bits;
}

// Each direction group gets a compacted entry stream of the instructions with work for it.
const TanPlan* tan_plan(Tape& t, int ndir, int dw, int ch, bool identity,
                        const std::vector<char>& seeded, const std::vector<int>& dirmap,
                        const std::vector<char>& wanted, int* err) {
  std::lock_guard<std::mutex> lk(t.shape_mtx);
  for (auto& p : t.tan_plans)
    if (p->ndir == ndir && p->dw == dw && p->ch == ch && p->identity == identity &&
        (identity ? p->dirmap == dirmap : p->seeded == seeded) && p->wanted == wanted)
      return p.get();
  auto p = std::make_unique<TanPlan>();
  p->ndir = ndir;
  p->dw = dw;
  p->ch = ch;
  p->identity = identity;
  p->dirmap = dirmap;
  p->seeded = seeded;
  p->wanted = wanted;
  p->groups = (ndir + dw - 1) / dw;
  const size_t nc = t.h_code.size();
  const std::vector<unsigned short> bits =
      tan_activity(t, ndir, dw, identity, seeded, dirmap, wanted);
  // one stream per group of dw directions (the union of their work); an entry whose flags
  // differ between the group's directions is mixed: the real kind in x bits 19-22 and the
  // flags of direction k in bits 24+2k (see the tangent kernel)
  const std::vector<int> pk = partial_starts(t);
  std::vector<uint4> all[kNumGroupSizes];
  for (int gs = 0; gs < kNumGroupSizes; ++gs) p->h_chunks[gs].resize(p->groups);
  std::vector<size_t> len(p->groups, 0);
  for (int g = 0; g < p->groups; ++g) {
    if (!identity && g > 0) {
      // general seeds: one stream serves every group
      for (int gs = 0; gs < kNumGroupSizes; ++gs) p->h_chunks[gs][g] = p->h_chunks[gs][0];
      len[g] = len[0];
      continue;
    }
    const int kv = std::min(dw, ndir - g * dw);  // directions in this group
    std::vector<TanRaw> raw;
    for (size_t k = 0; k < nc; ++k) {
      const u64 w = t.h_code[k];
      const unsigned op = dec_op(w);
      const unsigned gb = bits[static_cast<size_t>(g) * nc + k];
      if (!gb && op != D_OUTPUT) continue;
      const unsigned f0 = gb & 3u;
      bool uniform = true;
      for (int d = 1; d < kv; ++d) uniform = uniform && ((gb >> (2 * d)) & 3u) == f0;
      if (uniform) {
        raw.push_back(tan_raw(w, f0, pk[k]));
      } else {
        TanRaw e = tan_raw(w, 0, pk[k]);
        e.x |= (lean_kind(op) << 19) | ((gb & 0xffu) << 24);
        e.mixed = true;
        raw.push_back(e);
      }
    }
    std::vector<KEnt> ents(raw.size());
    for (size_t q = 0; q < raw.size(); ++q)
      if (!tan_keyed(raw[q], &ents[q])) {
        *err = fail(CASADI_GB300_ERR_UNSUPPORTED, "tangent entry of op %u has no form",
                    raw[q].op);
        return nullptr;
      }
    for (int gs = 0; gs < kNumGroupSizes; ++gs)
      p->h_chunks[gs][g] = lay_out(all[gs], ents, kGroupSizeOf[gs]);
    len[g] = ents.size();
  }
  // the groups of one tile are claimed longest first, so the last items of a sweep are the
  // short ones
  std::vector<int> order(p->groups);
  for (int g = 0; g < p->groups; ++g) order[g] = g;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return len[x] > len[y]; });
  bool natural = true;
  for (int g = 0; g < p->groups; ++g) natural = natural && order[g] == g;
  cudaError_t e = cudaSuccess;
  for (int gs = 0; gs < kNumGroupSizes && e == cudaSuccess; ++gs)
    if ((e = upload(&p->d_stream[gs], all[gs])) == cudaSuccess)
      e = upload(&p->d_chunks[gs], p->h_chunks[gs]);
  if (e != cudaSuccess ||
      (!natural && (e = upload(&p->d_order, order)) != cudaSuccess) ||
      (identity && !dirmap.empty() && (e = upload(&p->d_dirmap, dirmap)) != cudaSuccess)) {
    *err = cuda_fail(e, "upload tangent plan");
    return nullptr;
  }
  t.tan_plans.push_back(std::move(p));
  return t.tan_plans.back().get();
}

// The windowed tangent sweep's plan. Directions per CTA and ring stages come from the
// shared-memory budget (each direction's work vector, sz_w x 256 bytes, plus the stages);
// the stage bytes are split between partial rows and entry-block room in the proportion the
// tape needs them; windows are cut greedily, instruction by instruction, so that a window's
// partial rows and its largest group's entry block (header included) fit one stage. Fewer
// than 4 directions, or a work vector too long for 4 of them, give an unusable plan.
constexpr int kWinMinDirs = 4;
const WinPlan* win_plan(Tape& t, int ndir, bool identity, const std::vector<char>& seeded,
                        const std::vector<int>& dirmap, const std::vector<char>& wanted,
                        int* err) {
  std::lock_guard<std::mutex> lk(t.shape_mtx);
  for (auto& p : t.win_plans)
    if (p->ndir == ndir && p->identity == identity &&
        (identity ? p->dirmap == dirmap : p->seeded == seeded) && p->wanted == wanted)
      return p.get();
  auto p = std::make_unique<WinPlan>();
  p->ndir = ndir;
  p->identity = identity;
  p->dirmap = dirmap;
  p->seeded = seeded;
  p->wanted = wanted;
  const long long wv = static_cast<long long>(std::max(1, t.sz_w)) * 256;
  const long long budget = static_cast<long long>(max_smem_optin()) - 1024 - kWinBarBytes;
  constexpr long long kMinStage = 16 * 256 + 256 * 16;
  int dirs = std::min(ndir, kWinMaxDirs);
  while (dirs >= kWinMinDirs && budget - dirs * wv < 2 * kMinStage) --dirs;
  if (ndir < kWinMinDirs || dirs < kWinMinDirs) {
    t.win_plans.push_back(std::move(p));
    return t.win_plans.back().get();
  }
  p->groups = (ndir + dirs - 1) / dirs;
  p->dirs = dirs = (ndir + p->groups - 1) / p->groups;  // balanced groups
  const long long left = budget - dirs * wv;
  p->stages = left >= 3 * kMinStage ? 3 : 2;
  const long long per_stage = left / p->stages / 16 * 16;

  const size_t nc = t.h_code.size();
  const std::vector<int> pk = partial_starts(t);
  const std::vector<unsigned short> bits =
      tan_activity(t, ndir, 1, identity, seeded, dirmap, wanted);
  // entries of every stream (identity: one per direction; general seeds: one for all), with
  // the instruction each belongs to, operand forwarding marked over the whole stream
  const int nstreams = identity ? ndir : 1;
  std::vector<std::vector<uint4>> ents(nstreams);
  std::vector<std::vector<int>> at(nstreams);
  for (int d = 0; d < nstreams; ++d) {
    for (size_t k = 0; k < nc; ++k) {
      const u64 w = t.h_code[k];
      const unsigned op = dec_op(w);
      const unsigned b = bits[static_cast<size_t>(d) * nc + k] & 3u;
      if (!b && op != D_OUTPUT) continue;
      ents[d].push_back(dir_entry(w, b, pk[k]));
      at[d].push_back(static_cast<int>(k));
    }
    forward_operands(ents[d]);
  }
  // per instruction: partial rows, and the largest group's entry count
  std::vector<int> rows_k(nc), ents_k(nc, 0);
  long long rows_total = 0, ents_total = 0;
  for (size_t k = 0; k < nc; ++k) {
    rows_k[k] = (k + 1 < nc ? pk[k + 1] : t.n_partials) - pk[k];
    rows_total += rows_k[k];
  }
  {
    std::vector<int> cnt(static_cast<size_t>(p->groups) * nc, 0);
    for (int d = 0; d < nstreams; ++d)
      for (int k : at[d]) ++cnt[static_cast<size_t>(d / dirs) * nc + k];
    for (int g = 0; g < (identity ? p->groups : 1); ++g)
      for (size_t k = 0; k < nc; ++k)
        ents_k[k] = std::max(ents_k[k], cnt[static_cast<size_t>(g) * nc + k]);
    for (size_t k = 0; k < nc; ++k) ents_total += ents_k[k];
  }
  const int hdr_u4 = win_header_words(dirs) / 4;
  // split a stage between partial rows and entry room as the tape needs them
  const double share = static_cast<double>(rows_total * 256) /
                       std::max<double>(1.0, rows_total * 256.0 + ents_total * 16.0);
  p->rows = std::max(4, static_cast<int>(per_stage * share / 256));
  p->ents = static_cast<int>((per_stage - static_cast<long long>(p->rows) * 256) / 16);
  if (p->ents < hdr_u4 + dirs + 1) {
    p->ents = hdr_u4 + dirs + 1;
    p->rows = static_cast<int>((per_stage - p->ents * 16ll) / 256);
  }
  // windows: [win_k[w], win_k[w+1])
  std::vector<int> win_k{0};
  {
    int r = 0, e = 0;
    for (size_t k = 0; k < nc; ++k) {
      if (r + rows_k[k] > p->rows || hdr_u4 + e + ents_k[k] > p->ents) {
        win_k.push_back(static_cast<int>(k));
        r = e = 0;
      }
      r += rows_k[k];
      e += ents_k[k];
    }
    win_k.push_back(static_cast<int>(nc));
    if (win_k.size() >= 2 && win_k[win_k.size() - 2] == static_cast<int>(nc)) win_k.pop_back();
  }
  p->nwin = static_cast<int>(win_k.size()) - 1;
  // blocks: header words [p0, rows, off_0 .. off_dirs] padded to 16 bytes, then the entries of
  // the group's directions in order
  std::vector<unsigned> words;
  std::vector<int4> meta(static_cast<size_t>(p->groups) * p->nwin);
  std::vector<size_t> pos(nstreams, 0);  // next entry of each stream
  for (int g = 0; g < (identity ? p->groups : 1); ++g) {
    for (int w = 0; w < p->nwin; ++w) {
      const int k0 = win_k[w], k1 = win_k[w + 1];
      const int p0 = k0 < static_cast<int>(nc) ? pk[k0] : t.n_partials;
      const int p1 = k1 < static_cast<int>(nc) ? pk[k1] : t.n_partials;
      const size_t start = words.size();
      words.resize(start + win_header_words(dirs), 0u);
      words[start] = static_cast<unsigned>(p0);
      words[start + 1] = static_cast<unsigned>(p1 - p0);
      unsigned off = 0;
      for (int j = 0; j < dirs; ++j) {
        words[start + 2 + j] = off;
        const int d = identity ? g * dirs + j : 0;
        if ((identity || j == 0) && d < nstreams) {
          size_t& q = pos[d];
          while (q < at[d].size() && at[d][q] < k1) {
            const uint4 e = ents[d][q++];
            words.insert(words.end(), {e.x, e.y, e.z, e.w});
            ++off;
          }
        }
      }
      words[start + 2 + dirs] = off;
      meta[static_cast<size_t>(g) * p->nwin + w] =
          make_int4(p0, p1 - p0, static_cast<int>(start / 4),
                    static_cast<int>((words.size() - start) / 4));
    }
  }
  if (!identity)  // general seeds: every group walks the same blocks
    for (int g = 1; g < p->groups; ++g)
      for (int w = 0; w < p->nwin; ++w)
        meta[static_cast<size_t>(g) * p->nwin + w] = meta[w];
  std::vector<uint4> blocks(words.size() / 4);
  std::memcpy(blocks.data(), words.data(), blocks.size() * sizeof(uint4));
  cudaError_t e;
  if ((e = upload(&p->d_blocks, blocks)) != cudaSuccess ||
      (e = upload(&p->d_meta, meta)) != cudaSuccess) {
    *err = cuda_fail(e, "upload window plan");
    return nullptr;
  }
  p->usable = true;
  t.win_plans.push_back(std::move(p));
  return t.win_plans.back().get();
}

// Structural activity of the adjoint sweep (direction-independent), last instruction first.
// Flags: 1 adjoint of the result is nonzero, 2/4 operand b/c receives a contribution,
// 8/16 that contribution is the first to b/c, 32 a seeded output. Entries without work are
// left out of the stream; inputs whose adjoint is structurally zero go to the zero list.
const AdjPlan* adj_plan(Tape& t, int dw, int ch, const std::vector<char>& seeded, int* err) {
  std::lock_guard<std::mutex> lk(t.shape_mtx);
  for (auto& p : t.adj_plans)
    if (p->ch == ch && p->dw == dw && p->seeded == seeded) return p.get();
  auto p = std::make_unique<AdjPlan>();
  p->ch = ch;
  p->dw = dw;
  p->seeded = seeded;
  const size_t nc = t.h_code.size();
  std::vector<unsigned char> bits(nc, 0);
  std::vector<char> act(std::max(1, t.sz_w), 0);
  std::vector<int2> zero(t.absent_in);
  for (size_t kk = nc; kk-- > 0;) {
    const u64 w = t.h_code[kk];
    const unsigned op = dec_op(w), A = dec_a(w), B = dec_b(w), C = dec_c(w);
    unsigned f = 0;
    if (op == D_NOP) continue;
    if (op == D_OUTPUT) {
      if (seeded[A]) {
        f = 32u | (act[B] ? 0u : 8u);
        act[B] = 1;
      }
    } else if (op == D_INPUT) {
      if (act[A]) {
        f = 1;
        act[A] = 0;
      } else {
        zero.push_back(make_int2(static_cast<int>(B), static_cast<int>(C)));
      }
    } else if (op == D_CONST) {
      if (act[A]) {
        f = 1;
        act[A] = 0;
      }
    } else if (act[A]) {
      f = 1;
      act[A] = 0;
      if (carries_d0(op)) {
        f |= 2u | (act[B] ? 0u : 8u);
        act[B] = 1;
      }
      if (carries_d1(op)) {
        f |= 4u | (act[C] ? 0u : 16u);
        act[C] = 1;
      }
    }
    bits[kk] = static_cast<unsigned char>(f);
  }
  // keyed entries in sweep order (last instruction first). Constants and arithmetic entries
  // that pass nothing on are left out: every slot's first contribution is assigned, so no
  // adjoint needs resetting after it is read.
  const std::vector<int> pk = partial_starts(t);
  std::vector<KEnt> ents;
  for (size_t kk = nc; kk-- > 0;) {
    const unsigned f = bits[kk];
    if (!f) continue;
    const u64 w = t.h_code[kk];
    const unsigned op = dec_op(w), A = dec_a(w), B = dec_b(w), C = dec_c(w);
    KEnt e;
    if (op == D_OUTPUT) {
      e.x = A, e.y = B * 256u, e.z = C;
      e.key = (f & 8u) ? AK_OUT_SET : AK_OUT_ADD;
    } else if (op == D_INPUT) {
      e.x = A * 256u, e.y = B, e.z = C;
      e.key = AK_IN;
    } else if (op == D_CONST) {
      continue;
    } else {
      const unsigned kind = lean_kind(op), pm = dec_pmask(w);
      const int bf = adj_bform(op, kind, pm, f), cf = adj_cform(kind, pm, f);
      if (bf == CF_N && cf == CF_N) continue;
      e.x = A * 256u, e.y = B * 256u, e.z = C * 256u;
      e.key = (bf < 0 || cf < 0) ? ~0u : adj_key_of(bf, cf);
      if (e.key == ~0u) {
        *err = fail(CASADI_GB300_ERR_UNSUPPORTED, "adjoint entry of op %u has no form", op);
        return nullptr;
      }
      e.pinfo = pinfo_of(bf == CF_RF || bf == CF_RA,
                         cf == CF_RF || cf == CF_RA || cf == CF_IF || cf == CF_IA, pm, pk[kk]);
    }
    ents.push_back(e);
  }
  p->n_zero = static_cast<int>(zero.size());
  cudaError_t e = cudaSuccess;
  for (int gs = 0; gs < kNumGroupSizes && e == cudaSuccess; ++gs) {
    std::vector<uint4> all;
    p->h_chunks[gs] = lay_out(all, ents, kGroupSizeOf[gs]);
    if ((e = upload(&p->d_stream[gs], all)) == cudaSuccess)
      e = upload(&p->d_chunks[gs], std::vector<int2>{p->h_chunks[gs]});
  }
  if (e != cudaSuccess || (e = upload(&p->d_zero, zero)) != cudaSuccess) {
    *err = cuda_fail(e, "upload adjoint plan");
    return nullptr;
  }
  t.adj_plans.push_back(std::move(p));
  return t.adj_plans.back().get();
}

// Runs `fn` (launches on stream s) once between two events and waits for it.
template <class F>
int time_once(cudaStream_t s, F fn, float* ms) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaEventRecord(e0, s);
  if (e == cudaSuccess) e = fn();
  if (e == cudaSuccess) e = cudaEventRecord(e1, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return e == cudaSuccess ? 0 : cuda_fail(e, "autotune timing");
}

// Values + partials (record sweep) followed by the derivative sweep, in waves of as many
// instances as the scratch holds. `in/out/seed/sens` address the whole instance range.
// Value-type sweeps (eval, record, both sparsity sweeps) over one instance range: the shared-
// memory kernels with the tape's block size, or the global-work-vector kernels.
enum PrimalKind { PK_EVAL = 0, PK_RECORD, PK_SP_FORWARD, PK_SP_REVERSE, PK_ACTIVITY };

// Level schedule of the cooperative sweeps (host scheduling + upload, once per tape). Returns
// whether it is available; never called while the stream is being captured.
constexpr int kLevelWidth = 64;      // instructions per level
// CTA size of the cooperative value/record/sparsity sweeps: 256, 512 or 1024 threads (tuned);
// without tuning, enough warps per tile that the tiles of the launch fill the GPU
int coop_threads_for(long long tiles) {
  const long long want = static_cast<long long>(sm_count()) * 32 / std::max(1ll, tiles);
  return want >= 32 ? 1024 : (want >= 16 ? 512 : 256);
}
bool ensure_levels(Tape& t, bool reverse = false) {
  std::lock_guard<std::mutex> lk(t.shape_mtx);
  int& state = reverse ? t.rlv_state : t.lv_state;
  if (state != 0) return state > 0;
  state = -1;
  Levels lv;
  std::string err;
  const int cap = t.sz_w <= 400 ? 400 : t.sz_w + kLevelWidth;
  const int nl = level_schedule(t.h_code, kLevelWidth, cap, lv, err, reverse);
  if (nl <= 0 || lv.code.empty()) return false;
  u64* code = nullptr;
  int *begin = nullptr, *pidx = nullptr;
  bool ok = cudaMalloc(&code, lv.code.size() * sizeof(u64)) == cudaSuccess &&
            cudaMalloc(&begin, lv.begin.size() * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&pidx, lv.pidx.size() * sizeof(int)) == cudaSuccess;
  ok = ok &&
       cudaMemcpy(code, lv.code.data(), lv.code.size() * sizeof(u64), cudaMemcpyHostToDevice) ==
           cudaSuccess &&
       cudaMemcpy(begin, lv.begin.data(), lv.begin.size() * sizeof(int),
                  cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(pidx, lv.pidx.data(), lv.pidx.size() * sizeof(int), cudaMemcpyHostToDevice) ==
           cudaSuccess;
  if (!ok) {
    cudaFree(code);
    cudaFree(begin);
    cudaFree(pidx);
    cudaGetLastError();
    return false;
  }
  if (reverse) {
    t.d_rcode = code;
    t.d_rbegin = begin;
    t.d_rpidx = pidx;
    t.n_rlevels = nl;
    t.rlv_sz_w = lv.sz_w;
  } else {
    t.d_lcode = code;
    t.d_lbegin = begin;
    t.d_lpidx = pidx;
    t.n_levels = nl;
    t.lv_sz_w = lv.sz_w;
  }
  state = 1;
  return true;
}

void reset_primal_tuning(Tape& t) {
  for (auto& k : t.primal_tuned) k[0] = k[1] = -1;
}

int primal_launch(Tape& t, SweepArgs& a, long long m, PrimalKind kind, cudaStream_t s) {
  static const int fam[] = {F_EVAL, F_RECORD, F_SP_FORWARD, F_SP_REVERSE, F_ACTIVITY};
  static const char* what[] = {"eval launch", "record sweep launch", "sp_forward launch",
                               "sp_reverse launch", "activity launch"};
  // modes: shared, global, cooperative with 256, 512 or 1024 threads per CTA
  enum { M_SHARED = 0, M_GLOBAL = 1, M_COOP = 2, M_COOP_LAST = 4 };
  auto coop_threads = [](int mode) { return 256 << (mode - M_COOP); };
  const bool sp_kind = kind == PK_SP_FORWARD || kind == PK_SP_REVERSE;
  auto go = [&](int grid) {
    switch (kind) {
      case PK_EVAL: return launch_eval(a, grid, s);
      case PK_RECORD: return launch_record(a, grid, s);
      case PK_SP_FORWARD: return launch_sp_forward(a, grid, s);
      case PK_ACTIVITY: return launch_activity(a, grid, s);
      default: return launch_sp_reverse(a, grid, s);
    }
  };
  // one launch: work vector in shared or global memory, or the cooperative level sweep
  auto run = [&](int mode, bool profile) -> int {
    int grid;
    bool global = mode == M_GLOBAL;
    if (mode >= M_COOP && sp_kind) {
      a.block = coop_threads(mode);
      a.t = t.view();
      a.wglob = nullptr;
      const size_t sm = smem_coop(kind == PK_SP_REVERSE ? t.rlv_sz_w : t.lv_sz_w);
      grid = grid_for((m + 31) / 32, std::max(1, occupancy_coop_sp(a.block, sm)) * sm_count());
    } else if (mode >= M_COOP) {
      a.block = coop_threads(mode);
      a.t = t.view();
      const size_t sm = smem_coop(t.lv_sz_w);
      global = sm > static_cast<size_t>(max_smem_optin());
      const int occ = std::max(1, occupancy_coop(a.block, sm, global));
      grid = grid_for((m + 31) / 32, occ * sm_count());
      a.wglob = nullptr;
      if (global)
        if (int rc = gw_prepare(t, a, &grid, static_cast<size_t>(t.lv_sz_w) * 32 * 8, s)) return rc;
    } else if (global) {
      a.block = kGwBlock;
      const int occ =
          std::max(1, kind >= PK_SP_FORWARD ? occupancy_gw_sp()
                                            : occupancy_gw_primal(kind == PK_RECORD));
      grid = grid_for((m + kGwBlock - 1) / kGwBlock, occ * sm_count());
      const size_t elem = 8;  // a double or a bvec_t per slot and instance
      if (int rc = gw_prepare(t, a, &grid,
                              static_cast<size_t>(std::max(1, t.sz_w)) * kGwBlock * elem, s))
        return rc;
    } else {
      a.block = t.primal_block;
      a.wglob = nullptr;
      grid = grid_for((m + a.block - 1) / a.block, t.primal_grid_cap);
    }
    auto launch = [&] {
      if (mode >= M_COOP)
        return sp_kind ? launch_coop_sp(a, kind == PK_SP_REVERSE, grid, s)
                       : launch_coop(a, kind == PK_RECORD, grid, s);
      return go(grid);
    };
    cudaError_t e = profile ? timed(fam[kind], s, launch) : launch();
    if (e != cudaSuccess) return cuda_fail(e, what[kind]);
    if (global) {
      a.wglob = nullptr;
      if (int rc = gw_done(t, s)) return rc;
    }
    return 0;
  };
  const bool coop_kind = kind == PK_EVAL || kind == PK_RECORD || sp_kind;
  const bool rev = kind == PK_SP_REVERSE;
  const int cls = (m + 31) / 32 <= 16ll * sm_count() ? 0 : 1;
  // the cooperative sweep is a candidate for launches of few tiles (or when forced); the
  // sparsity sweeps' version needs its schedule's work vector in shared memory
  const bool want_coop = coop_kind && (cls == 0 || t.residence == 3);
  bool can_coop = want_coop && (capturing(s) ? (rev ? t.rlv_state : t.lv_state) > 0
                                             : ensure_levels(t, rev));
  if (can_coop && sp_kind)
    can_coop = smem_coop(rev ? t.rlv_sz_w : t.lv_sz_w) <= static_cast<size_t>(max_smem_optin());
  const int coop_default = M_COOP + (coop_threads_for((m + 31) / 32) == 1024
                                         ? 2 : coop_threads_for((m + 31) / 32) == 512 ? 1 : 0);
  if (t.residence == 3 && coop_kind && can_coop) return run(coop_default, true);
  if (t.residence == 1 || !fits_smem(t.sz_w)) {
    if (!(coop_kind && can_coop && cls == 0 && t.residence != 1)) return run(M_GLOBAL, true);
  } else if (t.residence == 2) {
    return run(M_SHARED, true);
  }
  int cand[5], nc = 0;
  if (fits_smem(t.sz_w)) cand[nc++] = M_SHARED;
  cand[nc++] = M_GLOBAL;
  if (coop_kind && can_coop && (cls == 0 || t.residence == 3))
    for (int c = M_COOP; c <= M_COOP_LAST; ++c) cand[nc++] = c;
  std::atomic<int>& choice = t.primal_tuned[kind][cls];
  // sp_reverse consumes its seeds and cannot be timed twice: it follows sp_forward's choice
  if (rev && choice < 0 && t.primal_tuned[PK_SP_FORWARD][cls] >= 0)
    choice = t.primal_tuned[PK_SP_FORWARD][cls].load();
  // residence is tuned like the derivative variants: every candidate timed once on the first
  // call of each kind and size class (every sweep here but sp_reverse, which consumes its
  // seeds, can run twice with the same results)
  std::unique_lock<std::mutex> tune_lock(t.tune_mtx, std::defer_lock);
  if (choice < 0 && nc > 1 && g_autotune && kind != PK_SP_REVERSE && !capturing(s) &&
      tune_lock.try_lock()) {
    float ms[5] = {0, 0, 0, 0, 0};
    for (int c = 0; c < nc; ++c) {
      int rc = 0;
      if (int trc = time_once(s, [&] { rc = run(cand[c], false); return cudaSuccess; }, &ms[c]))
        return trc;
      if (rc) return rc;
    }
    int best = 0;
    for (int c = 1; c < nc; ++c)
      if (ms[c] < ms[best]) best = c;
    choice = cand[best];
    return 0;  // every run produced the same (complete) results
  }
  const int chosen = choice;
  if (chosen >= 0 && (chosen < M_COOP || can_coop) && (chosen != M_SHARED || fits_smem(t.sz_w)))
    return run(chosen, true);
  return run(cand[0], true);
}

// One derivative sweep after the record sweep: ndir directions, forward (seeded or identity)
// or adjoint, with its seed and sensitivity descriptors over the whole instance range.
struct DerivReq {
  int ndir = 0;
  bool adjoint = false;
  bool identity = false;
  const std::vector<int>* dirmap = nullptr;  // identity mode: direction of each input nonzero
  const IoDesc* seed = nullptr;
  const IoDesc* sens = nullptr;
};

// Runs one derivative sweep of wave `a` (values and partials already recorded).
// Tangent sweep launch; with more items than CTAs the items past the grid come from the work
// counter a.queue (zeroed here), otherwise every CTA takes one item by index.
cudaError_t launch_tangent_queued(const SweepArgs& a, int grid, bool more_items, int variant,
                                  cudaStream_t s) {
  SweepArgs b = a;
  if (!more_items) b.queue = nullptr;
  if (b.queue)
    if (cudaError_t e = cudaMemsetAsync(b.queue, 0, sizeof(*b.queue), s)) return e;
  return launch_tangent(b, grid, variant, s);
}

// The keyed streams (every group-size layout) and work order of a tangent plan.
void set_streams(SweepArgs& a, const TanPlan* tp) {
  for (int gs = 0; gs < kNumGroupSizes; ++gs) {
    a.dstreams[gs] = tp->d_stream[gs];
    a.dchunkss[gs] = tp->d_chunks[gs];
  }
  a.gorder = tp->d_order;
}

int run_deriv(Tape& t, SweepArgs a, long long m, const DerivReq& rq, cudaStream_t s) {
  const int ndir = rq.ndir;
  const bool adjoint = rq.adjoint, identity = rq.identity;
  const int kind = adjoint ? 2 : (identity ? 1 : 0);
  const int sms = sm_count();
  int err = 0;
  const AdjPlan* ap = nullptr;
  std::vector<char> seeded_in(t.n_in);
  for (int j = 0; j < t.n_in; ++j) seeded_in[j] = rq.seed && rq.seed[j].ptr != nullptr;
  // tangents: outputs whose sensitivities are requested (the others' instructions are pruned)
  std::vector<char> wanted_out(adjoint ? 0 : t.n_out);
  for (int j = 0; j < static_cast<int>(wanted_out.size()); ++j)
    wanted_out[j] = rq.sens && rq.sens[j].ptr != nullptr;
  if (adjoint) {
    std::vector<char> seeded(t.n_out);
    for (int j = 0; j < t.n_out; ++j) seeded[j] = rq.seed[j].ptr != nullptr;
    ap = adj_plan(t, 1, 0, seeded, &err);
    if (!ap) return err ? err : fail(CASADI_GB300_ERR_CUDA, "activity plan");
  }
  a.ndir = ndir;
  a.identity_seed = identity ? 1 : 0;
  std::memcpy(a.seed, rq.seed, sizeof(IoDesc) * (adjoint ? t.n_out : t.n_in));
  std::memcpy(a.sens, rq.sens, sizeof(IoDesc) * (adjoint ? t.n_in : t.n_out));
  a.block = 32;
  a.chunk = 0;
  if (ap) {
    for (int gs = 0; gs < kNumGroupSizes; ++gs) {
      a.dstreams[gs] = ap->d_stream[gs];
      a.dchunkss[gs] = ap->d_chunks[gs];
    }
    a.zero_in = ap->d_zero;
    a.n_zero = ap->n_zero;
  }
  const long long tiles = (m + 31) / 32;
  auto shape = [&](int v, int* ipt, int* kd) {
    if (adjoint) {
      *ipt = adj_variant_ipt(v);
      *kd = 1;
    } else {
      tan_variant_shape(v, ipt, kd);
    }
  };
  // a variant whose work vector (IPT tiles x K directions per warp) does not fit, or whose
  // union-stream encoding does not (K > 1 needs slot offsets below 2^19), is never launched
  auto fits = [&](int v) {
    int ipt, kd;
    shape(v, &ipt, &kd);
    if (kd > 1 && static_cast<long long>(t.sz_w) * 256 >= (1ll << 19)) return false;
    return smem_lean(t.sz_w, ipt * kd, 0) <= static_cast<size_t>(max_smem_optin());
  };
  auto work_of = [&](int v) {
    int ipt, kd;
    shape(v, &ipt, &kd);
    return (tiles + ipt - 1) / ipt * ((ndir + kd - 1) / kd);
  };
  auto grid_of = [&](int v) {
    int ipt, kd;
    shape(v, &ipt, &kd);
    const long long vwork = work_of(v);
    const int occ = std::max(1, occupancy_dir(v, adjoint, smem_lean(t.sz_w, ipt * kd, 0)));
    return static_cast<int>(std::max<long long>(
        1, std::min<long long>(vwork, static_cast<long long>(sms) * occ)));
  };
  int plan_err = 0;
  auto launch = [&](int v) {
    if (adjoint) return launch_adjoint(a, grid_of(v), v, s);
    int ipt = 1, kd = 1;
    tan_variant_shape(v, &ipt, &kd);
    static const std::vector<int> kNoMap;
    const TanPlan* tp =
        tan_plan(t, ndir, kd, 0, identity, seeded_in, rq.dirmap ? *rq.dirmap : kNoMap,
                 wanted_out, &plan_err);
    if (!tp) return cudaErrorInvalidValue;
    set_streams(a, tp);
    const int grid = grid_of(v);
    return launch_tangent_queued(a, grid, grid < work_of(v), v, s);
  };
  const long long work = tiles * ndir;
  const int cls = tiles <= 16ll * sms ? 0 : 1;
  // the cooperative tangent sweep: a candidate for launches of few tiles whose level schedule
  // (tangents + activity bytes) fits shared memory
  const bool coop_ok =
      cls == 0 &&
      (capturing(s) ? (adjoint ? t.rlv_state : t.lv_state) > 0 : ensure_levels(t, adjoint)) &&
      smem_tangent_coop(adjoint ? t.rlv_sz_w : t.lv_sz_w, false) <=
          static_cast<size_t>(max_smem_optin());
  const int kCoop = adjoint ? AV_COUNT : TV_COUNT;
  auto launch_coop_adj = [&]() -> cudaError_t {
    SweepArgs c = a;
    c.t = t.view();
    c.block = kCoopTanThreads;
    c.wglob = nullptr;
    const int occ =
        std::max(1, occupancy_adjoint_coop(smem_tangent_coop(t.rlv_sz_w, false)));
    const int grid = static_cast<int>(std::max<long long>(
        1, std::min<long long>(work, static_cast<long long>(sms) * occ)));
    return launch_adjoint_coop(c, grid, s);
  };
  auto launch_coop_tan = [&]() -> cudaError_t {
    static const std::vector<int> kNoMap;
    const TanPlan* tp =
        tan_plan(t, ndir, 1, 0, identity, seeded_in, rq.dirmap ? *rq.dirmap : kNoMap,
                 wanted_out, &plan_err);
    if (!tp) return cudaErrorInvalidValue;
    SweepArgs c = a;
    c.t = t.view();
    c.block = kCoopTanThreads;
    c.wglob = nullptr;
    c.dirmap = tp->d_dirmap;
    const size_t sm = smem_tangent_coop(t.lv_sz_w, false);
    const int occ = std::max(1, occupancy_tangent_coop(sm, false));
    const int grid = static_cast<int>(std::max<long long>(
        1, std::min<long long>(work, static_cast<long long>(sms) * occ)));
    return launch_tangent_coop(c, grid, s);
  };
  if (dir_global(t)) {
    // global work vectors: one variant (G=2, 64 registers), one warp per CTA
    int grid = static_cast<int>(std::max<long long>(
        1, std::min<long long>(work, static_cast<long long>(sms) *
                                         std::max(1, occupancy_gw_dir(adjoint)))));
    if (int rc = gw_prepare(t, a, &grid, static_cast<size_t>(std::max(1, t.sz_w)) * 256, s))
      return rc;
    cudaError_t e = timed(adjoint ? F_ADJOINT : F_TANGENT, s, [&] {
      if (adjoint) return launch_adjoint(a, grid, 0, s);
      static const std::vector<int> kNoMap;
      const TanPlan* tp = tan_plan(t, ndir, 1, 0, identity, seeded_in,
                                   rq.dirmap ? *rq.dirmap : kNoMap, wanted_out, &plan_err);
      if (!tp) return cudaErrorInvalidValue;
      set_streams(a, tp);
      return launch_tangent_queued(a, grid, grid < work, 0, s);
    });
    if (plan_err) return plan_err;
    if (e != cudaSuccess) return cuda_fail(e, "derivative sweep launch");
    return gw_done(t, s);
  }
  // the windowed tangent sweep (directions of a tile co-scheduled on one SM, partials and
  // entries staged window by window): a candidate for tangent sweeps with enough directions
  const int kWin = TV_COUNT + 1;
  const WinPlan* wp = nullptr;
  auto win = [&]() -> const WinPlan* {
    static const std::vector<int> kNoMap;
    if (!wp && !plan_err)
      wp = win_plan(t, ndir, identity, seeded_in, rq.dirmap ? *rq.dirmap : kNoMap, wanted_out,
                    &plan_err);
    return wp;
  };
  auto launch_win = [&]() -> cudaError_t {
    const WinPlan* p = win();
    if (!p || !p->usable) return cudaErrorInvalidValue;
    SweepArgs c = a;
    c.win_blocks = p->d_blocks;
    c.win_meta = p->d_meta;
    c.win_n = p->nwin;
    c.win_dirs = p->dirs;
    c.win_stages = p->stages;
    c.win_rows = p->rows;
    c.win_ents = p->ents;
    c.block = (p->dirs + 1) * 32;
    const long long items = tiles * p->groups;
    const int grid = static_cast<int>(std::max<long long>(1, std::min<long long>(items, sms)));
    return launch_tangent_win(c, grid, s);
  };
  const int n_variants = adjoint ? AV_COUNT : TV_COUNT;
  auto usable = [&](int v) {
    if (v == kWin) return !adjoint && win() && win()->usable;
    return v == kCoop ? coop_ok : (v >= 0 && v < n_variants && fits(v));
  };
  auto run_v = [&](int v) {
    if (v == kWin) return launch_win();
    return v == kCoop ? (adjoint ? launch_coop_adj() : launch_coop_tan()) : launch(v);
  };
  std::atomic<int>& kept = t.tuned[kind][cls];
  int variant = kept;
  if (variant >= 0 && !usable(variant)) variant = -1;
  if (variant < 0) {
    // tune outside capture: on waves that fill the GPU at least twice at 8 warps per SM, and
    // on every small launch, where the cooperative sweep is a candidate too
    std::unique_lock<std::mutex> tune_lock(t.tune_mtx, std::defer_lock);
    if (g_autotune && !capturing(s) && (work >= 2ll * sms * 8 || cls == 0) &&
        tune_lock.try_lock()) {
      float best = 0;
      for (int c = 0; c <= n_variants + (adjoint ? 0 : 1); ++c) {
        // the variants of the kind, then the cooperative sweep, then (tangents) the windowed
        const int v = c < n_variants ? c : (c == n_variants ? kCoop : kWin);
        if (!usable(v)) continue;
        float ms = 0;
        if (int rc = time_once(s, [&] { return run_v(v); }, &ms)) return plan_err ? plan_err : rc;
        if (variant < 0 || ms < best) {
          best = ms;
          variant = v;
        }
      }
      kept = variant;
      return 0;  // every variant's run produced this wave's (identical) results
    }
    variant = 0;  // the first variant of each list: fastest on the tapes measured
    while (variant < n_variants && !fits(variant)) ++variant;
    if (variant == n_variants)
      return fail(CASADI_GB300_ERR_UNSUPPORTED, "no derivative-sweep variant fits");
  }
  cudaError_t e = timed(adjoint ? F_ADJOINT : F_TANGENT, s, [&] { return run_v(variant); });
  if (plan_err) return plan_err;
  if (e != cudaSuccess) return cuda_fail(e, "derivative sweep launch");
  return 0;
}

// Values + partials (record sweep) followed by the derivative sweeps `reqs`, which all read
// the same recorded partials, in waves of as many instances as the scratch holds.
// `in/out` and the requests' descriptors address the whole instance range.
int run_ad_multi(Tape& t, long long n, const IoDesc* in, const IoDesc* out,
                 const DerivReq* reqs, int nreq, void* scratch, size_t scratch_bytes,
                 cudaStream_t s, bool recorded = false) {
  if (n == 0) return 0;
  const long long cap = wave_capacity(t, n, scratch_bytes);
  // recorded: the scratch already holds the partials of all n instances (one wave), and the
  // values were written by that record sweep
  if (recorded && cap < n)
    return fail(CASADI_GB300_ERR_SCRATCH, "recorded partials cover fewer than %lld instances", n);
  if (t.n_partials > 0 && (scratch == nullptr || cap < 32))
    return fail(CASADI_GB300_ERR_SCRATCH,
                "scratch of %zu bytes is below the minimum of %lld bytes for this tape",
                scratch_bytes, 32ll * 8ll * t.n_partials);
  bool any = false;
  for (int r = 0; r < nreq; ++r) any = any || reqs[r].ndir > 0;
  if (any && static_cast<unsigned>(t.n_partials) >= kMaxPartials)
    return fail(CASADI_GB300_ERR_UNSUPPORTED, "tape records %d partials per instance (max %u)",
                t.n_partials, kMaxPartials - 1);
  for (long long i0 = 0; i0 < n; i0 += cap) {
    const long long m = std::min(cap, n - i0);
    SweepArgs a = base_args(t, m, i0);
    a.partials = static_cast<double*>(scratch);
    // the tangent sweep's work counter: 8 bytes past the wave's partials, where the scratch
    // has them (the scratch sizes this library reports always do); otherwise the sweep
    // strides statically
    const size_t used = 8ull * t.n_partials * static_cast<size_t>(cap);
    if (scratch && scratch_bytes >= used + sizeof(unsigned long long))
      a.queue = reinterpret_cast<unsigned long long*>(static_cast<char*>(scratch) + used);
    a.pofs = t.d_pofs;
    a.n_code = t.n_chunks * kChunk;
    for (int j = 0, off = 0; j < t.n_in; off += t.nnz_in[j], ++j) a.in_off[j] = off;
    std::memcpy(a.in, in, sizeof(IoDesc) * t.n_in);
    std::memcpy(a.out, out, sizeof(IoDesc) * t.n_out);
    if (!recorded)
      if (int rc = primal_launch(t, a, m, PK_RECORD, s)) return rc;
    for (int r = 0; r < nreq; ++r)
      if (reqs[r].ndir > 0)
        if (int rc = run_deriv(t, a, m, reqs[r], s)) return rc;
  }
  return 0;
}

int run_ad(Tape& t, long long n, const IoDesc* in, const IoDesc* out, const IoDesc* seed,
           const IoDesc* sens, int ndir, bool adjoint, bool identity, void* scratch,
           size_t scratch_bytes, cudaStream_t s, bool recorded = false) {
  DerivReq rq;
  rq.ndir = ndir;
  rq.adjoint = adjoint;
  rq.identity = identity;
  rq.seed = seed;
  rq.sens = sens;
  return run_ad_multi(t, n, in, out, &rq, 1, scratch, scratch_bytes, s, recorded);
}

// Pointer arrays of any element type, seen as untyped pointers (the kernels know the type).
template <class T>
void* const* vptrs(T* const* p) {
  return (void* const*)(p);
}

int check_n(long long n, long long ld) {
  if (n < 0) return fail(CASADI_GB300_ERR_ARG, "negative instance count");
  if (ld < n) return fail(CASADI_GB300_ERR_ARG, "leading dimension %lld < n %lld", ld, n);
  return 0;
}

// Validation and encoding of a reference-format tape (host only: no device calls, so the
// checks and the scheduler also run on machines without a GPU).
struct Encoded {
  std::vector<u64> code;  // reference order and slots
  std::vector<double> consts;
  std::vector<int2> absent_in;
  long long n_partials = 0;
};

// all_outputs: every output nonzero must be written (a user's tape); a segment tape of the
// checkpointed adjoint writes only the outputs of its own instructions.
int encode_tape(const casadi_gb300_atomic* alg, int n_instr, int n_in, const int* nnz_in,
                int n_out, const int* nnz_out, int sz_w, Encoded& enc_out,
                bool all_outputs = true) {
  if (n_instr < 0 || (n_instr > 0 && !alg)) return fail(CASADI_GB300_ERR_ARG, "no instructions");
  if (n_in < 0 || n_out < 0 || sz_w < 0) return fail(CASADI_GB300_ERR_ARG, "negative size");
  if ((n_in > 0 && !nnz_in) || (n_out > 0 && !nnz_out))
    return fail(CASADI_GB300_ERR_ARG, "missing nnz arrays");
  if (n_in > kMaxIo || n_out > kMaxIo)
    return fail(CASADI_GB300_ERR_UNSUPPORTED, "more than %d inputs or outputs", kMaxIo);
  if (static_cast<unsigned>(sz_w) > kFieldMax)
    return fail(CASADI_GB300_ERR_UNSUPPORTED, "work vector of %d slots exceeds %u", sz_w,
                kFieldMax);
  for (int j = 0; j < n_in; ++j)
    if (nnz_in[j] < 0 || static_cast<unsigned>(nnz_in[j]) > kFieldMax)
      return fail(CASADI_GB300_ERR_ARG, "bad nnz_in");
  for (int j = 0; j < n_out; ++j)
    if (nnz_out[j] < 0 || static_cast<unsigned>(nnz_out[j]) > kFieldMax)
      return fail(CASADI_GB300_ERR_ARG, "bad nnz_out");
  // every index is checked here; kernels trust the stream
  std::vector<u64>& code = enc_out.code;
  std::vector<double>& consts = enc_out.consts;
  std::vector<std::vector<char>> seen_in(n_in);
  std::vector<std::vector<char>> seen_out(n_out);
  for (int j = 0; j < n_in; ++j) seen_in[j].assign(nnz_in[j], 0);
  for (int j = 0; j < n_out; ++j) seen_out[j].assign(nnz_out[j], 0);
  code.reserve(n_instr);
  long long n_partials = 0;
  auto slot_ok = [&](int s) { return s >= 0 && s < sz_w; };
  for (int k = 0; k < n_instr; ++k) {
    const casadi_gb300_atomic& e = alg[k];
    const int op = e.op;
    if (op == kOpParameter)
      return fail(CASADI_GB300_ERR_UNSUPPORTED, "instruction %d: free parameter (OP_PARAMETER)", k);
    if (op == kOpCall)
      return fail(CASADI_GB300_ERR_UNSUPPORTED,
                  "instruction %d: OP_CALL needs its callees (casadi_gb300_tape_create_calls)", k);
    const int dop = device_opcode(op);
    if (dop < 0) return fail(CASADI_GB300_ERR_UNSUPPORTED, "instruction %d: unknown op %d", k, op);
    if (dop == D_CONST) {
      if (!slot_ok(e.i0)) return fail(CASADI_GB300_ERR_ARG, "instruction %d: slot out of range", k);
      if (consts.size() >= kFieldMax) return fail(CASADI_GB300_ERR_UNSUPPORTED, "too many constants");
      code.push_back(enc(D_CONST, e.i0, static_cast<unsigned>(consts.size()), 0));
      consts.push_back(e.a.d);
    } else if (dop == D_INPUT) {
      const int j = e.a.i[0], nz = e.a.i[1];
      if (!slot_ok(e.i0) || j < 0 || j >= n_in || nz < 0 || nz >= nnz_in[j])
        return fail(CASADI_GB300_ERR_ARG, "instruction %d: input reference out of range", k);
      seen_in[j][nz] = 1;
      code.push_back(enc(D_INPUT, e.i0, j, nz));
    } else if (dop == D_OUTPUT) {
      const int j = e.i0, s = e.a.i[0], nz = e.a.i[1];
      if (j < 0 || j >= n_out || !slot_ok(s) || nz < 0 || nz >= nnz_out[j])
        return fail(CASADI_GB300_ERR_ARG, "instruction %d: output reference out of range", k);
      if (seen_out[j][nz])
        return fail(CASADI_GB300_ERR_ARG, "instruction %d: output nonzero written twice", k);
      seen_out[j][nz] = 1;
      code.push_back(enc(D_OUTPUT, j, s, nz));
    } else {
      const int b = e.a.i[0], c = is_binary(dop) ? e.a.i[1] : e.a.i[0];
      if (!slot_ok(e.i0) || !slot_ok(b) || !slot_ok(c))
        return fail(CASADI_GB300_ERR_ARG, "instruction %d: slot out of range", k);
      code.push_back(enc(dop, e.i0, b, c));
      n_partials += __builtin_popcount(partial_mask(dop));
    }
  }
  for (int j = 0; j < n_out && all_outputs; ++j)
    for (int nz = 0; nz < nnz_out[j]; ++nz)
      if (!seen_out[j][nz])
        return fail(CASADI_GB300_ERR_ARG, "output %d nonzero %d is never written", j, nz);
  for (int j = 0; j < n_in; ++j)
    for (int nz = 0; nz < nnz_in[j]; ++nz)
      if (!seen_in[j][nz]) enc_out.absent_in.push_back(make_int2(j, nz));
  if (n_partials > (1ll << 31))
    return fail(CASADI_GB300_ERR_UNSUPPORTED, "tape records too many partials");
  enc_out.n_partials = n_partials;
  return 0;
}

// Sine/cosine pairs. The record sweeps compute sin and cos of the operand together for either
// op (one is the value, the other its partial), so a SIN or COS whose operand is the value the
// previous SIN/COS read -- no instruction rewrote that slot in between -- takes that result
// again: bit 63 of its word, which every decoder ignores; the first of such a pair gets bit 62
// (clear on unary ops otherwise), so the value sweeps compute it as one sincos where they would
// call sin and cos. Orders that differ (level schedules, segment tapes) are re-encoded without
// either bit. The 20-step rollout's 80 SIN/COS pairs each save one sincos.
void mark_sincos_pairs(std::vector<u64>& code) {
  unsigned slots = 1;
  for (u64 w : code) slots = std::max(slots, std::max(dec_a(w), std::max(dec_b(w), dec_c(w))) + 1);
  std::vector<long long> ver(slots, -1);  // slot -> instruction that last wrote it
  long long cache_slot = -1, cache_ver = -1, cache_at = -1;
  for (size_t k = 0; k < code.size(); ++k) {
    const u64 w = code[k];
    const unsigned op = dec_op(w);
    if (op == D_SIN || op == D_COS) {
      const unsigned b = dec_b(w);
      if (static_cast<long long>(b) == cache_slot && ver[b] == cache_ver) {
        code[k] = w | kSincosReuse;
        code[cache_at] |= kSincosFirst;  // the value sweeps compute the pair there
      } else {
        cache_slot = b;
        cache_ver = ver[b];
        cache_at = static_cast<long long>(k);
      }
    }
    if (op != D_OUTPUT && op != D_NOP) ver[dec_a(w)] = static_cast<long long>(k);
  }
}

// Encoded tape in the scheduled order; returns the scheduled work-vector length or a status.
int encode_and_schedule(const casadi_gb300_atomic* alg, int n_instr, int n_in,
                        const int* nnz_in, int n_out, const int* nnz_out, int sz_w,
                        Encoded& e, bool all_outputs = true) {
  if (int rc = encode_tape(alg, n_instr, n_in, nnz_in, n_out, nnz_out, sz_w, e, all_outputs))
    return rc;
  std::vector<u64> sched;
  std::string err;
  const int w = schedule_code(e.code, sched, err);
  if (w < 0) return fail(CASADI_GB300_ERR_ARG, "%s", err.c_str());
  e.code.swap(sched);
  mark_sincos_pairs(e.code);
  return w;
}

// One encoded instruction back in the reference's format.
casadi_gb300_atomic decode_atomic(u64 w, const std::vector<double>& consts) {
  casadi_gb300_atomic e;
  std::memset(&e, 0, sizeof(e));
  const unsigned op = dec_op(w);
  e.op = reference_opcode(op);
  e.i0 = static_cast<int>(dec_a(w));
  if (op == D_CONST) {
    e.a.d = consts[dec_b(w)];
  } else {
    e.a.i[0] = static_cast<int>(dec_b(w));
    e.a.i[1] = static_cast<int>(dec_c(w));
  }
  return e;
}

// Validates, encodes, schedules and uploads a tape without registering it. A non-null
// `absent` replaces the list of input nonzeros whose sensitivities the adjoint zeroes.
int make_tape(const casadi_gb300_atomic* alg, int n_instr, int n_in, const int* nnz_in,
              int n_out, const int* nnz_out, int sz_w, bool all_outputs,
              const std::vector<int2>* absent, std::unique_ptr<Tape>& out);

}  // namespace

extern "C" {

const char* casadi_gb300_last_error(void) { return g_err.c_str(); }

const char* casadi_gb300_version(void) { return "0.1.0"; }

int casadi_gb300_tape_create(const casadi_gb300_atomic* alg, int n_instr, int n_in,
                             const int* nnz_in, int n_out, const int* nnz_out, int sz_w) {
  std::unique_ptr<Tape> t;
  if (int rc = make_tape(alg, n_instr, n_in, nnz_in, n_out, nnz_out, sz_w, true, nullptr, t))
    return rc;
  std::lock_guard<std::mutex> lk(g_mtx);
  g_tapes.push_back(std::move(t));
  return static_cast<int>(g_tapes.size()) - 1;
}

}  // extern "C"

namespace {

int make_tape(const casadi_gb300_atomic* alg, int n_instr, int n_in, const int* nnz_in,
              int n_out, const int* nnz_out, int sz_w, bool all_outputs,
              const std::vector<int2>* absent, std::unique_ptr<Tape>& out) {
  Encoded en;
  const int wlen =
      encode_and_schedule(alg, n_instr, n_in, nnz_in, n_out, nnz_out, sz_w, en, all_outputs);
  if (wlen < 0) return wlen;
  auto t = std::make_unique<Tape>();
  t->n_instr = n_instr;
  t->n_in = n_in;
  t->n_out = n_out;
  t->sz_w = wlen;
  t->ref_sz_w = sz_w;
  t->nnz_in.assign(nnz_in, nnz_in + n_in);
  t->nnz_out.assign(nnz_out, nnz_out + n_out);
  t->absent_in = absent ? *absent : en.absent_in;
  std::vector<u64>& code = en.code;
  std::vector<double>& consts = en.consts;
  t->h_consts = consts;
  const long long n_partials = en.n_partials;
  t->n_partials = static_cast<int>(n_partials);
  t->n_chunks = std::max(1, (n_instr + kChunk - 1) / kChunk);
  code.resize(static_cast<size_t>(t->n_chunks) * kChunk, enc(D_NOP, 0, 0, 0));
  t->h_code = code;
  t->pofs.assign(code.size() / kPofsGran + 1, 0);
  for (size_t k = 0, acc = 0; k < code.size(); ++k) {
    if (k % kPofsGran == 0) t->pofs[k / kPofsGran] = static_cast<int>(acc);
    const unsigned op = dec_op(code[k]);
    if (op != D_CONST && op != D_INPUT && op != D_OUTPUT && op != D_NOP)
      acc += __builtin_popcount(partial_mask(op));
    if (k + 1 == code.size()) t->pofs[code.size() / kPofsGran] = static_cast<int>(acc);
  }
  if (consts.empty()) consts.push_back(0.0);

  cudaError_t e = cudaGetDevice(&t->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if ((e = cudaMalloc(&t->d_code, code.size() * sizeof(u64))) != cudaSuccess)
    return cuda_fail(e, "cudaMalloc(code)");
  if ((e = cudaMalloc(&t->d_consts, consts.size() * sizeof(double))) != cudaSuccess)
    return cuda_fail(e, "cudaMalloc(consts)");
  if ((e = cudaMalloc(&t->d_absent, std::max<size_t>(1, t->absent_in.size()) * sizeof(int2))) !=
      cudaSuccess)
    return cuda_fail(e, "cudaMalloc(absent)");
  if ((e = cudaMalloc(&t->d_err, sizeof(int))) != cudaSuccess) return cuda_fail(e, "cudaMalloc(err)");
  if ((e = cudaMalloc(&t->d_pofs, t->pofs.size() * sizeof(int))) != cudaSuccess)
    return cuda_fail(e, "cudaMalloc(pofs)");
  if ((e = cudaMemcpy(t->d_pofs, t->pofs.data(), t->pofs.size() * sizeof(int),
                      cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_fail(e, "upload partial offsets");
  if ((e = cudaMemcpy(t->d_code, code.data(), code.size() * sizeof(u64), cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return cuda_fail(e, "upload code");
  if ((e = cudaMemcpy(t->d_consts, consts.data(), consts.size() * sizeof(double),
                      cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_fail(e, "upload constants");
  if (!t->absent_in.empty() &&
      (e = cudaMemcpy(t->d_absent, t->absent_in.data(), t->absent_in.size() * sizeof(int2),
                      cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_fail(e, "upload absent inputs");
  if ((e = cudaMemset(t->d_err, 0, sizeof(int))) != cudaSuccess) return cuda_fail(e, "clear err");
  choose_shapes(*t);
  out = std::move(t);
  return 0;
}

}  // namespace

extern "C" {

int casadi_gb300_tape_schedule(const casadi_gb300_atomic* alg, int n_instr, int n_in,
                               const int* nnz_in, int n_out, const int* nnz_out, int sz_w,
                               casadi_gb300_atomic* out, int* sz_w_out) {
  if (!out || !sz_w_out) return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  Encoded en;
  const int wlen = encode_and_schedule(alg, n_instr, n_in, nnz_in, n_out, nnz_out, sz_w, en);
  if (wlen < 0) return wlen;
  for (int k = 0; k < n_instr; ++k) out[k] = decode_atomic(en.code[k], en.consts);
  *sz_w_out = wlen;
  return 0;
}

int casadi_gb300_tape_levels(const casadi_gb300_atomic* alg, int n_instr, int n_in,
                             const int* nnz_in, int n_out, const int* nnz_out, int sz_w,
                             int width, int slot_cap, casadi_gb300_atomic* out, int* source,
                             int* level_begin, int* n_levels, int* sz_w_out) {
  if (!n_levels || !sz_w_out || width == 0 || width < -(1 << 20) || slot_cap < 1)
    return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  // a negative width asks for the schedule of the cooperative reverse sweep (ordered users)
  const bool ordered = width < 0;
  if (ordered) width = -width;
  Encoded en;
  const int wlen = encode_and_schedule(alg, n_instr, n_in, nnz_in, n_out, nnz_out, sz_w, en);
  if (wlen < 0) return wlen;
  Levels lv;
  std::string err;
  const int nl = level_schedule(en.code, width, slot_cap, lv, err, ordered);
  if (nl < 0) return fail(CASADI_GB300_ERR_ARG, "%s", err.c_str());
  *n_levels = nl;
  *sz_w_out = lv.sz_w;
  if (level_begin)
    for (int l = 0; l <= nl; ++l) level_begin[l] = lv.begin[l];
  for (size_t k = 0; k < lv.code.size(); ++k) {
    if (source) source[k] = lv.src[k];
    if (!out) continue;
    const u64 w = lv.code[k];
    const unsigned op = dec_op(w);
    casadi_gb300_atomic& e = out[k];
    std::memset(&e, 0, sizeof(e));
    e.op = reference_opcode(op);
    e.i0 = static_cast<int>(dec_a(w));
    if (op == D_CONST) {
      e.a.d = en.consts[dec_b(w)];
    } else {
      e.a.i[0] = static_cast<int>(dec_b(w));
      e.a.i[1] = static_cast<int>(dec_c(w));
    }
  }
  return 0;
}

static int check_ccs(int nrow, int ncol, const int* colind, const int* row) {
  if (nrow < 0 || ncol < 0 || !colind) return fail(CASADI_GB300_ERR_ARG, "bad pattern size");
  if (colind[0] != 0) return fail(CASADI_GB300_ERR_ARG, "colind[0] must be 0");
  for (int j = 0; j < ncol; ++j)
    if (colind[j] > colind[j + 1]) return fail(CASADI_GB300_ERR_ARG, "colind not increasing");
  const int nnz = colind[ncol];
  if (nnz > 0 && !row) return fail(CASADI_GB300_ERR_ARG, "missing row array");
  for (int j = 0; j < ncol; ++j)
    for (int k = colind[j]; k < colind[j + 1]; ++k) {
      if (row[k] < 0 || row[k] >= nrow) return fail(CASADI_GB300_ERR_ARG, "row out of range");
      if (k > colind[j] && row[k] <= row[k - 1])
        return fail(CASADI_GB300_ERR_ARG, "rows not sorted within column %d", j);
    }
  return 0;
}

int casadi_gb300_uni_coloring(int nrow, int ncol, const int* colind, const int* row,
                              int* color) {
  if (int rc = check_ccs(nrow, ncol, colind, row)) return rc;
  if (ncol > 0 && !color) return fail(CASADI_GB300_ERR_ARG, "missing color array");
  return uni_coloring_ccs(nrow, ncol, colind, row, color);
}

int casadi_gb300_star_coloring(int n, const int* colind, const int* row, int ordering,
                               int* color) {
  if (int rc = check_ccs(n, n, colind, row)) return rc;
  if (n > 0 && !color) return fail(CASADI_GB300_ERR_ARG, "missing color array");
  if (ordering != 0 && ordering != 1) return fail(CASADI_GB300_ERR_ARG, "ordering must be 0 or 1");
  return star_coloring_ccs(n, colind, row, ordering, color);
}

int casadi_gb300_tape_create_calls(const casadi_gb300_atomic* alg, int n_instr, int n_in,
                                   const int* nnz_in, int n_out, const int* nnz_out, int sz_w,
                                   int n_calls, const int* call_tape,
                                   const int* const* call_dep, const int* const* call_res) {
  if (n_instr < 0 || (n_instr > 0 && !alg)) return fail(CASADI_GB300_ERR_ARG, "no instructions");
  if (n_calls < 0 || (n_calls > 0 && (!call_tape || !call_dep || !call_res)))
    return fail(CASADI_GB300_ERR_ARG, "missing call tables");
  if (sz_w < 0) return fail(CASADI_GB300_ERR_ARG, "negative size");
  // Inline every OP_CALL: the callee's instructions with their slots moved past the caller's
  // work vector, its inputs copied in from the call's dep slots and its outputs copied out to
  // the res slots (SXFunction::call_fwd, casadi/core/sx_function.cpp:1595-1621)
  std::vector<casadi_gb300_atomic> out;
  out.reserve(n_instr);
  long long wlen = sz_w;
  for (int k = 0; k < n_instr; ++k) {
    const casadi_gb300_atomic& e = alg[k];
    if (e.op != kOpCall) {
      out.push_back(e);
      continue;
    }
    const int ci = e.a.i[0];
    if (ci < 0 || ci >= n_calls)
      return fail(CASADI_GB300_ERR_ARG, "instruction %d: call index %d out of range", k, ci);
    Tape* f = get_tape(call_tape[ci]);
    if (!f) return fail(CASADI_GB300_ERR_ID, "call %d: no tape with id %d", ci, call_tape[ci]);
    const int* dep = call_dep[ci];
    const int* res = call_res[ci];
    int nzi = 0, nzo = 0;
    for (int v : f->nnz_in) nzi += v;
    for (int v : f->nnz_out) nzo += v;
    if ((nzi > 0 && !dep) || (nzo > 0 && !res))
      return fail(CASADI_GB300_ERR_ARG, "call %d: missing dep/res slots", ci);
    for (int i = 0; i < nzi; ++i)
      if (dep[i] < 0 || dep[i] >= sz_w)
        return fail(CASADI_GB300_ERR_ARG, "call %d: dep slot out of range", ci);
    for (int i = 0; i < nzo; ++i)
      if (res[i] < -1 || res[i] >= sz_w)
        return fail(CASADI_GB300_ERR_ARG, "call %d: res slot out of range", ci);
    std::vector<int> off_in(f->n_in + 1, 0), off_out(f->n_out + 1, 0);
    for (int j = 0; j < f->n_in; ++j) off_in[j + 1] = off_in[j] + f->nnz_in[j];
    for (int j = 0; j < f->n_out; ++j) off_out[j + 1] = off_out[j] + f->nnz_out[j];
    const long long base = wlen;
    wlen += std::max(1, f->sz_w);
    if (wlen > kFieldMax)
      return fail(CASADI_GB300_ERR_UNSUPPORTED, "inlined work vector exceeds %u slots", kFieldMax);
    auto emit = [&](int op, long long i0, int i1, int i2, double d) {
      casadi_gb300_atomic a;
      std::memset(&a, 0, sizeof(a));
      a.op = op;
      a.i0 = static_cast<int>(i0);
      if (op == kOpConst) {
        a.a.d = d;
      } else {
        a.a.i[0] = i1;
        a.a.i[1] = i2;
      }
      out.push_back(a);
    };
    for (u64 w : f->h_code) {
      const unsigned op = dec_op(w), A = dec_a(w), B = dec_b(w), C = dec_c(w);
      switch (op) {
        case D_NOP:
          break;
        case D_INPUT: {
          const int slot = dep[off_in[B] + static_cast<int>(C)];
          emit(0 /* OP_ASSIGN */, base + A, slot, slot, 0.0);
        } break;
        case D_OUTPUT: {
          const int r = res[off_out[A] + static_cast<int>(C)];
          if (r >= 0) emit(0 /* OP_ASSIGN */, r, static_cast<int>(base + B), static_cast<int>(base + B), 0.0);
        } break;
        case D_CONST:
          emit(kOpConst, base + A, 0, 0, f->h_consts[B]);
          break;
        default:
          emit(reference_opcode(op), base + A, static_cast<int>(base + B),
               static_cast<int>(base + C), 0.0);
      }
    }
  }
  if (out.size() > static_cast<size_t>(0x7fffffff))
    return fail(CASADI_GB300_ERR_UNSUPPORTED, "inlined tape too long");
  return casadi_gb300_tape_create(out.data(), static_cast<int>(out.size()), n_in, nnz_in, n_out,
                                  nnz_out, static_cast<int>(wlen));
}

// Tapes from CasADi's serialized text (serial.cu decodes it on the host).
int casadi_gb300_serialized_describe(const char* text, size_t len, char* buf, size_t cap,
                                     size_t* need) {
  SerialModel m;
  std::string err;
  if (int rc = decode_serialized(text, len, m, err)) return fail(rc, "%s", err.c_str());
  const std::string d = describe_serialized(m);
  if (need) *need = d.size() + 1;
  if (buf && cap > 0) {
    const size_t n = std::min(cap - 1, d.size());
    std::memcpy(buf, d.data(), n);
    buf[n] = '\0';
  }
  return 0;
}

extern "C++" {
namespace {
// The serialized top-level SXFunction, or an error.
int serialized_sx(const char* text, size_t len, SerialModel& m) {
  std::string err;
  if (int rc = decode_serialized(text, len, m, err)) return fail(rc, "%s", err.c_str());
  if (m.tops.size() != 1)
    return fail(CASADI_GB300_ERR_ARG, "the text holds %zu Functions (casadi_gb300_push_file "
                "loads them all)", m.tops.size());
  if (m.top < 0) return fail(CASADI_GB300_ERR_ARG, "the serialized Function is null");
  const SerialFunction& f = m.functions[static_cast<size_t>(m.top)];
  if (!f.complete)
    return fail(CASADI_GB300_ERR_UNSUPPORTED, "serialized %s '%s': only SXFunction tapes are read",
                f.cls.c_str(), f.name.c_str());
  return 0;
}

std::vector<int> nnz_of(const std::vector<SerialSparsity>& sp) {
  std::vector<int> n(sp.size());
  for (size_t j = 0; j < sp.size(); ++j) n[j] = static_cast<int>(sp[j].nnz);
  return n;
}

int check_serial_function(const SerialFunction& f) {
  if (f.n_free > 0)
    return fail(CASADI_GB300_ERR_UNSUPPORTED,
                "'%s' has %lld free variables (the reference cannot evaluate it either)",
                f.name.c_str(), f.n_free);
  if (f.alg.size() > static_cast<size_t>(1 << 30) || f.sz_w > (1LL << 30))
    return fail(CASADI_GB300_ERR_UNSUPPORTED, "'%s' is too large", f.name.c_str());
  for (const auto& sp : f.sp_in)
    if (sp.nnz > (1LL << 30)) return fail(CASADI_GB300_ERR_UNSUPPORTED, "input too large");
  for (const auto& sp : f.sp_out)
    if (sp.nnz > (1LL << 30)) return fail(CASADI_GB300_ERR_UNSUPPORTED, "output too large");
  return 0;
}

// Tape of function j of the model, its callees' tapes already in ids (they precede it).
int serial_tape_one(const SerialModel& m, int j, std::vector<int>& ids) {
  const SerialFunction& f = m.functions[static_cast<size_t>(j)];
  if (!f.complete)
    return fail(CASADI_GB300_ERR_UNSUPPORTED, "'%s' (%s) is not an SXFunction", f.name.c_str(),
                f.cls.c_str());
  if (int rc = check_serial_function(f)) return rc;
  const std::vector<int> nin = nnz_of(f.sp_in), nout = nnz_of(f.sp_out);
  std::vector<int> call_ids(f.calls.size());
  std::vector<const int*> deps(f.calls.size()), ress(f.calls.size());
  for (size_t c = 0; c < f.calls.size(); ++c) {
    const SerialCall& call = f.calls[c];
    const SerialFunction& g = m.functions[static_cast<size_t>(call.fn)];
    long long nzi = 0, nzo = 0;
    for (const auto& sp : g.sp_in) nzi += sp.nnz;
    for (const auto& sp : g.sp_out) nzo += sp.nnz;
    if (static_cast<long long>(call.dep.size()) != nzi ||
        static_cast<long long>(call.res.size()) != nzo)
      return fail(CASADI_GB300_ERR_ARG, "'%s': call %zu has %zu/%zu slots for %lld/%lld nonzeros",
                  f.name.c_str(), c, call.dep.size(), call.res.size(), nzi, nzo);
    call_ids[c] = ids[static_cast<size_t>(call.fn)];
    deps[c] = call.dep.data();
    ress[c] = call.res.data();
  }
  const int id = f.calls.empty()
      ? casadi_gb300_tape_create(f.alg.data(), static_cast<int>(f.alg.size()),
                                 static_cast<int>(nin.size()), nin.data(),
                                 static_cast<int>(nout.size()), nout.data(),
                                 static_cast<int>(f.sz_w))
      : casadi_gb300_tape_create_calls(
            f.alg.data(), static_cast<int>(f.alg.size()), static_cast<int>(nin.size()),
            nin.data(), static_cast<int>(nout.size()), nout.data(), static_cast<int>(f.sz_w),
            static_cast<int>(f.calls.size()), call_ids.data(), deps.data(), ress.data());
  if (id < 0) return id;
  ids[static_cast<size_t>(j)] = id;
  return 0;
}

// Tape of function k of the model, memoized in ids (-1: not created yet). A callee always
// precedes its caller in the model, so the functions k reaches are marked in one descending
// pass and created in index order: no recursion along call chains of any length.
int serial_tape(const SerialModel& m, int k, std::vector<int>& ids) {
  std::vector<char> need(m.functions.size(), 0);
  need[static_cast<size_t>(k)] = 1;
  for (int j = k; j >= 0; --j) {
    if (!need[static_cast<size_t>(j)] || ids[static_cast<size_t>(j)] >= 0) continue;
    const SerialFunction& f = m.functions[static_cast<size_t>(j)];
    for (size_t c = 0; c < f.calls.size(); ++c) {
      const int fn = f.calls[c].fn;
      if (fn < 0 || fn >= j)
        return fail(CASADI_GB300_ERR_ARG, "'%s': call %zu names no earlier function",
                    f.name.c_str(), c);
      need[static_cast<size_t>(fn)] = 1;
    }
  }
  for (int j = 0; j <= k; ++j)
    if (need[static_cast<size_t>(j)] && ids[static_cast<size_t>(j)] < 0)
      if (int rc = serial_tape_one(m, j, ids)) return rc;
  return ids[static_cast<size_t>(k)];
}
}  // namespace
}  // extern "C++"

int casadi_gb300_serialized_decode(const char* text, size_t len, casadi_gb300_atomic* alg,
                                   int cap, int* n_instr, int* n_in, int* nnz_in, int* n_out,
                                   int* nnz_out, int* sz_w) {
  SerialModel m;
  if (int rc = serialized_sx(text, len, m)) return rc;
  const SerialFunction& f = m.functions[static_cast<size_t>(m.top)];
  if (int rc = check_serial_function(f)) return rc;
  if (!f.calls.empty())
    return fail(CASADI_GB300_ERR_UNSUPPORTED,
                "'%s' calls %zu functions: use casadi_gb300_tape_deserialize", f.name.c_str(),
                f.calls.size());
  if (n_instr) *n_instr = static_cast<int>(f.alg.size());
  if (n_in) *n_in = static_cast<int>(f.sp_in.size());
  if (n_out) *n_out = static_cast<int>(f.sp_out.size());
  if (sz_w) *sz_w = static_cast<int>(f.sz_w);
  if (nnz_in)
    for (size_t j = 0; j < f.sp_in.size(); ++j) nnz_in[j] = static_cast<int>(f.sp_in[j].nnz);
  if (nnz_out)
    for (size_t j = 0; j < f.sp_out.size(); ++j) nnz_out[j] = static_cast<int>(f.sp_out[j].nnz);
  if (alg) {
    if (cap < static_cast<int>(f.alg.size()))
      return fail(CASADI_GB300_ERR_ARG, "instruction buffer of %d for %zu instructions", cap,
                  f.alg.size());
    std::memcpy(alg, f.alg.data(), f.alg.size() * sizeof(casadi_gb300_atomic));
  }
  return 0;
}

// Functions loaded from files, as casadi_c keeps them (casadi/core/casadi_c.cpp:31-130):
// names and tape ids, and how many each push added
extern "C++" {
namespace {
std::mutex g_loaded_mtx;
std::vector<std::pair<std::string, int>> g_loaded;
std::vector<int> g_load_stack;
}  // namespace
}  // extern "C++"

int casadi_gb300_push_file(const char* filename) {
  if (!filename) return fail(CASADI_GB300_ERR_ARG, "null file name");
  std::string text;
  {
    FILE* fh = std::fopen(filename, "rb");
    if (!fh) return fail(CASADI_GB300_ERR_ARG, "could not open '%s'", filename);
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), fh)) > 0) text.append(buf, got);
    std::fclose(fh);
  }
  SerialModel m;
  std::string err;
  if (int rc = decode_serialized(text.data(), text.size(), m, err))
    return fail(rc, "%s: %s", filename, err.c_str());
  if (!m.saved_form)
    return fail(CASADI_GB300_ERR_ARG, "%s holds no 'function' or 'function_vector'", filename);
  std::vector<int> ids(m.functions.size(), -1);
  std::vector<std::pair<std::string, int>> added;
  int rc = 0;
  for (int k : m.tops) {
    if (k < 0) {
      rc = fail(CASADI_GB300_ERR_ARG, "%s holds a null Function", filename);
      break;
    }
    const int id = serial_tape(m, k, ids);
    if (id < 0) {
      rc = id;
      break;
    }
    added.emplace_back(m.functions[static_cast<size_t>(k)].name, id);
  }
  // keep the tapes of the file's Functions, free the called ones (they were inlined)
  for (size_t k = 0; k < ids.size(); ++k) {
    if (ids[k] < 0) continue;
    bool keep = false;
    for (const auto& a : added) keep = keep || (rc == 0 && a.second == ids[k]);
    if (!keep) casadi_gb300_tape_free(ids[k]);
  }
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_loaded_mtx);
  g_loaded.insert(g_loaded.end(), added.begin(), added.end());
  g_load_stack.push_back(static_cast<int>(added.size()));
  return 0;
}

int casadi_gb300_n_loaded(void) {
  std::lock_guard<std::mutex> lk(g_loaded_mtx);
  return static_cast<int>(g_loaded.size());
}

int casadi_gb300_loaded_tape(const char* name) {
  std::lock_guard<std::mutex> lk(g_loaded_mtx);
  if (!name) return fail(CASADI_GB300_ERR_ARG, "null name");
  for (const auto& a : g_loaded)
    if (a.first == name) return a.second;
  std::string avail;
  for (const auto& a : g_loaded) avail += " " + a.first;
  return fail(CASADI_GB300_ERR_ID, "no loaded function named '%s' (loaded:%s)", name,
              avail.c_str());
}

const char* casadi_gb300_loaded_name(int k) {
  std::lock_guard<std::mutex> lk(g_loaded_mtx);
  if (k < 0 || k >= static_cast<int>(g_loaded.size())) return nullptr;
  return g_loaded[static_cast<size_t>(k)].first.c_str();
}

int casadi_gb300_pop_file(void) {
  std::lock_guard<std::mutex> lk(g_loaded_mtx);
  if (g_load_stack.empty()) return fail(CASADI_GB300_ERR_ARG, "nothing was pushed");
  for (int c = g_load_stack.back(); c > 0; --c) {
    casadi_gb300_tape_free(g_loaded.back().second);
    g_loaded.pop_back();
  }
  g_load_stack.pop_back();
  return 0;
}

int casadi_gb300_tape_deserialize(const char* text, size_t len) {
  SerialModel m;
  if (int rc = serialized_sx(text, len, m)) return rc;
  std::vector<int> ids(m.functions.size(), -1);
  const int id = serial_tape(m, m.top, ids);
  // the called functions' tapes were inlined into the caller's
  for (size_t k = 0; k < ids.size(); ++k)
    if (ids[k] >= 0 && static_cast<int>(k) != m.top) casadi_gb300_tape_free(ids[k]);
  return id;
}

int casadi_gb300_tape_free(int id) {
  std::lock_guard<std::mutex> lk(g_mtx);
  if (id < 0 || id >= static_cast<int>(g_tapes.size()) || !g_tapes[id])
    return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  g_tapes[id].reset();
  return 0;
}

int casadi_gb300_tape_info(int id, int* n_instr, int* n_in, int* n_out, int* sz_w,
                           int* n_partials) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (n_instr) *n_instr = t->n_instr;
  if (n_in) *n_in = t->n_in;
  if (n_out) *n_out = t->n_out;
  if (sz_w) *sz_w = t->sz_w;
  if (n_partials) *n_partials = t->n_partials;
  return 0;
}

int casadi_gb300_scratch_size(int id, int64_t n, size_t* bytes) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (!bytes || n < 0) return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  *bytes = static_cast<size_t>(8) * t->n_partials * static_cast<size_t>(((n + 31) / 32) * 32) +
           kQueueSlack;
  return 0;
}

int casadi_gb300_scratch_min(int id, size_t* bytes) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (!bytes) return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  *bytes = static_cast<size_t>(8) * 32 * t->n_partials + kQueueSlack;
  return 0;
}

int casadi_gb300_eval(int id, int64_t n, int64_t ld, const double* const* arg,
                      double* const* res, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (n == 0) return 0;
  SweepArgs a = base_args(*t, n, 0);
  fill_io(a.in, t->n_in, vptrs(arg), t->nnz_in, ld, false);
  fill_io(a.out, t->n_out, vptrs(res), t->nnz_out, ld, false);
  return primal_launch(*t, a, n, PK_EVAL, static_cast<cudaStream_t>(stream));
}

int casadi_gb300_forward(int id, int64_t n, int64_t ld, int nfwd, const double* const* arg,
                         double* const* res, const double* const* fseed, double* const* fsens,
                         void* scratch, size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (nfwd < 0 || nfwd > 65535) return fail(CASADI_GB300_ERR_ARG, "bad direction count %d", nfwd);
  IoDesc in[kMaxIo], out[kMaxIo], seed[kMaxIo], sens[kMaxIo];
  fill_io(in, t->n_in, vptrs(arg), t->nnz_in, ld, false);
  fill_io(out, t->n_out, vptrs(res), t->nnz_out, ld, false);
  fill_io(seed, t->n_in, vptrs(fseed), t->nnz_in, ld, true);
  fill_io(sens, t->n_out, vptrs(fsens), t->nnz_out, ld, true);
  return run_ad(*t, n, in, out, seed, sens, nfwd, false, false, scratch, scratch_bytes,
                static_cast<cudaStream_t>(stream));
}

int casadi_gb300_reverse(int id, int64_t n, int64_t ld, int nadj, const double* const* arg,
                         double* const* res, const double* const* aseed, double* const* asens,
                         void* scratch, size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (nadj < 0 || nadj > 65535) return fail(CASADI_GB300_ERR_ARG, "bad direction count %d", nadj);
  IoDesc in[kMaxIo], out[kMaxIo], seed[kMaxIo], sens[kMaxIo];
  fill_io(in, t->n_in, vptrs(arg), t->nnz_in, ld, false);
  fill_io(out, t->n_out, vptrs(res), t->nnz_out, ld, false);
  fill_io(seed, t->n_out, vptrs(aseed), t->nnz_out, ld, true);
  fill_io(sens, t->n_in, vptrs(asens), t->nnz_in, ld, true);
  return run_ad(*t, n, in, out, seed, sens, nadj, true, false, scratch, scratch_bytes,
                static_cast<cudaStream_t>(stream));
}

int casadi_gb300_jacobian(int id, int64_t n, int64_t ld, const double* const* arg,
                          double* const* res, double* const* jac, void* scratch,
                          size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  int nz = 0;
  for (int v : t->nnz_in) nz += v;
  if (nz == 0) return fail(CASADI_GB300_ERR_ARG, "tape has no input nonzeros");
  IoDesc in[kMaxIo], out[kMaxIo], seed[kMaxIo], sens[kMaxIo];
  fill_io(in, t->n_in, vptrs(arg), t->nnz_in, ld, false);
  fill_io(out, t->n_out, vptrs(res), t->nnz_out, ld, false);
  fill_io(seed, t->n_in, nullptr, t->nnz_in, ld, true);
  fill_io(sens, t->n_out, vptrs(jac), t->nnz_out, ld, true);
  return run_ad(*t, n, in, out, seed, sens, nz, false, true, scratch, scratch_bytes,
                static_cast<cudaStream_t>(stream));
}

int casadi_gb300_jacobian_colored(int id, int64_t n, int64_t ld, int n_colors,
                                  const int* color, const double* const* arg,
                                  double* const* res, double* const* comp, void* scratch,
                                  size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  int nz = 0;
  for (int v : t->nnz_in) nz += v;
  if (!color || n_colors < 1 || n_colors > nz)
    return fail(CASADI_GB300_ERR_ARG, "bad colouring (%d colours for %d input nonzeros)",
                n_colors, nz);
  std::vector<int> dirmap(color, color + nz);
  for (int v : dirmap)
    if (v < -1 || v >= n_colors) return fail(CASADI_GB300_ERR_ARG, "colour %d out of range", v);
  IoDesc in[kMaxIo], out[kMaxIo], seed[kMaxIo], sens[kMaxIo];
  fill_io(in, t->n_in, vptrs(arg), t->nnz_in, ld, false);
  fill_io(out, t->n_out, vptrs(res), t->nnz_out, ld, false);
  fill_io(seed, t->n_in, nullptr, t->nnz_in, ld, true);
  fill_io(sens, t->n_out, vptrs(comp), t->nnz_out, ld, true);
  DerivReq rq;
  rq.ndir = n_colors;
  rq.identity = true;
  rq.dirmap = &dirmap;
  rq.seed = seed;
  rq.sens = sens;
  return run_ad_multi(*t, n, in, out, &rq, 1, scratch, scratch_bytes,
                      static_cast<cudaStream_t>(stream));
}

int casadi_gb300_gather(int64_t n, int64_t ld, int count, const int64_t* src_row,
                        const double* src, double* dst, void* stream) {
  if (n < 0 || ld < n || count < 0 || (count > 0 && (!src_row || !src || !dst)))
    return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  if (n == 0 || count == 0) return 0;
  cudaError_t e = launch_gather(n, ld, count, reinterpret_cast<const long long*>(src_row), src,
                                dst, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "gather launch");
  return 0;
}

int casadi_gb300_jacobian_reverse(int id, int64_t n, int64_t ld, const double* const* arg,
                                  double* const* res, double* const* jac, int nadj,
                                  const double* const* aseed, double* const* asens,
                                  void* scratch, size_t scratch_bytes, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (nadj < 0) return fail(CASADI_GB300_ERR_ARG, "negative direction count");
  int nz = 0;
  for (int v : t->nnz_in) nz += v;
  if (nz == 0) return fail(CASADI_GB300_ERR_ARG, "tape has no input nonzeros");
  IoDesc in[kMaxIo], out[kMaxIo], fseed[kMaxIo], fsens[kMaxIo], aseedd[kMaxIo], asensd[kMaxIo];
  fill_io(in, t->n_in, vptrs(arg), t->nnz_in, ld, false);
  fill_io(out, t->n_out, vptrs(res), t->nnz_out, ld, false);
  fill_io(fseed, t->n_in, nullptr, t->nnz_in, ld, true);
  fill_io(fsens, t->n_out, vptrs(jac), t->nnz_out, ld, true);
  fill_io(aseedd, t->n_out, vptrs(aseed), t->nnz_out, ld, true);
  fill_io(asensd, t->n_in, vptrs(asens), t->nnz_in, ld, true);
  DerivReq rq[2];
  rq[0].ndir = nz;
  rq[0].identity = true;
  rq[0].seed = fseed;
  rq[0].sens = fsens;
  rq[1].ndir = nadj;
  rq[1].adjoint = true;
  rq[1].seed = aseedd;
  rq[1].sens = asensd;
  return run_ad_multi(*t, n, in, out, rq, 2, scratch, scratch_bytes,
                      static_cast<cudaStream_t>(stream));
}

int casadi_gb300_profile(int enable) {
  std::lock_guard<std::mutex> lk(g_prof_mtx);
  g_prof = enable != 0;
  return 0;
}

int casadi_gb300_autotune(int enable) {
  std::lock_guard<std::mutex> lk(g_mtx);
  g_autotune = enable != 0;
  return 0;
}

int casadi_gb300_tuned_variant(int id, int kind, int* variant) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (kind < 0 || kind > 2 || !variant) return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  *variant = t->tuned[kind][1] >= 0 ? t->tuned[kind][1] : t->tuned[kind][0];
  return 0;
}

int casadi_gb300_set_residence(int id, int mode) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (mode < 0 || mode > 3) return fail(CASADI_GB300_ERR_ARG, "residence must be 0, 1, 2 or 3");
  t->residence = mode;
  reset_primal_tuning(*t);
  return 0;
}

int casadi_gb300_set_variant(int id, int kind, int variant) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (kind < 0 || kind > 2 || variant < -1 || variant > (kind == 2 ? AV_COUNT : TV_COUNT + 1))
    return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  t->tuned[kind][0] = t->tuned[kind][1] = variant;
  return 0;
}

int casadi_gb300_profile_collect(double* ms, int* launches, int count) {
  if (!ms || !launches || count <= 0) return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  std::lock_guard<std::mutex> lk(g_prof_mtx);
  for (int k = 0; k < count; ++k) {
    ms[k] = 0;
    launches[k] = 0;
  }
  int rc = 0;
  for (ProfEntry& p : g_prof_live) {
    cudaError_t e = cudaEventSynchronize(p.stop);
    float t = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, p.start, p.stop);
    if (e != cudaSuccess) rc = cuda_fail(e, "profile events");
    if (p.family < count) {
      ms[p.family] += t;
      launches[p.family] += 1;
    }
    g_prof_pool.push_back(p.start);
    g_prof_pool.push_back(p.stop);
  }
  g_prof_live.clear();
  return rc;
}

int casadi_gb300_sp_forward(int id, int64_t n, int64_t ld, const uint64_t* const* arg,
                            uint64_t* const* res, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (n == 0) return 0;
  SweepArgs a = base_args(*t, n, 0);
  fill_io(a.in, t->n_in, vptrs(arg), t->nnz_in, ld, false);
  fill_io(a.out, t->n_out, vptrs(res), t->nnz_out, ld, false);
  return primal_launch(*t, a, n, PK_SP_FORWARD, static_cast<cudaStream_t>(stream));
}

int casadi_gb300_eval_activity(int id, int64_t n, int64_t ld, const uint64_t* const* arg,
                               uint64_t* const* res, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (n == 0) return 0;
  SweepArgs a = base_args(*t, n, 0);
  fill_io(a.in, t->n_in, vptrs(arg), t->nnz_in, ld, false);
  fill_io(a.out, t->n_out, vptrs(res), t->nnz_out, ld, false);
  return primal_launch(*t, a, n, PK_ACTIVITY, static_cast<cudaStream_t>(stream));
}

int casadi_gb300_sp_reverse(int id, int64_t n, int64_t ld, uint64_t* const* arg,
                            uint64_t* const* res, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  if (int rc = check_device(*t)) return rc;
  if (int rc = check_n(n, ld)) return rc;
  if (n == 0) return 0;
  SweepArgs a = base_args(*t, n, 0);
  fill_io(a.in, t->n_in, vptrs(arg), t->nnz_in, ld, false);
  fill_io(a.out, t->n_out, vptrs(res), t->nnz_out, ld, false);
  return primal_launch(*t, a, n, PK_SP_REVERSE, static_cast<cudaStream_t>(stream));
}

int casadi_gb300_sync(int id, void* stream) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  int flags = 0;
  if ((e = cudaMemcpy(&flags, t->d_err, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda_fail(e, "read error word");
  if (flags) {
    cudaMemset(t->d_err, 0, sizeof(int));
    return fail(CASADI_GB300_ERR_DEVICE, "device sweep reported error flags 0x%x%s", flags,
                (flags & kErrWaitTimeout) ? " (instruction staging wait timed out)" : "");
  }
  return 0;
}

int casadi_gb300_checkout(void) {
  auto m = std::make_unique<Mem>();
  cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
  std::lock_guard<std::mutex> lk(g_mtx);
  for (size_t k = 0; k < g_mems.size(); ++k) {
    if (!g_mems[k]) {
      g_mems[k] = std::move(m);
      return static_cast<int>(k);
    }
  }
  g_mems.push_back(std::move(m));
  return static_cast<int>(g_mems.size()) - 1;
}

int casadi_gb300_release(int mem) {
  std::lock_guard<std::mutex> lk(g_mtx);
  if (mem < 0 || mem >= static_cast<int>(g_mems.size()) || !g_mems[mem])
    return fail(CASADI_GB300_ERR_ID, "no memory object %d", mem);
  g_mems[mem].reset();
  return 0;
}

static Mem* get_mem(int mem) {
  std::lock_guard<std::mutex> lk(g_mtx);
  if (mem < 0 || mem >= static_cast<int>(g_mems.size()) || !g_mems[mem]) return nullptr;
  return g_mems[mem].get();
}

// Instance-major device blocks for the host-buffer Map path: block j holds
// n * per_inst[j] doubles; descriptor strides address (dir, nz, inst).
// dir_major: the host blocks hold direction d of instance i at (d*n + i)*nnz (the order of
// CasADi's Map::get_forward/get_reverse seeds and sensitivities, casadi/core/map.cpp:233-264);
// otherwise at (i*ndir + d)*nnz (the inner f.forward(ndir).map(n) order). The staging buffer
// takes the host block's order, so copies stay contiguous.
static int stage_blocks(Mem& m, size_t first_buf, int count, const std::vector<int>& nnz,
                        int ndir, long long n, const double* const* host, bool upload,
                        IoDesc* desc, cudaStream_t s, bool dir_major = false) {
  for (int j = 0; j < count; ++j) {
    desc[j].ptr = nullptr;
    if (!host || !host[j] || nnz[j] == 0) continue;
    const size_t bytes = sizeof(double) * static_cast<size_t>(n) * nnz[j] * std::max(1, ndir);
    cudaError_t e = cudaSuccess;
    void* d = m.buf(first_buf + j, bytes, &e);
    if (!d) return cuda_fail(e, "cudaMalloc(staging)");
    if (upload && (e = cudaMemcpyAsync(d, host[j], bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_fail(e, "cudaMemcpyAsync(H2D)");
    desc[j].ptr = d;
    desc[j].nz_stride = 1;
    if (dir_major) {
      desc[j].dir_stride = static_cast<long long>(nnz[j]) * n;
      desc[j].inst_stride = nnz[j];
    } else {
      desc[j].dir_stride = nnz[j];
      desc[j].inst_stride = static_cast<long long>(nnz[j]) * std::max(1, ndir);
    }
  }
  return 0;
}

extern "C++" {
namespace {
// Host blocks of a host-buffer call: each device descriptor (staging buffer in the host
// block's order, desc->inst_stride doubles per instance and direction block) with the host
// array it is uploaded from or downloaded to. dir_blocks > 1: direction-major blocks, one
// contiguous piece of an instance range per direction (desc->dir_stride apart).
struct HostBlock {
  const IoDesc* desc;
  const double* up;  // upload source (inputs, seeds) or null
  double* down;      // download target (outputs, sensitivities) or null
  int dir_blocks;
  bool early;        // downloaded once the chunk's early event has passed
};

void collect_blocks(std::vector<HostBlock>& v, const IoDesc* desc, int count, const double* const* up,
                double* const* down, int dir_blocks = 1, bool early = false) {
  for (int j = 0; j < count; ++j)
    if (desc[j].ptr)
      v.push_back({&desc[j], up ? up[j] : nullptr, down ? down[j] : nullptr, dir_blocks, early});
}

// Descriptors of instances [i0, ...) of instance-major staging descriptors.
void shift_io(const IoDesc* src, int count, long long i0, IoDesc* dst) {
  for (int j = 0; j < count; ++j) {
    dst[j] = src[j];
    if (src[j].ptr)
      dst[j].ptr = static_cast<double*>(src[j].ptr) + i0 * src[j].inst_stride;
  }
}

// Host-buffer call over n instances in up to kMaxChunks chunks: the upload of chunk c+1 (copy
// stream s_in) and the download of chunk c-1 (s_out) overlap the sweeps of chunk c (the
// memory object's stream). `compute(i0, count)` enqueues one chunk's sweeps on m.stream.
template <class F>
int run_pipelined(Mem& m, long long n, const std::vector<HostBlock>& blocks, F compute,
                  int max_chunks = kMaxChunks) {
  cudaError_t e = m.pipe();
  if (e != cudaSuccess) return cuda_fail(e, "copy streams");
  // chunks of at least 131072 instances: smaller launches lose more sweep efficiency than the
  // overlap gains (rollout Jacobian + adjoint, 262144 instances, without early downloads:
  // 1 chunk 34.9 ms, 2 chunks 34.8, 3 chunks 37.0, 4 chunks 39.0)
  int chunks = static_cast<int>(std::max(1ll, std::min<long long>(max_chunks, n / 131072)));
  const long long per = ((n + chunks - 1) / chunks + 31) / 32 * 32;
  chunks = static_cast<int>((n + per - 1) / per);
  bool any_early = false;
  for (const auto& b : blocks) any_early = any_early || (b.down && b.early);
  auto download = [&](long long i0, long long cnt, bool early) -> cudaError_t {
    for (const auto& b : blocks) {
      if (!b.down || b.early != early) continue;
      const size_t bytes = sizeof(double) * static_cast<size_t>(b.desc->inst_stride);
      for (int d = 0; d < b.dir_blocks; ++d) {
        const long long off = d * (b.dir_blocks > 1 ? b.desc->dir_stride : 0) +
                              i0 * b.desc->inst_stride;
        cudaError_t r = cudaMemcpyAsync(b.down + off, static_cast<double*>(b.desc->ptr) + off,
                                        bytes * cnt, cudaMemcpyDeviceToHost, m.s_out);
        if (r != cudaSuccess) return r;
      }
    }
    return cudaSuccess;
  };
  for (int c = 0; c < chunks; ++c) {
    const long long i0 = c * per, cnt = std::min(per, n - i0);
    for (const auto& b : blocks) {
      if (!b.up) continue;
      const size_t bytes = sizeof(double) * static_cast<size_t>(b.desc->inst_stride);
      for (int d = 0; d < b.dir_blocks; ++d) {
        const long long off = d * (b.dir_blocks > 1 ? b.desc->dir_stride : 0) +
                              i0 * b.desc->inst_stride;
        if ((e = cudaMemcpyAsync(static_cast<double*>(b.desc->ptr) + off, b.up + off,
                                 bytes * cnt, cudaMemcpyHostToDevice, m.s_in)) != cudaSuccess)
          return cuda_fail(e, "cudaMemcpyAsync(H2D)");
      }
    }
    if ((e = cudaEventRecord(m.ev_in[c], m.s_in)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(m.stream, m.ev_in[c], 0)) != cudaSuccess)
      return cuda_fail(e, "chunk ordering");
    // compute records m.ev_early[c] on m.stream when the early outputs are final
    if (int rc = compute(i0, cnt, m.ev_early[c])) return rc;
    if (any_early) {
      if ((e = cudaStreamWaitEvent(m.s_out, m.ev_early[c], 0)) != cudaSuccess)
        return cuda_fail(e, "chunk ordering");
      if ((e = download(i0, cnt, true)) != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(D2H)");
    }
    if ((e = cudaEventRecord(m.ev_done[c], m.stream)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(m.s_out, m.ev_done[c], 0)) != cudaSuccess)
      return cuda_fail(e, "chunk ordering");
    if ((e = download(i0, cnt, false)) != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(D2H)");
  }
  if ((e = cudaEventRecord(m.ev_out, m.s_out)) != cudaSuccess ||
      (e = cudaStreamWaitEvent(m.stream, m.ev_out, 0)) != cudaSuccess)
    return cuda_fail(e, "chunk ordering");
  return 0;
}
}  // namespace
}  // extern "C++"

// Partials scratch of a memory object for the host-buffer AD paths; waves keep it <= 8 GiB.
static int map_scratch(const Tape& t, Mem& m, long long n, void** scratch, size_t* bytes) {
  *scratch = nullptr;
  *bytes = 0;
  if (t.n_partials == 0) return 0;
  size_t need = 8ull * t.n_partials * static_cast<size_t>(((n + 31) / 32) * 32);
  const size_t kMaxScratch = 8ull << 30;
  need = std::min(need, std::max<size_t>(kMaxScratch, 8ull * 32 * t.n_partials)) + kQueueSlack;
  cudaError_t e = cudaSuccess;
  *scratch = m.buf(4 * kMaxIo, need, &e);
  if (!*scratch) return cuda_fail(e, "cudaMalloc(scratch)");
  *bytes = need;
  return 0;
}

int casadi_gb300_map_eval(int id, int mem, int64_t n, const double* const* arg,
                          double* const* res) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  Mem* m = get_mem(mem);
  if (!m) return fail(CASADI_GB300_ERR_ID, "no memory object %d", mem);
  if (int rc = check_device(*t)) return rc;
  if (n < 0) return fail(CASADI_GB300_ERR_ARG, "negative instance count");
  if (n == 0) return 0;
  cudaStream_t s = m->stream;
  IoDesc in[kMaxIo], out[kMaxIo];
  if (int rc = stage_blocks(*m, 0, t->n_in, t->nnz_in, 1, n, arg, false, in, s)) return rc;
  if (int rc = stage_blocks(*m, kMaxIo, t->n_out, t->nnz_out, 1, n,
                            reinterpret_cast<const double* const*>(res), false, out, s))
    return rc;
  std::vector<HostBlock> blocks;
  collect_blocks(blocks, in, t->n_in, arg, nullptr);
  collect_blocks(blocks, out, t->n_out, nullptr, res);
  if (int rc = run_pipelined(*m, n, blocks, [&](long long i0, long long cnt, cudaEvent_t) {
        SweepArgs a = base_args(*t, cnt, 0);
        shift_io(in, t->n_in, i0, a.in);
        shift_io(out, t->n_out, i0, a.out);
        return primal_launch(*t, a, cnt, PK_EVAL, s);
      }))
    return rc;
  return casadi_gb300_sync(id, s);
}

// bvec_t blocks travel through the same 8-byte staging as doubles (bit copies).
static int map_sp(int id, int mem, int64_t n, uint64_t* const* arg, uint64_t* const* res,
                  bool reverse) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  Mem* m = get_mem(mem);
  if (!m) return fail(CASADI_GB300_ERR_ID, "no memory object %d", mem);
  if (int rc = check_device(*t)) return rc;
  if (n < 0) return fail(CASADI_GB300_ERR_ARG, "negative instance count");
  if (n == 0) return 0;
  cudaStream_t s = m->stream;
  const double* const* harg = reinterpret_cast<const double* const*>(arg);
  const double* const* hres = reinterpret_cast<const double* const*>(res);
  IoDesc in[kMaxIo], out[kMaxIo];
  if (int rc = stage_blocks(*m, 0, t->n_in, t->nnz_in, 1, n, harg, false, in, s)) return rc;
  if (int rc = stage_blocks(*m, kMaxIo, t->n_out, t->nnz_out, 1, n, hres, false, out, s))
    return rc;
  std::vector<HostBlock> blocks;
  // forward: arg in, res out; reverse (in place): res seeds in and cleared, arg |= out
  collect_blocks(blocks, in, t->n_in, harg, reverse ? reinterpret_cast<double* const*>(arg)
                                                    : nullptr);
  collect_blocks(blocks, out, t->n_out, reverse ? hres : nullptr,
                 reinterpret_cast<double* const*>(res));
  if (int rc = run_pipelined(*m, n, blocks, [&](long long i0, long long cnt, cudaEvent_t) {
        SweepArgs a = base_args(*t, cnt, 0);
        shift_io(in, t->n_in, i0, a.in);
        shift_io(out, t->n_out, i0, a.out);
        return primal_launch(*t, a, cnt, reverse ? PK_SP_REVERSE : PK_SP_FORWARD, s);
      }))
    return rc;
  return casadi_gb300_sync(id, s);
}

int casadi_gb300_map_sp_forward(int id, int mem, int64_t n, const uint64_t* const* arg,
                                uint64_t* const* res) {
  return map_sp(id, mem, n, const_cast<uint64_t* const*>(arg), res, false);
}

int casadi_gb300_map_sp_reverse(int id, int mem, int64_t n, uint64_t* const* arg,
                                uint64_t* const* res) {
  return map_sp(id, mem, n, arg, res, true);
}

int casadi_gb300_map_jacobian(int id, int mem, int64_t n, const double* const* arg,
                              double* const* res, double* const* jac) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  Mem* m = get_mem(mem);
  if (!m) return fail(CASADI_GB300_ERR_ID, "no memory object %d", mem);
  if (int rc = check_device(*t)) return rc;
  if (n < 0) return fail(CASADI_GB300_ERR_ARG, "negative instance count");
  if (n == 0) return 0;
  int nz = 0;
  for (int v : t->nnz_in) nz += v;
  if (nz == 0) return fail(CASADI_GB300_ERR_ARG, "tape has no input nonzeros");
  cudaStream_t s = m->stream;
  IoDesc in[kMaxIo], out[kMaxIo], sens[kMaxIo];
  if (int rc = stage_blocks(*m, 0, t->n_in, t->nnz_in, 1, n, arg, false, in, s)) return rc;
  if (int rc = stage_blocks(*m, kMaxIo, t->n_out, t->nnz_out, 1, n,
                            reinterpret_cast<const double* const*>(res), false, out, s))
    return rc;
  if (int rc = stage_blocks(*m, 3 * kMaxIo, t->n_out, t->nnz_out, nz, n,
                            reinterpret_cast<const double* const*>(jac), false, sens, s))
    return rc;
  void* scratch = nullptr;
  size_t bytes = 0;
  if (int rc = map_scratch(*t, *m, n, &scratch, &bytes)) return rc;
  IoDesc seed[kMaxIo];
  std::memset(seed, 0, sizeof(seed));
  std::vector<HostBlock> blocks;
  collect_blocks(blocks, in, t->n_in, arg, nullptr);
  collect_blocks(blocks, out, t->n_out, nullptr, res);
  collect_blocks(blocks, sens, t->n_out, nullptr, jac);
  if (int rc = run_pipelined(*m, n, blocks, [&](long long i0, long long cnt, cudaEvent_t) {
        IoDesc in_c[kMaxIo], out_c[kMaxIo], sens_c[kMaxIo];
        shift_io(in, t->n_in, i0, in_c);
        shift_io(out, t->n_out, i0, out_c);
        shift_io(sens, t->n_out, i0, sens_c);
        return run_ad(*t, cnt, in_c, out_c, seed, sens_c, nz, false, true, scratch, bytes, s);
      }))
    return rc;
  return casadi_gb300_sync(id, s);
}

static int map_forward_impl(int id, int mem, int64_t n, int nfwd, const double* const* arg,
                            double* const* res, const double* const* fseed,
                            double* const* fsens, bool outer) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  Mem* m = get_mem(mem);
  if (!m) return fail(CASADI_GB300_ERR_ID, "no memory object %d", mem);
  if (int rc = check_device(*t)) return rc;
  if (n < 0 || nfwd < 1 || nfwd > 65535) return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  if (n == 0) return 0;
  cudaStream_t s = m->stream;
  IoDesc in[kMaxIo], out[kMaxIo], seed[kMaxIo], sens[kMaxIo];
  if (int rc = stage_blocks(*m, 0, t->n_in, t->nnz_in, 1, n, arg, false, in, s)) return rc;
  if (int rc = stage_blocks(*m, kMaxIo, t->n_out, t->nnz_out, 1, n,
                            reinterpret_cast<const double* const*>(res), false, out, s))
    return rc;
  if (int rc = stage_blocks(*m, 2 * kMaxIo, t->n_in, t->nnz_in, nfwd, n, fseed, false, seed, s,
                            outer))
    return rc;
  if (int rc = stage_blocks(*m, 3 * kMaxIo, t->n_out, t->nnz_out, nfwd, n,
                            reinterpret_cast<const double* const*>(fsens), false, sens, s,
                            outer))
    return rc;
  void* scratch = nullptr;
  size_t bytes = 0;
  if (int rc = map_scratch(*t, *m, n, &scratch, &bytes)) return rc;
  std::vector<HostBlock> blocks;
  collect_blocks(blocks, in, t->n_in, arg, nullptr);
  collect_blocks(blocks, seed, t->n_in, fseed, nullptr, outer ? nfwd : 1);
  collect_blocks(blocks, out, t->n_out, nullptr, res);
  collect_blocks(blocks, sens, t->n_out, nullptr, fsens, outer ? nfwd : 1);
  if (int rc = run_pipelined(*m, n, blocks, [&](long long i0, long long cnt, cudaEvent_t) {
        IoDesc in_c[kMaxIo], out_c[kMaxIo], seed_c[kMaxIo], sens_c[kMaxIo];
        shift_io(in, t->n_in, i0, in_c);
        shift_io(out, t->n_out, i0, out_c);
        shift_io(seed, t->n_in, i0, seed_c);
        shift_io(sens, t->n_out, i0, sens_c);
        return run_ad(*t, cnt, in_c, out_c, seed_c, sens_c, nfwd, false, false, scratch, bytes,
                      s);
      }))
    return rc;
  return casadi_gb300_sync(id, s);
}

static int map_reverse_impl(int id, int mem, int64_t n, int nadj, const double* const* arg,
                            double* const* res, const double* const* aseed,
                            double* const* asens, bool outer) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  Mem* m = get_mem(mem);
  if (!m) return fail(CASADI_GB300_ERR_ID, "no memory object %d", mem);
  if (int rc = check_device(*t)) return rc;
  if (n < 0 || nadj < 1 || nadj > 65535) return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  if (n == 0) return 0;
  cudaStream_t s = m->stream;
  IoDesc in[kMaxIo], out[kMaxIo], seed[kMaxIo], sens[kMaxIo];
  if (int rc = stage_blocks(*m, 0, t->n_in, t->nnz_in, 1, n, arg, false, in, s)) return rc;
  if (int rc = stage_blocks(*m, kMaxIo, t->n_out, t->nnz_out, 1, n,
                            reinterpret_cast<const double* const*>(res), false, out, s))
    return rc;
  if (int rc = stage_blocks(*m, 2 * kMaxIo, t->n_out, t->nnz_out, nadj, n, aseed, false, seed, s,
                            outer))
    return rc;
  if (int rc = stage_blocks(*m, 3 * kMaxIo, t->n_in, t->nnz_in, nadj, n,
                            reinterpret_cast<const double* const*>(asens), false, sens, s,
                            outer))
    return rc;
  void* scratch = nullptr;
  size_t bytes = 0;
  if (int rc = map_scratch(*t, *m, n, &scratch, &bytes)) return rc;
  std::vector<HostBlock> blocks;
  collect_blocks(blocks, in, t->n_in, arg, nullptr);
  collect_blocks(blocks, seed, t->n_out, aseed, nullptr, outer ? nadj : 1);
  collect_blocks(blocks, out, t->n_out, nullptr, res);
  collect_blocks(blocks, sens, t->n_in, nullptr, asens, outer ? nadj : 1);
  if (int rc = run_pipelined(*m, n, blocks, [&](long long i0, long long cnt, cudaEvent_t) {
        IoDesc in_c[kMaxIo], out_c[kMaxIo], seed_c[kMaxIo], sens_c[kMaxIo];
        shift_io(in, t->n_in, i0, in_c);
        shift_io(out, t->n_out, i0, out_c);
        shift_io(seed, t->n_out, i0, seed_c);
        shift_io(sens, t->n_in, i0, sens_c);
        return run_ad(*t, cnt, in_c, out_c, seed_c, sens_c, nadj, true, false, scratch, bytes, s);
      }))
    return rc;
  return casadi_gb300_sync(id, s);
}

int casadi_gb300_map_forward(int id, int mem, int64_t n, int nfwd, const double* const* arg,
                             double* const* res, const double* const* fseed,
                             double* const* fsens) {
  return map_forward_impl(id, mem, n, nfwd, arg, res, fseed, fsens, false);
}

int casadi_gb300_map_forward_outer(int id, int mem, int64_t n, int nfwd,
                                   const double* const* arg, double* const* res,
                                   const double* const* fseed, double* const* fsens) {
  return map_forward_impl(id, mem, n, nfwd, arg, res, fseed, fsens, true);
}

int casadi_gb300_map_reverse(int id, int mem, int64_t n, int nadj, const double* const* arg,
                             double* const* res, const double* const* aseed,
                             double* const* asens) {
  return map_reverse_impl(id, mem, n, nadj, arg, res, aseed, asens, false);
}

int casadi_gb300_map_reverse_outer(int id, int mem, int64_t n, int nadj,
                                   const double* const* arg, double* const* res,
                                   const double* const* aseed, double* const* asens) {
  return map_reverse_impl(id, mem, n, nadj, arg, res, aseed, asens, true);
}

int casadi_gb300_map_jacobian_reverse(int id, int mem, int64_t n, const double* const* arg,
                                      double* const* res, double* const* jac, int nadj,
                                      const double* const* aseed, double* const* asens) {
  Tape* t = get_tape(id);
  if (!t) return fail(CASADI_GB300_ERR_ID, "no tape with id %d", id);
  Mem* m = get_mem(mem);
  if (!m) return fail(CASADI_GB300_ERR_ID, "no memory object %d", mem);
  if (int rc = check_device(*t)) return rc;
  if (n < 0 || nadj < 0 || nadj > 65535) return fail(CASADI_GB300_ERR_ARG, "bad arguments");
  if (n == 0) return 0;
  int nz = 0;
  for (int v : t->nnz_in) nz += v;
  if (nz == 0) return fail(CASADI_GB300_ERR_ARG, "tape has no input nonzeros");
  cudaStream_t s = m->stream;
  IoDesc in[kMaxIo], out[kMaxIo], fsens[kMaxIo], aseedd[kMaxIo], asensd[kMaxIo], fseed[kMaxIo];
  std::memset(fseed, 0, sizeof(fseed));
  // staging buffers only: the pipelined copies below move the data chunk by chunk
  if (int rc = stage_blocks(*m, 0, t->n_in, t->nnz_in, 1, n, arg, false, in, s)) return rc;
  if (int rc = stage_blocks(*m, kMaxIo, t->n_out, t->nnz_out, 1, n,
                            reinterpret_cast<const double* const*>(res), false, out, s))
    return rc;
  if (int rc = stage_blocks(*m, 2 * kMaxIo, t->n_out, t->nnz_out, nadj, n, aseed, false, aseedd,
                            s))
    return rc;
  if (int rc = stage_blocks(*m, 3 * kMaxIo, t->n_out, t->nnz_out, nz, n,
                            reinterpret_cast<const double* const*>(jac), false, fsens, s))
    return rc;
  if (int rc = stage_blocks(*m, 5 * kMaxIo, t->n_in, t->nnz_in, nadj, n,
                            reinterpret_cast<const double* const*>(asens), false, asensd, s))
    return rc;
  void* scratch = nullptr;
  size_t bytes = 0;
  if (int rc = map_scratch(*t, *m, n, &scratch, &bytes)) return rc;
  std::vector<HostBlock> blocks;
  collect_blocks(blocks, in, t->n_in, arg, nullptr);
  collect_blocks(blocks, aseedd, t->n_out, aseed, nullptr);
  collect_blocks(blocks, out, t->n_out, nullptr, res);
  // the Jacobian is final after the tangent sweep: its download overlaps the adjoint sweep
  collect_blocks(blocks, fsens, t->n_out, nullptr, jac, 1, true);
  collect_blocks(blocks, asensd, t->n_in, nullptr, asens);
  // one chunk when the partials of all instances fit one wave: the Jacobian's download then
  // hides behind the adjoint sweep, and full-size sweeps run faster than two half-size ones
  const int max_chunks = wave_capacity(*t, n, bytes) >= n ? 1 : kMaxChunks;
  if (int rc = run_pipelined(*m, n, blocks, [&](long long i0, long long cnt, cudaEvent_t early) {
        IoDesc in_c[kMaxIo], out_c[kMaxIo], fsens_c[kMaxIo], aseed_c[kMaxIo], asens_c[kMaxIo];
        shift_io(in, t->n_in, i0, in_c);
        shift_io(out, t->n_out, i0, out_c);
        shift_io(fsens, t->n_out, i0, fsens_c);
        shift_io(aseedd, t->n_out, i0, aseed_c);
        shift_io(asensd, t->n_in, i0, asens_c);
        DerivReq rq[2];
        rq[0].ndir = nz;
        rq[0].identity = true;
        rq[0].seed = fseed;
        rq[0].sens = fsens_c;
        rq[1].ndir = nadj;
        rq[1].adjoint = true;
        rq[1].seed = aseed_c;
        rq[1].sens = asens_c;
        // record + tangent, the early event, then the adjoint on the recorded partials (one
        // wave); with waves both requests run wave by wave and the event follows them
        if (wave_capacity(*t, cnt, bytes) < cnt) {
          if (int rc = run_ad_multi(*t, cnt, in_c, out_c, rq, 2, scratch, bytes, s)) return rc;
          cudaError_t e = cudaEventRecord(early, s);
          return e == cudaSuccess ? 0 : cuda_fail(e, "early event");
        }
        if (int rc = run_ad_multi(*t, cnt, in_c, out_c, rq, 1, scratch, bytes, s)) return rc;
        cudaError_t e = cudaEventRecord(early, s);
        if (e != cudaSuccess) return cuda_fail(e, "early event");
        return run_ad_multi(*t, cnt, in_c, out_c, rq + 1, 1, scratch, bytes, s, true);
      }, max_chunks))
    return rc;
  return casadi_gb300_sync(id, s);
}

}  // extern "C"

// The remaining entry points live in parts of this translation unit (they share the
// internal helpers above).
#include "abi_noalloc.cuh"
#include "abi_batch.cuh"
#include "abi_maps.cuh"
#include "abi_probe.cuh"
#include "abi_segments.cuh"
