// Launch interface between the C-ABI layer (abi.cu) and the tape-sweep kernels (sweeps.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "device_ops.cuh"

namespace cgb {

constexpr int kChunk = 256;      // instructions per staged chunk (2 KiB), value sweeps
constexpr int kPofsGran = 16;    // granularity of the per-chunk partial offsets
constexpr int kLeanPB = 63;      // partials per staged chunk block (plan-free adjoint)
// entries per software-pipelined group of the batch kernel's tangent and adjoint walks: small
// groups keep the kernel's code (value walk and both keyed walks) small; the tangent walk
// of the coloured MPC items wants two entries of partial loads in flight
constexpr int kBatchTanGroup = 2;
constexpr int kBatchAdjGroup = 1;
constexpr unsigned kMaxPartials = 1u << 21;  // recorded partials per instance the entries address

// Instruction kinds of the derivative sweeps (the windowed tangent sweep's entries carry them
// in bits 5-8 of their meta word; mixed tangent entries in bits 19-22 of x).
enum LeanKind : unsigned {
  LK_NOP = 0, LK_GEN, LK_ADD, LK_SUB, LK_NEG, LK_TWICE, LK_ASSIGN, LK_IFZ, LK_INPUT, LK_OUTPUT,
  LK_CONST, LK_MIXED
};
constexpr int kMaxIo = 64;       // inputs/outputs per tape handled by one launch

// ---------------------------------------------------------------------------------------------
// Keyed entry streams of the tangent and adjoint walks. An entry is {x, y, z, w}: x the slot
// the entry writes (tangent) or whose adjoint it reads (adjoint), y and z its operand slots,
// all as byte offsets into the warp's work vector (slot * 256); inputs and outputs put their
// I/O index and nonzero in the fields the walks name. w bits 0-5 are the entry's key, the
// walk's jump-table case: the arithmetic form, and for the adjoint which operand receives its
// first contribution. w bits 6-31 describe the recorded partials of the entry G positions
// later (G: entries per pipeline group of the walk that reads the stream), so a walk issues
// the loads of group g+1 while group g computes, with no decoding of g+1's entries first:
// bit 6 load P, bit 7 load Q, bit 8 Q is the partial after P's (otherwise at P's index),
// bits 9-31 P's partial index. A stream for group size G is a header group (no work; it carries
// the first group's partials), the body (an even number of groups, NOP-padded) and one
// trailing NOP group: the walks unroll two groups per iteration and read one group past the
// body. Key 0 is NOP in both walks.
// ---------------------------------------------------------------------------------------------
constexpr int kNumGroupSizes = 4;  // streams are laid out for G = 1, 2, 4, 8
__host__ __device__ constexpr int group_slot(int g) { return g >= 8 ? 3 : g >= 4 ? 2 : g >= 2 ? 1 : 0; }
__host__ __device__ constexpr unsigned ent_key(unsigned w) { return w & 63u; }
constexpr unsigned kPiP = 1u, kPiQ = 2u, kPiQNext = 4u;  // partial-info bits (w >> 6)
constexpr unsigned kPiShift = 6, kPiIndexShift = 9;
static_assert(kMaxPartials <= (1u << (32 - kPiIndexShift)), "partial indices fit the key word");

// Tangent forms: the tangent of one arithmetic entry from operand tangents a (y) and b (z) and
// the recorded partials p (d0) and q (d1).
enum TanForm : int {
  TF_PY,    // p*a                     (recorded d0)
  TF_QZ,    // q*b                     (recorded d1)
  TF_PYQZ,  // fma(p, a, q*b)
  TF_Y,     // a                       (d0 = 1: ADD, SUB, ASSIGN and GEN ops with a unit d0)
  TF_Z,     // b                       (ADD)
  TF_YQZ,   // a + q*b                 (d0 = 1, d1 recorded: FMOD, REMAINDER)
  TF_YZ,    // a + b                   (ADD)
  TF_NZ,    // -b                      (SUB)
  TF_YMZ,   // a - b                   (SUB)
  TF_NY,    // -a                      (NEG)
  TF_2Y,    // 2a                      (TWICE)
  TF_IFZ    // q == 0 ? 0 : b          (IF_ELSE_ZERO)
};
__host__ __device__ constexpr bool tf_uses_y(int f) {
  return f == TF_PY || f == TF_PYQZ || f == TF_Y || f == TF_YQZ || f == TF_YZ || f == TF_YMZ ||
         f == TF_NY || f == TF_2Y;
}
__host__ __device__ constexpr bool tf_uses_z(int f) {
  return f == TF_QZ || f == TF_PYQZ || f == TF_Z || f == TF_YQZ || f == TF_YZ || f == TF_NZ ||
         f == TF_YMZ || f == TF_IFZ;
}
__host__ __device__ constexpr bool tf_uses_p(int f) { return f == TF_PY || f == TF_PYQZ; }
__host__ __device__ constexpr bool tf_uses_q(int f) {
  return f == TF_QZ || f == TF_PYQZ || f == TF_YQZ || f == TF_IFZ;
}
// Arithmetic tangent keys: (key, form). Operands are read from the work vector: taking the
// previous result from a register instead (operand forwarding) doubles the cases, and the
// larger jump tables cost more in instruction fetch than the shared-memory loads they save.
#define CGB_TK_ARITH(X)                                                                      \
  X(TK_PY, TF_PY) X(TK_QZ, TF_QZ) X(TK_Y, TF_Y) X(TK_Z, TF_Z) X(TK_NZ, TF_NZ)                 \
  X(TK_NY, TF_NY) X(TK_2Y, TF_2Y) X(TK_IFZ, TF_IFZ) X(TK_PYQZ, TF_PYQZ) X(TK_YQZ, TF_YQZ)    \
  X(TK_YZ, TF_YZ) X(TK_YMZ, TF_YMZ)
#define CGB_KEY_ENUM(K, ...) K,
// TK_OUT0/TK_OUT: an output's sensitivity (x output, y slot, z nonzero) is 0 or the slot's
// tangent; TK_IN: an input's seed (x slot, y input, z nonzero); TK_MIXED + pm: a union-stream
// entry whose flags differ between the directions (x bits 19-22 kind, 24+2k flags of
// direction k), pm its recorded-partial mask.
enum TanKey : unsigned {
  TK_NOP = 0, TK_OUT0, TK_OUT, TK_IN, TK_MIXED, TK_MIXED_LAST = TK_MIXED + 3,
  CGB_TK_ARITH(CGB_KEY_ENUM) TK_COUNT
};
static_assert(TK_COUNT <= 64, "tangent keys fit 6 bits");

// Adjoint contributions of one entry to an operand slot w, from the entry's adjoint s and the
// operand's partial m: R recorded partial, U unit (ADD, SUB's first operand, ASSIGN and GEN ops
// with a unit d0), M minus one (NEG, SUB's second operand), T two (TWICE), I IF_ELSE_ZERO
// (s unless m is zero); F the slot's first contribution (assigned), A a later one (added).
enum AdjForm : int { CF_N, CF_RF, CF_RA, CF_UF, CF_UA, CF_MF, CF_MA, CF_TF, CF_TA, CF_IF, CF_IA };
__host__ __device__ constexpr bool cf_reads(int f) {
  return f == CF_RA || f == CF_UA || f == CF_MA || f == CF_TA || f == CF_IA;
}
// Arithmetic adjoint keys: (key, contribution to y, contribution to z).
#define CGB_AK_ARITH(X)                                                                      \
  X(AK_RF_N, CF_RF, CF_N) X(AK_RF_RF, CF_RF, CF_RF) X(AK_RF_RA, CF_RF, CF_RA)                \
  X(AK_RA_N, CF_RA, CF_N) X(AK_RA_RF, CF_RA, CF_RF) X(AK_RA_RA, CF_RA, CF_RA)                \
  X(AK_UF_N, CF_UF, CF_N) X(AK_UF_RF, CF_UF, CF_RF) X(AK_UF_RA, CF_UF, CF_RA)                \
  X(AK_UF_UF, CF_UF, CF_UF) X(AK_UF_UA, CF_UF, CF_UA) X(AK_UF_MF, CF_UF, CF_MF)              \
  X(AK_UF_MA, CF_UF, CF_MA)                                                                  \
  X(AK_UA_N, CF_UA, CF_N) X(AK_UA_RF, CF_UA, CF_RF) X(AK_UA_RA, CF_UA, CF_RA)                \
  X(AK_UA_UF, CF_UA, CF_UF) X(AK_UA_UA, CF_UA, CF_UA) X(AK_UA_MF, CF_UA, CF_MF)              \
  X(AK_UA_MA, CF_UA, CF_MA)                                                                  \
  X(AK_MF_N, CF_MF, CF_N) X(AK_MA_N, CF_MA, CF_N) X(AK_TF_N, CF_TF, CF_N)                    \
  X(AK_TA_N, CF_TA, CF_N)                                                                    \
  X(AK_N_RF, CF_N, CF_RF) X(AK_N_RA, CF_N, CF_RA) X(AK_N_IF, CF_N, CF_IF)                    \
  X(AK_N_IA, CF_N, CF_IA)
// AK_OUT_SET/AK_OUT_ADD: an output's seed (x output, y slot, z nonzero) assigned to or added
// into the slot's adjoint; AK_IN: an input's sensitivity (x slot, y input, z nonzero).
enum AdjKey : unsigned {
  AK_NOP = 0, AK_OUT_SET, AK_OUT_ADD, AK_IN, CGB_AK_ARITH(CGB_KEY_ENUM) AK_COUNT
};
static_assert(AK_COUNT <= 64, "adjoint keys fit 6 bits");
#undef CGB_KEY_ENUM

// One input/output block: element (direction d, nonzero k, instance i) lives at
// ptr[d*dir_stride + k*nz_stride + i*inst_stride].
struct IoDesc {
  void* ptr;
  long long nz_stride;
  long long inst_stride;
  long long dir_stride;
};

// What every sweep needs to know about the tape.
struct TapeView {
  const u64* code;          // kChunk-padded instruction stream (NOP padding)
  const int* pofs;          // pofs[k]: partials recorded before instruction k*kPofsGran
  const double* consts;     // constant pool
  const int2* absent_in;    // (input, nonzero) pairs the tape never reads
  int n_chunks;
  int n_absent_in;
  int sz_w;
  int n_partials;           // partials recorded per instance
  int* err;                 // device error word
  // level schedule of the cooperative value/record sweeps (null until first needed)
  const u64* lcode;         // instructions level by level, slots renamed
  const int* lbegin;        // level l is lcode[lbegin[l] .. lbegin[l+1])
  const int* lpidx;         // first recorded partial of each lcode instruction
  int n_levels;
  int lv_sz_w;              // work-vector length of the renamed slots
  // level schedule of the cooperative reverse sweep (users of each value in order)
  const u64* rcode;
  const int* rbegin;
  const int* rpidx;
  int n_rlevels;
  int rlv_sz_w;
};

struct SweepArgs {
  TapeView t;
  long long n;              // instances in this launch
  long long i_begin;        // offset of the first instance inside the IoDesc blocks
  int n_in, n_out;
  int ndir;                 // directions (forward/adjoint sweeps)
  int dir0;                 // first direction of this launch (identity seeds)
  int identity_seed;        // forward: seed of direction d is the d-th unit vector
  int block;                // threads per CTA
  double* partials;         // scratch, tile-major: partials[(tile*P + p)*32 + lane]
  const int* pofs;          // = t.pofs
  int chunk;                // instructions per staged chunk in the derivative sweeps
  int n_code;               // padded instruction count (multiple of kChunk)
  IoDesc in[kMaxIo];        // values in (eval / AD / sparsity)
  IoDesc out[kMaxIo];       // values out
  IoDesc seed[kMaxIo];      // forward: input seeds / adjoint: output seeds
  IoDesc sens[kMaxIo];      // forward: output sensitivities / adjoint: input sensitivities
  int in_off[kMaxIo];       // flat offset of each input's first nonzero (identity seeds)
  const int2* zero_in;              // adjoint: (input, nonzero) pairs with a zero sensitivity
  int n_zero;
  // keyed entry streams (host-compiled, one layout per group size; the launchers pick the
  // variant's into dstream/dchunks)
  const uint4* dstream;             // entries of all streams
  const int2* dchunks;              // per direction (tangent) or one (adjoint): first entry,
                                    // body entries
  const uint4* dstreams[kNumGroupSizes];
  const int2* dchunkss[kNumGroupSizes];
  // global work vector (null: shared memory): CTA b uses wglob + b*wglob_stride
  unsigned char* wglob;
  long long wglob_stride;
  const int* dirmap;                // cooperative tangent, identity seeds (see launch_tangent_coop)
  // tangent sweep work queue: items past the grid are claimed from *queue (zeroed before
  // each launch; null: static stride), direction groups of a tile in the order gorder
  // (longest entry stream first; null: natural order)
  unsigned long long* queue;
  const int* gorder;
  // windowed tangent sweep (launch_tangent_win): per (direction group, window) the window's
  // first partial row, partial rows, entry block start and length (uint4 units) in win_blocks;
  // win_dirs directions per CTA (one consumer warp each), win_stages ring stages of win_rows
  // partial rows + win_ents block uint4s each
  const uint4* win_blocks;
  const int4* win_meta;
  int win_n;
  int win_dirs;
  int win_stages;
  int win_rows;
  int win_ents;
};

// One item of a persistent batch: a tape over its own instance range.
struct BatchItem {
  TapeView t;
  int n_code;
  int ndir;                 // 0: value sweep only; >0: value + derivative directions
  int forward;              // directions are tangent (1, identity-seeded) or adjoint (0)
  long long n;              // instances
  const IoDesc* io;         // 4*kMaxIo descriptors: inputs, outputs, seeds, sensitivities
  const uint4* adj_stream;  // adjoint entry stream (ndir > 0, !forward)
  int adj_ngr;              // its groups of kBatchAdjGroup entries
  const int2* zero_in;      // inputs with a structurally zero adjoint
  int n_zero;
  const uint4* tan_stream;  // tangent entry streams (forward)
  const int2* tan_chunks;   // per direction: (first entry, entry count)
  // split items (two or more directions): one record unit per tile writes the tile's partials
  // here, (tile*P + p)*32 + lane, then sets ready[tile]; one unit per (tile, direction) waits
  // for the flag and walks its direction
  double* tile_partials;
  unsigned* ready;
};

struct BatchArgs {
  const BatchItem* items;
  const int4* units;        // (item, tile, direction or -1, 0): record/whole units longest
                            // first, then the direction units of split items
  int n_units;
  unsigned* counter;        // next unit (zeroed before each launch)
  unsigned* err;            // kErr* bits (zeroed before each launch)
  double* scratch;          // partials of whole units, scratch_stride doubles per CTA
  long long scratch_stride;
  unsigned char* wglob;     // global work vectors (GW instance): CTA b at wglob + b*wglob_stride
  long long wglob_stride;
};

constexpr int kGwBlock = 128;   // threads per CTA of the global-work-vector value sweeps
int occupancy_gw_primal(bool record);  // CTAs per SM of the global-work-vector value/record sweep
int occupancy_gw_sp();           // ... of the sparsity sweeps
int occupancy_gw_dir(bool adjoint);  // ... of the derivative sweeps (one warp per CTA)
cudaError_t launch_gather(long long n, long long ld, int count, const long long* src_row,
                          const double* src, double* dst, cudaStream_t s);
cudaError_t launch_batch(const BatchArgs& b, int grid, size_t smem, bool split, bool gw,
                         cudaStream_t s);
int occupancy_batch(size_t smem, bool split, bool gw);

// Error bits written to TapeView::err.
constexpr int kErrWaitTimeout = 1;   // a bounded wait on a staged chunk ran out
constexpr int kErrBadOpcode = 2;     // an instruction with an unknown opcode was met

// Shared memory a launch needs (bytes).
size_t smem_primal(int sz_w, int block);
size_t smem_dir(int sz_w, int dir_warps, int chunk);   // plan-free adjoint (8-byte stream)
size_t smem_lean(int sz_w, int dir_warps, int chunk);  // lean tangent / adjoint
int max_smem_optin();

cudaError_t launch_eval(const SweepArgs& a, int grid, cudaStream_t s);
cudaError_t launch_record(const SweepArgs& a, int grid, cudaStream_t s);
// Derivative sweeps: 1-D grid whose size is a multiple of the direction-group count
// ceil(ndir / (block/32)); CTA b works on direction group b % groups.
// Variants of the warp-independent derivative sweeps: entries per software-pipeline group,
// a register cap that lets more one-warp CTAs reside per SM, 32-instance tiles per warp (IPT)
// and, for the tangent sweep, directions per warp (K, walking the union stream of K
// directions). All variants do the same arithmetic in the same order; only speed differs, so
// the host may pick any. A variant's work vector takes smem_lean(sz_w, IPT*K, 0) bytes.
// G8/G4 variants keep more partial loads in flight per warp: for launches with few warps per SM
enum TanVariant : int {
  TV_G2_R80 = 0, TV_G2_R64, TV_G1_R64, TV_G2_K2, TV_G2_K4, TV_G4_R128, TV_G8_R256, TV_COUNT
};
enum AdjVariant : int {
  AV_G2_R80 = 0, AV_G1_R64, AV_G2_R64, AV_G2_I2_R128, AV_G4_R128, AV_G8_R256, AV_COUNT
};
void tan_variant_shape(int variant, int* ipt, int* k);
int adj_variant_ipt(int variant);
// entries per pipeline group (G) of a variant: the keyed-stream layout it reads
int tan_variant_group(int variant);
int adj_variant_group(int variant);
cudaError_t launch_tangent(const SweepArgs& a, int grid, int variant, cudaStream_t s);
// Windowed tangent sweep: one CTA per SM of a warp that stages, window by window, a tile's
// recorded partials and the window's entry block into a shared-memory ring with bulk copies,
// and win_dirs warps that each walk one direction's entries of the window from shared memory
// (the same arithmetic as k_tangent, so the same bits). Work items (tile, direction group)
// in a static stride over a persistent grid.
constexpr int kWinMaxDirs = 31;
constexpr int kWinBarBytes = 128;  // full/empty mbarriers of up to 8 stages
__host__ __device__ inline int win_header_words(int dirs) { return (dirs + 3 + 3) & ~3; }
size_t smem_tangent_win(int sz_w, int dirs, int stages, int rows, int ents);
cudaError_t launch_tangent_win(const SweepArgs& a, int grid, cudaStream_t s);
cudaError_t launch_adjoint(const SweepArgs& a, int grid, int variant, cudaStream_t s);
// The adjoint sweep without an activity plan (see k_adjoint<DW, true>).
cudaError_t launch_adjoint_dense(const SweepArgs& a, int grid, cudaStream_t s);
cudaError_t launch_sp_forward(const SweepArgs& a, int grid, cudaStream_t s);
cudaError_t launch_sp_reverse(const SweepArgs& a, int grid, cudaStream_t s);
cudaError_t launch_activity(const SweepArgs& a, int grid, cudaStream_t s);
// The persistent batch's bounded wait on flag (nonzero: ready); a timeout ORs kErrWaitTimeout
// into *err (one warp).
cudaError_t launch_wait_probe(const unsigned* flag, unsigned* err, cudaStream_t s);
// Cooperative value (record = false) or record sweep: a.block threads (a multiple of 32, at
// most kCoopMaxThreads) share one 32-instance tile and run its level schedule; the work vector
// in shared memory (lv_sz_w x 32 doubles), or in a.wglob blocks when set.
constexpr int kCoopMaxThreads = 1024;
cudaError_t launch_coop(const SweepArgs& a, bool record, int grid, cudaStream_t s);
// Cooperative sparsity sweeps (forward: the value sweep's levels; reverse: the reverse
// schedule's levels, last first); shared memory smem_coop of the schedule's work vector.
cudaError_t launch_coop_sp(const SweepArgs& a, bool reverse, int grid, cudaStream_t s);
int occupancy_coop_sp(int threads, size_t smem);
// Cooperative tangent sweep over recorded partials: one CTA of kCoopTanThreads threads per
// (tile, direction) item; identity seeds use a.dirmap (flat input nonzero -> direction, null:
// the nonzero's own index) and a.in_off. Shared memory: smem_tangent_coop.
constexpr int kCoopTanThreads = 512;
constexpr int kCoopTanQ = 4;  // instructions per warp and level handled at once
cudaError_t launch_tangent_coop(const SweepArgs& a, int grid, cudaStream_t s);
size_t smem_tangent_coop(int lv_sz_w, bool global);
int occupancy_tangent_coop(size_t smem, bool global);
// Cooperative adjoint sweep over recorded partials: one CTA of kCoopTanThreads threads per
// (tile, direction) item walks the reverse level schedule last level first; a.zero_in lists
// the inputs whose sensitivity is a structural zero. Shared memory: smem_tangent_coop of the
// reverse schedule's work-vector length.
cudaError_t launch_adjoint_coop(const SweepArgs& a, int grid, cudaStream_t s);
int occupancy_adjoint_coop(size_t smem);
size_t smem_coop(int lv_sz_w);
int occupancy_coop(int threads, size_t smem, bool global);

// Resident CTAs per SM for a given kernel family and shared-memory footprint.
int occupancy_primal(int block, size_t smem);
int occupancy_dir(int variant, bool adjoint, size_t smem);  // warp-independent sweeps
int occupancy_dense(int dir_warps, size_t smem);   // plan-free adjoint

}  // namespace cgb
