// Launch interface between the C-ABI layer (abi.cu) and the tape-sweep kernels (sweeps.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "device_ops.cuh"

namespace cgb {

constexpr int kChunk = 256;      // instructions per staged chunk (2 KiB), value sweeps
constexpr int kPofsGran = 16;    // granularity of the per-chunk partial offsets
constexpr int kLeanPB = 63;      // partials per staged chunk block (plan-free adjoint)
constexpr int kEntGroup = 8;     // entry streams are padded to a multiple of this
constexpr int kBatchGroup = 4;   // entries per software-pipelined group in the batch kernel
constexpr unsigned kMaxPartials = 1u << 21;  // recorded partials per instance the entries address

// Entry kinds of the lean derivative streams (bits 16-19 of an entry's meta word).
enum LeanKind : unsigned {
  LK_NOP = 0, LK_GEN, LK_ADD, LK_SUB, LK_NEG, LK_TWICE, LK_ASSIGN, LK_IFZ, LK_INPUT, LK_OUTPUT,
  LK_CONST, LK_MIXED
};
constexpr int kMaxIo = 64;       // inputs/outputs per tape handled by one launch

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
  // derivative entry streams (host-compiled; see the derivative sweeps)
  const uint4* dstream;             // entries of all streams
  const int2* dchunks;              // per direction (tangent) or one (adjoint): first entry, count
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
  int adj_ngr;              // its groups of kBatchGroup entries
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
int occupancy_gw_primal();       // CTAs per SM of the global-work-vector value/record sweep
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
