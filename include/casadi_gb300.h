/*
 * casadi_gb300.h — C ABI of the GB300 (sm_103a) evaluator for CasADi SX tapes.
 *
 * The library evaluates an SXFunction algorithm tape (CasADi's ScalarAtomic list,
 * casadi/core/sx_function.hpp:37-44) over many instances at once, on one GPU:
 *   eval         forward value sweep      (replaces SXFunction::eval,
 *                                          casadi/core/sx_function.cpp:72-127)
 *   forward      forward-mode AD sweep    (numeric analogue of SXFunction::ad_forward,
 *                                          casadi/core/sx_function.cpp:1194-1366)
 *   reverse      adjoint sweep            (numeric analogue of SXFunction::ad_reverse,
 *                                          casadi/core/sx_function.cpp:1368-1569)
 *   sp_forward   bvec_t sparsity, forward (SXFunction::sp_forward, sx_function.cpp:1657-1682)
 *   sp_reverse   bvec_t sparsity, reverse (SXFunction::sp_reverse, sx_function.cpp:1742-1782)
 *   map_eval     Map::eval with host buffers in the Map's instance-major layout
 *                (casadi/core/map.cpp:141-157, :327-386)
 *
 * Conventions follow CasADi's C API (casadi/casadi_c.h:76-127, casadi/core/casadi_c.cpp:298-332):
 * tapes are addressed by an int id from a process-wide registry, every entry point returns an
 * int status (0 = success, negative = failure), nothing throws, and the text of the last error
 * of the calling thread is available from casadi_gb300_last_error(). Registry creation and
 * destruction are not thread-safe with respect to each other (as noted in casadi_c.h:55-68);
 * evaluation calls on distinct streams are.
 *
 * Device data layout ("instance-minor"): for input j with nnz_in[j] nonzeros, nonzero k of
 * instance i is at arg[j][k*ld + i], ld >= n. Outputs likewise. Direction d of a seed or
 * sensitivity block is at ptr[(d*nnz + k)*ld + i]. A null pointer for an input reads zeros and
 * a null pointer for an output skips it, exactly as SXFunction::eval treats null arg/res.
 * All device pointers must be 8-byte aligned device memory of the current CUDA device.
 *
 * Streams are passed as void* (a cudaStream_t, 0 for the legacy default stream). Device-side
 * sweeps are asynchronous; casadi_gb300_sync() waits and reports device-side error flags.
 */
#ifndef CASADI_GB300_H
#define CASADI_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define CASADI_GB300_API __attribute__((visibility("default")))
#else
#define CASADI_GB300_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* One tape instruction, with the same 16-byte layout as CasADi's ScalarAtomic
 * (casadi/core/sx_function.hpp:37-44): op, i0, then either the constant d (OP_CONST)
 * or the two ints i1, i2. A CasADi build can pass algorithm_.data() unchanged. */
typedef struct {
  int op;
  int i0;
  union {
    double d;
    int i[2];
  } a;
} casadi_gb300_atomic;

/* Status codes (the negative values of casadi_c.cpp:320-332 plus device-specific ones). */
#define CASADI_GB300_OK 0
#define CASADI_GB300_ERR_ID (-1)       /* no tape with this id */
#define CASADI_GB300_ERR_ARG (-2)      /* invalid argument or tape */
#define CASADI_GB300_ERR_CUDA (-3)     /* a CUDA runtime call failed */
#define CASADI_GB300_ERR_DEVICE (-4)   /* a sweep reported a device-side error flag */
#define CASADI_GB300_ERR_SCRATCH (-5)  /* the scratch buffer is too small */
#define CASADI_GB300_ERR_UNSUPPORTED (-6)

/* Message of the last failed call on this thread ("" if none). */
CASADI_GB300_API const char* casadi_gb300_last_error(void);

/* Library version as "major.minor.patch". */
CASADI_GB300_API const char* casadi_gb300_version(void);

/* Register a tape. The tape is validated on the host: every slot index < sz_w, every
 * INPUT/OUTPUT reference inside nnz_in/nnz_out, every op a supported scalar op (OP_CALL and
 * free OP_PARAMETER are rejected with CASADI_GB300_ERR_UNSUPPORTED), then uploaded to the
 * current device. Returns the tape id (>= 0) or a negative status.
 * Replaces: SXFunction::init's product algorithm_/worksize_ (sx_function.cpp:476-841) as
 * consumed by the caller; the tape is taken, not rebuilt. */
CASADI_GB300_API int casadi_gb300_tape_create(const casadi_gb300_atomic* alg, int n_instr, int n_in,
                             const int* nnz_in, int n_out, const int* nnz_out, int sz_w);

/* Release a tape and its device memory. Cf. casadi_c_decref_id (casadi_c.h:113). */
CASADI_GB300_API int casadi_gb300_tape_free(int id);

/* A tape with OP_CALL instructions (nested Functions): instruction k with op OP_CALL (48)
 * names call a.i[0]; call c evaluates the registered tape call_tape[c] with its input
 * nonzeros read from the caller's work-vector slots call_dep[c][0 .. nnz_in-1] and its output
 * nonzeros written to call_res[c][0 .. nnz_out-1] (-1: not needed) — the reference's
 * ExtendedAlgEl dep/res (casadi/core/sx_function.cpp:630-661) and call_fwd (:1595-1621).
 * The calls are inlined on the host (callee slots placed past the caller's work vector, input
 * and output copies as OP_ASSIGN), then the tape is created as by casadi_gb300_tape_create, so
 * every sweep and derivative supports them. Returns the new tape id. */
CASADI_GB300_API int casadi_gb300_tape_create_calls(const casadi_gb300_atomic* alg,
                           int n_instr, int n_in, const int* nnz_in, int n_out,
                           const int* nnz_out, int sz_w, int n_calls, const int* call_tape,
                           const int* const* call_dep, const int* const* call_res);

/* Tapes from CasADi's serialized text: what Function::serialize() returns
 * (casadi/core/function.cpp:1477-1489) or what Function::save writes to a .casadi file
 * (serializer.cpp, FileSerializer; Function::load, function.cpp:1541-1549), both in either
 * debug mode, read without libcasadi. `text`/`len`: the characters (trailing whitespace is
 * ignored).
 *
 * Create the tape of a serialized SXFunction (SXFunction(DeserializingStream&),
 * casadi/core/sx_function.cpp:1926-1997): its algorithm as casadi_gb300_tape_create takes it,
 * with the SXFunctions it calls (OP_CALL) decoded and inlined as casadi_gb300_tape_create_calls
 * does. Returns the tape id, or a negative status: ERR_ARG for malformed text,
 * ERR_UNSUPPORTED for a Function of another class, free variables, or nested Functions that
 * are not SXFunctions. */
CASADI_GB300_API int casadi_gb300_tape_deserialize(const char* text, size_t len);

/* Loading serialized files as casadi_c does (casadi/casadi_c.h:52-86, casadi/core/
 * casadi_c.cpp:73-130), for SXFunctions: push_file reads a file Function::save or a
 * FileSerializer wrote (one Function or a vector of them) and creates a tape for each
 * Function in it; pop_file frees the tapes the last push created. Returns 0 or a negative
 * status (a file with a Function that is not an SXFunction loads nothing). */
CASADI_GB300_API int casadi_gb300_push_file(const char* filename);
CASADI_GB300_API int casadi_gb300_pop_file(void);
/* Number of loaded Functions; the tape id of the one named `name` (ERR_ID if none, like
 * casadi_c_id); the name of loaded Function k (NULL if out of range; valid until the next
 * push or pop). */
CASADI_GB300_API int casadi_gb300_n_loaded(void);
CASADI_GB300_API int casadi_gb300_loaded_tape(const char* name);
CASADI_GB300_API const char* casadi_gb300_loaded_name(int k);

/* The algorithm of a serialized SXFunction without OP_CALL instructions, on the host (no GPU
 * needed): call with alg == NULL for the sizes (n_instr, n_in, n_out, sz_w), then with alg
 * holding cap >= n_instr entries; nnz_in/nnz_out (if not NULL) receive n_in/n_out counts. */
CASADI_GB300_API int casadi_gb300_serialized_decode(const char* text, size_t len,
                           casadi_gb300_atomic* alg, int cap, int* n_instr, int* n_in,
                           int* nnz_in, int* n_out, int* nnz_out, int* sz_w);

/* A JSON summary of serialized text (any Function class: the class, name, input and output
 * names and sparsity sizes, the versions of the bodies read; for SXFunctions the instruction
 * count, work-vector size, free variables and called functions). Writes at most cap bytes
 * (NUL-terminated) to buf; *need receives the full length + 1. */
CASADI_GB300_API int casadi_gb300_serialized_describe(const char* text, size_t len, char* buf,
                           size_t cap, size_t* need);

/* The tape as the GPU sweeps run it: casadi_gb300_tape_create reorders the instructions so
 * fewer values are live at once (the work vector of every 32-instance tile sits in shared
 * memory, and its length decides how many tiles an SM runs at a time) and reassigns the slots.
 * Each instruction keeps its operation and operand values, and the users of every value keep
 * their relative order, so values, forward and adjoint sensitivities are bit-identical to the
 * original order. This entry point returns the scheduled tape (n_instr atomics written to out,
 * same layout as alg) and its work-vector length, without touching a device. It replaces the
 * reference's depth-first order and last-in first-out slot assignment for the GPU
 * (SXFunction::init, casadi/core/sx_function.cpp:530-540 and 690-753); the reference has no
 * separate call for it. */
CASADI_GB300_API int casadi_gb300_tape_schedule(const casadi_gb300_atomic* alg, int n_instr,
                               int n_in, const int* nnz_in, int n_out, const int* nnz_out,
                               int sz_w, casadi_gb300_atomic* out, int* sz_w_out);

/* Shape queries. Cf. casadi_c_n_in_id/casadi_c_n_out_id/casadi_c_work_id (casadi_c.h:115-124):
 * sz_w is the tape's work-vector length; n_partials the partial derivatives one instance
 * records for the AD sweeps. */
/* Host only (no device needed): the level schedule the cooperative value/record sweeps run
 * for this tape (after the scheduling of casadi_gb300_tape_schedule): instructions grouped
 * into levels of at most `width` mutually independent instructions, slots renamed (a slot
 * freed at a value's last use is reused from the next level on), the scheduler deferring new
 * values while `slot_cap` slots are live. out (n_instr entries, optional): the leveled tape in
 * the reference's format; source (optional): each one's index in the scheduled tape;
 * level_begin (n_levels + 1 entries, optional): level l is out[level_begin[l] ..
 * level_begin[l+1]). Executed in order it gives the same results as the tape. */
CASADI_GB300_API int casadi_gb300_tape_levels(const casadi_gb300_atomic* alg, int n_instr,
                            int n_in, const int* nnz_in, int n_out, const int* nnz_out,
                            int sz_w, int width, int slot_cap, casadi_gb300_atomic* out,
                            int* source, int* level_begin, int* n_levels, int* sz_w_out);

CASADI_GB300_API int casadi_gb300_tape_info(int id, int* n_instr, int* n_in, int* n_out, int* sz_w,
                           int* n_partials);

/* Scratch bytes the AD sweeps need to process n instances in one wave: the recorded partials
 * and a few bytes past them for the tangent sweep's work counter (a scratch without them runs
 * that sweep with a static work split, same results). A smaller scratch buffer is accepted
 * down to casadi_gb300_scratch_min(); the sweep then runs in waves. */
CASADI_GB300_API int casadi_gb300_scratch_size(int id, int64_t n, size_t* bytes);
CASADI_GB300_API int casadi_gb300_scratch_min(int id, size_t* bytes);

/* Forward value sweep over n instances (device pointers, instance-minor, leading dim ld).
 * Replaces SXFunction::eval (sx_function.cpp:72-127) called once per instance by
 * Map/OmpMap::eval (map.cpp:141-157, :340-386). */
CASADI_GB300_API int casadi_gb300_eval(int id, int64_t n, int64_t ld, const double* const* arg,
                      double* const* res, void* stream);

/* Forward-mode AD: values plus nfwd directional derivatives.
 * fseed[j]: nfwd x nnz_in[j] x ld, fsens[j]: nfwd x nnz_out[j] x ld (direction-major).
 * res may be all-null. scratch: device buffer of scratch_bytes (casadi_gb300_scratch_size).
 * A null fsens[j] leaves output j's sensitivities out, and the tangent sweep skips every
 * instruction that reaches no requested output (the same holds for the Jacobian entry
 * points' jac[j]); the requested ones are unchanged bit for bit.
 * Replaces evaluating Function::forward(nfwd) (function_internal.cpp:2220-2283, built by
 * SXFunction::ad_forward, sx_function.cpp:1194-1366) under a Map. */
CASADI_GB300_API int casadi_gb300_forward(int id, int64_t n, int64_t ld, int nfwd, const double* const* arg,
                         double* const* res, const double* const* fseed, double* const* fsens,
                         void* scratch, size_t scratch_bytes, void* stream);

/* Reverse-mode AD: values plus nadj adjoint sensitivities.
 * aseed[j]: nadj x nnz_out[j] x ld (output seeds), asens[j]: nadj x nnz_in[j] x ld
 * (overwritten, not accumulated). Replaces evaluating Function::reverse(nadj)
 * (function_internal.cpp:2285-2340, built by SXFunction::ad_reverse, sx_function.cpp:1368-1569)
 * under a Map. */
CASADI_GB300_API int casadi_gb300_reverse(int id, int64_t n, int64_t ld, int nadj, const double* const* arg,
                         double* const* res, const double* const* aseed, double* const* asens,
                         void* scratch, size_t scratch_bytes, void* stream);

/* Jacobian of every output with respect to every input nonzero, by forward mode with unit
 * seeds generated on the device (no seed memory). Direction d is the d-th input nonzero in
 * input order; jac[j] is nnz_in_total x nnz_out[j] x ld (direction-major), i.e. column d of
 * the Jacobian block of output j. Replaces evaluating Function::jacobian()
 * (casadi/core/function.cpp:1068-1074, function_internal.cpp:2403-2442, built by
 * XFunction::jac, casadi/core/x_function.hpp:441-840) under a Map. */
CASADI_GB300_API int casadi_gb300_jacobian(int id, int64_t n, int64_t ld, const double* const* arg,
                          double* const* res, double* const* jac, void* scratch,
                          size_t scratch_bytes, void* stream);

/* Jacobian and adjoint sensitivities in one call: one record sweep, then the identity-seeded
 * forward sweep (jac as in casadi_gb300_jacobian) and nadj adjoint directions (aseed/asens as
 * in casadi_gb300_reverse), both reading the same recorded partials. Results equal those of
 * the two separate calls bit for bit. Replaces evaluating CasADi's jacobian() and reverse()
 * Functions (casadi/core/function_internal.cpp:2285-2340) one after the other on a Map. */
CASADI_GB300_API int casadi_gb300_jacobian_reverse(int id, int64_t n, int64_t ld,
                           const double* const* arg, double* const* res, double* const* jac,
                           int nadj, const double* const* aseed, double* const* asens,
                           void* scratch, size_t scratch_bytes, void* stream);

/* Sparsity propagation with bvec_t = uint64_t (casadi/core/casadi_common.hpp:126-130).
 * sp_forward: res[j] = dependency bits of the outputs given arg bits
 * (SXFunction::sp_forward, sx_function.cpp:1657-1682).
 * sp_reverse: arg[j] |= bits propagated back from res[j]; res[j] is cleared
 * (SXFunction::sp_reverse, sx_function.cpp:1742-1782). */
CASADI_GB300_API int casadi_gb300_sp_forward(int id, int64_t n, int64_t ld, const uint64_t* const* arg,
                            uint64_t* const* res, void* stream);
CASADI_GB300_API int casadi_gb300_sp_reverse(int id, int64_t n, int64_t ld, uint64_t* const* arg,
                            uint64_t* const* res, void* stream);

/* Activity analysis over n instances (SXFunction::eval_activity, sx_function.cpp:1684-1718;
 * Function::eval_activity, function.cpp:1260-1267): arg words are the inputs' activity (a set
 * bit: possibly nonzero), res receives the outputs'. A constant is active when nonzero; an
 * arithmetic result is inactive only when its op gives zero for its inactive operands
 * (F0X/FX0/F00 checkers, calculus.hpp:485-540), else all bits are set. Null arg reads zeros,
 * null res is skipped. Layout as casadi_gb300_sp_forward. */
CASADI_GB300_API int casadi_gb300_eval_activity(int id, int64_t n, int64_t ld,
                            const uint64_t* const* arg, uint64_t* const* res, void* stream);

/* MapSum over n instances (MapSum::eval_gen, casadi/core/mapsum.cpp:153-181; created by
 * Function::map(name, parallelization, n, reduce_in, reduce_out), function.cpp:787-827).
 * reduce_in[j] != 0: input j is shared by every instance, arg[j] holds nnz_in[j] values
 * (seeds of a shared input: (ndir, nnz_in[j]) values). reduce_out[j] != 0: output j is summed
 * over the instances, res[j] receives nnz_out[j] values (sensitivities: (ndir, nnz_out[j])).
 * Null flag arrays mean no flags. Every other input/output uses the instance-minor layout of
 * casadi_gb300_eval with leading dimension ld. order 0 sums in instance order starting from
 * zero, MapSum's own order (the reference's bits); order 1 sums by a fixed blocked tree
 * (256-instance blocks, then their sums, until one value; the bits do not depend on the
 * launch), which does not form a chain of n dependent adds. */
typedef struct casadi_gb300_mapsum_spec {
  const int* reduce_in;  /* n_in flags, or null */
  const int* reduce_out; /* n_out flags, or null */
  int order;             /* 0: instance order, 1: blocked tree */
} casadi_gb300_mapsum_spec;

/* Device scratch the MapSum calls below need for n instances and up to ndir directions
 * (0 for eval and the sparsity sweeps): per-instance rows of the summed outputs and shared
 * inputs' sensitivities, the tree's level buffers and the derivative sweeps' partials. */
CASADI_GB300_API int casadi_gb300_mapsum_scratch_size(int id, int64_t n, int ndir,
                            const casadi_gb300_mapsum_spec* spec, size_t* bytes);
CASADI_GB300_API int casadi_gb300_mapsum_eval(int id, int64_t n, int64_t ld,
                            const casadi_gb300_mapsum_spec* spec, const double* const* arg,
                            double* const* res, void* scratch, size_t scratch_bytes,
                            void* stream);
/* Forward mode of a MapSum (MapSum::get_forward, mapsum.cpp:255-349): the seeds of shared
 * inputs are shared, the sensitivities of summed outputs are summed. */
CASADI_GB300_API int casadi_gb300_mapsum_forward(int id, int64_t n, int64_t ld,
                            const casadi_gb300_mapsum_spec* spec, int nfwd,
                            const double* const* arg, double* const* res,
                            const double* const* fseed, double* const* fsens, void* scratch,
                            size_t scratch_bytes, void* stream);
/* Reverse mode of a MapSum (MapSum::get_reverse, mapsum.cpp:351-413): the adjoint seeds of
 * summed outputs are shared, the adjoint sensitivities of shared inputs are summed. */
CASADI_GB300_API int casadi_gb300_mapsum_reverse(int id, int64_t n, int64_t ld,
                            const casadi_gb300_mapsum_spec* spec, int nadj,
                            const double* const* arg, double* const* res,
                            const double* const* aseed, double* const* asens, void* scratch,
                            size_t scratch_bytes, void* stream);
/* Sparsity of a MapSum (MapSum::sp_forward / sp_reverse, mapsum.cpp:190-232): summed outputs
 * OR over the instances; in reverse, a summed output's seed bits reach every instance and are
 * cleared afterwards, and a shared input receives (|=) the OR of every instance's bits. */
CASADI_GB300_API int casadi_gb300_mapsum_sp_forward(int id, int64_t n, int64_t ld,
                            const casadi_gb300_mapsum_spec* spec, const uint64_t* const* arg,
                            uint64_t* const* res, void* scratch, size_t scratch_bytes,
                            void* stream);
CASADI_GB300_API int casadi_gb300_mapsum_sp_reverse(int id, int64_t n, int64_t ld,
                            const casadi_gb300_mapsum_spec* spec, uint64_t* const* arg,
                            uint64_t* const* res, void* scratch, size_t scratch_bytes,
                            void* stream);

/* Mapaccum over n instances (Function::mapaccum(name, N, n_accum), casadi/core/
 * function.cpp:668-747): the tape is called N times; the first n_accum outputs of call k are
 * the first n_accum inputs of call k+1 (call 0 reads them from arg, nnz_in[i] per instance);
 * every other input j of call k is nonzeros [k*nnz_in[j], (k+1)*nnz_in[j]) of arg[j], and
 * output j of call k is nonzeros [k*nnz_out[j], (k+1)*nnz_out[j]) of res[j] (the horzcat of
 * the N calls). Instance-minor layout with leading dimension ld. An accumulator input and its
 * output have the same nonzeros. Accumulator outputs that res does not keep (null) live in
 * the scratch (casadi_gb300_mapaccum_scratch_size: enough for every call below with up to
 * ndir directions). Nothing is unrolled: one tape, N launches, outputs fed back in place. */
CASADI_GB300_API int casadi_gb300_mapaccum_scratch_size(int id, int N, int n_accum, int64_t n,
                            int ndir, size_t* bytes);
/* Scratch with which casadi_gb300_mapaccum_reverse records the partials of every call on the
 * way forward and runs adjoint sweeps only on the way back (same bits; no record per call in
 * the reverse pass): the size above plus N calls' partials. A smaller scratch (down to the
 * size above) runs the checkpointed form. */
CASADI_GB300_API int casadi_gb300_mapaccum_reverse_scratch_size(int id, int N, int n_accum,
                           int64_t n, int nadj, size_t* bytes);
CASADI_GB300_API int casadi_gb300_mapaccum_eval(int id, int N, int n_accum, int64_t n,
                            int64_t ld, const double* const* arg, double* const* res,
                            void* scratch, size_t scratch_bytes, void* stream);
/* Forward mode: seeds as arg with a leading direction axis ((nfwd, nnz, ld) for accumulators,
 * (nfwd, nnz*N, ld) otherwise), sensitivities as res; the tangents of call k's accumulator
 * outputs seed call k+1. */
CASADI_GB300_API int casadi_gb300_mapaccum_forward(int id, int N, int n_accum, int64_t n,
                            int64_t ld, int nfwd, const double* const* arg, double* const* res,
                            const double* const* fseed, double* const* fsens, void* scratch,
                            size_t scratch_bytes, void* stream);
/* Reverse mode: adjoint seeds for every call's outputs ((nadj, nnz_out*N, ld)), sensitivities
 * of x0 ((nadj, nnz, ld)) and of the stacked inputs ((nadj, nnz*N, ld)). The value sweeps of
 * all calls run first (keeping every accumulator value), then call k = N-1 .. 0 records again
 * from its stored inputs and runs its adjoint with the seed of its accumulator outputs plus
 * the adjoint call k+1 returned for them: checkpointing at every call boundary. */
CASADI_GB300_API int casadi_gb300_mapaccum_reverse(int id, int N, int n_accum, int64_t n,
                            int64_t ld, int nadj, const double* const* arg, double* const* res,
                            const double* const* aseed, double* const* asens, void* scratch,
                            size_t scratch_bytes, void* stream);

/* Wait for all work on `stream` and report device-side error flags raised by sweeps of this
 * tape (bounded waits that ran out, malformed instructions). Clears the flags. */
CASADI_GB300_API int casadi_gb300_sync(int id, void* stream);

/* Memory objects for the host-buffer path (cf. casadi_c_checkout_id/release_id,
 * casadi_c.h:114-115): each owns a CUDA stream and device staging buffers that grow on
 * demand and are reused across calls. */
CASADI_GB300_API int casadi_gb300_checkout(void);
CASADI_GB300_API int casadi_gb300_release(int mem);

/* Map::eval with HOST buffers in the Map's instance-major layout: input j of instance i at
 * arg[j] + i*nnz_in[j] (map.cpp:150-153). Copies in, runs the sweep, copies out, and waits.
 * Pinned host memory gives the fastest copies. Replaces OmpMap::eval (map.cpp:340-386). */
CASADI_GB300_API int casadi_gb300_map_eval(int id, int mem, int64_t n, const double* const* arg,
                          double* const* res);

/* Map over the Jacobian with host buffers: jac[j] is instance-major
 * (jac[j] + (i*nnz_in_total + d)*nnz_out[j] holds column d of instance i). */
/* Map over the bvec_t sparsity sweeps with host buffers in the Map layout (arg[j] +
 * i*nnz_in[j], res[j] + i*nnz_out[j]). Replaces: Map::sp_forward / Map::sp_reverse, which call
 * the function's sweep instance by instance (casadi/core/map.cpp:164-184); sp_reverse is in
 * place as there: arg[j] |= propagated bits, res[j] cleared. A null block is skipped. */
CASADI_GB300_API int casadi_gb300_map_sp_forward(int id, int mem, int64_t n,
                             const uint64_t* const* arg, uint64_t* const* res);
CASADI_GB300_API int casadi_gb300_map_sp_reverse(int id, int mem, int64_t n,
                             uint64_t* const* arg, uint64_t* const* res);
CASADI_GB300_API int casadi_gb300_map_jacobian(int id, int mem, int64_t n, const double* const* arg,
                              double* const* res, double* const* jac);

/* Map over the forward sweep with host buffers (the Map's forward(nfwd), map.cpp:219-271):
 * fseed[j] is instance-major (fseed[j] + (i*nfwd + d)*nnz_in[j] holds direction d of
 * instance i), fsens likewise with nnz_out[j]. */
CASADI_GB300_API int casadi_gb300_map_forward(int id, int mem, int64_t n, int nfwd,
                             const double* const* arg, double* const* res,
                             const double* const* fseed, double* const* fsens);

/* Map over the reverse sweep with host buffers: aseed[j] is instance-major
 * (aseed[j] + (i*nadj + d)*nnz_out[j] holds direction d of instance i), asens likewise. */
CASADI_GB300_API int casadi_gb300_map_reverse(int id, int mem, int64_t n, int nadj, const double* const* arg,
                             double* const* res, const double* const* aseed,
                             double* const* asens);
/* The same two calls with seeds and sensitivities in the order of the Map's own derivative
 * Functions: direction d of instance i of block j at fseed[j] + (d*n + i)*nnz_in[j] (and
 * likewise fsens, aseed, asens), values as above. Replaces: the MX index-slice reorders that
 * Map::get_forward / Map::get_reverse wrap around f.forward(nfwd).map(n) and
 * f.reverse(nadj).map(n) (casadi/core/map.cpp:219-325), so a cuda Map's derivative needs no
 * reorder pass: the sweeps address this order through their block strides. */
CASADI_GB300_API int casadi_gb300_map_forward_outer(int id, int mem, int64_t n, int nfwd,
                             const double* const* arg, double* const* res,
                             const double* const* fseed, double* const* fsens);
CASADI_GB300_API int casadi_gb300_map_reverse_outer(int id, int mem, int64_t n, int nadj,
                             const double* const* arg, double* const* res,
                             const double* const* aseed, double* const* asens);
/* Host-buffer form of casadi_gb300_jacobian_reverse: arg/res/aseed as in the two calls
 * above, jac[j] as in casadi_gb300_map_jacobian, asens[j] as in casadi_gb300_map_reverse. */
CASADI_GB300_API int casadi_gb300_map_jacobian_reverse(int id, int mem, int64_t n,
                           const double* const* arg, double* const* res, double* const* jac,
                           int nadj, const double* const* aseed, double* const* asens);

/* Autotuning of the derivative sweeps (on by default): the first call of each kind
 * (0 seeded forward, 1 Jacobian, 2 adjoint) and launch size (at most 16 tiles per SM, or more)
 * on a tape runs each kernel variant once on that wave (large launches: those that fill the
 * GPU several times; small launches also try the cooperative level sweep), keeps the fastest
 * for the tape and synchronizes the stream once; it is skipped while the stream is being
 * captured into a CUDA graph.
 * Variants differ only in speed: every variant does the same arithmetic in the same order.
 * casadi_gb300_tuned_variant reports the kept variant (-1: not tuned yet). No counterpart in
 * the reference, whose Map has one code path per parallelization (casadi/core/map.cpp:39-51). */
CASADI_GB300_API int casadi_gb300_autotune(int enable);
CASADI_GB300_API int casadi_gb300_tuned_variant(int id, int kind, int* variant);
/* Work-vector residence of a tape's sweeps: 0 (default) shared memory when the scheduled
 * work vector fits, global memory (L1/L2-cached per-CTA blocks owned by the tape) when it does
 * not, and for the value/record/sparsity sweeps the fastest candidate, timed by the autotuner
 * on the first call of each sweep kind and launch size (at most 16 tiles of 32 instances per
 * SM, or more): shared, global, and for value/record/sparsity sweeps of the smaller launches
 * the cooperative level sweep (several warps share a tile and run the tape's independent
 * instructions level by level; casadi_gb300_tape_levels shows the schedule; sp_reverse, which
 * consumes its seeds, follows sp_forward's choice); 1 always global memory; 2 shared memory
 * whenever it fits; 3 the cooperative sweep for value/record/sparsity sweeps.
 * Results are identical in every mode. A tape whose global work vectors must grow cannot be
 * first used inside a CUDA graph capture. No counterpart in the reference, whose work vector
 * is the caller's w array (casadi/core/function_internal.hpp:414). */
CASADI_GB300_API int casadi_gb300_set_residence(int id, int mode);
/* Fixes the variant of one kind on a tape (kinds 0 and 1: 0..8; kind 2: 0..6), or clears it
 * for retuning (-1). Tangent variant 7 and adjoint variant 6 are the cooperative level sweeps,
 * which only launches of at most 16 tiles per SM use; tangent variant 8 is the windowed sweep
 * (the directions of a tile on one SM, recorded partials and entries staged into shared memory
 * window by window), used when at least 4 directions are swept and their work vectors fit. */
CASADI_GB300_API int casadi_gb300_set_variant(int id, int kind, int variant);

/* Colour-compressed Jacobian: n_colors forward directions, direction d seeded with 1 on
 * every flat input nonzero k with color[k] == d (color: one entry per nonzero of all inputs
 * in order, -1 = not seeded). comp[j] receives the compressed block of output j, direction-
 * major as fsens in casadi_gb300_forward. Structural activity is computed per direction, so
 * a direction walks only the instructions its seeded inputs reach. Replaces the forward
 * seeding of the reference's coloured jacobian (FunctionInternal::get_partition,
 * casadi/core/function_internal.cpp:2068-2160, and XFunction::jac,
 * casadi/core/x_function.hpp:441-840). */
CASADI_GB300_API int casadi_gb300_jacobian_colored(int id, int64_t n, int64_t ld,
                           int n_colors, const int* color, const double* const* arg,
                           double* const* res, double* const* comp, void* scratch,
                           size_t scratch_bytes, void* stream);

/* Row gather on the device: dst[e*ld + i] = src[src_row[e]*ld + i] for e < count, i < n
 * (src_row a device array). Recovers sparse Jacobian/Hessian nonzeros from colour-compressed
 * blocks; replaces the reference's scatter of compressed results into nonzeros
 * (casadi/core/x_function.hpp:702-826). */
CASADI_GB300_API int casadi_gb300_gather(int64_t n, int64_t ld, int count,
                                         const int64_t* src_row, const double* src,
                                         double* dst, void* stream);

/* Seed colourings for compressed Jacobians and Hessians (host only, no device). Patterns
 * are compressed-column arrays with sorted rows (CasADi's Sparsity layout). Both write one
 * colour per column and return the number of colours (or a negative status).
 *   uni_coloring: columns of one colour share no row (forward-mode seeds of a Jacobian);
 *     restates SparsityInternal::uni_coloring (casadi/core/sparsity_internal.cpp:2959-3045).
 *   star_coloring: star colouring of a symmetric pattern (Hessian seeds), ordering 1 =
 *     largest-first (the reference's default), 0 = index order; restates
 *     SparsityInternal::star_coloring and ::largest_first (:3398-3509, :3511-3545). */
CASADI_GB300_API int casadi_gb300_uni_coloring(int nrow, int ncol, const int* colind,
                                               const int* row, int* color);
CASADI_GB300_API int casadi_gb300_star_coloring(int n, const int* colind, const int* row,
                                                int ordering, int* color);

/* Persistent multi-tape batches. A batch is a list of items, each one tape over its own
 * instance range (device pointers, instance-minor layout as above): nadj == 0 runs the value
 * sweep, nadj > 0 the value sweep plus nadj adjoint directions (aseed/asens as in
 * casadi_gb300_reverse). casadi_gb300_batch_run evaluates every item in ONE persistent launch
 * whose warps drain a longest-first list of (item, 32-instance tile) units, so tapes of
 * uneven length and instance count keep the GPU full. With use_graph the launch is captured
 * once into a CUDA graph (on a stream the batch owns, ordered after and before the caller's
 * stream) and replayed; adding items or changing the scratch buffer re-captures it.
 * casadi_gb300_batch_add returns the item index. An item with two or more directions is
 * split: one unit per tile records its partials into a buffer the batch owns, and one unit
 * per (tile, direction) walks that direction after the tile's record unit has finished (a
 * bounded wait on a per-tile flag; record units precede direction units in the list), so the
 * directions of a tile run in parallel. No counterpart in the reference: a CasADi Map
 * evaluates one Function per call (casadi/core/map.cpp:141-157). */
CASADI_GB300_API int casadi_gb300_batch_create(void);
CASADI_GB300_API int casadi_gb300_batch_free(int batch);
CASADI_GB300_API int casadi_gb300_batch_add(int batch, int id, int64_t n, int64_t ld, int nadj,
                           const double* const* arg, double* const* res,
                           const double* const* aseed, double* const* asens);
/* A batch item of colour-compressed forward directions: as casadi_gb300_jacobian_colored
 * (color, comp), run in the batch's single launch. Returns the item index. */
CASADI_GB300_API int casadi_gb300_batch_add_jacobian_colored(int batch, int id, int64_t n,
                           int64_t ld, int n_colors, const int* color,
                           const double* const* arg, double* const* res, double* const* comp);
CASADI_GB300_API int casadi_gb300_batch_scratch_size(int batch, size_t* bytes);
/* Work-vector residence of a batch's launch: 0 (default) the faster of shared and global
 * memory, timed on the first run; 1 global memory; 2 shared memory. Same results either way. */
CASADI_GB300_API int casadi_gb300_batch_set_residence(int batch, int mode);
/* Waits for the batch's stream and reports a device-side failure of its last run (a
 * direction unit whose tile's record unit did not finish within its bounded wait). */
CASADI_GB300_API int casadi_gb300_batch_status(int batch);
CASADI_GB300_API int casadi_gb300_batch_run(int batch, void* scratch, size_t scratch_bytes,
                           int use_graph, void* stream);

/* Reverse-mode AD with segment checkpointing, for tapes whose recorded partials (8 bytes x
 * partials x instances) would not fit: the tape is cut into `segments` runs of consecutive
 * instructions (at most one per instruction), near equal shares of the partials and where the
 * fewest work-vector slots are live. The forward pass keeps only the live slots at each cut;
 * the backward pass re-records one segment at a time from its checkpoint and sweeps it in
 * reverse, so partials are held for one segment. Arguments as casadi_gb300_reverse; values
 * equal casadi_gb300_eval's, sensitivities casadi_gb300_reverse's up to the rounding of adjoint
 * sums that a cut associates differently. The scratch holds the checkpoints, two adjoint
 * buffers and one segment's partials: casadi_gb300_checkpoint_scratch_size gives its size for
 * one wave of all n instances and its minimum (below that: CASADI_GB300_ERR_SCRATCH; between
 * the two the segments' sweeps run in instance waves). Both return the number of segments
 * made, or a negative status. The segment tapes are built on the first call for a segment
 * count and kept with the tape; calls on one tape are serialised. Replaces the reverse sweep
 * over a stored work vector (SXFunction::ad_reverse, sx_function.cpp:1454-1560) when the
 * storage does not fit. */
CASADI_GB300_API int casadi_gb300_checkpoint_scratch_size(int id, int segments, int nadj,
                                                          int64_t n, size_t* bytes,
                                                          size_t* min_bytes);
CASADI_GB300_API int casadi_gb300_reverse_checkpointed(int id, int64_t n, int64_t ld, int nadj,
                                                       int segments, const double* const* arg,
                                                       double* const* res,
                                                       const double* const* aseed,
                                                       double* const* asens, void* scratch,
                                                       size_t scratch_bytes, void* stream);

/* Host only (no GPU needed): the segment plan of casadi_gb300_reverse_checkpointed for a
 * tape in the reference's format, after this library's scheduling (sz_w_out: its work-vector
 * length). cut[0..k]: positions in the scheduled instruction list; live_count[0..k]: live
 * slots at each cut; seg_len[0..k-1]: instructions of each segment tape, written one after
 * another to seg_alg (capacity entries; each segment tape has the tape's inputs plus input
 * n_in, the live slots at its first cut, and its outputs plus output n_out, the live slots at
 * its last cut). Returns k, the number of segments made. */
CASADI_GB300_API int casadi_gb300_tape_segments(const casadi_gb300_atomic* alg, int n_instr,
                                                int n_in, const int* nnz_in, int n_out,
                                                const int* nnz_out, int sz_w, int segments,
                                                int* cut, int* live_count, int* seg_len,
                                                casadi_gb300_atomic* seg_alg, int capacity,
                                                int* sz_w_out);

/* Allocation-free adjoint sweep: the same values and adjoint sensitivities as
 * casadi_gb300_reverse (arguments and layouts alike, no scratch argument), for callers that
 * cannot allocate device memory when they need derivatives -- real-time loops that forbid
 * allocation after start-up, plugins whose host framework owns the device allocator. It has
 * no counterpart in the reference.
 * Scratch is a fixed 64 MiB file-scope device array that each GPU loading the library holds
 * until exit; a call needing more (8 bytes x recorded partials x instances rounded up to 32)
 * is rejected with CASADI_GB300_ERR_SCRATCH. The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress), so make that first call before any stream capture.
 * All calls share the array and it keeps the last call's contents (nothing in it needs to
 * start at zero): calls that overlap on the GPU race, so serialize them, e.g. on one stream.
 * It uses no activity plan: contributions are always added to a zeroed adjoint, which can
 * differ from casadi_gb300_reverse only in the sign of zero results and in inf/NaN cases.
 * Both of its sweeps keep the work vector in shared memory: a tape whose work vector does not
 * fit there (sz_w x 256 bytes per 32-instance tile beyond the device's per-CTA limit, about
 * 880 slots on GB300) is refused with CASADI_GB300_ERR_UNSUPPORTED; casadi_gb300_reverse
 * handles it with global-memory work vectors. */
CASADI_GB300_API int casadi_gb300_reverse_noalloc(int id, int64_t n, int64_t ld, int nadj,
                                 const double* const* arg, double* const* res,
                                 const double* const* aseed, double* const* asens, void* stream);

/* Per-launch timing. While enabled, every sweep kernel launch is bracketed by CUDA events
 * recorded on its own stream. casadi_gb300_profile_collect waits for the recorded launches
 * and returns, per kernel family, the summed device milliseconds and the launch count, then
 * forgets them. Families: 0 eval, 1 record (values + partials), 2 tangent, 3 adjoint,
 * 4 sp_forward, 5 sp_reverse, 6 batch. This has no counterpart in the reference (CasADi's FStats
 * timers, casadi/core/timing.hpp:60-80, time host calls). */
CASADI_GB300_API int casadi_gb300_profile(int enable);
CASADI_GB300_API int casadi_gb300_profile_collect(double* ms, int* launches, int count);

/* Self-check of the device-side failure path: one warp runs the persistent batch's bounded
 * wait on a flag that nothing sets. The wait gives up after about a second, the kernel records
 * the timeout in its error word and returns, and this call reports it as
 * CASADI_GB300_ERR_DEVICE ("bounded wait ran out"); the CUDA context stays usable. Any other
 * result is an error of the failure path itself. */
CASADI_GB300_API int casadi_gb300_check_wait_timeout(void* stream);

/* FP64 pipe rate of the current device, the ceiling of the sweeps: a full grid of threads
 * each running independent dependent chains of one FP64 instruction kind (0 DFMA, 1 DADD,
 * 2 DMUL, 3 a product issued as DFMA with a -0 addend, 4 a sum issued as DFMA with a unit
 * factor); writes the best of reps timed launches as thread-level instructions per second.
 * Synchronous; creates and destroys its own stream and events. No counterpart in the
 * reference (a measurement of the hardware the sweeps run on). */
CASADI_GB300_API int casadi_gb300_fp64_rate(int kind, int reps, double* instr_per_s);

#ifdef __cplusplus
}
#endif

#endif /* CASADI_GB300_H */
