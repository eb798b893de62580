/*
 * rils_rols_gb300 - C ABI of the GB300 fitness path of RILS-ROLS.
 *
 * The reference evaluates one candidate at a time through two private member
 * functions of its search class:
 *     tune_constants(tree, X, y) -> tree      rils_rols_cpp/rils_rols_cpp.cpp:445-518
 *     fitness(tree, X, y) -> (1-R2, RMSE, size) rils_rols_cpp/rils_rols_cpp.cpp:520-541
 * both driving the recursive evaluator node::evaluate_all (rils_rols_cpp/node.cpp:5-95)
 * and Eigen's column-pivoted QR (rils_rols_cpp/rils_rols_cpp.cpp:484).
 * This ABI replaces that pair with a batched call: the host flattens every
 * candidate of one local-search round into postfix programs (one program per
 * top-level factor, see rrg_op below) and submits them together; the device
 * evaluates the factors, refits the linear coefficients and returns the
 * fitness tuple of the rebuilt tree for every candidate.
 *
 * Plain pointers and sizes only; every call returns an rrg_status.  No call
 * exits the process (the reference calls exit(1) on bad input,
 * rils_rols_cpp.cpp:722-725).
 */
#ifndef RILS_ROLS_GB300_H
#define RILS_ROLS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RRG_ABI_VERSION 1
#define RRG_MAX_TERMS 64   /* factors + free term of one tuned candidate */
#define RRG_MAX_STACK 16   /* spill-stack depth of one factor program */

typedef enum {
  RRG_OK = 0,
  RRG_E_INVALID = 1,      /* bad argument or malformed batch */
  RRG_E_CUDA = 2,         /* CUDA runtime error (message via rrg_last_error) */
  RRG_E_NO_DEVICE = 3,    /* no usable GB300 device / extension not loaded */
  RRG_E_TIMEOUT = 4,      /* bounded wait ran out; the context stays usable */
  RRG_E_TOO_LARGE = 5,    /* a candidate exceeds RRG_MAX_TERMS or RRG_MAX_STACK */
  RRG_E_OOM = 6,          /* device memory budget exceeded */
  RRG_E_DEVICE_FAULT = 7  /* a kernel reported an error status (bounded wait, bad code) */
} rrg_status;

/* Arithmetic of one round. */
typedef enum {
  RRG_PLAIN_FP64 = 0,        /* FP64 evaluation, column-pivoted Householder OLS, FP64 residual */
  RRG_MIXED = 1,             /* double-float (FP32-pair) evaluation of the round's distinct factors, Gram sums
                                per distinct factor pair, FP64 pivoted Cholesky + refinement; non-finite and
                                ill-conditioned systems re-solved by the FP64 path */
  RRG_MIXED_CERTIFIED = 2    /* RRG_MIXED, and every result whose fitness error cannot be bounded below
                                5e-7 relative (or whose rank / drop / snap decision is ambiguous) is
                                re-scored by the FP64 path: results equal the FP64 path's within 1e-6 */
} rrg_precision;

/* How one candidate is scored. */
typedef enum {
  RRG_UNTUNED = 0,  /* fitness(tree): yp = factor 0 (the whole tree), rils_rols_cpp.cpp:520-541 */
  RRG_TUNED = 1     /* fitness(tune_constants(tree)): OLS over [factors..., 1] then the rebuilt sum */
} rrg_mode;

/* Result flag bits. */
#define RRG_F_NONFINITE      0x1u   /* R2 or RMSE was NaN: the (1000,1000,1000) sentinel was returned */
#define RRG_F_RANK_DEFICIENT 0x2u   /* numerical rank < number of columns */
#define RRG_F_QR_FALLBACK    0x4u   /* mixed round: ill-conditioned Gram, re-solved by the FP64 QR path */
#define RRG_F_VERIFIED_FP64  0x8u   /* mixed round: re-scored by the FP64 path (argbest verification) */
#define RRG_F_TOO_LARGE      0x10u  /* candidate rejected: RRG_MAX_TERMS / RRG_MAX_STACK exceeded */

/*
 * Postfix code.  One 32-bit word per instruction: low 8 bits opcode, high 24
 * bits argument (feature index, constant-pool index or factor slot).
 * The evaluator keeps the top of stack (TOS) in registers and spills older
 * values to a per-thread stack.  Binary operators take their second operand
 * from the spill stack (S), a feature column (V) or the constant pool (C);
 * the direction bit says whether TOS is the right (N) or the left (R) operand:
 *     N: TOS = op(other, TOS)      R: TOS = op(TOS, other)
 * Element-wise semantics are those of node::evaluate_inner (node.cpp:23-95).
 */
enum rrg_op {
  RRG_OP_LDV = 1,   /* TOS = X[arg] */
  RRG_OP_LDC = 2,   /* TOS = K[arg] */
  RRG_OP_PSV = 3,   /* spill TOS; TOS = X[arg] */
  RRG_OP_PSC = 4,   /* spill TOS; TOS = K[arg] */
  RRG_OP_SIN = 5, RRG_OP_COS = 6, RRG_OP_LN = 7, RRG_OP_EXP = 8, RRG_OP_SQRT = 9, RRG_OP_SQR = 10,
  RRG_OP_EMIT = 11, /* factor slot arg = TOS; the stack is empty afterwards */
  RRG_OP_BIN = 16   /* binary: RRG_OP_BIN + 8*base + 2*src + dir */
};
enum rrg_bin_base { RRG_ADD = 0, RRG_SUB, RRG_MUL, RRG_DIV, RRG_POW, RRG_LT, RRG_EQ, RRG_NE, RRG_MIN, RRG_MAX, RRG_N_BASE };
enum rrg_bin_src { RRG_SRC_S = 0, RRG_SRC_V = 1, RRG_SRC_C = 2 };
enum rrg_bin_dir { RRG_DIR_N = 0, RRG_DIR_R = 1 };
#define RRG_BIN_OP(base, src, dir) (RRG_OP_BIN + 8 * (base) + 2 * (src) + (dir))
#define RRG_INSN(op, arg) ((uint32_t)(op) | ((uint32_t)(arg) << 8))

typedef struct {
  int32_t code_offset;  /* first instruction of the candidate (all its factors, in order) */
  int32_t code_len;     /* instructions of all its factors; each factor ends with EMIT */
  int32_t first_factor; /* index of its first rrg_factor */
  int32_t n_factors;    /* non-constant factors (tuned) or 1 (untuned) */
  int32_t mode;         /* rrg_mode */
  int32_t coef_offset;  /* tuned: n_factors + 1 coefficients written at coefs[coef_offset] */
  int32_t stack_need;   /* deepest spill of its programs (<= RRG_MAX_STACK) */
  int32_t reserved;
} rrg_cand;

typedef struct {
  int32_t n_nodes;      /* node count of the factor subtree (node.h:311-322) */
  int32_t reserved;
} rrg_factor;

typedef struct {
  int32_t n_cand;
  int32_t n_factors;
  int32_t n_code;
  int32_t n_consts;
  const rrg_cand* cands;
  const rrg_factor* factors;
  const uint32_t* code;
  const double* consts;
} rrg_batch;

typedef struct {
  double loss;      /* 1 - R2 (also the classifier loss, rils_rols_cpp.cpp:526-531); 1000 on NaN */
  double rmse;      /* sqrt(mean((y - yp)^2)); 1000 on NaN */
  int32_t size;     /* node count of the rebuilt tree (tuned) or of the tree (untuned); 1000 on NaN */
  int32_t rank;     /* tuned: nonzero pivots of the OLS design; untuned: 0 */
  uint32_t flags;   /* RRG_F_* */
  int32_t n_coef;   /* tuned: n_factors + 1 (free term last); untuned: 0 */
} rrg_result;

typedef struct rrg_context rrg_context;
typedef struct rrg_dataset rrg_dataset;

/* Version of this ABI (RRG_ABI_VERSION). */
int32_t rrg_abi_version(void);

/* Text of the last error on this thread (never NULL). */
const char* rrg_last_error(void);

/* One context per device: owns a stream, pinned staging and scratch arenas.
 * Destroying a context also releases the device memory of the datasets
 * created on it; their handles stay valid for rrg_dataset_destroy only (any
 * other call on them returns RRG_E_INVALID), so the two may be destroyed in
 * either order (garbage-collected bindings cannot always choose). */
rrg_status rrg_context_create(int32_t device, rrg_context** out);
rrg_status rrg_context_destroy(rrg_context* ctx);

/*
 * Make a dataset resident on the device.  X_col is d columns of n FP64 values
 * (column-major, the layout get_x builds, rils_rols_cpp.cpp:675-698); y has n
 * values.  Both are copied; the caller keeps ownership.  The device keeps FP64
 * and FP32 copies.  Replaces the `const vector<ArrayXd>& X, const ArrayXd& y`
 * arguments of tune_constants / fitness (rils_rols_cpp.cpp:445, 520).
 */
rrg_status rrg_dataset_create(rrg_context* ctx, const double* X_col, const double* y, int64_t n, int32_t d,
                              rrg_dataset** out);
/* The same dataset from X given row-major (n rows of d values, the buffer the
 * reference's pybind fit receives before get_x splits it into columns,
 * rils_rols_cpp.cpp:675-698); the transposition runs on the device.  A pinned
 * X (or y) is copied by DMA straight from the caller's memory. */
rrg_status rrg_dataset_create_rows(rrg_context* ctx, const double* X_rows, const double* y, int64_t n, int32_t d,
                                   rrg_dataset** out);
rrg_status rrg_dataset_destroy(rrg_dataset* ds);

/*
 * Score a batch of candidates (one local-search round).  Asynchronous: the
 * batch is copied into pinned staging before the call returns, so the caller
 * may reuse its buffers at once; `results` (n_cand entries) and `coefs` (the
 * sum of n_coef over tuned candidates, may be NULL) are written when
 * rrg_round_wait returns RRG_OK.  One round in flight per context.  The
 * call returns once every launch of the round is queued: it waits on the
 * device only for a launch-shape trial (the first launch of a shape class,
 * see rrg_tune_set_mode) and for mixed rounds that need table sub-rounds or
 * run with rrg_context_set_async off.
 * Replaces, per candidate j: tune_constants (rils_rols_cpp.cpp:615) followed
 * by fitness (:616), or fitness alone (:828, :842) for RRG_UNTUNED.
 */
rrg_status rrg_round_submit(rrg_dataset* ds, const rrg_batch* batch, int32_t precision, rrg_result* results,
                            double* coefs);
/* Bounded wait for the round in flight; RRG_E_TIMEOUT leaves it in flight. */
rrg_status rrg_round_wait(rrg_context* ctx, int32_t timeout_ms);

/* submit + wait (no timeout). */
rrg_status rrg_eval(rrg_dataset* ds, const rrg_batch* batch, int32_t precision, rrg_result* results,
                    double* coefs);

/*
 * Values of candidate 0 of `batch` (RRG_UNTUNED, one factor) on every row of
 * the dataset, FP64, written to values[n].  Replaces
 * final_solution->evaluate_all(X) in predict (rils_rols_cpp.cpp:738).
 */
rrg_status rrg_predict(rrg_dataset* ds, const rrg_batch* batch, double* values);

/*
 * Allocation-free scoring of one candidate (batch->n_cand == 1) by the plain
 * FP64 path, for callers that may not allocate device memory or have a
 * library allocate it for them (a framework that owns every device byte
 * through its own pool; a loop that cannot take cudaMalloc / cudaFree
 * stalls).  It has no counterpart in the reference.  It scores one tuned or
 * untuned candidate on data the caller already holds on the device, with no
 * context or dataset object.
 *   X_col: device, d columns of ld >= n FP64 values (column j at X_col + j*ld);
 *   y: device, n values; result: device, one rrg_result; coefs: device,
 *   n_factors + 1 doubles for a tuned candidate (may be NULL when untuned);
 *   batch: host; stream: a cudaStream_t (NULL = legacy default stream).
 * Runs on the current device and returns after the stream has finished it.
 * Scratch is a fixed 32 MiB device array inside the library (about
 * (2k + 1) * ld * 8 bytes are needed for k = n_factors + 1); a larger call
 * returns RRG_E_TOO_LARGE and allocates nothing.  The first call on each
 * device looks up the scratch address: make it before any stream capture
 * begins on that device.  Calls share the scratch, so calls that overlap on
 * a device race: serialise them.  Results equal rrg_eval(RRG_PLAIN_FP64) on
 * the same data bit for bit (the same QR in the same summation order).
 */
rrg_status rrg_eval_plain_noalloc(const double* X_col, int64_t ld, const double* y, int64_t n, int32_t d,
                                  const rrg_batch* batch, rrg_result* result, double* coefs, void* stream);

/* Host-side check of a batch against a dataset of d features: opcodes,
 * feature / constant / slot indices and spill depths.  rrg_round_submit runs
 * the same check; no device is needed. */
rrg_status rrg_batch_validate(const rrg_batch* batch, int32_t d);

/* Rows and columns of a dataset. */
int64_t rrg_dataset_rows(const rrg_dataset* ds);
int32_t rrg_dataset_cols(const rrg_dataset* ds);

/* Kernels launched by the last completed round on this context (for audits). */
int64_t rrg_last_round_launches(const rrg_context* ctx);

/* Statistics of the last completed round, written to out[0..n):
 *   [0] kernels launched   [1] candidates routed to the FP64 path (beyond the
 *   mixed kernels' limits)  [2] mixed candidates re-scored by the FP64 path
 *   [3] candidates that needed the residual pass  [4..14] re-scoring reasons:
 *   FP32/FP64 non-finite mismatch on a probe row, FP64 overflow, FP32
 *   overflow, NaN factor beside a rank-deficient rest, rank cut,
 *   ill-conditioning, coefficient near 1, coefficient near 0, one-pass SSE
 *   inaccurate, certified error bound too large, other NaN.  [15] FP64-path
 *   candidates whose pivoted QR was not run: a non-finite column norm makes its
 *   outcome certainly all-NaN coefficients (the fitness sentinel).  [16]
 *   candidates scored after merging those with identical factor lists.
 *   [17] 0 (formerly a tiled-QR flag: every round now solves by the direct
 *   column-pivoted QR, bit-identical to the oracle).  [18] 1 when the last
 *   round ran as a CUDA graph (rrg_context_set_graph).  [19] double-float
 *   factor columns read from the column cache (rrg_context_set_column_cache)
 *   [20] double-float table columns evaluated  [21] FP64 factor columns read
 *   from the column cache  [22] FP64 table columns evaluated  [23] cross-pair
 *   sums read from the column cache  [24] cross-pair sums formed.
 * Returns the count written. */
int32_t rrg_last_round_stats(const rrg_context* ctx, int64_t* out, int32_t n);

/* Device-memory limits of this context's scratch: FP64 tables and QR working
 * columns (scratch_bytes) and the mixed rounds' double-float factor table
 * (table_bytes).  By default they are set from the free memory at creation;
 * several contexts on one device (the serving loop) set them explicitly.
 * No counterpart in the reference (single-threaded, one fit per process). */
rrg_status rrg_context_set_limits(rrg_context* ctx, int64_t scratch_bytes, int64_t table_bytes);

/* Keep factor columns on the device across rounds (on by default).  A
 * factor column is a function of the factor's program (constants by value)
 * and of the dataset alone, and the consecutive rounds of a search share
 * most factors, so a round reads the columns an earlier round on the same
 * dataset evaluated instead of evaluating them again: the double-float
 * columns of mixed rounds (with their sums, probe records and cross-pair
 * sums) and the FP64 columns of FP64 rounds and of the mixed rounds' FP64
 * re-scoring, within the limits of rrg_context_set_limits, least
 * recently used columns replaced first.  Datasets of fewer than 8192 rows
 * do not use it (there evaluating a column costs less than finding it).
 * Results are the same bits either way.  Switching clears what is kept; so
 * do destroying the dataset, a round on another dataset and a failed round.
 * RRG_E_INVALID while a round is in flight.  No counterpart in the
 * reference. */
rrg_status rrg_context_set_column_cache(rrg_context* ctx, int32_t on);
/* Forget every kept column (the next round evaluates all its factors);
 * RRG_E_INVALID while a round is in flight. */
rrg_status rrg_context_clear_column_cache(rrg_context* ctx);

/* How a mixed or certified round decides its second half.  On (the
 * default): on the device, from the solve's flags (the residual-pass list,
 * which candidates the FP64 path re-scores, which table columns it
 * evaluates), so that rrg_round_submit returns with the whole round queued
 * and the host reads nothing back before the results.  Off: the host reads
 * the flags back twice in mid-round and builds the FP64 path's programs for
 * the re-scored candidates only.  Results are the same bits either way; a
 * round whose double-float table needs sub-rounds always takes the second
 * form, and so does a round of fewer than 64 mixed candidates when rounds
 * do not run as graphs (its read-back costs less than the device-decided
 * lane's launches).  RRG_E_INVALID while a round is in flight.  No counterpart in the
 * reference. */
rrg_status rrg_context_set_async(rrg_context* ctx, int32_t on);

/* Run every round as a CUDA graph (off by default): the round's launches,
 * copies and stream forks are captured from the context stream and launched
 * as one graph, the previous round's graph updated in place when the shapes
 * allow (rrg_last_round_stats [18] tells whether the last round ran so).  A
 * round that waits on the device in mid-round (a launch-shape trial, table
 * sub-rounds, rrg_context_set_async off) cannot be captured and is launched
 * directly; so are rounds with per-phase timing on.  Results are the same
 * bits either way.  RRG_E_INVALID while a round is in flight.  No
 * counterpart in the reference. */
rrg_status rrg_context_set_graph(rrg_context* ctx, int32_t on);

/* Rounds in RRG_MIXED / RRG_MIXED_CERTIFIED on datasets with fewer than
 * `rows` rows (default 8192) are computed in FP64 instead: there the mixed
 * form's probes, pair sums and read-backs cost more than the FP64 arithmetic
 * they replace, and FP64 results meet any certified bound.  0 always takes
 * the mixed form.  No counterpart in the reference. */
rrg_status rrg_context_set_mixed_min_rows(rrg_context* ctx, int64_t rows);

/* Device bytes a context's scratch holds (the buffers only grow; datasets
 * not included), or -1 for NULL.  For callers that keep a context across
 * jobs and account its memory (the serving loop).  No counterpart in the
 * reference. */
int64_t rrg_context_memory(rrg_context* ctx);

/* Free and total memory of a device (cudaMemGetInfo); RRG_E_NO_DEVICE without
 * one.  No counterpart in the reference. */
rrg_status rrg_device_memory(int32_t device, int64_t* free_bytes, int64_t* total_bytes);

/* The CUDA stream (cudaStream_t) every kernel of this context runs on, so that
 * a caller can order or time its own work against the rounds. */
void* rrg_context_stream(const rrg_context* ctx);

/* Per-phase device timing of later rounds (CUDA events around every launch on
 * the context stream); off by default. */
rrg_status rrg_context_set_timing(rrg_context* ctx, int32_t on);
/* Device milliseconds and launch counts of the last completed round, per
 * phase: [0] mixed factor-table evaluation (with the self sums), [1] mixed
 * solve (pair totals, probes, Cholesky), [2] mixed residual pass,
 * [3] finalize, [4] FP64 evaluation, [5] FP64 QR, [6] FP64 residual,
 * [7] mixed pair sums.  Returns the number of phases written. */
int32_t rrg_last_round_timing(const rrg_context* ctx, double* ms, int64_t* launches, int32_t n);
/* Algorithmic device-memory bytes of the last completed round, per phase (the
 * phases of rrg_last_round_timing): [0] X and y read once plus the
 * double-float table written once (8 B per row and column); [4] X read once
 * plus the FP64 table written once; [5] per factorised candidate with K
 * columns [A | 1 | y], the copy (K - 2 factor columns and y read, K written)
 * and, per step, every remaining column read and written once; [7] every
 * table column read once.  Phases without a count read 0.  Returns the
 * number of phases written.  No counterpart in the reference. */
int32_t rrg_last_round_bytes(const rrg_context* ctx, double* bytes, int32_t n);

/* Launch-shape tuner.  Only launch shapes that leave every result bit
 * unchanged are tuned: the FP64 evaluator's blocks per level launch in SM
 * waves (RRG_KNOB_EVAL_WAVES; bucket 0), and in mixed rounds the
 * double-float evaluator's factors per block (RRG_KNOB_FAC_GROUP: 64, 32,
 * 16; bucket 0) and the pair sums' partners per block (RRG_KNOB_PAIR_UNIT:
 * 65536, 512, 128; bucket 0) -- every factor's values and every pair's sum
 * are formed alone, whatever shares its block -- and whether that evaluator
 * reads X and y from global memory (1) or stages each block's rows of them
 * in shared memory by tensor copies (2) (RRG_KNOB_FAC_STAGE; bucket: the
 * feature count d, 1..64).  Knobs 0 and 5 (the warps per CTA of an earlier
 * cluster QR) are retired: the QR's passes have one shape.  With
 * RRG_TUNE_ON (the default) the first launch of a (knob, bucket, row class
 * floor(log2 n)) that carries enough work is timed in every shape, and the
 * fastest is kept for the process (and in the file named by the environment
 * variable RRG_TUNE_CACHE, when set); RRG_TUNE_OFF uses the built-in shapes.
 * No counterpart in the reference. */
#define RRG_TUNE_OFF 0
#define RRG_TUNE_ON 1
#define RRG_KNOB_EVAL_WAVES 1
#define RRG_KNOB_FAC_GROUP 2
#define RRG_KNOB_PAIR_UNIT 3
#define RRG_KNOB_FAC_STAGE 4
rrg_status rrg_tune_set_mode(int32_t mode);
/* Fix a knob's value in a bucket (value 0 releases it); RRG_E_INVALID for a
 * knob, bucket or value the kernels are not built for. */
rrg_status rrg_tune_pin(int32_t knob, int32_t bucket, int32_t value);
/* Forget every tuned choice and pin. */
rrg_status rrg_tune_reset(void);
/* The tuner's choices as text, one line per (knob, bucket, row class) with the
 * timed shapes ("fac_group bucket=0 row_class=19 value=16 ms=64:2.5,32:2.3,16:2.1"),
 * then the pins.  Writes at most cap bytes (NUL-terminated) and returns the
 * size needed. */
int64_t rrg_tune_report(char* buf, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
