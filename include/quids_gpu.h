/*
 * quids_gpu.h -- C ABI of the GB300-native QuIDS rule step.
 *
 * This library replaces, on one GPU, the two entry points of the reference
 * header-only library (jolatechno/QuIDS):
 *
 *   void quids::simulate(it_t &iteration, rule_t const *rule, it_t &next_iteration,
 *                        sy_it_t &symbolic_iteration, size_t max_num_object, debug_t)
 *                                                           src/quids.hpp:448-543
 *   void quids::simulate(it_t &iteration, modifier_t const rule)
 *                                                           src/quids.hpp:436-438
 *
 * The state (`it_t`, src/quids.hpp:149-335) lives in device memory as the same
 * packed structure of arrays: object bytes with every object padded to
 * align_byte_length (get_alignment_offset, src/quids.hpp:93-102), u64 begin
 * offsets (n+1), u32 sizes and complex<double> magnitudes (interleaved re, im).
 *
 * All calls return QUIDS_OK (0) or a negative status; no call throws, traps
 * the GPU or exits the process.  A context owns one CUDA stream and its
 * scratch memory; contexts are independent, a context is not thread-safe.
 */
#ifndef QUIDS_GPU_H
#define QUIDS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define QUIDS_OK 0
#define QUIDS_ERR_BAD_ARG (-1)              /* null/aliased handles, unknown kind */
#define QUIDS_ERR_OOM (-2)                  /* device allocation failed */
#define QUIDS_ERR_TABLE_FULL (-3)           /* collision table probe limit reached */
#define QUIDS_ERR_CHILD_COUNT_OVERFLOW (-4) /* a parent's child count does not fit u32 */
#define QUIDS_ERR_SIZE_BOUND (-5)           /* a child larger than the rule's max_child_size */
#define QUIDS_ERR_TIMEOUT (-6)              /* a bounded device wait gave up */
#define QUIDS_ERR_CUDA (-7)                 /* a CUDA runtime call failed */
#define QUIDS_ERR_NO_DEVICE (-8)            /* no CUDA device */
#define QUIDS_ERR_UNSUPPORTED (-9)          /* valid request this library does not implement */
#define QUIDS_ERR_NOALLOC_LIMIT (-10)       /* beyond the static scratch of quids_gpu_rule_children_noalloc */

/* ------------------------------------------------------- rules/modifiers */
/* rules (classes derived from quids::rule, src/quids.hpp:105-146) */
#define QUIDS_RULE_HADAMARD 1            /* quantum_computer::hadamard  src/rules/quantum_computer.hpp:31-50 */
#define QUIDS_RULE_QCGD_ERASE_CREATE 2   /* qcgd::erase_create          src/rules/qcgd.hpp:459-532 */
#define QUIDS_RULE_QCGD_COIN 3           /* qcgd::coin                  src/rules/qcgd.hpp:534-605 */
#define QUIDS_RULE_QCGD_SPLIT_MERGE 4    /* qcgd::split_merge           src/rules/qcgd.hpp:607-1036 */

/* modifiers (modifier_t, src/quids.hpp:86) */
#define QUIDS_MOD_CNOT 1                 /* quantum_computer::cnot   src/rules/quantum_computer.hpp:25-29 */
#define QUIDS_MOD_X 2                    /* quantum_computer::Xgate  :52-56 */
#define QUIDS_MOD_Y 3                    /* quantum_computer::Ygate  :58-66 */
#define QUIDS_MOD_Z 4                    /* quantum_computer::Zgate  :68-75 (negates AND flips) */
#define QUIDS_MOD_QCGD_STEP 5            /* qcgd::step               src/rules/qcgd.hpp:443-449 */
#define QUIDS_MOD_QCGD_REVERSED_STEP 6   /* qcgd::reversed_step      src/rules/qcgd.hpp:451-457 */

/* Parameters of a rule or modifier.  Unused fields are ignored.
 *   HADAMARD: bit            X/Y/Z: bit            CNOT: control, bit
 *   QCGD rules: theta, phi, xi (constructor arguments of the reference rules;
 *   do = polar(sin theta, phi), do_not = polar(cos theta, xi) are formed on
 *   the host exactly as src/rules/qcgd.hpp:466-471 does). */
typedef struct quids_gpu_rule_params {
    uint64_t bit;
    uint64_t control;
    double theta;
    double phi;
    double xi;
} quids_gpu_rule_params;

/* Knobs of one rule step: the reference's globals (src/quids.hpp:59-75) and
 * the max_num_object argument of simulate(). */
typedef struct quids_gpu_params {
    double tolerance;            /* quids::tolerance: keep children with norm > tolerance */
    uint64_t max_num_object;     /* UINT64_MAX = no cap ("-1"); 0 = automatic: as many as fit the
                                    device memory (free memory + what the context holds, less 20%),
                                    or memory_budget when set */
    int32_t simple_truncation;   /* 1: keep the largest norms; 0: probabilistic truncation (keep the
                                    smallest u / norm, u uniform from a generator seeded by `seed`) */
    uint32_t align_byte_length;  /* quids::align_byte_length for the output state */
    double table_load_factor;    /* collision table max load; 0 -> default 0.5 */
    uint32_t hash_ranges;        /* 0: one pass when the children fit (2^32 child indices, device memory),
                                    else as many hash-range passes as they need; k >= 2: at least k
                                    passes.  Range passes give the one-pass result bit for bit; the
                                    automatic truncation (max_num_object = 0) never uses them (it
                                    keeps fewer parents until one pass fits), nor does the adjoint
                                    forward (QUIDS_ERR_UNSUPPORTED) */
    uint32_t flags;              /* QUIDS_FLAG_* */
    uint64_t seed;               /* probabilistic truncation: generator seed (same seed and input,
                                    same result) */
    uint64_t memory_budget;      /* automatic truncation: bytes a step may use (0: from the device) */
    uint32_t max_probes;         /* collision-table probe limit (0: 65536); a child whose probe sequence
                                    reaches it stops the step with QUIDS_ERR_TABLE_FULL */
    uint32_t debug_flags;        /* QUIDS_DEBUG_*: failure injection for tests of the error paths; 0 */
    uint64_t max_alloc_bytes;    /* 0: no limit; else a device allocation of more bytes than this, by
                                    the step's scratch or its output, fails with QUIDS_ERR_OOM before
                                    cudaMalloc is called (a cap on what one call may grow to) */
} quids_gpu_params;

/* quids_gpu_params.debug_flags.  Each makes a bounded device wait run out on
 * purpose: the wait gives up after its poll limit (well under a second),
 * records QUIDS_ERR_TIMEOUT, and the call returns that status with the
 * context still usable.  Nothing faults, traps or hangs. */
#define QUIDS_DEBUG_STALL_LOOKBACK 1u  /* tile 1 of the child-offset scan never publishes its prefix, so
                                          the look-back of tile 2 waits for it until its poll limit */

/* quids_gpu_params.flags */
#define QUIDS_FLAG_NO_FAST_HASH 1u   /* hash children through populate_child + hasher, not hash_child */
#define QUIDS_FLAG_STAGE_TIMING 2u   /* record per-stage CUDA events and synchronise at the end of the
                                        step, so stats carries timings and total_proba */
#define QUIDS_FLAG_TABLE 4u          /* group colliding children in the open-addressing table in device memory
                                        (the default; the batched form and the adjoint's forward always use it) */
#define QUIDS_FLAG_PARTITION 8u      /* one-pass steps group colliding children by partition into per-block
                                        shared-memory tables instead (collide.cuh); the same result bits */
#define QUIDS_FLAG_NO_PLAN 16u       /* quids_gpu_run: always the synchronous steps (no planned run, no graph) */
#define QUIDS_FLAG_AUTOTUNE 32u      /* quids_gpu_run / quids_gpu_run_batched: before a planned run is first captured
                                        as a CUDA graph, time it under several launch configurations (collision-table
                                        load factor, table-pass block size, blocks per SM) and keep the fastest;
                                        every configuration gives the same result bits */

/* Counters of one rule step (the reference's public counters plus timing). */
typedef struct quids_gpu_step_stats {
    uint64_t num_parents;                    /* iteration.num_object */
    uint64_t num_parents_kept;               /* after parent pre-truncation */
    uint64_t num_object;                     /* symbolic_iteration.num_object (children) */
    uint64_t num_object_after_interferences; /* symbolic_iteration.num_object_after_interferences */
    uint64_t num_object_out;                 /* next_iteration.num_object */
    uint64_t max_child_size;                 /* max over parents of get_num_child's bound */
    uint64_t table_capacity;                 /* collision table slots */
    uint64_t out_bytes;                      /* object bytes of next_iteration */
    double total_proba;                      /* next_iteration.total_proba (before normalisation);
                                                NaN unless QUIDS_FLAG_STAGE_TIMING (read it from the state) */
    double algorithmic_bytes;                /* compulsory HBM traffic of this step */
    float ms_total;                          /* device time of the step (QUIDS_FLAG_STAGE_TIMING) */
    /* device time per stage (CUDA events bracketing each stage's launches,
     * QUIDS_FLAG_STAGE_TIMING only): 0 num_child + parent truncation + child
     * offsets, 1 symbolic iteration, 2 collision table (claim + accumulate),
     * 3 group compaction (+ output layout when no truncation is possible),
     * 4 truncation (select + compaction with output layout), 5 total
     * probability, 6 finalize populate with normalisation, 7 unused */
    float stage_ms[8];
    uint64_t kernel_launches;                /* kernels this step launched */
    uint64_t hash_ranges;                    /* hash-range passes the step ran in (0: one pass; the
                                                stage times of range passes are summed over the passes,
                                                stage 4 includes the merge and final selection) */
} quids_gpu_step_stats;

/* The outcome of the most recent autotuning (QUIDS_FLAG_AUTOTUNE) in a context. */
typedef struct quids_gpu_tuning {
    double table_load_factor;   /* chosen collision-table load factor */
    uint32_t table_block;       /* chosen block size of the collision-table passes */
    uint32_t blocks_per_sm;     /* chosen grid size of the grid-stride kernels, in blocks per SM */
    float ms_default;           /* run time (CUDA events, best of 3) under the default configuration */
    float ms_tuned;             /* run time under the chosen configuration */
    uint32_t trials;            /* configurations timed */
    uint32_t pad;
} quids_gpu_tuning;

typedef struct quids_gpu_ctx quids_gpu_ctx;
typedef struct quids_gpu_state quids_gpu_state;

/* ---------------------------------------------------------------- context */
int quids_gpu_ctx_create(int device, quids_gpu_ctx **out);
int quids_gpu_ctx_destroy(quids_gpu_ctx *ctx);
/* the cudaStream_t every call of this context is ordered on */
void *quids_gpu_ctx_stream(quids_gpu_ctx *ctx);
int quids_gpu_ctx_synchronize(quids_gpu_ctx *ctx);
/* bytes of device scratch memory currently held by the context */
uint64_t quids_gpu_ctx_scratch_bytes(quids_gpu_ctx *ctx);
/* release the context's scratch memory */
int quids_gpu_ctx_trim(quids_gpu_ctx *ctx);
const char *quids_gpu_status_string(int status);
/* number of kernels launched by this context since its creation */
uint64_t quids_gpu_ctx_launch_count(quids_gpu_ctx *ctx);
/* how the context's quids_gpu_run calls ran: synchronous steps (two host
 * waits per rule step), planned (one host wait per run), and of the planned
 * ones, replays of a captured CUDA graph.  Any pointer may be NULL. */
int quids_gpu_ctx_run_counts(quids_gpu_ctx *ctx, uint64_t *sync_runs, uint64_t *planned_runs, uint64_t *graph_runs);
/* the most recent autotuning of this context (all zero if none ran) */
int quids_gpu_ctx_last_tuning(quids_gpu_ctx *ctx, quids_gpu_tuning *out);

/* ----------------------------------------------------------------- states
 * A state is the device-resident `it_t`.  Handles are not copyable;
 * `next_iteration` must be a different handle from `iteration`
 * (src/quids.hpp:443, it_t has no copy semantics). */
int quids_gpu_state_create(quids_gpu_ctx *ctx, quids_gpu_state **out);
int quids_gpu_state_destroy(quids_gpu_state *st);
/* Host -> device.  object i = objects[begin[i] .. begin[i] + size[i]);
 * magnitude = 2 n doubles; num_bytes = bytes of `objects` to copy (begin[n]).
 * The layout is kept as given (offsets need not follow the alignment). */
int quids_gpu_state_upload(quids_gpu_state *st, uint64_t num_object, const uint8_t *objects,
                           const uint64_t *begin, const uint32_t *size, const double *magnitude,
                           uint64_t num_bytes);
int quids_gpu_state_num_object(const quids_gpu_state *st, uint64_t *num_object);
int quids_gpu_state_num_bytes(const quids_gpu_state *st, uint64_t *num_bytes);
int quids_gpu_state_total_proba(const quids_gpu_state *st, double *total_proba);
/* Device -> host into caller buffers sized from num_object / num_bytes
 * (begin has num_object + 1 entries).  Any pointer may be NULL to skip it. */
int quids_gpu_state_download(quids_gpu_state *st, uint8_t *objects, uint64_t *begin,
                             uint32_t *size, double *magnitude);
/* No counterpart in the reference (its states live in host memory).  The
 * copies of quids_gpu_state_download, issued on the context's copy stream
 * after the work already issued on the context: the call returns at once,
 * so a loop can download one step's result while the next step runs.  The
 * host buffers must stay valid, and should be pinned (page-locked) for the
 * copies to overlap anything.  Until quids_gpu_state_download_wait(st)
 * returns, the buffers are not complete.  Work that writes the state
 * (upload, simulate, run, modifiers, a tape's final state) waits for the
 * copies on the device, so it cannot overwrite what is still being read. */
int quids_gpu_state_download_async(quids_gpu_state *st, uint8_t *objects, uint64_t *begin,
                                   uint32_t *size, double *magnitude);
int quids_gpu_state_download_wait(quids_gpu_state *st);
/* Device pointers of the state's arrays (valid until the next call that
 * writes the state). */
int quids_gpu_state_device_arrays(quids_gpu_state *st, void **objects, void **begin, void **size,
                                  void **magnitude);

/* ------------------------------------------------------------- the step */
/* quids::simulate(iteration, rule, next_iteration, symbolic_iteration,
 * max_num_object)  src/quids.hpp:448-543.  `stats` may be NULL. */
int quids_gpu_simulate(quids_gpu_ctx *ctx, quids_gpu_state *iteration, int rule_kind,
                       const quids_gpu_rule_params *rule, quids_gpu_state *next_iteration,
                       const quids_gpu_params *params, quids_gpu_step_stats *stats);

/* quids::simulate(iteration, modifier)  src/quids.hpp:436-438 -> apply_modifier
 * src/quids.hpp:973-980: in place, sizes unchanged, no normalisation. */
int quids_gpu_apply_modifier(quids_gpu_ctx *ctx, quids_gpu_state *iteration, int modifier_kind,
                             const quids_gpu_rule_params *modifier);

/* A loop of quids::simulate calls in one call: ops are applied in order,
 * modifiers in place (src/quids.hpp:436) and rules from the current state
 * into the other of the two handles (src/quids.hpp:448), the ping-pong of the
 * reference's examples (examples/quantum_computer_test.cpp:26-49).  The
 * final state is *a (*final_index = 0) or *b (1).  rule_stats, if not NULL,
 * receives one entry per rule op, in order. */
typedef struct quids_gpu_op {
    int32_t is_rule;              /* 1: rule (QUIDS_RULE_*), 0: modifier (QUIDS_MOD_*) */
    int32_t kind;
    quids_gpu_rule_params params;
} quids_gpu_op;
int quids_gpu_run(quids_gpu_ctx *ctx, quids_gpu_state *a, quids_gpu_state *b, const quids_gpu_op *ops,
                  uint64_t n_ops, const quids_gpu_params *params, quids_gpu_step_stats *rule_stats,
                  int *final_index);

/* ------------------------------------------------------------ batched form
 * No counterpart in the reference, which steps one state per call: the
 * loop `for each instance: quids::simulate(...)` over many independent
 * states (different graphs, different angles), in one pipeline per step.
 * A batched state holds n_inst instances, each a contiguous run of objects
 * [inst_begin[g], inst_begin[g+1]).  quids_gpu_simulate_batched applies, to
 * every instance g, quids::simulate with rule parameters rules[g] and the
 * same params (max_num_object caps every instance; 0, the memory-driven cap,
 * is QUIDS_ERR_UNSUPPORTED here), and normalises each instance by its own
 * total probability (its value before normalisation is returned by
 * quids_gpu_state_instances).  Each instance's survivors and magnitudes are
 * those of quids_gpu_simulate on that instance alone (magnitudes within the
 * 1e-12 relative tolerance of the normalisation sums); the probabilistic
 * truncation draws differ.  Modifiers (quids_gpu_apply_modifier) act on
 * every object and keep the instances.  A plain step of a batched state
 * gives a plain state. */
#define QUIDS_MAX_INSTANCES 65536u
int quids_gpu_state_upload_batched(quids_gpu_state *st, uint64_t num_object, const uint8_t *objects,
                                   const uint64_t *begin, const uint32_t *size, const double *magnitude,
                                   uint64_t num_bytes, uint32_t n_inst, const uint64_t *inst_begin);
/* *n_inst = 0 for a plain state.  inst_begin (n_inst + 1 entries) and
 * inst_total (n_inst) may be NULL. */
int quids_gpu_state_instances(quids_gpu_state *st, uint32_t *n_inst, uint64_t *inst_begin, double *inst_total);
/* rules: n_inst entries.  inst_stats: NULL or 3 * n_inst entries, per instance
 * {symbolic num_object, num_object_after_interferences, survivors}. */
int quids_gpu_simulate_batched(quids_gpu_ctx *ctx, quids_gpu_state *iteration, int rule_kind,
                               const quids_gpu_rule_params *rules, quids_gpu_state *next_iteration,
                               const quids_gpu_params *params, uint64_t *inst_stats,
                               quids_gpu_step_stats *stats);
/* quids_gpu_run over a batched state: rule op r takes its per-instance
 * parameters from inst_params + r * n_inst (or op.params for every instance
 * when inst_params is NULL); modifiers take op.params. */
int quids_gpu_run_batched(quids_gpu_ctx *ctx, quids_gpu_state *a, quids_gpu_state *b, const quids_gpu_op *ops,
                          uint64_t n_ops, const quids_gpu_rule_params *inst_params, const quids_gpu_params *params,
                          quids_gpu_step_stats *rule_stats, int *final_index);

/* ------------------------------------------------------ rule-level access
 * Materialises every child of every parent of `iteration` (the symbolic
 * iteration of src/quids.hpp:647-721 with the child bytes kept): children
 * are numbered parent by parent, child_id ascending.  Call once with
 * child_bytes = NULL to get *num_children and *bytes_needed (children are
 * packed at stride max_child_size rounded up to 8); then with buffers of
 * those sizes.  hash / size / magnitude get one entry per child. */
int quids_gpu_rule_children(quids_gpu_ctx *ctx, quids_gpu_state *iteration, int rule_kind,
                            const quids_gpu_rule_params *rule, uint64_t *num_children,
                            uint64_t *stride, uint8_t *child_bytes, uint64_t *hash,
                            uint32_t *size, double *magnitude);

/* No counterpart in the reference.  The children enumeration of
 * quids_gpu_rule_children for callers that must not allocate device memory:
 * code whose device memory is all owned by another allocator (a pool or a
 * fixed per-process budget that a stray cudaMalloc would break) and code that
 * cannot pay the implicit device synchronisation of cudaMalloc/cudaFree.  It
 * needs no context and allocates nothing; the caller passes device pointers
 * to the input state (as quids_gpu_state_device_arrays gives them) and to the
 * outputs, and a stream.  Its scratch is a static device array of
 * QUIDS_NOALLOC_SCRATCH_BYTES (about 3 MiB) that every GPU loading this
 * library holds until the process exits; a state of more than
 * QUIDS_NOALLOC_MAX_PARENTS objects is rejected with QUIDS_ERR_NOALLOC_LIMIT.
 * The stream must belong to the current device (QUIDS_ERR_BAD_ARG
 * otherwise).  Every call synchronises its stream, so a call can never be
 * part of a stream capture.  Calls share the array, so calls whose GPU work
 * overlaps race on it.
 * Call with d_child_bytes = NULL to get *num_children and *stride; then with
 * capacity >= *num_children and buffers of capacity * stride bytes, capacity
 * u64 hashes, capacity u32 sizes and 2 * capacity doubles.  Synchronises the
 * stream before returning. */
#define QUIDS_NOALLOC_MAX_PARENTS (1u << 18)
#define QUIDS_NOALLOC_SCRATCH_BYTES 3147520u
int quids_gpu_rule_children_noalloc(void *stream, uint64_t num_object, const uint8_t *d_objects,
                                    const uint64_t *d_begin, const uint32_t *d_size, const double *d_magnitude,
                                    int rule_kind, const quids_gpu_rule_params *rule, uint64_t capacity,
                                    uint64_t *num_children, uint64_t *stride, uint8_t *d_child_bytes,
                                    uint64_t *d_hash, uint32_t *d_child_size, double *d_child_magnitude);

/* ------------------------------------------------------------ observables
 * iteration::average_value(observable) (src/quids.hpp:208-234):
 * sum over objects of observable(object) * |mag|^2, reduced on the GPU in a
 * fixed order.  Built-in observables: */
#define QUIDS_OBS_QCGD_NUM_NODES 1     /* graphs::num_nodes            (src/rules/qcgd.hpp:317-319) */
#define QUIDS_OBS_QCGD_NUM_NODES_SQ 2  /* num_nodes^2                  (:320-323) */
#define QUIDS_OBS_QCGD_DENSITY 3       /* (sum left + right) / 2n      (:324-333) */
#define QUIDS_OBS_QCGD_DENSITY_SQ 4    /* density^2                    (:334-343) */
#define QUIDS_OBS_QC_BIT 5             /* byte `bit` of the object is non-zero (qubit `bit` is 1) */
int quids_gpu_average_value(quids_gpu_ctx *ctx, quids_gpu_state *iteration, int observable_kind,
                            const quids_gpu_rule_params *params, double *value);

/* The statistics qcgd::utils::serialize prints (src/rules/qcgd.hpp:309-366),
 * computed on the GPU; sy_num_object / sy_num_object_after_interferences are
 * the counters of the step that produced the state.  std_dev_size follows the
 * reference's formula (sqrt of the mean square size when the variance is
 * above tolerance, :345-346). */
typedef struct quids_gpu_qcgd_stats {
    double total_proba, num_graphs, avg_size, std_dev_size, avg_density, std_dev_density, interference_ratio,
        deletion_ratio;
} quids_gpu_qcgd_stats;
int quids_gpu_qcgd_statistics(quids_gpu_ctx *ctx, quids_gpu_state *iteration, uint64_t sy_num_object,
                              uint64_t sy_num_object_after_interferences, double tolerance,
                              quids_gpu_qcgd_stats *out);

/* ---------------------------------------------------------------- adjoint
 * No counterpart in the reference.  Reverse mode through a run of rule and
 * modifier ops with respect to the rule angles (theta, phi, xi of the QCGD
 * rules), with every step's structure held fixed: the same children,
 * collisions, zero elimination and truncation as the forward run.
 *
 * quids_gpu_forward runs `ops` from `initial` (as quids_gpu_run does) and
 * records a tape: the state at the start of every segment of
 * checkpoint_every rule applications, and the rule inputs of the last
 * segment.  The final state is copied to final_out when not NULL.  Modifiers
 * must be X, CNOT, QCGD step or reversed_step (they move bytes and keep
 * magnitudes); max_num_object must not be 0 (the memory-driven cap depends
 * on free memory, so a replay could differ).
 *
 * quids_gpu_simulate_backward: loss_adjoint (2 * n doubles, n = objects of
 * the final state) is a = 2 dL/d(conj m) of a real loss L of the final
 * magnitudes m (for L = sum w_s |m_s|^2, a_s = 2 w_s m_s).  The backward
 * recomputes each segment's states from its checkpoint, replays every rule
 * step and gathers the adjoint from survivors to children to parents.
 * grad_angles receives 3 * n_ops doubles: dL/dtheta, dL/dphi, dL/dxi of
 * each op (zero for modifiers and the Hadamard rule).
 * quids_gpu_simulate_backward_observable takes L = average_value of a
 * built-in observable of the final state (QUIDS_OBS_*), computed with its
 * adjoint on the GPU, and returns L in *loss.
 * quids_gpu_observable_adjoint: L and a for one state (adjoint may be NULL). */
typedef struct quids_gpu_tape quids_gpu_tape;
int quids_gpu_tape_create(quids_gpu_ctx *ctx, quids_gpu_tape **out);
int quids_gpu_tape_destroy(quids_gpu_tape *tape);
int quids_gpu_forward(quids_gpu_ctx *ctx, quids_gpu_tape *tape, quids_gpu_state *initial, const quids_gpu_op *ops,
                      uint64_t n_ops, const quids_gpu_params *params, uint64_t checkpoint_every,
                      quids_gpu_state *final_out, quids_gpu_step_stats *rule_stats);
int quids_gpu_tape_final_state(quids_gpu_tape *tape, quids_gpu_state *out);
int quids_gpu_simulate_backward(quids_gpu_ctx *ctx, quids_gpu_tape *tape, const double *loss_adjoint,
                                double *grad_angles);
int quids_gpu_simulate_backward_observable(quids_gpu_ctx *ctx, quids_gpu_tape *tape, int observable_kind,
                                           const quids_gpu_rule_params *params, double *loss,
                                           double *grad_angles);
int quids_gpu_observable_adjoint(quids_gpu_ctx *ctx, quids_gpu_state *iteration, int observable_kind,
                                 const quids_gpu_rule_params *params, double *value, double *adjoint);

/* MurmurHash64A of libstdc++'s std::hash<std::string_view> (seed 0xc70f6907),
 * the reference's default hasher (src/quids.hpp:143-145), computed on the GPU
 * for `n` byte strings of one state.  out = n u64. */
int quids_gpu_state_hash(quids_gpu_ctx *ctx, quids_gpu_state *st, int rule_kind,
                         const quids_gpu_rule_params *rule, uint64_t *out);

#ifdef __cplusplus
}
#endif
#endif /* QUIDS_GPU_H */
