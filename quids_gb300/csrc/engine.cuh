// engine.cuh -- the GB300 rule step: device state, scratch memory, the
// templated per-rule kernels and the host orchestration of
// quids::simulate(iteration, rule, next_iteration, sy_it, max_num_object)
// (src/quids.hpp:448-543) and of apply_modifier (src/quids.hpp:973-980).
//
// A user rule is any struct with the reference's callbacks as __device__
// members (see rules_qc.cuh); `simulate_rule<Rule>` instantiates the step
// for it.
#pragma once
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>
#include <unordered_set>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/quids_gpu.h"
#include "prims.cuh"
#include "qd_common.cuh"

// --------------------------------------------------------------- buffers
struct qd_dbuf {
    void *p = nullptr;
    size_t cap = 0;
};

enum qd_buf_id {
    B_NCHILD,      // u32 [N] children per parent
    B_CBEGIN,      // u64 [NP+1] child offsets over the kept parents
    B_PIDX,        // u64 [NP] kept parents (parent pre-truncation)
    B_HASH,        // u64 [NC] child hashes
    B_CMAG,        // double2 [NC] child magnitudes
    B_CSIZE,       // u32 [NC] child sizes
    B_SLOT,        // u32 [NC] collision-table slot of each child
    B_KEYS,        // table_slot [M+1] table keys and group representatives
    B_ACC,         // u64 [4(M+1)] group magnitude sums, 128-bit fixed point
    B_UCHILD,      // u64 [NU] groups kept after zero elimination (truncation path)
    B_UMAG,        // double2 [NU]
    B_UNORM,       // u64 [NU] IEEE bits of the group norm
    B_SCHILD,      // u64 [NS] representative child of each survivor
    B_LOOKBACK,    // u64 [3 (tiles + 2)] look-back chains
    B_TILENORM,    // double [blocks] per-block partial sums of an observable
    B_RHASH,       // u64 [NC] child hashes in bucket order (partitioned collisions)
    B_RIDX,        // u32 [NC] child indices in bucket order
    B_RMAG,        // double2 [NC] child magnitudes in bucket order
    B_RSLOT,       // u32 [NC] representative of each group (partitioned collisions)
    B_NOTREP,      // u8 [NC] child is not its group's representative
    B_HASJOIN,     // u8 [NC] child's group has more than one member (for the representative)
    B_RHIST,       // u32 [2 NB] children per bucket, bucket write cursors
    B_ROFF,        // u64 [NB+1] bucket offsets
    B_RCUR,        // (unused)
    B_TILEPAR,     // u64 [tiles+1] first parent of each tile of children
    B_CPAR,        // u32 [NC] kept-parent index of each child
    B_MODSTATUS,   // int: sticky error of modifier launches (reported by the next step)
    B_LBEG,        // u64 [NP+1] leader offsets of the grouped symbolic pass
    // batched steps
    B_RULES,       // Rule [G] per-instance rules
    B_BCOUNT,      // u64 [4G] per-instance tie counts and fixed-point totals
    B_BSEL,        // select_state [G]
    B_BHIST,       // u32 [256 G] per-instance radix histograms
    B_BOFF,        // u64 [G+1] per-instance tie offsets
    B_UINST,       // u32 [NU] instance of each group kept after zero elimination
    B_UBEGIN,      // u64 [G+1] instance offsets over the groups
    B_PBEGIN,      // u64 [G+1] instance offsets over the kept parents
    B_BFACTOR,     // double [G] per-instance sqrt(total)
    B_SELCAND,     // u64 [NC/8 + 2^16] keys left in a truncation's selection after its first two digits
    B_KEEPCAND,    // u32 [NC] children selected or tied at a truncation's cutoff, in child order
    B_TILECNT,     // u32 [NC / kCandTile + 1] their count per tile of children, then u64 tile offsets
    // partitioned collision stage (collide.cuh)
    B_BITMAP,      // u32 [2 (NC/32 + 1)] survivors and cutoff ties, one bit per child
    B_BITPREFIX,   // u64 [2 (NC/32 + 1)] their popcount prefixes
    B_COUNT
};

// device words of one step (u64 each)
enum qd_word {
    W_N = 0,      // parents
    W_NP,         // kept parents
    W_NC,         // children
    W_NU,         // unique non-zero children
    W_NS,         // survivors
    W_OUTBYTES,
    W_MAXABS,     // bit pattern of max |component| over children
    W_MAXSIZE,    // max_child_size over parents
    W_STATUS,     // first error code (int)
    W_TOTAL,      // total probability (double)
    W_FACTOR,     // sqrt(total) (double)
    W_TMP,
    W_MAXNORM,    // bit pattern of the largest survivor norm
    W_ACC,        // 2 words: fixed-point total probability
    W_DONE = W_ACC + 2,  // blocks done with the total (u32)
    W_DONE_SCAN,         // blocks done with the child-offset scan (u32)
    W_DONE_LAYOUT,       // blocks done with the layout compaction (u32)
    W_FAILAPP,           // planned run: the step at which it stopped (~0: none)
    W_M,                 // planned run: collision table slots of the step
    W_SELN,              // truncation select: items of its later passes
    W_SELUSE,            // truncation select: the later passes read the kept candidates
    W_SELCNT,            // truncation select: candidates kept
    W_NTILES,            // keep layout: tiles of the candidate filter
    W_NCAND,             // keep layout: children selected or tied at the cutoff
    W_PCSNB,             // partitioned collisions: buckets
    W_PCSNW,             // partitioned collisions: bitmap words
    W_COUNT_WORDS = 32
};

namespace qd::planned {
struct run_plan;
}

// Launch knobs a planned run can be tuned over (none changes a result bit):
// the collision table's load factor (0: the step's table_load_factor), the
// block size of the table passes, and the blocks per SM of the grid-stride
// kernels.
struct qd_knobs {
    double load = 0;
    unsigned table_block = 256;
    int per_sm = 8;
};

struct quids_gpu_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    qd_dbuf buf[B_COUNT];
    uint64_t *d_words = nullptr;             // W_COUNT_WORDS
    uint64_t *h_words = nullptr;             // mapped pinned mirror: W_COUNT_WORDS words + a sequence word
    uint64_t *h_words_dev = nullptr;         // its device address
    uint64_t publish_seq = 0;
    qd::prim::select_state *d_sel = nullptr; // two states
    unsigned long long *d_hist = nullptr;    // 256
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_stage[16] = {};  // start/end of the 8 stages of a step
    // asynchronous downloads: a copy stream, ordered after `stream` by ev_copy
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copy = nullptr;
    uint64_t launches = 0;          // kernels launched by this context
    // live states: destroying the context releases their device memory and
    // orphans them, so states may be destroyed after their context
    std::unordered_set<struct quids_gpu_state *> states;
    // planned runs of quids_gpu_run (most recent last), and the mapped host
    // words their steps report into
    std::vector<qd::planned::run_plan *> plans;
    uint64_t *h_plan = nullptr, *h_plan_dev = nullptr;
    size_t h_plan_words = 0;
    uint64_t runs_sync = 0, runs_planned = 0, runs_graph = 0;
    qd_knobs tune;                    // in effect while a planned run is launched or captured
    quids_gpu_tuning last_tuning{};   // the most recent autotuning of a planned run
};

struct quids_gpu_state {
    quids_gpu_ctx *ctx = nullptr;  // null once the context is destroyed
    uint64_t n = 0;
    uint64_t nbytes = 0;
    // total probability: known on the host, or still in d_total on the device
    // (written by the last step without a host synchronisation)
    mutable double total_proba = 1;
    mutable bool total_pending = false;
    qd_dbuf objects, begin, size, mag, d_total;
    // u64 [2] {n, nbytes} on the device, written by the steps of a planned
    // run (the host fields are updated when the run ends)
    qd_dbuf meta;
    // batched state: n_inst independent instances, each a contiguous run of
    // objects (inst: instance of each object; inst_begin: u64 [n_inst+1]
    // offsets, mirrored in h_inst_begin; inst_total: double [n_inst] total
    // probability of each instance before its normalisation).  n_inst = 0:
    // a plain state.
    uint32_t n_inst = 0;
    qd_dbuf inst, inst_begin, inst_total;
    std::vector<uint64_t> h_inst_begin;
    // an asynchronous download still reading the buffers: work that writes
    // them waits on dl_done first (on the device), the host in
    // quids_gpu_state_download_wait
    cudaEvent_t dl_done = nullptr;
    bool dl_pending = false;
};

namespace qd::engine {

inline int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return QUIDS_OK;
    if (e == cudaErrorMemoryAllocation) return QUIDS_ERR_OOM;
    return QUIDS_ERR_CUDA;
}

#define QD_TRY(expr)                                   \
    do {                                               \
        int _rc = (expr);                              \
        if (_rc != QUIDS_OK) return _rc;               \
    } while (0)
#define QD_CUDA(expr) QD_TRY(::qd::engine::cuda_status(expr))

// Bumped by every device (re)allocation or release of a buffer: a captured
// CUDA graph, which names buffers by address, stays valid while it is
// unchanged.
inline std::atomic<uint64_t> g_alloc_epoch{0};
// Set while a planned run is captured into a graph: a buffer that would have
// to grow makes ensure() fail with kAllocFrozen instead.
inline thread_local bool g_alloc_frozen = false;
constexpr int kAllocFrozen = -1001;
// The largest device allocation the current call may make
// (quids_gpu_params::max_alloc_bytes; 0: no limit), set for the duration of
// a call by alloc_limit_scope.
inline thread_local size_t g_alloc_limit = 0;
struct alloc_limit_scope {
    size_t saved;
    explicit alloc_limit_scope(uint64_t limit) : saved(g_alloc_limit) { g_alloc_limit = (size_t)limit; }
    ~alloc_limit_scope() { g_alloc_limit = saved; }
};

inline int ensure(qd_dbuf &b, size_t bytes, bool headroom = true) {
    if (bytes == 0) bytes = 8;
    if (b.cap >= bytes) return QUIDS_OK;
    if (g_alloc_frozen) return kAllocFrozen;
    if (g_alloc_limit && bytes > g_alloc_limit) return QUIDS_ERR_OOM;
    if (g_alloc_limit && bytes + bytes / 4 > g_alloc_limit) headroom = false;
    g_alloc_epoch.fetch_add(1);
    if (b.p) {
        cudaError_t e = cudaFree(b.p);
        b.p = nullptr;
        b.cap = 0;
        if (e != cudaSuccess) return cuda_status(e);
    }
    size_t want = headroom ? bytes + bytes / 4 : bytes;
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        e = cudaMalloc(&b.p, bytes);  // retry without headroom
        if (e != cudaSuccess) {
            cudaGetLastError();
            b.p = nullptr;
            return QUIDS_ERR_OOM;
        }
        want = bytes;
    }
    b.cap = want;
    return QUIDS_OK;
}
inline void release(qd_dbuf &b);
// ensure() that keeps the buffer's contents when it grows (a state that is
// still to be read)
inline int ensure_keep(qd_dbuf &b, size_t bytes, cudaStream_t s) {
    if (bytes == 0) bytes = 8;
    if (b.cap >= bytes) return QUIDS_OK;
    if (g_alloc_frozen) return kAllocFrozen;
    qd_dbuf nb;
    QD_TRY(ensure(nb, bytes));
    if (b.p) {
        cudaError_t e = cudaMemcpyAsync(nb.p, b.p, b.cap, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            release(nb);
            return cuda_status(e);
        }
        release(b);
    }
    b = nb;
    return QUIDS_OK;
}
inline void release(qd_dbuf &b) {
    if (b.p) {
        g_alloc_epoch.fetch_add(1);
        cudaFree(b.p);
    }
    b.p = nullptr;
    b.cap = 0;
}
// the context's stream waits for a pending asynchronous download of st (a
// device-side wait: the host does not block)
inline int after_download(const quids_gpu_state *st) {
    if (!st || !st->ctx || !st->dl_pending) return QUIDS_OK;
    return cuda_status(cudaStreamWaitEvent(st->ctx->stream, st->dl_done, 0));
}

inline void release_state(quids_gpu_state *st) {
    for (qd_dbuf *b : {&st->objects, &st->begin, &st->size, &st->mag, &st->d_total, &st->meta, &st->inst,
                       &st->inst_begin, &st->inst_total})
        release(*b);
    st->n = st->nbytes = 0;
    st->n_inst = 0;
    st->h_inst_begin.clear();
    st->total_pending = false;
}

template <class T>
inline T *bufp(quids_gpu_ctx *ctx, qd_buf_id id) {
    return (T *)ctx->buf[id].p;
}

// collision-table probe limit of a step (quids_gpu_params::max_probes)
inline uint32_t probe_limit(const quids_gpu_params &prm) { return prm.max_probes ? prm.max_probes : 65536u; }

// A one-pass step groups its children by partition (collide.cuh) when
// QUIDS_FLAG_PARTITION asks for it, else in the open-addressing table.
inline bool use_partition(const quids_gpu_params &prm, uint64_t) {
    return (prm.flags & QUIDS_FLAG_PARTITION) && !(prm.flags & QUIDS_FLAG_TABLE);
}

// Blocks of `kernel` (at `threads` per block, `smem` dynamic shared bytes)
// one SM holds at once: a grid of that many per SM is one full wave.
// Queried once per kernel (and shared-memory size) and device.
template <class K>
inline int resident_per_sm(K kernel, int threads, size_t smem = 0) {
    static thread_local const void *cached_fn = nullptr;  // kernels of one signature share K
    static thread_local int cached_dev = -1;
    static thread_local size_t cached_smem = 0;
    static thread_local int cached = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    if ((const void *)kernel != cached_fn || dev != cached_dev || smem != cached_smem || cached <= 0) {
        cached_fn = (const void *)kernel;
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            n = 8;
        }
        cached_dev = dev;
        cached_smem = smem;
        cached = n;
    }
    return cached;
}

inline unsigned grid_for(quids_gpu_ctx *ctx, uint64_t n, int per_sm = 0) {
    if (per_sm <= 0) per_sm = ctx->tune.per_sm;
    uint64_t g = (n + prim::kThreads - 1) / prim::kThreads;
    uint64_t cap = (uint64_t)ctx->num_sms * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (unsigned)g;
}

// The step's words on the host, without a stream synchronisation: a
// one-warp kernel copies them into mapped pinned memory and then writes a
// sequence number; the host waits for that number (checking the stream for
// errors as it waits) and reads the words.  The stream keeps running.
static __global__ void k_publish_words(const uint64_t *w, volatile uint64_t *h, uint64_t seq) {
    if (threadIdx.x < W_COUNT_WORDS) h[threadIdx.x] = w[threadIdx.x];
    __threadfence_system();
    __syncwarp();
    if (threadIdx.x == 0) h[W_COUNT_WORDS] = seq;
}

// the publication a kernel's last block makes of the step's words (the
// host then waits with wait_words(ctx, pb.seq))
inline prim::publish publish_words(quids_gpu_ctx *ctx, qd_word done) {
    prim::publish pb;
    pb.words = ctx->d_words;
    pb.host = ctx->h_words_dev;
    pb.count = W_COUNT_WORDS;
    pb.seq = ++ctx->publish_seq;
    pb.done = (unsigned int *)(ctx->d_words + done);
    return pb;
}

inline int wait_words(quids_gpu_ctx *ctx, uint64_t seq) {
    volatile uint64_t *hw = ctx->h_words;
    for (uint64_t it = 1; hw[W_COUNT_WORDS] != seq; ++it) {
        if ((it & 1023) == 0) {
            const cudaError_t e = cudaStreamQuery(ctx->stream);
            if (e == cudaSuccess) {
                if (hw[W_COUNT_WORDS] != seq) {  // the stream is done: read the words directly
                    QD_CUDA(cudaMemcpy((void *)ctx->h_words, ctx->d_words, W_COUNT_WORDS * sizeof(uint64_t),
                                       cudaMemcpyDeviceToHost));
                }
                break;
            }
            if (e != cudaErrorNotReady) return cuda_status(e);
        }
    }
    std::atomic_thread_fence(std::memory_order_acquire);
    return (int)(int64_t)hw[W_STATUS];
}

inline int read_words(quids_gpu_ctx *ctx) {
    const uint64_t seq = ++ctx->publish_seq;
    k_publish_words<<<1, 32, 0, ctx->stream>>>(ctx->d_words, ctx->h_words_dev, seq);
    ctx->launches += 1;
    QD_CUDA(cudaGetLastError());
    return wait_words(ctx, seq);
}

// bookkeeping after a launch: count it, report a launch error
inline int launched(quids_gpu_ctx *ctx, uint64_t n = 1) {
    ctx->launches += n;
    return cuda_status(cudaGetLastError());
}

static __global__ void k_set_word(uint64_t *w, uint64_t v) { *w = v; }

// moves a sticky modifier error into the step's status word
static __global__ void k_take_status(int *src, uint64_t *status_word) {
    int e = *src;
    if (e) {
        *(int *)status_word = e;
        *src = 0;
    }
}

// stream-ordered write of one device word (no host synchronisation)
inline int set_word(quids_gpu_ctx *ctx, qd_word w, uint64_t v) {
    k_set_word<<<1, 1, 0, ctx->stream>>>(ctx->d_words + w, v);
    return launched(ctx);
}

// Start of a step, one launch: the step's words (zero but the parent
// counts, and a sticky modifier status moved in) and `nzero` zeroed words of
// look-back chains.
static __global__ void __launch_bounds__(256)
    k_step_begin(uint64_t *words, uint64_t n, uint64_t np, int *modstatus, uint64_t *zero, uint64_t nzero) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid < W_COUNT_WORDS) {
        uint64_t v = 0;
        if (tid == W_N) v = n;
        if (tid == W_NP) v = np;
        if (tid == W_STATUS && modstatus) {
            v = (uint64_t)(uint32_t)*modstatus;
            *modstatus = 0;
        }
        words[tid] = v;
    }
    for (uint64_t i = tid; i < nzero; i += (uint64_t)gridDim.x * blockDim.x) zero[i] = 0;
}

// Several byte fills in one launch (regions 16-byte aligned).
struct fill_set {
    static constexpr int kMax = 6;
    unsigned char *p[kMax];
    uint64_t n[kMax];
    uint32_t v[kMax];  // the byte replicated
    int count;
    // region r has (*dn[r]) * mul[r] + add[r] bytes when dn[r] is set (a size
    // known only on the device; n[r] is then its bound)
    const uint64_t *dn[kMax];
    uint64_t mul[kMax], add[kMax];
};
static __global__ void __launch_bounds__(256) k_fill(fill_set f) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
    for (int r = 0; r < f.count; ++r) {
        const uint32_t w = f.v[r] * 0x01010101u;
        const uint4 q = make_uint4(w, w, w, w);
        const uint64_t nb = f.dn[r] ? (*f.dn[r]) * f.mul[r] + f.add[r] : f.n[r];
        const uint64_t n16 = nb / 16;
        for (uint64_t i = tid; i < n16; i += stride) ((uint4 *)f.p[r])[i] = q;
        for (uint64_t i = n16 * 16 + tid; i < nb; i += stride) f.p[r][i] = (unsigned char)f.v[r];
    }
}
inline int fill(quids_gpu_ctx *ctx, const fill_set &f) {
    uint64_t most = 0;
    for (int r = 0; r < f.count; ++r) most = f.n[r] > most ? f.n[r] : most;
    uint64_t g = (most / 16 + 255) / 256;
    const uint64_t cap = (uint64_t)ctx->num_sms * 8;
    g = g < 1 ? 1 : (g > cap ? cap : g);
    k_fill<<<(unsigned)g, 256, 0, ctx->stream>>>(f);
    return launched(ctx);
}


// ---------------------------------------------------------- rule traits
// rules whose children come in groups sharing factor prefixes
// (grouped_children = true, template expand_group<H>(pb, pe, e, s, mag, emit))
template <class R, class = void>
struct has_grouped : std::false_type {};
template <class R>
struct has_grouped<R, std::void_t<decltype(R::grouped_children)>> : std::bool_constant<R::grouped_children> {};
// blocks per SM the grouped pass with a fused table claim is compiled for
// (the register cap of __launch_bounds__): claimed_pass_blocks in the rule,
// else 1 (no cap).  The flip rules' walk keeps its FP64 pipe busy only with
// several resident blocks (four, some spilling, ran fastest); split_merge's
// larger walk is slower when capped.
// The batched pass (per-instance rules, more live state) is not capped.
template <class R, class = void>
struct claimed_pass_blocks : std::integral_constant<int, 1> {};
template <class R>
struct claimed_pass_blocks<R, std::void_t<decltype(R::claimed_pass_blocks)>>
    : std::integral_constant<int, R::claimed_pass_blocks> {};

template <class R, class = void>
struct has_hash_child : std::false_type {};
template <class R>
struct has_hash_child<R, std::void_t<decltype(std::declval<const R &>().hash_child(
                             (const char *)0, (const char *)0, 0u, std::declval<uint32_t &>(),
                             std::declval<mag_t &>()))>> : std::true_type {};

template <class R, class = void>
struct has_hasher : std::false_type {};
template <class R>
struct has_hasher<R, std::void_t<decltype(std::declval<const R &>().hasher((const char *)0, (const char *)0))>>
    : std::true_type {};

template <class R, class = void>
struct has_populate_simple : std::false_type {};
template <class R>
struct has_populate_simple<R, std::void_t<decltype(std::declval<const R &>().populate_child_simple(
                                  (const char *)0, (const char *)0, (char *)0, 0u))>> : std::true_type {};

// rules that can tell when a parent's child count overflows the u32 of
// get_num_child (child_count_overflows(pb, pe) -> bool)
template <class R, class = void>
struct has_count_check : std::false_type {};
template <class R>
struct has_count_check<R, std::void_t<decltype(std::declval<const R &>().child_count_overflows(
                              (const char *)0, (const char *)0))>> : std::true_type {};

template <class R, class = void>
struct has_fits : std::false_type {};
template <class R>
struct has_fits<R, std::void_t<decltype(std::declval<const R &>().fits(0u))>> : std::true_type {};

// false when the rule/modifier declares the object unfit (e.g. a qubit index
// beyond the object's bytes)
template <class R>
QD_HD bool object_fits(const R &r, uint32_t size) {
    if constexpr (has_fits<R>::value)
        return r.fits(size);
    else
        return true;
}

template <class R>
QD_HD uint64_t rule_hash(const R &r, const char *b, const char *e) {
    if constexpr (has_hasher<R>::value)
        return r.hasher(b, e);
    else
        return murmur64a(b, (uint64_t)(e - b));
}
template <class R>
QD_HD void rule_populate_simple(const R &r, const char *pb, const char *pe, char *cb, uint32_t cid) {
    if constexpr (has_populate_simple<R>::value) {
        r.populate_child_simple(pb, pe, cb, cid);
    } else {
        uint32_t sz;
        mag_t m{0, 0};
        r.populate_child(pb, pe, cb, cid, sz, m);
    }
}

// ------------------------------------------------------- rule sources
// The rule of a parent: one rule for every parent, or (batched states) one
// rule per instance, looked up by the parent's instance.  Child hashes are
// tagged with the instance so that groups never span instances.
template <class Rule>
struct single_rule {
    using rule_type = Rule;
    static constexpr bool single = true;
    Rule r;
    __device__ __forceinline__ const Rule &get(uint64_t) const { return r; }
    __device__ __forceinline__ uint64_t tag(uint64_t h, uint64_t) const { return h; }
};
template <class Rule>
struct instance_rules {
    using rule_type = Rule;
    static constexpr bool single = false;
    const Rule *rules;    // [instances]
    const uint32_t *inst; // instance of each parent
    __device__ __forceinline__ Rule get(uint64_t parent) const { return rules[inst[parent]]; }
    __device__ __forceinline__ uint64_t tag(uint64_t h, uint64_t parent) const {
        return h ^ (0x9E3779B97F4A7C15ull * ((uint64_t)inst[parent] + 1));
    }
};

// ------------------------------------------------------- per-rule kernels
template <class RS>
__global__ void __launch_bounds__(prim::kThreads)
    k_num_child(RS rs, const char *objects, const uint64_t *begin, const uint32_t *size, uint64_t n,
                uint32_t *nchild, unsigned long long *d_maxsize, int *err, const uint64_t *d_n = nullptr) {
    if (d_n) n = *d_n;  // the parent count on the device (n is then a bound)
    uint32_t mx = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const auto &rule = rs.get(i);
        const char *pb = objects + begin[i];
        if (!object_fits(rule, size[i])) {
            nchild[i] = 0;
            prim::set_error(err, QUIDS_ERR_BAD_ARG);
            continue;
        }
        uint32_t nc, mcs;
        rule.get_num_child(pb, pb + size[i], nc, mcs);
        if constexpr (has_count_check<std::decay_t<decltype(rule)>>::value) {
            if (rule.child_count_overflows(pb, pb + size[i])) {
                nc = 0;
                prim::set_error(err, QUIDS_ERR_CHILD_COUNT_OVERFLOW);
            }
        }
        nchild[i] = nc;
        mx = mx > mcs ? mx : mcs;
    }
    for (int o = 16; o > 0; o >>= 1) {
        uint32_t y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = mx > y ? mx : y;
    }
    if ((threadIdx.x & 31) == 0 && mx) atomicMax(d_maxsize, (unsigned long long)mx);
}

// parent index p of child c: the last p with cbeg[p] <= c
__device__ __forceinline__ uint64_t parent_of(const uint64_t *cbeg, uint64_t np, uint64_t c) {
    uint64_t lo = 0, hi = np;  // cbeg[lo] <= c < cbeg[hi]
    while (hi - lo > 1) {
        uint64_t mid = (lo + hi) >> 1;
        if (cbeg[mid] <= c) lo = mid; else hi = mid;
    }
    return lo;
}

struct parents_view {
    const char *objects;
    const uint64_t *begin;
    const uint32_t *size;
    const double2 *mag;
    const uint64_t *cbeg;  // [np+1]
    const uint64_t *pidx;  // kept parent -> parent index, or null (identity)
    uint64_t np;
    const uint64_t *d_np = nullptr;  // if set, the parent count on the device (np is then a bound)
    __device__ __forceinline__ uint64_t nparents() const { return d_np ? *d_np : np; }
};


// The children of one tile of kTileChildren come from a contiguous run of
// parents, [tile_first[t], tile_first[t+1]]; their offsets are staged in
// shared memory so each child finds its parent with a short search there.
constexpr int kSymItems = 4;
constexpr int kTileChildren = prim::kThreads * kSymItems;
constexpr int kStagedParents = 4 * kTileChildren;

// tile_first[t] = the parent holding child t * kTileChildren; tile_first[tiles] = np - 1
static __global__ void __launch_bounds__(prim::kThreads)
    k_tile_parents(const uint64_t *cbeg, uint64_t np, uint64_t tiles, uint64_t *tile_first) {
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t lo = cbeg[p], hi = cbeg[p + 1];
        if (hi > lo) {
            for (uint64_t t = (lo + kTileChildren - 1) / kTileChildren; t * kTileChildren < hi; ++t) tile_first[t] = p;
        }
        if (p == np - 1) tile_first[tiles] = np - 1;
    }
}

// the same map written by the child-offset scan as each parent's offset is
// known (entries beyond `cap` are left to k_tile_parents)
template <uint64_t TILE>
struct tile_map_epilogue {
    uint64_t *tile_first;
    uint64_t cap;  // entries
    __device__ __forceinline__ void operator()(uint64_t p, uint64_t lo, uint64_t cnt, uint64_t np) const {
        const uint64_t hi = lo + cnt;
        for (uint64_t t = (lo + TILE - 1) / TILE; t * TILE < hi && t < cap; ++t) tile_first[t] = p;
        if (p == np - 1) {
            const uint64_t tiles = (hi + TILE - 1) / TILE;
            if (tiles < cap) tile_first[tiles] = np - 1;
        }
    }
};
using tile_parents_epilogue = tile_map_epilogue<kTileChildren>;

// Symbolic iteration (src/quids.hpp:705-719): per child, its magnitude,
// size, hash and parent.  FAST: the rule's hash_child; otherwise
// populate_child into a per-thread buffer of MAXC bytes followed by the
// rule's hasher.
template <class RS, int MAXC, bool FAST>
__global__ void __launch_bounds__(prim::kThreads)
    k_symbolic(RS rs, parents_view pv, const uint64_t *tile_first, const uint64_t *d_nc, uint64_t *hash,
               double2 *cmag, uint32_t *csize, uint32_t *cpar, unsigned long long *d_maxabs, int *err,
               const uint64_t *d_bound) {
    __shared__ uint64_t s_cb[kStagedParents + 1];
    const uint64_t nc = *d_nc;
    // the step's child size bound: the largest max_child_size its parents
    // declared (get_num_child), which sized the per-thread child buffer; a
    // rule reporting a larger child breaks its contract
    const uint64_t bound = *d_bound;
    const uint64_t ntiles = (nc + kTileChildren - 1) / kTileChildren;
    double mx = 0;
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const uint64_t c0 = t * kTileChildren;
        const uint64_t c1 = c0 + kTileChildren < nc ? c0 + kTileChildren : nc;
        const uint64_t plo = tile_first[t], phi = tile_first[t + 1];
        const int count = phi - plo + 1 <= (uint64_t)kStagedParents ? (int)(phi - plo + 1) : -1;
        __syncthreads();  // the previous tile is done with s_cb
        for (int k = threadIdx.x; k <= count; k += blockDim.x) s_cb[k] = pv.cbeg[plo + k];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kSymItems; ++k) {
            const uint64_t c = c0 + threadIdx.x + (uint64_t)k * prim::kThreads;
            if (c >= c1) break;
            uint64_t p;
            if (count > 0) {
                int lo = 0, hi = count;  // s_cb[lo] <= c < s_cb[hi]
                while (hi - lo > 1) {
                    int mid = (lo + hi) >> 1;
                    if (s_cb[mid] <= c) lo = mid; else hi = mid;
                }
                p = plo + (uint64_t)lo;
            } else {
                p = parent_of(pv.cbeg, pv.nparents(), c);
            }
            uint64_t oid = pv.pidx ? pv.pidx[p] : p;
            uint32_t cid = (uint32_t)(c - pv.cbeg[p]);
            const char *pb = pv.objects + pv.begin[oid];
            const char *pe = pb + pv.size[oid];
            double2 pm = pv.mag[oid];
            mag_t m{pm.x, pm.y};
            uint32_t sz = 0;
            uint64_t h;
            const auto &rule = rs.get(oid);
            if constexpr (FAST) {
                h = rule.hash_child(pb, pe, cid, sz, m);
                if (sz > bound) prim::set_error(err, QUIDS_ERR_SIZE_BOUND);
            } else {
                uint64_t buf[MAXC / 8];
                rule.populate_child(pb, pe, (char *)buf, cid, sz, m);
                if (sz > bound || sz > MAXC) {
                    prim::set_error(err, QUIDS_ERR_SIZE_BOUND);
                    if (sz > MAXC) sz = MAXC;
                }
                h = rule_hash(rule, (const char *)buf, (const char *)buf + sz);
            }
            h = rs.tag(h, oid);
            hash[c] = h;
            cmag[c] = make_double2(m.re, m.im);
            csize[c] = sz;
            cpar[c] = (uint32_t)p;
            double a = fabs(m.re) > fabs(m.im) ? fabs(m.re) : fabs(m.im);
            mx = mx > a ? mx : a;
        }
    }
    unsigned long long bits = (unsigned long long)__double_as_longlong(mx);
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long y = __shfl_xor_sync(0xffffffffu, bits, o);
        bits = bits > y ? bits : y;
    }
    if ((threadIdx.x & 31) == 0 && bits) atomicMax(d_maxabs, bits);
}

// What runs on each survivor right after populate (the modifiers that
// follow a rule in a run); nothing by default.
struct no_post {
    static constexpr bool active = false;
    __device__ __forceinline__ void operator()(char *, char *, mag_t &, int *) const {}
};

// Grouped symbolic iteration for rules with grouped_children: a parent
// with 2^s children (one factor per site) is handled by "leaders", each
// expanding the 2^H children whose ids share their low s-H bits
// (expand_group); parents with fewer than H sites have one leader that
// walks its children one by one.  The leaders of each parent come from a
// scan of leader counts (lbeg).  The output is that of k_symbolic.
constexpr int kGroupBits = 2;
constexpr int kLeaderTile = prim::kThreads;          // leaders per tile
constexpr int kStagedLeaderParents = 4 * kLeaderTile;
struct scan_leaders {
    const uint32_t *nchild;
    const uint64_t *pidx;
    __device__ uint64_t operator()(uint64_t i) const {
        const uint32_t nc = nchild[pidx ? pidx[i] : i];
        if (nc == 0) return 0;
        const int s = __ffs((int)nc) - 1;  // nc = 2^s
        return s >= kGroupBits ? (uint64_t)(nc >> kGroupBits) : 1;
    }
};
using leader_tile_epilogue = tile_map_epilogue<kLeaderTile>;

// what the grouped pass does with child c (hash already tagged): its
// records ...
struct child_records {
    uint64_t *hash;
    double2 *cmag;
    uint32_t *csize;
    uint32_t *cpar;
    __device__ __forceinline__ void operator()(uint64_t c, uint64_t h, const mag_t &m, uint32_t sz, uint64_t p) const {
        hash[c] = h;
        cmag[c] = make_double2(m.re, m.im);
        csize[c] = sz;
        cpar[c] = (uint32_t)p;
    }
};

// The grouped pass can also claim its children's collision-table slots
// (the work of prim::k_table_claim, same table, same outcome per child): a
// child's first compare-and-swap is issued as soon as its hash is known, and
// its result is used after the leader's expansion (claimed, joined, or probe
// on), so the atomics, bound by L2 misses, overlap the walk's FP64 work
// instead of running as a pass of their own.  The table is cleared before
// the pass.
struct no_claim {
    static constexpr bool active = false;
    __device__ __forceinline__ uint64_t slots() const { return 0; }
    __device__ __forceinline__ unsigned long long first(uint64_t, uint64_t) const { return 0; }
    __device__ __forceinline__ void finish(uint64_t, uint64_t, unsigned long long, uint64_t) const {}
};
struct table_claim {
    static constexpr bool active = true;
    prim::table t;
    uint32_t *slot_out;
    int *err;
    __device__ __forceinline__ uint64_t slots() const { return t.d_m ? *t.d_m : t.m; }
    // the first probe of child c (hash h, home slot s): the old key
    __device__ __forceinline__ unsigned long long first(uint64_t h, uint64_t m) const {
        if (h == prim::kEmptyKey) return 0;
        return atomicCAS(&t.slots[prim::table_home(h, m)].key, prim::kEmptyKey, h);
    }
    // the rest of k_table_claim's protocol for child c, given the first probe's key
    __device__ __forceinline__ void finish(uint64_t c, uint64_t h, unsigned long long key, uint64_t m) const {
        uint64_t sl;
        bool claimed = false;
        if (h == prim::kEmptyKey) {
            sl = m;
        } else {
            sl = prim::table_home(h, m);
            uint32_t probe = 0;
            while (true) {
                if (key == prim::kEmptyKey) {
                    *(uint2 *)&t.slots[sl].rep = make_uint2((uint32_t)c, (uint32_t)c);
                    claimed = true;
                    break;
                }
                if (key == h) {
                    ulonglong4_32a z;
                    z.x = z.y = z.z = z.w = 0;
                    *(ulonglong4_32a *)&t.acc[4 * sl] = z;
                    break;
                }
                if (++sl == m) sl = 0;
                if (++probe >= t.max_probes) {
                    prim::set_error(err, QUIDS_ERR_TABLE_FULL);
                    sl = ~0ull;
                    break;
                }
                key = atomicCAS(&t.slots[sl].key, prim::kEmptyKey, h);
            }
        }
        slot_out[c] = sl == ~0ull ? prim::kNoSlot : (claimed ? (uint32_t)sl : (uint32_t)sl | prim::kJoin);
    }
};

// The parents of a tile are contiguous in the state's byte array (without a
// parent index map), so a tile whose parents' bytes fit kParentStage is
// staged in shared memory first: the 16-byte aligned body in one bulk copy
// (cp.async.bulk, completing on an mbarrier), the last few bytes by plain
// loads; the walks then read their parents there.  The wait is bounded: one
// that runs out records QUIDS_ERR_TIMEOUT, waits (bounded again) for the
// copy, and the block stops.
constexpr uint32_t kParentStage = 36 * 1024;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t it = 0; it < prim::kSpinLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

template <class RS, class Out, class Claim = no_claim>
__global__ void __launch_bounds__(prim::kThreads,
                                  Claim::active && RS::single ? claimed_pass_blocks<typename RS::rule_type>::value : 1)
    k_symbolic_grouped(RS rs, parents_view pv, const uint64_t *lbeg, const uint64_t *tile_first, const uint64_t *d_nl,
                       Out emit_child, unsigned long long *d_maxabs, int *err, Claim claim = Claim{}) {
    using Rule = typename RS::rule_type;
    constexpr int H = kGroupBits;
    __shared__ uint64_t s_lb[kStagedLeaderParents + 1];
    __shared__ __align__(128) unsigned char s_par[kParentStage];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ int s_stop;
    const uint64_t nl = *d_nl;
    const uint64_t ntiles = (nl + kLeaderTile - 1) / kLeaderTile;
    const uint32_t bar = smem_u32(&s_bar);
    const bool can_stage = !pv.pidx && ((uintptr_t)pv.objects & 15) == 0;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_stop = 0;
    }
    uint32_t parity = 0;
    unsigned long long mx = 0;  // IEEE bits of the largest |component| (ordered like the values)
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const uint64_t plo = tile_first[t], phi = tile_first[t + 1];
        const int count = phi - plo + 1 <= (uint64_t)kStagedLeaderParents ? (int)(phi - plo + 1) : -1;
        __syncthreads();  // the previous tile is done with s_lb and s_par
        for (int k = threadIdx.x; k <= count; k += blockDim.x) s_lb[k] = lbeg[plo + k];
        // the tile's parent bytes [lo, hi), staged from a0 = lo rounded down to 16
        uint64_t a0 = 0, hi = 0;
        bool staged = false;
        if (can_stage) {
            const uint64_t lo = pv.begin[plo];
            hi = pv.begin[phi] + pv.size[phi];
            a0 = lo & ~15ull;
            staged = hi > lo && hi - a0 <= kParentStage;
        }
        if (staged) {
            const uint64_t a1 = hi & ~15ull;  // the bulk copy's end; [a1, hi) by plain loads
            if (threadIdx.x == 0 && a1 > a0) {
                const uint32_t bytes = (uint32_t)(a1 - a0);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                             : "memory");
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        smem_u32(s_par)),
                    "l"(pv.objects + a0), "r"(bytes), "r"(bar)
                    : "memory");
            }
            if (threadIdx.x < hi - a1) s_par[a1 - a0 + threadIdx.x] = (unsigned char)pv.objects[a1 + threadIdx.x];
            if (a1 > a0) {
                if (!mbar_wait(bar, parity)) {
                    if (threadIdx.x == 0) {
                        prim::set_error(err, QUIDS_ERR_TIMEOUT);
                        s_stop = 1;
                    }
                    mbar_wait(bar, parity);
                }
                parity ^= 1;
            }
        }
        __syncthreads();
        if (s_stop) break;
        const uint64_t l = t * kLeaderTile + threadIdx.x;
        if (l >= nl) continue;
        uint64_t p;
        if (count > 0) {
            int lo = 0, hi = count;  // s_lb[lo] <= l < s_lb[hi]
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (s_lb[mid] <= l) lo = mid; else hi = mid;
            }
            p = plo + (uint64_t)lo;
        } else {
            p = parent_of(lbeg, pv.nparents(), l);
        }
        const uint64_t oid = pv.pidx ? pv.pidx[p] : p;
        const uint64_t c0 = pv.cbeg[p];
        const uint64_t nch = pv.cbeg[p + 1] - c0;
        const int s = __ffsll((long long)nch) - 1;
        const uint32_t e = (uint32_t)(l - lbeg[p]);
        const uint64_t ob = pv.begin[oid];
        const uint32_t osz = pv.size[oid];
        // (a state may place its objects in any order: only a parent inside
        // the staged range reads there)
        const char *pb = staged && ob >= a0 && ob + osz <= hi ? (const char *)s_par + (ob - a0) : pv.objects + ob;
        const char *pe = pb + osz;
        const double2 pm = pv.mag[oid];
        const Rule &rule = rs.get(oid);
        // with a claim: child k of this leader's (k = j, or the child id
        // when the parent has fewer than 2^H children), its tagged hash and
        // its first probe's key
        constexpr int K = 1 << H;
        static_assert(K == 4, "the claim keeps four children per leader");
        uint64_t kh0 = 0, kh1 = 0, kh2 = 0, kh3 = 0;
        unsigned long long kk0 = 0, kk1 = 0, kk2 = 0, kk3 = 0;
        const uint64_t m_slots = Claim::active ? claim.slots() : 0;
        auto out = [&](int k, uint64_t c, uint64_t h, const mag_t &m, uint32_t sz) {
            const uint64_t ht = rs.tag(h, oid);
            emit_child(c, ht, m, sz, p);
            if constexpr (Claim::active) {
                const unsigned long long key = claim.first(ht, m_slots);
                switch (k) {
                case 0: kh0 = ht, kk0 = key; break;
                case 1: kh1 = ht, kk1 = key; break;
                case 2: kh2 = ht, kk2 = key; break;
                default: kh3 = ht, kk3 = key; break;
                }
            }
            const unsigned long long a = (unsigned long long)__double_as_longlong(m.re) & 0x7fffffffffffffffull;
            const unsigned long long b = (unsigned long long)__double_as_longlong(m.im) & 0x7fffffffffffffffull;
            const unsigned long long ab = a > b ? a : b;
            mx = mx > ab ? mx : ab;
        };
        int nk;
        if (s >= H) {
            rule.template expand_group<H>(pb, pe, e, s, mag_t{pm.x, pm.y},
                                          [&](uint32_t j, uint64_t h, const mag_t &m, uint32_t sz) {
                                              out((int)j, c0 + e + ((uint64_t)j << (s - H)), h, m, sz);
                                          });
            nk = K;
        } else {
            for (uint32_t cid = 0; cid < (uint32_t)nch; ++cid) {
                mag_t m{pm.x, pm.y};
                uint32_t sz = 0;
                const uint64_t h = rule.hash_child(pb, pe, cid, sz, m);
                out((int)cid, c0 + cid, h, m, sz);
            }
            nk = (int)nch;
        }
        if constexpr (Claim::active) {
            auto cidx = [&](int k) { return s >= H ? c0 + e + ((uint64_t)k << (s - H)) : c0 + (uint64_t)k; };
            if (nk > 0) claim.finish(cidx(0), kh0, kk0, m_slots);
            if (nk > 1) claim.finish(cidx(1), kh1, kk1, m_slots);
            if (nk > 2) claim.finish(cidx(2), kh2, kk2, m_slots);
            if (nk > 3) claim.finish(cidx(3), kh3, kk3, m_slots);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = mx > y ? mx : y;
    }
    if ((threadIdx.x & 31) == 0 && mx) atomicMax(d_maxabs, mx);
}

// Finalize (src/quids.hpp:958-967) fused with normalisation (:1008-1013):
// populate_child_simple of each survivor straight into its slot of the
// packed output (padding zeroed), mag /= sqrt(total) when that factor is
// not 1 (batched: the survivor's instance factor), then `post`.
// the (kept parent, child id) of each survivor: from its representative
// child index (schild) and the children's parents (cpar) ...
struct schild_source {
    const uint64_t *schild;
    const uint32_t *cpar;
    const uint64_t *cbeg;
    __device__ __forceinline__ void get(uint64_t i, uint64_t &p, uint32_t &cid) const {
        const uint64_t c = schild[i];
        p = cpar[c];
        cid = (uint32_t)(c - cbeg[p]);
    }
};
// ... or stored per survivor
struct pc_source {
    const uint32_t *par;
    const uint32_t *cid;
    __device__ __forceinline__ void get(uint64_t i, uint64_t &p, uint32_t &c) const {
        p = par[i];
        c = cid[i];
    }
};

// Finalize (src/quids.hpp:958-967): each survivor's bytes by the rule's
// populate_child_simple, padding zeroed, magnitude normalised (and the fused
// modifiers applied), one survivor per thread.  Small objects (a few words)
// are written by their thread directly: neighbouring threads write
// neighbouring bytes.  For large objects (the step's child size bound above
// kStageMin bytes) a thread writing its own object would scatter small
// stores over many lines; instead each warp walks its 32 consecutive
// survivors in batches that fit its own kPopWarpStage bytes of shared memory
// (up to 32, one per lane), populates a batch there and writes its
// contiguous byte range out with coalesced 16-byte stores.  The warps of a
// block never wait on one another (a block-wide chunk made every warp wait
// for the block's longest object).
constexpr uint64_t kStageMin = 64;
constexpr int kPopWarps = 4;                   // warps per block of the staged form
constexpr uint32_t kPopWarpStage = 12 * 1024;  // bytes per warp: 4 x 12 KB, the static shared memory limit

template <class RS, class SS, class Post>
__device__ __forceinline__ void populate_one(const RS &rs, const parents_view &pv, const SS &ss, uint64_t i,
                                             const uint64_t *obegin, const uint32_t *osize, char *dst,
                                             double2 *omag, const double *d_factor, double f0, const uint32_t *finst,
                                             int *err, const Post &post) {
    uint64_t p;
    uint32_t cid;
    ss.get(i, p, cid);
    const uint64_t oid = pv.pidx ? pv.pidx[p] : p;
    const char *pb = pv.objects + pv.begin[oid];
    const char *pe = pb + pv.size[oid];
    const uint64_t len = obegin[i + 1] - obegin[i];
    const uint32_t sz = osize[i];
    rule_populate_simple(rs.get(oid), pb, pe, dst, cid);
    for (uint64_t q = sz; q < len; ++q) dst[q] = 0;
    const double f = finst ? d_factor[finst[i]] : f0;  // batched: the survivor's instance factor
    if (f != 1.0 || Post::active) {
        const double2 m = omag[i];
        mag_t mm{m.x, m.y};
        if (f != 1.0) mm = mag_t{__ddiv_rn(mm.re, f), __ddiv_rn(mm.im, f)};
        post(dst, dst + sz, mm, err);
        omag[i] = make_double2(mm.re, mm.im);
    }
}

template <class RS, class SS, class Post>
__global__ void __launch_bounds__(prim::kThreads)
    k_populate(RS rs, parents_view pv, SS ss, const uint64_t *d_ns, const uint64_t *obegin, const uint32_t *osize,
               char *objects, double2 *omag, const double *d_factor, const uint32_t *finst, int *err, Post post) {
    const uint64_t ns = *d_ns;
    if (ns == 0) return;
    const double f0 = finst ? 1.0 : *d_factor;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += (uint64_t)gridDim.x * blockDim.x)
        populate_one(rs, pv, ss, i, obegin, osize, objects + obegin[i], omag, d_factor, f0, finst, err, post);
}

template <class RS, class SS, class Post>
__global__ void __launch_bounds__(kPopWarps * 32)
    k_populate_staged(RS rs, parents_view pv, SS ss, const uint64_t *d_ns, const uint64_t *obegin,
                      const uint32_t *osize, char *objects, double2 *omag, const double *d_factor,
                      const uint32_t *finst, int *err, Post post) {
    __shared__ __align__(16) unsigned char s_stage[kPopWarps][kPopWarpStage];
    const uint64_t ns = *d_ns;
    if (ns == 0) return;
    const double f0 = finst ? 1.0 : *d_factor;
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned char *st = s_stage[w];
    const uint64_t ngroups = (ns + 31) / 32;
    for (uint64_t g = (uint64_t)blockIdx.x * kPopWarps + w; g < ngroups; g += (uint64_t)gridDim.x * kPopWarps) {
        const uint64_t i1 = (g + 1) * 32 < ns ? (g + 1) * 32 : ns;
        for (uint64_t cur = g * 32; cur < i1;) {
            // a batch: the longest run of survivors from cur whose bytes fit
            // the warp's buffer (obegin is nondecreasing: `fits` holds for a
            // prefix of the lanes)
            const uint64_t base = obegin[cur];
            const uint32_t shift = (uint32_t)(base & 15);
            const uint64_t e = cur + lane + 1;
            const bool fits = e <= i1 && obegin[e] - base + shift <= kPopWarpStage;
            const uint32_t k = (uint32_t)__popc(__ballot_sync(0xffffffffu, fits));
            if (k == 0) {  // one object longer than the buffer: written in place
                if (lane == 0)
                    populate_one(rs, pv, ss, cur, obegin, osize, objects + base, omag, d_factor, f0, finst, err, post);
                ++cur;
                continue;
            }
            if (lane < k)
                populate_one(rs, pv, ss, cur + lane, obegin, osize, (char *)st + shift + (obegin[cur + lane] - base),
                             omag, d_factor, f0, finst, err, post);
            __syncwarp();
            // st[shift + q] is objects[base + q]: both have the same address modulo 16
            const uint32_t nbytes = (uint32_t)(obegin[cur + k] - base);
            const uint32_t head = ((16 - shift) & 15) < nbytes ? ((16 - shift) & 15) : nbytes;
            const uint32_t body = (nbytes - head) / 16;
            char *gp = objects + base;
            if (lane < head) gp[lane] = (char)st[shift + lane];
            const uint4 *sv = (const uint4 *)(st + shift + head);
            uint4 *gv = (uint4 *)(gp + head);
            for (uint32_t q = lane; q < body; q += 32) gv[q] = sv[q];
            for (uint32_t q = head + body * 16 + lane; q < nbytes; q += 32) gp[q] = (char)st[shift + q];
            __syncwarp();  // the warp's next batch reuses st
            cur += k;
        }
    }
}

// one populate launch over n (a bound of *d_ns) survivors, staged or direct
template <class RS, class SS, class Post>
inline int launch_populate_kernel(quids_gpu_ctx *ctx, uint64_t n, bool staged, const RS &rs, const parents_view &pv,
                                  const SS &ss, const uint64_t *d_ns, const uint64_t *obegin, const uint32_t *osize,
                                  char *objects, double2 *omag, const double *d_factor, const uint32_t *finst,
                                  int *err, const Post &post) {
    if (staged) {
        auto kernel = k_populate_staged<RS, SS, Post>;
        const uint64_t blocks = ((n + 31) / 32 + kPopWarps - 1) / kPopWarps;
        const uint64_t cap = (uint64_t)ctx->num_sms * resident_per_sm(kernel, kPopWarps * 32);
        const unsigned grid = (unsigned)(blocks < cap ? (blocks ? blocks : 1) : cap);
        kernel<<<grid, kPopWarps * 32, 0, ctx->stream>>>(rs, pv, ss, d_ns, obegin, osize, objects, omag, d_factor,
                                                         finst, err, post);
    } else {
        k_populate<RS, SS, Post><<<grid_for(ctx, n), prim::kThreads, 0, ctx->stream>>>(
            rs, pv, ss, d_ns, obegin, osize, objects, omag, d_factor, finst, err, post);
    }
    return launched(ctx);
}

// every child of every parent, bytes at a fixed stride (rule-level access)
template <class Rule>
__global__ void __launch_bounds__(prim::kThreads)
    k_children(Rule rule, parents_view pv, uint64_t nc, uint64_t stride, char *bytes, uint64_t *hash, uint32_t *csize,
               double2 *cmag) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t p = parent_of(pv.cbeg, pv.np, c);
        uint64_t oid = pv.pidx ? pv.pidx[p] : p;
        uint32_t cid = (uint32_t)(c - pv.cbeg[p]);
        const char *pb = pv.objects + pv.begin[oid];
        const char *pe = pb + pv.size[oid];
        double2 pm = pv.mag[oid];
        mag_t m{pm.x, pm.y};
        uint32_t sz = 0;
        char *dst = bytes + c * stride;
        rule.populate_child(pb, pe, dst, cid, sz, m);
        hash[c] = rule_hash(rule, dst, dst + sz);
        csize[c] = sz;
        cmag[c] = make_double2(m.re, m.im);
    }
}

template <class Mod>
__global__ void __launch_bounds__(prim::kThreads)
    k_modifier(Mod mod, char *objects, const uint64_t *begin, const uint32_t *size, double2 *mag, uint64_t n,
               int *err, const uint64_t *d_n = nullptr, const uint64_t *stop = nullptr) {
    if (stop && *stop) return;  // a planned run stopped at an earlier step
    if (d_n) n = *d_n;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        char *b = objects + begin[i];
        if (!object_fits(mod, size[i])) {
            prim::set_error(err, QUIDS_ERR_BAD_ARG);
            continue;
        }
        double2 pm = mag[i];
        mag_t m{pm.x, pm.y};
        mod(b, b + size[i], m);
        mag[i] = make_double2(m.re, m.im);
    }
}

template <class Rule>
__global__ void __launch_bounds__(prim::kThreads)
    k_state_hash(Rule rule, const char *objects, const uint64_t *begin, const uint32_t *size, uint64_t n,
                 uint64_t *out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const char *b = objects + begin[i];
        out[i] = rule_hash(rule, b, b + size[i]);
    }
}

// ------------------------------------------------------ step functors
struct scan_nchild {
    const uint32_t *nchild;
    const uint64_t *pidx;
    __device__ uint64_t operator()(uint64_t i) const { return nchild[pidx ? pidx[i] : i]; }
};

__device__ __forceinline__ uint32_t padded_size(uint32_t sz, uint32_t align) {
    if (align <= 1) return sz;
    uint32_t pad = align - sz % align;
    return pad == align ? sz : sz + pad;
}

// A child represents its group when it is the group's lowest symbolic index
// (src/quids.hpp:785-809 keeps one member per hash); the group survives zero
// elimination when its summed norm is above tolerance (src/quids.hpp:819-823).
// A group of one keeps its member's own magnitude; larger groups read their
// exact fixed-point sum.
struct group_view {
    const uint32_t *slot_of;  // by child index
    const uint8_t *not_rep;
    const uint8_t *has_join;
    const double2 *cmag;
    const unsigned long long *acc;
    const uint64_t *d_nc;
    const unsigned long long *d_maxabs;
    double tolerance;
    __device__ __forceinline__ mag_t sum(uint32_t s) const {
        const int F = fix_scale(__longlong_as_double((long long)*d_maxabs), *d_nc);
        const ulonglong4_32a a = *(const ulonglong4_32a *)&acc[4ull * s];
        return mag_t{from_fix(fix128{a.x, a.y}, F), from_fix(fix128{a.z, a.w}, F)};
    }
    // the group magnitude if c is a representative, else false (the child's
    // own records are loaded before any branch)
    __device__ __forceinline__ bool rep_mag(uint64_t c, mag_t &m) const {
        const uint8_t nr = not_rep[c], hj = has_join[c];
        const uint32_t s = slot_of[c];
        const double2 v = cmag[c];
        if (nr || s == prim::kNoSlot) return false;
        m = hj ? sum(s) : mag_t{v.x, v.y};
        return true;
    }
    __device__ __forceinline__ bool kept(uint64_t c, mag_t &m) const { return rep_mag(c, m) && cnorm(m) > tolerance; }
};

// items of the collision-table insert: children in index order ...
struct direct_src {
    const uint64_t *hash_;
    const double2 *mag_;
    __device__ __forceinline__ uint64_t hash(uint64_t k) const { return hash_[k]; }
    __device__ __forceinline__ uint64_t child(uint64_t k) const { return k; }
    __device__ __forceinline__ double2 mag(uint64_t k) const { return mag_[k]; }
};

// no truncation possible: survivors straight into the output layout
struct groups_layout {
    group_view g;
    const uint32_t *csize;
    uint32_t align;
    double2 *omag;
    uint32_t *osize;
    uint64_t *obegin;
    uint64_t *schild;
    struct item {
        mag_t m;
        uint32_t size;
    };
    __device__ bool tie(uint64_t) const { return false; }
    __device__ bool load(uint64_t c, uint64_t, item &it) const {
        it.size = csize[c];
        return g.kept(c, it.m);
    }
    __device__ uint64_t bytes(const item &it) const { return padded_size(it.size, align); }
    __device__ double emit(uint64_t c, uint64_t j, uint64_t off, const item &it) const {
        omag[j] = make_double2(it.m.re, it.m.im);
        osize[j] = it.size;
        obegin[j] = off;
        schild[j] = c;
        return cnorm(it.m);
    }
};

// radix-select keys
// Truncation keys, larger = kept first.  Simple truncation: the IEEE bits
// of the norm (src/quids.hpp:884-889).  Probabilistic truncation
// (src/quids.hpp:594-608, :829-845, :890-895) keeps the smallest selectors
// u / norm with u uniform in (0, 1]; here u comes from a counter-based
// generator keyed on (seed, item id) and the key is the complement of the
// selector's bits, so the same descending selection applies.
struct trunc_key {
    bool probabilistic;
    uint64_t seed;
    __device__ __forceinline__ uint64_t operator()(double norm, uint64_t id) const {
        if (!probabilistic) return (uint64_t)__double_as_longlong(norm);
        uint64_t z = seed + 0x9E3779B97F4A7C15ull * (id + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        const double u = (double)((z >> 11) + 1) * 0x1.0p-53;  // (0, 1]
        const double sel = norm > 0 ? __ddiv_rn(u, norm) : __longlong_as_double(0x7ff0000000000000ll);
        return ~(uint64_t)__double_as_longlong(sel);
    }
};

struct key_unorm {
    const uint64_t *unorm;
    const uint64_t *uchild;
    trunc_key tk;
    __device__ uint64_t key(uint64_t i) const {
        return tk.probabilistic ? tk(__longlong_as_double((long long)unorm[i]), uchild[i]) : unorm[i];
    }
};
struct key_parent_norm {
    const double2 *mag;
    trunc_key tk;
    __device__ uint64_t key(uint64_t i) const {
        double2 m = mag[i];
        return tk(cnorm(mag_t{m.x, m.y}), i);
    }
};
static __global__ void k_select_init(prim::select_state *st, const uint64_t *d_n, uint64_t k,
                                     uint64_t *zero = nullptr) {
    prim::select_state s{};
    s.k_rem = k;
    s.active = k < *d_n ? 1u : 0u;
    st[0] = s;
    if (zero) *zero = 0;
}

// After the first digits of a selection: the keys still matching its prefix
// (st->n_equal of them), copied into cand in any order when they fit
// (st->n_equal <= cap), so the later passes read only those.  Sets the later
// passes' item count and whether they read cand.
template <class K>
__global__ void __launch_bounds__(prim::kThreads)
    k_radix_filter(K kf, const uint64_t *d_n, const prim::select_state *st, uint64_t *cand, uint64_t cap,
                   uint64_t *words) {
    const uint64_t n = *d_n;
    const bool use = st->active && st->n_equal <= cap;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        words[W_SELUSE] = use ? 1 : 0;
        words[W_SELN] = use ? st->n_equal : n;
    }
    if (!use) return;
    const uint64_t prefix = st->prefix, mask = st->mask;
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    const uint64_t warp = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (uint64_t base = warp * 32; base < n; base += warps * 32) {
        const uint64_t i = base + lane;
        uint64_t k = 0;
        bool m = false;
        if (i < n) {
            k = kf.key(i);
            m = (k & mask) == prefix;
        }
        const unsigned ball = __ballot_sync(0xffffffffu, m);
        if (!ball) continue;
        unsigned long long pos = 0;
        if (lane == 0) pos = atomicAdd((unsigned long long *)(words + W_SELCNT), (unsigned long long)__popc(ball));
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (m) cand[pos + __popc(ball & ((1u << lane) - 1))] = k;
    }
}
template <class K>
struct filtered_key {
    K kf;
    const uint64_t *cand;
    const uint64_t *use;
    __device__ __forceinline__ uint64_t key(uint64_t i) const { return *use ? cand[i] : kf.key(i); }
};
// The truncation path over the children themselves, with no list of groups:
// k_group_keys gives each child the truncation key of its group if it
// represents one kept after zero elimination (src/quids.hpp:819-823), else 0
// (a kept group's key is never 0), and counts those groups (*d_nu).  The
// selection then runs over the children's keys, and child_keep_layout lays
// out the selected representatives in child order, recomputing the few
// selected groups' magnitudes.
static __global__ void __launch_bounds__(prim::kThreads)
    k_group_keys(group_view g, trunc_key tk, const uint64_t *d_nc, uint64_t *key, unsigned long long *d_nu) {
    const uint64_t n = *d_nc;
    unsigned long long kept = 0;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x) {
        mag_t m;
        uint64_t k = 0;
        if (g.kept(c, m)) {
            k = tk(cnorm(m), c);
            ++kept;
        }
        key[c] = k;
    }
    for (int o = 16; o > 0; o >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, o);
    if ((threadIdx.x & 31) == 0 && kept) atomicAdd(d_nu, kept);
}
struct key_direct {
    const uint64_t *k;
    __device__ __forceinline__ uint64_t key(uint64_t i) const { return k[i]; }
};
struct child_keep_layout {
    group_view g;
    const uint64_t *key;
    const prim::select_state *st;
    const uint32_t *csize;
    uint32_t align;
    double2 *omag;
    uint32_t *osize;
    uint64_t *obegin;
    uint64_t *schild;
    // a selected group's size; its magnitude is recomputed when it is laid out
    // (few groups are selected, and holding it for all would cost registers)
    struct item {
        uint32_t size;
    };
    __device__ bool tie(uint64_t c) const { return st->active && key[c] == st->prefix; }
    __device__ bool rank_needed() const { return st->active && st->n_equal > st->k_rem; }
    __device__ bool load(uint64_t c, uint64_t tie_rank, item &it) const {
        const uint64_t k = key[c];
        if (k == 0) return false;
        const bool keep = !st->active || k > st->prefix || (k == st->prefix && tie_rank < st->k_rem);
        if (keep) it.size = csize[c];
        return keep;
    }
    __device__ uint64_t bytes(const item &it) const { return padded_size(it.size, align); }
    __device__ double emit(uint64_t c, uint64_t j, uint64_t off, const item &it) const {
        mag_t m;
        g.rep_mag(c, m);
        omag[j] = make_double2(m.re, m.im);
        osize[j] = it.size;
        obegin[j] = off;
        schild[j] = c;
        return cnorm(m);
    }
};
constexpr int kKeepItems = 16;  // items per thread of the truncation's keep layout (a sparse selection)

// A truncation keeps few of many children.  Rather than one look-back
// compaction over every child, the children the selection can keep (a key
// above the cutoff, or tied with it) are listed first, in child order, by
// a filter without inter-block waits: per-tile counts, a scan of the counts,
// then each tile writes its candidates at its offset.  The keep layout then
// runs over that short list.
constexpr int kCandItems = 16;
constexpr uint64_t kCandTile = (uint64_t)prim::kThreads * kCandItems;
struct keep_candidate {
    const uint64_t *key;
    const prim::select_state *st;
    __device__ __forceinline__ bool operator()(uint64_t c) const {
        const uint64_t k = key[c];
        return k != 0 && (!st->active || k >= st->prefix);
    }
};
// per tile of kCandTile children: how many are candidates (any order of reads)
template <class Pred>
__global__ void __launch_bounds__(prim::kThreads)
    k_tile_counts(Pred pred, const uint64_t *d_n, uint32_t *cnt, uint64_t *d_ntiles) {
    __shared__ uint32_t s_w[prim::kThreads / 32];
    const uint64_t n = *d_n;
    const uint64_t ntiles = (n + kCandTile - 1) / kCandTile;
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_ntiles = ntiles;
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        uint32_t c = 0;
#pragma unroll
        for (int k = 0; k < kCandItems; ++k) {
            const uint64_t i = t * kCandTile + (uint64_t)k * prim::kThreads + threadIdx.x;
            c += (i < n && pred(i)) ? 1u : 0u;
        }
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t sum = 0;
            for (int w = 0; w < prim::kThreads / 32; ++w) sum += s_w[w];
            cnt[t] = sum;
        }
        __syncthreads();
    }
}
struct scan_u32 {
    const uint32_t *v;
    __device__ uint64_t operator()(uint64_t i) const { return v[i]; }
};
// each tile writes its candidates, in child order, at its offset
template <class Pred>
__global__ void __launch_bounds__(prim::kThreads)
    k_tile_write(Pred pred, const uint64_t *d_n, const uint64_t *tile_off, uint32_t *cand) {
    __shared__ uint64_t sm[prim::kThreads / 32 + 1];
    const uint64_t n = *d_n;
    const uint64_t ntiles = (n + kCandTile - 1) / kCandTile;
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const uint64_t base = t * kCandTile + (uint64_t)threadIdx.x * kCandItems;  // a run per thread: child order
        uint32_t flags = 0;
        uint64_t c = 0;
#pragma unroll
        for (int k = 0; k < kCandItems; ++k) {
            const uint64_t i = base + k;
            if (i < n && pred(i)) {
                flags |= 1u << k;
                ++c;
            }
        }
        uint64_t agg;
        uint64_t j = tile_off[t] + prim::block_excl_scan(c, sm, agg);
#pragma unroll
        for (int k = 0; k < kCandItems; ++k)
            if (flags & (1u << k)) cand[j++] = (uint32_t)(base + k);
    }
}
// child_keep_layout over the candidate list
struct cand_keep_layout {
    child_keep_layout kl;
    const uint32_t *cand;
    using item = child_keep_layout::item;
    __device__ bool tie(uint64_t i) const { return kl.tie(cand[i]); }
    __device__ bool rank_needed() const { return kl.rank_needed(); }
    __device__ bool load(uint64_t i, uint64_t tie_rank, item &it) const { return kl.load(cand[i], tie_rank, it); }
    __device__ uint64_t bytes(const item &it) const { return kl.bytes(it); }
    __device__ double emit(uint64_t i, uint64_t j, uint64_t off, const item &it) const {
        return kl.emit(cand[i], j, off, it);
    }
};


struct keep_parents {
    key_parent_norm kf;
    const prim::select_state *st;
    uint64_t *pidx;
    __device__ uint64_t key(uint64_t i) const { return kf.key(i); }
    __device__ bool tie(uint64_t i) const { return st->active && key(i) == st->prefix; }
    __device__ bool select(uint64_t i, uint64_t tie_rank) const {
        if (!st->active) return true;
        uint64_t k = key(i);
        if (k > st->prefix) return true;
        if (k < st->prefix) return false;
        return tie_rank < st->k_rem;
    }
    __device__ void emit(uint64_t i, uint64_t j) const { pidx[j] = i; }
};

// children of the parents a threshold selection keeps, ties included (an
// upper bound used by the memory-driven truncation)
template <class K>
__global__ void __launch_bounds__(prim::kThreads)
    k_sum_selected_children(K kf, const prim::select_state *st, const uint32_t *nchild, const uint64_t *d_n,
                            unsigned long long *out) {
    const uint64_t n = *d_n;
    unsigned long long acc = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        if (!st->active || kf.key(i) >= st->prefix) acc += nchild[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

// ------------------------------------------------------------ radix select
// Runs the 8 passes of a top-k threshold selection on the stream.
template <class K1>
inline int radix_select(quids_gpu_ctx *ctx, const uint64_t *d_n, uint64_t n_host, uint64_t k, K1 k1) {
    unsigned grid = grid_for(ctx, n_host);
    k_select_init<<<1, 1, 0, ctx->stream>>>(ctx->d_sel, d_n, k);
    QD_CUDA(cudaMemsetAsync(ctx->d_hist, 0, prim::kBins * sizeof(unsigned long long), ctx->stream));
    for (int shift = 64 - prim::kDigitBits; shift >= 0; shift -= prim::kDigitBits) {
        prim::k_radix_hist<<<grid, prim::kThreads, 0, ctx->stream>>>(k1, d_n, ctx->d_sel, shift, ctx->d_hist);
        prim::k_radix_pick<<<1, prim::kBins, 0, ctx->stream>>>(ctx->d_sel, ctx->d_hist, shift, true);
    }
    return launched(ctx, 1 + 2 * 64 / prim::kDigitBits);
}

// radix_select for a truncation over many items: after the first two digits
// (16 bits: the sign, exponent and 4 mantissa bits of a norm), the keys that
// still match are copied aside when they fit cand's cap_items, and the 6 later
// passes read those instead of every item.  The result is radix_select's.
inline uint64_t filter_cap(uint64_t n) { return n / 8 + 65536; }
// d_active: the count of items that can be selected (default *d_n; the
// children's keys hold 0 for the children that represent no kept group).
template <class K1>
inline int radix_select_filtered(quids_gpu_ctx *ctx, const uint64_t *d_n, uint64_t n_host, uint64_t k, K1 k1,
                                 uint64_t *cand, uint64_t cap_items, const uint64_t *d_active = nullptr) {
    unsigned grid = grid_for(ctx, n_host);
    uint64_t *words = ctx->d_words;
    k_select_init<<<1, 1, 0, ctx->stream>>>(ctx->d_sel, d_active ? d_active : d_n, k, words + W_SELCNT);
    QD_CUDA(cudaMemsetAsync(ctx->d_hist, 0, prim::kBins * sizeof(unsigned long long), ctx->stream));
    int shift = 64 - prim::kDigitBits;
    for (int pass = 0; pass < 2; ++pass, shift -= prim::kDigitBits) {
        prim::k_radix_hist<<<grid, prim::kThreads, 0, ctx->stream>>>(k1, d_n, ctx->d_sel, shift, ctx->d_hist);
        prim::k_radix_pick<<<1, prim::kBins, 0, ctx->stream>>>(ctx->d_sel, ctx->d_hist, shift, true);
    }
    k_radix_filter<<<grid, prim::kThreads, 0, ctx->stream>>>(k1, d_n, ctx->d_sel, cand, cap_items, words);
    const filtered_key<K1> kf{k1, cand, words + W_SELUSE};
    for (; shift >= 0; shift -= prim::kDigitBits) {
        prim::k_radix_hist<<<grid, prim::kThreads, 0, ctx->stream>>>(kf, words + W_SELN, ctx->d_sel, shift,
                                                                    ctx->d_hist);
        prim::k_radix_pick<<<1, prim::kBins, 0, ctx->stream>>>(ctx->d_sel, ctx->d_hist, shift, true);
    }
    return launched(ctx, 2 + 2 * 64 / prim::kDigitBits);
}

inline uint64_t next_pow2(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

// ------------------------------------------------------------- the step
template <class RS, int MAXC>
inline int launch_symbolic(quids_gpu_ctx *ctx, const RS &rule, const parents_view &pv, uint64_t nc, bool fast) {
    using Rule = typename RS::rule_type;
    uint64_t tiles = (nc + kTileChildren - 1) / kTileChildren;
    uint64_t *d_nc = ctx->d_words + W_NC;
    unsigned long long *d_maxabs = (unsigned long long *)(ctx->d_words + W_MAXABS);
    int *err = (int *)(ctx->d_words + W_STATUS);
    const uint64_t *d_bound = ctx->d_words + W_MAXSIZE;
    const size_t smem = 0;
    // one full wave of resident blocks (each strides over tiles)
    auto wave = [&](auto kernel) {
        const uint64_t w = (uint64_t)ctx->num_sms * resident_per_sm(kernel, prim::kThreads, smem);
        return (unsigned)(tiles < w ? (tiles ? tiles : 1) : w);
    };
    if constexpr (has_hash_child<Rule>::value) {
        if (fast) {
            const unsigned grid = wave(k_symbolic<RS, 8, true>);
            k_symbolic<RS, 8, true><<<grid, prim::kThreads, smem, ctx->stream>>>(
                rule, pv, bufp<uint64_t>(ctx, B_TILEPAR), d_nc, bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG),
                bufp<uint32_t>(ctx, B_CSIZE), bufp<uint32_t>(ctx, B_CPAR), d_maxabs, err, d_bound);
            return launched(ctx);
        }
    }
    const unsigned grid = wave(k_symbolic<RS, MAXC, false>);
    k_symbolic<RS, MAXC, false><<<grid, prim::kThreads, smem, ctx->stream>>>(
        rule, pv, bufp<uint64_t>(ctx, B_TILEPAR), d_nc, bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG),
        bufp<uint32_t>(ctx, B_CSIZE), bufp<uint32_t>(ctx, B_CPAR), d_maxabs, err, d_bound);
    return launched(ctx);
}

template <class RS, class Post>
inline int launch_populate(quids_gpu_ctx *ctx, const RS &rule, const parents_view &pv, uint64_t ns,
                           quids_gpu_state *out, const Post &post, uint64_t max_child_size) {
    return launch_populate_kernel(ctx, ns, max_child_size > kStageMin, rule, pv,
                                  schild_source{bufp<uint64_t>(ctx, B_SCHILD), bufp<uint32_t>(ctx, B_CPAR), pv.cbeg},
                                  ctx->d_words + W_NS, (const uint64_t *)out->begin.p, (const uint32_t *)out->size.p,
                                  (char *)out->objects.p, (double2 *)out->mag.p,
                                  (const double *)(ctx->d_words + W_FACTOR), nullptr,
                                  (int *)(ctx->d_words + W_STATUS), post);
}

inline int ensure_state(quids_gpu_state *st, uint64_t n, uint64_t nbytes) {
    QD_TRY(ensure(st->objects, nbytes));
    QD_TRY(ensure(st->begin, (n + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(st->size, n * sizeof(uint32_t)));
    QD_TRY(ensure(st->mag, n * sizeof(double2)));
    QD_TRY(ensure(st->d_total, sizeof(double)));
    return QUIDS_OK;
}

// zeroed look-back chain `slot` (0..2) of the step for a pass over n items
inline int lookback_chain(quids_gpu_ctx *ctx, uint64_t n_cap, int slot, prim::lookback &lb) {
    const uint64_t words = (n_cap + prim::kTile - 1) / prim::kTile + 2;
    uint64_t *ws = bufp<uint64_t>(ctx, B_LOOKBACK) + (uint64_t)slot * words;
    QD_CUDA(cudaMemsetAsync(ws, 0, words * sizeof(uint64_t), ctx->stream));
    lb.status = ws + 1;
    lb.counter = (uint32_t *)ws;
    lb.err = (int *)(ctx->d_words + W_STATUS);
    return QUIDS_OK;
}
// chain `slot` of a region zeroed beforehand (k_step_begin, k_fill)
inline void lookback_view(quids_gpu_ctx *ctx, uint64_t n_cap, int slot, prim::lookback &lb) {
    const uint64_t words = (n_cap + prim::kTile - 1) / prim::kTile + 2;
    uint64_t *ws = bufp<uint64_t>(ctx, B_LOOKBACK) + (uint64_t)slot * words;
    lb.status = ws + 1;
    lb.counter = (uint32_t *)ws;
    lb.err = (int *)(ctx->d_words + W_STATUS);
}
inline uint64_t lookback_words(uint64_t n_cap) { return 3 * ((n_cap + prim::kTile - 1) / prim::kTile + 2); }
inline unsigned lookback_grid(quids_gpu_ctx *ctx, uint64_t n) {
    uint64_t tiles = (n + prim::kTile - 1) / prim::kTile;
    uint64_t cap = (uint64_t)ctx->num_sms * 4;
    return (unsigned)(tiles < 1 ? 1 : (tiles < cap ? tiles : cap));
}

inline uint64_t cand_tiles(uint64_t n) { return (n + kCandTile - 1) / kCandTile + 1; }
// The candidate list of a truncation over NC children (bounds: nc_cap) into
// B_KEEPCAND, its length in W_NCAND; uses look-back chain 3 (zeroed with the
// table).
inline int list_keep_candidates(quids_gpu_ctx *ctx, const keep_candidate &pred, uint64_t nc_cap) {
    uint64_t *words = ctx->d_words;
    const uint64_t tiles = cand_tiles(nc_cap);
    uint32_t *cnt = bufp<uint32_t>(ctx, B_TILECNT);
    uint64_t *off = (uint64_t *)(cnt + (tiles + 1) / 2 * 2);
    const unsigned g = (unsigned)std::min<uint64_t>(tiles, (uint64_t)ctx->num_sms * 8);
    k_tile_counts<<<g, prim::kThreads, 0, ctx->stream>>>(pred, words + W_NC, cnt, words + W_NTILES);
    prim::lookback lb;
    lookback_view(ctx, nc_cap, 3, lb);
    prim::k_scan_excl<<<lookback_grid(ctx, tiles), prim::kThreads, 0, ctx->stream>>>(
        scan_u32{cnt}, words + W_NTILES, off, words + W_NCAND, lb);
    k_tile_write<<<g, prim::kThreads, 0, ctx->stream>>>(pred, words + W_NC, off, bufp<uint32_t>(ctx, B_KEEPCAND));
    return launched(ctx, 3);
}
inline size_t tilecnt_bytes(uint64_t nc_cap) {
    const uint64_t tiles = cand_tiles(nc_cap);
    return ((tiles + 1) / 2 * 2) * sizeof(uint32_t) + (tiles + 1) * sizeof(uint64_t);
}

// leader offsets and their tile map (one scan), `pre` (after the scan,
// whose look-back chain it may clear: the table fill of a fused claim), then
// the grouped pass
struct no_pre {
    int operator()() const { return QUIDS_OK; }
};
template <class RS, class Claim = no_claim, class Pre = no_pre>
inline int launch_symbolic_grouped(quids_gpu_ctx *ctx, const RS &rs, const parents_view &pv, uint64_t nc,
                                   Claim claim = Claim{}, Pre pre = Pre{}) {
    const uint64_t np = pv.np;
    const uint64_t ltiles_cap = nc / kLeaderTile + 2;  // leaders <= children
    QD_TRY(ensure(ctx->buf[B_LBEG], (np + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_TILEPAR], ltiles_cap * sizeof(uint64_t)));
    prim::lookback lb;
    QD_TRY(lookback_chain(ctx, np, 0, lb));
    scan_leaders f{bufp<uint32_t>(ctx, B_NCHILD), pv.pidx};
    prim::k_scan_excl<<<lookback_grid(ctx, np), prim::kThreads, 0, ctx->stream>>>(
        f, ctx->d_words + W_NP, bufp<uint64_t>(ctx, B_LBEG), ctx->d_words + W_TMP, lb,
        leader_tile_epilogue{bufp<uint64_t>(ctx, B_TILEPAR), ltiles_cap});
    QD_TRY(launched(ctx));
    QD_TRY(pre());
    const uint64_t est_tiles = (nc >> kGroupBits) / kLeaderTile + 1;
    const unsigned g = (unsigned)std::min<uint64_t>(
        est_tiles,
        (uint64_t)ctx->num_sms * resident_per_sm(k_symbolic_grouped<RS, child_records, Claim>, prim::kThreads));
    const child_records rec{bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG), bufp<uint32_t>(ctx, B_CSIZE),
                            bufp<uint32_t>(ctx, B_CPAR)};
    k_symbolic_grouped<RS, child_records, Claim><<<g, prim::kThreads, 0, ctx->stream>>>(
        rs, pv, bufp<uint64_t>(ctx, B_LBEG), bufp<uint64_t>(ctx, B_TILEPAR), ctx->d_words + W_TMP, rec,
        (unsigned long long *)(ctx->d_words + W_MAXABS), (int *)(ctx->d_words + W_STATUS), claim);
    return launched(ctx);
}


#include "collide.cuh"

// simulate_rule's answer for a step beyond one pass (2^32 children, or
// records and table beyond the device memory) or with hash-range passes
// asked for: nothing of it is done yet, the caller runs the range passes
constexpr int kNeedRanges = 1;

template <class Rule, class Post = no_post>
int simulate_rule(quids_gpu_ctx *ctx, quids_gpu_state *in, const Rule &rule_, quids_gpu_state *out,
                  const quids_gpu_params &prm, quids_gpu_step_stats *stats, const Post &post = Post{}) {
    const single_rule<Rule> rule{rule_};
    if (!ctx || !in || !out || in == out || in->ctx != ctx || out->ctx != ctx) return QUIDS_ERR_BAD_ARG;
    const trunc_key tk{prm.simple_truncation == 0, prm.seed};
    const bool auto_max = prm.max_num_object == 0;  // memory-driven truncation (src/quids.hpp:459-485, :510-536)
    QD_CUDA(cudaSetDevice(ctx->device));
    const uint64_t N = in->n;
    const uint64_t maxn = auto_max ? ~0ull : prm.max_num_object;
    const double load = prm.table_load_factor > 0 && prm.table_load_factor < 0.95 ? prm.table_load_factor : 0.5;
    const bool timing = (prm.flags & QUIDS_FLAG_STAGE_TIMING) != 0;
    const bool fast = (prm.flags & QUIDS_FLAG_NO_FAST_HASH) == 0;
    const uint64_t launches0 = ctx->launches;
    quids_gpu_step_stats s{};
    s.num_parents = N;
    s.total_proba = std::numeric_limits<double>::quiet_NaN();  // until known on the host
    bool used[8] = {};
    auto begin_stage = [&](int k) {
        if (timing) {
            cudaEventRecord(ctx->ev_stage[2 * k], ctx->stream);
            used[k] = true;
        }
    };
    auto end_stage = [&](int k) {
        if (timing) cudaEventRecord(ctx->ev_stage[2 * k + 1], ctx->stream);
    };
    auto finish = [&](bool empty) -> int {
        out->n_inst = 0;  // a plain step makes a plain state
        out->h_inst_begin.clear();
        if (empty) {
            out->n = 0;
            out->nbytes = 0;
            out->total_proba = 0;  // normalize() of an empty state (src/quids.hpp:986-992)
            out->total_pending = false;
            QD_TRY(ensure_state(out, 0, 8));
            QD_CUDA(cudaMemsetAsync(out->begin.p, 0, sizeof(uint64_t), ctx->stream));
        }
        if (timing) {
            QD_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
            QD_CUDA(cudaStreamSynchronize(ctx->stream));
            cudaEventElapsedTime(&s.ms_total, ctx->ev0, ctx->ev1);
            for (int k = 0; k < 8; ++k)
                if (used[k]) cudaEventElapsedTime(&s.stage_ms[k], ctx->ev_stage[2 * k], ctx->ev_stage[2 * k + 1]);
            double tp;
            if (out->total_pending) {
                QD_CUDA(cudaMemcpy(&tp, out->d_total.p, sizeof(double), cudaMemcpyDeviceToHost));
                out->total_proba = tp;
                out->total_pending = false;
            }
            s.total_proba = out->total_proba;
        } else if (empty) {
            s.total_proba = 0;
        }
        s.kernel_launches = ctx->launches - launches0;
        if (stats) *stats = s;
        return QUIDS_OK;
    };
    if (timing) QD_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    // the step's words, the sticky status of earlier modifiers (an unfit
    // object), and the zeroed look-back chains of stage 0, in one launch
    QD_TRY(ensure(ctx->buf[B_NCHILD], (N ? N : 1) * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_LOOKBACK], lookback_words(N) * sizeof(uint64_t)));
    const uint64_t nzero0 = N ? lookback_words(N) : 0;
    k_step_begin<<<(unsigned)std::min<uint64_t>((nzero0 + 255) / 256 + 1, (uint64_t)ctx->num_sms * 4), 256, 0,
                   ctx->stream>>>(
        ctx->d_words, N, maxn < N ? 0 : N, bufp<int>(ctx, B_MODSTATUS), bufp<uint64_t>(ctx, B_LOOKBACK), nzero0);
    QD_TRY(launched(ctx));
    if (N == 0) return finish(true);
    int *err = (int *)(ctx->d_words + W_STATUS);

    // ---- stage 0: num_child (src/quids.hpp:548-569), parent pre-truncation
    // (src/quids.hpp:613-642, ties by lower index), child offsets (:666-673)
    begin_stage(0);
    k_num_child<<<grid_for(ctx, N), prim::kThreads, 0, ctx->stream>>>(
        rule, (const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p, N,
        bufp<uint32_t>(ctx, B_NCHILD), (unsigned long long *)(ctx->d_words + W_MAXSIZE), err);
    QD_TRY(launched(ctx));
    uint64_t NP = N;
    const uint64_t *pidx = nullptr;
    if (maxn < N) {
        QD_TRY(ensure(ctx->buf[B_PIDX], maxn * sizeof(uint64_t)));
        key_parent_norm k1{(const double2 *)in->mag.p, tk};
        QD_TRY(radix_select(ctx, ctx->d_words + W_N, N, maxn, k1));
        prim::lookback lb, lbt;
        lookback_view(ctx, N, 0, lb);
        lookback_view(ctx, N, 2, lbt);
        keep_parents kp{k1, ctx->d_sel, bufp<uint64_t>(ctx, B_PIDX)};
        prim::k_compact_ranked<<<lookback_grid(ctx, N), prim::kThreads, 0, ctx->stream>>>(
            kp, ctx->d_words + W_N, ctx->d_words + W_NP, lb, lbt);
        QD_TRY(launched(ctx));
        NP = maxn;
        pidx = bufp<uint64_t>(ctx, B_PIDX);
    }
    s.num_parents_kept = NP;
    QD_TRY(ensure(ctx->buf[B_CBEGIN], (NP + 1) * sizeof(uint64_t)));
    // the scan also writes the symbolic pass's tile -> first parent map, as
    // far as the map's buffer already reaches
    uint64_t *tile_map = bufp<uint64_t>(ctx, B_TILEPAR);
    uint64_t tile_map_cap = ctx->buf[B_TILEPAR].cap / sizeof(uint64_t);
    const prim::publish pb0 = publish_words(ctx, W_DONE_SCAN);
    {
        prim::lookback lb;
        lookback_view(ctx, N, 1, lb);
        if (prm.debug_flags & QUIDS_DEBUG_STALL_LOOKBACK) lb.stall_tile = 1;
        scan_nchild f{bufp<uint32_t>(ctx, B_NCHILD), pidx};
        prim::k_scan_excl<<<lookback_grid(ctx, NP), prim::kThreads, 0, ctx->stream>>>(
            f, ctx->d_words + W_NP, bufp<uint64_t>(ctx, B_CBEGIN), ctx->d_words + W_NC, lb,
            tile_parents_epilogue{tile_map, tile_map_cap}, pb0);
        QD_TRY(launched(ctx));
    }
    end_stage(0);
    int st = wait_words(ctx, pb0.seq);  // host wait 1: child count and size bound
    if (st) return st;
    uint64_t maxc = maxn;  // children cap
    if (auto_max && ctx->h_words[W_NC] > 0) {
        // The memory a step may use: the device's free memory plus what this
        // context and the output already hold, less the reference's 20%
        // safety margin (SAFETY_MARGIN, src/quids.hpp:33-35); or an explicit
        // budget.  A child costs its records, its share of the table and of
        // the truncation arrays; a survivor its output object.
        size_t free_b = 0, total_b = 0;
        QD_CUDA(cudaMemGetInfo(&free_b, &total_b));
        double held = 0;
        for (auto &b : ctx->buf) held += (double)b.cap;
        held += (double)(out->objects.cap + out->begin.cap + out->size.cap + out->mag.cap);
        const double budget = prm.memory_budget ? (double)prm.memory_budget : 0.8 * ((double)free_b + held);
        const double per_child = 38.0 + 48.0 / load + 32.0;
        const double per_survivor = (double)((ctx->h_words[W_MAXSIZE] + 7) / 8 * 8) + 36.0;
        uint64_t kp = N;
        if ((double)ctx->h_words[W_NC] * per_child > budget) {
            // largest number of top-norm parents whose children fit (binary
            // search, as iteration::truncate is probed by the reference)
            uint64_t lo = 0, hi = N;
            key_parent_norm k1{(const double2 *)in->mag.p, tk};
            while (hi - lo > 1) {
                const uint64_t mid = (lo + hi) / 2;
                QD_TRY(radix_select(ctx, ctx->d_words + W_N, N, mid, k1));
                QD_TRY(set_word(ctx, W_TMP, 0));
                k_sum_selected_children<<<grid_for(ctx, N), prim::kThreads, 0, ctx->stream>>>(
                    k1, ctx->d_sel, bufp<uint32_t>(ctx, B_NCHILD), ctx->d_words + W_N,
                    (unsigned long long *)(ctx->d_words + W_TMP));
                QD_TRY(launched(ctx));
                st = read_words(ctx);
                if (st) return st;
                if ((double)ctx->h_words[W_TMP] * per_child <= budget) lo = mid; else hi = mid;
            }
            kp = lo > 0 ? lo : 1;
        }
        if (kp < N) {  // pre-truncate to kp parents and recount
            QD_TRY(ensure(ctx->buf[B_PIDX], kp * sizeof(uint64_t)));
            key_parent_norm k1{(const double2 *)in->mag.p, tk};
            QD_TRY(radix_select(ctx, ctx->d_words + W_N, N, kp, k1));
            prim::lookback lb, lbt, lbs;
            QD_TRY(lookback_chain(ctx, N, 0, lb));
            QD_TRY(lookback_chain(ctx, N, 2, lbt));
            keep_parents kpf{k1, ctx->d_sel, bufp<uint64_t>(ctx, B_PIDX)};
            prim::k_compact_ranked<<<lookback_grid(ctx, N), prim::kThreads, 0, ctx->stream>>>(
                kpf, ctx->d_words + W_N, ctx->d_words + W_NP, lb, lbt);
            NP = kp;
            pidx = bufp<uint64_t>(ctx, B_PIDX);
            QD_TRY(lookback_chain(ctx, N, 1, lbs));
            scan_nchild f{bufp<uint32_t>(ctx, B_NCHILD), pidx};
            prim::k_scan_excl<<<lookback_grid(ctx, NP), prim::kThreads, 0, ctx->stream>>>(
                f, ctx->d_words + W_NP, bufp<uint64_t>(ctx, B_CBEGIN), ctx->d_words + W_NC, lbs);
            tile_map_cap = 0;  // the map of the first scan is stale
            QD_TRY(launched(ctx, 2));
            st = read_words(ctx);
            if (st) return st;
            s.num_parents_kept = NP;
        }
        const double left = budget - (double)ctx->h_words[W_NC] * per_child;
        const double fit = left > per_survivor ? left / per_survivor : 1.0;
        maxc = fit >= 1.8e19 ? ~0ull : (uint64_t)fit;
    }
    const uint64_t NC = ctx->h_words[W_NC];
    const uint64_t maxsize = ctx->h_words[W_MAXSIZE];
    s.num_object = NC;
    s.max_child_size = maxsize;
    parents_view pv{(const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p,
                    (const double2 *)in->mag.p, bufp<uint64_t>(ctx, B_CBEGIN), pidx, NP};
    if (NC == 0) return finish(true);
    if (maxsize > 4096) return QUIDS_ERR_SIZE_BOUND;  // per-thread child buffer bound
    const bool may_truncate = maxc < NC;
    if (!auto_max) {
        // one pass holds every child's records and table with 32-bit child
        // indices; beyond that (or when asked) the step runs in hash ranges
        if (prm.hash_ranges >= 2 || NC >= 0xffffffffull) return kNeedRanges;
        if ((double)NC / load + 1 >= (double)0x7ffffff0ull) return kNeedRanges;  // 31-bit table slots
        const double need = (double)NC * (38.0 + 48.0 / load + (may_truncate ? 32.0 : 0.0));
        if (need > 1e9) {
            size_t free_b = 0, total_b = 0;
            QD_CUDA(cudaMemGetInfo(&free_b, &total_b));
            double held = 0;
            for (auto &b : ctx->buf) held += (double)b.cap;
            // buffers grow with 25 % headroom
            if (need > 0.7 * ((double)free_b + held)) return kNeedRanges;
        }
    } else if (NC >= 0xffffffffull) {
        return QUIDS_ERR_UNSUPPORTED;  // child indices are u32 in the table
    }
    const uint64_t NSB = may_truncate ? maxc : NC;  // bound on the survivors

    // collisions: the open-addressing table, or the partitioned stage
    // (collide.cuh) when QUIDS_FLAG_PARTITION asks for it
    const bool pcs = use_partition(prm, NC);
    uint64_t M = (uint64_t)((double)NC / load) + 1;
    if (M < 1024) M = 1024;
    if (!pcs && M >= 0x7ffffff0ull) return QUIDS_ERR_OOM;  // slot indices are 31-bit (the top bit marks joiners)
    s.table_capacity = pcs ? 0 : M;
    const uint64_t tiles_nc = (NC + prim::kTile - 1) / prim::kTile;
    QD_TRY(ensure(ctx->buf[B_HASH], NC * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_CMAG], NC * sizeof(double2)));
    QD_TRY(ensure(ctx->buf[B_CSIZE], NC * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_SCHILD], NSB * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_LOOKBACK], 4 * (tiles_nc + 2) * sizeof(uint64_t)));
    QD_TRY(ensure(out->begin, (NSB + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(out->size, NSB * sizeof(uint32_t)));
    QD_TRY(ensure(out->mag, NSB * sizeof(double2)));
    QD_TRY(ensure(out->d_total, sizeof(double)));
    if (pcs) {
        QD_TRY(pcs_ensure(ctx, NC, may_truncate));
    } else {
        QD_TRY(ensure(ctx->buf[B_SLOT], NC * sizeof(uint32_t)));
        QD_TRY(ensure(ctx->buf[B_NOTREP], NC));
        QD_TRY(ensure(ctx->buf[B_HASJOIN], NC));
        QD_TRY(ensure(ctx->buf[B_KEYS], (M + 1) * sizeof(prim::table_slot)));
        QD_TRY(ensure(ctx->buf[B_ACC], 4 * (M + 1) * sizeof(uint64_t)));
        if (may_truncate) {
            QD_TRY(ensure(ctx->buf[B_UNORM], NC * sizeof(uint64_t)));
            QD_TRY(ensure(ctx->buf[B_KEEPCAND], NC * sizeof(uint32_t)));
            QD_TRY(ensure(ctx->buf[B_TILECNT], tilecnt_bytes(NC)));
        }
    }

    const uint64_t sym_tiles = (NC + kTileChildren - 1) / kTileChildren;
    QD_TRY(ensure(ctx->buf[B_TILEPAR], (sym_tiles + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_CPAR], NC * sizeof(uint32_t)));

    // the collision table and its fill (slots free, the extra slot's sum, the
    // group marks, the look-back chains of stages 3-4)
    prim::table tb{bufp<prim::table_slot>(ctx, B_KEYS), bufp<unsigned long long>(ctx, B_ACC), M, probe_limit(prm)};
    fill_set ftab{};
    if (!pcs) {
        ftab.p[0] = (unsigned char *)tb.slots, ftab.n[0] = (M + 1) * sizeof(prim::table_slot), ftab.v[0] = 0xff;
        ftab.p[1] = (unsigned char *)(tb.acc + 4 * M), ftab.n[1] = 4 * sizeof(uint64_t), ftab.v[1] = 0;
        ftab.p[2] = bufp<unsigned char>(ctx, B_NOTREP), ftab.n[2] = NC, ftab.v[2] = 0;
        ftab.p[3] = bufp<unsigned char>(ctx, B_HASJOIN), ftab.n[3] = NC, ftab.v[3] = 0;
        ftab.p[4] = bufp<unsigned char>(ctx, B_LOOKBACK), ftab.n[4] = 4 * (tiles_nc + 2) * sizeof(uint64_t),
        ftab.v[4] = 0;
        ftab.count = 5;
    }

    // ---- stage 1: symbolic iteration (src/quids.hpp:647-721); the grouped
    // pass claims the table slots as well
    begin_stage(1);
    bool grouped = false;
    if constexpr (has_grouped<Rule>::value) grouped = fast;
    const bool fused = grouped && !pcs;
    if constexpr (has_grouped<Rule>::value) {
        if (fused)
            QD_TRY(launch_symbolic_grouped(ctx, rule, pv, NC, table_claim{tb, bufp<uint32_t>(ctx, B_SLOT), err},
                                           [&] { return fill(ctx, ftab); }));
        else if (grouped)
            QD_TRY(launch_symbolic_grouped(ctx, rule, pv, NC));
    }
    if (!grouped) {
        if (sym_tiles + 1 > tile_map_cap || bufp<uint64_t>(ctx, B_TILEPAR) != tile_map) {
            k_tile_parents<<<grid_for(ctx, NP), prim::kThreads, 0, ctx->stream>>>(
                bufp<uint64_t>(ctx, B_CBEGIN), NP, sym_tiles, bufp<uint64_t>(ctx, B_TILEPAR));
            QD_TRY(launched(ctx));
        }
        if (maxsize <= 256) {
            QD_TRY((launch_symbolic<single_rule<Rule>, 256>(ctx, rule, pv, NC, fast)));
        } else {
            QD_TRY((launch_symbolic<single_rule<Rule>, 4096>(ctx, rule, pv, NC, fast)));
        }
    }
    end_stage(1);

    const uint32_t align = prm.align_byte_length;
    const prim::publish pb1 = publish_words(ctx, W_DONE_LAYOUT);
    unsigned long long *d_maxnorm = (unsigned long long *)(ctx->d_words + W_MAXNORM);
    if (pcs) {
        // ---- stages 2-4 by partition (src/quids.hpp:726-948): groups, truncation, layout
        begin_stage(2);
        QD_TRY(pcs_stage(ctx, NC, may_truncate, maxc, tk, prm.tolerance, align, out, pb1));
        end_stage(2);
    } else {
        // ---- stage 2: collision table (src/quids.hpp:726-809)
        begin_stage(2);
        if (!fused) QD_TRY(fill(ctx, ftab));
        uint8_t *not_rep = bufp<uint8_t>(ctx, B_NOTREP), *has_join = bufp<uint8_t>(ctx, B_HASJOIN);
        const unsigned long long *d_maxabs = (const unsigned long long *)(ctx->d_words + W_MAXABS);
        {
            direct_src src{bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG)};
            if (!fused) {
                prim::k_table_claim<<<grid_for(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
                    tb, src, ctx->d_words + W_NC, bufp<uint32_t>(ctx, B_SLOT), err);
                QD_TRY(launched(ctx));
            }
            prim::k_table_accumulate<<<grid_for(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
                tb, src, bufp<uint32_t>(ctx, B_SLOT), ctx->d_words + W_NC, d_maxabs, not_rep, has_join);
            QD_TRY(launched(ctx));
        }
        end_stage(2);

        // ---- stage 3 (+4): representatives above tolerance (src/quids.hpp:819-823),
        // truncation (src/quids.hpp:866-900, ties by lower child index) and the
        // output layout (src/quids.hpp:927-948), with the largest survivor norm
        group_view gv{bufp<uint32_t>(ctx, B_SLOT), not_rep, has_join, bufp<double2>(ctx, B_CMAG),
                      bufp<unsigned long long>(ctx, B_ACC), ctx->d_words + W_NC, d_maxabs, prm.tolerance};
        begin_stage(3);
        if (!may_truncate) {
            prim::lookback lbc, lbb;
            lookback_view(ctx, NC, 0, lbc);
            lookback_view(ctx, NC, 1, lbb);
            groups_layout f{gv, bufp<uint32_t>(ctx, B_CSIZE), align, (double2 *)out->mag.p, (uint32_t *)out->size.p,
                            (uint64_t *)out->begin.p, bufp<uint64_t>(ctx, B_SCHILD)};
            prim::k_compact_layout<groups_layout, false><<<lookback_grid(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
                f, ctx->d_words + W_NC, ctx->d_words + W_NS, ctx->d_words + W_OUTBYTES, (uint64_t *)out->begin.p,
                d_maxnorm, lbc, lbb, lbb, pb1);
            QD_TRY(launched(ctx));
            end_stage(3);
        } else {
            uint64_t *gkey = bufp<uint64_t>(ctx, B_UNORM);  // per child: its group's truncation key, or 0
            k_group_keys<<<grid_for(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
                gv, tk, ctx->d_words + W_NC, gkey, (unsigned long long *)(ctx->d_words + W_NU));
            QD_TRY(launched(ctx));
            end_stage(3);
            begin_stage(4);
            QD_TRY(ensure(ctx->buf[B_SELCAND], filter_cap(NC) * sizeof(uint64_t)));
            QD_TRY(radix_select_filtered(ctx, ctx->d_words + W_NC, NC, maxc, key_direct{gkey},
                                         bufp<uint64_t>(ctx, B_SELCAND), filter_cap(NC), ctx->d_words + W_NU));
            prim::lookback lbc, lbb, lbt;
            lookback_view(ctx, NC, 0, lbt);
            lookback_view(ctx, NC, 1, lbc);
            lookback_view(ctx, NC, 2, lbb);
            QD_TRY(list_keep_candidates(ctx, keep_candidate{gkey, ctx->d_sel}, NC));
            const cand_keep_layout kl{{gv, gkey, ctx->d_sel, bufp<uint32_t>(ctx, B_CSIZE), align, (double2 *)out->mag.p,
                                       (uint32_t *)out->size.p, (uint64_t *)out->begin.p, bufp<uint64_t>(ctx, B_SCHILD)},
                                      bufp<uint32_t>(ctx, B_KEEPCAND)};
            prim::k_compact_layout<cand_keep_layout, true><<<lookback_grid(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
                kl, ctx->d_words + W_NCAND, ctx->d_words + W_NS, ctx->d_words + W_OUTBYTES, (uint64_t *)out->begin.p,
                d_maxnorm, lbc, lbb, lbt, pb1);
            QD_TRY(launched(ctx));
            end_stage(4);
        }
}
    st = wait_words(ctx, pb1.seq);  // host wait 2: survivors and their bytes
    if (st) return st;
    const uint64_t NS = ctx->h_words[W_NS];
    const uint64_t NU = (pcs || may_truncate) ? ctx->h_words[W_NU] : NS;
    const uint64_t outbytes = ctx->h_words[W_OUTBYTES];
    s.num_object_after_interferences = NU;
    if (NS == 0) return finish(true);
    QD_TRY(ensure(out->objects, outbytes));

    // ---- stage 5: total probability (src/quids.hpp:1002-1008), exact
    begin_stage(5);
    prim::k_fix_total<<<grid_for(ctx, NS, 4), prim::kThreads, 0, ctx->stream>>>(
        (const double2 *)out->mag.p, ctx->d_words + W_NS, d_maxnorm, (unsigned long long *)(ctx->d_words + W_ACC),
        (unsigned int *)(ctx->d_words + W_DONE), (double *)(ctx->d_words + W_TOTAL),
        (double *)(ctx->d_words + W_FACTOR));
    QD_TRY(launched(ctx));
    QD_CUDA(cudaMemcpyAsync(out->d_total.p, ctx->d_words + W_TOTAL, sizeof(double), cudaMemcpyDeviceToDevice,
                            ctx->stream));
    end_stage(5);

    // ---- stage 6: finalize populate (src/quids.hpp:958-967) + normalisation
    begin_stage(6);
    QD_TRY((launch_populate<single_rule<Rule>, Post>(ctx, rule, pv, NS, out, post, maxsize)));
    end_stage(6);
    out->n = NS;
    out->nbytes = outbytes;
    out->total_pending = true;

    s.num_object_out = NS;
    s.out_bytes = outbytes;
    double sp = (double)in->nbytes, sbar_p = N ? sp / (double)N : 0, sbar_c = NS ? (double)outbytes / NS : 0;
    s.algorithmic_bytes = sp + 24.0 * N + 72.0 * NC + 24.0 * NU + (double)NS * (sbar_p + sbar_c + 24.0);
    return finish(false);
}

template <class Mod>
int apply_modifier(quids_gpu_ctx *ctx, quids_gpu_state *st, const Mod &mod) {
    if (!ctx || !st || st->ctx != ctx) return QUIDS_ERR_BAD_ARG;
    if (st->n == 0) return QUIDS_OK;
    QD_CUDA(cudaSetDevice(ctx->device));
    if (!ctx->buf[B_MODSTATUS].p) {
        QD_TRY(ensure(ctx->buf[B_MODSTATUS], sizeof(uint64_t)));
        QD_CUDA(cudaMemsetAsync(ctx->buf[B_MODSTATUS].p, 0, sizeof(uint64_t), ctx->stream));
    }
    int *merr = bufp<int>(ctx, B_MODSTATUS);
    k_modifier<Mod><<<grid_for(ctx, st->n), prim::kThreads, 0, ctx->stream>>>(
        mod, (char *)st->objects.p, (const uint64_t *)st->begin.p, (const uint32_t *)st->size.p, (double2 *)st->mag.p,
        st->n, merr);
    return launched(ctx);
}

template <class Rule>
int rule_children(quids_gpu_ctx *ctx, quids_gpu_state *in, const Rule &rule, uint64_t *num_children,
                  uint64_t *stride_out, uint8_t *bytes, uint64_t *hash, uint32_t *size, double *magnitude) {
    if (!ctx || !in || in->ctx != ctx || !num_children || !stride_out) return QUIDS_ERR_BAD_ARG;
    QD_CUDA(cudaSetDevice(ctx->device));
    const uint64_t N = in->n;
    QD_CUDA(cudaMemsetAsync(ctx->d_words, 0, W_COUNT_WORDS * sizeof(uint64_t), ctx->stream));
    if (N == 0) {
        *num_children = 0;
        *stride_out = 8;
        return QUIDS_OK;
    }
    QD_TRY(set_word(ctx, W_NP, N));
    QD_TRY(ensure(ctx->buf[B_NCHILD], N * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_LOOKBACK], 3 * ((N + prim::kTile - 1) / prim::kTile + 2) * sizeof(uint64_t)));
    k_num_child<<<grid_for(ctx, N), prim::kThreads, 0, ctx->stream>>>(
        single_rule<Rule>{rule}, (const char *)in->objects.p, (const uint64_t *)in->begin.p,
        (const uint32_t *)in->size.p, N, bufp<uint32_t>(ctx, B_NCHILD),
        (unsigned long long *)(ctx->d_words + W_MAXSIZE), (int *)(ctx->d_words + W_STATUS));
    QD_TRY(launched(ctx));
    QD_TRY(ensure(ctx->buf[B_CBEGIN], (N + 1) * sizeof(uint64_t)));
    {
        prim::lookback lb;
        QD_TRY(lookback_chain(ctx, N, 0, lb));
        scan_nchild f{bufp<uint32_t>(ctx, B_NCHILD), nullptr};
        prim::k_scan_excl<<<lookback_grid(ctx, N), prim::kThreads, 0, ctx->stream>>>(
            f, ctx->d_words + W_NP, bufp<uint64_t>(ctx, B_CBEGIN), ctx->d_words + W_NC, lb);
        QD_TRY(launched(ctx));
    }
    int st = read_words(ctx);
    if (st) return st;
    const uint64_t NC = ctx->h_words[W_NC];
    const uint64_t stride = (ctx->h_words[W_MAXSIZE] + 7) / 8 * 8 + 8;
    *num_children = NC;
    *stride_out = stride;
    if (!bytes || NC == 0) return QUIDS_OK;
    qd_dbuf dbytes, dhash, dsize, dmag;
    int rc = QUIDS_OK;
    if ((rc = ensure(dbytes, NC * stride)) || (rc = ensure(dhash, NC * 8)) || (rc = ensure(dsize, NC * 4)) ||
        (rc = ensure(dmag, NC * 16))) {
        release(dbytes); release(dhash); release(dsize); release(dmag);
        return rc;
    }
    parents_view pv{(const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p,
                    (const double2 *)in->mag.p, bufp<uint64_t>(ctx, B_CBEGIN), nullptr, N};
    QD_CUDA(cudaMemsetAsync(dbytes.p, 0, NC * stride, ctx->stream));
    k_children<Rule><<<grid_for(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
        rule, pv, NC, stride, (char *)dbytes.p, (uint64_t *)dhash.p, (uint32_t *)dsize.p, (double2 *)dmag.p);
    rc = launched(ctx);
    if (!rc) rc = cuda_status(cudaMemcpyAsync(bytes, dbytes.p, NC * stride, cudaMemcpyDeviceToHost, ctx->stream));
    if (!rc && hash) rc = cuda_status(cudaMemcpyAsync(hash, dhash.p, NC * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (!rc && size) rc = cuda_status(cudaMemcpyAsync(size, dsize.p, NC * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (!rc && magnitude)
        rc = cuda_status(cudaMemcpyAsync(magnitude, dmag.p, NC * 16, cudaMemcpyDeviceToHost, ctx->stream));
    if (!rc) rc = cuda_status(cudaStreamSynchronize(ctx->stream));
    release(dbytes); release(dhash); release(dsize); release(dmag);
    return rc;
}

// ------------------------------------------------------------ observables
// sum over objects of obs(object) * |mag|^2 (iteration::average_value,
// src/quids.hpp:208-234): block b sums a fixed chunk in a fixed tree, one
// block sums the partials in order, so the value is deterministic.
constexpr int kObsBlocks = 1024;

template <class Obs>
__global__ void __launch_bounds__(prim::kThreads)
    k_observable_partial(Obs obs, const char *objects, const uint64_t *begin, const uint32_t *size, const double2 *mag,
                         uint64_t n, double *partial) {
    __shared__ double sm[prim::kThreads];
    const uint64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const uint64_t b = (uint64_t)blockIdx.x * chunk, e = b + chunk < n ? b + chunk : n;
    double acc = 0;
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const char *o = objects + begin[i];
        const double2 m = mag[i];
        acc = dadd(acc, dmul(obs(o, o + size[i]), cnorm(mag_t{m.x, m.y})));
    }
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int o = prim::kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] = dadd(sm[threadIdx.x], sm[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

static __global__ void __launch_bounds__(kObsBlocks) k_sum_partials(const double *partial, double *out) {
    __shared__ double sm[kObsBlocks];
    sm[threadIdx.x] = partial[threadIdx.x];
    __syncthreads();
    for (int o = kObsBlocks / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] = dadd(sm[threadIdx.x], sm[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sm[0];
}

template <class Obs>
int average_value(quids_gpu_ctx *ctx, quids_gpu_state *st, const Obs &obs, double *value) {
    if (!ctx || !st || st->ctx != ctx || !value) return QUIDS_ERR_BAD_ARG;
    *value = 0;
    if (st->n == 0) return QUIDS_OK;  // src/quids.hpp:210-211
    QD_CUDA(cudaSetDevice(ctx->device));
    QD_TRY(ensure(ctx->buf[B_TILENORM], (kObsBlocks + 1) * sizeof(double)));
    double *partial = bufp<double>(ctx, B_TILENORM);
    k_observable_partial<Obs><<<kObsBlocks, prim::kThreads, 0, ctx->stream>>>(
        obs, (const char *)st->objects.p, (const uint64_t *)st->begin.p, (const uint32_t *)st->size.p,
        (const double2 *)st->mag.p, st->n, partial);
    k_sum_partials<<<1, kObsBlocks, 0, ctx->stream>>>(partial, partial + kObsBlocks);
    QD_TRY(launched(ctx, 2));
    QD_CUDA(cudaMemcpyAsync(value, partial + kObsBlocks, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    return QUIDS_OK;
}

}  // namespace qd::engine
