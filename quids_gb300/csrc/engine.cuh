// engine.cuh -- the GB300 rule step: device state, scratch memory, the
// templated per-rule kernels and the host orchestration of
// quids::simulate(iteration, rule, next_iteration, sy_it, max_num_object)
// (src/quids.hpp:448-543) and of apply_modifier (src/quids.hpp:973-980).
//
// A user rule is any struct with the reference's callbacks as __device__
// members (see rules_qc.cuh); `simulate_rule<Rule>` instantiates the step
// for it.
#pragma once
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <unordered_set>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/quids_gpu.h"
#include "prims.cuh"
#include "qd_common.cuh"

#define QUIDS_FLAG_NO_FAST_HASH 1u

// --------------------------------------------------------------- buffers
struct qd_dbuf {
    void *p = nullptr;
    size_t cap = 0;
};

enum qd_buf_id {
    B_NCHILD,      // u32 [N]
    B_CBEGIN,      // u64 [NP+1]
    B_PIDX,        // u64 [NP] kept parents (pre-truncation)
    B_PKEY,        // unused
    B_HASH,        // u64 [NC]
    B_CMAG,        // double2 [NC]
    B_CSIZE,       // u32 [NC]
    B_SLOT,        // u32 [NC]
    B_KEYS,        // u64 [M]
    B_REP,         // u64 [M+1]
    B_ACC,         // u64 [4(M+1)]
    B_UCHILD,      // u64 [NU]
    B_UMAG,        // double2 [NU]
    B_UNORM,       // u64 [NU]
    B_UHASH,       // u64 [NU]
    B_SCHILD,      // u64 [NS]
    B_SMAG,        // double2 [NS]
    B_LOOKBACK,    // u64 [tiles + 1]
    B_NORM,        // double [kNormBlocks]
    B_MODSTATUS,   // int: sticky error of modifier launches (checked at the next step)
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
    W_COUNT_WORDS = 16
};

struct quids_gpu_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    qd_dbuf buf[B_COUNT];
    uint64_t *d_words = nullptr;             // W_COUNT_WORDS
    uint64_t *h_words = nullptr;             // pinned mirror
    qd::prim::select_state *d_sel = nullptr; // two states
    unsigned long long *d_hist = nullptr;    // 256
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_stage[16] = {};  // start/end of the 8 stages of a step
    uint64_t launches = 0;          // kernels launched by this context
    // live states: destroying the context releases their device memory and
    // orphans them, so states may be destroyed after their context
    std::unordered_set<struct quids_gpu_state *> states;
};

struct quids_gpu_state {
    quids_gpu_ctx *ctx = nullptr;  // null once the context is destroyed
    uint64_t n = 0;
    uint64_t nbytes = 0;
    double total_proba = 1;
    qd_dbuf objects, begin, size, mag;
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

inline int ensure(qd_dbuf &b, size_t bytes) {
    if (bytes == 0) bytes = 8;
    if (b.cap >= bytes) return QUIDS_OK;
    if (b.p) {
        cudaError_t e = cudaFree(b.p);
        b.p = nullptr;
        b.cap = 0;
        if (e != cudaSuccess) return cuda_status(e);
    }
    size_t want = bytes + bytes / 4;
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
inline void release(qd_dbuf &b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
}

template <class T>
inline T *bufp(quids_gpu_ctx *ctx, qd_buf_id id) {
    return (T *)ctx->buf[id].p;
}

inline unsigned grid_for(quids_gpu_ctx *ctx, uint64_t n, int per_sm = 8) {
    uint64_t g = (n + prim::kThreads - 1) / prim::kThreads;
    uint64_t cap = (uint64_t)ctx->num_sms * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (unsigned)g;
}

// zeroed look-back workspace for a single-pass scan/compaction over n items
inline int lookback_ws(quids_gpu_ctx *ctx, uint64_t n, prim::lookback &lb, unsigned &grid) {
    uint64_t tiles = (n + prim::kTile - 1) / prim::kTile;
    QD_TRY(ensure(ctx->buf[B_LOOKBACK], (tiles + 2) * sizeof(uint64_t)));
    uint64_t *ws = bufp<uint64_t>(ctx, B_LOOKBACK);
    QD_CUDA(cudaMemsetAsync(ws, 0, (tiles + 2) * sizeof(uint64_t), ctx->stream));
    lb.status = ws + 1;
    lb.counter = (uint32_t *)ws;
    lb.err = (int *)(ctx->d_words + W_STATUS);
    uint64_t g = tiles < 1 ? 1 : tiles;
    uint64_t cap = (uint64_t)ctx->num_sms * 4;
    grid = (unsigned)(g < cap ? g : cap);
    return QUIDS_OK;
}

inline int read_words(quids_gpu_ctx *ctx) {
    QD_CUDA(cudaMemcpyAsync(ctx->h_words, ctx->d_words, W_COUNT_WORDS * sizeof(uint64_t),
                            cudaMemcpyDeviceToHost, ctx->stream));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    int st = (int)(int64_t)ctx->h_words[W_STATUS];
    return st;
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

inline void stage_begin(quids_gpu_ctx *ctx, int k) { cudaEventRecord(ctx->ev_stage[2 * k], ctx->stream); }
inline void stage_end(quids_gpu_ctx *ctx, int k) { cudaEventRecord(ctx->ev_stage[2 * k + 1], ctx->stream); }

// ---------------------------------------------------------- rule traits
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

// ------------------------------------------------------- per-rule kernels
template <class Rule>
__global__ void __launch_bounds__(prim::kThreads)
    k_num_child(Rule rule, const char *objects, const uint64_t *begin, const uint32_t *size, uint64_t n,
                uint32_t *nchild, unsigned long long *d_maxsize, int *err) {
    uint32_t mx = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const char *pb = objects + begin[i];
        if (!object_fits(rule, size[i])) {
            nchild[i] = 0;
            prim::set_error(err, QUIDS_ERR_BAD_ARG);
            continue;
        }
        uint32_t nc, mcs;
        rule.get_num_child(pb, pb + size[i], nc, mcs);
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
};

// Symbolic iteration (src/quids.hpp:705-719): per child, its magnitude,
// size and hash.  FAST: the rule's hash_child; otherwise populate_child into
// a per-thread buffer of MAXC bytes followed by the rule's hasher.
template <class Rule, int MAXC, bool FAST>
__global__ void __launch_bounds__(prim::kThreads)
    k_symbolic(Rule rule, parents_view pv, const uint64_t *d_nc, uint64_t *hash, double2 *cmag, uint32_t *csize,
               unsigned long long *d_maxabs, int *err) {
    const uint64_t nc = *d_nc;
    double mx = 0;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t p = parent_of(pv.cbeg, pv.np, c);
        uint64_t oid = pv.pidx ? pv.pidx[p] : p;
        uint32_t cid = (uint32_t)(c - pv.cbeg[p]);
        const char *pb = pv.objects + pv.begin[oid];
        const char *pe = pb + pv.size[oid];
        double2 pm = pv.mag[oid];
        mag_t m{pm.x, pm.y};
        uint32_t sz = 0;
        uint64_t h;
        if constexpr (FAST) {
            h = rule.hash_child(pb, pe, cid, sz, m);
        } else {
            uint64_t buf[MAXC / 8];
            rule.populate_child(pb, pe, (char *)buf, cid, sz, m);
            if (sz > MAXC) {
                prim::set_error(err, QUIDS_ERR_SIZE_BOUND);
                sz = MAXC;
            }
            h = rule_hash(rule, (const char *)buf, (const char *)buf + sz);
        }
        hash[c] = h;
        cmag[c] = make_double2(m.re, m.im);
        csize[c] = sz;
        double a = fabs(m.re) > fabs(m.im) ? fabs(m.re) : fabs(m.im);
        mx = mx > a ? mx : a;
    }
    unsigned long long bits = (unsigned long long)__double_as_longlong(mx);
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long y = __shfl_xor_sync(0xffffffffu, bits, o);
        bits = bits > y ? bits : y;
    }
    if ((threadIdx.x & 31) == 0 && bits) atomicMax(d_maxabs, bits);
}

// Finalize (src/quids.hpp:958-967): populate_child_simple of each survivor
// into the packed output, padding zeroed.
template <class Rule, int MAXC>
__global__ void __launch_bounds__(prim::kThreads)
    k_populate(Rule rule, parents_view pv, const uint64_t *schild, const uint64_t *d_ns, const uint64_t *obegin,
               const uint32_t *osize, char *objects, int *err) {
    const uint64_t ns = *d_ns;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t c = schild[i];
        uint64_t p = parent_of(pv.cbeg, pv.np, c);
        uint64_t oid = pv.pidx ? pv.pidx[p] : p;
        uint32_t cid = (uint32_t)(c - pv.cbeg[p]);
        const char *pb = pv.objects + pv.begin[oid];
        const char *pe = pb + pv.size[oid];
        uint64_t buf[MAXC / 8];
        rule_populate_simple(rule, pb, pe, (char *)buf, cid);
        uint32_t sz = osize[i];
        if (sz > MAXC) {
            prim::set_error(err, QUIDS_ERR_SIZE_BOUND);
            sz = MAXC;
        }
        char *dst = objects + obegin[i];
        copy_bytes(dst, (const char *)buf, sz);
        for (uint64_t k = obegin[i] + sz; k < obegin[i + 1]; ++k) objects[k] = 0;
    }
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
               int *err) {
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

// a child is kept after collisions if it is its group's representative and
// the group's summed norm is above tolerance (src/quids.hpp:785-823)
struct compact_groups {
    const uint32_t *slot_of;
    const uint64_t *rep;
    const unsigned long long *acc;
    const uint64_t *hash;
    const uint64_t *d_nc;
    const unsigned long long *d_maxabs;
    double tolerance;
    uint64_t *uchild;
    double2 *umag;
    uint64_t *unorm;
    uint64_t *uhash;
    __device__ bool select(uint64_t c) const {
        uint32_t s = slot_of[c];
        if (s == 0xffffffffu) return false;
        if (rep[s] != c) return false;
        int F = fix_scale(__longlong_as_double((long long)*d_maxabs), *d_nc);
        double re = from_fix(fix128{acc[4ull * s], acc[4ull * s + 1]}, F);
        double im = from_fix(fix128{acc[4ull * s + 2], acc[4ull * s + 3]}, F);
        return cnorm(mag_t{re, im}) > tolerance;
    }
    __device__ void emit(uint64_t c, uint64_t j) const {
        uint32_t s = slot_of[c];
        int F = fix_scale(__longlong_as_double((long long)*d_maxabs), *d_nc);
        double re = from_fix(fix128{acc[4ull * s], acc[4ull * s + 1]}, F);
        double im = from_fix(fix128{acc[4ull * s + 2], acc[4ull * s + 3]}, F);
        uchild[j] = c;
        umag[j] = make_double2(re, im);
        double nrm = cnorm(mag_t{re, im});
        unorm[j] = (uint64_t)__double_as_longlong(nrm);
        uhash[j] = hash[c];
    }
};

// radix-select keys
struct key_unorm {
    const uint64_t *unorm;
    __device__ uint64_t key(uint64_t i) const { return unorm[i]; }
    __device__ bool eligible(uint64_t) const { return true; }
};
struct key_uhash_ties {
    const uint64_t *unorm;
    const uint64_t *uhash;
    const prim::select_state *first;
    __device__ uint64_t key(uint64_t i) const { return uhash[i]; }
    __device__ bool eligible(uint64_t i) const { return unorm[i] == first->prefix; }
};
struct key_parent_norm {
    const double2 *mag;
    __device__ uint64_t key(uint64_t i) const {
        double2 m = mag[i];
        return (uint64_t)__double_as_longlong(cnorm(mag_t{m.x, m.y}));
    }
    __device__ bool eligible(uint64_t) const { return true; }
};
struct key_parent_index_ties {
    const double2 *mag;
    const prim::select_state *first;
    __device__ uint64_t key(uint64_t i) const { return i; }
    __device__ bool eligible(uint64_t i) const {
        double2 m = mag[i];
        return (uint64_t)__double_as_longlong(cnorm(mag_t{m.x, m.y})) == first->prefix;
    }
};

static __global__ void k_select_init(prim::select_state *st, const uint64_t *d_n, uint64_t k) {
    prim::select_state s{};
    s.k_rem = k;
    s.active = k < *d_n ? 1u : 0u;
    st[0] = s;
    st[1] = prim::select_state{};
}
// second selection among threshold ties, only when not all ties are kept
static __global__ void k_select_ties_init(prim::select_state *st) {
    prim::select_state s{};
    s.k_rem = st[0].k_rem;
    s.active = (st[0].active && st[0].k_rem < st[0].n_equal) ? 1u : 0u;
    st[1] = s;
}

struct keep_truncated {
    const uint64_t *unorm;
    const uint64_t *uhash;
    const uint64_t *uchild;
    const double2 *umag;
    const prim::select_state *st;
    uint64_t *schild;
    double2 *smag;
    __device__ bool select(uint64_t i) const {
        if (!st[0].active) return true;
        uint64_t k = unorm[i];
        if (k > st[0].prefix) return true;
        if (k < st[0].prefix) return false;
        return !st[1].active || uhash[i] <= st[1].prefix;
    }
    __device__ void emit(uint64_t i, uint64_t j) const {
        schild[j] = uchild[i];
        smag[j] = umag[i];
    }
};

struct keep_parents {
    const double2 *mag;
    const prim::select_state *st;
    uint64_t *pidx;
    __device__ bool select(uint64_t i) const {
        if (!st[0].active) return true;
        double2 m = mag[i];
        uint64_t k = (uint64_t)__double_as_longlong(cnorm(mag_t{m.x, m.y}));
        if (k > st[0].prefix) return true;
        if (k < st[0].prefix) return false;
        return !st[1].active || i <= st[1].prefix;
    }
    __device__ void emit(uint64_t i, uint64_t j) const { pidx[j] = i; }
};

// output layout: size, magnitude and padded size of survivor i
struct scan_out_sizes {
    const uint64_t *schild;
    const double2 *smag;
    const uint32_t *csize;
    uint32_t *osize;
    double2 *omag;
    uint32_t align;
    __device__ uint64_t operator()(uint64_t i) const {
        uint32_t sz = csize[schild[i]];
        osize[i] = sz;
        omag[i] = smag[i];
        uint32_t pad = 0;
        if (align > 1) {
            pad = align - sz % align;
            if (pad == align) pad = 0;
        }
        return (uint64_t)sz + pad;
    }
};

// ------------------------------------------------------------ radix select
// Runs the 8 passes of a top-k selection (and the tie passes) on the stream.
template <class K1, class K2>
inline int radix_select(quids_gpu_ctx *ctx, const uint64_t *d_n, uint64_t n_host, uint64_t k, K1 k1, K2 k2,
                        bool tie_descending) {
    unsigned grid = grid_for(ctx, n_host);
    k_select_init<<<1, 1, 0, ctx->stream>>>(ctx->d_sel, d_n, k);
    QD_CUDA(cudaMemsetAsync(ctx->d_hist, 0, 256 * sizeof(unsigned long long), ctx->stream));
    for (int shift = 56; shift >= 0; shift -= 8) {
        prim::k_radix_hist<<<grid, prim::kThreads, 0, ctx->stream>>>(k1, d_n, ctx->d_sel, shift, ctx->d_hist);
        prim::k_radix_pick<<<1, 32, 0, ctx->stream>>>(ctx->d_sel, ctx->d_hist, shift, true);
    }
    k_select_ties_init<<<1, 1, 0, ctx->stream>>>(ctx->d_sel);
    for (int shift = 56; shift >= 0; shift -= 8) {
        prim::k_radix_hist<<<grid, prim::kThreads, 0, ctx->stream>>>(k2, d_n, ctx->d_sel + 1, shift, ctx->d_hist);
        prim::k_radix_pick<<<1, 32, 0, ctx->stream>>>(ctx->d_sel + 1, ctx->d_hist, shift, tie_descending);
    }
    return launched(ctx, 34);
}

inline uint64_t next_pow2(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}
inline int ilog2(uint64_t v) {
    int l = 0;
    while ((1ull << l) < v) ++l;
    return l;
}

// ------------------------------------------------------------- the step
template <class Rule, int MAXC>
inline int launch_symbolic(quids_gpu_ctx *ctx, const Rule &rule, const parents_view &pv, uint64_t nc, bool fast) {
    unsigned grid = grid_for(ctx, nc);
    uint64_t *d_nc = ctx->d_words + W_NC;
    unsigned long long *d_maxabs = (unsigned long long *)(ctx->d_words + W_MAXABS);
    int *err = (int *)(ctx->d_words + W_STATUS);
    if constexpr (has_hash_child<Rule>::value) {
        if (fast) {
            k_symbolic<Rule, 8, true><<<grid, prim::kThreads, 0, ctx->stream>>>(
                rule, pv, d_nc, bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG), bufp<uint32_t>(ctx, B_CSIZE),
                d_maxabs, err);
            return launched(ctx);
        }
    }
    k_symbolic<Rule, MAXC, false><<<grid, prim::kThreads, 0, ctx->stream>>>(
        rule, pv, d_nc, bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG), bufp<uint32_t>(ctx, B_CSIZE), d_maxabs,
        err);
    return launched(ctx);
}

template <class Rule, int MAXC>
inline int launch_populate(quids_gpu_ctx *ctx, const Rule &rule, const parents_view &pv, const uint64_t *schild,
                           uint64_t ns, quids_gpu_state *out) {
    unsigned grid = grid_for(ctx, ns);
    k_populate<Rule, MAXC><<<grid, prim::kThreads, 0, ctx->stream>>>(
        rule, pv, schild, ctx->d_words + W_NS, (const uint64_t *)out->begin.p, (const uint32_t *)out->size.p,
        (char *)out->objects.p, (int *)(ctx->d_words + W_STATUS));
    return launched(ctx);
}

inline int normalize(quids_gpu_ctx *ctx, quids_gpu_state *st) {
    QD_TRY(ensure(ctx->buf[B_NORM], prim::kNormBlocks * sizeof(double)));
    double *partial = bufp<double>(ctx, B_NORM);
    prim::k_norm_partial<<<prim::kNormBlocks, prim::kThreads, 0, ctx->stream>>>((const double2 *)st->mag.p,
                                                                              ctx->d_words + W_NS, partial);
    prim::k_norm_final<<<1, 512, 0, ctx->stream>>>(partial, prim::kNormBlocks, (double *)(ctx->d_words + W_TOTAL),
                                                  (double *)(ctx->d_words + W_FACTOR));
    prim::k_norm_scale<<<grid_for(ctx, st->n ? st->n : 1), prim::kThreads, 0, ctx->stream>>>(
        (double2 *)st->mag.p, ctx->d_words + W_NS, (const double *)(ctx->d_words + W_FACTOR));
    return launched(ctx, 3);
}

inline int ensure_state(quids_gpu_state *st, uint64_t n, uint64_t nbytes) {
    QD_TRY(ensure(st->objects, nbytes));
    QD_TRY(ensure(st->begin, (n + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(st->size, n * sizeof(uint32_t)));
    QD_TRY(ensure(st->mag, n * sizeof(double2)));
    return QUIDS_OK;
}

template <class Rule>
int simulate_rule(quids_gpu_ctx *ctx, quids_gpu_state *in, const Rule &rule, quids_gpu_state *out,
                  const quids_gpu_params &prm, quids_gpu_step_stats *stats) {
    if (!ctx || !in || !out || in == out || in->ctx != ctx || out->ctx != ctx) return QUIDS_ERR_BAD_ARG;
    if (!prm.simple_truncation) return QUIDS_ERR_UNSUPPORTED;
    if (prm.max_num_object == 0) return QUIDS_ERR_UNSUPPORTED;
    QD_CUDA(cudaSetDevice(ctx->device));
    const uint64_t N = in->n;
    const uint64_t maxn = prm.max_num_object;
    const double load = prm.table_load_factor > 0 && prm.table_load_factor < 0.95 ? prm.table_load_factor : 0.5;
    const uint64_t launches0 = ctx->launches;
    quids_gpu_step_stats s{};
    s.num_parents = N;
    bool stage_used[8] = {};
    auto finish_empty = [&]() -> int {
        out->n = 0;
        out->nbytes = 0;
        out->total_proba = 0;  // normalize() of an empty state (src/quids.hpp:986-992)
        QD_TRY(ensure_state(out, 0, 8));
        QD_CUDA(cudaMemsetAsync(out->begin.p, 0, sizeof(uint64_t), ctx->stream));
        QD_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
        QD_CUDA(cudaStreamSynchronize(ctx->stream));
        cudaEventElapsedTime(&s.ms_total, ctx->ev0, ctx->ev1);
        s.kernel_launches = ctx->launches - launches0;
        if (stats) *stats = s;
        return QUIDS_OK;
    };
    QD_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    QD_CUDA(cudaMemsetAsync(ctx->d_words, 0, W_COUNT_WORDS * sizeof(uint64_t), ctx->stream));
    if (ctx->buf[B_MODSTATUS].p) {  // an earlier modifier met an unfit object
        k_take_status<<<1, 1, 0, ctx->stream>>>(bufp<int>(ctx, B_MODSTATUS), ctx->d_words + W_STATUS);
        QD_TRY(launched(ctx));
    }
    if (N == 0) return finish_empty();
    int *err = (int *)(ctx->d_words + W_STATUS);

    // ---- stage 0: num_child (src/quids.hpp:548-569), parent pre-truncation
    // (src/quids.hpp:613-642, ties by lower index), child offsets (:666-673)
    stage_begin(ctx, 0);
    stage_used[0] = true;
    QD_TRY(set_word(ctx, W_N, N));
    QD_TRY(ensure(ctx->buf[B_NCHILD], N * sizeof(uint32_t)));
    k_num_child<Rule><<<grid_for(ctx, N), prim::kThreads, 0, ctx->stream>>>(
        rule, (const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p, N,
        bufp<uint32_t>(ctx, B_NCHILD), (unsigned long long *)(ctx->d_words + W_MAXSIZE), err);
    QD_TRY(launched(ctx));
    uint64_t NP = N;
    const uint64_t *pidx = nullptr;
    if (maxn < N) {
        QD_TRY(ensure(ctx->buf[B_PIDX], maxn * sizeof(uint64_t)));
        key_parent_norm k1{(const double2 *)in->mag.p};
        key_parent_index_ties k2{(const double2 *)in->mag.p, ctx->d_sel};
        QD_TRY(radix_select(ctx, ctx->d_words + W_N, N, maxn, k1, k2, false));
        prim::lookback lb;
        unsigned g;
        QD_TRY(lookback_ws(ctx, N, lb, g));
        keep_parents kp{(const double2 *)in->mag.p, ctx->d_sel, bufp<uint64_t>(ctx, B_PIDX)};
        prim::k_compact<<<g, prim::kThreads, 0, ctx->stream>>>(kp, ctx->d_words + W_N, ctx->d_words + W_NP, lb);
        QD_TRY(launched(ctx));
        NP = maxn;
        pidx = bufp<uint64_t>(ctx, B_PIDX);
    } else {
        QD_TRY(set_word(ctx, W_NP, N));
    }
    s.num_parents_kept = NP;
    QD_TRY(ensure(ctx->buf[B_CBEGIN], (NP + 1) * sizeof(uint64_t)));
    {
        prim::lookback lb;
        unsigned g;
        QD_TRY(lookback_ws(ctx, NP, lb, g));
        scan_nchild f{bufp<uint32_t>(ctx, B_NCHILD), pidx};
        prim::k_scan_excl<<<g, prim::kThreads, 0, ctx->stream>>>(f, ctx->d_words + W_NP, bufp<uint64_t>(ctx, B_CBEGIN),
                                                               ctx->d_words + W_NC, lb);
        QD_TRY(launched(ctx));
    }
    stage_end(ctx, 0);
    int st = read_words(ctx);
    if (st) return st;
    const uint64_t NC = ctx->h_words[W_NC];
    const uint64_t maxsize = ctx->h_words[W_MAXSIZE];
    s.num_object = NC;
    s.max_child_size = maxsize;
    parents_view pv{(const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p,
                    (const double2 *)in->mag.p, bufp<uint64_t>(ctx, B_CBEGIN), pidx, NP};
    if (NC == 0) return finish_empty();
    const bool fast = !(prm.reserved & QUIDS_FLAG_NO_FAST_HASH);
    if (maxsize > 4096) return QUIDS_ERR_SIZE_BOUND;  // per-thread child buffer bound

    // ---- stage 1: symbolic iteration (src/quids.hpp:647-721)
    QD_TRY(ensure(ctx->buf[B_HASH], NC * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_CMAG], NC * sizeof(double2)));
    QD_TRY(ensure(ctx->buf[B_CSIZE], NC * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_SLOT], NC * sizeof(uint32_t)));
    uint64_t M = next_pow2((uint64_t)((double)NC / load) + 1);
    if (M < 1024) M = 1024;
    if (M > (1ull << 31)) return QUIDS_ERR_OOM;  // slot indices (and the extra slot M) are u32
    s.table_capacity = M;
    QD_TRY(ensure(ctx->buf[B_KEYS], M * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_REP], (M + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_ACC], 4 * (M + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_UCHILD], NC * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_UMAG], NC * sizeof(double2)));
    QD_TRY(ensure(ctx->buf[B_UNORM], NC * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_UHASH], NC * sizeof(uint64_t)));
    stage_begin(ctx, 1);
    stage_used[1] = true;
    if (maxsize <= 256) {
        QD_TRY((launch_symbolic<Rule, 256>(ctx, rule, pv, NC, fast)));
    } else {
        QD_TRY((launch_symbolic<Rule, 4096>(ctx, rule, pv, NC, fast)));
    }
    stage_end(ctx, 1);

    // ---- stage 2: collision table (src/quids.hpp:726-809)
    stage_begin(ctx, 2);
    stage_used[2] = true;
    QD_CUDA(cudaMemsetAsync(ctx->buf[B_KEYS].p, 0xff, M * sizeof(uint64_t), ctx->stream));
    QD_CUDA(cudaMemsetAsync(ctx->buf[B_REP].p, 0xff, (M + 1) * sizeof(uint64_t), ctx->stream));
    QD_CUDA(cudaMemsetAsync(ctx->buf[B_ACC].p, 0, 4 * (M + 1) * sizeof(uint64_t), ctx->stream));
    prim::table tb{bufp<uint64_t>(ctx, B_KEYS), bufp<uint64_t>(ctx, B_REP), bufp<unsigned long long>(ctx, B_ACC), M - 1,
                   ilog2(M), (uint32_t)(M < 65536 ? M : 65536)};
    prim::k_table_insert<<<grid_for(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
        tb, bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG), ctx->d_words + W_NC,
        (const unsigned long long *)(ctx->d_words + W_MAXABS), bufp<uint32_t>(ctx, B_SLOT), err);
    QD_TRY(launched(ctx));
    stage_end(ctx, 2);

    // ---- stage 3: representatives with norm > tolerance, in symbolic order (src/quids.hpp:819-823)
    stage_begin(ctx, 3);
    stage_used[3] = true;
    {
        prim::lookback lb;
        unsigned g;
        QD_TRY(lookback_ws(ctx, NC, lb, g));
        compact_groups cg{bufp<uint32_t>(ctx, B_SLOT), bufp<uint64_t>(ctx, B_REP), bufp<unsigned long long>(ctx, B_ACC),
                          bufp<uint64_t>(ctx, B_HASH), ctx->d_words + W_NC,
                          (const unsigned long long *)(ctx->d_words + W_MAXABS), prm.tolerance,
                          bufp<uint64_t>(ctx, B_UCHILD), bufp<double2>(ctx, B_UMAG), bufp<uint64_t>(ctx, B_UNORM),
                          bufp<uint64_t>(ctx, B_UHASH)};
        prim::k_compact<<<g, prim::kThreads, 0, ctx->stream>>>(cg, ctx->d_words + W_NC, ctx->d_words + W_NU, lb);
        QD_TRY(launched(ctx));
    }
    stage_end(ctx, 3);
    st = read_words(ctx);
    if (st) return st;
    const uint64_t NU = ctx->h_words[W_NU];
    s.num_object_after_interferences = NU;
    if (NU == 0) return finish_empty();

    // ---- stage 4: truncation (src/quids.hpp:866-900), ties by lower hash
    const uint64_t *schild = bufp<uint64_t>(ctx, B_UCHILD);
    const double2 *smag = bufp<double2>(ctx, B_UMAG);
    uint64_t NS = NU;
    if (maxn < NU) {
        QD_TRY(ensure(ctx->buf[B_SCHILD], maxn * sizeof(uint64_t)));
        QD_TRY(ensure(ctx->buf[B_SMAG], maxn * sizeof(double2)));
        stage_begin(ctx, 4);
        stage_used[4] = true;
        key_unorm k1{bufp<uint64_t>(ctx, B_UNORM)};
        key_uhash_ties k2{bufp<uint64_t>(ctx, B_UNORM), bufp<uint64_t>(ctx, B_UHASH), ctx->d_sel};
        QD_TRY(radix_select(ctx, ctx->d_words + W_NU, NU, maxn, k1, k2, false));
        prim::lookback lb;
        unsigned g;
        QD_TRY(lookback_ws(ctx, NU, lb, g));
        keep_truncated kt{bufp<uint64_t>(ctx, B_UNORM), bufp<uint64_t>(ctx, B_UHASH), bufp<uint64_t>(ctx, B_UCHILD),
                          bufp<double2>(ctx, B_UMAG), ctx->d_sel, bufp<uint64_t>(ctx, B_SCHILD),
                          bufp<double2>(ctx, B_SMAG)};
        prim::k_compact<<<g, prim::kThreads, 0, ctx->stream>>>(kt, ctx->d_words + W_NU, ctx->d_words + W_NS, lb);
        QD_TRY(launched(ctx));
        stage_end(ctx, 4);
        schild = bufp<uint64_t>(ctx, B_SCHILD);
        smag = bufp<double2>(ctx, B_SMAG);
        NS = maxn;
    } else {
        QD_TRY(set_word(ctx, W_NS, NU));
    }

    // ---- stage 5: output layout (src/quids.hpp:927-948)
    QD_TRY(ensure(out->begin, (NS + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(out->size, NS * sizeof(uint32_t)));
    QD_TRY(ensure(out->mag, NS * sizeof(double2)));
    stage_begin(ctx, 5);
    stage_used[5] = true;
    {
        prim::lookback lb;
        unsigned g;
        QD_TRY(lookback_ws(ctx, NS, lb, g));
        scan_out_sizes f{schild, smag, bufp<uint32_t>(ctx, B_CSIZE), (uint32_t *)out->size.p, (double2 *)out->mag.p,
                         prm.align_byte_length};
        prim::k_scan_excl<<<g, prim::kThreads, 0, ctx->stream>>>(f, ctx->d_words + W_NS, (uint64_t *)out->begin.p,
                                                               ctx->d_words + W_OUTBYTES, lb);
        QD_TRY(launched(ctx));
    }
    stage_end(ctx, 5);
    st = read_words(ctx);
    if (st) return st;
    const uint64_t outbytes = ctx->h_words[W_OUTBYTES];
    QD_TRY(ensure(out->objects, outbytes));

    // ---- stage 6: finalize populate (src/quids.hpp:958-967)
    stage_begin(ctx, 6);
    stage_used[6] = true;
    if (maxsize <= 256) {
        QD_TRY((launch_populate<Rule, 256>(ctx, rule, pv, schild, NS, out)));
    } else {
        QD_TRY((launch_populate<Rule, 4096>(ctx, rule, pv, schild, NS, out)));
    }
    stage_end(ctx, 6);
    out->n = NS;
    out->nbytes = outbytes;

    // ---- stage 7: normalize (src/quids.hpp:985-1017)
    stage_begin(ctx, 7);
    stage_used[7] = true;
    QD_TRY(normalize(ctx, out));
    stage_end(ctx, 7);
    QD_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    st = read_words(ctx);
    if (st) return st;
    std::memcpy(&out->total_proba, &ctx->h_words[W_TOTAL], sizeof(double));
    cudaEventElapsedTime(&s.ms_total, ctx->ev0, ctx->ev1);
    for (int k = 0; k < 8; ++k)
        if (stage_used[k]) cudaEventElapsedTime(&s.stage_ms[k], ctx->ev_stage[2 * k], ctx->ev_stage[2 * k + 1]);

    s.num_object_out = NS;
    s.out_bytes = outbytes;
    s.total_proba = out->total_proba;
    s.kernel_launches = ctx->launches - launches0;
    double sp = (double)in->nbytes, sbar_p = N ? sp / (double)N : 0, sbar_c = NS ? (double)outbytes / NS : 0;
    s.algorithmic_bytes = sp + 24.0 * N + 72.0 * NC + 24.0 * NU + (double)NS * (sbar_p + sbar_c + 24.0);
    if (stats) *stats = s;
    return QUIDS_OK;
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
    k_num_child<Rule><<<grid_for(ctx, N), prim::kThreads, 0, ctx->stream>>>(
        rule, (const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p, N,
        bufp<uint32_t>(ctx, B_NCHILD), (unsigned long long *)(ctx->d_words + W_MAXSIZE),
        (int *)(ctx->d_words + W_STATUS));
    QD_TRY(ensure(ctx->buf[B_CBEGIN], (N + 1) * sizeof(uint64_t)));
    {
        prim::lookback lb;
        unsigned g;
        QD_TRY(lookback_ws(ctx, N, lb, g));
        scan_nchild f{bufp<uint32_t>(ctx, B_NCHILD), nullptr};
        prim::k_scan_excl<<<g, prim::kThreads, 0, ctx->stream>>>(f, ctx->d_words + W_NP, bufp<uint64_t>(ctx, B_CBEGIN),
                                                               ctx->d_words + W_NC, lb);
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
    rc = cuda_status(cudaGetLastError());
    if (!rc) rc = cuda_status(cudaMemcpyAsync(bytes, dbytes.p, NC * stride, cudaMemcpyDeviceToHost, ctx->stream));
    if (!rc && hash) rc = cuda_status(cudaMemcpyAsync(hash, dhash.p, NC * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (!rc && size) rc = cuda_status(cudaMemcpyAsync(size, dsize.p, NC * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (!rc && magnitude)
        rc = cuda_status(cudaMemcpyAsync(magnitude, dmag.p, NC * 16, cudaMemcpyDeviceToHost, ctx->stream));
    if (!rc) rc = cuda_status(cudaStreamSynchronize(ctx->stream));
    release(dbytes); release(dhash); release(dsize); release(dmag);
    return rc;
}

}  // namespace qd::engine
