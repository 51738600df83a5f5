// ranges.cuh -- rule steps whose children do not fit one pass, in
// hash-range passes.
//
// One pass holds every child's records and the collision table at once,
// with 32-bit child indices.  A step whose children exceed that (2^32
// children, or the device memory) is split by hash into K ranges (a mix of
// the hash independent of the table's home slot): equal hashes fall in the
// same range, so every collision group lies in one range.  Pass k computes
// every child (the symbolic iteration), keeps those of range k in child
// order, and runs the collision table, zero elimination and a
// top-max_num_object selection on them; the selected groups (candidates)
// are appended in child order.  Every group of the global top
// max_num_object is in its range's top max_num_object, so the candidates
// hold the result: they are merged back into child order (their child
// indices are distinct) and the usual selection, layout, normalisation and
// populate follow.
//
// The result is the one-pass result bit for bit: the group sums use the
// fixed-point scale of the whole step (largest component over every child,
// the step's child count), a group's representative is its lowest child
// index, the truncation keys and their ties (lower child index first) are
// the same, and the survivors come out in child order.
//
// The reference's counterpart is its MPI engine, which gives each node the
// children of one hash range (src/quids_mpi.hpp:624-865, owner by the hash's
// top bits :665-669) and merges collisions on the owner; here one GPU runs
// the ranges one after another and recomputes the children for each.
#pragma once
#include "engine.cuh"

namespace qd::ranges {

using namespace qd::engine;

// the range of a child hash among k (a mixer unrelated to table_home, so
// one range's children spread over its table)
__device__ __forceinline__ uint32_t range_of(uint64_t h, uint32_t k) {
    uint64_t r = h ^ (h >> 31);
    r *= 0x7FB5D329728EA185ull;
    r ^= r >> 27;
    return (uint32_t)__umul64hi(r, (uint64_t)k);
}

// ------------------------------------------------------------------ kernels
// the kept parent holding child c of a tile whose parents' child offsets are
// staged in s_cb (count + 1 of them), else found in global memory
__device__ __forceinline__ uint64_t tile_parent(const uint64_t *s_cb, int count, uint64_t plo,
                                                const parents_view &pv, uint64_t c) {
    if (count <= 0) return parent_of(pv.cbeg, pv.nparents(), c);
    int lo = 0, hi = count;  // s_cb[lo] <= c < s_cb[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (s_cb[mid] <= c) lo = mid; else hi = mid;
    }
    return plo + (uint64_t)lo;
}

// The first pass of the symbolic iteration over the children of the kept
// parents (rules without grouped children): every child is computed
// (hash_child; blocked items in child order, a look-back chain over tiles of
// kTileChildren children), its range stored in rid[c], and the children of
// range 0 kept: written at their rank among them (records past `cap` are
// not written; *d_count gets the range's full count).  It also takes the
// largest |component| over every child of the step into *d_maxabs.
template <class RS>
__global__ void __launch_bounds__(prim::kThreads)
    k_symbolic_first(RS rs, parents_view pv, const uint64_t *tile_first, uint64_t nc, uint32_t K, uint8_t *rid,
                     uint64_t cap, uint64_t *rhash, double2 *rmag, uint32_t *rsize, uint32_t *rpar, uint32_t *rcid,
                     uint64_t *d_count, prim::lookback lb, unsigned long long *d_maxabs) {
    static_assert(kSymItems == 4, "one 32-bit word of range ids per thread");
    __shared__ uint64_t s_cb[kStagedParents + 1];
    __shared__ uint64_t sm[prim::kThreads / 32 + 1];
    __shared__ uint64_t bcast;
    __shared__ uint32_t sm_tile;
    const uint64_t ntiles = (nc + kTileChildren - 1) / kTileChildren;
    unsigned long long mx = 0;
    while (true) {
        const uint32_t tile = prim::next_tile(lb, &sm_tile);
        if (tile >= ntiles) break;
        const uint64_t c0 = (uint64_t)tile * kTileChildren;
        const uint64_t cb = c0 + (uint64_t)threadIdx.x * kSymItems;  // the thread's first child
        const uint64_t plo = tile_first[tile], phi = tile_first[tile + 1];
        const int count = phi - plo + 1 <= (uint64_t)kStagedParents ? (int)(phi - plo + 1) : -1;
        for (int q = threadIdx.x; q <= count; q += blockDim.x) s_cb[q] = pv.cbeg[plo + q];
        __syncthreads();
        uint64_t hh[kSymItems];
        double2 mm[kSymItems];
        uint32_t ss[kSymItems], pp[kSymItems], cc[kSymItems];
        uint32_t sel = 0, ids = 0;
        uint64_t nsel = 0;
#pragma unroll
        for (int u = 0; u < kSymItems; ++u) {
            const uint64_t c = cb + u;
            if (c >= nc) break;
            const uint64_t p = tile_parent(s_cb, count, plo, pv, c);
            const uint64_t oid = pv.pidx ? pv.pidx[p] : p;
            const uint32_t cid = (uint32_t)(c - pv.cbeg[p]);
            const char *pb = pv.objects + pv.begin[oid];
            const char *pe = pb + pv.size[oid];
            const double2 pm = pv.mag[oid];
            mag_t m{pm.x, pm.y};
            uint32_t sz = 0;
            const uint64_t h = rs.tag(rs.get(oid).hash_child(pb, pe, cid, sz, m), oid);
            const unsigned long long a = (unsigned long long)__double_as_longlong(m.re) & 0x7fffffffffffffffull;
            const unsigned long long b = (unsigned long long)__double_as_longlong(m.im) & 0x7fffffffffffffffull;
            mx = mx > a ? mx : a;
            mx = mx > b ? mx : b;
            const uint32_t r = range_of(h, K);
            ids |= r << (8 * u);
            hh[u] = h;
            mm[u] = make_double2(m.re, m.im);
            ss[u] = sz;
            pp[u] = (uint32_t)p;
            cc[u] = cid;
            if (r == 0) {
                sel |= 1u << u;
                ++nsel;
            }
        }
        if (cb + kSymItems <= nc) {
            *(uint32_t *)(rid + cb) = ids;  // cb is a multiple of 4
        } else {
            for (int u = 0; u < kSymItems && cb + u < nc; ++u) rid[cb + u] = (uint8_t)(ids >> (8 * u));
        }
        uint64_t agg;
        const uint64_t excl = prim::block_excl_scan(nsel, sm, agg);  // also orders the reuse of s_cb
        const uint64_t pre = prim::tile_prefix(lb, tile, agg, &bcast);
        uint64_t j = pre + excl;
#pragma unroll
        for (int u = 0; u < kSymItems; ++u) {
            if (!(sel & (1u << u))) continue;
            if (j < cap) {
                rhash[j] = hh[u];
                rmag[j] = mm[u];
                rsize[j] = ss[u];
                rpar[j] = pp[u];
                rcid[j] = cc[u];
            }
            ++j;
        }
        if (tile == ntiles - 1 && threadIdx.x == prim::kThreads - 1) *d_count = pre + agg;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = mx > y ? mx : y;
    }
    if ((threadIdx.x & 31) == 0 && mx) atomicMax(d_maxabs, mx);
}

// the grouped pass's output when it only sorts children into ranges
struct range_ids {
    uint8_t *rid;
    uint32_t K;
    __device__ __forceinline__ void operator()(uint64_t c, uint64_t h, const mag_t &, uint32_t, uint64_t) const {
        rid[c] = (uint8_t)range_of(h, K);
    }
};

// Pass k over children whose range ids are known: a block takes
// kListTiles symbolic tiles at a time, lists their children of range k in
// shared memory (in child order) and computes only those (hash_child),
// spread over its threads, writing each at its rank among them (a
// look-back chain over the block tiles).  Records past `cap` are not
// written; *d_count gets the range's full count.
constexpr int kListTiles = 8;
constexpr int kListChildren = kListTiles * kTileChildren;         // 8192 (u16 offsets)
constexpr int kListPerThread = kListChildren / prim::kThreads;    // 32 range ids per thread
constexpr int kListStaged = 1024;                                 // parents whose offsets are staged
template <class RS>
__global__ void __launch_bounds__(prim::kThreads)
    k_symbolic_list(RS rs, parents_view pv, const uint64_t *tile_first, uint64_t sym_tiles, uint64_t nc, uint32_t k,
                    const uint8_t *rid, uint64_t cap, uint64_t *rhash, double2 *rmag, uint32_t *rsize, uint32_t *rpar,
                    uint32_t *rcid, uint64_t *d_count, prim::lookback lb) {
    static_assert(kListPerThread == 32, "one 32-bit selection mask per thread");
    __shared__ uint64_t s_cb[kListStaged + 1];
    __shared__ uint16_t s_list[kListChildren];
    __shared__ uint64_t sm[prim::kThreads / 32 + 1];
    __shared__ uint64_t bcast;
    __shared__ uint32_t sm_tile;
    const uint64_t nblk = (nc + kListChildren - 1) / kListChildren;
    const uint32_t kk = k * 0x01010101u;
    while (true) {
        const uint32_t t = prim::next_tile(lb, &sm_tile);
        if (t >= nblk) break;
        const uint64_t c0 = (uint64_t)t * kListChildren;
        const uint64_t t0 = (uint64_t)t * kListTiles;
        const uint64_t t1 = t0 + kListTiles < sym_tiles ? t0 + kListTiles : sym_tiles;
        const uint64_t plo = tile_first[t0], phi = tile_first[t1];
        const int count = phi - plo + 1 <= (uint64_t)kListStaged ? (int)(phi - plo + 1) : -1;
        for (int q = threadIdx.x; q <= count; q += blockDim.x) s_cb[q] = pv.cbeg[plo + q];
        const uint64_t cb = c0 + (uint64_t)threadIdx.x * kListPerThread;
        uint32_t mine = 0;
        if (cb + kListPerThread <= nc) {
            const uint4 *w = (const uint4 *)(rid + cb);  // 32-byte aligned
#pragma unroll
            for (int v = 0; v < 2; ++v) {
                const uint4 q = w[v];
                const uint32_t ws[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int x = 0; x < 4; ++x) {
                    const uint32_t eq = __vcmpeq4(ws[x], kk);  // 0xff in each byte equal to k
#pragma unroll
                    for (int b = 0; b < 4; ++b) mine |= ((eq >> (8 * b)) & 1u) << (16 * v + 4 * x + b);
                }
            }
        } else {
            for (int u = 0; u < kListPerThread && cb + u < nc; ++u) mine |= (rid[cb + u] == k ? 1u : 0u) << u;
        }
        uint64_t agg;
        uint64_t e = prim::block_excl_scan((uint64_t)__popc(mine), sm, agg);
        for (uint32_t m = mine; m; m &= m - 1) s_list[e++] = (uint16_t)(threadIdx.x * kListPerThread + __ffs(m) - 1);
        const uint64_t pre = prim::tile_prefix(lb, t, agg, &bcast);  // its barriers publish s_list and s_cb
        for (uint32_t q = threadIdx.x; q < (uint32_t)agg; q += blockDim.x) {
            const uint64_t c = c0 + s_list[q];
            const uint64_t p = tile_parent(s_cb, count, plo, pv, c);
            const uint64_t oid = pv.pidx ? pv.pidx[p] : p;
            const uint32_t cid = (uint32_t)(c - pv.cbeg[p]);
            const char *pb = pv.objects + pv.begin[oid];
            const char *pe = pb + pv.size[oid];
            const double2 pm = pv.mag[oid];
            mag_t m{pm.x, pm.y};
            uint32_t sz = 0;
            const uint64_t h = rs.tag(rs.get(oid).hash_child(pb, pe, cid, sz, m), oid);
            const uint64_t j = pre + q;
            if (j < cap) {
                rhash[j] = h;
                rmag[j] = make_double2(m.re, m.im);
                rsize[j] = sz;
                rpar[j] = (uint32_t)p;
                rcid[j] = cid;
            }
        }
        if (t == nblk - 1 && threadIdx.x == 0) *d_count = pre + agg;
    }
}

// the groups of a range above tolerance, with their global child index
struct range_collect {
    group_view g;
    const uint32_t *rpar, *rcid, *rsize;
    const uint64_t *cbeg;
    uint64_t *uglob;
    double2 *umag;
    uint64_t *unorm;
    uint32_t *usize, *upar, *ucid;
    using item = mag_t;
    __device__ bool load(uint64_t c, item &m) const { return g.kept(c, m); }
    __device__ void emit(uint64_t c, uint64_t j, const item &m) const {
        const uint32_t p = rpar[c], cid = rcid[c];
        uglob[j] = cbeg[p] + cid;
        umag[j] = make_double2(m.re, m.im);
        unorm[j] = (uint64_t)__double_as_longlong(cnorm(m));
        usize[j] = rsize[c];
        upar[j] = p;
        ucid[j] = cid;
    }
};

// candidate records (one run per range, each in child order)
struct candidates {
    uint64_t *glob;  // global child index of the group's representative
    double2 *mag;
    uint64_t *norm;  // IEEE bits
    uint32_t *size, *par, *cid;
};

// a range's top groups (ties at the cutoff by lower child index), appended
// to the candidates at `base`
struct range_keep {
    key_unorm kf;  // {unorm, global child index, truncation key}
    const prim::select_state *st;
    const double2 *umag;
    const uint32_t *usize, *upar, *ucid;
    candidates out;
    uint64_t base;
    __device__ uint64_t key(uint64_t i) const { return kf.key(i); }
    __device__ bool tie(uint64_t i) const { return st->active && key(i) == st->prefix; }
    __device__ bool select(uint64_t i, uint64_t tie_rank) const {
        if (!st->active) return true;
        const uint64_t k = key(i);
        if (k > st->prefix) return true;
        if (k < st->prefix) return false;
        return tie_rank < st->k_rem;
    }
    __device__ void emit(uint64_t i, uint64_t j) const {
        const uint64_t o = base + j;
        out.glob[o] = kf.uchild[i];
        out.mag[o] = umag[i];
        out.norm[o] = kf.unorm[i];
        out.size[o] = usize[i];
        out.par[o] = upar[i];
        out.cid[o] = ucid[i];
    }
};

static __global__ void k_iota_keys(const uint64_t *glob, uint64_t n, uint64_t *key, uint32_t *perm) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        key[e] = glob[e];
        perm[e] = (uint32_t)e;
    }
}

// One merge round over sorted runs [off[r], off[r+1]): runs 2q and 2q+1
// (adjacent) become one sorted run.  Keys are distinct, so an element's
// place in the merged run is its index in its own run plus the number of
// smaller keys in the other run (a binary search).  perm follows its key.
static __global__ void __launch_bounds__(prim::kThreads)
    k_merge_round(const uint64_t *key, const uint32_t *perm, uint64_t *key_out, uint32_t *perm_out,
                  const uint64_t *off, uint32_t nruns, uint64_t n) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t r = 0;  // the run holding e (runs are few; empty runs are skipped)
        while (r + 1 < nruns && off[r + 1] <= e) ++r;
        const uint32_t mate = r ^ 1u;
        const uint64_t v = key[e];
        uint64_t dst = e;  // an unpaired last run stays in place
        if (mate < nruns) {
            const uint64_t lo = off[mate], hi = off[mate + 1];
            uint64_t a = lo, b = hi;  // mate keys below v: [lo, a)
            while (a < b) {
                const uint64_t mid = (a + b) >> 1;
                if (key[mid] < v) a = mid + 1; else b = mid;
            }
            dst = off[r & ~1u] + (e - off[r]) + (a - lo);
        }
        key_out[dst] = v;
        perm_out[dst] = perm[e];
    }
}

// the truncation key of the merged candidates
struct key_merged {
    candidates c;
    const uint32_t *perm;  // merged position -> candidate
    trunc_key tk;
    __device__ uint64_t key(uint64_t i) const {
        const uint32_t q = perm[i];
        return tk.probabilistic ? tk(__longlong_as_double((long long)c.norm[q]), c.glob[q]) : c.norm[q];
    }
};

// the final selection over the merged candidates into the output layout
struct merged_layout {
    key_merged kf;
    const prim::select_state *st;
    uint32_t align;
    double2 *omag;
    uint32_t *osize;
    uint64_t *obegin;
    uint32_t *spar, *scid;
    __device__ bool tie(uint64_t i) const { return st->active && kf.key(i) == st->prefix; }
    __device__ bool rank_needed() const { return st->active && st->n_equal > st->k_rem; }
    struct item {
        uint32_t q;
        uint32_t size;
    };
    __device__ bool load(uint64_t i, uint64_t tie_rank, item &it) const {
        bool keep = true;
        if (st->active) {
            const uint64_t k = kf.key(i);
            keep = k > st->prefix || (k == st->prefix && tie_rank < st->k_rem);
        }
        if (keep) {
            it.q = kf.perm[i];
            it.size = kf.c.size[it.q];
        }
        return keep;
    }
    __device__ uint64_t bytes(const item &it) const { return padded_size(it.size, align); }
    __device__ double emit(uint64_t, uint64_t j, uint64_t off, const item &it) const {
        const uint32_t q = it.q;
        omag[j] = kf.c.mag[q];
        osize[j] = it.size;
        obegin[j] = off;
        spar[j] = kf.c.par[q];
        scid[j] = kf.c.cid[q];
        return __longlong_as_double((long long)kf.c.norm[q]);
    }
};

// ------------------------------------------------------------------- the step
// buffers of the range passes that the context does not keep
struct range_buffers {
    qd_dbuf rid, ltile, rcid, usize, upar, ucid, cand[6], key[2], perm[2], off, spar, scid;
    ~range_buffers() {
        for (qd_dbuf *b : {&rid, &ltile, &rcid, &usize, &upar, &ucid, &key[0], &key[1], &perm[0], &perm[1], &off, &spar, &scid})
            release(*b);
        for (auto &b : cand) release(b);
    }
};

// device bytes per child of a range (records, group marks, table at load
// 1/2, kept groups) and per candidate (records and the merge's keys)
constexpr double kRangeChildBytes = 36.0 + 6.0 + 96.0 + 44.0;
constexpr double kCandidateBytes = 44.0 + 24.0;

// per-stage device time summed over the passes (QUIDS_FLAG_STAGE_TIMING):
// events bracket a stage and are read after the host wait that follows
struct stage_clock {
    quids_gpu_ctx *ctx;
    bool on;
    float *acc;  // [8]
    bool used[8] = {};
    void begin(int k) {
        if (!on) return;
        cudaEventRecord(ctx->ev_stage[2 * k], ctx->stream);
        used[k] = true;
    }
    void end(int k) {
        if (on) cudaEventRecord(ctx->ev_stage[2 * k + 1], ctx->stream);
    }
    void harvest() {
        for (int k = 0; on && k < 8; ++k)
            if (used[k]) {
                float ms = 0;
                cudaEventElapsedTime(&ms, ctx->ev_stage[2 * k], ctx->ev_stage[2 * k + 1]);
                acc[k] += ms;
                used[k] = false;
            }
    }
};

// zeroed look-back chain of `words` words at word `at` of the chain buffer
inline int chain_at(quids_gpu_ctx *ctx, uint64_t at, uint64_t words, prim::lookback &lb) {
    uint64_t *ws = bufp<uint64_t>(ctx, B_LOOKBACK) + at;
    QD_CUDA(cudaMemsetAsync(ws, 0, words * sizeof(uint64_t), ctx->stream));
    lb.status = ws + 1;
    lb.counter = (uint32_t *)ws;
    lb.err = (int *)(ctx->d_words + W_STATUS);
    return QUIDS_OK;
}

template <class Rule, class Post = no_post>
int simulate_ranges(quids_gpu_ctx *ctx, quids_gpu_state *in, const Rule &rule_, quids_gpu_state *out,
                    const quids_gpu_params &prm, quids_gpu_step_stats *stats, const Post &post = Post{}) {
    if (!ctx || !in || !out || in == out || in->ctx != ctx || out->ctx != ctx) return QUIDS_ERR_BAD_ARG;
    // the memory-driven truncation cuts parents until one pass fits instead
    if (prm.max_num_object == 0) return QUIDS_ERR_UNSUPPORTED;
    const single_rule<Rule> rs{rule_};
    QD_CUDA(cudaSetDevice(ctx->device));
    const bool timing = (prm.flags & QUIDS_FLAG_STAGE_TIMING) != 0;
    if (timing) QD_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    const uint64_t launches0 = ctx->launches;
    const trunc_key tk{prm.simple_truncation == 0, prm.seed};
    const double load = prm.table_load_factor > 0 && prm.table_load_factor < 0.95 ? prm.table_load_factor : 0.5;
    const uint64_t N = in->n;
    const uint64_t maxn = prm.max_num_object;
    quids_gpu_step_stats s{};
    s.num_parents = N;
    s.total_proba = std::numeric_limits<double>::quiet_NaN();
    stage_clock clk{ctx, timing, s.stage_ms};
    // the context's scratch is sized afresh, without headroom (all but the
    // sticky modifier status)
    for (int b = 0; b < B_COUNT; ++b)
        if (b != B_MODSTATUS) release(ctx->buf[b]);

    // ---- num_child, parent pre-truncation, child offsets (as in one pass)
    QD_TRY(ensure(ctx->buf[B_NCHILD], (N ? N : 1) * sizeof(uint32_t)));
    clk.begin(0);
    QD_TRY(ensure(ctx->buf[B_LOOKBACK], lookback_words(N) * sizeof(uint64_t)));
    const uint64_t nzero0 = N ? lookback_words(N) : 0;
    k_step_begin<<<(unsigned)std::min<uint64_t>((nzero0 + 255) / 256 + 1, (uint64_t)ctx->num_sms * 4), 256, 0,
                   ctx->stream>>>(ctx->d_words, N, maxn < N ? 0 : N, bufp<int>(ctx, B_MODSTATUS),
                                  bufp<uint64_t>(ctx, B_LOOKBACK), nzero0);
    QD_TRY(launched(ctx));
    if (N == 0) return QUIDS_ERR_BAD_ARG;  // an empty state never needs ranges
    int *err = (int *)(ctx->d_words + W_STATUS);
    k_num_child<<<grid_for(ctx, N), prim::kThreads, 0, ctx->stream>>>(
        rs, (const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p, N,
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
    {
        prim::lookback lb;
        lookback_view(ctx, N, 1, lb);
        scan_nchild f{bufp<uint32_t>(ctx, B_NCHILD), pidx};
        prim::k_scan_excl<<<lookback_grid(ctx, NP), prim::kThreads, 0, ctx->stream>>>(
            f, ctx->d_words + W_NP, bufp<uint64_t>(ctx, B_CBEGIN), ctx->d_words + W_NC, lb);
        QD_TRY(launched(ctx));
    }
    clk.end(0);
    int st = read_words(ctx);
    if (st) return st;
    clk.harvest();
    const uint64_t NC = ctx->h_words[W_NC], maxsize = ctx->h_words[W_MAXSIZE];
    s.num_object = NC;
    s.max_child_size = maxsize;
    if (NC == 0) return QUIDS_ERR_BAD_ARG;
    if (maxsize > 4096) return QUIDS_ERR_SIZE_BOUND;
    parents_view pv{(const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p,
                    (const double2 *)in->mag.p, bufp<uint64_t>(ctx, B_CBEGIN), pidx, NP};

    // ---- how many ranges: a range's records and table within the memory
    // left after the candidates and the output
    size_t free_b = 0, total_b = 0;
    QD_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const double out_est = (double)std::min(NC, maxn) * (28.0 + (double)((maxsize + 7) / 8 * 8));
    auto cand_count = [&](uint64_t k) { return maxn >= NC ? NC : std::min<uint64_t>(NC, maxn * k); };
    const double avail = 0.8 * (double)free_b - out_est - (double)NC;  // NC: the children's range ids
    uint32_t K = prm.hash_ranges >= 2 ? prm.hash_ranges : 2;
    while (K < (1u << 16) && ((double)NC / K * 1.07 * kRangeChildBytes + (double)cand_count(K) * kCandidateBytes >
                                  avail ||
                              (double)NC / K * 1.07 / load + 4096 >= (double)0x7ff00000ull))
        ++K;
    if (K > 255) return QUIDS_ERR_OOM;  // range ids are bytes; such a step's ids alone exceed the device
    const uint64_t cand_cap = cand_count(K);
    if (cand_cap >= 0xffffffffull) return QUIDS_ERR_OOM;  // candidate indices are u32
    uint64_t cap = NC / K + NC / K / 16 + 4096;             // a range's share with slack (grown on demand)

    // ---- buffers
    range_buffers rb;
    const uint64_t sym_tiles = (NC + kTileChildren - 1) / kTileChildren;
    auto grow_ranges = [&](uint64_t c) -> int {
        QD_TRY(ensure(ctx->buf[B_HASH], c * 8, false));
        QD_TRY(ensure(ctx->buf[B_CMAG], c * 16, false));
        QD_TRY(ensure(ctx->buf[B_CSIZE], c * 4, false));
        QD_TRY(ensure(ctx->buf[B_CPAR], c * 4, false));
        QD_TRY(ensure(rb.rcid, c * 4, false));
        QD_TRY(ensure(ctx->buf[B_SLOT], c * 4, false));
        QD_TRY(ensure(ctx->buf[B_NOTREP], c, false));
        QD_TRY(ensure(ctx->buf[B_HASJOIN], c, false));
        QD_TRY(ensure(ctx->buf[B_UCHILD], c * 8, false));
        QD_TRY(ensure(ctx->buf[B_UMAG], c * 16, false));
        QD_TRY(ensure(ctx->buf[B_UNORM], c * 8, false));
        QD_TRY(ensure(rb.usize, c * 4, false));
        QD_TRY(ensure(rb.upar, c * 4, false));
        QD_TRY(ensure(rb.ucid, c * 4, false));
        const uint64_t Mc = std::max<uint64_t>((uint64_t)((double)c / load) + 1, 1024);
        if (Mc >= 0x7ffffff0ull) return QUIDS_ERR_OOM;  // slot indices are 31-bit
        QD_TRY(ensure(ctx->buf[B_KEYS], (Mc + 1) * sizeof(prim::table_slot), false));
        QD_TRY(ensure(ctx->buf[B_ACC], 4 * (Mc + 1) * sizeof(uint64_t), false));
        const uint64_t chains =
            std::max<uint64_t>(sym_tiles + 2, 3 * ((std::max(c, cand_cap) + prim::kTile - 1) / prim::kTile + 2));
        QD_TRY(ensure(ctx->buf[B_LOOKBACK], chains * sizeof(uint64_t), false));
        return QUIDS_OK;
    };
    QD_TRY(ensure(ctx->buf[B_TILEPAR], (sym_tiles + 1) * sizeof(uint64_t), false));
    QD_TRY(ensure(rb.rid, (NC + 31) / 32 * 32, false));
    QD_TRY(grow_ranges(cap));
    const size_t cw[6] = {8, 16, 8, 4, 4, 4};
    for (int q = 0; q < 6; ++q) QD_TRY(ensure(rb.cand[q], (cand_cap ? cand_cap : 1) * cw[q], false));
    const candidates cand{(uint64_t *)rb.cand[0].p, (double2 *)rb.cand[1].p, (uint64_t *)rb.cand[2].p,
                          (uint32_t *)rb.cand[3].p, (uint32_t *)rb.cand[4].p, (uint32_t *)rb.cand[5].p};
    k_tile_parents<<<grid_for(ctx, NP), prim::kThreads, 0, ctx->stream>>>(bufp<uint64_t>(ctx, B_CBEGIN), NP, sym_tiles,
                                                                         bufp<uint64_t>(ctx, B_TILEPAR));
    QD_TRY(launched(ctx));
    // the step's child count, for the fixed-point scale of the group sums
    QD_TRY(set_word(ctx, W_TMP, NC));

    // ---- the children's ranges: for rules with grouped children, a grouped
    // pass over every child (leader offsets and their tile map from one
    // scan, the leader count in W_NU); otherwise the first range pass
    bool ids_known = false;
    if constexpr (has_grouped<Rule>::value) {
        const uint64_t ltiles_cap = NC / kLeaderTile + 2;  // leaders <= children
        QD_TRY(ensure(ctx->buf[B_LBEG], (NP + 1) * sizeof(uint64_t), false));
        QD_TRY(ensure(rb.ltile, ltiles_cap * sizeof(uint64_t), false));
        clk.begin(1);
        prim::lookback lb;
        QD_TRY(chain_at(ctx, 0, (NP + prim::kTile - 1) / prim::kTile + 2, lb));
        scan_leaders f{bufp<uint32_t>(ctx, B_NCHILD), pidx};
        prim::k_scan_excl<<<lookback_grid(ctx, NP), prim::kThreads, 0, ctx->stream>>>(
            f, ctx->d_words + W_NP, bufp<uint64_t>(ctx, B_LBEG), ctx->d_words + W_NU, lb,
            leader_tile_epilogue{(uint64_t *)rb.ltile.p, ltiles_cap});
        const uint64_t est_tiles = (NC >> kGroupBits) / kLeaderTile + 1;
        const unsigned g = (unsigned)std::min<uint64_t>(est_tiles, (uint64_t)ctx->num_sms * 8);
        k_symbolic_grouped<single_rule<Rule>, range_ids><<<g, prim::kThreads, 0, ctx->stream>>>(
            rs, pv, bufp<uint64_t>(ctx, B_LBEG), (const uint64_t *)rb.ltile.p, ctx->d_words + W_NU,
            range_ids{(uint8_t *)rb.rid.p, K}, (unsigned long long *)(ctx->d_words + W_MAXABS),
            (int *)(ctx->d_words + W_STATUS));
        QD_TRY(launched(ctx, 2));
        clk.end(1);
        ids_known = true;
    }

    // ---- the range passes
    std::vector<uint64_t> run_off(1, 0);
    uint64_t NU = 0, Mmax = 0;
    const unsigned long long *d_maxabs = (const unsigned long long *)(ctx->d_words + W_MAXABS);
    for (uint32_t k = 0; k < K; ++k) {
        uint64_t nk = 0;
        while (true) {
            prim::lookback lb;
            clk.begin(1);
            if (k == 0 && !ids_known) {
                QD_TRY(chain_at(ctx, 0, sym_tiles + 2, lb));
                const unsigned g = (unsigned)std::min<uint64_t>(sym_tiles, (uint64_t)ctx->num_sms * 4);
                k_symbolic_first<single_rule<Rule>><<<g, prim::kThreads, 0, ctx->stream>>>(
                    rs, pv, bufp<uint64_t>(ctx, B_TILEPAR), NC, K, (uint8_t *)rb.rid.p, cap,
                    bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG), bufp<uint32_t>(ctx, B_CSIZE),
                    bufp<uint32_t>(ctx, B_CPAR), (uint32_t *)rb.rcid.p, ctx->d_words + W_NC, lb,
                    (unsigned long long *)(ctx->d_words + W_MAXABS));
            } else {
                const uint64_t nblk = (NC + kListChildren - 1) / kListChildren;
                QD_TRY(chain_at(ctx, 0, nblk + 2, lb));
                const unsigned g = (unsigned)std::min<uint64_t>(nblk, (uint64_t)ctx->num_sms * 8);
                k_symbolic_list<single_rule<Rule>><<<g, prim::kThreads, 0, ctx->stream>>>(
                    rs, pv, bufp<uint64_t>(ctx, B_TILEPAR), sym_tiles, NC, k, (const uint8_t *)rb.rid.p, cap,
                    bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG), bufp<uint32_t>(ctx, B_CSIZE),
                    bufp<uint32_t>(ctx, B_CPAR), (uint32_t *)rb.rcid.p, ctx->d_words + W_NC, lb);
            }
            QD_TRY(launched(ctx));
            clk.end(1);
            st = read_words(ctx);
            if (st) return st;
            clk.harvest();
            nk = ctx->h_words[W_NC];
            if (nk <= cap) break;
            // a range above its share (large collision groups): its records
            // are recomputed into larger buffers
            cap = nk + nk / 16;
            QD_TRY(grow_ranges(cap));
        }
        if (nk == 0) {
            run_off.push_back(run_off.back());
            continue;
        }
        const uint64_t Mk = std::max<uint64_t>((uint64_t)((double)nk / load) + 1, 1024);
        Mmax = std::max(Mmax, Mk);
        const prim::table tb{bufp<prim::table_slot>(ctx, B_KEYS), bufp<unsigned long long>(ctx, B_ACC), Mk, probe_limit(prm)};
        const uint64_t words = (nk + prim::kTile - 1) / prim::kTile + 2;
        clk.begin(2);
        {
            fill_set f{};
            f.p[0] = (unsigned char *)tb.slots, f.n[0] = (Mk + 1) * sizeof(prim::table_slot), f.v[0] = 0xff;
            f.p[1] = (unsigned char *)(tb.acc + 4 * Mk), f.n[1] = 4 * sizeof(uint64_t), f.v[1] = 0;
            f.p[2] = bufp<unsigned char>(ctx, B_NOTREP), f.n[2] = nk, f.v[2] = 0;
            f.p[3] = bufp<unsigned char>(ctx, B_HASJOIN), f.n[3] = nk, f.v[3] = 0;
            f.p[4] = bufp<unsigned char>(ctx, B_LOOKBACK), f.n[4] = 3 * words * sizeof(uint64_t), f.v[4] = 0;
            f.count = 5;
            QD_TRY(fill(ctx, f));
        }
        const direct_src src{bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG)};
        uint8_t *not_rep = bufp<uint8_t>(ctx, B_NOTREP), *has_join = bufp<uint8_t>(ctx, B_HASJOIN);
        prim::k_table_claim<<<grid_for(ctx, nk), prim::kThreads, 0, ctx->stream>>>(
            tb, src, ctx->d_words + W_NC, bufp<uint32_t>(ctx, B_SLOT), err);
        prim::k_table_accumulate<<<grid_for(ctx, nk), prim::kThreads, 0, ctx->stream>>>(
            tb, src, bufp<uint32_t>(ctx, B_SLOT), ctx->d_words + W_NC, d_maxabs, not_rep, has_join,
            ctx->d_words + W_TMP);
        QD_TRY(launched(ctx, 2));
        clk.end(2);
        clk.begin(3);
        const group_view gv{bufp<uint32_t>(ctx, B_SLOT), not_rep, has_join, bufp<double2>(ctx, B_CMAG),
                            bufp<unsigned long long>(ctx, B_ACC), ctx->d_words + W_TMP, d_maxabs, prm.tolerance};
        prim::lookback lb0, lb1, lb2;
        lookback_view(ctx, nk, 0, lb0);
        lookback_view(ctx, nk, 1, lb1);
        lookback_view(ctx, nk, 2, lb2);
        const range_collect fc{gv,
                               bufp<uint32_t>(ctx, B_CPAR),
                               (const uint32_t *)rb.rcid.p,
                               bufp<uint32_t>(ctx, B_CSIZE),
                               bufp<uint64_t>(ctx, B_CBEGIN),
                               bufp<uint64_t>(ctx, B_UCHILD),
                               bufp<double2>(ctx, B_UMAG),
                               bufp<uint64_t>(ctx, B_UNORM),
                               (uint32_t *)rb.usize.p,
                               (uint32_t *)rb.upar.p,
                               (uint32_t *)rb.ucid.p};
        prim::k_compact<<<lookback_grid(ctx, nk), prim::kThreads, 0, ctx->stream>>>(fc, ctx->d_words + W_NC,
                                                                                   ctx->d_words + W_NU, lb0);
        QD_TRY(launched(ctx));
        clk.end(3);
        clk.begin(4);
        // the range's top max_num_object groups, appended to the candidates
        const key_unorm ku{bufp<uint64_t>(ctx, B_UNORM), bufp<uint64_t>(ctx, B_UCHILD), tk};
        QD_TRY(radix_select(ctx, ctx->d_words + W_NU, nk, maxn, ku));
        const range_keep fk{ku,   ctx->d_sel, bufp<double2>(ctx, B_UMAG), (const uint32_t *)rb.usize.p,
                            (const uint32_t *)rb.upar.p, (const uint32_t *)rb.ucid.p, cand, run_off.back()};
        prim::k_compact_ranked<<<lookback_grid(ctx, nk), prim::kThreads, 0, ctx->stream>>>(
            fk, ctx->d_words + W_NU, ctx->d_words + W_NS, lb1, lb2);
        QD_TRY(launched(ctx));
        clk.end(4);
        st = read_words(ctx);
        if (st) return st;
        clk.harvest();
        NU += ctx->h_words[W_NU];
        const uint64_t kept = ctx->h_words[W_NS];
        if (run_off.back() + kept > cand_cap) return QUIDS_ERR_CUDA;  // at most max_num_object per range
        run_off.push_back(run_off.back() + kept);
    }
    s.num_object_after_interferences = NU;
    s.table_capacity = Mmax;
    s.hash_ranges = K;
    const uint64_t NCAND = run_off.back();

    // ---- the candidates back in child order
    for (int q = 0; q < 2; ++q) {
        QD_TRY(ensure(rb.key[q], (NCAND ? NCAND : 1) * 8, false));
        QD_TRY(ensure(rb.perm[q], (NCAND ? NCAND : 1) * 4, false));
    }
    int cur = 0;
    clk.begin(4);
    if (NCAND) {
        k_iota_keys<<<grid_for(ctx, NCAND), prim::kThreads, 0, ctx->stream>>>(cand.glob, NCAND, (uint64_t *)rb.key[0].p,
                                                                              (uint32_t *)rb.perm[0].p);
        QD_TRY(launched(ctx));
        std::vector<uint64_t> offs = run_off;
        QD_TRY(ensure(rb.off, offs.size() * 8));
        while (offs.size() > 2) {
            const uint32_t nruns = (uint32_t)(offs.size() - 1);
            QD_CUDA(cudaMemcpyAsync(rb.off.p, offs.data(), offs.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
            k_merge_round<<<grid_for(ctx, NCAND), prim::kThreads, 0, ctx->stream>>>(
                (const uint64_t *)rb.key[cur].p, (const uint32_t *)rb.perm[cur].p, (uint64_t *)rb.key[cur ^ 1].p,
                (uint32_t *)rb.perm[cur ^ 1].p, (const uint64_t *)rb.off.p, nruns, NCAND);
            QD_TRY(launched(ctx));
            QD_CUDA(cudaStreamSynchronize(ctx->stream));  // the host offsets are rewritten next
            cur ^= 1;
            std::vector<uint64_t> next(1, 0);
            for (uint32_t r = 0; r < nruns; r += 2) next.push_back(offs[std::min<uint32_t>(r + 2, nruns)]);
            offs.swap(next);
        }
    }

    // ---- the final selection, layout, normalisation and populate
    QD_TRY(set_word(ctx, W_NU, NCAND));
    const uint64_t NSB = std::min<uint64_t>(NCAND, maxn);
    QD_TRY(ensure(out->begin, (NSB + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(out->size, (NSB ? NSB : 1) * sizeof(uint32_t)));
    QD_TRY(ensure(out->mag, (NSB ? NSB : 1) * sizeof(double2)));
    QD_TRY(ensure(out->d_total, sizeof(double)));
    QD_TRY(ensure(rb.spar, (NSB ? NSB : 1) * 4));
    QD_TRY(ensure(rb.scid, (NSB ? NSB : 1) * 4));
    const key_merged km{cand, (const uint32_t *)rb.perm[cur].p, tk};
    QD_TRY(radix_select(ctx, ctx->d_words + W_NU, NCAND, maxn, km));
    {
        prim::lookback lbt, lbc, lbb;
        QD_TRY(lookback_chain(ctx, NCAND, 0, lbt));
        QD_TRY(lookback_chain(ctx, NCAND, 1, lbc));
        QD_TRY(lookback_chain(ctx, NCAND, 2, lbb));
        QD_TRY(set_word(ctx, W_MAXNORM, 0));
        const merged_layout f{km, ctx->d_sel, prm.align_byte_length, (double2 *)out->mag.p, (uint32_t *)out->size.p,
                              (uint64_t *)out->begin.p, (uint32_t *)rb.spar.p, (uint32_t *)rb.scid.p};
        prim::k_compact_layout<merged_layout, true><<<lookback_grid(ctx, NCAND), prim::kThreads, 0, ctx->stream>>>(
            f, ctx->d_words + W_NU, ctx->d_words + W_NS, ctx->d_words + W_OUTBYTES, (uint64_t *)out->begin.p,
            (unsigned long long *)(ctx->d_words + W_MAXNORM), lbc, lbb, lbt);
        QD_TRY(launched(ctx));
    }
    clk.end(4);
    st = read_words(ctx);
    if (st) return st;
    clk.harvest();
    const uint64_t NS = ctx->h_words[W_NS], outbytes = ctx->h_words[W_OUTBYTES];
    out->n_inst = 0;
    out->h_inst_begin.clear();
    if (NS == 0) {
        out->n = 0;
        out->nbytes = 0;
        out->total_proba = 0;
        out->total_pending = false;
        QD_TRY(ensure(out->objects, 8));
        QD_CUDA(cudaMemsetAsync(out->begin.p, 0, sizeof(uint64_t), ctx->stream));
    } else {
        QD_TRY(ensure(out->objects, outbytes));
        QD_TRY(set_word(ctx, W_ACC, 0));
        QD_TRY(set_word(ctx, (qd_word)(W_ACC + 1), 0));
        QD_TRY(set_word(ctx, W_DONE, 0));
        clk.begin(5);
        prim::k_fix_total<<<grid_for(ctx, NS, 4), prim::kThreads, 0, ctx->stream>>>(
            (const double2 *)out->mag.p, ctx->d_words + W_NS, (const unsigned long long *)(ctx->d_words + W_MAXNORM),
            (unsigned long long *)(ctx->d_words + W_ACC), (unsigned int *)(ctx->d_words + W_DONE),
            (double *)(ctx->d_words + W_TOTAL), (double *)(ctx->d_words + W_FACTOR));
        QD_TRY(launched(ctx));
        QD_CUDA(cudaMemcpyAsync(out->d_total.p, ctx->d_words + W_TOTAL, sizeof(double), cudaMemcpyDeviceToDevice,
                                ctx->stream));
        clk.end(5);
        clk.begin(6);
        QD_TRY(launch_populate_kernel(
            ctx, NS, maxsize > kStageMin, rs, pv, pc_source{(const uint32_t *)rb.spar.p, (const uint32_t *)rb.scid.p},
            ctx->d_words + W_NS, (const uint64_t *)out->begin.p, (const uint32_t *)out->size.p,
            (char *)out->objects.p, (double2 *)out->mag.p, (const double *)(ctx->d_words + W_FACTOR), nullptr, err,
            post));
        clk.end(6);
        out->n = NS;
        out->nbytes = outbytes;
        out->total_pending = true;
    }
    // the range buffers are released on return; this also reads the status
    // of the last kernels
    st = read_words(ctx);
    if (st) return st;
    clk.harvest();
    s.num_object_out = NS;
    s.out_bytes = outbytes;
    if (timing) {
        QD_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
        QD_CUDA(cudaStreamSynchronize(ctx->stream));
        cudaEventElapsedTime(&s.ms_total, ctx->ev0, ctx->ev1);
        if (out->total_pending) {
            double tp;
            QD_CUDA(cudaMemcpy(&tp, out->d_total.p, sizeof(double), cudaMemcpyDeviceToHost));
            out->total_proba = tp;
            out->total_pending = false;
        }
        s.total_proba = out->total_proba;
    } else if (NS == 0) {
        s.total_proba = 0;
    }
    s.kernel_launches = ctx->launches - launches0;
    const double sp = (double)in->nbytes, sbar_p = N ? sp / (double)N : 0, sbar_c = NS ? (double)outbytes / NS : 0;
    s.algorithmic_bytes = sp + 24.0 * N + 72.0 * (double)NC + 24.0 * (double)NU + (double)NS * (sbar_p + sbar_c + 24.0);
    if (stats) *stats = s;
    return QUIDS_OK;
}

// a rule step: one pass, or hash-range passes when its children need them
template <class Rule, class Post = no_post>
int simulate_step(quids_gpu_ctx *ctx, quids_gpu_state *in, const Rule &rule, quids_gpu_state *out,
                  const quids_gpu_params &prm, quids_gpu_step_stats *stats, const Post &post = Post{}) {
    const int rc = simulate_rule(ctx, in, rule, out, prm, stats, post);
    if (rc != kNeedRanges) return rc;
    // the range passes recompute the children with the rule's hash_child
    if constexpr (has_hash_child<Rule>::value)
        return simulate_ranges(ctx, in, rule, out, prm, stats, post);
    else
        return QUIDS_ERR_UNSUPPORTED;
}

}  // namespace qd::ranges
