// batch.cuh -- many independent QuIDS states ("instances") stepped together.
//
// A batched state is an ordinary state whose objects carry an instance id,
// each instance's objects contiguous and in instance order.  One rule step
// runs one pipeline over all instances: the rule of a parent comes from a
// per-instance table (different angles per instance), child hashes are
// tagged with the instance so groups never span instances, both truncations
// are segmented top-k selections with the same cap for every instance, and
// each instance is normalised by its own total probability.  Every instance
// goes through the step of quids::simulate (src/quids.hpp:448-543) with
// max_num_object > 0.
//
// Every list the step builds (parents, children, groups, survivors) stays
// sorted by instance, so instance offsets are found from the boundaries of
// the instance ids, with no atomics per item.
#pragma once
#include "engine.cuh"

namespace qd::batch {

using namespace qd::engine;

constexpr uint32_t kMaxInstances = 65536;

// ------------------------------------------------------------ kernels
// Instance offsets of a list sorted by instance: begin[g] = the first item
// of instance g (items of the empty instances start where the next begins),
// begin[G] = n.  Item j writes begin[g] for g in (inst(j-1), inst(j)], which
// partitions [0, G]: every entry is written exactly once.
template <class A>
__global__ void __launch_bounds__(prim::kThreads)
    k_inst_bounds(A inst, const uint64_t *d_n, uint32_t G, uint64_t *begin, const uint64_t *stop = nullptr) {
    if (stop && *stop) return;  // a planned run stopped: the output state is left alone
    const uint64_t n = *d_n;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j <= n; j += (uint64_t)gridDim.x * blockDim.x) {
        const int64_t prev = j == 0 ? -1 : (int64_t)inst(j - 1);
        const int64_t cur = j == n ? (int64_t)G : (int64_t)inst(j);
        for (int64_t g = prev + 1; g <= cur; ++g) begin[g] = j;
    }
}
struct inst_direct {
    const uint32_t *inst;
    __device__ __forceinline__ uint32_t operator()(uint64_t j) const { return inst[j]; }
};
struct inst_of_kept {
    const uint32_t *inst;
    const uint64_t *pidx;
    __device__ __forceinline__ uint32_t operator()(uint64_t j) const { return inst[pidx[j]]; }
};

// one selection per instance: keep the top k of begin[g+1] - begin[g] items
static __global__ void k_bselect_init(prim::select_state *st, const uint64_t *begin, uint32_t G, uint64_t k) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < G; g += gridDim.x * blockDim.x) {
        prim::select_state s{};
        s.k_rem = k;
        s.active = begin[g + 1] - begin[g] > k ? 1u : 0u;
        st[g] = s;
    }
}

// histogram of the next digit, per instance (bins g * 256 + digit); lanes
// with the same bin aggregate their count
template <class K>
__global__ void __launch_bounds__(prim::kThreads)
    k_bradix_hist(K kf, const uint32_t *item_inst, const uint64_t *d_n, const prim::select_state *st, int shift,
                  unsigned int *hist) {
    const uint64_t n = *d_n;
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    const uint64_t warp = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (uint64_t base = warp * 32; base < n; base += warps * 32) {
        const uint64_t i = base + lane;
        uint64_t bin = ~0ull;
        if (i < n) {
            const uint32_t g = item_inst[i];
            const prim::select_state &s = st[g];
            if (s.active) {
                const uint64_t k = kf.key(i);
                if ((k & s.mask) == s.prefix) bin = (uint64_t)g * prim::kBins + ((k >> shift) & (prim::kBins - 1));
            }
        }
        const unsigned same = __match_any_sync(0xffffffffu, bin);
        if (bin != ~0ull && lane == __ffs(same) - 1) atomicAdd(&hist[bin], (unsigned)__popc(same));
    }
}

// one block per instance: the digit holding the instance's k-th item (larger
// keys first); clears the instance's histogram
static __global__ void __launch_bounds__(prim::kBins) k_bradix_pick(prim::select_state *st, unsigned int *hist,
                                                                     int shift) {
    __shared__ uint64_t sm[prim::kBins];
    prim::select_state *s = st + blockIdx.x;
    unsigned int *h = hist + (uint64_t)blockIdx.x * prim::kBins;
    if (!s->active) return;  // uniform over the block
    const int t = threadIdx.x;
    const int d = prim::kBins - 1 - t;
    const uint64_t c = h[d];
    sm[t] = c;
    __syncthreads();
    for (int o = 1; o < prim::kBins; o <<= 1) {
        uint64_t v = t >= o ? sm[t - o] : 0;
        __syncthreads();
        sm[t] += v;
        __syncthreads();
    }
    const uint64_t incl = sm[t], excl = incl - c, k = s->k_rem;
    __syncthreads();
    if (excl < k && k <= incl) {
        s->prefix |= (uint64_t)d << shift;
        s->mask |= (uint64_t)(prim::kBins - 1) << shift;
        s->n_better += excl;
        s->k_rem = k - excl;
        s->n_equal = c;
    }
    h[d] = 0;
}

// items equal to their instance's threshold
template <class K>
__global__ void __launch_bounds__(prim::kThreads)
    k_btie_counts(K kf, const uint32_t *item_inst, const uint64_t *d_n, const prim::select_state *st,
                  unsigned long long *tiecnt) {
    const uint64_t n = *d_n;
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    const uint64_t warp = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (uint64_t base = warp * 32; base < n; base += warps * 32) {
        const uint64_t i = base + lane;
        uint32_t g = ~0u;
        if (i < n) {
            const uint32_t gi = item_inst[i];
            if (st[gi].active && kf.key(i) == st[gi].prefix) g = gi;
        }
        const unsigned same = __match_any_sync(0xffffffffu, g);
        if (g != ~0u && lane == __ffs(same) - 1) atomicAdd(&tiecnt[g], (unsigned long long)__popc(same));
    }
}

// out[i] = in[0] + ... + in[i-1] over a short array (one block), out[n] = total
static __global__ void __launch_bounds__(1024) k_small_excl_scan(const unsigned long long *in, uint32_t n,
                                                                  uint64_t *out) {
    __shared__ uint64_t sm[1024];
    const uint32_t per = (n + 1023) / 1024;
    uint64_t sum = 0;
    for (uint32_t k = 0; k < per; ++k) {
        uint32_t i = threadIdx.x * per + k;
        if (i < n) sum += in[i];
    }
    sm[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        uint64_t v = threadIdx.x >= (unsigned)o ? sm[threadIdx.x - o] : 0;
        __syncthreads();
        sm[threadIdx.x] += v;
        __syncthreads();
    }
    uint64_t run = threadIdx.x ? sm[threadIdx.x - 1] : 0;
    for (uint32_t k = 0; k < per; ++k) {
        uint32_t i = threadIdx.x * per + k;
        if (i < n) {
            out[i] = run;
            run += in[i];
        }
    }
    if (threadIdx.x == 1023) out[n] = sm[1023];
}

// per-instance thresholds (st), and tie_off[g] = ties of the instances
// before g, so a compaction's global tie rank minus tie_off is the rank
// within the instance
template <class K>
inline int segmented_select(quids_gpu_ctx *ctx, K kf, const uint32_t *item_inst, const uint64_t *d_n,
                            uint64_t n_host, const uint64_t *inst_begin, uint32_t G, uint64_t k,
                            prim::select_state *st, unsigned int *hist, unsigned long long *tiecnt,
                            uint64_t *tie_off) {
    const unsigned gsmall = (G + 255) / 256;
    k_bselect_init<<<gsmall, 256, 0, ctx->stream>>>(st, inst_begin, G, k);
    QD_CUDA(cudaMemsetAsync(hist, 0, (size_t)G * prim::kBins * sizeof(unsigned int), ctx->stream));
    QD_CUDA(cudaMemsetAsync(tiecnt, 0, (size_t)G * sizeof(unsigned long long), ctx->stream));
    const unsigned grid = grid_for(ctx, n_host);
    for (int shift = 64 - prim::kDigitBits; shift >= 0; shift -= prim::kDigitBits) {
        k_bradix_hist<<<grid, prim::kThreads, 0, ctx->stream>>>(kf, item_inst, d_n, st, shift, hist);
        k_bradix_pick<<<G, prim::kBins, 0, ctx->stream>>>(st, hist, shift);
    }
    k_btie_counts<<<grid, prim::kThreads, 0, ctx->stream>>>(kf, item_inst, d_n, st, tiecnt);
    k_small_excl_scan<<<1, 1024, 0, ctx->stream>>>(tiecnt, G, tie_off);
    return launched(ctx, 3 + 2 * 64 / prim::kDigitBits);
}

// parents kept by the per-instance pre-truncation (src/quids.hpp:486-487)
struct bkeep_parents {
    key_parent_norm kf;
    const uint32_t *inst;
    const prim::select_state *st;
    const uint64_t *tie_off;
    uint64_t *pidx;
    __device__ bool tie(uint64_t i) const {
        const prim::select_state &s = st[inst[i]];
        return s.active && kf.key(i) == s.prefix;
    }
    __device__ bool select(uint64_t i, uint64_t tie_rank) const {
        const uint32_t g = inst[i];
        const prim::select_state &s = st[g];
        if (!s.active) return true;
        const uint64_t k = kf.key(i);
        if (k > s.prefix) return true;
        if (k < s.prefix) return false;
        return tie_rank - tie_off[g] < s.k_rem;
    }
    __device__ void emit(uint64_t i, uint64_t j) const { pidx[j] = i; }
};

// groups kept after zero elimination, with their instance
struct bgroups_collect {
    group_view g;
    const uint32_t *cpar;
    const uint64_t *pidx;   // kept parent -> parent, or null
    const uint32_t *pinst;  // instance of each parent
    uint64_t *uchild;
    double2 *umag;
    uint64_t *unorm;
    uint32_t *uinst;
    using item = mag_t;
    __device__ bool load(uint64_t c, item &m) const { return g.kept(c, m); }
    __device__ void emit(uint64_t c, uint64_t j, const item &m) const {
        const uint64_t p = cpar[c];
        uchild[j] = c;
        umag[j] = make_double2(m.re, m.im);
        unorm[j] = (uint64_t)__double_as_longlong(cnorm(m));
        uinst[j] = pinst[pidx ? pidx[p] : p];
    }
};

// survivors of every instance's truncation into the output layout
// (src/quids.hpp:866-948; ties at an instance's cutoff by lower child index)
struct bkeep_layout {
    key_unorm kf;
    const uint64_t *uchild;
    const double2 *umag;
    const uint32_t *uinst;
    const prim::select_state *st;
    const uint64_t *tie_off;
    const uint32_t *csize;
    uint32_t align;
    double2 *omag;
    uint32_t *osize;
    uint64_t *obegin;
    uint64_t *schild;
    uint32_t *oinst;
    __device__ bool tie(uint64_t i) const {
        const prim::select_state &s = st[uinst[i]];
        return s.active && kf.key(i) == s.prefix;
    }
    __device__ bool rank_needed() const { return true; }  // ranks are offset per instance
    struct item {
        uint64_t c;
        uint32_t g;
        uint32_t size;
    };
    __device__ bool load(uint64_t i, uint64_t tie_rank, item &it) const {
        const uint32_t g = uinst[i];
        const prim::select_state &s = st[g];
        bool keep = true;
        if (s.active) {
            const uint64_t k = kf.key(i);
            keep = k > s.prefix || (k == s.prefix && tie_rank - tie_off[g] < s.k_rem);
        }
        if (keep) {
            it.c = uchild[i];
            it.g = g;
            it.size = csize[it.c];
        }
        return keep;
    }
    __device__ uint64_t bytes(const item &it) const { return padded_size(it.size, align); }
    // (returns 0: instances are normalised separately)
    __device__ double emit(uint64_t i, uint64_t j, uint64_t off, const item &it) const {
        const uint64_t c = it.c;
        omag[j] = umag[i];
        osize[j] = it.size;
        obegin[j] = off;
        schild[j] = c;
        oinst[j] = it.g;
        return 0.0;
    }
};

// Per-instance sums over a list sorted by instance: a lane takes a run of
// kRun consecutive items; the lanes of a warp, holding consecutive runs and
// so sorted by instance, combine with a segmented shuffle reduction, and the
// first lane of each instance segment commits the instance's partial.
constexpr int kRun = 8;

// largest survivor norm of each instance (IEEE bits of non-negative doubles
// order as integers)
static __global__ void __launch_bounds__(prim::kThreads)
    k_binst_max(const double2 *omag, const uint32_t *oinst, const uint64_t *d_ns, unsigned long long *maxn) {
    const uint64_t n = *d_ns;
    const uint64_t runs = (n + kRun - 1) / kRun;
    const int lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < runs; base += stride) {
        const uint64_t r = base + lane;
        uint32_t g = ~0u;
        unsigned long long mx = 0;
        if (r < runs) {
            const uint64_t j1 = r * kRun + kRun < n ? r * kRun + kRun : n;
            for (uint64_t j = r * kRun; j < j1; ++j) {
                const uint32_t gj = oinst[j];
                if (gj != g) {
                    if (g != ~0u) atomicMax(&maxn[g], mx);
                    g = gj;
                    mx = 0;
                }
                const double2 m = omag[j];
                const unsigned long long b = (unsigned long long)__double_as_longlong(cnorm(mag_t{m.x, m.y}));
                mx = mx > b ? mx : b;
            }
        }
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long v = __shfl_down_sync(0xffffffffu, mx, o);
            const uint32_t go = __shfl_down_sync(0xffffffffu, g, o);
            if (lane + o < 32 && go == g) mx = mx > v ? mx : v;
        }
        const uint32_t gp = __shfl_up_sync(0xffffffffu, g, 1);
        if (g != ~0u && (lane == 0 || gp != g)) atomicMax(&maxn[g], mx);
    }
}

// the fixed-point scale of instance g: that of the plain step on the
// instance alone (F of its largest norm and its survivor count), so each
// instance's total has the same bits as the plain step's
__device__ __forceinline__ int inst_scale(const unsigned long long *maxn, const uint64_t *obegin, uint32_t g) {
    return fix_scale(__longlong_as_double((long long)maxn[g]), obegin[g + 1] - obegin[g]);
}

// each instance's total probability, exact (k_fix_total per instance)
static __global__ void __launch_bounds__(prim::kThreads)
    k_binst_totals(const double2 *omag, const uint32_t *oinst, const uint64_t *d_ns, const uint64_t *obegin,
                   const unsigned long long *maxn, unsigned long long *tot) {
    const uint64_t n = *d_ns;
    const uint64_t runs = (n + kRun - 1) / kRun;
    const int lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < runs; base += stride) {
        const uint64_t r = base + lane;
        uint32_t g = ~0u;
        int F = 0;
        fix128 acc{0, 0};
        if (r < runs) {
            const uint64_t j1 = r * kRun + kRun < n ? r * kRun + kRun : n;
            for (uint64_t j = r * kRun; j < j1; ++j) {
                const uint32_t gj = oinst[j];
                if (gj != g) {
                    if (g != ~0u) prim::fix_atomic_add(&tot[2ull * g], acc);
                    g = gj;
                    F = inst_scale(maxn, obegin, g);
                    acc = fix128{0, 0};
                }
                const double2 m = omag[j];
                acc = fix_add(acc, to_fix(cnorm(mag_t{m.x, m.y}), F));
            }
        }
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t lo = __shfl_down_sync(0xffffffffu, acc.lo, o);
            const uint64_t hi = __shfl_down_sync(0xffffffffu, acc.hi, o);
            const uint32_t go = __shfl_down_sync(0xffffffffu, g, o);
            if (lane + o < 32 && go == g) acc = fix_add(acc, fix128{lo, hi});
        }
        const uint32_t gp = __shfl_up_sync(0xffffffffu, g, 1);
        if (g != ~0u && (lane == 0 || gp != g)) prim::fix_atomic_add(&tot[2ull * g], acc);
    }
}

static __global__ void k_binst_factors(const unsigned long long *tot, uint32_t G, const uint64_t *obegin,
                                       const unsigned long long *maxn, double *total, double *factor,
                                       const uint64_t *stop = nullptr) {
    if (stop && *stop) return;  // a planned run stopped: the output state is left alone
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < G; g += gridDim.x * blockDim.x) {
        const double t = from_fix(fix128{tot[2ull * g], tot[2ull * g + 1]}, inst_scale(maxn, obegin, g));
        total[g] = t;
        factor[g] = __dsqrt_rn(t);
    }
}

// per instance: children, groups after interference, survivors
static __global__ void k_binst_stats(const uint64_t *cbeg, const uint64_t *pbegin, const uint64_t *ubegin,
                                     const uint64_t *obegin, uint32_t G, uint64_t *out) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < G; g += gridDim.x * blockDim.x) {
        out[3ull * g + 0] = cbeg[pbegin[g + 1]] - cbeg[pbegin[g]];
        out[3ull * g + 1] = ubegin ? ubegin[g + 1] - ubegin[g] : 0;
        out[3ull * g + 2] = obegin ? obegin[g + 1] - obegin[g] : 0;
    }
}

// ------------------------------------------------------------ the step
// inst_stats: null, or [3 G] per-instance {children, groups after
// interference and zero elimination, survivors}.
template <class Rule>
int simulate_batched(quids_gpu_ctx *ctx, quids_gpu_state *in, const Rule *rules_host, quids_gpu_state *out,
                     const quids_gpu_params &prm, uint64_t *inst_stats, quids_gpu_step_stats *stats) {
    if (!ctx || !in || !out || in == out || in->ctx != ctx || out->ctx != ctx || !rules_host) return QUIDS_ERR_BAD_ARG;
    const uint32_t G = in->n_inst;
    if (G == 0 || in->h_inst_begin.size() != (size_t)G + 1) return QUIDS_ERR_BAD_ARG;
    if (prm.max_num_object == 0) return QUIDS_ERR_UNSUPPORTED;  // memory-driven truncation: plain steps only
    QD_CUDA(cudaSetDevice(ctx->device));
    const uint64_t N = in->n;
    const uint64_t maxc = prm.max_num_object;
    const double load = prm.table_load_factor > 0 && prm.table_load_factor < 0.95 ? prm.table_load_factor : 0.5;
    const bool fast = (prm.flags & QUIDS_FLAG_NO_FAST_HASH) == 0;
    const trunc_key tk{prm.simple_truncation == 0, prm.seed};
    const uint64_t launches0 = ctx->launches;
    quids_gpu_step_stats s{};
    s.num_parents = s.num_parents_kept = N;
    s.total_proba = std::numeric_limits<double>::quiet_NaN();

    QD_TRY(ensure(ctx->buf[B_RULES], (size_t)G * sizeof(Rule)));
    QD_TRY(ensure(ctx->buf[B_BCOUNT], (size_t)G * 7 * sizeof(unsigned long long)));
    QD_TRY(ensure(ctx->buf[B_BSEL], (size_t)G * sizeof(prim::select_state)));
    QD_TRY(ensure(ctx->buf[B_BHIST], (size_t)G * prim::kBins * sizeof(unsigned int)));
    QD_TRY(ensure(ctx->buf[B_BOFF], (size_t)(G + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_UBEGIN], (size_t)(G + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_PBEGIN], (size_t)(G + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_BFACTOR], (size_t)G * sizeof(double)));
    QD_CUDA(cudaMemcpyAsync(ctx->buf[B_RULES].p, rules_host, (size_t)G * sizeof(Rule), cudaMemcpyHostToDevice,
                            ctx->stream));
    unsigned long long *cnt = bufp<unsigned long long>(ctx, B_BCOUNT);
    unsigned long long *tiecnt = cnt, *tot = cnt + G;
    uint64_t *d_inst_stats = (uint64_t *)(cnt + 3ull * G);
    unsigned long long *maxn = cnt + 6ull * G;
    prim::select_state *bst = bufp<prim::select_state>(ctx, B_BSEL);
    unsigned int *bhist = bufp<unsigned int>(ctx, B_BHIST);
    uint64_t *tie_off = bufp<uint64_t>(ctx, B_BOFF);
    uint64_t *pbegin = bufp<uint64_t>(ctx, B_PBEGIN), *ubegin = bufp<uint64_t>(ctx, B_UBEGIN);
    QD_CUDA(cudaMemsetAsync(ctx->d_words, 0, W_COUNT_WORDS * sizeof(uint64_t), ctx->stream));
    if (ctx->buf[B_MODSTATUS].p) {
        k_take_status<<<1, 1, 0, ctx->stream>>>(bufp<int>(ctx, B_MODSTATUS), ctx->d_words + W_STATUS);
        QD_TRY(launched(ctx));
    }
    int *err = (int *)(ctx->d_words + W_STATUS);
    const uint32_t *pinst = (const uint32_t *)in->inst.p;
    const instance_rules<Rule> rs{bufp<Rule>(ctx, B_RULES), pinst};

    // an empty result: every instance without objects
    auto empty_out = [&]() -> int {
        out->n = 0;
        out->nbytes = 0;
        out->total_proba = 0;
        out->total_pending = false;
        QD_TRY(ensure_state(out, 0, 8));
        QD_TRY(ensure(out->inst, 8));
        QD_TRY(ensure(out->inst_begin, (size_t)(G + 1) * sizeof(uint64_t)));
        QD_TRY(ensure(out->inst_total, (size_t)G * sizeof(double)));
        QD_CUDA(cudaMemsetAsync(out->begin.p, 0, sizeof(uint64_t), ctx->stream));
        QD_CUDA(cudaMemsetAsync(out->inst_begin.p, 0, (size_t)(G + 1) * sizeof(uint64_t), ctx->stream));
        QD_CUDA(cudaMemsetAsync(out->inst_total.p, 0, (size_t)G * sizeof(double), ctx->stream));
        QD_CUDA(cudaStreamSynchronize(ctx->stream));
        out->n_inst = G;
        out->h_inst_begin.assign((size_t)G + 1, 0);
        s.kernel_launches = ctx->launches - launches0;
        if (stats) *stats = s;
        return QUIDS_OK;
    };
    if (N == 0) {
        if (inst_stats) std::memset(inst_stats, 0, (size_t)G * 3 * sizeof(uint64_t));
        return empty_out();
    }

    // ---- num_child (src/quids.hpp:686-701)
    QD_TRY(set_word(ctx, W_N, N));
    QD_TRY(ensure(ctx->buf[B_NCHILD], N * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_CBEGIN], (N + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_LOOKBACK], 3 * ((N + prim::kTile - 1) / prim::kTile + 2) * sizeof(uint64_t)));
    k_num_child<<<grid_for(ctx, N), prim::kThreads, 0, ctx->stream>>>(
        rs, (const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p, N,
        bufp<uint32_t>(ctx, B_NCHILD), (unsigned long long *)(ctx->d_words + W_MAXSIZE), err);
    QD_TRY(launched(ctx));

    // ---- per-instance parent pre-truncation (src/quids.hpp:486-487), only
    // when some instance holds more than max_num_object parents
    bool cut_parents = false;
    for (uint32_t g = 0; g < G; ++g)
        if (in->h_inst_begin[g + 1] - in->h_inst_begin[g] > maxc) cut_parents = true;
    const uint64_t *pidx = nullptr;
    if (cut_parents) {
        QD_TRY(ensure(ctx->buf[B_PIDX], N * sizeof(uint64_t)));
        key_parent_norm kp{(const double2 *)in->mag.p, tk};
        QD_TRY(segmented_select(ctx, kp, pinst, ctx->d_words + W_N, N, (const uint64_t *)in->inst_begin.p, G, maxc,
                                bst, bhist, tiecnt, tie_off));
        prim::lookback lb, lbt;
        QD_TRY(lookback_chain(ctx, N, 0, lb));
        QD_TRY(lookback_chain(ctx, N, 2, lbt));
        bkeep_parents f{kp, pinst, bst, tie_off, bufp<uint64_t>(ctx, B_PIDX)};
        prim::k_compact_ranked<<<lookback_grid(ctx, N), prim::kThreads, 0, ctx->stream>>>(
            f, ctx->d_words + W_N, ctx->d_words + W_NP, lb, lbt);
        QD_TRY(launched(ctx));
        pidx = bufp<uint64_t>(ctx, B_PIDX);
        k_inst_bounds<<<grid_for(ctx, N), prim::kThreads, 0, ctx->stream>>>(inst_of_kept{pinst, pidx},
                                                                           ctx->d_words + W_NP, G, pbegin);
        QD_TRY(launched(ctx));
    } else {
        QD_TRY(set_word(ctx, W_NP, N));
        QD_CUDA(cudaMemcpyAsync(pbegin, in->inst_begin.p, (size_t)(G + 1) * sizeof(uint64_t),
                                cudaMemcpyDeviceToDevice, ctx->stream));
    }

    // ---- child offsets over the kept parents
    {
        prim::lookback lb;
        QD_TRY(lookback_chain(ctx, N, 1, lb));
        scan_nchild f{bufp<uint32_t>(ctx, B_NCHILD), pidx};
        prim::k_scan_excl<<<lookback_grid(ctx, N), prim::kThreads, 0, ctx->stream>>>(
            f, ctx->d_words + W_NP, bufp<uint64_t>(ctx, B_CBEGIN), ctx->d_words + W_NC, lb);
        QD_TRY(launched(ctx));
    }
    int st = read_words(ctx);  // host synchronisation 1: buffer sizes
    if (st) return st;
    const uint64_t NP = ctx->h_words[W_NP];
    const uint64_t NC = ctx->h_words[W_NC];
    const uint64_t maxsize = ctx->h_words[W_MAXSIZE];
    s.num_parents_kept = NP;
    s.num_object = NC;
    s.max_child_size = maxsize;
    if (NC == 0) {
        if (inst_stats) std::memset(inst_stats, 0, (size_t)G * 3 * sizeof(uint64_t));
        return empty_out();
    }
    if (NC >= 0xffffffffull || maxsize > 4096) {  // child indices are u32 in the table
        if (stats) *stats = s;
        return NC >= 0xffffffffull ? QUIDS_ERR_CHILD_COUNT_OVERFLOW : QUIDS_ERR_SIZE_BOUND;
    }
    parents_view pv{(const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p,
                    (const double2 *)in->mag.p, bufp<uint64_t>(ctx, B_CBEGIN), pidx, NP};

    uint64_t M = (uint64_t)((double)NC / load) + 1;
    if (M < 1024) M = 1024;
    if (M >= 0x7ffffff0ull) return QUIDS_ERR_OOM;
    s.table_capacity = M;
    const uint64_t tiles_nc = (NC + prim::kTile - 1) / prim::kTile;
    const uint64_t sym_tiles = (NC + kTileChildren - 1) / kTileChildren;
    const uint64_t NSB = NC < maxc * (uint64_t)G ? NC : maxc * (uint64_t)G;
    QD_TRY(ensure(ctx->buf[B_HASH], NC * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_CMAG], NC * sizeof(double2)));
    QD_TRY(ensure(ctx->buf[B_CSIZE], NC * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_CPAR], NC * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_SLOT], NC * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_NOTREP], NC));
    QD_TRY(ensure(ctx->buf[B_HASJOIN], NC));
    QD_TRY(ensure(ctx->buf[B_KEYS], (M + 1) * sizeof(prim::table_slot)));
    QD_TRY(ensure(ctx->buf[B_ACC], 4 * (M + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_UCHILD], NC * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_UMAG], NC * sizeof(double2)));
    QD_TRY(ensure(ctx->buf[B_UNORM], NC * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_UINST], NC * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_SCHILD], NSB * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_LOOKBACK], 3 * (tiles_nc + 2) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_TILEPAR], (sym_tiles + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(out->begin, (NSB + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(out->size, NSB * sizeof(uint32_t)));
    QD_TRY(ensure(out->mag, NSB * sizeof(double2)));
    QD_TRY(ensure(out->inst, NSB * sizeof(uint32_t)));
    QD_TRY(ensure(out->inst_begin, (size_t)(G + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(out->inst_total, (size_t)G * sizeof(double)));
    QD_TRY(ensure(out->d_total, sizeof(double)));

    // the collision table, cleared before the symbolic pass (whose grouped
    // form claims the slots)
    prim::table tb{bufp<prim::table_slot>(ctx, B_KEYS), bufp<unsigned long long>(ctx, B_ACC), M, probe_limit(prm)};
    QD_CUDA(cudaMemsetAsync(tb.slots, 0xff, (M + 1) * sizeof(prim::table_slot), ctx->stream));
    QD_CUDA(cudaMemsetAsync(tb.acc + 4 * M, 0, 4 * sizeof(uint64_t), ctx->stream));
    QD_CUDA(cudaMemsetAsync(ctx->buf[B_NOTREP].p, 0, NC, ctx->stream));
    QD_CUDA(cudaMemsetAsync(ctx->buf[B_HASJOIN].p, 0, NC, ctx->stream));

    // ---- symbolic iteration (src/quids.hpp:705-719), instance-tagged hashes
    bool grouped = false;
    if constexpr (has_grouped<Rule>::value) {
        if (fast) {
            QD_TRY(launch_symbolic_grouped(ctx, rs, pv, NC, table_claim{tb, bufp<uint32_t>(ctx, B_SLOT), err}));
            grouped = true;
        }
    }
    if (!grouped) {
        k_tile_parents<<<grid_for(ctx, NP), prim::kThreads, 0, ctx->stream>>>(
            bufp<uint64_t>(ctx, B_CBEGIN), NP, sym_tiles, bufp<uint64_t>(ctx, B_TILEPAR));
        QD_TRY(launched(ctx));
        if (maxsize <= 256) {
            QD_TRY((launch_symbolic<instance_rules<Rule>, 256>(ctx, rs, pv, NC, fast)));
        } else {
            QD_TRY((launch_symbolic<instance_rules<Rule>, 4096>(ctx, rs, pv, NC, fast)));
        }
    }

    // ---- collision elimination (src/quids.hpp:785-809)
    uint8_t *not_rep = bufp<uint8_t>(ctx, B_NOTREP), *has_join = bufp<uint8_t>(ctx, B_HASJOIN);
    const unsigned long long *d_maxabs = (const unsigned long long *)(ctx->d_words + W_MAXABS);
    direct_src src{bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG)};
    if (!grouped) {
        prim::k_table_claim<<<grid_for(ctx, NC), prim::kThreads, 0, ctx->stream>>>(tb, src, ctx->d_words + W_NC,
                                                                                  bufp<uint32_t>(ctx, B_SLOT), err);
        QD_TRY(launched(ctx));
    }
    prim::k_table_accumulate<<<grid_for(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
        tb, src, bufp<uint32_t>(ctx, B_SLOT), ctx->d_words + W_NC, d_maxabs, not_rep, has_join);
    QD_TRY(launched(ctx));

    // ---- zero elimination (src/quids.hpp:819-823), groups with their instance
    group_view gv{bufp<uint32_t>(ctx, B_SLOT), not_rep, has_join, bufp<double2>(ctx, B_CMAG),
                  bufp<unsigned long long>(ctx, B_ACC), ctx->d_words + W_NC, d_maxabs, prm.tolerance};
    {
        prim::lookback lb;
        QD_TRY(lookback_chain(ctx, NC, 0, lb));
        bgroups_collect f{gv, bufp<uint32_t>(ctx, B_CPAR), pidx, pinst, bufp<uint64_t>(ctx, B_UCHILD),
                          bufp<double2>(ctx, B_UMAG), bufp<uint64_t>(ctx, B_UNORM), bufp<uint32_t>(ctx, B_UINST)};
        prim::k_compact<<<lookback_grid(ctx, NC), prim::kThreads, 0, ctx->stream>>>(f, ctx->d_words + W_NC,
                                                                                   ctx->d_words + W_NU, lb);
        k_inst_bounds<<<grid_for(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
            inst_direct{bufp<uint32_t>(ctx, B_UINST)}, ctx->d_words + W_NU, G, ubegin);
        QD_TRY(launched(ctx, 2));
    }

    // ---- per-instance truncation (src/quids.hpp:866-900) and layout
    key_unorm k1{bufp<uint64_t>(ctx, B_UNORM), bufp<uint64_t>(ctx, B_UCHILD), tk};
    QD_TRY(segmented_select(ctx, k1, bufp<uint32_t>(ctx, B_UINST), ctx->d_words + W_NU, NC, ubegin, G, maxc, bst,
                            bhist, tiecnt, tie_off));
    {
        prim::lookback lbc, lbb, lbt;
        QD_TRY(lookback_chain(ctx, NC, 0, lbt));
        QD_TRY(lookback_chain(ctx, NC, 1, lbc));
        QD_TRY(lookback_chain(ctx, NC, 2, lbb));
        bkeep_layout kl{k1, bufp<uint64_t>(ctx, B_UCHILD), bufp<double2>(ctx, B_UMAG), bufp<uint32_t>(ctx, B_UINST),
                        bst, tie_off, bufp<uint32_t>(ctx, B_CSIZE), prm.align_byte_length, (double2 *)out->mag.p,
                        (uint32_t *)out->size.p, (uint64_t *)out->begin.p, bufp<uint64_t>(ctx, B_SCHILD),
                        (uint32_t *)out->inst.p};
        prim::k_compact_layout<bkeep_layout, true><<<lookback_grid(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
            kl, ctx->d_words + W_NU, ctx->d_words + W_NS, ctx->d_words + W_OUTBYTES, (uint64_t *)out->begin.p,
            nullptr, lbc, lbb, lbt);
        QD_TRY(launched(ctx));
    }
    st = read_words(ctx);  // host synchronisation 2: output size
    if (st) return st;
    const uint64_t NS = ctx->h_words[W_NS], NU = ctx->h_words[W_NU], outbytes = ctx->h_words[W_OUTBYTES];
    s.num_object_after_interferences = NU;
    if (NS == 0) {
        if (inst_stats) {
            k_binst_stats<<<(G + 255) / 256, 256, 0, ctx->stream>>>(bufp<uint64_t>(ctx, B_CBEGIN), pbegin, ubegin,
                                                                  nullptr, G, d_inst_stats);
            QD_TRY(launched(ctx));
            QD_CUDA(cudaMemcpyAsync(inst_stats, d_inst_stats, (size_t)G * 3 * sizeof(uint64_t),
                                    cudaMemcpyDeviceToHost, ctx->stream));
        }
        return empty_out();
    }
    QD_TRY(ensure(out->objects, outbytes));

    // ---- per-instance normalisation (src/quids.hpp:1004-1013) and finalize
    uint64_t *obegin = (uint64_t *)out->inst_begin.p;
    QD_CUDA(cudaMemsetAsync(tot, 0, (size_t)G * 2 * sizeof(unsigned long long), ctx->stream));
    QD_CUDA(cudaMemsetAsync(maxn, 0, (size_t)G * sizeof(unsigned long long), ctx->stream));
    k_inst_bounds<<<grid_for(ctx, NS), prim::kThreads, 0, ctx->stream>>>(
        inst_direct{(const uint32_t *)out->inst.p}, ctx->d_words + W_NS, G, obegin);
    const unsigned grid_runs = grid_for(ctx, (NS + kRun - 1) / kRun);
    k_binst_max<<<grid_runs, prim::kThreads, 0, ctx->stream>>>((const double2 *)out->mag.p,
                                                              (const uint32_t *)out->inst.p, ctx->d_words + W_NS, maxn);
    k_binst_totals<<<grid_runs, prim::kThreads, 0, ctx->stream>>>(
        (const double2 *)out->mag.p, (const uint32_t *)out->inst.p, ctx->d_words + W_NS, obegin, maxn, tot);
    k_binst_factors<<<(G + 255) / 256, 256, 0, ctx->stream>>>(tot, G, obegin, maxn, (double *)out->inst_total.p,
                                                             bufp<double>(ctx, B_BFACTOR));
    QD_TRY(launched(ctx, 4));
    QD_TRY(launch_populate_kernel(
        ctx, NS, maxsize > kStageMin, rs, pv,
        schild_source{bufp<uint64_t>(ctx, B_SCHILD), bufp<uint32_t>(ctx, B_CPAR), pv.cbeg}, ctx->d_words + W_NS,
        (const uint64_t *)out->begin.p, (const uint32_t *)out->size.p, (char *)out->objects.p, (double2 *)out->mag.p,
        bufp<double>(ctx, B_BFACTOR), (const uint32_t *)out->inst.p, err, no_post{}));
    if (inst_stats) {
        k_binst_stats<<<(G + 255) / 256, 256, 0, ctx->stream>>>(bufp<uint64_t>(ctx, B_CBEGIN), pbegin, ubegin,
                                                              (const uint64_t *)out->inst_begin.p, G, d_inst_stats);
        QD_TRY(launched(ctx));
        QD_CUDA(cudaMemcpyAsync(inst_stats, d_inst_stats, (size_t)G * 3 * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                                ctx->stream));
    }
    out->h_inst_begin.resize((size_t)G + 1);
    QD_CUDA(cudaMemcpyAsync(out->h_inst_begin.data(), out->inst_begin.p, (size_t)(G + 1) * sizeof(uint64_t),
                            cudaMemcpyDeviceToHost, ctx->stream));
    st = read_words(ctx);  // host synchronisation 3: instance offsets, status
    if (st) return st;
    out->n = NS;
    out->nbytes = outbytes;
    out->n_inst = G;
    out->total_pending = false;
    out->total_proba = std::numeric_limits<double>::quiet_NaN();  // per instance: inst_total
    s.num_object_out = NS;
    s.out_bytes = outbytes;
    s.kernel_launches = ctx->launches - launches0;
    const double sp = (double)in->nbytes, sbar_p = N ? sp / (double)N : 0, sbar_c = (double)outbytes / NS;
    s.algorithmic_bytes = sp + 28.0 * N + 76.0 * NC + 28.0 * NU + (double)NS * (sbar_p + sbar_c + 28.0);
    if (stats) *stats = s;
    return QUIDS_OK;
}

}  // namespace qd::batch
