// planned.cuh -- planned rule steps: the step of engine.cuh without its two
// host waits, for runs whose sizes are known beforehand (the reference's
// examples loop over simulate calls, examples/quantum_computer_test.cpp:26-49,
// each step sizing its buffers as it goes, src/quids.hpp:448-543).
//
// A step sizes its buffers from the child count and from the survivors'
// bytes, so simulate_rule waits for both on the host.  A run of ops that is
// repeated (the same gate list from an input of the same size) has the sizes
// of its earlier run: a *plan* holds, per rule step, bounds on its parents,
// children, survivors and output bytes.  A planned step allocates to those
// bounds and launches its kernels with grids that cover them; the kernels
// read the true counts from device words, as they always do.  So nothing
// waits on the host, the whole run is one stream of launches, and it can be
// captured once as a CUDA graph and replayed.
//
// Guards on the device keep the result exact:
//  * k_plan_begin: the step's parents fit the plan (and need no parent
//    pre-truncation);
//  * plan_sizes, run by the last block of the child-offset scan: the
//    children fit, the child size bound fits the symbolic pass chosen, and a
//    step planned without truncation still needs none;
//  * plan_end, run by the last block of the layout compaction: the output
//    bytes fit.
// A step that does not fit sets the status kReplan and the step index, and
// from then on every step and modifier of the run does nothing: the failed
// step's input state is left as it was (no kernel writes it), so the host
// resumes the run there with the synchronous steps.  A real error (an unfit
// object, a full table, ...) stops the run the same way and is returned.
#pragma once
#include <cstring>
#include <limits>
#include <vector>

#include "engine.cuh"

namespace qd::planned {
using namespace qd::engine;

constexpr int kReplan = -1000;  // internal: a planned step's sizes exceeded its plan
constexpr int kNotRun = -1002;  // internal: the plan's buffers could not be had; nothing was launched

// bounds of one rule step of a planned run
struct app_plan {
    uint64_t n_cap;        // parents
    uint64_t nc_cap;       // children
    uint64_t ns_cap;       // survivors
    uint64_t bytes_cap;    // output object bytes
    uint64_t maxsize_lim;  // child size bound of the generic symbolic pass (256 or 4096)
    uint64_t maxsize;      // the recorded child size bound (the populate stages objects above kStageMin)
    bool may_truncate;     // the step takes the truncation path (select, then keep + layout)
    bool partition = false;  // collisions by partition (collide.cuh), else the table
};

// A plan: the op list and knobs it was made for, the two state handles, and
// the bounds of each rule step; once a planned run of it has succeeded, the
// run captured as a CUDA graph (valid while no buffer has been reallocated
// and the input has the size it was captured with).
struct run_plan {
    std::vector<quids_gpu_op> ops;
    quids_gpu_params prm{};
    quids_gpu_state *a = nullptr, *b = nullptr;
    std::vector<app_plan> apps;
    uint64_t runs = 0;                 // planned runs that succeeded
    cudaGraphExec_t exec = nullptr;
    uint64_t epoch = 0;                // allocation epoch of the capture
    uint64_t n0 = 0, bytes0 = 0;       // input size of the capture
    uint64_t graph_launches = 0;       // kernels in the graph
    // batched runs: the instances, the per-step per-instance rule parameters
    // (empty: every instance takes its op's), and every step's rules on the
    // device (rule_off: byte offset of each step's)
    uint32_t n_inst = 0;
    std::vector<quids_gpu_rule_params> inst_params;
    qd_dbuf rules;
    std::vector<uint64_t> rule_off;
    bool rules_ready = false;
    // launch knobs of the run (QUIDS_FLAG_AUTOTUNE: chosen by timing before the first capture)
    qd_knobs knobs;
    bool tuned = false;
    qd_dbuf backup[6];  // the run's input while it is autotuned
    ~run_plan() {
        if (exec) cudaGraphExecDestroy(exec);
        release(rules);
        for (auto &b : backup) release(b);
    }
};

inline run_plan *find_plan(quids_gpu_ctx *ctx, const quids_gpu_state *a, const quids_gpu_state *b,
                           const quids_gpu_op *ops, uint64_t n_ops, const quids_gpu_params &prm, uint32_t n_inst,
                           const quids_gpu_rule_params *inst_params) {
    uint64_t n_rules = 0;
    for (uint64_t i = 0; i < n_ops; ++i) n_rules += ops[i].is_rule ? 1 : 0;
    const size_t n_ip = inst_params ? (size_t)n_rules * n_inst : 0;
    for (run_plan *p : ctx->plans)
        if (p->a == a && p->b == b && p->n_inst == n_inst && p->ops.size() == n_ops &&
            (n_ops == 0 || std::memcmp(p->ops.data(), ops, n_ops * sizeof(quids_gpu_op)) == 0) &&
            std::memcmp(&p->prm, &prm, sizeof(prm)) == 0 && p->inst_params.size() == n_ip &&
            (n_ip == 0 || std::memcmp(p->inst_params.data(), inst_params, n_ip * sizeof(quids_gpu_rule_params)) == 0))
            return p;
    return nullptr;
}

inline void drop_plan(quids_gpu_ctx *ctx, run_plan *p) {
    for (size_t k = 0; k < ctx->plans.size(); ++k)
        if (ctx->plans[k] == p) {
            ctx->plans.erase(ctx->plans.begin() + (long)k);
            delete p;
            return;
        }
}

inline void drop_plans_of(quids_gpu_ctx *ctx, const quids_gpu_state *st) {
    for (size_t k = ctx->plans.size(); k-- > 0;)
        if (ctx->plans[k]->a == st || ctx->plans[k]->b == st) {
            delete ctx->plans[k];
            ctx->plans.erase(ctx->plans.begin() + (long)k);
        }
}

// what each planned step reports (words per step, written by plan_end
// into mapped host memory)
enum { R_N, R_NC, R_NU, R_NS, R_BYTES, R_MAXSIZE, R_M, R_DONE, R_WORDS };

__device__ __forceinline__ bool stopped(const uint64_t *words) { return (uint32_t)words[W_STATUS] != 0; }
__device__ __forceinline__ void stop_at(uint64_t *words, uint32_t app, int code) {
    if (!stopped(words)) words[W_STATUS] = (uint64_t)(uint32_t)code;
    if (words[W_FAILAPP] == ~0ull) words[W_FAILAPP] = app;
}

// Start of a planned run: no status, no failing step.
static __global__ void k_plan_start(uint64_t *words) {
    words[W_STATUS] = 0;
    words[W_FAILAPP] = ~0ull;
}

// Start of planned step `app`: the step's words (the run's status and
// failing step carried over), a sticky modifier status moved in, the parent
// count from the input state's device words (or n_host for the run's
// input), and nzero zeroed words of look-back chains.
static __global__ void __launch_bounds__(256)
    k_plan_begin(uint64_t *words, uint32_t app, uint64_t n_host, const uint64_t *in_meta, uint64_t n_cap,
                 uint64_t maxn, int *modstatus, uint64_t *zero, uint64_t nzero) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid == 0) {
        uint64_t st = words[W_STATUS];
        uint64_t fail = words[W_FAILAPP];
        if (modstatus && *modstatus) {
            if (!(uint32_t)st) st = (uint64_t)(uint32_t)*modstatus;
            *modstatus = 0;
        }
        uint64_t n = in_meta ? in_meta[0] : n_host;
        if (!(uint32_t)st && (n > n_cap || n > maxn)) st = (uint64_t)(uint32_t)kReplan;
        if ((uint32_t)st && fail == ~0ull) fail = app;
        if ((uint32_t)st) n = 0;
        for (int w = 0; w < W_COUNT_WORDS; ++w) words[w] = 0;
        words[W_N] = n;
        words[W_NP] = n;
        words[W_STATUS] = st;
        words[W_FAILAPP] = fail;
    }
    for (uint64_t i = tid; i < nzero; i += (uint64_t)gridDim.x * blockDim.x) zero[i] = 0;
}

// After the child count: check the children against the plan, stop the
// step if they do not fit (or an earlier kernel failed), and size the
// collision table on the device: M = max(NC / load + 1, 1024) slots as the
// synchronous step computes it, with the extra slot's sum cleared.
// (run by the last block of the child-offset scan: plan_sizes_hook)
__device__ __forceinline__ void plan_sizes(uint64_t *words, uint32_t app, uint64_t nc_cap, uint64_t maxsize_lim,
                                           uint64_t nc_no_trunc, double load, unsigned long long *acc) {
    uint64_t nc = words[W_NC];
    if (!stopped(words) && nc > 0) {
        const uint64_t ms = words[W_MAXSIZE];
        if (ms > 4096)
            stop_at(words, app, QUIDS_ERR_SIZE_BOUND);  // per-thread child buffer bound, as the synchronous step
        else if (nc > nc_cap || ms > maxsize_lim || nc > nc_no_trunc)
            stop_at(words, app, kReplan);
    }
    if (stopped(words)) {
        stop_at(words, app, 0);
        words[W_NC] = 0;
        words[W_NP] = 0;
        nc = 0;
    }
    if (!acc) return;  // collisions by partition: no table
    uint64_t m = (uint64_t)((double)nc / load) + 1;
    if (m < 1024) m = 1024;
    words[W_M] = m;
    for (int k = 0; k < 4; ++k) acc[4 * m + k] = 0;
}

struct plan_sizes_hook {
    static constexpr bool active = true;
    uint64_t *words;
    uint32_t app;
    uint64_t nc_cap, maxsize_lim, nc_no_trunc;
    double load;
    unsigned long long *acc;
    __device__ void operator()() const { plan_sizes(words, app, nc_cap, maxsize_lim, nc_no_trunc, load, acc); }
};

// After the output layout: check the output bytes, publish the output
// state's size on the device and the step's counts to the host; a stopped
// step keeps no survivors (so the total and the populate do nothing) and
// leaves the output state's words alone.  (Run by the last block of the
// layout compaction: plan_end_hook.)
__device__ __forceinline__ void plan_end(uint64_t *words, uint32_t app, uint64_t bytes_cap, bool truncating,
                                         uint64_t *out_meta, volatile uint64_t *rec) {
    if (!stopped(words) && words[W_OUTBYTES] > bytes_cap) stop_at(words, app, kReplan);
    if (stopped(words)) {
        stop_at(words, app, 0);
        words[W_NS] = 0;
        return;
    }
    out_meta[0] = words[W_NS];
    out_meta[1] = words[W_OUTBYTES];
    rec[R_N] = words[W_N];
    rec[R_NC] = words[W_NC];
    rec[R_NU] = truncating ? words[W_NU] : words[W_NS];
    rec[R_NS] = words[W_NS];
    rec[R_BYTES] = words[W_OUTBYTES];
    rec[R_MAXSIZE] = words[W_MAXSIZE];
    rec[R_M] = words[W_M];
    rec[R_DONE] = 1;
}
struct plan_end_hook {
    static constexpr bool active = true;
    uint64_t *words;
    uint32_t app;
    uint64_t bytes_cap;
    bool truncating;
    uint64_t *out_meta;
    uint64_t *rec;
    __device__ void operator()() const { plan_end(words, app, bytes_cap, truncating, out_meta, rec); }
};
// the hooks' block counters (zeroed by k_plan_begin)
inline prim::publish hook_counter(quids_gpu_ctx *ctx, qd_word done) {
    prim::publish pb;
    pb.done = (unsigned int *)(ctx->d_words + done);
    return pb;
}

// The run's end: its status, failing step and the two states' sizes.
static __global__ void k_plan_finish(const uint64_t *words, const uint64_t *meta_a, const uint64_t *meta_b,
                                     volatile uint64_t *out) {
    out[0] = words[W_STATUS];
    out[1] = words[W_FAILAPP];
    out[2] = meta_a ? meta_a[0] : 0;
    out[3] = meta_a ? meta_a[1] : 0;
    out[4] = meta_b ? meta_b[0] : 0;
    out[5] = meta_b ? meta_b[1] : 0;
    __threadfence_system();
}

inline uint64_t sym_tiles_of(uint64_t nc) { return (nc + kTileChildren - 1) / kTileChildren; }

// the collision table's load factor of a step's knobs, and of a planned
// step: the tuned one, else the step's
inline double prm_load(const quids_gpu_params &prm) {
    return prm.table_load_factor > 0 && prm.table_load_factor < 0.95 ? prm.table_load_factor : 0.5;
}
inline double eff_load(const quids_gpu_ctx *ctx, const quids_gpu_params &prm) {
    return ctx->tune.load > 0 ? ctx->tune.load : prm_load(prm);
}

// The buffers of a planned step, at the plan's bounds (nothing grows while a
// run is captured).  keep: the output state's arrays keep their contents as
// they grow (the run's input state, which later steps write into).
inline int ensure_planned(quids_gpu_ctx *ctx, quids_gpu_state *out, const app_plan &ap, double load, bool keep) {
    const uint64_t N = ap.n_cap, NC = ap.nc_cap, NS = ap.ns_cap;
    const uint64_t M = std::max<uint64_t>((uint64_t)((double)NC / load) + 1, 1024);
    const uint64_t tiles_nc = (NC + prim::kTile - 1) / prim::kTile;
    QD_TRY(ensure(ctx->buf[B_NCHILD], (N ? N : 1) * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_LOOKBACK], std::max(lookback_words(N), 4 * (tiles_nc + 2)) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_CBEGIN], (N + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_LBEG], (N + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_TILEPAR], (std::max(sym_tiles_of(NC), NC / kLeaderTile) + 2) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_HASH], NC * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_CMAG], NC * sizeof(double2)));
    QD_TRY(ensure(ctx->buf[B_CSIZE], NC * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_CPAR], NC * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_SCHILD], NS * sizeof(uint64_t)));
    if (ap.may_truncate) QD_TRY(ensure(ctx->buf[B_SELCAND], filter_cap(NC) * sizeof(uint64_t)));
    if (ap.partition) {
        QD_TRY(pcs_ensure(ctx, NC, ap.may_truncate));
        QD_CUDA(cudaFuncSetAttribute(k_pcs_group, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)pcs_smem_bytes()));
    } else {
        QD_TRY(ensure(ctx->buf[B_SLOT], NC * sizeof(uint32_t)));
        QD_TRY(ensure(ctx->buf[B_NOTREP], NC));
        QD_TRY(ensure(ctx->buf[B_HASJOIN], NC));
        QD_TRY(ensure(ctx->buf[B_KEYS], (M + 1) * sizeof(prim::table_slot)));
        QD_TRY(ensure(ctx->buf[B_ACC], 4 * (M + 1) * sizeof(uint64_t)));
        if (ap.may_truncate) {
            QD_TRY(ensure(ctx->buf[B_UNORM], NC * sizeof(uint64_t)));
            QD_TRY(ensure(ctx->buf[B_KEEPCAND], NC * sizeof(uint32_t)));
            QD_TRY(ensure(ctx->buf[B_TILECNT], tilecnt_bytes(NC)));
        }
    }
    QD_TRY(ensure(ctx->buf[B_MODSTATUS], sizeof(uint64_t)));
    auto grow = [&](qd_dbuf &b, size_t bytes) { return keep ? ensure_keep(b, bytes, ctx->stream) : ensure(b, bytes); };
    QD_TRY(grow(out->objects, ap.bytes_cap));
    QD_TRY(grow(out->begin, (NS + 1) * sizeof(uint64_t)));
    QD_TRY(grow(out->size, NS * sizeof(uint32_t)));
    QD_TRY(grow(out->mag, NS * sizeof(double2)));
    QD_TRY(grow(out->d_total, sizeof(double)));
    QD_TRY(grow(out->meta, 2 * sizeof(uint64_t)));
    return QUIDS_OK;
}

// One planned rule step from `in` into `out` (src/quids.hpp:448-543 as
// simulate_rule runs it, with the plan's bounds in place of the host
// waits).  in_meta: the input state's device size words (null for the run's
// input, whose size n_host is known on the host).  rec: the step's report
// words in mapped host memory.
template <class Rule, class Post = no_post>
int simulate_planned(quids_gpu_ctx *ctx, quids_gpu_state *in, const uint64_t *in_meta, uint64_t n_host,
                     const Rule &rule_, quids_gpu_state *out, const quids_gpu_params &prm, const app_plan &ap,
                     uint32_t app, uint64_t *rec, const Post &post = Post{}) {
    const single_rule<Rule> rule{rule_};
    const trunc_key tk{prm.simple_truncation == 0, prm.seed};
    const uint64_t maxn = prm.max_num_object;
    const double load = eff_load(ctx, prm);
    const bool fast = (prm.flags & QUIDS_FLAG_NO_FAST_HASH) == 0;
    QD_TRY(ensure_planned(ctx, out, ap, load, true));  // nothing grows here: the run ensured every step first
    const uint64_t N = ap.n_cap, NC = ap.nc_cap, NSB = ap.ns_cap;
    const uint64_t Mb = std::max<uint64_t>((uint64_t)((double)NC / load) + 1, 1024);
    uint64_t *words = ctx->d_words;
    int *err = (int *)(words + W_STATUS);
    out->n_inst = 0;
    out->h_inst_begin.clear();

    // ---- stage 0: step words, num_child, child offsets (+ the symbolic tile map)
    const uint64_t nzero0 = lookback_words(N);
    k_plan_begin<<<(unsigned)std::min<uint64_t>((nzero0 + 255) / 256 + 1, (uint64_t)ctx->num_sms * 4), 256, 0,
                   ctx->stream>>>(words, app, n_host, in_meta, N, maxn, bufp<int>(ctx, B_MODSTATUS),
                                  bufp<uint64_t>(ctx, B_LOOKBACK), nzero0);
    k_num_child<<<grid_for(ctx, N), prim::kThreads, 0, ctx->stream>>>(
        rule, (const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p, N,
        bufp<uint32_t>(ctx, B_NCHILD), (unsigned long long *)(words + W_MAXSIZE), err, words + W_N);
    QD_TRY(launched(ctx, 2));
    const uint64_t sym_tiles = sym_tiles_of(NC);
    {
        prim::lookback lb;
        lookback_view(ctx, N, 1, lb);
        scan_nchild f{bufp<uint32_t>(ctx, B_NCHILD), nullptr};
        const plan_sizes_hook hook{words, app, ap.nc_cap, ap.maxsize_lim, ap.may_truncate ? ~0ull : maxn, load,
                                   ap.partition ? nullptr : bufp<unsigned long long>(ctx, B_ACC)};
        prim::k_scan_excl<<<lookback_grid(ctx, N), prim::kThreads, 0, ctx->stream>>>(
            f, words + W_NP, bufp<uint64_t>(ctx, B_CBEGIN), words + W_NC, lb,
            tile_parents_epilogue{bufp<uint64_t>(ctx, B_TILEPAR), sym_tiles + 2}, hook_counter(ctx, W_DONE_SCAN),
            hook);
    }
    QD_TRY(launched(ctx));
    parents_view pv{(const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p,
                    (const double2 *)in->mag.p, bufp<uint64_t>(ctx, B_CBEGIN), nullptr, N, words + W_NP};

    // the collision table, sized on the device, and its fill
    const uint64_t tiles_nc = (NC + prim::kTile - 1) / prim::kTile;
    prim::table tb{bufp<prim::table_slot>(ctx, B_KEYS), bufp<unsigned long long>(ctx, B_ACC), Mb, probe_limit(prm),
                   words + W_M};
    fill_set ftab{};
    if (!ap.partition) {
        ftab.p[0] = (unsigned char *)tb.slots, ftab.n[0] = (Mb + 1) * sizeof(prim::table_slot), ftab.v[0] = 0xff;
        ftab.dn[0] = words + W_M, ftab.mul[0] = sizeof(prim::table_slot), ftab.add[0] = sizeof(prim::table_slot);
        ftab.p[1] = bufp<unsigned char>(ctx, B_NOTREP), ftab.n[1] = NC, ftab.v[1] = 0;
        ftab.dn[1] = words + W_NC, ftab.mul[1] = 1, ftab.add[1] = 0;
        ftab.p[2] = bufp<unsigned char>(ctx, B_HASJOIN), ftab.n[2] = NC, ftab.v[2] = 0;
        ftab.dn[2] = words + W_NC, ftab.mul[2] = 1, ftab.add[2] = 0;
        ftab.p[3] = bufp<unsigned char>(ctx, B_LOOKBACK), ftab.n[3] = 4 * (tiles_nc + 2) * sizeof(uint64_t);
        ftab.v[3] = 0;
        ftab.count = 4;
    }

    // ---- stage 1: symbolic iteration (the grouped pass claims the table slots as well)
    bool grouped = false;
    if constexpr (has_grouped<Rule>::value) grouped = fast;
    const bool fused = grouped && !ap.partition;
    if constexpr (has_grouped<Rule>::value) {
        if (fused)
            QD_TRY(launch_symbolic_grouped(ctx, rule, pv, NC, table_claim{tb, bufp<uint32_t>(ctx, B_SLOT), err},
                                           [&] { return fill(ctx, ftab); }));
        else if (grouped)
            QD_TRY(launch_symbolic_grouped(ctx, rule, pv, NC));
    }
    if (!grouped) {
        if (ap.maxsize_lim <= 256) {
            QD_TRY((launch_symbolic<single_rule<Rule>, 256>(ctx, rule, pv, NC, fast)));
        } else {
            QD_TRY((launch_symbolic<single_rule<Rule>, 4096>(ctx, rule, pv, NC, fast)));
        }
    }

    const uint32_t align = prm.align_byte_length;
    unsigned long long *d_maxnorm = (unsigned long long *)(words + W_MAXNORM);
    const plan_end_hook end_hook{words, app, ap.bytes_cap, ap.may_truncate, (uint64_t *)out->meta.p, rec};
    if (ap.partition) {
        // ---- stages 2-4 by partition, counts on the device
        QD_TRY(pcs_stage(ctx, NC, ap.may_truncate, maxn, tk, prm.tolerance, align, out,
                         hook_counter(ctx, W_DONE_LAYOUT), end_hook));
    } else {
        // ---- stage 2: collision table, sized on the device
        if (!fused) QD_TRY(fill(ctx, ftab));
        uint8_t *not_rep = bufp<uint8_t>(ctx, B_NOTREP), *has_join = bufp<uint8_t>(ctx, B_HASJOIN);
        const unsigned long long *d_maxabs = (const unsigned long long *)(words + W_MAXABS);
        {
            direct_src src{bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG)};
            if (!fused) {
                prim::k_table_claim<<<grid_for(ctx, NC), ctx->tune.table_block, 0, ctx->stream>>>(
                    tb, src, words + W_NC, bufp<uint32_t>(ctx, B_SLOT), err);
                QD_TRY(launched(ctx));
            }
            prim::k_table_accumulate<<<grid_for(ctx, NC), ctx->tune.table_block, 0, ctx->stream>>>(
                tb, src, bufp<uint32_t>(ctx, B_SLOT), words + W_NC, d_maxabs, not_rep, has_join);
            QD_TRY(launched(ctx));
        }

        // ---- stages 3-4: groups above tolerance, truncation, output layout
        group_view gv{bufp<uint32_t>(ctx, B_SLOT), not_rep, has_join, bufp<double2>(ctx, B_CMAG),
                      bufp<unsigned long long>(ctx, B_ACC), words + W_NC, d_maxabs, prm.tolerance};
        if (!ap.may_truncate) {
            prim::lookback lbc, lbb;
            lookback_view(ctx, NC, 0, lbc);
            lookback_view(ctx, NC, 1, lbb);
            groups_layout f{gv, bufp<uint32_t>(ctx, B_CSIZE), align, (double2 *)out->mag.p, (uint32_t *)out->size.p,
                            (uint64_t *)out->begin.p, bufp<uint64_t>(ctx, B_SCHILD)};
            prim::k_compact_layout<groups_layout, false><<<lookback_grid(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
                f, words + W_NC, words + W_NS, words + W_OUTBYTES, (uint64_t *)out->begin.p, d_maxnorm, lbc, lbb, lbb,
                hook_counter(ctx, W_DONE_LAYOUT), end_hook);
            QD_TRY(launched(ctx));
        } else {
            uint64_t *gkey = bufp<uint64_t>(ctx, B_UNORM);  // per child: its group's truncation key, or 0
            k_group_keys<<<grid_for(ctx, NC), prim::kThreads, 0, ctx->stream>>>(gv, tk, words + W_NC, gkey,
                                                                               (unsigned long long *)(words + W_NU));
            QD_TRY(launched(ctx));
            QD_TRY(radix_select_filtered(ctx, words + W_NC, NC, maxn, key_direct{gkey}, bufp<uint64_t>(ctx, B_SELCAND),
                                         filter_cap(NC), words + W_NU));
            prim::lookback lbc, lbb, lbt;
            lookback_view(ctx, NC, 0, lbt);
            lookback_view(ctx, NC, 1, lbc);
            lookback_view(ctx, NC, 2, lbb);
            QD_TRY(list_keep_candidates(ctx, keep_candidate{gkey, ctx->d_sel}, NC));
            const cand_keep_layout kl{{gv, gkey, ctx->d_sel, bufp<uint32_t>(ctx, B_CSIZE), align, (double2 *)out->mag.p,
                                       (uint32_t *)out->size.p, (uint64_t *)out->begin.p, bufp<uint64_t>(ctx, B_SCHILD)},
                                      bufp<uint32_t>(ctx, B_KEEPCAND)};
            prim::k_compact_layout<cand_keep_layout, true, plan_end_hook><<<lookback_grid(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
                kl, words + W_NCAND, words + W_NS, words + W_OUTBYTES, (uint64_t *)out->begin.p, d_maxnorm, lbc, lbb, lbt,
                hook_counter(ctx, W_DONE_LAYOUT), end_hook);
            QD_TRY(launched(ctx));
        }
    }

    // ---- stage 5: exact total probability, into the output state
    prim::k_fix_total<<<grid_for(ctx, NSB, 4), prim::kThreads, 0, ctx->stream>>>(
        (const double2 *)out->mag.p, words + W_NS, d_maxnorm, (unsigned long long *)(words + W_ACC),
        (unsigned int *)(words + W_DONE), (double *)(words + W_TOTAL), (double *)(words + W_FACTOR),
        (double *)out->d_total.p, words + W_STATUS);
    QD_TRY(launched(ctx));

    // ---- stage 6: finalize populate + normalisation (+ the fused modifiers)
    QD_TRY((launch_populate<single_rule<Rule>, Post>(ctx, rule, pv, NSB, out, post, ap.maxsize)));
    out->total_pending = true;
    return QUIDS_OK;
}

// A modifier inside a planned run: the state's size from its device words
// (or n_host for the run's input); nothing once the run has stopped.
template <class Mod>
int apply_modifier_planned(quids_gpu_ctx *ctx, quids_gpu_state *st, const uint64_t *meta, uint64_t n_host,
                           uint64_t n_cap, const Mod &mod) {
    QD_TRY(ensure(ctx->buf[B_MODSTATUS], sizeof(uint64_t)));
    k_modifier<Mod><<<grid_for(ctx, n_cap), prim::kThreads, 0, ctx->stream>>>(
        mod, (char *)st->objects.p, (const uint64_t *)st->begin.p, (const uint32_t *)st->size.p, (double2 *)st->mag.p,
        n_host, bufp<int>(ctx, B_MODSTATUS), meta, ctx->d_words + W_STATUS);
    return launched(ctx);
}

// A planned run captured as a CUDA graph (the launch knobs are ctx->tune).
template <class Enqueue>
int capture_planned(quids_gpu_ctx *ctx, Enqueue &&enqueue, cudaGraphExec_t *exec, uint64_t *n_launch) {
    const uint64_t l0 = ctx->launches;
    *exec = nullptr;
    g_alloc_frozen = true;
    cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    int rc = e == cudaSuccess ? enqueue() : QUIDS_ERR_CUDA;
    cudaGraph_t g = nullptr;
    if (e == cudaSuccess) {
        const cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &g);
        if (e2 != cudaSuccess && !rc) rc = QUIDS_ERR_CUDA;
    }
    g_alloc_frozen = false;
    *n_launch = ctx->launches - l0;
    ctx->launches = l0;
    if (!rc && g && cudaGraphInstantiate(exec, g, 0) != cudaSuccess) {
        *exec = nullptr;
        rc = QUIDS_ERR_CUDA;
    }
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();  // a failed capture leaves nothing behind
    return rc;
}

// Autotuning (QUIDS_FLAG_AUTOTUNE) of a plan, before its first capture: the
// run is captured and timed (CUDA events on the stream, best of 3, the input
// restored before each) under the default knobs, then one knob at a time
// over its candidates (collision-table load factor, table-pass block size,
// blocks per SM), keeping a value only when it is faster by more than 2 %.
// A timed run that stops (beyond its bounds) does not count.
template <class Ensure, class Enqueue, class Restore>
int autotune_planned(quids_gpu_ctx *ctx, run_plan &p, Ensure &&ensure_all, Enqueue &&enqueue, Restore &&restore,
                     const volatile uint64_t *fin) {
    const float kInf = 3.0e38f;
    uint32_t trials = 0;
    auto trial = [&](const qd_knobs &k) -> float {
        ctx->tune = k;
        ++trials;
        if (ensure_all()) return kInf;
        cudaGraphExec_t ex = nullptr;
        uint64_t nl = 0;
        if (capture_planned(ctx, enqueue, &ex, &nl)) return kInf;
        float best = kInf;
        for (int rep = 0; rep < 3; ++rep) {
            if (restore()) break;
            cudaEventRecord(ctx->ev0, ctx->stream);
            if (cudaGraphLaunch(ex, ctx->stream) != cudaSuccess) break;
            cudaEventRecord(ctx->ev1, ctx->stream);
            if (cudaEventSynchronize(ctx->ev1) != cudaSuccess) break;
            float ms = kInf;
            cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
            if ((uint32_t)fin[0] != 0) {  // the run stopped: not a measurement of this configuration
                best = kInf;
                break;
            }
            best = ms < best ? ms : best;
        }
        cudaGraphExecDestroy(ex);
        cudaGetLastError();
        return best;
    };
    qd_knobs best = p.knobs;
    const double load0 = best.load > 0 ? best.load : prm_load(p.prm);
    const float t0 = trial(best);
    float t_best = t0;
    const double loads[] = {0.3, 0.5, 0.7};
    const unsigned blocks[] = {128, 256, 512};
    const int sms[] = {4, 8, 16};
    for (double v : loads) {
        qd_knobs k = best;
        k.load = v;
        if ((best.load > 0 ? best.load : load0) == v) continue;
        const float t = trial(k);
        if (t < 0.98f * t_best) best = k, t_best = t;
    }
    for (unsigned v : blocks) {
        if (v == best.table_block) continue;
        qd_knobs k = best;
        k.table_block = v;
        const float t = trial(k);
        if (t < 0.98f * t_best) best = k, t_best = t;
    }
    for (int v : sms) {
        if (v == best.per_sm) continue;
        qd_knobs k = best;
        k.per_sm = v;
        const float t = trial(k);
        if (t < 0.98f * t_best) best = k, t_best = t;
    }
    p.knobs = best;
    p.tuned = true;
    ctx->tune = best;
    quids_gpu_tuning &tu = ctx->last_tuning;
    tu.table_load_factor = best.load > 0 ? best.load : load0;
    tu.table_block = best.table_block;
    tu.blocks_per_sm = (uint32_t)best.per_sm;
    tu.ms_default = t0;
    tu.ms_tuned = t_best;
    tu.trials = trials;
    QD_TRY(ensure_all());
    return restore();
}

// The launch of a planned run: the mapped host words its steps report into,
// then a replay of its CUDA graph (same buffers, same input size), or its
// capture once a planned run of it has succeeded (autotuned first with
// QUIDS_FLAG_AUTOTUNE), or its launches on the stream; then the run's one
// host wait.  *fin: the words of k_plan_finish.  ensure_all: every buffer at
// the plan's bounds for the knobs in ctx->tune; backup / restore: a copy of
// the run's input, for the autotuning's repeated runs.
template <class Ensure, class Enqueue, class Backup, class Restore>
int launch_planned(quids_gpu_ctx *ctx, run_plan &p, const quids_gpu_state *a, Ensure &&ensure_all,
                   Enqueue &&enqueue, Backup &&backup, Restore &&restore, const volatile uint64_t **fin) {
    const uint64_t R = p.apps.size();
    const size_t words = R * R_WORDS + 8;
    ctx->tune = p.knobs;
    struct reset_knobs {
        quids_gpu_ctx *c;
        ~reset_knobs() { c->tune = qd_knobs{}; }
    } reset{ctx};
    if (ensure_all()) return kNotRun;
    if (ctx->h_plan_words < words) {
        if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return QUIDS_ERR_CUDA;
        if (ctx->h_plan) cudaFreeHost(ctx->h_plan);
        ctx->h_plan = ctx->h_plan_dev = nullptr;
        ctx->h_plan_words = 0;
        const size_t want = words + words / 2;
        if (cudaHostAlloc((void **)&ctx->h_plan, want * sizeof(uint64_t), cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer((void **)&ctx->h_plan_dev, ctx->h_plan, 0) != cudaSuccess) {
            cudaGetLastError();
            if (ctx->h_plan) cudaFreeHost(ctx->h_plan);
            ctx->h_plan = ctx->h_plan_dev = nullptr;
            return kNotRun;
        }
        ctx->h_plan_words = want;
        g_alloc_epoch.fetch_add(1);  // graphs name the old words
    }
    *fin = ctx->h_plan + R * R_WORDS;
    if (p.exec && !(p.epoch == g_alloc_epoch.load() && p.n0 == a->n && p.bytes0 == a->nbytes)) {
        cudaGraphExecDestroy(p.exec);
        p.exec = nullptr;
    }
    if (!p.exec && p.runs >= 1 && (p.prm.flags & QUIDS_FLAG_AUTOTUNE) && !p.tuned) {
        QD_TRY(backup());
        QD_TRY(autotune_planned(ctx, p, ensure_all, enqueue, restore, *fin));
    }
    bool launched_run = false;
    if (p.exec) {
        QD_CUDA(cudaGraphLaunch(p.exec, ctx->stream));
        ctx->launches += p.graph_launches;
        ++ctx->runs_graph;
        launched_run = true;
    } else if (p.runs >= 1) {  // capture the run once a planned run has succeeded
        uint64_t n_launch = 0;
        const uint64_t epoch = g_alloc_epoch.load();
        if (capture_planned(ctx, enqueue, &p.exec, &n_launch) == QUIDS_OK) {
            p.epoch = epoch;
            p.n0 = a->n;
            p.bytes0 = a->nbytes;
            p.graph_launches = n_launch;
            QD_CUDA(cudaGraphLaunch(p.exec, ctx->stream));
            ctx->launches += n_launch;
            ++ctx->runs_graph;
            launched_run = true;
        }
    }
    if (!launched_run) {
        const int rc = enqueue();
        if (rc) {
            cudaStreamSynchronize(ctx->stream);
            return rc;
        }
    }
    ++ctx->runs_planned;
    QD_CUDA(cudaStreamSynchronize(ctx->stream));  // the run's one host wait
    return QUIDS_OK;
}

// A copy of the arrays of a run's input state in the plan (copy = true), or
// the input restored from it, on the stream.  Batched states add the
// instance ids and offsets.
inline int backup_input(quids_gpu_ctx *ctx, run_plan &p, quids_gpu_state *a, bool copy) {
    qd_dbuf *src[6] = {&a->objects, &a->begin, &a->size, &a->mag, &a->inst, &a->inst_begin};
    const size_t bytes[6] = {a->nbytes, (a->n + 1) * sizeof(uint64_t), a->n * sizeof(uint32_t), a->n * sizeof(double2),
                             a->n_inst ? a->n * sizeof(uint32_t) : 0,
                             a->n_inst ? ((size_t)a->n_inst + 1) * sizeof(uint64_t) : 0};
    for (int k = 0; k < 6; ++k) {
        if (!bytes[k]) continue;
        if (copy) QD_TRY(ensure(p.backup[k], bytes[k], false));
        void *dst = copy ? p.backup[k].p : src[k]->p;
        const void *from = copy ? src[k]->p : p.backup[k].p;
        QD_CUDA(cudaMemcpyAsync(dst, from, bytes[k], cudaMemcpyDeviceToDevice, ctx->stream));
    }
    return QUIDS_OK;
}

// The counters of the first `done` rule steps of a planned run from its
// report words (in_bytes: the run's input bytes).
inline void read_stats(const quids_gpu_ctx *ctx, uint64_t R, uint64_t done, uint64_t in_bytes, bool batched,
                       quids_gpu_step_stats *st) {
    const double per_n = batched ? 28.0 : 24.0, per_c = batched ? 76.0 : 72.0;
    for (uint64_t r = 0; r < done && r < R; ++r) {
        const volatile uint64_t *rec = ctx->h_plan + r * R_WORDS;
        quids_gpu_step_stats s{};
        s.num_parents = s.num_parents_kept = rec[R_N];
        s.num_object = rec[R_NC];
        s.num_object_after_interferences = rec[R_NU];
        s.num_object_out = rec[R_NS];
        s.out_bytes = rec[R_BYTES];
        s.max_child_size = rec[R_MAXSIZE];
        s.table_capacity = s.num_object ? rec[R_M] : 0;
        s.total_proba = std::numeric_limits<double>::quiet_NaN();
        const double N = (double)s.num_parents, NS = (double)s.num_object_out;
        const double sbar_p = N ? (double)in_bytes / N : 0, sbar_c = NS ? (double)s.out_bytes / NS : 0;
        s.algorithmic_bytes = (double)in_bytes + per_n * N + per_c * (double)s.num_object +
                              per_n * (double)s.num_object_after_interferences + NS * (sbar_p + sbar_c + per_n);
        in_bytes = s.out_bytes;
        st[r] = s;
    }
}

}  // namespace qd::planned
