// batch.cu -- the extern "C" entry points of the batched form
// (include/quids_gpu.h, "batched form").
#include <cstring>
#include <limits>
#include <new>
#include <utility>
#include <vector>

#include "batch.cuh"
#include "factories.cuh"
#include "planned_batch.cuh"

using namespace qd;
using namespace qd::engine;

namespace {

template <class Make>
int simulate_batched_with(quids_gpu_ctx *ctx, quids_gpu_state *in, const quids_gpu_rule_params *rules,
                          quids_gpu_state *out, const quids_gpu_params &prm, uint64_t *inst_stats,
                          quids_gpu_step_stats *stats, Make make) {
    using Rule = decltype(make(rules));
    std::vector<Rule> host(in->n_inst);
    for (uint32_t g = 0; g < in->n_inst; ++g) host[g] = make(rules + g);
    return batch::simulate_batched(ctx, in, host.data(), out, prm, inst_stats, stats);
}

// f(make) with make(p) forming the device rule of `kind` from its parameters
template <class F>
int with_rule_maker(int kind, F &&f) {
    switch (kind) {
    case QUIDS_RULE_HADAMARD: return f([](const quids_gpu_rule_params *p) { return host::make_hadamard(p); });
    case QUIDS_RULE_QCGD_ERASE_CREATE:
        return f([](const quids_gpu_rule_params *p) { return qcgd::erase_create{host::make_factors(p)}; });
    case QUIDS_RULE_QCGD_COIN: return f([](const quids_gpu_rule_params *p) { return qcgd::coin{host::make_factors(p)}; });
    case QUIDS_RULE_QCGD_SPLIT_MERGE:
        return f([](const quids_gpu_rule_params *p) { return qcgd::split_merge{host::make_factors(p)}; });
    }
    return QUIDS_ERR_BAD_ARG;
}

// ------------------------------------------------------ planned batched runs
// As quids_gpu_run's planned runs (capi.cu, planned.cuh): the first run of an
// op list records each rule step's counts, the next ones run from those
// bounds without host synchronisations, and from the third on the run is a
// replayed CUDA graph.
using planned::app_plan;
using planned::run_plan;
constexpr size_t kMaxPlans = 8;

bool plannable_batched(const quids_gpu_params &prm) {
    return prm.max_num_object != 0 &&
           !(prm.flags & (QUIDS_FLAG_STAGE_TIMING | QUIDS_FLAG_NO_PLAN));
}

// the rule parameters of rule step r of instance g
const quids_gpu_rule_params *params_of(const run_plan &p, const quids_gpu_op &op, uint64_t r, uint32_t g) {
    return p.inst_params.empty() ? &op.params : &p.inst_params[r * p.n_inst + g];
}

// bounds from a synchronous run: the batched step always selects per
// instance, and is planned only when no instance needed a parent pre-truncation
bool make_plan_batched(run_plan &p, const quids_gpu_step_stats *st, uint64_t n_rules, const quids_gpu_params &prm,
                       uint32_t G) {
    const double load = prm.table_load_factor > 0 && prm.table_load_factor < 0.95 ? prm.table_load_factor : 0.5;
    auto pad = [](uint64_t v) { return v + v / 16 + 64; };
    p.apps.clear();
    for (uint64_t r = 0; r < n_rules; ++r) {
        const quids_gpu_step_stats &s = st[r];
        if (s.num_parents_kept != s.num_parents) return false;
        app_plan ap;
        ap.n_cap = pad(s.num_parents);
        ap.nc_cap = pad(s.num_object);
        if (ap.nc_cap >= 0xffffffffull || (double)ap.nc_cap / load + 2 >= (double)0x7ffffff0ull) return false;
        ap.may_truncate = true;
        const double all = (double)prm.max_num_object * (double)G;
        ap.ns_cap = all < (double)ap.nc_cap ? prm.max_num_object * (uint64_t)G : ap.nc_cap;
        ap.bytes_cap = pad(s.out_bytes) + 4096;
        ap.maxsize_lim = s.max_child_size <= 256 ? 256 : 4096;
        ap.maxsize = s.max_child_size;
        p.apps.push_back(ap);
    }
    return true;
}

// every rule step's per-instance rules into the plan's device buffer
int upload_rules(quids_gpu_ctx *ctx, run_plan &p) {
    std::vector<uint8_t> bytes;
    p.rule_off.clear();
    uint64_t r = 0;
    for (const quids_gpu_op &op : p.ops) {
        if (!op.is_rule) continue;
        const uint64_t off = (bytes.size() + 15) / 16 * 16;
        p.rule_off.push_back(off);
        QD_TRY(with_rule_maker(op.kind, [&](auto make) {
            using Rule = decltype(make(&op.params));
            bytes.resize(off + (size_t)p.n_inst * sizeof(Rule));
            for (uint32_t g = 0; g < p.n_inst; ++g) {
                const Rule rule = make(params_of(p, op, r, g));
                std::memcpy(bytes.data() + off + g * sizeof(Rule), &rule, sizeof(Rule));
            }
            return QUIDS_OK;
        }));
        ++r;
    }
    QD_TRY(ensure(p.rules, bytes.size(), false));
    // on the context's stream: a plain cudaMemcpy from pageable memory may return before its DMA
    // lands, and the legacy stream does not order the non-blocking stream's kernels after it
    QD_CUDA(cudaMemcpyAsync(p.rules.p, bytes.data(), bytes.size(), cudaMemcpyHostToDevice, ctx->stream));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    p.rules_ready = true;
    return QUIDS_OK;
}

int enqueue_planned_batched(quids_gpu_ctx *ctx, run_plan &p, quids_gpu_state *a, quids_gpu_state *b) {
    const quids_gpu_op *ops = p.ops.data();
    const uint64_t n_ops = p.ops.size(), R = p.apps.size();
    planned::k_plan_start<<<1, 1, 0, ctx->stream>>>(ctx->d_words);
    QD_TRY(launched(ctx));
    quids_gpu_state *cur = a, *other = b;
    const uint64_t *cur_meta = nullptr;
    const uint64_t n0 = a->n;
    uint64_t r = 0;
    for (uint64_t i = 0; i < n_ops; ++i) {
        const quids_gpu_op &op = ops[i];
        if (op.is_rule) {
            uint64_t *rec = ctx->h_plan_dev + r * planned::R_WORDS;
            const uint8_t *rules = (const uint8_t *)p.rules.p + p.rule_off[r];
            QD_TRY(with_rule_maker(op.kind, [&](auto make) {
                using Rule = decltype(make(&op.params));
                return planned::simulate_batched_planned<Rule>(ctx, cur, cur_meta, n0, (const Rule *)rules, other,
                                                               p.prm, p.apps[r], (uint32_t)r, rec);
            }));
            std::swap(cur, other);
            cur_meta = (const uint64_t *)cur->meta.p;
            ++r;
        } else {
            const uint64_t cap = r == 0 ? n0 : p.apps[r - 1].ns_cap;
            int rc = QUIDS_ERR_BAD_ARG;
            const quids_gpu_rule_params *mp = &op.params;
            switch (op.kind) {
            case QUIDS_MOD_CNOT: rc = planned::apply_modifier_planned(ctx, cur, cur_meta, n0, cap, rules::cnot{mp->control, mp->bit}); break;
            case QUIDS_MOD_X: rc = planned::apply_modifier_planned(ctx, cur, cur_meta, n0, cap, rules::xgate{mp->bit}); break;
            case QUIDS_MOD_Y: rc = planned::apply_modifier_planned(ctx, cur, cur_meta, n0, cap, rules::ygate{mp->bit}); break;
            case QUIDS_MOD_Z: rc = planned::apply_modifier_planned(ctx, cur, cur_meta, n0, cap, rules::zgate{mp->bit}); break;
            case QUIDS_MOD_QCGD_STEP: rc = planned::apply_modifier_planned(ctx, cur, cur_meta, n0, cap, qcgd::step{}); break;
            case QUIDS_MOD_QCGD_REVERSED_STEP:
                rc = planned::apply_modifier_planned(ctx, cur, cur_meta, n0, cap, qcgd::reversed_step{});
                break;
            }
            QD_TRY(rc);
        }
    }
    planned::k_plan_finish<<<1, 1, 0, ctx->stream>>>(ctx->d_words, R >= 2 ? (const uint64_t *)a->meta.p : nullptr,
                                                     R >= 1 ? (const uint64_t *)b->meta.p : nullptr,
                                                     ctx->h_plan_dev + R * planned::R_WORDS);
    return launched(ctx);
}

// the host mirror of a batched state written on the device
int set_batched_state(quids_gpu_state *x, uint64_t n, uint64_t nbytes, uint32_t G) {
    x->n = n;
    x->nbytes = nbytes;
    x->n_inst = G;
    x->total_pending = false;
    x->total_proba = std::numeric_limits<double>::quiet_NaN();
    x->h_inst_begin.resize((size_t)G + 1);
    QD_CUDA(cudaMemcpy(x->h_inst_begin.data(), x->inst_begin.p, ((size_t)G + 1) * sizeof(uint64_t),
                       cudaMemcpyDeviceToHost));
    return QUIDS_OK;
}

int run_planned_batched(quids_gpu_ctx *ctx, run_plan &p, quids_gpu_state *a, quids_gpu_state *b,
                        quids_gpu_step_stats *st, uint64_t *fail_app) {
    const uint64_t R = p.apps.size();
    const uint32_t G = p.n_inst;
    if (!p.rules_ready && upload_rules(ctx, p)) return planned::kNotRun;
    auto ensure_all = [&]() -> int {
        if (!ctx->buf[B_MODSTATUS].p) {
            QD_TRY(ensure(ctx->buf[B_MODSTATUS], sizeof(uint64_t)));
            QD_CUDA(cudaMemsetAsync(ctx->buf[B_MODSTATUS].p, 0, sizeof(uint64_t), ctx->stream));
        }
        const double load = planned::eff_load(ctx, p.prm);
        for (uint64_t r = 0; r < R; ++r)
            QD_TRY(planned::ensure_planned_batched(ctx, r % 2 ? a : b, p.apps[r], load, r % 2 == 1, G));
        return QUIDS_OK;
    };
    const volatile uint64_t *fin = nullptr;
    QD_TRY(planned::launch_planned(
        ctx, p, a, ensure_all, [&] { return enqueue_planned_batched(ctx, p, a, b); },
        [&] { return planned::backup_input(ctx, p, a, true); }, [&] { return planned::backup_input(ctx, p, a, false); },
        &fin));
    const int status = (int)(uint32_t)fin[0];
    const uint64_t fa = status ? fin[1] : R;
    planned::read_stats(ctx, R, fa, a->nbytes, true, st);
    const uint64_t na = fin[2], ba = fin[3], nb = fin[4], bb = fin[5];
    if (!status) {
        if (R >= 1) QD_TRY(set_batched_state(b, nb, bb, G));
        if (R >= 2) QD_TRY(set_batched_state(a, na, ba, G));
        ++p.runs;
        return QUIDS_OK;
    }
    quids_gpu_state *in = fa % 2 ? b : a, *out = fa % 2 ? a : b;
    if (fa >= 1) QD_TRY(set_batched_state(in, fa % 2 ? nb : na, fa % 2 ? bb : ba, G));
    out->n = out->nbytes = 0;
    *fail_app = fa;
    return status;
}

// the ops of a batched run from ops[i0] (rule r0) on, synchronously
int run_sync_batched(quids_gpu_ctx *ctx, quids_gpu_state *&cur, quids_gpu_state *&other, const quids_gpu_op *ops,
                     uint64_t n_ops, uint64_t i0, uint64_t r0, const quids_gpu_rule_params *inst_params,
                     const quids_gpu_params &prm, quids_gpu_step_stats *st) {
    const uint32_t G = cur->n_inst;
    std::vector<quids_gpu_rule_params> same;
    uint64_t r = r0;
    for (uint64_t i = i0; i < n_ops; ++i) {
        const quids_gpu_op &op = ops[i];
        int rc;
        if (op.is_rule) {
            const quids_gpu_rule_params *rp;
            if (inst_params) {
                rp = inst_params + r * G;
            } else {
                same.assign(G, op.params);
                rp = same.data();
            }
            rc = quids_gpu_simulate_batched(ctx, cur, op.kind, rp, other, &prm, nullptr, st + r);
            ++r;
            if (!rc) std::swap(cur, other);
        } else {
            rc = quids_gpu_apply_modifier(ctx, cur, op.kind, &op.params);
        }
        if (rc) return rc;
    }
    return QUIDS_OK;
}

}  // namespace

extern "C" {

int quids_gpu_state_upload_batched(quids_gpu_state *st, uint64_t n, const uint8_t *objects, const uint64_t *begin,
                                   const uint32_t *size, const double *magnitude, uint64_t num_bytes,
                                   uint32_t n_inst, const uint64_t *inst_begin) {
    if (!st || !st->ctx || !inst_begin || n_inst == 0 || n_inst > batch::kMaxInstances) return QUIDS_ERR_BAD_ARG;
    if (inst_begin[0] != 0 || inst_begin[n_inst] != n) return QUIDS_ERR_BAD_ARG;
    for (uint32_t g = 0; g < n_inst; ++g)
        if (inst_begin[g + 1] < inst_begin[g]) return QUIDS_ERR_BAD_ARG;
    if (n >= 0xffffffffull) return QUIDS_ERR_UNSUPPORTED;
    QD_TRY(quids_gpu_state_upload(st, n, objects, begin, size, magnitude, num_bytes));
    quids_gpu_ctx *ctx = st->ctx;
    std::vector<uint32_t> inst(n);
    for (uint32_t g = 0; g < n_inst; ++g)
        for (uint64_t j = inst_begin[g]; j < inst_begin[g + 1]; ++j) inst[j] = g;
    std::vector<double> ones(n_inst, 1.0);
    QD_TRY(ensure(st->inst, n * sizeof(uint32_t)));
    QD_TRY(ensure(st->inst_begin, ((size_t)n_inst + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(st->inst_total, (size_t)n_inst * sizeof(double)));
    if (n) QD_CUDA(cudaMemcpyAsync(st->inst.p, inst.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream));
    QD_CUDA(cudaMemcpyAsync(st->inst_begin.p, inst_begin, ((size_t)n_inst + 1) * sizeof(uint64_t),
                            cudaMemcpyHostToDevice, ctx->stream));
    QD_CUDA(cudaMemcpyAsync(st->inst_total.p, ones.data(), (size_t)n_inst * sizeof(double), cudaMemcpyHostToDevice,
                            ctx->stream));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    st->n_inst = n_inst;
    st->h_inst_begin.assign(inst_begin, inst_begin + n_inst + 1);
    return QUIDS_OK;
}

int quids_gpu_state_instances(quids_gpu_state *st, uint32_t *n_inst, uint64_t *inst_begin, double *inst_total) {
    if (!st || !n_inst) return QUIDS_ERR_BAD_ARG;
    *n_inst = st->n_inst;
    if (st->n_inst == 0) return QUIDS_OK;
    if (inst_begin) std::memcpy(inst_begin, st->h_inst_begin.data(), ((size_t)st->n_inst + 1) * sizeof(uint64_t));
    if (inst_total) {
        if (!st->ctx) return QUIDS_ERR_BAD_ARG;
        QD_CUDA(cudaSetDevice(st->ctx->device));
        QD_CUDA(cudaMemcpyAsync(inst_total, st->inst_total.p, (size_t)st->n_inst * sizeof(double),
                                cudaMemcpyDeviceToHost, st->ctx->stream));
        QD_CUDA(cudaStreamSynchronize(st->ctx->stream));
    }
    return QUIDS_OK;
}

int quids_gpu_simulate_batched(quids_gpu_ctx *ctx, quids_gpu_state *iteration, int rule_kind,
                               const quids_gpu_rule_params *rules, quids_gpu_state *next_iteration,
                               const quids_gpu_params *params, uint64_t *inst_stats, quids_gpu_step_stats *stats) {
    if (!ctx || !iteration || !rules || !params) return QUIDS_ERR_BAD_ARG;
    if (iteration->n_inst == 0) return QUIDS_ERR_BAD_ARG;
    const quids_gpu_params prm = *params;
    const alloc_limit_scope alloc_limit(prm.max_alloc_bytes);
    QD_CUDA(cudaSetDevice(ctx->device));
    QD_TRY(after_download(iteration));
    QD_TRY(after_download(next_iteration));
    switch (rule_kind) {
    case QUIDS_RULE_HADAMARD:
        return simulate_batched_with(ctx, iteration, rules, next_iteration, prm, inst_stats, stats,
                                     [](const quids_gpu_rule_params *p) { return host::make_hadamard(p); });
    case QUIDS_RULE_QCGD_ERASE_CREATE:
        return simulate_batched_with(ctx, iteration, rules, next_iteration, prm, inst_stats, stats,
                                     [](const quids_gpu_rule_params *p) {
                                         return qcgd::erase_create{host::make_factors(p)};
                                     });
    case QUIDS_RULE_QCGD_COIN:
        return simulate_batched_with(ctx, iteration, rules, next_iteration, prm, inst_stats, stats,
                                     [](const quids_gpu_rule_params *p) { return qcgd::coin{host::make_factors(p)}; });
    case QUIDS_RULE_QCGD_SPLIT_MERGE:
        return simulate_batched_with(ctx, iteration, rules, next_iteration, prm, inst_stats, stats,
                                     [](const quids_gpu_rule_params *p) {
                                         return qcgd::split_merge{host::make_factors(p)};
                                     });
    }
    return QUIDS_ERR_BAD_ARG;
}

int quids_gpu_run_batched(quids_gpu_ctx *ctx, quids_gpu_state *a, quids_gpu_state *b, const quids_gpu_op *ops,
                          uint64_t n_ops, const quids_gpu_rule_params *inst_params, const quids_gpu_params *params,
                          quids_gpu_step_stats *rule_stats, int *final_index) {
    if (!ctx || !a || !b || a == b || (!ops && n_ops) || !params || !final_index) return QUIDS_ERR_BAD_ARG;
    if (a->n_inst == 0 || a->ctx != ctx || b->ctx != ctx) return QUIDS_ERR_BAD_ARG;
    QD_CUDA(cudaSetDevice(ctx->device));
    QD_TRY(after_download(a));
    QD_TRY(after_download(b));
    const uint32_t G = a->n_inst;
    const quids_gpu_params prm = *params;
    const alloc_limit_scope alloc_limit(prm.max_alloc_bytes);
    uint64_t n_rules = 0;
    for (uint64_t i = 0; i < n_ops; ++i) n_rules += ops[i].is_rule ? 1 : 0;
    std::vector<quids_gpu_step_stats> st(n_rules ? n_rules : 1);
    quids_gpu_state *cur = a, *other = b;
    uint64_t i0 = 0, r0 = 0;
    run_plan *p = n_rules && plannable_batched(prm) ? planned::find_plan(ctx, a, b, ops, n_ops, prm, G, inst_params)
                                                    : nullptr;
    bool replan = false;
    if (p) {
        uint64_t fa = 0;
        const int rc = run_planned_batched(ctx, *p, a, b, st.data(), &fa);
        if (rc == QUIDS_OK) {
            if (rule_stats) std::memcpy(rule_stats, st.data(), n_rules * sizeof(quids_gpu_step_stats));
            *final_index = n_rules % 2 ? 1 : 0;
            return QUIDS_OK;
        }
        if (rc == planned::kNotRun) {
            planned::drop_plan(ctx, p);
            p = nullptr;
        } else if (rc != planned::kReplan) {
            *final_index = fa % 2 ? 1 : 0;
            if (rule_stats) std::memcpy(rule_stats, st.data(), std::min(fa, n_rules) * sizeof(quids_gpu_step_stats));
            return rc;
        } else {
            replan = true;
            for (uint64_t i = 0, r = 0; i < n_ops; ++i) {
                if (!ops[i].is_rule) continue;
                if (r == fa) {
                    i0 = i;
                    break;
                }
                ++r;
            }
            r0 = fa;
            if (fa % 2) std::swap(cur, other);
        }
    }
    ++ctx->runs_sync;
    const int rc = run_sync_batched(ctx, cur, other, ops, n_ops, i0, r0, inst_params, prm, st.data());
    *final_index = cur == a ? 0 : 1;
    if (rule_stats) std::memcpy(rule_stats, st.data(), n_rules * sizeof(quids_gpu_step_stats));
    if (rc) return rc;
    if (n_rules && plannable_batched(prm)) {
        if (!p) {
            p = new (std::nothrow) run_plan();
            if (!p) return QUIDS_OK;
            p->ops.assign(ops, ops + n_ops);
            p->prm = prm;
            p->a = a;
            p->b = b;
            p->n_inst = G;
            if (inst_params) p->inst_params.assign(inst_params, inst_params + n_rules * G);
            ctx->plans.push_back(p);
            if (ctx->plans.size() > kMaxPlans) planned::drop_plan(ctx, ctx->plans.front());
        }
        if (!make_plan_batched(*p, st.data(), n_rules, prm, G)) {
            planned::drop_plan(ctx, p);
        } else if (replan) {
            p->runs = 0;
            if (p->exec) cudaGraphExecDestroy(p->exec);
            p->exec = nullptr;
        }
    }
    return QUIDS_OK;
}

}  // extern "C"
