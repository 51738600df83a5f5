// batch.cu -- the extern "C" entry points of the batched form
// (include/quids_gpu.h, "batched form").
#include <cstring>
#include <utility>
#include <vector>

#include "batch.cuh"
#include "factories.cuh"

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
    if (a->n_inst == 0) return QUIDS_ERR_BAD_ARG;
    const uint32_t G = a->n_inst;
    quids_gpu_state *cur = a, *other = b;
    std::vector<quids_gpu_rule_params> same;
    uint64_t r = 0;
    for (uint64_t i = 0; i < n_ops; ++i) {
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
            rc = quids_gpu_simulate_batched(ctx, cur, op.kind, rp, other, params, nullptr,
                                            rule_stats ? rule_stats + r : nullptr);
            ++r;
            if (!rc) std::swap(cur, other);
        } else {
            rc = quids_gpu_apply_modifier(ctx, cur, op.kind, &op.params);
        }
        if (rc) {
            *final_index = cur == a ? 0 : 1;
            return rc;
        }
    }
    *final_index = cur == a ? 0 : 1;
    return QUIDS_OK;
}

}  // extern "C"
