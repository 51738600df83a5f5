// adjoint.cu -- the tape (a forward run of rule and modifier ops with
// checkpoints) and simulate_backward, the extern "C" entry points of the
// adjoint (include/quids_gpu.h, "adjoint").
//
// Checkpointing: the ops are cut into segments of `checkpoint_every` rule
// applications.  The forward keeps the state at the start of every segment
// and, for the last segment, the input state and the structure record
// (adjoint.cuh) of each rule step.  The backward walks the segments from the
// last: it recomputes a segment's rule steps from its checkpoint, keeping
// their inputs and records (the last segment's come from the forward), then
// goes through the segment's ops in reverse, running the adjoint kernels of
// each rule step on its input and record.  Modifiers supported by the
// backward permute bytes without touching magnitudes (X, CNOT, QCGD step /
// reversed_step), so the adjoint passes through them.
#include <cstring>
#include <new>
#include <utility>
#include <vector>

#include "adjoint.cuh"
#include "factories.cuh"

using namespace qd;
using namespace qd::engine;

struct quids_gpu_tape {
    quids_gpu_ctx *ctx = nullptr;
    std::vector<quids_gpu_op> ops;
    quids_gpu_params prm{};
    uint64_t every = 1;
    std::vector<uint64_t> seg_begin;             // first op of each segment (plus n_ops at the end)
    std::vector<quids_gpu_state *> ckpt;         // state before seg_begin[k] (null for the last segment)
    std::vector<quids_gpu_state *> last_inputs;  // [n_ops] rule inputs of the last segment
    std::vector<qd::adjoint::step_record> last_records;  // [n_ops] their structure records
    quids_gpu_state *final = nullptr;
    bool ready = false;
    qd::adjoint::scratch sc;
    qd_dbuf a0, a1, grads;
};

namespace {

int new_state(quids_gpu_ctx *ctx, quids_gpu_state **out) { return quids_gpu_state_create(ctx, out); }

void drop(quids_gpu_state *&st) {
    if (st) quids_gpu_state_destroy(st);
    st = nullptr;
}

int copy_state(quids_gpu_ctx *ctx, const quids_gpu_state *src, quids_gpu_state *dst) {
    QD_TRY(ensure_state(dst, src->n, src->nbytes));
    cudaStream_t s = ctx->stream;
    if (src->nbytes) QD_CUDA(cudaMemcpyAsync(dst->objects.p, src->objects.p, src->nbytes, cudaMemcpyDeviceToDevice, s));
    QD_CUDA(cudaMemcpyAsync(dst->begin.p, src->begin.p, (src->n + 1) * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
    if (src->n) {
        QD_CUDA(cudaMemcpyAsync(dst->size.p, src->size.p, src->n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
        QD_CUDA(cudaMemcpyAsync(dst->mag.p, src->mag.p, src->n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    }
    if (src->total_pending)
        QD_CUDA(cudaMemcpyAsync(dst->d_total.p, src->d_total.p, sizeof(double), cudaMemcpyDeviceToDevice, s));
    dst->n = src->n;
    dst->nbytes = src->nbytes;
    dst->total_proba = src->total_proba;
    dst->total_pending = src->total_pending;
    dst->n_inst = 0;
    dst->h_inst_begin.clear();
    return QUIDS_OK;
}

void clear_tape(quids_gpu_tape *t) {
    for (auto *&s : t->ckpt) drop(s);
    for (auto *&s : t->last_inputs) drop(s);
    for (auto &r : t->last_records) adjoint::release_record(r);
    drop(t->final);
    t->ckpt.clear();
    t->last_inputs.clear();
    t->last_records.clear();
    t->seg_begin.clear();
    t->ready = false;
}

bool backward_modifier(int kind) {
    return kind == QUIDS_MOD_X || kind == QUIDS_MOD_CNOT || kind == QUIDS_MOD_QCGD_STEP ||
           kind == QUIDS_MOD_QCGD_REVERSED_STEP;
}

// one rule op from `cur` into a new state
int forward_rule(quids_gpu_tape *t, const quids_gpu_op &op, quids_gpu_state *cur, quids_gpu_state **out,
                 quids_gpu_step_stats *stats) {
    QD_TRY(new_state(t->ctx, out));
    quids_gpu_params prm = t->prm;
    prm.flags |= QUIDS_FLAG_TABLE;  // the step records read the table's slots
    prm.hash_ranges = 0;  // the step records are those of one pass
    const int rc = host::dispatch_rule(op.kind, &op.params, [&](auto r) {
        return simulate_rule(t->ctx, cur, r, *out, prm, stats);
    });
    return rc == kNeedRanges ? QUIDS_ERR_UNSUPPORTED : rc;
}

// the rule inputs and records of segment k, recomputed from its checkpoint;
// *last_out: the output of the segment's last rule step (its record points
// at it)
int recompute_segment(quids_gpu_tape *t, size_t k, std::vector<quids_gpu_state *> &inputs,
                      std::vector<adjoint::step_record> &records, quids_gpu_state **last_out) {
    quids_gpu_state *cur = nullptr;
    QD_TRY(new_state(t->ctx, &cur));
    int rc = copy_state(t->ctx, t->ckpt[k], cur);
    for (uint64_t i = t->seg_begin[k]; !rc && i < t->seg_begin[k + 1]; ++i) {
        const quids_gpu_op &op = t->ops[i];
        if (op.is_rule) {
            quids_gpu_state *out = nullptr;
            quids_gpu_step_stats st{};
            rc = forward_rule(t, op, cur, &out, &st);
            if (!rc) rc = adjoint::capture_record(t->ctx, st, cur, out, records[i]);
            if (rc) {
                drop(out);
                break;
            }
            inputs[i] = cur;
            cur = out;
        } else {
            rc = quids_gpu_apply_modifier(t->ctx, cur, op.kind, &op.params);
        }
    }
    *last_out = cur;
    return rc;
}

}  // namespace

extern "C" {

int quids_gpu_tape_create(quids_gpu_ctx *ctx, quids_gpu_tape **out) {
    if (!ctx || !out) return QUIDS_ERR_BAD_ARG;
    auto *t = new (std::nothrow) quids_gpu_tape();
    if (!t) return QUIDS_ERR_OOM;
    t->ctx = ctx;
    *out = t;
    return QUIDS_OK;
}

int quids_gpu_tape_destroy(quids_gpu_tape *t) {
    if (!t) return QUIDS_ERR_BAD_ARG;
    clear_tape(t);
    release(t->sc.surv);
    release(t->sc.partial);
    release(t->a0);
    release(t->a1);
    release(t->grads);
    delete t;
    return QUIDS_OK;
}

int quids_gpu_forward(quids_gpu_ctx *ctx, quids_gpu_tape *t, quids_gpu_state *initial, const quids_gpu_op *ops,
                      uint64_t n_ops, const quids_gpu_params *params, uint64_t checkpoint_every,
                      quids_gpu_state *final_out, quids_gpu_step_stats *rule_stats) {
    if (!ctx || !t || t->ctx != ctx || !initial || initial->ctx != ctx || (!ops && n_ops) || !params ||
        checkpoint_every == 0)
        return QUIDS_ERR_BAD_ARG;
    if (final_out && (final_out->ctx != ctx || final_out == initial)) return QUIDS_ERR_BAD_ARG;
    if (params->max_num_object == 0 || initial->n_inst) return QUIDS_ERR_UNSUPPORTED;
    for (uint64_t i = 0; i < n_ops; ++i)
        if (!ops[i].is_rule && !backward_modifier(ops[i].kind)) return QUIDS_ERR_UNSUPPORTED;
    QD_CUDA(cudaSetDevice(ctx->device));
    const alloc_limit_scope alloc_limit(params->max_alloc_bytes);
    clear_tape(t);
    t->ops.assign(ops, ops + n_ops);
    t->prm = *params;
    t->every = checkpoint_every;
    // segments of `every` rule applications
    t->seg_begin.push_back(0);
    uint64_t rules = 0;
    for (uint64_t i = 0; i < n_ops; ++i)
        if (ops[i].is_rule && ++rules % checkpoint_every == 0 && i + 1 < n_ops) t->seg_begin.push_back(i + 1);
    t->seg_begin.push_back(n_ops);
    const size_t nseg = t->seg_begin.size() - 1;
    t->ckpt.assign(nseg, nullptr);
    t->last_inputs.assign(n_ops, nullptr);
    t->last_records.assign(n_ops, adjoint::step_record{});

    quids_gpu_state *cur = nullptr;
    QD_TRY(new_state(ctx, &cur));
    int rc = copy_state(ctx, initial, cur);
    size_t k = 0;
    uint64_t r = 0;
    for (uint64_t i = 0; !rc && i < n_ops; ++i) {
        if (k + 1 < nseg && i == t->seg_begin[k + 1]) ++k;
        if (i == t->seg_begin[k] && k + 1 < nseg) {  // checkpoint (the last segment keeps its inputs instead)
            rc = new_state(ctx, &t->ckpt[k]);
            if (!rc) rc = copy_state(ctx, cur, t->ckpt[k]);
            if (rc) break;
        }
        const quids_gpu_op &op = ops[i];
        if (op.is_rule) {
            quids_gpu_state *out = nullptr;
            quids_gpu_step_stats st{};
            rc = forward_rule(t, op, cur, &out, &st);
            if (rule_stats) rule_stats[r] = st;
            ++r;
            if (!rc && k + 1 == nseg) rc = adjoint::capture_record(ctx, st, cur, out, t->last_records[i]);
            if (rc) {
                drop(out);
                break;
            }
            if (k + 1 == nseg) {
                t->last_inputs[i] = cur;
            } else {
                drop(cur);
            }
            cur = out;
        } else {
            rc = quids_gpu_apply_modifier(ctx, cur, op.kind, &op.params);
        }
    }
    if (rc) {
        drop(cur);
        clear_tape(t);
        return rc;
    }
    t->final = cur;
    if (final_out) QD_TRY(copy_state(ctx, cur, final_out));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    t->ready = true;
    return QUIDS_OK;
}

int quids_gpu_tape_final_state(quids_gpu_tape *t, quids_gpu_state *out) {
    if (!t || !t->ready || !out || out->ctx != t->ctx) return QUIDS_ERR_BAD_ARG;
    QD_CUDA(cudaSetDevice(t->ctx->device));
    QD_TRY(after_download(out));
    QD_TRY(copy_state(t->ctx, t->final, out));
    return cuda_status(cudaStreamSynchronize(t->ctx->stream));
}

}  // extern "C"

namespace {

// the backward pass from the adjoint of the final state (in t->a0)
int backward_from(quids_gpu_tape *t, double *grad_angles) {
    quids_gpu_ctx *ctx = t->ctx;
    const uint64_t n_ops = t->ops.size();
    QD_TRY(ensure(t->grads, (n_ops * 3 + 3) * sizeof(double)));
    QD_CUDA(cudaMemsetAsync(t->grads.p, 0, (n_ops * 3 + 3) * sizeof(double), ctx->stream));
    double *grads = (double *)t->grads.p;
    const size_t nseg = t->seg_begin.size() - 1;
    int rc = QUIDS_OK;
    for (size_t k = nseg; k-- > 0 && !rc;) {
        const bool last = k + 1 == nseg;
        std::vector<quids_gpu_state *> inputs(n_ops, nullptr);
        std::vector<adjoint::step_record> records;
        quids_gpu_state *seg_out = nullptr;
        if (!last) {
            records.assign(n_ops, adjoint::step_record{});
            rc = recompute_segment(t, k, inputs, records, &seg_out);
        }
        const std::vector<quids_gpu_state *> &in_of = last ? t->last_inputs : inputs;
        const std::vector<adjoint::step_record> &rec_of = last ? t->last_records : records;
        for (uint64_t i = t->seg_begin[k + 1]; !rc && i-- > t->seg_begin[k];) {
            const quids_gpu_op &op = t->ops[i];
            if (!op.is_rule) continue;  // magnitude-preserving permutation of the bytes
            quids_gpu_state *in = in_of[i];
            rc = ensure(t->a1, (in->n ? in->n : 1) * sizeof(double2));
            if (rc) break;
            rc = host::dispatch_rule(op.kind, &op.params, [&](auto r) {
                const adjoint::rule_angles ang{op.params.theta, op.params.phi, op.params.xi};
                return adjoint::backward_rule(ctx, t->sc, in, r, ang, rec_of[i], (double2 *)t->a0.p,
                                              (double2 *)t->a1.p, grads + 3 * i);
            });
            std::swap(t->a0, t->a1);
        }
        if (!last) {
            for (auto *&s : inputs) drop(s);
            for (auto &r : records) adjoint::release_record(r);
            drop(seg_out);
        }
    }
    if (rc) return rc;
    QD_CUDA(cudaMemcpyAsync(grad_angles, grads, n_ops * 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

template <class F>
int with_observable(int kind, const quids_gpu_rule_params *p, F &&f) {
    switch (kind) {
    case QUIDS_OBS_QCGD_NUM_NODES: return f(qcgd::obs_num_nodes{false});
    case QUIDS_OBS_QCGD_NUM_NODES_SQ: return f(qcgd::obs_num_nodes{true});
    case QUIDS_OBS_QCGD_DENSITY: return f(qcgd::obs_density{false});
    case QUIDS_OBS_QCGD_DENSITY_SQ: return f(qcgd::obs_density{true});
    case QUIDS_OBS_QC_BIT:
        if (!p) return QUIDS_ERR_BAD_ARG;
        return f(rules::obs_bit{p->bit});
    }
    return QUIDS_ERR_BAD_ARG;
}

}  // namespace

extern "C" {

int quids_gpu_simulate_backward(quids_gpu_ctx *ctx, quids_gpu_tape *t, const double *loss_adjoint,
                                double *grad_angles) {
    if (!ctx || !t || t->ctx != ctx || !t->ready || !grad_angles || (!loss_adjoint && t->final->n))
        return QUIDS_ERR_BAD_ARG;
    QD_CUDA(cudaSetDevice(ctx->device));
    const alloc_limit_scope alloc_limit(t->prm.max_alloc_bytes);  // the forward's limit
    const uint64_t n = t->final->n;
    QD_TRY(ensure(t->a0, (n ? n : 1) * sizeof(double2)));
    if (n)
        QD_CUDA(cudaMemcpyAsync(t->a0.p, loss_adjoint, n * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
    return backward_from(t, grad_angles);
}

int quids_gpu_simulate_backward_observable(quids_gpu_ctx *ctx, quids_gpu_tape *t, int observable_kind,
                                           const quids_gpu_rule_params *params, double *loss,
                                           double *grad_angles) {
    if (!ctx || !t || t->ctx != ctx || !t->ready || !grad_angles) return QUIDS_ERR_BAD_ARG;
    QD_CUDA(cudaSetDevice(ctx->device));
    const alloc_limit_scope alloc_limit(t->prm.max_alloc_bytes);  // the forward's limit
    const uint64_t n = t->final->n;
    QD_TRY(ensure(t->a0, (n ? n : 1) * sizeof(double2)));
    QD_TRY(ensure(t->grads, (t->ops.size() * 3 + 3) * sizeof(double)));
    double *d_loss = (double *)t->grads.p + t->ops.size() * 3;
    QD_TRY(with_observable(observable_kind, params, [&](auto obs) {
        return adjoint::loss_adjoint(ctx, t->sc, t->final, obs, (double2 *)t->a0.p, d_loss);
    }));
    double l = 0;
    QD_CUDA(cudaMemcpyAsync(&l, d_loss, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    if (loss) *loss = l;
    return backward_from(t, grad_angles);
}

int quids_gpu_observable_adjoint(quids_gpu_ctx *ctx, quids_gpu_state *st, int observable_kind,
                                 const quids_gpu_rule_params *params, double *value, double *adjoint) {
    if (!ctx || !st || st->ctx != ctx || !value) return QUIDS_ERR_BAD_ARG;
    QD_CUDA(cudaSetDevice(ctx->device));
    qd::adjoint::scratch sc;
    qd_dbuf a, d;
    int rc = ensure(a, (st->n ? st->n : 1) * sizeof(double2));
    if (!rc) rc = ensure(d, sizeof(double));
    if (!rc)
        rc = with_observable(observable_kind, params, [&](auto obs) {
            return adjoint::loss_adjoint(ctx, sc, st, obs, (double2 *)a.p, (double *)d.p);
        });
    if (!rc) rc = cuda_status(cudaMemcpyAsync(value, d.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (!rc && adjoint && st->n)
        rc = cuda_status(cudaMemcpyAsync(adjoint, a.p, st->n * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
    if (!rc) rc = cuda_status(cudaStreamSynchronize(ctx->stream));
    release(a);
    release(d);
    release(sc.partial);
    release(sc.surv);
    return rc;
}

}  // extern "C"
