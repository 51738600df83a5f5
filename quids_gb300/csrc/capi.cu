// capi.cu -- the extern "C" entry points of include/quids_gpu.h.
//
// Built-in rules are instantiated here; the rule and modifier objects are
// formed on the host from quids_gpu_rule_params (factories.cuh).
#include <cmath>
#include <complex>
#include <cstring>
#include <new>
#include <utility>

#include "engine.cuh"
#include "ranges.cuh"
#include "rules_qc.cuh"
#include "rules_qcgd.cuh"
#include "factories.cuh"

using namespace qd;
using namespace qd::engine;
using qd::host::dispatch_rule;

namespace {

// The modifiers that follow a rule in a run, applied to each survivor
// right after its populate (in order, like the separate modifier launches
// they replace).  An object a modifier does not fit sets the sticky modifier
// status, as a separate modifier launch does.
struct mod_chain {
    static constexpr bool active = true;
    static constexpr int kMax = 16;
    int n = 0;
    int32_t kind[kMax];
    uint64_t bit[kMax], control[kMax];
    int *status = nullptr;

    template <class M>
    __device__ static void apply(const M &mod, char *b, char *e, mag_t &m, int *err) {
        if (!object_fits(mod, (uint32_t)(e - b))) {
            prim::set_error(err, QUIDS_ERR_BAD_ARG);
            return;
        }
        mod(b, e, m);
    }
    __device__ void operator()(char *b, char *e, mag_t &m, int *) const {
        int *err = status;
        for (int k = 0; k < n; ++k) {
            switch (kind[k]) {
            case QUIDS_MOD_CNOT: apply(rules::cnot{control[k], bit[k]}, b, e, m, err); break;
            case QUIDS_MOD_X: apply(rules::xgate{bit[k]}, b, e, m, err); break;
            case QUIDS_MOD_Y: apply(rules::ygate{bit[k]}, b, e, m, err); break;
            case QUIDS_MOD_Z: apply(rules::zgate{bit[k]}, b, e, m, err); break;
            case QUIDS_MOD_QCGD_STEP: apply(qcgd::step{}, b, e, m, err); break;
            case QUIDS_MOD_QCGD_REVERSED_STEP: apply(qcgd::reversed_step{}, b, e, m, err); break;
            }
        }
    }
};

bool chainable(int kind) { return kind >= QUIDS_MOD_CNOT && kind <= QUIDS_MOD_QCGD_REVERSED_STEP; }

__global__ void k_set_words_zero(uint64_t *w, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) w[i] = 0;
}

}  // namespace

extern "C" {

const char *quids_gpu_status_string(int s) {
    switch (s) {
    case QUIDS_OK: return "ok";
    case QUIDS_ERR_BAD_ARG: return "bad argument";
    case QUIDS_ERR_OOM: return "device out of memory";
    case QUIDS_ERR_TABLE_FULL: return "collision table full";
    case QUIDS_ERR_CHILD_COUNT_OVERFLOW: return "child count overflow";
    case QUIDS_ERR_SIZE_BOUND: return "child larger than max_child_size bound";
    case QUIDS_ERR_TIMEOUT: return "bounded device wait expired";
    case QUIDS_ERR_CUDA: return "CUDA runtime error";
    case QUIDS_ERR_NO_DEVICE: return "no CUDA device";
    case QUIDS_ERR_UNSUPPORTED: return "unsupported request";
    case QUIDS_ERR_NOALLOC_LIMIT: return "beyond the static scratch of the no-allocation entry point";
    }
    return "unknown status";
}

int quids_gpu_ctx_create(int device, quids_gpu_ctx **out) {
    if (!out) return QUIDS_ERR_BAD_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return QUIDS_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return QUIDS_ERR_BAD_ARG;
    QD_CUDA(cudaSetDevice(device));
    auto *ctx = new (std::nothrow) quids_gpu_ctx();
    if (!ctx) return QUIDS_ERR_OOM;
    ctx->device = device;
    int rc = QUIDS_OK;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) rc = QUIDS_ERR_CUDA;
    if (!rc) ctx->num_sms = prop.multiProcessorCount;
    if (!rc) rc = cuda_status(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    if (!rc) rc = cuda_status(cudaMalloc(&ctx->d_words, W_COUNT_WORDS * sizeof(uint64_t)));
    if (!rc) rc = cuda_status(cudaHostAlloc((void **)&ctx->h_words, (W_COUNT_WORDS + 1) * sizeof(uint64_t),
                                            cudaHostAllocMapped));
    if (!rc) {
        std::memset(ctx->h_words, 0, (W_COUNT_WORDS + 1) * sizeof(uint64_t));
        rc = cuda_status(cudaHostGetDevicePointer((void **)&ctx->h_words_dev, ctx->h_words, 0));
    }
    if (!rc) rc = cuda_status(cudaMalloc(&ctx->d_sel, 2 * sizeof(qd::prim::select_state)));
    if (!rc) rc = cuda_status(cudaMalloc(&ctx->d_hist, qd::prim::kBins * sizeof(unsigned long long)));
    if (!rc) rc = cuda_status(cudaEventCreate(&ctx->ev0));
    if (!rc) rc = cuda_status(cudaEventCreate(&ctx->ev1));
    for (int k = 0; k < 16 && !rc; ++k) rc = cuda_status(cudaEventCreate(&ctx->ev_stage[k]));
    if (!rc) {
        k_set_words_zero<<<1, 32, 0, ctx->stream>>>(ctx->d_words, W_COUNT_WORDS);
        rc = cuda_status(cudaStreamSynchronize(ctx->stream));
    }
    if (rc) {
        quids_gpu_ctx_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return QUIDS_OK;
}

int quids_gpu_ctx_destroy(quids_gpu_ctx *ctx) {
    if (!ctx) return QUIDS_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (quids_gpu_state *st : ctx->states) {
        release_state(st);
        st->ctx = nullptr;
    }
    ctx->states.clear();
    for (auto &b : ctx->buf) release(b);
    if (ctx->d_words) cudaFree(ctx->d_words);
    if (ctx->h_words) cudaFreeHost(ctx->h_words);
    if (ctx->d_sel) cudaFree(ctx->d_sel);
    if (ctx->d_hist) cudaFree(ctx->d_hist);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (auto &e : ctx->ev_stage)
        if (e) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return QUIDS_OK;
}

void *quids_gpu_ctx_stream(quids_gpu_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

uint64_t quids_gpu_ctx_launch_count(quids_gpu_ctx *ctx) { return ctx ? ctx->launches : 0; }

int quids_gpu_ctx_synchronize(quids_gpu_ctx *ctx) {
    if (!ctx) return QUIDS_ERR_BAD_ARG;
    QD_CUDA(cudaSetDevice(ctx->device));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    return QUIDS_OK;
}

uint64_t quids_gpu_ctx_scratch_bytes(quids_gpu_ctx *ctx) {
    if (!ctx) return 0;
    uint64_t t = 0;
    for (auto &b : ctx->buf) t += b.cap;
    return t;
}

int quids_gpu_ctx_trim(quids_gpu_ctx *ctx) {
    if (!ctx) return QUIDS_ERR_BAD_ARG;
    QD_CUDA(cudaSetDevice(ctx->device));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    for (auto &b : ctx->buf) release(b);
    return QUIDS_OK;
}

int quids_gpu_state_create(quids_gpu_ctx *ctx, quids_gpu_state **out) {
    if (!ctx || !out) return QUIDS_ERR_BAD_ARG;
    auto *st = new (std::nothrow) quids_gpu_state();
    if (!st) return QUIDS_ERR_OOM;
    st->ctx = ctx;
    ctx->states.insert(st);
    *out = st;
    return QUIDS_OK;
}

int quids_gpu_state_destroy(quids_gpu_state *st) {
    if (!st) return QUIDS_ERR_BAD_ARG;
    if (!st->ctx) {  // its context is gone and has already released the memory
        delete st;
        return QUIDS_OK;
    }
    cudaSetDevice(st->ctx->device);
    cudaStreamSynchronize(st->ctx->stream);
    st->ctx->states.erase(st);
    release_state(st);
    delete st;
    return QUIDS_OK;
}

int quids_gpu_state_upload(quids_gpu_state *st, uint64_t n, const uint8_t *objects, const uint64_t *begin,
                           const uint32_t *size, const double *magnitude, uint64_t num_bytes) {
    if (!st || !st->ctx) return QUIDS_ERR_BAD_ARG;
    if (n && (!begin || !size || !magnitude)) return QUIDS_ERR_BAD_ARG;
    if (num_bytes && !objects) return QUIDS_ERR_BAD_ARG;
    for (uint64_t i = 0; i < n; ++i)
        if (begin[i] + size[i] > num_bytes) return QUIDS_ERR_BAD_ARG;
    quids_gpu_ctx *ctx = st->ctx;
    QD_CUDA(cudaSetDevice(ctx->device));
    QD_TRY(ensure_state(st, n, num_bytes));
    cudaStream_t s = ctx->stream;
    if (num_bytes) QD_CUDA(cudaMemcpyAsync(st->objects.p, objects, num_bytes, cudaMemcpyHostToDevice, s));
    if (n) {
        QD_CUDA(cudaMemcpyAsync(st->begin.p, begin, (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
        QD_CUDA(cudaMemcpyAsync(st->size.p, size, n * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        QD_CUDA(cudaMemcpyAsync(st->mag.p, magnitude, n * 2 * sizeof(double), cudaMemcpyHostToDevice, s));
    } else {
        QD_CUDA(cudaMemsetAsync(st->begin.p, 0, sizeof(uint64_t), s));
    }
    QD_CUDA(cudaStreamSynchronize(s));
    st->n = n;
    st->nbytes = num_bytes;
    st->total_proba = 1;
    st->total_pending = false;
    st->n_inst = 0;
    st->h_inst_begin.clear();
    return QUIDS_OK;
}

int quids_gpu_state_num_object(const quids_gpu_state *st, uint64_t *n) {
    if (!st || !n) return QUIDS_ERR_BAD_ARG;
    *n = st->n;
    return QUIDS_OK;
}

int quids_gpu_state_num_bytes(const quids_gpu_state *st, uint64_t *nb) {
    if (!st || !nb) return QUIDS_ERR_BAD_ARG;
    *nb = st->nbytes;
    return QUIDS_OK;
}

int quids_gpu_state_total_proba(const quids_gpu_state *st, double *p) {
    if (!st || !p) return QUIDS_ERR_BAD_ARG;
    if (st->total_pending && st->ctx) {  // written on the device by the last step
        QD_CUDA(cudaSetDevice(st->ctx->device));
        double v = 0;
        QD_CUDA(cudaMemcpyAsync(&v, st->d_total.p, sizeof(double), cudaMemcpyDeviceToHost, st->ctx->stream));
        QD_CUDA(cudaStreamSynchronize(st->ctx->stream));
        st->total_proba = v;
        st->total_pending = false;
    }
    *p = st->total_proba;
    return QUIDS_OK;
}

int quids_gpu_state_download(quids_gpu_state *st, uint8_t *objects, uint64_t *begin, uint32_t *size,
                             double *magnitude) {
    if (!st || !st->ctx) return QUIDS_ERR_BAD_ARG;
    quids_gpu_ctx *ctx = st->ctx;
    QD_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    if (objects && st->nbytes)
        QD_CUDA(cudaMemcpyAsync(objects, st->objects.p, st->nbytes, cudaMemcpyDeviceToHost, s));
    if (begin) {
        if (st->n)
            QD_CUDA(cudaMemcpyAsync(begin, st->begin.p, (st->n + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        else
            begin[0] = 0;
    }
    if (size && st->n) QD_CUDA(cudaMemcpyAsync(size, st->size.p, st->n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    if (magnitude && st->n)
        QD_CUDA(cudaMemcpyAsync(magnitude, st->mag.p, st->n * 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    QD_CUDA(cudaStreamSynchronize(s));
    return QUIDS_OK;
}

int quids_gpu_state_device_arrays(quids_gpu_state *st, void **objects, void **begin, void **size, void **magnitude) {
    if (!st) return QUIDS_ERR_BAD_ARG;
    if (objects) *objects = st->objects.p;
    if (begin) *begin = st->begin.p;
    if (size) *size = st->size.p;
    if (magnitude) *magnitude = st->mag.p;
    return QUIDS_OK;
}

int quids_gpu_simulate(quids_gpu_ctx *ctx, quids_gpu_state *iteration, int rule_kind,
                       const quids_gpu_rule_params *rule, quids_gpu_state *next_iteration,
                       const quids_gpu_params *params, quids_gpu_step_stats *stats) {
    if (!params) return QUIDS_ERR_BAD_ARG;
    quids_gpu_params prm = *params;
    return dispatch_rule(rule_kind, rule, [&](auto r) {
        return ranges::simulate_step(ctx, iteration, r, next_iteration, prm, stats);
    });
}

int quids_gpu_apply_modifier(quids_gpu_ctx *ctx, quids_gpu_state *st, int kind, const quids_gpu_rule_params *p) {
    if (!p) return QUIDS_ERR_BAD_ARG;
    switch (kind) {
    case QUIDS_MOD_CNOT: return apply_modifier(ctx, st, rules::cnot{p->control, p->bit});
    case QUIDS_MOD_X: return apply_modifier(ctx, st, rules::xgate{p->bit});
    case QUIDS_MOD_Y: return apply_modifier(ctx, st, rules::ygate{p->bit});
    case QUIDS_MOD_Z: return apply_modifier(ctx, st, rules::zgate{p->bit});
    case QUIDS_MOD_QCGD_STEP: return apply_modifier(ctx, st, qcgd::step{});
    case QUIDS_MOD_QCGD_REVERSED_STEP: return apply_modifier(ctx, st, qcgd::reversed_step{});
    }
    return QUIDS_ERR_BAD_ARG;
}

int quids_gpu_run(quids_gpu_ctx *ctx, quids_gpu_state *a, quids_gpu_state *b, const quids_gpu_op *ops,
                  uint64_t n_ops, const quids_gpu_params *params, quids_gpu_step_stats *rule_stats,
                  int *final_index) {
    if (!ctx || !a || !b || a == b || (!ops && n_ops) || !params || !final_index) return QUIDS_ERR_BAD_ARG;
    quids_gpu_state *cur = a, *other = b;
    uint64_t r = 0;
    const quids_gpu_params prm = *params;
    for (uint64_t i = 0; i < n_ops; ++i) {
        const quids_gpu_op &op = ops[i];
        int rc;
        if (op.is_rule) {
            // the modifiers up to the next rule run inside this rule's populate
            mod_chain chain;
            uint64_t j = i + 1;
            while (j < n_ops && !ops[j].is_rule && chainable(ops[j].kind) && chain.n < mod_chain::kMax) {
                chain.kind[chain.n] = ops[j].kind;
                chain.bit[chain.n] = ops[j].params.bit;
                chain.control[chain.n] = ops[j].params.control;
                ++chain.n;
                ++j;
            }
            if (chain.n) {
                if (!ctx->buf[B_MODSTATUS].p) {
                    QD_TRY(ensure(ctx->buf[B_MODSTATUS], sizeof(uint64_t)));
                    QD_CUDA(cudaMemsetAsync(ctx->buf[B_MODSTATUS].p, 0, sizeof(uint64_t), ctx->stream));
                }
                chain.status = bufp<int>(ctx, B_MODSTATUS);
            }
            quids_gpu_step_stats *st = rule_stats ? rule_stats + r : nullptr;
            rc = dispatch_rule(op.kind, &op.params, [&](auto rule) {
                return chain.n ? ranges::simulate_step(ctx, cur, rule, other, prm, st, chain)
                               : ranges::simulate_step(ctx, cur, rule, other, prm, st);
            });
            ++r;
            if (!rc) {
                std::swap(cur, other);
                i = j - 1;
            }
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

int quids_gpu_rule_children(quids_gpu_ctx *ctx, quids_gpu_state *iteration, int rule_kind,
                            const quids_gpu_rule_params *rule, uint64_t *num_children, uint64_t *stride,
                            uint8_t *child_bytes, uint64_t *hash, uint32_t *size, double *magnitude) {
    return dispatch_rule(rule_kind, rule, [&](auto r) {
        return rule_children(ctx, iteration, r, num_children, stride, child_bytes, hash, size, magnitude);
    });
}

int quids_gpu_average_value(quids_gpu_ctx *ctx, quids_gpu_state *st, int kind, const quids_gpu_rule_params *p,
                            double *value) {
    switch (kind) {
    case QUIDS_OBS_QCGD_NUM_NODES: return average_value(ctx, st, qcgd::obs_num_nodes{false}, value);
    case QUIDS_OBS_QCGD_NUM_NODES_SQ: return average_value(ctx, st, qcgd::obs_num_nodes{true}, value);
    case QUIDS_OBS_QCGD_DENSITY: return average_value(ctx, st, qcgd::obs_density{false}, value);
    case QUIDS_OBS_QCGD_DENSITY_SQ: return average_value(ctx, st, qcgd::obs_density{true}, value);
    case QUIDS_OBS_QC_BIT:
        if (!p) return QUIDS_ERR_BAD_ARG;
        return average_value(ctx, st, rules::obs_bit{p->bit}, value);
    }
    return QUIDS_ERR_BAD_ARG;
}

int quids_gpu_qcgd_statistics(quids_gpu_ctx *ctx, quids_gpu_state *st, uint64_t sy_n, uint64_t sy_nu, double tol,
                              quids_gpu_qcgd_stats *out) {
    if (!ctx || !st || !out) return QUIDS_ERR_BAD_ARG;
    // src/rules/qcgd.hpp:309-366
    quids_gpu_qcgd_stats r{};
    r.interference_ratio = 1;
    r.deletion_ratio = 1;
    if (sy_n > 0) {
        r.interference_ratio = (double)sy_nu / (double)sy_n;
        r.deletion_ratio = (double)st->n / (double)sy_nu;
    }
    double sq_size, sq_density;
    QD_TRY(average_value(ctx, st, qcgd::obs_num_nodes{false}, &r.avg_size));
    QD_TRY(average_value(ctx, st, qcgd::obs_num_nodes{true}, &sq_size));
    QD_TRY(average_value(ctx, st, qcgd::obs_density{false}, &r.avg_density));
    QD_TRY(average_value(ctx, st, qcgd::obs_density{true}, &sq_density));
    double v = sq_size - r.avg_size * r.avg_size;
    r.std_dev_size = v < tol ? 0 : std::sqrt(sq_size);
    v = sq_density - r.avg_density * r.avg_density;
    r.std_dev_density = v < tol ? 0 : std::sqrt(v);
    QD_TRY(quids_gpu_state_total_proba(st, &r.total_proba));
    r.num_graphs = (double)st->n;
    *out = r;
    return QUIDS_OK;
}

int quids_gpu_state_hash(quids_gpu_ctx *ctx, quids_gpu_state *st, int rule_kind, const quids_gpu_rule_params *rule,
                         uint64_t *out) {
    if (!ctx || !st || !out || st->ctx != ctx) return QUIDS_ERR_BAD_ARG;
    if (st->n == 0) return QUIDS_OK;
    QD_CUDA(cudaSetDevice(ctx->device));
    qd_dbuf d;
    QD_TRY(ensure(d, st->n * sizeof(uint64_t)));
    int rc = dispatch_rule(rule_kind, rule, [&](auto r) {
        k_state_hash<<<grid_for(ctx, st->n), prim::kThreads, 0, ctx->stream>>>(
            r, (const char *)st->objects.p, (const uint64_t *)st->begin.p, (const uint32_t *)st->size.p, st->n,
            (uint64_t *)d.p);
        return launched(ctx);
    });
    if (!rc) rc = cuda_status(cudaMemcpyAsync(out, d.p, st->n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (!rc) rc = cuda_status(cudaStreamSynchronize(ctx->stream));
    release(d);
    return rc;
}

}  // extern "C"
