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
#include "planned.cuh"
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
    static constexpr int kMax = 32;
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

// f(modifier) for the modifier of `kind` built from p
template <class F>
int dispatch_modifier(int kind, const quids_gpu_rule_params *p, F &&f) {
    if (!p) return QUIDS_ERR_BAD_ARG;
    switch (kind) {
    case QUIDS_MOD_CNOT: return f(rules::cnot{p->control, p->bit});
    case QUIDS_MOD_X: return f(rules::xgate{p->bit});
    case QUIDS_MOD_Y: return f(rules::ygate{p->bit});
    case QUIDS_MOD_Z: return f(rules::zgate{p->bit});
    case QUIDS_MOD_QCGD_STEP: return f(qcgd::step{});
    case QUIDS_MOD_QCGD_REVERSED_STEP: return f(qcgd::reversed_step{});
    }
    return QUIDS_ERR_BAD_ARG;
}

// The modifiers after the rule at ops[i], up to the next rule, that run
// inside its populate; returns the index of the op after them.
uint64_t gather_chain(const quids_gpu_op *ops, uint64_t n_ops, uint64_t i, mod_chain &chain) {
    uint64_t j = i + 1;
    while (j < n_ops && !ops[j].is_rule && chainable(ops[j].kind) && chain.n < mod_chain::kMax) {
        chain.kind[chain.n] = ops[j].kind;
        chain.bit[chain.n] = ops[j].params.bit;
        chain.control[chain.n] = ops[j].params.control;
        ++chain.n;
        ++j;
    }
    return j;
}

int ensure_modstatus(quids_gpu_ctx *ctx) {
    if (!ctx->buf[B_MODSTATUS].p) {
        QD_TRY(ensure(ctx->buf[B_MODSTATUS], sizeof(uint64_t)));
        QD_CUDA(cudaMemsetAsync(ctx->buf[B_MODSTATUS].p, 0, sizeof(uint64_t), ctx->stream));
    }
    return QUIDS_OK;
}

// The ops of a run from ops[i0] (rule i0_rule) on, synchronously, from the
// state `cur` (the other state is written by the next rule).  st: one entry
// per rule of the whole run.
int run_sync(quids_gpu_ctx *ctx, quids_gpu_state *&cur, quids_gpu_state *&other, const quids_gpu_op *ops,
             uint64_t n_ops, uint64_t i0, uint64_t r0, const quids_gpu_params &prm, quids_gpu_step_stats *st) {
    uint64_t r = r0;
    for (uint64_t i = i0; i < n_ops; ++i) {
        const quids_gpu_op &op = ops[i];
        int rc;
        if (op.is_rule) {
            // the modifiers up to the next rule run inside this rule's populate
            mod_chain chain;
            const uint64_t j = gather_chain(ops, n_ops, i, chain);
            if (chain.n) {
                QD_TRY(ensure_modstatus(ctx));
                chain.status = bufp<int>(ctx, B_MODSTATUS);
            }
            quids_gpu_step_stats *s = st + r;
            rc = dispatch_rule(op.kind, &op.params, [&](auto rule) {
                return chain.n ? ranges::simulate_step(ctx, cur, rule, other, prm, s, chain)
                               : ranges::simulate_step(ctx, cur, rule, other, prm, s);
            });
            ++r;
            if (!rc) {
                std::swap(cur, other);
                i = j - 1;
            }
        } else {
            rc = quids_gpu_apply_modifier(ctx, cur, op.kind, &op.params);
        }
        if (rc) return rc;
    }
    return QUIDS_OK;
}

// ------------------------------------------------------------ planned runs
// quids_gpu_run keeps, per context, the plans of the runs it has seen (op
// list, knobs and state handles): the first run of an op list is
// synchronous and records each rule step's counts; the next runs are
// planned (planned.cuh); from the third on, the planned run is a captured
// CUDA graph, replayed while its buffers and input size are unchanged.
using planned::app_plan;
using planned::run_plan;
constexpr size_t kMaxPlans = 8;

bool plannable(const quids_gpu_params &prm, const quids_gpu_state *a) {
    return prm.max_num_object != 0 &&
           !(prm.flags & (QUIDS_FLAG_STAGE_TIMING | QUIDS_FLAG_NO_PLAN)) &&
           prm.hash_ranges < 2 && a->n_inst == 0;
}

// The bounds of each rule step from a synchronous run's counts (1/16 and a
// little more of headroom); false when a step cannot be planned (parent
// pre-truncation, hash-range passes, 32-bit limits).
bool make_plan(run_plan &p, const quids_gpu_step_stats *st, uint64_t n_rules, const quids_gpu_params &prm) {
    const double load = prm.table_load_factor > 0 && prm.table_load_factor < 0.95 ? prm.table_load_factor : 0.5;
    auto pad = [](uint64_t v) { return v + v / 16 + 64; };
    p.apps.clear();
    for (uint64_t r = 0; r < n_rules; ++r) {
        const quids_gpu_step_stats &s = st[r];
        if (s.num_parents_kept != s.num_parents || s.hash_ranges) return false;
        app_plan ap;
        ap.n_cap = pad(s.num_parents);
        ap.nc_cap = pad(s.num_object);
        if (ap.nc_cap >= 0xffffffffull || (double)ap.nc_cap / load + 2 >= (double)0x7ffffff0ull) return false;
        ap.may_truncate = s.num_object > prm.max_num_object;
        ap.partition = use_partition(prm, ap.nc_cap);
        ap.ns_cap = ap.may_truncate ? std::min<uint64_t>(prm.max_num_object, ap.nc_cap) : ap.nc_cap;
        ap.bytes_cap = pad(s.out_bytes) + 4096;
        ap.maxsize_lim = s.max_child_size <= 256 ? 256 : 4096;
        ap.maxsize = s.max_child_size;
        p.apps.push_back(ap);
    }
    return true;
}

// The launches of a planned run on the stream (captured or not).
int enqueue_planned(quids_gpu_ctx *ctx, run_plan &p, quids_gpu_state *a, quids_gpu_state *b) {
    const quids_gpu_op *ops = p.ops.data();
    const uint64_t n_ops = p.ops.size(), R = p.apps.size();
    planned::k_plan_start<<<1, 1, 0, ctx->stream>>>(ctx->d_words);
    QD_TRY(launched(ctx));
    quids_gpu_state *cur = a, *other = b;
    const uint64_t *cur_meta = nullptr;  // null: the run's input, of known size
    const uint64_t n0 = a->n;
    uint64_t r = 0;
    for (uint64_t i = 0; i < n_ops; ++i) {
        const quids_gpu_op &op = ops[i];
        if (op.is_rule) {
            mod_chain chain;
            const uint64_t j = gather_chain(ops, n_ops, i, chain);
            if (chain.n) chain.status = bufp<int>(ctx, B_MODSTATUS);
            uint64_t *rec = ctx->h_plan_dev + r * planned::R_WORDS;
            QD_TRY(dispatch_rule(op.kind, &op.params, [&](auto rule) {
                return chain.n ? planned::simulate_planned(ctx, cur, cur_meta, n0, rule, other, p.prm, p.apps[r],
                                                           (uint32_t)r, rec, chain)
                               : planned::simulate_planned(ctx, cur, cur_meta, n0, rule, other, p.prm, p.apps[r],
                                                           (uint32_t)r, rec);
            }));
            std::swap(cur, other);
            cur_meta = (const uint64_t *)cur->meta.p;
            ++r;
            i = j - 1;
        } else {
            const uint64_t cap = r == 0 ? n0 : p.apps[r - 1].ns_cap;
            QD_TRY(dispatch_modifier(op.kind, &op.params, [&](auto mod) {
                return planned::apply_modifier_planned(ctx, cur, cur_meta, n0, cap, mod);
            }));
        }
    }
    planned::k_plan_finish<<<1, 1, 0, ctx->stream>>>(ctx->d_words, R >= 2 ? (const uint64_t *)a->meta.p : nullptr,
                                                     R >= 1 ? (const uint64_t *)b->meta.p : nullptr,
                                                     ctx->h_plan_dev + R * planned::R_WORDS);
    return launched(ctx);
}

// One planned run of p from *a.  Returns QUIDS_OK (stats filled, both
// states' host sizes updated), an error, or planned::kReplan with *fail_app
// the rule step to resume from synchronously (its input state intact).
int run_planned(quids_gpu_ctx *ctx, run_plan &p, quids_gpu_state *a, quids_gpu_state *b, quids_gpu_step_stats *st,
                uint64_t *fail_app) {
    const uint64_t R = p.apps.size();
    // every buffer at the plan's bounds before anything is launched
    // (the input state *a keeps its contents; *b is written before it is read)
    auto ensure_all = [&]() -> int {
        QD_TRY(ensure_modstatus(ctx));
        const double load = planned::eff_load(ctx, p.prm);
        for (uint64_t r = 0; r < R; ++r) QD_TRY(planned::ensure_planned(ctx, r % 2 ? a : b, p.apps[r], load, r % 2));
        return QUIDS_OK;
    };
    const volatile uint64_t *fin = nullptr;
    QD_TRY(planned::launch_planned(
        ctx, p, a, ensure_all, [&] { return enqueue_planned(ctx, p, a, b); },
        [&] { return planned::backup_input(ctx, p, a, true); }, [&] { return planned::backup_input(ctx, p, a, false); },
        &fin));
    const int status = (int)(uint32_t)fin[0];
    const uint64_t fa = status ? fin[1] : R;
    planned::read_stats(ctx, R, fa, a->nbytes, false, st);
    auto set_state = [](quids_gpu_state *x, uint64_t n, uint64_t nbytes) {
        x->n = n;
        x->nbytes = nbytes;
        x->total_pending = true;
        x->n_inst = 0;
        x->h_inst_begin.clear();
    };
    if (!status) {
        if (R >= 1) set_state(b, fin[4], fin[5]);
        if (R >= 2) set_state(a, fin[2], fin[3]);
        ++p.runs;
        return QUIDS_OK;
    }
    // stopped at rule step fa: its input (a for even fa) is intact, the other state is not
    quids_gpu_state *in = fa % 2 ? b : a, *out = fa % 2 ? a : b;
    if (fa >= 1) set_state(in, fa % 2 ? fin[4] : fin[2], fa % 2 ? fin[5] : fin[3]);
    out->n = out->nbytes = 0;
    out->total_pending = false;
    out->total_proba = 0;
    *fail_app = fa;
    return status;
}

__global__ void k_set_words_zero(uint64_t *w, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) w[i] = 0;
}

// Device -> host copies of a state.  Into page-locked host memory the SMs
// store the bytes themselves, through the buffer's device-mapped address: on
// GB300 the copy engine's device-to-host rate varied between about 25 and
// 190 GB/s from one copy of a 5.7 GB state to the next, while SM stores over
// the CPU link ran at 193 GB/s every time.  Pageable memory (or a buffer
// whose address is not 16-byte aligned) goes through cudaMemcpyAsync.
__global__ void k_to_host(const uint4 *__restrict__ src, uint4 *__restrict__ dst, uint64_t n16,
                          const unsigned char *__restrict__ tail_src, unsigned char *__restrict__ tail_dst,
                          uint32_t tail) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) dst[i] = src[i];
    if (blockIdx.x == 0 && threadIdx.x < tail) tail_dst[threadIdx.x] = tail_src[threadIdx.x];
}

int copy_to_host(quids_gpu_ctx *ctx, cudaStream_t s, void *dst, const void *src, uint64_t bytes, uint64_t max_blocks) {
    if (!bytes) return QUIDS_OK;
    cudaPointerAttributes a{};
    void *mapped = nullptr;
    if (cudaPointerGetAttributes(&a, dst) == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer)
        mapped = a.devicePointer;
    else
        cudaGetLastError();
    if (!mapped || ((uintptr_t)mapped & 15) || ((uintptr_t)src & 15))
        return cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
    const uint64_t n16 = bytes / 16;
    const uint32_t tail = (uint32_t)(bytes - n16 * 16);
    const uint64_t want = (n16 + 255) / 256;
    const uint64_t cap = max_blocks;
    const unsigned grid = (unsigned)(want < cap ? (want ? want : 1) : cap);
    k_to_host<<<grid, 256, 0, s>>>((const uint4 *)src, (uint4 *)mapped, n16, (const unsigned char *)src + n16 * 16,
                                   (unsigned char *)mapped + n16 * 16, tail);
    return launched(ctx);
}

// the copies of a download, on stream s, by at most `blocks` blocks of SM
// stores (a download that overlaps a step leaves it most of the SMs)
int download_on(quids_gpu_ctx *ctx, quids_gpu_state *st, cudaStream_t s, uint8_t *objects, uint64_t *begin,
                uint32_t *size, double *magnitude, uint64_t blocks) {
    if (objects) QD_TRY(copy_to_host(ctx, s, objects, st->objects.p, st->nbytes, blocks));
    if (begin) {
        if (st->n)
            QD_TRY(copy_to_host(ctx, s, begin, st->begin.p, (st->n + 1) * sizeof(uint64_t), blocks));
        else
            begin[0] = 0;
    }
    if (size) QD_TRY(copy_to_host(ctx, s, size, st->size.p, st->n * sizeof(uint32_t), blocks));
    if (magnitude) QD_TRY(copy_to_host(ctx, s, magnitude, st->mag.p, st->n * 2 * sizeof(double), blocks));
    return QUIDS_OK;
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
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    for (quids_gpu_state *st : ctx->states) {
        release_state(st);
        st->ctx = nullptr;
    }
    ctx->states.clear();
    for (auto *p : ctx->plans) delete p;
    ctx->plans.clear();
    if (ctx->h_plan) cudaFreeHost(ctx->h_plan);
    for (auto &b : ctx->buf) release(b);
    if (ctx->d_words) cudaFree(ctx->d_words);
    if (ctx->h_words) cudaFreeHost(ctx->h_words);
    if (ctx->d_sel) cudaFree(ctx->d_sel);
    if (ctx->d_hist) cudaFree(ctx->d_hist);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (auto &e : ctx->ev_stage)
        if (e) cudaEventDestroy(e);
    if (ctx->ev_copy) cudaEventDestroy(ctx->ev_copy);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return QUIDS_OK;
}

void *quids_gpu_ctx_stream(quids_gpu_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

uint64_t quids_gpu_ctx_launch_count(quids_gpu_ctx *ctx) { return ctx ? ctx->launches : 0; }

int quids_gpu_ctx_last_tuning(quids_gpu_ctx *ctx, quids_gpu_tuning *out) {
    if (!ctx || !out) return QUIDS_ERR_BAD_ARG;
    *out = ctx->last_tuning;
    return QUIDS_OK;
}

int quids_gpu_ctx_run_counts(quids_gpu_ctx *ctx, uint64_t *sync_runs, uint64_t *planned_runs, uint64_t *graph_runs) {
    if (!ctx) return QUIDS_ERR_BAD_ARG;
    if (sync_runs) *sync_runs = ctx->runs_sync;
    if (planned_runs) *planned_runs = ctx->runs_planned;
    if (graph_runs) *graph_runs = ctx->runs_graph;
    return QUIDS_OK;
}

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
    if (st->dl_done) {  // (a pending download ends before the buffers go)
        cudaEventSynchronize(st->dl_done);
        cudaEventDestroy(st->dl_done);
        st->dl_done = nullptr;
        st->dl_pending = false;
    }
    if (!st->ctx) {  // its context is gone and has already released the memory
        delete st;
        return QUIDS_OK;
    }
    cudaSetDevice(st->ctx->device);
    cudaStreamSynchronize(st->ctx->stream);
    planned::drop_plans_of(st->ctx, st);
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
    QD_TRY(after_download(st));
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
    QD_TRY(download_on(ctx, st, s, objects, begin, size, magnitude, (uint64_t)ctx->num_sms * 8));
    QD_CUDA(cudaStreamSynchronize(s));
    return QUIDS_OK;
}

// The copies of quids_gpu_state_download on the context's copy stream,
// ordered after the work already issued on its stream; st->dl_done marks
// their end.  Later work that writes the state waits for it on the device
// (after_download); the host waits in quids_gpu_state_download_wait.
int quids_gpu_state_download_async(quids_gpu_state *st, uint8_t *objects, uint64_t *begin, uint32_t *size,
                                   double *magnitude) {
    if (!st || !st->ctx) return QUIDS_ERR_BAD_ARG;
    quids_gpu_ctx *ctx = st->ctx;
    QD_CUDA(cudaSetDevice(ctx->device));
    if (!ctx->copy_stream) QD_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    if (!ctx->ev_copy) QD_CUDA(cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming));
    if (!st->dl_done) QD_CUDA(cudaEventCreateWithFlags(&st->dl_done, cudaEventDisableTiming));
    cudaStream_t s = ctx->copy_stream;
    QD_CUDA(cudaEventRecord(ctx->ev_copy, ctx->stream));
    QD_CUDA(cudaStreamWaitEvent(s, ctx->ev_copy, 0));
    QD_TRY(download_on(ctx, st, s, objects, begin, size, magnitude, (uint64_t)(ctx->num_sms + 1) / 2));
    QD_CUDA(cudaEventRecord(st->dl_done, s));
    st->dl_pending = true;
    return QUIDS_OK;
}

int quids_gpu_state_download_wait(quids_gpu_state *st) {
    if (!st) return QUIDS_ERR_BAD_ARG;
    if (!st->dl_pending) return QUIDS_OK;
    if (st->ctx) QD_CUDA(cudaSetDevice(st->ctx->device));
    QD_CUDA(cudaEventSynchronize(st->dl_done));
    st->dl_pending = false;
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
    const alloc_limit_scope alloc_limit(prm.max_alloc_bytes);
    if (ctx) {
        QD_CUDA(cudaSetDevice(ctx->device));
        QD_TRY(after_download(iteration));
        QD_TRY(after_download(next_iteration));
    }
    return dispatch_rule(rule_kind, rule, [&](auto r) {
        return ranges::simulate_step(ctx, iteration, r, next_iteration, prm, stats);
    });
}

int quids_gpu_apply_modifier(quids_gpu_ctx *ctx, quids_gpu_state *st, int kind, const quids_gpu_rule_params *p) {
    if (!p) return QUIDS_ERR_BAD_ARG;
    if (ctx && st && st->ctx == ctx) {
        QD_CUDA(cudaSetDevice(ctx->device));
        QD_TRY(after_download(st));
    }
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
    if (a->ctx != ctx || b->ctx != ctx) return QUIDS_ERR_BAD_ARG;
    QD_CUDA(cudaSetDevice(ctx->device));
    QD_TRY(after_download(a));
    QD_TRY(after_download(b));
    QD_CUDA(cudaSetDevice(ctx->device));
    const quids_gpu_params prm = *params;
    const alloc_limit_scope alloc_limit(prm.max_alloc_bytes);
    uint64_t n_rules = 0;
    for (uint64_t i = 0; i < n_ops; ++i) n_rules += ops[i].is_rule ? 1 : 0;
    std::vector<quids_gpu_step_stats> st(n_rules ? n_rules : 1);
    quids_gpu_state *cur = a, *other = b;
    uint64_t i0 = 0, r0 = 0;
    run_plan *p = n_rules && plannable(prm, a) ? planned::find_plan(ctx, a, b, ops, n_ops, prm, 0, nullptr) : nullptr;
    bool replan = false;
    if (p) {
        uint64_t fa = 0;
        const int rc = run_planned(ctx, *p, a, b, st.data(), &fa);
        if (rc == QUIDS_OK) {
            if (rule_stats) std::memcpy(rule_stats, st.data(), n_rules * sizeof(quids_gpu_step_stats));
            *final_index = n_rules % 2 ? 1 : 0;
            return QUIDS_OK;
        }
        if (rc == planned::kNotRun) {  // the plan's bounds do not fit: synchronous from now on
            planned::drop_plan(ctx, p);
            p = nullptr;
        } else if (rc != planned::kReplan) {
            *final_index = fa % 2 ? 1 : 0;
            if (rule_stats) std::memcpy(rule_stats, st.data(), std::min(fa, n_rules) * sizeof(quids_gpu_step_stats));
            return rc;
        } else {
            // resume synchronously at rule step fa, from its intact input
            replan = true;
            for (uint64_t i = 0, r = 0; i < n_ops; ++i) {
                if (!ops[i].is_rule) continue;
                if (r == fa) {
                    i0 = i;
                    break;
                }
                mod_chain chain;
                i = gather_chain(ops, n_ops, i, chain) - 1;
                ++r;
            }
            r0 = fa;
            if (fa % 2) std::swap(cur, other);
        }
    }
    ++ctx->runs_sync;
    const int rc = run_sync(ctx, cur, other, ops, n_ops, i0, r0, prm, st.data());
    *final_index = cur == a ? 0 : 1;
    if (rule_stats) std::memcpy(rule_stats, st.data(), n_rules * sizeof(quids_gpu_step_stats));
    if (rc) return rc;
    // a successful run of a plannable op list: (re)make its plan
    if (n_rules && plannable(prm, a)) {
        if (!p) {
            p = new (std::nothrow) run_plan();
            if (!p) return QUIDS_OK;
            p->ops.assign(ops, ops + n_ops);
            p->prm = prm;
            p->a = a;
            p->b = b;
            ctx->plans.push_back(p);
            if (ctx->plans.size() > kMaxPlans) planned::drop_plan(ctx, ctx->plans.front());
        }
        if (!make_plan(*p, st.data(), n_rules, prm)) {
            planned::drop_plan(ctx, p);
        } else if (replan) {
            p->runs = 0;  // the new bounds are tried uncaptured first
            if (p->exec) cudaGraphExecDestroy(p->exec);
            p->exec = nullptr;
        }
    }
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
