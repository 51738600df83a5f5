// planned_batch.cuh -- planned rule steps of the batched form: the step of
// batch.cuh without its host synchronisations, for runs whose sizes are known
// from an earlier run of the same op list (planned.cuh has the scheme).  The
// per-instance rules of every step sit in a device buffer of the plan, so a
// run captured as a CUDA graph reads nothing from host memory.
#pragma once
#include "batch.cuh"
#include "planned.cuh"

namespace qd::planned {
using namespace qd::engine;

// Before a planned batched step: every instance of the input holds at most
// max_num_object parents (the plan has no per-instance pre-truncation).
static __global__ void k_bplan_parents(uint64_t *words, uint32_t app, const uint64_t *inst_begin, uint32_t G,
                                       uint64_t maxc) {
    if (stopped(words)) return;
    bool over = false;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < G; g += gridDim.x * blockDim.x)
        over |= inst_begin[g + 1] - inst_begin[g] > maxc;
    if (__syncthreads_or(over) && threadIdx.x == 0) {
        // one block: G <= 65536 instances are read by 1024 threads
        stop_at(words, app, kReplan);
    }
}

// the buffers of a planned batched step at the plan's bounds
inline int ensure_planned_batched(quids_gpu_ctx *ctx, quids_gpu_state *out, const app_plan &ap, double load,
                                  bool keep, uint32_t G) {
    QD_TRY(ensure_planned(ctx, out, ap, load, keep));
    QD_TRY(ensure(ctx->buf[B_BCOUNT], (size_t)G * 7 * sizeof(unsigned long long)));
    QD_TRY(ensure(ctx->buf[B_BSEL], (size_t)G * sizeof(prim::select_state)));
    QD_TRY(ensure(ctx->buf[B_BHIST], (size_t)G * prim::kBins * sizeof(unsigned int)));
    QD_TRY(ensure(ctx->buf[B_BOFF], (size_t)(G + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_UBEGIN], (size_t)(G + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_PBEGIN], (size_t)(G + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_BFACTOR], (size_t)G * sizeof(double)));
    QD_TRY(ensure(ctx->buf[B_UINST], ap.nc_cap * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_UCHILD], ap.nc_cap * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_UMAG], ap.nc_cap * sizeof(double2)));
    auto grow = [&](qd_dbuf &b, size_t bytes) { return keep ? ensure_keep(b, bytes, ctx->stream) : ensure(b, bytes); };
    QD_TRY(grow(out->inst, ap.ns_cap * sizeof(uint32_t)));
    QD_TRY(grow(out->inst_begin, (size_t)(G + 1) * sizeof(uint64_t)));
    QD_TRY(grow(out->inst_total, (size_t)G * sizeof(double)));
    return QUIDS_OK;
}

// One planned batched rule step from `in` into `out` (batch::simulate_batched
// with the plan's bounds in place of its host synchronisations).  rules: the
// step's per-instance rules on the device.
template <class Rule>
int simulate_batched_planned(quids_gpu_ctx *ctx, quids_gpu_state *in, const uint64_t *in_meta, uint64_t n_host,
                             const Rule *rules, quids_gpu_state *out, const quids_gpu_params &prm,
                             const app_plan &ap, uint32_t app, uint64_t *rec) {
    using namespace qd::batch;
    const uint32_t G = in->n_inst;
    const uint64_t maxc = prm.max_num_object;
    const double load = eff_load(ctx, prm);
    const bool fast = (prm.flags & QUIDS_FLAG_NO_FAST_HASH) == 0;
    const trunc_key tk{prm.simple_truncation == 0, prm.seed};
    QD_TRY(ensure_planned_batched(ctx, out, ap, load, true, G));  // no-ops: the run ensured every step first
    const uint64_t N = ap.n_cap, NC = ap.nc_cap, NSB = ap.ns_cap;
    const uint64_t Mb = std::max<uint64_t>((uint64_t)((double)NC / load) + 1, 1024);
    uint64_t *words = ctx->d_words;
    int *err = (int *)(words + W_STATUS);
    const uint64_t *stop = words + W_STATUS;
    unsigned long long *cnt = bufp<unsigned long long>(ctx, B_BCOUNT);
    unsigned long long *tiecnt = cnt, *tot = cnt + G;
    unsigned long long *maxn = cnt + 6ull * G;
    prim::select_state *bst = bufp<prim::select_state>(ctx, B_BSEL);
    unsigned int *bhist = bufp<unsigned int>(ctx, B_BHIST);
    uint64_t *tie_off = bufp<uint64_t>(ctx, B_BOFF);
    uint64_t *pbegin = bufp<uint64_t>(ctx, B_PBEGIN), *ubegin = bufp<uint64_t>(ctx, B_UBEGIN);
    const uint32_t *pinst = (const uint32_t *)in->inst.p;
    const instance_rules<Rule> rs{rules, pinst};
    out->n_inst = G;

    // ---- step words (no instance may need a parent pre-truncation), num_child, offsets
    k_bplan_parents<<<1, 1024, 0, ctx->stream>>>(words, app, (const uint64_t *)in->inst_begin.p, G, maxc);
    const uint64_t nzero0 = lookback_words(N);
    k_plan_begin<<<(unsigned)std::min<uint64_t>((nzero0 + 255) / 256 + 1, (uint64_t)ctx->num_sms * 4), 256, 0,
                   ctx->stream>>>(words, app, n_host, in_meta, N, ~0ull, bufp<int>(ctx, B_MODSTATUS),
                                  bufp<uint64_t>(ctx, B_LOOKBACK), nzero0);
    k_num_child<<<grid_for(ctx, N), prim::kThreads, 0, ctx->stream>>>(
        rs, (const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p, N,
        bufp<uint32_t>(ctx, B_NCHILD), (unsigned long long *)(words + W_MAXSIZE), err, words + W_N);
    QD_TRY(launched(ctx, 3));
    QD_CUDA(cudaMemcpyAsync(pbegin, in->inst_begin.p, (size_t)(G + 1) * sizeof(uint64_t), cudaMemcpyDeviceToDevice,
                            ctx->stream));
    const uint64_t sym_tiles = sym_tiles_of(NC);
    {
        prim::lookback lb;
        lookback_view(ctx, N, 1, lb);
        scan_nchild f{bufp<uint32_t>(ctx, B_NCHILD), nullptr};
        const plan_sizes_hook hook{words, app, ap.nc_cap, ap.maxsize_lim, ~0ull, load,
                                   bufp<unsigned long long>(ctx, B_ACC)};
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
    ftab.p[0] = (unsigned char *)tb.slots, ftab.n[0] = (Mb + 1) * sizeof(prim::table_slot), ftab.v[0] = 0xff;
    ftab.dn[0] = words + W_M, ftab.mul[0] = sizeof(prim::table_slot), ftab.add[0] = sizeof(prim::table_slot);
    ftab.p[1] = bufp<unsigned char>(ctx, B_NOTREP), ftab.n[1] = NC, ftab.v[1] = 0;
    ftab.dn[1] = words + W_NC, ftab.mul[1] = 1, ftab.add[1] = 0;
    ftab.p[2] = bufp<unsigned char>(ctx, B_HASJOIN), ftab.n[2] = NC, ftab.v[2] = 0;
    ftab.dn[2] = words + W_NC, ftab.mul[2] = 1, ftab.add[2] = 0;
    ftab.p[3] = bufp<unsigned char>(ctx, B_LOOKBACK), ftab.n[3] = 4 * (tiles_nc + 2) * sizeof(uint64_t);
    ftab.v[3] = 0;
    ftab.count = 4;

    // ---- symbolic iteration, instance-tagged hashes (the grouped pass claims the table slots as well)
    bool grouped = false;
    if constexpr (has_grouped<Rule>::value) grouped = fast;
    if constexpr (has_grouped<Rule>::value)
        if (grouped)
            QD_TRY(launch_symbolic_grouped(ctx, rs, pv, NC, table_claim{tb, bufp<uint32_t>(ctx, B_SLOT), err},
                                           [&] { return fill(ctx, ftab); }));
    if (!grouped) {
        if (ap.maxsize_lim <= 256) {
            QD_TRY((launch_symbolic<instance_rules<Rule>, 256>(ctx, rs, pv, NC, fast)));
        } else {
            QD_TRY((launch_symbolic<instance_rules<Rule>, 4096>(ctx, rs, pv, NC, fast)));
        }
    }

    // ---- collision elimination, table sized on the device
    if (!grouped) QD_TRY(fill(ctx, ftab));
    uint8_t *not_rep = bufp<uint8_t>(ctx, B_NOTREP), *has_join = bufp<uint8_t>(ctx, B_HASJOIN);
    const unsigned long long *d_maxabs = (const unsigned long long *)(words + W_MAXABS);
    direct_src src{bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG)};
    if (!grouped) {
        prim::k_table_claim<<<grid_for(ctx, NC), ctx->tune.table_block, 0, ctx->stream>>>(
            tb, src, words + W_NC, bufp<uint32_t>(ctx, B_SLOT), err);
        QD_TRY(launched(ctx));
    }
    prim::k_table_accumulate<<<grid_for(ctx, NC), ctx->tune.table_block, 0, ctx->stream>>>(
        tb, src, bufp<uint32_t>(ctx, B_SLOT), words + W_NC, d_maxabs, not_rep, has_join);
    QD_TRY(launched(ctx));

    // ---- zero elimination, groups with their instance
    group_view gv{bufp<uint32_t>(ctx, B_SLOT), not_rep, has_join, bufp<double2>(ctx, B_CMAG),
                  bufp<unsigned long long>(ctx, B_ACC), words + W_NC, d_maxabs, prm.tolerance};
    {
        prim::lookback lb;
        lookback_view(ctx, NC, 3, lb);
        bgroups_collect f{gv, bufp<uint32_t>(ctx, B_CPAR), nullptr, pinst, bufp<uint64_t>(ctx, B_UCHILD),
                          bufp<double2>(ctx, B_UMAG), bufp<uint64_t>(ctx, B_UNORM), bufp<uint32_t>(ctx, B_UINST)};
        prim::k_compact<<<lookback_grid(ctx, NC), prim::kThreads, 0, ctx->stream>>>(f, words + W_NC, words + W_NU, lb);
        k_inst_bounds<<<grid_for(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
            inst_direct{bufp<uint32_t>(ctx, B_UINST)}, words + W_NU, G, ubegin);
        QD_TRY(launched(ctx, 2));
    }

    // ---- per-instance truncation and layout
    key_unorm k1{bufp<uint64_t>(ctx, B_UNORM), bufp<uint64_t>(ctx, B_UCHILD), tk};
    QD_TRY(segmented_select(ctx, k1, bufp<uint32_t>(ctx, B_UINST), words + W_NU, NC, ubegin, G, maxc, bst, bhist,
                            tiecnt, tie_off));
    {
        prim::lookback lbc, lbb, lbt;
        lookback_view(ctx, NC, 0, lbt);
        lookback_view(ctx, NC, 1, lbc);
        lookback_view(ctx, NC, 2, lbb);
        bkeep_layout kl{k1, bufp<uint64_t>(ctx, B_UCHILD), bufp<double2>(ctx, B_UMAG), bufp<uint32_t>(ctx, B_UINST),
                        bst, tie_off, bufp<uint32_t>(ctx, B_CSIZE), prm.align_byte_length, (double2 *)out->mag.p,
                        (uint32_t *)out->size.p, (uint64_t *)out->begin.p, bufp<uint64_t>(ctx, B_SCHILD),
                        (uint32_t *)out->inst.p};
        prim::k_compact_layout<bkeep_layout, true><<<lookback_grid(ctx, NC), prim::kThreads, 0, ctx->stream>>>(
            kl, words + W_NU, words + W_NS, words + W_OUTBYTES, (uint64_t *)out->begin.p, nullptr, lbc, lbb, lbt,
            hook_counter(ctx, W_DONE_LAYOUT), plan_end_hook{words, app, ap.bytes_cap, true, (uint64_t *)out->meta.p, rec});
        QD_TRY(launched(ctx));
    }

    // ---- per-instance normalisation and finalize
    uint64_t *obegin = (uint64_t *)out->inst_begin.p;
    QD_CUDA(cudaMemsetAsync(tot, 0, (size_t)G * 2 * sizeof(unsigned long long), ctx->stream));
    QD_CUDA(cudaMemsetAsync(maxn, 0, (size_t)G * sizeof(unsigned long long), ctx->stream));
    k_inst_bounds<<<grid_for(ctx, NSB), prim::kThreads, 0, ctx->stream>>>(
        inst_direct{(const uint32_t *)out->inst.p}, words + W_NS, G, obegin, stop);
    const unsigned grid_runs = grid_for(ctx, (NSB + kRun - 1) / kRun);
    k_binst_max<<<grid_runs, prim::kThreads, 0, ctx->stream>>>((const double2 *)out->mag.p,
                                                              (const uint32_t *)out->inst.p, words + W_NS, maxn);
    k_binst_totals<<<grid_runs, prim::kThreads, 0, ctx->stream>>>(
        (const double2 *)out->mag.p, (const uint32_t *)out->inst.p, words + W_NS, obegin, maxn, tot);
    k_binst_factors<<<(G + 255) / 256, 256, 0, ctx->stream>>>(tot, G, obegin, maxn, (double *)out->inst_total.p,
                                                             bufp<double>(ctx, B_BFACTOR), stop);
    QD_TRY(launched(ctx, 4));
    QD_TRY(launch_populate_kernel(
        ctx, NSB, ap.maxsize > kStageMin, rs, pv,
        schild_source{bufp<uint64_t>(ctx, B_SCHILD), bufp<uint32_t>(ctx, B_CPAR), pv.cbeg}, words + W_NS,
        (const uint64_t *)out->begin.p, (const uint32_t *)out->size.p, (char *)out->objects.p, (double2 *)out->mag.p,
        bufp<double>(ctx, B_BFACTOR), (const uint32_t *)out->inst.p, err, no_post{}));
    out->total_pending = false;
    out->total_proba = std::numeric_limits<double>::quiet_NaN();  // per instance: inst_total
    return QUIDS_OK;
}

}  // namespace qd::planned
