// adjoint.cuh -- reverse mode through rule steps, with respect to the rule
// angles (theta, phi, xi of the QCGD rules).
//
// With the step's structure held fixed (which children a parent has, which
// children collide, which groups survive zero elimination and truncation),
// a rule step of quids::simulate (src/quids.hpp:448-543) is linear in the
// magnitudes up to the final normalisation:
//   v_c = f_c(theta, phi, xi) * m_parent(c)          (symbolic iteration)
//   u_s = sum of v_c over the children c of group s   (collision sum)
//   m'_s = u_s / ||u||                                 (normalize)
// where f_c is a product of the rule's four factors
//   d = sin(theta) e^{i phi}, conj(d), dn = cos(theta) e^{i xi}, -conj(dn)
// (src/rules/qcgd.hpp:466-471).  A child's factor counts (n_d, n_dc, n_dn,
// n_ndnc) give f_c and its derivatives in closed form:
//   f = (-1)^n_ndnc sin^a cos^b e^{i(phi (n_d - n_dc) + xi (n_dn - n_ndnc))},
//   a = n_d + n_dc, b = n_dn + n_ndnc,
//   df/dtheta = (-1)^n_ndnc e^{i...} (a sin^(a-1) cos^(b+1) - b sin^(a+1) cos^(b-1)),
//   df/dphi = i (n_d - n_dc) f,  df/dxi = i (n_dn - n_ndnc) f.
// Adjoints are a = 2 dL/d(conj z), so dL = Re sum conj(a) dz:
//   normalize:  a_u = (a' - Re<a', m'> m') / ||u||
//   collisions: a_v(c) = a_u(group of c), or 0 when the group was dropped
//   children:   a_m(p) = sum over children c of p of conj(f_c) a_v(c)
//   angles:     dL/dtheta += Re(conj(a_v(c)) m_p df_c/dtheta), and so on.
// A backward rule step reads the structure its forward step left (a record:
// table slots, child offsets, representatives, normalisation factor), taken
// during the forward or the recomputation of its segment; the pipeline is
// deterministic, so a recomputed step has the forward's structure.  Every
// reduction has a fixed order: one warp per parent gathers its children,
// and the angle sums go through a fixed grid of per-block partials.
#pragma once
#include <type_traits>

#include "engine.cuh"
#include "rules_qcgd.cuh"

namespace qd::adjoint {

using namespace qd::engine;

struct rule_angles {
    double theta, phi, xi;
};

template <class R, class = void>
struct has_factor_counts : std::false_type {};
template <class R>
struct has_factor_counts<R, std::void_t<decltype(std::declval<const R &>().factor_counts(
                                (const char *)0, (const char *)0, 0u, std::declval<qcgd::factor_count &>()))>>
    : std::true_type {};

__device__ __forceinline__ double ipow(double x, int k) {
    double r = 1;
    for (int i = 0; i < k; ++i) r *= x;
    return r;
}

struct child_factor {
    mag_t f, dth, dph, dxi;
};

__device__ __forceinline__ child_factor factor_of(const qcgd::factor_count &fc, double s, double c,
                                                  const rule_angles &ang) {
    const int a = fc.n[qcgd::F_D] + fc.n[qcgd::F_DC], b = fc.n[qcgd::F_DN] + fc.n[qcgd::F_NDNC];
    const int kp = (int)fc.n[qcgd::F_D] - (int)fc.n[qcgd::F_DC];
    const int kx = (int)fc.n[qcgd::F_DN] - (int)fc.n[qcgd::F_NDNC];
    double sp, cp;
    sincos(ang.phi * kp + ang.xi * kx, &sp, &cp);
    const double sign = (fc.n[qcgd::F_NDNC] & 1) ? -1.0 : 1.0;
    const double r = sign * ipow(s, a) * ipow(c, b);
    double dr = 0;
    if (a) dr += a * ipow(s, a - 1) * ipow(c, b + 1);
    if (b) dr -= b * ipow(s, a + 1) * ipow(c, b - 1);
    dr *= sign;
    child_factor out;
    out.f = mag_t{r * cp, r * sp};
    out.dth = mag_t{dr * cp, dr * sp};
    out.dph = mag_t{-kp * out.f.im, kp * out.f.re};
    out.dxi = mag_t{-kx * out.f.im, kx * out.f.re};
    return out;
}

// fixed grid of the adjoint reductions (partials summed by k_sum_partials)
constexpr int kAdjBlocks = kObsBlocks;

// partial[b] = sum over block b's chunk of Re(conj(a_j) m_j)
static __global__ void __launch_bounds__(prim::kThreads)
    k_dot_partial(const double2 *a, const double2 *m, uint64_t n, double *partial) {
    __shared__ double sm[prim::kThreads];
    const uint64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const uint64_t b = (uint64_t)blockIdx.x * chunk, e = b + chunk < n ? b + chunk : n;
    double acc = 0;
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const double2 x = a[i], y = m[i];
        acc += x.x * y.x + x.y * y.y;
    }
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int o = prim::kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

// a <- (a - dot m) / factor  (the adjoint through normalize)
static __global__ void __launch_bounds__(prim::kThreads)
    k_norm_adjoint(double2 *a, const double2 *m, uint64_t n, const double *dot, const double *d_factor) {
    const double d = *dot, f = *d_factor;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const double2 x = a[i], y = m[i];
        a[i] = make_double2((x.x - d * y.x) / f, (x.y - d * y.y) / f);
    }
}

// survivor index of each table slot: surv[slot of survivor j's representative] = j
static __global__ void __launch_bounds__(prim::kThreads)
    k_surv_of_slot(const uint64_t *schild, const uint32_t *slot_of, uint64_t ns, uint64_t m_slots, uint32_t *surv) {
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < ns; j += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = slot_of[schild[j]] & ~prim::kJoin;
        if (s < m_slots) surv[s] = (uint32_t)j;
    }
}

// Per-block tables for the closed forms: sin^k, cos^k (k <= kMaxSites) and
// e^{i phi k}, e^{i xi k} (|k| <= kMaxSites).  Beyond them, the direct form.
constexpr int kMaxSites = 63;
struct factor_tables {
    double sp[kMaxSites + 2], cp[kMaxSites + 2];
    double2 ephi[2 * kMaxSites + 1], exi[2 * kMaxSites + 1];
};
__device__ __forceinline__ void fill_tables(factor_tables &t, const rule_angles &ang) {
    double s, c;
    sincos(ang.theta, &s, &c);
    for (int k = threadIdx.x; k < kMaxSites + 2; k += blockDim.x) {
        t.sp[k] = ipow(s, k);
        t.cp[k] = ipow(c, k);
    }
    for (int k = threadIdx.x; k < 2 * kMaxSites + 1; k += blockDim.x) {
        double a, b;
        sincos(ang.phi * (k - kMaxSites), &a, &b);
        t.ephi[k] = make_double2(b, a);
        sincos(ang.xi * (k - kMaxSites), &a, &b);
        t.exi[k] = make_double2(b, a);
    }
}
__device__ __forceinline__ child_factor factor_from_tables(const qcgd::factor_count &fc, const factor_tables &t,
                                                           double s, double c, const rule_angles &ang) {
    const int a = fc.n[qcgd::F_D] + fc.n[qcgd::F_DC], b = fc.n[qcgd::F_DN] + fc.n[qcgd::F_NDNC];
    const int kp = (int)fc.n[qcgd::F_D] - (int)fc.n[qcgd::F_DC];
    const int kx = (int)fc.n[qcgd::F_DN] - (int)fc.n[qcgd::F_NDNC];
    if (a > kMaxSites || b > kMaxSites) return factor_of(fc, s, c, ang);
    const double2 ep = t.ephi[kp + kMaxSites], ex = t.exi[kx + kMaxSites];
    const double pr = ep.x * ex.x - ep.y * ex.y, pi = ep.x * ex.y + ep.y * ex.x;
    const double sign = (fc.n[qcgd::F_NDNC] & 1) ? -1.0 : 1.0;
    const double r = sign * t.sp[a] * t.cp[b];
    double dr = 0;
    if (a) dr += a * t.sp[a - 1] * t.cp[b + 1];
    if (b) dr -= b * t.sp[a + 1] * t.cp[b - 1];
    dr *= sign;
    child_factor out;
    out.f = mag_t{r * pr, r * pi};
    out.dth = mag_t{dr * pr, dr * pi};
    out.dph = mag_t{-kp * out.f.im, kp * out.f.re};
    out.dxi = mag_t{-kx * out.f.im, kx * out.f.re};
    return out;
}

// One warp per kept parent: the parent's adjoint from its children (in child
// order, then a fixed shuffle tree), and the children's angle derivatives.
// gpartial: [3][kAdjBlocks] per-block angle sums.
template <class RS>
__global__ void __launch_bounds__(prim::kThreads)
    k_adj_parents(RS rs, parents_view pv, const uint32_t *slot_of, const uint32_t *surv, uint64_t m_slots,
                  const double2 *a_u, rule_angles ang, double2 *a_in, double *gpartial) {
    using Rule = typename RS::rule_type;
    __shared__ double sm[3][prim::kThreads / 32];
    __shared__ factor_tables tab;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    double s_th, c_th;
    sincos(ang.theta, &s_th, &c_th);
    if constexpr (has_factor_counts<Rule>::value) fill_tables(tab, ang);
    __syncthreads();
    double g0 = 0, g1 = 0, g2 = 0;
    for (uint64_t p = (uint64_t)blockIdx.x * (blockDim.x >> 5) + wib; p < pv.np; p += warps) {
        const uint64_t oid = pv.pidx ? pv.pidx[p] : p;
        const double2 pm = pv.mag[oid];
        const uint64_t lo = pv.cbeg[p], hi = pv.cbeg[p + 1];
        const char *pb = pv.objects + pv.begin[oid];
        const char *pe = pb + pv.size[oid];
        const Rule &rule = rs.get(oid);
        double ar = 0, ai = 0;
        for (uint64_t c = lo + lane; c < hi; c += 32) {
            const uint32_t sl = slot_of[c] & ~prim::kJoin;
            if (sl >= m_slots) continue;
            const uint32_t j = surv[sl];
            if (j == 0xffffffffu) continue;  // the child's group was dropped
            const double2 au = a_u[j];
            const uint32_t cid = (uint32_t)(c - lo);
            mag_t f;
            if constexpr (has_factor_counts<Rule>::value) {
                qcgd::factor_count fc{};
                rule.factor_counts(pb, pe, cid, fc);
                const child_factor cf = factor_from_tables(fc, tab, s_th, c_th, ang);
                f = cf.f;
                // Re(conj(a_v) m_p df)
                const mag_t d0 = cmul(mag_t{pm.x, pm.y}, cf.dth), d1 = cmul(mag_t{pm.x, pm.y}, cf.dph),
                            d2 = cmul(mag_t{pm.x, pm.y}, cf.dxi);
                g0 += au.x * d0.re + au.y * d0.im;
                g1 += au.x * d1.re + au.y * d1.im;
                g2 += au.x * d2.re + au.y * d2.im;
            } else {
                uint32_t sz;
                f = mag_t{1.0, 0.0};
                rule.hash_child(pb, pe, cid, sz, f);  // the child's factor: its magnitude from a unit parent
            }
            ar += f.re * au.x + f.im * au.y;  // conj(f) a_v
            ai += f.re * au.y - f.im * au.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
            ar += __shfl_xor_sync(0xffffffffu, ar, o);
            ai += __shfl_xor_sync(0xffffffffu, ai, o);
        }
        if (lane == 0) a_in[oid] = make_double2(ar, ai);
    }
    for (int o = 16; o > 0; o >>= 1) {
        g0 += __shfl_xor_sync(0xffffffffu, g0, o);
        g1 += __shfl_xor_sync(0xffffffffu, g1, o);
        g2 += __shfl_xor_sync(0xffffffffu, g2, o);
    }
    if (lane == 0) {
        sm[0][wib] = g0;
        sm[1][wib] = g1;
        sm[2][wib] = g2;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0;
        for (int w = 0; w < prim::kThreads / 32; ++w) t += sm[threadIdx.x][w];
        gpartial[(uint64_t)threadIdx.x * gridDim.x + blockIdx.x] = t;
    }
}

// loss = sum obs(o) |m|^2 and its adjoint a = 2 obs(o) m (chunked like the
// observable reduction, fixed order)
template <class Obs>
__global__ void __launch_bounds__(prim::kThreads)
    k_loss_adjoint(Obs obs, const char *objects, const uint64_t *begin, const uint32_t *size, const double2 *mag,
                   uint64_t n, double2 *a, double *partial) {
    __shared__ double sm[prim::kThreads];
    const uint64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const uint64_t b = (uint64_t)blockIdx.x * chunk, e = b + chunk < n ? b + chunk : n;
    double acc = 0;
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const char *o = objects + begin[i];
        const double w = obs(o, o + size[i]);
        const double2 m = mag[i];
        a[i] = make_double2(2 * w * m.x, 2 * w * m.y);
        acc += w * (m.x * m.x + m.y * m.y);
    }
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int o = prim::kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

// scratch of a backward pass (owned by the tape)
struct scratch {
    qd_dbuf surv;     // u32 [table slots]
    qd_dbuf partial;  // double [4 kAdjBlocks + 4]
};

// What the backward of one rule step needs from its forward: the children's
// table slots, the child offsets over the kept parents (and the kept
// parents), each survivor's representative child, the normalisation factor
// and the output state (its magnitudes).  Captured right after the step
// (capture_record), so the backward needs no replay of the step.
struct step_record {
    qd_dbuf slot_of, cbeg, pidx, schild, factor;
    uint64_t N = 0, NP = 0, NC = 0, NS = 0, M = 0;
    bool has_pidx = false;
    quids_gpu_state *out = nullptr;  // not owned
};
inline void release_record(step_record &r) {
    for (qd_dbuf *b : {&r.slot_of, &r.cbeg, &r.pidx, &r.schild, &r.factor}) release(*b);
    r = step_record{};
}
inline int capture_record(quids_gpu_ctx *ctx, const quids_gpu_step_stats &st, const quids_gpu_state *in,
                          quids_gpu_state *out, step_record &r) {
    r.N = in->n;
    r.NP = st.num_parents_kept;
    r.NC = st.num_object;
    r.NS = out->n;
    r.M = st.table_capacity;
    r.out = out;
    r.has_pidx = r.NP < r.N;
    if (r.NC == 0 || r.NS == 0) return QUIDS_OK;
    cudaStream_t s = ctx->stream;
    QD_TRY(ensure(r.slot_of, r.NC * sizeof(uint32_t)));
    QD_TRY(ensure(r.cbeg, (r.NP + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(r.schild, r.NS * sizeof(uint64_t)));
    QD_TRY(ensure(r.factor, sizeof(double)));
    QD_CUDA(cudaMemcpyAsync(r.slot_of.p, ctx->buf[B_SLOT].p, r.NC * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    QD_CUDA(cudaMemcpyAsync(r.cbeg.p, ctx->buf[B_CBEGIN].p, (r.NP + 1) * sizeof(uint64_t), cudaMemcpyDeviceToDevice,
                            s));
    QD_CUDA(cudaMemcpyAsync(r.schild.p, ctx->buf[B_SCHILD].p, r.NS * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
    QD_CUDA(cudaMemcpyAsync(r.factor.p, ctx->d_words + W_FACTOR, sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (r.has_pidx) {
        QD_TRY(ensure(r.pidx, r.NP * sizeof(uint64_t)));
        QD_CUDA(cudaMemcpyAsync(r.pidx.p, ctx->buf[B_PIDX].p, r.NP * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
    }
    return QUIDS_OK;
}

// The backward rule step from its forward's record.  a_out: adjoint of the
// output magnitudes (replaced by the adjoint before normalisation); a_in:
// adjoint of in's magnitudes (written for every object); grad3: the three
// angle derivatives (device).
template <class Rule>
int backward_rule(quids_gpu_ctx *ctx, scratch &sc, quids_gpu_state *in, const Rule &rule_, const rule_angles &ang,
                  const step_record &r, double2 *a_out, double2 *a_in, double *grad3) {
    const uint64_t N = in->n, NS = r.NS, NP = r.NP, M = r.M;
    QD_CUDA(cudaMemsetAsync(a_in, 0, (N ? N : 1) * sizeof(double2), ctx->stream));
    QD_CUDA(cudaMemsetAsync(grad3, 0, 3 * sizeof(double), ctx->stream));
    if (N == 0 || NS == 0 || r.NC == 0) return QUIDS_OK;
    QD_TRY(ensure(sc.partial, (4 * kAdjBlocks + 4) * sizeof(double)));
    QD_TRY(ensure(sc.surv, (M + 1) * sizeof(uint32_t)));
    double *partial = (double *)sc.partial.p;
    double *dot = partial + 4 * kAdjBlocks;
    const double2 *mout = (const double2 *)r.out->mag.p;
    // normalize
    k_dot_partial<<<kAdjBlocks, prim::kThreads, 0, ctx->stream>>>(a_out, mout, NS, partial);
    k_sum_partials<<<1, kAdjBlocks, 0, ctx->stream>>>(partial, dot);
    k_norm_adjoint<<<grid_for(ctx, NS), prim::kThreads, 0, ctx->stream>>>(a_out, mout, NS, dot,
                                                                         (const double *)r.factor.p);
    // collisions and truncation: each slot's survivor
    uint32_t *surv = (uint32_t *)sc.surv.p;
    QD_CUDA(cudaMemsetAsync(surv, 0xff, (M + 1) * sizeof(uint32_t), ctx->stream));
    k_surv_of_slot<<<grid_for(ctx, NS), prim::kThreads, 0, ctx->stream>>>(
        (const uint64_t *)r.schild.p, (const uint32_t *)r.slot_of.p, NS, M + 1, surv);
    // children -> parents, angle derivatives
    parents_view pv{(const char *)in->objects.p, (const uint64_t *)in->begin.p, (const uint32_t *)in->size.p,
                    (const double2 *)in->mag.p, (const uint64_t *)r.cbeg.p,
                    r.has_pidx ? (const uint64_t *)r.pidx.p : nullptr, NP};
    const single_rule<Rule> rs{rule_};
    k_adj_parents<single_rule<Rule>><<<kAdjBlocks, prim::kThreads, 0, ctx->stream>>>(
        rs, pv, (const uint32_t *)r.slot_of.p, surv, M + 1, a_out, ang, a_in, partial);
    for (int k = 0; k < 3; ++k)
        k_sum_partials<<<1, kAdjBlocks, 0, ctx->stream>>>(partial + (uint64_t)k * kAdjBlocks, grad3 + k);
    return launched(ctx, 9);
}

template <class Obs>
int loss_adjoint(quids_gpu_ctx *ctx, scratch &sc, quids_gpu_state *st, const Obs &obs, double2 *a, double *d_loss) {
    QD_TRY(ensure(sc.partial, (4 * kAdjBlocks + 4) * sizeof(double)));
    double *partial = (double *)sc.partial.p;
    if (st->n == 0) return cuda_status(cudaMemsetAsync(d_loss, 0, sizeof(double), ctx->stream));
    k_loss_adjoint<Obs><<<kAdjBlocks, prim::kThreads, 0, ctx->stream>>>(
        obs, (const char *)st->objects.p, (const uint64_t *)st->begin.p, (const uint32_t *)st->size.p,
        (const double2 *)st->mag.p, st->n, a, partial);
    k_sum_partials<<<1, kAdjBlocks, 0, ctx->stream>>>(partial, d_loss);
    return launched(ctx, 2);
}

}  // namespace qd::adjoint
