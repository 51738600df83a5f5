// collide.cuh -- partitioned collision elimination and survivor layout for
// steps whose children are far more than L2 holds.
//
// The reference groups the children of a step by hash and sums their
// magnitudes (src/quids.hpp:726-824), keeps the top max_num_object groups
// (:866-900) and lays the survivors out in increasing symbolic index
// (:905-948).  The open-addressing table of engine.cuh does the grouping with
// one random access per child into a table of 16 bytes per slot at load 1/2:
// past about 1 GB every access is a DRAM round trip (about 2.2e10 random
// atomics/s on GB300, against 1.3e11/s for a table that L2 holds and
// 6.8e11/s in shared memory).  Here no table outlives a thread block:
//
//  1. k_pcs_count, a scan, k_pcs_scatter: the children's (hash, index,
//     magnitude) records are partitioned by hash into buckets of about a
//     thousand records (counts and cursors are a few MB, held in L2; the
//     scatter's writes combine in L2);
//  2. k_pcs_group: one block per bucket groups its records in a
//     shared-memory table: representative = the lowest child index (atomic
//     minimum), magnitude = the member's own for a group of one, else the
//     exact 128-bit fixed-point sum with the table path's scale, rounded
//     once -- the same bits as the table path; groups of norm above
//     tolerance leave one record (representative, magnitude, truncation key);
//  3. the truncation selects among the group records (radix select), and
//     the survivors' order comes from bitmaps indexed by child: kept groups
//     set their representative's bit (ties at the cutoff first get their
//     rank in child order from a tie bitmap), and a scan of the bitmap's
//     popcounts gives every survivor its slot in child order;
//  4. k_pcs_emit writes each survivor's magnitude, size and representative
//     at its slot; a scan of the padded sizes gives the byte offsets.
//
// The group records come out in an order that depends on scheduling; no
// result does: the sums are exact, the representatives are minima, and the
// selection and the layout depend only on keys and child indices.
//
// Included by engine.cuh inside namespace qd::engine, after the step's
// helpers it uses (trunc_key, fill, look-back chains, radix select).
#pragma once

constexpr int kPcsThreads = 512;           // block of the grouping kernel
constexpr int kPcsSlots = 2048;            // its shared-memory table (distinct hashes per bucket)
constexpr uint64_t kPcsBucketTarget = 768; // mean children per bucket
constexpr int kPcsMaxBits = 24;

inline int pcs_bucket_bits(uint64_t nc) {
    int bits = 0;
    while (bits < kPcsMaxBits && (kPcsBucketTarget << bits) < nc) ++bits;
    return bits;
}
__device__ __forceinline__ uint32_t pcs_bucket(uint64_t h, int bits) {
    return bits ? (uint32_t)((h * 0x9E3779B97F4A7C15ull) >> (64 - bits)) : 0u;
}
// home slot in the block's table, from bits the bucket does not fix
__device__ __forceinline__ uint32_t pcs_home(uint64_t h) {
    return (uint32_t)(((h ^ (h >> 31)) * 0xBF58476D1CE4E5B9ull) >> (64 - 11)) & (kPcsSlots - 1);
}
static_assert(kPcsSlots == 2048, "pcs_home takes 11 bits");

// children per bucket (warp-aggregated atomics on an array L2 holds)
static __global__ void __launch_bounds__(prim::kThreads)
    k_pcs_count(const uint64_t *hash, const uint64_t *d_n, int bits, unsigned int *count) {
    const uint64_t n = *d_n;
    const int lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint64_t c = base + threadIdx.x;
        const uint32_t b = c < n ? pcs_bucket(hash[c], bits) : 0xffffffffu;
        const unsigned same = __match_any_sync(0xffffffffu, b);
        if (b != 0xffffffffu && lane == __ffs(same) - 1) atomicAdd(&count[b], (unsigned)__popc(same));
    }
}
struct scan_count {
    const unsigned int *count;
    __device__ uint64_t operator()(uint64_t i) const { return count[i]; }
};
// records in bucket order: boff[b] + a rank taken from the bucket's cursor
static __global__ void __launch_bounds__(prim::kThreads)
    k_pcs_scatter(const uint64_t *hash, const double2 *mag, const uint64_t *d_n, int bits, const uint64_t *boff,
                  unsigned int *cursor, uint64_t *rhash, uint32_t *ridx, double2 *rmag, int *err) {
    const uint64_t n = *d_n;
    const int lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint64_t c = base + threadIdx.x;
        uint64_t h = 0;
        uint32_t b = 0xffffffffu;
        if (c < n) {
            h = hash[c];
            b = pcs_bucket(h, bits);
        }
        const unsigned same = __match_any_sync(0xffffffffu, b);
        const int leader = __ffs(same) - 1;
        unsigned first = 0;
        if (b != 0xffffffffu && lane == leader) first = atomicAdd(&cursor[b], (unsigned)__popc(same));
        first = __shfl_sync(0xffffffffu, first, leader);
        if (b == 0xffffffffu) continue;
        const uint64_t pos = boff[b] + first + (unsigned)__popc(same & ((1u << lane) - 1));
        if (pos >= boff[b + 1]) {  // counts and cursors disagree
            prim::set_error(err, QUIDS_ERR_CUDA);
            continue;
        }
        rhash[pos] = h;
        ridx[pos] = (uint32_t)c;
        rmag[pos] = mag[c];
    }
}

// What the grouping kernel writes per kept group (norm above tolerance).
struct pcs_groups {
    uint32_t *child;   // representative (lowest child index)
    double2 *mag;      // group magnitude
    uint64_t *key;     // truncation key (null: no truncation possible)
};

// One block per bucket at a time.  Shared memory: kPcsSlots + 1 slots (the
// extra one for the hash kEmptyKey, which the table cannot hold as a key):
// key, representative, member count, and 32 bytes holding either the single
// member's magnitude or the group's fixed-point sum (re lo, re hi, im lo,
// im hi).
struct pcs_smem {
    unsigned long long key[kPcsSlots + 1];
    unsigned int rep[kPcsSlots + 1];
    unsigned int cnt[kPcsSlots + 1];
    unsigned long long sum[4 * (kPcsSlots + 1)];
    uint64_t scan[kPcsThreads / 32 + 1];
    unsigned long long base;
};

__device__ __forceinline__ int pcs_slot(pcs_smem &s, uint64_t h, bool insert) {
    if (h == prim::kEmptyKey) return kPcsSlots;
    uint32_t i = pcs_home(h);
    for (int probe = 0; probe < kPcsSlots; ++probe) {
        const unsigned long long k = insert ? atomicCAS(&s.key[i], prim::kEmptyKey, h) : s.key[i];
        if (k == prim::kEmptyKey || k == h) return (int)i;
        i = (i + 1) & (kPcsSlots - 1);
    }
    return -1;  // more distinct hashes than slots in one bucket
}

__device__ __forceinline__ void smem_fix_add(unsigned long long *w, fix128 v) {
    if ((v.lo | v.hi) == 0) return;
    const unsigned long long old = atomicAdd(&w[0], (unsigned long long)v.lo);
    const unsigned long long carry = (old + v.lo) < old ? 1ull : 0ull;
    const unsigned long long hi = v.hi + carry;
    if (hi) atomicAdd(&w[1], hi);
}

static __global__ void __launch_bounds__(kPcsThreads)
    k_pcs_group(const uint64_t *rhash, const uint32_t *ridx, const double2 *rmag, const uint64_t *boff, uint32_t nb,
                const uint64_t *d_nc, const unsigned long long *d_maxabs, double tolerance, trunc_key tk,
                pcs_groups out, unsigned long long *d_nu, int *err) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    pcs_smem &s = *(pcs_smem *)s_raw;
    const int F = fix_scale(__longlong_as_double((long long)*d_maxabs), *d_nc);
    constexpr int kPer = (kPcsSlots + 1 + kPcsThreads - 1) / kPcsThreads;  // slots per thread in the emit
    for (uint32_t b = blockIdx.x; b < nb; b += gridDim.x) {
        const uint64_t lo = boff[b], hi = boff[b + 1];
        if (lo == hi) continue;
        for (int i = threadIdx.x; i <= kPcsSlots; i += blockDim.x) {
            s.key[i] = prim::kEmptyKey;
            s.rep[i] = 0xffffffffu;
            s.cnt[i] = 0;
            s.sum[4 * i] = s.sum[4 * i + 1] = s.sum[4 * i + 2] = s.sum[4 * i + 3] = 0;
        }
        __syncthreads();
        // members: slot, lowest child index, count
        for (uint64_t k = lo + threadIdx.x; k < hi; k += blockDim.x) {
            const int sl = pcs_slot(s, rhash[k], true);
            if (sl < 0) {
                prim::set_error(err, QUIDS_ERR_TABLE_FULL);
                continue;
            }
            atomicMin(&s.rep[sl], ridx[k]);
            atomicAdd(&s.cnt[sl], 1u);
        }
        __syncthreads();
        // magnitudes: a group of one keeps its member's, others sum exactly
        for (uint64_t k = lo + threadIdx.x; k < hi; k += blockDim.x) {
            const int sl = pcs_slot(s, rhash[k], false);
            if (sl < 0) continue;
            const double2 m = rmag[k];
            if (s.cnt[sl] == 1) {
                s.sum[4 * sl] = (unsigned long long)__double_as_longlong(m.x);
                s.sum[4 * sl + 1] = (unsigned long long)__double_as_longlong(m.y);
            } else {
                smem_fix_add(&s.sum[4 * sl], to_fix(m.x, F));
                smem_fix_add(&s.sum[4 * sl + 2], to_fix(m.y, F));
            }
        }
        __syncthreads();
        // groups above tolerance: one record each, at a block-reserved range
        mag_t gm[kPer];
        uint32_t keep = 0, nkeep = 0;
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const int sl = threadIdx.x + q * kPcsThreads;
            if (sl > kPcsSlots || s.cnt[sl] == 0) continue;
            mag_t m;
            if (s.cnt[sl] == 1) {
                m = mag_t{__longlong_as_double((long long)s.sum[4 * sl]),
                          __longlong_as_double((long long)s.sum[4 * sl + 1])};
            } else {
                m = mag_t{from_fix(fix128{s.sum[4 * sl], s.sum[4 * sl + 1]}, F),
                          from_fix(fix128{s.sum[4 * sl + 2], s.sum[4 * sl + 3]}, F)};
            }
            gm[q] = m;
            if (cnorm(m) > tolerance) {
                keep |= 1u << q;
                ++nkeep;
            }
        }
        // exclusive scan of nkeep over the block's kPcsThreads threads
        uint32_t x = nkeep;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s.scan[warp] = x;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint64_t run = 0;
            for (int w = 0; w < kPcsThreads / 32; ++w) {
                const uint64_t t = s.scan[w];
                s.scan[w] = run;
                run += t;
            }
            s.base = run ? atomicAdd(d_nu, (unsigned long long)run) : 0;
        }
        __syncthreads();
        uint64_t at = s.base + s.scan[warp] + (x - nkeep);
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            if (!(keep & (1u << q))) continue;
            const int sl = threadIdx.x + q * kPcsThreads;
            const uint32_t c = s.rep[sl];
            out.child[at] = c;
            out.mag[at] = make_double2(gm[q].re, gm[q].im);
            if (out.key) out.key[at] = tk(cnorm(gm[q]), c);
            ++at;
        }
        __syncthreads();  // the table is cleared for the next bucket
    }
}

// Survivor marks in child-indexed bitmaps (32 children per word).  With a
// selection: key above the threshold -> keep; equal -> keep when every tie
// is kept, else tie (ranked in child order afterwards).  Without one, every
// group is kept.
struct pcs_bitmaps {
    unsigned int *keep;
    unsigned int *tie;
};
static __global__ void __launch_bounds__(prim::kThreads)
    k_pcs_mark(const uint32_t *gchild, const uint64_t *gkey, const unsigned long long *d_nu,
               const prim::select_state *st, pcs_bitmaps bm) {
    const uint64_t n = *d_nu;
    const bool active = gkey && st->active;
    const bool rank_ties = active && st->n_equal > st->k_rem;
    const uint64_t prefix = active ? st->prefix : 0;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = gchild[g];
        bool keep = true, tie = false;
        if (active) {
            const uint64_t k = gkey[g];
            keep = k > prefix || (k == prefix && !rank_ties);
            tie = k == prefix && rank_ties;
        }
        if (keep) atomicOr(&bm.keep[c >> 5], 1u << (c & 31));
        if (tie) atomicOr(&bm.tie[c >> 5], 1u << (c & 31));
    }
}
struct scan_popc {
    const unsigned int *w;
    __device__ uint64_t operator()(uint64_t i) const { return (uint64_t)__popc(w[i]); }
};
__device__ __forceinline__ uint64_t bit_rank(const unsigned int *w, const uint64_t *prefix, uint32_t c) {
    return prefix[c >> 5] + (uint64_t)__popc(w[c >> 5] & ((1u << (c & 31)) - 1u));
}
// the first k_rem ties in child order join the kept groups
static __global__ void __launch_bounds__(prim::kThreads)
    k_pcs_ties(const uint64_t *d_nw, const prim::select_state *st, pcs_bitmaps bm, const uint64_t *tie_prefix) {
    if (!(st->active && st->n_equal > st->k_rem)) return;
    const uint64_t nw = *d_nw, k_rem = st->k_rem;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += (uint64_t)gridDim.x * blockDim.x) {
        unsigned int w = bm.tie[i];
        if (!w) continue;
        uint64_t r = tie_prefix[i];
        unsigned int add = 0;
        while (w) {
            const int b = __ffs(w) - 1;
            w &= w - 1;
            if (r++ < k_rem) add |= 1u << b;
        }
        if (add) bm.keep[i] |= add;  // the tie and keep bits of a word are disjoint
    }
}
// survivor j = rank of its representative among the kept: magnitude, size,
// representative; the largest survivor norm (IEEE bits) for the total
static __global__ void __launch_bounds__(prim::kThreads)
    k_pcs_emit(const uint32_t *gchild, const double2 *gmag, const unsigned long long *d_nu, const unsigned int *keep,
               const uint64_t *keep_prefix, const uint32_t *csize, double2 *omag, uint32_t *osize, uint64_t *schild,
               unsigned long long *d_maxnorm) {
    const uint64_t n = *d_nu;
    unsigned long long mx = 0;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = gchild[g];
        if (!(keep[c >> 5] & (1u << (c & 31)))) continue;
        const uint64_t j = bit_rank(keep, keep_prefix, c);
        const double2 m = gmag[g];
        omag[j] = m;
        osize[j] = csize[c];
        schild[j] = c;
        const unsigned long long nb = (unsigned long long)__double_as_longlong(cnorm(mag_t{m.x, m.y}));
        mx = mx > nb ? mx : nb;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = mx > y ? mx : y;
    }
    if ((threadIdx.x & 31) == 0 && mx) atomicMax(d_maxnorm, mx);
}
struct scan_padded {
    const uint32_t *size;
    uint32_t align;
    __device__ uint64_t operator()(uint64_t i) const { return padded_size(size[i], align); }
};

// Buffers of the partitioned stage, in the context's scratch (reused ids:
// the region-ordered records hold the partitioned children, B_RSLOT/B_UMAG/
// B_UNORM the group records).
struct pcs_buffers {
    unsigned int *count, *cursor;
    uint64_t *boff;
    uint64_t *rhash;
    uint32_t *ridx;
    double2 *rmag;
    pcs_groups groups;
    pcs_bitmaps bm;
    uint64_t *keep_prefix, *tie_prefix;
    uint64_t nb, nw;
};
inline size_t pcs_smem_bytes() { return sizeof(pcs_smem); }
inline uint64_t pcs_words(uint64_t nc) { return (nc + 31) / 32; }

inline int pcs_ensure(quids_gpu_ctx *ctx, uint64_t nc, bool truncating) {
    const uint64_t nb = 1ull << pcs_bucket_bits(nc), nw = pcs_words(nc);
    QD_TRY(ensure(ctx->buf[B_RHIST], 2 * nb * sizeof(unsigned int)));
    QD_TRY(ensure(ctx->buf[B_ROFF], (nb + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_RHASH], nc * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_RIDX], nc * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_RMAG], nc * sizeof(double2)));
    QD_TRY(ensure(ctx->buf[B_RSLOT], nc * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_UMAG], nc * sizeof(double2)));
    if (truncating) QD_TRY(ensure(ctx->buf[B_UNORM], nc * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_BITMAP], 2 * (nw + 1) * sizeof(unsigned int)));
    QD_TRY(ensure(ctx->buf[B_BITPREFIX], 2 * (nw + 1) * sizeof(uint64_t)));
    return QUIDS_OK;
}
inline pcs_buffers pcs_view(quids_gpu_ctx *ctx, uint64_t nc, bool truncating) {
    pcs_buffers b{};
    b.nb = 1ull << pcs_bucket_bits(nc);
    b.nw = pcs_words(nc);
    b.count = bufp<unsigned int>(ctx, B_RHIST);
    b.cursor = b.count + b.nb;
    b.boff = bufp<uint64_t>(ctx, B_ROFF);
    b.rhash = bufp<uint64_t>(ctx, B_RHASH);
    b.ridx = bufp<uint32_t>(ctx, B_RIDX);
    b.rmag = bufp<double2>(ctx, B_RMAG);
    b.groups = pcs_groups{bufp<uint32_t>(ctx, B_RSLOT), bufp<double2>(ctx, B_UMAG),
                          truncating ? bufp<uint64_t>(ctx, B_UNORM) : nullptr};
    b.bm = pcs_bitmaps{bufp<unsigned int>(ctx, B_BITMAP), bufp<unsigned int>(ctx, B_BITMAP) + b.nw + 1};
    b.keep_prefix = bufp<uint64_t>(ctx, B_BITPREFIX);
    b.tie_prefix = b.keep_prefix + b.nw + 1;
    return b;
}

static __global__ void k_pcs_words(uint64_t *words, uint64_t nb, uint64_t nw) {
    words[W_PCSNB] = nb;
    words[W_PCSNW] = nw;
}

// Stages 2-4 of a one-pass step by partition, all on the context's stream
// with the counts on the device: nc_bound bounds the children (the host's
// count, or a planned run's bound); a truncation to maxc is possible when
// `truncating`.  Leaves N_u, N_s, the output bytes and the largest survivor
// norm in the step's words, the survivors' magnitudes, sizes, offsets and
// representatives in `out` and B_SCHILD; pb publishes the words (and `hook`
// runs) when the offsets are done.  The buffers come from pcs_ensure.
template <class L = prim::no_last>
inline int pcs_stage(quids_gpu_ctx *ctx, uint64_t nc_bound, bool truncating, uint64_t maxc, const trunc_key &tk,
                     double tolerance, uint32_t align, quids_gpu_state *out, const prim::publish &pb,
                     const L &hook = L{}) {
    const pcs_buffers b = pcs_view(ctx, nc_bound, truncating);
    const int bits = pcs_bucket_bits(nc_bound);
    uint64_t *words = ctx->d_words;
    int *err = (int *)(words + W_STATUS);
    const uint64_t tiles = (nc_bound + prim::kTile - 1) / prim::kTile;
    {  // bucket counts and cursors, bitmaps, look-back chains 0-3
        fill_set f{};
        f.p[0] = (unsigned char *)b.count, f.n[0] = 2 * b.nb * sizeof(unsigned int), f.v[0] = 0;
        f.p[1] = (unsigned char *)b.bm.keep, f.n[1] = 2 * (b.nw + 1) * sizeof(unsigned int), f.v[1] = 0;
        f.p[2] = bufp<unsigned char>(ctx, B_LOOKBACK), f.n[2] = 4 * (tiles + 2) * sizeof(uint64_t), f.v[2] = 0;
        f.count = 3;
        QD_TRY(fill(ctx, f));
    }
    k_pcs_words<<<1, 1, 0, ctx->stream>>>(words, b.nb, b.nw);
    k_pcs_count<<<grid_for(ctx, nc_bound), prim::kThreads, 0, ctx->stream>>>(bufp<uint64_t>(ctx, B_HASH),
                                                                            words + W_NC, bits, b.count);
    QD_TRY(launched(ctx, 2));
    prim::lookback lb[4];
    for (int k = 0; k < 4; ++k) lookback_view(ctx, nc_bound, k, lb[k]);
    prim::k_scan_excl<<<lookback_grid(ctx, b.nb), prim::kThreads, 0, ctx->stream>>>(
        scan_count{b.count}, words + W_PCSNB, b.boff, (uint64_t *)nullptr, lb[0]);
    k_pcs_scatter<<<grid_for(ctx, nc_bound), prim::kThreads, 0, ctx->stream>>>(
        bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG), words + W_NC, bits, b.boff, b.cursor, b.rhash,
        b.ridx, b.rmag, err);
    QD_TRY(launched(ctx, 2));
    const size_t smem = pcs_smem_bytes();
    QD_CUDA(cudaFuncSetAttribute(k_pcs_group, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const uint64_t gw = (uint64_t)ctx->num_sms * resident_per_sm(k_pcs_group, kPcsThreads, smem);
    k_pcs_group<<<(unsigned)std::min<uint64_t>(b.nb, gw), kPcsThreads, smem, ctx->stream>>>(
        b.rhash, b.ridx, b.rmag, b.boff, (uint32_t)b.nb, words + W_NC, (const unsigned long long *)(words + W_MAXABS),
        tolerance, tk, b.groups, (unsigned long long *)(words + W_NU), err);
    QD_TRY(launched(ctx));
    const uint64_t *d_nu = words + W_NU;
    if (truncating) {
        QD_TRY(ensure(ctx->buf[B_SELCAND], filter_cap(nc_bound) * sizeof(uint64_t)));
        QD_TRY(radix_select_filtered(ctx, d_nu, nc_bound, maxc, key_direct{b.groups.key},
                                     bufp<uint64_t>(ctx, B_SELCAND), filter_cap(nc_bound), d_nu));
    }
    k_pcs_mark<<<grid_for(ctx, nc_bound), prim::kThreads, 0, ctx->stream>>>(
        b.groups.child, truncating ? b.groups.key : nullptr, (const unsigned long long *)d_nu, ctx->d_sel, b.bm);
    QD_TRY(launched(ctx));
    if (truncating) {
        prim::k_scan_excl<<<lookback_grid(ctx, b.nw), prim::kThreads, 0, ctx->stream>>>(
            scan_popc{b.bm.tie}, words + W_PCSNW, b.tie_prefix, (uint64_t *)nullptr, lb[1]);
        k_pcs_ties<<<grid_for(ctx, b.nw), prim::kThreads, 0, ctx->stream>>>(words + W_PCSNW, ctx->d_sel, b.bm,
                                                                         b.tie_prefix);
        QD_TRY(launched(ctx, 2));
    }
    prim::k_scan_excl<<<lookback_grid(ctx, b.nw), prim::kThreads, 0, ctx->stream>>>(
        scan_popc{b.bm.keep}, words + W_PCSNW, b.keep_prefix, words + W_NS, lb[2]);
    k_pcs_emit<<<grid_for(ctx, nc_bound), prim::kThreads, 0, ctx->stream>>>(
        b.groups.child, b.groups.mag, (const unsigned long long *)d_nu, b.bm.keep, b.keep_prefix,
        bufp<uint32_t>(ctx, B_CSIZE), (double2 *)out->mag.p, (uint32_t *)out->size.p, bufp<uint64_t>(ctx, B_SCHILD),
        (unsigned long long *)(words + W_MAXNORM));
    QD_TRY(launched(ctx, 2));
    prim::k_scan_excl<<<lookback_grid(ctx, nc_bound), prim::kThreads, 0, ctx->stream>>>(
        scan_padded{(const uint32_t *)out->size.p, align}, words + W_NS, (uint64_t *)out->begin.p,
        words + W_OUTBYTES, lb[3], prim::no_epilogue{}, pb, hook);
    return launched(ctx);
}
