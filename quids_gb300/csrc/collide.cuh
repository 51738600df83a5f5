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
//  1. k_pcs_count, a scan, then two scatters: the children's (hash, index,
//     magnitude) records are partitioned by hash into buckets of one to two
//     thousand records.  A single scatter into that many buckets keeps too
//     many partly written sectors open for L2 to combine them, so the first
//     scatter goes to at most 1024 level-1 buckets (tiles reserve their runs
//     with one atomic per bucket), the second splits each level-1 bucket,
//     whose records L2 then holds; the counts and cursors sit in L2;
//  2. k_pcs_group: one block per bucket groups its records in a
//     shared-memory table: representative = the lowest child index (atomic
//     minimum), magnitude = the member's own for a group of one, else the
//     exact 128-bit fixed-point sum with the table path's scale, rounded
//     once -- the same bits as the table path (the sums go to the block's
//     own scratch, which L2 holds); groups of norm above tolerance leave one
//     record (representative, magnitude, truncation key) at the bucket's
//     positions, the rest of the bucket's positions are marked empty;
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

constexpr int kPcsThreads = 512;            // block of the grouping kernel
constexpr int kPcsSlots = 4096;             // its shared-memory table (distinct hashes per bucket)
constexpr int kPcsHomeBits = 12;
constexpr uint64_t kPcsBucketTarget = 1536; // largest mean of children per bucket
constexpr int kPcsMaxBits = 24;
constexpr int kPcsL1Bits = 10;              // level-1 buckets of the first scatter: at most 1024
constexpr int kPcsScatterItems = 16;        // records per thread of a first-scatter tile
constexpr uint32_t kPcsEmpty = 0xffffffffu; // a bucket position that holds no group
static_assert(kPcsSlots == 1 << kPcsHomeBits, "table size");

inline int pcs_bucket_bits(uint64_t nc) {
    int bits = 0;
    while (bits < kPcsMaxBits && (kPcsBucketTarget << bits) < nc) ++bits;
    return bits;
}
inline int pcs_l1_bits(int bits) { return bits < kPcsL1Bits ? bits : kPcsL1Bits; }
__device__ __forceinline__ uint32_t pcs_bucket(uint64_t h, int bits) {
    return bits ? (uint32_t)((h * 0x9E3779B97F4A7C15ull) >> (64 - bits)) : 0u;
}
// home slot in the block's table, from bits the bucket does not fix
__device__ __forceinline__ uint32_t pcs_home(uint64_t h) {
    return (uint32_t)(((h ^ (h >> 31)) * 0xBF58476D1CE4E5B9ull) >> (64 - kPcsHomeBits));
}

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

// The children's records, level-1 bucket order.  A tile of kThreads x
// kPcsScatterItems children counts its records per level-1 bucket in shared
// memory and reserves each bucket's run with one atomic; level-1 bucket g
// starts where its first bucket starts (boff[g << l2bits]).
static __global__ void __launch_bounds__(prim::kThreads)
    k_pcs_scatter1(const uint64_t *hash, const double2 *mag, const uint64_t *d_n, int bits, int l2bits,
                   const uint64_t *boff, unsigned long long *cursor1, uint64_t *lhash, uint32_t *lidx, double2 *lmag,
                   int *err) {
    __shared__ unsigned int s_cnt[1 << kPcsL1Bits];
    __shared__ unsigned long long s_base[1 << kPcsL1Bits];
    const uint64_t n = *d_n;
    const int lane = threadIdx.x & 31;
    const uint32_t ng = 1u << (bits - l2bits);
    constexpr uint64_t kTileN = (uint64_t)prim::kThreads * kPcsScatterItems;
    const uint64_t ntiles = (n + kTileN - 1) / kTileN;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        for (uint32_t i = threadIdx.x; i < ng; i += blockDim.x) s_cnt[i] = 0;
        __syncthreads();
        const uint64_t base = tile * kTileN;
        uint32_t grp[kPcsScatterItems], rank[kPcsScatterItems];
#pragma unroll
        for (int k = 0; k < kPcsScatterItems; ++k) {
            const uint64_t c = base + threadIdx.x + (uint64_t)k * prim::kThreads;
            const uint32_t g = c < n ? pcs_bucket(hash[c], bits) >> l2bits : 0xffffffffu;
            const unsigned same = __match_any_sync(0xffffffffu, g);
            const int leader = __ffs(same) - 1;
            unsigned first = 0;
            if (g != 0xffffffffu && lane == leader) first = atomicAdd(&s_cnt[g], (unsigned)__popc(same));
            first = __shfl_sync(0xffffffffu, first, leader);
            grp[k] = g;
            rank[k] = first + (unsigned)__popc(same & ((1u << lane) - 1));
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < ng; i += blockDim.x)
            if (s_cnt[i]) s_base[i] = boff[(uint64_t)i << l2bits] + atomicAdd(&cursor1[i], (unsigned long long)s_cnt[i]);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kPcsScatterItems; ++k) {
            const uint64_t c = base + threadIdx.x + (uint64_t)k * prim::kThreads;
            if (c >= n) break;
            const uint32_t g = grp[k];
            const uint64_t pos = s_base[g] + rank[k];
            if (pos >= boff[(uint64_t)(g + 1) << l2bits]) {  // counts and cursors disagree
                prim::set_error(err, QUIDS_ERR_CUDA);
                continue;
            }
            lhash[pos] = hash[c];
            lidx[pos] = (uint32_t)c;
            lmag[pos] = mag[c];
        }
        __syncthreads();
    }
}
// The records in bucket order, from level-1 order: the blocks in flight read
// about one level-1 bucket, whose buckets' runs L2 then holds.
static __global__ void __launch_bounds__(prim::kThreads)
    k_pcs_scatter2(const uint64_t *lhash, const uint32_t *lidx, const double2 *lmag, const uint64_t *d_n, int bits,
                   const uint64_t *boff, unsigned int *cursor, uint64_t *fhash, uint32_t *fidx, double2 *fmag,
                   int *err) {
    const uint64_t n = *d_n;
    const int lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint64_t k = base + threadIdx.x;
        uint64_t h = 0;
        uint32_t b = 0xffffffffu;
        if (k < n) {
            h = lhash[k];
            b = pcs_bucket(h, bits);
        }
        const unsigned same = __match_any_sync(0xffffffffu, b);
        const int leader = __ffs(same) - 1;
        unsigned first = 0;
        if (b != 0xffffffffu && lane == leader) first = atomicAdd(&cursor[b], (unsigned)__popc(same));
        first = __shfl_sync(0xffffffffu, first, leader);
        if (b == 0xffffffffu) continue;
        const uint64_t pos = boff[b] + first + (unsigned)__popc(same & ((1u << lane) - 1));
        if (pos >= boff[b + 1]) {
            prim::set_error(err, QUIDS_ERR_CUDA);
            continue;
        }
        fhash[pos] = h;
        fidx[pos] = lidx[k];
        fmag[pos] = lmag[k];
    }
}

// What the grouping kernel leaves at each bucket position: a group
// (representative = lowest child index, magnitude, truncation key) or
// child = kPcsEmpty (key 0).
struct pcs_groups {
    uint32_t *child;
    double2 *mag;
    uint64_t *key;  // null: no truncation possible
};

// Shared memory of the grouping kernel: kPcsSlots + 1 slots (the extra one
// for the hash kEmptyKey, which the table cannot hold as a key): key, lowest
// child index, member count, and the bucket position of the first member.
struct pcs_smem {
    unsigned long long key[kPcsSlots + 1];
    unsigned int rep[kPcsSlots + 1];
    unsigned int cnt[kPcsSlots + 1];
    unsigned int first[kPcsSlots + 1];
    unsigned int scan[kPcsThreads / 32];
    unsigned int total;
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

// exclusive scan of v over the block (kPcsThreads threads); total = the sum
__device__ __forceinline__ uint32_t pcs_block_scan(pcs_smem &s, uint32_t v, uint32_t &total) {
    constexpr int kWarps = kPcsThreads / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s.scan[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < kWarps ? s.scan[lane] : 0;
        uint32_t inc = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane < kWarps) s.scan[lane] = inc - w;
        if (lane == kWarps - 1) s.total = inc;
    }
    __syncthreads();
    total = s.total;
    return s.scan[warp] + x - v;
}

// a group's magnitude: the single member's, or the exact sum (the block's
// scratch words are cleared for the next bucket when `clear`)
__device__ __forceinline__ mag_t pcs_group_mag(const pcs_smem &s, int sl, const double2 *fmag,
                                               unsigned long long *acc, int F, bool clear) {
    if (s.cnt[sl] == 1) {
        const double2 m = fmag[s.first[sl]];
        return mag_t{m.x, m.y};
    }
    unsigned long long *w = acc + 4ull * sl;
    const mag_t m{from_fix(fix128{w[0], w[1]}, F), from_fix(fix128{w[2], w[3]}, F)};
    if (clear) w[0] = w[1] = w[2] = w[3] = 0;
    return m;
}

static __global__ void __launch_bounds__(kPcsThreads)
    k_pcs_group(const uint64_t *fhash, const uint32_t *fidx, const double2 *fmag, const uint64_t *boff, uint32_t nb,
                const uint64_t *d_nc, const unsigned long long *d_maxabs, double tolerance, trunc_key tk,
                unsigned long long *scratch, pcs_groups out, unsigned long long *d_nu, int *err) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    pcs_smem &s = *(pcs_smem *)s_raw;
    unsigned long long *acc = scratch + (uint64_t)blockIdx.x * 4 * (kPcsSlots + 1);  // this block's sums (zeroed)
    const int F = fix_scale(__longlong_as_double((long long)*d_maxabs), *d_nc);
    constexpr int kPer = (kPcsSlots + 1 + kPcsThreads - 1) / kPcsThreads;  // slots per thread in the emit
    unsigned long long groups = 0;  // kept groups of this block (thread 0)
    for (uint32_t b = blockIdx.x; b < nb; b += gridDim.x) {
        const uint64_t lo = boff[b], hi = boff[b + 1];
        if (lo == hi) continue;
        for (int i = threadIdx.x; i <= kPcsSlots; i += blockDim.x) {
            s.key[i] = prim::kEmptyKey;
            s.rep[i] = 0xffffffffu;
            s.cnt[i] = 0;
        }
        __syncthreads();
        // members: slot, lowest child index, count, first member
        for (uint64_t k = lo + threadIdx.x; k < hi; k += blockDim.x) {
            const int sl = pcs_slot(s, fhash[k], true);
            if (sl < 0) {
                prim::set_error(err, QUIDS_ERR_TABLE_FULL);
                continue;
            }
            atomicMin(&s.rep[sl], fidx[k]);
            if (atomicAdd(&s.cnt[sl], 1u) == 0) s.first[sl] = (uint32_t)k;
        }
        __syncthreads();
        // groups of several members: exact sums in the block's scratch
        for (uint64_t k = lo + threadIdx.x; k < hi; k += blockDim.x) {
            const int sl = pcs_slot(s, fhash[k], false);
            if (sl < 0 || s.cnt[sl] < 2) continue;
            const double2 m = fmag[k];
            prim::fix_atomic_add(&acc[4ull * sl], to_fix(m.x, F));
            prim::fix_atomic_add(&acc[4ull * sl + 2], to_fix(m.y, F));
        }
        __syncthreads();
        // groups above tolerance, at the bucket's first positions
        uint32_t keep = 0, nkeep = 0;
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const int sl = threadIdx.x + q * kPcsThreads;
            if (sl > kPcsSlots || s.cnt[sl] == 0) continue;
            const mag_t m = pcs_group_mag(s, sl, fmag, acc, F, false);
            if (cnorm(m) > tolerance) {
                keep |= 1u << q;
                ++nkeep;
            }
        }
        uint32_t total = 0;
        uint64_t at = lo + pcs_block_scan(s, nkeep, total);
        if (threadIdx.x == 0) groups += total;
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const int sl = threadIdx.x + q * kPcsThreads;
            if (sl > kPcsSlots || s.cnt[sl] == 0) continue;
            const mag_t m = pcs_group_mag(s, sl, fmag, acc, F, true);
            if (!(keep & (1u << q))) continue;
            const uint32_t c = s.rep[sl];
            out.child[at] = c;
            out.mag[at] = make_double2(m.re, m.im);
            if (out.key) out.key[at] = tk(cnorm(m), c);
            ++at;
        }
        for (uint64_t k = lo + total + threadIdx.x; k < hi; k += blockDim.x) {
            out.child[k] = kPcsEmpty;
            if (out.key) out.key[k] = 0;
        }
        __syncthreads();  // the table and the scratch are clear for the next bucket
    }
    if (threadIdx.x == 0 && groups) atomicAdd(d_nu, groups);
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
    k_pcs_mark(const uint32_t *gchild, const uint64_t *gkey, const uint64_t *d_n, const prim::select_state *st,
               pcs_bitmaps bm) {
    const uint64_t n = *d_n;
    const bool active = gkey && st->active;
    const bool rank_ties = active && st->n_equal > st->k_rem;
    const uint64_t prefix = active ? st->prefix : 0;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (uint64_t)gridDim.x * blockDim.x) {
        bool keep = true, tie = false;
        if (active) {
            const uint64_t k = gkey[g];
            if (k < prefix) continue;
            keep = k > prefix || !rank_ties;
            tie = !keep;
        }
        const uint32_t c = gchild[g];
        if (c == kPcsEmpty) continue;
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
    k_pcs_emit(const uint32_t *gchild, const double2 *gmag, const uint64_t *gkey, const uint64_t *d_n,
               const prim::select_state *st, const unsigned int *keep, const uint64_t *keep_prefix,
               const uint32_t *csize, double2 *omag, uint32_t *osize, uint64_t *schild, unsigned long long *d_maxnorm) {
    const uint64_t n = *d_n;
    const uint64_t prefix = gkey && st->active ? st->prefix : 0;
    unsigned long long mx = 0;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (uint64_t)gridDim.x * blockDim.x) {
        if (prefix && gkey[g] < prefix) continue;  // below the cutoff: not kept
        const uint32_t c = gchild[g];
        if (c == kPcsEmpty || !(keep[c >> 5] & (1u << (c & 31)))) continue;
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

// Buffers of the partitioned stage, in the context's scratch.  The child-
// ordered hashes and magnitudes (B_HASH, B_CMAG) are read once, by the first
// scatter, and then hold the bucket-ordered records; the level-1 records
// (B_RHASH, B_RIDX, B_RMAG) then hold the group records; B_ACC the grouping
// blocks' sums.
struct pcs_buffers {
    unsigned int *count, *cursor;
    unsigned long long *cursor1;
    uint64_t *boff;
    uint64_t *lhash;
    uint32_t *lidx;
    double2 *lmag;
    uint32_t *fidx;
    unsigned long long *scratch;
    pcs_groups groups;
    pcs_bitmaps bm;
    uint64_t *keep_prefix, *tie_prefix;
    uint64_t nb, nw;
};
inline size_t pcs_smem_bytes() { return sizeof(pcs_smem); }
inline uint64_t pcs_words(uint64_t nc) { return (nc + 31) / 32; }
// grouping blocks: two per SM (the shared-memory table takes 80 KB)
inline uint64_t pcs_group_blocks(quids_gpu_ctx *ctx) { return 2ull * (uint64_t)ctx->num_sms; }

inline int pcs_ensure(quids_gpu_ctx *ctx, uint64_t nc, bool truncating) {
    const uint64_t nb = 1ull << pcs_bucket_bits(nc), nw = pcs_words(nc);
    QD_TRY(ensure(ctx->buf[B_RHIST], 2 * nb * sizeof(unsigned int)));
    QD_TRY(ensure(ctx->buf[B_RCUR], (1ull << kPcsL1Bits) * sizeof(unsigned long long)));
    QD_TRY(ensure(ctx->buf[B_ROFF], (nb + 1) * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_RHASH], nc * sizeof(uint64_t)));
    QD_TRY(ensure(ctx->buf[B_RIDX], nc * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_RMAG], nc * sizeof(double2)));
    QD_TRY(ensure(ctx->buf[B_SLOT], nc * sizeof(uint32_t)));
    QD_TRY(ensure(ctx->buf[B_ACC], pcs_group_blocks(ctx) * 4 * (kPcsSlots + 1) * sizeof(unsigned long long)));
    QD_TRY(ensure(ctx->buf[B_BITMAP], 2 * (nw + 1) * sizeof(unsigned int)));
    QD_TRY(ensure(ctx->buf[B_BITPREFIX], 2 * (nw + 1) * sizeof(uint64_t)));
    (void)truncating;
    return QUIDS_OK;
}
inline pcs_buffers pcs_view(quids_gpu_ctx *ctx, uint64_t nc, bool truncating) {
    pcs_buffers b{};
    b.nb = 1ull << pcs_bucket_bits(nc);
    b.nw = pcs_words(nc);
    b.count = bufp<unsigned int>(ctx, B_RHIST);
    b.cursor = b.count + b.nb;
    b.cursor1 = bufp<unsigned long long>(ctx, B_RCUR);
    b.boff = bufp<uint64_t>(ctx, B_ROFF);
    b.lhash = bufp<uint64_t>(ctx, B_RHASH);
    b.lidx = bufp<uint32_t>(ctx, B_RIDX);
    b.lmag = bufp<double2>(ctx, B_RMAG);
    b.fidx = bufp<uint32_t>(ctx, B_SLOT);
    b.scratch = bufp<unsigned long long>(ctx, B_ACC);
    b.groups = pcs_groups{b.lidx, b.lmag, truncating ? b.lhash : nullptr};
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
    const int bits = pcs_bucket_bits(nc_bound), l2bits = bits - pcs_l1_bits(bits);
    uint64_t *words = ctx->d_words;
    int *err = (int *)(words + W_STATUS);
    const uint64_t tiles = (nc_bound + prim::kTile - 1) / prim::kTile;
    const uint64_t gblocks = pcs_group_blocks(ctx);
    {  // bucket counts and cursors, level-1 cursors, the grouping blocks' sums, bitmaps, look-back chains 0-3
        fill_set f{};
        f.p[0] = (unsigned char *)b.count, f.n[0] = 2 * b.nb * sizeof(unsigned int), f.v[0] = 0;
        f.p[1] = (unsigned char *)b.cursor1, f.n[1] = (1ull << kPcsL1Bits) * sizeof(unsigned long long), f.v[1] = 0;
        f.p[2] = (unsigned char *)b.scratch, f.n[2] = gblocks * 4 * (kPcsSlots + 1) * 8, f.v[2] = 0;
        f.p[3] = (unsigned char *)b.bm.keep, f.n[3] = 2 * (b.nw + 1) * sizeof(unsigned int), f.v[3] = 0;
        f.p[4] = bufp<unsigned char>(ctx, B_LOOKBACK), f.n[4] = 4 * (tiles + 2) * sizeof(uint64_t), f.v[4] = 0;
        f.count = 5;
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
    const uint64_t tiles1 = (nc_bound + (uint64_t)prim::kThreads * kPcsScatterItems - 1) /
                            ((uint64_t)prim::kThreads * kPcsScatterItems);
    const unsigned g1 = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(tiles1, (uint64_t)ctx->num_sms * 4));
    k_pcs_scatter1<<<g1, prim::kThreads, 0, ctx->stream>>>(
        bufp<uint64_t>(ctx, B_HASH), bufp<double2>(ctx, B_CMAG), words + W_NC, bits, l2bits, b.boff, b.cursor1,
        b.lhash, b.lidx, b.lmag, err);
    k_pcs_scatter2<<<grid_for(ctx, nc_bound), prim::kThreads, 0, ctx->stream>>>(
        b.lhash, b.lidx, b.lmag, words + W_NC, bits, b.boff, b.cursor, bufp<uint64_t>(ctx, B_HASH), b.fidx,
        bufp<double2>(ctx, B_CMAG), err);
    QD_TRY(launched(ctx, 3));
    const size_t smem = pcs_smem_bytes();
    if (!g_alloc_frozen)  // (a planned run sets it before its capture)
        QD_CUDA(cudaFuncSetAttribute(k_pcs_group, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_pcs_group<<<(unsigned)std::min<uint64_t>(b.nb, gblocks), kPcsThreads, smem, ctx->stream>>>(
        bufp<uint64_t>(ctx, B_HASH), b.fidx, bufp<double2>(ctx, B_CMAG), b.boff, (uint32_t)b.nb, words + W_NC,
        (const unsigned long long *)(words + W_MAXABS), tolerance, tk, b.scratch, b.groups,
        (unsigned long long *)(words + W_NU), err);
    QD_TRY(launched(ctx));
    const uint64_t *d_nc = words + W_NC;
    if (truncating) {
        QD_TRY(ensure(ctx->buf[B_SELCAND], filter_cap(nc_bound) * sizeof(uint64_t)));
        QD_TRY(radix_select_filtered(ctx, d_nc, nc_bound, maxc, key_direct{b.groups.key},
                                     bufp<uint64_t>(ctx, B_SELCAND), filter_cap(nc_bound), words + W_NU));
    }
    k_pcs_mark<<<grid_for(ctx, nc_bound), prim::kThreads, 0, ctx->stream>>>(
        b.groups.child, truncating ? b.groups.key : nullptr, d_nc, ctx->d_sel, b.bm);
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
        b.groups.child, b.groups.mag, truncating ? b.groups.key : nullptr, d_nc, ctx->d_sel, b.bm.keep,
        b.keep_prefix, bufp<uint32_t>(ctx, B_CSIZE), (double2 *)out->mag.p, (uint32_t *)out->size.p,
        bufp<uint64_t>(ctx, B_SCHILD), (unsigned long long *)(words + W_MAXNORM));
    QD_TRY(launched(ctx, 2));
    prim::k_scan_excl<<<lookback_grid(ctx, nc_bound), prim::kThreads, 0, ctx->stream>>>(
        scan_padded{(const uint32_t *)out->size.p, align}, words + W_NS, (uint64_t *)out->begin.p,
        words + W_OUTBYTES, lb[3], prim::no_epilogue{}, pb, hook);
    return launched(ctx);
}
