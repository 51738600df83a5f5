// prims.cuh -- rule-independent device primitives of the rule step:
//   * single-pass scan and stream compaction with decoupled look-back
//     (tiles taken in order from an atomic counter, bounded waits),
//   * top-k radix select on 64-bit keys,
//   * the collision table (open addressing, 64-bit keys, exact fixed-point
//     magnitude sums),
//   * deterministic normalisation.
// Every wait on another block is bounded: on expiry it records
// QUIDS_ERR_TIMEOUT in the status word and the kernel returns.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/quids_gpu.h"
#include "qd_common.cuh"

namespace qd::prim {

constexpr int kThreads = 256;
constexpr int kMaxTableThreads = 512;  // block size bound of the collision-table passes (a tuning knob)
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;
constexpr uint64_t kFlagAgg = 1ull << 62;
constexpr uint64_t kFlagInc = 2ull << 62;
constexpr uint64_t kValMask = (1ull << 62) - 1;
constexpr uint32_t kSpinLimit = 1u << 22;  // x ~64 ns sleep: well under a second
constexpr uint64_t kEmptyKey = ~0ull;

__device__ __forceinline__ void set_error(int *err, int code) { atomicCAS(err, 0, code); }

__device__ __forceinline__ uint64_t warp_sum(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ uint64_t ld_volatile_u64(const uint64_t *p) {
    return *(const volatile uint64_t *)p;
}
__device__ __forceinline__ void st_volatile_u64(uint64_t *p, uint64_t v) { *(volatile uint64_t *)p = v; }

// Block-wide exclusive scan of one u64 per thread; returns the exclusive
// value, writes the block total to *total.  Uses `sm` (kThreads/32 + 1 u64).
__device__ __forceinline__ uint64_t block_excl_scan(uint64_t v, uint64_t *sm, uint64_t &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sm[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint64_t w = lane < kThreads / 32 ? sm[lane] : 0;
        uint64_t s = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kThreads / 32) sm[lane] = s - w;
        if (lane == kThreads / 32 - 1) sm[kThreads / 32] = s;
    }
    __syncthreads();
    uint64_t r = sm[warp] + x - v;
    total = sm[kThreads / 32];
    __syncthreads();
    return r;
}

struct lookback {
    uint64_t *status;   // one word per tile, zeroed before the launch
    uint32_t *counter;  // tile ticket, zeroed before the launch
    int *err;
    // failure injection (QUIDS_DEBUG_STALL_LOOKBACK): this tile never
    // publishes, so the next tile's bounded wait runs out (~0: none)
    uint32_t stall_tile = 0xffffffffu;
};

// Warp-level decoupled look-back of tile `tile` (> 0): publishes its
// aggregate, sums its predecessors' values back to the nearest inclusive one,
// publishes its own inclusive value and returns its exclusive prefix (in every
// lane).  Each round looks at 32 * kLookWindow predecessors, every lane
// loading kLookWindow status words at once (measured on GB300: a window of
// 128 tiles was slower than 32, the nearest inclusive value being usually
// close).  Waits are bounded (kSpinLimit polls): a wait that runs out records
// QUIDS_ERR_TIMEOUT and counts the tile as an inclusive zero.
constexpr int kLookWindow = 1;
static __device__ uint64_t warp_lookback(const lookback &lb, uint32_t tile, uint64_t aggregate) {
    const int lane = threadIdx.x & 31;
    if (tile == lb.stall_tile) return 0;  // injected failure: publishes nothing
    if (lane == 0) st_volatile_u64(&lb.status[tile], kFlagAgg | (aggregate & kValMask));
    int64_t base = (int64_t)tile - 1;
    uint64_t prefix = 0;
    bool failed = false;
    while (true) {
        uint64_t s[kLookWindow];
#pragma unroll
        for (int r = 0; r < kLookWindow; ++r) {
            const int64_t j = base - lane - 32 * r;
            s[r] = j >= 0 ? ld_volatile_u64(&lb.status[j]) : kFlagInc;  // before tile 0: an inclusive 0
        }
#pragma unroll
        for (int r = 0; r < kLookWindow; ++r) {
            const int64_t j = base - lane - 32 * r;
            uint32_t it = 0;
            while ((s[r] >> 62) == 0 && ++it < kSpinLimit) {
                __nanosleep(64);
                s[r] = ld_volatile_u64(&lb.status[j]);
            }
            if ((s[r] >> 62) == 0) {
                failed = true;
                s[r] = kFlagInc;
            }
        }
        bool done = false;  // uniform over the warp
#pragma unroll
        for (int r = 0; r < kLookWindow; ++r) {
            if (!done) {
                const unsigned inc = __ballot_sync(0xffffffffu, (s[r] >> 62) == 2);
                uint64_t v = s[r] & kValMask;
                if (inc) {
                    if (lane > __ffs(inc) - 1) v = 0;  // beyond the nearest inclusive value
                    done = true;
                }
                prefix += warp_sum(v);
            }
        }
        if (done) break;
        base -= 32 * kLookWindow;
    }
    if (__any_sync(0xffffffffu, failed) && lane == 0) set_error(lb.err, QUIDS_ERR_TIMEOUT);
    if (lane == 0) st_volatile_u64(&lb.status[tile], kFlagInc | ((prefix + aggregate) & kValMask));
    return prefix;
}

// Exclusive prefix of tile `tile` given its aggregate; all threads call it.
static __device__ uint64_t tile_prefix(const lookback &lb, uint32_t tile, uint64_t aggregate, uint64_t *bcast) {
    if (threadIdx.x < 32) {
        uint64_t prefix = 0;
        if (tile == 0) {
            if (threadIdx.x == 0) st_volatile_u64(&lb.status[0], kFlagInc | (aggregate & kValMask));
        } else {
            prefix = warp_lookback(lb, tile, aggregate);
        }
        if (threadIdx.x == 0) *bcast = prefix;
    }
    __syncthreads();
    uint64_t p = *bcast;
    __syncthreads();
    return p;
}

// Exclusive prefixes of one tile on two chains at once: warp 0 looks back on
// chain a while warp 1 looks back on chain b.
static __device__ void tile_prefix2(const lookback &la, uint64_t agg_a, const lookback &lbb, uint64_t agg_b,
                                    uint32_t tile, uint64_t *bcast2, uint64_t &pa, uint64_t &pb) {
    const int warp = threadIdx.x >> 5;
    if (warp < 2) {
        const lookback &lb = warp == 0 ? la : lbb;
        const uint64_t aggregate = warp == 0 ? agg_a : agg_b;
        const int lane = threadIdx.x & 31;
        uint64_t prefix = 0;
        if (tile == 0) {
            if (lane == 0) st_volatile_u64(&lb.status[0], kFlagInc | (aggregate & kValMask));
        } else {
            prefix = warp_lookback(lb, tile, aggregate);
        }
        if (lane == 0) bcast2[warp] = prefix;
    }
    __syncthreads();
    pa = bcast2[0];
    pb = bcast2[1];
    __syncthreads();
}

__device__ __forceinline__ uint32_t next_tile(const lookback &lb, uint32_t *sm_tile) {
    if (threadIdx.x == 0) *sm_tile = atomicAdd(lb.counter, 1u);
    __syncthreads();
    uint32_t t = *sm_tile;
    __syncthreads();
    return t;
}

// --------------------------------------------------------------- scan
// out[i] = sum_{j<i} f(j) for i in [0, n], *total = sum; f(i) is called
// exactly once per item (it may have side effects, e.g. gathers).
// A kernel's last block to finish copies `count` words of the step into
// mapped host memory and then writes `seq` after them, so the host learns
// the step's counts without a separate launch (host == nullptr: nothing).
// `done` is a block counter zeroed beforehand.
struct publish {
    const uint64_t *words = nullptr;
    volatile uint64_t *host = nullptr;
    uint32_t count = 0;
    uint64_t seq = 0;
    unsigned int *done = nullptr;
};
// A last-block hook L (L::active): one thread of the kernel's last block to
// finish runs last() once every other block is done (before the words are
// published), so a follow-up that needs the whole kernel's results costs no
// launch.  It needs pb.done even when nothing is published.
struct no_last {
    static constexpr bool active = false;
    __device__ void operator()() const {}
};
template <class L = no_last>
__device__ __forceinline__ void publish_at_exit(const publish &pb, const L &hook = L{}) {
    __shared__ bool last;
    if (!pb.host && !L::active) return;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(pb.done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) {
        __threadfence();
        if constexpr (L::active) {
            if (threadIdx.x == 0) {
                hook();
                __threadfence();
            }
            __syncthreads();
        }
        if (!pb.host) return;
        for (uint32_t i = threadIdx.x; i < pb.count; i += blockDim.x)
            pb.host[i] = ((const volatile uint64_t *)pb.words)[i];
        __threadfence_system();
        __syncthreads();
        if (threadIdx.x == 0) pb.host[pb.count] = pb.seq;
    }
}

struct no_epilogue {
    __device__ __forceinline__ void operator()(uint64_t, uint64_t, uint64_t, uint64_t) const {}
};

// E::operator()(i, out[i], f(i), n) runs once per item after its prefix is known.
template <class F, class E = no_epilogue, class L = no_last>
__global__ void __launch_bounds__(kThreads) k_scan_excl(F f, const uint64_t *d_n, uint64_t *out,
                                                         uint64_t *d_total, lookback lb, E epi = E{},
                                                         publish pb = publish{}, L hook = L{}) {
    __shared__ uint64_t sm[kThreads / 32 + 1];
    __shared__ uint64_t bcast;
    __shared__ uint32_t sm_tile;
    const uint64_t n = *d_n;
    const uint64_t ntiles = (n + kTile - 1) / kTile;
    if (n == 0 && blockIdx.x == 0 && threadIdx.x == 0) {
        out[0] = 0;
        if (d_total) *d_total = 0;
    }
    while (n) {
        uint32_t tile = next_tile(lb, &sm_tile);
        if (tile >= ntiles) break;
        const uint64_t base = (uint64_t)tile * kTile + (uint64_t)threadIdx.x * kItems;
        uint64_t v[kItems];
        uint64_t tsum = 0;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            uint64_t i = base + k;
            v[k] = i < n ? f(i) : 0;
            tsum += v[k];
        }
        uint64_t agg;
        uint64_t texcl = block_excl_scan(tsum, sm, agg);
        uint64_t prefix = tile_prefix(lb, tile, agg, &bcast);
        uint64_t run = prefix + texcl;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            uint64_t i = base + k;
            if (i < n) {
                out[i] = run;
                epi(i, run, v[k], n);
            }
            run += v[k];
        }
        if (tile == ntiles - 1 && threadIdx.x == kThreads - 1) {
            out[n] = prefix + agg;
            if (d_total) *d_total = prefix + agg;
        }
    }
    publish_at_exit(pb, hook);
}

// ------------------------------------------------------------- compact
// Stream compaction preserving order: P::load(i, item&) -> bool selects item
// i and keeps what its output needs in a P::item (loaded once), P::emit(i, j,
// item) writes it to output slot j.  *d_count = number selected.
template <class P>
__global__ void __launch_bounds__(kThreads) k_compact(P p, const uint64_t *d_n, uint64_t *d_count,
                                                       lookback lb) {
    __shared__ uint64_t sm[kThreads / 32 + 1];
    __shared__ uint64_t bcast;
    __shared__ uint32_t sm_tile;
    const uint64_t n = *d_n;
    const uint64_t ntiles = (n + kTile - 1) / kTile;
    if (n == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *d_count = 0;
        return;
    }
    while (true) {
        uint32_t tile = next_tile(lb, &sm_tile);
        if (tile >= ntiles) break;
        const uint64_t base = (uint64_t)tile * kTile + (uint64_t)threadIdx.x * kItems;
        uint32_t flags = 0;
        uint64_t cnt = 0;
        typename P::item it[kItems];
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            uint64_t i = base + k;
            if (i < n && p.load(i, it[k])) {
                flags |= 1u << k;
                ++cnt;
            }
        }
        uint64_t agg;
        uint64_t texcl = block_excl_scan(cnt, sm, agg);
        uint64_t prefix = tile_prefix(lb, tile, agg, &bcast);
        uint64_t j = prefix + texcl;
#pragma unroll
        for (int k = 0; k < kItems; ++k)
            if (flags & (1u << k)) p.emit(base + k, j++, it[k]);
        if (tile == ntiles - 1 && threadIdx.x == kThreads - 1) *d_count = prefix + agg;
    }
}

// Compaction like k_compact where P::select(i, tie_rank) also sees the rank
// of the item among the ties (P::tie(i)) in item order.
template <class P>
__global__ void __launch_bounds__(kThreads) k_compact_ranked(P p, const uint64_t *d_n, uint64_t *d_count,
                                                              lookback lb, lookback lb_ties) {
    __shared__ uint64_t sm[kThreads / 32 + 1];
    __shared__ uint64_t bcast;
    __shared__ uint32_t sm_tile;
    const uint64_t n = *d_n;
    const uint64_t ntiles = (n + kTile - 1) / kTile;
    if (n == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *d_count = 0;
        return;
    }
    while (true) {
        uint32_t tile = next_tile(lb, &sm_tile);
        if (tile >= ntiles) break;
        const uint64_t base = (uint64_t)tile * kTile + (uint64_t)threadIdx.x * kItems;
        uint32_t ties = 0;
        uint64_t tcnt = 0;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            uint64_t i = base + k;
            if (i < n && p.tie(i)) {
                ties |= 1u << k;
                ++tcnt;
            }
        }
        uint64_t agg_t;
        uint64_t excl_t = block_excl_scan(tcnt, sm, agg_t);
        uint64_t rank = tile_prefix(lb_ties, tile, agg_t, &bcast) + excl_t;
        uint32_t flags = 0;
        uint64_t cnt = 0;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            uint64_t i = base + k;
            if (i < n && p.select(i, rank)) {
                flags |= 1u << k;
                ++cnt;
            }
            if (ties & (1u << k)) ++rank;
        }
        uint64_t agg;
        uint64_t texcl = block_excl_scan(cnt, sm, agg);
        uint64_t prefix = tile_prefix(lb, tile, agg, &bcast);
        uint64_t j = prefix + texcl;
#pragma unroll
        for (int k = 0; k < kItems; ++k)
            if (flags & (1u << k)) p.emit(base + k, j++);
        if (tile == ntiles - 1 && threadIdx.x == kThreads - 1) *d_count = prefix + agg;
    }
}

// --------------------------------------------------------- radix select
// Threshold of a top-k selection on 64-bit keys, 8 bits per pass from the top
// (8 passes).  State is device resident so the passes need no host round trip.
// Afterwards: keys > prefix are kept, and k_rem of the n_equal keys equal to
// prefix (the ties), taken in item order by the keep compaction.
constexpr int kDigitBits = 8;
constexpr int kBins = 1 << kDigitBits;

struct select_state {
    uint64_t prefix;     // key bits fixed so far (the threshold at the end)
    uint64_t mask;       // which bits of prefix are fixed
    uint64_t k_rem;      // how many items still to take among those matching prefix
    uint64_t n_better;   // items strictly better than the threshold
    uint64_t n_equal;    // items equal to the threshold (after the last pass)
    uint32_t active;     // 0: nothing to select (k >= n), pass kernels return
    uint32_t pad;
};

// K::key(i) -> u64.  Shared-memory histogram; lanes holding the same digit
// aggregate their count (keys often share their leading bits).
template <class K>
__global__ void __launch_bounds__(kThreads) k_radix_hist(K kf, const uint64_t *d_n, const select_state *st,
                                                          int shift, unsigned long long *hist) {
    __shared__ unsigned int sh[kBins];
    if (!st->active) return;
    for (int i = threadIdx.x; i < kBins; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    const uint64_t n = *d_n, prefix = st->prefix, mask = st->mask;
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    const uint64_t warp = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (uint64_t base = warp * 32; base < n; base += warps * 32) {
        const uint64_t i = base + lane;
        unsigned d = kBins;
        if (i < n) {
            uint64_t k = kf.key(i);
            if ((k & mask) == prefix) d = (unsigned)((k >> shift) & (kBins - 1));
        }
        const unsigned same = __match_any_sync(0xffffffffu, d);
        if (d < (unsigned)kBins && lane == __ffs(same) - 1) atomicAdd(&sh[d], (unsigned)__popc(same));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kBins; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], (unsigned long long)sh[i]);
}

// picks the digit holding the k-th item in preference order and clears the
// histogram (256 threads scan the 256 bins)
static __global__ void __launch_bounds__(kBins) k_radix_pick(select_state *st, unsigned long long *hist, int shift,
                                                              bool descending) {
    __shared__ uint64_t sm[kBins];
    if (!st->active) return;
    const int t = threadIdx.x;
    const int d = descending ? kBins - 1 - t : t;  // t-th bin in preference order
    const uint64_t c = hist[d];
    sm[t] = c;
    __syncthreads();
    for (int o = 1; o < kBins; o <<= 1) {
        uint64_t v = t >= o ? sm[t - o] : 0;
        __syncthreads();
        sm[t] += v;
        __syncthreads();
    }
    const uint64_t incl = sm[t], excl = incl - c;
    const uint64_t k = st->k_rem;
    __syncthreads();
    if (excl < k && k <= incl) {  // exactly one bin holds the k-th item
        st->prefix |= (uint64_t)d << shift;
        st->mask |= (uint64_t)(kBins - 1) << shift;
        st->n_better += excl;
        st->k_rem = k - excl;
        st->n_equal = c;
    }
    hist[d] = 0;
}

// ---------------------------------------------------- collision table
// slots[M+1] {key, rep, claimer} (16 bytes; cleared to all-ones before each
// step) and acc[M+1][4] (re lo, re hi, im lo, im hi: one 32-byte sector per
// slot).  Pass 1 claims slots (CAS from kEmptyKey); the claiming item leaves
// its index in `claimer` and touches nothing else, and every other member
// (a joiner) clears the group's sum.  Pass 2, a separate launch (no fences),
// adds the joiners' magnitudes, and the first joiner to take `claimer` adds
// the claimer's too.  A group of one never touches acc: its representative
// keeps its own magnitude.  So only the slots need clearing, and a child of
// a singleton group costs one random 16-byte access.
// Children whose hash is kEmptyKey use the extra slot M (no claimer; its sum
// is cleared by the step's fill).  M need not be a power of two: the home
// slot is the high half of (mixed hash) * M.
struct __align__(16) table_slot {
    unsigned long long key;  // kEmptyKey = free
    unsigned int rep;        // minimum child index of the group
    unsigned int claimer;    // item that claimed the slot; 0xffffffff once taken by a joiner
};

struct table {
    table_slot *slots;       // [M+1], memset to 0xff before each step
    unsigned long long *acc;
    uint64_t m;              // slots
    uint32_t max_probes;
    const uint64_t *d_m = nullptr;  // if set, the slot count on the device (m is then a bound)
};

__device__ __forceinline__ uint64_t table_home(uint64_t h, uint64_t m) {
    return __umul64hi(h * 0x9E3779B97F4A7C15ull, m);
}

__device__ __forceinline__ void fix_atomic_add(unsigned long long *w, fix128 v) {
    if ((v.lo | v.hi) == 0) return;
    unsigned long long old = atomicAdd(&w[0], (unsigned long long)v.lo);
    unsigned long long carry = (old + v.lo) < old ? 1ull : 0ull;
    unsigned long long hi = v.hi + carry;
    if (hi) atomicAdd(&w[1], hi);
}

// Pass 1: every child item (src.hash(k)) finds or claims the slot of its
// hash.  The claiming item writes rep = its child index and claimer = its
// item index; slot_out[k] = slot | kJoin for the others, which clear the
// group's sum for pass 2.  0xffffffff at the probe limit
// (QUIDS_ERR_TABLE_FULL).  Item counts stay below 2^32 - 1.
constexpr uint32_t kJoin = 0x80000000u;
constexpr uint32_t kNoSlot = 0xffffffffu;

template <class Src>
__global__ void __launch_bounds__(kMaxTableThreads) k_table_claim(table t, Src src, const uint64_t *d_n, uint32_t *slot_out,
                                                           int *err) {
    const uint64_t n = *d_n;
    const uint64_t m = t.d_m ? *t.d_m : t.m;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t h = src.hash(k);
        uint64_t s;
        bool claimed = false;
        if (h == kEmptyKey) {
            s = m;
        } else {
            s = table_home(h, m);
            uint32_t probe = 0;
            while (true) {
                const unsigned long long key = atomicCAS(&t.slots[s].key, kEmptyKey, h);
                if (key == kEmptyKey) {  // claimed: rep and claimer in one 8-byte store
                    *(uint2 *)&t.slots[s].rep = make_uint2((uint32_t)src.child(k), (uint32_t)k);
                    claimed = true;
                    break;
                }
                if (key == h) {  // a joiner: the group's sum starts at zero
                    ulonglong4_32a z;
                    z.x = z.y = z.z = z.w = 0;
                    *(ulonglong4_32a *)&t.acc[4 * s] = z;
                    break;
                }
                if (++s == m) s = 0;
                if (++probe >= t.max_probes) {
                    set_error(err, QUIDS_ERR_TABLE_FULL);
                    s = ~0ull;
                    break;
                }
            }
        }
        slot_out[k] = s == ~0ull ? kNoSlot : (claimed ? (uint32_t)s : (uint32_t)s | kJoin);
    }
}

// Pass 2: the joiners: rep = minimum child index of the group; acc +=
// magnitude as an exact 128-bit fixed-point sum per component (scale 2^-F, F
// from the largest component and the child count *d_nf -- default: the *d_n
// items; a hash-range pass gives the whole step's count, so its sums are
// those of one pass), independent of the order of the atomics.  The joiner
// that takes the slot's claimer adds the claimer's magnitude as well, so
// every member is added exactly once.  Clears the join marks.  Each
// atomicMin compares two members: the larger is marked not_rep, the smaller
// has_join; at the end the representative is the one member never marked
// not_rep, and it is marked has_join exactly when its group has more than
// one member.  With not_rep = has_join = null nothing is marked (the region
// path reads the marks from the final slots instead).
template <class Src>
__global__ void __launch_bounds__(kMaxTableThreads) k_table_accumulate(table t, Src src, uint32_t *slot_of,
                                                                const uint64_t *d_n,
                                                                const unsigned long long *d_maxabs,
                                                                uint8_t *not_rep, uint8_t *has_join,
                                                                const uint64_t *d_nf = nullptr) {
    const uint64_t n = *d_n;
    const int F = fix_scale(__longlong_as_double((long long)*d_maxabs), d_nf ? *d_nf : n);
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s = slot_of[k];
        if (s == kNoSlot || !(s & kJoin)) continue;
        s &= ~kJoin;
        slot_of[k] = s;
        const uint32_t c = (uint32_t)src.child(k);
        const uint32_t old = atomicMin(&t.slots[s].rep, c);
        if (not_rep && old != 0xffffffffu) {  // slot M starts without a member
            not_rep[old > c ? old : c] = 1;
            has_join[old < c ? old : c] = 1;
        }
        const uint32_t k0 = atomicExch(&t.slots[s].claimer, 0xffffffffu);
        const double2 m = src.mag(k);
        fix128 re = to_fix(m.x, F), im = to_fix(m.y, F);
        if (k0 != 0xffffffffu) {
            const double2 m0 = src.mag(k0);
            re = fix_add(re, to_fix(m0.x, F));
            im = fix_add(im, to_fix(m0.y, F));
        }
        fix_atomic_add(&t.acc[4ull * s + 0], re);
        fix_atomic_add(&t.acc[4ull * s + 2], im);
    }
}

// --------------------------------------------- compaction + byte offsets
// Order-preserving compaction that also lays out the selected items'
// variable-size payloads.  P::load(i, tie_rank, item&) -> bool selects item i
// and keeps what the layout needs in a P::item (loaded once), P::bytes(item)
// -> padded size (asked for selected items only), P::norm(item) -> double,
// P::emit(i, j, byte_offset, item).  With TIES, P::tie(i) -> bool marks the
// items equal to a selection threshold and tie_rank is the item's rank among
// them in item order (a third look-back chain), so a selection can take the
// first ties; P::rank_needed() -> bool (the same for every thread) skips the
// ranking when the selection keeps every tie, and load then gets tie_rank 0.
// The largest selected norm goes to *d_maxnorm (as IEEE bits) when d_maxnorm
// is not null.  At the end: *d_count, *d_bytes and begin_out[count] = total
// bytes.
template <class P, bool TIES, class L = no_last, int ITEMS = kItems>
__global__ void __launch_bounds__(kThreads, 3) k_compact_layout(P p, const uint64_t *d_n, uint64_t *d_count,
                                                              uint64_t *d_bytes, uint64_t *begin_out,
                                                              unsigned long long *d_maxnorm, lookback lb_count,
                                                              lookback lb_bytes, lookback lb_ties,
                                                              publish pb = publish{}, L hook = L{}) {
    __shared__ uint64_t sm[kThreads / 32 + 1];
    __shared__ uint64_t bcast;
    __shared__ uint32_t sm_tile;
    const uint64_t n = *d_n;
    constexpr uint64_t kT = (uint64_t)kThreads * ITEMS;
    const uint64_t ntiles = (n + kT - 1) / kT;
    if (n == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            *d_count = 0;
            *d_bytes = 0;
            begin_out[0] = 0;
        }
        publish_at_exit(pb, hook);
        return;
    }
    __shared__ uint64_t bcast2[2];
    unsigned long long mx = 0;
    bool ranked = false;
    if constexpr (TIES) ranked = p.rank_needed();  // uniform over the launch
    while (true) {
        uint32_t tile = next_tile(lb_count, &sm_tile);
        if (tile >= ntiles) break;
        const uint64_t base = (uint64_t)tile * kT + (uint64_t)threadIdx.x * ITEMS;
        uint64_t rank = 0;
        uint32_t ties = 0;
        if (ranked) {
            uint64_t tcnt = 0;
#pragma unroll
            for (int k = 0; k < ITEMS; ++k) {
                uint64_t i = base + k;
                if (i < n && p.tie(i)) {
                    ties |= 1u << k;
                    ++tcnt;
                }
            }
            uint64_t agg_t;
            uint64_t excl_t = block_excl_scan(tcnt, sm, agg_t);
            rank = tile_prefix(lb_ties, tile, agg_t, &bcast) + excl_t;
        }
        uint32_t flags = 0;
        uint64_t cnt = 0, bytes = 0;
        // the selection of the thread's items, with every load unguarded (an
        // item past the end reads item n-1 and is dropped), so the loads of
        // all items are in flight together
        bool sel[ITEMS];
        typename P::item it[ITEMS];
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const uint64_t i = base + k;
            const uint64_t ic = i < n ? i : n - 1;
            sel[k] = p.load(ic, rank, it[k]) && i < n;
            if (ties & (1u << k)) ++rank;
        }
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            if (sel[k]) {
                flags |= 1u << k;
                ++cnt;
                bytes += p.bytes(it[k]);
            }
        }
        uint64_t agg_c, agg_b;
        uint64_t excl_c = block_excl_scan(cnt, sm, agg_c);
        uint64_t excl_b = block_excl_scan(bytes, sm, agg_b);
        uint64_t pre_c, pre_b;
        tile_prefix2(lb_count, agg_c, lb_bytes, agg_b, tile, bcast2, pre_c, pre_b);
        uint64_t j = pre_c + excl_c, off = pre_b + excl_b;
#pragma unroll
        for (int k = 0; k < ITEMS; ++k)
            if (flags & (1u << k)) {
                const double nrm = p.emit(base + k, j++, off, it[k]);
                const unsigned long long b = (unsigned long long)__double_as_longlong(nrm);
                mx = mx > b ? mx : b;
                off += p.bytes(it[k]);
            }
        if (tile == ntiles - 1 && threadIdx.x == kThreads - 1) {
            *d_count = pre_c + agg_c;
            *d_bytes = pre_b + agg_b;
            begin_out[pre_c + agg_c] = pre_b + agg_b;
        }
    }
    if (d_maxnorm) {
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
            mx = mx > y ? mx : y;
        }
        if ((threadIdx.x & 31) == 0 && mx) atomicMax(d_maxnorm, mx);
    }
    publish_at_exit(pb, hook);
}

// --------------------------------------------------------- normalisation
// Total probability (src/quids.hpp:1002-1008) of the n magnitudes, exact:
// every norm is converted to 128-bit fixed point with F = fix_scale(max
// norm, n) and the integers are summed (any order gives the same bits).
// One fixed-point atomic add per block into acc[2] (zero beforehand); the
// last block to finish (ticket from *done, zero beforehand) converts the
// sum: total = acc 2^-F, factor = sqrt(total).
static __global__ void __launch_bounds__(kThreads)
    k_fix_total(const double2 *mag, const uint64_t *d_n, const unsigned long long *d_maxnorm,
                unsigned long long *acc, unsigned int *done, double *d_total, double *d_factor,
                double *out_total = nullptr, const uint64_t *stop = nullptr) {
    __shared__ fix128 sm[kThreads / 32];
    __shared__ bool last;
    const uint64_t n = *d_n;
    const int F = fix_scale(__longlong_as_double((long long)*d_maxnorm), n);
    fix128 a{0, 0};
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x) {
        const double2 m = mag[j];
        a = fix_add(a, to_fix(cnorm(mag_t{m.x, m.y}), F));
    }
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t lo = __shfl_xor_sync(0xffffffffu, a.lo, o);
        const uint64_t hi = __shfl_xor_sync(0xffffffffu, a.hi, o);
        a = fix_add(a, fix128{lo, hi});
    }
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        fix128 t{0, 0};
        for (int w = 0; w < kThreads / 32; ++w) t = fix_add(t, sm[w]);
        fix_atomic_add(acc, t);
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        const fix128 tot{atomicAdd(&acc[0], 0ull), atomicAdd(&acc[1], 0ull)};
        const double t = from_fix(tot, F);
        *d_total = t;
        *d_factor = __dsqrt_rn(t);
        // the output state's total, unless a planned run stopped (its state is kept as it was)
        if (out_total && !(stop && *stop)) *out_total = t;
    }
}

}  // namespace qd::prim
