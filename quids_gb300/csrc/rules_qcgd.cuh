// rules_qcgd.cuh -- QCGD (quantum causal graph dynamics) rules as device rules.
//
// Reference: src/rules/qcgd.hpp.  Object layout (:63-112):
//   [u16 n][u8 left[n]][u8 right[n]][u16 name_begin[n+1]][name sub-nodes]
// A name sub-node (:35-61) is 16 bytes {i16 hmlz_and_element,
// i16 right_or_type, 4 padding bytes, u64 hash}; the sub-node array starts at
// byte 4+4n, so its u64 fields are misaligned for even n.  Every access here
// goes through qd_common's alignment-safe helpers.
//
// The graph hash (hash_graph, :122-146) and the name algebra
// (operations::left/right/merge, :181-209) are restated bit for bit; the
// rules add a hash_child fast path that yields the child's hash, size and
// magnitude without writing its bytes (the child's hash depends only on the
// root sub-node hash of each node and the left/right bits).
#pragma once
#include "qd_common.cuh"

namespace qd::qcgd {

enum : int16_t { dot_l_t = -3, dot_r_t = -2, element_t = -1 };

// utils::hash_combine, src/rules/qcgd.hpp:11-25
QD_HD void hash_combine(uint64_t &seed, uint64_t v) {
    constexpr uint64_t m = 0xc6a4a7935bd1e995ull;
    seed *= m;
    seed ^= v >> 47;
    seed *= m;
    seed ^= v;
    seed *= m;
    seed += 0xe6546b64ull;
}

// trailing zeros of v > 0 (small v; constant once unrolled)
QD_HD constexpr int ctz_small(int v) {
    int c = 0;
    while (!(v & 1)) {
        v >>= 1;
        ++c;
    }
    return c;
}

// ---- accessors (n passed explicitly: the count is read once per object)
QD_HD int num_nodes(const char *o) { return ld_u16(o); }
QD_HD bool L(const char *o, int i) { return o[2 + i] != 0; }
QD_HD bool R(const char *o, int n, int i) { return o[2 + n + i] != 0; }
QD_HD int name_begin(const char *o, int n, int i) { return ld_u16(o + 2 + 2 * n + 2 * i); }
QD_HD const char *names(const char *o, int n) { return o + 4 + 4 * n; }
QD_HD char *names(char *o, int n) { return o + 4 + 4 * n; }

struct sub_node {
    int16_t hmlz, rot;
    uint32_t pad;
    uint64_t hash;
};
QD_HD sub_node get_node(const char *base, int k) {
    const char *p = base + 16 * k;
    uint32_t w = ld_u32(p);
    sub_node s;
    s.hmlz = (int16_t)(w & 0xffff);
    s.rot = (int16_t)(w >> 16);
    s.pad = ld_u32(p + 4);
    s.hash = ld_u64(p + 8);
    return s;
}
QD_HD int16_t node_rot(const char *base, int k) { return (int16_t)ld_u16(base + 16 * k + 2); }
QD_HD int16_t node_hmlz(const char *base, int k) { return (int16_t)ld_u16(base + 16 * k); }
QD_HD uint64_t node_hash(const char *base, int k) { return ld_u64(base + 16 * k + 8); }
QD_HD void put_node(char *base, int k, sub_node s) {
    char *p = base + 16 * k;
    st_u16(p, (uint16_t)s.hmlz);
    st_u16(p + 2, (uint16_t)s.rot);
    st_u16(p + 4, 0);
    st_u16(p + 6, 0);
    st_u64(p + 8, s.hash);
}

// sub_node constructors, :43-60
QD_HD sub_node make_dot(sub_node x, int16_t type) {
    sub_node s;
    s.rot = type;
    s.hmlz = (type == dot_l_t && x.hmlz < 0) ? -1 : 1;
    s.pad = 0;
    s.hash = x.hash;
    hash_combine(s.hash, (uint64_t)(int64_t)type);
    return s;
}
QD_HD sub_node make_pair(sub_node l, sub_node r, int16_t right_offset) {
    sub_node s;
    s.rot = right_offset;
    s.hmlz = (l.hmlz < 0 || r.hmlz < 0) ? -1 : 1;
    s.pad = 0;
    s.hash = l.hash;
    hash_combine(s.hash, r.hash);
    return s;
}

// graphs::hash_graph, :122-146
QD_HD uint64_t hash_graph(const char *o) {
    int n = num_nodes(o);
    const char *nm = names(o, n);
    uint64_t lh = 0, rh = 0, nh = 0;
    for (int i = 0; i < n; ++i) {
        if (L(o, i)) hash_combine(lh, (uint64_t)i);
        if (R(o, n, i)) hash_combine(rh, (uint64_t)i);
        hash_combine(nh, node_hash(nm, name_begin(o, n, i)));
    }
    hash_combine(nh, lh);
    hash_combine(nh, rh);
    return nh;
}

// operations::get_operations, :174-179
QD_HD void get_operations(const char *p, int n, int i, bool &split, bool &merge) {
    merge = false;
    split = L(p, i) && R(p, n, i);
    if (!split && i + 1 < n) merge = L(p, i) && R(p, n, i + 1) && !L(p, i + 1);
}

// ---------------------------------------------------------------- name ops
// A child node's name is one operation on parent name ranges [b, e)
// (sub-node indices into the parent's name array).
enum name_op { OP_COPY = 0, OP_LEFT = 1, OP_RIGHT = 2, OP_MERGE = 3 };

// writes the name into dst[d..) and returns the end index
// The name writer's copies go through one out-of-line function: inlined at
// its eight call sites, the copy loops made split_merge's populate kernel large
// enough to stall on instruction fetch (qcgd12: 22.4 ms, against 9.5 ms with
// the call).
QD_HD_CALL void copy_name_bytes(char *dst, const char *src, uint32_t n) { copy_bytes(dst, src, n); }

QD_HD int write_name(const char *src, char *dst, int d, int op, int b1, int e1, int b2, int e2) {
    switch (op) {
    case OP_COPY:
        copy_name_bytes(dst + 16 * d, src + 16 * b1, 16u * (uint32_t)(e1 - b1));
        return d + (e1 - b1);
    case OP_LEFT: {  // operations::left, :194-200
        int16_t rot = node_rot(src, b1);
        if (rot >= 0) {
            copy_name_bytes(dst + 16 * d, src + 16 * (b1 + 1), 16u * (uint32_t)(rot - 1));
            return d + rot - 1;
        }
        put_node(dst, d, make_dot(get_node(src, b1), dot_l_t));
        copy_name_bytes(dst + 16 * (d + 1), src + 16 * b1, 16u * (uint32_t)(e1 - b1));
        return d + 1 + (e1 - b1);
    }
    case OP_RIGHT: {  // operations::right, :202-208
        int16_t rot = node_rot(src, b1);
        if (rot >= 0) {
            copy_name_bytes(dst + 16 * d, src + 16 * (b1 + rot), 16u * (uint32_t)(e1 - b1 - rot));
            return d + (e1 - b1 - rot);
        }
        put_node(dst, d, make_dot(get_node(src, b1), dot_r_t));
        copy_name_bytes(dst + 16 * (d + 1), src + 16 * b1, 16u * (uint32_t)(e1 - b1));
        return d + 1 + (e1 - b1);
    }
    default: {  // operations::merge, :181-192
        if (node_rot(src, b1) == dot_l_t && node_rot(src, b2) == dot_r_t &&
            node_hash(src, b1 + 1) == node_hash(src, b2 + 1)) {
            copy_name_bytes(dst + 16 * d, src + 16 * (b1 + 1), 16u * (uint32_t)(e1 - b1 - 1));
            return d + (e1 - b1 - 1);
        }
        put_node(dst, d, make_pair(get_node(src, b1), get_node(src, b2), (int16_t)(e1 - b1 + 1)));
        copy_name_bytes(dst + 16 * (d + 1), src + 16 * b1, 16u * (uint32_t)(e1 - b1));
        copy_name_bytes(dst + 16 * (d + 1 + e1 - b1), src + 16 * b2, 16u * (uint32_t)(e2 - b2));
        return d + 1 + (e1 - b1) + (e2 - b2);
    }
    }
}

// root hash and sub-node count of the name an operation would write
QD_HD uint64_t name_root_hash(const char *src, int op, int b1, int e1, int b2, int e2, int &len) {
    switch (op) {
    case OP_COPY:
        len = e1 - b1;
        return node_hash(src, b1);
    case OP_LEFT: {
        int16_t rot = node_rot(src, b1);
        if (rot >= 0) {
            len = rot - 1;
            return node_hash(src, b1 + 1);
        }
        len = 1 + (e1 - b1);
        uint64_t h = node_hash(src, b1);
        hash_combine(h, (uint64_t)(int64_t)dot_l_t);
        return h;
    }
    case OP_RIGHT: {
        int16_t rot = node_rot(src, b1);
        if (rot >= 0) {
            len = e1 - b1 - rot;
            return node_hash(src, b1 + rot);
        }
        len = 1 + (e1 - b1);
        uint64_t h = node_hash(src, b1);
        hash_combine(h, (uint64_t)(int64_t)dot_r_t);
        return h;
    }
    default: {
        // a dot node is always followed by its operand, so b1+1 / b2+1 are
        // only read when both roots are dot nodes
        if (node_rot(src, b1) == dot_l_t && node_rot(src, b2) == dot_r_t) {
            uint64_t hl1 = node_hash(src, b1 + 1);
            if (hl1 == node_hash(src, b2 + 1)) {
                len = e1 - b1 - 1;
                return hl1;
            }
        }
        len = 1 + (e1 - b1) + (e2 - b2);
        uint64_t h = node_hash(src, b1);
        hash_combine(h, node_hash(src, b2));
        return h;
    }
    }
}

// ------------------------------------------------------------ the factors
// do = polar(sin theta, phi), do_not = polar(cos theta, xi), formed on the
// host (:466-471); the rules use do, conj(do), do_not and -conj(do_not).
struct factors {
    mag_t d, dc, dn, ndnc;
};

// A rule multiplies a child's magnitude by a product of the four factors.
// The rules name the factor they apply (F_D .. F_NDNC); with a magnitude the
// factor's value multiplies it, with a factor_count (used by the adjoint)
// the factor's occurrence is counted instead.
enum { F_D = 0, F_DC = 1, F_DN = 2, F_NDNC = 3 };
struct factor_count {
    uint16_t n[4];
};
QD_HD void mulf(mag_t *m, const factors &f, int k) {
    if (!m) return;
    const mag_t &v = k == F_D ? f.d : k == F_DC ? f.dc : k == F_DN ? f.dn : f.ndnc;
    *m = cmul(*m, v);
}
QD_HD void mulf(factor_count *m, const factors &, int k) {
    if (m) ++m->n[k];
}

// ---------------------------------------------------- erase_create / coin
// erase_create (:459-532): a site is a node with left == right;
// coin (:534-605): a site is a node with left != right.  Children = 2^sites
// (u32, wraps to 0 at 32 sites like the reference's uint).  Per site, in node
// order, using child_id bits LSB first: bit 1 flips both bits and multiplies
// by conj? conj(do) : do; bit 0 multiplies by conj? -conj(do_not) : do_not,
// with conj = both set (erase_create) or left set (coin).
template <bool ON_XOR>
struct flip_rule {
    factors f;
    static constexpr bool grouped_children = true;  // 2^sites children, one factor per site
    static constexpr int claimed_pass_blocks = 4;    // resident blocks of the grouped pass with a table claim

    QD_HD static bool site(bool l, bool r) { return ON_XOR ? (l != r) : (l == r); }
    QD_HD static bool conj_of(bool l, bool r) { return ON_XOR ? l : (l && r); }

    QD_HD void get_num_child(const char *pb, const char *pe, uint32_t &num_child,
                             uint32_t &max_child_size) const {
        max_child_size = (uint32_t)(pe - pb);
        int n = num_nodes(pb);
        uint32_t nc = 1;
        for (int i = 0; i < n; ++i)
            if (site(L(pb, i), R(pb, n, i))) nc *= 2;
        num_child = nc;
    }
    // 2^sites does not fit the u32 child count (32 sites or more): the
    // reference's uint wraps to 0 and loses the parent's children
    // (src/rules/qcgd.hpp:480-485, :555-560); this library reports
    // QUIDS_ERR_CHILD_COUNT_OVERFLOW instead
    QD_HD bool child_count_overflows(const char *pb, const char *) const {
        const int n = num_nodes(pb);
        int sites = 0;
        for (int i = 0; i < n; ++i) sites += site(L(pb, i), R(pb, n, i)) ? 1 : 0;
        return sites >= 32;
    }
    template <class M>
    QD_HD void apply(const char *pb, int n, uint32_t cid, M *mag, char *cb, uint64_t *lh, uint64_t *rh) const {
        for (int i = 0; i < n; ++i) {
            bool l = L(pb, i), r = R(pb, n, i);
            if (site(l, r)) {
                bool c = conj_of(l, r);
                if (cid & 1) {
                    mulf(mag, f, c ? F_DC : F_D);
                    l = !l;
                    r = !r;
                    if (cb) {
                        cb[2 + i] = l;
                        cb[2 + n + i] = r;
                    }
                } else {
                    mulf(mag, f, c ? F_NDNC : F_DN);
                }
                cid >>= 1;
            }
            if (lh) {
                if (l) hash_combine(*lh, (uint64_t)i);
                if (r) hash_combine(*rh, (uint64_t)i);
            }
        }
    }
    QD_HD void populate_child(const char *pb, const char *pe, char *cb, uint32_t child_id,
                              uint32_t &size, mag_t &mag) const {
        size = (uint32_t)(pe - pb);
        copy_bytes(cb, pb, size);
        apply(pb, num_nodes(pb), child_id, &mag, cb, nullptr, nullptr);
    }
    QD_HD void populate_child_simple(const char *pb, const char *pe, char *cb,
                                     uint32_t child_id) const {
        copy_bytes(cb, pb, (uint32_t)(pe - pb));
        apply(pb, num_nodes(pb), child_id, (mag_t *)nullptr, cb, nullptr, nullptr);
    }
    QD_HD void factor_counts(const char *pb, const char *, uint32_t child_id, factor_count &fc) const {
        apply(pb, num_nodes(pb), child_id, &fc, nullptr, nullptr, nullptr);
    }
    QD_HD uint64_t hasher(const char *b, const char *) const { return hash_graph(b); }

    // The 2^H children of a parent with s >= H sites whose child ids share
    // the low s-H bits `e` (children e + j 2^(s-H), j < 2^H), as hash_child
    // computes them, bit for bit: a child's magnitude is the parent's times
    // one factor per site in site order, so these children share the
    // products over the first s-H sites, and the last H sites form a binary
    // tree walked with the j bits reversed, so consecutive children redo
    // only the products that differ (2^(H+1) - 2 complex products for
    // 2^H children instead of H 2^H).  The left/right hashes share their
    // prefixes the same way.  emit(j, hash, magnitude, size).
    struct walk_state {
        mag_t m;
        uint64_t lh, rh;
    };
    template <int H, class Emit>
    QD_HD void expand_group(const char *pb, const char *pe, uint32_t e, int s, mag_t pm, Emit &&emit) const {
        const uint32_t size = (uint32_t)(pe - pb);
        const int n = num_nodes(pb);
        const char *nm = names(pb, n);
        uint64_t nh = 0;
        for (int i = 0; i < n; ++i) hash_combine(nh, node_hash(nm, name_begin(pb, n, i)));
        // shared prefix: the nodes before the first of the last H sites
        walk_state w{pm, 0, 0};
        int i = 0, k = 0;
        uint32_t bits = e;
        for (; i < n; ++i) {
            bool l = L(pb, i), r = R(pb, n, i);
            if (site(l, r)) {
                if (k == s - H) break;
                const bool c = conj_of(l, r);
                if (bits & 1) {
                    mulf(&w.m, f, c ? F_DC : F_D);
                    l = !l;
                    r = !r;
                } else {
                    mulf(&w.m, f, c ? F_NDNC : F_DN);
                }
                bits >>= 1;
                ++k;
            }
            if (l) hash_combine(w.lh, (uint64_t)i);
            if (r) hash_combine(w.rh, (uint64_t)i);
        }
        int q[H + 1];  // node index of each suffix site, then n
        {
            int x = i, m = 0;
            for (; x < n && m < H; ++x)
                if (site(L(pb, x), R(pb, n, x))) q[m++] = x;
            q[H] = n;
        }
        walk_state P[H + 1];  // P[lv]: the state before suffix site lv (P[H] is the child's)
        P[0] = w;
#pragma unroll
        for (int t = 0; t < (1 << H); ++t) {
            int j = 0;
#pragma unroll
            for (int b = 0; b < H; ++b) j |= ((t >> b) & 1) << (H - 1 - b);
            const int k0 = t == 0 ? 0 : H - 1 - ctz_small(t);
#pragma unroll
            for (int lv = 0; lv < H; ++lv) {
                if (lv < k0) continue;
                walk_state x = P[lv];
                const int node = q[lv];
                bool l = L(pb, node), r = R(pb, n, node);
                const bool c = conj_of(l, r);
                if ((j >> lv) & 1) {
                    mulf(&x.m, f, c ? F_DC : F_D);
                    l = !l;
                    r = !r;
                } else {
                    mulf(&x.m, f, c ? F_NDNC : F_DN);
                }
                if (l) hash_combine(x.lh, (uint64_t)node);
                if (r) hash_combine(x.rh, (uint64_t)node);
                for (int y = node + 1; y < q[lv + 1]; ++y) {
                    if (L(pb, y)) hash_combine(x.lh, (uint64_t)y);
                    if (R(pb, n, y)) hash_combine(x.rh, (uint64_t)y);
                }
                P[lv + 1] = x;
            }
            uint64_t hh = nh;
            hash_combine(hh, P[H].lh);
            hash_combine(hh, P[H].rh);
            emit((uint32_t)j, hh, P[H].m, size);
        }
    }

    QD_HD uint64_t hash_child(const char *pb, const char *pe, uint32_t child_id, uint32_t &size,
                              mag_t &mag) const {
        size = (uint32_t)(pe - pb);
        int n = num_nodes(pb);
        uint64_t lh = 0, rh = 0, nh = 0;
        apply(pb, n, child_id, &mag, nullptr, &lh, &rh);
        const char *nm = names(pb, n);
        for (int i = 0; i < n; ++i) hash_combine(nh, node_hash(nm, name_begin(pb, n, i)));
        hash_combine(nh, lh);
        hash_combine(nh, rh);
        return nh;
    }
};
using erase_create = flip_rule<false>;
using coin = flip_rule<true>;

// ------------------------------------------------------------ split_merge
// split_merge, :607-1036.  Sites: a split at node i (left && right) or a
// merge of nodes i, i+1 (left_i && right_{i+1} && !left_{i+1}); the wrap
// sites are a split of node 0 and a merge of nodes n-1 and 0.  The child's
// nodes are produced in increasing index order by `walk`, which hands each
// (index, left, right, name operation) to a sink: a byte writer for
// populate_child, a hash accumulator for hash_child.
struct split_merge {
    factors f;

    QD_HD static void wrap_sites(const char *p, int n, bool &first_split, bool &last_merge) {
        last_merge = false;
        first_split = L(p, 0) && R(p, n, 0);
        if (!first_split && n > 1) last_merge = R(p, n, 0) && L(p, n - 1) && !R(p, n, n - 1);
    }

    QD_HD void get_num_child(const char *pb, const char *pe, uint32_t &num_child,
                             uint32_t &max_child_size) const {
        max_child_size = 4 * (uint32_t)(pe - pb);
        int n = num_nodes(pb);
        bool fs, lm;
        wrap_sites(pb, n, fs, lm);
        uint32_t nc = (fs || lm) ? 2 : 1;
        for (int i = fs; i < n - lm; ++i) {
            bool s, m;
            get_operations(pb, n, i, s, m);
            if (s || m) nc *= 2;
        }
        num_child = nc;
    }
    // the child count 2^(sites + wrap site) does not fit u32 (the reference's
    // uint wraps, src/rules/qcgd.hpp:623-642)
    QD_HD bool child_count_overflows(const char *pb, const char *) const {
        const int n = num_nodes(pb);
        bool fs, lm;
        wrap_sites(pb, n, fs, lm);
        int bits = (fs || lm) ? 1 : 0;
        for (int i = fs; i < n - lm; ++i) {
            bool s, m;
            get_operations(pb, n, i, s, m);
            bits += (s || m) ? 1 : 0;
        }
        return bits >= 32;
    }

    // first pass (:647-700): wrap decisions, child node count, magnitude
    struct plan {
        bool fs, lm;
        int n, cn;
        uint32_t cid;  // child id with the wrap bits consumed
    };
    // the wrap decisions alone (their factors first, as the reference applies
    // them); cn counts the nodes before the middle sites' splits and merges
    template <class M>
    QD_HD plan wrap_plan(const char *p, uint32_t cid, M *mag) const {
        plan pl;
        int n = pl.n = num_nodes(p);
        bool fs, lm;
        wrap_sites(p, n, fs, lm);
        fs = fs && (cid & 1);
        if (fs) {
            mulf(mag, f, F_D);
            cid >>= 1;
        }
        if (lm) {
            if (cid & 1) {
                mulf(mag, f, F_DC);
            } else {
                lm = false;
                mulf(mag, f, F_NDNC);
            }
            cid >>= 1;
        }
        pl.fs = fs;
        pl.lm = lm;
        pl.cn = n + fs - lm;
        pl.cid = cid;
        return pl;
    }
    template <class M>
    QD_HD plan make_plan(const char *p, uint32_t cid, M *mag) const {
        plan pl = wrap_plan(p, cid, mag);
        const int n = pl.n;
        const bool fs = pl.fs, lm = pl.lm;
        int cn = pl.cn;
        uint32_t bits = pl.cid;
        for (int i = fs + lm; i < n - lm; ++i) {
            bool s, m;
            get_operations(p, n, i, s, m);
            if (!(s || m)) continue;
            if (bits & 1) {
                cn += (int)s - (int)m;
                mulf(mag, f, s ? F_D : F_DC);
            } else {
                mulf(mag, f, s ? F_DN : F_NDNC);
            }
            bits >>= 1;
        }
        pl.cn = cn;
        return pl;
    }

    // second pass (:702-845).  With mag, the middle sites' factors are applied
    // on the way, in the order make_plan applies them (a site's node comes
    // before the next site's; a taken merge's second node is never a site), so
    // wrap_plan + walk(mag) is make_plan + walk in one pass over the nodes.
    template <class Sink, class M = mag_t>
    QD_HD void walk(const char *p, const plan &pl, Sink &sink, M *mag = nullptr) const {
        const int n = pl.n;
        int cn = pl.n + pl.fs - pl.lm;  // the child's nodes, counted as the sites are taken
        const bool fs = pl.fs, lm = pl.lm;
        uint32_t cid = pl.cid;
        const char *pn = names(p, n);
        bool overflow = false;
        if (fs) {
            bool most_left_zero = true;
            if (node_rot(pn, 0) >= 0 && node_hmlz(pn, 1) > 0) most_left_zero = false;
            int e0 = name_begin(p, n, 1);
            if (most_left_zero) {
                sink.emit(0, true, false, OP_LEFT, 0, e0, 0, 0);
                sink.emit(1, false, true, OP_RIGHT, 0, e0, 0, 0);
            } else {
                overflow = true;
                sink.emit(0, false, true, OP_RIGHT, 0, e0, 0, 0);
            }
        }
        if (lm)
            sink.emit(0, true, true, OP_MERGE, name_begin(p, n, n - 1), name_begin(p, n, n), 0,
                      name_begin(p, n, 1));
        int off = (int)fs - (int)overflow;
        for (int i = fs + lm; i < n - lm; ++i) {
            bool s, m;
            get_operations(p, n, i, s, m);
            if (s || m) {
                i = walk_site(p, n, i, s, m, cid & 1, sink, mag, off, cn);
                cid >>= 1;
            } else {
                sink.emit(i + off, L(p, i), R(p, n, i), OP_COPY, name_begin(p, n, i), name_begin(p, n, i + 1), 0,
                          0);
            }
        }
        if (overflow) sink.emit(cn - 1, true, false, OP_LEFT, 0, name_begin(p, n, 1), 0, 0);
    }
    // the first pass's handling of the wrap split of node 0 (:702-735):
    // true when its left half overflows to the end of the child
    QD_HD static bool first_split_overflows(const char *p, int n) {
        const char *pn = names(p, n);
        return node_rot(pn, 0) >= 0 && node_hmlz(pn, 1) > 0;
    }
    // one middle site, split (s) or merge (m) of node i, taken or not: its
    // factor, its nodes; returns the last node it consumed (a taken merge
    // consumes node i + 1, which is never a site)
    template <class Sink, class M>
    QD_HD int walk_site(const char *p, int n, int i, bool s, bool m, bool taken, Sink &sink, M *mag, int &off,
                        int &cn) const {
        mulf(mag, f, taken ? (s ? F_D : F_DC) : (s ? F_DN : F_NDNC));
        if (!taken) {
            sink.emit(i + off, L(p, i), R(p, n, i), OP_COPY, name_begin(p, n, i), name_begin(p, n, i + 1), 0, 0);
            return i;
        }
        cn += (int)s - (int)m;
        const int b = name_begin(p, n, i), e = name_begin(p, n, i + 1);
        if (s) {
            sink.emit(i + off, true, false, OP_LEFT, b, e, 0, 0);
            sink.emit(i + off + 1, false, true, OP_RIGHT, b, e, 0, 0);
        } else {
            sink.emit(i + off, true, true, OP_MERGE, b, e, e, name_begin(p, n, i + 2));
        }
        off += (int)s - (int)m;
        return i + (int)m;
    }

    struct byte_sink {
        const char *pn;
        char *c;
        int cn;
        char *cnm;
        QD_HD void emit(int k, bool l, bool r, int op, int b1, int e1, int b2, int e2) {
            c[2 + k] = l;
            c[2 + cn + k] = r;
            int d = ld_u16(c + 2 + 2 * cn + 2 * k);
            int e = write_name(pn, cnm, d, op, b1, e1, b2, e2);
            st_u16(c + 2 + 2 * cn + 2 * (k + 1), (uint16_t)e);
        }
    };
    struct hash_sink {
        const char *pn;
        uint64_t lh, rh, nh;
        int len;
        int cn = 0;  // nodes emitted
        QD_HD void emit(int k, bool l, bool r, int op, int b1, int e1, int b2, int e2) {
            ++cn;
            if (l) hash_combine(lh, (uint64_t)k);
            if (r) hash_combine(rh, (uint64_t)k);
            int ln;
            hash_combine(nh, name_root_hash(pn, op, b1, e1, b2, e2, ln));
            len += ln;
        }
    };

    QD_HD void build(const char *p, char *c, uint32_t child_id, mag_t *mag, uint32_t *size) const {
        plan pl = make_plan(p, child_id, mag);
        st_u16(c, (uint16_t)pl.cn);
        st_u16(c + 2 + 2 * pl.cn, 0);
        byte_sink s{names(p, pl.n), c, pl.cn, names(c, pl.cn)};
        walk(p, pl, s);
        if (size) *size = 4 + 4 * (uint32_t)pl.cn + 16 * (uint32_t)ld_u16(c + 2 + 2 * pl.cn + 2 * pl.cn);
    }
    QD_HD void populate_child(const char *pb, const char *, char *cb, uint32_t child_id,
                              uint32_t &size, mag_t &mag) const {
        build(pb, cb, child_id, &mag, &size);
    }
    QD_HD void populate_child_simple(const char *pb, const char *, char *cb, uint32_t child_id) const {
        build(pb, cb, child_id, nullptr, nullptr);
    }
    QD_HD void factor_counts(const char *pb, const char *, uint32_t child_id, factor_count &fc) const {
        make_plan(pb, child_id, &fc);
    }
    QD_HD uint64_t hasher(const char *b, const char *) const { return hash_graph(b); }
    QD_HD uint64_t hash_child(const char *pb, const char *, uint32_t child_id, uint32_t &size,
                              mag_t &mag) const {
        plan pl = wrap_plan(pb, child_id, &mag);
        hash_sink s{names(pb, pl.n), 0, 0, 0, 0};
        walk(pb, pl, s, &mag);
        pl.cn = s.cn;
        hash_combine(s.nh, s.lh);
        hash_combine(s.nh, s.rh);
        size = 4 + 4 * (uint32_t)pl.cn + 16 * (uint32_t)s.len;
        return s.nh;
    }

    // The grouped symbolic pass (as flip_rule's): the 2^H children e +
    // j 2^(s-H) share their child id's low s-H bits, so they share the wrap
    // decisions and the walk up to the first of the last H middle sites (the
    // bits are consumed in node order).  That prefix is walked once, and
    // the last H sites as a binary tree with the j bits reversed; each level
    // keeps the walk's state (magnitude, hash sink, index offset, node
    // count).  Bit for bit what hash_child gives each child.  A group whose
    // top H bits are not all middle sites (a wrap bit among them) is
    // computed child by child.  emit(j, hash, magnitude, size).
    static constexpr bool grouped_children = true;
    struct tree_state {
        mag_t m;
        hash_sink s;
        int off, cn;
    };
    template <int H, class Emit>
    QD_HD void expand_group(const char *pb, const char *pe, uint32_t e, int s, mag_t pm, Emit &&emit) const {
        mag_t m0 = pm;
        plan pl = wrap_plan(pb, e, &m0);
        const int n = pl.n;
        bool fs0, lm0;
        wrap_sites(pb, n, fs0, lm0);
        // bit 0 decides a possible wrap site (taken or not, it shapes the
        // walk), so it must be one of e's bits; it is consumed as a wrap bit
        // when the first split is taken or a last merge is possible, and is
        // node 0's middle-site bit when the first split is not taken
        const int wrap_bits = (int)pl.fs + (int)lm0;
        if (s - H < ((fs0 || lm0) ? 1 : 0)) {
            for (uint32_t j = 0; j < (1u << H); ++j) {
                mag_t m = pm;
                uint32_t sz = 0;
                const uint64_t h = hash_child(pb, pe, e + (j << (s - H)), sz, m);
                emit(j, h, m, sz);
            }
            return;
        }
        // the prefix: wrap nodes and middle sites before the last H (as walk)
        const char *pn = names(pb, n);
        tree_state w{m0, hash_sink{pn, 0, 0, 0, 0}, 0, n + (int)pl.fs - (int)pl.lm};
        const bool fs = pl.fs, lm = pl.lm;
        bool overflow = false;
        if (fs) {
            overflow = first_split_overflows(pb, n);
            const int e0 = name_begin(pb, n, 1);
            if (!overflow) {
                w.s.emit(0, true, false, OP_LEFT, 0, e0, 0, 0);
                w.s.emit(1, false, true, OP_RIGHT, 0, e0, 0, 0);
            } else {
                w.s.emit(0, false, true, OP_RIGHT, 0, e0, 0, 0);
            }
        }
        if (lm)
            w.s.emit(0, true, true, OP_MERGE, name_begin(pb, n, n - 1), name_begin(pb, n, n), 0,
                     name_begin(pb, n, 1));
        w.off = (int)fs - (int)overflow;
        const int prefix_sites = s - H - wrap_bits;
        uint32_t bits = pl.cid;
        int i = fs + lm, k = 0;
        for (; i < n - lm; ++i) {
            bool sp, mg;
            get_operations(pb, n, i, sp, mg);
            if (sp || mg) {
                if (k == prefix_sites) break;
                i = walk_site(pb, n, i, sp, mg, bits & 1, w.s, &w.m, w.off, w.cn);
                bits >>= 1;
                ++k;
            } else {
                w.s.emit(i + w.off, L(pb, i), R(pb, n, i), OP_COPY, name_begin(pb, n, i), name_begin(pb, n, i + 1),
                         0, 0);
            }
        }
        int q[H + 1];  // node index of each of the last H sites, then the end of the middle nodes
        {
            int x = i, c = 0;
            for (; x < n - lm && c < H; ++x) {
                bool sp, mg;
                get_operations(pb, n, x, sp, mg);
                if (sp || mg) q[c++] = x;
            }
            q[H] = n - lm;
        }
        tree_state P[H + 1];  // P[lv]: the state before site lv (P[H]: the child's)
        P[0] = w;
#pragma unroll
        for (int t = 0; t < (1 << H); ++t) {
            int j = 0;
#pragma unroll
            for (int b = 0; b < H; ++b) j |= ((t >> b) & 1) << (H - 1 - b);
            const int k0 = t == 0 ? 0 : H - 1 - ctz_small(t);
#pragma unroll
            for (int lv = 0; lv < H; ++lv) {
                if (lv < k0) continue;
                tree_state x = P[lv];
                bool sp, mg;
                get_operations(pb, n, q[lv], sp, mg);
                const int last = walk_site(pb, n, q[lv], sp, mg, (j >> lv) & 1, x.s, &x.m, x.off, x.cn);
                for (int y = last + 1; y < q[lv + 1]; ++y)
                    x.s.emit(y + x.off, L(pb, y), R(pb, n, y), OP_COPY, name_begin(pb, n, y),
                             name_begin(pb, n, y + 1), 0, 0);
                P[lv + 1] = x;
            }
            hash_sink hs = P[H].s;
            if (overflow) hs.emit(P[H].cn - 1, true, false, OP_LEFT, 0, name_begin(pb, n, 1), 0, 0);
            hash_combine(hs.nh, hs.lh);
            hash_combine(hs.nh, hs.rh);
            emit((uint32_t)j, hs.nh, P[H].m, 4 + 4 * (uint32_t)hs.cn + 16 * (uint32_t)hs.len);
        }
    }
};

// step / reversed_step modifiers, :443-457: rotate `left` one place towards
// index 0 and `right` one place away from it (step), or the reverse.
template <bool REVERSED>
struct step_mod {
    QD_HD void operator()(char *b, char *, mag_t &) const {
        int n = num_nodes(b);
        if (n <= 0) return;
        char *l = b + 2, *r = b + 2 + n;
        char *a = REVERSED ? r : l;  // rotated towards 0
        char *z = REVERSED ? l : r;  // rotated away from 0
        char a0 = a[0];
        for (int i = 0; i + 1 < n; ++i) a[i] = a[i + 1];
        a[n - 1] = a0;
        char zl = z[n - 1];
        for (int i = n - 1; i > 0; --i) z[i] = z[i - 1];
        z[0] = zl;
    }
};
using step = step_mod<false>;
using reversed_step = step_mod<true>;

// ------------------------------------------------------------ observables
// the observables qcgd::utils::serialize averages (src/rules/qcgd.hpp:317-343)
struct obs_num_nodes {
    bool squared;
    QD_HD double operator()(const char *b, const char *) const {
        double n = (double)num_nodes(b);
        return squared ? dmul(n, n) : n;
    }
};
struct obs_density {
    bool squared;
    QD_HD double operator()(const char *b, const char *) const {
        const int n = num_nodes(b);
        double d = 0;
        for (int i = 0; i < n; ++i) d = dadd(d, (double)(L(b, i) + R(b, n, i)));
        d = d / (2.0 * n);
        return squared ? dmul(d, d) : d;
    }
};

}  // namespace qd::qcgd
