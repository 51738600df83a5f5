/*
 * quids_port.cpp -- CPU restatement of the QuIDS rule step, written for this
 * project.  TEST INFRASTRUCTURE: it is the parity oracle and the timed CPU
 * baseline, never part of the product path (see oracle_api.h).
 *
 * It restates, stage by stage and with OpenMP + libstdc++ parallel mode like
 * the reference, the algorithm of src/quids.hpp:
 *   simulate(it, rule, next, sy, max)   src/quids.hpp:448-543
 *   compute_num_child                   src/quids.hpp:548-569
 *   iteration::truncate (simple)        src/quids.hpp:613-642
 *   generate_symbolic_iteration         src/quids.hpp:647-721
 *   compute_collisions                  src/quids.hpp:726-824
 *     hash-bucket partition             src/utils/algorithm.hpp:170-227
 *     first-insert-wins map per bucket  src/quids.hpp:785-809
 *   symbolic_iteration::truncate        src/quids.hpp:866-900
 *   finalize                            src/quids.hpp:905-968
 *   apply_modifier                      src/quids.hpp:973-980
 *   normalize                           src/quids.hpp:985-1017
 * and the rules of src/rules/quantum_computer.hpp and src/rules/qcgd.hpp.
 * The default hasher is the reference's: std::hash<std::string_view>
 * (src/quids.hpp:143-145).  Object storage pads every object to
 * align_byte_length exactly like get_alignment_offset (src/quids.hpp:93-102).
 *
 * Parity of this port is pinned against the compiled reference
 * (oracle/_ref/libquids_ref.so) by tests/test_oracle_pin.py and against the
 * golden fixtures in tests/golden/.
 */
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <numeric>
#include <string_view>
#include <vector>

#include <omp.h>
#include <parallel/algorithm>
#include <parallel/numeric>

#include "oracle_api.h"

namespace port {

using mag_t = std::complex<double>;

double g_tolerance = 1e-30;
bool g_simple_truncation = true;
uint32_t g_align = 8;

uint32_t align_pad(uint32_t size) {
    if (g_align <= 1) return 0;
    uint32_t off = g_align - size % g_align;
    return off == g_align ? 0 : off;
}

/* ------------------------------------------------------------------ state */
struct state {
    uint64_t n = 0;
    double total_proba = 1;
    std::vector<mag_t> mag;
    std::vector<char> objects;
    std::vector<uint64_t> begin{0};
    std::vector<uint32_t> size;

    void append(const char *b, uint32_t sz, mag_t m) {
        uint64_t off = begin[n];
        uint64_t padded = (uint64_t)sz + align_pad(sz);
        objects.resize(off + padded);
        std::memcpy(objects.data() + off, b, sz);
        std::memset(objects.data() + off + sz, 0, padded - sz);
        mag.push_back(m);
        size.push_back(sz);
        begin.push_back(off + padded);
        ++n;
    }
    const char *obj(uint64_t i) const { return objects.data() + begin[i]; }
    char *obj(uint64_t i) { return objects.data() + begin[i]; }
};

/* ------------------------------------------------------------------ rules */
struct rule {
    virtual ~rule() {}
    virtual void num_child(const char *pb, const char *pe, uint32_t &nc, uint32_t &mcs) const = 0;
    virtual void populate(const char *pb, const char *pe, char *cb, uint32_t cid, uint32_t &sz,
                          mag_t &m) const = 0;
    virtual void populate_simple(const char *pb, const char *pe, char *cb, uint32_t cid) const {
        uint32_t sz;
        mag_t m;
        populate(pb, pe, cb, cid, sz, m);
    }
    virtual uint64_t hash(const char *b, const char *e) const {
        return std::hash<std::string_view>()(std::string_view(b, (size_t)(e - b)));
    }
};

/* quantum_computer.hpp:31-50 */
struct hadamard_rule : rule {
    uint64_t bit;
    double inv_sqrt2;
    explicit hadamard_rule(uint64_t b) : bit(b), inv_sqrt2(1 / std::sqrt(2)) {}
    void num_child(const char *pb, const char *pe, uint32_t &nc, uint32_t &mcs) const override {
        nc = 2;
        mcs = (uint32_t)(pe - pb);
    }
    void populate(const char *pb, const char *pe, char *cb, uint32_t cid, uint32_t &sz,
                  mag_t &m) const override {
        m *= (pb[bit] && cid) ? -inv_sqrt2 : inv_sqrt2;
        sz = (uint32_t)(pe - pb);
        std::memcpy(cb, pb, sz);
        cb[bit] ^= (char)(cid == 0);
    }
};

/* ----- QCGD graph encoding, qcgd.hpp:11-146 ----- */
namespace graph {
enum : int16_t { dot_l = -3, dot_r = -2, element = -1 };

struct node_name {  // 16 bytes: i16, i16, 4 bytes padding, u64
    int16_t hmlz;
    int16_t rot;
    uint32_t pad;
    uint64_t hash;
};
static_assert(sizeof(node_name) == 16, "node name layout");

inline void combine(uint64_t &seed, uint64_t v) {
    const uint64_t m = 0xc6a4a7935bd1e995ull;
    seed *= m;
    seed ^= v >> 47;
    seed *= m;
    seed ^= v;
    seed *= m;
    seed += 0xe6546b64ull;
}

inline uint16_t nodes(const char *o) { uint16_t v; std::memcpy(&v, o, 2); return v; }
inline void set_nodes(char *o, uint16_t v) { std::memcpy(o, &v, 2); }
inline bool L(const char *o, int i) { return o[2 + i] != 0; }
inline bool R(const char *o, int i) { return o[2 + nodes(o) + i] != 0; }
inline void setL(char *o, int i, bool v) { o[2 + i] = v; }
inline void setR(char *o, int i, bool v) { o[2 + nodes(o) + i] = v; }
inline uint16_t nb(const char *o, int i) { uint16_t v; std::memcpy(&v, o + 2 + 2 * nodes(o) + 2 * i, 2); return v; }
inline void set_nb(char *o, int i, uint16_t v) { std::memcpy(o + 2 + 2 * nodes(o) + 2 * i, &v, 2); }
inline char *names(char *o) { return o + 4 + 4 * nodes(o); }
inline const char *names(const char *o) { return o + 4 + 4 * nodes(o); }
inline node_name get(const char *names_base, int k) { node_name s; std::memcpy(&s, names_base + 16 * k, 16); return s; }
inline void put(char *names_base, int k, const node_name &s) { std::memcpy(names_base + 16 * k, &s, 16); }

inline node_name make_element(int16_t e) {
    node_name s{};
    s.rot = element;
    s.hash = (uint64_t)(int64_t)e;
    s.hmlz = e == 0 ? -1 : (int16_t)(e + 1);
    return s;
}
inline node_name make_dot(const node_name &x, int16_t type) {
    node_name s{};
    s.rot = type;
    s.hmlz = (type == dot_l && x.hmlz < 0) ? -1 : 1;
    s.hash = x.hash;
    combine(s.hash, (uint64_t)(int64_t)type);
    return s;
}
inline node_name make_pair(const node_name &l, const node_name &r, int16_t right_offset) {
    node_name s{};
    s.rot = right_offset;
    s.hmlz = (l.hmlz < 0 || r.hmlz < 0) ? -1 : 1;
    s.hash = l.hash;
    combine(s.hash, r.hash);
    return s;
}

/* qcgd.hpp:122-146 */
inline uint64_t hash_graph(const char *o) {
    uint64_t lh = 0, rh = 0, nh = 0;
    int n = nodes(o);
    const char *nm = names(o);
    for (int i = 0; i < n; ++i) {
        if (L(o, i)) combine(lh, (uint64_t)i);
        if (R(o, i)) combine(rh, (uint64_t)i);
        combine(nh, get(nm, nb(o, i)).hash);
    }
    combine(nh, lh);
    combine(nh, rh);
    return nh;
}

/* name algebra, qcgd.hpp:149-209; ranges are sub-node indices into a names base */
inline int copy_names(const char *src, int b, int e, char *dst, int d) {
    std::memcpy(dst + 16 * d, src + 16 * b, 16 * (size_t)(e - b));
    return d + (e - b);
}
inline int name_left(const char *src, int b, int e, char *dst, int d) {
    node_name h = get(src, b);
    if (h.rot >= 0) return copy_names(src, b + 1, b + h.rot, dst, d);
    put(dst, d, make_dot(h, dot_l));
    return copy_names(src, b, e, dst, d + 1);
}
inline int name_right(const char *src, int b, int e, char *dst, int d) {
    node_name h = get(src, b);
    if (h.rot >= 0) return copy_names(src, b + h.rot, e, dst, d);
    put(dst, d, make_dot(h, dot_r));
    return copy_names(src, b, e, dst, d + 1);
}
inline int name_merge(const char *src, int lb, int le, int rb, int re, char *dst, int d) {
    node_name l = get(src, lb), r = get(src, rb);
    if (l.rot == dot_l && r.rot == dot_r && get(src, lb + 1).hash == get(src, rb + 1).hash)
        return copy_names(src, lb + 1, le, dst, d);
    put(dst, d, make_pair(l, r, (int16_t)(le - lb + 1)));
    d = copy_names(src, lb, le, dst, d + 1);
    return copy_names(src, rb, re, dst, d);
}

inline void operations(const char *p, int i, bool &split, bool &merge) {
    merge = false;
    split = L(p, i) && R(p, i);
    if (!split && i + 1 < nodes(p)) merge = L(p, i) && R(p, i + 1) && !L(p, i + 1);
}
} // namespace graph

struct qcgd_angles {
    mag_t d, dn, dc, dnc;
    qcgd_angles(double theta, double phi, double xi) {
        d = std::polar(std::sin(theta), phi);
        dn = std::polar(std::cos(theta), xi);
        dc = std::conj(d);
        dnc = std::conj(dn);
    }
};

/* erase_create qcgd.hpp:459-532 (flip_on_xor = false) and coin :534-605 (true) */
struct flip_rule : rule, qcgd_angles {
    bool on_xor;
    flip_rule(bool x, double t, double p, double xi) : qcgd_angles(t, p, xi), on_xor(x) {}
    bool site(bool l, bool r) const { return on_xor ? (l ^ r) : !(l ^ r); }
    uint64_t hash(const char *b, const char *) const override { return graph::hash_graph(b); }
    void num_child(const char *pb, const char *pe, uint32_t &nc, uint32_t &mcs) const override {
        mcs = (uint32_t)(pe - pb);
        int n = graph::nodes(pb);
        nc = 1;
        for (int i = 0; i < n; ++i)
            if (site(graph::L(pb, i), graph::R(pb, i))) nc *= 2;  // wraps like the reference's uint
    }
    void flip(const char *pb, const char *pe, char *cb, uint32_t cid, mag_t *m) const {
        std::memcpy(cb, pb, (size_t)(pe - pb));
        int n = graph::nodes(pb);
        for (int i = 0; i < n; ++i) {
            bool l = graph::L(cb, i), r = graph::R(cb, i);
            if (!site(l, r)) continue;
            bool conj = on_xor ? l : (l && r);
            if (cid & 1) {
                if (m) *m *= conj ? dc : d;
                graph::setL(cb, i, !l);
                graph::setR(cb, i, !r);
            } else if (m) {
                *m *= conj ? -dnc : dn;
            }
            cid >>= 1;
        }
    }
    void populate(const char *pb, const char *pe, char *cb, uint32_t cid, uint32_t &sz,
                  mag_t &m) const override {
        flip(pb, pe, cb, cid, &m);
        sz = (uint32_t)(pe - pb);
    }
    void populate_simple(const char *pb, const char *pe, char *cb, uint32_t cid) const override {
        flip(pb, pe, cb, cid, nullptr);
    }
};

/* split_merge qcgd.hpp:607-1036 */
struct split_merge_rule : rule, qcgd_angles {
    split_merge_rule(double t, double p, double xi) : qcgd_angles(t, p, xi) {}
    uint64_t hash(const char *b, const char *) const override { return graph::hash_graph(b); }

    static void wrap_sites(const char *p, bool &first_split, bool &last_merge) {
        using namespace graph;
        int n = nodes(p);
        last_merge = false;
        first_split = L(p, 0) && R(p, 0);
        if (!first_split && n > 1) last_merge = R(p, 0) && L(p, n - 1) && !R(p, n - 1);
    }

    void num_child(const char *pb, const char *pe, uint32_t &nc, uint32_t &mcs) const override {
        mcs = 4 * (uint32_t)(pe - pb);
        int n = graph::nodes(pb);
        bool fs, lm;
        wrap_sites(pb, fs, lm);
        nc = (fs || lm) ? 2 : 1;
        for (int i = fs; i < n - lm; ++i) {
            bool s, mg;
            graph::operations(pb, i, s, mg);
            if (s || mg) nc *= 2;
        }
    }

    void build(const char *p, char *c, uint32_t cid, mag_t *m, uint32_t *sz) const {
        using namespace graph;
        int n = nodes(p);
        bool fs, lm;
        wrap_sites(p, fs, lm);
        bool overflow = false;

        fs = fs && (cid & 1);
        if (fs) {
            if (m) *m *= d;
            cid >>= 1;
        }
        if (lm) {
            if (cid & 1) {
                if (m) *m *= dc;
            } else {
                lm = false;
                if (m) *m *= -dnc;
            }
            cid >>= 1;
        }

        /* node count and magnitude of the remaining sites */
        int cn = n + fs - lm;
        uint32_t bits = cid;
        for (int i = fs + lm; i < n - lm; ++i) {
            bool s, mg;
            operations(p, i, s, mg);
            if (!(s || mg)) continue;
            if (bits & 1) {
                cn += (int)s - (int)mg;
                if (m) *m *= s ? d : dc;
            } else if (m) {
                *m *= s ? dn : -dnc;
            }
            bits >>= 1;
        }

        set_nodes(c, (uint16_t)cn);
        const char *pn = names(p);
        char *cnm = names(c);
        set_nb(c, 0, 0);

        if (fs) {
            node_name h = get(pn, 0);
            bool most_left_zero = true;
            if (h.rot >= 0 && get(pn, 1).hmlz > 0) most_left_zero = false;
            if (most_left_zero) {
                setL(c, 0, true); setR(c, 0, false);
                setL(c, 1, false); setR(c, 1, true);
                int e = name_left(pn, 0, nb(p, 1), cnm, 0);
                set_nb(c, 1, (uint16_t)e);
                e = name_right(pn, 0, nb(p, 1), cnm, e);
                set_nb(c, 2, (uint16_t)e);
            } else {
                overflow = true;
                setL(c, cn - 1, true); setR(c, cn - 1, false);
                setL(c, 0, false); setR(c, 0, true);
                int e = name_right(pn, 0, nb(p, 1), cnm, 0);
                set_nb(c, 1, (uint16_t)e);
            }
        }
        if (lm) {
            setL(c, 0, true); setR(c, 0, true);
            int e = name_merge(pn, nb(p, n - 1), nb(p, n), 0, nb(p, 1), cnm, 0);
            set_nb(c, 1, (uint16_t)e);
        }

        int off = (int)fs - (int)overflow;
        for (int i = fs + lm; i < n - lm; ++i) {
            bool s, mg;
            operations(p, i, s, mg);
            bool taken = false;
            if (s || mg) {
                taken = cid & 1;
                if (taken) {
                    if (s) {
                        setL(c, i + off, true); setR(c, i + off, false);
                        setL(c, i + off + 1, false); setR(c, i + off + 1, true);
                        int e = name_left(pn, nb(p, i), nb(p, i + 1), cnm, nb(c, i + off));
                        set_nb(c, i + off + 1, (uint16_t)e);
                        e = name_right(pn, nb(p, i), nb(p, i + 1), cnm, nb(c, i + off + 1));
                        set_nb(c, i + off + 2, (uint16_t)e);
                    } else {
                        setL(c, i + off, true); setR(c, i + off, true);
                        int e = name_merge(pn, nb(p, i), nb(p, i + 1), nb(p, i + 1), nb(p, i + 2), cnm,
                                           nb(c, i + off));
                        set_nb(c, i + off + 1, (uint16_t)e);
                    }
                    off += (int)s - (int)mg;
                    i += mg;
                }
                cid >>= 1;
            }
            if (!taken) {
                setL(c, i + off, L(p, i));
                setR(c, i + off, R(p, i));
                int e = copy_names(pn, nb(p, i), nb(p, i + 1), cnm, nb(c, i + off));
                set_nb(c, i + off + 1, (uint16_t)e);
            }
        }
        if (overflow) {
            int e = name_left(pn, 0, nb(p, 1), cnm, nb(c, cn - 1));
            set_nb(c, cn, (uint16_t)e);
        }
        if (sz) *sz = 4 + 4 * (uint32_t)cn + 16 * (uint32_t)nb(c, cn);
    }

    void populate(const char *pb, const char *, char *cb, uint32_t cid, uint32_t &sz,
                  mag_t &m) const override {
        build(pb, cb, cid, &m, &sz);
    }
    void populate_simple(const char *pb, const char *, char *cb, uint32_t cid) const override {
        build(pb, cb, cid, nullptr, nullptr);
    }
};

enum { R_HADAMARD = 1, R_ERASE_CREATE = 2, R_COIN = 3, R_SPLIT_MERGE = 4 };
enum { M_CNOT = 1, M_X = 2, M_Y = 3, M_Z = 4, M_STEP = 5, M_REVERSED_STEP = 6 };

std::unique_ptr<rule> make_rule(int kind, const double *p) {
    switch (kind) {
    case R_HADAMARD: return std::make_unique<hadamard_rule>((uint64_t)p[0]);
    case R_ERASE_CREATE: return std::make_unique<flip_rule>(false, p[0], p[1], p[2]);
    case R_COIN: return std::make_unique<flip_rule>(true, p[0], p[1], p[2]);
    case R_SPLIT_MERGE: return std::make_unique<split_merge_rule>(p[0], p[1], p[2]);
    }
    return nullptr;
}

/* modifiers, quantum_computer.hpp:25-75 and qcgd.hpp:443-457 */
void apply_modifier_one(int kind, const double *p, char *b, mag_t &m) {
    switch (kind) {
    case M_CNOT: b[(uint64_t)p[1]] ^= b[(uint64_t)p[0]]; break;
    case M_X: { uint64_t k = (uint64_t)p[0]; b[k] = !b[k]; break; }
    case M_Y: {
        uint64_t k = (uint64_t)p[0];
        m *= mag_t(0, 1);
        if (b[k]) m *= -1;
        b[k] = !b[k];
        break;
    }
    case M_Z: {
        uint64_t k = (uint64_t)p[0];
        if (b[k]) m *= -1;
        b[k] = !b[k];
        break;
    }
    case M_STEP: case M_REVERSED_STEP: {
        int n = graph::nodes(b);
        char *l = b + 2, *r = b + 2 + n;
        if (n == 0) break;
        if (kind == M_STEP) {
            std::rotate(l, l + 1, l + n);
            std::rotate(r, r + n - 1, r + n);
        } else {
            std::rotate(r, r + 1, r + n);
            std::rotate(l, l + n - 1, l + n);
        }
        break;
    }
    }
}

/* ------------------------------------------------------------------ step */
struct symbolic {
    uint64_t n = 0, n_after = 0;
    std::vector<mag_t> mag;
    std::vector<uint64_t> next_oid, hash, parent;
    std::vector<uint32_t> size, child_id;
};

uint64_t next_pow2(uint64_t v) { uint64_t p = 1; while (p < v) p <<= 1; return p; }
int log2_ceil(uint64_t v) { int i = 1; while ((1ull << i) < v) ++i; return i; }

/* first-insert-wins open addressing map (the semantics of the reference's
 * robin_hood::unordered_map::insert, src/quids.hpp:799) */
struct first_wins_map {
    std::vector<uint64_t> key, val;
    std::vector<uint8_t> used;
    uint64_t mask = 0;
    void reset(uint64_t n) {
        uint64_t cap = next_pow2(2 * n + 2);
        key.assign(cap, 0);
        val.assign(cap, 0);
        used.assign(cap, 0);
        mask = cap - 1;
    }
    /* returns the stored value; inserted = true if the key was new */
    uint64_t insert(uint64_t k, uint64_t v, bool &inserted) {
        uint64_t h = (k ^ (k >> 29)) * 0xbf58476d1ce4e5b9ull;
        for (uint64_t s = h & mask;; s = (s + 1) & mask) {
            if (!used[s]) { used[s] = 1; key[s] = k; val[s] = v; inserted = true; return v; }
            if (key[s] == k) { inserted = false; return val[s]; }
        }
    }
};

void normalize(state &st) {
    st.total_proba = 0;
    if (st.n == 0) return;
    double total = 0;
#pragma omp parallel for reduction(+ : total)
    for (int64_t i = 0; i < (int64_t)st.n; ++i) total += std::norm(st.mag[i]);
    st.total_proba = total;
    double f = std::sqrt(total);
    if (f != 1) {
#pragma omp parallel for
        for (int64_t i = 0; i < (int64_t)st.n; ++i) st.mag[i] /= f;
    }
}

void simulate(state &in, const rule &r, state &out, symbolic &sy, uint64_t max_num_object) {
    const uint64_t N = in.n;
    std::vector<uint32_t> nchild(N);
    uint32_t ub = 0;
    /* compute_num_child, src/quids.hpp:548-569 */
#pragma omp parallel for reduction(max : ub)
    for (int64_t i = 0; i < (int64_t)N; ++i) {
        uint32_t mcs;
        r.num_child(in.obj(i), in.obj(i) + in.size[i], nchild[i], mcs);
        ub = std::max(ub, mcs);
    }

    /* parent pre-truncation, src/quids.hpp:613-642 (simple truncation) */
    std::vector<uint64_t> toid(N);
    std::iota(toid.begin(), toid.end(), 0);
    uint64_t NP = N;
    if (max_num_object < N) {
        __gnu_parallel::nth_element(toid.begin(), toid.begin() + max_num_object, toid.end(),
                                    [&](uint64_t a, uint64_t b) {
                                        return std::norm(in.mag[a]) > std::norm(in.mag[b]);
                                    });
        NP = max_num_object;
    }

    /* symbolic iteration, src/quids.hpp:647-721 */
    std::vector<uint64_t> cbeg(NP + 1, 0);
    for (uint64_t i = 0; i < NP; ++i) cbeg[i + 1] = cbeg[i] + nchild[toid[i]];
    const uint64_t NC = cbeg[NP];
    sy.n = NC;
    sy.mag.resize(NC);
    sy.next_oid.resize(NC);
    sy.hash.resize(NC);
    sy.parent.resize(NC);
    sy.size.resize(NC);
    sy.child_id.resize(NC);

#pragma omp parallel
    {
        std::vector<char> scratch((size_t)ub + 16);
#pragma omp for
        for (int64_t i = 0; i < (int64_t)NP; ++i) {
            uint64_t oid = toid[i];
            for (uint64_t c = cbeg[i]; c < cbeg[i + 1]; ++c) {
                sy.parent[c] = oid;
                sy.child_id[c] = (uint32_t)(c - cbeg[i]);
            }
        }
#pragma omp for
        for (int64_t c = 0; c < (int64_t)NC; ++c) {
            uint64_t p = sy.parent[c];
            sy.mag[c] = in.mag[p];
            r.populate(in.obj(p), in.obj(p) + in.size[p], scratch.data(), sy.child_id[c], sy.size[c],
                       sy.mag[c]);
            sy.hash[c] = r.hash(scratch.data(), scratch.data() + sy.size[c]);
        }
    }

    /* compute_collisions, src/quids.hpp:726-824 */
    if (NC > 0) {
        int T = omp_get_max_threads();
        int nbucket = (int)next_pow2((uint64_t)32 * T);
        int shift = 64 - log2_ceil((uint64_t)nbucket);
        auto key_of = [&](uint64_t c) -> int { return (int)(sy.hash[c] >> shift); };
        /* per-thread counting partition, src/utils/algorithm.hpp:170-227: buckets
         * in key order, threads in order within a bucket, descending symbolic index
         * within each (bucket, thread) cell */
        std::vector<uint64_t> count((size_t)nbucket * T, 0);
#pragma omp parallel num_threads(T)
        {
            int t = omp_get_thread_num();
            int64_t b = (int64_t)NC * t / T, e = (int64_t)NC * (t + 1) / T;
            for (int64_t c = b; c < e; ++c) ++count[(size_t)key_of(c) * T + t];
        }
        std::partial_sum(count.begin(), count.end(), count.begin());
        std::vector<uint64_t> bucket_begin(nbucket + 1, 0);
        for (int k = 1; k <= nbucket; ++k) bucket_begin[k] = count[(size_t)k * T - 1];
#pragma omp parallel num_threads(T)
        {
            int t = omp_get_thread_num();
            int64_t b = (int64_t)NC * t / T, e = (int64_t)NC * (t + 1) / T;
            for (int64_t c = b; c < e; ++c) sy.next_oid[--count[(size_t)key_of(c) * T + t]] = (uint64_t)c;
        }
        /* first-insert-wins elimination per bucket, src/quids.hpp:785-809 */
#pragma omp parallel
        {
            first_wins_map map;
#pragma omp for schedule(dynamic, 1)
            for (int k = 0; k < nbucket; ++k) {
                uint64_t b = bucket_begin[k], e = bucket_begin[k + 1];
                map.reset(e - b);
                for (uint64_t i = b; i < e; ++i) {
                    uint64_t c = sy.next_oid[i];
                    bool inserted;
                    uint64_t first = map.insert(sy.hash[c], c, inserted);
                    if (!inserted) {
                        sy.mag[first] += sy.mag[c];
                        sy.mag[c] = 0;
                    }
                }
            }
        }
        /* zero elimination, src/quids.hpp:819-823 */
        double tol = g_tolerance;
        auto it = __gnu_parallel::partition(sy.next_oid.begin(), sy.next_oid.end(),
                                            [&](uint64_t c) { return std::norm(sy.mag[c]) > tol; });
        sy.n_after = (uint64_t)(it - sy.next_oid.begin());
    } else {
        sy.n_after = 0;
    }

    /* truncation, src/quids.hpp:866-900 (simple truncation) */
    uint64_t NS = sy.n_after;
    if (max_num_object < NS) {
        __gnu_parallel::nth_element(sy.next_oid.begin(), sy.next_oid.begin() + max_num_object,
                                    sy.next_oid.begin() + NS, [&](uint64_t a, uint64_t b) {
                                        return std::norm(sy.mag[a]) > std::norm(sy.mag[b]);
                                    });
        NS = max_num_object;
    }

    /* finalize, src/quids.hpp:905-968 */
    __gnu_parallel::sort(sy.next_oid.begin(), sy.next_oid.begin() + NS);
    out.n = NS;
    out.mag.resize(NS);
    out.size.resize(NS);
    out.begin.assign(NS + 1, 0);
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)NS; ++i) {
        uint64_t c = sy.next_oid[i];
        out.size[i] = sy.size[c];
        out.begin[i + 1] = (uint64_t)sy.size[c] + align_pad(sy.size[c]);
        out.mag[i] = sy.mag[c];
    }
    std::partial_sum(out.begin.begin(), out.begin.end(), out.begin.begin());
    out.objects.assign(out.begin[NS], 0);
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)NS; ++i) {
        uint64_t c = sy.next_oid[i];
        uint64_t p = sy.parent[c];
        r.populate_simple(in.obj(p), in.obj(p) + in.size[p], out.obj(i), sy.child_id[c]);
    }
    normalize(out);
}

symbolic &scratch() {
    static symbolic sy;
    return sy;
}

} // namespace port

extern "C" {

void *qo_state_new(void) { return new port::state(); }
void qo_state_free(void *st) { delete (port::state *)st; }

int qo_state_load(void *st, uint64_t n, const uint8_t *objects, const uint64_t *begin,
                  const uint32_t *size, const double *mag) {
    auto *s = (port::state *)st;
    for (uint64_t i = 0; i < n; ++i)
        s->append((const char *)objects + begin[i], size[i], port::mag_t(mag[2 * i], mag[2 * i + 1]));
    return 0;
}

uint64_t qo_state_num_object(void *st) { return ((port::state *)st)->n; }

uint64_t qo_state_num_bytes(void *st) {
    auto *s = (port::state *)st;
    uint64_t t = 0;
    for (uint64_t i = 0; i < s->n; ++i) t += (uint64_t)s->size[i] + port::align_pad(s->size[i]);
    return t;
}

int qo_state_store(void *st, uint8_t *objects, uint64_t *begin, uint32_t *size, double *mag) {
    auto *s = (port::state *)st;
    uint64_t off = 0;
    for (uint64_t i = 0; i < s->n; ++i) {
        uint32_t sz = s->size[i];
        uint64_t padded = (uint64_t)sz + port::align_pad(sz);
        begin[i] = off;
        size[i] = sz;
        mag[2 * i] = s->mag[i].real();
        mag[2 * i + 1] = s->mag[i].imag();
        std::memcpy(objects + off, s->obj(i), sz);
        std::memset(objects + off + sz, 0, padded - sz);
        off += padded;
    }
    begin[s->n] = off;
    return 0;
}

double qo_state_total_proba(void *st) { return ((port::state *)st)->total_proba; }

void qo_set_globals(double tolerance, int simple_truncation, uint32_t align_byte_length) {
    port::g_tolerance = tolerance;
    port::g_simple_truncation = simple_truncation != 0;
    port::g_align = align_byte_length;
}

void qo_set_threads(int n) { omp_set_num_threads(n); }
int qo_get_threads(void) { return omp_get_max_threads(); }

int qo_simulate(void *in, int rule_kind, const double *params, void *out,
                uint64_t max_num_object, uint64_t *counters) {
    if (!port::g_simple_truncation) return -1;  // probabilistic truncation is not restated
    auto r = port::make_rule(rule_kind, params);
    if (!r || in == out) return -1;
    auto &sy = port::scratch();
    port::simulate(*(port::state *)in, *r, *(port::state *)out, sy, max_num_object);
    if (counters) {
        counters[0] = sy.n;
        counters[1] = sy.n_after;
    }
    return 0;
}

int qo_modifier(void *st, int modifier_kind, const double *params) {
    if (modifier_kind < 1 || modifier_kind > 6) return -1;
    auto *s = (port::state *)st;
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)s->n; ++i)
        port::apply_modifier_one(modifier_kind, params, s->obj(i), s->mag[i]);
    return 0;
}

uint64_t qo_hash_bytes(const uint8_t *b, uint64_t len) {
    return std::hash<std::string_view>()(std::string_view((const char *)b, len));
}

uint64_t qo_qcgd_hash_graph(const uint8_t *b) { return port::graph::hash_graph((const char *)b); }

int qo_num_child(int rule_kind, const double *params, const uint8_t *obj, uint32_t size,
                 uint32_t *num_child, uint32_t *max_child_size) {
    auto r = port::make_rule(rule_kind, params);
    if (!r) return -1;
    r->num_child((const char *)obj, (const char *)obj + size, *num_child, *max_child_size);
    return 0;
}

int qo_populate_child(int rule_kind, const double *params, const uint8_t *parent, uint32_t psize,
                      uint32_t child_id, uint8_t *child, uint32_t *csize, double *mag) {
    auto r = port::make_rule(rule_kind, params);
    if (!r) return -1;
    port::mag_t m(mag[0], mag[1]);
    r->populate((const char *)parent, (const char *)parent + psize, (char *)child, child_id, *csize, m);
    mag[0] = m.real();
    mag[1] = m.imag();
    return 0;
}

uint64_t qo_rule_hash(int rule_kind, const double *params, const uint8_t *obj, uint32_t size) {
    auto r = port::make_rule(rule_kind, params);
    if (!r) return 0;
    return r->hash((const char *)obj, (const char *)obj + size);
}

} // extern "C"
