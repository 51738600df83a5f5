// Host build of the device rule headers (quids_gb300/csrc/rules_*.cuh) for
// CPU tests: the same source the GPU kernels instantiate, compiled by g++,
// exposed through a small C interface so tests can compare every rule
// callback with the oracle on the CPU.
#include <cstdint>
#include "../../quids_gb300/csrc/rules_qc.cuh"
#include "../../quids_gb300/csrc/rules_qcgd.cuh"
#include <cmath>
#include <complex>

using namespace qd;

namespace {
qcgd::factors factors(const double *p) {
    std::complex<double> d = std::polar(std::sin(p[0]), p[1]);
    std::complex<double> dn = std::polar(std::cos(p[0]), p[2]);
    std::complex<double> ndnc = -std::conj(dn);
    return {{d.real(), d.imag()}, {d.real(), -d.imag()}, {dn.real(), dn.imag()}, {ndnc.real(), ndnc.imag()}};
}
template <class F> int with_rule(int kind, const double *p, F f) {
    switch (kind) {
    case 1: { rules::hadamard h{(uint64_t)p[0], 1 / std::sqrt(2)}; return f(h); }
    case 2: return f(qcgd::erase_create{factors(p)});
    case 3: return f(qcgd::coin{factors(p)});
    case 4: return f(qcgd::split_merge{factors(p)});
    }
    return -1;
}
}

extern "C" {
int shim_num_child(int kind, const double *p, const uint8_t *o, uint32_t sz, uint32_t *nc, uint32_t *mcs) {
    return with_rule(kind, p, [&](auto r) { r.get_num_child((const char *)o, (const char *)o + sz, *nc, *mcs); return 0; });
}
int shim_populate_child(int kind, const double *p, const uint8_t *o, uint32_t sz, uint32_t cid, uint8_t *c,
                        uint32_t *csz, double *mag) {
    return with_rule(kind, p, [&](auto r) {
        mag_t m{mag[0], mag[1]};
        r.populate_child((const char *)o, (const char *)o + sz, (char *)c, cid, *csz, m);
        mag[0] = m.re; mag[1] = m.im;
        return 0;
    });
}
int shim_populate_child_simple(int kind, const double *p, const uint8_t *o, uint32_t sz, uint32_t cid, uint8_t *c) {
    return with_rule(kind, p, [&](auto r) { r.populate_child_simple((const char *)o, (const char *)o + sz, (char *)c, cid); return 0; });
}
uint64_t shim_hash_child(int kind, const double *p, const uint8_t *o, uint32_t sz, uint32_t cid, uint32_t *csz,
                         double *mag) {
    uint64_t h = 0;
    with_rule(kind, p, [&](auto r) {
        mag_t m{mag[0], mag[1]};
        h = r.hash_child((const char *)o, (const char *)o + sz, cid, *csz, m);
        mag[0] = m.re; mag[1] = m.im;
        return 0;
    });
    return h;
}
// the grouped expansion of the QCGD rules (kind 2, 3, 4) with H = h (2 or 3)
// for the children whose ids share the low s-h bits e: writes 2^h hashes and
// 2^(h+1) doubles (child e + j 2^(s-h) at slot j); returns s, or -1
int shim_expand_group(int kind, int h, const double *p, const uint8_t *o, uint32_t sz, uint32_t e,
                      const double *mag, uint64_t *hashes, double *mags) {
    auto run = [&](auto r) {
        uint32_t nc, mcs;
        r.get_num_child((const char *)o, (const char *)o + sz, nc, mcs);
        int s = 0;
        while ((1u << s) < nc) ++s;
        auto emit = [&](uint32_t j, uint64_t hv, const mag_t &m, uint32_t) {
            hashes[j] = hv;
            mags[2 * j] = m.re;
            mags[2 * j + 1] = m.im;
        };
        const mag_t pm{mag[0], mag[1]};
        if (h == 2) r.template expand_group<2>((const char *)o, (const char *)o + sz, e, s, pm, emit);
        else r.template expand_group<3>((const char *)o, (const char *)o + sz, e, s, pm, emit);
        return s;
    };
    if (kind == 2) return run(qcgd::erase_create{factors(p)});
    if (kind == 3) return run(qcgd::coin{factors(p)});
    if (kind == 4) return run(qcgd::split_merge{factors(p)});
    return -1;
}
uint64_t shim_murmur(const uint8_t *b, uint64_t len) { return murmur64a((const char *)b, len); }
// a collision group's sum as the table forms it: from_fix of the 128-bit sum
// of to_fix(x_i, F), F = fix_scale(maxabs, n_scale)
double shim_fix_sum(const double *x, uint64_t n, double maxabs, uint64_t n_scale, int *F_out) {
    const int F = fix_scale(maxabs, n_scale);
    fix128 s{0, 0};
    for (uint64_t i = 0; i < n; ++i) s = fix_add(s, to_fix(x[i], F));
    if (F_out) *F_out = F;
    return from_fix(s, F);
}
uint64_t shim_hash_graph(const uint8_t *b) { return qcgd::hash_graph((const char *)b); }
int shim_modifier(int kind, const double *p, uint8_t *o, uint32_t sz, double *mag) {
    mag_t m{mag[0], mag[1]};
    char *b = (char *)o, *e = b + sz;
    switch (kind) {
    case 1: rules::cnot{(uint64_t)p[0], (uint64_t)p[1]}(b, e, m); break;
    case 2: rules::xgate{(uint64_t)p[0]}(b, e, m); break;
    case 3: rules::ygate{(uint64_t)p[0]}(b, e, m); break;
    case 4: rules::zgate{(uint64_t)p[0]}(b, e, m); break;
    case 5: qcgd::step{}(b, e, m); break;
    case 6: qcgd::reversed_step{}(b, e, m); break;
    default: return -1;
    }
    mag[0] = m.re; mag[1] = m.im;
    return 0;
}
}
