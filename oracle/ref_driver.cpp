/*
 * Driver that exposes the reference QuIDS headers through oracle_api.h.
 *
 * TEST INFRASTRUCTURE (see oracle_api.h).  Built by oracle/Makefile with
 * -I<reference>/src; it includes the reference headers where they lie and
 * contains no reference code of its own.  Every call goes through the
 * reference's public API:
 *   quids::it_t::append / get_object            src/quids.hpp:174-188, :254-258
 *   quids::simulate(it, rule, next, sy, max)    src/quids.hpp:448-543
 *   quids::simulate(it, modifier)               src/quids.hpp:436-438
 *   rules                                       src/rules/quantum_computer.hpp,
 *                                               src/rules/qcgd.hpp
 */
#include "quids.hpp"
#include "rules/quantum_computer.hpp"
#include "rules/qcgd.hpp"

#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <omp.h>
#include <vector>

#include "oracle_api.h"

namespace {

enum { R_HADAMARD = 1, R_ERASE_CREATE = 2, R_COIN = 3, R_SPLIT_MERGE = 4 };
enum { M_CNOT = 1, M_X = 2, M_Y = 3, M_Z = 4, M_STEP = 5, M_REVERSED_STEP = 6 };

std::unique_ptr<quids::rule_t> make_rule(int kind, const double *p) {
    namespace qc = quids::rules::quantum_computer;
    namespace qg = quids::rules::qcgd;
    switch (kind) {
    case R_HADAMARD: return std::make_unique<qc::hadamard>((size_t)p[0]);
    case R_ERASE_CREATE: return std::make_unique<qg::erase_create>(p[0], p[1], p[2]);
    case R_COIN: return std::make_unique<qg::coin>(p[0], p[1], p[2]);
    case R_SPLIT_MERGE: return std::make_unique<qg::split_merge>(p[0], p[1], p[2]);
    }
    return nullptr;
}

quids::modifier_t make_modifier(int kind, const double *p) {
    namespace qc = quids::rules::quantum_computer;
    namespace qg = quids::rules::qcgd;
    switch (kind) {
    case M_CNOT: return qc::cnot((uint32_t)p[0], (uint32_t)p[1]);
    case M_X: return qc::Xgate((size_t)p[0]);
    case M_Y: return qc::Ygate((size_t)p[0]);
    case M_Z: return qc::Zgate((size_t)p[0]);
    case M_STEP: return qg::step;
    case M_REVERSED_STEP: return qg::reversed_step;
    }
    return nullptr;
}

uint64_t padded(uint64_t size) { return size + quids::get_alignment_offset((uint)size); }

quids::sy_it_t &symbolic_scratch() {
    static quids::sy_it_t sy;
    return sy;
}

} // namespace

extern "C" {

void *qo_state_new(void) { return new quids::it_t(); }
void qo_state_free(void *st) { delete (quids::it_t *)st; }

int qo_state_load(void *st, uint64_t n, const uint8_t *objects, const uint64_t *begin,
                  const uint32_t *size, const double *mag) {
    auto *it = (quids::it_t *)st;
    for (uint64_t i = 0; i < n; ++i) {
        const char *b = (const char *)objects + begin[i];
        it->append(b, b + size[i], quids::mag_t(mag[2 * i], mag[2 * i + 1]));
    }
    return 0;
}

uint64_t qo_state_num_object(void *st) { return ((quids::it_t *)st)->num_object; }

uint64_t qo_state_num_bytes(void *st) {
    auto *it = (quids::it_t *)st;
    uint64_t total = 0;
    for (size_t i = 0; i < it->num_object; ++i) {
        char const *b;
        uint sz;
        quids::mag_t m;
        it->get_object(i, b, sz, m);
        total += padded(sz);
    }
    return total;
}

int qo_state_store(void *st, uint8_t *objects, uint64_t *begin, uint32_t *size, double *mag) {
    auto const *it = (quids::it_t const *)st;
    uint64_t off = 0;
    for (size_t i = 0; i < it->num_object; ++i) {
        char const *b;
        uint sz;
        quids::mag_t m;
        it->get_object(i, b, sz, m);
        begin[i] = off;
        size[i] = sz;
        mag[2 * i] = m.real();
        mag[2 * i + 1] = m.imag();
        std::memcpy(objects + off, b, sz);
        std::memset(objects + off + sz, 0, padded(sz) - sz);
        off += padded(sz);
    }
    begin[it->num_object] = off;
    return 0;
}

double qo_state_total_proba(void *st) { return ((quids::it_t *)st)->total_proba; }

void qo_set_globals(double tolerance, int simple_truncation, uint32_t align_byte_length) {
    quids::tolerance = tolerance;
    quids::simple_truncation = simple_truncation != 0;
    quids::align_byte_length = align_byte_length;
}

void qo_set_threads(int n) { omp_set_num_threads(n); }
int qo_get_threads(void) { return omp_get_max_threads(); }

int qo_simulate(void *in, int rule_kind, const double *params, void *out,
                uint64_t max_num_object, uint64_t *counters) {
    auto rule = make_rule(rule_kind, params);
    if (!rule) return -1;
    auto &sy = symbolic_scratch();
    quids::simulate(*(quids::it_t *)in, rule.get(), *(quids::it_t *)out, sy,
                    (size_t)max_num_object);
    if (counters) {
        counters[0] = sy.num_object;
        counters[1] = sy.num_object_after_interferences;
    }
    return 0;
}

int qo_modifier(void *st, int modifier_kind, const double *params) {
    auto m = make_modifier(modifier_kind, params);
    if (!m) return -1;
    quids::simulate(*(quids::it_t *)st, m);
    return 0;
}

uint64_t qo_hash_bytes(const uint8_t *b, uint64_t len) {
    return std::hash<std::string_view>()(std::string_view((const char *)b, len));
}

uint64_t qo_qcgd_hash_graph(const uint8_t *b) {
    return quids::rules::qcgd::graphs::hash_graph((const char *)b);
}

int qo_num_child(int rule_kind, const double *params, const uint8_t *obj, uint32_t size,
                 uint32_t *num_child, uint32_t *max_child_size) {
    auto rule = make_rule(rule_kind, params);
    if (!rule) return -1;
    uint nc, mcs;
    rule->get_num_child((const char *)obj, (const char *)obj + size, nc, mcs);
    *num_child = nc;
    *max_child_size = mcs;
    return 0;
}

int qo_populate_child(int rule_kind, const double *params, const uint8_t *parent, uint32_t psize,
                      uint32_t child_id, uint8_t *child, uint32_t *csize, double *mag) {
    auto rule = make_rule(rule_kind, params);
    if (!rule) return -1;
    uint sz = 0;
    quids::mag_t m(mag[0], mag[1]);
    rule->populate_child((const char *)parent, (const char *)parent + psize, (char *)child,
                         child_id, sz, m);
    *csize = sz;
    mag[0] = m.real();
    mag[1] = m.imag();
    return 0;
}

uint64_t qo_rule_hash(int rule_kind, const double *params, const uint8_t *obj, uint32_t size) {
    auto rule = make_rule(rule_kind, params);
    if (!rule) return 0;
    return rule->hasher((const char *)obj, (const char *)obj + size);
}

// Reference-only (the QCGD simulation string, src/rules/qcgd.hpp:1086-1166):
// flags::read_n_iter on `settings` (it seeds rand()) then flags::read_state
// on `state_arg` into st.
int qo_ref_read_state(const char *settings, const char *state_arg, void *st) {
    quids::rules::qcgd::flags::read_n_iter(settings);
    quids::rules::qcgd::flags::read_state(state_arg, *(quids::it_t *)st);
    return 0;
}

// flags::read_rule: per entry its n_iter, whether it is a rule, and for
// rules the magnitudes of children 0..3 of `probe` (from magnitude 1) under
// the rule and under its reversed form: out[entry][2][4] complex.
int qo_ref_read_rules(const char *rules_arg, const uint8_t *probe, uint32_t size, int max_entries, int *n_iter,
                      int *is_rule, double *out) {
    auto sim = quids::rules::qcgd::flags::read_rule(rules_arg);
    int n = 0;
    for (auto &e : sim) {
        if (n >= max_entries) break;
        n_iter[n] = std::get<0>(e);
        is_rule[n] = std::get<1>(e) ? 1 : 0;
        if (is_rule[n]) {
            quids::rule_t *rs[2] = {std::get<3>(e), std::get<5>(e)};
            for (int v = 0; v < 2; ++v) {
                uint nc, mcs;
                rs[v]->get_num_child((const char *)probe, (const char *)probe + size, nc, mcs);
                std::vector<char> child(mcs + 64);
                for (uint c = 0; c < 4; ++c) {
                    double *o = out + ((size_t)n * 8 + v * 4 + c) * 2;
                    if (c >= nc) {
                        o[0] = o[1] = 0;
                        continue;
                    }
                    uint sz = 0;
                    quids::mag_t m(1, 0);
                    rs[v]->populate_child((const char *)probe, (const char *)probe + size, child.data(), c, sz, m);
                    o[0] = m.real();
                    o[1] = m.imag();
                }
            }
        }
        ++n;
    }
    return n;
}

} // extern "C"
