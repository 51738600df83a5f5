// factories.cuh -- built-in rules formed on the host from
// quids_gpu_rule_params exactly as the reference's constructors form them
// (src/rules/quantum_computer.hpp, src/rules/qcgd.hpp).
#pragma once
#include <cmath>
#include <complex>

#include "../../include/quids_gpu.h"
#include "rules_qc.cuh"
#include "rules_qcgd.cuh"

namespace qd::host {

inline qcgd::factors make_factors(const quids_gpu_rule_params *p) {
    // src/rules/qcgd.hpp:466-471
    std::complex<double> d = std::polar(std::sin(p->theta), p->phi);
    std::complex<double> dn = std::polar(std::cos(p->theta), p->xi);
    std::complex<double> dc = std::conj(d), dnc = std::conj(dn);
    std::complex<double> ndnc = -dnc;
    qcgd::factors f;
    f.d = {d.real(), d.imag()};
    f.dc = {dc.real(), dc.imag()};
    f.dn = {dn.real(), dn.imag()};
    f.ndnc = {ndnc.real(), ndnc.imag()};
    return f;
}

inline rules::hadamard make_hadamard(const quids_gpu_rule_params *p) {
    rules::hadamard h;
    h.bit = p->bit;
    h.inv_sqrt2 = 1 / std::sqrt(2);  // quantum_computer.hpp:41
    return h;
}

// f(rule) for the rule of `kind` built from p
template <class F>
int dispatch_rule(int kind, const quids_gpu_rule_params *p, F &&f) {
    if (!p) return QUIDS_ERR_BAD_ARG;
    switch (kind) {
    case QUIDS_RULE_HADAMARD: return f(make_hadamard(p));
    case QUIDS_RULE_QCGD_ERASE_CREATE: return f(qcgd::erase_create{make_factors(p)});
    case QUIDS_RULE_QCGD_COIN: return f(qcgd::coin{make_factors(p)});
    case QUIDS_RULE_QCGD_SPLIT_MERGE: return f(qcgd::split_merge{make_factors(p)});
    }
    return QUIDS_ERR_BAD_ARG;
}

}  // namespace qd::host
