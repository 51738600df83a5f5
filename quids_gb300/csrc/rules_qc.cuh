// rules_qc.cuh -- the quantum_computer rules as device rules.
//
// Reference: src/rules/quantum_computer.hpp.  Objects are one byte per qubit.
// Device rules keep the reference's callback names and argument meaning
// (quids::rule, src/quids.hpp:105-146):
//   get_num_child(parent_begin, parent_end, num_child, max_child_size)
//   populate_child(parent_begin, parent_end, child_begin, child_id, size, mag)
// and may add
//   populate_child_simple(...)             (bytes only)
//   hasher(object_begin, object_end)       (default: std::hash<string_view>)
//   hash_child(parent_begin, parent_end, child_id, size, mag) -> hash
// The last one is this library's fast path: the child's hash, size and
// magnitude without materialising its bytes; it must equal
// hasher(populate_child(...)).
#pragma once
#include "qd_common.cuh"

namespace qd::rules {

// quantum_computer::hadamard, src/rules/quantum_computer.hpp:31-50.
// Two children of the parent's size; child 0 flips the target byte
// (child[bit] ^= !child_id) and both get mag *= +-1/sqrt(2), negative for
// child 1 of a parent whose target byte is set.
struct hadamard {
    uint64_t bit;
    double inv_sqrt2;  // 1/std::sqrt(2) evaluated on the host, as the reference's static

    // objects too short for the target qubit are rejected (the reference
    // would write past the object)
    QD_HD bool fits(uint32_t size) const { return bit < size; }

    QD_HD void get_num_child(const char *pb, const char *pe, uint32_t &num_child,
                             uint32_t &max_child_size) const {
        num_child = 2;
        max_child_size = (uint32_t)(pe - pb);
    }
    QD_HD void populate_child(const char *pb, const char *pe, char *cb, uint32_t child_id,
                              uint32_t &size, mag_t &mag) const {
        mag = cscale(mag, (pb[bit] && child_id) ? -inv_sqrt2 : inv_sqrt2);
        size = (uint32_t)(pe - pb);
        copy_bytes(cb, pb, size);
        cb[bit] ^= (char)(child_id == 0);
    }
    QD_HD void populate_child_simple(const char *pb, const char *pe, char *cb,
                                     uint32_t child_id) const {
        copy_bytes(cb, pb, (uint32_t)(pe - pb));
        cb[bit] ^= (char)(child_id == 0);
    }
    QD_HD uint64_t hash_child(const char *pb, const char *pe, uint32_t child_id, uint32_t &size,
                              mag_t &mag) const {
        mag = cscale(mag, (pb[bit] && child_id) ? -inv_sqrt2 : inv_sqrt2);
        size = (uint32_t)(pe - pb);
        return murmur64a_patched(pb, size, bit, (uint8_t)(child_id == 0));
    }
};

// ---------------------------------------------------------------- modifiers
// modifier_t (src/quids.hpp:86): operator()(begin, end, mag), in place.

// cnot(control, bit): begin[bit] ^= begin[control]   (:25-29)
struct cnot {
    uint64_t control, bit;
    QD_HD bool fits(uint32_t size) const { return bit < size && control < size; }
    QD_HD void operator()(char *b, char *, mag_t &) const { b[bit] ^= b[control]; }
};
// Xgate: begin[bit] = !begin[bit]   (:52-56)
struct xgate {
    uint64_t bit;
    QD_HD bool fits(uint32_t size) const { return bit < size; }
    QD_HD void operator()(char *b, char *, mag_t &) const { b[bit] = !b[bit]; }
};
// Ygate: mag *= i; negate if the bit is set; flip the bit   (:58-66)
struct ygate {
    uint64_t bit;
    QD_HD bool fits(uint32_t size) const { return bit < size; }
    QD_HD void operator()(char *b, char *, mag_t &m) const {
        m = cmul(m, mag_t{0.0, 1.0});
        if (b[bit]) m = cscale(m, -1.0);
        b[bit] = !b[bit];
    }
};
// Zgate: negate if the bit is set AND flip the bit (the reference's Z also
// flips, :68-75; reproduced for parity)
struct zgate {
    uint64_t bit;
    QD_HD bool fits(uint32_t size) const { return bit < size; }
    QD_HD void operator()(char *b, char *, mag_t &m) const {
        if (b[bit]) m = cscale(m, -1.0);
        b[bit] = !b[bit];
    }
};

// probability observable of one qubit: 1 when its byte is non-zero
struct obs_bit {
    uint64_t bit;
    QD_HD double operator()(const char *b, const char *e) const {
        return (bit < (uint64_t)(e - b) && b[bit]) ? 1.0 : 0.0;
    }
};

}  // namespace qd::rules
