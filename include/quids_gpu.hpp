/*
 * quids_gpu.hpp -- header-only C++ API of the GB300 rule step, with the
 * names and argument meaning of the reference's header-only library
 * (jolatechno/QuIDS, src/quids.hpp):
 *
 *   quids::gpu::it_t / sy_it_t           iteration, symbolic_iteration  src/quids.hpp:149-429
 *   quids::gpu::simulate(it, rule, next, sy, max_num_object)             src/quids.hpp:448-543
 *   quids::gpu::simulate(it, modifier)                                   src/quids.hpp:436-438
 *   quids::gpu::tolerance, simple_truncation, align_byte_length          src/quids.hpp:59-75
 *   quids::gpu::rules::quantum_computer / qcgd                           src/rules/*.hpp
 *
 * A rule is any struct with the reference's callbacks (class rule,
 * src/quids.hpp:105-146) as __host__ __device__ const members:
 *
 *   void get_num_child(char const *parent_begin, char const *parent_end,
 *                      uint &num_child, uint &max_child_size) const;
 *   void populate_child(char const *parent_begin, char const *parent_end,
 *                       char *const child_begin, uint const child_id,
 *                       uint &size, mag_t &mag) const;
 *   optional: void populate_child_simple(parent_begin, parent_end, child_begin, child_id) const;
 *   optional: size_t hasher(char const *begin, char const *end) const;
 *             (default: std::hash<std::string_view> of the bytes, as the reference)
 *   optional: this library's fast path
 *             size_t hash_child(parent_begin, parent_end, child_id, uint &size, mag_t &mag) const;
 *             equal to hasher(populate_child(...)) without writing the child.
 *
 * simulate<Rule> instantiates the whole GPU step for that struct in the
 * caller's translation unit (compile it with nvcc for sm_103a, -std=c++17
 * --expt-relaxed-constexpr, and link libquids_gb300.so, which provides the
 * non-template C ABI of quids_gpu.h).  A modifier is any struct with a
 * __host__ __device__ `void operator()(char *begin, char *end, mag_t &mag) const`.
 *
 * mag_t is complex<double> as the reference computes it (no FMA contraction)
 * with the usual operators; its parts are .re and .im.
 *
 * Objects live in device memory.  it_t keeps a host copy for append, pop and
 * get_object: appended objects go to the device before the next simulate;
 * get_object reads the state back once after each step.  Failures throw
 * quids::gpu::error (the reference throws std::runtime_error on allocation
 * failure, src/utils/vector.hpp:127) carrying the library's status code.
 */
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "quids_gpu.h"
#include "../quids_gb300/csrc/factories.cuh"
#include "../quids_gb300/csrc/ranges.cuh"

// complex<double> arithmetic on mag_t for user rules, each product and sum
// rounded separately like libstdc++ on x86-64 (found by argument-dependent
// lookup from any namespace)
namespace qd {
QD_HD mag_t operator+(mag_t a, mag_t b) { return {dadd(a.re, b.re), dadd(a.im, b.im)}; }
QD_HD mag_t operator-(mag_t a, mag_t b) { return {dsub(a.re, b.re), dsub(a.im, b.im)}; }
QD_HD mag_t operator-(mag_t a) { return cneg(a); }
QD_HD mag_t operator*(mag_t a, mag_t b) { return cmul(a, b); }
QD_HD mag_t operator*(mag_t a, double s) { return cscale(a, s); }
QD_HD mag_t operator*(double s, mag_t a) { return cscale(a, s); }
QD_HD mag_t operator/(mag_t a, double s) {
#ifdef __CUDA_ARCH__
    return {__ddiv_rn(a.re, s), __ddiv_rn(a.im, s)};
#else
    return {a.re / s, a.im / s};
#endif
}
QD_HD mag_t &operator+=(mag_t &a, mag_t b) { return a = a + b; }
QD_HD mag_t &operator-=(mag_t &a, mag_t b) { return a = a - b; }
QD_HD mag_t &operator*=(mag_t &a, mag_t b) { return a = cmul(a, b); }
QD_HD mag_t &operator*=(mag_t &a, double s) { return a = cscale(a, s); }
QD_HD mag_t &operator/=(mag_t &a, double s) { return a = a / s; }
QD_HD bool operator==(mag_t a, mag_t b) { return a.re == b.re && a.im == b.im; }
QD_HD bool operator!=(mag_t a, mag_t b) { return !(a == b); }
QD_HD double real(mag_t a) { return a.re; }
QD_HD double imag(mag_t a) { return a.im; }
QD_HD double norm(mag_t a) { return cnorm(a); }
QD_HD mag_t conj(mag_t a) { return cconj(a); }
}  // namespace qd

namespace quids::gpu {

using mag_t = qd::mag_t;
using uint = unsigned int;
typedef std::function<double(char const *object_begin, char const *object_end)> observable_t;
typedef std::function<void(const char *step)> debug_t;

// ---------------------------------------------------------------- globals
// The reference's knobs (src/quids.hpp:59-75), with its defaults; read at
// every simulate() call.
inline uint align_byte_length = 8;    // ALIGNMENT_BYTE_LENGTH
inline double tolerance = 1e-30;      // TOLERANCE: children of norm <= tolerance are dropped
#ifdef SIMPLE_TRUNCATION
inline bool simple_truncation = true;  // keep the largest norms
#else
inline bool simple_truncation = false;  // probabilistic truncation
#endif
inline uint64_t truncation_seed = 0;  // generator of the probabilistic truncation (no counterpart: rand())
inline double table_load_factor = 0.5;  // collision table maximum load (no counterpart)
inline int device = 0;                // the GPU of default_context()

// ----------------------------------------------------------------- errors
class error : public std::runtime_error {
public:
    int status;
    error(int s, const char *what)
        : std::runtime_error(std::string(what) + ": " + quids_gpu_status_string(s)), status(s) {}
};
inline void check(int status, const char *what) {
    if (status != QUIDS_OK) throw error(status, what);
}

// ---------------------------------------------------------------- context
// One CUDA stream and the scratch memory of the steps.  The reference has
// none (its state is host memory); default_context() serves every it_t
// constructed without one.
class context {
public:
    explicit context(int dev = device) { check(quids_gpu_ctx_create(dev, &h_), "quids_gpu_ctx_create"); }
    ~context() {
        if (h_) quids_gpu_ctx_destroy(h_);
    }
    context(const context &) = delete;
    context &operator=(const context &) = delete;
    quids_gpu_ctx *handle() const { return h_; }

private:
    quids_gpu_ctx *h_ = nullptr;
};
inline context &default_context() {
    static context c(device);
    return c;
}

class iteration;
class symbolic_iteration;
typedef iteration it_t;
typedef symbolic_iteration sy_it_t;

// ------------------------------------------------------ symbolic iteration
// The counters of the last step (src/quids.hpp:336-347); the children
// themselves stay in the context's scratch.
class symbolic_iteration {
public:
    size_t num_object = 0;                      // children of the step
    size_t num_object_after_interferences = 0;  // distinct children of norm above tolerance
    quids_gpu_step_stats stats{};               // this library's counters of the step
};

// -------------------------------------------------------------- iteration
class iteration {
public:
    size_t num_object = 0;  // objects of the wave function
    double total_proba = 1;  // probability kept by the previous truncation

    explicit iteration(context &c = default_context()) : ctx_(&c) {
        check(quids_gpu_state_create(ctx_->handle(), &h_), "quids_gpu_state_create");
        begin_.assign(1, 0);
        host_valid_ = true;
    }
    // one object of magnitude 1 (src/quids.hpp:163-165)
    iteration(char const *object_begin, char const *object_end) : iteration() { append(object_begin, object_end); }
    ~iteration() {
        if (h_) quids_gpu_state_destroy(h_);
    }
    iteration(const iteration &) = delete;
    iteration &operator=(const iteration &) = delete;
    iteration(iteration &&o) noexcept { swap(o); }
    iteration &operator=(iteration &&o) noexcept {
        swap(o);
        return *this;
    }
    void swap(iteration &o) noexcept {
        std::swap(num_object, o.num_object);
        std::swap(total_proba, o.total_proba);
        std::swap(ctx_, o.ctx_);
        std::swap(h_, o.h_);
        objects_.swap(o.objects_);
        begin_.swap(o.begin_);
        size_.swap(o.size_);
        mag_.swap(o.mag_);
        std::swap(host_valid_, o.host_valid_);
        std::swap(host_dirty_, o.host_dirty_);
    }

    // src/quids.hpp:174-188: the object, padded to align_byte_length
    void append(char const *object_begin, char const *object_end, mag_t mag = mag_t{1, 0}) {
        pull();
        const size_t sz = (size_t)(object_end - object_begin);
        const size_t off = begin_[num_object];
        const size_t pad = align_byte_length <= 1 || sz % align_byte_length == 0
                               ? 0
                               : align_byte_length - sz % align_byte_length;
        objects_.resize(off + sz + pad, 0);
        for (size_t i = 0; i < sz; ++i) objects_[off + i] = (uint8_t)object_begin[i];
        size_.push_back((uint32_t)sz);
        mag_.push_back(mag);
        begin_.push_back(off + sz + pad);
        ++num_object;
        host_dirty_ = true;
    }
    // src/quids.hpp:194-203: drop the last n objects, then normalize
    void pop(size_t n = 1, bool normalize_ = true) {
        if (n < 1) return;
        pull();
        num_object -= n;
        objects_.resize(begin_[num_object]);
        begin_.resize(num_object + 1);
        size_.resize(num_object);
        mag_.resize(num_object);
        host_dirty_ = true;
        if (normalize_) normalize();
    }
    // src/quids.hpp:985-1017: total_proba = sum of norms; magnitudes divided by its root
    void normalize() {
        pull();
        total_proba = 0;
        for (size_t i = 0; i < num_object; ++i) total_proba += qd::norm(mag_[i]);
        const double f = std::sqrt(total_proba);
        if (num_object && f != 1)
            for (size_t i = 0; i < num_object; ++i) mag_[i] = mag_[i] / f;
        host_dirty_ = true;
    }
    // src/quids.hpp:242-258 (read-write: the object goes back to the device
    // before the next step)
    void get_object(size_t object_id, char *&object_begin, uint &object_size, mag_t *&mag) {
        pull();
        host_dirty_ = true;
        object_size = size_[object_id];
        mag = &mag_[object_id];
        object_begin = (char *)objects_.data() + begin_[object_id];
    }
    void get_object(size_t object_id, char const *&object_begin, uint &object_size, mag_t &mag) const {
        pull();
        object_size = size_[object_id];
        mag = mag_[object_id];
        object_begin = (char const *)objects_.data() + begin_[object_id];
    }
    // src/quids.hpp:208-234, on the host over the state read back
    double average_value(const observable_t &observable) const {
        pull();
        double avg = 0;
        for (size_t i = 0; i < num_object; ++i) {
            char const *b = (char const *)objects_.data() + begin_[i];
            avg += observable(b, b + size_[i]) * qd::norm(mag_[i]);
        }
        return avg;
    }
    // the same on the GPU for an observable that is a __host__ __device__
    // functor double(char const *begin, char const *end), reduced in a fixed order
    template <class Obs>
    double device_average_value(const Obs &observable) {
        push();
        double v = 0;
        check(qd::engine::average_value(ctx_->handle(), h_, observable, &v), "average_value");
        return v;
    }

    quids_gpu_state *handle() { return h_; }
    context &ctx() { return *ctx_; }

    // host copy -> device (before a step reads the state)
    void push() {
        if (!host_dirty_) return;
        std::vector<double> m(2 * num_object);
        for (size_t i = 0; i < num_object; ++i) {
            m[2 * i] = mag_[i].re;
            m[2 * i + 1] = mag_[i].im;
        }
        check(quids_gpu_state_upload(h_, num_object, objects_.data(), begin_.data(), size_.data(), m.data(),
                                     begin_[num_object]),
              "quids_gpu_state_upload");
        host_dirty_ = false;
    }
    // the device state changed (a step wrote it)
    void device_changed(size_t n, double total) {
        num_object = n;
        total_proba = total;
        host_valid_ = false;
        host_dirty_ = false;
    }

private:
    // device -> host copy, once after each change on the device
    void pull() const {
        if (host_valid_) return;
        uint64_t nb = 0;
        check(quids_gpu_state_num_bytes(h_, &nb), "quids_gpu_state_num_bytes");
        objects_.resize(nb);
        begin_.resize(num_object + 1);
        size_.resize(num_object);
        std::vector<double> m(2 * num_object);
        check(quids_gpu_state_download(h_, objects_.data(), begin_.data(), size_.data(), m.data()),
              "quids_gpu_state_download");
        mag_.resize(num_object);
        for (size_t i = 0; i < num_object; ++i) mag_[i] = mag_t{m[2 * i], m[2 * i + 1]};
        host_valid_ = true;
    }

    context *ctx_ = nullptr;
    quids_gpu_state *h_ = nullptr;
    mutable std::vector<uint8_t> objects_;
    mutable std::vector<uint64_t> begin_;
    mutable std::vector<uint32_t> size_;
    mutable std::vector<mag_t> mag_;
    mutable bool host_valid_ = false;
    bool host_dirty_ = false;
};

inline quids_gpu_params step_params(size_t max_num_object) {
    quids_gpu_params p{};
    p.tolerance = tolerance;
    p.max_num_object = (uint64_t)max_num_object;
    p.simple_truncation = simple_truncation ? 1 : 0;
    p.align_byte_length = align_byte_length;
    p.table_load_factor = table_load_factor;
    p.seed = truncation_seed;
    return p;
}

// ------------------------------------------------------------- simulate
// src/quids.hpp:448-543.  max_num_object: 0 keeps as many objects as fit the
// device memory, size_t(-1) keeps all.  The step runs on the GPU as one
// unit; mid_step_function is called with "end" once it is done.
template <class Rule>
void simulate(it_t &iteration, Rule const *rule, it_t &next_iteration, sy_it_t &symbolic_iteration,
              size_t max_num_object = 0, debug_t mid_step_function = [](const char *) {}) {
    if (!rule) throw error(QUIDS_ERR_BAD_ARG, "simulate: null rule");
    if (&iteration == &next_iteration) throw error(QUIDS_ERR_BAD_ARG, "simulate: next_iteration is iteration");
    if (&iteration.ctx() != &next_iteration.ctx()) throw error(QUIDS_ERR_BAD_ARG, "simulate: two contexts");
    iteration.push();
    const quids_gpu_params prm = step_params(max_num_object);
    quids_gpu_step_stats st{};
    check(qd::ranges::simulate_step(iteration.ctx().handle(), iteration.handle(), *rule, next_iteration.handle(),
                                    prm, &st),
          "simulate");
    double total = 0;
    check(quids_gpu_state_total_proba(next_iteration.handle(), &total), "quids_gpu_state_total_proba");
    next_iteration.device_changed(st.num_object_out, total);
    symbolic_iteration.num_object = st.num_object;
    symbolic_iteration.num_object_after_interferences = st.num_object_after_interferences;
    symbolic_iteration.stats = st;
    if (mid_step_function) mid_step_function("end");
}
template <class Rule>
void simulate(it_t &iteration, Rule const &rule, it_t &next_iteration, sy_it_t &symbolic_iteration,
              size_t max_num_object = 0, debug_t mid_step_function = [](const char *) {}) {
    simulate(iteration, &rule, next_iteration, symbolic_iteration, max_num_object, mid_step_function);
}

// src/quids.hpp:436-438: the modifier on every object, in place
template <class Modifier>
void simulate(it_t &iteration, Modifier const &modifier) {
    iteration.push();
    check(qd::engine::apply_modifier(iteration.ctx().handle(), iteration.handle(), modifier), "simulate(modifier)");
    check(quids_gpu_ctx_synchronize(iteration.ctx().handle()), "simulate(modifier)");
    iteration.device_changed(iteration.num_object, iteration.total_proba);
}

// ------------------------------------------------------------ built-in rules
namespace rules {
namespace quantum_computer {
// src/rules/quantum_computer.hpp:31-50
struct hadamard : qd::rules::hadamard {
    explicit hadamard(size_t bit_) : qd::rules::hadamard(make(bit_)) {}

private:
    static qd::rules::hadamard make(size_t bit) {
        const quids_gpu_rule_params p{(uint64_t)bit, 0, 0, 0, 0};
        return qd::host::make_hadamard(&p);  // 1 / std::sqrt(2) on the host, as the reference
    }
};
// :25-29, :52-75 (Z negates and flips, as the reference)
inline qd::rules::cnot cnot(uint32_t control_bit, uint32_t bit) { return qd::rules::cnot{control_bit, bit}; }
inline qd::rules::xgate Xgate(size_t bit) { return qd::rules::xgate{bit}; }
inline qd::rules::ygate Ygate(size_t bit) { return qd::rules::ygate{bit}; }
inline qd::rules::zgate Zgate(size_t bit) { return qd::rules::zgate{bit}; }
}  // namespace quantum_computer

namespace qcgd {
inline qd::qcgd::factors angles(double theta, double phi, double xi) {
    const quids_gpu_rule_params p{0, 0, theta, phi, xi};
    return qd::host::make_factors(&p);
}
// src/rules/qcgd.hpp:459-532, :534-605, :607-1036
struct erase_create : qd::qcgd::erase_create {
    explicit erase_create(double theta, double phi = 0, double xi = 0) : qd::qcgd::erase_create{angles(theta, phi, xi)} {}
};
struct coin : qd::qcgd::coin {
    explicit coin(double theta, double phi = 0, double xi = 0) : qd::qcgd::coin{angles(theta, phi, xi)} {}
};
struct split_merge : qd::qcgd::split_merge {
    explicit split_merge(double theta, double phi = 0, double xi = 0) : qd::qcgd::split_merge{angles(theta, phi, xi)} {}
};
// :443-457 (modifiers)
inline constexpr qd::qcgd::step step{};
inline constexpr qd::qcgd::reversed_step reversed_step{};
}  // namespace qcgd
}  // namespace rules

}  // namespace quids::gpu
