// A program written against the public C++ header the way a user of the
// reference writes one against src/quids.hpp: rules and a modifier defined
// here, outside the library, stepped through quids::gpu::simulate.  Built
// and run by tests/test_gpu_cpp_api.py, which checks the results against the
// CPU oracle.
//
//   user_rules <in.state> <out_dir> <bit>
//
// reads a packed state (see read_state), and writes into out_dir:
//   user_hadamard.state  the state after the Hadamard rule defined below on `bit`
//   builtin_hadamard.state  the same step with the library's built-in rule
//   user_x.state         the input after the X modifier defined below, then the user Hadamard
//   counts.txt           per step: num_object, num_object_after_interferences, total_proba
//   errors.txt           the status of the rule that breaks its size bound, then of
//                        a normal step on the same context
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "quids_gpu.hpp"

using quids::gpu::mag_t;
using quids::gpu::uint;

// The reference's Hadamard rule (src/rules/quantum_computer.hpp:31-50),
// written as a user would port it: populate_child only, the default hasher.
struct user_hadamard {
    size_t bit;
    __host__ __device__ void get_num_child(char const *parent_begin, char const *parent_end, uint &num_child,
                                           uint &max_child_size) const {
        num_child = 2;
        max_child_size = (uint)(parent_end - parent_begin);
    }
    __host__ __device__ void populate_child(char const *parent_begin, char const *parent_end, char *const child_begin,
                                            uint const child_id, uint &size, mag_t &mag) const {
        mag *= (parent_begin[bit] && child_id) ? -1 / sqrt(2.0) : 1 / sqrt(2.0);
        size = (uint)(parent_end - parent_begin);
        for (uint i = 0; i < size; ++i) child_begin[i] = parent_begin[i];
        child_begin[bit] ^= !child_id;
    }
};

// A rule that breaks its contract: it declares children of the parent's
// size but reports 8 bytes more (it writes only the declared bytes).
struct oversized_rule {
    __host__ __device__ void get_num_child(char const *pb, char const *pe, uint &num_child,
                                           uint &max_child_size) const {
        num_child = 1;
        max_child_size = (uint)(pe - pb);
    }
    __host__ __device__ void populate_child(char const *pb, char const *pe, char *const cb, uint const, uint &size,
                                            mag_t &) const {
        for (const char *p = pb; p != pe; ++p) cb[p - pb] = *p;
        size = (uint)(pe - pb) + 8;
    }
};

// The reference's X gate (src/rules/quantum_computer.hpp:52-56) as a modifier
struct user_xgate {
    size_t bit;
    __host__ __device__ void operator()(char *begin, char *, mag_t &) const { begin[bit] = !begin[bit]; }
};

static bool read_state(const char *path, quids::gpu::it_t &it) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    uint64_t n = 0, nb = 0;
    bool ok = std::fread(&n, 8, 1, f) == 1 && std::fread(&nb, 8, 1, f) == 1;
    std::vector<char> objects(nb);
    std::vector<uint64_t> begin(n + 1);
    std::vector<uint32_t> size(n);
    std::vector<double> mag(2 * n);
    ok = ok && std::fread(objects.data(), 1, nb, f) == nb && std::fread(begin.data(), 8, n + 1, f) == n + 1 &&
         std::fread(size.data(), 4, n, f) == n && std::fread(mag.data(), 8, 2 * n, f) == 2 * n;
    std::fclose(f);
    for (uint64_t i = 0; ok && i < n; ++i)
        it.append(objects.data() + begin[i], objects.data() + begin[i] + size[i], mag_t{mag[2 * i], mag[2 * i + 1]});
    return ok;
}

// the same layout, read back object by object through get_object
static bool write_state(const std::string &path, const quids::gpu::it_t &it) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    std::vector<char> objects;
    std::vector<uint64_t> begin{0};
    std::vector<uint32_t> size;
    std::vector<double> mag;
    for (size_t i = 0; i < it.num_object; ++i) {
        char const *b;
        uint sz;
        mag_t m;
        it.get_object(i, b, sz, m);
        objects.insert(objects.end(), b, b + sz);
        begin.push_back(objects.size());
        size.push_back(sz);
        mag.push_back(m.re);
        mag.push_back(m.im);
    }
    const uint64_t n = it.num_object, nb = objects.size();
    bool ok = std::fwrite(&n, 8, 1, f) == 1 && std::fwrite(&nb, 8, 1, f) == 1 &&
              std::fwrite(objects.data(), 1, nb, f) == nb && std::fwrite(begin.data(), 8, n + 1, f) == n + 1 &&
              std::fwrite(size.data(), 4, n, f) == n && std::fwrite(mag.data(), 8, 2 * n, f) == 2 * n;
    std::fclose(f);
    return ok;
}

int main(int argc, char **argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s <in.state> <out_dir> <bit>\n", argv[0]);
        return 2;
    }
    const std::string out = argv[2];
    const size_t bit = std::strtoull(argv[3], nullptr, 10);
    quids::gpu::tolerance = 1e-18;
    quids::gpu::simple_truncation = true;
    FILE *counts = std::fopen((out + "/counts.txt").c_str(), "w");
    FILE *errors = std::fopen((out + "/errors.txt").c_str(), "w");
    if (!counts || !errors) return 3;
    try {
        quids::gpu::it_t state, next;
        quids::gpu::sy_it_t sy;
        if (!read_state(argv[1], state)) return 4;

        // the user rule, through a pointer as the reference's examples pass it
        const user_hadamard *h = new user_hadamard{bit};
        quids::gpu::simulate(state, h, next, sy, size_t(-1));
        std::fprintf(counts, "%zu %zu %.17g\n", sy.num_object, sy.num_object_after_interferences, next.total_proba);
        if (!write_state(out + "/user_hadamard.state", next)) return 5;
        delete h;

        // the library's built-in rule on the same input
        quids::gpu::it_t next2;
        quids::gpu::simulate(state, quids::gpu::rules::quantum_computer::hadamard(bit), next2, sy, size_t(-1));
        std::fprintf(counts, "%zu %zu %.17g\n", sy.num_object, sy.num_object_after_interferences, next2.total_proba);
        if (!write_state(out + "/builtin_hadamard.state", next2)) return 5;

        // the user modifier in place, then the user rule
        quids::gpu::simulate(state, user_xgate{bit});
        quids::gpu::it_t next3;
        quids::gpu::simulate(state, user_hadamard{bit}, next3, sy, size_t(-1));
        std::fprintf(counts, "%zu %zu %.17g\n", sy.num_object, sy.num_object_after_interferences, next3.total_proba);
        if (!write_state(out + "/user_x.state", next3)) return 5;

        // a rule that reports children larger than it declared: an error
        // status, and the context steps on normally afterwards
        int status = 0;
        try {
            quids::gpu::it_t bad;
            quids::gpu::simulate(next3, oversized_rule{}, bad, sy, size_t(-1));
        } catch (const quids::gpu::error &e) {
            status = e.status;
        }
        std::fprintf(errors, "%d\n", status);
        quids::gpu::it_t again;
        quids::gpu::simulate(next3, user_hadamard{bit}, again, sy, size_t(-1));
        std::fprintf(errors, "%zu\n", again.num_object);
    } catch (const quids::gpu::error &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 6;
    }
    std::fclose(counts);
    std::fclose(errors);
    return 0;
}
