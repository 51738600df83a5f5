// Host check of quids_gb300/csrc/softfp64.cuh: the integer multiply and add
// against the host's IEEE-754 binary64 arithmetic (round to nearest even, no
// contraction), bit for bit, on operand families chosen to hit every path:
// random significands over a wide and a narrow exponent range, operands with
// few significant bits (exact products and sums, so exact ties), sums that
// cancel, every exponent gap from 0 to 70, and results at the edges of the
// normal range (handed to the hardware path).
//   softfp_check <trials per family> <seed>   -> prints "<checked> <mismatches>"
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../quids_gb300/csrc/softfp64.cuh"

namespace sf = qd::softfp;

static uint64_t s_state;
static uint64_t next() {  // splitmix64
    uint64_t z = (s_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double make(uint64_t sign, int64_t e, uint64_t mant) {
    return sf::from_bits((sign << 63) | ((uint64_t)e << 52) | (mant & sf::kMant));
}
static double wide() {  // any finite value, subnormals and zeros included
    uint64_t b;
    do b = next(); while (((b >> 52) & 0x7ff) == 0x7ff);
    return sf::from_bits(b);
}
static double narrow(int lo, int hi) { return make(next() & 1, 1023 + lo + (int64_t)(next() % (uint64_t)(hi - lo + 1)), next()); }
static double few_bits(int lo, int hi) {  // k significant bits, k in 1..30
    const int k = 1 + (int)(next() % 30);
    const uint64_t m = (next() | 1) & ((1ull << k) - 1);
    const int sh = 52 - (63 - __builtin_clzll(m));
    return make(next() & 1, 1023 + lo + (int64_t)(next() % (uint64_t)(hi - lo + 1)), m << sh);
}

static uint64_t checked = 0, bad = 0;
static void check(double x, double y) {
    volatile double vx = x, vy = y;
    const double pm = vx * vy, ps = vx + vy, pd = vx - vy;
    const double m = sf::mul(x, y), s = sf::add(x, y), d = sf::sub(x, y);
    checked += 3;
    if (sf::to_bits(m) != sf::to_bits(pm)) {
        if (bad < 5) std::fprintf(stderr, "mul %a * %a: %a != %a\n", x, y, m, pm);
        ++bad;
    }
    if (sf::to_bits(s) != sf::to_bits(ps)) {
        if (bad < 5) std::fprintf(stderr, "add %a + %a: %a != %a\n", x, y, s, ps);
        ++bad;
    }
    if (sf::to_bits(d) != sf::to_bits(pd)) {
        if (bad < 5) std::fprintf(stderr, "sub %a - %a: %a != %a\n", x, y, d, pd);
        ++bad;
    }
}

int main(int argc, char **argv) {
    const uint64_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 1000000;
    s_state = argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1;
    for (uint64_t i = 0; i < n; ++i) {
        check(wide(), wide());
        check(narrow(-40, 5), narrow(-40, 5));                  // magnitudes of the rule steps
        check(few_bits(-20, 20), few_bits(-20, 20));            // exact products / sums, ties
        const double x = narrow(-30, 30);                      // cancellation: y close to -x
        const uint64_t xb = sf::to_bits(x);
        check(x, sf::from_bits((xb ^ sf::kSign) + (next() % 9) - 4));
        const int gap = (int)(next() % 71);                    // every exponent gap
        const double a = few_bits(-10, 10), b = make(next() & 1, (int64_t)((sf::to_bits(a) >> 52) & 0x7ff) - gap,
                                                      next());
        if (((sf::to_bits(a) >> 52) & 0x7ff) > (uint64_t)gap) check(a, b);
        check(narrow(1000, 1023), narrow(0, 23));              // near overflow
        check(narrow(-1022, -1000), narrow(-23, 0));           // near underflow
    }
    std::printf("%llu %llu\n", (unsigned long long)checked, (unsigned long long)bad);
    return bad != 0;
}
