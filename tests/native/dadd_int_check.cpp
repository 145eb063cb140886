// Checks the integer-pipe binary64 addition against the host's FP64 adder
// (IEEE-754 round to nearest even) on seeded inputs.  Usage:
//   dadd_int_check N SEED   -> prints "cases fast mismatches", exit 1 on a mismatch
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../masterthesis_gb300/csrc/dadd_int.cuh"

static uint64_t rng_state;
static uint64_t next() {  // xorshift64*
    rng_state ^= rng_state >> 12;
    rng_state ^= rng_state << 25;
    rng_state ^= rng_state >> 27;
    return rng_state * 0x2545F4914F6CDD1Dull;
}

static uint64_t with_exp(uint64_t sign, uint64_t e, uint64_t frac) {
    return (sign << 63) | ((e & 0x7ff) << 52) | (frac & 0x000fffffffffffffull);
}

// A significand whose low bits are all zeros or all ones (ties, carries).
static uint64_t shaped_frac() {
    uint64_t f = next();
    const int k = (int)(next() % 53);
    const uint64_t mask = k ? ((1ull << k) - 1) : 0;
    switch (next() % 4) {
        case 0: return f & ~mask;
        case 1: return f | mask;
        case 2: return mask;
        default: return f;
    }
}

static void make(int mode, uint64_t& a, uint64_t& b) {
    const uint64_t s = next() & 1;
    switch (mode) {
        case 0:  // any bit patterns
            a = next();
            b = next();
            break;
        case 1: {  // one sign, small exponent differences
            const uint64_t ea = 1 + next() % 2046;
            const uint64_t d = (next() % 4) ? next() % 12 : next() % 72;
            const uint64_t eb = ea > d ? ea - d : 1 + next() % 3;
            a = with_exp(s, ea, next());
            b = with_exp(s, eb, next());
            break;
        }
        case 2: {  // shaped significands: exact ties, carries into the exponent
            const uint64_t ea = 1 + next() % 2046;
            const uint64_t d = (next() % 4) ? next() % 12 : next() % 60;
            const uint64_t eb = ea > d ? ea - d : 1;
            a = with_exp(s, ea, shaped_frac());
            b = with_exp(s, eb, shaped_frac());
            break;
        }
        case 3: {  // near the overflow threshold and near the subnormals
            const uint64_t ea = (next() & 1) ? 2040 + next() % 8 : next() % 8;
            const uint64_t eb = ea - (ea ? next() % (ea < 60 ? ea + 1 : 60) : 0);
            a = with_exp(s, ea, shaped_frac());
            b = with_exp(s ^ ((next() % 8) == 0), eb, shaped_frac());
            break;
        }
        default: {  // neighbouring values of a smooth field
            a = with_exp(s, 1000 + next() % 48, next());
            b = a + (uint64_t)((int64_t)(next() % 4097) - 2048) * (next() % 2 ? 1 : (1ull << 30));
            if (next() % 16 == 0) b ^= 1ull << 63;
            break;
        }
    }
    if (next() % 2) { const uint64_t t = a; a = b; b = t; }
}

int main(int argc, char** argv) {
    const long long n = argc > 1 ? atoll(argv[1]) : 1000000;
    rng_state = argc > 2 ? strtoull(argv[2], nullptr, 10) * 0x9E3779B97F4A7C15ull + 1 : 1;
    long long fast = 0, bad = 0;
    for (long long i = 0; i < n; ++i) {
        uint64_t a, b;
        make((int)(i % 5), a, b);
        bool ok;
        const uint64_t r = scafes::dadd_same_sign_bits(a, b, ok);
        // The documented range: one sign, exponents at most 10 apart, the
        // smaller one in [1, 2035].
        const uint64_t ea = (a >> 52) & 0x7ff, eb = (b >> 52) & 0x7ff;
        const uint64_t lo = ea < eb ? ea : eb, hi = ea < eb ? eb : ea;
        const bool in_range = (a >> 63) == (b >> 63) && lo >= 1 && lo <= 2035 && hi - lo <= 10;
        if (ok != in_range) {
            if (bad < 8)
                printf("range a=%016llx b=%016llx ok=%d\n", (unsigned long long)a, (unsigned long long)b, (int)ok);
            ++bad;
            continue;
        }
        if (!ok) continue;
        ++fast;
        double x, y;
        memcpy(&x, &a, 8);
        memcpy(&y, &b, 8);
        volatile double z = x + y;
        uint64_t want;
        double zz = z;
        memcpy(&want, &zz, 8);
        if (want != r) {
            if (bad < 8)
                printf("mismatch a=%016llx b=%016llx got=%016llx want=%016llx\n", (unsigned long long)a,
                       (unsigned long long)b, (unsigned long long)r, (unsigned long long)want);
            ++bad;
        }
    }
    printf("%lld %lld %lld\n", n, fast, bad);
    return bad ? 1 : 0;
}
