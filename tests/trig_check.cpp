/*
 * trig_check.cpp — b2g_sincosf (float fast path with fallback) against b2g_sincosf_ref (the
 * double evaluation that defines the results) on every float x with |x| <= 8192, or on every
 * stride-th one. Prints the number of inputs checked, of bit mismatches and of fallbacks taken,
 * and exits non-zero on any mismatch.
 *
 * Usage: trig_check [stride] [threads]
 */
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "b2g_trig.h"

static uint32_t f2u(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
static float u2f(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

int main(int argc, char** argv) {
    const uint32_t stride = argc > 1 ? (uint32_t)std::strtoul(argv[1], nullptr, 10) : 1u;
    const int nthreads = argc > 2 ? std::atoi(argv[2]) : (int)std::thread::hardware_concurrency();
    const uint32_t top = f2u(8192.0f);  /* positive floats 0 < x <= 8192; negatives by symmetry of the loop */
    std::atomic<unsigned long long> checked{0}, mismatches{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t) {
        pool.emplace_back([&, t]() {
            unsigned long long n = 0, bad = 0;
            for (uint32_t u = 1u + (uint32_t)t * stride; u <= top; u += (uint32_t)nthreads * stride) {
                for (int sign = 0; sign < 2; ++sign) {
                    const float x = sign ? -u2f(u) : u2f(u);
                    float s1, c1, s2, c2;
                    b2g_sincosf(x, &s1, &c1);
                    b2g_sincosf_ref(x, &s2, &c2);
                    if (f2u(s1) != f2u(s2) || f2u(c1) != f2u(c2)) {
                        if (bad < 5) std::printf("mismatch x=%a sin %a vs %a cos %a vs %a\n", x, s1, s2, c1, c2);
                        ++bad;
                    }
                    ++n;
                }
            }
            checked += n;
            mismatches += bad;
        });
    }
    for (auto& th : pool) th.join();
    std::printf("checked %llu mismatches %llu\n", (unsigned long long)checked, (unsigned long long)mismatches);
    return mismatches ? 1 : 0;
}
