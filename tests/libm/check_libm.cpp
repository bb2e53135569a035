// check_libm.cpp — physecs_gb300/csrc/libm_f32.cuh against the host's C library (test
// infrastructure).  Every float in [-1, 1] for acosf, and seeded arguments (random bit
// patterns, quotients near the reduction breakpoints, special values) for atanf and
// atan2f.  Prints the mismatch counts and a few examples.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "libm_f32.cuh"

static float fb(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static uint32_t bf(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static bool same(float a, float b) { return bf(a) == bf(b) || (std::isnan(a) && std::isnan(b)); }

int main(int argc, char** argv) {
    long n_atan2 = argc > 1 ? std::atol(argv[1]) : 20000000;
    long bad[3] = {0, 0, 0}, n[3] = {0, 0, 0};
    // acosf: every float of [0, 1] and [-1, 0]
    for (uint32_t u = 0; u <= 0x3f800000u; u += 1) {
        for (int s = 0; s < 2; ++s) {
            const float x = fb(u | (s ? 0x80000000u : 0u));
            const float a = psx::libm::acosf(x), b = ::acosf(x);
            ++n[0];
            if (!same(a, b)) { if (bad[0]++ < 5) std::printf("acosf %a: %a vs libc %a\n", x, a, b); }
        }
    }
    uint64_t st = 0x9E3779B97F4A7C15ull;
    auto next = [&]() { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; };
    for (long i = 0; i < n_atan2; ++i) {
        const uint64_t r = next();
        const float x = fb((uint32_t)r);
        const float a = psx::libm::atanf(x), b = ::atanf(x);
        ++n[1];
        if (!same(a, b)) { if (bad[1]++ < 5) std::printf("atanf %a: %a vs libc %a\n", x, a, b); }
        float y = fb((uint32_t)(r >> 32)), z = fb((uint32_t)next());
        if (i & 1) {   // moderate magnitudes, where joint angles live
            y = std::ldexp((float)(r >> 40) / 16777216.0f - 0.5f, (int)(r % 7) - 3);
            z = std::ldexp((float)((r >> 16) & 0xffffff) / 16777216.0f - 0.5f, (int)((r >> 8) % 7) - 3);
        }
        const float c = psx::libm::atan2f(y, z), d = ::atan2f(y, z);
        ++n[2];
        if (!same(c, d)) { if (bad[2]++ < 5) std::printf("atan2f %a %a: %a vs libc %a\n", y, z, c, d); }
    }
    const float sp[] = {0.0f, -0.0f, 1.0f, -1.0f, INFINITY, -INFINITY, NAN, 1e-40f, -1e-40f, 0.4375f, 0.6875f, 1.1875f, 2.4375f};
    for (float y : sp)
        for (float z : sp) {
            ++n[2];
            if (!same(psx::libm::atan2f(y, z), ::atan2f(y, z))) {
                if (bad[2]++ < 10) std::printf("atan2f %a %a: %a vs libc %a\n", y, z, psx::libm::atan2f(y, z), ::atan2f(y, z));
            }
        }
    std::printf("acosf %ld/%ld atanf %ld/%ld atan2f %ld/%ld\n", bad[0], n[0], bad[1], n[1], bad[2], n[2]);
    return (bad[0] || bad[1] || bad[2]) ? 1 : 0;
}
