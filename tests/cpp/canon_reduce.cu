// Host-side check of canon() (device.cuh): x mod q in [0, q) for int32 x,
// against the % operator, at the extremes of the int32 range and on a
// pseudo-random sample, for the moduli the library's designs use.
#include <cstdint>
#include <cstdio>

#include "../../ntts_on_amd_ai_engines_aie1_gb300/csrc/device.cuh"

int main() {
    const int64_t qs[] = {3, 5, 17, 97, 257, 7681, 10753, 12289, 18433, 19457, 65537,
                          998244353, 469762049, 167772161, 754974721, 1073707009, 1431580673};
    uint64_t state = 0x9E3779B97F4A7C15ull, checked = 0, bad = 0;
    for (int64_t q : qs) {
        const int c = (int)((((uint64_t)1 << 32) + (uint64_t)q / 2) / (uint64_t)q);
        auto check = [&](int32_t x) {
            int64_t want = (int64_t)x % q;
            if (want < 0) want += q;
            ++checked;
            if (gbntt::canon(x, (int)q, c) != want) {
                if (bad < 10) std::printf("q %lld x %d: %d, want %lld\n", (long long)q, x, gbntt::canon(x, (int)q, c),
                                          (long long)want);
                ++bad;
            }
        };
        const int32_t edge[] = {INT32_MIN, INT32_MAX, 0, -1, 1, (int32_t)q, (int32_t)-q, (int32_t)(q - 1),
                                (int32_t)(1 - q), INT32_MIN + 1, INT32_MAX - 1};
        for (int32_t x : edge) check(x);
        for (int i = 0; i < 1000000; ++i) {
            state = state * 6364136223846793005ull + 1442695040888963407ull;
            check((int32_t)(state >> 32));
        }
    }
    std::printf("%llu values checked, %llu failures\n", (unsigned long long)checked, (unsigned long long)bad);
    return bad ? 1 : 0;
}
