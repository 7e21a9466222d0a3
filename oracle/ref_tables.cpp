/*
 * ref_tables.cpp -- runs the reference's own table generators on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile (target `ref`) into
 * oracle/_ref/ref_tables, and only where the reference sources are present.
 * It includes the reference's src/twiddle.h and src/auxiliary.h unmodified
 * (from the reference checkout, through -I), with oracle/ref_stub/adf.h
 * standing in for AMD's <adf.h>, and prints every table the graph
 * constructors build for a fixed list of configurations:
 *
 *   <family> <n> <q> <root> <which> <layer> <len>: v0 v1 ...
 *
 * which: 0 = per-layer combined / twiddle table, 1 = per-layer Barrett
 * multipliers, 2 = radix-8 F8 matrix, 3/4 = radix-8 reduction twiddles /
 * multipliers, 5 = compile-time constants (n^-1, log2 root order, omega_4).
 * tests/golden/make_golden.py turns this into tests/golden/ref_tables.json.
 */
#include <adf.h>
#include "twiddle.h"

#include <cstdio>
#include <vector>

template <typename T>
static void emit(const char* fam, unsigned n, long long q, long long root, int which, int layer,
                 const std::vector<T>& v) {
    std::printf("%s %u %lld %lld %d %d %zu:", fam, n, q, root, which, layer, v.size());
    for (const T& x : v) std::printf(" %lld", (long long)x);
    std::printf("\n");
}

/* src/ntt.h:80 (forward int16) */
template <unsigned N, int16 Q, int16 ROOT>
static void r2f16() {
    constexpr uint16 L = DETERMINE_LOG_ROOT_SIZE<Q, ROOT>::value;
    std::vector<std::vector<int16>> f(L);
    determine_factors<int16, N, Q, ROOT, 16, NTT_KERNEL_TYPE::CT_NO_to_BO, false, L, L>(f);
    for (unsigned i = 0; i < L; i++) emit("r2f16", N, Q, ROOT, 0, i, f[i]);
    std::vector<long long> c = {ExtendedGCD<N, Q>::value, L};
    emit("r2f16", N, Q, ROOT, 5, 0, c);
}

/* src/ntt.h:75-76 (inverse int16) */
template <unsigned N, int16 Q, int16 ROOT>
static void r2i16() {
    constexpr uint16 L = DETERMINE_LOG_ROOT_SIZE<Q, ROOT>::value;
    std::vector<std::vector<int16>> tw(L), wq(L);
    determine_twiddle_and_barrett<int16, N, Q, ROOT, 16, NTT_KERNEL_TYPE::CT_NO_to_BO, true, L, L>(tw, wq);
    for (unsigned i = 0; i < L; i++) {
        emit("r2i16", N, Q, ROOT, 0, i, tw[i]);
        emit("r2i16", N, Q, ROOT, 1, i, wq[i]);
    }
}

/* src/ntt_int32.h:61 (forward CT and inverse GS) */
template <unsigned N, int32 Q, int32 ROOT>
static void r2i32() {
    constexpr uint16 L = DETERMINE_LOG_ROOT_SIZE<Q, ROOT>::value;
    std::vector<std::vector<int32>> f(L), g(L);
    determine_factors<int32, N, Q, ROOT, 32, NTT_KERNEL_TYPE::CT_NO_to_BO, false, L, L>(f);
    determine_factors<int32, N, Q, ROOT, 32, NTT_KERNEL_TYPE::GS_BO_to_NO, true, L, L>(g);
    for (unsigned i = 0; i < L; i++) emit("r2f32", N, Q, ROOT, 0, i, f[i]);
    for (unsigned i = 0; i < L; i++) emit("r2g32", N, Q, ROOT, 0, i, g[i]);
    std::vector<long long> c = {ExtendedGCD<N, Q>::value, L};
    emit("r2f32", N, Q, ROOT, 5, 0, c);
}

/* src/ntt_r4.h:69 */
template <unsigned N, int16 Q, int16 ROOT>
static void r4f16() {
    constexpr uint16 L = DETERMINE_LOG_ROOT_SIZE<Q, ROOT>::value;
    constexpr int ROOT_SIZE = DETERMINE_ROOT_SIZE<Q, ROOT>::value;
    std::vector<std::vector<int16>> f(L / 2);
    determine_factors_radix4<int16, N, Q, ROOT, ROOT_SIZE, 16, NTT_KERNEL_TYPE::CT_NO_to_BO, false, L / 2>(f);
    for (unsigned i = 0; i < L / 2; i++) emit("r4f16", N, Q, ROOT, 0, i, f[i]);
    std::vector<long long> c = {Power<ROOT, ROOT_SIZE / 4, Q>::value};
    emit("r4f16", N, Q, ROOT, 5, 0, c);
}

/* src/ntt_r8.h:41 */
template <unsigned N, uint16 Q, uint16 ROOT>
static void r8f16() {
    std::vector<std::vector<int16>> a(1), b(1);
    std::vector<std::vector<int32>> c(1);
    determine_factors_r8<Q, ROOT, N>(a, b, c);
    emit("r8f16", N, Q, ROOT, 2, 0, a[0]);
    emit("r8f16", N, Q, ROOT, 3, 0, b[0]);
    emit("r8f16", N, Q, ROOT, 4, 0, c[0]);
}

int main() {
    /* q = 12289 with 41 of order 4096 (src/project.cpp:47-48) and its powers */
    r2f16<4096, 12289, 41>();
    r2f16<1024, 12289, 11580>();
    r2f16<256, 12289, 145>();
    r2f16<16, 12289, 11567>();
    r2i16<4096, 12289, 41>();
    r2i16<1024, 12289, 11580>();
    r2i16<256, 12289, 145>();
    r2i16<16, 12289, 11567>();
    r4f16<4096, 12289, 41>();
    r4f16<1024, 12289, 11580>();
    r4f16<256, 12289, 145>();
    r4f16<16, 12289, 11567>();
    r4f16<256, 7681, 2028>();
    r4f16<256, 10753, 4305>();
    r8f16<4096, 12289, 41>();
    r8f16<512, 12289, 11121>();
    r8f16<64, 12289, 3006>();
    /* q = 1073707009 with 992735929 of order 2048 (src/project.cpp:50-51) */
    r2i32<2048, 1073707009, 992735929>();
    r2i32<256, 1073707009, 196914830>();
    /* four 30-bit RNS primes */
    r2i32<4096, 998244353, 63912897>();
    r2i32<4096, 469762049, 244412522>();
    r2i32<4096, 167772161, 150794572>();
    r2i32<4096, 754974721, 259521057>();
    r2i32<256, 998244353, 476477967>();
    r2i32<16, 754974721, 49823357>();
    return 0;
}
