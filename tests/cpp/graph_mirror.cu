// Drives the C++ graph classes of include/gb300_ntt.hpp the way the
// reference's src/project.cpp drives its graphs: init(); run(ITERATIONS);
// end().  Checks forward -> inverse -> n^-1 round trips for NTT_CONFIG 0/1/7,
// 4/5 and the radix-4 pair, exact round trips of the canonical arithmetic
// (GBNTT_FLAG_CANONICAL as the constructor argument), and writes the NTT_CONFIG 0 forward output to the
// file given as argv[1] so the Python test can compare it with the oracle.
#include <cuda_runtime.h>

#include <cstdio>
#include <random>
#include <vector>

#include "gb300_ntt.hpp"

using namespace gb300ntt;

static constexpr unsigned ITERATIONS = 100;   // src/project.cpp:42

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { std::printf("cuda: %s\n", cudaGetErrorString(e_)); return 2; } } while (0)

template <typename T>
static int roundtrip(graph& fwd, graph& inv, uint32_t n, int64_t q, const std::vector<T>& x,
                     std::vector<T>& y_host) {
    const size_t bytes = x.size() * sizeof(T);
    T *dx, *dy, *dz;
    CK(cudaMalloc(&dx, bytes)); CK(cudaMalloc(&dy, bytes)); CK(cudaMalloc(&dz, bytes));
    CK(cudaMemcpy(dx, x.data(), bytes, cudaMemcpyHostToDevice));
    fwd.init(); inv.init();
    fwd.in_data = dx; fwd.out_data = dy; fwd.run(ITERATIONS);
    inv.in_data = dy; inv.out_data = dz; inv.run(ITERATIONS);
    std::vector<T> z(x.size());
    y_host.resize(x.size());
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(z.data(), dz, bytes, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(y_host.data(), dy, bytes, cudaMemcpyDeviceToHost));
    fwd.end(); inv.end();
    cudaFree(dx); cudaFree(dy); cudaFree(dz);
    for (size_t i = 0; i < x.size(); ++i) {
        const int64_t want = (int64_t)x[i] * n % q;
        const int64_t got = (((int64_t)z[i] % q) + q) % q;
        if (want != got) { std::printf("mismatch at %zu\n", i); return 1; }
    }
    return 0;
}

// canonical residues: the forward's outputs lie in [0, q) and the inverse
// with the fused n^-1 scaling returns the input exactly
template <typename T>
static int exact_roundtrip(graph& fwd, graph& inv, int64_t q, const std::vector<T>& x) {
    const size_t bytes = x.size() * sizeof(T);
    T *dx, *dy, *dz;
    CK(cudaMalloc(&dx, bytes)); CK(cudaMalloc(&dy, bytes)); CK(cudaMalloc(&dz, bytes));
    CK(cudaMemcpy(dx, x.data(), bytes, cudaMemcpyHostToDevice));
    fwd.init(); inv.init();
    fwd.in_data = dx; fwd.out_data = dy; fwd.run(ITERATIONS);
    inv.in_data = dy; inv.out_data = dz; inv.run(ITERATIONS);
    std::vector<T> y(x.size()), z(x.size());
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(y.data(), dy, bytes, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(z.data(), dz, bytes, cudaMemcpyDeviceToHost));
    fwd.end(); inv.end();
    cudaFree(dx); cudaFree(dy); cudaFree(dz);
    for (size_t i = 0; i < x.size(); ++i) {
        if (y[i] < 0 || (int64_t)y[i] >= q) { std::printf("canonical output out of range at %zu\n", i); return 1; }
        if (z[i] != x[i]) { std::printf("canonical round trip mismatch at %zu\n", i); return 1; }
    }
    return 0;
}

int main(int argc, char** argv) {
    std::mt19937_64 rng(20261203);
    // NTT_CONFIG 0 / 1 / 7
    constexpr uint32_t N16 = 4096;
    std::vector<int16_t> x16(N16 * ITERATIONS);
    for (auto& v : x16) v = (int16_t)(rng() % Q_INT16);
    std::vector<int16_t> y16;
    NTT<N16, Q_INT16, ROOT_INT16, NTT_TYPE::TYPE_NTT_NO_to_BO> fwd16;
    NTT<N16, Q_INT16, ROOT_INT16, NTT_TYPE::TYPE_INTT_BO_to_NO> inv16;
    if (roundtrip(fwd16, inv16, N16, Q_INT16, x16, y16)) return 1;
    {
        // n^-1 scaling of the inverse output with the full Barrett unit
        NTT<N16, Q_INT16, ROOT_INT16, NTT_TYPE::TYPE_INTT_BO_to_NO> inv;
        FULL_BARRETT_MULTIPLICATION<N16, Q_INT16, (uint32_t)mod_inverse(N16, Q_INT16)> norm;
        int16_t *dy, *dz, *dw;
        const size_t bytes = y16.size() * 2;
        CK(cudaMalloc(&dy, bytes)); CK(cudaMalloc(&dz, bytes)); CK(cudaMalloc(&dw, bytes));
        CK(cudaMemcpy(dy, y16.data(), bytes, cudaMemcpyHostToDevice));
        inv.in_data = dy; inv.out_data = dz; inv.run(ITERATIONS);
        norm.in_data = dz; norm.out_data = dw; norm.run(ITERATIONS);
        std::vector<int16_t> w(y16.size());
        CK(cudaDeviceSynchronize());
        CK(cudaMemcpy(w.data(), dw, bytes, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < w.size(); ++i)
            if ((w[i] % (int)Q_INT16 + (int)Q_INT16) % (int)Q_INT16 != x16[i] || w[i] < 0 || w[i] > (int)Q_INT16) {
                std::printf("normalised mismatch at %zu\n", i);
                return 1;
            }
        cudaFree(dy); cudaFree(dz); cudaFree(dw);
    }
    // NTT_CONFIG 4 / 5
    constexpr uint32_t N32 = 2048;
    std::vector<int32_t> x32(N32 * ITERATIONS), y32;
    for (auto& v : x32) v = (int32_t)(rng() % Q_INT32);
    NTT_INT32<N32, Q_INT32, ROOT_INT32, NTT_INT32_TYPE::FORWARD_CT_NO_TO_BO> fwd32;
    NTT_INT32<N32, Q_INT32, ROOT_INT32, NTT_INT32_TYPE::INVERSE_GS_BO_TO_NO> inv32;
    if (roundtrip(fwd32, inv32, N32, Q_INT32, x32, y32)) return 1;
    // radix-4 forward + inverse (NTT_CONFIG 2 and its described inverse)
    std::vector<int16_t> y4;
    NTT_R4<N16, Q_INT16, ROOT_INT16, NTT_R4_TYPE::FORWARD_CT_NO_TO_BO> fwd4;
    NTT_R4<N16, Q_INT16, ROOT_INT16, NTT_R4_TYPE::INVERSE_BO_TO_NO> inv4;
    if (roundtrip(fwd4, inv4, N16, Q_INT16, x16, y4)) return 1;
    // the canonical arithmetic through the same classes (flags as the constructor argument)
    {
        NTT<N16, Q_INT16, ROOT_INT16, NTT_TYPE::TYPE_NTT_NO_to_BO> fwd(GBNTT_FLAG_CANONICAL);
        NTT<N16, Q_INT16, ROOT_INT16, NTT_TYPE::TYPE_INTT_BO_to_NO> inv(GBNTT_FLAG_CANONICAL | GBNTT_FLAG_SCALE_NINV);
        if (exact_roundtrip(fwd, inv, Q_INT16, x16)) return 1;
        // an NTT prime below 2^30 (the canonical int32 family's range) and a
        // root of order 2048: 3^((q - 1) / 2048)
        constexpr uint32_t QC = 998244353, RC = 584193783;
        std::vector<int32_t> xc(N32 * ITERATIONS);
        for (auto& v : xc) v = (int32_t)(rng() % QC);
        NTT_INT32<N32, QC, RC, NTT_INT32_TYPE::FORWARD_CT_NO_TO_BO> fwdi(GBNTT_FLAG_CANONICAL);
        NTT_INT32<N32, QC, RC, NTT_INT32_TYPE::INVERSE_GS_BO_TO_NO> invi(GBNTT_FLAG_CANONICAL | GBNTT_FLAG_SCALE_NINV);
        if (exact_roundtrip(fwdi, invi, QC, xc)) return 1;
    }
    // unsupported parameters are reported, not silently accepted
    try {
        graph bad(GBNTT_R2_I16_FWD, 4096, 12289, 2, 0, 0);
        bad.init();
        std::printf("bad root accepted\n");
        return 1;
    } catch (const Error& e) {
        if (e.code != GBNTT_ERR_ROOT) return 1;
    }
    if (argc > 1) {
        FILE* f = std::fopen(argv[1], "wb");
        std::fwrite(y16.data(), 2, y16.size(), f);
        std::fclose(f);
    }
    std::printf("graph mirror ok\n");
    return 0;
}
