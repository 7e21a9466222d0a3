// kernels_large.cu -- int32 transforms of 2^16 .. 2^22 coefficients in two passes.
//
// The reference's layers are in-place butterflies on position bits (see
// device.cuh).  For n = 2^(L1 + L2), the forward layers on the L1 high bits
// touch, for each fixed low part c, only the positions (j << L2) | c; their
// twiddle block is j's bits above the butterfly, independent of c.  So the
// first L1 layers are 2^L2 independent L1-bit sub-transforms over "columns"
// (stride 2^L2), and the last L2 layers are 2^L1 sub-transforms over
// contiguous "rows" whose block index is (row << L2 | s) >> (bit + 1).  The
// inverse (Gentleman-Sande, low bits first) runs rows first, then columns.
// Every butterfly keeps the reference's arithmetic, so outputs stay bit-exact.
#include "device.cuh"

namespace gbntt {

namespace {

// 16 coefficients per thread (measured against 32 on GB300, same box: n = 2^20
// forward 0.77 vs 0.86 ms, inverse 0.67 vs 0.85 ms for 64 polynomials)
constexpr int LARGE_EL = 4;
constexpr int COLS_PER_CTA = 16;   // fewer when 16 columns would need more than 1024 threads

// one CTA: COLS adjacent columns of one polynomial, G threads per column
template <int FAM, int L1, int COLS>
__global__ void __launch_bounds__(COLS << (L1 - LARGE_EL)) k_cols(const __grid_constant__ KArgs a, int L2) {
    constexpr int EL = LARGE_EL, G = 1 << (L1 - EL), E = 1 << EL, NS = nsteps(FAM, L1);
    constexpr int LO0 = window_lo(FAM, L1, EL, 0), LOZ = window_lo(FAM, L1, EL, NS - 1);
    extern __shared__ int csmem[];
    grid_dep_start();
    const int tid = threadIdx.x, cl = tid % COLS, g = tid / COLS;
    const long long blocks_per_poly = (1LL << L2) / COLS;
    const long long poly = blockIdx.x / blocks_per_poly;
    const long long c0 = (blockIdx.x % blocks_per_poly) * COLS;
    const long long base = (poly << (L1 + L2)) + c0 + cl;
    const int* in = static_cast<const int*>(a.in) + base;
    int* out = static_cast<int*>(a.out) + base;
    int v[E];
#pragma unroll
    for (int k = 0; k < E; ++k) v[k] = __ldg(in + ((long long)posmap<LO0, EL>(g, k) << L2));
    const KC kc = make_kc(a);
    run_steps_x<FAM, L1, EL, COLS, false>(v, csmem, g, kc, 0, cl, std::make_integer_sequence<int, NS>{});
    epilogue_all<false>(v, a);
    __syncthreads();   // every read of `in` is done before an in-place store lands
#pragma unroll
    for (int k = 0; k < E; ++k) out[(long long)posmap<LOZ, EL>(g, k) << L2] = v[k];
}

// one CTA: P rows of 2^L2 coefficients, G threads per row
template <int FAM, int L2, int P>
__global__ void __launch_bounds__(P << (L2 - LARGE_EL)) k_rows(const __grid_constant__ KArgs a, int L1) {
    constexpr int EL = LARGE_EL, G = 1 << (L2 - EL), E = 1 << EL, NS = nsteps(FAM, L2), N = 1 << L2;
    constexpr int LO0 = window_lo(FAM, L2, EL, 0), LOZ = window_lo(FAM, L2, EL, NS - 1);
    extern __shared__ int rsmem[];
    grid_dep_start();
    const int tid = threadIdx.x, lp = tid / G, g = tid % G;
    const long long row = (long long)blockIdx.x * P + lp;        // rows of all polynomials, in order
    const bool active = row < (a.batch << L1);
    const int hi = (int)(row & ((1LL << L1) - 1));               // row index inside its polynomial
    int* sp = rsmem + lp * xwords(L2);
    int v[E];
    // rows are contiguous: every thread moves E consecutive coefficients with
    // 16-byte accesses, and the exchange buffer turns them into (and back
    // from) the transform's first (last) window
    if (active) {
        const int4* src = reinterpret_cast<const int4*>(static_cast<const int*>(a.in) + row * N) + g * (E / 4);
#pragma unroll
        for (int j = 0; j < E / 4; ++j) {
            const int4 w = __ldg(src + j);
            v[4 * j] = w.x; v[4 * j + 1] = w.y; v[4 * j + 2] = w.z; v[4 * j + 3] = w.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < E; ++k) v[k] = 0;
    }
    if constexpr (LO0 != 0) exchange_windows<L2, EL, 0, LO0>(v, sp, g);
    const KC kc = make_kc(a);
    run_steps_x<FAM, L2, EL, 0, true>(v, sp, g, kc, hi, 0, std::make_integer_sequence<int, NS>{});
    epilogue_all<false>(v, a);
    if constexpr (LOZ != 0) exchange_windows<L2, EL, LOZ, 0>(v, sp, g);
    if (active) {
        int4* dst = reinterpret_cast<int4*>(static_cast<int*>(a.out) + row * N) + g * (E / 4);
#pragma unroll
        for (int j = 0; j < E / 4; ++j) dst[j] = make_int4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
    }
}

template <int FAM, int L1, int L2>
LargeInfo make_large() {
    LargeInfo li;
    li.L1 = L1;
    li.L2 = L2;
    constexpr int C = (COLS_PER_CTA << (L1 - LARGE_EL)) > 1024 ? (1024 >> (L1 - LARGE_EL)) : COLS_PER_CTA;
    li.cols = reinterpret_cast<const void*>(&k_cols<FAM, L1, C>);
    li.cols_threads = C << (L1 - LARGE_EL);
    li.cols_smem = C * (1 << L1) * 4;
    li.cols_per_cta = C;
    constexpr int G2 = 1 << (L2 - LARGE_EL);
    constexpr int P = G2 >= 256 ? 1 : 256 / G2;
    li.rows = reinterpret_cast<const void*>(&k_rows<FAM, L2, P>);
    li.rows_threads = P * G2;
    li.rows_smem = P * xwords(L2) * 4;
    li.rows_per_cta = P;
    return li;
}

template <int FAM>
LargeInfo large_for(int L) {
    switch (L) {
    case 16: return make_large<FAM, 8, 8>();
    case 17: return make_large<FAM, 9, 8>();
    case 18: return make_large<FAM, 9, 9>();
    case 19: return make_large<FAM, 10, 9>();
    case 20: return make_large<FAM, 10, 10>();
    case 21: return make_large<FAM, 11, 10>();
    case 22: return make_large<FAM, 11, 11>();
    default: return LargeInfo();
    }
}

}  // namespace

LargeInfo large_info(int fam, int L) {
    if (fam == F_R2F32) return large_for<F_R2F32>(L);
    if (fam == F_R2G32) return large_for<F_R2G32>(L);
    return LargeInfo();
}

}  // namespace gbntt
