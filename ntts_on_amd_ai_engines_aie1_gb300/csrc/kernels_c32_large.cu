// kernels_c32_large.cu -- canonical int32 transforms of 2^14 .. 2^22
// coefficients as a four-step (column pass, twist, row pass).
//
// With n = n1 n2 and the polynomial viewed as n1 rows of n2 coefficients
// (row-major, no transpose in memory), the forward transform with output in
// bit-reversed order is
//   1. every column c: the length-n1 transform with root^n2, bit-reversed
//      along the column (row r then holds frequency k1 = bitrev(r));
//   2. the twist: row r, column c times root^(c bitrev(r));
//   3. every row: the length-n2 transform with root^n1, bit-reversed along
//      the row,
// and the inverse (bit-reversed in, natural out, no n^-1) runs the inverse
// steps in the opposite order: rows, untwist by root^-(c bitrev(r)), columns.
// Polynomials go through both passes in chunks of at most large_chunk_bytes(), so the
// intermediate stays in L2 between the passes.
//
// The column pass moves 2D tiles (COLS adjacent columns x n1 rows) between
// global and shared memory with the Tensor Memory Accelerator
// (cp.async.bulk.tensor.2d, an mbarrier with a bounded wait for the load, a
// bulk-group store); with lane = column every shared-memory access of a warp
// touches 32 distinct banks.  The row pass reads and writes whole rows with
// coalesced accesses and applies the twist as two Shoup multiplications by
// factors from two small tables (the twist of row r at column c = t + G k, with
// t the thread's column and k its register, is A[r][t] * B[r][k]).
#include <cuda.h>

#include "canon_tables.h"
#include "device.cuh"
#include "persist.cuh"

namespace gbntt {

namespace {

constexpr int ROW_EL = 4;            // 16 coefficients per thread in the row pass

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c, int r,
                                            unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(c), "r"(r), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int c, int r, const void* src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     reinterpret_cast<unsigned long long>(map)),
                 "r"(c), "r"(r), "r"(smem_addr(src))
                 : "memory");
}

// the column pass: COLS adjacent columns x N1 rows of one polynomial per CTA,
// G = N1 / 2^EL threads per column
template <int FAM, int L1, int EL, int COLS>
__global__ void __launch_bounds__(COLS << (L1 - EL))
    k_ccols(const __grid_constant__ CUtensorMap min, const __grid_constant__ CUtensorMap mout,
            const __grid_constant__ KArgs a, int n2, long long tile0, unsigned* err) {
    constexpr int E = 1 << EL, N1 = 1 << L1, NS = nsteps(FAM, L1);
    constexpr int R = N1 < 256 ? N1 : 256, NB = N1 / R;       // TMA boxes of at most 256 rows
    constexpr int LO0 = window_lo(FAM, L1, EL, 0), LOZ = window_lo(FAM, L1, EL, NS - 1);
    constexpr bool FWD = topdown(FAM);
    extern __shared__ __align__(128) unsigned char csm[];
    int* tile = reinterpret_cast<int*>(csm);
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(csm + N1 * COLS * 4);
    const int tid = threadIdx.x, cl = tid % COLS, g = tid / COLS;
    const long long tpp = n2 / COLS;                           // column tiles per polynomial
    const long long t = tile0 + blockIdx.x;
    const int c0 = (int)((t % tpp) * COLS);
    const int r0 = (int)((t / tpp) * N1);
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    grid_dep_start();
    if (tid == 0) {
        mbar_expect_tx(bar, N1 * COLS * 4);
#pragma unroll
        for (int b = 0; b < NB; ++b) tma_load_2d(tile + b * R * COLS, &min, c0, r0 + b * R, bar);
    }
    const bool ok = mbar_wait(bar, 0);
    if (!__syncthreads_and(ok)) {
        // the tile did not arrive in time: record it, let the copy land, stop
        if (tid == 0) {
            atomicOr(err, 1u);
            mbar_wait(bar, 0);
        }
        return;
    }
    int v[E];
#pragma unroll
    for (int k = 0; k < E; ++k) v[k] = tile[posmap<LO0, EL>(g, k) * COLS + cl];
    if constexpr (FWD) prologue<FAM>(v, a);                    // raw input (the first pass)
    const KC kc = make_kc(a);
    run_steps_x<FAM, L1, EL, COLS, false>(v, tile, g, kc, 0, cl, std::make_integer_sequence<int, NS>{});
    if constexpr (!FWD) epilogue<FAM, false>(v, a);            // the inverse's last pass
    __syncthreads();                                           // every read of the tile is done
#pragma unroll
    for (int k = 0; k < E; ++k) tile[posmap<LOZ, EL>(g, k) * COLS + cl] = v[k];
    fence_proxy_async();                                       // visible to the bulk store
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int b = 0; b < NB; ++b) tma_store_2d(&mout, c0, r0 + b * R, tile + b * R * COLS);
        bulk_commit();
        bulk_wait_read();                                      // the tile is read before the CTA leaves
    }
}

// the row pass: P rows of N2 coefficients per CTA, G = N2 / 2^EL threads per
// row; rows are numbered over the whole call, row r of its polynomial = r mod n1
template <int FAM, int L2, int EL, int P>
__global__ void __launch_bounds__(P << (L2 - EL)) k_crows(const __grid_constant__ KArgs a, int L1, long long row0,
                                                          long long rows) {
    constexpr int G = 1 << (L2 - EL), E = 1 << EL, N2 = 1 << L2, NS = nsteps(FAM, L2);
    constexpr int LO0 = window_lo(FAM, L2, EL, 0), LOZ = window_lo(FAM, L2, EL, NS - 1);
    constexpr bool FWD = topdown(FAM);
    // the twist sits on the window whose thread part is the low column bits
    static_assert((FWD ? LO0 : LOZ) == L2 - EL, "twist layout");
    static_assert((FWD ? LOZ : LO0) == 0, "contiguous runs on the other side");
    extern __shared__ int rsm[];
    grid_dep_start();
    const int tid = threadIdx.x, lp = tid / G, g = tid % G;
    const long long row = row0 + (long long)blockIdx.x * P + lp;
    const bool active = row < row0 + rows;
    const int n1 = 1 << L1;
    const int r = (int)(row & (n1 - 1));
    int* sp = rsm + lp * xwords(L2);
    const unsigned q = (unsigned)a.q;
    int v[E];
    if constexpr (FWD) {
        // strided window: thread g holds columns g + G k
        if (active) {
            const int* src = static_cast<const int*>(a.in) + row * N2;
#pragma unroll
            for (int k = 0; k < E; ++k) v[k] = __ldg(src + posmap<LO0, EL>(g, k));
            const int2 A = __ldg(&a.twist[r * G + g]);
            const int2* B = a.twist + (long long)n1 * G + r * E;
#pragma unroll
            for (int k = 0; k < E; ++k) {
                const int2 b = __ldg(B + k);
                v[k] = (int)shoup_mul(shoup_mul((unsigned)v[k], (unsigned)A.x, (unsigned)A.y, q), (unsigned)b.x,
                                      (unsigned)b.y, q);
            }
        } else {
#pragma unroll
            for (int k = 0; k < E; ++k) v[k] = 0;
        }
    } else {
        // contiguous run: thread g holds columns g E .. g E + E - 1
        if (active) {
            const int4* src = reinterpret_cast<const int4*>(static_cast<const int*>(a.in) + row * N2) + g * (E / 4);
#pragma unroll
            for (int j = 0; j < E / 4; ++j) {
                const int4 w = __ldg(src + j);
                v[4 * j] = w.x; v[4 * j + 1] = w.y; v[4 * j + 2] = w.z; v[4 * j + 3] = w.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < E; ++k) v[k] = 0;
        }
        prologue<FAM>(v, a);                                   // raw input (the first pass)
    }
    const KC kc = make_kc(a);
    run_steps<FAM, L2, EL>(v, sp, g, kc, true, std::make_integer_sequence<int, NS>{});   // sp untouched so far
    if (!active) return;                                       // no exchange follows
    if constexpr (FWD) {
        epilogue<FAM, false>(v, a);                            // the forward's last pass
        int4* dst = reinterpret_cast<int4*>(static_cast<int*>(a.out) + row * N2) + g * (E / 4);
#pragma unroll
        for (int j = 0; j < E / 4; ++j) dst[j] = make_int4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
    } else {
        const int2 A = __ldg(&a.twist[r * G + g]);
        const int2* B = a.twist + (long long)n1 * G + r * E;
        int* dst = static_cast<int*>(a.out) + row * N2;
#pragma unroll
        for (int k = 0; k < E; ++k) {
            const int2 b = __ldg(B + k);
            dst[posmap<LOZ, EL>(g, k)] = (int)shoup_mul(
                shoup_mul((unsigned)v[k], (unsigned)A.x, (unsigned)A.y, q), (unsigned)b.x, (unsigned)b.y, q);
        }
    }
}

// split of 2^L: rows of 2^12 (2^13 for L = 22), columns of the rest
constexpr int split_l2(int L) { return L >= 22 ? 13 : 12; }
constexpr int col_el(int L1) { return L1 <= 4 ? L1 : (L1 <= 8 ? 4 : 5); }
constexpr int col_width(int L1) {
    const int G = 1 << (L1 - col_el(L1));
    const int c = 256 / G;
    return c < 32 ? 32 : (c > 256 ? 256 : c);
}

template <int FAM, int L>
CanonLarge make_canon_large() {
    constexpr int L2 = split_l2(L), L1 = L - L2;
    constexpr int ELC = col_el(L1), COLS = col_width(L1);
    CanonLarge li;
    li.L1 = L1;
    li.L2 = L2;
    li.row_el = ROW_EL;
    li.cols = reinterpret_cast<const void*>(&k_ccols<FAM, L1, ELC, COLS>);
    li.cols_threads = COLS << (L1 - ELC);
    li.cols_smem = (1 << L1) * COLS * 4 + 16;
    li.cols_width = COLS;
    li.rows = reinterpret_cast<const void*>(&k_crows<FAM, L2, ROW_EL, 1>);
    li.rows_threads = 1 << (L2 - ROW_EL);
    li.rows_smem = xwords(L2) * 4;
    li.rows_per_cta = 1;
    return li;
}

template <int FAM>
CanonLarge canon_large_for(int L) {
    switch (L) {
    case 14: return make_canon_large<FAM, 14>();
    case 15: return make_canon_large<FAM, 15>();
    case 16: return make_canon_large<FAM, 16>();
    case 17: return make_canon_large<FAM, 17>();
    case 18: return make_canon_large<FAM, 18>();
    case 19: return make_canon_large<FAM, 19>();
    case 20: return make_canon_large<FAM, 20>();
    case 21: return make_canon_large<FAM, 21>();
    case 22: return make_canon_large<FAM, 22>();
    default: return CanonLarge();
    }
}

// cuTensorMapEncodeTiled (driver API, version 12000), reached through the runtime
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult qr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &qr) !=
                cudaSuccess ||
            qr != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// a 2D view of `rows` rows of n2 int32 coefficients, COLS x R boxes
cudaError_t make_map(CUtensorMap* map, const void* base, long long rows, int n2, int cols, int box_rows) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return cudaErrorNotSupported;
    const cuuint64_t dims[2] = {(cuuint64_t)n2, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)n2 * 4};
    const cuuint32_t box[2] = {(cuuint32_t)cols, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_INT32, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace

CanonLarge canon_large_info(int fam, int L) {
    if (fam == F_C32F) return canon_large_for<F_C32F>(L);
    if (fam == F_C32I) return canon_large_for<F_C32I>(L);
    return CanonLarge();
}

cudaError_t launch_canon_large(const CanonLarge& li, const KArgs& base, const int2* tab_cols, const int2* tab_rows,
                               const int2* twist, const void* in, void* out, long long batch, bool inverse,
                               unsigned* err, cudaStream_t s, int* launches) {
    const int n1 = 1 << li.L1, n2 = 1 << li.L2;
    const long long n = (long long)n1 * n2;
    const int box_rows = n1 < 256 ? n1 : 256;
    CUtensorMap map_in, map_out;
    cudaError_t e = make_map(&map_out, out, batch * n1, n2, li.cols_width, box_rows);
    if (e != cudaSuccess) return e;
    // the forward's column pass reads the input; the inverse's runs in place
    if (!inverse && in != out) {
        e = make_map(&map_in, in, batch * n1, n2, li.cols_width, box_rows);
        if (e != cudaSuccess) return e;
    } else {
        map_in = map_out;
    }
    long long chunk = large_chunk_bytes() / (n * 4);
    if (chunk < 1) chunk = 1;
    const long long tpp = n2 / li.cols_width;
    KArgs ac = base, ar = base;
    ac.tab = tab_cols;
    ar.tab = tab_rows;
    ar.twist = twist;
    int nl = 0;
    for (long long p0 = 0; p0 < batch; p0 += chunk) {
        const long long np = chunk < batch - p0 ? chunk : batch - p0;
        const long long tile0 = p0 * tpp, row0 = p0 * n1, rows = np * n1;
        int L1 = li.L1;
        // programmatic dependent launches (grid_dep_start)
        auto launch = [&](const void* fn, unsigned grid, int threads, int smem, void** args) {
            ++nl;
            return launch_kernel(fn, grid, threads, smem, args, s, true);
        };
        auto cols = [&]() {
            void* args[] = {&map_in, &map_out, &ac, const_cast<int*>(&n2), const_cast<long long*>(&tile0), &err};
            return launch(li.cols, (unsigned)(np * tpp), li.cols_threads, li.cols_smem, args);
        };
        auto rowsk = [&](const void* src) {
            ar.in = src;
            ar.out = out;
            void* args[] = {&ar, &L1, const_cast<long long*>(&row0), const_cast<long long*>(&rows)};
            return launch(li.rows, (unsigned)((rows + li.rows_per_cta - 1) / li.rows_per_cta), li.rows_threads,
                          li.rows_smem, args);
        };
        if (!inverse) {
            e = cols();
            if (e == cudaSuccess) e = rowsk(out);
        } else {
            e = rowsk(in);
            if (e == cudaSuccess) e = cols();
        }
        if (e != cudaSuccess) return e;
    }
    if (launches) *launches = nl;
    return cudaSuccess;
}

}  // namespace gbntt
