// persist.cuh -- the persistent batched transform kernel.
//
// One launch transforms every polynomial of a batch made of segments (design,
// n, q, input, output, count).  Work is cut into tiles of P polynomials
// (P = CTA threads / G, G = threads per polynomial) and handed out by a global
// atomic counter, largest n first.  Each CTA double-buffers its tiles in
// shared memory with the Tensor Memory Accelerator's bulk copies:
//
//   cp.async.bulk global->shared (mbarrier complete_tx) prefetches tile t+1
//   while tile t is transformed; the results are written back into the same
//   shared buffer and leave with cp.async.bulk shared->global.
//
// Inside a tile every polynomial is transformed by the window/exchange scheme
// of device.cuh with 16, 32 or 64 coefficients per thread (the configuration's
// width; the autotuner picks it per batch).  The strided staging layout is
// conflict-free at every width; the padded exchange layout (one spare word
// per 32) is conflict-free at 32 and leaves some two-way conflicts at 16.
#pragma once

#include "device.cuh"

namespace gbntt {

// scratch words of a batch (device memory owned by the batch object)
enum { CTR_NEXT = 0, CTR_DONE = 1, CTR_ERROR = 2, CTR_WORDS = 4 };
enum { BERR_TIMEOUT = 1 };

struct SegDev {
    KArgs a;              // in, out, batch (= polynomial count), tables, constants
    long long tile0;      // first tile of the segment in the global tile order
    long long tiles;      // number of tiles
    int variant;          // (family << 4) | L
    int polys_per_tile;   // P
    int n;
    int elem_bytes;
};

struct BatchDev {
    const SegDev* segs;
    int nsegs;
    long long total_tiles;
    unsigned long long* ctr;   // CTR_WORDS scratch words, zero between launches
    unsigned wait_polls;       // poll limit of a tile load's wait (BATCH_WAIT_POLLS; smaller in tests)
};

// The poll limit of every bounded wait: far beyond any real copy's latency,
// short enough that a lost copy ends the launch with an error in seconds.
constexpr unsigned BATCH_WAIT_POLLS = 1u << 22;

// coefficients per thread (log2) of a persistent-kernel configuration
__host__ __device__ constexpr int batch_el(int L, int elmax) { return L < elmax ? L : elmax; }
__host__ __device__ constexpr int variant_id(int fam, int L) { return (fam << 4) | L; }

// ---------------------------------------------------------------------------
// PTX wrappers: mbarrier and bulk (TMA) copies
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned smem_addr(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Bounded wait for the phase `parity` of the barrier: at most `polls` polls.
// Returns false when they ran out (the caller records an error and stops).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity,
                                          unsigned polls = BATCH_WAIT_POLLS) {
    const unsigned a = smem_addr(bar);
    for (unsigned it = 0; it < polls; ++it) {
        unsigned ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void bulk_load(void* dst_smem, const void* src_gmem, unsigned bytes,
                                          unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst_smem)),
        "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void bulk_store(void* dst_gmem, const void* src_smem, unsigned bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst_gmem),
                 "r"(smem_addr(src_smem)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// wait until the shared-memory sources of all committed bulk stores have been read
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// wait until all committed bulk stores are complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// make generic-proxy shared-memory writes visible to the bulk-copy (async) proxy
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---------------------------------------------------------------------------
// one tile: P polynomials staged contiguously in shared memory
// ---------------------------------------------------------------------------

// reads one staged polynomial into the window layout LOS; BRV: the staged
// polynomial is in natural order and the transform wants it bit-reversed
template <bool I32, int L, int EL, int LOS, bool BRV>
__device__ __forceinline__ void stage_read(int (&v)[1 << EL], const void* stage, int lp, int g) {
    constexpr int E = 1 << EL, N = 1 << L;
    // bitrev of a position = bitrev(thread bits) | bitrev(register bits)
    const int base = lp * N + (BRV ? (int)(__brev((unsigned)posmap<LOS, EL>(g, 0)) >> (32 - L)) : 0);
#pragma unroll
    for (int k = 0; k < E; ++k) {
        const int p = BRV ? base + brev_c<L>(k << LOS) : lp * N + posmap<LOS, EL>(g, k);
        if constexpr (I32) v[k] = static_cast<const int*>(stage)[p];
        else v[k] = static_cast<const short*>(stage)[p];
    }
}

// reads one staged polynomial in the window at bit 0: thread g's contiguous
// run of E coefficients, with 16-byte accesses
template <bool I32, int L, int EL>
__device__ __forceinline__ void stage_read_run(int (&v)[1 << EL], const void* stage, int lp, int g) {
    constexpr int E = 1 << EL, N = 1 << L;
    if constexpr (I32) {
        const int4* s4 = reinterpret_cast<const int4*>(static_cast<const int*>(stage) + lp * N + g * E);
#pragma unroll
        for (int j = 0; j < E / 4; ++j) {
            const int4 w = s4[j];
            v[4 * j] = w.x; v[4 * j + 1] = w.y; v[4 * j + 2] = w.z; v[4 * j + 3] = w.w;
        }
    } else {
        const int4* s4 = reinterpret_cast<const int4*>(static_cast<const short*>(stage) + lp * N + g * E);
#pragma unroll
        for (int j = 0; j < E / 8; ++j) {
            const int4 w = s4[j];
            const int ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                v[8 * j + 2 * h] = (int)(short)(ww[h] & 0xFFFF);
                v[8 * j + 2 * h + 1] = ww[h] >> 16;
            }
        }
    }
}

// ka: the segment's arguments in shared memory, read only where the output
// options are applied (natural order, n^-1 scaling, canonical form)
template <int FAM, int L, int CTA, int ELMAX>
__device__ __forceinline__ void tile_transform(void* stage, int* xbuf, const KC& a, const KArgs& ka, int npolys) {
    constexpr int EL = batch_el(L, ELMAX);
    constexpr int G = 1 << (L - EL), N = 1 << L, E = 1 << EL;
    constexpr int SW = xwords(L);
    constexpr int NS = nsteps(FAM, L);
    constexpr int LOS = L - EL;                          // staging layout: strided, conflict-free
    constexpr int LO0 = window_lo(FAM, L, EL, 0);
    constexpr int LOZ = window_lo(FAM, L, EL, NS - 1);
    constexpr bool I32 = fam_i32(FAM);
    static_assert(CTA % G == 0, "a polynomial must not straddle CTAs");
    const int tid = threadIdx.x;
    const int lp = tid / G, g = tid % G;
    const bool active = lp < npolys;
    int* sp = xbuf + lp * SW;
    int v[E];
    // A first window on the low bits (the inverse designs) reads each thread's
    // contiguous run with 16-byte accesses, unless the input is in natural
    // order; otherwise the strided read, then an exchange to the first window.
    constexpr bool RUN_READ = LO0 == 0 && LO0 != LOS && (I32 ? E >= 4 : E >= 8);
    bool in_window = false;
    if (active) {
        // natural-order input of an inverse design: the bit reversal is the read pattern
        if constexpr (fam_natural_in(FAM, false)) {
            if (ka.natural_in) {
                stage_read<I32, L, EL, LOS, true>(v, stage, lp, g);
            } else if constexpr (RUN_READ) {
                stage_read_run<I32, L, EL>(v, stage, lp, g);
                in_window = true;
            } else {
                stage_read<I32, L, EL, LOS, false>(v, stage, lp, g);
            }
        } else {
            stage_read<I32, L, EL, LOS, false>(v, stage, lp, g);
        }
    } else {
#pragma unroll
        for (int k = 0; k < E; ++k) v[k] = 0;
    }
    prologue<FAM>(v, ka);
    // The exchange buffer was last read before the barrier that ends the
    // caller's previous tile (or never), so the tile's first exchange needs no
    // leading barrier.
    bool fresh = true;
    if constexpr (LO0 != LOS) {
        // the CTA agrees on the path (natural_in is the segment's): every
        // thread takes the exchange or none does
        if constexpr (RUN_READ) {
            if (!__syncthreads_or(in_window)) {
                exchange_windows<L, EL, LOS, LO0>(v, sp, g, false);
                fresh = false;
            }
        } else {
            exchange_windows<L, EL, LOS, LO0>(v, sp, g, false);
            fresh = false;
        }
    }
    run_steps<FAM, L, EL>(v, sp, g, a, fresh, std::make_integer_sequence<int, NS>{});
    epilogue<FAM, false>(v, ka);
    if (!active) return;
    if constexpr (fam_natural_out(FAM, false)) {
        if (ka.natural_out) {
            // natural-order output of a forward design: bit-reversed scatter into the tile
            const int base = lp * N + (int)(__brev((unsigned)posmap<LOZ, EL>(g, 0)) >> (32 - L));
#pragma unroll
            for (int k = 0; k < E; ++k) {
                const int p = base + brev_c<L>(k << LOZ);
                if constexpr (I32) static_cast<int*>(stage)[p] = v[k];
                else static_cast<short*>(stage)[p] = (short)v[k];
            }
            return;
        }
    }
    if constexpr (LOZ == 0 && (I32 ? E >= 4 : E >= 8)) {
        // thread owns E consecutive coefficients: 16-byte stores
        if constexpr (I32) {
            int4* d = reinterpret_cast<int4*>(static_cast<int*>(stage) + lp * N + g * E);
#pragma unroll
            for (int j = 0; j < E / 4; ++j) d[j] = make_int4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        } else {
            int4* d = reinterpret_cast<int4*>(static_cast<short*>(stage) + lp * N + g * E);
#pragma unroll
            for (int j = 0; j < E / 8; ++j) {
                int w[4];
#pragma unroll
                for (int h = 0; h < 4; ++h) w[h] = (v[8 * j + 2 * h] & 0xFFFF) | (v[8 * j + 2 * h + 1] << 16);
                d[j] = make_int4(w[0], w[1], w[2], w[3]);
            }
        }
    } else {
        if constexpr (I32) {
            int* d = static_cast<int*>(stage) + lp * N;
#pragma unroll
            for (int k = 0; k < E; ++k) d[posmap<LOZ, EL>(g, k)] = v[k];
        } else {
            short* d = static_cast<short*>(stage) + lp * N;
#pragma unroll
            for (int k = 0; k < E; ++k) d[posmap<LOZ, EL>(g, k)] = (short)v[k];
        }
    }
}

// shared-memory bytes the persistent kernel needs for the largest variant of a batch
__host__ __device__ constexpr int batch_stage_bytes(int cta, int L, int elem, int elmax) {
    // P * N = cta * E coefficients per tile
    return cta * (1 << batch_el(L, elmax)) * elem;
}
__host__ __device__ constexpr int batch_xbuf_bytes(int cta, int L, int elmax) {
    return batch_el(L, elmax) == L ? 0 : (cta >> (L - batch_el(L, elmax))) * xwords(L) * 4;
}

}  // namespace gbntt
