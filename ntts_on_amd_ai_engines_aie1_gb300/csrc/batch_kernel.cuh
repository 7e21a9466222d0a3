// batch_kernel.cuh -- the persistent batch kernel template (instantiated in
// batch_k16.cu and batch_k32.cu, launched by batch.cu).
#pragma once

#include "persist.cuh"

namespace gbntt {

constexpr int SMEM_HEADER = 1024;   // mbarriers + the current segment's KArgs
constexpr int BATCH_CTA = 256;

// every (family, L) the persistent kernels implement, per storage type
#define GB_I16_VARIANTS(X)                                                                                   \
    X(F_R2F16, 3) X(F_R2F16, 4) X(F_R2F16, 5) X(F_R2F16, 6) X(F_R2F16, 7) X(F_R2F16, 8) X(F_R2F16, 9)         \
    X(F_R2F16, 10) X(F_R2F16, 11) X(F_R2F16, 12)                                                             \
    X(F_R2I16, 3) X(F_R2I16, 4) X(F_R2I16, 5) X(F_R2I16, 6) X(F_R2I16, 7) X(F_R2I16, 8) X(F_R2I16, 9)         \
    X(F_R2I16, 10) X(F_R2I16, 11) X(F_R2I16, 12)                                                             \
    X(F_R4F16, 4) X(F_R4F16, 6) X(F_R4F16, 8) X(F_R4F16, 10) X(F_R4F16, 12)                                   \
    X(F_R8F16, 3) X(F_R8F16, 4) X(F_R8F16, 5) X(F_R8F16, 6) X(F_R8F16, 7) X(F_R8F16, 8) X(F_R8F16, 9)         \
    X(F_R8F16, 10) X(F_R8F16, 11) X(F_R8F16, 12)
#define GB_I32_VARIANTS(X)                                                                                   \
    X(F_R2F32, 2) X(F_R2F32, 3) X(F_R2F32, 4) X(F_R2F32, 5) X(F_R2F32, 6) X(F_R2F32, 7) X(F_R2F32, 8)         \
    X(F_R2F32, 9) X(F_R2F32, 10) X(F_R2F32, 11) X(F_R2F32, 12) X(F_R2F32, 13)                                \
    X(F_R2G32, 2) X(F_R2G32, 3) X(F_R2G32, 4) X(F_R2G32, 5) X(F_R2G32, 6) X(F_R2G32, 7) X(F_R2G32, 8)         \
    X(F_R2G32, 9) X(F_R2G32, 10) X(F_R2G32, 11) X(F_R2G32, 12) X(F_R2G32, 13)

// the canonical families (int16 storage 2^3 .. 2^12, int32 2^2 .. 2^13: every
// polynomial is a multiple of 16 bytes, as the bulk copies require)
#define GB_C16_VARIANTS(X)                                                                                   \
    X(F_C16F, 3) X(F_C16F, 4) X(F_C16F, 5) X(F_C16F, 6) X(F_C16F, 7) X(F_C16F, 8) X(F_C16F, 9)               \
    X(F_C16F, 10) X(F_C16F, 11) X(F_C16F, 12)                                                                \
    X(F_C16I, 3) X(F_C16I, 4) X(F_C16I, 5) X(F_C16I, 6) X(F_C16I, 7) X(F_C16I, 8) X(F_C16I, 9)               \
    X(F_C16I, 10) X(F_C16I, 11) X(F_C16I, 12)
#define GB_C32_VARIANTS(X)                                                                                   \
    X(F_C32F, 2) X(F_C32F, 3) X(F_C32F, 4) X(F_C32F, 5) X(F_C32F, 6) X(F_C32F, 7) X(F_C32F, 8)               \
    X(F_C32F, 9) X(F_C32F, 10) X(F_C32F, 11) X(F_C32F, 12) X(F_C32F, 13)                                     \
    X(F_C32I, 2) X(F_C32I, 3) X(F_C32I, 4) X(F_C32I, 5) X(F_C32I, 6) X(F_C32I, 7) X(F_C32I, 8)               \
    X(F_C32I, 9) X(F_C32I, 10) X(F_C32I, 11) X(F_C32I, 12) X(F_C32I, 13)
#define GB_ALL_VARIANTS(X) GB_I16_VARIANTS(X) GB_I32_VARIANTS(X) GB_C16_VARIANTS(X) GB_C32_VARIANTS(X)

// a polynomial of 2^L coefficients fits one CTA of `cta` threads at 2^elmax per thread
__host__ __device__ constexpr bool batch_fits(int L, int cta, int elmax) {
    return (1 << (L - (L < elmax ? L : elmax))) <= cta;
}

// resident CTAs per SM the register budget is sized for
__host__ __device__ constexpr int batch_min_blocks(bool i32, int cta, int elmax) {
    return cta >= 512 ? 1 : (i32 || elmax > 5) ? 2 : elmax == 5 ? 3 : 4;
}

// SET: bit mask of the families whose variants this instantiation carries
// (one kernel per family keeps the register allocation of one design).
// OCC: resident CTAs per SM the registers are budgeted for (0: batch_min_blocks)
template <bool I32, int CTA, int ELMAX, int SET, int OCC = 0>
__global__ void __launch_bounds__(CTA, OCC ? OCC : batch_min_blocks(I32, CTA, ELMAX))
    k_batch(const BatchDev b, int stage_bytes) {
    extern __shared__ __align__(128) unsigned char bsmem[];
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(bsmem);
    KArgs* ka = reinterpret_cast<KArgs*>(bsmem + 64);
    unsigned char* stage0 = bsmem + SMEM_HEADER;
    int* xbuf = reinterpret_cast<int*>(bsmem + SMEM_HEADER + 2 * stage_bytes);
    // sh_next[i]: the tile after the one in buffer i.  Thread 0 writes slot
    // buf at the top of an iteration and every thread reads it after the
    // iteration's last barrier; the next write to that slot comes two
    // iterations later, after the next iteration's last barrier, so no thread
    // can read a value from the wrong iteration.
    __shared__ long long sh_next[2];
    __shared__ int sh_pending[2];
    __shared__ int sh_failed;
    const int tid = threadIdx.x, lane = tid & 31;
    const long long total = b.total_tiles;

    // Segment of tile t: the last segment whose first tile is <= t (tile0 does
    // not decrease; segment 0 starts at tile 0), searched in [lo, nsegs), lo a
    // segment known to start at or before t.
    // seg_find: a whole warp, 32 candidates per round, so a round costs one
    // load latency however many segments the batch has (a CTA's first tile).
    auto seg_find = [&](long long t, int lo) {
        int hi = b.nsegs;
        while (hi - lo > 1) {
            const int step = (hi - lo + 31) >> 5;
            const int j = lo + step * lane;
            const unsigned m = __ballot_sync(0xffffffffu, j < hi && __ldg(&b.segs[j].tile0) <= t);
            lo += step * (31 - __clz(m));                 // lane 0 (j = lo) always qualifies
            hi = min(hi, lo + step);
        }
        return lo;
    };
    // seg_of: one thread; a CTA's tiles increase, so the common case is t still
    // in segment lo (one load); past it, a binary search
    auto seg_of = [&](long long t, int lo) {
        int hi = b.nsegs;
        if (lo + 1 >= hi || __ldg(&b.segs[lo + 1].tile0) > t) return lo;
        ++lo;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(&b.segs[mid].tile0) <= t) lo = mid;
            else hi = mid;
        }
        return lo;
    };
    // one thread: start the bulk load of tile t (segment s) into buffer i
    auto issue = [&](long long t, int i, int s) {
        const SegDev* sd = &b.segs[s];
        const long long lt = t - sd->tile0;
        const long long P = sd->polys_per_tile;
        const long long count = sd->a.batch;
        const long long np = min(P, count - lt * P);
        const unsigned bytes = (unsigned)(np * sd->n * sd->elem_bytes);
        const char* src = static_cast<const char*>(sd->a.in) + lt * P * sd->n * sd->elem_bytes;
        mbar_expect_tx(&bar[i], bytes);
        bulk_load(stage0 + i * stage_bytes, src, bytes, &bar[i]);
    };

    // The first tile of a CTA is its block index (the grid never exceeds the
    // tile count), the later ones come from the counter, offset by the grid:
    // the first load leaves without waiting for an atomic, and the segment's
    // arguments reach shared memory while it is in flight.
    const long long t0 = (long long)blockIdx.x;
    int cur_seg = -1;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sh_pending[0] = 0;
        sh_pending[1] = 0;
        sh_failed = 0;
    }
    if (t0 < total) {
        const int s0 = seg_find(t0, 0);
        if (tid == 0) {
            issue(t0, 0, s0);
            sh_pending[0] = 1;
        }
        const int* src = reinterpret_cast<const int*>(&b.segs[s0].a);
        int* dst = reinterpret_cast<int*>(ka);
        for (int w = tid; w < (int)(sizeof(KArgs) / 4); w += CTA) dst[w] = src[w];
        cur_seg = s0;
    }
    __syncthreads();
    long long t = t0;
    unsigned phases = 0u;    // bit i: parity of the next completion of bar[i]
    int buf = 0;
    KC kc;
    if (cur_seg >= 0) kc = make_kc(*ka);
    while (t < total) {
        const int s = seg_of(t, cur_seg);
        const SegDev* sd = &b.segs[s];
        if (tid == 0) {
            // claim the next tile and start its load into the other buffer
            const long long tn = (long long)gridDim.x + (long long)atomicAdd(&b.ctr[CTR_NEXT], 1ull);
            sh_next[buf] = tn;
            if (tn < total) {
                bulk_wait_read();           // the other buffer's last store has left shared memory
                issue(tn, buf ^ 1, seg_of(tn, s));
                sh_pending[buf ^ 1] = 1;
            }
        }
        if (s != cur_seg) {
            // every thread finished the previous tile (barrier at the loop end)
            const int* src = reinterpret_cast<const int*>(&sd->a);
            int* dst = reinterpret_cast<int*>(ka);
            for (int w = tid; w < (int)(sizeof(KArgs) / 4); w += CTA) dst[w] = src[w];
            cur_seg = s;
            __syncthreads();
            kc = make_kc(*ka);
        }
        if (!mbar_wait(&bar[buf], (phases >> buf) & 1u, b.wait_polls)) sh_failed = 1;
        phases ^= 1u << buf;
        const long long lt = t - sd->tile0;
        const int P = sd->polys_per_tile;
        const int np = (int)min((long long)P, sd->a.batch - lt * P);
        const int variant = sd->variant;
        void* st = stage0 + buf * stage_bytes;
        switch (variant) {
#define GB_CASE(F, L)                                                     \
    case variant_id(F, L):                                                \
        if constexpr (fam_i32(F) == I32 && ((SET >> F) & 1) && batch_fits(L, CTA, ELMAX))            \
            tile_transform<F, L, CTA, ELMAX>(st, xbuf, kc, *ka, np);                                       \
        break;
            GB_ALL_VARIANTS(GB_CASE)
#undef GB_CASE
            default: break;
        }
        __syncthreads();
        const long long tnext = sh_next[buf];
        if (sh_failed) break;
        if (tid == 0) {
            sh_pending[buf] = 0;
            fence_proxy_async();
            const long long off = lt * P * (long long)sd->n * sd->elem_bytes;
            bulk_store(static_cast<char*>(sd->a.out) + off, st, (unsigned)(np * sd->n * sd->elem_bytes));
            bulk_commit();
        }
        t = tnext;
        buf ^= 1;
    }
    if (tid == 0) {
        if (sh_failed) {
            atomicMax(&b.ctr[CTR_ERROR], (unsigned long long)BERR_TIMEOUT);
            // let a prefetch that is still in flight land before the CTA leaves
            // (bounded by the full limit whatever b.wait_polls is; bar[buf]'s
            // parity bit was already advanced past the load it waited for)
            for (int i = 0; i < 2; ++i)
                if (sh_pending[i]) mbar_wait(&bar[i], ((phases >> i) & 1u) ^ (i == buf ? 1u : 0u), BATCH_WAIT_POLLS);
        }
        bulk_wait_all();
        __threadfence();
        if (atomicAdd(&b.ctr[CTR_DONE], 1ull) == (unsigned long long)gridDim.x - 1) {
            // last CTA of the launch: rearm the tile counter for the next launch
            b.ctr[CTR_NEXT] = 0;
            b.ctr[CTR_DONE] = 0;
            __threadfence();
        }
    }
}

// Zero-copy form of the persistent kernel, for segments whose buffers are
// page-locked host memory mapped into the device's address space: the same
// tile loop and transform, but each tile moves with cooperative 16-byte loads
// and stores (whole cache lines per warp, which the host-device link carries
// efficiently) instead of bulk copies, with one staging buffer per CTA; the
// CTAs resident on an SM overlap one another's transfers.
template <bool I32, int CTA, int ELMAX, int SET, int OCC = 0>
__global__ void __launch_bounds__(CTA, OCC ? OCC : batch_min_blocks(I32, CTA, ELMAX))
    k_batch_zc(const BatchDev b, int stage_bytes) {
    extern __shared__ __align__(128) unsigned char bsmem[];
    KArgs* ka = reinterpret_cast<KArgs*>(bsmem + 64);
    unsigned char* stage = bsmem + SMEM_HEADER;
    int* xbuf = reinterpret_cast<int*>(bsmem + SMEM_HEADER + stage_bytes);
    __shared__ long long sh_next;
    const int tid = threadIdx.x;
    const long long total = b.total_tiles;
    // segment of tile t, searched from segment `from`: a CTA's tiles come from
    // the counter in increasing order, so its search never goes back
    auto seg_of = [&](long long t, int from) {
        int s = from < 0 ? 0 : from;
        while (s + 1 < b.nsegs && __ldg(&b.segs[s + 1].tile0) <= t) ++s;
        return s;
    };
    if (tid == 0) sh_next = (long long)atomicAdd(&b.ctr[CTR_NEXT], 1ull);
    __syncthreads();
    long long t = sh_next;
    int cur_seg = -1;
    KC kc;
    while (t < total) {
        const int s = seg_of(t, cur_seg);
        const SegDev* sd = &b.segs[s];
        if (s != cur_seg) {
            const int* src = reinterpret_cast<const int*>(&sd->a);
            int* dst = reinterpret_cast<int*>(ka);
            for (int w = tid; w < (int)(sizeof(KArgs) / 4); w += CTA) dst[w] = src[w];
            cur_seg = s;
            __syncthreads();
            kc = make_kc(*ka);
        }
        const long long lt = t - sd->tile0;
        const int P = sd->polys_per_tile;
        const int np = (int)min((long long)P, sd->a.batch - lt * P);
        const long long off = lt * P * (long long)sd->n * sd->elem_bytes;
        const int words = np * sd->n * sd->elem_bytes / 16;
        const uint4* gin = reinterpret_cast<const uint4*>(static_cast<const char*>(sd->a.in) + off);
        uint4* st4 = reinterpret_cast<uint4*>(stage);
        for (int i = tid; i < words; i += CTA) st4[i] = gin[i];
        if (tid == 0) sh_next = (long long)atomicAdd(&b.ctr[CTR_NEXT], 1ull);
        __syncthreads();
        switch (sd->variant) {
#define GB_CASE(F, L)                                                     \
    case variant_id(F, L):                                                \
        if constexpr (fam_i32(F) == I32 && ((SET >> F) & 1) && batch_fits(L, CTA, ELMAX))            \
            tile_transform<F, L, CTA, ELMAX>(stage, xbuf, kc, *ka, np);                                    \
        break;
            GB_ALL_VARIANTS(GB_CASE)
#undef GB_CASE
            default: break;
        }
        __syncthreads();
        uint4* gout = reinterpret_cast<uint4*>(static_cast<char*>(sd->a.out) + off);
        for (int i = tid; i < words; i += CTA) gout[i] = st4[i];
        t = sh_next;
        __syncthreads();   // the stage is drained and sh_next read before the next tile
    }
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&b.ctr[CTR_DONE], 1ull) == (unsigned long long)gridDim.x - 1) {
            b.ctr[CTR_NEXT] = 0;   // last CTA: rearm the tile counter for the next launch
            b.ctr[CTR_DONE] = 0;
            __threadfence();
        }
    }
}

inline bool variant_supported(int fam, int L) {
#define GB_HAS(F, L_) if (fam == F && L == L_) return true;
    GB_ALL_VARIANTS(GB_HAS)
#undef GB_HAS
    return false;
}


// one compiled configuration of the persistent kernel
struct BatchConfig {
    bool i32;
    int elmax;   // log2 coefficients per thread
    int set;     // families covered (bit F)
    const void* fn;
    const void* zfn;   // zero-copy form (k_batch_zc), or nullptr
    int cta;           // threads per CTA
    int occ;           // resident CTAs per SM the registers are budgeted for (0: the default)
};

// the configuration carries a transform of 2^L coefficients
inline bool config_fits(const BatchConfig& c, int L) { return batch_fits(L, c.cta, c.elmax); }

// the persistent launch of a batch part: storage type and arithmetic
// (the reference's lanes or the canonical families) -- 4 parts
__host__ __device__ constexpr int batch_part_of(int fam) { return (fam_i32(fam) ? 1 : 0) | (fam_canon(fam) ? 2 : 0); }
constexpr int BATCH_PARTS = 4;

// Raises a kernel's dynamic shared-memory limit on the current device to at
// least `bytes`, never lowering it: several batches, servers and no-alloc calls
// share one kernel function with different needs, and a lower setting made
// after a higher one would make the earlier user's launches fail.  Serialised
// across host threads (batch.cu).
cudaError_t raise_smem_limit(const void* fn, int bytes);

// the poll limit of tile-load waits for launches enqueued now
// (gbntt_set_wait_limit; BATCH_WAIT_POLLS by default)
unsigned batch_wait_polls();

// the configurations compiled into the library
int batch_configs_i16(const BatchConfig** out);
const void* batch_zc_kernel_i16(int set, int elmax);   // k_batch_zc<int16, 2^elmax coefficients per thread, set>
int batch_configs_i32(const BatchConfig** out);

}  // namespace gbntt
