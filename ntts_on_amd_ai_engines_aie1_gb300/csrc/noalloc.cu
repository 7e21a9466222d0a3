// noalloc.cu -- gbntt_batch_execute_noalloc: the persistent batch kernel run
// without any device allocation, and gbntt_noalloc_status.
//
// gbntt_batch_create allocates device memory for the tile descriptors and the
// tile counters of a batch.  Some callers cannot allocate device memory at the
// point where they transform: a host application that hands the library only
// buffers it owns (its own allocator or memory pool, a fixed arena sized at
// start-up), a latency-bound serving loop where a cudaMalloc/cudaFree would
// synchronise the device in the middle of a request, or a plugin that must
// leave the device's free memory untouched.  For them this entry point keeps
// the descriptors and counters in one file-scope __device__ array of fixed size
// (NOALLOC_SCRATCH_BYTES below), present on every GPU that loads the library
// until the process exits.  The plans' tables are allocated when the plans are
// created; the call itself allocates nothing.
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/gb300_ntt.h"
#include "batch_kernel.cuh"
#include "plan_internal.h"

using namespace gbntt;

namespace {

// descriptors of up to GBNTT_NOALLOC_MAX_SEGMENTS segments, then the tile
// counters of the (at most BATCH_PARTS) persistent launches
constexpr size_t NOALLOC_DESC_BYTES = sizeof(SegDev) * GBNTT_NOALLOC_MAX_SEGMENTS;
constexpr size_t NOALLOC_CTR_OFFSET = (NOALLOC_DESC_BYTES + 255) & ~size_t(255);
constexpr size_t NOALLOC_CTR_BYTES = BATCH_PARTS * CTR_WORDS * sizeof(unsigned long long);
constexpr size_t NOALLOC_SCRATCH_BYTES = NOALLOC_CTR_OFFSET + NOALLOC_CTR_BYTES;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// The descriptors travel as a kernel parameter (copied by the launch itself)
// and a one-CTA kernel writes them into the array: no host staging buffer, no
// copy from pageable memory.
struct DescBlock {
    SegDev d[GBNTT_NOALLOC_MAX_SEGMENTS];
    int count;
};
static_assert(sizeof(DescBlock) < 30000, "the descriptor block must fit the kernel parameter space");

__global__ void k_noalloc_descs(const __grid_constant__ DescBlock blk, SegDev* dst) {
    const int words = blk.count * (int)(sizeof(SegDev) / 4);
    const int* src = reinterpret_cast<const int*>(blk.d);
    int* out = reinterpret_cast<int*>(dst);
    for (int w = threadIdx.x; w < words; w += blockDim.x) out[w] = src[w];
}
static_assert(sizeof(SegDev) % 4 == 0, "descriptors are copied in words");

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[MAX_DEVICES] = {};   // device address of g_noalloc_scratch, per device

int fail(int code, const std::string& msg) { return gbntt_internal_fail(code, msg); }

// Once per device, with that device current: the device address of the
// array.  (In host code g_noalloc_scratch names a host-side stand-in, not
// device memory, so it must never be passed to a kernel directly.)
int scratch_for_current_device(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(GBNTT_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES) return fail(GBNTT_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(GBNTT_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[dev];
    return GBNTT_OK;
}

// one persistent launch of the call, fully prepared before anything is enqueued
struct PartLaunch {
    const BatchConfig* cfg = nullptr;
    int first = 0, count = 0;        // its descriptors in the block
    long long tiles = 0;
    int stage = 0, smem = 0;
    long long grid = 0;
};

}  // namespace

extern "C" int gbntt_batch_execute_noalloc(const gbntt_segment* segs, uint32_t nsegs, void* stream) {
    if (nsegs == 0) return GBNTT_OK;
    if (!segs) return fail(GBNTT_ERR_ARG, "segments pointer is null");
    if (nsegs > GBNTT_NOALLOC_MAX_SEGMENTS)
        return fail(GBNTT_ERR_ARG, "gbntt_batch_execute_noalloc takes at most " +
                                       std::to_string(GBNTT_NOALLOC_MAX_SEGMENTS) + " segments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != GBNTT_OK) return rc;

    // 1. validate and sort every segment into its part (storage type and
    //    arithmetic); segments without a persistent form run as plan launches
    SegDev desc[BATCH_PARTS][GBNTT_NOALLOC_MAX_SEGMENTS];
    int nd[BATCH_PARTS] = {}, fam_mask[BATCH_PARTS] = {}, Ls[BATCH_PARTS][GBNTT_NOALLOC_MAX_SEGMENTS];
    bool batched[GBNTT_NOALLOC_MAX_SEGMENTS] = {};
    for (uint32_t k = 0; k < nsegs; ++k) {
        const gbntt_segment& u = segs[k];
        if (!u.plan) return fail(GBNTT_ERR_ARG, "segment without a plan");
        if (u.count == 0) continue;
        if (!u.d_in || !u.d_out || ((reinterpret_cast<uintptr_t>(u.d_in) | reinterpret_cast<uintptr_t>(u.d_out)) & 15))
            return fail(GBNTT_ERR_ARG, "device buffers must be non-null and 16-byte aligned");
        int fam, L, eb;
        KArgs a;
        gbntt_internal_plan_args(u.plan, &fam, &L, &eb, &a);
        if (fam < 0 || !variant_supported(fam, L) || u.d_in == u.d_out) continue;   // runs as a plan launch
        const int part = batch_part_of(fam);
        SegDev& sd = desc[part][nd[part]];
        std::memset(&sd, 0, sizeof(sd));
        sd.a = a;
        sd.a.in = u.d_in;
        sd.a.out = u.d_out;
        sd.a.batch = (long long)u.count;
        sd.n = 1 << L;
        sd.elem_bytes = eb;
        sd.variant = variant_id(fam, L);
        Ls[part][nd[part]] = L;
        fam_mask[part] |= 1 << fam;
        ++nd[part];
        batched[k] = true;
    }

    // 2. choose every part's configuration, order its tiles and size its
    //    launch; nothing is enqueued until all parts are ready
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    DescBlock blk;
    std::memset(&blk, 0, sizeof(blk));
    PartLaunch pl[BATCH_PARTS];
    for (int part = 0; part < BATCH_PARTS; ++part) {
        if (!nd[part]) continue;
        PartLaunch& P = pl[part];
        // the narrowest compiled configuration covering these families and
        // lengths, with the most resident CTAs among those (the serving loop's rule)
        const BatchConfig* cfgs = nullptr;
        const int ncfg = (part & 1) ? batch_configs_i32(&cfgs) : batch_configs_i16(&cfgs);
        int maxL = 0;
        for (int i = 0; i < nd[part]; ++i) maxL = Ls[part][i] > maxL ? Ls[part][i] : maxL;
        auto resident = [](const BatchConfig& c) { return c.occ ? c.occ : batch_min_blocks(c.i32, c.cta, c.elmax); };
        for (int c = 0; c < ncfg; ++c)
            if (cfgs[c].cta == BATCH_CTA && (cfgs[c].set & fam_mask[part]) == fam_mask[part] &&
                config_fits(cfgs[c], maxL) &&
                (!P.cfg || cfgs[c].elmax < P.cfg->elmax ||
                 (cfgs[c].elmax == P.cfg->elmax && resident(cfgs[c]) > resident(*P.cfg))))
                P.cfg = &cfgs[c];
        if (!P.cfg) return fail(GBNTT_ERR_ARG, "no persistent kernel covers these designs");
        // tiles, largest n first
        int order[GBNTT_NOALLOC_MAX_SEGMENTS];
        for (int i = 0; i < nd[part]; ++i) order[i] = i;
        for (int i = 1; i < nd[part]; ++i)
            for (int j = i; j > 0 && Ls[part][order[j]] > Ls[part][order[j - 1]]; --j) {
                const int t = order[j]; order[j] = order[j - 1]; order[j - 1] = t;
            }
        P.first = blk.count;
        P.count = nd[part];
        int xbytes = 0;
        for (int i = 0; i < nd[part]; ++i) {
            SegDev sd = desc[part][order[i]];
            const int L = Ls[part][order[i]];
            const int G = 1 << (L - batch_el(L, P.cfg->elmax));
            sd.polys_per_tile = BATCH_CTA / G;
            sd.tiles = (sd.a.batch + sd.polys_per_tile - 1) / sd.polys_per_tile;
            sd.tile0 = P.tiles;
            P.tiles += sd.tiles;
            const int st = batch_stage_bytes(BATCH_CTA, L, sd.elem_bytes, P.cfg->elmax);
            const int xb = batch_xbuf_bytes(BATCH_CTA, L, P.cfg->elmax);
            P.stage = P.stage > st ? P.stage : st;
            xbytes = xbytes > xb ? xbytes : xb;
            blk.d[blk.count++] = sd;
        }
        P.stage = (P.stage + 127) & ~127;
        P.smem = SMEM_HEADER + 2 * P.stage + xbytes;
        cudaError_t e = raise_smem_limit(P.cfg->fn, P.smem);
        int per_sm = 0;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, P.cfg->fn, BATCH_CTA, P.smem);
        if (e != cudaSuccess || per_sm < 1)
            return fail(GBNTT_ERR_CUDA, std::string("kernel configuration: ") + cudaGetErrorString(e));
        P.grid = (long long)per_sm * sms < P.tiles ? (long long)per_sm * sms : P.tiles;
    }

    // 3. enqueue: descriptors, counter reset, the persistent launches, then
    //    the plan launches
    SegDev* d_desc = reinterpret_cast<SegDev*>(scratch);
    unsigned long long* ctr = reinterpret_cast<unsigned long long*>(scratch + NOALLOC_CTR_OFFSET);
    cudaError_t e = cudaSuccess;
    if (blk.count) {
        k_noalloc_descs<<<1, 256, 0, s>>>(blk, d_desc);
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail(GBNTT_ERR_CUDA, std::string("descriptors: ") + cudaGetErrorString(e));
        gbntt_internal_count_launch();
        // every call reuses the same counters: the tile counters (CTR_NEXT,
        // CTR_DONE of each part) start at zero; the error words are kept
        // until gbntt_noalloc_status reads them
        e = cudaMemset2DAsync(ctr, CTR_WORDS * sizeof(unsigned long long), 0, 2 * sizeof(unsigned long long),
                              BATCH_PARTS, s);
        if (e != cudaSuccess) return fail(GBNTT_ERR_CUDA, std::string("counter reset: ") + cudaGetErrorString(e));
    }
    for (int part = 0; part < BATCH_PARTS; ++part) {
        const PartLaunch& P = pl[part];
        if (!P.count) continue;
        BatchDev bd;
        bd.segs = d_desc + P.first;
        bd.nsegs = P.count;
        bd.total_tiles = P.tiles;
        bd.ctr = ctr + CTR_WORDS * part;
        bd.wait_polls = batch_wait_polls();
        int sb = P.stage;
        void* args[] = {&bd, &sb};
        e = cudaLaunchKernel(P.cfg->fn, dim3((unsigned)P.grid), dim3(BATCH_CTA), args, P.smem, s);
        if (e != cudaSuccess) return fail(GBNTT_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
        gbntt_internal_count_launch();
    }
    for (uint32_t k = 0; k < nsegs; ++k) {
        if (batched[k] || segs[k].count == 0) continue;
        rc = gbntt_execute(segs[k].plan, segs[k].d_in, segs[k].d_out, segs[k].count, stream);
        if (rc != GBNTT_OK) return rc;
    }
    return GBNTT_OK;
}

extern "C" int gbntt_noalloc_status(void) {
    unsigned char* scratch = nullptr;
    const int rc = scratch_for_current_device(&scratch);
    if (rc != GBNTT_OK) return rc;
    unsigned long long* ctr = reinterpret_cast<unsigned long long*>(scratch + NOALLOC_CTR_OFFSET);
    unsigned long long w[BATCH_PARTS * CTR_WORDS];
    cudaError_t e = cudaMemcpy(w, ctr, sizeof(w), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(GBNTT_ERR_CUDA, std::string("status read: ") + cudaGetErrorString(e));
    bool timed_out = false;
    for (int p = 0; p < BATCH_PARTS; ++p) timed_out |= w[CTR_WORDS * p + CTR_ERROR] != 0;
    if (!timed_out) return GBNTT_OK;
    for (int p = 0; p < BATCH_PARTS; ++p) {
        e = cudaMemset(ctr + CTR_WORDS * p + CTR_ERROR, 0, sizeof(unsigned long long));
        if (e != cudaSuccess) return fail(GBNTT_ERR_CUDA, std::string("status reset: ") + cudaGetErrorString(e));
    }
    return fail(GBNTT_ERR_TIMEOUT, "a tile load of a no-alloc launch did not arrive within the wait limit");
}
