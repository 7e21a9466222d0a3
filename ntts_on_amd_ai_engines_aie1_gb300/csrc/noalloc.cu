// noalloc.cu -- gbntt_batch_execute_noalloc: the persistent batch kernel run
// without any device allocation.
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
// counters of the (at most two) persistent launches
constexpr size_t NOALLOC_DESC_BYTES = sizeof(SegDev) * GBNTT_NOALLOC_MAX_SEGMENTS;
constexpr size_t NOALLOC_CTR_OFFSET = (NOALLOC_DESC_BYTES + 255) & ~size_t(255);
constexpr size_t NOALLOC_SCRATCH_BYTES = NOALLOC_CTR_OFFSET + 2 * CTR_WORDS * sizeof(unsigned long long);

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

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

    // Descriptors on the stack: [0] int16 part, [1] int32 part.
    SegDev desc[2][GBNTT_NOALLOC_MAX_SEGMENTS];
    int nd[2] = {0, 0}, fam_mask[2] = {0, 0}, Ls[2][GBNTT_NOALLOC_MAX_SEGMENTS];
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
        const int part = fam_i32(fam) ? 1 : 0;
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
    // every call reuses the same scratch: the tile counters must start at zero
    unsigned long long* ctr = reinterpret_cast<unsigned long long*>(scratch + NOALLOC_CTR_OFFSET);
    cudaError_t e = cudaMemsetAsync(ctr, 0, 2 * CTR_WORDS * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return fail(GBNTT_ERR_CUDA, std::string("counter reset: ") + cudaGetErrorString(e));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    size_t desc_off = 0;
    for (int part = 0; part < 2; ++part) {
        if (!nd[part]) continue;
        // the narrowest compiled configuration covering these families and
        // lengths, with the most resident CTAs among those (the choice the
        // autotuner makes on the benchmark batch; the serving loop's rule)
        const BatchConfig* cfgs = nullptr;
        const int ncfg = part ? batch_configs_i32(&cfgs) : batch_configs_i16(&cfgs);
        int maxL = 0;
        for (int i = 0; i < nd[part]; ++i) maxL = Ls[part][i] > maxL ? Ls[part][i] : maxL;
        auto resident = [](const BatchConfig& c) { return c.occ ? c.occ : batch_min_blocks(c.i32, c.cta, c.elmax); };
        const BatchConfig* cfg = nullptr;
        for (int c = 0; c < ncfg; ++c)
            if (cfgs[c].cta == BATCH_CTA && (cfgs[c].set & fam_mask[part]) == fam_mask[part] &&
                config_fits(cfgs[c], maxL) &&
                (!cfg || cfgs[c].elmax < cfg->elmax ||
                 (cfgs[c].elmax == cfg->elmax && resident(cfgs[c]) > resident(*cfg))))
                cfg = &cfgs[c];
        if (!cfg) return fail(GBNTT_ERR_ARG, "no persistent kernel covers these designs");
        // tiles, largest n first
        int order[GBNTT_NOALLOC_MAX_SEGMENTS];
        for (int i = 0; i < nd[part]; ++i) order[i] = i;
        for (int i = 1; i < nd[part]; ++i)
            for (int j = i; j > 0 && Ls[part][order[j]] > Ls[part][order[j - 1]]; --j) {
                const int t = order[j]; order[j] = order[j - 1]; order[j - 1] = t;
            }
        SegDev sorted[GBNTT_NOALLOC_MAX_SEGMENTS];
        long long tiles = 0;
        int stage = 0, xbytes = 0;
        for (int i = 0; i < nd[part]; ++i) {
            SegDev sd = desc[part][order[i]];
            const int L = Ls[part][order[i]];
            const int G = 1 << (L - batch_el(L, cfg->elmax));
            sd.polys_per_tile = BATCH_CTA / G;
            sd.tiles = (sd.a.batch + sd.polys_per_tile - 1) / sd.polys_per_tile;
            sd.tile0 = tiles;
            tiles += sd.tiles;
            stage = stage > batch_stage_bytes(BATCH_CTA, L, sd.elem_bytes, cfg->elmax)
                        ? stage : batch_stage_bytes(BATCH_CTA, L, sd.elem_bytes, cfg->elmax);
            xbytes = xbytes > batch_xbuf_bytes(BATCH_CTA, L, cfg->elmax) ? xbytes
                                                                          : batch_xbuf_bytes(BATCH_CTA, L, cfg->elmax);
            sorted[i] = sd;
        }
        stage = (stage + 127) & ~127;
        const int smem = SMEM_HEADER + 2 * stage + xbytes;
        SegDev* d_desc = reinterpret_cast<SegDev*>(scratch) + desc_off;
        e = cudaMemcpyAsync(d_desc, sorted, sizeof(SegDev) * nd[part], cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return fail(GBNTT_ERR_CUDA, std::string("descriptor copy: ") + cudaGetErrorString(e));
        desc_off += nd[part];
        e = cudaFuncSetAttribute(cfg->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        int per_sm = 0;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cfg->fn, BATCH_CTA, smem);
        if (e != cudaSuccess || per_sm < 1)
            return fail(GBNTT_ERR_CUDA, std::string("kernel configuration: ") + cudaGetErrorString(e));
        BatchDev bd;
        bd.segs = d_desc;
        bd.nsegs = nd[part];
        bd.total_tiles = tiles;
        bd.ctr = ctr + CTR_WORDS * part;
        int sb = stage;
        void* args[] = {&bd, &sb};
        const long long grid = (long long)per_sm * sms < tiles ? (long long)per_sm * sms : tiles;
        e = cudaLaunchKernel(cfg->fn, dim3((unsigned)grid), dim3(BATCH_CTA), args, smem, s);
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
