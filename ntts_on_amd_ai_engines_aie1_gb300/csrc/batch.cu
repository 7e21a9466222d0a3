// batch.cu -- persistent batched launches (gbntt_batch_* in include/gb300_ntt.h):
// segment descriptors, tile order, configuration autotuning, graph replay.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gb300_ntt.h"
#include "batch_kernel.cuh"
#include "plan_internal.h"

using namespace gbntt;


using namespace gbntt;

struct gbntt_batch {
    struct Layout {                     // one configuration of one persistent launch
        BatchConfig cfg{};
        std::vector<SegDev> segs;
        SegDev* d_segs = nullptr;
        std::vector<SegDev> live;       // zero-copy layout: the descriptors d_segs holds now
        long long total_tiles = 0;
        int stage_bytes = 0, smem = 0, grid = 0;
        float ms = -1.f;                // autotuner timing
    };
    struct Pending {                    // a batched segment before the layouts are built
        int k, fam, L, eb;
        KArgs a;
    };
    struct Part {                       // the int16 or the int32 segments
        bool i32 = false;
        int fam_mask = 0;
        std::vector<Pending> pending;
        std::vector<Layout> layouts;    // candidate configurations
        int chosen = 0;
        std::vector<int> user_index;    // caller's segment of each SegDev
        Layout zlay;                    // zero-copy launch (k_batch_zc), when a configuration has one
    };
    Part parts[BATCH_PARTS];            // one persistent launch per storage type and arithmetic
    int nparts = 0;
    std::vector<int> part_of;           // segment -> part (or -1: separate per-plan launch)
    std::vector<int> index_in_part;
    std::vector<gbntt_segment> user;    // the caller's segments
    unsigned long long* d_ctr = nullptr;   // CTR_WORDS per part; then CTR_WORDS per part for zero copy
                                           // (BATCH_PARTS each)
    cudaGraphExec_t graph = nullptr;
};

namespace gbntt {

namespace {
std::atomic<unsigned> g_wait_polls{BATCH_WAIT_POLLS};
}

unsigned batch_wait_polls() { return g_wait_polls.load(std::memory_order_relaxed); }

cudaError_t raise_smem_limit(const void* fn, int bytes) {
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    cudaFuncAttributes at;
    cudaError_t e = cudaFuncGetAttributes(&at, fn);
    if (e != cudaSuccess) return e;
    if (at.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

}  // namespace gbntt

namespace {

int batch_fail(int code, const std::string& msg) { return gbntt_internal_fail(code, msg); }

int launch_layout(gbntt_batch* b, int pi, const gbntt_batch::Layout& lay, cudaStream_t s) {
    if (lay.total_tiles == 0) return GBNTT_OK;
    BatchDev bd;
    bd.segs = lay.d_segs;
    bd.nsegs = (int)lay.segs.size();
    bd.total_tiles = lay.total_tiles;
    bd.ctr = b->d_ctr + CTR_WORDS * pi;
    bd.wait_polls = batch_wait_polls();
    int sb = lay.stage_bytes;
    void* args[] = {&bd, &sb};
    cudaError_t e = cudaLaunchKernel(lay.cfg.fn, dim3(lay.grid), dim3(lay.cfg.cta), args, lay.smem, s);
    if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, std::string("batch launch: ") + cudaGetErrorString(e));
    gbntt_internal_count_launch();
    return GBNTT_OK;
}

int launch_batch(gbntt_batch* b, cudaStream_t s) {
    for (int i = 0; i < b->nparts; ++i) {
        auto& p = b->parts[i];
        const int rc = launch_layout(b, i, p.layouts[p.chosen], s);
        if (rc != GBNTT_OK) return rc;
    }
    for (size_t k = 0; k < b->user.size(); ++k) {
        if (b->part_of[k] >= 0) continue;
        const gbntt_segment& u = b->user[k];
        const int rc = gbntt_execute(u.plan, u.d_in, u.d_out, u.count, s);
        if (rc != GBNTT_OK) return rc;
    }
    return GBNTT_OK;
}

// Times every candidate configuration of every part on the batch itself (the
// outputs it writes are the batch's own results) and keeps the fastest.
// A batch whose inputs and outputs fit in L2 would be timed from L2 if its
// launches ran back to back, which is not how it meets its data in use: each
// of its timed launches then follows a write of a buffer twice the L2 size.
// (On a ragged radix-8 batch of 13 MB, back-to-back timing chose 32
// coefficients per thread, 18.8 against 20.2 us; from HBM the choice it
// missed runs 27.9 against 35.3 us.)
int autotune(gbntt_batch* b) {
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
        return batch_fail(GBNTT_ERR_CUDA, "autotune stream");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    size_t footprint = 0;
    for (const auto& u : b->user) {
        int64_t n = 0, eb = 0;
        gbntt_plan_query(u.plan, GBNTT_Q_N, &n);
        gbntt_plan_query(u.plan, GBNTT_Q_ELEM_BYTES, &eb);
        footprint += 2 * (size_t)u.count * (size_t)n * (size_t)eb;
    }
    int dev = 0, l2 = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
    void* flush = nullptr;
    const size_t flush_bytes = 2 * (size_t)l2;
    if (l2 > 0 && footprint < (size_t)l2 && cudaMalloc(&flush, flush_bytes) != cudaSuccess) {
        cudaGetLastError();   // no room: time back to back
        flush = nullptr;
    }
    int rc = GBNTT_OK;
    for (int i = 0; i < b->nparts && rc == GBNTT_OK; ++i) {
        auto& p = b->parts[i];
        if (p.layouts.size() < 2) continue;
        for (size_t c = 0; c < p.layouts.size() && rc == GBNTT_OK; ++c)
            for (int w = 0; w < 2 && rc == GBNTT_OK; ++w) rc = launch_layout(b, i, p.layouts[c], s);
        // five interleaved rounds, best round per configuration (clock drift
        // hits all alike; configurations 3 % apart were ranked inconsistently
        // with three)
        for (int round = 0; round < 5 && rc == GBNTT_OK; ++round) {
            if (flush) {
                // every configuration three times, each launch after the fill
                // and timed alone, the whole round enqueued before one wait:
                // the launches meet the GPU as timed steps do (the next one
                // queued while the fill runs), not after an idle gap
                const size_t nl = p.layouts.size() * 3;
                std::vector<cudaEvent_t> ev(2 * nl);
                for (auto& x : ev) cudaEventCreate(&x);
                for (size_t c = 0; c < p.layouts.size() && rc == GBNTT_OK; ++c)
                    for (int w = 0; w < 3 && rc == GBNTT_OK; ++w) {
                        cudaMemsetAsync(flush, w, flush_bytes, s);
                        cudaEventRecord(ev[2 * (3 * c + w)], s);
                        rc = launch_layout(b, i, p.layouts[c], s);
                        cudaEventRecord(ev[2 * (3 * c + w) + 1], s);
                    }
                if (rc == GBNTT_OK && cudaStreamSynchronize(s) != cudaSuccess)
                    rc = batch_fail(GBNTT_ERR_CUDA, "autotune timing");
                for (size_t c = 0; c < p.layouts.size() && rc == GBNTT_OK; ++c) {
                    float ms = 0.f;
                    for (int w = 0; w < 3; ++w) {
                        float one = 0.f;
                        cudaEventElapsedTime(&one, ev[2 * (3 * c + w)], ev[2 * (3 * c + w) + 1]);
                        ms += one / 3.f;
                    }
                    if (p.layouts[c].ms < 0.f || ms < p.layouts[c].ms) p.layouts[c].ms = ms;
                }
                for (auto& x : ev) cudaEventDestroy(x);
                continue;
            }
            // inputs larger than L2: five launches back to back
            for (size_t c = 0; c < p.layouts.size() && rc == GBNTT_OK; ++c) {
                float ms = 0.f;
                cudaEventRecord(e0, s);
                for (int w = 0; w < 5 && rc == GBNTT_OK; ++w) rc = launch_layout(b, i, p.layouts[c], s);
                cudaEventRecord(e1, s);
                if (cudaEventSynchronize(e1) != cudaSuccess) rc = batch_fail(GBNTT_ERR_CUDA, "autotune timing");
                cudaEventElapsedTime(&ms, e0, e1);
                ms /= 5.f;
                if (p.layouts[c].ms < 0.f || ms < p.layouts[c].ms) p.layouts[c].ms = ms;
            }
        }
        size_t best = 0;
        for (size_t c = 1; c < p.layouts.size(); ++c)
            if (p.layouts[c].ms >= 0.f && p.layouts[c].ms < p.layouts[best].ms) best = c;
        // GBNTT_TUNE_FORCE="<log2 coefficients per thread>,<CTAs per SM>" pins the
        // choice (the timing launches still run), e.g. to profile the kernel a
        // normal run picks while a profiler slows every launch down
        if (const char* f = std::getenv("GBNTT_TUNE_FORCE")) {
            int el = -1, occ = -1;
            if (std::sscanf(f, "%d,%d", &el, &occ) == 2)
                for (size_t c = 0; c < p.layouts.size(); ++c)
                    if (p.layouts[c].cfg.elmax == el && p.layouts[c].cfg.occ == occ) {
                        best = c;
                        break;
                    }
        }
        p.chosen = (int)best;
        if (const char* log = std::getenv("GBNTT_TUNE_LOG"); log && *log == '1')
            for (size_t c = 0; c < p.layouts.size(); ++c)
                std::fprintf(stderr, "gbntt autotune: %s part, %d coefficients/thread, %d threads/CTA, %d CTAs/SM, "
                             "families 0x%x: %.2f us%s\n", p.i32 ? "int32" : "int16", 1 << p.layouts[c].cfg.elmax,
                             p.layouts[c].cfg.cta, p.layouts[c].cfg.occ, p.layouts[c].cfg.set,
                             1e3 * p.layouts[c].ms, c == best ? "  <- chosen" : "");
    }
    if (flush) cudaFree(flush);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    return rc;
}

// zero-copy scratch of one plan (gbntt_execute_host on mapped host buffers)
struct ZcPlanState {
    bool tried = false, usable = false;
    BatchConfig cfg{};
    int stage = 0, smem = 0, grid_cap = 0;
    SegDev* d_seg = nullptr;
    unsigned long long* d_ctr = nullptr;
    SegDev live{};              // the descriptor d_seg holds (valid when has_live)
    bool has_live = false;
};

}  // namespace

int gbntt_internal_zc_plan(void** state, const gbntt_plan* p, const void* m_in, void* m_out, uint64_t count,
                           cudaStream_t s) {
    if (!count) return GBNTT_OK;
    int fam, L, eb;
    KArgs a;
    gbntt_internal_plan_args(p, &fam, &L, &eb, &a);
    if (fam < 0 || !variant_supported(fam, L)) return GBNTT_ERR_KIND;
    if (!*state) *state = new ZcPlanState();
    ZcPlanState& st = *static_cast<ZcPlanState*>(*state);
    if (!st.tried) {
        st.tried = true;
        const bool i32 = fam_i32(fam);
        const BatchConfig* cfgs = nullptr;
        const int ncfg = i32 ? batch_configs_i32(&cfgs) : batch_configs_i16(&cfgs);
        const BatchConfig* cfg = nullptr;   // the narrowest covering configuration with a zero-copy kernel
        for (int c = 0; c < ncfg; ++c)
            if (cfgs[c].zfn && ((cfgs[c].set >> fam) & 1) && config_fits(cfgs[c], L) &&
                (!cfg || cfgs[c].elmax < cfg->elmax))
                cfg = &cfgs[c];
        if (!cfg) return GBNTT_ERR_KIND;
        st.cfg = *cfg;
        st.stage = (batch_stage_bytes(cfg->cta, L, eb, cfg->elmax) + 127) & ~127;
        st.smem = SMEM_HEADER + st.stage + batch_xbuf_bytes(cfg->cta, L, cfg->elmax);
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaError_t e = raise_smem_limit(cfg->zfn, st.smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cfg->zfn, cfg->cta, st.smem);
        if (e != cudaSuccess || per_sm < 1)
            return batch_fail(GBNTT_ERR_CUDA, std::string("zero-copy kernel configuration: ") + cudaGetErrorString(e));
        st.grid_cap = std::min(per_sm, 2) * sms;   // two CTAs per SM, as for batches
        e = cudaMalloc(&st.d_seg, sizeof(SegDev));
        if (e == cudaSuccess) e = cudaMalloc(&st.d_ctr, sizeof(unsigned long long) * CTR_WORDS);
        if (e == cudaSuccess) e = cudaMemset(st.d_ctr, 0, sizeof(unsigned long long) * CTR_WORDS);
        if (e != cudaSuccess) return batch_fail(GBNTT_ERR_NOMEM, "zero-copy scratch allocation failed");
        st.usable = true;
    }
    if (!st.usable) return GBNTT_ERR_KIND;
    SegDev sd;
    std::memset(&sd, 0, sizeof(sd));
    sd.a = a;
    sd.a.in = m_in;
    sd.a.out = m_out;
    sd.a.batch = (long long)count;
    sd.n = 1 << L;
    sd.elem_bytes = eb;
    sd.variant = variant_id(fam, L);
    sd.polys_per_tile = st.cfg.cta >> (L - batch_el(L, st.cfg.elmax));
    sd.tiles = ((long long)count + sd.polys_per_tile - 1) / sd.polys_per_tile;
    // repeated calls on the same buffers reuse the descriptor already on the device
    cudaError_t e = cudaSuccess;
    if (!st.has_live || std::memcmp(&st.live, &sd, sizeof(SegDev)) != 0) {
        st.has_live = false;
        e = cudaMemcpyAsync(st.d_seg, &sd, sizeof(SegDev), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, std::string("descriptor: ") + cudaGetErrorString(e));
        st.live = sd;
        st.has_live = true;
    }
    BatchDev bd;
    bd.segs = st.d_seg;
    bd.nsegs = 1;
    bd.total_tiles = sd.tiles;
    bd.ctr = st.d_ctr;
    bd.wait_polls = BATCH_WAIT_POLLS;   // the zero-copy kernel has no bounded waits
    int sb = st.stage;
    void* args[] = {&bd, &sb};
    const unsigned grid = (unsigned)std::min<long long>(st.grid_cap, sd.tiles);
    e = cudaLaunchKernel(st.cfg.zfn, dim3(grid), dim3(st.cfg.cta), args, st.smem, s);
    if (e != cudaSuccess) {
        st.has_live = false;
        return batch_fail(GBNTT_ERR_CUDA, std::string("zero-copy launch: ") + cudaGetErrorString(e));
    }
    gbntt_internal_count_launch();
    return GBNTT_OK;
}

void gbntt_internal_zc_free(void* state) {
    ZcPlanState* st = static_cast<ZcPlanState*>(state);
    if (!st) return;
    if (st->d_seg) cudaFree(st->d_seg);
    if (st->d_ctr) cudaFree(st->d_ctr);
    delete st;
}

extern "C" {

int gbntt_set_wait_limit(uint32_t polls) {
    static_assert(GBNTT_WAIT_POLLS_DEFAULT == BATCH_WAIT_POLLS, "one default poll limit");
    g_wait_polls.store(polls, std::memory_order_relaxed);
    return GBNTT_OK;
}

int gbntt_batch_create(gbntt_batch** out, const gbntt_segment* segs, uint32_t nsegs, uint32_t flags) {
    if (!out || (!segs && nsegs)) return batch_fail(GBNTT_ERR_ARG, "null argument");
    *out = nullptr;
    gbntt_batch* b = new gbntt_batch();
    b->user.assign(segs, segs + nsegs);
    b->part_of.assign(nsegs, -1);
    b->index_in_part.assign(nsegs, -1);
    // order: largest n first (longest tiles first), then the caller's order
    std::vector<int> order(nsegs);
    for (uint32_t k = 0; k < nsegs; ++k) order[k] = (int)k;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return gbntt_internal_plan_L(segs[x].plan) > gbntt_internal_plan_L(segs[y].plan);
    });
    int pid[BATCH_PARTS] = {-1, -1, -1, -1};
    for (int k : order) {
        const gbntt_segment& u = segs[k];
        if (!u.plan) { delete b; return batch_fail(GBNTT_ERR_ARG, "segment without a plan"); }
        if (u.count && (!u.d_in || !u.d_out)) { delete b; return batch_fail(GBNTT_ERR_ARG, "segment without buffers"); }
        if ((reinterpret_cast<uintptr_t>(u.d_in) | reinterpret_cast<uintptr_t>(u.d_out)) & 15) {
            delete b;
            return batch_fail(GBNTT_ERR_ARG, "device buffers must be 16-byte aligned");
        }
        int fam, L, eb;
        KArgs a;
        gbntt_internal_plan_args(u.plan, &fam, &L, &eb, &a);
        if (fam < 0 || !variant_supported(fam, L) || u.d_in == u.d_out || u.count == 0) continue;   // per-plan launch
        const bool i32 = fam_i32(fam);
        int& id = pid[batch_part_of(fam)];
        if (id < 0) {
            id = b->nparts++;
            b->parts[id].i32 = i32;
        }
        auto& part = b->parts[id];
        b->part_of[k] = id;
        b->index_in_part[k] = (int)part.user_index.size();
        part.user_index.push_back(k);
        part.fam_mask |= 1 << fam;
        part.pending.push_back({k, fam, L, eb, a});
    }
    // candidate configurations of each part: those whose family set covers it
    // and whose CTAs hold its longest transform
    for (int i = 0; i < b->nparts; ++i) {
        auto& part = b->parts[i];
        int maxL = 0;
        for (const auto& pe : part.pending) maxL = std::max(maxL, pe.L);
        const BatchConfig* cfgs = nullptr;
        const int ncfg = part.i32 ? batch_configs_i32(&cfgs) : batch_configs_i16(&cfgs);
        auto covers = [&](const BatchConfig& c) {
            return (c.set & part.fam_mask) == part.fam_mask && config_fits(c, maxL);
        };
        for (int c = 0; c < ncfg; ++c)
            if (covers(cfgs[c])) {
                gbntt_batch::Layout lay;
                lay.cfg = cfgs[c];
                part.layouts.push_back(lay);
            }
        if (part.layouts.empty()) {
            gbntt_batch_destroy(b);
            return batch_fail(GBNTT_ERR_ARG, "no persistent kernel covers these designs");
        }
        if (flags & GBNTT_BATCH_NO_TUNE) part.layouts.resize(1);   // the first (widest, most specific) one
        // zero copy: the narrowest covering configuration
        for (int c = 0; c < ncfg; ++c)
            if (cfgs[c].zfn && covers(cfgs[c]) && (!part.zlay.cfg.zfn || cfgs[c].elmax < part.zlay.cfg.elmax))
                part.zlay.cfg = cfgs[c];
    }
    for (int i = 0; i < b->nparts; ++i) {
      auto& part = b->parts[i];
      for (const auto& pe : part.pending) {
        const gbntt_segment& u = segs[pe.k];
        const int fam = pe.fam, L = pe.L, eb = pe.eb;
        const KArgs& a = pe.a;
        std::vector<gbntt_batch::Layout*> lays;
        for (auto& lay : part.layouts) lays.push_back(&lay);
        if (part.zlay.cfg.zfn) lays.push_back(&part.zlay);
        for (gbntt_batch::Layout* lp : lays) {
            gbntt_batch::Layout& lay = *lp;
            const int elmax = lay.cfg.elmax;
            SegDev sd;
            std::memset(&sd, 0, sizeof(sd));
            sd.a = a;
            sd.a.in = u.d_in;
            sd.a.out = u.d_out;
            sd.a.batch = (long long)u.count;
            sd.n = 1 << L;
            sd.elem_bytes = eb;
            sd.variant = variant_id(fam, L);
            const int G = 1 << (L - batch_el(L, elmax));
            sd.polys_per_tile = lay.cfg.cta / G;
            sd.tiles = ((long long)u.count + sd.polys_per_tile - 1) / sd.polys_per_tile;
            sd.tile0 = lay.total_tiles;
            lay.total_tiles += sd.tiles;
            lay.stage_bytes = std::max(lay.stage_bytes, batch_stage_bytes(lay.cfg.cta, L, eb, elmax));
            lay.smem = std::max(lay.smem, batch_xbuf_bytes(lay.cfg.cta, L, elmax));
            lay.segs.push_back(sd);
        }
      }
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (int i = 0; i < b->nparts; ++i) {
        std::vector<gbntt_batch::Layout*> lays;
        for (auto& lay : b->parts[i].layouts) lays.push_back(&lay);
        if (b->parts[i].zlay.cfg.zfn) lays.push_back(&b->parts[i].zlay);
        for (gbntt_batch::Layout* lp : lays) {
            gbntt_batch::Layout& lay = *lp;
            const bool zc = (lp == &b->parts[i].zlay);     // one staging buffer instead of two
            lay.stage_bytes = (lay.stage_bytes + 127) & ~127;
            lay.smem = SMEM_HEADER + (zc ? 1 : 2) * lay.stage_bytes + lay.smem;
            const void* fn = zc ? lay.cfg.zfn : lay.cfg.fn;
            cudaError_t e = raise_smem_limit(fn, lay.smem);
            int per_sm = 0;
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, lay.cfg.cta, lay.smem);
            if (e != cudaSuccess || per_sm < 1) {
                gbntt_batch_destroy(b);
                return batch_fail(GBNTT_ERR_CUDA, std::string("batch kernel configuration: ") + cudaGetErrorString(e));
            }
            // Zero copy: two CTAs per SM.  The link, not the SMs, is the limit;
            // fewer tiles in flight shorten the read-only start and the
            // write-only end of the launch (benchmark batch end to end: 1, 2, 3,
            // 4 CTAs/SM -> 100, 106, 103, 100 M NTT/s on one box).
            const int resident = zc ? std::min(per_sm, 2) : per_sm;
            lay.grid = (int)std::min<long long>((long long)resident * sms, lay.total_tiles);
            e = cudaMalloc(&lay.d_segs, sizeof(SegDev) * lay.segs.size());
            if (e == cudaSuccess)
                e = cudaMemcpy(lay.d_segs, lay.segs.data(), sizeof(SegDev) * lay.segs.size(), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) {
                gbntt_batch_destroy(b);
                return batch_fail(GBNTT_ERR_NOMEM, "batch descriptor allocation failed");
            }
        }
    }
    cudaError_t e = cudaMalloc(&b->d_ctr, sizeof(unsigned long long) * CTR_WORDS * 2 * BATCH_PARTS);
    if (e == cudaSuccess) e = cudaMemset(b->d_ctr, 0, sizeof(unsigned long long) * CTR_WORDS * 2 * BATCH_PARTS);
    if (e != cudaSuccess) {
        gbntt_batch_destroy(b);
        return batch_fail(GBNTT_ERR_NOMEM, "batch scratch allocation failed");
    }
    if (!(flags & GBNTT_BATCH_NO_TUNE)) {
        const int rc = autotune(b);
        if (rc != GBNTT_OK) {
            gbntt_batch_destroy(b);
            return rc;
        }
    }
    *out = b;
    return GBNTT_OK;
}

int gbntt_batch_execute(gbntt_batch* b, void* stream) {
    if (!b) return batch_fail(GBNTT_ERR_ARG, "batch is null");
    return launch_batch(b, static_cast<cudaStream_t>(stream));
}

int gbntt_batch_graph_launch(gbntt_batch* b, void* stream) {
    if (!b) return batch_fail(GBNTT_ERR_ARG, "batch is null");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!b->graph) {
        // capture on a private stream so the caller's stream may be the legacy default stream
        cudaStream_t cs;
        cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, "stream creation failed");
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        int rc = GBNTT_OK;
        if (e == cudaSuccess) rc = launch_batch(b, cs);
        cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        cudaStreamDestroy(cs);
        if (e != cudaSuccess || e2 != cudaSuccess || rc != GBNTT_OK || !g)
            return rc != GBNTT_OK ? rc : batch_fail(GBNTT_ERR_CUDA, "graph capture failed");
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->graph = nullptr;
            return batch_fail(GBNTT_ERR_CUDA, std::string("graph instantiation: ") + cudaGetErrorString(e));
        }
    }
    cudaError_t e = cudaGraphLaunch(b->graph, s);
    if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
    for (int i = 0; i < b->nparts; ++i)
        if (b->parts[i].layouts[b->parts[i].chosen].total_tiles) gbntt_internal_count_launch();
    for (size_t k = 0; k < b->user.size(); ++k)
        if (b->part_of[k] < 0 && b->user[k].count) gbntt_internal_count_launch();
    return GBNTT_OK;
}

int gbntt_batch_execute_host(gbntt_batch* b, const void* const* h_in, void* const* h_out, void* stream) {
    if (!b || !h_in || !h_out) return batch_fail(GBNTT_ERR_ARG, "null argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    auto bytes_of = [&](size_t k) {
        const gbntt_segment& u = b->user[k];
        int64_t n = 0, eb = 0;
        gbntt_plan_query(u.plan, GBNTT_Q_N, &n);
        gbntt_plan_query(u.plan, GBNTT_Q_ELEM_BYTES, &eb);
        return (size_t)u.count * (size_t)n * (size_t)eb;
    };
    // Zero copy: when every batched segment's host buffers are page-locked and
    // mapped, one k_batch_zc launch per storage type reads and writes them in
    // place, so inbound and outbound traffic overlap on the host-device link
    // instead of running as two copy phases.  Segments outside the persistent
    // kernel still go through their device buffers.
    bool zero_copy = true;
    std::vector<const void*> mapped_in(b->user.size()), mapped_out(b->user.size());
    for (size_t k = 0; k < b->user.size() && zero_copy; ++k) {
        if (b->part_of[k] < 0 || !bytes_of(k)) continue;
        const void* mi = mapped_in[k] = gbntt_internal_mapped(h_in[k]);
        const void* mo = mapped_out[k] = gbntt_internal_mapped(h_out[k]);
        zero_copy = b->parts[b->part_of[k]].zlay.cfg.zfn && mi && mo &&
                    !((reinterpret_cast<uintptr_t>(mi) | reinterpret_cast<uintptr_t>(mo)) & 15);
    }
    if (zero_copy) {
        std::vector<SegDev> uploaded[2];   // committed as the live descriptors once the call completed
        for (int i = 0; i < b->nparts; ++i) {
            auto& part = b->parts[i];
            auto& lay = part.zlay;
            if (!lay.total_tiles) continue;
            std::vector<SegDev> segs = lay.segs;
            for (size_t j = 0; j < segs.size(); ++j) {
                const int k = part.user_index[j];
                segs[j].a.in = mapped_in[k];
                segs[j].a.out = const_cast<void*>(mapped_out[k]);
            }
            // the same host buffers as the previous call (every earlier call
            // synchronised its stream): the device descriptors are current
            cudaError_t e = cudaSuccess;
            if (lay.live.size() != segs.size() ||
                std::memcmp(lay.live.data(), segs.data(), sizeof(SegDev) * segs.size()) != 0) {
                lay.live.clear();
                e = cudaMemcpyAsync(lay.d_segs, segs.data(), sizeof(SegDev) * segs.size(), cudaMemcpyHostToDevice, s);
                if (e != cudaSuccess)
                    return batch_fail(GBNTT_ERR_CUDA, std::string("descriptors: ") + cudaGetErrorString(e));
                uploaded[i] = std::move(segs);
            }
            BatchDev bd;
            bd.segs = lay.d_segs;
            bd.nsegs = (int)lay.segs.size();
            bd.total_tiles = lay.total_tiles;
            bd.ctr = b->d_ctr + CTR_WORDS * (BATCH_PARTS + i);
            bd.wait_polls = BATCH_WAIT_POLLS;
            int sb = lay.stage_bytes;
            void* args[] = {&bd, &sb};
            e = cudaLaunchKernel(lay.cfg.zfn, dim3(lay.grid), dim3(lay.cfg.cta), args, lay.smem, s);
            if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, std::string("zero-copy launch: ") + cudaGetErrorString(e));
            gbntt_internal_count_launch();
        }
        for (size_t k = 0; k < b->user.size(); ++k) {
            const size_t bytes = bytes_of(k);
            if (b->part_of[k] >= 0 || !bytes) continue;
            const gbntt_segment& u = b->user[k];
            cudaError_t e = cudaMemcpyAsync(const_cast<void*>(u.d_in), h_in[k], bytes, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, std::string("H2D: ") + cudaGetErrorString(e));
            const int rc = gbntt_execute(u.plan, u.d_in, u.d_out, u.count, s);
            if (rc != GBNTT_OK) return rc;
            e = cudaMemcpyAsync(h_out[k], u.d_out, bytes, cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, std::string("D2H: ") + cudaGetErrorString(e));
        }
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, std::string("synchronize: ") + cudaGetErrorString(e));
        for (int i = 0; i < b->nparts; ++i)
            if (!uploaded[i].empty()) b->parts[i].zlay.live = std::move(uploaded[i]);
        return GBNTT_OK;
    }
    for (size_t k = 0; k < b->user.size(); ++k) {
        const size_t bytes = bytes_of(k);
        if (!bytes) continue;
        cudaError_t e = cudaMemcpyAsync(const_cast<void*>(b->user[k].d_in), h_in[k], bytes, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, std::string("H2D: ") + cudaGetErrorString(e));
    }
    int rc = gbntt_batch_graph_launch(b, stream);
    if (rc != GBNTT_OK) return rc;
    for (size_t k = 0; k < b->user.size(); ++k) {
        const size_t bytes = bytes_of(k);
        if (!bytes) continue;
        cudaError_t e = cudaMemcpyAsync(h_out[k], b->user[k].d_out, bytes, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, std::string("D2H: ") + cudaGetErrorString(e));
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, std::string("synchronize: ") + cudaGetErrorString(e));
    return GBNTT_OK;
}

int gbntt_batch_set_io(gbntt_batch* b, uint32_t seg, const void* d_in, void* d_out) {
    if (!b || seg >= b->user.size()) return batch_fail(GBNTT_ERR_ARG, "bad segment");
    if (!d_in || !d_out || ((reinterpret_cast<uintptr_t>(d_in) | reinterpret_cast<uintptr_t>(d_out)) & 15))
        return batch_fail(GBNTT_ERR_ARG, "device buffers must be non-null and 16-byte aligned");
    const int pi = b->part_of[seg];
    if (pi >= 0 && d_in == d_out) return batch_fail(GBNTT_ERR_ARG, "batched segments cannot run in place");
    b->user[seg].d_in = d_in;
    b->user[seg].d_out = d_out;
    if (pi >= 0) {
        const int j = b->index_in_part[seg];
        for (auto& lay : b->parts[pi].layouts) {
            SegDev& sd = lay.segs[j];
            sd.a.in = d_in;
            sd.a.out = d_out;
            cudaError_t e = cudaMemcpy(lay.d_segs + j, &sd, sizeof(SegDev), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, "descriptor update failed");
        }
    } else if (b->graph) {
        cudaGraphExecDestroy(b->graph);   // per-plan launches captured the old pointers
        b->graph = nullptr;
    }
    return GBNTT_OK;
}

int gbntt_batch_status(gbntt_batch* b) {
    if (!b) return batch_fail(GBNTT_ERR_ARG, "batch is null");
    unsigned long long w[CTR_WORDS * BATCH_PARTS];
    cudaError_t e = cudaMemcpy(w, b->d_ctr, sizeof(w), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, std::string("status read: ") + cudaGetErrorString(e));
    bool timed_out = false;
    for (int i = 0; i < BATCH_PARTS; ++i) timed_out |= w[CTR_WORDS * i + CTR_ERROR] != 0;
    if (timed_out) {
        cudaMemset(b->d_ctr, 0, sizeof(w));
        return batch_fail(GBNTT_ERR_TIMEOUT, "a tile load did not arrive within the wait limit");
    }
    return GBNTT_OK;
}

int gbntt_batch_query(const gbntt_batch* b, int what, int64_t* value) {
    if (!b || !value) return batch_fail(GBNTT_ERR_ARG, "null argument");
    int64_t v = 0;
    for (int i = 0; i < b->nparts; ++i) {
        const auto& lay = b->parts[i].layouts[b->parts[i].chosen];
        switch (what) {
        case GBNTT_BQ_LAUNCHES: v += lay.total_tiles ? 1 : 0; break;
        case GBNTT_BQ_TILES: v += lay.total_tiles; break;
        case GBNTT_BQ_GRID: v = std::max<int64_t>(v, lay.grid); break;
        case GBNTT_BQ_SMEM: v = std::max<int64_t>(v, lay.smem); break;
        case GBNTT_BQ_EL16: if (!b->parts[i].i32) v = lay.cfg.elmax; break;
        case GBNTT_BQ_FAMSET: if (!b->parts[i].i32) v = lay.cfg.set; break;
        case GBNTT_BQ_CTA: if (!b->parts[i].i32) v = lay.cfg.cta; break;
        case GBNTT_BQ_OCC: if (!b->parts[i].i32) v = lay.cfg.occ; break;
        default: return batch_fail(GBNTT_ERR_ARG, "unknown query");
        }
    }
    if (what == GBNTT_BQ_LAUNCHES)
        for (size_t k = 0; k < b->user.size(); ++k) v += (b->part_of[k] < 0 && b->user[k].count) ? 1 : 0;
    *value = v;
    return GBNTT_OK;
}

int gbntt_batch_destroy(gbntt_batch* b) {
    if (!b) return GBNTT_OK;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (int i = 0; i < b->nparts; ++i) {
        for (auto& lay : b->parts[i].layouts)
            if (lay.d_segs) cudaFree(lay.d_segs);
        if (b->parts[i].zlay.d_segs) cudaFree(b->parts[i].zlay.d_segs);
    }
    if (b->d_ctr) cudaFree(b->d_ctr);
    delete b;
    return GBNTT_OK;
}

}  // extern "C"
