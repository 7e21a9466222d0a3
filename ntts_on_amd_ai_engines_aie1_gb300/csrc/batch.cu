// batch.cu -- persistent batched launches (gbntt_batch_* in include/gb300_ntt.h).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gb300_ntt.h"
#include "persist.cuh"
#include "plan_internal.h"

namespace gbntt {

namespace {

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

constexpr int SMEM_HEADER = 1024;   // mbarriers + the current segment's KArgs

template <bool I32, int CTA, int ELMAX>
__global__ void __launch_bounds__(CTA, (I32 || ELMAX > 5) ? 2 : 3) k_batch(const BatchDev b, int stage_bytes) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem);
    KArgs* ka = reinterpret_cast<KArgs*>(smem + 64);
    unsigned char* stage0 = smem + SMEM_HEADER;
    int* xbuf = reinterpret_cast<int*>(smem + SMEM_HEADER + 2 * stage_bytes);
    __shared__ long long sh_next;
    __shared__ int sh_pending[2];
    __shared__ int sh_failed;
    const int tid = threadIdx.x;
    const long long total = b.total_tiles;

    auto seg_of = [&](long long t) {
        int s = 0;
        while (s + 1 < b.nsegs && __ldg(&b.segs[s + 1].tile0) <= t) ++s;
        return s;
    };
    // thread 0: start the bulk load of tile t into buffer i
    auto issue = [&](long long t, int i) {
        const SegDev* sd = &b.segs[seg_of(t)];
        const long long lt = t - sd->tile0;
        const long long P = sd->polys_per_tile;
        const long long count = sd->a.batch;
        const long long np = min(P, count - lt * P);
        const unsigned bytes = (unsigned)(np * sd->n * sd->elem_bytes);
        const char* src = static_cast<const char*>(sd->a.in) + lt * P * sd->n * sd->elem_bytes;
        mbar_expect_tx(&bar[i], bytes);
        bulk_load(stage0 + i * stage_bytes, src, bytes, &bar[i]);
    };

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        const long long t0 = (long long)atomicAdd(&b.ctr[CTR_NEXT], 1ull);
        sh_next = t0;
        sh_pending[0] = 0;
        sh_pending[1] = 0;
        sh_failed = 0;
        if (t0 < total) {
            issue(t0, 0);
            sh_pending[0] = 1;
        }
    }
    __syncthreads();
    long long t = sh_next;
    unsigned phases = 0u;    // bit i: parity of the next completion of bar[i]
    int buf = 0;
    int cur_seg = -1;
    KC kc;
    while (t < total) {
        const int s = seg_of(t);
        const SegDev* sd = &b.segs[s];
        if (tid == 0) {
            const long long tn = (long long)atomicAdd(&b.ctr[CTR_NEXT], 1ull);
            sh_next = tn;
            if (tn < total) {
                bulk_wait_read();           // the other buffer's last store has left shared memory
                issue(tn, buf ^ 1);
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
        if (!mbar_wait(&bar[buf], (phases >> buf) & 1u)) sh_failed = 1;
        phases ^= 1u << buf;
        const long long lt = t - sd->tile0;
        const int P = sd->polys_per_tile;
        const int np = (int)min((long long)P, sd->a.batch - lt * P);
        const int variant = sd->variant;
        void* st = stage0 + buf * stage_bytes;
        switch (variant) {
#define GB_CASE(F, L)                                                     \
    case variant_id(F, L):                                                \
        if constexpr (fam_i32(F) == I32) tile_transform<F, L, CTA, ELMAX>(st, xbuf, kc, np); \
        break;
            GB_I16_VARIANTS(GB_CASE)
            GB_I32_VARIANTS(GB_CASE)
#undef GB_CASE
            default: break;
        }
        __syncthreads();
        const long long tnext = sh_next;
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
            // let a prefetch that is still in flight land before the CTA leaves (bounded)
            // (bar[buf]'s parity bit was already advanced past the load it waited for)
            for (int i = 0; i < 2; ++i)
                if (sh_pending[i]) mbar_wait(&bar[i], ((phases >> i) & 1u) ^ (i == buf ? 1u : 0u));
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

bool variant_supported(int fam, int L) {
#define GB_HAS(F, L_) if (fam == F && L == L_) return true;
    GB_I16_VARIANTS(GB_HAS)
    GB_I32_VARIANTS(GB_HAS)
#undef GB_HAS
    return false;
}

constexpr int BATCH_CTA = 256;

}  // namespace

// persistent-kernel configurations: (storage type, coefficients per thread)
struct BatchConfig {
    bool i32;
    int elmax;
    const void* fn;
};

static const BatchConfig kConfigs[] = {
    {false, 6, reinterpret_cast<const void*>(&k_batch<false, BATCH_CTA, 6>)},
    {false, 5, reinterpret_cast<const void*>(&k_batch<false, BATCH_CTA, 5>)},
    {true, 5, reinterpret_cast<const void*>(&k_batch<true, BATCH_CTA, 5>)},
};

}  // namespace gbntt

using namespace gbntt;

struct gbntt_batch {
    struct Layout {                     // one configuration of one persistent launch
        int cfg = -1;                   // index into kConfigs
        std::vector<SegDev> segs;
        SegDev* d_segs = nullptr;
        long long total_tiles = 0;
        int stage_bytes = 0, smem = 0, grid = 0;
        float ms = -1.f;                // autotuner timing
    };
    struct Part {                       // the int16 or the int32 segments
        bool i32 = false;
        std::vector<Layout> layouts;    // candidate configurations
        int chosen = 0;
        std::vector<int> user_index;    // caller's segment of each SegDev
    };
    Part parts[2];
    int nparts = 0;
    std::vector<int> part_of;           // segment -> part (or -1: separate per-plan launch)
    std::vector<int> index_in_part;
    std::vector<gbntt_segment> user;    // the caller's segments
    unsigned long long* d_ctr = nullptr;   // CTR_WORDS per part
    cudaGraphExec_t graph = nullptr;
};

namespace {

int batch_fail(int code, const std::string& msg) { return gbntt_internal_fail(code, msg); }

int launch_layout(gbntt_batch* b, int pi, const gbntt_batch::Layout& lay, cudaStream_t s) {
    if (lay.total_tiles == 0) return GBNTT_OK;
    BatchDev bd;
    bd.segs = lay.d_segs;
    bd.nsegs = (int)lay.segs.size();
    bd.total_tiles = lay.total_tiles;
    bd.ctr = b->d_ctr + CTR_WORDS * pi;
    int sb = lay.stage_bytes;
    void* args[] = {&bd, &sb};
    cudaError_t e = cudaLaunchKernel(kConfigs[lay.cfg].fn, dim3(lay.grid), dim3(BATCH_CTA), args, lay.smem, s);
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
int autotune(gbntt_batch* b) {
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
        return batch_fail(GBNTT_ERR_CUDA, "autotune stream");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = GBNTT_OK;
    for (int i = 0; i < b->nparts && rc == GBNTT_OK; ++i) {
        auto& p = b->parts[i];
        if (p.layouts.size() < 2) continue;
        for (size_t c = 0; c < p.layouts.size() && rc == GBNTT_OK; ++c) {
            for (int w = 0; w < 2 && rc == GBNTT_OK; ++w) rc = launch_layout(b, i, p.layouts[c], s);
            cudaEventRecord(e0, s);
            for (int w = 0; w < 5 && rc == GBNTT_OK; ++w) rc = launch_layout(b, i, p.layouts[c], s);
            cudaEventRecord(e1, s);
            if (cudaEventSynchronize(e1) != cudaSuccess) rc = batch_fail(GBNTT_ERR_CUDA, "autotune timing");
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            p.layouts[c].ms = ms / 5.f;
        }
        size_t best = 0;
        for (size_t c = 1; c < p.layouts.size(); ++c)
            if (p.layouts[c].ms >= 0.f && p.layouts[c].ms < p.layouts[best].ms) best = c;
        p.chosen = (int)best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    return rc;
}

}  // namespace

extern "C" {

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
    int pid[2] = {-1, -1};
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
        int& id = pid[i32 ? 1 : 0];
        if (id < 0) {
            id = b->nparts++;
            b->parts[id].i32 = i32;
            for (int c = 0; c < (int)(sizeof(kConfigs) / sizeof(kConfigs[0])); ++c)
                if (kConfigs[c].i32 == i32) {
                    gbntt_batch::Layout lay;
                    lay.cfg = c;
                    b->parts[id].layouts.push_back(lay);
                }
        }
        auto& part = b->parts[id];
        b->part_of[k] = id;
        b->index_in_part[k] = (int)part.user_index.size();
        part.user_index.push_back(k);
        for (auto& lay : part.layouts) {
            const int elmax = kConfigs[lay.cfg].elmax;
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
            sd.polys_per_tile = BATCH_CTA / G;
            sd.tiles = ((long long)u.count + sd.polys_per_tile - 1) / sd.polys_per_tile;
            sd.tile0 = lay.total_tiles;
            lay.total_tiles += sd.tiles;
            lay.stage_bytes = std::max(lay.stage_bytes, batch_stage_bytes(BATCH_CTA, L, eb, elmax));
            lay.smem = std::max(lay.smem, batch_xbuf_bytes(BATCH_CTA, L, elmax));
            lay.segs.push_back(sd);
        }
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (int i = 0; i < b->nparts; ++i) {
        for (auto& lay : b->parts[i].layouts) {
            lay.stage_bytes = (lay.stage_bytes + 127) & ~127;
            lay.smem = SMEM_HEADER + 2 * lay.stage_bytes + lay.smem;
            const void* fn = kConfigs[lay.cfg].fn;
            cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, lay.smem);
            int per_sm = 0;
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, BATCH_CTA, lay.smem);
            if (e != cudaSuccess || per_sm < 1) {
                gbntt_batch_destroy(b);
                return batch_fail(GBNTT_ERR_CUDA, std::string("batch kernel configuration: ") + cudaGetErrorString(e));
            }
            lay.grid = (int)std::min<long long>((long long)per_sm * sms, lay.total_tiles);
            e = cudaMalloc(&lay.d_segs, sizeof(SegDev) * lay.segs.size());
            if (e == cudaSuccess)
                e = cudaMemcpy(lay.d_segs, lay.segs.data(), sizeof(SegDev) * lay.segs.size(), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) {
                gbntt_batch_destroy(b);
                return batch_fail(GBNTT_ERR_NOMEM, "batch descriptor allocation failed");
            }
        }
    }
    cudaError_t e = cudaMalloc(&b->d_ctr, sizeof(unsigned long long) * CTR_WORDS * 2);
    if (e == cudaSuccess) e = cudaMemset(b->d_ctr, 0, sizeof(unsigned long long) * CTR_WORDS * 2);
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
    unsigned long long w[CTR_WORDS * 2];
    cudaError_t e = cudaMemcpy(w, b->d_ctr, sizeof(w), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return batch_fail(GBNTT_ERR_CUDA, std::string("status read: ") + cudaGetErrorString(e));
    if (w[CTR_ERROR] || w[CTR_WORDS + CTR_ERROR]) {
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
        case GBNTT_BQ_EL16: if (!b->parts[i].i32) v = kConfigs[lay.cfg].elmax; break;
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
    for (int i = 0; i < b->nparts; ++i)
        for (auto& lay : b->parts[i].layouts)
            if (lay.d_segs) cudaFree(lay.d_segs);
    if (b->d_ctr) cudaFree(b->d_ctr);
    delete b;
    return GBNTT_OK;
}

}  // extern "C"
