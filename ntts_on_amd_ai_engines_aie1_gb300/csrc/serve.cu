// serve.cu -- the serving loop (gbntt_server_* in include/gb300_ntt.h).
//
// Requests (plan, host input, host output, polynomial count) arrive from any
// host thread.  One worker thread runs continuous batching:
//   * admission: a request is admitted when the device arena (sized from the
//     free HBM at start-up) has room for its polynomials; requests larger than
//     the whole arena are refused;
//   * micro-batches: the admitted requests that are waiting when a stream
//     slot is free are grouped by plan; each plan group gets one contiguous
//     arena block and its inputs are copied in; one in-place launch of the
//     persistent kernel per storage type transforms every group at once (one
//     segment per group; int32 transforms of n >= 2^16 run their plan's
//     two-pass launches); the outputs are copied back and an event closes
//     the slot;
//   * copies: requests whose host buffers are page-locked and mapped into the
//     device's address space move through one gather kernel (host -> arena)
//     and one scatter kernel (arena -> host) per micro-batch, driven by a
//     descriptor table uploaded with one copy, so the host issues a handful of
//     calls per micro-batch instead of two per request; other requests use
//     one cudaMemcpyAsync per direction;
//   * while slots are busy on the GPU, newly arrived requests are admitted
//     into the next micro-batch, so copies and kernels of different
//     micro-batches overlap on the device;
//   * completion is observed by polling the slots' events; latencies (submit
//     to completion) feed the p50/p99 statistics.
// All waits on the host are bounded by the caller's timeout.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/gb300_ntt.h"
#include "batch_kernel.cuh"
#include "plan_internal.h"

namespace gbntt {

// First-fit allocator over one device arena, in units of ALIGN bytes.  Host
// bookkeeping only (no CUDA calls), so it is tested without a GPU.
class Arena {
public:
    static constexpr size_t ALIGN = 256;
    explicit Arena(size_t bytes = 0) { reset(bytes); }
    void reset(size_t bytes) {
        cap_ = bytes / ALIGN * ALIGN;
        free_.clear();
        if (cap_) free_[0] = cap_;
        used_ = 0;
    }
    // offset of a block of `bytes`, or SIZE_MAX when it does not fit now
    size_t alloc(size_t bytes) {
        const size_t need = (bytes + ALIGN - 1) / ALIGN * ALIGN;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= need) {
                const size_t off = it->first, len = it->second;
                free_.erase(it);
                if (len > need) free_[off + need] = len - need;
                used_ += need;
                return off;
            }
        }
        return SIZE_MAX;
    }
    void release(size_t off, size_t bytes) {
        const size_t need = (bytes + ALIGN - 1) / ALIGN * ALIGN;
        used_ -= need;
        auto it = free_.emplace(off, need).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {   // merge with the next block
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {                                        // and with the previous one
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t capacity() const { return cap_; }
    size_t used() const { return used_; }
    size_t largest_free() const {
        size_t m = 0;
        for (const auto& f : free_) m = std::max(m, f.second);
        return m;
    }

private:
    size_t cap_ = 0, used_ = 0;
    std::map<size_t, size_t> free_;   // offset -> length
};

// p-th percentile (0..100) by nearest rank of an unsorted sample
double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    size_t rank = (size_t)std::ceil(p / 100.0 * (double)v.size());
    if (rank < 1) rank = 1;
    if (rank > v.size()) rank = v.size();
    return v[rank - 1];
}

}  // namespace gbntt

using namespace gbntt;
using Clock = std::chrono::steady_clock;

namespace {

struct Request {
    uint64_t ticket;
    uint32_t plan;
    const void* h_in;
    void* h_out;
    uint64_t count;
    size_t bytes;
    Clock::time_point t_submit;
    const void* m_in;   // device addresses of mapped host buffers (nullptr: copy engine)
    void* m_out;
};

// one host<->arena copy of the gather/scatter kernels, cut into COPY_CHUNK pieces
struct CopyDesc {
    const unsigned char* src;
    unsigned char* dst;
    unsigned long long bytes;
    unsigned long long chunk0;   // first chunk index of this copy
};
constexpr unsigned long long COPY_CHUNK = 16384;
constexpr int COPY_THREADS = 256;

// block c copies chunk c: it finds its descriptor by binary search over chunk0
__global__ void __launch_bounds__(COPY_THREADS) k_copy_desc(const CopyDesc* __restrict__ d, int nd) {
    const unsigned long long c = blockIdx.x;
    int lo = 0, hi = nd - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (d[mid].chunk0 <= c) lo = mid;
        else hi = mid - 1;
    }
    const unsigned long long off = (c - d[lo].chunk0) * COPY_CHUNK;
    const unsigned long long rem = d[lo].bytes - off;
    const unsigned len = (unsigned)(rem < COPY_CHUNK ? rem : COPY_CHUNK);
    const unsigned char* s = d[lo].src + off;
    unsigned char* t = d[lo].dst + off;
    const unsigned long long mis = reinterpret_cast<unsigned long long>(s) | reinterpret_cast<unsigned long long>(t) | len;
    if (!(mis & 15)) {
        for (unsigned i = threadIdx.x; i < len / 16; i += COPY_THREADS)
            reinterpret_cast<uint4*>(t)[i] = reinterpret_cast<const uint4*>(s)[i];
    } else if (!(mis & 3)) {
        for (unsigned i = threadIdx.x; i < len / 4; i += COPY_THREADS)
            reinterpret_cast<unsigned*>(t)[i] = reinterpret_cast<const unsigned*>(s)[i];
    } else {
        for (unsigned i = threadIdx.x; i < len; i += COPY_THREADS) t[i] = s[i];
    }
}

struct Group {                  // one plan's requests in one micro-batch
    uint32_t plan;
    size_t off = 0, bytes = 0;
    uint64_t count = 0;
    std::vector<Request> reqs;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaStream_t aux = nullptr;            // the int32 persistent launch, beside the int16 one
    cudaEvent_t done = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    bool busy = false;
    std::vector<Group> groups;
    // page-locked descriptor block of one micro-batch: the gather copies, the
    // scatter copies (the last one returns the error words), then the segment
    // descriptors of the int16 and the int32 persistent launches; it goes to
    // d_blk with one copy
    unsigned char* h_blk = nullptr;
    unsigned char* d_blk = nullptr;
    unsigned long long* d_ctr = nullptr;   // tile counters of the persistent launches (one per part)
    unsigned long long* h_err = nullptr;   // their error words (mapped), written by the scatter kernel
    unsigned long long* m_err = nullptr;   // device address of h_err
};

constexpr size_t ERR_BYTES = BATCH_PARTS * CTR_WORDS * sizeof(unsigned long long);
constexpr size_t BLK_ALIGN = 128;
size_t blk_round(size_t b) { return (b + BLK_ALIGN - 1) / BLK_ALIGN * BLK_ALIGN; }

// a plan as the persistent kernel sees it
struct PlanInfo {
    int fam = -1, L = 0, eb = 0;
    gbntt::KArgs a;
    int part = -1;   // persistent launch (batch_part_of), -1: the plan's own launches
};

// one persistent launch configuration per storage type and arithmetic
struct PartCfg {
    const gbntt::BatchConfig* cfg = nullptr;
    int stage = 0, smem = 0, grid = 0;
};

}  // namespace

struct gbntt_server {
    std::vector<const gbntt_plan*> plans;
    std::vector<int64_t> plan_bytes;   // bytes of one polynomial
    std::vector<PlanInfo> pinfo;
    PartCfg part[BATCH_PARTS];
    std::vector<Slot> slots;
    Arena arena;
    char* d_arena = nullptr;
    uint32_t max_group_requests = 0;
    int device = 0;

    // submissions: a short-held inbox the worker swaps out, so submitting never
    // waits for the worker's micro-batch formation
    std::mutex inbox_mu;
    std::condition_variable cv_work;           // with inbox_mu: new requests or stop
    std::vector<Request> inbox;
    std::deque<Request> pending;               // the worker's own queue (arrival order)
    std::atomic<uint64_t> next_ticket{1};
    std::atomic<long long> outstanding{0};     // admitted and not yet completed
    std::atomic<bool> stop{false};
    std::atomic<int> worker_error{GBNTT_OK};
    std::thread worker;

    std::mutex mu;                             // status, statistics, worker_msg
    std::condition_variable cv_done;           // with mu: completions
    std::unordered_map<uint64_t, int> status;  // ticket -> status (absent: in flight)
    std::string worker_msg;

    // statistics (guarded by mu)
    std::vector<double> lat_us;
    uint64_t completed = 0, refused = 0, polys = 0, microbatches = 0, launches = 0;
    size_t peak_used = 0;
    Clock::time_point t_first, t_last;
};

namespace {

int sfail(int code, const std::string& m) { return gbntt_internal_fail(code, m); }

// the worker thread's error: stops the loop and fails every later wait
void set_worker_error(gbntt_server* s, int code, const std::string& msg) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->worker_msg = msg;
    s->worker_error = code;
    s->stop = true;
    s->cv_done.notify_all();
}

void finish_slot(gbntt_server* s, Slot& sl) {
    const auto now = Clock::now();
    bool timed_out = false;   // a tile load ran out of its wait limit
    for (int p = 0; p < BATCH_PARTS; ++p) timed_out |= sl.h_err[CTR_WORDS * p + CTR_ERROR] != 0;
    if (timed_out)
        set_worker_error(s, GBNTT_ERR_TIMEOUT, "serve: a tile load did not arrive within the wait limit");
    long long done = 0;
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto& g : sl.groups) {
        s->arena.release(g.off, g.bytes);   // the arena is the worker's; released under mu for the stats
        for (auto& r : g.reqs) {
            s->status[r.ticket] = GBNTT_OK;
            s->lat_us.push_back(std::chrono::duration<double, std::micro>(now - r.t_submit).count());
            s->polys += r.count;
            ++s->completed;
            ++done;
        }
    }
    s->t_last = now;
    sl.groups.clear();
    sl.busy = false;
    s->outstanding -= done;
    s->cv_done.notify_all();
}

// Issue one micro-batch on slot sl: one descriptor upload, the gather kernel
// for mapped requests (copy engine for the others), the int16 and int32
// persistent launches side by side, the plans' own launches, the scatter
// kernel (which also returns the persistent launches' error words), event.
int issue(gbntt_server* s, Slot& sl) {
    uint64_t nl = 0;   // launches of this micro-batch (published under the lock at the end)
    CopyDesc* desc = reinterpret_cast<CopyDesc*>(sl.h_blk);
    int nin = 0;
    unsigned long long cin = 0;
    for (auto& g : sl.groups) {               // gather descriptors
        size_t at = 0;
        for (auto& r : g.reqs) {
            if (r.m_in) {
                desc[nin++] = CopyDesc{static_cast<const unsigned char*>(r.m_in),
                                       reinterpret_cast<unsigned char*>(s->d_arena + g.off + at), r.bytes, cin};
                cin += (r.bytes + COPY_CHUNK - 1) / COPY_CHUNK;
            }
            at += r.bytes;
        }
    }
    int nout = 0;
    unsigned long long cout = 0;
    CopyDesc* od = desc + nin;
    for (auto& g : sl.groups) {               // scatter descriptors
        size_t at = 0;
        for (auto& r : g.reqs) {
            if (r.m_out) {
                od[nout++] = CopyDesc{reinterpret_cast<const unsigned char*>(s->d_arena + g.off + at),
                                      static_cast<unsigned char*>(r.m_out), r.bytes, cout};
                cout += (r.bytes + COPY_CHUNK - 1) / COPY_CHUNK;
            }
            at += r.bytes;
        }
    }
    od[nout++] = CopyDesc{reinterpret_cast<const unsigned char*>(sl.d_ctr),
                          reinterpret_cast<unsigned char*>(sl.m_err), ERR_BYTES, cout};
    cout += 1;

    // segment descriptors, one persistent launch per storage type, largest n first
    std::vector<const Group*> order;
    for (auto& g : sl.groups) order.push_back(&g);
    std::stable_sort(order.begin(), order.end(), [&](const Group* x, const Group* y) {
        return s->pinfo[x->plan].L > s->pinfo[y->plan].L;
    });
    int nseg[BATCH_PARTS] = {};
    for (const Group* g : order)
        if (s->pinfo[g->plan].part >= 0) ++nseg[s->pinfo[g->plan].part];
    const size_t seg_off = blk_round((size_t)(nin + nout) * sizeof(CopyDesc));
    SegDev* segs = reinterpret_cast<SegDev*>(sl.h_blk + seg_off);
    int first[BATCH_PARTS], fill[BATCH_PARTS], total_segs = 0;
    for (int p = 0; p < BATCH_PARTS; ++p) {
        first[p] = fill[p] = total_segs;
        total_segs += nseg[p];
    }
    long long tiles[BATCH_PARTS] = {};
    for (const Group* g : order) {
        const PlanInfo& pi = s->pinfo[g->plan];
        if (pi.part < 0) continue;
        SegDev& sd = segs[fill[pi.part]++];
        std::memset(&sd, 0, sizeof(sd));
        sd.a = pi.a;
        sd.a.in = s->d_arena + g->off;
        sd.a.out = s->d_arena + g->off;
        sd.a.batch = (long long)g->count;
        sd.n = 1 << pi.L;
        sd.elem_bytes = pi.eb;
        sd.variant = variant_id(pi.fam, pi.L);
        sd.polys_per_tile = BATCH_CTA >> (pi.L - batch_el(pi.L, s->part[pi.part].cfg->elmax));
        sd.tiles = (sd.a.batch + sd.polys_per_tile - 1) / sd.polys_per_tile;
        sd.tile0 = tiles[pi.part];
        tiles[pi.part] += sd.tiles;
    }
    const size_t used = seg_off + (size_t)total_segs * sizeof(SegDev);
    cudaError_t e = cudaMemcpyAsync(sl.d_blk, sl.h_blk, used, cudaMemcpyHostToDevice, sl.stream);
    if (e != cudaSuccess) return sfail(GBNTT_ERR_CUDA, std::string("serve descriptors: ") + cudaGetErrorString(e));
    const CopyDesc* d_desc = reinterpret_cast<const CopyDesc*>(sl.d_blk);
    SegDev* d_segs = reinterpret_cast<SegDev*>(sl.d_blk + seg_off);

    if (nin) {
        k_copy_desc<<<(unsigned)cin, COPY_THREADS, 0, sl.stream>>>(d_desc, nin);
        gbntt_internal_count_launch();
        ++nl;
    }
    for (auto& g : sl.groups) {
        char* base = s->d_arena + g.off;
        size_t at = 0;
        for (auto& r : g.reqs) {
            if (!r.m_in) {
                e = cudaMemcpyAsync(base + at, r.h_in, r.bytes, cudaMemcpyHostToDevice, sl.stream);
                if (e != cudaSuccess) return sfail(GBNTT_ERR_CUDA, std::string("serve H2D: ") + cudaGetErrorString(e));
            }
            at += r.bytes;
        }
    }
    auto launch_part = [&](int p, cudaStream_t st) -> cudaError_t {
        const PartCfg& pc = s->part[p];
        BatchDev bd;
        bd.segs = d_segs + first[p];
        bd.nsegs = nseg[p];
        bd.total_tiles = tiles[p];
        bd.ctr = sl.d_ctr + CTR_WORDS * p;
        bd.wait_polls = batch_wait_polls();
        int sb = pc.stage;
        void* args[] = {&bd, &sb};
        const unsigned grid = (unsigned)std::min<long long>(pc.grid, tiles[p]);
        const cudaError_t le = cudaLaunchKernel(pc.cfg->fn, dim3(grid), dim3(BATCH_CTA), args, pc.smem, st);
        if (le == cudaSuccess) {
            gbntt_internal_count_launch();
            ++nl;
        }
        return le;
    };
    int used_parts[BATCH_PARTS], nparts = 0;
    for (int p = 0; p < BATCH_PARTS; ++p)
        if (nseg[p]) used_parts[nparts++] = p;
    if (nparts >= 2) {
        // the launches share nothing but the gather before them: the first on
        // the slot's stream, the others beside it on the second stream
        e = cudaEventRecord(sl.fork, sl.stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sl.aux, sl.fork, 0);
        for (int i = 1; i < nparts && e == cudaSuccess; ++i) e = launch_part(used_parts[i], sl.aux);
        if (e == cudaSuccess) e = cudaEventRecord(sl.join, sl.aux);
        if (e == cudaSuccess) e = launch_part(used_parts[0], sl.stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sl.stream, sl.join, 0);
    } else if (nparts == 1) {
        e = launch_part(used_parts[0], sl.stream);
    }
    if (e != cudaSuccess) return sfail(GBNTT_ERR_CUDA, std::string("serve launch: ") + cudaGetErrorString(e));
    for (const Group* g : order) {
        if (s->pinfo[g->plan].part >= 0) continue;
        const int rc = gbntt_execute(s->plans[g->plan], s->d_arena + g->off, s->d_arena + g->off, g->count,
                                     sl.stream);
        if (rc != GBNTT_OK) return rc;
        ++nl;
    }
    k_copy_desc<<<(unsigned)cout, COPY_THREADS, 0, sl.stream>>>(d_desc + nin, nout);
    gbntt_internal_count_launch();
    ++nl;
    for (auto& g : sl.groups) {
        char* base = s->d_arena + g.off;
        size_t at = 0;
        for (auto& r : g.reqs) {
            if (!r.m_out) {
                e = cudaMemcpyAsync(r.h_out, base + at, r.bytes, cudaMemcpyDeviceToHost, sl.stream);
                if (e != cudaSuccess) return sfail(GBNTT_ERR_CUDA, std::string("serve D2H: ") + cudaGetErrorString(e));
            }
            at += r.bytes;
        }
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return sfail(GBNTT_ERR_CUDA, std::string("serve copy kernel: ") + cudaGetErrorString(e));
    e = cudaEventRecord(sl.done, sl.stream);
    if (e != cudaSuccess) return sfail(GBNTT_ERR_CUDA, std::string("serve event: ") + cudaGetErrorString(e));
    sl.busy = true;
    std::lock_guard<std::mutex> lk(s->mu);
    s->launches += nl;
    ++s->microbatches;
    return GBNTT_OK;
}

void worker_main(gbntt_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        // 1. completions
        bool any_busy = false;
        for (auto& sl : s->slots) {
            if (!sl.busy) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaSuccess) finish_slot(s, sl);
            else if (q == cudaErrorNotReady) any_busy = true;
            else set_worker_error(s, GBNTT_ERR_CUDA, std::string("serve: ") + cudaGetErrorString(q));
        }
        // 2. new requests
        {
            std::lock_guard<std::mutex> lk(s->inbox_mu);
            if (!s->inbox.empty()) {
                if (s->pending.empty()) {   // the first request since the statistics were reset
                    std::lock_guard<std::mutex> lk2(s->mu);
                    if (s->completed == 0 && s->microbatches == 0) s->t_first = Clock::now();
                }
                for (auto& r : s->inbox) s->pending.push_back(r);
                s->inbox.clear();
            }
        }
        if (s->stop && (s->pending.empty() || s->worker_error) && !any_busy) {
            std::lock_guard<std::mutex> lk(s->inbox_mu);
            if (s->inbox.empty() || s->worker_error) break;
            continue;
        }
        // 3. admission into a free slot: waiting requests in arrival order while the arena has room
        Slot* free_slot = nullptr;
        for (auto& sl : s->slots)
            if (!sl.busy) { free_slot = &sl; break; }
        std::vector<Group> groups;
        if (free_slot && !s->pending.empty() && !s->worker_error) {
            std::map<uint32_t, size_t> gi;
            uint32_t taken = 0;
            size_t mb_bytes = 0;
            const size_t budget = s->arena.capacity() / s->slots.size();   // one slot's share
            while (!s->pending.empty() && taken < s->max_group_requests) {
                Request& r = s->pending.front();
                if (taken && mb_bytes + r.bytes > budget) break;
                mb_bytes += r.bytes;
                auto it = gi.find(r.plan);
                Group* g;
                if (it == gi.end()) {
                    gi[r.plan] = groups.size();
                    groups.push_back(Group());
                    g = &groups.back();
                    g->plan = r.plan;
                } else {
                    g = &groups[it->second];
                }
                g->reqs.push_back(r);
                g->count += r.count;
                g->bytes += r.bytes;
                s->pending.pop_front();
                ++taken;
            }
            // one arena block per group; what does not fit goes back to the front of the queue
            std::lock_guard<std::mutex> lk(s->mu);
            for (size_t i = groups.size(); i-- > 0;) {
                Group& g = groups[i];
                g.off = s->arena.alloc(g.bytes);
                if (g.off == SIZE_MAX) {
                    for (auto r = g.reqs.rbegin(); r != g.reqs.rend(); ++r) s->pending.push_front(*r);
                    groups.erase(groups.begin() + (long)i);
                }
            }
            s->peak_used = std::max(s->peak_used, s->arena.used());
        } else if (!any_busy && s->pending.empty()) {
            std::unique_lock<std::mutex> lk(s->inbox_mu);
            s->cv_work.wait_for(lk, std::chrono::milliseconds(2), [&] { return !s->inbox.empty() || s->stop; });
            continue;
        }
        if (!groups.empty()) {
            // Groups that run their plan's own launches (int32 n >= 2^16 two-pass,
            // radix-4 inverse, ...) take longer than the persistent launch: with a
            // second free slot they form their own micro-batch, so the other
            // requests complete without waiting for them.
            std::vector<Group> slow;
            for (auto it = groups.begin(); it != groups.end();) {
                if (s->pinfo[it->plan].part < 0) {
                    slow.push_back(std::move(*it));
                    it = groups.erase(it);
                } else {
                    ++it;
                }
            }
            Slot* second = nullptr;
            if (!slow.empty() && !groups.empty())
                for (auto& sl : s->slots)
                    if (!sl.busy && &sl != free_slot) { second = &sl; break; }
            if (!second) {
                for (auto& g : slow) groups.push_back(std::move(g));
                slow.clear();
            }
            free_slot->groups = std::move(groups);
            int rc = issue(s, *free_slot);
            if (rc == GBNTT_OK && second) {
                second->groups = std::move(slow);
                rc = issue(s, *second);
            }
            if (rc != GBNTT_OK) set_worker_error(s, rc, gbntt_last_error());
        } else if (any_busy) {
            std::this_thread::yield();
        }
    }
}

}  // namespace

extern "C" {

int gbntt_server_create(gbntt_server** out, const gbntt_plan* const* plans, uint32_t nplans,
                        const gbntt_server_config* cfg) {
    if (!out || !plans || !nplans) return sfail(GBNTT_ERR_ARG, "server needs at least one plan");
    *out = nullptr;
    gbntt_server* s = new gbntt_server();
    s->plans.assign(plans, plans + nplans);
    for (auto* p : s->plans) {
        int64_t n = 0, eb = 0;
        if (!p || gbntt_plan_query(p, GBNTT_Q_N, &n) || gbntt_plan_query(p, GBNTT_Q_ELEM_BYTES, &eb)) {
            delete s;
            return sfail(GBNTT_ERR_ARG, "invalid plan");
        }
        int64_t kind = 0;
        gbntt_plan_query(p, GBNTT_Q_KIND, &kind);
        if (kind == GBNTT_R8_I16_STAGE) {
            delete s;
            return sfail(GBNTT_ERR_ARG, "the radix-8 stage cannot run in place and is not served");
        }
        s->plan_bytes.push_back(n * eb);
        PlanInfo pi;
        gbntt_internal_plan_args(p, &pi.fam, &pi.L, &pi.eb, &pi.a);
        if (pi.fam >= 0 && variant_supported(pi.fam, pi.L)) pi.part = batch_part_of(pi.fam);
        s->pinfo.push_back(pi);
    }
    // per storage type: one persistent configuration covering the served families
    {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        for (int p = 0; p < BATCH_PARTS; ++p) {
            int mask = 0, stage = 0, xbytes = 0, maxL = 0;
            for (const auto& pi : s->pinfo)
                if (pi.part == p) {
                    mask |= 1 << pi.fam;
                    maxL = std::max(maxL, pi.L);
                }
            if (!mask) continue;
            const BatchConfig* cfgs = nullptr;
            const int ncfg = (p & 1) ? batch_configs_i32(&cfgs) : batch_configs_i16(&cfgs);
            // the narrowest covering configuration (16 coefficients per thread
            // measured faster than 32 on mixed radix-4 batches), with the most
            // resident CTAs among those
            const BatchConfig* cfg = nullptr;
            auto resident = [&](const BatchConfig& c) {
                return c.occ ? c.occ : batch_min_blocks(c.i32, c.cta, c.elmax);
            };
            for (int c = 0; c < ncfg; ++c)
                if (cfgs[c].cta == BATCH_CTA && (cfgs[c].set & mask) == mask && config_fits(cfgs[c], maxL) &&
                    (!cfg || cfgs[c].elmax < cfg->elmax ||
                     (cfgs[c].elmax == cfg->elmax && resident(cfgs[c]) > resident(*cfg))))
                    cfg = &cfgs[c];
            if (!cfg) {   // no persistent kernel covers them: the plans launch on their own
                for (auto& pi : s->pinfo)
                    if (pi.part == p) pi.part = -1;
                continue;
            }
            for (const auto& pi : s->pinfo) {
                if (pi.part != p) continue;
                stage = std::max(stage, batch_stage_bytes(BATCH_CTA, pi.L, pi.eb, cfg->elmax));
                xbytes = std::max(xbytes, batch_xbuf_bytes(BATCH_CTA, pi.L, cfg->elmax));
            }
            PartCfg& pc = s->part[p];
            pc.cfg = cfg;
            pc.stage = (stage + 127) & ~127;
            pc.smem = SMEM_HEADER + 2 * pc.stage + xbytes;
            int per_sm = 0;
            cudaError_t e = raise_smem_limit(cfg->fn, pc.smem);
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cfg->fn, BATCH_CTA, pc.smem);
            if (e != cudaSuccess || per_sm < 1) {
                delete s;
                return sfail(GBNTT_ERR_CUDA, std::string("serve kernel configuration: ") + cudaGetErrorString(e));
            }
            pc.grid = per_sm * sms;
        }
    }
    // 8 slots: C5 mix at half load p50/p99 164/333 us vs 201/480 us with 4 (16: 156/311, less capacity)
    const uint32_t nslots = cfg && cfg->slots ? cfg->slots : 8;
    s->max_group_requests = cfg && cfg->max_requests_per_batch ? cfg->max_requests_per_batch : 4096;
    cudaGetDevice(&s->device);
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) {
        delete s;
        return sfail(GBNTT_ERR_CUDA, std::string("cudaMemGetInfo: ") + cudaGetErrorString(e));
    }
    // admission budget: the configured bytes, capped at half of the free HBM
    size_t want = cfg && cfg->device_bytes ? (size_t)cfg->device_bytes : (size_t)1 << 30;
    want = std::min(want, free_b / 2);
    s->arena.reset(want);
    if (s->arena.capacity() == 0) {
        delete s;
        return sfail(GBNTT_ERR_ADMISSION, "no device memory for the request arena");
    }
    e = cudaMalloc(&s->d_arena, s->arena.capacity());
    if (e != cudaSuccess) {
        delete s;
        return sfail(GBNTT_ERR_NOMEM, "request arena allocation failed");
    }
    s->slots.resize(nslots);
    for (auto& sl : s->slots) {
        cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        cudaStreamCreateWithFlags(&sl.aux, cudaStreamNonBlocking);
        cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&sl.fork, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&sl.join, cudaEventDisableTiming);
        // gather + scatter copies of every request, the error-word copy, the segments
        const size_t bb = blk_round((2 * (size_t)s->max_group_requests + 1) * sizeof(CopyDesc)) +
                          2 * s->plans.size() * sizeof(SegDev);
        if (cudaHostAlloc(&sl.h_blk, bb, cudaHostAllocDefault) != cudaSuccess ||
            cudaMalloc(&sl.d_blk, bb) != cudaSuccess ||
            cudaHostAlloc(&sl.h_err, ERR_BYTES, cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer(reinterpret_cast<void**>(&sl.m_err), sl.h_err, 0) != cudaSuccess ||
            cudaMalloc(&sl.d_ctr, ERR_BYTES) != cudaSuccess || cudaMemset(sl.d_ctr, 0, ERR_BYTES) != cudaSuccess) {
            cudaGetLastError();
            gbntt_server_destroy(s);
            return sfail(GBNTT_ERR_NOMEM, "descriptor tables allocation failed");
        }
        std::memset(sl.h_err, 0, ERR_BYTES);
    }
    s->t_first = s->t_last = Clock::now();
    s->worker = std::thread(worker_main, s);
    *out = s;
    return GBNTT_OK;
}

namespace {

// queues one request whose host buffers' device addresses are already known
int enqueue(gbntt_server* s, uint32_t plan, const void* h_in, void* h_out, uint64_t count, uint64_t* ticket,
            const void* m_in, void* m_out) {
    if (!s || !ticket) return sfail(GBNTT_ERR_ARG, "null argument");
    if (plan >= s->plans.size()) return sfail(GBNTT_ERR_ARG, "plan index out of range");
    if (!h_in || !h_out || !count) return sfail(GBNTT_ERR_ARG, "request without data");
    const size_t bytes = (size_t)count * (size_t)s->plan_bytes[plan];
    if (s->worker_error) {
        std::lock_guard<std::mutex> lk(s->mu);
        return sfail(s->worker_error, s->worker_msg);
    }
    const uint64_t t = s->next_ticket++;
    *ticket = t;
    if ((bytes + Arena::ALIGN - 1) / Arena::ALIGN * Arena::ALIGN > s->arena.capacity()) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->status[t] = GBNTT_ERR_ADMISSION;   // can never fit: refused, not queued
        ++s->refused;
        s->cv_done.notify_all();
        return GBNTT_OK;
    }
    ++s->outstanding;
    {
        std::lock_guard<std::mutex> lk(s->inbox_mu);
        s->inbox.push_back(Request{t, plan, h_in, h_out, count, bytes, Clock::now(), m_in, m_out});
    }
    s->cv_work.notify_one();
    return GBNTT_OK;
}

}  // namespace

int gbntt_server_submit(gbntt_server* s, uint32_t plan, const void* h_in, void* h_out, uint64_t count,
                        uint64_t* ticket) {
    if (!h_in || !h_out) return sfail(GBNTT_ERR_ARG, "request without data");
    return enqueue(s, plan, h_in, h_out, count, ticket, gbntt_internal_mapped(h_in),
                   const_cast<void*>(gbntt_internal_mapped(h_out)));
}

int gbntt_server_wait(gbntt_server* s, uint64_t ticket, uint32_t timeout_ms) {
    if (!s) return sfail(GBNTT_ERR_ARG, "server is null");
    std::unique_lock<std::mutex> lk(s->mu);
    const auto deadline = Clock::now() + std::chrono::milliseconds(timeout_ms);
    for (;;) {
        auto it = s->status.find(ticket);
        if (it != s->status.end()) {
            const int st = it->second;
            s->status.erase(it);
            return st == GBNTT_OK ? GBNTT_OK : sfail(st, "request refused: larger than the admission budget");
        }
        if (s->worker_error) return sfail(s->worker_error, s->worker_msg);
        if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout) {
            if (s->status.count(ticket)) continue;
            return sfail(GBNTT_ERR_TIMEOUT, "request not finished within the timeout");
        }
    }
}

int gbntt_server_drain(gbntt_server* s, uint32_t timeout_ms) {
    if (!s) return sfail(GBNTT_ERR_ARG, "server is null");
    std::unique_lock<std::mutex> lk(s->mu);
    const auto deadline = Clock::now() + std::chrono::milliseconds(timeout_ms);
    for (;;) {
        if (s->outstanding.load() == 0) return GBNTT_OK;
        if (s->worker_error) return sfail(s->worker_error, s->worker_msg);
        if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && s->outstanding.load() != 0)
            return sfail(GBNTT_ERR_TIMEOUT, "server did not drain within the timeout");
    }
}

int gbntt_server_get_stats(gbntt_server* s, gbntt_server_stats* st, int reset) {
    if (!s || !st) return sfail(GBNTT_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(st, 0, sizeof(*st));
    st->completed = s->completed;
    st->refused = s->refused;
    st->polynomials = s->polys;
    st->microbatches = s->microbatches;
    st->launches = s->launches;
    st->p50_us = percentile(s->lat_us, 50.0);
    st->p99_us = percentile(s->lat_us, 99.0);
    st->max_us = s->lat_us.empty() ? 0.0 : *std::max_element(s->lat_us.begin(), s->lat_us.end());
    const double secs = std::chrono::duration<double>(s->t_last - s->t_first).count();
    st->polys_per_s = secs > 0 ? (double)s->polys / secs : 0.0;
    st->arena_bytes = s->arena.capacity();
    st->peak_arena_bytes = s->peak_used;
    if (reset) {
        s->lat_us.clear();
        s->completed = s->refused = s->polys = s->microbatches = s->launches = 0;
        s->peak_used = 0;
        s->t_first = s->t_last = Clock::now();
    }
    return GBNTT_OK;
}

int gbntt_server_destroy(gbntt_server* s) {
    if (!s) return GBNTT_OK;
    {
        std::lock_guard<std::mutex> lk(s->inbox_mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (auto& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.fork) cudaEventDestroy(sl.fork);
        if (sl.join) cudaEventDestroy(sl.join);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.aux) cudaStreamDestroy(sl.aux);
        if (sl.h_blk) cudaFreeHost(sl.h_blk);
        if (sl.d_blk) cudaFree(sl.d_blk);
        if (sl.h_err) cudaFreeHost(sl.h_err);
        if (sl.d_ctr) cudaFree(sl.d_ctr);
    }
    if (s->d_arena) cudaFree(s->d_arena);
    delete s;
    return GBNTT_OK;
}

// Open-loop load generator: submits request i at arrival_us[i] microseconds
// after the call (busy-waiting between arrivals), from the calling thread.
int gbntt_server_submit_schedule(gbntt_server* s, uint64_t nreq, const uint32_t* plan,
                                 const void* const* h_in, void* const* h_out, const uint64_t* count,
                                 const double* arrival_us, uint64_t* tickets) {
    if (!s || (nreq && (!plan || !h_in || !h_out || !count || !arrival_us || !tickets)))
        return sfail(GBNTT_ERR_ARG, "null argument");
    // The caller keeps every buffer of the schedule alive for the whole call,
    // so each distinct buffer's device address is looked up once.
    std::unordered_map<const void*, const void*> mapped;
    auto lookup = [&](const void* h) {
        auto it = mapped.find(h);
        if (it != mapped.end()) return it->second;
        const void* m = gbntt_internal_mapped(h);
        mapped.emplace(h, m);
        return m;
    };
    for (uint64_t i = 0; i < nreq; ++i) {   // resolve before the clock starts
        if (h_in[i]) lookup(h_in[i]);
        if (h_out[i]) lookup(h_out[i]);
    }
    const auto t0 = Clock::now();
    for (uint64_t i = 0; i < nreq; ++i) {
        const auto due = t0 + std::chrono::nanoseconds((long long)(arrival_us[i] * 1000.0));
        while (Clock::now() < due) {
        }
        if (!h_in[i] || !h_out[i]) return sfail(GBNTT_ERR_ARG, "request without data");
        const int rc = enqueue(s, plan[i], h_in[i], h_out[i], count[i], &tickets[i], lookup(h_in[i]),
                               const_cast<void*>(lookup(h_out[i])));
        if (rc != GBNTT_OK) return rc;
    }
    return GBNTT_OK;
}

// Host-side self test of the admission arena and the percentile code (no CUDA).
int gbntt_server_selftest(void) {
    Arena a(4096);
    const size_t x = a.alloc(1000), y = a.alloc(1000), z = a.alloc(1000);
    if (x != 0 || y != 1024 || z != 2048 || a.used() != 3072) return sfail(GBNTT_ERR_ARG, "arena: first fit");
    if (a.alloc(2000) != SIZE_MAX) return sfail(GBNTT_ERR_ARG, "arena: over-admission");
    a.release(y, 1000);
    if (a.alloc(1024) != 1024) return sfail(GBNTT_ERR_ARG, "arena: reuse");
    a.release(x, 1000);
    a.release(1024, 1024);
    a.release(z, 1000);
    if (a.used() != 0 || a.largest_free() != 4096) return sfail(GBNTT_ERR_ARG, "arena: coalescing");
    std::vector<double> v;
    for (int i = 1; i <= 100; ++i) v.push_back(101 - i);
    if (percentile(v, 50) != 50 || percentile(v, 99) != 99 || percentile(v, 100) != 100)
        return sfail(GBNTT_ERR_ARG, "percentile");
    return GBNTT_OK;
}

}  // extern "C"
