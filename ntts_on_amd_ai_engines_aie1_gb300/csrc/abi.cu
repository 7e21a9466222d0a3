// abi.cu -- the C ABI of libgb300ntt.so (declared in include/gb300_ntt.h).
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "../../include/gb300_ntt.h"
#include "batch_kernel.cuh"
#include "canon_tables.h"
#include "device.cuh"
#include "plan_internal.h"
#include "tables.h"

namespace gbntt {
const void* bitrev_kernel_ptr();
}

using namespace gbntt;

struct gbntt_plan {
    HostPlan hp;
    int fam = -1;          // transform family of k_ntt, -1 for the single-purpose kernels
    bool br = false;       // bit-reversed load and store (radix-4 inverse)
    KernelInfo ki;
    KernelInfo kl;         // latency form for launches of at most one CTA per SM (fn nullptr: none)
    LargeInfo large;       // int32 n >= 2^16: two-pass schedule (large.cols != nullptr)
    CanonLarge clarge;     // canonical int32 n >= 2^16: four-step (clarge.cols != nullptr)
    const int2* tab_rows = nullptr;   // four-step: the row transforms' table (inside d_tab)
    const int2* twist = nullptr;      // four-step: twist factors (inside d_tab)
    unsigned* d_err = nullptr;        // four-step: set when a bounded wait ran out
    KArgs base;            // constants shared by every launch
    int2* d_tab = nullptr;
    size_t tab_bytes = 0;
    int device = 0;
    std::mutex stage_mu;   // serialises gbntt_execute_host on this plan
    void* d_stage = nullptr;
    size_t stage_bytes = 0;
    void* zc_state = nullptr;   // zero-copy scratch (batch.cu), created on first use
};

namespace {

thread_local std::string g_err;
std::atomic<unsigned long long> g_launches{0};

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return GBNTT_ERR_CUDA;
}

int family_of(int kind) {
    switch (kind) {
    case K_R2_I16_FWD: return F_R2F16;
    case K_R2_I16_INV: return F_R2I16;
    case K_R4_I16_FWD: return F_R4F16;
    case K_R4_I16_INV: return F_R4F16;
    case K_R8_I16_FWD: return F_R8F16;
    case K_R2_I32_FWD: return F_R2F32;
    case K_R2_I32_INV: return F_R2G32;
    default: return -1;
    }
}

KernelInfo kernel_for(int fam, int L, bool br, bool lat) {
    if (fam_canon(fam)) return kinfo_canon(fam, L, lat);
    switch (fam) {
    case F_R2F16: return kinfo_r2f16(L, lat);
    case F_R2I16: return kinfo_r2i16(L, lat);
    case F_R4F16: return kinfo_r4(L, br, lat);
    case F_R8F16: return kinfo_r8(L, lat);
    case F_R2F32: return kinfo_r2f32(L, lat);
    case F_R2G32: return kinfo_r2g32(L, lat);
    default: return KernelInfo();
    }
}

// Canonical int32 lengths from 2^L on run as the four-step (two passes);
// shorter ones (up to 2^15) in one CTA per polynomial.  GBNTT_FOURSTEP_MIN_L
// (14 .. 16) overrides the default, read once per process.
int fourstep_min_L() {
    static const int v = [] {
        const char* e = std::getenv("GBNTT_FOURSTEP_MIN_L");
        const int x = e ? std::atoi(e) : 16;
        return x >= 14 && x <= 16 ? x : 16;
    }();
    return v;
}

int launch(const gbntt_plan* p, const void* d_in, void* d_out, uint64_t batch, cudaStream_t s) {
    KArgs a = p->base;
    a.in = d_in;
    a.out = d_out;
    a.batch = (long long)batch;
    cudaError_t e = cudaSuccess;
    if (p->clarge.cols) {
        const bool inverse = (p->hp.kind == K_R2_I32_INV);
        int nl = 0;
        e = launch_canon_large(p->clarge, a, p->d_tab, p->tab_rows, p->twist, d_in, d_out, (long long)batch, inverse,
                               p->d_err, s, &nl);
        if (e != cudaSuccess) return cuda_fail(e, "four-step launch");
        g_launches.fetch_add((unsigned long long)nl, std::memory_order_relaxed);
        return GBNTT_OK;
    } else if (p->large.cols) {
        // two passes per chunk of polynomials; a chunk (large_chunk_bytes())
        // stays in L2 between its passes.  Forward: columns then rows; inverse:
        // rows first.  Programmatic dependent launches (grid_dep_start).
        const LargeInfo& li = p->large;
        const long long n = (long long)p->hp.n;
        long long chunk = large_chunk_bytes() / (n * 4);
        if (chunk < 1) chunk = 1;
        const bool inverse = (p->hp.kind == K_R2_I32_INV);
        for (long long p0 = 0; p0 < (long long)batch; p0 += chunk) {
            const long long np = std::min<long long>(chunk, (long long)batch - p0);
            KArgs first = a, last = a;
            first.in = static_cast<const int*>(d_in) + p0 * n;
            first.out = static_cast<int*>(d_out) + p0 * n;
            first.batch = np;
            first.canonical = 0;    // the epilogue belongs to the last pass only
            first.scale = 0;
            last.in = first.out;
            last.out = first.out;
            last.batch = np;
            int L1 = li.L1, L2 = li.L2;
            void* cargs_first[] = {&first, &L2};
            void* rargs_first[] = {&first, &L1};
            void* cargs_last[] = {&last, &L2};
            void* rargs_last[] = {&last, &L1};
            const unsigned cgrid = (unsigned)(np * ((1LL << li.L2) / li.cols_per_cta));
            const unsigned rgrid = (unsigned)(((np << li.L1) + li.rows_per_cta - 1) / li.rows_per_cta);
            auto cols = [&](void** args) {
                return launch_kernel(li.cols, cgrid, li.cols_threads, li.cols_smem, args, s, true);
            };
            auto rows = [&](void** args) {
                return launch_kernel(li.rows, rgrid, li.rows_threads, li.rows_smem, args, s, true);
            };
            if (!inverse) {
                e = cols(cargs_first);
                if (e == cudaSuccess) e = rows(rargs_last);
            } else {
                e = rows(rargs_first);
                if (e == cudaSuccess) e = cols(cargs_last);
            }
            if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
            g_launches.fetch_add(2, std::memory_order_relaxed);
        }
        return GBNTT_OK;
    } else if (p->fam >= 0) {
        // A launch of at most one CTA per SM is latency-bound: it takes the
        // latency form (one polynomial per CTA over up to 256 threads) where
        // the design has one, and its CTAs pull the table into L1 up front (a
        // large launch finds it there already, and the extra prefetches
        // measured 6-8 % slower for int32 and radix-8).
        static const int sms = [] {
            int dev = 0, n = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
            return n > 0 ? n : 1;
        }();
        const bool small = batch <= (uint64_t)sms;
        const KernelInfo& k = small && p->kl.fn ? p->kl : p->ki;
        const unsigned long long blocks = (batch + k.polys - 1) / k.polys;
        if (blocks > 0x7FFFFFFFull) return fail(GBNTT_ERR_ARG, "batch too large for one launch");
        a.tab_bytes = blocks <= (unsigned long long)sms ? (int)p->tab_bytes : 0;
        void* args[] = {&a};
        e = launch_kernel(k.fn, (unsigned)blocks, k.threads, k.smem, args, s, true);
    } else if (p->hp.kind == K_R8_I16_STAGE) {
        e = launch_r8_stage(a, p->hp.L, s);
    } else if (p->hp.kind == K_BITREV_I16) {
        e = launch_bitrev(a, p->hp.L, s);
    } else if (p->hp.kind == K_FULL_BARRETT_I16) {
        e = launch_full_barrett(a, (long long)batch * p->hp.n, p->hp.fb_fs, p->hp.fb_wq, s);
    }
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return GBNTT_OK;
}

}  // namespace

int gbntt_internal_fail(int code, const std::string& msg) { return fail(code, msg); }

void gbntt_internal_count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int gbntt_internal_plan_L(const gbntt_plan* p) { return p ? p->hp.L : 0; }

void gbntt_internal_plan_args(const gbntt_plan* p, int* fam, int* L, int* elem_bytes, KArgs* a) {
    *fam = p->br ? -1 : p->fam;
    *L = p->hp.L;
    *elem_bytes = p->hp.elem_bytes;
    *a = p->base;
}

const void* gbntt_internal_mapped(const void* h) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
        cudaGetLastError();   // an unknown pointer is an answer, not an error
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

extern "C" {

int gbntt_abi_version(void) { return GBNTT_ABI_VERSION; }

const char* gbntt_last_error(void) { return g_err.c_str(); }

uint64_t gbntt_launch_count(void) { return g_launches.load(); }

const char* gbntt_status_string(int status) {
    switch (status) {
    case GBNTT_OK: return "ok";
    case GBNTT_ERR_ARG: return "invalid argument";
    case GBNTT_ERR_LENGTH: return "unsupported length";
    case GBNTT_ERR_MODULUS: return "invalid modulus";
    case GBNTT_ERR_ROOT: return "root of unity has the wrong order";
    case GBNTT_ERR_LAYERS: return "radix-4 needs an even number of layers";
    case GBNTT_ERR_KIND: return "unknown design kind";
    case GBNTT_ERR_CUDA: return "CUDA error";
    case GBNTT_ERR_NOMEM: return "out of memory";
    case GBNTT_ERR_TIMEOUT: return "timeout";
    case GBNTT_ERR_ADMISSION: return "admission refused";
    default: return "unknown status";
    }
}

int gbntt_host_tables(int kind, uint32_t n, int64_t q, int64_t root, int64_t factor, uint32_t flags,
                      int which, int64_t* dst, int64_t cap, int64_t* len) {
    HostPlan hp;
    std::string err;
    const int rc = build_host_plan(kind, n, q, root, factor, flags, hp, err);
    if (rc != GBNTT_OK) return fail(rc, err);
    std::vector<int64_t> v;
    if (which == 0) {
        v.assign(hp.tab.begin(), hp.tab.end());
    } else if (which == 1) {
        v = {hp.c, hp.r4_fneg, hp.r4_wc, hp.fb_fs, hp.fb_wq, hp.tail_wq, hp.tail_bits, hp.r8_sym, hp.stages};
    } else if (which == 2) {
        v.assign(hp.f8, hp.f8 + 64);
    } else {
        return fail(GBNTT_ERR_ARG, "unknown table selector");
    }
    if (len) *len = (int64_t)v.size();
    if (dst)
        for (int64_t i = 0; i < (int64_t)v.size() && i < cap; ++i) dst[i] = v[i];
    return GBNTT_OK;
}

int gbntt_plan_create(gbntt_plan** out, int kind, uint32_t n, int64_t q, int64_t root, int64_t factor,
                      uint32_t flags) {
    if (!out) return fail(GBNTT_ERR_ARG, "plan pointer is null");
    *out = nullptr;
    gbntt_plan* p = new (std::nothrow) gbntt_plan();
    if (!p) return fail(GBNTT_ERR_NOMEM, "host allocation failed");
    std::string err;
    int rc = build_host_plan(kind, n, q, root, factor, flags, p->hp, err);
    if (rc != GBNTT_OK) {
        delete p;
        return fail(rc, err);
    }
    const HostPlan& hp = p->hp;
    // GBNTT_FLAG_CANONICAL without GBNTT_FLAG_LANE_EXACT: the canonical family
    // of the design's direction and storage type (the two-pass int32 lengths
    // keep the reference's lane arithmetic plus the final reduction)
    const bool canon = canonical_fast(kind, hp.q, flags);
    p->fam = canon ? canonical_family(kind) : family_of(kind);
    p->br = !canon && (kind == K_R4_I16_INV);
    if (canon && hp.elem_bytes == 4 && hp.L >= fourstep_min_L() &&
        (hp.L >= 16 || !(flags & FLAG_NATURAL_ORDER))) {   // the four-step has no natural-order form
        p->clarge = canon_large_info(p->fam, hp.L);
        if (!p->clarge.cols) {
            delete p;
            return fail(GBNTT_ERR_LENGTH, "no kernel for this length");
        }
    } else if (p->fam >= 0 && hp.L >= 16) {
        p->large = large_info(p->fam, hp.L);
        if (!p->large.cols) {
            delete p;
            return fail(GBNTT_ERR_LENGTH, "no kernel for this length");
        }
    } else if (p->fam >= 0) {
        p->ki = kernel_for(p->fam, hp.L, p->br, false);
        p->kl = kernel_for(p->fam, hp.L, p->br, true);
        if (!p->ki.fn) {
            delete p;
            return fail(GBNTT_ERR_LENGTH, "no kernel for this length");
        }
    }
    cudaError_t e = cudaGetDevice(&p->device);
    if (e != cudaSuccess) {
        delete p;
        return cuda_fail(e, "cudaGetDevice");
    }
    if (p->fam >= 0 && p->ki.smem > 48 * 1024) {
        e = cudaFuncSetAttribute(p->ki.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, p->ki.smem);
        if (e != cudaSuccess) {
            delete p;
            return cuda_fail(e, "cudaFuncSetAttribute");
        }
    }
    if (p->clarge.cols) {
        e = raise_smem_limit(p->clarge.cols, p->clarge.cols_smem);
        if (e == cudaSuccess) e = raise_smem_limit(p->clarge.rows, p->clarge.rows_smem);
        if (e != cudaSuccess) {
            delete p;
            return cuda_fail(e, "cudaFuncSetAttribute");
        }
    }
    if (p->large.cols) {
        e = cudaFuncSetAttribute(p->large.cols, cudaFuncAttributeMaxDynamicSharedMemorySize, p->large.cols_smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(p->large.rows, cudaFuncAttributeMaxDynamicSharedMemorySize, p->large.rows_smem);
        if (e != cudaSuccess) {
            delete p;
            return cuda_fail(e, "cudaFuncSetAttribute");
        }
    }
    if (kind == K_BITREV_I16 && bitrev_smem_bytes(hp.L) > 48 * 1024) {
        e = raise_smem_limit(bitrev_kernel_ptr(), bitrev_smem_bytes(hp.L));
        if (e != cudaSuccess) {
            delete p;
            return cuda_fail(e, "cudaFuncSetAttribute");
        }
    }
    // int16 radix-2/4 designs: (tw, w') packed into one word (both fit int16)
    const bool packed = (p->fam == F_R2F16 || p->fam == F_R2I16 || p->fam == F_R4F16);
    const bool inverse = (kind == K_R2_I16_INV || kind == K_R2_I32_INV || kind == K_R4_I16_INV);
    std::vector<int32_t> dev_tab;
    if (canon) {
        // canonical families: (w, w') pairs computed on the device; the
        // four-step holds the column and row transforms' tables and the twist
        const CanonLarge& cl = p->clarge;
        size_t n_cols = canon_table_entries(hp.L, inverse), n_rows = 0, n_twist = 0;
        if (cl.cols) {
            n_cols = canon_table_entries(cl.L1, inverse);
            n_rows = canon_table_entries(cl.L2, inverse);
            n_twist = canon_twist_entries(cl.L1, cl.L2, cl.row_el);
        }
        p->tab_bytes = (n_cols + n_rows + n_twist) * sizeof(int2);
        e = cudaMalloc(&p->d_tab, p->tab_bytes);
        if (e == cudaSuccess && cl.cols) e = cudaMalloc(&p->d_err, 256);
        if (e != cudaSuccess) {
            if (p->d_tab) cudaFree(p->d_tab);
            delete p;
            return e == cudaErrorMemoryAllocation ? fail(GBNTT_ERR_NOMEM, "device allocation failed")
                                                  : cuda_fail(e, "cudaMalloc");
        }
        const uint32_t q32 = (uint32_t)hp.q;
        if (cl.cols) {
            const int64_t n1 = (int64_t)1 << cl.L1, n2 = (int64_t)1 << cl.L2;
            p->tab_rows = p->d_tab + n_cols;
            p->twist = p->d_tab + n_cols + n_rows;
            e = make_canon_table(p->d_tab, cl.L1, q32, (uint32_t)powmod(hp.root, (uint64_t)n2, hp.q), inverse, 0);
            if (e == cudaSuccess)
                e = make_canon_table(p->d_tab + n_cols, cl.L2, q32, (uint32_t)powmod(hp.root, (uint64_t)n1, hp.q),
                                     inverse, 0);
            if (e == cudaSuccess)
                e = make_canon_twist(p->d_tab + n_cols + n_rows, cl.L1, cl.L2, cl.row_el, q32, (uint32_t)hp.root,
                                     inverse, 0);
            if (e == cudaSuccess) e = cudaMemsetAsync(p->d_err, 0, 256, 0);
        } else {
            e = make_canon_table(p->d_tab, hp.L, q32, (uint32_t)hp.root, inverse, 0);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(0);
        if (e != cudaSuccess) {
            cudaFree(p->d_tab);
            if (p->d_err) cudaFree(p->d_err);
            delete p;
            return cuda_fail(e, "canonical table");
        }
    } else if (packed) {
        dev_tab.resize(hp.tab.size() / 2);
        for (size_t i = 0; i < dev_tab.size(); ++i)
            dev_tab[i] = (int32_t)(((uint32_t)hp.tab[2 * i] & 0xFFFFu) | ((uint32_t)hp.tab[2 * i + 1] << 16));
    } else {
        dev_tab = hp.tab;
    }
    if (!dev_tab.empty()) {
        p->tab_bytes = dev_tab.size() * sizeof(int32_t);
        e = cudaMalloc(&p->d_tab, p->tab_bytes);
        if (e != cudaSuccess) {
            delete p;
            return e == cudaErrorMemoryAllocation ? fail(GBNTT_ERR_NOMEM, "device allocation failed")
                                                  : cuda_fail(e, "cudaMalloc");
        }
        e = cudaMemcpy(p->d_tab, dev_tab.data(), p->tab_bytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(p->d_tab);
            delete p;
            return cuda_fail(e, "cudaMemcpy (tables)");
        }
    }
    KArgs& a = p->base;
    std::memset(&a, 0, sizeof(a));
    a.tab = packed ? nullptr : p->d_tab;
    a.tab16 = packed ? reinterpret_cast<const int*>(p->d_tab) : nullptr;
    a.wq1 = (p->fam == F_R4F16 && hp.tab.size() >= 2) ? hp.tab[1] : 0;
    a.q = (int)hp.q;
    a.c = hp.c;
    a.fneg = hp.r4_fneg;
    a.wc = hp.r4_wc;
    a.canonical = (flags & FLAG_CANONICAL) ? 1 : 0;
    a.canon_c = hp.q >= 3 ? (int)((((uint64_t)1 << 32) + hp.q / 2) / hp.q) : 0;
    if (canon) {
        a.canonical = 1;
        a.cq = (unsigned)((((uint64_t)1) << 32) / (uint64_t)hp.q);
        if (hp.elem_bytes == 2) {
            const int64_t m = hp.q * ((32768 + hp.q - 1) / hp.q);     // a multiple of q, >= 2^15
            a.in_off = (int)(2 * m);
        } else {
            a.in_off = (int)(hp.q - ((int64_t)1 << 31) % hp.q);      // residue of -2^31, in (0, q]
        }
        const uint64_t ninv = (uint64_t)modinv((int64_t)hp.n, hp.q);
        a.ninv = (unsigned)ninv;
        a.ninv_q = (unsigned)((ninv << 32) / (uint64_t)hp.q);
    }
    a.natural_in = ((flags & FLAG_NATURAL_ORDER) && inverse) ? 1 : 0;
    a.natural_out = ((flags & FLAG_NATURAL_ORDER) && !inverse) ? 1 : 0;
    a.scale = (flags & FLAG_SCALE_NINV) ? 1 : 0;
    a.fb_fs = hp.fb_fs;
    a.fb_wq = hp.fb_wq;
    a.r8_sym = hp.r8_sym;
    // radix-8: the multiplier of the twiddle 1, also for the k = 0 outputs of
    // every stage (table entry 0 is that twiddle, in the plan's w' mode)
    a.tail_wq = (p->fam == F_R8F16 && hp.tab.size() >= 2) ? hp.tab[1] : hp.tail_wq;
    for (int i = 0; i < 64; ++i) a.f8[i] = hp.f8[i];
    for (int i = 0; i < 4; ++i) a.f8s[i] = hp.f8s[i];
    for (int i = 0; i < 16; ++i) a.ftail[i] = hp.ftail[i];
    *out = p;
    return GBNTT_OK;
}

int gbntt_plan_destroy(gbntt_plan* p) {
    if (!p) return GBNTT_OK;
    if (p->d_tab) cudaFree(p->d_tab);
    if (p->d_err) cudaFree(p->d_err);
    if (p->d_stage) cudaFree(p->d_stage);
    if (p->zc_state) gbntt_internal_zc_free(p->zc_state);
    delete p;
    return GBNTT_OK;
}

int gbntt_plan_status(const gbntt_plan* p) {
    if (!p) return fail(GBNTT_ERR_ARG, "plan is null");
    if (!p->d_err) return GBNTT_OK;
    unsigned w = 0;
    cudaError_t e = cudaMemcpy(&w, p->d_err, sizeof(w), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "status read");
    if (!w) return GBNTT_OK;
    e = cudaMemset(p->d_err, 0, sizeof(w));
    if (e != cudaSuccess) return cuda_fail(e, "status reset");
    return fail(GBNTT_ERR_TIMEOUT, "a tile load of the four-step column pass did not arrive within the wait limit");
}

int gbntt_plan_query(const gbntt_plan* p, int what, int64_t* value) {
    if (!p || !value) return fail(GBNTT_ERR_ARG, "null argument");
    switch (what) {
    case GBNTT_Q_N: *value = p->hp.n; break;
    case GBNTT_Q_MODULUS: *value = p->hp.q; break;
    case GBNTT_Q_ELEM_BYTES: *value = p->hp.elem_bytes; break;
    case GBNTT_Q_STAGES: *value = p->hp.stages; break;
    case GBNTT_Q_KIND: *value = p->hp.kind; break;
    case GBNTT_Q_TABLE_BYTES: *value = (int64_t)p->tab_bytes; break;
    default: return fail(GBNTT_ERR_ARG, "unknown query");
    }
    return GBNTT_OK;
}

int gbntt_execute(const gbntt_plan* p, const void* d_in, void* d_out, uint64_t batch, void* stream) {
    if (!p) return fail(GBNTT_ERR_ARG, "plan is null");
    if (batch == 0) return GBNTT_OK;
    if (!d_in || !d_out) return fail(GBNTT_ERR_ARG, "null buffer");
    if ((reinterpret_cast<uintptr_t>(d_in) | reinterpret_cast<uintptr_t>(d_out)) & 15)
        return fail(GBNTT_ERR_ARG, "device buffers must be 16-byte aligned");
    if (p->hp.kind == K_R8_I16_STAGE && d_in == d_out)
        return fail(GBNTT_ERR_ARG, "the radix-8 stage cannot run in place");
    return launch(p, d_in, d_out, batch, static_cast<cudaStream_t>(stream));
}

int gbntt_execute_host(gbntt_plan* p, const void* h_in, void* h_out, uint64_t batch, void* stream) {
    if (!p) return fail(GBNTT_ERR_ARG, "plan is null");
    if (batch == 0) return GBNTT_OK;
    if (!h_in || !h_out) return fail(GBNTT_ERR_ARG, "null buffer");
    std::lock_guard<std::mutex> lock(p->stage_mu);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    {
        // page-locked, mapped host buffers: the zero-copy persistent kernel reads
        // and writes them directly, both directions of the link at once
        const void* mi = gbntt_internal_mapped(h_in);
        const void* mo = gbntt_internal_mapped(h_out);
        if (mi && mo && !((reinterpret_cast<uintptr_t>(mi) | reinterpret_cast<uintptr_t>(mo)) & 15) &&
            !(p->hp.kind == K_R8_I16_STAGE && h_in == h_out)) {
            const int rc = gbntt_internal_zc_plan(&p->zc_state, p, mi, const_cast<void*>(mo), batch, s);
            if (rc == GBNTT_OK) {
                const cudaError_t e = cudaStreamSynchronize(s);
                return e == cudaSuccess ? GBNTT_OK : cuda_fail(e, "cudaStreamSynchronize");
            }
            if (rc != GBNTT_ERR_KIND) return rc;
        }
    }
    const size_t bytes = (size_t)batch * p->hp.n * (size_t)p->hp.elem_bytes;
    // the radix-8 stage reads other threads' outputs, so it gets its own output half
    const bool split = (p->hp.kind == K_R8_I16_STAGE);
    const size_t need = split ? 2 * bytes : bytes;
    cudaError_t e;
    if (p->stage_bytes < need) {
        if (p->d_stage) cudaFree(p->d_stage);
        p->d_stage = nullptr;
        p->stage_bytes = 0;
        e = cudaMalloc(&p->d_stage, need);
        if (e != cudaSuccess) return fail(GBNTT_ERR_NOMEM, "staging allocation failed");
        p->stage_bytes = need;
    }
    void* d_out = split ? static_cast<char*>(p->d_stage) + bytes : p->d_stage;
    e = cudaMemcpyAsync(p->d_stage, h_in, bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync H2D");
    int rc = launch(p, p->d_stage, d_out, batch, s);
    if (rc != GBNTT_OK) return rc;
    e = cudaMemcpyAsync(h_out, d_out, bytes, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync D2H");
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    return GBNTT_OK;
}

}  // extern "C"
