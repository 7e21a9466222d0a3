// kernels_misc.cu -- the single-pass designs: one radix-8 stage, the
// bit-reversal unit and the full Barrett multiplication by a constant.
#include <cstdlib>

#include "device.cuh"

namespace gbntt {

namespace {

// One radix-8 stage exactly as the reference's NTT_R8 graph (butterfly tile
// src/kernels/ntt_r8_kernels.cc:214-404 + reduction tile :30-177): thread t of
// polynomial p reads x[i + M m] (M = n/8), forms y_k = sum_m x_m F8[m][k] in
// int32, reduces y_k with twiddle root^(i k) and writes the eight results
// (de-interleaved and 3-bit reversed, :152-154) as one 16-byte store at 8 i.
// W = 2: a thread takes two adjacent i (n >= 16), so its inputs arrive as
// 4-byte pairs, its twiddles as 16-byte pairs and its outputs leave as two
// 16-byte stores (65536 x 4096: 2.9 TB/s with one i per thread).
template <int W>
__global__ void __launch_bounds__(256) k_r8_stage(const KArgs a, int L) {
    grid_dep_start();
    const int n = 1 << L, M = n >> 3;
    const int GL = L - 3 - (W == 2 ? 1 : 0);             // log2 thread groups per polynomial
    const long long total = a.batch << GL;
    const short* in = static_cast<const short*>(a.in);
    short* out = static_cast<short*>(a.out);
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long poly = idx >> GL;
        const int i = (int)(idx & ((1 << GL) - 1)) * W;
        const short* src = in + poly * n + i;
        int x[W][8], y[W][8];
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            if constexpr (W == 2) {
                const int v = __ldg(reinterpret_cast<const int*>(src + m * M));
                x[0][m] = (short)(v & 0xFFFF);
                x[1][m] = v >> 16;
            } else {
                x[0][m] = __ldg(src + m * M);
            }
        }
#pragma unroll
        for (int w = 0; w < W; ++w) {
            if (a.r8_sym) {
                const int f1 = a.f8s[1], f2 = a.f8s[2], f3 = a.f8s[3];
                const int* xw = x[w];
                const int a0 = xw[0] + xw[4], a1 = xw[1] + xw[5], a2 = xw[2] + xw[6], a3 = xw[3] + xw[7];
                const int b0 = xw[0] - xw[4], b1 = xw[1] - xw[5], b2 = xw[2] - xw[6], b3 = xw[3] - xw[7];
                const int c0 = a0 + a2, c1 = a1 + a3, d0 = a0 - a2, d1 = a1 - a3;
                y[w][0] = c0 + c1;
                y[w][4] = c0 - c1;
                const int t2 = f2 * d1;
                y[w][2] = d0 + t2;
                y[w][6] = d0 - t2;
                const int e0 = b0 + f2 * b2, e1 = b0 - f2 * b2;
                const int h1 = f1 * b1 + f3 * b3, h3 = f3 * b1 + f1 * b3;
                y[w][1] = e0 + h1;
                y[w][5] = e0 - h1;
                y[w][3] = e1 + h3;
                y[w][7] = e1 - h3;
            } else {
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    int acc = 0;
#pragma unroll
                    for (int m = 0; m < 8; ++m) acc += x[w][m] * a.f8[8 * m + k];
                    y[w][k] = acc;
                }
            }
        }
        int o[W][8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            int2 t[W];
            if constexpr (W == 2) {
                const int4 tt = __ldg(reinterpret_cast<const int4*>(&a.tab[k * M + i]));
                t[0] = make_int2(tt.x, tt.y);
                t[1] = make_int2(tt.z, tt.w);
            } else {
                t[0] = __ldg(&a.tab[k * M + i]);
            }
#pragma unroll
            for (int w = 0; w < W; ++w) {
                int z = r8red(y[w][k], t[w].x, t[w].y, a.q);
                if (a.canonical) z = canon(z, a.q, a.canon_c);
                o[w][brev_c<3>(k)] = z;
            }
        }
#pragma unroll
        for (int w = 0; w < W; ++w) {
            int4 v;
            v.x = (o[w][0] & 0xFFFF) | (o[w][1] << 16);
            v.y = (o[w][2] & 0xFFFF) | (o[w][3] << 16);
            v.z = (o[w][4] & 0xFFFF) | (o[w][5] << 16);
            v.w = (o[w][6] & 0xFFFF) | (o[w][7] << 16);
            *reinterpret_cast<int4*>(out + poly * n + 8 * (i + w)) = v;
        }
    }
}

// Bit-reversal unit (src/kernels/bitreverse_kernels.cc:54-143):
// out[bitrev(i)] = in[i].  P polynomials per CTA are staged in shared memory
// with coalesced 16-byte loads, then written back in order, each thread
// reading the bit-reversed source position from shared memory.  Used for
// n < 64 and for n >= 2^13 in place (a whole polynomial per CTA); the tiled
// k_bitrev_t below, free of its bank conflicts, takes every other case.
__global__ void __launch_bounds__(256) k_bitrev(const KArgs a, int L, int P) {
    grid_dep_start();
    extern __shared__ short sb[];
    const int n = 1 << L;
    const long long poly0 = (long long)blockIdx.x * P;
    long long np = a.batch - poly0;
    if (np > P) np = P;
    const int count = (int)np << L;
    const short* src = static_cast<const short*>(a.in) + poly0 * n;
    short* dst = static_cast<short*>(a.out) + poly0 * n;
    if (n >= 8) {
        for (int j = threadIdx.x; j < count / 8; j += blockDim.x)
            reinterpret_cast<int4*>(sb)[j] = __ldg(reinterpret_cast<const int4*>(src) + j);
    } else {
        for (int j = threadIdx.x; j < count; j += blockDim.x) sb[j] = src[j];
    }
    __syncthreads();
    for (int j = threadIdx.x; j < count; j += blockDim.x) {
        const int lp = j >> L, jj = j & (n - 1);
        dst[j] = sb[(lp << L) + (int)(__brev((unsigned)jj) >> (32 - L))];
    }
}

// Bit reversal of 2^L coefficients (L >= 6) as a transpose.  With
// K = min(floor(L/2), 6), m = L - 2K middle bits and the index split as (a, b, c) --
// a the top K bits, b the m middle ones, c the bottom K -- the reversed index
// is (bitrev(c), bitrev(b), bitrev(a)): for each b, the 2^K x 2^K tile
// in[a][c] lands transposed, both indices reversed, at out[bitrev(c)][bitrev(a)].
// A CTA stages whole tiles (all of a polynomial's when m = 0, so in place is
// safe) in shared memory, one word per coefficient and rows padded by one
// word: 16-byte loads along c, 16-byte stores along the output rows, each
// side with at most 2-way bank conflicts.  128-thread CTAs let more tiles be
// in flight per SM.  (The first form read the staged polynomial at reversed
// positions, all 32 lanes on one bank: 1.14 TB/s for 65536 x 4096.)
constexpr int BR_THREADS = 128;
template <int K>
__global__ void __launch_bounds__(BR_THREADS) k_bitrev_t(const KArgs a, int L, long long ntiles) {
    grid_dep_start();
    constexpr int S = 1 << K, TE = S * S, V = TE / 8;    // 8 coefficients per 16-byte access
    constexpr int TPC = TE >= 4096 ? 1 : 4096 / TE;     // tiles per CTA
    __shared__ int tile[TPC][S][S + 1];
    const int m = L - 2 * K;
    const long long t0 = (long long)blockIdx.x * TPC;
    const short* in = static_cast<const short*>(a.in);
    short* out = static_cast<short*>(a.out);
    for (int e = threadIdx.x; e < TPC * V; e += BR_THREADS) {
        const int tt = e / V, r = e % V;
        const int row = r / (S / 8), c8 = (r % (S / 8)) * 8;
        const long long t = t0 + tt;
        if (t >= ntiles) break;
        const long long poly = t >> m;
        const int b = (int)(t & ((1 << m) - 1));
        const long long src = (poly << L) + ((long long)row << (m + K)) + ((long long)b << K) + c8;
        const int4 w = __ldg(reinterpret_cast<const int4*>(in + src));
        const int ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            tile[tt][row][c8 + 2 * h] = ws[h];             // the low half
            tile[tt][row][c8 + 2 * h + 1] = ws[h] >> 16;   // the high half
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < TPC * V; e += BR_THREADS) {
        const int tt = e / V, r = e % V;
        const int R = r / (S / 8), C8 = (r % (S / 8)) * 8;
        const long long t = t0 + tt;
        if (t >= ntiles) break;
        const long long poly = t >> m;
        const int b = (int)(t & ((1 << m) - 1));
        const int br = m ? (int)(__brev((unsigned)b) >> (32 - m)) : 0;
        const int col = (int)(__brev((unsigned)R) >> (32 - K));
        int ws[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const int lo = tile[tt][__brev((unsigned)(C8 + 2 * h)) >> (32 - K)][col];
            const int hi = tile[tt][__brev((unsigned)(C8 + 2 * h + 1)) >> (32 - K)][col];
            ws[h] = (lo & 0xFFFF) | (hi << 16);
        }
        const long long dst = (poly << L) + ((long long)R << (m + K)) + ((long long)br << K) + C8;
        *reinterpret_cast<int4*>(out + dst) = make_int4(ws[0], ws[1], ws[2], ws[3]);
    }
}

__global__ void __launch_bounds__(256) k_full_barrett(const KArgs a, long long total, int fs, int wq) {
    grid_dep_start();
    const short* in = static_cast<const short*>(a.in);
    short* out = static_cast<short*>(a.out);
    const long long nvec = total >> 3;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nvec; j += stride) {
        const int4 w = __ldg(reinterpret_cast<const int4*>(in) + j);
        int ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const int lo = fb16((int)(short)(ww[h] & 0xFFFF), fs, wq, a.q);
            const int hi = fb16(ww[h] >> 16, fs, wq, a.q);
            ww[h] = (lo & 0xFFFF) | (hi << 16);
        }
        reinterpret_cast<int4*>(out)[j] = make_int4(ww[0], ww[1], ww[2], ww[3]);
    }
    for (long long j = (nvec << 3) + (long long)blockIdx.x * blockDim.x + threadIdx.x; j < total; j += stride)
        out[j] = (short)fb16(in[j], fs, wq, a.q);
}

// grid of a grid-stride kernel: enough CTAs for the work, at most 16 per SM
int grid_for(long long work, int threads) {
    static const int sms = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    }();
    long long b = (work + threads - 1) / threads;
    const long long cap = (long long)sms * 16;
    if (b > cap) b = cap;
    return b < 1 ? 1 : (int)b;
}

}  // namespace

int bitrev_smem_bytes(int L) {
    const int n = 1 << L;
    const int P = n >= 8192 ? 1 : 8192 / n;
    return P * n * 2;
}

cudaError_t launch_r8_stage(const KArgs& a, int L, cudaStream_t s) {
    const bool pair = L >= 4;
    const long long work = a.batch << (L - 3 - (pair ? 1 : 0));
    KArgs ka = a;
    void* args[] = {&ka, &L};
    const void* fn = pair ? reinterpret_cast<const void*>(&k_r8_stage<2>) : reinterpret_cast<const void*>(&k_r8_stage<1>);
    return launch_kernel(fn, grid_for(work, 256), 256, 0, args, s, true);
}

cudaError_t launch_bitrev(const KArgs& a, int L, cudaStream_t s) {
    // buffers are 16-byte aligned (checked by the caller); beyond 2^12 a
    // polynomial's tiles spread over several CTAs, so only out of place
    if (L >= 6 && (L <= 12 || a.in != a.out)) {
        const int K = L / 2 < 6 ? L / 2 : 6;
        const long long ntiles = a.batch << (L - 2 * K);
        const int tpc = 2 * K >= 12 ? 1 : 4096 >> (2 * K);
        const unsigned grid = (unsigned)((ntiles + tpc - 1) / tpc);
        KArgs ka = a;
        int Lv = L;
        long long nt = ntiles;
        void* args[] = {&ka, &Lv, &nt};
        const void* fn = K == 3 ? reinterpret_cast<const void*>(&k_bitrev_t<3>)
                       : K == 4 ? reinterpret_cast<const void*>(&k_bitrev_t<4>)
                       : K == 5 ? reinterpret_cast<const void*>(&k_bitrev_t<5>)
                                : reinterpret_cast<const void*>(&k_bitrev_t<6>);
        return launch_kernel(fn, grid, BR_THREADS, 0, args, s, true);
    }
    const int n = 1 << L;
    const int P = n >= 8192 ? 1 : 8192 / n;
    const long long blocks = (a.batch + P - 1) / P;
    const int smem = P * n * 2;
    KArgs ka = a;
    int Lv = L, Pv = P;
    void* args[] = {&ka, &Lv, &Pv};
    return launch_kernel(reinterpret_cast<const void*>(&k_bitrev), (unsigned)blocks, 256, smem, args, s, true);
}

cudaError_t launch_full_barrett(const KArgs& a, long long total, int fs, int wq, cudaStream_t s) {
    KArgs ka = a;
    void* args[] = {&ka, &total, &fs, &wq};
    return launch_kernel(reinterpret_cast<const void*>(&k_full_barrett), grid_for((total + 7) / 8, 256), 256, 0, args,
                         s, true);
}

const void* bitrev_kernel_ptr() { return reinterpret_cast<const void*>(&k_bitrev); }

cudaError_t launch_kernel(const void* fn, unsigned grid, int threads, int smem, void** args, cudaStream_t s,
                          bool dependent) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = (size_t)smem;
    cfg.stream = s;
    cfg.attrs = dependent ? attr : nullptr;
    cfg.numAttrs = dependent ? 1 : 0;
    return cudaLaunchKernelExC(&cfg, fn, args);
}

long long large_chunk_bytes() {
    static const long long v = [] {
        const char* e = std::getenv("GBNTT_FOURSTEP_CHUNK_MB");
        const long long x = e ? std::atoll(e) : 96;
        return (x >= 8 && x <= 120 ? x : 96) << 20;
    }();
    return v;
}

}  // namespace gbntt
