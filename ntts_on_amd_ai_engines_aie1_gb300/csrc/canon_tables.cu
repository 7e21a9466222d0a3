// canon_tables.cu -- twiddle tables of the canonical families, computed on
// the device at plan creation and kept resident.
//
// Every entry is a pair (w, w') with w = root^e mod q in [0, q) and
// w' = floor(w 2^32 / q), the quotient Shoup's multiplication needs.  Each
// thread computes its entries independently (square-and-multiply with 64-bit
// products), so the tables need no host arithmetic and no upload.
#include "canon_tables.h"

namespace gbntt {

namespace {

__device__ __forceinline__ unsigned mulmod(unsigned a, unsigned b, unsigned q) {
    return (unsigned)(((unsigned long long)a * b) % q);
}

__device__ unsigned powmod_dev(unsigned b, unsigned long long e, unsigned q) {
    unsigned r = 1u % q;
    while (e) {
        if (e & 1) r = mulmod(r, b, q);
        b = mulmod(b, b, q);
        e >>= 1;
    }
    return r;
}

__device__ __forceinline__ int2 shoup_pair(unsigned w, unsigned q) {
    return make_int2((int)w, (int)(unsigned)(((unsigned long long)w << 32) / q));
}

// n entries: entry 2^B + j = root^(+-j 2^(L-1-B)) (+ forward, - inverse), the
// twiddle of the layer on bit B at low position bits j; entry 0 = 1.
__global__ void k_canon_table(int2* tab, int L, unsigned q, unsigned root, int inverse) {
    const int n = 1 << L;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned long long e = 0;
        if (i > 0) {
            const int B = 31 - __clz(i);
            const unsigned long long j = (unsigned long long)(i - (1 << B));
            e = (j << (L - 1 - B)) & (unsigned long long)(n - 1);
            if (inverse && e) e = (unsigned long long)n - e;
        }
        tab[i] = shoup_pair(powmod_dev(root, e, q), q);
    }
}

// four-step twist factors of row hi: rho = root^(s bitrev_{L1}(hi)) for the
// forward transform (root^-... for the inverse), split as rho^s = A[hi][s mod G]
// * B[hi][s div G] with G = 2^(L2 - EL) (thread part) and E = 2^EL (register
// part): A at [hi * G + t], B after all A entries at [2^L1 G + hi * E + k].
__global__ void k_canon_twist(int2* tab, int L1, int L2, int EL, unsigned q, unsigned root, int inverse) {
    const int G = 1 << (L2 - EL), E = 1 << EL, R = 1 << L1;
    const unsigned long long n = 1ull << (L1 + L2);
    const int count = R * (G + E);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        int hi;
        unsigned long long s;
        if (i < R * G) {
            hi = i / G;
            s = (unsigned long long)(i % G);
        } else {
            hi = (i - R * G) / E;
            s = (unsigned long long)((i - R * G) % E) * G;
        }
        const unsigned long long b = L1 ? (__brev((unsigned)hi) >> (32 - L1)) : 0;
        unsigned long long e = (b * s) % n;
        if (inverse && e) e = n - e;
        tab[i] = shoup_pair(powmod_dev(root, e, q), q);
    }
}

int grid_of(long long count) {
    long long b = (count + 255) / 256;
    return (int)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

}  // namespace

size_t canon_table_entries(int L, bool) { return (size_t)1 << L; }

cudaError_t make_canon_table(int2* d_tab, int L, uint32_t q, uint32_t root, bool inverse, cudaStream_t s) {
    k_canon_table<<<grid_of((long long)canon_table_entries(L, inverse)), 256, 0, s>>>(d_tab, L, q, root,
                                                                                    inverse ? 1 : 0);
    return cudaGetLastError();
}

size_t canon_twist_entries(int L1, int L2, int EL) { return ((size_t)1 << L1) * (((size_t)1 << (L2 - EL)) + ((size_t)1 << EL)); }

cudaError_t make_canon_twist(int2* d_tab, int L1, int L2, int EL, uint32_t q, uint32_t root, bool inverse,
                             cudaStream_t s) {
    k_canon_twist<<<grid_of((long long)canon_twist_entries(L1, L2, EL)), 256, 0, s>>>(d_tab, L1, L2, EL, q, root,
                                                                                     inverse ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace gbntt
