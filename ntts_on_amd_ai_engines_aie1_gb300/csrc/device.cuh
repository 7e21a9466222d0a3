// device.cuh -- sm_103a device code of the GB300 NTT library.
//
// The reference runs one radix-2 (radix-4, radix-8) layer per AIE tile in
// constant geometry (Pease): every tile reads positions j and j + n/2 and
// writes 2j, 2j + 1.  Constant geometry only moves data between tiles; the
// arithmetic of every butterfly is fixed by which values meet, with which
// twiddle, and where the partial Barrett reductions sit.  These kernels
// therefore run the same butterflies in place, in registers: a group of G
// threads owns one polynomial of n = 2^L coefficients, each thread holds
// E = 2^EL of them, and a "window" of EL position bits is resident in each
// thread at a time.  All layers whose butterfly bits lie in the window run in
// registers; between windows the polynomial is exchanged through shared
// memory.  The values computed are bit-identical to the reference's:
//   * partial Barrett with K = 16 / 32 / 31 and rounding of the SRS unit in
//     symmetric_zero mode (nearest, ties toward zero);
//   * int16 / int32 two's-complement wrap wherever the AIE code stores to
//     int16 / int32 lanes (saturation mode none).
// The canonical families (F_C16F ... F_C32I) run the same transforms with
// their own arithmetic instead: Shoup multiplication by precomputed quotients
// and lazily reduced 32-bit lanes, reduced to [0, q) once at the end (see
// "canonical arithmetic" below).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <utility>

namespace gbntt {

// F_R2F16 ... F_R2G32: the reference's lane arithmetic (partially reduced
// outputs, bit for bit).  F_C16F ... F_C32I: canonical arithmetic, forward
// (natural order in, bit-reversed out) and inverse (bit-reversed in, natural
// out, no n^-1), int16 or int32 storage; every forward design of the reference
// computes the forward transform's residues and every inverse design the
// inverse's, so one canonical family per direction and storage type serves
// them all.
enum Fam {
    F_R2F16 = 0, F_R2I16 = 1, F_R4F16 = 2, F_R8F16 = 3, F_R2F32 = 4, F_R2G32 = 5,
    F_C16F = 6, F_C16I = 7, F_C32F = 8, F_C32I = 9, F_NUM = 10
};
__host__ __device__ constexpr bool fam_canon(int fam) { return fam >= F_C16F && fam <= F_C32I; }

// Programmatic dependent launch.  The library's per-plan launches (every
// design's kernel, the two passes of a long transform and its chunks; not the
// persistent batch kernels) carry the programmatic-stream-serialization
// attribute, so when the previous operation is a grid that has signalled
// launch_dependents, their CTAs take the SM slots its last CTAs free, with no
// launch gap.  Every such kernel starts with grid_dep_start(): it signals its
// own dependents (safe this early: their wait covers this whole grid and its
// memory operations) and waits for the previous grid's completion and results
// before touching global memory.  After any other operation, or without the
// attribute, the launch is ordered as usual and both instructions are no-ops.
__device__ __forceinline__ void grid_dep_start() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Per-launch arguments (by value; the kernel reads the constants from the
// parameter bank).
struct KArgs {
    const void* in;
    void* out;
    long long batch;
    const int2* tab;      // (tw, w') pairs of the design (int32 designs, radix-8)
    const int* tab16;     // int16 designs: tw | w' << 16 packed in one word
    int wq1;              // radix-4: multiplier of the twiddle 1 (table entry 0)
    int q;
    int c;                // Barrett constant of the reduction (K = 16 or 32)
    int fneg, wc;         // radix-4 omega_4 and its multiplier
    int canonical;        // reduce outputs to [0, q)
    int canon_c;          // its Barrett constant round(2^32 / q)
    int natural_in;       // input in natural order (inverse designs): bit reversal fused into the load
    int natural_out;      // output in natural order (forward designs): bit reversal fused into the store
    int scale;            // inverse designs: full Barrett multiplication by n^-1 fused into the store
    int fb_fs, fb_wq;     // its signed factor and multiplier
    int r8_sym;           // radix-8 matrix symmetric: use the factored butterfly
    int tail_wq;          // radix-8: multiplier of the twiddle 1 (output 0 of every stage, the tail stage)
    int tab_bytes;        // per-plan launch: table bytes to prefetch into L1 first (0: none)
    int f8[64];           // radix-8 matrix [m][k]
    int f8s[4];           // f1, f2, f3
    int ftail[16];        // tail matrix [m][k]
    // canonical families (tab: (w, floor(w 2^32 / q)) pairs)
    unsigned cq;          // floor(2^32 / q)
    int in_off;           // int16: 2M, M = q ceil(2^15 / q); int32: q - (2^31 mod q)
    unsigned ninv, ninv_q;   // n^-1 mod q and its Shoup quotient (n^-1 scaling of inverse designs)
    const int2* twist;    // four-step row twist factors (two-pass canonical int32 transforms)
};

// The scalar constants of one design, held in registers while a polynomial is
// transformed (the matrices stay in parameter or shared memory).
struct KC {
    const int2* tab;
    const int* tab16;
    const int* f8;
    const int* ftail;
    int q, c, fneg, wc, r8_sym, tail_wq, f1, f2, f3, wq1;
    int in_off;
};

__device__ __forceinline__ KC make_kc(const KArgs& a) {
    KC k;
    k.tab = a.tab;
    k.tab16 = a.tab16;
    k.wq1 = a.wq1;
    k.f8 = a.f8;
    k.ftail = a.ftail;
    k.q = a.q;
    k.c = a.c;
    k.fneg = a.fneg;
    k.wc = a.wc;
    k.r8_sym = a.r8_sym;
    k.tail_wq = a.tail_wq;
    k.f1 = a.f8s[1];
    k.f2 = a.f8s[2];
    k.f3 = a.f8s[3];
    k.in_off = a.in_off;
    return k;
}

// ---------------------------------------------------------------------------
// lane arithmetic
// ---------------------------------------------------------------------------

// round(p / 2^16), ties toward zero (SRS, symmetric_zero)
__device__ __forceinline__ int rsz16(int p) { return (p + 0x7FFF + (int)((unsigned)p >> 31)) >> 16; }

// round(p / 2^32), ties toward zero
__host__ __device__ __forceinline__ int rsz32(long long p) {
    return (int)((p + 0x7FFFFFFFLL + (long long)((unsigned long long)p >> 63)) >> 32);
}

// round(p / 2^31), ties toward zero
__device__ __forceinline__ int rsz31(long long p) {
    return (int)((p + 0x3FFFFFFFLL + (long long)((unsigned long long)p >> 63)) >> 31);
}

__device__ __forceinline__ int wrap16(int x) { return (int)(short)x; }
// halves of a packed (tw | w' << 16) table word
__device__ __forceinline__ int lo16(int w) { return (int)(short)w; }
__device__ __forceinline__ int hi16(int w) { return w >> 16; }

// Partial Barrett reduction / multiplication, int16: a - round(a c / 2^16) q
// and a w - round(a w' / 2^16) q.  The reference stores both results as int16
// lanes (a wrap), which never changes them: every multiplier of the tables is
// within 1.5 of w 2^16 / q (0.5 for the float and constant ones, < 1.5 for
// round<T>'s truncation of negative values), so for |a| <= 2^15 the quotient
// error is at most 0.5 + 0.75 and |result| <= 1.25 q < 2^15 for q < 2^16 / 3.
__device__ __forceinline__ int br16(int a, int c, int q) { return a - rsz16(a * c) * q; }
__device__ __forceinline__ int bm16(int a, int tw, int wq, int q) { return a * tw - rsz16(a * wq) * q; }
// The same product when only its low 16 bits are used (it feeds sums that are
// wrapped to int16): the packed table word t = (tw & 0xFFFF) | (w' << 16)
// multiplies like tw modulo 2^16, so tw need not be sign-extended out of it.
__device__ __forceinline__ unsigned bm16_lo(int a, int t, int q) {
    return (unsigned)a * (unsigned)t - (unsigned)rsz16(a * hi16(t)) * (unsigned)q;
}

// int32 variants, computed modulo 2^32 like the int32 lanes
__host__ __device__ __forceinline__ int br32(int a, int c, int q) {
    return (int)((unsigned)a - (unsigned)rsz32((long long)a * c) * (unsigned)q);
}
__device__ __forceinline__ int bm32(int a, int tw, int wq, int q) {
    return (int)((unsigned)a * (unsigned)tw - (unsigned)rsz32((long long)a * wq) * (unsigned)q);
}
__device__ __forceinline__ int add32(int a, int b) { return (int)((unsigned)a + (unsigned)b); }
__device__ __forceinline__ int sub32(int a, int b) { return (int)((unsigned)a - (unsigned)b); }

// radix-8 reduction tile: m' = round(y w' / 2^31) truncated to int16, then
// y w - m' q kept as int16 (ntt_r8_kernels.cc:30-177)
__device__ __forceinline__ int r8red(int y, int tw, int wq, int q) {
    const int m16 = (int)(short)rsz31((long long)y * wq);
    return wrap16((int)((unsigned)y * (unsigned)tw - (unsigned)m16 * (unsigned)q));
}

// Full Barrett multiplication by a constant, fully reduced
// (src/kernels/full_reduction_kernels.cc:33-195).
__device__ __forceinline__ int fb16(int x, int fs, int wq, int q) {
    const int mb = wrap16(rsz16(x * wq));     // m' = SRS_16(x w'), symmetric_zero (:204-212)
    const int r = x * fs - q * mb;            // x F_s - m' q (:234-238)
    const int lo = wrap16(r);                 // low 16 bits (:241)
    const int sign = wrap16(r >> 16);         // floor(r / 2^16) (:228, :242)
    return wrap16(lo - sign * q);             // (:261-272)
}

// x mod q in [0, q) for any int32 x: one 32-bit Barrett step with
// c = round(2^32 / q) leaves |r| <= 0.75 q (quotient error at most
// 2^31 * 0.5 / 2^32 from c plus 0.5 from the rounding), and one conditional
// addition of q finishes it; an integer division by a runtime q costs several
// times as many instructions
__host__ __device__ __forceinline__ int canon(int x, int q, int c) {
    const int r = br32(x, c, q);
    return r + ((r >> 31) & q);
}

// ---------------------------------------------------------------------------
// canonical arithmetic (families F_C16F ... F_C32I)
//
// Lanes are unsigned 32-bit values congruent to the coefficient, reduced only
// as far as the next operation needs:
//   * Shoup multiplication (V. Shoup's precomputed-quotient modular multiply,
//     as in D. Harvey, "Faster arithmetic for number-theoretic transforms",
//     2014): for a twiddle w < q with w' = floor(w 2^32 / q) and any y < 2^32,
//     y w - floor(y w' / 2^32) q lies in [0, 2q); the low 32 bits of the two
//     products give it exactly (mul.hi + two IMADs);
//   * the inverse runs Cooley-Tukey butterflies: x +- t (t the Shoup product)
//     leaves x + t and x - t + 2q, so the bound on the lanes grows by 2q per
//     layer.  int16 moduli (q < 2^15) start below 2^18 and stay below 2^20
//     in 12 layers: no correction at all.  int32 moduli (q < 2^30) keep
//     Harvey's bound: x is brought from [0, 4q) to [0, 2q) before each
//     butterfly (one subtraction and an unsigned minimum), outputs below 4q;
//   * the forward runs Gentleman-Sande butterflies: x + y and (x - y + c) w
//     with c a multiple of q above y's bound.  int16 sums double the bound
//     each layer and stay below 2^29 in 12 layers; int32 sums are folded
//     back below 2q, so every lane stays in [0, 2q);
//   * one reduction to [0, q) at the end.
// Both cost three multiplies and two (int16) or four (int32) additions,
// subtractions and minimums per butterfly.
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned shoup_mul(unsigned y, unsigned w, unsigned wq, unsigned q) {
    return y * w - __umulhi(y, wq) * q;
}
// [0, 2m) -> [0, m) for an unsigned lane (x - m wraps to a large value when x < m)
__device__ __forceinline__ unsigned lazy_sub(unsigned x, unsigned m) { return min(x, x - m); }

// int32 input coefficient (any signed value) -> a lane in [0, 2q): x + 2^31 is
// reduced by one Barrett step with floor(2^32 / q) (error below 2q), then the
// residue of -2^31 is added back and the sum folded below 2q
__device__ __forceinline__ unsigned canon_in32(int x, unsigned q, unsigned cq, unsigned k31) {
    const unsigned u = (unsigned)x ^ 0x80000000u;
    const unsigned r = u - __umulhi(u, cq) * q;
    return lazy_sub(r + k31, 2u * q);
}
// a lane below 2^32 -> [0, q)
__device__ __forceinline__ unsigned canon_out(unsigned v, unsigned q, unsigned cq) {
    return lazy_sub(v - __umulhi(v, cq) * q, q);
}

// Which output options a design accepts (checked by the host as well): the
// fused n^-1 scaling belongs to the int16 inverse designs, natural-order input
// to the inverse designs and natural-order output to the forward designs.
// BR marks the radix-4 inverse, which runs the radix-4 kernel between two bit
// reversals.  Gating them at compile time keeps their registers and code out
// of the designs that never use them.
__host__ __device__ constexpr bool fam_scales(int fam, bool br) {
    return fam == F_R2I16 || (fam == F_R4F16 && br) || fam == F_C16I || fam == F_C32I;
}
__host__ __device__ constexpr bool fam_natural_in(int fam, bool br) {
    return fam == F_R2I16 || fam == F_R2G32 || (fam == F_R4F16 && br) || fam == F_C16I || fam == F_C32I;
}
__host__ __device__ constexpr bool fam_natural_out(int fam, bool br) { return !fam_natural_in(fam, br); }

// The output epilogue: fused n^-1 scaling (SCALE designs), canonical form.
// The flags are read from the kernel arguments where they are used, so they
// hold no registers through the transform.
template <bool SCALE, int E>
__device__ __forceinline__ void epilogue_all(int (&v)[E], const KArgs& a);

// Canonical families: every lane to [0, q), or n^-1 times it (a Shoup
// multiplication, [0, 2q), then one subtraction) for a scaled inverse.  (int32
// lanes end below 4q, so two subtract-and-minimum steps would reduce them
// without a multiply; measured mixed against the Barrett step, -4 % to +12 %
// per design, so every family keeps the Barrett step.)
template <bool I32, int E>
__device__ __forceinline__ void epilogue_canon(int (&v)[E], const KArgs& a, bool scale) {
    const unsigned q = (unsigned)a.q;
    if (scale) {
        const unsigned w = a.ninv, wq = a.ninv_q;
#pragma unroll
        for (int k = 0; k < E; ++k) v[k] = (int)lazy_sub(shoup_mul((unsigned)v[k], w, wq, q), q);
    } else {
        const unsigned cq = a.cq;
#pragma unroll
        for (int k = 0; k < E; ++k) v[k] = (int)canon_out((unsigned)v[k], q, cq);
    }
}

// the epilogue of family FAM (BR: the radix-4 inverse's form)
template <int FAM, bool BR, int E>
__device__ __forceinline__ void epilogue(int (&v)[E], const KArgs& a) {
    if constexpr (fam_canon(FAM)) {
        epilogue_canon<FAM == F_C32F || FAM == F_C32I>(v, a, fam_scales(FAM, BR) && a.scale);
    } else {
        epilogue_all<fam_scales(FAM, BR)>(v, a);
    }
}

// The input prologue: canonical int32 lanes start in [0, 2q) (int16 inputs
// stay raw; the first layer adds an offset instead).
template <int FAM, int E>
__device__ __forceinline__ void prologue(int (&v)[E], const KArgs& a) {
    if constexpr (FAM == F_C32F || FAM == F_C32I) {
        const unsigned q = (unsigned)a.q, cq = a.cq, k31 = (unsigned)a.in_off;
#pragma unroll
        for (int k = 0; k < E; ++k) v[k] = (int)canon_in32(v[k], q, cq, k31);
    }
}

template <bool SCALE, int E>
__device__ __forceinline__ void epilogue_all(int (&v)[E], const KArgs& a) {
    if constexpr (SCALE) {
        if (a.scale) {
            const int fs = a.fb_fs, wq = a.fb_wq, q = a.q;
#pragma unroll
            for (int k = 0; k < E; ++k) v[k] = fb16(v[k], fs, wq, q);
        }
    }
    if (a.canonical) {
        const int q = a.q, c = a.canon_c;
#pragma unroll
        for (int k = 0; k < E; ++k) v[k] = canon(v[k], q, c);
    }
}

// ---------------------------------------------------------------------------
// compile-time schedule
// ---------------------------------------------------------------------------

__host__ __device__ constexpr bool fam_i32(int fam) {
    return fam == F_R2F32 || fam == F_R2G32 || fam == F_C32F || fam == F_C32I;
}
// forward designs consume position bits from the top, inverse ones from the bottom
__host__ __device__ constexpr bool topdown(int fam) {
    return fam != F_R2I16 && fam != F_R2G32 && fam != F_C16I && fam != F_C32I;
}
__host__ __device__ constexpr int nsteps(int fam, int L) {
    return fam == F_R4F16 ? L / 2 : fam == F_R8F16 ? L / 3 + (L % 3 ? 1 : 0) : L;
}
__host__ __device__ constexpr int step_w(int fam, int L, int s) {
    return fam == F_R4F16 ? 2 : fam == F_R8F16 ? (s < L / 3 ? 3 : L % 3) : 1;
}
__host__ __device__ constexpr int step_b(int fam, int L, int s) {
    return fam == F_R4F16 ? L - 2 - 2 * s
         : fam == F_R8F16 ? (s < L / 3 ? L - 3 - 3 * s : 0)
         : topdown(fam) ? L - 1 - s : s;
}
// lowest position bit of the register window used by step s
__host__ __device__ constexpr int window_lo(int fam, int L, int EL, int s) {
    int lo = topdown(fam) ? L - EL : 0;
    for (int i = 0; i <= s; ++i) {
        const int b = step_b(fam, L, i), w = step_w(fam, L, i);
        if (b < lo || b + w > lo + EL)
            lo = topdown(fam) ? (b + w - EL < 0 ? 0 : b + w - EL) : (b > L - EL ? L - EL : b);
    }
    return lo;
}
// the first step that changes window (-1: one window)
__host__ __device__ constexpr int first_exchange_step(int fam, int L, int EL) {
    for (int s = 1; s < nsteps(fam, L); ++s)
        if (window_lo(fam, L, EL, s) != window_lo(fam, L, EL, s - 1)) return s;
    return -1;
}
__host__ __device__ constexpr int num_windows(int fam, int L, int EL) {
    int c = 1;
    for (int s = 1; s < nsteps(fam, L); ++s)
        if (window_lo(fam, L, EL, s) != window_lo(fam, L, EL, s - 1)) ++c;
    return c;
}

// first table entry of radix-8 stage s (8 * 2^(L-3-3t) entries per stage t)
__host__ __device__ constexpr int r8_stage_offset(int L, int s) {
    int o = 0;
    for (int t = 0; t < s; ++t) o += 8 << (L - 3 - 3 * t);
    return o;
}

// shared-memory words per polynomial of the exchange buffer (16-byte
// multiple): room for the padded exchange layouts below (at most one spare
// word per 16 positions)
__host__ __device__ constexpr int xwords(int L) { return (((1 << L) + (1 << L) / 16) + 3) & ~3; }

// position of register k of thread g when the window starts at bit LO
__host__ __device__ constexpr int posmap_c(int LO, int EL, int g, int k) {
    return ((g >> LO) << (LO + EL)) | (k << LO) | (g & ((1 << LO) - 1));
}
template <int LO, int EL>
__device__ __forceinline__ int posmap(int g, int k) { return posmap_c(LO, EL, g, k); }

// ---------------------------------------------------------------------------
// Exchange layouts.  An exchange writes every register of the window starting
// at bit LOA and reads back the window starting at LOB.  Both access patterns
// are fixed at compile time, so each exchange gets its own layout, chosen so
// that the 32 lanes of a warp hit distinct banks on both sides (lanes past a
// short polynomial belong to the next one, xwords(L) words further).
//
// Scalar exchanges (no position bit shared by the two windows): word =
// pos + (pos >> S) * T, one to two spare words every 32.  The padding is a sum
// over disjoint bit fields, so the address of register k is the thread's base
// plus a compile-time constant.
//
// Vectorised exchanges: when the windows share position bits [OLO, OLO + VB),
// the 2^VB values that differ only in those bits stay in one thread on both
// sides and move as one 8- or 16-byte access.  The word address keeps those
// bits lowest; the remaining bits form the chunk index c, whose bank-group
// bits are XOR-folded with c >> F (F = 0: no fold).  The fold is linear, so the
// register-dependent part is again a compile-time constant.
// ---------------------------------------------------------------------------

__host__ __device__ constexpr int xpad(int p, int s, int t) { return p + (p >> s) * t; }

__host__ __device__ constexpr int brev_n(int x, int nb) {
    int r = 0;
    for (int i = 0; i < nb; ++i) r |= ((x >> i) & 1) << (nb - 1 - i);
    return r;
}

// Bank-conflict degree of a padded layout, summed over the writing side
// (window LOA, at bit-reversed positions when BRA) and the reading side
// (window LOB): 2 = conflict free.
__host__ __device__ constexpr int pad_degree(int L, int EL, int LOA, bool BRA, int LOB, int s, int t) {
    const int G = 1 << (L - EL);
    int total = 0;
    for (int side = 0; side < 2; ++side) {
        int cnt[32] = {};
        int worst = 0;
        for (int lane = 0; lane < 32; ++lane) {
            int p = posmap_c(side ? LOB : LOA, EL, lane % G, 0);
            if (!side && BRA) p = brev_n(p, L);
            const int w = (lane / G) * xwords(L) + xpad(p, s, t);
            const int c = ++cnt[w & 31];
            worst = c > worst ? c : worst;
        }
        total += worst;
    }
    return total;
}

struct XPad { int s, t; };

// the padding with the fewest conflicts (the first such candidate, one spare
// word every 32 positions first) that fits xwords(L)
__host__ __device__ constexpr XPad pad_layout(int L, int EL, int LOA, bool BRA, int LOB) {
    XPad best{5, 1};
    int bd = pad_degree(L, EL, LOA, BRA, LOB, 5, 1);
    for (int s = 4; s <= L && bd > 2; ++s)
        for (int t = 1; t <= 16 && bd > 2; t *= 2) {
            if (t * 32 > (2 << s) || xpad((1 << L) - 1, s, t) >= xwords(L)) continue;
            const int d = pad_degree(L, EL, LOA, BRA, LOB, s, t);
            if (d < bd) { bd = d; best = XPad{s, t}; }
        }
    return best;
}
// a scalar exchange from window LOA to window LOB
__host__ __device__ constexpr XPad scalar_layout(int L, int EL, int LOA, int LOB) {
    return pad_layout(L, EL, LOA, false, LOB);
}
// the bit-reversal permutation of window LO: the register of position p is
// written at bitrev(p) and read back at p
__host__ __device__ constexpr XPad brev_layout(int L, int EL, int LO) { return pad_layout(L, EL, LO, true, LO); }

__host__ __device__ constexpr int vchunk(int pos, int OLO, int VB) {
    return ((pos >> (OLO + VB)) << OLO) | (pos & ((1 << OLO) - 1));
}
// fold of the chunk index: bank-group bits (5 - VB of them) XOR c >> F
__host__ __device__ constexpr int vfold(int c, int VB, int F) {
    return F ? c ^ ((c >> F) & ((1 << (5 - VB)) - 1)) : c;
}
__host__ __device__ constexpr int vword(int pos, int OLO, int VB, int F) {
    return (vfold(vchunk(pos, OLO, VB), VB, F) << VB) | ((pos >> OLO) & ((1 << VB) - 1));
}

// shared-memory wavefronts of one warp over both sides of a vectorised
// exchange (a 16-byte access is served per quarter warp, an 8-byte access per
// half warp)
__host__ __device__ constexpr int vector_wavefronts(int L, int EL, int LOA, int LOB, int VB, int F) {
    const int G = 1 << (L - EL), E = 1 << EL, V = 1 << VB;
    const int OLO = LOA > LOB ? LOA : LOB;
    const int per = 8 * (4 / V);            // lanes per phase
    int total = 0;
    for (int side = 0; side < 2; ++side) {
        const int LO = side ? LOB : LOA, KX = OLO - LO;
        for (int r = 0; r < (E >> VB); ++r) {
            const int k = ((r >> KX) << (KX + VB)) | (r & ((1 << KX) - 1));
            for (int ph = 0; ph < 32 / per; ++ph) {
                int cnt[32] = {};
                int worst = 0;
                for (int lane = ph * per; lane < (ph + 1) * per; ++lane) {
                    const int w = (lane / G) * xwords(L) + vword(posmap_c(LO, EL, lane % G, k), OLO, VB, F);
                    for (int j = 0; j < V; ++j) {
                        const int c = ++cnt[(w + j) & 31];
                        worst = c > worst ? c : worst;
                    }
                }
                total += worst;
            }
        }
    }
    return total;
}

// the fold of a vectorised exchange: fewest wavefronts, no fold on a tie
__host__ __device__ constexpr int vector_layout(int L, int EL, int LOA, int LOB, int VB) {
    int best = 0;
    int bw = vector_wavefronts(L, EL, LOA, LOB, VB, 0);
    const int ideal = 2 * (1 << EL);        // E / V accesses of V wavefronts per side
    for (int f = 1; f < L - VB && bw > ideal; ++f) {
        const int w = vector_wavefronts(L, EL, LOA, LOB, VB, f);
        if (w < bw) { bw = w; best = f; }
    }
    return best;
}

template <int G>
__device__ __forceinline__ void group_sync() {
    if constexpr (G > 32) __syncthreads();
    else __syncwarp();
}

// Moves the thread's registers from the window starting at bit LOA to the
// window starting at LOB through the shared buffer sp.  lead: wait first for
// the group's earlier reads of sp; a caller passes false (uniformly) when no
// thread has touched sp since the last barrier of the whole CTA.
template <int L, int EL, int LOA, int LOB>
__device__ __forceinline__ void exchange_windows(int (&v)[1 << EL], int* sp, int g, bool lead = true) {
    constexpr int E = 1 << EL, G = 1 << (L - EL);
    constexpr int OLO = LOA > LOB ? LOA : LOB;
    constexpr int OHI = (LOA < LOB ? LOA : LOB) + EL;
    constexpr int W = OHI > OLO ? OHI - OLO : 0;
    constexpr int VB = W >= 2 ? 2 : W;
    if (lead) group_sync<G>();
    if constexpr (VB == 0) {
        constexpr XPad X = scalar_layout(L, EL, LOA, LOB);
        int* const pa = sp + xpad(posmap<LOA, EL>(g, 0), X.s, X.t);
#pragma unroll
        for (int k = 0; k < E; ++k) pa[xpad(k << LOA, X.s, X.t)] = v[k];
        group_sync<G>();
        const int* const pb = sp + xpad(posmap<LOB, EL>(g, 0), X.s, X.t);
#pragma unroll
        for (int k = 0; k < E; ++k) v[k] = pb[xpad(k << LOB, X.s, X.t)];
    } else {
        constexpr int F = vector_layout(L, EL, LOA, LOB, VB);
        constexpr int V = 1 << VB, MB = (1 << (5 - VB)) - 1;   // bank-group bits of the chunk
        constexpr int KA = OLO - LOA, KB = OLO - LOB;           // register bit of the shared bits
        // chunk word of the thread's part of the position; the register part
        // is XORed into the bank-group bits and added above them
        const int xa = vfold(vchunk(posmap<LOA, EL>(g, 0), OLO, VB), VB, F) << VB;
#pragma unroll
        for (int r = 0; r < (E >> VB); ++r) {
            const int k = ((r >> KA) << (KA + VB)) | (r & ((1 << KA) - 1));
            const int kc = vfold(vchunk(k << LOA, OLO, VB), VB, F);
            const int a = (xa ^ ((kc & MB) << VB)) + ((kc & ~MB) << VB);
            if constexpr (V == 4)
                *reinterpret_cast<int4*>(sp + a) =
                    make_int4(v[k], v[k | (1 << KA)], v[k | (2 << KA)], v[k | (3 << KA)]);
            else
                *reinterpret_cast<int2*>(sp + a) = make_int2(v[k], v[k | (1 << KA)]);
        }
        group_sync<G>();
        const int xb = vfold(vchunk(posmap<LOB, EL>(g, 0), OLO, VB), VB, F) << VB;
#pragma unroll
        for (int r = 0; r < (E >> VB); ++r) {
            const int k = ((r >> KB) << (KB + VB)) | (r & ((1 << KB) - 1));
            const int kc = vfold(vchunk(k << LOB, OLO, VB), VB, F);
            const int a = (xb ^ ((kc & MB) << VB)) + ((kc & ~MB) << VB);
            if constexpr (V == 4) {
                const int4 w = *reinterpret_cast<const int4*>(sp + a);
                v[k] = w.x; v[k | (1 << KB)] = w.y; v[k | (2 << KB)] = w.z; v[k | (3 << KB)] = w.w;
            } else {
                const int2 w = *reinterpret_cast<const int2*>(sp + a);
                v[k] = w.x; v[k | (1 << KB)] = w.y;
            }
        }
    }
}

template <int NB>
__host__ __device__ constexpr int brev_c(int x) {
    int r = 0;
    for (int i = 0; i < NB; ++i) r |= ((x >> i) & 1) << (NB - 1 - i);
    return r;
}

// ---------------------------------------------------------------------------
// butterflies of one step (all groups of the thread's window)
// ---------------------------------------------------------------------------

// Column-interleaved exchange for the column pass of the two-pass schedule:
// XC adjacent columns share the buffer, word = position * XC + column.
template <int L, int EL, int LOA, int LOB, int XC>
__device__ __forceinline__ void exchange_cols(int (&v)[1 << EL], int* sp, int g, int cl) {
    constexpr int E = 1 << EL;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < E; ++k) sp[posmap<LOA, EL>(g, k) * XC + cl] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < E; ++k) v[k] = sp[posmap<LOB, EL>(g, k) * XC + cl];
}

// XC > 0: column pass (XC columns per CTA, exchanges through exchange_cols);
// HIB: row pass, the polynomial is row `hi` of a longer transform and the
// twiddle block index carries hi in its top bits.
// fresh: no thread of the CTA has touched sp since the CTA's last barrier, so
// the transform's first exchange needs no leading barrier (uniform)
template <int FAM, int L, int EL, int S, int XC = 0, bool HIB = false>
__device__ __forceinline__ void do_step(int (&v)[1 << EL], int* sp, int g, const KC& a, int hi = 0, int cl = 0,
                                        bool fresh = false) {
    constexpr int E = 1 << EL;
    constexpr int G = 1 << (L - EL);
    constexpr int LO = window_lo(FAM, L, EL, S);
    constexpr int B = step_b(FAM, L, S);
    constexpr int W = step_w(FAM, L, S);
    constexpr int KB = B - LO;
    static_assert(B >= LO && B + W <= LO + EL, "step outside its window");
    if constexpr (S > 0) {
        constexpr int PLO = window_lo(FAM, L, EL, S - 1);
        if constexpr (PLO != LO) {
            if constexpr (XC > 0) exchange_cols<L, EL, PLO, LO, XC>(v, sp, g, cl);
            else exchange_windows<L, EL, PLO, LO>(v, sp, g, !(fresh && S == first_exchange_step(FAM, L, EL)));
        }
    }
    const int q = a.q;
#pragma unroll
    for (int r = 0; r < (E >> W); ++r) {
        const int k0 = ((r >> KB) << (KB + W)) | (r & ((1 << KB) - 1));
        if constexpr (fam_canon(FAM)) {
            // Canonical butterflies.  Both directions index the table by the
            // position bits below the butterfly bit B, j = pos mod 2^B, at entry
            // 2^B + j, so a warp's twiddle loads are one broadcast (j from the
            // registers) or consecutive entries (j from the lane index).
            static_assert(!HIB, "the canonical families run whole sub-transforms (the four-step twist is separate)");
            const int k1 = k0 | (1 << KB);
            const unsigned uq = (unsigned)q, q2 = uq << 1;
            if constexpr (topdown(FAM)) {
                // Forward: Gentleman-Sande, natural order in, bit-reversed out.
                // Layer S pairs the positions differing in bit B = L-1-S:
                // (x, y) -> (x + y, (x - y) w), w = root^(j 2^(L-1-B)).  The
                // last layer (B = 0) has w = 1.
                const unsigned x = (unsigned)v[k0], y = (unsigned)v[k1];
                unsigned s, d;
                if constexpr (fam_i32(FAM)) {
                    // lanes in [0, 2q): the sum is folded back below 2q
                    s = x + y;
                    d = x + q2 - y;
                    if constexpr (S != L - 1) s = lazy_sub(s, q2);
                } else if constexpr (S == 0) {
                    // raw int16 inputs in [-2^15, 2^15): 2M (a multiple of q,
                    // M >= 2^15) makes both lanes non-negative, below 2^18
                    s = (unsigned)((int)x + (int)y + a.in_off);
                    d = (unsigned)((int)x - (int)y + a.in_off);
                } else {
                    // int16 lanes below 2^(S+1) 2M: sums double the bound each
                    // layer (below 2^29 after 12 layers); the difference takes
                    // the offset 2^S 2M, a multiple of q above the bound
                    s = x + y;
                    d = x + ((unsigned)a.in_off << S) - y;
                }
                if constexpr (S != L - 1) {
                    const int2 t = __ldg(&a.tab[(1 << B) + (posmap<LO, EL>(g, k0) & ((1 << B) - 1))]);
                    d = shoup_mul(d, (unsigned)t.x, (unsigned)t.y, uq);
                }
                v[k0] = (int)s;
                v[k1] = (int)d;
            } else if constexpr (S == 0) {
                // Inverse: Cooley-Tukey on bit-reversed input, natural order
                // out.  Layer S pairs the positions differing in bit B = S:
                // (x, y) -> (x + w y, x - w y), w = root^(-j 2^(L-1-B)); the
                // first layer (span 1) has w = 1.
                if constexpr (fam_i32(FAM)) {
                    // lanes in [0, 2q) from the prologue
                    const unsigned x = (unsigned)v[k0], y = (unsigned)v[k1];
                    v[k0] = (int)(x + y);
                    v[k1] = (int)(x + q2 - y);
                } else {
                    // raw int16 inputs: the offset 2M as in the forward
                    const int x = v[k0], y = v[k1];
                    v[k0] = x + y + a.in_off;
                    v[k1] = x - y + a.in_off;
                }
            } else {
                // the lane bound grows by 2q per layer (int16: below 2^20 after
                // 12 layers); int32 lanes keep Harvey's bound, x < 2q before the
                // butterfly and both outputs below 4q
                const int2 t = __ldg(&a.tab[(1 << B) + (posmap<LO, EL>(g, k0) & ((1 << B) - 1))]);
                unsigned x = (unsigned)v[k0];
                if constexpr (fam_i32(FAM)) x = lazy_sub(x, q2);
                const unsigned m = shoup_mul((unsigned)v[k1], (unsigned)t.x, (unsigned)t.y, uq);
                v[k0] = (int)(x + m);
                v[k1] = (int)(x + q2 - m);
            }
        } else if constexpr (FAM == F_R2F16 || FAM == F_R2F32) {
            // forward CT layer S: block = position bits above B (src/kernels/
            // ntt_r2_kernels.cc:434-472, ntt_r2_int32_kernels.cc:267-295)
            const int k1 = k0 | (1 << KB);
            const int blk = ((HIB ? (hi << L) : 0) | posmap<LO, EL>(g, k0)) >> (B + 1);
            if constexpr (FAM == F_R2F16) {
                const int t = __ldg(&a.tab16[blk]);
                const unsigned u = (unsigned)br16(v[k0], a.c, q), w = bm16_lo(v[k1], t, q);
                v[k0] = wrap16((int)(u + w));
                v[k1] = wrap16((int)(u - w));
            } else {
                const int2 t = __ldg(&a.tab[blk]);
                const int u = br32(v[k0], a.c, q), w = bm32(v[k1], t.x, t.y, q);
                v[k0] = add32(u, w);
                v[k1] = sub32(u, w);
            }
        } else if constexpr (FAM == F_R2G32) {
            // inverse GS layer S (ntt_r2_int32_kernels.cc:305-336)
            const int k1 = k0 | (1 << KB);
            const int blk = ((HIB ? (hi << L) : 0) | posmap<LO, EL>(g, k0)) >> (B + 1);
            const int2 t = __ldg(&a.tab[blk]);
            const int s = add32(v[k0], v[k1]), d = sub32(v[k0], v[k1]);
            v[k0] = br32(s, a.c, q);
            v[k1] = bm32(d, t.x, t.y, q);
        } else if constexpr (FAM == F_R2I16) {
            // inverse CT layer S on bit-reversed input (ntt_r2_kernels.cc:484-540)
            const int k1 = k0 | (1 << KB);
            if constexpr (S == 0) {
                const int s = wrap16(v[k0] + v[k1]), d = wrap16(v[k0] - v[k1]);
                v[k0] = s;
                v[k1] = d;
            } else {
                const int tpos = posmap<LO, EL>(g, k0) & ((1 << B) - 1);
                const int t = __ldg(&a.tab16[(1 << B) + tpos]);
                const unsigned u = (unsigned)br16(v[k0], a.c, q), w = bm16_lo(v[k1], t, q);
                v[k0] = wrap16((int)(u + w));
                v[k1] = wrap16((int)(u - w));
            }
        } else if constexpr (FAM == F_R4F16) {
            // radix-4 layer S (ntt_r4_kernels.cc:243-261)
            // input 0 always has twiddle 1 (power 0), and so has every input
            // of stage 0 (block 0): those products are plain reductions with
            // the multiplier of 1, read from table entry 0.
            constexpr int OFF = 4 * (((1 << (2 * S)) - 1) / 3);
            const int ka = k0, kb1 = k0 | (1 << KB), kb2 = k0 | (2 << KB), kb3 = k0 | (3 << KB);
            // A0 always uses the multiplier of twiddle 1; A2 only feeds the
            // wrapped sums, so it may keep bits above 16 (bm16_lo); A1 and A3
            // are multiplied again by omega_4 and must be exact.
            int A1, A3;
            unsigned A2;
            const int A0 = br16(v[ka], a.wq1, q);
            if constexpr (S == 0) {
                A1 = br16(v[kb1], a.wq1, q);
                A2 = (unsigned)br16(v[kb2], a.wq1, q);
                A3 = br16(v[kb3], a.wq1, q);
            } else {
                const int blk = posmap<LO, EL>(g, k0) >> (B + 2);
                const int4 t = __ldg(reinterpret_cast<const int4*>(a.tab16 + OFF + 4 * blk));
                A1 = bm16(v[kb1], lo16(t.y), hi16(t.y), q);
                A2 = bm16_lo(v[kb2], t.z, q);
                A3 = bm16(v[kb3], lo16(t.w), hi16(t.w), q);
            }
            const int A5 = bm16(A1, a.fneg, a.wc, q);
            const int A6 = bm16(A3, a.fneg, a.wc, q);
            const unsigned s02 = (unsigned)A0 + A2, d02 = (unsigned)A0 - A2;
            const unsigned s13 = (unsigned)A1 + (unsigned)A3, d13 = (unsigned)A1 - (unsigned)A3;
            const unsigned d56 = (unsigned)A5 - (unsigned)A6;
            v[ka] = wrap16((int)(s02 + s13));      // y0
            v[kb1] = wrap16((int)(s02 - s13));     // y2 -> digit bitrev2(2) = 1
            v[kb2] = wrap16((int)(d02 + d56));     // y1 -> digit 2
            v[kb3] = wrap16((int)(d02 - d56));     // y3 -> digit 3
        } else if constexpr (FAM == F_R8F16) {
            if constexpr (W == 3) {
                // radix-8 stage S: y = x F8 (int32), then the reduction tile
                // with twiddle root^(8^S r k) (ntt_r8_kernels.cc:30-404)
                constexpr int OFF = r8_stage_offset(L, S);
                const int rr = posmap<LO, EL>(g, k0) & ((1 << B) - 1);
                int x[8], y[8];
#pragma unroll
                for (int m = 0; m < 8; ++m) x[m] = v[k0 | (m << KB)];
                if (a.r8_sym) {
                    const int f1 = a.f1, f2 = a.f2, f3 = a.f3;
                    const int a0 = x[0] + x[4], a1 = x[1] + x[5], a2 = x[2] + x[6], a3 = x[3] + x[7];
                    const int b0 = x[0] - x[4], b1 = x[1] - x[5], b2 = x[2] - x[6], b3 = x[3] - x[7];
                    const int c0 = a0 + a2, c1 = a1 + a3, d0 = a0 - a2, d1 = a1 - a3;
                    y[0] = c0 + c1;
                    y[4] = c0 - c1;
                    const int t2 = f2 * d1;
                    y[2] = d0 + t2;
                    y[6] = d0 - t2;
                    const int e0 = b0 + f2 * b2, e1 = b0 - f2 * b2;
                    const int h1 = f1 * b1 + f3 * b3, h3 = f3 * b1 + f1 * b3;
                    y[1] = e0 + h1;
                    y[5] = e0 - h1;
                    y[3] = e1 + h3;
                    y[7] = e1 - h3;
                } else {
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        int acc = 0;
#pragma unroll
                        for (int m = 0; m < 8; ++m) acc += x[m] * a.f8[8 * m + k];
                        y[k] = acc;
                    }
                }
                // output 0 has the twiddle 1 in every stage: its multiplier is an argument
                v[k0] = r8red(y[0], 1, a.tail_wq, q);
#pragma unroll
                for (int k = 1; k < 8; ++k) {
                    const int2 t = __ldg(&a.tab[OFF + (k << B) + rr]);
                    v[k0 | (brev_c<3>(k) << KB)] = r8red(y[k], t.x, t.y, q);
                }
            } else {
                // radix-2^W tail stage, twiddle 1
                constexpr int R = 1 << W;
                int x[R];
#pragma unroll
                for (int m = 0; m < R; ++m) x[m] = v[k0 | (m << KB)];
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    int acc = 0;
#pragma unroll
                    for (int m = 0; m < R; ++m) acc += x[m] * a.ftail[R * m + k];
                    v[k0 | (brev_c<W>(k) << KB)] = r8red(acc, 1, a.tail_wq, q);
                }
            }
        }
    }
}

template <int FAM, int L, int EL, int... S>
__device__ __forceinline__ void run_steps(int (&v)[1 << EL], int* sp, int g, const KC& a, bool fresh,
                                          std::integer_sequence<int, S...>) {
    (do_step<FAM, L, EL, S>(v, sp, g, a, 0, 0, fresh), ...);
}

template <int FAM, int L, int EL, int XC, bool HIB, int... S>
__device__ __forceinline__ void run_steps_x(int (&v)[1 << EL], int* sp, int g, const KC& a, int hi, int cl,
                                            std::integer_sequence<int, S...>) {
    (do_step<FAM, L, EL, S, XC, HIB>(v, sp, g, a, hi, cl), ...);
}

// ---------------------------------------------------------------------------
// load / store of one polynomial in a window layout
// ---------------------------------------------------------------------------

// Bit-reversal permutation of one polynomial held in the window layout LO:
// afterwards the register of position p holds the value that was at position
// bitrev_L(p).  Within one thread (L == EL) it is a renaming of registers;
// otherwise it goes through the polynomial's exchange buffer, so the global
// accesses around it stay coalesced.
template <int L, int EL, int LO>
__device__ __forceinline__ void permute_br(int (&v)[1 << EL], int* sp, int g) {
    constexpr int E = 1 << EL, G = 1 << (L - EL);
    if constexpr (G == 1) {
        int t[E];
#pragma unroll
        for (int k = 0; k < E; ++k) t[k] = v[k];
#pragma unroll
        for (int k = 0; k < E; ++k) v[k] = t[brev_c<L>(k)];
    } else {
        // the thread bits and the register bits of a position are disjoint, so
        // bitrev(pos) = bitrev(thread part) | bitrev(register part), and the
        // padding (chosen like an exchange's) splits the same way: one runtime
        // base plus a constant per register
        constexpr XPad X = brev_layout(L, EL, LO);
        const int wb = xpad((int)(__brev((unsigned)posmap<LO, EL>(g, 0)) >> (32 - L)), X.s, X.t);
        group_sync<G>();
#pragma unroll
        for (int k = 0; k < E; ++k) sp[wb + xpad(brev_c<L>(k << LO), X.s, X.t)] = v[k];
        group_sync<G>();
        const int rb = xpad(posmap<LO, EL>(g, 0), X.s, X.t);
#pragma unroll
        for (int k = 0; k < E; ++k) v[k] = sp[rb + xpad(k << LO, X.s, X.t)];
    }
}

template <bool I32, int L, int EL, int LO>
__device__ __forceinline__ void load_poly(int (&v)[1 << EL], const KArgs& a, long long poly, int g) {
    constexpr int E = 1 << EL;
    constexpr long long N = 1LL << L;
    if constexpr (I32) {
        const int* src = static_cast<const int*>(a.in) + poly * N;
        if constexpr (LO == 0 && E >= 4) {
            const int4* s4 = reinterpret_cast<const int4*>(src + (long long)g * E);
#pragma unroll
            for (int j = 0; j < E / 4; ++j) {
                const int4 w = __ldg(s4 + j);
                v[4 * j] = w.x; v[4 * j + 1] = w.y; v[4 * j + 2] = w.z; v[4 * j + 3] = w.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < E; ++k) {
                v[k] = __ldg(src + posmap<LO, EL>(g, k));
            }
        }
    } else {
        const short* src = static_cast<const short*>(a.in) + poly * N;
        if constexpr (LO == 0 && E >= 8) {
            const int4* s4 = reinterpret_cast<const int4*>(src + (long long)g * E);
#pragma unroll
            for (int j = 0; j < E / 8; ++j) {
                const int4 w = __ldg(s4 + j);
                const int ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    v[8 * j + 2 * h] = (int)(short)(ww[h] & 0xFFFF);
                    v[8 * j + 2 * h + 1] = ww[h] >> 16;
                }
            }
        } else {
#pragma unroll
            for (int k = 0; k < E; ++k) {
                v[k] = (int)__ldg(src + posmap<LO, EL>(g, k));
            }
        }
    }
}

template <bool I32, int L, int EL, int LO>
__device__ __forceinline__ void store_poly(int (&v)[1 << EL], const KArgs& a, long long poly, int g) {
    constexpr int E = 1 << EL;
    constexpr long long N = 1LL << L;
    if constexpr (I32) {
        int* dst = static_cast<int*>(a.out) + poly * N;
        if constexpr (LO == 0 && E >= 4) {
            int4* d4 = reinterpret_cast<int4*>(dst + (long long)g * E);
#pragma unroll
            for (int j = 0; j < E / 4; ++j) d4[j] = make_int4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        } else {
#pragma unroll
            for (int k = 0; k < E; ++k) {
                dst[posmap<LO, EL>(g, k)] = v[k];
            }
        }
    } else {
        short* dst = static_cast<short*>(a.out) + poly * N;
        if constexpr (LO == 0 && E >= 8) {
            int4* d4 = reinterpret_cast<int4*>(dst + (long long)g * E);
#pragma unroll
            for (int j = 0; j < E / 8; ++j) {
                int ww[4];
#pragma unroll
                for (int h = 0; h < 4; ++h)
                    ww[h] = (v[8 * j + 2 * h] & 0xFFFF) | (v[8 * j + 2 * h + 1] << 16);
                d4[j] = make_int4(ww[0], ww[1], ww[2], ww[3]);
            }
        } else {
#pragma unroll
            for (int k = 0; k < E; ++k) {
                dst[posmap<LO, EL>(g, k)] = (short)v[k];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// the transform kernel: P polynomials per CTA, G = 2^(L-EL) threads each
// ---------------------------------------------------------------------------

template <int FAM, int L, int EL, int P, bool BR>
__device__ __forceinline__ void k_ntt_body(const KArgs& a) {
    constexpr int G = 1 << (L - EL);
    constexpr int NS = nsteps(FAM, L);
    constexpr int N = 1 << L;
    constexpr int SW = xwords(L);
    constexpr bool I32 = fam_i32(FAM);
    extern __shared__ int smem[];
    const int tid = threadIdx.x;
    const int lp = tid / G, g = tid % G;
    const long long poly = (long long)blockIdx.x * P + lp;
    const bool active = poly < a.batch;
    int* sp = smem + lp * SW;
    int v[1 << EL];
    constexpr int LO0 = window_lo(FAM, L, EL, 0);
    constexpr int LOZ = window_lo(FAM, L, EL, NS - 1);
    // Every stage's table loads sit on the transform's dependent path; in a
    // launch of a few polynomials (latency) they would wait stage by stage, so
    // the host asks for the whole table in L1 first, beside the polynomial's load.
    {
        const char* tb = a.tab16 ? reinterpret_cast<const char*>(a.tab16) : reinterpret_cast<const char*>(a.tab);
        for (int off = tid * 128; off < a.tab_bytes; off += (int)blockDim.x * 128)
            asm volatile("prefetch.global.L1 [%0];" ::"l"(tb + off));
    }
    if (active) {
        load_poly<I32, L, EL, LO0>(v, a, poly, g);
    } else {
#pragma unroll
        for (int k = 0; k < (1 << EL); ++k) v[k] = 0;
    }
    // bit-reversed input: the radix-4 inverse reads bit-reversed order unless
    // the input is natural; the other inverse designs read natural order on request
    bool fresh = true;   // the exchange buffer is untouched until the transform's first exchange
    if constexpr (BR) {
        if (!a.natural_in) {
            permute_br<L, EL, LO0>(v, sp, g);
            fresh = false;
        }
    } else if constexpr (fam_natural_in(FAM, BR)) {
        if (a.natural_in) {
            permute_br<L, EL, LO0>(v, sp, g);
            fresh = false;
        }
    }
    prologue<FAM>(v, a);
    const KC kc = make_kc(a);
    run_steps<FAM, L, EL>(v, sp, g, kc, fresh, std::make_integer_sequence<int, NS>{});
    epilogue<FAM, BR>(v, a);
    if constexpr (BR) {
        permute_br<L, EL, LOZ>(v, sp, g);
    } else if constexpr (fam_natural_out(FAM, BR)) {
        if (a.natural_out) permute_br<L, EL, LOZ>(v, sp, g);
    }
    if (active) store_poly<I32, L, EL, LOZ>(v, a, poly, g);
}

// Two entry points over the same body.  Capping the int32 and radix-4 designs
// at two resident 256-thread CTAs per SM (128 registers) raised their
// throughput by up to a fifth on GB300; the same hint made the radix-2 and
// radix-8 int16 code a fifth slower, so those keep the compiler's default.
__host__ __device__ constexpr bool kntt_two_ctas(int fam, int threads) {
    return threads <= 256 && !fam_canon(fam) && (fam_i32(fam) || fam == F_R4F16);
}

template <int FAM, int L, int EL, int P, bool BR>
__global__ void __launch_bounds__(P << (L - EL)) k_ntt(const __grid_constant__ KArgs a) {
    grid_dep_start();
    k_ntt_body<FAM, L, EL, P, BR>(a);
}

template <int FAM, int L, int EL, int P, bool BR>
__global__ void __launch_bounds__(P << (L - EL), 2) k_ntt2(const __grid_constant__ KArgs a) {
    grid_dep_start();
    k_ntt_body<FAM, L, EL, P, BR>(a);
}

struct KernelInfo {
    const void* fn = nullptr;
    int threads = 0;
    int smem = 0;
    int polys = 0;
    int el = 0;
};

// elements per thread (log2) and polynomials per CTA of each design
// Measured on GB300 (one box, same call): 16 coefficients per thread beat 32
// and 64 for radix-2 int16 forward, radix-4, radix-8 and int32 up to n = 4096
// (int32 n = 4096: 0.30 vs 0.43 vs 0.49 ms); 32 won for the radix-2 int16
// inverse at n = 1024 and for int32 n = 2^14 (0.44 vs 0.50 vs 0.54 ms).  At
// most 1024 threads per polynomial.
__host__ __device__ constexpr int choose_el(int fam, int L) {
    if (L <= 5) return L;
    if (fam == F_R2I16) return L <= 12 ? (L + 1) / 2 : 6;
    if (fam_i32(fam)) return L <= 12 ? 4 : (L - 10 > 5 ? L - 10 : 5);
    return 4;
}
__host__ __device__ constexpr int choose_polys(int fam, int L) {
    const int G = 1 << (L - choose_el(fam, L));
    const int p = 256 / G;
    return p < 1 ? 1 : p;
}

// The latency form of a per-plan launch (a launch of at most one CTA per SM):
// one polynomial per CTA spread over up to 256 threads, so each thread's
// share of every stage is short; at least one butterfly step per window.
// Measured for n = 1024 radix-2 int16, one polynomial, L2 flushed: forward +
// inverse 17.5 -> 10.5 us against 16 (forward) / 32 (inverse) coefficients
// per thread.
__host__ __device__ constexpr int lat_el(int fam, int L) {
    const int lo = fam == F_R8F16 ? 3 : 2;
    return L - 8 > lo ? L - 8 : lo;
}
// the latency form exists where it differs from the throughput form
__host__ __device__ constexpr bool has_lat(int fam, int L) {
    return L >= 9 && L <= 12 && (lat_el(fam, L) != choose_el(fam, L) || choose_polys(fam, L) != 1);
}

template <int FAM, int L, bool BR, bool LAT = false>
KernelInfo make_kernel_info() {
    constexpr int EL = LAT ? lat_el(FAM, L) : choose_el(FAM, L);
    constexpr int P = LAT ? 1 : choose_polys(FAM, L);
    KernelInfo ki;
    if constexpr (kntt_two_ctas(FAM, P << (L - EL)))
        ki.fn = reinterpret_cast<const void*>(&k_ntt2<FAM, L, EL, P, BR>);
    else
        ki.fn = reinterpret_cast<const void*>(&k_ntt<FAM, L, EL, P, BR>);
    ki.threads = P << (L - EL);
    ki.smem = num_windows(FAM, L, EL) > 1 ? P * xwords(L) * 4 : 0;
    ki.polys = P;
    ki.el = EL;
    return ki;
}

// kernel tables, one per family (kernels_*.cu)
// lat: the latency form (an empty KernelInfo where the design has none)
KernelInfo kinfo_r2f16(int L, bool lat);
KernelInfo kinfo_r2i16(int L, bool lat);
KernelInfo kinfo_r2f32(int L, bool lat);
KernelInfo kinfo_r2g32(int L, bool lat);
KernelInfo kinfo_r4(int L, bool br, bool lat);
KernelInfo kinfo_r8(int L, bool lat);
// canonical families (kernels_c16.cu, kernels_c32.cu)
KernelInfo kinfo_canon(int fam, int L, bool lat);

// two-pass schedule for int32 transforms longer than one CTA holds (kernels_large.cu)
struct LargeInfo {
    const void* cols = nullptr;   // column pass kernel
    const void* rows = nullptr;   // row pass kernel
    int cols_threads = 0, cols_smem = 0, cols_per_cta = 0;
    int rows_threads = 0, rows_smem = 0, rows_per_cta = 0;
    int L1 = 0, L2 = 0;           // high (column-pass) and low (row-pass) index bits
};
LargeInfo large_info(int fam, int L);

// Canonical int32 transforms of 2^14 .. 2^22 coefficients as a four-step
// (kernels_c32_large.cu): n = n1 n2, rows of n2 coefficients.  Forward:
// column transforms (length n1, root^n2, bit-reversed along the column), the
// twist root^(c bitrev(r)) of row r at column c, row transforms (length n2,
// root^n1, bit-reversed along the row).  Inverse: the same steps reversed.
struct CanonLarge {
    const void* cols = nullptr;   // k_ccols: TMA-tiled column pass
    const void* rows = nullptr;   // k_crows: row pass with the twist
    int cols_threads = 0, cols_smem = 0, cols_width = 0;   // columns per CTA
    int rows_threads = 0, rows_smem = 0, rows_per_cta = 0;
    int L1 = 0, L2 = 0, row_el = 0;
};
CanonLarge canon_large_info(int fam, int L);
// the four-step launches of one call: `in` -> `out` (in place allowed);
// tab_cols/tab_rows: the sub-transforms' tables, twist: the factors;
// err: a device word set when a bounded wait runs out
cudaError_t launch_canon_large(const CanonLarge& li, const KArgs& base, const int2* tab_cols, const int2* tab_rows,
                               const int2* twist, const void* in, void* out, long long batch, bool inverse,
                               unsigned* err, cudaStream_t s, int* launches);

// kernels_misc.cu: fn on stream s, as a programmatic dependent launch when
// `dependent` (see grid_dep_start)
cudaError_t launch_kernel(const void* fn, unsigned grid, int threads, int smem, void** args, cudaStream_t s,
                          bool dependent);
// the polynomials of a call go through the two passes of the long int32
// transforms in chunks of at most this many bytes, so the intermediate stays
// in L2 (96 MiB; GBNTT_FOURSTEP_CHUNK_MB, 8 .. 120, read once per process)
long long large_chunk_bytes();

// single-purpose kernels (kernels_misc.cu)
cudaError_t launch_r8_stage(const KArgs& a, int L, cudaStream_t s);
cudaError_t launch_bitrev(const KArgs& a, int L, cudaStream_t s);
cudaError_t launch_full_barrett(const KArgs& a, long long total, int fs, int wq, cudaStream_t s);
int bitrev_smem_bytes(int L);

}  // namespace gbntt

