// tables.cpp -- host-side tables of every design (see tables.h).
//
// The values follow the reference's table code exactly, including its
// rounding conventions; only the layout differs:
//   * round<T>(x) of src/twiddle.h:28-31 is T(x + 0.5), i.e. truncation toward
//     zero of x + 1/2 (not nearest for negative x).  x = tw * 2^K / q is never
//     within long-double precision of a half-integer, so it is evaluated here
//     exactly in 128-bit integers.
//   * the "kyber" multipliers (src/twiddle.h:96) and the radix-8 K=31
//     multipliers (:372) are computed in IEEE single precision and rounded
//     with C round() (the template round<T> cannot be deduced there).
//   * the full-Barrett multiplier (full_reduction_kernels.cc:187) adds 0.5f in
//     float before std::round.
// This file must be compiled without fast-math or FMA contraction.
#include "tables.h"

#include <cmath>
#include <cstring>

#include "../../include/gb300_ntt.h"

namespace gbntt {

int64_t powmod(int64_t b, uint64_t e, int64_t q) {
    __int128 r = 1, x = ((b % q) + q) % q;
    while (e) {
        if (e & 1) r = r * x % q;
        x = x * x % q;
        e >>= 1;
    }
    return (int64_t)r;
}

int64_t modinv(int64_t a, int64_t m) {
    int64_t r0 = m, r1 = ((a % m) + m) % m, s0 = 0, s1 = 1;
    while (r1) {
        int64_t t = r0 / r1;
        int64_t r2 = r0 - t * r1, s2 = s0 - t * s1;
        r0 = r1; r1 = r2; s0 = s1; s1 = s2;
    }
    return ((s0 % m) + m) % m;
}

// Smallest L with root^(2^L) == 1 (src/auxiliary.h:35-46).
int log_root_order(int64_t q, int64_t root) {
    int64_t x = ((root % q) + q) % q;
    for (int L = 0; L <= 100; ++L) {
        if (x == 1) return L;
        x = (int64_t)((__int128)x * x % q);
    }
    return -1;
}

bool canonical_fast(int kind, int64_t q, uint32_t flags) {
    if (!(flags & FLAG_CANONICAL) || (flags & FLAG_LANE_EXACT)) return false;
    switch (kind) {
    case K_R2_I16_FWD: case K_R2_I16_INV: case K_R4_I16_FWD: case K_R4_I16_INV:
        return true;
    case K_R8_I16_FWD:
        return !(flags & FLAG_R8_FLOAT);
    case K_R2_I32_FWD: case K_R2_I32_INV:
        return q < (1LL << 30);
    default:
        return false;
    }
}

int canonical_family(int kind) {
    switch (kind) {
    case K_R2_I16_FWD: case K_R4_I16_FWD: case K_R8_I16_FWD: return 6;    // F_C16F
    case K_R2_I16_INV: case K_R4_I16_INV: return 7;                       // F_C16I
    case K_R2_I32_FWD: return 8;                                          // F_C32F
    case K_R2_I32_INV: return 9;                                          // F_C32I
    default: return -1;
    }
}

uint32_t bitrev(uint32_t a, int bits) {
    uint32_t r = 0;
    for (int i = 0; i < bits; ++i) r |= ((a >> i) & 1u) << (bits - 1 - i);
    return r;
}

namespace {

// Representative in [-(q-1)/2, (q-1)/2] (src/twiddle.h:61-69).
int64_t centered(int64_t a, int64_t q) {
    a %= q;
    if (a > (q - 1) / 2) a -= q;
    else if (a < -(q - 1) / 2) a += q;
    return a;
}

// trunc(num/den + 1/2), den > 0 (src/twiddle.h:28-31 evaluated exactly).
int64_t trunc_half(int64_t num, int64_t den) {
    __int128 a = (__int128)2 * num + den, b = (__int128)2 * den;
    return (int64_t)(a / b);
}

int16_t kyber_multiplier(int16_t tw, int32_t q) {
    volatile float num = (float)((int32_t)tw * 65536);
    volatile float quo = num / (float)q;
    return (int16_t)std::round((double)quo);
}

int32_t r8_multiplier(int32_t tw, int32_t q, bool exact) {
    if (exact) return (int32_t)(((__int128)2 * ((int64_t)tw << 31) + q) / ((__int128)2 * q));
    volatile float num = (float)((int64_t)tw << 31);
    volatile float quo = num / (float)q;
    return (int32_t)std::round((double)quo);
}

int16_t fb_multiplier(int32_t fs, int32_t q) {
    volatile float num = (float)(fs * 65536);
    volatile float quo = num / (float)q;
    volatile float sum = quo + 0.5f;
    return (int16_t)std::round(sum);
}

// Forward radix-2 compact table (src/twiddle.h:108-136): tw[bitrev_{L-1}(i)]
// = centered(root^(+-i)), w' = round<T>(tw * 2^K / q), i < n/2.  The layer-l
// table of the reference is tw[j mod 2^l] (src/twiddle.h:141-170), so block b
// of layer l reads entry b.
void t1_compact(int64_t q, int64_t root, int L, int K, bool inverse, std::vector<int32_t>& tab) {
    const int64_t half = (int64_t)1 << (L - 1);
    std::vector<int64_t> tw(half);
    const int64_t F = inverse ? modinv(root, q) : root;
    int64_t cur = 1;
    tw[0] = 1;
    for (int64_t i = 1; i < half; ++i) {
        cur = centered(cur * F, q);
        tw[bitrev((uint32_t)i, L - 1)] = cur;
    }
    tab.assign(2 * half, 0);
    for (int64_t b = 0; b < half; ++b) {
        tab[2 * b] = (int32_t)tw[b];
        tab[2 * b + 1] = (int32_t)trunc_half(tw[b] * ((int64_t)1 << K), q);
    }
}

// Natural-order int16 table and float multipliers (src/twiddle.h:74-102).
void kyber(int32_t q, int32_t root, int size, bool inverse, std::vector<int16_t>& tw, std::vector<int16_t>& wq) {
    tw.assign(size, 0);
    wq.assign(size, 0);
    const int16_t F = (int16_t)(inverse ? modinv(root, q) : root);
    int16_t cur = 1;
    tw[0] = 1;
    for (int i = 1; i < size; ++i) {
        cur = (int16_t)(((int32_t)cur * (int32_t)F) % q);
        cur = (int16_t)centered(cur, q);
        tw[i] = cur;
    }
    for (int i = 0; i < size; ++i) wq[i] = kyber_multiplier(tw[i], q);
}

int16_t r8_signed(int64_t f, int64_t q) { return (int16_t)(f < (q - 1) / 2 ? f : f - q); }

}  // namespace

int build_host_plan(int kind, uint32_t n, int64_t q, int64_t root, int64_t factor, uint32_t flags,
                    HostPlan& hp, std::string& err) {
    hp = HostPlan();
    if (kind < 0 || kind >= K_NUM_KINDS) { err = "unknown design kind"; return GBNTT_ERR_KIND; }
    const bool is32 = (kind == K_R2_I32_FWD || kind == K_R2_I32_INV);
    int L = -1;
    if (n >= 1 && (n & (n - 1)) == 0) { L = 0; while ((1u << L) < n) ++L; }
    if (kind == K_FULL_BARRETT_I16) {
        if (n < 1 || n > (1u << 28)) { err = "n out of range"; return GBNTT_ERR_LENGTH; }
    } else if (L < 1) {
        err = "n must be a power of two >= 2 (src/auxiliary.h:11)";
        return GBNTT_ERR_LENGTH;
    }
    const int max_L = is32 ? 22 : (kind == K_BITREV_I16 ? 16 : 12);
    if (kind != K_FULL_BARRETT_I16 && L > max_L) { err = "n above the supported maximum for this design"; return GBNTT_ERR_LENGTH; }
    if (kind == K_R8_I16_STAGE && n < 16) { err = "the radix-8 stage needs n >= 16"; return GBNTT_ERR_LENGTH; }
    if (kind == K_R8_I16_FWD && n < 8) { err = "the radix-8 transform needs n >= 8"; return GBNTT_ERR_LENGTH; }
    if (kind != K_BITREV_I16) {
        const int64_t qmax = is32 ? 1431655765LL : 21845LL;   // < 2^32/3 (ntt_int32.h:16), < 2^16/3 (ntt.h:118)
        if (q < 3 || (q & 1) == 0 || q > qmax) {
            err = "modulus must be odd and below the lazy-reduction bound of its storage type";
            return GBNTT_ERR_MODULUS;
        }
    }
    if (kind != K_BITREV_I16 && kind != K_FULL_BARRETT_I16) {
        if (log_root_order(q, root) != L) {
            err = "ROOT is not correct: its order must be exactly n (src/auxiliary.h:37,44)";
            return GBNTT_ERR_ROOT;
        }
    }
    if ((kind == K_R4_I16_FWD || kind == K_R4_I16_INV) && (L & 1)) {
        err = "MUST BE EVEN AMOUNT OF LAYERS (src/ntt_r4.h:62-63)";
        return GBNTT_ERR_LAYERS;
    }
    if (kind == K_FULL_BARRETT_I16 && (factor < 0 || factor >= q)) { err = "factor must lie in [0, q)"; return GBNTT_ERR_ARG; }

    const bool inverse = (kind == K_R2_I16_INV || kind == K_R2_I32_INV || kind == K_R4_I16_INV);
    const bool transform = (kind != K_BITREV_I16 && kind != K_FULL_BARRETT_I16 && kind != K_R8_I16_STAGE);
    if ((flags & FLAG_NATURAL_ORDER) && !transform) {
        err = "natural order applies to the transform designs only";
        return GBNTT_ERR_ARG;
    }
    if ((flags & FLAG_NATURAL_ORDER) && is32 && L >= 16) {
        err = "natural order is not available for the two-pass int32 lengths (n >= 2^16)";
        return GBNTT_ERR_ARG;
    }
    if ((flags & FLAG_SCALE_NINV) && !(kind == K_R2_I16_INV || kind == K_R4_I16_INV) &&
        !(kind == K_R2_I32_INV && canonical_fast(kind, q, flags))) {
        err = "the n^-1 epilogue applies to the int16 inverse designs (and to the canonical int32 inverse) only";
        return GBNTT_ERR_ARG;
    }
    (void)inverse;
    hp.kind = kind; hp.n = n; hp.L = L < 0 ? 0 : L; hp.q = q; hp.root = root; hp.factor = factor;
    hp.flags = flags; hp.elem_bytes = is32 ? 4 : 2;
    if (kind != K_BITREV_I16) {
        hp.c = is32 ? (int32_t)trunc_half((int64_t)1 << 32, q)   // ntt_r2_int32_kernels.cc:102
                    : (int32_t)trunc_half(65536, q);             // ntt_r2_kernels.cc:388
    }

    switch (kind) {
    case K_R2_I16_FWD:
        t1_compact(q, root, L, 16, false, hp.tab);
        hp.stages = L;
        break;
    case K_R2_I32_FWD:
        t1_compact(q, root, L, 32, false, hp.tab);
        hp.stages = L;
        break;
    case K_R2_I32_INV:
        // GS layer i uses the table of level L-1-i (src/twiddle.h:238); the
        // kernel indexes it by block, so the compact table is shared.
        t1_compact(q, root, L, 32, true, hp.tab);
        hp.stages = L;
        break;
    case K_R2_I16_INV: {
        // src/twiddle.h:248-266 and :177-222: layer i twiddle for position t
        // inside its block is tw[t * n/2^(i+1)] of the natural inverse table.
        std::vector<int16_t> tw, wq;
        kyber((int32_t)q, (int32_t)root, (int)n, true, tw, wq);
        hp.tab.assign(2 * (size_t)n, 0);
        for (int i = 1; i < L; ++i) {
            const uint32_t rep = n >> (i + 1);
            for (uint32_t t = 0; t < (1u << i); ++t) {
                const size_t e = (1u << i) + t;
                hp.tab[2 * e] = tw[t * rep];
                hp.tab[2 * e + 1] = wq[t * rep];
            }
        }
        hp.stages = L;
        break;
    }
    case K_R4_I16_FWD:
    case K_R4_I16_INV: {
        // src/twiddle.h:403-454: stage l, block b (its top 2l position bits),
        // input d: power = (4^(R-l-1) mod q) * d * bitrev_{2l}(b) mod n.
        const bool inverse = (kind == K_R4_I16_INV);
        std::vector<int16_t> tw, wq;
        kyber((int32_t)q, (int32_t)root, (int)n, inverse, tw, wq);
        const int R = L / 2;
        size_t total = 0;
        for (int l = 0; l < R; ++l) total += (size_t)4 << (2 * l);
        hp.tab.assign(2 * total, 0);
        size_t off = 0;
        for (int l = 0; l < R; ++l) {
            uint64_t op = 1;
            for (int i = 0; i < R - l - 1; ++i) op = (op * 4u) % (uint64_t)q;   // modular_exponentation, twiddle.h:53-57
            for (uint32_t b = 0; b < (1u << (2 * l)); ++b)
                for (uint32_t d = 0; d < 4; ++d) {
                    const uint64_t pw = (op * d * bitrev(b, 2 * l)) % n;
                    const size_t e = off + 4 * b + d;
                    hp.tab[2 * e] = tw[pw];
                    hp.tab[2 * e + 1] = wq[pw];
                }
            off += (size_t)4 << (2 * l);
        }
        const int64_t rt = inverse ? modinv(root, q) : root;
        const int64_t w4 = powmod(rt, n / 4, q);                       // ROOT_4, src/ntt_r4.h:46
        const int64_t fneg = w4 <= (q - 1) / 2 ? w4 : w4 - q;          // ntt_r4_kernels.cc:112
        hp.r4_fneg = (int32_t)fneg;
        hp.r4_wc = (int32_t)trunc_half(fneg * 65536, q);               // ntt_r4_kernels.cc:113
        hp.stages = R + (inverse ? 2 : 0);
        break;
    }
    case K_R8_I16_STAGE:
    case K_R8_I16_FWD: {
        // src/twiddle.h:273-399.
        const bool exact = (kind == K_R8_I16_FWD) ? !(flags & FLAG_R8_FLOAT) : (flags & FLAG_R8_EXACT) != 0;
        const int64_t w8 = powmod(root, n / 8, q);
        int64_t p8[8];
        p8[0] = 1;
        for (int i = 1; i < 8; ++i) p8[i] = p8[i - 1] * w8 % q;
        for (int m = 0; m < 8; ++m)
            for (int k = 0; k < 8; ++k) hp.f8[8 * m + k] = r8_signed(p8[(m * k) % 8], q);
        hp.r8_sym = (hp.f8[8 * 1 + 0] == 1 && hp.f8[8 * 1 + 4] == -1);
        for (int j = 1; j < 4; ++j) hp.r8_sym = hp.r8_sym && (hp.f8[8 + j + 4] == -hp.f8[8 + j]);
        for (int j = 0; j < 4; ++j) hp.f8s[j] = hp.f8[8 + j];
        std::vector<int64_t> pw(n);
        pw[0] = 1;
        for (uint32_t i = 1; i < n; ++i) pw[i] = pw[i - 1] * root % q;
        if (kind == K_R8_I16_STAGE) {
            // Reduction twiddle of 8-NTT i, output k: root^(i k mod n) in
            // [0, q) (src/twiddle.h:381-389), stored here as [k][i].
            const uint32_t M = n / 8;
            hp.tab.assign(2 * (size_t)n, 0);
            for (uint32_t i = 0; i < M; ++i)
                for (uint32_t k = 0; k < 8; ++k) {
                    const int32_t t = (int32_t)pw[((uint64_t)i * k) % n];
                    const size_t e = (size_t)k * M + i;
                    hp.tab[2 * e] = t;
                    hp.tab[2 * e + 1] = r8_multiplier(t, (int32_t)q, exact);
                }
            hp.stages = 2;   // butterfly tile + reduction tile (src/ntt_r8.h:149-159)
        } else {
            // Stage t (digit bits [b, b+3), b = L-3-3t): twiddle of output k
            // at low position bits r is root^(8^t r k mod n); table [t][k][r].
            const int S = L / 3;
            hp.tail_bits = L % 3;
            size_t total = 0;
            for (int t = 0; t < S; ++t) total += (size_t)8 << (L - 3 - 3 * t);
            hp.tab.assign(2 * (total ? total : 1), 0);
            size_t off = 0;
            for (int t = 0; t < S; ++t) {
                const int b = L - 3 - 3 * t;
                const uint64_t s8 = (uint64_t)1 << (3 * t);
                for (uint32_t k = 0; k < 8; ++k)
                    for (uint32_t r = 0; r < (1u << b); ++r) {
                        const int32_t tv = (int32_t)pw[(s8 * r * k) % n];
                        const size_t e = off + ((size_t)k << b) + r;
                        hp.tab[2 * e] = tv;
                        hp.tab[2 * e + 1] = r8_multiplier(tv, (int32_t)q, exact);
                    }
                off += (size_t)8 << b;
            }
            if (hp.tail_bits) {
                const int R = 1 << hp.tail_bits;
                for (int m = 0; m < R; ++m)
                    for (int k = 0; k < R; ++k)
                        hp.ftail[R * m + k] = r8_signed(pw[((uint64_t)(n / R) * m * k) % n], q);
                hp.tail_wq = r8_multiplier(1, (int32_t)q, exact);
            }
            hp.stages = 2 * S + (hp.tail_bits ? 2 : 0);
        }
        break;
    }
    case K_BITREV_I16:
        hp.stages = 1;
        break;
    case K_FULL_BARRETT_I16: {
        const int64_t fs = factor <= (q - 1) / 2 ? factor : factor - q;   // full_reduction_kernels.cc:186
        hp.fb_fs = (int32_t)fs;
        hp.fb_wq = fb_multiplier((int32_t)fs, (int32_t)q);
        hp.stages = 1;
        break;
    }
    }
    if ((flags & FLAG_SCALE_NINV) && !is32) {
        // the FULL_BARRETT_MULTIPLICATION<n, q, n^-1> unit fused after the inverse
        // (src/project.cpp:154, src/standalone_units.h:40)
        const int64_t ninv = modinv(n, q);
        const int64_t fs = ninv <= (q - 1) / 2 ? ninv : ninv - q;
        hp.fb_fs = (int32_t)fs;
        hp.fb_wq = fb_multiplier((int32_t)fs, (int32_t)q);
        hp.stages += 1;
    }
    return GBNTT_OK;
}

}  // namespace gbntt
