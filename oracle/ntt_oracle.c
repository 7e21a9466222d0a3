/*
 * ntt_oracle.c -- CPU restatement of the AIE1 NTT artifact's hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU baseline.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may load this
 * library.  The GPU product never links or calls it.
 *
 * Every function cites the reference file:line it restates (paths inside the
 * reference project).  The AIE1 vector semantics emulated here are:
 *   - SRS (shift-round-saturate) with rounding mode symmetric_zero, i.e. round
 *     to nearest with ties toward zero (set_modes_ntt_layer,
 *     src/kernels/ntt_r2_kernels.cc:543-547);
 *   - saturation mode none: conversions to int16/int32 keep the low bits
 *     (two's-complement wrap);
 *   - floor rounding for the sign extraction of the full Barrett kernel
 *     (src/kernels/full_reduction_kernels.cc:228).
 * Parity status: tables pinned against the reference's own twiddle.h /
 * auxiliary.h compiled here (tests/golden/ref_tables.json); kernel loops
 * pinned against the O(n^2) DFT below (canonical residues) and round trips.
 */
#include "ntt_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* number theory                                                             */
/* ------------------------------------------------------------------------- */

/* src/twiddle.h:18-23 */
uint32_t orc_bitrev(uint32_t a, int bits) {
    uint32_t r = 0;
    for (int i = 0; i < bits; i++)
        if (a & (1u << i)) r |= 1u << (bits - 1 - i);
    return r;
}

int64_t orc_powmod(int64_t base, uint64_t e, int64_t q) {
    __int128 r = 1, b = ((base % q) + q) % q;
    while (e) {
        if (e & 1) r = (r * b) % q;
        b = (b * b) % q;
        e >>= 1;
    }
    return (int64_t)r;
}

/* src/twiddle.h:61-69: reduce to [-(q-1)/2, (q-1)/2] (C remainder keeps the
 * dividend's sign, then one conditional correction). */
int64_t orc_red_neg(int64_t a, int64_t q) {
    a = a % q;
    if (a > (q - 1) / 2) a -= q;
    else if (a < -(q - 1) / 2) a += q;
    return a;
}

/* src/twiddle.h:35-49 and src/auxiliary.h:66-79 (both return the inverse in [0,q)). */
int64_t orc_modinv(int64_t n, int64_t m) {
    int64_t a = n, b = m, x0 = 1, x1 = 0;
    while (b) {
        int64_t qq = a / b, t = a % b;
        a = b; b = t;
        t = x1; x1 = x0 - qq * x1; x0 = t;
    }
    return (x0 % m + m) % m;
}

/* src/auxiliary.h:35-46: the smallest L with root^(2^L) == 1 (mod q), L <= 100.
 * Power<> (auxiliary.h:26-32) is only exact for power-of-two exponents, which
 * is the only way DETERMINE_LOG_ROOT_SIZE uses it. */
int orc_log_root_order(int64_t q, int64_t root) {
    int64_t x = ((root % q) + q) % q;
    for (int L = 0; L <= 100; L++) {
        if (x == 1 % q) return L;
        x = (int64_t)(((__int128)x * x) % q);
    }
    return -1;
}

/* src/twiddle.h:28-31: round<T>(a) = T(a + 0.5), a conversion that truncates
 * toward zero, so negative inputs are not rounded to nearest (-7887.43 ->
 * -7886).  The reference evaluates a = num/den in long double; num/den is
 * never within the long-double error of a half-integer for the table values
 * (den odd, |num/den| < 2^31), so the exact rational evaluation below gives
 * the same integers on every host. */
int64_t orc_round_trunc_half(int64_t num, int64_t den) {
    __int128 n2 = (__int128)2 * num + den, d2 = (__int128)2 * den;
    return (int64_t)(n2 / d2); /* C division truncates toward zero */
}

/* src/twiddle.h:96: the call round(float(tw * 2^16) / float(q)) cannot deduce
 * T of the template round<T>, so it binds to C's round(): IEEE single
 * precision conversion and division, then round half away from zero. */
int16_t orc_kyber_wq(int16_t tw, int32_t q) {
    volatile float num = (float)((int32_t)tw * 65536);
    volatile float quo = num / (float)q;
    return (int16_t)round((double)quo);
}

/* src/twiddle.h:372: round(float(int64(tw) << 31) / float(q)), again C's
 * round() on single-precision values.  Up to ~64 off the exact multiplier. */
int32_t orc_r8_wq_float(int32_t tw, int32_t q) {
    volatile float num = (float)((int64_t)tw << 31);
    volatile float quo = num / (float)q;
    return (int32_t)round((double)quo);
}

/* Exact nearest K=31 multiplier (no ties: q is odd).  Used by the chained
 * radix-8 transform so that every output is correct modulo q. */
int32_t orc_r8_wq_exact(int32_t tw, int32_t q) {
    int64_t num = (int64_t)tw << 31;
    return (int32_t)((2 * (__int128)num + q) / (2 * (__int128)q));
}

/* src/kernels/full_reduction_kernels.cc:187:
 * int16(std::round(float(int32(F_s) << 16) / float(q) + 0.5f)), all in float. */
int16_t orc_fb_wq(int32_t fs, int32_t q) {
    volatile float num = (float)(fs * 65536);
    volatile float quo = num / (float)q;
    volatile float sum = quo + 0.5f;
    return (int16_t)roundf(sum);
}

/* ------------------------------------------------------------------------- */
/* AIE1 lane arithmetic                                                       */
/* ------------------------------------------------------------------------- */

static inline int16_t w16(int64_t v) { return (int16_t)(uint16_t)(uint64_t)v; }
static inline int32_t w32(int64_t v) { return (int32_t)(uint32_t)(uint64_t)v; }

/* SRS by s with rounding mode symmetric_zero (nearest, ties toward zero). */
static inline int64_t srs_sz(int64_t v, int s) {
    int64_t half = (int64_t)1 << (s - 1);
    if (v >= 0) return (v + half - 1) >> s;
    return -((-v + half - 1) >> s);
}

/* Partial Barrett multiplication, int16, K = 16
 * (src/kernels/ntt_r2_kernels.cc:306-368; identical in ntt_r4_kernels.cc:28-94):
 * mul16 forms a*w' + a*w' and SRS shifts by K+1 = 17; the second mul16 forms
 * a*w - m'*q, kept as int16. */
static inline int16_t bm16(int16_t a, int16_t tw, int16_t wq, int32_t q) {
    int64_t mb = w16(srs_sz(2 * (int64_t)a * wq, 17));
    return w16((int64_t)a * tw - mb * q);
}

/* Partial Barrett reduction, int16 (src/kernels/ntt_r2_kernels.cc:372-419):
 * constant multiplier c = int16(2^16/q + 0.5) (:388), output a - m'*q. */
static inline int16_t br16(int16_t a, int16_t c, int32_t q) {
    int64_t mb = w16(srs_sz(2 * (int64_t)a * c, 17));
    return w16((int64_t)a - mb * q);
}

/* Partial Barrett multiplication, int32, K = 32
 * (src/kernels/ntt_r2_int32_kernels.cc:32-88): m' = SRS_32(a*w') in acc80,
 * then a*w - m'*q converted to int32. */
static inline int32_t bm32(int32_t a, int32_t tw, int32_t wq, int64_t q) {
    int64_t mb = w32(srs_sz((int64_t)a * wq, 32));
    return w32((int64_t)a * tw - mb * q);
}

/* Partial Barrett reduction, int32 (src/kernels/ntt_r2_int32_kernels.cc:91-136):
 * c = int32(2^32/q + 0.5) (:102). */
static inline int32_t br32(int32_t a, int32_t c, int64_t q) {
    int64_t mb = w32(srs_sz((int64_t)a * c, 32));
    return w32((int64_t)a - mb * q);
}

/* ------------------------------------------------------------------------- */
/* plan                                                                       */
/* ------------------------------------------------------------------------- */

struct orc_plan {
    int kind, n, L, layers, r8_exact;
    int64_t q, root, factor;
    /* radix-2 forward int16/int32 and int32 inverse: per layer [tw n/2 | w' n/2] */
    int32_t* comb;
    /* radix-2 inverse int16: per layer twiddles (n/2) and multipliers (n/2) */
    int32_t* itw;
    int32_t* iwq;
    /* radix-4: per layer [tw n | w' n] */
    int32_t* r4;
    int16_t r4_fneg, r4_wc;
    /* radix-8: F8 in the reference MAC layout (64), F8 by [m][k], reduction
     * twiddles/multipliers in the reference layout (stage 0, n each) */
    int16_t r8_f8_ref[64];
    int16_t r8_f8[8][8];
    int32_t* r8_tw_ref;
    int32_t* r8_wq_ref;
    /* chained radix-8: stage t twiddle for (i, k) at [t][i*8 + k] (i < n/8) */
    int r8_stages, r8_tail_bits;
    int32_t* r8c_tw;
    int32_t* r8c_wq;
    int16_t r8_tail_f[4][4];
    int32_t r8_tail_wq;
    /* constants */
    int32_t c16, c32;
    int16_t fb_fs, fb_wq;
};

static int ilog2_exact(int64_t n) {
    int l = 0;
    if (n <= 0 || (n & (n - 1))) return -1;
    while ((1LL << l) < n) l++;
    return l;
}

/* src/twiddle.h:108-119 (compute_twiddle_factors) and :124-136
 * (compute_barret_factors): tw[bitrev_{L-1}(i)] = red_neg(root^(+-i)) for
 * i < 2^(L-1), w'[i] = round<T>(tw[i] * 2^K / q). */
static void t1_compact(int64_t q, int64_t root, int L, int K, int inverse,
                       int64_t* tw, int64_t* wq) {
    int64_t len = (int64_t)1 << (L - 1);
    int64_t F = inverse ? orc_modinv(root, q) : root;
    int64_t cur = 1;
    tw[0] = 1;
    for (int64_t i = 1; i < len; i++) {
        cur = orc_red_neg(cur * F, q);
        tw[orc_bitrev((uint32_t)i, L - 1)] = cur;
    }
    for (int64_t i = 0; i < len; i++) wq[i] = orc_round_trunc_half(tw[i] * ((int64_t)1 << K), q);
}

/* src/twiddle.h:141-170 (expand_factors): layer l repeats the first 2^l
 * factors n/2^(l+1) times, twiddles in [0,n/2), multipliers in [n/2,n). */
static void t1_expand(int n, const int64_t* tw, const int64_t* wq, int layer, int32_t* out) {
    int64_t nf = (int64_t)1 << layer;
    for (int j = 0; j < n / 2; j++) {
        out[j] = (int32_t)tw[j % nf];
        out[n / 2 + j] = (int32_t)wq[j % nf];
    }
}

/* src/twiddle.h:74-87 (compute_twiddle_factors_kyber) and :92-102
 * (compute_barrett_factors_kyber): natural order, int16 arithmetic. */
static void kyber_tables(int32_t q, int32_t root, int size, int inverse, int16_t* tw, int16_t* wq) {
    int16_t F = (int16_t)(inverse ? orc_modinv(root, q) : root);
    int16_t cur = 1;
    tw[0] = 1;
    for (int i = 1; i < size; i++) {
        cur = (int16_t)(((int32_t)cur * (int32_t)F) % q);
        cur = (int16_t)orc_red_neg(cur, q);
        tw[i] = cur;
    }
    for (int i = 0; i < size; i++) wq[i] = orc_kyber_wq(tw[i], q);
}

/* src/twiddle.h:177-222 (expand_twiddle_and_barrett_factors): pairs
 * (tw[2g*rep], tw[(2g+1)*rep]) repeated rep = n/2^(layer+1) times, for
 * g < 2^layer / 2.  Layer 0 writes nothing (the vector stays zero). */
static void t2_expand(int n, const int16_t* tw, const int16_t* wq, int layer, int32_t* otw, int32_t* owq) {
    int rep = n >> (layer + 1);
    int nf = 1 << layer;
    int w = 0;
    memset(otw, 0, sizeof(int32_t) * (size_t)(n / 2));
    memset(owq, 0, sizeof(int32_t) * (size_t)(n / 2));
    for (int g = 0; g < nf / 2; g++) {
        int i1 = g * 2 * rep, i2 = i1 + rep;
        for (int r = 0; r < rep; r++) {
            otw[w] = tw[i1]; owq[w] = wq[i1]; w++;
            otw[w] = tw[i2]; owq[w] = wq[i2]; w++;
        }
    }
}

/* src/twiddle.h:403-429 (expand_factors_layer_r4) for ROOT_SIZE == n. */
static void r4_expand(int n, int32_t q, const int16_t* tw, const int16_t* wq, int layer, int max_r4, int32_t* out) {
    int N = 1;
    for (int i = 0; i <= layer; i++) N *= 4;
    /* modular_exponentation (twiddle.h:53-57) reduces 4^(R-l-1) modulo q */
    unsigned op = 1;
    for (int i = 0; i < max_r4 - layer - 1; i++) op = (op * 4u) % (unsigned)q;
    int bits = 2 * layer;
    for (unsigned n1 = 0; n1 < 4; n1++) {
        for (int t = 0; t < n / 4; t++) {
            int k2 = t % (N / 4);
            int idx = (n / 4) * (int)n1 + t;
            unsigned long long power = ((unsigned long long)op * n1 * orc_bitrev((uint32_t)k2, bits)) % (unsigned)n;
            out[idx] = tw[power];
            out[n + idx] = wq[power];
        }
    }
}

static inline int16_t r8_signed(int32_t f, int32_t q) {
    /* src/twiddle.h:334: f < (q-1)/2 ? f : f - q */
    return (int16_t)(f < (q - 1) / 2 ? f : f - q);
}

orc_plan* orc_plan_create(int kind, int n, int64_t q, int64_t root, int64_t factor,
                          int r8_exact, int* err) {
    int e = 0;
    orc_plan* p = NULL;
    int L = ilog2_exact(n);
    int is32 = (kind == ORC_R2_I32_FWD || kind == ORC_R2_I32_INV);
    if (kind < 0 || kind > ORC_R4_I16_INV) { e = 6; goto fail; }
    if (kind == ORC_FULL_BARRETT_I16) {
        if (n < 1) { e = 1; goto fail; }   /* elementwise: any length */
        if (L < 0) L = 0;
    } else if (L < 1 || L > 24) { e = 1; goto fail; }
    if (kind != ORC_BITREV_I16) {
        if (q < 3 || !(q & 1)) { e = 2; goto fail; }
        if (is32 ? (q >= 1431655765LL) : (q >= 21846)) { e = 4; goto fail; }
    }
    if (kind != ORC_BITREV_I16 && kind != ORC_FULL_BARRETT_I16) {
        if (orc_log_root_order(q, root) != L) { e = 3; goto fail; }
    }
    if ((kind == ORC_R4_I16_FWD || kind == ORC_R4_I16_INV) && (L & 1)) { e = 5; goto fail; }
    if (kind == ORC_R8_I16_STAGE && n < 16) { e = 1; goto fail; }
    if (kind == ORC_R8_I16_FWD && n < 8) { e = 1; goto fail; }
    if (kind == ORC_FULL_BARRETT_I16 && (factor < 0 || factor >= q)) { e = 2; goto fail; }

    p = (orc_plan*)calloc(1, sizeof(orc_plan));
    p->kind = kind; p->n = n; p->L = L; p->q = q; p->root = root; p->factor = factor;
    p->r8_exact = r8_exact;
    /* ntt_r2_kernels.cc:388 and ntt_r2_int32_kernels.cc:102 */
    if (q >= 3) {
        p->c16 = (int32_t)orc_round_trunc_half(65536, q);
        p->c32 = (int32_t)orc_round_trunc_half((int64_t)1 << 32, q);
    }

    switch (kind) {
    case ORC_R2_I16_FWD:
    case ORC_R2_I32_FWD:
    case ORC_R2_I32_INV: {
        /* determine_factors (src/twiddle.h:226-243); src/ntt.h:80, src/ntt_int32.h:61 */
        int K = is32 ? 32 : 16;
        int inverse = (kind == ORC_R2_I32_INV);
        int64_t* tw = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n / 2));
        int64_t* wq = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n / 2));
        t1_compact(q, root, L, K, inverse, tw, wq);
        p->layers = L;
        p->comb = (int32_t*)malloc(sizeof(int32_t) * (size_t)n * (size_t)L);
        for (int i = 0; i < L; i++) {
            int layer = inverse ? (L - i - 1) : i; /* twiddle.h:238 (GS layers reversed) */
            t1_expand(n, tw, wq, layer, p->comb + (size_t)i * (size_t)n);
        }
        free(tw); free(wq);
        break;
    }
    case ORC_R2_I16_INV: {
        /* determine_twiddle_and_barrett (src/twiddle.h:248-266), called with
         * KERNEL_TYPE CT_NO_to_BO (src/ntt.h:75), so layer i uses table i. */
        int16_t* tw = (int16_t*)malloc(sizeof(int16_t) * (size_t)n);
        int16_t* wq = (int16_t*)malloc(sizeof(int16_t) * (size_t)n);
        kyber_tables((int32_t)q, (int32_t)root, n, 1, tw, wq);
        p->layers = L;
        p->itw = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n / 2) * (size_t)L);
        p->iwq = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n / 2) * (size_t)L);
        for (int i = 0; i < L; i++)
            t2_expand(n, tw, wq, i, p->itw + (size_t)i * (size_t)(n / 2), p->iwq + (size_t)i * (size_t)(n / 2));
        free(tw); free(wq);
        break;
    }
    case ORC_R4_I16_FWD:
    case ORC_R4_I16_INV: {
        /* determine_factors_radix4 (src/twiddle.h:432-454), ROOT_4
         * (src/ntt_r4.h:46), constant multiplier (ntt_r4_kernels.cc:112-113). */
        int inverse = (kind == ORC_R4_I16_INV);
        int16_t* tw = (int16_t*)malloc(sizeof(int16_t) * (size_t)n);
        int16_t* wq = (int16_t*)malloc(sizeof(int16_t) * (size_t)n);
        kyber_tables((int32_t)q, (int32_t)root, n, inverse, tw, wq);
        int R = L / 2;
        p->layers = R;
        p->r4 = (int32_t*)malloc(sizeof(int32_t) * (size_t)(2 * n) * (size_t)R);
        for (int i = 0; i < R; i++) r4_expand(n, (int32_t)q, tw, wq, i, R, p->r4 + (size_t)i * (size_t)(2 * n));
        int64_t rt = inverse ? orc_modinv(root, q) : root;
        int64_t root4 = orc_powmod(rt, (uint64_t)(n / 4), q);
        int64_t fneg = root4 <= (q - 1) / 2 ? root4 : root4 - q;
        p->r4_fneg = (int16_t)fneg;
        p->r4_wc = (int16_t)orc_round_trunc_half(fneg * 65536, q);
        free(tw); free(wq);
        break;
    }
    case ORC_R8_I16_STAGE:
    case ORC_R8_I16_FWD: {
        /* determine_factors_r8 (src/twiddle.h:273-399). */
        int32_t qq = (int32_t)q;
        int64_t root8 = orc_powmod(root, (uint64_t)(n / 8), q);
        int32_t tw8[8];
        tw8[0] = 1;
        for (int i = 1; i < 8; i++) tw8[i] = (int32_t)(((int64_t)tw8[i - 1] * root8) % q);
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++)
                for (int k = 0; k < 4; k++)
                    for (int l = 0; l < 4; l++) {
                        int in_ = 4 * i + l, outk = 4 * j + k;
                        p->r8_f8_ref[32 * i + 16 * j + 4 * k + (int)orc_bitrev((uint32_t)l, 2)] =
                            r8_signed(tw8[(outk * in_) % 8], qq);
                    }
        for (int m = 0; m < 8; m++)
            for (int k = 0; k < 8; k++) p->r8_f8[m][k] = r8_signed(tw8[(m * k) % 8], qq);
        int32_t* pw = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
        pw[0] = 1;
        for (int i = 1; i < n; i++) pw[i] = (int32_t)(((int64_t)pw[i - 1] * root) % q);
        /* the reference layout pairs 8-NTTs, so it needs n/8 even (n >= 16) */
        p->r8_tw_ref = (int32_t*)calloc((size_t)(n < 16 ? 16 : n), sizeof(int32_t));
        p->r8_wq_ref = (int32_t*)calloc((size_t)(n < 16 ? 16 : n), sizeof(int32_t));
        for (int i = 0; i < (n >= 16 ? n / 8 : 0); i++)
            for (int j = 0; j < 8; j++) {
                int idx = 2 * (i / 2) * 8 + j * 2 + (i % 2); /* twiddle.h:381-389 */
                int32_t t = pw[((int64_t)i * j) % n];
                p->r8_tw_ref[idx] = t;
                p->r8_wq_ref[idx] = orc_r8_wq_float(t, qq);
            }
        if (kind == ORC_R8_I16_STAGE) {
            p->layers = 1;
        } else {
            /* Chained stages (src/ntt_r8.h:15-19): stage t twiddle
             * w^(8^t * (i >> 3t) * k); a final radix-2^c stage when log2 n is
             * not a multiple of 3. */
            p->r8_stages = L / 3;
            p->r8_tail_bits = L % 3;
            p->layers = p->r8_stages + (p->r8_tail_bits ? 1 : 0);
            size_t per = (size_t)n; /* (n/8) * 8 */
            p->r8c_tw = (int32_t*)malloc(sizeof(int32_t) * per * (size_t)(p->r8_stages ? p->r8_stages : 1));
            p->r8c_wq = (int32_t*)malloc(sizeof(int32_t) * per * (size_t)(p->r8_stages ? p->r8_stages : 1));
            for (int t = 0; t < p->r8_stages; t++) {
                int64_t s8 = 1;
                for (int u = 0; u < t; u++) s8 *= 8;
                for (int i = 0; i < n / 8; i++)
                    for (int k = 0; k < 8; k++) {
                        int64_t pwr = (s8 * (int64_t)(i >> (3 * t)) * k) % n;
                        int32_t tv = pw[pwr];
                        p->r8c_tw[(size_t)t * per + (size_t)i * 8 + (size_t)k] = tv;
                        p->r8c_wq[(size_t)t * per + (size_t)i * 8 + (size_t)k] =
                            r8_exact ? orc_r8_wq_exact(tv, qq) : orc_r8_wq_float(tv, qq);
                    }
            }
            if (p->r8_tail_bits) {
                int R = 1 << p->r8_tail_bits;
                for (int m = 0; m < R; m++)
                    for (int k = 0; k < R; k++)
                        p->r8_tail_f[m][k] = r8_signed(pw[((int64_t)(n / R) * m * k) % n], qq);
                p->r8_tail_wq = r8_exact ? orc_r8_wq_exact(1, qq) : orc_r8_wq_float(1, qq);
            }
        }
        free(pw);
        break;
    }
    case ORC_BITREV_I16:
        p->layers = 1;
        break;
    case ORC_FULL_BARRETT_I16: {
        /* src/kernels/full_reduction_kernels.cc:186-187 */
        int64_t fs = factor <= (q - 1) / 2 ? factor : factor - q;
        p->fb_fs = (int16_t)fs;
        p->fb_wq = orc_fb_wq((int32_t)fs, (int32_t)q);
        p->layers = 1;
        break;
    }
    }
    if (kind == ORC_R4_I16_INV) p->layers += 2; /* bitrev, r4 stages, bitrev */
    if (err) *err = 0;
    return p;
fail:
    if (err) *err = e;
    return NULL;
}

void orc_plan_destroy(orc_plan* p) {
    if (!p) return;
    free(p->comb); free(p->itw); free(p->iwq); free(p->r4);
    free(p->r8_tw_ref); free(p->r8_wq_ref); free(p->r8c_tw); free(p->r8c_wq);
    free(p);
}

int orc_plan_layers(const orc_plan* p) { return p->layers; }

int orc_elem_bytes(const orc_plan* p) {
    return (p->kind == ORC_R2_I32_FWD || p->kind == ORC_R2_I32_INV) ? 4 : 2;
}

int64_t orc_plan_table(const orc_plan* p, int which, int layer, int64_t* dst) {
    int n = p->n;
    const int32_t* src = NULL;
    int64_t len = 0;
    if (which == 0) {
        if (p->comb && layer < p->layers) { src = p->comb + (size_t)layer * (size_t)n; len = n; }
        else if (p->itw && layer < p->layers) { src = p->itw + (size_t)layer * (size_t)(n / 2); len = n / 2; }
        else if (p->r4 && layer < p->L / 2) { src = p->r4 + (size_t)layer * (size_t)(2 * n); len = 2 * n; }
    } else if (which == 1) {
        if (p->iwq && layer < p->layers) { src = p->iwq + (size_t)layer * (size_t)(n / 2); len = n / 2; }
    } else if (which == 2) {
        if (p->r8_tw_ref) {
            if (dst) for (int i = 0; i < 64; i++) dst[i] = p->r8_f8_ref[i];
            return 64;
        }
    } else if (which == 3) {
        if (p->r8_tw_ref) { src = p->r8_tw_ref; len = n; }
    } else if (which == 4) {
        if (p->r8_wq_ref) { src = p->r8_wq_ref; len = n; }
    } else if (which == 5) {
        int64_t c[6] = {p->c16, p->c32, p->r4_fneg, p->r4_wc, p->fb_fs, p->fb_wq};
        if (dst) for (int i = 0; i < 6; i++) dst[i] = c[i];
        return 6;
    }
    if (src && dst)
        for (int64_t i = 0; i < len; i++) dst[i] = src[i];
    return len;
}

/* ------------------------------------------------------------------------- */
/* per-tile kernels (constant-geometry form, one polynomial)                  */
/* ------------------------------------------------------------------------- */

/* NTT_CT_NO_to_BO, int16 (src/kernels/ntt_r2_kernels.cc:434-472): for each
 * half, barrett_reduction of the top quarter (:443/:458),
 * barrett_multiplication of the bottom quarter (:447/:462), then
 * CT_add_sub_interleave (:451/:466, :101-149): out[2j] = u+v, out[2j+1] = u-v. */
static void k_r2_i16_fwd(const orc_plan* p, int layer, const int16_t* in, int16_t* out) {
    int n = p->n, h = n / 2;
    int32_t q = (int32_t)p->q;
    int16_t c = (int16_t)p->c16;
    const int32_t* f = p->comb + (size_t)layer * (size_t)n;
    for (int j = 0; j < h; j++) {
        int16_t u = br16(in[j], c, q);
        int16_t v = bm16(in[h + j], (int16_t)f[j], (int16_t)f[h + j], q);
        out[2 * j] = w16((int32_t)u + v);
        out[2 * j + 1] = w16((int32_t)u - v);
    }
}

/* NTT_CT_BO_to_NO, int16 (src/kernels/ntt_r2_kernels.cc:484-540).
 * Layer 0: GS_unshuffle_add_sub with pair unshuffle (:491-494, :37-99).
 * Other layers: barrett_multiplication of the bottom half (:504),
 * barrett_reduction of the top half (:511, :526), then CT_add_sub_unshuffle
 * (:516, :531, :152-251) into quarters Q0..Q3, or CT_add_sub (:519, :534,
 * :254-295) in the last layer. */
static void k_r2_i16_inv(const orc_plan* p, int layer, const int16_t* in, int16_t* out) {
    int n = p->n, h = n / 2;
    int32_t q = (int32_t)p->q;
    int16_t c = (int16_t)p->c16;
    if (layer == 0) {
        for (int pp = 0; pp < h; pp++) {
            int16_t s = w16((int32_t)in[2 * pp] + in[2 * pp + 1]);
            int16_t d = w16((int32_t)in[2 * pp] - in[2 * pp + 1]);
            int base = (pp & 1) ? h : 0;
            out[base + 2 * (pp >> 1)] = s;
            out[base + 2 * (pp >> 1) + 1] = d;
        }
        return;
    }
    const int32_t* tw = p->itw + (size_t)layer * (size_t)h;
    const int32_t* wq = p->iwq + (size_t)layer * (size_t)h;
    int last = (layer == p->L - 1);
    for (int j = 0; j < h; j++) {
        int16_t u = br16(in[j], c, q);
        int16_t v = bm16(in[h + j], (int16_t)tw[j], (int16_t)wq[j], q);
        int16_t s = w16((int32_t)u + v), d = w16((int32_t)u - v);
        if (last) {
            out[j] = s;
            out[h + j] = d;
        } else {
            int pr = j >> 1, e = j & 1;
            int idx = (pr >> 1) * 2 + e + ((pr & 1) ? h : 0);
            out[idx] = s;
            out[idx + n / 4] = d;
        }
    }
}

/* NTT_CT_NO_to_BO, int32 (src/kernels/ntt_r2_int32_kernels.cc:267-295). */
static void k_r2_i32_fwd(const orc_plan* p, int layer, const int32_t* in, int32_t* out) {
    int n = p->n, h = n / 2;
    int64_t q = p->q;
    int32_t c = p->c32;
    const int32_t* f = p->comb + (size_t)layer * (size_t)n;
    for (int j = 0; j < h; j++) {
        int32_t u = br32(in[j], c, q);
        int32_t v = bm32(in[h + j], f[j], f[h + j], q);
        out[2 * j] = w32((int64_t)u + v);     /* ntt_int32_CT_add_sub_interleave :138-192 */
        out[2 * j + 1] = w32((int64_t)u - v);
    }
}

/* NTT_GS_BO_to_NO, int32 (src/kernels/ntt_r2_int32_kernels.cc:305-336):
 * GS_unshuffle_add_sub (:196-256) then reduction of the sums and Barrett
 * multiplication of the differences. */
static void k_r2_i32_inv(const orc_plan* p, int layer, const int32_t* in, int32_t* out) {
    int n = p->n, h = n / 2;
    int64_t q = p->q;
    int32_t c = p->c32;
    const int32_t* f = p->comb + (size_t)layer * (size_t)n;
    for (int j = 0; j < h; j++) {
        int32_t s = w32((int64_t)in[2 * j] + in[2 * j + 1]);
        int32_t d = w32((int64_t)in[2 * j] - in[2 * j + 1]);
        out[j] = br32(s, c, q);
        out[h + j] = bm32(d, f[j], f[h + j], q);
    }
}

/* barrett_multiplication_constant (src/kernels/ntt_r4_kernels.cc:96-149). */
static inline int16_t bmc16(int16_t a, int16_t fneg, int16_t wc, int32_t q) {
    int64_t mb = w16(srs_sz(2 * (int64_t)a * wc, 17));
    return w16((int64_t)a * fneg - mb * q);
}

/* NTT_R4 layer (src/kernels/ntt_r4_kernels.cc:243-261): four
 * barrett_multiplication loops (:251-254), omega_4 times the 2nd and 4th
 * input (:256), r4_matmul (:153-235) with outputs in per-4-NTT bit-reversed
 * order, left unreduced. */
static void k_r4(const orc_plan* p, const int32_t* f, const int16_t* in, int16_t* out) {
    int n = p->n, n4 = n / 4;
    int32_t q = (int32_t)p->q;
    for (int t = 0; t < n4; t++) {
        int16_t A[4];
        for (int n1 = 0; n1 < 4; n1++) {
            int idx = n1 * n4 + t;
            A[n1] = bm16(in[idx], (int16_t)f[idx], (int16_t)f[n + idx], q);
        }
        int16_t A5 = bmc16(A[1], p->r4_fneg, p->r4_wc, q);
        int16_t A6 = bmc16(A[3], p->r4_fneg, p->r4_wc, q);
        int32_t y0 = (int32_t)A[0] + A[1] + A[2] + A[3];
        int32_t y1 = (int32_t)A[0] + A5 - A[2] - A6;
        int32_t y2 = (int32_t)A[0] - A[1] + A[2] - A[3];
        int32_t y3 = (int32_t)A[0] - A5 - A[2] + A6;
        out[4 * t + 0] = w16(y0);
        out[4 * t + 1] = w16(y2);
        out[4 * t + 2] = w16(y1);
        out[4 * t + 3] = w16(y3);
    }
}

/* One radix-8 stage: NTT_R8_LAYERS (src/kernels/ntt_r8_kernels.cc:214-404)
 * forms y[i][k] = sum_m x[i + M m] F8[m][k] in int32; NTT_R8_REDUCTION
 * (:30-177) forms m' = SRS_31(y w') (:59-106), truncates it to int16
 * (:120-134), and writes y*w - m'*q as int16 to out[8i + bitrev3(k)]
 * (:137-175; the permutation is described at :152-154). */
static inline int16_t r8_reduce(int32_t y, int32_t tw, int32_t wq, int32_t q) {
    int64_t mb = w32(srs_sz((int64_t)y * wq, 31));
    int16_t m16 = w16(mb);
    return w16((int64_t)y * tw - (int64_t)m16 * q);
}

static void k_r8_stage_ref(const orc_plan* p, const int16_t* in, int16_t* out) {
    int n = p->n, M = n / 8;
    int32_t q = (int32_t)p->q;
    for (int i = 0; i < M; i++)
        for (int k = 0; k < 8; k++) {
            int64_t y = 0;
            for (int m = 0; m < 8; m++) y += (int64_t)in[i + M * m] * p->r8_f8[m][k];
            int idx = 16 * (i / 2) + 2 * k + (i % 2);
            out[8 * i + (int)orc_bitrev((uint32_t)k, 3)] = r8_reduce(w32(y), p->r8_tw_ref[idx], p->r8_wq_ref[idx], q);
        }
}

static void k_r8_chained(const orc_plan* p, int stage, const int16_t* in, int16_t* out) {
    int n = p->n;
    int32_t q = (int32_t)p->q;
    if (stage < p->r8_stages) {
        int M = n / 8;
        const int32_t* tw = p->r8c_tw + (size_t)stage * (size_t)n;
        const int32_t* wq = p->r8c_wq + (size_t)stage * (size_t)n;
        for (int i = 0; i < M; i++)
            for (int k = 0; k < 8; k++) {
                int64_t y = 0;
                for (int m = 0; m < 8; m++) y += (int64_t)in[i + M * m] * p->r8_f8[m][k];
                out[8 * i + (int)orc_bitrev((uint32_t)k, 3)] = r8_reduce(w32(y), tw[i * 8 + k], wq[i * 8 + k], q);
            }
    } else {
        int c = p->r8_tail_bits, R = 1 << c, M = n / R;
        for (int i = 0; i < M; i++)
            for (int k = 0; k < R; k++) {
                int64_t y = 0;
                for (int m = 0; m < R; m++) y += (int64_t)in[i + M * m] * p->r8_tail_f[m][k];
                out[R * i + (int)orc_bitrev((uint32_t)k, c)] = r8_reduce(w32(y), 1, p->r8_tail_wq, q);
            }
    }
}

/* bitreverse_improved_kernel (src/kernels/bitreverse_kernels.cc:54-143):
 * out[bitrev(i)] = in[i]. */
static void k_bitrev(int n, int L, const int16_t* in, int16_t* out) {
    for (int i = 0; i < n; i++) out[orc_bitrev((uint32_t)i, L)] = in[i];
}

/* full_barrett_multiplication_kernel (src/kernels/full_reduction_kernels.cc:33-195). */
static void k_full_barrett(const orc_plan* p, const int16_t* in, int16_t* out) {
    int32_t q = (int32_t)p->q;
    for (int i = 0; i < p->n; i++) {
        int16_t x = in[i];
        int16_t mb = w16(srs_sz((int64_t)x * p->fb_wq, 16));   /* :204-212 */
        int64_t r = (int64_t)x * p->fb_fs - (int64_t)q * mb;     /* :234-238 */
        int16_t lo = w16(r);                                      /* :241 */
        int16_t sign = w16(r >> 16);                              /* :242, floor rounding */
        out[i] = w16((int64_t)lo - (int64_t)sign * q);            /* :261-272 */
    }
}

int orc_run_layer(const orc_plan* p, int layer, const void* in, void* out) {
    if (layer < 0 || layer >= p->layers) return -1;
    switch (p->kind) {
    case ORC_R2_I16_FWD: k_r2_i16_fwd(p, layer, (const int16_t*)in, (int16_t*)out); break;
    case ORC_R2_I16_INV: k_r2_i16_inv(p, layer, (const int16_t*)in, (int16_t*)out); break;
    case ORC_R2_I32_FWD: k_r2_i32_fwd(p, layer, (const int32_t*)in, (int32_t*)out); break;
    case ORC_R2_I32_INV: k_r2_i32_inv(p, layer, (const int32_t*)in, (int32_t*)out); break;
    case ORC_R4_I16_FWD: k_r4(p, p->r4 + (size_t)layer * (size_t)(2 * p->n), (const int16_t*)in, (int16_t*)out); break;
    case ORC_R4_I16_INV:
        if (layer == 0 || layer == p->layers - 1) k_bitrev(p->n, p->L, (const int16_t*)in, (int16_t*)out);
        else k_r4(p, p->r4 + (size_t)(layer - 1) * (size_t)(2 * p->n), (const int16_t*)in, (int16_t*)out);
        break;
    case ORC_R8_I16_STAGE: k_r8_stage_ref(p, (const int16_t*)in, (int16_t*)out); break;
    case ORC_R8_I16_FWD: k_r8_chained(p, layer, (const int16_t*)in, (int16_t*)out); break;
    case ORC_BITREV_I16: k_bitrev(p->n, p->L, (const int16_t*)in, (int16_t*)out); break;
    case ORC_FULL_BARRETT_I16: k_full_barrett(p, (const int16_t*)in, (int16_t*)out); break;
    default: return -1;
    }
    return 0;
}

/* Runs the tiles of the pipeline one after another (the graph's connect()
 * chain, e.g. src/ntt.h:107-116) with two ping-pong buffers. */
static void run_one(const orc_plan* p, const void* in, void* out, void* s0, void* s1) {
    size_t bytes = (size_t)p->n * (size_t)orc_elem_bytes(p);
    const void* cur = in;
    for (int l = 0; l < p->layers; l++) {
        void* dst = (l == p->layers - 1) ? out : ((l & 1) ? s1 : s0);
        orc_run_layer(p, l, cur, dst);
        cur = dst;
    }
    if (p->layers == 0) memcpy(out, in, bytes);
}

int orc_execute(const orc_plan* p, const void* in, void* out, int64_t batch) {
    size_t bytes = (size_t)p->n * (size_t)orc_elem_bytes(p);
    void* s0 = malloc(bytes);
    void* s1 = malloc(bytes);
    for (int64_t b = 0; b < batch; b++)
        run_one(p, (const char*)in + (size_t)b * bytes, (char*)out + (size_t)b * bytes, s0, s1);
    free(s0); free(s1);
    return 0;
}

/* the outputs of `count` polynomials reduced to [0, q) in place */
static void reduce_canonical(const orc_plan* p, void* out, int64_t count) {
    const int64_t total = count * (int64_t)p->n, q = p->q;
    if (orc_elem_bytes(p) == 2) {
        int16_t* y = (int16_t*)out;
        for (int64_t i = 0; i < total; i++) {
            int64_t r = y[i] % q;
            y[i] = (int16_t)(r < 0 ? r + q : r);
        }
    } else {
        int32_t* y = (int32_t*)out;
        for (int64_t i = 0; i < total; i++) {
            int64_t r = (int64_t)y[i] % q;
            y[i] = (int32_t)(r < 0 ? r + q : r);
        }
    }
}

typedef struct {
    const orc_plan* p;
    const char* in;
    char* out;
    int64_t b0, b1;
    int canonical;
} mt_arg;

static void* mt_worker(void* v) {
    mt_arg* a = (mt_arg*)v;
    size_t bytes = (size_t)a->p->n * (size_t)orc_elem_bytes(a->p);
    orc_execute(a->p, a->in + (size_t)a->b0 * bytes, a->out + (size_t)a->b0 * bytes, a->b1 - a->b0);
    if (a->canonical) reduce_canonical(a->p, a->out + (size_t)a->b0 * bytes, a->b1 - a->b0);
    return NULL;
}

int orc_execute_mt2(const orc_plan* p, const void* in, void* out, int64_t batch, int nthreads, int canonical) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > batch) nthreads = (int)(batch > 0 ? batch : 1);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    mt_arg* args = (mt_arg*)malloc(sizeof(mt_arg) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++) {
        args[t].p = p;
        args[t].in = (const char*)in;
        args[t].out = (char*)out;
        args[t].b0 = batch * t / nthreads;
        args[t].b1 = batch * (t + 1) / nthreads;
        args[t].canonical = canonical;
        pthread_create(&th[t], NULL, mt_worker, &args[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th); free(args);
    return 0;
}

int orc_execute_mt(const orc_plan* p, const void* in, void* out, int64_t batch, int nthreads) {
    if (nthreads <= 1 || batch <= 1) return orc_execute(p, in, out, batch);
    if (nthreads > batch) nthreads = (int)batch;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    mt_arg* args = (mt_arg*)malloc(sizeof(mt_arg) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++) {
        args[t].p = p;
        args[t].in = (const char*)in;
        args[t].out = (char*)out;
        args[t].b0 = batch * t / nthreads;
        args[t].b1 = batch * (t + 1) / nthreads;
        args[t].canonical = 0;
        pthread_create(&th[t], NULL, mt_worker, &args[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th); free(args);
    return 0;
}

void orc_dft(int n, int64_t q, int64_t root, int inverse, const int64_t* in, int64_t* out) {
    int64_t w = inverse ? orc_modinv(root, q) : root;
    for (int k = 0; k < n; k++) {
        int64_t wk = orc_powmod(w, (uint64_t)k, q), x = 1;
        __int128 acc = 0;
        for (int j = 0; j < n; j++) {
            int64_t v = ((in[j] % q) + q) % q;
            acc += (__int128)v * x;
            if ((j & 63) == 63) acc %= q;
            x = (int64_t)(((__int128)x * wk) % q);
        }
        out[k] = (int64_t)(acc % q);
    }
}

/* Exact transform in O(n log n), canonical residues: the iterative radix-2
 * Cooley-Tukey algorithm of the textbooks (bit-reversal permutation, then
 * log2 n layers of butterflies x +- w y mod q), with 64-bit products (q < 2^32).
 * Forward: natural-order input, DFT with `root` in bit-reversed order (the
 * order of every forward design of the reference); inverse: bit-reversed
 * input, DFT with root^-1 in natural order, no n^-1 (the inverse designs'
 * orders, README.md:157-160).  It restates no kernel of the reference: it is
 * the mathematical transform those kernels compute, checked against orc_dft
 * (the O(n^2) definition) in tests/test_oracle.py, and lets the tests check
 * canonical outputs at lengths where the O(n^2) sum is too slow. */
void orc_ntt_exact(int n, int64_t q, int64_t root, int inverse, const int64_t* in, int64_t* out) {
    int L = 0;
    while ((1 << L) < n) L++;
    const uint64_t uq = (uint64_t)q;
    const uint64_t w = (uint64_t)(inverse ? orc_modinv(root, q) : ((root % q) + q) % q);
    /* textbook form: bit-reversed copy of the natural-order sequence, then
     * butterflies of span 1, 2, 4, ... give the DFT in natural order */
    uint64_t* a = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)n);
    for (int i = 0; i < n; i++) {
        /* the forward input is natural: permute it; the inverse input is
         * already bit-reversed (it is a natural-order sequence permuted) */
        const int src = inverse ? i : (int)orc_bitrev((uint32_t)i, L);
        a[i] = (uint64_t)(((in[src] % q) + q) % q);
    }
    for (int m = 2; m <= n; m <<= 1) {
        const uint64_t wm = (uint64_t)orc_powmod((int64_t)w, (uint64_t)(n / m), q);
        for (int k = 0; k < n; k += m) {
            uint64_t wj = 1;
            for (int j = 0; j < m / 2; j++) {
                const uint64_t t = wj * a[k + j + m / 2] % uq, u = a[k + j];
                a[k + j] = (u + t) % uq;
                a[k + j + m / 2] = (u + uq - t) % uq;
                wj = wj * wm % uq;
            }
        }
    }
    /* natural order; the forward designs return bit-reversed order */
    for (int i = 0; i < n; i++) out[i] = (int64_t)(inverse ? a[i] : a[orc_bitrev((uint32_t)i, L)]);
    free(a);
}
