/*
 * ntt_oracle.h -- CPU restatement of the AIE1 NTT artifact's hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker and the
 * timed CPU baseline.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it.  The GPU product
 * (libgb300ntt.so) never links, loads or calls anything in oracle/.
 *
 * What it restates (file:line are paths inside the reference project):
 *   - table generation of src/twiddle.h and src/auxiliary.h, including the
 *     reference's rounding conventions (see ntt_oracle.c for each quirk);
 *   - the per-tile kernel loops of src/kernels/ sources in their constant-geometry
 *     (Pease) form, with AIE1 semantics: SRS rounding "symmetric_zero"
 *     (round half toward zero), saturation "none" (two's-complement wrap),
 *     and floor rounding inside the full Barrett kernel;
 *   - an O(n^2) modular DFT used to check the restatement.
 *
 * Parity pinning: the generated tables are checked against tables produced by
 * compiling the reference's own src/twiddle.h + src/auxiliary.h (recipe in
 * oracle/Makefile, golden hashes in tests/golden/).  The kernel loops cannot
 * be compiled (they need the AMD AIE toolchain); their restatement is pinned
 * by the modular DFT (canonical outputs) and by round-trip properties.
 */
#ifndef GB300_NTT_ORACLE_H
#define GB300_NTT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Design kinds.  0..7 follow NTT_CONFIG in src/project.cpp:35,139-157. */
enum {
    ORC_R2_I16_FWD = 0,      /* NTT<..., TYPE_NTT_NO_to_BO>           src/ntt.h:43  */
    ORC_R2_I16_INV = 1,      /* NTT<..., TYPE_INTT_BO_to_NO>          src/ntt.h:43  */
    ORC_R4_I16_FWD = 2,      /* NTT_R4<...>                           src/ntt_r4.h:30 */
    ORC_R8_I16_STAGE = 3,    /* NTT_R8<...> (one radix-8 stage)       src/ntt_r8.h:22 */
    ORC_R2_I32_FWD = 4,      /* NTT_INT32<..., FORWARD_CT_NO_TO_BO>   src/ntt_int32.h:27 */
    ORC_R2_I32_INV = 5,      /* NTT_INT32<..., INVERSE_GS_BO_TO_NO>   src/ntt_int32.h:27 */
    ORC_BITREV_I16 = 6,      /* BITREVERSE<N>                         src/standalone_units.h:17 */
    ORC_FULL_BARRETT_I16 = 7,/* FULL_BARRETT_MULTIPLICATION<N,q,F>    src/standalone_units.h:40 */
    ORC_R8_I16_FWD = 8,      /* chained radix-8 stages (src/ntt_r8.h:17-19 describes, does not ship) */
    ORC_R4_I16_INV = 9       /* bitrev + forward r4 with inverse twiddles (src/ntt_r4.h:18-20) */
};

/* ---- number theory (src/twiddle.h, src/auxiliary.h) ---- */
uint32_t orc_bitrev(uint32_t a, int bits);
int64_t  orc_powmod(int64_t base, uint64_t e, int64_t q);
int64_t  orc_red_neg(int64_t a, int64_t q);
int64_t  orc_modinv(int64_t a, int64_t q);
int      orc_log_root_order(int64_t q, int64_t root);      /* -1 if none <= 100 */
int64_t  orc_round_trunc_half(int64_t num, int64_t den);   /* trunc(num/den + 1/2), exact */

/* ---- individual Barrett multipliers as the reference computes them ---- */
int16_t orc_kyber_wq(int16_t tw, int32_t q);          /* twiddle.h:96      */
int32_t orc_r8_wq_float(int32_t tw, int32_t q);       /* twiddle.h:372     */
int32_t orc_r8_wq_exact(int32_t tw, int32_t q);       /* exact nearest      */
int16_t orc_fb_wq(int32_t factor_signed, int32_t q);  /* full_reduction_kernels.cc:187 */

/* ---- plans ---- */
typedef struct orc_plan orc_plan;

/* factor: FULL_BARRETT multiplier (ignored otherwise).  r8_exact: 0 = the
 * reference's float-derived K=31 multipliers, 1 = exact integer ones.
 * Returns NULL and sets *err (if non-NULL) on invalid parameters. */
orc_plan* orc_plan_create(int kind, int n, int64_t q, int64_t root, int64_t factor,
                          int r8_exact, int* err);
void      orc_plan_destroy(orc_plan* p);
int       orc_plan_layers(const orc_plan* p);   /* pipeline stages (tiles) */
int       orc_elem_bytes(const orc_plan* p);

/* Per-layer tables exactly as the reference graph constructors hold them.
 * which: 0 = combined/twiddle table of layer `layer`, 1 = Barrett multipliers
 * (separate-buffer families), 2 = radix-8 F8 matrix, 3 = radix-8 reduction
 * twiddles, 4 = radix-8 reduction multipliers.  Values are widened to int64.
 * Returns the number of entries written (dst may be NULL to query). */
int64_t orc_plan_table(const orc_plan* p, int which, int layer, int64_t* dst);

/* Run one stage (layer) of the pipeline on one polynomial. */
int orc_run_layer(const orc_plan* p, int layer, const void* in, void* out);

/* Run the whole pipeline on `batch` polynomials (contiguous). */
int orc_execute(const orc_plan* p, const void* in, void* out, int64_t batch);
int orc_execute_mt(const orc_plan* p, const void* in, void* out, int64_t batch, int nthreads);
/* the same; canonical != 0 also reduces every output to [0, q), in each thread */
int orc_execute_mt2(const orc_plan* p, const void* in, void* out, int64_t batch, int nthreads, int canonical);

/* O(n^2) modular DFT, canonical residues.  out[k] = sum_j in[j] w^(+-jk). */
void orc_dft(int n, int64_t q, int64_t root, int inverse, const int64_t* in, int64_t* out);

/* Exact transform in O(n log n), canonical residues, in the designs' orders:
 * forward = orc_dft(root) permuted to bit-reversed order; inverse = orc_dft
 * with root^-1 of the bit-reversed input read back in natural order. */
void orc_ntt_exact(int n, int64_t q, int64_t root, int inverse, const int64_t* in, int64_t* out);

#ifdef __cplusplus
}
#endif
#endif
