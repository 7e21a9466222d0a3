// tables.h -- host-side twiddle / Barrett tables of every design.
//
// The reference computes its tables at graph-construction time on the host
// (src/twiddle.h, src/auxiliary.h) and stores one expanded copy per pipeline
// tile.  Here the same values are computed once per plan and laid out for the
// CTA-resident kernels: one compact table per design, indexed by the
// butterfly's block (or position) instead of being repeated per layer.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace gbntt {

enum Kind {
    K_R2_I16_FWD = 0, K_R2_I16_INV = 1, K_R4_I16_FWD = 2, K_R8_I16_STAGE = 3,
    K_R2_I32_FWD = 4, K_R2_I32_INV = 5, K_BITREV_I16 = 6, K_FULL_BARRETT_I16 = 7,
    K_R8_I16_FWD = 8, K_R4_I16_INV = 9, K_NUM_KINDS = 10
};

constexpr uint32_t FLAG_CANONICAL = 0x1u;
constexpr uint32_t FLAG_R8_EXACT = 0x2u;
constexpr uint32_t FLAG_R8_FLOAT = 0x4u;
constexpr uint32_t FLAG_NATURAL_ORDER = 0x8u;
constexpr uint32_t FLAG_SCALE_NINV = 0x10u;
constexpr uint32_t FLAG_LANE_EXACT = 0x20u;

// Largest two-pass (four-step) length of the canonical int32 family.
constexpr int CANON_MAX_L32 = 22;

// The plan runs a canonical family (Shoup multiplication, lazy lanes, one
// final reduction): GBNTT_FLAG_CANONICAL without GBNTT_FLAG_LANE_EXACT on a
// transform design (not the radix-8 single stage, not the radix-8 chain with
// the reference's float multipliers), int32 moduli below 2^30.
bool canonical_fast(int kind, int64_t q, uint32_t flags);
// its family (F_C16F, F_C16I, F_C32F or F_C32I of device.cuh)
int canonical_family(int kind);

struct HostPlan {
    int kind = 0;
    uint32_t n = 0;
    int L = 0;                 // log2 n
    int64_t q = 0, root = 0, factor = 0;
    uint32_t flags = 0;
    int elem_bytes = 2;
    int stages = 0;            // pipeline stages (tiles) of the reference design
    // (tw, w') pairs, flattened: tab[2*i] = tw, tab[2*i+1] = w'
    std::vector<int32_t> tab;
    int32_t c = 0;             // Barrett constant of the reduction: int16(2^16/q+0.5) or int32(2^32/q+0.5)
    int32_t r4_fneg = 0;       // omega_4 as a signed residue (ntt_r4_kernels.cc:112)
    int32_t r4_wc = 0;         // its K=16 multiplier (ntt_r4_kernels.cc:113)
    int32_t f8[64] = {};       // radix-8 matrix F8[m][k] (signed, src/twiddle.h:326-344)
    int r8_sym = 0;            // F8 has the symmetries f[j+4] = -f[j] (fast butterfly allowed)
    int32_t f8s[4] = {};       // f1, f2, f3 (f0 = 1) when r8_sym
    int tail_bits = 0;         // radix-2^c tail stage of the chained radix-8 transform
    int32_t ftail[16] = {};    // tail matrix [m][k]
    int32_t tail_wq = 0;       // K=31 multiplier of the twiddle 1
    int32_t fb_fs = 0;         // full Barrett: signed factor (full_reduction_kernels.cc:186)
    int32_t fb_wq = 0;         // its multiplier (full_reduction_kernels.cc:187)
};

// Validates the parameters like the reference's static_asserts and builds the
// tables.  Returns a gbntt_status code (0 = OK) and a message in err.
int build_host_plan(int kind, uint32_t n, int64_t q, int64_t root, int64_t factor, uint32_t flags,
                    HostPlan& hp, std::string& err);

// Number theory helpers shared with the batch and serving code.
int64_t powmod(int64_t b, uint64_t e, int64_t q);
int64_t modinv(int64_t a, int64_t q);
int log_root_order(int64_t q, int64_t root);
uint32_t bitrev(uint32_t a, int bits);

}  // namespace gbntt
