// batch_k16.cu -- the configuration table of the int16 persistent kernels.
// The kernels are instantiated in batch_k16_w64.cu, batch_k16_w32.cu,
// batch_k16_w32g.cu, batch_k16_w16.cu, batch_k16_w16g.cu, batch_c16.cu and
// batch_c16_small.cu (compiled in parallel); the zero-copy forms in
// batch_k16_zc.cu.
#include "batch_kernel.cuh"

namespace gbntt {

const void* batch_kernels_i16_w64(int el, int set, int occ);
const void* batch_kernels_i16_w32(int el, int set, int occ);
const void* batch_kernels_i16_w32g(int el, int set, int occ);
const void* batch_kernels_i16_w16(int el, int set, int occ);
const void* batch_kernels_i16_w16g(int el, int set, int occ);
const void* batch_kernels_c16(int el, int set, int occ);
const void* batch_kernels_c16_small(int el, int set, int occ, int cta);
const void* batch_zc_kernel_c16(int set, int el);

namespace {
constexpr int R2 = (1 << F_R2F16) | (1 << F_R2I16);
constexpr int R4 = 1 << F_R4F16;
constexpr int R8 = 1 << F_R8F16;
constexpr int ALL16 = R2 | R4 | R8;
constexpr int C16 = (1 << F_C16F) | (1 << F_C16I);   // canonical forward + inverse

struct Key {
    int el, set, occ;
    int cta = BATCH_CTA;
};
// 256-thread CTAs with 64, 32 or 16 coefficients per thread; the narrower
// ones carry less unrolled code per variant and fit more CTAs per SM (occ:
// the residency the registers are budgeted for, 0 = the default of the width).
// The order matters: GBNTT_BATCH_NO_TUNE takes the first covering entry.
// (768-thread CTAs, one per SM, measured no faster on GB300.)
constexpr Key kKeys[] = {
    {6, R4, 0}, {5, R4, 0}, {6, R2, 0}, {5, R2, 0}, {6, R8, 0}, {5, R8, 0}, {5, ALL16, 0},
    {4, R4, 0}, {4, R4, 5}, {4, R4, 6}, {4, R2, 0}, {4, R2, 5}, {4, R8, 0}, {4, R8, 5}, {4, ALL16, 0},
    // canonical families: 16 coefficients per thread at 4, 5 and 6 CTAs/SM, 32 at 3
    // and 4 (8 per thread at 8 CTAs/SM spilled at its 32-register budget)
    {4, C16, 6}, {4, C16, 5}, {4, C16, 0}, {5, C16, 0}, {5, C16, 4},
    // 128-thread CTAs (tiles of 2048 coefficients, n <= 2^11 at 16 per thread):
    // half the work per tile, so a batch's last wave of tiles ends sooner
    {4, C16, 12, 128}, {4, C16, 10, 128},
    // 32 coefficients per thread in 64-thread CTAs (n <= 2^11): one warp per
    // 1024-point polynomial (the fastest on batches of 4x the benchmark's)
    {5, C16, 12, 64},
};
constexpr int kN = (int)(sizeof(kKeys) / sizeof(kKeys[0]));
BatchConfig kI16[kN];
}  // namespace

int batch_configs_i16(const BatchConfig** out) {
    static const bool built = [] {
        for (int i = 0; i < kN; ++i) {
            const Key k = kKeys[i];
            const void* fn = nullptr;
            if (k.cta != BATCH_CTA) {
                fn = batch_kernels_c16_small(k.el, k.set, k.occ, k.cta);
            } else {
                for (auto get : {batch_kernels_i16_w64, batch_kernels_i16_w32, batch_kernels_i16_w32g,
                                 batch_kernels_i16_w16, batch_kernels_i16_w16g, batch_kernels_c16})
                    if (!fn) fn = get(k.el, k.set, k.occ);
            }
            const void* zfn = k.cta != BATCH_CTA ? nullptr
                              : k.set == C16 ? (k.occ == 0 ? batch_zc_kernel_c16(k.set, k.el) : nullptr)
                                             : batch_zc_kernel_i16(k.set, k.el);
            kI16[i] = BatchConfig{false, k.el, k.set, fn, zfn, k.cta, k.occ};
        }
        return true;
    }();
    (void)built;
    *out = kI16;
    return kN;
}

}  // namespace gbntt
