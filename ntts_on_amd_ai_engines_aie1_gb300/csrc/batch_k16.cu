// batch_k16.cu -- persistent-kernel instantiations for the int16 designs:
// one per family (radix-2 forward + inverse, radix-4, radix-8) and a generic
// one, each with 32 and 64 coefficients per thread (the generic one: 32).
#include "batch_kernel.cuh"

namespace gbntt {

namespace {
constexpr int R2 = (1 << F_R2F16) | (1 << F_R2I16);
constexpr int R4 = 1 << F_R4F16;
constexpr int R8 = 1 << F_R8F16;
constexpr int ALL16 = R2 | R4 | R8;

#define GB_CFG(EL, SET, CTA) \
    {false, EL, SET, reinterpret_cast<const void*>(&k_batch<false, CTA, EL, SET>), nullptr, CTA}
// 256-thread CTAs.  (768-thread CTAs, one per SM so that every warp of an SM
// runs the same phase of the same tile, measured no faster on GB300.)
BatchConfig kI16[] = {
    GB_CFG(6, R4, 256), GB_CFG(5, R4, 256), GB_CFG(6, R2, 256), GB_CFG(5, R2, 256), GB_CFG(6, R8, 256),
    GB_CFG(5, R8, 256), GB_CFG(5, ALL16, 256),
};
#undef GB_CFG
}  // namespace

int batch_configs_i16(const BatchConfig** out) {
    // the 32-coefficient configurations also carry the zero-copy form (batch_k16_zc.cu)
    static const bool linked = [] {
        for (auto& c : kI16)
            if (c.elmax == 5 && c.cta == BATCH_CTA) c.zfn = batch_zc_kernel_i16(c.set);
        return true;
    }();
    (void)linked;
    *out = kI16;
    return (int)(sizeof(kI16) / sizeof(kI16[0]));
}

}  // namespace gbntt
