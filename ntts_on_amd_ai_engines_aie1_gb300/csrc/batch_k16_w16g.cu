// batch_k16_w16g.cu -- persistent-kernel instantiations for the int16 designs (16 coefficients per thread, radix-8 and every int16 family),
// one translation unit per group so the groups compile in parallel;
// batch_k16.cu assembles the configuration table.
#include "batch_kernel.cuh"

namespace gbntt {

const void* batch_kernels_i16_w16g(int el, int set, int occ) {
    constexpr int R2 = (1 << F_R2F16) | (1 << F_R2I16);
    constexpr int R4 = 1 << F_R4F16;
    constexpr int R8 = 1 << F_R8F16;
    constexpr int ALL16 = R2 | R4 | R8;
    (void)R2; (void)R4; (void)R8; (void)ALL16;
#define GB_K(EL, SET, OCC) \
    if (el == EL && set == SET && occ == OCC) return reinterpret_cast<const void*>(&k_batch<false, BATCH_CTA, EL, SET, OCC>);
    GB_K(4, R8, 0)
    GB_K(4, R8, 5)
    GB_K(4, ALL16, 0)
#undef GB_K
    return nullptr;
}

}  // namespace gbntt
