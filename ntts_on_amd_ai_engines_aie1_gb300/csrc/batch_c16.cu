// batch_c16.cu -- persistent-kernel instantiations for the canonical int16
// families (forward and inverse in one kernel), in their own translation unit
// so they compile in parallel; batch_k16.cu lists them in the configuration
// table.
#include "batch_kernel.cuh"

namespace gbntt {

const void* batch_kernels_c16(int el, int set, int occ) {
    constexpr int C16 = (1 << F_C16F) | (1 << F_C16I);
    if (set != C16) return nullptr;
#define GB_K(EL, OCC) \
    if (el == EL && occ == OCC) return reinterpret_cast<const void*>(&k_batch<false, BATCH_CTA, EL, C16, OCC>);
    GB_K(5, 0)
    GB_K(5, 4)
    GB_K(4, 0)
    GB_K(4, 6)
    GB_K(4, 5)
#undef GB_K
    return nullptr;
}

const void* batch_zc_kernel_c16(int set, int el) {
    constexpr int C16 = (1 << F_C16F) | (1 << F_C16I);
    if (set == C16 && el == 4) return reinterpret_cast<const void*>(&k_batch_zc<false, BATCH_CTA, 4, C16>);
    return nullptr;
}

}  // namespace gbntt
