// batch_c32.cu -- persistent-kernel instantiations for the canonical int32
// families (forward and inverse in one kernel); batch_k32.cu lists them in the
// configuration table.
#include "batch_kernel.cuh"

namespace gbntt {

const void* batch_kernels_c32(int el, int occ, bool zero_copy) {
    constexpr int C32 = (1 << F_C32F) | (1 << F_C32I);
    if (zero_copy) {
        if (occ != 0) return nullptr;
        if (el == 4) return reinterpret_cast<const void*>(&k_batch_zc<true, BATCH_CTA, 4, C32>);
        if (el == 5) return reinterpret_cast<const void*>(&k_batch_zc<true, BATCH_CTA, 5, C32>);
        return nullptr;
    }
#define GB_K(EL, OCC) \
    if (el == EL && occ == OCC) return reinterpret_cast<const void*>(&k_batch<true, BATCH_CTA, EL, C32, OCC>);
    GB_K(5, 0)
    GB_K(4, 0)
    GB_K(4, 4)
#undef GB_K
    return nullptr;
}

}  // namespace gbntt
