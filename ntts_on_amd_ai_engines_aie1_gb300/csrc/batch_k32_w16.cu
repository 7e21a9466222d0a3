// batch_k32_w16.cu -- int32 persistent kernels at 16 coefficients per thread
// (transforms up to 2^12 coefficients), in their own translation unit.
#include "batch_kernel.cuh"

namespace gbntt {

const void* batch_kernels_i32_w16(int occ, bool zero_copy) {
    constexpr int I32SET = (1 << F_R2F32) | (1 << F_R2G32);
    if (zero_copy) return occ == 0 ? reinterpret_cast<const void*>(&k_batch_zc<true, BATCH_CTA, 4, I32SET>) : nullptr;
    if (occ == 0) return reinterpret_cast<const void*>(&k_batch<true, BATCH_CTA, 4, I32SET>);
    if (occ == 4) return reinterpret_cast<const void*>(&k_batch<true, BATCH_CTA, 4, I32SET, 4>);
    return nullptr;
}

}  // namespace gbntt
