// batch_k16_zc.cu -- zero-copy persistent-kernel instantiations for the int16
// designs (32 coefficients per thread for every family set, 16 for radix-4),
// in their own translation unit so they compile in parallel.
#include "batch_kernel.cuh"

namespace gbntt {

const void* batch_zc_kernel_i16(int set, int elmax) {
    constexpr int R2 = (1 << F_R2F16) | (1 << F_R2I16);
    constexpr int R4 = 1 << F_R4F16;
    constexpr int R8 = 1 << F_R8F16;
    if (elmax == 5) {
        switch (set) {
        case R2: return reinterpret_cast<const void*>(&k_batch_zc<false, BATCH_CTA, 5, R2>);
        case R4: return reinterpret_cast<const void*>(&k_batch_zc<false, BATCH_CTA, 5, R4>);
        case R8: return reinterpret_cast<const void*>(&k_batch_zc<false, BATCH_CTA, 5, R8>);
        case R2 | R4 | R8: return reinterpret_cast<const void*>(&k_batch_zc<false, BATCH_CTA, 5, R2 | R4 | R8>);
        default: return nullptr;
        }
    }
    if (elmax == 4) {
        switch (set) {
        case R4: return reinterpret_cast<const void*>(&k_batch_zc<false, BATCH_CTA, 4, R4>);
        default: return nullptr;
        }
    }
    return nullptr;
}

}  // namespace gbntt
