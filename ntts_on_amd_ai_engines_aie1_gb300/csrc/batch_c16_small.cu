// batch_c16_small.cu -- persistent-kernel instantiations for the canonical
// int16 families with CTAs of fewer than 256 threads (smaller tiles, so a
// batch's last wave of tiles ends sooner), in their own translation unit so
// they compile in parallel; batch_k16.cu lists them in the configuration table.
#include "batch_kernel.cuh"

namespace gbntt {

const void* batch_kernels_c16_small(int el, int set, int occ, int cta) {
    constexpr int C16 = (1 << F_C16F) | (1 << F_C16I);
    if (set != C16) return nullptr;
#define GB_K(CTA, EL, OCC) \
    if (cta == CTA && el == EL && occ == OCC) return reinterpret_cast<const void*>(&k_batch<false, CTA, EL, C16, OCC>);
    // 16 coefficients per thread, 128 threads: a 1024-point polynomial spans two warps
    GB_K(128, 4, 12)
    GB_K(128, 4, 10)
    // 32 coefficients per thread, 64 threads: a 1024-point polynomial is one
    // warp (one exchange, warp-synchronous), two of them per tile
    GB_K(64, 5, 12)
#undef GB_K
    return nullptr;
}

}  // namespace gbntt
