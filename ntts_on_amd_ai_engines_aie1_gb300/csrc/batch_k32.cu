// batch_k32.cu -- persistent-kernel configurations for the int32 designs:
// 32 coefficients per thread (n up to 2^13) here, 16 (n up to 2^12) in
// batch_k32_w16.cu, which compiles in parallel.
#include "batch_kernel.cuh"

namespace gbntt {

const void* batch_kernels_i32_w16(int occ, bool zero_copy);
const void* batch_kernels_c32(int el, int occ, bool zero_copy);

namespace {
constexpr int I32SET = (1 << F_R2F32) | (1 << F_R2G32);
constexpr int C32 = (1 << F_C32F) | (1 << F_C32I);   // canonical forward + inverse
BatchConfig kI32[6];
}  // namespace

int batch_configs_i32(const BatchConfig** out) {
    static const bool built = [] {
        kI32[0] = BatchConfig{true, 5, I32SET, reinterpret_cast<const void*>(&k_batch<true, BATCH_CTA, 5, I32SET>),
                              reinterpret_cast<const void*>(&k_batch_zc<true, BATCH_CTA, 5, I32SET>), BATCH_CTA, 0};
        kI32[1] = BatchConfig{true, 4, I32SET, batch_kernels_i32_w16(0, false), batch_kernels_i32_w16(0, true),
                              BATCH_CTA, 0};
        kI32[2] = BatchConfig{true, 4, I32SET, batch_kernels_i32_w16(4, false), nullptr, BATCH_CTA, 4};
        kI32[3] = BatchConfig{true, 5, C32, batch_kernels_c32(5, 0, false), batch_kernels_c32(5, 0, true),
                              BATCH_CTA, 0};
        kI32[4] = BatchConfig{true, 4, C32, batch_kernels_c32(4, 0, false), batch_kernels_c32(4, 0, true),
                              BATCH_CTA, 0};
        kI32[5] = BatchConfig{true, 4, C32, batch_kernels_c32(4, 4, false), nullptr, BATCH_CTA, 4};
        return true;
    }();
    (void)built;
    *out = kI32;
    return 6;
}

}  // namespace gbntt
