// batch_k32.cu -- persistent-kernel instantiation for the int32 designs.
#include "batch_kernel.cuh"

namespace gbntt {

namespace {
constexpr int I32SET = (1 << F_R2F32) | (1 << F_R2G32);
const BatchConfig kI32[] = {
    {true, 5, I32SET, reinterpret_cast<const void*>(&k_batch<true, BATCH_CTA, 5, I32SET>),
     reinterpret_cast<const void*>(&k_batch_zc<true, BATCH_CTA, 5, I32SET>), BATCH_CTA, 0},
};
}  // namespace

int batch_configs_i32(const BatchConfig** out) {
    *out = kI32;
    return (int)(sizeof(kI32) / sizeof(kI32[0]));
}

}  // namespace gbntt
