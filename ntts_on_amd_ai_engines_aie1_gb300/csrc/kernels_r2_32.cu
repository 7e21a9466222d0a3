// Instantiations of the radix-2 int32 transform kernels (forward CT, inverse GS).
#include "device.cuh"

namespace gbntt {

#define GB_CASE(F, L) case L: return make_kernel_info<F, L, false>();
// the latency form of design F at L, or none
#define GB_LAT(F, L) case L: if constexpr (has_lat(F, L)) return make_kernel_info<F, L, false, true>(); else return KernelInfo();

KernelInfo kinfo_r2f32(int L, bool lat) {
    if (lat) {
        switch (L) {
            GB_LAT(F_R2F32, 9) GB_LAT(F_R2F32, 10) GB_LAT(F_R2F32, 11) GB_LAT(F_R2F32, 12)
            default: return KernelInfo();
        }
    }
    switch (L) {
        GB_CASE(F_R2F32, 1) GB_CASE(F_R2F32, 2) GB_CASE(F_R2F32, 3) GB_CASE(F_R2F32, 4)
        GB_CASE(F_R2F32, 5) GB_CASE(F_R2F32, 6) GB_CASE(F_R2F32, 7) GB_CASE(F_R2F32, 8)
        GB_CASE(F_R2F32, 9) GB_CASE(F_R2F32, 10) GB_CASE(F_R2F32, 11) GB_CASE(F_R2F32, 12)
        GB_CASE(F_R2F32, 13) GB_CASE(F_R2F32, 14) GB_CASE(F_R2F32, 15)
        default: return KernelInfo();
    }
}

KernelInfo kinfo_r2g32(int L, bool lat) {
    if (lat) {
        switch (L) {
            GB_LAT(F_R2G32, 9) GB_LAT(F_R2G32, 10) GB_LAT(F_R2G32, 11) GB_LAT(F_R2G32, 12)
            default: return KernelInfo();
        }
    }
    switch (L) {
        GB_CASE(F_R2G32, 1) GB_CASE(F_R2G32, 2) GB_CASE(F_R2G32, 3) GB_CASE(F_R2G32, 4)
        GB_CASE(F_R2G32, 5) GB_CASE(F_R2G32, 6) GB_CASE(F_R2G32, 7) GB_CASE(F_R2G32, 8)
        GB_CASE(F_R2G32, 9) GB_CASE(F_R2G32, 10) GB_CASE(F_R2G32, 11) GB_CASE(F_R2G32, 12)
        GB_CASE(F_R2G32, 13) GB_CASE(F_R2G32, 14) GB_CASE(F_R2G32, 15)
        default: return KernelInfo();
    }
}

}  // namespace gbntt
