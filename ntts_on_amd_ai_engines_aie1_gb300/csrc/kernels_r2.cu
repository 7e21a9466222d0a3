// Instantiations of the radix-2 int16 transform kernels (forward and inverse).
#include "device.cuh"

namespace gbntt {

#define GB_CASE(F, L) case L: return make_kernel_info<F, L, false>();
// the latency form of design F at L, or none
#define GB_LAT(F, L) case L: if constexpr (has_lat(F, L)) return make_kernel_info<F, L, false, true>(); else return KernelInfo();

KernelInfo kinfo_r2f16(int L, bool lat) {
    if (lat) {
        switch (L) {
            GB_LAT(F_R2F16, 9) GB_LAT(F_R2F16, 10) GB_LAT(F_R2F16, 11) GB_LAT(F_R2F16, 12)
            default: return KernelInfo();
        }
    }
    switch (L) {
        GB_CASE(F_R2F16, 1) GB_CASE(F_R2F16, 2) GB_CASE(F_R2F16, 3) GB_CASE(F_R2F16, 4)
        GB_CASE(F_R2F16, 5) GB_CASE(F_R2F16, 6) GB_CASE(F_R2F16, 7) GB_CASE(F_R2F16, 8)
        GB_CASE(F_R2F16, 9) GB_CASE(F_R2F16, 10) GB_CASE(F_R2F16, 11) GB_CASE(F_R2F16, 12)
        default: return KernelInfo();
    }
}

KernelInfo kinfo_r2i16(int L, bool lat) {
    if (lat) {
        switch (L) {
            GB_LAT(F_R2I16, 9) GB_LAT(F_R2I16, 10) GB_LAT(F_R2I16, 11) GB_LAT(F_R2I16, 12)
            default: return KernelInfo();
        }
    }
    switch (L) {
        GB_CASE(F_R2I16, 1) GB_CASE(F_R2I16, 2) GB_CASE(F_R2I16, 3) GB_CASE(F_R2I16, 4)
        GB_CASE(F_R2I16, 5) GB_CASE(F_R2I16, 6) GB_CASE(F_R2I16, 7) GB_CASE(F_R2I16, 8)
        GB_CASE(F_R2I16, 9) GB_CASE(F_R2I16, 10) GB_CASE(F_R2I16, 11) GB_CASE(F_R2I16, 12)
        default: return KernelInfo();
    }
}

}  // namespace gbntt
