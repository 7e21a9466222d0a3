// Instantiations of the canonical int16 transform kernels (forward, inverse).
#include "device.cuh"

namespace gbntt {

#define GB_CASE(F, L) case L: return make_kernel_info<F, L, false>();
#define GB_LAT(F, L) case L: if constexpr (has_lat(F, L)) return make_kernel_info<F, L, false, true>(); else return KernelInfo();
#define GB_ALL(F)                                                                                 \
    if (lat) {                                                                                    \
        switch (L) {                                                                              \
            GB_LAT(F, 9) GB_LAT(F, 10) GB_LAT(F, 11) GB_LAT(F, 12)                                \
            default: return KernelInfo();                                                         \
        }                                                                                         \
    }                                                                                             \
    switch (L) {                                                                                  \
        GB_CASE(F, 1) GB_CASE(F, 2) GB_CASE(F, 3) GB_CASE(F, 4) GB_CASE(F, 5) GB_CASE(F, 6)       \
        GB_CASE(F, 7) GB_CASE(F, 8) GB_CASE(F, 9) GB_CASE(F, 10) GB_CASE(F, 11) GB_CASE(F, 12)    \
        default: return KernelInfo();                                                             \
    }

KernelInfo kinfo_c16f(int L, bool lat) { GB_ALL(F_C16F) }
KernelInfo kinfo_c16i(int L, bool lat) { GB_ALL(F_C16I) }

}  // namespace gbntt
