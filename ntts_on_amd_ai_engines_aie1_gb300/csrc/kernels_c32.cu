// Instantiations of the canonical int32 transform kernels (forward, inverse)
// up to 2^15 coefficients (one CTA per polynomial at most); the dispatch of
// every canonical family.
#include "device.cuh"

namespace gbntt {

KernelInfo kinfo_c16f(int L, bool lat);
KernelInfo kinfo_c16i(int L, bool lat);

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
        GB_CASE(F, 13) GB_CASE(F, 14) GB_CASE(F, 15)                                              \
        default: return KernelInfo();                                                             \
    }

namespace {
KernelInfo kinfo_c32f(int L, bool lat) { GB_ALL(F_C32F) }
KernelInfo kinfo_c32i(int L, bool lat) { GB_ALL(F_C32I) }
}  // namespace

KernelInfo kinfo_canon(int fam, int L, bool lat) {
    switch (fam) {
    case F_C16F: return kinfo_c16f(L, lat);
    case F_C16I: return kinfo_c16i(L, lat);
    case F_C32F: return kinfo_c32f(L, lat);
    case F_C32I: return kinfo_c32i(L, lat);
    default: return KernelInfo();
    }
}

}  // namespace gbntt
