// Instantiations of the radix-4 (forward, and bit-reversed in/out for the
// inverse) and chained radix-8 transform kernels.
#include "device.cuh"

namespace gbntt {

#define GB_R4(L) case L: return br ? make_kernel_info<F_R4F16, L, true>() : make_kernel_info<F_R4F16, L, false>();
#define GB_R8(L) case L: return make_kernel_info<F_R8F16, L, false>();
// the latency forms, or none
#define GB_R4L(L) case L: if constexpr (has_lat(F_R4F16, L)) return br ? make_kernel_info<F_R4F16, L, true, true>() : make_kernel_info<F_R4F16, L, false, true>(); else return KernelInfo();
#define GB_R8L(L) case L: if constexpr (has_lat(F_R8F16, L)) return make_kernel_info<F_R8F16, L, false, true>(); else return KernelInfo();

KernelInfo kinfo_r4(int L, bool br, bool lat) {
    if (lat) {
        switch (L) {
            GB_R4L(10) GB_R4L(12)
            default: return KernelInfo();
        }
    }
    switch (L) {
        GB_R4(2) GB_R4(4) GB_R4(6) GB_R4(8) GB_R4(10) GB_R4(12)
        default: return KernelInfo();
    }
}

KernelInfo kinfo_r8(int L, bool lat) {
    if (lat) {
        switch (L) {
            GB_R8L(9) GB_R8L(10) GB_R8L(11) GB_R8L(12)
            default: return KernelInfo();
        }
    }
    switch (L) {
        GB_R8(3) GB_R8(4) GB_R8(5) GB_R8(6) GB_R8(7) GB_R8(8) GB_R8(9) GB_R8(10) GB_R8(11) GB_R8(12)
        default: return KernelInfo();
    }
}

}  // namespace gbntt
