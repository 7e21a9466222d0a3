// Host-side check of the compile-time shared-memory layouts of device.cuh:
// for every exchange (and bit-reversal permutation) of the persistent kernel's
// variants with at least 32 threads per polynomial, the chosen layout must be
// free of bank conflicts on both sides, and the padded layouts must fit the
// per-polynomial buffer.  Prints one line per failure and exits non-zero.
#include <cstdio>

#include "../../ntts_on_amd_ai_engines_aie1_gb300/csrc/device.cuh"

using namespace gbntt;

int main() {
    int bad = 0, checked = 0;
    const int fams[] = {F_R2F16, F_R2I16, F_R4F16, F_R8F16, F_R2F32, F_R2G32};
    for (int fam : fams)
        for (int EL = 4; EL <= 6; ++EL)
            for (int L = EL + 5; L <= 13; ++L) {   // at least 32 threads per polynomial
                if (fam == F_R4F16 && (L & 1)) continue;
                const int NS = nsteps(fam, L);
                int prev = L - EL;   // the staging layout's window
                for (int st = 0; st <= NS; ++st) {
                    const int lo = st < NS ? window_lo(fam, L, EL, st) : prev;
                    if (lo != prev) {
                        const int olo = lo > prev ? lo : prev;
                        const int ohi = (lo < prev ? lo : prev) + EL;
                        const int w = ohi > olo ? ohi - olo : 0;
                        const int vb = w >= 2 ? 2 : w;
                        ++checked;
                        if (vb == 0) {
                            const XPad x = scalar_layout(L, EL, prev, lo);
                            if (pad_degree(L, EL, prev, false, lo, x.s, x.t) != 2 ||
                                xpad((1 << L) - 1, x.s, x.t) >= xwords(L)) {
                                std::printf("scalar fam %d L %d EL %d %d->%d\n", fam, L, EL, prev, lo);
                                ++bad;
                            }
                        } else {
                            const int f = vector_layout(L, EL, prev, lo, vb);
                            if (vector_wavefronts(L, EL, prev, lo, vb, f) != 2 * (1 << EL)) {
                                std::printf("vector fam %d L %d EL %d %d->%d\n", fam, L, EL, prev, lo);
                                ++bad;
                            }
                        }
                    }
                    prev = lo;
                }
                // the bit-reversal permutations of the first and last windows
                for (int lo : {window_lo(fam, L, EL, 0), window_lo(fam, L, EL, NS - 1)}) {
                    const XPad x = brev_layout(L, EL, lo);
                    ++checked;
                    if (xpad((1 << L) - 1, x.s, x.t) >= xwords(L) || pad_degree(L, EL, lo, true, lo, x.s, x.t) > 3) {
                        std::printf("bitrev fam %d L %d EL %d lo %d\n", fam, L, EL, lo);
                        ++bad;
                    }
                }
            }
    std::printf("%d layouts checked, %d failures\n", checked, bad);
    return bad ? 1 : 0;
}
