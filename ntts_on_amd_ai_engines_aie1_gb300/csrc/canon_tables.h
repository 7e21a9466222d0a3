// canon_tables.h -- device-built twiddle tables of the canonical families
// (canon_tables.cu).
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace gbntt {

// (w, floor(w 2^32 / q)) pairs, n entries: root^(+-j 2^(L-1-B)) at 2^B + j
size_t canon_table_entries(int L, bool inverse);
cudaError_t make_canon_table(int2* d_tab, int L, uint32_t q, uint32_t root, bool inverse, cudaStream_t s);

// the four-step twist of a two-pass transform of 2^(L1+L2) coefficients
size_t canon_twist_entries(int L1, int L2, int EL);
cudaError_t make_canon_twist(int2* d_tab, int L1, int L2, int EL, uint32_t q, uint32_t root, bool inverse,
                             cudaStream_t s);

}  // namespace gbntt
