// plan_internal.h -- accessors shared by abi.cu and batch.cu (not part of the ABI).
#pragma once

#include <string>

#include "device.cuh"

struct gbntt_plan;

int gbntt_internal_fail(int code, const std::string& msg);
void gbntt_internal_count_launch();
int gbntt_internal_plan_L(const gbntt_plan* p);
// family (-1 when the design has no persistent-kernel variant), log2 n, element bytes, launch constants
void gbntt_internal_plan_args(const gbntt_plan* p, int* fam, int* L, int* elem_bytes, gbntt::KArgs* a);
// Device address of a page-locked host buffer that is mapped into the device's
// address space (cudaHostAlloc / cudaHostRegister memory under unified
// addressing), or nullptr for any other pointer.  A buffer with such an address
// can be read and written by the transform kernels directly over the
// host-device link (zero copy).
const void* gbntt_internal_mapped(const void* h);
// Zero-copy execution of one plan on mapped host buffers through the zero-copy
// persistent kernel (batch.cu).  `state` is the plan's scratch (descriptor and
// tile counters, created on first use; freed with gbntt_internal_zc_free).
// Returns GBNTT_ERR_KIND when no zero-copy kernel carries the design (the
// caller then copies through device staging memory).
int gbntt_internal_zc_plan(void** state, const gbntt_plan* p, const void* m_in, void* m_out, uint64_t count,
                           cudaStream_t s);
void gbntt_internal_zc_free(void* state);
