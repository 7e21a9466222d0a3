/*
 * Minimal stand-in for AMD's <adf.h>, written for this project.  It declares
 * only what the reference's host-side table code (src/twiddle.h,
 * src/auxiliary.h, src/kernels/kernels.h) needs to compile with g++, so that
 * the reference's own table generators can be run on the CPU as a parity
 * source.  No AIE functionality is provided.
 */
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <utility>
#include <vector>

typedef int16_t int16;
typedef uint16_t uint16;
typedef int32_t int32;
typedef uint32_t uint32;
typedef int64_t int64;
typedef uint64_t uint64;

namespace adf {
template <typename T> struct input_buffer { T* data() { return nullptr; } };
template <typename T> struct output_buffer { T* data() { return nullptr; } };
struct kernel {
    template <class C, class... A> static kernel create_object(A&&...) { return kernel(); }
};
}  // namespace adf

#define REGISTER_FUNCTION(...)
#define REGISTER_PARAMETER(...)
