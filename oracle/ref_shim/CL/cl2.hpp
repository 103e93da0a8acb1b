/*
 * Minimal stand-in for the Khronos C++ bindings header, providing only the
 * scalar and vector typedefs that the reference's host-side type header
 * (include/nbody/device/types.h, host branch) needs so that
 * src/naive_simulation.cpp compiles from its own sources.
 * TEST INFRASTRUCTURE ONLY.
 */
#ifndef NBODY_CL2_TYPEDEF_SHIM
#define NBODY_CL2_TYPEDEF_SHIM
#include <cstdint>
typedef uint32_t cl_uint;
typedef int32_t cl_int;
typedef float cl_float;
typedef uint8_t cl_uchar;
typedef uint64_t cl_ulong;
typedef struct { alignas(16) cl_float s[4]; } cl_float4;
#endif
