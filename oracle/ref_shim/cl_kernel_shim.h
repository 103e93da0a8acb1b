/*
 * cl_kernel_shim.h -- lets the reference's OpenCL C kernel files
 * (src/moment.cl, src/interaction.cl, src/field.cl, src/force.cl) compile
 * unmodified as C++ and run on the CPU, one work-item at a time.
 *
 * TEST INFRASTRUCTURE ONLY (oracle pinning).  Provides the OpenCL built-ins
 * those files use: address-space qualifiers, uint/uchar, a float4 with the
 * arithmetic the kernels need, dot/sqrt/min, work-item queries and the two
 * atomics.  None of the kernels uses local memory or barriers, so running
 * work-items sequentially is a valid schedule.
 *
 * One known difference from an OpenCL compiler: a vector literal
 * "(vector_t)(a, b, c, d)" is a C++ comma expression here and yields a
 * splat of its last element.  In the reference it appears only in the
 * quadrupole terms of src/moment.cl:45-54 (never read by the field or force
 * kernels) and as the zero vector of src/force.cl:246,277 (0 either way).
 */
#ifndef NBODY_CL_KERNEL_SHIM_H
#define NBODY_CL_KERNEL_SHIM_H

#include <cmath>
#include <cstddef>
#include <cstdint>

#define __OPENCL_VERSION__ 120
#define kernel
#define global

typedef unsigned int uint;
typedef unsigned char uchar;

struct alignas(16) float4 {
    float x, y, z, w;
    float4() : x(0), y(0), z(0), w(0) {}
    float4(float s) : x(s), y(s), z(s), w(s) {}
    float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    float4& operator+=(const float4& o) { x += o.x; y += o.y; z += o.z; w += o.w; return *this; }
};
static inline float4 operator+(float4 a, float4 b) { return float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline float4 operator-(float4 a, float4 b) { return float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static inline float4 operator*(float4 a, float4 b) { return float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
static inline float4 operator/(float4 a, float4 b) { return float4(a.x / b.x, a.y / b.y, a.z / b.z, a.w / b.w); }
static inline float4 operator*(float s, float4 a) { return float4(s * a.x, s * a.y, s * a.z, s * a.w); }
static inline float4 operator*(float4 a, float s) { return float4(a.x * s, a.y * s, a.z * s, a.w * s); }
static inline float4 operator/(float4 a, float s) { return float4(a.x / s, a.y / s, a.z / s, a.w / s); }
static inline float4 operator-(float4 a) { return float4(-a.x, -a.y, -a.z, -a.w); }
static inline float dot(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }

static inline float nbody_shim_sqrt(float v) { return std::sqrt(v); }
#define sqrt(v) nbody_shim_sqrt(v)

template <typename T> static inline T min(T a, T b) { return b < a ? b : a; }

/* work-item state, set by the launcher before each work-item runs */
struct nbody_shim_item {
    size_t gid[3], lid[3], grp[3], lsz[3];
};
extern nbody_shim_item nbody_shim_cur;
static inline size_t get_global_id(int d) { return nbody_shim_cur.gid[d]; }
static inline size_t get_local_id(int d) { return nbody_shim_cur.lid[d]; }
static inline size_t get_group_id(int d) { return nbody_shim_cur.grp[d]; }
static inline size_t get_local_size(int d) { return nbody_shim_cur.lsz[d]; }

static inline uint atomic_inc(uint* p) { return (*p)++; }
static inline uint atomic_max(uint* p, uint v) { uint o = *p; if (v > o) *p = v; return o; }

#endif
