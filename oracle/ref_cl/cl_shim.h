// cl_shim.h -- just enough of OpenCL C for g++ to compile the reference's SPH kernel sources
// (resources/kernels/sph_common.cl and sph_grid.cl) as C++ and run them on the CPU, one
// work-item at a time. Test infrastructure for the oracle: not part of the product.
//
// Vector types evaluate component-wise in IEEE single precision (compile without FP
// contraction). Built-ins map to the C library's float functions.
//
// Known limit: OpenCL vector literals "(float3)(a, b, c)" parse in C++ as a cast of a comma
// expression and yield (float3)(c). They occur only in update_grid_positions and
// walls_collision, which the harness therefore never calls: it computes the grid positions
// itself, and the walls (whose GPU kernel also adds a constant (1, 1, 0) that the reference's
// CPU simulator does not have) are compared separately.
#ifndef CL_SHIM_H
#define CL_SHIM_H

#define __kernel
#define __global
#define __local
#define __private
#define __constant const
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2

// The types and built-ins live in namespace clt, which the harness's kernel namespaces use:
// the OpenCL built-ins (sqrt, pow, floor, dot) then never meet the C++ library's overloads,
// and argument-dependent lookup on the vector types finds no kernel function.
namespace clt {

typedef unsigned int uint;

struct float3 {
    float x, y, z, w_;
    float3() : x(0), y(0), z(0), w_(0) {}
    float3(float v) : x(v), y(v), z(v), w_(0) {}
    float3(float a, float b, float c) : x(a), y(b), z(c), w_(0) {}
    float3 &operator+=(const float3 &o) { x += o.x; y += o.y; z += o.z; return *this; }
    float3 &operator-=(const float3 &o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    float3 &operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
};
inline float3 operator+(const float3 &a, const float3 &b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(const float3 &a, const float3 &b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(const float3 &a, const float3 &b) { return float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator*(const float3 &a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator*(float s, const float3 &a) { return float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator/(const float3 &a, float s) { return float3(a.x / s, a.y / s, a.z / s); }
inline float3 operator/(const float3 &a, const float3 &b) { return float3(a.x / b.x, a.y / b.y, a.z / b.z); }

struct int3;
struct int3_xyz {
    int x, y, z, w_;
    int3_xyz &operator=(const int3 &o);
};
struct int3 {
    union {
        struct {
            int x, y, z, w_;
        };
        int3_xyz xyz;
    };
    int3() : x(0), y(0), z(0), w_(0) {}
    int3(int v) : x(v), y(v), z(v), w_(0) {}
};
inline int3_xyz &int3_xyz::operator=(const int3 &o)
{
    x = o.x;
    y = o.y;
    z = o.z;
    return *this;
}

// OpenCL dot(): a.x*b.x + a.y*b.y + a.z*b.z, left to right
inline float dot(const float3 &a, const float3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline float pow(float x, float y) { return __builtin_powf(x, y); }
inline float floor(float x) { return __builtin_floorf(x); }

// the work-item being run (the harness sets it before each call)
extern thread_local unsigned long cl_shim_gid;
inline unsigned long get_global_id(uint) { return cl_shim_gid; }
inline unsigned long get_global_size(uint) { return 0; }
inline unsigned long get_local_id(uint) { return 0; }
inline unsigned long get_local_size(uint) { return 1; }
inline unsigned long get_group_id(uint) { return 0; }
inline unsigned long get_num_groups(uint) { return 1; }
inline void barrier(int) {}
inline int atomic_inc(volatile int *p)
{
    const int old = *p;
    *p = old + 1;
    return old;
}

}  // namespace clt

#endif  // CL_SHIM_H
