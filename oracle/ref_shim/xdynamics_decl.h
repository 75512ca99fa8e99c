/* Stand-in for the reference's include/xdynamics_decl.h when its DEM kernels
 * are compiled for the host (oracle/Makefile, target _ref).  It supplies only
 * what include/xdynamics_parallel/xParallelDEM_decl.cuh and _impl.cuh use:
 * the export macro, the small POD types of include/xTypes.h and the CUDA
 * execution-space keywords and built-ins as host equivalents. */
#ifndef XDEM_REF_SHIM_DECL_H
#define XDEM_REF_SHIM_DECL_H

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <iostream>

#include <vector_types.h>
#include <vector_functions.h>

#define XDYNAMICS_API
#define __declspec(x)
#define VERSION_NUMBER 2
#ifndef __constant__
#define __constant__
#endif
#ifndef __shared__
#define __shared__
#endif
#ifndef __global__
#define __global__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __host__
#define __host__
#endif

using namespace std;

typedef struct { unsigned int sid, scid, count, neach; } xClusterInformation;
typedef struct { unsigned int id, sid, ntsda; } xSpringDamperConnectionInformation;
typedef struct { unsigned int jd, kc_id; double init_l; } xSpringDamperConnectionData;
typedef struct { double k, c; } xSpringDamperCoefficient;
typedef struct {
    double a00, a01, a02, a03, a10, a11, a12, a13;
    double a20, a21, a22, a23, a30, a31, a32, a33;
} matrix44d;

/* Launch coordinates of the emulated thread (one OS thread runs one id at a
 * time). */
extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

inline void __syncthreads() {}
inline unsigned int __umul24(unsigned int a, unsigned int b)
{
    return (unsigned int)((unsigned long long)(a & 0xffffffu) * (unsigned long long)(b & 0xffffffu));
}
inline int __mul24(int a, int b)
{
    long long x = (long long)((a << 8) >> 8), y = (long long)((b << 8) >> 8);
    return (int)(x * y);
}

/* The reference's vector operators take non-const references (MSVC binds
 * temporaries to them); these overloads give g++ the same meaning for
 * temporaries.  Lvalue calls still pick the reference's own operators. */
inline double3 operator-(const double3& a, const double3& b) { return make_double3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline double4 operator-(const double4& a, const double4& b) { return make_double4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline double4 operator+(const double4& a, const double4& b) { return make_double4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline double3 operator+(const double3& a, const double3& b) { return make_double3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline double3 operator-(const double3& a) { return make_double3(-a.x, -a.y, -a.z); }
inline double3 operator*(double s, const double3& a) { return make_double3(s * a.x, s * a.y, s * a.z); }
inline double4 operator*(double s, const double4& a) { return make_double4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline double3 operator/(const double3& a, double s) { return make_double3(a.x / s, a.y / s, a.z / s); }
inline double4 operator/(const double4& a, double s) { return make_double4(a.x / s, a.y / s, a.z / s, a.w / s); }

#endif
