/* Stand-in for the OptiX device API (oracle harness only).  optixTrace asks the
 * harness's visibility callback; the launch index is set by the harness loop
 * that stands in for optixLaunch; the atomics run single-threaded. */
#pragma once
#include <cstring>
#include "optix.h"

extern "C" int ref_vis_call(float ox, float oy, float oz, float dx, float dy, float dz, float tmin, float tmax);
extern "C" unsigned int ref_launch_x;

static inline void optixTrace(OptixTraversableHandle, float3 o, float3 d, float tmin, float tmax, float,
                              OptixVisibilityMask, unsigned int, unsigned int, unsigned int, unsigned int,
                              unsigned int &p0)
{
    p0 = (unsigned int)ref_vis_call(o.x, o.y, o.z, d.x, d.y, d.z, tmin, tmax);
}
static inline uint3 optixGetLaunchIndex() { uint3 u; u.x = ref_launch_x; u.y = 0; u.z = 0; return u; }
static inline void optixSetPayload_0(unsigned int) {}

static inline unsigned long long ref_atomic_cas(unsigned long long *a, unsigned long long cmp, unsigned long long v)
{
    unsigned long long old = *a;
    if (old == cmp) *a = v;
    return old;
}
static inline long long ref_d2ll(double d) { long long r; std::memcpy(&r, &d, 8); return r; }
static inline double ref_ll2d(long long l) { double r; std::memcpy(&r, &l, 8); return r; }
#define atomicCAS ref_atomic_cas
#define __double_as_longlong ref_d2ll
#define __longlong_as_double ref_ll2d
