// surface.cu -- headless surface colouring of pressure grids.
//
// The reference colours every facet's pressure grid into a GL texture
// (MakeSurface, src/FacetCuda.cu:43-72, with hsv2rgb at :10-41) and draws it
// through EGL/OpenGL.  There is no graphics stack here, so the same colour
// map is written into a device buffer (one float4 RGBA per cell, in the
// pressure layout: facet-major, row-major y*numXpnts + x -- the texel the
// reference writes with surf2Dwrite(value, surface, x * 16, y)).
//
// Arithmetic follows the reference expression by expression, including its
// float/double promotions: |p| of the FP32 complex pressure, 20 log10(|p| +
// 1e-8), the clamp to [min_dB, max_dB], grey level 0.8 * mag, or with the
// phase flag an HSV colour with hue (atan2(p) + pi) / (2 pi), saturation 0.8
// and value mag.
#include <cuda_runtime.h>

#include "sonar_internal.h"

namespace sonar {
namespace {

__device__ __forceinline__ float4 hsv_to_rgb(float h, float s, float v)
{
    const float c = v * s;
    const float x = c * (1.0 - fabs(fmod(h * 6.0, 2.0) - 1.0));
    const float m = v - c;
    const float alpha = 1;
    if (h < 1.0 / 6.0) return make_float4(c + m, x + m, 0.0 + m, alpha);
    if (h < 2.0 / 6.0) return make_float4(x + m, c + m, 0.0 + m, alpha);
    if (h < 3.0 / 6.0) return make_float4(0.0 + m, c + m, x + m, alpha);
    if (h < 4.0 / 6.0) return make_float4(0.0 + m, x + m, c + m, alpha);
    if (h < 5.0 / 6.0) return make_float4(x + m, 0.0 + m, c + m, alpha);
    return make_float4(c + m, 0.0 + m, x + m, alpha);
}

__global__ void k_colour_map(const double2 *P, long long n, float min_db, float max_db, int phase, float4 *out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 q = P[i];
    const float pr = (float)q.x, pi = (float)q.y;
    const float saturation = 0.8f;
    const float dB = 20.0f * log10f(hypotf(pr, pi) + 1e-8f);
    float mag = (dB - min_db) / (max_db - min_db);
    mag = fminf(fmaxf(mag, 0.0f), 1.0f);
    float4 value = make_float4(saturation * mag, saturation * mag, saturation * mag, 1.0f);
    if (phase) {
        const float h = (atan2f(pi, pr) + 3.14159265358979323846) / (2.0f * 3.14159265358979323846);
        value = hsv_to_rgb(h, 0.8f, mag);
    }
    out[i] = value;
}

}  // namespace

void launch_colour_map(const double2 *P, long long n, float min_db, float max_db, int phase, float4 *out,
                       cudaStream_t s)
{
    if (n > 0) k_colour_map<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, n, min_db, max_db, phase, out);
}

}  // namespace sonar
