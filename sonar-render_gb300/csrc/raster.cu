// raster.cu -- headless rendering of the textured facets (RenderOpenGL).
//
// The reference draws every facet of the target and field objects with its
// pressure colour map as a texture (ModelGl.cpp:222-341, ObjectGl.cpp:64-110,
// the texture written by MakeSurface, FacetCuda.cu:43-72) through EGL/GL and
// saves the frame buffer as a PNG.  There is no graphics stack here, so the
// same picture is computed by two CUDA kernels:
//   * k_raster: one CTA per (triangle, 32 x 32-pixel tile) of the triangle's
//     screen box; every pixel centre inside the triangle (either winding, no
//     culling) whose window depth lies in [0, 1] competes through a 64-bit
//     atomicMin on (depth bits, triangle index): the nearest wins and equal
//     depths go to the first triangle drawn, as GL_LESS does;
//   * k_shade: the winner's perspective-correct texture coordinates, a
//     bilinear sample of its facet's colour cells with repeat addressing (the
//     GL defaults of the reference's texture: GL_LINEAR, GL_REPEAT), the
//     colour rounded to 8 bits; pixels without a triangle get the reference's
//     clear colour (0.96, 0.96, 0.86).  Rows are written top row first, as the
//     reference's flipped PNG.
// Camera: glm::perspective(45 deg, width / height, 0.1, 10000) and
// glm::lookAt(eye, centre, up) from the nine view settings (ModelGl.cpp:98-106),
// composed on the host into one 4 x 4 matrix (row-major, clip = M [x y z 1]).
// Triangles with a vertex behind the near plane are not drawn.
#include "sonar_internal.h"

namespace sonar {
namespace {

constexpr int kRasterTile = 32;

__device__ __forceinline__ float4 to_clip(const float *M, float4 v)
{
    return make_float4(M[0] * v.x + M[1] * v.y + M[2] * v.z + M[3], M[4] * v.x + M[5] * v.y + M[6] * v.z + M[7],
                       M[8] * v.x + M[9] * v.y + M[10] * v.z + M[11], M[12] * v.x + M[13] * v.y + M[14] * v.z + M[15]);
}

struct Screen {
    float x[3], y[3], z[3], iw[3];  // window x, y; NDC z; 1 / w
    float area;
    bool ok;
};

__device__ __forceinline__ Screen project(const RasterArgs &a, const RasterTri &T)
{
    Screen s;
    s.ok = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float4 c = to_clip(a.mvp, T.v[k]);
        if (!(c.w > 0.1f)) s.ok = false;
        const float iw = 1.0f / c.w;
        s.x[k] = (c.x * iw + 1.0f) * 0.5f * (float)a.width;
        s.y[k] = (c.y * iw + 1.0f) * 0.5f * (float)a.height;
        s.z[k] = c.z * iw;
        s.iw[k] = iw;
    }
    s.area = (s.x[1] - s.x[0]) * (s.y[2] - s.y[0]) - (s.x[2] - s.x[0]) * (s.y[1] - s.y[0]);
    return s;
}

// barycentric weights of the point (px, py); false when outside
__device__ __forceinline__ bool bary(const Screen &s, float px, float py, float &b0, float &b1, float &b2)
{
    const float e0 = (s.x[2] - s.x[1]) * (py - s.y[1]) - (s.y[2] - s.y[1]) * (px - s.x[1]);
    const float e1 = (s.x[0] - s.x[2]) * (py - s.y[2]) - (s.y[0] - s.y[2]) * (px - s.x[2]);
    const float e2 = (s.x[1] - s.x[0]) * (py - s.y[0]) - (s.y[1] - s.y[0]) * (px - s.x[0]);
    if (s.area > 0.0f) {
        if (e0 < 0.0f || e1 < 0.0f || e2 < 0.0f) return false;
    } else if (s.area < 0.0f) {
        if (e0 > 0.0f || e1 > 0.0f || e2 > 0.0f) return false;
    } else {
        return false;
    }
    const float inv = 1.0f / s.area;
    b0 = e0 * inv;
    b1 = e1 * inv;
    b2 = e2 * inv;
    return true;
}

__global__ void __launch_bounds__(256) k_raster(RasterArgs a)
{
    const int4 w = a.work[blockIdx.x];  // triangle, tile x, tile y
    const RasterTri T = a.tris[w.x];
    const Screen s = project(a, T);
    if (!s.ok) return;
    for (int e = threadIdx.x; e < kRasterTile * kRasterTile; e += blockDim.x) {
        const int px = w.y * kRasterTile + (e % kRasterTile), py = w.z * kRasterTile + (e / kRasterTile);
        if (px >= a.width || py >= a.height) continue;
        float b0, b1, b2;
        if (!bary(s, px + 0.5f, py + 0.5f, b0, b1, b2)) continue;
        const float z = b0 * s.z[0] + b1 * s.z[1] + b2 * s.z[2];
        if (!(z >= -1.0f && z <= 1.0f)) continue;
        const float depth = (z + 1.0f) * 0.5f;
        const unsigned long long key = ((unsigned long long)__float_as_uint(depth) << 32) | (unsigned)w.x;
        atomicMin(a.zbuf + (long long)py * a.width + px, key);
    }
}

__device__ __forceinline__ float4 texel(const RasterArgs &a, const RasterTex &t, int x, int y)
{
    x %= t.nx;
    if (x < 0) x += t.nx;
    y %= t.ny;
    if (y < 0) y += t.ny;
    return a.colours[t.cell0 + (long long)y * t.nx + x];
}

__device__ __forceinline__ unsigned char unorm8(float c)
{
    return (unsigned char)__float2int_rn(fminf(fmaxf(c, 0.0f), 1.0f) * 255.0f);
}

__global__ void __launch_bounds__(256) k_shade(RasterArgs a)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (long long)a.width * a.height) return;
    const int px = (int)(p % a.width), py = (int)(p / a.width);
    float4 c = make_float4(0.96f, 0.96f, 0.86f, 1.0f);
    const unsigned long long key = a.zbuf[p];
    if (key != ~0ull) {
        const int tri = (int)(key & 0xFFFFFFFFull);
        const RasterTri T = a.tris[tri];
        const Screen s = project(a, T);
        float b0, b1, b2;
        if (bary(s, px + 0.5f, py + 0.5f, b0, b1, b2)) {
            // perspective-correct texture coordinates
            const float q0 = b0 * s.iw[0], q1 = b1 * s.iw[1], q2 = b2 * s.iw[2];
            const float qs = 1.0f / (q0 + q1 + q2);
            const float u = (q0 * T.uv[0].x + q1 * T.uv[1].x + q2 * T.uv[2].x) * qs;
            const float v = (q0 * T.uv[0].y + q1 * T.uv[1].y + q2 * T.uv[2].y) * qs;
            const RasterTex t = a.tex[T.facet];
            const float fx = u * (float)t.nx - 0.5f, fy = v * (float)t.ny - 0.5f;
            const float x0 = floorf(fx), y0 = floorf(fy);
            const float ax = fx - x0, ay = fy - y0;
            const int ix = (int)x0, iy = (int)y0;
            const float4 c00 = texel(a, t, ix, iy), c10 = texel(a, t, ix + 1, iy);
            const float4 c01 = texel(a, t, ix, iy + 1), c11 = texel(a, t, ix + 1, iy + 1);
            c.x = (1.0f - ay) * ((1.0f - ax) * c00.x + ax * c10.x) + ay * ((1.0f - ax) * c01.x + ax * c11.x);
            c.y = (1.0f - ay) * ((1.0f - ax) * c00.y + ax * c10.y) + ay * ((1.0f - ax) * c01.y + ax * c11.y);
            c.z = (1.0f - ay) * ((1.0f - ax) * c00.z + ax * c10.z) + ay * ((1.0f - ax) * c01.z + ax * c11.z);
        }
    }
    unsigned char *o = a.rgb + 3 * ((long long)(a.height - 1 - py) * a.width + px);
    o[0] = unorm8(c.x);
    o[1] = unorm8(c.y);
    o[2] = unorm8(c.z);
}

}  // namespace

int raster_tile() { return kRasterTile; }

void launch_raster(const RasterArgs &a, int nwork, cudaStream_t s)
{
    const long long npix = (long long)a.width * a.height;
    cudaMemsetAsync(a.zbuf, 0xff, (size_t)npix * sizeof(unsigned long long), s);
    if (nwork > 0) k_raster<<<nwork, 256, 0, s>>>(a);
    k_shade<<<(unsigned)((npix + 255) / 256), 256, 0, s>>>(a);
}

}  // namespace sonar
