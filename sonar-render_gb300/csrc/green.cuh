// green.cuh -- the FP32 pair arithmetic shared by the kernels that evaluate
// single FACET_SELF entries: the reference's rounded dot product and cosine
// gate (src/OptiX.cu:267-330) and the entry T(j, i) of the low-rank blocks
// (the Green's function of the symmetric bounce sum, src/OptiX.cu:340-390).
#pragma once

#include "sonar_internal.h"

namespace sonar {
namespace {

constexpr float kInv4Pi = 0.0795774715459476679f;  // 1 / (4 pi)
constexpr float kTwoPi = 6.28318530717958647692f;

__device__ __forceinline__ float dot_rn(float ax, float ay, float az, float bx, float by, float bz)
{
    // a.x*b.x + a.y*b.y + a.z*b.z evaluated left to right, every product and
    // sum rounded separately (the reference's vec_math dot without contraction)
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// Cosine gates.  The reference's decision is "cos < 1e-6 -> skip" with
// cos = dot(v * (1/r), n) in FP32 without contraction (exact_cos below).  A
// cheaper estimate dot(v, n) * rsqrt(v.v) differs from it by less than 7e-7
// (both are within a few ulp of the true cosine, |cos| <= 1), so outside the
// band [0, 2e-6] the estimate decides the same way; inside it the exact
// expression is evaluated.
__device__ __forceinline__ float exact_cos(float vx, float vy, float vz, float sign, float nx, float ny, float nz)
{
    const float r = __fsqrt_rn(dot_rn(vx, vy, vz, vx, vy, vz));
    const float inv = __frcp_rn(r);
    const float ux = __fmul_rn(vx, inv), uy = __fmul_rn(vy, inv), uz = __fmul_rn(vz, inv);
    return dot_rn(sign * ux, sign * uy, sign * uz, nx, ny, nz);
}

// The exact FP32 cosine gate where the estimate is inside the band (rare):
// kept out of line so that kernels that unroll several entries carry one
// copy of it.
__device__ __noinline__ bool gate_exact(float vx, float vy, float vz, float sign, float nx, float ny, float nz)
{
    return !(exact_cos(vx, vy, vz, sign, nx, ny, nz) < 1e-6f);
}

__device__ __forceinline__ bool gate_est(float est, float vx, float vy, float vz, float sign, float nx, float ny,
                                         float nz)
{
    if (est > 2e-6f) return true;
    if (est < 0.0f) return false;
    return gate_exact(vx, vy, vz, sign, nx, ny, nz);
}

// T(j, i) of one pair of a block of class cls (bit: the pair's mask bit for
// BITS; CLEAR blocks evaluate the cosine gates inline).  One code path for
// every class: the Green's function of sym_pair (same operations, same
// rounding), then the pair's gate.
template <bool ATT>
__device__ __forceinline__ float2 lr_entry(const SumArgs &a, int cls, bool bit, float4 pi, float4 ni, float4 pj,
                                           float4 nj)
{
    const float vx = __fsub_rn(pj.x, pi.x), vy = __fsub_rn(pj.y, pi.y), vz = __fsub_rn(pj.z, pi.z);
    const float r2 = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
    const float rinv = rsqrtf(r2);
    const float r0 = r2 * rinv;
    const float r = fmaf(fmaf(-r0, r0, r2), 0.5f * rinv, r0);
    const float th = __fmul_rn(r, a.k2hi);
    const float tl = fmaf(r, a.k2lo, fmaf(r, a.k2hi, -th));
    const float frac = (th - rintf(th)) + tl;
    float sn, cs;
    __sincosf(frac * kTwoPi, &sn, &cs);
    const float d1 = vx * ni.x + vy * ni.y + vz * ni.z;  // r cos_scat
    const float d2 = vx * nj.x + vy * nj.y + vz * nj.z;  // -r cos_inc
    const float rinv2 = rinv * rinv;
    const float u = (d1 * d2) * (-rinv2);
    float Tr, Ti;
    if (ATT) {
        const float amp = rinv * kInv4Pi * __expf(-a.ka * r);
        Tr = u * fmaf(amp, fmaf(a.ka, cs, a.kr * sn), rinv2);
        Ti = u * (amp * fmaf(a.ka, sn, -a.kr * cs));
    } else {
        const float ua = (u * rinv) * a.kr4pi;
        Tr = fmaf(ua, sn, u * rinv2);
        Ti = -ua * cs;
    }
    float rr = r;
    if (fabsf(r - a.rmin) <= a.rmin * 1e-6f) rr = __fsqrt_rn(dot_rn(vx, vy, vz, vx, vy, vz));
    if (rr < a.rmin) {
        Tr = u * (-a.ka * kInv4Pi);
        Ti = u * (a.kr * kInv4Pi);
    }
    bool ok = cls == kFlagBits ? bit : true;
    if (cls == kFlagClear)
        ok = gate_est(d1 * rinv, vx, vy, vz, 1.0f, ni.x, ni.y, ni.z) &&
             gate_est(-d2 * rinv, vx, vy, vz, -1.0f, nj.x, nj.y, nj.z);
    return ok ? make_float2(Tr, Ti) : make_float2(0.0f, 0.0f);
}

}  // namespace
}  // namespace sonar
