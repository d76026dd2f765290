// kernels.cu -- sm_103a kernels of the discrete Kirchhoff path.
//
// Two kernel families replace the reference's single OptiX ray-generation
// program (src/OptiX.cu:408-445, one thread per facet with serial loops and
// FP64 CAS atomics):
//
//  k_mask<HOP>  one CTA per (256 destinations, 256 sources) block.  Every pair
//               runs the reference's discrete gates with its FP32 arithmetic in
//               source order (IEEE sqrt and reciprocal, no fused multiply-add),
//               so the cosine decisions are bit-identical to the reference's
//               expressions; pairs that pass are tested for occlusion by a BVH
//               segment walk over the target triangles (replacing optixTrace).
//               Output: one bit per pair plus one flag per block.
//
//  k_sum<HOP>   destination-owned sums.  A CTA owns 256 destinations and a
//               range of 256-source tiles; each tile's positions, normals and
//               complex weights are staged in shared memory with 16-byte
//               loads and read as warp broadcasts; each thread evaluates the
//               Green's function for its destination in FP32 with a
//               split-precision phase and accumulates the tile in FP32, then
//               in FP64.  No atomics: partial sums per source split are
//               reduced in a fixed order (deterministic results).
//
// Hop formulas (the reference's, "as coded"):
//   SRC     P_j += cos_inc P_i e^{ikr} / r                      (OptiX.cu:100-106)
//   FP      P_j += A_i cos_scat P_i G(r)                        (OptiX.cu:182-186)
//   F2F     P_out_j += A_i cos_scat cos_inc P_in_i 0.9 G_reg(r) (OptiX.cu:340-390)
//   NORESP  P_j += A_i cos_scat P_i 0.9 G_reg(r)                (OptiX.cu:340-362)
//   G(r) = -e^{ikr}/(4 pi) (ik/r) + 1/r^2,  G_reg = ik/(4 pi) when r < delta_src.
#include "sonar_internal.h"
#include "green.cuh"

#include <algorithm>
#include <cstdio>

namespace sonar {
namespace {


// ---------------------------------------------------------------- visibility
// Does the part [tlo, 1] of segment o + t (e - o) touch the box?  (inv =
// componentwise 1 / (e - o))
__device__ __forceinline__ bool seg_box(float3 o, float3 inv, float4 a, float4 b, float tlo = 0.0f, float thi = 1.0f)
{
    const float tx0 = (a.x - o.x) * inv.x, tx1 = (b.x - o.x) * inv.x;
    const float ty0 = (a.y - o.y) * inv.y, ty1 = (b.y - o.y) * inv.y;
    const float tz0 = (a.z - o.z) * inv.z, tz1 = (b.z - o.z) * inv.z;
    const float t0 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tlo));
    const float t1 = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), thi));
    return t0 <= t1;
}

// Segment o -> e against one triangle (n, c; edge planes m_k, c_k):
// occludes when the segment strictly crosses the plane at distance
// t = r |d0| / (|d0| + |d1|) <= tmax and the crossing point is inside every
// edge plane; a plane within eps of the origin never occludes.
__device__ __forceinline__ bool tri_blocks(const float4 *__restrict__ T, float3 o, float3 e, float3 d, float r,
                                           float tmax, float eps)
{
    const float4 P = __ldg(T);
    const float d0 = fmaf(P.x, o.x, fmaf(P.y, o.y, P.z * o.z)) - P.w;
    if (fabsf(d0) <= eps) return false;
    const float d1 = fmaf(P.x, e.x, fmaf(P.y, e.y, P.z * e.z)) - P.w;
    if (!((d0 > 0.0f && d1 < 0.0f) || (d0 < 0.0f && d1 > 0.0f))) return false;
    const float ad0 = fabsf(d0), den = ad0 + fabsf(d1);
    if (r * ad0 > tmax * den) return false;
    const float s = ad0 / den;
    const float Xx = fmaf(d.x, s, o.x), Xy = fmaf(d.y, s, o.y), Xz = fmaf(d.z, s, o.z);
#pragma unroll
    for (int k = 1; k <= 3; ++k) {
        const float4 M = __ldg(T + k);
        if (fmaf(M.x, Xx, fmaf(M.y, Xy, M.z * Xz)) < M.w) return false;
    }
    return true;
}

// The same test on triangle records already in registers (shared-memory
// candidate lists).
__device__ __forceinline__ bool tri_blocks_v(float4 P, float4 M1, float4 M2, float4 M3, float3 o, float3 e, float3 d,
                                             float r, float tmax, float eps)
{
    const float d0 = fmaf(P.x, o.x, fmaf(P.y, o.y, P.z * o.z)) - P.w;
    if (fabsf(d0) <= eps) return false;
    const float d1 = fmaf(P.x, e.x, fmaf(P.y, e.y, P.z * e.z)) - P.w;
    if (!((d0 > 0.0f && d1 < 0.0f) || (d0 < 0.0f && d1 > 0.0f))) return false;
    const float ad0 = fabsf(d0), den = ad0 + fabsf(d1);
    if (r * ad0 > tmax * den) return false;
    const float s = ad0 / den;
    const float Xx = fmaf(d.x, s, o.x), Xy = fmaf(d.y, s, o.y), Xz = fmaf(d.z, s, o.z);
    if (fmaf(M1.x, Xx, fmaf(M1.y, Xy, M1.z * Xz)) < M1.w) return false;
    if (fmaf(M2.x, Xx, fmaf(M2.y, Xy, M2.z * Xz)) < M2.w) return false;
    if (fmaf(M3.x, Xx, fmaf(M3.y, Xy, M3.z * Xz)) < M3.w) return false;
    return true;
}

constexpr int kStack = 64;

// tlo, thi: only BVH boxes that the part [tlo, thi] of the segment touches
// are opened (callers narrow it only where no triangle can hold a crossing
// point outside it; the triangle tests themselves are unchanged).
__device__ bool occluded(const BvhView &B, float3 o, float3 e, float r, float tmax, float tlo = 0.0f,
                         float thi = 1.0f)
{
    if (B.ntri == 0) return false;
    const float sc = 1.0f + fmaxf(fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fmaxf(fabsf(o.z), fabsf(e.x))),
                                  fmaxf(fabsf(e.y), fabsf(e.z)));
    const float eps = 1e-4f * sc;
    const float3 d = make_float3(e.x - o.x, e.y - o.y, e.z - o.z);
    const float3 inv = make_float3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    int stack[kStack];
    int sp = 0;
    int node = 0;
    // The tree has nnodes nodes and is walked depth first: every node is
    // visited at most once, so the loop ends after at most nnodes iterations.
    for (int guard = 0; guard < B.nnodes; ++guard) {
        const float4 a = __ldg(B.nodes + 2 * node), b = __ldg(B.nodes + 2 * node + 1);
        bool descend = false;
        if (seg_box(o, inv, a, b, tlo, thi)) {
            const int left = __float_as_int(a.w), right = __float_as_int(b.w);
            if (left < 0) {
                const int t0 = -left - 1;
                for (int t = t0; t < t0 + right; ++t)
                    if (tri_blocks(B.tris + 4 * t, o, e, d, r, tmax, eps)) return true;
            } else {
                if (sp < kStack) stack[sp++] = right;  // the builder keeps depth < kStack
                node = left;
                descend = true;
            }
        }
        if (!descend) {
            if (sp == 0) return false;
            node = stack[--sp];
        }
    }
    return false;
}

// ---------------------------------------------------------------- gates

// true when cos(sign * v, n) passes the reference's ">= 1e-6" gate
__device__ __forceinline__ bool cos_gate(float vx, float vy, float vz, float rinv, float sign, float nx, float ny,
                                         float nz)
{
    const float est = sign * fmaf(vx, nx, fmaf(vy, ny, vz * nz)) * rinv;
    if (est > 2e-6f) return true;
    if (est < 0.0f) return false;
    return !(exact_cos(vx, vy, vz, sign, nx, ny, nz) < 1e-6f);
}

// Branch-free form of cos_gate for the mask kernel's pair loop: the estimate
// decides outside the band; lanes inside it (rare) are settled by the exact
// expression under a warp vote, so the common path carries no divergent
// branch.
__device__ __forceinline__ bool cos_gate_vote(float vx, float vy, float vz, float rinv, float sign, float nx,
                                              float ny, float nz, bool active)
{
    const float est = sign * fmaf(vx, nx, fmaf(vy, ny, vz * nz)) * rinv;
    bool pass = est > 2e-6f;
    const bool unsure = active && !pass && !(est < 0.0f);
    if (__any_sync(0xffffffffu, unsure)) {
        if (unsure) pass = !(exact_cos(vx, vy, vz, sign, nx, ny, nz) < 1e-6f);
    }
    return pass;
}

template <int HOP>
__device__ __forceinline__ bool pair_gates_vote(const MaskArgs &a, float4 s, float4 ns, float4 t, float4 nt, int ft,
                                                bool active)
{
    const float vx = __fsub_rn(t.x, s.x), vy = __fsub_rn(t.y, s.y), vz = __fsub_rn(t.z, s.z);
    const float rinv = rsqrtf(fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
    if (HOP == HOP_SRC) {
        if (a.dst_is_field) return true;
        return cos_gate_vote(vx, vy, vz, rinv, -1.0f, nt.x, nt.y, nt.z, active);
    }
    if (HOP == HOP_FP || HOP == HOP_NORESP) return cos_gate_vote(vx, vy, vz, rinv, 1.0f, ns.x, ns.y, ns.z, active);
    // FACET_RESP: two objects, no same-facet rule
    const bool other = HOP == HOP_RESP || __float_as_int(ns.w) != ft;
    const bool g1 = cos_gate_vote(vx, vy, vz, rinv, 1.0f, ns.x, ns.y, ns.z, active && other);
    const bool g2 = cos_gate_vote(vx, vy, vz, rinv, -1.0f, nt.x, nt.y, nt.z, active && other);
    return other && g1 && g2;
}

// Gates of one pair (the reference's discrete decisions).  For FACET_SELF
// the two cosines are the same pair of numbers whichever fragment is the
// enumeration's "A" side (u and -u give exactly negated dot products), so
// they are evaluated with v = p_dst - p_src and no orientation select.
template <int HOP>
__device__ __forceinline__ bool pair_gates(const MaskArgs &a, float4 s, float4 ns, float4 t, float4 nt, int ft)
{
    const float vx = __fsub_rn(t.x, s.x), vy = __fsub_rn(t.y, s.y), vz = __fsub_rn(t.z, s.z);
    if (HOP == HOP_SRC && a.dst_is_field) return true;  // cos_inc = 1 (OptiX.cu:67-72)
    if (HOP == HOP_F2F && __float_as_int(ns.w) == ft) return false;  // same facet (OptiX.cu:247-262)
    const float rinv = rsqrtf(fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
    if (HOP == HOP_SRC) return cos_gate(vx, vy, vz, rinv, -1.0f, nt.x, nt.y, nt.z);   // cos_inc = dot(-uv, n_B)
    if (HOP == HOP_FP) return cos_gate(vx, vy, vz, rinv, 1.0f, ns.x, ns.y, ns.z);     // cos_scat = dot(-uv_ji, n_A)
    if (HOP == HOP_NORESP) return cos_gate(vx, vy, vz, rinv, 1.0f, ns.x, ns.y, ns.z); // cos_scat = dot(uv, n_A)
    // FACET_SELF and FACET_RESP: cos_scat at the source's facet, cos_inc at the destination's
    return cos_gate(vx, vy, vz, rinv, 1.0f, ns.x, ns.y, ns.z) && cos_gate(vx, vy, vz, rinv, -1.0f, nt.x, nt.y, nt.z);
}

// The shadow ray of a pair: origin and end point (OptiX.cu:81-93, 163-175, 321-333).
// FACET_RESP: from the point of the enumeration's source object (the lower
// object index), i.e. from the destination when dst_origin.
template <int HOP>
__device__ __forceinline__ void pair_ray(float4 s, float4 ns, float4 t, int ft, float3 &o, float3 &e,
                                         bool dst_origin = false)
{
    bool src_first = true;  // source point, target fragment (NO_RESP), lower facet (SELF)
    if (HOP == HOP_FP) src_first = false;  // from the field point
    if (HOP == HOP_F2F) src_first = __float_as_int(ns.w) < ft;
    if (HOP == HOP_RESP) src_first = !dst_origin;
    o = src_first ? make_float3(s.x, s.y, s.z) : make_float3(t.x, t.y, t.z);
    e = src_first ? make_float3(t.x, t.y, t.z) : make_float3(s.x, s.y, s.z);
}

// Occlusion by the block's candidate triangles held in shared memory.  A
// triangle whose plane the segment does not cross strictly (the first test
// of tri_blocks_v, which needs neither the length nor the exclusion radius)
// is passed over before those are computed; the verdict is tri_blocks_v's.
__device__ __forceinline__ bool occluded_list(const float4 *sT, int n, float3 o, float3 e)
{
    bool ready = false;
    float r = 0.0f, tmax = 0.0f, eps = 0.0f;
    const float3 d = make_float3(e.x - o.x, e.y - o.y, e.z - o.z);
    for (int k = 0; k < n; ++k) {
        const float4 P = sT[4 * k];
        const float d0 = fmaf(P.x, o.x, fmaf(P.y, o.y, P.z * o.z)) - P.w;
        const float d1 = fmaf(P.x, e.x, fmaf(P.y, e.y, P.z * e.z)) - P.w;
        if (!((d0 > 0.0f && d1 < 0.0f) || (d0 < 0.0f && d1 > 0.0f))) continue;
        if (!ready) {
            const float vx = __fsub_rn(e.x, o.x), vy = __fsub_rn(e.y, o.y), vz = __fsub_rn(e.z, o.z);
            r = __fsqrt_rn(dot_rn(vx, vy, vz, vx, vy, vz));
            tmax = __fsub_rn(r, 1e-3f);
            const float sc = 1.0f + fmaxf(fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fmaxf(fabsf(o.z), fabsf(e.x))),
                                          fmaxf(fabsf(e.y), fabsf(e.z)));
            eps = 1e-4f * sc;
            ready = true;
        }
        if (tri_blocks_v(P, sT[4 * k + 1], sT[4 * k + 2], sT[4 * k + 3], o, e, d, r, tmax, eps)) return true;
    }
    return false;
}

__device__ __forceinline__ bool occluded_full(const BvhView &B, float3 o, float3 e, float reach = 3.0e38f,
                                              float near = 3.0e38f)
{
    const float vx = __fsub_rn(e.x, o.x), vy = __fsub_rn(e.y, o.y), vz = __fsub_rn(e.z, o.z);
    const float r = __fsqrt_rn(dot_rn(vx, vy, vz, vx, vy, vz));
    // reach: only the last `reach` metres of the ray can hold a crossing
    // point; near: only the first `near` metres can
    const float tlo = reach < r ? 1.0f - reach / r : 0.0f;
    const float thi = near < r ? near / r : 1.0f;
    return occluded(B, o, e, r, __fsub_rn(r, 1e-3f), tlo, thi);
}

// ---- block-level occluder culling
constexpr int kMaxCand = 32;  // candidate triangles tested per block in shared memory

// order-preserving float <-> int map for shared-memory atomic min / max
__device__ __forceinline__ int f2o(float f)
{
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__device__ __forceinline__ float warp_min(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ float plane_dist(const float4 P, float x, float y, float z)
{
    // the same expression as tri_blocks, so verdicts derived from it agree
    return fmaf(P.x, x, fmaf(P.y, y, P.z * z)) - P.w;
}

// Can a triangle with signed-distance ranges [o_lo, o_hi] over the ray
// origins and [e_lo, e_hi] over the endpoints occlude any ray of the block?
// rmax bounds every ray's length.  false only when provably not:
//  (a) all origins and endpoints on one closed side: no strict crossing;
//  (b) every origin within 1e-4 of the plane: the origin-plane exclusion
//      (eps = 1e-4 * scale >= 1e-4) removes it from every ray;
//  (c) every origin that can cross is at distance >= o0 from the plane --
//      o0 = 1e-4 by the exclusion of (b), or the nearest origin's distance
//      when all origins lie on one side -- and the endpoints lie within e1
//      of it: a crossing lies within rmax*e1/o0 of the endpoint, beyond
//      tmax = r - 1e-3 when o0 * 0.8e-3 > 1.1 * rmax * e1 (the margins cover
//      the rounding of tmax for rays shorter than 1,000 m and of the FP32
//      comparison in tri_blocks).  Endpoints on the plane itself (e1 = 0:
//      rays ending on the triangle's own facet) never cross.
__device__ __forceinline__ bool may_occlude(float o_lo, float o_hi, float e_lo, float e_hi, float rmax)
{
    if (fminf(o_lo, e_lo) >= 0.0f || fmaxf(o_hi, e_hi) <= 0.0f) return false;
    if (fmaxf(fabsf(o_lo), fabsf(o_hi)) <= 1e-4f) return false;
    if (rmax < 1000.0f) {
        const bool one_side = o_lo > 0.0f || o_hi < 0.0f;
        const float o0 = fmaxf(one_side ? fminf(fabsf(o_lo), fabsf(o_hi)) : 0.0f, 1e-4f);
        const float e1 = fmaxf(fabsf(e_lo), fabsf(e_hi));
        if (o0 * 0.8e-3f > rmax * e1 * 1.1f + 1e-30f) return false;
    }
    return true;
}

// Shadow test of one pair when every target triangle lies on or behind every
// target triangle's plane (a convex target, within tau = 1e-6 (1 + vmax)).
// A crossing that tri_blocks reports lies inside a triangle, so behind the
// fragment's facet plane up to E = 2e-6 (1 + vmax + sc) (tau plus the FP32
// errors of the fragment's position, of the crossing point and of the edge
// tests, each a few ulp of sc = 1 + the largest coordinate of the ray, with
// a factor two to spare); a ray point at distance rho from the fragment is
// rho cos in front of that plane (cos > 0: the pair passed its gate there).
//  * Rays that leave a target fragment (FACET_NO_RESP): a crossing has
//    rho <= E / cos, and its triangle's plane is at least 1e-4 sc from the
//    origin (tri_blocks' exclusion), so rho >= 1e-4 sc: no room, no test;
//    else only the first 1.1 E / cos metres of the ray are searched.
//  * Rays that end on a target fragment (source hop onto a target, readout
//    from a field point): tri_blocks ignores crossings within 1e-3 of the end
//    (tmax = r - 1e-3), so no test when 0.9e-3 cos > E; else only the last
//    1.1 E / cos metres.
// Every triangle that can report a hit is still tested, so the verdict is the
// full walk's.
template <int HOP>
__device__ __forceinline__ bool occluded_pair(const MaskArgs &a, float4 ns, float4 nt, float3 o, float3 e)
{
    if (a.convex && (HOP == HOP_NORESP || HOP == HOP_FP || (HOP == HOP_SRC && !a.dst_is_field))) {
        const float vx = __fsub_rn(e.x, o.x), vy = __fsub_rn(e.y, o.y), vz = __fsub_rn(e.z, o.z);
        const float rinv = rsqrtf(fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
        const float sc = 1.0f + fmaxf(fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fmaxf(fabsf(o.z), fabsf(e.x))),
                                      fmaxf(fabsf(e.y), fabsf(e.z)));
        const float E = 2e-6f * (1.0f + a.convex_vmax + sc);
        if (HOP == HOP_NORESP) {
            const float cosv = fmaf(vx, ns.x, fmaf(vy, ns.y, vz * ns.z)) * rinv;  // leaving the source fragment
            if (cosv > 0.0f) {
                if (E < 0.99e-4f * sc * cosv) return false;
                return occluded_full(a.bvh, o, e, 3.0e38f, 1.1f * E / cosv);
            }
        } else {
            // arriving at the fragment: the readout's source, the source hop's destination
            const float4 n = HOP == HOP_FP ? ns : nt;
            const float cosv = -fmaf(vx, n.x, fmaf(vy, n.y, vz * n.z)) * rinv;
            if (cosv > 0.0f) {
                if (cosv * 0.9e-3f > E) return false;
                return occluded_full(a.bvh, o, e, 1.1f * E / cosv);
            }
        }
    }
    return occluded_full(a.bvh, o, e);
}

// false when occluded_pair is sure to answer "not occluded" without a walk
template <int HOP>
__device__ __forceinline__ bool convex_needs_test(const MaskArgs &a, float4 ns, float4 nt, float3 o, float3 e)
{
    const float vx = __fsub_rn(e.x, o.x), vy = __fsub_rn(e.y, o.y), vz = __fsub_rn(e.z, o.z);
    const float rinv = rsqrtf(fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
    const float sc = 1.0f + fmaxf(fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fmaxf(fabsf(o.z), fabsf(e.x))),
                                  fmaxf(fabsf(e.y), fabsf(e.z)));
    const float E = 2e-6f * (1.0f + a.convex_vmax + sc);
    if (HOP == HOP_NORESP) {
        const float cosv = fmaf(vx, ns.x, fmaf(vy, ns.y, vz * ns.z)) * rinv;
        return !(cosv > 0.0f && E < 0.99e-4f * sc * cosv);
    }
    const float4 n = HOP == HOP_FP ? ns : nt;
    const float cosv = -fmaf(vx, n.x, fmaf(vy, n.y, vz * n.z)) * rinv;
    return !(cosv > 0.0f && cosv * 0.9e-3f > E);
}

// One block of k_mask: (destination block blockIdx.x, source tile
// blockIdx.y), or with a block list its entry qb.  Every early return is
// taken by the whole CTA.
template <int HOP>
__device__ __forceinline__ void mask_block(const MaskArgs &a, const int qb)
{
    __shared__ float4 sP[kTile];
    __shared__ float4 sN[kTile];
    __shared__ float4 sTri[4 * kMaxCand];
    __shared__ int sCand[kMaxCand];
    __shared__ int sRed[kMaxCand][4];  // ordered-int min/max of distances: src lo, src hi, dst lo, dst hi
    __shared__ int sBox[18];           // ordered-int boxes (lo xyz, hi xyz): union, sources, destinations
    __shared__ int sAllOcc;
    __shared__ int sFac[4];            // src facet lo/hi, dst facet lo/hi
    __shared__ int sNc, sKeep, sOverflow;
    const int tid = threadIdx.x;
    int tile = blockIdx.y, jb = blockIdx.x;
    if (HOP == HOP_F2F && a.blist) {
        const int2 e = a.blist[qb];
        tile = e.x;
        jb = e.y;
    }
    const int i0 = tile * kTile;
    const int j = jb * kTile + tid;
    const bool src_ok = i0 + tid < a.nsrc;
    const bool live = j < a.ndst;
    const long long fidx = (long long)tile * a.mask.ndstblocks + jb;
    if (HOP == HOP_F2F && a.upper_only && tile > jb) {
        // the symmetric bounce sum reads each unordered block once, from its upper side
        if (tid == 0) a.mask.flags[fidx] = kFlagNone;
        return;
    }
    if (tid < 18) sBox[tid] = (tid % 6) < 3 ? f2o(3.0e38f) : f2o(-3.0e38f);
    if (tid < 4) sFac[tid] = (tid & 1) ? -2147483647 : 2147483647;
    if (tid == 0) {
        sNc = 0;
        sKeep = 0;
        sOverflow = 0;
        sAllOcc = 0;
    }
    float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 n = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
    if (src_ok) {
        p = a.src_pos[i0 + tid];
        if (a.src_facet) {
            const int f = a.src_facet[i0 + tid];
            const float4 fn = a.src_facet_n[f];
            n = make_float4(fn.x, fn.y, fn.z, __int_as_float(f));
        }
    }
    sP[tid] = p;
    sN[tid] = n;
    float4 t = make_float4(0.0f, 0.0f, 0.0f, 0.0f), nt = t;
    int ft = -2;
    if (live) {
        t = a.dst_pos[j];
        if (a.dst_facet) {
            ft = a.dst_facet[j];
            nt = a.dst_facet_n[ft];
        }
    }
    // boxes of the block's sources and destinations and the facet ranges of both sides
    {
        float slo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, shi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        float dlo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, dhi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        if (src_ok) {
            slo[0] = shi[0] = p.x; slo[1] = shi[1] = p.y; slo[2] = shi[2] = p.z;
        }
        if (live) {
            dlo[0] = dhi[0] = t.x; dlo[1] = dhi[1] = t.y; dlo[2] = dhi[2] = t.z;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            for (int off = 16; off > 0; off >>= 1) {
                slo[k] = fminf(slo[k], __shfl_xor_sync(0xffffffffu, slo[k], off));
                shi[k] = fmaxf(shi[k], __shfl_xor_sync(0xffffffffu, shi[k], off));
                dlo[k] = fminf(dlo[k], __shfl_xor_sync(0xffffffffu, dlo[k], off));
                dhi[k] = fmaxf(dhi[k], __shfl_xor_sync(0xffffffffu, dhi[k], off));
            }
        }
        float lo[3], hi[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(slo[k], dlo[k]);
            hi[k] = fmaxf(shi[k], dhi[k]);
        }
        int fs_lo = src_ok ? __float_as_int(n.w) : 2147483647, fs_hi = src_ok ? __float_as_int(n.w) : -2147483647;
        int fd_lo = live ? ft : 2147483647, fd_hi = live ? ft : -2147483647;
        for (int off = 16; off > 0; off >>= 1) {
            fs_lo = min(fs_lo, __shfl_xor_sync(0xffffffffu, fs_lo, off));
            fs_hi = max(fs_hi, __shfl_xor_sync(0xffffffffu, fs_hi, off));
            fd_lo = min(fd_lo, __shfl_xor_sync(0xffffffffu, fd_lo, off));
            fd_hi = max(fd_hi, __shfl_xor_sync(0xffffffffu, fd_hi, off));
        }
        __syncthreads();  // shared-memory initialisation above is complete
        if ((tid & 31) == 0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                atomicMin(&sBox[k], f2o(lo[k]));
                atomicMax(&sBox[3 + k], f2o(hi[k]));
                atomicMin(&sBox[6 + k], f2o(slo[k]));
                atomicMax(&sBox[9 + k], f2o(shi[k]));
                atomicMin(&sBox[12 + k], f2o(dlo[k]));
                atomicMax(&sBox[15 + k], f2o(dhi[k]));
            }
            atomicMin(&sFac[0], fs_lo);
            atomicMax(&sFac[1], fs_hi);
            atomicMin(&sFac[2], fd_lo);
            atomicMax(&sFac[3], fd_hi);
        }
    }
    __syncthreads();

    // ---- FACET_SELF blocks whose fragments all share one facet interact nowhere
    if (HOP == HOP_F2F && sFac[0] == sFac[1] && sFac[2] == sFac[3] && sFac[0] == sFac[2]) {
        if (tid == 0) a.mask.flags[fidx] = kFlagNone;
        return;
    }

    // ---- block culling of occluders
    const bool have_tris = a.bvh.ntri > 0;
    if (have_tris) {
        // candidate triangles: all of them in small scenes, else the BVH leaves
        // whose boxes overlap the block's union box
        if (tid == 0) {
            if (a.bvh.ntri <= kMaxCand) {
                for (int q = 0; q < a.bvh.ntri; ++q) sCand[q] = q;
                sNc = a.bvh.ntri;
            } else {
                const float bl[3] = {o2f(sBox[0]), o2f(sBox[1]), o2f(sBox[2])};
                const float bh[3] = {o2f(sBox[3]), o2f(sBox[4]), o2f(sBox[5])};
                int stack[kStack];
                int sp = 0, node = 0, nc = 0;
                bool over = false;
                for (int guard = 0; guard < a.bvh.nnodes && !over; ++guard) {
                    const float4 na = __ldg(a.bvh.nodes + 2 * node), nb = __ldg(a.bvh.nodes + 2 * node + 1);
                    bool descend = false;
                    if (na.x <= bh[0] && nb.x >= bl[0] && na.y <= bh[1] && nb.y >= bl[1] && na.z <= bh[2] &&
                        nb.z >= bl[2]) {
                        const int left = __float_as_int(na.w), right = __float_as_int(nb.w);
                        if (left < 0) {
                            for (int q = -left - 1; q < -left - 1 + right; ++q) {
                                if (nc >= kMaxCand) {
                                    over = true;
                                    break;
                                }
                                sCand[nc++] = q;
                            }
                        } else {
                            if (sp < kStack) stack[sp++] = right;
                            node = left;
                            descend = true;
                        }
                    }
                    if (!descend) {
                        if (sp == 0) break;
                        node = stack[--sp];
                    }
                }
                sNc = nc;
                sOverflow = over ? 1 : 0;
            }
        }
        __syncthreads();
        const int nc = sNc;
        if (!sOverflow && nc > 0) {
            // signed-distance ranges of every candidate over the block's points
            for (int c = tid; c < nc * 4; c += kTile) sRed[c >> 2][c & 3] = (c & 1) ? f2o(-3.0e38f) : f2o(3.0e38f);
            __syncthreads();
            for (int c = 0; c < nc; ++c) {
                const float4 P = __ldg(a.bvh.tris + 4 * sCand[c]);
                float sl = 3.0e38f, sh = -3.0e38f, dl = 3.0e38f, dh = -3.0e38f;
                if (src_ok) sl = sh = plane_dist(P, p.x, p.y, p.z);
                if (live) dl = dh = plane_dist(P, t.x, t.y, t.z);
                for (int off = 16; off > 0; off >>= 1) {
                    sl = fminf(sl, __shfl_xor_sync(0xffffffffu, sl, off));
                    sh = fmaxf(sh, __shfl_xor_sync(0xffffffffu, sh, off));
                    dl = fminf(dl, __shfl_xor_sync(0xffffffffu, dl, off));
                    dh = fmaxf(dh, __shfl_xor_sync(0xffffffffu, dh, off));
                }
                if ((tid & 31) == 0) {
                    atomicMin(&sRed[c][0], f2o(sl));
                    atomicMax(&sRed[c][1], f2o(sh));
                    atomicMin(&sRed[c][2], f2o(dl));
                    atomicMax(&sRed[c][3], f2o(dh));
                }
            }
            __syncthreads();
            if (tid == 0) {
                const float dx = o2f(sBox[3]) - o2f(sBox[0]), dy = o2f(sBox[4]) - o2f(sBox[1]),
                            dz = o2f(sBox[5]) - o2f(sBox[2]);
                const float rmax = sqrtf(dx * dx + dy * dy + dz * dz) * 1.0001f;
                // which side holds the ray origins
                bool src_origin = (HOP == HOP_SRC || HOP == HOP_NORESP || (HOP == HOP_RESP && !a.resp_dst_origin));
                bool dst_origin = (HOP == HOP_FP || (HOP == HOP_RESP && a.resp_dst_origin));
                if (HOP == HOP_F2F) {
                    src_origin = sFac[0] < sFac[3];  // some source facet below some destination facet
                    dst_origin = sFac[2] < sFac[1];
                }
                int keep = 0;
                for (int c = 0; c < nc; ++c) {
                    const float sl = o2f(sRed[c][0]), sh = o2f(sRed[c][1]), dl = o2f(sRed[c][2]), dh = o2f(sRed[c][3]);
                    bool m = false;
                    if (src_origin) m = m || may_occlude(sl, sh, dl, dh, rmax);
                    if (dst_origin) m = m || may_occlude(dl, dh, sl, sh, rmax);
                    if (m) {
                        const float4 *T = a.bvh.tris + 4 * sCand[c];
                        sTri[4 * keep] = T[0];
                        sTri[4 * keep + 1] = T[1];
                        sTri[4 * keep + 2] = T[2];
                        sTri[4 * keep + 3] = T[3];
                        ++keep;
                    }
                }
                sKeep = keep;
            }
            __syncthreads();
            // ALL OCCLUDED: one kept triangle that every ray of the block crosses,
            // inside, before tmax (ray origins on one side: sources for the
            // source hop and NO_RESP, destinations for the field-point readout)
            if (HOP != HOP_F2F && sKeep > 0) {
                const bool from_dst = HOP == HOP_FP || (HOP == HOP_RESP && a.resp_dst_origin);
                const int ob = from_dst ? 12 : 6, eb = from_dst ? 6 : 12;
                const float ol[3] = {o2f(sBox[ob]), o2f(sBox[ob + 1]), o2f(sBox[ob + 2])};
                const float oh[3] = {o2f(sBox[ob + 3]), o2f(sBox[ob + 4]), o2f(sBox[ob + 5])};
                const float el[3] = {o2f(sBox[eb]), o2f(sBox[eb + 1]), o2f(sBox[eb + 2])};
                const float eh[3] = {o2f(sBox[eb + 3]), o2f(sBox[eb + 4]), o2f(sBox[eb + 5])};
                float S = 1.0f;
#pragma unroll
                for (int k = 0; k < 3; ++k) S = fmaxf(S, 1.0f + fmaxf(fmaxf(fabsf(ol[k]), fabsf(oh[k])),
                                                                    fmaxf(fabsf(el[k]), fabsf(eh[k]))));
                const float tol = 1e-5f * S;
                // shortest possible ray of the block (box gap)
                float g2 = 0.0f;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float gk = fmaxf(0.0f, fmaxf(ol[k] - eh[k], el[k] - oh[k]));
                    g2 = fmaf(gk, gk, g2);
                }
                const float rmin_pair = sqrtf(g2);
                for (int c = 0; c < sKeep; ++c) {
                    const float4 P = sTri[4 * c];
                    // plane distances over the two boxes (exact ranges of an affine function)
                    float o_lo = -P.w, o_hi = -P.w, e_lo = -P.w, e_hi = -P.w;
                    const float nv[3] = {P.x, P.y, P.z};
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        o_lo += fminf(nv[k] * ol[k], nv[k] * oh[k]);
                        o_hi += fmaxf(nv[k] * ol[k], nv[k] * oh[k]);
                        e_lo += fminf(nv[k] * el[k], nv[k] * eh[k]);
                        e_hi += fmaxf(nv[k] * el[k], nv[k] * eh[k]);
                    }
                    const bool split = (o_lo > 1.2e-4f * S && e_hi < -tol) || (o_hi < -1.2e-4f * S && e_lo > tol);
                    if (!split) continue;  // uniform per block
                    const float a0 = fminf(fabsf(o_lo), fabsf(o_hi)), a0max = fmaxf(fabsf(o_lo), fabsf(o_hi));
                    const float a1 = fminf(fabsf(e_lo), fabsf(e_hi)), a1max = fmaxf(fabsf(e_lo), fabsf(e_hi));
                    // every crossing at least rmin_pair * a1 / (a0max + a1max) before the end point
                    if (!(rmin_pair * a1 > 1.2e-3f * (a0max + a1max) + tol)) continue;
                    // the 64 corner-to-corner crossings must lie inside the triangle
                    bool inside = true;
                    if (tid < 64) {
                        const int oc = tid & 7, ec = tid >> 3;
                        const float ox = (oc & 1) ? oh[0] : ol[0], oy = (oc & 2) ? oh[1] : ol[1],
                                    oz = (oc & 4) ? oh[2] : ol[2];
                        const float ex = (ec & 1) ? eh[0] : el[0], ey = (ec & 2) ? eh[1] : el[1],
                                    ez = (ec & 4) ? eh[2] : el[2];
                        const float d0 = plane_dist(P, ox, oy, oz), d1 = plane_dist(P, ex, ey, ez);
                        const float sp = d0 / (d0 - d1);
                        const float X = fmaf(ex - ox, sp, ox), Y = fmaf(ey - oy, sp, oy), Z = fmaf(ez - oz, sp, oz);
#pragma unroll
                        for (int q = 1; q <= 3; ++q) {
                            const float4 M = sTri[4 * c + q];
                            if (!(fmaf(M.x, X, fmaf(M.y, Y, M.z * Z)) - M.w > tol)) inside = false;
                        }
                    }
                    if (__syncthreads_and(inside)) {
                        if (tid == 0) sAllOcc = 1;
                        break;
                    }
                }
                __syncthreads();
            }
        }
    }
    if (sAllOcc) {
        if (tid == 0) a.mask.flags[fidx] = kFlagNone;
        if (a.full) {
            const int ntile = min(kTile, a.nsrc - i0);
            const int nw = (ntile + 31) >> 5;
            if (live)
                for (int w = 0; w < nw; ++w) a.mask.bits[(long long)(tile * kWordsPerTile + w) * a.mask.pitch + j] = 0u;
        }
        return;
    }
    const int nkeep = sKeep;
    const bool overflow = have_tris && sOverflow;

    // ---- block class.  CLEAR: no triangle can occlude any pair, so the sum
    // kernel evaluates the gates inline and no bits are stored (unless the full
    // mask is requested).  FACET_SELF blocks whose sides share a facet range
    // keep per-pair bits: the inline gates do not see the source facet.
    bool clear = !overflow && nkeep == 0;
    if (HOP == HOP_F2F) clear = clear && (sFac[1] < sFac[2] || sFac[3] < sFac[0]);
    // ALL GATES: every pair passes its cosine gates with margin.  With one
    // source facet normal n_s and one destination facet normal n_d per block,
    // the gate values are dot(+-v, n) / |v| with v = p_dst - p_src; their minima
    // are bounded below by plane-distance ranges over the block divided by
    // the longest pair distance.  When the bound clears 1e-5 (the per-pair
    // estimates are within 1e-6 of the exact values, so the exact gates pass),
    // no pair needs a gate.  (Uniform facets on both sides of a FACET_SELF
    // block that is not NONE are two different facets.)  A CLEAR block with
    // all gates passing is ALL; a block with per-pair bits skips the gates.
    bool gates_all = false;
    // FACET_SELF blocks with one facet on each side: the per-point
    // projections on both normals decide most pairs' gates without the
    // pair's own vector (see the pair loop)
    bool proj = false;
    float t_s = 0.0f, t_d = 0.0f, proj_hi = 0.0f, proj_lo = 0.0f;
    __shared__ float2 sProj[kTile];
    __shared__ float4 sWP[kWordsPerTile];  // per word: min, max of p.n_s; min, max of p.n_d
    {
        const bool need_s = HOP != HOP_SRC,
                   need_d = (HOP == HOP_SRC && !a.dst_is_field) || HOP == HOP_F2F || HOP == HOP_RESP;
        const bool uni = (!need_s || sFac[0] == sFac[1]) && (!need_d || sFac[2] == sFac[3]);
        if (uni) {
            const float4 ns = sN[0];
            float4 nd = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (need_d) nd = a.dst_facet_n[a.dst_facet[jb * kTile]];
            // ranges of p.n_s and p.n_d over sources and destinations
            float s_s = -3.0e38f, s_d = 3.0e38f, d_s = 3.0e38f, d_d = -3.0e38f;
            if (src_ok) {
                s_s = fmaf(p.x, ns.x, fmaf(p.y, ns.y, p.z * ns.z));
                s_d = fmaf(p.x, nd.x, fmaf(p.y, nd.y, p.z * nd.z));
            }
            if (live) {
                d_s = fmaf(t.x, ns.x, fmaf(t.y, ns.y, t.z * ns.z));
                d_d = fmaf(t.x, nd.x, fmaf(t.y, nd.y, t.z * nd.z));
            }
            float ps_min = 3.0e38f, pd_max = -3.0e38f;
            if (HOP == HOP_F2F && a.gate_proj) {
                proj = true;
                sProj[tid] = make_float2(s_s, s_d);
                t_s = d_s;
                t_d = d_d;
                if (src_ok) {
                    ps_min = s_s;
                    pd_max = s_d;
                }
            }
            for (int off = 16; off > 0; off >>= 1) {
                s_s = fmaxf(s_s, __shfl_xor_sync(0xffffffffu, s_s, off));
                s_d = fminf(s_d, __shfl_xor_sync(0xffffffffu, s_d, off));
                d_s = fminf(d_s, __shfl_xor_sync(0xffffffffu, d_s, off));
                d_d = fmaxf(d_d, __shfl_xor_sync(0xffffffffu, d_d, off));
                ps_min = fminf(ps_min, __shfl_xor_sync(0xffffffffu, ps_min, off));
                pd_max = fmaxf(pd_max, __shfl_xor_sync(0xffffffffu, pd_max, off));
            }
            // warp w holds the sources of mask word w: their projection ranges
            if (proj && (tid & 31) == 0) sWP[tid >> 5] = make_float4(ps_min, s_s, s_d, pd_max);
            __syncthreads();  // every thread has read the candidate ranges in sRed
            if (tid < 4) sRed[0][tid] = (tid == 0 || tid == 3) ? f2o(-3.0e38f) : f2o(3.0e38f);
            __syncthreads();
            if ((tid & 31) == 0) {
                atomicMax(&sRed[0][0], f2o(s_s));
                atomicMin(&sRed[0][1], f2o(s_d));
                atomicMin(&sRed[0][2], f2o(d_s));
                atomicMax(&sRed[0][3], f2o(d_d));
            }
            __syncthreads();
            const float dx = o2f(sBox[3]) - o2f(sBox[0]), dy = o2f(sBox[4]) - o2f(sBox[1]),
                        dz = o2f(sBox[5]) - o2f(sBox[2]);
            const float rmax = sqrtf(dx * dx + dy * dy + dz * dz) * 1.0001f;
            float S = 1.0f;
#pragma unroll
            for (int k = 0; k < 6; ++k) S = fmaxf(S, 1.0f + fabsf(o2f(sBox[k])));
            const float thr = rmax * 1e-5f + S * 1e-6f;
            // source-side gate: dot(v, n_s) >= d_s - s_s ; destination side: -dot(v, n_d) >= s_d - d_d
            const bool ok_s = !need_s || (o2f(sRed[0][2]) - o2f(sRed[0][0]) > thr);
            const bool ok_d = !need_d || (o2f(sRed[0][1]) - o2f(sRed[0][3]) > thr);
            gates_all = ok_s && ok_d;
            if (proj) {
                // D = dot(v, n) of a pair (v = p_dst - p_src rounded to FP32)
                // differs from the difference of the two points' projections
                // by at most 1e-6 (rmax + sum_k max |coordinate_k|) (rounding
                // of v, of the projections and of their difference); with
                // |v| <= rmax, D above proj_hi means a gate value above
                // 3e-6 (cos_gate's estimate above 2e-6: pass) and D below
                // proj_lo one below -2e-6 (estimate negative: fail)
                float Ssum = 0.0f;
#pragma unroll
                for (int k = 0; k < 3; ++k) Ssum += fmaxf(fabsf(o2f(sBox[k])), fabsf(o2f(sBox[3 + k])));
                const float E = 1e-6f * (rmax + Ssum);
                proj_hi = E + 3e-6f * rmax;
                proj_lo = -(E + 2e-6f * rmax);
            }
        }
    }
    // Hops whose only gate is the source fragment's (readout, target -> field
    // object): per source s the range of dot(t - s, n_s) over the
    // destination box (exact ranges of an affine function) bounds every
    // pair's gate value, whatever the facets of the tile.  No pair passes when
    // the largest upper bound is below -thr; every pair passes when the
    // smallest lower bound clears thr (the margins of the ALL test).  With a
    // convex target and every pair passing by a wide margin, no pair can be
    // occluded either (occluded_pair's bounds, with the block's largest
    // coordinate and cos >= the smallest bound / rmax): the block is ALL.
    // Facet runs of each source word (word w = warp w's sources, in facet
    // order): per run its facet normal, the range of s.n over its sources and
    // their bits.  A destination t then bounds the gate values n.(t - s) of
    // a whole run with one dot product.  Words of more than kRuns runs are
    // evaluated pair by pair.
    constexpr int kRuns = 8;
    __shared__ float4 sRunN[kWordsPerTile][kRuns];  // normal, (unused)
    __shared__ float2 sRunB[kWordsPerTile][kRuns];  // min, max of s.n
    __shared__ uint32_t sRunM[kWordsPerTile][kRuns];
    __shared__ int sRunC[kWordsPerTile];
    float sg_thr = 0.0f, sg_rmax = 1.0f, sg_E = 0.0f;
    if (HOP == HOP_NORESP || HOP == HOP_FP) {
        __shared__ int sGB[2];
        {
            const int lane_ = tid & 31, wq = tid >> 5;
            const int fac = src_ok ? __float_as_int(n.w) : -1;
            const int prev = __shfl_up_sync(0xffffffffu, fac, 1);
            const bool start = src_ok && (lane_ == 0 || prev != fac);
            const unsigned starts = __ballot_sync(0xffffffffu, start);
            const int nruns = __popc(starts);
            const int myrun = src_ok ? __popc(starts & ((2u << lane_) - 1u)) - 1 : -1;
            const float b = fmaf(p.x, n.x, fmaf(p.y, n.y, p.z * n.z));
            if (nruns <= kRuns) {
                for (int r = 0; r < nruns; ++r) {
                    const bool in = myrun == r;
                    const unsigned m = __ballot_sync(0xffffffffu, in);
                    const float bl = warp_min(in ? b : 3.0e38f), bh = warp_max(in ? b : -3.0e38f);
                    if (lane_ == __ffs(m) - 1) {
                        sRunN[wq][r] = make_float4(n.x, n.y, n.z, 0.0f);
                        sRunB[wq][r] = make_float2(bl, bh);
                        sRunM[wq][r] = m;
                    }
                }
            }
            if (lane_ == 0) sRunC[wq] = nruns <= kRuns ? nruns : -1;
        }
        const float dl[3] = {o2f(sBox[12]), o2f(sBox[13]), o2f(sBox[14])};
        const float dh[3] = {o2f(sBox[15]), o2f(sBox[16]), o2f(sBox[17])};
        float lo = 3.0e38f, hi = -3.0e38f;
        if (src_ok) {
            const float nv[3] = {n.x, n.y, n.z};
            float bmin = 0.0f, bmax = 0.0f;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                bmin += fminf(nv[k] * dl[k], nv[k] * dh[k]);
                bmax += fmaxf(nv[k] * dl[k], nv[k] * dh[k]);
            }
            const float sp = fmaf(p.x, n.x, fmaf(p.y, n.y, p.z * n.z));
            lo = bmin - sp;
            hi = bmax - sp;
        }
        lo = warp_min(lo);
        hi = warp_max(hi);
        __syncthreads();  // sGB is free
        if (tid == 0) {
            sGB[0] = f2o(3.0e38f);
            sGB[1] = f2o(-3.0e38f);
        }
        __syncthreads();
        if ((tid & 31) == 0) {
            atomicMin(&sGB[0], f2o(lo));
            atomicMax(&sGB[1], f2o(hi));
        }
        __syncthreads();
        const float LO = o2f(sGB[0]), HI = o2f(sGB[1]);
        const float dx = o2f(sBox[3]) - o2f(sBox[0]), dy = o2f(sBox[4]) - o2f(sBox[1]),
                    dz = o2f(sBox[5]) - o2f(sBox[2]);
        const float rmax = sqrtf(dx * dx + dy * dy + dz * dz) * 1.0001f;
        float S = 1.0f;
#pragma unroll
        for (int k = 0; k < 6; ++k) S = fmaxf(S, 1.0f + fabsf(o2f(sBox[k])));
        const float thr = rmax * 1e-5f + S * 1e-6f;
        sg_thr = thr;
        sg_rmax = rmax;
        sg_E = 2e-6f * (1.0f + a.convex_vmax + S);
        const int ntile = min(kTile, a.nsrc - i0);
        const int nw = (ntile + 31) >> 5;
        if (HI < -thr) {
            // no pair passes its gate
            if (tid == 0) a.mask.flags[fidx] = kFlagNone;
            if (a.full && live)
                for (int w = 0; w < nw; ++w) a.mask.bits[(long long)(tile * kWordsPerTile + w) * a.mask.pitch + j] = 0u;
            return;
        }
        if (LO > thr) {
            gates_all = true;
            const float E = 2e-6f * (1.0f + a.convex_vmax + S);
            const float cmin = LO / rmax;
            const bool no_occ = clear || (a.convex && (HOP == HOP_NORESP ? E < 0.99e-4f * 0.999f * cmin
                                                                          : cmin * 0.9e-3f * 0.999f > E));
            if (no_occ) {
                if (tid == 0) a.mask.flags[fidx] = kFlagAll;
                if (a.full && live)
                    for (int w = 0; w < nw; ++w) {
                        const int bmax = min(32, ntile - w * 32);
                        a.mask.bits[(long long)(tile * kWordsPerTile + w) * a.mask.pitch + j] =
                            bmax == 32 ? 0xffffffffu : ((1u << bmax) - 1u);
                    }
                return;
            }
        }
    }
    if (clear && !a.full) {
        if (tid == 0) a.mask.flags[fidx] = gates_all ? kFlagAll : kFlagClear;
        return;
    }

    // ---- pairs, one 32-source word at a time per destination thread.
    // Gates: with the projections, a word whose extreme sources pass (or
    // fail) with certainty decides all its pairs at once -- the difference
    // of projections is monotone in the source's projection, so the
    // per-pair differences lie between the extremes' -- otherwise the pairs
    // of the word are decided one by one (projections where certain, the
    // exact gates under a warp vote where not).
    // Occlusion, with a candidate list: a pair needs the test only when some
    // candidate's plane separates its two points strictly (the first test of
    // tri_blocks_v, on the same plane distances); the sources on each side of
    // each plane are bit masks per word, so the pairs to test are found for
    // 32 sources at once.  They are queued with their bit set, and tested
    // by all threads together after the word, clearing the bits of the
    // occluded pairs: the few segments that cross a plane do not hold whole
    // warps.  Without a list (too many candidates) the test runs in place.
    constexpr int kQCap = kTile * 32;  // one word's pairs
    __shared__ uint32_t sPos[kMaxCand][kWordsPerTile], sNeg[kMaxCand][kWordsPerTile];
    __shared__ unsigned short sQ[kQCap];
    __shared__ uint32_t sW[kWordsPerTile][kTile];
    __shared__ float4 sTd[kTile];
    __shared__ int sQn[2];
    const int lane = tid & 31;
    // convex targets: each pair's test is first narrowed by occluded_pair (most
    // need none), so the candidate-list queue is not used
    const bool convex_hop = a.convex && (HOP == HOP_NORESP || HOP == HOP_FP || (HOP == HOP_SRC && !a.dst_is_field));
    const bool signs = !clear && !overflow && nkeep > 0 && !convex_hop;
    const bool use_queue = signs || (!clear && convex_hop && (overflow || nkeep > 0));
    unsigned tpos = 0u, tneg = 0u;
    if (signs) {
        for (int c = 0; c < nkeep; ++c) {
            const float4 Pl = sTri[4 * c];
            const float ds = plane_dist(Pl, p.x, p.y, p.z), dd = plane_dist(Pl, t.x, t.y, t.z);
            const unsigned bp = __ballot_sync(0xffffffffu, src_ok && ds > 0.0f);
            const unsigned bn = __ballot_sync(0xffffffffu, src_ok && ds < 0.0f);
            if (lane == 0) {
                sPos[c][tid >> 5] = bp;
                sNeg[c][tid >> 5] = bn;
            }
            tpos |= (dd > 0.0f ? 1u : 0u) << c;
            tneg |= (dd < 0.0f ? 1u : 0u) << c;
        }
    }
    if (use_queue) {
        sTd[tid] = make_float4(t.x, t.y, t.z, __int_as_float(ft));
        if (tid < 2) sQn[tid] = 0;
    }
    __syncthreads();
    const int ntile = min(kTile, a.nsrc - i0);
    const int nw = (ntile + 31) >> 5;
    for (int w = 0; w < nw; ++w) {
        const int bmax = min(32, ntile - w * 32);
        const uint32_t valid = live ? (bmax == 32 ? 0xffffffffu : ((1u << bmax) - 1u)) : 0u;
        uint32_t word = valid;
        bool mixed = !gates_all && live;
        uint32_t todo = valid;    // pairs whose gates are evaluated one by one
        uint32_t no_walk = 0u;    // pairs that pass by a margin that rules out a crossing
        if ((HOP == HOP_NORESP || HOP == HOP_FP) && mixed) {
            const int nr = sRunC[w];
            if (nr >= 0) {
                // per run: n.t - max(s.n) <= n.(t - s) <= n.t - min(s.n) (thr for rounding)
                uint32_t pass = 0u;
                todo = 0u;
                for (int r = 0; r < nr; ++r) {
                    const float4 rn = sRunN[w][r];
                    const float2 rb = sRunB[w][r];
                    const uint32_t rm = sRunM[w][r];
                    const float vt = fmaf(rn.x, t.x, fmaf(rn.y, t.y, rn.z * t.z));
                    const float lower = vt - rb.y, upper = vt - rb.x;
                    if (upper < -sg_thr) continue;
                    if (lower > sg_thr) {
                        pass |= rm;
                        const float cmin = lower / sg_rmax;
                        if (a.convex && (HOP == HOP_NORESP ? sg_E < 0.99e-4f * 0.999f * cmin
                                                           : cmin * 0.9e-3f * 0.999f > sg_E))
                            no_walk |= rm;
                    } else {
                        todo |= rm;
                    }
                }
                word = pass & valid;
                todo &= valid;
                mixed = todo != 0u;
            }
        }
        if (mixed && proj) {
            const float4 wp = sWP[w];
            const bool all_ok = (t_s - wp.y > proj_hi) && (wp.z - t_d > proj_hi);
            const bool all_fail = (t_s - wp.x < proj_lo) || (wp.w - t_d < proj_lo);
            if (all_ok || all_fail) {
                mixed = false;
                word = all_ok ? valid : 0u;
            }
        }
        if (__any_sync(0xffffffffu, mixed)) {
            uint32_t pw = 0;
#pragma unroll 4
            for (int b = 0; b < 32; ++b) {
                const int q = w * 32 + b;
                const bool act = mixed && ((todo >> b) & 1u);
                bool pass = act, unsure = act;
                if (proj) {
                    // gate 1: cos(v, n_s) from D1 = (t - p).n_s; gate 2:
                    // cos(-v, n_d) from D2 = (p - t).n_d
                    const float2 pq = sProj[q];
                    const float D1 = t_s - pq.x, D2 = pq.y - t_d;
                    const bool fail = D1 < proj_lo || D2 < proj_lo;
                    const bool ok = D1 > proj_hi && D2 > proj_hi;
                    pass = act && ok;
                    unsure = act && !fail && !ok;
                }
                if (__any_sync(0xffffffffu, unsure)) {
                    const bool g = pair_gates_vote<HOP>(a, sP[q], sN[q], t, nt, ft, unsure);
                    if (unsure) pass = g;
                }
                pw |= pass ? (1u << b) : 0u;
            }
            if (mixed) word = (word & ~todo) | (pw & todo);
        }
        if (!clear && (overflow || nkeep > 0)) {
            uint32_t tq = 0u;  // this lane's pairs of the word to test after the word
            if (signs) {
                uint32_t cross = 0u;
                for (int c = 0; c < nkeep; ++c) {
                    if ((tneg >> c) & 1u) cross |= sPos[c][w];
                    if ((tpos >> c) & 1u) cross |= sNeg[c][w];
                }
                tq = word & cross;
            } else if (convex_hop) {
                uint32_t c = word & ~no_walk;
                while (c) {
                    const int b = __ffs(c) - 1;
                    c &= c - 1u;
                    const int q = w * 32 + b;
                    float3 o, e;
                    pair_ray<HOP>(sP[q], sN[q], t, ft, o, e, a.resp_dst_origin);
                    if (convex_needs_test<HOP>(a, sN[q], nt, o, e)) tq |= 1u << b;
                }
            } else {
                uint32_t c = word;
                while (c) {
                    const int b = __ffs(c) - 1;
                    c &= c - 1u;
                    const int q = w * 32 + b;
                    float3 o, e;
                    pair_ray<HOP>(sP[q], sN[q], t, ft, o, e, a.resp_dst_origin);
                    if (occluded_full(a.bvh, o, e)) word &= ~(1u << b);
                }
            }
            if (use_queue) {
                // one slot range per warp; the warp's pairs in source-major
                // order (per source bit, the lanes that test it in lane order),
                // so that the stores here and the tests' bit clears in sW
                // after the word touch consecutive entries, not one lane's run
                int tot = __popc(tq);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
                int base = 0;
                if (lane == 0 && tot > 0) base = atomicAdd(&sQn[w & 1], tot);
                base = __shfl_sync(0xffffffffu, base, 0);
                const unsigned below = (1u << lane) - 1u;
                unsigned srcs = __reduce_or_sync(0xffffffffu, tq);
                while (srcs) {  // warp-uniform
                    const int b = __ffs(srcs) - 1;
                    srcs &= srcs - 1u;
                    const bool mine = (tq >> b) & 1u;
                    const unsigned m = __ballot_sync(0xffffffffu, mine);
                    if (mine) sQ[base + __popc(m & below)] = (unsigned short)(((w * 32 + b) << 8) | tid);
                    base += __popc(m);
                }
            }
        }
        sW[w][tid] = word;
        if (use_queue) {
            if (tid == 0) sQn[(w + 1) & 1] = 0;  // last read before the previous word's second barrier
            __syncthreads();
            const int nq = sQn[w & 1];
            for (int e = tid; e < nq; e += kTile) {
                const unsigned code = sQ[e];
                const int q = (int)(code >> 8), jl = (int)(code & 255u);
                const float4 td = sTd[jl];
                const int fd = __float_as_int(td.w);
                float3 o, en;
                pair_ray<HOP>(sP[q], sN[q], td, fd, o, en, a.resp_dst_origin);
                bool occ;
                if (signs) {
                    occ = occluded_list(sTri, nkeep, o, en);
                } else {
                    const float4 ntd = (a.dst_facet && fd >= 0) ? a.dst_facet_n[fd] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    occ = occluded_pair<HOP>(a, sN[q], ntd, o, en);
                }
                if (occ) atomicAnd(&sW[w][jl], ~(1u << (q & 31)));
            }
            __syncthreads();
        }
    }
    __syncthreads();
    uint32_t any = 0;
    for (int w = 0; w < nw; ++w) {
        const uint32_t word = sW[w][tid];
        if (live) a.mask.bits[(long long)(tile * kWordsPerTile + w) * a.mask.pitch + j] = word;
        any |= word;
    }
    const int blk = __syncthreads_or(any != 0u);
    if (tid == 0) a.mask.flags[fidx] = clear ? kFlagClear : (blk ? kFlagBits : kFlagNone);
}

// k_mask<HOP>: one CTA per block of the grid (destination block x, source
// tile y).
template <int HOP>
__global__ void __launch_bounds__(kTile) k_mask(MaskArgs a)
{
    mask_block<HOP>(a, (int)blockIdx.x);
}

// The pair kernel of a bounce mask on the blocks a classification pass left
// for per-pair bits (counted on the device): a grid of resident CTAs takes
// the listed blocks one at a time from a counter (their costs differ by an
// order of magnitude), so the host need not read the count first.  The
// counter only grows: every CTA leaves once it passes the count.
__global__ void __launch_bounds__(kTile) k_mask_listed(MaskArgs a)
{
    __shared__ int s_q;
    const int n = *a.blist_count;
    for (;;) {
        if (threadIdx.x == 0) s_q = atomicAdd(a.blist_next, 1);
        __syncthreads();
        const int q = s_q;  // CTA-uniform
        if (q >= n) break;
        mask_block<HOP_F2F>(a, q);
        __syncthreads();  // s_q and the shared state are rewritten next
    }
}

// ---------------------------------------------------------------- bounce-mask classification
// The block decisions of k_mask<HOP_F2F> (same facet, occluder culling, the
// ALL test of the cosine gates) taken by one warp per block from the same
// values -- min / max reductions of the same per-point expressions, which
// do not depend on the order of reduction -- so every verdict equals
// k_mask's.  NONE, CLEAR and ALL blocks get their flag here (the flags start
// at NONE); blocks that need per-pair bits are appended to a list that
// k_mask then runs on (it repeats the culling to build its triangle list and
// writes the flag).  The order of the list does not matter: each block's
// bits and flag depend only on the block.
constexpr int kClsWarps = 8;

struct WarpRange {
    float lo, hi;
};


__global__ void __launch_bounds__(32 * kClsWarps, 3) k_mask_classify_f2f(MaskArgs a, int2 *blist, int *count)
{
    __shared__ int sCand[kClsWarps][kMaxCand];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int I = blockIdx.y;
    const int J = (a.upper_only ? I : 0) + (int)blockIdx.x * kClsWarps + warp;
    const int nt = a.mask.ntiles, nb = a.mask.ndstblocks;
    if (J >= nb || I >= nt) return;  // warp-uniform; no block-wide barrier below
    if (a.src_frange && a.dst_frange) {
        // both tiles inside one facet: no pair interacts (the flag stays NONE)
        const int2 fs = __ldg(a.src_frange + I), fd = __ldg(a.dst_frange + J);
        if (fs.x == fs.y && fd.x == fd.y && fs.x == fd.x) return;
    }
    const int i0 = I * kTile, j0 = J * kTile;
    const int ni = min(kTile, a.nsrc - i0), nj = min(kTile, a.ndst - j0);
    // this lane's points: q = lane + 32 m, m < 8, of both tiles
    float4 P[8], T[8];
    int fs_lo = 2147483647, fs_hi = -2147483647, fd_lo = 2147483647, fd_hi = -2147483647;
    float slo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, shi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    float dlo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, dhi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int q = lane + 32 * m;
        P[m] = q < ni ? __ldg(a.src_pos + i0 + q) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        T[m] = q < nj ? __ldg(a.dst_pos + j0 + q) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (q < ni) {
            const int f = __ldg(a.src_facet + i0 + q);
            fs_lo = min(fs_lo, f);
            fs_hi = max(fs_hi, f);
            slo[0] = fminf(slo[0], P[m].x); shi[0] = fmaxf(shi[0], P[m].x);
            slo[1] = fminf(slo[1], P[m].y); shi[1] = fmaxf(shi[1], P[m].y);
            slo[2] = fminf(slo[2], P[m].z); shi[2] = fmaxf(shi[2], P[m].z);
        }
        if (q < nj) {
            const int f = __ldg(a.dst_facet + j0 + q);
            fd_lo = min(fd_lo, f);
            fd_hi = max(fd_hi, f);
            dlo[0] = fminf(dlo[0], T[m].x); dhi[0] = fmaxf(dhi[0], T[m].x);
            dlo[1] = fminf(dlo[1], T[m].y); dhi[1] = fmaxf(dhi[1], T[m].y);
            dlo[2] = fminf(dlo[2], T[m].z); dhi[2] = fmaxf(dhi[2], T[m].z);
        }
    }
    fs_lo = __reduce_min_sync(0xffffffffu, fs_lo);
    fs_hi = __reduce_max_sync(0xffffffffu, fs_hi);
    fd_lo = __reduce_min_sync(0xffffffffu, fd_lo);
    fd_hi = __reduce_max_sync(0xffffffffu, fd_hi);
    // blocks whose fragments all share one facet interact nowhere (flag stays NONE)
    if (fs_lo == fs_hi && fd_lo == fd_hi && fs_lo == fd_lo) return;
    float lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        slo[k] = warp_min(slo[k]);
        shi[k] = warp_max(shi[k]);
        dlo[k] = warp_min(dlo[k]);
        dhi[k] = warp_max(dhi[k]);
        lo[k] = fminf(slo[k], dlo[k]);
        hi[k] = fmaxf(shi[k], dhi[k]);
    }
    const long long fidx = (long long)I * nb + J;
    bool bits = false;
    if (a.bvh.ntri > 0) {
        // candidates: every triangle in small scenes, else the BVH leaves
        // whose boxes overlap the union box (the walk of k_mask, by lane 0)
        int nc = 0;
        bool over = false;
        if (a.bvh.ntri <= kMaxCand) {
            nc = a.bvh.ntri;
        } else if (lane == 0) {
            int stack[kStack];
            int sp = 0, node = 0;
            for (int guard = 0; guard < a.bvh.nnodes && !over; ++guard) {
                const float4 na = __ldg(a.bvh.nodes + 2 * node), nb4 = __ldg(a.bvh.nodes + 2 * node + 1);
                bool descend = false;
                if (na.x <= hi[0] && nb4.x >= lo[0] && na.y <= hi[1] && nb4.y >= lo[1] && na.z <= hi[2] &&
                    nb4.z >= lo[2]) {
                    const int left = __float_as_int(na.w), right = __float_as_int(nb4.w);
                    if (left < 0) {
                        for (int q = -left - 1; q < -left - 1 + right; ++q) {
                            if (nc >= kMaxCand) {
                                over = true;
                                break;
                            }
                            sCand[warp][nc++] = q;
                        }
                    } else {
                        if (sp < kStack) stack[sp++] = right;
                        node = left;
                        descend = true;
                    }
                }
                if (!descend) {
                    if (sp == 0) break;
                    node = stack[--sp];
                }
            }
        }
        __syncwarp();
        nc = __shfl_sync(0xffffffffu, nc, 0);
        over = __shfl_sync(0xffffffffu, (int)over, 0) != 0;
        if (over) {
            bits = true;
        } else {
            const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
            const float rmax = sqrtf(dx * dx + dy * dy + dz * dz) * 1.0001f;
            const bool src_origin = fs_lo < fd_hi, dst_origin = fd_lo < fs_hi;
            for (int c = 0; c < nc && !bits; ++c) {
                const int tri = a.bvh.ntri <= kMaxCand ? c : sCand[warp][c];
                const float4 Pl = __ldg(a.bvh.tris + 4 * tri);
                float sl = 3.0e38f, sh = -3.0e38f, dl = 3.0e38f, dh = -3.0e38f;
#pragma unroll
                for (int m = 0; m < 8; ++m) {
                    const int q = lane + 32 * m;
                    if (q < ni) {
                        const float v = plane_dist(Pl, P[m].x, P[m].y, P[m].z);
                        sl = fminf(sl, v);
                        sh = fmaxf(sh, v);
                    }
                    if (q < nj) {
                        const float v = plane_dist(Pl, T[m].x, T[m].y, T[m].z);
                        dl = fminf(dl, v);
                        dh = fmaxf(dh, v);
                    }
                }
                sl = warp_min(sl);
                sh = warp_max(sh);
                dl = warp_min(dl);
                dh = warp_max(dh);
                bool mo = false;
                if (src_origin) mo = mo || may_occlude(sl, sh, dl, dh, rmax);
                if (dst_origin) mo = mo || may_occlude(dl, dh, sl, sh, rmax);
                bits = mo;
            }
        }
    }
    // overlapping facet ranges keep per-pair bits (the inline gates do not see the source facet)
    if (!(fs_hi < fd_lo || fd_hi < fs_lo)) bits = true;
    if (bits) {
        if (lane == 0) {
            const int slot = atomicAdd(count, 1);
            blist[slot] = make_int2(I, J);
        }
        return;
    }
    // ALL: both cosine gates of every pair pass with margin (the test of k_mask)
    bool all = false;
    if (fs_lo == fs_hi && fd_lo == fd_hi) {
        const float4 ns = __ldg(a.src_facet_n + fs_lo), nd = __ldg(a.dst_facet_n + fd_lo);
        float s_s = -3.0e38f, s_d = 3.0e38f, d_s = 3.0e38f, d_d = -3.0e38f;
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const int q = lane + 32 * m;
            if (q < ni) {
                s_s = fmaxf(s_s, fmaf(P[m].x, ns.x, fmaf(P[m].y, ns.y, P[m].z * ns.z)));
                s_d = fminf(s_d, fmaf(P[m].x, nd.x, fmaf(P[m].y, nd.y, P[m].z * nd.z)));
            }
            if (q < nj) {
                d_s = fminf(d_s, fmaf(T[m].x, ns.x, fmaf(T[m].y, ns.y, T[m].z * ns.z)));
                d_d = fmaxf(d_d, fmaf(T[m].x, nd.x, fmaf(T[m].y, nd.y, T[m].z * nd.z)));
            }
        }
        s_s = warp_max(s_s);
        s_d = warp_min(s_d);
        d_s = warp_min(d_s);
        d_d = warp_max(d_d);
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        const float rmax = sqrtf(dx * dx + dy * dy + dz * dz) * 1.0001f;
        float S = 1.0f;
#pragma unroll
        for (int k = 0; k < 3; ++k) S = fmaxf(S, fmaxf(1.0f + fabsf(lo[k]), 1.0f + fabsf(hi[k])));
        const float thr = rmax * 1e-5f + S * 1e-6f;
        all = (d_s - s_s > thr) && (s_d - d_d > thr);
    }
    if (lane == 0) a.mask.flags[fidx] = all ? kFlagAll : kFlagClear;
}

// ---------------------------------------------------------------- batch visibility
// Interaction bits of the two hops of a batch item, per fragment: bit q of
// the source word when source q -> fragment passes the cos_inc gate and is
// not shadowed (ray from the source to the source-hop centroid), bit p of
// the receiver word when fragment -> receiver p passes the cos_scat gate
// and is not shadowed (ray from the receiver to the readout centroid).  The
// gates are the reference's exact FP32 decisions (cos_gate).
//
// Convex scenes (every vertex on or behind every triangle's plane within
// 1e-6 (1 + max |coordinate|), checked on the host): a ray from a point in
// front of the fragment's facet plane stays in front of it up to tmax =
// r - 1e-3, at least 1e-3 cos from the plane, while every triangle lies on
// or behind it; no triangle can hold the crossing point.  With a cosine of at
// least kConvexCos that margin (5e-5 m) exceeds the convexity tolerance and
// the FP32 rounding of the crossing test, so such pairs need no occlusion
// test.  Below it, a crossing point before the last 1e-4 / cos + 1e-3 metres
// of the ray lies at least 1e-4 m in front of the plane, beyond the reach of
// the same tolerances, so the BVH walk opens only boxes near the end of the
// ray.  Every pair of a non-convex scene walks the whole ray.
constexpr float kConvexCos = 0.05f;

__device__ __forceinline__ float convex_reach(float cosv) { return 1e-4f / fmaxf(cosv, 1e-9f) + 1e-3f; }

// Pass 1: one thread per fragment evaluates the 128 cosine gates; a pair
// that passes and needs a shadow test is appended to a queue (pair id
// 128 n + point, warp-aggregated) and provisionally marked visible; when the
// queue is full the thread tests it itself.  Pass 2 (k_batch_vis_hard) walks
// the BVH for the queued pairs, one thread each, and clears the bits of the
// shadowed ones: the divergent walks no longer hold warps of easy pairs.
// The fragment's data of a pair: its readout centroid, its source-hop
// centroid and its facet normal.
struct VisFrag {
    float4 pos, spos, n;
};

__device__ __forceinline__ VisFrag vis_frag(const BatchVisArgs &a, long long n)
{
    return VisFrag{a.frag_pos[n], a.frag_spos[n], a.frag_n[n]};
}

__device__ __forceinline__ void vis_pair(const BatchItem &it, const VisFrag &F, int pt, const float4 P, bool &gate,
                                         bool &hard, float &est)
{
    const bool readout = pt < kBatchMaxPoints;
    const float4 f = readout ? F.pos : F.spos;
    const float4 nf = F.n;
    // readout: v = field point - fragment, cos_scat = dot(v, n) / r (OptiX.cu:150-160);
    // source hop: v = fragment - source, cos_inc = dot(-v, n) / r (OptiX.cu:60-79)
    const float sg = readout ? 1.0f : -1.0f;
    const float vx = readout ? __fsub_rn(P.x, f.x) : __fsub_rn(f.x, P.x);
    const float vy = readout ? __fsub_rn(P.y, f.y) : __fsub_rn(f.y, P.y);
    const float vz = readout ? __fsub_rn(P.z, f.z) : __fsub_rn(f.z, P.z);
    const float rinv = rsqrtf(fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
    gate = cos_gate(vx, vy, vz, rinv, sg, nf.x, nf.y, nf.z);
    est = sg * fmaf(vx, nf.x, fmaf(vy, nf.y, vz * nf.z)) * rinv;
    hard = gate && !(it.convex && est >= kConvexCos);
}

__device__ __forceinline__ bool vis_shadowed(const BatchVisArgs &a, const BatchItem &it, const VisFrag &F, int pt,
                                             const float4 P, float est)
{
    const bool readout = pt < kBatchMaxPoints;
    const float4 f = readout ? F.pos : F.spos;
    return occluded_full(a.bvh[it.scene], make_float3(P.x, P.y, P.z), make_float3(f.x, f.y, f.z),
                         it.convex ? convex_reach(est) : 3.0e38f);
}

__device__ __forceinline__ int item_of(const BatchVisArgs &a, long long n)
{
    int lo = 0, hi = a.nitems - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.items[mid].frag0 <= n) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(kTile) k_batch_vis(BatchVisArgs a)
{
    __shared__ float4 sP[2 * kBatchMaxPoints];  // receivers at 0.., sources at 64..
    const int tid = threadIdx.x, lane = tid & 31;
    for (int q = tid; q < 2 * kBatchMaxPoints; q += kTile) {
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (q < kBatchMaxPoints && q < a.nrx) v = a.rx[q];
        if (q >= kBatchMaxPoints && q - kBatchMaxPoints < a.nsrc) v = a.src[q - kBatchMaxPoints];
        sP[q] = v;
    }
    __syncthreads();
    const long long n = (long long)blockIdx.x * kTile + tid;
    const bool live = n < a.nfrag;
    const BatchItem it = live ? a.items[item_of(a, n)] : BatchItem{};
    const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const VisFrag F = live ? vis_frag(a, n) : VisFrag{z4, z4, z4};
    // one word per 32 points: receivers 0-31, 32-63, sources 0-31, 32-63; the
    // hop (and so the centroid and the sign of the gate) is fixed per word
    unsigned w[4];
#pragma unroll
    for (int seg = 0; seg < 4; ++seg) {
        const bool readout = seg < 2;
        const int npts = readout ? a.nrx : a.nsrc;
        unsigned word = 0u;
#pragma unroll 2
        for (int b = 0; b < 32; ++b) {
            const int pt = seg * 32 + b;
            const bool active = live && (seg & 1) * 32 + b < npts;  // uniform over the warp but for live
            bool gate = false, hard = false;
            float est = 0.0f;
            if (active) vis_pair(it, F, pt, sP[pt], gate, hard, est);
            bool vis = gate;
            // queue the shadow tests of this point, one atomic per warp
            const unsigned need = __ballot_sync(0xffffffffu, hard);
            if (need) {
                unsigned base = 0u;
                if (lane == 0) base = atomicAdd(a.hard_count, (unsigned)__popc(need));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (hard) {
                    const unsigned slot = base + (unsigned)__popc(need & ((1u << lane) - 1u));
                    if (slot < a.hard_cap) a.hard[slot] = (unsigned)(n * (2 * kBatchMaxPoints) + pt);
                    else vis = !vis_shadowed(a, it, F, pt, sP[pt], est);  // queue full: test here
                }
            }
            word |= vis ? (1u << b) : 0u;
        }
        w[seg] = word;
    }
    if (live) a.vis[n] = make_uint4(w[0], w[1], w[2], w[3]);
}

// Pass 2: the queued shadow tests (grid-stride over the device count).
__global__ void __launch_bounds__(kTile) k_batch_vis_hard(BatchVisArgs a)
{
    const unsigned cnt = min(*a.hard_count, a.hard_cap);
    for (unsigned e = blockIdx.x * kTile + threadIdx.x; e < cnt; e += gridDim.x * kTile) {
        const unsigned id = a.hard[e];
        const long long n = id / (2 * kBatchMaxPoints);
        const int pt = (int)(id % (2 * kBatchMaxPoints));
        const BatchItem it = a.items[item_of(a, n)];
        const float4 P = pt < kBatchMaxPoints ? a.rx[pt] : a.src[pt - kBatchMaxPoints];
        bool gate, hard;
        float est;
        const VisFrag F = vis_frag(a, n);
        vis_pair(it, F, pt, P, gate, hard, est);
        if (vis_shadowed(a, it, F, pt, P, est))
            atomicAnd(reinterpret_cast<unsigned *>(a.vis + n) + (pt >> 5), ~(1u << (pt & 31)));
    }
}

// ---------------------------------------------------------------- sums
struct Dst {
    float px, py, pz;
    float nx, ny, nz;
};

// Gate from an estimate already at hand (same band rule as cos_gate): the
// decision always equals the reference's exact FP32 one.
__device__ __forceinline__ bool gate_from(float est, float vx, float vy, float vz, float sign, float nx, float ny,
                                          float nz)
{
    if (est > 2e-6f) return true;
    if (est < 0.0f) return false;
    return !(exact_cos(vx, vy, vz, sign, nx, ny, nz) < 1e-6f);
}

// One pair's term.  GATE: also evaluate the pair's cosine gates inline (CLEAR
// blocks) and return them in ok.
template <int HOP, bool ATT, bool GATE>
__device__ __forceinline__ void pair_term(const SumArgs &a, const float4 A, const float4 B, const Dst &d, float &tr,
                                          float &ti, bool &ok)
{
    // v = p_dst - p_src; |v|^2 with the reference's rounding (its r feeds the phase)
    const float vx = __fsub_rn(d.px, A.x), vy = __fsub_rn(d.py, A.y), vz = __fsub_rn(d.pz, A.z);
    const float r2 = dot_rn(vx, vy, vz, vx, vy, vz);
    // r: one Newton step on the reciprocal square root, r = r0 + (r2 - r0^2) / (2 r0)
    // with r0 = r2 * rsqrt(r2); within an ulp of the correctly rounded root
    const float rinv = rsqrtf(r2);
    const float r0 = r2 * rinv;
    const float r = fmaf(fmaf(-r0, r0, r2), 0.5f * rinv, r0);
    // phase k r in turns: r * (k / 2 pi) as an exact two-float product plus the
    // low part of k / 2 pi, the integer part removed exactly
    const float th = __fmul_rn(r, a.k2hi);
    const float tl = fmaf(r, a.k2lo, fmaf(r, a.k2hi, -th));
    const float frac = (th - rintf(th)) + tl;
    float sn, cs;
    __sincosf(frac * kTwoPi, &sn, &cs);
    const float damp = ATT ? __expf(-a.ka * r) : 1.0f;
    ok = true;
    if (HOP == HOP_SRC) {
        // cos_inc P e^{ikr} / r
        float ci = -(vx * d.nx + vy * d.ny + vz * d.nz) * rinv;
        if (a.dst_is_field)
            ci = 1.0f;
        else if (GATE)
            ok = gate_from(ci, vx, vy, vz, -1.0f, d.nx, d.ny, d.nz);
        const float amp = ATT ? ci * rinv * damp : ci * rinv;
        const float er = amp * cs, ei = amp * sn;
        tr = er * A.w - ei * B.w;
        ti = er * B.w + ei * A.w;
    } else {
        // -e^{ikr}/(4 pi) * (ik/r) + 1/r^2
        const float rinv2 = rinv * rinv;
        float gr, gi;
        if (ATT) {
            const float amp = rinv * kInv4Pi * damp;
            gr = fmaf(amp, fmaf(a.ka, cs, a.kr * sn), rinv2);
            gi = amp * fmaf(a.ka, sn, -a.kr * cs);
        } else {
            const float ampk = rinv * (kInv4Pi * a.kr);
            gr = fmaf(ampk, sn, rinv2);
            gi = -ampk * cs;
        }
        const float c1 = (vx * B.x + vy * B.y + vz * B.z) * rinv;  // cos_scat (source side)
        float wgt;
        if (HOP == HOP_F2F || HOP == HOP_RESP) {
            const float c2 = -(vx * d.nx + vy * d.ny + vz * d.nz) * rinv;  // cos_inc (destination side)
            wgt = c1 * c2;
            if (GATE) ok = gate_from(c1, vx, vy, vz, 1.0f, B.x, B.y, B.z) && gate_from(c2, vx, vy, vz, -1.0f, d.nx, d.ny, d.nz);
        } else {
            wgt = c1;
            if (GATE) ok = gate_from(c1, vx, vy, vz, 1.0f, B.x, B.y, B.z);
        }
        if (HOP != HOP_FP) {
            // regularised G below r_min = delta_src (OptiX.cu:340-346); near the
            // threshold the branch uses the correctly rounded r, as the reference
            float rr = r;
            if (fabsf(r - a.rmin) <= a.rmin * 4e-7f) rr = __fsqrt_rn(r2);
            if (rr < a.rmin) {
                gr = -a.ka * kInv4Pi;
                gi = a.kr * kInv4Pi;
            }
        }
        gr *= wgt;
        gi *= wgt;
        tr = gr * A.w - gi * B.w;
        ti = gr * B.w + gi * A.w;
    }
}

// pair_term of the source hop and the readout with the phase distance taken
// relative to an FP64 reference (o: the fragment's offset from its tile
// centroid for the readout).  The source hop evaluates its distance in FP64
// outright: it has S x N_cells pairs, a few per fragment.
struct RelRef;
template <int HOP, bool ATT>
__device__ __forceinline__ void pair_term_rel(const SumArgs &a, const float4 A, const float4 B, const Dst &d,
                                              const RelRef &ref, float4 o, bool gate, float &tr, float &ti, bool &ok);

// Phase of a pair in turns from a distance known in FP64 to within FP32
// round-off of a small correction: r = R + dr, R (FP64) the distance to a
// reference point, phase0 = frac(R k / 2 pi) reduced in FP64 once, dr in FP32.
__device__ __forceinline__ float rel_turns(float phase0, float dr, const SumArgs &a)
{
    const float th = __fmul_rn(dr, a.k2hi);
    const float tl = fmaf(dr, a.k2lo, fmaf(dr, a.k2hi, -th));
    const float f = phase0 + ((th - rintf(th)) + tl);
    return f - rintf(f);
}

// Relative geometry of the readout (HOP_FP): with o = p_i - c (fragment from
// its tile's centroid, small) and D = p_j - c (field point from the centroid,
// R = |D| in FP64), r^2 = R^2 - 2 o.D + |o|^2, so r - R = (|o|^2 - 2 o.D) /
// (r + R): FP32 arithmetic on small numbers, no cancellation at large R.
struct RelRef {
    float dx, dy, dz, R, phase0;
};

__device__ __forceinline__ RelRef rel_ref(const SumArgs &a, double px, double py, double pz, float4 c)
{
    const double dx = px - (double)c.x, dy = py - (double)c.y, dz = pz - (double)c.z;
    const double R = sqrt(dx * dx + dy * dy + dz * dz);
    const double t = R * a.k2pi;
    return RelRef{(float)dx, (float)dy, (float)dz, (float)R, (float)(t - floor(t))};
}

template <int HOP, bool ATT>
__device__ __forceinline__ void pair_term_rel(const SumArgs &a, const float4 A, const float4 B, const Dst &d,
                                              const RelRef &ref, float4 o, bool gate, float &tr, float &ti, bool &ok)
{
    // direction, cosines and amplitudes from the FP32 difference (relative
    // accuracy ~1e-7 is enough for them); only the phase needs r to ~1e-9 m
    const float vx = __fsub_rn(d.px, A.x), vy = __fsub_rn(d.py, A.y), vz = __fsub_rn(d.pz, A.z);
    const float r2 = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
    const float rinv = rsqrtf(r2);
    const float r = r2 * rinv;
    float turns;
    if (HOP == HOP_SRC) {
        const double ex = (double)d.px - (double)A.x, ey = (double)d.py - (double)A.y, ez = (double)d.pz - (double)A.z;
        const double t = sqrt(ex * ex + ey * ey + ez * ez) * a.k2pi;
        turns = (float)(t - rint(t));
    } else {
        // r - R = (|o|^2 - 2 o.D) / (r + R)
        const float num = fmaf(-2.0f, fmaf(o.x, ref.dx, fmaf(o.y, ref.dy, o.z * ref.dz)), o.w);
        turns = rel_turns(ref.phase0, num / (r + ref.R), a);
    }
    float sn, cs;
    __sincosf(turns * kTwoPi, &sn, &cs);
    const float damp = ATT ? __expf(-a.ka * r) : 1.0f;
    ok = true;
    if (HOP == HOP_SRC) {
        float ci = -(vx * d.nx + vy * d.ny + vz * d.nz) * rinv;
        if (a.dst_is_field)
            ci = 1.0f;
        else if (gate)
            ok = gate_from(ci, vx, vy, vz, -1.0f, d.nx, d.ny, d.nz);
        const float amp = ATT ? ci * rinv * damp : ci * rinv;
        const float er = amp * cs, ei = amp * sn;
        tr = er * A.w - ei * B.w;
        ti = er * B.w + ei * A.w;
    } else {
        const float rinv2 = rinv * rinv;
        float gr, gi;
        if (ATT) {
            const float amp = rinv * kInv4Pi * damp;
            gr = fmaf(amp, fmaf(a.ka, cs, a.kr * sn), rinv2);
            gi = amp * fmaf(a.ka, sn, -a.kr * cs);
        } else {
            const float ampk = rinv * (kInv4Pi * a.kr);
            gr = fmaf(ampk, sn, rinv2);
            gi = -ampk * cs;
        }
        const float c1 = (vx * B.x + vy * B.y + vz * B.z) * rinv;  // cos_scat
        if (gate) ok = gate_from(c1, vx, vy, vz, 1.0f, B.x, B.y, B.z);
        gr *= c1;
        gi *= c1;
        tr = gr * A.w - gi * B.w;
        ti = gr * B.w + gi * A.w;
    }
}

template <int HOP, bool ATT, bool REL = false>
__global__ void __launch_bounds__(kTile) k_sum(SumArgs a)
{
    __shared__ float4 sA[kTile];
    __shared__ float4 sB[kTile];
    __shared__ float4 sO[REL && HOP == HOP_FP ? kTile : 1];  // fragment offsets from the tile centroid
    const int tid = threadIdx.x;
    const int j = blockIdx.x * kTile + tid;
    const bool live = j < a.ndst;
    Dst d{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    int limit = a.nsrc;
    if (live) {
        const float4 p = a.dst_pos[j];
        d.px = p.x; d.py = p.y; d.pz = p.z;
        if (a.dst_facet) {
            const float4 n = a.dst_facet_n[a.dst_facet[j]];
            d.nx = n.x; d.ny = n.y; d.nz = n.z;
        }
        if (HOP == HOP_F2F) limit = a.dst_limit[j];
    }
    double accr = 0.0, acci = 0.0;
    const int t0 = blockIdx.y * a.tiles_per_split;
    const int t1 = min(t0 + a.tiles_per_split, a.mask.ntiles);
    for (int t = t0; t < t1; ++t) {
        const uint8_t fl = a.mask.flags[(long long)t * a.mask.ndstblocks + blockIdx.x];  // uniform per CTA
        if (fl == kFlagNone) continue;
        __syncthreads();
        RelRef ref{};
        {
            const int i = t * kTile + tid;
            const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            sA[tid] = i < a.nsrc ? a.srcA[i] : z;
            sB[tid] = i < a.nsrc ? a.srcB[i] : z;
            if (REL && HOP == HOP_FP) {
                const float4 c = a.tile_cen[t];
                const float4 p = sA[tid];
                const float ox = p.x - c.x, oy = p.y - c.y, oz = p.z - c.z;
                sO[tid] = make_float4(ox, oy, oz, fmaf(ox, ox, fmaf(oy, oy, oz * oz)));
                ref = rel_ref(a, (double)d.px, (double)d.py, (double)d.pz, c);
            }
        }
        __syncthreads();
        const int ntile = min(kTile, a.nsrc - t * kTile);
        const int nw = (ntile + 31) >> 5;
        float fr = 0.0f, fi = 0.0f;
        for (int w = 0; w < nw; ++w) {
            uint32_t m;
            if (fl == kFlagBits) {
                m = live ? a.mask.bits[(long long)(t * kWordsPerTile + w) * a.mask.pitch + j] : 0u;
            } else {
                const int nb = ntile - w * 32;  // CLEAR / ALL: every valid source
                m = !live ? 0u : (nb >= 32 ? 0xffffffffu : ((1u << nb) - 1u));
            }
            if (HOP == HOP_F2F) {
                // FACET_SELF zero-input rule: when this destination's input is 0
                // the sources of higher facets (its reciprocal partners) drop out
                const int keep = limit - (t * kTile + w * 32);
                m &= keep >= 32 ? 0xffffffffu : (keep <= 0 ? 0u : ((1u << keep) - 1u));
            }
            if (!__any_sync(0xffffffffu, m != 0u)) continue;
            if (REL) {
                // centroid-relative phase (the gates of CLEAR blocks inline as below)
#pragma unroll 4
                for (int b = 0; b < 32; ++b) {
                    const float4 A = sA[w * 32 + b];
                    const float4 B = sB[w * 32 + b];
                    float tr, ti;
                    bool ok;
                    pair_term_rel<HOP, ATT>(a, A, B, d, ref, REL && HOP == HOP_FP ? sO[w * 32 + b] : A,
                                            fl == kFlagClear, tr, ti, ok);
                    const bool on = ((m >> b) & 1u) && ok;
                    fr += on ? tr : 0.0f;
                    fi += on ? ti : 0.0f;
                }
            } else if (fl != kFlagClear) {
#pragma unroll 8
                for (int b = 0; b < 32; ++b) {
                    const float4 A = sA[w * 32 + b];
                    const float4 B = sB[w * 32 + b];
                    float tr, ti;
                    bool ok;
                    pair_term<HOP, ATT, false>(a, A, B, d, tr, ti, ok);
                    const bool on = (m >> b) & 1u;
                    fr += on ? tr : 0.0f;
                    fi += on ? ti : 0.0f;
                }
            } else {
#pragma unroll 8
                for (int b = 0; b < 32; ++b) {
                    const float4 A = sA[w * 32 + b];
                    const float4 B = sB[w * 32 + b];
                    float tr, ti;
                    bool ok;
                    pair_term<HOP, ATT, true>(a, A, B, d, tr, ti, ok);
                    const bool on = ((m >> b) & 1u) && ok;
                    fr += on ? tr : 0.0f;
                    fi += on ? ti : 0.0f;
                }
            }
        }
        accr += (double)fr;
        acci += (double)fi;
    }
    if (live) a.partial[(long long)blockIdx.y * a.ndst + j] = make_double2(accr, acci);
}

// ---------------------------------------------------------------- symmetric bounce sum
// FACET_SELF with reciprocity evaluated once per unordered pair, as the
// reference does (OptiX.cu:367-390): for source tile I < destination tile J
// the CTA computes T_ij = 0.9-free G(r_ij) cos_scat cos_inc once per pair and
// adds T_ij w_i into its destination row j (registers) and T_ij w_j into the
// column of i (warp reductions, per-warp shared sums, one write per (I, J)).
// Tiles are in facet order, so every interacting pair of such a block has
// facet(i) < facet(j): the row term is the forward term and the column term
// the reciprocal one, dropped in the final reduction when P_in[i] == 0.
// The diagonal tile (I == J) runs the destination-owned loop.  Column sums of
// (I, J) land at colpart[256 J (J-1) / 2 + i]; k_finalize_f2f_sym adds them in
// a fixed order (deterministic results).
template <bool ATT, bool GATE, bool REG>
__device__ __forceinline__ void sym_pair(const SumArgs &a, const float4 A, const float4 B, const Dst &d, float &Tr,
                                         float &Ti, bool &ok)
{
    const float vx = __fsub_rn(d.px, A.x), vy = __fsub_rn(d.py, A.y), vz = __fsub_rn(d.pz, A.z);
    // |v|^2 with fused multiply-adds; r from one Newton step on rsqrt (within an
    // ulp or two of the reference's FP32 r; the regularisation branch below
    // recomputes the reference's r exactly where it decides)
    const float r2 = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
    const float rinv = rsqrtf(r2);
    const float r0 = r2 * rinv;
    const float r = fmaf(fmaf(-r0, r0, r2), 0.5f * rinv, r0);
    const float th = __fmul_rn(r, a.k2hi);
    const float tl = fmaf(r, a.k2lo, fmaf(r, a.k2hi, -th));
    const float frac = (th - rintf(th)) + tl;
    float sn, cs;
    __sincosf(frac * kTwoPi, &sn, &cs);
    const float d1 = vx * B.x + vy * B.y + vz * B.z;    // r cos_scat (source side)
    const float d2 = vx * d.nx + vy * d.ny + vz * d.nz;  // -r cos_inc (destination side)
    ok = true;
    if (GATE)
        ok = gate_from(d1 * rinv, vx, vy, vz, 1.0f, B.x, B.y, B.z) &&
             gate_from(-d2 * rinv, vx, vy, vz, -1.0f, d.nx, d.ny, d.nz);
    // T = cos_scat cos_inc G,  G = -e^{ikr}/(4 pi) (ik/r) + 1/r^2
    const float rinv2 = rinv * rinv;
    const float u = (d1 * d2) * (-rinv2);  // cos_scat cos_inc
    if (ATT) {
        const float amp = rinv * kInv4Pi * __expf(-a.ka * r);
        Tr = u * fmaf(amp, fmaf(a.ka, cs, a.kr * sn), rinv2);
        Ti = u * (amp * fmaf(a.ka, sn, -a.kr * cs));
    } else {
        const float ua = (u * rinv) * a.kr4pi;
        Tr = fmaf(ua, sn, u * rinv2);
        Ti = -ua * cs;
    }
    if (REG) {
        // regularised G below r_min = delta_src (OptiX.cu:340-346), decided with
        // the reference's r where it is close to the threshold
        float rr = r;
        if (fabsf(r - a.rmin) <= a.rmin * 1e-6f) rr = __fsqrt_rn(dot_rn(vx, vy, vz, vx, vy, vz));
        if (rr < a.rmin) {
            Tr = u * (-a.ka * kInv4Pi);
            Ti = u * (a.kr * kInv4Pi);
        }
    }
}


// minimum distance between two axis-aligned boxes
__device__ __forceinline__ float box_gap(const float *lo1, const float *hi1, const float *lo2, const float *hi2)
{
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float g = fmaxf(0.0f, fmaxf(lo1[k] - hi2[k], lo2[k] - hi1[k]));
        s = fmaf(g, g, s);
    }
    return sqrtf(s);
}

// Shared-memory transpose of one warp's column terms, 16 sources at a time:
// row = lane (destination), column = source; pitch 17 keeps the row-wise
// writes and the column-wise reads free of bank conflicts.
constexpr int kTrPitch = 17;
constexpr size_t kSymDynSmem = sizeof(float2) * (kTile / 32) * 32 * kTrPitch;

// one 32-source word of an off-diagonal block: row terms into the thread's
// destination, column terms summed over the warp into colw[word].  FULL:
// every pair of the word interacts (no per-pair mask or gate).
template <bool ATT, bool GATE, bool REG, bool FULL>
__device__ __forceinline__ void sym_word(const SumArgs &a, const float4 *sA, const float4 *sB, int w, uint32_t m,
                                         const Dst &d, float wjr, float wji, float &fr, float &fi, float2 *colw,
                                         float2 *tr, int lane)
{
#pragma unroll
    for (int h = 0; h < 2; ++h) {
#pragma unroll 4
        for (int b = 0; b < 16; ++b) {
            const int q = w * 32 + h * 16 + b;
            const float4 A = sA[q], B = sB[q];
            float Tr, Ti;
            bool ok;
            sym_pair<ATT, GATE, REG>(a, A, B, d, Tr, Ti, ok);
            if (!FULL) {
                const bool on = ((m >> (h * 16 + b)) & 1u) && ok;
                Tr = on ? Tr : 0.0f;
                Ti = on ? Ti : 0.0f;
            }
            fr = fmaf(Tr, A.w, fmaf(-Ti, B.w, fr));  // forward term into this destination
            fi = fmaf(Tr, B.w, fmaf(Ti, A.w, fi));
            tr[lane * kTrPitch + b] = make_float2(Tr * wjr - Ti * wji, Tr * wji + Ti * wjr);  // reciprocal term
        }
        __syncwarp();
        // lane l sums column (l & 15) over rows 16 (l >> 4) .. +15; the two halves combine
        const int c = lane & 15, r0 = (lane >> 4) * 16;
        float sr = 0.0f, si = 0.0f;
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const float2 v = tr[(r0 + r) * kTrPitch + c];
            sr += v.x;
            si += v.y;
        }
        sr += __shfl_xor_sync(0xffffffffu, sr, 16);
        si += __shfl_xor_sync(0xffffffffu, si, 16);
        if (lane < 16) colw[w * 32 + h * 16 + lane] = make_float2(sr, si);
        __syncwarp();
    }
}

template <bool ATT, bool GATE, bool REG>
__device__ __forceinline__ void diag_word(const SumArgs &a, const float4 *sA, const float4 *sB, int w, uint32_t m,
                                          const Dst &d, float &fr, float &fi)
{
#pragma unroll 4
    for (int b = 0; b < 32; ++b) {
        const float4 A = sA[w * 32 + b], B = sB[w * 32 + b];
        float Tr, Ti;
        bool ok;
        sym_pair<ATT, GATE, REG>(a, A, B, d, Tr, Ti, ok);
        const bool on = ((m >> b) & 1u) && ok;
        Tr = on ? Tr : 0.0f;
        Ti = on ? Ti : 0.0f;
        fr = fmaf(Tr, A.w, fmaf(-Ti, B.w, fr));
        fi = fmaf(Tr, B.w, fmaf(Ti, A.w, fi));
    }
}

// Work list of the symmetric bounce sum: the non-empty blocks of destination
// row J (source tiles t <= J whose flag is not NONE) in tile order,
// blist[J * ntiles + k], and their count.
__global__ void __launch_bounds__(kTile) k_sym_rows(const uint8_t *flags, int ntiles, int nb, int *blist,
                                                   int *rowcnt)
{
    __shared__ int sWarp[kTile / 32];
    const int J = blockIdx.x, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tmax = min(J, ntiles - 1);
    int base = 0;
    for (int t0 = 0; t0 <= tmax; t0 += kTile) {
        const int t = t0 + tid;
        const bool on = t <= tmax && flags[(long long)t * nb + J] != kFlagNone;
        const unsigned bal = __ballot_sync(0xffffffffu, on);
        if (lane == 0) sWarp[warp] = __popc(bal);
        __syncthreads();
        int woff = 0, tot = 0;
#pragma unroll
        for (int w = 0; w < kTile / 32; ++w) {
            woff += w < warp ? sWarp[w] : 0;
            tot += sWarp[w];
        }
        if (on) blist[(long long)J * ntiles + base + woff + __popc(bal & ((1u << lane) - 1u))] = t;
        base += tot;
        __syncthreads();
    }
    if (tid == 0) rowcnt[J] = base;
}

// Chunks of at most `per` blocks of one row: chunks[c] = (J, k0, k1),
// chunk_off[J] .. chunk_off[J + 1] the chunks of row J, *nchunks the total.
// One CTA of 1024 threads scans the rows in segments.
__global__ void __launch_bounds__(1024) k_sym_chunks(const int *rowcnt, int nb, int per, int *chunk_off, int4 *chunks,
                                                     int *nchunks)
{
    __shared__ int sW[32];
    __shared__ int sCarry;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) sCarry = 0;
    __syncthreads();
    for (int J0 = 0; J0 < nb; J0 += 1024) {
        const int J = J0 + tid;
        const int cnt = J < nb ? rowcnt[J] : 0;
        const int n = (cnt + per - 1) / per;
        int v = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        if (lane == 31) sW[warp] = v;
        __syncthreads();
        if (warp == 0) {
            int x = sW[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            sW[lane] = x;
        }
        __syncthreads();
        const int excl = sCarry + (warp > 0 ? sW[warp - 1] : 0) + v - n;
        if (J < nb) {
            chunk_off[J] = excl;
            for (int k = 0; k < n; ++k) chunks[excl + k] = make_int4(J, k * per, min(cnt, (k + 1) * per), 0);
        }
        __syncthreads();
        if (tid == 1023) sCarry = excl + n;
        __syncthreads();
    }
    if (tid == 0) {
        chunk_off[nb] = sCarry;
        *nchunks = sCarry;
    }
}

// Persistent CTAs take the chunks from a counter in chunk order, so chunks of
// uneven cost (diagonal blocks, the few dense blocks left by compression)
// balance over the CTAs; every chunk writes its own output locations, so the
// results do not depend on which CTA took it.  Per chunk: the row terms of
// its blocks into rowpart[chunk] (FP64), the column terms of block (t, J),
// t < J, into colpart[256 J (J-1) / 2 + i].
template <bool ATT>
__global__ void __launch_bounds__(kTile, 3) k_sum_f2f_sym(SumArgs a, SymWork wl, double2 *colpart, double2 *rowpart)
{
    extern __shared__ float2 sTr[];  // kSymDynSmem bytes: per-warp transpose tiles
    __shared__ float4 sA[kTile];
    __shared__ float4 sB[kTile];
    __shared__ float2 sCol[kTile / 32][kTile];
    __shared__ float sTb[6];  // source tile box
    __shared__ int sDb[6];    // destination block box
    __shared__ int sCh;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nch = *wl.nchunks;
    for (;;) {
        // sCh was last read before the previous chunk's barriers
        if (tid == 0) sCh = atomicAdd(wl.next, 1);
        __syncthreads();
        const int ch = sCh;
        if (ch >= nch) break;  // CTA-uniform
        const int4 cw = wl.chunks[ch];
        const int J = cw.x;
        const int j = J * kTile + tid;
        const bool live = j < a.ndst;
        Dst d{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        int limit = a.nsrc;
        float wjr = 0.0f, wji = 0.0f;  // this destination's own source weight (the reciprocal input)
        float dlo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, dhi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        if (live) {
            const float4 p = a.dst_pos[j];
            d.px = p.x; d.py = p.y; d.pz = p.z;
            const float4 n = a.dst_facet_n[a.dst_facet[j]];
            d.nx = n.x; d.ny = n.y; d.nz = n.z;
            limit = a.dst_limit[j];
            wjr = a.srcA[j].w;
            wji = a.srcB[j].w;
            dlo[0] = dhi[0] = p.x; dlo[1] = dhi[1] = p.y; dlo[2] = dhi[2] = p.z;
        }
        __syncthreads();  // the previous chunk is done with the shared arrays
        if (tid < 6) sDb[tid] = tid < 3 ? f2o(3.0e38f) : f2o(-3.0e38f);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 3; ++k)
            for (int off = 16; off > 0; off >>= 1) {
                dlo[k] = fminf(dlo[k], __shfl_xor_sync(0xffffffffu, dlo[k], off));
                dhi[k] = fmaxf(dhi[k], __shfl_xor_sync(0xffffffffu, dhi[k], off));
            }
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                atomicMin(&sDb[k], f2o(dlo[k]));
                atomicMax(&sDb[3 + k], f2o(dhi[k]));
            }
        __syncthreads();
        float blo[3], bhi[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            blo[k] = o2f(sDb[k]);
            bhi[k] = o2f(sDb[3 + k]);
        }
        const long long cbase = (long long)kTile * J * (J - 1) / 2;  // this J's column region
        double accr = 0.0, acci = 0.0;
        for (int kk = cw.y; kk < cw.z; ++kk) {
            const int t = wl.blist[(long long)J * wl.ntiles + kk];
            const uint8_t fl = a.mask.flags[(long long)t * a.mask.ndstblocks + J];
            const int i0 = t * kTile;
            __syncthreads();
            {
                const int i = i0 + tid;
                const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                const float4 A = i < a.nsrc ? a.srcA[i] : z;
                sA[tid] = A;
                sB[tid] = i < a.nsrc ? a.srcB[i] : z;
                float lo[3] = {A.x, A.y, A.z}, hi[3] = {A.x, A.y, A.z};
                if (i >= a.nsrc) {
                    lo[0] = lo[1] = lo[2] = 3.0e38f;
                    hi[0] = hi[1] = hi[2] = -3.0e38f;
                }
#pragma unroll
                for (int k = 0; k < 3; ++k)
                    for (int off = 16; off > 0; off >>= 1) {
                        lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], off));
                        hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], off));
                    }
                if (lane == 0) {
#pragma unroll
                    for (int k = 0; k < 3; ++k) sCol[warp][k] = make_float2(lo[k], hi[k]);
                }
            }
            __syncthreads();
            if (tid == 0) {
                float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
                for (int q = 0; q < kTile / 32; ++q)
                    for (int k = 0; k < 3; ++k) {
                        lo[k] = fminf(lo[k], sCol[q][k].x);
                        hi[k] = fmaxf(hi[k], sCol[q][k].y);
                    }
                for (int k = 0; k < 3; ++k) {
                    sTb[k] = lo[k];
                    sTb[3 + k] = hi[k];
                }
            }
            __syncthreads();
            // no pair of this block can be closer than r_min: skip the regularisation code
            const float tlo[3] = {sTb[0], sTb[1], sTb[2]}, thi[3] = {sTb[3], sTb[4], sTb[5]};
            const bool reg = box_gap(tlo, thi, blo, bhi) <= a.rmin * 1.001f;
            const int ntile = min(kTile, a.nsrc - i0);
            const int nw = (ntile + 31) >> 5;
            float fr = 0.0f, fi = 0.0f;
            const bool gate = fl == kFlagClear;
            for (int w = 0; w < nw; ++w) {
                uint32_t m;
                if (fl == kFlagBits) {
                    m = live ? a.mask.bits[(long long)(t * kWordsPerTile + w) * a.mask.pitch + j] : 0u;
                } else {
                    const int nb = ntile - w * 32;
                    m = !live ? 0u : (nb >= 32 ? 0xffffffffu : ((1u << nb) - 1u));
                }
                if (t == J) {
                    // diagonal tile: destination-owned, with the zero-input source limit
                    const int keep = limit - (i0 + w * 32);
                    m &= keep >= 32 ? 0xffffffffu : (keep <= 0 ? 0u : ((1u << keep) - 1u));
                    if (!__any_sync(0xffffffffu, m != 0u)) continue;
                    if (gate) diag_word<ATT, true, true>(a, sA, sB, w, m, d, fr, fi);
                    else diag_word<ATT, false, true>(a, sA, sB, w, m, d, fr, fi);
                } else {
                    if (!__any_sync(0xffffffffu, m != 0u)) {
                        sCol[warp][w * 32 + lane] = make_float2(0.0f, 0.0f);
                        continue;
                    }
                    float2 *colw = &sCol[warp][0];
                    float2 *trw = sTr + warp * 32 * kTrPitch;
                    const bool full = !gate && __all_sync(0xffffffffu, m == 0xffffffffu);
                    if (gate) {
                        if (reg) sym_word<ATT, true, true, false>(a, sA, sB, w, m, d, wjr, wji, fr, fi, colw, trw, lane);
                        else sym_word<ATT, true, false, false>(a, sA, sB, w, m, d, wjr, wji, fr, fi, colw, trw, lane);
                    } else if (full) {
                        if (reg) sym_word<ATT, false, true, true>(a, sA, sB, w, m, d, wjr, wji, fr, fi, colw, trw, lane);
                        else sym_word<ATT, false, false, true>(a, sA, sB, w, m, d, wjr, wji, fr, fi, colw, trw, lane);
                    } else {
                        if (reg) sym_word<ATT, false, true, false>(a, sA, sB, w, m, d, wjr, wji, fr, fi, colw, trw, lane);
                        else sym_word<ATT, false, false, false>(a, sA, sB, w, m, d, wjr, wji, fr, fi, colw, trw, lane);
                    }
                }
            }
            if (t < J) {
                for (int w = nw; w < kWordsPerTile; ++w) sCol[warp][w * 32 + lane] = make_float2(0.0f, 0.0f);
                __syncthreads();
                double sr = 0.0, si = 0.0;
#pragma unroll
                for (int k = 0; k < kTile / 32; ++k) {
                    const float2 v = sCol[k][tid];
                    sr += (double)v.x;
                    si += (double)v.y;
                }
                colpart[cbase + i0 + tid] = make_double2(sr, si);
            }
            accr += (double)fr;
            acci += (double)fi;
        }
        if (live) rowpart[(long long)ch * kTile + tid] = make_double2(accr, acci);
    }
}

// P_out[cell] = rows + (P_in[i] != 0 ? columns : 0); P[cell] += P_out[cell].
// Rows: the chunks of the fragment's row in chunk order; columns: every
// non-empty block (I, J > I) of its tile I in J order (deterministic).
// yrow / ycol: compressed-block rows and columns, may be null.
__global__ void k_finalize_f2f_sym(const double2 *rowpart, const int *chunk_off, int ndst, const double2 *colpart,
                                   const uint8_t *flags, int ntiles, const int *cell, const double2 *Pin,
                                   double2 *Pout, double2 *P, const double2 *yrow, const double2 *ycol)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ndst) return;
    const int I = q / kTile;
    double sr = 0.0, si = 0.0;
    for (int c = chunk_off[I]; c < chunk_off[I + 1]; ++c) {
        const double2 v = rowpart[(long long)c * kTile + (q & (kTile - 1))];
        sr += v.x;
        si += v.y;
    }
    const int c = cell[q];
    const double2 pin = Pin[c];
    if (yrow) {
        sr += yrow[q].x;
        si += yrow[q].y;
    }
    if (pin.x != 0.0 || pin.y != 0.0) {
        double cr = 0.0, ci = 0.0;
        // the tile's flag row, 16 flags at a time where aligned (rows of a
        // compressed bounce are mostly NONE); columns added in J order
        const uint8_t *frow = flags + (long long)I * ntiles;
        for (int J = I + 1; J < ntiles;) {
            if ((reinterpret_cast<uintptr_t>(frow + J) & 15u) == 0 && J + 16 <= ntiles) {
                const uint4 v = *reinterpret_cast<const uint4 *>(frow + J);
                if ((v.x | v.y | v.z | v.w) == 0u) {
                    J += 16;
                    continue;
                }
            }
            if (frow[J] != kFlagNone) {
                const double2 v = colpart[(long long)kTile * J * (J - 1) / 2 + q];
                cr += v.x;
                ci += v.y;
            }
            ++J;
        }
        if (ycol) {
            cr += ycol[q].x;
            ci += ycol[q].y;
        }
        sr += cr;
        si += ci;
    }
    Pout[c] = make_double2(sr, si);
    double2 o = P[c];
    o.x += sr;
    o.y += si;
    P[c] = o;
}

// ---------------------------------------------------------------- low-rank blocks
// Compressed FACET_SELF blocks.  For a block of source tile I and destination
// tile J (I < J) the interaction matrix T_ji = m_ji cos_scat cos_inc G(r_ji)
// (weights excluded; m_ji = 1 for class ALL, the inline cosine gates for
// CLEAR, the stored mask bit for BITS) is approximated by U V^T, U: 256 x k
// over the rows j of J, V: 256 x k over the columns i of I, by adaptive cross
// approximation with partial pivoting: each step takes the residual row at a
// pivot row, its largest entry as pivot column, the residual column there,
// and stops when |u_k| |v_k| falls below tol times the running Frobenius
// estimate.  Residual rows that vanish (rows the mask zeroes) are skipped.
// The forward terms are then U (V^T w_I) into J and the reciprocal ones
// V (U^T w_J) into I.  Factors of block b start at column off[b] (in 256-entry
// columns) of the U and V arrays; cap[b] columns are reserved.

__device__ __forceinline__ float block_sum(float v, float *sv)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    __syncthreads();
    if (lane == 0) sv[warp] = v;
    __syncthreads();
    float t = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sv[w];
    return t;
}




constexpr int kAcaMaxZeroRows = 48;
constexpr int kLrMaxRank = 64;
constexpr int kAcaWarps = kTile / 32;

// Block-wide argmax (ARG) of v >= 0 over the threads with valid set and
// block-wide sums (SUMS) of s0 and s1; every thread receives the results
// (v = -1 when no thread was valid).  The argmax key is the value's float
// bits with the low 8 mantissa bits replaced by 255 - idx (idx < 256): the
// largest value to 2^-15 relative wins, ties go to the lowest index.  A warp
// reduction (redux.sync) leaves one key per warp in slot[warp]; after the
// barrier every thread takes the maximum of the eight slots.  The sums go
// through one slot per warp, added in warp order (deterministic).  One
// barrier.  A slot array is rewritten only after every thread has passed a
// later barrier, so callers give each reduction site its own slots.
template <bool ARG, bool SUMS>
__device__ __forceinline__ void cta_reduce(float &v, int &idx, bool valid, float &s0, float &s1, unsigned *slot,
                                           float2 *sums)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned k = 0u;
    if (ARG) {
        if (valid) k = ((__float_as_uint(fmaxf(v, 0.0f)) + 0x100u) & 0xFFFFFF00u) | (255u - (unsigned)idx);
        k = __reduce_max_sync(0xffffffffu, k);
    }
    if (SUMS) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        }
    }
    if (lane == 0) {
        if (ARG) slot[warp] = k;
        if (SUMS) sums[warp] = make_float2(s0, s1);
    }
    __syncthreads();
    if (ARG) {
        static_assert(kAcaWarps == 8, "two 16-byte slot reads");
        const uint4 a = reinterpret_cast<const uint4 *>(slot)[0], b = reinterpret_cast<const uint4 *>(slot)[1];
        const unsigned w = max(max(max(a.x, a.y), max(a.z, a.w)), max(max(b.x, b.y), max(b.z, b.w)));
        v = w ? __uint_as_float((w & 0xFFFFFF00u) - 0x100u) : -1.0f;
        idx = (int)(255u - (w & 0xFFu));
    }
    if (SUMS) {
        float t0 = 0.0f, t1 = 0.0f;
#pragma unroll
        for (int q = 0; q < kAcaWarps; ++q) {
            const float2 o = sums[q];
            t0 += o.x;
            t1 += o.y;
        }
        s0 = t0;
        s1 = t1;
    }
}

// x - u v (complex)
__device__ __forceinline__ float2 csub_mul(float2 x, float2 u, float2 v)
{
    x.x = fmaf(u.y, v.y, fmaf(-u.x, v.x, x.x));
    x.y = fmaf(-u.y, v.x, fmaf(-u.x, v.y, x.y));
    return x;
}

// One CTA per block, thread t owns row t and column t of the block (its own
// fragment data stays in registers).  The factor columns of the first RS
// ranks live in shared memory (sU[m][j], sV[m][i]), later ones only in the
// U and V arrays in global memory, which the low-rank apply reads.  Each
// rank step has two barriers:
//   1. every thread stores its residual-row entry (r, t) in sRow and the
//      block argmax picks the pivot column c; everyone then reads the pivot
//      value sRow[c];
//   2. after the residual column c, the argmax over unused rows picks the
//      next pivot row and the same barrier carries the norms.
// Factor entries written before a barrier are read by other threads only
// after it: the pivot row's U entries (step 1 of the next rank) and the
// pivot column's V entries (the column residual) were all written at
// earlier ranks.
template <bool ATT, int RS, int MINB>
__global__ void __launch_bounds__(kTile, MINB) k_aca(SumArgs a, const int2 *blocks, const uint8_t *cls,
                                                     const int *cap, const long long *off, int nblocks, float tol,
                                                     float limit, float2 *U, float2 *V, int *rank, float *fro,
                                                     float *err, const int *list)
{
    extern __shared__ float2 aca_smem[];  // sU[RS][kTile], then sV[RS][kTile]
    float2 *sU = aca_smem, *sV = aca_smem + RS * kTile;
    __shared__ float2 sRow[kTile];
    __shared__ float4 sFrag[4][kTile];  // position and normal of the columns' (I) and rows' (J) fragments
    __shared__ __align__(16) unsigned slotA[kAcaWarps], slotB[kAcaWarps], slotZ[kAcaWarps];
    __shared__ float2 sumB[kAcaWarps];
    const int t = threadIdx.x;
    if ((int)blockIdx.x >= nblocks) return;  // CTA-uniform
    const int b = list ? list[blockIdx.x] : (int)blockIdx.x;  // kept block
    const int I = blocks[b].x, J = blocks[b].y, bc = cls[b], K = min(cap[b], kLrRankLimit);
    if (K <= 0) return;  // CTA-uniform: an interpolated block (the interpolation kernel writes its results)
    const int ni = min(kTile, a.nsrc - I * kTile), nj = min(kTile, a.nsrc - J * kTile);
    const float4 *PI = a.srcA + I * kTile, *NI = a.srcB + I * kTile, *PJ = a.srcA + J * kTile, *NJ = a.srcB + J * kTile;
    float2 *Ub = U + off[b] * kTile, *Vb = V + off[b] * kTile;
    // mask word w of destination row j: bw[w * pitch + j]
    const uint32_t *bw = a.mask.bits + (long long)I * kWordsPerTile * a.mask.pitch + (long long)J * kTile;
    const long long pitch = a.mask.pitch;
    const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float2 z2 = make_float2(0.0f, 0.0f);
    const bool coli = t < ni, rowj = t < nj;
    const float4 pi = coli ? __ldg(PI + t) : z4, qi = coli ? __ldg(NI + t) : z4;
    const float4 pj = rowj ? __ldg(PJ + t) : z4, qj = rowj ? __ldg(NJ + t) : z4;
    // both tiles' fragment data in shared memory: the pivots' data are read from here
    sFrag[0][t] = pi;
    sFrag[1][t] = qi;
    sFrag[2][t] = pj;
    sFrag[3][t] = qj;
    __syncthreads();
    bool used = !rowj;  // row t taken (or absent)
    int r = 0, k = 0, zero_rows = 0;
    float norm2 = 0.0f;
    while (k < K) {
        const int ks = min(k, RS);
        // ---- residual row r, entry (r, t)
        float2 val = z2;
        if (coli) {
            const bool bit = bc == kFlagBits ? ((bw[(long long)(t >> 5) * pitch + r] >> (t & 31)) & 1u) : true;
            val = lr_entry<ATT>(a, bc, bit, pi, qi, sFrag[2][r], sFrag[3][r]);
            for (int m = 0; m < ks; ++m) val = csub_mul(val, sU[m * kTile + r], sV[m * kTile + t]);
            for (int m = RS; m < k; ++m) val = csub_mul(val, Ub[m * kTile + r], Vb[m * kTile + t]);
        }
        sRow[t] = val;
        float best = val.x * val.x + val.y * val.y, d0 = 0.0f, d1 = 0.0f;
        int c = t;
        cta_reduce<true, false>(best, c, coli, d0, d1, slotA, nullptr);
        if (!(best > 1e-30f)) {
            // the residual row vanished: take the lowest unused row instead
            if (t == r) used = true;
            if (++zero_rows > kAcaMaxZeroRows) break;
            float f = 1.0f;
            int nr = t;
            cta_reduce<true, false>(f, nr, !used, d0, d1, slotZ, nullptr);
            if (f < 0.0f) break;
            r = nr;
            continue;
        }
        const float2 pv = sRow[c];
        const float inv = __frcp_rn(pv.x * pv.x + pv.y * pv.y);
        const float2 vv = coli ? make_float2((val.x * pv.x + val.y * pv.y) * inv, (val.y * pv.x - val.x * pv.y) * inv)
                               : z2;
        Vb[k * kTile + t] = vv;
        if (k < RS) sV[k * kTile + t] = vv;
        // ---- residual column c, entry (t, c)
        float2 uu = z2;
        if (rowj) {
            const bool bit = bc == kFlagBits ? ((bw[(long long)(c >> 5) * pitch + t] >> (c & 31)) & 1u) : true;
            uu = lr_entry<ATT>(a, bc, bit, sFrag[0][c], sFrag[1][c], pj, qj);
            for (int m = 0; m < ks; ++m) uu = csub_mul(uu, sU[m * kTile + t], sV[m * kTile + c]);
            for (int m = RS; m < k; ++m) uu = csub_mul(uu, Ub[m * kTile + t], Vb[m * kTile + c]);
        }
        Ub[k * kTile + t] = uu;
        if (k < RS) sU[k * kTile + t] = uu;
        if (t == r) used = true;
        // ---- norms and the next pivot row: the largest residual-column entry among unused rows
        float nu2 = uu.x * uu.x + uu.y * uu.y, nv2 = vv.x * vv.x + vv.y * vv.y;
        float bn = nu2;
        int nr = t;
        cta_reduce<true, true>(bn, nr, !used, nu2, nv2, slotB, sumB);
        norm2 += nu2 * nv2;
        ++k;
        if (nu2 * nv2 <= tol * tol * norm2) break;
        if (bn < 0.0f) break;  // every row taken
        r = nr;
    }
    // ---- the exact entries judge the approximation: every row once at a
    // hashed column, every column once at a hashed row; relative RMS error
    // against the sampled entries' RMS
    float e2 = 0.0f, x2 = 0.0f;
    const bool converged = k > 0 && k < K;
    __syncthreads();  // every factor entry is visible; the sum slots are free
    if (converged) {
        const int ks = min(k, RS);
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
            const int s = t + kTile * h2;  // sample 0..511
            unsigned h = (unsigned)b * 2654435761u + (unsigned)s * 40503u + 12345u;
            h ^= h >> 13;
            h *= 0x5bd1e995u;
            h ^= h >> 15;
            const int jj = h2 == 0 ? t : (int)(h & 255u), ii = h2 == 0 ? (int)(h & 255u) : t;
            if (ii < ni && jj < nj) {
                const bool bit = bc == kFlagBits ? ((bw[(long long)(ii >> 5) * pitch + jj] >> (ii & 31)) & 1u) : true;
                const float2 ex = lr_entry<ATT>(a, bc, bit, h2 == 0 ? sFrag[0][ii] : pi, h2 == 0 ? sFrag[1][ii] : qi,
                                                h2 == 0 ? pj : sFrag[2][jj], h2 == 0 ? qj : sFrag[3][jj]);
                float2 ap = z2;  // minus the approximation
                for (int m = 0; m < ks; ++m) ap = csub_mul(ap, sU[m * kTile + jj], sV[m * kTile + ii]);
                for (int m = RS; m < k; ++m) ap = csub_mul(ap, Ub[m * kTile + jj], Vb[m * kTile + ii]);
                e2 += (ex.x + ap.x) * (ex.x + ap.x) + (ex.y + ap.y) * (ex.y + ap.y);
                x2 += ex.x * ex.x + ex.y * ex.y;
            }
        }
    }
    {
        float f = 0.0f;
        int fi = 0;
        cta_reduce<false, true>(f, fi, false, e2, x2, nullptr, sumB);
    }
    if (t == 0) {
        const float rel = x2 > 0.0f ? sqrtf(e2 / x2) : (e2 > 0.0f ? 1.0f : 0.0f);
        rank[b] = converged && rel <= limit ? k : -1;
        fro[b] = sqrtf(norm2);
        err[b] = converged ? rel : -1.0f;
    }
}

// Low-rank apply of one accepted block of rank k, by the whole CTA of NT
// threads: tv = V^T w_I and su = U^T w_J (warp w takes the ranks m = w (mod
// NT / 32), each lane 8 rows, one warp reduction per rank; one barrier),
// then the block's forward terms U tv (rows of J) and reciprocal terms V su
// (columns of I) into its output slots brow_b, bcol_b (FP32).  The weights w
// are the packed inputs (srcA.w, srcB.w).  sW holds kTile float4, sTv and
// sSu kLrMaxRank float2.  Starts with a barrier (the caller may reuse the
// shared arrays).
// LDG: the factors were written by an earlier kernel, so the projections may
// read them through the read-only path (the fused caller wrote them itself).
template <int NT = kTile, bool LDG = false>
__device__ __forceinline__ void lr_block_apply(const SumArgs &a, int I, int J, const float2 *U0, const float2 *V0,
                                               int k, float2 *brow_b, float2 *bcol_b, float4 *sW, float2 *sTv,
                                               float2 *sSu)
{
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    __syncthreads();
#pragma unroll
    for (int h = 0; h < kTile / NT; ++h) {
        const int tt = t + h * NT, i = I * kTile + tt, j = J * kTile + tt;
        sW[tt] = make_float4(i < a.nsrc ? a.srcA[i].w : 0.0f, i < a.nsrc ? a.srcB[i].w : 0.0f,
                             j < a.nsrc ? a.srcA[j].w : 0.0f, j < a.nsrc ? a.srcB[j].w : 0.0f);
    }
    __syncthreads();
    for (int m = warp; m < k; m += NT / 32) {
        float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
        for (int r = 0; r < kTile / 32; ++r) {
            const int tt = lane + 32 * r;
            const float2 v = LDG ? __ldg(V0 + (size_t)m * kTile + tt) : V0[(size_t)m * kTile + tt];
            const float2 u = LDG ? __ldg(U0 + (size_t)m * kTile + tt) : U0[(size_t)m * kTile + tt];
            const float4 w = sW[tt];
            p.x = fmaf(v.x, w.x, fmaf(-v.y, w.y, p.x));
            p.y = fmaf(v.x, w.y, fmaf(v.y, w.x, p.y));
            p.z = fmaf(u.x, w.z, fmaf(-u.y, w.w, p.z));
            p.w = fmaf(u.x, w.w, fmaf(u.y, w.z, p.w));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            p.x += __shfl_xor_sync(0xffffffffu, p.x, o);
            p.y += __shfl_xor_sync(0xffffffffu, p.y, o);
            p.z += __shfl_xor_sync(0xffffffffu, p.z, o);
            p.w += __shfl_xor_sync(0xffffffffu, p.w, o);
        }
        if (lane == 0) {
            sTv[m] = make_float2(p.x, p.y);
            sSu[m] = make_float2(p.z, p.w);
        }
    }
    __syncthreads();
#pragma unroll
    for (int h = 0; h < kTile / NT; ++h) {
        const int tt = t + h * NT;
        const float2 *Ub = U0 + tt, *Vb = V0 + tt;
        float rr = 0.0f, ri = 0.0f, cr = 0.0f, ci = 0.0f;
        // the factors come back from L2: several ranks' loads in flight at once
#pragma unroll 4
        for (int m = 0; m < k; ++m) {
            const float2 u = Ub[m * kTile], v = Vb[m * kTile], c = sTv[m], e = sSu[m];
            rr += u.x * c.x - u.y * c.y;
            ri += u.x * c.y + u.y * c.x;
            cr += v.x * e.x - v.y * e.y;
            ci += v.x * e.y + v.y * e.x;
        }
        brow_b[tt] = make_float2(rr, ri);
        bcol_b[tt] = make_float2(cr, ci);
    }
}

// ---------------------------------------------------------------- block argmax helpers
// 32-bit argmax key of v >= 0 at index idx < 256 (0: not a candidate): the
// float bits with the low byte replaced by 255 - idx, as in cta_reduce
__device__ __forceinline__ unsigned argmax_key(float v, int idx, bool valid)
{
    return valid ? ((__float_as_uint(fmaxf(v, 0.0f)) + 0x100u) & 0xFFFFFF00u) | (255u - (unsigned)idx) : 0u;
}

__device__ __forceinline__ unsigned max8(const unsigned *slot)
{
    const uint4 a = reinterpret_cast<const uint4 *>(slot)[0], b = reinterpret_cast<const uint4 *>(slot)[1];
    return max(max(max(a.x, a.y), max(a.z, a.w)), max(max(b.x, b.y), max(b.z, b.w)));
}

__device__ __forceinline__ float key_value(unsigned w) { return w ? __uint_as_float((w & 0xFFFFFF00u) - 0x100u) : -1.0f; }

// mask bit of pair (row j of tile J, column i of tile I) of a BITS block
__device__ __forceinline__ bool block_bit(const uint32_t *bw, long long pitch, int j, int i)
{
    return (bw[(long long)(i >> 5) * pitch + j] >> (i & 31)) & 1u;
}

// ---------------------------------------------------------------- two entries per thread
// The classic cross approximation (k_aca's pivot order, stopping rule and
// judge) by a CTA of 128 threads for the 256 x 256 block: thread t owns rows
// t and t + 128 and columns t and t + 128.  Every per-step cost that does not
// depend on the number of entries -- the block argmax, the pivot value and
// its reciprocal, loop and branch work, the earlier ranks' factor entry at
// the pivot, which serves both of a thread's entries -- is paid once per two
// entries, and the two entries give each thread two independent chains.
// The reductions run over four warps.  Per-rank norms are summed in another
// order than k_aca's (so a stopping decision at the threshold can differ by
// rounding); the factors are otherwise those of k_aca.
constexpr int kAca2Threads = 128;
constexpr int kAca2Warps = kAca2Threads / 32;

// Block-wide argmax over two candidates per thread and block-wide sums of s0
// and s1 over four warps (one barrier; see cta_reduce).
template <bool ARG, bool SUMS>
__device__ __forceinline__ void cta_reduce2(float va, int ia, bool oka, float vb, int ib, bool okb, float &best,
                                            int &idx, float &s0, float &s1, unsigned *slot, float2 *sums)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned k = 0u;
    if (ARG) k = __reduce_max_sync(0xffffffffu, max(argmax_key(va, ia, oka), argmax_key(vb, ib, okb)));
    if (SUMS) {
        // two sums with five shuffles: lanes of the upper half keep s1, the lower s0
        const bool hi = lane & 16;
        float w = (hi ? s1 : s0) + __shfl_xor_sync(0xffffffffu, hi ? s0 : s1, 16);
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
        s0 = __shfl_sync(0xffffffffu, w, 0);
        s1 = __shfl_sync(0xffffffffu, w, 16);
    }
    if (lane == 0) {
        if (ARG) slot[warp] = k;
        if (SUMS) sums[warp] = make_float2(s0, s1);
    }
    __syncthreads();
    if (ARG) {
        static_assert(kAca2Warps == 4, "one 16-byte slot read");
        const uint4 a = reinterpret_cast<const uint4 *>(slot)[0];
        const unsigned w = max(max(a.x, a.y), max(a.z, a.w));
        best = key_value(w);
        idx = (int)(255u - (w & 0xFFu));
    }
    if (SUMS) {
        const float4 p = reinterpret_cast<const float4 *>(sums)[0], q = reinterpret_cast<const float4 *>(sums)[1];
        s0 = (p.x + p.z) + (q.x + q.z);
        s1 = (p.y + p.w) + (q.y + q.w);
    }
}

// FRAG: both tiles' fragment data staged in shared memory (16 KB) for the
// pivots' and the judge's reads; without it those reads go through L1 and
// the shared memory is left to factor ranks and CTAs.
template <bool ATT, int RS, int MINB, bool FRAG = true>
__global__ void __launch_bounds__(kAca2Threads, MINB) k_aca2(SumArgs a, const int2 *blocks, const uint8_t *cls,
                                                             const int *cap, const long long *off, int nblocks,
                                                             float tol, float limit, float2 *U, float2 *V, int *rank,
                                                             float *fro, float *err, float2 *brow, float2 *bcol,
                                                             const int *list)
{
    extern __shared__ float2 aca_smem[];  // sU[RS][kTile], then sV[RS][kTile]
    float2 *sU = aca_smem, *sV = aca_smem + RS * kTile;
    __shared__ float2 sRow[kTile];
    __shared__ float4 sFrag[FRAG ? 4 : 1][FRAG ? kTile : 1];  // position and normal of the columns' (I) and rows' (J) fragments
    __shared__ __align__(16) unsigned slotA[kAca2Warps], slotB[kAca2Warps], slotZ[kAca2Warps];
    __shared__ __align__(16) float2 sumB[kAca2Warps];
    const int t = threadIdx.x;
    const int ta = t, tb = t + kAca2Threads;  // this thread's two rows / columns
    if ((int)blockIdx.x >= nblocks) return;  // CTA-uniform
    const int b = list ? list[blockIdx.x] : (int)blockIdx.x;  // kept block
    const int I = blocks[b].x, J = blocks[b].y, bc = cls[b], K = min(cap[b], kLrRankLimit);
    if (K <= 0) return;  // CTA-uniform: an interpolated block (the interpolation kernel writes its results)
    const int ni = min(kTile, a.nsrc - I * kTile), nj = min(kTile, a.nsrc - J * kTile);
    const float4 *PI = a.srcA + I * kTile, *NI = a.srcB + I * kTile, *PJ = a.srcA + J * kTile, *NJ = a.srcB + J * kTile;
    float2 *Ub = U + off[b] * kTile, *Vb = V + off[b] * kTile;
    const uint32_t *bw = a.mask.bits + (long long)I * kWordsPerTile * a.mask.pitch + (long long)J * kTile;
    const long long pitch = a.mask.pitch;
    const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float2 z2 = make_float2(0.0f, 0.0f);
    const bool colA = ta < ni, colB = tb < ni, rowA = ta < nj, rowB = tb < nj;
    const float4 piA = colA ? __ldg(PI + ta) : z4, qiA = colA ? __ldg(NI + ta) : z4;
    const float4 piB = colB ? __ldg(PI + tb) : z4, qiB = colB ? __ldg(NI + tb) : z4;
    const float4 pjA = rowA ? __ldg(PJ + ta) : z4, qjA = rowA ? __ldg(NJ + ta) : z4;
    const float4 pjB = rowB ? __ldg(PJ + tb) : z4, qjB = rowB ? __ldg(NJ + tb) : z4;
    if (FRAG) {
        sFrag[0][ta] = piA; sFrag[0][tb] = piB;
        sFrag[1][ta] = qiA; sFrag[1][tb] = qiB;
        sFrag[2][ta] = pjA; sFrag[2][tb] = pjB;
        sFrag[3][ta] = qjA; sFrag[3][tb] = qjB;
    }
    __syncthreads();
    // fragment data of column i (tile I) and row j (tile J)
    auto fragI = [&](int i, float4 &p, float4 &n) {
        if (FRAG) { p = sFrag[0][i]; n = sFrag[1][i]; } else { p = __ldg(PI + i); n = __ldg(NI + i); }
    };
    auto fragJ = [&](int j, float4 &p, float4 &n) {
        if (FRAG) { p = sFrag[2][j]; n = sFrag[3][j]; } else { p = __ldg(PJ + j); n = __ldg(NJ + j); }
    };
    bool usedA = !rowA, usedB = !rowB;  // rows taken (or absent)
    int r = 0, k = 0, zero_rows = 0;
    float norm2 = 0.0f;
    while (k < K) {
        const int ks = min(k, RS);
        // ---- residual row r, entries (r, ta) and (r, tb)
        float2 va = z2, vb = z2;
        {
            float4 pr, qr;
            fragJ(r, pr, qr);
            if (colA) va = lr_entry<ATT>(a, bc, bc == kFlagBits ? block_bit(bw, pitch, r, ta) : true, piA, qiA, pr, qr);
            if (colB) vb = lr_entry<ATT>(a, bc, bc == kFlagBits ? block_bit(bw, pitch, r, tb) : true, piB, qiB, pr, qr);
            for (int m = 0; m < ks; ++m) {
                const float2 ur = sU[m * kTile + r];
                va = csub_mul(va, ur, sV[m * kTile + ta]);
                vb = csub_mul(vb, ur, sV[m * kTile + tb]);
            }
            for (int m = RS; m < k; ++m) {
                const float2 ur = Ub[m * kTile + r];
                va = csub_mul(va, ur, Vb[m * kTile + ta]);
                vb = csub_mul(vb, ur, Vb[m * kTile + tb]);
            }
        }
        sRow[ta] = va;
        sRow[tb] = vb;
        float best, d0 = 0.0f, d1 = 0.0f;
        int c;
        cta_reduce2<true, false>(va.x * va.x + va.y * va.y, ta, colA, vb.x * vb.x + vb.y * vb.y, tb, colB, best, c,
                                 d0, d1, slotA, nullptr);
        if (!(best > 1e-30f)) {
            // the residual row vanished: take the lowest unused row instead
            if (ta == r) usedA = true;
            if (tb == r) usedB = true;
            if (++zero_rows > kAcaMaxZeroRows) break;
            float f;
            int nr;
            cta_reduce2<true, false>(1.0f, ta, !usedA, 1.0f, tb, !usedB, f, nr, d0, d1, slotZ, nullptr);
            if (f < 0.0f) break;
            r = nr;
            continue;
        }
        const float2 pv = sRow[c];
        const float inv = __frcp_rn(pv.x * pv.x + pv.y * pv.y);
        const float2 wa = colA ? make_float2((va.x * pv.x + va.y * pv.y) * inv, (va.y * pv.x - va.x * pv.y) * inv) : z2;
        const float2 wb = colB ? make_float2((vb.x * pv.x + vb.y * pv.y) * inv, (vb.y * pv.x - vb.x * pv.y) * inv) : z2;
        Vb[k * kTile + ta] = wa;
        Vb[k * kTile + tb] = wb;
        if (k < RS) {
            sV[k * kTile + ta] = wa;
            sV[k * kTile + tb] = wb;
        }
        // ---- residual column c, entries (ta, c) and (tb, c)
        float2 ua = z2, ub = z2;
        {
            float4 pc, qc;
            fragI(c, pc, qc);
            if (rowA) ua = lr_entry<ATT>(a, bc, bc == kFlagBits ? block_bit(bw, pitch, ta, c) : true, pc, qc, pjA, qjA);
            if (rowB) ub = lr_entry<ATT>(a, bc, bc == kFlagBits ? block_bit(bw, pitch, tb, c) : true, pc, qc, pjB, qjB);
            for (int m = 0; m < ks; ++m) {
                const float2 vc = sV[m * kTile + c];
                ua = csub_mul(ua, sU[m * kTile + ta], vc);
                ub = csub_mul(ub, sU[m * kTile + tb], vc);
            }
            for (int m = RS; m < k; ++m) {
                const float2 vc = Vb[m * kTile + c];
                ua = csub_mul(ua, Ub[m * kTile + ta], vc);
                ub = csub_mul(ub, Ub[m * kTile + tb], vc);
            }
        }
        Ub[k * kTile + ta] = ua;
        Ub[k * kTile + tb] = ub;
        if (k < RS) {
            sU[k * kTile + ta] = ua;
            sU[k * kTile + tb] = ub;
        }
        if (ta == r) usedA = true;
        if (tb == r) usedB = true;
        // ---- norms and the next pivot row: the largest residual-column entry among unused rows
        const float ma = ua.x * ua.x + ua.y * ua.y, mb = ub.x * ub.x + ub.y * ub.y;
        float nu2 = ma + mb, nv2 = (wa.x * wa.x + wa.y * wa.y) + (wb.x * wb.x + wb.y * wb.y);
        float bn;
        int nr;
        cta_reduce2<true, true>(ma, ta, !usedA, mb, tb, !usedB, bn, nr, nu2, nv2, slotB, sumB);
        norm2 += nu2 * nv2;
        ++k;
        if (nu2 * nv2 <= tol * tol * norm2) break;
        if (bn < 0.0f) break;  // every row taken
        r = nr;
    }
    // ---- the exact entries judge the approximation: every row once at a
    // hashed column, every column once at a hashed row (as k_aca)
    float e2 = 0.0f, x2 = 0.0f;
    const bool converged = k > 0 && k < K;
    __syncthreads();
    if (converged) {
        const int ks = min(k, RS);
#pragma unroll 1
        for (int q = 0; q < 4; ++q) {
            const int tt = (q & 1) ? tb : ta, h2 = q >> 1;  // samples tt and tt + 256
            const int s = tt + kTile * h2;
            unsigned h = (unsigned)b * 2654435761u + (unsigned)s * 40503u + 12345u;
            h ^= h >> 13;
            h *= 0x5bd1e995u;
            h ^= h >> 15;
            const int jj = h2 == 0 ? tt : (int)(h & 255u), ii = h2 == 0 ? (int)(h & 255u) : tt;
            if (ii < ni && jj < nj) {
                const bool bit = bc == kFlagBits ? block_bit(bw, pitch, jj, ii) : true;
                float4 fpi, fni, fpj, fnj;
                fragI(ii, fpi, fni);
                fragJ(jj, fpj, fnj);
                const float2 ex = lr_entry<ATT>(a, bc, bit, fpi, fni, fpj, fnj);
                float2 ap = z2;
                for (int m = 0; m < ks; ++m) ap = csub_mul(ap, sU[m * kTile + jj], sV[m * kTile + ii]);
                for (int m = RS; m < k; ++m) ap = csub_mul(ap, Ub[m * kTile + jj], Vb[m * kTile + ii]);
                e2 += (ex.x + ap.x) * (ex.x + ap.x) + (ex.y + ap.y) * (ex.y + ap.y);
                x2 += ex.x * ex.x + ex.y * ex.y;
            }
        }
    }
    {
        float f;
        int fi;
        cta_reduce2<false, true>(0.0f, 0, false, 0.0f, 0, false, f, fi, e2, x2, nullptr, sumB);
    }
    const float rel = x2 > 0.0f ? sqrtf(e2 / x2) : (e2 > 0.0f ? 1.0f : 0.0f);  // the same in every thread
    const bool accepted = converged && rel <= limit;
    if (t == 0) {
        rank[b] = accepted ? k : -1;
        fro[b] = sqrtf(norm2);
        err[b] = converged ? rel : -1.0f;
    }
    if (brow && accepted) {
        // the fragment staging (or the factor ranks' shared memory) is free
        // now: weights and projections of the apply
        static_assert(FRAG || 2 * RS * kTile * sizeof(float2) >= (kTile + 2 * kLrMaxRank) * sizeof(float4) / 1,
                      "room for the apply's shared arrays");
        float4 *sW = FRAG ? &sFrag[0][0] : reinterpret_cast<float4 *>(aca_smem);
        float2 *sTv = FRAG ? reinterpret_cast<float2 *>(&sFrag[1][0]) : reinterpret_cast<float2 *>(sW + kTile);
        float2 *sSu = sTv + kLrMaxRank;
        lr_block_apply<kAca2Threads>(a, I, J, Ub, Vb, k, brow + (size_t)b * kTile, bcol + (size_t)b * kTile, sW, sTv,
                                     sSu);
    }
}

// ---------------------------------------------------------------- judge audit
// Full-tile check of accepted blocks: the relative RMS error of the factors
// over every one of the block's 256 x 256 entries (exact entries as the
// cross approximation evaluates them), one CTA per sampled block, thread t
// the column t.  It tells whether the judge's 512 sampled entries catch the
// blocks whose error concentrates in a few rows.
__global__ void __launch_bounds__(kTile) k_lr_audit(SumArgs a, const int2 *blocks, const uint8_t *cls,
                                                    const long long *off, const int *rank, const int *sample, int ns,
                                                    const float2 *U, const float2 *V, float *out_err,
                                                    const uint8_t *lev)
{
    __shared__ float4 sP[kTile], sN[kTile];
    __shared__ float2 sums[kAcaWarps];
    const int t = threadIdx.x;
    if (blockIdx.x >= ns) return;
    const int b = sample[blockIdx.x], k = rank[b];
    if (lev && lev[b]) return;  // an interpolated block (audited by the interpolation kernel)
    const int I = blocks[b].x, J = blocks[b].y, bc = cls[b];
    const int ni = min(kTile, a.nsrc - I * kTile), nj = min(kTile, a.nsrc - J * kTile);
    const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    sP[t] = t < nj ? a.srcA[J * kTile + t] : z4;
    sN[t] = t < nj ? a.srcB[J * kTile + t] : z4;
    __syncthreads();
    const uint32_t *bw = a.mask.bits + (long long)I * kWordsPerTile * a.mask.pitch + (long long)J * kTile;
    const float2 *U0 = U + off[b] * kTile, *V0 = V + off[b] * kTile;
    float e2 = 0.0f, x2 = 0.0f;
    if (t < ni && k > 0) {
        const float4 pi = a.srcA[I * kTile + t], qi = a.srcB[I * kTile + t];
        for (int j = 0; j < nj; ++j) {
            const bool bit = bc == kFlagBits ? block_bit(bw, a.mask.pitch, j, t) : true;
            const float2 ex = lr_entry<false>(a, bc, bit, pi, qi, sP[j], sN[j]);
            float2 ap = ex;
            for (int m = 0; m < k; ++m) ap = csub_mul(ap, U0[m * kTile + j], V0[m * kTile + t]);
            e2 += ap.x * ap.x + ap.y * ap.y;
            x2 += ex.x * ex.x + ex.y * ex.y;
        }
    }
    float f = 0.0f;
    int fi = 0;
    cta_reduce<false, true>(f, fi, false, e2, x2, nullptr, sums);
    if (t == 0) out_err[blockIdx.x] = x2 > 0.0f ? sqrtf(e2 / x2) : 0.0f;
}

// Block descriptors of the admissibility network, one warp per block:
// log2(1 + separation / lambda), log2(1 + radius / lambda) of both tiles, the
// cosines of both mean normals with the separation direction and with each
// other, (r_I + r_J) / separation (at most 4) and the fraction of the block's
// pairs that interact (1 for ALL, the stored bits for BITS, 256 sampled gate
// pairs for CLEAR).
__global__ void __launch_bounds__(128) k_block_desc(SumArgs a, const int2 *blocks, const uint8_t *cls, int nblocks,
                                                    const float4 *cen, const float4 *nm, float inv_lambda, float *X,
                                                    const int *ndev)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b = blockIdx.x * 4 + warp;
    if (b >= (ndev ? min(*ndev, nblocks) : nblocks)) return;
    const int I = blocks[b].x, J = blocks[b].y, bc = cls[b];
    const int ni = min(kTile, a.nsrc - I * kTile), nj = min(kTile, a.nsrc - J * kTile);
    float vis = 1.0f;
    if (bc == kFlagBits) {
        const uint32_t *bw = a.mask.bits + (long long)I * kWordsPerTile * a.mask.pitch + (long long)J * kTile;
        const int nw = (ni + 31) >> 5;
        int cnt = 0;
        for (int w = 0; w < nw; ++w)
            for (int j = lane; j < nj; j += 32) cnt += __popc(bw[(long long)w * a.mask.pitch + j]);
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        vis = (float)cnt / (float)(ni * nj);
    } else if (bc == kFlagClear) {
        int cnt = 0;
        for (int q = 0; q < 8; ++q) {
            const int s = lane + 32 * q;
            unsigned h = (unsigned)b * 2654435761u + (unsigned)s * 40503u + 777u;
            h ^= h >> 13;
            h *= 0x5bd1e995u;
            h ^= h >> 15;
            const int ii = (int)(h & 255u) % ni, jj = (int)((h >> 8) & 255u) % nj;
            const float4 pi = a.srcA[I * kTile + ii], qi = a.srcB[I * kTile + ii];
            const float4 pj = a.srcA[J * kTile + jj], qj = a.srcB[J * kTile + jj];
            const Dst d{pj.x, pj.y, pj.z, qj.x, qj.y, qj.z};
            float Tr, Ti;
            bool ok;
            sym_pair<false, true, false>(a, pi, qi, d, Tr, Ti, ok);
            cnt += ok ? 1 : 0;
        }
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        vis = (float)cnt / 256.0f;
    }
    if (lane == 0) {
        const float4 cI = cen[I], cJ = cen[J], nI = nm[I], nJ = nm[J];
        const float sx = cJ.x - cI.x, sy = cJ.y - cI.y, sz = cJ.z - cI.z;
        const float sep = sqrtf(sx * sx + sy * sy + sz * sz);
        const float is = sep > 0.0f ? 1.0f / sep : 0.0f;
        float *x = X + (size_t)b * 8;
        x[0] = log2f(1.0f + sep * inv_lambda);
        x[1] = log2f(1.0f + cI.w * inv_lambda);
        x[2] = log2f(1.0f + cJ.w * inv_lambda);
        x[3] = (nI.x * sx + nI.y * sy + nI.z * sz) * is;
        x[4] = (nJ.x * sx + nJ.y * sy + nJ.z * sz) * is;
        x[5] = nI.x * nJ.x + nI.y * nJ.y + nI.z * nJ.z;
        x[6] = sep > 0.0f ? fminf((cI.w + cJ.w) * is, 4.0f) : 4.0f;
        x[7] = vis;
    }
}

// Compressed bounce, one CTA per accepted block q (kept block b = bidx[q]):
// lr_block_apply into the block's output slots b.  The factors are read from
// HBM once; the second pass over them hits L2.
template <int MINB>
__global__ void __launch_bounds__(kTile, MINB) k_lr_block(SumArgs a, const int2 *blocks, const long long *off,
                                                          const int *bidx, int nb, const float2 *U, const float2 *V,
                                                          const int *rank, float2 *brow, float2 *bcol, const int *ndev,
                                                          const uint8_t *lev, const int *list)
{
    __shared__ float4 sW[kTile];  // (Re w_I, Im w_I, Re w_J, Im w_J) of every row t
    __shared__ float2 sTv[kLrMaxRank], sSu[kLrMaxRank];
    const int q = blockIdx.x;
    int b;
    if (list) {
        // the cross-approximated kept blocks; rejected ones stay dense
        if (q >= nb) return;
        b = list[q];
        if (rank[b] <= 0) return;
    } else {
        if (q >= (ndev ? min(*ndev, nb) : nb)) return;
        b = bidx[q];
        if (lev && lev[b]) return;  // an interpolated block
    }
    lr_block_apply<kTile, true>(a, blocks[b].x, blocks[b].y, U + off[b] * kTile, V + off[b] * kTile, rank[b],
                                brow + (size_t)b * kTile, bcol + (size_t)b * kTile, sW, sTv, sSu);
}

// Per owner tile X: rows of every accepted block with J = X and columns of
// every accepted block with I = X, in list order, summed with compensated
// FP32 (Kahan) arithmetic -- FP64 adds run at a small fraction of the FP32
// rate on this GPU -- and stored as FP64 (deterministic order).  The lists
// hold accepted-block positions q; their outputs sit at slot bidx[q].
__device__ __forceinline__ void kahan_add(float &s, float &c, float x)
{
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

// One CTA of kGatherSeg x 256 threads per tile X.  The tile's two lists --
// the blocks (., X), whose row outputs add into yrow, then the blocks (X, .),
// whose column outputs add into ycol -- are read as one sequence cut into
// kGatherSeg equal segments, one per 256-thread group; thread t of a group
// adds entry t of its segment's blocks in list order (compensated FP32) and
// the groups' sums are added in group order in FP64.  With upper-triangular
// block sets the two lists of tile X hold about X and ntiles - X blocks, so
// the cut bounds every thread's chain of loads by a quarter of both.
constexpr int kGatherSeg = 4;

__global__ void __launch_bounds__(kGatherSeg * kTile, 2) k_lr_gather(int n, const float2 *brow, const float2 *bcol,
                                                                     const int *byJ_off, const int *byJ,
                                                                     const int *byI_off, const int *byI,
                                                                     const int *bidx, double2 *yrow, double2 *ycol)
{
    __shared__ double2 part[2][kGatherSeg][kTile];  // [rows, columns][group][t]
    const int X = blockIdx.x, t = threadIdx.x & (kTile - 1), g = threadIdx.x / kTile;  // g warp-uniform
    const int r0 = byJ_off[X], nr = byJ_off[X + 1] - r0, c0 = byI_off[X], nc = byI_off[X + 1] - c0;
    const int L = nr + nc, p0 = (int)((long long)L * g / kGatherSeg), p1 = (int)((long long)L * (g + 1) / kGatherSeg);
    const int pm = min(max(nr, p0), p1);  // [p0, pm): rows, [pm, p1): columns
    float fr = 0.0f, fi = 0.0f, efr = 0.0f, efi = 0.0f;
#pragma unroll 8
    for (int p = p0; p < pm; ++p) {
        const float2 v = __ldg(brow + (size_t)bidx[byJ[r0 + p]] * kTile + t);
        kahan_add(fr, efr, v.x);
        kahan_add(fi, efi, v.y);
    }
    part[0][g][t] = make_double2((double)fr - (double)efr, (double)fi - (double)efi);
    fr = fi = efr = efi = 0.0f;
#pragma unroll 8
    for (int p = pm; p < p1; ++p) {
        const float2 v = __ldg(bcol + (size_t)bidx[byI[c0 + p - nr]] * kTile + t);
        kahan_add(fr, efr, v.x);
        kahan_add(fi, efi, v.y);
    }
    part[1][g][t] = make_double2((double)fr - (double)efr, (double)fi - (double)efi);
    __syncthreads();
    const int q = X * kTile + t;
    if (g < 2 && q < n) {
        double2 y = part[g][0][t];
#pragma unroll
        for (int k = 1; k < kGatherSeg; ++k) {
            y.x += part[g][k][t].x;
            y.y += part[g][k][t].y;
        }
        (g ? ycol : yrow)[q] = y;
    }
}

// Per-tile geometry for block descriptors: centroid, radius, mean normal.
__global__ void __launch_bounds__(kTile) k_tile_stats(const float4 *pos, const float4 *nrm, int n, float4 *cen,
                                                      float4 *nmean)
{
    __shared__ float sv[kTile / 32];
    const int T = blockIdx.x, t = threadIdx.x, i = T * kTile + t;
    const bool v = i < n;
    const float4 p = v ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 q = v ? nrm[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float cnt = block_sum(v ? 1.0f : 0.0f, sv);
    const float cx = block_sum(p.x, sv) / cnt, cy = block_sum(p.y, sv) / cnt, cz = block_sum(p.z, sv) / cnt;
    const float nx = block_sum(q.x, sv), ny = block_sum(q.y, sv), nz = block_sum(q.z, sv);
    const float dx = p.x - cx, dy = p.y - cy, dz = p.z - cz;
    float r = v ? sqrtf(dx * dx + dy * dy + dz * dz) : 0.0f;
    for (int off = 16; off > 0; off >>= 1) r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, off));
    __syncthreads();
    if ((t & 31) == 0) sv[t >> 5] = r;
    __syncthreads();
    if (t == 0) {
        float rm = 0.0f;
        for (int w = 0; w < kTile / 32; ++w) rm = fmaxf(rm, sv[w]);
        const float nl = sqrtf(nx * nx + ny * ny + nz * nz);
        cen[T] = make_float4(cx, cy, cz, rm);
        nmean[T] = nl > 0.0f ? make_float4(nx / nl, ny / nl, nz / nl, 0.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// ---------------------------------------------------------------- helpers
__global__ void k_pack_points(const float4 *pts, const double2 *P, int n, float4 *A, float4 *B)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pts[i];
    const double2 w = P[i];
    A[i] = make_float4(p.x, p.y, p.z, (float)w.x);
    B[i] = make_float4(0.0f, 0.0f, 0.0f, (float)w.y);
}

__global__ void k_pack_frags(const float4 *act_pos, const int *act_facet, const int *act_cell, const float4 *facet_n,
                             const double2 *P, float scale, int n, float4 *A, float4 *B)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = act_pos[i];
    const float4 fn = facet_n[act_facet[i]];
    const double2 v = P[act_cell[i]];
    const double s = (double)scale * (double)p.w;
    A[i] = make_float4(p.x, p.y, p.z, (float)(s * v.x));
    B[i] = make_float4(fn.x, fn.y, fn.z, (float)(s * v.y));
}

__global__ void k_f2f_limits(const int *act_facet, const int *act_cell, const int *facet_end, const double2 *Pin,
                             int n, int nsrc, int *limit)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double2 p = Pin[act_cell[j]];
    limit[j] = (p.x == 0.0 && p.y == 0.0) ? facet_end[act_facet[j]] : nsrc;
}

__global__ void k_finalize_add(const double2 *partial, int nsplit, int ndst, const int *cell, double2 *out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ndst) return;
    double sr = 0.0, si = 0.0;
    for (int k = 0; k < nsplit; ++k) {
        const double2 v = partial[(long long)k * ndst + j];
        sr += v.x;
        si += v.y;
    }
    const int c = cell ? cell[j] : j;
    double2 o = out[c];
    o.x += sr;
    o.y += si;
    out[c] = o;
}

__global__ void k_finalize_f2f(const double2 *partial, int nsplit, int ndst, const int *cell, double2 *Pout,
                               double2 *P)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ndst) return;
    double sr = 0.0, si = 0.0;
    for (int k = 0; k < nsplit; ++k) {
        const double2 v = partial[(long long)k * ndst + j];
        sr += v.x;
        si += v.y;
    }
    const int c = cell[j];
    Pout[c] = make_double2(sr, si);
    double2 o = P[c];
    o.x += sr;
    o.y += si;
    P[c] = o;
}

// FACET_RESP: P_out[cell] += s, P[cell] += s; with gate_pin, destinations
// whose P_in is 0 receive nothing (the zero-input skip of the first object's
// cell also kills its reciprocal term, OptiX.cu:241-245, :367-390)
__global__ void k_finalize_resp(const double2 *partial, int nsplit, int ndst, const int *cell,
                                const double2 *gate_pin, double2 *Pout, double2 *P)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ndst) return;
    const int c = cell[j];
    if (gate_pin) {
        const double2 g = gate_pin[c];
        if (g.x == 0.0 && g.y == 0.0) return;
    }
    double sr = 0.0, si = 0.0;
    for (int k = 0; k < nsplit; ++k) {
        const double2 v = partial[(long long)k * ndst + j];
        sr += v.x;
        si += v.y;
    }
    double2 o = Pout[c];
    o.x += sr;
    o.y += si;
    Pout[c] = o;
    o = P[c];
    o.x += sr;
    o.y += si;
    P[c] = o;
}

__global__ void k_mask_export(MaskView m, int nsrc, int ndst, uint8_t *out)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)ndst * m.nwords;
    if (idx >= total) return;
    const int j = (int)(idx / m.nwords);
    const int w = (int)(idx % m.nwords);
    const uint32_t word = m.bits[(long long)w * m.pitch + j];
    const int bmax = min(32, nsrc - w * 32);
    for (int b = 0; b < bmax; ++b) out[(long long)j * nsrc + w * 32 + b] = (word >> b) & 1u;
}

// the rows rows[0..nrows) of the mask (internal destination indices) as
// bytes, row q at out[q * nsrc]
__global__ void k_mask_export_rows(MaskView m, int nsrc, const int *rows, int nrows, uint8_t *out)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)nrows * m.nwords;
    if (idx >= total) return;
    const int q = (int)(idx / m.nwords);
    const int w = (int)(idx % m.nwords);
    const uint32_t word = m.bits[(long long)w * m.pitch + rows[q]];
    const int bmax = min(32, nsrc - w * 32);
    for (int b = 0; b < bmax; ++b) out[(long long)q * nsrc + w * 32 + b] = (word >> b) & 1u;
}

inline unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// ---------------------------------------------------------------- peaks
// Throughput probes for the roofline denominators: 8 independent FMA chains
// per thread (FP32 pipe) and a chain of __sinf (MUFU).  The results are kept
// live by a conditional store that never fires for the inputs used.
__global__ void k_peak_fma(int iters, float seed, float *sink)
{
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + (float)(threadIdx.x + k);
    const float m = 0.9999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], m, c);
    }
    float t = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) t += a[k];
    if (t == 12345.678f) sink[blockIdx.x] = t;
}

__global__ void k_peak_mufu(int iters, float seed, float *sink)
{
    float a[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) a[k] = seed + 1e-3f * (float)(threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 4; ++k) a[k] = __sinf(a[k]);
    }
    float t = a[0] + a[1] + a[2] + a[3];
    if (t == 12345.678f) sink[blockIdx.x] = t;
}

}  // namespace

double measure_peak(int which)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1.0;
    cudaStream_t st;
    cudaEvent_t e0, e1;
    float *sink = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return -1.0;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMalloc(&sink, sizeof(float) * sms * 64);
    const int blocks = sms * 8, threads = 256;
    const int iters = which == 0 ? 1 << 14 : 1 << 12;
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0, st);
        if (which == 0)
            k_peak_fma<<<blocks, threads, 0, st>>>(iters, 1.0f, sink);
        else
            k_peak_mufu<<<blocks, threads, 0, st>>>(iters, 0.5f, sink);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double ops = (double)blocks * threads * iters * (which == 0 ? 8.0 * 2.0 : 4.0);
        if (ms > 0.0f) best = std::max(best, ops / (ms * 1e-3));
    }
    const bool ok = cudaGetLastError() == cudaSuccess;
    cudaFree(sink);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    return ok ? best : -1.0;
}

int launch_mask_classified(const MaskArgs &a0, int2 *blist, int *count_dev, int nsm, cudaStream_t s)
{
    if (a0.nsrc <= 0 || a0.ndst <= 0) return 0;
    const size_t nflags = (size_t)a0.mask.ntiles * a0.mask.ndstblocks;
    cudaMemsetAsync(a0.mask.flags, kFlagNone, nflags, s);
    cudaMemsetAsync(count_dev, 0, 2 * sizeof(int), s);
    dim3 grid((a0.mask.ndstblocks + kClsWarps - 1) / kClsWarps, a0.mask.ntiles);
    k_mask_classify_f2f<<<grid, 32 * kClsWarps, 0, s>>>(a0, blist, count_dev);
    // the pair kernel on the listed blocks: resident CTAs read the count on the device
    static int per_sm = 0;
    if (per_sm == 0 &&
        (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mask_listed, kTile, 0) != cudaSuccess ||
         per_sm < 1))
        per_sm = 1;
    MaskArgs a = a0;
    a.blist = blist;
    a.blist_count = count_dev;
    a.blist_next = count_dev + 1;
    const size_t ctas = std::min<size_t>(nflags, (size_t)std::max(nsm, 1) * per_sm);
    k_mask_listed<<<(unsigned)ctas, kTile, 0, s>>>(a);
    return 2;
}

void launch_mask(const MaskArgs &a, cudaStream_t s)
{
    if (a.nsrc <= 0 || a.ndst <= 0) return;
    dim3 grid(a.mask.ndstblocks, a.mask.ntiles);
    switch (a.hop) {
    case HOP_SRC: k_mask<HOP_SRC><<<grid, kTile, 0, s>>>(a); break;
    case HOP_FP: k_mask<HOP_FP><<<grid, kTile, 0, s>>>(a); break;
    case HOP_F2F: k_mask<HOP_F2F><<<grid, kTile, 0, s>>>(a); break;
    case HOP_RESP: k_mask<HOP_RESP><<<grid, kTile, 0, s>>>(a); break;
    default: k_mask<HOP_NORESP><<<grid, kTile, 0, s>>>(a); break;
    }
}

void launch_batch_vis(const BatchVisArgs &a, int nsm, cudaStream_t s)
{
    if (a.nfrag <= 0) return;
    cudaMemsetAsync(a.hard_count, 0, sizeof(unsigned), s);
    k_batch_vis<<<(unsigned)((a.nfrag + kTile - 1) / kTile), kTile, 0, s>>>(a);
    k_batch_vis_hard<<<(unsigned)(8 * nsm), kTile, 0, s>>>(a);
}

void launch_sum(const SumArgs &a, cudaStream_t s)
{
    if (a.nsrc <= 0 || a.ndst <= 0) return;
    dim3 grid(a.mask.ndstblocks, a.nsplit);
    const bool att = a.ka != 0.0f;
    switch (a.hop) {
    case HOP_SRC:
        if (a.rel) {
            if (att) k_sum<HOP_SRC, true, true><<<grid, kTile, 0, s>>>(a);
            else k_sum<HOP_SRC, false, true><<<grid, kTile, 0, s>>>(a);
        } else {
            if (att) k_sum<HOP_SRC, true><<<grid, kTile, 0, s>>>(a);
            else k_sum<HOP_SRC, false><<<grid, kTile, 0, s>>>(a);
        }
        break;
    case HOP_FP:
        if (a.rel) {
            if (att) k_sum<HOP_FP, true, true><<<grid, kTile, 0, s>>>(a);
            else k_sum<HOP_FP, false, true><<<grid, kTile, 0, s>>>(a);
        } else {
            if (att) k_sum<HOP_FP, true><<<grid, kTile, 0, s>>>(a);
            else k_sum<HOP_FP, false><<<grid, kTile, 0, s>>>(a);
        }
        break;
    case HOP_F2F:
        if (att) k_sum<HOP_F2F, true><<<grid, kTile, 0, s>>>(a);
        else k_sum<HOP_F2F, false><<<grid, kTile, 0, s>>>(a);
        break;
    case HOP_RESP:
        if (att) k_sum<HOP_RESP, true><<<grid, kTile, 0, s>>>(a);
        else k_sum<HOP_RESP, false><<<grid, kTile, 0, s>>>(a);
        break;
    default:
        if (att) k_sum<HOP_NORESP, true><<<grid, kTile, 0, s>>>(a);
        else k_sum<HOP_NORESP, false><<<grid, kTile, 0, s>>>(a);
        break;
    }
}

void launch_sym_worklist(const uint8_t *flags, int ntiles, int nb, int per, int *blist, int *rowcnt, int *chunk_off,
                         int4 *chunks, int *nchunks, cudaStream_t s)
{
    if (nb <= 0) return;
    k_sym_rows<<<nb, kTile, 0, s>>>(flags, ntiles, nb, blist, rowcnt);
    k_sym_chunks<<<1, 1024, 0, s>>>(rowcnt, nb, per, chunk_off, chunks, nchunks);
}

void launch_sum_f2f_sym(const SumArgs &a, const SymWork &wl, int grid, double2 *colpart, double2 *rowpart,
                        cudaStream_t s)
{
    if (a.nsrc <= 0 || a.ndst <= 0 || grid <= 0) return;
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_sum_f2f_sym<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSymDynSmem);
        cudaFuncSetAttribute(k_sum_f2f_sym<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSymDynSmem);
        attr_set = true;
    }
    cudaMemsetAsync(wl.next, 0, sizeof(int), s);
    if (a.ka != 0.0f)
        k_sum_f2f_sym<true><<<grid, kTile, kSymDynSmem, s>>>(a, wl, colpart, rowpart);
    else
        k_sum_f2f_sym<false><<<grid, kTile, kSymDynSmem, s>>>(a, wl, colpart, rowpart);
}

void launch_finalize_f2f_sym(const double2 *rowpart, const int *chunk_off, int ndst, const double2 *colpart,
                             const uint8_t *flags, int ntiles, const int *cell, const double2 *Pin, double2 *Pout,
                             double2 *P, cudaStream_t s, const double2 *yrow, const double2 *ycol)
{
    if (ndst > 0)
        k_finalize_f2f_sym<<<blocks_for(ndst, 256), 256, 0, s>>>(rowpart, chunk_off, ndst, colpart, flags, ntiles,
                                                                 cell, Pin, Pout, P, yrow, ycol);
}

namespace {
template <bool ATT, int RS, int MINB>
void launch_aca_t(const SumArgs &a, const int2 *blocks, const uint8_t *cls, const int *cap, const long long *off,
                  int nblocks, float tol, float2 *U, float2 *V, int *rank, float *fro, float limit, float *err,
                  cudaStream_t s, const int *list)
{
    const size_t smem = (size_t)2 * RS * kTile * sizeof(float2);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_aca<ATT, RS, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    k_aca<ATT, RS, MINB><<<(unsigned)nblocks, kTile, smem, s>>>(a, blocks, cls, cap, off, nblocks, tol, limit, U, V,
                                                                 rank, fro, err, list);
}

template <bool ATT, int RS, int MINB, bool FRAG = true>
void launch_aca2_t(const SumArgs &a, const int2 *blocks, const uint8_t *cls, const int *cap, const long long *off,
                   int nblocks, float tol, float2 *U, float2 *V, int *rank, float *fro, float limit, float *err,
                   cudaStream_t s, float2 *brow, float2 *bcol, const int *list)
{
    const size_t smem = (size_t)2 * RS * kTile * sizeof(float2);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_aca2<ATT, RS, MINB, FRAG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    k_aca2<ATT, RS, MINB, FRAG><<<(unsigned)nblocks, kAca2Threads, smem, s>>>(
        a, blocks, cls, cap, off, nblocks, tol, limit, U, V, rank, fro, err, brow, bcol, list);
}

template <bool ATT>
bool launch_aca_v(int variant, const SumArgs &a, const int2 *blocks, const uint8_t *cls, const int *cap,
                  const long long *off, int nblocks, float tol, float2 *U, float2 *V, int *rank, float *fro,
                  float limit, float *err, cudaStream_t s, float2 *brow, float2 *bcol, const int *list)
{
    switch (variant) {
    case 3: launch_aca2_t<ATT, 8, 4>(a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, brow, bcol, list); return brow != nullptr;
    case 4: launch_aca2_t<ATT, 6, 5>(a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, brow, bcol, list); return brow != nullptr;
    case 5: launch_aca2_t<ATT, 4, 6>(a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, brow, bcol, list); return brow != nullptr;
    case 6: launch_aca2_t<ATT, 2, 8>(a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, brow, bcol, list); return brow != nullptr;
    case 7: launch_aca2_t<ATT, 3, 7>(a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, brow, bcol, list); return brow != nullptr;
    case 8: launch_aca2_t<ATT, 8, 6, false>(a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, brow, bcol, list); return brow != nullptr;
    case 9: launch_aca2_t<ATT, 6, 7, false>(a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, brow, bcol, list); return brow != nullptr;
    case 10: launch_aca2_t<ATT, 4, 8, false>(a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, brow, bcol, list); return brow != nullptr;
    case 1: launch_aca_t<ATT, 12, 4>(a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, list); break;
    case 2: launch_aca_t<ATT, 16, 3>(a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, list); break;
    default: launch_aca_t<ATT, 8, 4>(a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, list); break;
    }
    return false;
}
}  // namespace

// variant: factor ranks kept in shared memory and CTAs per SM -- k_aca (one
// row and one column per thread): 0: 8 ranks, 4 CTAs; 1: 12 ranks, 4 CTAs;
// 2: 16 ranks, 3 CTAs; k_aca2 (two rows and two columns per thread, the first
// bounce's apply fused): 3: 8 ranks, 4 CTAs; 4: 6 ranks, 5 CTAs; 5: 4 ranks,
// 6 CTAs (the fastest on the 60 kHz trihedral); 6: 2 ranks, 8 CTAs; 7: 3
// ranks, 7 CTAs; without the fragment staging: 8: 8 ranks, 6 CTAs; 9: 6
// ranks, 7 CTAs; 10: 4 ranks, 8 CTAs
bool launch_aca(const SumArgs &a, const int2 *blocks, const uint8_t *cls, const int *cap, const long long *off,
                int nblocks, float tol, float2 *U, float2 *V, int *rank, float *fro, float limit, float *err,
                cudaStream_t s, int variant, float2 *brow, float2 *bcol, const int *list)
{
    if (nblocks <= 0) return brow != nullptr && variant >= 3;  // nothing to build; outputs as the variant would write
    if (a.ka != 0.0f)
        return launch_aca_v<true>(variant, a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, brow,
                                  bcol, list);
    return launch_aca_v<false>(variant, a, blocks, cls, cap, off, nblocks, tol, U, V, rank, fro, limit, err, s, brow,
                               bcol, list);
}

void launch_lr_audit(const SumArgs &a, const int2 *blocks, const uint8_t *cls, const long long *off, const int *rank,
                     const int *sample, int ns, const float2 *U, const float2 *V, float *out_err, cudaStream_t s,
                     const uint8_t *lev)
{
    if (a.ka != 0.0f) return;  // the audit evaluates entries without attenuation only
    if (ns > 0) k_lr_audit<<<ns, kTile, 0, s>>>(a, blocks, cls, off, rank, sample, ns, U, V, out_err, lev);
}

void launch_block_desc(const SumArgs &a, const int2 *blocks, const uint8_t *cls, int nblocks, const float4 *cen,
                       const float4 *nm, float inv_lambda, float *X, cudaStream_t s, const int *ndev)
{
    if (nblocks > 0)
        k_block_desc<<<(nblocks + 3) / 4, 128, 0, s>>>(a, blocks, cls, nblocks, cen, nm, inv_lambda, X, ndev);
}

void launch_lr_apply(const SumArgs &a, const int2 *blocks, const long long *off, const int *bidx, int nb,
                     const float2 *U, const float2 *V, const int *rank, float2 *brow, float2 *bcol, int ntiles,
                     const int *byJ_off, const int *byJ, const int *byI_off, const int *byI, double2 *yrow,
                     double2 *ycol, cudaStream_t s, const int *ndev, bool outputs_ready, int lr_ctas,
                     const IpCtx *ip, const int *aca_list, int naca)
{
    // latency-bound on the factor stream: resident CTAs per SM are the lever
    // (registers capped to fit lr_ctas of them)
    if (nb > 0 && !outputs_ready) {
        const uint8_t *lev = ip ? ip->lev : nullptr;
        const bool ip_side = ip && ip->stream && ip->fork && ip->join;
        // with kept-block lists each kernel gets a grid of its own blocks
        const int nl = aca_list ? naca : nb;
        if (ip_side) {
            cudaEventRecord(ip->fork, s);
            cudaStreamWaitEvent(ip->stream, ip->fork, 0);
            launch_ip_apply(a, ip->tile, ip->fxy, ip->lev, ip->delta, blocks, off, bidx, nb, ndev, U, brow, bcol,
                            ip->stream, ip->list, ip->n, rank, ip->status);
            cudaEventRecord(ip->join, ip->stream);
        }
        if (nl > 0) {
            if (lr_ctas >= 8)
                k_lr_block<8><<<nl, kTile, 0, s>>>(a, blocks, off, bidx, nl, U, V, rank, brow, bcol, ndev, lev, aca_list);
            else if (lr_ctas >= 6)
                k_lr_block<6><<<nl, kTile, 0, s>>>(a, blocks, off, bidx, nl, U, V, rank, brow, bcol, ndev, lev, aca_list);
            else
                k_lr_block<4><<<nl, kTile, 0, s>>>(a, blocks, off, bidx, nl, U, V, rank, brow, bcol, ndev, lev, aca_list);
        }
        if (ip_side)
            cudaStreamWaitEvent(s, ip->join, 0);
        else if (ip)
            launch_ip_apply(a, ip->tile, ip->fxy, ip->lev, ip->delta, blocks, off, bidx, nb, ndev, U, brow, bcol, s,
                            ip->list, ip->n, rank, ip->status);
    }
    if (ntiles > 0)
        k_lr_gather<<<ntiles, kGatherSeg * kTile, 0, s>>>(a.nsrc, brow, bcol, byJ_off, byJ, byI_off, byI, bidx, yrow,
                                                          ycol);
}

void launch_tile_stats(const float4 *pos, const float4 *nrm, int n, float4 *cen, float4 *nmean, cudaStream_t s)
{
    if (n > 0) k_tile_stats<<<(n + kTile - 1) / kTile, kTile, 0, s>>>(pos, nrm, n, cen, nmean);
}

void launch_pack_points(const float4 *pts, const double2 *P, int n, float4 *A, float4 *B, cudaStream_t s)
{
    if (n > 0) k_pack_points<<<blocks_for(n, 256), 256, 0, s>>>(pts, P, n, A, B);
}

void launch_pack_frags(const float4 *act_pos, const int *act_facet, const int *act_cell, const float4 *facet_n,
                       const double2 *P, float scale, int n, float4 *A, float4 *B, cudaStream_t s)
{
    if (n > 0) k_pack_frags<<<blocks_for(n, 256), 256, 0, s>>>(act_pos, act_facet, act_cell, facet_n, P, scale, n, A, B);
}

void launch_f2f_limits(const int *act_facet, const int *act_cell, const int *facet_end, const double2 *Pin, int n,
                       int nsrc, int *limit, cudaStream_t s)
{
    if (n > 0) k_f2f_limits<<<blocks_for(n, 256), 256, 0, s>>>(act_facet, act_cell, facet_end, Pin, n, nsrc, limit);
}

void launch_finalize_add(const double2 *partial, int nsplit, int ndst, const int *cell, double2 *out, cudaStream_t s)
{
    if (ndst > 0) k_finalize_add<<<blocks_for(ndst, 256), 256, 0, s>>>(partial, nsplit, ndst, cell, out);
}

void launch_finalize_f2f(const double2 *partial, int nsplit, int ndst, const int *cell, double2 *Pout, double2 *P,
                         cudaStream_t s)
{
    if (ndst > 0) k_finalize_f2f<<<blocks_for(ndst, 256), 256, 0, s>>>(partial, nsplit, ndst, cell, Pout, P);
}

void launch_finalize_resp(const double2 *partial, int nsplit, int ndst, const int *cell, const double2 *gate_pin,
                          double2 *Pout, double2 *P, cudaStream_t s)
{
    if (ndst > 0) k_finalize_resp<<<blocks_for(ndst, 256), 256, 0, s>>>(partial, nsplit, ndst, cell, gate_pin, Pout, P);
}

void launch_mask_export(const MaskView &m, int nsrc, int ndst, uint8_t *out, cudaStream_t s)
{
    const long long total = (long long)ndst * m.nwords;
    if (total > 0) k_mask_export<<<blocks_for(total, 256), 256, 0, s>>>(m, nsrc, ndst, out);
}

void launch_mask_export_rows(const MaskView &m, int nsrc, const int *rows, int nrows, uint8_t *out, cudaStream_t s)
{
    const long long total = (long long)nrows * m.nwords;
    if (total > 0) k_mask_export_rows<<<blocks_for(total, 256), 256, 0, s>>>(m, nsrc, rows, nrows, out);
}

}  // namespace sonar
