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

#include <algorithm>
#include <cstdio>

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

// ---------------------------------------------------------------- visibility
__device__ __forceinline__ bool seg_box(float3 o, float3 inv, float4 a, float4 b)
{
    const float tx0 = (a.x - o.x) * inv.x, tx1 = (b.x - o.x) * inv.x;
    const float ty0 = (a.y - o.y) * inv.y, ty1 = (b.y - o.y) * inv.y;
    const float tz0 = (a.z - o.z) * inv.z, tz1 = (b.z - o.z) * inv.z;
    const float t0 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    const float t1 = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), 1.0f));
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

constexpr int kStack = 64;

__device__ bool occluded(const BvhView &B, float3 o, float3 e, float r, float tmax)
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
        if (seg_box(o, inv, a, b)) {
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
// Returns whether pair (source s, destination t) interacts.  s/t: positions
// (w = area); ns/nt: facet normals (w of ns = source facet index bits).
template <int HOP>
__device__ __forceinline__ bool pair_pass(const MaskArgs &a, float4 s, float4 ns, float4 t, float4 nt, int ft)
{
    if (HOP == HOP_SRC) {
        // OptiX.cu:59-98: v = p_j - p_i, uv = v * (1/r), cos_inc = dot(-uv, n_B)
        const float vx = __fsub_rn(t.x, s.x), vy = __fsub_rn(t.y, s.y), vz = __fsub_rn(t.z, s.z);
        const float r = __fsqrt_rn(dot_rn(vx, vy, vz, vx, vy, vz));
        const float inv = __frcp_rn(r);
        const float ux = __fmul_rn(vx, inv), uy = __fmul_rn(vy, inv), uz = __fmul_rn(vz, inv);
        float ci = dot_rn(-ux, -uy, -uz, nt.x, nt.y, nt.z);
        if (a.dst_is_field) ci = 1.0f;
        if (ci < 1e-6f) return false;
        return !occluded(a.bvh, make_float3(s.x, s.y, s.z), make_float3(t.x, t.y, t.z), r, __fsub_rn(r, 1e-3f));
    } else if (HOP == HOP_FP) {
        // OptiX.cu:147-180: v = p_i - p_j, cos_scat = dot(-uv, n_A), ray from the field point
        const float vx = __fsub_rn(s.x, t.x), vy = __fsub_rn(s.y, t.y), vz = __fsub_rn(s.z, t.z);
        const float r = __fsqrt_rn(dot_rn(vx, vy, vz, vx, vy, vz));
        const float inv = __frcp_rn(r);
        const float ux = __fmul_rn(vx, inv), uy = __fmul_rn(vy, inv), uz = __fmul_rn(vz, inv);
        const float cs = dot_rn(-ux, -uy, -uz, ns.x, ns.y, ns.z);
        if (cs < 1e-6f) return false;
        return !occluded(a.bvh, make_float3(t.x, t.y, t.z), make_float3(s.x, s.y, s.z), r, __fsub_rn(r, 1e-3f));
    } else if (HOP == HOP_F2F) {
        // OptiX.cu:247-338 in the enumeration orientation: the lower facet
        // index is the "A" side and the ray starts there
        const int fs = __float_as_int(ns.w);
        if (fs == ft) return false;
        const bool fwd = fs < ft;
        const float4 pA = fwd ? s : t, pB = fwd ? t : s;
        const float4 nA = fwd ? ns : nt, nB = fwd ? nt : ns;
        const float vx = __fsub_rn(pB.x, pA.x), vy = __fsub_rn(pB.y, pA.y), vz = __fsub_rn(pB.z, pA.z);
        const float r = __fsqrt_rn(dot_rn(vx, vy, vz, vx, vy, vz));
        const float inv = __frcp_rn(r);
        const float ux = __fmul_rn(vx, inv), uy = __fmul_rn(vy, inv), uz = __fmul_rn(vz, inv);
        const float cs = dot_rn(ux, uy, uz, nA.x, nA.y, nA.z);
        if (cs < 1e-6f) return false;
        const float ci = dot_rn(-ux, -uy, -uz, nB.x, nB.y, nB.z);
        if (ci < 1e-6f) return false;
        return !occluded(a.bvh, make_float3(pA.x, pA.y, pA.z), make_float3(pB.x, pB.y, pB.z), r,
                         __fsub_rn(r, 1e-3f));
    } else {
        // FACET_NO_RESP, OptiX.cu:281-338 with cos_inc = 1 (field destination)
        const float vx = __fsub_rn(t.x, s.x), vy = __fsub_rn(t.y, s.y), vz = __fsub_rn(t.z, s.z);
        const float r = __fsqrt_rn(dot_rn(vx, vy, vz, vx, vy, vz));
        const float inv = __frcp_rn(r);
        const float ux = __fmul_rn(vx, inv), uy = __fmul_rn(vy, inv), uz = __fmul_rn(vz, inv);
        const float cs = dot_rn(ux, uy, uz, ns.x, ns.y, ns.z);
        if (cs < 1e-6f) return false;
        return !occluded(a.bvh, make_float3(s.x, s.y, s.z), make_float3(t.x, t.y, t.z), r, __fsub_rn(r, 1e-3f));
    }
}

template <int HOP>
__global__ void __launch_bounds__(kTile) k_mask(MaskArgs a)
{
    __shared__ float4 sP[kTile];
    __shared__ float4 sN[kTile];
    const int tid = threadIdx.x;
    const int tile = blockIdx.y;
    const int i0 = tile * kTile;
    const int j = blockIdx.x * kTile + tid;
    {
        const int i = i0 + tid;
        float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float4 n = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
        if (i < a.nsrc) {
            p = a.src_pos[i];
            if (a.src_facet) {
                const int f = a.src_facet[i];
                const float4 fn = a.src_facet_n[f];
                n = make_float4(fn.x, fn.y, fn.z, __int_as_float(f));
            }
        }
        sP[tid] = p;
        sN[tid] = n;
    }
    const bool live = j < a.ndst;
    float4 t = make_float4(0.0f, 0.0f, 0.0f, 0.0f), nt = t;
    int ft = -2;
    if (live) {
        t = a.dst_pos[j];
        if (a.dst_facet) {
            ft = a.dst_facet[j];
            nt = a.dst_facet_n[ft];
        }
    }
    __syncthreads();
    const int ntile = min(kTile, a.nsrc - i0);
    const int nw = (ntile + 31) >> 5;
    uint32_t any = 0;
    for (int w = 0; w < nw; ++w) {
        uint32_t word = 0;
        if (live) {
            const int bmax = min(32, ntile - w * 32);
            for (int b = 0; b < bmax; ++b) {
                const int q = w * 32 + b;
                if (pair_pass<HOP>(a, sP[q], sN[q], t, nt, ft)) word |= 1u << b;
            }
            a.mask.bits[(long long)(tile * kWordsPerTile + w) * a.mask.pitch + j] = word;
        }
        any |= word;
    }
    const int blk = __syncthreads_or(any != 0u);
    if (tid == 0) a.mask.flags[(long long)tile * a.mask.ndstblocks + blockIdx.x] = blk ? 1 : 0;
}

// ---------------------------------------------------------------- sums
struct Dst {
    float px, py, pz;
    float nx, ny, nz;
};

template <int HOP>
__device__ __forceinline__ void pair_term(const SumArgs &a, const float4 A, const float4 B, const Dst &d, float &tr,
                                          float &ti)
{
    // v = p_dst - p_src; |v| with the reference's rounding (its r feeds the phase)
    const float vx = __fsub_rn(d.px, A.x), vy = __fsub_rn(d.py, A.y), vz = __fsub_rn(d.pz, A.z);
    const float r2 = dot_rn(vx, vy, vz, vx, vy, vz);
    const float r = __fsqrt_rn(r2);
    const float rinv = rsqrtf(r2);
    // phase k r in turns: r * (k / 2 pi) as an exact two-float product plus the
    // low part of k / 2 pi, the integer part removed exactly
    const float th = __fmul_rn(r, a.k2hi);
    const float tl = fmaf(r, a.k2lo, fmaf(r, a.k2hi, -th));
    const float frac = (th - rintf(th)) + tl;
    float sn, cs;
    __sincosf(frac * kTwoPi, &sn, &cs);
    float damp = 1.0f;
    if (a.ka != 0.0f) damp = __expf(-a.ka * r);
    if (HOP == HOP_SRC) {
        // cos_inc P e^{ikr} / r
        float ci = -(vx * d.nx + vy * d.ny + vz * d.nz) * rinv;
        if (a.dst_is_field) ci = 1.0f;
        const float amp = ci * rinv * damp;
        const float er = amp * cs, ei = amp * sn;
        tr = er * A.w - ei * B.w;
        ti = er * B.w + ei * A.w;
    } else {
        const float amp = rinv * kInv4Pi * damp;
        // -e^{ikr}/(4 pi) * (ik/r) + 1/r^2
        float gr = fmaf(amp, fmaf(a.ka, cs, a.kr * sn), rinv * rinv);
        float gi = amp * fmaf(a.ka, sn, -a.kr * cs);
        float wgt;
        if (HOP == HOP_FP) {
            wgt = (vx * B.x + vy * B.y + vz * B.z) * rinv;                     // cos_scat
        } else if (HOP == HOP_F2F) {
            wgt = -(vx * B.x + vy * B.y + vz * B.z) * (vx * d.nx + vy * d.ny + vz * d.nz) * (rinv * rinv);
        } else {
            wgt = (vx * B.x + vy * B.y + vz * B.z) * rinv;                     // cos_scat, cos_inc = 1
        }
        if (HOP != HOP_FP && r < a.rmin) {
            gr = -a.ka * kInv4Pi;
            gi = a.kr * kInv4Pi;
        }
        gr *= wgt;
        gi *= wgt;
        tr = gr * A.w - gi * B.w;
        ti = gr * B.w + gi * A.w;
    }
}

template <int HOP>
__global__ void __launch_bounds__(kTile) k_sum(SumArgs a)
{
    __shared__ float4 sA[kTile];
    __shared__ float4 sB[kTile];
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
        if (!a.mask.flags[(long long)t * a.mask.ndstblocks + blockIdx.x]) continue;  // uniform per CTA
        __syncthreads();
        {
            const int i = t * kTile + tid;
            const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            sA[tid] = i < a.nsrc ? a.srcA[i] : z;
            sB[tid] = i < a.nsrc ? a.srcB[i] : z;
        }
        __syncthreads();
        const int ntile = min(kTile, a.nsrc - t * kTile);
        const int nw = (ntile + 31) >> 5;
        float fr = 0.0f, fi = 0.0f;
        for (int w = 0; w < nw; ++w) {
            uint32_t m = live ? a.mask.bits[(long long)(t * kWordsPerTile + w) * a.mask.pitch + j] : 0u;
            if (HOP == HOP_F2F) {
                // FACET_SELF zero-input rule: when this destination's input is 0
                // the sources of higher facets (its reciprocal partners) drop out
                const int keep = limit - (t * kTile + w * 32);
                m &= keep >= 32 ? 0xffffffffu : (keep <= 0 ? 0u : ((1u << keep) - 1u));
            }
            if (!__any_sync(0xffffffffu, m != 0u)) continue;
#pragma unroll 8
            for (int b = 0; b < 32; ++b) {
                const float4 A = sA[w * 32 + b];
                const float4 B = sB[w * 32 + b];
                float tr, ti;
                pair_term<HOP>(a, A, B, d, tr, ti);
                const bool on = (m >> b) & 1u;
                fr += on ? tr : 0.0f;
                fi += on ? ti : 0.0f;
            }
        }
        accr += (double)fr;
        acci += (double)fi;
    }
    if (live) a.partial[(long long)blockIdx.y * a.ndst + j] = make_double2(accr, acci);
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

void launch_mask(const MaskArgs &a, cudaStream_t s)
{
    if (a.nsrc <= 0 || a.ndst <= 0) return;
    dim3 grid(a.mask.ndstblocks, a.mask.ntiles);
    switch (a.hop) {
    case HOP_SRC: k_mask<HOP_SRC><<<grid, kTile, 0, s>>>(a); break;
    case HOP_FP: k_mask<HOP_FP><<<grid, kTile, 0, s>>>(a); break;
    case HOP_F2F: k_mask<HOP_F2F><<<grid, kTile, 0, s>>>(a); break;
    default: k_mask<HOP_NORESP><<<grid, kTile, 0, s>>>(a); break;
    }
}

void launch_sum(const SumArgs &a, cudaStream_t s)
{
    if (a.nsrc <= 0 || a.ndst <= 0) return;
    dim3 grid(a.mask.ndstblocks, a.nsplit);
    switch (a.hop) {
    case HOP_SRC: k_sum<HOP_SRC><<<grid, kTile, 0, s>>>(a); break;
    case HOP_FP: k_sum<HOP_FP><<<grid, kTile, 0, s>>>(a); break;
    case HOP_F2F: k_sum<HOP_F2F><<<grid, kTile, 0, s>>>(a); break;
    default: k_sum<HOP_NORESP><<<grid, kTile, 0, s>>>(a); break;
    }
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

void launch_mask_export(const MaskView &m, int nsrc, int ndst, uint8_t *out, cudaStream_t s)
{
    const long long total = (long long)ndst * m.nwords;
    if (total > 0) k_mask_export<<<blocks_for(total, 256), 256, 0, s>>>(m, nsrc, ndst, out);
}

}  // namespace sonar
