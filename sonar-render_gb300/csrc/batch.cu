// batch.cu -- many sources, receivers, frequencies and scenes in one launch.
//
// The reference answers "what does receiver p hear when source q radiates"
// one source at a time: load_source_points({q}), ProjectSrcPointsToObjects
// (source -> every fragment cell, src/OptiX.cu:35-110) and
// ProjectTargetToFieldPoints (every fragment -> every field point,
// src/OptiX.cu:112-190).  For S sources and R receivers over N fragments
// that is S * (N + N * R) Green's function evaluations, and the readout
// kernel G(p, n) = A_n cos_scat(n -> p) G(r_pn) is recomputed for every
// source although it does not depend on it.
//
// Here the two hops of one (scene, frequency) item become one complex
// matrix product
//     out[p][q] = sum_n  G(p, n) * Pinc(n, q),
//     Pinc(n, q) = cos_inc(q -> n) e^{ikr}/r  (unit source pressure),
// with both factors materialised tile by tile in shared memory (R + S
// evaluations per fragment instead of S (1 + R)) and contracted on the
// tensor cores:
//   * complex -> real: D (128 x 64) = [[Gr, -Gi], [Gi, Gr]] (128 x 2K) times
//     [Pr; Pi] (2K x 64): rows 0..63 of D are Re out, rows 64..127 Im out;
//   * split BF16: every FP32 value x = hi + lo with hi = bf16(x),
//     lo = bf16(x - hi); D += Ahi Bhi + Ahi Blo + Alo Bhi (relative error of
//     a product about 2^-16), accumulated in FP32 in tensor memory;
//   * tcgen05.mma (kind::f16, M = 128, N = 64, K = 16) issued by one thread,
//     operands in the no-swizzle K-major canonical layout (8-row x 16-byte
//     core matrices), completion tracked by tcgen05.commit on an mbarrier per
//     operand stage (two stages: the next tile is generated while the tensor
//     core consumes the previous one);
//   * the accumulator is read back with tcgen05.ld at the end of each
//     segment (at most kBatchSegChunks chunks, so that an FP32 accumulation
//     never spans more than a few thousand fragments) into FP32 partials
//     that k_batch_reduce adds per item in a fixed order (compensated
//     FP32 summation, the head and tail combined in FP64).
// One persistent launch covers every chunk of every item: CTA b processes a
// contiguous range of the global chunk list (balanced over the grid), cut
// into segments at item boundaries.
//
// Visibility: per fragment one 64-bit word per hop (k_batch_vis: the cosine
// gates and the shadow test of every pair) gates the entries.
#include "sonar_internal.h"
#include "tc05.cuh"

#include <cuda_bf16.h>

#include <cstdint>

namespace sonar {
namespace {

constexpr float kInv4PiB = 0.0795774715459476679f;
constexpr float kTwoPiB = 6.28318530717958647692f;
constexpr int kBatchThreads = 256;
constexpr uint32_t kTmemCols = 64;          // FP32 accumulator: 128 lanes x 64 columns
#ifndef SONAR_GEN_GROUP
#define SONAR_GEN_GROUP 4
#endif
constexpr int kGenGroup = SONAR_GEN_GROUP;  // fragments whose entries are evaluated together

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = 64, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(64 >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);

// ---------------------------------------------------------------- the two kernels of an item
// Phase k r as a fraction of a turn: r * (k / 2 pi) as an exact two-float
// product plus the low part of k / 2 pi, the integer turns removed exactly.
__device__ __forceinline__ void phase(float r, float k2hi, float k2lo, float &sn, float &cs)
{
    const float th = __fmul_rn(r, k2hi);
    const float tl = fmaf(r, k2lo, fmaf(r, k2hi, -th));
    const float frac = (th - rintf(th)) + tl;
    __sincosf(frac * kTwoPiB, &sn, &cs);
}

__device__ __forceinline__ float dist(float vx, float vy, float vz, float &rinv)
{
    // |v|^2 rounded like the reference's dot; r within an ulp of the rounded root
    const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz));
    rinv = rsqrtf(r2);
    const float r0 = r2 * rinv;
    return fmaf(fmaf(-r0, r0, r2), 0.5f * rinv, r0);
}

// Readout entry G(p, n) = A_n cos_scat G(r), G = -e^{ikr}/(4 pi) (ik/r) + 1/r^2
// (src/OptiX.cu:150-186; cos_scat from the fragment's facet normal).
template <bool ATT>
__device__ __forceinline__ float2 readout_entry(const BatchItem &it, float4 f, float4 nf, float3 p)
{
    const float vx = __fsub_rn(p.x, f.x), vy = __fsub_rn(p.y, f.y), vz = __fsub_rn(p.z, f.z);
    float rinv;
    const float r = dist(vx, vy, vz, rinv);
    float sn, cs;
    phase(r, it.k2hi, it.k2lo, sn, cs);
    const float rinv2 = rinv * rinv;
    float gr, gi;
    if (ATT) {
        const float amp = rinv * kInv4PiB * __expf(-it.ka * r);
        gr = fmaf(amp, fmaf(it.ka, cs, it.kr * sn), rinv2);
        gi = amp * fmaf(it.ka, sn, -it.kr * cs);
    } else {
        const float ampk = rinv * it.kr4pi;
        gr = fmaf(ampk, sn, rinv2);
        gi = -ampk * cs;
    }
    const float w = (vx * nf.x + vy * nf.y + vz * nf.z) * rinv * f.w;  // cos_scat A_n
    return make_float2(gr * w, gi * w);
}

// Incident entry Pinc(n, q) = cos_inc e^{ikr} / r at the fragment's
// source-hop centroid (src/OptiX.cu:45-106; unit source pressure).
template <bool ATT>
__device__ __forceinline__ float2 incident_entry(const BatchItem &it, float3 q, float4 s, float4 nf)
{
    const float vx = __fsub_rn(s.x, q.x), vy = __fsub_rn(s.y, q.y), vz = __fsub_rn(s.z, q.z);
    float rinv;
    const float r = dist(vx, vy, vz, rinv);
    float sn, cs;
    phase(r, it.k2hi, it.k2lo, sn, cs);
    float amp = -(vx * nf.x + vy * nf.y + vz * nf.z) * rinv * rinv;  // cos_inc / r
    if (ATT) amp *= __expf(-it.ka * r);
    return make_float2(amp * cs, amp * sn);
}

// Centroid-relative forms of the two entries.  The point is given as
// D = p - c and R = |D| (c: the item's reference point, D rounded from the
// FP64 difference), the fragment as o = f - c and |o|^2 (formed once per
// chunk when its data is staged); r = |D - o| for the amplitude and the
// cosine.  The phase is k r = k R + k (r - R): the entry carries
// e^{ik (r - R)} with r - R = (|o|^2 - 2 o.D) / (r + R), free of
// cancellation, and e^{ik R} -- common to the point's row -- is applied in
// FP64 by the reduction (the host computes it from the FP64 R).  The
// readout's 1/r^2 term carries no phase, so the entry holds it times
// e^{-ik R} (the row's factor E, FP32).
// num = |o|^2 - 2 o.D = r^2 - R^2 (no cancellation); r^2 = R^2 + num is good
// to FP32's relative accuracy, enough for the amplitude, the cosine and r + R.
__device__ __forceinline__ float rel_num(float3 o, float oo, float4 D)
{
    return fmaf(-2.0f, fmaf(o.x, D.x, fmaf(o.y, D.y, o.z * D.z)), oo);
}

// the turns of k (r - R), r - R = num / (r + R)
__device__ __forceinline__ float rel_turns(float r, float R, float num, float k2hi, float k2lo)
{
    const float s = r + R;
    // the quotient from the approximate reciprocal, corrected by one Newton step
    const float y = __fdividef(1.0f, s);
    float dr = num * y;
    dr = fmaf(y, fmaf(-dr, s, num), dr);
    // |k dr| is at most a few tens of turns: the rounding of dr k2hi (half an
    // ulp of it, below 1e-6 turns) is kept, the low part of k / 2 pi added
    const float th = __fmul_rn(dr, k2hi);
    return fmaf(dr, k2lo, th - rintf(th));
}

// f: o and area; nf: the facet normal and |o|^2; D: the receiver's offset
// and R; R2 = R^2; E = e^{-ik R}
template <bool ATT>
__device__ __forceinline__ float2 readout_entry_rel(const BatchItem &it, float4 f, float4 nf, float4 D, float R2,
                                                    float2 E)
{
    const float3 o = make_float3(f.x, f.y, f.z);
    const float num = rel_num(o, nf.w, D);
    const float rinv = rsqrtf(R2 + num);
    const float r = (R2 + num) * rinv;
    const float tu = rel_turns(r, D.w, num, it.k2hi, it.k2lo);
    float sn, cs;
    __sincosf(kTwoPiB * tu, &sn, &cs);
    const float rinv2 = rinv * rinv;
    float gr, gi;
    if (ATT) {
        const float amp = rinv * kInv4PiB * __expf(-it.ka * r);
        gr = fmaf(amp, fmaf(it.ka, cs, it.kr * sn), rinv2 * E.x);
        gi = fmaf(amp, fmaf(it.ka, sn, -it.kr * cs), rinv2 * E.y);
    } else {
        const float ampk = rinv * it.kr4pi;
        gr = fmaf(ampk, sn, rinv2 * E.x);
        gi = fmaf(-ampk, cs, rinv2 * E.y);
    }
    // cos_scat: (p - f).n / r
    const float w = ((D.x - o.x) * nf.x + (D.y - o.y) * nf.y + (D.z - o.z) * nf.z) * rinv * f.w;
    return make_float2(gr * w, gi * w);
}

// s: o and |o|^2 of the source-hop centroid; D: the source's offset and R
template <bool ATT>
__device__ __forceinline__ float2 incident_entry_rel(const BatchItem &it, float4 D, float R2, float4 s, float4 nf)
{
    const float3 o = make_float3(s.x, s.y, s.z);
    const float num = rel_num(o, s.w, D);
    const float rinv = rsqrtf(R2 + num);
    const float r = (R2 + num) * rinv;
    const float tu = rel_turns(r, D.w, num, it.k2hi, it.k2lo);
    float sn, cs;
    __sincosf(kTwoPiB * tu, &sn, &cs);
    // cos_inc / r: -(s - q).n / r^2
    float amp = -((o.x - D.x) * nf.x + (o.y - D.y) * nf.y + (o.z - D.z) * nf.z) * rinv * rinv;
    if (ATT) amp *= __expf(-it.ka * r);
    return make_float2(amp * cs, amp * sn);
}

// The points of one thread for the current item: positions, or (relative
// phase) D, R and the turns of k R.
struct RowPoints {
    float3 prx, psrc;
    float4 Drx, Dsrc;
    float R2rx, R2src;
    float2 Erx;
};

// two FP32 values -> (hi, lo) BF16 pairs packed for a 16-byte row store
__device__ __forceinline__ void split8(const float *x, uint4 &hi, uint4 &lo)
{
    uint32_t h[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const __nv_bfloat16 h0 = __float2bfloat16_rn(x[2 * q]), h1 = __float2bfloat16_rn(x[2 * q + 1]);
        const __nv_bfloat16 l0 = __float2bfloat16_rn(x[2 * q] - __bfloat162float(h0));
        const __nv_bfloat16 l1 = __float2bfloat16_rn(x[2 * q + 1] - __bfloat162float(h1));
        h[q] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
        l[q] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ void st16(uint8_t *p, uint4 v) { *reinterpret_cast<uint4 *>(p) = v; }

// Operand stage of KC fragments: A (128 rows x 2KC) hi and lo, B (64 rows x
// 2KC) hi and lo, each row-group/k-group core matrix 128 bytes; element
// (row, k) of A at (k / 8) * 2048 + row * 16 + (k % 8) * 2.
template <int KC>
struct Stage {
    static constexpr int kA = 128 * 2 * KC * 2;  // bytes of one A copy (hi or lo)
    static constexpr int kB = 64 * 2 * KC * 2;
    static constexpr int kBytes = 2 * kA + 2 * kB;
    static constexpr int kLboA = 128 * 16, kLboB = 64 * 16;
};

// Fragment data of one chunk in shared memory: per fragment the readout
// centroid + area, the source-hop centroid, the facet normal and the
// visibility words (receiver bits x, y; source bits z, w).
template <int KC>
struct ChunkFrags {
    float4 v[KC][4];
};

// Element e (fragment e / 4, field e % 4) of chunk `chunk` of item it, zero
// past the item's fragments (their visibility words are zero, so padded
// fragments contribute nothing).  The relative phase stages it through
// stage_rel once the load has arrived.
__device__ __forceinline__ float4 fetch_frag(const BatchArgs &a, const BatchItem &it, int chunk, int kc, int e)
{
    const int n = chunk * kc + (e >> 2);
    if (n >= it.nfrag) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const long long g = (long long)it.frag0 + n;
    switch (e & 3) {
    case 0: return __ldg(a.frag_pos + g);
    case 1: return __ldg(a.frag_spos + g);
    case 2: return __ldg(a.frag_n + g);
    default: {
        const uint4 w = __ldg(a.vis + g);
        return make_float4(__uint_as_float(w.x), __uint_as_float(w.y), __uint_as_float(w.z), __uint_as_float(w.w));
    }
    }
}

// Relative phase: the centroids as offsets o from the item's reference
// point; the source-hop centroid's |o|^2 in its w, the readout centroid's in
// the normal's w (written by the readout centroid's thread, the normal's
// thread leaving w alone).
template <int KC>
__device__ __forceinline__ void stage_rel(ChunkFrags<KC> &F, const BatchItem &it, int e, float4 v)
{
    float4 *d = &F.v[e >> 2][e & 3];
    const int c = e & 3;
    if (c == 0 || c == 1) {
        v.x -= it.cx;
        v.y -= it.cy;
        v.z -= it.cz;
        const float oo = fmaf(v.x, v.x, fmaf(v.y, v.y, v.z * v.z));
        if (c == 1) v.w = oo;
        else F.v[e >> 2][2].w = oo;
        *d = v;
    } else if (c == 2) {
        d->x = v.x;
        d->y = v.y;
        d->z = v.z;
    } else {
        *d = v;
    }
}

template <int KC, bool ATT, bool REL>
__device__ __forceinline__ void generate(uint8_t *st, const ChunkFrags<KC> &F, const BatchItem &it, int tid,
                                         const RowPoints &pt, bool rx_ok, bool src_ok)
{
    using S = Stage<KC>;
    uint8_t *Ahi = st, *Alo = st + S::kA, *Bhi = st + 2 * S::kA, *Blo = st + 2 * S::kA + S::kB;
    const int row = tid & 63;  // receiver (A) or source (B)
#pragma unroll 1
    for (int q = tid >> 6; q < KC / 8; q += kBatchThreads / 64) {
        float gr[8], gi[8], pr[8], pi[8];
        // groups of kGenGroup fragments: a group's entries are evaluated
        // without branches (independent chains the scheduler interleaves)
        // when any lane of the warp needs one of them, and selected by the
        // lane's bits; a group no lane needs is skipped
#pragma unroll
        for (int j0 = 0; j0 < 8; j0 += kGenGroup) {
            unsigned mrx = 0u, msrc = 0u;
#pragma unroll
            for (int j = j0; j < j0 + kGenGroup; ++j) {
                const float4 w4 = F.v[8 * q + j][3];
                const unsigned wrx = __float_as_uint(row < 32 ? w4.x : w4.y);
                const unsigned wsrc = __float_as_uint(row < 32 ? w4.z : w4.w);
                mrx |= ((wrx >> (row & 31)) & 1u) << (j - j0);
                msrc |= ((wsrc >> (row & 31)) & 1u) << (j - j0);
            }
            if (!rx_ok) mrx = 0u;
            if (!src_ok) msrc = 0u;
#pragma unroll
            for (int j = j0; j < j0 + kGenGroup; ++j) gr[j] = gi[j] = pr[j] = pi[j] = 0.0f;
            if (__any_sync(0xffffffffu, mrx != 0u)) {
#pragma unroll
                for (int j = j0; j < j0 + kGenGroup; ++j) {
                    const float4 *f = F.v[8 * q + j];
                    const float2 v = REL ? readout_entry_rel<ATT>(it, f[0], f[2], pt.Drx, pt.R2rx, pt.Erx)
                                         : readout_entry<ATT>(it, f[0], f[2], pt.prx);
                    const bool on = (mrx >> (j - j0)) & 1u;
                    gr[j] = on ? v.x : 0.0f;
                    gi[j] = on ? v.y : 0.0f;
                }
            }
            if (__any_sync(0xffffffffu, msrc != 0u)) {
#pragma unroll
                for (int j = j0; j < j0 + kGenGroup; ++j) {
                    const float4 *f = F.v[8 * q + j];
                    const float2 v = REL ? incident_entry_rel<ATT>(it, pt.Dsrc, pt.R2src, f[1], f[2])
                                         : incident_entry<ATT>(it, pt.psrc, f[1], f[2]);
                    const bool on = (msrc >> (j - j0)) & 1u;
                    pr[j] = on ? v.x : 0.0f;
                    pi[j] = on ? v.y : 0.0f;
                }
            }
        }
        uint4 h, l;
        const int kr0 = q, ki0 = KC / 8 + q;  // k-groups of the real and imaginary halves
        // A row p:      [ Gr | -Gi ];  A row 64 + p: [ Gi | Gr ]
        split8(gr, h, l);
        st16(Ahi + kr0 * S::kLboA + row * 16, h);
        st16(Alo + kr0 * S::kLboA + row * 16, l);
        st16(Ahi + ki0 * S::kLboA + (64 + row) * 16, h);
        st16(Alo + ki0 * S::kLboA + (64 + row) * 16, l);
        split8(gi, h, l);
        st16(Ahi + kr0 * S::kLboA + (64 + row) * 16, h);
        st16(Alo + kr0 * S::kLboA + (64 + row) * 16, l);
        // -Gi: the same split with every sign bit flipped (exact)
        const uint4 sg = make_uint4(0x80008000u, 0x80008000u, 0x80008000u, 0x80008000u);
        st16(Ahi + ki0 * S::kLboA + row * 16, make_uint4(h.x ^ sg.x, h.y ^ sg.y, h.z ^ sg.z, h.w ^ sg.w));
        st16(Alo + ki0 * S::kLboA + row * 16, make_uint4(l.x ^ sg.x, l.y ^ sg.y, l.z ^ sg.z, l.w ^ sg.w));
        // B row q_src: [ Pr | Pi ]
        split8(pr, h, l);
        st16(Bhi + kr0 * S::kLboB + row * 16, h);
        st16(Blo + kr0 * S::kLboB + row * 16, l);
        split8(pi, h, l);
        st16(Bhi + ki0 * S::kLboB + row * 16, h);
        st16(Blo + ki0 * S::kLboB + row * 16, l);
    }
}

template <int KC, bool ATT, bool REL>
__global__ void __launch_bounds__(kBatchThreads, 1) k_batch(BatchArgs a)
{
    using S = Stage<KC>;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tmem_base;
    __shared__ ChunkFrags<KC> sfrag[2];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tmem_alloc(&tmem_base, kTmemCols);
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    const int row = tid & 63;
    const bool rx_ok = row < a.nrx, src_ok = row < a.nsrc;
    const float4 rx4 = rx_ok ? a.rx[row] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float4 sq4 = src_ok ? a.src[row] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    RowPoints pt{};
    pt.prx = make_float3(rx4.x, rx4.y, rx4.z);
    pt.psrc = make_float3(sq4.x, sq4.y, sq4.z);
    // the relative phase's per-item point data of this thread's row
    auto load_rel = [&](int item) {
        if (!REL) return;
        const size_t q = (size_t)item * kBatchMaxPoints + row;
        pt.Drx = __ldg(a.rel_rx + q);
        pt.Dsrc = __ldg(a.rel_src + q);
        pt.Erx = __ldg(a.rel_rx_e + q);
        pt.R2rx = pt.Drx.w * pt.Drx.w;
        pt.R2src = pt.Dsrc.w * pt.Dsrc.w;
    };
    const uint32_t sbase = smem_u32(smem);
    const bool loader = tid < 4 * KC;  // thread tid stages element tid of each chunk's fragment data
    // this CTA's chunks: segments [g0, g1), chunk cc of segment sg
    const int g0 = a.cta_seg[blockIdx.x], g1 = a.cta_seg[blockIdx.x + 1];
    int sg = g0, cc = 0;
    int4 seg = make_int4(0, 0, 0, 0);
    BatchItem it{};
    if (sg < g1) {
        seg = a.segs[sg];
        it = a.items[seg.x];
        load_rel(seg.x);
        if (loader) {
            const float4 v = fetch_frag(a, it, seg.y, KC, tid);
            if (REL) stage_rel(sfrag[0], it, tid, v);
            else sfrag[0].v[tid >> 2][tid & 3] = v;
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    uint32_t commits0 = 0, commits1 = 0;  // commits issued on each stage's barrier
    int last_st = -1;                     // stage of the most recent commit
    int local = 0;                        // chunks this CTA has generated
    bool ok = true;
    while (sg < g1 && ok) {
        const int st = local & 1;
        // the next chunk: its fragment data is loaded now and staged after this chunk's generation
        int nsg = sg, ncc = cc + 1;
        int4 nseg = seg;
        BatchItem nit = it;
        if (ncc >= seg.z) {
            nsg = sg + 1;
            ncc = 0;
            if (nsg < g1) {
                nseg = a.segs[nsg];
                nit = a.items[nseg.x];
            }
        }
        float4 nf = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (loader && nsg < g1) nf = fetch_frag(a, nit, nseg.y + ncc, KC, tid);
        // the operand stage is free once the MMAs that read it (two chunks back) completed
        if (local >= 2) {
            const uint32_t c = st ? commits1 : commits0;
            const bool done = mbar_wait(&bar[st], (c - 1) & 1u);
            ok = __syncthreads_and(done);
            if (!ok) break;
        }
        generate<KC, ATT, REL>(smem + st * S::kBytes, sfrag[st], it, tid, pt, rx_ok, src_ok);
        if (loader) {
            if (REL) stage_rel(sfrag[st ^ 1], nit, tid, nf);
            else sfrag[st ^ 1].v[tid >> 2][tid & 3] = nf;
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t sA = sbase + st * S::kBytes, sB = sA + 2 * S::kA;
#pragma unroll
            for (int ks = 0; ks < 2 * KC / 16; ++ks) {
                const uint64_t ahi = sdesc(sA + ks * 2 * S::kLboA, S::kLboA, 128);
                const uint64_t alo = sdesc(sA + S::kA + ks * 2 * S::kLboA, S::kLboA, 128);
                const uint64_t bhi = sdesc(sB + ks * 2 * S::kLboB, S::kLboB, 128);
                const uint64_t blo = sdesc(sB + S::kB + ks * 2 * S::kLboB, S::kLboB, 128);
                mma_bf16(tmem, ahi, bhi, kIdesc, (cc > 0 || ks > 0) ? 1u : 0u);
                mma_bf16(tmem, ahi, blo, kIdesc, 1u);
                mma_bf16(tmem, alo, bhi, kIdesc, 1u);
            }
            mma_commit(&bar[st]);
        }
        if (st) ++commits1;
        else ++commits0;
        last_st = st;
        ++local;
        if (cc + 1 == seg.z) {
            // ---- segment end: the accumulator -> FP32 partial [128][64]
            const uint32_t c = st ? commits1 : commits0;
            const bool done = mbar_wait(&bar[st], (c - 1) & 1u);
            ok = __syncthreads_and(done);
            if (!ok) break;
            tc_fence_after();
            const int quarter = warp & 3, half = warp >> 2;
            const int drow = quarter * 32 + lane;
            float v[32];
            const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(half * 32);
            tmem_ld16(taddr, v);
            tmem_ld16(taddr + 16, v + 16);
            float4 *out = reinterpret_cast<float4 *>(a.partial + ((long long)sg * 128 + drow) * 64 + half * 32);
#pragma unroll
            for (int q = 0; q < 8; ++q) out[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            tc_fence_before();
            __syncthreads();
        }
        if (nsg != sg && nsg < g1 && nseg.x != seg.x) load_rel(nseg.x);
        sg = nsg;
        cc = ncc;
        seg = nseg;
        it = nit;
    }
    // After a timed-out wait, MMAs committed earlier may still be writing the
    // accumulator and reading the operand stages.  tcgen05 operations of one
    // thread complete in issue order, so once the most recent commit has
    // arrived nothing is in flight: wait for it (bounded again) before the
    // tensor memory is released.  If that wait runs out as well, the tensor
    // memory is left allocated rather than released under a running MMA, and
    // the status says so (2).
    bool drained = true;
    if (!ok && last_st >= 0) {
        const uint32_t c = last_st ? commits1 : commits0;
        drained = __syncthreads_and(mbar_wait(&bar[last_st], (c - 1) & 1u));
    }
    if (!ok && tid == 0) atomicExch(a.status, drained ? 1 : 2);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0 && drained) tmem_dealloc(tmem, kTmemCols);
}

// Error-free sum of two FP32 values (Knuth's two-sum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// out[item][p][q] = sum over the item's segments in a fixed order, times
// the relative phase's row factors e^{ik R} of receiver p and source q when
// given.  The FP32 partials are added by compensated summation (a head and
// the sum of the two-sum error terms, all FP32: FP64 arithmetic is scarce on
// this part), the two words combined in FP64: the sum is exact to about
// 2^-46 of its terms' magnitude, as an FP64 accumulation would be for this
// many terms.  Grid (items, entry chunks of 256): one thread per (receiver,
// source) entry.
__global__ void __launch_bounds__(256) k_batch_reduce(const float *partial, const int *item_seg_off,
                                                      const int *item_segs, int nrx, int nsrc, const double2 *erx,
                                                      const double2 *esrc, double2 *out)
{
    const int item = blockIdx.x;
    const int e = blockIdx.y * 256 + threadIdx.x;
    if (e >= nrx * nsrc) return;
    const int s0 = item_seg_off[item], s1 = item_seg_off[item + 1];
    const int p = e / nsrc, q = e - p * nsrc;
    float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
    for (int s = s0; s < s1; ++s) {
        const float *P = partial + (long long)item_segs[s] * 128 * 64;
        float e;
        two_sum(rh, __ldg(P + p * 64 + q), rh, e);
        rl += e;
        two_sum(ih, __ldg(P + (64 + p) * 64 + q), ih, e);
        il += e;
    }
    double re = (double)rh + (double)rl, im = (double)ih + (double)il;
    if (erx) {
        const double2 a = erx[item * kBatchMaxPoints + p], b = esrc[item * kBatchMaxPoints + q];
        const double er = a.x * b.x - a.y * b.y, ei = a.x * b.y + a.y * b.x;
        const double t = re * er - im * ei;
        im = re * ei + im * er;
        re = t;
    }
    out[(long long)item * nrx * nsrc + e] = make_double2(re, im);
}

}  // namespace

size_t batch_smem_bytes(int kc)
{
    return kc == 64 ? (size_t)2 * Stage<64>::kBytes
                    : kc == 32 ? (size_t)2 * Stage<32>::kBytes : (size_t)2 * Stage<16>::kBytes;
}

namespace {
template <int KC>
cudaError_t prepare_k()
{
    const int sm = (int)batch_smem_bytes(KC);
    cudaError_t e = cudaFuncSetAttribute(k_batch<KC, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch<KC, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch<KC, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch<KC, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    return e;
}
}  // namespace

cudaError_t batch_prepare()
{
    cudaError_t e = prepare_k<32>();
    if (e == cudaSuccess) e = prepare_k<64>();
    if (e == cudaSuccess) e = prepare_k<16>();
    return e;
}

namespace {
template <int KC>
void launch_k(const BatchArgs &a, int grid, size_t sm, bool att, bool rel, cudaStream_t s)
{
    if (att) {
        if (rel) k_batch<KC, true, true><<<grid, kBatchThreads, sm, s>>>(a);
        else k_batch<KC, true, false><<<grid, kBatchThreads, sm, s>>>(a);
    } else {
        if (rel) k_batch<KC, false, true><<<grid, kBatchThreads, sm, s>>>(a);
        else k_batch<KC, false, false><<<grid, kBatchThreads, sm, s>>>(a);
    }
}
}  // namespace

void launch_batch(const BatchArgs &a, int kc, int grid, bool att, cudaStream_t s)
{
    const size_t sm = batch_smem_bytes(kc);
    if (grid <= 0) return;
    const bool rel = a.rel_rx != nullptr;
    if (kc == 64) launch_k<64>(a, grid, sm, att, rel, s);
    else if (kc == 16) launch_k<16>(a, grid, sm, att, rel, s);
    else launch_k<32>(a, grid, sm, att, rel, s);
}

void launch_batch_reduce(const float *partial, const int *item_seg_off, const int *item_segs, int nitems, int nrx,
                         int nsrc, const double2 *erx, const double2 *esrc, double2 *out, cudaStream_t s)
{
    if (nitems > 0)
        k_batch_reduce<<<dim3(nitems, (nrx * nsrc + 255) / 256), 256, 0, s>>>(partial, item_seg_off, item_segs, nrx,
                                                                            nsrc, erx, esrc, out);
}

}  // namespace sonar
