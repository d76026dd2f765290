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
//     that k_batch_reduce adds per item in a fixed order in FP64.
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
// fragments contribute nothing).
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

template <int KC, bool ATT>
__device__ __forceinline__ void generate(uint8_t *st, const ChunkFrags<KC> &F, const BatchItem &it, int tid,
                                         float3 prx, bool rx_ok, float3 psrc, bool src_ok)
{
    using S = Stage<KC>;
    uint8_t *Ahi = st, *Alo = st + S::kA, *Bhi = st + 2 * S::kA, *Blo = st + 2 * S::kA + S::kB;
    const int row = tid & 63;  // receiver (A) or source (B)
#pragma unroll 1
    for (int q = tid >> 6; q < KC / 8; q += kBatchThreads / 64) {
        float gr[8], gi[8], pr[8], pi[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float4 *f = F.v[8 * q + j];
            const float4 w4 = f[3];
            const unsigned wrx = __float_as_uint(row < 32 ? w4.x : w4.y);
            const unsigned wsrc = __float_as_uint(row < 32 ? w4.z : w4.w);
            gr[j] = gi[j] = pr[j] = pi[j] = 0.0f;
            if (rx_ok && ((wrx >> (row & 31)) & 1u)) {
                const float2 v = readout_entry<ATT>(it, f[0], f[2], prx);
                gr[j] = v.x;
                gi[j] = v.y;
            }
            if (src_ok && ((wsrc >> (row & 31)) & 1u)) {
                const float2 v = incident_entry<ATT>(it, psrc, f[1], f[2]);
                pr[j] = v.x;
                pi[j] = v.y;
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

template <int KC, bool ATT>
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
    const float3 prx = make_float3(rx4.x, rx4.y, rx4.z), psrc = make_float3(sq4.x, sq4.y, sq4.z);
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
        if (loader) sfrag[0].v[tid >> 2][tid & 3] = fetch_frag(a, it, seg.y, KC, tid);
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
        generate<KC, ATT>(smem + st * S::kBytes, sfrag[st], it, tid, prx, rx_ok, psrc, src_ok);
        if (loader) sfrag[st ^ 1].v[tid >> 2][tid & 3] = nf;
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

// out[item][p][q] = sum over the item's segments, fixed order, FP64.  Grid
// (items, entry chunks of 256): one thread per (receiver, source) entry.
__global__ void __launch_bounds__(256) k_batch_reduce(const float *partial, const int *item_seg_off,
                                                      const int *item_segs, int nrx, int nsrc, double2 *out)
{
    const int item = blockIdx.x;
    const int e = blockIdx.y * 256 + threadIdx.x;
    if (e >= nrx * nsrc) return;
    const int s0 = item_seg_off[item], s1 = item_seg_off[item + 1];
    const int p = e / nsrc, q = e - p * nsrc;
    double re = 0.0, im = 0.0;
    for (int s = s0; s < s1; ++s) {
        const float *P = partial + (long long)item_segs[s] * 128 * 64;
        re += (double)__ldg(P + p * 64 + q);
        im += (double)__ldg(P + (64 + p) * 64 + q);
    }
    out[(long long)item * nrx * nsrc + e] = make_double2(re, im);
}

}  // namespace

size_t batch_smem_bytes(int kc)
{
    return kc == 64 ? (size_t)2 * Stage<64>::kBytes
                    : kc == 32 ? (size_t)2 * Stage<32>::kBytes : (size_t)2 * Stage<16>::kBytes;
}

cudaError_t batch_prepare()
{
    cudaError_t e = cudaFuncSetAttribute(k_batch<32, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)batch_smem_bytes(32));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch<32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)batch_smem_bytes(32));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch<64, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)batch_smem_bytes(64));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch<64, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)batch_smem_bytes(64));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch<16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)batch_smem_bytes(16));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch<16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)batch_smem_bytes(16));
    return e;
}

void launch_batch(const BatchArgs &a, int kc, int grid, bool att, cudaStream_t s)
{
    const size_t sm = batch_smem_bytes(kc);
    if (grid <= 0) return;
    if (kc == 64) {
        if (att) k_batch<64, true><<<grid, kBatchThreads, sm, s>>>(a);
        else k_batch<64, false><<<grid, kBatchThreads, sm, s>>>(a);
    } else if (kc == 16) {
        if (att) k_batch<16, true><<<grid, kBatchThreads, sm, s>>>(a);
        else k_batch<16, false><<<grid, kBatchThreads, sm, s>>>(a);
    } else {
        if (att) k_batch<32, true><<<grid, kBatchThreads, sm, s>>>(a);
        else k_batch<32, false><<<grid, kBatchThreads, sm, s>>>(a);
    }
}

void launch_batch_reduce(const float *partial, const int *item_seg_off, const int *item_segs, int nitems, int nrx,
                         int nsrc, double2 *out, cudaStream_t s)
{
    if (nitems > 0)
        k_batch_reduce<<<dim3(nitems, (nrx * nsrc + 255) / 256), 256, 0, s>>>(partial, item_seg_off, item_segs, nrx,
                                                                            nsrc, out);
}

}  // namespace sonar
