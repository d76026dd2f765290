// noalloc.cu -- fragment -> field-point readout that allocates no memory.
//
// Who needs it: callers that cannot call cudaMalloc while the readout runs.
// Typical cases are a host framework that owns every device byte through its
// own pool and forbids other allocations, a real-time or embedded host that
// allocates only at start-up, and code that must not trigger the implicit
// synchronisation a cudaMalloc/cudaFree can cause.  Such a caller keeps its
// own device buffers for the inputs and the outputs and calls
// sonar_readout_noalloc with them.
//
// What it computes: the FIELD_POINTS sum of ProjectTargetToFieldPoints
// (the reference's projectFacetToFieldPoints, src/OptiX.cu:112-190), for
// fragments and field points given as plain device arrays, without shadowing
// (every fragment sees every field point, subject to the area gate
// A > 1e-6 and the cos_scat >= 1e-6 gate, both decided with the reference's
// FP32 rounding as in the library's interaction masks).  For scenes where
// nothing occludes the readout -- flat or convex targets seen from outside --
// the result equals the library's own readout.
//
// Scratch: the only working memory is the per-split partial sums, held in a
// file-scope __device__ array of kMaxPartials double2 (8 MiB).  Every GPU that
// loads this library reserves that array until the process exits.  Its
// device address is looked up on the first call made in each CUDA context
// (cudaGetSymbolAddress, with that device current) and cached under the
// context's unique id: a context that is destroyed and re-created (for
// example by cudaDeviceReset) gets the array at a new address, which the
// next call looks up again.  Make the first call in a context before any
// stream capture begins.  Every call reuses the same array, which keeps the
// previous call's contents: the sum kernel overwrites every partial it later
// reads, so nothing needs clearing, but two calls whose work overlaps on the
// GPU (for example on two streams) race on the array and give wrong results.
#include <climits>
#include <cstdint>
#include <cstdio>

#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/sonar_render.h"

namespace {

constexpr int kMaxPartials = 1 << 19;  // double2 entries: 8 MiB
constexpr int kBlock = 256;
constexpr int kMaxDevices = 64;
constexpr int kMaxSplit = 64;

static __device__ __align__(256) double2 g_noalloc_partials[kMaxPartials];

// host-side cache of the array's device address, one entry per device: the
// address and the unique id of the context it was looked up in
struct PartialsAddr {
    unsigned long long ctx_id;
    double2 *ptr;
};
PartialsAddr g_partials_addr[kMaxDevices] = {};

constexpr float kInv4Pi = 0.0795774715459476679f;
constexpr float kTwoPi = 6.28318530717958647692f;

__device__ __forceinline__ float dot3_rn(float ax, float ay, float az, float bx, float by, float bz)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// cos_scat >= 1e-6 (src/OptiX.cu:155-160) decided as the reference rounds it:
// the contracted estimate est decides outside the band [0, 2e-6] (it is
// within a few ulp of the true cosine); inside the band the reference's
// expression is evaluated with every operation rounded separately --
// r = sqrt(v.v), u = v * (1 / r), dot(u, n).
__device__ __forceinline__ bool cos_scat_gate(float est, float vx, float vy, float vz, float nx, float ny, float nz)
{
    if (est > 2e-6f) return true;
    if (est < 0.0f) return false;
    const float r = __fsqrt_rn(dot3_rn(vx, vy, vz, vx, vy, vz));
    const float inv = __frcp_rn(r);
    return !(dot3_rn(__fmul_rn(vx, inv), __fmul_rn(vy, inv), __fmul_rn(vz, inv), nx, ny, nz) < 1e-6f);
}

// One CTA: 256 field points x a range of 256-fragment tiles.  Same arithmetic
// as the library's readout sum kernel; the area and cos_scat gates are
// evaluated inline instead of being read from an interaction mask.
__global__ void __launch_bounds__(kBlock)
    k_readout_noalloc(const float4 *__restrict__ pos, const float4 *__restrict__ nrm,
                      const double2 *__restrict__ pres, int nsrc, const float4 *__restrict__ pts, int ndst, float kr,
                      float ka, float k2hi, float k2lo, int ntiles, int tiles_per_split, double2 *partials)
{
    __shared__ float4 sA[kBlock];
    __shared__ float4 sB[kBlock];
    const int tid = threadIdx.x;
    const int j = blockIdx.x * kBlock + tid;
    const bool live = j < ndst;
    float px = 0.0f, py = 0.0f, pz = 0.0f;
    if (live) {
        const float4 p = pts[j];
        px = p.x; py = p.y; pz = p.z;
    }
    double accr = 0.0, acci = 0.0;
    const int t0 = blockIdx.y * tiles_per_split;
    const int t1 = min(t0 + tiles_per_split, ntiles);
    for (int t = t0; t < t1; ++t) {
        __syncthreads();
        {
            const int i = t * kBlock + tid;
            float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f), b = a;
            if (i < nsrc) {
                const float4 q = pos[i];
                if (q.w > 1e-6f) {  // area gate, src/OptiX.cu:138
                    const float4 n = nrm[i];
                    const double2 w = pres[i];
                    a = make_float4(q.x, q.y, q.z, (float)((double)q.w * w.x));
                    b = make_float4(n.x, n.y, n.z, (float)((double)q.w * w.y));
                }
            }
            sA[tid] = a;
            sB[tid] = b;
        }
        __syncthreads();
        const int nt = min(kBlock, nsrc - t * kBlock);
        float fr = 0.0f, fi = 0.0f;
        for (int q = 0; q < nt; ++q) {
            const float4 A = sA[q], B = sB[q];
            const float vx = __fsub_rn(px, A.x), vy = __fsub_rn(py, A.y), vz = __fsub_rn(pz, A.z);
            const float r2 = dot3_rn(vx, vy, vz, vx, vy, vz);
            const float r = __fsqrt_rn(r2);
            const float rinv = rsqrtf(r2);
            const float cs = (vx * B.x + vy * B.y + vz * B.z) * rinv;  // cos_scat, src/OptiX.cu:155
            const float th = __fmul_rn(r, k2hi);
            const float tl = fmaf(r, k2lo, fmaf(r, k2hi, -th));
            const float frac = (th - rintf(th)) + tl;
            float sn, cn;
            __sincosf(frac * kTwoPi, &sn, &cn);
            float amp = rinv * kInv4Pi;
            if (ka != 0.0f) amp *= __expf(-ka * r);
            // -e^{ikr}/(4 pi) (ik/r) + 1/r^2  (src/OptiX.cu:182)
            const float gr = fmaf(amp, fmaf(ka, cn, kr * sn), rinv * rinv) * cs;
            const float gi = amp * fmaf(ka, sn, -kr * cn) * cs;
            const bool on = live && (A.w != 0.0f || B.w != 0.0f) && cos_scat_gate(cs, vx, vy, vz, B.x, B.y, B.z);
            fr += on ? gr * A.w - gi * B.w : 0.0f;
            fi += on ? gr * B.w + gi * A.w : 0.0f;
        }
        accr += (double)fr;
        acci += (double)fi;
    }
    if (live) partials[(long long)blockIdx.y * ndst + j] = make_double2(accr, acci);
}

__global__ void k_readout_noalloc_finalize(const double2 *partials, int nsplit, int ndst, double2 *out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ndst) return;
    double sr = 0.0, si = 0.0;
    for (int k = 0; k < nsplit; ++k) {
        const double2 v = partials[(long long)k * ndst + j];
        sr += v.x;
        si += v.y;
    }
    double2 o = out[j];
    o.x += sr;
    o.y += si;
    out[j] = o;
}

// Unique id of the calling thread's current CUDA context (0 when none is
// current), through the driver entry points the runtime hands out (the
// library does not link the driver library itself).
unsigned long long current_context_id()
{
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    if (!get_current || !get_id) {
        void *f0 = nullptr, *f1 = nullptr;
        cudaDriverEntryPointQueryResult q0, q1;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
            return 0;
        get_current = (GetCurrent)f0;
        get_id = (GetId)f1;
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the partials array in the current context, looked up
// on the first call made in that context.
int partials_for_current_device(double2 **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SONAR_NOALLOC_ECUDA;
    unsigned long long id = current_context_id();
    PartialsAddr &c = g_partials_addr[dev];
    if (id == 0 || c.ctx_id != id || !c.ptr) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);  // makes the context current
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "sonar_readout_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return SONAR_NOALLOC_ECUDA;
        }
        id = current_context_id();
        c.ctx_id = id;  // 0 (no id available): looked up again on every call
        c.ptr = (double2 *)p;
    }
    *out = c.ptr;
    return 0;
}

bool misaligned16(const void *p) { return ((uintptr_t)p & 15u) != 0; }

}  // namespace

extern "C" int sonar_readout_noalloc(const float *frag_pos, const float *frag_normal, const double *frag_pressure,
                                     int n_frag, const float *points, int n_points, float k_re, float k_im,
                                     double *out, void *stream)
{
    if (n_frag < 0 || n_points < 0 || n_frag > INT_MAX - kBlock) return SONAR_NOALLOC_EINVAL;
    if (n_points > SONAR_NOALLOC_MAX_POINTS) {
        fprintf(stderr, "sonar_readout_noalloc: %d field points exceed the maximum of %d\n", n_points,
                SONAR_NOALLOC_MAX_POINTS);
        return SONAR_NOALLOC_ETOOBIG;
    }
    if (n_points == 0) return 0;
    if (!points || !out || (n_frag > 0 && (!frag_pos || !frag_normal || !frag_pressure))) return SONAR_NOALLOC_EINVAL;
    // the kernels read float4 / double2 vectors: every buffer 16-byte aligned
    if (misaligned16(points) || misaligned16(out) ||
        (n_frag > 0 && (misaligned16(frag_pos) || misaligned16(frag_normal) || misaligned16(frag_pressure)))) {
        fprintf(stderr, "sonar_readout_noalloc: every buffer must start on a 16-byte boundary\n");
        return SONAR_NOALLOC_EINVAL;
    }
    // an error left pending by the caller's own work is reported, not taken over
    const cudaError_t prior = cudaPeekAtLastError();
    if (prior != cudaSuccess) {
        fprintf(stderr, "sonar_readout_noalloc: a CUDA error is already pending: %s\n", cudaGetErrorString(prior));
        return SONAR_NOALLOC_ECUDA;
    }
    double2 *partials = nullptr;
    const int st = partials_for_current_device(&partials);
    if (st != 0) return st;
    if (n_frag == 0) return 0;
    cudaStream_t s = (cudaStream_t)stream;
    const int ntiles = (n_frag + kBlock - 1) / kBlock;
    const int nblocks = (n_points + kBlock - 1) / kBlock;
    // source splits: enough CTAs to fill the GPU, bounded by the scratch size
    int nsplit = (2432 + nblocks - 1) / nblocks;
    nsplit = nsplit < 1 ? 1 : nsplit;
    nsplit = nsplit > kMaxSplit ? kMaxSplit : nsplit;
    nsplit = nsplit > ntiles ? ntiles : nsplit;
    const int fit = kMaxPartials / n_points;
    nsplit = nsplit > fit ? fit : nsplit;
    const int tps = (ntiles + nsplit - 1) / nsplit;
    nsplit = (ntiles + tps - 1) / tps;
    const double k2 = (double)k_re / (2.0 * 3.14159265358979323846);
    const float k2hi = (float)k2, k2lo = (float)(k2 - (double)k2hi);
    k_readout_noalloc<<<dim3(nblocks, nsplit), kBlock, 0, s>>>(
        (const float4 *)frag_pos, (const float4 *)frag_normal, (const double2 *)frag_pressure, n_frag,
        (const float4 *)points, n_points, k_re, k_im, k2hi, k2lo, ntiles, tps, partials);
    k_readout_noalloc_finalize<<<nblocks, kBlock, 0, s>>>(partials, nsplit, n_points, (double2 *)out);
    const cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "sonar_readout_noalloc: launch failed: %s\n", cudaGetErrorString(e));
        return SONAR_NOALLOC_ECUDA;
    }
    return 0;
}
