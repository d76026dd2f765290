// select.cu -- choice of the low-rank bounce blocks, on the device.
//
// The compressed bounce picks candidate blocks from the interaction mask's
// block classes, keeps those the admissibility network proposes (or all of
// them), gives each a rank cap and a column range of the factor arrays, and
// after the cross approximation lists the accepted blocks per destination
// tile (J) and per source tile (I) for the low-rank apply.  Every list is
// built by row-wise compaction: one CTA owns one row (or column) of the
// 256 x 256 block grid and scans it in tile order, so every output keeps the
// order of a host loop "for J, for I < J" and the results are deterministic.
#include "sonar_internal.h"

namespace sonar {
namespace {

constexpr int kSelThreads = 256;

// Exclusive block-wide scan of one int per thread (256 threads); returns
// the prefix and the block total.
__device__ __forceinline__ int block_scan(int v, int &total, int *sw)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();  // sw is free (the previous call's readers are past this point)
    if (lane == 31) sw[warp] = x;
    __syncthreads();
    int base = 0;
    total = 0;
#pragma unroll
    for (int w = 0; w < kSelThreads / 32; ++w) {
        const int s = sw[w];
        if (w < warp) base += s;
        total += s;
    }
    return base + x - v;
}

__device__ __forceinline__ bool cand_pred(const uint8_t *flags, int nb, int I, int J, int select, float eta,
                                          const float4 *cen, uint8_t &f)
{
    f = flags[(long long)I * nb + J];
    if (f == kFlagNone) return false;
    if (select != 0) return true;
    if (f != kFlagAll) return false;
    const float4 a = cen[I], b = cen[J];
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return sqrtf(dx * dx + dy * dy + dz * dz) > eta * (a.w + b.w);
}

// candidates of row J: I < min(J, nt) with a non-empty class (select 0:
// class ALL and separated by more than eta (r_I + r_J))
__global__ void __launch_bounds__(kSelThreads) k_cand_count(const uint8_t *flags, int nt, int nb, int select,
                                                            float eta, const float4 *cen, int *cnt)
{
    __shared__ int sw[kSelThreads / 32];
    const int J = blockIdx.x, n = min(J, nt);
    int c = 0;
    for (int I = threadIdx.x; I < n; I += kSelThreads) {
        uint8_t f;
        c += cand_pred(flags, nb, I, J, select, eta, cen, f) ? 1 : 0;
    }
    int tot;
    block_scan(c, tot, sw);
    if (threadIdx.x == 0) cnt[J] = tot;
}

__global__ void __launch_bounds__(kSelThreads) k_cand_fill(const uint8_t *flags, int nt, int nb, int select,
                                                           float eta, const float4 *cen, const int *off,
                                                           int2 *blocks, uint8_t *cls)
{
    __shared__ int sw[kSelThreads / 32];
    const int J = blockIdx.x, n = min(J, nt);
    int base = off[J];
    for (int I0 = 0; I0 < n; I0 += kSelThreads) {
        const int I = I0 + threadIdx.x;
        uint8_t f = 0;
        const bool p = I < n && cand_pred(flags, nb, I, J, select, eta, cen, f);
        int tot;
        const int pre = block_scan(p ? 1 : 0, tot, sw);
        if (p) {
            blocks[base + pre] = make_int2(I, J);
            cls[base + pre] = f;
        }
        base += tot;
    }
}

// Exclusive scan of n ints (one CTA); out[n] = total.
__global__ void __launch_bounds__(kSelThreads) k_scan(const int *in, int n, int *out)
{
    __shared__ int sw[kSelThreads / 32];
    int carry = 0;
    for (int i0 = 0; i0 < n; i0 += kSelThreads) {
        const int i = i0 + threadIdx.x;
        const int v = i < n ? in[i] : 0;
        int tot;
        const int pre = block_scan(v, tot, sw);
        if (i < n) out[i] = carry + pre;
        carry += tot;
    }
    if (threadIdx.x == 0) out[n] = carry;
}

// rank cap from the network's prediction of log2(1 + rank)
__device__ __forceinline__ int cap_of(const float *pred, int c, float cut, int rmax, bool &keep)
{
    if (!pred) {
        keep = true;
        return rmax;
    }
    const float p = pred[c];
    keep = p < cut;
    const float r = exp2f(p) - 1.0f;
    return max(4, min(rmax, (int)ceilf(1.5f * r) + 4));
}

// kept blocks and their caps per candidate row J; a block with an
// interpolation level is kept whatever the network predicts (its node count
// does not depend on the cross approximation's rank)
// factor columns a kept block reserves: its rank cap, or an interpolated
// block's node entries
__device__ __forceinline__ int cols_of(const uint8_t *clev, int c, int cap)
{
    const int L = clev ? clev[c] : 0;
    return L ? ip_columns(L) : cap;
}

__global__ void __launch_bounds__(kSelThreads) k_keep_count(const int *coff, const float *pred, float cut, int rmax,
                                                            const uint8_t *clev, int *kcnt, int *ksum)
{
    __shared__ int sw[kSelThreads / 32];
    const int J = blockIdx.x, c0 = coff[J], c1 = coff[J + 1];
    int k = 0, s = 0;
    for (int c = c0 + threadIdx.x; c < c1; c += kSelThreads) {
        bool keep;
        const int cap = cap_of(pred, c, cut, rmax, keep);
        keep = keep || (clev && clev[c]);
        if (keep) {
            k += 1;
            s += cols_of(clev, c, cap);
        }
    }
    int tk, ts;
    block_scan(k, tk, sw);
    block_scan(s, ts, sw);
    if (threadIdx.x == 0) {
        kcnt[J] = tk;
        ksum[J] = ts;
    }
}

__global__ void __launch_bounds__(kSelThreads) k_keep_fill(const int *coff, const float *pred, float cut, int rmax,
                                                           const int2 *cblocks, const uint8_t *ccls,
                                                           const uint8_t *clev, const int *koff, const int *kcoloff,
                                                           int2 *ab, uint8_t *acls, int *acap, long long *aoff,
                                                           int *kmap, uint8_t *alev)
{
    __shared__ int sw[kSelThreads / 32];
    const int J = blockIdx.x, c0 = coff[J], c1 = coff[J + 1];
    int kbase = koff[J], cbase = kcoloff[J];
    for (int i0 = c0; i0 < c1; i0 += kSelThreads) {
        const int c = i0 + threadIdx.x;
        bool keep = false;
        int cap = 0, cols = 0;
        if (c < c1) {
            cap = cap_of(pred, c, cut, rmax, keep);
            keep = keep || (clev && clev[c]);
            cols = cols_of(clev, c, cap);
        }
        int tk, tc;
        const int pk = block_scan(keep ? 1 : 0, tk, sw);
        const int pc = block_scan(keep ? cols : 0, tc, sw);
        if (keep) {
            const int k = kbase + pk;
            const int L = clev ? clev[c] : 0;
            ab[k] = cblocks[c];
            acls[k] = ccls[c];
            acap[k] = L ? 0 : cap;  // interpolated blocks: no cross approximation
            aoff[k] = (long long)(cbase + pc);
            kmap[k] = c;
            if (alev) alev[k] = (uint8_t)L;
        }
        kbase += tk;
        cbase += tc;
    }
}

// kept blocks of row J by kind: interpolated (level > 0) and cross-approximated
__global__ void __launch_bounds__(kSelThreads) k_split_count(const int *koff, const uint8_t *alev, int *icnt)
{
    __shared__ int sw[kSelThreads / 32];
    const int J = blockIdx.x, k0 = koff[J], k1 = koff[J + 1];
    int c = 0;
    for (int k = k0 + threadIdx.x; k < k1; k += kSelThreads) c += alev[k] ? 1 : 0;
    int tot;
    block_scan(c, tot, sw);
    if (threadIdx.x == 0) icnt[J] = tot;
}

__global__ void __launch_bounds__(kSelThreads) k_split_fill(const int *koff, const uint8_t *alev, const int *ioff,
                                                            int *aca_list, int *ip_list)
{
    __shared__ int sw[kSelThreads / 32];
    const int J = blockIdx.x, k0 = koff[J], k1 = koff[J + 1];
    int ib = ioff[J], ab = k0 - ioff[J];
    for (int i0 = k0; i0 < k1; i0 += kSelThreads) {
        const int k = i0 + threadIdx.x;
        const bool in = k < k1, ip = in && alev[k];
        int ti, ta;
        const int pi = block_scan(ip ? 1 : 0, ti, sw);
        const int pa = block_scan(in && !ip ? 1 : 0, ta, sw);
        if (ip) ip_list[ib + pi] = k;
        else if (in) aca_list[ab + pa] = k;
        ib += ti;
        ab += ta;
    }
}

// accepted blocks (rank > 0) of kept row J: counts, flags of the dense kernel
// cleared, the (I, J) bitmap for the per-I lists
__global__ void __launch_bounds__(kSelThreads) k_acc_count(const int *koff, const int2 *ab, const int *rank, int nb,
                                                           uint8_t *flags_out, uint8_t *accbm, int *acnt)
{
    __shared__ int sw[kSelThreads / 32];
    const int J = blockIdx.x, k0 = koff[J], k1 = koff[J + 1];
    int a = 0;
    for (int k = k0 + threadIdx.x; k < k1; k += kSelThreads) {
        if (rank[k] > 0) {
            const long long f = (long long)ab[k].x * nb + J;
            flags_out[f] = kFlagNone;
            accbm[f] = 1;
            ++a;
        }
    }
    int tot;
    block_scan(a, tot, sw);
    if (threadIdx.x == 0) acnt[J] = tot;
}

// accepted positions q (J-major order): bidx[q] = kept index, byJ[q] = q,
// qidx[I][J] = q
__global__ void __launch_bounds__(kSelThreads) k_acc_fill(const int *koff, const int2 *ab, const int *rank, int nb,
                                                          const int *aoff, int *bidx, int *byJ, int *qidx)
{
    __shared__ int sw[kSelThreads / 32];
    const int J = blockIdx.x, k0 = koff[J], k1 = koff[J + 1];
    int base = aoff[J];
    for (int i0 = k0; i0 < k1; i0 += kSelThreads) {
        const int k = i0 + threadIdx.x;
        const bool acc = k < k1 && rank[k] > 0;
        int tot;
        const int pre = block_scan(acc ? 1 : 0, tot, sw);
        if (acc) {
            const int q = base + pre;
            bidx[q] = k;
            byJ[q] = q;
            qidx[(long long)ab[k].x * nb + J] = q;
        }
        base += tot;
    }
}

// per source tile I: accepted blocks (I, J) in J order
__global__ void __launch_bounds__(kSelThreads) k_byI_count(const uint8_t *accbm, int nb, int *icnt)
{
    __shared__ int sw[kSelThreads / 32];
    const int I = blockIdx.x;
    int a = 0;
    for (int J = threadIdx.x; J < nb; J += kSelThreads) a += accbm[(long long)I * nb + J];
    int tot;
    block_scan(a, tot, sw);
    if (threadIdx.x == 0) icnt[I] = tot;
}

__global__ void __launch_bounds__(kSelThreads) k_byI_fill(const uint8_t *accbm, const int *qidx, int nb,
                                                          const int *ioff, int *byI)
{
    __shared__ int sw[kSelThreads / 32];
    const int I = blockIdx.x;
    int base = ioff[I];
    for (int J0 = 0; J0 < nb; J0 += kSelThreads) {
        const int J = J0 + threadIdx.x;
        const bool acc = J < nb && accbm[(long long)I * nb + J];
        int tot;
        const int pre = block_scan(acc ? 1 : 0, tot, sw);
        if (acc) byI[base + pre] = qidx[(long long)I * nb + J];
        base += tot;
    }
}

// statistics of the accepted blocks: count, rank sum of the cross-
// approximated ones, largest judged error, ordered pairs, interpolated
// blocks and their node sum; one partial per CTA (grid-stride over the kept
// blocks), the host adds the partials in order
constexpr int kStatCtas = 128;

__global__ void __launch_bounds__(kSelThreads) k_cmp_stats(const int *nkeep, const int2 *ab, const int *rank,
                                                           const float *err, int nsrc, const uint8_t *lev,
                                                           double *part)
{
    __shared__ double sd[kCmpStats][kSelThreads];
    const int n = *nkeep;
    double v[kCmpStats] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = blockIdx.x * kSelThreads + threadIdx.x; k < n; k += gridDim.x * kSelThreads) {
        const int r = rank[k];
        if (r > 0) {
            const bool ip = lev && lev[k];
            v[0] += 1.0;
            v[1] += ip ? 0.0 : (double)r;
            v[2] = fmax(v[2], (double)err[k]);
            const double ni = min(kTile, nsrc - ab[k].x * kTile), nj = min(kTile, nsrc - ab[k].y * kTile);
            v[3] += 2.0 * ni * nj;
            v[4] += ip ? 1.0 : 0.0;
            v[5] += ip ? (double)r : 0.0;
        }
    }
#pragma unroll
    for (int q = 0; q < kCmpStats; ++q) sd[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int s = kSelThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
#pragma unroll
            for (int q = 0; q < kCmpStats; ++q)
                sd[q][threadIdx.x] = q == 2 ? fmax(sd[q][threadIdx.x], sd[q][threadIdx.x + s])
                                            : sd[q][threadIdx.x] + sd[q][threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x < kCmpStats) part[blockIdx.x * kCmpStats + threadIdx.x] = sd[threadIdx.x][0];
}

}  // namespace

void launch_cand_lists(const uint8_t *flags, int nt, int nb, int select, float eta, const float4 *cen, int *cnt,
                       int *off, int2 *blocks, uint8_t *cls, cudaStream_t s)
{
    if (nb <= 0) return;
    k_cand_count<<<nb, kSelThreads, 0, s>>>(flags, nt, nb, select, eta, cen, cnt);
    k_scan<<<1, kSelThreads, 0, s>>>(cnt, nb, off);
    k_cand_fill<<<nb, kSelThreads, 0, s>>>(flags, nt, nb, select, eta, cen, off, blocks, cls);
}

void launch_keep_lists(int nb, const int *coff, const float *pred, float cut, int rmax, const int2 *cblocks,
                       const uint8_t *ccls, int *kcnt, int *ksum, int *koff, int *kcoloff, int2 *ab, uint8_t *acls,
                       int *acap, long long *aoff, int *kmap, cudaStream_t s, const uint8_t *clev, uint8_t *alev)
{
    if (nb <= 0) return;
    k_keep_count<<<nb, kSelThreads, 0, s>>>(coff, pred, cut, rmax, clev, kcnt, ksum);
    k_scan<<<1, kSelThreads, 0, s>>>(kcnt, nb, koff);
    k_scan<<<1, kSelThreads, 0, s>>>(ksum, nb, kcoloff);
    k_keep_fill<<<nb, kSelThreads, 0, s>>>(coff, pred, cut, rmax, cblocks, ccls, clev, koff, kcoloff, ab, acls, acap,
                                           aoff, kmap, alev);
}

void launch_split_kept(int nb, const int *koff, const uint8_t *alev, int *icnt, int *ioff, int *aca_list,
                       int *ip_list, cudaStream_t s)
{
    if (nb <= 0) return;
    k_split_count<<<nb, kSelThreads, 0, s>>>(koff, alev, icnt);
    k_scan<<<1, kSelThreads, 0, s>>>(icnt, nb, ioff);
    k_split_fill<<<nb, kSelThreads, 0, s>>>(koff, alev, ioff, aca_list, ip_list);
}

void launch_accept_lists(int nt, int nb, const int *koff, const int2 *ab, const int *rank, uint8_t *flags_out,
                         uint8_t *accbm, int *qidx, int *acnt, int *byJ_off, int *bidx, int *byJ, int *icnt,
                         int *byI_off, int *byI, cudaStream_t s)
{
    if (nb <= 0) return;
    cudaMemsetAsync(accbm, 0, (size_t)nt * nb, s);
    k_acc_count<<<nb, kSelThreads, 0, s>>>(koff, ab, rank, nb, flags_out, accbm, acnt);
    k_scan<<<1, kSelThreads, 0, s>>>(acnt, nb, byJ_off);
    k_acc_fill<<<nb, kSelThreads, 0, s>>>(koff, ab, rank, nb, byJ_off, bidx, byJ, qidx);
    if (nt > 0) {
        k_byI_count<<<nt, kSelThreads, 0, s>>>(accbm, nb, icnt);
        k_scan<<<1, kSelThreads, 0, s>>>(icnt, nt, byI_off);
        k_byI_fill<<<nt, kSelThreads, 0, s>>>(accbm, qidx, nb, byI_off, byI);
    }
}

int cmp_stats_parts() { return kStatCtas; }

void launch_cmp_stats(const int *nkeep, const int2 *ab, const int *rank, const float *err, int nsrc, double *out,
                      cudaStream_t s, const uint8_t *lev)
{
    k_cmp_stats<<<kStatCtas, kSelThreads, 0, s>>>(nkeep, ab, rank, err, nsrc, lev, out);
}

}  // namespace sonar
