// interp.cu -- directional interpolation of far FACET_SELF blocks between
// planar tiles (an alternative to the cross approximation for blocks whose
// every pair interacts).
//
// A tile whose 256 fragments lie on one facet's fragment grid inside a box of
// at most 32 x 16 cells (the usual case: fragments are ordered in 16 x 16
// patches, so a tile is one patch or the tail of one and the head of the
// next) gets a frame: the box centre c, the facet's grid axes e1, e2 and each
// fragment's cell in the box.  For a block of tiles I (columns, points x) and
// J (rows, points y) with centre direction u = (c_J - c_I) / D, the entry
// T(j, i) = m cos_scat cos_inc G(r) of src/OptiX.cu:340-390 (weights
// excluded, m = 1: class ALL) splits into a smooth part S = u_ij / r^2 and an
// oscillatory part O = u_ij (k_a - i k_r) e^{-k_a r} e^{i k_r r} / (4 pi r).
// With the plane wave along u factored out, O e^{-i k u.(y - x)} is smooth
// over both tiles, so
//   O(x, y) ~ e^{i k D} e^{i k u.(y - c_J)} sum_b l_b(y) sum_a C_ba l_a(x) e^{-i k u.(x - c_I)}
//   C_ba = O(x_a, y_b) e^{-i k u.(y_b - c_J)} e^{i k u.(x_a - c_I)} e^{-i k D}
// with tensor Chebyshev nodes x_a, y_b on the boxes and their Lagrange
// polynomials l (px nodes along e1, py along e2; the level picks
// (6, 4), (7, 5) or (8, 6)), and S ~ sum Ls_b(y) Cs_ba Ls_a(x) on 4 x 3
// nodes without a phase.  On the planar grid both the Lagrange products and
// the plane-wave phase factor into x and y parts, so projecting a tile's
// weights onto the nodes and expanding node values back onto fragments are
// two short passes over the box's columns and rows.  C is evaluated once per
// build (stored in the factor array, ip_columns(level) columns) and
// judged against exact entries (lr_entry) on an 8 x 8 grid of sampled rows
// and columns; accepted blocks feed the same per-block output slots as the
// cross approximation's (gathered by k_lr_gather).
#include "sonar_internal.h"
#include "green.cuh"
#include "tc05.cuh"

namespace sonar {
namespace {

constexpr int kIpThreads = 256;
constexpr int kIpMaxP = 8;                     // oscillatory nodes per axis
constexpr int kIpMaxBX = 32, kIpMaxBY = 16;    // box of a tile, in cells
constexpr int kIpSx = 4, kIpSy = 3;            // smooth-part nodes per axis
constexpr int kIpSmooth = kIpSx * kIpSy;
constexpr int kIpMaxNodes = 48;                // px * py at the highest level
constexpr int kIpCPitch = 49;                  // largest row pitch of C (odd: no bank conflicts)
constexpr int kIpSPitch = 13;
constexpr int kIpCols = 8, kIpRows = 8;        // judged columns of I and rows of J (64 entries)

// Chebyshev points of the first kind cos((2a + 1) pi / (2p)) and the inverse
// denominators 1 / prod_{b != a} (x_a - x_b) of their Lagrange polynomials,
// row p (entries a < p)
__constant__ float kChebX[9][8] = {
    {0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {7.071067812e-01f, -7.071067812e-01f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {8.660254038e-01f, 0.000000000e+00f, -8.660254038e-01f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {9.238795325e-01f, 3.826834324e-01f, -3.826834324e-01f, -9.238795325e-01f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {9.510565163e-01f, 5.877852523e-01f, 0.000000000e+00f, -5.877852523e-01f, -9.510565163e-01f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {9.659258263e-01f, 7.071067812e-01f, 2.588190451e-01f, -2.588190451e-01f, -7.071067812e-01f, -9.659258263e-01f, 0.000000000e+00f, 0.000000000e+00f},
    {9.749279122e-01f, 7.818314825e-01f, 4.338837391e-01f, 0.000000000e+00f, -4.338837391e-01f, -7.818314825e-01f, -9.749279122e-01f, 0.000000000e+00f},
    {9.807852804e-01f, 8.314696123e-01f, 5.555702330e-01f, 1.950903220e-01f, -1.950903220e-01f, -5.555702330e-01f, -8.314696123e-01f, -9.807852804e-01f}};
__constant__ float kChebW[9][8] = {
    {0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {1.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {7.071067812e-01f, -7.071067812e-01f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {6.666666667e-01f, -1.333333333e+00f, 6.666666667e-01f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {7.653668647e-01f, -1.847759065e+00f, 1.847759065e+00f, -7.653668647e-01f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {9.888543820e-01f, -2.588854382e+00f, 3.200000000e+00f, -2.588854382e+00f, 9.888543820e-01f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {1.380368241e+00f, -3.771236166e+00f, 5.151604407e+00f, -5.151604407e+00f, 3.771236166e+00f, -1.380368241e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {2.034477110e+00f, -5.700478188e+00f, 8.237429649e+00f, -9.142857143e+00f, 8.237429649e+00f, -5.700478188e+00f, 2.034477110e+00f, 0.000000000e+00f},
    {3.121445152e+00f, -8.889123728e+00f, 1.330351380e+01f, -1.569256449e+01f, 1.569256449e+01f, -1.330351380e+01f, 8.889123728e+00f, -3.121445152e+00f}};

// oscillatory nodes (along e1, along e2) per level
// levels 1-3 for elongated boxes (px along the long side), 4-6 square for
// tiles of one 16 x 16 patch
__constant__ int kLvlPx[7] = {0, 6, 7, 8, 4, 5, 6};
__constant__ int kLvlPy[7] = {0, 4, 5, 6, 4, 5, 6};
static_assert(ip_nodes(1) == 6 * 4 && ip_nodes(2) == 7 * 5 && ip_nodes(3) == 8 * 6 && ip_nodes(3) == kIpMaxNodes &&
                  ip_nodes(4) == 4 * 4 && ip_nodes(5) == 5 * 5 && ip_nodes(6) == 6 * 6,
              "level tables");
static_assert(kIpSmooth * kIpSPitch == 156, "smooth nodes in ip_columns");

__device__ __forceinline__ float2 cmul(float2 x, float2 y)
{
    return make_float2(fmaf(x.x, y.x, -x.y * y.y), fmaf(x.x, y.y, x.y * y.x));
}

// c + x y (complex)
__device__ __forceinline__ float2 cfma(float2 x, float2 y, float2 c)
{
    c.x = fmaf(x.x, y.x, fmaf(-x.y, y.y, c.x));
    c.y = fmaf(x.x, y.y, fmaf(x.y, y.x, c.y));
    return c;
}

// c + x y (x real)
__device__ __forceinline__ float2 rfma(float x, float2 y, float2 c)
{
    c.x = fmaf(x, y.x, c.x);
    c.y = fmaf(x, y.y, c.y);
    return c;
}

// The p Lagrange polynomials of the p Chebyshev points at sigma in [-1, 1]
// (out[a], zero for a >= p): prefix and suffix products of sigma - x_q
__device__ __forceinline__ void lagrange_all(int p, float sigma, float (&out)[kIpMaxP])
{
    float d[kIpMaxP], pre[kIpMaxP], suf[kIpMaxP];
#pragma unroll
    for (int q = 0; q < kIpMaxP; ++q) d[q] = q < p ? sigma - kChebX[p][q] : 1.0f;
    pre[0] = 1.0f;
#pragma unroll
    for (int q = 1; q < kIpMaxP; ++q) pre[q] = pre[q - 1] * d[q - 1];
    suf[kIpMaxP - 1] = 1.0f;
#pragma unroll
    for (int q = kIpMaxP - 2; q >= 0; --q) suf[q] = suf[q + 1] * d[q + 1];
#pragma unroll
    for (int q = 0; q < kIpMaxP; ++q) out[q] = q < p ? kChebW[p][q] * pre[q] * suf[q] : 0.0f;
}

struct IpTile {
    float3 c, e1, e2, n;
    int bx, by;
    bool cap;
};

// tile record (kIpTileRec float4): (c, capable), (e1, 0), (e2, 0), (normal,
// box bx | by << 8), then the occupied column range of each box row y
// (bytes 2y: first, 2y + 1: last; an empty row has first > last)
__device__ __forceinline__ IpTile ip_tile(const float4 *tile, int T)
{
    const float4 *R = tile + (size_t)kIpTileRec * T;
    const float4 p = R[0], q = R[1], r = R[2], s = R[3];
    IpTile o;
    o.c = make_float3(p.x, p.y, p.z);
    o.cap = p.w != 0.0f;
    o.e1 = make_float3(q.x, q.y, q.z);
    o.e2 = make_float3(r.x, r.y, r.z);
    o.n = make_float3(s.x, s.y, s.z);
    const int bb = __float_as_int(s.w);
    o.bx = bb & 255;
    o.by = bb >> 8;
    return o;
}

__device__ __forceinline__ float dot3(float3 x, float3 y) { return fmaf(x.x, y.x, fmaf(x.y, y.y, x.z * y.z)); }

// ---------------------------------------------------------------- tile frames
// One CTA per tile: the tile is capable when every fragment lies on the first
// fragment's facet and their cells fit a box of 4..32 x 2..16 cells; the box
// centre's position follows from the first fragment's (the facet's grid is
// spaced delta along both axes); fxy = the fragment's cell in the box.  A
// box taller than wide is transposed (e1 the grid's y axis, e2 its x axis),
// so that the longer side lies along e1: the strips of partial patches along
// a facet's slanted edge (16 x 30 cells) fit the box that way.
__global__ void __launch_bounds__(kTile) k_ip_tiles(const float4 *pos, const float4 *nrm, const int *act_facet,
                                                    const int *act_cell, const float4 *facet_grid, int n,
                                                    float delta, bool transpose, float4 *tile, uint16_t *fxy)
{
    __shared__ int s_f, s_bad, s_min[2], s_max[2], s_rlo[kIpMaxBY], s_rhi[kIpMaxBY];
    const int T = blockIdx.x, t = threadIdx.x, i0 = T * kTile, i = i0 + t;
    const bool v = i < n;
    if (t < kIpMaxBY) {
        s_rlo[t] = 255;
        s_rhi[t] = 0;
    }
    if (t == 0) {
        s_f = act_facet[i0];
        s_bad = 0;
        s_min[0] = s_min[1] = 1 << 30;
        s_max[0] = s_max[1] = -(1 << 30);
    }
    __syncthreads();
    int x = 0, y = 0;
    if (v) {
        const int f = act_facet[i];
        if (f != s_f) atomicOr(&s_bad, 1);
        const float4 g0 = facet_grid[2 * f], g1 = facet_grid[2 * f + 1];
        const int nx = max(__float_as_int(g0.w), 1), c = act_cell[i] - __float_as_int(g1.w);
        x = c % nx;
        y = c / nx;
        atomicMin(&s_min[0], x);
        atomicMax(&s_max[0], x);
        atomicMin(&s_min[1], y);
        atomicMax(&s_max[1], y);
    }
    __syncthreads();
    const int x0 = s_min[0], y0 = s_min[1], gx = s_max[0] - x0 + 1, gy = s_max[1] - y0 + 1;
    const bool tr = transpose && gy > gx;  // CTA-uniform
    const int bx = tr ? gy : gx, by = tr ? gx : gy;
    const bool cap = !s_bad && bx >= 4 && by >= 2 && bx <= kIpMaxBX && by <= kIpMaxBY;
    const int cx = tr ? y - y0 : x - x0, cy = tr ? x - x0 : y - y0;  // the cell in the box
    if (v) fxy[i] = cap ? (uint16_t)(cx | (cy << 8)) : (uint16_t)0;
    if (v && cap) {
        atomicMin(&s_rlo[cy], cx);
        atomicMax(&s_rhi[cy], cx);
    }
    __syncthreads();
    if (t == 0) {
        float4 *R = tile + (size_t)kIpTileRec * T;
        unsigned w[2 * kIpMaxBY / 4];
        for (int q = 0; q < kIpMaxBY / 2; ++q)
            w[q] = (unsigned)s_rlo[2 * q] | ((unsigned)s_rhi[2 * q] << 8) | ((unsigned)s_rlo[2 * q + 1] << 16) |
                   ((unsigned)s_rhi[2 * q + 1] << 24);
        R[4] = make_float4(__uint_as_float(w[0]), __uint_as_float(w[1]), __uint_as_float(w[2]), __uint_as_float(w[3]));
        R[5] = make_float4(__uint_as_float(w[4]), __uint_as_float(w[5]), __uint_as_float(w[6]), __uint_as_float(w[7]));
        const float4 g0 = facet_grid[2 * s_f], g1 = facet_grid[2 * s_f + 1];
        const float4 p = pos[i0], q = nrm[i0];
        const float ox = delta * ((float)x0 + 0.5f * (float)(gx - 1) - (float)x);
        const float oy = delta * ((float)y0 + 0.5f * (float)(gy - 1) - (float)y);
        R[0] = make_float4(fmaf(g1.x, oy, fmaf(g0.x, ox, p.x)), fmaf(g1.y, oy, fmaf(g0.y, ox, p.y)),
                           fmaf(g1.z, oy, fmaf(g0.z, ox, p.z)), cap ? 1.0f : 0.0f);
        const float4 a1 = tr ? g1 : g0, a2 = tr ? g0 : g1;
        R[1] = make_float4(a1.x, a1.y, a1.z, 0.0f);
        R[2] = make_float4(a2.x, a2.y, a2.z, 0.0f);
        R[3] = make_float4(q.x, q.y, q.z, __int_as_float(cap ? (bx | (by << 8)) : 0));
    }
}

// ---------------------------------------------------------------- levels
// Candidate c (class ALL, both tiles capable, centres at least two box
// lengths apart): the interpolation level from kappa = k (W_I^2 + W_J^2) / D,
// the phase curvature of the plane-wave remainder over the boxes (W: the
// longer box side); 0 leaves the block to the cross approximation.  Blocks
// of two square tiles (one 16 x 16 patch each) take the square levels 4-6
// (4 x 4, 5 x 5, 6 x 6 nodes), the others the elongated levels 1-3.  The
// limits were fitted to hold the full-block relative error of 97 % of the
// blocks of a 60 kHz trihedral to 2 tol (tol = 5e-4 at kscale 1; the judge
// accepts up to 3 tol); kscale = (tol / 5e-4)^(1 / 4.3) follows the error's
// growth with kappa.  Sampled at tol 7e-4 with the boundary-ordered tiles,
// every square block holds 2 tol, while 13 % of the elongated ones (boxes of
// 22 x 15 and 30 x 16 cells) exceed it and 5 % exceed 3 tol.
__global__ void k_ip_level(const int2 *cb, const uint8_t *ccls, const int *ncand, const float4 *tile, float delta,
                           float kr, float kscale, uint8_t *lev)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= *ncand) return;
    uint8_t L = 0;
    if (ccls[c] == kFlagAll) {
        const int2 b = cb[c];
        const IpTile A = ip_tile(tile, b.x), B = ip_tile(tile, b.y);
        if (A.cap && B.cap) {
            const float dx = B.c.x - A.c.x, dy = B.c.y - A.c.y, dz = B.c.z - A.c.z;
            const float D = sqrtf(dx * dx + dy * dy + dz * dz);
            const float wa = delta * (float)max(A.bx, A.by), wb = delta * (float)max(B.bx, B.by);
            if (D >= 2.0f * fmaxf(wa, wb)) {
                const float kap = kr * (wa * wa + wb * wb) / D;
                const bool square = A.bx <= 16 && A.by <= 16 && B.bx <= 16 && B.by <= 16;
                if (square)
                    L = kap <= 2.08f * kscale ? 4 : kap <= 3.96f * kscale ? 5 : kap <= 7.33f * kscale ? 6 : 0;
                else
                    L = kap <= 6.0f * kscale ? 1 : kap <= 14.0f * kscale ? 2 : kap <= 20.0f * kscale ? 3 : 0;
            }
        }
    }
    lev[c] = L;
}

// Row pitches (in elements) chosen so that the threads of a warp that read
// one column of a table, or one row, hit distinct banks.
constexpr int kLsPitch = kIpMaxP + 1, kSsPitch = kIpSx + 1, kYvPitch = kIpMaxBY + 1;

struct __align__(16) IpShared {
    float2 zg[2][kIpMaxBY][kIpMaxBX + 1];  // weights on the box grids (node tables and the judge's scratch before)
    float2 ls[2][kIpMaxBX][kLsPitch];      // phased Lagrange values along e1, per box column
    float2 lt[2][kIpMaxBY][kLsPitch];      // along e2, per box row
    float ss[2][kIpMaxBX][kSsPitch];       // smooth part, along e1
    float st[2][kIpMaxBY][kSsPitch];       // along e2
    float2 yv[2][kIpMaxP][kYvPitch];       // half-projected weights; later the half-expanded node values
    float2 ys[2][kIpSx][kYvPitch];
    float2 g[2][kIpMaxNodes], gs[2][kIpSmooth];  // node values of the weights (I, J)
    float2 h[2][kIpMaxNodes], hs[2][kIpSmooth];  // coupled node values (into I, into J)
    __align__(16) float2 c[kIpMaxNodes * kIpCPitch];  // C[b][a], b: node of J, a: node of I
    __align__(16) float2 cs[kIpSmooth * kIpSPitch];
    float red[2][2];
    float2 eD;  // e^{i k D}
    int si[kIpCols], sj[kIpRows];
    __align__(8) uint64_t cbar;  // the apply: the node entries' bulk copy
};
static_assert(sizeof(IpShared) <= 48 * 1024, "static shared memory");
// scratch in the weight grids: the node offset tables ((2 x 48 + 2 x 12)
// float4) while the entries are evaluated, then the judge's
constexpr int kIpNodeTab = 0;
static_assert((2 * kIpMaxNodes + 2 * kIpSmooth) * (int)sizeof(float4) <=
                  (int)sizeof(float2) * 2 * kIpMaxBY * (kIpMaxBX + 1),
              "node tables in the weight grids");
static_assert((kIpCols * kIpCPitch + (kIpMaxNodes + kIpSmooth) * kIpCols) * (int)sizeof(float2) +
                      kIpCols * kIpSmooth * (int)sizeof(float) <=
                  (int)sizeof(float2) * 2 * kIpMaxBY * (kIpMaxBX + 1),
              "judge scratch in the weight grids");

using IpArgs = IpCtx;

// Geometry of one block: tiles, levels, centre distance and direction.
struct IpBlock {
    IpTile TI, TJ;
    int I, J, px, py, P, ni, nj;
    float D;
    float3 u;
};

__device__ __forceinline__ IpBlock ip_block(const SumArgs &a, const IpArgs &ip, const int2 *blocks, int b, int L)
{
    IpBlock B;
    B.I = blocks[b].x;
    B.J = blocks[b].y;
    B.TI = ip_tile(ip.tile, B.I);
    B.TJ = ip_tile(ip.tile, B.J);
    B.px = kLvlPx[L];
    B.py = kLvlPy[L];
    B.P = B.px * B.py;
    B.ni = min(kTile, a.nsrc - B.I * kTile);
    B.nj = min(kTile, a.nsrc - B.J * kTile);
    const float dx = B.TJ.c.x - B.TI.c.x, dy = B.TJ.c.y - B.TI.c.y, dz = B.TJ.c.z - B.TI.c.z;
    B.D = sqrtf(dx * dx + dy * dy + dz * dz);
    const float Dinv = 1.0f / B.D;
    B.u = make_float3(dx * Dinv, dy * Dinv, dz * Dinv);
    return B;
}

// e^{i k D}, the phase reduced in turns with the split k / (2 pi)
__device__ __forceinline__ float2 ip_phase_D(const SumArgs &a, float D)
{
    const float th = __fmul_rn(D, a.k2hi);
    const float tl = fmaf(D, a.k2lo, fmaf(D, a.k2hi, -th));
    const float fr = (th - rintf(th)) + tl;
    float2 e;
    sincospif(2.0f * fr, &e.y, &e.x);
    return e;
}

// e^{2 pi i turns} for a phase of a few hundred turns at most: the whole
// turns dropped, the remainder (|.| <= 1/2) through the fast sine / cosine
// (absolute error ~1e-6, far below the interpolation's)
__device__ __forceinline__ float2 turn_phase(float turns)
{
    float sn, cs;
    __sincosf(kTwoPi * (turns - rintf(turns)), &sn, &cs);
    return make_float2(cs, sn);
}

// Lagrange tables of both boxes (threads 0..191; the caller synchronises):
// ls, lt with the plane-wave phase e^{-i k u.(x - c_I)} on I, e^{+i k u.(y - c_J)}
// on J, and the smooth part's ss, st
__device__ __forceinline__ void ip_tables(IpShared &S, const SumArgs &a, const IpBlock &B, float delta)
{
    const int t = threadIdx.x;
    if (t < 64) {
        const int s = t >> 5, x = t & 31, bx = s ? B.TJ.bx : B.TI.bx;
        const float al = dot3(B.u, s ? B.TJ.e1 : B.TI.e1);
        float2 ph = make_float2(0.0f, 0.0f);
        float sig = 0.0f;
        if (x < bx) {
            const float hc = 0.5f * (float)(bx - 1);
            sig = ((float)x - hc) / hc;
            ph = turn_phase((s ? a.k2hi : -a.k2hi) * al * (delta * ((float)x - hc)));
        }
        float l[kIpMaxP];
        lagrange_all(B.px, sig, l);
#pragma unroll
        for (int q = 0; q < kIpMaxP; ++q) S.ls[s][x][q] = make_float2(l[q] * ph.x, l[q] * ph.y);
    } else if (t < 96) {
        const int s = (t - 64) >> 4, y = (t - 64) & 15, by = s ? B.TJ.by : B.TI.by;
        const float be = dot3(B.u, s ? B.TJ.e2 : B.TI.e2);
        float2 ph = make_float2(0.0f, 0.0f);
        float sig = 0.0f;
        if (y < by) {
            const float hc = 0.5f * (float)(by - 1);
            sig = ((float)y - hc) / hc;
            ph = turn_phase((s ? a.k2hi : -a.k2hi) * be * (delta * ((float)y - hc)));
        }
        float l[kIpMaxP];
        lagrange_all(B.py, sig, l);
#pragma unroll
        for (int q = 0; q < kIpMaxP; ++q) S.lt[s][y][q] = make_float2(l[q] * ph.x, l[q] * ph.y);
    } else if (t < 160) {
        const int s = (t - 96) >> 5, x = (t - 96) & 31, bx = s ? B.TJ.bx : B.TI.bx;
        const float hc = 0.5f * (float)(bx - 1), sig = ((float)x - hc) / hc;
        float l[kIpMaxP];
        lagrange_all(kIpSx, sig, l);
#pragma unroll
        for (int q = 0; q < kIpSx; ++q) S.ss[s][x][q] = x < bx ? l[q] : 0.0f;
    } else if (t == kIpThreads - 1) {
        S.eD = ip_phase_D(a, B.D);
    }
    if (t >= 160 && t < 192) {
        const int s = (t - 160) >> 4, y = (t - 160) & 15, by = s ? B.TJ.by : B.TI.by;
        const float hc = 0.5f * (float)(by - 1), sig = ((float)y - hc) / hc;
        float l[kIpMaxP];
        lagrange_all(kIpSy, sig, l);
#pragma unroll
        for (int q = 0; q < kIpSy; ++q) S.st[s][y][q] = y < by ? l[q] : 0.0f;
    }
}

// Node entries are stored as in shared memory: C with the odd row pitch
// P | 1 (rows and columns both read without bank conflicts), then the smooth
// part's 12 x 13; the apply copies them linearly.
__device__ __forceinline__ int ip_smooth_at(int P) { return (P * (P | 1) + 1) & ~1; }

__device__ __forceinline__ void ip_load_entries(IpShared &S, const float2 *cst, int P)
{
    // 16-byte copies: both parts start on even entries of a 2 KB aligned column
    const int n4 = ip_smooth_at(P) >> 1;
    const float4 *src = reinterpret_cast<const float4 *>(cst);
    float4 *dc = reinterpret_cast<float4 *>(S.c), *ds = reinterpret_cast<float4 *>(S.cs);
    for (int e = threadIdx.x; e < n4; e += kIpThreads) dc[e] = __ldg(src + e);
    for (int e = threadIdx.x; e < kIpSmooth * kIpSPitch / 2; e += kIpThreads) ds[e] = __ldg(src + n4 + e);
}

// One CTA of 256 threads per block.  BUILD: kept block blockIdx.x -- node
// entries, store, judge, and (brow given, block accepted) the apply to the
// packed inputs; otherwise accepted block bidx[blockIdx.x] with the stored
// entries, apply only.  Blocks of level 0 belong to the cross approximation.
template <bool ATT, bool BUILD>
__global__ void __launch_bounds__(kIpThreads, 5) k_ip(SumArgs a, IpArgs ip, const int2 *blocks, const long long *off,
                                                   const int *bidx, const int *ndev, int n, float limit,
                                                   float2 *store, int *rank, float *fro, float *err, float2 *brow,
                                                   float2 *bcol, const int *list)
{
    __shared__ IpShared S;
    const int t = threadIdx.x;
    int b;
    if ((int)blockIdx.x >= n) return;
    if (list) {
        b = list[blockIdx.x];  // an interpolated kept block
        if (!BUILD && rank[b] <= 0) return;  // rejected by the judge: dense
    } else if (BUILD) {
        b = blockIdx.x;
    } else {
        if (ndev && (int)blockIdx.x >= *ndev) return;
        b = bidx[blockIdx.x];
    }
    const int L = ip.lev[b];
    if (L == 0) return;  // CTA-uniform
    const IpBlock B = ip_block(a, ip, blocks, b, L);
    const IpTile &TI = B.TI, &TJ = B.TJ;
    const int I = B.I, J = B.J, px = B.px, py = B.py, P = B.P, ni = B.ni, nj = B.nj;
    const float D = B.D, delta = ip.delta;
    const float3 u = B.u;
    float2 *cst = store + (size_t)off[b] * kTile;
    ip_tables(S, a, B, delta);
    // ---- node entries: evaluated (BUILD) or read back
    if (BUILD) {
        // node offsets from the tile centres: oscillatory nodes of I and J,
        // then the smooth part's
        float4 *nI = reinterpret_cast<float4 *>(reinterpret_cast<char *>(&S.zg[0][0][0]) + kIpNodeTab);
        float4 *nJ = nI + kIpMaxNodes, *mI = nJ + kIpMaxNodes, *mJ = mI + kIpSmooth;
        if (t < 2 * kIpMaxNodes + 2 * kIpSmooth) {
            const bool smooth = t >= 2 * kIpMaxNodes;
            const int k = smooth ? t - 2 * kIpMaxNodes : t;
            const int side = smooth ? (k >= kIpSmooth) : (k >= kIpMaxNodes);
            const int q = k - side * (smooth ? kIpSmooth : kIpMaxNodes);
            const int qy = smooth ? kIpSy : py, qx = smooth ? kIpSx : px;
            if (q < qx * qy) {
                const IpTile &T = side ? TJ : TI;
                const int ax = q / qy, ay = q - ax * qy;
                const float sx = 0.5f * delta * (float)(T.bx - 1) * kChebX[qx][ax];
                const float sy = 0.5f * delta * (float)(T.by - 1) * kChebX[qy][ay];
                const float4 o = make_float4(fmaf(sx, T.e1.x, sy * T.e2.x), fmaf(sx, T.e1.y, sy * T.e2.y),
                                             fmaf(sx, T.e1.z, sy * T.e2.z), 0.0f);
                (smooth ? (side ? mJ : mI) : (side ? nJ : nI))[q] = o;
            }
        }
        if (t < kIpCols + kIpRows) {
            // judged columns of I and rows of J, one per 32-fragment band
            const bool col = t < kIpCols;
            const int q = col ? t : t - kIpCols, band = col ? kTile / kIpCols : kTile / kIpRows;
            unsigned hsh = (unsigned)b * 2654435761u + (unsigned)t * 40503u + 977u;
            hsh ^= hsh >> 13;
            hsh *= 0x5bd1e995u;
            hsh ^= hsh >> 15;
            const int idx = min((col ? ni : nj) - 1, band * q + (int)(hsh % (unsigned)band));
            if (col) S.si[q] = idx; else S.sj[q] = idx;
        }
        __syncthreads();
        const float invP = 1.0f / (float)P;
        const int cp = P | 1, nc = ip_smooth_at(P);
        if (cp != P && t < P) {  // the pad column, zero in the store too
            S.c[t * cp + P] = make_float2(0.0f, 0.0f);
            cst[t * cp + P] = make_float2(0.0f, 0.0f);
        }
        if (t < kIpSmooth) {
            S.cs[t * kIpSPitch + kIpSmooth] = make_float2(0.0f, 0.0f);
            cst[nc + t * kIpSPitch + kIpSmooth] = make_float2(0.0f, 0.0f);
        }
        for (int e = t; e < P * P; e += kIpThreads) {
            const int bj = __float2int_rz(((float)e + 0.5f) * invP), ai = e - bj * P;
            const float4 ob = nJ[bj], oa = nI[ai];
            const float3 w = make_float3(ob.x - oa.x, ob.y - oa.y, ob.z - oa.z);
            // O(x_a, y_b) / (e^{i k D} and the nodes' plane-wave phases): with
            // Delta = D u + w the phase left is k (r - u.Delta) =
            // k |w_perp|^2 / (r + u.Delta) (no cancellation)
            const float uw = dot3(u, w);
            const float qx = fmaf(-uw, u.x, w.x), qy = fmaf(-uw, u.y, w.y), qz = fmaf(-uw, u.z, w.z);
            const float p2 = fmaf(qx, qx, fmaf(qy, qy, qz * qz));
            const float ud = D + uw;
            const float r2 = fmaf(ud, ud, p2);
            const float rinv = rsqrtf(r2), r = r2 * rinv;
            const float3 v = make_float3(fmaf(D, u.x, w.x), fmaf(D, u.y, w.y), fmaf(D, u.z, w.z));
            const float uu = (dot3(v, TI.n) * dot3(v, TJ.n)) * (-rinv * rinv);
            const float2 ph = turn_phase(a.k2hi * __fdividef(p2, r + ud));
            float2 val;
            if (ATT) {
                const float amp = uu * rinv * kInv4Pi * __expf(-a.ka * r);
                val = make_float2(amp * fmaf(a.ka, ph.x, a.kr * ph.y), amp * fmaf(a.ka, ph.y, -a.kr * ph.x));
            } else {
                const float amp = uu * rinv * a.kr4pi;  // amp (-i) e^{i phase}
                val = make_float2(amp * ph.y, -amp * ph.x);
            }
            S.c[bj * cp + ai] = val;
            cst[bj * cp + ai] = val;
        }
        for (int e = t; e < kIpSmooth * kIpSmooth; e += kIpThreads) {
            const int bj = e / kIpSmooth, ai = e - bj * kIpSmooth;
            const float4 ob = mJ[bj], oa = mI[ai];
            const float3 v = make_float3(fmaf(D, u.x, ob.x - oa.x), fmaf(D, u.y, ob.y - oa.y),
                                         fmaf(D, u.z, ob.z - oa.z));
            const float r2 = dot3(v, v);
            const float val = -(dot3(v, TI.n) * dot3(v, TJ.n)) / (r2 * r2);  // u_ij / r^2
            S.cs[bj * kIpSPitch + ai] = make_float2(val, 0.0f);
            cst[nc + bj * kIpSPitch + ai] = make_float2(val, 0.0f);
        }
    } else if (t == 0) {
        // the stored node entries come in by bulk copies while the tables,
        // weights and projections are computed; waited for at the coupling
        const uint32_t nb4 = (uint32_t)ip_smooth_at(P) * sizeof(float2);
        const uint32_t sb4 = (uint32_t)(kIpSmooth * kIpSPitch) * sizeof(float2);
        mbar_init(&S.cbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mbar_expect_tx(&S.cbar, nb4 + sb4);
        bulk_g2s(S.c, cst, nb4, &S.cbar);
        bulk_g2s(S.cs, cst + ip_smooth_at(P), sb4, &S.cbar);
    }
    __syncthreads();
    if (BUILD) {
        // ---- judge: exact entries (the dense path's arithmetic) against the
        // interpolant on the 8 x 8 grid of sampled rows and columns
        // scratch in the weight grids: the sampled columns' basis values
        // (oscillatory rows of pitch 49, smooth rows of 12), then
        // W = C L_I(samples), Ws = Cs Ls_I(samples)
        float2 *LIq = &S.zg[0][0][0];                      // [sample][node of I]
        float2 *W = LIq + kIpCols * kIpCPitch;             // [node of J][sample]
        float2 *Ws = W + kIpMaxNodes * kIpCols;            // [smooth node of J][sample]
        float *LsIq = reinterpret_cast<float *>(Ws + kIpSmooth * kIpCols);  // [sample][smooth node of I]
        for (int e = t; e < kIpCols * (P + kIpSmooth); e += kIpThreads) {
            const int q = e / (P + kIpSmooth), ai = e - q * (P + kIpSmooth), xy = ip.fxy[I * kTile + S.si[q]];
            if (ai < P) {
                const int aix = ai / py;
                LIq[q * kIpCPitch + ai] = cmul(S.ls[0][xy & 255][aix], S.lt[0][xy >> 8][ai - aix * py]);
            } else {
                const int k = ai - P;
                LsIq[q * kIpSmooth + k] = S.ss[0][xy & 255][k / kIpSy] * S.st[0][xy >> 8][k % kIpSy];
            }
        }
        __syncthreads();
        for (int e = t; e < (P + kIpSmooth) * kIpCols; e += kIpThreads) {
            const int bj = e / kIpCols, q = e - bj * kIpCols;
            float2 acc0 = make_float2(0.0f, 0.0f), acc1 = acc0;
            if (bj < P) {
                const float2 *cr = S.c + bj * (P | 1), *lq = LIq + q * kIpCPitch;
                int ai = 0;
#pragma unroll 4
                for (; ai + 1 < P; ai += 2) {
                    acc0 = cfma(cr[ai], lq[ai], acc0);
                    acc1 = cfma(cr[ai + 1], lq[ai + 1], acc1);
                }
                if (ai < P) acc0 = cfma(cr[ai], lq[ai], acc0);
                W[bj * kIpCols + q] = make_float2(acc0.x + acc1.x, acc0.y + acc1.y);
            } else {
                const float2 *cr = S.cs + (bj - P) * kIpSPitch;
                const float *lq = LsIq + q * kIpSmooth;
#pragma unroll
                for (int ai = 0; ai < kIpSmooth; ++ai) acc0 = rfma(lq[ai], cr[ai], acc0);
                Ws[(bj - P) * kIpCols + q] = acc0;
            }
        }
        __syncthreads();
        float e2 = 0.0f, x2 = 0.0f;
        if (t < kIpRows * kIpCols) {
            const int qj = t / kIpCols, qi = t - qj * kIpCols;
            const int i = I * kTile + S.si[qi], j = J * kTile + S.sj[qj];
            const int xyj = ip.fxy[j], xj = xyj & 255, yj = xyj >> 8;
            float2 ap = make_float2(0.0f, 0.0f);
            for (int bjx = 0; bjx < px; ++bjx) {
                float2 in = make_float2(0.0f, 0.0f);
                for (int bjy = 0; bjy < py; ++bjy)
                    in = cfma(S.lt[1][yj][bjy], W[(bjx * py + bjy) * kIpCols + qi], in);
                ap = cfma(S.ls[1][xj][bjx], in, ap);
            }
            ap = cmul(ap, S.eD);
#pragma unroll
            for (int bj = 0; bj < kIpSmooth; ++bj)
                ap = rfma(S.ss[1][xj][bj / kIpSy] * S.st[1][yj][bj % kIpSy], Ws[bj * kIpCols + qi], ap);
            const float2 ex = lr_entry<ATT>(a, kFlagAll, true, a.srcA[i], a.srcB[i], a.srcA[j], a.srcB[j]);
            e2 = (ex.x - ap.x) * (ex.x - ap.x) + (ex.y - ap.y) * (ex.y - ap.y);
            x2 = ex.x * ex.x + ex.y * ex.y;
        }
        if (t < 64) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                e2 += __shfl_xor_sync(0xffffffffu, e2, o);
                x2 += __shfl_xor_sync(0xffffffffu, x2, o);
            }
            if ((t & 31) == 0) {
                S.red[t >> 5][0] = e2;
                S.red[t >> 5][1] = x2;
            }
        }
        __syncthreads();
        const float se = S.red[0][0] + S.red[1][0], sx = S.red[0][1] + S.red[1][1];
        const float rel = sx > 0.0f ? sqrtf(se / sx) : (se > 0.0f ? 1.0f : 0.0f);
        const bool accepted = sx > 0.0f && rel <= limit;
        if (t == 0) {
            rank[b] = accepted ? P : -1;
            fro[b] = sqrtf(sx * (float)(ni * nj) / (float)(kIpRows * kIpCols));
            err[b] = rel;
        }
        if (!accepted || !brow) return;  // CTA-uniform
        __syncthreads();                  // the scratch becomes the weight grids
    }
    // ---- the apply: weights onto the box grids (zero where the box has no fragment)
    for (int e = t; e < kIpMaxBY * (kIpMaxBX + 1); e += kIpThreads)
        reinterpret_cast<float4 *>(&S.zg[0][0][0])[e] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    __syncthreads();
    if (t < ni) {
        const int i = I * kTile + t, xy = ip.fxy[i];
        S.zg[0][xy >> 8][xy & 255] = make_float2(a.srcA[i].w, a.srcB[i].w);
    }
    if (t < nj) {
        const int j = J * kTile + t, xy = ip.fxy[j];
        S.zg[1][xy >> 8][xy & 255] = make_float2(a.srcA[j].w, a.srcB[j].w);
    }
    __syncthreads();
    // projections along e1 (box columns; tables and grids are zero past the
    // box): oscillatory nodes ax < px, and the smooth part's ax < 4 from the
    // same weight loads
    {
        const int s = t >> 7, ax = (t >> 4) & 7, y = t & 15;
        // the row's occupied columns, widened to whole pairs (zero outside)
        const unsigned rw = __float_as_uint(
            reinterpret_cast<const float *>(ip.tile + (size_t)kIpTileRec * (s ? J : I) + 4)[y >> 1]);
        const int rg = (rw >> (16 * (y & 1))) & 0xFFFF;
        const int x0 = (rg & 255) & ~1, x1 = min((rg >> 8) | 1, kIpMaxBX - 1);
        float2 acc0 = make_float2(0.0f, 0.0f), acc1 = acc0, sm0 = acc0, sm1 = acc0;
        if (ax < kIpSx) {
#pragma unroll 4
            for (int x = x0; x < x1; x += 2) {
                const float2 z0 = S.zg[s][y][x], z1 = S.zg[s][y][x + 1];
                acc0 = cfma(S.ls[s][x][ax], z0, acc0);
                acc1 = cfma(S.ls[s][x + 1][ax], z1, acc1);
                sm0 = rfma(S.ss[s][x][ax], z0, sm0);
                sm1 = rfma(S.ss[s][x + 1][ax], z1, sm1);
            }
            S.ys[s][ax][y] = make_float2(sm0.x + sm1.x, sm0.y + sm1.y);
        } else if (ax < px) {
#pragma unroll 4
            for (int x = x0; x < x1; x += 2) {
                acc0 = cfma(S.ls[s][x][ax], S.zg[s][y][x], acc0);
                acc1 = cfma(S.ls[s][x + 1][ax], S.zg[s][y][x + 1], acc1);
            }
        }
        S.yv[s][ax][y] = make_float2(acc0.x + acc1.x, acc0.y + acc1.y);
    }
    __syncthreads();
    // along e2: the node values (rows past the box are zero)
    if (t < 2 * kIpMaxNodes) {
        const int s = t >= kIpMaxNodes, k = t - s * kIpMaxNodes, by2 = ((s ? TJ.by : TI.by) + 1) & ~1;
        if (k < P) {
            const int ax = k / py, ay = k - ax * py;
            float2 acc0 = make_float2(0.0f, 0.0f), acc1 = acc0;
#pragma unroll 4
            for (int y = 0; y < by2; y += 2) {
                acc0 = cfma(S.lt[s][y][ay], S.yv[s][ax][y], acc0);
                acc1 = cfma(S.lt[s][y + 1][ay], S.yv[s][ax][y + 1], acc1);
            }
            S.g[s][k] = make_float2(acc0.x + acc1.x, acc0.y + acc1.y);
        }
    } else if (t >= 128 && t < 128 + 2 * kIpSmooth) {
        const int s = (t - 128) / kIpSmooth, k = (t - 128) - s * kIpSmooth, by = s ? TJ.by : TI.by;
        const int ax = k / kIpSy, ay = k - ax * kIpSy;
        float2 acc = make_float2(0.0f, 0.0f);
        for (int y = 0; y < by; ++y) acc = rfma(S.st[s][y][ay], S.ys[s][ax][y], acc);
        S.gs[s][k] = acc;
    }
    if (!BUILD && !mbar_wait(&S.cbar, 0)) {
        // the copy did not arrive in time: wait once more (bounded) so that it
        // cannot land after the CTA is gone, and report the block
        if (!mbar_wait(&S.cbar, 0) && t == 0 && ip.status) atomicExch(ip.status, 2);
        else if (t == 0 && ip.status) atomicExch(ip.status, 1);
    }
    __syncthreads();
    // coupling, two threads per node (even / odd terms, then a lane swap):
    // into J (forward) from the nodes of I, into I (reciprocal) from those of J
    if (t < 2 * kIpMaxNodes) {
        const int bj = t >> 1, h0 = t & 1;
        float2 acc = make_float2(0.0f, 0.0f), acc2 = acc;
        if (bj < P) {
            const float2 *cr = S.c + bj * (P | 1);
            int ai = h0;
#pragma unroll 2
            for (; ai + 2 < P; ai += 4) {
                acc = cfma(cr[ai], S.g[0][ai], acc);
                acc2 = cfma(cr[ai + 2], S.g[0][ai + 2], acc2);
            }
            if (ai < P) acc = cfma(cr[ai], S.g[0][ai], acc);
            acc.x += acc2.x;
            acc.y += acc2.y;
        }
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 1);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 1);
        if (bj < P && h0 == 0) S.h[1][bj] = cmul(acc, S.eD);
    } else if (t >= 128 && t < 128 + 2 * kIpMaxNodes) {
        const int ai = (t - 128) >> 1, h0 = t & 1, cp = P | 1;
        float2 acc = make_float2(0.0f, 0.0f), acc2 = acc;
        if (ai < P) {
            int bj = h0;
#pragma unroll 2
            for (; bj + 2 < P; bj += 4) {
                acc = cfma(S.c[bj * cp + ai], S.g[1][bj], acc);
                acc2 = cfma(S.c[(bj + 2) * cp + ai], S.g[1][bj + 2], acc2);
            }
            if (bj < P) acc = cfma(S.c[bj * cp + ai], S.g[1][bj], acc);
            acc.x += acc2.x;
            acc.y += acc2.y;
        }
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 1);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 1);
        if (ai < P && h0 == 0) S.h[0][ai] = cmul(acc, S.eD);
    } else if (t >= 96 && t < 96 + kIpSmooth) {
        const int bj = t - 96;
        float2 acc = make_float2(0.0f, 0.0f);
        for (int ai = 0; ai < kIpSmooth; ++ai) acc = cfma(S.cs[bj * kIpSPitch + ai], S.gs[0][ai], acc);
        S.hs[1][bj] = acc;
    } else if (t >= 224 && t < 224 + kIpSmooth) {
        const int ai = t - 224;
        float2 acc = make_float2(0.0f, 0.0f);
        for (int bj = 0; bj < kIpSmooth; ++bj) acc = cfma(S.cs[bj * kIpSPitch + ai], S.gs[1][bj], acc);
        S.hs[0][ai] = acc;
    }
    __syncthreads();
    // expansion along e2 (box rows)
    {
        const int s = t >> 7, ax = (t >> 4) & 7, y = t & 15;
        float2 acc = make_float2(0.0f, 0.0f);
        if (ax < px) {
            const float2 *hh = S.h[s] + ax * py;
#pragma unroll
            for (int ay = 0; ay < kIpMaxP; ++ay)
                if (ay < py) acc = cfma(S.lt[s][y][ay], hh[ay], acc);
        }
        S.yv[s][ax][y] = acc;
    }
    if (t < 128) {
        const int s = t >> 6, ax = (t >> 4) & 3, y = t & 15;
        float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int ay = 0; ay < kIpSy; ++ay) acc = rfma(S.st[s][y][ay], S.hs[s][ax * kIpSy + ay], acc);
        S.ys[s][ax][y] = acc;
    }
    __syncthreads();
    // onto the fragments: row t of J (forward) and column t of I (reciprocal)
    float2 fr = make_float2(0.0f, 0.0f), fc = make_float2(0.0f, 0.0f);
    if (t < nj) {
        const int xy = ip.fxy[J * kTile + t], x = xy & 255, y = xy >> 8;
#pragma unroll
        for (int ax = 0; ax < kIpMaxP; ++ax)
            if (ax < px) fr = cfma(S.ls[1][x][ax], S.yv[1][ax][y], fr);
#pragma unroll
        for (int ax = 0; ax < kIpSx; ++ax) fr = rfma(S.ss[1][x][ax], S.ys[1][ax][y], fr);
    }
    if (t < ni) {
        const int xy = ip.fxy[I * kTile + t], x = xy & 255, y = xy >> 8;
#pragma unroll
        for (int ax = 0; ax < kIpMaxP; ++ax)
            if (ax < px) fc = cfma(S.ls[0][x][ax], S.yv[0][ax][y], fc);
#pragma unroll
        for (int ax = 0; ax < kIpSx; ++ax) fc = rfma(S.ss[0][x][ax], S.ys[0][ax][y], fc);
    }
    brow[(size_t)b * kTile + t] = fr;
    bcol[(size_t)b * kTile + t] = fc;
}

// Full-tile audit of sampled accepted interpolated blocks (no attenuation):
// the relative RMS error of the interpolant over all of the block's entries
// against the exact ones.  One CTA per block, thread t the column t of I;
// the rows of J in turn, each row's node vector v = L_J(j) C shared through
// shared memory.
__global__ void __launch_bounds__(kIpThreads) k_ip_audit(SumArgs a, IpArgs ip, const int2 *blocks,
                                                         const long long *off, const int *sample, int ns,
                                                         const float2 *store, float *out_err)
{
    __shared__ IpShared S;
    __shared__ float2 v[kIpMaxNodes], vs[kIpSmooth];
    const int t = threadIdx.x;
    if ((int)blockIdx.x >= ns) return;
    const int b = sample[blockIdx.x], L = ip.lev[b];
    if (L == 0) return;  // CTA-uniform: a cross-approximated block (the other audit's)
    float e2 = 0.0f, x2 = 0.0f;
    {
        const IpBlock B = ip_block(a, ip, blocks, b, L);
        ip_tables(S, a, B, ip.delta);
        ip_load_entries(S, store + (size_t)off[b] * kTile, B.P);
        __syncthreads();
        const int i = B.I * kTile + t;
        const bool col = t < B.ni;
        const int xyi = col ? ip.fxy[i] : 0, xi = xyi & 255, yi = xyi >> 8;
        const float4 pi = col ? a.srcA[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float4 qi = col ? a.srcB[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (int jr = 0; jr < B.nj; ++jr) {
            const int j = B.J * kTile + jr, xyj = ip.fxy[j], xj = xyj & 255, yj = xyj >> 8;
            if (t < B.P) {
                float2 acc = make_float2(0.0f, 0.0f);
                for (int bj = 0; bj < B.P; ++bj) {
                    const int bjx = bj / B.py;
                    acc = cfma(cmul(S.ls[1][xj][bjx], S.lt[1][yj][bj - bjx * B.py]), S.c[bj * (B.P | 1) + t], acc);
                }
                v[t] = cmul(acc, S.eD);
            } else if (t >= 64 && t < 64 + kIpSmooth) {
                const int ai = t - 64;
                float2 acc = make_float2(0.0f, 0.0f);
                for (int bj = 0; bj < kIpSmooth; ++bj)
                    acc = rfma(S.ss[1][xj][bj / kIpSy] * S.st[1][yj][bj % kIpSy], S.cs[bj * kIpSPitch + ai], acc);
                vs[ai] = acc;
            }
            __syncthreads();
            if (col) {
                float2 ap = make_float2(0.0f, 0.0f);
                for (int ai = 0; ai < B.P; ++ai) {
                    const int aix = ai / B.py;
                    ap = cfma(cmul(S.ls[0][xi][aix], S.lt[0][yi][ai - aix * B.py]), v[ai], ap);
                }
                for (int ai = 0; ai < kIpSmooth; ++ai)
                    ap = rfma(S.ss[0][xi][ai / kIpSy] * S.st[0][yi][ai % kIpSy], vs[ai], ap);
                const float2 ex = lr_entry<false>(a, kFlagAll, true, pi, qi, a.srcA[j], a.srcB[j]);
                e2 += (ex.x - ap.x) * (ex.x - ap.x) + (ex.y - ap.y) * (ex.y - ap.y);
                x2 += ex.x * ex.x + ex.y * ex.y;
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e2 += __shfl_xor_sync(0xffffffffu, e2, o);
        x2 += __shfl_xor_sync(0xffffffffu, x2, o);
    }
    __shared__ float2 red[kIpThreads / 32];
    if ((t & 31) == 0) red[t >> 5] = make_float2(e2, x2);
    __syncthreads();
    if (t == 0) {
        float se = 0.0f, sx = 0.0f;
        for (int w = 0; w < kIpThreads / 32; ++w) {
            se += red[w].x;
            sx += red[w].y;
        }
        out_err[blockIdx.x] = sx > 0.0f ? sqrtf(se / sx) : 0.0f;
    }
}

}  // namespace

void launch_ip_tiles(const float4 *pos, const float4 *nrm, const int *act_facet, const int *act_cell,
                     const float4 *facet_grid, int n, float delta, bool transpose, float4 *tile, uint16_t *fxy,
                     cudaStream_t s)
{
    if (n > 0)
        k_ip_tiles<<<(n + kTile - 1) / kTile, kTile, 0, s>>>(pos, nrm, act_facet, act_cell, facet_grid, n, delta,
                                                            transpose, tile, fxy);
}

void launch_ip_level(const int2 *cb, const uint8_t *ccls, const int *ncand, int nmax, const float4 *tile,
                     float delta, float kr, float tol, uint8_t *lev, cudaStream_t s)
{
    if (nmax <= 0) return;
    const float kscale = powf(fmaxf(tol, 1e-7f) / 5e-4f, 1.0f / 4.3f);
    k_ip_level<<<(nmax + 255) / 256, 256, 0, s>>>(cb, ccls, ncand, tile, delta, kr, kscale, lev);
}

void launch_ip_build(const SumArgs &a, const float4 *tile, const uint16_t *fxy, const uint8_t *lev, float delta,
                     const int2 *blocks, const long long *off, int n, float limit, float2 *store, int *rank,
                     float *fro, float *err, float2 *brow, float2 *bcol, cudaStream_t s, const int *list)
{
    if (n <= 0) return;
    IpArgs ip;
    ip.tile = tile;
    ip.fxy = fxy;
    ip.lev = lev;
    ip.delta = delta;
    if (a.ka != 0.0f)
        k_ip<true, true><<<n, kIpThreads, 0, s>>>(a, ip, blocks, off, nullptr, nullptr, n, limit, store, rank, fro, err,
                                                   brow, bcol, list);
    else
        k_ip<false, true><<<n, kIpThreads, 0, s>>>(a, ip, blocks, off, nullptr, nullptr, n, limit, store, rank, fro,
                                                    err, brow, bcol, list);
}

void launch_ip_apply(const SumArgs &a, const float4 *tile, const uint16_t *fxy, const uint8_t *lev, float delta,
                     const int2 *blocks, const long long *off, const int *bidx, int nb, const int *ndev,
                     const float2 *store, float2 *brow, float2 *bcol, cudaStream_t s, const int *list, int nlist,
                     const int *rank, int *status)
{
    if (list) {
        nb = nlist;
        ndev = nullptr;
    }
    if (nb <= 0) return;
    IpArgs ip;
    ip.tile = tile;
    ip.fxy = fxy;
    ip.lev = lev;
    ip.delta = delta;
    ip.status = status;
    float2 *st = const_cast<float2 *>(store);  // read only in the apply
    if (a.ka != 0.0f)
        k_ip<true, false><<<nb, kIpThreads, 0, s>>>(a, ip, blocks, off, bidx, ndev, nb, 0.0f, st,
                                                     const_cast<int *>(rank), nullptr, nullptr, brow, bcol, list);
    else
        k_ip<false, false><<<nb, kIpThreads, 0, s>>>(a, ip, blocks, off, bidx, ndev, nb, 0.0f, st,
                                                      const_cast<int *>(rank), nullptr, nullptr, brow, bcol, list);
}

void launch_ip_audit(const SumArgs &a, const float4 *tile, const uint16_t *fxy, const uint8_t *lev, float delta,
                     const int2 *blocks, const long long *off, const int *sample, int ns, const float2 *store,
                     float *out_err, cudaStream_t s)
{
    if (ns <= 0) return;
    IpArgs ip;
    ip.tile = tile;
    ip.fxy = fxy;
    ip.lev = lev;
    ip.delta = delta;
    k_ip_audit<<<ns, kIpThreads, 0, s>>>(a, ip, blocks, off, sample, ns, store, out_err);
}

}  // namespace sonar
