// sonar_internal.h -- structures shared by the host model (model.cpp) and the
// CUDA kernels (kernels.cu).  All device buffers are structure-of-arrays.
//
// Device layout of one object (HBM):
//   cells      every fragment cell of every facet, facet-major, row-major
//              y*numXpnts + x inside a facet (the reference's P layout,
//              src/OptiX.cu:49).  cell_pos (float4 x,y,z,area) holds the
//              source-hop centroid (x offset + delta/2, src/OptiX.cu:51);
//              cell_facet the facet index; P/Pin/Pout are double2.
//   active     cells with area > 1e-6 (the area gates of src/OptiX.cu:138,
//              :219, :286), in cell order: act_pos (float4 x,y,z,area) with
//              the centroid WITHOUT the delta/2 x shift (src/OptiX.cu:129,
//              :210, :273), act_facet, act_cell.
//   facet_n    unit normal per facet (float4).
// Interaction masks: one flag byte per (source tile of 256, destination block
// of 256): nothing interacts, per-pair bits stored, or CLEAR (no triangle can
// occlude any pair; the sum kernel evaluates the cosine gates inline).  Bits
// are uint32 words [src_word][dst_pitch] -- bit b of word (w, j) is the pair
// (source 32w+b, destination j).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sonar {

// HOP_RESP: target object -> another target object with reciprocity
// (FACET_RESP); mask and sum of one direction, keyed (source object,
// destination object); the ray starts at the lower-index object's point
enum Hop : int { HOP_SRC = 0, HOP_FP = 1, HOP_F2F = 2, HOP_NORESP = 3, HOP_RESP = 4 };
// Hops of piston source objects (host bookkeeping; the kernels run them as
// HOP_RESP and HOP_NORESP): source object -> target, source object -> field object
constexpr int HOP_PISTON_T = 5, HOP_PISTON_F = 6;

constexpr int kTile = 256;          // sources per tile, destinations per block
constexpr int kWordsPerTile = kTile / 32;

// Per-block mask flags: no pair interacts / per-pair bits stored / no triangle
// can occlude any pair of the block, gates are evaluated inline by the sums /
// every pair of the block interacts (no occluder, every cosine gate passes).
constexpr uint8_t kFlagNone = 0, kFlagBits = 1, kFlagClear = 2, kFlagAll = 3;

struct BvhNode {                    // 32 bytes
    float lo[3];
    int left;                       // >= 0 inner child, < 0 leaf: first triangle = -left-1
    float hi[3];
    int right;                      // inner: right child; leaf: triangle count
};

struct BvhView {
    const float4 *nodes;            // BvhNode as 2 float4
    const float4 *tris;             // 4 float4 per triangle: (n,c) (m0,c0) (m1,c1) (m2,c2)
    int nnodes;
    int ntri;
};

struct MaskView {
    uint32_t *bits;
    uint8_t *flags;
    long long pitch;                // words per source-word row (>= ndst, multiple of 32)
    int nwords;                     // ceil(nsrc / 32)
    int ntiles;                     // ceil(nsrc / 256)
    int ndstblocks;                 // ceil(ndst / 256)
};

struct MaskArgs {
    int hop;
    int nsrc, ndst;
    const float4 *src_pos;          // x, y, z, area
    const int *src_facet;           // may be null (points)
    const float4 *src_facet_n;
    const float4 *dst_pos;
    const int *dst_facet;           // may be null (points)
    const float4 *dst_facet_n;
    int dst_is_field;               // cos_inc forced to 1 (src/OptiX.cu:67-72, :308-312)
    int full;                       // store per-pair bits for CLEAR blocks too (diagnostic export)
    int upper_only;                 // FACET_SELF: only blocks with source tile <= destination block
    BvhView bvh;
    MaskView mask;
    const int2 *blist = nullptr;    // optional: (source tile, destination block) of the blocks to build
    const int *blist_count = nullptr;
    int *blist_next = nullptr;      // k_mask_listed: the next listed block to take (starts at 0)
    int gate_proj = 1;              // FACET_SELF: decide gates from per-point projections where certain
    int resp_dst_origin = 0;        // FACET_RESP: the ray starts at the destination point
    int convex = 0;                 // every target vertex on or behind every target triangle's plane
    float convex_vmax = 0.0f;       // largest |coordinate| of the target vertices
    // optional: per source tile / destination block, the lowest and highest
    // facet index of its fragments (blocks within one facet skip their loads)
    const int2 *src_frange = nullptr, *dst_frange = nullptr;
};

struct SumArgs {
    int hop;
    int nsrc, ndst;
    const float4 *srcA;             // x, y, z, Re(weight)
    const float4 *srcB;             // nx, ny, nz, Im(weight)
    const float4 *dst_pos;
    const int *dst_facet;
    const float4 *dst_facet_n;
    const int *dst_limit;           // FACET_SELF: sources at or past this index are dropped
    int dst_is_field;
    MaskView mask;
    float kr, ka;                   // Re k, Im k (FP32 values of the reference's k_wave)
    float k2hi, k2lo;               // Re k / (2 pi) split in two floats
    float rmin;                     // regularisation radius (source object delta)
    float kr4pi;                    // Re k / (4 pi)
    double2 *partial;               // [nsplit][ndst]
    int nsplit;
    int tiles_per_split;
    // centroid-relative geometry (source hop and field-point readout, option
    // relative_geometry): the phase distance from FP64 references instead of
    // the reference's FP32 r; tile_cen: per source tile the centroid of its
    // fragments (readout), k2pi = Re k / (2 pi) in FP64
    int rel = 0;
    const float4 *tile_cen = nullptr;
    double k2pi = 0.0;
};

// kernels.cu
void launch_mask(const MaskArgs &a, cudaStream_t s);
// FACET_RESP finalize: partial sums into P_out and P of the destination
// cells; with gate_pin, destinations whose P_in is 0 receive nothing
void launch_finalize_resp(const double2 *partial, int nsplit, int ndst, const int *cell, const double2 *gate_pin,
                          double2 *Pout, double2 *P, cudaStream_t s);
// Bounce masks (HOP_F2F, no full export): classification pass, then the pair
// kernel on the blocks it lists (blist: one entry per block at most; count_dev
// holds two ints: their count and the pair kernel's next-block counter), on a
// grid of resident CTAs (nsm SMs) that reads the count on the device: no host
// synchronisation.  Returns the number of kernels launched.
int launch_mask_classified(const MaskArgs &a, int2 *blist, int *count_dev, int nsm, cudaStream_t s);
void launch_sum(const SumArgs &a, cudaStream_t s);
void launch_pack_points(const float4 *pts, const double2 *P, int n, float4 *A, float4 *B, cudaStream_t s);
void launch_pack_frags(const float4 *act_pos, const int *act_facet, const int *act_cell, const float4 *facet_n,
                       const double2 *P, float scale, int n, float4 *A, float4 *B, cudaStream_t s);
void launch_f2f_limits(const int *act_facet, const int *act_cell, const int *facet_end, const double2 *Pin, int n,
                       int nsrc, int *limit, cudaStream_t s);
// out[cell[j]] += sum over splits (cell == nullptr: out[j])
void launch_finalize_add(const double2 *partial, int nsplit, int ndst, const int *cell, double2 *out,
                         cudaStream_t s);
// Pout[cell[j]] = sum, P[cell[j]] += sum
void launch_finalize_f2f(const double2 *partial, int nsplit, int ndst, const int *cell, double2 *Pout,
                         double2 *P, cudaStream_t s);
void launch_mask_export(const MaskView &m, int nsrc, int ndst, uint8_t *out, cudaStream_t s);
void launch_mask_export_rows(const MaskView &m, int nsrc, const int *rows, int nrows, uint8_t *out, cudaStream_t s);
// FACET_SELF with reciprocity: one Green's function per unordered pair, over
// a work list of the non-empty upper blocks cut into chunks of `per` blocks
// of one destination row.  colpart holds 256 * ntiles * (ntiles - 1) / 2
// double2, rowpart 256 per chunk.
struct SymWork {
    const int *blist;      // [nb][ntiles]: row J's non-empty source tiles
    const int4 *chunks;    // (J, k0, k1)
    const int *nchunks;    // device count
    int ntiles;
    int *next;             // device counter of the next chunk to take (zeroed by the launcher)
};
void launch_sym_worklist(const uint8_t *flags, int ntiles, int nb, int per, int *blist, int *rowcnt, int *chunk_off,
                         int4 *chunks, int *nchunks, cudaStream_t s);
void launch_sum_f2f_sym(const SumArgs &a, const SymWork &wl, int grid, double2 *colpart, double2 *rowpart,
                        cudaStream_t s);
void launch_finalize_f2f_sym(const double2 *rowpart, const int *chunk_off, int ndst, const double2 *colpart,
                             const uint8_t *flags, int ntiles, const int *cell, const double2 *Pin, double2 *Pout,
                             double2 *P, cudaStream_t s, const double2 *yrow = nullptr,
                             const double2 *ycol = nullptr);
// Low-rank FACET_SELF blocks (adaptive cross approximation of blocks of any
// interacting class, judged on sampled exact entries; rank -1 = keep dense),
// the admissibility network's block descriptors, and the application of the
// accepted blocks in a bounce.  Block b's factors start at column off[b].
constexpr int kLrRankLimit = 64;
// Returns true when the kernel also wrote the low-rank apply's block outputs
// for the packed inputs of this launch (panel variants given brow, bcol).
// list (optional): the kept blocks to build (nblocks of them); otherwise blocks 0 .. nblocks - 1
bool launch_aca(const SumArgs &a, const int2 *blocks, const uint8_t *cls, const int *cap, const long long *off,
                int nblocks, float tol, float2 *U, float2 *V, int *rank, float *fro, float limit, float *err,
                cudaStream_t s, int variant = 0, float2 *brow = nullptr, float2 *bcol = nullptr,
                const int *list = nullptr);
// Full-tile relative RMS error of the sampled accepted blocks (no attenuation)
void launch_lr_audit(const SumArgs &a, const int2 *blocks, const uint8_t *cls, const long long *off, const int *rank,
                     const int *sample, int ns, const float2 *U, const float2 *V, float *out_err, cudaStream_t s,
                     const uint8_t *lev = nullptr);
// ndev (optional): the block count in device memory; nblocks / nb bound the grid
void launch_block_desc(const SumArgs &a, const int2 *blocks, const uint8_t *cls, int nblocks, const float4 *cen,
                       const float4 *nm, float inv_lambda, float *X, cudaStream_t s, const int *ndev = nullptr);
// interp.cu: directional interpolation of far blocks of class ALL between
// planar tiles.  Per tile a frame (4 float4: box centre and capability, the
// facet's grid axes, normal and box size), per fragment its cell in the box;
// per kept block a level (0: cross approximation; 1..3: nodes (6, 4), (7, 5),
// (8, 6) of the oscillatory part on elongated boxes, 4..6: (4, 4), (5, 5),
// (6, 6) on square ones; 4 x 3 nodes of the smooth part), whose node entries
// take ip_columns(level) columns of the U array.
__host__ __device__ constexpr int ip_nodes(int level)
{
    return level == 1 ? 24 : level == 2 ? 35 : level == 3 ? 48 : level == 4 ? 16 : level == 5 ? 25 : level == 6 ? 36 : 0;
}
__host__ __device__ constexpr int ip_columns(int level)
{
    // C with rows of odd pitch (P | 1), then (from an even entry) the smooth part's 12 x 13
    return ip_nodes(level) > 0
               ? ((((ip_nodes(level) * (ip_nodes(level) | 1)) + 1) & ~1) + 156 + kTile - 1) / kTile
               : 0;
}
static_assert(ip_columns(4) > 0 && ip_columns(6) > 0 && ip_columns(7) == 0, "levels with node entries");
constexpr int kIpTileRec = 6;  // float4 per tile record
struct IpCtx {
    const float4 *tile = nullptr;
    const uint16_t *fxy = nullptr;
    const uint8_t *lev = nullptr;
    float delta = 0.0f;
    // the interpolated kept blocks (n of them)
    const int *list = nullptr;
    int n = 0;
    int *status = nullptr;  // apply: 1 when a node-entry copy arrived late, 2 when not at all
    // optional: the apply runs on this stream beside the factor blocks
    // (fork / join: events the launcher records to order the two)
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
// facet_grid: per facet (xAxis, nx as int bits), (yAxis, first cell as int bits)
void launch_ip_tiles(const float4 *pos, const float4 *nrm, const int *act_facet, const int *act_cell,
                     const float4 *facet_grid, int n, float delta, bool transpose, float4 *tile, uint16_t *fxy,
                     cudaStream_t s);
// levels of the candidates (ncand: their count on the device, nmax bounds the grid)
void launch_ip_level(const int2 *cb, const uint8_t *ccls, const int *ncand, int nmax, const float4 *tile,
                     float delta, float kr, float tol, uint8_t *lev, cudaStream_t s);
// node entries, judge (rank = node count or -1) and, given brow, the apply to
// the packed inputs; kept blocks of level 0 are left alone.  list
// (optional): the interpolated kept blocks, n of them.
void launch_ip_build(const SumArgs &a, const float4 *tile, const uint16_t *fxy, const uint8_t *lev, float delta,
                     const int2 *blocks, const long long *off, int n, float limit, float2 *store, int *rank,
                     float *fro, float *err, float2 *brow, float2 *bcol, cudaStream_t s, const int *list = nullptr);
// the apply of the accepted interpolated blocks: over list (nlist kept
// blocks, rank > 0) when given, else over the accepted positions bidx
void launch_ip_apply(const SumArgs &a, const float4 *tile, const uint16_t *fxy, const uint8_t *lev, float delta,
                     const int2 *blocks, const long long *off, const int *bidx, int nb, const int *ndev,
                     const float2 *store, float2 *brow, float2 *bcol, cudaStream_t s, const int *list = nullptr,
                     int nlist = 0, const int *rank = nullptr, int *status = nullptr);
// full-tile relative RMS error of sampled accepted interpolated blocks (no attenuation)
void launch_ip_audit(const SumArgs &a, const float4 *tile, const uint16_t *fxy, const uint8_t *lev, float delta,
                     const int2 *blocks, const long long *off, const int *sample, int ns, const float2 *store,
                     float *out_err, cudaStream_t s);
// Low-rank apply of the accepted blocks (factors by k_lr_block, interpolated
// blocks by the interpolation kernel when ip is given) and the per-tile gather.
void launch_lr_apply(const SumArgs &a, const int2 *blocks, const long long *off, const int *bidx, int nb,
                     const float2 *U, const float2 *V, const int *rank, float2 *brow, float2 *bcol, int ntiles,
                     const int *byJ_off, const int *byJ, const int *byI_off, const int *byI, double2 *yrow,
                     double2 *ycol, cudaStream_t s, const int *ndev = nullptr, bool outputs_ready = false,
                     int lr_ctas = 4, const IpCtx *ip = nullptr, const int *aca_list = nullptr, int naca = 0);
// select.cu: block lists of the compressed bounce, built on the device
void launch_cand_lists(const uint8_t *flags, int nt, int nb, int select, float eta, const float4 *cen, int *cnt,
                       int *off, int2 *blocks, uint8_t *cls, cudaStream_t s);
// clev (optional): candidate levels; an interpolated block reserves
// ip_columns(level) factor columns and gets rank cap 0 (alev: kept levels)
void launch_keep_lists(int nb, const int *coff, const float *pred, float cut, int rmax, const int2 *cblocks,
                       const uint8_t *ccls, int *kcnt, int *ksum, int *koff, int *kcoloff, int2 *ab, uint8_t *acls,
                       int *acap, long long *aoff, int *kmap, cudaStream_t s, const uint8_t *clev = nullptr,
                       uint8_t *alev = nullptr);
// kept blocks by kind, in kept order: the cross-approximated ones
// (aca_list) and the interpolated ones (ip_list); ioff[nb] = their count
void launch_split_kept(int nb, const int *koff, const uint8_t *alev, int *icnt, int *ioff, int *aca_list,
                       int *ip_list, cudaStream_t s);
void launch_accept_lists(int nt, int nb, const int *koff, const int2 *ab, const int *rank, uint8_t *flags_out,
                         uint8_t *accbm, int *qidx, int *acnt, int *byJ_off, int *bidx, int *byJ, int *icnt,
                         int *byI_off, int *byI, cudaStream_t s);
// out: cmp_stats_parts() x kCmpStats doubles (accepted, rank sum of the
// cross-approximated ones, largest error, ordered pairs, interpolated blocks
// accepted, their node sum) to add in order
constexpr int kCmpStats = 6;
int cmp_stats_parts();
void launch_cmp_stats(const int *nkeep, const int2 *ab, const int *rank, const float *err, int nsrc, double *out,
                      cudaStream_t s, const uint8_t *lev = nullptr);
void launch_tile_stats(const float4 *pos, const float4 *nrm, int n, float4 *cen, float4 *nmean, cudaStream_t s);
// mlp.cu: the admissibility network (8 -> w -> w -> w -> 1, ReLU; w = 64 or 128)
size_t mlp_param_count();
bool mlp_ready();
cudaError_t mlp_set_width(int width);  // 64 or 128 (drops the parameters)
int mlp_width();
int mlp_take_status();                 // tensor-core inference: 0 fine, 1 a wait ran out, 2 and TMEM kept
cudaError_t mlp_init(unsigned seed);
cudaError_t mlp_set_params(const float *p, size_t n);
cudaError_t mlp_get_params(float *p, size_t n);
cudaError_t mlp_grad(const float *X, const float *y, int B, float *grad, float *loss);
cudaError_t mlp_train(const float *X, const float *y, int n, int epochs, int batch, float lr, unsigned seed,
                      float *last_loss);
cudaError_t mlp_infer_dev(const float *dX, int n, float *dY, cudaStream_t s);  // fused inference kernel
// surface.cu: pressure -> RGBA colour map of the reference's surface textures
void launch_colour_map(const double2 *P, long long n, float min_db, float max_db, int phase, float4 *out,
                       cudaStream_t s);
// batch.cu: many (scene, frequency) items, each a source hop from up to 64
// sources and a readout to up to 64 receivers, contracted on the tensor cores.
struct BatchItem {
    int frag0, nfrag;              // the item's fragments [frag0, frag0 + nfrag) of the batch arrays
    int scene, convex;             // scene index (occluders); 1 when the scene is convex
    float kr, ka, k2hi, k2lo, kr4pi;
    float cx, cy, cz;              // reference point of the centroid-relative phase (the scene's box centre)
};
struct BatchArgs {
    const BatchItem *items;
    const int4 *segs;              // (item, first chunk, chunk count, -)
    const int *cta_seg;            // segments [cta_seg[b], cta_seg[b + 1]) of CTA b
    const float4 *frag_pos;        // readout centroid (no x shift), area
    const float4 *frag_spos;       // source-hop centroid (x shift)
    const float4 *frag_n;          // facet normal
    const uint4 *vis;              // per fragment: receiver bits (x, y), source bits (z, w)
    const float4 *rx, *src;        // receivers, sources (at most 64 each)
    int nrx, nsrc;
    float *partial;                // [segment][128][64] FP32
    int *status;                   // set to 1 when a CTA gave up waiting on the tensor core
    // centroid-relative phase (null: absolute FP32 distances as the
    // reference): per item and point (64 rows) D = point - item centre and
    // R = |D| (float4); the factors e^{ik R} go to the reduction, and the
    // receivers' e^{-ik R} (FP32) multiplies the readout's 1/r^2 term
    const float4 *rel_rx = nullptr, *rel_src = nullptr;
    const float2 *rel_rx_e = nullptr;
};
// kernels.cu: interaction bits of both batch hops, one thread per fragment
struct BatchVisArgs {
    const BatchItem *items;
    int nitems;
    long long nfrag;               // fragments of all items
    const float4 *frag_pos, *frag_spos, *frag_n;
    const float4 *rx, *src;
    int nrx, nsrc;
    const BvhView *bvh;            // per scene
    uint4 *vis;
    unsigned *hard;                // queue of pairs that need a shadow test: 128 fragment + point
    unsigned *hard_count;          // (points: receivers 0-63, sources 64-127)
    unsigned hard_cap;
};
// nsm: SM count (grid of the queue pass); the queue count is reset on the stream
void launch_batch_vis(const BatchVisArgs &a, int nsm, cudaStream_t s);
constexpr int kBatchMaxPoints = 64;  // sources and receivers per item
size_t batch_smem_bytes(int kc);
cudaError_t batch_prepare();        // dynamic shared-memory limits of the batch kernels (outside stream capture)
void launch_batch(const BatchArgs &a, int kc, int grid, bool att, cudaStream_t s);
void launch_batch_reduce(const float *partial, const int *item_seg_off, const int *item_segs, int nitems, int nrx,
                         int nsrc, const double2 *erx, const double2 *esrc, double2 *out, cudaStream_t s);

// raster.cu: headless rendering of the textured facets (RenderOpenGL)
struct RasterTri {
    float4 v[3];                   // vertices (w unused)
    float2 uv[3];                  // texture coordinates of the vertices
    int facet, pad;                // index into the facet texture table
};
struct RasterTex {
    long long cell0;               // first colour cell of the facet
    int nx, ny;                    // texture size (the facet's fragment grid)
};
struct RasterArgs {
    const RasterTri *tris;
    const RasterTex *tex;
    const float4 *colours;         // RGBA per cell
    const int4 *work;              // (triangle, tile x, tile y, -)
    float mvp[16];                 // row-major, clip = M [x y z 1]
    int width, height;
    unsigned long long *zbuf;      // width x height
    unsigned char *rgb;            // height x width x 3, top row first
};
int raster_tile();
void launch_raster(const RasterArgs &a, int nwork, cudaStream_t s);

// FP32 FMA rate in FLOP/s (which = 0) or MUFU sine rate in op/s (which = 1)
// on the current device; < 0 on failure.
double measure_peak(int which);

}  // namespace sonar
