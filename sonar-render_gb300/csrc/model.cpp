// model.cpp -- the process-global scene and the C ABI (include/sonar_render.h).
//
// Mirrors the reference's one global Model (src/python_interface.cpp:11) and
// its call sequence: load_* and set_initial_conditions collect the scene,
// render_cuda fragments it and uploads it, the Project* calls run the hops
// synchronously, TearDownCuda frees everything.  Differences by design:
//   - device memory is structure-of-arrays per object (sonar_internal.h), and
//     a hop is two kernels (interaction mask + sum) instead of one OptiX launch
//     per facet;
//   - masks depend only on geometry, so they are built once per (hop, source,
//     destination) after render_cuda and reused by later calls (bounces,
//     frequency changes through set_initial_conditions);
//   - nothing throws across the ABI: errors set a status and a message, and
//     calls are skipped until TearDownCuda or sonar_clear_error;
//   - all work runs on one library stream; each entry point returns after the
//     stream is idle, as the reference's DoProjection does (OptiX.cpp:163).
#include <algorithm>
#include <tuple>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sonar_render.h"
#include "devpool.h"
#include "host.h"

namespace sonar {

bool write_png(const std::string &path, int width, int height, const unsigned char *rgb);  // png.cpp

namespace {

constexpr int OBJ_TARGET = 0, OBJ_SOURCE = 1, OBJ_FIELD = 2;

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw Error(code, buf);
}

#define CK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) fail(-10, "%s failed: %s", #call, cudaGetErrorString(e_));          \
    } while (0)

// The render's stream (null before render_cuda: the legacy stream).
cudaStream_t alloc_stream();

double host_ms()
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Device buffers come from the stream-ordered pool, ordered on the render's
// stream, which is the only stream that uses them.
template <class T>
T *dalloc(size_t n)
{
    void *p = nullptr;
    if (n == 0) n = 1;
    CK(pool_alloc(&p, n * sizeof(T), alloc_stream()));
    return (T *)p;
}

template <class T>
void dfree(T *&p)
{
    pool_free(p, alloc_stream());
    p = nullptr;
}

struct Object {
    int type = 0;
    float delta = 0.0f;
    std::vector<FacetFrame> facets;
    // after render
    std::vector<long long> cell0;
    long long ncells = 0;
    std::vector<float> area;
    std::vector<int> act_cell;
    std::vector<int> facet_act_end;  // active index one past facet f's last active cell
    std::vector<long long> facet_nact;
    // device
    float4 *d_cell_pos = nullptr;
    int *d_cell_facet = nullptr;
    float4 *d_facet_n = nullptr;
    float4 *d_facet_grid = nullptr;  // per facet (xAxis, nx), (yAxis, first cell): the interpolated blocks' tile frames
    double2 *d_P = nullptr, *d_Pin = nullptr, *d_Pout = nullptr;
    float4 *d_act_pos = nullptr;
    int *d_act_facet = nullptr, *d_act_cell = nullptr, *d_facet_end = nullptr;
    int2 *d_tile_frange = nullptr;  // per 256-fragment tile: lowest and highest facet index

    int nact() const { return (int)act_cell.size(); }
    void free_device()
    {
        dfree(d_cell_pos); dfree(d_cell_facet); dfree(d_facet_n); dfree(d_facet_grid); dfree(d_P); dfree(d_Pin);
        dfree(d_Pout);
        dfree(d_act_pos); dfree(d_act_facet); dfree(d_act_cell); dfree(d_facet_end); dfree(d_tile_frange);
    }
};

struct MaskEntry {
    int hop, a, b;
    int upper_only = 0;
    long long classes[4] = {0, 0, 0, 0};  // blocks per flag: none, bits, clear, all
    int nsrc, ndst;
    MaskView view{};
    int2 *blist = nullptr;  // bounce masks: blocks the classification pass leaves for per-pair bits
    int *bcount = nullptr;
    float mask_ms = 0.0f;
    bool fresh = false;  // built for the next hop (its time read, from ev6 to ev7, once that hop has ended)
    bool stale = false;  // rebuild into the same buffers before the next use
    void free_device()
    {
        dfree(view.bits);
        dfree(view.flags);
        dfree(blist);
        dfree(bcount);
    }
};

// Low-rank compression of the FACET_SELF blocks of one object (built with its
// mask, rebuilt when the mask or k changes).
// Grow-only device arena: a build carves its arrays from it in order and the
// next build starts over (one pool block, replaced only when it must grow).
struct Arena {
    char *base = nullptr;
    size_t cap = 0, used = 0;
    void reserve(size_t bytes)
    {
        used = 0;
        if (bytes <= cap) return;
        dfree(base);
        cap = 0;
        base = dalloc<char>(bytes);
        cap = bytes;
    }
    template <class T>
    T *take(size_t n)
    {
        const size_t bytes = (std::max<size_t>(n, 1) * sizeof(T) + 255) / 256 * 256;
        if (used + bytes > cap) fail(-10, "internal: arena overflow (%zu + %zu > %zu)", used, bytes, cap);
        T *p = (T *)(base + used);
        used += bytes;
        return p;
    }
    void release()
    {
        dfree(base);
        cap = used = 0;
    }
    static size_t bytes_of(size_t n, size_t elem) { return (std::max<size_t>(n, 1) * elem + 255) / 256 * 256; }
};

struct Compression {
    bool valid = false;
    int obj = -1;
    double kr = 0.0, ki = 0.0;
    int select = 0;             // 0 rule, 1 exhaustive, 2 network
    int rmax = 0;
    int ncand = 0;              // candidate blocks before selection
    int nblocks = 0;            // blocks approximated (after selection)
    int naccepted = 0;
    int nip = 0;                // accepted interpolated blocks
    double mean_rank = 0.0, max_err = 0.0, ip_mean_nodes = 0.0;
    double pairs_cmp = 0.0;     // ordered pairs of the accepted blocks
    // build: whole, selection, cross approximation, interpolation (both on
    // their own streams), both together
    float build_ms = 0.0f, select_ms = 0.0f, aca_ms = 0.0f, ip_ms = 0.0f, approx_ms = 0.0f;
    long long ncols = 0;        // factor columns reserved (sum of caps)
    int2 *d_blocks = nullptr;
    uint8_t *d_cls = nullptr;
    int *d_cap = nullptr;
    long long *d_off = nullptr;
    float2 *d_U = nullptr, *d_V = nullptr, *d_brow = nullptr, *d_bcol = nullptr;
    int *d_rank = nullptr, *d_bidx = nullptr;
    float *d_fro = nullptr, *d_err = nullptr;
    int *d_byJ_off = nullptr, *d_byJ = nullptr, *d_byI_off = nullptr, *d_byI = nullptr;
    uint8_t *d_flags = nullptr;  // the mask flags with accepted blocks removed (dense kernel)
    double2 *d_yrow = nullptr, *d_ycol = nullptr;
    const int *d_nacc = nullptr;    // accepted-block count (device)
    double *d_stats = nullptr;      // accepted count, rank sum, largest judged error, ordered pairs
    float *d_desc = nullptr;        // descriptors of the candidates
    int *d_kmap = nullptr, *d_acap = nullptr;  // kept block -> candidate, rank caps
    bool interp = false;        // interpolated blocks in this build
    uint8_t *d_lev = nullptr;   // per kept block: 0 cross approximation, 1..3 interpolation level
    int *d_aca_list = nullptr, *d_ip_list = nullptr;  // kept blocks by kind
    int naca_kept = 0, nip_kept = 0;
    IpCtx ip;                   // tile frames and box cells of the interpolated blocks
    bool stats_pending = false;     // statistics and timings not read back yet
    bool outputs_ready = false;     // the build also wrote the block outputs of its bounce's inputs
    // descriptors and rank labels of the approximated blocks (network training)
    std::vector<float> desc, label;
    Arena arena;    // the candidate- and block-level arrays above
    Arena factors;  // U, V and the per-block outputs (sized after the selection)
    void release() { valid = false; }
    void free_all()
    {
        arena.release();
        factors.release();
        valid = false;
    }
};

struct HopRecord {
    int hop;
    long long pairs;
    float mask_ms;   // interaction mask kernel (0 when the cached mask was reused)
    float sum_ms;    // sum kernel alone
    float total_ms;  // pack + sum + finalize
    int nsplit;
    int launches;    // kernels launched by this hop, mask included
    // compressed bounce blocks (FACET_SELF with compression on)
    int cmp_cand = 0, cmp_blocks = 0, cmp_accepted = 0, cmp_select = 0, cmp_ip_blocks = 0, cmp_ip_kept = 0;
    double cmp_mean_rank = 0.0, cmp_max_err = 0.0, cmp_pairs = 0.0, cmp_ip_nodes = 0.0;
    float cmp_build_ms = 0.0f, cmp_select_ms = 0.0f, cmp_aca_ms = 0.0f, cmp_ip_ms = 0.0f, cmp_approx_ms = 0.0f;
    float lr_ms = 0.0f;
};

struct Model {
    std::vector<std::unique_ptr<Object>> obj[3];
    std::vector<Vec3> src, fp;
    float cp = 1480.0f, freq = 0.0f, att = 0.0f, density = 0.0f;
    double kr = 0.0, ki = 0.0;
    float max_db = 0.0f, min_db = -100.0f;
    bool phase_target = false, phase_field = false;
    bool rendered = false;
    int status = 0;
    std::string err;
    // device
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr, ev4 = nullptr, ev5 = nullptr;
    cudaEvent_t ev6 = nullptr, ev7 = nullptr, ev8 = nullptr;
    // second stream of a compressed bounce: the low-rank apply (HBM-bound)
    // runs there beside the dense remainder (FP32 / SFU-bound)
    cudaStream_t side = nullptr, side2 = nullptr;  // low-rank work beside the dense remainder
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_fork2 = nullptr, ev_join2 = nullptr;
    // compression build: start, selected, cross approximation end, end,
    // interpolation end, interpolation start (second stream), both joined
    cudaEvent_t evb[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    float4 *d_src_pos = nullptr, *d_fp_pos = nullptr;
    double2 *d_src_P = nullptr, *d_fp_P = nullptr;
    // field points are kept in Morton (spatial) order on the device so that a
    // block of 256 destinations covers a small region; fp_order[k] is the load
    // index of the k-th stored point
    std::vector<int> fp_order;
    int *d_fp_order = nullptr;
    float4 *d_nodes = nullptr, *d_tris = nullptr;
    int nnodes = 0, ntri = 0;
    std::vector<MaskEntry> masks;
    float4 *d_packA = nullptr, *d_packB = nullptr;
    size_t pack_cap = 0;
    double2 *d_partial = nullptr;
    size_t partial_cap = 0;
    int *d_limit = nullptr;
    size_t limit_cap = 0;
    double2 *d_colpart = nullptr;
    float4 *d_tilecen = nullptr, *d_tilenm = nullptr;  // tile centroids of the relative geometry
    size_t tilecen_cap = 0;
    size_t colpart_cap = 0;
    // work list of the symmetric bounce sum
    int *d_blist = nullptr, *d_rowcnt = nullptr, *d_chunk_off = nullptr, *d_nchunks = nullptr;
    int4 *d_chunks = nullptr;
    double2 *d_rowpart = nullptr;
    int sym_tiles = 0;
    int nsm = 0;
    // options and statistics
    int opt_split = 0;
    int verbose = 0;
    int opt_f2f_sym = 1;
    int opt_class_stats = 0;
    // compression of the bounce blocks
    int opt_compress = 0;
    float opt_cmp_tol = 1e-4f, opt_cmp_judge = 3e-4f, opt_cmp_eta = 1.0f;
    int opt_cmp_rmax = 32;
    int opt_cmp_select = 0;     // 0 rule (class ALL, eta-separated), 1 every interacting block, 2 the network
    float opt_cmp_rcut = 32.0f; // network: propose blocks whose predicted rank is below this
    int opt_aca_variant = 8;    // cross-approximation kernel shape (k_aca / k_aca2, factor ranks in shared memory, CTAs per SM)
    int opt_lr_ctas = 4;        // low-rank apply: resident CTAs per SM its register cap allows (4, 6, 8)
    int opt_rel_geom = 0;       // source hop and readout: phase distances relative to FP64 references
    int opt_fused_apply = 1;    // k_aca2: apply the accepted blocks to the building bounce's inputs in the same kernel
    int opt_cmp_interp = 1;     // far class-ALL blocks between planar tiles by directional interpolation (not with select 1)
    int opt_mask_classify = 1;  // bounce masks: warp-per-block classification, pair kernel on the listed blocks
    int opt_gate_proj = 1;      // bounce masks: gates decided from per-point projections where certain
    int opt_cross_objects = 0;  // bounces also between different targets (FACET_RESP); 0: the reference's behaviour
    int opt_convex_masks = 1;   // convex targets: shadow tests search only where a crossing is possible
    int opt_overlap = 1;        // compressed bounce: low-rank apply on the second stream beside the dense remainder
    int opt_build_overlap = 1;  // compressed build: interpolated blocks on the second stream beside the cross approximation
    int opt_tile_align = 1;     // active fragments: full patches on 256-fragment tile boundaries (align_patches)
    int opt_ip_transpose = 0;   // interpolation tile frames: boxes taller than wide transposed (k_ip_tiles)
    int scene_convex = 0;       // every target vertex on or behind every target triangle's plane
    float scene_vmax = 0.0f;    // largest |coordinate| of the target vertices
    Compression cmp;
    std::vector<HopRecord> log;
    long long launches = 0, h2d_bytes = 0, d2h_bytes = 0;
    double render_ms[5] = {0, 0, 0, 0, 0};  // host time of render_cuda: setup, fragments, uploads, occluders, points

    void free_device()
    {
        for (int t = 0; t < 3; t++)
            for (auto &o : obj[t]) o->free_device();
        dfree(d_src_pos); dfree(d_fp_pos); dfree(d_src_P); dfree(d_fp_P); dfree(d_fp_order);
        dfree(d_nodes); dfree(d_tris);
        for (auto &m : masks) m.free_device();
        masks.clear();
        cmp.free_all();
        dfree(d_packA); dfree(d_packB); dfree(d_partial); dfree(d_limit); dfree(d_colpart);
        dfree(d_tilecen); dfree(d_tilenm);
        tilecen_cap = 0;
        dfree(d_blist); dfree(d_rowcnt); dfree(d_chunk_off); dfree(d_nchunks); dfree(d_chunks); dfree(d_rowpart);
        pack_cap = partial_cap = limit_cap = colpart_cap = 0;
        sym_tiles = 0;
        for (cudaEvent_t *e : {&ev0, &ev1, &ev2, &ev3, &ev4, &ev5, &ev6, &ev7, &ev8, &evb[0], &evb[1], &evb[2], &evb[3],
                               &evb[4], &evb[5], &evb[6]})
            if (*e) {
                cudaEventDestroy(*e);
                *e = nullptr;
            }
        for (cudaEvent_t *e : {&ev_fork, &ev_join, &ev_fork2, &ev_join2})
            if (*e) {
                cudaEventDestroy(*e);
                *e = nullptr;
            }
        if (side) cudaStreamDestroy(side);
        side = nullptr;
        if (side2) cudaStreamDestroy(side2);
        side2 = nullptr;
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
        nnodes = ntri = 0;
    }
};

Model g;

cudaStream_t alloc_stream() { return g.stream; }

// ---------------------------------------------------------------- render
// A host array built for one upload: in the pinned arena when it has room
// (copied by DMA; the arena is reset after the render's final
// synchronisation), else on the heap (copied through the staging chunks).
template <class T>
struct UploadArray {
    T *p = nullptr;
    bool pinned = false;
    std::vector<T> heap;
    explicit UploadArray(size_t n)
    {
        p = (T *)host_arena_take(std::max<size_t>(n, 1) * sizeof(T));
        pinned = p != nullptr;
        if (!pinned) {
            heap.resize(std::max<size_t>(n, 1));
            p = heap.data();
        }
    }
    T &operator[](size_t i) { return p[i]; }
    T *data() { return p; }
};

template <class T>
void upload(T *dst, const UploadArray<T> &a, size_t n, cudaStream_t s)
{
    if (n == 0) return;
    if (a.pinned)
        CK(cudaMemcpyAsync(dst, a.p, n * sizeof(T), cudaMemcpyHostToDevice, s));
    else
        CK(stage_to_device(dst, a.p, n * sizeof(T), s));
}

// Patch-aligned tiles.  In patch order a facet's partial patches (along its
// slanted edges) shift every later patch off the 256-fragment tile grid, so
// that most tiles hold the tail of one patch and the head of the next (a box
// of 32 x 16 cells, half of it empty).  Within each facet this moves just
// enough cells of its partial patches in front of its full patches to bring
// the first full patch onto a tile boundary (all full patches then follow on
// boundaries), the rest of the partial cells after them.  The partial
// patches are taken along the facet's boundary -- those left of each patch
// row's full patches upwards, the rows without full patches, those right of
// them downwards -- so that consecutive ones are neighbours and the tiles
// they form stay compact.  The cells moved to the front are the last ones
// of that sequence: the tile they share with the previous facet's last
// cells then joins two far ends of the facets' slanted edges rather than two
// cells on either side of a shared corner, whose near pairs a sampled judge
// could miss.  Edge
// cells -- whose readout centroid (the cell's left edge, without the x
// shift) lies on or outside the facet's triangle, so on or behind the plane
// of a facet that shares the edge -- go last: their pairs are gated or
// shadowed, and grouped in their own tiles they leave the blocks of the
// other partial tiles free of per-pair bits.  Facets stay contiguous and in
// order (the zero-input rule's facet ends are unchanged); outputs are mapped
// through act_cell as before.
void align_patches(Object &o, const std::vector<long long> &unit_act, const std::vector<long long> &unit0,
                   const std::vector<std::vector<int>> &patch_cnt, float4 *act_pos, int *act_facet)
{
    const int nf = (int)o.facets.size();
    parallel_units(nf, [&](long long fl) {
        const int f = (int)fl;
        const long long a0 = unit_act[(size_t)unit0[f]], a1 = unit_act[(size_t)unit0[f + 1]];
        if (a1 - a0 < 2 * kTile) return;
        // the patches in patch order, from the counts pass 2 recorded
        std::vector<PatchRun> runs;
        for (long long u = unit0[f]; u < unit0[f + 1]; u++) {
            long long b = unit_act[(size_t)u] - a0;
            const std::vector<int> &pc = patch_cnt[(size_t)u];
            for (int c = 0; c < (int)pc.size(); c++) {
                if (pc[c] == 0) continue;
                runs.push_back(PatchRun{b, b + pc[c], (int)(u - unit0[f]), c});
                b += pc[c];
            }
        }
        const std::vector<int> order = patch_aligned_order(o.facets[f], runs, act_pos + a0, a0);
        if (order.empty()) return;
        const size_t n = order.size();
        std::vector<float4> pos(n);
        std::vector<int> fac(n), cell(n);
        for (size_t i = 0; i < n; i++) {
            pos[i] = act_pos[a0 + order[i]];
            fac[i] = act_facet[a0 + order[i]];
            cell[i] = o.act_cell[(size_t)(a0 + order[i])];
        }
        memcpy(act_pos + a0, pos.data(), n * sizeof(float4));
        memcpy(act_facet + a0, fac.data(), n * sizeof(int));
        memcpy(o.act_cell.data() + a0, cell.data(), n * sizeof(int));
    });
}

void render_object(Object &o)
{
    const double t0 = host_ms();
    const int nf = (int)o.facets.size();
    o.cell0.assign(nf + 1, 0);
    for (int f = 0; f < nf; f++) o.cell0[f + 1] = o.cell0[f] + (long long)o.facets[f].nx * o.facets[f].ny;
    o.ncells = o.cell0[nf];
    if (o.ncells > (1LL << 31) - 1) fail(-3, "object has %lld cells (limit 2^31-1)", o.ncells);
    o.area.assign((size_t)o.ncells, 0.0f);
    UploadArray<float4> cell_pos((size_t)o.ncells);
    UploadArray<int> cell_facet((size_t)o.ncells);
    std::vector<float4> facet_n(std::max(nf, 1));
    o.act_cell.clear();
    o.facet_act_end.assign(std::max(nf, 1), 0);
    o.facet_nact.assign(std::max(nf, 1), 0);
    // work units: one row of 16-cell patches of one facet.  Pass 1 fills
    // the areas, the source-hop positions and the facet of every cell and
    // counts the active ones; pass 2 writes the active cells at their offsets
    // in compact 16 x 16-cell patches (patch row, patch column, then
    // row-major inside the patch), so that 256 consecutive fragments -- one
    // source tile or destination block of the kernels -- cover a small area
    std::vector<long long> unit0(nf + 1, 0);
    for (int f = 0; f < nf; f++) {
        const FacetFrame &F = o.facets[f];
        unit0[f + 1] = unit0[f] + (F.ny + kPatch - 1) / kPatch;
        facet_n[f] = make_float4(F.normal.x, F.normal.y, F.normal.z, 0.0f);
    }
    const long long nunits = unit0[nf];
    std::vector<int> unit_facet((size_t)nunits);
    for (int f = 0; f < nf; f++)
        for (long long u = unit0[f]; u < unit0[f + 1]; u++) unit_facet[(size_t)u] = f;
    std::vector<long long> unit_act((size_t)nunits + 1, 0);
    parallel_units(nunits, [&](long long u) {
        const int f = unit_facet[(size_t)u];
        const FacetFrame &F = o.facets[f];
        const int y0 = (int)(u - unit0[f]) * kPatch, y1 = std::min(F.ny, y0 + kPatch);
        float *A = o.area.data() + o.cell0[f];
        fragment_area_rows(F, A, y0, y1);
        long long cnt = 0;
        for (int y = y0; y < y1; y++)
            for (int x = 0; x < F.nx; x++) {
                const long long c = o.cell0[f] + (long long)y * F.nx + x;
                const float a = A[(long long)y * F.nx + x];
                const Vec3 ps = fragment_centroid(F, x, y, true);
                cell_pos[c] = make_float4(ps.x, ps.y, ps.z, a);
                cell_facet[c] = f;
                cnt += a > 1e-6f;
            }
        unit_act[(size_t)u + 1] = cnt;
    });
    for (long long u = 0; u < nunits; u++) unit_act[(size_t)u + 1] += unit_act[(size_t)u];
    const long long na_total = unit_act[(size_t)nunits];
    if (na_total > (1LL << 31) - 1) fail(-3, "object has %lld active cells (limit 2^31-1)", na_total);
    UploadArray<float4> act_pos((size_t)na_total);
    UploadArray<int> act_facet((size_t)na_total);
    o.act_cell.resize((size_t)na_total);
    std::vector<std::vector<int>> patch_cnt((size_t)nunits);  // active cells of each patch of a unit
    parallel_units(nunits, [&](long long u) {
        const int f = unit_facet[(size_t)u];
        const FacetFrame &F = o.facets[f];
        const int py = (int)(u - unit0[f]) * kPatch;
        const float *A = o.area.data() + o.cell0[f];
        size_t k = (size_t)unit_act[(size_t)u];
        std::vector<int> &pc = patch_cnt[(size_t)u];
        pc.reserve((size_t)((F.nx + kPatch - 1) / kPatch));
        for (int px = 0; px < F.nx; px += kPatch) {
            const size_t k0 = k;
            for (int y = py; y < std::min(F.ny, py + kPatch); y++)
                for (int x = px; x < std::min(F.nx, px + kPatch); x++) {
                    const float a = A[(long long)y * F.nx + x];
                    if (!(a > 1e-6f)) continue;
                    const Vec3 pa = fragment_centroid(F, x, y, false);
                    act_pos[k] = make_float4(pa.x, pa.y, pa.z, a);
                    act_facet[k] = f;
                    o.act_cell[k] = (int)(o.cell0[f] + (long long)y * F.nx + x);
                    k++;
                }
            pc.push_back((int)(k - k0));
        }
    });
    for (int f = 0; f < nf; f++) {
        o.facet_act_end[f] = (int)unit_act[(size_t)unit0[f + 1]];
        o.facet_nact[f] = unit_act[(size_t)unit0[f + 1]] - unit_act[(size_t)unit0[f]];
    }
    if (g.opt_tile_align) align_patches(o, unit_act, unit0, patch_cnt, act_pos.data(), act_facet.data());
    const size_t nc = (size_t)o.ncells, na = o.act_cell.size();
    const double t1 = host_ms();
    g.render_ms[1] += t1 - t0;
    o.d_cell_pos = dalloc<float4>(nc);
    o.d_cell_facet = dalloc<int>(nc);
    o.d_facet_n = dalloc<float4>(facet_n.size());
    std::vector<float4> facet_grid(2 * facet_n.size());
    for (int f = 0; f < nf; f++) {
        const FacetFrame &F = o.facets[f];
        int nx = F.nx, c0 = (int)o.cell0[f];
        facet_grid[2 * f] = make_float4(F.xAxis.x, F.xAxis.y, F.xAxis.z, 0.0f);
        facet_grid[2 * f + 1] = make_float4(F.yAxis.x, F.yAxis.y, F.yAxis.z, 0.0f);
        memcpy(&facet_grid[2 * f].w, &nx, sizeof(int));
        memcpy(&facet_grid[2 * f + 1].w, &c0, sizeof(int));
    }
    o.d_facet_grid = dalloc<float4>(facet_grid.size());
    o.d_P = dalloc<double2>(nc);
    o.d_act_pos = dalloc<float4>(na);
    o.d_act_facet = dalloc<int>(na);
    o.d_act_cell = dalloc<int>(na);
    o.d_facet_end = dalloc<int>(o.facet_act_end.size());
    cudaStream_t s = g.stream;
    upload(o.d_cell_pos, cell_pos, nc, s);
    upload(o.d_cell_facet, cell_facet, nc, s);
    CK(stage_to_device(o.d_facet_n, facet_n.data(), facet_n.size() * sizeof(float4), s));
    CK(stage_to_device(o.d_facet_grid, facet_grid.data(), facet_grid.size() * sizeof(float4), s));
    CK(cudaMemsetAsync(o.d_P, 0, std::max<size_t>(nc, 1) * sizeof(double2), s));
    if (na) {
        upload(o.d_act_pos, act_pos, na, s);
        upload(o.d_act_facet, act_facet, na, s);
        CK(stage_to_device(o.d_act_cell, o.act_cell.data(), na * sizeof(int), s));
        const size_t ntl = (na + kTile - 1) / kTile;
        std::vector<int2> fr(ntl, make_int2(INT32_MAX, -1));
        for (size_t k = 0; k < na; k++) {
            int2 &r = fr[k / kTile];
            r.x = std::min(r.x, act_facet[k]);
            r.y = std::max(r.y, act_facet[k]);
        }
        o.d_tile_frange = dalloc<int2>(ntl);
        CK(stage_to_device(o.d_tile_frange, fr.data(), ntl * sizeof(int2), s));
        g.h2d_bytes += (long long)(ntl * sizeof(int2));
    }
    CK(stage_to_device(o.d_facet_end, o.facet_act_end.data(), o.facet_act_end.size() * sizeof(int), s));
    g.h2d_bytes += (long long)(nc * (sizeof(float4) + sizeof(int)) + facet_n.size() * sizeof(float4) +
                               na * (sizeof(float4) + 2 * sizeof(int)) + o.facet_act_end.size() * sizeof(int));
    if (o.type == OBJ_TARGET) {
        o.d_Pin = dalloc<double2>(nc);
        o.d_Pout = dalloc<double2>(nc);
        CK(cudaMemsetAsync(o.d_Pin, 0, std::max<size_t>(nc, 1) * sizeof(double2), s));
        CK(cudaMemsetAsync(o.d_Pout, 0, std::max<size_t>(nc, 1) * sizeof(double2), s));
    }
    // the staged copies have read their host arrays; the pinned ones are read
    // by the DMA before render's final synchronisation resets the arena
    g.render_ms[2] += host_ms() - t1;
}

void upload_points(const std::vector<Vec3> &pts, float4 *&d_pos, double2 *&d_P, double value)
{
    const size_t n = pts.size();
    UploadArray<float4> pos(n);
    UploadArray<double2> P(n);
    for (size_t i = 0; i < n; i++) {
        pos[i] = make_float4(pts[i].x, pts[i].y, pts[i].z, 0.0f);
        P[i] = make_double2(value, 0.0);
    }
    d_pos = dalloc<float4>(n);
    d_P = dalloc<double2>(n);
    upload(d_pos, pos, n, g.stream);
    upload(d_P, P, n, g.stream);
    g.h2d_bytes += (long long)(n * (sizeof(float4) + sizeof(double2)));
}

// Order of points along a Morton (Z-order) curve of their bounding box.
std::vector<int> morton_order(const std::vector<Vec3> &pts)
{
    std::vector<int> order(pts.size());
    for (size_t k = 0; k < pts.size(); k++) order[k] = (int)k;
    if (pts.size() < 2) return order;
    float lo[3] = {pts[0].x, pts[0].y, pts[0].z}, hi[3] = {lo[0], lo[1], lo[2]};
    for (auto &p : pts) {
        const float c[3] = {p.x, p.y, p.z};
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], c[k]);
            hi[k] = std::max(hi[k], c[k]);
        }
    }
    auto spread = [](uint64_t v) {  // 21 bits -> every third bit
        v &= 0x1fffff;
        v = (v | v << 32) & 0x1f00000000ffffULL;
        v = (v | v << 16) & 0x1f0000ff0000ffULL;
        v = (v | v << 8) & 0x100f00f00f00f00fULL;
        v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
        v = (v | v << 2) & 0x1249249249249249ULL;
        return v;
    };
    std::vector<uint64_t> code(pts.size());
    for (size_t i = 0; i < pts.size(); i++) {
        const float c[3] = {pts[i].x, pts[i].y, pts[i].z};
        uint64_t q[3];
        for (int k = 0; k < 3; k++) {
            const double ext = (double)hi[k] - (double)lo[k];
            const double u = ext > 0 ? ((double)c[k] - (double)lo[k]) / ext : 0.0;
            q[k] = (uint64_t)std::min(2097151.0, std::max(0.0, u * 2097151.0));
        }
        code[i] = spread(q[0]) | (spread(q[1]) << 1) | (spread(q[2]) << 2);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return code[a] < code[b]; });
    return order;
}

void render()
{
    if (g.rendered) fail(-2, "render_cuda called twice without TearDownCuda");
    const double t0 = host_ms();
    // a render that failed part-way may have left copies in flight out of
    // the pinned arena
    if (g.stream) CK(cudaStreamSynchronize(g.stream));
    host_arena_reset();
    for (double &v : g.render_ms) v = 0.0;
    CK(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
    for (cudaEvent_t *e : {&g.ev0, &g.ev1, &g.ev2, &g.ev3, &g.ev4, &g.ev5, &g.ev6, &g.ev7, &g.ev8, &g.evb[0], &g.evb[1],
                           &g.evb[2], &g.evb[3], &g.evb[4], &g.evb[5], &g.evb[6]})
        CK(cudaEventCreate(e));
    CK(cudaStreamCreateWithFlags(&g.side, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&g.side2, cudaStreamNonBlocking));
    for (cudaEvent_t *e : {&g.ev_fork, &g.ev_join, &g.ev_fork2, &g.ev_join2})
        CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    g.render_ms[0] = host_ms() - t0;
    for (int t : {OBJ_TARGET, OBJ_SOURCE, OBJ_FIELD})
        for (auto &o : g.obj[t]) render_object(*o);
    // piston source objects: unit surface pressure on every cell
    for (auto &o : g.obj[OBJ_SOURCE]) {
        const size_t nc = (size_t)o->ncells;
        UploadArray<double2> P(nc);
        for (size_t c = 0; c < nc; c++) P[c] = make_double2(1.0, 0.0);
        if (nc) upload(o->d_P, P, nc, g.stream);
        g.h2d_bytes += (long long)(nc * sizeof(double2));
    }
    const double t2 = host_ms();
    // occluders: every triangle of every target object (OptiX.cpp:264-296)
    std::vector<std::array<float, 9>> tris;
    double maxc = 0.0;
    for (auto &o : g.obj[OBJ_TARGET])
        for (auto &F : o->facets) {
            std::array<float, 9> t = {F.v1.x, F.v1.y, F.v1.z, F.v2.x, F.v2.y, F.v2.z, F.v3.x, F.v3.y, F.v3.z};
            for (float v : t) maxc = std::max(maxc, (double)std::fabs(v));
            tris.push_back(t);
        }
    // convex target (every target vertex on or behind every target triangle's
    // plane): the masks' shadow tests then search only the part of a ray
    // where a crossing is possible
    g.scene_vmax = (float)maxc;
    g.scene_convex = scene_is_convex(tris, 1e-6 * (1.0 + maxc)) ? 1 : 0;
    for (auto &p : g.src) maxc = std::max({maxc, (double)std::fabs(p.x), (double)std::fabs(p.y), (double)std::fabs(p.z)});
    for (auto &p : g.fp) maxc = std::max({maxc, (double)std::fabs(p.x), (double)std::fabs(p.y), (double)std::fabs(p.z)});
    // node boxes padded by 1e-5 (1 + largest coordinate of triangles and points):
    // the FP32 slab test and the crossing point of a hit are within a few 1e-7
    // (1 + coordinate) of exact, so every box a hit needs is opened
    BvhHost bvh = build_bvh(tris, 1e-5 * (1.0 + maxc));
    g.ntri = (int)tris.size();
    g.nnodes = (int)bvh.nodes.size();
    g.d_nodes = dalloc<float4>(2 * bvh.nodes.size());
    g.d_tris = dalloc<float4>(bvh.tris.size());
    if (g.ntri) {
        CK(stage_to_device(g.d_nodes, bvh.nodes.data(), bvh.nodes.size() * sizeof(BvhNode), g.stream));
        CK(stage_to_device(g.d_tris, bvh.tris.data(), bvh.tris.size() * sizeof(float4), g.stream));
        g.h2d_bytes += (long long)(bvh.nodes.size() * sizeof(BvhNode) + bvh.tris.size() * sizeof(float4));
    }
    const double t3 = host_ms();
    g.render_ms[3] = t3 - t2;
    upload_points(g.src, g.d_src_pos, g.d_src_P, 1.0);  // unit source pressure (Model.cpp:16-19)
    g.fp_order = morton_order(g.fp);
    std::vector<Vec3> fp_sorted(g.fp.size());
    for (size_t k = 0; k < g.fp.size(); k++) fp_sorted[k] = g.fp[g.fp_order[k]];
    upload_points(fp_sorted, g.d_fp_pos, g.d_fp_P, 0.0);
    g.d_fp_order = dalloc<int>(g.fp_order.size());
    if (!g.fp_order.empty()) {
        CK(stage_to_device(g.d_fp_order, g.fp_order.data(), g.fp_order.size() * sizeof(int), g.stream));
    }
    CK(cudaStreamSynchronize(g.stream));
    host_arena_reset();  // every copy out of it is done
    g.render_ms[4] = host_ms() - t3;
    g.rendered = true;
}

// ---------------------------------------------------------------- hops
Object &get(int type, int idx)
{
    if (type < 0 || type > 2 || idx < 0 || idx >= (int)g.obj[type].size())
        fail(-4, "no object %d of type %d", idx, type);
    return *g.obj[type][idx];
}

struct HopSets {
    MaskArgs m{};
    int nsrc = 0, ndst = 0;
};

HopSets hop_sets(int hop, int a, int b)
{
    HopSets h;
    MaskArgs &m = h.m;
    m.hop = hop;
    m.bvh = BvhView{g.d_nodes, g.d_tris, g.nnodes, g.ntri};
    m.convex = g.opt_convex_masks ? g.scene_convex : 0;
    m.convex_vmax = g.scene_vmax;
    if (hop == HOP_SRC) {
        Object &B = get(a, b);  // a = object type (target or field), b = index
        m.nsrc = (int)g.src.size();
        m.src_pos = g.d_src_pos;
        m.ndst = (int)B.ncells;
        m.dst_pos = B.d_cell_pos;
        m.dst_facet = B.d_cell_facet;
        m.dst_facet_n = B.d_facet_n;
        m.dst_is_field = B.type == OBJ_FIELD;
    } else if (hop == HOP_FP) {
        Object &A = get(OBJ_TARGET, a);
        m.nsrc = A.nact();
        m.src_pos = A.d_act_pos;
        m.src_facet = A.d_act_facet;
        m.src_facet_n = A.d_facet_n;
        m.ndst = (int)g.fp.size();
        m.dst_pos = g.d_fp_pos;
    } else if (hop == HOP_F2F) {
        Object &A = get(OBJ_TARGET, a);
        m.nsrc = m.ndst = A.nact();
        m.src_pos = m.dst_pos = A.d_act_pos;
        m.src_facet = m.dst_facet = A.d_act_facet;
        m.src_facet_n = m.dst_facet_n = A.d_facet_n;
        m.src_frange = m.dst_frange = A.d_tile_frange;
    } else if (hop == HOP_RESP) {
        // FACET_RESP between two targets: sources of a, destinations of b; the
        // ray starts at the lower-index object's point
        if (a == b) fail(-6, "FACET_RESP needs two different target objects (got %d and %d)", a, b);
        Object &A = get(OBJ_TARGET, a);
        Object &B = get(OBJ_TARGET, b);
        m.nsrc = A.nact();
        m.src_pos = A.d_act_pos;
        m.src_facet = A.d_act_facet;
        m.src_facet_n = A.d_facet_n;
        m.ndst = B.nact();
        m.dst_pos = B.d_act_pos;
        m.dst_facet = B.d_act_facet;
        m.dst_facet_n = B.d_facet_n;
        m.resp_dst_origin = a > b ? 1 : 0;
    } else if (hop == HOP_PISTON_T || hop == HOP_PISTON_F) {
        // a piston source object's fragments -> the active cells of a target
        // (both cosine gates, the FACET_RESP form) or of a field object
        // (cos_inc = 1, the FACET_NO_RESP form); the ray starts at the
        // piston fragment.  The convex-target shortcuts assume rays that
        // leave or end on a target: off here.
        Object &A = get(OBJ_SOURCE, a);
        Object &B = get(hop == HOP_PISTON_T ? OBJ_TARGET : OBJ_FIELD, b);
        m.hop = hop == HOP_PISTON_T ? HOP_RESP : HOP_NORESP;
        m.convex = 0;
        m.nsrc = A.nact();
        m.src_pos = A.d_act_pos;
        m.src_facet = A.d_act_facet;
        m.src_facet_n = A.d_facet_n;
        m.ndst = B.nact();
        m.dst_pos = B.d_act_pos;
        m.dst_facet = B.d_act_facet;
        m.dst_facet_n = B.d_facet_n;
        m.dst_is_field = hop == HOP_PISTON_F ? 1 : 0;
        m.resp_dst_origin = 0;
    } else {
        Object &A = get(OBJ_TARGET, a);
        Object &B = get(OBJ_FIELD, b);
        m.nsrc = A.nact();
        m.src_pos = A.d_act_pos;
        m.src_facet = A.d_act_facet;
        m.src_facet_n = A.d_facet_n;
        m.ndst = B.nact();
        m.dst_pos = B.d_act_pos;
        m.dst_facet = B.d_act_facet;
        m.dst_facet_n = B.d_facet_n;
        m.dst_is_field = 1;
    }
    h.nsrc = m.nsrc;
    h.ndst = m.ndst;
    return h;
}

// Build one interaction mask.  full = 0: CLEAR blocks store no bits (the sum
// kernels evaluate their gates inline); full = 1: every block stores its bits
// (diagnostic export).
MaskEntry build_mask(int hop, int a, int b, int full, const MaskEntry *reuse = nullptr)
{
    HopSets hs = hop_sets(hop, a, b);
    MaskEntry e{};
    e.hop = hop;
    e.a = a;
    e.b = b;
    e.upper_only = (hop == HOP_F2F && !full && g.opt_f2f_sym) ? 1 : 0;
    e.nsrc = hs.nsrc;
    e.ndst = hs.ndst;
    MaskView &v = e.view;
    v.nwords = (hs.nsrc + 31) / 32;
    v.ntiles = (hs.nsrc + kTile - 1) / kTile;
    v.ndstblocks = (hs.ndst + kTile - 1) / kTile;
    v.pitch = ((long long)hs.ndst + 31) / 32 * 32;
    if (v.ntiles > 65535) fail(-3, "hop %d has %d sources (limit %d)", hop, hs.nsrc, 65535 * kTile);
    const size_t words = (size_t)v.ntiles * kWordsPerTile * (size_t)v.pitch;
    const size_t nflags = (size_t)v.ntiles * v.ndstblocks;
    if (reuse) {
        v.bits = reuse->view.bits;
        v.flags = reuse->view.flags;
        e.blist = reuse->blist;
        e.bcount = reuse->bcount;
    } else {
        v.bits = dalloc<uint32_t>(words);
        v.flags = dalloc<uint8_t>(nflags);
    }
    // bounce masks: one warp per block classifies, only the blocks that need
    // per-pair bits run the pair kernel
    const bool classify = hop == HOP_F2F && !full && g.opt_mask_classify;
    if (classify && !e.blist) {
        e.blist = dalloc<int2>(std::max<size_t>(nflags, 1));
        e.bcount = dalloc<int>(2);  // listed blocks, the pair kernel's next-block counter
    }
    // every block writes its flag, and the sums read bits only of blocks that
    // stored them; the full export also reads blocks that store none
    if (full) CK(cudaMemsetAsync(v.bits, 0, std::max<size_t>(words, 1) * sizeof(uint32_t), g.stream));
    hs.m.mask = v;
    hs.m.full = full;
    hs.m.gate_proj = g.opt_gate_proj;
    hs.m.upper_only = (hop == HOP_F2F && !full && g.opt_f2f_sym) ? 1 : 0;
    // timed by ev6 .. ev7, read after the hop that uses the mask (no host
    // synchronisation here); full exports are not timed, so that they leave
    // the events of a mask built for the next hop alone
    if (!full) CK(cudaEventRecord(g.ev6, g.stream));
    if (classify) {
        if (g.nsm == 0) {
            int dev = 0;
            CK(cudaGetDevice(&dev));
            CK(cudaDeviceGetAttribute(&g.nsm, cudaDevAttrMultiProcessorCount, dev));
        }
        g.launches += launch_mask_classified(hs.m, e.blist, e.bcount, g.nsm, g.stream);
    } else {
        launch_mask(hs.m, g.stream);
        g.launches += (hs.nsrc > 0 && hs.ndst > 0) ? 1 : 0;
    }
    CK(cudaGetLastError());
    if (!full) {
        CK(cudaEventRecord(g.ev7, g.stream));
        e.fresh = true;
    }
    if (g.opt_class_stats && nflags > 0) {
        CK(cudaStreamSynchronize(g.stream));
        std::vector<uint8_t> fl(nflags);
        CK(cudaMemcpy(fl.data(), v.flags, nflags, cudaMemcpyDeviceToHost));
        for (uint8_t f : fl) e.classes[f & 3]++;
    }
    return e;
}

MaskEntry &get_mask(int hop, int a, int b)
{
    const int upper = (hop == HOP_F2F && g.opt_f2f_sym) ? 1 : 0;
    for (auto &e : g.masks)
        if (e.hop == hop && e.a == a && e.b == b) {
            if (e.stale || e.upper_only != upper) e = build_mask(hop, a, b, 0, &e);
            return e;
        }
    g.masks.push_back(build_mask(hop, a, b, 0));
    return g.masks.back();
}

void ensure_scratch(int nsrc, int ndst, int nsplit)
{
    if ((size_t)nsrc > g.pack_cap) {
        dfree(g.d_packA);
        dfree(g.d_packB);
        g.d_packA = dalloc<float4>(nsrc);
        g.d_packB = dalloc<float4>(nsrc);
        g.pack_cap = nsrc;
    }
    const size_t np = (size_t)ndst * nsplit;
    if (np > g.partial_cap) {
        dfree(g.d_partial);
        g.d_partial = dalloc<double2>(np);
        g.partial_cap = np;
    }
    if ((size_t)ndst > g.limit_cap) {
        dfree(g.d_limit);
        g.d_limit = dalloc<int>(ndst);
        g.limit_cap = ndst;
    }
}

// Blocks per chunk of the symmetric bounce sum's work list.
constexpr int kSymChunk = 2;

// Work-list buffers for ntiles x ntiles blocks: at most ceil((J + 1) / per)
// chunks in row J.
void ensure_symwork(int ntiles)
{
    if (ntiles <= g.sym_tiles) return;
    dfree(g.d_blist); dfree(g.d_rowcnt); dfree(g.d_chunk_off); dfree(g.d_nchunks); dfree(g.d_chunks);
    dfree(g.d_rowpart);
    size_t maxch = 0;
    for (int J = 0; J < ntiles; J++) maxch += (size_t)(J + kSymChunk) / kSymChunk;
    g.d_blist = dalloc<int>((size_t)ntiles * ntiles);
    g.d_rowcnt = dalloc<int>(ntiles);
    g.d_chunk_off = dalloc<int>(ntiles + 1);
    g.d_nchunks = dalloc<int>(2);  // chunk count, next-chunk counter
    g.d_chunks = dalloc<int4>(maxch);
    g.d_rowpart = dalloc<double2>(maxch * kTile);
    g.sym_tiles = ntiles;
    if (g.nsm == 0) {
        int dev = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&g.nsm, cudaDevAttrMultiProcessorCount, dev));
    }
}

void ensure_colpart(int ntiles)
{
    const size_t n = (size_t)kTile * ntiles * (ntiles > 0 ? ntiles - 1 : 0) / 2;
    if (n > g.colpart_cap) {
        dfree(g.d_colpart);
        g.d_colpart = dalloc<double2>(n);
        g.colpart_cap = n;
    }
}

// Choose and compress blocks of a FACET_SELF hop (upper blocks I < J).
// Candidates: with the rule (select 0), blocks whose every pair interacts
// (mask class ALL) and whose tile centroids are farther apart than
// eta (r_I + r_J); otherwise every interacting off-diagonal block.  With the
// network (select 2) each candidate's descriptors go through the
// admissibility network, which predicts log2(1 + rank): blocks predicted
// below the rank cut are approximated with a rank cap from the prediction,
// the rest stay dense without an attempt.  Every approximated block is
// built by adaptive cross approximation and judged on sampled exact entries;
// accepted blocks leave the dense kernel's flags.  The lists are built on the
// device (select.cu); the host reads back only the kept-block count and the
// factor-column total, to size the factor arrays.  Statistics (and, for
// select 1, the training samples: descriptors with log2(1 + rank) labels,
// log2(1 + 2 cap) when rejected) are read after the hop (finish_compression).
void build_compression(int a, MaskEntry &M, const SumArgs &s)
{
    Compression &C = g.cmp;
    C.release();
    const int nt = M.view.ntiles, nb = M.view.ndstblocks;
    const int rmax = std::min(g.opt_cmp_rmax, kLrRankLimit);
    const int select = g.opt_cmp_select;
    if (select == 2 && !mlp_ready())
        fail(-2, "compress_select 2 needs the admissibility network's parameters (train or load them first)");
    cudaStream_t st = g.stream;
    CK(cudaEventRecord(g.evb[0], st));
    // every upper block I < J, I < nt
    const size_t nmax = std::max<size_t>((size_t)nt * (nt - 1) / 2 + (size_t)nt * std::max(nb - nt, 0), 1);
    const size_t ngrid = (size_t)nt * nb;
    {
        size_t bytes = 2 * Arena::bytes_of(nt, sizeof(float4)) + 6 * Arena::bytes_of(nb + 1, sizeof(int)) +
                       2 * Arena::bytes_of(nt + 1, sizeof(int)) + 2 * Arena::bytes_of(nmax, sizeof(int2)) +
                       2 * Arena::bytes_of(nmax, 1) + Arena::bytes_of(nmax * 8, sizeof(float)) +
                       Arena::bytes_of(nmax, sizeof(float)) + Arena::bytes_of(nmax, sizeof(long long)) +
                       9 * Arena::bytes_of(nmax, sizeof(int)) + 3 * Arena::bytes_of(nmax, sizeof(float)) +
                       Arena::bytes_of(nmax * 64, 1) + 2 * Arena::bytes_of(ngrid, 1) +
                       Arena::bytes_of(ngrid, sizeof(int)) + 2 * Arena::bytes_of(M.nsrc, sizeof(double2)) +
                       Arena::bytes_of((size_t)kCmpStats * cmp_stats_parts(), sizeof(double)) +
                       Arena::bytes_of((size_t)kIpTileRec * nt, sizeof(float4)) + Arena::bytes_of(M.nsrc, sizeof(uint16_t)) +
                       2 * Arena::bytes_of(nmax, 1) + 2 * Arena::bytes_of(nmax, sizeof(int)) +
                       2 * Arena::bytes_of(nb + 1, sizeof(int)) + Arena::bytes_of(1, sizeof(int)) + 8192;
        C.arena.reserve(bytes);
    }
    Arena &ar = C.arena;
    float4 *d_cen = ar.take<float4>(nt), *d_nm = ar.take<float4>(nt);
    launch_tile_stats(g.d_packA, g.d_packB, M.nsrc, d_cen, d_nm, st);
    // interpolated blocks: far class-ALL blocks between planar tiles (not
    // when the cross approximation labels training blocks)
    Object &A = get(OBJ_TARGET, a);
    C.interp = g.opt_cmp_interp && select != 1;
    C.d_lev = nullptr;
    C.ip = IpCtx{};
    if (C.interp) {
        C.ip.tile = ar.take<float4>((size_t)kIpTileRec * nt);
        uint16_t *fxy = ar.take<uint16_t>(M.nsrc);
        launch_ip_tiles(g.d_packA, g.d_packB, A.d_act_facet, A.d_act_cell, A.d_facet_grid, M.nsrc, A.delta,
                        g.opt_ip_transpose != 0, const_cast<float4 *>(C.ip.tile), fxy, st);
        C.ip.fxy = fxy;
        C.ip.delta = A.delta;
        C.ip.status = ar.take<int>(1);
        CK(cudaMemsetAsync(C.ip.status, 0, sizeof(int), st));
    }
    // ---- candidates
    int *d_ccnt = ar.take<int>(nb), *d_coff = ar.take<int>(nb + 1);
    int2 *d_cblocks = ar.take<int2>(nmax);
    uint8_t *d_ccls = ar.take<uint8_t>(nmax);
    launch_cand_lists(M.view.flags, nt, nb, select, g.opt_cmp_eta, d_cen, d_ccnt, d_coff, d_cblocks, d_ccls, st);
    C.d_desc = ar.take<float>(nmax * 8);
    const float inv_lambda = (float)(g.kr / (2.0 * M_PI));
    launch_block_desc(s, d_cblocks, d_ccls, (int)nmax, d_cen, d_nm, inv_lambda, C.d_desc, st, d_coff + nb);
    float *d_pred = nullptr;
    if (select == 2) {
        d_pred = ar.take<float>(nmax);
        CK(mlp_infer_dev(C.d_desc, (int)nmax, d_pred, st));  // rows past the candidate count are not read
    }
    uint8_t *d_clev = nullptr;
    if (C.interp) {
        d_clev = ar.take<uint8_t>(nmax);
        launch_ip_level(d_cblocks, d_ccls, d_coff + nb, (int)nmax, C.ip.tile, A.delta, (float)g.kr, g.opt_cmp_tol,
                        d_clev, st);
        C.d_lev = ar.take<uint8_t>(nmax);
        C.ip.lev = C.d_lev;
    }
    // ---- kept blocks, rank caps, factor columns
    int *d_kcnt = ar.take<int>(nb), *d_ksum = ar.take<int>(nb);
    int *d_koff = ar.take<int>(nb + 1), *d_kcol = ar.take<int>(nb + 1);
    C.d_blocks = ar.take<int2>(nmax);
    C.d_cls = ar.take<uint8_t>(nmax);
    C.d_acap = ar.take<int>(nmax);
    C.d_off = ar.take<long long>(nmax);
    C.d_kmap = ar.take<int>(nmax);
    const float cut = std::log2(1.0f + g.opt_cmp_rcut);
    launch_keep_lists(nb, d_coff, d_pred, cut, rmax, d_cblocks, d_ccls, d_kcnt, d_ksum, d_koff, d_kcol, C.d_blocks,
                      C.d_cls, C.d_acap, C.d_off, C.d_kmap, st, d_clev, C.d_lev);
    int *d_ioff = nullptr;
    C.d_aca_list = C.d_ip_list = nullptr;
    if (C.interp) {
        // each kind's kernels get grids of their own blocks only
        int *d_icnt = ar.take<int>(nb);
        d_ioff = ar.take<int>(nb + 1);
        C.d_aca_list = ar.take<int>(nmax);
        C.d_ip_list = ar.take<int>(nmax);
        launch_split_kept(nb, d_koff, C.d_lev, d_icnt, d_ioff, C.d_aca_list, C.d_ip_list, st);
    }
    CK(cudaEventRecord(g.evb[1], st));
    int hcnt[4] = {0, 0, 0, 0};  // candidates, kept blocks, factor columns, interpolated kept blocks
    CK(cudaMemcpyAsync(&hcnt[0], d_coff + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&hcnt[1], d_koff + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&hcnt[2], d_kcol + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (d_ioff) CK(cudaMemcpyAsync(&hcnt[3], d_ioff + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const int n = hcnt[1];
    const long long cols = hcnt[2];
    C.nip_kept = C.interp ? hcnt[3] : 0;
    C.naca_kept = n - C.nip_kept;
    C.ip.list = C.d_ip_list;
    C.ip.n = C.nip_kept;
    C.select = select;
    C.ncand = hcnt[0];
    C.nblocks = n;
    C.ncols = cols;
    C.rmax = rmax;
    C.obj = a;
    C.kr = g.kr;
    C.ki = g.ki;
    // ---- cross approximation of the kept blocks
    C.factors.reserve(2 * Arena::bytes_of((size_t)std::max<long long>(cols, 1) * kTile, sizeof(float2)) +
                      2 * Arena::bytes_of((size_t)std::max(n, 1) * kTile, sizeof(float2)));
    C.d_U = C.factors.take<float2>((size_t)std::max<long long>(cols, 1) * kTile);
    C.d_V = C.factors.take<float2>((size_t)std::max<long long>(cols, 1) * kTile);
    C.d_brow = C.factors.take<float2>((size_t)std::max(n, 1) * kTile);
    C.d_bcol = C.factors.take<float2>((size_t)std::max(n, 1) * kTile);
    C.d_rank = ar.take<int>(nmax);
    C.d_fro = ar.take<float>(nmax);
    C.d_err = ar.take<float>(nmax);
    // the interpolated blocks on the second stream beside the cross
    // approximation (disjoint blocks and output slots; each kernel writes the
    // rank, error and outputs of its own blocks only)
    const bool ip_side = C.interp && g.opt_overlap && g.opt_build_overlap;
    const cudaStream_t ist = ip_side ? g.side : st;
    if (ip_side) {
        CK(cudaEventRecord(g.ev_fork, st));
        CK(cudaStreamWaitEvent(g.side, g.ev_fork, 0));
    }
    // the panel kernels also apply the accepted blocks to this bounce's packed
    // inputs: the first bounce's low-rank apply then only gathers
    C.outputs_ready = launch_aca(s, C.d_blocks, C.d_cls, C.d_acap, C.d_off, C.interp ? C.naca_kept : n, g.opt_cmp_tol,
                                 C.d_U, C.d_V, C.d_rank, C.d_fro, g.opt_cmp_judge, C.d_err, st, g.opt_aca_variant,
                                 g.opt_fused_apply ? C.d_brow : nullptr, g.opt_fused_apply ? C.d_bcol : nullptr,
                                 C.d_aca_list);
    CK(cudaGetLastError());
    CK(cudaEventRecord(g.evb[2], st));
    if (C.interp) {
        // node entries, judge, and the fused apply when the cross
        // approximation applies its own blocks too
        const bool fused = C.outputs_ready;
        CK(cudaEventRecord(g.evb[5], ist));
        launch_ip_build(s, C.ip.tile, C.ip.fxy, C.ip.lev, A.delta, C.d_blocks, C.d_off, C.nip_kept, g.opt_cmp_judge,
                        C.d_U, C.d_rank, C.d_fro, C.d_err, fused ? C.d_brow : nullptr, fused ? C.d_bcol : nullptr, ist,
                        C.d_ip_list);
        CK(cudaGetLastError());
    } else {
        CK(cudaEventRecord(g.evb[5], ist));
    }
    CK(cudaEventRecord(g.evb[4], ist));
    if (ip_side) {
        CK(cudaEventRecord(g.ev_join, g.side));
        CK(cudaStreamWaitEvent(st, g.ev_join, 0));
    }
    CK(cudaEventRecord(g.evb[6], st));
    // ---- accepted blocks: dense flags off, owner lists, statistics
    C.d_flags = ar.take<uint8_t>(ngrid);
    CK(cudaMemcpyAsync(C.d_flags, M.view.flags, ngrid, cudaMemcpyDeviceToDevice, st));
    uint8_t *d_accbm = ar.take<uint8_t>(ngrid);
    int *d_qidx = ar.take<int>(ngrid);
    int *d_acnt = ar.take<int>(nb), *d_icnt = ar.take<int>(nt);
    C.d_byJ_off = ar.take<int>(nb + 1);
    C.d_byI_off = ar.take<int>(nt + 1);
    C.d_bidx = ar.take<int>(nmax);
    C.d_byJ = ar.take<int>(nmax);
    C.d_byI = ar.take<int>(nmax);
    launch_accept_lists(nt, nb, d_koff, C.d_blocks, C.d_rank, C.d_flags, d_accbm, d_qidx, d_acnt, C.d_byJ_off, C.d_bidx,
                        C.d_byJ, d_icnt, C.d_byI_off, C.d_byI, st);
    C.d_nacc = C.d_byJ_off + nb;
    C.d_stats = ar.take<double>((size_t)kCmpStats * cmp_stats_parts());
    launch_cmp_stats(d_koff + nb, C.d_blocks, C.d_rank, C.d_err, M.nsrc, C.d_stats, st, C.d_lev);
    C.d_yrow = ar.take<double2>(M.nsrc);
    C.d_ycol = ar.take<double2>(M.nsrc);
    CK(cudaEventRecord(g.evb[3], st));
    C.valid = true;
    C.stats_pending = true;
}

// a failed wait in the tensor-core inference kernel becomes an error
static void check_mlp_status()
{
    const int st = mlp_take_status();
    if (st) fail(-10, "network inference on the tensor cores timed out (status %d)", st);
}

// Statistics, timings and (select 1) training samples of the last build,
// once the stream has passed it.
void finish_compression()
{
    Compression &C = g.cmp;
    if (!C.stats_pending) return;
    C.stats_pending = false;
    if (C.select == 2) check_mlp_status();
    std::vector<double> part((size_t)kCmpStats * cmp_stats_parts());
    CK(cudaMemcpy(part.data(), C.d_stats, part.size() * sizeof(double), cudaMemcpyDeviceToHost));
    double st[kCmpStats] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (size_t b = 0; b < part.size() / kCmpStats; b++)
        for (int q = 0; q < kCmpStats; q++)
            st[q] = q == 2 ? std::max(st[q], part[kCmpStats * b + q]) : st[q] + part[kCmpStats * b + q];
    C.naccepted = (int)st[0];
    C.nip = (int)st[4];
    C.mean_rank = st[0] - st[4] > 0.0 ? st[1] / (st[0] - st[4]) : 0.0;  // of the cross-approximated blocks
    C.ip_mean_nodes = st[4] > 0.0 ? st[5] / st[4] : 0.0;
    C.max_err = st[2];
    C.pairs_cmp = st[3];
    CK(cudaEventElapsedTime(&C.build_ms, g.evb[0], g.evb[3]));
    CK(cudaEventElapsedTime(&C.select_ms, g.evb[0], g.evb[1]));
    CK(cudaEventElapsedTime(&C.aca_ms, g.evb[1], g.evb[2]));
    CK(cudaEventElapsedTime(&C.ip_ms, g.evb[5], g.evb[4]));
    CK(cudaEventElapsedTime(&C.approx_ms, g.evb[1], g.evb[6]));
    C.desc.clear();
    C.label.clear();
    if (C.select == 1 && C.nblocks > 0) {
        const int n = C.nblocks;
        std::vector<float> desc((size_t)C.ncand * 8);
        std::vector<int> kmap(n), rank(n), cap(n);
        CK(cudaMemcpy(desc.data(), C.d_desc, desc.size() * sizeof(float), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(kmap.data(), C.d_kmap, n * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(rank.data(), C.d_rank, n * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(cap.data(), C.d_acap, n * sizeof(int), cudaMemcpyDeviceToHost));
        C.desc.resize((size_t)n * 8);
        C.label.resize(n);
        for (int b = 0; b < n; b++) {
            std::copy(desc.begin() + (size_t)kmap[b] * 8, desc.begin() + (size_t)kmap[b] * 8 + 8,
                      C.desc.begin() + (size_t)b * 8);
            C.label[b] = rank[b] > 0 ? std::log2(1.0f + (float)rank[b]) : std::log2(1.0f + 2.0f * (float)cap[b]);
        }
    }
}

int choose_split(int ntiles, int ndstblocks)
{
    if (g.opt_split > 0) return std::min(g.opt_split, std::max(ntiles, 1));
    // aim for ~16 resident-CTA waves' worth of CTAs on 152 SMs, at least 2 tiles per split
    const int want = (2432 + ndstblocks - 1) / std::max(ndstblocks, 1);
    return std::max(1, std::min(want, std::max(1, ntiles / 2)));
}

long long pair_count(int hop, int a, int b)
{
    if (hop == HOP_SRC) return (long long)g.src.size() * get(a, b).ncells;
    if (hop == HOP_FP) return (long long)get(OBJ_TARGET, a).nact() * (long long)g.fp.size();
    if (hop == HOP_F2F) {
        Object &A = get(OBJ_TARGET, a);
        long long tot = A.nact(), sq = 0;
        for (long long n : A.facet_nact) sq += n * n;
        return tot * tot - sq;
    }
    if (hop == HOP_RESP) return (long long)get(OBJ_TARGET, a).nact() * get(OBJ_TARGET, b).nact();
    if (hop == HOP_PISTON_T) return (long long)get(OBJ_SOURCE, a).nact() * get(OBJ_TARGET, b).nact();
    if (hop == HOP_PISTON_F) return (long long)get(OBJ_SOURCE, a).nact() * get(OBJ_FIELD, b).nact();
    return (long long)get(OBJ_TARGET, a).nact() * get(OBJ_FIELD, b).nact();
}

// The sum kernel bracketed by its own events (per-launch duration of the
// dominant kernel).
void timed_sum(const SumArgs &s, cudaStream_t st)
{
    CK(cudaEventRecord(g.ev2, st));
    launch_sum(s, st);
    CK(cudaEventRecord(g.ev3, st));
}

// One hop: mask (cached), pack the source weights, sum, finalize.
void run_hop(int hop, int a, int b)
{
    MaskEntry &M = get_mask(hop, a, b);
    const bool mask_rebuilt = M.fresh;  // built for this call (reported once)
    float rec_cmp_build = 0.0f;
    bool rec_cmp = false, built = false;
    if (M.nsrc == 0 || M.ndst == 0) return;
    HopSets hs = hop_sets(hop, a, b);
    SumArgs s{};
    s.hop = hs.m.hop;  // the kernels' hop (the piston hops run as FACET_RESP / FACET_NO_RESP)
    s.nsrc = M.nsrc;
    s.ndst = M.ndst;
    s.dst_pos = hs.m.dst_pos;
    s.dst_facet = hs.m.dst_facet;
    s.dst_facet_n = hs.m.dst_facet_n;
    s.dst_is_field = hs.m.dst_is_field;
    s.mask = M.view;
    s.kr = (float)g.kr;
    s.ka = (float)g.ki;
    const double k2 = g.kr / (2.0 * M_PI);
    s.k2hi = (float)k2;
    s.k2lo = (float)(k2 - (double)s.k2hi);
    s.kr4pi = (float)(g.kr / (4.0 * M_PI));
    s.nsplit = choose_split(M.view.ntiles, M.view.ndstblocks);
    s.tiles_per_split = (M.view.ntiles + s.nsplit - 1) / s.nsplit;
    s.nsplit = (M.view.ntiles + s.tiles_per_split - 1) / s.tiles_per_split;
    ensure_scratch(M.nsrc, M.ndst, s.nsplit);
    s.srcA = g.d_packA;
    s.srcB = g.d_packB;
    s.partial = g.d_partial;
    s.dst_limit = g.d_limit;
    cudaStream_t st = g.stream;

    CK(cudaEventRecord(g.ev0, st));
    s.rel = (g.opt_rel_geom && (hop == HOP_SRC || hop == HOP_FP)) ? 1 : 0;
    s.k2pi = k2;
    if (hop == HOP_SRC) {
        launch_pack_points(g.d_src_pos, g.d_src_P, M.nsrc, g.d_packA, g.d_packB, st);
        timed_sum(s, st);
        launch_finalize_add(g.d_partial, s.nsplit, M.ndst, nullptr, get(a, b).d_P, st);
    } else if (hop == HOP_FP) {
        Object &A = get(OBJ_TARGET, a);
        launch_pack_frags(A.d_act_pos, A.d_act_facet, A.d_act_cell, A.d_facet_n, A.d_P, 1.0f, M.nsrc, g.d_packA,
                          g.d_packB, st);
        if (s.rel) {
            // reference points of the relative geometry: the centroid of every source tile
            const size_t nt = (size_t)M.view.ntiles;
            if (nt > g.tilecen_cap) {
                dfree(g.d_tilecen);
                dfree(g.d_tilenm);
                g.d_tilecen = dalloc<float4>(nt);
                g.d_tilenm = dalloc<float4>(nt);
                g.tilecen_cap = nt;
            }
            launch_tile_stats(g.d_packA, g.d_packB, M.nsrc, g.d_tilecen, g.d_tilenm, st);
            s.tile_cen = g.d_tilecen;
        }
        timed_sum(s, st);
        launch_finalize_add(g.d_partial, s.nsplit, M.ndst, g.d_fp_order, g.d_fp_P, st);
    } else if (hop == HOP_F2F) {
        Object &A = get(OBJ_TARGET, a);
        s.rmin = A.delta;
        launch_f2f_limits(A.d_act_facet, A.d_act_cell, A.d_facet_end, A.d_Pin, M.ndst, M.nsrc, g.d_limit, st);
        launch_pack_frags(A.d_act_pos, A.d_act_facet, A.d_act_cell, A.d_facet_n, A.d_Pin, 0.9f, M.nsrc, g.d_packA,
                          g.d_packB, st);
        if (g.opt_f2f_sym) {
            ensure_colpart(M.view.ntiles);
            const double2 *yrow = nullptr, *ycol = nullptr;
            if (g.opt_compress) {
                Compression &C = g.cmp;
                if (!C.valid || C.obj != a || C.kr != g.kr || C.ki != g.ki || mask_rebuilt) {
                    build_compression(a, M, s);
                    built = true;
                }
                s.mask.flags = C.d_flags;  // accepted blocks are left to the low-rank path
                // both paths read the packed inputs and write their own buffers;
                // the finalize below waits for the low-rank stream
                cudaStream_t lst = st;
                if (g.opt_overlap) {
                    CK(cudaEventRecord(g.ev_fork, st));
                    CK(cudaStreamWaitEvent(g.side, g.ev_fork, 0));
                    lst = g.side;
                }
                CK(cudaEventRecord(g.ev4, lst));
                // the interpolated blocks' apply on a third stream beside the
                // factor stream (compute- and memory-bound work side by side)
                IpCtx ipc = C.ip;
                if (g.opt_overlap) {
                    ipc.stream = g.side2;
                    ipc.fork = g.ev_fork2;
                    ipc.join = g.ev_join2;
                }
                launch_lr_apply(s, C.d_blocks, C.d_off, C.d_bidx, C.nblocks, C.d_U, C.d_V, C.d_rank, C.d_brow, C.d_bcol,
                                M.view.ndstblocks, C.d_byJ_off, C.d_byJ, C.d_byI_off, C.d_byI, C.d_yrow, C.d_ycol, lst,
                                C.d_nacc, built && C.outputs_ready, g.opt_lr_ctas, C.interp ? &ipc : nullptr,
                                C.interp ? C.d_aca_list : nullptr, C.naca_kept);
                CK(cudaEventRecord(g.ev5, lst));
                if (g.opt_overlap) CK(cudaEventRecord(g.ev_join, lst));
                yrow = C.d_yrow;
                ycol = C.d_ycol;
                rec_cmp = true;
            }
            // work list of the non-empty blocks (the dense kernel's flags)
            ensure_symwork(M.view.ntiles);
            launch_sym_worklist(s.mask.flags, M.view.ntiles, M.view.ndstblocks, kSymChunk, g.d_blist, g.d_rowcnt,
                                g.d_chunk_off, g.d_chunks, g.d_nchunks, st);
            const SymWork wl{g.d_blist, g.d_chunks, g.d_nchunks, M.view.ntiles, g.d_nchunks + 1};
            CK(cudaEventRecord(g.ev2, st));
            launch_sum_f2f_sym(s, wl, 3 * g.nsm, g.d_colpart, g.d_rowpart, st);
            CK(cudaEventRecord(g.ev3, st));
            if (yrow && g.opt_overlap) CK(cudaStreamWaitEvent(st, g.ev_join, 0));
            launch_finalize_f2f_sym(g.d_rowpart, g.d_chunk_off, M.ndst, g.d_colpart, s.mask.flags, M.view.ntiles,
                                    A.d_act_cell, A.d_Pin, A.d_Pout, A.d_P, st, yrow, ycol);
        } else {
            timed_sum(s, st);
            launch_finalize_f2f(g.d_partial, s.nsplit, M.ndst, A.d_act_cell, A.d_Pout, A.d_P, st);
        }
    } else if (hop == HOP_PISTON_T || hop == HOP_PISTON_F) {
        // a piston source object (unit pressure, 0.9 A_i weights as every
        // facet -> facet projection) into the active cells of a target or a
        // field object; r_min is the piston's delta
        Object &A = get(OBJ_SOURCE, a);
        Object &B = get(hop == HOP_PISTON_T ? OBJ_TARGET : OBJ_FIELD, b);
        s.rmin = A.delta;
        launch_pack_frags(A.d_act_pos, A.d_act_facet, A.d_act_cell, A.d_facet_n, A.d_P, 0.9f, M.nsrc, g.d_packA,
                          g.d_packB, st);
        timed_sum(s, st);
        launch_finalize_add(g.d_partial, s.nsplit, M.ndst, B.d_act_cell, B.d_P, st);
    } else if (hop == HOP_RESP) {
        // FACET_RESP, one direction: sources of target a (their P_in, 0.9 A_i),
        // destinations of target b; r_min is the delta of the lower-index
        // object (the reference's source object of the FACET_RESP call)
        Object &A = get(OBJ_TARGET, a);
        Object &B = get(OBJ_TARGET, b);
        s.rmin = get(OBJ_TARGET, std::min(a, b)).delta;
        launch_pack_frags(A.d_act_pos, A.d_act_facet, A.d_act_cell, A.d_facet_n, A.d_Pin, 0.9f, M.nsrc, g.d_packA,
                          g.d_packB, st);
        timed_sum(s, st);
        // reciprocal direction (into the lower-index object): gated by its P_in
        launch_finalize_resp(g.d_partial, s.nsplit, M.ndst, B.d_act_cell, a > b ? B.d_Pin : nullptr, B.d_Pout, B.d_P,
                             st);
    } else {
        Object &A = get(OBJ_TARGET, a);
        Object &B = get(OBJ_FIELD, b);
        s.rmin = A.delta;
        launch_pack_frags(A.d_act_pos, A.d_act_facet, A.d_act_cell, A.d_facet_n, A.d_P, 0.9f, M.nsrc, g.d_packA,
                          g.d_packB, st);
        timed_sum(s, st);
        launch_finalize_add(g.d_partial, s.nsplit, M.ndst, B.d_act_cell, B.d_P, st);
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(g.ev1, st));
    CK(cudaEventSynchronize(g.ev1));
    if (rec_cmp && g.cmp.interp && g.cmp.ip.status) {
        int ist = 0;
        CK(cudaMemcpy(&ist, g.cmp.ip.status, sizeof(int), cudaMemcpyDeviceToHost));
        if (ist) fail(-10, "interpolated blocks: a node-entry copy %s", ist == 2 ? "did not arrive" : "arrived late");
    }
    if (built) {
        finish_compression();
        rec_cmp_build = g.cmp.build_ms;
    }
    float ms = 0.0f, sum_ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, g.ev0, g.ev1));
    CK(cudaEventElapsedTime(&sum_ms, g.ev2, g.ev3));
    if (M.fresh) CK(cudaEventElapsedTime(&M.mask_ms, g.ev6, g.ev7));
    const int lr_launches = rec_cmp ? (built && g.cmp.outputs_ready ? 1 : 2 + (g.cmp.interp ? 1 : 0)) : 0;
    const int nl = (hop == HOP_F2F ? (g.opt_f2f_sym ? 6 : 4) : 3) + (M.fresh ? 1 : 0) + lr_launches;
    g.launches += (hop == HOP_F2F ? (g.opt_f2f_sym ? 6 : 4) : 3) + lr_launches +
                  (rec_cmp_build > 0.0f ? 4 + (g.cmp.interp ? 3 : 0) : 0);
    HopRecord rec{hop, pair_count(hop, a, b), M.mask_ms, sum_ms, ms, s.nsplit, nl};
    if (rec_cmp) {
        rec.cmp_cand = g.cmp.ncand;
        rec.cmp_blocks = g.cmp.nblocks;
        rec.cmp_accepted = g.cmp.naccepted;
        rec.cmp_select = g.cmp.select;
        rec.cmp_mean_rank = g.cmp.mean_rank;
        rec.cmp_ip_blocks = g.cmp.nip;
        rec.cmp_ip_kept = g.cmp.nip_kept;
        rec.cmp_ip_nodes = g.cmp.ip_mean_nodes;
        rec.cmp_max_err = g.cmp.max_err;
        rec.cmp_pairs = g.cmp.pairs_cmp;
        rec.cmp_build_ms = rec_cmp_build;
        if (rec_cmp_build > 0.0f) {
            rec.cmp_select_ms = g.cmp.select_ms;
            rec.cmp_aca_ms = g.cmp.aca_ms;
            rec.cmp_ip_ms = g.cmp.ip_ms;
            rec.cmp_approx_ms = g.cmp.approx_ms;
        }
        CK(cudaEventElapsedTime(&rec.lr_ms, g.ev4, g.ev5));
    }
    g.log.push_back(rec);
    M.mask_ms = 0.0f;  // reported once, with the first use
    M.fresh = false;
}

void need_render()
{
    if (!g.rendered) fail(-5, "render_cuda has not been called");
}

// ---------------------------------------------------------------- headless rendering
// glm::perspective(radians(45), width / height, 0.1, 10000) times
// glm::lookAt(eye, centre, up) (src/ModelGl.cpp:98-106), row-major.
void camera_matrix(int width, int height, const float *vs, float *M)
{
    const float fovy = 45.0f * (float)M_PI / 180.0f, aspect = (float)width / (float)height;
    const float zn = 0.1f, zf = 10000.0f, th = std::tan(fovy / 2.0f);
    float P[16] = {1.0f / (aspect * th), 0, 0, 0, 0, 1.0f / th, 0, 0, 0, 0, -(zf + zn) / (zf - zn),
                   -(2.0f * zf * zn) / (zf - zn), 0, 0, -1.0f, 0};
    const float ex = vs[0], ey = vs[1], ez = vs[2];
    float fx = vs[3] - ex, fy = vs[4] - ey, fz = vs[5] - ez;
    float L = std::sqrt(fx * fx + fy * fy + fz * fz);
    if (!(L > 0.0f)) fail(-6, "view settings: the camera looks at its own position");
    fx /= L; fy /= L; fz /= L;
    const float ux0 = vs[6], uy0 = vs[7], uz0 = vs[8];
    float sx = fy * uz0 - fz * uy0, sy = fz * ux0 - fx * uz0, sz = fx * uy0 - fy * ux0;
    L = std::sqrt(sx * sx + sy * sy + sz * sz);
    if (!(L > 0.0f)) fail(-6, "view settings: the up vector is parallel to the view direction");
    sx /= L; sy /= L; sz /= L;
    const float ux = sy * fz - sz * fy, uy = sz * fx - sx * fz, uz = sx * fy - sy * fx;
    const float V[16] = {sx, sy, sz, -(sx * ex + sy * ey + sz * ez), ux, uy, uz, -(ux * ex + uy * ey + uz * ez),
                         -fx, -fy, -fz, fx * ex + fy * ey + fz * ez, 0, 0, 0, 1};
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            float acc = 0.0f;
            for (int k = 0; k < 4; k++) acc += P[4 * r + k] * V[4 * k + c];
            M[4 * r + c] = acc;
        }
}

// The picture RenderOpenGL draws, into rgb (height x width x 3, top row first).
void render_image(int width, int height, const float *vs, unsigned char *rgb_host)
{
    need_render();
    if (width <= 0 || height <= 0 || (long long)width * height > (1LL << 28))
        fail(-6, "render: image size %d x %d out of range", width, height);
    if (!vs || !rgb_host) fail(-6, "render: null argument");
    for (int k = 0; k < 9; k++)
        if (!std::isfinite(vs[k])) fail(-6, "render: non-finite view setting");
    RasterArgs ra{};
    camera_matrix(width, height, vs, ra.mvp);
    ra.width = width;
    ra.height = height;
    // triangles and textures: target objects, then field objects (ModelGl.cpp:311-319)
    std::vector<RasterTri> tris;
    std::vector<RasterTex> tex;
    long long cells = 0;
    std::vector<std::pair<Object *, long long>> objs;
    for (int t : {OBJ_TARGET, OBJ_FIELD})
        for (auto &o : g.obj[t]) {
            objs.push_back({o.get(), cells});
            for (size_t f = 0; f < o->facets.size(); f++) {
                const FacetFrame &F = o->facets[f];
                RasterTri T{};
                const Vec3 vv[3] = {F.v1, F.v2, F.v3};
                // texture coordinates: base origin (0, 0), base end (1, 0), apex
                // (BaseLengthNeg / BaseLength, 1) (src/Facet.cpp:18-60)
                const float e[3] = {std::sqrt((F.v1.x - F.v2.x) * (F.v1.x - F.v2.x) + (F.v1.y - F.v2.y) * (F.v1.y - F.v2.y) +
                                              (F.v1.z - F.v2.z) * (F.v1.z - F.v2.z)),
                                    std::sqrt((F.v1.x - F.v3.x) * (F.v1.x - F.v3.x) + (F.v1.y - F.v3.y) * (F.v1.y - F.v3.y) +
                                              (F.v1.z - F.v3.z) * (F.v1.z - F.v3.z)),
                                    std::sqrt((F.v2.x - F.v3.x) * (F.v2.x - F.v3.x) + (F.v2.y - F.v3.y) * (F.v2.y - F.v3.y) +
                                              (F.v2.z - F.v3.z) * (F.v2.z - F.v3.z))};
                int m = 0;
                if (e[1] > e[m]) m = 1;
                if (e[2] > e[m]) m = 2;
                const int origin = m == 2 ? 1 : 0, end = m == 0 ? 1 : 2, apex = m == 0 ? 2 : (m == 1 ? 1 : 0);
                const float ua = F.baseNeg / (F.basePos + F.baseNeg);
                for (int k = 0; k < 3; k++) T.v[k] = make_float4(vv[k].x, vv[k].y, vv[k].z, 1.0f);
                T.uv[origin] = make_float2(0.0f, 0.0f);
                T.uv[end] = make_float2(1.0f, 0.0f);
                T.uv[apex] = make_float2(ua, 1.0f);
                T.facet = (int)tex.size();
                tris.push_back(T);
                tex.push_back(RasterTex{cells + o->cell0[f], std::max(F.nx, 1), std::max(F.ny, 1)});
            }
            cells += o->ncells;
        }
    // work list: 32 x 32-pixel tiles of each triangle's screen box
    const int tile = raster_tile();
    std::vector<int4> work;
    for (size_t i = 0; i < tris.size(); i++) {
        float xmin = 3e38f, xmax = -3e38f, ymin = 3e38f, ymax = -3e38f;
        bool ok = true;
        for (int k = 0; k < 3; k++) {
            const float4 v = tris[i].v[k];
            const float *M = ra.mvp;
            const float cx = M[0] * v.x + M[1] * v.y + M[2] * v.z + M[3];
            const float cy = M[4] * v.x + M[5] * v.y + M[6] * v.z + M[7];
            const float cw = M[12] * v.x + M[13] * v.y + M[14] * v.z + M[15];
            if (!(cw > 0.1f)) ok = false;
            const float sx = (cx / cw + 1.0f) * 0.5f * width, sy = (cy / cw + 1.0f) * 0.5f * height;
            xmin = std::min(xmin, sx); xmax = std::max(xmax, sx);
            ymin = std::min(ymin, sy); ymax = std::max(ymax, sy);
        }
        if (!ok || xmax < 0.0f || ymax < 0.0f || xmin > (float)width || ymin > (float)height) continue;
        const int tx0 = std::max(0, (int)std::floor(xmin) / tile), tx1 = std::min((width - 1) / tile, (int)std::ceil(xmax) / tile);
        const int ty0 = std::max(0, (int)std::floor(ymin) / tile), ty1 = std::min((height - 1) / tile, (int)std::ceil(ymax) / tile);
        for (int ty = ty0; ty <= ty1; ty++)
            for (int tx = tx0; tx <= tx1; tx++) work.push_back(make_int4((int)i, tx, ty, 0));
    }
    cudaStream_t st = g.stream;
    RasterTri *d_tris = dalloc<RasterTri>(tris.size());
    RasterTex *d_tex = dalloc<RasterTex>(tex.size());
    float4 *d_col = dalloc<float4>((size_t)std::max<long long>(cells, 1));
    int4 *d_work = dalloc<int4>(work.size());
    unsigned long long *d_z = dalloc<unsigned long long>((size_t)width * height);
    unsigned char *d_rgb = dalloc<unsigned char>((size_t)width * height * 3);
    cudaError_t e = cudaSuccess;
    if (!tris.empty()) e = cudaMemcpyAsync(d_tris, tris.data(), tris.size() * sizeof(RasterTri), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !tex.empty())
        e = cudaMemcpyAsync(d_tex, tex.data(), tex.size() * sizeof(RasterTex), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !work.empty())
        e = cudaMemcpyAsync(d_work, work.data(), work.size() * sizeof(int4), cudaMemcpyHostToDevice, st);
    for (auto &oc : objs) {
        Object *o = oc.first;
        if (e != cudaSuccess || o->ncells == 0) continue;
        const int phase = o->type == OBJ_FIELD ? g.phase_field : g.phase_target;
        launch_colour_map(o->d_P, o->ncells, g.min_db, g.max_db, phase, d_col + oc.second, st);
    }
    ra.tris = d_tris;
    ra.tex = d_tex;
    ra.colours = d_col;
    ra.work = d_work;
    ra.zbuf = d_z;
    ra.rgb = d_rgb;
    if (e == cudaSuccess) {
        launch_raster(ra, (int)work.size(), st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(rgb_host, d_rgb, (size_t)width * height * 3, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dfree(d_tris); dfree(d_tex); dfree(d_col); dfree(d_work); dfree(d_z); dfree(d_rgb);
    if (e != cudaSuccess) fail(-10, "render failed: %s", cudaGetErrorString(e));
    g.launches += 3 + (long long)objs.size();
}

// ---------------------------------------------------------------- ABI glue
template <class F>
int guarded(F &&f)
{
    if (g.status != 0) return g.status;
    try {
        f();
        return 0;
    } catch (const Error &e) {
        g.status = e.code;
        g.err = e.what();
    } catch (const std::exception &e) {
        g.status = -1;
        g.err = e.what();
    } catch (...) {
        g.status = -1;
        g.err = "unknown error";
    }
    if (g.verbose) fprintf(stderr, "sonar: %s\n", g.err.c_str());
    return g.status;
}

bool finite3(const float *p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

}  // namespace

void set_error_message(const std::string &m) { g.err = m; }

}  // namespace sonar

using namespace sonar;

extern "C" {

void set_initial_conditions(float cp, float frequency, float attenuation, float density)
{
    guarded([&] {
        // src/Model.cpp:44-54: omega and k are FP32
        const float omega = (float)(2 * M_PI * (double)frequency);
        const float k = omega / cp;
        g.cp = cp;
        g.freq = frequency;
        g.att = attenuation;
        g.density = density;
        g.kr = (double)k;
        g.ki = (double)attenuation;
    });
}

void load_geometry(float *v1, int num_vertices, int objectType, float resolution)
{
    guarded([&] {
        if (objectType < OBJ_TARGET || objectType > OBJ_FIELD) fail(-6, "invalid objectType %d", objectType);
        if (num_vertices < 0 || (num_vertices > 0 && !v1)) fail(-6, "invalid triangle buffer");
        if (!(resolution > 0.0f) || !std::isfinite(resolution)) fail(-6, "invalid resolution %g", (double)resolution);
        auto o = std::make_unique<Object>();
        o->type = objectType;
        o->delta = resolution;
        o->facets.reserve(num_vertices);
        for (int i = 0; i < num_vertices; i++) {
            const float *t = v1 + 9L * i;
            if (!finite3(t) || !finite3(t + 3) || !finite3(t + 6)) fail(-6, "triangle %d has a non-finite vertex", i);
            o->facets.push_back(make_frame({t[0], t[1], t[2]}, {t[3], t[4], t[5]}, {t[6], t[7], t[8]}, resolution));
        }
        g.obj[objectType].push_back(std::move(o));
    });
}

void load_field_points(float *v1, int num_feild_points)
{
    guarded([&] {
        if (num_feild_points < 0 || (num_feild_points > 0 && !v1)) fail(-6, "invalid field point buffer");
        if (g.rendered) fail(-7, "load_field_points after render_cuda");
        for (int i = 0; i < num_feild_points; i++) {
            if (!finite3(v1 + 3L * i)) fail(-6, "field point %d is not finite", i);
            g.fp.push_back({v1[3L * i], v1[3L * i + 1], v1[3L * i + 2]});
        }
    });
}

void load_source_points(float *v1, int num_source_points)
{
    guarded([&] {
        if (num_source_points < 0 || (num_source_points > 0 && !v1)) fail(-6, "invalid source point buffer");
        if (g.rendered) fail(-7, "load_source_points after render_cuda");
        for (int i = 0; i < num_source_points; i++) {
            if (!finite3(v1 + 3L * i)) fail(-6, "source point %d is not finite", i);
            g.src.push_back({v1[3L * i], v1[3L * i + 1], v1[3L * i + 2]});
        }
    });
}

void render_cuda(void)
{
    guarded([] { render(); });
}

void ProjectSrcPointsToObjects(bool projectFieldObjects)
{
    guarded([&] {
        need_render();
        for (int i = 0; i < (int)g.obj[OBJ_TARGET].size(); i++) run_hop(HOP_SRC, OBJ_TARGET, i);
        if (projectFieldObjects)
            for (int i = 0; i < (int)g.obj[OBJ_FIELD].size(); i++) run_hop(HOP_SRC, OBJ_FIELD, i);
        // piston source objects (objectType 1) radiate their unit surface
        // pressure into the targets and, with projectFieldObjects, the field objects
        for (int p = 0; p < (int)g.obj[OBJ_SOURCE].size(); p++) {
            for (int i = 0; i < (int)g.obj[OBJ_TARGET].size(); i++) run_hop(HOP_PISTON_T, p, i);
            if (projectFieldObjects)
                for (int i = 0; i < (int)g.obj[OBJ_FIELD].size(); i++) run_hop(HOP_PISTON_F, p, i);
        }
    });
}

void ProjectTargetToFieldObjects(void)
{
    guarded([] {
        need_render();
        for (int t = 0; t < (int)g.obj[OBJ_TARGET].size(); t++)
            for (int f = 0; f < (int)g.obj[OBJ_FIELD].size(); f++) run_hop(HOP_NORESP, t, f);
    });
}

void ProjectTargetToFieldPoints(void)
{
    guarded([] {
        need_render();
        for (int t = 0; t < (int)g.obj[OBJ_TARGET].size(); t++) run_hop(HOP_FP, t, 0);
    });
}

void ProjectTargetToTargetObjects(int number_reflections)
{
    guarded([&] {
        need_render();
        // src/ModelCuda.cpp:323-356: prime P_out <- P; per bounce P_in <- P_out,
        // P_out <- 0, project, P += P_out.  Objects never interact, so each
        // object runs its bounces in turn; P_in/P_out swap by pointer.
        // With the cross_objects option (an extension: FACET_RESP, which the
        // reference's host never calls) every bounce also carries the terms
        // between every pair of targets: all targets swap, then each runs its
        // FACET_SELF projection (which writes P_out and adds it to P), then
        // each pair a < b adds its forward terms into b and its reciprocal
        // terms into a (to P_out and P), all from this bounce's P_in.
        const int nt = (int)g.obj[OBJ_TARGET].size();
        if (g.opt_cross_objects && nt > 1) {
            for (int t = 0; t < nt; t++) {
                Object &A = *g.obj[OBJ_TARGET][t];
                const size_t bytes = std::max<size_t>((size_t)A.ncells, 1) * sizeof(double2);
                CK(cudaMemcpyAsync(A.d_Pout, A.d_P, bytes, cudaMemcpyDeviceToDevice, g.stream));
            }
            for (int b = 0; b < number_reflections; b++) {
                for (int t = 0; t < nt; t++) {
                    Object &A = *g.obj[OBJ_TARGET][t];
                    const size_t bytes = std::max<size_t>((size_t)A.ncells, 1) * sizeof(double2);
                    std::swap(A.d_Pin, A.d_Pout);
                    CK(cudaMemsetAsync(A.d_Pout, 0, bytes, g.stream));
                }
                for (int t = 0; t < nt; t++) run_hop(HOP_F2F, t, 0);
                for (int t = 0; t < nt; t++)
                    for (int u = t + 1; u < nt; u++) {
                        run_hop(HOP_RESP, t, u);
                        run_hop(HOP_RESP, u, t);
                    }
            }
            CK(cudaStreamSynchronize(g.stream));
            return;
        }
        for (int t = 0; t < nt; t++) {
            Object &A = *g.obj[OBJ_TARGET][t];
            const size_t bytes = std::max<size_t>((size_t)A.ncells, 1) * sizeof(double2);
            CK(cudaMemcpyAsync(A.d_Pout, A.d_P, bytes, cudaMemcpyDeviceToDevice, g.stream));
            for (int b = 0; b < number_reflections; b++) {
                std::swap(A.d_Pin, A.d_Pout);
                CK(cudaMemsetAsync(A.d_Pout, 0, bytes, g.stream));
                run_hop(HOP_F2F, t, 0);
            }
        }
        CK(cudaStreamSynchronize(g.stream));
    });
}

void GetFieldPointPressures(dcomplex *field_points_pressure, int NumPoints)
{
    guarded([&] {
        need_render();
        const size_t n = std::min<size_t>(NumPoints < 0 ? 0 : (size_t)NumPoints, g.fp.size());
        if (n && !field_points_pressure) fail(-6, "null output buffer");
        if (n) {
            CK(stage_to_host(field_points_pressure, g.d_fp_P, n * sizeof(double2), g.stream));
            g.d2h_bytes += (long long)(n * sizeof(double2));
        }
        if ((size_t)std::max(NumPoints, 0) < g.fp.size())
            fail(-8, "GetFieldPointPressures: buffer holds %d of %zu field points", NumPoints, g.fp.size());
    });
}

void RenderOpenGL(int width, int height, char *filename, float viewSettings[9])
{
    guarded([&] {
        if (!filename) fail(-6, "RenderOpenGL: null file name");
        std::vector<unsigned char> rgb((size_t)std::max(width, 0) * std::max(height, 0) * 3);
        render_image(width, height, viewSettings, rgb.data());
        if (!write_png(filename, width, height, rgb.data())) fail(-7, "RenderOpenGL: cannot write %s", filename);
    });
}

void TearDownCuda(void)
{
    // src/Model.cpp:115-129, src/ModelCuda.cpp:124-181: points, target and
    // field objects are dropped
    try {
        // every stream, as the cudaFree of the buffers used to: a caller may
        // still read a result on a stream of its own
        cudaDeviceSynchronize();
        g.free_device();
    } catch (...) {
    }
    // piston source objects are dropped too: they radiate in this library
    // (the reference stores them without using them, src/Model.cpp:33-35)
    g.obj[OBJ_TARGET].clear();
    g.obj[OBJ_SOURCE].clear();
    g.obj[OBJ_FIELD].clear();
    g.src.clear();
    g.fp.clear();
    g.rendered = false;
    g.status = 0;
    g.err.clear();
    g.log.clear();
}

void SoundVisualisationInit(float maxDbValue, float minDbValue, bool renderPhaseTarget, bool renderPhaseField)
{
    g.max_db = maxDbValue;
    g.min_db = minDbValue;
    g.phase_target = renderPhaseTarget;
    g.phase_field = renderPhaseField;
}

int sonar_status(void) { return g.status; }

const char *sonar_last_error(void) { return g.err.c_str(); }

void sonar_clear_error(void)
{
    g.status = 0;
    g.err.clear();
}

int sonar_get_object_count(int objectType)
{
    return (objectType >= 0 && objectType <= 2) ? (int)g.obj[objectType].size() : -1;
}

long long sonar_get_object_cells(int objectType, int objIdx)
{
    if (objectType < 0 || objectType > 2 || objIdx < 0 || objIdx >= (int)g.obj[objectType].size()) return -1;
    const Object &o = *g.obj[objectType][objIdx];
    if (!g.rendered) {
        long long n = 0;
        for (auto &F : o.facets) n += (long long)F.nx * F.ny;
        return n;
    }
    return o.ncells;
}

int sonar_get_object_pressures(int objectType, int objIdx, dcomplex *out, long long n)
{
    int written = 0;
    int st = guarded([&] {
        need_render();
        Object &o = get(objectType, objIdx);
        if (o.type == OBJ_SOURCE || !o.d_P) fail(-4, "object has no pressures");
        if (n < o.ncells) fail(-8, "buffer holds %lld of %lld cells", n, o.ncells);
        if (o.ncells) {
            CK(stage_to_host(out, o.d_P, (size_t)o.ncells * sizeof(double2), g.stream));
            g.d2h_bytes += o.ncells * (long long)sizeof(double2);
        }
        written = (int)o.ncells;
    });
    return st != 0 ? st : written;
}

int sonar_get_fragment_layout(int objectType, int objIdx, int *nx_ny_neg, int nfacets_cap, float *areas,
                              long long ncells_cap)
{
    int nf = 0;
    int st = guarded([&] {
        Object &o = get(objectType, objIdx);
        nf = (int)o.facets.size();
        if (nx_ny_neg) {
            if (nfacets_cap < nf) fail(-8, "layout buffer holds %d of %d facets", nfacets_cap, nf);
            for (int f = 0; f < nf; f++) {
                nx_ny_neg[3 * f] = o.facets[f].nx;
                nx_ny_neg[3 * f + 1] = o.facets[f].ny;
                nx_ny_neg[3 * f + 2] = o.facets[f].neg;
            }
        }
        if (areas) {
            long long total = 0;
            for (auto &F : o.facets) total += (long long)F.nx * F.ny;
            if (ncells_cap < total) fail(-8, "area buffer holds %lld of %lld cells", ncells_cap, total);
            long long off = 0;
            for (auto &F : o.facets) {
                fragment_areas(F, areas + off);
                off += (long long)F.nx * F.ny;
            }
        }
    });
    return st != 0 ? st : nf;
}

int sonar_get_stats(char *json, int cap)
{
    std::string s = "{\"hops\": [";
    char buf[1024];
    for (size_t i = 0; i < g.log.size(); i++) {
        const HopRecord &r = g.log[i];
        snprintf(buf, sizeof(buf),
                 "%s{\"hop\": %d, \"pairs\": %lld, \"mask_ms\": %.6f, \"sum_ms\": %.6f, \"total_ms\": %.6f, "
                 "\"nsplit\": %d, \"launches\": %d, \"cmp_select\": %d, \"cmp_cand\": %d, \"cmp_blocks\": %d, "
                 "\"cmp_accepted\": %d, \"cmp_pairs\": %.0f, \"cmp_mean_rank\": %.3f, \"cmp_max_err\": %.3e, "
                 "\"cmp_ip_blocks\": %d, \"cmp_ip_kept\": %d, \"cmp_ip_nodes\": %.3f, "
                 "\"cmp_build_ms\": %.6f, \"cmp_select_ms\": %.6f, \"cmp_aca_ms\": %.6f, \"cmp_ip_ms\": %.6f, "
                 "\"cmp_approx_ms\": %.6f, \"lr_ms\": %.6f}",
                 i ? ", " : "", r.hop, r.pairs, r.mask_ms, r.sum_ms, r.total_ms, r.nsplit, r.launches, r.cmp_select,
                 r.cmp_cand, r.cmp_blocks, r.cmp_accepted, r.cmp_pairs, r.cmp_mean_rank, r.cmp_max_err,
                 r.cmp_ip_blocks, r.cmp_ip_kept, r.cmp_ip_nodes, r.cmp_build_ms, r.cmp_select_ms, r.cmp_aca_ms, r.cmp_ip_ms,
                 r.cmp_approx_ms, r.lr_ms);
        s += buf;
    }
    snprintf(buf, sizeof(buf),
             "], \"ntri\": %d, \"nnodes\": %d, \"masks\": %zu, \"launches\": %lld, \"h2d_bytes\": %lld, "
             "\"d2h_bytes\": %lld, \"pool_reserved_bytes\": %llu, \"render_host_ms\": {\"setup\": %.4f, "
             "\"fragments\": %.4f, \"uploads\": %.4f, \"occluders\": %.4f, \"points\": %.4f}, \"mask_classes\": [",
             g.ntri, g.nnodes, g.masks.size(), g.launches, g.h2d_bytes, g.d2h_bytes, pool_reserved_bytes(),
             g.render_ms[0], g.render_ms[1], g.render_ms[2], g.render_ms[3], g.render_ms[4]);
    s += buf;
    for (size_t i = 0; i < g.masks.size(); i++) {
        const MaskEntry &m = g.masks[i];
        snprintf(buf, sizeof(buf), "%s{\"hop\": %d, \"none\": %lld, \"bits\": %lld, \"clear\": %lld, \"all\": %lld}",
                 i ? ", " : "", m.hop, m.classes[0], m.classes[1], m.classes[2], m.classes[3]);
        s += buf;
    }
    s += "]}";
    if (json && cap > 0) {
        const size_t n = std::min<size_t>(s.size(), (size_t)cap - 1);
        memcpy(json, s.data(), n);
        json[n] = 0;
    }
    return (int)s.size();
}

int sonar_set_option(const char *key, double value)
{
    if (!key) return -1;
    if (!strcmp(key, "memory_cache_mb")) {
        if (!(value >= 0.0)) return -6;
        pool_set_cache_limit((unsigned long long)(value * 1048576.0));
        return 0;
    }
    if (!strcmp(key, "release_memory")) return pool_trim() == cudaSuccess ? 0 : -10;
    if (!strcmp(key, "split")) { g.opt_split = (int)value; return 0; }
    if (!strcmp(key, "f2f_symmetric")) { g.opt_f2f_sym = value != 0.0; return 0; }
    if (!strcmp(key, "class_stats")) { g.opt_class_stats = value != 0.0; return 0; }
    if (!strcmp(key, "compress")) { g.opt_compress = value != 0.0; g.cmp.release(); return 0; }
    if (!strcmp(key, "compress_tol")) { g.opt_cmp_tol = (float)value; g.cmp.release(); return 0; }
    if (!strcmp(key, "compress_judge")) { g.opt_cmp_judge = (float)value; g.cmp.release(); return 0; }
    if (!strcmp(key, "compress_eta")) { g.opt_cmp_eta = (float)value; g.cmp.release(); return 0; }
    if (!strcmp(key, "compress_select")) {
        g.opt_cmp_select = std::max(0, std::min(2, (int)value));
        g.cmp.release();
        return 0;
    }
    if (!strcmp(key, "overlap_streams")) {
        g.opt_overlap = value != 0.0 ? 1 : 0;
        return 0;
    }
    if (!strcmp(key, "tile_align")) {
        g.opt_tile_align = value != 0.0 ? 1 : 0;
        return 0;
    }
    if (!strcmp(key, "ip_transpose")) {
        g.opt_ip_transpose = value != 0.0 ? 1 : 0;
        g.cmp.release();
        return 0;
    }
    if (!strcmp(key, "compress_build_overlap")) {
        g.opt_build_overlap = value != 0.0 ? 1 : 0;
        return 0;
    }
    if (!strcmp(key, "convex_masks")) {
        g.opt_convex_masks = value != 0.0 ? 1 : 0;
        for (auto &m : g.masks) m.stale = true;
        return 0;
    }
    if (!strcmp(key, "cross_objects")) {
        g.opt_cross_objects = value != 0.0 ? 1 : 0;
        return 0;
    }
    if (!strcmp(key, "mask_gate_proj")) {
        g.opt_gate_proj = value != 0.0 ? 1 : 0;
        for (auto &m : g.masks) m.stale = true;
        return 0;
    }
    if (!strcmp(key, "mask_classify")) {
        g.opt_mask_classify = value != 0.0 ? 1 : 0;
        for (auto &m : g.masks) m.stale = true;
        return 0;
    }
    if (!strcmp(key, "lr_block_ctas")) {
        if (value != 4 && value != 6 && value != 8) return -1;
        g.opt_lr_ctas = (int)value;
        return 0;
    }
    if (!strcmp(key, "relative_geometry")) { g.opt_rel_geom = value != 0.0; return 0; }
    if (!strcmp(key, "aca_fused_apply")) { g.opt_fused_apply = value != 0.0; g.cmp.release(); return 0; }
    if (!strcmp(key, "compress_interp")) { g.opt_cmp_interp = value != 0.0; g.cmp.release(); return 0; }
    if (!strcmp(key, "aca_variant")) {
        if (value < 0 || value > 10) return -1;
        g.opt_aca_variant = (int)value;
        return 0;
    }
    if (!strcmp(key, "compress_rcut")) { g.opt_cmp_rcut = (float)value; g.cmp.release(); return 0; }
    if (!strcmp(key, "compress_rmax")) {
        g.opt_cmp_rmax = std::max(2, std::min(kLrRankLimit, (int)value));
        g.cmp.release();
        return 0;
    }
    if (!strcmp(key, "verbose")) { g.verbose = (int)value; return 0; }
    if (!strcmp(key, "reset_stats")) {
        g.log.clear();
        g.launches = g.h2d_bytes = g.d2h_bytes = 0;
        return 0;
    }
    if (!strcmp(key, "reset_pressures")) {
        // zero every surface and field-point pressure (benchmark steps start clean)
        return guarded([] {
            need_render();
            for (int t : {OBJ_TARGET, OBJ_FIELD})
                for (auto &o : g.obj[t]) {
                    const size_t b = std::max<size_t>((size_t)o->ncells, 1) * sizeof(double2);
                    CK(cudaMemsetAsync(o->d_P, 0, b, g.stream));
                    if (o->d_Pin) CK(cudaMemsetAsync(o->d_Pin, 0, b, g.stream));
                    if (o->d_Pout) CK(cudaMemsetAsync(o->d_Pout, 0, b, g.stream));
                }
            if (!g.fp.empty()) CK(cudaMemsetAsync(g.d_fp_P, 0, g.fp.size() * sizeof(double2), g.stream));
            CK(cudaStreamSynchronize(g.stream));
        });
    }
    if (!strcmp(key, "drop_masks")) {
        // rebuild every mask (same buffers) at its next use
        for (auto &m : g.masks) m.stale = true;
        return 0;
    }
    if (!strcmp(key, "free_masks")) {
        for (auto &m : g.masks) m.free_device();
        g.masks.clear();
        return 0;
    }
    return -1;
}

long long sonar_get_mask(int hop, int srcIdx, int dstIdx, unsigned char *out, long long cap)
{
    long long nbytes = 0;
    int st = guarded([&] {
        need_render();
        if (hop < HOP_SRC || hop > HOP_PISTON_F) fail(-6, "invalid hop %d", hop);
        HopSets hs = hop_sets(hop, srcIdx, dstIdx);
        nbytes = (long long)hs.nsrc * hs.ndst;
        if (!out) return;
        if (cap < nbytes) fail(-8, "mask buffer holds %lld of %lld bytes", cap, nbytes);
        if (nbytes == 0) return;
        // a full mask (bits in every block), built for the export and freed
        MaskEntry M = build_mask(hop, srcIdx, dstIdx, 1);
        uint8_t *d = nullptr;
        cudaError_t e = pool_alloc((void **)&d, (size_t)nbytes, g.stream);
        if (e == cudaSuccess) {
            launch_mask_export(M.view, M.nsrc, M.ndst, d, g.stream);
            e = cudaGetLastError();
        }
        std::vector<uint8_t> tmp((size_t)nbytes);
        if (e == cudaSuccess) e = stage_to_host(tmp.data(), d, (size_t)nbytes, g.stream);
        dfree(d);
        M.free_device();
        if (e != cudaSuccess) fail(-10, "mask export failed: %s", cudaGetErrorString(e));
        // active fragments are stored in patch order; report them in cell order
        auto canon = [](const Object &o) {
            std::vector<int> idx(o.act_cell.size()), rank(o.act_cell.size());
            for (size_t q = 0; q < idx.size(); q++) idx[q] = (int)q;
            std::sort(idx.begin(), idx.end(), [&](int x, int y) { return o.act_cell[x] < o.act_cell[y]; });
            for (size_t k = 0; k < idx.size(); k++) rank[idx[k]] = (int)k;
            return rank;
        };
        std::vector<int> rs, rd;  // internal index -> canonical index (empty: identity)
        if (hop == HOP_FP || hop == HOP_F2F || hop == HOP_NORESP || hop == HOP_RESP) rs = canon(get(OBJ_TARGET, srcIdx));
        if (hop == HOP_F2F) rd = rs;
        if (hop == HOP_RESP) rd = canon(get(OBJ_TARGET, dstIdx));
        if (hop == HOP_FP) rd = g.fp_order;  // stored field point k is load index fp_order[k]
        if (hop == HOP_NORESP) rd = canon(get(OBJ_FIELD, dstIdx));
        if (hop == HOP_PISTON_T || hop == HOP_PISTON_F) {
            rs = canon(get(OBJ_SOURCE, srcIdx));
            rd = canon(get(hop == HOP_PISTON_T ? OBJ_TARGET : OBJ_FIELD, dstIdx));
        }
        for (long long jd = 0; jd < M.ndst; jd++) {
            const long long cd = rd.empty() ? jd : rd[jd];
            const uint8_t *row = tmp.data() + jd * M.nsrc;
            uint8_t *orow = out + cd * M.nsrc;
            if (rs.empty())
                memcpy(orow, row, (size_t)M.nsrc);
            else
                for (long long js = 0; js < M.nsrc; js++) orow[rs[js]] = row[js];
        }
    });
    return st != 0 ? st : nbytes;
}

int sonar_audit_compression(int nsample, unsigned seed, float *full_err, float *judged_err, int cap)
{
    int nout = 0;
    int st = guarded([&] {
        need_render();
        Compression &C = g.cmp;
        if (!C.valid || !C.d_U || C.nblocks <= 0) fail(-6, "no compressed blocks to audit: run a compressed bounce first");
        if (g.ki != 0.0) fail(-6, "the audit evaluates entries without attenuation");
        if (nsample < 0 || cap < 0 || (cap > 0 && (!full_err || !judged_err))) fail(-6, "invalid audit arguments");
        finish_compression();
        MaskEntry &M = get_mask(HOP_F2F, C.obj, 0);
        Object &A = get(OBJ_TARGET, C.obj);
        const int n = C.nblocks;
        std::vector<int> rk(n);
        std::vector<float> er(n);
        std::vector<uint8_t> lv(n, 0);
        CK(cudaMemcpy(rk.data(), C.d_rank, n * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(er.data(), C.d_err, n * sizeof(float), cudaMemcpyDeviceToHost));
        if (C.interp) CK(cudaMemcpy(lv.data(), C.d_lev, n, cudaMemcpyDeviceToHost));
        std::vector<int> acc;
        for (int b = 0; b < n; b++)
            if (rk[b] > 0) acc.push_back(b);
        std::mt19937 rng(seed);
        std::shuffle(acc.begin(), acc.end(), rng);
        const int ns = std::min({nsample, cap, (int)acc.size()});
        acc.resize(ns);
        std::sort(acc.begin(), acc.end());
        if (ns == 0) return;
        ensure_scratch(M.nsrc, M.ndst, 1);
        launch_pack_frags(A.d_act_pos, A.d_act_facet, A.d_act_cell, A.d_facet_n, A.d_Pin, 0.9f, M.nsrc, g.d_packA,
                          g.d_packB, g.stream);
        SumArgs s{};
        s.hop = HOP_F2F;
        s.nsrc = s.ndst = M.nsrc;
        s.srcA = g.d_packA;
        s.srcB = g.d_packB;
        s.mask = M.view;
        s.kr = (float)g.kr;
        s.ka = (float)g.ki;
        const double k2 = g.kr / (2.0 * M_PI);
        s.k2hi = (float)k2;
        s.k2lo = (float)(k2 - (double)s.k2hi);
        s.kr4pi = (float)(g.kr / (4.0 * M_PI));
        s.rmin = A.delta;
        int *d_sample = dalloc<int>(ns);
        float *d_err = dalloc<float>(ns);
        CK(cudaMemcpyAsync(d_sample, acc.data(), ns * sizeof(int), cudaMemcpyHostToDevice, g.stream));
        // cross-approximated and interpolated blocks each by their own audit
        // kernel (the other kind's CTAs return at once)
        launch_lr_audit(s, C.d_blocks, C.d_cls, C.d_off, C.d_rank, d_sample, ns, C.d_U, C.d_V, d_err, g.stream,
                        C.interp ? C.d_lev : nullptr);
        if (C.interp)
            launch_ip_audit(s, C.ip.tile, C.ip.fxy, C.ip.lev, C.ip.delta, C.d_blocks, C.d_off, d_sample, ns, C.d_U,
                            d_err, g.stream);
        CK(cudaGetLastError());
        std::vector<float> fe(ns);
        CK(cudaMemcpyAsync(fe.data(), d_err, ns * sizeof(float), cudaMemcpyDeviceToHost, g.stream));
        CK(cudaStreamSynchronize(g.stream));
        dfree(d_sample);
        dfree(d_err);
        for (int q = 0; q < ns; q++) {
            full_err[q] = fe[q];
            judged_err[q] = er[acc[q]];
        }
        nout = ns;
    });
    return st != 0 ? st : nout;
}

long long sonar_get_mask_rows(int hop, int srcIdx, int dstIdx, const int *rows, int nrows, unsigned char *out,
                              long long cap)
{
    long long nbytes = 0;
    int st = guarded([&] {
        need_render();
        if (hop < HOP_SRC || hop > HOP_PISTON_F) fail(-6, "invalid hop %d", hop);
        if (nrows < 0 || (nrows > 0 && !rows)) fail(-6, "invalid row list");
        HopSets hs = hop_sets(hop, srcIdx, dstIdx);
        nbytes = (long long)hs.nsrc * nrows;
        if (!out) return;
        if (cap < nbytes) fail(-8, "mask buffer holds %lld of %lld bytes", cap, nbytes);
        if (nbytes == 0) return;
        auto canon = [](const Object &o) {
            std::vector<int> idx(o.act_cell.size()), rank(o.act_cell.size());
            for (size_t q = 0; q < idx.size(); q++) idx[q] = (int)q;
            std::sort(idx.begin(), idx.end(), [&](int x, int y) { return o.act_cell[x] < o.act_cell[y]; });
            for (size_t k = 0; k < idx.size(); k++) rank[idx[k]] = (int)k;
            return rank;
        };
        std::vector<int> rs, rd;  // internal index -> canonical index (empty: identity)
        if (hop == HOP_FP || hop == HOP_F2F || hop == HOP_NORESP || hop == HOP_RESP) rs = canon(get(OBJ_TARGET, srcIdx));
        if (hop == HOP_F2F) rd = rs;
        if (hop == HOP_RESP) rd = canon(get(OBJ_TARGET, dstIdx));
        if (hop == HOP_FP) rd = g.fp_order;
        if (hop == HOP_NORESP) rd = canon(get(OBJ_FIELD, dstIdx));
        if (hop == HOP_PISTON_T || hop == HOP_PISTON_F) {
            rs = canon(get(OBJ_SOURCE, srcIdx));
            rd = canon(get(hop == HOP_PISTON_T ? OBJ_TARGET : OBJ_FIELD, dstIdx));
        }
        // canonical destination -> internal row
        std::vector<int> inv(hs.ndst);
        for (int jd = 0; jd < hs.ndst; jd++) inv[rd.empty() ? jd : rd[jd]] = jd;
        std::vector<int> irow(nrows);
        for (int q = 0; q < nrows; q++) {
            if (rows[q] < 0 || rows[q] >= hs.ndst) fail(-6, "row %d outside [0, %d)", rows[q], hs.ndst);
            irow[q] = inv[rows[q]];
        }
        MaskEntry M = build_mask(hop, srcIdx, dstIdx, 1);
        uint8_t *d = nullptr;
        int *drows = nullptr;
        cudaError_t e = pool_alloc((void **)&d, (size_t)nbytes, g.stream);
        if (e == cudaSuccess) e = pool_alloc((void **)&drows, sizeof(int) * (size_t)nrows, g.stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(drows, irow.data(), sizeof(int) * (size_t)nrows, cudaMemcpyHostToDevice, g.stream);
        if (e == cudaSuccess) {
            launch_mask_export_rows(M.view, M.nsrc, drows, nrows, d, g.stream);
            e = cudaGetLastError();
        }
        std::vector<uint8_t> tmp((size_t)nbytes);
        if (e == cudaSuccess) e = stage_to_host(tmp.data(), d, (size_t)nbytes, g.stream);
        dfree(d);
        dfree(drows);
        M.free_device();
        if (e != cudaSuccess) fail(-10, "mask export failed: %s", cudaGetErrorString(e));
        for (int q = 0; q < nrows; q++) {
            const uint8_t *row = tmp.data() + (size_t)q * M.nsrc;
            uint8_t *orow = out + (size_t)q * M.nsrc;
            if (rs.empty())
                memcpy(orow, row, (size_t)M.nsrc);
            else
                for (long long js = 0; js < M.nsrc; js++) orow[rs[js]] = row[js];
        }
    });
    return st != 0 ? st : nbytes;
}

int sonar_render_image(int width, int height, const float *viewSettings, unsigned char *rgb)
{
    return guarded([&] { render_image(width, height, viewSettings, rgb); });
}

int sonar_get_surface_colours(int objectType, int objIdx, float *rgba, long long ncells)
{
    int written = 0;
    int st = guarded([&] {
        need_render();
        Object &o = get(objectType, objIdx);
        if (o.type == OBJ_SOURCE || !o.d_P) fail(-4, "object has no pressures");
        if (ncells < o.ncells) fail(-8, "colour buffer holds %lld of %lld cells", ncells, o.ncells);
        if (o.ncells == 0) return;
        float4 *d = dalloc<float4>((size_t)o.ncells);
        const int phase = o.type == OBJ_FIELD ? g.phase_field : g.phase_target;
        launch_colour_map(o.d_P, o.ncells, g.min_db, g.max_db, phase, d, g.stream);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(rgba, d, (size_t)o.ncells * sizeof(float4), cudaMemcpyDeviceToHost, g.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(g.stream);
        dfree(d);
        if (e != cudaSuccess) fail(-10, "colour map failed: %s", cudaGetErrorString(e));
        written = (int)o.ncells;
    });
    return st != 0 ? st : written;
}

void *sonar_get_stream(void) { return (void *)g.stream; }

double sonar_measure_peak(int which) { return measure_peak(which); }

/* Host-only: frame and area grid of one triangle (no GPU needed). */
long long sonar_fragment_triangle(const float *tri9, float delta, int *nx_ny_neg, float *frame17, float *areas,
                                  long long cap)
{
    if (!tri9 || !(delta > 0.0f)) return -6;
    FacetFrame F = make_frame({tri9[0], tri9[1], tri9[2]}, {tri9[3], tri9[4], tri9[5]}, {tri9[6], tri9[7], tri9[8]}, delta);
    if (nx_ny_neg) {
        nx_ny_neg[0] = F.nx;
        nx_ny_neg[1] = F.ny;
        nx_ny_neg[2] = F.neg;
    }
    if (frame17) {
        const float v[17] = {F.normal.x, F.normal.y, F.normal.z, F.base.x, F.base.y, F.base.z, F.xAxis.x, F.xAxis.y,
                             F.xAxis.z, F.yAxis.x, F.yAxis.y, F.yAxis.z, F.baseLen, F.height, F.baseNeg, F.basePos,
                             F.area};
        memcpy(frame17, v, sizeof(v));
    }
    const long long n = (long long)F.nx * F.ny;
    if (areas && cap >= n) fragment_areas(F, areas);
    return n;
}

long long sonar_tile_order(const float *tri9, float delta, long long start, int *xy, long long cap)
{
    if (!tri9 || !(delta > 0.0f) || start < 0) return -6;
    const FacetFrame F =
        make_frame({tri9[0], tri9[1], tri9[2]}, {tri9[3], tri9[4], tri9[5]}, {tri9[6], tri9[7], tri9[8]}, delta);
    std::vector<float> area((size_t)std::max(F.nx * F.ny, 1));
    fragment_areas(F, area.data());
    // active cells in patch order (patch row, patch column, row-major inside)
    std::vector<int> cx, cy;
    std::vector<float4> pos;
    std::vector<PatchRun> runs;
    for (int py = 0; py < F.ny; py += kPatch)
        for (int px = 0; px < F.nx; px += kPatch) {
            const long long b = (long long)cx.size();
            for (int y = py; y < std::min(F.ny, py + kPatch); y++)
                for (int x = px; x < std::min(F.nx, px + kPatch); x++) {
                    if (!(area[(size_t)y * F.nx + x] > 1e-6f)) continue;
                    const Vec3 p = fragment_centroid(F, x, y, false);
                    cx.push_back(x);
                    cy.push_back(y);
                    pos.push_back(make_float4(p.x, p.y, p.z, 0.0f));
                }
            if ((long long)cx.size() > b) runs.push_back(PatchRun{b, (long long)cx.size(), py / kPatch, px / kPatch});
        }
    const long long n = (long long)cx.size();
    if (n >= 2 * kTile && xy && cap >= n) {
        const std::vector<int> order = patch_aligned_order(F, runs, pos.data(), start);
        for (long long i = 0; i < n; i++) {
            const int k = order.empty() ? (int)i : order[(size_t)i];
            xy[2 * i] = cx[(size_t)k];
            xy[2 * i + 1] = cy[(size_t)k];
        }
    } else if (xy && cap >= n) {
        for (long long i = 0; i < n; i++) {
            xy[2 * i] = cx[(size_t)i];
            xy[2 * i + 1] = cy[(size_t)i];
        }
    }
    return n;
}

// ---- admissibility network
int sonar_mlp_param_count(void) { return (int)mlp_param_count(); }

int sonar_mlp_set_width(int width)
{
    return guarded([&] {
        if (mlp_set_width(width) != cudaSuccess) fail(-6, "network width %d (64 or 128)", width);
        g.cmp.release();
    });
}

int sonar_mlp_width(void) { return mlp_width(); }


int sonar_mlp_init(unsigned seed)
{
    return guarded([&] {
        cudaError_t e = mlp_init(seed);
        if (e != cudaSuccess) fail(-10, "network init failed: %s", cudaGetErrorString(e));
    });
}

int sonar_mlp_set_params(const float *params, long long n)
{
    return guarded([&] {
        if (!params || n != (long long)mlp_param_count())
            fail(-6, "the network has %zu parameters, %lld given", mlp_param_count(), n);
        cudaError_t e = mlp_set_params(params, (size_t)n);
        if (e != cudaSuccess) fail(-10, "network parameter upload failed: %s", cudaGetErrorString(e));
        g.cmp.release();
    });
}

int sonar_mlp_get_params(float *params, long long n)
{
    return guarded([&] {
        if (!params || n != (long long)mlp_param_count())
            fail(-6, "the network has %zu parameters, %lld requested", mlp_param_count(), n);
        if (!mlp_ready()) fail(-2, "the network has no parameters");
        cudaError_t e = mlp_get_params(params, (size_t)n);
        if (e != cudaSuccess) fail(-10, "network parameter read failed: %s", cudaGetErrorString(e));
    });
}

int sonar_mlp_grad(const float *X, const float *y, int n, float *grad, float *loss)
{
    return guarded([&] {
        if (!X || !y || !grad || !loss || n <= 0) fail(-6, "sonar_mlp_grad: bad arguments");
        if (!mlp_ready()) fail(-2, "the network has no parameters");
        cudaError_t e = mlp_grad(X, y, n, grad, loss);
        if (e != cudaSuccess) fail(-10, "network gradient failed: %s", cudaGetErrorString(e));
    });
}

int sonar_mlp_train(const float *X, const float *y, int n, int epochs, int batch, float lr, unsigned seed,
                    float *loss)
{
    return guarded([&] {
        if (!X || !y || n <= 0 || epochs < 0 || batch <= 0 || !(lr > 0.0f)) fail(-6, "sonar_mlp_train: bad arguments");
        if (!mlp_ready()) fail(-2, "the network has no parameters");
        cudaError_t e = mlp_train(X, y, n, epochs, batch, lr, seed, loss);
        if (e != cudaSuccess) fail(-10, "network training failed: %s", cudaGetErrorString(e));
        g.cmp.release();
    });
}

int sonar_mlp_predict(const float *X, int n, float *out)
{
    return guarded([&] {
        if (!X || !out || n < 0) fail(-6, "sonar_mlp_predict: bad arguments");
        if (!mlp_ready()) fail(-2, "the network has no parameters");
        if (n == 0) return;
        float *dX = dalloc<float>((size_t)n * 8), *dY = dalloc<float>(n);
        cudaStream_t s = alloc_stream();  // the stream the pool ordered the two blocks on
        cudaError_t e = cudaMemcpyAsync(dX, X, (size_t)n * 8 * sizeof(float), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = mlp_infer_dev(dX, n, dY, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out, dY, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        dfree(dX);
        dfree(dY);
        if (e != cudaSuccess) fail(-10, "network inference failed: %s", cudaGetErrorString(e));
        check_mlp_status();
    });
}

long long sonar_get_block_samples(float *X, float *y, long long cap)
{
    const Compression &C = g.cmp;
    const long long n = C.valid ? (long long)C.label.size() : 0;
    if (X && y && cap >= n && n > 0) {
        memcpy(X, C.desc.data(), (size_t)n * 8 * sizeof(float));
        memcpy(y, C.label.data(), (size_t)n * sizeof(float));
    }
    return n;
}

}  // extern "C"
