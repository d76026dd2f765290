// batch_host.cpp -- host side of the multi-source, multi-frequency batch
// (sonar_batch_plan, sonar_batch_run, sonar_batch_stats, sonar_batch_free,
// sonar_run_batch).
//
// A plan holds one batch: scenes (triangle lists, all of them target
// objects), source and receiver points (at most 64 each), frequencies.  Every
// (scene, frequency) item is fragmented on the host with the reference's
// fragment size rule (delta = cp / f / per_wavelength, src/Facet.cpp:111-339
// through geometry.cpp) and uploaded once.  A run is one CUDA graph: the
// interaction bits of both hops of every fragment (k_batch_vis), the
// persistent tensor-core launch over every item (batch.cu) and the per-item
// reduction.  The graph is captured once, after the autotuner
// has timed the candidate tile shapes (fragments per operand stage,
// persistent CTAs per SM) on the plan's own items and kept the fastest.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sonar_render.h"
#include "devpool.h"
#include "host.h"

namespace sonar {

// model.cpp: the message sonar_last_error() reports
void set_error_message(const std::string &m);

namespace {

constexpr int kPatchB = 16;        // active fragments in 16 x 16-cell patches (as the single-scene path)
constexpr int kSegFragments = 2048;  // FP32 accumulation span of one segment, in fragments

struct BatchError : std::runtime_error {
    int code;
    BatchError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void bfail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw BatchError(code, buf);
}

#define BCK(call)                                                                                   \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) bfail(-10, "%s failed: %s", #call, cudaGetErrorString(e_));         \
    } while (0)

// A plan's buffers come from the stream-ordered pool, ordered on the plan's
// stream.
template <class T>
T *balloc(cudaStream_t s, size_t n)
{
    void *p = nullptr;
    BCK(pool_alloc(&p, std::max<size_t>(n, 1) * sizeof(T), s));
    return (T *)p;
}

template <class T>
void bfree(cudaStream_t s, T *&p)
{
    pool_free(p, s);
    p = nullptr;
}

struct Tuning {
    int kc = 32, grid = 0;
    float ms = 0.0f;
};

struct WorkList {
    std::vector<int4> segs;
    std::vector<int> cta_seg, item_seg_off;
};

// Item fragments on the host
struct ItemFrags {
    std::vector<float4> pos, spos, nrm;
    std::vector<int> facet;
    long long ncells = 0;
};

struct Plan {
    int nscenes = 0, nfreq = 0, nsrc = 0, nrx = 0, nitems = 0;
    float cp = 0.0f, att = 0.0f, per_wl = 0.0f;
    long long nfrag = 0, ncells = 0;
    double pairs = 0.0;
    std::vector<BatchItem> items;
    std::vector<long long> item_cells;
    std::vector<int> convex;      // per scene
    std::vector<float> h_src, h_rx;  // the points of the next run (xyz)
    bool relative = false;           // centroid-relative phase (BatchArgs::rel_*)
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // device
    float4 *d_pos = nullptr, *d_spos = nullptr, *d_nrm = nullptr, *d_facet_n = nullptr;
    int *d_facet = nullptr;
    float4 *d_src = nullptr, *d_rx = nullptr;
    float4 *d_rel_rx = nullptr, *d_rel_src = nullptr;
    double2 *d_erx = nullptr, *d_esrc = nullptr;
    float2 *d_erx_conj = nullptr;
    float4 *d_nodes = nullptr, *d_tris = nullptr;
    BvhView *d_bvh = nullptr;
    uint4 *d_vis = nullptr;
    unsigned *d_hard = nullptr, *d_hard_count = nullptr;
    unsigned hard_cap = 0;
    int nsm = 0;
    BatchItem *d_items = nullptr;
    int4 *d_segs = nullptr;
    int *d_cta_seg = nullptr, *d_item_seg_off = nullptr, *d_item_segs = nullptr, *d_status = nullptr;
    float *d_partial = nullptr;
    double2 *d_out = nullptr;
    size_t segs_cap = 0, partial_cap = 0, cta_cap = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    Tuning tune;
    std::vector<Tuning> tried;
    float vis_ms = 0.0f, gemm_ms = 0.0f, reduce_ms = 0.0f;
    int nseg = 0, runs = 0;
    bool tune_cached = false;

    ~Plan()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        bfree(stream, d_pos); bfree(stream, d_spos); bfree(stream, d_nrm); bfree(stream, d_facet_n);
        bfree(stream, d_facet); bfree(stream, d_src); bfree(stream, d_rx); bfree(stream, d_nodes);
        bfree(stream, d_tris); bfree(stream, d_bvh); bfree(stream, d_vis); bfree(stream, d_hard);
        bfree(stream, d_hard_count); bfree(stream, d_items); bfree(stream, d_segs); bfree(stream, d_cta_seg);
        bfree(stream, d_item_seg_off); bfree(stream, d_item_segs); bfree(stream, d_status);
        bfree(stream, d_partial); bfree(stream, d_out);
        bfree(stream, d_rel_rx); bfree(stream, d_rel_src); bfree(stream, d_erx); bfree(stream, d_esrc);
        bfree(stream, d_erx_conj);
        for (cudaEvent_t &e : ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

std::mutex g_lock;
std::map<long long, std::unique_ptr<Plan>> g_plans;
long long g_next = 1;

// One item's active fragments, in patch order (src/Facet.cpp fragment grid;
// area gate 1e-6 as src/OptiX.cu:138), with both centroids: without the x
// shift (readout, src/OptiX.cu:129) and with it (source hop, src/OptiX.cu:51).
void fragment_item(const float *tris, int ntri, int facet0, float delta, ItemFrags &out)
{
    std::vector<float> area;
    for (int t = 0; t < ntri; t++) {
        const float *v = tris + 9 * (size_t)t;
        const FacetFrame F = make_frame({v[0], v[1], v[2]}, {v[3], v[4], v[5]}, {v[6], v[7], v[8]}, delta);
        const long long nc = (long long)F.nx * F.ny;
        out.ncells += nc;
        if (nc <= 0) continue;
        area.assign((size_t)nc, 0.0f);
        fragment_areas(F, area.data());
        const float4 n = make_float4(F.normal.x, F.normal.y, F.normal.z, 0.0f);
        for (int py = 0; py < F.ny; py += kPatchB)
            for (int px = 0; px < F.nx; px += kPatchB)
                for (int y = py; y < std::min(F.ny, py + kPatchB); y++)
                    for (int x = px; x < std::min(F.nx, px + kPatchB); x++) {
                        const float a = area[(size_t)y * F.nx + x];
                        if (!(a > 1e-6f)) continue;
                        const Vec3 pa = fragment_centroid(F, x, y, false);
                        const Vec3 ps = fragment_centroid(F, x, y, true);
                        out.pos.push_back(make_float4(pa.x, pa.y, pa.z, a));
                        out.spos.push_back(make_float4(ps.x, ps.y, ps.z, a));
                        out.nrm.push_back(n);
                        out.facet.push_back(facet0 + t);
                    }
    }
}

WorkList make_worklist(const Plan &p, int kc, int grid)
{
    WorkList w;
    std::vector<long long> first(p.nitems + 1, 0);  // global chunk index of each item's first chunk
    for (int i = 0; i < p.nitems; i++) first[i + 1] = first[i] + (p.items[i].nfrag + kc - 1) / kc;
    const long long total = first[p.nitems];
    const int segmax = std::max(1, kSegFragments / kc);
    w.cta_seg.assign(grid + 1, 0);
    int item = 0;
    for (int b = 0; b < grid; b++) {
        const long long c0 = total * b / grid, c1 = total * (b + 1) / grid;
        w.cta_seg[b] = (int)w.segs.size();
        long long c = c0;
        while (c < c1) {
            while (first[item + 1] <= c) item++;
            const long long end = std::min(c1, first[item + 1]);
            const long long n = std::min<long long>(end - c, segmax);
            w.segs.push_back(make_int4(item, (int)(c - first[item]), (int)n, 0));
            c += n;
        }
    }
    w.cta_seg[grid] = (int)w.segs.size();
    // segments are in global chunk order, so each item's are contiguous
    w.item_seg_off.assign(p.nitems + 1, 0);
    for (const int4 &s : w.segs) w.item_seg_off[s.x + 1]++;
    for (int i = 0; i < p.nitems; i++) w.item_seg_off[i + 1] += w.item_seg_off[i];
    return w;
}

void upload_worklist(Plan &p, const WorkList &w, int grid)
{
    const size_t nseg = w.segs.size();
    if (nseg > p.segs_cap) {
        bfree(p.stream, p.d_segs);
        bfree(p.stream, p.d_item_segs);
        bfree(p.stream, p.d_partial);
        p.d_segs = balloc<int4>(p.stream, nseg);
        p.d_item_segs = balloc<int>(p.stream, nseg);
        p.d_partial = balloc<float>(p.stream, nseg * 128 * 64);
        p.segs_cap = nseg;
    }
    if ((size_t)grid + 1 > p.cta_cap) {
        bfree(p.stream, p.d_cta_seg);
        p.d_cta_seg = balloc<int>(p.stream, (size_t)grid + 1);
        p.cta_cap = (size_t)grid + 1;
    }
    std::vector<int> ids(nseg);
    for (size_t i = 0; i < nseg; i++) ids[i] = (int)i;
    BCK(stage_to_device(p.d_segs, w.segs.data(), nseg * sizeof(int4), p.stream));
    BCK(stage_to_device(p.d_item_segs, ids.data(), nseg * sizeof(int), p.stream));
    BCK(stage_to_device(p.d_cta_seg, w.cta_seg.data(), (grid + 1) * sizeof(int), p.stream));
    BCK(stage_to_device(p.d_item_seg_off, w.item_seg_off.data(), (p.nitems + 1) * sizeof(int), p.stream));
    BCK(cudaStreamSynchronize(p.stream));
    p.nseg = (int)nseg;
}

BatchArgs batch_args(const Plan &p)
{
    BatchArgs a{};
    a.items = p.d_items;
    a.segs = p.d_segs;
    a.cta_seg = p.d_cta_seg;
    a.frag_pos = p.d_pos;
    a.frag_spos = p.d_spos;
    a.frag_n = p.d_nrm;
    a.vis = p.d_vis;
    a.rx = p.d_rx;
    a.src = p.d_src;
    a.nrx = p.nrx;
    a.nsrc = p.nsrc;
    a.partial = p.d_partial;
    a.status = p.d_status;
    if (p.relative) {
        a.rel_rx = p.d_rel_rx;
        a.rel_src = p.d_rel_src;
        a.rel_rx_e = p.d_erx_conj;
    }
    return a;
}

// Per item and point (rows padded to 64): D = point - item centre rounded to
// FP32 with R = |D|, and the point's phase factor e^{ik R} (FP64; for the
// receivers also its conjugate in FP32), both from the FP64 difference of
// the FP32 point and centre (k R reduced in turns).
void upload_relative(Plan &p)
{
    const size_t n = (size_t)p.nitems * kBatchMaxPoints;
    if (!p.d_rel_rx) {
        p.d_rel_rx = balloc<float4>(p.stream, n);
        p.d_rel_src = balloc<float4>(p.stream, n);
        p.d_erx = balloc<double2>(p.stream, n);
        p.d_esrc = balloc<double2>(p.stream, n);
        p.d_erx_conj = balloc<float2>(p.stream, n);
    }
    std::vector<float4> Drx(n, make_float4(0.0f, 0.0f, 0.0f, 1.0f)), Dsrc(n, make_float4(0.0f, 0.0f, 0.0f, 1.0f));
    std::vector<double2> erx(n, make_double2(0.0, 0.0)), esrc(n, make_double2(0.0, 0.0));
    auto fill = [&](const std::vector<float> &pts, int np, const BatchItem &b, float4 *D, double2 *e) {
        const double k2 = (double)b.kr / (2.0 * M_PI);
        for (int i = 0; i < np; i++) {
            const double dx = (double)pts[3 * i] - (double)b.cx, dy = (double)pts[3 * i + 1] - (double)b.cy,
                         dz = (double)pts[3 * i + 2] - (double)b.cz;
            const double R = std::sqrt(dx * dx + dy * dy + dz * dz);
            const double tu = R * k2, th = 2.0 * M_PI * (tu - std::nearbyint(tu));
            D[i] = make_float4((float)dx, (float)dy, (float)dz, (float)R);
            e[i] = make_double2(std::cos(th), std::sin(th));
        }
    };
    for (int it = 0; it < p.nitems; it++) {
        const size_t o = (size_t)it * kBatchMaxPoints;
        fill(p.h_rx, p.nrx, p.items[it], Drx.data() + o, erx.data() + o);
        fill(p.h_src, p.nsrc, p.items[it], Dsrc.data() + o, esrc.data() + o);
    }
    BCK(stage_to_device(p.d_rel_rx, Drx.data(), n * sizeof(float4), p.stream));
    BCK(stage_to_device(p.d_rel_src, Dsrc.data(), n * sizeof(float4), p.stream));
    BCK(stage_to_device(p.d_erx, erx.data(), n * sizeof(double2), p.stream));
    BCK(stage_to_device(p.d_esrc, esrc.data(), n * sizeof(double2), p.stream));
    std::vector<float2> ec(n);
    for (size_t i = 0; i < n; i++) ec[i] = make_float2((float)erx[i].x, (float)-erx[i].y);
    BCK(stage_to_device(p.d_erx_conj, ec.data(), n * sizeof(float2), p.stream));
    BCK(cudaStreamSynchronize(p.stream));
}

BatchVisArgs vis_args(const Plan &p)
{
    BatchVisArgs v{};
    v.items = p.d_items;
    v.nitems = p.nitems;
    v.nfrag = p.nfrag;
    v.frag_pos = p.d_pos;
    v.frag_spos = p.d_spos;
    v.frag_n = p.d_nrm;
    v.rx = p.d_rx;
    v.src = p.d_src;
    v.nrx = p.nrx;
    v.nsrc = p.nsrc;
    v.bvh = p.d_bvh;
    v.vis = p.d_vis;
    v.hard = p.d_hard;
    v.hard_count = p.d_hard_count;
    v.hard_cap = p.hard_cap;
    return v;
}

// The device work of one run on the plan's stream (captured into the graph;
// the events are external event-record nodes, readable after a replay).
void enqueue_run(Plan &p)
{
    BCK(cudaEventRecordWithFlags(p.ev[0], p.stream, cudaEventRecordExternal));
    launch_batch_vis(vis_args(p), p.nsm, p.stream);
    BCK(cudaEventRecordWithFlags(p.ev[1], p.stream, cudaEventRecordExternal));
    launch_batch(batch_args(p), p.tune.kc, p.tune.grid, p.att != 0.0f, p.stream);
    BCK(cudaEventRecordWithFlags(p.ev[2], p.stream, cudaEventRecordExternal));
    launch_batch_reduce(p.d_partial, p.d_item_seg_off, p.d_item_segs, p.nitems, p.nrx, p.nsrc,
                        p.relative ? p.d_erx : nullptr, p.relative ? p.d_esrc : nullptr, p.d_out, p.stream);
    BCK(cudaEventRecordWithFlags(p.ev[3], p.stream, cudaEventRecordExternal));
}

void check_status(Plan &p)
{
    int st = 0;
    BCK(cudaMemcpyAsync(&st, p.d_status, sizeof(int), cudaMemcpyDeviceToHost, p.stream));
    BCK(cudaStreamSynchronize(p.stream));
    if (st != 0)
        bfail(-11, "batch: a CTA gave up waiting for the tensor core (status %d%s)", st,
              st == 2 ? ": its tensor memory was left allocated because an MMA was still in flight" : "");
}

// Time the candidate tile shapes on this plan's items and keep the fastest.
// Tuning results of this process, keyed by device, item count, fragment
// count (to 1/64 of a power of two), sources and receivers: a plan of the
// same shape skips the timing runs.
struct TuneKey {
    int dev, nitems, nsrc, nrx, att;
    long long frag_bucket;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(dev, nitems, nsrc, nrx, att, frag_bucket) <
               std::tie(o.dev, o.nitems, o.nsrc, o.nrx, o.att, o.frag_bucket);
    }
};
std::map<TuneKey, Tuning> g_tune_cache;

long long frag_bucket(long long n)
{
    int e = 0;
    while ((n >> e) > 64) e++;
    return ((n >> e) << 8) | e;
}

void autotune(Plan &p)
{
    int dev = 0, nsm = 0;
    BCK(cudaGetDevice(&dev));
    const TuneKey key{dev, p.nitems, p.nsrc, p.nrx, p.att != 0.0f ? 1 : 0, frag_bucket(p.nfrag)};
    auto hit = g_tune_cache.find(key);
    if (hit != g_tune_cache.end()) {
        p.tune = hit->second;
        p.tune_cached = true;
        WorkList w = make_worklist(p, p.tune.kc, p.tune.grid);
        upload_worklist(p, w, p.tune.grid);
        return;
    }
    BCK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    int smem_optin = 0;
    BCK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    std::vector<Tuning> cand;
    // fragments per operand stage x persistent CTAs per SM (as many as shared
    // memory holds, up to four; each CTA takes 64 of the SM's 512 tensor-memory columns)
    for (int kc : {16, 32, 64}) {
        const size_t sm = batch_smem_bytes(kc) + 10240;  // + static shared memory and the per-CTA reserve
        const int per_sm = std::max(1, std::min(4, (int)((size_t)smem_optin / sm)));
        for (int c = 1; c <= per_sm; c++) {
            Tuning t;
            t.kc = kc;
            t.grid = c * nsm;
            cand.push_back(t);
        }
    }
    // interaction bits once (the candidates share them)
    launch_batch_vis(vis_args(p), p.nsm, p.stream);
    BCK(cudaGetLastError());
    p.tried.clear();
    Tuning best;
    best.ms = 3.0e38f;
    for (Tuning t : cand) {
        WorkList w = make_worklist(p, t.kc, t.grid);
        upload_worklist(p, w, t.grid);
        float tot = 0.0f;
        for (int rep = 0; rep < 3; rep++) {
            BCK(cudaEventRecord(p.ev[1], p.stream));
            launch_batch(batch_args(p), t.kc, t.grid, p.att != 0.0f, p.stream);
            BCK(cudaGetLastError());
            BCK(cudaEventRecord(p.ev[2], p.stream));
            BCK(cudaEventSynchronize(p.ev[2]));
            float ms = 0.0f;
            BCK(cudaEventElapsedTime(&ms, p.ev[1], p.ev[2]));
            if (rep > 0) tot += ms;  // the first run warms up
        }
        check_status(p);
        t.ms = tot / 2.0f;
        p.tried.push_back(t);
        if (t.ms < best.ms) best = t;
    }
    p.tune = best;
    g_tune_cache[key] = best;
    WorkList w = make_worklist(p, best.kc, best.grid);
    upload_worklist(p, w, best.grid);
}

void capture(Plan &p)
{
    if (p.exec) {
        cudaGraphExecDestroy(p.exec);
        p.exec = nullptr;
    }
    if (p.graph) {
        cudaGraphDestroy(p.graph);
        p.graph = nullptr;
    }
    BCK(cudaStreamBeginCapture(p.stream, cudaStreamCaptureModeThreadLocal));
    try {
        enqueue_run(p);
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(p.stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    BCK(cudaStreamEndCapture(p.stream, &p.graph));
    BCK(cudaGraphInstantiate(&p.exec, p.graph, 0));
}

std::unique_ptr<Plan> make_plan(const float *tris, const int *tri_off, int nscenes, const float *src, int nsrc,
                                const float *rx, int nrx, const float *freqs, int nfreq, float cp, float att,
                                float per_wl)
{
    if (!tris || !tri_off || !src || !rx || !freqs) bfail(-6, "sonar_batch_plan: null argument");
    if (nscenes <= 0 || nfreq <= 0) bfail(-6, "sonar_batch_plan: %d scenes, %d frequencies", nscenes, nfreq);
    if (nsrc <= 0 || nsrc > kBatchMaxPoints || nrx <= 0 || nrx > kBatchMaxPoints)
        bfail(-6, "sonar_batch_plan: %d sources and %d receivers (1 to %d each)", nsrc, nrx, kBatchMaxPoints);
    if (!(cp > 0.0f) || !(per_wl > 0.0f) || !std::isfinite(att) || att < 0.0f)
        bfail(-6, "sonar_batch_plan: invalid cp %g, per_wavelength %g or attenuation %g", cp, per_wl, att);
    if (tri_off[0] != 0) bfail(-6, "sonar_batch_plan: scene_tri_off[0] must be 0");
    for (int s = 0; s < nscenes; s++)
        if (tri_off[s + 1] <= tri_off[s]) bfail(-6, "sonar_batch_plan: scene %d has no triangles", s);
    for (int f = 0; f < nfreq; f++)
        if (!(freqs[f] > 0.0f) || !std::isfinite(freqs[f])) bfail(-6, "sonar_batch_plan: frequency %d invalid", f);
    const long long ntri = tri_off[nscenes];
    for (long long i = 0; i < 9 * ntri; i++)
        if (!std::isfinite(tris[i])) bfail(-6, "sonar_batch_plan: non-finite vertex coordinate");
    for (int i = 0; i < 3 * nsrc; i++)
        if (!std::isfinite(src[i])) bfail(-6, "sonar_batch_plan: non-finite source coordinate");
    for (int i = 0; i < 3 * nrx; i++)
        if (!std::isfinite(rx[i])) bfail(-6, "sonar_batch_plan: non-finite receiver coordinate");

    auto p = std::make_unique<Plan>();
    p->nscenes = nscenes;
    p->nfreq = nfreq;
    p->nsrc = nsrc;
    p->nrx = nrx;
    p->nitems = nscenes * nfreq;
    p->cp = cp;
    p->att = att;
    p->per_wl = per_wl;
    BCK(batch_prepare());
    BCK(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    for (cudaEvent_t &e : p->ev) BCK(cudaEventCreate(&e));

    // ---- fragments of every item, in parallel over items
    std::vector<ItemFrags> frags(p->nitems);
    {
        const unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        std::vector<std::string> errs(nth);
        for (unsigned w = 0; w < nth; w++)
            pool.emplace_back([&, w] {
                try {
                    for (int it = (int)w; it < p->nitems; it += (int)nth) {
                        const int s = it / nfreq, f = it % nfreq;
                        const float delta = cp / freqs[f] / per_wl;
                        fragment_item(tris + 9 * (size_t)tri_off[s], tri_off[s + 1] - tri_off[s], tri_off[s], delta,
                                      frags[it]);
                    }
                } catch (const std::exception &e) {
                    errs[w] = e.what();
                }
            });
        for (auto &t : pool) t.join();
        for (auto &e : errs)
            if (!e.empty()) bfail(-3, "sonar_batch_plan: fragmentation failed: %s", e.c_str());
    }
    // ---- items
    long long frag0 = 0;
    p->items.resize(p->nitems);
    p->item_cells.resize(p->nitems);
    for (int it = 0; it < p->nitems; it++) {
        const ItemFrags &F = frags[it];
        const long long n = (long long)F.pos.size();
        if (n > (1LL << 30)) bfail(-3, "sonar_batch_plan: item %d has %lld fragments", it, n);
        const int f = it % nfreq;
        // src/Model.cpp:44-54: omega and k are FP32
        const float omega = (float)(2 * M_PI * (double)freqs[f]);
        const float k = omega / cp;
        const double kr = (double)k, k2 = kr / (2.0 * M_PI);
        BatchItem &b = p->items[it];
        b = BatchItem{};
        b.frag0 = (int)frag0;
        b.nfrag = (int)n;
        b.scene = it / nfreq;
        b.kr = (float)kr;
        b.ka = att;
        b.k2hi = (float)k2;
        b.k2lo = (float)(k2 - (double)b.k2hi);
        b.kr4pi = (float)(kr / (4.0 * M_PI));
        p->item_cells[it] = F.ncells;
        p->pairs += (double)nsrc * ((double)F.ncells + (double)n * nrx);
        frag0 += n;
        p->ncells += F.ncells;
    }
    if (frag0 > (1LL << 31) - 1) bfail(-3, "sonar_batch_plan: %lld fragments in all (limit 2^31 - 1)", frag0);
    p->nfrag = frag0;
    // ---- uploads
    std::vector<float4> pos, spos, nrm;
    std::vector<int> facet;
    pos.reserve(frag0);
    spos.reserve(frag0);
    nrm.reserve(frag0);
    facet.reserve(frag0);
    for (auto &F : frags) {
        pos.insert(pos.end(), F.pos.begin(), F.pos.end());
        spos.insert(spos.end(), F.spos.begin(), F.spos.end());
        nrm.insert(nrm.end(), F.nrm.begin(), F.nrm.end());
        facet.insert(facet.end(), F.facet.begin(), F.facet.end());
        F = ItemFrags();
    }
    std::vector<float4> facet_n(ntri);
    for (long long t = 0; t < ntri; t++) {
        const float *v = tris + 9 * t;
        const FacetFrame F = make_frame({v[0], v[1], v[2]}, {v[3], v[4], v[5]}, {v[6], v[7], v[8]}, 1.0f);
        facet_n[t] = make_float4(F.normal.x, F.normal.y, F.normal.z, 0.0f);
    }
    std::vector<float4> s4(nsrc), r4(nrx);
    for (int i = 0; i < nsrc; i++) s4[i] = make_float4(src[3 * i], src[3 * i + 1], src[3 * i + 2], 0.0f);
    for (int i = 0; i < nrx; i++) r4[i] = make_float4(rx[3 * i], rx[3 * i + 1], rx[3 * i + 2], 0.0f);
    p->d_pos = balloc<float4>(p->stream, frag0);
    p->d_spos = balloc<float4>(p->stream, frag0);
    p->d_nrm = balloc<float4>(p->stream, frag0);
    p->d_facet = balloc<int>(p->stream, frag0);
    p->d_facet_n = balloc<float4>(p->stream, ntri);
    p->d_src = balloc<float4>(p->stream, nsrc);
    p->d_rx = balloc<float4>(p->stream, nrx);
    p->d_vis = balloc<uint4>(p->stream, frag0);
    // shadow-test queue: pair ids 128 n + point fit 32 bits below 2^25 fragments (else every
    // pair is tested where it is found); up to 1/16 of all pairs or 32 M entries
    p->hard_cap = frag0 < (1LL << 25) ? (unsigned)std::min<long long>(1LL << 25, std::max<long long>(frag0 * 8, 1024))
                                      : 0u;
    p->d_hard = balloc<unsigned>(p->stream, std::max<unsigned>(p->hard_cap, 1u));
    p->d_hard_count = balloc<unsigned>(p->stream, 1);
    {
        int dev = 0;
        BCK(cudaGetDevice(&dev));
        BCK(cudaDeviceGetAttribute(&p->nsm, cudaDevAttrMultiProcessorCount, dev));
    }
    p->d_items = balloc<BatchItem>(p->stream, p->nitems);
    p->d_item_seg_off = balloc<int>(p->stream, p->nitems + 1);
    p->d_status = balloc<int>(p->stream, 1);
    p->d_out = balloc<double2>(p->stream, (size_t)p->nitems * nrx * nsrc);
    cudaStream_t st = p->stream;
    if (frag0) {
        BCK(stage_to_device(p->d_pos, pos.data(), frag0 * sizeof(float4), st));
        BCK(stage_to_device(p->d_spos, spos.data(), frag0 * sizeof(float4), st));
        BCK(stage_to_device(p->d_nrm, nrm.data(), frag0 * sizeof(float4), st));
        BCK(stage_to_device(p->d_facet, facet.data(), frag0 * sizeof(int), st));
    }
    BCK(stage_to_device(p->d_facet_n, facet_n.data(), ntri * sizeof(float4), st));
    BCK(stage_to_device(p->d_src, s4.data(), nsrc * sizeof(float4), st));
    BCK(stage_to_device(p->d_rx, r4.data(), nrx * sizeof(float4), st));
    BCK(cudaMemsetAsync(p->d_status, 0, sizeof(int), st));
    // ---- occluders of each scene (every triangle of the scene, OptiX.cpp:264-296)
    // and its convexity: every vertex on or behind every triangle's plane
    std::vector<BvhView> views(nscenes);
    std::vector<int> node0(nscenes + 1, 0), tri0(nscenes + 1, 0);
    std::vector<BvhNode> nodes;
    std::vector<float4> trec;
    double maxp = 0.0;
    for (int i = 0; i < 3 * nsrc; i++) maxp = std::max(maxp, (double)std::fabs(src[i]));
    for (int i = 0; i < 3 * nrx; i++) maxp = std::max(maxp, (double)std::fabs(rx[i]));
    p->convex.assign(nscenes, 0);
    std::vector<std::array<float, 3>> centre(nscenes);
    for (int s = 0; s < nscenes; s++) {
        std::vector<std::array<float, 9>> t;
        double maxc = maxp, maxv = 0.0;
        for (int q = tri_off[s]; q < tri_off[s + 1]; q++) {
            std::array<float, 9> a;
            for (int k = 0; k < 9; k++) {
                a[k] = tris[9 * (size_t)q + k];
                maxc = std::max(maxc, (double)std::fabs(a[k]));
                maxv = std::max(maxv, (double)std::fabs(a[k]));
            }
            t.push_back(a);
        }
        p->convex[s] = scene_is_convex(t, 1e-6 * (1.0 + maxv)) ? 1 : 0;
        {
            float lo[3] = {t[0][0], t[0][1], t[0][2]}, hi[3] = {lo[0], lo[1], lo[2]};
            for (const auto &a : t)
                for (int v = 0; v < 3; v++)
                    for (int k = 0; k < 3; k++) {
                        lo[k] = std::min(lo[k], a[3 * v + k]);
                        hi[k] = std::max(hi[k], a[3 * v + k]);
                    }
            centre[s] = {(float)(0.5 * ((double)lo[0] + hi[0])), (float)(0.5 * ((double)lo[1] + hi[1])),
                         (float)(0.5 * ((double)lo[2] + hi[2]))};
        }
        // node boxes padded by 1e-5 (1 + largest coordinate of triangles and points):
        // the FP32 slab test and the crossing point of a hit are within a few 1e-7
        // (1 + coordinate) of exact, so every box a hit needs is opened
        BvhHost b = build_bvh(t, 1e-5 * (1.0 + maxc));
        node0[s] = (int)nodes.size();
        tri0[s] = (int)(trec.size() / 4);
        nodes.insert(nodes.end(), b.nodes.begin(), b.nodes.end());
        trec.insert(trec.end(), b.tris.begin(), b.tris.end());
        node0[s + 1] = (int)nodes.size();
        tri0[s + 1] = (int)(trec.size() / 4);
    }
    p->d_nodes = balloc<float4>(p->stream, 2 * nodes.size());
    p->d_tris = balloc<float4>(p->stream, trec.size());
    for (int s = 0; s < nscenes; s++)
        views[s] = BvhView{p->d_nodes + 2 * (size_t)node0[s], p->d_tris + 4 * (size_t)tri0[s],
                           node0[s + 1] - node0[s], tri0[s + 1] - tri0[s]};
    for (int it = 0; it < p->nitems; it++) {
        BatchItem &b = p->items[it];
        b.convex = p->convex[b.scene];
        b.cx = centre[b.scene][0];
        b.cy = centre[b.scene][1];
        b.cz = centre[b.scene][2];
    }
    p->h_src.assign(src, src + 3 * (size_t)nsrc);
    p->h_rx.assign(rx, rx + 3 * (size_t)nrx);
    p->d_bvh = balloc<BvhView>(p->stream, nscenes);
    BCK(stage_to_device(p->d_nodes, nodes.data(), nodes.size() * sizeof(BvhNode), st));
    BCK(stage_to_device(p->d_tris, trec.data(), trec.size() * sizeof(float4), st));
    BCK(stage_to_device(p->d_bvh, views.data(), nscenes * sizeof(BvhView), st));
    BCK(stage_to_device(p->d_items, p->items.data(), p->nitems * sizeof(BatchItem), st));
    BCK(cudaStreamSynchronize(st));
    autotune(*p);
    capture(*p);
    return p;
}

void run_plan(Plan &p, double *out)
{
    BCK(cudaMemsetAsync(p.d_status, 0, sizeof(int), p.stream));
    BCK(cudaGraphLaunch(p.exec, p.stream));
    if (out)
        BCK(stage_to_host(out, p.d_out, (size_t)p.nitems * p.nrx * p.nsrc * sizeof(double2), p.stream));
    BCK(cudaStreamSynchronize(p.stream));
    check_status(p);
    BCK(cudaEventElapsedTime(&p.vis_ms, p.ev[0], p.ev[1]));
    BCK(cudaEventElapsedTime(&p.gemm_ms, p.ev[1], p.ev[2]));
    BCK(cudaEventElapsedTime(&p.reduce_ms, p.ev[2], p.ev[3]));
    p.runs++;
}

template <class F>
long long bguard(F &&f)
{
    try {
        return f();
    } catch (const BatchError &e) {
        set_error_message(e.what());
        return e.code;
    } catch (const std::exception &e) {
        set_error_message(e.what());
        return -1;
    } catch (...) {
        set_error_message("batch: unknown error");
        return -1;
    }
}

Plan &find(long long id)
{
    auto it = g_plans.find(id);
    if (it == g_plans.end()) bfail(-4, "no batch plan %lld", id);
    return *it->second;
}

}  // namespace
}  // namespace sonar

using namespace sonar;

extern "C" {

long long sonar_batch_plan(const float *tris, const int *scene_tri_off, int nscenes, const float *src_xyz, int nsrc,
                           const float *rx_xyz, int nrx, const float *freqs, int nfreq, float cp, float attenuation,
                           float per_wavelength)
{
    std::lock_guard<std::mutex> lk(g_lock);
    return bguard([&]() -> long long {
        auto p = make_plan(tris, scene_tri_off, nscenes, src_xyz, nsrc, rx_xyz, nrx, freqs, nfreq, cp, attenuation,
                           per_wavelength);
        const long long id = g_next++;
        g_plans[id] = std::move(p);
        return id;
    });
}

int sonar_batch_run(long long plan, double *out)
{
    std::lock_guard<std::mutex> lk(g_lock);
    return (int)bguard([&]() -> long long {
        run_plan(find(plan), out);
        return 0;
    });
}

int sonar_batch_set_points(long long plan, const float *src_xyz, int nsrc, const float *rx_xyz, int nrx)
{
    std::lock_guard<std::mutex> lk(g_lock);
    return (int)bguard([&]() -> long long {
        Plan &p = find(plan);
        if (!src_xyz || !rx_xyz) bfail(-6, "sonar_batch_set_points: null argument");
        if (nsrc != p.nsrc || nrx != p.nrx)
            bfail(-6, "sonar_batch_set_points: the plan has %d sources and %d receivers (got %d, %d)", p.nsrc, p.nrx,
                  nsrc, nrx);
        std::vector<float4> s4(nsrc), r4(nrx);
        for (int i = 0; i < nsrc; i++) s4[i] = make_float4(src_xyz[3 * i], src_xyz[3 * i + 1], src_xyz[3 * i + 2], 0.0f);
        for (int i = 0; i < nrx; i++) r4[i] = make_float4(rx_xyz[3 * i], rx_xyz[3 * i + 1], rx_xyz[3 * i + 2], 0.0f);
        BCK(stage_to_device(p.d_src, s4.data(), nsrc * sizeof(float4), p.stream));
        BCK(stage_to_device(p.d_rx, r4.data(), nrx * sizeof(float4), p.stream));
        p.h_src.assign(src_xyz, src_xyz + 3 * (size_t)nsrc);
        p.h_rx.assign(rx_xyz, rx_xyz + 3 * (size_t)nrx);
        if (p.relative) upload_relative(p);
        return 0;
    });
}

int sonar_batch_set_relative(long long plan, int on)
{
    std::lock_guard<std::mutex> lk(g_lock);
    return (int)bguard([&]() -> long long {
        Plan &p = find(plan);
        if ((on != 0) == p.relative) return 0;
        p.relative = on != 0;
        if (p.relative) upload_relative(p);
        capture(p);
        return 0;
    });
}

int sonar_batch_set_shape(long long plan, int fragments_per_stage, int ctas_per_sm)
{
    std::lock_guard<std::mutex> lk(g_lock);
    return (int)bguard([&]() -> long long {
        Plan &p = find(plan);
        if (fragments_per_stage != 16 && fragments_per_stage != 32 && fragments_per_stage != 64)
            bfail(-6, "sonar_batch_set_shape: fragments per stage must be 16, 32 or 64 (got %d)", fragments_per_stage);
        int dev = 0, nsm = 0, smem_optin = 0;
        BCK(cudaGetDevice(&dev));
        BCK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        BCK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
        const int fit = std::max(1, std::min(4, (int)((size_t)smem_optin / (batch_smem_bytes(fragments_per_stage) + 10240))));
        if (ctas_per_sm < 1 || ctas_per_sm > fit)
            bfail(-6, "sonar_batch_set_shape: %d CTAs per SM (1 to %d fit at %d fragments per stage)", ctas_per_sm, fit,
                  fragments_per_stage);
        p.tune.kc = fragments_per_stage;
        p.tune.grid = ctas_per_sm * nsm;
        WorkList w = make_worklist(p, p.tune.kc, p.tune.grid);
        upload_worklist(p, w, p.tune.grid);
        capture(p);
        return 0;
    });
}

int sonar_batch_stream(long long plan, void **stream)
{
    std::lock_guard<std::mutex> lk(g_lock);
    return (int)bguard([&]() -> long long {
        if (!stream) bfail(-6, "sonar_batch_stream: null argument");
        *stream = (void *)find(plan).stream;
        return 0;
    });
}

int sonar_batch_stats(long long plan, char *json, int cap)
{
    std::lock_guard<std::mutex> lk(g_lock);
    return (int)bguard([&]() -> long long {
        const Plan &p = find(plan);
        std::string s;
        char buf[640];
        // pairs queued for a shadow test by the last run
        unsigned hard = 0;
        if (p.runs > 0) {
            BCK(cudaStreamSynchronize(p.stream));
            BCK(cudaMemcpy(&hard, p.d_hard_count, sizeof(unsigned), cudaMemcpyDeviceToHost));
        }
        snprintf(buf, sizeof(buf),
                 "{\"items\": %d, \"scenes\": %d, \"frequencies\": %d, \"sources\": %d, \"receivers\": %d, "
                 "\"fragments\": %lld, \"cells\": %lld, \"pairs\": %.0f, \"segments\": %d, \"convex_scenes\": %d, "
                 "\"runs\": %d, \"vis_ms\": %.6f, \"gemm_ms\": %.6f, \"reduce_ms\": %.6f, \"shadow_tests\": %u, "
                 "\"relative\": %s, "
                 "\"tuning\": {\"fragments_per_stage\": %d, \"grid\": %d, \"cached\": %s, \"candidates\": [",
                 p.nitems, p.nscenes, p.nfreq, p.nsrc, p.nrx, p.nfrag, p.ncells, p.pairs, p.nseg,
                 (int)std::count(p.convex.begin(), p.convex.end(), 1),
                 p.runs, p.vis_ms, p.gemm_ms, p.reduce_ms, hard, p.relative ? "true" : "false", p.tune.kc, p.tune.grid,
                 p.tune_cached ? "true" : "false");
        s += buf;
        for (size_t i = 0; i < p.tried.size(); i++) {
            snprintf(buf, sizeof(buf), "%s{\"fragments_per_stage\": %d, \"grid\": %d, \"ms\": %.6f}", i ? ", " : "",
                     p.tried[i].kc, p.tried[i].grid, p.tried[i].ms);
            s += buf;
        }
        s += "]}, \"item_fragments\": [";
        for (int i = 0; i < p.nitems; i++) {
            snprintf(buf, sizeof(buf), "%s%d", i ? ", " : "", p.items[i].nfrag);
            s += buf;
        }
        s += "], \"item_cells\": [";
        for (int i = 0; i < p.nitems; i++) {
            snprintf(buf, sizeof(buf), "%s%lld", i ? ", " : "", p.item_cells[i]);
            s += buf;
        }
        s += "]}";
        if (json && cap > 0) {
            const size_t n = std::min<size_t>(s.size(), (size_t)cap - 1);
            memcpy(json, s.data(), n);
            json[n] = 0;
        }
        return (long long)s.size();
    });
}

int sonar_batch_free(long long plan)
{
    std::lock_guard<std::mutex> lk(g_lock);
    return (int)bguard([&]() -> long long {
        find(plan);
        g_plans.erase(plan);
        return 0;
    });
}

int sonar_run_batch(const float *tris, const int *scene_tri_off, int nscenes, const float *src_xyz, int nsrc,
                    const float *rx_xyz, int nrx, const float *freqs, int nfreq, float cp, float attenuation,
                    float per_wavelength, double *out)
{
    std::lock_guard<std::mutex> lk(g_lock);
    return (int)bguard([&]() -> long long {
        if (!out) bfail(-6, "sonar_run_batch: null output");
        auto p = make_plan(tris, scene_tri_off, nscenes, src_xyz, nsrc, rx_xyz, nrx, freqs, nfreq, cp, attenuation,
                           per_wavelength);
        run_plan(*p, out);
        return 0;
    });
}

}  // extern "C"
