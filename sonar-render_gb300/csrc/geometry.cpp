// geometry.cpp -- facet frames, fragment grids and the occluder BVH.
//
// The frame and the area grid must reproduce the reference's FP32 results bit
// for bit (src/Facet.cpp:6-339, src/GeoMath.h:19-106), so every expression
// keeps the reference's operation order; build with -ffp-contract=off.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <pthread.h>
#include <mutex>
#include <numeric>
#include <stdexcept>
#include <string>
#include <tuple>
#include <thread>

#include "host.h"

namespace sonar {
namespace {

inline Vec3 sub(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float dot3(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float len3(Vec3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline Vec3 unit3(Vec3 a)
{
    const float L = len3(a);
    return {a.x / L, a.y / L, a.z / L};
}
inline Vec3 cross3(Vec3 a, Vec3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

}  // namespace

FacetFrame make_frame(Vec3 v1, Vec3 v2, Vec3 v3, float delta)
{
    FacetFrame f;
    f.v1 = v1;
    f.v2 = v2;
    f.v3 = v3;
    f.delta = delta;
    // normal = unit((v1 - v2) x (v1 - v3)) == unit((v2 - v1) x (v3 - v1))
    f.normal = unit3(cross3(sub(v1, v2), sub(v1, v3)));

    // the longest edge (first maximum wins) is the base, running origin -> end;
    // the remaining vertex is the apex
    const float e[3] = {len3(sub(v1, v2)), len3(sub(v1, v3)), len3(sub(v2, v3))};
    int m = 0;
    if (e[1] > e[m]) m = 1;
    if (e[2] > e[m]) m = 2;
    const Vec3 origin = (m == 2) ? v2 : v1;
    const Vec3 end = (m == 0) ? v2 : v3;
    const Vec3 apex = (m == 0) ? v3 : (m == 1) ? v2 : v1;

    const Vec3 along = sub(end, origin);
    const Vec3 u = unit3(along);
    const float proj = dot3(u, sub(apex, origin));
    f.base = {origin.x + u.x * proj, origin.y + u.y * proj, origin.z + u.z * proj};
    const Vec3 alt = sub(apex, f.base);

    f.baseLen = e[m];
    f.height = len3(alt);
    f.baseNeg = len3(sub(origin, f.base));
    f.basePos = len3(sub(f.base, end));
    f.xAxis = u;
    f.yAxis = unit3(alt);
    f.area = (f.baseLen * f.height) / 2.0f;

    const float cn = std::ceil(std::fabs(f.baseNeg) / delta);
    const float cp = std::ceil(std::fabs(f.basePos) / delta);
    const float cy = std::ceil(f.height / delta);
    // a triangle whose frame is not finite (coincident vertices) gets no cells;
    // a zero-height one gets numYpnts = 0 as in the reference
    if (!std::isfinite(cn) || !std::isfinite(cp) || !std::isfinite(cy)) {
        f.nx = f.ny = f.neg = 0;
    } else {
        f.neg = (int)cn;
        f.nx = f.neg + (int)cp;
        f.ny = (int)cy;
    }
    return f;
}

void fragment_areas(const FacetFrame &f, float *area) { fragment_area_rows(f, area, 0, f.ny); }

// Each cell's area depends only on the tests at its own four corners, so any
// range of rows gives the same values as the whole grid.
void fragment_area_rows(const FacetFrame &f, float *area, int j0, int j1)
{
    const int nx = f.nx, neg = f.neg;
    const float d = f.delta, H = f.height, h = d / 2;
    std::fill(area + (size_t)j0 * nx, area + (size_t)j1 * nx, 0.0f);
    // slopes of the two sloping sides: x > 0 is the positive-base side
    const float mPos = H / (-f.basePos);
    const float mNeg = H / (f.baseNeg);
    std::vector<unsigned char> inL(j1 - j0 + 1), inR(j1 - j0 + 1);

    for (int i = 0; i < nx; i++) {
        const float xc = ((float)(i - neg) * d) + h;  // column centre
        const float xL = xc - h, xR = xc + h;
        const bool pos = xc > 0;
        const float m = pos ? mPos : mNeg;
        const float yL = m * xL + H;  // side line at the column's left and right edges
        const float yR = m * xR + H;
        for (int j = j0; j <= j1; j++) {
            inL[j - j0] = d * (float)j <= yL;
            inR[j - j0] = d * (float)j <= yR;
        }
        for (int j = j0; j < j1; j++) {
            const bool lb = inL[j - j0], rb = inR[j - j0], lt = inL[j - j0 + 1], rt = inR[j - j0 + 1];
            float *A = area + (size_t)j * nx + i;
            if (!lb && !rb && !lt && !rt) break;  // above the triangle: rest of column empty
            if (lb && rb && lt && rt) {
                *A = d * d;
                continue;
            }
            const float yB = d * (float)j;
            if (pos) {
                const float yT = d * (float)(j + 1);
                if (lb && rb && lt && !rt) {
                    const float xTop = (yT - H) / mPos;
                    *A = d * d - (yT - yR) * (xR - xTop) / 2;
                } else if (lb && rb && !lt && !rt) {
                    *A = ((yL - yR) * d / 2) + (yR - yB) * d;
                } else if (lb && !rb && lt && !rt) {
                    const float xTop = ((yT - H) / mPos) - xL;
                    const float xBot = ((yB - H) / mPos) - xL;
                    *A = (xTop * d) + (xBot - xTop) * d / 2;
                } else if (lb && !rb && !lt && !rt) {
                    *A = (yL - yB) * (((yB - H) / mPos) - xL) / 2;
                }
            } else {
                const float yc = ((float)j * d) + h;  // row centre
                if (lb && rb && !lt && rt) {
                    *A = d * d - (yc + h - yL) * (-(xL - ((yc + h - H) / mNeg)) / 2);
                } else if (lb && rb && !lt && !rt) {
                    *A = (yR - yL) * d / 2 + ((yL - (yc - h)) * d);
                } else if (!lb && rb && !lt && rt) {
                    *A = -((yc - h - H) / mNeg - (yc + h - H) / mNeg) * d / 2 - (((yc + h - H) / mNeg) - xR) * d;
                } else if (!lb && rb && !lt && !rt) {
                    *A = (yR - (yc - h)) * (-((((yc - h) - H) / mNeg) - xR)) / 2;
                }
            }
        }
    }
}

namespace {

// Host workers kept for the process (min(16, cores) - 1 threads; the calling
// thread is the last worker).  One job at a time: a call made while a job
// runs -- from another thread, or from inside a unit -- runs its units
// serially instead of waiting.
thread_local bool tl_in_job = false;

class UnitPool {
  public:
    static UnitPool &get()
    {
        static UnitPool *p = new UnitPool();  // never destroyed: the workers outlive static destructors
        return *p;
    }

    bool run(long long n, const std::function<void(long long)> &fn)
    {
        if (tl_in_job || nworkers_ == 0) return false;
        std::unique_lock<std::mutex> busy(run_mu_, std::try_to_lock);
        if (!busy.owns_lock()) return false;
        {
            std::lock_guard<std::mutex> lk(mu_);
            fn_ = &fn;
            n_ = n;
            next_ = 0;
            err_.clear();
            remaining_ = nworkers_;
            gen_++;
        }
        cv_.notify_all();
        tl_in_job = true;
        drain();
        tl_in_job = false;
        std::unique_lock<std::mutex> lk(mu_);
        done_.wait(lk, [&] { return remaining_ == 0; });
        fn_ = nullptr;
        if (!err_.empty()) throw std::runtime_error(err_);
        return true;
    }

    // a forked child has none of the workers: every call there runs serially
    void forget_workers() { nworkers_ = 0; }

  private:
    UnitPool()
    {
        pthread_atfork(nullptr, nullptr, [] { UnitPool::get().forget_workers(); });
        const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        for (unsigned w = 0; w + 1 < hw; w++) {
            try {
                std::thread([this] { loop(); }).detach();
                nworkers_++;
            } catch (...) {
                break;
            }
        }
    }

    void loop()
    {
        tl_in_job = true;
        unsigned long long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
            }
            drain();
            std::lock_guard<std::mutex> lk(mu_);
            if (--remaining_ == 0) done_.notify_all();
        }
    }

    void drain()
    {
        for (long long u = next_++; u < n_; u = next_++) {
            try {
                (*fn_)(u);
            } catch (const std::exception &e) {
                std::lock_guard<std::mutex> lk(err_mu_);
                if (err_.empty()) err_ = e.what();
                next_ = n_;
            }
        }
    }

    std::mutex run_mu_, mu_, err_mu_;
    std::condition_variable cv_, done_;
    const std::function<void(long long)> *fn_ = nullptr;
    long long n_ = 0;
    std::atomic<long long> next_{0};
    unsigned long long gen_ = 0;
    int nworkers_ = 0, remaining_ = 0;
    std::string err_;
};

}  // namespace

void parallel_units(long long n, const std::function<void(long long)> &fn)
{
    if (n <= 0) return;
    if (n > 1 && UnitPool::get().run(n, fn)) return;
    for (long long u = 0; u < n; u++) fn(u);
}

Vec3 fragment_centroid(const FacetFrame &f, int x, int y, bool source_hop)
{
    const float d = f.delta;
    float xo = d * (float)(x - f.neg);
    if (source_hop) xo = xo + d / 2;
    const float yo = d * (float)y + d / 2;
    const Vec3 xa = {f.xAxis.x * xo, f.xAxis.y * xo, f.xAxis.z * xo};
    const Vec3 ya = {f.yAxis.x * yo, f.yAxis.y * yo, f.yAxis.z * yo};
    return {(f.base.x + xa.x) + ya.x, (f.base.y + xa.y) + ya.y, (f.base.z + xa.z) + ya.z};
}

// Every vertex of the scene on or behind every triangle's plane (within tol,
// in double).  Scenes of more than 20,000 triangles are not checked (treated
// as non-convex: every pair gets the exact shadow test).
bool scene_is_convex(const std::vector<std::array<float, 9>> &t, double tol)
{
    if (t.size() > 20000) return false;
    constexpr long long kChunk = 64;  // planes per work unit
    std::atomic<bool> convex{true};
    parallel_units(((long long)t.size() + kChunk - 1) / kChunk, [&](long long u) {
        const size_t i1 = std::min(t.size(), (size_t)((u + 1) * kChunk));
        for (size_t i = (size_t)u * kChunk; i < i1 && convex.load(std::memory_order_relaxed); i++) {
            const auto &a = t[i];
            const double ux = (double)a[3] - a[0], uy = (double)a[4] - a[1], uz = (double)a[5] - a[2];
            const double vx = (double)a[6] - a[0], vy = (double)a[7] - a[1], vz = (double)a[8] - a[2];
            double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
            const double L = std::sqrt(nx * nx + ny * ny + nz * nz);
            if (!(L > 0.0)) {
                convex = false;
                return;
            }
            nx /= L;
            ny /= L;
            nz /= L;
            const double c = nx * a[0] + ny * a[1] + nz * a[2];
            for (const auto &b : t)
                for (int k = 0; k < 3; k++)
                    if (nx * b[3 * k] + ny * b[3 * k + 1] + nz * b[3 * k + 2] - c > tol) {
                        convex = false;
                        return;
                    }
        }
    });
    return convex;
}

// ---------------------------------------------------------------- BVH
namespace {

struct TriBox {
    double lo[3], hi[3], c[3];
};

struct Builder {
    const std::vector<TriBox> &box;
    std::vector<int> &order;
    std::vector<BvhNode> &nodes;
    double pad;
    int depth = 0;

    int build(int t0, int tn, int level)
    {
        depth = std::max(depth, level);
        const int id = (int)nodes.size();
        nodes.push_back(BvhNode{});
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        double clo[3] = {1e300, 1e300, 1e300}, chi[3] = {-1e300, -1e300, -1e300};
        for (int i = t0; i < t0 + tn; i++) {
            const TriBox &b = box[order[i]];
            for (int k = 0; k < 3; k++) {
                lo[k] = std::min(lo[k], b.lo[k]);
                hi[k] = std::max(hi[k], b.hi[k]);
                clo[k] = std::min(clo[k], b.c[k]);
                chi[k] = std::max(chi[k], b.c[k]);
            }
        }
        BvhNode n{};
        for (int k = 0; k < 3; k++) {
            n.lo[k] = (float)(lo[k] - pad);
            n.hi[k] = (float)(hi[k] + pad);
        }
        if (tn <= 4 || level >= 48) {
            n.left = -(t0 + 1);
            n.right = tn;
            nodes[id] = n;
            return id;
        }
        int ax = 0;
        for (int k = 1; k < 3; k++)
            if (chi[k] - clo[k] > chi[ax] - clo[ax]) ax = k;
        const int half = tn / 2;
        std::nth_element(order.begin() + t0, order.begin() + t0 + half, order.begin() + t0 + tn,
                         [&](int a, int b) { return box[a].c[ax] < box[b].c[ax]; });
        const int l = build(t0, half, level + 1);
        const int r = build(t0 + half, tn - half, level + 1);
        n.left = l;
        n.right = r;
        nodes[id] = n;
        return id;
    }
};

}  // namespace

BvhHost build_bvh(const std::vector<std::array<float, 9>> &tris, double pad)
{
    BvhHost out;
    const int n = (int)tris.size();
    std::vector<TriBox> box(n);
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < 3; k++) {
            const double a = tris[i][k], b = tris[i][3 + k], c = tris[i][6 + k];
            box[i].lo[k] = std::min(a, std::min(b, c));
            box[i].hi[k] = std::max(a, std::max(b, c));
            box[i].c[k] = 0.5 * (box[i].lo[k] + box[i].hi[k]);
        }
    }
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    if (n > 0) {
        Builder b{box, order, out.nodes, pad};
        b.build(0, n, 0);
        out.depth = b.depth;
    }
    // triangle records in leaf order: plane (n, c) and the three inward edge
    // planes (m_k, c_k), computed in double from the FP32 vertices
    out.tris.resize((size_t)4 * n);
    for (int q = 0; q < n; q++) {
        const auto &t = tris[order[q]];
        const double v[3][3] = {{t[0], t[1], t[2]}, {t[3], t[4], t[5]}, {t[6], t[7], t[8]}};
        double e1[3], e2[3], nn[3];
        for (int k = 0; k < 3; k++) {
            e1[k] = v[1][k] - v[0][k];
            e2[k] = v[2][k] - v[0][k];
        }
        nn[0] = e1[1] * e2[2] - e1[2] * e2[1];
        nn[1] = e1[2] * e2[0] - e1[0] * e2[2];
        nn[2] = e1[0] * e2[1] - e1[1] * e2[0];
        const double L = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
        float4 *rec = &out.tris[(size_t)4 * q];
        if (!(L > 0.0)) {
            // degenerate: a plane no segment can cross strictly (d0 = d1 = 0)
            for (int k = 0; k < 4; k++) rec[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            continue;
        }
        for (double &x : nn) x /= L;
        const double c = nn[0] * v[0][0] + nn[1] * v[0][1] + nn[2] * v[0][2];
        rec[0] = make_float4((float)nn[0], (float)nn[1], (float)nn[2], (float)c);
        for (int e = 0; e < 3; e++) {
            const double *p = v[e], *qv = v[(e + 1) % 3];
            const double dd[3] = {qv[0] - p[0], qv[1] - p[1], qv[2] - p[2]};
            double m[3] = {nn[1] * dd[2] - nn[2] * dd[1], nn[2] * dd[0] - nn[0] * dd[2], nn[0] * dd[1] - nn[1] * dd[0]};
            const double ml = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
            for (double &x : m) x /= ml;
            const double cm = m[0] * p[0] + m[1] * p[1] + m[2] * p[2];
            rec[1 + e] = make_float4((float)m[0], (float)m[1], (float)m[2], (float)cm);
        }
    }
    return out;
}

std::vector<int> patch_aligned_order(const FacetFrame &F, const std::vector<PatchRun> &runs, const float4 *readout,
                                     long long start)
{
    std::vector<PatchRun> full, part;
    for (const PatchRun &r : runs) (r.end - r.begin == (long long)kPatch * kPatch ? full : part).push_back(r);
    if (full.empty() || part.empty()) return {};
    // partial patches along the boundary: left of the full ones (rows
    // upwards), rows without full patches, right of the full ones (rows downwards)
    {
        const int npy = (F.ny + kPatch - 1) / kPatch;
        std::vector<int> fmin(std::max(npy, 1), INT32_MAX), fmax(std::max(npy, 1), -1);
        for (const PatchRun &r : full) {
            fmin[r.row] = std::min(fmin[r.row], r.col);
            fmax[r.row] = std::max(fmax[r.row], r.col);
        }
        auto key = [&](const PatchRun &r) {
            if (fmax[r.row] < 0) return std::make_tuple(1, r.row, r.col);   // no full patch in the row
            if (r.col < fmin[r.row]) return std::make_tuple(0, r.row, r.col);  // left, upwards
            return std::make_tuple(2, -r.row, r.col);                          // right, downwards
        };
        std::stable_sort(part.begin(), part.end(),
                         [&](const PatchRun &x, const PatchRun &y) { return key(x) < key(y); });
    }
    // the facet's triangle: inward normals of its edges (FP64)
    const double v[3][3] = {{F.v1.x, F.v1.y, F.v1.z}, {F.v2.x, F.v2.y, F.v2.z}, {F.v3.x, F.v3.y, F.v3.z}};
    double nrm[3], ein[3][3], eoff[3], lmax = 1.0;
    {
        const double e1[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
        const double e2[3] = {v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2]};
        nrm[0] = e1[1] * e2[2] - e1[2] * e2[1];
        nrm[1] = e1[2] * e2[0] - e1[0] * e2[2];
        nrm[2] = e1[0] * e2[1] - e1[1] * e2[0];
    }
    for (int q = 0; q < 3; q++) {
        const double *a = v[q], *b = v[(q + 1) % 3];
        const double e[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        lmax = std::max(lmax, std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]));
        const double n[3] = {nrm[1] * e[2] - nrm[2] * e[1], nrm[2] * e[0] - nrm[0] * e[2],
                             nrm[0] * e[1] - nrm[1] * e[0]};
        const double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int c = 0; c < 3; c++) ein[q][c] = l > 0.0 ? n[c] / l : 0.0;
        eoff[q] = ein[q][0] * a[0] + ein[q][1] * a[1] + ein[q][2] * a[2];
    }
    auto inside = [&](long long k) {
        const float4 p = readout[k];
        for (int q = 0; q < 3; q++)
            if (!(ein[q][0] * p.x + ein[q][1] * p.y + ein[q][2] * p.z - eoff[q] > 1e-6 * lmax)) return false;
        return true;
    };
    std::vector<int> good, edge;
    for (const PatchRun &r : part)
        for (long long k = r.begin; k < r.end; k++) (inside(k) ? good : edge).push_back((int)k);
    const long long ngood = (long long)good.size();
    const long long need = (kTile - start % kTile) % kTile;
    if (need > ngood) return {};
    long long n = 0;
    for (const PatchRun &r : runs) n += r.end - r.begin;
    std::vector<int> order;
    order.reserve((size_t)n);
    order.insert(order.end(), good.end() - need, good.end());
    for (const PatchRun &r : full)
        for (long long k = r.begin; k < r.end; k++) order.push_back((int)k);
    order.insert(order.end(), good.begin(), good.end() - need);
    order.insert(order.end(), edge.begin(), edge.end());
    return order;
}

}  // namespace sonar
