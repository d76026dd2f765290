/*
 * ref_harness.cpp -- runs the reference's own hot-path sources on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.sh from the reference's
 * unmodified src/Facet.cpp, src/Globals.cpp and src/OptiX.cu (compiled as host
 * C++, no fused multiply-add) into oracle/_ref/libsonar_ref.so.  It is used to
 * pin the oracle restatement and to write the golden fixtures under
 * tests/golden/.  It needs the reference's sources, so it only builds where
 * they are present.
 *
 * What is the reference's code here and what is not:
 *   - Facet construction and fragmentation: the reference's Facet class
 *     (src/Facet.cpp), unchanged.
 *   - The three sums: the reference's __raygen__rg and project* functions
 *     (src/OptiX.cu:35-445), unchanged; optixLaunch is a loop over the launch
 *     index (one call per facet, like src/OptiX.cpp:144-159) and optixTrace
 *     calls ref_vis_call() below.
 *   - Buffers and sequencing restate src/FacetCuda.cpp:8-62,114-137,
 *     src/ObjectCuda.cpp:33-52, src/FacetCuda.cu:87-101 and
 *     src/ModelCuda.cpp:242-356 with host memory standing in for device memory,
 *     and k restates src/Model.cpp:44-54 (Model.cpp needs the CUDA/OptiX model).
 *   - Visibility (ref_vis_call) is a plain FP64 ray/triangle test over the
 *     target triangles with t in (0, tmax] that ignores triangles whose plane
 *     holds the ray origin.  Fixtures use scenes whose shadow verdicts are far
 *     from every tolerance, so any reasonable ray test gives the same answer.
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <iomanip>
#include <vector>
#include <cuda_runtime.h>
#include <thrust/complex.h>
#include "optix.h"

#define private public
#define protected public
#include "Facet.hpp"
#undef private
#undef protected
#include "ModelShared.h"

extern "C" {
globalParams params;
unsigned int ref_launch_x = 0;
void __raygen__rg();
}

/* The GL/CUDA base classes of Facet are not built here: their constructors and
 * the device allocation are empty stand-ins (memory stays on the host). */
FacetGl::FacetGl() {}
FacetGl::~FacetGl() {}
FacetCuda::FacetCuda() {}
FacetCuda::~FacetCuda() {}
void FacetCuda::AllocateCuda(float3 &, float3 &, float3 &, float3 &, float *) {}

namespace {

struct Tri { double v[3][3]; };

struct RObj {
    int type = 0;
    float delta = 0.0f;
    std::vector<Facet *> facets;
    std::vector<std::vector<dcomplex>> P, Pin, Pout;
    std::vector<dev_facet> dev;
    bool structMade = false;
};

struct RScene {
    std::vector<RObj *> obj[3];
    std::vector<float3> src, fp;
    std::vector<dcomplex> srcP, fpP;
    dcomplex k{0, 0};
    bool rendered = false;
    std::vector<Tri> tris;
};

RScene *g_scene = nullptr;

bool ray_tri(const Tri &t, const double o[3], const double d[3], double tmax)
{
    double e1[3], e2[3], n[3];
    for (int k = 0; k < 3; k++) { e1[k] = t.v[1][k] - t.v[0][k]; e2[k] = t.v[2][k] - t.v[0][k]; }
    n[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n[2] = e1[0] * e2[1] - e1[1] * e2[0];
    double L = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(L > 0)) return false;
    for (double &x : n) x /= L;
    double sc = 1.0;
    for (int k = 0; k < 3; k++) sc = std::fmax(sc, 1.0 + std::fabs(o[k]));
    double dist0 = n[0] * (o[0] - t.v[0][0]) + n[1] * (o[1] - t.v[0][1]) + n[2] * (o[2] - t.v[0][2]);
    if (std::fabs(dist0) <= 1e-4 * sc) return false; /* origin on this triangle's plane */
    double dn = n[0] * d[0] + n[1] * d[1] + n[2] * d[2];
    if (dn == 0.0) return false;
    double tt = -dist0 / dn;
    if (!(tt > 0.0) || tt > tmax) return false;
    double X[3] = {o[0] + d[0] * tt, o[1] + d[1] * tt, o[2] + d[2] * tt};
    for (int e = 0; e < 3; e++) {
        const double *p = t.v[e], *q = t.v[(e + 1) % 3];
        double ed[3] = {q[0] - p[0], q[1] - p[1], q[2] - p[2]};
        double m[3] = {n[1] * ed[2] - n[2] * ed[1], n[2] * ed[0] - n[0] * ed[2], n[0] * ed[1] - n[1] * ed[0]};
        double g = m[0] * (X[0] - p[0]) + m[1] * (X[1] - p[1]) + m[2] * (X[2] - p[2]);
        if (g < 0.0) return false;
    }
    return true;
}

/* FacetCuda::AllocateCuda (FacetCuda.cpp:8-62) with host buffers */
void make_cuda(RObj *o)
{
    size_t nf = o->facets.size();
    o->P.assign(nf, {});
    o->Pin.assign(nf, {});
    o->Pout.assign(nf, {});
    o->dev.assign(nf, dev_facet{});
    for (size_t i = 0; i < nf; i++) {
        Facet *f = o->facets[i];
        size_t n = (size_t)f->numXpnts * f->numYpnts;
        dev_facet &d = o->dev[i];
        d.normal = f->Normal;
        d.base_point = f->pointOnBase;
        d.xAxis = f->xAxis;
        d.yAxis = f->yAxis;
        d.frag_points = make_int3(f->numXpnts, f->numYpnts, f->numXpntsNegative);
        d.frag_area = f->fragArea;
        o->P[i].assign(n, dcomplex{0, 0});
        d.P = o->P[i].data();
        d.P_in = d.P_out = d.P;
        if (o->type == OBJECT_TYPE_TARGET) {
            o->Pin[i].assign(n, dcomplex{0, 0});
            o->Pout[i].assign(n, dcomplex{0, 0});
            d.P_in = o->Pin[i].data();
            d.P_out = o->Pout[i].data();
        }
    }
}

/* ObjectCuda::MakeOptixStructArray (ObjectCuda.cpp:33-52): the first call zeroes
 * P_out of target facets (FacetCuda::MakeOptixStruct, FacetCuda.cpp:114-122). */
dev_object struct_array(RObj *o)
{
    if (!o->structMade && !o->facets.empty()) {
        if (o->type == OBJECT_TYPE_TARGET)
            for (auto &v : o->Pout) std::fill(v.begin(), v.end(), dcomplex{0, 0});
        o->structMade = true;
    }
    dev_object d{};
    d.objectType = (ObjectType)o->type;
    d.numFacets = (int)o->facets.size();
    d.facets = o->dev.data();
    d.delta = o->delta;
    return d;
}

/* OptiX::DoProjection (OptiX.cpp:130-172): one raygen call per launch index */
void do_projection(const globalParams &gp)
{
    params = gp;
    int n = gp.srcObject.numFacets;
    if (gp.calcType == SOURCE_POINTS) n = gp.dstObject.numFacets;
    for (int i = 0; i < n; i++) {
        ref_launch_x = (unsigned)i;
        __raygen__rg();
    }
}

} // namespace

extern "C" {

int ref_vis_call(float ox, float oy, float oz, float dx, float dy, float dz, float tmin, float tmax)
{
    (void)tmin;
    if (!g_scene) return 0;
    double o[3] = {ox, oy, oz}, d[3] = {dx, dy, dz};
    for (const Tri &t : g_scene->tris)
        if (ray_tri(t, o, d, (double)tmax)) return 1;
    return 0;
}

void ref_reset(void)
{
    if (g_scene) {
        for (int t = 0; t < 3; t++)
            for (RObj *o : g_scene->obj[t]) {
                for (Facet *f : o->facets) delete f;
                delete o;
            }
        delete g_scene;
    }
    g_scene = new RScene();
}

int ref_add_object(const float *tri9, int ntri, int type, float delta)
{
    if (!g_scene) ref_reset();
    ObjectType ot = safeConvertToEnum(type);
    RObj *o = new RObj();
    o->type = ot;
    o->delta = delta;
    for (int i = 0; i < ntri; i++) {
        const float *t = tri9 + 9L * i;
        float3 a = {t[0], t[1], t[2]}, b = {t[3], t[4], t[5]}, c = {t[6], t[7], t[8]};
        o->facets.push_back(new Facet(a, b, c, ot, delta));
    }
    g_scene->obj[ot].push_back(o);
    return (int)g_scene->obj[ot].size() - 1;
}

void ref_add_sources(const float *xyz, int n)
{
    for (int i = 0; i < n; i++) {
        g_scene->src.push_back(make_float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]));
        g_scene->srcP.push_back(dcomplex{1.0, 0.0});
    }
}

void ref_add_field_points(const float *xyz, int n)
{
    for (int i = 0; i < n; i++) {
        g_scene->fp.push_back(make_float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]));
        g_scene->fpP.push_back(dcomplex{0.0, 0.0});
    }
}

/* Model::set_inital_conditions (Model.cpp:44-54) */
void ref_set_conditions(float cp, float f, float att, float density)
{
    (void)density;
    float omega = 2 * M_PI * f;
    float k = omega / cp;
    g_scene->k.r = (double)k;
    g_scene->k.i = (double)att;
}

/* Model::MakeFragments + the parts of Model::RenderCuda that set up buffers */
int ref_render(void)
{
    if (g_scene->rendered) return -1;
    for (int t : {0, 2})
        for (RObj *o : g_scene->obj[t]) {
            for (Facet *f : o->facets) f->MakeFragmentData();
            make_cuda(o);
        }
    g_scene->tris.clear();
    for (RObj *o : g_scene->obj[0])
        for (Facet *f : o->facets) {
            Tri t;
            float3 v[3] = {f->v1, f->v2, f->v3};
            for (int q = 0; q < 3; q++) { t.v[q][0] = v[q].x; t.v[q][1] = v[q].y; t.v[q][2] = v[q].z; }
            g_scene->tris.push_back(t);
        }
    g_scene->rendered = true;
    return 0;
}

/* ModelCuda::ProjectSrcPointsToObjects (ModelCuda.cpp:242-278) */
void ref_project_sources(int field_objects)
{
    globalParams gp = {};
    gp.calcType = SOURCE_POINTS;
    gp.k_wave = g_scene->k;
    gp.srcPoints.numPnts = (int)g_scene->src.size();
    gp.srcPoints.position = g_scene->src.data();
    gp.srcPoints.pressure = g_scene->srcP.data();
    for (RObj *o : g_scene->obj[0]) {
        gp.dstObject = struct_array(o);
        do_projection(gp);
    }
    if (field_objects)
        for (RObj *o : g_scene->obj[2]) {
            gp.dstObject = struct_array(o);
            do_projection(gp);
        }
}

/* ModelCuda::ProjectTargetToFieldObjects (ModelCuda.cpp:280-301) */
void ref_project_field_objects(void)
{
    globalParams gp = {};
    gp.calcType = FACET_NO_RESP;
    gp.k_wave = g_scene->k;
    for (RObj *t : g_scene->obj[0]) {
        gp.srcObject = struct_array(t);
        for (RObj *f : g_scene->obj[2]) {
            gp.dstObject = struct_array(f);
            do_projection(gp);
        }
    }
}

/* ModelCuda::ProjectTargetToFieldPoints (ModelCuda.cpp:302-321) */
void ref_project_field_points(void)
{
    globalParams gp = {};
    gp.calcType = FIELD_POINTS;
    gp.k_wave = g_scene->k;
    gp.dstPoints.numPnts = (int)g_scene->fp.size();
    gp.dstPoints.position = g_scene->fp.data();
    gp.dstPoints.pressure = g_scene->fpP.data();
    for (RObj *t : g_scene->obj[0]) {
        gp.srcObject = struct_array(t);
        do_projection(gp);
    }
}

/* ModelCuda::ProjectTargetToTargetObjects (ModelCuda.cpp:323-356) with
 * FacetCuda::PrimeReflections / SwapOutputToInputPressure (FacetCuda.cpp:124-137)
 * and AccumulatePressureKernel (FacetCuda.cu:87-101). */
void ref_project_bounces(int n)
{
    globalParams gp = {};
    gp.calcType = FACET_SELF;
    gp.k_wave = g_scene->k;
    for (RObj *o : g_scene->obj[0])
        for (size_t i = 0; i < o->facets.size(); i++) o->Pout[i] = o->P[i];
    for (int b = 0; b < n; b++) {
        for (RObj *o : g_scene->obj[0]) {
            gp.srcObject = struct_array(o);
            for (size_t i = 0; i < o->facets.size(); i++) {
                o->Pin[i] = o->Pout[i];
                std::fill(o->Pout[i].begin(), o->Pout[i].end(), dcomplex{0, 0});
            }
            gp.dstObject = gp.srcObject;
            do_projection(gp);
            for (size_t i = 0; i < o->facets.size(); i++)
                for (size_t c = 0; c < o->P[i].size(); c++) {
                    o->P[i][c].r = o->P[i][c].r + o->Pout[i][c].r;
                    o->P[i][c].i = o->P[i][c].i + o->Pout[i][c].i;
                }
        }
    }
}

long ref_object_ncells(int type, int idx)
{
    RObj *o = g_scene->obj[type][idx];
    long n = 0;
    for (Facet *f : o->facets) n += (long)f->numXpnts * f->numYpnts;
    return n;
}

/* P of every facet, facet-major, each facet row-major y*nx + x */
int ref_get_object_pressures(int type, int idx, double *out)
{
    RObj *o = g_scene->obj[type][idx];
    long k = 0;
    for (size_t i = 0; i < o->facets.size(); i++)
        for (const dcomplex &p : o->P[i]) { out[2 * k] = p.r; out[2 * k + 1] = p.i; k++; }
    return 0;
}

int ref_get_field_points(double *out)
{
    for (size_t j = 0; j < g_scene->fpP.size(); j++) {
        out[2 * j] = g_scene->fpP[j].r;
        out[2 * j + 1] = g_scene->fpP[j].i;
    }
    return (int)g_scene->fpP.size();
}

/* One triangle through the reference's Facet class: nx, ny, neg; 17 floats
 * normal(3) base(3) xAxis(3) yAxis(3) baseLen height baseNeg basePos area;
 * the area grid when cap allows. */
long ref_fragment_triangle(const float *tri9, float delta, int *ints, float *floats, float *areas, long cap)
{
    float3 a = {tri9[0], tri9[1], tri9[2]}, b = {tri9[3], tri9[4], tri9[5]}, c = {tri9[6], tri9[7], tri9[8]};
    Facet f(a, b, c, OBJECT_TYPE_TARGET, delta);
    f.MakeFragmentData();
    ints[0] = f.numXpnts; ints[1] = f.numYpnts; ints[2] = f.numXpntsNegative;
    float v[17] = {f.Normal.x, f.Normal.y, f.Normal.z, f.pointOnBase.x, f.pointOnBase.y, f.pointOnBase.z,
                   f.xAxis.x, f.xAxis.y, f.xAxis.z, f.yAxis.x, f.yAxis.y, f.yAxis.z,
                   f.BaseLength, f.Height, f.BaseLengthNeg, f.BaseLengthPos, f.Area};
    std::memcpy(floats, v, sizeof(v));
    long n = (long)f.numXpnts * f.numYpnts;
    if (areas && cap >= n) std::memcpy(areas, f.fragArea, sizeof(float) * n);
    return n;
}

} // extern "C"
