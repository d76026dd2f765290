/*
 * sonar_oracle.c -- CPU restatement of sonar-render's discrete Kirchhoff hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke
 * check in __graft_entry__ and bench.py's CPU-baseline / reference legs load it.
 * The product library (sonar-render_gb300/) never links, loads or calls it.
 *
 * Arithmetic model: exactly the reference's.  Geometry (facet frames, fragment
 * areas, fragment centroids, r, unit vectors, cosines) is FP32 with the same
 * operation order as the reference source (build with -ffp-contract=off so no
 * multiply-add is fused, matching the reference's x86-64 host build).  The
 * Green's-function terms and all accumulation are FP64, as the reference's
 * thrust::complex<double> code is.
 *
 * What each part restates (paths inside the sonar-render project):
 *   facet_init()            src/Facet.cpp:95-109 (normal) and :6-86 (frame)
 *   facet_fragment()        src/Facet.cpp:111-339 (clipped area grid)
 *   len_between() etc.      src/GeoMath.h:19-106
 *   orc_set_conditions()    src/Model.cpp:44-54 (k computed in FP32)
 *   hop_source_cell()       src/OptiX.cu:35-110   (source point -> fragment)
 *   hop_fieldpoint()        src/OptiX.cu:112-190  (fragment -> field point)
 *   hop_f2f_cell()          src/OptiX.cu:192-406  (FACET_SELF with reciprocity)
 *   hop_noresp_cell()       src/OptiX.cu:192-406  (FACET_NO_RESP, target -> field object)
 *   hop_resp_cell()         src/OptiX.cu:192-406, :427-429 (FACET_RESP, target -> other target)
 *   orc_project_*()         src/ModelCuda.cpp:242-356, src/FacetCuda.cpp:114-137,
 *                           src/FacetCuda.cu:87-101 (prime / swap / accumulate)
 *
 * Visibility.  The reference fires OptiX shadow rays (src/OptiX.cu:81-93,
 * 163-175, 321-333: tmin 0, tmax r - 1e-3, terminate on first hit) against a
 * triangle acceleration structure built over all TARGET triangles
 * (src/OptiX.cpp:264-350).  OptiX's intersection rounding is not documented,
 * so the visibility test is restated with explicit semantics (seg_occluded):
 *   - the segment runs from the ray origin o to the ray's destination point e;
 *     a triangle occludes when the segment strictly crosses its plane at a
 *     distance t <= tmax = (float)(r - 1e-3f) from o and the crossing point
 *     lies inside the triangle (edge tests >= 0);
 *   - a triangle whose plane passes within eps_plane of the ORIGIN never
 *     occludes (a ray leaving a surface is not shadowed by that surface; with
 *     tmin = 0 the reference's answer there is decided by rounding);
 *   - a verdict that could flip under perturbations of size tol (FP32-level
 *     errors) is classified "grazing"; the product must agree with this test
 *     on every non-grazing pair, and grazing pairs are counted.
 */
#define _GNU_SOURCE
#include <math.h>
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OBJ_TARGET 0
#define OBJ_SOURCE 1
#define OBJ_FIELD 2

typedef struct { float x, y, z; } f3;

/* ------------------------------------------------------------------------- */
/* GeoMath (src/GeoMath.h:19-106), FP32, same expression order.              */
/* ------------------------------------------------------------------------- */
static float len_between(f3 p1, f3 p2)
{
    float dx = p1.x - p2.x, dy = p1.y - p2.y, dz = p1.z - p2.z;
    return sqrtf(dx * dx + dy * dy + dz * dz);
}
static f3 vec_sc(f3 origin, f3 dest)
{
    f3 v = {dest.x - origin.x, dest.y - origin.y, dest.z - origin.z};
    return v;
}
static f3 unit_sc(f3 v)
{
    float L = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    f3 u = {v.x / L, v.y / L, v.z / L};
    return u;
}
static float dot_sc(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static float vlen(f3 v) { return sqrtf(v.x * v.x + v.y * v.y + v.z * v.z); }
static f3 cross_sc(f3 a, f3 b)
{
    f3 c = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return c;
}
/* GeoMath.h MakeVectorThroughPointPerpToVector */
static f3 perp_through(f3 vp, f3 vect, f3 pp, f3 *pol)
{
    f3 vpp = vec_sc(vp, pp);
    f3 u = unit_sc(vect);
    float pl = dot_sc(u, vpp);
    pol->x = vp.x + u.x * pl;
    pol->y = vp.y + u.y * pl;
    pol->z = vp.z + u.z * pl;
    return vec_sc(*pol, pp);
}

/* ------------------------------------------------------------------------- */
/* Facet frame and fragmentation.                                            */
/* ------------------------------------------------------------------------- */
typedef struct {
    f3 v1, v2, v3;
    f3 normal, xAxis, yAxis, base;
    float baseLen, height, baseNeg, basePos, area, delta;
    int nx, ny, neg;
    long cell0; /* first cell of this facet in the object's cell arrays */
} facet_t;

/* src/Facet.cpp:95-109 and :6-86 */
static void facet_init(facet_t *f, f3 v1, f3 v2, f3 v3, float delta)
{
    memset(f, 0, sizeof(*f));
    f->v1 = v1; f->v2 = v2; f->v3 = v3; f->delta = delta;
    f3 a = vec_sc(v2, v1), b = vec_sc(v3, v1);
    f->normal = unit_sc(cross_sc(a, b));

    float L[3];
    L[0] = len_between(v1, v2);
    L[1] = len_between(v1, v3);
    L[2] = len_between(v2, v3);
    int mi = 0;
    float mv = L[0];
    for (int i = 1; i < 3; i++)
        if (L[i] > mv) { mv = L[i]; mi = i; }
    f3 vx, vy;
    switch (mi) {
    case 0:
        vx = vec_sc(v1, v2);
        vy = perp_through(v1, vx, v3, &f->base);
        f->baseLen = L[0];
        f->height = vlen(vy);
        f->baseNeg = len_between(v1, f->base);
        f->basePos = len_between(f->base, v2);
        break;
    case 1:
        vx = vec_sc(v1, v3);
        vy = perp_through(v1, vx, v2, &f->base);
        f->baseLen = L[1];
        f->height = vlen(vy);
        f->baseNeg = len_between(v1, f->base);
        f->basePos = len_between(f->base, v3);
        break;
    default:
        vx = vec_sc(v2, v3);
        vy = perp_through(v2, vx, v1, &f->base);
        f->baseLen = L[2];
        f->height = vlen(vy);
        f->baseNeg = len_between(v2, f->base);
        f->basePos = len_between(f->base, v3);
        break;
    }
    f->xAxis = unit_sc(vx);
    f->yAxis = unit_sc(vy);
    f->area = (f->baseLen * f->height) / 2.0f;
    f->neg = (int)ceilf(fabsf(f->baseNeg) / delta);
    f->nx = f->neg + (int)ceilf(fabsf(f->basePos) / delta);
    f->ny = (int)ceilf(f->height / delta);
}

/* src/Facet.cpp:111-339.  area must hold nx*ny floats (row-major y*nx + x). */
static void facet_fragment(const facet_t *f, float *area)
{
    const int nx = f->nx, ny = f->ny, neg = f->neg;
    const float delta = f->delta, H = f->height;
    float *vX = (float *)malloc(sizeof(float) * (nx > 0 ? nx : 1));
    float *vY = (float *)malloc(sizeof(float) * (ny > 0 ? ny : 1));
    unsigned char *yxL = (unsigned char *)malloc(ny + 1);
    unsigned char *yxR = (unsigned char *)malloc(ny + 1);
    for (int i = 0; i < nx; i++) {
        if (i < neg)
            vX[i] = ((float)(-neg + i) * delta) + delta / 2;
        else
            vX[i] = ((float)(i - neg) * delta) + delta / 2;
    }
    for (int i = 0; i < ny; i++) vY[i] = ((float)i * delta) + delta / 2;
    for (long i = 0; i < (long)nx * ny; i++) area[i] = 0.0f;

    const float m1 = H / (-f->basePos);
    const float m2 = H / (f->baseNeg);

    for (int i = 0; i < nx; i++) {
        const float x = vX[i];
        const float xL = x - (delta / 2);
        const float xR = x + (delta / 2);
        if (x > 0) {
            const float yL = m1 * xL + H;
            const float yR = m1 * xR + H;
            for (int j = 0; j < ny + 1; j++) {
                yxL[j] = delta * (float)j <= yL;
                yxR[j] = delta * (float)j <= yR;
            }
            for (int j = 0; j < ny; j++) {
                const float yB = delta * (float)j;
                const float yT = delta * (float)(j + 1);
                float *A = &area[(long)j * nx + i];
                if (!yxL[j] && !yxR[j] && !yxL[j + 1] && !yxR[j + 1]) break;
                if (yxL[j] && yxR[j] && yxL[j + 1] && yxR[j + 1]) { *A = delta * delta; continue; }
                if (yxL[j] && yxR[j] && yxL[j + 1] && !yxR[j + 1]) {
                    /* upper right out */
                    float xit = (yT - H) / m1;
                    float pixel_area = delta * delta;
                    float sub = (yT - yR) * (xR - xit) / 2;
                    *A = pixel_area - sub;
                    continue;
                }
                if (yxL[j] && yxR[j] && !yxL[j + 1] && !yxR[j + 1]) {
                    /* upper right and upper left out */
                    *A = ((yL - yR) * delta / 2) + (yR - yB) * delta;
                    continue;
                }
                if (yxL[j] && !yxR[j] && yxL[j + 1] && !yxR[j + 1]) {
                    /* upper right and lower right out */
                    float xit = ((yT - H) / m1) - xL;
                    float xib = ((yB - H) / m1) - xL;
                    *A = (xit * delta) + (xib - xit) * delta / 2;
                    continue;
                }
                if (yxL[j] && !yxR[j] && !yxL[j + 1] && !yxR[j + 1]) {
                    /* only lower left in */
                    *A = (yL - yB) * (((yB - H) / m1) - xL) / 2;
                    continue;
                }
            }
        } else {
            const float yL = m2 * xL + H;
            const float yR = m2 * xR + H;
            for (int j = 0; j < ny + 1; j++) {
                yxL[j] = delta * (float)j <= yL;
                yxR[j] = delta * (float)j <= yR;
            }
            for (int j = 0; j < ny; j++) {
                float *A = &area[(long)j * nx + i];
                if (!yxL[j] && !yxR[j] && !yxL[j + 1] && !yxR[j + 1]) break;
                if (yxL[j] && yxR[j] && yxL[j + 1] && yxR[j + 1]) { *A = delta * delta; continue; }
                if (yxL[j] && yxR[j] && !yxL[j + 1] && yxR[j + 1]) {
                    /* upper left out */
                    *A = delta * delta - (vY[j] + delta / 2 - yL) * (-(xL - ((vY[j] + (delta / 2) - H) / m2)) / 2);
                    continue;
                }
                if (yxL[j] && yxR[j] && !yxL[j + 1] && !yxR[j + 1]) {
                    /* upper right and upper left out */
                    *A = (yR - yL) * delta / 2 + ((yL - (vY[j] - delta / 2)) * delta);
                    continue;
                }
                if (!yxL[j] && yxR[j] && !yxL[j + 1] && yxR[j + 1]) {
                    /* upper left and lower left out */
                    *A = -((vY[j] - (delta / 2) - H) / m2 - (vY[j] + (delta / 2) - H) / m2) * delta / 2 -
                         (((vY[j] + (delta / 2) - H) / m2) - xR) * delta;
                    continue;
                }
                if (!yxL[j] && yxR[j] && !yxL[j + 1] && !yxR[j + 1]) {
                    /* only right in */
                    *A = (yR - (vY[j] - delta / 2)) * (-((((vY[j] - delta / 2) - H) / m2) - xR)) / 2;
                    continue;
                }
            }
        }
    }
    free(vX); free(vY); free(yxL); free(yxR);
}

/* Fragment centroid as the kernels compute it (src/OptiX.cu:51-57 with the
 * +delta/2 x shift for the source hop; :129-135, :210-216, :273-279 without). */
static f3 frag_pos(const facet_t *f, int x, int y, int src_hop)
{
    const float d = f->delta;
    float xoff = d * (float)(x - f->neg);
    if (src_hop) xoff = xoff + d / 2;
    const float yoff = d * (float)y + d / 2;
    f3 xa = {f->xAxis.x * xoff, f->xAxis.y * xoff, f->xAxis.z * xoff};
    f3 ya = {f->yAxis.x * yoff, f->yAxis.y * yoff, f->yAxis.z * yoff};
    f3 p = {(f->base.x + xa.x) + ya.x, (f->base.y + xa.y) + ya.y, (f->base.z + xa.z) + ya.z};
    return p;
}

/* ------------------------------------------------------------------------- */
/* Scene                                                                      */
/* ------------------------------------------------------------------------- */
typedef struct {
    int type;
    float delta;
    int nf;
    facet_t *f;
    long ncells;
    float *area;      /* per cell */
    int *cell_facet;  /* per cell */
    double *P, *Pin, *Pout; /* complex, 2 doubles per cell */
    long nact;        /* cells with area > 1e-6f */
    long *act;        /* active cell indices, ascending */
} object_t;

typedef struct {
    double n[3], c, m[3][3], cm[3];
    double lo[3], hi[3];
    int ok;
} otri_t;

typedef struct {
    double lo[3], hi[3];
    int left, right; /* children, or -1 */
    int t0, tn;      /* leaf triangle range in tri_order */
} bnode_t;

typedef struct {
    object_t *obj[3][64];
    int nobj[3];
    f3 *src; int nsrc; double *srcP;
    f3 *fp; int nfp; double *fpP;
    float cp, freq, att, density;
    double kr, ki;
    int rendered;
    /* 0: the reference's FP32 geometry (r = sqrtf of an FP32 dot); 1: the
     * source hop and the field-point readout take the distance and cosines
     * in FP64 from the same FP32 positions (the accuracy yardstick of the
     * library's centroid-relative geometry; the gates stay FP32) */
    int exact_geom;
    /* occluders */
    otri_t *tri; int ntri;
    bnode_t *node; int nnode;
    int *tri_order;
    /* counters (visibility evaluations in the last hop) */
    long long c_pairs, c_graze, c_selfplane;
} scene_t;

void *orc_new(void)
{
    scene_t *s = (scene_t *)calloc(1, sizeof(scene_t));
    return s;
}

static void obj_free(object_t *o)
{
    if (!o) return;
    free(o->f); free(o->area); free(o->cell_facet); free(o->P); free(o->Pin); free(o->Pout); free(o->act);
    free(o);
}

void orc_free(void *h)
{
    scene_t *s = (scene_t *)h;
    if (!s) return;
    for (int t = 0; t < 3; t++)
        for (int i = 0; i < s->nobj[t]; i++) obj_free(s->obj[t][i]);
    free(s->src); free(s->srcP); free(s->fp); free(s->fpP);
    free(s->tri); free(s->node); free(s->tri_order);
    free(s);
}

/* python_interface.cpp:26-41 (load_geometry): 9 floats per triangle. */
int orc_add_object(void *h, const float *tri9, int ntri, int type, float delta)
{
    scene_t *s = (scene_t *)h;
    if (type < 0 || type > 2 || ntri < 0 || s->nobj[type] >= 64) return -1;
    object_t *o = (object_t *)calloc(1, sizeof(object_t));
    o->type = type; o->delta = delta; o->nf = ntri;
    o->f = (facet_t *)calloc(ntri > 0 ? ntri : 1, sizeof(facet_t));
    for (int i = 0; i < ntri; i++) {
        const float *t = tri9 + 9L * i;
        f3 a = {t[0], t[1], t[2]}, b = {t[3], t[4], t[5]}, c = {t[6], t[7], t[8]};
        facet_init(&o->f[i], a, b, c, delta);
    }
    s->obj[type][s->nobj[type]] = o;
    return s->nobj[type]++;
}

int orc_add_sources(void *h, const float *xyz, int n)
{
    scene_t *s = (scene_t *)h;
    s->src = (f3 *)realloc(s->src, sizeof(f3) * (s->nsrc + n + 1));
    s->srcP = (double *)realloc(s->srcP, sizeof(double) * 2 * (s->nsrc + n + 1));
    for (int i = 0; i < n; i++) {
        f3 p = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
        s->src[s->nsrc + i] = p;
        s->srcP[2 * (s->nsrc + i)] = 1.0; /* Model.cpp:18 */
        s->srcP[2 * (s->nsrc + i) + 1] = 0.0;
    }
    s->nsrc += n;
    return 0;
}

int orc_add_field_points(void *h, const float *xyz, int n)
{
    scene_t *s = (scene_t *)h;
    s->fp = (f3 *)realloc(s->fp, sizeof(f3) * (s->nfp + n + 1));
    s->fpP = (double *)realloc(s->fpP, sizeof(double) * 2 * (s->nfp + n + 1));
    for (int i = 0; i < n; i++) {
        f3 p = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
        s->fp[s->nfp + i] = p;
        s->fpP[2 * (s->nfp + i)] = 0.0;
        s->fpP[2 * (s->nfp + i) + 1] = 0.0;
    }
    s->nfp += n;
    return 0;
}

/* src/Model.cpp:44-54: omega and k are FP32 members; k_wave = ((double)k, att). */
void orc_set_exact_geometry(void *h, int on)
{
    ((scene_t *)h)->exact_geom = on != 0;
}

void orc_set_conditions(void *h, float cp, float f, float att, float density)
{
    scene_t *s = (scene_t *)h;
    s->cp = cp; s->freq = f; s->att = att; s->density = density;
    float omega = (float)(2 * M_PI * (double)f);
    float k = omega / cp;
    s->kr = (double)k;
    s->ki = (double)att;
}

double orc_get_k(void *h, int imag)
{
    scene_t *s = (scene_t *)h;
    return imag ? s->ki : s->kr;
}

/* ---- occluder set ------------------------------------------------------- */
static void tri_prep(otri_t *t, f3 a, f3 b, f3 c)
{
    double v[3][3] = {{a.x, a.y, a.z}, {b.x, b.y, b.z}, {c.x, c.y, c.z}};
    double e1[3], e2[3], n[3];
    for (int k = 0; k < 3; k++) { e1[k] = v[1][k] - v[0][k]; e2[k] = v[2][k] - v[0][k]; }
    n[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n[2] = e1[0] * e2[1] - e1[1] * e2[0];
    double L = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    t->ok = L > 0.0;
    if (!t->ok) return;
    for (int k = 0; k < 3; k++) t->n[k] = n[k] / L;
    t->c = t->n[0] * v[0][0] + t->n[1] * v[0][1] + t->n[2] * v[0][2];
    for (int e = 0; e < 3; e++) {
        const double *p = v[e], *q = v[(e + 1) % 3];
        double d[3] = {q[0] - p[0], q[1] - p[1], q[2] - p[2]};
        double m[3] = {t->n[1] * d[2] - t->n[2] * d[1], t->n[2] * d[0] - t->n[0] * d[2], t->n[0] * d[1] - t->n[1] * d[0]};
        double ml = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
        if (!(ml > 0.0)) { t->ok = 0; return; }
        for (int k = 0; k < 3; k++) t->m[e][k] = m[k] / ml;
        t->cm[e] = t->m[e][0] * p[0] + t->m[e][1] * p[1] + t->m[e][2] * p[2];
    }
    for (int k = 0; k < 3; k++) {
        t->lo[k] = fmin(v[0][k], fmin(v[1][k], v[2][k]));
        t->hi[k] = fmax(v[0][k], fmax(v[1][k], v[2][k]));
    }
}

static double g_pad = 1e-3;

static int bvh_build_rec(scene_t *s, int t0, int tn)
{
    int id = s->nnode++;
    bnode_t *nd = &s->node[id];
    for (int k = 0; k < 3; k++) { nd->lo[k] = 1e300; nd->hi[k] = -1e300; }
    for (int i = t0; i < t0 + tn; i++) {
        const otri_t *t = &s->tri[s->tri_order[i]];
        for (int k = 0; k < 3; k++) {
            nd->lo[k] = fmin(nd->lo[k], t->lo[k] - g_pad);
            nd->hi[k] = fmax(nd->hi[k], t->hi[k] + g_pad);
        }
    }
    nd->left = nd->right = -1;
    nd->t0 = t0; nd->tn = tn;
    if (tn <= 4) return id;
    /* median split on the longest axis of centroid bounds */
    double clo[3] = {1e300, 1e300, 1e300}, chi[3] = {-1e300, -1e300, -1e300};
    for (int i = t0; i < t0 + tn; i++) {
        const otri_t *t = &s->tri[s->tri_order[i]];
        for (int k = 0; k < 3; k++) {
            double c = 0.5 * (t->lo[k] + t->hi[k]);
            clo[k] = fmin(clo[k], c); chi[k] = fmax(chi[k], c);
        }
    }
    int ax = 0;
    for (int k = 1; k < 3; k++)
        if (chi[k] - clo[k] > chi[ax] - clo[ax]) ax = k;
    /* insertion-free selection: simple sort of the range by centroid */
    for (int i = t0 + 1; i < t0 + tn; i++) {
        int key = s->tri_order[i];
        double kv = s->tri[key].lo[ax] + s->tri[key].hi[ax];
        int j = i - 1;
        while (j >= t0 && s->tri[s->tri_order[j]].lo[ax] + s->tri[s->tri_order[j]].hi[ax] > kv) {
            s->tri_order[j + 1] = s->tri_order[j];
            j--;
        }
        s->tri_order[j + 1] = key;
    }
    int half = tn / 2;
    int l = bvh_build_rec(s, t0, half);
    int r = bvh_build_rec(s, t0 + half, tn - half);
    s->node[id].left = l;
    s->node[id].right = r;
    return id;
}

static void build_occluders(scene_t *s)
{
    free(s->tri); free(s->node); free(s->tri_order);
    int n = 0;
    for (int i = 0; i < s->nobj[OBJ_TARGET]; i++) n += s->obj[OBJ_TARGET][i]->nf;
    s->ntri = n;
    s->tri = (otri_t *)calloc(n > 0 ? n : 1, sizeof(otri_t));
    s->tri_order = (int *)calloc(n > 0 ? n : 1, sizeof(int));
    s->node = (bnode_t *)calloc(2 * (n > 0 ? n : 1) + 2, sizeof(bnode_t));
    s->nnode = 0;
    double maxc = 0.0;
    int k = 0;
    for (int i = 0; i < s->nobj[OBJ_TARGET]; i++) {
        object_t *o = s->obj[OBJ_TARGET][i];
        for (int j = 0; j < o->nf; j++) {
            tri_prep(&s->tri[k], o->f[j].v1, o->f[j].v2, o->f[j].v3);
            for (int q = 0; q < 3; q++) {
                maxc = fmax(maxc, fabs(s->tri[k].lo[q]));
                maxc = fmax(maxc, fabs(s->tri[k].hi[q]));
            }
            s->tri_order[k] = k;
            k++;
        }
    }
    for (int i = 0; i < s->nsrc; i++) maxc = fmax(maxc, fmax(fabs(s->src[i].x), fmax(fabs(s->src[i].y), fabs(s->src[i].z))));
    for (int i = 0; i < s->nfp; i++) maxc = fmax(maxc, fmax(fabs(s->fp[i].x), fmax(fabs(s->fp[i].y), fabs(s->fp[i].z))));
    g_pad = 1e-3 * (1.0 + maxc);
    if (n > 0) bvh_build_rec(s, 0, n);
}

/* Tolerances of the visibility classification; see the header comment. */
/* The tolerances bound the error of an FP32 evaluation of the same quantities
 * at coordinate scale sc: a plane distance n.x - c from FP32 n, c and x has an
 * error of a few units in the last place of sc (~2e-7 sc); the crossing
 * distance and the edge distances of the crossing point add one rounding of
 * the segment parameter. */
#define VIS_TOL_D_REL 4e-7   /* plane distances */
#define VIS_TOL_T_REL 1e-6   /* crossing distance vs tmax */
#define VIS_TOL_E_REL 1e-6   /* crossing point vs triangle edges */
#define VIS_EPS_PLANE_REL 1e-4 /* origin-plane exclusion */

static int seg_box(const double o[3], const double d[3], const double lo[3], const double hi[3])
{
    double t0 = 0.0, t1 = 1.0;
    for (int k = 0; k < 3; k++) {
        if (d[k] == 0.0) {
            if (o[k] < lo[k] || o[k] > hi[k]) return 0;
        } else {
            double a = (lo[k] - o[k]) / d[k], b = (hi[k] - o[k]) / d[k];
            if (a > b) { double t = a; a = b; b = t; }
            if (a > t0) t0 = a;
            if (b < t1) t1 = b;
            if (t0 > t1) return 0;
        }
    }
    return 1;
}

/* Verdict of one triangle for the segment o -> e.  Returns the nominal verdict
 * (1 = occludes); *robust = 0 when a perturbation of the plane distances by
 * tol_d, of the crossing distance by tol_t or of the edge distances by tol_e
 * (FP32-level errors of a single-precision evaluation) could flip it. */
static int tri_verdict(const otri_t *t, const double o[3], const double e[3], double r, double tmax,
                       double tol_d, double tol_t, double tol_e, double eps_plane, int *robust,
                       int *selfplane)
{
    const double d0 = t->n[0] * o[0] + t->n[1] * o[1] + t->n[2] * o[2] - t->c;
    const double d1 = t->n[0] * e[0] + t->n[1] * e[1] + t->n[2] * e[2] - t->c;
    const double ad0 = fabs(d0), ad1 = fabs(d1);
    const int excl = ad0 <= eps_plane;
    const int excl_band = fabs(ad0 - eps_plane) < tol_d;
    if (excl) *selfplane = 1;

    /* verdict without the origin-plane exclusion */
    const int cross = (d0 > 0.0 && d1 < 0.0) || (d0 < 0.0 && d1 > 0.0);
    const int near = (ad0 < tol_d) || (ad1 < tol_d);
    int hit = 0, rob = 1;
    if (cross || near) {
        const double den = ad0 + ad1;
        const double sp = den > 0.0 ? ad0 / den : 0.0;
        const double tc = r * sp;
        /* bounds of the crossing distance t = r a0 / (a0 + a1) when |d0|, |d1|
         * move by tol_d (t grows with a0 and shrinks with a1) */
        const double t_lo = (ad0 > tol_d) ? r * (ad0 - tol_d) / den : 0.0;
        const double a1_lo = ad1 > tol_d ? ad1 - tol_d : 0.0;
        const double t_hi = r * (ad0 + tol_d) / (ad0 + tol_d + a1_lo);
        double X[3], gmin = 1e300;
        for (int k = 0; k < 3; k++) X[k] = o[k] + (e[k] - o[k]) * sp;
        for (int q = 0; q < 3; q++) {
            const double g = t->m[q][0] * X[0] + t->m[q][1] * X[1] + t->m[q][2] * X[2] - t->cm[q];
            if (g < gmin) gmin = g;
        }
        hit = cross && tc <= tmax && gmin >= 0.0;
        if (gmin < -tol_e || t_lo > tmax + tol_t)
            rob = 1; /* robust miss; the nominal verdict is a miss as well */
        else if (cross && !near && t_hi < tmax - tol_t && gmin > tol_e)
            rob = 1; /* robust hit */
        else
            rob = 0;
    }
    if (excl) {
        /* excluded: the verdict is "no hit"; ambiguous only inside the exclusion
         * band when the un-excluded verdict could be a hit */
        *robust = !(excl_band && (hit || !rob));
        return 0;
    }
    if (excl_band && (hit || !rob)) rob = 0;
    *robust = rob;
    return hit;
}

/* Occlusion of the segment o -> e (see header).  r is the reference's FP32
 * distance, tmax = (float)(r - 1e-3f).  Returns 1 when occluded; *graze = 1 when
 * the verdict is not robust. */
static int seg_occluded(const scene_t *s, const double o[3], const double e[3], double tmax, int *graze,
                        int *selfplane)
{
    *graze = 0;
    *selfplane = 0;
    if (s->ntri == 0) return 0;
    double sc = 1.0;
    for (int k = 0; k < 3; k++) { sc = fmax(sc, 1.0 + fabs(o[k])); sc = fmax(sc, 1.0 + fabs(e[k])); }
    const double tol_d = VIS_TOL_D_REL * sc, tol_t = VIS_TOL_T_REL * sc, tol_e = VIS_TOL_E_REL * sc;
    const double eps_plane = VIS_EPS_PLANE_REL * sc;
    double d[3] = {e[0] - o[0], e[1] - o[1], e[2] - o[2]};
    const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    int any_hit = 0, robust_hit = 0, ambiguous = 0;
    int stack[256], sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const bnode_t *nd = &s->node[stack[--sp]];
        if (!seg_box(o, d, nd->lo, nd->hi)) continue;
        if (nd->left < 0) {
            for (int i = nd->t0; i < nd->t0 + nd->tn; i++) {
                const otri_t *t = &s->tri[s->tri_order[i]];
                if (!t->ok) continue;
                int rob = 1, spf = 0;
                int h = tri_verdict(t, o, e, r, tmax, tol_d, tol_t, tol_e, eps_plane, &rob, &spf);
                if (spf) *selfplane = 1;
                if (h) any_hit = 1;
                if (h && rob) robust_hit = 1;
                if (!rob) ambiguous = 1;
            }
        } else {
            if (sp < 254) { stack[sp++] = nd->left; stack[sp++] = nd->right; }
        }
    }
    *graze = (!robust_hit && ambiguous);
    return any_hit;
}

/* ---- render (python_interface.cpp:61-65 -> Model::MakeFragments/RenderCuda) */
static void obj_fragment(object_t *o)
{
    long nc = 0;
    for (int i = 0; i < o->nf; i++) { o->f[i].cell0 = nc; nc += (long)o->f[i].nx * o->f[i].ny; }
    o->ncells = nc;
    o->area = (float *)calloc(nc > 0 ? nc : 1, sizeof(float));
    o->cell_facet = (int *)calloc(nc > 0 ? nc : 1, sizeof(int));
    o->P = (double *)calloc(2 * (nc > 0 ? nc : 1), sizeof(double));
    o->Pin = (double *)calloc(2 * (nc > 0 ? nc : 1), sizeof(double));
    o->Pout = (double *)calloc(2 * (nc > 0 ? nc : 1), sizeof(double));
    for (int i = 0; i < o->nf; i++) {
        facet_fragment(&o->f[i], o->area + o->f[i].cell0);
        for (long c = 0; c < (long)o->f[i].nx * o->f[i].ny; c++) o->cell_facet[o->f[i].cell0 + c] = i;
    }
    o->nact = 0;
    for (long c = 0; c < nc; c++) if (o->area[c] > 1e-6f) o->nact++;
    o->act = (long *)calloc(o->nact > 0 ? o->nact : 1, sizeof(long));
    long k = 0;
    for (long c = 0; c < nc; c++) if (o->area[c] > 1e-6f) o->act[k++] = c;
}

int orc_render(void *h)
{
    scene_t *s = (scene_t *)h;
    if (s->rendered) return -1;
    for (int i = 0; i < s->nobj[OBJ_TARGET]; i++) obj_fragment(s->obj[OBJ_TARGET][i]);
    for (int i = 0; i < s->nobj[OBJ_FIELD]; i++) obj_fragment(s->obj[OBJ_FIELD][i]);
    /* piston source objects: fragmented like the others, unit surface pressure */
    for (int i = 0; i < s->nobj[OBJ_SOURCE]; i++) {
        object_t *o = s->obj[OBJ_SOURCE][i];
        obj_fragment(o);
        for (long c = 0; c < o->ncells; c++) {
            o->P[2 * c] = o->Pin[2 * c] = 1.0;
            o->P[2 * c + 1] = o->Pin[2 * c + 1] = 0.0;
        }
    }
    build_occluders(s);
    s->rendered = 1;
    return 0;
}

/* cell index -> (facet, x, y) */
static void cell_xy(const object_t *o, long cell, int *fi, int *x, int *y)
{
    int f = o->cell_facet[cell];
    long c = cell - o->f[f].cell0;
    *fi = f;
    *y = (int)(c / o->f[f].nx);
    *x = (int)(c % o->f[f].nx);
}

static void to_d3(f3 p, double out[3]) { out[0] = p.x; out[1] = p.y; out[2] = p.z; }

/* Green's function of src/OptiX.cu:182 / :350 with r in FP32:
 *   -exp(i k r)/(4 pi) * (i k / r) + 1/(r*r)   (the last term FP32) */
static void green(const scene_t *s, float r, double *gr, double *gi)
{
    const double rd = (double)r;
    const double ea = exp(-s->ki * rd);
    const double er = ea * cos(s->kr * rd), ei = ea * sin(s->kr * rd);
    const double a_r = -er / (4 * M_PI), a_i = -ei / (4 * M_PI);
    const double b_r = (-s->ki) / rd, b_i = s->kr / rd; /* (i k)/r */
    *gr = a_r * b_r - a_i * b_i + (double)(1.0f / (r * r));
    *gi = a_r * b_i + a_i * b_r;
}

/* G at an FP64 distance (exact-geometry mode) */
static void green_d(const scene_t *s, double rd, double *gr, double *gi)
{
    const double ea = exp(-s->ki * rd);
    const double er = ea * cos(s->kr * rd), ei = ea * sin(s->kr * rd);
    const double a_r = -er / (4 * M_PI), a_i = -ei / (4 * M_PI);
    const double b_r = (-s->ki) / rd, b_i = s->kr / rd;
    *gr = a_r * b_r - a_i * b_i + 1.0 / (rd * rd);
    *gi = a_r * b_i + a_i * b_r;
}

/* FP64 distance and unit vector of b - a from FP32 points */
static double dist_d(f3 a, f3 b, double *u)
{
    const double vx = (double)b.x - (double)a.x, vy = (double)b.y - (double)a.y, vz = (double)b.z - (double)a.z;
    const double r = sqrt(vx * vx + vy * vy + vz * vz);
    u[0] = vx / r; u[1] = vy / r; u[2] = vz / r;
    return r;
}

/* ---- hop a4: src/OptiX.cu:35-110 ---------------------------------------- */
static void hop_source_cell(scene_t *s, const object_t *B, long cell, double *acc, uint8_t *mask_row,
                            long long *cnt)
{
    int fi, x, y;
    cell_xy(B, cell, &fi, &x, &y);
    const facet_t *F = &B->f[fi];
    f3 pj = frag_pos(F, x, y, 1);
    double ar = 0.0, ai = 0.0;
    for (int i = 0; i < s->nsrc; i++) {
        f3 pi = s->src[i];
        f3 v = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
        float r = sqrtf(dot_sc(v, v));
        float inv = 1.0f / r;
        f3 uv = {v.x * inv, v.y * inv, v.z * inv};
        f3 nuv = {-uv.x, -uv.y, -uv.z};
        float ci = dot_sc(nuv, F->normal);
        if (B->type == OBJ_FIELD) ci = 1;
        uint8_t m = 0;
        if (!(ci < 1e-6f)) {
            double o[3], e[3];
            to_d3(pi, o); to_d3(pj, e);
            int graze, spf;
            int hit = seg_occluded(s, o, e, (double)(r - 1e-3f), &graze, &spf);
            if (graze) { m |= 2; cnt[1]++; }
            if (spf) cnt[2]++;
            if (!hit) {
                m |= 1;
                double rd = (double)r, cid = (double)ci;
                if (s->exact_geom) {
                    double u[3];
                    rd = dist_d(pi, pj, u);
                    if (B->type != OBJ_FIELD)
                        cid = -(u[0] * F->normal.x + u[1] * F->normal.y + u[2] * F->normal.z);
                }
                const double ea = exp(-s->ki * rd);
                const double er = ea * cos(s->kr * rd), ei = ea * sin(s->kr * rd);
                const double Pr = s->srcP[2 * i], Pi = s->srcP[2 * i + 1];
                const double tr = Pr * er - Pi * ei, ti = Pr * ei + Pi * er;
                ar += (cid * tr) / rd;
                ai += (cid * ti) / rd;
            }
        }
        cnt[0]++;
        if (mask_row) mask_row[i] = m;
    }
    acc[0] = ar; acc[1] = ai;
}

/* ---- hop a5: src/OptiX.cu:112-190 --------------------------------------- */
static void hop_fieldpoint(scene_t *s, const object_t *A, int j, double *acc, uint8_t *mask_row, long long *cnt)
{
    f3 pj = s->fp[j];
    double ar = 0.0, ai = 0.0;
    for (long q = 0; q < A->nact; q++) {
        long cell = A->act[q];
        int fi, x, y;
        cell_xy(A, cell, &fi, &x, &y);
        const facet_t *F = &A->f[fi];
        f3 pi = frag_pos(F, x, y, 0);
        const float Ai = A->area[cell];
        f3 v = {pi.x - pj.x, pi.y - pj.y, pi.z - pj.z};
        float r = sqrtf(dot_sc(v, v));
        float inv = 1.0f / r;
        f3 uv = {v.x * inv, v.y * inv, v.z * inv};
        f3 nuv = {-uv.x, -uv.y, -uv.z};
        float cs = dot_sc(nuv, F->normal);
        uint8_t m = 0;
        if (!(cs < 1e-6f)) {
            double o[3], e[3];
            to_d3(pj, o); to_d3(pi, e);
            int graze, spf;
            int hit = seg_occluded(s, o, e, (double)(r - 1e-3f), &graze, &spf);
            if (graze) { m |= 2; cnt[1]++; }
            if (spf) cnt[2]++;
            if (!hit) {
                m |= 1;
                double gr, gi, w;
                if (s->exact_geom) {
                    double u[3];
                    const double rd = dist_d(pj, pi, u);  /* u: field point -> fragment */
                    green_d(s, rd, &gr, &gi);
                    w = (double)Ai * -(u[0] * F->normal.x + u[1] * F->normal.y + u[2] * F->normal.z);
                } else {
                    green(s, r, &gr, &gi);
                    w = (double)(Ai * cs);
                }
                const double pr = w * A->P[2 * cell], pim = w * A->P[2 * cell + 1];
                ar += pr * gr - pim * gi;
                ai += pr * gi + pim * gr;
            }
        }
        cnt[0]++;
        if (mask_row) mask_row[q] = m;
    }
    acc[0] = ar; acc[1] = ai;
}

/* G of src/OptiX.cu:340-352: regularised below r_min = delta_src, damped by 0.9 */
static void green_f2f(const scene_t *s, float r, float rmin, double *gr, double *gi)
{
    if (r < rmin) {
        *gr = (0.0 * s->kr - 1.0 * s->ki) / (4.0 * M_PI);
        *gi = (0.0 * s->ki + 1.0 * s->kr) / (4.0 * M_PI);
    } else {
        green(s, r, gr, gi);
    }
    *gr *= 0.9;
    *gi *= 0.9;
}

/* ---- hop a6, FACET_SELF: src/OptiX.cu:192-406 with useReciprocity, isSelf.
 * Destination-owned restatement: cell j of facet b receives
 *   - the forward term from every active cell i of a facet a < b, traced i -> j,
 *     skipped when Pin[i] == 0 (OptiX.cu:241-245);
 *   - the reciprocal term from every active cell i of a facet a > b, computed in
 *     the pair's enumeration order (A = b holding j, B = a holding i), traced
 *     j -> i, and dropped entirely when Pin[j] == 0 (the zero-input skip of
 *     the A side also kills the reciprocal write, OptiX.cu:241-245, :367-390). */
static void hop_f2f_cell(scene_t *s, const object_t *O, long q_j, const double *Pin, double *acc,
                         uint8_t *mask_row, long long *cnt)
{
    const long cj = O->act[q_j];
    int fb, xj, yj;
    cell_xy(O, cj, &fb, &xj, &yj);
    const facet_t *Fb = &O->f[fb];
    const f3 pj = frag_pos(Fb, xj, yj, 0);
    const int pj_zero = (Pin[2 * cj] == 0.0 && Pin[2 * cj + 1] == 0.0);
    const float rmin = O->delta;
    double ar = 0.0, ai = 0.0;
    for (long q = 0; q < O->nact; q++) {
        const long ci_ = O->act[q];
        int fa, xi, yi;
        cell_xy(O, ci_, &fa, &xi, &yi);
        uint8_t m = 0;
        if (fa != fb) {
            const facet_t *Fa = &O->f[fa];
            const f3 pi = frag_pos(Fa, xi, yi, 0);
            /* enumeration orientation: lower facet index is the "A" side */
            const int fwd = fa < fb;
            const f3 pA = fwd ? pi : pj, pB = fwd ? pj : pi;
            const facet_t *FA = fwd ? Fa : Fb, *FB = fwd ? Fb : Fa;
            f3 v = {pB.x - pA.x, pB.y - pA.y, pB.z - pA.z};
            float r = sqrtf(dot_sc(v, v));
            float inv = 1.0f / r;
            f3 uv = {v.x * inv, v.y * inv, v.z * inv};
            float cs = dot_sc(uv, FA->normal);
            f3 nuv = {-uv.x, -uv.y, -uv.z};
            float cin = dot_sc(nuv, FB->normal);
            if (!(cs < 1e-6f) && !(cin < 1e-6f)) {
                double o[3], e[3];
                to_d3(pA, o); to_d3(pB, e);
                int graze, spf;
                int hit = seg_occluded(s, o, e, (double)(r - 1e-3f), &graze, &spf);
                if (graze) { m |= 2; cnt[1]++; }
                if (spf) cnt[2]++;
                if (!hit) {
                    m |= 1;
                    const int allowed = fwd ? 1 : !pj_zero;
                    const double Pr = Pin[2 * ci_], Pim = Pin[2 * ci_ + 1];
                    const int src_zero = (Pr == 0.0 && Pim == 0.0);
                    if (allowed && !(fwd && src_zero)) {
                        double gr, gi;
                        green_f2f(s, r, rmin, &gr, &gi);
                        const double w = (double)((O->area[ci_] * cs) * cin);
                        const double pr = w * Pr, pim = w * Pim;
                        ar += pr * gr - pim * gi;
                        ai += pr * gi + pim * gr;
                    }
                }
            }
            cnt[0]++;
        }
        if (mask_row) mask_row[q] = m;
    }
    acc[0] = ar; acc[1] = ai;
}

/* ---- hop a6, FACET_NO_RESP (target object A -> field object B): the
 * input is A's total pressure P (OptiX.cu:231-238), cos_inc = 1 for the field
 * destination (:308-312), the ray runs from the target fragment. */
static void hop_noresp_cell(scene_t *s, const object_t *A, const object_t *B, long q_j, double *acc,
                            uint8_t *mask_row, long long *cnt)
{
    const long cj = B->act[q_j];
    int fb, xj, yj;
    cell_xy(B, cj, &fb, &xj, &yj);
    const f3 pj = frag_pos(&B->f[fb], xj, yj, 0);
    const float rmin = A->delta;
    double ar = 0.0, ai = 0.0;
    for (long q = 0; q < A->nact; q++) {
        const long ci_ = A->act[q];
        int fa, xi, yi;
        cell_xy(A, ci_, &fa, &xi, &yi);
        const facet_t *Fa = &A->f[fa];
        const f3 pi = frag_pos(Fa, xi, yi, 0);
        uint8_t m = 0;
        f3 v = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
        float r = sqrtf(dot_sc(v, v));
        float inv = 1.0f / r;
        f3 uv = {v.x * inv, v.y * inv, v.z * inv};
        float cs = dot_sc(uv, Fa->normal);
        float cin = 1;
        if (!(cs < 1e-6f)) {
            double o[3], e[3];
            to_d3(pi, o); to_d3(pj, e);
            int graze, spf;
            int hit = seg_occluded(s, o, e, (double)(r - 1e-3f), &graze, &spf);
            if (graze) { m |= 2; cnt[1]++; }
            if (spf) cnt[2]++;
            if (!hit) {
                m |= 1;
                const double Pr = A->P[2 * ci_], Pim = A->P[2 * ci_ + 1];
                if (!(Pr == 0.0 && Pim == 0.0)) {
                    double gr, gi;
                    green_f2f(s, r, rmin, &gr, &gi);
                    const double w = (double)((A->area[ci_] * cs) * cin);
                    const double pr = w * Pr, pim = w * Pim;
                    ar += pr * gr - pim * gi;
                    ai += pr * gi + pim * gr;
                }
            }
        }
        cnt[0]++;
        if (mask_row) mask_row[q] = m;
    }
    acc[0] = ar; acc[1] = ai;
}

/* ---- hop a6, FACET_RESP (target object A -> another target object B, with
 * reciprocity): src/OptiX.cu:192-406 with useReciprocity and not isSelf
 * (:427-429; the reference has no host caller for it).  Every active cell
 * pair (i of A, j of B): uv from p_i to p_j, cos_scat at A's normal, cos_inc
 * at B's, the ray from p_i, G regularised below A's delta and damped by 0.9.
 * Destination-owned restatement:
 *   fwd = 1: cell j of B receives A_i cos_scat cos_inc P_in,A[i] G from every
 *            cell i of A with P_in,A[i] != 0 (OptiX.cu:241-245, :354-364);
 *   fwd = 0: cell i of A receives B_j cos_scat cos_inc P_in,B[j] G from every
 *            cell j of B (the reciprocal write, :367-390), nothing at all when
 *            P_in,A[i] == 0 (the zero-input skip of the A side kills it). */
static void hop_resp_cell(scene_t *s, const object_t *A, const object_t *B, int fwd, long q_d, double *acc,
                          uint8_t *mask_row, long long *cnt)
{
    const object_t *D = fwd ? B : A, *S = fwd ? A : B;
    const long cd = D->act[q_d];
    int fd, xd, yd;
    cell_xy(D, cd, &fd, &xd, &yd);
    const facet_t *Fd = &D->f[fd];
    const f3 pd = frag_pos(Fd, xd, yd, 0);
    const float rmin = A->delta;
    const int gate_zero = !fwd && A->Pin[2 * cd] == 0.0 && A->Pin[2 * cd + 1] == 0.0;
    double ar = 0.0, ai = 0.0;
    for (long q = 0; q < S->nact; q++) {
        const long cs_ = S->act[q];
        int fs, xs, ys;
        cell_xy(S, cs_, &fs, &xs, &ys);
        const facet_t *Fs = &S->f[fs];
        const f3 ps = frag_pos(Fs, xs, ys, 0);
        const f3 pA = fwd ? ps : pd, pB = fwd ? pd : ps;
        const facet_t *FA = fwd ? Fs : Fd, *FB = fwd ? Fd : Fs;
        uint8_t m = 0;
        f3 v = {pB.x - pA.x, pB.y - pA.y, pB.z - pA.z};
        float r = sqrtf(dot_sc(v, v));
        float inv = 1.0f / r;
        f3 uv = {v.x * inv, v.y * inv, v.z * inv};
        float cs = dot_sc(uv, FA->normal);
        f3 nuv = {-uv.x, -uv.y, -uv.z};
        float cin = dot_sc(nuv, FB->normal);
        if (!(cs < 1e-6f) && !(cin < 1e-6f)) {
            double o[3], e[3];
            to_d3(pA, o); to_d3(pB, e);
            int graze, spf;
            int hit = seg_occluded(s, o, e, (double)(r - 1e-3f), &graze, &spf);
            if (graze) { m |= 2; cnt[1]++; }
            if (spf) cnt[2]++;
            if (!hit) {
                m |= 1;
                const double Pr = S->Pin[2 * cs_], Pim = S->Pin[2 * cs_ + 1];
                if (!gate_zero && !(Pr == 0.0 && Pim == 0.0)) {
                    double gr, gi;
                    green_f2f(s, r, rmin, &gr, &gi);
                    const double w = (double)((S->area[cs_] * cs) * cin);
                    const double pr = w * Pr, pim = w * Pim;
                    ar += pr * gr - pim * gi;
                    ai += pr * gi + pim * gr;
                }
            }
        }
        cnt[0]++;
        if (mask_row) mask_row[q] = m;
    }
    acc[0] = ar; acc[1] = ai;
}

static void reset_counters(scene_t *s) { s->c_pairs = s->c_graze = s->c_selfplane = 0; }

#define OMP_COUNTERS long long c0 = 0, c1 = 0, c2 = 0;
#define OMP_COUNTERS_ADD s->c_pairs += c0; s->c_graze += c1; s->c_selfplane += c2;

/* ---- sequencing ---------------------------------------------------------- */
/* ModelCuda::ProjectSrcPointsToObjects (ModelCuda.cpp:242-278): P += sum */
static void project_sources_obj(scene_t *s, object_t *B)
{
    OMP_COUNTERS
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : c0, c1, c2)
    for (long c = 0; c < B->ncells; c++) {
        double acc[2];
        long long cnt[3] = {0, 0, 0};
        hop_source_cell(s, B, c, acc, NULL, cnt);
        B->P[2 * c] += acc[0];
        B->P[2 * c + 1] += acc[1];
        c0 += cnt[0]; c1 += cnt[1]; c2 += cnt[2];
    }
    OMP_COUNTERS_ADD
}

/* Piston source objects (objectType 1; the reference stores them unused,
 * src/Model.cpp:33-35): every fragment radiates its unit surface pressure
 * through the facet -> facet projection of src/OptiX.cu:192-406 -- area,
 * cos_scat at the piston, cos_inc at a target destination (1 at a field
 * object), r < delta regularisation and 0.9 factor, shadow ray from the
 * piston fragment, destinations gated by their area -- into the active cells
 * of the target (field) object B: the FACET_RESP (FACET_NO_RESP) cell sums
 * with the piston in the source object's place. */
static void project_piston(scene_t *s, object_t *S, object_t *B, int field)
{
    OMP_COUNTERS
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : c0, c1, c2)
    for (long q = 0; q < B->nact; q++) {
        double acc[2];
        long long cnt[3] = {0, 0, 0};
        if (field)
            hop_noresp_cell(s, S, B, q, acc, NULL, cnt);
        else
            hop_resp_cell(s, S, B, 1, q, acc, NULL, cnt);
        const long c = B->act[q];
        B->P[2 * c] += acc[0];
        B->P[2 * c + 1] += acc[1];
        c0 += cnt[0]; c1 += cnt[1]; c2 += cnt[2];
    }
    OMP_COUNTERS_ADD
}

int orc_project_sources(void *h, int field_objects)
{
    scene_t *s = (scene_t *)h;
    if (!s->rendered) return -1;
    reset_counters(s);
    for (int i = 0; i < s->nobj[OBJ_TARGET]; i++) project_sources_obj(s, s->obj[OBJ_TARGET][i]);
    if (field_objects)
        for (int i = 0; i < s->nobj[OBJ_FIELD]; i++) project_sources_obj(s, s->obj[OBJ_FIELD][i]);
    for (int p = 0; p < s->nobj[OBJ_SOURCE]; p++) {
        for (int i = 0; i < s->nobj[OBJ_TARGET]; i++) project_piston(s, s->obj[OBJ_SOURCE][p], s->obj[OBJ_TARGET][i], 0);
        if (field_objects)
            for (int i = 0; i < s->nobj[OBJ_FIELD]; i++)
                project_piston(s, s->obj[OBJ_SOURCE][p], s->obj[OBJ_FIELD][i], 1);
    }
    return 0;
}

/* Bounces with cross-object terms (an extension; the reference's host never
 * calls FACET_RESP): prime P_out <- P on every target; per bounce every
 * target takes P_in <- P_out, P_out <- 0; then each target's FACET_SELF
 * projection, then FACET_RESP for every pair a < b (forward into b, the
 * reciprocal terms into a), all from this bounce's inputs; then P += P_out
 * on every target. */
int orc_project_bounces_cross(void *h, int nb)
{
    scene_t *s = (scene_t *)h;
    if (!s->rendered) return -1;
    reset_counters(s);
    const int nt = s->nobj[OBJ_TARGET];
    for (int oi = 0; oi < nt; oi++) {
        object_t *O = s->obj[OBJ_TARGET][oi];
        memcpy(O->Pout, O->P, sizeof(double) * 2 * O->ncells);
    }
    for (int b = 0; b < nb; b++) {
        for (int oi = 0; oi < nt; oi++) {
            object_t *O = s->obj[OBJ_TARGET][oi];
            memcpy(O->Pin, O->Pout, sizeof(double) * 2 * O->ncells);
            memset(O->Pout, 0, sizeof(double) * 2 * O->ncells);
        }
        for (int oi = 0; oi < nt; oi++) {
            object_t *O = s->obj[OBJ_TARGET][oi];
            OMP_COUNTERS
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : c0, c1, c2)
            for (long q = 0; q < O->nact; q++) {
                double acc[2];
                long long cnt[3] = {0, 0, 0};
                hop_f2f_cell(s, O, q, O->Pin, acc, NULL, cnt);
                O->Pout[2 * O->act[q]] = acc[0];
                O->Pout[2 * O->act[q] + 1] = acc[1];
                c0 += cnt[0]; c1 += cnt[1]; c2 += cnt[2];
            }
            OMP_COUNTERS_ADD
        }
        for (int ai_ = 0; ai_ < nt; ai_++)
            for (int bi_ = ai_ + 1; bi_ < nt; bi_++) {
                object_t *A = s->obj[OBJ_TARGET][ai_], *B = s->obj[OBJ_TARGET][bi_];
                for (int fwd = 1; fwd >= 0; fwd--) {
                    object_t *D = fwd ? B : A;
                    OMP_COUNTERS
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : c0, c1, c2)
                    for (long q = 0; q < D->nact; q++) {
                        double acc[2];
                        long long cnt[3] = {0, 0, 0};
                        hop_resp_cell(s, A, B, fwd, q, acc, NULL, cnt);
                        D->Pout[2 * D->act[q]] += acc[0];
                        D->Pout[2 * D->act[q] + 1] += acc[1];
                        c0 += cnt[0]; c1 += cnt[1]; c2 += cnt[2];
                    }
                    OMP_COUNTERS_ADD
                }
            }
        for (int oi = 0; oi < nt; oi++) {
            object_t *O = s->obj[OBJ_TARGET][oi];
            for (long c = 0; c < O->ncells; c++) {
                O->P[2 * c] += O->Pout[2 * c];
                O->P[2 * c + 1] += O->Pout[2 * c + 1];
            }
        }
    }
    return 0;
}

/* ModelCuda::ProjectTargetToTargetObjects (ModelCuda.cpp:323-356):
 * prime P_out <- P; per bounce: P_in <- P_out, P_out <- 0, project, P += P_out. */
int orc_project_bounces(void *h, int nb)
{
    scene_t *s = (scene_t *)h;
    if (!s->rendered) return -1;
    reset_counters(s);
    for (int oi = 0; oi < s->nobj[OBJ_TARGET]; oi++) {
        object_t *O = s->obj[OBJ_TARGET][oi];
        memcpy(O->Pout, O->P, sizeof(double) * 2 * O->ncells);
        for (int b = 0; b < nb; b++) {
            memcpy(O->Pin, O->Pout, sizeof(double) * 2 * O->ncells);
            memset(O->Pout, 0, sizeof(double) * 2 * O->ncells);
            OMP_COUNTERS
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : c0, c1, c2)
            for (long q = 0; q < O->nact; q++) {
                double acc[2];
                long long cnt[3] = {0, 0, 0};
                hop_f2f_cell(s, O, q, O->Pin, acc, NULL, cnt);
                O->Pout[2 * O->act[q]] = acc[0];
                O->Pout[2 * O->act[q] + 1] = acc[1];
                c0 += cnt[0]; c1 += cnt[1]; c2 += cnt[2];
            }
            OMP_COUNTERS_ADD
            for (long c = 0; c < O->ncells; c++) {
                O->P[2 * c] += O->Pout[2 * c];
                O->P[2 * c + 1] += O->Pout[2 * c + 1];
            }
        }
    }
    return 0;
}

/* ModelCuda::ProjectTargetToFieldObjects (ModelCuda.cpp:280-301) */
int orc_project_field_objects(void *h)
{
    scene_t *s = (scene_t *)h;
    if (!s->rendered) return -1;
    reset_counters(s);
    for (int ti = 0; ti < s->nobj[OBJ_TARGET]; ti++) {
        object_t *A = s->obj[OBJ_TARGET][ti];
        for (int fi = 0; fi < s->nobj[OBJ_FIELD]; fi++) {
            object_t *B = s->obj[OBJ_FIELD][fi];
            OMP_COUNTERS
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : c0, c1, c2)
            for (long q = 0; q < B->nact; q++) {
                double acc[2];
                long long cnt[3] = {0, 0, 0};
                hop_noresp_cell(s, A, B, q, acc, NULL, cnt);
                B->P[2 * B->act[q]] += acc[0];
                B->P[2 * B->act[q] + 1] += acc[1];
                c0 += cnt[0]; c1 += cnt[1]; c2 += cnt[2];
            }
            OMP_COUNTERS_ADD
        }
    }
    return 0;
}

/* ModelCuda::ProjectTargetToFieldPoints (ModelCuda.cpp:302-321) */
int orc_project_field_points(void *h)
{
    scene_t *s = (scene_t *)h;
    if (!s->rendered) return -1;
    reset_counters(s);
    for (int ti = 0; ti < s->nobj[OBJ_TARGET]; ti++) {
        object_t *A = s->obj[OBJ_TARGET][ti];
        OMP_COUNTERS
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : c0, c1, c2)
        for (int j = 0; j < s->nfp; j++) {
            double acc[2];
            long long cnt[3] = {0, 0, 0};
            hop_fieldpoint(s, A, j, acc, NULL, cnt);
            s->fpP[2 * j] += acc[0];
            s->fpP[2 * j + 1] += acc[1];
            c0 += cnt[0]; c1 += cnt[1]; c2 += cnt[2];
        }
        OMP_COUNTERS_ADD
    }
    return 0;
}

/* ---- subset evaluation (no state change): large scenes are checked on a
 * seeded subset of destinations given the inputs of the hop. ---------------- */
/* hop: 0 source->object cells, 1 target->field points, 2 f2f self, 3 target->field object.
 * src_type/src_idx, dst_type/dst_idx select the objects (ignored where not used).
 * dst: destination indices (cells for hop 0, field points for hop 1, active
 * positions q for hops 2 and 3).  pin: input pressures for hop 2 (2 per cell of
 * the object); NULL uses the object's current P_in.  out: 2 doubles per dst.
 * mask (optional): n x nsrc bytes (bit0 interacts, bit1 grazing). */
long orc_hop_subset(void *h, int hop, int a_idx, int b_idx, const long *dst, long n, const double *pin,
                    double *out, uint8_t *mask)
{
    scene_t *s = (scene_t *)h;
    if (!s->rendered) return -1;
    reset_counters(s);
    long nsrc = 0;
    object_t *A = NULL, *B = NULL;
    switch (hop) {
    case 0:
        if (a_idx < 0 || a_idx > 2 || b_idx < 0 || b_idx >= s->nobj[a_idx]) return -2;
        B = s->obj[a_idx][b_idx];
        nsrc = s->nsrc;
        break;
    case 1:
        if (a_idx < 0 || a_idx >= s->nobj[OBJ_TARGET]) return -2;
        A = s->obj[OBJ_TARGET][a_idx];
        nsrc = A->nact;
        break;
    case 2:
        if (a_idx < 0 || a_idx >= s->nobj[OBJ_TARGET]) return -2;
        A = s->obj[OBJ_TARGET][a_idx];
        nsrc = A->nact;
        if (!pin) pin = A->Pin;
        break;
    case 3:
        if (a_idx < 0 || a_idx >= s->nobj[OBJ_TARGET] || b_idx < 0 || b_idx >= s->nobj[OBJ_FIELD]) return -2;
        A = s->obj[OBJ_TARGET][a_idx];
        B = s->obj[OBJ_FIELD][b_idx];
        nsrc = A->nact;
        break;
    case 4:
        /* FACET_RESP between targets a_idx (sources) and b_idx (destinations):
         * the forward terms when a_idx < b_idx, the reciprocal ones when
         * a_idx > b_idx; the inputs are the objects' P_in */
        if (a_idx < 0 || a_idx >= s->nobj[OBJ_TARGET] || b_idx < 0 || b_idx >= s->nobj[OBJ_TARGET] || a_idx == b_idx)
            return -2;
        A = s->obj[OBJ_TARGET][a_idx < b_idx ? a_idx : b_idx];
        B = s->obj[OBJ_TARGET][a_idx < b_idx ? b_idx : a_idx];
        nsrc = s->obj[OBJ_TARGET][a_idx]->nact;
        break;
    case 5:
    case 6:
        /* piston source object a_idx -> target (5) or field object (6) b_idx */
        if (a_idx < 0 || a_idx >= s->nobj[OBJ_SOURCE] || b_idx < 0 ||
            b_idx >= s->nobj[hop == 5 ? OBJ_TARGET : OBJ_FIELD])
            return -2;
        A = s->obj[OBJ_SOURCE][a_idx];
        B = s->obj[hop == 5 ? OBJ_TARGET : OBJ_FIELD][b_idx];
        nsrc = A->nact;
        break;
    default:
        return -3;
    }
    OMP_COUNTERS
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : c0, c1, c2)
    for (long k = 0; k < n; k++) {
        double acc[2] = {0.0, 0.0};
        long long cnt[3] = {0, 0, 0};
        uint8_t *row = mask ? mask + k * nsrc : NULL;
        switch (hop) {
        case 0: hop_source_cell(s, B, dst[k], acc, row, cnt); break;
        case 1: hop_fieldpoint(s, A, (int)dst[k], acc, row, cnt); break;
        case 2: hop_f2f_cell(s, A, dst[k], pin, acc, row, cnt); break;
        case 3: hop_noresp_cell(s, A, B, dst[k], acc, row, cnt); break;
        case 4: hop_resp_cell(s, A, B, a_idx < b_idx, dst[k], acc, row, cnt); break;
        case 5: hop_resp_cell(s, A, B, 1, dst[k], acc, row, cnt); break;
        case 6: hop_noresp_cell(s, A, B, dst[k], acc, row, cnt); break;
        }
        out[2 * k] = acc[0];
        out[2 * k + 1] = acc[1];
        c0 += cnt[0]; c1 += cnt[1]; c2 += cnt[2];
    }
    OMP_COUNTERS_ADD
    return nsrc;
}

/* ---- accessors ---------------------------------------------------------- */
long long orc_counter(void *h, int which)
{
    scene_t *s = (scene_t *)h;
    return which == 0 ? s->c_pairs : which == 1 ? s->c_graze : s->c_selfplane;
}

int orc_num_objects(void *h, int type)
{
    scene_t *s = (scene_t *)h;
    return (type >= 0 && type <= 2) ? s->nobj[type] : -1;
}

static object_t *get_obj(scene_t *s, int type, int idx)
{
    if (type < 0 || type > 2 || idx < 0 || idx >= s->nobj[type]) return NULL;
    return s->obj[type][idx];
}

long orc_object_ncells(void *h, int type, int idx)
{
    object_t *o = get_obj((scene_t *)h, type, idx);
    return o ? o->ncells : -1;
}

long orc_object_nact(void *h, int type, int idx)
{
    object_t *o = get_obj((scene_t *)h, type, idx);
    return o ? o->nact : -1;
}

int orc_object_nfacets(void *h, int type, int idx)
{
    object_t *o = get_obj((scene_t *)h, type, idx);
    return o ? o->nf : -1;
}

/* which: 0 P, 1 P_in, 2 P_out */
int orc_get_object_pressures(void *h, int type, int idx, int which, double *out)
{
    object_t *o = get_obj((scene_t *)h, type, idx);
    if (!o || !o->P) return -1;
    const double *src = which == 0 ? o->P : which == 1 ? o->Pin : o->Pout;
    memcpy(out, src, sizeof(double) * 2 * o->ncells);
    return 0;
}

int orc_set_object_pressures(void *h, int type, int idx, int which, const double *in)
{
    object_t *o = get_obj((scene_t *)h, type, idx);
    if (!o || !o->P) return -1;
    double *dst = which == 0 ? o->P : which == 1 ? o->Pin : o->Pout;
    memcpy(dst, in, sizeof(double) * 2 * o->ncells);
    return 0;
}

int orc_get_areas(void *h, int type, int idx, float *out)
{
    object_t *o = get_obj((scene_t *)h, type, idx);
    if (!o || !o->area) return -1;
    memcpy(out, o->area, sizeof(float) * o->ncells);
    return 0;
}

long orc_get_active(void *h, int type, int idx, long *out)
{
    object_t *o = get_obj((scene_t *)h, type, idx);
    if (!o || !o->act) return -1;
    if (out) memcpy(out, o->act, sizeof(long) * o->nact);
    return o->nact;
}

/* per facet: nx, ny, neg (3 ints) and 17 floats:
 * normal(3) base(3) xAxis(3) yAxis(3) baseLen height baseNeg basePos area */
int orc_get_facets(void *h, int type, int idx, int *ints, float *floats)
{
    object_t *o = get_obj((scene_t *)h, type, idx);
    if (!o) return -1;
    for (int i = 0; i < o->nf; i++) {
        const facet_t *f = &o->f[i];
        ints[3 * i] = f->nx; ints[3 * i + 1] = f->ny; ints[3 * i + 2] = f->neg;
        float *q = floats + 17 * i;
        q[0] = f->normal.x; q[1] = f->normal.y; q[2] = f->normal.z;
        q[3] = f->base.x; q[4] = f->base.y; q[5] = f->base.z;
        q[6] = f->xAxis.x; q[7] = f->xAxis.y; q[8] = f->xAxis.z;
        q[9] = f->yAxis.x; q[10] = f->yAxis.y; q[11] = f->yAxis.z;
        q[12] = f->baseLen; q[13] = f->height; q[14] = f->baseNeg; q[15] = f->basePos; q[16] = f->area;
    }
    return o->nf;
}

int orc_get_field_points(void *h, double *out)
{
    scene_t *s = (scene_t *)h;
    memcpy(out, s->fpP, sizeof(double) * 2 * s->nfp);
    return s->nfp;
}

/* Fragment one triangle (no scene): returns the cell count, fills nx/ny/neg,
 * the 17 frame floats and up to cap areas. */
long orc_fragment_triangle(const float *tri9, float delta, int *ints, float *floats, float *areas, long cap)
{
    facet_t f;
    f3 a = {tri9[0], tri9[1], tri9[2]}, b = {tri9[3], tri9[4], tri9[5]}, c = {tri9[6], tri9[7], tri9[8]};
    facet_init(&f, a, b, c, delta);
    ints[0] = f.nx; ints[1] = f.ny; ints[2] = f.neg;
    floats[0] = f.normal.x; floats[1] = f.normal.y; floats[2] = f.normal.z;
    floats[3] = f.base.x; floats[4] = f.base.y; floats[5] = f.base.z;
    floats[6] = f.xAxis.x; floats[7] = f.xAxis.y; floats[8] = f.xAxis.z;
    floats[9] = f.yAxis.x; floats[10] = f.yAxis.y; floats[11] = f.yAxis.z;
    floats[12] = f.baseLen; floats[13] = f.height; floats[14] = f.baseNeg; floats[15] = f.basePos; floats[16] = f.area;
    long n = (long)f.nx * f.ny;
    if (areas && cap >= n) facet_fragment(&f, areas);
    return n;
}

/* Occlusion query (tests): returns 1 occluded; graze/selfplane flags out. */
int orc_segment(void *h, const double *o, const double *e, double tmax, int *flags)
{
    scene_t *s = (scene_t *)h;
    int g, sp;
    int hit = seg_occluded(s, o, e, tmax, &g, &sp);
    flags[0] = g; flags[1] = sp;
    return hit;
}

/* Surface colour map of src/FacetCuda.cu:10-72 (hsv2rgb, MakeSurface) with the
 * reference's float/double promotions: P (2 doubles per cell) -> RGBA floats. */
static void hsv2rgb_ref(float h, float s, float v, float *o)
{
    float c = v * s;
    float x = c * (1.0 - fabs(fmod(h * 6.0, 2.0) - 1.0));
    float m = v - c;
    float alpha = 1;
    float r, g, b;
    if (h < 1.0 / 6.0) { r = c + m; g = x + m; b = 0.0 + m; }
    else if (h < 2.0 / 6.0) { r = x + m; g = c + m; b = 0.0 + m; }
    else if (h < 3.0 / 6.0) { r = 0.0 + m; g = c + m; b = x + m; }
    else if (h < 4.0 / 6.0) { r = 0.0 + m; g = x + m; b = c + m; }
    else if (h < 5.0 / 6.0) { r = x + m; g = 0.0 + m; b = c + m; }
    else { r = c + m; g = 0.0 + m; b = x + m; }
    o[0] = r; o[1] = g; o[2] = b; o[3] = alpha;
}

void orc_colour_map(const double *P, long n, float min_db, float max_db, int phase, float *rgba)
{
    for (long i = 0; i < n; i++) {
        float pr = (float)P[2 * i], pi = (float)P[2 * i + 1];
        const float saturation = 0.8f;
        float dB = 20.0f * log10f(hypotf(pr, pi) + 1e-8f);
        float mag = (dB - min_db) / (max_db - min_db);
        mag = fminf(fmaxf(mag, 0.0f), 1.0f);
        float *o = rgba + 4 * i;
        o[0] = o[1] = o[2] = saturation * mag;
        o[3] = 1.0f;
        if (phase) {
            float h = (atan2f(pi, pr) + M_PI) / (2.0f * M_PI);
            hsv2rgb_ref(h, 0.8f, mag, o);
        }
    }
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
