// host.h -- host-side geometry of the GB300 library: facet frames and
// fragment grids (bit-identical to the reference's FP32 arithmetic) and the
// occluder BVH.
#pragma once
#include <array>
#include <functional>
#include <vector>

#include "sonar_internal.h"

namespace sonar {

struct Vec3 {
    float x, y, z;
};

// Frame of one facet (src/Facet.cpp:6-109): unit normal, the longest edge as
// the x axis, the foot of the altitude from the opposite vertex as the base
// point, the unit altitude as the y axis; fragment grid sizes
// (numXpnts, numYpnts, numXpntsNegative) from src/Facet.cpp:124-127.
struct FacetFrame {
    Vec3 v1, v2, v3;
    Vec3 normal, xAxis, yAxis, base;
    float baseLen = 0, height = 0, baseNeg = 0, basePos = 0, area = 0, delta = 0;
    int nx = 0, ny = 0, neg = 0;
};

FacetFrame make_frame(Vec3 v1, Vec3 v2, Vec3 v3, float delta);

// Clipped fragment areas, row-major y*nx + x (src/Facet.cpp:111-339).
void fragment_areas(const FacetFrame &f, float *area);
// The same for rows [j0, j1) only (area still points at row 0).
void fragment_area_rows(const FacetFrame &f, float *area, int j0, int j1);

// fn(u) for every u in [0, n), on up to 16 host threads taking units from a
// shared counter; an exception in any unit is rethrown (as runtime_error).
void parallel_units(long long n, const std::function<void(long long)> &fn);

// Fragment centroid of cell (x, y) as the kernels use it: with the +delta/2 x
// shift for the source hop (src/OptiX.cu:51), without it for the others
// (src/OptiX.cu:129, :210, :273).
Vec3 fragment_centroid(const FacetFrame &f, int x, int y, bool source_hop);

// Side, in cells, of the patches that order a facet's active fragments.
constexpr int kPatch = 16;

// A patch's active cells, consecutive in patch order: [begin, end) counted
// from the facet's first active cell; its patch row and column.
struct PatchRun {
    long long begin, end;
    int row, col;
};

// Patch-aligned order of one facet's active cells (given in patch order by
// their runs and readout centroids, the first of them at global index
// start): order[i] is the patch-order index of the cell placed at i.  Full
// patches start on 256-cell tile boundaries, a few cells of the partial
// patches (taken along the facet's boundary) in front of them and the rest
// after, the edge cells (readout centroid on or outside the triangle) last.
// Empty when the facet has no full or no partial patch, or too few partial
// cells to align: patch order stays.
std::vector<int> patch_aligned_order(const FacetFrame &F, const std::vector<PatchRun> &runs, const float4 *readout,
                                     long long start);

struct BvhHost {
    std::vector<BvhNode> nodes;
    std::vector<float4> tris;  // 4 per triangle
    int depth = 0;
};

// Median-split BVH over triangles (9 floats each), boxes padded by pad.
BvhHost build_bvh(const std::vector<std::array<float, 9>> &tris, double pad);

// Every vertex of the scene on or behind every triangle's plane (within tol,
// in double); scenes of more than 20,000 triangles count as non-convex.
bool scene_is_convex(const std::vector<std::array<float, 9>> &t, double tol);

}  // namespace sonar
