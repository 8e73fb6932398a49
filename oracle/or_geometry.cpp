// or_geometry.cpp — oracle: geometry placement.  TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// A restatement of src/geometry: ImplicitEvaluator::isInside / evaluate
// (implicit/ImplicitEvaluator.cpp:8-98), GeometryDescriptor::computeTransformedAABB
// (include/fluidloom/geometry/GeometryDescriptor.h:70-113), SimpleSTLVoxelizer::voxelize /
// isInside / rayIntersectsTriangle (voxelizer/SimpleSTLVoxelizer.cpp:119-247) and
// GeometryPlacer::generateCandidates (placer/GeometryPlacer.cpp:98-118), operation by
// operation (compiled with -ffp-contract=off).  Pinned against the reference's own sources
// compiled in place (oracle/Makefile.ref, ref_geometry.cpp) where the reference tree exists.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

namespace {

bool inside_implicit(const or_geometry* g, float x, float y, float z) {
    float lx = (x - g->translate[0]) / g->scale[0];
    float ly = (y - g->translate[1]) / g->scale[1];
    float lz = (z - g->translate[2]) / g->scale[2];
    switch (g->type) {
        case 3: {  // sphere
            float d = lx * lx;
            d = d + ly * ly;
            d = d + lz * lz;
            return d <= g->radius * g->radius;
        }
        case 2: {  // box
            float hw = g->width * 0.5f, hh = g->height * 0.5f, hl = g->length * 0.5f;
            return std::fabs(lx) <= hw && std::fabs(ly) <= hh && std::fabs(lz) <= hl;
        }
        case 4: {  // cylinder about y
            float d = lx * lx;
            d = d + lz * lz;
            return d <= g->radius * g->radius && std::fabs(ly) <= g->height * 0.5f;
        }
        default:
            return false;
    }
}

struct Tri {
    float v[9];
    float lo[3], hi[3];
};

bool ray_hits(const Tri& t, float ox, float oy, float oz) {
    const float eps = 1e-6f;
    float e1[3] = {t.v[3] - t.v[0], t.v[4] - t.v[1], t.v[5] - t.v[2]};
    float e2[3] = {t.v[6] - t.v[0], t.v[7] - t.v[1], t.v[8] - t.v[2]};
    volatile float dx = 1.0f, dy = 0.0f, dz = 0.0f;  // the reference passes the ray direction in
    float h0 = dy * e2[2] - dz * e2[1];
    float h1 = dz * e2[0] - dx * e2[2];
    float h2 = dx * e2[1] - dy * e2[0];
    float a = e1[0] * h0 + e1[1] * h1 + e1[2] * h2;
    if (a > -eps && a < eps) return false;
    float f = 1.0f / a;
    float s0 = ox - t.v[0], s1 = oy - t.v[1], s2 = oz - t.v[2];
    float u = f * (s0 * h0 + s1 * h1 + s2 * h2);
    if (u < 0.0f || u > 1.0f) return false;
    float q0 = s1 * e1[2] - s2 * e1[1];
    float q1 = s2 * e1[0] - s0 * e1[2];
    float q2 = s0 * e1[1] - s1 * e1[0];
    float v = f * (dx * q0 + dy * q1 + dz * q2);
    if (v < 0.0f || u + v > 1.0f) return false;
    float tt = f * (e2[0] * q0 + e2[1] * q1 + e2[2] * q2);
    return tt > eps;
}

}  // namespace

extern "C" {

void or_geometry_aabb(const or_geometry* g, float* b) {
    float lo[3], hi[3];
    switch (g->type) {
        case 3:
            for (int a = 0; a < 3; ++a) { lo[a] = -g->radius; hi[a] = g->radius; }
            break;
        case 2:
            lo[0] = -g->width / 2; hi[0] = g->width / 2;
            lo[1] = -g->height / 2; hi[1] = g->height / 2;
            lo[2] = -g->length / 2; hi[2] = g->length / 2;
            break;
        case 4:
            lo[0] = -g->radius; hi[0] = g->radius;
            lo[1] = -g->height / 2; hi[1] = g->height / 2;
            lo[2] = -g->radius; hi[2] = g->radius;
            break;
        default:
            for (int a = 0; a < 3; ++a) { lo[a] = -0.5f; hi[a] = 0.5f; }
    }
    for (int a = 0; a < 3; ++a) {
        lo[a] *= g->scale[a];
        hi[a] *= g->scale[a];
        b[a] = lo[a] + g->translate[a];
        b[3 + a] = hi[a] + g->translate[a];
    }
}

void or_geometry_inside(const or_geometry* g, const float* x, const float* y, const float* z, size_t n,
                        uint8_t* out) {
    for (size_t i = 0; i < n; ++i) out[i] = inside_implicit(g, x[i], y[i], z[i]) ? 1 : 0;
}

void or_geometry_evaluate(const or_geometry* g, const int32_t* x, const int32_t* y, const int32_t* z, size_t n,
                          uint8_t* out) {
    for (size_t i = 0; i < n; ++i)
        out[i] = inside_implicit(g, (float)x[i] + 0.5f, (float)y[i] + 0.5f, (float)z[i] + 0.5f) ? 1 : 0;
}

// Cells (z, y, x loop order) of the STL voxelisation; returns the count, writes at most cap.
size_t or_stl_voxelize(const float* tris, size_t ntri, const or_geometry* g, float cell, int32_t* ox, int32_t* oy,
                       int32_t* oz, size_t cap) {
    if (!ntri) return 0;
    std::vector<Tri> T(ntri);
    float mlo[3] = {std::numeric_limits<float>::max(), std::numeric_limits<float>::max(),
                    std::numeric_limits<float>::max()};
    float mhi[3] = {std::numeric_limits<float>::lowest(), std::numeric_limits<float>::lowest(),
                    std::numeric_limits<float>::lowest()};
    for (size_t k = 0; k < ntri; ++k) {
        for (int j = 0; j < 9; ++j) T[k].v[j] = tris[k * 9 + j];
        for (int a = 0; a < 3; ++a) {
            T[k].lo[a] = std::min({T[k].v[a], T[k].v[3 + a], T[k].v[6 + a]});
            T[k].hi[a] = std::max({T[k].v[a], T[k].v[3 + a], T[k].v[6 + a]});
            mlo[a] = std::min(mlo[a], T[k].lo[a]);
            mhi[a] = std::max(mhi[a], T[k].hi[a]);
        }
    }
    int s[3], e[3];
    for (int a = 0; a < 3; ++a) {
        float lo = mlo[a] * g->scale[a] + g->translate[a];
        float hi = mhi[a] * g->scale[a] + g->translate[a];
        s[a] = (int)std::floor(lo / cell);
        e[a] = (int)std::ceil(hi / cell);
    }
    size_t n = 0;
    for (int z = s[2]; z <= e[2]; ++z)
        for (int y = s[1]; y <= e[1]; ++y)
            for (int x = s[0]; x <= e[0]; ++x) {
                float wx = ((float)x + 0.5f) * cell, wy = ((float)y + 0.5f) * cell, wz = ((float)z + 0.5f) * cell;
                float lx = (wx - g->translate[0]) / g->scale[0];
                float ly = (wy - g->translate[1]) / g->scale[1];
                float lz = (wz - g->translate[2]) / g->scale[2];
                if (lx < mlo[0] || lx > mhi[0] || ly < mlo[1] || ly > mhi[1] || lz < mlo[2] || lz > mhi[2]) continue;
                int hits = 0;
                for (const Tri& t : T) {
                    if (ly < t.lo[1] || ly > t.hi[1] || lz < t.lo[2] || lz > t.hi[2]) continue;
                    if (lx > t.hi[0]) continue;
                    if (ray_hits(t, lx, ly, lz)) ++hits;
                }
                if (hits % 2 == 1) {
                    if (n < cap) { ox[n] = x; oy[n] = y; oz[n] = z; }
                    ++n;
                }
            }
    return n;
}

// GeometryPlacer::processGeometry for implicit types: candidates [floor, ceil) of the AABB
// clipped to the domain, kept where inside at their centres.
size_t or_geometry_candidates(const or_geometry* g, float cell, const float* dom, int32_t* ox, int32_t* oy,
                              int32_t* oz, size_t cap) {
    float b[6];
    or_geometry_aabb(g, b);
    int s[3], e[3];
    for (int a = 0; a < 3; ++a) {
        float lo = std::max(b[a], dom[a]), hi = std::min(b[3 + a], dom[3 + a]);
        s[a] = (int)std::floor(lo / cell);
        e[a] = (int)std::ceil(hi / cell);
    }
    size_t n = 0;
    for (int z = s[2]; z < e[2]; ++z)
        for (int y = s[1]; y < e[1]; ++y)
            for (int x = s[0]; x < e[0]; ++x)
                if (inside_implicit(g, (float)x + 0.5f, (float)y + 0.5f, (float)z + 0.5f)) {
                    if (n < cap) { ox[n] = x; oy[n] = y; oz[n] = z; }
                    ++n;
                }
    return n;
}

}  // extern "C"
