// Test-infrastructure: plain C entry points over the reference's geometry sources
// (ImplicitEvaluator.cpp, SimpleSTLVoxelizer.cpp, GeometryPlacer.cpp) compiled in place
// by oracle/Makefile.ref, to pin oracle/or_geometry.cpp.  Never part of the product.
#include "fluidloom/geometry/GeometryPlacer.h"
#include "fluidloom/geometry/ImplicitEvaluator.h"
#include "fluidloom/geometry/SimpleSTLVoxelizer.h"
#include <cstddef>
#include <cstdint>
#include <vector>

using fluidloom::CellCoord;
using fluidloom::geometry::GeometryDescriptor;

namespace {
GeometryDescriptor desc(int type, const float* t, const float* s, float radius, float height, float width,
                        float length, int material) {
    GeometryDescriptor g;
    static const GeometryDescriptor::Type kTypes[] = {GeometryDescriptor::Type::STL_MESH,
                                                      GeometryDescriptor::Type::IMPLICIT_FUNC,
                                                      GeometryDescriptor::Type::BOX, GeometryDescriptor::Type::SPHERE,
                                                      GeometryDescriptor::Type::CYLINDER};
    g.type = kTypes[type];
    g.name = "g";
    g.material_id = material;
    g.transform.tx = t[0]; g.transform.ty = t[1]; g.transform.tz = t[2];
    g.transform.sx = s[0]; g.transform.sy = s[1]; g.transform.sz = s[2];
    g.params.radius = radius; g.params.height = height; g.params.width = width; g.params.length = length;
    return g;
}
}  // namespace

extern "C" void ref_geometry_inside(int type, const float* t, const float* s, float radius, float height, float width,
                                    float length, const float* x, const float* y, const float* z, size_t n,
                                    uint8_t* out) {
    fluidloom::geometry::ImplicitEvaluator ev;
    GeometryDescriptor g = desc(type, t, s, radius, height, width, length, 1);
    for (size_t i = 0; i < n; ++i) out[i] = ev.isInside(g, x[i], y[i], z[i]) ? 1 : 0;
}

extern "C" size_t ref_stl_voxelize(const char* path, const float* t, const float* s, float cell, int32_t* ox,
                                   int32_t* oy, int32_t* oz, size_t cap) {
    fluidloom::geometry::SimpleSTLVoxelizer vox;
    if (!vox.loadSTL(path)) return (size_t)-1;
    GeometryDescriptor g = desc(0, t, s, 1, 1, 1, 1, 1);
    std::vector<CellCoord> cells = vox.voxelize(g, cell);
    for (size_t i = 0; i < cells.size() && i < cap; ++i) { ox[i] = cells[i].x; oy[i] = cells[i].y; oz[i] = cells[i].z; }
    return cells.size();
}

extern "C" void ref_geometry_aabb(int type, const float* t, const float* s, float radius, float height, float width,
                                  float length, float* b) {
    GeometryDescriptor g = desc(type, t, s, radius, height, width, length, 1);
    GeometryDescriptor::AABB a = g.computeTransformedAABB();
    b[0] = a.min_x; b[1] = a.min_y; b[2] = a.min_z; b[3] = a.max_x; b[4] = a.max_y; b[5] = a.max_z;
}
