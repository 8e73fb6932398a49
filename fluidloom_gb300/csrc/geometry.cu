// geometry.cu — geometry placement on the GPU: implicit solids (sphere, box,
// cylinder) evaluated at cell centres, STL meshes voxelised by ray casting, and
// the merge of geometry cells into a cell list.
//
// Replaces src/geometry: ImplicitEvaluator (implicit/ImplicitEvaluator.cpp:8-98:
// translate then inverse-scale the point, rotation not applied; sphere
// x^2+y^2+z^2 <= r^2, box |x|,|y|,|z| <= w/2, h/2, l/2, cylinder about the y
// axis; implicit functions evaluate to outside), GeometryDescriptor::
// computeTransformedAABB (include/fluidloom/geometry/GeometryDescriptor.h:
// 70-113), SimpleSTLVoxelizer::voxelize / isInside / rayIntersectsTriangle
// (voxelizer/SimpleSTLVoxelizer.cpp:119-247: grid range floor/ceil of the
// transformed mesh bounds, inclusive; voxel centre mapped back to mesh space;
// +x ray, Moller-Trumbore with epsilon 1e-6, odd crossing count) and
// GeometryPlacer::processGeometry / generateCandidates / placeGeometry
// (placer/GeometryPlacer.cpp:14-118).  Every voxel or candidate is one
// thread; hits are compacted in the reference's z, y, x loop order by a scan.
// Built without FMA contraction, so results equal the oracle's bit for bit.
#include "common.cuh"
#include "scan.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace {

struct GeomDev {
    int type;
    float tx, ty, tz, sx, sy, sz;
    float radius, height, width, length;
};

GeomDev to_dev(const fl_geometry_desc& d) {
    GeomDev g;
    g.type = d.type;
    g.tx = d.translate[0]; g.ty = d.translate[1]; g.tz = d.translate[2];
    g.sx = d.scale[0]; g.sy = d.scale[1]; g.sz = d.scale[2];
    g.radius = d.radius; g.height = d.height; g.width = d.width; g.length = d.length;
    return g;
}

__device__ __forceinline__ bool implicit_inside(const GeomDev& g, float x, float y, float z) {
    float lx = (x - g.tx) / g.sx, ly = (y - g.ty) / g.sy, lz = (z - g.tz) / g.sz;
    if (g.type == FL_GEOM_SPHERE) {
        float d = lx * lx;
        d = d + ly * ly;
        d = d + lz * lz;
        return d <= g.radius * g.radius;
    }
    if (g.type == FL_GEOM_BOX) {
        float hw = g.width * 0.5f, hh = g.height * 0.5f, hl = g.length * 0.5f;
        return fabsf(lx) <= hw && fabsf(ly) <= hh && fabsf(lz) <= hl;
    }
    if (g.type == FL_GEOM_CYLINDER) {
        float d = lx * lx;
        d = d + lz * lz;
        return d <= g.radius * g.radius && fabsf(ly) <= g.height * 0.5f;
    }
    return false;  // implicit functions and meshes are not evaluated here
}

__global__ void k_geom_points(GeomDev g, const float* __restrict__ x, const float* __restrict__ y,
                              const float* __restrict__ z, size_t n, uint8_t* __restrict__ out) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = implicit_inside(g, x[i], y[i], z[i]) ? 1 : 0;
}

__global__ void k_geom_cells(GeomDev g, const int32_t* __restrict__ x, const int32_t* __restrict__ y,
                             const int32_t* __restrict__ z, size_t n, uint8_t* __restrict__ out) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = implicit_inside(g, (float)x[i] + 0.5f, (float)y[i] + 0.5f, (float)z[i] + 0.5f) ? 1 : 0;
}

// Triangles as v1, v2, v3 (9 floats) followed by their bounds min xyz, max xyz.
constexpr int kTri = 15;

__device__ bool ray_hits(const float* t, float ox, float oy, float oz) {
    const float eps = 1e-6f;
    float e1[3] = {t[3] - t[0], t[4] - t[1], t[5] - t[2]};
    float e2[3] = {t[6] - t[0], t[7] - t[1], t[8] - t[2]};
    // h = (1, 0, 0) x e2, written as the reference's general cross product
    const float dx = 1.0f, dy = 0.0f, dz = 0.0f;
    float h0 = dy * e2[2] - dz * e2[1];
    float h1 = dz * e2[0] - dx * e2[2];
    float h2 = dx * e2[1] - dy * e2[0];
    float a = e1[0] * h0 + e1[1] * h1 + e1[2] * h2;
    if (a > -eps && a < eps) return false;
    float f = 1.0f / a;
    float s0 = ox - t[0], s1 = oy - t[1], s2 = oz - t[2];
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

// One voxel of the grid [x0, x0 + nx) x ... per thread (z outermost, as the
// reference's loops); flag = inside the mesh.
__global__ void k_stl_voxels(const float* __restrict__ tris, uint32_t ntri, const float* __restrict__ mb, GeomDev g,
                             float cell, int x0, int y0, int z0, int nx, int ny, size_t nv, uint32_t* __restrict__ flag) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride) {
        const int x = x0 + (int)(i % nx), y = y0 + (int)((i / nx) % ny), z = z0 + (int)(i / ((size_t)nx * ny));
        float wx = ((float)x + 0.5f) * cell, wy = ((float)y + 0.5f) * cell, wz = ((float)z + 0.5f) * cell;
        float lx = (wx - g.tx) / g.sx, ly = (wy - g.ty) / g.sy, lz = (wz - g.tz) / g.sz;
        uint32_t inside = 0;
        if (!(lx < mb[0] || lx > mb[3] || ly < mb[1] || ly > mb[4] || lz < mb[2] || lz > mb[5])) {
            uint32_t hits = 0;
            for (uint32_t k = 0; k < ntri; ++k) {
                const float* t = tris + (size_t)k * kTri;
                if (ly < t[10] || ly > t[13] || lz < t[11] || lz > t[14]) continue;
                if (lx > t[12]) continue;
                if (ray_hits(t, lx, ly, lz)) ++hits;
            }
            inside = hits & 1u;
        }
        flag[i] = inside;
    }
}

__global__ void k_implicit_candidates(GeomDev g, int x0, int y0, int z0, int nx, int ny, size_t nv,
                                      uint32_t* __restrict__ flag) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride) {
        const int x = x0 + (int)(i % nx), y = y0 + (int)((i / nx) % ny), z = z0 + (int)(i / ((size_t)nx * ny));
        flag[i] = implicit_inside(g, (float)x + 0.5f, (float)y + 0.5f, (float)z + 0.5f) ? 1u : 0u;
    }
}

// Scatter the flagged grid cells (exclusive-scan offsets).
__global__ void k_grid_scatter(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ off, size_t nv, int x0,
                               int y0, int z0, int nx, int ny, size_t cap, int32_t* __restrict__ ox,
                               int32_t* __restrict__ oy, int32_t* __restrict__ oz) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride) {
        if (!flag[i]) continue;
        const size_t o = off[i];
        if (o >= cap) continue;
        const int x = x0 + (int)(i % nx), y = y0 + (int)((i / nx) % ny), z = z0 + (int)(i / ((size_t)nx * ny));
        ox[o] = x; oy[o] = y; oz[o] = z;
    }
}

void aabb_of(const fl_geometry_desc& d, float* b) {
    float lo[3], hi[3];
    switch (d.type) {
        case FL_GEOM_SPHERE:
            for (int a = 0; a < 3; ++a) { lo[a] = -d.radius; hi[a] = d.radius; }
            break;
        case FL_GEOM_BOX:
            lo[0] = -d.width / 2; hi[0] = d.width / 2;
            lo[1] = -d.height / 2; hi[1] = d.height / 2;
            lo[2] = -d.length / 2; hi[2] = d.length / 2;
            break;
        case FL_GEOM_CYLINDER:
            lo[0] = -d.radius; hi[0] = d.radius;
            lo[1] = -d.height / 2; hi[1] = d.height / 2;
            lo[2] = -d.radius; hi[2] = d.radius;
            break;
        default:
            for (int a = 0; a < 3; ++a) { lo[a] = -0.5f; hi[a] = 0.5f; }
    }
    for (int a = 0; a < 3; ++a) {
        lo[a] *= d.scale[a];
        hi[a] *= d.scale[a];
        b[a] = lo[a] + d.translate[a];
        b[3 + a] = hi[a] + d.translate[a];
    }
}

bool valid_desc(const fl_geometry_desc* d) {
    return d && d->type >= FL_GEOM_STL && d->type <= FL_GEOM_CYLINDER && d->scale[0] > 0 && d->scale[1] > 0 &&
           d->scale[2] > 0;
}

// Compacts the flagged cells of a grid range into device outputs (z, y, x order).
int compact_grid(fl_ctx* ctx, uint32_t* flag, size_t nv, int x0, int y0, int z0, int nx, int ny, size_t cap,
                 int32_t* ox, int32_t* oy, int32_t* oz, size_t* count) {
    uint32_t* off = nullptr;
    uint32_t* dtot = nullptr;
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&off, nv * 4 + 256, ctx->stream), "geometry offsets");
    dtot = off + ((nv + 63) / 64) * 64;
    int rc = fl_scan_exclusive_u32(ctx, flag, off, nv, dtot);
    if (rc) { cudaFreeAsync(off, ctx->stream); return rc; }
    k_grid_scatter<<<fl_blocks(nv, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(flag, off, nv, x0, y0, z0, nx, ny,
                                                                                  cap, ox, oy, oz);
    FL_CHECK_LAUNCH(ctx, "k_grid_scatter");
    uint32_t tot = 0;
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(&tot, dtot, 4, cudaMemcpyDeviceToHost, ctx->stream), "geometry count");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "geometry count");
    cudaFreeAsync(off, ctx->stream);
    *count = tot;
    if (tot > cap) return fl_set_error(ctx, FL_E_CAPACITY, "geometry: more cells than the output holds");
    return FL_OK;
}

int grid_range(fl_ctx* ctx, const float* lo, const float* hi, float cell, bool inclusive, int* o, int* ext,
               size_t* nv) {
    for (int a = 0; a < 3; ++a) {
        const double s = std::floor((double)(lo[a] / cell)), e = std::ceil((double)(hi[a] / cell));
        if (s < -(1 << 30) || e > (1 << 30)) return fl_set_error(ctx, FL_E_INVALID_ARG, "geometry: grid range too large");
        o[a] = (int)s;
        ext[a] = (int)e - (int)s + (inclusive ? 1 : 0);
        if (ext[a] < 0) ext[a] = 0;
    }
    *nv = (size_t)ext[0] * ext[1] * ext[2];
    if (*nv > ((size_t)1 << 32)) return fl_set_error(ctx, FL_E_INVALID_ARG, "geometry: more than 2^32 voxels");
    return FL_OK;
}

// Material id and hilbert::encode(x, y, z) at the default level 8 of each
// placed cell (GeometryPlacer.cpp:86-90), with the host codec (the reference's
// truncation of negative or wide coordinates included).
int material_and_keys(fl_ctx* ctx, int32_t material_id, const int32_t* x, const int32_t* y, const int32_t* z,
                      size_t n, int32_t* material, uint64_t* key) {
    if (!n || (!material && !key)) return FL_OK;
    std::vector<int32_t> hx(n), hy(n), hz(n), mat(n, material_id);
    std::vector<uint64_t> k(n);
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(hx.data(), x, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "cells");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(hy.data(), y, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "cells");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(hz.data(), z, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "cells");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cells");
    for (size_t i = 0; i < n; ++i) k[i] = fl_hilbert_encode_host(hx[i], hy[i], hz[i], 8);
    if (material)
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(material, mat.data(), n * 4, cudaMemcpyHostToDevice, ctx->stream), "material");
    if (key) FL_TRY_CUDA(ctx, cudaMemcpyAsync(key, k.data(), n * 8, cudaMemcpyHostToDevice, ctx->stream), "keys");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cells");
    return FL_OK;
}

}  // namespace

extern "C" {

int fl_geometry_aabb(const fl_geometry_desc* d, float* box6) {
    if (!valid_desc(d) || !box6) return FL_E_INVALID_ARG;
    aabb_of(*d, box6);
    return FL_OK;
}

int fl_geometry_inside(fl_ctx* ctx, const fl_geometry_desc* d, const float* x, const float* y, const float* z,
                       size_t n, uint8_t* inside) {
    if (!ctx || !valid_desc(d) || (n && (!x || !y || !z || !inside))) return FL_E_INVALID_ARG;
    if (!n) return FL_OK;
    k_geom_points<<<fl_blocks(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(to_dev(*d), x, y, z, n, inside);
    FL_CHECK_LAUNCH(ctx, "k_geom_points");
    return FL_OK;
}

int fl_geometry_evaluate(fl_ctx* ctx, const fl_geometry_desc* d, const int32_t* x, const int32_t* y,
                         const int32_t* z, size_t n, uint8_t* inside) {
    if (!ctx || !valid_desc(d) || (n && (!x || !y || !z || !inside))) return FL_E_INVALID_ARG;
    if (!n) return FL_OK;
    k_geom_cells<<<fl_blocks(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(to_dev(*d), x, y, z, n, inside);
    FL_CHECK_LAUNCH(ctx, "k_geom_cells");
    return FL_OK;
}

int fl_stl_voxelize(fl_ctx* ctx, const float* tris, size_t ntri, const fl_geometry_desc* d, float cell_size,
                    int32_t* x, int32_t* y, int32_t* z, size_t cap, size_t* count) {
    if (!ctx || !valid_desc(d) || !count || !(cell_size > 0.0f) || (ntri && !tris)) return FL_E_INVALID_ARG;
    *count = 0;
    if (!ntri) return FL_OK;
    // triangles with their bounds; mesh bounds (loadBinarySTL / loadAsciiSTL bookkeeping)
    std::vector<float> t(ntri * kTri);
    float mb[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (size_t k = 0; k < ntri; ++k) {
        const float* v = tris + k * 9;
        float* o = t.data() + k * kTri;
        for (int j = 0; j < 9; ++j) o[j] = v[j];
        for (int a = 0; a < 3; ++a) {
            o[9 + a] = std::min({v[a], v[3 + a], v[6 + a]});
            o[12 + a] = std::max({v[a], v[3 + a], v[6 + a]});
            mb[a] = std::min(mb[a], o[9 + a]);
            mb[3 + a] = std::max(mb[3 + a], o[12 + a]);
        }
    }
    // transformed bounds -> grid range, inclusive (SimpleSTLVoxelizer.cpp:124-141)
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = mb[a] * d->scale[a] + d->translate[a];
        hi[a] = mb[3 + a] * d->scale[a] + d->translate[a];
    }
    int o[3], e[3];
    size_t nv = 0;
    int rc = grid_range(ctx, lo, hi, cell_size, true, o, e, &nv);
    if (rc || !nv) return rc;
    float* dt = nullptr;
    uint32_t* flag = nullptr;
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&dt, t.size() * 4 + 32, ctx->stream), "triangles");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&flag, nv * 4, ctx->stream), "voxel flags");
    float* dmb = dt + t.size();
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(dt, t.data(), t.size() * 4, cudaMemcpyHostToDevice, ctx->stream), "triangles");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(dmb, mb, 24, cudaMemcpyHostToDevice, ctx->stream), "mesh bounds");
    k_stl_voxels<<<fl_blocks(nv, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
        dt, (uint32_t)ntri, dmb, to_dev(*d), cell_size, o[0], o[1], o[2], e[0], e[1], nv, flag);
    FL_CHECK_LAUNCH(ctx, "k_stl_voxels");
    rc = compact_grid(ctx, flag, nv, o[0], o[1], o[2], e[0], e[1], cap, x, y, z, count);
    cudaFreeAsync(dt, ctx->stream);
    cudaFreeAsync(flag, ctx->stream);
    return rc;
}

int fl_geometry_process(fl_ctx* ctx, const fl_geometry_desc* d, const float* tris, size_t ntri, float cell_size,
                        const float* domain_box6, int32_t* x, int32_t* y, int32_t* z, int32_t* material,
                        uint64_t* key, size_t cap, size_t* count) {
    if (!ctx || !valid_desc(d) || !count || !(cell_size > 0.0f) || !domain_box6) return FL_E_INVALID_ARG;
    *count = 0;
    if (d->type == FL_GEOM_STL) {
        int rc = fl_stl_voxelize(ctx, tris, ntri, d, cell_size, x, y, z, cap, count);
        if (rc) return rc;
        return material_and_keys(ctx, d->material_id, x, y, z, *count, material, key);
    }
    // implicit: the transformed AABB clipped to the domain, cells [floor, ceil) (generateCandidates)
    float b[6];
    aabb_of(*d, b);
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = std::max(b[a], domain_box6[a]);
        hi[a] = std::min(b[3 + a], domain_box6[3 + a]);
    }
    int o[3], e[3];
    size_t nv = 0;
    int rc = grid_range(ctx, lo, hi, cell_size, false, o, e, &nv);
    if (rc || !nv) return rc;
    uint32_t* flag = nullptr;
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&flag, nv * 4, ctx->stream), "candidate flags");
    k_implicit_candidates<<<fl_blocks(nv, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(to_dev(*d), o[0], o[1], o[2],
                                                                                        e[0], e[1], nv, flag);
    FL_CHECK_LAUNCH(ctx, "k_implicit_candidates");
    rc = compact_grid(ctx, flag, nv, o[0], o[1], o[2], e[0], e[1], cap, x, y, z, count);
    cudaFreeAsync(flag, ctx->stream);
    if (rc) return rc;
    return material_and_keys(ctx, d->material_id, x, y, z, *count, material, key);
}

}  // extern "C"
