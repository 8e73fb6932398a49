// ghost.cu — same-GPU ghost pack / unpack, coarse->fine interpolation and
// fine->coarse restriction over cell fields (AoS, C floats per cell).
//
// Replaces the halo kernels of the reference, which do not compile as OpenCL
// (kernels/halo/pack.cl:4-5, interpolate_trilinear.cl:4,38-42):
//  * pack_fields / unpack_fields (kernels/halo_pack.cl:3-45): a float field
//    copied to / from a byte buffer at a byte offset;
//  * pack_halo (kernels/halo/pack.cl:8-52): gather listed cells' components
//    into a pack buffer, optionally by coarse->fine interpolation;
//  * unpack_halo / volume_weighted_average (kernels/halo/unpack.cl,
//    interpolate_average.cl:12-32): scatter pre-averaged values back;
//  * trilinear_interpolate (interpolate_trilinear.cl:12-56 with
//    TrilinearParams::initializeDefault, InterpolationParams.h:34-43): coarse =
//    fine / 2, 8 corners coarse + {0,1}^3 in corner order, weight 0.125 each,
//    missing corners contribute nothing (corner cells looked up exactly at the
//    coarser level through the hash table);
//  * restriction of sibling groups (merge_fields, merge_cells.cl:123-159, in
//    the summation order of FieldAveragingRules.h:31-52).
#include "common.cuh"
#include "amr.cuh"
#include "hash.cuh"
#include "keys.cuh"

namespace {

__global__ void k_pack_fields(const float* __restrict__ field, uint8_t* __restrict__ packed, size_t n, size_t off) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float v = field[i];
        memcpy(packed + off + i * 4, &v, 4);
    }
}

__global__ void k_unpack_fields(const uint8_t* __restrict__ packed, float* __restrict__ field, size_t n, size_t off) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float v;
        memcpy(&v, packed + off + i * 4, 4);
        field[i] = v;
    }
}

// Row kernels: a warp covers 32 / C rows (one row when C > 16), lane j the
// column j % C of row j / C, so every row is read and written by one warp
// instruction (its two or three sectors fetched once) and the index math is
// 32-bit per row.  Rows of up to 32 columns move kRowUnroll row groups per
// warp round, their index and value loads issued together (random rows need
// many bytes in flight); wider rows one group at a time.
constexpr int kRowUnroll = 8;

template <bool SCATTER>
__global__ void k_move_rows(const float* __restrict__ src, uint32_t C, const uint32_t* __restrict__ idx, size_t n,
                            float* __restrict__ dst) {
    const uint32_t lane = threadIdx.x & 31u, rpw = C <= 32u ? 32u / C : 1u;
    const uint32_t r = C <= 32u ? lane / C : 0u, c = lane - r * C;
    const bool on = r < rpw;
    const size_t nw = ((size_t)gridDim.x * blockDim.x) >> 5;
    const size_t per_round = (size_t)rpw * kRowUnroll;
    for (size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * per_round < n; w += nw) {
        const size_t k0 = w * per_round + r;
        if (C <= 32u) {
            uint32_t id[kRowUnroll];
            float v[kRowUnroll];
#pragma unroll
            for (int u = 0; u < kRowUnroll; ++u) {
                const size_t k = k0 + (size_t)u * rpw;
                id[u] = on && k < n ? idx[k] : 0u;
            }
#pragma unroll
            for (int u = 0; u < kRowUnroll; ++u) {
                const size_t k = k0 + (size_t)u * rpw;
                v[u] = on && k < n ? (SCATTER ? src[k * C + c] : src[(size_t)id[u] * C + c]) : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < kRowUnroll; ++u) {
                const size_t k = k0 + (size_t)u * rpw;
                if (on && k < n) {
                    if (SCATTER) dst[(size_t)id[u] * C + c] = v[u];
                    else dst[k * C + c] = v[u];
                }
            }
        } else {
            for (int u = 0; u < kRowUnroll; ++u) {
                const size_t k = k0 + (size_t)u;
                if (k >= n) break;
                const size_t row = idx[k];
                const float* s = SCATTER ? src + k * C : src + row * C;
                float* d = SCATTER ? dst + row * C : dst + k * C;
                for (uint32_t j = lane; j < C; j += 32u) d[j] = s[j];
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_interp(fl_mesh_dev m, fl_domain_dev dom, const uint64_t* __restrict__ tk,
                                                const uint32_t* __restrict__ tv, int lg, const float* __restrict__ field,
                                                uint32_t C, const int32_t* __restrict__ fx, const int32_t* __restrict__ fy,
                                                const int32_t* __restrict__ fz, const uint8_t* __restrict__ flevel,
                                                size_t nq, float* __restrict__ out) {
    __shared__ uint8_t t1[96];
    __shared__ uint16_t t3[12 * 512];
    fl_keys_fill_tables(t1, t3, false);
    __syncthreads();
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += stride) {
        float* o = out + i * C;
        for (uint32_t c = 0; c < C; ++c) o[c] = 0.0f;
        if (flevel[i] == 0) continue;
        int l = flevel[i] - 1;
        int32_t cx = fx[i] / 2, cy = fy[i] / 2, cz = fz[i] / 2;
        int sh = dom.anchor_level - l;
        for (int k = 0; k < 8; ++k) {
            int64_t p[3] = {cx + (k & 1), cy + ((k >> 1) & 1), cz + ((k >> 2) & 1)};
            if (p[0] < 0 || p[1] < 0 || p[2] < 0) continue;
            uint64_t key = fl_anchor_key(t1, t3, dom.depth, 0, false, p[0] << sh, p[1] << sh, p[2] << sh);
            const uint32_t hv = fl_hash_lookup(tk, tv, lg, key);
            if (hv == FL_INVALID_INDEX || fl_packed_level(hv) != l) continue;
            const uint32_t j = fl_packed_idx(hv);
            const float* v = field + (size_t)j * C;
            for (uint32_t c = 0; c < C; ++c) o[c] = __fadd_rn(o[c], __fmul_rn(0.125f, v[c]));
        }
    }
}

// Restriction, laid out like the row kernels (a warp per 32 / C groups).
__global__ void k_restrict(const float* __restrict__ field, uint32_t C, const uint32_t* __restrict__ members,
                           size_t G, int rule, float* __restrict__ out) {
    const uint32_t lane = threadIdx.x & 31u, rpw = C <= 32u ? 32u / C : 1u;
    const uint32_t r = lane / C, c = lane - r * C;
    const size_t nw = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * rpw < G; w += nw) {
        const size_t g = w * rpw + r;
        if (r >= rpw || g >= G) continue;
        uint32_t mem[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) mem[q] = members[g * 8 + q];
        for (uint32_t j = c; j < C; j += 32u) {
            float s = 0.0f;
#pragma unroll
            for (int q = 0; q < 8; ++q) s = __fadd_rn(s, field[(size_t)mem[q] * C + j]);
            out[g * C + j] = rule == 1 ? s : __fmul_rn(s, 0.125f);
        }
    }
}

// Blocks for the row kernels: 8 warps a block, a warp per 32 / C rows.
unsigned row_blocks(fl_ctx* ctx, size_t n, uint32_t C) {
    const size_t rpw = C <= 32u ? 32u / C : 1u;
    return fl_blocks((n + rpw - 1) / rpw * 32, 256, ctx->num_sms * 8);
}

}  // namespace

extern "C" {

int fl_pack_fields(fl_ctx* ctx, const float* field, void* packed, size_t num_cells, size_t field_offset_bytes) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (!num_cells) return FL_OK;
    if (!field || !packed || (field_offset_bytes & 3))
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_pack_fields: null pointer or unaligned offset");
    k_pack_fields<<<fl_blocks(num_cells, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(field, (uint8_t*)packed,
                                                                                      num_cells, field_offset_bytes);
    FL_CHECK_LAUNCH(ctx, "k_pack_fields");
    return FL_OK;
}

int fl_unpack_fields(fl_ctx* ctx, const void* packed, float* field, size_t num_cells, size_t field_offset_bytes) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (!num_cells) return FL_OK;
    if (!field || !packed || (field_offset_bytes & 3))
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_unpack_fields: null pointer or unaligned offset");
    k_unpack_fields<<<fl_blocks(num_cells, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>((const uint8_t*)packed, field,
                                                                                        num_cells, field_offset_bytes);
    FL_CHECK_LAUNCH(ctx, "k_unpack_fields");
    return FL_OK;
}

int fl_pack_halo(fl_ctx* ctx, const float* field, uint32_t C, const uint32_t* cell_indices, size_t n, float* pack) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (!n || !C) return FL_OK;
    if (!field || !cell_indices || !pack) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_pack_halo: null pointer");
    k_move_rows<false><<<row_blocks(ctx, n, C), 256, 0, ctx->stream>>>(field, C, cell_indices, n, pack);
    FL_CHECK_LAUNCH(ctx, "k_move_rows gather");
    return FL_OK;
}

int fl_unpack_halo(fl_ctx* ctx, const float* pack, uint32_t C, const uint32_t* cell_indices, size_t n, float* field) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (!n || !C) return FL_OK;
    if (!field || !cell_indices || !pack) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_unpack_halo: null pointer");
    k_move_rows<true><<<row_blocks(ctx, n, C), 256, 0, ctx->stream>>>(pack, C, cell_indices, n, field);
    FL_CHECK_LAUNCH(ctx, "k_move_rows scatter");
    return FL_OK;
}

int fl_interp_trilinear(fl_ctx* ctx, const fl_mesh* mesh, const fl_adapt_config* cfg, const float* field, uint32_t C,
                        const int32_t* fx, const int32_t* fy, const int32_t* fz, const uint8_t* flevel, size_t nq,
                        float* out) {
    if (!ctx || !mesh || !cfg) return FL_E_INVALID_ARG;
    if (!nq) return FL_OK;
    if (!field || !fx || !fy || !fz || !flevel || !out || C == 0 || C > 32)
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_interp_trilinear: bad arguments (C in 1..32)");
    if (mesh->case_id) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_interp_trilinear: single-case meshes only");
    size_t n = mesh->num_cells;
    uint64_t cap = fl_table_capacity(n ? n : 1);
    int rc = fl_scratch_reserve(ctx, 256 + fl_align256(n * 8 + 8) + fl_align256(cap * 16) + fl_align256(cap * 4));
    if (rc) return rc;
    char* p = (char*)ctx->scratch;
    void* dcase = p; p += 256;
    uint64_t* keys = (uint64_t*)p; p += fl_align256(n * 8 + 8);
    uint64_t* tk = (uint64_t*)p; p += fl_align256(cap * 16);
    uint32_t* tv = nullptr;  // 16-byte slots
    uint32_t* win = (uint32_t*)p;
    fl_domain_dev dom = fl_domain_from_config(ctx, cfg, dcase);
    if (n) {
        rc = fl_launch_cell_keys(ctx, mesh->x, mesh->y, mesh->z, mesh->level, nullptr, dom.depth, dom.anchor_level,
                                 keys, n);
        if (rc) return rc;
    }
    rc = fl_hash_build_with(ctx, tk, tv, cap, keys, nullptr, n, win, mesh->level);
    if (rc) return rc;
    fl_mesh_dev md{mesh->x, mesh->y, mesh->z, mesh->level, mesh->state, mesh->flags, mesh->material, nullptr, n};
    k_interp<<<fl_blocks(nq, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(md, dom, tk, tv, fl_hash_lg(cap), field, C,
                                                                          fx, fy, fz, flevel, nq, out);
    FL_CHECK_LAUNCH(ctx, "k_interp");
    return fl_collect_device_status(ctx, "fl_interp_trilinear");
}

int fl_restrict_groups(fl_ctx* ctx, const float* field, uint32_t C, const uint32_t* members, size_t ngroups, int rule,
                       float* out) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (!ngroups || !C) return FL_OK;
    if (!field || !members || !out) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_restrict_groups: null pointer");
    k_restrict<<<row_blocks(ctx, ngroups, C), 256, 0, ctx->stream>>>(field, C, members, ngroups, rule, out);
    FL_CHECK_LAUNCH(ctx, "k_restrict");
    return FL_OK;
}

}  // extern "C"
