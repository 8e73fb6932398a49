// keys.cu — 12-state Hilbert key encode/decode, the 8-level AMR key, cell keys.
//
// The 12-state table is the reference's (src/core/hilbert/HilbertCodec.cpp:13-42,
// entry = next_state << 3 | output); bit-exact keys need its values.  On the
// GPU the table is expanded once per CTA into a 3-levels-at-a-time table in
// shared memory (12 states x 512 inputs, entry = next_state << 9 | 9 output
// bits), so a 21-level key takes 7 dependent lookups instead of 21.
#include "common.cuh"
#include "keys.cuh"

namespace {
constexpr unsigned kThreads = 256;
}  // namespace

namespace {

__global__ void __launch_bounds__(kThreads) k_hilbert_encode(const int32_t* __restrict__ x,
                                                             const int32_t* __restrict__ y,
                                                             const int32_t* __restrict__ z, int level,
                                                             uint64_t* __restrict__ keys,
                                                             uint32_t* __restrict__ ids, size_t n) {
    __shared__ uint8_t t1[96];
    __shared__ uint16_t t3c[12 * 512];
    fl_keys_fill_tables_cat(t1, t3c);
    __syncthreads();
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        keys[i] = fl_hilbert_encode_cat(t1, t3c, (uint32_t)__ldg(x + i), (uint32_t)__ldg(y + i),
                                        (uint32_t)__ldg(z + i), level);
        if (ids) ids[i] = (uint32_t)i;
    }
}

// hilbert::decode (HilbertCodec.cpp:82-115).
__global__ void __launch_bounds__(kThreads) k_hilbert_decode(const uint64_t* __restrict__ keys, int level,
                                                             int32_t* __restrict__ x, int32_t* __restrict__ y,
                                                             int32_t* __restrict__ z, size_t n) {
    __shared__ uint8_t t1[96];
    __shared__ uint16_t t3[12 * 512];
    fl_keys_fill_tables(t1, t3, true);
    __syncthreads();
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (level == 0) { x[i] = y[i] = z[i] = 0; continue; }
        uint64_t t = keys[i] << (64 - level * 3);
        // walk the key MSB first; r single levels then triples
        uint64_t quads = 0;  // collected 3-bit quadrants, MSB level first
        unsigned s = 0;
        int r = level % 3;
        int done = 0;
        for (int k = 0; k < r; ++k) {
            unsigned c = (unsigned)(t >> 61) & 7u;
            unsigned v = t1[s * 8 + c];
            quads = (quads << 3) | (v & 7u);
            s = v >> 3;
            t <<= 3;
            ++done;
        }
        while (done < level) {
            unsigned c = (unsigned)(t >> 55) & 511u;
            unsigned v = t3[s * 512 + c];
            quads = (quads << 9) | (v & 511u);
            s = v >> 9;
            t <<= 9;
            done += 3;
        }
        x[i] = (int32_t)compact3(quads);
        y[i] = (int32_t)compact3(quads >> 1);
        z[i] = (int32_t)compact3(quads >> 2);
    }
}

// adaptation::hilbert_encode_3d(x, y, z, 8): interleave of bits 7..0
// (x -> bit 0, y -> bit 1, z -> bit 2 of each triple); the rotation tables of
// HilbertCodec3D.cpp:7-27 never leave the identity row.
__global__ void __launch_bounds__(kThreads) k_morton8(const int32_t* __restrict__ x, const int32_t* __restrict__ y,
                                                      const int32_t* __restrict__ z, uint64_t* __restrict__ keys,
                                                      size_t n) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        keys[i] = interleave3((uint32_t)x[i] & 255u, (uint32_t)y[i] & 255u, (uint32_t)z[i] & 255u);
}

__global__ void __launch_bounds__(kThreads) k_cell_keys(const int32_t* __restrict__ x, const int32_t* __restrict__ y,
                                                        const int32_t* __restrict__ z,
                                                        const uint8_t* __restrict__ level,
                                                        const uint16_t* __restrict__ cs, int depth, int anchor_level,
                                                        uint64_t* __restrict__ keys, size_t n) {
    __shared__ uint8_t t1[96];
    __shared__ uint16_t t3c[12 * 512];
    fl_keys_fill_tables_cat(t1, t3c);
    __syncthreads();
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        int sh = anchor_level - (int)level[i];
        uint64_t k = fl_hilbert_encode_cat(t1, t3c, (uint32_t)x[i] << sh, (uint32_t)y[i] << sh,
                                           (uint32_t)z[i] << sh, depth);
        if (cs) k |= (uint64_t)cs[i] << (3 * depth);
        keys[i] = k;
    }
}

}  // namespace

int fl_launch_cell_keys(fl_ctx* ctx, const int32_t* x, const int32_t* y, const int32_t* z, const uint8_t* level,
                        const uint16_t* cs, int depth, int anchor_level, uint64_t* keys, size_t n) {
    if (n == 0) return FL_OK;
    unsigned blocks = fl_blocks(n, kThreads, (unsigned)ctx->num_sms * 8);
    k_cell_keys<<<blocks, kThreads, 0, ctx->stream>>>(x, y, z, level, cs, depth, anchor_level, keys, n);
    FL_CHECK_LAUNCH(ctx, "k_cell_keys");
    return FL_OK;
}

extern "C" {

int fl_hilbert_encode(fl_ctx* ctx, const int32_t* x, const int32_t* y, const int32_t* z, uint8_t level,
                      uint64_t* keys, uint32_t* ids, size_t n) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (n == 0) return FL_OK;
    if (!x || !y || !z || !keys || level > 21)
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_hilbert_encode: null pointer or level > 21");
    unsigned blocks = fl_blocks(n, kThreads, (unsigned)ctx->num_sms * 8);
    k_hilbert_encode<<<blocks, kThreads, 0, ctx->stream>>>(x, y, z, level, keys, ids, n);
    FL_CHECK_LAUNCH(ctx, "k_hilbert_encode");
    return FL_OK;
}

int fl_hilbert_decode(fl_ctx* ctx, const uint64_t* keys, uint8_t level, int32_t* x, int32_t* y, int32_t* z,
                      size_t n) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (n == 0) return FL_OK;
    if (!x || !y || !z || !keys || level > 21)
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_hilbert_decode: null pointer or level > 21");
    unsigned blocks = fl_blocks(n, kThreads, (unsigned)ctx->num_sms * 8);
    k_hilbert_decode<<<blocks, kThreads, 0, ctx->stream>>>(keys, level, x, y, z, n);
    FL_CHECK_LAUNCH(ctx, "k_hilbert_decode");
    return FL_OK;
}

int fl_morton8_encode(fl_ctx* ctx, const int32_t* x, const int32_t* y, const int32_t* z, uint64_t* keys,
                      size_t n) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (n == 0) return FL_OK;
    if (!x || !y || !z || !keys) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_morton8_encode: null pointer");
    unsigned blocks = fl_blocks(n, kThreads, (unsigned)ctx->num_sms * 16);
    k_morton8<<<blocks, kThreads, 0, ctx->stream>>>(x, y, z, keys, n);
    FL_CHECK_LAUNCH(ctx, "k_morton8");
    return FL_OK;
}

int fl_cell_keys(fl_ctx* ctx, const int32_t* x, const int32_t* y, const int32_t* z, const uint8_t* level,
                 const uint16_t* case_id, int depth, int anchor_level, uint64_t* keys, size_t n) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (n == 0) return FL_OK;
    if (!x || !y || !z || !level || !keys || depth < 1 || depth > 21 || anchor_level < 0 || anchor_level > 21 ||
        (case_id && depth > 17))
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_cell_keys: bad pointer, depth or anchor level");
    return fl_launch_cell_keys(ctx, x, y, z, level, case_id, depth, anchor_level, keys, n);
}

// Host restatement of the same codec for host-side callers (CellCoord-style use).
static const uint8_t h_enc[12][8] = {
    {8, 17, 27, 18, 47, 38, 28, 37},   {16, 71, 1, 62, 51, 52, 2, 61},
    {0, 75, 95, 76, 9, 10, 86, 85},    {4, 77, 55, 78, 3, 66, 80, 65},
    {50, 49, 45, 46, 67, 88, 68, 7},   {6, 57, 39, 72, 5, 58, 84, 83},
    {12, 11, 29, 90, 79, 32, 30, 89},  {74, 91, 73, 40, 69, 92, 70, 15},
    {14, 13, 81, 82, 63, 36, 24, 35},  {20, 31, 19, 56, 53, 54, 42, 41},
    {26, 93, 43, 44, 25, 94, 64, 23},  {22, 87, 21, 60, 33, 48, 34, 59},
};
static const uint8_t h_dec[12][8] = {
    {8, 17, 19, 26, 30, 39, 37, 44},   {16, 2, 6, 52, 53, 63, 59, 65},
    {0, 12, 13, 73, 75, 87, 86, 90},   {86, 71, 69, 4, 0, 73, 75, 50},
    {93, 49, 48, 68, 70, 42, 43, 7},   {75, 57, 61, 87, 86, 4, 0, 34},
    {37, 95, 91, 9, 8, 26, 30, 76},    {43, 74, 72, 89, 93, 68, 70, 15},
    {30, 82, 83, 39, 37, 9, 8, 60},    {59, 47, 46, 18, 16, 52, 53, 25},
    {70, 28, 24, 42, 43, 89, 93, 23},  {53, 36, 38, 63, 59, 18, 16, 81},
};

uint64_t fl_hilbert_encode_host(int32_t x, int32_t y, int32_t z, uint8_t level) {
    const uint32_t m = (1u << 21) - 1;
    uint32_t ux = (uint32_t)x & m, uy = (uint32_t)y & m, uz = (uint32_t)z & m;
    uint64_t h = 0;
    unsigned s = 0;
    for (int i = (int)level - 1; i >= 0; --i) {
        unsigned q = (((uz >> i) & 1u) << 2) | (((uy >> i) & 1u) << 1) | ((ux >> i) & 1u);
        unsigned v = h_enc[s][q];
        h = (h << 3) | (v & 7u);
        s = v >> 3;
    }
    unsigned shift = (unsigned)(uint8_t)(64 - level * 3);
    if (shift < 64) { h <<= shift; h >>= shift; }
    return h;
}

void fl_hilbert_decode_host(uint64_t key, uint8_t level, int32_t* x, int32_t* y, int32_t* z) {
    if (level == 0) { *x = *y = *z = 0; return; }
    uint64_t t = key << (64 - level * 3);
    uint32_t ux = 0, uy = 0, uz = 0;
    unsigned s = 0;
    for (int l = 0; l < level; ++l) {
        unsigned v = h_dec[s][(t >> 61) & 7u];
        unsigned q = v & 7u;
        s = v >> 3;
        ux = (ux << 1) | (q & 1u);
        uy = (uy << 1) | ((q >> 1) & 1u);
        uz = (uz << 1) | ((q >> 2) & 1u);
        t <<= 3;
    }
    *x = (int32_t)ux; *y = (int32_t)uy; *z = (int32_t)uz;
}

uint64_t fl_hilbert_get_parent(uint64_t key, uint8_t level) { return level == 0 ? FL_EMPTY_KEY : key >> 3; }

uint64_t fl_hilbert_get_child(uint64_t key, uint8_t level, uint8_t quadrant) {
    if (level >= 21 || quadrant > 7) return FL_EMPTY_KEY;
    return (key << 3) | quadrant;
}

int fl_hilbert_is_valid(uint64_t key, uint8_t level) {
    if (key == FL_EMPTY_KEY) return 0;
    if (key & (1ull << 63)) return 0;
    unsigned unused = (unsigned)(uint8_t)(64 - level * 3);
    if (unused > 0 && unused < 64 && (key >> (level * 3))) return 0;
    return 1;
}

}  // extern "C"
