// keys.cuh — device-side key codec pieces shared by the kernels that need keys.
// The 12-state table values are the reference's (src/core/hilbert/HilbertCodec.cpp:13-42);
// bit-exact keys require them.
#pragma once
#include "common.cuh"

static __constant__ uint8_t c_enc[12][8] = {
    {8, 17, 27, 18, 47, 38, 28, 37},   {16, 71, 1, 62, 51, 52, 2, 61},
    {0, 75, 95, 76, 9, 10, 86, 85},    {4, 77, 55, 78, 3, 66, 80, 65},
    {50, 49, 45, 46, 67, 88, 68, 7},   {6, 57, 39, 72, 5, 58, 84, 83},
    {12, 11, 29, 90, 79, 32, 30, 89},  {74, 91, 73, 40, 69, 92, 70, 15},
    {14, 13, 81, 82, 63, 36, 24, 35},  {20, 31, 19, 56, 53, 54, 42, 41},
    {26, 93, 43, 44, 25, 94, 64, 23},  {22, 87, 21, 60, 33, 48, 34, 59},
};
static __constant__ uint8_t c_dec[12][8] = {
    {8, 17, 19, 26, 30, 39, 37, 44},   {16, 2, 6, 52, 53, 63, 59, 65},
    {0, 12, 13, 73, 75, 87, 86, 90},   {86, 71, 69, 4, 0, 73, 75, 50},
    {93, 49, 48, 68, 70, 42, 43, 7},   {75, 57, 61, 87, 86, 4, 0, 34},
    {37, 95, 91, 9, 8, 26, 30, 76},    {43, 74, 72, 89, 93, 68, 70, 15},
    {30, 82, 83, 39, 37, 9, 8, 60},    {59, 47, 46, 18, 16, 52, 53, 25},
    {70, 28, 24, 42, 43, 89, 93, 23},  {53, 36, 38, 63, 59, 18, 16, 81},
};


// Fill the shared tables: t1[s*8+q] (single level) and t3[s*512+w] where w
// packs three levels of input (MSB level first, 3 bits each).
// Both fills are called by every thread of the block at kernel start: the
// one-level table goes to shared memory first (scattered reads of constant
// memory serialise across a warp), then the three-level table is built from it.
static __device__ __forceinline__ void fl_keys_fill_tables(uint8_t* t1, uint16_t* t3, bool decode) {
    for (int i = threadIdx.x; i < 96; i += blockDim.x) t1[i] = decode ? c_dec[i >> 3][i & 7] : c_enc[i >> 3][i & 7];
    __syncthreads();
    for (int i = threadIdx.x; i < 12 * 512; i += blockDim.x) {
        unsigned s = i >> 9, w = i & 511, out = 0;
        for (int k = 2; k >= 0; --k) {
            unsigned q = (w >> (3 * k)) & 7u;
            unsigned v = t1[s * 8 + q];
            out = (out << 3) | (v & 7u);
            s = v >> 3;
        }
        t3[i] = (uint16_t)((s << 9) | out);
    }
}

// The three-level encode table re-indexed by concatenated coordinate bits:
// t3c[s*512 + (x3 << 6 | y3 << 3 | z3)] holds what t3 holds for the interleaved
// input of the same three levels, so an encoder reads each 9-bit step straight
// from the coordinates without interleaving them first.
static __device__ __forceinline__ void fl_keys_fill_tables_cat(uint8_t* t1, uint16_t* t3c) {
    for (int i = threadIdx.x; i < 96; i += blockDim.x) t1[i] = c_enc[i >> 3][i & 7];
    __syncthreads();
    for (int i = threadIdx.x; i < 12 * 512; i += blockDim.x) {
        unsigned s = i >> 9, out = 0;
        const unsigned x3 = (i >> 6) & 7u, y3 = (i >> 3) & 7u, z3 = i & 7u;
        for (int k = 2; k >= 0; --k) {
            unsigned q = (((z3 >> k) & 1u) << 2) | (((y3 >> k) & 1u) << 1) | ((x3 >> k) & 1u);
            unsigned v = t1[s * 8 + q];
            out = (out << 3) | (v & 7u);
            s = v >> 3;
        }
        t3c[i] = (uint16_t)((s << 9) | out);
    }
}

// hilbert::encode of the low `level` bits of x, y, z with the re-indexed table
// (same keys as fl_hilbert_encode_dev).
static __device__ __forceinline__ uint64_t fl_hilbert_encode_cat(const uint8_t* t1, const uint16_t* t3c, uint32_t x,
                                                                 uint32_t y, uint32_t z, int level) {
    uint64_t h = 0;
    unsigned s = 0;
    int i = level;
    for (int k = 0; k < level % 3; ++k) {  // leading single levels
        --i;
        unsigned q = (((z >> i) & 1u) << 2) | (((y >> i) & 1u) << 1) | ((x >> i) & 1u);
        unsigned v = t1[s * 8 + q];
        h = (h << 3) | (v & 7u);
        s = v >> 3;
    }
    while (i > 0) {
        i -= 3;
        unsigned c = (((x >> i) & 7u) << 6) | (((y >> i) & 7u) << 3) | ((z >> i) & 7u);
        unsigned v = t3c[s * 512 + c];
        h = (h << 9) | (v & 511u);
        s = v >> 9;
    }
    return h;
}

// Encoder state after the low `level` bits of x, y, z (most significant
// first): the digit of child (c & 1, c >> 1 & 1, c >> 2) of the cell (x, y, z)
// is then t1[state * 8 + c] & 7.
static __device__ __forceinline__ unsigned fl_hilbert_state_cat(const uint8_t* t1, const uint16_t* t3c, uint32_t x,
                                                                uint32_t y, uint32_t z, int level) {
    unsigned s = 0;
    int i = level;
    for (int k = 0; k < level % 3; ++k) {
        --i;
        s = t1[s * 8 + ((((z >> i) & 1u) << 2) | (((y >> i) & 1u) << 1) | ((x >> i) & 1u))] >> 3;
    }
    while (i > 0) {
        i -= 3;
        s = t3c[s * 512 + ((((x >> i) & 7u) << 6) | (((y >> i) & 7u) << 3) | ((z >> i) & 7u))] >> 9;
    }
    return s;
}

// Interleave up to 21 bits of three coordinates: bit i of x -> 3i, y -> 3i+1, z -> 3i+2.
static __device__ __forceinline__ uint64_t interleave3(uint32_t x, uint32_t y, uint32_t z) {
    auto sp = [](uint64_t v) {
        v &= 0x1FFFFFull;
        v = (v | (v << 32)) & 0x1F00000000FFFFull;
        v = (v | (v << 16)) & 0x1F0000FF0000FFull;
        v = (v | (v << 8)) & 0x100F00F00F00F00Full;
        v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
        v = (v | (v << 2)) & 0x1249249249249249ull;
        return v;
    };
    return sp(x) | (sp(y) << 1) | (sp(z) << 2);
}

static __device__ __forceinline__ uint32_t compact3(uint64_t v) {
    v &= 0x1249249249249249ull;
    v = (v ^ (v >> 2)) & 0x10C30C30C30C30C3ull;
    v = (v ^ (v >> 4)) & 0x100F00F00F00F00Full;
    v = (v ^ (v >> 8)) & 0x1F0000FF0000FFull;
    v = (v ^ (v >> 16)) & 0x1F00000000FFFFull;
    v = (v ^ (v >> 32)) & 0x1FFFFFull;
    return (uint32_t)v;
}

// hilbert::encode semantics (HilbertCodec.cpp:44-80) using the shared tables.
static __device__ __forceinline__ uint64_t fl_hilbert_encode_dev(const uint8_t* t1, const uint16_t* t3, uint32_t x, uint32_t y,
                                          uint32_t z, int level) {
    const uint32_t m = (1u << 21) - 1;
    uint64_t w = interleave3(x & m, y & m, z & m);  // 3-bit quadrant (z<<2|y<<1|x) per level
    uint64_t h = 0;
    unsigned s = 0;
    int i = level;
    int r = level % 3;
    for (int k = 0; k < r; ++k) {  // leading single levels
        --i;
        unsigned q = (unsigned)(w >> (3 * i)) & 7u;
        unsigned v = t1[s * 8 + q];
        h = (h << 3) | (v & 7u);
        s = v >> 3;
    }
    while (i > 0) {
        i -= 3;
        unsigned q = (unsigned)(w >> (3 * i)) & 511u;
        unsigned v = t3[s * 512 + q];
        h = (h << 9) | (v & 511u);
        s = v >> 9;
    }
    unsigned shift = (unsigned)(uint8_t)(64 - level * 3);
    if (shift < 64) { h <<= shift; h >>= shift; }
    return h;
}


int fl_launch_cell_keys(fl_ctx* ctx, const int32_t* x, const int32_t* y, const int32_t* z, const uint8_t* level,
                        const uint16_t* cs, int depth, int anchor_level, uint64_t* keys, size_t n);
