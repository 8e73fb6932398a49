// or_keys_prims.cpp — oracle: key codecs, sort, scan, compaction, hash table.
// TEST INFRASTRUCTURE ONLY (see oracle.h).
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

namespace {

// 12-state key tables, as published in src/core/hilbert/HilbertCodec.cpp:13-42
// (entry = next_state << 3 | output).  The key must equal the reference's bit
// for bit, so the tables are the reference's values.
const uint8_t kEnc[12][8] = {
    {8, 17, 27, 18, 47, 38, 28, 37},   {16, 71, 1, 62, 51, 52, 2, 61},
    {0, 75, 95, 76, 9, 10, 86, 85},    {4, 77, 55, 78, 3, 66, 80, 65},
    {50, 49, 45, 46, 67, 88, 68, 7},   {6, 57, 39, 72, 5, 58, 84, 83},
    {12, 11, 29, 90, 79, 32, 30, 89},  {74, 91, 73, 40, 69, 92, 70, 15},
    {14, 13, 81, 82, 63, 36, 24, 35},  {20, 31, 19, 56, 53, 54, 42, 41},
    {26, 93, 43, 44, 25, 94, 64, 23},  {22, 87, 21, 60, 33, 48, 34, 59},
};
const uint8_t kDec[12][8] = {
    {8, 17, 19, 26, 30, 39, 37, 44},   {16, 2, 6, 52, 53, 63, 59, 65},
    {0, 12, 13, 73, 75, 87, 86, 90},   {86, 71, 69, 4, 0, 73, 75, 50},
    {93, 49, 48, 68, 70, 42, 43, 7},   {75, 57, 61, 87, 86, 4, 0, 34},
    {37, 95, 91, 9, 8, 26, 30, 76},    {43, 74, 72, 89, 93, 68, 70, 15},
    {30, 82, 83, 39, 37, 9, 8, 60},    {59, 47, 46, 18, 16, 52, 53, 25},
    {70, 28, 24, 42, 43, 89, 93, 23},  {53, 36, 38, 63, 59, 18, 16, 81},
};

}  // namespace

// hilbert::encode, src/core/hilbert/HilbertCodec.cpp:44-80: mask to 21 bits,
// walk levels MSB first through the state table, then clear bits above 3*level.
extern "C" uint64_t or_hilbert_encode1(int32_t x, int32_t y, int32_t z, uint8_t level) {
    const uint32_t m = (1u << 21) - 1;
    uint32_t ux = (uint32_t)x & m, uy = (uint32_t)y & m, uz = (uint32_t)z & m;
    uint64_t h = 0;
    unsigned s = 0;
    for (int i = (int)level - 1; i >= 0; --i) {
        unsigned q = (((uz >> i) & 1u) << 2) | (((uy >> i) & 1u) << 1) | ((ux >> i) & 1u);
        unsigned v = kEnc[s][q];
        h = (h << 3) | (v & 7u);
        s = v >> 3;
    }
    unsigned shift = (unsigned)(uint8_t)(64 - level * 3);
    if (shift < 64) { h <<= shift; h >>= shift; }
    return h;
}

extern "C" void or_hilbert_encode(const int32_t* x, const int32_t* y, const int32_t* z, uint8_t level,
                                  uint64_t* keys, uint32_t* ids, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        keys[i] = or_hilbert_encode1(x[i], y[i], z[i], level);
        if (ids) ids[i] = (uint32_t)i;
    }
}

// hilbert::decode, src/core/hilbert/HilbertCodec.cpp:82-115.
extern "C" void or_hilbert_decode(const uint64_t* keys, uint8_t level, int32_t* x, int32_t* y,
                                  int32_t* z, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        if (level == 0) { x[i] = y[i] = z[i] = 0; continue; }
        uint64_t t = keys[i] << (64 - level * 3);
        uint32_t ux = 0, uy = 0, uz = 0;
        unsigned s = 0;
        for (int l = 0; l < level; ++l) {
            unsigned c = (unsigned)((t >> 61) & 7u);
            unsigned v = kDec[s][c];
            unsigned q = v & 7u;
            s = v >> 3;
            ux = (ux << 1) | (q & 1u);
            uy = (uy << 1) | ((q >> 1) & 1u);
            uz = (uz << 1) | ((q >> 2) & 1u);
            t <<= 3;
        }
        x[i] = (int32_t)ux; y[i] = (int32_t)uy; z[i] = (int32_t)uz;
    }
}

// adaptation::hilbert_encode_3d, src/adaptation/utils/HilbertCodec3D.cpp:29-53,
// called with max_level 8 (CellDescriptor.h:49-51).  Its rotation starts at 0
// and direction_table[0] is all zeros, so the rotation never leaves row 0 of
// rotation_table (the identity): the key is the plain interleave
// x->bit0, y->bit1, z->bit2 of bits 7..0 taken with arithmetic shifts.
extern "C" void or_morton8_encode(const int32_t* x, const int32_t* y, const int32_t* z, uint64_t* keys,
                                  size_t n) {
    for (size_t i = 0; i < n; ++i) {
        uint64_t h = 0;
        for (int l = 7; l >= 0; --l) {
            unsigned b = (unsigned)((x[i] >> l) & 1) | ((unsigned)((y[i] >> l) & 1) << 1) |
                         ((unsigned)((z[i] >> l) & 1) << 2);
            h = (h << 3) | b;
        }
        keys[i] = h;
    }
}

// Composite cell key used for ordering and lookup: the 12-state key of the
// cell's anchor (native << (anchor_level - level)) over `depth` levels, with
// the case id above bit 3*depth.  Single-case meshes use depth 21 -> the
// 63-bit key of hilbert::encode(anchor, 21); this is the sort key of the reference's CPU
// rebuild (AdaptationEngine.cpp:212-217) with the mixed-level Morton key
// replaced by a key that is unique per leaf (deviation: the reference key ties).
extern "C" void or_cell_keys(const int32_t* x, const int32_t* y, const int32_t* z, const uint8_t* level,
                             const uint16_t* case_id, int depth, int anchor_level, uint64_t* keys, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        int sh = anchor_level - (int)level[i];
        uint64_t k = or_hilbert_encode1(x[i] << sh, y[i] << sh, z[i] << sh, (uint8_t)depth);
        if (case_id) k |= (uint64_t)case_id[i] << (3 * depth);
        keys[i] = k;
    }
}

// Ascending stable sort of (key, value): the reference's GPU sort is a stub
// (RadixSort.cpp:72-86) and its scatter is unstable (radix_sort.cl:100); its
// CPU path sorts with std::sort (AdaptationEngine.cpp:215).  The oracle fixes
// ties by input order (stable).
extern "C" void or_sort_pairs_u64_u32(uint64_t* keys, uint32_t* vals, size_t n) {
    std::vector<uint32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
    std::vector<uint64_t> k2(n);
    std::vector<uint32_t> v2(n);
    for (size_t i = 0; i < n; ++i) { k2[i] = keys[idx[i]]; v2[i] = vals[idx[i]]; }
    std::memcpy(keys, k2.data(), n * 8);
    std::memcpy(vals, v2.data(), n * 4);
}

// Exclusive scan of uint32 (wrapping), exact for any n (the reference's
// two-level scan is exact only up to 65,536 elements, AdaptationEngine.cpp:378).
extern "C" uint32_t or_scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n) {
    uint32_t s = 0;
    for (size_t i = 0; i < n; ++i) { uint32_t v = in[i]; out[i] = s; s += v; }
    return s;
}

// CompactionEngine::compactAndPermute, src/core/hashmap/CompactionEngine.cpp:34-96:
// keep state != 0 && key != EMPTY, sort kept keys (stably), perm[old] = new,
// INVALID (0xFFFFFFFF) for dropped entries.
extern "C" size_t or_compact_and_permute(const uint64_t* keys, const uint32_t* state, size_t n,
                                         uint32_t* perm) {
    std::vector<uint64_t> k;
    std::vector<uint32_t> v;
    for (size_t i = 0; i < n; ++i)
        if (state[i] != 0 && keys[i] != ~0ull) { k.push_back(keys[i]); v.push_back((uint32_t)i); }
    for (size_t i = 0; i < n; ++i) perm[i] = 0xFFFFFFFFu;
    or_sort_pairs_u64_u32(k.data(), v.data(), k.size());
    for (size_t j = 0; j < k.size(); ++j) perm[v[j]] = (uint32_t)j;
    return k.size();
}

// applyPermutationToFields (CompactionEngine.cpp:98-112, a stub in the
// reference): dst[perm[i]] = src[i] for perm[i] != INVALID.
extern "C" void or_apply_permutation(const void* src, void* dst, size_t elem, size_t old_n,
                                     const uint32_t* perm) {
    const char* s = (const char*)src;
    char* d = (char*)dst;
    for (size_t i = 0; i < old_n; ++i)
        if (perm[i] != 0xFFFFFFFFu) std::memcpy(d + (size_t)perm[i] * elem, s + i * elem, elem);
}

// HashTableManager::computeCapacity, src/core/hashmap/HashTableManager.cpp:47-57.
extern "C" uint64_t or_hash_capacity(size_t n) {
    double minc = (double)n / 0.6f;
    uint32_t lg = n ? (uint32_t)std::ceil(std::log2(minc)) : 0u;
    lg = std::max<uint32_t>(lg, 20u);
    lg = std::min<uint32_t>(lg, 30u);
    return 1ull << lg;
}

namespace {
const int kProbeLimit = 256;
inline uint64_t slot_of(uint64_t key, uint64_t cap) {
    // Fibonacci hashing takes the HIGH bits of key * 2^64/phi.  The reference
    // masks the low bits (hash_build.cl:23-25), which for 12-state keys of
    // coarse anchors collapse to a handful of slots; see the hash table notes.
    int lg = 0;
    while ((1ull << lg) < cap) ++lg;
    uint64_t h = key * 0x9e3779b97f4a7c15ull;
    return lg ? (h >> (64 - lg)) : 0;
}
}  // namespace

// hash_build, kernels/hashmap/hash_build.cl:19-67: open addressing, linear
// probing, a repeated key overwrites the value (the last input wins, which is
// the sequential order of insertion).  Returns the number of keys that did not
// fit within the probe limit (the reference drops them silently).
extern "C" int or_hash_build(const uint64_t* keys, const uint32_t* vals, size_t n, uint64_t cap,
                             uint64_t* tk, uint32_t* tv) {
    for (uint64_t i = 0; i < cap; ++i) { tk[i] = ~0ull; tv[i] = 0xFFFFFFFFu; }
    int overflow = 0;
    for (size_t i = 0; i < n; ++i) {
        uint64_t k = keys[i];
        if (k == ~0ull) continue;
        uint64_t s = slot_of(k, cap);
        int p = 0;
        for (; p < kProbeLimit; ++p) {
            if (tk[s] == ~0ull) { tk[s] = k; tv[s] = vals[i]; break; }
            if (tk[s] == k) { tv[s] = vals[i]; break; }
            s = (s + 1) & (cap - 1);
        }
        if (p == kProbeLimit) ++overflow;
    }
    return overflow;
}

// hash_query, kernels/hashmap/hash_query.cl:22-56.
extern "C" void or_hash_query(const uint64_t* tk, const uint32_t* tv, uint64_t cap, const uint64_t* q,
                              uint32_t* out, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        uint64_t k = q[i];
        out[i] = 0xFFFFFFFFu;
        if (k == ~0ull) continue;
        uint64_t s = slot_of(k, cap);
        for (int p = 0; p < kProbeLimit; ++p) {
            if (tk[s] == k) { out[i] = tv[s]; break; }
            if (tk[s] == ~0ull) break;
            s = (s + 1) & (cap - 1);
        }
    }
}
