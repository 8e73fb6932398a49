// hash.cu — GPU open-addressing hash table (key -> index) and the neighbour
// table rebuild built on it.
//
// Replaces HashTableManager::rebuild/query (src/core/hashmap/HashTableManager.cpp:101-159,
// which launch nothing) with the kernels they name (kernels/hashmap/hash_build.cl:19-82,
// kernels/hashmap/hash_query.cl:22-98): EMPTY key = ~0, INVALID value = ~0,
// power-of-two capacity, linear probing, a repeated key keeps the value of
// the LAST input carrying it (the order sequential insertion gives; resolved
// here with an atomicMax on the input index so the result does not depend
// on thread timing).  The slot is the high bits of key * 0x9e3779b97f4a7c15
// (Fibonacci hashing); the reference masks the low bits, which for 12-state
// keys of coarse anchors fall on a handful of slots.
#include "common.cuh"
#include "hash.cuh"
#include "keys.cuh"

namespace {

constexpr int kProbeLimit = 256;

__global__ void k_hash_clear(uint64_t* __restrict__ tk, uint32_t* __restrict__ tv, uint32_t* __restrict__ win,
                             uint64_t cap) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += stride) {
        if (tv) {
            tk[i] = FL_EMPTY_KEY;
            tv[i] = FL_INVALID_INDEX;
        } else {
            reinterpret_cast<ulonglong2*>(tk)[i] = make_ulonglong2(FL_EMPTY_KEY, FL_INVALID_INDEX);
        }
        if (win) win[i] = 0u;
    }
}

__global__ void k_hash_insert(uint64_t* __restrict__ tk, int slot_words, uint32_t* __restrict__ win, int lg,
                              const uint64_t* __restrict__ keys, size_t n, uint32_t* dev_status) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    const uint64_t mask = (1ull << lg) - 1;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t k = keys[i];
        if (k == FL_EMPTY_KEY) continue;
        uint64_t s = fl_hash_slot(k, lg);
        int p = 0;
        for (; p < kProbeLimit; ++p) {
            unsigned long long prev = atomicCAS((unsigned long long*)(tk + s * slot_words), FL_EMPTY_KEY, k);
            if (prev == FL_EMPTY_KEY || prev == k) {
                atomicMax(win + s, (uint32_t)(i + 1));
                break;
            }
            s = (s + 1) & mask;
        }
        if (p == kProbeLimit) atomicAdd(dev_status + FL_DEVSTAT_HASH_OVERFLOW, 1u);
    }
}

__global__ void k_hash_values(uint64_t* __restrict__ tk, uint32_t* __restrict__ tv, const uint32_t* __restrict__ win,
                              const uint32_t* __restrict__ vals, const uint8_t* __restrict__ levels, uint64_t cap) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += stride) {
        uint32_t w = win[i];
        if (!w) continue;
        uint32_t v;
        if (vals) v = vals[w - 1];
        else if (levels) v = ((uint32_t)levels[w - 1] << kPackedIdxBits) | (w - 1);
        else v = w - 1;
        if (tv) tv[i] = v;
        else tk[2 * i + 1] = v;
    }
}

__global__ void k_hash_query(const uint64_t* __restrict__ tk, const uint32_t* __restrict__ tv, int lg,
                             const uint64_t* __restrict__ q, uint32_t* __restrict__ out, size_t n) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = fl_hash_lookup(tk, tv, lg, q[i]);
}

__device__ __forceinline__ int fold_axis(int64_t* p, int64_t ext, int periodic) {
    if (*p < 0 || *p >= ext) {
        if (!periodic) return 0;
        *p = ((*p % ext) + ext) % ext;
    }
    return 1;
}

// nbr[(i*26 + k)*S + s] = leaf containing the probe point of direction k,
// sub-slot s; the point-location rule of balance_enforce.cl:107-143 (the cell
// whose level is l and whose anchor is the point with the low (A - l) bits
// cleared), probed outward from the cell's own level.
__global__ void __launch_bounds__(256) k_neighbours(fl_mesh_dev m, fl_domain_dev dom, const uint64_t* __restrict__ tk,
                                                    const uint32_t* __restrict__ tv, int lg, int S,
                                                    uint32_t* __restrict__ nbr, uint32_t* dev_status) {
    __shared__ uint8_t t1[96];
    __shared__ uint16_t t3[12 * 512];
    fl_keys_fill_tables(t1, t3, false);
    __syncthreads();
    size_t total = m.n * 26 * (size_t)S;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        size_t i = t / (26 * S);
        int r = (int)(t - i * 26 * S);
        int k = r / S, s = r - k * S;
        uint16_t cs = m.case_id ? m.case_id[i] : 0;
        const fl_domain_dev::Case& d = dom.c[m.case_id ? cs : 0];
        int lvl = m.level[i];
        int sh = dom.anchor_level - lvl;
        int64_t anc[3] = {(int64_t)m.x[i] << sh, (int64_t)m.y[i] << sh, (int64_t)m.z[i] << sh};
        int64_t size = (int64_t)1 << sh;
        int kk = k < 13 ? k : k + 1;
        int dv[3] = {kk % 3 - 1, (kk / 3) % 3 - 1, kk / 9 - 1};
        int64_t p[3];
        int bit = 0;
        for (int a = 0; a < 3; ++a) {
            if (dv[a] < 0) p[a] = anc[a] - 1;
            else if (dv[a] > 0) p[a] = anc[a] + size;
            else { p[a] = anc[a] + (((s >> bit) & 1) ? (size >> 1) : 0); ++bit; }
        }
        uint32_t res = FL_INVALID_INDEX;
        bool in = true;
        for (int a = 0; a < 3; ++a)
            in = in && fold_axis(&p[a], (int64_t)d.ext[a] << dom.anchor_level, d.periodic[a]);
        if (in) res = fl_locate(t1, t3, tk, tv, lg, nullptr, dom, cs, m.case_id != nullptr, p, lvl);
        nbr[t] = res;
    }
}

}  // namespace

int fl_hash_lg(uint64_t cap) {
    int lg = 0;
    while ((1ull << lg) < cap) ++lg;
    return lg;
}

int fl_hash_build_with(fl_ctx* ctx, uint64_t* tk, uint32_t* tv, uint64_t cap, const uint64_t* keys,
                       const uint32_t* vals, size_t n, uint32_t* win, const uint8_t* levels) {
    if (levels && !vals && n >= ((size_t)1 << kPackedIdxBits))
        return fl_set_error(ctx, FL_E_CAPACITY, "a mesh of 2^27 or more cells");
    unsigned cb = fl_blocks(cap, 256, ctx->num_sms * 8);
    k_hash_clear<<<cb, 256, 0, ctx->stream>>>(tk, tv, win, cap);
    FL_CHECK_LAUNCH(ctx, "k_hash_clear");
    if (n == 0) return FL_OK;
    int lg = fl_hash_lg(cap);
    k_hash_insert<<<fl_blocks(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(tk, tv ? 1 : 2, win, lg, keys, n,
                                                                                 ctx->dev_status);
    FL_CHECK_LAUNCH(ctx, "k_hash_insert");
    k_hash_values<<<cb, 256, 0, ctx->stream>>>(tk, tv, win, vals, vals ? nullptr : levels, cap);
    FL_CHECK_LAUNCH(ctx, "k_hash_values");
    return FL_OK;
}

int fl_neighbours_with(fl_ctx* ctx, const fl_mesh_dev& m, const fl_domain_dev& dom, const uint64_t* tk,
                       const uint32_t* tv, uint64_t cap, int subslots, uint32_t* nbr) {
    if (m.n == 0) return FL_OK;
    size_t total = m.n * 26 * (size_t)subslots;
    k_neighbours<<<fl_blocks(total, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(m, dom, tk, tv, fl_hash_lg(cap),
                                                                                 subslots, nbr, ctx->dev_status);
    FL_CHECK_LAUNCH(ctx, "k_neighbours");
    return FL_OK;
}

uint64_t fl_table_capacity(size_t n) {
    uint64_t c = 1024;
    while (c < 2 * (uint64_t)n) c <<= 1;
    return c;
}

extern "C" {

uint64_t fl_hash_compute_capacity(size_t n) {
    // HashTableManager::computeCapacity (HashTableManager.cpp:47-57)
    double minc = (double)n / 0.6f;
    uint32_t lg = 0;
    while (n && (double)(1ull << lg) < minc) ++lg;
    if (lg < 20) lg = 20;
    if (lg > 30) lg = 30;
    return 1ull << lg;
}

int fl_hash_build(fl_ctx* ctx, uint64_t* table_keys, uint32_t* table_vals, uint64_t capacity, const uint64_t* keys,
                  const uint32_t* vals, size_t n) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (!table_keys || !table_vals || capacity == 0 || (capacity & (capacity - 1)) || (n && !keys))
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_hash_build: bad table or capacity not a power of two");
    if (n > capacity) return fl_set_error(ctx, FL_E_CAPACITY, "fl_hash_build: more keys than slots");
    int rc = fl_scratch_reserve(ctx, capacity * 4);
    if (rc) return rc;
    rc = fl_hash_build_with(ctx, table_keys, table_vals, capacity, keys, vals, n, (uint32_t*)ctx->scratch);
    if (rc) return rc;
    return fl_collect_device_status(ctx, "fl_hash_build");
}

int fl_hash_query(fl_ctx* ctx, const uint64_t* table_keys, const uint32_t* table_vals, uint64_t capacity,
                  const uint64_t* queries, uint32_t* out, size_t n) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (n == 0) return FL_OK;
    if (!table_keys || !table_vals || !queries || !out || capacity == 0 || (capacity & (capacity - 1)))
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_hash_query: bad arguments");
    k_hash_query<<<fl_blocks(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(table_keys, table_vals,
                                                                             fl_hash_lg(capacity), queries, out, n);
    FL_CHECK_LAUNCH(ctx, "k_hash_query");
    return FL_OK;
}

}  // extern "C"
