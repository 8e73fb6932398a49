// hash.cu — GPU open-addressing hash table (key -> index) and the neighbour
// table rebuild built on it.
//
// Replaces HashTableManager::rebuild/query (src/core/hashmap/HashTableManager.cpp:101-159,
// which launch nothing) with the kernels they name (kernels/hashmap/hash_build.cl:19-82,
// kernels/hashmap/hash_query.cl:22-98): EMPTY key = ~0, INVALID value = ~0,
// power-of-two capacity, linear probing, a repeated key keeps the value of
// the LAST input carrying it (the order sequential insertion gives; resolved,
// only when a build meets repeated keys, with an atomicMax on the input index
// so the result does not depend on thread timing).  The slot is the high bits of key * 0x9e3779b97f4a7c15
// (Fibonacci hashing); the reference masks the low bits, which for 12-state
// keys of coarse anchors fall on a handful of slots.
#include "common.cuh"
#include "hash.cuh"
#include "keys.cuh"
#include "scan.cuh"

namespace {

constexpr int kProbeLimit = 256;

__global__ void k_hash_clear(uint64_t* __restrict__ tk, uint32_t* __restrict__ tv, uint64_t cap) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += stride) {
        if (tv) {
            tk[i] = FL_EMPTY_KEY;
            tv[i] = FL_INVALID_INDEX;
        } else {
            reinterpret_cast<ulonglong2*>(tk)[i] = make_ulonglong2(FL_EMPTY_KEY, FL_INVALID_INDEX);
        }
    }
}

// The value input i stores: vals[i], or (level << kPackedIdxBits) | i, or i.
__device__ __forceinline__ uint32_t hash_value_of(size_t i, const uint32_t* __restrict__ vals,
                                                  const uint8_t* __restrict__ levels) {
    if (vals) return vals[i];
    if (levels) return ((uint32_t)levels[i] << kPackedIdxBits) | (uint32_t)i;
    return (uint32_t)i;
}

__device__ __forceinline__ void hash_store_value(uint64_t* tk, uint32_t* tv, uint64_t s, uint32_t v) {
    if (tv) tv[s] = v;
    else tk[2 * s + 1] = v;
}

// Insertion: the thread whose CAS claims an empty slot stores its value with a
// plain store; a thread that finds its key already there flags the build
// (FL_DEVSTAT_HASH_DUPS) and stores nothing.  Without repeated keys that is
// the table; with them the three passes below give each repeated key the
// value of its last input.
__global__ void k_hash_insert(uint64_t* __restrict__ tk, uint32_t* __restrict__ tv, int lg,
                              const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                              const uint8_t* __restrict__ levels, size_t n, uint32_t* dev_status) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const uint64_t mask = (1ull << lg) - 1;
    const int sw = tv ? 1 : 2;
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const size_t i = base + threadIdx.x;
        bool dup = false;
        if (i < n) {
            const uint64_t k = keys[i];
            if (k != FL_EMPTY_KEY) {
                uint64_t s = fl_hash_slot(k, lg);
                int p = 0;
                for (; p < kProbeLimit; ++p) {
                    unsigned long long prev = atomicCAS((unsigned long long*)(tk + s * sw), FL_EMPTY_KEY, k);
                    if (prev == FL_EMPTY_KEY) {
                        hash_store_value(tk, tv, s, hash_value_of(i, vals, levels));
                        break;
                    }
                    if (prev == k) {
                        dup = true;
                        break;
                    }
                    s = (s + 1) & mask;
                }
                if (p == kProbeLimit) atomicAdd(dev_status + FL_DEVSTAT_HASH_OVERFLOW, 1u);
            }
        }
        if (__any_sync(0xFFFFFFFFu, dup) && (threadIdx.x & 31) == 0) atomicOr(dev_status + FL_DEVSTAT_HASH_DUPS, 1u);
    }
}

// Repeated keys only (each kernel returns at once when the build met none):
// clear the winner words, let every input take the maximum of its slot's
// winner (input index + 1), then store each claimed slot's winning value.
__global__ void k_hash_dup_clear(uint32_t* __restrict__ win, uint64_t cap, const uint32_t* dev_status) {
    if (!*(volatile const uint32_t*)(dev_status + FL_DEVSTAT_HASH_DUPS)) return;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += stride) win[i] = 0u;
}

__global__ void k_hash_dup_winners(const uint64_t* __restrict__ tk, int sw, uint32_t* __restrict__ win, int lg,
                                   const uint64_t* __restrict__ keys, size_t n, const uint32_t* dev_status) {
    if (!*(volatile const uint32_t*)(dev_status + FL_DEVSTAT_HASH_DUPS)) return;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    const uint64_t mask = (1ull << lg) - 1;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t k = keys[i];
        if (k == FL_EMPTY_KEY) continue;
        uint64_t s = fl_hash_slot(k, lg);
        for (int p = 0; p < kProbeLimit; ++p) {
            const uint64_t cur = tk[s * sw];
            if (cur == k) {
                atomicMax(win + s, (uint32_t)(i + 1));
                break;
            }
            if (cur == FL_EMPTY_KEY) break;  // not inserted (probe overflow, reported by the insertion)
            s = (s + 1) & mask;
        }
    }
}

__global__ void k_hash_dup_values(uint64_t* __restrict__ tk, uint32_t* __restrict__ tv,
                                  const uint32_t* __restrict__ win, const uint32_t* __restrict__ vals,
                                  const uint8_t* __restrict__ levels, uint64_t cap, const uint32_t* dev_status) {
    if (!*(volatile const uint32_t*)(dev_status + FL_DEVSTAT_HASH_DUPS)) return;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += stride) {
        const uint32_t w = win[i];
        if (w) hash_store_value(tk, tv, i, hash_value_of(w - 1, vals, levels));
    }
}

__global__ void k_hash_query(const uint64_t* __restrict__ tk, const uint32_t* __restrict__ tv, int lg,
                             const uint64_t* __restrict__ q, uint32_t* __restrict__ out, size_t n) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = fl_hash_lookup(tk, tv, lg, q[i]);
}

// flags[1] = the deepest leaf level.
__global__ void k_deepest(const uint8_t* __restrict__ level, size_t n, uint32_t* __restrict__ flags) {
    int deepest = 0;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        deepest = max(deepest, (int)level[i]);
    deepest = __reduce_max_sync(0xFFFFFFFFu, deepest);
    if ((threadIdx.x & 31) == 0 && deepest > 0) atomicMax(flags + 1, (uint32_t)deepest);
}

// Run start of every leaf divided by 8^cut: the anchor shifted down by cut,
// encoded at depth - cut levels, the low 3(A - l - cut) bits cleared (the case
// id above bit 3 * (depth - cut)); ids[i] = i.
__global__ void __launch_bounds__(256) k_run_keys(fl_mesh_dev m, fl_domain_dev dom, int cut,
                                                  uint64_t* __restrict__ keys, uint32_t* __restrict__ ids) {
    __shared__ uint8_t t1[96];
    __shared__ uint16_t t3c[12 * 512];
    fl_keys_fill_tables_cat(t1, t3c);
    __syncthreads();
    const int dc = dom.depth - cut;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.n; i += stride) {
        const int sh = dom.anchor_level - m.level[i];
        uint64_t k = fl_hilbert_encode_cat(t1, t3c, ((uint32_t)m.x[i] << sh) >> cut, ((uint32_t)m.y[i] << sh) >> cut,
                                           ((uint32_t)m.z[i] << sh) >> cut, dc);
        k &= ~((1ull << (3 * (sh - cut))) - 1);
        if (m.case_id) k |= (uint64_t)m.case_id[i] << (3 * dc);
        keys[i] = k;
        ids[i] = (uint32_t)i;
    }
}

// flag = 1 when some run start is smaller than the one before it.
__global__ void k_check_sorted(const uint64_t* __restrict__ keys, size_t n, uint32_t* __restrict__ flag) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x + 1; i < n; i += stride)
        bad = bad || keys[i] < keys[i - 1];
    if (__syncthreads_or(bad) && threadIdx.x == 0) *flag = 1u;
}

// dir[b] = first run whose bucket is >= b, b in [0, nb]: run i fills the
// buckets after its predecessor's up to its own.  A wide range (a gap in the
// keys, between cases say) is filled by the whole warp, so it costs 1/32 of
// its length; the buckets after the last run's (n: none starts there), up to
// a directory's worth when the keys span less than the directory (a uniform
// mesh), by the whole grid.
__global__ void k_locator_dir(const uint64_t* __restrict__ keys, size_t n, int log2nb, uint32_t* __restrict__ dir) {
    const uint64_t nb = 1ull << log2nb;
    const uint64_t k0 = keys[0], span = keys[n - 1] - k0;
    const int bits = span ? 64 - __clzll((long long)span) : 0;
    const int shift = bits > log2nb ? bits - log2nb : 0;
    const int lane = threadIdx.x & 31;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (uint64_t b = (span >> shift) + 1 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; b <= nb; b += stride)
        dir[b] = (uint32_t)n;
    for (size_t base = (size_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        const size_t i = base + lane;
        uint64_t bl = 1, bh = 0;  // empty unless i < n
        if (i < n) {
            bh = (keys[i] - k0) >> shift;
            bl = i > 0 ? ((keys[i - 1] - k0) >> shift) + 1 : 0;
        }
        // short ranges (the common case: one or two buckets) by their own lane,
        // coalesced across the warp; long ones by the whole warp
        const bool wide = bl <= bh && bh - bl >= 4;
        if (!wide)
            for (uint64_t b = bl; b <= bh; ++b) dir[b] = (uint32_t)i;
        for (unsigned w = __ballot_sync(0xFFFFFFFFu, wide); w; w &= w - 1) {
            const int j = __ffs(w) - 1;
            const uint64_t lo = __shfl_sync(0xFFFFFFFFu, bl, j), hi = __shfl_sync(0xFFFFFFFFu, bh, j);
            for (uint64_t b = lo + lane; b <= hi; b += 32) dir[b] = (uint32_t)(base + j);
        }
    }
}

// Neighbour rows in two passes over 13 directions each.  Direction k and
// 25 - k are opposite, and a same-level neighbour relation is symmetric: when
// the first pass (k < 13) finds a leaf j of cell i's own level, i is j's
// neighbour in direction 25 - k on every sub-slot, so it writes that entry of
// j's row too and marks it (bit 12 - k of marks[j]); the second pass probes
// only the unmarked directions 13..25.  Blocks of kNbrThreads: kNbrCells / S cells
// x 13 directions x S sub-slots, a cell's probes in consecutive threads; three
// blocks per SM (32 registers a thread).
constexpr int kNbrCells = 48;        // cells per block at one sub-slot
constexpr int kNbrBlocksPerSM = 3;
constexpr int kNbrThreads = kNbrCells * 13;

template <int S, bool kFirst>
__global__ void __launch_bounds__(kNbrThreads, kNbrBlocksPerSM) k_neighbours_sorted(fl_mesh_dev m, fl_domain_dev dom,
                                                                        fl_locator L, uint32_t* __restrict__ nbr,
                                                                        uint32_t* __restrict__ marks) {
    constexpr int kCells = kNbrCells / S;
    __shared__ uint8_t t1[96];
    __shared__ uint16_t t3c[12 * 512];
    fl_keys_fill_tables_cat(t1, t3c);
    __syncthreads();
    const fl_probe P = fl_probe_make(t1, t3c, L, dom);
    const int cl = threadIdx.x / (13 * S);
    const int r = threadIdx.x - cl * (13 * S);
    const int k = r / S + (kFirst ? 0 : 13), s = r % S;
    const int kk = k < 13 ? k : k + 1;
    const int dv[3] = {kk % 3 - 1, (kk / 3) % 3 - 1, kk / 9 - 1};
    for (size_t base = (size_t)blockIdx.x * kCells; base < m.n; base += (size_t)gridDim.x * kCells) {
        const size_t i = base + cl;
        if (i >= m.n) continue;
        if (!kFirst && ((marks[i] >> (k - 13)) & 1u)) continue;
        const uint16_t cs = m.case_id ? m.case_id[i] : 0;
        const fl_domain_dev::Case& d = dom.c[m.case_id ? cs : 0];
        const int lvl = m.level[i];
        const int sh = dom.anchor_level - lvl;
        const int32_t anc[3] = {m.x[i] << sh, m.y[i] << sh, m.z[i] << sh};
        const int32_t size = 1 << sh;
        int32_t p[3];
        int bit = 0;
        bool in = true;
        for (int a = 0; a < 3; ++a) {
            if (dv[a] < 0) p[a] = anc[a] - 1;
            else if (dv[a] > 0) p[a] = anc[a] + size;
            else { p[a] = anc[a] + (((s >> bit) & 1) ? (size >> 1) : 0); ++bit; }
            in = in && fl_fold32(p[a], d.ext[a] << dom.anchor_level, d.periodic[a]);
        }
        const uint32_t res =
            in ? fl_probe_point(P, m.case_id != nullptr, cs, (uint32_t)p[0], (uint32_t)p[1], (uint32_t)p[2])
               : FL_INVALID_INDEX;
        nbr[i * (26 * S) + k * S + s] = res;
        if (kFirst && res != FL_INVALID_INDEX && m.level[res] == lvl) {
            nbr[(size_t)res * (26 * S) + (25 - k) * S + s] = (uint32_t)i;
            if (s == 0) atomicOr(marks + res, 1u << (12 - k));
        }
    }
}

int locator_log2nb(size_t n) {
    int lg = 0;
    while ((1ull << lg) < n) ++lg;
    return lg > 11 ? lg + 1 : 10;  // about two buckets per run: most searches end in the directory
}

}  // namespace

size_t fl_locator_scratch_bytes(size_t n) {
    const size_t nb = (size_t)1 << locator_log2nb(n);
    return fl_align256(n * 8) + fl_align256(n * 4) + fl_align256((nb + 1) * 4) + 256 + fl_sort_scratch_bytes(n, 8);
}

uint32_t* fl_locator_ids(void* scratch, size_t n) { return (uint32_t*)((char*)scratch + fl_align256(n * 8)); }

int fl_locator_build(fl_ctx* ctx, const fl_mesh_dev& m, const fl_domain_dev& dom, void* scratch, fl_locator* L,
                     int level_bound, bool in_key_order) {
    const size_t n = m.n;
    const int log2nb = locator_log2nb(n);
    char* p = (char*)scratch;
    uint64_t* keys = (uint64_t*)p; p += fl_align256(n * 8);
    uint32_t* ids = (uint32_t*)p; p += fl_align256(n * 4);
    uint32_t* dir = (uint32_t*)p; p += fl_align256((((size_t)1 << log2nb) + 1) * 4);
    uint32_t* flag = (uint32_t*)p; p += 256;
    *L = fl_locator{keys, nullptr, dir, m.level, n, log2nb, 0};
    if (n == 0) return FL_OK;
    FL_TRY_CUDA(ctx, cudaMemsetAsync(flag, 0, 8, ctx->stream), "locator");
    uint32_t hf[2] = {0, (uint32_t)std::max(level_bound, 0)};  // unsorted, deepest level
    if (level_bound < 0) {
        k_deepest<<<fl_blocks(n, 256, ctx->num_sms * 4), 256, 0, ctx->stream>>>(m.level, n, flag);
        FL_CHECK_LAUNCH(ctx, "k_deepest");
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(hf, flag, 8, cudaMemcpyDeviceToHost, ctx->stream), "locator");
        FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "locator");
    }
    L->cut = dom.anchor_level > (int)hf[1] ? dom.anchor_level - (int)hf[1] : 0;
    k_run_keys<<<fl_blocks(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(m, dom, L->cut, keys, ids);
    FL_CHECK_LAUNCH(ctx, "k_run_keys");
    hf[0] = 0;
    if (!in_key_order) {
        k_check_sorted<<<fl_blocks(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(keys, n, flag);
        FL_CHECK_LAUNCH(ctx, "k_check_sorted");
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(hf, flag, 4, cudaMemcpyDeviceToHost, ctx->stream), "locator");
        FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "locator");
    }
    if (hf[0]) {  // stable: equal run starts keep mesh order, so the last of them is found
        // the keys hold 3 (depth - cut) bits, plus 16 for case ids
        const int end_bit = std::min(64, 3 * (dom.depth - L->cut) + (m.case_id ? 16 : 0));
        int rc = fl_sort_pairs_with(ctx, keys, ids, n, 0, end_bit, p);
        if (rc) return rc;
        L->ids = ids;
    }
    k_locator_dir<<<fl_blocks(n + 1, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(keys, n, log2nb, dir);
    FL_CHECK_LAUNCH(ctx, "k_locator_dir");
    return FL_OK;
}

int fl_neighbours_sorted(fl_ctx* ctx, const fl_mesh_dev& m, const fl_domain_dev& dom, const fl_locator& L,
                         int subslots, uint32_t* nbr, uint32_t* marks) {
    if (m.n == 0) return FL_OK;
    FL_TRY_CUDA(ctx, cudaMemsetAsync(marks, 0, m.n * 4, ctx->stream), "neighbour marks");
    const size_t cells = (size_t)(kNbrCells / subslots);
    const unsigned grid =
        (unsigned)std::min<size_t>((m.n + cells - 1) / cells, (size_t)ctx->num_sms * kNbrBlocksPerSM);
    if (subslots == 4) {
        k_neighbours_sorted<4, true><<<grid, kNbrThreads, 0, ctx->stream>>>(m, dom, L, nbr, marks);
        FL_CHECK_LAUNCH(ctx, "k_neighbours_sorted");
        k_neighbours_sorted<4, false><<<grid, kNbrThreads, 0, ctx->stream>>>(m, dom, L, nbr, marks);
    } else {
        k_neighbours_sorted<1, true><<<grid, kNbrThreads, 0, ctx->stream>>>(m, dom, L, nbr, marks);
        FL_CHECK_LAUNCH(ctx, "k_neighbours_sorted");
        k_neighbours_sorted<1, false><<<grid, kNbrThreads, 0, ctx->stream>>>(m, dom, L, nbr, marks);
    }
    FL_CHECK_LAUNCH(ctx, "k_neighbours_sorted");
    return FL_OK;
}

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
    k_hash_clear<<<cb, 256, 0, ctx->stream>>>(tk, tv, cap);
    FL_CHECK_LAUNCH(ctx, "k_hash_clear");
    if (n == 0) return FL_OK;
    const uint8_t* lv = vals ? nullptr : levels;
    FL_TRY_CUDA(ctx, cudaMemsetAsync(ctx->dev_status + FL_DEVSTAT_HASH_DUPS, 0, 4, ctx->stream), "hash flag");
    int lg = fl_hash_lg(cap);
    unsigned nb = fl_blocks(n, 256, ctx->num_sms * 8);
    k_hash_insert<<<nb, 256, 0, ctx->stream>>>(tk, tv, lg, keys, vals, lv, n, ctx->dev_status);
    FL_CHECK_LAUNCH(ctx, "k_hash_insert");
    k_hash_dup_clear<<<cb, 256, 0, ctx->stream>>>(win, cap, ctx->dev_status);
    FL_CHECK_LAUNCH(ctx, "k_hash_dup_clear");
    k_hash_dup_winners<<<nb, 256, 0, ctx->stream>>>(tk, tv ? 1 : 2, win, lg, keys, n, ctx->dev_status);
    FL_CHECK_LAUNCH(ctx, "k_hash_dup_winners");
    k_hash_dup_values<<<cb, 256, 0, ctx->stream>>>(tk, tv, win, vals, lv, cap, ctx->dev_status);
    FL_CHECK_LAUNCH(ctx, "k_hash_dup_values");
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
