// sort.cu — LSD onesweep radix sort of uint64 keys with uint32 payloads.
//
// Replaces RadixSort::sortByKey (src/core/hashmap/RadixSort.cpp:55-104, a stub
// that launches nothing) and its kernels (kernels/hashmap/radix_sort.cl:14-122,
// whose atomic_inc scatter is unstable).  Design (onesweep, Adinets & Merrill 2022):
//  1. one upfront pass histograms every 8-bit digit of every pass at once
//     (per-CTA shared histograms, then global atomics), and one tiny kernel
//     turns each pass histogram into exclusive bin offsets;
//  2. per pass, one kernel: each CTA takes the next tile (atomic ticket), ranks
//     its keys stably with warp __match_any_sync peer groups and per-warp
//     digit counters, publishes its per-digit counts, resolves its global
//     per-digit base by decoupled look-back over earlier tiles (one thread per
//     digit, bounded spin), stages the tile in shared memory in rank order and
//     writes it out with coalesced runs.
// Stable: ties keep input order, so (key, payload) pairs match std::stable_sort.
#include "common.cuh"
#include "scan.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 12;
constexpr int kTile = kThreads * kItems;  // 3072 keys
constexpr int kRadix = 256;

constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kFlagMask = 3u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1;

__global__ void __launch_bounds__(kThreads) k_histogram(const uint64_t* __restrict__ keys, size_t n, int begin_bit,
                                                        int end_bit, int passes, uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[8][kRadix];
    for (int i = threadIdx.x; i < 8 * kRadix; i += kThreads) (&h[0][0])[i] = 0;
    __syncthreads();
    size_t stride = (size_t)gridDim.x * kThreads;
    for (size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += stride) {
        uint64_t k = keys[i];
        for (int p = 0; p < passes; ++p) {
            int sh = begin_bit + 8 * p;
            uint32_t m = end_bit - sh >= 8 ? 255u : ((1u << (end_bit - sh)) - 1u);
            atomicAdd(&h[p][(k >> sh) & m], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kRadix; i += kThreads) {
        uint32_t v = (&h[0][0])[i];
        if (v) atomicAdd(hist + i, v);
    }
}

// Exclusive scan of each pass's 256 bins (one CTA per pass).
__global__ void k_bin_offsets(uint32_t* hist) {
    __shared__ uint32_t s[kRadix];
    uint32_t* h = hist + blockIdx.x * kRadix;
    int t = threadIdx.x;
    s[t] = h[t];
    __syncthreads();
    for (int o = 1; o < kRadix; o <<= 1) {
        uint32_t v = t >= o ? s[t - o] : 0u;
        __syncthreads();
        s[t] += v;
        __syncthreads();
    }
    h[t] = s[t] - h[t];
}

__device__ __forceinline__ uint32_t ld_vol(const uint32_t* p) { return *(volatile const uint32_t*)p; }

__global__ void __launch_bounds__(kThreads, 4) k_onesweep(const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                       uint64_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                       size_t n, int shift, uint32_t dmask,
                                                       const uint32_t* __restrict__ bin_off,
                                                       uint32_t* status, unsigned* ticket, uint32_t* dev_status) {
    __shared__ uint32_t s_warp_hist[kWarps][kRadix];
    __shared__ uint32_t s_tile_excl[kRadix];
    __shared__ uint32_t s_glob[kRadix];
    __shared__ uint64_t s_keys[kTile];
    __shared__ uint32_t s_vals[kTile];
    __shared__ int s_tile;
    __shared__ int s_bad;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) { s_tile = (int)atomicAdd(ticket, 1u); s_bad = 0; }
    for (int i = threadIdx.x; i < kWarps * kRadix; i += kThreads) (&s_warp_hist[0][0])[i] = 0;
    __syncthreads();
    const int tile = s_tile;
    const size_t tbase = (size_t)tile * kTile;
    const size_t wbase = tbase + (size_t)warp * 32 * kItems;
    const unsigned lt = (1u << lane) - 1u;

    uint64_t k[kItems];
    uint32_t v[kItems];
    uint32_t rank[kItems];
    // stable in-warp ranking: iteration i handles keys wbase + i*32 + lane
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        size_t g = wbase + (size_t)i * 32 + lane;
        bool ok = g < n;
        k[i] = ok ? kin[g] : 0ull;
        v[i] = ok ? vin[g] : 0u;
        uint32_t d = ok ? (uint32_t)((k[i] >> shift) & dmask) : 256u;
        unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        // the group's first lane adds the group to the warp's digit counter and
        // hands the old count to its peers (one shared atomic, no warp barrier)
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0u;
        if (d < 256u && lane == leader) base = atomicAdd(&s_warp_hist[warp][d], (uint32_t)__popc(peers));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        rank[i] = base + __popc(peers & lt);
    }
    __syncthreads();
    // per-digit: tile count, cross-warp exclusive offsets (thread = digit)
    {
        const int d = threadIdx.x;
        uint32_t run = 0;
        for (int w = 0; w < kWarps; ++w) {
            uint32_t c = s_warp_hist[w][d];
            s_warp_hist[w][d] = run;
            run += c;
        }
        // publish aggregate, look back, publish inclusive
        uint32_t* st = status + (size_t)tile * kRadix + d;
        uint32_t prefix = 0;
        // a status word carries its own value: no fence orders it after other data
        if (tile == 0) {
            *(volatile uint32_t*)st = kFlagInc | run;
        } else {
            *(volatile uint32_t*)st = kFlagAgg | run;
            int t = tile - 1;
            unsigned spins = 0;
            while (t >= 0) {
                uint32_t s = ld_vol(status + (size_t)t * kRadix + d);
                if ((s & kFlagMask) == 0) {
                    if (++spins > FL_SPIN_LIMIT) {
                        atomicAdd(dev_status + FL_DEVSTAT_TIMEOUT, 1u);
                        s_bad = 1;
                        break;
                    }
                    continue;
                }
                prefix += s & kValMask;
                if ((s & kFlagMask) == kFlagInc) break;
                --t;
            }
            *(volatile uint32_t*)st = kFlagInc | ((prefix + run) & kValMask);
        }
        s_glob[d] = bin_off[d] + prefix;
        // tile-local exclusive scan over digits of the tile counts
        s_tile_excl[d] = run;
    }
    __syncthreads();
    // block exclusive scan of s_tile_excl (256 entries, one per thread)
    {
        const int d = threadIdx.x;
        uint32_t c = s_tile_excl[d];
        uint32_t incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += t;
        }
        __shared__ uint32_t s_wsum[kWarps];
        if (lane == 31) s_wsum[warp] = incl;
        __syncthreads();
        uint32_t wofs = 0;
        for (int w = 0; w < warp; ++w) wofs += s_wsum[w];
        __syncthreads();
        s_tile_excl[d] = wofs + incl - c;
    }
    __syncthreads();
    // stage in rank order
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        size_t g = wbase + (size_t)i * 32 + lane;
        if (g < n) {
            uint32_t d = (uint32_t)((k[i] >> shift) & dmask);
            uint32_t pos = s_tile_excl[d] + s_warp_hist[warp][d] + rank[i];
            s_keys[pos] = k[i];
            s_vals[pos] = v[i];
        }
    }
    __syncthreads();
    if (s_bad) return;  // a timed-out look-back leaves this tile unwritten; the host reports the error
    size_t count = n - tbase < (size_t)kTile ? n - tbase : (size_t)kTile;
    for (int i = threadIdx.x; i < (int)count; i += kThreads) {
        uint64_t kk = s_keys[i];
        uint32_t d = (uint32_t)((kk >> shift) & dmask);
        size_t pos = (size_t)s_glob[d] + (size_t)(i - (int)s_tile_excl[d]);
        if (pos >= n) { atomicAdd(dev_status + FL_DEVSTAT_BOUNDS, 1u); continue; }
        kout[pos] = kk;
        vout[pos] = s_vals[i];
    }
}

}  // namespace

size_t fl_sort_scratch_bytes(size_t n, int passes) {
    size_t tiles = (n + kTile - 1) / kTile;
    return fl_align256(n * 8) + fl_align256(n * 4) + fl_align256((size_t)passes * kRadix * 4) +
           (size_t)passes * fl_align256(tiles * kRadix * 4 + 4) + 256;
}

int fl_sort_pairs_with(fl_ctx* ctx, uint64_t* keys, uint32_t* vals, size_t n, int begin_bit, int end_bit,
                       void* scratch) {
    if (n <= 1) return FL_OK;
    int passes = (end_bit - begin_bit + 7) / 8;
    if (passes <= 0) return FL_OK;
    size_t tiles = (n + kTile - 1) / kTile;
    char* p = (char*)scratch;
    uint64_t* kalt = (uint64_t*)p; p += fl_align256(n * 8);
    uint32_t* valt = (uint32_t*)p; p += fl_align256(n * 4);
    uint32_t* hist = (uint32_t*)p; p += fl_align256((size_t)passes * kRadix * 4);
    char* stat0 = p;
    size_t stat_stride = fl_align256(tiles * kRadix * 4 + 4);
    // clear histograms + per-pass status/tickets in one memset
    FL_TRY_CUDA(ctx, cudaMemsetAsync(hist, 0, fl_align256((size_t)passes * kRadix * 4) + passes * stat_stride,
                                     ctx->stream), "sort clear");
    unsigned hb = fl_blocks(n, kThreads, ctx->num_sms * 4);
    k_histogram<<<hb, kThreads, 0, ctx->stream>>>(keys, n, begin_bit, end_bit, passes, hist);
    FL_CHECK_LAUNCH(ctx, "k_histogram");
    k_bin_offsets<<<passes, kRadix, 0, ctx->stream>>>(hist);
    FL_CHECK_LAUNCH(ctx, "k_bin_offsets");
    uint64_t* ks[2] = {keys, kalt};
    uint32_t* vs[2] = {vals, valt};
    int cur = 0;
    for (int ps = 0; ps < passes; ++ps) {
        uint32_t* status = (uint32_t*)(stat0 + ps * stat_stride);
        unsigned* ticket = (unsigned*)(status + tiles * kRadix);
        int sh = begin_bit + 8 * ps;
        uint32_t dmask = end_bit - sh >= 8 ? 255u : ((1u << (end_bit - sh)) - 1u);
        k_onesweep<<<(unsigned)tiles, kThreads, 0, ctx->stream>>>(ks[cur], vs[cur], ks[cur ^ 1], vs[cur ^ 1], n, sh,
                                                                  dmask, hist + ps * kRadix, status, ticket,
                                                                  ctx->dev_status);
        FL_CHECK_LAUNCH(ctx, "k_onesweep");
        cur ^= 1;
    }
    if (cur == 1) {
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(keys, kalt, n * 8, cudaMemcpyDeviceToDevice, ctx->stream), "sort copy");
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(vals, valt, n * 4, cudaMemcpyDeviceToDevice, ctx->stream), "sort copy");
    }
    return FL_OK;
}

extern "C" int fl_sort_pairs_u64_u32(fl_ctx* ctx, uint64_t* keys, uint32_t* vals, size_t n, int begin_bit,
                                     int end_bit) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (n <= 1) return FL_OK;
    if (!keys || !vals || begin_bit < 0 || end_bit > 64 || begin_bit >= end_bit)
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_sort_pairs_u64_u32: bad pointer or bit range");
    if (n >= (1ull << 30)) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_sort_pairs_u64_u32: n >= 2^30");
    int passes = (end_bit - begin_bit + 7) / 8;
    int rc = fl_scratch_reserve(ctx, fl_sort_scratch_bytes(n, passes));
    if (rc) return rc;
    return fl_sort_pairs_with(ctx, keys, vals, n, begin_bit, end_bit, ctx->scratch);
}
