// sort.cu — LSD onesweep radix sort of uint64 keys with uint32 payloads.
//
// Replaces RadixSort::sortByKey (src/core/hashmap/RadixSort.cpp:55-104, a stub
// that launches nothing) and its kernels (kernels/hashmap/radix_sort.cl:14-122,
// whose atomic_inc scatter is unstable and whose digit is fixed at 8 bits,
// radix_sort.cl:5-6).  Design (onesweep, Adinets & Merrill 2022):
//  1. one upfront pass histograms every digit of every pass at once
//     (per-CTA shared histograms, then global atomics), and one tiny kernel
//     turns each pass histogram into exclusive bin offsets;
//  2. per pass, one kernel: each CTA takes the next tile (atomic ticket), ranks
//     its keys stably with warp __match_any_sync peer groups and per-warp
//     digit counters, publishes its per-digit counts, resolves its global
//     per-digit base by decoupled look-back over earlier tiles (one thread per
//     digit, bounded spin), stages the tile in shared memory in rank order and
//     writes it out with coalesced runs.
// Four shapes, chosen per context (fl_sort_set_config): 8- or 9-bit digits (9:
// 7 passes over 63-bit keys instead of 8) on tiles of 256 or 512 threads x 12
// keys (512: half the tiles and twice the keys per digit run written, at 2
// CTAs per SM; 256: 4 CTAs per SM with 8-bit digits, 3 with 9-bit, whose
// threads then take two digits each).
// Stable: ties keep input order, so (key, payload) pairs match std::stable_sort.
#include "common.cuh"
#include "scan.cuh"

namespace {

constexpr int kItems = 12;                 // keys per thread in a tile
constexpr int kTileMin = 256 * kItems;     // the smallest tile: scratch is sized for it
constexpr int kMaxRadix = 512;
constexpr int kMaxPasses = 8;              // 64-bit keys, 8- or 9-bit digits

constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kFlagMask = 3u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1;

__host__ __device__ constexpr uint32_t digit_mask(int end_bit, int sh, int bits) {
    return end_bit - sh >= bits ? (1u << bits) - 1u : (1u << (end_bit - sh)) - 1u;
}

template <int kBits>
__global__ void __launch_bounds__(256) k_histogram(const uint64_t* __restrict__ keys, size_t n, int begin_bit,
                                                   int end_bit, int passes, uint32_t* __restrict__ hist) {
    constexpr int R = 1 << kBits;
    __shared__ uint32_t h[kMaxPasses][R];
    for (int i = threadIdx.x; i < kMaxPasses * R; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t k = keys[i];
        for (int p = 0; p < passes; ++p) {
            int sh = begin_bit + kBits * p;
            atomicAdd(&h[p][(k >> sh) & digit_mask(end_bit, sh, kBits)], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * R; i += blockDim.x) {
        uint32_t v = (&h[0][0])[i];
        if (v) atomicAdd(hist + i, v);
    }
}

// Exclusive scan of each pass's bins (one CTA of R threads per pass).
template <int kBits>
__global__ void k_bin_offsets(uint32_t* hist) {
    constexpr int R = 1 << kBits;
    __shared__ uint32_t s[R];
    uint32_t* h = hist + blockIdx.x * R;
    int t = threadIdx.x;
    s[t] = h[t];
    __syncthreads();
    for (int o = 1; o < R; o <<= 1) {
        uint32_t v = t >= o ? s[t - o] : 0u;
        __syncthreads();
        s[t] += v;
        __syncthreads();
    }
    h[t] = s[t] - h[t];
}

__device__ __forceinline__ uint32_t ld_vol(const uint32_t* p) { return *(volatile const uint32_t*)p; }

// Dynamic shared memory of one onesweep tile: keys and values staged in rank
// order, per-warp digit counters, per-digit tile offsets and global bases,
// per-warp sums of the digit scan.
template <int kThreads, int kBits>
__host__ __device__ constexpr size_t onesweep_smem() {
    return (size_t)kThreads * kItems * 12 +
           ((size_t)(kThreads / 32) * (1 << kBits) + 2 * (1 << kBits) + kThreads / 32) * 4;
}

template <int kThreads, int kBits>
__global__ void __launch_bounds__(kThreads, kThreads == 512 ? 2 : (kBits == 8 ? 4 : 3))
    k_onesweep(const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
               uint32_t* __restrict__ vout, size_t n, int shift, uint32_t dmask,
               const uint32_t* __restrict__ bin_off, uint32_t* status, unsigned* ticket, uint32_t* dev_status) {
    constexpr int R = 1 << kBits;
    constexpr int kWarps = kThreads / 32;
    constexpr int kTile = kThreads * kItems;
    // digit scan: each of the first R / D threads takes D consecutive digits
    constexpr int D = R > kThreads ? R / kThreads : 1;
    static_assert(R % 32 == 0 && (R <= kThreads || R % kThreads == 0), "whole warps of digits");
    extern __shared__ __align__(16) unsigned char s_dyn[];
    uint64_t* s_keys = (uint64_t*)s_dyn;
    uint32_t* s_vals = (uint32_t*)(s_keys + kTile);
    uint32_t* s_warp_hist = s_vals + kTile;  // [kWarps][R]
    uint32_t* s_tile_excl = s_warp_hist + kWarps * R;
    uint32_t* s_glob = s_tile_excl + R;
    uint32_t* s_wsum = s_glob + R;
    __shared__ int s_tile;
    __shared__ int s_bad;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) { s_tile = (int)atomicAdd(ticket, 1u); s_bad = 0; }
    for (int i = threadIdx.x; i < kWarps * R; i += kThreads) s_warp_hist[i] = 0;
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
        uint32_t d = ok ? (uint32_t)((k[i] >> shift) & dmask) : (uint32_t)R;
        unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        // the group's first lane adds the group to the warp's digit counter and
        // hands the old count to its peers (one shared atomic, no warp barrier)
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0u;
        if (d < (uint32_t)R && lane == leader) base = atomicAdd(&s_warp_hist[warp * R + d], (uint32_t)__popc(peers));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        rank[i] = base + __popc(peers & lt);
    }
    __syncthreads();
    // per-digit: tile count, cross-warp exclusive offsets (a thread per digit, or
    // R / kThreads digits per thread one after another)
    for (int d = threadIdx.x; d < R; d += kThreads) {
        uint32_t run = 0;
        for (int w = 0; w < kWarps; ++w) {
            uint32_t c = s_warp_hist[w * R + d];
            s_warp_hist[w * R + d] = run;
            run += c;
        }
        // publish aggregate, look back, publish inclusive
        uint32_t* st = status + (size_t)tile * R + d;
        uint32_t prefix = 0;
        // a status word carries its own value: no fence orders it after other data
        if (tile == 0) {
            *(volatile uint32_t*)st = kFlagInc | run;
        } else {
            *(volatile uint32_t*)st = kFlagAgg | run;
            int t = tile - 1;
            unsigned spins = 0;
            while (t >= 0) {
                uint32_t s = ld_vol(status + (size_t)t * R + d);
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
    // block exclusive scan of s_tile_excl (R entries; thread t < R / D holds digits
    // tD .. tD + D - 1)
    {
        const int t0 = threadIdx.x * D;
        uint32_t c[D], sum = 0, incl = 0;
        if (t0 < R) {
#pragma unroll
            for (int j = 0; j < D; ++j) {
                c[j] = s_tile_excl[t0 + j];
                sum += c[j];
            }
            incl = sum;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= o) incl += t;
            }
            if (lane == 31) s_wsum[warp] = incl;
        }
        __syncthreads();
        if (t0 < R) {
            uint32_t ex = incl - sum;
            for (int w = 0; w < warp; ++w) ex += s_wsum[w];
#pragma unroll
            for (int j = 0; j < D; ++j) {
                s_tile_excl[t0 + j] = ex;
                ex += c[j];
            }
        }
    }
    __syncthreads();
    // stage in rank order
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        size_t g = wbase + (size_t)i * 32 + lane;
        if (g < n) {
            uint32_t d = (uint32_t)((k[i] >> shift) & dmask);
            uint32_t pos = s_tile_excl[d] + s_warp_hist[warp * R + d] + rank[i];
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

// Bytes of one pass's tile status words and ticket, for every shape: at most
// ceil(n / kTileMin) tiles of at most kMaxRadix digits (9-bit digits on the
// smallest tile reach both bounds at once).
size_t status_stride_min(size_t n) {
    return fl_align256(((n + kTileMin - 1) / kTileMin) * kMaxRadix * 4 + 4) + 4096;
}

// All passes of one shape.  The scratch layout (fl_sort_scratch_bytes): the
// alternate key and value buffers, the pass histograms (kMaxPasses x
// kMaxRadix), then per pass its tile status words and ticket, at a stride that
// fits every shape's tiles (status_stride_min).
template <int kThreads, int kBits>
int sort_passes(fl_ctx* ctx, uint64_t* keys, uint32_t* vals, size_t n, int begin_bit, int end_bit, void* scratch) {
    constexpr int R = 1 << kBits;
    constexpr int kTile = kThreads * kItems;
    const int passes = (end_bit - begin_bit + kBits - 1) / kBits;
    if (passes <= 0) return FL_OK;
    const size_t tiles = (n + kTile - 1) / kTile;
    char* p = (char*)scratch;
    uint64_t* kalt = (uint64_t*)p; p += fl_align256(n * 8);
    uint32_t* valt = (uint32_t*)p; p += fl_align256(n * 4);
    uint32_t* hist = (uint32_t*)p; p += fl_align256((size_t)kMaxPasses * kMaxRadix * 4);
    char* stat0 = p;
    const size_t stat_stride = status_stride_min(n);
    // clear histograms + per-pass status/tickets in one memset
    FL_TRY_CUDA(ctx, cudaMemsetAsync(hist, 0, fl_align256((size_t)kMaxPasses * kMaxRadix * 4) + passes * stat_stride,
                                     ctx->stream), "sort clear");
    constexpr size_t smem = onesweep_smem<kThreads, kBits>();
    FL_TRY_CUDA(ctx, cudaFuncSetAttribute(k_onesweep<kThreads, kBits>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem), "sort shared memory");
    unsigned hb = fl_blocks(n, 256, ctx->num_sms * 4);
    k_histogram<kBits><<<hb, 256, 0, ctx->stream>>>(keys, n, begin_bit, end_bit, passes, hist);
    FL_CHECK_LAUNCH(ctx, "k_histogram");
    k_bin_offsets<kBits><<<passes, R, 0, ctx->stream>>>(hist);
    FL_CHECK_LAUNCH(ctx, "k_bin_offsets");
    uint64_t* ks[2] = {keys, kalt};
    uint32_t* vs[2] = {vals, valt};
    int cur = 0;
    for (int ps = 0; ps < passes; ++ps) {
        uint32_t* status = (uint32_t*)(stat0 + ps * stat_stride);
        unsigned* ticket = (unsigned*)(status + tiles * R);
        int sh = begin_bit + kBits * ps;
        k_onesweep<kThreads, kBits><<<(unsigned)tiles, kThreads, smem, ctx->stream>>>(
            ks[cur], vs[cur], ks[cur ^ 1], vs[cur ^ 1], n, sh, digit_mask(end_bit, sh, kBits), hist + ps * R, status,
            ticket, ctx->dev_status);
        FL_CHECK_LAUNCH(ctx, "k_onesweep");
        cur ^= 1;
    }
    if (cur == 1) {
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(keys, kalt, n * 8, cudaMemcpyDeviceToDevice, ctx->stream), "sort copy");
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(vals, valt, n * 4, cudaMemcpyDeviceToDevice, ctx->stream), "sort copy");
    }
    return FL_OK;
}

}  // namespace

// passes: the 8-bit pass count of the key range (every shape needs at most as many).
size_t fl_sort_scratch_bytes(size_t n, int passes) {
    return fl_align256(n * 8) + fl_align256(n * 4) + fl_align256((size_t)kMaxPasses * kMaxRadix * 4) +
           (size_t)passes * status_stride_min(n) + 256;
}

int fl_sort_pairs_with(fl_ctx* ctx, uint64_t* keys, uint32_t* vals, size_t n, int begin_bit, int end_bit,
                       void* scratch) {
    if (n <= 1 || end_bit <= begin_bit) return FL_OK;
    if (ctx->sort_digit_bits == 9 && ctx->sort_tile_threads == 256)
        return sort_passes<256, 9>(ctx, keys, vals, n, begin_bit, end_bit, scratch);
    if (ctx->sort_digit_bits == 9) return sort_passes<512, 9>(ctx, keys, vals, n, begin_bit, end_bit, scratch);
    if (ctx->sort_tile_threads == 512) return sort_passes<512, 8>(ctx, keys, vals, n, begin_bit, end_bit, scratch);
    return sort_passes<256, 8>(ctx, keys, vals, n, begin_bit, end_bit, scratch);
}

extern "C" int fl_sort_set_config(fl_ctx* ctx, int digit_bits, int tile_threads) {
    if (!ctx) return FL_E_INVALID_ARG;
    const bool ok = (digit_bits == 8 || digit_bits == 9) && (tile_threads == 256 || tile_threads == 512);
    if (!ok)
        return fl_set_error(ctx, FL_E_INVALID_ARG,
                            "fl_sort_set_config: digit_bits 8 or 9, tile_threads 256 or 512");
    ctx->sort_digit_bits = digit_bits;
    ctx->sort_tile_threads = tile_threads;
    return FL_OK;
}

extern "C" int fl_sort_get_config(fl_ctx* ctx, int* digit_bits, int* tile_threads) {
    if (!ctx || !digit_bits || !tile_threads) return FL_E_INVALID_ARG;
    *digit_bits = ctx->sort_digit_bits;
    *tile_threads = ctx->sort_tile_threads;
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
