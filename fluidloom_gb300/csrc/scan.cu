// scan.cu — single-pass exclusive scan of uint32 with decoupled look-back,
// stream compaction and permutation.
//
// Replaces the reference's three-phase work-group scan (AdaptationEngine::exclusiveScan,
// src/adaptation/AdaptationEngine.cpp:360-415 with scan_local/scan_add_sums,
// src/adaptation/kernels/compact_cells.cl:61-125), which is exact only up to
// 65,536 elements (:378).  Here one launch scans any n: each CTA takes the next
// tile in launch order (atomic ticket), publishes its aggregate, looks back
// over its predecessors one warp-wide window at a time, publishes its
// inclusive prefix and writes its slice.  Every wait is bounded
// (FL_SPIN_LIMIT); on expiry the CTA records FL_DEVSTAT_TIMEOUT and finishes
// with a partial prefix so the host can report the error.
#include "common.cuh"
#include "scan.cuh"

#include <cuda.h>

#include <mutex>

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;

constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagInc = 2ull << 62;
constexpr unsigned long long kFlagMask = 3ull << 62;

__device__ __forceinline__ unsigned long long ld_status(const unsigned long long* p) {
    return *(volatile const unsigned long long*)p;
}
// A status word carries its flag and its value together, so publishing it
// needs no fence against other stores.
__device__ __forceinline__ void st_status(unsigned long long* p, unsigned long long v) {
    *(volatile unsigned long long*)p = v;
}

// Warp-wide look-back: returns the exclusive prefix of tile `t` (lane 0 holds it).
// Gives up after `limit` polls of an unpublished window, records
// FL_DEVSTAT_TIMEOUT and returns the partial prefix.
__device__ uint32_t lookback_limited(unsigned long long* status, int t, uint32_t* dev_status, unsigned limit) {
    const int lane = threadIdx.x & 31;
    uint32_t prefix = 0;
    int base = t - 1;
    unsigned spins = 0;
    while (base >= 0) {
        int idx = base - lane;
        unsigned long long s = idx >= 0 ? ld_status(status + idx) : kFlagInc;
        // wait until every lane of the window sees a published word
        while (true) {
            bool ready = (s & kFlagMask) != 0;
            if (__all_sync(0xFFFFFFFFu, ready)) break;
            if (++spins > limit) {
                if (lane == 0) atomicAdd(dev_status + FL_DEVSTAT_TIMEOUT, 1u);
                return prefix;
            }
            if (!ready) s = ld_status(status + idx);
        }
        unsigned inc_mask = __ballot_sync(0xFFFFFFFFu, (s & kFlagMask) == kFlagInc);
        int stop = inc_mask ? __ffs(inc_mask) - 1 : 31;  // lanes 0..stop contribute
        uint32_t v = (lane <= stop) ? (uint32_t)(s & 0xFFFFFFFFull) : 0u;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        prefix += v;
        if (inc_mask) break;
        base -= 32;
    }
    return prefix;
}

__device__ __forceinline__ uint32_t lookback(unsigned long long* status, int t, uint32_t* dev_status) {
    return lookback_limited(status, t, dev_status, FL_SPIN_LIMIT);
}

// One warp looks back from tile 1 at a tile-0 word that nothing publishes:
// the wait runs out after `limit` polls and the kernel returns normally.
__global__ void k_lookback_probe(unsigned long long* status, uint32_t* dev_status, unsigned limit) {
    lookback_limited(status, 1, dev_status, limit);
}

// VEC: `in` and `out` are 16-byte aligned plain arrays; full tiles then move
// each thread's 16 items as four 128-bit loads and stores.
template <bool VEC = false, typename Load>
__device__ void scan_tile(Load load, uint32_t* __restrict__ out, size_t n, unsigned long long* status,
                          unsigned* ticket, uint32_t* total, uint32_t* dev_status, const uint32_t* in = nullptr) {
    __shared__ int s_tile;
    __shared__ uint32_t s_warp[kThreads / 32];
    __shared__ uint32_t s_prefix;
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(ticket, 1u);
    __syncthreads();
    const int tile = s_tile;
    const size_t base = (size_t)tile * kTile;
    // blocked arrangement: thread t owns items [t*kItems, t*kItems+kItems)
    uint32_t v[kItems];
    uint32_t sum = 0;
    const bool full = VEC && base + kTile <= n;
    if (full) {
        const uint4* p4 = (const uint4*)(in + base + (size_t)threadIdx.x * kItems);
#pragma unroll
        for (int j = 0; j < kItems / 4; ++j) {
            const uint4 a = __ldg(p4 + j);
            v[4 * j] = a.x; v[4 * j + 1] = a.y; v[4 * j + 2] = a.z; v[4 * j + 3] = a.w;
        }
#pragma unroll
        for (int i = 0; i < kItems; ++i) sum += v[i];
    } else {
#pragma unroll
        for (int i = 0; i < kItems; ++i) {
            size_t g = base + (size_t)threadIdx.x * kItems + i;
            v[i] = g < n ? load(g) : 0u;
            sum += v[i];
        }
    }
    // block exclusive scan of per-thread sums
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kThreads / 32 ? s_warp[lane] : 0u;
        uint32_t wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < kThreads / 32) s_warp[lane] = wi - w;  // exclusive per warp
        uint32_t agg = __shfl_sync(0xFFFFFFFFu, wi, kThreads / 32 - 1);
        uint32_t prefix = 0;
        if (tile == 0) {
            if (lane == 0) st_status(status, kFlagInc | agg);
        } else {
            if (lane == 0) st_status(status + tile, kFlagAgg | agg);
            prefix = lookback(status, tile, dev_status);
            if (lane == 0) st_status(status + tile, kFlagInc | (uint32_t)(prefix + agg));
        }
        if (lane == 0) {
            s_prefix = prefix;
            if (total && base + kTile >= n) *total = prefix + agg;
        }
    }
    __syncthreads();
    uint32_t run = s_prefix + s_warp[warp] + (incl - sum);
    if (full) {
        uint4* o4 = (uint4*)(out + base + (size_t)threadIdx.x * kItems);
#pragma unroll
        for (int j = 0; j < kItems / 4; ++j) {
            uint4 a;
            a.x = run; run += v[4 * j];
            a.y = run; run += v[4 * j + 1];
            a.z = run; run += v[4 * j + 2];
            a.w = run; run += v[4 * j + 3];
            o4[j] = a;
        }
    } else {
#pragma unroll
        for (int i = 0; i < kItems; ++i) {
            size_t g = base + (size_t)threadIdx.x * kItems + i;
            if (g < n) out[g] = run;
            run += v[i];
        }
    }
}

struct LoadU32 {
    const uint32_t* p;
    __device__ uint32_t operator()(size_t i) const { return __ldg(p + i); }
};

template <bool VEC>
__global__ void __launch_bounds__(kThreads) k_scan(const uint32_t* in, uint32_t* out, size_t n,
                                                   unsigned long long* status, unsigned* ticket, uint32_t* total,
                                                   uint32_t* dev_status) {
    scan_tile<VEC>(LoadU32{in}, out, n, status, ticket, total, dev_status, in);
}

// CompactionEngine::compactAndPermute predicate (CompactionEngine.cpp:51-56).
struct LoadKeep {
    const uint64_t* keys;
    const uint32_t* state;
    __device__ uint32_t operator()(size_t i) const {
        return (state[i] != 0u && keys[i] != FL_EMPTY_KEY) ? 1u : 0u;
    }
};

__global__ void __launch_bounds__(kThreads) k_scan_keep(LoadKeep ld, uint32_t* out, size_t n,
                                                        unsigned long long* status, unsigned* ticket,
                                                        uint32_t* total, uint32_t* dev_status) {
    scan_tile(ld, out, n, status, ticket, total, dev_status);
}

__global__ void k_gather_kept(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ state,
                              const uint32_t* __restrict__ off, size_t n, uint64_t* __restrict__ okeys,
                              uint32_t* __restrict__ oids) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (state[i] != 0u && keys[i] != FL_EMPTY_KEY) {
            okeys[off[i]] = keys[i];
            oids[off[i]] = (uint32_t)i;
        }
    }
}

__global__ void k_fill_u32(uint32_t* p, uint32_t v, size_t n) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) p[i] = v;
}

__global__ void k_invert_perm(const uint32_t* __restrict__ sorted_ids, uint32_t m, uint32_t* __restrict__ perm) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += stride) perm[sorted_ids[j]] = (uint32_t)j;
}

template <int E>
struct Elem { uint32_t w[E / 4]; };

template <typename T>
__global__ void k_apply_perm(const T* __restrict__ src, T* __restrict__ dst, size_t n, const uint32_t* __restrict__ perm) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint32_t p = perm[i];
        if (p != FL_INVALID_INDEX) dst[p] = src[i];
    }
}

__global__ void k_apply_perm_bytes(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, size_t elem, size_t n,
                                   const uint32_t* __restrict__ perm) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint32_t p = perm[i];
        if (p == FL_INVALID_INDEX) continue;
        for (size_t b = 0; b < elem; ++b) dst[(size_t)p * elem + b] = src[i * elem + b];
    }
}

}  // namespace

size_t fl_scan_scratch_bytes(size_t n) {
    size_t tiles = (n + kTile - 1) / kTile;
    return fl_align256(tiles * 8 + 8) + 256;
}

int fl_scan_u32_with(fl_ctx* ctx, const uint32_t* in, uint32_t* out, size_t n, uint32_t* total, void* scratch) {
    if (n == 0) {
        if (total) FL_TRY_CUDA(ctx, cudaMemsetAsync(total, 0, 4, ctx->stream), "scan total");
        return FL_OK;
    }
    size_t tiles = (n + kTile - 1) / kTile;
    unsigned long long* status = (unsigned long long*)scratch;
    unsigned* ticket = (unsigned*)((char*)scratch + fl_align256(tiles * 8 + 8));
    FL_TRY_CUDA(ctx, cudaMemsetAsync(scratch, 0, fl_scan_scratch_bytes(n), ctx->stream), "scan status clear");
    // in == out (an in-place scan) is fine: each thread reads its items before writing them
    if ((((uintptr_t)in | (uintptr_t)out) & 15u) == 0)
        k_scan<true><<<(unsigned)tiles, kThreads, 0, ctx->stream>>>(in, out, n, status, ticket, total, ctx->dev_status);
    else
        k_scan<false><<<(unsigned)tiles, kThreads, 0, ctx->stream>>>(in, out, n, status, ticket, total, ctx->dev_status);
    FL_CHECK_LAUNCH(ctx, "k_scan");
    return FL_OK;
}

int fl_launch_fill_u32(fl_ctx* ctx, uint32_t* p, uint32_t v, size_t n) {
    if (!n) return FL_OK;
    k_fill_u32<<<fl_blocks(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(p, v, n);
    FL_CHECK_LAUNCH(ctx, "k_fill_u32");
    return FL_OK;
}

extern "C" {

int fl_scan_exclusive_u32(fl_ctx* ctx, const uint32_t* in, uint32_t* out, size_t n, uint32_t* total) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (n && (!in || !out)) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_scan_exclusive_u32: null pointer");
    if (n >= (1ull << 32)) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_scan_exclusive_u32: n >= 2^32");
    int rc = fl_scratch_reserve(ctx, fl_scan_scratch_bytes(n));
    if (rc) return rc;
    return fl_scan_u32_with(ctx, in, out, n, total, ctx->scratch);
}

int fl_lookback_timeout_probe(fl_ctx* ctx, uint32_t spin_limit) {
    if (!ctx || spin_limit == 0 || spin_limit > FL_SPIN_LIMIT) return FL_E_INVALID_ARG;
    int rc = fl_scratch_reserve(ctx, 256);
    if (rc) return rc;
    FL_TRY_CUDA(ctx, cudaMemsetAsync(ctx->scratch, 0, 256, ctx->stream), "probe clear");
    k_lookback_probe<<<1, 32, 0, ctx->stream>>>((unsigned long long*)ctx->scratch, ctx->dev_status, spin_limit);
    FL_CHECK_LAUNCH(ctx, "k_lookback_probe");
    return fl_collect_device_status(ctx, "fl_lookback_timeout_probe");
}

int fl_compact_and_permute(fl_ctx* ctx, const uint64_t* keys, const uint32_t* state, size_t n, uint32_t* perm,
                           uint64_t* sorted_keys, uint32_t* sorted_ids, size_t* num_valid) {
    if (!ctx || !num_valid) return FL_E_INVALID_ARG;
    *num_valid = 0;
    if (n == 0) return FL_OK;
    if (!keys || !state || !perm || !sorted_keys || !sorted_ids)
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_compact_and_permute: null pointer");
    size_t sb = fl_scan_scratch_bytes(n);
    size_t off_b = fl_align256(n * 4);
    int rc = fl_scratch_reserve(ctx, sb + off_b + 256);
    if (rc) return rc;
    uint32_t* off = (uint32_t*)((char*)ctx->scratch + sb);
    uint32_t* total = (uint32_t*)((char*)ctx->scratch + sb + off_b);
    size_t tiles = (n + kTile - 1) / kTile;
    unsigned long long* status = (unsigned long long*)ctx->scratch;
    unsigned* ticket = (unsigned*)((char*)ctx->scratch + fl_align256(tiles * 8 + 8));
    FL_TRY_CUDA(ctx, cudaMemsetAsync(ctx->scratch, 0, sb, ctx->stream), "status clear");
    k_scan_keep<<<(unsigned)tiles, kThreads, 0, ctx->stream>>>(LoadKeep{keys, state}, off, n, status, ticket, total,
                                                               ctx->dev_status);
    FL_CHECK_LAUNCH(ctx, "k_scan_keep");
    unsigned blocks = fl_blocks(n, 256, ctx->num_sms * 8);
    k_gather_kept<<<blocks, 256, 0, ctx->stream>>>(keys, state, off, n, sorted_keys, sorted_ids);
    FL_CHECK_LAUNCH(ctx, "k_gather_kept");
    uint32_t m = 0;
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(&m, total, 4, cudaMemcpyDeviceToHost, ctx->stream), "total read");
    rc = fl_collect_device_status(ctx, "fl_compact_and_permute scan");
    if (rc) return rc;
    rc = fl_sort_pairs_u64_u32(ctx, sorted_keys, sorted_ids, m, 0, 64);
    if (rc) return rc;
    rc = fl_launch_fill_u32(ctx, perm, FL_INVALID_INDEX, n);
    if (rc) return rc;
    if (m) {
        k_invert_perm<<<fl_blocks(m, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(sorted_ids, m, perm);
        FL_CHECK_LAUNCH(ctx, "k_invert_perm");
    }
    *num_valid = m;
    return FL_OK;
}

int fl_apply_permutation(fl_ctx* ctx, const void* src, void* dst, size_t elem_size, size_t old_n,
                         const uint32_t* perm) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (old_n == 0) return FL_OK;
    if (!src || !dst || !perm || elem_size == 0 || src == dst)
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_apply_permutation: bad arguments (src must differ from dst)");
    unsigned blocks = fl_blocks(old_n, 256, ctx->num_sms * 8);
    switch (elem_size) {
        case 1: k_apply_perm<uint8_t><<<blocks, 256, 0, ctx->stream>>>((const uint8_t*)src, (uint8_t*)dst, old_n, perm); break;
        case 2: k_apply_perm<uint16_t><<<blocks, 256, 0, ctx->stream>>>((const uint16_t*)src, (uint16_t*)dst, old_n, perm); break;
        case 4: k_apply_perm<uint32_t><<<blocks, 256, 0, ctx->stream>>>((const uint32_t*)src, (uint32_t*)dst, old_n, perm); break;
        case 8: k_apply_perm<uint64_t><<<blocks, 256, 0, ctx->stream>>>((const uint64_t*)src, (uint64_t*)dst, old_n, perm); break;
        default:
            k_apply_perm_bytes<<<blocks, 256, 0, ctx->stream>>>((const uint8_t*)src, (uint8_t*)dst, elem_size, old_n, perm);
    }
    FL_CHECK_LAUNCH(ctx, "k_apply_perm");
    return FL_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Exclusive scan for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: embedders that own every device
// allocation through their own pool or arena sized at start-up, hosts running
// under a fixed device-memory budget that must not grow, and FFI hosts that
// must not allocate on their hot path (cudaMalloc and cudaFree can synchronize
// the whole device).  For them this entry point takes no context and allocates
// nothing: the scan's only scratch (one status word per 4,096-element tile, a
// tile ticket and a timeout word) lives in the file-scope array below, sized
// for at most kNoAllocMaxN elements (128 KiB + 512 B); every GPU that loads
// this library keeps that array until the process exits.  The caller passes
// the input, the output and (optionally) the total.
namespace {

constexpr size_t kNoAllocMaxN = (size_t)1 << 26;                 // 67,108,864 elements
constexpr size_t kNoAllocTiles = kNoAllocMaxN / kTile;           // 16,384 tile status words
constexpr size_t kNoAllocStatusBytes = kNoAllocTiles * 8;        // 128 KiB
constexpr size_t kNoAllocBytes = kNoAllocStatusBytes + 512;      // + ticket and timeout words

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of g_noalloc_scratch: the array's name is only a host-side
// stand-in, so host code asks the runtime for the address with the device
// current.  The address belongs to one context instance; it is cached with
// that context's unique id (cuCtxGetId, which allocates nothing) and looked up
// again when a call finds another context current on the device -- after a
// cudaDeviceReset or a primary-context reset by the embedding host.
struct NoAllocSlot {
    unsigned long long ctx_id;
    void* ptr;
};
std::mutex g_noalloc_mu;
NoAllocSlot g_noalloc_slot[64] = {};

// The two driver calls come through the runtime's entry-point query, so the
// library does not link libcuda itself (it loads on hosts without a driver).
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

int current_ctx_id(unsigned long long* id) {
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 4000, cudaEnableDefault, &qa) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
            qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b)
            return FL_E_CUDA;
        g_ctx_get_current = (CtxGetCurrentFn)a;
        g_ctx_get_id = (CtxGetIdFn)b;
    }
    CUcontext c = nullptr;
    if (g_ctx_get_current(&c) != CUDA_SUCCESS) return FL_E_CUDA;
    if (!c) { *id = 0; return FL_OK; }
    return g_ctx_get_id(c, id) == CUDA_SUCCESS ? FL_OK : FL_E_CUDA;
}

int noalloc_scratch(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FL_E_CUDA;
    if (dev < 0 || dev >= 64) return FL_E_INVALID_ARG;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);  // also guards the driver entry points' first lookup
    unsigned long long id = 0;
    if (current_ctx_id(&id)) return FL_E_CUDA;
    NoAllocSlot& s = g_noalloc_slot[dev];
    if (!s.ptr || id == 0 || s.ctx_id != id) {
        void* p = nullptr;  // the lookup makes the device's primary context current if none was
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return FL_E_CUDA;
        if (current_ctx_id(&id) || id == 0) return FL_E_CUDA;
        s.ptr = p;
        s.ctx_id = id;
    }
    *out = s.ptr;
    return FL_OK;
}

}  // namespace

extern "C" int fl_scan_exclusive_u32_noalloc(const uint32_t* in, uint32_t* out, size_t n, uint32_t* total,
                                             void* cuda_stream) {
    if (n > kNoAllocMaxN) return FL_E_CAPACITY;
    if (n && (!in || !out)) return FL_E_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    void* base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc) return rc;
    if (n == 0) {
        if (total && cudaMemsetAsync(total, 0, 4, st) != cudaSuccess) return FL_E_CUDA;
        return cudaStreamSynchronize(st) == cudaSuccess ? FL_OK : FL_E_CUDA;
    }
    size_t tiles = (n + kTile - 1) / kTile;
    unsigned long long* status = (unsigned long long*)base;
    unsigned* ticket = (unsigned*)((char*)base + kNoAllocStatusBytes);
    uint32_t* timeout = (uint32_t*)((char*)base + kNoAllocStatusBytes + 256);
    // the array keeps the previous call's contents: clear the words this call reads as zero
    if (cudaMemsetAsync(status, 0, tiles * 8, st) != cudaSuccess) return FL_E_CUDA;
    if (cudaMemsetAsync(ticket, 0, 256 + FL_DEVSTAT_WORDS * 4, st) != cudaSuccess) return FL_E_CUDA;
    // An error the embedding host left pending is its own: only an error that
    // appears with this launch is reported (and cleared) as this call's failure.
    const cudaError_t pending = cudaPeekAtLastError();
    if ((((uintptr_t)in | (uintptr_t)out) & 15u) == 0)
        k_scan<true><<<(unsigned)tiles, kThreads, 0, st>>>(in, out, n, status, ticket, total, timeout);
    else
        k_scan<false><<<(unsigned)tiles, kThreads, 0, st>>>(in, out, n, status, ticket, total, timeout);
    if (pending == cudaSuccess && cudaPeekAtLastError() != cudaSuccess) {
        cudaGetLastError();
        return FL_E_CUDA;
    }
    uint32_t expired = 0;  // a pageable destination makes this copy wait for the scan
    if (cudaMemcpyAsync(&expired, timeout + FL_DEVSTAT_TIMEOUT, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return FL_E_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return FL_E_CUDA;
    return expired ? FL_E_DEVICE_TIMEOUT : FL_OK;
}
