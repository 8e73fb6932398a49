// common.cuh — shared definitions for the fluidloom_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include <string>

#include "fluidloom_gb300.h"

#define FL_INVALID_INDEX 0xFFFFFFFFu
#define FL_EMPTY_KEY 0xFFFFFFFFFFFFFFFFull

// Per-context state.  One host thread drives a context; all work is ordered on
// its stream.  Scratch is a growable device buffer (never shrunk) so steady
// state launches allocate nothing.
struct fl_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    uint32_t* dev_status = nullptr;     // device-side status words (see FL_DEVSTAT_*)
    uint32_t* host_status = nullptr;    // pinned mirror
    std::string last_error;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // fl_ctx_timer_start / stop
    void* soa = nullptr;                       // structure-of-arrays field manager (fields.cu)
    uint64_t launches = 0;                     // kernels launched on behalf of this context
    int64_t alloc_fail_countdown = -1;         // fault injection: allocations left before they fail (-1 off)
    int sort_digit_bits = 8;                   // radix sort shape (fl_sort_set_config)
    int sort_tile_threads = 256;
};

// Every device allocation the library makes goes through these two: cudaMalloc
// or cudaMallocAsync on st, unless the context's fault-injection countdown
// (fl_ctx_inject_alloc_failure) has run out, in which case nothing is
// allocated and cudaErrorMemoryAllocation is returned as CUDA would.
cudaError_t fl_dev_malloc(fl_ctx* ctx, void** p, size_t bytes);
cudaError_t fl_dev_malloc_async(fl_ctx* ctx, void** p, size_t bytes, cudaStream_t st);

void fl_soa_release_all(fl_ctx* ctx);
int fl_soa_bind_external(fl_ctx* ctx, const fl_field_desc* d, size_t num_cells, size_t pitch, void* base,
                         uint64_t* handle);

// Device status words written by kernels instead of trapping.
enum {
    FL_DEVSTAT_TIMEOUT = 0,     // a bounded spin gave up
    FL_DEVSTAT_HASH_OVERFLOW = 1,
    FL_DEVSTAT_LEVEL_JUMP = 2,  // a neighbour more than one level away
    FL_DEVSTAT_BOUNDS = 3,      // an index failed a bounds check and the access was skipped
    FL_DEVSTAT_HASH_DUPS = 4,   // the current hash build met a repeated key (not an error)
    FL_DEVSTAT_WORDS = 8
};

int fl_set_error(fl_ctx* ctx, int code, const std::string& msg);
int fl_check_cuda(fl_ctx* ctx, cudaError_t e, const char* what);
// Ensure ctx->scratch holds at least `bytes` (256-byte aligned sub-buffers are carved by callers).
int fl_scratch_reserve(fl_ctx* ctx, size_t bytes);
// Read back and clear the device status words; returns FL_OK or the first error.
int fl_collect_device_status(fl_ctx* ctx, const char* what);

#define FL_TRY_CUDA(ctx, expr, what)                                  \
    do {                                                              \
        cudaError_t _e = (expr);                                      \
        if (_e != cudaSuccess) return fl_check_cuda((ctx), _e, what); \
    } while (0)

// After each kernel launch: counts it and checks the launch.
#define FL_CHECK_LAUNCH(ctx, what)                    \
    do {                                              \
        ++(ctx)->launches;                            \
        FL_TRY_CUDA(ctx, cudaGetLastError(), what);   \
    } while (0)
// After a batch of launches counted by the caller.
#define FL_CHECK_ERRORS(ctx, what) FL_TRY_CUDA(ctx, cudaGetLastError(), what)

static inline size_t fl_align256(size_t b) { return (b + 255) & ~(size_t)255; }

static inline unsigned fl_blocks(size_t n, unsigned threads, unsigned cap) {
    size_t b = (n + threads - 1) / threads;
    if (b == 0) b = 1;
    if (b > cap) b = cap;
    return (unsigned)b;
}

// Bounded spin budget for decoupled look-back (iterations of a polling loop).
#define FL_SPIN_LIMIT (1u << 22)
