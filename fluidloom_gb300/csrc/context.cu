// context.cu — context, errors, scratch and memory helpers of the C ABI.
#include "common.cuh"

#include <cstdio>
#include <cstring>

int fl_set_error(fl_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

int fl_check_cuda(fl_ctx* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return FL_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) return fl_set_error(ctx, FL_E_OOM, m);
    return fl_set_error(ctx, FL_E_CUDA, m);
}

static bool injected_alloc_failure(fl_ctx* ctx) {
    if (!ctx || ctx->alloc_fail_countdown < 0) return false;
    if (ctx->alloc_fail_countdown == 0) return true;
    --ctx->alloc_fail_countdown;
    return false;
}

// A failed allocation always leaves *p null, so cleanup paths never free a
// stale pointer.
cudaError_t fl_dev_malloc(fl_ctx* ctx, void** p, size_t bytes) {
    *p = nullptr;
    if (injected_alloc_failure(ctx)) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) *p = nullptr;
    return e;
}

cudaError_t fl_dev_malloc_async(fl_ctx* ctx, void** p, size_t bytes, cudaStream_t st) {
    *p = nullptr;
    if (injected_alloc_failure(ctx)) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMallocAsync(p, bytes, st);
    if (e != cudaSuccess) *p = nullptr;
    return e;
}

int fl_scratch_reserve(fl_ctx* ctx, size_t bytes) {
    if (bytes <= ctx->scratch_bytes) return FL_OK;
    size_t want = bytes + bytes / 4 + (1 << 20);
    if (ctx->scratch) {
        // the stream may still use the old buffer
        FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "scratch sync");
        cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
    }
    FL_TRY_CUDA(ctx, fl_dev_malloc(ctx, &ctx->scratch, want), "scratch allocation");
    ctx->scratch_bytes = want;
    return FL_OK;
}

int fl_collect_device_status(fl_ctx* ctx, const char* what) {
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->host_status, ctx->dev_status, FL_DEVSTAT_WORDS * 4,
                                     cudaMemcpyDeviceToHost, ctx->stream), "status read");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), what);
    uint32_t s[FL_DEVSTAT_WORDS];
    std::memcpy(s, ctx->host_status, sizeof(s));
    if (s[FL_DEVSTAT_TIMEOUT] | s[FL_DEVSTAT_HASH_OVERFLOW] | s[FL_DEVSTAT_LEVEL_JUMP] | s[FL_DEVSTAT_BOUNDS]) {
        FL_TRY_CUDA(ctx, cudaMemsetAsync(ctx->dev_status, 0, FL_DEVSTAT_WORDS * 4, ctx->stream), "status clear");
        FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "status clear");
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: device status timeout=%u hash_overflow=%u level_jump=%u bounds=%u",
                      what, s[0], s[1], s[2], s[3]);
        if (s[FL_DEVSTAT_TIMEOUT]) return fl_set_error(ctx, FL_E_DEVICE_TIMEOUT, buf);
        if (s[FL_DEVSTAT_HASH_OVERFLOW]) return fl_set_error(ctx, FL_E_HASH_OVERFLOW, buf);
        if (s[FL_DEVSTAT_LEVEL_JUMP]) return fl_set_error(ctx, FL_E_LEVEL_JUMP, buf);
        return fl_set_error(ctx, FL_E_INVALID_ARG, buf);
    }
    return FL_OK;
}

extern "C" {

int fl_version(void) { return 10000; }

const char* fl_status_string(int s) {
    switch (s) {
        case FL_OK: return "ok";
        case FL_E_INVALID_ARG: return "invalid argument";
        case FL_E_OOM: return "out of device memory";
        case FL_E_CAPACITY: return "capacity exceeded";
        case FL_E_HASH_OVERFLOW: return "hash table probe limit exceeded";
        case FL_E_BALANCE_NOT_CONVERGED: return "2:1 balance did not converge";
        case FL_E_DEVICE_TIMEOUT: return "device-side wait timed out";
        case FL_E_CUDA: return "CUDA error";
        case FL_E_NO_DEVICE: return "no CUDA device";
        case FL_E_LEVEL_JUMP: return "neighbouring leaves more than one level apart";
        default: return "unknown status";
    }
}

int fl_ctx_create(int device, fl_ctx** out) {
    if (!out) return FL_E_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return FL_E_NO_DEVICE;
    }
    if (device < 0 || device >= count) return FL_E_INVALID_ARG;
    fl_ctx* c = new fl_ctx();
    c->device = device;
    int rc = FL_OK;
    if (cudaSetDevice(device) != cudaSuccess) rc = FL_E_CUDA;
    if (rc == FL_OK && cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        rc = FL_E_CUDA;
    if (rc == FL_OK && cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) rc = FL_E_CUDA;
    c->own_stream = true;
    if (rc == FL_OK && cudaMalloc(&c->dev_status, FL_DEVSTAT_WORDS * 4) != cudaSuccess) rc = FL_E_OOM;
    if (rc == FL_OK && cudaMemset(c->dev_status, 0, FL_DEVSTAT_WORDS * 4) != cudaSuccess) rc = FL_E_CUDA;
    if (rc == FL_OK && cudaMallocHost(&c->host_status, FL_DEVSTAT_WORDS * 4) != cudaSuccess) rc = FL_E_OOM;
    if (rc != FL_OK) {
        cudaGetLastError();
        fl_ctx_destroy(c);
        return rc;
    }
    *out = c;
    return FL_OK;
}

int fl_ctx_destroy(fl_ctx* ctx) {
    if (!ctx) return FL_OK;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    fl_soa_release_all(ctx);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->dev_status) cudaFree(ctx->dev_status);
    if (ctx->host_status) cudaFreeHost(ctx->host_status);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return FL_OK;
}

int fl_ctx_set_stream(fl_ctx* ctx, void* s) {
    if (!ctx) return FL_E_INVALID_ARG;
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "stream switch");
    if (s == nullptr) {
        if (!ctx->own_stream) {
            FL_TRY_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "stream create");
            ctx->own_stream = true;
        }
        return FL_OK;
    }
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    ctx->stream = (cudaStream_t)s;
    ctx->own_stream = false;
    return FL_OK;
}

void* fl_ctx_stream(fl_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int fl_ctx_synchronize(fl_ctx* ctx) {
    if (!ctx) return FL_E_INVALID_ARG;
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronize");
    return FL_OK;
}

int fl_ctx_inject_alloc_failure(fl_ctx* ctx, int64_t after) {
    if (!ctx) return FL_E_INVALID_ARG;
    ctx->alloc_fail_countdown = after < 0 ? -1 : after;
    return FL_OK;
}

const char* fl_last_error(fl_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

int fl_device_alloc(fl_ctx* ctx, size_t bytes, void** out) {
    if (!ctx || !out) return FL_E_INVALID_ARG;
    *out = nullptr;
    if (bytes == 0) return FL_OK;
    FL_TRY_CUDA(ctx, fl_dev_malloc(ctx, out, bytes), "fl_device_alloc");
    return FL_OK;
}

int fl_device_free(fl_ctx* ctx, void* p) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (!p) return FL_OK;
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "fl_device_free sync");
    FL_TRY_CUDA(ctx, cudaFree(p), "fl_device_free");
    return FL_OK;
}

int fl_memcpy_h2d(fl_ctx* ctx, void* dst, const void* src, size_t bytes) {
    if (!ctx || (bytes && (!dst || !src))) return FL_E_INVALID_ARG;
    if (!bytes) return FL_OK;
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream), "fl_memcpy_h2d");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "fl_memcpy_h2d sync");
    return FL_OK;
}

int fl_memcpy_d2h(fl_ctx* ctx, void* dst, const void* src, size_t bytes) {
    if (!ctx || (bytes && (!dst || !src))) return FL_E_INVALID_ARG;
    if (!bytes) return FL_OK;
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream), "fl_memcpy_d2h");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "fl_memcpy_d2h sync");
    return FL_OK;
}

int fl_host_alloc_pinned(fl_ctx* ctx, size_t bytes, void** out) {
    if (!ctx || !out) return FL_E_INVALID_ARG;
    *out = nullptr;
    if (!bytes) return FL_OK;
    FL_TRY_CUDA(ctx, cudaMallocHost(out, bytes), "fl_host_alloc_pinned");
    return FL_OK;
}

int fl_host_free_pinned(fl_ctx* ctx, void* p) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (p) FL_TRY_CUDA(ctx, cudaFreeHost(p), "fl_host_free_pinned");
    return FL_OK;
}

int fl_ctx_timer_start(fl_ctx* ctx) {
    if (!ctx) return FL_E_INVALID_ARG;
    if (!ctx->ev0) {
        FL_TRY_CUDA(ctx, cudaEventCreate(&ctx->ev0), "event");
        FL_TRY_CUDA(ctx, cudaEventCreate(&ctx->ev1), "event");
    }
    FL_TRY_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    return FL_OK;
}

int fl_ctx_launch_count(fl_ctx* ctx, uint64_t* count) {
    if (!ctx || !count) return FL_E_INVALID_ARG;
    *count = ctx->launches;
    return FL_OK;
}

int fl_ctx_timer_stop(fl_ctx* ctx, float* ms) {
    if (!ctx || !ms || !ctx->ev0) return FL_E_INVALID_ARG;
    FL_TRY_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    FL_TRY_CUDA(ctx, cudaEventSynchronize(ctx->ev1), "event sync");
    FL_TRY_CUDA(ctx, cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1), "event elapsed");
    return FL_OK;
}

int fl_memset_d(fl_ctx* ctx, void* dst, int value, size_t bytes) {
    if (!ctx || (bytes && !dst)) return FL_E_INVALID_ARG;
    if (!bytes) return FL_OK;
    FL_TRY_CUDA(ctx, cudaMemsetAsync(dst, value, bytes, ctx->stream), "fl_memset_d");
    return FL_OK;
}

}  // extern "C"
