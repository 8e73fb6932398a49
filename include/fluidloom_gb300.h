/* fluidloom_gb300.h — C ABI of the GB300-native AMR lattice-Boltzmann hot path.
 *
 * Plain pointers and sizes only.  Every entry point returns an int status
 * (FL_OK = 0, negative on error; fl_last_error() gives the message).  Device
 * entry points take DEVICE pointers and are ordered on the context's CUDA
 * stream (asynchronous unless stated); host helpers are marked [host].
 *
 * Each declaration names the reference interface it replaces
 * (fedres/fluidloom, path:line).  Where the reference passes cl_mem handles
 * on a cl_command_queue, this ABI passes device pointers on a CUDA stream.
 */
#ifndef FLUIDLOOM_GB300_H
#define FLUIDLOOM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (replace the reference's FluidLoomError/OpenCLError
 *      exceptions, include/fluidloom/common/FluidLoomError.h:13-81) */
#define FL_OK 0
#define FL_E_INVALID_ARG (-1)
#define FL_E_OOM (-2)
#define FL_E_CAPACITY (-3)
#define FL_E_HASH_OVERFLOW (-4)
#define FL_E_BALANCE_NOT_CONVERGED (-5) /* warning class: result is usable (AdaptationEngine.cpp:54-56) */
#define FL_E_DEVICE_TIMEOUT (-6)        /* a bounded device-side wait gave up */
#define FL_E_CUDA (-7)
#define FL_E_NO_DEVICE (-8)
#define FL_E_LEVEL_JUMP (-9)            /* neighbours more than one level apart */

#define FL_INVALID 0xFFFFFFFFu
#define FL_EMPTY_KEY 0xFFFFFFFFFFFFFFFFull

typedef struct fl_ctx fl_ctx;

/* ---- context (replaces the cl_context + cl_command_queue pair every engine
 *      constructor takes, e.g. AdaptationEngine.h:36) */
int fl_ctx_create(int device, fl_ctx** out);
int fl_ctx_destroy(fl_ctx* ctx);
/* Use an external stream (a cudaStream_t passed as void*); NULL restores the context's own. */
int fl_ctx_set_stream(fl_ctx* ctx, void* cuda_stream);
void* fl_ctx_stream(fl_ctx* ctx);
int fl_ctx_synchronize(fl_ctx* ctx);
const char* fl_last_error(fl_ctx* ctx);
const char* fl_status_string(int status);
int fl_version(void);

/* ---- device memory helpers for FFI callers without an allocator
 *      (replaces IBackend::allocateBuffer/copyHostToDevice/copyDeviceToHost,
 *      include/fluidloom/core/backend/IBackend.h:25-119) */
int fl_device_alloc(fl_ctx* ctx, size_t bytes, void** out);
int fl_device_free(fl_ctx* ctx, void* ptr);
int fl_memcpy_h2d(fl_ctx* ctx, void* dst, const void* src, size_t bytes);   /* synchronous */
int fl_memcpy_d2h(fl_ctx* ctx, void* dst, const void* src, size_t bytes);   /* synchronous */
int fl_memset_d(fl_ctx* ctx, void* dst, int value, size_t bytes);           /* async */

/* ---- keys */
/* hilbert::encode over n cells (include/fluidloom/core/hilbert/HilbertCodec.h:29;
 * kernels/hilbert.cl:104-115).  ids (may be NULL) receives 0..n-1, the leaf-id
 * payload the sort carries. */
int fl_hilbert_encode(fl_ctx* ctx, const int32_t* x, const int32_t* y, const int32_t* z, uint8_t level,
                      uint64_t* keys, uint32_t* ids, size_t n);
/* hilbert::decode (HilbertCodec.h:40; kernels/hilbert.cl:118-130). */
int fl_hilbert_decode(fl_ctx* ctx, const uint64_t* keys, uint8_t level, int32_t* x, int32_t* y, int32_t* z,
                      size_t n);
/* adaptation::hilbert_encode_3d(x, y, z, 8) (include/fluidloom/adaptation/CellDescriptor.h:11,49-51). */
int fl_morton8_encode(fl_ctx* ctx, const int32_t* x, const int32_t* y, const int32_t* z, uint64_t* keys,
                      size_t n);
/* Cell order key: hilbert::encode(native << (anchor_level - level), depth) | case << 3*depth
 * (replaces CellDescriptor::getHilbert as the rebuild sort key, AdaptationEngine.cpp:212-217).
 * case_id may be NULL. */
int fl_cell_keys(fl_ctx* ctx, const int32_t* x, const int32_t* y, const int32_t* z, const uint8_t* level,
                 const uint16_t* case_id, int depth, int anchor_level, uint64_t* keys, size_t n);
/* [host] hilbert::getParent / getChild / isValid (HilbertCodec.h:49,59,68). */
uint64_t fl_hilbert_get_parent(uint64_t key, uint8_t level);
uint64_t fl_hilbert_get_child(uint64_t key, uint8_t level, uint8_t quadrant);
int fl_hilbert_is_valid(uint64_t key, uint8_t level);

#ifdef __cplusplus
}
#endif
#endif
