// Test-infrastructure: plain C entry points over the reference codec compiled
// in place (oracle/Makefile.ref), so Python tests can sweep it exhaustively.
#include "fluidloom/core/hilbert/HilbertCodec.h"
#include <cstdint>
#include <cstddef>
namespace fluidloom { namespace adaptation {
uint64_t hilbert_encode_3d(int32_t x, int32_t y, int32_t z, uint8_t max_level);
} }
extern "C" void ref_hilbert_encode(const int32_t* x, const int32_t* y, const int32_t* z,
                                   uint8_t level, uint64_t* out, size_t n) {
    for (size_t i = 0; i < n; ++i) out[i] = fluidloom::hilbert::encode(x[i], y[i], z[i], level);
}
extern "C" void ref_hilbert_decode(const uint64_t* k, uint8_t level, int32_t* x, int32_t* y,
                                   int32_t* z, size_t n) {
    for (size_t i = 0; i < n; ++i) fluidloom::hilbert::decode(k[i], level, x[i], y[i], z[i]);
}
extern "C" void ref_morton8_encode(const int32_t* x, const int32_t* y, const int32_t* z,
                                   uint64_t* out, size_t n) {
    for (size_t i = 0; i < n; ++i) out[i] = fluidloom::adaptation::hilbert_encode_3d(x[i], y[i], z[i], 8);
}
