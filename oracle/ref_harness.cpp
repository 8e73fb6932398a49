// Test-infrastructure harness: links the reference's own Hilbert codec
// (src/core/hilbert/HilbertCodec.cpp, src/adaptation/utils/HilbertCodec3D.cpp,
// compiled in place from the reference tree by oracle/Makefile.ref) and writes
// known-answer vectors that replay the reference's unit tests
// (tests/unit/hilbert/test_hilbert_codec.cpp:33-125) plus wider sweeps.
// Output: a flat binary stream read by tests/golden/make_golden.py.
#include "fluidloom/core/hilbert/HilbertCodec.h"
#include "fluidloom/core/hilbert/CellCoord.h"
#include <cstdio>
#include <cstdint>
#include <random>
#include <vector>

namespace fluidloom { namespace adaptation {
uint64_t hilbert_encode_3d(int32_t x, int32_t y, int32_t z, uint8_t max_level);
} }

using namespace fluidloom;

static void put_u32(FILE* f, uint32_t v) { fwrite(&v, 4, 1, f); }
static void rec(FILE* f, int32_t x, int32_t y, int32_t z, uint8_t lv, uint64_t k) {
    fwrite(&x, 4, 1, f); fwrite(&y, 4, 1, f); fwrite(&z, 4, 1, f);
    uint32_t l = lv; fwrite(&l, 4, 1, f); fwrite(&k, 8, 1, f);
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    FILE* f = fopen(argv[1], "wb");
    if (!f) return 3;
    // Section 1: level-1 corners (test_hilbert_codec.cpp:33-58).
    put_u32(f, 8);
    for (int z = 0; z < 2; ++z) for (int y = 0; y < 2; ++y) for (int x = 0; x < 2; ++x)
        rec(f, x, y, z, 1, hilbert::encode(x, y, z, 1));
    // Section 2: round trip levels 1..8, 1000 per level, mt19937_64 seeded 42
    // (test_hilbert_codec.cpp:13-30,72-92); same draw expression as the test.
    {
        std::mt19937_64 rng; rng.seed(42);
        put_u32(f, 8 * 1000);
        for (uint8_t level = 1; level <= 8; ++level) {
            for (int i = 0; i < 1000; ++i) {
                int32_t max_val = (1 << level) - 1;
                std::uniform_int_distribution<int32_t> dist(0, max_val);
                CellCoord c(dist(rng), dist(rng), dist(rng), level);
                rec(f, c.x, c.y, c.z, level, c.hilbert());
            }
        }
    }
    // Section 3: canonical form case (test_hilbert_codec.cpp:94-106).
    put_u32(f, 1);
    rec(f, 123, 456, 789, 5, hilbert::encode(123, 456, 789, 5));
    // Section 4: parent/child (test_hilbert_codec.cpp:108-125): parent + 8 children.
    {
        std::mt19937_64 rng; rng.seed(42);
        std::uniform_int_distribution<int32_t> dist(0, 7);
        CellCoord p(dist(rng), dist(rng), dist(rng), 3);
        put_u32(f, 9);
        rec(f, p.x, p.y, p.z, 3, p.hilbert());
        for (uint8_t q = 0; q < 8; ++q) { CellCoord c = p.child(q); rec(f, c.x, c.y, c.z, c.level, c.hilbert()); }
    }
    // Section 5: full 21-level keys of 21-bit coordinates (the 63-bit key space).
    {
        std::mt19937_64 rng(20240601ULL);
        put_u32(f, 4096);
        for (int i = 0; i < 4096; ++i) {
            int32_t x = (int32_t)(rng() & 0x1FFFFF), y = (int32_t)(rng() & 0x1FFFFF), z = (int32_t)(rng() & 0x1FFFFF);
            rec(f, x, y, z, 21, hilbert::encode(x, y, z, 21));
        }
    }
    // Section 6: every level 0..21 with random in-range and out-of-range coords
    // (masking to 21 bits, negative inputs).
    {
        std::mt19937_64 rng(7ULL);
        put_u32(f, 22 * 64);
        for (int lv = 0; lv <= 21; ++lv) for (int i = 0; i < 64; ++i) {
            int32_t x = (int32_t)rng(), y = (int32_t)rng(), z = (int32_t)rng();
            rec(f, x, y, z, (uint8_t)lv, hilbert::encode(x, y, z, (uint8_t)lv));
        }
    }
    // Section 7: the AMR-path 8-level encoder (HilbertCodec3D.cpp:29-53) on
    // random int32 coordinates (negative and wide values included).
    {
        std::mt19937_64 rng(99ULL);
        put_u32(f, 4096);
        for (int i = 0; i < 4096; ++i) {
            int32_t x = (int32_t)rng(), y = (int32_t)rng(), z = (int32_t)rng();
            if (i < 2048) { x &= 0x3FF; y &= 0x3FF; z &= 0x3FF; }
            rec(f, x, y, z, 8, adaptation::hilbert_encode_3d(x, y, z, 8));
        }
    }
    // Section 8: getParent of the 21-level keys of section 5 equals key >> 3
    // (HilbertCodec.cpp:117-123); written as (level, key, parent).
    {
        std::mt19937_64 rng(20240601ULL);
        put_u32(f, 64);
        for (int i = 0; i < 64; ++i) {
            int32_t x = (int32_t)(rng() & 0x1FFFFF), y = (int32_t)(rng() & 0x1FFFFF), z = (int32_t)(rng() & 0x1FFFFF);
            uint64_t k = hilbert::encode(x, y, z, 21);
            rec(f, (int32_t)(hilbert::getParent(k, 21) & 0x7FFFFFFF), (int32_t)(hilbert::getParent(k, 21) >> 31), 0, 21, k);
        }
    }
    fclose(f);
    return 0;
}
