// lbm.cu — D3Q19 BGK collide-stream over an octree of 8^3-site bricks, the
// brick pool that owns it (cases, populations, neighbour table, per-level
// brick lists), regrid with population remap, refinement flags and the FP64
// conservation sums.
//
// The reference has no lattice-Boltzmann code: its lbm_* kernels are
// generated empty (src/parsing/SimulationBuilder.cpp:394-400) and D3Q19 is
// only lattice metadata (include/fluidloom/parsing/LatticeDescriptor.h:15-44).
// The method is therefore the literature's, as the CPU oracle restates it:
// BGK equilibrium (Qian, d'Humieres & Lallemand 1992), half-way bounce-back
// with the moving-wall term 6 w_q rho0 (c_q . u_w) (Ladd 1994), equilibrium
// velocity inlet and zero-gradient outlet (Kruger et al. 2017), acoustic
// scaling across levels with tau_l = 2^l (tau_0 - 1/2) + 1/2 and level l
// sub-cycled 2^l times per level-0 step (Dupuis & Chopard 2003).  The
// coarse/fine coupling uses the reference's own prolongation (copy,
// split_cells.cl:110-132) and restriction (mean of 8, merge_cells.cl:123-159,
// FieldAveragingRules.h:31-41) per population, with the coarse side linearly
// interpolated in time for the second fine sub-step.
//
// Layout in HBM: populations are structure-of-arrays, f[q][brick][site] with
// site = x + 8y + 64z inside the brick, so a warp reading one population of
// 32 consecutive sites touches one 128-byte line.  Three population buffers
// are kept: A and B (per-level parity) and a spare that receives the remap
// at each regrid.  This unit is compiled with -fmad=false so its FP32 results
// are the IEEE sequence of operations written here, identical to the CPU
// restatement it is tested against.
#include "common.cuh"
#include "amr.cuh"
#include "bulk.cuh"
#include "hash.cuh"
#include "keys.cuh"
#include "scan.cuh"

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <vector>

namespace {

constexpr int Q = 19;
constexpr uint64_t kCXp = 0x1548889549ull;  // (c_x + 1) in 2 bits per population
constexpr uint64_t kCYp = 0x895609495ull;
constexpr uint64_t kCZp = 0x20a0954955ull;
__host__ __device__ constexpr int CXq(int q) { return (int)((kCXp >> (2 * q)) & 3u) - 1; }
__host__ __device__ constexpr int CYq(int q) { return (int)((kCYp >> (2 * q)) & 3u) - 1; }
__host__ __device__ constexpr int CZq(int q) { return (int)((kCZp >> (2 * q)) & 3u) - 1; }
__host__ __device__ constexpr int OPPq(int q) { return q == 0 ? 0 : ((q & 1) ? q + 1 : q - 1); }
__device__ __forceinline__ float Wq(int q) {
    return q == 0 ? (1.0f / 3.0f) : (q < 7 ? (1.0f / 18.0f) : (1.0f / 36.0f));
}

constexpr uint32_t kSlow = 0xFFFFFFFEu;

#define FL_POOL_USABLE(ctx, P)                                                                              \
    do {                                                                                                    \
        if ((P)->unusable)                                                                                  \
            return fl_set_error((ctx), FL_E_INVALID_ARG,                                                    \
                                "pool unusable: an earlier call on it failed part-way (destroy it)");       \
    } while (0)
constexpr int kMaxPoolLevels = 14;  // case max_level is 0..13

}  // namespace

// Per-case constants on the device.
struct LbmCaseDev {
    int32_t ext[3];
    int32_t periodic[3];
    int32_t bc[6];
    float wall_u[3], inlet_u[3], init_u[3];
    float omega[20];
    int32_t max_level, has_sphere;
    float sc[3], sr, refine_frac, coarsen_frac, band;
    // solid voxels of the case grid at mask_level (bit (z * Ny + y) * Nx + x,
    // N = ext * 8 << mask_level), or nullptr
    const uint32_t* mask;
    int32_t mask_level, mask_pad;
};

namespace {

// c_q . u as the sum of its non-zero terms in x, y, z order (c = +-1 is a
// sign, so no product is formed; c_0 . u = 0) -- the oracle's cdot().
__device__ __forceinline__ float cdot(int q, float ux, float uy, float uz) {
    const int c[3] = {CXq(q), CYq(q), CZq(q)};
    const float t[3] = {c[0] > 0 ? ux : -ux, c[1] > 0 ? uy : -uy, c[2] > 0 ? uz : -uz};
    float s = 0.0f;
    bool any = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (!c[k]) continue;
        s = any ? s + t[k] : t[k];
        any = true;
    }
    return s;
}

__device__ __forceinline__ float base_of(float ux, float uy, float uz) {
    float usq = ux * ux;
    usq = usq + uy * uy;
    usq = usq + uz * uz;
    float t = 1.5f * usq;
    return 1.0f - t;
}

__device__ __forceinline__ float feq1(int q, float rho, float ux, float uy, float uz, float base) {
    float cu = cdot(q, ux, uy, uz);
    float t = 4.5f * cu;
    t = 3.0f + t;
    t = cu * t;
    t = base + t;
    float wr = Wq(q) * rho;
    return wr * t;
}

__device__ __forceinline__ void moments(const float* f, float& rho, float& jx, float& jy, float& jz) {
    float r = f[0];
#pragma unroll
    for (int q = 1; q < Q; ++q) r = r + f[q];
    float a = f[1] - f[2];
    a = a + (f[7] - f[8]); a = a + (f[9] - f[10]); a = a + (f[11] - f[12]); a = a + (f[13] - f[14]);
    float b = f[3] - f[4];
    b = b + (f[7] - f[8]); b = b + (f[10] - f[9]); b = b + (f[15] - f[16]); b = b + (f[17] - f[18]);
    float c = f[5] - f[6];
    c = c + (f[11] - f[12]); c = c + (f[14] - f[13]); c = c + (f[15] - f[16]); c = c + (f[18] - f[17]);
    rho = r; jx = a; jy = b; jz = c;
}

// Double-single (hi, lo) FP32 pairs for the per-brick sums: Knuth's TwoSum
// (exact rounding error of one addition; needs no FMA contraction) and the
// pair addition with one renormalisation -- about 2^-44 relative per add.
struct DS {
    float hi, lo;
};
__device__ __forceinline__ DS ds_add(DS a, DS b) {
    float s = a.hi + b.hi;
    float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e = e + (a.lo + b.lo);
    float h = s + e;
    return DS{h, e - (h - s)};
}

// Voxel of the case's solid mask under the centre of level-l site (sx, sy, sz):
// a coarser site samples the voxel at its centre (the upper of the two middle
// ones), a finer site the voxel that holds it; sites outside the case grid are
// fluid.
__device__ __forceinline__ bool mask_at(const LbmCaseDev& c, int64_t sx, int64_t sy, int64_t sz, int l) {
    const int64_t G[3] = {sx, sy, sz};
    int64_t v[3], N[3];
    const int sh = c.mask_level - l;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (G[a] < 0 || G[a] >= ((int64_t)c.ext[a] * 8 << l)) return false;
        N[a] = (int64_t)c.ext[a] * 8 << c.mask_level;
        v[a] = sh >= 0 ? (G[a] << sh) + (sh ? (int64_t)1 << (sh - 1) : 0) : G[a] >> -sh;
    }
    const uint64_t i = ((uint64_t)v[2] * (uint64_t)N[1] + (uint64_t)v[1]) * (uint64_t)N[0] + (uint64_t)v[0];
    return (__ldg(c.mask + (i >> 5)) >> (i & 31)) & 1u;
}

// A site is solid inside the case's sphere or on a voxel of its solid mask.
__device__ __forceinline__ bool solid_at(const LbmCaseDev& c, int64_t sx, int64_t sy, int64_t sz, int l) {
    if (c.has_sphere) {
        float inv = 1.0f / (float)(1 << l);
        float px = ((float)sx + 0.5f) * inv, py = ((float)sy + 0.5f) * inv, pz = ((float)sz + 0.5f) * inv;
        float dx = px - c.sc[0], dy = py - c.sc[1], dz = pz - c.sc[2];
        float d2 = dx * dx;
        d2 = d2 + dy * dy;
        d2 = d2 + dz * dz;
        float r2 = c.sr * c.sr;
        if (d2 < r2) return true;
    }
    return c.mask != nullptr && mask_at(c, sx, sy, sz, l);
}

struct StepArgs {
    const uint32_t* list;
    uint32_t count;
    int level, sub;
    const float* R;      // own level, time t (post-collision)
    float* W;            // own level, t + dt
    const float* Cold;   // coarser level at the start of its step
    const float* Cnew;   // coarser level after its step
    const float* Fine;   // finer level, current
    size_t cap;          // bricks per population plane
    const int32_t* bx; const int32_t* by; const int32_t* bz;
    const uint8_t* blevel; const uint16_t* bcase;
    const uint32_t* nbr;  // [n][26][4]
    const LbmCaseDev* cases;
    uint32_t* dev_status;
    const uint64_t* desc;      // stencil descriptors of the general class (k_slow_emit)
    const uint32_t* desc_off;  // per list position: first descriptor; [count] = end
    const uint32_t* smask;     // [n][16]: own sites inside the sphere
    const uint4* qmask;        // [n][128]: per x-quad descriptor bits (4q + i) and first descriptor
    const float* pv;           // descriptor values of this sub-step (k_interface)
    float* part;               // non-null in each level's last sub-step of a level-0 step: the
                               // bricks' conservation sums are written there (brick_sums_store)
};

__device__ __forceinline__ size_t fidx(size_t cap, int q, size_t b, int s) { return ((size_t)q * cap + b) * 512 + s; }

// Could a site of brick b, or a source one site outside it, lie in the sphere?
// Minimal-image distance on periodic axes; a margin of two sites.
__device__ __forceinline__ int brick_near_sphere(const LbmCaseDev& c, int32_t bx, int32_t by, int32_t bz, int l) {
    if (!c.has_sphere) return 0;
    float inv = 1.0f / (float)(1 << l);
    int32_t o[3] = {bx * 8, by * 8, bz * 8};
    float dm = 0.0f;
    for (int ax = 0; ax < 3; ++ax) {
        float lo = (float)(o[ax] - 1) * inv, hi = (float)(o[ax] + 9) * inv;
        float best = 3.0e38f;
        for (int img = -1; img <= 1; ++img) {
            if (img != 0 && !c.periodic[ax]) continue;
            float cc = c.sc[ax] + (float)img * (float)(c.ext[ax] * 8);
            float cl = cc < lo ? lo : (cc > hi ? hi : cc);
            float d = cc - cl;
            best = fminf(best, d * d);
        }
        dm += best;
    }
    float rr = c.sr + 2.0f * inv;
    return dm <= rr * rr ? 1 : 0;
}

// Bit (x+1) + 10(y+1) + 100(z+1) of the 10^3 solid mask of a brick and its
// one-site halo, x, y, z in [-1, 8].
__device__ __forceinline__ int solid_bit(const uint32_t* s_solid, int x, int y, int z) {
    int i = (x + 1) + 10 * (y + 1) + 100 * (z + 1);
    return (s_solid[i >> 5] >> (i & 31)) & 1;
}

// The upstream row of population q for the x-quad (x0..x0+3, y, z) of the
// brick whose 27-entry same-level neighbour row is s_nb: one 128-bit load from
// this brick or a same-level neighbour, the x-shift from the partner lane (the
// other half of the row) by shuffle, and one extra scalar load at the brick's
// x face.  Every entry of s_nb must name a brick (callers replace missing
// neighbours by the brick itself and overwrite those elements afterwards).
template <int Q0, int Q1>
__device__ __forceinline__ void gather_quad(const StepArgs& a, const uint32_t* s_nb, int x0, int y, int z,
                                            float (&f)[Q][4]) {
    const int lane_odd = x0 != 0;
#pragma unroll
    for (int q = Q0; q < Q1; ++q) {
        const int cx = CXq(q), cy = CYq(q), cz = CZq(q);
        const int sy = y - cy, sz = z - cz;
        const int dy = sy >> 3, dz = sz >> 3;
        const int rowoff = (sy & 7) * 8 + (sz & 7) * 64;
        const uint32_t erow = s_nb[(dz + 1) * 9 + (dy + 1) * 3 + 1];
        const float4 A = __ldg((const float4*)(a.R + fidx(a.cap, q, erow, rowoff + x0)));
        if (cx == 0) {
            f[q][0] = A.x; f[q][1] = A.y; f[q][2] = A.z; f[q][3] = A.w;
        } else if (cx == 1) {
            float h = __shfl_xor_sync(0xFFFFFFFFu, A.w, 1);
            if (!lane_odd)  // x = -1: last column of the -x neighbour's row
                h = __ldg(a.R + fidx(a.cap, q, s_nb[(dz + 1) * 9 + (dy + 1) * 3 + 0], rowoff + 7));
            f[q][0] = h; f[q][1] = A.x; f[q][2] = A.y; f[q][3] = A.z;
        } else {
            float h = __shfl_xor_sync(0xFFFFFFFFu, A.x, 1);
            if (lane_odd)  // x = 8: first column of the +x neighbour's row
                h = __ldg(a.R + fidx(a.cap, q, s_nb[(dz + 1) * 9 + (dy + 1) * 3 + 2], rowoff + 0));
            f[q][0] = A.y; f[q][1] = A.z; f[q][2] = A.w; f[q][3] = h;
        }
    }
}

// BGK relaxation of one site in place (solid sites take the rest equilibrium).
__device__ __forceinline__ void relax_site(float (&g)[Q], float omega, bool solid) {
    float rho, jx, jy, jz;
    moments(g, rho, jx, jy, jz);
    float inv = 1.0f / rho;
    float ux = jx * inv, uy = jy * inv, uz = jz * inv;
    float base = base_of(ux, uy, uz);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        float fe = feq1(q, rho, ux, uy, uz, base);
        float dd = fe - g[q];
        dd = omega * dd;
        g[q] = solid ? Wq(q) : g[q] + dd;
    }
}

// The conservation sums of brick b from the values its 128 threads have just
// stored (thread t: the x-quad of k_brick_sums' thread t; bit i of solid4 marks
// site i of the quad solid), in k_brick_sums' arithmetic and order: each
// thread's fluid sites' moments in double-single, a warp xor-reduction, and
// per warp its (hi, lo) pairs of the four sums at part[((b * 4 + warp) * 4 + k)
// * 2] -- FP32 work only; k_chunk_sums combines the warps in FP64.  So part[b]
// holds what k_brick_sums would compute from the stored state.
__device__ __forceinline__ void brick_sums_store(const float (&f)[Q][4], uint32_t solid4, size_t b,
                                                 float* __restrict__ part) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    DS acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if ((solid4 >> i) & 1u) continue;
        float g[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) g[q] = f[q][i];
        float m[4];
        moments(g, m[0], m[1], m[2], m[3]);
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[k] = ds_add(acc[k], DS{m[k], 0.f});
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            DS other{__shfl_xor_sync(0xFFFFFFFFu, acc[k].hi, o), __shfl_xor_sync(0xFFFFFFFFu, acc[k].lo, o)};
            acc[k] = ds_add(acc[k], other);
        }
    }
    if (lane == 0) {
        float4* w = (float4*)(part + (b * 4 + wid) * 8);
        w[0] = make_float4(acc[0].hi, acc[0].lo, acc[1].hi, acc[1].lo);
        w[1] = make_float4(acc[2].hi, acc[2].lo, acc[3].hi, acc[3].lo);
    }
}

// Interior bricks: all 18 face/edge neighbours at this level, no sphere in
// reach.  One CTA per brick (persistent over the level's list), 128 threads;
// thread t owns the x-quad x0 = 4(t & 1), y = (t >> 1) & 7, z = t >> 4.  The
// 27-entry neighbour row comes precomputed (k_brick_table).
template <bool kSums>
__global__ void __launch_bounds__(128, 4) k_collide_fast(StepArgs a, const uint32_t* __restrict__ nb27) {
    __shared__ uint32_t s_nb[27];
    const int l = a.level;
    const int t = threadIdx.x;
    const int x0 = (t & 1) * 4, y = (t >> 1) & 7, z = t >> 4;
    const int own = x0 + 8 * y + 64 * z;
    // software pipeline: the next brick's list entry and neighbour row are
    // loaded while the current brick is gathered and relaxed
    uint32_t w = blockIdx.x;
    uint32_t b = w < a.count ? a.list[w] : 0u;
    uint32_t row = (w < a.count && t < 27) ? nb27[(size_t)b * 28 + t] : 0u;
    for (; w < a.count; w += gridDim.x) {
        if (t < 27) s_nb[t] = row;
        __syncthreads();
        const uint32_t wn = w + gridDim.x;
        const uint32_t bn = wn < a.count ? a.list[wn] : 0u;
        if (wn < a.count && t < 27) row = nb27[(size_t)bn * 28 + t];
        const float omega = a.cases[a.bcase[b]].omega[l];
        float f[Q][4];
        gather_quad<0, Q>(a, s_nb, x0, y, z, f);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float g[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) g[q] = f[q][i];
            relax_site(g, omega, false);
#pragma unroll
            for (int q = 0; q < Q; ++q) f[q][i] = g[q];
        }
#pragma unroll
        for (int q = 0; q < Q; ++q)
            *(float4*)(a.W + fidx(a.cap, q, b, own)) = make_float4(f[q][0], f[q][1], f[q][2], f[q][3]);
        if (kSums) brick_sums_store(f, 0u, b, a.part);
        __syncthreads();
        b = bn;
    }
}

// Stencil descriptors.  For the bricks of the general class, every element
// (population q of site s) whose upstream source is not a plain same-level
// load -- a source across a level interface, outside the domain or inside the
// sphere -- is resolved once per topology into one 64-bit word:
//   bits  0-31  source element (brick * 512 + site) within its population plane
//   bits 32-40  site s, bits 41-45 q, bits 46-48 kind
// so that a step only replays loads and the boundary arithmetic.  The
// resolution follows the oracle's pull() (or_lbm.cpp) branch for branch.
enum : uint32_t {
    kSrcSame = 0,    // R[q][src]: same-level neighbour (across a periodic wrap, or a corner)
    kSrcCoarse = 1,  // coarser neighbour: Cold[q][src], or (Cold + Cnew) / 2 on the second sub-step
    kSrcFine = 2,    // finer neighbour: mean of the 2x2x2 children at src + {0,1,8,9,64,65,72,73}
    kSrcBounce = 3,  // R[opp q][src]: half-way bounce-back (wall, sphere, missing neighbour)
    kSrcWall = 4,    // R[opp q][src] + 6 w_q (c_q . u_wall): moving wall
    kSrcInlet = 5,   // feq(1, u_inlet) (src: own element, names the brick)
    kSrcOutlet = 6,  // R[q][src]: zero-gradient outlet (own site)
};

__device__ __forceinline__ uint64_t make_desc(uint32_t kind, int q, int s, uint32_t src) {
    return (uint64_t)src | ((uint64_t)s << 32) | ((uint64_t)q << 41) | ((uint64_t)kind << 46);
}

struct BrickTopo {
    uint32_t nbr[104];  // 26 directions x 4 sub-slots
    uint8_t nlv[104];   // their levels (0xFF: none)
    uint32_t nb27[27];
    uint32_t solid[32];  // 10^3 bits: the brick and its one-site halo
    int near;
};

__device__ uint64_t resolve_source(const LbmCaseDev& c, const int32_t* bx, const int32_t* by, const int32_t* bz,
                                   uint32_t b, int q, int l, int s, const int64_t* G0, const BrickTopo& T,
                                   uint32_t* dev_status) {
    const uint32_t own = b * 512u + (uint32_t)s;
    const int sx = s & 7, sy = (s >> 3) & 7, sz = s >> 6;
    const int lx = sx - CXq(q), ly = sy - CYq(q), lz = sz - CZq(q);
    int64_t S[3] = {G0[0] + lx, G0[1] + ly, G0[2] + lz};
    int64_t N[3];
    for (int ax = 0; ax < 3; ++ax) N[ax] = ((int64_t)c.ext[ax] * 8) << l;
    int out_face[3] = {-1, -1, -1};
    bool out = false;
    for (int ax = 0; ax < 3; ++ax) {
        if (c.periodic[ax]) continue;
        if (S[ax] < 0) { out_face[ax] = 2 * ax; out = true; }
        else if (S[ax] >= N[ax]) { out_face[ax] = 2 * ax + 1; out = true; }
    }
    if (out) {
        bool inlet = false, outlet = false, moving = false;
        for (int ax = 0; ax < 3; ++ax) {
            if (out_face[ax] < 0) continue;
            int bt = c.bc[out_face[ax]];
            if (bt == 3) inlet = true;
            else if (bt == 4) outlet = true;
            else if (bt == 2) moving = true;
        }
        if (inlet) return make_desc(kSrcInlet, q, s, own);
        if (outlet) return make_desc(kSrcOutlet, q, s, own);
        return make_desc(moving ? kSrcWall : kSrcBounce, q, s, own);
    }
    int64_t Sw[3];  // the source is one site from G: wrapping is one add or subtract
    for (int ax = 0; ax < 3; ++ax)
        Sw[ax] = !c.periodic[ax] ? S[ax] : (S[ax] < 0 ? S[ax] + N[ax] : (S[ax] >= N[ax] ? S[ax] - N[ax] : S[ax]));
    if (T.near && solid_bit(T.solid, lx, ly, lz)) return make_desc(kSrcBounce, q, s, own);
    if (lx >= 0 && lx < 8 && ly >= 0 && ly < 8 && lz >= 0 && lz < 8)
        return make_desc(kSrcSame, q, s, b * 512u + (uint32_t)(lx + 8 * ly + 64 * lz));
    int d[3] = {lx < 0 ? -1 : (lx >= 8 ? 1 : 0), ly < 0 ? -1 : (ly >= 8 ? 1 : 0), lz < 0 ? -1 : (lz >= 8 ? 1 : 0)};
    int L3[3] = {lx, ly, lz};
    int sub_slot = 0, bit = 0;
    for (int ax = 0; ax < 3; ++ax)
        if (d[ax] == 0) { if (L3[ax] >= 4) sub_slot |= 1 << bit; ++bit; }
    int kk = (d[2] + 1) * 9 + (d[1] + 1) * 3 + (d[0] + 1);
    int k = kk < 13 ? kk : kk - 1;
    uint32_t nb = T.nbr[k * 4 + sub_slot];
    if (nb == FL_INVALID_INDEX) return make_desc(kSrcBounce, q, s, own);
    int ln = T.nlv[k * 4 + sub_slot];
    int64_t nx = (int64_t)bx[nb] * 8, ny = (int64_t)by[nb] * 8, nz = (int64_t)bz[nb] * 8;
    if (ln == l)
        return make_desc(kSrcSame, q, s, nb * 512u + (uint32_t)((Sw[0] - nx) + 8 * (Sw[1] - ny) + 64 * (Sw[2] - nz)));
    if (ln == l - 1) {
        int64_t px = (Sw[0] >> 1) - nx, py = (Sw[1] >> 1) - ny, pz = (Sw[2] >> 1) - nz;
        if (px < 0 || px > 7 || py < 0 || py > 7 || pz < 0 || pz > 7) {
            atomicAdd(dev_status + FL_DEVSTAT_BOUNDS, 1u);
            return make_desc(kSrcBounce, q, s, own);
        }
        return make_desc(kSrcCoarse, q, s, nb * 512u + (uint32_t)(px + 8 * py + 64 * pz));
    }
    if (ln == l + 1) {  // children 2S .. 2S+1 per axis; 2S - n is even, so one test per axis
        int64_t px = 2 * Sw[0] - nx, py = 2 * Sw[1] - ny, pz = 2 * Sw[2] - nz;
        if (px < 0 || px > 6 || py < 0 || py > 6 || pz < 0 || pz > 6) {
            atomicAdd(dev_status + FL_DEVSTAT_BOUNDS, 1u);
            return make_desc(kSrcBounce, q, s, own);
        }
        return make_desc(kSrcFine, q, s, nb * 512u + (uint32_t)(px + 8 * py + 64 * pz));
    }
    atomicAdd(dev_status + FL_DEVSTAT_LEVEL_JUMP, 1u);
    return make_desc(kSrcBounce, q, s, own);
}

// The descriptors of the general bricks, from k_brick_table's tables: one
// CTA per brick, one thread per descriptor.  Descriptor k of a brick lies in
// the x-quad with the largest first offset <= k (qmask .w); inside the quad
// they run q-major, then site.  Written to desc + off[p] + k.
__global__ void __launch_bounds__(256, 4) k_slow_emit(size_t ng, const uint32_t* __restrict__ gen,
                                                      const uint32_t* __restrict__ list,
                                                      const uint32_t* __restrict__ nbr,
                                                      const uint8_t* __restrict__ blevel,
                                                      const int32_t* __restrict__ bx, const int32_t* __restrict__ by,
                                                      const int32_t* __restrict__ bz,
                                                      const uint16_t* __restrict__ bcase,
                                                      const LbmCaseDev* __restrict__ cases,
                                                      const uint8_t* __restrict__ mnear,
                                                      const uint32_t* __restrict__ hsolid,
                                                      const uint4* __restrict__ qmask,
                                                      const uint32_t* __restrict__ cnt,
                                                      const uint32_t* __restrict__ off,
                                                      uint64_t* __restrict__ desc, uint32_t* dev_status) {
    __shared__ BrickTopo T;
    __shared__ uint4 Qm[128];
    const int t = threadIdx.x;
    for (size_t j = blockIdx.x; j < ng; j += gridDim.x) {
        const size_t p = gen[j];
        const uint32_t b = list[p];
        const int l = blevel[b];
        const LbmCaseDev& c = cases[bcase[b]];
        if (t < 104) {
            uint32_t nb = nbr[(size_t)b * 104 + t];
            T.nbr[t] = nb;
            T.nlv[t] = nb == FL_INVALID_INDEX ? 0xFF : blevel[nb];
        }
        if (t < 128) Qm[t] = qmask[(size_t)b * 128 + t];
        if (t >= 128 && t < 160) T.solid[t - 128] = hsolid[(size_t)b * 32 + (t - 128)];
        if (t == 160) T.near = brick_near_sphere(c, bx[b], by[b], bz[b], l) | (mnear ? mnear[b] & 1 : 0);
        const uint32_t total = cnt[p];
        uint64_t* out = desc + off[p];
        const int64_t G0[3] = {(int64_t)bx[b] * 8, (int64_t)by[b] * 8, (int64_t)bz[b] * 8};
        __syncthreads();
        for (uint32_t k = t; k < total; k += blockDim.x) {
            int lo = 0, hi = 127;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (Qm[mid].w <= k) lo = mid;
                else hi = mid - 1;
            }
            const uint4 w = Qm[lo];
            uint32_t r = k - w.w;
            int q = 1, i = 0;
            for (; q < Q; ++q) {
                const uint32_t word = (q >> 3) == 0 ? w.x : ((q >> 3) == 1 ? w.y : w.z);
                const uint32_t nib = (word >> ((q & 7) * 4)) & 0xFu;
                const uint32_t cq = __popc(nib);
                if (r < cq) {
                    uint32_t v = nib;
                    for (uint32_t skip = 0; skip < r; ++skip) v &= v - 1u;
                    i = __ffs(v) - 1;
                    break;
                }
                r -= cq;
            }
            if (q >= Q) {  // the quad masks do not hold k (not reached when they match cnt)
                atomicAdd(dev_status + FL_DEVSTAT_BOUNDS, 1u);
                q = 0;
            }
            out[k] = resolve_source(c, bx, by, bz, b, q, l, lo * 4 + i, G0, T, dev_status);
        }
        __syncthreads();
    }
}

// Value of one stencil descriptor at this sub-step.
__device__ __forceinline__ float desc_value(const StepArgs& a, uint64_t d, size_t plane) {
    const uint32_t src = (uint32_t)d;
    const int q = (int)((d >> 41) & 31u);
    const uint32_t kind = (uint32_t)(d >> 46) & 7u;
    float v;
    if (kind == kSrcSame || kind == kSrcOutlet) {
        v = a.R[q * plane + src];
    } else if (kind == kSrcBounce) {
        v = a.R[OPPq(q) * plane + src];
    } else if (kind == kSrcCoarse) {
        v = a.Cold[q * plane + src];
        if (a.sub) {
            float tt = v + a.Cnew[q * plane + src];
            v = tt * 0.5f;
        }
    } else if (kind == kSrcFine) {
        const float* F = a.Fine + q * plane + src;
        float sum = 0.0f;
#pragma unroll
        for (int kq = 0; kq < 8; ++kq) sum = sum + F[(kq & 1) + 8 * ((kq >> 1) & 1) + 64 * (kq >> 2)];
        v = sum * 0.125f;
    } else {
        const LbmCaseDev& c = a.cases[a.bcase[src >> 9]];
        if (kind == kSrcWall) {
            v = a.R[OPPq(q) * plane + src];
            float cu = cdot(q, c.wall_u[0], c.wall_u[1], c.wall_u[2]);
            float tt = 6.0f * Wq(q);
            tt = tt * cu;
            v = v + tt;
        } else {
            float base = base_of(c.inlet_u[0], c.inlet_u[1], c.inlet_u[2]);
            v = feq1(q, 1.0f, c.inlet_u[0], c.inlet_u[1], c.inlet_u[2], base);
        }
    }
    return v;
}

// The values of a level's stencil descriptors [d0, d1) at this sub-step,
// one thread per descriptor, into pv (same indices).
__global__ void __launch_bounds__(256) k_interface(StepArgs a, uint32_t d0, uint32_t d1, float* __restrict__ pv) {
    const size_t plane = a.cap * 512;
    for (uint32_t k = d0 + blockIdx.x * blockDim.x + threadIdx.x; k < d1; k += gridDim.x * blockDim.x)
        pv[k] = desc_value(a, __ldg(a.desc + k), plane);
}

// Bricks at a level interface, a domain boundary or near the sphere, in the
// interior kernel's layout (x-quads in registers, 128 threads, 4 CTAs/SM):
// the quad's rows are gathered with missing same-level neighbours replaced by
// the brick itself (every load stays in bounds); each thread then replaces
// its elements flagged in its quad mask -- bit 4q + i, ordered like the
// descriptors, from the quad's first descriptor on -- by the descriptor
// values k_interface computed for this sub-step, and relaxes the quad.  Sites
// inside the sphere take the rest equilibrium.
template <bool kSums>
__global__ void __launch_bounds__(128, 4) k_collide_general(StepArgs a, const uint32_t* __restrict__ nb27) {
    __shared__ uint32_t s_nb[27];
    const int l = a.level;
    const int t = threadIdx.x;
    const int x0 = (t & 1) * 4, y = (t >> 1) & 7, z = t >> 4;
    const int own = x0 + 8 * y + 64 * z;
    uint32_t w = blockIdx.x;
    uint32_t b = w < a.count ? a.list[w] : 0u;
    uint32_t row = (w < a.count && t < 27) ? nb27[(size_t)b * 28 + t] : 0u;
    for (; w < a.count; w += gridDim.x) {
        if (t < 27) s_nb[t] = row == kSlow ? b : row;
        __syncthreads();
        const uint32_t wn = w + gridDim.x;
        const uint32_t bn = wn < a.count ? a.list[wn] : 0u;
        if (wn < a.count && t < 27) row = nb27[(size_t)bn * 28 + t];
        const uint4 qm = a.qmask[(size_t)b * 128 + t];
        const uint32_t sw = a.smask[(size_t)b * 16 + (own >> 5)];
        const float omega = a.cases[a.bcase[b]].omega[l];
        float f[Q][4];
        gather_quad<0, Q>(a, s_nb, x0, y, z, f);
        const float* pv = a.pv + a.desc_off[w];
        uint32_t r = qm.w;
        if (qm.x) {
#pragma unroll
            for (int q = 0; q < 8; ++q)
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    if ((qm.x >> (q * 4 + i)) & 1u) f[q][i] = __ldg(pv + r++);
        }
        if (qm.y) {
#pragma unroll
            for (int q = 8; q < 16; ++q)
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    if ((qm.y >> (q * 4 + i - 32)) & 1u) f[q][i] = __ldg(pv + r++);
        }
        if (qm.z) {
#pragma unroll
            for (int q = 16; q < Q; ++q)
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    if ((qm.z >> (q * 4 + i - 64)) & 1u) f[q][i] = __ldg(pv + r++);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float g[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) g[q] = f[q][i];
            relax_site(g, omega, (sw >> ((own + i) & 31)) & 1u);
#pragma unroll
            for (int q = 0; q < Q; ++q) f[q][i] = g[q];
        }
#pragma unroll
        for (int q = 0; q < Q; ++q)
            *(float4*)(a.W + fidx(a.cap, q, b, own)) = make_float4(f[q][0], f[q][1], f[q][2], f[q][3]);
        if (kSums) brick_sums_store(f, (sw >> (own & 31)) & 0xFu, b, a.part);
        __syncthreads();
        b = bn;
    }
}

// Staged variant of both collide kernels (fl_pool_set_staging): the brick's
// own 19 population planes (2 KB each, contiguous in f[q][brick][site]) --
// and, for general bricks with kDesc, its 128 quad masks and the values of its
// stencil descriptors -- arrive in shared memory by bulk copies (the TMA
// engine's linear mode) on an mbarrier, issued one brick ahead by thread 0
// while the block relaxes and stores the current brick.  Rows of the brick's
// own planes are then read from shared memory; halo rows and x-face columns
// of neighbours stay global loads, as in gather_quad.  Same arithmetic in the
// same order: the results equal the register kernels' bit for bit.
constexpr uint32_t kStagePlaneBytes = Q * 2048;
constexpr uint32_t kStagePv = 2048;  // descriptor values staged per brick (more: read from global)

__host__ __device__ constexpr uint32_t stage_bytes(bool general, bool desc) {
    return kStagePlaneBytes + (general && desc ? 2048 + kStagePv * 4 : 0);
}

template <int Q0, int Q1>
__device__ __forceinline__ void gather_quad_staged(const StepArgs& a, const uint32_t* s_nb, const float* s_f, int x0,
                                                   int y, int z, float (&f)[Q][4]) {
    const int lane_odd = x0 != 0;
#pragma unroll
    for (int q = Q0; q < Q1; ++q) {
        const int cx = CXq(q), cy = CYq(q), cz = CZq(q);
        const int sy = y - cy, sz = z - cz;
        const int dy = sy >> 3, dz = sz >> 3;
        const int rowoff = (sy & 7) * 8 + (sz & 7) * 64;
        const uint32_t erow = s_nb[(dz + 1) * 9 + (dy + 1) * 3 + 1];
        float4 A;
        if (dy == 0 && dz == 0) A = *(const float4*)(s_f + q * 512 + rowoff + x0);
        else A = __ldg((const float4*)(a.R + fidx(a.cap, q, erow, rowoff + x0)));
        if (cx == 0) {
            f[q][0] = A.x; f[q][1] = A.y; f[q][2] = A.z; f[q][3] = A.w;
        } else if (cx == 1) {
            float h = __shfl_xor_sync(0xFFFFFFFFu, A.w, 1);
            if (!lane_odd) h = __ldg(a.R + fidx(a.cap, q, s_nb[(dz + 1) * 9 + (dy + 1) * 3 + 0], rowoff + 7));
            f[q][0] = h; f[q][1] = A.x; f[q][2] = A.y; f[q][3] = A.z;
        } else {
            float h = __shfl_xor_sync(0xFFFFFFFFu, A.x, 1);
            if (lane_odd) h = __ldg(a.R + fidx(a.cap, q, s_nb[(dz + 1) * 9 + (dy + 1) * 3 + 2], rowoff + 0));
            f[q][0] = A.y; f[q][1] = A.z; f[q][2] = A.w; f[q][3] = h;
        }
    }
}

// The elements of an x-quad flagged in its quad mask qm (bit 4q + i, ordered
// like the descriptors, from the quad's first descriptor qm.w on) replaced by
// their descriptor values vals[qm.w ...]: from shared memory, or from global
// memory through the read-only path.
__device__ __forceinline__ void replace_described(const uint4 qm, const float* vals, float (&f)[Q][4]) {
    uint32_t r = qm.w;
    if (qm.x) {
#pragma unroll
        for (int q = 0; q < 8; ++q)
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if ((qm.x >> (q * 4 + i)) & 1u) f[q][i] = vals[r++];
    }
    if (qm.y) {
#pragma unroll
        for (int q = 8; q < 16; ++q)
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if ((qm.y >> (q * 4 + i - 32)) & 1u) f[q][i] = vals[r++];
    }
    if (qm.z) {
#pragma unroll
        for (int q = 16; q < Q; ++q)
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if ((qm.z >> (q * 4 + i - 64)) & 1u) f[q][i] = vals[r++];
    }
}

__device__ __forceinline__ void replace_described_global(const uint4 qm, const float* __restrict__ vals,
                                                         float (&f)[Q][4]) {
    uint32_t r = qm.w;
    if (qm.x) {
#pragma unroll
        for (int q = 0; q < 8; ++q)
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if ((qm.x >> (q * 4 + i)) & 1u) f[q][i] = __ldg(vals + r++);
    }
    if (qm.y) {
#pragma unroll
        for (int q = 8; q < 16; ++q)
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if ((qm.y >> (q * 4 + i - 32)) & 1u) f[q][i] = __ldg(vals + r++);
    }
    if (qm.z) {
#pragma unroll
        for (int q = 16; q < Q; ++q)
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if ((qm.z >> (q * 4 + i - 64)) & 1u) f[q][i] = __ldg(vals + r++);
    }
}

struct StageState {
    uint64_t bar;
    uint32_t pv_off;  // the brick's first descriptor within the staged values
    uint32_t pv_n;    // staged values (0: read them from global)
};

// Thread 0: arm the barrier and issue the copies of list position w (brick b).
template <bool kGeneral, bool kDesc>
__device__ __forceinline__ void stage_issue(const StepArgs& a, uint32_t w, uint32_t b, unsigned char* s_dyn,
                                            StageState* st) {
    uint32_t bytes = kStagePlaneBytes, pv0 = 0, pvn = 0;
    if (kGeneral && kDesc) {
        bytes += 2048;
        const uint32_t d0 = a.desc_off[w], d1 = a.desc_off[w + 1];
        const uint32_t s0 = d0 & ~3u, n = (d1 - s0 + 3u) & ~3u;  // 16-byte aligned superset (the buffer has slack)
        if (d1 > d0 && n <= kStagePv) {
            pv0 = s0;
            pvn = n;
            bytes += n * 4;
        }
        st->pv_off = d0 - s0;
        st->pv_n = pvn;
    }
    flbulk::mbar_arrive_expect_tx(&st->bar, bytes);
#pragma unroll 1
    for (int q = 0; q < Q; ++q)
        flbulk::copy_g2s(s_dyn + q * 2048, a.R + fidx(a.cap, q, b, 0), 2048, &st->bar);
    if (kGeneral && kDesc) {
        flbulk::copy_g2s(s_dyn + kStagePlaneBytes, a.qmask + (size_t)b * 128, 2048, &st->bar);
        if (pvn) flbulk::copy_g2s(s_dyn + kStagePlaneBytes + 2048, a.pv + pv0, pvn * 4, &st->bar);
    }
}

template <bool kGeneral, bool kDesc, bool kSums>
__global__ void __launch_bounds__(128, 4) k_collide_staged(StepArgs a, const uint32_t* __restrict__ nb27) {
    extern __shared__ __align__(128) unsigned char s_dyn[];
    __shared__ uint32_t s_nb[27];
    __shared__ StageState st;
    const float* s_f = (const float*)s_dyn;
    const uint4* s_qm = (const uint4*)(s_dyn + kStagePlaneBytes);
    const float* s_pv = (const float*)(s_dyn + kStagePlaneBytes + 2048);
    const int l = a.level;
    const int t = threadIdx.x;
    const int x0 = (t & 1) * 4, y = (t >> 1) & 7, z = t >> 4;
    const int own = x0 + 8 * y + 64 * z;
    if (t == 0) flbulk::mbar_init(&st.bar, 1);
    __syncthreads();
    uint32_t w = blockIdx.x;
    uint32_t b = w < a.count ? a.list[w] : 0u;
    if (t == 0 && w < a.count) stage_issue<kGeneral, kDesc>(a, w, b, s_dyn, &st);
    uint32_t row = (w < a.count && t < 27) ? nb27[(size_t)b * 28 + t] : 0u;
    uint32_t phase = 0;
    for (; w < a.count; w += gridDim.x) {
        if (t < 27) s_nb[t] = (kGeneral && row == kSlow) ? b : row;
        __syncthreads();
        const uint32_t wn = w + gridDim.x;
        const uint32_t bn = wn < a.count ? a.list[wn] : 0u;
        if (wn < a.count && t < 27) row = nb27[(size_t)bn * 28 + t];
        const float omega = a.cases[a.bcase[b]].omega[l];
        const uint32_t sw = kGeneral ? a.smask[(size_t)b * 16 + (own >> 5)] : 0u;
        const uint4 qm_g = (kGeneral && !kDesc) ? a.qmask[(size_t)b * 128 + t] : make_uint4(0, 0, 0, 0);
        const bool ok = flbulk::mbar_wait(&st.bar, phase, FL_SPIN_LIMIT);
        if (__syncthreads_or(!ok)) {
            // a copy never landed: report it, give the copies one more bounded
            // wait, and leave without touching the output
            if (t == 0) {
                atomicAdd(a.dev_status + FL_DEVSTAT_TIMEOUT, 1u);
                flbulk::mbar_wait(&st.bar, phase, FL_SPIN_LIMIT);
            }
            return;
        }
        phase ^= 1u;
        float f[Q][4];
        gather_quad_staged<0, Q>(a, s_nb, s_f, x0, y, z, f);
        if (kGeneral) {
            const uint4 qm = kDesc ? s_qm[t] : qm_g;
            if (kDesc && st.pv_n != 0)
                replace_described(qm, s_pv + st.pv_off, f);  // shared-memory reads
            else
                replace_described_global(qm, a.pv + a.desc_off[w], f);
        }
        __syncthreads();  // every read of the staged brick and of s_nb is done
        if (t == 0 && wn < a.count) {
            // order the block's shared-memory reads above before the copies that overwrite the stage
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            stage_issue<kGeneral, kDesc>(a, wn, bn, s_dyn, &st);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float g[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) g[q] = f[q][i];
            relax_site(g, omega, kGeneral && ((sw >> ((own + i) & 31)) & 1u));
#pragma unroll
            for (int q = 0; q < Q; ++q) f[q][i] = g[q];
        }
#pragma unroll
        for (int q = 0; q < Q; ++q)
            *(float4*)(a.W + fidx(a.cap, q, b, own)) = make_float4(f[q][0], f[q][1], f[q][2], f[q][3]);
        if (kSums) brick_sums_store(f, kGeneral ? (sw >> (own & 31)) & 0xFu : 0u, b, a.part);
        b = bn;
    }
}

// Every brick's populations, from the buffer its level's parity names (bit l
// of odd: level l's current populations are in f1), into dst, a float4 per
// thread: the current state in one buffer for a single device-to-host copy.
__global__ void k_gather_current(const float* __restrict__ f0, const float* __restrict__ f1, float* __restrict__ dst,
                                 size_t cap, size_t n, const uint8_t* __restrict__ level, uint32_t odd) {
    const size_t total = (size_t)Q * n * 128;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        const size_t qb = t >> 7, q = qb / n, b = qb - q * n;
        const size_t off = (q * cap + b) * 512 + (t & 127) * 4;
        const float* src = ((odd >> level[b]) & 1u) ? f1 : f0;
        *(float4*)(dst + off) = *(const float4*)(src + off);
    }
}

// The populations of the listed bricks from one buffer to the other, a float4
// per thread.
__global__ void k_copy_bricks(const float* __restrict__ src, float* __restrict__ dst, size_t cap,
                              const uint32_t* __restrict__ list, uint32_t count) {
    const size_t total = (size_t)count * Q * 128;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        const size_t w = t / (Q * 128);
        const int r = (int)(t - w * (Q * 128));
        const size_t off = ((size_t)(r >> 7) * cap + list[w]) * 512 + (size_t)(r & 127) * 4;
        *(float4*)(dst + off) = *(const float4*)(src + off);
    }
}

// Bricks whose 512 sites all lie in the sphere: rest equilibrium, no reads.
__global__ void k_collide_solid(StepArgs a) {
    size_t total = (size_t)a.count * 512;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        uint32_t b = a.list[t >> 9];
        int s = (int)(t & 511);
#pragma unroll
        for (int q = 0; q < Q; ++q) a.W[fidx(a.cap, q, b, s)] = Wq(q);
    }
}

// Per brick of a case with a solid mask (one warp per brick): bit 0 when a site
// of the brick or of its one-site halo (periodic axes wrapped) is solid, bit 1
// when all 512 of its own sites are; 0 for bricks of the other cases.
__global__ void k_mask_near(size_t n, const uint8_t* __restrict__ blevel, const int32_t* __restrict__ bx,
                            const int32_t* __restrict__ by, const int32_t* __restrict__ bz,
                            const uint16_t* __restrict__ bcase, const LbmCaseDev* __restrict__ cases,
                            uint8_t* __restrict__ mnear) {
    const int lane = threadIdx.x & 31;
    const size_t warps = (size_t)gridDim.x * (blockDim.x >> 5);
    for (size_t b = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < n; b += warps) {
        const LbmCaseDev& c = cases[bcase[b]];
        if (!c.mask) {
            if (lane == 0) mnear[b] = 0;
            continue;
        }
        const int l = blevel[b];
        const int64_t G0[3] = {(int64_t)bx[b] * 8, (int64_t)by[b] * 8, (int64_t)bz[b] * 8};
        bool any = false, all = true;
        for (int i = lane; i < 1000; i += 32) {
            const int h[3] = {i % 10, (i / 10) % 10, i / 100};
            int64_t G[3];
            for (int ax = 0; ax < 3; ++ax) {
                G[ax] = G0[ax] + h[ax] - 1;
                if (!c.periodic[ax]) continue;
                const int64_t N = ((int64_t)c.ext[ax] * 8) << l;
                G[ax] = G[ax] < 0 ? G[ax] + N : (G[ax] >= N ? G[ax] - N : G[ax]);
            }
            const bool sol = solid_at(c, G[0], G[1], G[2], l);
            const bool own = h[0] >= 1 && h[0] <= 8 && h[1] >= 1 && h[1] <= 8 && h[2] >= 1 && h[2] <= 8;
            any = any || sol;
            all = all && (sol || !own);
        }
        any = __any_sync(0xFFFFFFFFu, any);
        all = __all_sync(0xFFFFFFFFu, all);
        if (lane == 0) mnear[b] = (uint8_t)((any ? 1 : 0) | (all ? 2 : 0));
    }
}

// One warp per brick.  Lane d < 27 resolves entry d of the brick's 27-entry
// same-level neighbour row (centre = the brick, kSlow where the neighbour is
// missing or at another level; lane 27 writes the padding word).  A brick
// with a slow face or edge neighbour, or near a solid, is general (class 1);
// a general brick whose 512 sites are all solid is class 2; the rest are
// interior (class 0).  For each class-1 brick the warp then builds its
// stencil-descriptor tables: the solid bits of the brick and its one-site
// halo (hsolid, 32 words; zero away from solids), the own-site solid words
// (smask, 16), per x-quad the 76 bits "element (q, site) needs a descriptor"
// (bit 4q + i) with the quad's first descriptor (qmask, 128 entries, in site
// order), the descriptor count (cnt, by brick) and the fluid sites.  Lane L
// owns sites 16L .. 16L + 15, i.e. the quads 4L .. 4L + 3.  Own sites inside
// a solid get no descriptors: their relaxation ignores what they pulled.
__global__ void __launch_bounds__(256) k_brick_table(size_t n, const uint32_t* __restrict__ nbr,
                                                     const uint8_t* __restrict__ blevel,
                                                     const int32_t* __restrict__ bx, const int32_t* __restrict__ by,
                                                     const int32_t* __restrict__ bz, const uint16_t* __restrict__ bcase,
                                                     const LbmCaseDev* __restrict__ cases,
                                                     const uint8_t* __restrict__ mnear, uint32_t* __restrict__ nb27,
                                                     uint8_t* __restrict__ bclass, uint32_t* __restrict__ cnt,
                                                     uint32_t* __restrict__ smask, uint4* __restrict__ qmask,
                                                     uint32_t* __restrict__ hsolid, uint32_t* __restrict__ fluid) {
    __shared__ uint32_t s_solid[8][32];
    __shared__ uint32_t s_wq[8][32 * 12];
    const int lane = threadIdx.x & 31;
    uint32_t* S = s_solid[(threadIdx.x >> 5) & 7];
    const size_t warps = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t b = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < n; b += warps) {
        const int l = blevel[b];
        const LbmCaseDev& c = cases[bcase[b]];
        uint32_t e = lane == 27 ? 0u : (uint32_t)b;
        bool face_slow = false;
        if (lane < 27 && lane != 13) {
            const int k = lane < 13 ? lane : lane - 1;
            const uint32_t nb = nbr[(b * 26 + k) * 4];
            e = (nb != FL_INVALID_INDEX && blevel[nb] == l) ? nb : kSlow;
            const int dx = lane % 3 - 1, dy = (lane / 3) % 3 - 1, dz = lane / 9 - 1;
            face_slow = !(dx != 0 && dy != 0 && dz != 0) && e == kSlow;
        }
        if (lane < 28) nb27[b * 28 + lane] = e;
        const uint32_t slow_dirs = __ballot_sync(0xFFFFFFFFu, lane < 27 && e == kSlow);
        const int near = brick_near_sphere(c, bx[b], by[b], bz[b], l) | (mnear ? mnear[b] & 1 : 0);
        int general = (__any_sync(0xFFFFFFFFu, face_slow) ? 1 : 0) | near;
        if (general) {  // all 512 sites solid: the brick only ever holds the rest equilibrium
            bool all;
            if (c.mask) {
                all = mnear && ((mnear[b] >> 1) & 1);
            } else {
                bool mine = c.has_sphere != 0;
                for (int s = lane; s < 512 && mine; s += 32)
                    mine = solid_at(c, (int64_t)bx[b] * 8 + (s & 7), (int64_t)by[b] * 8 + ((s >> 3) & 7),
                                    (int64_t)bz[b] * 8 + (s >> 6), l);
                all = __all_sync(0xFFFFFFFFu, mine);
            }
            if (all) general = 2;
        }
        if (lane == 0) bclass[b] = (uint8_t)general;
        if (general != 1) continue;  // uniform over the warp
        const int64_t G0[3] = {(int64_t)bx[b] * 8, (int64_t)by[b] * 8, (int64_t)bz[b] * 8};
        uint32_t word = 0;  // word `lane` of the 10^3 halo bits
        if (near) {
            for (int k = 0; k < 32; ++k) {
                const int i = 32 * k + lane;
                bool sd = false;
                if (i < 1000) {
                    int64_t G[3] = {G0[0] + i % 10 - 1, G0[1] + (i / 10) % 10 - 1, G0[2] + i / 100 - 1};
                    for (int ax = 0; ax < 3; ++ax) {
                        if (!c.periodic[ax]) continue;
                        const int64_t N = ((int64_t)c.ext[ax] * 8) << l;
                        G[ax] = G[ax] < 0 ? G[ax] + N : (G[ax] >= N ? G[ax] - N : G[ax]);
                    }
                    sd = solid_at(c, G[0], G[1], G[2], l);
                }
                const uint32_t wd = __ballot_sync(0xFFFFFFFFu, sd);
                if (lane == k) word = wd;
            }
        }
        S[lane] = word;
        hsolid[b * 32 + lane] = word;
        __syncwarp();
        const int z = lane >> 2, y0 = 2 * (lane & 3);
        uint32_t* W = s_wq[(threadIdx.x >> 5) & 7] + lane * 12;  // this lane's 4 quads x 3 mask words
        uint32_t mine = 0, own16 = 0, qcs = 0;                    // qcs: per-quad counts (<= 72), a byte each
#pragma unroll 1
        for (int u = 0; u < 4; ++u) {  // quad 4L + u: row y0 + (u >> 1), x = 4 (u & 1) .. + 3
            const int y = y0 + (u >> 1);
            uint32_t w0 = 0u, w1 = 0u, w2 = 0u, qc = 0u;
#pragma unroll 1
            for (int k = 0; k < 4; ++k) {
                const int x = 4 * (u & 1) + k;
                const bool own_solid = near && solid_bit(S, x, y, z);
                own16 |= (uint32_t)own_solid << (4 * u + k);
                if (own_solid) continue;
#pragma unroll
                for (int q = 1; q < Q; ++q) {
                    const int xi = x - CXq(q), yi = y - CYq(q), zi = z - CZq(q);
                    const int dir = ((zi >> 3) + 1) * 9 + ((yi >> 3) + 1) * 3 + ((xi >> 3) + 1);
                    const bool sl = ((slow_dirs >> dir) & 1u) || (near && solid_bit(S, xi, yi, zi));
                    const uint32_t bit = (uint32_t)sl << ((q & 7) * 4 + k);  // bit 4q + k of the 96
                    if ((q >> 3) == 0) w0 |= bit;
                    else if ((q >> 3) == 1) w1 |= bit;
                    else w2 |= bit;
                    qc += sl ? 1u : 0u;
                }
            }
            W[3 * u] = w0;
            W[3 * u + 1] = w1;
            W[3 * u + 2] = w2;
            qcs |= qc << (8 * u);
            mine += qc;
        }
        uint32_t incl = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += v;
        }
        uint32_t base = incl - mine;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            qmask[b * 128 + 4 * lane + u] = make_uint4(W[3 * u], W[3 * u + 1], W[3 * u + 2], base);
            base += (qcs >> (8 * u)) & 0xFFu;
        }
        const uint32_t partner = __shfl_xor_sync(0xFFFFFFFFu, own16, 1);
        if (!(lane & 1)) smask[b * 16 + (lane >> 1)] = own16 | (partner << 16);
        const uint32_t nsolid = __reduce_add_sync(0xFFFFFFFFu, (uint32_t)__popc(own16));
        if (lane == 31) cnt[b] = incl;
        if (lane == 0) fluid[b] = 512u - nsolid;
        __syncwarp();  // S is rewritten for the next brick
    }
}

// Small per-topology results read back by the host: bricks and fluid sites
// per list bin (bin = level * 3 + class), the descriptor range of each level's
// general bricks and an error word.
constexpr int kBins = 3 * kMaxPoolLevels;
struct TopoCounters {
    uint32_t count[kBins];
    uint32_t err;  // bit 0: a level above the pool maximum, bit 1: a case id out of range, bit 2: case ids out of order
    uint32_t lvl_desc[kMaxPoolLevels + 1];
    unsigned long long fluid[kBins];
    unsigned long long desc64;  // descriptors, summed in 64 bits (the offsets are 32-bit)
};

// Per brick: its list bin as a sort key and its index as the value, the bin
// counts, and the case ranges (a pool keeps its bricks in case order:
// case_begin[c] = first brick of case c, case_begin[ncases] = n).
__global__ void k_topo_bins(size_t n, const uint8_t* __restrict__ blevel, const uint8_t* __restrict__ bclass,
                            const uint16_t* __restrict__ bcase, int maxL, uint32_t ncases,
                            uint64_t* __restrict__ keys, uint32_t* __restrict__ ids, TopoCounters* tc,
                            uint32_t* __restrict__ case_begin) {
    __shared__ uint32_t h[kBins];
    for (int i = threadIdx.x; i < kBins; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t rounds = (n + stride - 1) / stride;  // whole warps stay converged for the match below
    for (size_t r = 0; r < rounds; ++r) {
        const size_t i = r * stride + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
        uint32_t bin = 0xFFFFFFFFu;
        if (i < n) {
            int l = blevel[i], k = bclass[i];
            k = k > 2 ? 1 : k;
            if (l > maxL) {
                atomicOr(&tc->err, 1u);
                l = maxL;
            }
            bin = (uint32_t)(l * 3 + k);
            keys[i] = bin;
            ids[i] = (uint32_t)i;
            const uint32_t c = bcase[i], prev = i ? bcase[i - 1] : 0u;
            if (c >= ncases) {
                atomicOr(&tc->err, 2u);
            } else if (i && c < prev) {
                atomicOr(&tc->err, 4u);
            } else {
                for (uint32_t cc = i ? prev + 1 : 0u; cc <= c; ++cc) case_begin[cc] = (uint32_t)i;
                if (i == n - 1)
                    for (uint32_t cc = c + 1; cc <= ncases; ++cc) case_begin[cc] = (uint32_t)n;
            }
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, bin);
        if (bin != 0xFFFFFFFFu && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&h[bin], __popc(peers));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kBins; i += blockDim.x)
        if (h[i]) atomicAdd(&tc->count[i], h[i]);
}

// Positions in the level lists of the general bricks, level by level:
// general brick j of level l (base[l] <= j < base[l + 1]) sits at
// start[l] + j - base[l].  Its descriptor count moves from brick order (cnt_b)
// to list order (cnt, zero elsewhere).
struct GenTable {
    uint32_t base[kMaxPoolLevels + 1];
    uint32_t start[kMaxPoolLevels];
    int levels;
};

__global__ void k_gen_positions(size_t ng, const __grid_constant__ GenTable t, const uint32_t* __restrict__ list,
                                const uint32_t* __restrict__ cnt_b, uint32_t* __restrict__ gen,
                                uint32_t* __restrict__ cnt) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < ng; j += stride) {
        int l = 0;
        while (l + 1 < t.levels && j >= t.base[l + 1]) ++l;
        const uint32_t p = t.start[l] + (uint32_t)(j - t.base[l]);
        gen[j] = p;
        cnt[p] = cnt_b[list[p]];
    }
}

// Fluid sites per bin (interior bricks are all fluid, all-solid bricks none,
// general bricks as counted by k_brick_table), the 64-bit descriptor total and
// each level's first descriptor (t.start[l] = first list position of the
// level's general bricks; off holds n + 1 exclusive offsets).
__global__ void k_topo_sums(size_t n, const uint8_t* __restrict__ blevel, const uint8_t* __restrict__ bclass,
                            const uint32_t* __restrict__ fluid, const uint32_t* __restrict__ cnt,
                            const uint32_t* __restrict__ off, const __grid_constant__ GenTable t, int maxL,
                            TopoCounters* tc) {
    __shared__ unsigned long long h[kBins];
    __shared__ unsigned long long dsum;
    for (int i = threadIdx.x; i < kBins; i += blockDim.x) h[i] = 0ull;
    if (threadIdx.x == 0) dsum = 0ull;
    if (blockIdx.x == 0 && threadIdx.x <= maxL + 1)
        tc->lvl_desc[threadIdx.x] = off[threadIdx.x <= maxL ? t.start[threadIdx.x] : (uint32_t)n];
    __syncthreads();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    unsigned long long dmine = 0ull;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        int l = blevel[i], k = bclass[i];
        k = k > 2 ? 1 : k;
        l = l > maxL ? maxL : l;
        const uint32_t f = k == 1 ? fluid[i] : (k == 0 ? 512u : 0u);
        if (f) atomicAdd(&h[l * 3 + k], (unsigned long long)f);
        dmine += cnt[i];
    }
    if (dmine) atomicAdd(&dsum, dmine);
    __syncthreads();
    for (int i = threadIdx.x; i < kBins; i += blockDim.x)
        if (h[i]) atomicAdd(&tc->fluid[i], h[i]);
    if (threadIdx.x == 0 && dsum) atomicAdd(&tc->desc64, dsum);
}

__global__ void k_init_populations(float* f, size_t cap, size_t n, const uint16_t* bcase, const LbmCaseDev* cases) {
    size_t total = n * 512;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        size_t b = t >> 9;
        int s = (int)(t & 511);
        const LbmCaseDev& c = cases[bcase[b]];
        float base = base_of(c.init_u[0], c.init_u[1], c.init_u[2]);
#pragma unroll
        for (int q = 0; q < Q; ++q) f[fidx(cap, q, b, s)] = feq1(q, 1.0f, c.init_u[0], c.init_u[1], c.init_u[2], base);
    }
}

struct PoolView {
    const int32_t* bx; const int32_t* by; const int32_t* bz; const uint8_t* blevel; const uint16_t* bcase;
    const float* f0; const float* f1;  // A and B
    size_t cap;
    int parity[16];
    const LbmCaseDev* cases;
    const uint8_t* mnear;  // k_mask_near bits of the current mesh, or nullptr (no case has a mask)
};

__device__ __forceinline__ const float* cur_buf(const PoolView& p, int l) { return p.parity[l] ? p.f1 : p.f0; }

// Per-brick max |curl u| (physical scale 2^level), central differences inside
// the brick, one-sided at its faces; 0 in solid sites (oracle: brick_vorticity).
__global__ void __launch_bounds__(512) k_vorticity(PoolView p, size_t n, float* __restrict__ wmax,
                                                   unsigned* __restrict__ case_max) {
    __shared__ float U[3][512];
    __shared__ float red[16];
    for (size_t b = blockIdx.x; b < n; b += gridDim.x) {
        const int s = threadIdx.x;
        const int l = p.blevel[b];
        const LbmCaseDev& c = p.cases[p.bcase[b]];
        const float* F = cur_buf(p, l);
        int64_t G[3] = {(int64_t)p.bx[b] * 8 + (s & 7), (int64_t)p.by[b] * 8 + ((s >> 3) & 7),
                        (int64_t)p.bz[b] * 8 + (s >> 6)};
        if (solid_at(c, G[0], G[1], G[2], l)) {
            U[0][s] = U[1][s] = U[2][s] = 0.0f;
        } else {
            float f[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) f[q] = F[fidx(p.cap, q, b, s)];
            float rho, jx, jy, jz;
            moments(f, rho, jx, jy, jz);
            float inv = 1.0f / rho;
            U[0][s] = jx * inv; U[1][s] = jy * inv; U[2][s] = jz * inv;
        }
        __syncthreads();
        const int co[3] = {s & 7, (s >> 3) & 7, s >> 6};
        auto dd = [&](int comp, int axis) {
            int stride = axis == 0 ? 1 : (axis == 1 ? 8 : 64);
            if (co[axis] == 0) return U[comp][s + stride] - U[comp][s];
            if (co[axis] == 7) return U[comp][s] - U[comp][s - stride];
            float t = U[comp][s + stride] - U[comp][s - stride];
            return t * 0.5f;
        };
        float wx = dd(2, 1) - dd(1, 2);
        float wy = dd(0, 2) - dd(2, 0);
        float wz = dd(1, 0) - dd(0, 1);
        float w2 = wx * wx;
        w2 = w2 + wy * wy;
        w2 = w2 + wz * wz;
        float mag = sqrtf(w2) * (float)(1 << l);
        for (int o = 16; o > 0; o >>= 1) mag = fmaxf(mag, __shfl_xor_sync(0xFFFFFFFFu, mag, o));
        if ((s & 31) == 0) red[s >> 5] = mag;
        __syncthreads();
        if (s < 32) {
            float m = s < 16 ? red[s] : 0.0f;
            for (int o = 8; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
            if (s == 0) {
                wmax[b] = m;
                atomicMax(case_max + p.bcase[b], __float_as_uint(m));  // non-negative floats order as uints
            }
        }
        __syncthreads();
    }
}

__device__ bool in_band(const LbmCaseDev& c, int32_t bx, int32_t by, int32_t bz, int l) {
    if (!c.has_sphere) return false;
    float inv = 1.0f / (float)(1 << l);
    int32_t nat[3] = {bx, by, bz};
    float dmin = 0.0f, dmax = 0.0f;
    for (int ax = 0; ax < 3; ++ax) {
        float lo = (float)(nat[ax] * 8) * inv;
        float hi = (float)(nat[ax] * 8 + 8) * inv;
        float cc = c.sc[ax];
        float cl = cc < lo ? lo : (cc > hi ? hi : cc);
        float e = cc - cl;
        dmin = dmin + e * e;
        float f1 = fabsf(cc - lo), f2 = fabsf(cc - hi);
        float fm = f1 > f2 ? f1 : f2;
        dmax = dmax + fm * fm;
    }
    float ro = c.sr + c.band;
    float ri = c.sr - c.band;
    if (ri < 0.0f) ri = 0.0f;
    return dmin <= ro * ro && dmax >= ri * ri;
}

// Brick refine/coarsen flags (oracle: compute_flags): band bricks (near the
// sphere's surface, or holding both solid and fluid mask sites in the brick and
// its halo) refine to the case's max level; otherwise refine above
// refine_frac * case max |omega|, coarsen below coarsen_frac * case max.
__global__ void k_flags(PoolView p, size_t n, const float* __restrict__ wmax, const unsigned* __restrict__ case_max,
                        int use_vorticity, int32_t* __restrict__ flags) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < n; b += stride) {
        const LbmCaseDev& c = p.cases[p.bcase[b]];
        int l = p.blevel[b];
        bool band = in_band(c, p.bx[b], p.by[b], p.bz[b], l) || (c.mask && p.mnear && (p.mnear[b] & 3) == 1);
        float wm = use_vorticity ? wmax[b] : 0.0f;
        float cm = use_vorticity ? __uint_as_float(case_max[p.bcase[b]]) : 0.0f;
        int32_t fl = 0;
        if (band) fl = l < c.max_level ? 1 : 0;
        else if (cm > 0.0f && wm > c.refine_frac * cm && l < c.max_level) fl = 1;
        else if (wm < c.coarsen_frac * cm && l > 0) fl = -1;
        flags[b] = fl;
    }
}

// Population remap after a regrid (oracle: regrid()).
__global__ void k_remap(PoolView p, size_t M, const uint32_t* __restrict__ osrc, const uint8_t* __restrict__ okind,
                        const uint32_t* __restrict__ members, float* __restrict__ out, size_t out_cap) {
    size_t total = M * 512;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        size_t j = t >> 9;
        int s = (int)(t & 511);
        int I = s & 7, J = (s >> 3) & 7, K = s >> 6;
        int kind = okind[j];
        uint32_t src = osrc[j];
        if (kind == 8) {
            const float* F = cur_buf(p, p.blevel[src]);
#pragma unroll
            for (int q = 0; q < Q; ++q) out[fidx(out_cap, q, j, s)] = F[fidx(p.cap, q, src, s)];
        } else if (kind < 8) {
            const float* F = cur_buf(p, p.blevel[src]);
            int ps = (4 * (kind & 1) + I / 2) + 8 * (4 * ((kind >> 1) & 1) + J / 2) + 64 * (4 * ((kind >> 2) & 1) + K / 2);
#pragma unroll
            for (int q = 0; q < Q; ++q) out[fidx(out_cap, q, j, s)] = F[fidx(p.cap, q, src, ps)];
        } else {
            int oc = (I >> 2) | ((J >> 2) << 1) | ((K >> 2) << 2);
            uint32_t cb = members[(size_t)src * 8 + oc];
            const float* F = cur_buf(p, p.blevel[cb]);
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                float sum = 0.0f;
                for (int tt = 0; tt < 8; ++tt) {
                    int fs = (2 * (I & 3) + (tt & 1)) + 8 * (2 * (J & 3) + ((tt >> 1) & 1)) + 64 * (2 * (K & 3) + ((tt >> 2) & 1));
                    sum = sum + F[fidx(p.cap, q, cb, fs)];
                }
                out[fidx(out_cap, q, j, s)] = sum * 0.125f;
            }
        }
    }
}

// One CTA of 128 threads per brick (persistent), thread = x-quad: per brick
// the sums of rho and j over its fluid sites.  Quads accumulate in
// double-single, warps reduce in double-single by shuffles, and each warp
// stores its (hi, lo) pairs (layout of brick_sums_store); k_chunk_sums
// combines the four warps in FP64 and weights the brick by its site volume.
__global__ void __launch_bounds__(128) k_brick_sums(PoolView p, size_t n, float* __restrict__ part) {
    const int t = threadIdx.x;
    const int x0 = (t & 1) * 4, y = (t >> 1) & 7, z = t >> 4;
    const int own = x0 + 8 * y + 64 * z;
    for (size_t b = blockIdx.x; b < n; b += gridDim.x) {
        const int l = p.blevel[b];
        const LbmCaseDev& c = p.cases[p.bcase[b]];
        const float* F = cur_buf(p, l);
        float f[Q][4];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const float4 v = __ldg((const float4*)(F + fidx(p.cap, q, b, own)));
            f[q][0] = v.x; f[q][1] = v.y; f[q][2] = v.z; f[q][3] = v.w;
        }
        uint32_t solid4 = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (solid_at(c, (int64_t)p.bx[b] * 8 + x0 + i, (int64_t)p.by[b] * 8 + y, (int64_t)p.bz[b] * 8 + z, l))
                solid4 |= 1u << i;
        brick_sums_store(f, solid4, b, part);
    }
}

// Macroscopic fields of every site: rho and u from the current populations
// (FP32, the collision's moment order); sites inside the sphere report 0.
__global__ void __launch_bounds__(128) k_macroscopic(PoolView p, size_t n, float* __restrict__ rho,
                                                     float* __restrict__ ux, float* __restrict__ uy,
                                                     float* __restrict__ uz) {
    const int t = threadIdx.x;
    const int x0 = (t & 1) * 4, y = (t >> 1) & 7, z = t >> 4;
    const int own = x0 + 8 * y + 64 * z;
    for (size_t b = blockIdx.x; b < n; b += gridDim.x) {
        const int l = p.blevel[b];
        const LbmCaseDev& c = p.cases[p.bcase[b]];
        const float* F = cur_buf(p, l);
        float4 v4[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) v4[q] = __ldg((const float4*)(F + fidx(p.cap, q, b, own)));
        float o[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float f[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) f[q] = i == 0 ? v4[q].x : (i == 1 ? v4[q].y : (i == 2 ? v4[q].z : v4[q].w));
            float r, jx, jy, jz;
            moments(f, r, jx, jy, jz);
            const bool solid =
                solid_at(c, (int64_t)p.bx[b] * 8 + x0 + i, (int64_t)p.by[b] * 8 + y, (int64_t)p.bz[b] * 8 + z, l);
            const float inv = 1.0f / r;
            o[0][i] = solid ? 0.0f : r;
            o[1][i] = solid ? 0.0f : jx * inv;
            o[2][i] = solid ? 0.0f : jy * inv;
            o[3][i] = solid ? 0.0f : jz * inv;
        }
        const size_t at = b * 512 + own;
        *(float4*)(rho + at) = make_float4(o[0][0], o[0][1], o[0][2], o[0][3]);
        *(float4*)(ux + at) = make_float4(o[1][0], o[1][1], o[1][2], o[1][3]);
        *(float4*)(uy + at) = make_float4(o[2][0], o[2][1], o[2][2], o[2][3]);
        *(float4*)(uz + at) = make_float4(o[3][0], o[3][1], o[3][2], o[3][3]);
    }
}

// Per chunk of up to 1024 consecutive bricks of one case (one CTA each): the
// bricks' partials summed in a fixed order -- thread t takes bricks t, t+256,
// ..., then a fixed tree across threads.  Chunks start at each case's first
// brick, so a case's sums do not depend on the other cases of the pool.
constexpr uint32_t kChunkBricks = 1024;

__global__ void __launch_bounds__(256) k_chunk_sums(const float* __restrict__ part, const uint8_t* __restrict__ level,
                                                    const uint2* __restrict__ chunks, uint32_t nchunks,
                                                    double* __restrict__ chunk_part) {
    __shared__ double red[4][256];
    for (uint32_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const uint2 r = chunks[c];
        double acc[4] = {0, 0, 0, 0};
        for (uint32_t b = r.x + threadIdx.x; b < r.y; b += 256) {
            // the brick's four warp totals in order, times its site volume 8^-level (exact)
            const double vol = __longlong_as_double((long long)(1023 - 3 * (int)level[b]) << 52);
            const float* w = part + (size_t)b * 32;
            for (int k = 0; k < 4; ++k) {
                double s4 = (double)w[2 * k] + (double)w[2 * k + 1];
                for (int v = 1; v < 4; ++v) s4 = s4 + ((double)w[v * 8 + 2 * k] + (double)w[v * 8 + 2 * k + 1]);
                acc[k] += s4 * vol;
            }
        }
        for (int k = 0; k < 4; ++k) red[k][threadIdx.x] = acc[k];
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (threadIdx.x < o)
                for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x < 4) chunk_part[(size_t)c * 4 + threadIdx.x] = red[threadIdx.x][0];
        __syncthreads();
    }
}

// Per case (thread = case and component): its chunks' sums in chunk order.
__global__ void k_case_sums(const double* __restrict__ chunk_part, const uint32_t* __restrict__ case_chunk,
                            int ncases, double* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncases * 4) return;
    const int cs = t >> 2, k = t & 3;
    double s = 0.0;
    for (uint32_t c = case_chunk[cs]; c < case_chunk[cs + 1]; ++c) s += chunk_part[(size_t)c * 4 + k];
    out[t] = s;
}

// exp(x) for x <= 0 from the mathematics: x = n ln2 + r with |r| <= ln2/2
// (Cody & Waite 1980 two-constant reduction; the split ln2 = 0.693145752 +
// 1.42860677e-6 is the one published with fdlibm's single-precision expf,
// e_expf.c, whose high part has a short mantissa so n * ln2_hi is exact),
// e^r by its Taylor series to r^7, then an exact scaling by 2^n.  Written
// operation by operation (this unit has no FMA contraction) so the CPU
// restatement gives the same bits.
__device__ __forceinline__ float fl_exp_neg(float x) {
    if (x < -87.0f) return 0.0f;
    float t = x * 1.44269504f;
    t = t + 0.5f;
    float n = floorf(t);
    float r = x - n * 0.693145752f;
    r = r - n * 1.42860677e-06f;
    float p = 1.0f / 5040.0f;
    p = p * r; p = p + 1.0f / 720.0f;
    p = p * r; p = p + 1.0f / 120.0f;
    p = p * r; p = p + 1.0f / 24.0f;
    p = p * r; p = p + 1.0f / 6.0f;
    p = p * r; p = p + 0.5f;
    p = p * r; p = p + 1.0f;
    p = p * r; p = p + 1.0f;
    return ldexpf(p, (int)n);
}

// Synthetic refine/coarsen flags: the sum of Gaussian blobs at each cell's
// centre (unit cube, native coords at `level`, anchor level A), refine above
// `hi`, coarsen below `lo` (the regrid microbenchmark's flag source).
__global__ void k_blob_flags(fl_mesh_dev m, const float* __restrict__ blobs, int nblobs, int anchor_level, float lo,
                             float hi, int max_level, int32_t* __restrict__ flags) {
    extern __shared__ float sb[];
    for (int i = threadIdx.x; i < nblobs * 5; i += blockDim.x) sb[i] = blobs[i];
    __syncthreads();
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.n; i += stride) {
        int l = m.level[i];
        float inv = 1.0f / (float)(1 << l);
        float px = ((float)m.x[i] + 0.5f) * inv, py = ((float)m.y[i] + 0.5f) * inv, pz = ((float)m.z[i] + 0.5f) * inv;
        float v = 0.0f;
        for (int k = 0; k < nblobs; ++k) {
            const float* B = sb + 5 * k;  // cx, cy, cz, 1/(2 sigma^2), amplitude
            float dx = px - B[0], dy = py - B[1], dz = pz - B[2];
            float d2 = dx * dx;
            d2 = d2 + dy * dy;
            d2 = d2 + dz * dz;
            float e = fl_exp_neg(-(d2 * B[3]));
            v = v + B[4] * e;
        }
        int32_t f = 0;
        if (v > hi && l < max_level) f = 1;
        else if (v < lo) f = -1;
        flags[i] = f;
    }
}

}  // namespace

extern "C" int fl_flags_from_blobs(fl_ctx* ctx, fl_mesh* mesh, const float* blobs_host, int nblobs, float lo, float hi,
                                   int max_level) {
    if (!ctx || !mesh || (nblobs && !blobs_host) || nblobs < 0 || nblobs > 1024) return FL_E_INVALID_ARG;
    if (mesh->num_cells == 0) return FL_OK;
    int rc = fl_scratch_reserve(ctx, (size_t)nblobs * 20 + 256);
    if (rc) return rc;
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->scratch, blobs_host, (size_t)nblobs * 20, cudaMemcpyHostToDevice, ctx->stream),
                "blobs");
    fl_mesh_dev md{mesh->x, mesh->y, mesh->z, mesh->level, mesh->state, mesh->flags, mesh->material, mesh->case_id,
                   mesh->num_cells};
    k_blob_flags<<<fl_blocks(mesh->num_cells, 256, ctx->num_sms * 8), 256, (size_t)nblobs * 20, ctx->stream>>>(
        md, (const float*)ctx->scratch, nblobs, 0, lo, hi, max_level, mesh->flags);
    FL_CHECK_LAUNCH(ctx, "k_blob_flags");
    return FL_OK;
}

namespace {

// Keep only the flags of bricks whose case is due for a regrid.
__global__ void k_mask_flags(size_t n, const uint16_t* __restrict__ bcase, const uint8_t* __restrict__ due,
                             int32_t* __restrict__ flags) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < n; b += stride)
        if (!due[bcase[b]]) flags[b] = 0;
}

// Solid-mask bits of the cells (x, y, z) inside the nx * ny * nz grid; cells
// outside it are ignored.
__global__ void k_mask_cells(const int32_t* __restrict__ x, const int32_t* __restrict__ y,
                             const int32_t* __restrict__ z, size_t n, int64_t nx, int64_t ny, int64_t nz,
                             uint32_t* __restrict__ words) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int64_t a = x[i], b = y[i], c = z[i];
        if (a < 0 || b < 0 || c < 0 || a >= nx || b >= ny || c >= nz) continue;
        const uint64_t bit = ((uint64_t)c * (uint64_t)ny + (uint64_t)b) * (uint64_t)nx + (uint64_t)a;
        atomicOr(words + (bit >> 5), 1u << (bit & 31));
    }
}

__global__ void k_keep_bricks(size_t n, const uint16_t* __restrict__ bcase, const uint8_t* __restrict__ active,
                              uint32_t* __restrict__ keep) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < n; b += stride) keep[b] = active[bcase[b]];
}

// Order-preserving compaction of the brick columns; osrc/okind feed k_remap as survivors.
__global__ void k_compact_bricks(fl_mesh_dev m, const uint32_t* __restrict__ keep, const uint32_t* __restrict__ off,
                                 fl_mesh_out o, uint32_t* __restrict__ osrc, uint8_t* __restrict__ okind) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.n; i += stride) {
        if (!keep[i]) continue;
        uint32_t j = off[i];
        o.x[j] = m.x[i]; o.y[j] = m.y[i]; o.z[j] = m.z[i];
        o.level[j] = m.level[i]; o.state[j] = m.state[i]; o.flags[j] = 0; o.material[j] = m.material[i];
        o.case_id[j] = m.case_id[i];
        osrc[j] = (uint32_t)i;
        okind[j] = 8;
    }
}

}  // namespace

// ------------------------------------------------------------------ pool
constexpr int kMaxCases = 4096;  // case ids live in 12 key bits

struct fl_pool {
    // Set while a call that replaces the pool's bricks or tables is past its
    // point of no return; left set when such a call fails there, after which
    // every entry point refuses the pool (FL_POOL_USABLE) instead of launching
    // on tables that no longer match its bricks.  Destroying it stays allowed.
    bool unusable = false;
    std::vector<fl_lbm_case> cases;   // one entry per slot (case id)
    std::vector<uint8_t> active;      // slot in use
    uint8_t* d_mask = nullptr;        // per-slot byte mask on the device (regrid / removal)
    std::vector<LbmCaseDev> hcases;
    LbmCaseDev* d_cases = nullptr;
    fl_domain_dev::Case* d_dom = nullptr;
    fl_mesh mesh{};
    size_t cap = 0;
    uint32_t* nbr = nullptr;
    float* f[3] = {nullptr, nullptr, nullptr};
    int parity[16] = {0};
    int maxL = 0;
    uint32_t* list = nullptr;
    std::vector<uint32_t> lvl_off;  // maxL + 2 entries
    // per brick class (0 interior, 1 general, 2 all-solid) and level: offset and count into `list`
    std::vector<uint32_t> cls_off[3], cls_cnt[3];
    uint64_t fluid_cls[3][16] = {};
    uint32_t* nb27 = nullptr;
    uint8_t* bclass = nullptr;
    uint8_t* mnear = nullptr;       // k_mask_near bits per brick (valid while any_mask)
    std::vector<uint32_t*> dmask;   // per slot: its solid-mask words on the device, or nullptr
    bool any_mask = false;
    uint32_t* slow_cnt = nullptr;   // per list position: descriptors of the brick
    uint32_t* slow_off = nullptr;   // exclusive prefix of slow_cnt, n + 1 entries
    uint32_t* smask = nullptr;      // [cap][16] own-site solid bits of general bricks
    uint4* qmask = nullptr;         // [cap][128] per x-quad descriptor bits and offsets
    uint32_t* hsolid = nullptr;     // [cap][32] solid bits of general bricks and their one-site halo
    uint64_t* desc = nullptr;       // stencil descriptors
    float* pv = nullptr;            // their values at the current sub-step
    size_t desc_cap = 0;
    std::vector<uint32_t> lvl_desc;  // per level: first descriptor of its general bricks; [maxL + 1] = end
    uint64_t num_desc = 0;
    std::vector<uint32_t> case_begin;
    uint32_t* d_case_begin = nullptr;
    TopoCounters* d_topo = nullptr;       // k_topo_bins / k_topo_sums results
    uint2* d_chunks = nullptr;            // brick ranges of <= 1024 bricks, each within one case
    uint32_t* d_case_chunk = nullptr;     // per case: first chunk; [ncases] = end
    double* chunk_part = nullptr;
    uint32_t nchunks = 0;
    float* wmax = nullptr;
    unsigned* case_max = nullptr;
    float* part = nullptr;            // per brick and warp: (hi, lo) of the four conservation sums
    double* cons = nullptr;
    uint32_t* fluid = nullptr;
    uint64_t lups = 0;
    uint64_t fluid_per_level[16] = {0};
    int graphs = 1;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};  // one level-0 step, per level-0 parity
    uint64_t graph_kernels[2] = {0, 0};             // kernel nodes of each
    bool graph_ok[2] = {false, false};              // graph[k] matches the current pool
    // the same with every level's all-solid bricks written in every sub-step, replayed
    // while some level still owes such writes (after its populations were replaced)
    cudaGraphExec_t graph_solid[2] = {nullptr, nullptr};
    uint64_t graph_solid_kernels[2] = {0, 0};
    bool graph_solid_ok[2] = {false, false};
    uint64_t version = 0;                           // bumped whenever the emitted launches change
    void* adapt_scratch = nullptr;
    size_t adapt_scratch_bytes = 0;
    int grid_mult = 4;
    // the bricks are the output of an adapt whose FULL26 balance converged (no two
    // touching bricks more than one level apart): the next regrid's adapt may say so
    bool mesh_balanced = false;
    // fl_pool_set_step_sums: each level's last sub-step of a level-0 step writes its
    // bricks' conservation sums into `part` (never once the populations were exported
    // as a writable field); sums_fresh: `part` holds the sums of the current state
    bool sums_enabled = false;
    bool field_exported = false;
    bool sums_fresh = false;
    // 0: collide kernels load straight into registers; 1: the brick's own
    // population planes bulk-copied into shared memory one brick ahead
    // (k_collide_staged); 2: as 1, with the general bricks' quad masks and
    // descriptor values staged too
    int staging = 0;
    // All-solid bricks only ever hold the rest equilibrium: once both
    // population buffers of a level hold it (two sub-steps after any change of
    // the bricks or populations), rewriting it changes nothing and its launch
    // is left out.  solid_due[l] counts the level's sub-steps that must still
    // write them; emit_solid forces the launch (a caller's stream capture,
    // which may be replayed at any time).
    int solid_due[kMaxPoolLevels] = {};
    bool emit_solid = false;
    // dependency-graph launch order: per level a stream for the general,
    // interface and all-solid bricks and one for the interior bricks
    int streams = 2;
    cudaStream_t sg[kMaxPoolLevels] = {}, sf[kMaxPoolLevels] = {};
    cudaEvent_t evg[kMaxPoolLevels][2] = {}, evf[kMaxPoolLevels][2] = {}, ev_root = nullptr;
};

namespace {

void to_dev_case(const fl_lbm_case& c, LbmCaseDev& d) {
    std::memset(&d, 0, sizeof(d));
    for (int a = 0; a < 3; ++a) {
        d.ext[a] = c.ext[a];
        d.periodic[a] = c.bc[2 * a] == 0;
        d.wall_u[a] = c.wall_u[a];
        d.inlet_u[a] = c.inlet_u[a];
        d.init_u[a] = c.init_u[a];
        d.sc[a] = c.sphere_c[a];
    }
    for (int k = 0; k < 6; ++k) d.bc[k] = c.bc[k];
    for (int l = 0; l < 20; ++l) {
        float t = c.tau0 - 0.5f;
        t = (float)(1 << l) * t;
        t = t + 0.5f;
        d.omega[l] = 1.0f / t;
    }
    d.max_level = c.max_level;
    d.has_sphere = c.has_sphere;
    d.sr = c.sphere_r;
    d.refine_frac = c.refine_frac;
    d.coarsen_frac = c.coarsen_frac;
    d.band = c.band;
}

fl_domain_dev pool_domain(fl_pool* P) {
    fl_domain_dev d;
    d.depth = 17;
    d.anchor_level = 13;
    d.max_level = 13;
    d.c = P->d_dom;
    return d;
}

PoolView view(fl_pool* P) {
    PoolView v;
    v.bx = P->mesh.x; v.by = P->mesh.y; v.bz = P->mesh.z; v.blevel = P->mesh.level; v.bcase = P->mesh.case_id;
    v.f0 = P->f[0]; v.f1 = P->f[1];
    v.cap = P->cap;
    for (int l = 0; l < 16; ++l) v.parity[l] = P->parity[l];
    v.cases = P->d_cases;
    v.mnear = P->any_mask ? P->mnear : nullptr;
    return v;
}

int alloc_brick_arrays(fl_ctx* ctx, fl_pool* P, size_t cap) {
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->nbr, cap * 26 * 4 * 4, ctx->stream), "pool nbr");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->list, cap * 8, ctx->stream), "pool list");  // list + general positions
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->wmax, cap * 4, ctx->stream), "pool wmax");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->part, cap * 128, ctx->stream), "pool partials");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->fluid, cap * 4, ctx->stream), "pool fluid");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->nb27, cap * 28 * 4, ctx->stream), "pool nb27");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->bclass, cap, ctx->stream), "pool classes");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->mnear, cap, ctx->stream), "pool mask bits");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->slow_cnt, cap * 4, ctx->stream), "pool descriptor counts");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->slow_off, (cap + 1) * 4, ctx->stream), "pool descriptor offsets");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->smask, cap * 64, ctx->stream), "pool solid masks");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->qmask, cap * 128 * sizeof(uint4), ctx->stream), "pool quad masks");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->hsolid, cap * 32 * 4, ctx->stream), "pool halo solid bits");
    const size_t max_chunks = cap / kChunkBricks + kMaxCases + 1;  // one partial chunk per case at most
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->d_chunks, max_chunks * sizeof(uint2), ctx->stream), "pool chunks");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->chunk_part, max_chunks * 32, ctx->stream), "pool chunk sums");
    return FL_OK;
}

// The pool's 15 per-brick arrays as one set of pointers, so that a grown set can
// be allocated beside the current one and swapped in only when complete.
struct BrickArrays {
    void* p[15];
};

void brick_slots(fl_pool* P, void** s[15]) {
    s[0] = (void**)&P->nbr; s[1] = (void**)&P->list; s[2] = (void**)&P->wmax; s[3] = (void**)&P->part;
    s[4] = (void**)&P->fluid; s[5] = (void**)&P->nb27; s[6] = (void**)&P->bclass; s[7] = (void**)&P->slow_cnt;
    s[8] = (void**)&P->slow_off; s[9] = (void**)&P->smask; s[10] = (void**)&P->qmask; s[11] = (void**)&P->d_chunks;
    s[12] = (void**)&P->chunk_part; s[13] = (void**)&P->mnear; s[14] = (void**)&P->hsolid;
}

BrickArrays get_brick_arrays(fl_pool* P) {
    void** s[15];
    brick_slots(P, s);
    BrickArrays b;
    for (int k = 0; k < 15; ++k) b.p[k] = *s[k];
    return b;
}

void put_brick_arrays(fl_pool* P, const BrickArrays& b) {
    void** s[15];
    brick_slots(P, s);
    for (int k = 0; k < 15; ++k) *s[k] = b.p[k];
}

void release_brick_arrays(fl_ctx* ctx, const BrickArrays& b) {
    for (void* p : b.p)
        if (p) cudaFreeAsync(p, ctx->stream);
}

void free_brick_arrays(fl_ctx* ctx, fl_pool* P) {
    release_brick_arrays(ctx, get_brick_arrays(P));
    put_brick_arrays(P, BrickArrays{});
}

// A new set of per-brick arrays for cap bricks in *fresh, leaving the pool's own
// set in place; nothing stays allocated on failure.
int alloc_brick_arrays_beside(fl_ctx* ctx, fl_pool* P, size_t cap, BrickArrays* fresh) {
    const BrickArrays cur = get_brick_arrays(P);
    put_brick_arrays(P, BrickArrays{});
    int rc = alloc_brick_arrays(ctx, P, cap);
    *fresh = get_brick_arrays(P);
    put_brick_arrays(P, cur);
    if (rc) {
        release_brick_arrays(ctx, *fresh);
        *fresh = BrickArrays{};
    }
    return rc;
}

// The captured steps no longer match the pool: mark them stale.  The next
// capture updates the instantiated graph in place when its shape is unchanged
// (cudaGraphExecUpdate) instead of instantiating anew.  Every change of the
// bricks or populations passes here, so it also makes each level write its
// all-solid bricks for its next two sub-steps (both buffers).
void populations_replaced(fl_pool* P) {
    ++P->version;
    P->sums_fresh = false;
    for (int l = 0; l < kMaxPoolLevels; ++l) P->solid_due[l] = 2;
}

void drop_graph(fl_pool* P) {
    populations_replaced(P);
    P->graph_ok[0] = P->graph_ok[1] = false;
    P->graph_solid_ok[0] = P->graph_solid_ok[1] = false;
}

void free_graphs(fl_pool* P) {
    for (int k = 0; k < 2; ++k) {
        if (P->graph[k]) cudaGraphExecDestroy(P->graph[k]);
        P->graph[k] = nullptr;
        P->graph_ok[k] = false;
        if (P->graph_solid[k]) cudaGraphExecDestroy(P->graph_solid[k]);
        P->graph_solid[k] = nullptr;
        P->graph_solid_ok[k] = false;
    }
}

// Neighbour table, per-level lists, case ranges and fluid count for the current mesh.
int pool_topology_build(fl_ctx* ctx, fl_pool* P);

// Rebuild the tables of the pool's current bricks; the pool is unusable until
// this succeeds.
int pool_topology(fl_ctx* ctx, fl_pool* P) {
    P->unusable = true;
    int rc = pool_topology_build(ctx, P);
    if (rc == FL_OK) {
        // all-solid bricks hold no fluid: their sums stay 0 (the fused sums never write them)
        P->sums_fresh = false;
        if (cudaMemsetAsync(P->part, 0, P->cap * 128, ctx->stream) != cudaSuccess)
            rc = fl_set_error(ctx, FL_E_CUDA, "conservation partials clear");
    }
    if (rc == FL_OK) P->unusable = false;
    return rc;
}

int pool_topology_build(fl_ctx* ctx, fl_pool* P) {
    size_t n = P->mesh.num_cells;
    if (P->cap >= (1u << 23))  // descriptors address elements as brick * 512 + site in 32 bits
        return fl_set_error(ctx, FL_E_CAPACITY, "a pool holds fewer than 2^23 bricks");
    const size_t ncases = P->cases.size();
    // scratch: neighbour marks + the point locator, later the list sort keys,
    // the sort's and the scan's own scratch
    const size_t lists_bytes = fl_align256(n * 8) + fl_sort_scratch_bytes(n, 1) + fl_scan_scratch_bytes(n);
    int rc = fl_scratch_reserve(ctx, std::max(fl_align256(n * 4) + fl_locator_scratch_bytes(n),
                                              lists_bytes + fl_align256(n * 4)));
    if (rc) return rc;
    fl_domain_dev dom = pool_domain(P);
    fl_mesh_dev md{P->mesh.x, P->mesh.y, P->mesh.z, P->mesh.level, P->mesh.state, P->mesh.flags, P->mesh.material,
                   P->mesh.case_id, n};
    fl_locator L;
    uint32_t* marks = (uint32_t*)ctx->scratch;
    // a pool's bricks are in key order whenever its topology is rebuilt (every
    // regrid emits them so; removal compacts in order)
    rc = fl_locator_build(ctx, md, dom, (char*)ctx->scratch + fl_align256(n * 4), &L, P->maxL, true);
    if (rc) return rc;
    rc = fl_neighbours_sorted(ctx, md, dom, L, 4, P->nbr, marks);
    if (rc) return rc;
    const uint8_t* mnear = P->any_mask ? P->mnear : nullptr;
    if (mnear) {
        k_mask_near<<<fl_blocks(n * 32, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
            n, P->mesh.level, P->mesh.x, P->mesh.y, P->mesh.z, P->mesh.case_id, P->d_cases, P->mnear);
        FL_CHECK_LAUNCH(ctx, "k_mask_near");
    }
    // classes and descriptor tables (the locator's scratch is free again: the
    // per-brick descriptor counts go behind the list-building scratch)
    uint64_t* bin_keys = (uint64_t*)ctx->scratch;
    void* sort_scratch = (char*)ctx->scratch + fl_align256(n * 8);
    void* scan_scratch = (char*)sort_scratch + fl_sort_scratch_bytes(n, 1);
    uint32_t* cnt_b = (uint32_t*)((char*)ctx->scratch + lists_bytes);
    k_brick_table<<<fl_blocks(n * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
        n, P->nbr, P->mesh.level, P->mesh.x, P->mesh.y, P->mesh.z, P->mesh.case_id, P->d_cases, mnear, P->nb27,
        P->bclass, cnt_b, P->smask, P->qmask, P->hsolid, P->fluid);
    FL_CHECK_LAUNCH(ctx, "k_brick_table");
    // level lists: the bricks stably sorted by bin = level * 3 + class (interior,
    // general, all-solid), so each level's classes follow one another in brick order
    TopoCounters* tc = P->d_topo;
    FL_TRY_CUDA(ctx, cudaMemsetAsync(tc, 0, sizeof(TopoCounters), ctx->stream), "topology counters");
    k_topo_bins<<<fl_blocks(n, 256, ctx->num_sms * 4), 256, 0, ctx->stream>>>(
        n, P->mesh.level, P->bclass, P->mesh.case_id, P->maxL, (uint32_t)ncases, bin_keys, P->list, tc,
        P->d_case_begin);
    FL_CHECK_LAUNCH(ctx, "k_topo_bins");
    if (n == 0) FL_TRY_CUDA(ctx, cudaMemsetAsync(P->d_case_begin, 0, (ncases + 1) * 4, ctx->stream), "case ranges");
    int bits = 1;
    while ((1 << bits) < 3 * (P->maxL + 1)) ++bits;
    rc = fl_sort_pairs_with(ctx, bin_keys, P->list, n, 0, bits, sort_scratch);
    if (rc) return rc;
    TopoCounters h{};
    P->case_begin.assign(ncases + 1, 0);
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(&h, tc, sizeof(TopoCounters), cudaMemcpyDeviceToHost, ctx->stream), "counts");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->case_begin.data(), P->d_case_begin, (ncases + 1) * 4, cudaMemcpyDeviceToHost,
                                     ctx->stream), "case ranges");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "topology sync");
    if (h.err & 1u) return fl_set_error(ctx, FL_E_INVALID_ARG, "brick level above the pool maximum");
    if (h.err & 6u) return fl_set_error(ctx, FL_E_INVALID_ARG, "pool bricks not in case order");
    P->lvl_off.assign(P->maxL + 2, 0);
    for (int k = 0; k < 3; ++k) {
        P->cls_off[k].assign(P->maxL + 1, 0);
        P->cls_cnt[k].assign(P->maxL + 1, 0);
    }
    GenTable gt{};
    gt.levels = P->maxL + 1;
    uint32_t run = 0, ng = 0;
    for (int l = 0; l <= P->maxL; ++l) {
        P->lvl_off[l] = run;
        for (int k = 0; k < 3; ++k) {
            P->cls_off[k][l] = run;
            P->cls_cnt[k][l] = h.count[l * 3 + k];
            run += h.count[l * 3 + k];
        }
        gt.base[l] = ng;
        gt.start[l] = P->cls_off[1][l];
        ng += P->cls_cnt[1][l];
    }
    gt.base[P->maxL + 1] = ng;
    P->lvl_off[P->maxL + 1] = run;
    if (run != n) return fl_set_error(ctx, FL_E_INVALID_ARG, "brick classes do not cover the pool");
    uint32_t* d_gen = P->list + n;  // general bricks' list positions
    FL_TRY_CUDA(ctx, cudaMemsetAsync(P->slow_cnt, 0, n * 4, ctx->stream), "descriptor counts");
    if (ng) {
        k_gen_positions<<<fl_blocks(ng, 256, ctx->num_sms * 4), 256, 0, ctx->stream>>>(ng, gt, P->list, cnt_b, d_gen,
                                                                                     P->slow_cnt);
        FL_CHECK_LAUNCH(ctx, "k_gen_positions");
    }
    {  // conservation-sum chunks
        std::vector<uint2> chunks;
        std::vector<uint32_t> case_chunk(ncases + 1, 0);
        for (size_t c = 0; c < ncases; ++c) {
            case_chunk[c] = (uint32_t)chunks.size();
            for (uint32_t b = P->case_begin[c]; b < P->case_begin[c + 1]; b += kChunkBricks)
                chunks.push_back(make_uint2(b, std::min(b + kChunkBricks, P->case_begin[c + 1])));
        }
        case_chunk[ncases] = (uint32_t)chunks.size();
        P->nchunks = (uint32_t)chunks.size();
        if (P->nchunks)
            FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->d_chunks, chunks.data(), chunks.size() * sizeof(uint2),
                                             cudaMemcpyHostToDevice, ctx->stream), "chunks");
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->d_case_chunk, case_chunk.data(), case_chunk.size() * 4,
                                         cudaMemcpyHostToDevice, ctx->stream), "case chunks");
    }
    // stencil descriptors of the general class: offsets by a device scan over
    // the list positions, words written by k_slow_emit
    rc = fl_scan_u32_with(ctx, P->slow_cnt, P->slow_off, n, P->slow_off + n, scan_scratch);
    if (rc) return rc;
    k_topo_sums<<<fl_blocks(n, 256, ctx->num_sms * 4), 256, 0, ctx->stream>>>(
        n, P->mesh.level, P->bclass, P->fluid, P->slow_cnt, P->slow_off, gt, P->maxL, tc);
    FL_CHECK_LAUNCH(ctx, "k_topo_sums");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(&h, tc, sizeof(TopoCounters), cudaMemcpyDeviceToHost, ctx->stream), "sums");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "topology sync");
    if (h.desc64 >= (1ull << 32)) return fl_set_error(ctx, FL_E_CAPACITY, "more than 2^32 stencil descriptors");
    P->num_desc = h.desc64;
    P->lvl_desc.assign(h.lvl_desc, h.lvl_desc + P->maxL + 2);
    if (P->num_desc + 4 > P->desc_cap) {  // k_collide_staged reads up to 3 values past the last
        // no pointer is left naming freed memory if an allocation fails
        if (P->desc) cudaFreeAsync(P->desc, ctx->stream);
        if (P->pv) cudaFreeAsync(P->pv, ctx->stream);
        P->desc = nullptr;
        P->pv = nullptr;
        P->desc_cap = 0;
        const size_t want = P->num_desc + P->num_desc / 4 + 1024;
        FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->desc, want * 8, ctx->stream), "stencil descriptors");
        FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&P->pv, want * 4, ctx->stream), "descriptor values");
        P->desc_cap = want;
    }
    if (ng) {
        const unsigned egrid = (unsigned)std::min<size_t>(ng, (size_t)ctx->num_sms * 4);
        k_slow_emit<<<egrid, 256, 0, ctx->stream>>>(ng, d_gen, P->list, P->nbr, P->mesh.level, P->mesh.x, P->mesh.y,
                                                    P->mesh.z, P->mesh.case_id, P->d_cases, mnear, P->hsolid, P->qmask,
                                                    P->slow_cnt, P->slow_off, P->desc, ctx->dev_status);
        FL_CHECK_LAUNCH(ctx, "k_slow_emit");
    }
    P->lups = 0;
    for (int l = 0; l < 16; ++l) P->fluid_per_level[l] = P->fluid_cls[0][l] = P->fluid_cls[1][l] = P->fluid_cls[2][l] = 0;
    for (int l = 0; l <= P->maxL; ++l)
        for (int k = 0; k < 3; ++k) {
            P->fluid_cls[k][l] = h.fluid[l * 3 + k];
            P->fluid_per_level[l] += h.fluid[l * 3 + k];
        }
    for (int l = 0; l <= P->maxL; ++l) P->lups += P->fluid_per_level[l] << l;
    drop_graph(P);
    return fl_collect_device_status(ctx, "pool topology");
}

int pool_init_populations(fl_ctx* ctx, fl_pool* P) {
    size_t n = P->mesh.num_cells;
    k_init_populations<<<fl_blocks(n * 512, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
        P->f[0], P->cap, n, P->mesh.case_id, P->d_cases);
    FL_CHECK_LAUNCH(ctx, "k_init_populations");
    for (int l = 0; l < 16; ++l) P->parity[l] = 0;
    drop_graph(P);
    return FL_OK;
}

// use_vorticity: 0 band only, 1 band + vorticity, -1 all flags 0 (the regrid then only sorts)
int pool_flags(fl_ctx* ctx, fl_pool* P, int use_vorticity) {
    size_t n = P->mesh.num_cells;
    if (use_vorticity < 0) {
        FL_TRY_CUDA(ctx, cudaMemsetAsync(P->mesh.flags, 0, n * 4, ctx->stream), "flags clear");
        return FL_OK;
    }
    PoolView v = view(P);
    FL_TRY_CUDA(ctx, cudaMemsetAsync(P->case_max, 0, P->cases.size() * 4, ctx->stream), "case max");
    if (use_vorticity) {
        k_vorticity<<<fl_blocks(n, 1, ctx->num_sms * 8), 512, 0, ctx->stream>>>(v, n, P->wmax, P->case_max);
        FL_CHECK_LAUNCH(ctx, "k_vorticity");
    }
    k_flags<<<fl_blocks(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(v, n, P->wmax, P->case_max, use_vorticity,
                                                                          P->mesh.flags);
    FL_CHECK_LAUNCH(ctx, "k_flags");
    return FL_OK;
}

// One regrid: flags, adapt (FULL26), population remap into the spare buffer.
// host_flags (one int32 per brick, pool order) replace the computed flags.
int pool_regrid(fl_ctx* ctx, fl_pool* P, int use_vorticity, fl_adapt_stats* st, const uint8_t* due = nullptr,
                const int32_t* host_flags = nullptr) {
    size_t n = P->mesh.num_cells;
    int rc = FL_OK;
    if (host_flags)
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.flags, host_flags, n * 4, cudaMemcpyHostToDevice, ctx->stream),
                    "flags");
    else
        rc = pool_flags(ctx, P, use_vorticity);
    if (rc) return rc;
    if (due) {  // cases not due keep flag 0 and come out of the regrid unchanged
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->d_mask, due, P->cases.size(), cudaMemcpyHostToDevice, ctx->stream), "due");
        k_mask_flags<<<fl_blocks(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(n, P->mesh.case_id, P->d_mask,
                                                                                  P->mesh.flags);
        FL_CHECK_LAUNCH(ctx, "k_mask_flags");
    }
    fl_adapt_config cfg{};
    cfg.max_refinement_level = (uint8_t)P->maxL;
    cfg.min_refinement_level = 0;
    cfg.max_balance_iterations = 10;
    cfg.enforce_2_1_balance = 1;
    cfg.balance_mode = 1;
    cfg.averaging_rule = 0;
    cfg.input_balanced = P->mesh_balanced ? 1 : 0;
    P->mesh_balanced = false;  // until this regrid has succeeded
    fl_domain_dev dom = pool_domain(P);
    size_t sb = fl_adapt_scratch_bytes(n, fl_table_capacity(n));
    if (sb > P->adapt_scratch_bytes) {
        void* ns = nullptr;
        const size_t want = sb + sb / 4;
        FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, &ns, want, ctx->stream), "adapt scratch");
        if (P->adapt_scratch) cudaFreeAsync(P->adapt_scratch, ctx->stream);
        P->adapt_scratch = ns;
        P->adapt_scratch_bytes = want;
    }
    size_t M = 0;
    fl_adapt_stats s{};
    rc = fl_adapt_prepare(ctx, &P->mesh, &cfg, dom, true, P->adapt_scratch, &M, &s, P->maxL);
    if (rc) return rc;
    // Nothing splits and nothing merges: the bricks, their key order, the tables
    // and the populations all stay as they are (AdaptationEngine.cpp:72-78 returns
    // early the same way); only the flags are reset.  The sort-only regrid after
    // cases were appended (use_vorticity < 0) must still reorder.
    if (use_vorticity >= 0 && s.num_split == 0 && s.num_groups == 0) {
        FL_TRY_CUDA(ctx, cudaMemsetAsync(P->mesh.flags, 0, n * 4, ctx->stream), "flags reset");
        P->mesh_balanced = s.balance.converged != 0;
        if (st) *st = s;
        return FL_OK;
    }
    size_t new_cap = P->cap;
    if (M > P->cap) new_cap = std::max((size_t)(M * 1.5), M + 64);
    const bool grew = new_cap != P->cap;
    // Everything the new mesh needs is allocated before the pool is touched: a
    // failure up to the remap returns with the pool as it was.
    fl_mesh out{};
    uint32_t *osrc = nullptr, *members = nullptr;
    uint8_t* okind = nullptr;
    float* nf[3] = {nullptr, nullptr, nullptr};
    BrickArrays fresh{};
    auto undo = [&](int code) {
        if (out.x) fl_mesh_free(ctx, &out);
        void* tmp[6] = {osrc, okind, members, nf[0], nf[1], nf[2]};
        for (void* p : tmp)
            if (p) cudaFreeAsync(p, ctx->stream);
        release_brick_arrays(ctx, fresh);
        return code;
    };
    rc = fl_mesh_alloc(ctx, new_cap, 1, &out);
    if (rc) return rc;
    cudaError_t e = fl_dev_malloc_async(ctx, (void**)&osrc, (M + 1) * 4, ctx->stream);
    if (e == cudaSuccess) e = fl_dev_malloc_async(ctx, (void**)&okind, M + 1, ctx->stream);
    if (e == cudaSuccess) e = fl_dev_malloc_async(ctx, (void**)&members, (size_t)s.num_groups * 32 + 32, ctx->stream);
    for (int k = 0; grew && k < 3 && e == cudaSuccess; ++k)
        e = fl_dev_malloc_async(ctx, (void**)&nf[k], new_cap * 512 * Q * 4, ctx->stream);
    if (e != cudaSuccess) return undo(fl_check_cuda(ctx, e, "regrid buffers"));
    if (grew) {
        rc = alloc_brick_arrays_beside(ctx, P, new_cap, &fresh);
        if (rc) return undo(rc);
    }
    rc = fl_adapt_finish(ctx, &P->mesh, &cfg, dom, P->adapt_scratch, M, nullptr, 0, &out, nullptr, osrc, okind, members,
                         s.num_groups);
    if (rc) return undo(rc);
    float* target = grew ? nf[0] : P->f[2];
    k_remap<<<fl_blocks(M * 512, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(view(P), M, osrc, okind, members,
                                                                                target, new_cap);
    ++ctx->launches;
    e = cudaGetLastError();
    if (e != cudaSuccess) return undo(fl_check_cuda(ctx, e, "k_remap"));
    // From here the pool is being replaced: nothing below allocates until the
    // topology rebuild, whose failure leaves the pool unusable.
    cudaFreeAsync(osrc, ctx->stream);
    cudaFreeAsync(okind, ctx->stream);
    cudaFreeAsync(members, ctx->stream);
    fl_mesh old = P->mesh;
    fl_mesh_free(ctx, &old);
    out.num_cells = M;
    out.capacity = new_cap;
    P->mesh = out;
    if (grew) {
        for (int k = 0; k < 3; ++k) {
            cudaFreeAsync(P->f[k], ctx->stream);
            P->f[k] = nf[k];
        }
        release_brick_arrays(ctx, get_brick_arrays(P));
        put_brick_arrays(P, fresh);
        P->cap = new_cap;
    } else {
        // spare <- remapped; old A/B become free
        float* old0 = P->f[0];
        P->f[0] = target;
        P->f[2] = old0;
    }
    for (int l = 0; l < 16; ++l) P->parity[l] = 0;
    rc = pool_topology(ctx, P);
    if (rc == FL_OK) P->mesh_balanced = s.balance.converged != 0;
    if (st) *st = s;
    return rc;
}

// Grow every per-brick array to new_cap, keeping the first n bricks (both
// population buffers A and B are copied, so each level's parity stays valid).
// Grow the pool's per-brick storage to new_cap bricks.  Everything new is
// allocated before anything is copied or freed, so an allocation failure
// returns with the pool exactly as it was.
int pool_grow(fl_ctx* ctx, fl_pool* P, size_t new_cap) {
    if (new_cap <= P->cap) return FL_OK;
    size_t n = P->mesh.num_cells;
    fl_mesh m2{};
    int rc = fl_mesh_alloc(ctx, new_cap, 1, &m2);
    if (rc) return rc;
    float* nf[3] = {nullptr, nullptr, nullptr};
    auto undo = [&](int code) {
        for (float* p : nf)
            if (p) cudaFreeAsync(p, ctx->stream);
        fl_mesh_free(ctx, &m2);
        return code;
    };
    for (int k = 0; k < 3; ++k) {
        cudaError_t e = fl_dev_malloc_async(ctx, (void**)&nf[k], new_cap * 512 * Q * 4, ctx->stream);
        if (e != cudaSuccess) return undo(fl_check_cuda(ctx, e, "grow populations"));
    }
    BrickArrays fresh;
    rc = alloc_brick_arrays_beside(ctx, P, new_cap, &fresh);
    if (rc) return undo(rc);
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(m2.x, P->mesh.x, n * 4, cudaMemcpyDeviceToDevice, ctx->stream), "grow");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(m2.y, P->mesh.y, n * 4, cudaMemcpyDeviceToDevice, ctx->stream), "grow");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(m2.z, P->mesh.z, n * 4, cudaMemcpyDeviceToDevice, ctx->stream), "grow");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(m2.level, P->mesh.level, n, cudaMemcpyDeviceToDevice, ctx->stream), "grow");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(m2.state, P->mesh.state, n, cudaMemcpyDeviceToDevice, ctx->stream), "grow");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(m2.flags, P->mesh.flags, n * 4, cudaMemcpyDeviceToDevice, ctx->stream), "grow");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(m2.material, P->mesh.material, n * 4, cudaMemcpyDeviceToDevice, ctx->stream), "grow");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(m2.case_id, P->mesh.case_id, n * 2, cudaMemcpyDeviceToDevice, ctx->stream), "grow");
    m2.num_cells = n;
    fl_mesh old = P->mesh;
    fl_mesh_free(ctx, &old);
    P->mesh = m2;
    for (int k = 0; k < 3; ++k) {
        if (k < 2)
            for (int q = 0; q < Q; ++q)
                FL_TRY_CUDA(ctx, cudaMemcpyAsync(nf[k] + (size_t)q * new_cap * 512, P->f[k] + (size_t)q * P->cap * 512,
                                                 n * 512 * 4, cudaMemcpyDeviceToDevice, ctx->stream), "grow");
        cudaFreeAsync(P->f[k], ctx->stream);
        P->f[k] = nf[k];
    }
    release_brick_arrays(ctx, get_brick_arrays(P));
    put_brick_arrays(P, fresh);
    P->cap = new_cap;
    drop_graph(P);
    return FL_OK;
}

struct LaunchTimer {
    std::vector<cudaEvent_t> ev;  // start/stop pairs
    std::vector<uint64_t> sites;  // fluid sites processed by each launch
    std::vector<int> kind;        // 0 interior kernel, 1 general kernel, 2 all-solid bricks
    std::vector<int> level;       // the level of each launch
};

StepArgs level_args(fl_ctx* ctx, fl_pool* P, int l, int sub) {
    StepArgs a{};
    a.level = l;
    a.sub = sub;
    a.R = P->f[P->parity[l]];
    a.W = P->f[1 - P->parity[l]];
    a.Cold = l > 0 ? P->f[1 - P->parity[l - 1]] : nullptr;
    a.Cnew = l > 0 ? P->f[P->parity[l - 1]] : nullptr;
    a.Fine = l < 15 ? P->f[P->parity[l + 1]] : nullptr;
    a.cap = P->cap;
    a.bx = P->mesh.x; a.by = P->mesh.y; a.bz = P->mesh.z; a.blevel = P->mesh.level; a.bcase = P->mesh.case_id;
    a.nbr = P->nbr;
    a.cases = P->d_cases;
    a.dev_status = ctx->dev_status;
    a.desc = P->desc;
    a.smask = P->smask;
    a.qmask = P->qmask;
    a.pv = P->pv;
    return a;
}

// One brick class of level l on stream st (kind 0 interior, 1 general with its
// descriptor values, 2 all-solid), bracketed by timing events when tm is set.
void launch_class(fl_ctx* ctx, fl_pool* P, StepArgs a, int l, int kind, cudaStream_t st, LaunchTimer* tm) {
    const uint32_t off = P->cls_off[kind][l], cnt = P->cls_cnt[kind][l];
    if (!cnt) return;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (tm) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, st);
    }
    a.list = P->list + off;
    a.count = cnt;
    ctx->launches += (kind == 1 && P->lvl_desc[l + 1] > P->lvl_desc[l]) ? 2 : 1;
    const bool sums = a.part != nullptr;
    if (kind == 0) {
        unsigned grid = std::min<unsigned>(cnt, (unsigned)ctx->num_sms * P->grid_mult);
        if (P->staging) {
            if (sums) k_collide_staged<false, false, true><<<grid, 128, stage_bytes(false, false), st>>>(a, P->nb27);
            else k_collide_staged<false, false, false><<<grid, 128, stage_bytes(false, false), st>>>(a, P->nb27);
        } else {
            if (sums) k_collide_fast<true><<<grid, 128, 0, st>>>(a, P->nb27);
            else k_collide_fast<false><<<grid, 128, 0, st>>>(a, P->nb27);
        }
    } else if (kind == 1) {
        a.desc_off = P->slow_off + off;
        const uint32_t dd0 = P->lvl_desc[l], dd1 = P->lvl_desc[l + 1];
        if (dd1 > dd0) k_interface<<<fl_blocks(dd1 - dd0, 256, ctx->num_sms * 8), 256, 0, st>>>(a, dd0, dd1, P->pv);
        const unsigned grid = std::min<unsigned>(cnt, (unsigned)ctx->num_sms * 4);
        if (P->staging == 2) {
            if (sums) k_collide_staged<true, true, true><<<grid, 128, stage_bytes(true, true), st>>>(a, P->nb27);
            else k_collide_staged<true, true, false><<<grid, 128, stage_bytes(true, true), st>>>(a, P->nb27);
        } else if (P->staging == 1) {
            if (sums) k_collide_staged<true, false, true><<<grid, 128, stage_bytes(true, false), st>>>(a, P->nb27);
            else k_collide_staged<true, false, false><<<grid, 128, stage_bytes(true, false), st>>>(a, P->nb27);
        } else {
            if (sums) k_collide_general<true><<<grid, 128, 0, st>>>(a, P->nb27);
            else k_collide_general<false><<<grid, 128, 0, st>>>(a, P->nb27);
        }
    } else {
        k_collide_solid<<<fl_blocks((size_t)cnt * 512, 256, ctx->num_sms * 8), 256, 0, st>>>(a);
    }
    if (tm) {
        cudaEventRecord(e1, st);
        tm->ev.push_back(e0);
        tm->ev.push_back(e1);
        tm->sites.push_back(P->fluid_cls[kind][l]);
        tm->kind.push_back(kind);
        tm->level.push_back(l);
    }
}

// Sub-steps emitted per level within one level-0 step (dependency graph mode).
struct Dag {
    int k[kMaxPoolLevels] = {};
};

// One sub-step of level l.  Without a Dag every class runs in order on the
// context stream.  With one, level l's general, interface and all-solid bricks
// (the only bricks other levels read or that read other levels: coarse and
// fine sources are always interface bricks) run on P->sg[l], after level l's
// previous interior sub-step and the latest general sub-steps of levels l - 1
// and l + 1; its interior bricks run on P->sf[l], after level l's previous
// general sub-step.  Same-stream order covers the rest, including the
// write-after-read of each level's two population buffers.
void launch_level(fl_ctx* ctx, fl_pool* P, int l, int sub, LaunchTimer* tm, Dag* dag, bool last) {
    StepArgs a = level_args(ctx, P, l, sub);
    if (last && P->sums_enabled) a.part = P->part;  // the level's state after this level-0 step
    const bool solid = P->emit_solid || P->solid_due[l] > 0;
    if (!P->emit_solid && P->solid_due[l] > 0) --P->solid_due[l];
    if (!dag) {
        for (int kind = 0; kind < (solid ? 3 : 2); ++kind) launch_class(ctx, P, a, l, kind, ctx->stream, tm);
    } else {
        const int k = dag->k[l]++;
        cudaStream_t sg = P->sg[l], sf = P->sf[l];
        if (k > 0) cudaStreamWaitEvent(sg, P->evf[l][(k - 1) & 1], 0);
        if (l > 0 && dag->k[l - 1] > 0) cudaStreamWaitEvent(sg, P->evg[l - 1][(dag->k[l - 1] - 1) & 1], 0);
        if (l < P->maxL && dag->k[l + 1] > 0) cudaStreamWaitEvent(sg, P->evg[l + 1][(dag->k[l + 1] - 1) & 1], 0);
        launch_class(ctx, P, a, l, 1, sg, nullptr);
        if (solid) launch_class(ctx, P, a, l, 2, sg, nullptr);
        cudaEventRecord(P->evg[l][k & 1], sg);
        if (k > 0) cudaStreamWaitEvent(sf, P->evg[l][(k - 1) & 1], 0);
        launch_class(ctx, P, a, l, 0, sf, nullptr);
        cudaEventRecord(P->evf[l][k & 1], sf);
    }
    P->parity[l] ^= 1;
}

// last: this is level l's last sub-step of the level-0 step (every coarser
// level is in its last sub-step too).
void step_level(fl_ctx* ctx, fl_pool* P, int l, int sub, LaunchTimer* tm, Dag* dag, bool last) {
    launch_level(ctx, P, l, sub, tm, dag, last);
    if (l < P->maxL) {
        step_level(ctx, P, l + 1, 0, tm, dag, false);
        step_level(ctx, P, l + 1, 1, tm, dag, last);
    }
}

// One level-0 step: in order on the context stream, or as the dependency graph
// forked from and joined back into the context stream.
void level0_step(fl_ctx* ctx, fl_pool* P, LaunchTimer* tm = nullptr) {
    if (tm || P->streams < 2) {
        step_level(ctx, P, 0, 0, tm, nullptr, true);
        return;
    }
    Dag dag;
    cudaEventRecord(P->ev_root, ctx->stream);
    for (int l = 0; l <= P->maxL; ++l) {
        cudaStreamWaitEvent(P->sg[l], P->ev_root, 0);
        cudaStreamWaitEvent(P->sf[l], P->ev_root, 0);
    }
    step_level(ctx, P, 0, 0, nullptr, &dag, true);
    for (int l = 0; l <= P->maxL; ++l) {
        cudaStreamWaitEvent(ctx->stream, P->evg[l][(dag.k[l] - 1) & 1], 0);
        cudaStreamWaitEvent(ctx->stream, P->evf[l][(dag.k[l] - 1) & 1], 0);
    }
}

}  // namespace

// Accessors for the execution graph (graph.cu): what a captured step depends
// on, and the level-0 parity change a replay of n captured steps makes.
uint64_t fl_pool_launch_key(const fl_pool* P) { return (P->version << 1) | (uint64_t)(P->parity[0] & 1); }
void fl_pool_advance_parity(fl_pool* P, int nsteps) { P->parity[0] ^= (nsteps & 1); }

namespace {

// The solid-mask grid of active case `id` at `level` (ext * 8 << level voxels per axis).
int mask_grid(fl_ctx* ctx, fl_pool* P, int id, int level, uint64_t* N) {
    if (!ctx || !P) return FL_E_INVALID_ARG;
    if (id < 0 || id >= (int)P->active.size() || !P->active[id])
        return fl_set_error(ctx, FL_E_INVALID_ARG, "solid mask: not an active case");
    if (level < 0 || level >= kMaxPoolLevels) return fl_set_error(ctx, FL_E_INVALID_ARG, "solid mask: level out of range");
    for (int a = 0; a < 3; ++a) N[a] = (uint64_t)P->cases[id].ext[a] * 8 << level;
    if (N[0] * N[1] * N[2] > (1ull << 38)) return fl_set_error(ctx, FL_E_CAPACITY, "solid mask: more than 2^38 voxels");
    return FL_OK;
}

// Make `words` (device memory the pool now owns, or nullptr) the solid mask of
// case `id` and rebuild the topology: classes, descriptors and fluid counts
// follow the new solid sites; the populations are left as they are (solid
// sites take the rest state at the next step).
int install_mask(fl_ctx* ctx, fl_pool* P, int id, int level, uint32_t* words) {
    if (P->dmask.size() < P->cases.size()) P->dmask.resize(P->cases.size(), nullptr);
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "solid mask");
    if (P->dmask[id]) cudaFree(P->dmask[id]);
    P->dmask[id] = words;
    P->hcases[id].mask = words;
    P->hcases[id].mask_level = words ? level : 0;
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->d_cases + id, &P->hcases[id], sizeof(LbmCaseDev), cudaMemcpyHostToDevice,
                                     ctx->stream), "solid mask case");
    P->any_mask = false;
    for (size_t c = 0; c < P->dmask.size(); ++c)
        if (P->dmask[c] && c < P->active.size() && P->active[c]) P->any_mask = true;
    int rc = pool_topology(ctx, P);
    if (rc) return rc;
    return fl_collect_device_status(ctx, "solid mask");
}

// Free the solid masks of slots that are no longer active.
void release_masks(fl_ctx* ctx, fl_pool* P) {
    bool any = false;
    for (size_t c = 0; c < P->dmask.size(); ++c) {
        if (P->dmask[c] && !(c < P->active.size() && P->active[c])) {
            cudaFree(P->dmask[c]);
            P->dmask[c] = nullptr;
            P->hcases[c].mask = nullptr;
            cudaMemcpyAsync(P->d_cases + c, &P->hcases[c], sizeof(LbmCaseDev), cudaMemcpyHostToDevice, ctx->stream);
        }
        any = any || P->dmask[c] != nullptr;
    }
    P->any_mask = any;
}

}  // namespace

extern "C" {

int fl_pool_create(fl_ctx* ctx, const fl_lbm_case* cases, int ncases, fl_pool** out) {
    if (!ctx || !cases || ncases <= 0 || ncases > 4096 || !out) return FL_E_INVALID_ARG;
    *out = nullptr;
    fl_pool* P = new fl_pool();
    P->cases.assign(cases, cases + ncases);
    P->hcases.resize(ncases);
    std::vector<fl_domain_dev::Case> dom(ncases);
    size_t n0 = 0;
    for (int i = 0; i < ncases; ++i) {
        const fl_lbm_case& c = cases[i];
        for (int a = 0; a < 3; ++a)
            if (c.ext[a] < 1 || c.ext[a] > 16) { delete P; return fl_set_error(ctx, FL_E_INVALID_ARG, "case extent must be 1..16 bricks per axis"); }
        if (c.max_level < 0 || c.max_level > 13 || c.tau0 <= 0.5f) {
            delete P;
            return fl_set_error(ctx, FL_E_INVALID_ARG, "case max_level must be 0..13 and tau0 > 0.5");
        }
        to_dev_case(c, P->hcases[i]);
        for (int a = 0; a < 3; ++a) { dom[i].ext[a] = c.ext[a]; dom[i].periodic[a] = c.bc[2 * a] == 0; }
        P->maxL = std::max(P->maxL, (int)c.max_level);
        n0 += (size_t)c.ext[0] * c.ext[1] * c.ext[2];
    }
    int rc = FL_OK;
    auto fail = [&](int r) { fl_pool_destroy(ctx, P); return r; };
    bool sok = cudaEventCreateWithFlags(&P->ev_root, cudaEventDisableTiming) == cudaSuccess;
    for (int l = 0; l < kMaxPoolLevels && sok; ++l) {
        sok = cudaStreamCreateWithFlags(&P->sg[l], cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&P->sf[l], cudaStreamNonBlocking) == cudaSuccess;
        for (int j = 0; j < 2 && sok; ++j)
            sok = cudaEventCreateWithFlags(&P->evg[l][j], cudaEventDisableTiming) == cudaSuccess &&
                  cudaEventCreateWithFlags(&P->evf[l][j], cudaEventDisableTiming) == cudaSuccess;
    }
    if (!sok) return fail(fl_set_error(ctx, FL_E_CUDA, "fl_pool_create: stream or event creation failed"));
    // case tables sized for every slot a pool can hold (cases may be added later)
    if (fl_dev_malloc(ctx, (void**)&P->d_cases, kMaxCases * sizeof(LbmCaseDev)) != cudaSuccess) return fail(FL_E_OOM);
    if (fl_dev_malloc(ctx, (void**)&P->d_dom, kMaxCases * sizeof(fl_domain_dev::Case)) != cudaSuccess) return fail(FL_E_OOM);
    if (fl_dev_malloc(ctx, (void**)&P->d_case_begin, (kMaxCases + 1) * 4) != cudaSuccess) return fail(FL_E_OOM);
    if (fl_dev_malloc(ctx, (void**)&P->d_topo, sizeof(TopoCounters)) != cudaSuccess) return fail(FL_E_OOM);
    if (fl_dev_malloc(ctx, (void**)&P->d_case_chunk, (kMaxCases + 1) * 4) != cudaSuccess) return fail(FL_E_OOM);
    if (fl_dev_malloc(ctx, (void**)&P->case_max, kMaxCases * 4) != cudaSuccess) return fail(FL_E_OOM);
    if (fl_dev_malloc(ctx, (void**)&P->cons, kMaxCases * 32) != cudaSuccess) return fail(FL_E_OOM);
    if (fl_dev_malloc(ctx, (void**)&P->d_mask, kMaxCases) != cudaSuccess) return fail(FL_E_OOM);
    P->active.assign(ncases, 1);
    cudaMemcpy(P->d_cases, P->hcases.data(), ncases * sizeof(LbmCaseDev), cudaMemcpyHostToDevice);
    cudaMemcpy(P->d_dom, dom.data(), ncases * sizeof(fl_domain_dev::Case), cudaMemcpyHostToDevice);
    // level-0 bricks, unsorted
    std::vector<int32_t> x, y, z;
    std::vector<uint16_t> cs;
    for (int i = 0; i < ncases; ++i)
        for (int32_t k = 0; k < cases[i].ext[2]; ++k)
            for (int32_t j = 0; j < cases[i].ext[1]; ++j)
                for (int32_t a = 0; a < cases[i].ext[0]; ++a) {
                    x.push_back(a); y.push_back(j); z.push_back(k); cs.push_back((uint16_t)i);
                }
    P->cap = std::max<size_t>(n0 * 2, 64);
    rc = fl_mesh_alloc(ctx, P->cap, 1, &P->mesh);
    if (rc) return fail(rc);
    cudaMemcpyAsync(P->mesh.x, x.data(), n0 * 4, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(P->mesh.y, y.data(), n0 * 4, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(P->mesh.z, z.data(), n0 * 4, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(P->mesh.case_id, cs.data(), n0 * 2, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(P->mesh.level, 0, n0, ctx->stream);
    cudaMemsetAsync(P->mesh.state, 0, n0, ctx->stream);
    cudaMemsetAsync(P->mesh.flags, 0, n0 * 4, ctx->stream);
    cudaMemsetAsync(P->mesh.material, 0, n0 * 4, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    P->mesh.num_cells = n0;
    for (int k = 0; k < 3; ++k)
        if (fl_dev_malloc_async(ctx, (void**)&P->f[k], P->cap * 512 * Q * 4, ctx->stream) != cudaSuccess) return fail(FL_E_OOM);
    rc = alloc_brick_arrays(ctx, P, P->cap);
    if (rc) return fail(rc);
    // an adapt with all flags 0 only sorts: bricks into key order
    rc = pool_init_populations(ctx, P);
    if (rc) return fail(rc);
    rc = pool_regrid(ctx, P, -1, nullptr);
    if (rc) return fail(rc);
    for (int r = 0; r < P->maxL; ++r) {
        rc = pool_regrid(ctx, P, 0, nullptr);
        if (rc) return fail(rc);
    }
    rc = pool_init_populations(ctx, P);
    if (rc) return fail(rc);
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "pool create");
    *out = P;
    return FL_OK;
}

int fl_pool_destroy(fl_ctx* ctx, fl_pool* P) {
    if (!ctx || !P) return FL_E_INVALID_ARG;
    cudaStreamSynchronize(ctx->stream);
    free_graphs(P);
    free_brick_arrays(ctx, P);
    for (int k = 0; k < 3; ++k)
        if (P->f[k]) cudaFreeAsync(P->f[k], ctx->stream);
    if (P->mesh.x) fl_mesh_free(ctx, &P->mesh);
    if (P->adapt_scratch) cudaFreeAsync(P->adapt_scratch, ctx->stream);
    if (P->desc) cudaFreeAsync(P->desc, ctx->stream);
    if (P->pv) cudaFreeAsync(P->pv, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    if (P->d_cases) cudaFree(P->d_cases);
    if (P->d_dom) cudaFree(P->d_dom);
    if (P->d_case_begin) cudaFree(P->d_case_begin);
    if (P->d_topo) cudaFree(P->d_topo);
    if (P->d_case_chunk) cudaFree(P->d_case_chunk);
    if (P->case_max) cudaFree(P->case_max);
    if (P->cons) cudaFree(P->cons);
    if (P->d_mask) cudaFree(P->d_mask);
    for (uint32_t* m : P->dmask)
        if (m) cudaFree(m);
    for (int l = 0; l < kMaxPoolLevels; ++l) {
        if (P->sg[l]) cudaStreamDestroy(P->sg[l]);
        if (P->sf[l]) cudaStreamDestroy(P->sf[l]);
        for (int j = 0; j < 2; ++j) {
            if (P->evg[l][j]) cudaEventDestroy(P->evg[l][j]);
            if (P->evf[l][j]) cudaEventDestroy(P->evf[l][j]);
        }
    }
    if (P->ev_root) cudaEventDestroy(P->ev_root);
    delete P;
    return FL_OK;
}

int fl_pool_step(fl_ctx* ctx, fl_pool* P, int nsteps) {
    if (!ctx || !P || nsteps < 0) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
    FL_TRY_CUDA(ctx, cudaStreamIsCapturing(ctx->stream, &capturing), "capture status");
    P->emit_solid = capturing != cudaStreamCaptureStatusNone;
    for (int i = 0; i < nsteps; ++i) {
        // inside a caller's stream capture the launches join that capture directly
        if (!P->graphs || capturing != cudaStreamCaptureStatusNone) {
            level0_step(ctx, P);
            FL_CHECK_ERRORS(ctx, "k_collide_stream");
            continue;
        }
        // One level-0 step changes only level 0's parity (level l >= 1 runs an
        // even number of sub-steps), so two captured graphs, one per level-0
        // parity, replay every step until the topology changes.  While some
        // level still owes all-solid writes (both buffers must hold the rest
        // state), a second pair, captured with those bricks written in every
        // sub-step, replays instead: writing the rest state once more changes
        // nothing, so the populations are those of the uncaptured steps.
        bool settled = true;
        for (int l = 0; l <= P->maxL; ++l) settled = settled && P->solid_due[l] == 0;
        const int p0 = P->parity[0];
        cudaGraphExec_t* exec = settled ? &P->graph[p0] : &P->graph_solid[p0];
        bool* ok = settled ? &P->graph_ok[p0] : &P->graph_solid_ok[p0];
        uint64_t* kernels = settled ? &P->graph_kernels[p0] : &P->graph_solid_kernels[p0];
        if (!*ok) {
            int saved[16];
            std::memcpy(saved, P->parity, sizeof(saved));
            int saved_due[kMaxPoolLevels];
            std::memcpy(saved_due, P->solid_due, sizeof(saved_due));
            cudaGraph_t g;
            const uint64_t c0 = ctx->launches;
            P->emit_solid = !settled;
            FL_TRY_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "capture begin");
            level0_step(ctx, P);
            cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
            P->emit_solid = false;
            *kernels = ctx->launches - c0;  // recorded, not launched: counted per replay
            ctx->launches = c0;
            std::memcpy(P->parity, saved, sizeof(saved));
            std::memcpy(P->solid_due, saved_due, sizeof(saved_due));
            FL_TRY_CUDA(ctx, e, "capture end");
            bool updated = false;
            if (*exec) {
                cudaGraphExecUpdateResultInfo info;
                updated = cudaGraphExecUpdate(*exec, g, &info) == cudaSuccess;
                if (!updated) {
                    cudaGetLastError();  // a failed update leaves no sticky error; clear the last one
                    cudaGraphExecDestroy(*exec);
                    *exec = nullptr;
                }
            }
            if (!updated) e = cudaGraphInstantiate(exec, g, 0);
            cudaGraphDestroy(g);
            FL_TRY_CUDA(ctx, e, "graph instantiate");
            *ok = true;
        }
        FL_TRY_CUDA(ctx, cudaGraphLaunch(*exec, ctx->stream), "graph launch");
        ctx->launches += *kernels;
        P->parity[0] ^= 1;
        if (!settled)  // level l ran 2^l sub-steps, each of which pays one owed write
            for (int l = 0; l <= P->maxL; ++l) P->solid_due[l] = std::max(0, P->solid_due[l] - (1 << l));
    }
    // the steps wrote the sums of the state they leave (a caller's capture only recorded them)
    if (nsteps > 0) P->sums_fresh = P->sums_enabled && capturing == cudaStreamCaptureStatusNone;
    return FL_OK;
}

int fl_pool_regrid(fl_ctx* ctx, fl_pool* P, fl_adapt_stats* st) {
    if (!ctx || !P) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    int rc = pool_regrid(ctx, P, 1, st);
    if (rc) return rc;
    return fl_collect_device_status(ctx, "fl_pool_regrid");
}

int fl_pool_info_get(fl_ctx* ctx, fl_pool* P, fl_pool_info* info) {
    if (!ctx || !P || !info) return FL_E_INVALID_ARG;
    std::memset(info, 0, sizeof(*info));
    info->num_bricks = P->mesh.num_cells;
    info->capacity = P->cap;
    info->num_cases = (int32_t)P->cases.size();
    info->num_active_cases = (int32_t)std::count(P->active.begin(), P->active.end(), (uint8_t)1);
    info->max_level = P->maxL;
    for (int l = 0; l <= P->maxL && l < 16; ++l) info->bricks_per_level[l] = P->lvl_off[l + 1] - P->lvl_off[l];
    info->fluid_lups_per_step = P->lups;
    for (int l = 0; l < 16; ++l) info->fluid_sites_per_level[l] = P->fluid_per_level[l];
    info->population_bytes = (uint64_t)P->cap * 512 * Q * 4 * 3;
    info->usable = P->unusable ? 0 : 1;
    for (int l = 0; l <= P->maxL && l < 16; ++l) {
        info->general_bricks_per_level[l] = P->cls_cnt[1].size() > (size_t)l ? P->cls_cnt[1][l] : 0;
        info->stencil_descriptors_per_level[l] =
            P->lvl_desc.size() > (size_t)l + 1 ? (uint64_t)(P->lvl_desc[l + 1] - P->lvl_desc[l]) : 0;
    }
    return FL_OK;
}

int fl_pool_download(fl_ctx* ctx, fl_pool* P, int32_t* x, int32_t* y, int32_t* z, uint8_t* level, uint16_t* case_id,
                     float* f) {
    if (!ctx || !P) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    size_t n = P->mesh.num_cells;
    if (x) FL_TRY_CUDA(ctx, cudaMemcpyAsync(x, P->mesh.x, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "dl");
    if (y) FL_TRY_CUDA(ctx, cudaMemcpyAsync(y, P->mesh.y, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "dl");
    if (z) FL_TRY_CUDA(ctx, cudaMemcpyAsync(z, P->mesh.z, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "dl");
    if (level) FL_TRY_CUDA(ctx, cudaMemcpyAsync(level, P->mesh.level, n, cudaMemcpyDeviceToHost, ctx->stream), "dl");
    if (case_id) FL_TRY_CUDA(ctx, cudaMemcpyAsync(case_id, P->mesh.case_id, n * 2, cudaMemcpyDeviceToHost, ctx->stream), "dl");
    if (f && n) {
        // the levels' current buffers: one of the two for all of them (one copy per population), or
        // mixed -- level 0 has flipped once more than the others after an odd number of level-0 steps --
        // and then gathered on the device into the spare buffer first
        uint32_t odd = 0, present = 0;
        for (int l = 0; l <= P->maxL; ++l) {
            if (P->lvl_off[l + 1] == P->lvl_off[l]) continue;
            present |= 1u << l;
            if (P->parity[l]) odd |= 1u << l;
        }
        const float* src = P->f[odd ? 1 : 0];
        if (odd && odd != present) {
            k_gather_current<<<fl_blocks((size_t)Q * n * 128, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
                P->f[0], P->f[1], P->f[2], P->cap, n, P->mesh.level, odd);
            FL_CHECK_LAUNCH(ctx, "k_gather_current");
            src = P->f[2];
        }
        for (int q = 0; q < Q; ++q)
            FL_TRY_CUDA(ctx, cudaMemcpyAsync(f + (size_t)q * n * 512, src + (size_t)q * P->cap * 512, n * 512 * 4,
                                             cudaMemcpyDeviceToHost, ctx->stream), "dl f");
    }
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "download");
    return FL_OK;
}

int fl_pool_nbr(fl_ctx* ctx, fl_pool* P, uint32_t* nbr) {
    if (!ctx || !P || !nbr) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(nbr, P->nbr, P->mesh.num_cells * 26 * 4 * 4, cudaMemcpyDeviceToHost, ctx->stream), "nbr");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "nbr");
    return FL_OK;
}

int fl_pool_flags(fl_ctx* ctx, fl_pool* P, int32_t* flags, float* wmax) {
    if (!ctx || !P) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    int rc = pool_flags(ctx, P, 1);
    if (rc) return rc;
    size_t n = P->mesh.num_cells;
    if (flags) FL_TRY_CUDA(ctx, cudaMemcpyAsync(flags, P->mesh.flags, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "flags");
    if (wmax) FL_TRY_CUDA(ctx, cudaMemcpyAsync(wmax, P->wmax, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "wmax");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "flags");
    return FL_OK;
}

int fl_pool_conservation(fl_ctx* ctx, fl_pool* P, double* out) {
    int rc = fl_pool_conservation_async(ctx, P, out);
    if (rc) return rc;
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "conservation");
    return fl_collect_device_status(ctx, "fl_pool_conservation");
}

int fl_pool_conservation_async(fl_ctx* ctx, fl_pool* P, double* out) {
    if (!ctx || !P || !out) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    size_t n = P->mesh.num_cells;
    if (!P->sums_fresh) {  // else the last step's collide kernels wrote them (brick_sums_store)
        k_brick_sums<<<fl_blocks(n, 1, ctx->num_sms * 16), 128, 0, ctx->stream>>>(view(P), n, P->part);
        FL_CHECK_LAUNCH(ctx, "k_brick_sums");
        P->sums_fresh = P->sums_enabled;
    }
    int nc = (int)P->cases.size();
    if (P->nchunks) {
        k_chunk_sums<<<std::min<uint32_t>(P->nchunks, (uint32_t)ctx->num_sms * 8), 256, 0, ctx->stream>>>(
            P->part, P->mesh.level, P->d_chunks, P->nchunks, P->chunk_part);
        FL_CHECK_LAUNCH(ctx, "k_chunk_sums");
    }
    k_case_sums<<<(nc * 4 + 255) / 256, 256, 0, ctx->stream>>>(P->chunk_part, P->d_case_chunk, nc, P->cons);
    FL_CHECK_LAUNCH(ctx, "k_case_sums");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(out, P->cons, nc * 32, cudaMemcpyDefault, ctx->stream), "conservation");
    return FL_OK;
}

// Per-launch timing pass shared by the two profile entry points: totals per
// [level][class] (16 x 3 each).
int profile_levels(fl_ctx* ctx, fl_pool* P, int nsteps, double* ms, uint32_t* cnt, uint64_t* sites) {
    LaunchTimer tm;
    for (int i = 0; i < nsteps; ++i) level0_step(ctx, P, &tm);
    FL_CHECK_ERRORS(ctx, "collide-stream");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "profile sync");
    for (int k = 0; k < 48; ++k) { ms[k] = 0.0; cnt[k] = 0; sites[k] = 0; }
    for (size_t k = 0; k < tm.ev.size(); k += 2) {
        float t = 0.0f;
        cudaEventElapsedTime(&t, tm.ev[k], tm.ev[k + 1]);
        const int slot = tm.level[k / 2] * 3 + tm.kind[k / 2];
        ms[slot] += t;
        sites[slot] += tm.sites[k / 2];
        cnt[slot] += 1;
        cudaEventDestroy(tm.ev[k]);
        cudaEventDestroy(tm.ev[k + 1]);
    }
    return FL_OK;  // the topology and buffers are unchanged: the captured steps stay valid
}

int fl_pool_profile_steps(fl_ctx* ctx, fl_pool* P, int nsteps, double* kernel_ms, uint32_t* launches,
                          uint64_t* fluid_sites) {
    if (!ctx || !P || nsteps < 0) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    double ms[48];
    uint32_t cnt[48];
    uint64_t sites[48];
    int rc = profile_levels(ctx, P, nsteps, ms, cnt, sites);
    if (rc) return rc;
    for (int k = 0; k < 3; ++k) {
        double m = 0.0;
        uint32_t c = 0;
        uint64_t st = 0;
        for (int l = 0; l < 16; ++l) { m += ms[l * 3 + k]; c += cnt[l * 3 + k]; st += sites[l * 3 + k]; }
        if (kernel_ms) kernel_ms[k] = m;
        if (launches) launches[k] = c;
        if (fluid_sites) fluid_sites[k] = st;
    }
    return fl_collect_device_status(ctx, "fl_pool_profile_steps");
}

int fl_pool_profile_levels(fl_ctx* ctx, fl_pool* P, int nsteps, double* kernel_ms, uint32_t* launches,
                           uint64_t* fluid_sites) {
    if (!ctx || !P || nsteps < 0 || !kernel_ms || !launches || !fluid_sites) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    int rc = profile_levels(ctx, P, nsteps, kernel_ms, launches, fluid_sites);
    if (rc) return rc;
    return fl_collect_device_status(ctx, "fl_pool_profile_levels");
}

int fl_pool_upload(fl_ctx* ctx, fl_pool* P, const float* f) {
    if (!ctx || !P || !f) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    size_t n = P->mesh.num_cells;
    for (int q = 0; q < Q; ++q)
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->f[0] + (size_t)q * P->cap * 512, f + (size_t)q * n * 512, n * 512 * 4,
                                         cudaMemcpyHostToDevice, ctx->stream), "upload");
    // level l >= 1 is back to parity 0 at every level-0 step boundary, so the captured
    // steps stay valid; only the all-solid bricks must be written again
    for (int l = 0; l < 16; ++l) P->parity[l] = 0;
    populations_replaced(P);
    return FL_OK;
}

int fl_pool_macroscopic(fl_ctx* ctx, fl_pool* P, float* rho, float* ux, float* uy, float* uz) {
    if (!ctx || !P || !rho || !ux || !uy || !uz) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    const size_t n = P->mesh.num_cells, sites = n * 512;
    if (!n) return FL_OK;
    float* d = nullptr;
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&d, sites * 16, ctx->stream), "macroscopic buffer");
    k_macroscopic<<<fl_blocks(n, 1, ctx->num_sms * 16), 128, 0, ctx->stream>>>(view(P), n, d, d + sites,
                                                                               d + 2 * sites, d + 3 * sites);
    FL_CHECK_LAUNCH(ctx, "k_macroscopic");
    float* out[4] = {rho, ux, uy, uz};
    for (int k = 0; k < 4; ++k)
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(out[k], d + k * sites, sites * 4, cudaMemcpyDeviceToHost, ctx->stream),
                    "macroscopic download");
    cudaFreeAsync(d, ctx->stream);
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "macroscopic");
    return fl_collect_device_status(ctx, "fl_pool_macroscopic");
}

int fl_pool_load(fl_ctx* ctx, fl_pool* P, size_t n, const int32_t* x, const int32_t* y, const int32_t* z,
                 const uint8_t* level, const uint16_t* case_id, const float* f) {
    if (!ctx || !P || !n || !x || !y || !z || !level || !case_id || !f) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    for (size_t i = 0; i < n; ++i) {
        const int cs = case_id[i], l = level[i];
        if (cs >= (int)P->cases.size() || !P->active[cs] || l > P->maxL)
            return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_pool_load: brick with an unknown case or a level above the pool maximum");
        const int32_t c[3] = {x[i], y[i], z[i]};
        for (int a = 0; a < 3; ++a)
            if (c[a] < 0 || c[a] >= (P->cases[cs].ext[a] << l))
                return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_pool_load: brick outside its case's domain");
    }
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "load");
    if (n > P->cap) {
        int rc = pool_grow(ctx, P, std::max((size_t)(n * 1.5), n + 64));
        if (rc) return rc;
    }
    P->unusable = true;  // until the loaded bricks' tables are rebuilt
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.x, x, n * 4, cudaMemcpyHostToDevice, ctx->stream), "load");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.y, y, n * 4, cudaMemcpyHostToDevice, ctx->stream), "load");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.z, z, n * 4, cudaMemcpyHostToDevice, ctx->stream), "load");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.level, level, n, cudaMemcpyHostToDevice, ctx->stream), "load");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.case_id, case_id, n * 2, cudaMemcpyHostToDevice, ctx->stream), "load");
    FL_TRY_CUDA(ctx, cudaMemsetAsync(P->mesh.state, 0, n, ctx->stream), "load");
    FL_TRY_CUDA(ctx, cudaMemsetAsync(P->mesh.flags, 0, n * 4, ctx->stream), "load");
    FL_TRY_CUDA(ctx, cudaMemsetAsync(P->mesh.material, 0, n * 4, ctx->stream), "load");
    P->mesh.num_cells = n;
    P->mesh_balanced = false;  // bricks from outside
    for (int q = 0; q < Q; ++q)
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->f[0] + (size_t)q * P->cap * 512, f + (size_t)q * n * 512, n * 512 * 4,
                                         cudaMemcpyHostToDevice, ctx->stream), "load populations");
    for (int l = 0; l < 16; ++l) P->parity[l] = 0;
    // an adapt with every flag 0 only sorts: bricks (and their populations) into key order
    int rc = pool_regrid(ctx, P, -1, nullptr);
    if (rc) return rc;
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "load");
    return fl_collect_device_status(ctx, "fl_pool_load");
}

int fl_pool_set_velocities(fl_ctx* ctx, fl_pool* P, const float* wall_u, const float* inlet_u) {
    if (!ctx || !P) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    // per case 3 floats each; a host->device copy ordered on the stream, read by the next step
    for (size_t c = 0; c < P->cases.size(); ++c) {
        char* base = (char*)P->d_cases + c * sizeof(LbmCaseDev);
        if (wall_u)
            FL_TRY_CUDA(ctx, cudaMemcpyAsync(base + offsetof(LbmCaseDev, wall_u), wall_u + 3 * c, 12,
                                             cudaMemcpyHostToDevice, ctx->stream), "velocities");
        if (inlet_u)
            FL_TRY_CUDA(ctx, cudaMemcpyAsync(base + offsetof(LbmCaseDev, inlet_u), inlet_u + 3 * c, 12,
                                             cudaMemcpyHostToDevice, ctx->stream), "velocities");
    }
    return FL_OK;
}

int fl_pool_set_solid_mask(fl_ctx* ctx, fl_pool* P, int32_t id, int32_t level, const uint32_t* bits, size_t nwords) {
    uint64_t N[3];
    int rc = mask_grid(ctx, P, id, level, N);
    if (rc) return rc;
    if (!bits) return install_mask(ctx, P, id, 0, nullptr);
    const uint64_t words = (N[0] * N[1] * N[2] + 31) / 32;
    if (nwords != words) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_pool_set_solid_mask: nwords != ceil(Nx*Ny*Nz/32)");
    uint32_t* d = nullptr;
    if (fl_dev_malloc(ctx, (void**)&d, words * 4) != cudaSuccess) return fl_set_error(ctx, FL_E_OOM, "solid mask");
    if (cudaMemcpyAsync(d, bits, words * 4, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess) {
        cudaFree(d);
        return fl_set_error(ctx, FL_E_CUDA, "solid mask upload");
    }
    return install_mask(ctx, P, id, level, d);
}

int fl_pool_set_solid_cells(fl_ctx* ctx, fl_pool* P, int32_t id, int32_t level, const int32_t* x, const int32_t* y,
                            const int32_t* z, size_t n) {
    uint64_t N[3];
    int rc = mask_grid(ctx, P, id, level, N);
    if (rc) return rc;
    if (n && (!x || !y || !z)) return FL_E_INVALID_ARG;
    const uint64_t words = (N[0] * N[1] * N[2] + 31) / 32;
    uint32_t* d = nullptr;
    if (fl_dev_malloc(ctx, (void**)&d, words * 4) != cudaSuccess) return fl_set_error(ctx, FL_E_OOM, "solid mask");
    cudaMemsetAsync(d, 0, words * 4, ctx->stream);
    if (n) {
        k_mask_cells<<<fl_blocks(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(x, y, z, n, (int64_t)N[0],
                                                                                   (int64_t)N[1], (int64_t)N[2], d);
        if (cudaPeekAtLastError() != cudaSuccess) {
            cudaFree(d);
            return fl_set_error(ctx, FL_E_CUDA, "k_mask_cells launch");
        }
        ++ctx->launches;
    }
    return install_mask(ctx, P, id, level, d);
}

int fl_pool_get_solid_mask(fl_ctx* ctx, fl_pool* P, int32_t id, int32_t* level, uint32_t* bits, size_t nwords) {
    if (!ctx || !P || !level || id < 0 || id >= (int)P->active.size() || !P->active[id])
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_pool_get_solid_mask: not an active case");
    FL_POOL_USABLE(ctx, P);
    FL_POOL_USABLE(ctx, P);
    FL_POOL_USABLE(ctx, P);
    const bool has = id < (int)P->dmask.size() && P->dmask[id];
    *level = has ? P->hcases[id].mask_level : -1;
    if (!has || !bits) return FL_OK;
    uint64_t N[3];
    int rc = mask_grid(ctx, P, id, *level, N);
    if (rc) return rc;
    const uint64_t words = (N[0] * N[1] * N[2] + 31) / 32;
    if (nwords < words) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_pool_get_solid_mask: buffer too small");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(bits, P->dmask[id], words * 4, cudaMemcpyDeviceToHost, ctx->stream), "mask");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "mask");
    return FL_OK;
}

int fl_pool_regrid_flags(fl_ctx* ctx, fl_pool* P, const int32_t* flags, fl_adapt_stats* st) {
    if (!ctx || !P || !flags) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    int rc = pool_regrid(ctx, P, 0, st, nullptr, flags);
    if (rc) return rc;
    return fl_collect_device_status(ctx, "fl_pool_regrid_flags");
}

int fl_pool_regrid_cases(fl_ctx* ctx, fl_pool* P, const uint8_t* due, fl_adapt_stats* st) {
    if (!ctx || !P || !due) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    int rc = pool_regrid(ctx, P, 1, st, due);
    if (rc) return rc;
    return fl_collect_device_status(ctx, "fl_pool_regrid_cases");
}

int fl_pool_add_cases(fl_ctx* ctx, fl_pool* P, const fl_lbm_case* cases, int ncases, int32_t* ids) {
    if (!ctx || !P || !cases || ncases <= 0 || !ids) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    // slots: freed ids first, then ids past the last one used
    std::vector<int> slot;
    for (int i = 0; i < (int)P->active.size() && (int)slot.size() < ncases; ++i)
        if (!P->active[i]) slot.push_back(i);
    for (int next = (int)P->active.size(); (int)slot.size() < ncases && next < kMaxCases; ++next) slot.push_back(next);
    if ((int)slot.size() < ncases) return fl_set_error(ctx, FL_E_CAPACITY, "fl_pool_add_cases: no free case slots");
    // build the new cases exactly as a pool of their own would start
    fl_pool* T = nullptr;
    int rc = fl_pool_create(ctx, cases, ncases, &T);
    if (rc) return rc;
    size_t n = P->mesh.num_cells, nt = T->mesh.num_cells;
    if (n + nt > P->cap) {
        rc = pool_grow(ctx, P, std::max((size_t)((n + nt) * 1.5), n + nt + 64));
        if (rc) { fl_pool_destroy(ctx, T); return rc; }
    }
    // append columns (case ids mapped to the slots) and populations (into A and B);
    // the pool is unusable until the regrid below has rebuilt its tables
    P->unusable = true;
    std::vector<uint16_t> tc(nt);
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(tc.data(), T->mesh.case_id, nt * 2, cudaMemcpyDeviceToHost, ctx->stream), "add");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "add");
    for (auto& v : tc) v = (uint16_t)slot[v];
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.case_id + n, tc.data(), nt * 2, cudaMemcpyHostToDevice, ctx->stream), "add");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.x + n, T->mesh.x, nt * 4, cudaMemcpyDeviceToDevice, ctx->stream), "add");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.y + n, T->mesh.y, nt * 4, cudaMemcpyDeviceToDevice, ctx->stream), "add");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.z + n, T->mesh.z, nt * 4, cudaMemcpyDeviceToDevice, ctx->stream), "add");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.level + n, T->mesh.level, nt, cudaMemcpyDeviceToDevice, ctx->stream), "add");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.state + n, T->mesh.state, nt, cudaMemcpyDeviceToDevice, ctx->stream), "add");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.flags + n, T->mesh.flags, nt * 4, cudaMemcpyDeviceToDevice, ctx->stream), "add");
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->mesh.material + n, T->mesh.material, nt * 4, cudaMemcpyDeviceToDevice, ctx->stream), "add");
    for (int k = 0; k < 2; ++k)
        for (int q = 0; q < Q; ++q)
            FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->f[k] + ((size_t)q * P->cap + n) * 512, T->f[0] + (size_t)q * T->cap * 512,
                                             nt * 512 * 4, cudaMemcpyDeviceToDevice, ctx->stream), "add");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "add");
    // case tables
    for (int i = 0; i < ncases; ++i) {
        int sl = slot[i];
        if (sl >= (int)P->cases.size()) {
            P->cases.resize(sl + 1);
            P->hcases.resize(sl + 1);
            P->active.resize(sl + 1, 0);
        }
        P->cases[sl] = cases[i];
        to_dev_case(cases[i], P->hcases[sl]);
        P->active[sl] = 1;
        fl_domain_dev::Case d;
        for (int a = 0; a < 3; ++a) { d.ext[a] = cases[i].ext[a]; d.periodic[a] = cases[i].bc[2 * a] == 0; }
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->d_cases + sl, &P->hcases[sl], sizeof(LbmCaseDev), cudaMemcpyHostToDevice,
                                         ctx->stream), "add tables");
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->d_dom + sl, &d, sizeof(d), cudaMemcpyHostToDevice, ctx->stream), "add tables");
        FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "add tables");
        P->maxL = std::max(P->maxL, (int)cases[i].max_level);
        ids[i] = sl;
    }
    fl_pool_destroy(ctx, T);
    P->mesh.num_cells = n + nt;
    P->mesh_balanced = false;  // new cases' bricks
    // one regrid with every flag 0 only re-sorts by (case, key) and rebuilds the topology
    rc = pool_regrid(ctx, P, -1, nullptr);
    if (rc) return rc;
    return fl_collect_device_status(ctx, "fl_pool_add_cases");
}

int fl_pool_remove_cases(fl_ctx* ctx, fl_pool* P, const int32_t* ids, int nids) {
    if (!ctx || !P || (nids && !ids)) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    for (int i = 0; i < nids; ++i) {
        if (ids[i] < 0 || ids[i] >= (int)P->active.size() || !P->active[ids[i]])
            return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_pool_remove_cases: not an active case");
    }
    P->unusable = true;  // until the compacted pool's tables are rebuilt
    for (int i = 0; i < nids; ++i) P->active[ids[i]] = 0;
    release_masks(ctx, P);
    size_t n = P->mesh.num_cells;
    if (n == 0) return FL_OK;
    size_t sb = 3 * fl_align256(n * 4) + fl_scan_scratch_bytes(n) + 512;
    int rc = fl_scratch_reserve(ctx, sb);
    if (rc) return rc;
    char* p = (char*)ctx->scratch;
    uint32_t* keep = (uint32_t*)p; p += fl_align256(n * 4);
    uint32_t* off = (uint32_t*)p; p += fl_align256(n * 4);
    uint32_t* total = (uint32_t*)p; p += fl_align256(n * 4);
    void* ss = p;
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(P->d_mask, P->active.data(), P->active.size(), cudaMemcpyHostToDevice, ctx->stream),
                "active");
    k_keep_bricks<<<fl_blocks(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(n, P->mesh.case_id, P->d_mask, keep);
    FL_CHECK_LAUNCH(ctx, "k_keep_bricks");
    rc = fl_scan_u32_with(ctx, keep, off, n, total, ss);
    if (rc) return rc;
    uint32_t M = 0;
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(&M, total, 4, cudaMemcpyDeviceToHost, ctx->stream), "kept");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "kept");
    fl_mesh out{};
    rc = fl_mesh_alloc(ctx, P->cap, 1, &out);
    if (rc) return rc;
    uint32_t* osrc = nullptr;
    uint8_t* okind = nullptr;
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&osrc, (M + 1) * 4, ctx->stream), "remove src");
    FL_TRY_CUDA(ctx, fl_dev_malloc_async(ctx, (void**)&okind, M + 1, ctx->stream), "remove kind");
    fl_mesh_dev md{P->mesh.x, P->mesh.y, P->mesh.z, P->mesh.level, P->mesh.state, P->mesh.flags, P->mesh.material,
                   P->mesh.case_id, n};
    fl_mesh_out o{out.x, out.y, out.z, out.level, out.state, out.flags, out.material, out.case_id};
    k_compact_bricks<<<fl_blocks(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(md, keep, off, o, osrc, okind);
    FL_CHECK_LAUNCH(ctx, "k_compact_bricks");
    if (M) {
        k_remap<<<fl_blocks((size_t)M * 512, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(view(P), M, osrc, okind,
                                                                                        nullptr, P->f[2], P->cap);
        FL_CHECK_LAUNCH(ctx, "k_remap");
    }
    cudaFreeAsync(osrc, ctx->stream);
    cudaFreeAsync(okind, ctx->stream);
    fl_mesh old = P->mesh;
    fl_mesh_free(ctx, &old);
    out.num_cells = M;
    out.capacity = P->cap;
    P->mesh = out;
    float* old0 = P->f[0];
    P->f[0] = P->f[2];
    P->f[2] = old0;
    for (int l = 0; l < 16; ++l) P->parity[l] = 0;
    rc = pool_topology(ctx, P);
    if (rc) return rc;
    return fl_collect_device_status(ctx, "fl_pool_remove_cases");
}

int fl_pool_download_case(fl_ctx* ctx, fl_pool* P, int32_t id, int32_t* x, int32_t* y, int32_t* z, uint8_t* level,
                          float* f, size_t* nbricks) {
    if (!ctx || !P || !nbricks || id < 0 || id >= (int)P->active.size() || !P->active[id]) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    uint32_t b0 = P->case_begin[id], b1 = P->case_begin[id + 1];
    size_t n = b1 - b0;
    *nbricks = n;
    if (!n) return FL_OK;
    std::vector<uint8_t> lv(n);
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(lv.data(), P->mesh.level + b0, n, cudaMemcpyDeviceToHost, ctx->stream), "dl");
    if (x) FL_TRY_CUDA(ctx, cudaMemcpyAsync(x, P->mesh.x + b0, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "dl");
    if (y) FL_TRY_CUDA(ctx, cudaMemcpyAsync(y, P->mesh.y + b0, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "dl");
    if (z) FL_TRY_CUDA(ctx, cudaMemcpyAsync(z, P->mesh.z + b0, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "dl");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "dl");
    if (level) std::memcpy(level, lv.data(), n);
    if (f) {
        for (int q = 0; q < Q; ++q) {
            size_t b = 0;
            while (b < n) {
                int par = P->parity[lv[b]];
                size_t e = b + 1;
                while (e < n && P->parity[lv[e]] == par) ++e;
                FL_TRY_CUDA(ctx, cudaMemcpyAsync(f + ((size_t)q * n + b) * 512,
                                                 P->f[par] + ((size_t)q * P->cap + b0 + b) * 512, (e - b) * 512 * 4,
                                                 cudaMemcpyDeviceToHost, ctx->stream), "dl f");
                b = e;
            }
        }
        FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "dl");
    }
    return FL_OK;
}

int fl_pool_populations_field(fl_ctx* ctx, fl_pool* P, const char* name, uint64_t* handle) {
    if (!ctx || !P || !name || !handle) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    // Gather the current populations into buffer A: a level whose parity is odd
    // (between level-0 steps only level 0 can be) has them in B; copying them
    // makes both buffers current for it, so its next step reads A consistently.
    for (int l = 0; l <= P->maxL && l < 16; ++l) {
        if (!P->parity[l]) continue;
        const uint32_t b0 = P->lvl_off[l], cnt = P->lvl_off[l + 1] - b0;
        if (cnt) {
            k_copy_bricks<<<fl_blocks((size_t)cnt * Q * 128, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
                P->f[1], P->f[0], P->cap, P->list + b0, cnt);
            FL_CHECK_LAUNCH(ctx, "k_copy_bricks");
        }
        P->parity[l] = 0;
    }
    // writes through the view are invisible to the pool: from here on the conservation sums are
    // always recomputed from the stored state (k_brick_sums)
    P->field_exported = true;
    if (P->sums_enabled) {
        P->sums_enabled = false;
        drop_graph(P);
    }
    P->sums_fresh = false;
    fl_field_desc d;
    if (fl_field_make(name, 0, Q, 1, 0, 0, &d) != FL_OK)
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_pool_populations_field: bad field name");
    int rc = fl_soa_bind_external(ctx, &d, P->mesh.num_cells * 512, P->cap * 512 * sizeof(float), P->f[0], handle);
    if (rc) return rc;
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "fl_pool_populations_field");
    return FL_OK;
}

int fl_pool_set_options(fl_ctx* ctx, fl_pool* P, int use_graphs, int grid_mult) {
    if (!ctx || !P) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    P->graphs = use_graphs;
    if (grid_mult > 0) P->grid_mult = grid_mult;
    drop_graph(P);
    return FL_OK;
}

int fl_pool_set_staging(fl_ctx* ctx, fl_pool* P, int mode) {
    if (!ctx || !P || mode < 0 || mode > 2) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    if (mode) {
        // above the default 48 KB of dynamic shared memory per block
        FL_TRY_CUDA(ctx, cudaFuncSetAttribute(k_collide_staged<true, true, false>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stage_bytes(true, true)),
                    "staged kernel shared memory");
        FL_TRY_CUDA(ctx, cudaFuncSetAttribute(k_collide_staged<true, true, true>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stage_bytes(true, true)),
                    "staged kernel shared memory");
    }
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "fl_pool_set_staging");
    P->staging = mode;
    drop_graph(P);
    return FL_OK;
}

int fl_pool_set_step_sums(fl_ctx* ctx, fl_pool* P, int on) {
    if (!ctx || !P) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    const bool want = on != 0 && !P->field_exported;
    if (want != P->sums_enabled) {
        P->sums_enabled = want;
        drop_graph(P);  // the captured steps launch other kernels
    }
    return FL_OK;
}

int fl_pool_set_class_streams(fl_ctx* ctx, fl_pool* P, int streams) {
    if (!ctx || !P || streams < 1 || streams > 2) return FL_E_INVALID_ARG;
    FL_POOL_USABLE(ctx, P);
    cudaStreamSynchronize(ctx->stream);
    P->streams = streams;
    drop_graph(P);
    return FL_OK;
}

}  // extern "C"
