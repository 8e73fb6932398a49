// amr.cu — octree regrid on the GPU: 2:1 balance, split, merge and the
// rebuild into key order, fully device-resident.
//
// Replaces AdaptationEngine::adapt (src/adaptation/AdaptationEngine.cpp:37-102),
// BalanceEnforcer::enforce (src/adaptation/BalanceEnforcer.cpp:145-263),
// SplitEngine::split (src/adaptation/SplitEngine.cpp:95-267),
// MergeEngine::merge (src/adaptation/MergeEngine.cpp:140-334) and the GPU
// rebuild (AdaptationEngine.cpp:417-656).  The reference moves every
// intermediate result through the host (about a dozen blocking transfers per
// call); here the only host reads are two words of the point locator (the
// deepest level, whether the cells are in key order), the balance counters
// (one per iteration) and the output cell count.  Point location goes through
// the sorted locator of hash.cuh (the hash table only serves FACE6's
// shadow-level probes), and the new cells are emitted directly in key order,
// so no sort runs after the split/merge.  Semantics (the oracle's):
//  * balance FACE6 = the reference kernels (shadow levels, six face probes at
//    anchor-1 / anchor+size, found at the cell whose shadow level matches,
//    violation if found level > shadow + 1, at most max_balance_iterations);
//    FULL26 = every leaf probes its 26 neighbours at its own size and forces
//    a leaf two or more target levels coarser to refine, to a fixed point;
//  * split: flag > 0, FLUID, level < max (split_cells.cl:31-33), children
//    (p << 1) | bit with bit 0 = x, 1 = y, 2 = z (split_cells.cl:87-93);
//  * merge: first siblings (all coordinates even) with flag -1, FLUID, whose
//    eight siblings are leaves with flag -1, FLUID at the same level
//    (merge_cells.cl:11-106), above min_level, numbered by first-sibling index;
//    in FULL26 mode also no touching leaf outside the group may end above it;
//  * rebuild: survivors + children (fields copied from the parent) + parents
//    (children 0..7 summed in order, x0.125 for the arithmetic rule), sorted by
//    the cell key, flags reset to 0 (the CPU rebuild, AdaptationEngine.cpp:104-276).
#include "common.cuh"
#include "amr.cuh"
#include "hash.cuh"
#include "keys.cuh"
#include "scan.cuh"

#include <vector>

namespace {

constexpr int kT = 256;

struct KeyTables {
    uint8_t t1[96];
    uint16_t t3[12 * 512];
};

__device__ __forceinline__ bool fold3(int64_t* p, const fl_domain_dev::Case& d, int A) {
    for (int a = 0; a < 3; ++a) {
        int64_t ext = (int64_t)d.ext[a] << A;
        if (p[a] < 0 || p[a] >= ext) {
            if (!d.periodic[a]) return false;
            p[a] = ((p[a] % ext) + ext) % ext;
        }
    }
    return true;
}

__device__ __forceinline__ bool fold3_32(int32_t* p, const fl_domain_dev::Case& d, int A) {
    bool in = true;
    for (int a = 0; a < 3; ++a) in = in && fl_fold32(p[a], d.ext[a] << A, d.periodic[a]);
    return in;
}

// Shadow level = the level a cell will have.  FACE6 follows the reference
// (level + (flag > 0), update_shadow_levels, BalanceEnforcer.cpp:53-62; the
// first round starts from the levels); FULL26 counts a flag only where the
// cell will split (fluid, below the maximum level), so a flagged cell at the
// maximum level does not push its neighbours.
__device__ __forceinline__ uint8_t shadow_of(const fl_mesh_dev& m, size_t i, int mode, int max_level) {
    const bool up = mode == 1 ? (m.flags[i] > 0 && m.state[i] == 0 && m.level[i] < max_level) : m.flags[i] > 0;
    return (uint8_t)(m.level[i] + (up ? 1 : 0));
}

// Shadow levels; lowest[0] / lowest[1] (when given) receive their minimum and
// maximum; refining (when given) a byte per leaf, set where the leaf will split.
__global__ void k_shadow(fl_mesh_dev m, int mode, int max_level, uint8_t* __restrict__ shadow,
                         uint32_t* __restrict__ lowest, uint8_t* __restrict__ refining) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    unsigned lo = 255u, hi = 0u;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.n; i += stride) {
        const uint8_t v = mode == 0 ? m.level[i] : shadow_of(m, i, mode, max_level);
        shadow[i] = v;
        if (refining) refining[i] = v > m.level[i] ? 1 : 0;
        lo = min(lo, (unsigned)v);
        hi = max(hi, (unsigned)v);
    }
    lo = __reduce_min_sync(0xFFFFFFFFu, lo);
    hi = __reduce_max_sync(0xFFFFFFFFu, hi);
    if (lowest && (threadIdx.x & 31) == 0) {
        atomicMin(lowest, lo);
        atomicMax(lowest + 1, hi);
    }
}

__global__ void k_shadow_update(fl_mesh_dev m, int mode, int max_level, uint8_t* __restrict__ shadow,
                                uint32_t* __restrict__ lowest) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    unsigned lo = 255u, hi = 0u;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.n; i += stride) {
        const uint8_t v = shadow_of(m, i, mode, max_level);
        shadow[i] = v;
        lo = min(lo, (unsigned)v);
        hi = max(hi, (unsigned)v);
    }
    lo = __reduce_min_sync(0xFFFFFFFFu, lo);
    hi = __reduce_max_sync(0xFFFFFFFFu, hi);
    if (lowest && (threadIdx.x & 31) == 0) {
        atomicMin(lowest, lo);
        atomicMax(lowest + 1, hi);
    }
}

// detect_balance_violations (balance_enforce.cl:57-147), exact lookups.
__global__ void __launch_bounds__(kT) k_detect_face6(fl_mesh_dev m, fl_domain_dev dom, const uint64_t* __restrict__ tk,
                                                     const uint32_t* __restrict__ tv, int lg,
                                                     const uint8_t* __restrict__ shadow, uint8_t* __restrict__ viol,
                                                     uint32_t* __restrict__ count) {
    __shared__ KeyTables T;
    fl_keys_fill_tables(T.t1, T.t3, false);
    __syncthreads();
    size_t stride = (size_t)gridDim.x * blockDim.x;
    uint32_t local = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.n; i += stride) {
        viol[i] = 0;
        if (m.state[i] != 0) continue;
        uint16_t cs = m.case_id ? m.case_id[i] : 0;
        const fl_domain_dev::Case& d = dom.c[m.case_id ? cs : 0];
        int sl = shadow[i];
        int sh = dom.anchor_level - m.level[i];
        int64_t anc[3] = {(int64_t)m.x[i] << sh, (int64_t)m.y[i] << sh, (int64_t)m.z[i] << sh};
        int ex = dom.anchor_level - sl;
        int64_t ss = ex > 0 ? ((int64_t)1 << ex) : 1;
        for (int f = 0; f < 6; ++f) {
            int64_t p[3] = {anc[0], anc[1], anc[2]};
            p[f >> 1] += (f & 1) ? ss : -1;
            if (!fold3(p, d, dom.anchor_level)) continue;
            uint32_t r = fl_locate(T.t1, T.t3, tk, tv, lg, shadow, dom, cs, m.case_id != nullptr, p, sl);
            if (r == FL_INVALID_INDEX) continue;
            if ((int)shadow[r] > sl + 1) { viol[i] = 1; ++local; break; }
        }
    }
    if (local) atomicAdd(count, local);
}

// Every leaf probes, through the sorted locator, its neighbour points at its
// own size in the 19 directions that leave its parent cell (32 leaves x 19
// directions per block); a leaf found two or more shadow levels coarser is a
// violation.  The 7 directions that stay inside the parent (towards the
// leaf's siblings' places) cannot find one: a leaf there coarser than this
// one would contain the parent and so overlap this leaf.  A leaf less than
// two shadow levels above the mesh's lowest (lowest[0]) cannot find one either
// and does not probe; with the highest (lowest[1]) below lowest + 2 no block
// probes.  list (with its length at *list_n) restricts the probing leaves, in
// any order: violations and counts do not depend on it.
constexpr int kDetectThreads = 32 * 19;
__global__ void __launch_bounds__(kDetectThreads, 3) k_detect_full26(fl_mesh_dev m, fl_domain_dev dom, fl_locator L,
                                                                     const uint8_t* __restrict__ shadow,
                                                                     const uint32_t* __restrict__ lowest,
                                                                     const uint32_t* __restrict__ list,
                                                                     const uint32_t* __restrict__ list_n,
                                                                     uint8_t* __restrict__ nxt,
                                                                     uint8_t* __restrict__ viol,
                                                                     uint32_t* __restrict__ count) {
    __shared__ uint8_t t1[96];
    __shared__ uint16_t t3c[12 * 512];
    __shared__ uint8_t s_dir[8][19];  // per child position (x&1 | (y&1)<<1 | (z&1)<<2): outward directions
    fl_keys_fill_tables_cat(t1, t3c);
    if (threadIdx.x < 8) {
        const int c = threadIdx.x;
        int e = 0;
        for (int kk = 0; kk < 27; ++kk) {
            if (kk == 13) continue;
            const int d[3] = {kk % 3 - 1, (kk / 3) % 3 - 1, kk / 9 - 1};
            bool out = false;
            for (int a = 0; a < 3; ++a) out |= d[a] == (((c >> a) & 1) ? 1 : -1);
            if (out) s_dir[c][e++] = (uint8_t)kk;
        }
    }
    __syncthreads();
    const fl_probe P = fl_probe_make(t1, t3c, L, dom);
    const int cl = threadIdx.x / 19, k = threadIdx.x - cl * 19;
    const int low = (int)lowest[0];
    if ((int)lowest[1] < low + 2) return;  // no leaf anywhere is two levels above another
    const size_t n = list ? (size_t)*list_n : m.n;
    uint32_t local = 0;
    for (size_t base = (size_t)blockIdx.x * 32; base < n; base += (size_t)gridDim.x * 32) {
        const size_t j = base + cl;
        if (j >= n) continue;
        const size_t i = list ? (size_t)list[j] : j;
        const int si = shadow[i];
        if (si < low + 2) continue;
        const uint16_t cs = m.case_id ? m.case_id[i] : 0;
        const fl_domain_dev::Case& d = dom.c[m.case_id ? cs : 0];
        const int sh = dom.anchor_level - m.level[i];
        const int32_t size = 1 << sh;
        const int32_t cx = m.x[i], cy = m.y[i], cz = m.z[i];
        const int kk = s_dir[(cx & 1) | ((cy & 1) << 1) | ((cz & 1) << 2)][k];
        const int dv[3] = {kk % 3 - 1, (kk / 3) % 3 - 1, kk / 9 - 1};
        int32_t p[3] = {cx << sh, cy << sh, cz << sh};
        for (int a = 0; a < 3; ++a) p[a] += dv[a] < 0 ? -1 : (dv[a] > 0 ? size : 0);
        if (!fold3_32(p, d, dom.anchor_level)) continue;
        const uint32_t r = fl_probe_point(P, m.case_id != nullptr, cs, (uint32_t)p[0], (uint32_t)p[1], (uint32_t)p[2]);
        if (r == FL_INVALID_INDEX) continue;
        if (si >= (int)shadow[r] + 2) {
            viol[r] = 1;
            if (nxt) nxt[i] = 1;
            ++local;
        }
    }
    if (local) atomicAdd(count, local);
}

// The leaves whose byte is set, into list (in any order; their number added
// to *list_n), and the bytes cleared.
__global__ void k_compact_active(uint8_t* __restrict__ flags, size_t n, uint32_t* __restrict__ list,
                                 uint32_t* __restrict__ list_n) {
    const int lane = threadIdx.x & 31;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x - lane; i0 < n; i0 += stride) {
        const size_t i = i0 + lane;
        const bool on = i < n && flags[i];
        const unsigned bal = __ballot_sync(0xFFFFFFFFu, on);
        if (!bal) continue;
        uint32_t first = 0;
        if (lane == 0) first = atomicAdd(list_n, (uint32_t)__popc(bal));
        first = __shfl_sync(0xFFFFFFFFu, first, 0);
        if (on) {
            flags[i] = 0;
            list[first + __popc(bal & ((1u << lane) - 1u))] = (uint32_t)i;
        }
    }
}

// mark_cascading_refinement (balance_enforce.cl:150-172).
__global__ void k_mark(fl_mesh_dev m, int32_t* __restrict__ flags, const uint8_t* __restrict__ viol, int max_level,
                       uint8_t* __restrict__ nxt, uint32_t* __restrict__ count) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    uint32_t local = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.n; i += stride) {
        if (!viol[i] || m.state[i] != 0 || m.level[i] >= max_level) continue;
        if (flags[i] <= 0) {
            flags[i] = 1;
            if (nxt) nxt[i] = 1;
            ++local;
        }
    }
    if (local) atomicAdd(count, local);
}

__global__ void k_clear_u8(uint8_t* p, size_t n) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) p[i] = 0;
}

// A merge candidate: a FLUID first sibling (all coordinates even) flagged -1
// above min_level.
__device__ __forceinline__ bool merge_candidate(const fl_mesh_dev& m, size_t i, int min_level) {
    return m.flags[i] == -1 && m.state[i] == 0 && !((m.x[i] | m.y[i] | m.z[i]) & 1) && m.level[i] > min_level;
}

// Lane c < 8 of a warp: sibling c of candidate i (the leaf holding its anchor
// point, if that leaf has the octet's level), FL_INVALID_INDEX otherwise;
// `ok` tells whether it is a mergeable member (flag -1, FLUID).
__device__ __forceinline__ uint32_t sibling_of(const fl_probe& P, const fl_mesh_dev& m, const fl_domain_dev& dom,
                                               size_t i, int c, bool* ok) {
    const int l = m.level[i];
    const uint16_t cs = m.case_id ? m.case_id[i] : 0;
    const int sh = dom.anchor_level - l;
    const uint32_t sx = (uint32_t)(m.x[i] | (c & 1)) << sh, sy = (uint32_t)(m.y[i] | ((c >> 1) & 1)) << sh,
                   sz = (uint32_t)(m.z[i] | ((c >> 2) & 1)) << sh;
    uint32_t j = fl_probe_point(P, m.case_id != nullptr, cs, sx, sy, sz);
    if (j != FL_INVALID_INDEX && m.level[j] != l) j = FL_INVALID_INDEX;
    *ok = j != FL_INVALID_INDEX && m.flags[j] == -1 && m.state[j] == 0;
    return j;
}

// The same without a search, for a mesh in key order (the locator's run order
// is the mesh order, L.ids == nullptr): the parent's run holds its children's
// runs, so a complete octet of leaves is 8 consecutive cells, starting h cells
// before the candidate, h = the candidate's Hilbert digit at its level (read
// from its run key).  Lane c takes the c-th of them, in key order; it is a
// member when it is a leaf of the candidate's level under the same parent
// (case, x >> 1, y >> 1, z >> 1).  Eight members <=> the eight children are
// leaves of that level <=> sibling_of finds all eight; `ok` as there.  The
// members come in key order, not by child position (their child bits say
// which is which).
__device__ __forceinline__ uint32_t sibling_in_run(const fl_probe& P, const fl_mesh_dev& m, size_t i, int c, bool* ok) {
    const int l = m.level[i];
    const int h = (int)((__ldg((const unsigned long long*)(P.L.keys + i)) >> (3 * (P.top - l))) & 7u);
    *ok = false;
    if (i < (size_t)h) return FL_INVALID_INDEX;
    const size_t j = i - h + c;
    if (j >= m.n || m.level[j] != l || (m.x[j] >> 1) != (m.x[i] >> 1) || (m.y[j] >> 1) != (m.y[i] >> 1) ||
        (m.z[j] >> 1) != (m.z[i] >> 1) || (m.case_id && m.case_id[j] != m.case_id[i]))
        return FL_INVALID_INDEX;
    *ok = m.flags[j] == -1 && m.state[j] == 0;
    return (uint32_t)j;
}

// Leaders: a warp screens 32 cells, a lane each, then checks the chunk's
// candidates four at a time -- lanes 8s .. 8s + 7 locate the eight siblings of
// the s-th (all must be mergeable leaves of its level) -- and, for the FULL26
// merge condition, spreads the probes around each surviving octet over the
// lanes, the candidates' probes one after another: no leaf touching an octet
// from outside may end above its level.  The reference's probes are each
// child's 26 neighbour points at the child's size; per axis they take five
// coordinates -- the last fine point below the octet, the first and last of
// its lower cell, the first of its upper cell, the first point above -- and
// the 98 combinations with at least one outside coordinate are the distinct
// probes outside the octet.  They fall into the 56 cells of the children's
// size around the octet (4 per axis: below, lower, upper, above).  One point
// per cell decides the cell whenever it finds a leaf: a leaf of the octet's
// level or coarser holding it holds the whole cell, and a finer one is above
// the octet's level wherever in the cell it lies; only when that point is
// not covered (a mesh that does not fill its domain) are the cell's other
// probe points tried.  Same answer as the 98 probes, from 56 on a filled mesh.
__global__ void __launch_bounds__(kT) k_leaders(fl_mesh_dev m, fl_domain_dev dom, fl_locator L, int min_level,
                                                int check26, const uint8_t* __restrict__ shadow,
                                                uint32_t* __restrict__ is_leader) {
    __shared__ uint8_t t1[96];
    __shared__ uint16_t t3c[12 * 512];
    __shared__ uint8_t surf[56];  // the outside cells k = ux + 4 uy + 16 uz of the 4^3 grid of child-sized cells
    fl_keys_fill_tables_cat(t1, t3c);
    if (threadIdx.x == 0) {
        int e = 0;
        for (int k = 0; k < 64; ++k) {
            const int ux = k & 3, uy = (k >> 2) & 3, uz = k >> 4;
            if (ux == 0 || ux == 3 || uy == 0 || uy == 3 || uz == 0 || uz == 3) surf[e++] = (uint8_t)k;
        }
    }
    __syncthreads();
    const fl_probe P = fl_probe_make(t1, t3c, L, dom);
    const int lane = threadIdx.x & 31, grp = lane >> 3;
    const size_t warps = (size_t)gridDim.x * (blockDim.x >> 5);
    for (size_t base = ((size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < m.n;
         base += warps * 32) {
        const size_t mine = base + lane;
        const bool cand = mine < m.n && merge_candidate(m, mine, min_level);
        if (mine < m.n && !cand) is_leader[mine] = 0u;
        unsigned cm = __ballot_sync(0xFFFFFFFFu, cand);
        while (cm) {
            const int n4 = min(__popc(cm), 4);  // candidates of this round
            unsigned pick = cm;
            for (int s = 0; s < grp && pick; ++s) pick &= pick - 1;
            for (int s = 0; s < 4 && cm; ++s) cm &= cm - 1;
            const bool have = grp < n4;
            const size_t i = have ? base + (__ffs(pick) - 1) : 0;
            bool ok = true;
            uint32_t j = FL_INVALID_INDEX;
            if (have) j = P.L.ids ? sibling_of(P, m, dom, i, lane & 7, &ok) : sibling_in_run(P, m, i, lane & 7, &ok);
            const unsigned okm = __ballot_sync(0xFFFFFFFFu, ok);
            unsigned lead4 = 0;  // bit s: candidate s has eight mergeable siblings
            for (int s = 0; s < n4; ++s)
                if (((okm >> (8 * s)) & 0xFFu) == 0xFFu) lead4 |= 1u << s;
            unsigned bad4 = 0;  // bit s: a probe of candidate s found a leaf ending above its level
            if (lead4 && check26) {
                // per-candidate values, held by every lane of its group
                const uint16_t cs_m = have && m.case_id ? m.case_id[i] : 0;
                const int l_m = have ? m.level[i] : 0;
                const int sh_m = dom.anchor_level - l_m;
                const int32_t b_m[3] = {have ? m.x[i] << sh_m : 0, have ? m.y[i] << sh_m : 0,
                                        have ? m.z[i] << sh_m : 0};
                const int nc = __popc(lead4);
                for (int e0 = 0; e0 < nc * 56; e0 += 32) {
                    const int e = e0 + lane;
                    const bool act = e < nc * 56;
                    int t = act ? e / 56 : 0;  // t-th surviving candidate ...
                    unsigned lm = lead4;
                    for (int k = 0; k < t; ++k) lm &= lm - 1;
                    const int s = __ffs(lm) - 1;  // ... is candidate s
                    const int src = 8 * s;
                    const uint16_t cs = (uint16_t)__shfl_sync(0xFFFFFFFFu, (int)cs_m, src);
                    const int l = __shfl_sync(0xFFFFFFFFu, l_m, src);
                    const int32_t b3[3] = {__shfl_sync(0xFFFFFFFFu, b_m[0], src), __shfl_sync(0xFFFFFFFFu, b_m[1], src),
                                           __shfl_sync(0xFFFFFFFFu, b_m[2], src)};
                    uint32_t mem[8];
                    for (int c = 0; c < 8; ++c) mem[c] = __shfl_sync(0xFFFFFFFFu, j, src + c);
                    if (!act) continue;
                    const fl_domain_dev::Case& d = dom.c[m.case_id ? cs : 0];
                    const int32_t size = 1 << (dom.anchor_level - l);
                    const int k = surf[e - t * 56];
                    const int uc[3] = {k & 3, (k >> 2) & 3, k >> 4};
                    // the cell's probe point with alt set on the axes where the cell is the lower child's
                    // span: its last point there instead of its first
                    auto point = [&](int alt, int32_t (&p)[3]) {
                        for (int a = 0; a < 3; ++a) {
                            const int u = uc[a];
                            p[a] = u == 0 ? b3[a] - 1
                                          : (u == 1 ? b3[a] + (((alt >> a) & 1) ? size - 1 : 0)
                                                    : (u == 2 ? b3[a] + size : b3[a] + 2 * size));
                        }
                        return fold3_32(p, d, dom.anchor_level);
                    };
                    auto found = [&](uint32_t r) {
                        bool inside = false;  // only on a periodic axis of one octet's extent
                        for (int q = 0; q < 8; ++q) inside |= (mem[q] == r);
                        if (!inside && (int)shadow[r] > l) bad4 |= 1u << s;
                    };
                    int32_t p[3];
                    if (!point(0, p)) continue;
                    const uint32_t r =
                        fl_probe_point(P, m.case_id != nullptr, cs, (uint32_t)p[0], (uint32_t)p[1], (uint32_t)p[2]);
                    if (r != FL_INVALID_INDEX) {
                        found(r);
                        continue;
                    }
                    const int multi = (uc[0] == 1) | ((uc[1] == 1) << 1) | ((uc[2] == 1) << 2);
                    for (int v = multi; v; v = (v - 1) & multi) {  // the cell's other probe points
                        if (!point(v, p)) continue;
                        const uint32_t r2 =
                            fl_probe_point(P, m.case_id != nullptr, cs, (uint32_t)p[0], (uint32_t)p[1], (uint32_t)p[2]);
                        if (r2 != FL_INVALID_INDEX) found(r2);
                    }
                }
                bad4 = __reduce_or_sync(0xFFFFFFFFu, bad4);
            }
            if (have && (lane & 7) == 0) is_leader[i] = ((lead4 >> grp) & 1u) && !((bad4 >> grp) & 1u) ? 1u : 0u;
        }
    }
}

// Members of each leader's group: a warp locates the siblings of four leaders
// at a time (lane 8s + c: sibling c of the s-th).
__global__ void __launch_bounds__(kT) k_members(fl_mesh_dev m, fl_domain_dev dom, fl_locator L,
                                                const uint32_t* __restrict__ is_leader,
                                                const uint32_t* __restrict__ gid, uint32_t* __restrict__ members,
                                                uint32_t* __restrict__ group_of) {
    __shared__ uint8_t t1[96];
    __shared__ uint16_t t3c[12 * 512];
    fl_keys_fill_tables_cat(t1, t3c);
    __syncthreads();
    const fl_probe P = fl_probe_make(t1, t3c, L, dom);
    const int lane = threadIdx.x & 31;
    const size_t warps = (size_t)gridDim.x * (blockDim.x >> 5);
    for (size_t base = ((size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < m.n;
         base += warps * 32) {
        const size_t mine = base + lane;
        const bool lead = mine < m.n && is_leader[mine];
        unsigned cm = __ballot_sync(0xFFFFFFFFu, lead);
        while (cm) {
            // up to four leaders per round: lanes 8s .. 8s + 7 take the s-th next one
            unsigned pick = cm;
            for (int s = 0; s < (lane >> 3) && pick; ++s) pick &= pick - 1;
            for (int s = 0; s < 4 && cm; ++s) cm &= cm - 1;
            if (pick) {
                const size_t i = base + (__ffs(pick) - 1);
                bool ok;
                uint32_t j;
                int c = lane & 7;
                if (P.L.ids) {
                    j = sibling_of(P, m, dom, i, c, &ok);
                } else {  // the octet's c-th cell in key order: file it under its child position
                    j = sibling_in_run(P, m, i, c, &ok);
                    c = (m.x[j] & 1) | ((m.y[j] & 1) << 1) | ((m.z[j] & 1) << 2);
                }
                const uint32_t g = gid[i];
                members[(size_t)g * 8 + c] = j;
                group_of[j] = g;
            }
        }
    }
}

// Output count per old cell, in visiting order (order[t] = the cell visited
// t-th, or t when order is null).
__global__ void k_counts(fl_mesh_dev m, int max_level, const uint32_t* __restrict__ order,
                         const uint32_t* __restrict__ is_leader, const uint32_t* __restrict__ group_of,
                         uint32_t* __restrict__ cnt) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < m.n; t += stride) {
        const size_t i = order ? order[t] : t;
        bool split = m.flags[i] > 0 && m.state[i] == 0 && m.level[i] < max_level;
        uint32_t c;
        if (split) c = 8;
        else if (group_of[i] != FL_INVALID_INDEX) c = is_leader[i] ? 1u : 0u;
        else c = 1;
        cnt[t] = c;
    }
}

// The new cells in key order, written straight into the output mesh with no
// sort: the old cells are visited in key order (the locator's order) and every
// new cell lies inside the run of the old cell that makes it -- a survivor in
// its own run, the children of a split cell in its run, placed by their
// Hilbert digit under the cell's curve state, a merged group's parent at its
// leader's place (the eight members' runs are consecutive and the other seven
// emit nothing).  Fields (C per cell, AoS) follow the reference: children copy
// their parent (prolongation), a parent sums its children 0..7 in order, x0.125
// for the arithmetic rule (restriction).
__global__ void __launch_bounds__(kT) k_emit(fl_mesh_dev m, fl_domain_dev dom, int max_level,
                                             const uint32_t* __restrict__ order, const uint32_t* __restrict__ off,
                                             const uint32_t* __restrict__ is_leader,
                                             const uint32_t* __restrict__ group_of,
                                             const uint32_t* __restrict__ members, fl_mesh_out out,
                                             uint32_t* __restrict__ osrc, uint8_t* __restrict__ okind,
                                             const float* __restrict__ fin, float* __restrict__ fout, uint32_t C,
                                             int rule) {
    __shared__ uint8_t t1[96];
    __shared__ uint16_t t3c[12 * 512];
    __shared__ uint32_t stage[kT / 32][256];  // one column of a warp's (at most 256) new cells
    fl_keys_fill_tables_cat(t1, t3c);
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t* S = stage[threadIdx.x >> 5];
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t rounds = (m.n + stride - 1) / stride;  // whole warps stay in the loop
    for (size_t rr = 0; rr < rounds; ++rr) {
        const size_t t = rr * stride + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
        // kind: 0 nothing (a merged non-leader or past the end), 1 split, 2 group leader, 3 kept
        int kind = 0, l = 0;
        size_t i = 0;
        uint32_t o = 0, cnt = 0, g = FL_INVALID_INDEX;
        unsigned st = 0;
        if (t < m.n) {
            i = order ? order[t] : t;
            o = off[t];
            l = m.level[i];
            if (m.flags[i] > 0 && m.state[i] == 0 && l < max_level) {
                kind = 1;
                cnt = 8;
                st = fl_hilbert_state_cat(t1, t3c, (uint32_t)m.x[i], (uint32_t)m.y[i], (uint32_t)m.z[i],
                                          dom.depth - dom.anchor_level + l);
            } else if ((g = group_of[i]) != FL_INVALID_INDEX) {
                if (is_leader[i]) { kind = 2; cnt = 1; }
            } else {
                kind = 3;
                cnt = 1;
            }
        }
        // a warp's new cells are one contiguous range (off is the exclusive scan of
        // the counts in visiting order, and lane 0 visits first): each column is
        // staged in shared memory, then stored coalesced
        const uint32_t total = __reduce_add_sync(0xFFFFFFFFu, cnt);
        if (total == 0) continue;
        const uint32_t base = __shfl_sync(0xFFFFFFFFu, o, 0), rel = o - base;
        const int32_t mx = kind ? m.x[i] : 0, my = kind ? m.y[i] : 0, mz = kind ? m.z[i] : 0;
        auto stage_col = [&](auto value_of) {
            if (kind == 1) {
                for (int c = 0; c < 8; ++c) S[rel + (t1[st * 8 + c] & 7u)] = value_of(c);
            } else if (kind >= 2) {
                S[rel] = value_of(-1);
            }
            __syncwarp();
        };
        auto axis = [&](int32_t v, int bit) {
            return [=](int c) -> uint32_t {
                return (uint32_t)(c >= 0 ? (v << 1) | ((c >> bit) & 1) : (kind == 2 ? v >> 1 : v));
            };
        };
        stage_col(axis(mx, 0));
        for (uint32_t e = lane; e < total; e += 32u) out.x[base + e] = (int32_t)S[e];
        __syncwarp();
        stage_col(axis(my, 1));
        for (uint32_t e = lane; e < total; e += 32u) out.y[base + e] = (int32_t)S[e];
        __syncwarp();
        stage_col(axis(mz, 2));
        for (uint32_t e = lane; e < total; e += 32u) out.z[base + e] = (int32_t)S[e];
        __syncwarp();
        stage_col([&](int c) -> uint32_t { return (uint32_t)(c >= 0 ? l + 1 : (kind == 2 ? l - 1 : l)); });
        for (uint32_t e = lane; e < total; e += 32u) out.level[base + e] = (uint8_t)S[e];
        __syncwarp();
        const uint32_t mstate = kind ? m.state[i] : 0u, mmat = kind ? m.material[i] : 0u;
        stage_col([&](int) -> uint32_t { return mstate; });
        for (uint32_t e = lane; e < total; e += 32u) out.state[base + e] = (uint8_t)S[e];
        __syncwarp();
        stage_col([&](int) -> uint32_t { return mmat; });
        for (uint32_t e = lane; e < total; e += 32u) out.material[base + e] = S[e];
        __syncwarp();
        for (uint32_t e = lane; e < total; e += 32u) out.flags[base + e] = 0;
        if (out.case_id) {
            const uint32_t cs = kind && m.case_id ? m.case_id[i] : 0u;
            stage_col([&](int) -> uint32_t { return cs; });
            for (uint32_t e = lane; e < total; e += 32u) out.case_id[base + e] = (uint16_t)S[e];
            __syncwarp();
        }
        if (osrc) {
            stage_col([&](int) -> uint32_t { return kind == 2 ? g : (uint32_t)i; });
            for (uint32_t e = lane; e < total; e += 32u) osrc[base + e] = S[e];
            __syncwarp();
        }
        if (okind) {
            stage_col([&](int c) -> uint32_t { return c >= 0 ? (uint32_t)c : (kind == 2 ? 9u : 8u); });
            for (uint32_t e = lane; e < total; e += 32u) okind[base + e] = (uint8_t)S[e];
            __syncwarp();
        }
        if (fin && C && kind) {  // fields: copied from the source cell, or the mean of a group's members
            auto copy_row = [&](uint32_t j) {
                const float* sp = fin + i * C;
                float* fo = fout + (size_t)j * C;
                for (uint32_t c = 0; c < C; ++c) fo[c] = sp[c];
            };
            if (kind == 1) {
                for (int c = 0; c < 8; ++c) copy_row(o + (t1[st * 8 + c] & 7u));
            } else if (kind == 3) {
                copy_row(o);
            } else {
                const uint32_t* mem = members + (size_t)g * 8;
                float* fo = fout + (size_t)o * C;
                for (uint32_t c = 0; c < C; ++c) {
                    float sum = 0.0f;
                    for (int q = 0; q < 8; ++q) sum = __fadd_rn(sum, fin[(size_t)mem[q] * C + c]);
                    fo[c] = rule == 1 ? sum : __fmul_rn(sum, 0.125f);
                }
            }
        }
    }
}

// SplitEngine::split pieces (split_cells.cl:15-132): predicate, then children
// at the scanned block start, fields copied from the parent.
__global__ void k_split_pred(fl_mesh_dev m, int max_level, uint32_t* __restrict__ pred) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.n; i += stride)
        pred[i] = (m.flags[i] > 0 && m.state[i] == 0 && m.level[i] < max_level) ? 1u : 0u;
}

__global__ void k_split_children(fl_mesh_dev m, const uint32_t* __restrict__ pred, const uint32_t* __restrict__ off,
                                 fl_mesh_out ch, uint32_t* __restrict__ p2c, const float* __restrict__ fin,
                                 float* __restrict__ fout, uint32_t C) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.n; i += stride) {
        if (!pred[i]) {
            if (p2c) p2c[i] = FL_INVALID_INDEX;
            continue;
        }
        uint32_t start = off[i] * 8;
        if (p2c) p2c[i] = start;
        for (int c = 0; c < 8; ++c) {
            uint32_t j = start + c;
            ch.x[j] = (m.x[i] << 1) | (c & 1);
            ch.y[j] = (m.y[i] << 1) | ((c >> 1) & 1);
            ch.z[j] = (m.z[i] << 1) | ((c >> 2) & 1);
            ch.level[j] = (uint8_t)(m.level[i] + 1);
            ch.state[j] = m.state[i];
            ch.material[j] = m.material[i];
            ch.flags[j] = 0;
            if (ch.case_id) ch.case_id[j] = m.case_id[i];
            if (fin && fout)
                for (uint32_t k = 0; k < C; ++k) fout[(size_t)j * C + k] = fin[(size_t)i * C + k];
        }
    }
}

// MergeEngine::merge pieces (merge_cells.cl:123-199): group ids by leader
// order, parents from the first sibling, fields restricted in child order.
__global__ void k_merge_parents(fl_mesh_dev m, const uint32_t* __restrict__ members, uint32_t G, fl_mesh_out par,
                                const float* __restrict__ fin, float* __restrict__ fout, uint32_t C, int rule) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x; g < G; g += stride) {
        uint32_t i = members[g * 8];
        par.x[g] = m.x[i] >> 1; par.y[g] = m.y[i] >> 1; par.z[g] = m.z[i] >> 1;
        par.level[g] = (uint8_t)(m.level[i] - 1);
        par.state[g] = m.state[i];
        par.material[g] = m.material[i];
        par.flags[g] = 0;
        if (par.case_id) par.case_id[g] = m.case_id[i];
        if (fin && fout)
            for (uint32_t k = 0; k < C; ++k) {
                float s = 0.0f;
                for (int q = 0; q < 8; ++q) s = __fadd_rn(s, fin[(size_t)members[g * 8 + q] * C + k]);
                fout[(size_t)g * C + k] = rule == 1 ? s : __fmul_rn(s, 0.125f);
            }
    }
}

// Scratch carving helper.
struct Carver {
    char* p;
    template <typename T>
    T* take(size_t n) {
        T* r = (T*)p;
        p += fl_align256(n * sizeof(T));
        return r;
    }
};

}  // namespace

bool fl_domain_config_valid(const fl_adapt_config* cfg) {
    int D = cfg->key_depth ? cfg->key_depth : 21;
    int A = cfg->anchor_level ? cfg->anchor_level : 21;
    if (D < 1 || D > 21 || A < 0 || A > D || cfg->max_refinement_level > A) return false;
    for (int a = 0; a < 3; ++a) {
        int64_t e = cfg->ext[a] > 0 ? cfg->ext[a] : 1;
        if ((e << A) > ((int64_t)1 << D)) return false;
    }
    return true;
}

fl_domain_dev fl_domain_from_config(fl_ctx* ctx, const fl_adapt_config* cfg, void* dev_case_slot) {
    fl_domain_dev d;
    d.depth = cfg->key_depth ? cfg->key_depth : 21;
    d.anchor_level = cfg->anchor_level ? cfg->anchor_level : 21;
    d.max_level = d.anchor_level;
    fl_domain_dev::Case h;
    for (int a = 0; a < 3; ++a) {
        h.ext[a] = cfg->ext[a] > 0 ? cfg->ext[a] : 1;
        h.periodic[a] = cfg->periodic[a];
    }
    cudaMemcpyAsync(dev_case_slot, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream);
    d.c = (const fl_domain_dev::Case*)dev_case_slot;
    return d;
}

// FULL26 balance's probing-leaf state for n leaves: a byte per leaf, then a list of leaf ids.
static size_t fl_balance_act_bytes(size_t n) { return fl_align256(n) + fl_align256(n * 4); }

size_t fl_adapt_scratch_bytes(size_t n, uint64_t cap) {
    size_t b = 0;
    b += fl_align256(n * 8);                 // cell keys (FACE6's hash table)
    b += fl_align256(cap * 16) + fl_align256(cap * 4);  // 16-byte-slot table + win
    b += 2 * fl_align256(n) + fl_balance_act_bytes(n);  // shadow, viol, probing leaves
    b += 4 * fl_align256(n * 4);             // leader, gid, group_of, cnt/off
    b += fl_align256(n * 4);                 // members (n/8 groups * 8)
    b += fl_align256(64);                    // counters
    b += fl_scan_scratch_bytes(n) + fl_align256(fl_locator_scratch_bytes(n)) + 4096;
    return b;
}

// Balance over a mesh with an already-built table (shared by fl_balance_enforce and fl_adapt).
// FULL26 probes from every leaf in the first round only.  A pair (i, r)
// violates when shadow(i) >= shadow(r) + 2, and a round changes shadow levels
// only by raising those of the leaves it marks; so a pair can violate in round
// k + 1 only if i was marked in round k or i already found a violation in
// round k.  Those leaves are the only ones that probe afterwards, which gives
// the same violations, marks and counts.  act (fl_balance_act_bytes(n), or
// nullptr to probe from every leaf each round) holds one byte per leaf, set
// for the next round's probing leaves, then at offset fl_align256(n) the list
// they are gathered into before that round.
// balanced_input: the caller states that no two touching leaves differ by more
// than one level.  A violation needs shadow[i] >= shadow[r] + 2 with shadow[i]
// <= level[i] + 1 and shadow[r] >= level[r] >= level[i] - 1, so in the first
// round only a leaf that will split can find one: only those probe (through the
// list, like the later rounds).
int fl_balance_run(fl_ctx* ctx, fl_mesh_dev md, int32_t* flags, const fl_domain_dev& dom, const uint64_t* tk,
                   const uint32_t* tv, uint64_t cap, const fl_locator* L, int mode, int max_level, int max_iters,
                   uint8_t* shadow, uint8_t* viol, uint8_t* act, uint32_t* counters, fl_balance_result* res,
                   bool balanced_input) {
    fl_balance_result r{};
    if (md.n == 0) { r.converged = 1; if (res) *res = r; return FL_OK; }
    unsigned nb = fl_blocks(md.n, kT, ctx->num_sms * 8);
    int lg = fl_hash_lg(cap);
    uint32_t* lowest = counters + 2;  // lowest and highest shadow level, for FULL26's early outs
    const uint32_t extremes[2] = {0xFFFFFFFFu, 0u};
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(lowest, extremes, 8, cudaMemcpyHostToDevice, ctx->stream), "balance extremes");
    // a balanced input: the first round probes only from the leaves that will split
    const bool first_listed = act && mode == 1 && balanced_input;
    k_shadow<<<nb, kT, 0, ctx->stream>>>(md, mode, max_level, shadow, lowest, first_listed ? act : nullptr);
    FL_CHECK_LAUNCH(ctx, "k_shadow");
    int cap_it = mode == 0 ? max_iters : 4096;
    uint32_t it = 0;
    uint32_t h[2];
    for (; it < (uint32_t)cap_it; ++it) {
        FL_TRY_CUDA(ctx, cudaMemsetAsync(counters, 0, 8, ctx->stream), "balance counters");
        // this round's probing leaves (all of them in the first round) and the next round's
        uint8_t* nxt = (act && mode == 1) ? act : nullptr;
        uint32_t* list = (act && mode == 1 && (it > 0 || first_listed)) ? (uint32_t*)(act + fl_align256(md.n)) : nullptr;
        uint32_t* list_n = counters + 4;  // free until the merge grouping after balance
        if (mode == 0) {
            k_detect_face6<<<nb, kT, 0, ctx->stream>>>(md, dom, tk, tv, lg, shadow, viol, counters);
        } else {
            k_clear_u8<<<nb, kT, 0, ctx->stream>>>(viol, md.n);
            if (list) {
                // this round's probing leaves: those flagged in the last round, or (first round of a
                // balanced input) those that will split; the flags are cleared
                FL_TRY_CUDA(ctx, cudaMemsetAsync(list_n, 0, 4, ctx->stream), "balance list");
                k_compact_active<<<nb, kT, 0, ctx->stream>>>(nxt, md.n, list, list_n);
            } else if (nxt) {
                k_clear_u8<<<nb, kT, 0, ctx->stream>>>(nxt, md.n);
            }
            const unsigned pb = (unsigned)std::min<size_t>((md.n + 31) / 32, (size_t)ctx->num_sms * 3);
            k_detect_full26<<<pb, kDetectThreads, 0, ctx->stream>>>(md, dom, *L, shadow, lowest, list, list_n, nxt,
                                                                    viol, counters);
        }
        FL_CHECK_LAUNCH(ctx, "k_detect");
        k_mark<<<nb, kT, 0, ctx->stream>>>(md, flags, viol, max_level, nxt, counters + 1);
        FL_CHECK_LAUNCH(ctx, "k_mark");
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(h, counters, 8, cudaMemcpyDeviceToHost, ctx->stream), "balance read");
        FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "balance sync");
        r.total_violations_detected += h[0];
        if (h[0] == 0) { r.converged = 1; r.iterations = it + 1; break; }
        // k_mark ran after detection regardless; with zero violations it marks nothing
        r.total_cells_marked_for_balance += h[1];
        if (h[1] == 0) { r.converged = 0; r.iterations = it + 1; break; }
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(lowest, extremes, 8, cudaMemcpyHostToDevice, ctx->stream),
                    "balance extremes");
        k_shadow_update<<<nb, kT, 0, ctx->stream>>>(md, mode, max_level, shadow, lowest);
        FL_CHECK_LAUNCH(ctx, "k_shadow_update");
    }
    if (it == (uint32_t)cap_it) { r.converged = 0; r.iterations = it; }
    if (res) *res = r;
    return FL_OK;
}

// Scratch layout of one regrid (carved identically by both phases).
struct AdaptWork {
    uint64_t cap;
    uint64_t* keys; uint64_t* tk; uint32_t* tv; uint32_t* win;
    uint8_t* shadow; uint8_t* viol; uint8_t* act;
    uint32_t* leader; uint32_t* gid; uint32_t* group_of; uint32_t* cnt; uint32_t* members; uint32_t* counters;
    void* scan_scratch;
    void* locator;  // fl_locator_build scratch
};

static AdaptWork carve_adapt(void* scratch, size_t n, bool with_case) {
    AdaptWork w;
    w.cap = fl_table_capacity(n);
    Carver cv{(char*)scratch};
    w.keys = cv.take<uint64_t>(n);
    w.tk = cv.take<uint64_t>(2 * w.cap);
    w.tv = nullptr;  // 16-byte slots
    w.win = cv.take<uint32_t>(w.cap);
    w.shadow = cv.take<uint8_t>(n);
    w.viol = cv.take<uint8_t>(n);
    w.act = cv.take<uint8_t>(fl_balance_act_bytes(n));
    w.leader = cv.take<uint32_t>(n);
    w.gid = cv.take<uint32_t>(n);
    w.group_of = cv.take<uint32_t>(n);
    w.cnt = cv.take<uint32_t>(n);
    w.members = cv.take<uint32_t>(n + 8);
    w.counters = cv.take<uint32_t>(16);
    w.scan_scratch = cv.take<char>(fl_scan_scratch_bytes(n));
    w.locator = cv.take<char>(fl_locator_scratch_bytes(n));
    return w;
}

__global__ void k_count_kinds(fl_mesh_dev m, int max_level, const uint32_t* __restrict__ group_of,
                              uint32_t* __restrict__ counters) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    uint32_t ns = 0, nv = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.n; i += stride) {
        bool split = m.flags[i] > 0 && m.state[i] == 0 && m.level[i] < max_level;
        if (split) ++ns;
        else if (group_of[i] == FL_INVALID_INDEX) ++nv;
    }
    if (ns) atomicAdd(counters + 4, ns);
    if (nv) atomicAdd(counters + 5, nv);
}

// Phase 1: balance, classify, emit the unsorted new cell list; returns its size.
int fl_adapt_prepare(fl_ctx* ctx, const fl_mesh* mesh, const fl_adapt_config* cfg, const fl_domain_dev& dom,
                     bool run_balance, void* scratch, size_t* M_out, fl_adapt_stats* st, int level_bound) {
    size_t n = mesh->num_cells;
    fl_adapt_stats s{};
    *M_out = 0;
    if (n == 0) { if (st) *st = s; return FL_OK; }
    AdaptWork w = carve_adapt(scratch, n, mesh->case_id != nullptr);
    fl_mesh_dev md{mesh->x, mesh->y, mesh->z, mesh->level, mesh->state, mesh->flags, mesh->material,
                   mesh->case_id, n};
    // the sorted locator serves FULL26 detection and merge grouping; the
    // FACE6 detection (shadow-level probes) keeps the hash table
    fl_locator L;
    int rc = fl_locator_build(ctx, md, dom, w.locator, &L, level_bound);
    if (rc) return rc;
    if (run_balance && cfg->balance_mode == 0) {
        rc = fl_launch_cell_keys(ctx, mesh->x, mesh->y, mesh->z, mesh->level, mesh->case_id, dom.depth,
                                 dom.anchor_level, w.keys, n);
        if (rc) return rc;
        rc = fl_hash_build_with(ctx, w.tk, w.tv, w.cap, w.keys, nullptr, n, w.win, mesh->level);  // level | index
        if (rc) return rc;
    }
    FL_TRY_CUDA(ctx, cudaMemsetAsync(w.counters, 0, 64, ctx->stream), "adapt counters");
    if (run_balance) {
        rc = fl_balance_run(ctx, md, mesh->flags, dom, w.tk, w.tv, w.cap, &L, cfg->balance_mode,
                            cfg->max_refinement_level, (int)cfg->max_balance_iterations, w.shadow, w.viol, w.act,
                            w.counters + 8, &s.balance, cfg->input_balanced != 0);
        if (rc) return rc;
    }
    unsigned nb = fl_blocks(n, kT, ctx->num_sms * 8);
    k_shadow_update<<<nb, kT, 0, ctx->stream>>>(md, 1, cfg->max_refinement_level, w.shadow, nullptr);  // final levels
    FL_CHECK_LAUNCH(ctx, "k_shadow_update");
    int check26 = cfg->enforce_2_1_balance && cfg->balance_mode == 1;
    const unsigned wb = fl_blocks((n + 31) / 32 * 32, kT, ctx->num_sms * 8);  // a warp per 32 cells
    k_leaders<<<wb, kT, 0, ctx->stream>>>(md, dom, L, cfg->min_refinement_level, check26, w.shadow, w.leader);
    FL_CHECK_LAUNCH(ctx, "k_leaders");
    rc = fl_scan_u32_with(ctx, w.leader, w.gid, n, w.counters + 2, w.scan_scratch);
    if (rc) return rc;
    rc = fl_launch_fill_u32(ctx, w.group_of, FL_INVALID_INDEX, n);
    if (rc) return rc;
    k_members<<<wb, kT, 0, ctx->stream>>>(md, dom, L, w.leader, w.gid, w.members, w.group_of);
    FL_CHECK_LAUNCH(ctx, "k_members");
    k_counts<<<nb, kT, 0, ctx->stream>>>(md, cfg->max_refinement_level, L.ids, w.leader, w.group_of, w.cnt);
    FL_CHECK_LAUNCH(ctx, "k_counts");
    k_count_kinds<<<nb, kT, 0, ctx->stream>>>(md, cfg->max_refinement_level, w.group_of, w.counters);
    FL_CHECK_LAUNCH(ctx, "k_count_kinds");
    rc = fl_scan_u32_with(ctx, w.cnt, w.cnt, n, w.counters + 3, w.scan_scratch);
    if (rc) return rc;
    uint32_t hc[6] = {0, 0, 0, 0, 0, 0};
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(hc, w.counters, 24, cudaMemcpyDeviceToHost, ctx->stream), "adapt counts");
    rc = fl_collect_device_status(ctx, "fl_adapt");
    if (rc) return rc;
    s.num_groups = hc[2];
    s.num_merged = hc[2] * 8;
    s.num_split = hc[4];
    s.num_children = hc[4] * 8;
    s.num_survivors = hc[5];
    s.num_cells_out = hc[3];
    *M_out = hc[3];
    if (st) *st = s;
    return FL_OK;
}

// Phase 2: the new cells straight into `out` (capacity >= M), in key order.
int fl_adapt_finish(fl_ctx* ctx, const fl_mesh* mesh, const fl_adapt_config* cfg, const fl_domain_dev& dom,
                    void* scratch, size_t M, const float* fields, uint32_t C, fl_mesh* out, float* out_fields,
                    uint32_t* osrc, uint8_t* okind, uint32_t* omembers, uint32_t num_groups) {
    size_t n = mesh->num_cells;
    if (n == 0 || M == 0) return FL_OK;
    AdaptWork w = carve_adapt(scratch, n, mesh->case_id != nullptr);
    fl_mesh_dev md{mesh->x, mesh->y, mesh->z, mesh->level, mesh->state, mesh->flags, mesh->material,
                   mesh->case_id, n};
    fl_mesh_out o{out->x, out->y, out->z, out->level, out->state, out->flags, out->material,
                  mesh->case_id ? out->case_id : nullptr};
    k_emit<<<fl_blocks(n, kT, ctx->num_sms * 8), kT, 0, ctx->stream>>>(
        md, dom, cfg->max_refinement_level, fl_locator_ids(w.locator, n), w.cnt, w.leader, w.group_of, w.members, o,
        osrc, okind, fields, out_fields, C, cfg->averaging_rule);
    FL_CHECK_LAUNCH(ctx, "k_emit");
    if (omembers && num_groups)
        FL_TRY_CUDA(ctx, cudaMemcpyAsync(omembers, w.members, (size_t)num_groups * 32, cudaMemcpyDeviceToDevice,
                                         ctx->stream), "members copy");
    return FL_OK;
}

extern "C" {

int fl_mesh_alloc(fl_ctx* ctx, size_t capacity, int with_case_id, fl_mesh* m) {
    if (!ctx || !m) return FL_E_INVALID_ARG;
    *m = fl_mesh{};
    if (capacity == 0) capacity = 1;
    void** col[8] = {(void**)&m->x, (void**)&m->y, (void**)&m->z, (void**)&m->level, (void**)&m->state,
                     (void**)&m->flags, (void**)&m->material, (void**)&m->case_id};
    const size_t width[8] = {4, 4, 4, 1, 1, 4, 4, 2};
    for (int k = 0; k < (with_case_id ? 8 : 7); ++k) {
        cudaError_t e = fl_dev_malloc_async(ctx, col[k], capacity * width[k], ctx->stream);
        if (e != cudaSuccess) {  // nothing half-allocated is left behind
            for (int j = 0; j < k; ++j) cudaFreeAsync(*col[j], ctx->stream);
            *m = fl_mesh{};
            return fl_check_cuda(ctx, e, "mesh alloc");
        }
    }
    m->capacity = capacity;
    m->num_cells = 0;
    return FL_OK;
}

int fl_mesh_free(fl_ctx* ctx, fl_mesh* m) {
    if (!ctx || !m) return FL_E_INVALID_ARG;
    void* ps[8] = {m->x, m->y, m->z, m->level, m->state, m->flags, m->material, m->case_id};
    for (void* p : ps)
        if (p) cudaFreeAsync(p, ctx->stream);
    *m = fl_mesh{};
    FL_TRY_CUDA(ctx, cudaGetLastError(), "mesh free");
    return FL_OK;
}

int fl_balance_enforce(fl_ctx* ctx, fl_mesh* mesh, const fl_adapt_config* cfg, fl_balance_result* res) {
    if (!ctx || !mesh || !cfg) return FL_E_INVALID_ARG;
    if (!fl_domain_config_valid(cfg))
        return fl_set_error(ctx, FL_E_INVALID_ARG, "key geometry: need anchor_level <= key_depth <= 21, max level <= anchor_level, ext << anchor_level <= 2^key_depth");
    size_t n = mesh->num_cells;
    if (res) *res = fl_balance_result{};
    if (n == 0) { if (res) res->converged = 1; return FL_OK; }
    const bool face6 = cfg->balance_mode == 0;  // FACE6 probes shadow levels through the hash table
    uint64_t cap = face6 ? fl_table_capacity(n) : 0;
    size_t need = fl_align256(n * 8) + fl_align256(cap * 16) + fl_align256(cap * 4) + 2 * fl_align256(n) +
                  fl_balance_act_bytes(n) + 512 + 256 +
                  (face6 ? 0 : fl_locator_scratch_bytes(n));
    int rc = fl_scratch_reserve(ctx, need);
    if (rc) return rc;
    Carver cv{(char*)ctx->scratch};
    void* dcase = cv.take<char>(256);
    uint64_t* keys = cv.take<uint64_t>(n);
    uint64_t* tk = cv.take<uint64_t>(2 * cap);
    uint32_t* tv = nullptr;  // 16-byte slots
    uint32_t* win = cv.take<uint32_t>(cap);
    uint8_t* shadow = cv.take<uint8_t>(n);
    uint8_t* viol = cv.take<uint8_t>(n);
    uint8_t* act = cv.take<uint8_t>(fl_balance_act_bytes(n));
    uint32_t* counters = cv.take<uint32_t>(16);
    fl_domain_dev dom = fl_domain_from_config(ctx, cfg, dcase);
    fl_mesh_dev md{mesh->x, mesh->y, mesh->z, mesh->level, mesh->state, mesh->flags, mesh->material, mesh->case_id, n};
    fl_locator L{};
    if (face6) {
        rc = fl_launch_cell_keys(ctx, mesh->x, mesh->y, mesh->z, mesh->level, mesh->case_id, dom.depth,
                                 dom.anchor_level, keys, n);
        if (rc) return rc;
        rc = fl_hash_build_with(ctx, tk, tv, cap, keys, nullptr, n, win, mesh->level);
    } else {
        rc = fl_locator_build(ctx, md, dom, cv.p, &L);
    }
    if (rc) return rc;
    fl_balance_result r;
    rc = fl_balance_run(ctx, md, mesh->flags, dom, tk, tv, cap, &L, cfg->balance_mode, cfg->max_refinement_level,
                        (int)cfg->max_balance_iterations, shadow, viol, act, counters, &r, cfg->input_balanced != 0);
    if (rc) return rc;
    rc = fl_collect_device_status(ctx, "fl_balance_enforce");
    if (rc) return rc;
    if (res) *res = r;
    return r.converged ? FL_OK : FL_E_BALANCE_NOT_CONVERGED;
}

int fl_neighbour_rebuild(fl_ctx* ctx, const fl_mesh* mesh, const fl_adapt_config* cfg, int subslots, uint32_t* nbr) {
    if (!ctx || !mesh || !cfg || !nbr || (subslots != 1 && subslots != 4)) return FL_E_INVALID_ARG;
    if (!fl_domain_config_valid(cfg))
        return fl_set_error(ctx, FL_E_INVALID_ARG, "key geometry: need anchor_level <= key_depth <= 21, max level <= anchor_level, ext << anchor_level <= 2^key_depth");
    size_t n = mesh->num_cells;
    if (n == 0) return FL_OK;
    int rc = fl_scratch_reserve(ctx, 256 + fl_align256(n * 4) + fl_locator_scratch_bytes(n));
    if (rc) return rc;
    Carver cv{(char*)ctx->scratch};
    void* dcase = cv.take<char>(256);
    uint32_t* marks = cv.take<uint32_t>(n);
    fl_domain_dev dom = fl_domain_from_config(ctx, cfg, dcase);
    dom.max_level = cfg->max_refinement_level;
    fl_mesh_dev md{mesh->x, mesh->y, mesh->z, mesh->level, mesh->state, mesh->flags, mesh->material, mesh->case_id, n};
    fl_locator L;
    rc = fl_locator_build(ctx, md, dom, cv.p, &L);
    if (rc) return rc;
    rc = fl_neighbours_sorted(ctx, md, dom, L, subslots, nbr, marks);
    if (rc) return rc;
    return fl_collect_device_status(ctx, "fl_neighbour_rebuild");
}

int fl_adapt(fl_ctx* ctx, fl_mesh* mesh, const fl_adapt_config* cfg, float** fields, uint32_t C,
             fl_adapt_stats* stats) {
    if (!ctx || !mesh || !cfg) return FL_E_INVALID_ARG;
    if (C && (!fields || !*fields)) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_adapt: components without fields");
    if (cfg->max_refinement_level > 21 || cfg->min_refinement_level > cfg->max_refinement_level)
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_adapt: bad level limits (AdaptationConfig::validate)");
    if (!fl_domain_config_valid(cfg))
        return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_adapt: key geometry needs ext << anchor_level <= 2^key_depth");
    size_t n = mesh->num_cells;
    if (stats) *stats = fl_adapt_stats{};
    if (n == 0) return FL_OK;
    int rc = fl_scratch_reserve(ctx, fl_adapt_scratch_bytes(n, fl_table_capacity(n)) + 512);
    if (rc) return rc;
    void* dcase = ctx->scratch;
    void* scratch = (char*)ctx->scratch + 512;
    fl_domain_dev dom = fl_domain_from_config(ctx, cfg, dcase);
    dom.max_level = cfg->max_refinement_level > 0 ? cfg->max_refinement_level : dom.anchor_level;
    size_t M = 0;
    fl_adapt_stats s{};
    rc = fl_adapt_prepare(ctx, mesh, cfg, dom, cfg->enforce_2_1_balance != 0, scratch, &M, &s);
    if (rc) return rc;
    // no change: keep the buffers (AdaptationEngine.cpp:72-77), flags still reset below
    size_t cap_out = mesh->capacity;
    if (M > cap_out) {  // growth rule of AdaptationEngine.cpp:473-478
        double g = cfg->buffer_growth_factor > 1.0 ? cfg->buffer_growth_factor : 1.5;
        size_t a = (size_t)((double)M * g), b = M + 1024;
        cap_out = a > b ? a : b;
    }
    fl_mesh out{};
    rc = fl_mesh_alloc(ctx, cap_out, mesh->case_id != nullptr, &out);
    if (rc) return rc;
    float* nf = nullptr;
    if (C) {
        cudaError_t e = fl_dev_malloc_async(ctx, (void**)&nf, cap_out * C * 4, ctx->stream);
        if (e != cudaSuccess) {  // the input mesh and fields stay as they were
            fl_mesh_free(ctx, &out);
            return fl_check_cuda(ctx, e, "fields alloc");
        }
    }
    rc = fl_adapt_finish(ctx, mesh, cfg, dom, scratch, M, C ? *fields : nullptr, C, &out, nf, nullptr, nullptr,
                         nullptr, s.num_groups);
    if (rc) {
        fl_mesh_free(ctx, &out);
        if (nf) cudaFreeAsync(nf, ctx->stream);
        return rc;
    }
    fl_mesh old = *mesh;
    fl_mesh_free(ctx, &old);
    if (C) {
        cudaFreeAsync(*fields, ctx->stream);
        *fields = nf;
    }
    out.num_cells = M;
    out.capacity = cap_out;
    *mesh = out;
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "fl_adapt");
    if (stats) *stats = s;
    return (s.balance.converged || !cfg->enforce_2_1_balance) ? FL_OK : FL_E_BALANCE_NOT_CONVERGED;
}

int fl_split(fl_ctx* ctx, const fl_mesh* mesh, const fl_adapt_config* cfg, const float* fields, uint32_t C,
             fl_mesh* children, float* child_fields, uint32_t* parent_to_child, size_t* num_children) {
    if (!ctx || !mesh || !cfg || !children || !num_children) return FL_E_INVALID_ARG;
    *num_children = 0;
    size_t n = mesh->num_cells;
    if (n == 0) return FL_OK;
    int rc = fl_scratch_reserve(ctx, 2 * fl_align256(n * 4) + fl_scan_scratch_bytes(n) + 512);
    if (rc) return rc;
    Carver cv{(char*)ctx->scratch};
    uint32_t* pred = cv.take<uint32_t>(n);
    uint32_t* off = cv.take<uint32_t>(n);
    uint32_t* total = cv.take<uint32_t>(4);
    void* ss = cv.p;
    fl_mesh_dev md{mesh->x, mesh->y, mesh->z, mesh->level, mesh->state, mesh->flags, mesh->material, mesh->case_id, n};
    unsigned nb = fl_blocks(n, kT, ctx->num_sms * 8);
    k_split_pred<<<nb, kT, 0, ctx->stream>>>(md, cfg->max_refinement_level, pred);
    FL_CHECK_LAUNCH(ctx, "k_split_pred");
    rc = fl_scan_u32_with(ctx, pred, off, n, total, ss);
    if (rc) return rc;
    uint32_t h = 0;
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(&h, total, 4, cudaMemcpyDeviceToHost, ctx->stream), "split count");
    rc = fl_collect_device_status(ctx, "fl_split");
    if (rc) return rc;
    size_t nc = (size_t)h * 8;
    if (nc > children->capacity) {
        *num_children = nc;
        return fl_set_error(ctx, FL_E_CAPACITY, "fl_split: children capacity too small (count returned)");
    }
    fl_mesh_out o{children->x, children->y, children->z, children->level, children->state, children->flags,
                  children->material, mesh->case_id ? children->case_id : nullptr};
    k_split_children<<<nb, kT, 0, ctx->stream>>>(md, pred, off, o, parent_to_child, fields, child_fields, C);
    FL_CHECK_LAUNCH(ctx, "k_split_children");
    children->num_cells = nc;
    *num_children = nc;
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "fl_split");
    return FL_OK;
}

int fl_merge(fl_ctx* ctx, const fl_mesh* mesh, const fl_adapt_config* cfg, const float* fields, uint32_t C,
             fl_mesh* parents, float* parent_fields, uint32_t* merge_group_id, size_t* num_parents) {
    if (!ctx || !mesh || !cfg || !parents || !num_parents) return FL_E_INVALID_ARG;
    if (!fl_domain_config_valid(cfg)) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_merge: bad key geometry");
    *num_parents = 0;
    size_t n = mesh->num_cells;
    if (n == 0) return FL_OK;
    int rc = fl_scratch_reserve(ctx, 256 + fl_align256(fl_locator_scratch_bytes(n)) + 4 * fl_align256(n * 4) +
                                         fl_align256(n * 4 + 64) + fl_scan_scratch_bytes(n) + 512);
    if (rc) return rc;
    Carver cv{(char*)ctx->scratch};
    void* dcase = cv.take<char>(256);
    void* loc = cv.take<char>(fl_locator_scratch_bytes(n));
    uint32_t* leader = cv.take<uint32_t>(n);
    uint32_t* gid = cv.take<uint32_t>(n);
    uint32_t* group_of = merge_group_id ? merge_group_id : cv.take<uint32_t>(n);
    uint32_t* members = cv.take<uint32_t>(n + 16);
    uint32_t* total = cv.take<uint32_t>(4);
    void* ss = cv.p;
    fl_domain_dev dom = fl_domain_from_config(ctx, cfg, dcase);
    fl_mesh_dev md{mesh->x, mesh->y, mesh->z, mesh->level, mesh->state, mesh->flags, mesh->material, mesh->case_id, n};
    fl_locator L;
    rc = fl_locator_build(ctx, md, dom, loc, &L);
    if (rc) return rc;
    const unsigned wb = fl_blocks((n + 31) / 32 * 32, kT, ctx->num_sms * 8);  // a warp per 32 cells
    k_leaders<<<wb, kT, 0, ctx->stream>>>(md, dom, L, cfg->min_refinement_level, 0, nullptr, leader);
    FL_CHECK_LAUNCH(ctx, "k_leaders");
    rc = fl_scan_u32_with(ctx, leader, gid, n, total, ss);
    if (rc) return rc;
    rc = fl_launch_fill_u32(ctx, group_of, FL_INVALID_INDEX, n);
    if (rc) return rc;
    k_members<<<wb, kT, 0, ctx->stream>>>(md, dom, L, leader, gid, members, group_of);
    FL_CHECK_LAUNCH(ctx, "k_members");
    uint32_t G = 0;
    FL_TRY_CUDA(ctx, cudaMemcpyAsync(&G, total, 4, cudaMemcpyDeviceToHost, ctx->stream), "merge count");
    rc = fl_collect_device_status(ctx, "fl_merge");
    if (rc) return rc;
    if (G > parents->capacity) {
        *num_parents = G;
        return fl_set_error(ctx, FL_E_CAPACITY, "fl_merge: parents capacity too small (count returned)");
    }
    if (G) {
        fl_mesh_out o{parents->x, parents->y, parents->z, parents->level, parents->state, parents->flags,
                      parents->material, mesh->case_id ? parents->case_id : nullptr};
        k_merge_parents<<<fl_blocks(G, kT, ctx->num_sms * 8), kT, 0, ctx->stream>>>(md, members, G, o, fields,
                                                                                   parent_fields, C, cfg->averaging_rule);
        FL_CHECK_LAUNCH(ctx, "k_merge_parents");
    }
    parents->num_cells = G;
    *num_parents = G;
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "fl_merge");
    return FL_OK;
}

}  // extern "C"
