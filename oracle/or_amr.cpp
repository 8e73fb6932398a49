// or_amr.cpp — oracle: point location, neighbour tables, 2:1 balance, split,
// merge, one regrid (adapt), coarse/fine interpolation and restriction.
// TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// Coordinates are native-level (child = parent << 1 | bit, CellDescriptor.h:67-79
// and split_cells.cl:90-92).  A cell's anchor is native << (A - level); the
// domain array `dom` is indexed by case id (index 0 when a mesh has none).
#include "oracle.h"

#include <algorithm>
#include <cstring>
#include <unordered_map>
#include <vector>

namespace {

const uint32_t INV = 0xFFFFFFFFu;

struct Index {
    std::unordered_map<uint64_t, uint32_t> map;
};

inline uint64_t anchor_key(int depth, uint16_t cs, int64_t ax, int64_t ay, int64_t az) {
    uint64_t k = or_hilbert_encode1((int32_t)ax, (int32_t)ay, (int32_t)az, (uint8_t)depth);
    return k | ((uint64_t)cs << (3 * depth));
}

inline uint16_t case_of(const or_mesh* m, size_t i) { return m->case_id ? m->case_id[i] : 0; }

void build_index(const or_mesh* m, const or_domain* dom, Index& ix) {
    ix.map.clear();
    ix.map.reserve(m->n * 2);
    for (size_t i = 0; i < m->n; ++i) {
        const or_domain& d = dom[case_of(m, i)];
        int sh = d.anchor_level - m->level[i];
        uint64_t k = anchor_key(d.depth, case_of(m, i), (int64_t)m->x[i] << sh, (int64_t)m->y[i] << sh,
                                (int64_t)m->z[i] << sh);
        ix.map[k] = (uint32_t)i;  // last writer wins, as sequential insertion
    }
}

// Wrap / reject a probe point against the domain; returns false if outside.
inline bool fold(const or_domain& d, int64_t* p) {
    for (int a = 0; a < 3; ++a) {
        int64_t ext = (int64_t)(d.ext[a] ? d.ext[a] : 1) << d.anchor_level;
        if (p[a] < 0 || p[a] >= ext) {
            if (!d.periodic[a]) return false;
            p[a] = ((p[a] % ext) + ext) % ext;
        }
    }
    return true;
}

// Point location (balance_enforce.cl:107-143 rule, without its probe cap):
// the cell whose `lv` equals l and whose anchor equals p with the low
// (A - l) bits cleared, for some l in [0, max_level].  In a valid leaf set at
// most one l matches, so the probing order does not change the answer.
uint32_t locate(const Index& ix, const or_domain& d, uint16_t cs, const int64_t* p, const uint8_t* lv) {
    for (int l = 0; l <= d.max_level; ++l) {
        int sh = d.anchor_level - l;
        int64_t mask = ~(((int64_t)1 << sh) - 1);
        uint64_t k = anchor_key(d.depth, cs, p[0] & mask, p[1] & mask, p[2] & mask);
        auto it = ix.map.find(k);
        if (it != ix.map.end() && lv[it->second] == l) return it->second;
    }
    return INV;
}

// 26 directions: dz outer, dy, dx inner, centre skipped.
inline void dir_of(int k, int* d) {
    int kk = k < 13 ? k : k + 1;
    d[0] = kk % 3 - 1; d[1] = (kk / 3) % 3 - 1; d[2] = kk / 9 - 1;
}

// Probe point of direction d, sub-slot s (bits over the zero axes in x,y,z order).
inline void probe_point(const int64_t* anc, int64_t size, const int* d, int s, int64_t* p) {
    int bit = 0;
    for (int a = 0; a < 3; ++a) {
        if (d[a] < 0) p[a] = anc[a] - 1;
        else if (d[a] > 0) p[a] = anc[a] + size;
        else { p[a] = anc[a] + (((s >> bit) & 1) ? (size >> 1) : 0); ++bit; }
    }
}

inline void anchor_of(const or_mesh* m, const or_domain& d, size_t i, int64_t* anc, int64_t* size) {
    int sh = d.anchor_level - m->level[i];
    anc[0] = (int64_t)m->x[i] << sh; anc[1] = (int64_t)m->y[i] << sh; anc[2] = (int64_t)m->z[i] << sh;
    *size = (int64_t)1 << sh;
}

}  // namespace

// Neighbour table: nbr[i][k][s] = leaf containing the probe point of direction
// k, sub-slot s (subslots 1 or 4), INVALID outside a non-periodic domain.
extern "C" void or_neighbours(const or_mesh* m, const or_domain* dom, int subslots, uint32_t* nbr) {
    Index ix;
    build_index(m, dom, ix);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)m->n; ++i) {
        const or_domain& d = dom[case_of(m, i)];
        int64_t anc[3], size;
        anchor_of(m, d, i, anc, &size);
        for (int k = 0; k < 26; ++k) {
            int dv[3];
            dir_of(k, dv);
            for (int s = 0; s < subslots; ++s) {
                int64_t p[3];
                probe_point(anc, size, dv, s, p);
                uint32_t r = INV;
                if (fold(d, p)) r = locate(ix, d, case_of(m, i), p, m->level);
                nbr[((size_t)i * 26 + k) * subslots + s] = r;
            }
        }
    }
}

// 2:1 balance.
//  mode 0 (FACE6): BalanceEnforcer::enforce, src/adaptation/BalanceEnforcer.cpp:145-263,
//    with detect_balance_violations / mark_cascading_refinement
//    (src/adaptation/kernels/balance_enforce.cl:57-172): shadow levels start
//    as the levels, six face probes at anchor-1 / anchor+size(shadow), a probe
//    is "found" at the cell whose SHADOW level equals the probed level, a
//    violation is found level > shadow + 1, violators (FLUID, below max level,
//    flag <= 0) get flag 1, shadow = level + (flag > 0), at most max_iters
//    rounds.  Deviation: lookups are exact (the reference's 64-probe cap over a
//    Morton-low-bits hash silently misses cells).
//  mode 1 (FULL26): face+edge+corner balance to a fixed point.  Every leaf
//    probes its 26 neighbour points at its own size; a leaf n found with
//    shadow(i) >= shadow(n) + 2 must refine, where shadow = level + 1 only
//    for a cell that will split (flag > 0, fluid, below the maximum level).
extern "C" int or_balance(or_mesh* m, const or_domain* dom, int mode, int max_level, int max_iters,
                          or_balance_stats* st) {
    std::memset(st, 0, sizeof(*st));
    size_t n = m->n;
    if (n == 0) { st->converged = 1; return 0; }
    Index ix;
    build_index(m, dom, ix);
    std::vector<uint8_t> shadow(n), viol(n);
    // FULL26: a flag raises the shadow level only where the cell will split
    auto up = [&](size_t i) {
        return mode == 0 ? m->flags[i] > 0 : (m->flags[i] > 0 && m->state[i] == 0 && m->level[i] < max_level);
    };
    for (size_t i = 0; i < n; ++i) shadow[i] = mode == 0 ? m->level[i] : (uint8_t)(m->level[i] + (up(i) ? 1 : 0));
    int cap = mode == 0 ? max_iters : 4096;
    uint32_t it = 0;
    for (; it < (uint32_t)cap; ++it) {
        uint32_t nviol = 0;
        std::fill(viol.begin(), viol.end(), 0);
        for (size_t i = 0; i < n; ++i) {
            const or_domain& d = dom[case_of(m, i)];
            int64_t anc[3], size;
            anchor_of(m, d, i, anc, &size);
            if (mode == 0) {
                if (m->state[i] != 0) continue;
                int sl = shadow[i];
                int ex = d.anchor_level - sl;
                int64_t ss = ex > 0 ? ((int64_t)1 << ex) : 1;
                for (int f = 0; f < 6; ++f) {
                    int64_t p[3] = {anc[0], anc[1], anc[2]};
                    p[f >> 1] += (f & 1) ? ss : -1;
                    if (!fold(d, p)) continue;
                    uint32_t r = locate(ix, d, case_of(m, i), p, shadow.data());
                    if (r == INV) continue;
                    if ((int)shadow[r] > sl + 1) { viol[i] = 1; ++nviol; break; }
                }
            } else {
                for (int k = 0; k < 26; ++k) {
                    int dv[3];
                    dir_of(k, dv);
                    int64_t p[3];
                    probe_point(anc, size, dv, 0, p);
                    if (!fold(d, p)) continue;
                    uint32_t r = locate(ix, d, case_of(m, i), p, m->level);
                    if (r == INV) continue;
                    if ((int)shadow[i] >= (int)shadow[r] + 2) { viol[r] = 1; ++nviol; }
                }
            }
        }
        if (it < 64) st->per_iter_violations[it] = nviol;
        st->violations += nviol;
        if (nviol == 0) { st->converged = 1; st->iterations = it + 1; return 0; }
        uint32_t marked = 0;
        for (size_t i = 0; i < n; ++i) {
            if (!viol[i] || m->state[i] != 0 || m->level[i] >= max_level) continue;
            if (m->flags[i] <= 0) { m->flags[i] = 1; ++marked; }
        }
        if (it < 64) st->per_iter_marked[it] = marked;
        st->marked += marked;
        if (marked == 0) { st->converged = 0; st->iterations = it + 1; return 0; }
        for (size_t i = 0; i < n; ++i) shadow[i] = (uint8_t)(m->level[i] + (up(i) ? 1 : 0));
    }
    st->converged = 0;
    st->iterations = it;
    return 0;
}

// One regrid (AdaptationEngine::adapt, src/adaptation/AdaptationEngine.cpp:37-102):
// balance -> split (SplitEngine::split, SplitEngine.cpp:95-267; split_cells.cl:15-106)
// -> merge (MergeEngine::merge, MergeEngine.cpp:140-334; merge_cells.cl:11-199)
// -> rebuild in the order of the CPU rebuild (AdaptationEngine.cpp:104-276):
// survivors, children (fields copied from the parent), parents (fields
// averaged), sorted by key, flags reset to 0.  Deviations: group ids follow the
// first-sibling index (not atomic_inc, merge_cells.cl:99); restriction sums
// children 0..7 in order then scales (FieldAveragingRules.h:31-52, not float
// CAS atomics); merging stops at min_level (the reference would wrap level 0
// to 255); the sort key is the unique anchor key; in FULL26 mode a group is
// merged only if no touching leaf outside it ends above the group's level.
// sites_mode 0: fields are AoS [cell][C] (the reference layout).
extern "C" size_t or_adapt(or_mesh* m, const or_domain* dom, const or_adapt_cfg* cfg, const float* fields,
                           uint32_t C, int sites_mode, int32_t* ox, int32_t* oy, int32_t* oz, uint8_t* olevel,
                           uint8_t* ostate, int32_t* oflags, uint32_t* omat, uint16_t* ocase, float* ofields,
                           uint32_t* osrc, uint8_t* okind, uint32_t* omembers, or_adapt_stats* st) {
    (void)sites_mode;
    std::memset(st, 0, sizeof(*st));
    size_t n = m->n;
    if (cfg->enforce_balance)
        or_balance(m, dom, cfg->balance_mode, cfg->max_level, cfg->max_balance_iterations, &st->balance);
    Index ix;
    build_index(m, dom, ix);
    std::vector<uint8_t> split(n, 0), merged(n, 0), leader(n, 0);
    for (size_t i = 0; i < n; ++i)
        split[i] = m->flags[i] > 0 && m->state[i] == 0 && m->level[i] < cfg->max_level;
    std::vector<uint8_t> shadow(n);  // final levels (the FULL26 merge condition)
    for (size_t i = 0; i < n; ++i) shadow[i] = (uint8_t)(m->level[i] + (split[i] ? 1 : 0));
    std::vector<uint32_t> members;  // [group][8]
    std::vector<uint32_t> group_of(n, INV);
    for (size_t i = 0; i < n; ++i) {
        if (m->flags[i] != -1 || m->state[i] != 0) continue;
        if ((m->x[i] & 1) || (m->y[i] & 1) || (m->z[i] & 1)) continue;
        int l = m->level[i];
        if (l <= cfg->min_level) continue;
        const or_domain& d = dom[case_of(m, i)];
        uint32_t mem[8];
        bool ok = true;
        for (int c = 0; c < 8 && ok; ++c) {
            int32_t sx = m->x[i] | (c & 1), sy = m->y[i] | ((c >> 1) & 1), sz = m->z[i] | ((c >> 2) & 1);
            int sh = d.anchor_level - l;
            auto it = ix.map.find(anchor_key(d.depth, case_of(m, i), (int64_t)sx << sh, (int64_t)sy << sh,
                                             (int64_t)sz << sh));
            if (it == ix.map.end()) { ok = false; break; }
            uint32_t j = it->second;
            if (m->level[j] != l || m->flags[j] != -1 || m->state[j] != 0) { ok = false; break; }
            mem[c] = j;
        }
        if (ok && cfg->enforce_balance && cfg->balance_mode == 1) {
            for (int c = 0; c < 8 && ok; ++c) {
                int64_t anc[3], size;
                anchor_of(m, d, mem[c], anc, &size);
                for (int k = 0; k < 26 && ok; ++k) {
                    int dv[3];
                    dir_of(k, dv);
                    int64_t p[3];
                    probe_point(anc, size, dv, 0, p);
                    if (!fold(d, p)) continue;
                    uint32_t r = locate(ix, d, case_of(m, i), p, m->level);
                    if (r == INV) continue;
                    bool inside = false;
                    for (int q = 0; q < 8; ++q) inside |= (mem[q] == r);
                    if (!inside && (int)shadow[r] > l) ok = false;
                }
            }
        }
        if (!ok) continue;
        leader[i] = 1;
        uint32_t g = (uint32_t)(members.size() / 8);
        for (int c = 0; c < 8; ++c) { members.push_back(mem[c]); merged[mem[c]] = 1; group_of[mem[c]] = g; }
    }
    size_t ngroups = members.size() / 8;
    // Intermediate list in old-index order.
    struct Item { int32_t x, y, z; uint8_t l, s; uint32_t mat; uint16_t cs; uint32_t src; uint8_t kind; };
    std::vector<Item> items;
    items.reserve(n + 8 * n / 4);
    for (size_t i = 0; i < n; ++i) {
        uint16_t cs = case_of(m, i);
        if (split[i]) {
            st->num_split++;
            for (int c = 0; c < 8; ++c)
                items.push_back({(m->x[i] << 1) | (c & 1), (m->y[i] << 1) | ((c >> 1) & 1),
                                 (m->z[i] << 1) | ((c >> 2) & 1), (uint8_t)(m->level[i] + 1), m->state[i],
                                 m->material[i], cs, (uint32_t)i, (uint8_t)c});
        } else if (merged[i]) {
            if (leader[i])
                items.push_back({m->x[i] >> 1, m->y[i] >> 1, m->z[i] >> 1, (uint8_t)(m->level[i] - 1), m->state[i],
                                 m->material[i], cs, group_of[i], 9});
        } else {
            items.push_back({m->x[i], m->y[i], m->z[i], m->level[i], m->state[i], m->material[i], cs, (uint32_t)i, 8});
            st->num_survivors++;
        }
    }
    st->num_children = st->num_split * 8;
    st->num_groups = (uint32_t)ngroups;
    st->num_merged = (uint32_t)(ngroups * 8);
    size_t M = items.size();
    std::vector<uint64_t> keys(M);
    std::vector<uint32_t> perm(M);
    for (size_t j = 0; j < M; ++j) {
        const or_domain& d = dom[items[j].cs];
        int sh = d.anchor_level - items[j].l;
        keys[j] = anchor_key(d.depth, m->case_id ? items[j].cs : 0, (int64_t)items[j].x << sh,
                             (int64_t)items[j].y << sh, (int64_t)items[j].z << sh);
        perm[j] = (uint32_t)j;
    }
    or_sort_pairs_u64_u32(keys.data(), perm.data(), M);
    for (size_t j = 0; j < M; ++j) {
        const Item& it = items[perm[j]];
        ox[j] = it.x; oy[j] = it.y; oz[j] = it.z; olevel[j] = it.l; ostate[j] = it.s;
        oflags[j] = 0; omat[j] = it.mat;
        if (ocase) ocase[j] = it.cs;
        if (osrc) osrc[j] = it.src;
        if (okind) okind[j] = it.kind;
        if (fields && ofields && C) {
            float* o = ofields + j * C;
            if (it.kind == 8) std::memcpy(o, fields + (size_t)it.src * C, C * 4);
            else if (it.kind < 8) std::memcpy(o, fields + (size_t)it.src * C, C * 4);
            else {
                const uint32_t* mem = &members[(size_t)it.src * 8];
                for (uint32_t c = 0; c < C; ++c) {
                    float s = 0.0f;
                    for (int q = 0; q < 8; ++q) s = s + fields[(size_t)mem[q] * C + c];
                    o[c] = cfg->averaging_rule == 1 ? s : s * 0.125f;
                }
            }
        }
    }
    if (omembers) std::memcpy(omembers, members.data(), members.size() * 4);
    st->num_out = (uint32_t)M;
    return M;
}

// trilinear_interpolate, kernels/halo/interpolate_trilinear.cl:12-56 with
// TrilinearParams::initializeDefault (include/fluidloom/halo/InterpolationParams.h:34-43):
// coarse = fine / 2 (C division), 8 corners coarse + {0,1}^3 in corner order,
// weight 0.125 each, a missing corner contributes nothing.  The corner cell is
// looked up exactly at level (fine level - 1).
extern "C" void or_interp_trilinear(const or_mesh* m, const or_domain* dom, const float* fields, uint32_t C,
                                    const int32_t* fx, const int32_t* fy, const int32_t* fz,
                                    const uint8_t* flevel, size_t nq, float* out) {
    Index ix;
    build_index(m, dom, ix);
    const or_domain& d = dom[0];
    for (size_t i = 0; i < nq; ++i) {
        float* o = out + i * C;
        for (uint32_t c = 0; c < C; ++c) o[c] = 0.0f;
        if (flevel[i] == 0) continue;
        int l = flevel[i] - 1;
        int32_t cx = fx[i] / 2, cy = fy[i] / 2, cz = fz[i] / 2;
        for (int k = 0; k < 8; ++k) {
            int64_t p[3] = {cx + (k & 1), cy + ((k >> 1) & 1), cz + ((k >> 2) & 1)};
            if (p[0] < 0 || p[1] < 0 || p[2] < 0) continue;
            int sh = d.anchor_level - l;
            auto it = ix.map.find(anchor_key(d.depth, 0, p[0] << sh, p[1] << sh, p[2] << sh));
            if (it == ix.map.end() || m->level[it->second] != l) continue;
            const float* v = fields + (size_t)it->second * C;
            for (uint32_t c = 0; c < C; ++c) o[c] = o[c] + 0.125f * v[c];
        }
    }
}

// Restriction of sibling groups (merge_fields, merge_cells.cl:123-159, with the
// sum order of FieldAveragingRules.h:31-52): children 0..7 summed in order,
// x 0.125 for rule 0 (arithmetic), unscaled for rule 1 (volume weighted).
extern "C" void or_restrict_groups(const float* fields, uint32_t C, const uint32_t* members, size_t ngroups,
                                   int rule, float* out) {
    for (size_t g = 0; g < ngroups; ++g)
        for (uint32_t c = 0; c < C; ++c) {
            float s = 0.0f;
            for (int q = 0; q < 8; ++q) s = s + fields[(size_t)members[g * 8 + q] * C + c];
            out[g * C + c] = rule == 1 ? s : s * 0.125f;
        }
}
