// ref_kernels.cpp -- drives the reference's OpenCL kernels, compiled unmodified
// as C++ from the reference tree (oracle/Makefile.ref, shim/opencl_c.h), on the
// CPU.  TEST INFRASTRUCTURE ONLY: the oracle restatement (or_amr.cpp,
// or_keys_prims.cpp) is diffed against these results.
//
// The kernel bodies are the reference's.  What this file adds is the host
// side that enqueues them, restated step by step from the reference's engines
// (cited per function, paths inside the fedres/fluidloom tree): buffer
// set-up, the host-built lookup tables, the host scans and the iteration
// loops.  Host memory stands in for cl_mem buffers; a kernel "launch" is one
// flcl::run over the same global and local sizes the engine enqueues.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "ndrange.h"

namespace {

const uint32_t INV = 0xFFFFFFFFu;
const size_t LOCAL = 256;  // every engine enqueues 256-wide groups

size_t global_for(size_t n) { return ((n + LOCAL - 1) / LOCAL) * LOCAL; }

// Morton-style 3-D key of the engines' host tables: the same function as the
// kernels' hilbert_encode_3d (src/adaptation/utils/HilbertCodec3D.cpp:29-53,
// compiled in place into this library).
}  // namespace

namespace fluidloom { namespace adaptation {
uint64_t hilbert_encode_3d(int32_t x, int32_t y, int32_t z, uint8_t max_level);
} }

namespace {

// Host-built open-addressing table of cell indices keyed by the 8-level key of
// the coordinates, slot = key % size, linear probing, size = pow2 >= 2n and
// >= 1024 (BalanceEnforcer::buildHashTable, src/adaptation/BalanceEnforcer.cpp:100-143;
// MergeEngine::buildHashTable, src/adaptation/MergeEngine.cpp:90-138, identical).
// *max_disp = the longest distance from a key's home slot to its slot: a
// kernel probing at most P slots finds every stored key when max_disp < P.
// min_size (a power of two, 0 = the engines' sizing) is this harness's one
// knob: with min_size = 2^24, at least every 8-level key, each key sits in its
// home slot, so the kernels' lookups are exact whatever the mesh and the
// kernels' own semantics can be compared apart from the table's sizing.
std::vector<uint32_t> engine_table(const int32_t* x, const int32_t* y, const int32_t* z, size_t n,
                                   uint32_t min_size, uint32_t* max_disp) {
    size_t size = 1;
    while (size < n * 2) size *= 2;
    if (size < 1024) size = 1024;
    if (size < min_size) size = min_size;
    std::vector<uint32_t> t(size, INV);
    uint32_t md = 0;
    for (size_t i = 0; i < n; ++i) {
        uint64_t h = fluidloom::adaptation::hilbert_encode_3d(x[i], y[i], z[i], 8);
        uint32_t slot = (uint32_t)(h % size);
        size_t probes = 0;
        while (t[slot] != INV && probes < size) { slot = (uint32_t)((slot + 1) % size); ++probes; }
        if (t[slot] == INV) t[slot] = (uint32_t)i;
        md = std::max<uint32_t>(md, (uint32_t)probes);
    }
    if (max_disp) *max_disp = md;
    return t;
}

}  // namespace

extern "C" {

typedef struct rk_balance_stats {
    int32_t converged; uint32_t iterations; uint32_t violations; uint32_t marked;
    uint32_t per_iter_violations[64]; uint32_t per_iter_marked[64];
    uint32_t table_max_displacement;
} rk_balance_stats;

// BalanceEnforcer::enforce (src/adaptation/BalanceEnforcer.cpp:145-263).  The
// coordinates are what the kernels read them as: level-8 anchors
// (balance_enforce.cl:76: size = 1 << (8 - level)).  Shadow levels start as the
// levels; each round runs detect_balance_violations on the shadow levels and
// mark_cascading_refinement on the levels, stops on zero violations
// (converged) or zero marks (not converged), then recomputes the shadow levels
// as level + (flag > 0) -- the engine's inline update_shadow_levels kernel
// (BalanceEnforcer.cpp:53-62), restated here because it lives in a C++ string.
void rk_balance(const int32_t* ax, const int32_t* ay, const int32_t* az, const uint8_t* level,
                const uint8_t* state, int32_t* flags, size_t n, uint32_t max_iters, uint32_t table_min_size,
                rk_balance_stats* st) {
    std::memset(st, 0, sizeof(*st));
    if (n == 0) return;
    std::vector<uint32_t> table = engine_table(ax, ay, az, n, table_min_size, &st->table_max_displacement);
    std::vector<uint8_t> viol(n), shadow(level, level + n);
    uint32_t vcount = 0, mcount = 0;
    const uint nn = (uint)n, tsize = (uint)table.size();
    for (uint32_t it = 0; it < max_iters; ++it) {
        vcount = mcount = 0;
        flcl::run(global_for(n), LOCAL, [&] {
            detect_balance_violations(ax, ay, az, shadow.data(), state, nullptr, table.data(), tsize, viol.data(),
                                      &vcount, nn);
        }, flcl::kSequential);
        st->violations += vcount;
        if (vcount == 0) { st->converged = 1; st->iterations = it + 1; break; }
        flcl::run(global_for(n), LOCAL, [&] {
            mark_cascading_refinement(ax, ay, az, level, state, viol.data(), flags, &mcount, nn);
        }, flcl::kSequential);
        st->marked += mcount;
        if (it < 64) { st->per_iter_violations[it] = vcount; st->per_iter_marked[it] = mcount; }
        if (mcount == 0) { st->converged = 0; st->iterations = it + 1; break; }
        for (size_t i = 0; i < n; ++i) shadow[i] = (uint8_t)(level[i] + (flags[i] > 0 ? 1 : 0));
        st->iterations = it + 1;
    }
}

// SplitEngine::split (src/adaptation/SplitEngine.cpp:95-267): the count kernel
// (split_count_and_allocate, a barrier kernel) writes the 0/1 predicate; the
// host scans it serially into child block starts (8 per split parent, INVALID
// otherwise); split_generate_children writes the children and their 8-level
// keys; interpolate_split_fields copies the parent's field row to each child.
// Returns the number of children.  fields may be NULL (C = 0).  count_out (may
// be NULL) receives the block starts the count kernel itself wrote before the
// engine replaced them with its host scan.
uint32_t rk_split(const int32_t* x, const int32_t* y, const int32_t* z, const uint8_t* level, const uint8_t* state,
                  const int32_t* flags, const uint32_t* mat, size_t n, const float* fields, uint32_t C,
                  uint32_t* child_block_start, int32_t* cx, int32_t* cy, int32_t* cz, uint8_t* clevel,
                  uint8_t* cstate, uint32_t* cmat, uint64_t* chilbert, float* cfields, uint32_t* count_out) {
    if (n == 0) return 0;
    std::vector<uint32_t> scratch(n);
    const uint nn = (uint)n;
    flcl::run(global_for(n), LOCAL, [&] {
        split_count_and_allocate(x, y, z, level, flags, state, child_block_start, scratch.data(), nn);
    }, flcl::kGroupFibers);
    if (count_out) std::memcpy(count_out, child_block_start, n * sizeof(uint32_t));
    uint32_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        if (scratch[i] == 1) { child_block_start[i] = total; total += 8; }
        else child_block_start[i] = INV;
    }
    if (total == 0) return 0;
    flcl::run(global_for(n), LOCAL, [&] {
        split_generate_children(x, y, z, level, state, mat, child_block_start, cx, cy, cz, clevel, cstate, cmat,
                                chilbert, nn);
    }, flcl::kSequential);
    if (fields && C > 0)
        flcl::run(global_for(n), LOCAL, [&] {
            interpolate_split_fields(child_block_start, fields, cfields, C, nn);
        }, flcl::kSequential);
    return total;
}

// MergeEngine::merge (src/adaptation/MergeEngine.cpp:140-334): host table over
// the (native) coordinates, mark_sibling_groups with a zeroed group counter,
// group_to_parent = identity, create_parent_cells, and -- with fields --
// merge_fields into a zero-filled parent field buffer.  Returns the number of
// groups; group_id[n] receives merge_group_id.
// mark_sibling_groups stores INVALID into its own work-item's group id
// (merge_cells.cl:29) in the same launch in which a leader stores the group id
// of all eight siblings (:101-104), so a sibling whose work-item runs after
// its leader's store loses its id.  sequential = 0 runs it with every
// work-item's first store before any leader's (flcl::kAllFibers: the atomic
// that precedes the leaders' stores is a scheduling point), the kernel's
// intended result; sequential = 1 runs work-items in order, where every
// sibling after its leader is cleared.
uint32_t rk_merge(const int32_t* x, const int32_t* y, const int32_t* z, const uint8_t* level, const uint8_t* state,
                  const int32_t* flags, const uint32_t* mat, size_t n, const float* fields, uint32_t C,
                  uint32_t rule, uint32_t table_min_size, int sequential, uint32_t* group_id, int32_t* px,
                  int32_t* py, int32_t* pz, uint8_t* plevel, uint8_t* pstate, uint32_t* pmat, float* pfields,
                  uint32_t* table_max_displacement) {
    if (n == 0) return 0;
    std::vector<uint32_t> table = engine_table(x, y, z, n, table_min_size, table_max_displacement);
    uint32_t counter = 0;
    const uint nn = (uint)n, tsize = (uint)table.size();
    flcl::run(global_for(n), LOCAL, [&] {
        mark_sibling_groups(x, y, z, level, flags, state, group_id, &counter, nullptr, table.data(), tsize, nn);
    }, sequential ? flcl::kSequential : flcl::kAllFibers);
    if (counter == 0) return 0;
    std::vector<uint32_t> g2p(counter);
    for (uint32_t i = 0; i < counter; ++i) g2p[i] = i;
    flcl::run(global_for(n), LOCAL, [&] {
        create_parent_cells(x, y, z, level, state, mat, group_id, g2p.data(), px, py, pz, plevel, pstate, pmat, nn);
    }, flcl::kSequential);
    if (fields && C > 0) {
        std::fill(pfields, pfields + (size_t)counter * C, 0.0f);
        flcl::run(global_for(n), LOCAL, [&] {
            merge_fields(group_id, g2p.data(), fields, pfields, C, rule, nn);
        }, flcl::kSequential);
    }
    return counter;
}

// AdaptationEngine::exclusiveScan (src/adaptation/AdaptationEngine.cpp:360-415):
// scan_local (a barrier kernel, 256 items of __local memory) per group with
// block sums, then -- with more than one group -- scan_local over the block
// sums and scan_add_sums.  The block sums' own scan is one level deep, so the
// result is exact only up to 256 x 256 elements.  Returns the engine's total
// (last output + last input).
uint32_t rk_exclusive_scan(const uint32_t* in, uint32_t* out, size_t n) {
    if (n == 0) return 0;
    std::vector<uint32_t> input(in, in + n);
    size_t ngroups = (n + LOCAL - 1) / LOCAL;
    std::vector<uint32_t> sums(ngroups), sums_scanned(ngroups), temp(LOCAL);
    const uint nn = (uint)n, ng = (uint)ngroups;
    flcl::run(ngroups * LOCAL, LOCAL, [&] { scan_local(input.data(), out, sums.data(), nn, temp.data()); }, flcl::kGroupFibers);
    if (ngroups > 1) {
        flcl::run(global_for(ngroups), LOCAL, [&] {
            scan_local(sums.data(), sums_scanned.data(), nullptr, ng, temp.data());
        }, flcl::kGroupFibers);
        flcl::run(ngroups * LOCAL, LOCAL, [&] { scan_add_sums(out, sums_scanned.data(), nn); }, flcl::kSequential);
    }
    return out[n - 1] + in[n - 1];
}

typedef struct rk_adapt_stats {
    uint32_t num_children, num_groups, num_survivors, num_out;
    rk_balance_stats balance;
    uint32_t merge_table_max_displacement;
} rk_adapt_stats;

// AdaptationEngine::adapt (src/adaptation/AdaptationEngine.cpp:37-102) with the
// GPU rebuild compactAndRebuildGPU (:417-656): balance (when enabled), split,
// merge on the balanced flags, then mark_valid_cells over a merged-cell mask,
// the engine's exclusive scan, compact_cells of the survivors, append_cells of
// the children after them and of the parents after those.  The output order
// is the reference's: survivors in input order, children in split order,
// parents in group order.  Fields (AoS, C per cell): survivors are copied by
// compact_cells, parents get merge_fields' values, children get nothing --
// the rebuild appends them without fields (:560-575) -- so their rows keep
// `child_fill`.  Flags are not part of the rebuild (the caller's flag buffer is
// left as it was); *flags_after_balance receives the flags the engines used.
// Coordinates are native-level (the split/merge kernels' convention); the
// balance kernels read finest-level anchors, so they are given native << (8 -
// level), the one conversion this harness makes.  out_* sized >= 8 n.
size_t rk_adapt(const int32_t* x, const int32_t* y, const int32_t* z, const uint8_t* level, const uint8_t* state,
                const int32_t* flags_in, const uint32_t* mat, size_t n, const float* fields, uint32_t C,
                int enforce_balance, uint32_t max_balance_iters, uint32_t rule, uint32_t table_min_size,
                float child_fill,
                int32_t* ox, int32_t* oy, int32_t* oz, uint8_t* olevel, uint8_t* ostate, uint32_t* omat,
                float* ofields, int32_t* flags_after_balance, rk_adapt_stats* st) {
    std::memset(st, 0, sizeof(*st));
    std::vector<int32_t> flags(flags_in, flags_in + n);
    if (enforce_balance && n) {
        std::vector<int32_t> ax(n), ay(n), az(n);
        for (size_t i = 0; i < n; ++i) {
            int sh = 8 - level[i];
            ax[i] = x[i] << sh; ay[i] = y[i] << sh; az[i] = z[i] << sh;
        }
        rk_balance(ax.data(), ay.data(), az.data(), level, state, flags.data(), n, max_balance_iters, table_min_size,
                   &st->balance);
    }
    if (flags_after_balance) std::memcpy(flags_after_balance, flags.data(), n * 4);
    std::vector<uint32_t> cbs(n);
    std::vector<int32_t> cx(8 * n + 1), cy(8 * n + 1), cz(8 * n + 1);
    std::vector<uint8_t> cl(8 * n + 1), cs(8 * n + 1);
    std::vector<uint32_t> cm(8 * n + 1);
    std::vector<uint64_t> ch(8 * n + 1);
    uint32_t nchild = rk_split(x, y, z, level, state, flags.data(), mat, n, nullptr, 0, cbs.data(), cx.data(),
                               cy.data(), cz.data(), cl.data(), cs.data(), cm.data(), ch.data(), nullptr, nullptr);
    std::vector<uint32_t> gid(n);
    std::vector<int32_t> px(n + 1), py(n + 1), pz(n + 1);
    std::vector<uint8_t> pl(n + 1), ps(n + 1);
    std::vector<uint32_t> pm(n + 1);
    std::vector<float> pf((size_t)(n + 1) * (C ? C : 1));
    uint32_t ngroups = rk_merge(x, y, z, level, state, flags.data(), mat, n, fields, C, rule, table_min_size, 0,
                                gid.data(), px.data(),
                                py.data(), pz.data(), pl.data(), ps.data(), pm.data(), pf.data(),
                                &st->merge_table_max_displacement);
    st->num_children = nchild;
    st->num_groups = ngroups;
    if (nchild == 0 && ngroups == 0) {  // early return (:73-78): the mesh is unchanged
        for (size_t i = 0; i < n; ++i) {
            ox[i] = x[i]; oy[i] = y[i]; oz[i] = z[i]; olevel[i] = level[i]; ostate[i] = state[i]; omat[i] = mat[i];
        }
        if (fields && C && ofields) std::memcpy(ofields, fields, n * C * sizeof(float));
        st->num_survivors = st->num_out = (uint32_t)n;
        return n;
    }
    // merged-cell mask as the rebuild uploads it (:436-441): 1 for merged cells, INVALID otherwise
    std::vector<uint32_t> merge_mask(n, INV), valid(n), offs(n);
    for (size_t i = 0; i < n; ++i) if (gid[i] != INV) merge_mask[i] = 1;
    const uint nn = (uint)n;
    flcl::run(global_for(n), LOCAL, [&] {
        mark_valid_cells(flags.data(), state, merge_mask.data(), valid.data(), nn);
    }, flcl::kSequential);
    uint32_t nsurv = rk_exclusive_scan(valid.data(), offs.data(), n);
    size_t total = (size_t)nsurv + nchild + ngroups;
    if (fields && C && ofields)
        for (size_t i = 0; i < total * C; ++i) ofields[i] = child_fill;
    const uint cc = C;
    flcl::run(global_for(n), LOCAL, [&] {
        compact_cells(x, y, z, level, state, mat, (fields && ofields) ? fields : nullptr, valid.data(), offs.data(),
                      ox, oy, oz, olevel, ostate, omat, (fields && ofields) ? ofields : nullptr, nn, cc);
    }, flcl::kSequential);
    if (nchild)
        flcl::run(global_for(nchild), LOCAL, [&] {
            append_cells(cx.data(), cy.data(), cz.data(), cl.data(), cs.data(), cm.data(), nullptr, ox, oy, oz,
                         olevel, ostate, omat, nullptr, nchild, nsurv, cc);
        }, flcl::kSequential);
    if (ngroups)
        flcl::run(global_for(ngroups), LOCAL, [&] {
            append_cells(px.data(), py.data(), pz.data(), pl.data(), ps.data(), pm.data(),
                         (fields && C) ? pf.data() : nullptr, ox, oy, oz, olevel, ostate, omat,
                         (fields && ofields) ? ofields : nullptr, ngroups, nsurv + nchild, cc);
        }, flcl::kSequential);
    st->num_survivors = nsurv;
    st->num_out = (uint32_t)total;
    return total;
}

// The hash table kernels the HashTableManager would launch
// (src/core/hashmap/HashTableManager.cpp:117-159, whose launches are still
// TODO): hash_clear over the capacity, hash_build of the pairs (its per-input
// probe counts, 32 = dropped), then hash_validate of the queries (results and
// probe counts).  capacity is a power of two.
void rk_hash(const uint64_t* keys, const uint32_t* vals, size_t n, uint64_t capacity, const uint64_t* q, size_t nq,
             uint32_t* results, uint32_t* query_probes, uint32_t* build_probes) {
    std::vector<uint64_t> tk(capacity);
    std::vector<uint32_t> tv(capacity);
    flcl::run(global_for(capacity), LOCAL, [&] { hash_clear(tk.data(), tv.data(), capacity); }, flcl::kSequential);
    if (n)
        flcl::run(global_for(n), LOCAL, [&] {
            hash_build(tk.data(), tv.data(), keys, vals, capacity, (uint)n, build_probes);
        }, flcl::kSequential);
    if (nq)
        flcl::run(global_for(nq), LOCAL, [&] {
            hash_validate(tk.data(), tv.data(), capacity, q, results, query_probes, (uint)nq);
        }, flcl::kSequential);
}

// pack_fields / unpack_fields (kernels/halo_pack.cl:3-45): one float field
// into a byte buffer at a byte offset and back.
void rk_pack_unpack(const float* field, size_t n, uint64_t offset_bytes, uint8_t* packed, float* unpacked) {
    flcl::run(global_for(n), LOCAL, [&] { pack_fields(field, packed, n, offset_bytes); }, flcl::kSequential);
    flcl::run(global_for(n), LOCAL, [&] { unpack_fields(packed, unpacked, n, offset_bytes); }, flcl::kSequential);
}

}  // extern "C"
