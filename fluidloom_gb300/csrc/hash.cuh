// hash.cuh — device hash lookup, mesh/domain views and point location.
#pragma once
#include "common.cuh"
#include "keys.cuh"

// Device view of a mesh (native-level coordinates, one entry per leaf).
struct fl_mesh_dev {
    const int32_t* x;
    const int32_t* y;
    const int32_t* z;
    const uint8_t* level;
    const uint8_t* state;
    const int32_t* flags;
    const uint32_t* material;
    const uint16_t* case_id;  // may be null: one case
    size_t n;
};

// Key/anchor geometry plus per-case extent (level-0 cells) and periodicity.
struct fl_domain_dev {
    int depth;         // key levels: hilbert::encode(anchor, depth)
    int anchor_level;  // anchor = native << (anchor_level - level)
    int max_level;     // deepest level a probe may land on
    struct Case {
        int32_t ext[3];
        int32_t periodic[3];
    };
    const Case* c;     // device array indexed by case id ([0] when the mesh has none)
};

static __device__ __forceinline__ uint64_t fl_hash_slot(uint64_t key, int lg) {
    uint64_t h = key * 0x9e3779b97f4a7c15ull;
    return lg ? (h >> (64 - lg)) : 0ull;
}

// Two layouts: the API tables keep keys and values in separate arrays (tk, tv,
// HashTableManager's getKeysDevicePtr / getValuesDevicePtr); the tables the
// library builds for itself store each slot as 16 bytes -- key, value, padding
// -- so one probe reads one 32-byte sector instead of two.  tv == nullptr marks
// such a table, tk then pointing at 2 * capacity words.
// hash_query (kernels/hashmap/hash_query.cl:22-56) with the slot rule above.
static __device__ __forceinline__ uint32_t fl_hash_lookup(const uint64_t* __restrict__ tk,
                                                          const uint32_t* __restrict__ tv, int lg, uint64_t key) {
    if (key == FL_EMPTY_KEY) return FL_INVALID_INDEX;
    const uint64_t mask = (1ull << lg) - 1;
    uint64_t s = fl_hash_slot(key, lg);
    if (!tv) {
        const ulonglong2* S = reinterpret_cast<const ulonglong2*>(tk);
        for (int p = 0; p < 256; ++p) {
            const ulonglong2 w = __ldg(S + s);
            if (w.x == key) return (uint32_t)w.y;
            if (w.x == FL_EMPTY_KEY) return FL_INVALID_INDEX;
            s = (s + 1) & mask;
        }
        return FL_INVALID_INDEX;
    }
    for (int p = 0; p < 256; ++p) {
        uint64_t k = __ldg((const unsigned long long*)(tk + s));
        if (k == key) return __ldg(tv + s);
        if (k == FL_EMPTY_KEY) return FL_INVALID_INDEX;
        s = (s + 1) & mask;
    }
    return FL_INVALID_INDEX;
}

static __device__ __forceinline__ uint64_t fl_anchor_key(const uint8_t* t1, const uint16_t* t3, int depth,
                                                         uint16_t cs, bool has_case, int64_t ax, int64_t ay,
                                                         int64_t az) {
    uint64_t k = fl_hilbert_encode_dev(t1, t3, (uint32_t)ax, (uint32_t)ay, (uint32_t)az, depth);
    if (has_case) k |= (uint64_t)cs << (3 * depth);
    return k;
}

// Tables over a mesh's own cells (built with the mesh's level column) store
// level << 27 | cell index, so a probe learns the leaf's level without a
// second random read.  Meshes of such tables hold fewer than 2^27 cells.
constexpr int kPackedIdxBits = 27;
constexpr uint32_t kPackedIdxMask = (1u << kPackedIdxBits) - 1;
static __device__ __forceinline__ uint32_t fl_packed_idx(uint32_t v) {
    return v == FL_INVALID_INDEX ? FL_INVALID_INDEX : (v & kPackedIdxMask);
}
static __device__ __forceinline__ int fl_packed_level(uint32_t v) { return (int)(v >> kPackedIdxBits); }

// Point location: the leaf whose level (packed in the table value, or lv[]
// when lv is given -- the balance's shadow levels) equals l and whose anchor
// equals p with the low (A - l) bits cleared.  Levels are probed outward from
// `start`; in a valid leaf set at most one level matches, so the order does
// not change the answer, only the number of lookups.  Returns the cell index.
static __device__ __forceinline__ uint32_t fl_locate(const uint8_t* t1, const uint16_t* t3,
                                                     const uint64_t* __restrict__ tk, const uint32_t* __restrict__ tv,
                                                     int lg, const uint8_t* __restrict__ lv, const fl_domain_dev& dom,
                                                     uint16_t cs, bool has_case, const int64_t* p, int start) {
    int maxl = dom.max_level;
    if (start > maxl) start = maxl;
    if (start < 0) start = 0;
    for (int step = 0; step <= 2 * maxl + 1; ++step) {
        int off = (step + 1) >> 1;
        int l = (step & 1) ? start - off : start + off;
        if (step == 0) l = start;
        if (l < 0 || l > maxl) continue;
        int sh = dom.anchor_level - l;
        int64_t mask = ~(((int64_t)1 << sh) - 1);
        uint64_t key = fl_anchor_key(t1, t3, dom.depth, cs, has_case, p[0] & mask, p[1] & mask, p[2] & mask);
        const uint32_t v = fl_hash_lookup(tk, tv, lg, key);
        if (v == FL_INVALID_INDEX) continue;
        const uint32_t idx = v & kPackedIdxMask;
        if ((lv ? (int)lv[idx] : fl_packed_level(v)) == l) return idx;
    }
    return FL_INVALID_INDEX;
}

// Sorted point locator.  On the depth-D Hilbert curve a leaf of level l covers
// one aligned run of 8^(A-l) finest keys, starting at its anchor's key with the
// low 3(A-l) bits cleared; with the runs in ascending order, the leaf holding
// a point is the predecessor of the point's key, if the key falls inside its
// run.  Every run starts on a multiple of 8^cut (cut = A - the deepest leaf
// level), so keys are kept divided by 8^cut: the key of a point is then the
// encoding of the point shifted down by cut at depth - cut levels.  A linear
// directory over the key span (bucket b starts at the first run whose
// (start - k0) >> shift >= b) narrows the search to one bucket.  Consecutive
// threads probe neighbouring points, whose keys lie close together, so the
// reads hit L1/L2 where a hash table scatters them.
struct fl_locator {
    const uint64_t* keys;  // ascending run starts / 8^cut, case id above bit 3 * (depth - cut)
    const uint32_t* ids;   // cell of each run; nullptr: runs in mesh order
    const uint32_t* dir;   // (1 << log2nb) + 1 bucket starts
    const uint8_t* level;  // mesh levels by cell index
    size_t n;
    int log2nb;
    int cut;               // anchor_level - the deepest leaf level
};

struct fl_locator_base {
    uint64_t k0;
    int shift;
};

static __device__ __forceinline__ fl_locator_base fl_locator_base_of(const fl_locator& L) {
    fl_locator_base B{0, 0};
    if (L.n == 0) return B;
    B.k0 = __ldg((const unsigned long long*)L.keys);
    const uint64_t span = __ldg((const unsigned long long*)(L.keys + L.n - 1)) - B.k0;
    const int bits = span ? 64 - __clzll((long long)span) : 0;
    B.shift = bits > L.log2nb ? bits - L.log2nb : 0;
    return B;
}

// The leaf whose run holds key q (a point's key as above, with its case
// bits), FL_INVALID_INDEX if none or if that leaf lies below max_level; top =
// anchor_level - cut.
static __device__ __forceinline__ uint32_t fl_locate_sorted(const fl_locator& L, const fl_locator_base& B, int top,
                                                            int max_level, uint64_t q) {
    if (L.n == 0 || q < B.k0) return FL_INVALID_INDEX;
    const uint64_t nb = 1ull << L.log2nb;
    uint64_t b = (q - B.k0) >> B.shift;
    if (b >= nb) b = nb - 1;
    const uint32_t lo = __ldg(L.dir + b), hi = __ldg(L.dir + b + 1);
    uint32_t j;
    uint64_t kj = lo < hi ? __ldg((const unsigned long long*)(L.keys + lo)) : ~0ull;
    if (kj > q) {
        if (lo == 0) return FL_INVALID_INDEX;
        j = lo - 1;  // the last run of the buckets before b
        kj = __ldg((const unsigned long long*)(L.keys + j));
    } else {
        uint32_t a = lo, c = hi;  // keys[a] = kj <= q; the predecessor lies in [a, c)
        while (c - a > 1) {
            const uint32_t m = (a + c) >> 1;
            const uint64_t km = __ldg((const unsigned long long*)(L.keys + m));
            if (km <= q) { a = m; kj = km; }
            else c = m;
        }
        j = a;
    }
    const uint32_t id = L.ids ? __ldg(L.ids + j) : j;
    const int l = __ldg(L.level + id);
    if (l > max_level) return FL_INVALID_INDEX;
    const int sh = 3 * (top - l);
    const uint64_t run = sh >= 64 ? ~0ull : (1ull << sh);
    return q - kj < run ? id : FL_INVALID_INDEX;
}

// Threads of a probe block: 32 cells x 26 directions.
constexpr int kProbeThreads = 832;

// Per-kernel state of sorted-locator probes (tables in shared memory).
struct fl_probe {
    const uint8_t* t1;
    const uint16_t* t3c;
    fl_locator L;
    fl_locator_base B;
    int cut, depth_cut, top, max_level;  // L.cut, depth - cut, anchor_level - cut
};

static __device__ __forceinline__ fl_probe fl_probe_make(const uint8_t* t1, const uint16_t* t3c, const fl_locator& L,
                                                         const fl_domain_dev& dom) {
    fl_probe P{t1, t3c, L, fl_locator_base_of(L), L.cut, dom.depth - L.cut, dom.anchor_level - L.cut,
               dom.max_level};
    return P;
}

// The leaf holding point (px, py, pz) (anchor units, inside the case) of case cs.
static __device__ __forceinline__ uint32_t fl_probe_point(const fl_probe& P, bool has_case, uint16_t cs, uint32_t px,
                                                          uint32_t py, uint32_t pz) {
    uint64_t q = fl_hilbert_encode_cat(P.t1, P.t3c, px >> P.cut, py >> P.cut, pz >> P.cut, P.depth_cut);
    if (has_case) q |= (uint64_t)cs << (3 * P.depth_cut);
    return fl_locate_sorted(P.L, P.B, P.top, P.max_level, q);
}

// A probe coordinate one cell or less outside [0, n): wrapped on a periodic
// axis, false on a closed one.
static __device__ __forceinline__ bool fl_fold32(int32_t& p, int32_t n, int periodic) {
    if (p >= 0 && p < n) return true;
    if (!periodic) return false;
    while (p < 0) p += n;
    while (p >= n) p -= n;
    return true;
}

// Scratch of fl_locator_build for n cells.
size_t fl_locator_scratch_bytes(size_t n);
// Run starts of the mesh's leaves, sorted (with their cell ids) when the mesh
// is not already in key order, and the bucket directory; L points into scratch.
// level_bound >= 0: no leaf is deeper (saves a host read); in_key_order: the
// caller knows the mesh is in key order (saves the check and its host read).
int fl_locator_build(fl_ctx* ctx, const fl_mesh_dev& m, const fl_domain_dev& dom, void* scratch, fl_locator* L,
                     int level_bound = -1, bool in_key_order = false);
// The locator's run order (cell of each run in key order) inside the scratch
// that fl_locator_build carved for n cells: the identity when the mesh was
// already in key order.
uint32_t* fl_locator_ids(void* scratch, size_t n);
// nbr[(i*26 + k)*S + s] through the sorted locator; marks: n words of scratch.
int fl_neighbours_sorted(fl_ctx* ctx, const fl_mesh_dev& m, const fl_domain_dev& dom, const fl_locator& L,
                         int subslots, uint32_t* nbr, uint32_t* marks);

int fl_hash_lg(uint64_t cap);
uint64_t fl_table_capacity(size_t n);
// Clear + build; `win` is cap uint32 of scratch; tv == nullptr builds the
// 16-byte-slot layout in tk (2 * cap words).  With `levels` (and no vals) the
// values are levels[i] << 27 | i (n < 2^27, else FL_E_CAPACITY).
int fl_hash_build_with(fl_ctx* ctx, uint64_t* tk, uint32_t* tv, uint64_t cap, const uint64_t* keys,
                       const uint32_t* vals, size_t n, uint32_t* win, const uint8_t* levels = nullptr);
