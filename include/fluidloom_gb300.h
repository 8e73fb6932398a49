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
/* Host-side fault injection for failure tests (no reference counterpart; the reference's device
 * allocations throw from OpenCL wrappers, include/fluidloom/common/FluidLoomError.h:77-81): after
 * `after` more device allocations made by the library for this context, every allocation fails as
 * out of memory (the call returns FL_E_OOM) until it is switched off with after < 0.  Nothing is
 * allocated by a failed allocation; the context stays usable. */
int fl_ctx_inject_alloc_failure(fl_ctx* ctx, int64_t after);
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
/* Page-locked host memory for asynchronous copies. */
int fl_host_alloc_pinned(fl_ctx* ctx, size_t bytes, void** out);
int fl_host_free_pinned(fl_ctx* ctx, void* ptr);
/* CUDA-event timer on the context stream: start records, stop records, waits and returns ms. */
int fl_ctx_timer_start(fl_ctx* ctx);
int fl_ctx_timer_stop(fl_ctx* ctx, float* ms);
/* Kernels this context has launched so far (a replayed graph counts its kernel nodes). */
int fl_ctx_launch_count(fl_ctx* ctx, uint64_t* count);

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
/* [host] hilbert::encode / decode for one cell (HilbertCodec.h:29,40). */
uint64_t fl_hilbert_encode_host(int32_t x, int32_t y, int32_t z, uint8_t level);
void fl_hilbert_decode_host(uint64_t key, uint8_t level, int32_t* x, int32_t* y, int32_t* z);
/* [host] hilbert::getParent / getChild / isValid (HilbertCodec.h:49,59,68). */
uint64_t fl_hilbert_get_parent(uint64_t key, uint8_t level);
uint64_t fl_hilbert_get_child(uint64_t key, uint8_t level, uint8_t quadrant);
int fl_hilbert_is_valid(uint64_t key, uint8_t level);

/* ---- scan / sort / compaction */
/* Exclusive scan of uint32 (single pass, decoupled look-back), any n < 2^32.
 * Replaces AdaptationEngine::exclusiveScan (src/adaptation/AdaptationEngine.cpp:360-415).
 * total (device pointer, may be NULL) receives the sum.  in == out is allowed. */
int fl_scan_exclusive_u32(fl_ctx* ctx, const uint32_t* in, uint32_t* out, size_t n, uint32_t* total);
/* The same scan for callers that cannot allocate device memory (no counterpart in the reference):
 * embedders that own every device allocation through their own pool, hosts under a fixed device
 * memory budget, FFI hosts that must not allocate on their hot path.  No context, no
 * cudaMalloc/cudaFree or allocating library call; its scratch is a fixed array inside the library
 * (128 KiB + 512 B per GPU, held until exit), so n is limited to 2^26 (67,108,864) elements and
 * larger n returns FL_E_CAPACITY.  Runs on cuda_stream (a cudaStream_t the caller owns; NULL is
 * the legacy default stream, which orders against every blocking stream of the device) and
 * synchronizes that stream before it returns (it reads the look-back timeout word back).  The
 * first call on a device, and the first after the device's context was reset, looks up the
 * array's device address: make that first call before any stream capture.  All calls share the
 * array and each clears the words it uses, so calls that overlap on the GPU (other threads or
 * streams) race.  n == 0 sets *total (if given) to 0.  A CUDA error pending from the caller's
 * own earlier calls is left pending and not reported. */
int fl_scan_exclusive_u32_noalloc(const uint32_t* in, uint32_t* out, size_t n, uint32_t* total, void* cuda_stream);
/* Failure-detection check of the bounded device waits (no reference counterpart: the reference
 * has no device-side wait limits): one warp polls a look-back word that nothing publishes; after
 * spin_limit polls it records a timeout and exits, and the call returns FL_E_DEVICE_TIMEOUT with
 * the context still usable. */
int fl_lookback_timeout_probe(fl_ctx* ctx, uint32_t spin_limit);
/* Stable ascending LSD radix sort of (key, value) pairs in place on bits [begin_bit, end_bit).
 * Replaces RadixSort::sortByKey (include/fluidloom/core/hashmap/RadixSort.h:33-35). */
int fl_sort_pairs_u64_u32(fl_ctx* ctx, uint64_t* keys, uint32_t* vals, size_t n, int begin_bit, int end_bit);
/* The radix sort's shape for every later sort on this context (the reference fixes 8-bit digits,
 * kernels/hashmap/radix_sort.cl:5-6 BITS_PER_PASS; the tile shape has no reference counterpart):
 * digit_bits 8 (default) or 9 (ceil(bits / 9) passes instead of ceil(bits / 8)) on tiles of
 * tile_threads 256 (default) or 512 threads x 12 keys.  Every shape gives the same sorted output;
 * any other pair returns FL_E_INVALID_ARG and keeps the current shape. */
int fl_sort_set_config(fl_ctx* ctx, int digit_bits, int tile_threads);
int fl_sort_get_config(fl_ctx* ctx, int* digit_bits, int* tile_threads);
/* CompactionEngine::compactAndPermute (include/fluidloom/core/hashmap/CompactionEngine.h:43-46):
 * keep state != 0 && key != EMPTY, sort kept keys, perm[old] = new (FL_INVALID if dropped).
 * sorted_keys / sorted_ids need n entries; *num_valid is written (the call synchronizes). */
int fl_compact_and_permute(fl_ctx* ctx, const uint64_t* keys, const uint32_t* state, size_t n, uint32_t* perm,
                           uint64_t* sorted_keys, uint32_t* sorted_ids, size_t* num_valid);
/* CompactionEngine::applyPermutationToFields (CompactionEngine.h:54-59): dst[perm[i]] = src[i]. */
int fl_apply_permutation(fl_ctx* ctx, const void* src, void* dst, size_t elem_size, size_t old_n,
                         const uint32_t* perm);

/* ---- hash table (HashTableManager, include/fluidloom/core/hashmap/HashTableManager.h:34-56;
 *      kernels/hashmap/hash_build.cl, hash_query.cl) */
/* [host] HashTableManager::computeCapacity (HashTableManager.cpp:47-57). */
uint64_t fl_hash_compute_capacity(size_t n);
/* Clear and build: table_keys[capacity], table_vals[capacity]; vals may be NULL (value = input index).
 * A repeated key keeps the value of its last occurrence.  Synchronizes; FL_E_HASH_OVERFLOW if a
 * key found no slot within the probe limit. */
int fl_hash_build(fl_ctx* ctx, uint64_t* table_keys, uint32_t* table_vals, uint64_t capacity, const uint64_t* keys,
                  const uint32_t* vals, size_t n);
/* out[i] = value of queries[i] or FL_INVALID. */
int fl_hash_query(fl_ctx* ctx, const uint64_t* table_keys, const uint32_t* table_vals, uint64_t capacity,
                  const uint64_t* queries, uint32_t* out, size_t n);

/* ---- AMR mesh and regrid */
/* Device columns of a leaf set, native-level coordinates (CellDescriptor.h:32-104 split into SoA,
 * as AdaptationEngine::adapt takes them, AdaptationEngine.h:56-65). */
typedef struct fl_mesh {
    int32_t* x;
    int32_t* y;
    int32_t* z;
    uint8_t* level;
    uint8_t* state;      /* CellState: 0 FLUID, 1 SOLID, ... (CellDescriptor.h:107-114) */
    int32_t* flags;      /* refine flags: > 0 split, -1 merge, 0 keep */
    uint32_t* material;
    uint16_t* case_id;   /* NULL for a single case */
    size_t num_cells;
    size_t capacity;
} fl_mesh;

/* AdaptationConfig (include/fluidloom/adaptation/AdaptationTypes.h:117-157) plus key geometry. */
typedef struct fl_adapt_config {
    uint8_t max_refinement_level;   /* <= 21 */
    uint8_t min_refinement_level;
    uint32_t max_balance_iterations;
    int32_t enforce_2_1_balance;
    int32_t balance_mode;           /* 0 FACE6 (reference semantics), 1 FULL26 to a fixed point */
    int32_t averaging_rule;         /* 0 arithmetic, 1 volume weighted */
    double buffer_growth_factor;
    int32_t key_depth;              /* 0 -> 21 */
    int32_t anchor_level;           /* 0 -> 21: anchor = native << (anchor_level - level) */
    int32_t ext[3];                 /* level-0 extent in cells (0 -> 1) */
    int32_t periodic[3];
    int32_t input_balanced;         /* no reference counterpart; 1: the caller states that no two touching
                                       leaves of the input differ by more than one level (faces, edges,
                                       corners), as after an adapt whose FULL26 balance converged.  The
                                       first FULL26 round then probes only from the leaves that will split,
                                       the only ones that can find a violation in such a mesh; results
                                       equal those with 0 (every leaf probes) whenever the statement holds */
} fl_adapt_config;

/* BalanceResult (AdaptationTypes.h:94-109). */
typedef struct fl_balance_result {
    int32_t converged;
    uint32_t iterations;
    uint32_t total_violations_detected;
    uint32_t total_cells_marked_for_balance;
} fl_balance_result;

/* SplitResult / MergeResult counts (AdaptationTypes.h:27-87). */
typedef struct fl_adapt_stats {
    uint32_t num_split;
    uint32_t num_children;
    uint32_t num_groups;
    uint32_t num_merged;
    uint32_t num_survivors;
    size_t num_cells_out;
    fl_balance_result balance;
} fl_adapt_stats;

int fl_mesh_alloc(fl_ctx* ctx, size_t capacity, int with_case_id, fl_mesh* mesh);
int fl_mesh_free(fl_ctx* ctx, fl_mesh* mesh);
/* BalanceEnforcer::enforce (include/fluidloom/adaptation/BalanceEnforcer.h:48-53): updates flags.
 * Returns FL_E_BALANCE_NOT_CONVERGED (warning) when it stops without converging. */
int fl_balance_enforce(fl_ctx* ctx, fl_mesh* mesh, const fl_adapt_config* cfg, fl_balance_result* res);
/* AdaptationEngine::adapt (AdaptationEngine.h:56-65): balance, split, merge, rebuild in key order.
 * The mesh columns (and *fields, AoS with C floats per cell) are replaced by new allocations when
 * the cell set changes capacity, as the reference releases and replaces its cl_mem handles. */
int fl_adapt(fl_ctx* ctx, fl_mesh* mesh, const fl_adapt_config* cfg, float** fields, uint32_t C,
             fl_adapt_stats* stats);
/* SplitEngine::split (include/fluidloom/adaptation/SplitEngine.h:51-59): children of every cell with
 * flag > 0, FLUID state and level < max (split_cells.cl:31-33), in parent order, 8 per parent
 * (child bit 0 = x, 1 = y, 2 = z); child fields (AoS, C per cell, may be NULL) copied from the parent;
 * parent_to_child[i] = first child index or FL_INVALID (may be NULL).  FL_E_CAPACITY with the
 * count in *num_children when children->capacity is too small.  Synchronizes. */
int fl_split(fl_ctx* ctx, const fl_mesh* mesh, const fl_adapt_config* cfg, const float* fields, uint32_t C,
             fl_mesh* children, float* child_fields, uint32_t* parent_to_child, size_t* num_children);
/* MergeEngine::merge (include/fluidloom/adaptation/MergeEngine.h:51-59): complete sibling octets
 * with flag -1, FLUID, same level, above min level (merge_cells.cl:11-106), numbered in first-sibling
 * order; parents (level - 1) with fields summed over children 0..7 in order, x0.125 for the arithmetic
 * rule (FieldAveragingRules.h:31-52); merge_group_id[i] = group or FL_INVALID (may be NULL).
 * Synchronizes. */
int fl_merge(fl_ctx* ctx, const fl_mesh* mesh, const fl_adapt_config* cfg, const float* fields, uint32_t C,
             fl_mesh* parents, float* parent_fields, uint32_t* merge_group_id, size_t* num_parents);
/* Neighbour table: nbr[(i*26 + k)*subslots + s] = leaf containing the probe point of direction k
 * (dz outer, dy, dx inner, centre skipped) at sub-slot s, FL_INVALID outside the domain
 * (point-location rule of src/adaptation/kernels/balance_enforce.cl:107-143).  subslots 1 or 4. */
int fl_neighbour_rebuild(fl_ctx* ctx, const fl_mesh* mesh, const fl_adapt_config* cfg, int subslots, uint32_t* nbr);

/* ---- fields: descriptor, registry, structure-of-arrays manager */
/* FieldDescriptor (include/fluidloom/core/fields/FieldDescriptor.h:40-83).  type: 0 FLOAT32, 1 FLOAT64,
 * 2 INT32, 3 INT64, 4 UINT8; avg_rule and solid_scheme as the reference enums. */
typedef struct fl_field_desc {
    char name[72];          /* 1..64 characters, NUL-terminated */
    int32_t type;
    uint16_t num_components; /* 1..32 */
    uint8_t halo_depth;     /* 0..2 */
    uint8_t avg_rule;
    uint8_t solid_scheme;
    uint8_t reserved[7];
    uint64_t id;            /* FNV-1a 64 of the name (include/fluidloom/common/Hash.h:13-22) */
} fl_field_desc;

/* [host] hash::fnv1a_64 and FieldDescriptor's constructor checks (FieldDescriptor.cpp:8-43). */
uint64_t fl_fnv1a_64(const char* s);
int fl_field_make(const char* name, int32_t type, uint16_t components, uint8_t halo_depth, uint8_t avg_rule,
                  uint8_t solid_scheme, fl_field_desc* out);
size_t fl_field_bytes_per_cell(const fl_field_desc* desc);
/* [host] FieldRegistry::instance() (src/core/registry/FieldRegistry.cpp:7-66): register returns
 * FL_E_CAPACITY when the name exists (the reference's false). */
int fl_field_register(const fl_field_desc* desc);
int fl_field_lookup_name(const char* name, fl_field_desc* out);
int fl_field_lookup_id(uint64_t id, fl_field_desc* out);
size_t fl_field_registry_count(void);
void fl_field_registry_clear(void);
/* SOAFieldManager (include/fluidloom/core/fields/SOAFieldManager.h:26-51), per context:
 * component-major device storage with a 128-byte aligned pitch; handle = field id. */
int fl_soa_allocate(fl_ctx* ctx, const fl_field_desc* desc, size_t num_cells, uint64_t* handle);
int fl_soa_resize(fl_ctx* ctx, uint64_t handle, size_t new_num_cells);
int fl_soa_deallocate(fl_ctx* ctx, uint64_t handle);
int fl_soa_device_ptr(fl_ctx* ctx, uint64_t handle, uint16_t component, void** out);
int fl_soa_info(fl_ctx* ctx, uint64_t handle, size_t* num_cells, size_t* pitch_bytes, uint64_t* version);
size_t fl_soa_total_bytes(fl_ctx* ctx);

/* ---- same-GPU ghost pack / unpack, interpolation, restriction (fields AoS, C floats per cell) */
/* pack_fields / unpack_fields (kernels/halo_pack.cl:3-45): float field <-> byte buffer at a byte offset. */
int fl_pack_fields(fl_ctx* ctx, const float* field, void* packed, size_t num_cells, size_t field_offset_bytes);
int fl_unpack_fields(fl_ctx* ctx, const void* packed, float* field, size_t num_cells, size_t field_offset_bytes);
/* pack_halo direct copy (kernels/halo/pack.cl:8-52): pack[k*C + c] = field[cell_indices[k]*C + c]. */
int fl_pack_halo(fl_ctx* ctx, const float* field, uint32_t C, const uint32_t* cell_indices, size_t n, float* pack);
/* unpack_halo with pre-averaged values (kernels/halo/unpack.cl, interpolate_average.cl:12-32). */
int fl_unpack_halo(fl_ctx* ctx, const float* pack, uint32_t C, const uint32_t* cell_indices, size_t n, float* field);
/* trilinear_interpolate (kernels/halo/interpolate_trilinear.cl:12-56, default weights
 * InterpolationParams.h:34-43) for nq fine cells (native coords + level): the 8 cells at the coarser
 * level around fine / 2, 0.125 each, missing ones contribute nothing.  Single-case meshes, C <= 32. */
int fl_interp_trilinear(fl_ctx* ctx, const fl_mesh* mesh, const fl_adapt_config* cfg, const float* field, uint32_t C,
                        const int32_t* fx, const int32_t* fy, const int32_t* fz, const uint8_t* flevel, size_t nq,
                        float* out);
/* Restriction of sibling groups members[g][8] (merge_fields, merge_cells.cl:123-159): children 0..7
 * summed in order, x0.125 for rule 0 (arithmetic), unscaled for rule 1 (volume weighted). */
int fl_restrict_groups(fl_ctx* ctx, const float* field, uint32_t C, const uint32_t* members, size_t ngroups, int rule,
                       float* out);

/* Refine/coarsen flags from a sum of Gaussian blobs over the unit cube (the flag source of the
 * regrid microbenchmark; the reference's flags come from DSL loops, benchmarks/lid_driven_cavity.fl:37-45).
 * blobs: nblobs x {cx, cy, cz, 1/(2 sigma^2), amplitude} (host); flag 1 above hi (below max_level),
 * -1 below lo, else 0.  Cell centres are (native + 0.5) / 2^level (single level-0 cell). */
int fl_flags_from_blobs(fl_ctx* ctx, fl_mesh* mesh, const float* blobs, int nblobs, float lo, float hi, int max_level);

/* ---- D3Q19 BGK collide-stream over an octree of 8^3-site bricks.
 * The reference emits empty lbm_* kernels (src/parsing/SimulationBuilder.cpp:394-400) behind
 * KernelNode (include/fluidloom/runtime/nodes/KernelNode.h:46-72) and stores fields through
 * SOAFieldManager (include/fluidloom/core/fields/SOAFieldManager.h:26-51); a pool owns the
 * leaves of one or more independent cases (a "cell" of the AMR API is one brick here), their
 * 19-component FP32 populations in SoA layout, the neighbour table and the per-level lists. */
typedef struct fl_lbm_case {
    int32_t ext[3];        /* level-0 bricks per axis (1..16); a brick is 8^3 sites */
    int32_t bc[6];         /* faces -x,+x,-y,+y,-z,+z: 0 periodic, 1 wall, 2 moving wall, 3 inlet, 4 outlet */
    float wall_u[3];       /* moving-wall velocity */
    float inlet_u[3];      /* inlet velocity */
    float tau0;            /* relaxation time at level 0 */
    int32_t max_level;     /* 0..13 */
    int32_t has_sphere;
    float sphere_c[3];     /* centre, level-0 site units */
    float sphere_r;        /* radius, level-0 site units */
    float refine_frac;     /* refine a brick whose max |vorticity| exceeds this fraction of the case max */
    float coarsen_frac;    /* coarsen below this fraction */
    float band;            /* bricks within this distance of the sphere surface refine to max_level */
    float init_u[3];       /* initial velocity (density 1) */
} fl_lbm_case;

typedef struct fl_pool fl_pool;

typedef struct fl_pool_info {
    size_t num_bricks;
    size_t capacity;
    int32_t num_cases;
    int32_t max_level;
    uint32_t bricks_per_level[16];
    uint64_t fluid_lups_per_step;   /* fluid site updates per level-0 step: sum of 2^level */
    uint64_t population_bytes;
    uint64_t fluid_sites_per_level[16];
    int32_t num_active_cases;       /* num_cases counts slots, including freed ones */
    int32_t usable;                 /* 0 after a call failed part-way through replacing the pool's bricks or
                                       tables: every call but fl_pool_destroy and this one then returns
                                       FL_E_INVALID_ARG without touching the device */
    uint32_t general_bricks_per_level[16];         /* bricks with stencil descriptors (interface, boundary,
                                                      near the sphere) */
    uint64_t stencil_descriptors_per_level[16];    /* elements whose source is not a plain same-level load */
} fl_pool_info;

/* Build the cases: level-0 bricks, max_level rounds of sphere-band refinement, equilibrium start. */
int fl_pool_create(fl_ctx* ctx, const fl_lbm_case* cases, int ncases, fl_pool** out);
int fl_pool_destroy(fl_ctx* ctx, fl_pool* pool);
/* Advance every case by nsteps level-0 steps (levels sub-cycled), asynchronously. */
int fl_pool_step(fl_ctx* ctx, fl_pool* pool, int nsteps);
/* Regrid all cases: vorticity/band flags, FULL26 adapt, population remap, neighbour rebuild
 * (the AdaptMeshNode::execute path, src/runtime/nodes/AdaptMeshNode.cpp:9-64). */
int fl_pool_regrid(fl_ctx* ctx, fl_pool* pool, fl_adapt_stats* stats);
int fl_pool_info_get(fl_ctx* ctx, fl_pool* pool, fl_pool_info* info);
/* Host copies of the bricks and (f != NULL) the current populations as [19][n][512]. */
int fl_pool_download(fl_ctx* ctx, fl_pool* pool, int32_t* x, int32_t* y, int32_t* z, uint8_t* level,
                     uint16_t* case_id, float* f);
int fl_pool_nbr(fl_ctx* ctx, fl_pool* pool, uint32_t* nbr);
/* Refinement flags and per-brick max |vorticity| of the current state (host outputs). */
int fl_pool_flags(fl_ctx* ctx, fl_pool* pool, int32_t* flags, float* wmax);
/* Per case: fluid mass and momentum (FP64, sites weighted by 8^-level) -> out[ncases][4] (host). */
int fl_pool_conservation(fl_ctx* ctx, fl_pool* pool, double* out);
/* The same sums enqueued on the context stream without waiting: out (ncases x 4 doubles, pinned
 * host memory or device memory for the call not to block) holds them once the stream has reached
 * this point (fl_ctx_synchronize, or any later call that synchronises).  Device-side status is
 * collected by the next call that synchronises. */
int fl_pool_conservation_async(fl_ctx* ctx, fl_pool* pool, double* out);
/* on != 0: every level-0 step also writes the conservation sums of the state it leaves (each
 * level's last sub-step sums the values it stores, in the arithmetic of the separate pass), so a
 * conservation call after a step reads no populations; for callers that read the sums every step.
 * Off (the default) the steps carry no extra work and a conservation call reads the populations.
 * Results are identical either way.  Ignored (stays off) once the populations were exported as a
 * field (fl_pool_populations_field), whose writes the pool cannot see. */
int fl_pool_set_step_sums(fl_ctx* ctx, fl_pool* pool, int on);
/* Advance nsteps with a CUDA event pair around every collide-stream launch (no graphs); returns,
 * per kernel ([0] interior bricks, [1] interface/boundary/near-sphere bricks, [2] all-solid bricks),
 * the summed kernel time, the launch count and the fluid sites those launches updated (each output
 * an array of 3). */
int fl_pool_profile_steps(fl_ctx* ctx, fl_pool* pool, int nsteps, double* kernel_ms, uint32_t* launches,
                          uint64_t* fluid_sites);
/* The same timing pass, totals per level and kernel: kernel_ms, launches and fluid_sites are arrays
 * of 16 x 3 ([level][kernel], kernels as above).  A launch of kernel 1 covers the level's
 * descriptor values (k_interface) and its general bricks. */
int fl_pool_profile_levels(fl_ctx* ctx, fl_pool* pool, int nsteps, double* kernel_ms, uint32_t* launches,
                           uint64_t* fluid_sites);
/* Replace the populations with a host array [19][n][512] (the layout fl_pool_download gives). */
int fl_pool_upload(fl_ctx* ctx, fl_pool* pool, const float* f);
/* Density and velocity of every site ([nbricks][512] host arrays each, bricks in pool order),
 * computed on the device from the current populations; sites inside the sphere report 0.
 * Replaces reading back the reference's density/velocity fields (SOAFieldManager::getDevicePtr,
 * src/core/fields/SOAFieldManager.cpp:140-160) for output. */
int fl_pool_macroscopic(fl_ctx* ctx, fl_pool* pool, float* rho, float* ux, float* uy, float* uz);
/* Replace the pool's bricks and populations by a saved state (bricks of active cases, any order;
 * f is [19][n][512]): the pool continues exactly as the pool the state came from.  Snapshot /
 * restart (the reference keeps only placeholders for it, tests/restart/checkpoint_restart_test.cpp:17-60). */
int fl_pool_load(fl_ctx* ctx, fl_pool* pool, size_t n, const int32_t* x, const int32_t* y, const int32_t* z,
                 const uint8_t* level, const uint16_t* case_id, const float* f);
/* Per-case moving-wall and inlet velocities ([ncases][3] host arrays, either may be NULL),
 * copied on the stream and used from the next step on. */
int fl_pool_set_velocities(fl_ctx* ctx, fl_pool* pool, const float* wall_u, const float* inlet_u);
/* Solid voxels of one case, OR-ed with its sphere: bit (z * Ny + y) * Nx + x of `bits` (host,
 * nwords = ceil(Nx * Ny * Nz / 32), N = ext * 8 << level) marks voxel (x, y, z) of the case's grid
 * at `level`.  A site of level l samples the voxel under its centre (the upper middle voxel
 * when l < level).  bits == NULL removes the mask.  Classes, descriptors and fluid counts are
 * rebuilt; populations are unchanged (solid sites take the rest state at the next step), and the
 * next regrid refines bricks holding both solid and fluid sites (their own or in a one-site
 * halo) to max_level.  Uploads the solid cells the reference's builder generates from its
 * geometries but leaves on the host (src/parsing/SimulationBuilder.cpp:112-126). */
int fl_pool_set_solid_mask(fl_ctx* ctx, fl_pool* pool, int32_t case_id, int32_t level, const uint32_t* bits,
                           size_t nwords);
/* The same from n solid cells given as DEVICE columns x, y, z of the level-`level` grid, e.g.
 * the cells fl_geometry_process gives for a geometry written in level-`level` voxel units with
 * cell_size 1; cells outside the case grid are ignored. */
int fl_pool_set_solid_cells(fl_ctx* ctx, fl_pool* pool, int32_t case_id, int32_t level, const int32_t* x,
                            const int32_t* y, const int32_t* z, size_t n);
/* The case's mask level (-1: none) and, when bits != NULL, its words (nwords at least the mask's). */
int fl_pool_get_solid_mask(fl_ctx* ctx, fl_pool* pool, int32_t case_id, int32_t* level, uint32_t* bits, size_t nwords);
/* Regrid with caller-given flags (one int32 per brick in pool order: > 0 split, -1 merge, 0 keep),
 * 2:1 balanced like every regrid: the refine_flags buffer AdaptMeshNode passes to the
 * reference's adapt (src/runtime/nodes/AdaptMeshNode.cpp:52-63). */
int fl_pool_regrid_flags(fl_ctx* ctx, fl_pool* pool, const int32_t* flags, fl_adapt_stats* stats);
/* Regrid only the cases whose due[case id] is non-zero (host array of num_cases bytes); the other
 * cases come out unchanged. */
int fl_pool_regrid_cases(fl_ctx* ctx, fl_pool* pool, const uint8_t* due, fl_adapt_stats* stats);
/* Merge new cases into a running pool at a step boundary: each starts exactly as fl_pool_create
 * would start it alone; ids[i] receives its case id (freed ids are reused). */
int fl_pool_add_cases(fl_ctx* ctx, fl_pool* pool, const fl_lbm_case* cases, int ncases, int32_t* ids);
/* Remove finished cases at a step boundary (their bricks are compacted away). */
int fl_pool_remove_cases(fl_ctx* ctx, fl_pool* pool, const int32_t* ids, int nids);
/* Host copies of one case's bricks and populations ([19][nbricks][512]); any pointer may be NULL
 * except nbricks.  Call with f == NULL first to learn nbricks. */
int fl_pool_download_case(fl_ctx* ctx, fl_pool* pool, int32_t id, int32_t* x, int32_t* y, int32_t* z,
                          uint8_t* level, float* f, size_t* nbricks);
/* The pool's populations as a 19-component FP32 field of this context's structure-of-arrays manager,
 * as the reference allocates them (SOAFieldManager::allocate, src/core/fields/SOAFieldManager.cpp:17-131)
 * and binds them to its LBM kernel nodes (KernelNode::bindField, src/runtime/nodes/KernelNode.cpp:27-29):
 * cell = brick * 512 + site over the pool's bricks in order, component q = population q;
 * fl_soa_device_ptr(handle, q) gives its device pointer and fl_soa_info its pitch (capacity * 512
 * floats).  The field is a view of the pool's current population buffer, not a copy: writes through
 * it change the pool.  It stays valid until the next call that steps, regrids, loads, adds or removes
 * cases; call again to refresh it (the handle stays, its version grows when the storage moved). */
int fl_pool_populations_field(fl_ctx* ctx, fl_pool* pool, const char* name, uint64_t* handle);
/* use_graphs: replay captured CUDA graphs per level-0 step; grid_mult: CTAs per SM (0 keeps). */
int fl_pool_set_options(fl_ctx* ctx, fl_pool* pool, int use_graphs, int grid_mult);
/* How the collide-stream kernels read a brick's own populations: 0 (default) straight into
 * registers with 128-bit loads; 1 its 19 population planes bulk-copied into shared memory by the
 * TMA engine (cp.async.bulk on an mbarrier), one brick ahead of the one being relaxed; 2 as 1,
 * with the general bricks' quad masks and stencil-descriptor values staged the same way.
 * Results are identical in every mode. */
int fl_pool_set_staging(fl_ctx* ctx, fl_pool* pool, int mode);
/* streams = 2 (default): each level-0 step runs as a dependency graph over two streams per
 * level -- general, interface and all-solid bricks on one, interior bricks on the other --
 * joined by events (coarse and fine sources are always interface bricks, so only the
 * general launches of neighbouring levels wait on each other); the graph is forked from and
 * joined back into the context stream and captured like the rest of the step.
 * streams = 1: every launch in order on the context stream. */
int fl_pool_set_class_streams(fl_ctx* ctx, fl_pool* pool, int streams);

/* ---- Geometry placement ----
 * Replaces src/geometry: GeometryDescriptor (include/fluidloom/geometry/GeometryDescriptor.h:19-113),
 * ImplicitEvaluator::isInside / evaluate (implicit/ImplicitEvaluator.cpp:8-98), SimpleSTLVoxelizer::voxelize
 * (voxelizer/SimpleSTLVoxelizer.cpp:119-247) and GeometryPlacer::processGeometry
 * (placer/GeometryPlacer.cpp:55-118).  Types in GeometryDescriptor::Type order; rotation is carried
 * but, as in the reference, not applied. */
enum { FL_GEOM_STL = 0, FL_GEOM_IMPLICIT = 1, FL_GEOM_BOX = 2, FL_GEOM_SPHERE = 3, FL_GEOM_CYLINDER = 4 };
typedef struct fl_geometry_desc {
    int32_t type;
    int32_t material_id;
    float translate[3];
    float scale[3];       /* > 0 */
    float rotate[3];      /* degrees; not applied */
    float radius, height, width, length;
} fl_geometry_desc;
/* computeTransformedAABB: box6 = min xyz, max xyz. */
int fl_geometry_aabb(const fl_geometry_desc* geom, float* box6);
/* isInside at n points (device float arrays), inside[i] = 0/1 (device). */
int fl_geometry_inside(fl_ctx* ctx, const fl_geometry_desc* geom, const float* x, const float* y, const float* z,
                       size_t n, uint8_t* inside);
/* ImplicitEvaluator::evaluate: cells (device int32 arrays) tested at their centres coord + 0.5. */
int fl_geometry_evaluate(fl_ctx* ctx, const fl_geometry_desc* geom, const int32_t* x, const int32_t* y,
                         const int32_t* z, size_t n, uint8_t* inside);
/* SimpleSTLVoxelizer::voxelize of a triangle mesh (host array [ntri][9]: v1, v2, v3): the cells of the
 * inclusive grid range of the transformed mesh bounds whose centre lies inside (+x ray casting), in
 * z, y, x order, into device arrays of cap entries; count = cells found (FL_E_CAPACITY if > cap). */
int fl_stl_voxelize(fl_ctx* ctx, const float* triangles, size_t ntri, const fl_geometry_desc* geom, float cell_size,
                    int32_t* x, int32_t* y, int32_t* z, size_t cap, size_t* count);
/* GeometryPlacer::processGeometry: STL -> fl_stl_voxelize; implicit -> candidates of the transformed AABB
 * clipped to domain_box6 ([floor, ceil) cells) evaluated at their centres; material[] = material_id and
 * key[] = hilbert::encode(x, y, z) at level 8 (any output may be NULL except x, y, z). */
int fl_geometry_process(fl_ctx* ctx, const fl_geometry_desc* geom, const float* triangles, size_t ntri,
                        float cell_size, const float* domain_box6, int32_t* x, int32_t* y, int32_t* z,
                        int32_t* material, uint64_t* key, size_t cap, size_t* count);

/* ---- Execution graph ----
 * Replaces the reference runtime: ExecutionNode (include/fluidloom/runtime/nodes/ExecutionNode.h:37-169,
 * read/write field sets, AMR level, halo depth), HazardAnalyzer::analyzeNodes/enforceHazards
 * (src/runtime/dependency/HazardAnalyzer.cpp:8-136), DependencyGraph (DependencyGraphBuilder.cpp:12-131:
 * Kahn's order, cycles rejected) and TopologicalScheduler::execute (TopologicalScheduler.cpp:16-71).
 * Node kinds follow ExecutionNode::NodeType (KERNEL, HALO_EXCHANGE, BARRIER, ADAPT_MESH) plus the
 * lattice-Boltzmann step of a pool (the reference's generated lbm_* KernelNodes) and host callbacks. */
typedef struct fl_graph fl_graph;
enum {
    FL_NODE_KERNEL = 0,        /* fn(ctx, stream, user) enqueues asynchronous work on `stream` */
    FL_NODE_HALO_EXCHANGE = 1, /* one GPU: ordering only (coarse/fine coupling is inside the step) */
    FL_NODE_BARRIER = 2,       /* ordering only */
    FL_NODE_ADAPT_MESH = 3,    /* fl_pool_regrid(pool): waits on the host, splits capture segments */
    FL_NODE_LBM_STEP = 4,      /* fl_pool_step(pool, nsteps) */
    FL_NODE_HOST = 5           /* host_fn(user) in stream order */
};
enum { FL_HAZARD_RAW = 0, FL_HAZARD_WAW = 1, FL_HAZARD_WAR = 2, FL_HAZARD_LEVEL_BARRIER = 3 };
typedef int (*fl_node_fn)(fl_ctx* ctx, void* stream, void* user);
typedef void (*fl_host_fn)(void* user);
typedef struct fl_node_desc {
    int32_t type;
    char name[64];
    int32_t level;       /* AMR level, -1 = none (ExecutionNode::amr_level) */
    int32_t halo_depth;
    const char* reads;   /* comma-separated field names, may be NULL (copied) */
    const char* writes;
    fl_node_fn fn;
    fl_host_fn host_fn;
    void* user;
    fl_pool* pool;
    int32_t nsteps;
} fl_node_desc;
typedef struct fl_hazard {
    uint64_t from, to;   /* node ids (insertion order), from < to */
    int32_t type;        /* FL_HAZARD_* */
    char field[68];
} fl_hazard;
/* ctx may be NULL for a graph that is only analysed and ordered, never executed. */
int fl_graph_create(fl_ctx* ctx, fl_graph** out);
int fl_graph_destroy(fl_graph* graph);
const char* fl_graph_last_error(fl_graph* graph);
/* ids are 0, 1, 2, ... in insertion order (DependencyGraphBuilder assigns them the same way). */
int fl_graph_add_node(fl_graph* graph, const fl_node_desc* desc, int64_t* id);
/* An explicit edge (ExecutionNode::addSuccessor / addPredecessor). */
int fl_graph_add_edge(fl_graph* graph, int64_t from, int64_t to);
/* HazardAnalyzer::analyzeNodes + enforceHazards: every RAW, then WAW, WAR and level-barrier pair
 * (i < j in insertion order) becomes one edge i -> j; count = hazards found, out[] the first cap. */
int fl_graph_analyze(fl_graph* graph, fl_hazard* out, size_t cap, size_t* count);
/* The hazards the last fl_graph_analyze found (n = their number, out[] the first cap). */
int fl_graph_hazards(fl_graph* graph, fl_hazard* out, size_t cap, size_t* n);
/* Topological order (Kahn, FIFO ready queue); FL_E_INVALID_ARG "Dependency graph contains cycles". */
int fl_graph_build(fl_graph* graph);
int fl_graph_order(fl_graph* graph, int64_t* ids, size_t cap, size_t* n);
int fl_graph_num_edges(fl_graph* graph, size_t* n);
/* Runs every node once in dependency order on up to 8 streams joined by events, forked from and
 * joined into the context stream.  use_cuda_graphs: each stretch between ADAPT_MESH nodes is
 * captured once and replayed while the pools it steps keep their topology and level-0 parity. */
int fl_graph_execute(fl_graph* graph, int use_cuda_graphs);
/* Per-node execution count and total time (CUDA events) while profiling is on (eager runs). */
int fl_graph_set_profiling(fl_graph* graph, int on);
int fl_graph_node_stats(fl_graph* graph, int64_t id, uint64_t* count, double* total_ms);
/* Graphviz text of the graph (ExecutionNode::toDOT); len = full length, buf gets up to cap - 1. */
int fl_graph_dot(fl_graph* graph, char* buf, size_t cap, size_t* len);

#ifdef __cplusplus
}
#endif
#endif
