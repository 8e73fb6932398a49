/* oracle.h — CPU oracle for the fluidloom_gb300 hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library, and only as
 * the checker or the timed CPU baseline.  The product (fluidloom_gb300) never
 * links, loads or calls it.
 *
 * Every routine restates the reference algorithm it follows (cited file:line,
 * paths relative to the fedres/fluidloom tree) or, where the reference is
 * broken or nondeterministic, its intended semantics (the deviation is named
 * at the routine).  The D3Q19 collide-stream has no reference implementation
 * (its kernels are generated empty, src/parsing/SimulationBuilder.cpp:394-400),
 * so that part is a from-the-literature restatement and its parity is
 * UNPINNED by the reference; everything else is pinned against the reference's
 * own codec (compiled in place) and its unit-test known answers.
 */
#ifndef FLUIDLOOM_ORACLE_H
#define FLUIDLOOM_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- keys (src/core/hilbert/HilbertCodec.cpp, src/adaptation/utils/HilbertCodec3D.cpp) */
uint64_t or_hilbert_encode1(int32_t x, int32_t y, int32_t z, uint8_t level);
void or_hilbert_encode(const int32_t* x, const int32_t* y, const int32_t* z, uint8_t level,
                       uint64_t* keys, uint32_t* ids, size_t n);
void or_hilbert_decode(const uint64_t* keys, uint8_t level, int32_t* x, int32_t* y, int32_t* z, size_t n);
void or_morton8_encode(const int32_t* x, const int32_t* y, const int32_t* z, uint64_t* keys, size_t n);
void or_cell_keys(const int32_t* x, const int32_t* y, const int32_t* z, const uint8_t* level,
                  const uint16_t* case_id, int depth, int anchor_level, uint64_t* keys, size_t n);

/* ---- primitives */
void or_sort_pairs_u64_u32(uint64_t* keys, uint32_t* vals, size_t n);
uint32_t or_scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n);
size_t or_compact_and_permute(const uint64_t* keys, const uint32_t* state, size_t n, uint32_t* perm);
void or_apply_permutation(const void* src, void* dst, size_t elem, size_t old_n, const uint32_t* perm);
uint64_t or_hash_capacity(size_t n);
int or_hash_build(const uint64_t* keys, const uint32_t* vals, size_t n, uint64_t capacity,
                  uint64_t* table_keys, uint32_t* table_vals);
void or_hash_query(const uint64_t* table_keys, const uint32_t* table_vals, uint64_t capacity,
                   const uint64_t* q, uint32_t* out, size_t n);

/* ---- AMR mesh (native-level coordinates) */
typedef struct or_mesh {
    int32_t* x; int32_t* y; int32_t* z;
    uint8_t* level; uint8_t* state; int32_t* flags; uint32_t* material;
    uint16_t* case_id;          /* may be NULL (single case) */
    size_t n;
} or_mesh;

typedef struct or_domain {
    int depth;                  /* key levels D: hilbert::encode(anchor, D), 3*D key bits */
    int anchor_level;           /* A: anchor = native << (A - level); levels <= A */
    int max_level;              /* deepest level a probe may land on (<= A) */
    int32_t ext[3];             /* extent in level-0 cells per axis (ext << A <= 2^D) */
    int32_t periodic[3];
} or_domain;

void or_neighbours(const or_mesh* m, const or_domain* dom, int subslots, uint32_t* nbr);

typedef struct or_balance_stats {
    int32_t converged; uint32_t iterations; uint32_t violations; uint32_t marked;
    uint32_t per_iter_violations[64]; uint32_t per_iter_marked[64];
} or_balance_stats;

int or_balance(or_mesh* m, const or_domain* dom, int mode, int max_level, int max_iters,
               or_balance_stats* st);

typedef struct or_adapt_cfg {
    int max_level, min_level, balance_mode, max_balance_iterations, enforce_balance;
    int averaging_rule;          /* 0 arithmetic, 1 volume weighted */
} or_adapt_cfg;

typedef struct or_adapt_stats {
    uint32_t num_split, num_children, num_groups, num_merged, num_survivors, num_out;
    or_balance_stats balance;
} or_adapt_stats;

/* out_* arrays sized >= returned count (upper bound n*8).  fields: AoS, C per cell. */
size_t or_adapt(or_mesh* m, const or_domain* dom, const or_adapt_cfg* cfg,
                const float* fields, uint32_t C, int sites_mode,
                int32_t* ox, int32_t* oy, int32_t* oz, uint8_t* olevel, uint8_t* ostate,
                int32_t* oflags, uint32_t* omat, uint16_t* ocase, float* ofields,
                uint32_t* osrc, uint8_t* okind, uint32_t* omembers, or_adapt_stats* st);

void or_interp_trilinear(const or_mesh* m, const or_domain* dom, const float* fields, uint32_t C,
                         const int32_t* fx, const int32_t* fy, const int32_t* fz, const uint8_t* flevel,
                         size_t nq, float* out);
void or_restrict_groups(const float* fields, uint32_t C, const uint32_t* members, size_t ngroups,
                        int rule, float* out);

/* ---- D3Q19 brick pool (no reference implementation: parity unpinned) */
typedef struct or_lbm_case {
    int32_t ext[3]; int32_t bc[6];
    float wall_u[3]; float inlet_u[3];
    float tau0; int32_t max_level;
    int32_t has_sphere; float sphere_c[3]; float sphere_r;
    float refine_frac, coarsen_frac, band;
    float init_u[3];
} or_lbm_case;

void or_blob_flags(const int32_t* x, const int32_t* y, const int32_t* z, const uint8_t* level, size_t n,
                   const float* blobs, int nblobs, float lo, float hi, int max_level, int32_t* flags);

/* Opaque pool of cases (or_lbm.cpp). */
void* or_pool_new(const or_lbm_case* cases, int ncases);
void or_pool_free(void* h);
void or_pool_steps(void* h, int nsteps, int nthreads);
void or_pool_regrid(void* h);
void or_pool_regrid_flags(void* h, const int32_t* flags);
void or_pool_upload(void* h, const float* f);
void or_pool_flags(void* h, int32_t* flags, float* wmax);
size_t or_pool_size(void* h);
void or_pool_bricks(void* h, int32_t* x, int32_t* y, int32_t* z, uint8_t* level, uint16_t* cs);
void or_pool_nbr(void* h, uint32_t* out);
void or_pool_populations(void* h, float* out);
/* The next nsteps level-0 steps in FP64 from the pool's current state, on its current mesh (the pool is
 * left unchanged); out as or_pool_populations, in double. */
void or_pool_fp64_steps(void* h, int nsteps, int nthreads, double* out);
void or_pool_conservation(void* h, double* out);
uint64_t or_pool_fluid_lups(void* h);
/* Solid voxels of one case at `level` (bit (z * Ny + y) * Nx + x); bits == NULL removes them. */
void or_pool_set_mask(void* h, int case_id, int level, const uint32_t* bits, size_t nwords);

/* Geometry placement (or_geometry.cpp).  type: 0 STL, 1 implicit function, 2 box, 3 sphere, 4 cylinder. */
typedef struct or_geometry {
    int32_t type;
    int32_t material_id;
    float translate[3];
    float scale[3];
    float rotate[3];
    float radius, height, width, length;
} or_geometry;
void or_geometry_aabb(const or_geometry* g, float* box6);
void or_geometry_inside(const or_geometry* g, const float* x, const float* y, const float* z, size_t n, uint8_t* out);
void or_geometry_evaluate(const or_geometry* g, const int32_t* x, const int32_t* y, const int32_t* z, size_t n,
                          uint8_t* out);
size_t or_stl_voxelize(const float* tris, size_t ntri, const or_geometry* g, float cell, int32_t* ox, int32_t* oy,
                       int32_t* oz, size_t cap);
size_t or_geometry_candidates(const or_geometry* g, float cell, const float* dom, int32_t* ox, int32_t* oy,
                              int32_t* oz, size_t cap);

#ifdef __cplusplus
}
#endif
#endif
