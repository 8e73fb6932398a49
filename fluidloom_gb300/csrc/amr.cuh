// amr.cuh — internal pieces of the regrid shared with the LBM pool.
#pragma once
#include "common.cuh"
#include "hash.cuh"

struct fl_mesh_out {
    int32_t* x; int32_t* y; int32_t* z;
    uint8_t* level; uint8_t* state; int32_t* flags; uint32_t* material; uint16_t* case_id;
};

fl_domain_dev fl_domain_from_config(fl_ctx* ctx, const fl_adapt_config* cfg, void* dev_case_slot);
size_t fl_adapt_scratch_bytes(size_t n, uint64_t cap);
// mode 0 (FACE6) probes through the hash table (tk, tv, cap); mode 1 (FULL26)
// through the sorted locator L.
int fl_balance_run(fl_ctx* ctx, fl_mesh_dev md, int32_t* flags, const fl_domain_dev& dom, const uint64_t* tk,
                   const uint32_t* tv, uint64_t cap, const fl_locator* L, int mode, int max_level, int max_iters,
                   uint8_t* shadow, uint8_t* viol, uint8_t* act, uint32_t* counters, fl_balance_result* res,
                   bool balanced_input = false);
// level_bound >= 0: no cell of the mesh is deeper (the point locator then skips a host read).
int fl_adapt_prepare(fl_ctx* ctx, const fl_mesh* mesh, const fl_adapt_config* cfg, const fl_domain_dev& dom,
                     bool run_balance, void* scratch, size_t* M_out, fl_adapt_stats* st, int level_bound = -1);
int fl_adapt_finish(fl_ctx* ctx, const fl_mesh* mesh, const fl_adapt_config* cfg, const fl_domain_dev& dom,
                    void* scratch, size_t M, const float* fields, uint32_t C, fl_mesh* out, float* out_fields,
                    uint32_t* osrc, uint8_t* okind, uint32_t* omembers, uint32_t num_groups);
