// ndrange.h -- the CPU NDRange runner and the signatures of the reference's
// OpenCL kernels as they compile through shim/opencl_c.h.  TEST
// INFRASTRUCTURE ONLY.  Each declaration names the kernel file and line it
// comes from (paths inside the fedres/fluidloom tree); the kernel bodies are
// the reference's own, compiled in place by oracle/Makefile.ref.
#ifndef FLUIDLOOM_ORACLE_NDRANGE_H
#define FLUIDLOOM_ORACLE_NDRANGE_H

#include <functional>

#include "shim/opencl_c.h"

namespace flcl {
enum Schedule { kSequential, kGroupFibers, kAllFibers };
// Run body() once per work-item of a 1-D NDRange (global a multiple of local)
// under one of the schedules described in ndrange.cpp.
void run(size_t global, size_t local, const std::function<void()>& body, Schedule mode);
}  // namespace flcl

// src/adaptation/kernels/split_cells.cl:15-24 (barrier kernel)
void split_count_and_allocate(const int*, const int*, const int*, const uchar*, const int*, const uchar*,
                              uint*, uint*, uint);
// split_cells.cl:53-68
void split_generate_children(const int*, const int*, const int*, const uchar*, const uchar*, const uint*,
                             const uint*, int*, int*, int*, uchar*, uchar*, uint*, ulong*, uint);
// split_cells.cl:110-115
void interpolate_split_fields(const uint*, const float*, float*, uint, uint);

// src/adaptation/kernels/merge_cells.cl:11-23
void mark_sibling_groups(const int*, const int*, const int*, const uchar*, const int*, const uchar*, uint*, uint*,
                         const ulong*, const uint*, uint, uint);
// merge_cells.cl:123-130
void merge_fields(const uint*, const uint*, const float*, float*, uint, uint, uint);
// merge_cells.cl:162-177
void create_parent_cells(const int*, const int*, const int*, const uchar*, const uchar*, const uint*, const uint*,
                         const uint*, int*, int*, int*, uchar*, uchar*, uint*, uint);

// src/adaptation/kernels/balance_enforce.cl:57-68
void detect_balance_violations(const int*, const int*, const int*, const uchar*, const uchar*, const ulong*,
                               const uint*, uint, uchar*, uint*, uint);
// balance_enforce.cl:150-159
void mark_cascading_refinement(const int*, const int*, const int*, const uchar*, const uchar*, const uchar*, int*,
                               uint*, uint);

// src/adaptation/kernels/compact_cells.cl:9-33
void mark_valid_cells(const int*, const uchar*, const uint*, uint*, uint);
// compact_cells.cl:61-66 (barrier kernel)
void scan_local(uint*, uint*, uint*, uint, uint*);
// compact_cells.cl:114-117
void scan_add_sums(uint*, const uint*, uint);
// compact_cells.cl:129-150
void compact_cells(const int*, const int*, const int*, const uchar*, const uchar*, const uint*, const float*,
                   const uint*, const uint*, int*, int*, int*, uchar*, uchar*, uint*, float*, uint, uint);
// compact_cells.cl:176-195
void append_cells(const int*, const int*, const int*, const uchar*, const uchar*, const uint*, const float*, int*,
                  int*, int*, uchar*, uchar*, uint*, float*, uint, uint, uint);

// kernels/hashmap/hash_build.cl:19-27
void hash_build(ulong*, uint*, const ulong*, const uint*, ulong, uint, uint*);
// hash_build.cl:72-76
void hash_clear(ulong*, uint*, ulong);
// kernels/hashmap/hash_query.cl:61-69
void hash_validate(const ulong*, const uint*, ulong, const ulong*, uint*, uint*, uint);

// kernels/halo_pack.cl:3-8, 28-33
void pack_fields(const float*, uchar*, const ulong, const ulong);
void unpack_fields(const uchar*, float*, const ulong, const ulong);

#endif
