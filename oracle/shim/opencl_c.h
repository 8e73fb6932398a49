/* opencl_c.h -- OpenCL C built-ins for compiling the reference's .cl kernels
 * unmodified as C++ (TEST INFRASTRUCTURE ONLY: it lets the oracle be diffed
 * against the reference's own kernels on the CPU; nothing in the product uses it).
 *
 * Forced in front of each kernel file with `g++ -x c++ -include opencl_c.h`
 * (recipe: oracle/Makefile.ref).  It supplies what the OpenCL C dialect adds
 * to C99 and what the reference kernels use:
 *   - the scalar type names uchar / ushort / uint / ulong (OpenCL C 6.1.1);
 *   - the address-space qualifiers __kernel, __global, __local, __constant,
 *     constant, __private as no-ops (one flat host address space);
 *   - restrict as the C++ __restrict__ extension;
 *   - the work-item functions get_global_id / get_local_id / get_group_id and
 *     the size queries, read from the work-item the NDRange runner is executing
 *     (oracle/ndrange.cpp);
 *   - barrier(): the runner executes every work-group of a kernel that has
 *     barriers as cooperative fibers, and barrier() yields to the next
 *     work-item of the group until all of them have reached it;
 *   - the 32-bit atomics atomic_inc / atomic_cmpxchg and the 64-bit
 *     atom_cmpxchg (cl_khr_int64_base_atomics), returning the old value; each
 *     is a scheduling point when the runner executes a whole NDRange as fibers.
 * OpenCL C's char is signed; the recipe compiles with -fsigned-char so the
 * kernels' `char` loop counters behave as on an OpenCL device on every host.
 */
#ifndef FLUIDLOOM_ORACLE_OPENCL_C_H
#define FLUIDLOOM_ORACLE_OPENCL_C_H

#include <cstddef>
#include <cstdint>
#include <sys/types.h>

typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned long ulong;
static_assert(sizeof(ulong) == 8, "ulong must be 64-bit (LP64 host)");

namespace flcl {
struct WorkItem {
    size_t gid, lid, grp, gsize, lsize, ngroups;
};
extern thread_local const WorkItem* g_item;
void barrier_wait();
void atomic_point();  // a scheduling point in the runner's all-fibers mode, else nothing
}  // namespace flcl

inline size_t get_global_id(uint d) { return d == 0 ? flcl::g_item->gid : 0; }
inline size_t get_local_id(uint d) { return d == 0 ? flcl::g_item->lid : 0; }
inline size_t get_group_id(uint d) { return d == 0 ? flcl::g_item->grp : 0; }
inline size_t get_global_size(uint d) { return d == 0 ? flcl::g_item->gsize : 1; }
inline size_t get_local_size(uint d) { return d == 0 ? flcl::g_item->lsize : 1; }
inline size_t get_num_groups(uint d) { return d == 0 ? flcl::g_item->ngroups : 1; }

#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2
inline void barrier(int) { flcl::barrier_wait(); }

inline uint atomic_inc(volatile uint* p) {
    flcl::atomic_point();
    return __atomic_fetch_add(const_cast<uint*>(p), 1u, __ATOMIC_SEQ_CST);
}
inline uint atomic_cmpxchg(volatile uint* p, uint cmp, uint val) {
    flcl::atomic_point();
    __atomic_compare_exchange_n(const_cast<uint*>(p), &cmp, val, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
    return cmp;
}
inline ulong atom_cmpxchg(volatile ulong* p, ulong cmp, ulong val) {
    flcl::atomic_point();
    __atomic_compare_exchange_n(const_cast<ulong*>(p), &cmp, val, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
    return cmp;
}

#define __kernel
#define __global
#define __local
#define __private
#define __constant const
#define constant const
#define restrict __restrict__

#endif
