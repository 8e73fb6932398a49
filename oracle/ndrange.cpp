// ndrange.cpp -- a CPU NDRange runner for the reference's OpenCL kernels
// compiled as C++ through shim/opencl_c.h.  TEST INFRASTRUCTURE ONLY.
//
// One-dimensional NDRanges (the only kind the reference enqueues), run in one
// of three schedules, each a schedule an OpenCL device may legally produce:
//   kSequential   work-items one after another in work-item order (kernels
//                 without barriers);
//   kGroupFibers  each work-group as `local` cooperative fibers (POSIX
//                 ucontext): barrier() switches to the next unfinished
//                 work-item of the group, so every work-item reaches a
//                 barrier before any passes it; groups one after another;
//   kAllFibers    every work-item of the NDRange as a fiber, with each atomic
//                 and each barrier a scheduling point: all work-items run up
//                 to their first atomic before any goes past it.  This is the
//                 schedule of a device that keeps the whole range resident in
//                 lockstep; kernels that race a plain store against another
//                 work-item's later store (merge_cells.cl's group ids) give
//                 their intended result under it.
// Executing on one thread fixes the order in which atomics are taken
// (atomic_inc hands out ids in work-item order), which a device does not:
// tests that compare such ids compare them as sets.
#include "ndrange.h"

#include <ucontext.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

namespace flcl {

thread_local const WorkItem* g_item = nullptr;

namespace {

struct Fiber {
    ucontext_t ctx;
    WorkItem item;
    bool done;
    std::vector<char> stack;
};

thread_local ucontext_t* t_sched = nullptr;
thread_local Fiber* t_fiber = nullptr;
thread_local const std::function<void()>* t_body = nullptr;
thread_local bool t_yield_atomics = false;

void trampoline() {
    (*t_body)();
    t_fiber->done = true;  // returning resumes uc_link, the scheduler
}

// Run the fibers round-robin until all are done; each round runs every
// unfinished fiber up to its next scheduling point (or its end).
void schedule(std::vector<Fiber>& fib, ucontext_t* sched) {
    for (bool any = true; any;) {
        any = false;
        for (auto& f : fib) {
            if (f.done) continue;
            t_fiber = &f;
            g_item = &f.item;
            swapcontext(sched, &f.ctx);
            if (!f.done) any = true;
        }
    }
}

void start(Fiber& f, const WorkItem& w, ucontext_t* sched) {
    f.item = w;
    f.done = false;
    getcontext(&f.ctx);
    f.ctx.uc_stack.ss_sp = f.stack.data();
    f.ctx.uc_stack.ss_size = f.stack.size();
    f.ctx.uc_link = sched;
    makecontext(&f.ctx, trampoline, 0);
}

}  // namespace

void barrier_wait() {
    if (!t_sched || !t_fiber) {
        std::fprintf(stderr, "ndrange: barrier() in a kernel launched without fibers\n");
        std::abort();
    }
    swapcontext(&t_fiber->ctx, t_sched);
}

void atomic_point() {
    if (t_yield_atomics && t_fiber) swapcontext(&t_fiber->ctx, t_sched);
}

void run(size_t global, size_t local, const std::function<void()>& body, Schedule mode) {
    if (local == 0 || global % local != 0) {
        std::fprintf(stderr, "ndrange: global size %zu is not a multiple of local size %zu\n", global, local);
        std::abort();
    }
    const size_t ngroups = global / local;
    if (mode == kSequential) {
        WorkItem w{0, 0, 0, global, local, ngroups};
        g_item = &w;
        for (size_t g = 0; g < ngroups; ++g)
            for (size_t l = 0; l < local; ++l) {
                w.gid = g * local + l; w.lid = l; w.grp = g;
                body();
            }
        g_item = nullptr;
        return;
    }
    ucontext_t sched;
    t_sched = &sched;
    t_body = &body;
    if (mode == kGroupFibers) {
        std::vector<Fiber> fib(local);
        for (auto& f : fib) f.stack.resize(64 * 1024);
        for (size_t g = 0; g < ngroups; ++g) {
            for (size_t l = 0; l < local; ++l)
                start(fib[l], WorkItem{g * local + l, l, g, global, local, ngroups}, &sched);
            schedule(fib, &sched);
        }
    } else {
        std::vector<Fiber> fib(global);
        for (auto& f : fib) f.stack.resize(16 * 1024);
        for (size_t i = 0; i < global; ++i)
            start(fib[i], WorkItem{i, i % local, i / local, global, local, ngroups}, &sched);
        t_yield_atomics = true;
        schedule(fib, &sched);
        t_yield_atomics = false;
    }
    t_sched = nullptr;
    t_fiber = nullptr;
    t_body = nullptr;
    g_item = nullptr;
}

}  // namespace flcl
