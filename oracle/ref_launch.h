// ORACLE - test infrastructure only. CPU "launch" of a reference kernel
// body: blocks run in order on one OS thread; within a block every thread is
// a fiber (ucontext) so that __syncthreads() is a real barrier. Kernels
// without barriers run each thread to completion in turn.
#pragma once

#include <ucontext.h>

#include <functional>
#include <vector>

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

namespace refcpu {

thread_local ucontext_t g_sched;
thread_local std::vector<ucontext_t>* g_fibers = nullptr;
thread_local int g_cur = 0;
thread_local std::function<void()>* g_body = nullptr;
thread_local std::vector<char>* g_done = nullptr;

inline void fiber_entry() {
    (*g_body)();
    (*g_done)[g_cur] = 1;
    // returning resumes uc_link (the scheduler)
}

/// Run `body` as a grid of `grid` blocks of `block` threads.
inline void launch(unsigned grid, unsigned block, std::function<void()> body, bool barriers) {
    gridDim = dim3(grid, 1, 1);
    blockDim = dim3(block, 1, 1);
    if (!barriers) {
        for (unsigned b = 0; b < grid; ++b) {
            blockIdx = make_uint3(b, 0, 0);
            for (unsigned t = 0; t < block; ++t) {
                threadIdx = make_uint3(t, 0, 0);
                body();
            }
        }
        return;
    }
    constexpr size_t kStack = 64 * 1024;
    std::vector<ucontext_t> fibers(block);
    std::vector<std::vector<char>> stacks(block, std::vector<char>(kStack));
    std::vector<char> done(block);
    g_fibers = &fibers;
    g_body = &body;
    g_done = &done;
    for (unsigned b = 0; b < grid; ++b) {
        blockIdx = make_uint3(b, 0, 0);
        for (unsigned t = 0; t < block; ++t) {
            done[t] = 0;
            getcontext(&fibers[t]);
            fibers[t].uc_stack.ss_sp = stacks[t].data();
            fibers[t].uc_stack.ss_size = kStack;
            fibers[t].uc_link = &g_sched;
            makecontext(&fibers[t], fiber_entry, 0);
        }
        bool any = true;
        while (any) {
            any = false;
            for (unsigned t = 0; t < block; ++t) {
                if (done[t]) continue;
                g_cur = static_cast<int>(t);
                threadIdx = make_uint3(t, 0, 0);
                swapcontext(&g_sched, &fibers[t]);
                if (!done[t]) any = true;
            }
        }
    }
    g_fibers = nullptr;
}

} // namespace refcpu

void __syncthreads() {
    swapcontext(&(*refcpu::g_fibers)[refcpu::g_cur], &refcpu::g_sched);
}
