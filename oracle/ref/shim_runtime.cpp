// The host implementation of the CUDA runtime subset in shim/cuda_runtime.h
// (test infrastructure: host execution of the reference's kernels).
#include <ucontext.h>

#include <atomic>
#include <chrono>
#include <vector>

#include "shim/cuda_runtime.h"

namespace sbref {

thread_local Builtins tl;

namespace {

thread_local int g_last_error = cudaSuccess;

// coroutine state of the block that runs in coroutine mode (one at a time)
struct CoBlock {
    ucontext_t sched;
    std::vector<ucontext_t> ctx;
    std::vector<std::vector<char>> stacks;
    std::vector<int> done;
    const std::function<void()>* fn = nullptr;
    unsigned current = 0;
    bool active = false;
};
CoBlock g_co;
constexpr size_t kStack = 256 * 1024;

void co_entry() {
    (*g_co.fn)();
    g_co.done[g_co.current] = 1;
    // returning resumes uc_link (the scheduler)
}

void set_thread(dim3 grid, dim3 block, unsigned b, unsigned t) {
    tl.gdim = grid;
    tl.bdim = block;
    tl.bid = {b % grid.x, (b / grid.x) % grid.y, b / (grid.x * grid.y)};
    tl.tid = {t % block.x, (t / block.x) % block.y, t / (block.x * block.y)};
}

}  // namespace

void syncthreads() {
    if (!g_co.active) throw BarrierInPlainMode();
    swapcontext(&g_co.ctx[g_co.current], &g_co.sched);
}

bool run_block_plain(const std::function<void()>& fn, dim3 grid, dim3 block, unsigned b) {
    const unsigned nt = block.x * block.y * block.z;
    try {
        for (unsigned t = 0; t < nt; ++t) {
            set_thread(grid, block, b, t);
            fn();
        }
    } catch (const BarrierInPlainMode&) {
        return false;
    }
    return true;
}

void run_block_coroutines(const std::function<void()>& fn, dim3 grid, dim3 block, unsigned b) {
    const unsigned nt = block.x * block.y * block.z;
    g_co.ctx.assign(nt, ucontext_t{});
    if (g_co.stacks.size() < nt) g_co.stacks.resize(nt);
    g_co.done.assign(nt, 0);
    g_co.fn = &fn;
    for (unsigned t = 0; t < nt; ++t) {
        g_co.stacks[t].resize(kStack);
        getcontext(&g_co.ctx[t]);
        g_co.ctx[t].uc_stack.ss_sp = g_co.stacks[t].data();
        g_co.ctx[t].uc_stack.ss_size = kStack;
        g_co.ctx[t].uc_link = &g_co.sched;
        makecontext(&g_co.ctx[t], co_entry, 0);
    }
    g_co.active = true;
    for (;;) {
        bool any = false;
        for (unsigned t = 0; t < nt; ++t) {
            if (g_co.done[t]) continue;
            any = true;
            g_co.current = t;
            set_thread(grid, block, b, t);
            swapcontext(&g_co.sched, &g_co.ctx[t]);
        }
        if (!any) break;
    }
    g_co.active = false;
}

void run_grid(const std::function<void()>& fn, dim3 grid, dim3 block) {
    const unsigned nb = grid.x * grid.y * grid.z;
    if (nb == 0) return;
    // the first block tells whether the kernel uses block barriers
    if (!run_block_plain(fn, grid, block, 0)) {
        for (unsigned b = 0; b < nb; ++b) run_block_coroutines(fn, grid, block, b);
        return;
    }
#pragma omp parallel for schedule(dynamic, 4)
    for (unsigned b = 1; b < nb; ++b) run_block_plain(fn, grid, block, b);
}

}  // namespace sbref

using namespace sbref;

const char* cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "error"; }
const char* cudaGetErrorName(cudaError_t e) { return cudaGetErrorString(e); }
cudaError_t cudaGetLastError() {
    const int e = g_last_error;
    g_last_error = cudaSuccess;
    return e;
}
cudaError_t cudaPeekAtLastError() { return g_last_error; }
cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
cudaError_t cudaDeviceReset() { return cudaSuccess; }
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaGetDevice(int* d) {
    *d = 0;
    return cudaSuccess;
}
cudaError_t cudaGetDeviceCount(int* n) {
    *n = 1;
    return cudaSuccess;
}
cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int) {
    memset(p, 0, sizeof(*p));
    strcpy(p->name, "host execution");
    p->maxThreadsDim[0] = p->maxThreadsDim[1] = 1024;
    p->maxThreadsDim[2] = 64;
    p->maxThreadsPerBlock = 1024;
    p->multiProcessorCount = 1;
    p->major = 10;
    return cudaSuccess;
}
cudaError_t sbref_malloc(void** p, size_t n) {
    *p = calloc(n ? n : 1, 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t sbref_malloc_pitch(void** p, size_t* pitch, size_t w, size_t h) {
    *pitch = (w + 511) / 512 * 512;
    return sbref_malloc(p, *pitch * h);
}
cudaError_t cudaFree(void* p) {
    free(p);
    return cudaSuccess;
}
cudaError_t cudaMemset(void* p, int v, size_t n) {
    memset(p, v, n);
    return cudaSuccess;
}
cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, cudaMemcpyKind) {
    memmove(dst, src, n);
    return cudaSuccess;
}
cudaError_t cudaMemcpy2D(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width,
                         size_t height, cudaMemcpyKind) {
    for (size_t r = 0; r < height; ++r)
        memmove((char*)dst + r * dpitch, (const char*)src + r * spitch, width);
    return cudaSuccess;
}

struct sbref_event {
    std::chrono::steady_clock::time_point t;
};
cudaError_t cudaEventCreate(cudaEvent_t* e) {
    *e = new sbref_event();
    return cudaSuccess;
}
cudaError_t cudaEventDestroy(cudaEvent_t e) {
    delete e;
    return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t) {
    e->t = std::chrono::steady_clock::now();
    return cudaSuccess;
}
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b) {
    *ms = std::chrono::duration<float, std::milli>(b->t - a->t).count();
    return cudaSuccess;
}
