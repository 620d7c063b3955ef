// Grid-wide barrier with a bounded wait, for the cooperative kernels (the
// implicit solve and the map re-initialisation).
//
// The kernels are launched cooperatively, so every block is resident and a
// barrier completes as soon as every block reaches it.  The wait is bounded
// all the same: a block whose wait gives up counts a fault (reported by
// sb_get_stats as an error) and leaves the kernel, so that a bug that sends
// blocks down different paths ends the launch with an error instead of
// leaving the GPU waiting.
//
// Memory (kGridBarWords words, zeroed when the bubble or batch is made): word 0 holds
// the arrivals in its low 31 bits and the generation in bit 31.  Every block
// adds 1 except block 0, which adds 2^31 - (nblocks - 1); the adds of one
// barrier sum to 2^31, so bit 31 flips exactly when the last block arrives
// and the low bits return to zero for the next barrier.  Thread 0 of each
// block knows the generation it waits to see change (read once at kernel
// start: it cannot flip before this block arrives, and it flips once per
// barrier), so a block arrives with a fire-and-forget reduction and polls
// the word: no atomic round trip on the way to the barrier.  Ordering: the
// block barrier, then a release reduction by thread 0, publishes the block's
// writes; the acquire load that sees the flip, then the block barrier, makes
// every write before the barrier visible to the block.  The launches of one
// bubble or batch share the word: a launch that completes leaves its low
// bits at zero for the next.  After a wait gave up the word is no longer
// trusted, so the cooperative kernels of a bubble with a counted fault return
// at once, the bubble halts at the end of that step (k_flip; every member of
// a batch whose launch counted it), and sb_get_stats keeps reporting the
// fault.
#pragma once
#include <cuda_runtime.h>

#include "sb_internal.h"

namespace sb {

constexpr unsigned kGridBarPolls = 1u << 22;  // polls before a wait gives up (~1-2 s)
constexpr unsigned kGridBarSpin = 1u << 10;   // polls before each poll also sleeps briefly
constexpr unsigned kGridBarGenBit = 0x80000000u;

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// The generation bit at kernel start (meaningful in thread 0 only).
__device__ __forceinline__ unsigned grid_barrier_gen(const unsigned* bar) {
    return threadIdx.x == 0 ? (ld_acquire_gpu(bar) & kGridBarGenBit) : 0u;
}

// Returns true in every thread of the block, or false in every thread when
// this block's wait gave up after `limit` polls (one fault counted in
// *faults).  gen: thread 0's copy of the current generation bit, advanced by
// the call.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned& gen, unsigned nblocks,
                                             int* faults, unsigned limit = kGridBarPolls) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned add = blockIdx.x == 0 ? kGridBarGenBit - (nblocks - 1u) : 1u;
        asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(bar), "r"(add) : "memory");
        unsigned polls = 0;
        while ((ld_acquire_gpu(bar) & kGridBarGenBit) == gen) {
            if (++polls > limit) {
                atomicAdd(faults, 1);
                ok = 0;
                break;
            }
            if (polls > kGridBarSpin) __nanosleep(64);
        }
        gen ^= kGridBarGenBit;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

}  // namespace sb
