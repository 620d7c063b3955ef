// Host execution of CUDA C++ sources: the subset of the CUDA runtime, of the
// vector types and of the kernel launch that the reference's step code uses,
// implemented on the CPU.  Test infrastructure only: it lets the reference's
// own kernels (kernel/*.cu of RiverIntheSky/SoapBubble) run unchanged on the
// host so that their outputs pin the FP64 oracle.
//
// Execution model.  A launch runs the grid's blocks one after another (the
// blocks of a kernel that never reaches __syncthreads run in parallel on
// OpenMP threads, since CUDA gives blocks no order).  Inside a block the
// threads run one after another as plain calls; a thread that reaches
// __syncthreads makes the launcher rerun that block with one coroutine per
// thread (ucontext), where each barrier switches to the next thread until
// every thread of the block has arrived.  __shared__ variables are static
// (one copy, shared by the block's threads).  Device memory is host memory;
// cudaMallocPitch pads rows to 512 bytes as the GPU's pitched allocations do.
#pragma once

#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cassert>
#include <cmath>
#include <functional>
#include <limits>

using std::isinf;
using std::isnan;

#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#define __noinline__
#define __inline__ inline
#define __constant__
#define __shared__ static
#define __launch_bounds__(...)
#define __align__(n) alignas(n)
#define __restrict__ __restrict
#define __CUDA_RUNTIME_H__
#define CUDART_VERSION 13000

// ---------------------------------------------------------------------------
// vector types
struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct uint3 {
    unsigned x, y, z;
};
struct int1 { int x; };
struct int2 { int x, y; };
struct int3 { int x, y, z; };
struct int4 { int x, y, z, w; };
struct uint1 { unsigned x; };
struct uint2 { unsigned x, y; };
struct uint4 { unsigned x, y, z, w; };
struct float1 { float x; };
struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct double1 { double x; };
struct double2 { double x, y; };
struct double3 { double x, y, z; };
struct double4 { double x, y, z, w; };
struct uchar4 { unsigned char x, y, z, w; };
inline int2 make_int2(int x, int y) { return {x, y}; }
inline int3 make_int3(int x, int y, int z) { return {x, y, z}; }
inline int4 make_int4(int x, int y, int z, int w) { return {x, y, z, w}; }
inline uint2 make_uint2(unsigned x, unsigned y) { return {x, y}; }
inline uint3 make_uint3(unsigned x, unsigned y, unsigned z) { return {x, y, z}; }
inline uint4 make_uint4(unsigned x, unsigned y, unsigned z, unsigned w) { return {x, y, z, w}; }
inline float2 make_float2(float x, float y) { return {x, y}; }
inline float3 make_float3(float x, float y, float z) { return {x, y, z}; }
inline float4 make_float4(float x, float y, float z, float w) { return {x, y, z, w}; }
inline double2 make_double2(double x, double y) { return {x, y}; }
inline double3 make_double3(double x, double y, double z) { return {x, y, z}; }
inline uchar4 make_uchar4(unsigned char x, unsigned char y, unsigned char z, unsigned char w) {
    return {x, y, z, w};
}

// ---------------------------------------------------------------------------
// built-in variables (per host thread; the launcher sets them)
namespace sbref {
struct Builtins {
    uint3 tid, bid;
    dim3 bdim, gdim;
};
extern thread_local Builtins tl;
}  // namespace sbref
#define threadIdx (::sbref::tl.tid)
#define blockIdx (::sbref::tl.bid)
#define blockDim (::sbref::tl.bdim)
#define gridDim (::sbref::tl.gdim)
#define warpSize 32

// ---------------------------------------------------------------------------
// device math that CUDA provides as overloads in the global namespace
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
inline long long min(long long a, long long b) { return a < b ? a : b; }
inline long long max(long long a, long long b) { return a > b ? a : b; }
inline unsigned long min(unsigned long a, unsigned long b) { return a < b ? a : b; }
inline unsigned long max(unsigned long a, unsigned long b) { return a > b ? a : b; }
inline float min(float a, float b) { return fminf(a, b); }
inline float max(float a, float b) { return fmaxf(a, b); }
inline double min(double a, double b) { return fmin(a, b); }
inline double max(double a, double b) { return fmax(a, b); }
inline double min(float a, double b) { return fmin((double)a, b); }
inline double min(double a, float b) { return fmin(a, (double)b); }
inline double max(float a, double b) { return fmax((double)a, b); }
inline double max(double a, float b) { return fmax(a, (double)b); }
inline float rsqrtf(float x) { return 1.0f / sqrtf(x); }
inline double rsqrt(double x) { return 1.0 / sqrt(x); }
inline float __saturatef(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
inline float saturate(float x) { return __saturatef(x); }

// ---------------------------------------------------------------------------
// runtime API
typedef int cudaError_t;
enum : int {
    cudaSuccess = 0,
    cudaErrorInvalidValue = 1,
    cudaErrorMemoryAllocation = 2,
};
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3,
    cudaMemcpyDefault = 4
};
typedef struct sbref_stream* cudaStream_t;
typedef struct sbref_event* cudaEvent_t;
struct cudaDeviceProp {
    char name[256];
    int maxThreadsDim[3];
    int maxThreadsPerBlock;
    int multiProcessorCount;
    size_t totalGlobalMem;
    int major, minor;
};
enum cudaChannelFormatKind { cudaChannelFormatKindSigned, cudaChannelFormatKindUnsigned,
                             cudaChannelFormatKindFloat, cudaChannelFormatKindNone };
struct cudaChannelFormatDesc {
    int x, y, z, w;
    cudaChannelFormatKind f;
};
template <class T>
inline cudaChannelFormatDesc cudaCreateChannelDesc() {
    return {8 * (int)sizeof(T), 0, 0, 0, cudaChannelFormatKindFloat};
}

const char* cudaGetErrorString(cudaError_t e);
const char* cudaGetErrorName(cudaError_t e);
cudaError_t cudaGetLastError();
cudaError_t cudaPeekAtLastError();
cudaError_t cudaDeviceSynchronize();
cudaError_t cudaDeviceReset();
cudaError_t cudaSetDevice(int dev);
cudaError_t cudaGetDevice(int* dev);
cudaError_t cudaGetDeviceCount(int* n);
cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int dev);
cudaError_t sbref_malloc(void** p, size_t n);
cudaError_t sbref_malloc_pitch(void** p, size_t* pitch, size_t width, size_t height);
template <class T>
inline cudaError_t cudaMalloc(T** p, size_t n) { return sbref_malloc((void**)p, n); }
template <class T>
inline cudaError_t cudaMallocPitch(T** p, size_t* pitch, size_t w, size_t h) {
    return sbref_malloc_pitch((void**)p, pitch, w, h);
}
cudaError_t cudaFree(void* p);
cudaError_t cudaMemset(void* p, int v, size_t n);
cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, cudaMemcpyKind k);
cudaError_t cudaMemcpy2D(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width,
                         size_t height, cudaMemcpyKind k);
template <class T>
inline cudaError_t cudaMemcpyToSymbol(T& sym, const void* src, size_t n, size_t off = 0,
                                      cudaMemcpyKind = cudaMemcpyHostToDevice) {
    memcpy((char*)&sym + off, src, n);
    return cudaSuccess;
}
template <class T>
inline cudaError_t cudaMemcpyFromSymbol(void* dst, const T& sym, size_t n, size_t off = 0,
                                        cudaMemcpyKind = cudaMemcpyDeviceToHost) {
    memcpy(dst, (const char*)&sym + off, n);
    return cudaSuccess;
}
cudaError_t cudaEventCreate(cudaEvent_t* e);
cudaError_t cudaEventDestroy(cudaEvent_t e);
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t s = nullptr);
cudaError_t cudaEventSynchronize(cudaEvent_t e);
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b);

// ---------------------------------------------------------------------------
// kernel launches: `k<<<grid, block>>>(args)` is rewritten (by the build
// recipe) as `sbref::Launcher(grid, block).bind(k)(args)`.
namespace sbref {

struct BarrierInPlainMode {};

// runs fn for every thread of block `b` of a launch; returns false when a
// thread reached __syncthreads in plain mode (the block must be rerun with
// coroutines)
bool run_block_plain(const std::function<void()>& fn, dim3 grid, dim3 block, unsigned b);
void run_block_coroutines(const std::function<void()>& fn, dim3 grid, dim3 block, unsigned b);
void run_grid(const std::function<void()>& fn, dim3 grid, dim3 block);
void syncthreads();

struct Launcher {
    dim3 grid, block;
    Launcher(dim3 g, dim3 b, size_t = 0, cudaStream_t = nullptr) : grid(g), block(b) {}
    template <class F>
    auto bind(F* kernel) const {
        const dim3 g = grid, b = block;
        return [g, b, kernel](auto... args) {
            run_grid([&]() { kernel(args...); }, g, b);
        };
    }
};

}  // namespace sbref

inline void __syncthreads() { sbref::syncthreads(); }
