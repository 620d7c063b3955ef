// Mass integrals without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need a
// result: a host framework that owns every byte of device memory through its
// own pool (a stray cudaMalloc breaks its accounting or fails outright), a
// plug-in that its host application forbids to allocate once it has
// started, or a real-time loop that may not pay for cudaMalloc's implicit
// device-wide synchronisation.  For them, sb_mass_integrals_noalloc computes
// the same two integrals as sb_update_mass (sum of eta sin(theta) and
// gamma sin(theta) over a bubble's cells) from fields the caller already
// holds, using only a fixed scratch array that is compiled into this
// library.
//
// The scratch is the file-scope __device__ array g_noalloc_scratch below
// (20 KiB: 2 x 1024 FP64 per-block partial sums and a 1024-entry sin table),
// so the largest grid it serves is nTheta = 1024.  Every GPU that loads the
// library holds it until the process exits.  Host code cannot use the
// symbol's name as a device address: its address is looked up with
// cudaGetSymbolAddress on the first call made in a CUDA context (the
// device's primary context; a cudaDeviceReset ends that context, and the
// next call looks the address up again in the new one).  That first call
// should therefore happen before any stream capture begins.  Every call
// rewrites the whole array before reading it, so no state carries over
// between calls; but all calls share the one array, so calls whose kernels
// overlap on the GPU (different streams or host threads at once) race on it
// and must be serialised by the caller.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/soapbubble.h"

namespace sb {
int api_fail(int code, const char* msg);  // sets sb_last_error (sb_api.cu)
}

namespace {

constexpr int kNaMaxTheta = 1024;
constexpr int kNaBlocks = 1024;
constexpr int kNaThreads = 256;
constexpr int kNaMaxDevices = 64;

struct NoAllocScratch {
    double partial[2 * kNaBlocks];  // per-block sums of eta sin, gamma sin
    float sin_c[kNaMaxTheta];       // sin((i + 0.5) pi / nTheta)
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Per device: the context the address was looked up in (its unique id) and
// the address.
struct ScratchSlot {
    unsigned long long ctx_id;
    NoAllocScratch* addr;
};
ScratchSlot g_scratch[kNaMaxDevices] = {};
std::mutex g_scratch_mu;

__global__ void k_na_table(NoAllocScratch* s, int nT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nT) s->sin_c[i] = (float)sin((i + 0.5) * (3.14159265358979323846 / nT));
}

__device__ __forceinline__ double na_warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Grid-stride sums; every block writes its two partials, so the whole
// partial array is rewritten by every call.
__global__ void __launch_bounds__(kNaThreads)
k_na_mass(NoAllocScratch* s, const float* __restrict__ eta, const float* __restrict__ gam,
          int N, int logP) {
    double me = 0.0, mg = 0.0;
    for (int c = blockIdx.x * kNaThreads + threadIdx.x; c < N; c += kNaBlocks * kNaThreads) {
        const double sn = (double)s->sin_c[c >> logP];
        me += (double)eta[c] * sn;
        mg += (double)gam[c] * sn;
    }
    __shared__ double sm[2][kNaThreads / 32];
    me = na_warp_sum(me);
    mg = na_warp_sum(mg);
    if ((threadIdx.x & 31) == 0) {
        sm[0][threadIdx.x >> 5] = me;
        sm[1][threadIdx.x >> 5] = mg;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        double a = threadIdx.x < kNaThreads / 32 ? sm[0][threadIdx.x] : 0.0;
        double b = threadIdx.x < kNaThreads / 32 ? sm[1][threadIdx.x] : 0.0;
        a = na_warp_sum(a);
        b = na_warp_sum(b);
        if (threadIdx.x == 0) {
            s->partial[2 * blockIdx.x] = a;
            s->partial[2 * blockIdx.x + 1] = b;
        }
    }
}

// Ordered final sum of the partials into the caller's two doubles.
__global__ void k_na_final(const NoAllocScratch* s, double* out) {
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < kNaBlocks; k += 32) {
        a += s->partial[2 * k];
        b += s->partial[2 * k + 1];
    }
    a = na_warp_sum(a);
    b = na_warp_sum(b);
    if (threadIdx.x == 0) {
        out[0] = a;
        out[1] = b;
    }
}

// The current context's unique id through the driver entry points that the
// runtime hands out (no link against the driver library); 0 when there is
// no current context yet.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

int current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    *id = 0;
    if (!get_current || !get_id) {
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault,
                                             &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) !=
                cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return sb::api_fail(SB_ERR_CUDA,
                                "sb_mass_integrals_noalloc: driver context queries unavailable");
        get_current = (CtxGetCurrentFn)f1;
        get_id = (CtxGetIdFn)f2;
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS) return sb::api_fail(SB_ERR_CUDA, "cuCtxGetCurrent failed");
    if (ctx && get_id(ctx, id) != CUDA_SUCCESS) return sb::api_fail(SB_ERR_CUDA, "cuCtxGetId failed");
    return SB_OK;
}

// Device address of the scratch array in the current device's context:
// looked up with cudaGetSymbolAddress once per context (again after a
// cudaDeviceReset has replaced the context, whose module, and so the
// array's address, are new).
int scratch_for_current_device(NoAllocScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return sb::api_fail(SB_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kNaMaxDevices)
        return sb::api_fail(SB_ERR_INVALID, "sb_mass_integrals_noalloc: device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    unsigned long long id = 0;
    int rc = current_context_id(&id);
    if (rc != SB_OK) return rc;
    ScratchSlot& slot = g_scratch[dev];
    if (id == 0 || slot.ctx_id != id || !slot.addr) {
        NoAllocScratch* ptr = nullptr;
        e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return sb::api_fail(SB_ERR_CUDA, "sb_mass_integrals_noalloc: cudaGetSymbolAddress failed");
        // the lookup made the device's primary context current if it was not
        rc = current_context_id(&id);
        if (rc != SB_OK) return rc;
        slot.ctx_id = id;
        slot.addr = ptr;
    }
    *out = slot.addr;
    return SB_OK;
}

}  // namespace

extern "C" int sb_mass_integrals_noalloc(int nTheta, const float* eta, const float* gamma,
                                         double* mass_out, void* stream) {
    if (!eta || !gamma || !mass_out)
        return sb::api_fail(SB_ERR_INVALID, "sb_mass_integrals_noalloc: null pointer");
    if (nTheta < 8 || nTheta > kNaMaxTheta || (nTheta & (nTheta - 1)) != 0)
        return sb::api_fail(SB_ERR_INVALID,
                            "sb_mass_integrals_noalloc: nTheta must be a power of two in [8, 1024] "
                            "(the fixed scratch array holds 1024 rows)");
    NoAllocScratch* s = nullptr;
    int rc = scratch_for_current_device(&s);
    if (rc != SB_OK) return rc;
    const int nP = 2 * nTheta;
    int logP = 0;
    while ((1 << logP) < nP) ++logP;
    cudaStream_t st = (cudaStream_t)stream;
    // an error left pending by earlier work is the caller's to see: do no
    // work and leave it in place
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess)
        return sb::api_fail(SB_ERR_CUDA, "sb_mass_integrals_noalloc: an earlier CUDA error is pending");
    k_na_table<<<(nTheta + 255) / 256, 256, 0, st>>>(s, nTheta);
    if ((e = cudaGetLastError()) != cudaSuccess) return sb::api_fail(SB_ERR_CUDA, cudaGetErrorString(e));
    k_na_mass<<<kNaBlocks, kNaThreads, 0, st>>>(s, eta, gamma, nTheta * nP, logP);
    if ((e = cudaGetLastError()) != cudaSuccess) return sb::api_fail(SB_ERR_CUDA, cudaGetErrorString(e));
    k_na_final<<<1, 32, 0, st>>>(s, mass_out);
    if ((e = cudaGetLastError()) != cudaSuccess) return sb::api_fail(SB_ERR_CUDA, cudaGetErrorString(e));
    return SB_OK;
}
