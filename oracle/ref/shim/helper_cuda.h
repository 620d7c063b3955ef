// Host execution shim: the error check of the CUDA samples' helper_cuda.h
// (aborts with the failing call, as the reference's checkCudaErrors exits).
#pragma once
#include "cuda_runtime.h"
inline void sbref_check(int e, const char* what, const char* file, int line) {
    if (e != 0) {
        fprintf(stderr, "CUDA error %d at %s:%d: %s\n", e, file, line, what);
        abort();
    }
}
#define checkCudaErrors(val) sbref_check((int)(val), #val, __FILE__, __LINE__)
#define getLastCudaError(msg) sbref_check(cudaGetLastError(), msg, __FILE__, __LINE__)
