// Host execution shim: the reference's own vendored helper_math.h (float
// vector operations, clamp, smoothstep), included with its host-compiler
// block switched off because shim/cuda_runtime.h already provides those
// host functions.
#pragma once
#include "cuda_runtime.h"
#define __CUDACC__
#include_next <helper_math.h>
#undef __CUDACC__
