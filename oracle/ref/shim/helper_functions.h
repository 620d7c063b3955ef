// Host execution shim: nothing of the CUDA samples' helper_functions.h is used.
#pragma once
#include "cuda_runtime.h"
