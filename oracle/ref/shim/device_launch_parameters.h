// Host execution shim: the built-in variables live in cuda_runtime.h.
#pragma once
#include "cuda_runtime.h"
