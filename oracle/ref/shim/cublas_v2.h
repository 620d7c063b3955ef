// Host execution shim: the reference names cuBLAS types in error macros only.
#pragma once
typedef int cublasStatus_t;
#define CUBLAS_STATUS_SUCCESS 0
