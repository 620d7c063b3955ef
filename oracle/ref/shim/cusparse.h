// Host execution shim: the reference names cuSPARSE types in error macros only.
#pragma once
typedef int cusparseStatus_t;
#define CUSPARSE_STATUS_SUCCESS 0
inline const char* cusparseGetErrorString(cusparseStatus_t) { return "cusparse"; }
