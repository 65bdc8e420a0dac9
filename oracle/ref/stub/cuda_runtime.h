/* stand-in for cuda_runtime.h in the CPU build of the reference's host
   routines: only the error query used by checkCUDAError (routines.cu:17-23). */
#pragma once
#include "ref_shim.h"
static inline cudaError_t cudaGetLastError(void) { return cudaSuccess; }
static inline const char *cudaGetErrorString(cudaError_t) { return "no error"; }
