/*
 * ref_shim.h -- force-included (g++ -include) when the reference's CUDA
 * sources kernel1.cu .. kernel5.cu and routines.cu are compiled as plain
 * C++ for the CPU.  TEST INFRASTRUCTURE ONLY: it lets the reference's own
 * kernel bodies run here as the strongest parity pin for the oracle.
 *
 * CUDA qualifiers become empty; blockIdx/threadIdx/blockDim/gridDim are
 * globals set by the emulator (ref_harness.cpp) before a simulated thread runs;
 * __syncthreads() yields to the emulator's block scheduler, which runs every
 * simulated thread of the block up to the barrier before any goes on.
 * Device malloc/free/printf map to the C library; abs/min/lgamma/log/exp/pow
 * map to the C++ <cmath> double overloads (CUDA's abs(double) is fabs).
 */
#ifndef EDDY_REF_SHIM_H
#define EDDY_REF_SHIM_H
#include <assert.h>
#include <errno.h>
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef __cplusplus
#include <cmath>
#include <cstdlib>
using std::abs;
#endif

#define __global__
#define __device__
#define __host__
#define __shared__

typedef int cudaError_t;
#define cudaSuccess 0

struct emu_dim3 {
  unsigned x, y, z;
};
extern emu_dim3 blockIdx, threadIdx, blockDim, gridDim;

void emu_syncthreads(void);
#define __syncthreads() emu_syncthreads()

static inline double min(double a, double b) { return a < b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }

#endif
