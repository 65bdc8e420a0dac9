// eddy_kernels.h -- host-callable launchers of the sm_103a kernels.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "eddy_internal.h"

namespace eddy {
size_t unit_scratch_bytes(int c, int S, int kmax);
size_t unit_smem_size(int g, int W, int nwarps);
cudaError_t launch_prep(const int8_t *vals, int g, int n, int W, int c, uint64_t *planes,
                        uint64_t *valid, uint16_t *ctot, int8_t *valsT, cudaStream_t st);
cudaError_t launch_counter_masks(int n, int nA, int W, uint64_t seed, const int32_t *unit_set,
                                 const int32_t *unit_perm, const uint64_t *mask0, uint64_t *masks,
                                 int B, cudaStream_t st);
// Popcount contingency and decision kernel for a batch (sets: its device
// set table, uslot: each unit's set; cmax: the largest pair count).
cudaError_t launch_pairs(const BatchSet *sets, const int32_t *uslot, const uint64_t *masks,
                         uint32_t *dmask, int B, int W, int cmax, unsigned long long *stats,
                         cudaStream_t st);
// Network, BDeu and JS kernels of a batch (gmax: the largest set); ev_mid,
// when given, is recorded between the network kernel and the JS kernel.
cudaError_t launch_units(const BatchDev &bd, int gmax, int W, cudaStream_t st,
                         cudaEvent_t ev_mid = nullptr, bool ev_external = false);
cudaError_t set_divisor_map(const int8_t *map82);
}  // namespace eddy
