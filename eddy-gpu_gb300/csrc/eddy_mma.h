// eddy_mma.h -- tensor-core (tcgen05) contingency kernel launchers.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "eddy_internal.h"

namespace eddy {
int mma_ntiles(int c);
int mma_npad(int n);
int mma_bpad(int B);
size_t mma_y_bytes(int c, int n);
// Builds the pair-cell indicator operand Y of the current set and, after it,
// the FP32 copy of the full-sample tables the epilogue reads.
cudaError_t launch_build_y(const SetDev &sd, uint8_t *Y, cudaStream_t st);
// Masks -> e4m3 operand (Afp8, mma_bpad(B) x mma_npad(n) bytes), then the
// GEMM + decision kernel; *err is set on a bounded-wait timeout.
// variant 0: 16 epilogue warps (one column group each); variant 1: 8
// epilogue warps (two groups each); both a 4-stage ring, one CTA per SM.
int mma_variants();
cudaError_t launch_pairs_mma(const SetDev &sd, const uint64_t *masks, int B, uint8_t *Afp8,
                             const uint8_t *Y, uint32_t *dmask, unsigned long long *stats,
                             unsigned *err, int sms, cudaStream_t st, int variant);
}  // namespace eddy
