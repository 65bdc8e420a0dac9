// eddy_mma.h -- tensor-core (tcgen05) contingency kernel launchers.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "eddy_internal.h"

namespace eddy {
// pair groups (3 pairs, 32 operand rows each) padded for every variant
int mma_ngroups_pad(int c);
int mma_npad(int n);
int mma_bpad(int B);
// bytes of the Afp8 scratch for a batch of B units of a set with c pairs
// (operand + general-path queue)
size_t mma_a_bytes(int B, int n, int c);
size_t mma_y_bytes(int c, int n);
// Builds the pair-cell indicator operand Y of the current set and, after it,
// the FP32 copy of the full-sample tables the epilogue reads.
cudaError_t launch_build_y(const SetDev &sd, uint8_t *Y, cudaStream_t st);
// Masks -> e4m3 operand (Afp8, mma_a_bytes(B, n, c) bytes), then the GEMM +
// decision kernel, the general-path kernel for the tables its filter could
// not settle and the exact-path kernel for that path's guard-band cases.  Only bits of dmask are set: its masks and chunk bitmap
// must be zero when the launch starts.  *err: bit 0 = a bounded wait timed
// out, bit 1 = the general-path queue overflowed (the batch must be decided
// another way).  Variants (mma_variants()): tile widths N = 128 / 192 / 256
// with 16, 8, 12 or 16 epilogue warps, one CTA per SM.
int mma_variants();
cudaError_t launch_pairs_mma(const SetDev &sd, const uint64_t *masks, int B, uint8_t *Afp8,
                             const uint8_t *Y, uint32_t *dmask, unsigned long long *stats,
                             unsigned *err, int sms, cudaStream_t st, int variant);
}  // namespace eddy
