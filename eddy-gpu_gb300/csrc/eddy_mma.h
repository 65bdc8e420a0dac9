// eddy_mma.h -- tensor-core (tcgen05) contingency kernel launchers.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "eddy_internal.h"

namespace eddy {
// pair groups (32 operand rows each: 3 pairs x 9 cells, or 8 pairs of one
// row gene x 4 cells in the layout of sets with no missing values) padded
// for every variant
int mma_ngroups_pad(const SetDev &sd, bool core);
int mma_npad(int n);
int mma_bpad(int B);
// bytes of the Afp8 scratch for a batch of B units of the set (operand,
// general-path queue and, in the 4-cell layout, the units' class counts)
size_t mma_a_bytes(const SetDev &sd, int B);
size_t mma_y_bytes(const SetDev &sd);
// Builds the pair-cell indicator operand Y of the current set and, after it,
// the FP32 copy of the full-sample tables the epilogue reads (and, in the
// 4-cell layout, the genes' full-sample state counts).
cudaError_t launch_build_y(const SetDev &sd, uint8_t *Y, cudaStream_t st);
int mma_build_launches(const SetDev &sd);
// Masks -> e4m3 operand (Afp8, mma_a_bytes(sd, B) bytes) and, in the 4-cell
// layout, the units' class counts per gene state; then the GEMM + decision
// kernel, the general-path kernel for the tables its filter could not settle
// and the exact-path kernel for that path's guard-band cases (mma_launches()
// kernels in all).  Only bits of dmask are set: its masks and chunk bitmap
// must be zero when the launch starts.  *err: bit 0 = a bounded wait timed
// out, bit 1 = the general-path queue overflowed (the batch must be decided
// another way).  Variants (mma_variants()): tile widths N = 128 / 192 / 256
// with 16, 8, 12 or 16 epilogue warps, one CTA per SM.
int mma_variants();
int mma_launches(const SetDev &sd);
cudaError_t launch_pairs_mma(const SetDev &sd, const uint64_t *masks, int B, uint8_t *Afp8,
                             const uint8_t *Y, uint32_t *dmask, unsigned long long *stats,
                             unsigned *err, int sms, cudaStream_t st, int variant);
}  // namespace eddy
