// eddy_mma.h -- tensor-core (tcgen05) contingency kernel launchers.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "eddy_internal.h"

namespace eddy {
// pair groups of a set in a layout (32 operand rows each: 3 pairs x 9
// cells, or in the layout of sets with no missing values (core) 8 pairs of
// one row gene x 4 cells), padded for every tile shape
int mma_ngroups_pad(const SetDev &sd, bool core);
int mma_npad(int n);

// The Y arena of the sets of a batch: their column groups, G in all, and
// their genes, `genes` in all, at a sample count n.  Set k's groups start at
// its grp0 and its genes at its gc0.
struct YArena {
  uint8_t *base;
  int G, genes, n;
};
size_t mma_y_bytes(int G, int genes, int n);
// Builds one set's slice of the arena: its pair-cell indicator operand Y,
// the FP32 copy of its full-sample tables the epilogue reads and (4-cell
// layout) its group table and genes' full-sample state counts.
cudaError_t launch_build_y(const SetDev &sd, bool core, const YArena &y, int grp0, int gc0,
                           cudaStream_t st);
int mma_build_launches(const SetDev &sd);

// The contingency plan of a batch for a tile shape (variant) and layout:
// fills each set's mb0, mblocks, tile0, ntn, marg_b0 and mg0; the totals
// size the A operand (rowsA rows), the launch (ntot tiles), the class-count
// work (bM blocks, marg_words words) and the general-path queue (tables).
struct MmaPlan {
  int rowsA, ntot, bM;
  long long marg_words, tables;
};
MmaPlan mma_plan(BatchSet *sets, int nsets, int variant, bool core);
// bytes of the Afp8 scratch of a batch: the A operand, the general-path
// queue and, in the 4-cell layout, the sets' class counts
size_t mma_a_bytes(const MmaPlan &p, int n, bool core);
// Masks -> e4m3 operand A and (4-cell layout) the units' class counts per
// gene state; then the GEMM + decision kernel, the general-path kernel for
// the tables its filter could not settle and the exact-path kernel for that
// path's guard-band cases (mma_launches() kernels in all).  sets: the
// batch's set table on the device, planned by mma_plan for this variant and
// layout; uslot: each unit's set; g_single: the set's g when the batch has
// one set (its gene counts are then staged in shared memory).  Only bits of
// dmask are set: its masks and chunk bitmaps must be zero when the launch
// starts.  *err: bit 0 = a bounded wait timed out, bit 1 = the general-path
// queue overflowed (the batch must be decided another way).  Variants
// (mma_variants()): tile widths N = 128 / 192 / 256 with 16, 8, 12 or 16
// epilogue warps, one CTA per SM.
int mma_variants();
int mma_launches();
cudaError_t launch_pairs_mma(const BatchSet *sets, int nsets, const MmaPlan &plan,
                             const uint64_t *masks, const int32_t *uslot, int n, int W,
                             uint8_t *Afp8, const YArena &y, uint32_t *dmask,
                             unsigned long long *stats, unsigned *err, int sms, cudaStream_t st,
                             int variant, bool core, int g_single, cudaEvent_t ev_mid = nullptr,
                             bool ev_external = false);
}  // namespace eddy
