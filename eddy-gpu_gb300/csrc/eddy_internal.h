// eddy_internal.h -- layouts shared by the host side (eddy_api.cu) and the
// sm_103a kernels (eddy_kernels.cu) of libeddy_gpu.
//
// Vocabulary follows the reference: a gene set of g genes, n samples split
// into class 1 (label 0, nA samples) and class 2 (label 1, nB samples); a
// "unit" is one gene set under one labelling (one permutation); each unit
// has S = nA + nB + 2 leave-one-out networks (kernel1.cu:85-88, 412-416);
// pair p enumerates (row, col), row > col, row-major lower triangle
// (main.cu:615-632).
#pragma once
#include <stdint.h>

namespace eddy {

constexpr int kDofSlots = 3;        // dof 1, 2, 4 (dof 0 never gives an edge)
constexpr int kMaxBdeuParents = 3;  // kernel5.cu:119-130 caps at 1 + 3
constexpr int kDivisors = 15;       // distinct q and q*r of the BDeu terms
constexpr uint32_t kUnitOk = 0;
constexpr uint32_t kUnitKmaxOverflow = 1u;   // more changed nodes than kmax;
                                             // bits 16-31 then hold the most
                                             // changed nodes of its networks
constexpr uint32_t kUnitHashCollision = 2u;  // equal hash, unequal networks
constexpr uint32_t kUnitBadShape = 4u;

// Decision thresholds for one (alpha selector, dof) in chi-square units.
// True scale (the reference's FP64 chi-square): edge is certain on
// (chiB, kLo), certainly absent below chiA and above kHi; [chiA, chiB] and
// [kLo, kHi] need the exact FP64 re-evaluation.  f* are the same bounds
// moved inward by the FP32 chi-square error so they apply to FP32 values.
struct Thr {
  float chiA, chiB, kLo, kHi;   // true scale, rounded outward
  float fA, fB, fKlo, fKhi;     // FP32-value scale
};

struct SetDev {
  int g, n, W, c;         // genes, samples, 64-bit words per sample row, pairs
  int nA, nB, S;          // class sizes (fixed under permutation), networks
  int mp;                 // -mp
  int GW;                 // 32-bit words per network row bitset (ceil(g/32))
  int bonf;               // Bonferroni on
  int exact_all;          // pathological alphas: every table goes exact
  int core;               // every value of the set is -1/0/1: the tensor-core
                          // path counts 4 cells per table and derives the
                          // other 5 from the genes' class counts
  double alpha_edge, alpha_edge_prior;
  Thr thr[2][kDofSlots];  // [0] = no prior (alpha_edge), [1] = prior pairs
  const uint64_t *planes; // [g][3][W]  bit s of plane (i, a) = (x_i(s) == a-1)
  const uint64_t *planesT; // [W][g][3] the same planes word-major (follows planes)
  const uint64_t *valid;  // [W] all-sample mask
  const int8_t *vals;     // [g][n]  -1/0/1, 2 = any other value
  const int8_t *valsT;    // [n][st_stride(g)] states 0-3 (st_of) of the same,
                          // sample-major, rows padded with 3 to 16 bytes
  const uint16_t *ctot;   // [c][9]  permutation-invariant full-sample table
  const uint8_t *prior;   // [c]     prior bit of pair p
  const int64_t *lg;      // [kDivisors][n+1] fixed-point lgamma(m+4/d)-lgamma(4/d)
  int lg_stride;          // n+1
  int lg_shift;           // fixed-point scale 2^lg_shift
  uint64_t salt;          // network hash salt
};

// Decision masks of a batch, per set: [nb][c] u32 (class 1 in bits 0-9,
// class 2 in bits 16-25), followed by a bitmap per unit of the 32-pair
// chunks that hold a nonzero mask ([nb][chunk_words(c)] u32).  Between
// batches the whole buffer is zero: the decision kernels only set bits
// (and a chunk's bit with every nonzero mask in it), and the unit kernel
// clears each mask word and chunk bit it reads.
#ifdef __CUDACC__
#define EDDY_HD __host__ __device__
#else
#define EDDY_HD
#endif
// Row stride of the sample-major state matrix: genes rounded up to 16, so
// that every row starts on a 16-byte boundary.
EDDY_HD constexpr int st_stride(int g) { return (g + 15) & ~15; }
EDDY_HD constexpr int chunk_words(int c) { return ((c + 31) / 32 + 31) / 32; }
// u32 words of one set's decision masks and chunk bitmaps for nb units
EDDY_HD constexpr size_t dmask_words(int nb, int c) {
  return (size_t)nb * (c > 0 ? c : 1) + (size_t)nb * chunk_words(c > 0 ? c : 1);
}
EDDY_HD constexpr size_t dmask_bytes(int B, int c) { return sizeof(uint32_t) * dmask_words(B, c); }

// One gene set of a batch.  A batch holds the units (labellings) of one or
// more sets of the same sample count: set k's units are [u0, u0 + nb) of
// the batch, in order.  Its decision masks and per-unit scratch are its
// slices of the batch's buffers; in the contingency GEMM its units are the
// A-operand rows [128 mb0, 128 (mb0 + mblocks)) (the rest of the last
// block is padding) and its pair groups the column groups [grp0, grp0 +
// groups) of the batch's operand Y, full-sample tables and group table, and
// its tiles are [tile0, tile0 + ntn * mblocks) of the launch.
struct BatchSet {
  SetDev sd;
  int u0, nb;          // units
  int mb0, mblocks;    // A-operand row blocks of 128 units
  int tile0, ntn;      // contingency tiles (ntn column tiles per row block)
  int grp0;            // first column group of the set in the batch's Y
  int gc0;             // first gene of the set in the batch's gene counts
  int marg_b0;         // first block of its class-count work (4-cell layout)
  int pad_;
  long long dm0;       // u32 words: its decision masks, then its chunk bitmap
  long long sc0;       // bytes: its per-unit scratch, unit_bytes per unit
  long long mg0;       // u32 words (4-cell layout): class counts [g][128
                       // mblocks], then the class-1 sizes [128 mblocks]
  long long unit_bytes;
};
#ifdef __CUDACC__
__device__ __forceinline__ uint32_t *unit_dmask(uint32_t *dmask, const BatchSet &bs, int u) {
  return dmask + bs.dm0 + (size_t)(u - bs.u0) * bs.sd.c;
}
__device__ __forceinline__ uint32_t *unit_chunks(uint32_t *dmask, const BatchSet &bs, int u) {
  return dmask + bs.dm0 + (size_t)bs.nb * bs.sd.c + (size_t)(u - bs.u0) * chunk_words(bs.sd.c);
}
// marks the chunk of pair p in a unit's chunk bitmap
__device__ __forceinline__ void mark_chunk(uint32_t *ucb, int p) {
  atomicOr(ucb + (p >> 10), 1u << ((p >> 5) & 31));
}
#endif

// Per-batch pointers for the unit kernel.
struct BatchDev {
  int B;                       // units in the batch
  int nsets;                   // sets in the batch
  int kmax;                    // changed-node records per network
  int key_walk;                // 1: the key table from a walk over the unique
                               // networks' records (EDDY_KEY_WALK, a test switch)
  const BatchSet *sets;        // [nsets]
  const int32_t *uslot;        // [B] set of each unit (index into sets)
  const uint64_t *masks;       // [B][W] class-1 sample mask per unit
  uint32_t *dmask;             // decision masks and chunk bitmaps (per set: dm0)
  uint8_t *scratch;            // per-unit scratch (per set: sc0)
  double *js;                  // [B]
  int32_t *U;                  // [B]
  uint32_t *status;            // [B]
  int32_t *keep_slot;          // [B] -1 or slot of detailed output
  // detailed outputs for kept units (one slot per kept unit; node arrays
  // strided by keep_g nodes and rows by keep_gw words):
  int keep_g, keep_gw;
  int32_t *out_ids;            // [slots][S]   unique network -> network id
  int32_t *out_cnt;            // [slots][S][keep_g] capped parent counts
  int32_t *out_par;            // [slots][S][keep_g][mpk] parent lists
  int mpk;                     // list capacity per node in out_par
  double *out_dist;            // [slots][2][S] node-summed BDeu (double)
  double *out_lval;            // [slots][2][S] normalised likelihoods
  uint32_t *out_rows;          // [slots][2][keep_g][keep_gw] full-network edge rows
  unsigned long long *stats;   // [nsets][4] per set: exact rechecks, tables decided,
                               // tables settled by a filter, duplicate networks
};

}  // namespace eddy
