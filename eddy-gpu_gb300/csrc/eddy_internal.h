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
  const int8_t *valsT;    // [n][g]  the same, sample-major
  const uint16_t *ctot;   // [c][9]  permutation-invariant full-sample table
  const uint8_t *prior;   // [c]     prior bit of pair p
  const int64_t *lg;      // [kDivisors][n+1] fixed-point lgamma(m+4/d)-lgamma(4/d)
  int lg_stride;          // n+1
  int lg_shift;           // fixed-point scale 2^lg_shift
  uint64_t salt;          // network hash salt
};

// Per-batch pointers for the unit kernel.
// Decision masks of a batch: [B][c] u32, followed by a bitmap per unit of
// the 32-pair chunks that hold a nonzero mask ([B][chunk_words(c)] u32).
// Between batches the whole buffer is zero: the decision kernels only set
// bits (and a chunk's bit with every nonzero mask in it), and the unit
// kernel clears each mask word and chunk bit it reads.
#ifdef __CUDACC__
#define EDDY_HD __host__ __device__
#else
#define EDDY_HD
#endif
EDDY_HD constexpr int chunk_words(int c) { return ((c + 31) / 32 + 31) / 32; }
EDDY_HD constexpr size_t dmask_bytes(int B, int c) {
  const int cc = c > 0 ? c : 1;
  return sizeof(uint32_t) * ((size_t)B * cc + (size_t)B * chunk_words(cc));
}
#ifdef __CUDACC__
__device__ __forceinline__ uint32_t *chunk_bits(uint32_t *dmask, int B, int c, int u) {
  return dmask + (size_t)B * c + (size_t)u * chunk_words(c);
}
__device__ __forceinline__ void mark_chunk(uint32_t *dmask, int B, int c, int u, int p) {
  atomicOr(chunk_bits(dmask, B, c, u) + (p >> 10), 1u << ((p >> 5) & 31));
}
#endif

struct BatchDev {
  int B;                       // units in the batch
  int kmax;                    // changed-node records per network
  const uint64_t *masks;       // [B][W] class-1 sample mask per unit
  uint32_t *dmask;             // [B][c] decision masks (class 1 bits 0-9, class 2 bits 16-25)
  uint8_t *scratch;            // per-unit scratch, unit_bytes each
  size_t unit_bytes;
  double *js;                  // [B]
  int32_t *U;                  // [B]
  uint32_t *status;            // [B]
  int32_t *keep_slot;          // [B] -1 or slot of detailed output
  // detailed outputs for kept units (one slot per kept unit):
  int32_t *out_ids;            // [slots][S]   unique network -> network id
  int32_t *out_cnt;            // [slots][S][g] capped parent counts
  int32_t *out_par;            // [slots][S][g][mpk] parent lists
  int mpk;                     // list capacity per node in out_par
  double *out_dist;            // [slots][2][S] node-summed BDeu (double)
  double *out_lval;            // [slots][2][S] normalised likelihoods
  uint32_t *out_rows;          // [slots][2][g][GW] full-network edge rows
  unsigned long long *stats;   // [4] exact rechecks, tables, filtered, verifications
};

}  // namespace eddy
