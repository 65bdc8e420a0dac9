// eddy_kernels.cu -- sm_103a kernels of the EDDY hot path.
//
//   k_planes / k_ctot   set preparation: per-gene state bit-planes over the
//                       samples and the permutation-invariant full-sample
//                       3x3 table of every pair.
//   k_counter_masks     counter-based labelling (Philox-4x32-10) -> class-1
//                       sample masks, one block per unit.
//   k_pairs             contingency counts of class 1 for every (unit, pair)
//                       (class 2 = full table - class 1), and the 10-bit
//                       leave-one-out decision mask per class: the reference's
//                       run2/run2Scalable (kernel1.cu:389-477) over all S
//                       networks collapsed to <= 10 distinct tables per class.
//   k_units             one block per unit: full networks, flip lists,
//                       per-network capped parent lists as deltas
//                       (kernel2.cu:114-142, kernel3.cu:134-165), network
//                       hashing and first-occurrence dedup with exact
//                       verification (kernel4.cu:72-84, main.cu:1060-1121),
//                       BDeu over the unique networks in fixed point
//                       (kernel5.cu:237-257), normalisation and JS
//                       (main.cu:1293-1428).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <climits>

#include "eddy_device.cuh"
#include "eddy_kernels.h"

namespace eddy {

// ----------------------------------------------------------- set prep
__global__ void k_planes(const int8_t *vals, int g, int n, int W, uint64_t *planes,
                         uint64_t *valid) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g * W) return;
  int i = idx / W, w = idx % W;
  uint64_t b0 = 0, b1 = 0, b2 = 0, v = 0;
  for (int k = 0; k < 64; k++) {
    int s = w * 64 + k;
    if (s >= n) break;
    v |= 1ull << k;
    int8_t x = vals[(size_t)i * n + s];
    if (x == -1) b0 |= 1ull << k;
    else if (x == 0) b1 |= 1ull << k;
    else if (x == 1) b2 |= 1ull << k;
  }
  planes[((size_t)i * 3 + 0) * W + w] = b0;
  planes[((size_t)i * 3 + 1) * W + w] = b1;
  planes[((size_t)i * 3 + 2) * W + w] = b2;
  // the word-major copy after the planes: [W][g][3]
  uint64_t *planesT = planes + (size_t)g * 3 * W + (size_t)w * g * 3 + (size_t)i * 3;
  planesT[0] = b0;
  planesT[1] = b1;
  planesT[2] = b2;
  if (i == 0) valid[w] = v;
}

// Sample-major states: valsT[s][i] = st_of(vals[i][s]), rows of
// st_stride(g) bytes padded with state 3 (no value).
__global__ void k_transpose(const int8_t *vals, int g, int n, int8_t *valsT) {
  const int gp = st_stride(g);
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= gp * n) return;
  const int s = idx / gp, i = idx % gp;
  valsT[idx] = (int8_t)(i < g ? st_of(vals[(size_t)i * n + s]) : 3);
}

__global__ void k_ctot(const uint64_t *planes, int g, int W, int c, uint16_t *ctot) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c) return;
  int row, col;
  pair_rc(p, row, col);
  const uint64_t *Pr = planes + (size_t)row * 3 * W, *Pc = planes + (size_t)col * 3 * W;
  int cnt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int w = 0; w < W; w++) {
    uint64_t r0 = Pr[w], r1 = Pr[W + w], r2 = Pr[2 * W + w];
    uint64_t c0 = Pc[w], c1 = Pc[W + w], c2 = Pc[2 * W + w];
    cnt[0] += __popcll(r0 & c0); cnt[1] += __popcll(r0 & c1); cnt[2] += __popcll(r0 & c2);
    cnt[3] += __popcll(r1 & c0); cnt[4] += __popcll(r1 & c1); cnt[5] += __popcll(r1 & c2);
    cnt[6] += __popcll(r2 & c0); cnt[7] += __popcll(r2 & c1); cnt[8] += __popcll(r2 & c2);
  }
  for (int k = 0; k < 9; k++) ctot[(size_t)p * 9 + k] = (uint16_t)cnt[k];
}

// ---------------------------------------------------- counter labelling
__device__ __forceinline__ void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// One block per unit.  key(s) = word s mod 4 of Philox(ctr = (s / 4, perm,
// set, 0), key = seed); the nA samples with the smallest (key, s) are class 1.
// Selection: a histogram of the keys' top 11 bits finds the bin that holds
// the nA-th smallest key; the samples of that bin (about n / 2048 of them)
// are ranked by (key, s) against each other, which gives the last one in,
// (T, sT); sample s is in when (key, s) <= (T, sT).  The same set as
// sorting the pairs and taking the first nA.
constexpr int kCmBlock = 128, kCmBins = 2048, kCmShift = 21;
__global__ void __launch_bounds__(kCmBlock) k_counter_masks(int n, int nA, int W, uint64_t seed,
                                                            const int32_t *unit_set,
                                                            const int32_t *unit_perm,
                                                            const uint64_t *mask0,
                                                            uint64_t *masks) {
  // keys [n] u32 (padded to 8 bytes), the W mask words, then the bin's
  // samples [n] u16
  extern __shared__ uint32_t key[];
  __shared__ int hist[kCmBins];
  __shared__ int wsum[kCmBlock / 32];
  __shared__ int s_bin, s_need, s_cnt;
  __shared__ uint32_t s_T;
  __shared__ int s_sT;
  const int u = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int perm = unit_perm[u];
  uint64_t *out = masks + (size_t)u * W;
  if (perm == 0) {
    for (int w = tid; w < W; w += kCmBlock) out[w] = mask0[w];
    return;
  }
  unsigned long long *mw = reinterpret_cast<unsigned long long *>(key + ((n + 1) & ~1));
  uint16_t *cand = reinterpret_cast<uint16_t *>(mw + W);
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  // one Philox call gives the keys of four samples
  for (int s4 = tid; 4 * s4 < n; s4 += kCmBlock) {
    uint32_t c[4] = {(uint32_t)s4, (uint32_t)perm, (uint32_t)unit_set[u], 0u};
    philox10(c, k0, k1);
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (4 * s4 + j < n) key[4 * s4 + j] = c[j];
  }
  for (int w = tid; w < W; w += kCmBlock) mw[w] = 0ull;
  for (int i = tid; i < kCmBins; i += kCmBlock) hist[i] = 0;
  if (tid == 0) s_cnt = 0;
  __syncthreads();
  for (int s = tid; s < n; s += kCmBlock) atomicAdd(&hist[key[s] >> kCmShift], 1);
  __syncthreads();
  // the bin of the nA-th smallest key: thread t sums bins [16 t, 16 t + 16),
  // then a block scan of those sums
  constexpr int kPer = kCmBins / kCmBlock;
  int loc = 0;
#pragma unroll
  for (int j = 0; j < kPer; j++) loc += hist[tid * kPer + j];
  int incl = loc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  int before = incl - loc;
  for (int w = 0; w < warp; w++) before += wsum[w];
  if (before < nA && nA <= before + loc) {
    for (int j = 0; j < kPer; j++) {
      const int h = hist[tid * kPer + j];
      if (before < nA && nA <= before + h) {
        s_bin = tid * kPer + j;
        s_need = nA - before;
      }
      before += h;
    }
  }
  __syncthreads();
  const uint32_t bin = (uint32_t)s_bin;
  const int need = s_need;
  for (int s = tid; s < n; s += kCmBlock)
    if ((key[s] >> kCmShift) == bin) cand[atomicAdd(&s_cnt, 1)] = (uint16_t)s;
  __syncthreads();
  // rank of each of the bin's samples among them by (key, s): the one of
  // rank need - 1 is the last one in
  const int cnt = s_cnt;
  for (int c = tid; c < cnt; c += kCmBlock) {
    const int s = cand[c];
    const uint32_t k = key[s];
    int rank = 0;
    for (int d = 0; d < cnt; d++) {
      const int t = cand[d];
      const uint32_t kt = key[t];
      rank += (kt < k || (kt == k && t < s)) ? 1 : 0;
    }
    if (rank == need - 1) {
      s_T = k;
      s_sT = s;
    }
  }
  __syncthreads();
  const uint32_t T = s_T;
  const int sT = s_sT;
  for (int s = tid; s < n; s += kCmBlock) {
    const uint32_t k = key[s];
    if (k < T || (k == T && s <= sT)) atomicOr(&mw[s >> 6], 1ull << (s & 63));
  }
  __syncthreads();
  for (int w = tid; w < W; w += kCmBlock) out[w] = mw[w];
}

// ------------------------------------------------------------ k_pairs
__global__ void __launch_bounds__(128) k_pairs(const BatchSet *__restrict__ sets,
                                               const int32_t *__restrict__ uslot,
                                               const uint64_t *masks, uint32_t *dmask,
                                               unsigned long long *stats) {
  extern __shared__ uint64_t smask[];
  const int u = blockIdx.y;
  const BatchSet &bs = sets[uslot[u]];
  const SetDev &sd = bs.sd;
  const int W = sd.W;
  for (int w = threadIdx.x; w < W; w += blockDim.x) smask[w] = masks[(size_t)u * W + w];
  __syncthreads();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned nexact = 0, nfilt = 0, ntab = 0;
  if (p < sd.c) {
    int row, col;
    pair_rc(p, row, col);
    const uint64_t *Pr = sd.planes + (size_t)row * 3 * W;
    const uint64_t *Pc = sd.planes + (size_t)col * 3 * W;
    int tA[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int w = 0; w < W; w++) {
      const uint64_t m = smask[w];
      const uint64_t r0 = Pr[w] & m, r1 = Pr[W + w] & m, r2 = Pr[2 * W + w] & m;
      const uint64_t c0 = Pc[w], c1 = Pc[W + w], c2 = Pc[2 * W + w];
      tA[0] += __popcll(r0 & c0); tA[1] += __popcll(r0 & c1); tA[2] += __popcll(r0 & c2);
      tA[3] += __popcll(r1 & c0); tA[4] += __popcll(r1 & c1); tA[5] += __popcll(r1 & c2);
      tA[6] += __popcll(r2 & c0); tA[7] += __popcll(r2 & c1); tA[8] += __popcll(r2 & c2);
    }
    int tB[9];
    const uint16_t *ct = sd.ctot + (size_t)p * 9;
#pragma unroll
    for (int k = 0; k < 9; k++) tB[k] = (int)ct[k] - tA[k];
    const int prior = sd.prior[p] ? 1 : 0;
    uint32_t mA = pair_mask(tA, prior, sd, nexact, nfilt);
    uint32_t mB = pair_mask(tB, prior, sd, nexact, nfilt);
    unit_dmask(dmask, bs, u)[p] = mA | (mB << 16);
    if (mA | mB) mark_chunk(unit_chunks(dmask, bs, u), p);
    ntab = 2;
  }
  if (stats) {
    // warp-aggregated counters
    for (int o = 16; o > 0; o >>= 1) {
      nexact += __shfl_down_sync(0xffffffffu, nexact, o);
      nfilt += __shfl_down_sync(0xffffffffu, nfilt, o);
      ntab += __shfl_down_sync(0xffffffffu, ntab, o);
    }
    if ((threadIdx.x & 31) == 0) {
      unsigned long long *sk = stats + 4 * (size_t)uslot[u];  // the set's row
      if (nexact) atomicAdd(&sk[0], (unsigned long long)nexact);
      if (ntab) atomicAdd(&sk[1], (unsigned long long)ntab);
      if (nfilt) atomicAdd(&sk[2], (unsigned long long)nfilt);
    }
  }
}

// ------------------------------------------------------------ k_units
// Open-addressing table: key -> smallest value inserted with it.  `empty`
// marks a free slot (no real key equals it); probing stops after `probes`
// slots (an insert that finds no place returns false).
struct MinTable {
  unsigned long long *key;
  int *val;
  unsigned mask;
  unsigned long long empty;
  unsigned probes;
  __device__ bool insert_min(unsigned long long k, int v) const {
    unsigned slot = (unsigned)(mix64(k) & mask);
    for (unsigned i = 0; i < probes; i++, slot = (slot + 1) & mask) {
      const unsigned long long prev = atomicCAS(&key[slot], empty, k);
      if (prev == empty || prev == k) {
        atomicMin(&val[slot], v);
        return true;
      }
    }
    return false;
  }
  // value of a key that was inserted
  __device__ int get(unsigned long long k) const {
    unsigned slot = (unsigned)(mix64(k) & mask);
    while (key[slot] != k) slot = (slot + 1) & mask;
    return val[slot];
  }
};
// slots of the shared-memory tables (in the BDeu work region, idle then)
constexpr int kSmSlots = 512;
constexpr unsigned kSmProbes = 64;

struct UnitLayout {
  size_t phi[2], pcol[2], rec, htk, htv, dist, uid, urep, sig;
  size_t skey, sbits, srep, hsk, hsv, wl, ksc, memo, total;
  int HT, rec_words;  // rec_words: 64-bit words per network record
};
// Rows with at most kMemoE kept flip entries have their capped list under
// every non-empty subset of those entries tabulated once per unit:
// [2 g rows][kMemoSub subsets][2 words] (record entry or ~0 when the list
// is the full network's, and the list's hash).
constexpr int kMemoE = 6, kMemoSub = (1 << kMemoE) - 1;
// genes of a set of c pairs (c = g (g - 1) / 2, so 1 + 8 c = (2 g - 1)^2)
__host__ __device__ inline int genes_of_pairs(int c) {
  int r = (int)sqrt((double)(1 + 8 * (long long)c));
  while ((long long)r * r > 1 + 8 * (long long)c) r--;
  while ((long long)(r + 1) * (r + 1) <= 1 + 8 * (long long)c) r++;
  return (r + 1) / 2;
}

__host__ __device__ inline UnitLayout unit_layout(int c, int S, int kmax) {
  UnitLayout L;
  size_t o = 0;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  for (int k = 0; k < 2; k++) {
    L.phi[k] = o;
    o = al(o + sizeof(uint32_t) * (size_t)(c > 0 ? c : 1));
    L.pcol[k] = o;
    o = al(o + sizeof(uint16_t) * (size_t)(c > 0 ? c : 1));
  }
  L.rec_words = 2 + kmax;  // [H, nchg | flags, chg...]
  L.rec = o;
  o = al(o + sizeof(uint64_t) * (size_t)L.rec_words * S);
  int HT = 1;
  while (HT < 2 * S) HT <<= 1;
  L.HT = HT;
  L.htk = o;
  o = al(o + sizeof(uint64_t) * (size_t)HT);
  L.htv = o;
  o = al(o + sizeof(int32_t) * (size_t)HT);
  L.dist = o;
  o = al(o + sizeof(int64_t) * 2 * (size_t)S);
  L.uid = o;
  o = al(o + sizeof(int32_t) * (size_t)S);
  L.urep = o;
  o = al(o + sizeof(int32_t) * (size_t)S);
  L.sig = o;  // class-1 samples then class-2 samples, in index order
  o = al(o + sizeof(int32_t) * (size_t)S);
  L.skey = o;  // per network: signature key (0 = no flip entry triggered)
  o = al(o + sizeof(uint64_t) * (size_t)S);
  L.sbits = o;  // per network: triggered entries as a bitset (<= 64 entries)
  o = al(o + sizeof(uint64_t) * (size_t)S);
  L.srep = o;  // per network: first network with the same signature
  o = al(o + sizeof(int32_t) * (size_t)S);
  L.hsk = o;  // signature hash table
  o = al(o + sizeof(uint64_t) * (size_t)HT);
  L.hsv = o;
  o = al(o + sizeof(int32_t) * (size_t)HT);
  L.wl = o;  // work list of networks
  o = al(o + sizeof(int32_t) * (size_t)S);
  L.ksc = o;  // scores of the distinct changed-node keys: [HT][2 classes]
  o = al(o + 2 * sizeof(int64_t) * (size_t)HT);
  L.memo = o;  // per-row capped lists under each subset of the row's entries
  o = al(o + 2 * sizeof(uint64_t) * kMemoSub * 2 * (size_t)genes_of_pairs(c));
  L.total = o;
  return L;
}

size_t unit_scratch_bytes(int c, int S, int kmax) { return unit_layout(c, S, kmax).total; }

// Block-wide exclusive scan (blockDim multiple of 32, <= 1024).
__device__ __forceinline__ int block_scan(int v, int &total, int *sbuf) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sbuf[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int t = (lane < nw) ? sbuf[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    sbuf[lane] = t;
  }
  __syncthreads();
  int excl = x - v + (warp ? sbuf[warp - 1] : 0);
  total = sbuf[nw - 1];
  __syncthreads();
  return excl;
}

struct UnitSmem {
  // fixed part; variable arrays follow in dynamic shared memory
  SetDev sd;    // the unit's set (copied from the batch's set table)
  unsigned long long HF[2];
  long long base[2][2];  // [data class][full network of class]
  int nphi[2];
  int ndab;
  int nrphi[2];
  int tfull;    // a shared-memory table ran out of probes
  int nent[2];  // flip entries per class
  int nwl;      // work-list length
  int firstB0;  // first class-2 network equal to the class-2 full network
  int firstE2;  // first class-2 network with an empty signature (S - 1: none)
  int ncand;    // candidates for unique networks
  int maxchg;   // most changed nodes of a network past kmax (0: none)
  int nlg;      // keys of merged-row lists logged by the records
  int scan[32];
  unsigned status;
  int U;
  double red_d[32];
  long long red_l[32];
};

// BDeu work items (node scores) processed per round
constexpr int kItems = 512;
// the task prefix array (2 kItems + 1 ints) also holds the memo offsets of
// the 2g rows of a unit, g <= 512 (the library's gene-set limit)
static_assert(2 * 512 <= 2 * kItems + 1, "memo offsets do not fit the task prefix array");

struct UnitPtrs {
  uint64_t *mA, *mB;      // [W]
  int *pcA, *pcB;         // [W]
  uint32_t *rows;         // [2][g][GW]
  uint16_t *cnt3;         // [2][g][3] state counts per class
  uint16_t *fcnt;         // [2][g] capped count of full networks
  uint16_t *fps;          // [2][g][3] first three parents
  unsigned long long *fh; // [2][g] node hash of full networks
  int *phs, *phe;         // [2][g] flip-entry range per row
  uint16_t *dab;          // [g] nodes whose full lists differ between classes
  uint16_t *rphi;         // [2][g] rows that hold flip entries, per class
  int8_t *stsig;          // [nwarps][g] states at sigma
  unsigned long long *itk;   // [kItems] node-score items: t | np << 14 | parents
  long long *acc;            // [kItems][2] their scores per class
  int *tq;                   // [2 kItems + 1] task prefix per (item, class)
  int8_t *dmap;              // [96] divisor map (copy of the constant one)
  long long *fsc;            // [2 full][2 data][g] base node scores
  uint32_t *ephi;            // [kEntCache] the kept flip entries, compacted
  uint16_t *epcol;           // [kEntCache] their columns
};
// flip entries a unit keeps in shared memory (more stay in its scratch)
constexpr int kEntCache = 1536;
// slots of the shared table of distinct changed-node keys, which takes the
// place of the flip-entry cache (ephi, then epcol) once the records are made
constexpr int kKeyT = 1024;
static_assert(kKeyT * sizeof(unsigned long long) <=
                  kEntCache * (sizeof(uint32_t) + sizeof(uint16_t)),
              "key table larger than the flip-entry cache");

__host__ __device__ inline size_t unit_smem_bytes(int g, int W, int GW, int nwarps) {
  size_t o = sizeof(UnitSmem);
  auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
  o = al(o) + 2 * sizeof(uint64_t) * W;
  o = al(o) + 2 * sizeof(int) * W;
  o = al(o) + 2 * sizeof(uint32_t) * (size_t)g * GW;
  o = al(o) + 2 * 3 * sizeof(uint16_t) * g;
  o = al(o) + 2 * sizeof(uint16_t) * g;
  o = al(o) + 2 * 3 * sizeof(uint16_t) * g;
  o = al(o) + 2 * sizeof(unsigned long long) * g;
  o = al(o) + 4 * sizeof(int) * g;
  o = al(o) + sizeof(uint16_t) * g;
  o = al(o) + 2 * sizeof(uint16_t) * g;
  o = al(o) + (size_t)nwarps * st_stride(g);
  o = al(o) + sizeof(unsigned long long) * kItems;
  o = al(o) + 2 * sizeof(long long) * kItems;
  o = al(o) + sizeof(int) * (2 * kItems + 1);
  o = al(o) + 96;
  o = al(o) + 4 * sizeof(long long) * g;
  o = al(o) + sizeof(uint32_t) * kEntCache;
  o = al(o) + sizeof(uint16_t) * kEntCache;
  return al(o);
}

size_t unit_smem_size(int g, int W, int nwarps) { return unit_smem_bytes(g, W, (g + 31) / 32, nwarps); }

__device__ inline UnitPtrs carve(char *base, int g, int W, int GW, int nwarps) {
  UnitPtrs P;
  size_t o = sizeof(UnitSmem);
  auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
  o = al(o); P.mA = (uint64_t *)(base + o); P.mB = P.mA + W; o += 2 * sizeof(uint64_t) * W;
  o = al(o); P.pcA = (int *)(base + o); P.pcB = P.pcA + W; o += 2 * sizeof(int) * W;
  o = al(o); P.rows = (uint32_t *)(base + o); o += 2 * sizeof(uint32_t) * (size_t)g * GW;
  o = al(o); P.cnt3 = (uint16_t *)(base + o); o += 2 * 3 * sizeof(uint16_t) * g;
  o = al(o); P.fcnt = (uint16_t *)(base + o); o += 2 * sizeof(uint16_t) * g;
  o = al(o); P.fps = (uint16_t *)(base + o); o += 2 * 3 * sizeof(uint16_t) * g;
  o = al(o); P.fh = (unsigned long long *)(base + o); o += 2 * sizeof(unsigned long long) * g;
  o = al(o); P.phs = (int *)(base + o); P.phe = P.phs + 2 * g; o += 4 * sizeof(int) * g;
  o = al(o); P.dab = (uint16_t *)(base + o); o += sizeof(uint16_t) * g;
  o = al(o); P.rphi = (uint16_t *)(base + o); o += 2 * sizeof(uint16_t) * g;
  o = al(o); P.stsig = (int8_t *)(base + o); o += (size_t)nwarps * st_stride(g);
  o = al(o); P.itk = (unsigned long long *)(base + o); o += sizeof(unsigned long long) * kItems;
  o = al(o); P.acc = (long long *)(base + o); o += 2 * sizeof(long long) * kItems;
  o = al(o); P.tq = (int *)(base + o); o += sizeof(int) * (2 * kItems + 1);
  o = al(o); P.dmap = (int8_t *)(base + o); o += 96;
  o = al(o); P.fsc = (long long *)(base + o); o += 4 * sizeof(long long) * g;
  o = al(o); P.ephi = (uint32_t *)(base + o); o += sizeof(uint32_t) * kEntCache;
  o = al(o); P.epcol = (uint16_t *)(base + o);
  return P;
}

// Network s of a unit: class k (0 = class 1, 1 = class 2) and left-out
// sample sigma (-1 for the two full networks), kernel1.cu:85-88, 412-416.
// sig: class-1 samples then class-2 samples in index order.
__device__ __forceinline__ void net_of(int s, const SetDev &sd, const int *sig, int &k, int &sigma) {
  if (s == 0) { k = 0; sigma = -1; return; }
  if (s == sd.S - 1) { k = 1; sigma = -1; return; }
  // class-1 sample s-1 sits at s-1; class-2 sample s-nA-1 at nA+(s-nA-1) = s-1
  k = (s <= sd.nA) ? 0 : 1;
  sigma = sig[s - 1];
}

// The states of every gene at sample sigma (3 for all when sigma < 0) into a
// warp's row of st_stride(g) bytes (16-byte aligned), 16 bytes per lane.
__device__ __forceinline__ void load_stsig(const SetDev &sd, int sigma, int8_t *dst, int lane) {
  const int nv = st_stride(sd.g) / 16;
  const uint4 *src = reinterpret_cast<const uint4 *>(sd.valsT + (size_t)(sigma >= 0 ? sigma : 0) * st_stride(sd.g));
  uint4 *d = reinterpret_cast<uint4 *>(dst);
  for (int i = lane; i < nv; i += 32)
    d[i] = sigma >= 0 ? __ldg(src + i) : make_uint4(0x03030303u, 0x03030303u, 0x03030303u, 0x03030303u);
  __syncwarp();
}

__device__ __forceinline__ void gen_for(ListGen &G, const SetDev &sd, const UnitPtrs &P,
                                        const uint32_t *phi, const uint16_t *pcol, int k, int t,
                                        const int8_t *st) {
  const int GW = sd.GW;
  const int strow = st ? st[t] : 3;
  G.init(P.rows + ((size_t)k * sd.g + t) * GW, GW, phi, pcol, P.phs[k * sd.g + t],
         P.phe[k * sd.g + t], st, strow);
}

// Exact comparison of the capped lists of node t in two networks.
__device__ bool lists_equal(const SetDev &sd, const UnitPtrs &P, const uint32_t *const *phi,
                            const uint16_t *const *pcol, int t, int k1, const int8_t *st1, int k2,
                            const int8_t *st2) {
  ListGen a, b;
  gen_for(a, sd, P, phi[k1], pcol[k1], k1, t, st1);
  gen_for(b, sd, P, phi[k2], pcol[k2], k2, t, st2);
  for (int i = 0; i < sd.mp; i++) {
    int x = a.next(), y = b.next();
    if (x != y) return false;
    if (x < 0) return true;
  }
  return true;
}


// Node scores of `n` items, kItems per round, as a flat task list over the
// block: task (item, class, parent configuration j).  get(i) -> the item's
// key (t | np << 14 | p0 << 16 | p1 << 32 | p2 << 48; np = 0 or a key of ~0
// = nothing to score); emit(i, class-1 score, class-2 score).  Fixed-point
// terms are summed with atomics: exact, in any order.
template <class Get, class Emit>
__device__ void bdeu_items(const SetDev &sd, const UnitPtrs &P, int *scan, int n, Get get,
                           Emit emit) {
  const int tid = threadIdx.x, nt = blockDim.x, g = sd.g;
  for (int b0 = 0; b0 < n; b0 += kItems) {
    const int m = n - b0 < kItems ? n - b0 : kItems;
    for (int i = tid; i < m; i += nt) {
      const unsigned long long key = get(b0 + i);
      P.itk[i] = key;
      const int np = (key == ~0ull) ? 0 : (int)((key >> 14) & 3);
      const int p0 = (int)((key >> 16) & 0xFFFF), p1 = (int)((key >> 32) & 0xFFFF),
                p2 = (int)((key >> 48) & 0xFFFF);
      for (int cls = 0; cls < 2; cls++) {
        P.tq[2 * i + cls] = np ? bdeu_tasks(P.cnt3 + 3 * g * cls, np, p0, p1, p2) : 0;
        P.acc[2 * i + cls] = 0;
      }
    }
    __syncthreads();
    int running = 0;
    for (int c0 = 0; c0 < 2 * m; c0 += nt) {
      const int e = c0 + tid;
      const int v = e < 2 * m ? P.tq[e] : 0;
      int total;
      const int off = block_scan(v, total, scan);
      if (e < 2 * m) P.tq[e] = running + off;
      running += total;
    }
    __syncthreads();
    // tasks in (item, class) order: a warp's consecutive lanes mostly share
    // one score, so their terms are summed in the warp (segmented) and each
    // score takes one atomic per warp
    const int lane = tid & 31;
    for (int base = tid - lane; base < running; base += nt) {
      const int task = base + lane;
      int seg = -1;
      long long term = 0;
      if (task < running) {
        int lo = 0, hi = 2 * m - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (P.tq[mid] <= task) lo = mid;
          else hi = mid - 1;
        }
        const int i = lo >> 1, cls = lo & 1, j = task - P.tq[lo];
        const unsigned long long key = P.itk[i];
        const int t = (int)(key & 0x3FFF), np = (int)((key >> 14) & 3);
        term = bdeu_config_term(sd, t, np, (int)((key >> 16) & 0xFFFF),
                                (int)((key >> 32) & 0xFFFF), (int)((key >> 48) & 0xFFFF),
                                cls ? P.mB : P.mA, P.cnt3 + 3 * g * cls, j, P.dmap);
        seg = lo;
      }
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, term, d);
        const int sy = __shfl_up_sync(0xffffffffu, seg, d);
        if (lane >= d && sy == seg) term += y;
      }
      const int sn = __shfl_down_sync(0xffffffffu, seg, 1);
      if (seg >= 0 && (lane == 31 || sn != seg))
        atomicAdd((unsigned long long *)&P.acc[seg], (unsigned long long)term);
    }
    __syncthreads();
    for (int i = tid; i < m; i += nt) emit(b0 + i, P.acc[2 * i], P.acc[2 * i + 1]);
    __syncthreads();
  }
}



__global__ void __launch_bounds__(256, 3) k_units(const __grid_constant__ BatchDev bd) {
  extern __shared__ __align__(16) char smraw[];
  UnitSmem &SM = *reinterpret_cast<UnitSmem *>(smraw);
  const int nw = blockDim.x >> 5, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int u = blockIdx.x;
  // the unit's set: its descriptor into shared memory, its slices of the
  // batch's masks and scratch
  const BatchSet &bs = bd.sets[bd.uslot[u]];
  const int ul = u - bs.u0, bs_nb = bs.nb;
  const long long bs_dm0 = bs.dm0;
  uint8_t *scr = bd.scratch + bs.sc0 + (size_t)ul * bs.unit_bytes;
  {
    const int *src = reinterpret_cast<const int *>(&bs.sd);
    int *dst = reinterpret_cast<int *>(&SM.sd);
    for (int i = threadIdx.x; i < (int)(sizeof(SetDev) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const SetDev &sd = SM.sd;
  const int g = sd.g, W = sd.W, GW = sd.GW, S = sd.S, c = sd.c;
  UnitPtrs P = carve(smraw, g, W, GW, nw);
  const UnitLayout L = unit_layout(c, S, bd.kmax);
  uint32_t *ucb = bd.dmask + bs_dm0 + (size_t)bs_nb * c + (size_t)ul * chunk_words(c);
  uint32_t *phi[2] = {(uint32_t *)(scr + L.phi[0]), (uint32_t *)(scr + L.phi[1])};
  uint16_t *pcol[2] = {(uint16_t *)(scr + L.pcol[0]), (uint16_t *)(scr + L.pcol[1])};
  unsigned long long *rec = (unsigned long long *)(scr + L.rec);
  unsigned long long *htk = (unsigned long long *)(scr + L.htk);
  int *htv = (int *)(scr + L.htv);
  long long *dist = (long long *)(scr + L.dist);
  int *uid = (int *)(scr + L.uid);
  int *urep = (int *)(scr + L.urep);
  int *sig = (int *)(scr + L.sig);
  unsigned long long *skey = (unsigned long long *)(scr + L.skey);
  unsigned long long *sbits = (unsigned long long *)(scr + L.sbits);
  int *srep = (int *)(scr + L.srep);
  unsigned long long *hsk = (unsigned long long *)(scr + L.hsk);
  int *hsv = (int *)(scr + L.hsv);
  int *wl = (int *)(scr + L.wl);
  uint32_t *dm = bd.dmask + bs_dm0 + (size_t)ul * c;
  const int tid = threadIdx.x, nt = blockDim.x;

  // ---- P0: masks, state counts, selection prefixes, init
  if (tid == 0) {
    SM.HF[0] = SM.HF[1] = 0;
    SM.nphi[0] = SM.nphi[1] = 0;
    SM.ndab = 0;
    SM.status = 0;
    SM.maxchg = 0;
    for (int a = 0; a < 2; a++)
      for (int b = 0; b < 2; b++) SM.base[a][b] = 0;
  }
  for (int w = tid; w < W; w += nt) {
    uint64_t m = bd.masks[(size_t)u * W + w];
    P.mA[w] = m;
    P.mB[w] = sd.valid[w] & ~m;
  }
  for (int i = tid; i < 2 * g * GW; i += nt) P.rows[i] = 0;
  // entry ranges of rows: start = INT_MAX, end = 0 until an entry lands
  for (int i = tid; i < 4 * g; i += nt) P.phs[i] = (i < 2 * g) ? 0x7fffffff : 0;
  for (int i = tid; i < 82; i += nt) P.dmap[i] = c_dmap[i];
  __syncthreads();
  // state counts per class from the word-major planes: a warp's loads of a
  // word are 32 consecutive planes
  for (int i = tid; i < g * 3; i += nt) {
    const uint64_t *pl = sd.planesT + i;
    int a = 0, b = 0;
    for (int w = 0; w < W; w++) {
      const uint64_t x = pl[(size_t)w * 3 * g];
      a += __popcll(x & P.mA[w]);
      b += __popcll(x & P.mB[w]);
    }
    P.cnt3[i] = (uint16_t)a;
    P.cnt3[3 * g + i] = (uint16_t)b;
  }
  if (warp == 0) {
    for (int cls = 0; cls < 2; cls++) {
      const uint64_t *m = cls ? P.mB : P.mA;
      int *pc = cls ? P.pcB : P.pcA;
      int run = 0;
      for (int w0 = 0; w0 < W; w0 += 32) {
        int w = w0 + lane;
        int v = (w < W) ? __popcll(m[w]) : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
          int y = __shfl_up_sync(0xffffffffu, x, o);
          if (lane >= o) x += y;
        }
        if (w < W) pc[w] = run + x - v;
        run += __shfl_sync(0xffffffffu, x, 31);
      }
    }
  }

  __syncthreads();
  // sample lists of both classes in index order (network -> left-out
  // sample): thread per sample bit
  for (int i = tid; i < 64 * W; i += nt) {
    const int w = i >> 6, bit = i & 63;
    const uint64_t below64 = (bit ? (~0ull >> (64 - bit)) : 0ull);
    const uint64_t a = P.mA[w], b = P.mB[w];
    if ((a >> bit) & 1ull) sig[P.pcA[w] + __popcll(a & below64)] = i;
    else if ((b >> bit) & 1ull) sig[sd.nA + P.pcB[w] + __popcll(b & below64)] = i;
  }

  // ---- P1: full-network rows and flip lists, from the 32-pair chunks that
  // hold a nonzero mask (the decision kernel's bitmap; the other chunks are
  // all zero).  Each nonzero mask word read is set back to zero.  Warp w
  // owns the rows whose pairs start in [w c/nw, (w+1) c/nw) and walks its
  // flagged chunks in pair order, four loads at a time.  Edge bits go into
  // the row bitsets; the flip entries land, in pair
  // order, in the warp's own segment of the list (which starts at its first
  // pair); a row's entry range is the min / max position of its entries
  // (rows without entries keep start > end).
  {
    const long long p_lo = (long long)warp * c / nw, p_hi = (long long)(warp + 1) * c / nw;
    int r0, c0;
    pair_rc((int)(p_lo < c ? p_lo : 0), r0, c0);
    if (c0 != 0) r0++;  // rows are owned by the warp holding their first pair
    int r1 = g;
    if (p_hi < c) {
      int c1;
      pair_rc((int)p_hi, r1, c1);
      if (c1 != 0) r1++;
    }
    if (p_lo >= c) r0 = g;
    if (r0 < 1) r0 = 1;  // row 0 has no pairs
    const int pa = r0 * (r0 - 1) / 2, pb = r0 < r1 ? r1 * (r1 - 1) / 2 : pa;
    int wpos0 = pa, wpos1 = pa;
    const uint32_t below = (1u << lane) - 1u;
    const uint32_t *cbits = ucb;
    const int k0 = pa >> 5, k1 = (pb + 31) >> 5;  // chunks [k0, k1)
    auto chunk = [&](int k, uint32_t m) {
      const int p = 32 * k + lane;
      const bool in = p >= pa && p < pb;
      int t = 0, j = 0;
      if (in) pair_rc(p, t, j);
      if (in && (m & 1u)) atomicOr(&P.rows[((size_t)0 * g + t) * GW + (j >> 5)], 1u << (j & 31));
      if (in && ((m >> 16) & 1u))
        atomicOr(&P.rows[((size_t)1 * g + t) * GW + (j >> 5)], 1u << (j & 31));
#pragma unroll
      for (int cls = 0; cls < 2; cls++) {
        const uint32_t mm = (m >> (16 * cls)) & 0x3FFu;
        const uint32_t fb = (mm >> 1) ^ ((mm & 1u) ? 0x1FFu : 0u);
        const bool flag = in && fb != 0u;
        const uint32_t bal = __ballot_sync(0xffffffffu, flag);
        const int wpos = cls ? wpos1 : wpos0;
        const int pos = wpos + __popc(bal & below);
        if (flag) {
          phi[cls][pos] = ((uint32_t)p << 9) | fb;
          pcol[cls][pos] = (uint16_t)j;
          atomicMin(&P.phs[cls * g + t], pos);
          atomicMax(&P.phe[cls * g + t], pos + 1);
        }
        if (cls) wpos1 += __popc(bal); else wpos0 += __popc(bal);
      }
    };
    for (int kw = k0 >> 5; pa < pb && kw <= (k1 - 1) >> 5; kw++) {
      uint32_t bits = cbits[kw];
      if (kw == (k0 >> 5)) bits &= ~0u << (k0 & 31);
      if (kw == ((k1 - 1) >> 5) && (k1 & 31)) bits &= ~0u >> (32 - (k1 & 31));
      while (bits) {
        int ks[4];
        uint32_t mv[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          ks[q] = -1;
          if (bits) {
            ks[q] = 32 * kw + __ffs(bits) - 1;
            bits &= bits - 1;
          }
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int p = 32 * ks[q] + lane;
          mv[q] = (ks[q] >= 0 && p >= pa && p < pb) ? dm[p] : 0u;
        }
#pragma unroll
        for (int q = 0; q < 4; q++)
          if (ks[q] >= 0) {
            chunk(ks[q], mv[q]);
            if (mv[q]) dm[32 * ks[q] + lane] = 0u;  // read once: left zero
          }
      }
    }
  }
  __syncthreads();
  // every warp has read the unit's chunk bitmap: zero it for the next batch
  {
    for (int i = tid; i < chunk_words(c); i += nt) ucb[i] = 0u;
  }

  // ---- P1b: only flip entries that can change a capped list are kept.
  // Node t's capped list is its first mp parents.  If R of the row's
  // entries are edges of the full network (the flips that can remove an
  // edge), every network of the class has at least mp edges in the columns
  // up to the (mp + R)-th edge of the full row, so its capped list lies
  // there: entries at later columns change no list and no network, and are
  // dropped (networks that differ only in them are the same network).  A
  // row's entries are contiguous and in column order.
  for (int i = tid; i < 2 * g; i += nt) {
    const int e0 = P.phs[i], e1 = P.phe[i];
    if (e0 >= e1) continue;
    const int k = i / g, t = i - k * g;
    const uint32_t *row = P.rows + (size_t)i * GW;
    int R = 0;
    for (int e = e0; e < e1; e++) {
      const int j = pcol[k][e];
      R += (row[j >> 5] >> (j & 31)) & 1u;
    }
    int need = sd.mp + R, reach = t;  // t: every column of the row
    for (int w = 0; w < GW; w++) {
      uint32_t x = row[w];
      const int pc = __popc(x);
      if (pc >= need) {
        for (int q = 1; q < need; q++) x &= x - 1;
        reach = 32 * w + __ffs(x) - 1;
        break;
      }
      need -= pc;
    }
    int e = e0;
    while (e < e1 && pcol[k][e] <= reach) e++;
    if (e == e0) {
      P.phs[i] = 0x7fffffff;
      P.phe[i] = 0;
    } else {
      P.phe[i] = e;
    }
  }
  __syncthreads();
  // ---- P1c: the kept entries, when they fit, compacted into shared memory
  // (rows in (class, node) order), where every later phase reads them
  bool compacted = false;
  {
    int kept = 0;
    for (int i0 = 0; i0 < 2 * g; i0 += nt) {
      const int i = i0 + tid;
      const int cnt = (i < 2 * g && P.phs[i] < P.phe[i]) ? P.phe[i] - P.phs[i] : 0;
      int total;
      block_scan(cnt, total, SM.scan);
      kept += total;
    }
    if (kept <= kEntCache) {
      int running = 0;
      for (int i0 = 0; i0 < 2 * g; i0 += nt) {
        const int i = i0 + tid;
        const int e0 = i < 2 * g ? P.phs[i] : 0, e1 = i < 2 * g ? P.phe[i] : 0;
        const int cnt = e0 < e1 ? e1 - e0 : 0;
        int total;
        const int off = running + block_scan(cnt, total, SM.scan);
        if (cnt) {
          const int k = i / g;
          for (int q = 0; q < cnt; q++) {
            P.ephi[off + q] = phi[k][e0 + q];
            P.epcol[off + q] = pcol[k][e0 + q];
          }
          P.phs[i] = off;
          P.phe[i] = off + cnt;
        }
        running += total;
      }
      phi[0] = phi[1] = P.ephi;
      pcol[0] = pcol[1] = P.epcol;
      compacted = true;
      __syncthreads();
    }
  }

  // rows holding flip entries, ascending, per class, and entry totals
  if (tid == 0) SM.nent[0] = SM.nent[1] = 0;
  for (int k = 0; k < 2; k++) {
    int running = 0;
    for (int t0 = 0; t0 < g; t0 += nt) {
      const int t = t0 + tid;
      const int ne = (t < g) ? P.phe[k * g + t] - P.phs[k * g + t] : 0;
      int total;
      const int off = block_scan(ne > 0 ? 1 : 0, total, SM.scan);
      if (ne > 0) {
        P.rphi[k * g + running + off] = (uint16_t)t;
        atomicAdd(&SM.nent[k], ne);
      }
      running += total;
    }
    if (tid == 0) SM.nrphi[k] = running;
  }
  __syncthreads();

  // ---- P2: capped lists of the two full networks; their hashes summed per
  // warp, then one atomic per warp and class
  unsigned long long hsum[2] = {0ull, 0ull};
  for (int i = tid; i < 2 * g; i += nt) {
    const int k = i / g, t = i % g;
    ListGen G;
    gen_for(G, sd, P, phi[k], pcol[k], k, t, nullptr);
    uint64_t h = node_hash_init(sd.salt, t);
    int cnt = 0;
    int ps[3] = {0xFFFF, 0xFFFF, 0xFFFF};
    while (cnt < sd.mp) {
      int j = G.next();
      if (j < 0) break;
      if (cnt < 3) ps[cnt] = j;
      h = node_hash_step(h, j);
      cnt++;
    }
    P.fcnt[i] = (uint16_t)cnt;
    for (int q = 0; q < 3; q++) P.fps[i * 3 + q] = (uint16_t)ps[q];
    P.fh[i] = h;
    hsum[k] += h;
  }
  for (int o = 16; o > 0; o >>= 1) {
    hsum[0] += __shfl_xor_sync(0xffffffffu, hsum[0], o);
    hsum[1] += __shfl_xor_sync(0xffffffffu, hsum[1], o);
  }
  if (lane == 0) {
    atomicAdd(&SM.HF[0], hsum[0]);
    atomicAdd(&SM.HF[1], hsum[1]);
  }
  __syncthreads();
  for (int t = tid; t < g; t += nt) {
    if (!lists_equal(sd, P, phi, pcol, t, 0, nullptr, 1, nullptr)) {
      int idx = atomicAdd(&SM.ndab, 1);
      P.dab[idx] = (uint16_t)t;
    }
  }
  __syncthreads();

  // ---- P3: networks grouped by signature.  The network of left-out sample
  // sigma is its class's full network with the pair tables of sigma's cells
  // removed, i.e. the full rows XOR the flip entries that sigma triggers (entry
  // (t, j, fb) fires when fb holds the bit of sigma's states at t and j).
  // Samples that trigger the same entries have equal networks, so lists are
  // generated once per distinct signature.  Signature = additive hash of the
  // triggered entry ordinals (salted per class; never 0 when non-empty), with
  // the exact bitset alongside when the class has <= 64 entries.
  const unsigned long long ksalt0 = mix64(sd.salt ^ 0x243F6A8885A308D3ull);
  const unsigned long long ksalt1 = mix64(sd.salt ^ 0x13198A2E03707344ull);
  const int n = sd.n;
  const int HTs = L.HT;
  auto class_of = [&](int s) -> int { return (s == 0) ? 0 : (s == S - 1) ? 1 : (s <= sd.nA ? 0 : 1); };
  // triggered entries of sample sigma in class k: hash (0 when none) and bits
  auto signature = [&](int k, int sigma, unsigned long long &bits) -> unsigned long long {
    const int nrk = SM.nrphi[k];
    const bool exact = SM.nent[k] <= 64;
    const unsigned long long ks = k ? ksalt1 : ksalt0;
    const uint32_t *ph = phi[k];
    const uint16_t *pc = pcol[k];
    unsigned long long key = 0;
    bits = 0;
    int ord = 0, any = 0;
    for (int r = 0; r < nrk; r++) {
      const int t = P.rphi[k * g + r];
      const int e0 = P.phs[k * g + t], e1 = P.phe[k * g + t];
      const int a = st_of(sd.vals[(size_t)t * n + sigma]);
      if (a <= 2) {
        for (int e = e0; e < e1; e++) {
          const int b = st_of(sd.vals[(size_t)pc[e] * n + sigma]);
          if (b <= 2 && ((ph[e] >> (3 * a + b)) & 1u)) {
            const int o = ord + (e - e0);
            key += mix64(ks + (unsigned long long)o);
            if (exact) bits |= 1ull << o;
            any = 1;
          }
        }
      }
      ord += e1 - e0;
    }
    return any ? (key | 1ull) : 0ull;
  };
  // The same from the trigger bitsets: entry o of class k fires for sample
  // sigma when bit sigma of trig[(koff + o) W ..] is set.  Until the BDeu
  // phase, the task prefix (tq) holds the entries by ordinal and the base
  // score array (fsc) the bitsets.
  uint32_t *ent = (uint32_t *)P.tq;
  uint64_t *trig = (uint64_t *)P.fsc;
  auto signature_t = [&](int k, int sigma, unsigned long long &bits) -> unsigned long long {
    const int ne = SM.nent[k];
    const bool exact = ne <= 64;
    const unsigned long long ks = k ? ksalt1 : ksalt0;
    const uint64_t *T = trig + (size_t)(k ? SM.nent[0] : 0) * W + (sigma >> 6);
    const int sh = sigma & 63;
    unsigned long long key = 0;
    bits = 0;
    int any = 0;
    for (int o = 0; o < ne; o++) {
      if ((T[(size_t)o * W] >> sh) & 1ull) {
        key += mix64(ks + (unsigned long long)o);
        if (exact) bits |= 1ull << o;
        any = 1;
      }
    }
    return any ? (key | 1ull) : 0ull;
  };
  // Trigger bitsets, when they fit: entries by ordinal (rows in order, then
  // entries in position order, as signature() counts them), then per entry
  // and sample word the OR over the set bits (a, b) of fb of
  // plane(t, a) & plane(j, b), read 64 samples at a time.
  const int ne0 = SM.nent[0], ne1 = SM.nent[1];
  const bool tbits = ne0 + ne1 <= 2 * kItems + 1 && (ne0 + ne1) * W <= 4 * g;
  if (tbits) {
    for (int k = 0; k < 2; k++) {
      const int nrk = SM.nrphi[k];
      int running = k ? ne0 : 0;
      for (int r0 = 0; r0 < nrk; r0 += nt) {
        const int r = r0 + tid;
        int t = 0, e0 = 0, cnt = 0;
        if (r < nrk) {
          t = P.rphi[k * g + r];
          e0 = P.phs[k * g + t];
          cnt = P.phe[k * g + t] - e0;
        }
        int total;
        const int off = block_scan(cnt, total, SM.scan);
        for (int i = 0; i < cnt; i++)
          ent[running + off + i] = (uint32_t)t | ((uint32_t)pcol[k][e0 + i] << 9) |
                                     ((phi[k][e0 + i] & 0x1FFu) << 18);
        running += total;
      }
    }
    __syncthreads();
    for (int idx = tid; idx < (ne0 + ne1) * W; idx += nt) {
      const int o = idx / W, w = idx - o * W;
      const uint32_t en = ent[o];
      const uint32_t fb = en >> 18;
      const uint64_t *pt = sd.planes + (size_t)(en & 0x1FFu) * 3 * W + w;
      const uint64_t *pj = sd.planes + (size_t)((en >> 9) & 0x1FFu) * 3 * W + w;
      const uint64_t t0 = pt[0], t1 = pt[W], t2 = pt[2 * W];
      const uint64_t j0 = pj[0], j1 = pj[W], j2 = pj[2 * W];
      uint64_t x = 0;
      if (fb & 0x001u) x |= t0 & j0;
      if (fb & 0x002u) x |= t0 & j1;
      if (fb & 0x004u) x |= t0 & j2;
      if (fb & 0x008u) x |= t1 & j0;
      if (fb & 0x010u) x |= t1 & j1;
      if (fb & 0x020u) x |= t1 & j2;
      if (fb & 0x040u) x |= t2 & j0;
      if (fb & 0x080u) x |= t2 & j1;
      if (fb & 0x100u) x |= t2 & j2;
      trig[idx] = x;
    }
  }
  // Tables (key -> smallest network index) in shared memory first; a unit
  // whose keys do not fit there within kSmProbes probes uses its global
  // table of HT slots instead (initialised only then).
  unsigned long long *smk = P.itk;
  int *smv = (int *)P.acc;
  auto table_init = [&](unsigned long long *k, int *v, int slots, unsigned long long empty) {
    for (int i = tid; i < slots; i += nt) {
      k[i] = empty;
      v[i] = 0x7fffffff;
    }
  };
  const MinTable sig_sm{smk, smv, kSmSlots - 1, 0ull, kSmProbes};
  const MinTable sig_gl{hsk, hsv, (unsigned)HTs - 1, 0ull, (unsigned)HTs};
  table_init(smk, smv, kSmSlots, 0ull);
  if (tid == 0) {
    skey[0] = skey[S - 1] = 0ull;
    sbits[0] = sbits[S - 1] = 0ull;
    srep[0] = 0;
    srep[S - 1] = S - 1;
    SM.tfull = 0;
    SM.firstE2 = S - 1;
  }
  __syncthreads();
  for (int s = 1 + tid; s < S - 1; s += nt) {
    unsigned long long bits;
    const unsigned long long key = tbits ? signature_t(class_of(s), sig[s - 1], bits)
                                         : signature(class_of(s), sig[s - 1], bits);
    skey[s] = key;
    sbits[s] = bits;
    if (key && !sig_sm.insert_min(key, s)) SM.tfull = 1;
    if (!key && s > sd.nA) atomicMin(&SM.firstE2, s);
  }
  if (tid == 0) SM.nwl = 0;
  __syncthreads();
  const bool sig_global = SM.tfull != 0;
  if (sig_global) {
    table_init(hsk, hsv, HTs, 0ull);
    __syncthreads();
    for (int s = 1 + tid; s < S - 1; s += nt)
      if (skey[s]) sig_gl.insert_min(skey[s], s);
    __syncthreads();
  }
  const MinTable &sig_tab = sig_global ? sig_gl : sig_sm;
  // representatives, the work list of distinct signatures, and an exact check
  // that every network shares its representative's triggered entries
  for (int s = 1 + tid; s < S - 1; s += nt) {
    const unsigned long long key = skey[s];
    int rep = s;
    if (key) {
      rep = sig_tab.get(key);
      if (rep == s) {
        wl[atomicAdd(&SM.nwl, 1)] = s;
      } else {
        const int k = class_of(s);
        bool ok = (class_of(rep) == k);
        if (ok && SM.nent[k] <= 64) {
          ok = (sbits[s] == sbits[rep]);
        } else if (ok) {
          // more than 64 entries: compare the triggered sets entry by entry
          const int sa = sig[s - 1], sb = sig[rep - 1];
          const int nrk = SM.nrphi[k];
          for (int r = 0; ok && r < nrk; r++) {
            const int t = P.rphi[k * g + r];
            const int aa = st_of(sd.vals[(size_t)t * n + sa]), ab = st_of(sd.vals[(size_t)t * n + sb]);
            for (int e = P.phs[k * g + t]; ok && e < P.phe[k * g + t]; e++) {
              const int j = pcol[k][e];
              const int ba = st_of(sd.vals[(size_t)j * n + sa]), bb = st_of(sd.vals[(size_t)j * n + sb]);
              const bool fa = aa <= 2 && ba <= 2 && ((phi[k][e] >> (3 * aa + ba)) & 1u);
              const bool fbb = ab <= 2 && bb <= 2 && ((phi[k][e] >> (3 * ab + bb)) & 1u);
              ok = (fa == fbb);
            }
          }
        }
        if (!ok) atomicOr(&SM.status, kUnitHashCollision);
      }
    }
    srep[s] = rep;
  }
  if (tid == 0) {
    unsigned long long *R0 = rec;
    unsigned long long *R1 = rec + (size_t)(S - 1) * L.rec_words;
    R0[0] = SM.HF[0];
    R0[1] = 0;
    R1[0] = SM.HF[1];
    R1[1] = 0;
  }
  __syncthreads();
  // the capped list of each row with 1..kMemoE kept entries under every
  // non-empty subset of them (the entries a left-out sample triggers):
  // the record entry (t, first three parents) when it differs from the
  // full network's list, and its hash; one thread per (row, subset).
  // Packed by row: row i's 2^e - 1 lists from moff[i] on (the task prefix
  // array is free from the signatures until the BDeu phase), so the lists
  // the records read lie close together.
  unsigned long long *memo = (unsigned long long *)(scr + L.memo);
  int *moff = P.tq;
  uint32_t *used = (uint32_t *)P.fsc;
  // a changed node's key (node, first three parents) unless it equals the
  // full network's: the items scored in the BDeu phase
  auto differs = [&](int k, unsigned long long e) -> bool {
    const int t = (int)(e & 0x3FFF), np = (int)((e >> 14) & 3);
    const int fnp = P.fcnt[k * g + t] < 3 ? P.fcnt[k * g + t] : 3;
    if (np != fnp) return true;
    for (int q = 0; q < np; q++)
      if ((int)((e >> (16 + 16 * q)) & 0xFFFF) != (int)P.fps[(k * g + t) * 3 + q]) return true;
    return false;
  };
  {
    int running = 0;
    for (int i0 = 0; i0 < 2 * g; i0 += nt) {
      const int i = i0 + tid;
      int sz = 0;
      if (i < 2 * g) {
        const int e = P.phe[i] - P.phs[i];
        sz = (e >= 1 && e <= kMemoE) ? (1 << e) - 1 : 0;
      }
      int total;
      const int off = block_scan(sz, total, SM.scan);
      if (i < 2 * g) moff[i] = running + off;
      running += total;
    }
    // the lists the records use, one bit each (the base score array is
    // free until the BDeu phase: 32 g bytes >= 2 g kMemoSub bits)
    for (int w = tid; w < (running + 31) / 32; w += nt) used[w] = 0u;
    if (tid == 0) SM.nlg = 0;
    __syncthreads();
  }
  for (int task = tid; task < 2 * g * kMemoSub; task += nt) {
    const int i = task / kMemoSub, msub = task - i * kMemoSub + 1;
    const int e0 = P.phs[i], e1 = P.phe[i];
    if (e0 >= e1 || e1 - e0 > kMemoE || msub >= (1 << (e1 - e0))) continue;
    const int k = i / g, t = i - k * g;
    const uint32_t *row = P.rows + (size_t)i * GW;
    ListGen Go;
    gen_for(Go, sd, P, phi[k], pcol[k], k, t, nullptr);
    uint64_t h = node_hash_init(sd.salt, t);
    int cnt = 0, ps[3] = {0xFFFF, 0xFFFF, 0xFFFF};
    bool diff = false;
    for (int w = 0; w < GW && cnt < sd.mp; w++) {
      uint32_t x = row[w];
      for (int q = 0; q < e1 - e0; q++) {
        const int j = pcol[k][e0 + q];
        if (((msub >> q) & 1) && (j >> 5) == w) x ^= 1u << (j & 31);
      }
      while (x && cnt < sd.mp) {
        const int j = 32 * w + __ffs(x) - 1;
        x &= x - 1;
        if (Go.next() != j) diff = true;
        if (cnt < 3) ps[cnt] = j;
        h = node_hash_step(h, j);
        cnt++;
      }
    }
    // a shorter list than the full network's differs too
    if (cnt < sd.mp && Go.next() >= 0) diff = true;
    unsigned long long *M = memo + ((size_t)moff[i] + (msub - 1)) * 2;
    M[0] = diff ? ((unsigned long long)t | ((unsigned long long)(cnt < 3 ? cnt : 3) << 14) |
                   ((unsigned long long)(ps[0] & 0xFFFF) << 16) |
                   ((unsigned long long)(ps[1] & 0xFFFF) << 32) |
                   ((unsigned long long)(ps[2] & 0xFFFF) << 48))
                : ~0ull;
    M[1] = h;
  }
  __syncthreads();

  // one record per distinct signature: changed nodes (capped list differs
  // from the full network's) with their lists, and the network hash.  A
  // warp per network.  A first pass over the rows holding entries finds
  // the rows whose entries the left-out sample triggers (shared memory
  // only) and lists them (row | subset << 16, or a merged-row mark) in the
  // warp's part of the BDeu item arrays, idle from the signatures until the
  // dedup; a second pass looks up (or merges) the listed rows' lists 32 at
  // a time, so a network's memo loads are in flight together.
  constexpr int kMergedRow = 0x8000;  // a row with more than kMemoE entries
  int8_t *myst = P.stsig + (size_t)warp * st_stride(g);
  uint32_t *lsts = reinterpret_cast<uint32_t *>(P.itk);  // P.acc follows P.itk
  const int lcap = (int)((reinterpret_cast<uint32_t *>(P.acc + 2 * kItems) - lsts) / nw) & ~31;
  uint32_t *lst = lsts + (size_t)warp * lcap;
  const int nwl = SM.nwl;
  for (int wi = warp; wi < nwl; wi += nw) {
    const int s = wl[wi];
    const int k = class_of(s);
    const int sigma = sig[s - 1];
    unsigned long long *R = rec + (size_t)s * L.rec_words;
    const int nrk = SM.nrphi[k];
    load_stsig(sd, sigma, myst, lane);
    unsigned long long dh = 0;
    int nchg = 0, nl = 0;
    auto flush = [&]() {
      __syncwarp();
      for (int l0 = 0; l0 < nl; l0 += 32) {
        const int l = l0 + lane;
        bool changed = false;
        unsigned long long hn = 0, ent = 0;
        int t = 0;
        if (l < nl) {
          const uint32_t le = lst[l];
          t = (int)(le & 0xFFFFu);
          const int sub = (int)(le >> 16);
          if (sub != kMergedRow) {
            const int mi = moff[k * g + t] + sub - 1;
            const unsigned long long *M = memo + (size_t)mi * 2;
            if (M[0] != ~0ull) {
              changed = true;
              ent = M[0];
              hn = M[1];
              if (!((used[mi >> 5] >> (mi & 31)) & 1u)) atomicOr(&used[mi >> 5], 1u << (mi & 31));
            }
          } else {
            ListGen Gn, Go;
            gen_for(Gn, sd, P, phi[k], pcol[k], k, t, myst);
            gen_for(Go, sd, P, phi[k], pcol[k], k, t, nullptr);
            uint64_t h = node_hash_init(sd.salt, t);
            int cnt = 0, ps[3] = {0xFFFF, 0xFFFF, 0xFFFF};
            bool diff = false;
            for (int i = 0; i < sd.mp; i++) {
              int x = Gn.next(), y = Go.next();
              if (x != y) diff = true;
              if (x < 0) break;
              if (cnt < 3) ps[cnt] = x;
              h = node_hash_step(h, x);
              cnt++;
            }
            if (diff) {
              changed = true;
              hn = h;
              ent = (unsigned long long)t | ((unsigned long long)(cnt < 3 ? cnt : 3) << 14) |
                    ((unsigned long long)(ps[0] & 0xFFFF) << 16) |
                    ((unsigned long long)(ps[1] & 0xFFFF) << 32) |
                    ((unsigned long long)(ps[2] & 0xFFFF) << 48);
              if (differs(k, ent)) {
                // logged in the signature table's keys (free from here on)
                const int ix = atomicAdd(&SM.nlg, 1);
                if (ix < HTs) hsk[ix] = ent;
              }
            }
          }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, changed);
        if (changed) {
          const int pos = nchg + __popc(bal & ((1u << lane) - 1u));
          dh += hn - P.fh[k * g + t];
          if (pos < bd.kmax) R[2 + pos] = ent;
        }
        nchg += __popc(bal);
      }
      nl = 0;
      __syncwarp();
    };
    for (int t0 = 0; t0 < nrk; t0 += 32) {
      const int t = (t0 + lane < nrk) ? (int)P.rphi[k * g + t0 + lane] : -1;
      int sub = 0;
      if (t >= 0 && myst[t] <= 2) {
        // the entries of row t that sample sigma triggers
        const int sr = myst[t] * 3;
        const int e0 = P.phs[k * g + t], e1 = P.phe[k * g + t];
        if (e1 - e0 <= kMemoE) {
          for (int q = 0; q < e1 - e0; q++) {
            const int sc = myst[pcol[k][e0 + q]];
            if (sc <= 2 && (((phi[k][e0 + q] & 0x1FFu) >> (sr + sc)) & 1u)) sub |= 1 << q;
          }
        } else {
          bool flips = false;
          for (int i = e0; i < e1 && !flips; i++) {
            const int sc = myst[pcol[k][i]];
            flips = sc <= 2 && (((phi[k][i] & 0x1FFu) >> (sr + sc)) & 1u);
          }
          if (flips) sub = kMergedRow;
        }
      }
      const unsigned bal = __ballot_sync(0xffffffffu, sub != 0);
      if (sub) lst[nl + __popc(bal & ((1u << lane) - 1u))] = (uint32_t)t | ((uint32_t)sub << 16);
      nl += __popc(bal);
      if (nl > lcap - 32) flush();
    }
    flush();
    for (int o = 16; o > 0; o >>= 1) dh += __shfl_down_sync(0xffffffffu, dh, o);
    if (lane == 0) {
      R[0] = SM.HF[k] + dh;
      R[1] = (unsigned long long)nchg;
      if (nchg > bd.kmax) {
        atomicOr(&SM.status, kUnitKmaxOverflow);
        atomicMax(&SM.maxchg, nchg);
      }
    }
  }
  __syncthreads();
  if (SM.status & kUnitKmaxOverflow) {
    if (tid == 0) {
      // bits 16-31: the records the unit needs (the host re-runs it with
      // room for them)
      bd.status[u] = SM.status | ((unsigned)min(SM.maxchg, 0xFFFF) << 16);
      bd.js[u] = __longlong_as_double(0x7ff8000000000000ll);
      bd.U[u] = -1;
    }
    return;
  }
  // record of any network: the full network's for an empty signature, else
  // its signature representative's
  auto rec_of = [&](int s) -> const unsigned long long * {
    const int r = (s == 0 || s == S - 1) ? s : (skey[s] == 0 ? (class_of(s) ? S - 1 : 0) : srep[s]);
    return rec + (size_t)r * L.rec_words;
  };

  // ---- P4: first-occurrence dedup.  Networks without changed nodes are
  // their class's full network: class-1 ones duplicate network 0, class-2
  // ones the first class-2 network without changes (firstB0).  Every other
  // network shares its signature representative's network, and that
  // representative comes first.  So the unique networks are the candidates
  // -- network 0, firstB0 and the signature representatives with changes --
  // that are the first occurrence of their network hash; only they go into
  // the table, and only they are looked up.
  const int HT = L.HT;
  const int nrep = SM.nwl;  // signature representatives in wl
  // firstB0: the first class-2 network with an empty signature, or a class-2
  // representative (its group's first network) whose record has no changes
  if (tid == 0) {
    SM.firstB0 = SM.firstE2;
    SM.ncand = 2;
  }
  __syncthreads();
  for (int i = tid; i < nrep; i += nt) {
    const int s = wl[i];
    if (s > sd.nA && rec[(size_t)s * L.rec_words + 1] == 0) atomicMin(&SM.firstB0, s);
  }
  __syncthreads();
  const int firstB0 = SM.firstB0;
  // candidates (in the per-network id array, no longer needed per network)
  int *cand = uid;
  if (tid == 0) {
    cand[0] = 0;
    cand[1] = firstB0;
  }
  for (int i = tid; i < nrep; i += nt) {
    const int s = wl[i];
    if (rec[(size_t)s * L.rec_words + 1] != 0) cand[atomicAdd(&SM.ncand, 1)] = s;
  }
  // network table: shared memory first (the signature table is done with),
  // the global one when the candidates do not fit
  const MinTable net_sm{smk, smv, kSmSlots - 1, ~0ull, kSmProbes};
  const MinTable net_gl{htk, htv, (unsigned)HT - 1, ~0ull, (unsigned)HT};
  auto net_key = [&](int s) -> unsigned long long {
    unsigned long long key = rec_of(s)[0];
    return key == ~0ull ? key ^ 1ull : key;
  };
  table_init(smk, smv, kSmSlots, ~0ull);
  if (tid == 0) SM.tfull = 0;
  __syncthreads();
  const int m = SM.ncand;
  for (int i = tid; i < m; i += nt)
    if (!net_sm.insert_min(net_key(cand[i]), cand[i])) SM.tfull = 1;
  // bitmap of the unique networks over the network ids, and the merged
  // candidates with their representatives (both in the signature-bitset
  // scratch, free after the signature phase)
  uint32_t *ubits = (uint32_t *)sbits;
  const int nbw = (S + 31) >> 5;
  int *vrep = (int *)sbits + nbw;
  for (int i = tid; i < nbw; i += nt) ubits[i] = 0u;
  if (tid == 0) SM.nwl = 0;
  __syncthreads();
  const bool net_global = SM.tfull != 0;
  if (net_global) {
    table_init(htk, htv, HT, ~0ull);
    __syncthreads();
    for (int i = tid; i < m; i += nt) net_gl.insert_min(net_key(cand[i]), cand[i]);
    __syncthreads();
  }
  const MinTable &net_tab = net_global ? net_gl : net_sm;
  for (int i = tid; i < m; i += nt) {
    const int c = cand[i];
    const int r = net_tab.get(net_key(c));
    if (r == c) {
      atomicOr(&ubits[c >> 5], 1u << (c & 31));
    } else {
      // merged by hash: checked list by list below
      const int k = atomicAdd(&SM.nwl, 1);
      wl[k] = c;
      vrep[k] = r;
    }
  }
  __syncthreads();
  // unique networks in network order: the set bits before each one
  int running = 0;
  for (int w0 = 0; w0 < nbw; w0 += nt) {
    const int w = w0 + tid;
    const uint32_t word = w < nbw ? ubits[w] : 0u;
    int total;
    const int off = block_scan(__popc(word), total, SM.scan);
    for (uint32_t x = word; x; x &= x - 1) {
      const int b = __ffs(x) - 1;
      urep[running + off + __popc(word & ((1u << b) - 1u))] = 32 * w + b;
    }
    running += total;
  }
  if (tid == 0) SM.U = running;
  __syncthreads();
  const int U = SM.U;
  // exact check of every hash merge (warp per merged network)
  const int nver = SM.nwl;
  for (int wi = warp; wi < nver; wi += nw) {
    const int s = wl[wi];
    const int r = vrep[wi];
    int ks, ss, kr, sr;
    net_of(s, sd, sig, ks, ss);
    net_of(r, sd, sig, kr, sr);
    const unsigned long long *Rs = rec_of(s);
    const unsigned long long *Rr = rec_of(r);
    const int ns = (int)Rs[1], nr = (int)Rr[1];
    // both are their class's full network: equal by construction
    if (ks == kr && ns == 0 && nr == 0) continue;
    bool ok = true;
    // states at the left-out sample of s, shared by the warp
    load_stsig(sd, ss, myst, lane);
    if (ks == kr) {
      if (ns != nr) ok = false;
      // every changed node of s must be changed in r
      for (int i = lane; ok && i < ns; i += 32) {
        int t = (int)(Rs[2 + i] & 0x3FFF);
        bool found = false;
        for (int j = 0; j < nr; j++)
          if ((int)(Rr[2 + j] & 0x3FFF) == t) { found = true; break; }
        if (!found) ok = false;
      }
      ok = __all_sync(0xffffffffu, ok);
    }
    // node-by-node list comparison: s's lists from the shared states, r's
    // lists with the states of r's left-out sample read from global memory
    if (ok) {
      // nodes to compare: changed of s, changed of r, and DAB when classes differ
      const int nd = (ks != kr) ? SM.ndab : 0;
      const int total = ns + nr + nd;
      for (int i = lane; i < total; i += 32) {
        int t;
        if (i < ns) t = (int)(Rs[2 + i] & 0x3FFF);
        else if (i < ns + nr) t = (int)(Rr[2 + (i - ns)] & 0x3FFF);
        else t = P.dab[i - ns - nr];
        ListGen a;
        gen_for(a, sd, P, phi[ks], pcol[ks], ks, t, ss >= 0 ? myst : nullptr);
        const int GWl = sd.GW;
        const int8_t *rT = sd.valsT + (size_t)(sr >= 0 ? sr : 0) * st_stride(sd.g);
        const int strow_r = (sr >= 0) ? rT[t] : 3;
        const uint32_t *rowr = P.rows + ((size_t)kr * g + t) * GWl;
        int fi = P.phs[kr * g + t], fe = P.phe[kr * g + t];
        int w = 0;
        auto flipw = [&](int ww) -> uint32_t {
          uint32_t mm = 0;
          if (sr < 0 || strow_r > 2) return 0u;
          const int hi = 32 * (ww + 1);
          while (fi < fe) {
            int col = pcol[kr][fi];
            if (col >= hi) break;
            int sc = rT[col];
            if (sc <= 2 && ((phi[kr][fi] & 0x1FFu) >> (strow_r * 3 + sc)) & 1u) mm |= 1u << (col - 32 * ww);
            fi++;
          }
          return mm;
        };
        uint32_t word = GWl > 0 ? (rowr[0] ^ flipw(0)) : 0u;
        auto nextb = [&]() -> int {
          while (true) {
            if (word) {
              int j = __ffs(word) - 1;
              word &= word - 1;
              return 32 * w + j;
            }
            if (++w >= GWl) return -1;
            word = rowr[w] ^ flipw(w);
          }
        };
        for (int q = 0; q < sd.mp; q++) {
          int x = a.next(), y = nextb();
          if (x != y) { ok = false; break; }
          if (x < 0) break;
        }
      }
      ok = __all_sync(0xffffffffu, ok);
    }
    if (!ok && lane == 0) atomicOr(&SM.status, kUnitHashCollision);
    __syncwarp();
  }
  __syncthreads();
  if (bd.stats && tid == 0)
    atomicAdd(&bd.stats[4 * (size_t)bd.uslot[u] + 3], (unsigned long long)(S - U));

  // ---- Keys of the changed nodes' lists.  The leave-one-out networks of a
  // unit share most of their changed nodes' lists (one flip near a
  // threshold changes the same node in every network whose left-out sample
  // triggers it), so the items hold few distinct keys (node, first three
  // parents): ~240 among ~24000 items per unit when nearly every pair sits
  // near the threshold.  Each distinct key is scored once, in a
  // shared-memory table of KT slots (in the flip-entry cache, which no phase
  // reads from here on), and every item adds its key's score.  The keys are
  // the memo lists the records used and the logged merged-row lists; when
  // more were logged than the log holds, the items are walked instead.  A
  // key that finds no slot within kKeyProbes probes: every item is scored
  // on its own.
  constexpr int kKeyProbes = 64;
  const int KT = HT < kKeyT ? HT : kKeyT;  // slot-indexed scores fit ksc ([HT][2])
  unsigned long long *kt = (unsigned long long *)P.ephi;
  const unsigned kmask = (unsigned)KT - 1u;
  if (compacted && bd.keep_slot && bd.keep_slot[u] >= 0) {
    // the detailed outputs still read the flip entries: back to the
    // unit's scratch, each class's (nent[k] <= c) to its own arrays, the
    // class-2 row ranges shifted to start at 0
    const int ne0 = SM.nent[0], ne = ne0 + SM.nent[1];
    for (int k = 0; k < 2; k++) {
      uint32_t *gphi = (uint32_t *)(scr + L.phi[k]);
      uint16_t *gpcol = (uint16_t *)(scr + L.pcol[k]);
      const int e0 = k ? ne0 : 0, e1 = k ? ne : ne0;
      for (int i = e0 + tid; i < e1; i += nt) {
        gphi[i - e0] = P.ephi[i];
        gpcol[i - e0] = P.epcol[i];
      }
      phi[k] = gphi;
      pcol[k] = gpcol;
    }
    for (int t = tid; t < g; t += nt)
      if (P.phs[g + t] < P.phe[g + t]) {
        P.phs[g + t] -= ne0;
        P.phe[g + t] -= ne0;
      }
    __syncthreads();
  }
  for (int i = tid; i < KT; i += nt) kt[i] = ~0ull;
  if (tid == 0) SM.tfull = 0;
  __syncthreads();
  auto insert_key = [&](unsigned long long rc) {
    unsigned slot = (unsigned)(mix64(rc) & kmask);
    for (int pr = 0; pr < kKeyProbes; pr++, slot = (slot + 1u) & kmask) {
      // a slot only ever goes from empty to its final key: a read first,
      // the atomic only on an empty slot
      unsigned long long cur = kt[slot];
      if (cur == ~0ull) cur = atomicCAS(&kt[slot], ~0ull, rc);
      if (cur == ~0ull || cur == rc) return;
    }
    SM.tfull = 1;
  };
  const bool keys_logged = !bd.key_walk && SM.nlg <= HTs;
  if (keys_logged) {
    for (int task = tid; task < 2 * g * kMemoSub; task += nt) {
      const int i = task / kMemoSub, q = task - i * kMemoSub;
      const int e = P.phe[i] - P.phs[i];
      if (e < 1 || e > kMemoE || q >= (1 << e) - 1) continue;
      const int mi = moff[i] + q;
      if (!((used[mi >> 5] >> (mi & 31)) & 1u)) continue;
      const unsigned long long ent = memo[(size_t)mi * 2];
      if (differs(i / g, ent)) insert_key(ent);
    }
    for (int x = tid; x < SM.nlg; x += nt) insert_key(hsk[x]);
  }
  __syncthreads();

  // ---- P5: BDeu.  Base node scores of the two full networks: nodes
  // without parents from the state counts, the others as flat tasks; a
  // class-2 node whose capped parents equal the class-1 one copies its score.
  auto same_as_class1 = [&](int t) -> bool {
    const int a = P.fcnt[t] < 3 ? P.fcnt[t] : 3, b = P.fcnt[g + t] < 3 ? P.fcnt[g + t] : 3;
    if (a != b) return false;
    for (int q = 0; q < a; q++)
      if (P.fps[t * 3 + q] != P.fps[(g + t) * 3 + q]) return false;
    return true;
  };
  for (int i = tid; i < 2 * g; i += nt) {
    if (P.fcnt[i] != 0) continue;
    const int k = i / g, t = i % g;
    P.fsc[(k * 2 + 0) * g + t] = bdeu_score0(sd, t, P.cnt3);
    P.fsc[(k * 2 + 1) * g + t] = bdeu_score0(sd, t, P.cnt3 + 3 * g);
  }
  bdeu_items(
      sd, P, SM.scan, 2 * g,
      [&](int i) -> unsigned long long {
        const int k = i / g, t = i % g;
        if (P.fcnt[i] == 0 || (k == 1 && same_as_class1(t))) return ~0ull;
        const int np = P.fcnt[i] < 3 ? P.fcnt[i] : 3;
        return (unsigned long long)t | ((unsigned long long)np << 14) |
               ((unsigned long long)P.fps[i * 3] << 16) |
               ((unsigned long long)P.fps[i * 3 + 1] << 32) |
               ((unsigned long long)P.fps[i * 3 + 2] << 48);
      },
      [&](int i, long long s1, long long s2) {
        const int k = i / g, t = i % g;
        if (P.fcnt[i] == 0 || (k == 1 && same_as_class1(t))) return;
        P.fsc[(k * 2 + 0) * g + t] = s1;
        P.fsc[(k * 2 + 1) * g + t] = s2;
      });
  for (int t = tid; t < g; t += nt)
    if (P.fcnt[g + t] != 0 && same_as_class1(t)) {
      P.fsc[(1 * 2 + 0) * g + t] = P.fsc[(0 * 2 + 0) * g + t];
      P.fsc[(1 * 2 + 1) * g + t] = P.fsc[(0 * 2 + 1) * g + t];
    }
  __syncthreads();
  for (int i = tid; i < 4; i += nt) {
    const int k = i / 2, cls = i % 2;
    long long s = 0;
    for (int t = 0; t < g; t++) s += P.fsc[(k * 2 + cls) * g + t];
    SM.base[cls][k] = s;
  }
  __syncthreads();
  // unique networks: base of their class + deltas of the changed nodes whose
  // capped list (first three parents) differs from the full network's; the
  // changed nodes of all unique networks form one flat item list
  // (prefix over the networks in wl)
  for (int uu = tid; uu < U; uu += nt) {
    int k, sigma;
    net_of(urep[uu], sd, sig, k, sigma);
    dist[uu] = SM.base[0][k];
    dist[S + uu] = SM.base[1][k];
  }
  {
    int running = 0;
    for (int u0 = 0; u0 < U; u0 += nt) {
      const int uu = u0 + tid;
      const int v = uu < U ? (int)rec_of(urep[uu])[1] : 0;
      int total;
      const int off = block_scan(v, total, SM.scan);
      if (uu < U) wl[uu] = running + off;
      running += total;
    }
    if (tid == 0) SM.nwl = running;
    __syncthreads();
  }
  const int nchg_all = SM.nwl;
  // item e -> (unique network, changed-node record)
  auto item_of = [&](int e, int &uu, int &k, unsigned long long &rec) {
    int lo = 0, hi = U - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (wl[mid] <= e) lo = mid;
      else hi = mid - 1;
    }
    uu = lo;
    int sigma;
    const int s = urep[uu];
    net_of(s, sd, sig, k, sigma);
    rec = rec_of(s)[2 + (e - wl[uu])];
  };
  // the score delta of item e, given its key's scores in both classes
  auto add_delta = [&](int uu, int k, unsigned long long rec, long long s1, long long s2) {
    const int t = (int)(rec & 0x3FFF), np = (int)((rec >> 14) & 3);
    if (np == 0) {
      s1 = bdeu_score0(sd, t, P.cnt3);
      s2 = bdeu_score0(sd, t, P.cnt3 + 3 * g);
    }
    atomicAdd((unsigned long long *)&dist[uu],
              (unsigned long long)(s1 - P.fsc[(k * 2 + 0) * g + t]));
    atomicAdd((unsigned long long *)&dist[S + uu],
              (unsigned long long)(s2 - P.fsc[(k * 2 + 1) * g + t]));
  };
  // the items of unique network uu whose list differs from the full
  // network's, in record order, read four records at a time
  auto for_items = [&](int uu, auto &&fn) {
    constexpr int kRecBatch = 4;
    const unsigned long long *R = rec_of(urep[uu]);
    const int nrec = (int)R[1];
    const int k = class_of(urep[uu]);
    for (int e0 = 0; e0 < nrec; e0 += kRecBatch) {
      unsigned long long rb[kRecBatch];
#pragma unroll
      for (int q = 0; q < kRecBatch; q++) rb[q] = e0 + q < nrec ? R[2 + e0 + q] : ~0ull;
#pragma unroll
      for (int q = 0; q < kRecBatch; q++)
        if (rb[q] != ~0ull && differs(k, rb[q])) fn(k, rb[q]);
    }
  };
  int *kpos = htv;  // key list index -> slot
  unsigned long long *klist = hsk;
  long long *ksc = (long long *)(scr + L.ksc);
  if (!keys_logged) {
    // a thread per unique network inserts its items' keys
    for (int uu = tid; uu < U; uu += nt)
      for_items(uu, [&](int, unsigned long long rc) { insert_key(rc); });
    __syncthreads();
  }
  if (!SM.tfull) {
    // the keys in slot order: key list and slot -> list index
    int nk = 0;
    for (int i0 = 0; i0 < KT; i0 += nt) {
      const int i = i0 + tid;
      const unsigned long long key = i < KT ? kt[i] : ~0ull;
      const bool has = key != ~0ull;
      int total;
      const int off = block_scan(has ? 1 : 0, total, SM.scan);
      if (has) {
        kpos[nk + off] = i;
        klist[nk + off] = key;
      }
      nk += total;
    }
    __syncthreads();
    bdeu_items(
        sd, P, SM.scan, nk, [&](int i) -> unsigned long long { return klist[i]; },
        [&](int i, long long s1, long long s2) {
          ksc[2 * kpos[i]] = s1;
          ksc[2 * kpos[i] + 1] = s2;
        });
    __syncthreads();
    // each network's deltas summed by its thread (exact integer sums)
    for (int uu = tid; uu < U; uu += nt) {
      long long d1 = 0, d2 = 0;
      for_items(uu, [&](int k, unsigned long long rc) {
        unsigned slot = (unsigned)(mix64(rc) & kmask);
        int pr = 0;
        while (kt[slot] != rc && ++pr < kKeyProbes) slot = (slot + 1u) & kmask;
        if (pr >= kKeyProbes) {  // not found: cannot happen; the unit is re-run
          atomicOr(&SM.status, kUnitHashCollision);
          return;
        }
        const int t = (int)(rc & 0x3FFF), np = (int)((rc >> 14) & 3);
        long long s1 = ksc[2 * slot], s2 = ksc[2 * slot + 1];
        if (np == 0) {
          s1 = bdeu_score0(sd, t, P.cnt3);
          s2 = bdeu_score0(sd, t, P.cnt3 + 3 * g);
        }
        d1 += s1 - P.fsc[(k * 2 + 0) * g + t];
        d2 += s2 - P.fsc[(k * 2 + 1) * g + t];
      });
      dist[uu] += d1;
      dist[S + uu] += d2;
    }
    __syncthreads();  // every network's score is complete before it is read
  } else {
    bdeu_items(
        sd, P, SM.scan, nchg_all,
        [&](int e) -> unsigned long long {
          int uu, k;
          unsigned long long rec;
          item_of(e, uu, k, rec);
          if (!differs(k, rec)) return ~0ull;
          return rec;  // t | np << 14 | parents: the item key format
        },
        [&](int e, long long s1, long long s2) {
          int uu, k;
          unsigned long long rec;
          item_of(e, uu, k, rec);
          if (!differs(k, rec)) return;
          add_delta(uu, k, rec, s1, s2);
        });
  }

  // ---- P6: unique count and status; the normalisation and JS follow in
  // k_js (up to 32 units per warp) from the fixed-point scores in dist
  const int keep = bd.keep_slot ? bd.keep_slot[u] : -1;
  if (tid == 0) {
    bd.U[u] = U;
    bd.status[u] = SM.status;
  }

  // ---- P7: detailed outputs of kept units
  if (keep >= 0) {
    const int mpk = bd.mpk;
    const double fx = ldexp(1.0, -sd.lg_shift);
    for (int uu = tid; uu < U; uu += nt) {
      bd.out_ids[(size_t)keep * S + uu] = urep[uu];
      bd.out_dist[((size_t)keep * 2 + 0) * S + uu] = (double)dist[uu] * fx;
      bd.out_dist[((size_t)keep * 2 + 1) * S + uu] = (double)dist[S + uu] * fx;
    }
    for (int i = tid; i < 2 * g * GW; i += nt) {
      const int kt = i / GW, w = i - kt * GW;  // (class, node) row, word
      bd.out_rows[((size_t)keep * 2 * bd.keep_g + (kt / g) * bd.keep_g + kt % g) * bd.keep_gw + w] =
          P.rows[i];
    }
    // full capped lists of every unique network: warp per network
    for (int uu = warp; uu < U; uu += nw) {
      const int s = urep[uu];
      int k, sigma;
      net_of(s, sd, sig, k, sigma);
      load_stsig(sd, sigma, myst, lane);
      for (int t = lane; t < g; t += 32) {
        ListGen G;
        gen_for(G, sd, P, phi[k], pcol[k], k, t, sigma >= 0 ? myst : nullptr);
        int cnt = 0;
        while (cnt < sd.mp) {
          int j = G.next();
          if (j < 0) break;
          if (cnt < mpk) bd.out_par[(((size_t)keep * S + uu) * bd.keep_g + t) * mpk + cnt] = j;
          cnt++;
        }
        bd.out_cnt[((size_t)keep * S + uu) * bd.keep_g + t] = cnt;
      }
      __syncwarp();
    }
  }
}

// Normalisation (main.cu:1302-1404) and JS (main.cu:1406-1428) of every
// unit of a batch from the node-summed fixed-point scores k_units left in
// the unit's scratch: per class min, max and mean of the scores,
// likelihoods exp((d - mean) 10 / (max - min)) normalised to sum 1, then the
// two KL terms of kool() (routines.cu:42-60), zeros skipped, in FP64.  A
// unit k_units gave up on (U < 0) is left as it is.
//
// One warp per upw <= 32 units.  Lane l < upw holds unit upw w + l's
// minimum, maximum and mean (an exact integer sum); the warp then walks the
// units' unique networks as one flattened list, 32 at a time, so that every
// lane runs an FP64 exponential or logarithm whatever the units' sizes
// (units have ~8 unique networks, and FP64 is slow on this part: one warp
// per unit leaves three lanes in four idle).  upw is chosen so that the
// grid still covers the GPU (one unit per warp for small batches).  A
// unit's sums are formed in a fixed order: a segmented tree sum within each
// 32-network pass, the passes added in turn.  Between the two passes a
// network's exponentials replace its scores in the unit's dist array (the
// scores are not read after this kernel).
constexpr int kJsWarps = 8;
__global__ void __launch_bounds__(32 * kJsWarps) k_js(const __grid_constant__ BatchDev bd, int upw) {
  __shared__ int pre[kJsWarps][33];
  __shared__ double acc[kJsWarps][3][32];
  __shared__ long long red[kJsWarps][6][32];  // per unit: min, max (class 1, 2), sums
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int u0 = (blockIdx.x * kJsWarps + warp) * upw, u = u0 + lane;
  const bool mine = lane < upw && u < bd.B;
  const int Ur = mine ? bd.U[u] : 0;
  const int U = Ur > 0 ? Ur : 0;
  const int S = bd.sets[0].sd.S;  // n + 2, the same for every set of a batch
  // this lane's unit's scores (its set's slice of the scratch), shared with
  // the warp through shuffles
  unsigned long long dptr = 0ull;
  if (mine) {
    const BatchSet &bs = bd.sets[bd.uslot[u]];
    const UnitLayout L = unit_layout(bs.sd.c, S, bd.kmax);
    dptr = (unsigned long long)(bd.scratch + bs.sc0 + (size_t)(u - bs.u0) * bs.unit_bytes + L.dist);
  }
  auto dist_of = [&](int o) {
    return (long long *)__shfl_sync(0xffffffffu, dptr, o);
  };
  const int keep = (U > 0 && bd.keep_slot) ? bd.keep_slot[u] : -1;
  // the warp's units as prefix intervals of the flattened list
  int incl = U;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  pre[warp][lane] = incl - U;
  if (lane == 31) pre[warp][32] = incl;
  acc[warp][0][lane] = acc[warp][1][lane] = acc[warp][2][lane] = 0.0;
  red[warp][0][lane] = red[warp][2][lane] = LLONG_MAX;
  red[warp][1][lane] = red[warp][3][lane] = LLONG_MIN;
  red[warp][4][lane] = red[warp][5][lane] = 0;
  __syncwarp();
  const int total = pre[warp][32];
  // owner of network i: the last unit whose interval starts at or before i
  auto owner = [&](int i) {
    int lo = 0, hi = 31;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (pre[warp][mid] <= i) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  };
  // the run's last live lane: the one after it has another owner or is dead
  auto run_end = [&](int o, bool live) {
    const int on = __shfl_down_sync(0xffffffffu, o, 1);
    const bool nlive = __shfl_down_sync(0xffffffffu, live ? 1 : 0, 1) != 0;
    return live && (lane == 31 || on != o || !nlive);
  };
  // v combined (op) over this lane's run of equal owners, ending at the
  // run's last lane
  auto seg_scan = [&](long long v, int o, auto op) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, v, d);
      const int oy = __shfl_up_sync(0xffffffffu, o, d);
      if (lane >= d && oy == o) v = op(v, y);
    }
    return v;
  };
  auto mn = [](long long a, long long b) { return a < b ? a : b; };
  auto mx = [](long long a, long long b) { return a > b ? a : b; };
  auto ad = [](long long a, long long b) { return a + b; };
  // pass 0: each unit's smallest and largest score per class, then the sum
  // of the scores less the smallest (exact integers), over the flattened list
  for (int i0 = 0; i0 < total; i0 += 32) {
    const int i = i0 + lane;
    const bool live = i < total;
    const int o = live ? owner(i) : 31;
    const long long *d = dist_of(o);
    long long a = LLONG_MAX, b = LLONG_MAX;
    if (live) {
      const int uu = i - pre[warp][o];
      a = d[uu];
      b = d[S + uu];
    }
    const long long a0 = seg_scan(a, o, mn), a1 = seg_scan(live ? a : LLONG_MIN, o, mx);
    const long long b0 = seg_scan(b, o, mn), b1 = seg_scan(live ? b : LLONG_MIN, o, mx);
    if (run_end(o, live)) {
      red[warp][0][o] = mn(red[warp][0][o], a0);
      red[warp][1][o] = mx(red[warp][1][o], a1);
      red[warp][2][o] = mn(red[warp][2][o], b0);
      red[warp][3][o] = mx(red[warp][3][o], b1);
    }
    __syncwarp();
  }
  const long long l0 = red[warp][0][lane], h0 = red[warp][1][lane];
  const long long l1 = red[warp][2][lane], h1 = red[warp][3][lane];
  for (int i0 = 0; i0 < total; i0 += 32) {
    const int i = i0 + lane;
    const bool live = i < total;
    const int o = live ? owner(i) : 31;
    const long long *d = dist_of(o);
    const long long ol0 = __shfl_sync(0xffffffffu, l0, o), ol1 = __shfl_sync(0xffffffffu, l1, o);
    long long a = 0, b = 0;
    if (live) {
      const int uu = i - pre[warp][o];
      a = d[uu] - ol0;
      b = d[S + uu] - ol1;
    }
    const long long qa = seg_scan(a, o, ad), qb = seg_scan(b, o, ad);
    if (run_end(o, live)) {
      red[warp][4][o] += qa;
      red[warp][5][o] += qb;
    }
    __syncwarp();
  }
  double m0 = 0.0, m1 = 0.0, sA = 0.0, sB = 0.0;
  if (U > 0) {
    m0 = (double)red[warp][4][lane] / (double)U;
    m1 = (double)red[warp][5][lane] / (double)U;
    sA = 10.0 / (double)(h0 - l0);
    sB = 10.0 / (double)(h1 - l1);
  }
  // sum of v over this lane's run of equal owners, added to dst[owner] by
  // the run's last live lane
  auto seg_add = [&](double v, int o, bool live, double *dst) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, v, d);
      const int oy = __shfl_up_sync(0xffffffffu, o, d);
      if (lane >= d && oy == o) v += y;
    }
    const int on = __shfl_down_sync(0xffffffffu, o, 1);
    const bool nlive = __shfl_down_sync(0xffffffffu, live ? 1 : 0, 1) != 0;
    if (live && (lane == 31 || on != o || !nlive)) dst[o] += v;
  };
  // pass 1: the likelihoods, summed per unit and class
  for (int i0 = 0; i0 < total; i0 += 32) {
    const int i = i0 + lane;
    const bool live = i < total;
    const int o = live ? owner(i) : 31;
    const long long ol0 = __shfl_sync(0xffffffffu, l0, o), ol1 = __shfl_sync(0xffffffffu, l1, o);
    const double om0 = __shfl_sync(0xffffffffu, m0, o), om1 = __shfl_sync(0xffffffffu, m1, o);
    const double osA = __shfl_sync(0xffffffffu, sA, o), osB = __shfl_sync(0xffffffffu, sB, o);
    long long *d = dist_of(o);
    double ea = 0.0, eb = 0.0;
    if (live) {
      const int uu = i - pre[warp][o];
      ea = exp(((double)(d[uu] - ol0) - om0) * osA);
      eb = exp(((double)(d[S + uu] - ol1) - om1) * osB);
      d[uu] = __double_as_longlong(ea);
      d[S + uu] = __double_as_longlong(eb);
    }
    seg_add(ea, o, live, acc[warp][0]);
    seg_add(eb, o, live, acc[warp][1]);
  }
  __syncwarp();
  // pass 2: the normalised likelihoods and the two KL terms
  for (int i0 = 0; i0 < total; i0 += 32) {
    const int i = i0 + lane;
    const bool live = i < total;
    const int o = live ? owner(i) : 31;
    const int okeep = __shfl_sync(0xffffffffu, keep, o);
    const long long *d = dist_of(o);
    double t = 0.0;
    if (live) {
      const int uu = i - pre[warp][o];
      const double Pu = __longlong_as_double(d[uu]) / acc[warp][0][o];
      const double Qu = __longlong_as_double(d[S + uu]) / acc[warp][1][o];
      const double M = (Pu + Qu) / 2;
      if (M != 0) {
        if (Pu != 0) t += 0.5 * (Pu * log(Pu / M));
        if (Qu != 0) t += 0.5 * (Qu * log(Qu / M));
      }
      if (okeep >= 0) {
        bd.out_lval[((size_t)okeep * 2 + 0) * S + uu] = Pu;
        bd.out_lval[((size_t)okeep * 2 + 1) * S + uu] = Qu;
      }
    }
    seg_add(t, o, live, acc[warp][2]);
  }
  __syncwarp();
  if (U > 0) {
    double js = acc[warp][2][lane] / log(2.0);
    if (h0 == l0 || h1 == l1) js = __longlong_as_double(0x7ff8000000000000ll);
    bd.js[u] = js;
  }
}

// ------------------------------------------------------------ launchers
cudaError_t launch_prep(const int8_t *vals, int g, int n, int W, int c, uint64_t *planes,
                        uint64_t *valid, uint16_t *ctot, int8_t *valsT, cudaStream_t st) {
  int tot = g * W;
  k_planes<<<(tot + 127) / 128, 128, 0, st>>>(vals, g, n, W, planes, valid);
  k_transpose<<<(st_stride(g) * n + 255) / 256, 256, 0, st>>>(vals, g, n, valsT);
  if (c > 0) k_ctot<<<(c + 127) / 128, 128, 0, st>>>(planes, g, W, c, ctot);
  return cudaGetLastError();
}

cudaError_t launch_counter_masks(int n, int nA, int W, uint64_t seed, const int32_t *unit_set,
                                 const int32_t *unit_perm, const uint64_t *mask0, uint64_t *masks,
                                 int B, cudaStream_t st) {
  // keys [n] u32 (padded to 8 bytes), the W mask words, then [n] u16
  // sample indices; 128-thread blocks (more blocks per SM hide the barriers)
  const size_t smem = sizeof(uint32_t) * (size_t)((n + 1) & ~1) + sizeof(uint64_t) * W +
                      sizeof(uint16_t) * (size_t)n;
  if (smem > 48 * 1024) {
    cudaError_t e =
        cudaFuncSetAttribute(k_counter_masks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k_counter_masks<<<B, kCmBlock, smem, st>>>(n, nA, W, seed, unit_set, unit_perm, mask0, masks);
  return cudaGetLastError();
}

cudaError_t launch_pairs(const BatchSet *sets, const int32_t *uslot, const uint64_t *masks,
                         uint32_t *dmask, int B, int W, int cmax, unsigned long long *stats,
                         cudaStream_t st) {
  if (cmax <= 0) return cudaSuccess;
  dim3 grid((cmax + 127) / 128, B);
  k_pairs<<<grid, 128, sizeof(uint64_t) * W, st>>>(sets, uslot, masks, dmask, stats);
  return cudaGetLastError();
}

cudaError_t launch_units(const BatchDev &bd, int gmax, int W, cudaStream_t st, cudaEvent_t ev_mid,
                         bool ev_external) {
  const int threads = 256;
  size_t smem = unit_smem_bytes(gmax, W, (gmax + 31) / 32, threads / 32);
  cudaError_t e = cudaFuncSetAttribute(k_units, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_units<<<bd.B, threads, smem, st>>>(bd);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (ev_mid) {
    e = ev_external ? cudaEventRecordWithFlags(ev_mid, st, cudaEventRecordExternal)
                    : cudaEventRecord(ev_mid, st);
    if (e != cudaSuccess) return e;
  }
  // units per warp: as many as keep about eight warps per SM busy (the SM
  // count read once, thread-safely, from the current device)
  static const int sms = [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1)
      v = 148;
    return v;
  }();
  const int upw = std::max(1, std::min(32, bd.B / (sms * kJsWarps)));
  const int warps = (bd.B + upw - 1) / upw;
  k_js<<<(warps + kJsWarps - 1) / kJsWarps, 32 * kJsWarps, 0, st>>>(bd, upw);
  return cudaGetLastError();
}

cudaError_t set_divisor_map(const int8_t *map82) {
  return cudaMemcpyToSymbol(c_dmap, map82, 82);
}

}  // namespace eddy
