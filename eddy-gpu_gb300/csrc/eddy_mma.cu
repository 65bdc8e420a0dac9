// eddy_mma.cu -- contingency counts on the 5th-generation tensor cores.
//
// For a batch of units (labellings) of one gene set, the class-1 3x3 table
// of every pair is one GEMM over the samples:
//     D[u][p*9 + 3a + b] = sum_s  M[u][s] * Y[p*9 + 3a + b][s]
// M = class-1 sample mask of unit u, Y = indicator of (x_row(s) = a-1,
// x_col(s) = b-1) of pair p.  Both are 0/1 in e4m3 (kind::f8f6f4) with FP32
// accumulation in TMEM, exact for counts < 2^24.  This replaces the S x c x n
// tally loops of the reference's run2/run2Scalable (kernel1.cu:76-336);
// class 2 = full-sample table - class 1.  The epilogue reads the counts out
// of TMEM and settles, in the same kernel, every table whose ten
// leave-one-out variants provably hold no edge; the others are queued for
// k_general, which sets the bits of the 10-bit decision masks of both
// classes (kernel1.cu:121-203, 419-431) in a buffer that starts at zero.
//
// When every value of the set is -1/0/1 (kCore), a table's margins are the
// two genes' own class counts, which a small kernel counts per unit: the
// GEMM then holds only cells (-1,-1), (-1,0), (0,-1) and (0,0) of each table
// (8 pairs per 32-column group instead of 3) and the epilogue derives the
// other five by subtraction, exactly.
//
// Tile: 128 units (TMEM lanes) x kGroups column groups of 32 pair-cells
// (3 pairs x 9 cells + 5 pad columns, or 8 pairs x 4 cells; N = 128, 192 or
// 256) x K in
// 128-sample chunks; operands staged by TMA (cp.async.bulk.tensor, 128B
// swizzle) through an mbarrier ring.  Warp roles: 0 = TMA producer, 1 =
// TMEM owner + MMA issuer (it also stages each tile's full-sample tables
// into shared memory with cp.async.bulk), 2.. = epilogue warps (kEpi of
// them; each owns one TMEM lane quadrant and kGroups / (kEpi / 4) column
// groups, reads them with tcgen05.ld and decides their pairs from
// registers).  Accumulators are double-buffered.  Every mbarrier wait is
// bounded (2 s on %globaltimer); a timeout sets an error word, every role
// drains its own asynchronous work, and TMEM is released before the block
// exits.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include "eddy_device.cuh"
#include "eddy_kernels.h"
#include "eddy_mma.h"

namespace eddy {

namespace {
constexpr int kTM = 128, kPairsPerGroup = 3, kCorePairs = 8, kKC = 128;
// the pair groups of Y are padded to a multiple of every variant's groups
// per tile (4, 6, 8)
constexpr int kGroupPad = 24;
constexpr int kMaxGroups = 8;
constexpr unsigned long long kTimeoutNs = 2000000000ull;
// tables the quick filter cannot settle go into one queue per launch that
// k_general decides afterwards: a 4-word header (word 0 = tables, word 1 =
// decisions deferred to k_exact), 6-word items, then the list of deferred
// decisions; a full queue or list sets bit 2 of the error word and the batch
// is re-run elsewhere
constexpr int kQWords = 6;
// full-sample tables of one group: 3 pairs x 12 floats (nine counts, the
// prior flag, two pad), or in the 4-cell layout 8 pairs x 4 floats (the four
// counted cells) followed by the group's prior bits and three pad words
constexpr uint32_t kGroupCtBytes = kPairsPerGroup * 12 * sizeof(float);
static_assert(kGroupCtBytes == (kCorePairs * 4 + 4) * sizeof(float), "group table size");
constexpr uint32_t kBarBytes = 4096;  // barriers and table buffers after the stage ring
constexpr uint32_t kCtOff = 256;      // table buffers inside the barrier block

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{.reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p;}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false (and the error word set) after kTimeoutNs.
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, volatile unsigned *err) {
  if (mbar_try(a, parity)) return true;
  const unsigned long long t0 = gtimer();
  for (unsigned it = 1;; it++) {
    if (mbar_try(a, parity)) return true;
    // another role's timeout: checked every 256 tries (a global read)
    if ((it & 255u) == 0 && *err) return false;
    if (gtimer() - t0 > kTimeoutNs) {
      atomicExch((unsigned *)err, 1u);
      return false;
    }
  }
}
// Wait for this block's own asynchronous work before it exits: bounded by
// the same limit, regardless of the error word.
__device__ __forceinline__ void mbar_drain(uint32_t a, uint32_t parity) {
  const unsigned long long t0 = gtimer();
  while (!mbar_try(a, parity))
    if (gtimer() - t0 > kTimeoutNs) return;
}
// 1-D bulk copy global -> shared, completion counted on an mbarrier
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes,
                                          uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"((uint64_t)src), "r"(bytes), "r"(mbar)
      : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(mbar)
      : "memory");
}
// UMMA shared-memory descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;                    // LBO (unused with swizzle)
  d |= (uint64_t)(1024 >> 4) << 32;          // SBO
  d |= (uint64_t)1 << 46;                    // version
  d |= (uint64_t)2 << 61;                    // SWIZZLE_128B
  return d;
}
// Instruction descriptor: D f32, A/B e4m3, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_for(int n) {
  return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(kTM >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                     uint32_t acc) {
  asm volatile(
      "{.reg .pred p; setp.ne.b32 p, %4, 0;"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;}" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   mbar)
               : "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ------------------------------------------------------ the 4-cell layout
// One gene of a pair: its counts {class 1, class 2} of the states -1, 0
// and 1, the products of the other two states' counts, the product of all
// three (the factors quick_zero_f2 forms from a table's margins) and the
// smallest count minus one.  w = class-1 counts of states -1 and 0 (16 bits
// each), F = the full-sample counts, N = the class sizes; a gene of this
// layout has no missing value, so its class-2 counts and its state-1 count
// follow by subtraction.  Every value is an exact integer in FP32, equal to
// the margin quick_zero_f2 sums from the nine cells.
struct CoreGene {
  f32x2 M0, M1, M2, P0, P1, P2, Dg, m1;
  float mx, my;
};
__device__ __forceinline__ void core_gene(CoreGene &G, uint32_t w, float4 F, f32x2 N) {
  // 2^23 + c as a float, minus 2^23: the 16-bit count c, exactly
  const float c0 = __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7610)) - 8388608.f;
  const float c1 = __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7632)) - 8388608.f;
  G.M0 = f2_pack(c0, F.x - c0);
  G.M1 = f2_pack(c1, F.y - c1);
  G.M2 = f2_sub(f2_sub(N, G.M0), G.M1);
  G.P0 = f2_mul(G.M1, G.M2);
  G.P1 = f2_mul(G.M0, G.M2);
  G.P2 = f2_mul(G.M0, G.M1);
  G.Dg = f2_mul(G.M0, G.P0);
  G.mx = fminf(f2_x(G.M0), fminf(f2_x(G.M1), f2_x(G.M2)));
  G.my = fminf(f2_y(G.M0), fminf(f2_y(G.M1), f2_y(G.M2)));
  G.m1 = f2_sub(f2_pack(G.mx, G.my), f2_pack(1.f, 1.f));
}
// Terms of the bound that depend on a unit's class sizes N only.
struct CoreN {
  f32x2 N;
  float n5m_x, n5m_y, n5_x, n5_y;
  bool okx, oky;
};
__device__ __forceinline__ void core_n(f32x2 N, CoreN &K) {
  const float Nx = f2_x(N), Ny = f2_y(N);
  K.N = N;
  K.okx = Nx >= 32.f && Nx <= 4096.f;
  K.oky = Ny >= 32.f && Ny <= 4096.f;
  K.n5m_x = 5.f * (Nx - 1.f);
  K.n5m_y = 5.f * (Ny - 1.f);
  K.n5_x = 5.f * Nx;
  K.n5_y = 5.f * Ny;
}
// The nine cells {class 1, class 2} of a table, o[3a + b] for states a - 1
// (row gene) and b - 1 (column gene), from its four counted class-1 cells
// a[0..3] (TMEM columns), their full-sample counts F and the genes' counts.
__device__ __forceinline__ void core_cells(const uint32_t *a, float4 F, const CoreGene &R,
                                           const CoreGene &C, f32x2 *o) {
  const float a0 = __uint_as_float(a[0]), a1 = __uint_as_float(a[1]);
  const float a3 = __uint_as_float(a[2]), a4 = __uint_as_float(a[3]);
  o[0] = f2_pack(a0, F.x - a0);
  o[1] = f2_pack(a1, F.y - a1);
  o[3] = f2_pack(a3, F.z - a3);
  o[4] = f2_pack(a4, F.w - a4);
  o[2] = f2_sub(f2_sub(R.M0, o[0]), o[1]);
  o[5] = f2_sub(f2_sub(R.M1, o[3]), o[4]);
  o[6] = f2_sub(f2_sub(C.M0, o[0]), o[3]);
  o[7] = f2_sub(f2_sub(C.M1, o[1]), o[4]);
  o[8] = f2_sub(f2_sub(R.M2, o[6]), o[7]);
}
// quick_zero_f2 on a table of the 4-cell layout: the same operations on the
// same values (margins, their products and minima from the genes' terms),
// so the same outcome, bit for bit.
__device__ __forceinline__ unsigned core_zero_f2(const f32x2 *o, const CoreGene &R,
                                                 const CoreGene &C, const CoreN &K, float chiA) {
  const f32x2 N = K.N;
  const f32x2 rm = f2_pack(R.mx, R.my), cm = f2_pack(C.mx, C.my);
  const f32x2 q = f2_mul(R.m1, C.m1), rc = f2_mul(rm, cm);
  const bool okx = K.okx && R.mx >= 2.f && C.mx >= 2.f && f2_x(q) >= K.n5m_x && f2_x(rc) >= K.n5_x;
  const bool oky = K.oky && R.my >= 2.f && C.my >= 2.f && f2_y(q) >= K.n5m_y && f2_y(rc) >= K.n5_y;
  const f32x2 D = f2_mul(R.Dg, C.Dg);
  const f32x2 s0 = f2_fma(f2_mul(o[0], o[0]), C.P0,
                          f2_fma(f2_mul(o[1], o[1]), C.P1, f2_mul(f2_mul(o[2], o[2]), C.P2)));
  const f32x2 s1 = f2_fma(f2_mul(o[3], o[3]), C.P0,
                          f2_fma(f2_mul(o[4], o[4]), C.P1, f2_mul(f2_mul(o[5], o[5]), C.P2)));
  const f32x2 s2 = f2_fma(f2_mul(o[6], o[6]), C.P0,
                          f2_fma(f2_mul(o[7], o[7]), C.P1, f2_mul(f2_mul(o[8], o[8]), C.P2)));
  const f32x2 QD = f2_fma(R.P0, s0, f2_fma(R.P1, s1, f2_mul(R.P2, s2)));
  const f32x2 rcN = f2_mul(rc, N);
  // (rm - 1) + cm = (rm + cm) - 1: exact integers
  const f32x2 t1 = f2_fma(N, f2_add(R.m1, cm), f2_mul(rcN, f2_pack(1e-5f, 1e-5f)));
  const f32x2 lhs = f2_fma(t1, D, f2_mul(rcN, f2_sub(QD, D)));
  const f32x2 qD = f2_mul(q, D);
  const f32x2 L = f2_fma(lhs, f2_pack(1.0001f, 1.0001f), f2_mul(f2_pack(1e-3f, 1e-3f), qD));
  const f32x2 Rr = f2_mul(f2_pack(chiA, chiA), qD);
  return ((okx && f2_x(L) < f2_x(Rr)) ? 1u : 0u) | ((oky && f2_y(L) < f2_y(Rr)) ? 2u : 0u);
}
// The class-1 table of pair q of a group as integers, for the queue: the
// four counted cells from TMEM and the five derived from the row gene's and
// the column gene's class-1 counts wr, wc and the class-1 size n1.
__device__ __forceinline__ void core_table(const uint32_t *r, int q, uint32_t wr, uint32_t wc,
                                           int n1, int *t) {
  t[0] = (int)__uint_as_float(r[4 * q]);
  t[1] = (int)__uint_as_float(r[4 * q + 1]);
  t[3] = (int)__uint_as_float(r[4 * q + 2]);
  t[4] = (int)__uint_as_float(r[4 * q + 3]);
  const int r0 = (int)(wr & 0xFFFFu), r1 = (int)(wr >> 16);
  const int c0 = (int)(wc & 0xFFFFu), c1 = (int)(wc >> 16);
  t[2] = r0 - t[0] - t[1];
  t[5] = r1 - t[3] - t[4];
  t[6] = c0 - t[0] - t[3];
  t[7] = c1 - t[1] - t[4];
  t[8] = (n1 - r0 - r1) - t[6] - t[7];
}

}  // namespace

// Tile t of a batch's launch: its set k (sets ordered by tile0), column
// tile tn and 128-unit row block mb within the set.
struct TileAt {
  int k, tn, mb;
};
__device__ __forceinline__ TileAt tile_at(const BatchSet *sets, int nsets, int t) {
  int lo = 0, hi = nsets - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (sets[mid].tile0 <= t) lo = mid;
    else hi = mid - 1;
  }
  const int l = t - sets[lo].tile0, mbk = sets[lo].mblocks;
  return {lo, l / mbk, l % mbk};
}

template <int kStages>
struct MmaSmem {
  unsigned long long full[kStages], empty[kStages], accfull[2], accempty[2], ctfull[2], drain;
  uint32_t tmem_base;
};
static_assert(sizeof(MmaSmem<8>) <= kCtOff &&
                  kCtOff + 2 * kMaxGroups * kGroupCtBytes <= kBarBytes,
              "barrier block");

// registers per thread for one CTA of 2 + kEpi warps: each of the four SM
// sub-partitions holds 16384 registers and ceil((2 + kEpi) / 4) of the warps
template <int kEpi>
constexpr int max_regs() {
  return (16384 / (32 * ((2 + kEpi + 3) / 4))) / 8 * 8 > 255
             ? 255
             : (16384 / (32 * ((2 + kEpi + 3) / 4))) / 8 * 8;
}

// kStages: depth of the TMA ring; kEpi: epilogue warps (a multiple of 4);
// kGroups: 32-column pair groups per tile (N = 32 kGroups).  One CTA per SM.
// All variants produce identical masks; the autotuner picks by time.
template <int kStages, int kEpi, int kGroups, bool kCore>
__global__ void __maxnreg__(max_regs<kEpi>())
    k_pairs_mma(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                const BatchSet *__restrict__ sets, int nsets, const float *__restrict__ ctotf,
                int nk, int ntot, unsigned long long *stats, unsigned *err, unsigned *gqueue,
                unsigned qcap, const uint32_t *__restrict__ margc,
                const float4 *__restrict__ gcnt, const uint32_t *__restrict__ gtab) {
  constexpr int kTN = 32 * kGroups;
  constexpr int kPPG = kCore ? kCorePairs : kPairsPerGroup;  // pairs per column group
  constexpr int kPairsPerTile = kGroups * kPPG;
  constexpr uint32_t kStageBytes = (kTM + kTN) * kKC;
  constexpr uint32_t kCtBytes = kGroups * kGroupCtBytes;
  constexpr uint32_t kTmemCols = 2 * kTN <= 256 ? 256u : 512u;
  constexpr uint32_t kIdesc = idesc_for(kTN);
  constexpr int kPerQuad = kEpi / 4, kGpw = kGroups / kPerQuad;
  static_assert(kEpi % 4 == 0 && kGroups % kPerQuad == 0 && kGroups <= kMaxGroups, "shape");
  extern __shared__ __align__(1024) uint8_t smraw[];
  // 1024-byte aligned stage ring, then barriers, then the epilogue buffer
  uint8_t *base = (uint8_t *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  MmaSmem<kStages> &S = *reinterpret_cast<MmaSmem<kStages> *>(base + kStages * kStageBytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile unsigned *verr = err;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; s++) {
      mbar_init(smem_u32(&S.full[s]), 1);
      mbar_init(smem_u32(&S.empty[s]), 1);
    }
    for (int a = 0; a < 2; a++) {
      mbar_init(smem_u32(&S.accfull[a]), 1);
      mbar_init(smem_u32(&S.accempty[a]), 32 * kEpi);
      mbar_init(smem_u32(&S.ctfull[a]), 1);
    }
    mbar_init(smem_u32(&S.drain), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    // two kTN-column fp32 accumulators
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&S.tmem_base)),
                 "n"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  // 4-cell layout: a batch of one set has its genes' full-sample counts in
  // shared memory, after the barrier block (others read them from global
  // memory, at the set's offset)
  float4 *sgcnt = reinterpret_cast<float4 *>(base + kStages * kStageBytes + kBarBytes);
  if constexpr (kCore)
    if (nsets == 1)
      for (int i = threadIdx.x; i < sets[0].sd.g; i += blockDim.x) sgcnt[i] = gcnt[i];
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem_base;

  if (warp == 0) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      long long nfill = 0;
      bool live = true;  // false after a wait gave up (the error word is set)
      for (int t = blockIdx.x; t < ntot && live; t += gridDim.x) {
        const TileAt ta = tile_at(sets, nsets, t);
        const int arow = (sets[ta.k].mb0 + ta.mb) * kTM;
        const int brow = (sets[ta.k].grp0 + ta.tn * kGroups) * 32;
        for (int kc = 0; kc < nk; kc++) {
          if (!mbar_wait(smem_u32(&S.empty[stage]), phase ^ 1u, verr)) {
            live = false;
            break;
          }
          const uint32_t fb = smem_u32(&S.full[stage]);
          mbar_expect_tx(fb, kStageBytes);
          const uint32_t sa = smem_u32(base + stage * kStageBytes);
          tma_load_2d(sa, &tmA, kc * kKC, arow, fb);
          tma_load_2d(sa + kTM * kKC, &tmB, kc * kKC, brow, fb);
          nfill++;
          if (++stage == kStages) {
            stage = 0;
            phase ^= 1u;
          }
        }
      }
      // the last fills have landed before the block may exit
      for (long long i = nfill > kStages ? nfill - kStages : 0; i < nfill; i++)
        mbar_drain(smem_u32(&S.full[i % kStages]), (uint32_t)((i / kStages) & 1));
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int stage = 0, acc = 0;
      uint32_t phase = 0, accphase = 0;
      long long nct = 0;
      for (int t = blockIdx.x; t < ntot; t += gridDim.x) {
        if (!mbar_wait(smem_u32(&S.accempty[acc]), accphase ^ 1u, verr)) break;
        tc_fence_after();
        {
          // the tile's full-sample tables into the slot's buffer
          const TileAt ta = tile_at(sets, nsets, t);
          const int grp = sets[ta.k].grp0 + ta.tn * kGroups;
          const uint32_t cb = smem_u32(&S.ctfull[acc]);
          mbar_expect_tx(cb, kCtBytes);
          bulk_load(smem_u32(base + kStages * kStageBytes + kCtOff + acc * kCtBytes),
                    ctotf + (size_t)grp * (kGroupCtBytes / 4), kCtBytes, cb);
          nct++;
        }
        const uint32_t dcol = tmem + (uint32_t)(acc * kTN);
        bool ok = true;
        for (int kc = 0; kc < nk; kc++) {
          if (!mbar_wait(smem_u32(&S.full[stage]), phase, verr)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t sa = smem_u32(base + stage * kStageBytes);
          const uint32_t sb = sa + kTM * kKC;
#pragma unroll
          for (int k = 0; k < kKC / 32; k++)
            umma(dcol, sdesc(sa + 32 * k), sdesc(sb + 32 * k), kIdesc, (kc | k) ? 1u : 0u);
          umma_commit(smem_u32(&S.empty[stage]));
          if (++stage == kStages) {
            stage = 0;
            phase ^= 1u;
          }
        }
        if (!ok) break;
        umma_commit(smem_u32(&S.accfull[acc]));
        if (++acc == 2) {
          acc = 0;
          accphase ^= 1u;
        }
      }
      // every MMA issued here and the last table copies complete before exit
      umma_commit(smem_u32(&S.drain));
      mbar_drain(smem_u32(&S.drain), 0);
      for (long long i = nct > 2 ? nct - 2 : 0; i < nct; i++)
        mbar_drain(smem_u32(&S.ctfull[i & 1]), (uint32_t)((i >> 1) & 1));
    }
  } else {
    // epilogue: TMEM lane quadrant = warp % 4; the kEpi/4 warps of a quadrant
    // split the column groups (kGpw each)
    const int quad = warp & 3, wq = (warp - 2) >> 2;
    const int row = quad * 32 + lane;  // TMEM lane = unit within the tile
    int acc = 0;
    uint32_t accphase = 0;
    unsigned nexact = 0, nfilt = 0, ntab = 0;
    // the counters go to their set's row of stats ([nsets][4]): added when
    // the warp moves to a tile of another set, and at the end
    int stat_k = -1;
    auto flush_stats = [&](int k) {
      if (!stats || k < 0) return;
      for (int o = 16; o > 0; o >>= 1) {
        nexact += __shfl_down_sync(0xffffffffu, nexact, o);
        nfilt += __shfl_down_sync(0xffffffffu, nfilt, o);
        ntab += __shfl_down_sync(0xffffffffu, ntab, o);
      }
      if (lane == 0) {
        unsigned long long *sk = stats + 4 * (size_t)k;
        if (nexact) atomicAdd(&sk[0], (unsigned long long)nexact);
        if (ntab) atomicAdd(&sk[1], (unsigned long long)ntab);
        if (nfilt) atomicAdd(&sk[2], (unsigned long long)nfilt);
      }
      nexact = nfilt = ntab = 0;
    };
    unsigned *qitems = gqueue + 4;
    // 4-cell layout: the class-1 count words of a group for this thread's
    // unit (w[q] = column gene of pair q, w[8] = the row gene) and the
    // unit's class-1 size, fetched one group ahead so that their L2 latency
    // passes while the previous group is decided (the next group may be in
    // the next tile, of another set: class counts [g][Bp] at the set's mg0,
    // then its class-1 sizes)
    uint32_t wcur[kCorePairs + 1], wnext[kCorePairs + 1];
    float n1next = 0.f;
    auto fetch = [&](int t2, int gi2) {
      if constexpr (kCore) {
        if (t2 >= ntot) return;
        const TileAt ta = tile_at(sets, nsets, t2);
        const BatchSet &b2 = sets[ta.k];
        const int u2 = ta.mb * kTM + row, Bp2 = b2.mblocks * kTM;
        const uint32_t *mc = margc + b2.mg0;
        const uint32_t e = gtab[b2.grp0 + ta.tn * kGroups + wq + gi2 * kPerQuad];
        const int r2 = (int)(e >> 16), c2 = (int)(e & 0xFFFFu);
        if (r2 != 0xFFFF) {
          wnext[kCorePairs] = mc[(size_t)r2 * Bp2 + u2];
#pragma unroll
          for (int q = 0; q < kCorePairs; q++)
            wnext[q] = mc[(size_t)(c2 + q < r2 ? c2 + q : r2 - 1) * Bp2 + u2];
        }
        if (gi2 == 0)
          n1next = reinterpret_cast<const float *>(mc + (size_t)b2.sd.g * Bp2)[u2];
      }
    };
    // with 16 epilogue warps the warps themselves hide the latency and the
    // registers of a second word set would spill: words are loaded when used
    constexpr bool kAhead = kEpi <= 12;
    if (kAhead) fetch(blockIdx.x, 0);
    for (int t = blockIdx.x; t < ntot; t += gridDim.x) {
      const TileAt ta = tile_at(sets, nsets, t);
      const int tn = ta.tn, mb = ta.mb;
      const BatchSet &bs = sets[ta.k];
      if (ta.k != stat_k) {
        flush_stats(stat_k);
        stat_k = ta.k;
      }
      const SetDev &sd = bs.sd;
      if (!mbar_wait(smem_u32(&S.accfull[acc]), accphase, verr)) break;
      if (!mbar_wait(smem_u32(&S.ctfull[acc]), accphase, verr)) break;
      tc_fence_after();
      const float *ctile =
          reinterpret_cast<const float *>(base + kStages * kStageBytes + kCtOff + acc * kCtBytes);
      // the unit: TMEM lane row of the set's row block mb (past nb: padding)
      const int ul = mb * kTM + row;
      const bool ulive = ul < bs.nb;
      const int u = bs.u0 + ul;
      // no-edge thresholds of dof 4 without / with a prior (quick_zero_f2)
      const float thr0 = sd.exact_all ? -1.f : sd.thr[0][2].chiA;
      const float thr1 = sd.exact_all ? -1.f : sd.thr[1][2].chiA;
      const int cset = sd.c;
      const int grp_base = bs.grp0 + tn * kGroups;
      // 4-cell layout: the unit's class sizes {class 1, class 2} and the
      // set's genes' full-sample counts
      f32x2 N = f2_pack(0.f, 0.f);
      CoreN NC{};
      const float4 *gc4 = nsets == 1 ? sgcnt : gcnt + bs.gc0;
      if constexpr (kCore) {
        const float n1 = kAhead ? n1next
                                : reinterpret_cast<const float *>(
                                      margc + bs.mg0 + (size_t)sd.g * bs.mblocks * kTM)[ul];
        N = f2_pack(n1, (float)sd.n - n1);
        core_n(N, NC);
      }
      // the warp's column groups, one at a time out of TMEM; pairs past c
      // (the last tile's tail) are padding
#pragma unroll 1
      for (int gi = 0; gi < kGpw; gi++) {
        const int grp = wq + gi * kPerQuad;
        // the group's 32 TMEM columns (the 4-cell layout reads them in two
        // halves in pass 1, and again in full for pass 2)
        const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(acc * kTN + grp * 32);
        uint32_t r[32];
        if constexpr (!kCore) {
          tmem_ld32(taddr, r);
          tmem_ld_wait();
        }
        // pass 1: the all-zero bound of the group's tables, both classes of
        // a pair in the two lanes of packed FP32 pairs; bit 2 q + class of
        // qmask = the table goes to the general path
        uint32_t qmask = 0u, vmask = 0u;
        const float *gct = ctile + grp * (int)(kGroupCtBytes / 4);
        const int p0 = tn * kPairsPerTile + grp * kPPG;
        // 4-cell layout: the group's row gene and first column gene
        int crow = 0, ccol0 = 0;
        if constexpr (kCore) {
          const uint32_t e = gtab[grp_base + grp];
          crow = (int)(e >> 16);
          ccol0 = (int)(e & 0xFFFFu);
          if (!kAhead) fetch(t, gi);
#pragma unroll
          for (int k = 0; k <= kCorePairs; k++) wcur[k] = wnext[k];
          if (kAhead) {
            if (gi + 1 < kGpw) fetch(t, gi + 1);
            else fetch(t + gridDim.x, 0);
          }
        }
        if constexpr (kCore) {
          // pair q = columns 4q .. 4q+3 (cells (-1,-1), (-1,0), (0,-1),
          // (0,0)) = genes (crow, ccol0 + q), live while ccol0 + q < crow;
          // straight-line code over the eight pairs (a padding group has
          // crow = 0xFFFF)
          const uint32_t pbits = __float_as_uint(gct[32]);
          if (crow != 0xFFFF) {
            CoreGene Rg;
            core_gene(Rg, wcur[kCorePairs], gc4[crow], N);
#pragma unroll
            for (int h = 0; h < 2; h++) {
              uint32_t rh[16];
              tmem_ld16(taddr + 16 * h, rh);
              tmem_ld_wait();
#pragma unroll
              for (int qq = 0; qq < kPPG / 2; qq++) {
                const int q = h * (kPPG / 2) + qq;
                const bool live = ccol0 + q < crow;
                const int col = live ? ccol0 + q : crow - 1;
                CoreGene Cg;
                core_gene(Cg, wcur[q], gc4[col], N);
                const float4 F = reinterpret_cast<const float4 *>(gct)[q];
                f32x2 o[9];
                core_cells(rh + 4 * qq, F, Rg, Cg, o);
                const float chiA = ((pbits >> q) & 1u) ? thr1 : thr0;
                const unsigned settled = core_zero_f2(o, Rg, Cg, NC, chiA);
                qmask |= (live ? (~settled & 3u) : 0u) << (2 * q);
                vmask |= (live ? 3u : 0u) << (2 * q);
              }
            }
          }
        } else {
          // pair q = columns 9q .. 9q+8
#pragma unroll
          for (int q = 0; q < kPPG; q++) {
            const float *f = gct + q * 12;
            f32x2 o2[9];
#pragma unroll
            for (int k = 0; k < 9; k++) {
              const float a = __uint_as_float(r[9 * q + k]);
              o2[k] = f2_pack(a, f[k] - a);
            }
            const float chiA = (f[9] != 0.f) ? thr1 : thr0;
            qmask |= (~quick_zero_f2(o2, chiA) & 3u) << (2 * q);
            vmask |= (p0 + q < cset ? 3u : 0u) << (2 * q);
          }
        }
        if (!ulive) vmask = 0u;
        qmask &= vmask;
        ntab += (unsigned)__popc(vmask);
        nfilt += (unsigned)__popc(vmask & ~qmask);
        // pass 2 (rare): the flagged tables into the launch's queue, one
        // atomic per warp: counts, class, prior, pair and unit
        if (__any_sync(0xffffffffu, qmask != 0u)) {
          const unsigned cnt = (unsigned)__popc(qmask);
          unsigned incl = cnt;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
          }
          unsigned qbase = 0;
          if (lane == 31) qbase = atomicAdd(gqueue, incl);
          unsigned idx = __shfl_sync(0xffffffffu, qbase, 31) + incl - cnt;
          if constexpr (kCore) {
            tmem_ld32(taddr, r);
            tmem_ld_wait();
          }
#pragma unroll
          for (int q = 0; q < kPPG; q++) {
            if (((qmask >> (2 * q)) & 3u) == 0u) continue;
            // pair index (row-major over the lower triangle)
            const int p = kCore ? crow * (crow - 1) / 2 + ccol0 + q : p0 + q;
            // the class-1 table and the full-sample table, as integers
            int t1[9], tf[9], prior;
            if constexpr (kCore) {
              prior = (int)((__float_as_uint(gct[32]) >> q) & 1u);
              core_table(r, q, wcur[kCorePairs], wcur[q], (int)f2_x(N), t1);
#pragma unroll
              for (int k = 0; k < 9; k++) tf[k] = (int)sd.ctot[(size_t)p * 9 + k];
            } else {
              const float *f = gct + q * 12;
              prior = (f[9] != 0.f) ? 1 : 0;
#pragma unroll
              for (int k = 0; k < 9; k++) {
                t1[k] = (int)__uint_as_float(r[9 * q + k]);
                tf[k] = (int)f[k];
              }
            }
#pragma unroll
            for (int cls = 0; cls < 2; cls++) {
              if (!((qmask >> (2 * q + cls)) & 1u)) continue;
              uint32_t o[9];
#pragma unroll
              for (int k = 0; k < 9; k++) o[k] = (uint32_t)(cls ? tf[k] - t1[k] : t1[k]);
              if (idx < qcap) {
                unsigned *it = qitems + (size_t)idx * kQWords;
                it[0] = o[0] | (o[1] << 16);
                it[1] = o[2] | (o[3] << 16);
                it[2] = o[4] | (o[5] << 16);
                it[3] = o[6] | (o[7] << 16);
                it[4] = o[8] | ((uint32_t)cls << 16) | ((uint32_t)prior << 17);
                it[5] = (uint32_t)p | ((uint32_t)u << 17);  // pair < 2^17, batch unit < 2^15
              } else {
                atomicOr(err, 2u);
              }
              idx++;
            }
          }
        }
      }
      // the slot (accumulator and table buffer) is free again
      tc_fence_before();
      mbar_arrive(smem_u32(&S.accempty[acc]));
      if (++acc == 2) {
        acc = 0;
        accphase ^= 1u;
      }
    }
    flush_stats(stat_k);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "n"(kTmemCols));
  }
}

// Decision `slot` of queued table `it`: 0 = the full table, 1 + 3a + b =
// the table with one sample of cell (a, b) removed.  The full table is
// decided in FP32, and when the Minkowski leave-one-out window settles the
// cells (or the cell is empty) the slot shares its decision; otherwise the
// slot decides its own cell-removed table.  A decision in a guard band needs
// the exact FP64 path: with allow_exact it is taken, else 2 is returned.
__device__ __forceinline__ int general_task(const unsigned *it, int slot, const SetDev &sd,
                                            bool allow_exact, unsigned &nexact,
                                            unsigned &nfilt) {
  const int prior = (it[4] >> 17) & 1;
  int t[9] = {(int)(it[0] & 0xFFFFu), (int)(it[0] >> 16), (int)(it[1] & 0xFFFFu),
              (int)(it[1] >> 16),     (int)(it[2] & 0xFFFFu), (int)(it[2] >> 16),
              (int)(it[3] & 0xFFFFu), (int)(it[3] >> 16),     (int)(it[4] & 0xFFFFu)};
  TabInfo ti;
  table_info(t, ti);
  const bool safe = loo_safe(ti, prior, sd);
  if (slot == 0 && safe) nfilt++;
  const int cell = slot - 1;
  if (slot == 0 || safe || t[cell] == 0) {
    int bit0 = fast_decision(ti, prior, sd);
    if (bit0 == 2) {
      if (!allow_exact) return 2;
      nexact++;
      bit0 = exact_decision(t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8], prior, sd);
    }
    return bit0;
  }
  t[cell]--;
  TabInfo tj;
  table_info(t, tj);
  int bit = fast_decision(tj, prior, sd);
  if (bit == 2) {
    if (!allow_exact) return 2;
    nexact++;
    bit = exact_decision(t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8], prior, sd);
  }
  return bit;
}

__device__ __forceinline__ void set_decision(uint32_t *dmask, const BatchSet &bs,
                                             const unsigned *it, int slot) {
  const int cls = (it[4] >> 16) & 1;
  const int p = (int)(it[5] & 0x1FFFFu), u = (int)(it[5] >> 17);
  atomicOr(&unit_dmask(dmask, bs, u)[p], 1u << (slot + 16 * cls));
  mark_chunk(unit_chunks(dmask, bs, u), p);
}

// A thread's counters of the general and exact paths, per set: added to
// the set's row of stats ([nsets][4]) when the thread's next table belongs
// to another set, and at the end.
struct SetStats {
  unsigned long long *stats;
  int k = -1;
  unsigned nexact = 0, nfilt = 0;
  __device__ explicit SetStats(unsigned long long *s) : stats(s) {}
  __device__ void flush() {
    if (stats && k >= 0) {
      if (nexact) atomicAdd(&stats[4 * (size_t)k], (unsigned long long)nexact);
      if (nfilt) atomicAdd(&stats[4 * (size_t)k + 2], (unsigned long long)nfilt);
    }
    nexact = nfilt = 0;
  }
  __device__ void to(int k2) {
    if (k2 != k) {
      flush();
      k = k2;
    }
  }
};

// The general path for the queued tables of a launch, one thread per
// table: the full table's FP32 decision and its Minkowski leave-one-out
// window once, then, when the window cannot settle them, the nine
// cell-removed tables (an empty cell shares the full table's decision).  A
// table's bits go into its mask with one atomic.  Decisions in a guard band
// are listed (queue word 1 counts them) for k_exact: on this part a
// dependent FP64 operation costs ~128 cycles and an SM issues one FP64 warp
// instruction per ~32 cycles, so rechecks spread one per warp over the grid
// would share the SMs' FP64 units, while k_exact runs them 32 to a warp.
__global__ void __launch_bounds__(256) k_general(const BatchSet *__restrict__ sets,
                                                 const int32_t *__restrict__ uslot,
                                                 unsigned *queue, unsigned qcap,
                                                 uint32_t *dmask, unsigned long long *stats,
                                                 unsigned *err) {
  const unsigned cnt = queue[0] < qcap ? queue[0] : qcap;
  const unsigned *items = queue + 4;
  unsigned *elist = queue + 4 + (size_t)qcap * kQWords;
  SetStats ss(stats);
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    const unsigned *it = items + (size_t)i * kQWords;
    const int k = uslot[it[5] >> 17];
    const BatchSet &bs = sets[k];
    const SetDev &sd = bs.sd;
    ss.to(k);
    const int prior = (it[4] >> 17) & 1;
    int t[9] = {(int)(it[0] & 0xFFFFu), (int)(it[0] >> 16), (int)(it[1] & 0xFFFFu),
                (int)(it[1] >> 16),     (int)(it[2] & 0xFFFFu), (int)(it[2] >> 16),
                (int)(it[3] & 0xFFFFu), (int)(it[3] >> 16),     (int)(it[4] & 0xFFFFu)};
    TabInfo ti;
    table_info(t, ti);
    const bool safe = loo_safe(ti, prior, sd);
    if (safe) ss.nfilt++;
    const int bit0 = fast_decision(ti, prior, sd);
    uint32_t bits = 0u;
    auto put = [&](int slot, int bit) {
      if (bit == 2) {
        const unsigned k = atomicAdd(&queue[1], 1u);
        if (k < qcap) elist[k] = i * 10u + (unsigned)slot;
        else atomicOr(err, 2u);
      } else {
        bits |= (uint32_t)bit << slot;
      }
    };
    put(0, bit0);
#pragma unroll
    for (int cell = 0; cell < 9; cell++) {
      if (safe || t[cell] == 0) {
        put(1 + cell, bit0);
      } else {
        t[cell]--;
        TabInfo tj;
        table_info(t, tj);
        put(1 + cell, fast_decision(tj, prior, sd));
        t[cell]++;
      }
    }
    if (bits) {
      const int cls = (it[4] >> 16) & 1;
      const int p = (int)(it[5] & 0x1FFFFu), u = (int)(it[5] >> 17);
      atomicOr(&unit_dmask(dmask, bs, u)[p], bits << (16 * cls));
      mark_chunk(unit_chunks(dmask, bs, u), p);
    }
  }
  ss.flush();
}

// The listed decisions of k_general through the exact FP64 path, one lane
// each, one warp per block.
__global__ void __launch_bounds__(32) k_exact(const BatchSet *__restrict__ sets,
                                              const int32_t *__restrict__ uslot,
                                              const unsigned *queue, unsigned qcap,
                                              uint32_t *dmask, unsigned long long *stats) {
  const unsigned n = queue[1] < qcap ? queue[1] : qcap;
  const unsigned *items = queue + 4;
  const unsigned *elist = queue + 4 + (size_t)qcap * kQWords;
  SetStats ss(stats);
  for (unsigned k = blockIdx.x * 32u + threadIdx.x; k < n; k += gridDim.x * 32u) {
    const unsigned task = elist[k];
    const unsigned *it = items + (size_t)(task / 10) * kQWords;
    const int slot = (int)(task % 10);
    unsigned nf = 0;
    const int ks = uslot[it[5] >> 17];
    const BatchSet &bs = sets[ks];
    ss.to(ks);
    if (general_task(it, slot, bs.sd, true, ss.nexact, nf)) set_decision(dmask, bs, it, slot);
  }
  ss.flush();
}

// -------------------------------------------------------------- operands
// 16 samples of an indicator row as e4m3 0/1 (1.0 = 0x38)
__device__ __forceinline__ void store_e4m3_16(uint8_t *dst, uint32_t bits) {
  uint8_t v[16];
#pragma unroll
  for (int k = 0; k < 16; k++) v[k] = ((bits >> k) & 1u) ? 0x38 : 0x00;
  uint4 o;
  memcpy(&o, v, 16);
  *reinterpret_cast<uint4 *>(dst) = o;
}
// samples [16 ch, 16 ch + 16) of plane(row, a) & plane(col, b)
__device__ __forceinline__ uint32_t pair_bits16(const uint64_t *planes, int W, int row, int a,
                                                int col, int b, int ch) {
  const int s0 = ch * 16, w = s0 >> 6, sh = s0 & 63;
  if (w >= W) return 0u;
  const uint64_t x = planes[((size_t)row * 3 + a) * W + w] & planes[((size_t)col * 3 + b) * W + w];
  return (uint32_t)(x >> sh) & 0xFFFFu;
}

// 9-cell Y: row (group*32 + q*9 + 3a + b), q < 3 = indicator over the
// samples of pair group*3 + q having (x_row = a-1, x_col = b-1); rows 27..31
// of each group and out-of-range pairs are zero.  A tile of any variant is
// a run of whole groups.  Work item = one 16-sample chunk of one row.
__device__ __forceinline__ void build_y_chunk(const uint64_t *planes, int W, int c, int n_pad,
                                              long long idx, uint8_t *Y) {
  const int chunks = n_pad / 16;
  const int rr = (int)(idx / chunks), ch = (int)(idx % chunks);
  const int grp = rr / 32, r32 = rr % 32;
  const int q = r32 / 9, cell = r32 % 9;
  const int p = grp * kPairsPerGroup + q;
  uint32_t bits = 0;
  if (r32 < kPairsPerGroup * 9 && p < c) {
    int row, col;
    pair_rc(p, row, col);
    bits = pair_bits16(planes, W, row, cell / 3, col, cell % 3, ch);
  }
  store_e4m3_16(Y + (size_t)rr * n_pad + ch * 16, bits);
}

// 9-cell full-sample tables as FP32 for the epilogue: pair p -> 12 floats
// (nine counts, the prior flag, two pad), 48 bytes, float4-aligned; pairs
// past c up to whole groups are zero.
__device__ __forceinline__ void ctot_f_pair(const uint16_t *ctot, const uint8_t *prior, int c,
                                            int p, float *out) {
  float v[12];
#pragma unroll
  for (int k = 0; k < 9; k++) v[k] = p < c ? (float)ctot[(size_t)p * 9 + k] : 0.f;
  v[9] = (p < c && prior[p]) ? 1.f : 0.f;
  v[10] = v[11] = 0.f;
  float4 *o = reinterpret_cast<float4 *>(out + (size_t)p * 12);
  o[0] = make_float4(v[0], v[1], v[2], v[3]);
  o[1] = make_float4(v[4], v[5], v[6], v[7]);
  o[2] = make_float4(v[8], v[9], v[10], v[11]);
}

// The 4-cell layout's column groups are row-aligned: group k holds the
// pairs (row, col0 + q), q < 8, of entry k = row << 16 | col0; row r owns
// ceil(r / 8) groups, rows 1 .. g-1 in order, and pairs with col0 + q >= row
// are padding (as are whole groups past the last row: row 0xFFFF).  Groups
// of the rows below r:
__host__ __device__ constexpr int core_groups_before(int r) {
  return r <= 1 ? 0 : 4 * ((r - 1) / 8) * ((r - 1) / 8 + 1) + ((r - 1) % 8) * ((r - 1) / 8 + 1);
}
static_assert(core_groups_before(9) == 8 && core_groups_before(10) == 10 &&
                  core_groups_before(17) == 24,
              "row-aligned group count");
__device__ __forceinline__ uint32_t core_group_entry(int k, int g) {
  if (k >= core_groups_before(g)) return 0xFFFF0000u;
  int lo = 1, hi = g - 1;  // the row r with groups_before(r) <= k < groups_before(r + 1)
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (core_groups_before(mid) <= k) lo = mid;
    else hi = mid - 1;
  }
  return ((uint32_t)lo << 16) | (uint32_t)(8 * (k - core_groups_before(lo)));
}

// 4-cell Y: row (group*32 + 4q + 2a + b) = indicator over the samples of
// pair q of the group having (x_row = a-1, x_col = b-1), a, b in {0, 1};
// padding pairs are zero.
__device__ __forceinline__ void build_y_core_chunk(const uint64_t *planes, int g, int W, int n_pad,
                                                   long long idx, uint8_t *Y) {
  const int chunks = n_pad / 16;
  const int rr = (int)(idx / chunks), ch = (int)(idx % chunks);
  const uint32_t e = core_group_entry(rr / 32, g);
  const int row = (int)(e >> 16), col = (int)(e & 0xFFFFu) + (rr % 32) / 4;
  uint32_t bits = 0;
  if (row != 0xFFFF && col < row) bits = pair_bits16(planes, W, row, (rr >> 1) & 1, col, rr & 1, ch);
  store_e4m3_16(Y + (size_t)rr * n_pad + ch * 16, bits);
}

// 4-cell full-sample tables, one group: 8 float4 of the counted cells (0, 1,
// 3, 4 of the nine; zero for padding pairs), then the prior bits of the
// group's pairs and three zero words (144 bytes).
__device__ __forceinline__ void ctot_core_group(const uint16_t *ctot, const uint8_t *prior, int g,
                                                int grp, float *out) {
  float4 *o = reinterpret_cast<float4 *>(out + (size_t)grp * (kGroupCtBytes / 4));
  const uint32_t e = core_group_entry(grp, g);
  const int row = (int)(e >> 16), col0 = (int)(e & 0xFFFFu);
  uint32_t pb = 0;
  for (int q = 0; q < kCorePairs; q++) {
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (row != 0xFFFF && col0 + q < row) {
      const int p = row * (row - 1) / 2 + col0 + q;
      const uint16_t *t = ctot + (size_t)p * 9;
      v = make_float4((float)t[0], (float)t[1], (float)t[3], (float)t[4]);
      if (prior[p]) pb |= 1u << q;
    }
    o[q] = v;
  }
  o[kCorePairs] = make_float4(__uint_as_float(pb), 0.f, 0.f, 0.f);
}

// Full-sample counts of gene i's states -1, 0, 1 (4-cell layout).
__device__ __forceinline__ void gene_counts(const uint64_t *planes, int W, int i, float4 *out) {
  int cnt[3] = {0, 0, 0};
  for (int a = 0; a < 3; a++)
    for (int w = 0; w < W; w++) cnt[a] += __popcll(planes[((size_t)i * 3 + a) * W + w]);
  out[i] = make_float4((float)cnt[0], (float)cnt[1], (float)cnt[2], 0.f);
}

// The per-set operands in one launch of 128-thread blocks: blocks [0, b[0])
// build Y, [b[0], b[1]) the FP32 tables and, in the 4-cell layout,
// [b[1], b[2]) the group table and [b[2], b[3]) the genes' counts.
struct SetupArgs {
  const uint64_t *planes;
  const uint16_t *ctot;
  const uint8_t *prior;
  int g, W, c, n_pad, ngroups, core;
  int b[4];
  uint8_t *Y;
  float *ctf;
  uint32_t *gtab;
  float4 *gcnt;
};
__global__ void __launch_bounds__(128) k_setup(const __grid_constant__ SetupArgs a) {
  const int blk = blockIdx.x;
  if (blk < a.b[0]) {
    const long long idx = (long long)blk * 128 + threadIdx.x;
    if (idx >= (long long)a.ngroups * 32 * (a.n_pad / 16)) return;
    if (a.core) build_y_core_chunk(a.planes, a.g, a.W, a.n_pad, idx, a.Y);
    else build_y_chunk(a.planes, a.W, a.c, a.n_pad, idx, a.Y);
  } else if (blk < a.b[1]) {
    const int i = (blk - a.b[0]) * 128 + threadIdx.x;
    if (a.core) {
      if (i < a.ngroups) ctot_core_group(a.ctot, a.prior, a.g, i, a.ctf);
    } else if (i < a.ngroups * kPairsPerGroup) {
      ctot_f_pair(a.ctot, a.prior, a.c, i, a.ctf);
    }
  } else if (blk < a.b[2]) {
    const int k = (blk - a.b[1]) * 128 + threadIdx.x;
    if (k < a.ngroups) a.gtab[k] = core_group_entry(k, a.g);
  } else if (blk < a.b[3]) {
    const int i = (blk - a.b[2]) * 128 + threadIdx.x;
    if (i < a.g) gene_counts(a.planes, a.W, i, a.gcnt);
  }
}

// Class-1 counts of kMargGenes genes' states -1 and 0 for unit u (4-cell
// layout): margc[i * Bp + u] = count(-1) | count(0) << 16 over the unit's
// class-1 samples, and (for the first gene block) nc1[u] = its class-1
// sample count; units >= B count nothing.  The mask word is read once for
// all the genes.
constexpr int kMargGenes = 8;
__device__ __forceinline__ void margins_unit(const uint64_t *masks, const uint64_t *planes, int B,
                                             int Bp, int g, int W, int u, int i0, uint32_t *margc,
                                             float *nc1) {
  int cnt[kMargGenes][2];
#pragma unroll
  for (int k = 0; k < kMargGenes; k++) cnt[k][0] = cnt[k][1] = 0;
  int tot = 0;
  for (int w = 0; w < W; w++) {
    const uint64_t m = u < B ? masks[(size_t)u * W + w] : 0ull;
    tot += __popcll(m);
#pragma unroll
    for (int k = 0; k < kMargGenes; k++) {
      if (i0 + k < g) {
        cnt[k][0] += __popcll(m & planes[((size_t)(i0 + k) * 3 + 0) * W + w]);
        cnt[k][1] += __popcll(m & planes[((size_t)(i0 + k) * 3 + 1) * W + w]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kMargGenes; k++)
    if (i0 + k < g) margc[(size_t)(i0 + k) * Bp + u] = (uint32_t)cnt[k][0] | ((uint32_t)cnt[k][1] << 16);
  if (i0 == 0) nc1[u] = (float)tot;
}

// The per-batch operands in one launch of 128-thread blocks.  Blocks
// [0, bA): the A operand, one 16-sample chunk of one row per thread; row r
// of set k (128 mb0 <= r < 128 (mb0 + mblocks)) is the class-1 mask of its
// unit r - 128 mb0, e4m3 0/1, and zero past the set's nb units.  Then, in
// the 4-cell layout, each set's mblocks x ceil(g / 8) blocks of class
// counts (from its marg_b0).  Block 0 also zeroes the general-path queue's
// header.
__global__ void __launch_bounds__(128)
    k_operands(const BatchSet *__restrict__ sets, int nsets, const uint64_t *masks, int W,
               int n_pad, int rowsA, int bA, uint8_t *A, uint32_t *margc, unsigned *gqueue) {
  const int blk = blockIdx.x;
  if (blk == 0 && threadIdx.x < 4) gqueue[threadIdx.x] = 0u;  // the queue header
  if (blk < bA) {
    const int chunks = n_pad / 16;
    const long long idx = (long long)blk * 128 + threadIdx.x;
    if (idx >= (long long)rowsA * chunks) return;
    const int r = (int)(idx / chunks), ch = (int)(idx % chunks);
    int lo = 0, hi = nsets - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sets[mid].mb0 * 128 <= r) lo = mid;
      else hi = mid - 1;
    }
    const BatchSet &bs = sets[lo];
    const int ul = r - bs.mb0 * 128;
    const int s0 = ch * 16, w = s0 >> 6, sh = s0 & 63;
    uint32_t bits = 0;
    if (ul < bs.nb && w < W) bits = (uint32_t)(masks[(size_t)(bs.u0 + ul) * W + w] >> sh) & 0xFFFFu;
    store_e4m3_16(A + (size_t)r * n_pad + ch * 16, bits);
    return;
  }
  const int m = blk - bA;
  int lo = 0, hi = nsets - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (sets[mid].marg_b0 <= m) lo = mid;
    else hi = mid - 1;
  }
  const BatchSet &bs = sets[lo];
  const int mm = m - bs.marg_b0, ub = bs.mblocks, Bp = ub * 128;
  const int ul = (mm % ub) * 128 + threadIdx.x, i0 = (mm / ub) * kMargGenes;
  uint32_t *mc = margc + bs.mg0;
  margins_unit(masks + (size_t)bs.u0 * W, bs.sd.planes, bs.nb, Bp, bs.sd.g, W, ul, i0, mc,
               reinterpret_cast<float *>(mc + (size_t)bs.sd.g * Bp));
}

// ------------------------------------------------------------ host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

static bool make_map(CUtensorMap *m, void *ptr, int cols, int rows, int box_rows) {
  EncodeTiledFn f = encode_fn();
  if (!f) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols};
  cuuint32_t box[2] = {(cuuint32_t)kKC, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1u, 1u};
  return f(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, ptr, dims, strides, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// pair groups of a set, and that count padded for every variant
static int ngroups_of(const SetDev &sd, bool core) {
  return core ? core_groups_before(sd.g) : (sd.c + kPairsPerGroup - 1) / kPairsPerGroup;
}
int mma_ngroups_pad(const SetDev &sd, bool core) {
  const int g = ngroups_of(sd, core);
  return (g > 0 ? (g + kGroupPad - 1) / kGroupPad : 1) * kGroupPad;
}
int mma_npad(int n) { return (n + kKC - 1) / kKC * kKC; }
// The Y arena: the operand Y (G x 32 rows of n_pad samples), the FP32
// full-sample tables (a multiple of 128 bytes in, kGroupCtBytes per group),
// the group table (4 bytes per group) and, 16-byte aligned, the genes'
// full-sample state counts (16 bytes per gene).
static size_t y_ct_offset(const YArena &y) { return (size_t)y.G * 32 * mma_npad(y.n); }
static size_t y_gt_offset(const YArena &y) { return y_ct_offset(y) + (size_t)kGroupCtBytes * y.G; }
static size_t y_gc_offset(const YArena &y) {
  return (y_gt_offset(y) + sizeof(uint32_t) * (size_t)y.G + 15) & ~(size_t)15;
}
size_t mma_y_bytes(int G, int genes, int n) {
  const YArena y{nullptr, G, genes, n};
  return y_gc_offset(y) + sizeof(float4) * (size_t)genes;
}
// the A operand, then the general-path queue: a 16-byte counter and room
// for every table of the batch (near-threshold workloads send half of them
// or more to the general path), at least 65536 and at most 2^28 items
// (7.5 GB with the deferred list; the list's entries, item * 10 + slot,
// stay below 2^32)
static size_t a_operand_bytes(int rowsA, int n) { return (size_t)rowsA * mma_npad(n); }
static unsigned queue_cap(long long tables) {
  const long long t = tables < (1ll << 28) ? tables : (1ll << 28);
  return (unsigned)(t < 65536 ? 65536 : t);
}
// EDDY_GENERAL_QUEUE_CAP lowers the queue's capacity (tests of the
// overflow path: the batch is then decided by the popcount kernel)
static unsigned queue_cap_used(long long tables) {
  const unsigned cap = queue_cap(tables);
  const char *e = getenv("EDDY_GENERAL_QUEUE_CAP");
  if (!e) return cap;
  const long v = atol(e);
  return (v >= 1 && (unsigned long)v < cap) ? (unsigned)v : cap;
}
// operand, queue header, items and the list of exact decisions, then (4-cell
// layout, 256-byte aligned) the sets' class counts and class sizes
static size_t margins_offset(const MmaPlan &p, int n) {
  const size_t q = a_operand_bytes(p.rowsA, n) + 16 +
                   (size_t)queue_cap(p.tables) * (kQWords + 1) * sizeof(uint32_t);
  return (q + 255) & ~(size_t)255;
}
size_t mma_a_bytes(const MmaPlan &p, int n, bool core) {
  if (!core)
    return a_operand_bytes(p.rowsA, n) + 16 +
           (size_t)queue_cap(p.tables) * (kQWords + 1) * sizeof(uint32_t);
  return margins_offset(p, n) + sizeof(uint32_t) * (size_t)p.marg_words;
}

// column groups per tile of each variant (see launch_shape)
static int groups_of_variant(int v) {
  static const int kg[5] = {4, 4, 6, 8, 8};
  return kg[v % 5];
}

MmaPlan mma_plan(BatchSet *sets, int nsets, int variant, bool core) {
  const int kg = groups_of_variant(variant);
  MmaPlan p{};
  int mb = 0, tile = 0, bm = 0;
  long long mg = 0, tables = 0;
  for (int k = 0; k < nsets; k++) {
    BatchSet &b = sets[k];
    b.mblocks = (b.nb + kTM - 1) / kTM;
    b.mb0 = mb;
    mb += b.mblocks;
    const int ng = ngroups_of(b.sd, core);
    b.ntn = ng > 0 ? (ng + kg - 1) / kg : 1;
    b.tile0 = tile;
    tile += b.ntn * b.mblocks;
    b.marg_b0 = bm;
    b.mg0 = mg;
    if (core) {
      bm += b.mblocks * ((b.sd.g + kMargGenes - 1) / kMargGenes);
      mg += (long long)(b.sd.g + 1) * kTM * b.mblocks;
    }
    tables += 2ll * b.nb * (b.sd.c > 0 ? b.sd.c : 1);
  }
  p.rowsA = mb * kTM;
  p.ntot = tile;
  p.bM = bm;
  p.marg_words = mg;
  p.tables = tables;
  return p;
}

cudaError_t launch_build_y(const SetDev &sd, bool core, const YArena &y, int grp0, int gc0,
                           cudaStream_t st) {
  const int ng = mma_ngroups_pad(sd, core), np = mma_npad(sd.n);
  const long long work = (long long)ng * 32 * (np / 16);
  SetupArgs a{};
  a.planes = sd.planes;
  a.ctot = sd.ctot;
  a.prior = sd.prior;
  a.g = sd.g;
  a.W = sd.W;
  a.c = sd.c;
  a.n_pad = np;
  a.ngroups = ng;
  a.core = core ? 1 : 0;
  a.Y = y.base + (size_t)grp0 * 32 * np;
  a.ctf = reinterpret_cast<float *>(y.base + y_ct_offset(y)) + (size_t)grp0 * (kGroupCtBytes / 4);
  a.b[0] = (int)((work + 127) / 128);
  a.b[1] = a.b[0] + (core ? (ng + 127) / 128 : (ng * kPairsPerGroup + 127) / 128);
  a.b[2] = a.b[1];
  a.b[3] = a.b[1];
  if (core) {
    a.gtab = reinterpret_cast<uint32_t *>(y.base + y_gt_offset(y)) + grp0;
    a.gcnt = reinterpret_cast<float4 *>(y.base + y_gc_offset(y)) + gc0;
    a.b[2] = a.b[1] + (ng + 127) / 128;
    a.b[3] = a.b[2] + (sd.g + 127) / 128;
  }
  k_setup<<<a.b[3], 128, 0, st>>>(a);
  return cudaGetLastError();
}
int mma_build_launches(const SetDev &) { return 1; }

template <int kStages, int kEpi, int kGroups, bool kCore>
static cudaError_t launch_variant(const BatchSet *sets, int nsets, const MmaPlan &plan,
                                  const int32_t *uslot, int n, const uint8_t *Afp8,
                                  const YArena &y, unsigned *gqueue, unsigned qcap,
                                  uint32_t *dmask, unsigned long long *stats, unsigned *err,
                                  int sms, cudaStream_t st, int g_single) {
  constexpr int kTN = 32 * kGroups;
  const int np = mma_npad(n);
  CUtensorMap ma, mb;
  if (!make_map(&ma, (void *)Afp8, np, plan.rowsA, kTM) ||
      !make_map(&mb, (void *)y.base, np, y.G * 32, kTN))
    return cudaErrorNotSupported;
  const float *ctotf = reinterpret_cast<const float *>(y.base + y_ct_offset(y));
  const uint32_t *margc = nullptr;
  const float4 *gcnt = nullptr;
  const uint32_t *gtab = nullptr;
  if (kCore) {
    margc = reinterpret_cast<const uint32_t *>(Afp8 + margins_offset(plan, n));
    gcnt = reinterpret_cast<const float4 *>(y.base + y_gc_offset(y));
    gtab = reinterpret_cast<const uint32_t *>(y.base + y_gt_offset(y));
  }
  const size_t smem = 1024 + (size_t)kStages * (kTM + kTN) * kKC + kBarBytes +
                      (kCore && nsets == 1 ? sizeof(float4) * (size_t)g_single : 0);
  auto kern = k_pairs_mma<kStages, kEpi, kGroups, kCore>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int grid = plan.ntot < sms ? plan.ntot : sms;
  kern<<<grid, 32 * (2 + kEpi), smem, st>>>(ma, mb, sets, nsets, ctotf, np / kKC, plan.ntot,
                                            stats, err, gqueue, qcap, margc, gcnt, gtab);
  return cudaGetLastError();
}

// 0: N=128, 16 epilogue warps; 1: N=128, 8 warps; 2: N=192, 12 warps;
// 3: N=256, 8 warps; 4: N=256, 16 warps (ring depths fill the shared memory)
int mma_variants() { return 5; }
// operands (and class counts), GEMM + epilogue, general path, exact path
int mma_launches() { return 4; }

template <bool kCore>
static cudaError_t launch_shape(const BatchSet *sets, int nsets, const MmaPlan &plan,
                                const int32_t *uslot, int n, const uint8_t *Afp8,
                                const YArena &y, unsigned *gqueue, unsigned qcap,
                                uint32_t *dmask, unsigned long long *stats, unsigned *err,
                                int sms, cudaStream_t st, int variant, int g_single) {
#define EDDY_VARIANT(S_, E_, G_)                                                              \
  return launch_variant<S_, E_, G_, kCore>(sets, nsets, plan, uslot, n, Afp8, y, gqueue, qcap, \
                                           dmask, stats, err, sms, st, g_single)
  switch (variant) {
    case 1: EDDY_VARIANT(6, 8, 4);
    case 2: EDDY_VARIANT(5, 12, 6);
    case 3: EDDY_VARIANT(4, 8, 8);
    case 4: EDDY_VARIANT(4, 16, 8);
    default: EDDY_VARIANT(6, 16, 4);
  }
#undef EDDY_VARIANT
}

cudaError_t launch_pairs_mma(const BatchSet *sets, int nsets, const MmaPlan &plan,
                             const uint64_t *masks, const int32_t *uslot, int n, int W,
                             uint8_t *Afp8, const YArena &y, uint32_t *dmask,
                             unsigned long long *stats, unsigned *err, int sms, cudaStream_t st,
                             int variant, bool core, int g_single, cudaEvent_t ev_mid,
                             bool ev_external) {
  const int np = mma_npad(n);
  const long long work = (long long)plan.rowsA * (np / 16);
  const int bA = (int)((work + 127) / 128);
  unsigned *gqueue = reinterpret_cast<unsigned *>(Afp8 + a_operand_bytes(plan.rowsA, n));
  uint32_t *margc = core ? reinterpret_cast<uint32_t *>(Afp8 + margins_offset(plan, n)) : nullptr;
  k_operands<<<bA + (core ? plan.bM : 0), 128, 0, st>>>(sets, nsets, masks, W, np, plan.rowsA, bA,
                                                        Afp8, margc, gqueue);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const unsigned qcap = queue_cap_used(plan.tables);
  e = core ? launch_shape<true>(sets, nsets, plan, uslot, n, Afp8, y, gqueue, qcap, dmask, stats,
                                err, sms, st, variant % mma_variants(), g_single)
           : launch_shape<false>(sets, nsets, plan, uslot, n, Afp8, y, gqueue, qcap, dmask, stats,
                                 err, sms, st, variant % mma_variants(), g_single);
  if (e != cudaSuccess) return e;
  // the end of the contraction (a record node when the stream is captured)
  if (ev_mid) {
    e = ev_external ? cudaEventRecordWithFlags(ev_mid, st, cudaEventRecordExternal)
                    : cudaEventRecord(ev_mid, st);
    if (e != cudaSuccess) return e;
  }
  k_general<<<sms * 8, 256, 0, st>>>(sets, uslot, gqueue, qcap, dmask, stats, err);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // one-warp blocks: the first sms of them land one per SM, which is all a
  // short list needs; near-threshold batches (hundreds of thousands of
  // rechecks) fill eight per SM, whose independent FP64 chains keep the
  // SM's FP64 pipe busy while each waits on its own dependent operations
  k_exact<<<sms * 8, 32, 0, st>>>(sets, uslot, gqueue, qcap, dmask, stats);
  return cudaGetLastError();
}

}  // namespace eddy
