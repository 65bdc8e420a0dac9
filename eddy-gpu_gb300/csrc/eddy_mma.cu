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
// of TMEM and makes the 10-bit leave-one-out decision masks of both classes
// (kernel1.cu:121-203, 419-431) in the same kernel.
//
// Tile: 128 units (TMEM lanes) x 128 pair-cells (four 32-column groups, each
// 3 pairs x 9 cells + 5 pad columns) x K in 128-sample chunks; operands
// staged by TMA (cp.async.bulk.tensor, 128B swizzle) through an mbarrier
// ring.  Warp roles: 0 = TMA producer, 1 = TMEM owner + MMA issuer, 2.. =
// epilogue warps (kEpi of them; each owns one TMEM lane quadrant and one or
// two column groups, reads them with one tcgen05.ld each and decides their
// pairs from registers).  Accumulators are double-buffered (2 x 128 TMEM
// columns).  Every mbarrier wait is
// bounded (2 s on %globaltimer); a timeout sets an error word, every role
// drains, and TMEM is released before the block exits.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "eddy_device.cuh"
#include "eddy_kernels.h"
#include "eddy_mma.h"

namespace eddy {

namespace {
constexpr int kTM = 128, kTN = 128, kGroups = 4, kPairsPerGroup = 3, kKC = 128;
constexpr int kPairsPerTile = kGroups * kPairsPerGroup;
constexpr uint32_t kStageBytes = (kTM + kTN) * kKC;  // 32 KB
constexpr unsigned long long kTimeoutNs = 2000000000ull;
// general-path queue of an epilogue warp: room for every table of its tile
// share (32 units x 12 pairs x 2 classes / warps of a quadrant), 6 words each
constexpr int kQWords = 6;
constexpr uint32_t kBarBytes = 1024;  // barrier block after the stage ring

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
  while (true) {
    if (mbar_try(a, parity)) return true;
    if (*err) return false;
    if (gtimer() - t0 > kTimeoutNs) {
      atomicExch((unsigned *)err, 1u);
      return false;
    }
  }
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
// Instruction descriptor: D f32, A/B e4m3, both K-major, N = 128, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(kTN >> 3) << 17) |
                            ((uint32_t)(kTM >> 4) << 24);

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t acc) {
  asm volatile(
      "{.reg .pred p; setp.ne.b32 p, %4, 0;"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;}" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(kIdesc), "r"(acc));
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
__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
}  // namespace

template <int kStages>
struct MmaSmem {
  unsigned long long full[kStages], empty[kStages], accfull[2], accempty[2];
  uint32_t tmem_base;
};
static_assert(sizeof(MmaSmem<8>) <= kBarBytes, "barrier block");

// kStages: depth of the TMA ring; kEpi: epilogue warps (8 or 16);
// kMinBlocks: CTAs per SM the register budget is sized for (two CTAs share
// TMEM's 512 columns).  All variants produce identical masks; the autotuner
// picks by time.
template <int kStages, int kEpi, int kMinBlocks>
__global__ void __launch_bounds__(32 * (2 + kEpi), kMinBlocks)
    k_pairs_mma(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                const __grid_constant__ SetDev sd, const float *__restrict__ ctotf, int B, int nk,
                int ntiles, int mblocks, uint32_t *dmask, unsigned long long *stats,
                unsigned *err) {
  constexpr int kQCap = 32 * 2 * kPairsPerGroup * (kGroups / (kEpi / 4));
  extern __shared__ __align__(1024) uint8_t smraw[];
  // 1024-byte aligned stage ring, then barriers, then the epilogue buffer
  uint8_t *base = (uint8_t *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  MmaSmem<kStages> &S = *reinterpret_cast<MmaSmem<kStages> *>(base + kStages * kStageBytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile unsigned *verr = err;
  const int ntot = ntiles * mblocks;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; s++) {
      mbar_init(smem_u32(&S.full[s]), 1);
      mbar_init(smem_u32(&S.empty[s]), 1);
    }
    for (int a = 0; a < 2; a++) {
      mbar_init(smem_u32(&S.accfull[a]), 1);
      mbar_init(smem_u32(&S.accempty[a]), 32 * kEpi);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    // 256 TMEM columns: two 128-column fp32 accumulators
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(
                     smem_u32(&S.tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem_base;

  if (warp == 0) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      for (int t = blockIdx.x; t < ntot && !*verr; t += gridDim.x) {
        const int tn = t / mblocks, mb = t % mblocks;
        for (int kc = 0; kc < nk; kc++) {
          if (!mbar_wait(smem_u32(&S.empty[stage]), phase ^ 1u, verr)) break;
          const uint32_t fb = smem_u32(&S.full[stage]);
          mbar_expect_tx(fb, kStageBytes);
          const uint32_t sa = smem_u32(base + stage * kStageBytes);
          tma_load_2d(sa, &tmA, kc * kKC, mb * kTM, fb);
          tma_load_2d(sa + kTM * kKC, &tmB, kc * kKC, tn * kTN, fb);
          if (++stage == kStages) {
            stage = 0;
            phase ^= 1u;
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int stage = 0, acc = 0;
      uint32_t phase = 0, accphase = 0;
      for (int t = blockIdx.x; t < ntot && !*verr; t += gridDim.x) {
        if (!mbar_wait(smem_u32(&S.accempty[acc]), accphase ^ 1u, verr)) break;
        tc_fence_after();
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
            umma(dcol, sdesc(sa + 32 * k), sdesc(sb + 32 * k), (kc | k) ? 1u : 0u);
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
    }
  } else {
    // epilogue: TMEM lane quadrant = warp % 4; the kEpi/4 warps of a quadrant
    // split the four column groups (one or two each)
    constexpr int kPerQuad = kEpi / 4, kGpw = kGroups / kPerQuad;
    const int quad = warp & 3, wq = (warp - 2) >> 2;
    const int row = quad * 32 + lane;  // TMEM lane = unit within the tile
    int acc = 0;
    uint32_t accphase = 0;
    unsigned nexact = 0, nfilt = 0, ntab = 0;
    // no-edge thresholds of dof 4 without / with a prior (quick_zero_f)
    const float thr0 = sd.exact_all ? -1.f : sd.thr[0][2].chiA;
    const float thr1 = sd.exact_all ? -1.f : sd.thr[1][2].chiA;
    const uint32_t below = (1u << lane) - 1u;
    // this warp's queue of tables for the general path
    uint32_t *gq = reinterpret_cast<uint32_t *>(base + kStages * kStageBytes + kBarBytes) +
                   (size_t)(warp - 2) * kQCap * kQWords;
    for (int t = blockIdx.x; t < ntot && !*verr; t += gridDim.x) {
      const int tn = t / mblocks, mb = t % mblocks;
      if (!mbar_wait(smem_u32(&S.accfull[acc]), accphase, verr)) break;
      tc_fence_after();
      // counts of the warp's group(s): FP32 integers straight from TMEM
      uint32_t r[kGpw][32];
#pragma unroll
      for (int gi = 0; gi < kGpw; gi++) {
        const int grp = wq + gi * kPerQuad;
        tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(acc * kTN + grp * 32), r[gi]);
      }
      tmem_ld_wait();
      tc_fence_before();
      mbar_arrive(smem_u32(&S.accempty[acc]));
      if (++acc == 2) {
        acc = 0;
        accphase ^= 1u;
      }
      const int u = mb * kTM + row;
      const bool valid = u < B;
      // tables the quick filter cannot settle are queued (counts, class,
      // prior, pair, row) and decided after the loop, with the TMEM values
      // no longer live
      int nq = 0;
      auto enqueue = [&](bool flag, const float *o, int cls, int prior, int p) {
        const uint32_t bal = __ballot_sync(0xffffffffu, flag);
        if (flag) {
          uint32_t *it = gq + (size_t)(nq + __popc(bal & below)) * kQWords;
          it[0] = (uint32_t)o[0] | ((uint32_t)o[1] << 16);
          it[1] = (uint32_t)o[2] | ((uint32_t)o[3] << 16);
          it[2] = (uint32_t)o[4] | ((uint32_t)o[5] << 16);
          it[3] = (uint32_t)o[6] | ((uint32_t)o[7] << 16);
          it[4] = (uint32_t)o[8] | ((uint32_t)row << 16) | ((uint32_t)cls << 24) |
                  ((uint32_t)prior << 25);
          it[5] = (uint32_t)p;
        }
        nq += __popc(bal);
      };
#pragma unroll
      for (int gi = 0; gi < kGpw; gi++) {
        const int grp = wq + gi * kPerQuad;
#pragma unroll
        for (int q = 0; q < kPairsPerGroup; q++) {
          const int p = tn * kPairsPerTile + grp * kPairsPerGroup + q;
          if (p >= sd.c) continue;
          // full-sample table (nine counts) and the prior flag of pair p
          const float4 *cf = reinterpret_cast<const float4 *>(ctotf + (size_t)p * 12);
          const float4 f0 = cf[0], f1 = cf[1], f2 = cf[2];
          float oA[9], oB[9];
#pragma unroll
          for (int k = 0; k < 9; k++) oA[k] = __uint_as_float(r[gi][9 * q + k]);
          oB[0] = f0.x - oA[0]; oB[1] = f0.y - oA[1]; oB[2] = f0.z - oA[2];
          oB[3] = f0.w - oA[3]; oB[4] = f1.x - oA[4]; oB[5] = f1.y - oA[5];
          oB[6] = f1.z - oA[6]; oB[7] = f1.w - oA[7]; oB[8] = f2.x - oA[8];
          const int prior = (f2.y != 0.f) ? 1 : 0;
          const float chiA = prior ? thr1 : thr0;
          const bool qa = quick_zero_f(oA, chiA), qb = quick_zero_f(oB, chiA);
          enqueue(valid && !qa, oA, 0, prior, p);
          enqueue(valid && !qb, oB, 1, prior, p);
          if (valid) {
            dmask[(size_t)u * sd.c + p] = 0u;
            nfilt += (unsigned)qa + (unsigned)qb;
            ntab += 2;
          }
        }
      }
      __syncwarp();
      for (int i = lane; i < nq; i += 32) {
        const uint32_t *it = gq + (size_t)i * kQWords;
        const int cls = (it[4] >> 24) & 1, prior = (it[4] >> 25) & 1;
        const int uu = mb * kTM + (int)((it[4] >> 16) & 0xFFu), p = (int)it[5];
        const uint64_t rr = pair_mask_general(
            (int)(it[0] & 0xFFFFu), (int)(it[0] >> 16), (int)(it[1] & 0xFFFFu), (int)(it[1] >> 16),
            (int)(it[2] & 0xFFFFu), (int)(it[2] >> 16), (int)(it[3] & 0xFFFFu), (int)(it[3] >> 16),
            (int)(it[4] & 0xFFFFu), prior, sd);
        const uint32_t m = (uint32_t)rr & 0x3FFu;
        if (m) atomicOr(&dmask[(size_t)uu * sd.c + p], m << (16 * cls));
        nexact += (unsigned)(rr >> 32) & 0xFFFFu;
        nfilt += (unsigned)(rr >> 48) & 1u;
      }
      __syncwarp();
    }
    if (stats) {
      for (int o = 16; o > 0; o >>= 1) {
        nexact += __shfl_down_sync(0xffffffffu, nexact, o);
        nfilt += __shfl_down_sync(0xffffffffu, nfilt, o);
        ntab += __shfl_down_sync(0xffffffffu, ntab, o);
      }
      if (lane == 0) {
        if (nexact) atomicAdd(&stats[0], (unsigned long long)nexact);
        if (ntab) atomicAdd(&stats[1], (unsigned long long)ntab);
        if (nfilt) atomicAdd(&stats[2], (unsigned long long)nfilt);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
  }
}

// -------------------------------------------------------------- operands
// Y: row (tile*128 + h*32 + q*9 + 3a + b), h < 4, q < 3 = indicator over the
// samples of pair tile*12 + h*3 + q having (x_row = a-1, x_col = b-1);
// e4m3 1.0 = 0x38; columns 27..31 of each group and out-of-range pairs are
// zero.
__global__ void k_build_y(const uint64_t *planes, int g, int W, int c, int n_pad, int ntiles,
                          uint8_t *Y) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // 16-sample chunk
  const int chunks = n_pad / 16;
  const long long rows = (long long)ntiles * kTN;
  if (idx >= rows * chunks) return;
  const int rr = (int)(idx / chunks), ch = (int)(idx % chunks);
  const int tile = rr / kTN, r = rr % kTN;
  const int h = r / 32, r32 = r % 32;
  const int q = r32 / 9, cell = r32 % 9;
  const int p = tile * kPairsPerTile + h * kPairsPerGroup + q;
  uint8_t v[16];
  uint32_t bits = 0;
  if (r32 < kPairsPerGroup * 9 && p < c) {
    int row, col;
    pair_rc(p, row, col);
    const int a = cell / 3, b = cell % 3;
    const int s0 = ch * 16;
    const int w = s0 >> 6, sh = s0 & 63;
    if (w < W) {
      uint64_t x = planes[((size_t)row * 3 + a) * W + w] & planes[((size_t)col * 3 + b) * W + w];
      bits = (uint32_t)(x >> sh) & 0xFFFFu;
    }
  }
#pragma unroll
  for (int k = 0; k < 16; k++) v[k] = ((bits >> k) & 1u) ? 0x38 : 0x00;
  uint4 o;
  memcpy(&o, v, 16);
  *reinterpret_cast<uint4 *>(Y + (size_t)rr * n_pad + ch * 16) = o;
}

// Full-sample tables as FP32 for the epilogue: pair p -> 12 floats (nine
// counts, the prior flag, two pad), 48 bytes, float4-aligned.
__global__ void k_ctot_f(const uint16_t *ctot, const uint8_t *prior, int c, float *out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c) return;
  float v[12];
#pragma unroll
  for (int k = 0; k < 9; k++) v[k] = (float)ctot[(size_t)p * 9 + k];
  v[9] = prior[p] ? 1.f : 0.f;
  v[10] = v[11] = 0.f;
  float4 *o = reinterpret_cast<float4 *>(out + (size_t)p * 12);
  o[0] = make_float4(v[0], v[1], v[2], v[3]);
  o[1] = make_float4(v[4], v[5], v[6], v[7]);
  o[2] = make_float4(v[8], v[9], v[10], v[11]);
}

// A: row u = class-1 mask of unit u over the samples, e4m3 0/1; rows >= B zero.
__global__ void k_masks_fp8(const uint64_t *masks, int B, int B_pad, int W, int n_pad, uint8_t *A) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int chunks = n_pad / 16;
  if (idx >= (long long)B_pad * chunks) return;
  const int u = (int)(idx / chunks), ch = (int)(idx % chunks);
  uint32_t bits = 0;
  const int s0 = ch * 16, w = s0 >> 6, sh = s0 & 63;
  if (u < B && w < W) bits = (uint32_t)(masks[(size_t)u * W + w] >> sh) & 0xFFFFu;
  uint8_t v[16];
#pragma unroll
  for (int k = 0; k < 16; k++) v[k] = ((bits >> k) & 1u) ? 0x38 : 0x00;
  uint4 o;
  memcpy(&o, v, 16);
  *reinterpret_cast<uint4 *>(A + (size_t)u * n_pad + ch * 16) = o;
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

static bool make_map(CUtensorMap *m, void *ptr, int cols, int rows) {
  EncodeTiledFn f = encode_fn();
  if (!f) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols};
  cuuint32_t box[2] = {(cuuint32_t)kKC, 128u};
  cuuint32_t es[2] = {1u, 1u};
  return f(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, ptr, dims, strides, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int mma_ntiles(int c) { return (c + kPairsPerTile - 1) / kPairsPerTile; }
int mma_npad(int n) { return (n + kKC - 1) / kKC * kKC; }
// the operand Y, then the FP32 full-sample tables (a multiple of 128 bytes in)
static size_t y_operand_bytes(int c, int n) { return (size_t)mma_ntiles(c) * kTN * mma_npad(n); }
size_t mma_y_bytes(int c, int n) { return y_operand_bytes(c, n) + 48 * (size_t)(c > 0 ? c : 1); }
int mma_bpad(int B) { return (B + kTM - 1) / kTM * kTM; }

cudaError_t launch_build_y(const SetDev &sd, uint8_t *Y, cudaStream_t st) {
  const int nt = mma_ntiles(sd.c), np = mma_npad(sd.n);
  const long long work = (long long)nt * kTN * (np / 16);
  k_build_y<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(sd.planes, sd.g, sd.W, sd.c, np, nt, Y);
  if (sd.c > 0)
    k_ctot_f<<<(sd.c + 255) / 256, 256, 0, st>>>(sd.ctot, sd.prior, sd.c,
                                                  (float *)(Y + y_operand_bytes(sd.c, sd.n)));
  return cudaGetLastError();
}

template <int kStages, int kEpi, int kMinBlocks>
static cudaError_t launch_variant(const CUtensorMap &ma, const CUtensorMap &mb, const SetDev &sd,
                                  const float *ctotf, int B, int np, int nt, int mblocks,
                                  uint32_t *dmask,
                                  unsigned long long *stats, unsigned *err, int sms,
                                  cudaStream_t st) {
  constexpr int kQCap = 32 * 2 * kPairsPerGroup * (kGroups / (kEpi / 4));
  const size_t smem = 1024 + kStages * kStageBytes + kBarBytes +
                      (size_t)kEpi * kQCap * kQWords * sizeof(uint32_t);
  auto kern = k_pairs_mma<kStages, kEpi, kMinBlocks>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int ntot = nt * mblocks;
  const int grid = ntot < sms * kMinBlocks ? ntot : sms * kMinBlocks;
  kern<<<grid, 32 * (2 + kEpi), smem, st>>>(ma, mb, sd, ctotf, B, np / kKC, nt, mblocks, dmask,
                                            stats, err);
  return cudaGetLastError();
}

int mma_variants() { return 2; }

cudaError_t launch_pairs_mma(const SetDev &sd, const uint64_t *masks, int B, uint8_t *Afp8,
                             const uint8_t *Y, uint32_t *dmask, unsigned long long *stats,
                             unsigned *err, int sms, cudaStream_t st, int variant) {
  const int np = mma_npad(sd.n), Bp = mma_bpad(B), nt = mma_ntiles(sd.c);
  const long long work = (long long)Bp * (np / 16);
  k_masks_fp8<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(masks, B, Bp, sd.W, np, Afp8);
  CUtensorMap ma, mb;
  if (!make_map(&ma, Afp8, np, Bp) || !make_map(&mb, (void *)Y, np, nt * kTN))
    return cudaErrorNotSupported;
  const int mblocks = Bp / kTM;
  const float *ctotf = (const float *)(Y + y_operand_bytes(sd.c, sd.n));
  if (variant == 1)
    return launch_variant<4, 8, 1>(ma, mb, sd, ctotf, B, np, nt, mblocks, dmask, stats, err, sms,
                                   st);
  return launch_variant<4, 16, 1>(ma, mb, sd, ctotf, B, np, nt, mblocks, dmask, stats, err, sms,
                                  st);
}

}  // namespace eddy
