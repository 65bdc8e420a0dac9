// eddy_noalloc.cu -- eddy_unit_noalloc(): the per-labelling hot path with no
// device allocation at all.
//
// Who needs it: programs that embed EDDY in a host application that owns
// every byte of GPU memory through its own pool or arena (and cannot let a
// library call cudaMalloc behind its back), and pipelines that must not pay
// the implicit device-wide synchronisation that cudaFree can cause.  Such
// callers hand over host buffers and get host results back; everything in
// between lives in one file-scope device array of fixed size.
//
// The array (kNoAllocBytes, about 2.6 MB) is part of the library image: every
// GPU that loads libeddy_gpu holds it until the process exits.  Host code
// cannot use the array's name as a device address (in host code it is only
// a stand-in symbol), so the first call on each device resolves the address
// with cudaGetSymbolAddress while that device is current and caches it; make
// that first call before any stream capture.  All calls share the array and
// each call rewrites every region it reads, so nothing carries over from the
// previous call.  Calls from one process are serialised by a lock, and each
// call, including one that fails after it has queued work, waits for its
// stream before it returns; calls whose GPU work overlaps (other processes
// sharing the context, or work the caller enqueues on the array by other
// means) race on it.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <mutex>

#include "eddy_gpu.h"
#include "eddy_host.h"
#include "eddy_internal.h"
#include "eddy_kernels.h"

namespace eddy {
namespace {

constexpr int kNAMaxGenes = 64;
constexpr int kNAMaxSamples = 2048;
constexpr int kNAPairs = kNAMaxGenes * (kNAMaxGenes - 1) / 2;
constexpr int kNAW = kNAMaxSamples / 64;
constexpr int kNAKmax = kNAMaxGenes + 1;  // a network changes at most g nodes

__host__ __device__ constexpr size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// region sizes at the maximum shape
constexpr size_t kOffVals = 0;
constexpr size_t kOffValsT = kOffVals + al256((size_t)kNAMaxGenes * kNAMaxSamples);
constexpr size_t kOffPlanes = kOffValsT + al256((size_t)st_stride(kNAMaxGenes) * kNAMaxSamples);
constexpr size_t kOffValid = kOffPlanes + al256(2 * 8ull * kNAMaxGenes * 3 * kNAW);  // + word-major
constexpr size_t kOffCtot = kOffValid + al256(8ull * kNAW);
constexpr size_t kOffPrior = kOffCtot + al256(2ull * 9 * kNAPairs);
constexpr size_t kOffMask = kOffPrior + al256((size_t)kNAPairs);
constexpr size_t kOffLg = kOffMask + al256(8ull * kNAW);
constexpr size_t kOffDmask = kOffLg + al256(8ull * kDivisors * (kNAMaxSamples + 1));
constexpr size_t kOffOut = kOffDmask + al256(dmask_bytes(1, kNAPairs));  // js, U, status
constexpr size_t kOffSets = kOffOut + 256;  // the one-set table and the unit's slot (0)
constexpr size_t kOffSlot = kOffSets + al256(sizeof(BatchSet));
constexpr size_t kOffUnit = kOffSlot + 256;

}  // namespace

// size of the per-unit scratch at the maximum shape (computed at set-up)
size_t unit_scratch_bytes(int c, int S, int kmax);

namespace {
constexpr size_t kNoAllocBytes = kOffUnit + (2u << 20);  // unit scratch <= 2 MB (checked)

static __device__ __align__(256) unsigned char g_noalloc[kNoAllocBytes];

struct DevSlot {
  unsigned char *ptr = nullptr;
};
DevSlot g_slots[64];
// One call at a time per process: the device array and these host staging
// buffers are shared by every call.
std::mutex g_call;
int64_t g_lg_host[kDivisors * (kNAMaxSamples + 1)];
int8_t g_vals_host[kNAMaxGenes * kNAMaxSamples];

// Once per device, with that device current: the array's device address
// and the BDeu divisor map in constant memory (the map is the same for
// every sample count, so later calls never rewrite it).
int setup_device(int dev, unsigned char **out) {
  if (dev < 0 || dev >= 64) return EDDY_ERR_ARG;
  if (!g_slots[dev].ptr) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc) != cudaSuccess || p == nullptr) return EDDY_ERR_CUDA;
    int shift = 0;
    int8_t dmap[82];
    bdeu_table_into(1, g_lg_host, shift, dmap);
    if (set_divisor_map(dmap) != cudaSuccess) return EDDY_ERR_CUDA;
    g_slots[dev].ptr = (unsigned char *)p;
  }
  *out = g_slots[dev].ptr;
  return EDDY_OK;
}

}  // namespace
}  // namespace eddy

using namespace eddy;

extern "C" int eddy_unit_noalloc(const eddy_opts *opts, const int8_t *vals, int g, int n,
                                 const uint8_t *labels, const uint8_t *prior, void *stream,
                                 double *js, int32_t *unique) {
  if (!opts || !vals || !labels || !js || !unique) return EDDY_ERR_ARG;
  if (g < 2 || n < 2 || opts->max_parents < 1) return EDDY_ERR_ARG;
  if (g > kNAMaxGenes || n > kNAMaxSamples) return EDDY_ERR_CAPACITY;
  const int c = g * (g - 1) / 2, W = (n + 63) / 64, S = n + 2;
  if (unit_scratch_bytes(c, S, kNAKmax) > (2u << 20)) return EDDY_ERR_CAPACITY;
  int nA = 0;
  for (int s = 0; s < n; s++) {
    if (labels[s] > 1) return EDDY_ERR_ARG;
    nA += labels[s] == 0;
  }
  if (nA == 0 || nA == n) return EDDY_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return EDDY_ERR_CUDA;
  std::lock_guard<std::mutex> call_lock(g_call);
  unsigned char *base = nullptr;
  int rc = setup_device(dev, &base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;

  // host-side staging in fixed-size stack/static buffers (no heap)
  uint64_t mask[kNAW];
  for (int w = 0; w < W; w++) mask[w] = 0;
  for (int s = 0; s < n; s++)
    if (labels[s] == 0) mask[s >> 6] |= 1ull << (s & 63);
  uint8_t pbits[kNAPairs];
  for (int r = 1, p = 0; r < g; r++)
    for (int col = 0; col < r; col++, p++) pbits[p] = (prior && prior[(size_t)r * g + col] == 1) ? 1 : 0;
  int8_t *v8 = g_vals_host;
  for (size_t i = 0; i < (size_t)g * n; i++) v8[i] = (vals[i] >= -1 && vals[i] <= 1) ? vals[i] : 2;
  int shift = 0;
  int8_t dmap[82];
  bdeu_table_into(n, g_lg_host, shift, dmap);
  // From the first enqueue on, an error return first waits for this call's
  // work on the stream (ignoring that wait's own status): the lock must not
  // be released while copies or kernels of this call may still use the
  // shared array.
  auto bail = [st](int code) {
    cudaStreamSynchronize(st);
    return code;
  };
  if (cudaMemcpyAsync(base + kOffLg, g_lg_host, 8ull * kDivisors * (n + 1), cudaMemcpyHostToDevice,
                      st) != cudaSuccess)
    return bail(EDDY_ERR_CUDA);
  if (cudaMemcpyAsync(base + kOffVals, v8, (size_t)g * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(base + kOffMask, mask, 8ull * W, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(base + kOffPrior, pbits, (size_t)c, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return bail(EDDY_ERR_CUDA);
  if (launch_prep((const int8_t *)(base + kOffVals), g, n, W, c, (uint64_t *)(base + kOffPlanes),
                  (uint64_t *)(base + kOffValid), (uint16_t *)(base + kOffCtot),
                  (int8_t *)(base + kOffValsT), st) != cudaSuccess)
    return bail(EDDY_ERR_CUDA);

  SetDev sd{};
  sd.g = g;
  sd.n = n;
  sd.W = W;
  sd.c = c;
  sd.nA = nA;
  sd.nB = n - nA;
  sd.S = S;
  sd.mp = opts->max_parents;
  sd.GW = (g + 31) / 32;
  sd.bonf = opts->bonferroni ? 1 : 0;
  sd.alpha_edge = opts->alpha_edge;
  sd.alpha_edge_prior = opts->alpha_edge_prior;
  sd.exact_all = compute_thresholds(sd.alpha_edge, sd.alpha_edge_prior, g, sd.bonf, sd.thr) ? 1 : 0;
  sd.planes = (const uint64_t *)(base + kOffPlanes);
  sd.planesT = sd.planes + (size_t)g * 3 * W;
  sd.valid = (const uint64_t *)(base + kOffValid);
  sd.vals = (const int8_t *)(base + kOffVals);
  sd.valsT = (const int8_t *)(base + kOffValsT);
  sd.ctot = (const uint16_t *)(base + kOffCtot);
  sd.prior = (const uint8_t *)(base + kOffPrior);
  sd.lg = (const int64_t *)(base + kOffLg);
  sd.lg_stride = n + 1;
  sd.lg_shift = shift;

  double *d_js = (double *)(base + kOffOut);
  int32_t *d_U = (int32_t *)(base + kOffOut + 8);
  uint32_t *d_status = (uint32_t *)(base + kOffOut + 12);
  const BatchSet *d_sets = (const BatchSet *)(base + kOffSets);
  const int32_t *d_slot = (const int32_t *)(base + kOffSlot);
  if (cudaMemsetAsync(base + kOffSlot, 0, sizeof(int32_t), st) != cudaSuccess)
    return bail(EDDY_ERR_CUDA);
  uint64_t salt = 0x5EED5EEDull;
  for (int attempt = 0; attempt < 4; attempt++) {
    sd.salt = salt;
    // the batch's set table: this one set, its unit 0, its masks and
    // scratch at the start of their regions (a host copy on the stack)
    BatchSet bs{};
    bs.sd = sd;
    bs.nb = 1;
    bs.unit_bytes = (long long)unit_scratch_bytes(c, S, kNAKmax);
    // decisions (the unit kernel zeroes the masks it reads, so every attempt
    // decides again), from masks and a chunk bitmap that start at zero
    if (cudaMemcpyAsync(base + kOffSets, &bs, sizeof bs, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(base + kOffDmask, 0, dmask_bytes(1, c), st) != cudaSuccess ||
        launch_pairs(d_sets, d_slot, (const uint64_t *)(base + kOffMask),
                     (uint32_t *)(base + kOffDmask), 1, W, c, nullptr, st) != cudaSuccess)
      return bail(EDDY_ERR_CUDA);
    BatchDev bd{};
    bd.B = 1;
    bd.nsets = 1;
    bd.kmax = kNAKmax;
    bd.sets = d_sets;
    bd.uslot = d_slot;
    bd.masks = (const uint64_t *)(base + kOffMask);
    bd.dmask = (uint32_t *)(base + kOffDmask);
    bd.scratch = base + kOffUnit;
    bd.js = d_js;
    bd.U = d_U;
    bd.status = d_status;
    bd.keep_slot = nullptr;
    bd.stats = nullptr;
    if (launch_units(bd, g, W, st) != cudaSuccess) return bail(EDDY_ERR_CUDA);
    unsigned char out[16];
    if (cudaMemcpyAsync(out, base + kOffOut, 16, cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return bail(EDDY_ERR_CUDA);
    if (cudaStreamSynchronize(st) != cudaSuccess) return EDDY_ERR_CUDA;
    uint32_t status;
    memcpy(js, out, 8);
    memcpy(unique, out + 8, 4);
    memcpy(&status, out + 12, 4);
    if (status == kUnitOk) return EDDY_OK;
    if (!(status & kUnitHashCollision)) return EDDY_ERR_INTERNAL;
    salt = salt * 6364136223846793005ull + 1442695040888963407ull;  // new hash salt
  }
  return EDDY_ERR_INTERNAL;
}
