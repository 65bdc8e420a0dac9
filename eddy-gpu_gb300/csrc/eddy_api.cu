// eddy_api.cu -- the C ABI of libeddy_gpu (include/eddy_gpu.h): context,
// gene sets, the permutation driver (main.cu:538-1502) and device buffers.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "../../include/eddy_gpu.h"
#include "eddy_host.h"
#include "eddy_internal.h"
#include "eddy_kernels.h"
#include "eddy_mma.h"

using namespace eddy;

namespace {

// Page-locked host staging for the small per-batch transfers (indices in,
// results out): asynchronous copies without the driver's pageable path.
struct PinnedBuf {
  void *p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= n) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    const size_t want = std::max(bytes, (size_t)64 << 10);
    cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
    if (e == cudaSuccess) n = want;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
  }
  template <class T>
  T *as(size_t byte_off = 0) const {
    return reinterpret_cast<T *>(reinterpret_cast<char *>(p) + byte_off);
  }
};

struct DevBuf {
  void *p = nullptr;
  size_t n = 0;
  // grows by at least half its size: sets of varying size do not pay a
  // cudaFree (a device-wide synchronisation) for every small growth
  cudaError_t ensure(size_t bytes) {
    if (bytes <= n) return cudaSuccess;
    const size_t want = std::max(bytes, n + n / 2);
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      e = cudaMalloc(&p, bytes);  // no room for the margin: the exact size
      if (e == cudaSuccess) n = bytes;
      return e;
    }
    n = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  template <class T>
  T *as() const {
    return reinterpret_cast<T *>(p);
  }
};

struct SetHost {
  std::vector<int32_t> genes;
  std::vector<uint8_t> prior;  // g*g or empty
  std::vector<uint8_t> labels; // external labellings R x n
  int R_ext = 0;
  bool done = false;
  std::vector<double> js;
  std::vector<int32_t> U;
  int iterations = 0, failed = 0, betafit_ok = 0;
  double alpha = NAN, beta = NAN, pddn = NAN;
  unsigned long long exact = 0, tables = 0;
  // iteration-0 networks
  int U0 = 0;
  std::vector<int32_t> ids, nodes, epn, edges;
  std::vector<double> lval;
  std::vector<int32_t> el_nodes, el_epn, el_edges;
};

}  // namespace

struct eddy_ctx {
  eddy_opts o{};
  std::string err = "";
  int genes = 0, samples = 0, nA = 0, nB = 0, W = 0;
  std::vector<int8_t> data;
  std::vector<uint8_t> gene_full;  // gene i holds only -1/0/1 values
  std::vector<uint8_t> labels0;
  std::vector<SetHost> sets;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  GlibcRand rng{1};
  std::vector<uint8_t> seen;
  std::vector<int> order;
  // device data
  DevBuf d_lg, d_vals, d_valsT, d_planes, d_valid, d_ctot, d_prior, d_mask0;
  DevBuf d_masks, d_dmask, d_scratch, d_js, d_U, d_status, d_keep, d_uset, d_uperm;
  DevBuf d_oids, d_ocnt, d_opar, d_odist, d_olval, d_orows, d_stats;
  DevBuf d_Y, d_afp8, d_err;  // tensor-core contingency operands
  // d_dmask is all zero between batches (decisions only set bits, the unit
  // kernel clears what it reads) while this equals d_dmask.p; null = unknown
  void *dmask_clean = nullptr;
  PinnedBuf h_stage;          // per-batch indices and results
  PinnedBuf h_vals;           // the resident set's values on their way in
  int sms = 148;
  // autotuned contingency-kernel choice (layout and tile shape) per (n,
  // power of two of the pair count); tuned_variant: the last one used (-1 =
  // none yet)
  std::map<std::pair<int, int>, int> tuned;
  int tuned_variant = -1;
  float tuned_ms[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  // decision thresholds per gene-set size (the Bonferroni factor)
  struct ThrSet {
    Thr t[2][kDofSlots];
    bool exact_all;
  };
  std::map<int, ThrSet> thr_cache;
  // changed-node records per network that units of sets of g genes needed
  // beyond the default (kept across sets and eddy_clear_sets): later
  // batches start there
  std::map<int, int> kmax_hint;
  int lg_shift = 0;
  bool lg_ready = false;
  int lg_n = -1;  // sample count the fixed-point lgamma table was built for
  unsigned long long last_stats[4] = {0, 0, 0, 0};
  // timing of the last run
  double ms_total = 0, ms_pairs = 0, ms_units = 0;
  long long launches = 0;
  uint64_t salt = 0x5EED5EEDull;
  cudaStream_t own_stream = nullptr;
  // the steady-state batch as a CUDA graph: its parameters (key) and the
  // instantiated graph; prep_gen counts rebuilds of the resident set
  std::vector<uintptr_t> graph_key;
  cudaGraphExec_t graph_exec = nullptr;
  // the last batch launched directly: a batch that repeats it is captured
  // (a graph pays off only when it is replayed)
  std::vector<uintptr_t> direct_key;
  long long graph_launches = 0;  // kernels in one replay
  unsigned prep_gen = 0;
  int prepared_set = -1;  // set whose data is resident in d_vals/d_planes/d_ctot
  bool y_ready = false;
  int y_core = -1;  // layout the resident Y operand was built for
};

static int fail(eddy_ctx *c, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CK(call)                                                                            \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return fail(ctx, EDDY_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                  __LINE__);                                                                \
  } while (0)

namespace {

// Device state of the current set.
struct SetRun {
  SetDev sd{};
  int set_id = -1;
};

int prepare_set(eddy_ctx *ctx, int set_id, SetRun &sr) {
  SetHost &S = ctx->sets[set_id];
  const int g = (int)S.genes.size(), n = ctx->samples, W = ctx->W;
  const int c = g * (g - 1) / 2;
  if (g > 512) return fail(ctx, EDDY_ERR_CAPACITY, "gene set %d has %d genes (> 512)", set_id, g);
  CK(cudaSetDevice(ctx->o.device));
  if (!ctx->lg_ready || ctx->lg_n != n) {
    std::vector<int64_t> lg;
    int8_t dmap[82];
    bdeu_table(n, lg, ctx->lg_shift, dmap);
    CK(ctx->d_lg.ensure(lg.size() * sizeof(int64_t)));
    CK(cudaMemcpy(ctx->d_lg.p, lg.data(), lg.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
    CK(set_divisor_map(dmap));
    ctx->lg_ready = true;
    ctx->lg_n = n;
  }
  const bool resident = (ctx->prepared_set == set_id);
  int8_t *vals = nullptr;
  if (!resident) {
    // the previous set's copy out of this staging finished at that set's
    // first synchronisation
    CK(ctx->h_vals.ensure((size_t)g * n + 16));
    vals = ctx->h_vals.as<int8_t>();
    for (int i = 0; i < g; i++)
      memcpy(vals + (size_t)i * n, ctx->data.data() + (size_t)S.genes[i] * n, n);
  }
  std::vector<uint8_t> pbits(c > 0 ? c : 1, 0);
  if (!S.prior.empty() && !resident) {
    int p = 0;
    for (int r = 1; r < g; r++)
      for (int col = 0; col < r; col++, p++) pbits[p] = S.prior[(size_t)r * g + col] == 1 ? 1 : 0;
  }
  if (!resident) {
    ctx->prepared_set = -1;
    CK(ctx->d_vals.ensure((size_t)g * n + 16));
    CK(ctx->d_valsT.ensure((size_t)g * n + 16));
    CK(ctx->d_planes.ensure(2 * sizeof(uint64_t) * (size_t)g * 3 * W));  // planes, word-major copy
    CK(ctx->d_valid.ensure(sizeof(uint64_t) * W));
    CK(ctx->d_ctot.ensure(sizeof(uint16_t) * 9 * (size_t)(c > 0 ? c : 1)));
    CK(ctx->d_prior.ensure(pbits.size()));
    CK(cudaMemcpyAsync(ctx->d_vals.p, vals, (size_t)g * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_prior.p, pbits.data(), pbits.size(), cudaMemcpyHostToDevice, ctx->stream));
    CK(launch_prep(ctx->d_vals.as<int8_t>(), g, n, W, c, ctx->d_planes.as<uint64_t>(),
                   ctx->d_valid.as<uint64_t>(), ctx->d_ctot.as<uint16_t>(),
                   ctx->d_valsT.as<int8_t>(), ctx->stream));
    ctx->launches += 2 + (c > 0);
    ctx->prepared_set = set_id;
    ctx->y_ready = false;
    ctx->prep_gen++;
  }
  SetDev &sd = sr.sd;
  sd = SetDev{};
  sd.g = g;
  sd.n = n;
  sd.W = W;
  sd.c = c;
  sd.nA = ctx->nA;
  sd.nB = ctx->nB;
  sd.S = n + 2;
  sd.mp = ctx->o.max_parents;
  sd.GW = (g + 31) / 32;
  sd.bonf = ctx->o.bonferroni ? 1 : 0;
  sd.alpha_edge = ctx->o.alpha_edge;
  sd.alpha_edge_prior = ctx->o.alpha_edge_prior;
  {
    auto it = ctx->thr_cache.find(g);
    if (it == ctx->thr_cache.end()) {
      eddy_ctx::ThrSet ts;
      ts.exact_all = compute_thresholds(sd.alpha_edge, sd.alpha_edge_prior, g, sd.bonf, ts.t);
      it = ctx->thr_cache.emplace(g, ts).first;
    }
    memcpy(sd.thr, it->second.t, sizeof sd.thr);
    sd.exact_all = it->second.exact_all ? 1 : 0;
  }
  {
    // EDDY_DECISIONS=fp64: the plain FP64 form -- every table of every pair
    // evaluated with the reference's FP64 formula, no FP32 fast path, no
    // leave-one-out filter (the comparator of the batched FP32 form)
    const char *dm = getenv("EDDY_DECISIONS");
    if (dm && strcmp(dm, "fp64") == 0) sd.exact_all = 1;
  }
  {
    // the 4-cell tensor-core layout needs every sample of every gene in one
    // of the three states (a table's margins are then the genes' own class
    // counts); EDDY_PAIR_LAYOUT=full keeps the 9-cell layout
    const char *pl = getenv("EDDY_PAIR_LAYOUT");
    bool full = true;
    for (int v : S.genes) full = full && ctx->gene_full[v];
    sd.core = (full && !(pl && strcmp(pl, "full") == 0)) ? 1 : 0;
  }
  sd.planes = ctx->d_planes.as<uint64_t>();
  sd.planesT = sd.planes + (size_t)g * 3 * sd.W;
  sd.valid = ctx->d_valid.as<uint64_t>();
  sd.vals = ctx->d_vals.as<int8_t>();
  sd.valsT = ctx->d_valsT.as<int8_t>();
  sd.ctot = ctx->d_ctot.as<uint16_t>();
  sd.prior = ctx->d_prior.as<uint8_t>();
  sd.lg = ctx->d_lg.as<int64_t>();
  sd.lg_stride = n + 1;
  sd.lg_shift = ctx->lg_shift;
  sd.salt = ctx->salt;
  sr.set_id = set_id;
  return EDDY_OK;
}

void labels_to_mask(const uint8_t *labels, int n, int W, uint64_t *mask) {
  for (int w = 0; w < W; w++) mask[w] = 0;
  for (int s = 0; s < n; s++)
    if (labels[s] == 0) mask[s >> 6] |= 1ull << (s & 63);
}

// Detailed outputs of one kept unit (host copies).
struct KeepOut {
  int U = 0;
  std::vector<int32_t> ids, cnt, par;
  std::vector<double> dist, lval;
  std::vector<uint32_t> rows;
  int mpk = 0;
};

// Contingency + decision kernel of a batch: the tcgen05 GEMM path unless
// EDDY_PAIRS_KERNEL=popc selects the popcount kernel.
bool use_popc() {
  const char *e = getenv("EDDY_PAIRS_KERNEL");
  return e && strcmp(e, "popc") == 0;
}
// Sets whose every table goes through the exact FP64 formula (the plain
// FP64 form, or alphas outside (0, 1]) are decided by the popcount kernel
// in one pass: the tensor-core epilogue and its general path would settle
// nothing and list ten FP64 decisions per table.
bool use_popc(const SetDev &sd) { return use_popc() || sd.exact_all; }


// Contingency-kernel choices for a batch: tile shape v % mma_variants(), in
// the 4-cell layout when v >= mma_variants() and in the 9-cell layout
// otherwise.  The 4-cell layout is offered to sets that allow it (sd.core)
// from kCoreMinPairs pairs on, in its two shapes with 12 and 16 epilogue
// warps: on smaller sets its 2.67x wider tiles leave SMs idle (measured on
// sets of 30-150 genes), and with fewer warps its epilogue stalls.  Each
// choice costs one timed run of the tuning batch per (samples, pair-count
// class), which workloads of many small sets pay many times.
constexpr int kCoreMinPairs = 8192;
int choices(const SetDev &sd, int *v) {
  const int nv = mma_variants();
  int k = 0;
  if (sd.core && sd.c >= kCoreMinPairs) {
    v[k++] = nv + 4;
    v[k++] = nv + 2;
  }
  for (int i = nv - 1; i >= 0; i--) v[k++] = i;
  return k;
}
// autotuning key: samples, the power of two of the pair count (sets of
// similar size share a choice) and whether the 4-cell layout is on offer
// (a set with missing values must never take a choice tuned without them)
std::pair<int, int> tune_key(const SetDev &sd) {
  int lc = 0;
  while ((1 << lc) < sd.c) lc++;
  return {sd.n, 2 * lc + (sd.core && sd.c >= kCoreMinPairs ? 1 : 0)};
}
SetDev layout_of(const SetDev &sd, int v) {
  SetDev l = sd;
  l.core = v >= mma_variants() ? 1 : 0;
  return l;
}

// Choice for a batch of B units: the tile shape pinned by EDDY_MMA_VARIANT
// (in the set's own layout), the one tuned for the set's shape, or -1 when
// this batch is to tune (B >= 512).  The 4-cell layout wins on large sets;
// on small ones its 2.67x wider tiles leave SMs idle.
int pick_variant(eddy_ctx *ctx, const SetDev &sd, int B) {
  const int nv = mma_variants();
  const char *ev = getenv("EDDY_MMA_VARIANT");
  if (ev) return (sd.core ? nv : 0) + atoi(ev) % nv;
  auto it = ctx->tuned.find(tune_key(sd));
  if (it != ctx->tuned.end()) return it->second;
  if (B >= 512) return -1;
  // untuned small batch: what measured fastest on sets of 39 and of 200
  // genes (4-cell layout from kCoreMinPairs pairs: N = 192 with 12 epilogue
  // warps; else the 9-cell layout: N = 256 with 8)
  if (sd.core && sd.c >= kCoreMinPairs) return nv + 2 % nv;
  return 3 % nv;
}

// Buffers of the tensor-core path for a batch of B units (and the set's Y
// operand, built once per resident set).
int prepare_pairs(eddy_ctx *ctx, const SetDev &sd, int B) {
  if (!ctx->y_ready || ctx->y_core != sd.core) {
    CK(ctx->d_Y.ensure(mma_y_bytes(sd)));
    CK(launch_build_y(sd, ctx->d_Y.as<uint8_t>(), ctx->stream));
    ctx->launches += mma_build_launches(sd);
    ctx->y_ready = true;
    ctx->y_core = sd.core;
  }
  CK(ctx->d_afp8.ensure(mma_a_bytes(sd, B)));
  CK(ctx->d_err.ensure(sizeof(unsigned)));
  return EDDY_OK;
}

// A decision buffer for B units of c pairs that holds only zeros: cleared
// in full after an allocation or a batch that did not finish.
int dmask_ready(eddy_ctx *ctx, int B, int c) {
  CK(ctx->d_dmask.ensure(dmask_bytes(B, c)));
  if (ctx->dmask_clean != ctx->d_dmask.p) {
    CK(cudaMemsetAsync(ctx->d_dmask.p, 0, ctx->d_dmask.n, ctx->stream));
    ctx->dmask_clean = ctx->d_dmask.p;
  }
  return EDDY_OK;
}

int launch_pairs_any(eddy_ctx *ctx, const SetDev &sd, const uint64_t *masks, int B, uint32_t *dmask,
                     unsigned long long *stats, bool force_popc = false) {
  if (sd.c == 0) return EDDY_OK;
  if (use_popc(sd) || force_popc) {
    CK(launch_pairs(sd, masks, dmask, B, stats, ctx->stream));
    ctx->launches += 1;
    return EDDY_OK;
  }
  CK(ctx->d_err.ensure(sizeof(unsigned)));
  CK(cudaMemsetAsync(ctx->d_err.p, 0, sizeof(unsigned), ctx->stream));
  int variant = pick_variant(ctx, sd, B);
  if (variant < 0) {
    // autotune on this batch: time every choice once (same results), keep
    // the fastest for this (g, n); the last run leaves dmask filled
    float best = 1e30f;
    int bi = 0;
    int cand[16];
    const int ncand = choices(sd, cand);
    for (int ci = 0; ci < ncand; ci++) {
      const int v = cand[ci];
      const SetDev sv = layout_of(sd, v);
      {
        int rc = prepare_pairs(ctx, sv, B);  // (re)builds Y for the layout
        if (rc) return rc;
      }
      CK(cudaEventRecord(ctx->ev[2], ctx->stream));
      CK(launch_pairs_mma(sv, masks, B, ctx->d_afp8.as<uint8_t>(), ctx->d_Y.as<uint8_t>(), dmask,
                          nullptr, ctx->d_err.as<unsigned>(), ctx->sms, ctx->stream,
                          v % mma_variants()));
      CK(cudaEventRecord(ctx->ev[3], ctx->stream));
      CK(cudaEventSynchronize(ctx->ev[3]));
      float ms = 0;
      cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
      ctx->tuned_ms[v] = ms;
      if (ms < best) {
        best = ms;
        bi = v;
      }
      ctx->launches += mma_launches(sv);
    }
    ctx->tuned[tune_key(sd)] = bi;
    variant = bi;
  }
  ctx->tuned_variant = variant;
  const SetDev sv = layout_of(sd, variant);
  {
    int rc = prepare_pairs(ctx, sv, B);
    if (rc) return rc;
  }
  CK(launch_pairs_mma(sv, masks, B, ctx->d_afp8.as<uint8_t>(), ctx->d_Y.as<uint8_t>(), dmask, stats,
                      ctx->d_err.as<unsigned>(), ctx->sms, ctx->stream, variant % mma_variants()));
  ctx->launches += mma_launches(sv);
  return EDDY_OK;
}

int check_mma_error(eddy_ctx *ctx, const SetDev &sd) {
  if (use_popc(sd) || ctx->d_err.p == nullptr) return EDDY_OK;
  unsigned e = 0;
  CK(cudaMemcpyAsync(&e, ctx->d_err.p, sizeof e, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (e) return fail(ctx, EDDY_ERR_INTERNAL, "tensor-core pipeline wait timed out");
  return EDDY_OK;
}

// Runs units of one set.  masks_host: B x W host masks, or null to
// generate counter-mode masks for perms[] on the device.
int run_units(eddy_ctx *ctx, SetRun &sr, int nunits, const uint64_t *masks_host,
              const int32_t *perms, double *js, int32_t *U, KeepOut *keep, int mpk_req) {
  SetDev &sd = sr.sd;
  const int W = sd.W, c = sd.c, S = sd.S, g = sd.g;
  const bool keeping = keep != nullptr;
  // batch size: bounded by memory (masks, decisions and scratch);
  // kmax: changed-node records per network (EDDY_KMAX lowers it, to test the
  // re-run of the units that overflow it)
  // (records are written only for changed nodes, so room for more costs
  // memory, not time: 64 covers every network of sets whose pair tests all
  // sit near the threshold, measured at 200 genes)
  int kmax = std::min(g + 1, 64);
  const char *ek = getenv("EDDY_KMAX");
  if (ek) kmax = std::max(1, std::min(16, atoi(ek)));
  else {
    auto it = ctx->kmax_hint.find(g);
    if (it != ctx->kmax_hint.end()) kmax = std::max(kmax, std::min(g + 1, it->second));
  }
  size_t per_unit = unit_scratch_bytes(c, S, kmax) + sizeof(uint32_t) * (size_t)c + 8 * W + 64;
  // (up to 16 GB and 16384 units per batch: the general-path queue holds
  // unit indices below 2^15)
  int Bmax = (int)std::max<size_t>(1, ((size_t)16 << 30) / std::max<size_t>(per_unit, 1));
  Bmax = std::min(Bmax, 16384);
  // the general-path queue has room for every table of a batch, up to 2^28
  // (near-threshold sets queue most of them); the units are then split into
  // batches of equal size, which later calls of the same size replay
  Bmax = (int)std::min<size_t>((size_t)Bmax,
                               std::max<size_t>(1, ((size_t)1 << 28) / (2 * (size_t)std::max(c, 1))));
  {
    const int nb = std::max(1, (nunits + Bmax - 1) / Bmax);
    Bmax = std::max(1, (nunits + nb - 1) / nb);
  }
  std::vector<uint32_t> status;
  const int mpk = std::max(1, mpk_req);
  if (keeping) {
    CK(ctx->d_oids.ensure(sizeof(int32_t) * S));
    CK(ctx->d_ocnt.ensure(sizeof(int32_t) * (size_t)S * g));
    CK(ctx->d_opar.ensure(sizeof(int32_t) * (size_t)S * g * mpk));
    CK(ctx->d_odist.ensure(sizeof(double) * 2 * S));
    CK(ctx->d_olval.ensure(sizeof(double) * 2 * S));
    CK(ctx->d_orows.ensure(sizeof(uint32_t) * 2 * (size_t)g * sd.GW));
    CK(cudaMemsetAsync(ctx->d_opar.p, 0xff, sizeof(int32_t) * (size_t)S * g * mpk, ctx->stream));
  }
  CK(ctx->d_stats.ensure(sizeof(unsigned long long) * 4));
  CK(cudaMemsetAsync(ctx->d_stats.p, 0, sizeof(unsigned long long) * 4, ctx->stream));
  float t_pairs = 0, t_units = 0;
  for (int b0 = 0; b0 < nunits; b0 += Bmax) {
    const int B = std::min(Bmax, nunits - b0);
    int kmax_run = kmax;
    bool popc_batch = false;
    std::vector<int> todo(B);
    for (int i = 0; i < B; i++) todo[i] = i;
    // the batch is run once; units whose status asks for it are re-run
    for (int attempt = 0; attempt < 4 && !todo.empty(); attempt++) {
      const int Bt = (int)todo.size();
      const size_t ub = unit_scratch_bytes(c, S, kmax_run);
      CK(ctx->d_masks.ensure(sizeof(uint64_t) * (size_t)Bt * W));
      {
        int rc = dmask_ready(ctx, Bt, c);
        if (rc) return rc;
      }
      CK(ctx->d_scratch.ensure(ub * Bt));
      CK(ctx->d_js.ensure(sizeof(double) * Bt));
      CK(ctx->d_U.ensure(sizeof(int32_t) * Bt));
      CK(ctx->d_status.ensure(sizeof(uint32_t) * Bt));
      CK(ctx->d_keep.ensure(sizeof(int32_t) * Bt));
      // pinned staging for this attempt's indices and results (grown here,
      // before any copy uses it)
      CK(ctx->h_stage.ensure(16 * (size_t)Bt + 64));
      // steady state (device labellings, nothing kept, tile shape known, the
      // set's operand built): a batch that repeats the previous one's set /
      // shape / buffers is captured as one CUDA graph and later replayed (a
      // set that runs a single batch launches directly: no capture cost)
      const bool graphable = !masks_host && !keeping && !popc_batch && !use_popc(sd) && c > 0 &&
                             ctx->y_ready && ctx->stream != nullptr &&
                             pick_variant(ctx, sd, Bt) >= 0;
      if (masks_host) {
        std::vector<uint64_t> mh((size_t)Bt * W);
        for (int i = 0; i < Bt; i++)
          memcpy(mh.data() + (size_t)i * W, masks_host + (size_t)(b0 + todo[i]) * W, 8 * W);
        CK(cudaMemcpyAsync(ctx->d_masks.p, mh.data(), 8 * mh.size(), cudaMemcpyHostToDevice, ctx->stream));
      } else {
        // (staging: set ids, then permutation indices; the previous batch's
        // copies out of it completed at its synchronisation)
        int32_t *hs = ctx->h_stage.as<int32_t>(), *hp = hs + Bt;
        for (int i = 0; i < Bt; i++) {
          hs[i] = sr.set_id;
          hp[i] = perms[b0 + todo[i]];
        }
        CK(ctx->d_uset.ensure(sizeof(int32_t) * Bt));
        CK(ctx->d_uperm.ensure(sizeof(int32_t) * Bt));
        CK(cudaMemcpyAsync(ctx->d_uset.p, hs, 4 * Bt, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->d_uperm.p, hp, 4 * Bt, cudaMemcpyHostToDevice, ctx->stream));
      }
      // the kept unit (the first of the call) writes its detailed outputs;
      // slot -1 (every byte 0xFF) for the others
      int i0 = -1;
      for (int i = 0; i < Bt && keeping; i++)
        if (b0 + todo[i] == 0) i0 = i;
      CK(cudaMemsetAsync(ctx->d_keep.p, 0xFF, 4 * (size_t)Bt, ctx->stream));
      if (i0 >= 0) CK(cudaMemsetAsync(ctx->d_keep.as<int32_t>() + i0, 0, 4, ctx->stream));
      BatchDev bd{};
      bd.B = Bt;
      bd.kmax = kmax_run;
      bd.masks = ctx->d_masks.as<uint64_t>();
      bd.dmask = ctx->d_dmask.as<uint32_t>();
      bd.scratch = ctx->d_scratch.as<uint8_t>();
      bd.unit_bytes = ub;
      bd.js = ctx->d_js.as<double>();
      bd.U = ctx->d_U.as<int32_t>();
      bd.status = ctx->d_status.as<uint32_t>();
      bd.keep_slot = ctx->d_keep.as<int32_t>();
      bd.out_ids = ctx->d_oids.as<int32_t>();
      bd.out_cnt = ctx->d_ocnt.as<int32_t>();
      bd.out_par = ctx->d_opar.as<int32_t>();
      bd.mpk = mpk;
      bd.out_dist = ctx->d_odist.as<double>();
      bd.out_lval = ctx->d_olval.as<double>();
      bd.out_rows = ctx->d_orows.as<uint32_t>();
      bd.stats = ctx->d_stats.as<unsigned long long>();
      // the batch's device work: labellings, decisions, networks
      // (events become record nodes when captured)
      auto record = [&](cudaEvent_t e, bool capturing) -> cudaError_t {
        return capturing ? cudaEventRecordWithFlags(e, ctx->stream, cudaEventRecordExternal)
                         : cudaEventRecord(e, ctx->stream);
      };
      auto enqueue = [&](bool capturing) -> int {
        if (!masks_host) {
          CK(launch_counter_masks(sd.n, sd.nA, W, ctx->o.seed, ctx->d_uset.as<int32_t>(),
                                  ctx->d_uperm.as<int32_t>(), ctx->d_mask0.as<uint64_t>(),
                                  ctx->d_masks.as<uint64_t>(), Bt, ctx->stream));
          ctx->launches++;
        }
        CK(record(ctx->ev[0], capturing));
        {
          int rc = launch_pairs_any(ctx, sd, bd.masks, Bt, ctx->d_dmask.as<uint32_t>(), bd.stats,
                                    popc_batch);
          if (rc) return rc;
        }
        CK(record(ctx->ev[1], capturing));
        CK(launch_units(sd, bd, ctx->stream));
        CK(record(ctx->ev[2], capturing));
        ctx->launches += 2;  // networks, then normalisation and JS
        return EDDY_OK;
      };
      ctx->dmask_clean = nullptr;  // until the batch is seen to finish
      if (graphable) {
        {
          int rc = prepare_pairs(ctx, layout_of(sd, pick_variant(ctx, sd, Bt)), Bt);
          if (rc) return rc;
        }
        // everything a replay bakes in: the set, its state, the batch shape
        // and every buffer address
        std::vector<uintptr_t> key = {
            (uintptr_t)sr.set_id, (uintptr_t)ctx->prep_gen, (uintptr_t)sd.salt,
            (uintptr_t)sd.exact_all, (uintptr_t)sd.core, (uintptr_t)Bt, (uintptr_t)kmax_run, (uintptr_t)ub,
            (uintptr_t)pick_variant(ctx, sd, Bt), (uintptr_t)ctx->o.seed,
            (uintptr_t)ctx->d_masks.p, (uintptr_t)ctx->d_dmask.p, (uintptr_t)ctx->d_scratch.p,
            (uintptr_t)ctx->d_js.p, (uintptr_t)ctx->d_U.p, (uintptr_t)ctx->d_status.p,
            (uintptr_t)ctx->d_keep.p, (uintptr_t)ctx->d_uset.p, (uintptr_t)ctx->d_uperm.p,
            (uintptr_t)ctx->d_stats.p, (uintptr_t)ctx->d_afp8.p, (uintptr_t)ctx->d_Y.p,
            (uintptr_t)ctx->d_err.p, (uintptr_t)ctx->d_mask0.p, (uintptr_t)ctx->stream};
        const bool replay = ctx->graph_exec && key == ctx->graph_key;
        if (!replay && key != ctx->direct_key) {
          // first batch of this shape: direct launches, remembered
          ctx->direct_key = key;
          int rc = enqueue(false);
          if (rc) return rc;
        } else {
          if (!replay) {
            if (ctx->graph_exec) {
              cudaGraphExecDestroy(ctx->graph_exec);
              ctx->graph_exec = nullptr;
            }
            ctx->graph_key.clear();
            const long long l0 = ctx->launches;
            CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            const int rc = enqueue(true);
            cudaGraph_t graph = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
            if (rc) {
              if (graph) cudaGraphDestroy(graph);
              return rc;
            }
            CK(ce);
            const cudaError_t ie = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
            cudaGraphDestroy(graph);
            CK(ie);
            ctx->graph_key = key;
            ctx->graph_launches = ctx->launches - l0;
            ctx->launches = l0;
          }
          CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
          ctx->launches += ctx->graph_launches;
        }
      } else {
        int rc = enqueue(false);
        if (rc) return rc;
      }
      // results (and the tensor-core kernel's timeout word) through the
      // pinned staging: JS, U, status, error word
      double *hjs = ctx->h_stage.as<double>();
      int32_t *hU = ctx->h_stage.as<int32_t>(8 * (size_t)Bt);
      uint32_t *hst = ctx->h_stage.as<uint32_t>(12 * (size_t)Bt);
      unsigned *herr = ctx->h_stage.as<unsigned>(16 * (size_t)Bt);
      *herr = 0;
      CK(cudaMemcpyAsync(hjs, ctx->d_js.p, 8 * Bt, cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaMemcpyAsync(hU, ctx->d_U.p, 4 * Bt, cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaMemcpyAsync(hst, ctx->d_status.p, 4 * Bt, cudaMemcpyDeviceToHost, ctx->stream));
      const bool mma_used = !use_popc(sd) && !popc_batch && ctx->d_err.p != nullptr && c > 0;
      if (mma_used)
        CK(cudaMemcpyAsync(herr, ctx->d_err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
      const unsigned errw = *herr;
      std::vector<double> jsb(hjs, hjs + Bt);
      std::vector<int32_t> Ub(hU, hU + Bt);
      status.assign(hst, hst + Bt);
      if (errw & 1u) return fail(ctx, EDDY_ERR_INTERNAL, "tensor-core pipeline wait timed out");
      ctx->dmask_clean = ctx->d_dmask.p;  // the unit kernel cleared every bit set
      if (errw & 2u) {
        // the general-path queue overflowed (a large share of tables near a
        // threshold): decide this batch with the popcount kernel
        popc_batch = true;
        continue;
      }
      float a = 0, bms = 0;
      cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);
      cudaEventElapsedTime(&bms, ctx->ev[1], ctx->ev[2]);
      t_pairs += a;
      t_units += bms;
      std::vector<int> again;
      bool overflow = false, collision = false;
      int need = 0;  // most changed nodes of a network in an overflowed unit
      for (int i = 0; i < Bt; i++) {
        const int u = b0 + todo[i];
        if (status[i] & kUnitKmaxOverflow) {
          overflow = true;
          need = std::max(need, (int)(status[i] >> 16));
          again.push_back(todo[i]);
        } else if (status[i] & kUnitHashCollision) {
          collision = true;
          again.push_back(todo[i]);
        } else {
          js[u] = jsb[i];
          U[u] = Ub[i];
        }
      }
      if (i0 >= 0 && !(status[i0] & (kUnitKmaxOverflow | kUnitHashCollision))) {
        keep->mpk = mpk;
        keep->U = Ub[i0];
        const int Uk = Ub[i0];
        keep->ids.resize(Uk);
        keep->cnt.resize((size_t)Uk * g);
        keep->par.resize((size_t)Uk * g * mpk);
        keep->dist.resize(2 * (size_t)S);
        keep->lval.resize(2 * (size_t)S);
        keep->rows.resize(2 * (size_t)g * sd.GW);
        // through the pinned staging: six asynchronous copies, one wait
        const size_t b_ids = 4 * (size_t)Uk, b_cnt = 4 * (size_t)Uk * g,
                     b_par = 4 * (size_t)Uk * g * mpk, b_dist = 16 * (size_t)S,
                     b_rows = 4 * keep->rows.size();
        const size_t o_cnt = (b_ids + 15) & ~(size_t)15, o_par = o_cnt + ((b_cnt + 15) & ~(size_t)15),
                     o_dist = o_par + ((b_par + 15) & ~(size_t)15), o_lval = o_dist + b_dist,
                     o_rows = o_lval + b_dist;
        CK(ctx->h_stage.ensure(o_rows + b_rows));
        char *hk = ctx->h_stage.as<char>();
        CK(cudaMemcpyAsync(hk, ctx->d_oids.p, b_ids, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(hk + o_cnt, ctx->d_ocnt.p, b_cnt, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(hk + o_par, ctx->d_opar.p, b_par, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(hk + o_dist, ctx->d_odist.p, b_dist, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(hk + o_lval, ctx->d_olval.p, b_dist, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(hk + o_rows, ctx->d_orows.p, b_rows, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        memcpy(keep->ids.data(), hk, b_ids);
        memcpy(keep->cnt.data(), hk + o_cnt, b_cnt);
        memcpy(keep->par.data(), hk + o_par, b_par);
        memcpy(keep->dist.data(), hk + o_dist, b_dist);
        memcpy(keep->lval.data(), hk + o_lval, b_dist);
        memcpy(keep->rows.data(), hk + o_rows, b_rows);
      }
      if (overflow) {
        // the re-run holds every record these units need (their networks do
        // not change); the set's later batches start with a quarter more
        const int want = std::max(need, kmax_run + 1);
        kmax_run = std::min(g + 1, (want + 7) / 8 * 8);
        if (!ek) {
          int &hint = ctx->kmax_hint[g];
          hint = std::max(hint, std::min(g + 1, (want + want / 4 + 7) / 8 * 8));
        }
      }
      if (collision) {
        ctx->salt = ctx->salt * 6364136223846793005ull + 1442695040888963407ull;
        sd.salt = ctx->salt;
      }
      todo.swap(again);
    }
    if (!todo.empty())
      return fail(ctx, EDDY_ERR_INTERNAL, "units of set %d did not converge (status %u)", sr.set_id,
                  status.empty() ? 0u : status[0]);
  }
  ctx->ms_pairs += t_pairs;
  ctx->ms_units += t_units;
  ctx->ms_total += t_pairs + t_units;
  CK(cudaMemcpy(ctx->last_stats, ctx->d_stats.p, sizeof ctx->last_stats, cudaMemcpyDeviceToHost));
  return EDDY_OK;
}

// Capped or uncapped parent lists of a network given by its row bitsets.
void rows_to_lists(const uint32_t *rows, int g, int GW, int cap, std::vector<int32_t> &nodes,
                   std::vector<int32_t> &edges) {
  int run = 0;
  for (int t = 0; t < g; t++) {
    nodes.push_back(run);
    int cnt = 0;
    for (int j = 0; j < t && cnt < cap; j++)
      if ((rows[(size_t)t * GW + (j >> 5)] >> (j & 31)) & 1u) {
        edges.push_back(j);
        cnt++;
      }
    run += cnt;
  }
}

int store_keep(eddy_ctx *ctx, SetHost &S, const KeepOut &K, int g) {
  (void)ctx;
  S.U0 = K.U;
  S.ids.assign(K.ids.begin(), K.ids.end());
  S.nodes.assign((size_t)K.U * g, 0);
  S.epn.assign(K.U + 1, 0);
  S.edges.clear();
  for (int u = 0; u < K.U; u++) {
    int run = 0;
    for (int t = 0; t < g; t++) {
      S.nodes[(size_t)u * g + t] = run;
      const int cnt = K.cnt[(size_t)u * g + t];
      for (int k = 0; k < cnt && k < K.mpk; k++) S.edges.push_back(K.par[((size_t)u * g + t) * K.mpk + k]);
      run += cnt;
    }
    S.epn[u + 1] = S.epn[u] + run;
  }
  const int Sn = (int)K.dist.size() / 2;
  S.lval.assign(2 * (size_t)K.U, 0.0);
  for (int u = 0; u < K.U; u++) {
    S.lval[u] = K.lval[u];
    S.lval[K.U + u] = K.lval[Sn + u];
  }
  // uncapped lists of the two full networks (main.cu:1530-1617)
  const int GW = (g + 31) / 32;
  S.el_nodes.clear();
  S.el_edges.clear();
  std::vector<int32_t> e0, e1;
  rows_to_lists(K.rows.data(), g, GW, 0x7fffffff, S.el_nodes, e0);
  rows_to_lists(K.rows.data() + (size_t)g * GW, g, GW, 0x7fffffff, S.el_nodes, e1);
  S.el_epn = {0, (int32_t)e0.size(), (int32_t)(e0.size() + e1.size())};
  S.el_edges = e0;
  S.el_edges.insert(S.el_edges.end(), e1.begin(), e1.end());
  return EDDY_OK;
}

bool finite_js(double v) { return !isnan(v); }

}  // namespace

// ================================================================= C ABI
extern "C" {

int eddy_ctx_create(const eddy_opts *opts, eddy_ctx **out) {
  if (!opts || !out) return EDDY_ERR_ARG;
  *out = nullptr;
  if (opts->max_parents < 1 || opts->permutations < 1) return EDDY_ERR_ARG;
  if (opts->rng < EDDY_RNG_GLIBC || opts->rng > EDDY_RNG_EXTERNAL) return EDDY_ERR_ARG;
  eddy_ctx *ctx = new eddy_ctx();
  ctx->o = *opts;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || opts->device < 0 || opts->device >= ndev) {
    delete ctx;
    return EDDY_ERR_CUDA;
  }
  if (cudaSetDevice(opts->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return EDDY_ERR_CUDA;
  }
  ctx->stream = ctx->own_stream;
  for (auto &ev : ctx->ev) cudaEventCreate(&ev);
  cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, opts->device);
  *out = ctx;
  return EDDY_OK;
}

int eddy_ctx_destroy(eddy_ctx *ctx) {
  if (!ctx) return EDDY_ERR_ARG;
  cudaSetDevice(ctx->o.device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  DevBuf *bufs[] = {&ctx->d_lg, &ctx->d_vals, &ctx->d_valsT, &ctx->d_planes, &ctx->d_valid, &ctx->d_ctot,
                    &ctx->d_prior, &ctx->d_mask0, &ctx->d_masks, &ctx->d_dmask, &ctx->d_scratch,
                    &ctx->d_js, &ctx->d_U, &ctx->d_status, &ctx->d_keep, &ctx->d_uset,
                    &ctx->d_uperm, &ctx->d_oids, &ctx->d_ocnt, &ctx->d_opar, &ctx->d_odist,
                    &ctx->d_olval, &ctx->d_orows, &ctx->d_stats, &ctx->d_Y, &ctx->d_afp8,
                    &ctx->d_err};
  for (DevBuf *b : bufs) b->release();
  for (auto &ev : ctx->ev)
    if (ev) cudaEventDestroy(ev);
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  ctx->h_stage.release();
  ctx->h_vals.release();
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return EDDY_OK;
}

const char *eddy_last_error(const eddy_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int eddy_load_matrix(eddy_ctx *ctx, const int8_t *data, int genes, int samples,
                     const uint8_t *class_of_sample) {
  if (!ctx) return EDDY_ERR_ARG;
  if (!data || !class_of_sample || genes < 1 || samples < 2)
    return fail(ctx, EDDY_ERR_ARG, "bad matrix shape %d x %d", genes, samples);
  // class sizes and contingency counts are held as 16-bit integers on the GPU
  if (samples > 65535)
    return fail(ctx, EDDY_ERR_CAPACITY, "%d samples (> 65535)", samples);
  int nA = 0, nB = 0;
  for (int s = 0; s < samples; s++) {
    if (class_of_sample[s] == 0) nA++;
    else if (class_of_sample[s] == 1) nB++;
    else return fail(ctx, EDDY_ERR_ARG, "class label of sample %d is neither 0 nor 1", s);
  }
  if (nA == 0 || nB == 0) return fail(ctx, EDDY_ERR_ARG, "labels hold a single class");
  ctx->genes = genes;
  ctx->samples = samples;
  ctx->nA = nA;
  ctx->nB = nB;
  ctx->W = (samples + 63) / 64;
  ctx->data.assign(data, data + (size_t)genes * samples);
  // genes whose every value is -1, 0 or 1 (v + 1 in 0..2 as a byte): a
  // branch-free reduction per gene, which the compiler vectorises
  ctx->gene_full.assign(genes, 1);
  for (int i = 0; i < genes; i++) {
    const uint8_t *row = reinterpret_cast<const uint8_t *>(data) + (size_t)i * samples;
    unsigned bad = 0;
    for (int s = 0; s < samples; s++) bad |= (uint8_t)(row[s] + 1u) > 2u;
    ctx->gene_full[i] = bad ? 0 : 1;
  }
  ctx->labels0.assign(class_of_sample, class_of_sample + samples);
  ctx->prepared_set = -1;
  std::vector<uint64_t> m0(ctx->W);
  labels_to_mask(ctx->labels0.data(), samples, ctx->W, m0.data());
  CK(cudaSetDevice(ctx->o.device));
  CK(ctx->d_mask0.ensure(8 * m0.size()));
  CK(cudaMemcpy(ctx->d_mask0.p, m0.data(), 8 * m0.size(), cudaMemcpyHostToDevice));
  return EDDY_OK;
}

int eddy_add_set(eddy_ctx *ctx, const int32_t *gene_idx, int g, const uint8_t *prior, int *set_id) {
  if (!ctx) return EDDY_ERR_ARG;
  if (ctx->samples == 0) return fail(ctx, EDDY_ERR_STATE, "load the matrix first");
  if (!gene_idx || g < 0) return fail(ctx, EDDY_ERR_ARG, "bad gene set");
  if (g > 512) return fail(ctx, EDDY_ERR_CAPACITY, "gene set of %d genes (> 512)", g);
  SetHost S;
  S.genes.assign(gene_idx, gene_idx + g);
  for (int v : S.genes)
    if (v < 0 || v >= ctx->genes) return fail(ctx, EDDY_ERR_ARG, "gene index %d out of range", v);
  if (prior) S.prior.assign(prior, prior + (size_t)g * g);
  ctx->sets.push_back(std::move(S));
  if (set_id) *set_id = (int)ctx->sets.size() - 1;
  return EDDY_OK;
}

int eddy_set_labellings(eddy_ctx *ctx, int set_id, const uint8_t *labels, int R) {
  if (!ctx) return EDDY_ERR_ARG;
  if (set_id < 0 || set_id >= (int)ctx->sets.size() || !labels || R < 1)
    return fail(ctx, EDDY_ERR_ARG, "bad labellings");
  for (long i = 0; i < (long)R * ctx->samples; i++)
    if (labels[i] > 1) return fail(ctx, EDDY_ERR_ARG, "labels must be 0/1");
  SetHost &S = ctx->sets[set_id];
  S.labels.assign(labels, labels + (size_t)R * ctx->samples);
  S.R_ext = R;
  return EDDY_OK;
}

// Iterations of a set in eddy_run (0: EXTERNAL labellings missing).
static int set_iterations(const eddy_ctx *ctx, const SetHost &S) {
  return ctx->o.rng == EDDY_RNG_EXTERNAL ? std::max(S.R_ext, 0) : ctx->o.permutations;
}

static int run_set(eddy_ctx *ctx, int set_id) {
  SetHost &S = ctx->sets[set_id];
  const int n = ctx->samples, W = ctx->W;
  const int g = (int)S.genes.size();
  const int R = set_iterations(ctx, S);
  if (R < 1) return fail(ctx, EDDY_ERR_STATE, "set %d has no labellings", set_id);
  S.js.assign(R, NAN);
  S.U.assign(R, 0);
  S.iterations = 0;
  S.failed = 0;
  S.betafit_ok = 0;
  S.exact = S.tables = 0;
  if (g < 2) {
    // no pair: every network is empty, U = 1, JS is NaN (main.cu:1431)
    S.js[0] = NAN;
    S.U[0] = 1;
    S.iterations = 1;
    S.failed = 1;
    S.U0 = 1;
    if (ctx->o.rng == EDDY_RNG_GLIBC) {
      std::vector<uint8_t> lab(ctx->labels0);
      glibc_permutation(ctx->rng, n, ctx->nA, false, lab.data(), ctx->seen, ctx->order);
    }
    S.done = true;
    return EDDY_OK;
  }
  SetRun sr;
  int rc = prepare_set(ctx, set_id, sr);
  if (rc) return rc;
  const int mpk0 = std::min(ctx->o.max_parents, std::max(g - 1, 1));
  if (ctx->o.rng == EDDY_RNG_COUNTER && n <= 4096) {
    // counter stream: iteration 0 (the unpermuted labelling, kept) and the
    // permutations in one pass, labellings generated on the device.  A
    // non-finite JS at iteration 0 ends the set there (main.cu:1431-1435):
    // the permutations' results are then discarded.
    std::vector<int32_t> perms(R);
    for (int i = 0; i < R; i++) perms[i] = i;
    KeepOut K;
    rc = run_units(ctx, sr, R, nullptr, perms.data(), S.js.data(), S.U.data(),
                   ctx->o.keep_networks ? &K : nullptr, mpk0);
    if (rc) return rc;
    if (ctx->o.keep_networks) store_keep(ctx, S, K, g);
    else S.U0 = S.U[0];
    if (!finite_js(S.js[0])) {
      for (int i = 1; i < R; i++) {
        S.js[i] = NAN;
        S.U[i] = 0;
      }
      S.iterations = 1;
      S.failed = 1;
      S.done = true;
      return EDDY_OK;
    }
    S.iterations = R;
  } else {
    // iteration 0 (kept: networks and likelihoods for the output files)
    std::vector<uint64_t> masks((size_t)W);
    std::vector<uint8_t> lab(ctx->labels0);
    if (ctx->o.rng == EDDY_RNG_EXTERNAL) lab.assign(S.labels.begin(), S.labels.begin() + n);
    if (ctx->o.rng == EDDY_RNG_GLIBC)
      glibc_permutation(ctx->rng, n, ctx->nA, false, lab.data(), ctx->seen, ctx->order);
    labels_to_mask(lab.data(), n, W, masks.data());
    KeepOut K;
    rc = run_units(ctx, sr, 1, masks.data(), nullptr, S.js.data(), S.U.data(),
                   ctx->o.keep_networks ? &K : nullptr, mpk0);
    if (rc) return rc;
    if (ctx->o.keep_networks) store_keep(ctx, S, K, g);
    else S.U0 = S.U[0];
    S.iterations = 1;
    if (!finite_js(S.js[0])) {
      S.failed = 1;
      S.done = true;
      return EDDY_OK;  // main.cu:1431-1435: break after iteration 0
    }
    if (R > 1) {
      const int nu = R - 1;
      std::vector<int32_t> perms(nu);
      for (int i = 0; i < nu; i++) perms[i] = i + 1;
      const bool device_counter = ctx->o.rng == EDDY_RNG_COUNTER && n <= 4096;
      std::vector<uint64_t> mh;
      if (!device_counter) {
        mh.assign((size_t)nu * W, 0);
        std::vector<uint8_t> cur(ctx->labels0);
        for (int i = 0; i < nu; i++) {
          if (ctx->o.rng == EDDY_RNG_GLIBC) {
            glibc_permutation(ctx->rng, n, ctx->nA, true, cur.data(), ctx->seen, ctx->order);
          } else if (ctx->o.rng == EDDY_RNG_COUNTER) {
            counter_labels(ctx->o.seed, set_id, i + 1, n, ctx->nA, cur.data());
          } else {
            memcpy(cur.data(), S.labels.data() + (size_t)(i + 1) * n, n);
            int a = 0;
            for (int s = 0; s < n; s++) a += cur[s] == 0;
            if (a != ctx->nA) return fail(ctx, EDDY_ERR_ARG, "labelling %d changes the class sizes", i + 1);
          }
          labels_to_mask(cur.data(), n, W, mh.data() + (size_t)i * W);
        }
      }
      rc = run_units(ctx, sr, nu, device_counter ? nullptr : mh.data(), perms.data(), S.js.data() + 1,
                     S.U.data() + 1, nullptr, 1);
      if (rc) return rc;
    }
    S.iterations = R;
  }
  unsigned long long st[4];
  CK(cudaMemcpy(st, ctx->d_stats.p, sizeof st, cudaMemcpyDeviceToHost));
  S.exact += st[0];
  S.tables += st[1];
  for (int i = 0; i < R; i++)
    if (!finite_js(S.js[i])) S.failed = 1;
  // beta fit on the host: the sequential FP64 moment loop and the continued
  // fraction are chains of dependent FP64 operations, which run faster on
  // the host cores than on the GPU
  if (!S.failed) S.betafit_ok = beta_pddn(S.js.data(), R, S.alpha, S.beta, S.pddn) ? 1 : 0;
  S.done = true;
  return EDDY_OK;
}

int eddy_run(eddy_ctx *ctx) {
  if (!ctx) return EDDY_ERR_ARG;
  if (ctx->samples == 0) return fail(ctx, EDDY_ERR_STATE, "no matrix loaded");
  ctx->ms_total = ctx->ms_pairs = ctx->ms_units = 0;
  ctx->launches = 0;
  for (int s = 0; s < (int)ctx->sets.size(); s++) {
    if (ctx->sets[s].done) continue;
    int rc = run_set(ctx, s);
    if (rc) return rc;
  }
  return EDDY_OK;
}

int eddy_get_set_summary(const eddy_ctx *ctx, int set_id, eddy_set_summary *out) {
  if (!ctx || !out || set_id < 0 || set_id >= (int)ctx->sets.size()) return EDDY_ERR_ARG;
  const SetHost &S = ctx->sets[set_id];
  if (!S.done) return EDDY_ERR_STATE;
  out->genes = (int)S.genes.size();
  out->iterations = S.iterations;
  out->failed = S.failed;
  out->betafit_ok = S.betafit_ok;
  out->unique0 = S.U0;
  out->js0 = S.js.empty() ? NAN : S.js[0];
  out->alpha = S.alpha;
  out->beta = S.beta;
  out->pddn = S.pddn;
  out->exact_rechecks = S.exact;
  out->tables = S.tables;
  return EDDY_OK;
}

int eddy_get_js(const eddy_ctx *ctx, int set_id, double *js, int32_t *unique) {
  if (!ctx || set_id < 0 || set_id >= (int)ctx->sets.size()) return EDDY_ERR_ARG;
  const SetHost &S = ctx->sets[set_id];
  if (!S.done) return EDDY_ERR_STATE;
  for (int i = 0; i < S.iterations; i++) {
    if (js) js[i] = S.js[i];
    if (unique) unique[i] = S.U[i];
  }
  return EDDY_OK;
}

int eddy_get_networks(const eddy_ctx *ctx, int set_id, int *U, int *edges, int32_t *ids,
                      int32_t *nodes, int32_t *epn, int32_t *edges_out, double *lval) {
  if (!ctx || set_id < 0 || set_id >= (int)ctx->sets.size()) return EDDY_ERR_ARG;
  const SetHost &S = ctx->sets[set_id];
  if (!S.done || S.ids.empty()) return EDDY_ERR_STATE;
  if (U) *U = S.U0;
  if (edges) *edges = (int)S.edges.size();
  if (ids) memcpy(ids, S.ids.data(), 4 * S.ids.size());
  if (nodes) memcpy(nodes, S.nodes.data(), 4 * S.nodes.size());
  if (epn) memcpy(epn, S.epn.data(), 4 * S.epn.size());
  if (edges_out) memcpy(edges_out, S.edges.data(), 4 * S.edges.size());
  if (lval) memcpy(lval, S.lval.data(), 8 * S.lval.size());
  return EDDY_OK;
}

int eddy_get_edge_list(const eddy_ctx *ctx, int set_id, int *edges, int32_t *nodes, int32_t *epn,
                       int32_t *edges_out) {
  if (!ctx || set_id < 0 || set_id >= (int)ctx->sets.size()) return EDDY_ERR_ARG;
  const SetHost &S = ctx->sets[set_id];
  if (!S.done || S.el_nodes.empty()) return EDDY_ERR_STATE;
  if (edges) *edges = (int)S.el_edges.size();
  if (nodes) memcpy(nodes, S.el_nodes.data(), 4 * S.el_nodes.size());
  if (epn) memcpy(epn, S.el_epn.data(), 4 * S.el_epn.size());
  if (edges_out) memcpy(edges_out, S.el_edges.data(), 4 * S.el_edges.size());
  return EDDY_OK;
}

int eddy_run_labellings(eddy_ctx *ctx, int set_id, const uint8_t *labels, int R, double *js,
                        int32_t *unique) {
  if (!ctx) return EDDY_ERR_ARG;
  if (set_id < 0 || set_id >= (int)ctx->sets.size() || !labels || R < 1 || !js || !unique)
    return fail(ctx, EDDY_ERR_ARG, "bad arguments");
  const int n = ctx->samples, W = ctx->W;
  for (int r = 0; r < R; r++) {
    int a = 0;
    for (int s = 0; s < n; s++) a += labels[(size_t)r * n + s] == 0;
    if (a != ctx->nA) return fail(ctx, EDDY_ERR_ARG, "labelling %d has %d class-0 samples, expected %d", r, a, ctx->nA);
  }
  ctx->ms_total = ctx->ms_pairs = ctx->ms_units = 0;
  ctx->launches = 0;
  SetRun sr;
  int rc = prepare_set(ctx, set_id, sr);
  if (rc) return rc;
  std::vector<uint64_t> mh((size_t)R * W);
  for (int r = 0; r < R; r++) labels_to_mask(labels + (size_t)r * n, n, W, mh.data() + (size_t)r * W);
  return run_units(ctx, sr, R, mh.data(), nullptr, js, unique, nullptr, 1);
}

int eddy_debug_edges(eddy_ctx *ctx, int set_id, const uint8_t *labels, uint8_t *edges) {
  if (!ctx || !labels || !edges || set_id < 0 || set_id >= (int)ctx->sets.size()) return EDDY_ERR_ARG;
  const int n = ctx->samples, W = ctx->W;
  SetRun sr;
  int rc = prepare_set(ctx, set_id, sr);
  if (rc) return rc;
  const SetDev &sd = sr.sd;
  const int c = sd.c, S = sd.S;
  std::vector<uint64_t> m(W);
  labels_to_mask(labels, n, W, m.data());
  CK(ctx->d_masks.ensure(8 * W));
  rc = dmask_ready(ctx, 1, c);
  if (rc) return rc;
  ctx->dmask_clean = nullptr;  // no unit kernel reads (and clears) these masks
  CK(cudaMemcpyAsync(ctx->d_masks.p, m.data(), 8 * W, cudaMemcpyHostToDevice, ctx->stream));
  rc = launch_pairs_any(ctx, sd, ctx->d_masks.as<uint64_t>(), 1, ctx->d_dmask.as<uint32_t>(), nullptr);
  if (rc) return rc;
  rc = check_mma_error(ctx, sd);
  if (rc) return rc;
  std::vector<uint32_t> dm(c);
  CK(cudaMemcpyAsync(dm.data(), ctx->d_dmask.p, 4 * (size_t)c, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // expand the 10-bit masks to the S networks (kernel1.cu:85-88, 412-416)
  std::vector<int> la, lb;
  for (int s = 0; s < n; s++) (labels[s] == 0 ? la : lb).push_back(s);
  const int g = sd.g;
  auto st = [&](int gene, int smp) {
    int8_t v = ctx->data[(size_t)ctx->sets[set_id].genes[gene] * n + smp];
    return v == -1 ? 0 : v == 0 ? 1 : v == 1 ? 2 : 3;
  };
  for (int s = 0; s < S; s++) {
    int k, sigma;
    if (s == 0) { k = 0; sigma = -1; }
    else if (s == S - 1) { k = 1; sigma = -1; }
    else if (s <= sd.nA) { k = 0; sigma = la[s - 1]; }
    else { k = 1; sigma = lb[s - sd.nA - 1]; }
    int p = 0;
    for (int r = 1; r < g; r++)
      for (int col = 0; col < r; col++, p++) {
        uint32_t mm = (dm[p] >> (16 * k)) & 0x3FFu;
        int bit = mm & 1u;
        if (sigma >= 0) {
          int a = st(r, sigma), b = st(col, sigma);
          if (a <= 2 && b <= 2) bit = (mm >> (1 + 3 * a + b)) & 1u;
        }
        edges[(size_t)s * c + p] = (uint8_t)bit;
      }
  }
  return EDDY_OK;
}

int eddy_debug_unit(eddy_ctx *ctx, int set_id, const uint8_t *labels, int mpk, int *U, double *js,
                    int32_t *ids, int32_t *counts, int32_t *parents, double *dist, double *lval) {
  if (!ctx || !labels || set_id < 0 || set_id >= (int)ctx->sets.size() || mpk < 1) return EDDY_ERR_ARG;
  const int n = ctx->samples, W = ctx->W;
  SetRun sr;
  int rc = prepare_set(ctx, set_id, sr);
  if (rc) return rc;
  std::vector<uint64_t> m(W);
  labels_to_mask(labels, n, W, m.data());
  KeepOut K;
  double j = 0;
  int32_t u = 0;
  rc = run_units(ctx, sr, 1, m.data(), nullptr, &j, &u, &K, mpk);
  if (rc) return rc;
  const int g = sr.sd.g, S = sr.sd.S;
  if (U) *U = K.U;
  if (js) *js = j;
  for (int i = 0; i < K.U; i++) {
    if (ids) ids[i] = K.ids[i];
    for (int t = 0; t < g; t++) {
      if (counts) counts[(size_t)i * g + t] = K.cnt[(size_t)i * g + t];
      if (parents)
        for (int q = 0; q < mpk; q++) parents[((size_t)i * g + t) * mpk + q] = K.par[((size_t)i * g + t) * mpk + q];
    }
  }
  if (dist) memcpy(dist, K.dist.data(), 16 * (size_t)S);
  if (lval) memcpy(lval, K.lval.data(), 16 * (size_t)S);
  return EDDY_OK;
}

int eddy_run_permutations(eddy_ctx *ctx, int set_id, int first, int count, double *js,
                          int32_t *unique) {
  if (!ctx) return EDDY_ERR_ARG;
  if (set_id < 0 || set_id >= (int)ctx->sets.size() || first < 0 || count < 1 || !js || !unique)
    return fail(ctx, EDDY_ERR_ARG, "bad arguments");
  if (ctx->o.rng == EDDY_RNG_GLIBC)
    return fail(ctx, EDDY_ERR_STATE, "the GLIBC stream is sequential: use eddy_run");
  SetHost &S = ctx->sets[set_id];
  const int n = ctx->samples, W = ctx->W;
  ctx->ms_total = ctx->ms_pairs = ctx->ms_units = 0;
  ctx->launches = 0;
  if (S.genes.size() < 2) {
    for (int i = 0; i < count; i++) {
      js[i] = NAN;
      unique[i] = 1;
    }
    return EDDY_OK;
  }
  SetRun sr;
  int rc = prepare_set(ctx, set_id, sr);
  if (rc) return rc;
  std::vector<int32_t> perms(count);
  for (int i = 0; i < count; i++) perms[i] = first + i;
  if (ctx->o.rng == EDDY_RNG_COUNTER && n <= 4096)
    return run_units(ctx, sr, count, nullptr, perms.data(), js, unique, nullptr, 1);
  std::vector<uint64_t> mh((size_t)count * W);
  std::vector<uint8_t> cur(n);
  for (int i = 0; i < count; i++) {
    const int it = first + i;
    if (ctx->o.rng == EDDY_RNG_COUNTER) {
      if (it == 0) memcpy(cur.data(), ctx->labels0.data(), n);
      else counter_labels(ctx->o.seed, set_id, it, n, ctx->nA, cur.data());
    } else {
      if (it >= S.R_ext) return fail(ctx, EDDY_ERR_ARG, "iteration %d has no labelling", it);
      memcpy(cur.data(), S.labels.data() + (size_t)it * n, n);
    }
    labels_to_mask(cur.data(), n, W, mh.data() + (size_t)i * W);
  }
  return run_units(ctx, sr, count, mh.data(), nullptr, js, unique, nullptr, 1);
}

int eddy_set_stream(eddy_ctx *ctx, void *stream) {
  if (!ctx) return EDDY_ERR_ARG;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->own_stream;
  if (st != ctx->stream) CK(cudaStreamSynchronize(ctx->stream));
  ctx->stream = st;
  return EDDY_OK;
}

int eddy_clear_sets(eddy_ctx *ctx) {
  if (!ctx) return EDDY_ERR_ARG;
  ctx->sets.clear();
  ctx->prepared_set = -1;
  return EDDY_OK;
}

int eddy_device_info(int device, char *name, int name_len, int *sms, int *cc_major,
                     int *cc_minor) {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return EDDY_ERR_CUDA;
  if (name && name_len > 0) {
    strncpy(name, p.name, name_len - 1);
    name[name_len - 1] = 0;
  }
  if (sms) *sms = p.multiProcessorCount;
  if (cc_major) *cc_major = p.major;
  if (cc_minor) *cc_minor = p.minor;
  return EDDY_OK;
}

int eddy_last_stats(const eddy_ctx *ctx, uint64_t *stats4, int *variant) {
  if (!ctx || !stats4) return EDDY_ERR_ARG;
  for (int i = 0; i < 4; i++) stats4[i] = ctx->last_stats[i];
  if (variant) *variant = ctx->tuned_variant;
  return EDDY_OK;
}

int eddy_last_timing(const eddy_ctx *ctx, double *ms_kernels, double *ms_pairs, double *ms_units,
                     long long *launches) {
  if (!ctx) return EDDY_ERR_ARG;
  if (ms_kernels) *ms_kernels = ctx->ms_total;
  if (ms_pairs) *ms_pairs = ctx->ms_pairs;
  if (ms_units) *ms_units = ctx->ms_units;
  if (launches) *launches = ctx->launches;
  return EDDY_OK;
}

}  // extern "C"
