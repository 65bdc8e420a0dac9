// eddy_api.cu -- the C ABI of libeddy_gpu (include/eddy_gpu.h): context,
// gene sets, the permutation driver (main.cu:538-1502) and device buffers.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <condition_variable>
#include <map>
#include <mutex>
#include <string>
#include <thread>
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
  bool it0 = false;  // iteration 0 already run (JS, U, kept outputs), by the batched pass
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
  // batch boundaries: 0 before the decisions, 4 after the contraction, 1
  // after the decisions, 5 after the networks, 2 after the JS; 2 and 3 also
  // time the autotuner's choices
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  GlibcRand rng{1};
  std::vector<uint8_t> seen;
  std::vector<int> order;
  // device data: the fixed-point lgamma table, the resident sets' inputs
  // (one arena), the unpermuted labelling's mask; per batch: masks,
  // decisions, per-unit scratch, results, the set table and unit slots
  DevBuf d_lg, d_setdata, d_mask0;
  DevBuf d_masks, d_dmask, d_scratch, d_js, d_U, d_status, d_keep, d_uset, d_uperm;
  DevBuf d_uslot, d_sets;
  DevBuf d_oids, d_ocnt, d_opar, d_odist, d_olval, d_orows, d_stats;
  DevBuf d_Y, d_afp8, d_err;  // tensor-core contingency operands
  // d_dmask is all zero between batches (decisions only set bits, the unit
  // kernel clears what it reads) while this equals d_dmask.p; null = unknown
  void *dmask_clean = nullptr;
  PinnedBuf h_stage;          // per-batch uploads: unit sets, permutations, slots, set table
  PinnedBuf h_res;            // per-batch results
  PinnedBuf h_vals;           // the resident sets' values and prior bits on their way in
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
  // the same split by kernel: operands + contraction, general + exact
  // decisions, networks, normalisation + JS
  double ms_stage[4] = {0, 0, 0, 0};
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
  // the resident sets in slot order (their inputs are in d_setdata) and
  // their descriptors; the Y arena built for them in layout y_core, with
  // each slot's first column group and first gene
  std::vector<int> res_ids;
  std::vector<SetDev> res_sd;
  bool y_ready = false;
  int y_core = -1;
  std::vector<int> y_grp0, y_gc0;
  YArena y{};
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

// Shape of a set as the decision kernels see it (no device data): genes,
// pairs and whether every value is -1/0/1 (the 4-cell tensor-core layout
// needs that; EDDY_PAIR_LAYOUT=full keeps the 9-cell layout).
struct Shape {
  int g, c, core;
};
Shape shape_of(const eddy_ctx *ctx, int set_id) {
  const SetHost &S = ctx->sets[set_id];
  Shape sh;
  sh.g = (int)S.genes.size();
  sh.c = sh.g * (sh.g - 1) / 2;
  const char *pl = getenv("EDDY_PAIR_LAYOUT");
  bool full = true;
  for (int v : S.genes) full = full && ctx->gene_full[v];
  sh.core = (full && !(pl && strcmp(pl, "full") == 0)) ? 1 : 0;
  return sh;
}

// The fixed-point lgamma table and divisor map of the sample count.
int ensure_lg(eddy_ctx *ctx) {
  const int n = ctx->samples;
  if (ctx->lg_ready && ctx->lg_n == n) return EDDY_OK;
  std::vector<int64_t> lg;
  int8_t dmap[82];
  bdeu_table(n, lg, ctx->lg_shift, dmap);
  CK(ctx->d_lg.ensure(lg.size() * sizeof(int64_t)));
  CK(cudaMemcpy(ctx->d_lg.p, lg.data(), lg.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
  CK(set_divisor_map(dmap));
  ctx->lg_ready = true;
  ctx->lg_n = n;
  return EDDY_OK;
}

// Makes the sets `ids` resident, in this slot order: their values (gene
// rows gathered from the matrix), prior bits, state planes, sample-major
// values and full-sample tables in one device arena, laid out array by
// array (all sets' values, then all prior bits, ...), so that the host
// staging goes up in two copies.  The arena is rebuilt only when the list
// changes; the descriptors are re-derived every call (they also carry the
// run's switches).
int prepare_sets(eddy_ctx *ctx, const std::vector<int> &ids) {
  const int n = ctx->samples, W = ctx->W, ns = (int)ids.size();
  CK(cudaSetDevice(ctx->o.device));
  {
    int rc = ensure_lg(ctx);
    if (rc) return rc;
  }
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  std::vector<size_t> ov(ns), opr(ns), ovt(ns), opl(ns), ova(ns), oct(ns);
  size_t o = 0;
  for (int k = 0; k < ns; k++) {
    const int g = (int)ctx->sets[ids[k]].genes.size();
    if (g > 512) return fail(ctx, EDDY_ERR_CAPACITY, "gene set %d has %d genes (> 512)", ids[k], g);
    ov[k] = o;
    o += (size_t)g * n;
  }
  const size_t vals_bytes = o;
  o = al(o);
  const size_t pr0 = o;
  for (int k = 0; k < ns; k++) {
    const int g = (int)ctx->sets[ids[k]].genes.size(), c = g * (g - 1) / 2;
    opr[k] = o;
    o += (size_t)(c > 0 ? c : 1);
  }
  const size_t prior_bytes = o - pr0;
  for (int k = 0; k < ns; k++) {
    const int g = (int)ctx->sets[ids[k]].genes.size(), c = g * (g - 1) / 2;
    o = al(o);
    ovt[k] = o;
    o += (size_t)st_stride(g) * n + 16;
    o = al(o);
    opl[k] = o;  // planes, then their word-major copy
    o += 2 * sizeof(uint64_t) * (size_t)g * 3 * W;
    o = al(o);
    ova[k] = o;
    o += sizeof(uint64_t) * W;
    o = al(o);
    oct[k] = o;
    o += sizeof(uint16_t) * 9 * (size_t)(c > 0 ? c : 1);
  }
  const size_t total = al(o);
  if (ids != ctx->res_ids) {
    ctx->res_ids.clear();
    ctx->y_ready = false;
    // (the previous batch's copies out of the staging finished at its
    // synchronisation)
    CK(ctx->h_vals.ensure(al(vals_bytes) + prior_bytes + 16));
    int8_t *hv = ctx->h_vals.as<int8_t>();
    uint8_t *hp = ctx->h_vals.as<uint8_t>(al(vals_bytes));
    for (int k = 0; k < ns; k++) {
      const SetHost &S = ctx->sets[ids[k]];
      const int g = (int)S.genes.size();
      for (int i = 0; i < g; i++)
        memcpy(hv + ov[k] + (size_t)i * n, ctx->data.data() + (size_t)S.genes[i] * n, n);
      uint8_t *pb = hp + (opr[k] - pr0);
      const int c = g * (g - 1) / 2;
      memset(pb, 0, (size_t)(c > 0 ? c : 1));
      if (!S.prior.empty()) {
        int p = 0;
        for (int r = 1; r < g; r++)
          for (int col = 0; col < r; col++, p++) pb[p] = S.prior[(size_t)r * g + col] == 1 ? 1 : 0;
      }
    }
    CK(ctx->d_setdata.ensure(total));
    uint8_t *db = ctx->d_setdata.as<uint8_t>();
    CK(cudaMemcpyAsync(db, hv, vals_bytes, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(db + pr0, hp, prior_bytes, cudaMemcpyHostToDevice, ctx->stream));
    for (int k = 0; k < ns; k++) {
      const int g = (int)ctx->sets[ids[k]].genes.size(), c = g * (g - 1) / 2;
      CK(launch_prep((const int8_t *)(db + ov[k]), g, n, W, c, (uint64_t *)(db + opl[k]),
                     (uint64_t *)(db + ova[k]), (uint16_t *)(db + oct[k]), (int8_t *)(db + ovt[k]),
                     ctx->stream));
      ctx->launches += 2 + (c > 0);
    }
    ctx->res_ids = ids;
    ctx->prep_gen++;
  }
  // descriptors
  const char *dm = getenv("EDDY_DECISIONS");
  const bool fp64 = dm && strcmp(dm, "fp64") == 0;
  uint8_t *db = ctx->d_setdata.as<uint8_t>();
  ctx->res_sd.assign(ns, SetDev{});
  for (int k = 0; k < ns; k++) {
    const Shape sh = shape_of(ctx, ids[k]);
    SetDev &sd = ctx->res_sd[k];
    sd.g = sh.g;
    sd.n = n;
    sd.W = W;
    sd.c = sh.c;
    sd.nA = ctx->nA;
    sd.nB = ctx->nB;
    sd.S = n + 2;
    sd.mp = ctx->o.max_parents;
    sd.GW = (sh.g + 31) / 32;
    sd.bonf = ctx->o.bonferroni ? 1 : 0;
    sd.alpha_edge = ctx->o.alpha_edge;
    sd.alpha_edge_prior = ctx->o.alpha_edge_prior;
    auto it = ctx->thr_cache.find(sh.g);
    if (it == ctx->thr_cache.end()) {
      eddy_ctx::ThrSet ts;
      ts.exact_all = compute_thresholds(sd.alpha_edge, sd.alpha_edge_prior, sh.g, sd.bonf, ts.t);
      it = ctx->thr_cache.emplace(sh.g, ts).first;
    }
    memcpy(sd.thr, it->second.t, sizeof sd.thr);
    // EDDY_DECISIONS=fp64: the plain FP64 form -- every table of every pair
    // evaluated with the reference's FP64 formula, no FP32 fast path, no
    // leave-one-out filter (the comparator of the batched FP32 form)
    sd.exact_all = (it->second.exact_all || fp64) ? 1 : 0;
    sd.core = sh.core;
    sd.planes = (const uint64_t *)(db + opl[k]);
    sd.planesT = sd.planes + (size_t)sh.g * 3 * W;
    sd.valid = (const uint64_t *)(db + ova[k]);
    sd.vals = (const int8_t *)(db + ov[k]);
    sd.valsT = (const int8_t *)(db + ovt[k]);
    sd.ctot = (const uint16_t *)(db + oct[k]);
    sd.prior = (const uint8_t *)(db + opr[k]);
    sd.lg = ctx->d_lg.as<int64_t>();
    sd.lg_stride = n + 1;
    sd.lg_shift = ctx->lg_shift;
    sd.salt = ctx->salt;
  }
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
int choices(const Shape &sh, int *v) {
  const int nv = mma_variants();
  int k = 0;
  if (sh.core && sh.c >= kCoreMinPairs) {
    v[k++] = nv + 4;
    v[k++] = nv + 2;
  }
  for (int i = nv - 1; i >= 0; i--) v[k++] = i;
  return k;
}
// autotuning key: samples, the power of two of the pair count (sets of
// similar size share a choice) and whether the 4-cell layout is on offer
// (a set with missing values must never take a choice tuned without them)
std::pair<int, int> tune_key(int n, const Shape &sh) {
  int lc = 0;
  while ((1 << lc) < sh.c) lc++;
  return {n, 2 * lc + (sh.core && sh.c >= kCoreMinPairs ? 1 : 0)};
}
bool layout_core(int v) { return v >= mma_variants(); }

// Choice for a batch of B units: the tile shape pinned by EDDY_MMA_VARIANT
// (in the sets' own layout), the one tuned for their shape, or -1 when this
// batch is to tune (B >= 512).
int pick_variant(eddy_ctx *ctx, const Shape &sh, int B) {
  const int nv = mma_variants();
  const char *ev = getenv("EDDY_MMA_VARIANT");
  if (ev) return (sh.core ? nv : 0) + atoi(ev) % nv;
  auto it = ctx->tuned.find(tune_key(ctx->samples, sh));
  if (it != ctx->tuned.end()) return it->second;
  if (B >= 512) return -1;
  // untuned small batch: what measured fastest on sets of 39 and of 200
  // genes (4-cell layout from kCoreMinPairs pairs: N = 192 with 12 epilogue
  // warps; else the 9-cell layout: N = 256 with 8)
  if (sh.core && sh.c >= kCoreMinPairs) return nv + 2 % nv;
  return 3 % nv;
}

// The resident sets' Y arena in a layout (built once per resident list and
// layout): each slot's column groups from its grp0, its genes from its gc0.
int prepare_y(eddy_ctx *ctx, bool core) {
  if (ctx->y_ready && ctx->y_core == (core ? 1 : 0)) return EDDY_OK;
  const int ns = (int)ctx->res_sd.size();
  ctx->y_grp0.assign(ns, 0);
  ctx->y_gc0.assign(ns, 0);
  int G = 0, genes = 0;
  for (int k = 0; k < ns; k++) {
    ctx->y_grp0[k] = G;
    ctx->y_gc0[k] = genes;
    G += mma_ngroups_pad(ctx->res_sd[k], core);
    genes += ctx->res_sd[k].g;
  }
  CK(ctx->d_Y.ensure(mma_y_bytes(G, genes, ctx->samples)));
  ctx->y = YArena{ctx->d_Y.as<uint8_t>(), G, genes, ctx->samples};
  for (int k = 0; k < ns; k++) {
    if (ctx->res_sd[k].c == 0) continue;
    CK(launch_build_y(ctx->res_sd[k], core, ctx->y, ctx->y_grp0[k], ctx->y_gc0[k], ctx->stream));
    ctx->launches += mma_build_launches(ctx->res_sd[k]);
  }
  ctx->y_ready = true;
  ctx->y_core = core ? 1 : 0;
  return EDDY_OK;
}

// A decision buffer of `bytes` that holds only zeros: cleared in full
// after an allocation or a batch that did not finish.
int dmask_ready(eddy_ctx *ctx, size_t bytes) {
  const void *p0 = ctx->d_dmask.p;
  const size_t n0 = ctx->d_dmask.n;
  CK(ctx->d_dmask.ensure(bytes));
  // a new allocation can start at the freed one's address: any change of
  // the buffer means unknown contents
  if (ctx->d_dmask.p != p0 || ctx->d_dmask.n != n0) ctx->dmask_clean = nullptr;
  if (ctx->dmask_clean != ctx->d_dmask.p) {
    CK(cudaMemsetAsync(ctx->d_dmask.p, 0, ctx->d_dmask.n, ctx->stream));
    ctx->dmask_clean = ctx->d_dmask.p;
  }
  return EDDY_OK;
}

// A batch as the decision kernels see it: the host copy of its set table
// (device descriptors, unit ranges and slices filled in), each unit's slot,
// and the table's device copy.
struct BatchPlan {
  std::vector<BatchSet> sets;
  int B = 0, gmax = 0, cmax = 0;
  bool fp64 = false;  // every set decides in FP64 (the popcount path)
};

// The set table in layout `core` for tile shape `variant`: each slot's
// column groups and the contingency plan.
MmaPlan plan_mma(eddy_ctx *ctx, BatchPlan &bp, int variant) {
  const bool core = layout_core(variant);
  for (size_t k = 0; k < bp.sets.size(); k++) {
    bp.sets[k].grp0 = ctx->y_grp0[k];
    bp.sets[k].gc0 = ctx->y_gc0[k];
    bp.sets[k].sd.core = core ? 1 : 0;
  }
  return mma_plan(bp.sets.data(), (int)bp.sets.size(), variant, core);
}

// Uploads the set table through the pinned staging at byte offset `off`.
int upload_table(eddy_ctx *ctx, const BatchPlan &bp, size_t off) {
  const size_t tb = sizeof(BatchSet) * bp.sets.size();
  CK(ctx->d_sets.ensure(tb));
  memcpy(ctx->h_stage.as<char>(off), bp.sets.data(), tb);
  CK(cudaMemcpyAsync(ctx->d_sets.p, ctx->h_stage.as<char>(off), tb, cudaMemcpyHostToDevice,
                     ctx->stream));
  return EDDY_OK;
}

// Decisions of a batch: the popcount kernel, or the tensor-core path in the
// variant picked (tuning it on this batch when it is the first of its shape
// with >= 512 units: every choice is timed once, same results, the fastest
// kept).  The table is uploaded from the staging at byte offset toff.
// ev_mid, when given, is recorded where the contraction ends and the
// general-path decisions begin (right after the pair kernel on the popcount
// path, which has no separate decision kernels).
int launch_pairs_any(eddy_ctx *ctx, BatchPlan &bp, const uint64_t *masks, uint32_t *dmask,
                     unsigned long long *stats, size_t toff, bool force_popc = false,
                     cudaEvent_t ev_mid = nullptr) {
  auto mark = [&]() -> cudaError_t { return ev_mid ? cudaEventRecord(ev_mid, ctx->stream) : cudaSuccess; };
  if (bp.cmax == 0) {
    int rc = upload_table(ctx, bp, toff);
    if (rc) return rc;
    CK(mark());
    return EDDY_OK;
  }
  const int ns = (int)bp.sets.size();
  if (use_popc() || bp.fp64 || force_popc) {
    {
      int rc = upload_table(ctx, bp, toff);
      if (rc) return rc;
    }
    CK(launch_pairs(ctx->d_sets.as<BatchSet>(), ctx->d_uslot.as<int32_t>(), masks, dmask, bp.B,
                    ctx->W, bp.cmax, stats, ctx->stream));
    CK(mark());
    ctx->launches += 1;
    return EDDY_OK;
  }
  CK(ctx->d_err.ensure(sizeof(unsigned)));
  CK(cudaMemsetAsync(ctx->d_err.p, 0, sizeof(unsigned), ctx->stream));
  Shape sh{bp.sets[0].sd.g, bp.sets[0].sd.c, shape_of(ctx, ctx->res_ids[0]).core};
  int variant = pick_variant(ctx, sh, bp.B);
  const int g_single = ns == 1 ? bp.sets[0].sd.g : 0;
  auto run = [&](int v, unsigned long long *st, cudaEvent_t evm) -> int {
    {
      int rc = prepare_y(ctx, layout_core(v));
      if (rc) return rc;
    }
    const MmaPlan mp = plan_mma(ctx, bp, v);
    CK(ctx->d_afp8.ensure(mma_a_bytes(mp, ctx->samples, layout_core(v))));
    {
      int rc = upload_table(ctx, bp, toff);
      if (rc) return rc;
    }
    CK(launch_pairs_mma(ctx->d_sets.as<BatchSet>(), ns, mp, masks, ctx->d_uslot.as<int32_t>(),
                        ctx->samples, ctx->W, ctx->d_afp8.as<uint8_t>(), ctx->y, dmask, st,
                        ctx->d_err.as<unsigned>(), ctx->sms, ctx->stream, v, layout_core(v),
                        g_single, evm));
    ctx->launches += mma_launches();
    return EDDY_OK;
  };
  if (variant < 0) {
    // autotune on this batch: time every choice once (same results), keep
    // the fastest for this shape; the last run leaves dmask filled
    float best = 1e30f;
    int bi = 0;
    int cand[16];
    const int ncand = choices(sh, cand);
    for (int ci = 0; ci < ncand; ci++) {
      const int v = cand[ci];
      // (the staging slot of the table is rewritten for the next choice
      // only after this one's upload has run)
      if (ci > 0) CK(cudaStreamSynchronize(ctx->stream));
      CK(cudaEventRecord(ctx->ev[2], ctx->stream));
      {
        int rc = run(v, nullptr, nullptr);
        if (rc) return rc;
      }
      CK(cudaEventRecord(ctx->ev[3], ctx->stream));
      CK(cudaEventSynchronize(ctx->ev[3]));
      float ms = 0;
      cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
      ctx->tuned_ms[v] = ms;
      if (ms < best) {
        best = ms;
        bi = v;
      }
    }
    ctx->tuned[tune_key(ctx->samples, sh)] = bi;
    variant = bi;
    CK(cudaStreamSynchronize(ctx->stream));
  }
  ctx->tuned_variant = variant;
  return run(variant, stats, ev_mid);
}

int check_mma_error(eddy_ctx *ctx, const BatchPlan &bp) {
  if (use_popc() || bp.fp64 || ctx->d_err.p == nullptr) return EDDY_OK;
  unsigned e = 0;
  CK(cudaMemcpyAsync(&e, ctx->d_err.p, sizeof e, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (e) return fail(ctx, EDDY_ERR_INTERNAL, "tensor-core pipeline wait timed out");
  return EDDY_OK;
}

// One set's part of a batched run: its units (labellings), given as host
// masks or as permutation indices of the device-generated stream, and
// where their results go.  keep: unit 0's detailed outputs (its networks
// for the output files), or null.
struct Job {
  int set_id = -1;
  int n_units = 0;
  const uint64_t *masks_host = nullptr;  // [n_units][W], or null
  const int32_t *perms = nullptr;        // [n_units] (device labellings)
  double *js = nullptr;
  int32_t *U = nullptr;
  KeepOut *keep = nullptr;
  int mpk = 1;
  unsigned long long exact = 0, tables = 0;  // decision counters of its batches
};
struct UnitRef {
  int job, i;
};

// Runs the units `units` (in job order: a job's units are consecutive) as
// one batch: the sets' data resident, the set table, labellings, decisions,
// networks, normalisation and JS, one synchronisation.  Units whose status
// asks for a re-run go to *again (need: the records they want; collision:
// a hash collision was found); *queue_full: the general-path queue
// overflowed (nothing was stored: the batch must be decided another way).
int run_batch(eddy_ctx *ctx, std::vector<Job> &jobs, const std::vector<UnitRef> &units, int kmax,
              bool popc_batch, std::vector<UnitRef> *again, int *need, bool *collision,
              bool *queue_full, float *t_pairs, float *t_units) {
  const int Bt = (int)units.size(), W = ctx->W, n = ctx->samples, S = n + 2;
  // slots: the jobs of the batch, in order
  std::vector<int> slot_job, ids;
  std::vector<int32_t> uslot(Bt);
  for (int i = 0; i < Bt; i++) {
    if (slot_job.empty() || slot_job.back() != units[i].job) {
      slot_job.push_back(units[i].job);
      ids.push_back(jobs[units[i].job].set_id);
    }
    uslot[i] = (int32_t)slot_job.size() - 1;
  }
  const int ns = (int)slot_job.size();
  {
    int rc = prepare_sets(ctx, ids);
    if (rc) return rc;
  }
  BatchPlan bp;
  bp.B = Bt;
  bp.sets.assign(ns, BatchSet{});
  bp.fp64 = true;
  size_t dmw = 0, scb = 0;
  for (int k = 0, u = 0; k < ns; k++) {
    BatchSet &b = bp.sets[k];
    b.sd = ctx->res_sd[k];
    b.u0 = u;
    int nb = 0;
    while (u < Bt && uslot[u] == k) {
      u++;
      nb++;
    }
    b.nb = nb;
    b.dm0 = (long long)dmw;
    dmw += dmask_words(nb, b.sd.c);
    b.unit_bytes = (long long)unit_scratch_bytes(b.sd.c, S, kmax);
    b.sc0 = (long long)scb;
    scb += (size_t)nb * b.unit_bytes;
    bp.gmax = std::max(bp.gmax, b.sd.g);
    bp.cmax = std::max(bp.cmax, b.sd.c);
    bp.fp64 = bp.fp64 && use_popc(b.sd);
  }
  const bool masks_host = jobs[units[0].job].masks_host != nullptr;
  // kept units: unit 0 of a keeping job
  std::vector<int> kept;  // batch indices of kept units
  std::vector<int32_t> keep_slot(Bt, -1);
  int mpk = 1;
  for (int i = 0; i < Bt; i++)
    if (units[i].i == 0 && jobs[units[i].job].keep) {
      keep_slot[i] = (int32_t)kept.size();
      kept.push_back(i);
      mpk = std::max(mpk, jobs[units[i].job].mpk);
    }
  const int nk = (int)kept.size(), kg = bp.gmax, kgw = (kg + 31) / 32;
  if (nk) {
    CK(ctx->d_oids.ensure(sizeof(int32_t) * (size_t)nk * S));
    CK(ctx->d_ocnt.ensure(sizeof(int32_t) * (size_t)nk * S * kg));
    CK(ctx->d_opar.ensure(sizeof(int32_t) * (size_t)nk * S * kg * mpk));
    CK(ctx->d_odist.ensure(sizeof(double) * 2 * (size_t)nk * S));
    CK(ctx->d_olval.ensure(sizeof(double) * 2 * (size_t)nk * S));
    CK(ctx->d_orows.ensure(sizeof(uint32_t) * 2 * (size_t)nk * kg * kgw));
    CK(cudaMemsetAsync(ctx->d_opar.p, 0xff, sizeof(int32_t) * (size_t)nk * S * kg * mpk, ctx->stream));
  }
  CK(ctx->d_stats.ensure(sizeof(unsigned long long) * 4 * ns));
  CK(cudaMemsetAsync(ctx->d_stats.p, 0, sizeof(unsigned long long) * 4 * ns, ctx->stream));
  CK(ctx->d_masks.ensure(sizeof(uint64_t) * (size_t)Bt * W));
  {
    int rc = dmask_ready(ctx, sizeof(uint32_t) * std::max<size_t>(dmw, 1));
    if (rc) return rc;
  }
  CK(ctx->d_scratch.ensure(std::max<size_t>(scb, 1)));
  CK(ctx->d_js.ensure(sizeof(double) * Bt));
  CK(ctx->d_U.ensure(sizeof(int32_t) * Bt));
  CK(ctx->d_status.ensure(sizeof(uint32_t) * Bt));
  CK(ctx->d_keep.ensure(sizeof(int32_t) * Bt));
  CK(ctx->d_uslot.ensure(sizeof(int32_t) * Bt));
  CK(ctx->d_uset.ensure(sizeof(int32_t) * Bt));
  CK(ctx->d_uperm.ensure(sizeof(int32_t) * Bt));
  CK(ctx->d_sets.ensure(sizeof(BatchSet) * ns));
  // pinned staging: [set ids][permutations][slots][kept slots][set table]
  // (uploads); results in h_res
  const size_t o_tab = (16 * (size_t)Bt + 255) & ~(size_t)255;
  CK(ctx->h_stage.ensure(o_tab + sizeof(BatchSet) * ns + 64));
  CK(ctx->h_res.ensure(16 * (size_t)Bt + 64 + 32 * (size_t)ns));
  int32_t *hs = ctx->h_stage.as<int32_t>(), *hp = hs + Bt, *hsl = hp + Bt, *hk = hsl + Bt;
  for (int i = 0; i < Bt; i++) {
    const Job &J = jobs[units[i].job];
    hs[i] = J.set_id;
    hp[i] = J.perms ? J.perms[units[i].i] : 0;
    hsl[i] = uslot[i];
    hk[i] = keep_slot[i];
  }
  CK(cudaMemcpyAsync(ctx->d_uslot.p, hsl, 4 * (size_t)Bt, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_keep.p, hk, 4 * (size_t)Bt, cudaMemcpyHostToDevice, ctx->stream));
  if (masks_host) {
    std::vector<uint64_t> mh((size_t)Bt * W);
    for (int i = 0; i < Bt; i++)
      memcpy(mh.data() + (size_t)i * W, jobs[units[i].job].masks_host + (size_t)units[i].i * W, 8 * W);
    CK(cudaMemcpyAsync(ctx->d_masks.p, mh.data(), 8 * mh.size(), cudaMemcpyHostToDevice, ctx->stream));
  } else {
    CK(cudaMemcpyAsync(ctx->d_uset.p, hs, 4 * (size_t)Bt, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_uperm.p, hp, 4 * (size_t)Bt, cudaMemcpyHostToDevice, ctx->stream));
  }
  BatchDev bd{};
  bd.B = Bt;
  bd.nsets = ns;
  bd.kmax = kmax;
  bd.key_walk = getenv("EDDY_KEY_WALK") ? 1 : 0;
  bd.sets = ctx->d_sets.as<BatchSet>();
  bd.uslot = ctx->d_uslot.as<int32_t>();
  bd.masks = ctx->d_masks.as<uint64_t>();
  bd.dmask = ctx->d_dmask.as<uint32_t>();
  bd.scratch = ctx->d_scratch.as<uint8_t>();
  bd.js = ctx->d_js.as<double>();
  bd.U = ctx->d_U.as<int32_t>();
  bd.status = ctx->d_status.as<uint32_t>();
  bd.keep_slot = ctx->d_keep.as<int32_t>();
  bd.keep_g = kg;
  bd.keep_gw = kgw;
  bd.out_ids = ctx->d_oids.as<int32_t>();
  bd.out_cnt = ctx->d_ocnt.as<int32_t>();
  bd.out_par = ctx->d_opar.as<int32_t>();
  bd.mpk = mpk;
  bd.out_dist = ctx->d_odist.as<double>();
  bd.out_lval = ctx->d_olval.as<double>();
  bd.out_rows = ctx->d_orows.as<uint32_t>();
  bd.stats = ctx->d_stats.as<unsigned long long>();
  // the batch's device work: labellings, decisions, networks (events
  // become record nodes when captured)
  auto record = [&](cudaEvent_t e, bool capturing) -> cudaError_t {
    return capturing ? cudaEventRecordWithFlags(e, ctx->stream, cudaEventRecordExternal)
                     : cudaEventRecord(e, ctx->stream);
  };
  // a steady-state batch (device labellings, nothing kept, tile shape known,
  // the sets resident) that repeats the previous one's sets, shape and
  // buffers is captured as one CUDA graph and later replayed; the uploads
  // above stay outside the graph
  Shape sh0 = shape_of(ctx, ids[0]);
  const bool mma = !popc_batch && !use_popc() && !bp.fp64 && bp.cmax > 0;
  const bool graphable = !masks_host && nk == 0 && mma && ctx->stream != nullptr &&
                         pick_variant(ctx, sh0, Bt) >= 0;
  auto enqueue = [&](bool capturing) -> int {
    if (!masks_host) {
      CK(launch_counter_masks(n, ctx->nA, W, ctx->o.seed, ctx->d_uset.as<int32_t>(),
                              ctx->d_uperm.as<int32_t>(), ctx->d_mask0.as<uint64_t>(),
                              ctx->d_masks.as<uint64_t>(), Bt, ctx->stream));
      ctx->launches++;
    }
    CK(record(ctx->ev[0], capturing));
    {
      int rc = launch_pairs_any(ctx, bp, bd.masks, bd.dmask, bd.stats, o_tab, popc_batch,
                                ctx->ev[4]);
      if (rc) return rc;
    }
    CK(record(ctx->ev[1], capturing));
    CK(launch_units(bd, bp.gmax, W, ctx->stream, ctx->ev[5], capturing));
    CK(record(ctx->ev[2], capturing));
    ctx->launches += 2;  // networks, then normalisation and JS
    return EDDY_OK;
  };
  ctx->dmask_clean = nullptr;  // until the batch is seen to finish
  if (graphable) {
    // the table of the tuned shape, uploaded outside the graph
    const int v = pick_variant(ctx, sh0, Bt);
    {
      int rc = prepare_y(ctx, layout_core(v));
      if (rc) return rc;
    }
    const MmaPlan mp = plan_mma(ctx, bp, v);
    CK(ctx->d_afp8.ensure(mma_a_bytes(mp, n, layout_core(v))));
    CK(ctx->d_err.ensure(sizeof(unsigned)));
    // everything a replay bakes in: the sets, their state, the batch shape
    // and every buffer address
    std::vector<uintptr_t> key = {(uintptr_t)ctx->prep_gen, (uintptr_t)ctx->salt,
                                  (uintptr_t)Bt, (uintptr_t)kmax, (uintptr_t)v,
                                  (uintptr_t)ctx->o.seed, (uintptr_t)ctx->d_masks.p,
                                  (uintptr_t)ctx->d_dmask.p, (uintptr_t)ctx->d_scratch.p,
                                  (uintptr_t)ctx->d_js.p, (uintptr_t)ctx->d_U.p,
                                  (uintptr_t)ctx->d_status.p, (uintptr_t)ctx->d_keep.p,
                                  (uintptr_t)ctx->d_uset.p, (uintptr_t)ctx->d_uperm.p,
                                  (uintptr_t)ctx->d_uslot.p, (uintptr_t)ctx->d_sets.p,
                                  (uintptr_t)ctx->d_stats.p, (uintptr_t)ctx->d_afp8.p,
                                  (uintptr_t)ctx->d_Y.p, (uintptr_t)ctx->d_err.p,
                                  (uintptr_t)ctx->d_mask0.p, (uintptr_t)ctx->stream,
                                  (uintptr_t)bp.sets[0].sd.exact_all, (uintptr_t)bd.key_walk};
    for (int k = 0; k < ns; k++) {
      key.push_back((uintptr_t)ids[k]);
      key.push_back((uintptr_t)bp.sets[k].nb);
    }
    const bool replay = ctx->graph_exec && key == ctx->graph_key;
    if (!replay && key != ctx->direct_key) {
      // first batch of this shape: direct launches, remembered
      ctx->direct_key = key;
      int rc = enqueue(false);
      if (rc) return rc;
    } else {
      // the uploads of the table and the error word happen outside the
      // graph, before its launch
      {
        int rc = upload_table(ctx, bp, o_tab);
        if (rc) return rc;
      }
      CK(cudaMemsetAsync(ctx->d_err.p, 0, sizeof(unsigned), ctx->stream));
      if (!replay) {
        if (ctx->graph_exec) {
          cudaGraphExecDestroy(ctx->graph_exec);
          ctx->graph_exec = nullptr;
        }
        ctx->graph_key.clear();
        const long long l0 = ctx->launches;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int rc = EDDY_OK;
        {
          auto cap_ck = [&](cudaError_t e) {
            if (e != cudaSuccess && rc == EDDY_OK)
              rc = fail(ctx, EDDY_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
          };
          cap_ck(launch_counter_masks(n, ctx->nA, W, ctx->o.seed, ctx->d_uset.as<int32_t>(),
                                      ctx->d_uperm.as<int32_t>(), ctx->d_mask0.as<uint64_t>(),
                                      ctx->d_masks.as<uint64_t>(), Bt, ctx->stream));
          cap_ck(record(ctx->ev[0], true));
          cap_ck(launch_pairs_mma(ctx->d_sets.as<BatchSet>(), ns, mp, bd.masks, bd.uslot, n, W,
                                  ctx->d_afp8.as<uint8_t>(), ctx->y, bd.dmask, bd.stats,
                                  ctx->d_err.as<unsigned>(), ctx->sms, ctx->stream, v,
                                  layout_core(v), ns == 1 ? bp.sets[0].sd.g : 0, ctx->ev[4],
                                  true));
          cap_ck(record(ctx->ev[1], true));
          cap_ck(launch_units(bd, bp.gmax, W, ctx->stream, ctx->ev[5], true));
          cap_ck(record(ctx->ev[2], true));
          ctx->launches += 1 + mma_launches() + 2;
        }
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
      ctx->tuned_variant = v;
    }
  } else {
    int rc = enqueue(false);
    if (rc) return rc;
  }
  // results (and the tensor-core kernel's timeout word) through the pinned
  // staging: JS, U, status, error word
  double *hjs = ctx->h_res.as<double>();
  int32_t *hU = ctx->h_res.as<int32_t>(8 * (size_t)Bt);
  uint32_t *hst = ctx->h_res.as<uint32_t>(12 * (size_t)Bt);
  unsigned *herr = ctx->h_res.as<unsigned>(16 * (size_t)Bt);
  *herr = 0;
  CK(cudaMemcpyAsync(hjs, ctx->d_js.p, 8 * (size_t)Bt, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(hU, ctx->d_U.p, 4 * (size_t)Bt, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(hst, ctx->d_status.p, 4 * (size_t)Bt, cudaMemcpyDeviceToHost, ctx->stream));
  if (mma) CK(cudaMemcpyAsync(herr, ctx->d_err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  // the decision counters of each set
  const unsigned long long *hst4 = ctx->h_res.as<unsigned long long>(16 * (size_t)Bt + 8);
  CK(cudaMemcpyAsync(ctx->h_res.as<unsigned long long>(16 * (size_t)Bt + 8), ctx->d_stats.p,
                     sizeof(unsigned long long) * 4 * ns, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const unsigned errw = *herr;
  if (errw & 1u) return fail(ctx, EDDY_ERR_INTERNAL, "tensor-core pipeline wait timed out");
  ctx->dmask_clean = ctx->d_dmask.p;  // the unit kernel cleared every bit set
  if (errw & 2u) {
    // the general-path queue overflowed: the caller decides this batch with
    // the popcount kernel
    *queue_full = true;
    return EDDY_OK;
  }
  float a = 0, bms = 0;
  cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);
  cudaEventElapsedTime(&bms, ctx->ev[1], ctx->ev[2]);
  *t_pairs += a;
  *t_units += bms;
  {
    const int cut[5] = {0, 4, 1, 5, 2};
    for (int q = 0; q < 4; q++) {
      float m = 0;
      if (cudaEventElapsedTime(&m, ctx->ev[cut[q]], ctx->ev[cut[q + 1]]) == cudaSuccess)
        ctx->ms_stage[q] += m;
    }
  }
  for (int k = 0; k < ns; k++) {
    for (int q = 0; q < 4; q++) ctx->last_stats[q] += hst4[4 * k + q];
    jobs[slot_job[k]].exact += hst4[4 * k];
    jobs[slot_job[k]].tables += hst4[4 * k + 1];
  }
  for (int i = 0; i < Bt; i++) {
    Job &J = jobs[units[i].job];
    if (hst[i] & kUnitKmaxOverflow) {
      *need = std::max(*need, (int)(hst[i] >> 16));
      again->push_back(units[i]);
    } else if (hst[i] & kUnitHashCollision) {
      *collision = true;
      again->push_back(units[i]);
    } else {
      J.js[units[i].i] = hjs[i];
      J.U[units[i].i] = hU[i];
    }
  }
  // detailed outputs of the kept units that finished
  for (int q = 0; q < nk; q++) {
    const int i = kept[q];
    if (hst[i] & (kUnitKmaxOverflow | kUnitHashCollision)) continue;
    Job &J = jobs[units[i].job];
    KeepOut *K = J.keep;
    const int g = ctx->res_sd[uslot[i]].g, GW = (g + 31) / 32, Uk = hU[i];
    K->mpk = J.mpk;
    K->U = Uk;
    K->ids.resize(Uk);
    K->cnt.resize((size_t)Uk * g);
    K->par.resize((size_t)Uk * g * J.mpk);
    K->dist.resize(2 * (size_t)S);
    K->lval.resize(2 * (size_t)S);
    K->rows.resize(2 * (size_t)g * GW);
    std::vector<int32_t> cnt((size_t)S * kg), par((size_t)S * kg * mpk);
    std::vector<uint32_t> rows(2 * (size_t)kg * kgw);
    CK(cudaMemcpyAsync(K->ids.data(), ctx->d_oids.as<int32_t>() + (size_t)q * S, 4 * (size_t)Uk,
                       cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(cnt.data(), ctx->d_ocnt.as<int32_t>() + (size_t)q * S * kg,
                       4 * (size_t)Uk * kg, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(par.data(), ctx->d_opar.as<int32_t>() + (size_t)q * S * kg * mpk,
                       4 * (size_t)Uk * kg * mpk, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(K->dist.data(), ctx->d_odist.as<double>() + 2 * (size_t)q * S, 16 * (size_t)S,
                       cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(K->lval.data(), ctx->d_olval.as<double>() + 2 * (size_t)q * S, 16 * (size_t)S,
                       cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(rows.data(), ctx->d_orows.as<uint32_t>() + 2 * (size_t)q * kg * kgw,
                       4 * rows.size(), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int uu = 0; uu < Uk; uu++)
      for (int t = 0; t < g; t++) {
        K->cnt[(size_t)uu * g + t] = cnt[(size_t)uu * kg + t];
        for (int m = 0; m < J.mpk; m++)
          K->par[((size_t)uu * g + t) * J.mpk + m] = par[((size_t)uu * kg + t) * mpk + m];
      }
    for (int k = 0; k < 2; k++)
      for (int t = 0; t < g; t++)
        for (int w = 0; w < GW; w++)
          K->rows[((size_t)k * g + t) * GW + w] = rows[((size_t)k * kg + t) * kgw + w];
  }
  return EDDY_OK;
}

// Runs jobs of sets that share a contingency-kernel choice (one tuning key)
// in equal batches of units across the jobs (a batch may hold the units of
// several sets), each unit run again until its status is clean.
int run_jobs(eddy_ctx *ctx, std::vector<Job> &jobs) {
  if (jobs.empty()) return EDDY_OK;
  const int n = ctx->samples, S = n + 2, W = ctx->W;
  int gmax = 0, cmax = 1, total = 0;
  size_t per_unit_max = 1;
  // kmax: changed-node records per network (records are written only for
  // changed nodes, so room for more costs memory, not time).  64 covers the
  // networks of most sets; at 200 genes with ~3% of the pair tests within
  // 20% of the threshold, about one unit in eight of a context's first
  // batch needs more and is re-run, and the per-size hint gives later
  // batches that room.  EDDY_KMAX lowers it, to test those re-runs.
  const char *ek = getenv("EDDY_KMAX");
  int kmax = 1;
  for (const Job &J : jobs) {
    const int g = (int)ctx->sets[J.set_id].genes.size(), c = g * (g - 1) / 2;
    gmax = std::max(gmax, g);
    cmax = std::max(cmax, c);
    total += J.n_units;
    int k = std::min(g + 1, 64);
    auto it = ctx->kmax_hint.find(g);
    if (it != ctx->kmax_hint.end()) k = std::max(k, std::min(g + 1, it->second));
    kmax = std::max(kmax, k);
  }
  if (ek) kmax = std::max(1, std::min(16, atoi(ek)));
  for (const Job &J : jobs) {
    const int g = (int)ctx->sets[J.set_id].genes.size(), c = g * (g - 1) / 2;
    per_unit_max = std::max(per_unit_max, unit_scratch_bytes(c, S, kmax) + 4 * (size_t)c + 8 * W + 64);
  }
  // batch size: bounded by memory (masks, decisions and scratch, up to 16 GB),
  // by 16384 units (the general-path queue holds unit indices below 2^15)
  // and by the queue's room for every table of the batch (2^28): the units
  // are then split into batches of equal size (later calls of the same
  // size replay them)
  int Bmax = (int)std::max<size_t>(1, ((size_t)16 << 30) / per_unit_max);
  Bmax = std::min(Bmax, 16384);
  Bmax = (int)std::min<size_t>((size_t)Bmax, std::max<size_t>(1, ((size_t)1 << 28) / (2 * (size_t)cmax)));
  {
    const int nb = std::max(1, (total + Bmax - 1) / Bmax);
    Bmax = std::max(1, (total + nb - 1) / nb);
  }
  std::vector<UnitRef> all;
  all.reserve(total);
  for (int j = 0; j < (int)jobs.size(); j++)
    for (int i = 0; i < jobs[j].n_units; i++) all.push_back({j, i});
  ctx->last_stats[0] = ctx->last_stats[1] = ctx->last_stats[2] = ctx->last_stats[3] = 0;
  float t_pairs = 0, t_units = 0;
  for (int b0 = 0; b0 < total; b0 += Bmax) {
    std::vector<UnitRef> todo(all.begin() + b0, all.begin() + std::min(total, b0 + Bmax));
    int kmax_run = kmax;
    bool popc_batch = false;
    for (int attempt = 0; attempt < 4 && !todo.empty(); attempt++) {
      std::vector<UnitRef> again;
      int need = 0;
      bool collision = false, queue_full = false;
      int rc = run_batch(ctx, jobs, todo, kmax_run, popc_batch, &again, &need, &collision,
                         &queue_full, &t_pairs, &t_units);
      if (rc) return rc;
      if (queue_full) {
        // a large share of tables near a threshold: decide this batch with
        // the popcount kernel
        popc_batch = true;
        continue;
      }
      if (need) {
        // the re-run holds every record these units need (their networks do
        // not change); sets of this size start with a quarter more later
        const int want = std::max(need, kmax_run + 1);
        kmax_run = std::min(gmax + 1, (want + 7) / 8 * 8);
        if (!ek)
          for (const UnitRef &r : again) {
            const int g = (int)ctx->sets[jobs[r.job].set_id].genes.size();
            int &hint = ctx->kmax_hint[g];
            hint = std::max(hint, std::min(g + 1, (want + want / 4 + 7) / 8 * 8));
          }
      }
      if (collision) ctx->salt = ctx->salt * 6364136223846793005ull + 1442695040888963407ull;
      todo.swap(again);
    }
    if (!todo.empty())
      return fail(ctx, EDDY_ERR_INTERNAL, "units of set %d did not converge",
                  jobs[todo[0].job].set_id);
  }
  ctx->ms_pairs += t_pairs;
  ctx->ms_units += t_units;
  ctx->ms_total += t_pairs + t_units;
  return EDDY_OK;
}

// One set's units (the single-set entry points).
int run_units(eddy_ctx *ctx, int set_id, int nunits, const uint64_t *masks_host,
              const int32_t *perms, double *js, int32_t *U, KeepOut *keep, int mpk,
              unsigned long long *exact = nullptr, unsigned long long *tables = nullptr) {
  std::vector<Job> jobs(1);
  jobs[0].set_id = set_id;
  jobs[0].n_units = nunits;
  jobs[0].masks_host = masks_host;
  jobs[0].perms = perms;
  jobs[0].js = js;
  jobs[0].U = U;
  jobs[0].keep = keep;
  jobs[0].mpk = std::max(1, mpk);
  int rc = run_jobs(ctx, jobs);
  if (exact) *exact += jobs[0].exact;
  if (tables) *tables += jobs[0].tables;
  return rc;
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
  DevBuf *bufs[] = {&ctx->d_lg, &ctx->d_setdata, &ctx->d_mask0, &ctx->d_masks, &ctx->d_dmask,
                    &ctx->d_scratch, &ctx->d_js, &ctx->d_U, &ctx->d_status, &ctx->d_keep,
                    &ctx->d_uset, &ctx->d_uperm, &ctx->d_uslot, &ctx->d_sets, &ctx->d_oids,
                    &ctx->d_ocnt, &ctx->d_opar, &ctx->d_odist, &ctx->d_olval, &ctx->d_orows,
                    &ctx->d_stats, &ctx->d_Y, &ctx->d_afp8, &ctx->d_err};
  for (DevBuf *b : bufs) b->release();
  for (auto &ev : ctx->ev)
    if (ev) cudaEventDestroy(ev);
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  ctx->h_stage.release();
  ctx->h_res.release();
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
  ctx->res_ids.clear();
  ctx->res_sd.clear();
  ctx->y_ready = false;
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

namespace {
// The glibc label stream of iterations 1 .. R-1 of a set, generated on a
// thread of its own from a copy of the stream's state (main.cu:538-573):
// the GPU runs iteration 0, then the permutations chunk by chunk as they
// become ready, while the rest are drawn.  The stream is serial, so this
// only hides the GPU's time behind the draws (or the draws behind the
// GPU's).  A set whose iteration 0 breaks (NaN JS, main.cu:1431-1435)
// cancels the thread, and the next set starts from the state after its
// iteration 0.  The destructor cancels and joins.
class GlibcProducer {
 public:
  GlibcProducer(const GlibcRand &state, int n, int nA, int W, int count, const uint8_t *labels0)
      : rng_(state), n_(n), nA_(nA), W_(W), count_(count), labels_(labels0, labels0 + n),
        masks_((size_t)count * W, 0) {
    th_ = std::thread([this] { work(); });
  }
  ~GlibcProducer() {
    cancel_.store(true);
    if (th_.joinable()) th_.join();
  }
  // waits until at least `want` labellings are ready (or all); returns how
  // many are ready
  int wait_ready(int want) {
    std::unique_lock<std::mutex> lk(mu_);
    cv_.wait(lk, [&] { return ready_ >= want || ready_ >= count_; });
    return ready_;
  }
  const uint64_t *masks(int i) const { return masks_.data() + (size_t)i * W_; }
  // joins and returns the stream's state after the last labelling
  GlibcRand finish() {
    if (th_.joinable()) th_.join();
    return rng_;
  }

 private:
  void work() {
    std::vector<uint8_t> seen;
    std::vector<int> order;
    for (int i = 0; i < count_ && !cancel_.load(std::memory_order_relaxed); i++) {
      glibc_permutation(rng_, n_, nA_, true, labels_.data(), seen, order);
      uint64_t *m = masks_.data() + (size_t)i * W_;
      for (int s = 0; s < n_; s++)
        if (labels_[s] == 0) m[s >> 6] |= 1ull << (s & 63);
      if ((i & 31) == 31 || i + 1 == count_) {
        std::lock_guard<std::mutex> lk(mu_);
        ready_ = i + 1;
        cv_.notify_all();
      }
    }
  }
  GlibcRand rng_;
  const int n_, nA_, W_, count_;
  std::vector<uint8_t> labels_;
  std::vector<uint64_t> masks_;
  std::thread th_;
  std::mutex mu_;
  std::condition_variable cv_;
  int ready_ = 0;
  std::atomic<bool> cancel_{false};
};
}  // namespace

static void finish_set(SetHost &S, int R);
static void finish_counter_set(eddy_ctx *ctx, SetHost &S, const KeepOut &K, int R);

static int run_set(eddy_ctx *ctx, int set_id) {
  SetHost &S = ctx->sets[set_id];
  const int n = ctx->samples, W = ctx->W;
  const int g = (int)S.genes.size();
  const int R = set_iterations(ctx, S);
  if (R < 1) return fail(ctx, EDDY_ERR_STATE, "set %d has no labellings", set_id);
  if (!S.it0) {
    S.js.assign(R, NAN);
    S.U.assign(R, 0);
    S.iterations = 0;
    S.failed = 0;
    S.betafit_ok = 0;
    S.exact = S.tables = 0;
  }
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
  int rc = EDDY_OK;
  const int mpk0 = std::min(ctx->o.max_parents, std::max(g - 1, 1));
  if (ctx->o.rng == EDDY_RNG_COUNTER && n <= 4096) {
    // counter stream, labellings generated on the device: iteration 0 (the
    // unpermuted labelling, kept), then, unless its JS is not finite, which
    // ends the set there (main.cu:1431-1435), the permutations in one pass
    std::vector<int32_t> perms(R);
    for (int i = 0; i < R; i++) perms[i] = i;
    KeepOut K;
    rc = run_units(ctx, set_id, 1, nullptr, perms.data(), S.js.data(), S.U.data(),
                   ctx->o.keep_networks ? &K : nullptr, mpk0, &S.exact, &S.tables);
    if (rc) return rc;
    if (R > 1 && finite_js(S.js[0])) {
      rc = run_units(ctx, set_id, R - 1, nullptr, perms.data() + 1, S.js.data() + 1,
                     S.U.data() + 1, nullptr, 1, &S.exact, &S.tables);
      if (rc) return rc;
    }
    finish_counter_set(ctx, S, K, R);
    return EDDY_OK;
  } else {
    // iteration 0 (kept: networks and likelihoods for the output files)
    std::vector<uint64_t> masks((size_t)W);
    std::vector<uint8_t> lab(ctx->labels0);
    if (ctx->o.rng == EDDY_RNG_EXTERNAL) lab.assign(S.labels.begin(), S.labels.begin() + n);
    if (ctx->o.rng == EDDY_RNG_GLIBC)
      glibc_permutation(ctx->rng, n, ctx->nA, false, lab.data(), ctx->seen, ctx->order);
    labels_to_mask(lab.data(), n, W, masks.data());
    // glibc stream: the permutations are drawn while the GPU runs
    // iteration 0 and the earlier chunks (a set whose iteration 0 the
    // batched pass ran draws them only if it goes on)
    std::unique_ptr<GlibcProducer> prod;
    if (ctx->o.rng == EDDY_RNG_GLIBC && R > 1 && (!S.it0 || finite_js(S.js[0])))
      prod.reset(new GlibcProducer(ctx->rng, n, ctx->nA, W, R - 1, ctx->labels0.data()));
    if (!S.it0) {
      KeepOut K;
      rc = run_units(ctx, set_id, 1, masks.data(), nullptr, S.js.data(), S.U.data(),
                     ctx->o.keep_networks ? &K : nullptr, mpk0, &S.exact, &S.tables);
      if (rc) return rc;
      if (ctx->o.keep_networks) store_keep(ctx, S, K, g);
      else S.U0 = S.U[0];
      S.iterations = 1;
    }
    if (!finite_js(S.js[0])) {
      // main.cu:1431-1435: break after iteration 0 (the stream goes on from
      // the state after its draws: the producer's are discarded)
      S.failed = 1;
      S.done = true;
      return EDDY_OK;
    }
    if (prod) {
      const int nu = R - 1;
      std::vector<int32_t> perms(nu);
      for (int i = 0; i < nu; i++) perms[i] = i + 1;
      int done = 0;
      while (done < nu) {
        // at least 256 labellings per call (or what is left), more if ready
        const int ready = prod->wait_ready(std::min(nu, done + 256));
        const int cnt = ready - done;
        rc = run_units(ctx, set_id, cnt, prod->masks(done), perms.data() + done,
                       S.js.data() + 1 + done, S.U.data() + 1 + done, nullptr, 1, &S.exact,
                       &S.tables);
        if (rc) return rc;
        done = ready;
      }
      ctx->rng = prod->finish();
    } else if (R > 1) {
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
      rc = run_units(ctx, set_id, nu, device_counter ? nullptr : mh.data(), perms.data(),
                     S.js.data() + 1, S.U.data() + 1, nullptr, 1, &S.exact, &S.tables);
      if (rc) return rc;
    }
    S.iterations = R;
  }
  finish_set(S, R);
  return EDDY_OK;
}

// A set whose R iterations ran: the NaN check and the beta fit.
static void finish_set(SetHost &S, int R) {
  for (int i = 0; i < R; i++)
    if (!finite_js(S.js[i])) S.failed = 1;
  // beta fit on the host: the sequential FP64 moment loop and the continued
  // fraction are chains of dependent FP64 operations, which run faster on
  // the host cores than on the GPU
  if (!S.failed) S.betafit_ok = beta_pddn(S.js.data(), R, S.alpha, S.beta, S.pddn) ? 1 : 0;
  S.done = true;
}

// A set whose iteration 0 and permutations ran in one pass on the counter
// stream: a non-finite JS at iteration 0 ends the set there
// (main.cu:1431-1435) and the permutations' results are discarded.
static void finish_counter_set(eddy_ctx *ctx, SetHost &S, const KeepOut &K, int R) {
  const int g = (int)S.genes.size();
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
    return;
  }
  S.iterations = R;
  finish_set(S, R);
}

// Sets that share a contingency-kernel choice (one tuning key) on the
// counter stream, all in one run: their units go through batches that hold
// several sets each (one set table per batch).  Iteration 0 of every set
// runs first (kept for its output files); a set whose JS there is not
// finite stops (main.cu:1431-1435), so only the other sets' permutations
// are run, again batched across the sets.
static int run_counter_sets(eddy_ctx *ctx, const std::vector<int> &ids) {
  const int R = ctx->o.permutations;
  std::vector<Job> jobs(ids.size());
  std::vector<KeepOut> keeps(ids.size());
  std::vector<int32_t> perms(R);
  for (int i = 0; i < R; i++) perms[i] = i;
  for (size_t j = 0; j < ids.size(); j++) {
    SetHost &S = ctx->sets[ids[j]];
    const int g = (int)S.genes.size();
    S.js.assign(R, NAN);
    S.U.assign(R, 0);
    S.iterations = 0;
    S.failed = 0;
    S.betafit_ok = 0;
    S.exact = S.tables = 0;
    jobs[j].set_id = ids[j];
    jobs[j].n_units = 1;
    jobs[j].perms = perms.data();
    jobs[j].js = S.js.data();
    jobs[j].U = S.U.data();
    jobs[j].keep = ctx->o.keep_networks ? &keeps[j] : nullptr;
    jobs[j].mpk = std::min(ctx->o.max_parents, std::max(g - 1, 1));
  }
  int rc = run_jobs(ctx, jobs);
  if (rc) return rc;
  std::vector<Job> rest;
  std::vector<size_t> of;
  for (size_t j = 0; j < ids.size(); j++) {
    SetHost &S = ctx->sets[ids[j]];
    S.exact = jobs[j].exact;
    S.tables = jobs[j].tables;
    if (R < 2 || !finite_js(S.js[0])) continue;
    Job J;
    J.set_id = ids[j];
    J.n_units = R - 1;
    J.perms = perms.data() + 1;
    J.js = S.js.data() + 1;
    J.U = S.U.data() + 1;
    rest.push_back(J);
    of.push_back(j);
  }
  if (!rest.empty()) {
    rc = run_jobs(ctx, rest);
    if (rc) return rc;
    for (size_t k = 0; k < rest.size(); k++) {
      SetHost &S = ctx->sets[ids[of[k]]];
      S.exact += rest[k].exact;
      S.tables += rest[k].tables;
    }
  }
  for (size_t j = 0; j < ids.size(); j++)
    finish_counter_set(ctx, ctx->sets[ids[j]], keeps[j], R);
  return EDDY_OK;
}

// Iteration 0 of sets on the glibc stream, in shared batches.  Iteration 0
// labels the samples as given (its draws, main.cu:538-573, leave the labels
// unchanged), so its networks and JS do not depend on the stream; the
// stream itself is advanced set by set afterwards, in order (run_set), and
// only the sets whose iteration-0 JS is finite draw permutations.
static int run_iteration0_sets(eddy_ctx *ctx, const std::vector<int> &ids) {
  const int W = ctx->W;
  std::vector<uint64_t> mask0((size_t)W);
  labels_to_mask(ctx->labels0.data(), ctx->samples, W, mask0.data());
  std::vector<Job> jobs(ids.size());
  std::vector<KeepOut> keeps(ids.size());
  for (size_t j = 0; j < ids.size(); j++) {
    SetHost &S = ctx->sets[ids[j]];
    const int g = (int)S.genes.size(), R = set_iterations(ctx, S);
    S.js.assign(R, NAN);
    S.U.assign(R, 0);
    S.iterations = 0;
    S.failed = 0;
    S.betafit_ok = 0;
    S.exact = S.tables = 0;
    jobs[j].set_id = ids[j];
    jobs[j].n_units = 1;
    jobs[j].masks_host = mask0.data();
    jobs[j].js = S.js.data();
    jobs[j].U = S.U.data();
    jobs[j].keep = ctx->o.keep_networks ? &keeps[j] : nullptr;
    jobs[j].mpk = std::min(ctx->o.max_parents, std::max(g - 1, 1));
  }
  int rc = run_jobs(ctx, jobs);
  if (rc) return rc;
  for (size_t j = 0; j < ids.size(); j++) {
    SetHost &S = ctx->sets[ids[j]];
    S.exact = jobs[j].exact;
    S.tables = jobs[j].tables;
    if (ctx->o.keep_networks) store_keep(ctx, S, keeps[j], (int)S.genes.size());
    else S.U0 = S.U[0];
    S.iterations = 1;
    S.it0 = true;
  }
  return EDDY_OK;
}

int eddy_run(eddy_ctx *ctx) {
  if (!ctx) return EDDY_ERR_ARG;
  if (ctx->samples == 0) return fail(ctx, EDDY_ERR_STATE, "no matrix loaded");
  ctx->ms_total = ctx->ms_pairs = ctx->ms_units = 0;
  for (double &m : ctx->ms_stage) m = 0;
  ctx->launches = 0;
  if (ctx->o.rng == EDDY_RNG_COUNTER && ctx->samples <= 4096) {
    // the counter stream's sets (labellings drawn on the device, independent
    // of the other sets) run together, grouped by contingency-kernel choice
    std::map<std::pair<int, int>, std::vector<int>> groups;
    for (int s = 0; s < (int)ctx->sets.size(); s++) {
      if (ctx->sets[s].done || ctx->sets[s].genes.size() < 2) continue;
      groups[tune_key(ctx->samples, shape_of(ctx, s))].push_back(s);
    }
    for (auto &gr : groups) {
      int rc = run_counter_sets(ctx, gr.second);
      if (rc) return rc;
    }
  }
  if (ctx->o.rng == EDDY_RNG_GLIBC) {
    std::map<std::pair<int, int>, std::vector<int>> groups;
    for (int s = 0; s < (int)ctx->sets.size(); s++) {
      if (ctx->sets[s].done || ctx->sets[s].it0 || ctx->sets[s].genes.size() < 2) continue;
      groups[tune_key(ctx->samples, shape_of(ctx, s))].push_back(s);
    }
    for (auto &gr : groups) {
      int rc = run_iteration0_sets(ctx, gr.second);
      if (rc) return rc;
    }
  }
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
  for (double &m : ctx->ms_stage) m = 0;
  ctx->launches = 0;
  if (ctx->sets[set_id].genes.size() < 2) {
    for (int r = 0; r < R; r++) {
      js[r] = NAN;
      unique[r] = 1;
    }
    return EDDY_OK;
  }
  std::vector<uint64_t> mh((size_t)R * W);
  for (int r = 0; r < R; r++) labels_to_mask(labels + (size_t)r * n, n, W, mh.data() + (size_t)r * W);
  return run_units(ctx, set_id, R, mh.data(), nullptr, js, unique, nullptr, 1);
}

int eddy_debug_edges(eddy_ctx *ctx, int set_id, const uint8_t *labels, uint8_t *edges) {
  if (!ctx || !labels || !edges || set_id < 0 || set_id >= (int)ctx->sets.size()) return EDDY_ERR_ARG;
  const int n = ctx->samples, W = ctx->W;
  if (ctx->sets[set_id].genes.size() < 2) return EDDY_OK;  // no pair
  int rc = prepare_sets(ctx, {set_id});
  if (rc) return rc;
  // a batch of one unit of one set
  BatchPlan bp;
  bp.B = 1;
  bp.sets.assign(1, BatchSet{});
  bp.sets[0].sd = ctx->res_sd[0];
  bp.sets[0].nb = 1;
  bp.sets[0].unit_bytes = 0;
  bp.gmax = bp.sets[0].sd.g;
  bp.cmax = bp.sets[0].sd.c;
  bp.fp64 = use_popc(bp.sets[0].sd);
  const SetDev sd = bp.sets[0].sd;
  const int c = sd.c, S = sd.S;
  std::vector<uint64_t> m(W);
  labels_to_mask(labels, n, W, m.data());
  CK(ctx->d_masks.ensure(8 * W));
  rc = dmask_ready(ctx, dmask_bytes(1, c));
  if (rc) return rc;
  ctx->dmask_clean = nullptr;  // no unit kernel reads (and clears) these masks
  CK(ctx->h_stage.ensure(512 + sizeof(BatchSet)));
  CK(ctx->d_uslot.ensure(sizeof(int32_t)));
  CK(cudaMemsetAsync(ctx->d_uslot.p, 0, sizeof(int32_t), ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_masks.p, m.data(), 8 * W, cudaMemcpyHostToDevice, ctx->stream));
  rc = launch_pairs_any(ctx, bp, ctx->d_masks.as<uint64_t>(), ctx->d_dmask.as<uint32_t>(), nullptr,
                        256);
  if (rc) return rc;
  rc = check_mma_error(ctx, bp);
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
  if (ctx->sets[set_id].genes.size() < 2) return fail(ctx, EDDY_ERR_ARG, "set %d has no pair", set_id);
  std::vector<uint64_t> m(W);
  labels_to_mask(labels, n, W, m.data());
  KeepOut K;
  double j = 0;
  int32_t u = 0;
  int rc = run_units(ctx, set_id, 1, m.data(), nullptr, &j, &u, &K, mpk);
  if (rc) return rc;
  const int g = (int)ctx->sets[set_id].genes.size(), S = n + 2;
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
  for (double &m : ctx->ms_stage) m = 0;
  ctx->launches = 0;
  if (S.genes.size() < 2) {
    for (int i = 0; i < count; i++) {
      js[i] = NAN;
      unique[i] = 1;
    }
    return EDDY_OK;
  }
  std::vector<int32_t> perms(count);
  for (int i = 0; i < count; i++) perms[i] = first + i;
  if (ctx->o.rng == EDDY_RNG_COUNTER && n <= 4096)
    return run_units(ctx, set_id, count, nullptr, perms.data(), js, unique, nullptr, 1);
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
  return run_units(ctx, set_id, count, mh.data(), nullptr, js, unique, nullptr, 1);
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
  ctx->res_ids.clear();
  ctx->res_sd.clear();
  ctx->y_ready = false;
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

int eddy_last_stage_timing(const eddy_ctx *ctx, double *ms4) {
  if (!ctx || !ms4) return EDDY_ERR_ARG;
  for (int q = 0; q < 4; q++) ms4[q] = ctx->ms_stage[q];
  return EDDY_OK;
}

}  // extern "C"
