/*
 * eddy_gpu.h -- C ABI of libeddy_gpu, the GB300 (sm_103a) implementation of
 * EDDY's per-class dependency-network inference and class-label
 * permutation test (the hot path of skimlab/eddy-gpu's ./eddy).
 *
 * The reference has no library boundary: its interface is the process
 * (main.cu:27-1711).  Each entry point below replaces one block of that
 * process; the citation names it.  Conventions:
 *   - every function returns an int status (EDDY_OK = 0) and never exits;
 *   - the library copies all caller input buffers; result buffers are
 *     caller-allocated (sizes are queried first) and filled by copy;
 *   - one context = one CUDA device and one stream, single-threaded use;
 *   - arrays are plain C pointers and sizes, no framework types.
 * Vocabulary: genes x samples expression matrix (ternary -1/0/1, any other
 * value is "not counted" like the reference's sscanf("%d") values outside
 * {-1,0,1}, kernel1.cu:91-118); class 0 = the reference's class1 (first
 * label of the class file), class 1 = class2; a gene set of g genes; a
 * unit = one gene set under one labelling (permutation); S = n + 2
 * leave-one-out networks per unit.
 */
#ifndef EDDY_GPU_H
#define EDDY_GPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EDDY_OK 0
#define EDDY_ERR_ARG 1        /* invalid argument or size */
#define EDDY_ERR_CUDA 2       /* CUDA runtime error (message via eddy_last_error) */
#define EDDY_ERR_STATE 3      /* call out of order (e.g. results before eddy_run) */
#define EDDY_ERR_CAPACITY 4   /* too large for the GPU path (g > 512 genes, > 65535 samples) */
#define EDDY_ERR_BETAFIT 5    /* beta fit has alpha/beta <= 0 or non-finite */
#define EDDY_ERR_INTERNAL 6   /* an internal consistency check failed */

/* Label-permutation streams.  GLIBC reproduces main.cu:538-573 exactly
 * (glibc rand(), never reseeded, one stream across all gene sets);
 * COUNTER uses Philox-4x32-10 keyed by seed: sample s's key is word s mod 4
 * of the block with counter (s / 4, permutation, set, 0), and the n_A
 * samples with the smallest (key, s) form class 0 of that permutation;
 * EXTERNAL takes caller-supplied labellings (eddy_set_labellings). */
#define EDDY_RNG_GLIBC 0
#define EDDY_RNG_COUNTER 1
#define EDDY_RNG_EXTERNAL 2

/* Run options: the reference's command-line values after its defaults and
 * clamps (main.cu:118-202). */
typedef struct {
  int max_parents;          /* -mp (main.cu:129-130, 171-175) */
  double alpha_edge;        /* -pE, or 1-theta^(1/lambda) with -t (main.cu:188-192) */
  double alpha_edge_prior;  /* 1-(1-alpha_edge)*pw^(1/lambda) (main.cu:195) */
  int bonferroni;           /* 0 with -rawp (main.cu:141-142) */
  int permutations;         /* -r, iterations incl. the unpermuted one (main.cu:538) */
  int rng;                  /* EDDY_RNG_* */
  uint64_t seed;            /* COUNTER stream key */
  int device;               /* CUDA device ordinal */
  int keep_networks;        /* 1: keep iteration-0 networks for the output files */
} eddy_opts;

typedef struct eddy_ctx eddy_ctx;

/* Creates a context (replaces main.cu's globals and device choice). */
int eddy_ctx_create(const eddy_opts *opts, eddy_ctx **out);
/* Releases everything the context holds. */
int eddy_ctx_destroy(eddy_ctx *ctx);
/* Text of the last error of this context (never NULL). */
const char *eddy_last_error(const eddy_ctx *ctx);

/* Expression matrix and class labels (replaces main.cu:255-352: the
 * parsed `data` matrix, gene-major, and classIDs).  data: genes x samples,
 * class_of_sample: samples entries, 0 or 1. */
int eddy_load_matrix(eddy_ctx *ctx, const int8_t *data, int genes, int samples,
                     const uint8_t *class_of_sample);

/* Adds a gene set (replaces main.cu:375-503: genesetIndexIntoData and the
 * prior matrix).  gene_idx: g row indices into the matrix (duplicates
 * allowed, kept in order); prior: g x g 0/1 (NULL = no prior file).
 * *set_id receives the set's index (0, 1, ... in call order). */
int eddy_add_set(eddy_ctx *ctx, const int32_t *gene_idx, int g, const uint8_t *prior,
                 int *set_id);

/* Caller-supplied labellings for EDDY_RNG_EXTERNAL (replaces the
 * permutation loop's classIDs, main.cu:561-570).  labels: R x samples,
 * row 0 is the unpermuted labelling. */
int eddy_set_labellings(eddy_ctx *ctx, int set_id, const uint8_t *labels, int R);

/* Runs every set: all permutations of the hot path (main.cu:538-1460) and
 * the beta fit (main.cu:1465-1502). */
int eddy_run(eddy_ctx *ctx);

typedef struct {
  int genes;            /* g */
  int iterations;       /* JS values computed (R, or 1 after a NaN JS0 break) */
  int failed;           /* 1 = NaN JS (main.cu:1431-1435, 1465-1479) */
  int betafit_ok;       /* 0 when alpha/beta are not positive finite */
  int unique0;          /* unique networks of iteration 0 (main.cu:1123-1125) */
  double js0;           /* JS of iteration 0 (main.cu:1482) */
  double alpha, beta;   /* beta fit (main.cu:1491-1495) */
  double pddn;          /* ibetac(alpha, beta, js0) (main.cu:1497) */
  uint64_t exact_rechecks;  /* tables re-evaluated in FP64 */
  uint64_t tables;          /* tables decided */
} eddy_set_summary;

/* Per-set results (replaces the printed lines and results.txt row). */
int eddy_get_set_summary(const eddy_ctx *ctx, int set_id, eddy_set_summary *out);
/* JS value and unique-network count of every iteration (jsVals,
 * main.cu:1427; unisum, main.cu:1088-1103).  Arrays of `iterations`. */
int eddy_get_js(const eddy_ctx *ctx, int set_id, double *js, int32_t *unique);

/* Iteration-0 unique networks for the _Networks and _BDEU_SCORES files
 * (first_uniNodes/first_uniEdges/first_uniEpn/uniqueNetIds/first_lval1,
 * main.cu:1087-1187, 1406-1409).  Query with NULL arrays to get *U and
 * *edges; then ids[U], nodes[U*g] (exclusive prefix of capped parent
 * counts, pNodes layout), epn[U+1], edges_out[edges], lval[2*U]
 * (class-0 likelihoods then class-1). */
int eddy_get_networks(const eddy_ctx *ctx, int set_id, int *U, int *edges, int32_t *ids,
                      int32_t *nodes, int32_t *epn, int32_t *edges_out, double *lval);

/* Uncapped parent lists of the two full-data networks of iteration 0 for
 * the _EdgeList file (main.cu:1530-1617): nodes[2*g], epn[3], edges_out.
 * Query with NULL arrays for *edges. */
int eddy_get_edge_list(const eddy_ctx *ctx, int set_id, int *edges, int32_t *nodes,
                       int32_t *epn, int32_t *edges_out);

/* ------------------------------------------------ stage-level entry points
 * Direct access to the hot path for one gene set and explicit labellings,
 * without the permutation driver: the GPU counterparts of the reference's
 * per-permutation kernel sequence (run2 .. run4 + normalisation + JS).
 * labels: R x samples.  js[R], unique[R]. */
int eddy_run_labellings(eddy_ctx *ctx, int set_id, const uint8_t *labels, int R, double *js,
                        int32_t *unique);

/* Edge decisions of all S networks of one labelling, S x c bytes (the
 * reference's out23 array after run2/run2Scalable, kernel1.cu:426-431). */
int eddy_debug_edges(eddy_ctx *ctx, int set_id, const uint8_t *labels, uint8_t *edges);

/* Details of one labelling: unique network ids [S], capped parent counts
 * [S*g] and lists [S*g*mpk] (-1 padded), node-summed BDeu [2*S] and
 * normalised likelihoods [2*S] of the unique networks (class 0 block then
 * class 1, each S long); *U receives the unique count, *js the JS. */
int eddy_debug_unit(eddy_ctx *ctx, int set_id, const uint8_t *labels, int mpk, int *U,
                    double *js, int32_t *ids, int32_t *counts, int32_t *parents, double *dist,
                    double *lval);

/* Batched hot path: iterations [first, first+count) of a set under the
 * COUNTER stream (labellings generated on the device) or the EXTERNAL
 * labellings; the set's data stays resident between calls.  js[count],
 * unique[count].  The GLIBC stream is sequential and only runs in eddy_run. */
int eddy_run_permutations(eddy_ctx *ctx, int set_id, int first, int count, double *js,
                          int32_t *unique);

/* Use the caller's CUDA stream (a cudaStream_t on the context's device) for
 * every copy and kernel; NULL returns to the context's own stream. */
int eddy_set_stream(eddy_ctx *ctx, void *stream);

/* Drops every gene set and its results (the matrix stays loaded). */
int eddy_clear_sets(eddy_ctx *ctx);

/* ------------------------------------------------------------ output files
 * The reference's per-set files, byte for byte (routines.cu:217-492).
 * genes: g NUL-terminated names of the set's (adjusted) genes. */
/* <set>_Networks.txt: the iteration-0 unique networks (writeNetworkFile,
 * routines.cu:240-306); epn/nodes/edges/ids as eddy_get_networks returns. */
int eddy_write_networks(const char *path, const char *input, const char *cls, const char *set,
                        int U, const int32_t *epn, const char *const *genes, int g,
                        const int32_t *nodes, const int32_t *edges, int total_edges,
                        const int32_t *ids);
/* <set>_BDEU_SCORES.txt: the normalised likelihoods (writeBdeuScores,
 * routines.cu:217-238); lval[2*U]. */
int eddy_write_bdeu(const char *path, const char *input, const char *cls, const char *set,
                    const char *class1, const char *class2, int U, const double *lval);
/* <set>_EdgeList.txt: class / Both / Neither-PRIOR edges of the uncapped
 * full-data networks (writeEdgeListFile, routines.cu:308-492); nodes[2*g],
 * edges, epn[3] as eddy_get_edge_list returns; prior g x g or NULL. */
int eddy_write_edge_list(const char *path, const char *const *genes, int g, const int32_t *nodes,
                         const int32_t *edges, const int32_t *epn, const uint8_t *prior,
                         const char *class1, const char *class2);

/* ------------------------------------------------- no-allocation entry point
 * No counterpart in the reference.  One labelling of one gene set (the
 * S-network inference, BDeu, normalisation and JS of eddy_run_labellings)
 * for callers that may not allocate GPU memory: programs embedding EDDY in a
 * host application that owns every byte of device memory through its own
 * pool, or pipelines that must avoid the device-wide synchronisation
 * cudaFree can cause.  Inputs and results are HOST buffers; every
 * intermediate lives in one fixed array (~2.6 MB) compiled into the library,
 * held by each GPU that loads it until the process exits.  No cudaMalloc,
 * cudaFree or allocating library call is made.
 * Limits: 2 <= g <= 64 genes, 2 <= n <= 2048 samples (EDDY_ERR_CAPACITY
 * beyond).  vals: g x n int8, labels: n entries 0/1 (both classes present),
 * prior: g x g 0/1 or NULL, stream: a cudaStream_t of the current device or
 * NULL.  *js and *unique receive the JS (NaN when U == 1) and U.
 * The first call on a device looks up the array's device address (call it
 * once before any stream capture).  Calls share the array: one process's
 * calls are serialised by a lock and each call, also one that fails after
 * queueing work, ends with a stream synchronisation; GPU work that
 * overlaps a call from elsewhere races. */
int eddy_unit_noalloc(const eddy_opts *opts, const int8_t *vals, int g, int n,
                      const uint8_t *labels, const uint8_t *prior, void *stream, double *js,
                      int32_t *unique);

/* Decision-path counters of the last batch run: [0] tables re-evaluated in
 * FP64 (guard-band rechecks), [1] (pair, class) tables decided, [2] of them
 * whose ten leave-one-out tables the filter settled at once, [3] duplicate
 * networks; *variant: the contingency-kernel choice of the last batch (0-4:
 * tile shapes in the 9-cell layout, 5-9: the same in the 4-cell layout of
 * sets without missing values; -1: none). */
int eddy_last_stats(const eddy_ctx *ctx, uint64_t *stats4, int *variant);

/* Name, SM count and compute capability of a device (the reference's
 * device banner, main.cu:28-56, without the fields CUDA 13 removed). */
int eddy_device_info(int device, char *name, int name_len, int *sms, int *cc_major,
                     int *cc_minor);

/* Timing of the last eddy_run / eddy_run_labellings, device side (CUDA
 * events around the kernels) in milliseconds, and the number of kernel
 * launches it made. */
int eddy_last_timing(const eddy_ctx *ctx, double *ms_kernels, double *ms_pairs, double *ms_units,
                     long long *launches);

/* The same device time split by kernel, in milliseconds: ms4[0] the
 * operand and contraction kernels (k_operands, k_pairs_mma; k_pairs on the
 * popcount path), ms4[1] the general-path and exact decisions (k_general,
 * k_exact), ms4[2] the network kernel (k_units), ms4[3] normalisation and
 * JS (k_js).  ms4[0] + ms4[1] = ms_pairs, ms4[2] + ms4[3] = ms_units. */
int eddy_last_stage_timing(const eddy_ctx *ctx, double *ms4);

#ifdef __cplusplus
}
#endif
#endif
