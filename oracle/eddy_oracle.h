/*
 * eddy_oracle.h -- CPU restatement of the EDDY per-class dependency-network
 * inference and label-permutation test of skimlab/eddy-gpu.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle: the parity tests,
 * the smoke check and the CPU baseline leg of bench.py call it.  The product
 * (libeddy_gpu.so and the eddy CLI) never links or calls it.
 *
 * Every stage is restated from the reference sources (paths are relative to
 * the reference project root) in plain C with FP64 arithmetic, brute force,
 * one network at a time, so that it does not share any algorithmic shortcut
 * with the GPU path it checks:
 *   K1  kernel1.cu:76-203, 338-431   leave-one-out 3x3 tables, Yates, dof,
 *                                     chi-square, AS 147, Bonferroni, priors
 *   K2  kernel2.cu:114-142           capped edge count per network
 *   K3  kernel3.cu:41-165            capped parent lists (pNodes / pEdges)
 *   K4  kernel4.cu:5-84, routines.cu:25-40, main.cu:1060-1121
 *                                     first-occurrence network uniqueness
 *   --  routines.cu:63-115           unique-network compaction
 *   K5  kernel5.cu:4-257             BDeu score (N'=4, 3-parent cap)
 *   --  main.cu:1293-1435, routines.cu:42-60   likelihoods and JS divergence
 *   --  main.cu:1465-1502, routines.cu:494-508 beta fit and pDDN
 *   --  main.cu:538-573              glibc rand() label permutation
 *
 * Parity of this restatement is pinned by tests/golden (outputs of the
 * reference's own kernel and host-routine sources, compiled and run on the
 * CPU by oracle/ref/) and by known-answer tests (mpmath, scipy).
 */
#ifndef EDDY_ORACLE_H
#define EDDY_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int max_parents;          /* -mp (>=1) */
  double alpha_edge;        /* -pE / derived from -t */
  double alpha_edge_prior;  /* 1-(1-alpha_edge)*pw^(1/lambda) */
  int bonferroni;           /* 1 unless -rawp */
} or_params;

/* AS 147 lower regularised incomplete gamma, kernel1.cu:10-74. */
double or_gammds(double x, double p);

/* One 3x3 table -> chi-square and dof, kernel1.cu:121-201.
 * tally[r*3+c]: r = state of the row (larger-index) gene, c = column gene. */
double or_chisq(const int *tally, int *dof);

/* Edge decision for one table, kernel1.cu:419-431. */
int or_edge_decision(double chi, int dof, int num_genes, int prior,
                     const or_params *p);

/* K1 for all networks of one labelling.
 *   dA: g x nA int8 (class-1 samples, original order), dB: g x nB.
 *   prior: g x g 0/1 (may be NULL).
 *   edges_out: S x c bytes, S = nA+nB+2, c = g(g-1)/2 (pair p <-> row>col
 *   in row-major lower-triangular order, main.cu:615-632).
 *   ppn_out (2g) / stf_out (6g): observed-state counts/flags, may be NULL. */
void or_k1_edges(int g, int nA, int nB, const int8_t *dA, const int8_t *dB,
                 const uint8_t *prior, const or_params *p, uint8_t *edges_out,
                 int *ppn_out, int *stf_out);

/* K2+K3 for `nets` networks of edge bits: capped parent lists.
 *   pnodes: nets x g, edges_pn: nets+1 (exclusive prefix), pedges: total.
 *   Returns total edges; pedges may be NULL (then only counts). */
int or_parents(int nets, int g, const uint8_t *edges, int max_parents,
               int *pnodes, int *edges_pn, int *pedges);

/* K4 + sweep: unique[s] = 1 iff no earlier network is identical. Returns U. */
int or_unique(int nets, int g, const int *pnodes, const int *edges_pn,
              const int *pedges, uint8_t *unique);

/* K5: BDeu of one node given its parent list (first up to 3 are used).
 *   data: g x ns int8 of the class; ppn/stf of this class (g and 3g). */
double or_bdeu_node(int g, int ns, const int8_t *data, const int *ppn,
                    const int *stf, int node, int nparents, const int *parents);

/* Likelihood normalisation of one class, main.cu:1302-1404. */
void or_normalise(int U, const double *dist, double *lval);

/* JS divergence (already divided by ln 2), main.cu:1406-1428. */
double or_js(int U, const double *lvalA, const double *lvalB);

/* Full per-labelling computation (one unit = one gene set x one labelling).
 * Optional outputs may be NULL. Array capacities: edges S*c, pnodes S*g,
 * edges_pn S+1, unique_ids S, uni_nodes S*g, uni_edges S*g*min(mp,g),
 * uni_epn S+1, out5 2*S*g, lval 2*S. */
typedef struct {
  double js;       /* JS/ln2 (NaN when U==1) */
  int U;           /* unique networks */
  int S;           /* networks */
  int total_edges; /* sum of capped edges over the S networks */
  int uni_edges_total;
} or_unit_result;

void or_unit(int g, int n, const int8_t *data /* g x n */,
             const uint8_t *labels /* n, 0 = class 1, 1 = class 2 */,
             const uint8_t *prior, const or_params *p, or_unit_result *res,
             uint8_t *edges, int *unique_ids, int *uni_nodes, int *uni_edges,
             int *uni_epn, double *out5, double *lval);

/* Many labellings of one gene set in parallel (OpenMP over labellings).
 * labels: R x n. js/U: R. Returns 0. */
int or_units(int g, int n, const int8_t *data, int R, const uint8_t *labels,
             const uint8_t *prior, const or_params *p, double *js, int *U,
             int threads);

/* Label permutations exactly as main.cu:538-573, consuming libc rand().
 *   reset != 0 calls srand(1) first (glibc: identical to never seeding).
 *   labels0: initial labels (n). out: R x n; row r is iteration first+r
 *   (iteration 0 keeps labels0 but still consumes its draws). */
void or_glibc_labels(int n, int n_class1, const uint8_t *labels0, int R,
                     uint8_t *out, int reset, int first);

/* Number of libc rand() calls one permutation consumes (for stream tests). */
long long or_glibc_rand_calls(void);

/* Counter-based labelling: the key of sample s is word s mod 4 of
 * Philox-4x32-10 keyed by seed with counter (s / 4, perm, set, 0); the
 * n_class1 samples with the smallest (key, index) get label 0.  perm 0 =
 * labels0. */
void or_counter_labels(uint64_t seed, int set_id, int n, int n_class1,
                       const uint8_t *labels0, int R, uint8_t *out);
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                      uint32_t out[4]);

/* Regularised incomplete beta complement I_{1-x}(b,a) = 1 - I_x(a,b)
 * (Lentz continued fraction), replaces boost::math::ibetac. */
double or_ibetac(double a, double b, double x);

/* Beta fit of the JS values and pDDN, main.cu:1488-1497.
 * Returns 0, or -1 when alpha/beta are not positive finite. */
int or_pddn(int R, const double *js, double *alpha, double *beta,
            double *pddn);

#ifdef __cplusplus
}
#endif
#endif
