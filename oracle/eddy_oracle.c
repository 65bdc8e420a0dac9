/*
 * eddy_oracle.c -- CPU restatement of the EDDY hot path of skimlab/eddy-gpu.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  See eddy_oracle.h for the map
 * from each function to the reference file:line it restates.  FP64 and the
 * reference's operation order are kept wherever the reference's own result
 * depends on it (chi-square terms, AS 147 series, BDeu sums, normalisation,
 * JS), so that this file reproduces the reference bit for bit on the CPU
 * up to the libm (glibc vs CUDA) differences of lgamma/log/exp.
 */
#include "eddy_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ K1 */

/* AS 147 series for the lower regularised incomplete gamma,
 * kernel1.cu:10-74 (same code as the host twin routines.cu:117-184). */
double or_gammds(double x, double p) {
  const double e = 1.0e-09;
  const double uflo = 1.0e-37;
  if (x <= 0.0) return 0.0;
  if (p <= 0.0) return 0.0;
  double arg = p * log(x) - lgamma(p + 1.0) - x;
  if (arg < log(uflo)) return 0.0;
  double f = exp(arg);
  if (f == 0.0) return 0.0;
  double c = 1.0, value = 1.0, a = p;
  for (;;) {
    a = a + 1.0;
    c = c * x / a;
    value = value + c;
    if (c <= e * value) break;
  }
  return value * f;
}

/* kernel1.cu:121-201: marginals, expected counts, Yates flag, chi-square
 * with the |o-e|-yates term squared, and the dof rule. */
double or_chisq(const int *tally, int *dof) {
  int ex[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int c = 0; c < 3; c++) {
    for (int c1 = 0; c1 < 3; c1++) ex[c1] += tally[c * 3 + c1]; /* columns */
    for (int b = 0; b < 3; b++) ex[3 + b] += tally[b * 3 + c];  /* rows */
  }
  ex[6] = ex[0] + ex[1] + ex[2];
  double divisor = (double)ex[6];
  double expected[9];
  for (int c = 0; c < 3; c++)
    for (int c1 = 0; c1 < 3; c1++)
      expected[c * 3 + c1] = ((double)ex[c1] * (double)ex[c + 3] / divisor);
  double yates = 0.0;
  int flag = 0;
  for (int c = 0; c < 3 && !flag; c++)
    for (int c1 = 0; c1 < 3; c1++)
      if ((expected[c * 3 + c1] < 5) && (ex[c1] && ex[c + 3])) {
        yates = 0.5;
        flag = 1;
        break;
      }
  double chi = 0.0;
  int dofn = 0, dofm = 0;
  for (int ii = 0; ii < 3; ii++) {
    if (ex[ii] == 0) dofm++;
    if (ex[ii + 3] == 0) dofn++;
    for (int jj = 0; jj < 3; jj++)
      if ((ex[jj] * ex[ii + 3]) != 0)
        chi += pow(fabs((double)tally[ii * 3 + jj] - expected[ii * 3 + jj]) -
                       yates,
                   2) /
               expected[ii * 3 + jj];
  }
  *dof = ((3 - dofm) - 1) * ((3 - dofn) - 1);
  return chi;
}

/* kernel1.cu:419-431 (run2) / 462-475 (run2Scalable). */
int or_edge_decision(double chi, int dof, int num_genes, int prior,
                     const or_params *p) {
  double ev = 1.0 - or_gammds(chi / 2.0, ((double)dof) / 2.0);
  if (p->bonferroni) {
    double m = ev * (double)(((num_genes - 1) * num_genes) / 2);
    ev = (1.0 < m) ? 1.0 : m; /* CUDA min(1.0, x) */
  }
  return (ev < p->alpha_edge || (prior == 1 && ev < p->alpha_edge_prior)) ? 1
                                                                          : 0;
}

static inline int state_of(int8_t v) {
  return v == -1 ? 0 : v == 0 ? 1 : v == 1 ? 2 : 3; /* 3 = not counted */
}

/* kernel1.cu:338-387: observed-state count (ppn) and flags (stf). */
static void states_of(int g, int ns, const int8_t *d, int *ppn, int *stf) {
  for (int i = 0; i < g; i++) {
    unsigned cnt[3] = {0, 0, 0};
    for (int s = 0; s < ns; s++) {
      int st = state_of(d[(size_t)i * ns + s]);
      if (st < 3) cnt[st]++;
    }
    int r = 3;
    for (int k = 0; k < 3; k++) {
      stf[i * 3 + k] = 1;
      if (cnt[k] == 0) {
        stf[i * 3 + k] = 0;
        r--;
      }
    }
    ppn[i] = r;
  }
}

/* K1 over all S networks: network 0 = class 1 all samples, 1..nA drop class-1
 * sample s-1; nA+1..nA+nB drop class-2 sample s-nA-1; S-1 = class 2 all
 * (kernel1.cu:85-88, 412-416).  Brute-force tally per (network, pair). */
void or_k1_edges(int g, int nA, int nB, const int8_t *dA, const int8_t *dB,
                 const uint8_t *prior, const or_params *p, uint8_t *edges_out,
                 int *ppn_out, int *stf_out) {
  const int S = nA + nB + 2;
  const long c = (long)g * (g - 1) / 2;
  /* state-index copies so the inner loop is a table increment */
  uint8_t *sA = (uint8_t *)malloc((size_t)g * (nA > 0 ? nA : 1));
  uint8_t *sB = (uint8_t *)malloc((size_t)g * (nB > 0 ? nB : 1));
  for (long i = 0; i < (long)g * nA; i++) sA[i] = (uint8_t)state_of(dA[i]);
  for (long i = 0; i < (long)g * nB; i++) sB[i] = (uint8_t)state_of(dB[i]);
#pragma omp parallel for schedule(dynamic, 4)
  for (int s = 0; s < S; s++) {
    const uint8_t *d;
    int len, skip;
    if (s <= nA) {
      d = sA;
      len = nA;
      skip = s;
    } else {
      d = sB;
      len = nB;
      skip = s - nA;
    }
    long pidx = 0;
    for (int row = 1; row < g; row++) {
      const uint8_t *xr = d + (size_t)row * len;
      for (int col = 0; col < row; col++, pidx++) {
        const uint8_t *xc = d + (size_t)col * len;
        int t16[16] = {0};
        for (int k = 0; k < len; k++) {
          if (skip != 0 && k == skip - 1) continue;
          t16[xr[k] * 4 + xc[k]]++;
        }
        int tally[9];
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++) tally[a * 3 + b] = t16[a * 4 + b];
        int dof;
        double chi = or_chisq(tally, &dof);
        int pr = prior ? prior[(size_t)row * g + col] : 0;
        edges_out[(size_t)s * c + pidx] =
            (uint8_t)or_edge_decision(chi, dof, g, pr, p);
      }
    }
  }
  if (ppn_out && stf_out) {
    states_of(g, nA, dA, ppn_out, stf_out);
    states_of(g, nB, dB, ppn_out + g, stf_out + 3 * g);
  }
  free(sA);
  free(sB);
}

/* ----------------------------------------------------------- K2 + K3 */

/* kernel2.cu:114-142 (per-network capped edge count), host prefix
 * main.cu:849-858, kernel3.cu:41-165 (nodeMaker, nodeArrayParentCap,
 * edgeCounter) restated serially per network. */
int or_parents(int nets, int g, const uint8_t *edges, int max_parents,
               int *pnodes, int *edges_pn, int *pedges) {
  const long c = (long)g * (g - 1) / 2;
  edges_pn[0] = 0;
  for (int s = 0; s < nets; s++) {
    const uint8_t *e = edges + (size_t)s * c;
    int sum = 0;
    for (int i = 1; i < g; i++) {
      long start = (long)(i - 1) * i / 2, stop = (long)i * (i + 1) / 2;
      int ns = 0;
      for (long j = start; j < stop; j++) ns += (e[j] == 1);
      if (ns > max_parents) ns = max_parents;
      sum += ns;
    }
    edges_pn[s + 1] = edges_pn[s] + sum;
  }
  for (int s = 0; s < nets; s++) {
    const uint8_t *e = edges + (size_t)s * c;
    int *na = pnodes + (size_t)s * g;
    /* nodeMaker: uncapped prefix over rows 1..t-1 */
    na[0] = 0;
    for (int t = 1; t < g; t++) {
      long lim = (long)(t - 1) * t / 2; /* searcher[t-1] */
      int sum = 0;
      for (long i = 0; i < lim; i++) sum += (e[i] == 1);
      na[t] = sum;
    }
    /* nodeArrayParentCap, executed by one thread in the reference */
    for (int i = 0; i < g - 1; i++) {
      if ((na[i + 1] - na[i]) > max_parents) {
        int temp = na[i + 1];
        na[i + 1] = na[i] + max_parents;
        int decrement = temp - na[i + 1];
        for (int j = i + 2; j <= g - 1; j++) na[j] -= decrement;
      }
    }
    if (pedges) {
      for (int t = 1; t < g; t++) {
        int place = edges_pn[s] + na[t];
        int pos = 0, pc = 0;
        long start = (long)(t - 1) * t / 2, stop = (long)t * (t + 1) / 2;
        for (long i = start; i < stop; i++) {
          if (pc >= max_parents) break;
          if (e[i] == 1) {
            pedges[place++] = pos;
            pc++;
          }
          pos++;
        }
      }
    }
  }
  return edges_pn[nets];
}

/* --------------------------------------------------------------- K4 */

static int nets_equal(int g, const int *pnodes, const int *edges_pn,
                      const int *pedges, int a, int b) {
  /* kernel4.cu:55-70: nodes first, then edge slices */
  if (memcmp(pnodes + (size_t)a * g, pnodes + (size_t)b * g,
             sizeof(int) * g) != 0)
    return 0;
  int la = edges_pn[a + 1] - edges_pn[a], lb = edges_pn[b + 1] - edges_pn[b];
  if (la != lb) return 0;
  return memcmp(pedges + edges_pn[a], pedges + edges_pn[b],
                sizeof(int) * la) == 0;
}

/* run25 + the first-occurrence sweep of main.cu:1060-1121: network a is a
 * duplicate iff it equals some b < a.  Comparing against earlier unique
 * networks only is equivalent (equality is transitive). */
int or_unique(int nets, int g, const int *pnodes, const int *edges_pn,
              const int *pedges, uint8_t *unique) {
  int *reps = (int *)malloc(sizeof(int) * (nets > 0 ? nets : 1));
  int U = 0;
  for (int a = 0; a < nets; a++) {
    int dup = 0;
    for (int k = 0; k < U && !dup; k++)
      dup = nets_equal(g, pnodes, edges_pn, pedges, a, reps[k]);
    unique[a] = (uint8_t)!dup;
    if (!dup) reps[U++] = a;
  }
  free(reps);
  return U;
}

/* --------------------------------------------------------------- K5 */

/* kernel5.cu:4-236 (njLoop + bDeu3) for one (class, network, node).  The
 * counts N_ijk of kernel5.cu:30-110 (parent configuration j in mixed radix
 * over the parents' observed states, parent 1 fastest; child state k among
 * the node's observed states) are tallied in one pass over the samples: a
 * sample whose node or parent value is not an observed state (a value
 * outside -1/0/1) matches no configuration, as in the reference's scan.
 * The lgamma terms are then summed in the reference's order (j, then k). */
double or_bdeu_node(int g, int ns, const int8_t *data, const int *ppn,
                    const int *stf, int node, int nparents,
                    const int *parents) {
  (void)g;
  int noParents = 1 + nparents;
  if (noParents > 4) noParents = 4;
  int pa[4];
  pa[0] = node;
  for (int k = 0; k < noParents - 1; k++) pa[k + 1] = parents[k];
  /* rank of each value -1/0/1 among a gene's observed states (-1 = none) */
  int rank[4][3];
  for (int i = 0; i < noParents; i++) {
    int sc = 0;
    for (int st = 0; st < 3; st++) rank[i][st] = stf[pa[i] * 3 + st] != 0 ? sc++ : -1;
  }
  const int r = ppn[node];
  int q = 1;
  for (int i = 1; i < noParents; i++) q *= ppn[pa[i]];
  /* q <= 27 and r <= 3 (three observed states at most) */
  int nijk[27][3];
  memset(nijk, 0, sizeof nijk);
  for (int s = 0; s < ns; s++) {
    const int v0 = data[(size_t)node * ns + s];
    if (v0 < -1 || v0 > 1 || rank[0][v0 + 1] < 0) continue;
    int j = 0, div = 1, ok = 1;
    for (int i = 1; i < noParents && ok; i++) {
      const int v = data[(size_t)pa[i] * ns + s];
      if (v < -1 || v > 1 || rank[i][v + 1] < 0) {
        ok = 0;
        break;
      }
      j += rank[i][v + 1] * div;
      div *= ppn[pa[i]];
    }
    if (ok && rank[0][v0 + 1] < r) nijk[j][rank[0][v0 + 1]]++;
  }
  const int nPrime = 4;
  double sum2 = 0.0;
  for (int j = 0; j < q; j++) {
    int nij = 0;
    for (int k = 0; k < r; k++) nij += nijk[j][k];
    double sum1 = 0.0;
    for (int k = 0; k < r; k++)
      sum1 += lgamma((double)nijk[j][k] + (double)nPrime / (double)(q * r)) -
              lgamma((double)nPrime / (double)(q * r));
    sum2 += lgamma((double)nPrime / (double)q) -
            lgamma((double)nij + (double)nPrime / (double)q) + sum1;
  }
  return sum2;
}

/* ------------------------------------------------ normalisation + JS */

/* main.cu:1302-1404 for one class: the node-summed scores of the U unique
 * networks -> normalised likelihoods. */
void or_normalise(int U, const double *dist, double *lval) {
  double scoreSum = 0, mn = dist[0], mx = dist[0];
  for (int j = 0; j < U; j++) {
    scoreSum += dist[j];
    if (dist[j] > mx) mx = dist[j];
    if (dist[j] < mn) mn = dist[j];
  }
  double inAlpha = -1 * (scoreSum / U);
  double probScale = (10) / (mx - mn);
  double *lik = (double *)malloc(sizeof(double) * U);
  double *inf = (double *)malloc(sizeof(double) * U);
  double nonInf = 0, likeliSum = 0;
  for (int m = 0; m < U; m++) {
    double adj = (dist[m] + inAlpha) * probScale;
    lik[m] = exp(adj);
    nonInf += lik[m];
    inf[m] = 0.0;
    if (lik[m] >= INFINITY || lik[m] <= -INFINITY) {
      inf[m] = 1.0;
      likeliSum++;
    }
  }
  for (int m = 0; m < U; m++)
    lval[m] = (likeliSum == 0) ? lik[m] / nonInf : inf[m] / likeliSum;
  free(lik);
  free(inf);
}

/* routines.cu:42-60 (kool) */
static double kool(const double *P, const double *Q, int off, int cnt) {
  double D = 0;
  for (int i = 0; i < cnt; i++) {
    if (Q[i] == 0) continue;
    if (P[i + off] == 0) continue;
    D += P[i + off] * log(P[i + off] / Q[i]);
  }
  return D;
}

/* main.cu:1406-1428 */
double or_js(int U, const double *lvalA, const double *lvalB) {
  double *l = (double *)malloc(sizeof(double) * 2 * U);
  double *sea = (double *)malloc(sizeof(double) * U);
  memcpy(l, lvalA, sizeof(double) * U);
  memcpy(l + U, lvalB, sizeof(double) * U);
  for (int i = 0; i < U; i++) sea[i] = (l[i] + l[i + U]) / 2;
  double js = kool(l, sea, 0, U) / 2 + kool(l, sea, U, U) / 2;
  free(l);
  free(sea);
  return js / log(2.0);
}

/* ------------------------------------------------------------- unit */

void or_unit(int g, int n, const int8_t *data, const uint8_t *labels,
             const uint8_t *prior, const or_params *p, or_unit_result *res,
             uint8_t *edges_o, int *unique_ids, int *uni_nodes_o,
             int *uni_edges_o, int *uni_epn_o, double *out5_o,
             double *lval_o) {
  /* class split, main.cu:575-605 (sample order kept) */
  int nA = 0, nB = 0;
  for (int s = 0; s < n; s++) (labels[s] == 0) ? nA++ : nB++;
  int8_t *dA = (int8_t *)malloc((size_t)g * (nA ? nA : 1));
  int8_t *dB = (int8_t *)malloc((size_t)g * (nB ? nB : 1));
  for (int i = 0; i < g; i++) {
    int ja = 0, jb = 0;
    for (int s = 0; s < n; s++) {
      int8_t v = data[(size_t)i * n + s];
      if (labels[s] == 0)
        dA[(size_t)i * nA + ja++] = v;
      else
        dB[(size_t)i * nB + jb++] = v;
    }
  }
  const int S = nA + nB + 2;
  const long c = (long)g * (g - 1) / 2;
  uint8_t *edges = (uint8_t *)malloc((size_t)S * (c ? c : 1));
  int *ppn = (int *)malloc(sizeof(int) * 2 * g);
  int *stf = (int *)malloc(sizeof(int) * 6 * g);
  or_k1_edges(g, nA, nB, dA, dB, prior, p, edges, ppn, stf);
  if (edges_o) memcpy(edges_o, edges, (size_t)S * c);

  int *pnodes = (int *)malloc(sizeof(int) * (size_t)S * g);
  int *epn = (int *)malloc(sizeof(int) * (S + 1));
  or_parents(S, g, edges, p->max_parents, pnodes, epn, NULL);
  int E = epn[S];
  int *pedges = (int *)malloc(sizeof(int) * (E ? E : 1));
  or_parents(S, g, edges, p->max_parents, pnodes, epn, pedges);

  uint8_t *uq = (uint8_t *)malloc(S);
  int U = or_unique(S, g, pnodes, epn, pedges, uq);

  /* structureUnique, routines.cu:63-115 */
  int *un = (int *)malloc(sizeof(int) * (size_t)U * g);
  int *uepn = (int *)malloc(sizeof(int) * (U + 1));
  int ue_tot = 0;
  for (int s = 0; s < S; s++)
    if (uq[s]) ue_tot += epn[s + 1] - epn[s];
  int *ue = (int *)malloc(sizeof(int) * (ue_tot ? ue_tot : 1));
  {
    int k = 0, pos = 0;
    uepn[0] = 0;
    for (int s = 0; s < S; s++) {
      if (!uq[s]) continue;
      if (unique_ids) unique_ids[k] = s;
      int ne = epn[s + 1] - epn[s];
      memcpy(ue + pos, pedges + epn[s], sizeof(int) * ne);
      pos += ne;
      memcpy(un + (size_t)k * g, pnodes + (size_t)s * g, sizeof(int) * g);
      uepn[k + 1] = uepn[k] + ne;
      k++;
    }
  }

  /* K5 per class / unique network / node, run4 (kernel5.cu:237-257) */
  double *out5 = (double *)malloc(sizeof(double) * 2 * (size_t)U * g);
#pragma omp parallel for schedule(dynamic, 8)
  for (int cu = 0; cu < 2 * U; cu++) {
    const int cls = cu / U, u = cu % U;
    const int8_t *d = cls ? dB : dA;
    int ns = cls ? nB : nA;
    {
      int Eu = uepn[u + 1] - uepn[u];
      for (int t = 0; t < g; t++) {
        int np = (t == g - 1) ? Eu - un[(size_t)u * g + t]
                              : un[(size_t)u * g + t + 1] - un[(size_t)u * g + t];
        const int *pl = ue + uepn[u] + un[(size_t)u * g + t];
        out5[((size_t)cls * U + u) * g + t] =
            or_bdeu_node(g, ns, d, ppn + cls * g, stf + cls * 3 * g, t, np,
                         pl);
      }
    }
  }

  /* dist + normalisation + JS, main.cu:1293-1428 */
  double *dist = (double *)malloc(sizeof(double) * U);
  double *lval = (double *)malloc(sizeof(double) * 2 * U);
  for (int cls = 0; cls < 2; cls++) {
    for (int u = 0; u < U; u++) dist[u] = 0.0;
    for (long i = 0; i < (long)U * g; i++)
      dist[i / g] += out5[(size_t)cls * U * g + i];
    or_normalise(U, dist, lval + (size_t)cls * U);
  }
  double js = or_js(U, lval, lval + U);

  res->js = js;
  res->U = U;
  res->S = S;
  res->total_edges = E;
  res->uni_edges_total = ue_tot;
  if (uni_nodes_o) memcpy(uni_nodes_o, un, sizeof(int) * (size_t)U * g);
  if (uni_edges_o) memcpy(uni_edges_o, ue, sizeof(int) * ue_tot);
  if (uni_epn_o) memcpy(uni_epn_o, uepn, sizeof(int) * (U + 1));
  if (out5_o) memcpy(out5_o, out5, sizeof(double) * 2 * (size_t)U * g);
  if (lval_o) memcpy(lval_o, lval, sizeof(double) * 2 * U);

  free(dA); free(dB); free(edges); free(ppn); free(stf); free(pnodes);
  free(epn); free(pedges); free(uq); free(un); free(uepn); free(ue);
  free(out5); free(dist); free(lval);
}

int or_units(int g, int n, const int8_t *data, int R, const uint8_t *labels,
             const uint8_t *prior, const or_params *p, double *js, int *U,
             int threads) {
#ifdef _OPENMP
  int prev = omp_get_max_threads();
  if (threads > 0) omp_set_num_threads(threads);
  /* parallel over labellings (one level: loops inside a unit then run
   * serially), or inside each unit when labellings are fewer than threads */
  int nested = omp_get_max_active_levels();
  omp_set_max_active_levels(1);
#endif
  if (R >= omp_get_max_threads()) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int r = 0; r < R; r++) {
      or_unit_result res;
      or_unit(g, n, data, labels + (size_t)r * n, prior, p, &res, NULL, NULL,
              NULL, NULL, NULL, NULL, NULL);
      js[r] = res.js;
      U[r] = res.U;
    }
  } else {
    /* fewer labellings than threads: one at a time, each unit's network
     * and BDeu loops parallel (the results do not depend on the split) */
    for (int r = 0; r < R; r++) {
      or_unit_result res;
      or_unit(g, n, data, labels + (size_t)r * n, prior, p, &res, NULL, NULL,
              NULL, NULL, NULL, NULL, NULL);
      js[r] = res.js;
      U[r] = res.U;
    }
  }
#ifdef _OPENMP
  omp_set_max_active_levels(nested);
  omp_set_num_threads(prev);
#endif
  return 0;
}

/* ---------------------------------------------------- permutations */

static long long g_rand_calls = 0;
long long or_glibc_rand_calls(void) { return g_rand_calls; }

/* main.cu:538-573: n draws that are overwritten, then a rejection loop that
 * keeps the first n distinct values of rand()%n; permutation k>0 assigns
 * label 0 to the first n_class1 of them. */
void or_glibc_labels(int n, int n_class1, const uint8_t *labels0, int R,
                     uint8_t *out, int reset, int first) {
  if (reset) srand(1);
  uint8_t *cur = (uint8_t *)malloc(n);
  uint8_t *seen = (uint8_t *)malloc(n);
  int *order = (int *)malloc(sizeof(int) * n);
  memcpy(cur, labels0, n);
  for (int perm = 0; perm < R; perm++) {
    for (int c = 0; c < n; c++) {
      (void)(rand() % n);
      g_rand_calls++;
    }
    memset(seen, 0, n);
    int cnt = 0;
    while (cnt < n) {
      int r = rand() % n;
      g_rand_calls++;
      if (!seen[r]) {
        seen[r] = 1;
        order[cnt++] = r;
      }
    }
    if (first + perm > 0) {
      for (int k = 0; k < n_class1; k++) cur[order[k]] = 0;
      for (int k = n_class1; k < n; k++) cur[order[k]] = 1;
    }
    memcpy(out + (size_t)perm * n, cur, n);
  }
  free(cur);
  free(seen);
  free(order);
}

/* Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
void or_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2],
                      uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

typedef struct { uint32_t key; int idx; } kv_t;
static int kv_cmp(const void *a, const void *b) {
  const kv_t *x = (const kv_t *)a, *y = (const kv_t *)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

void or_counter_labels(uint64_t seed, int set_id, int n, int n_class1,
                       const uint8_t *labels0, int R, uint8_t *out) {
  kv_t *kv = (kv_t *)malloc(sizeof(kv_t) * n);
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  memcpy(out, labels0, n);
  for (int perm = 1; perm < R; perm++) {
    for (int s = 0; s < n; s += 4) {
      uint32_t ctr[4] = {(uint32_t)(s / 4), (uint32_t)perm, (uint32_t)set_id, 0u};
      uint32_t o[4];
      or_philox4x32_10(ctr, key, o);
      for (int j = 0; j < 4 && s + j < n; j++) {
        kv[s + j].key = o[j];
        kv[s + j].idx = s + j;
      }
    }
    qsort(kv, n, sizeof(kv_t), kv_cmp);
    uint8_t *row = out + (size_t)perm * n;
    for (int k = 0; k < n; k++) row[kv[k].idx] = (uint8_t)(k < n_class1 ? 0 : 1);
  }
  free(kv);
}

/* ------------------------------------------------- ibetac and pDDN */

/* Continued fraction for I_x(a,b), modified Lentz evaluation (Lentz 1976;
 * the even/odd coefficients of the incomplete-beta fraction as in Press et
 * al., Numerical Recipes, section 6.4). */
static double betacf(double a, double b, double x) {
  const int MAXIT = 100000;
  const double EPS = 1e-16, FPMIN = 1e-300;
  double qab = a + b, qap = a + 1.0, qam = a - 1.0;
  double c = 1.0, d = 1.0 - qab * x / qap;
  if (fabs(d) < FPMIN) d = FPMIN;
  d = 1.0 / d;
  double h = d;
  for (int m = 1; m <= MAXIT; m++) {
    int m2 = 2 * m;
    double aa = m * (b - m) * x / ((qam + m2) * (a + m2));
    d = 1.0 + aa * d;
    if (fabs(d) < FPMIN) d = FPMIN;
    c = 1.0 + aa / c;
    if (fabs(c) < FPMIN) c = FPMIN;
    d = 1.0 / d;
    h *= d * c;
    aa = -(a + m) * (qab + m) * x / ((a + m2) * (qap + m2));
    d = 1.0 + aa * d;
    if (fabs(d) < FPMIN) d = FPMIN;
    c = 1.0 + aa / c;
    if (fabs(c) < FPMIN) c = FPMIN;
    d = 1.0 / d;
    double del = d * c;
    h *= del;
    if (fabs(del - 1.0) < EPS) break;
  }
  return h;
}

double or_ibetac(double a, double b, double x) {
  if (!(a > 0) || !(b > 0) || !(x >= 0) || !(x <= 1) || !isfinite(a) ||
      !isfinite(b))
    return NAN;
  if (x == 0) return 1.0;
  if (x == 1) return 0.0;
  double lbt = lgamma(a + b) - lgamma(a) - lgamma(b) + a * log(x) +
               b * log1p(-x);
  double bt = exp(lbt);
  if (x < (a + 1.0) / (a + b + 2.0))
    return 1.0 - bt * betacf(a, b, x) / a;
  return bt * betacf(b, a, 1.0 - x) / b;
}

/* routines.cu:494-508 (mean, population variance), main.cu:1491-1497 */
int or_pddn(int R, const double *js, double *alpha, double *beta,
            double *pddn) {
  double sum = 0.0;
  for (int i = 0; i < R; i++) sum += js[i];
  double mu = sum / R;
  double v = 0.0;
  for (int i = 0; i < R; i++) v += pow(js[i] - mu, 2);
  double var = v / R;
  double a = (((1 - mu) / var) - (1 / mu)) * pow(mu, 2);
  double b = a * (1 / mu - 1);
  *alpha = a;
  *beta = b;
  if (!(a > 0) || !(b > 0) || !isfinite(a) || !isfinite(b) || !(js[0] >= 0) ||
      !(js[0] <= 1)) {
    *pddn = NAN;
    return -1;
  }
  *pddn = or_ibetac(a, b, js[0]);
  return 0;
}
