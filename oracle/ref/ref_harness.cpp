/*
 * ref_harness.cpp -- runs the reference's own kernels (kernel1.cu ..
 * kernel5.cu) and host routines (routines.cu) on the CPU, compiled from the
 * reference sources where they lie (the `ref` target of oracle/Makefile), through a
 * small CUDA-thread emulator.  TEST INFRASTRUCTURE ONLY: it produces the
 * golden vectors under tests/golden that pin the oracle restatement.
 *
 * The emulator: a launch runs blocks one after another; inside a block each
 * simulated thread is a ucontext fiber; __syncthreads() switches back to
 * the block scheduler, which resumes every fiber of the block up to its next
 * barrier before releasing any of them (kernel1.cu run2 and kernel3.cu
 * run22 use barriers).  Launches without barriers run their threads as a
 * plain loop.
 *
 * ref_unit() follows the per-permutation host flow of main.cu:607-1428
 * (pair tables, launch shapes, host prefix sums, the uniqueness sweep, the
 * likelihood normalisation), calling the reference kernels and routines for
 * every step they implement.
 */
#include <stdint.h>
#include <ucontext.h>

#include <functional>
#include <vector>

#include "definitions.cuh"

/* ------------------------------------------------------- emulator */
emu_dim3 blockIdx, threadIdx, blockDim, gridDim;

/* run2 (kernel1.cu:400) declares `extern __shared__ int sharedMatrix[]`. */
int sharedMatrix[1 << 20];

namespace {
struct Fiber {
  ucontext_t ctx;
  std::vector<char> stack;
  bool done;
};
bool g_fiber_mode = false;
ucontext_t g_sched;
std::vector<Fiber> g_fibers;
const std::function<void()> *g_body = nullptr;
int g_cur = 0;
const size_t kStack = 256 * 1024;

void fiber_entry() {
  (*g_body)();
  g_fibers[g_cur].done = true;
}

void emu_launch(unsigned grid, unsigned block, bool sync,
                const std::function<void()> &body) {
  gridDim = {grid, 1, 1};
  blockDim = {block, 1, 1};
  for (unsigned bx = 0; bx < grid; bx++) {
    blockIdx = {bx, 0, 0};
    if (!sync) {
      for (unsigned tx = 0; tx < block; tx++) {
        threadIdx = {tx, 0, 0};
        body();
      }
      continue;
    }
    if (g_fibers.size() < block) g_fibers.resize(block);
    for (unsigned t = 0; t < block; t++) {
      Fiber &f = g_fibers[t];
      if (f.stack.empty()) f.stack.resize(kStack);
      getcontext(&f.ctx);
      f.ctx.uc_stack.ss_sp = f.stack.data();
      f.ctx.uc_stack.ss_size = f.stack.size();
      f.ctx.uc_link = &g_sched;
      makecontext(&f.ctx, fiber_entry, 0);
      f.done = false;
    }
    g_fiber_mode = true;
    g_body = &body;
    unsigned live = block;
    while (live > 0) {
      for (unsigned t = 0; t < block; t++) {
        if (g_fibers[t].done) continue;
        g_cur = (int)t;
        threadIdx = {t, 0, 0};
        swapcontext(&g_sched, &g_fibers[t].ctx);
        if (g_fibers[t].done) live--;
      }
    }
    g_fiber_mode = false;
  }
}
} // namespace

void emu_syncthreads(void) {
  if (!g_fiber_mode) return;
  swapcontext(&g_fibers[g_cur].ctx, &g_sched);
}

/* ------------------------------------------------------ unit flow */
extern "C" {

/* Runs one permutation's hot path.  Returns 0, or -1 on a size error.
 * Inputs: tA (g x nA), tB (g x nB) int class data; prior g x g int.
 * Outputs (capacities in brackets; any may be NULL):
 *   out23 [S*c] edge bits; ppn [2g]; stf [6g]; edges_pn [S+1];
 *   pnodes [S*g]; pedges [pedges_cap]; unique_ids [S]; uni_nodes [S*g];
 *   uni_edges [pedges_cap]; uni_epn [S+1]; out5 [2*S*g]; lval [2*S];
 *   scal[4] = {U, total edges, unique edges, S}; js [1]. */
int ref_unit(int g, int nA, int nB, const int *tA, const int *tB,
             const int *prior, double alphaEdge, double alphaEdgePrior,
             int flag_pAdjust, int maxParents, int *out23_o, int *ppn_o,
             int *stf_o, int *edges_pn_o, int *pnodes_o, int *pedges_o,
             int pedges_cap, int *unique_ids_o, int *uni_nodes_o,
             int *uni_edges_o, int *uni_epn_o, double *out5_o,
             double *lval_o, int *scal_o, double *js_o) {
  const int genes = g, samples = nA, samples2 = nB;
  if (g < 2 || (long)g * g > (long)(sizeof(sharedMatrix) / sizeof(int)))
    return -1;
  const int c = ((genes * genes) - genes) / 2;
  const int scaler = samples + 1, scaler2 = samples2 + 1;
  const int scalerSum = scaler + scaler2;
  const int MAX_PARENTS = maxParents;

  /* main.cu:615-632 */
  std::vector<int> spacer1(c), ff1(c), searcher(genes);
  searcher[0] = 0;
  int position = 0;
  for (int row = 1; row < genes; row++) {
    for (int col = 0; col < row; col++) {
      spacer1[position] = row;
      ff1[position] = col;
      position++;
    }
    searcher[row] = searcher[row - 1] + row;
  }

  std::vector<int> dtriA(tA, tA + (size_t)genes * samples);
  std::vector<int> dtriAb(tB, tB + (size_t)genes * samples2);
  std::vector<int> dppn(2 * genes), dstf(6 * genes);
  std::vector<int> ddofout((size_t)c * scalerSum);
  /* one spare network row: edgePerNetworkKernel's extra block reads it
   * (main.cu:842), a read past the end of the reference's allocation */
  std::vector<int> dout23((size_t)c * (scalerSum + 1), 0);
  std::vector<int> dprior(prior, prior + (size_t)genes * genes);
  const int sampleSum = samples + samples2 + 2;
  bool fa = flag_pAdjust != 0;

  /* main.cu:737-755 */
  int *pA = dtriA.data(), *pB = dtriAb.data(), *psp = spacer1.data(),
      *pff = ff1.data(), *pdof = ddofout.data(), *pppn = dppn.data(),
      *pstf = dstf.data(), *po = dout23.data(), *ppr = dprior.data();
  if (c < MAX_THREADS) {
    emu_launch(sampleSum, c, true, [=] {
      run2(genes, samples, samples2, pA, pB, psp, pff, pdof, pppn, pstf, po,
           c, ppr, alphaEdgePrior, alphaEdge, fa);
    });
  } else {
    int BPN = (int)ceil((c * 1.0) / MAX_THREADS);
    int TPB = (int)ceil((c * 1.0) / BPN);
    emu_launch(sampleSum * BPN, TPB, false, [=] {
      run2Scalable(genes, samples, samples2, pA, pB, psp, pff, pdof, pppn,
                   pstf, po, c, ppr, alphaEdgePrior, alphaEdge, fa, BPN, TPB);
    });
  }

  /* main.cu:842-858 */
  std::vector<int> dedgesPN(scalerSum + 1, 0), edgesPN(scalerSum + 1, 0);
  int *pepn = dedgesPN.data(), *psr = searcher.data();
  emu_launch(sampleSum + 1, 1, false, [=] {
    edgePerNetworkKernel(po, pepn, psr, genes, MAX_PARENTS, c);
  });
  edgesPN[0] = 0;
  for (int i = 1; i < sampleSum + 1; i++)
    edgesPN[i] = edgesPN[i - 1] + dedgesPN[i - 1];
  dedgesPN = edgesPN;
  pepn = dedgesPN.data();
  const int numEdges = edgesPN[scalerSum];

  /* main.cu:894-932 */
  const int noNodes = genes;
  std::vector<int> dpNodes((size_t)noNodes * scalerSum, 0);
  std::vector<int> dpEdges(numEdges > 0 ? numEdges : 1, 0);
  int *pnd = dpNodes.data(), *ped = dpEdges.data();
  emu_launch(scalerSum, noNodes, true, [=] {
    run22(c, pepn, po, pnd, noNodes, numEdges, psr, ped, MAX_PARENTS);
  });

  /* main.cu:1001-1042 */
  const int scalerCombo = (scalerSum * scalerSum - scalerSum) / 2;
  std::vector<int> scalerTest(scalerCombo), shrunk(scalerCombo),
      shrunkPlc(scalerCombo);
  idPrep(scalerSum, scalerCombo, scalerTest.data(), shrunkPlc.data());
  int *pst = scalerTest.data(), *psh = shrunk.data(), *pspl = shrunkPlc.data();
  const int maxThreads = 1024;
  emu_launch((scalerCombo / (maxThreads - 1)) + 1, maxThreads - 1, false, [=] {
    run25(samples + 1, scalerSum, numEdges, genes, scalerCombo, pepn, pnd, ped,
          psh, pst, pspl);
  });

  /* main.cu:1060-1084 */
  std::vector<char> uniqueN(scalerSum), visted(scalerSum, 0);
  uniqueN[0] = true;
  for (int p = 0; p < scalerCombo; p++) {
    if (visted[scalerTest[p]]) continue;
    if (shrunk[p] == 0) {
      uniqueN[scalerTest[p]] = false;
      visted[scalerTest[p]] = true;
    } else {
      uniqueN[scalerTest[p]] = true;
    }
  }
  int unisum = 0, edSum = 0;
  for (int p = 0; p < scalerSum; p++) {
    if (uniqueN[p]) {
      if (unique_ids_o) unique_ids_o[unisum] = p;
      unisum++;
      if (p == scalerSum - 1)
        edSum += numEdges - edgesPN[p];
      else
        edSum += edgesPN[p + 1] - edgesPN[p];
    }
  }

  /* main.cu:1134-1145: the reference's compaction routine */
  std::vector<int> pUniNodes((size_t)unisum * noNodes);
  std::vector<int> pUniEdges(edSum > 0 ? edSum : 1);
  std::vector<int> pUniEpn(unisum + 1);
  std::vector<bool> uq_dummy;
  bool *uqb = new bool[scalerSum];
  for (int p = 0; p < scalerSum; p++) uqb[p] = uniqueN[p] != 0;
  structureUnique(unisum, numEdges, scaler, scalerSum, noNodes, uqb,
                  edgesPN.data(), dpEdges.data(), dpNodes.data(),
                  pUniEdges.data(), pUniNodes.data(), pUniEpn.data());
  delete[] uqb;

  /* main.cu:1204-1260 */
  const int U = unisum;
  std::vector<double> dout5((size_t)noNodes * U * 2, 0.0);
  std::vector<int> dNij((size_t)noNodes * U * 54), dNijk((size_t)noNodes * U * 162);
  std::vector<int> dUniEpn(pUniEpn.begin(), pUniEpn.begin() + U);
  int *pue = dUniEpn.data(), *pun = pUniNodes.data(), *pued = pUniEdges.data(),
      *pnij = dNij.data(), *pnijk = dNijk.data();
  double *po5 = dout5.data();
  const int dppnLength = genes * 2;
  emu_launch(U * 2, noNodes, false, [=] {
    run4(U, pue, genes, edSum, U, samples, samples2, pA, pB, pued, pun, pppn,
         pstf, pnij, pnijk, po5, dppnLength);
  });

  /* main.cu:1293-1404: likelihood normalisation per class */
  const int sc = U;
  std::vector<double> lval1((size_t)sc * 2, 0.0);
  for (int gg = 0; gg < 2; gg++) {
    int localoffset = gg < 1 ? 0 : sc;
    std::vector<double> dist(sc, 0.0), likeli1(sc), infFlag(sc, 0.0);
    int set = 0, place = 0;
    for (int i = 0; i < sc * noNodes; i++) {
      dist[place] += dout5[i + localoffset * noNodes];
      set++;
      if (set == noNodes) {
        set = 0;
        place++;
      }
    }
    double mn = dist[0], mx = dist[0], scoreSum = 0;
    for (int j3 = 0; j3 < sc; j3++) {
      scoreSum += dist[j3];
      if (dist[j3] > mx) mx = dist[j3];
      if (dist[j3] < mn) mn = dist[j3];
    }
    double inAlpha = -1 * (scoreSum / sc);
    double probScale = (10) / (mx - mn);
    double likeliSum = 0, nonInf = 0;
    for (int m = 0; m < sc; m++) {
      double adjusted = (dist[m] + inAlpha) * probScale;
      likeli1[m] = exp(adjusted);
      nonInf += likeli1[m];
      if (likeli1[m] >= INFINITY || likeli1[m] <= -INFINITY) {
        infFlag[m] = 1.0;
        likeliSum++;
      }
    }
    for (int m = 0; m < sc; m++)
      lval1[m + localoffset] =
          (likeliSum == 0) ? likeli1[m] / nonInf : infFlag[m] / likeliSum;
  }
  /* main.cu:1406-1428 with the reference's kool() */
  std::vector<double> sea(sc);
  for (int i = 0; i < sc; i++) sea[i] = (lval1[i] + lval1[i + sc]) / 2;
  double js = kool(lval1.data(), sea.data(), 0, sc) / 2 +
              kool(lval1.data(), sea.data(), sc, sc) / 2;
  js = js / log(2.0);

  if (out23_o) memcpy(out23_o, dout23.data(), sizeof(int) * (size_t)c * scalerSum);
  if (ppn_o) memcpy(ppn_o, dppn.data(), sizeof(int) * 2 * genes);
  if (stf_o) memcpy(stf_o, dstf.data(), sizeof(int) * 6 * genes);
  if (edges_pn_o) memcpy(edges_pn_o, edgesPN.data(), sizeof(int) * (scalerSum + 1));
  if (pnodes_o) memcpy(pnodes_o, dpNodes.data(), sizeof(int) * (size_t)noNodes * scalerSum);
  if (pedges_o && numEdges <= pedges_cap) memcpy(pedges_o, dpEdges.data(), sizeof(int) * numEdges);
  if (uni_nodes_o) memcpy(uni_nodes_o, pUniNodes.data(), sizeof(int) * (size_t)U * noNodes);
  if (uni_edges_o && edSum <= pedges_cap) memcpy(uni_edges_o, pUniEdges.data(), sizeof(int) * edSum);
  if (uni_epn_o) memcpy(uni_epn_o, pUniEpn.data(), sizeof(int) * (U + 1));
  if (out5_o) memcpy(out5_o, dout5.data(), sizeof(double) * 2 * (size_t)U * noNodes);
  if (lval_o) memcpy(lval_o, lval1.data(), sizeof(double) * 2 * U);
  if (scal_o) {
    scal_o[0] = U;
    scal_o[1] = numEdges;
    scal_o[2] = edSum;
    scal_o[3] = scalerSum;
  }
  if (js_o) js_o[0] = js;
  return 0;
}

/* Uncapped parent lists of two networks, main.cu:1530-1617 (edge-list
 * recompute with PARENTS_LIMIT = INT_MAX). nodes [2g], edges_pn [3],
 * edges [cap]. Returns total edges. */
int ref_uncapped(int g, const int *net0, const int *net1, int *nodes_o,
                 int *edges_pn_o, int *edges_o, int cap) {
  const int c = ((g * g) - g) / 2;
  std::vector<int> out23((size_t)c * 3, 0);
  memcpy(out23.data(), net0, sizeof(int) * c);
  memcpy(out23.data() + c, net1, sizeof(int) * c);
  std::vector<int> searcher(g);
  searcher[0] = 0;
  for (int row = 1; row < g; row++) searcher[row] = searcher[row - 1] + row;
  std::vector<int> dEdgesPN(3, 0);
  int *po = out23.data(), *pe = dEdgesPN.data(), *ps = searcher.data();
  const int PARENTS_LIMIT = INT_MAX;
  emu_launch(3, 1, false,
             [=] { edgePerNetworkKernel(po, pe, ps, g, PARENTS_LIMIT, c); });
  int edgesPN[3];
  edgesPN[0] = 0;
  for (int i = 1; i < 3; i++) edgesPN[i] = edgesPN[i - 1] + dEdgesPN[i - 1];
  dEdgesPN.assign(edgesPN, edgesPN + 3);
  pe = dEdgesPN.data();
  int totalEdges = edgesPN[2];
  std::vector<int> nodes(2 * g), edges(totalEdges > 0 ? totalEdges : 1);
  int *pn = nodes.data(), *ped = edges.data();
  emu_launch(2, g, true,
             [=] { run22(c, pe, po, pn, g, totalEdges, ps, ped, PARENTS_LIMIT); });
  memcpy(nodes_o, nodes.data(), sizeof(int) * 2 * g);
  memcpy(edges_pn_o, edgesPN, sizeof(int) * 3);
  if (totalEdges <= cap) memcpy(edges_o, edges.data(), sizeof(int) * totalEdges);
  return totalEdges;
}

/* routines.cu host AS 147 twin of the device series */
double ref_gammds(double x, double p) {
  int ifault = 0;
  return gammds(x, p, &ifault);
}

double ref_kool(const double *P, const double *Q, int off, int cnt) {
  return kool(const_cast<double *>(P), const_cast<double *>(Q), off, cnt);
}

double ref_mean(const double *a, int n) { return mean(const_cast<double *>(a), n); }
double ref_variance(double mu, const double *a, int n) {
  return variance(mu, const_cast<double *>(a), n);
}

/* The reference's writers (routines.cu:217-492).  names: g x 50 chars. */
void ref_write_networks(const char *path, const char *input, const char *cls,
                        const char *setname, int U, const int *uni_epn,
                        const char *names, int g, const int *uni_nodes,
                        const int *uni_edges, int total_edges,
                        const int *net_ids) {
  writeNetworkFile(const_cast<char *>(path), const_cast<char *>(input),
                   const_cast<char *>(cls), const_cast<char *>(setname), U,
                   const_cast<int *>(uni_epn),
                   (char(*)[MAX_LENGTH_NAME])const_cast<char *>(names), g,
                   const_cast<int *>(uni_nodes), const_cast<int *>(uni_edges),
                   total_edges, const_cast<int *>(net_ids));
}

void ref_write_bdeu(const char *path, const char *input, const char *cls,
                    const char *setname, const char *class1,
                    const char *class2, int U, const double *lval) {
  writeBdeuScores(const_cast<char *>(path), const_cast<char *>(input),
                  const_cast<char *>(cls), const_cast<char *>(setname),
                  const_cast<char *>(class1), const_cast<char *>(class2), U,
                  const_cast<double *>(lval));
}

void ref_write_edge_list(const char *path, const char *input, const char *cls,
                         const char *setname, const char *names, int g,
                         const int *nodes, const int *edges,
                         const int *edges_pn, const int *prior,
                         const char *class1, const char *class2) {
  char c1[MAX_LENGTH_NAME], c2[MAX_LENGTH_NAME];
  strncpy(c1, class1, MAX_LENGTH_NAME - 1);
  c1[MAX_LENGTH_NAME - 1] = 0;
  strncpy(c2, class2, MAX_LENGTH_NAME - 1);
  c2[MAX_LENGTH_NAME - 1] = 0;
  writeEdgeListFile(const_cast<char *>(path), const_cast<char *>(input),
                    const_cast<char *>(cls), const_cast<char *>(setname),
                    (char(*)[MAX_LENGTH_NAME])const_cast<char *>(names), g,
                    const_cast<int *>(nodes), const_cast<int *>(edges),
                    const_cast<int *>(edges_pn), const_cast<int *>(prior), c1,
                    c2);
}

} /* extern "C" */
