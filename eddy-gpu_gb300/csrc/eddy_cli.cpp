// eddy_cli.cpp -- drop-in replacement for the reference's ./eddy process
// (main.cu:27-1711) on top of the libeddy_gpu C ABI.
//
// Same flags (-d -c -g -mp -r -pw/pW -pE -pD -rawp -t -l -help, plus -p as
// an alias of -pD), same defaults and clamps (main.cu:118-202), same input
// parsing including its quirks (main.cu:255-503), the same stdout lines and
// the same results.txt / <set>_Networks.txt / <set>_BDEU_SCORES.txt /
// <set>_EdgeList.txt files (routines.cu:217-492, main.cu:1465-1659).
// Extra options: --rng glibc|counter (default glibc, the reference's
// stream), --seed N (counter stream key), --device N.
#include <errno.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include <algorithm>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "eddy_gpu.h"

namespace {

// printf into a string (a set's lines are printed when its turn comes)
void appendf(std::string &out, const char *fmt, ...) {
  char buf[4096];
  va_list ap;
  va_start(ap, fmt);
  const int m = vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (m > 0) out.append(buf, (size_t)std::min(m, (int)sizeof buf - 1));
}

double now_ms() {
  struct timeval tv;
  gettimeofday(&tv, nullptr);
  return tv.tv_sec * 1e3 + tv.tv_usec / 1e3;
}

// fgets-like line reader without a length limit (keeps the '\n').
bool read_line(FILE *f, std::string &out) {
  out.clear();
  int ch;
  while ((ch = fgetc(f)) != EOF) {
    out.push_back((char)ch);
    if (ch == '\n') break;
  }
  return !out.empty();
}

// The whole file in memory (the expression matrix is read once, in one go).
bool read_file(const char *path, std::vector<char> &buf) {
  FILE *f = fopen(path, "rb");
  if (!f) return false;
  buf.clear();
  char tmp[1 << 16];
  size_t got;
  while ((got = fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + got);
  fclose(f);
  return true;
}

// sscanf(token, "%d") on a token that ends at `end`: leading white space,
// an optional sign, then the digits (none: not a number).
bool scan_int(const char *p, const char *end, int &v) {
  while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\v' || *p == '\f')) p++;
  bool neg = false;
  if (p < end && (*p == '+' || *p == '-')) neg = (*p++ == '-');
  if (p >= end || *p < '0' || *p > '9') return false;
  long long x = 0;
  while (p < end && *p >= '0' && *p <= '9') {
    if (x < 1000000000ll) x = x * 10 + (*p - '0');
    p++;
  }
  v = (int)(neg ? -x : x);
  return true;
}

// One matrix row as strtok(row, "\t") sees it (empty fields skipped): the
// gene name, then up to n values; returns the number of value tokens.
int parse_row(const char *p, const char *end, int n, std::string &name, int8_t *out) {
  auto next = [&](const char *&b, const char *&e) -> bool {
    while (p < end && *p == '\t') p++;
    if (p >= end) return false;
    b = p;
    while (p < end && *p != '\t') p++;
    e = p;
    return true;
  };
  const char *b, *e;
  if (!next(b, e)) return -1;
  name.assign(b, e);
  int k = 0;
  while (k < n && next(b, e)) {
    int v = 2;
    if (!scan_int(b, e, v)) v = 2;
    out[k++] = (int8_t)((v >= -1 && v <= 1) ? v : 2);
  }
  return k;
}

// strtok(s, delims) over a std::string copy.
std::vector<std::string> tokens(const std::string &s, const char *delims) {
  std::vector<std::string> out;
  std::vector<char> buf(s.begin(), s.end());
  buf.push_back(0);
  for (char *t = strtok(buf.data(), delims); t; t = strtok(nullptr, delims)) out.emplace_back(t);
  return out;
}

}  // namespace

int main(int argc, char *argv[]) {
  // ---- device banner (main.cu:28-56), reduced to what CUDA 13 exposes
  {
    char name[256];
    int sms = 0, ma = 0, mi = 0;
    if (eddy_device_info(0, name, sizeof name, &sms, &ma, &mi) == EDDY_OK) {
      printf("Device Number: %d\n", 0);
      printf("  Device name: %s\n", name);
      printf("  Compute Capability : %d.%d\n", ma, mi);
      printf("  Device has %d SMs\n\n", sms);
    }
  }
  const char *inputFile = nullptr, *classFile = nullptr, *genesetFile = nullptr;
  int parentCap = 0, perms = 100, rng = EDDY_RNG_GLIBC, device = 0;
  unsigned long long seed = 0;
  double priorWeight = 0.5, alphaDDN = 0.05, theta = -1, lambda = 2.0;
  double alphaEdge = 0.05, alphaEdgePrior;
  bool flag_pAdjust = true;
  // main.cu:118-145
  for (int i = 1; i < argc; i++) {
    const char *nx = (i + 1 < argc) ? argv[i + 1] : "";
    if (strcmp(argv[i], "-d") == 0) inputFile = (i + 1 < argc) ? argv[i + 1] : nullptr;
    else if (strcmp(argv[i], "-g") == 0) genesetFile = (i + 1 < argc) ? argv[i + 1] : nullptr;
    else if (strcmp(argv[i], "-c") == 0) classFile = (i + 1 < argc) ? argv[i + 1] : nullptr;
    else if (strcmp(argv[i], "-l") == 0) lambda = atof(nx);
    else if (strcmp(argv[i], "-t") == 0) theta = atof(nx);
    else if (strcmp(argv[i], "-mp") == 0) parentCap = atoi(nx);
    else if (strcmp(argv[i], "-help") == 0 || strcmp(argv[i], "--help") == 0)
      printf("Required arguments : \n -d input.txt\n -c classfile.txt\n -g "
             "geneset.txt -mp # of parents\n -p pvalue for DDN significance "
             "testing\n");
    else if (strcmp(argv[i], "-r") == 0) perms = atoi(nx);
    else if (strcmp(argv[i], "-pw") == 0 || strcmp(argv[i], "pW") == 0) priorWeight = atof(nx);
    else if (strcmp(argv[i], "-pE") == 0) alphaEdge = atof(nx);
    else if (strcmp(argv[i], "-rawp") == 0) flag_pAdjust = false;
    else if (strcmp(argv[i], "-pD") == 0 || strcmp(argv[i], "-p") == 0) alphaDDN = atof(nx);
    else if (strcmp(argv[i], "--rng") == 0) rng = strcmp(nx, "counter") == 0 ? EDDY_RNG_COUNTER : EDDY_RNG_GLIBC;
    else if (strcmp(argv[i], "--seed") == 0) seed = strtoull(nx, nullptr, 10);
    else if (strcmp(argv[i], "--device") == 0) device = atoi(nx);
  }
  if (!inputFile) { printf("Invalid input file entered. Exiting...\n"); exit(EXIT_FAILURE); }
  if (!classFile) { printf("Invalid class file entered. Exiting...\n"); exit(EXIT_FAILURE); }
  if (!genesetFile) { printf("Invalid geneset file entered. Exiting...\n"); exit(EXIT_FAILURE); }
  printf("%s\n", genesetFile);
  if (alphaDDN < 0.0 || alphaDDN > 1.0) alphaDDN = .05;
  printf("alpha for signficance of DDN  = %f\n", alphaDDN);
  if (parentCap <= 0) parentCap = 3;
  printf("Max parents = %d\n", parentCap);
  if (perms <= 0) perms = 100;
  printf("Permutations = %d\n", perms);
  if (priorWeight < 0.0 || priorWeight > 1.0) priorWeight = 0.5;
  printf("priorWeight : %f\n", priorWeight);
  if (theta > 0) alphaEdge = 1 - pow(theta, 1.0 / lambda);
  else theta = pow(1 - alphaEdge, lambda);
  alphaEdgePrior = 1 - (1 - alphaEdge) * pow(priorWeight, 1 / lambda);
  printf("alphaEdge : %f, alphaEdgePrior : %f\n", alphaEdge, alphaEdgePrior);
  printf("Multiple testing correction (edge detection) : %s\n", flag_pAdjust ? "true" : "false");
  printf("[to be deprecated] lambda : %f, theta : %f\n", lambda, theta);

  FILE *fpExpr = fopen(inputFile, "r");
  FILE *fpClass = fopen(classFile, "r");
  FILE *fpGeneSet = fopen(genesetFile, "r");
  FILE *fpResults = fopen("results.txt", "w");
  if (!fpExpr) { printf("Expression file is NULL: %s [%d]\n", strerror(errno), errno); exit(EXIT_FAILURE); }
  if (!fpClass) { printf("Class File File is NULL: %s [%d]\n", strerror(errno), errno); exit(EXIT_FAILURE); }
  if (!fpGeneSet) { printf("Gene List File is NULL: %s [%d]\n", strerror(errno), errno); exit(EXIT_FAILURE); }
  if (!fpResults) { printf("results file is NULL: %s [%d]\n", strerror(errno), errno); exit(EXIT_FAILURE); }

  // ---- expression matrix, main.cu:255-301 (quirks kept: 1-character sample
  // names leave the count, the last row is dropped).  The file is read in
  // one go; the rows are parsed in parallel.
  std::string line;
  fclose(fpExpr);
  std::vector<char> text;
  if (!read_file(inputFile, text)) {
    printf("Expression file is NULL: %s [%d]\n", strerror(errno), errno);
    exit(EXIT_FAILURE);
  }
  std::vector<size_t> ls;  // line starts (each line keeps its '\n')
  for (size_t pos = 0; pos < text.size();) {
    ls.push_back(pos);
    const void *nl = memchr(text.data() + pos, '\n', text.size() - pos);
    pos = nl ? (size_t)((const char *)nl - text.data()) + 1 : text.size();
  }
  ls.push_back(text.size());
  const int nlines = (int)ls.size() - 1;
  line = nlines > 0 ? std::string(text.data() + ls[0], text.data() + ls[1]) : std::string();
  std::vector<std::string> sampleNames = tokens(line, "\t");
  if (!sampleNames.empty()) sampleNames.erase(sampleNames.begin());
  int numSamples = (int)sampleNames.size();
  for (int i = 0; i < numSamples; i++)
    if (sampleNames[i].size() == 1) numSamples--;
  printf("%d samples\n", numSamples);
  int numGenes = nlines - 2;  // rows after the header, the last one dropped
  if (numGenes < 0) numGenes = 0;
  printf("%d genes\n", numGenes);
  std::vector<std::string> geneNames(numGenes);
  std::vector<int8_t> data((size_t)numGenes * numSamples);
  {
    std::vector<int> got(numGenes, 0);
    const int nth = std::max(1, std::min((int)std::thread::hardware_concurrency(), 32));
    std::vector<std::thread> pool;
    for (int t = 0; t < nth; t++)
      pool.emplace_back([&, t]() {
        for (int i = t; i < numGenes; i += nth)
          got[i] = parse_row(text.data() + ls[1 + i], text.data() + ls[2 + i], numSamples,
                             geneNames[i], data.data() + (size_t)i * numSamples);
      });
    for (auto &th : pool) th.join();
    for (int i = 0; i < numGenes; i++)
      if (got[i] < numSamples) {
        fprintf(stderr, "eddy: row %d of %s has %d values, %d expected\n", i + 2, inputFile,
                got[i] < 0 ? 0 : got[i], numSamples);
        exit(EXIT_FAILURE);
      }
  }

  // ---- class labels, main.cu:303-352
  read_line(fpClass, line);
  std::vector<std::string> cn = tokens(line, "\t");
  if ((int)cn.size() < numSamples || numSamples < 1) {
    fprintf(stderr, "eddy: class file has %d labels, %d samples\n", (int)cn.size(), numSamples);
    exit(EXIT_FAILURE);
  }
  cn.resize(numSamples);
  int ci;
  for (ci = 1; ci < numSamples; ci++)
    if (cn[ci] != cn[0]) break;
  std::string class1 = cn[0];
  std::string class2 = ci < numSamples ? cn[ci] : std::string();
  if (!cn[numSamples - 1].empty() && cn[numSamples - 1].back() == '\n') cn[numSamples - 1].pop_back();
  int numClass1 = 0, numClass2 = 0;
  std::vector<uint8_t> classIDs(numSamples, 255);
  for (int i = 0; i < numSamples; i++) {
    if (cn[i] == class1) { numClass1++; classIDs[i] = 0; }
    if (cn[i] == class2) { numClass2++; classIDs[i] = 1; }
  }
  printf("Classes: %d %s, %d %s\n", numClass1, class1.c_str(), numClass2, class2.c_str());
  fclose(fpClass);
  for (int i = 0; i < numSamples; i++)
    if (classIDs[i] > 1) {
      fprintf(stderr, "eddy: sample %d has a label of neither class (the reference leaves it "
                      "undefined)\n", i);
      exit(EXIT_FAILURE);
    }

  eddy_opts o{};
  o.max_parents = parentCap;
  o.alpha_edge = alphaEdge;
  o.alpha_edge_prior = alphaEdgePrior;
  o.bonferroni = flag_pAdjust ? 1 : 0;
  o.permutations = perms;
  o.rng = rng;
  o.seed = seed;
  o.device = device;
  o.keep_networks = 1;
  eddy_ctx *ctx = nullptr;
  if (eddy_ctx_create(&o, &ctx) != EDDY_OK) {
    fprintf(stderr, "eddy: no usable CUDA device %d\n", device);
    exit(EXIT_FAILURE);
  }
  if (eddy_load_matrix(ctx, data.data(), numGenes, numSamples, classIDs.data()) != EDDY_OK) {
    fprintf(stderr, "eddy: %s\n", eddy_last_error(ctx));
    exit(EXIT_FAILURE);
  }

  fprintf(fpResults, "Pathway\tJS\tPval\tnGenes\n");
  // gene name -> its first row (main.cu:400-430 takes the first match)
  std::unordered_map<std::string, int> rowOf;
  rowOf.reserve((size_t)numGenes * 2);
  for (int j = 0; j < numGenes; j++) rowOf.emplace(geneNames[j], j);
  // Every set is read and added first (its lines of main.cu:359-503 kept
  // for its turn in the output), then one eddy_run runs them all, batched
  // across sets; the sets' lines, results and files then follow in order,
  // as the reference prints them.
  struct SetJob {
    std::string name, lines;
    std::vector<std::string> genes;
    std::vector<uint8_t> prior;
    bool havePrior = false;
    int sid = -1;
  };
  std::vector<SetJob> jobs;
  std::string addError, addLines;
  while (read_line(fpGeneSet, line)) {
    if (line[0] == '\n') continue;  // main.cu:361-363
    SetJob J;
    std::vector<std::string> lt = tokens(line, "\n");
    std::vector<std::string> tk = lt.empty() ? std::vector<std::string>() : tokens(lt[0], "\t");
    J.name = tk.empty() ? std::string() : tk[0];
    std::vector<std::string> setGenes(tk.size() > 2 ? tk.begin() + 2 : tk.end(), tk.end());
    appendf(J.lines, "%s\n", J.name.c_str());
    appendf(J.lines, "%d genes in geneset\n", (int)setGenes.size());
    // main.cu:400-430: first matching row, missing genes dropped
    std::vector<int32_t> gidx;
    for (auto &gs : setGenes) {
      auto it = rowOf.find(gs);
      if (it != rowOf.end()) {
        J.genes.push_back(geneNames[it->second]);
        gidx.push_back(it->second);
      }
    }
    const int g = (int)gidx.size();
    appendf(J.lines, "Adjusted genes : %d\n", g);
    // main.cu:432-503 prior file
    std::string dir = "PRIORS/" + J.name + ".prior";
    if (dir.find('\r') != std::string::npos) appendf(J.lines, "File problem! Uses window endings!\n");
    FILE *pf = fopen(dir.c_str(), "r");
    appendf(J.lines, "file : %s\n", dir.c_str());
    J.prior.assign((size_t)g * g, 0);
    J.havePrior = pf != nullptr;
    if (!pf) appendf(J.lines, "No prior file exists. Computing without prior knowledge\n");
    char pbuf[100];
    while (pf && fgets(pbuf, sizeof pbuf, pf)) {
      char *tok = strtok(pbuf, "\t");
      if (!tok) continue;
      int row = -1, col = -1;
      for (int k = 0; k < g; k++)
        if (J.genes[k] == tok) { row = k; break; }
      if (row < 0) continue;
      tok = strtok(nullptr, "\t");
      if (!tok || strcmp(tok, "neighbor-of") == 0) continue;
      tok = strtok(nullptr, "\t");
      if (!tok) continue;
      size_t L = strlen(tok);
      if (L > 0) tok[L - 1] = '\0';
      for (int k = 0; k < g; k++)
        if (J.genes[k] == tok) { col = k; break; }
      if (col < 0) continue;
      J.prior[(size_t)row * g + col] = J.prior[(size_t)col * g + row] = 1;
    }
    if (pf) fclose(pf);
    appendf(J.lines, "Permutations begin:\n");
    if (eddy_add_set(ctx, gidx.data(), g, J.havePrior ? J.prior.data() : nullptr, &J.sid) != EDDY_OK) {
      // the sets before it are still run and printed, then its lines
      addLines = J.lines;
      addError = eddy_last_error(ctx);
      break;
    }
    jobs.push_back(std::move(J));
  }
  std::string runError;
  if (!jobs.empty() && eddy_run(ctx) != EDDY_OK) runError = eddy_last_error(ctx);
  for (SetJob &J : jobs) {
    const double t_set = now_ms();
    eddy_set_summary sm;
    if (eddy_get_set_summary(ctx, J.sid, &sm) != EDDY_OK) break;  // not run: the run failed
    const int g = (int)J.genes.size();
    fputs(J.lines.c_str(), stdout);
    printf("Original Number of unique Networks : %d\n", sm.unique0);
    if (isnan(sm.js0)) printf("jsVal[0] NAN--Breaking permutation loop\n");
    for (int p = 100; p < sm.iterations; p += 100) printf("  Permutation %d finished\n", p);
    printf("permutation loop (%d) finished\n", perms);
    if (sm.failed) {
      fprintf(fpResults, "%s failed with %d genes- one of the js scores was nan\n",
              J.name.c_str(), g);
      printf("nan value- quiting!\n\n\n");
      continue;
    }
    printf("Original JS : %f\n", sm.js0);
    printf("alpha : %f beta : %f\n", sm.alpha, sm.beta);
    if (!sm.betafit_ok)
      fprintf(stderr, "eddy: beta fit of set %s has alpha/beta outside (0, inf); pDDN "
                      "undefined\n", J.name.c_str());
    printf("pDDN = %f\n", sm.pddn);
    fprintf(fpResults, "%s\t%f\t%f\t%d\n", J.name.c_str(), sm.js0, sm.pddn, g);
    fflush(fpResults);
    if (sm.pddn < alphaDDN) {
      int U = 0, E = 0;
      eddy_get_networks(ctx, J.sid, &U, &E, nullptr, nullptr, nullptr, nullptr, nullptr);
      std::vector<int32_t> ids(U), nodes((size_t)U * g), epn(U + 1), edges(E > 0 ? E : 1);
      std::vector<double> lval(2 * (size_t)U);
      eddy_get_networks(ctx, J.sid, &U, &E, ids.data(), nodes.data(), epn.data(), edges.data(),
                        lval.data());
      std::vector<const char *> gn(g);
      for (int k = 0; k < g; k++) gn[k] = J.genes[k].c_str();
      std::string pn = J.name + "_Networks.txt", pb = J.name + "_BDEU_SCORES.txt",
                  pe = J.name + "_EdgeList.txt";
      if (eddy_write_networks(pn.c_str(), inputFile, classFile, J.name.c_str(), U, epn.data(),
                              gn.data(), g, nodes.data(), edges.data(), epn[U], ids.data()) != EDDY_OK) {
        printf("output when accessing networkOutput.txt is NULL. Error code : %s. Exiting...\n",
               strerror(errno));
        exit(EXIT_FAILURE);
      }
      printf("Finished writing %s\n", pn.c_str());
      if (eddy_write_bdeu(pb.c_str(), inputFile, classFile, J.name.c_str(), class1.c_str(),
                          class2.c_str(), U, lval.data()) != EDDY_OK) {
        printf("scoreFile is NULL. Error code : %s. Exiting...\n", strerror(errno));
        exit(EXIT_FAILURE);
      }
      printf("Finished bdeu file %s\n", pb.c_str());
      int EL = 0;
      eddy_get_edge_list(ctx, J.sid, &EL, nullptr, nullptr, nullptr);
      std::vector<int32_t> eln(2 * (size_t)g), elp(3), ele(EL > 0 ? EL : 1);
      eddy_get_edge_list(ctx, J.sid, &EL, eln.data(), elp.data(), ele.data());
      eddy_write_edge_list(pe.c_str(), gn.data(), g, eln.data(), ele.data(), elp.data(),
                           J.havePrior ? J.prior.data() : nullptr, class1.c_str(), class2.c_str());
      printf("Finished writing edgelist file %s\n", pe.c_str());
      printf("Total run time : %f\n", now_ms() - t_set);
    }
    printf("\nPathway finished.\n\n");
    int msec = (int)(now_ms() - t_set);
    printf("Time taken %d seconds %d milliseconds\n\n\n", msec / 1000, msec % 1000);
  }
  if (runError.empty() && !addError.empty()) fputs(addLines.c_str(), stdout);
  if (!runError.empty() || !addError.empty()) {
    fprintf(stderr, "eddy: %s\n", (!runError.empty() ? runError : addError).c_str());
    exit(EXIT_FAILURE);
  }
  fclose(fpGeneSet);
  fclose(fpResults);
  eddy_ctx_destroy(ctx);
  return 0;
}
