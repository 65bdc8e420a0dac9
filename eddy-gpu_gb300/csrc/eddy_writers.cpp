// eddy_writers.cpp -- the reference's three per-set output files, byte for
// byte: <set>_Networks.txt (routines.cu:240-306), <set>_BDEU_SCORES.txt
// (routines.cu:217-238) and <set>_EdgeList.txt (routines.cu:308-492).
// Host code of the C ABI (include/eddy_gpu.h); the eddy CLI calls them.
#include <stdio.h>
#include <string.h>

#include <vector>

#include "eddy_gpu.h"

namespace {
struct Graph {
  int node, edge, inBoth;
};
}  // namespace

extern "C" int eddy_write_networks(const char *path, const char *input, const char *cls,
                                   const char *set, int U, const int32_t *epn,
                                   const char *const *genes, int g, const int32_t *nodes,
                                   const int32_t *edges, int total_edges, const int32_t *ids) {
  FILE *out = fopen(path, "w");
  if (!out) return EDDY_ERR_ARG;
  fprintf(out, "%s", "\t\tUnique Networks\n\n");
  fprintf(out, "input : %s\n", input);
  fprintf(out, "class : %s\n", cls);
  fprintf(out, "geneset : %s\n\n\n", set);
  int edgePos = 0;
  for (int i = 0; i < U; i++) {
    int total = (i == U - 1) ? total_edges - epn[i] : epn[i + 1] - epn[i];
    fprintf(out, "network %d (%d)\t number of edges : %d\n", i + 1, ids[i], total);
    fprintf(out, "%s", "---------------");
    fprintf(out, "%s", "---------------\n\n");
    if (total == 0) continue;
    for (int j = 0; j < g - 1; j++) {
      const int change = nodes[(size_t)i * g + j + 1] - nodes[(size_t)i * g + j];
      if (change != 0) {
        total -= change;
        for (int k = 0; k < change; k++) fprintf(out, "%s - %s\n", genes[j], genes[edges[edgePos++]]);
      }
      if (j + 1 == g - 1 && total > 0)
        for (int k = 0; k < total; k++) fprintf(out, "%s - %s\n", genes[j + 1], genes[edges[edgePos++]]);
    }
    fprintf(out, "%s", "\n");
    fprintf(out, "%s", "\n");
  }
  fclose(out);
  return EDDY_OK;
}

extern "C" int eddy_write_bdeu(const char *path, const char *input, const char *cls,
                               const char *set, const char *class1, const char *class2, int U,
                               const double *lval) {
  FILE *f = fopen(path, "w");
  if (!f) return EDDY_ERR_ARG;
  fprintf(f, "\t\t BDEU SCORES\n");
  fprintf(f, "input : %s\n", input);
  fprintf(f, "class : %s\n", cls);
  fprintf(f, "geneset : %s\n\n", set);
  fprintf(f, "Network \t  %s  \t   \t    %s\n", class1, class2);
  for (int j = 0; j < U; j++) fprintf(f, "Network %d\t %f \t %f \n", j + 1, lval[j], lval[j + U]);
  fclose(f);
  return EDDY_OK;
}

extern "C" int eddy_write_edge_list(const char *path, const char *const *genes, int g,
                                    const int32_t *nodes, const int32_t *edges,
                                    const int32_t *epn, const uint8_t *prior, const char *class1,
                                    const char *class2) {
  FILE *out = fopen(path, "w");
  if (!out) return EDDY_ERR_ARG;
  std::vector<Graph> c1, c2;
  int edgePos = 0;
  const char *classes[2] = {class1, class2};
  for (int i = 0; i < 2; i++) {
    int total = (i == 1) ? epn[2] - epn[i] : epn[i + 1] - epn[i];
    if (total == 0) continue;
    for (int j = 0; j < g - 1; j++) {
      const int change = nodes[(size_t)i * g + j + 1] - nodes[(size_t)i * g + j];
      if (change != 0) {
        total -= change;
        for (int k = 0; k < change; k++) {
          Graph t{j, edges[edgePos++], 0};
          (strcmp(classes[i], class1) == 0 ? c1 : c2).push_back(t);
        }
      }
      if (j + 1 == g - 1 && total > 0)
        for (int k = 0; k < total; k++) {
          Graph t{j + 1, edges[edgePos++], 0};
          (strcmp(classes[i], class1) == 0 ? c1 : c2).push_back(t);
        }
    }
  }
  for (auto &a : c1)
    for (auto &b : c2)
      if (a.node == b.node && a.edge == b.edge) a.inBoth = b.inBoth = 1;
  std::vector<uint8_t> found((size_t)g * g, 0);
  auto pr = [&](int r, int c) { return prior ? (int)(prior[(size_t)r * g + c] == 1) : 0; };
  static const char *ps[2] = {"NONE", "PRIOR"};
  for (auto &a : c1) {
    fprintf(out, "%s\t%s\t%s\t%s\n", genes[a.node], genes[a.edge], a.inBoth == 1 ? "Both" : class1,
            ps[pr(a.node, a.edge)]);
    found[(size_t)a.node * g + a.edge] = found[(size_t)a.edge * g + a.node] = 1;
  }
  for (auto &b : c2)
    if (b.inBoth != 1) {
      fprintf(out, "%s\t%s\t%s\t%s\n", genes[b.node], genes[b.edge], class2, ps[pr(b.node, b.edge)]);
      found[(size_t)b.node * g + b.edge] = found[(size_t)b.edge * g + b.node] = 1;
    }
  for (int row = 1; row < g; row++)
    for (int col = 0; col < row; col++)
      if (!found[(size_t)row * g + col] && pr(row, col) == 1)
        fprintf(out, "%s\t%s\t%s\t%s\n", genes[row], genes[col], "Neither", "PRIOR");
  fclose(out);
  return EDDY_OK;
}
