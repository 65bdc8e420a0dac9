// Prints iterations 0 .. R-1 of the reference's label stream (main.cu:538-573)
// as drawn by the library's host sampler (eddy_host.cpp), one line of 0/1
// per iteration, from srand(1) and the labelling s % 3 == 0 -> class 1; then
// checks that a copy of the generator taken mid-stream continues exactly as
// the original.  Built and run by test_glibc_stream.py.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "eddy_host.h"

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  const int n = atoi(argv[1]), n1 = atoi(argv[2]), R = atoi(argv[3]);
  eddy::GlibcRand rng(1);
  std::vector<uint8_t> lab(n), seen;
  std::vector<int> order;
  for (int s = 0; s < n; s++) lab[s] = s % 3 == 0 ? 0 : 1;
  for (int it = 0; it < R; it++) {
    eddy::glibc_permutation(rng, n, n1, it > 0, lab.data(), seen, order);
    for (int s = 0; s < n; s++) putchar('0' + lab[s]);
    putchar('\n');
  }
  eddy::GlibcRand copy = rng;
  int bad = 0;
  for (int k = 0; k < 5000; k++) bad += copy.next() != rng.next();
  printf("copy %s\n", bad ? "differs" : "ok");
  return 0;
}
