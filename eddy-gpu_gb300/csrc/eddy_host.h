// eddy_host.h -- host-side numerics of libeddy_gpu shared by the C ABI and
// the eddy CLI: decision thresholds, the glibc-compatible label stream,
// the counter label stream, incomplete beta and the beta fit.
#pragma once
#include <stdint.h>

#include <vector>

#include "eddy_internal.h"

namespace eddy {

// Thresholds of one set for both alpha selectors and dof 1, 2, 4.
// Returns true when the alphas are outside (0, 1] (every table then takes
// the exact FP64 path).
bool compute_thresholds(double alpha_edge, double alpha_edge_prior, int g, int bonferroni,
                        Thr out[2][kDofSlots]);

// Upper-tail chi-square probability for dof 1, 2, 4 (closed forms).
double chi2_sf(double chi, int dof);

// glibc random() TYPE_3 additive feedback generator (x_i = x_{i-3} + x_{i-31}
// mod 2^32, output x_i >> 1, 310 discarded outputs after an LCG fill with
// multiplier 16807 mod 2^31-1), the stream behind rand()/srand().
class GlibcRand {
 public:
  explicit GlibcRand(uint32_t seed = 1) { reseed(seed); }
  void reseed(uint32_t seed);
  inline uint32_t next() {
    if (pos_ == kEnd) refill();
    return buf_[pos_++] >> 1;
  }
  // the raw words of the next *avail draws (at least one; output = word >> 1):
  // a caller that uses k of them calls advance(k)
  const uint32_t *peek(int &avail) {
    if (pos_ == kEnd) refill();
    avail = kEnd - pos_;
    return buf_ + pos_;
  }
  void advance(int k) { pos_ += k; }
  // n draws, discarded
  void skip(int n) {
    while (n > 0) {
      if (pos_ == kEnd) refill();
      const int take = n < kEnd - pos_ ? n : kEnd - pos_;
      pos_ += take;
      n -= take;
    }
  }

 private:
  // The raw words r[i] = r[i-31] + r[i-3] (mod 2^32) in stream order, a
  // block at a time: buf_[pos_-31 .. pos_) are the last 31 drawn (the
  // generator's state), buf_[pos_ ..) the next ones, already computed.  A
  // copy carries on exactly where the original would.
  static constexpr int kBlock = 1024, kEnd = 31 + kBlock;
  void fill() {
    // the last three words in registers: each new word reads memory only
    // 31 words back
    uint32_t a = buf_[28], b = buf_[29], c = buf_[30];
    for (int j = 31; j < kEnd; j++) {
      const uint32_t v = buf_[j - 31] + a;
      buf_[j] = v;
      a = b;
      b = c;
      c = v;
    }
    pos_ = 31;
  }
  void refill() {
    for (int j = 0; j < 31; j++) buf_[j] = buf_[kBlock + j];
    fill();
  }
  uint32_t buf_[kEnd];
  int pos_ = kEnd;
};

// One iteration of main.cu:541-570: n discarded draws, then the first n
// distinct values of rand()%n; perm > 0 relabels (first n_class1 -> 0).
void glibc_permutation(GlibcRand &rng, int n, int n_class1, bool relabel, uint8_t *labels,
                       std::vector<uint8_t> &seen, std::vector<int> &order);

// Counter labelling (Philox-4x32-10), same definition as the GPU kernel.
void counter_labels(uint64_t seed, int set_id, int perm, int n, int n_class1, uint8_t *labels);

// 1 - I_x(a, b) (regularised incomplete beta complement).
double ibetac(double a, double b, double x);

// Beta fit of js[0..R) by moments and pDDN = ibetac(alpha, beta, js[0]).
// Returns false when alpha or beta is not positive finite.
bool beta_pddn(const double *js, int R, double &alpha, double &beta, double &pddn);

// Fixed-point BDeu table lg[d][m] = (lgamma(m + 4/d) - lgamma(4/d)) * 2^shift.
void bdeu_table(int n, std::vector<int64_t> &lg, int &shift, int8_t dmap[82]);
// The same into a caller array of kDivisors * (n + 1) entries (no allocation).
void bdeu_table_into(int n, int64_t *lg, int &shift, int8_t dmap[82]);

}  // namespace eddy
