// eddy_host.cpp -- host numerics of libeddy_gpu (see eddy_host.h).
#include "eddy_host.h"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <utility>

namespace eddy {

// ------------------------------------------------------------ thresholds
double chi2_sf(double chi, int dof) {
  if (chi <= 0) return 1.0;
  const double x = 0.5 * chi;
  switch (dof) {
    case 1: return erfc(sqrt(x));
    case 2: return exp(-x);
    case 4: return exp(-x) * (1.0 + x);
    default: return 1.0;
  }
}

// Chi-square at which AS 147 (kernel1.cu:36-42) stops returning a value:
// p log(x) - lgamma(p+1) - x < log(1e-37) with x = chi/2, p = dof/2, x > p.
static double cliff_chi(int dof) {
  const double p = 0.5 * dof, lim = log(1.0e-37);
  double lo = p + 1.0, hi = 4096.0;
  for (int i = 0; i < 200; i++) {
    double mid = 0.5 * (lo + hi);
    double arg = p * log(mid) - lgamma(p + 1.0) - mid;
    if (arg < lim) hi = mid; else lo = mid;
  }
  return lo + hi;  // 2 * x_c
}

// Smallest chi in [0, hi] with chi2_sf(chi) <= target (sf decreasing).
static double invert_sf(double target, int dof, double hi) {
  double lo = 0.0;
  for (int i = 0; i < 300; i++) {
    double mid = 0.5 * (lo + hi);
    if (chi2_sf(mid, dof) <= target) hi = mid; else lo = mid;
  }
  return hi;
}

static float round_down(double v) {
  float f = (float)v;
  if ((double)f > v) f = nextafterf(f, -INFINITY);
  return f;
}
static float round_up(double v) {
  float f = (float)v;
  if ((double)f < v) f = nextafterf(f, INFINITY);
  return f;
}

// Bound on |p_ref - p_true| for chi-square values near chi.  AS 147
// (kernel1.cu:10-74) sums the terms c_k = c_{k-1} x / (p + k) and stops at
// the first c_k <= 1e-9 x (the running sum); the terms after it fall at
// least geometrically from the ratio r = x / (p + k + 1) of the next one, so
// the dropped tail is at most 1e-9 r / (1 - r) of the sum, and the sum times
// its prefactor is P <= 1.  The ~k FP64 steps and the prefactor's log,
// lgamma and exp add well under 1e-12.  The stop is replayed at chi and at
// chi (1 +- 1e-3), which covers every chi-square of the guard band, with a
// quarter added for a stop one term earlier or later; a ratio above 0.8
// (far beyond any threshold below the underflow cliff) keeps 1e-8.
static double as147_eps(double chi, int dof) {
  const double p = 0.5 * dof;
  double worst = 0;
  for (const double f : {1 - 1e-3, 1.0, 1 + 1e-3}) {
    const double x = 0.5 * chi * f;
    double c = 1.0, v = 1.0, a = p;
    for (int k = 0; k < 100000; k++) {
      a += 1.0;
      c = c * x / a;
      v += c;
      if (c <= 1e-9 * v) break;
    }
    const double r = x / (a + 1.0);
    if (!(r < 0.8)) return 1e-8;
    worst = std::max(worst, r / (1.0 - r));
  }
  return 1e-9 * (worst + 0.25) + 1e-12;
}

bool compute_thresholds(double alpha_edge, double alpha_edge_prior, int g, int bonferroni,
                        Thr out[2][kDofSlots]) {
  const double aeff[2] = {alpha_edge, std::max(alpha_edge, alpha_edge_prior)};
  bool exact_all = false;
  for (int s = 0; s < 2; s++)
    if (!(aeff[s] > 0.0) || !(aeff[s] <= 1.0)) exact_all = true;
  // Bonferroni factor as the reference computes it: int ((g-1)*g)/2
  const double C = bonferroni ? (double)(((g - 1) * g) / 2) : 1.0;
  const double relf = 2e-5;  // FP32 chi-square relative error bound
  static const int dofs[kDofSlots] = {1, 2, 4};
  for (int s = 0; s < 2; s++) {
    for (int d = 0; d < kDofSlots; d++) {
      Thr &T = out[s][d];
      const int dof = dofs[d];
      const double kc = cliff_chi(dof);
      double chiA, chiB;
      if (exact_all || C <= 0) {
        chiA = -1;
        chiB = INFINITY;
      } else {
        const double t = aeff[s] / C;
        // |p_ref - p_true| < eps at the chi-square where p_true = t
        const double eps = chi2_sf(kc, dof) < t ? as147_eps(invert_sf(t, dof, kc), dof) : 1e-8;
        const double hiT = t * (1 + 1e-9) + eps;  // p above: surely no edge
        const double loT = t * (1 - 1e-9) - eps;  // p below: surely an edge
        if (chi2_sf(0.0, dof) < hiT) chiA = 0.0;
        else if (chi2_sf(kc, dof) >= hiT) chiA = kc;
        else chiA = invert_sf(hiT, dof, kc);  // sf(chi) < hiT for chi >= chiA
        // largest chi with sf >= hiT is just below chiA
        chiA *= (1 - 1e-7);
        if (loT <= 0 || chi2_sf(kc, dof) > loT) chiB = INFINITY;
        else chiB = invert_sf(loT, dof, kc) * (1 + 1e-7);
      }
      const double kLo = kc * (1 - 1e-8), kHi = kc * (1 + 1e-8);
      T.chiA = round_down(chiA);
      T.chiB = std::isinf(chiB) ? INFINITY : round_up(chiB);
      T.kLo = round_down(kLo);
      T.kHi = round_up(kHi);
      T.fA = round_down(chiA / (1 + relf));
      T.fB = std::isinf(chiB) ? INFINITY : round_up(chiB / (1 - relf));
      T.fKlo = round_down(kLo / (1 + relf));
      T.fKhi = round_up(kHi / (1 - relf));
    }
  }
  return exact_all;
}

// ------------------------------------------------------------ glibc stream
void GlibcRand::reseed(uint32_t seed) {
  uint32_t st[31];
  int32_t w = (int32_t)(seed == 0 ? 1u : seed);
  st[0] = (uint32_t)w;
  for (int i = 1; i < 31; i++) {
    // 16807 * w mod (2^31 - 1) by Schrage's method
    int32_t hi = w / 127773, lo = w % 127773;
    int32_t word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    w = word;
    st[i] = (uint32_t)w;
  }
  // glibc's first draw adds word 0 to word 3 (its front pointer starts 3
  // words ahead of the rear one): in stream order the oldest word is st[3],
  // then st[4..30], st[0..2]
  for (int k = 0; k < 31; k++) buf_[k] = st[(k + 3) % 31];
  fill();
  skip(310);
}

void glibc_permutation(GlibcRand &rng, int n, int n_class1, bool relabel, uint8_t *labels,
                       std::vector<uint8_t> &seen, std::vector<int> &order) {
  const uint32_t un = (uint32_t)n;
  // rand() % n without a division: Lemire, Kaser and Kurz, "Faster
  // remainder by direct computation" (2019), exact for 32-bit operands
  const uint64_t M = UINT64_C(0xFFFFFFFFFFFFFFFF) / un + 1;
  rng.skip(n);
  seen.assign(n, 0);
  order.resize((size_t)n + 1);
  int cnt = 0;
  uint8_t *sn = seen.data();
  int *od = order.data();
  // the first n distinct values in draw order, branch-free: every draw is
  // written at the end of the list, which grows only when it is new (a
  // block of the stream's words at a time, its position in registers)
  while (cnt < n) {
    int avail;
    const uint32_t *w = rng.peek(avail);
    int k = 0;
    for (; k < avail && cnt < n; k++) {
      const uint32_t r = (uint32_t)(((unsigned __int128)(M * (w[k] >> 1)) * un) >> 64);
      od[cnt] = (int)r;
      cnt += !sn[r];
      sn[r] = 1;
    }
    rng.advance(k);
  }
  if (relabel) {
    for (int k = 0; k < n_class1; k++) labels[order[k]] = 0;
    for (int k = n_class1; k < n; k++) labels[order[k]] = 1;
  }
}

// ------------------------------------------------------------ counter stream
static inline void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[1] = (uint32_t)p1;
    c[3] = (uint32_t)p0;
    c[0] = n0;
    c[2] = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

void counter_labels(uint64_t seed, int set_id, int perm, int n, int n_class1, uint8_t *labels) {
  std::vector<std::pair<uint32_t, int>> kv(n);
  for (int s = 0; s < n; s += 4) {
    uint32_t c[4] = {(uint32_t)(s / 4), (uint32_t)perm, (uint32_t)set_id, 0u};
    philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    for (int j = 0; j < 4 && s + j < n; j++) kv[s + j] = {c[j], s + j};
  }
  std::sort(kv.begin(), kv.end());
  for (int k = 0; k < n; k++) labels[kv[k].second] = (uint8_t)(k < n_class1 ? 0 : 1);
}

// ------------------------------------------------------------ incomplete beta
// Continued fraction of I_x(a,b) (DLMF 8.17.22):
//   I_x(a,b) = x^a (1-x)^b / (a B(a,b)) * 1/(1 + d1/(1 + d2/(1 + ...)))
//   d_{2m+1} = -(a+m)(a+b+m)x / ((a+2m)(a+2m+1)),
//   d_{2m}   =  m(b-m)x / ((a+2m-1)(a+2m)),
// evaluated with the modified Lentz method (Lentz 1976; Thompson & Barnett
// 1986).  Returns 1/(1 + d1/(1 + ...)).
static double beta_cf(double a, double b, double x) {
  const double tiny = 1e-300;
  double f = 1.0, C = 1.0, D = 0.0;
  for (int j = 1; j <= 400000; j++) {
    const int m = j / 2;
    const double dj = (j & 1) ? -((a + m) * (a + b + m) * x) / ((a + 2.0 * m) * (a + 2.0 * m + 1.0))
                              : (m * (b - m) * x) / ((a + 2.0 * m - 1.0) * (a + 2.0 * m));
    D = 1.0 + dj * D;
    if (fabs(D) < tiny) D = tiny;
    D = 1.0 / D;
    C = 1.0 + dj / C;
    if (fabs(C) < tiny) C = tiny;
    const double delta = C * D;
    f *= delta;
    if (fabs(delta - 1.0) < 1e-15) break;
  }
  return 1.0 / f;
}

static double ibeta_lower_cf(double a, double b, double x) {
  const double lfront = a * log(x) + b * log1p(-x) - (lgamma(a) + lgamma(b) - lgamma(a + b));
  return exp(lfront) / a * beta_cf(a, b, x);
}

double ibetac(double a, double b, double x) {
  if (!(a > 0) || !(b > 0) || !std::isfinite(a) || !std::isfinite(b) || !(x >= 0) || !(x <= 1))
    return NAN;
  if (x == 0) return 1.0;
  if (x == 1) return 0.0;
  if (x < (a + 1.0) / (a + b + 2.0)) return 1.0 - ibeta_lower_cf(a, b, x);
  return ibeta_lower_cf(b, a, 1.0 - x);
}

// routines.cu:494-508 and main.cu:1491-1497
bool beta_pddn(const double *js, int R, double &alpha, double &beta, double &pddn) {
  double sum = 0.0;
  for (int i = 0; i < R; i++) sum += js[i];
  const double mu = sum / R;
  double v = 0.0;
  for (int i = 0; i < R; i++) v += pow(js[i] - mu, 2);
  const double var = v / R;
  alpha = (((1 - mu) / var) - (1 / mu)) * pow(mu, 2);
  beta = alpha * (1 / mu - 1);
  if (!(alpha > 0) || !(beta > 0) || !std::isfinite(alpha) || !std::isfinite(beta) ||
      !(js[0] >= 0) || !(js[0] <= 1)) {
    pddn = NAN;
    return false;
  }
  pddn = ibetac(alpha, beta, js[0]);
  return true;
}

// ------------------------------------------------------------ BDeu table
void bdeu_table_into(int n, int64_t *lg, int &shift, int8_t dmap[82]) {
  static const int D[kDivisors] = {1, 2, 3, 4, 6, 8, 9, 12, 16, 18, 24, 27, 36, 54, 81};
  memset(dmap, -1, 82);
  for (int i = 0; i < kDivisors; i++) dmap[D[i]] = (int8_t)i;
  // |partial sums| <= 5 * 512 genes * lgamma(n + 5); keep them below 4e18
  const double bound = 5.0 * 512.0 * (double)lgamma((double)n + 5.0) + 1.0;
  shift = (int)floor(log2(4.0e18 / bound));
  if (shift > 44) shift = 44;
  const long double scale = ldexpl(1.0L, shift);
  for (int i = 0; i < kDivisors; i++) {
    const long double a = 4.0L / (long double)D[i];
    const long double la = lgammal(a);
    for (int m = 0; m <= n; m++)
      lg[(size_t)i * (n + 1) + m] = (int64_t)llroundl((lgammal((long double)m + a) - la) * scale);
  }
}

void bdeu_table(int n, std::vector<int64_t> &lg, int &shift, int8_t dmap[82]) {
  lg.assign((size_t)kDivisors * (n + 1), 0);
  bdeu_table_into(n, lg.data(), shift, dmap);
}

}  // namespace eddy
