// eddy_device.cuh -- device helpers of the EDDY hot path (sm_103a).
//
// Decision arithmetic (kernel1.cu:121-203, 419-431), the rigorous
// leave-one-out filter, capped-parent-list generators (kernel3.cu:41-165),
// network hashing, BDeu in fixed point (kernel5.cu:4-236).
#pragma once
#include <stdint.h>

#include "eddy_internal.h"

namespace eddy {

__device__ __forceinline__ int st_of(int8_t v) { return v == -1 ? 0 : v == 0 ? 1 : v == 1 ? 2 : 3; }

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  // splitmix64 finaliser (Steele, Lea, Flood, OOPSLA'14)
  z ^= z >> 30;
  z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 27;
  z *= 0x94D049BB133111EBull;
  z ^= z >> 31;
  return z;
}
__device__ __forceinline__ uint64_t node_hash_init(uint64_t salt, int t) {
  return mix64(salt ^ ((uint64_t)(t + 1) * 0x9E3779B97F4A7C15ull));
}
__device__ __forceinline__ uint64_t node_hash_step(uint64_t h, int j) {
  return mix64(h ^ ((uint64_t)(j + 1) * 0xC2B2AE3D27D4EB4Full));
}

__device__ __forceinline__ void pair_rc(int p, int &row, int &col) {
  int r = (int)((1.f + sqrtf(1.f + 8.f * (float)p)) * 0.5f);
  while ((long long)r * (r - 1) / 2 > p) r--;
  while ((long long)(r + 1) * r / 2 <= p) r++;
  row = r;
  col = p - r * (r - 1) / 2;
}

// ------------------------------------------------------------ decisions
// RN(n / a) for a divisor a whose odd part A (a = A 2^s) is below 2^18,
// given y = RN(1 / a).  With q0 = RN(n y) (within 1.5 ulp of n / a) and the
// residual r = RN(n - a q0) (one FMA), q0 + r y differs from n / a by less
// than 2^-50 ulp.  n / a is never closer than 2^-19 ulp to a rounding
// midpoint: a midpoint m has an odd 54-bit significand, so a m is a lattice
// point of spacing 2^-53 ulp(m) * a that no 53-bit double n equals, and
// |n / a - m| >= 2^-53 ulp(m) / A.  Hence RN(q0 + r y) = RN(n / a), the
// correctly rounded quotient, in three dependent operations instead of a
// full division.
__device__ __forceinline__ double div_by_small(double n, double a, double y) {
  const double q0 = __dmul_rn(n, y);
  const double r = __fma_rn(-q0, a, n);
  return __fma_rn(r, y, q0);
}

// Exact FP64 evaluation of one table exactly as kernel1.cu:121-203 and
// 419-431 compute it, without FMA contraction (explicit _rn intrinsics).
// Every rounding is the reference's: divisions by the table size use
// div_by_small (N < 2^16), and the AS 147 series step cc x / a, a = p + k
// (p = dof / 2, so the odd part of a is below 2^18), too.
static __device__ __noinline__ int exact_decision(int a0, int a1, int a2, int a3, int a4, int a5,
                                                  int a6, int a7, int a8, int prior,
                                                  const SetDev &sd) {
  const int t9[9] = {a0, a1, a2, a3, a4, a5, a6, a7, a8};
  int ex[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int c = 0; c < 3; c++) {
    for (int c1 = 0; c1 < 3; c1++) ex[c1] += t9[c * 3 + c1];
    for (int b = 0; b < 3; b++) ex[3 + b] += t9[b * 3 + c];
  }
  ex[6] = ex[0] + ex[1] + ex[2];
  const double divisor = (double)ex[6];
  const double rdiv = __drcp_rn(divisor);
  double e[9];
  for (int c = 0; c < 3; c++)
    for (int c1 = 0; c1 < 3; c1++)
      e[c * 3 + c1] = div_by_small(__dmul_rn((double)ex[c1], (double)ex[c + 3]), divisor, rdiv);
  double yates = 0.0;
  bool flag = false;
  for (int c = 0; c < 3 && !flag; c++)
    for (int c1 = 0; c1 < 3; c1++)
      if ((e[c * 3 + c1] < 5) && (ex[c1] && ex[c + 3])) {
        yates = 0.5;
        flag = true;
        break;
      }
  double chi = 0.0;
  int dofn = 0, dofm = 0;
  for (int ii = 0; ii < 3; ii++) {
    if (ex[ii] == 0) dofm++;
    if (ex[ii + 3] == 0) dofn++;
    for (int jj = 0; jj < 3; jj++)
      if ((ex[jj] * ex[ii + 3]) != 0) {
        double d = __dsub_rn(fabs(__dsub_rn((double)t9[ii * 3 + jj], e[ii * 3 + jj])), yates);
        chi = __dadd_rn(chi, __ddiv_rn(__dmul_rn(d, d), e[ii * 3 + jj]));
      }
  }
  const int dof = ((3 - dofm) - 1) * ((3 - dofn) - 1);
  // AS 147 (kernel1.cu:10-74)
  const double x = chi / 2.0, p = ((double)dof) / 2.0;
  double G = 0.0;
  if (x > 0.0 && p > 0.0) {
    double arg = __dsub_rn(__dsub_rn(__dmul_rn(p, log(x)), lgamma(p + 1.0)), x);
    if (!(arg < log(1.0e-37))) {
      double f = exp(arg);
      if (f != 0.0) {
        // for it < 100000: a += 1; cc = cc x / a; value += cc; stop when
        // cc <= 1e-9 value.  Four steps per round, the stop tests after
        // them (the steps past the stop are discarded); the reciprocals of
        // the next round's divisors are formed off the dependent chain.
        double cc = 1.0, value = 1.0, a = __dadd_rn(p, 1.0);
        double y0 = __drcp_rn(a), y1 = __drcp_rn(__dadd_rn(a, 1.0)),
               y2 = __drcp_rn(__dadd_rn(a, 2.0)), y3 = __drcp_rn(__dadd_rn(a, 3.0));
        for (int it = 0; it < 100000; it += 4) {
          const double a1 = __dadd_rn(a, 1.0), a2 = __dadd_rn(a, 2.0), a3 = __dadd_rn(a, 3.0);
          const double an = __dadd_rn(a, 4.0);
          const double z0 = __drcp_rn(an), z1 = __drcp_rn(__dadd_rn(an, 1.0)),
                       z2 = __drcp_rn(__dadd_rn(an, 2.0)), z3 = __drcp_rn(__dadd_rn(an, 3.0));
          const double c0 = div_by_small(__dmul_rn(cc, x), a, y0);
          const double c1 = div_by_small(__dmul_rn(c0, x), a1, y1);
          const double c2 = div_by_small(__dmul_rn(c1, x), a2, y2);
          const double c3 = div_by_small(__dmul_rn(c2, x), a3, y3);
          const double v0 = __dadd_rn(value, c0), v1 = __dadd_rn(v0, c1);
          const double v2 = __dadd_rn(v1, c2), v3 = __dadd_rn(v2, c3);
          if (c0 <= __dmul_rn(1.0e-09, v0)) { value = v0; break; }
          if (c1 <= __dmul_rn(1.0e-09, v1)) { value = v1; break; }
          if (c2 <= __dmul_rn(1.0e-09, v2)) { value = v2; break; }
          value = v3;
          if (c3 <= __dmul_rn(1.0e-09, v3)) break;
          cc = c3;
          a = an;
          y0 = z0;
          y1 = z1;
          y2 = z2;
          y3 = z3;
        }
        G = __dmul_rn(value, f);
      }
    }
  }
  double ev = 1.0 - G;
  if (sd.bonf) {
    double m = __dmul_rn(ev, (double)(((sd.g - 1) * sd.g) / 2));
    ev = (1.0 < m) ? 1.0 : m;
  }
  return (ev < sd.alpha_edge || (prior == 1 && ev < sd.alpha_edge_prior)) ? 1 : 0;
}

struct TabInfo {
  int R[3], C[3], N;
  int rm, cm;   // smallest nonzero row / column marginal
  int dof;      // (2 - #zero cols)(2 - #zero rows)
  int yates;    // 1 if the Yates correction applies
  float chi;    // FP32 chi-square
};

__device__ __forceinline__ int dof_slot(int dof) { return dof == 1 ? 0 : dof == 2 ? 1 : dof == 4 ? 2 : -1; }

// Hardware reciprocal approximation (relative error a few 1e-8 for normal
// inputs): every use below sits inside an error budget of >= 1e-5.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// FP32 chi-square of a 3x3 table: (1/N) sum (|N o - R C| - yN)^2 / (R C),
// numerators exact in 32-bit integers (tables of N <= 32767 samples; larger
// ones take the exact FP64 path).  Returns the marginals too.
constexpr int kFastMaxN = 32767;
__device__ __forceinline__ void table_info(const int *t, TabInfo &ti) {
  ti.R[0] = t[0] + t[1] + t[2];
  ti.R[1] = t[3] + t[4] + t[5];
  ti.R[2] = t[6] + t[7] + t[8];
  ti.C[0] = t[0] + t[3] + t[6];
  ti.C[1] = t[1] + t[4] + t[7];
  ti.C[2] = t[2] + t[5] + t[8];
  ti.N = ti.R[0] + ti.R[1] + ti.R[2];
  int zr = (ti.R[0] == 0) + (ti.R[1] == 0) + (ti.R[2] == 0);
  int zc = (ti.C[0] == 0) + (ti.C[1] == 0) + (ti.C[2] == 0);
  ti.dof = (2 - zc) * (2 - zr);
  const int N = ti.N;
  int rm = 0x7fffffff, cm = 0x7fffffff;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (ti.R[a] > 0 && ti.R[a] < rm) rm = ti.R[a];
    if (ti.C[a] > 0 && ti.C[a] < cm) cm = ti.C[a];
  }
  ti.rm = rm;
  ti.cm = cm;
  if (N > kFastMaxN) {
    ti.yates = 0;
    ti.chi = 0.f;
    return;
  }
  // rm * cm <= N^2 < 2^30 here
  ti.yates = (N > 0 && rm * cm < 5 * N) ? 1 : 0;
  // chi = (1/4N) sum_a (1/R_a) sum_b num_ab^2 / C_b: six reciprocals
  float invC[3];
#pragma unroll
  for (int b = 0; b < 3; b++) invC[b] = ti.C[b] ? rcp_approx((float)ti.C[b]) : 0.f;
  float chi = 0.f;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (ti.R[a] == 0) continue;
    float row = 0.f;
#pragma unroll
    for (int b = 0; b < 3; b++) {
      if (ti.C[b] != 0) {
        int d = N * t[a * 3 + b] - ti.R[a] * ti.C[b];
        d = d < 0 ? -d : d;
        const int num2 = ti.yates ? (2 * d - N) : (2 * d);  // 2(|d| - yN), |.| < 2^31
        const float nf = (float)num2;
        row = fmaf(nf * nf, invC[b], row);
      }
    }
    chi = fmaf(row, rcp_approx((float)ti.R[a]), chi);
  }
  ti.chi = (N > 0) ? chi * rcp_approx(4.f * (float)N) : 0.f;
}

// 0/1 when certain from the FP32 value, 2 when the exact path must decide.
__device__ __forceinline__ int fast_decision(const TabInfo &ti, int prior, const SetDev &sd) {
  if (sd.exact_all || ti.N == 0 || ti.N > kFastMaxN) return 2;
  int ds = dof_slot(ti.dof);
  if (ds < 0) return 0;  // dof 0: p = 1, never below an alpha <= 1
  const Thr &T = sd.thr[prior][ds];
  const float x = ti.chi;
  if (x < T.fA) return 0;
  if (x > T.fB && x < T.fKlo) return 1;
  if (x > T.fKhi) return 0;
  return 2;
}

__device__ __forceinline__ int decide(const int *t, int prior, const SetDev &sd, TabInfo &ti,
                                      unsigned &nexact) {
  table_info(t, ti);
  int d = fast_decision(ti, prior, sd);
  if (d == 2) {
    nexact++;
    d = exact_decision(t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8], prior, sd);
  }
  return d;
}

// Rigorous leave-one-out filter.  True when every table t - e_ab (one
// sample of any cell removed) is certain to get the same decision as t.
// Bound: with u_rc = (|o-e|-y)/sqrt(e), chi = |u|^2 and Minkowski,
// |sqrt(chi') - sqrt(chi)| <= A + B sqrt(chi), A^2 <= 15/e'min + 5/(N-1),
// B = max_rc |sqrt(e/e') - 1|; requires unchanged support (marginals >= 2),
// unchanged Yates flag and N >= 32.
__device__ __forceinline__ bool loo_safe(const TabInfo &ti, int prior, const SetDev &sd) {
  if (sd.exact_all || ti.N < 32 || ti.N > kFastMaxN) return false;
  const int rm = ti.rm, cm = ti.cm;
  if (rm < 2 || cm < 2) return false;
  const int ds = dof_slot(ti.dof);
  if (ds < 0) return true;  // support unchanged: dof stays 0, p = 1
  const int N = ti.N;  // <= 32767: the products below fit in 32 bits
  if (ti.yates) {
    if (!(rm * cm < 5 * (N - 1))) return false;
  } else {
    if (!((rm - 1) * (cm - 1) >= 5 * (N - 1))) return false;
  }
  // fast reciprocals / square roots (a few ulp) with explicit 1e-5 safety
  // factors in the conservative direction
  const float lo = 0.99999f, hi = 1.00001f;
  const float inv_n1 = rcp_approx((float)(N - 1));
  const float emin = (float)((rm - 1) * (cm - 1)) * inv_n1 * lo;       // lower bound
  const float a2 = (15.f * rcp_approx(emin) + 5.f * inv_n1) * hi;
  const float A = a2 * rsqrtf(a2) * hi;                                 // sqrt(a2), upper
  const float ratio = (float)(rm * cm) * rcp_approx((float)((rm - 1) * (cm - 1))) * hi;
  const float B = fmaxf(ratio * rsqrtf(ratio) * hi - 1.f, inv_n1 * hi) * 1.001f;
  const float rel = 2e-5f;
  const float xs = ti.chi * (1.f + rel);
  const float sup = (xs > 0.f ? xs * rsqrtf(xs) : 0.f) * hi;
  const float xl = ti.chi * (1.f - rel);
  const float slo = (xl > 0.f ? xl * rsqrtf(xl) : 0.f) * lo;
  const float D = (A + B * sup) * 1.01f + 1e-3f;
  const float whi = (sup + D) * (sup + D) * 1.0001f;
  const float wl = fmaxf(slo - D, 0.f);
  const float wlo = wl * wl * 0.9999f;
  const Thr &T = sd.thr[prior][ds];
  if (whi < T.chiA) return true;
  if (wlo > T.chiB && whi < T.kLo) return true;
  if (wlo > T.kHi) return true;
  return false;
}

// Cheap rigorous filter for the common case "no edge in any of the ten
// tables".  With every marginal >= 2 and every expected count >= 5 in t and
// in each t' = t - e_ab (support, dof and the Yates flag unchanged), chi^2 =
// N(Q - 1) with Q = sum o^2/(R C), and o' <= o, R' >= R - 1, C' >= C - 1 give
// Q' <= rho Q with rho = rm cm / ((rm - 1)(cm - 1)), so
//   chi^2(t') = (N - 1)(Q' - 1) <= N (rho - 1) + rho chi^2(t).
// Below the dof's no-edge threshold, all ten decisions are 0.
__device__ __forceinline__ bool quick_zero(const TabInfo &ti, int prior, const SetDev &sd) {
  const int N = ti.N, rm = ti.rm, cm = ti.cm;
  if (sd.exact_all || N < 32 || N > kFastMaxN || rm < 2 || cm < 2) return false;
  const int ds = dof_slot(ti.dof);
  if (ds < 0) return false;
  const int q = (rm - 1) * (cm - 1);  // products < 2^30 for N <= 32767
  if (q < 5 * (N - 1) || rm * cm < 5 * N) return false;
  // rho - 1 = (rm + cm - 1) / q; FP32 errors covered by the 1e-4 factors
  const float r1 = (float)(rm + cm - 1) * rcp_approx((float)q) * 1.0001f;
  const float xs = ti.chi * (1.f + 2e-5f);
  const float bound = fmaf((float)N, r1, (1.f + r1) * xs) * 1.0001f + 1e-3f;
  return bound < sd.thr[prior][ds].chiA;
}

// Packed FP32 pairs (add/sub/mul/fma .rn.f32x2, sm_100 and later): two
// lanes per instruction.  quick_zero_f2 (below) runs quick_zero's bound on
// both classes of a pair at once, lane x = class 1, lane y = class 2.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f2_pack(float x, float y) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
  return r;
}
__device__ __forceinline__ float f2_x(f32x2 v) {
  float x;
  asm("{.reg .f32 t; mov.b64 {%0, t}, %1;}" : "=f"(x) : "l"(v));
  return x;
}
__device__ __forceinline__ float f2_y(f32x2 v) {
  float y;
  asm("{.reg .f32 t; mov.b64 {t, %0}, %1;}" : "=f"(y) : "l"(v));
  return y;
}
__device__ __forceinline__ f32x2 f2_add(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
// quick_zero on the FP32 counts of the tensor-core epilogue, both classes
// of a pair at once: o[k] = {class-1 count, class-2 count} of cell k, exact
// floats; bit 0 / bit 1 of the result: class 1 / class 2 settled (no edge
// in any of its ten tables).  Demands every marginal >= 2 (dof 4 in t and every
// t', support unchanged), Yates off everywhere and N <= 4096, so that every
// marginal product below is an exact FP32 integer.  The test of quick_zero,
//   (N (rho - 1) + rho chi_hi) 1.0001 + 1e-3 < chiA,
// chi_hi = N (Q - 1) + 1e-5 N, rho = rm cm / q, q = (rm - 1)(cm - 1),
// multiplied through by q D with D = R0 R1 R2 C0 C1 C2 > 0, so no division
// is left on the path:  Q D = sum_a PR_a sum_b o_ab^2 PC_b, PR_a / PC_b =
// the products of the other two marginals.  FP32 error of Q D - D:
// <= 6e-7 D (all products of marginals exact, o^2 exact), i.e. <= 6e-7 N in
// chi^2, inside the 1e-5 N term; the other roundings are relative 1e-6,
// inside the 1.0001 and 1e-3 terms.  chiA: the no-edge threshold of dof 4
// (negative: never).
__device__ __forceinline__ unsigned quick_zero_f2(const f32x2 *o, float chiA) {
  const f32x2 one = f2_pack(1.f, 1.f);
  const f32x2 R0 = f2_add(f2_add(o[0], o[1]), o[2]), R1 = f2_add(f2_add(o[3], o[4]), o[5]),
              R2 = f2_add(f2_add(o[6], o[7]), o[8]);
  const f32x2 C0 = f2_add(f2_add(o[0], o[3]), o[6]), C1 = f2_add(f2_add(o[1], o[4]), o[7]),
              C2 = f2_add(f2_add(o[2], o[5]), o[8]);
  const f32x2 N = f2_add(f2_add(R0, R1), R2);
  const float rmx = fminf(f2_x(R0), fminf(f2_x(R1), f2_x(R2)));
  const float rmy = fminf(f2_y(R0), fminf(f2_y(R1), f2_y(R2)));
  const float cmx = fminf(f2_x(C0), fminf(f2_x(C1), f2_x(C2)));
  const float cmy = fminf(f2_y(C0), fminf(f2_y(C1), f2_y(C2)));
  const f32x2 rm = f2_pack(rmx, rmy), cm = f2_pack(cmx, cmy);
  const f32x2 q = f2_mul(f2_sub(rm, one), f2_sub(cm, one)), rc = f2_mul(rm, cm);
  const float Nx = f2_x(N), Ny = f2_y(N);
  const bool okx = rmx >= 2.f && cmx >= 2.f && Nx >= 32.f && Nx <= 4096.f &&
                   f2_x(q) >= 5.f * (Nx - 1.f) && f2_x(rc) >= 5.f * Nx;
  const bool oky = rmy >= 2.f && cmy >= 2.f && Ny >= 32.f && Ny <= 4096.f &&
                   f2_y(q) >= 5.f * (Ny - 1.f) && f2_y(rc) >= 5.f * Ny;
  const f32x2 PR0 = f2_mul(R1, R2), PR1 = f2_mul(R0, R2), PR2 = f2_mul(R0, R1);
  const f32x2 PC0 = f2_mul(C1, C2), PC1 = f2_mul(C0, C2), PC2 = f2_mul(C0, C1);
  const f32x2 D = f2_mul(f2_mul(R0, PR0), f2_mul(C0, PC0));
  const f32x2 s0 = f2_fma(f2_mul(o[0], o[0]), PC0,
                          f2_fma(f2_mul(o[1], o[1]), PC1, f2_mul(f2_mul(o[2], o[2]), PC2)));
  const f32x2 s1 = f2_fma(f2_mul(o[3], o[3]), PC0,
                          f2_fma(f2_mul(o[4], o[4]), PC1, f2_mul(f2_mul(o[5], o[5]), PC2)));
  const f32x2 s2 = f2_fma(f2_mul(o[6], o[6]), PC0,
                          f2_fma(f2_mul(o[7], o[7]), PC1, f2_mul(f2_mul(o[8], o[8]), PC2)));
  const f32x2 QD = f2_fma(PR0, s0, f2_fma(PR1, s1, f2_mul(PR2, s2)));
  // q D bound = (N (rm + cm - 1) + rc (N (Q - 1) + 1e-5 N)) D
  const f32x2 rcN = f2_mul(rc, N);
  const f32x2 t1 = f2_fma(N, f2_sub(f2_add(rm, cm), one), f2_mul(rcN, f2_pack(1e-5f, 1e-5f)));
  const f32x2 lhs = f2_fma(t1, D, f2_mul(rcN, f2_sub(QD, D)));
  const f32x2 qD = f2_mul(q, D);
  const f32x2 L = f2_fma(lhs, f2_pack(1.0001f, 1.0001f), f2_mul(f2_pack(1e-3f, 1e-3f), qD));
  const f32x2 Rr = f2_mul(f2_pack(chiA, chiA), qD);
  return ((okx && f2_x(L) < f2_x(Rr)) ? 1u : 0u) | ((oky && f2_y(L) < f2_y(Rr)) ? 2u : 0u);
}

// The general path: full-table decision, the Minkowski leave-one-out filter
// and, when that cannot settle them, the nine cell-removed tables one by one.
// Counts by value and not inlined: it runs for a small share of the tables.
// Returns the mask in bits 0-9, the number of exact evaluations in bits
// 32-47 and 1 in bit 48 when the filter settled the table.
static __device__ __noinline__ uint64_t pair_mask_general(int a0, int a1, int a2, int a3, int a4,
                                                          int a5, int a6, int a7, int a8,
                                                          int prior, const SetDev &sd) {
  int t[9] = {a0, a1, a2, a3, a4, a5, a6, a7, a8};
  TabInfo ti;
  unsigned nexact = 0;
  const int bit0 = decide(t, prior, sd, ti, nexact);
  if (loo_safe(ti, prior, sd))
    return (bit0 ? 0x3FFull : 0ull) | ((uint64_t)nexact << 32) | (1ull << 48);
  uint32_t m = (uint32_t)bit0;
#pragma unroll 1
  for (int cell = 0; cell < 9; cell++) {
    int bit = bit0;
    if (t[cell] > 0) {
      t[cell]--;
      TabInfo tj;
      bit = decide(t, prior, sd, tj, nexact);
      t[cell]++;
    }
    m |= (uint32_t)bit << (1 + cell);
  }
  return m | ((uint64_t)nexact << 32);
}

// 10-bit decision mask of one (pair, class) table: bit 0 = full table,
// bit 1+3a+b = table with one sample of cell (a,b) removed.
__device__ __forceinline__ uint32_t pair_mask(const int *t, int prior, const SetDev &sd,
                                              unsigned &nexact, unsigned &nfilt) {
  TabInfo ti;
  table_info(t, ti);
  if (quick_zero(ti, prior, sd)) {
    nfilt++;
    return 0u;
  }
  const uint64_t r =
      pair_mask_general(t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8], prior, sd);
  nexact += (unsigned)(r >> 32) & 0xFFFFu;
  nfilt += (unsigned)(r >> 48) & 1u;
  return (uint32_t)r & 0x3FFu;
}

// --------------------------------------------------- capped parent lists
// Generates the parent list of node t (ascending gene index) of the network
// "full network of class k with the pair tables of sample sigma removed":
// row bits of the full network XOR the flips that sigma's cells trigger.
struct ListGen {
  const uint32_t *row;   // GW words, bit j = edge (t, j), j < t
  const uint32_t *phi;   // flip entries (p << 9 | flipbits), sorted by p
  const uint16_t *pcol;  // column of each flip entry
  const int8_t *stsig;   // states (0..3) of all genes at sample sigma, or null
  int fi, fe, w, GW, strow;
  uint32_t word;

  __device__ __forceinline__ uint32_t flipword(int ww) {
    uint32_t m = 0;
    if (stsig == nullptr || strow > 2) {
      return 0;
    }
    const int hi = 32 * (ww + 1);
    while (fi < fe) {
      int col = pcol[fi];
      if (col >= hi) break;
      int sc = stsig[col];
      if (sc <= 2) {
        uint32_t bits = phi[fi] & 0x1FFu;
        if ((bits >> (strow * 3 + sc)) & 1u) m |= 1u << (col - 32 * ww);
      }
      fi++;
    }
    return m;
  }
  __device__ __forceinline__ void init(const uint32_t *row_, int GW_, const uint32_t *phi_,
                                       const uint16_t *pcol_, int fi_, int fe_,
                                       const int8_t *stsig_, int strow_) {
    row = row_;
    GW = GW_;
    phi = phi_;
    pcol = pcol_;
    fi = fi_;
    fe = fe_;
    stsig = stsig_;
    strow = strow_;
    w = 0;
    word = (GW > 0) ? (row[0] ^ flipword(0)) : 0u;
  }
  __device__ __forceinline__ int next() {
    while (true) {
      if (word) {
        int j = __ffs(word) - 1;
        word &= word - 1;
        return 32 * w + j;
      }
      if (++w >= GW) return -1;
      word = row[w] ^ flipword(w);
    }
  }
};

// ------------------------------------------------------------------ BDeu
static __device__ __constant__ int8_t c_dmap[82];

// BDeu score of node t without parents over the samples of one class
// (fixed point): with its observed-state count r and state counts N_k in
// the class (kernel5.cu:30-218 for q = 1), sum_k LG(r)[N_k] - LG(1)[sum_k
// N_k], LG(d)[m] = lgamma(m + 4/d) - lgamma(4/d).  Nodes with parents are
// scored as flat tasks (bdeu_config_term).
static __device__ int64_t bdeu_score0(const SetDev &sd, int t,
                                      const uint16_t *cnt3 /*[g][3] of this class*/) {
  int r = 0, nij = 0;
  int64_t sc = 0;
  for (int a = 0; a < 3; a++) r += cnt3[t * 3 + a] > 0;
  if (r == 0) return 0;
  const int64_t *LG1 = sd.lg + (size_t)c_dmap[r] * sd.lg_stride;
  for (int a = 0; a < 3; a++) {
    const int cnt = cnt3[t * 3 + a];
    if (cnt > 0) {
      nij += cnt;
      sc += LG1[cnt];
    }
  }
  return sc - sd.lg[(size_t)c_dmap[1] * sd.lg_stride + nij];
}

// Parent configurations of node t's score (np >= 1 parents) in one class:
// q = product of the parents' observed-state counts (0: the score is 0).
__device__ __forceinline__ int bdeu_q(const uint16_t *cnt3, int np, int p0, int p1, int p2) {
  const int idx[3] = {p0, p1, p2};
  int q = 1;
  for (int k = 0; k < np; k++) {
    const uint16_t *c = cnt3 + idx[k] * 3;
    q *= (c[0] > 0) + (c[1] > 0) + (c[2] > 0);
  }
  return q;
}
// Tasks of node t's score in one class: one per configuration of the
// parents after the first (the first parent's states are summed within a
// task), q / (the first parent's observed-state count), 0 when q is 0.
__device__ __forceinline__ int bdeu_tasks(const uint16_t *cnt3, int np, int p0, int p1, int p2) {
  const int q = bdeu_q(cnt3, np, p0, p1, p2);
  if (q == 0) return 0;
  const uint16_t *c = cnt3 + p0 * 3;
  return q / ((c[0] > 0) + (c[1] > 0) + (c[2] > 0));
}

// The terms of kernel5.cu:30-218 for the parent configurations of task j
// of node t's score over class mask m: configuration j of the parents after
// the first, with every observed state of the first parent, i.e.
//   sum over those configurations of  sum_k LG(q r)[N_jk] - LG(q)[N_j].
// Summing the terms of all tasks gives the node's score (fixed point,
// exact, in any order).  dmap: the divisor map in shared memory.
static __device__ __noinline__ int64_t bdeu_config_term(const SetDev &sd, int t, int np, int p0,
                                                        int p1, int p2, const uint64_t *m,
                                                        const uint16_t *cnt3, int j,
                                                        const int8_t *dmap) {
  int nstate[4], st[4][3];
  const int idx[4] = {t, p0, p1, p2};
  for (int k = 0; k <= np; k++) {
    int c = 0;
    for (int a = 0; a < 3; a++)
      if (cnt3[idx[k] * 3 + a] > 0) st[k][c++] = a;
    nstate[k] = c;
  }
  const int r = nstate[0];
  int q = 1;
  for (int k = 1; k <= np; k++) q *= nstate[k];
  const int W = sd.W;
  const uint64_t *P = sd.planes;
  const int64_t *LGq = sd.lg + (size_t)dmap[q] * sd.lg_stride;
  const int64_t *LGqr = (r > 0) ? sd.lg + (size_t)dmap[q * r] * sd.lg_stride : LGq;
  // plane rows as word offsets into the planes: the other parents' (the
  // first parent's own row again when absent: ANDing it twice changes
  // nothing), the first parent's observed states (repeated past its count;
  // unused), the child's states
  auto row_of = [&](int gene, int s) { return (gene * 3 + s) * W; };
  int rem = j;
  const int n1 = nstate[1];
  const int oa0 = row_of(p0, st[1][0]);
  const int oa1 = row_of(p0, st[1][n1 > 1 ? 1 : 0]);
  const int oa2 = row_of(p0, st[1][n1 > 2 ? 2 : 0]);
  int ob[2] = {-1, -1};
  for (int k = 2; k <= np; k++) {
    const int s = st[k][rem % nstate[k]];
    rem /= nstate[k];
    ob[k - 2] = row_of(idx[k], s);
  }
  const int ot0 = row_of(t, r > 0 ? st[0][0] : 0);
  const int ot1 = row_of(t, r > 1 ? st[0][1] : 0);
  const int ot2 = row_of(t, r > 2 ? st[0][2] : 0);
  int c00 = 0, c01 = 0, c02 = 0, c10 = 0, c11 = 0, c12 = 0, c20 = 0, c21 = 0, c22 = 0;
  const bool has2 = ob[0] >= 0, has3 = ob[1] >= 0;
  const int ob0 = has2 ? ob[0] : 0, ob1 = has3 ? ob[1] : 0;
  for (int w = 0; w < W; w++) {
    uint64_t pm = m[w];
    if (has2) pm &= P[ob0 + w];
    if (has3) pm &= P[ob1 + w];
    const uint64_t x0 = P[ot0 + w], x1 = P[ot1 + w], x2 = P[ot2 + w];
    const uint64_t y0 = pm & P[oa0 + w], y1 = pm & P[oa1 + w], y2 = pm & P[oa2 + w];
    c00 += __popcll(y0 & x0);
    c01 += __popcll(y0 & x1);
    c02 += __popcll(y0 & x2);
    c10 += __popcll(y1 & x0);
    c11 += __popcll(y1 & x1);
    c12 += __popcll(y1 & x2);
    c20 += __popcll(y2 & x0);
    c21 += __popcll(y2 & x1);
    c22 += __popcll(y2 & x2);
  }
  // one configuration's terms: counts x0, x1, x2 of the child's states
  auto conf = [&](int x0, int x1, int x2) -> int64_t {
    int64_t v = 0;
    int nij = 0;
    if (r > 0) { nij += x0; v += LGqr[x0]; }
    if (r > 1) { nij += x1; v += LGqr[x1]; }
    if (r > 2) { nij += x2; v += LGqr[x2]; }
    return v - LGq[nij];
  };
  int64_t term = conf(c00, c01, c02);
  if (n1 > 1) term += conf(c10, c11, c12);
  if (n1 > 2) term += conf(c20, c21, c22);
  return term;
}

}  // namespace eddy
