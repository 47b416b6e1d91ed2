// exact_fp.cuh -- decisions "u < exp(x)" and "log(u) < d" that agree with a
// correctly rounded libm, without paying for FP64 on the common path.
//
// The reference decides Metropolis moves with genrand() < exp(-beta*dE)
// (src/metropolis.F90:802) and Wang-Landau moves with
// log(genrand()) < lng(i) - lng(j) (src/wang-landau.F90:598), where
// genrand() = w * 2^-32 for a 32-bit word w.  On this GPU a dependent FP64
// add takes ~60 cycles and a double exp ~1000, so every decision is first
// tried in FP32 with a rigorous relative error bound; only when w falls
// inside that band is the FP64 value formed, and only when w is within a few
// ulps of the FP64 value is the double-double evaluation below used.
//
// The double-double routines are written from the published constructions:
// Knuth's TwoSum and the FMA-based exact product (Dekker 1971 / Ogita, Rump
// & Oishi 2005), argument reduction exp(x) = 2^k exp(r) with a three-part
// ln 2, and a degree-24 Taylor polynomial evaluated in double-double
// (|r| <= ln2/2 makes the truncation error below 2^-110).  log(u) is one
// Newton step y + (u exp(-y) - 1) in double-double from the FP64 estimate.
#pragma once

#include <cstdint>

namespace brawl {

struct dd {
  double hi, lo;
};

__device__ __forceinline__ dd dd_two_sum(double a, double b) {
  double s = __dadd_rn(a, b);
  double bb = __dsub_rn(s, a);
  double err = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
  return {s, err};
}

__device__ __forceinline__ dd dd_fast_two_sum(double a, double b) {
  double s = __dadd_rn(a, b);
  double err = __dsub_rn(b, __dsub_rn(s, a));
  return {s, err};
}

__device__ __forceinline__ dd dd_add(dd a, dd b) {
  dd s = dd_two_sum(a.hi, b.hi);
  dd t = dd_two_sum(a.lo, b.lo);
  s.lo = __dadd_rn(s.lo, t.hi);
  s = dd_fast_two_sum(s.hi, s.lo);
  s.lo = __dadd_rn(s.lo, t.lo);
  return dd_fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ dd dd_mul(dd a, dd b) {
  double p = __dmul_rn(a.hi, b.hi);
  double e = __fma_rn(a.hi, b.hi, -p);
  e = __fma_rn(a.hi, b.lo, e);
  e = __fma_rn(a.lo, b.hi, e);
  return dd_fast_two_sum(p, e);
}

__device__ __forceinline__ dd dd_mul_d(dd a, double b) {
  double p = __dmul_rn(a.hi, b);
  double e = __fma_rn(a.hi, b, -p);
  e = __fma_rn(a.lo, b, e);
  return dd_fast_two_sum(p, e);
}

// exp(x) for finite x in [-746, 0], to ~2^-104 relative (the result is
// returned unrounded as a double-double).
__device__ inline dd dd_exp(double x) {
  // ln 2 = c1 + c2 + c3 to ~2^-140; c1 and c2 carry 42 significant bits so
  // k*c1 and k*c2 are exact for |k| < 2^11 (values computed from the
  // decimal expansion of ln 2).
  const double ln2_1 = 0x1.62e42fefa3800p-1;
  const double ln2_2 = 0x1.ef35793c76800p-45;
  const double ln2_3 = -0x1.9ff0342542fc3p-90;
  const double inv_ln2 = 1.4426950408889634;
  double k = rint(__dmul_rn(x, inv_ln2));
  // r = x - k*ln2, accumulated in double-double
  dd r = dd_two_sum(x, -__dmul_rn(k, ln2_1));   // k*ln2_1 is exact
  r = dd_add(r, dd{-__dmul_rn(k, ln2_2), 0.0});   // k*ln2_2 is exact
  r = dd_add(r, dd{-__dmul_rn(k, ln2_3), -__fma_rn(k, ln2_3, -__dmul_rn(k, ln2_3))});
  // Taylor polynomial, Horner from degree 24
  dd acc = {1.0, 0.0};
  for (int n = 24; n >= 1; --n) {
    // acc = 1 + r * acc / n
    acc = dd_mul(acc, r);
    double q = __ddiv_rn(acc.hi, (double)n);
    // exact remainder of the division: acc.hi - q*n, plus the low part
    double rem = __fma_rn(-q, (double)n, acc.hi);
    double ql = __ddiv_rn(__dadd_rn(rem, acc.lo), (double)n);
    acc = dd_fast_two_sum(q, ql);
    acc = dd_add(acc, dd{1.0, 0.0});
  }
  int ki = (int)k;
  // scale by 2^k in two steps to stay clear of intermediate overflow/underflow
  int k1 = ki / 2, k2 = ki - k1;
  acc.hi = scalbn(scalbn(acc.hi, k1), k2);
  acc.lo = scalbn(scalbn(acc.lo, k1), k2);
  return acc;
}

// Correctly rounded exp for x <= 0 (ties resolved by the double-double
// renormalisation; a tie within 2^-104 of a rounding boundary is not
// distinguished).
__device__ inline double exp_rn(double x) {
  if (x != x) return x;
  if (x < -745.1332191019412) return 0.0;
  if (x == 0.0) return 1.0;
  dd e = dd_exp(x);
  return __dadd_rn(e.hi, e.lo);
}

// log(u) for u in (0, 1], double-double Newton refinement of the FP64 value.
__device__ inline double log_rn(double u) {
  if (u <= 0.0) return -__longlong_as_double(0x7ff0000000000000LL);  // -inf
  if (u == 1.0) return 0.0;
  double y = log(u);
  dd e = dd_exp(-y);          // exp(-y)
  dd t = dd_mul_d(e, u);      // u * exp(-y) ~ 1
  dd c = dd_add(t, dd{-1.0, 0.0});
  dd yy = dd_add(dd{y, 0.0}, c);
  return __dadd_rn(yy.hi, yy.lo);
}

// ---------------------------------------------------------------------------
// Decisions.  w is the 32-bit word behind genrand() = w * 2^-32.
// Result: 1 accept, 0 reject.  The counters record which tier decided.
// ---------------------------------------------------------------------------
struct DecideStats {
  uint32_t fp64;  // decided with the FP64 libm value
  uint32_t cr;    // needed the double-double value
};

// u < exp(x), x an exact FP64 value (x = -beta*dE as the reference forms it).
__device__ inline int u_lt_exp(uint32_t w, double x, DecideStats& st) {
  if (x != x) return 0;                 // exp(NaN) = NaN: the comparison is false
  if (x >= 0.0) {
    // exp(x) >= 1 > u for every w
    return 1;
  }
  float xf = __double2float_rn(x);
  float D = fabsf(xf) * 1.3e-7f;
  float M = 1.1f * D + 7.0e-7f;
  if (xf < -40.0f) {
    if (w != 0u) return 0;              // u >= 2^-32 > exp(x)
  } else if (M < 0.01f) {
    float thr = __fmul_rn(expf(xf), 4294967296.0f);
    float wf = __uint2float_rn(w);
    if (wf < __fmul_rn(thr, 1.0f - M)) return 1;
    if (wf > __fmul_rn(thr, 1.0f + M)) return 0;
  }
  st.fp64++;
  double E = exp(x);                    // within 1 ulp of exp(x)
  double wu = (double)w;
  double t = __dmul_rn(E, 4294967296.0);
  // a libm result within 1 ulp of exp(x) is within 2 ulp (4.5e-16) of E
  if (wu < __dmul_rn(t, 1.0 - 1.0e-15)) return 1;
  if (wu > __dmul_rn(t, 1.0 + 1.0e-15)) return 0;
  st.cr++;
  double Ecr = exp_rn(x);
  return __dmul_rn(wu, 2.3283064365386963e-10) < Ecr ? 1 : 0;
}

// log(u) < d, d an exact FP64 value.
__device__ inline int log_u_lt(uint32_t w, double d, DecideStats& st) {
  if (d != d) return 0;
  if (w == 0u) return d > -__longlong_as_double(0x7ff0000000000000LL) ? 1 : 0;  // log(0) = -inf
  // log(u) is in [-22.19, 0): decide in FP32 first
  float uf = __fmul_rn(__uint2float_rn(w), 2.3283064365386963e-10f);
  float lf = logf(uf);                  // <= 2 ulp, argument rel. error <= 6e-8
  float df = __double2float_rn(d);
  float tol = fabsf(lf) * 3.0e-7f + 2.0e-7f + fabsf(df) * 1.3e-7f;
  if (lf + tol < df) return 1;
  if (lf - tol > df) return 0;
  st.fp64++;
  double u = __dmul_rn((double)w, 2.3283064365386963e-10);
  double L = log(u);
  double tl = fabs(L) * 1.0e-15 + 1e-300;
  if (L + tl < d) return 1;
  if (L - tl > d) return 0;
  st.cr++;
  return log_rn(u) < d ? 1 : 0;
}

}  // namespace brawl
