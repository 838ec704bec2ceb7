// Double-float ("df64") arithmetic on the FP32 pipe: a value is the unevaluated
// sum hi + lo of two binary32 numbers (about 48 significant bits). Error-free
// transformations after Dekker (1971) and Knuth (TAOCP vol. 2, 4.2.2); all
// operations use the _rn intrinsics so the compiler cannot contract or
// reassociate them. GB300 issues FP32 at 64x its FP64 rate, so df64 arithmetic
// is several times faster than binary64 for multiply-add chains.
//
// Addition is the "sloppy" variant (error about 2^-48 of the larger operand),
// the same error model as a binary64 running sum; it is used only for sums whose
// accuracy target is absolute with respect to the summands.
#pragma once
#include <cuda_runtime.h>

namespace mfb {

struct ff {
  float hi, lo;
};
struct cf {
  ff re, im;
};

__device__ __forceinline__ ff ff_from(double x) {
  float h = __double2float_rn(x);
  float l = __double2float_rn(x - (double)h);
  return ff{h, l};
}
__device__ __forceinline__ double ff_to(ff a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ ff ff_zero() { return ff{0.0f, 0.0f}; }

// a + b
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  float s = __fadd_rn(a.hi, b.hi);
  float v = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  float h = __fadd_rn(s, e);
  return ff{h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
// a * b
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  float h = __fadd_rn(p, e);
  return ff{h, __fsub_rn(e, __fsub_rn(h, p))};
}
// c + a * b
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c) { return ff_add(ff_mul(a, b), c); }

__device__ __forceinline__ cf cf_from(double re, double im) { return cf{ff_from(re), ff_from(im)}; }
__device__ __forceinline__ cf cf_zero() { return cf{ff_zero(), ff_zero()}; }
__device__ __forceinline__ cf cf_add(cf a, cf b) { return cf{ff_add(a.re, b.re), ff_add(a.im, b.im)}; }
__device__ __forceinline__ cf cf_neg(cf a) { return cf{ff_neg(a.re), ff_neg(a.im)}; }
// a * s, s real
__device__ __forceinline__ cf cf_scale(cf a, ff s) { return cf{ff_mul(a.re, s), ff_mul(a.im, s)}; }
// a * b
__device__ __forceinline__ cf cf_mul(cf a, cf b) {
  return cf{ff_sub(ff_mul(a.re, b.re), ff_mul(a.im, b.im)), ff_add(ff_mul(a.re, b.im), ff_mul(a.im, b.re))};
}
// c + a * b
__device__ __forceinline__ cf cf_fma(cf a, cf b, cf c) { return cf_add(cf_mul(a, b), c); }
// c + a * s, s real
__device__ __forceinline__ cf cf_fma_r(cf a, ff s, cf c) { return cf{ff_fma(a.re, s, c.re), ff_fma(a.im, s, c.im)}; }

// Accumulators for long sums of products: (hi, lo) kept unnormalised, each
// product's rounding error (Dekker's exact product) and the addition's error
// (Knuth's TwoSum) gathered in lo -- the compensated dot product of Ogita,
// Rump and Oishi (SIAM J. Sci. Comput. 26(6), 2005) with double-float inputs;
// 12 operations per real multiply-add instead of 17. Normalise before use.
__device__ __forceinline__ void acc_mac(ff& acc, ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const float s = __fadd_rn(acc.hi, p);
  const float bp = __fsub_rn(s, acc.hi);
  const float t = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(t, e));
}
// acc += a * b (complex)
__device__ __forceinline__ void acc_cmac(cf& acc, cf a, cf b) {
  acc_mac(acc.re, a.re, b.re);
  acc_mac(acc.re, ff_neg(a.im), b.im);
  acc_mac(acc.im, a.re, b.im);
  acc_mac(acc.im, a.im, b.re);
}
// acc += a * s (s real)
__device__ __forceinline__ void acc_cmac_r(cf& acc, cf a, ff s) {
  acc_mac(acc.re, a.re, s);
  acc_mac(acc.im, a.im, s);
}
__device__ __forceinline__ ff ff_norm(ff a) {
  const float h = __fadd_rn(a.hi, a.lo);
  return ff{h, __fsub_rn(a.lo, __fsub_rn(h, a.hi))};
}
__device__ __forceinline__ cf cf_norm(cf a) { return cf{ff_norm(a.re), ff_norm(a.im)}; }

}  // namespace mfb

namespace mfb {

// ---------------------------------------------------------------------------
// Elementary functions in df64, written from their Taylor series with
// Cody-Waite argument reduction (W. J. Cody and W. Waite, "Software Manual for
// the Elementary Functions", 1980): e^x = 2^k e^r with |r| <= ln2/2, and
// sin/cos of t = x - q pi/2 with |t| <= pi/4. The reduction constants are held
// as three binary32 parts (72 bits), so the reduced argument keeps full df64
// accuracy for |q| up to 2^20. Constants are split on the host (df_constants_host).
// ---------------------------------------------------------------------------
struct DfConst {
  ff inv_fact[20];  // 1/k!
  ff inv[24];       // 1/k (inv[0] unused)
  ff sin_c[9];      // (-1)^k / (2k+1)!, k = 0..8
  ff cos_c[10];     // (-1)^k / (2k)!,   k = 0..9
  ff zc[16];        // 6! / (6+m)!, m = 0..15: the E_6 series t = sum c_m z^m
  float zc32[16];   // the same in FP32 (the series tail)
  float ln2[3], pio2[3];
};
#ifdef __CUDACC__
__constant__ DfConst c_df;
#endif
inline DfConst df_constants_host() {
  DfConst c;
  auto split = [](long double x) {
    float h = (float)x;
    float l = (float)(x - (long double)h);
    return ff{h, l};
  };
  auto split3 = [](long double x, float* o) {
    o[0] = (float)x;
    long double r = x - (long double)o[0];
    o[1] = (float)r;
    o[2] = (float)(r - (long double)o[1]);
  };
  long double f = 1.0L;
  for (int k = 0; k < 20; ++k) {
    if (k > 0) f *= (long double)k;
    c.inv_fact[k] = split(1.0L / f);
  }
  for (int k = 0; k < 24; ++k) c.inv[k] = k > 0 ? split(1.0L / (long double)k) : ff{0.0f, 0.0f};
  long double g = 1.0L;  // (2k)!
  for (int k = 0; k < 10; ++k) {
    if (k > 0) g *= (long double)(2 * k - 1) * (long double)(2 * k);
    c.cos_c[k] = split((k & 1 ? -1.0L : 1.0L) / g);
    if (k < 9) c.sin_c[k] = split((k & 1 ? -1.0L : 1.0L) / (g * (long double)(2 * k + 1)));
  }
  long double q = 1.0L;
  for (int m = 0; m < 16; ++m) {
    if (m > 0) q /= (long double)(6 + m);
    c.zc[m] = split(q);
    c.zc32[m] = (float)q;
  }
  split3(0.693147180559945309417232121458176568L, c.ln2);
  split3(1.570796326794896619231321691639751442L, c.pio2);
  return c;
}

#ifdef __CUDACC__
// x - q (c0 + c1 + c2) with q an integer-valued float (|q| < 2^20)
__device__ __forceinline__ ff ff_reduce(ff x, float q, const float c[3]) {
  float p0 = __fmul_rn(q, c[0]), e0 = __fmaf_rn(q, c[0], -p0);  // q c0 = p0 + e0 exactly
  float p1 = __fmul_rn(q, c[1]), e1 = __fmaf_rn(q, c[1], -p1);
  ff t = ff_sub(x, ff{p0, e0});
  t = ff_sub(t, ff{p1, e1});
  return ff_sub(t, ff{__fmul_rn(q, c[2]), 0.0f});
}
// sqrt(a), a > 0: one Newton correction of the binary32 root
__device__ __forceinline__ ff ff_sqrt(ff a) {
  float x = __fsqrt_rn(a.hi);
  float p = __fmul_rn(x, x), e = __fmaf_rn(x, x, -p);
  ff d = ff_sub(a, ff{p, e});
  float c = __fdiv_rn(d.hi, __fmul_rn(2.0f, x));
  float h = __fadd_rn(x, c);
  return ff{h, __fsub_rn(c, __fsub_rn(h, x))};
}
// 1 / b: one Newton correction of the binary32 reciprocal
__device__ __forceinline__ ff ff_rcp(ff b) {
  float y = __frcp_rn(b.hi);
  ff e = ff_sub(ff{1.0f, 0.0f}, ff_mul(b, ff{y, 0.0f}));
  float c = __fmul_rn(e.hi, y);
  float h = __fadd_rn(y, c);
  return ff{h, __fsub_rn(c, __fsub_rn(h, y))};
}
// e^x for -87 <= x <= 80 (0 below -87, x clamped to 80 above)
__device__ __forceinline__ ff ff_exp(ff x) {
  if (x.hi < -87.0f) return ff{0.0f, 0.0f};
  if (x.hi > 80.0f) x = ff{80.0f, 0.0f};
  const float k = rintf(__fmul_rn(x.hi, 1.44269504088896340736f));
  ff r = ff_reduce(x, k, c_df.ln2);
  // sum_{i<=13} r^i / i!, |r| <= 0.35: truncation below 2e-18
  ff p = c_df.inv_fact[13];
#pragma unroll 1
  for (int i = 12; i >= 0; --i) p = ff_fma(p, r, c_df.inv_fact[i]);
  // 2^k as a binary32 (k in [-126, 116] for -87 <= x <= 80): exact scaling
  const float s2 = __int_as_float(((int)k + 127) << 23);
  return ff{__fmul_rn(p.hi, s2), __fmul_rn(p.lo, s2)};
}
// sin x, cos x for |x| < 1e6
__device__ __forceinline__ void ff_sincos(ff x, ff* s, ff* c) {
  const float q = rintf(__fmul_rn(x.hi, 0.636619772367581343076f));
  ff t = ff_reduce(x, q, c_df.pio2);
  ff t2 = ff_mul(t, t);
  // |t| <= pi/4: sin to t^17, cos to t^18 (truncation below 1e-19)
  ff ps = c_df.sin_c[8], pc = c_df.cos_c[9];
#pragma unroll 1
  for (int k = 7; k >= 0; --k) {
    ps = ff_fma(ps, t2, c_df.sin_c[k]);
    pc = ff_fma(pc, t2, c_df.cos_c[k + 1]);
  }
  pc = ff_fma(pc, t2, c_df.cos_c[0]);
  const ff sn = ff_mul(ps, t), cs = pc;
  const int qi = ((int)q) & 3;
  if (qi == 0) { *s = sn; *c = cs; }
  else if (qi == 1) { *s = cs; *c = ff_neg(sn); }
  else if (qi == 2) { *s = ff_neg(sn); *c = ff_neg(cs); }
  else { *s = ff_neg(cs); *c = sn; }
}
#endif

}  // namespace mfb
