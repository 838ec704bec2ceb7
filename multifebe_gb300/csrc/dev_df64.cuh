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

}  // namespace mfb

namespace mfb {

// ---------------------------------------------------------------------------
// Elementary functions in df64, written from their Taylor series with
// Cody-Waite argument reduction (W. J. Cody and W. Waite, "Software Manual for
// the Elementary Functions", 1980): exp on |r| <= ln2/2, sin/cos on |t| <= pi/4.
// Constants are split into hi + lo binary32 pairs on the host (DfConst).
// ---------------------------------------------------------------------------
struct DfConst {
  ff inv_fact[24];  // 1/k!
  ff inv[24];       // 1/k
  ff ln2, pio2;     // ln 2, pi/2
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
  long double f = 1.0L;
  for (int k = 0; k < 24; ++k) {
    if (k > 0) f *= (long double)k;
    c.inv_fact[k] = split(1.0L / f);
    c.inv[k] = k > 0 ? split(1.0L / (long double)k) : ff{0.0f, 0.0f};
  }
  c.ln2 = split(0.693147180559945309417232121458176568L);
  c.pio2 = split(1.570796326794896619231321691639751442L);
  return c;
}

// e^x for |x| <= ~40
__device__ __forceinline__ ff ff_exp(ff x) {
  const float k = rintf(__fmul_rn(x.hi, 1.44269504088896340736f));
  ff r = ff_sub(x, ff_mul(ff{k, 0.0f}, c_df.ln2));
  // sum_{i<=13} r^i / i!
  ff p = c_df.inv_fact[13];
#pragma unroll
  for (int i = 12; i >= 0; --i) p = ff_fma(p, r, c_df.inv_fact[i]);
  const int ki = (int)k;
  return ff{ldexpf(p.hi, ki), ldexpf(p.lo, ki)};
}
// sin x, cos x for |x| <= ~1e4
__device__ __forceinline__ void ff_sincos(ff x, ff* s, ff* c) {
  const float q = rintf(__fmul_rn(x.hi, 0.636619772367581343076f));
  ff t = ff_sub(x, ff_mul(ff{q, 0.0f}, c_df.pio2));
  ff t2 = ff_mul(t, t);
  // sin t = t (1 - t^2/3! + ... - t^18/19!)
  ff ps = ff_neg(c_df.inv_fact[19]);
  ps = ff_fma(ps, t2, c_df.inv_fact[17]);
  ps = ff_fma(ps, t2, ff_neg(c_df.inv_fact[15]));
  ps = ff_fma(ps, t2, c_df.inv_fact[13]);
  ps = ff_fma(ps, t2, ff_neg(c_df.inv_fact[11]));
  ps = ff_fma(ps, t2, c_df.inv_fact[9]);
  ps = ff_fma(ps, t2, ff_neg(c_df.inv_fact[7]));
  ps = ff_fma(ps, t2, c_df.inv_fact[5]);
  ps = ff_fma(ps, t2, ff_neg(c_df.inv_fact[3]));
  ps = ff_fma(ps, t2, c_df.inv_fact[1]);
  ff sn = ff_mul(ps, t);
  // cos t = 1 - t^2/2! + t^4/4! - ... + t^18/18!
  ff pc = c_df.inv_fact[18];
  pc = ff_fma(pc, t2, ff_neg(c_df.inv_fact[16]));
  pc = ff_fma(pc, t2, c_df.inv_fact[14]);
  pc = ff_fma(pc, t2, ff_neg(c_df.inv_fact[12]));
  pc = ff_fma(pc, t2, c_df.inv_fact[10]);
  pc = ff_fma(pc, t2, ff_neg(c_df.inv_fact[8]));
  pc = ff_fma(pc, t2, c_df.inv_fact[6]);
  pc = ff_fma(pc, t2, ff_neg(c_df.inv_fact[4]));
  pc = ff_fma(pc, t2, c_df.inv_fact[2]);
  pc = ff_fma(pc, t2, ff_neg(c_df.inv_fact[0]));
  ff cs = ff_neg(pc);
  const int qi = ((int)q) & 3;
  if (qi == 0) { *s = sn; *c = cs; }
  else if (qi == 1) { *s = cs; *c = ff_neg(sn); }
  else if (qi == 2) { *s = ff_neg(sn); *c = ff_neg(cs); }
  else { *s = ff_neg(cs); *c = sn; }
}

}  // namespace mfb
