// Minimal complex(real64) arithmetic for device code. Division follows Smith's
// scaled algorithm, the rule complex(real64) division uses in the reference's
// compiler settings.
#pragma once
#include <cuda_runtime.h>
#include <cmath>

namespace mfb {

struct cd {
  double re, im;
};
__host__ __device__ __forceinline__ cd mk(double r, double i = 0.0) { return cd{r, i}; }
__host__ __device__ __forceinline__ cd operator+(cd a, cd b) { return cd{a.re + b.re, a.im + b.im}; }
__host__ __device__ __forceinline__ cd operator-(cd a, cd b) { return cd{a.re - b.re, a.im - b.im}; }
__host__ __device__ __forceinline__ cd operator-(cd a) { return cd{-a.re, -a.im}; }
__host__ __device__ __forceinline__ cd operator*(cd a, cd b) {
  return cd{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__host__ __device__ __forceinline__ cd operator*(cd a, double s) { return cd{a.re * s, a.im * s}; }
__host__ __device__ __forceinline__ cd operator*(double s, cd a) { return cd{a.re * s, a.im * s}; }
__host__ __device__ __forceinline__ cd operator+(cd a, double s) { return cd{a.re + s, a.im}; }
__host__ __device__ __forceinline__ cd operator+(double s, cd a) { return cd{a.re + s, a.im}; }
__host__ __device__ __forceinline__ cd operator-(cd a, double s) { return cd{a.re - s, a.im}; }
__host__ __device__ __forceinline__ cd operator-(double s, cd a) { return cd{s - a.re, -a.im}; }
__host__ __device__ __forceinline__ cd operator/(cd a, double s) { return cd{a.re / s, a.im / s}; }
__host__ __device__ __forceinline__ cd operator/(cd a, cd b) {
  // Smith (1962)
  if (fabs(b.re) >= fabs(b.im)) {
    double r = b.im / b.re, den = b.re + b.im * r;
    return cd{(a.re + a.im * r) / den, (a.im - a.re * r) / den};
  } else {
    double r = b.re / b.im, den = b.im + b.re * r;
    return cd{(a.re * r + a.im) / den, (a.im * r - a.re) / den};
  }
}
__host__ __device__ __forceinline__ cd operator/(double s, cd b) { return mk(s) / b; }
__host__ __device__ __forceinline__ double cabs_(cd a) { return hypot(a.re, a.im); }
// principal square root
__host__ __device__ __forceinline__ cd csqrt_(cd z) {
  if (z.re == 0.0 && z.im == 0.0) return cd{0.0, z.im};
  double m = hypot(z.re, z.im);
  double t = sqrt(0.5 * (fabs(z.re) + m));
  if (z.re >= 0.0) return cd{t, z.im / (2.0 * t)};
  return cd{fabs(z.im) / (2.0 * t), copysign(t, z.im)};
}
__device__ __forceinline__ cd cexp_(cd z) {
  double s, c;
  sincos(z.im, &s, &c);
  double e = exp(z.re);
  return cd{e * c, e * s};
}

}  // namespace mfb
