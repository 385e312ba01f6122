// afg_math.h -- exp, log and pow in FP64 written for this project, for the
// analytic rate forms of the FP64 transport path.  The same code compiles as
// device code (nvcc) and as host code (g++), and built without floating-point
// contraction (--fmad=false, -ffp-contract=off; the fused multiply-adds are
// written out, and IEEE fma rounds once everywhere) it gives bit-identical
// results on the GPU and in the CPU restatement, which the vendor libraries'
// exp and pow (CUDA's and the C library's) do not.  Accuracy: within two
// units in the last place of the exact value (tested against 60-digit
// values), pow within about |y log x| + 4 units.
//
// exp: the table-driven method of P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989: x = (32 m + j) ln2/32 + r with
// |r| <= ln2/64, exp(x) = 2^m 2^(j/32) exp(r); 2^(j/32) as a leading and a
// trailing double (computed to 200 bits), exp(r) - 1 by its Taylor series
// to r^6 (the first omitted term is below 4e-18 relative).
// log: x = 2^k m with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s) with
// s = (m - 1)/(m + 1), the series 2 (s + s^3/3 + s^5/5 + ...) to s^21
// (Abramowitz and Stegun 4.1.27); ln2 split so that k ln2_hi is exact.
// pow(x, y) = exp(y log x) for x > 0, with the exact cases y = 0, 1, 2 and
// x = 1, and the sign rule for negative x with integer y.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define AFG_MATH_HD __host__ __device__ __forceinline__
#else
#define AFG_MATH_HD inline
#endif

namespace afg_math {

// 2^(j/32), j = 0..31: leading and trailing parts
#define AFG_EXP2_TABLE { \
    {0x1.0000000000000p+0, 0x0.0p+0}, \
    {0x1.059b0d3158574p+0, 0x1.d73e2a475b465p-55}, \
    {0x1.0b5586cf9890fp+0, 0x1.8a62e4adc610bp-54}, \
    {0x1.11301d0125b51p+0, -0x1.6c51039449b3ap-54}, \
    {0x1.172b83c7d517bp+0, -0x1.19041b9d78a76p-55}, \
    {0x1.1d4873168b9aap+0, 0x1.e016e00a2643cp-54}, \
    {0x1.2387a6e756238p+0, 0x1.9b07eb6c70573p-54}, \
    {0x1.29e9df51fdee1p+0, 0x1.612e8afad1255p-55}, \
    {0x1.306fe0a31b715p+0, 0x1.6f46ad23182e4p-55}, \
    {0x1.371a7373aa9cbp+0, -0x1.63aeabf42eae2p-54}, \
    {0x1.3dea64c123422p+0, 0x1.ada0911f09ebcp-55}, \
    {0x1.44e086061892dp+0, 0x1.89b7a04ef80d0p-59}, \
    {0x1.4bfdad5362a27p+0, 0x1.d4397afec42e2p-56}, \
    {0x1.5342b569d4f82p+0, -0x1.07abe1db13cadp-55}, \
    {0x1.5ab07dd485429p+0, 0x1.6324c054647adp-54}, \
    {0x1.6247eb03a5585p+0, -0x1.383c17e40b497p-54}, \
    {0x1.6a09e667f3bcdp+0, -0x1.bdd3413b26456p-54}, \
    {0x1.71f75e8ec5f74p+0, -0x1.16e4786887a99p-55}, \
    {0x1.7a11473eb0187p+0, -0x1.41577ee04992fp-55}, \
    {0x1.82589994cce13p+0, -0x1.d4c1dd41532d8p-54}, \
    {0x1.8ace5422aa0dbp+0, 0x1.6e9f156864b27p-54}, \
    {0x1.93737b0cdc5e5p+0, -0x1.75fc781b57ebcp-57}, \
    {0x1.9c49182a3f090p+0, 0x1.c7c46b071f2bep-56}, \
    {0x1.a5503b23e255dp+0, -0x1.d2f6edb8d41e1p-54}, \
    {0x1.ae89f995ad3adp+0, 0x1.7a1cd345dcc81p-54}, \
    {0x1.b7f76f2fb5e47p+0, -0x1.5584f7e54ac3bp-56}, \
    {0x1.c199bdd85529cp+0, 0x1.11065895048ddp-55}, \
    {0x1.cb720dcef9069p+0, 0x1.503cbd1e949dbp-56}, \
    {0x1.d5818dcfba487p+0, 0x1.2ed02d75b3707p-55}, \
    {0x1.dfc97337b9b5fp+0, -0x1.1a5cd4f184b5cp-54}, \
    {0x1.ea4afa2a490dap+0, -0x1.e9c23179c2893p-54}, \
    {0x1.f50765b6e4540p+0, 0x1.9d3e12dd8a18bp-54} }

#if defined(__CUDACC__)
static __device__ const double kExp2Dev[32][2] = AFG_EXP2_TABLE;
#endif
static const double kExp2Host[32][2] = AFG_EXP2_TABLE;
#undef AFG_EXP2_TABLE

AFG_MATH_HD uint64_t as_u64(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  memcpy(&u, &d, sizeof u);
  return u;
#endif
}
AFG_MATH_HD double as_f64(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double d;
  memcpy(&d, &u, sizeof d);
  return d;
#endif
}
AFG_MATH_HD double exp2_lead(int j) {
#if defined(__CUDA_ARCH__)
  return kExp2Dev[j][0];
#else
  return kExp2Host[j][0];
#endif
}
AFG_MATH_HD double exp2_trail(int j) {
#if defined(__CUDA_ARCH__)
  return kExp2Dev[j][1];
#else
  return kExp2Host[j][1];
#endif
}
// 2^e for e in [-1022, 1023]
AFG_MATH_HD double pow2i(int e) { return as_f64((uint64_t)(e + 1023) << 52); }
AFG_MATH_HD double inf() { return as_f64(0x7FF0000000000000ull); }
AFG_MATH_HD double qnan() { return as_f64(0x7FF8000000000000ull); }
AFG_MATH_HD bool is_nan(double x) { return x != x; }
AFG_MATH_HD double floor_d(double x) {
#if defined(__CUDA_ARCH__)
  return floor(x);
#else
  return __builtin_floor(x);
#endif
}

// a * b + c rounded once (IEEE fused multiply-add, exact on both sides)
AFG_MATH_HD double fma_d(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
  return fma(a, b, c);
#else
  return __builtin_fma(a, b, c);
#endif
}

// y 2^m for y in [0.5, 4) and m in [-1076, 1024], one rounding at most
AFG_MATH_HD double scale(double y, int m) {
  if (m > 1023) return y * pow2i(1023) * pow2i(m - 1023);
  if (m < -1022) return (y * pow2i(m + 600)) * pow2i(-600);
  return y * pow2i(m);
}

AFG_MATH_HD double exp(double x) {
  if (is_nan(x)) return x;
  if (x > 0x1.62e42fefa39efp+9) return inf();   // above log(DBL_MAX)
  if (x < -0x1.74910d52d3052p+9) return 0.0;  // below log of half the smallest subnormal
  const double inv_l = 0x1.71547652b82fep+5;        // 32/ln2
  const double l1 = 0x1.62e42fefa0000p-6;           // ln2/32, 37 leading bits
  const double l2 = 0x1.cf79abc9e3b3ap-45;          // ln2/32 - l1
  const double kd = floor_d(x * inv_l + 0.5);
  const int n = (int)kd;
  const int j = n & 31;
  const int m = (n - j) / 32;
  const double r1 = x - kd * l1;
  const double r2 = -(kd * l2);
  const double r = r1 + r2;
  double poly = fma_d(r, 0x1.6c16c16c16c17p-10, 0x1.1111111111111p-7);
  poly = fma_d(r, poly, 0x1.5555555555555p-5);
  poly = fma_d(r, poly, 0x1.5555555555555p-3);
  poly = fma_d(r, poly, 0x1.0000000000000p-1);
  const double q = (r * r) * poly;
  const double p = r1 + (r2 + q);  // exp(r) - 1
  const double lead = exp2_lead(j), trail = exp2_trail(j);
  const double s = lead + trail;
  return scale(lead + fma_d(s, p, trail), m);
}

AFG_MATH_HD double log(double x) {
  if (is_nan(x)) return x;
  if (x < 0.0) return qnan();
  if (x == 0.0) return -inf();
  uint64_t u = as_u64(x);
  if (u >= 0x7FF0000000000000ull) return x;  // +infinity
  int k = 0;
  if (u < 0x0010000000000000ull) {  // subnormal: scale into the normal range
    x = x * pow2i(54);
    u = as_u64(x);
    k = -54;
  }
  k += (int)(u >> 52) - 1023;
  double mant = as_f64((u & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull);  // [1, 2)
  if (mant > 0x1.6a09e667f3bcdp+0) {
    mant = mant * 0.5;
    k += 1;
  }
  const double f = mant - 1.0;  // exact
  const double s = f / (2.0 + f);
  const double z = s * s;
  double poly = 0x1.8618618618618p-5;
  poly = fma_d(z, poly, 0x1.af286bca1af28p-5);
  poly = fma_d(z, poly, 0x1.e1e1e1e1e1e1ep-5);
  poly = fma_d(z, poly, 0x1.1111111111111p-4);
  poly = fma_d(z, poly, 0x1.3b13b13b13b14p-4);
  poly = fma_d(z, poly, 0x1.745d1745d1746p-4);
  poly = fma_d(z, poly, 0x1.c71c71c71c71cp-4);
  poly = fma_d(z, poly, 0x1.2492492492492p-3);
  poly = fma_d(z, poly, 0x1.999999999999ap-3);
  poly = fma_d(z, poly, 0x1.5555555555555p-2);
  const double s2 = s + s;
  const double lm = fma_d(s2, z * poly, s2);
  if (k == 0) return lm;
  const double kd = (double)k;
  const double ln2_hi = 0x1.62e42fefa3800p-1;  // 42 leading bits of ln2
  const double ln2_lo = 0x1.ef35793c76730p-45; // ln2 - ln2_hi
  return kd * ln2_hi + (kd * ln2_lo + lm);
}

AFG_MATH_HD double pow(double x, double y) {
  if (y == 0.0 || x == 1.0) return 1.0;
  if (is_nan(x) || is_nan(y)) return qnan();
  if (y == 1.0) return x;
  if (y == 2.0) return x * x;
  if (x > 0.0) {
    if (as_u64(x) == 0x7FF0000000000000ull) return y > 0.0 ? x : 0.0;
    return afg_math::exp(y * afg_math::log(x));
  }
  if (x == 0.0) return y > 0.0 ? 0.0 : inf();
  // x < 0: defined for integer y only, negative for odd y
  if (floor_d(y) != y) return qnan();
  const double r = afg_math::exp(y * afg_math::log(-x));
  const double h = y * 0.5;
  return floor_d(h) != h ? -r : r;
}

}  // namespace afg_math
