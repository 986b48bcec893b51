// morton_grid.h -- one axis of the 64-bit Morton grid coordinate on the
// single-precision pipe, for the device kernels and a host test.
//
// The reference computes (c * scale + offset) * 2^21 in f64 and converts it
// with `as u32` (src/ploc/mod.rs:782-785, src/ploc/morton.rs); the kernels
// fold 2^21 into S and O, so the coordinate is sat_u32(RN(RN(c * S) + O))
// with c the f32 centre widened to f64.  GB300's double-precision pipe is
// narrow, so where it is provably the same value, this computes the floor
// from float pieces instead:
//
//   S = s1 + s2 + s3 and O = o1 + o2 + o3 exactly (mg_split3, per block;
//   |s2| <= 2^-24 |s1|, |s3| <= 2^-48 |s1|, the same for O); c * s1 as a
//   rounded product and its exact error (an fma: the fma two-product of
//   Ogita, Rump and Oishi, "Accurate sum and dot product", 2005), c * s2
//   rounded; p1 + o1 = h + t by Knuth's exact two-sum (TAOCP vol. 2, 4.2.2);
//   l = (t + q1) + (p2 + o2).  With M = max(|p1|, |o1|, |h|), the terms left
//   out (c * s3, the error of c * s2, o3) are below 3.1 * 2^-48 M and l's
//   three roundings below 2^-44.9 M, so h + l is within 2^-44.4 M of
//   v = c * S + O, and the reference's two roundings put px within
//   2^-51.9 M of v.  With f = RN(frac(h) + l), px is within
//   E = 2^-40 M + 2^-22 |f| + 2^-21 of floor(h) + f (margins of 16x and 4x,
//   and an absolute slack for tiny terms), so when frac(f) lies in (E, 1 - E)
//   floor(px) = floor(h) + floor(f).  Otherwise (a value within E of an
//   integer, a scene far from the origin for its size, inputs outside the
//   ranges the bound assumes) morton_floor_fast returns false and the caller
//   computes in double precision.
//
// Host builds must not contract a * b + c into an fma (-ffp-contract=off):
// every operation here is one IEEE single-precision operation, rounded to
// nearest, on both sides.
#pragma once
#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define MG_HD __host__ __device__ __forceinline__
#else
#define MG_HD static inline
#endif

MG_HD float mg_mul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
MG_HD float mg_add(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
MG_HD float mg_sub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
MG_HD float mg_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}

struct MortonAxis {
  float s1, s2, o1, o2;  // the leading two floats of S's and O's exact three-float splits
  int ok;                // both splits exact, |s1| in [2^-20, 2^60], |o1| <= 2^60
};

// d = f1 + f2 + f3 exactly (each difference below is exact in double);
// false when the three floats do not hold d.
MG_HD int mg_split3(double d, float* f1, float* f2, float* f3) {
  const float a = (float)d;
  const double r1 = d - (double)a;
  const float b = (float)r1;
  const double r2 = r1 - (double)b;
  const float c = (float)r2;
  *f1 = a;
  *f2 = b;
  *f3 = c;
  return isfinite(a) && isfinite(d) && r2 - (double)c == 0.0;
}

MG_HD struct MortonAxis morton_axis(double S, double O) {
  struct MortonAxis m;
  float s3, o3;
  const int sok = mg_split3(S, &m.s1, &m.s2, &s3);
  const int ook = mg_split3(O, &m.o1, &m.o2, &o3);
  const float as = fabsf(m.s1), ao = fabsf(m.o1);
  m.ok = sok && ook && as >= 0x1p-20f && as <= 0x1p60f && ao <= 0x1p60f;
  return m;
}

// floor(RN(RN(c * S) + O)) into *k when the float pieces decide it (true);
// false: the caller computes the coordinate in double precision.
MG_HD int morton_floor_fast(float c, const struct MortonAxis* a, long long* k) {
  const float ac = fabsf(c);
  if (!a->ok || !(ac <= 0x1p40f) || (ac != 0.0f && ac < 0x1p-20f)) return 0;  // NaN fails ac <= 2^40
  const float p1 = mg_mul(c, a->s1), q1 = mg_fma(c, a->s1, -p1);
  const float p2 = mg_mul(c, a->s2);
  const float h = mg_add(p1, a->o1);
  const float z = mg_sub(h, p1);
  const float t = mg_add(mg_sub(p1, mg_sub(h, z)), mg_sub(a->o1, z));
  const float l = mg_add(mg_add(t, q1), mg_add(p2, a->o2));
  const float m = fmaxf(fabsf(p1), fmaxf(fabsf(a->o1), fabsf(h)));
  const float fh = floorf(h);
  const float f = mg_add(mg_sub(h, fh), l);
  const float g = floorf(f);
  const float fr = mg_sub(f, g);
  const float e = mg_add(mg_add(mg_mul(m, 0x1p-40f), mg_mul(fabsf(f), 0x1p-22f)), 0x1p-21f);
  if (!(fr > e && fr < mg_sub(1.0f, e))) return 0;
  *k = (long long)fh + (long long)g;
  return 1;
}
