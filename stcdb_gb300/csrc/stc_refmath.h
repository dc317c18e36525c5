/*
 * The reference's geographic arithmetic, evaluated bit-exactly on host and
 * device.
 *
 * The reference computes (util/util.h:57-66, geometry/geometry.h:40-48,
 * :166-185), in IEEE double with no fused multiply-add (its x86-64 build has
 * no FMA):
 *   dpm_lat     = 360.0/(40076.0*1000.0)
 *   dpml(lat)   = 360.0/(sin((90-|lat|)*PI/180)*40076.0*1000.0), PI = 3.14159265
 *   distance    = sqrt(dx*dx+dy*dy), dx = (x1-x2)/dpml(y1), dy = (y1-y2)/dpm_lat
 * Every +, -, *, /, sqrt below is spelled with a round-to-nearest primitive
 * so that no compiler can contract or reassociate it.
 *
 * sin: correctly rounded sine for |x| <= 2, written for this project from the
 * Taylor series sin x = sum (-1)^k x^(2k+1)/(2k+1)! evaluated in double-double
 * arithmetic (Dekker 1971 / Knuth TwoSum and TwoProduct via fma), then rounded
 * to the nearest double. The double-double sum has relative error below
 * 2^-100, so the rounding is correct except when sin x lies within 2^-100 of
 * a rounding midpoint. It is tested against host libm sin over the latitude
 * range in tests/test_refmath.py.
 */
#ifndef STC_REFMATH_H
#define STC_REFMATH_H

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define STC_HD __host__ __device__ __forceinline__
#else
#define STC_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define RN_ADD(a, b) __dadd_rn((a), (b))
#define RN_SUB(a, b) __dsub_rn((a), (b))
#define RN_MUL(a, b) __dmul_rn((a), (b))
#define RN_DIV(a, b) __ddiv_rn((a), (b))
#define RN_SQRT(a) __dsqrt_rn(a)
#define RN_FMA(a, b, c) __fma_rn((a), (b), (c))
#else
/* host: compiled with -ffp-contract=off, so plain operators are exact IEEE */
#define RN_ADD(a, b) ((a) + (b))
#define RN_SUB(a, b) ((a) - (b))
#define RN_MUL(a, b) ((a) * (b))
#define RN_DIV(a, b) ((a) / (b))
#define RN_SQRT(a) sqrt(a)
#define RN_FMA(a, b, c) fma((a), (b), (c))
#endif

#define STC_REF_PI 3.14159265
#define STC_EMPTY_KEY (1ULL << 62)

STC_HD double stc_dpm_lat() { return RN_DIV(360.0, RN_MUL(40076.0, 1000.0)); }

/* double-double helpers */
typedef struct { double hi, lo; } stc_dd;

STC_HD stc_dd dd_two_sum(double a, double b) {
  double s = RN_ADD(a, b);
  double bb = RN_SUB(s, a);
  double e = RN_ADD(RN_SUB(a, RN_SUB(s, bb)), RN_SUB(b, bb));
  stc_dd r = {s, e};
  return r;
}

STC_HD stc_dd dd_fast_two_sum(double a, double b) {
  double s = RN_ADD(a, b);
  double e = RN_SUB(b, RN_SUB(s, a));
  stc_dd r = {s, e};
  return r;
}

STC_HD stc_dd dd_add(stc_dd a, stc_dd b) {
  stc_dd s = dd_two_sum(a.hi, b.hi);
  stc_dd t = dd_two_sum(a.lo, b.lo);
  s.lo = RN_ADD(s.lo, t.hi);
  s = dd_fast_two_sum(s.hi, s.lo);
  s.lo = RN_ADD(s.lo, t.lo);
  return dd_fast_two_sum(s.hi, s.lo);
}

STC_HD stc_dd dd_mul(stc_dd a, stc_dd b) {
  double p = RN_MUL(a.hi, b.hi);
  double e = RN_FMA(a.hi, b.hi, -p);
  e = RN_ADD(e, RN_ADD(RN_MUL(a.hi, b.lo), RN_MUL(a.lo, b.hi)));
  return dd_fast_two_sum(p, e);
}

STC_HD stc_dd dd_div_d(stc_dd a, double b) {
  double q1 = RN_DIV(a.hi, b);
  /* r = a - q1*b exactly enough */
  double p = RN_MUL(q1, b);
  double pe = RN_FMA(q1, b, -p);
  stc_dd r = dd_two_sum(a.hi, -p);
  r.lo = RN_ADD(RN_SUB(r.lo, pe), a.lo);
  double q2 = RN_DIV(RN_ADD(r.hi, r.lo), b);
  return dd_fast_two_sum(q1, q2);
}

/* Correctly rounded sin(x) for |x| <= 2 (see the file comment). */
STC_HD double stc_sin_cr(double x) {
  stc_dd xx = {x, 0.0};
  stc_dd x2 = dd_mul(xx, xx);
  stc_dd term = xx;
  stc_dd sum = xx;
  for (int k = 1; k <= 22; k++) {
    /* term *= -x^2 / ((2k)(2k+1)) */
    term = dd_mul(term, x2);
    term = dd_div_d(term, (double)((2 * k) * (2 * k + 1)));
    term.hi = -term.hi;
    term.lo = -term.lo;
    sum = dd_add(sum, term);
  }
  return RN_ADD(sum.hi, sum.lo);
}

/* util/util.h:59-66, with the correctly rounded sine. */
STC_HD double stc_dpml_ref(double latitude) {
  double absla = fabs(latitude);
  if (absla == 90) absla = 89;
  double arg = RN_DIV(RN_MUL(RN_SUB(90.0, absla), STC_REF_PI), 180.0);
  return RN_DIV(360.0, RN_MUL(RN_MUL(stc_sin_cr(arg), 40076.0), 1000.0));
}

/* geometry/geometry.h:40-48 (p1 = this: longitude scale at y1). */
STC_HD double stc_distance_ref(double x1, double y1, double x2, double y2, double dpml1) {
  double dx = RN_SUB(x1, x2);
  double dy = RN_SUB(y1, y2);
  dy = RN_DIV(dy, stc_dpm_lat());
  dx = RN_DIV(dx, dpml1);
  return RN_SQRT(RN_ADD(RN_MUL(dx, dx), RN_MUL(dy, dy)));
}

/* geometry/geometry.h:174-185 (box::distance, geography = true). */
STC_HD double stc_box_distance_ref(double lx, double ly, double hx, double hy, double x, double y,
                                   double dpml_y) {
  if (x >= lx && x <= hx && y >= ly && y <= hy) return 0;
  /* x/2 and x*0.5 round identically (exact scaling by a power of two) */
  double dx = RN_SUB(fabs(RN_SUB(x, RN_MUL(RN_ADD(lx, hx), 0.5))), RN_MUL(RN_SUB(hx, lx), 0.5));
  double dy = RN_SUB(fabs(RN_SUB(y, RN_MUL(RN_ADD(ly, hy), 0.5))), RN_MUL(RN_SUB(hy, ly), 0.5));
  if (dx < 0.0) dx = 0.0;
  if (dy < 0.0) dy = 0.0;
  dy = RN_DIV(dy, stc_dpm_lat());
  dx = RN_DIV(dx, dpml_y);
  return RN_SQRT(RN_ADD(RN_MUL(dx, dx), RN_MUL(dy, dy)));
}

/* geometry/geometry.h:166-172 (box::width, geography = true). */
STC_HD double stc_box_width_ref(double lx, double ly, double hx) {
  return RN_DIV(RN_SUB(hx, lx), stc_dpml_ref(ly));
}

/* util/util.h:68-70 */
STC_HD uint64_t stc_cantor(uint32_t a, uint32_t b) {
  uint64_t s = (uint64_t)(uint32_t)(a + b);
  return s * (uint64_t)(uint32_t)(a + b + 1) / 2 + b;
}

#endif
