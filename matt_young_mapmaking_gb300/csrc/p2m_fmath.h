/*
 * p2m_fmath.h -- exact-rounding arithmetic macros and a portable single-precision
 * math library shared by the GPU painter and the CPU oracle.
 *
 * Why this exists.  The reference (Fortran, pks2map_src/) evaluates its per-halo and
 * per-pixel quantities in single precision with the compiler runtime's float
 * intrinsics: asin (haloproject.f90:47,105-106), x**(1./3.) (pks2map.f90:298),
 * log and tan (maptable.f90:185,196-202), exp/atan/sin/x**y in the table maker
 * (maptable.f90:100-118, bbps_profile.f90:91-111, integrate_profiles.f90:28,70).
 * Several of those results feed integer truncations (table indices, flat-sky box
 * bounds) and the float-rounded disc test, so two implementations that differ by one
 * ulp give visibly different maps.  Rather than depend on whichever libm or CUDA math
 * library is linked, both sides call the functions below, which are built from IEEE
 * basic operations only (+ - * / sqrt with round-to-nearest, no FMA contraction) and
 * therefore return bit-identical results on x86-64, aarch64 and sm_103a.
 *
 * Methods (all standard, coefficients are exact Taylor coefficients rounded to float):
 *   log:  x = 2^e m, m in (sqrt(1/2), sqrt(2)];  log m = 2 atanh((m-1)/(m+1)) by its
 *         odd series; e*ln2 added with a Cody-Waite split of ln2.
 *   exp:  x = k ln2 + r (Cody-Waite), |r| <= ln2/2, Taylor series to r^7, scale by 2^k.
 *   pow:  2^(y log2 x) with y*e split so the integer part is exact (see p2m_powf).
 *   asin: odd Taylor series on |x| <= 1/2; asin x = pi/2 - 2 asin(sqrt((1-x)/2)) above.
 *   atan: odd Taylor series on |x| <= sqrt(2)-1; pi/4 + atan((x-1)/(x+1)) up to 1;
 *         pi/2 - atan(1/x) beyond.
 *   sin/cos/tan: x = k pi/2 + r with a three-part Cody-Waite split of pi/2 (valid for
 *         |x| < 2^12 pi/2), Taylor series for sin r and cos r on |r| <= pi/4.
 * Accuracy against correctly rounded results (a few ulp) is tested by
 * tests/test_capi_cpu.py (test_float_math_accuracy, test_pow_accuracy_and_special_cases);
 * bit-identity between host and device by
 * tests/test_gpu_parity.py::test_fmath_bit_identical_host_device.
 */
#ifndef P2M_FMATH_H
#define P2M_FMATH_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define P2M_HD __host__ __device__ __forceinline__
#else
#define P2M_HD static inline
#endif

/* ---- exact basic operations: never contracted into FMA ------------------------ */
#if defined(__CUDA_ARCH__)
#define FADD(a, b) __fadd_rn((a), (b))
#define FSUB(a, b) __fsub_rn((a), (b))
#define FMUL(a, b) __fmul_rn((a), (b))
#define FDIV(a, b) __fdiv_rn((a), (b))
#define FSQRT(a) __fsqrt_rn((a))
#define DADD(a, b) __dadd_rn((a), (b))
#define DSUB(a, b) __dsub_rn((a), (b))
#define DMUL(a, b) __dmul_rn((a), (b))
#define DDIV(a, b) __ddiv_rn((a), (b))
#define DSQRT(a) __dsqrt_rn((a))
#else
/* host code is compiled with -ffp-contract=off; SSE2/NEON float ops are IEEE */
#define FADD(a, b) ((float)((float)(a) + (float)(b)))
#define FSUB(a, b) ((float)((float)(a) - (float)(b)))
#define FMUL(a, b) ((float)((float)(a) * (float)(b)))
#define FDIV(a, b) ((float)((float)(a) / (float)(b)))
#define FSQRT(a) p2m_host_sqrtf((float)(a))
#define DADD(a, b) ((double)(a) + (double)(b))
#define DSUB(a, b) ((double)(a) - (double)(b))
#define DMUL(a, b) ((double)(a) * (double)(b))
#define DDIV(a, b) ((double)(a) / (double)(b))
#define DSQRT(a) p2m_host_sqrt((double)(a))
#include <math.h>
static inline float p2m_host_sqrtf(float a) { return sqrtf(a); }
static inline double p2m_host_sqrt(double a) { return sqrt(a); }
#endif

P2M_HD uint32_t p2m_f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}
P2M_HD float p2m_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

P2M_HD int p2m_isnanf(float x) { return x != x; }
P2M_HD float p2m_nanf(void) { return p2m_u2f(0x7fc00000u); }
P2M_HD float p2m_inff(void) { return p2m_u2f(0x7f800000u); }
P2M_HD float p2m_fabsf(float x) { return p2m_u2f(p2m_f2u(x) & 0x7fffffffu); }

/* 2^k as a float for -126 <= k <= 127 */
P2M_HD float p2m_pow2i(int k) { return p2m_u2f((uint32_t)(k + 127) << 23); }

/* round to nearest integer, ties away from zero (|x| < 2^30) */
P2M_HD int p2m_rint_away(float x) {
  return (int)(x >= 0.0f ? FADD(x, 0.5f) : FSUB(x, 0.5f));
}

/* ---- constants ------------------------------------------------------------------ */
#define P2M_LN2_HI 6.931457520e-01f   /* 0x3f317200: ln2 with 16 significant bits */
#define P2M_LN2_LO 1.428606765e-06f   /* 0x35bfbe8e: ln2 - LN2_HI */
#define P2M_LN2 6.931471825e-01f      /* 0x3f317218 */
#define P2M_INV_LN2 1.442695022e+00f  /* 0x3fb8aa3b */
#define P2M_SQRT2 1.414213538e+00f    /* 0x3fb504f3 */
#define P2M_SQRT2M1 4.142135680e-01f  /* 0x3ed413cd */
#define P2M_PIO2_1 1.570312500e+00f   /* 0x3fc90000: pi/2, first 12 bits */
#define P2M_PIO2_2 4.837512970e-04f   /* 0x39fda000: next 12 bits */
#define P2M_PIO2_3 7.549790126e-08f   /* 0x33a22169: remainder */
#define P2M_TWO_OVER_PI 6.366197467e-01f /* 0x3f22f983 */
#define P2M_PIO2_HI 1.570796371e+00f  /* 0x3fc90fdb: float(pi/2) */
#define P2M_PIO2_LO -4.371138829e-08f /* 0xb33bbd2e: pi/2 - PIO2_HI */
#define P2M_PIO4_HI 7.853981853e-01f  /* 0x3f490fdb: float(pi/4) */
#define P2M_PIO4_LO -2.185569414e-08f /* 0xb2bbbd2e */

/* ---- log -------------------------------------------------------------------------- */
/* splits x > 0 (finite) into m in (sqrt(1/2), sqrt(2)] and integer e, x = m 2^e */
P2M_HD float p2m_frexp_centered(float x, int *e_out) {
  uint32_t u = p2m_f2u(x);
  int e = (int)((u >> 23) & 0xffu);
  if (e == 0) { /* subnormal: scale by 2^24 exactly */
    x = FMUL(x, 16777216.0f);
    u = p2m_f2u(x);
    e = (int)((u >> 23) & 0xffu) - 24;
  }
  e -= 127;
  float m = p2m_u2f((u & 0x007fffffu) | 0x3f800000u);
  if (m > P2M_SQRT2) {
    m = FMUL(m, 0.5f);
    e += 1;
  }
  *e_out = e;
  return m;
}

/* log(m) for m in (sqrt(1/2), sqrt(2)]: 2 atanh(f), f = (m-1)/(m+1), |f| <= 0.1716 */
P2M_HD float p2m_log_core(float m) {
  float f = FDIV(FSUB(m, 1.0f), FADD(m, 1.0f));
  float f2 = FADD(f, f);
  float w = FMUL(f, f);
  /* 1/3 + w/5 + w^2/7 + w^3/9 + w^4/11; truncation error < 2.1e-9 relative */
  float t = FADD(1.111111119e-01f, FMUL(w, 9.090909362e-02f));
  t = FADD(1.428571492e-01f, FMUL(w, t));
  t = FADD(2.000000030e-01f, FMUL(w, t));
  t = FADD(3.333333433e-01f, FMUL(w, t));
  t = FMUL(w, t);
  return FADD(f2, FMUL(f2, t));
}

P2M_HD float p2m_logf(float x) {
  if (p2m_isnanf(x) || x < 0.0f) return p2m_nanf();
  if (x == 0.0f) return -p2m_inff();
  if (x == p2m_inff()) return x;
  int e;
  float m = p2m_frexp_centered(x, &e);
  float lm = p2m_log_core(m);
  float fe = (float)e;
  /* e*LN2_HI is exact (|e| <= 150, LN2_HI has 16 significant bits) */
  return FADD(FMUL(fe, P2M_LN2_HI), FADD(lm, FMUL(fe, P2M_LN2_LO)));
}

/* p2m_logf for a positive, normal, finite x, without the special-value tests (which
   such an x never takes): the same result bit for bit */
P2M_HD float p2m_logf_normal(float x) {
  int e;
  float m = p2m_frexp_centered(x, &e);
  float lm = p2m_log_core(m);
  float fe = (float)e;
  return FADD(FMUL(fe, P2M_LN2_HI), FADD(lm, FMUL(fe, P2M_LN2_LO)));
}

/* ---- exp -------------------------------------------------------------------------- */
/* exp(r) for |r| <= ~0.36 */
P2M_HD float p2m_exp_core(float r) {
  float p = FADD(1.388888923e-03f, FMUL(r, 1.984127011e-04f));
  p = FADD(8.333333768e-03f, FMUL(r, p));
  p = FADD(4.166666791e-02f, FMUL(r, p));
  p = FADD(1.666666716e-01f, FMUL(r, p));
  p = FADD(5.000000000e-01f, FMUL(r, p));
  p = FMUL(FMUL(r, r), p); /* r^2/2 + r^3/6 + ... + r^7/5040 */
  return FADD(1.0f, FADD(r, p));
}

/* p * 2^k for any integer k in [-300, 300] */
P2M_HD float p2m_scale2(float p, int k) {
  if (k > 127) {
    p = FMUL(p, p2m_pow2i(127));
    k -= 127;
    if (k > 127) k = 127;
    return FMUL(p, p2m_pow2i(k));
  }
  if (k < -126) {
    p = FMUL(p, p2m_pow2i(-126));
    k += 126;
    if (k < -126) k = -126;
    return FMUL(p, p2m_pow2i(k));
  }
  return FMUL(p, p2m_pow2i(k));
}

P2M_HD float p2m_expf(float x) {
  if (p2m_isnanf(x)) return x;
  if (x > 88.7228394f) return p2m_inff();
  if (x < -104.0f) return 0.0f;
  int k = p2m_rint_away(FMUL(x, P2M_INV_LN2));
  float fk = (float)k;
  float r = FSUB(FSUB(x, FMUL(fk, P2M_LN2_HI)), FMUL(fk, P2M_LN2_LO));
  return p2m_scale2(p2m_exp_core(r), k);
}

/* ---- pow -------------------------------------------------------------------------- */
/*
 * x^y for x > 0 as 2^(y log2 x).  With x = m 2^e, y*log2 x = y*e + y*log2(m).  y is
 * split into yh (12 leading bits) + yl so that yh*e and yl*e are exact; the integer
 * part n of yh*e is removed exactly, leaving |r| <~ 0.5 + |y|/2 whose only rounding
 * error is that of y*log2(m).  Special cases follow C99 for the arguments this code
 * meets: y == 0 or x == 1 -> 1, y == 1 -> x, x == 0 -> 0 (y > 0) or inf (y < 0).
 */
P2M_HD float p2m_powf(float x, float y) {
  if (y == 0.0f || x == 1.0f) return 1.0f;
  if (p2m_isnanf(x) || p2m_isnanf(y)) return p2m_nanf();
  if (y == 1.0f) return x;
  if (x < 0.0f) return p2m_nanf(); /* never reached by the map-making path */
  if (x == 0.0f) return y > 0.0f ? 0.0f : p2m_inff();
  if (x == p2m_inff()) return y > 0.0f ? x : 0.0f;
  int e;
  float m = p2m_frexp_centered(x, &e);
  float l2m = FMUL(p2m_log_core(m), P2M_INV_LN2); /* log2(m), |l2m| <= 1/2 */
  float yh = p2m_u2f(p2m_f2u(y) & 0xfffff000u);
  float yl = FSUB(y, yh);
  float fe = (float)e;
  float ph = FMUL(yh, fe); /* exact */
  float pl = FMUL(yl, fe); /* exact */
  float q = FMUL(y, l2m);
  float t_est = FADD(FADD(ph, pl), q);
  if (t_est > 128.5f) return p2m_inff();
  if (t_est < -150.5f) return 0.0f;
  int n = p2m_rint_away(ph);
  float r = FADD(FADD(FSUB(ph, (float)n), pl), q); /* ph - n exact */
  int n2 = p2m_rint_away(r);
  r = FSUB(r, (float)n2);
  n += n2;
  /* 2^r = exp(r ln2) with r ln2 carried in two parts */
  float rl = FADD(FMUL(r, P2M_LN2_HI), FMUL(r, P2M_LN2_LO));
  return p2m_scale2(p2m_exp_core(rl), n);
}

/* ---- asin ------------------------------------------------------------------------- */
/* asin(x) for |x| <= 1/2: x + x w P(w), w = x^2 (Taylor through x^21) */
P2M_HD float p2m_asin_core(float x) {
  float w = FMUL(x, x);
  float p = FADD(9.761609137e-03f, FMUL(w, 8.390335366e-03f));
  p = FADD(1.155180112e-02f, FMUL(w, p));
  p = FADD(1.396484394e-02f, FMUL(w, p));
  p = FADD(1.735276356e-02f, FMUL(w, p));
  p = FADD(2.237215824e-02f, FMUL(w, p));
  p = FADD(3.038194403e-02f, FMUL(w, p));
  p = FADD(4.464285821e-02f, FMUL(w, p));
  p = FADD(7.500000298e-02f, FMUL(w, p));
  p = FADD(1.666666716e-01f, FMUL(w, p));
  return FADD(x, FMUL(FMUL(x, w), p));
}

P2M_HD float p2m_asinf(float x) {
  if (p2m_isnanf(x)) return x;
  float a = p2m_fabsf(x);
  if (a > 1.0f) return p2m_nanf();
  float r;
  if (a <= 0.5f) {
    r = p2m_asin_core(a);
  } else {
    float z = FSQRT(FMUL(FSUB(1.0f, a), 0.5f)); /* 1-a exact */
    float s = p2m_asin_core(z);
    /* pi/2 - 2s with pi/2 in two parts */
    r = FADD(FSUB(P2M_PIO2_HI, FADD(s, s)), P2M_PIO2_LO);
  }
  return x < 0.0f ? -r : r;
}

/* ---- atan ------------------------------------------------------------------------- */
/* atan(x) for |x| <= sqrt(2)-1 (Taylor through x^21) */
P2M_HD float p2m_atan_core(float x) {
  float w = FMUL(x, x);
  float p = FADD(-5.263157934e-02f, FMUL(w, 4.761904851e-02f));
  p = FADD(5.882352963e-02f, FMUL(w, p));
  p = FADD(-6.666667014e-02f, FMUL(w, p));
  p = FADD(7.692307979e-02f, FMUL(w, p));
  p = FADD(-9.090909362e-02f, FMUL(w, p));
  p = FADD(1.111111119e-01f, FMUL(w, p));
  p = FADD(-1.428571492e-01f, FMUL(w, p));
  p = FADD(2.000000030e-01f, FMUL(w, p));
  p = FADD(-3.333333433e-01f, FMUL(w, p));
  return FADD(x, FMUL(FMUL(x, w), p));
}

P2M_HD float p2m_atanf(float x) {
  if (p2m_isnanf(x)) return x;
  float a = p2m_fabsf(x);
  float r;
  if (a > 1.0f) {
    if (a == p2m_inff()) {
      r = P2M_PIO2_HI;
    } else {
      float inv = FDIV(1.0f, a);
      float t = (inv <= P2M_SQRT2M1)
                    ? p2m_atan_core(inv)
                    : FADD(FADD(P2M_PIO4_HI, p2m_atan_core(FDIV(FSUB(inv, 1.0f), FADD(inv, 1.0f)))),
                           P2M_PIO4_LO);
      r = FADD(FSUB(P2M_PIO2_HI, t), P2M_PIO2_LO);
    }
  } else if (a <= P2M_SQRT2M1) {
    r = p2m_atan_core(a);
  } else {
    r = FADD(FADD(P2M_PIO4_HI, p2m_atan_core(FDIV(FSUB(a, 1.0f), FADD(a, 1.0f)))), P2M_PIO4_LO);
  }
  return x < 0.0f ? -r : r;
}

/* ---- sin / cos / tan ----------------------------------------------------------- */
P2M_HD float p2m_sin_core(float r) { /* |r| <= pi/4 */
  float w = FMUL(r, r);
  float p = FADD(2.755731884e-06f, FMUL(w, -2.505210794e-08f));
  p = FADD(-1.984127011e-04f, FMUL(w, p));
  p = FADD(8.333333768e-03f, FMUL(w, p));
  p = FADD(-1.666666716e-01f, FMUL(w, p));
  return FADD(r, FMUL(FMUL(r, w), p));
}
P2M_HD float p2m_cos_core(float r) { /* |r| <= pi/4 */
  float w = FMUL(r, r);
  float p = FADD(-2.755731998e-07f, FMUL(w, 2.087675588e-09f));
  p = FADD(2.480158764e-05f, FMUL(w, p));
  p = FADD(-1.388888923e-03f, FMUL(w, p));
  p = FADD(4.166666791e-02f, FMUL(w, p));
  float hw = FMUL(w, 0.5f);
  /* 1 - w/2 + w^2 p */
  return FADD(FSUB(1.0f, hw), FMUL(FMUL(w, w), p));
}
/* x = k pi/2 + r, returns r and k mod 4 (for |x| < 2^12 pi/2) */
P2M_HD float p2m_reduce_pio2(float x, int *q) {
  int k = p2m_rint_away(FMUL(x, P2M_TWO_OVER_PI));
  float fk = (float)k;
  float r = FSUB(FSUB(FSUB(x, FMUL(fk, P2M_PIO2_1)), FMUL(fk, P2M_PIO2_2)), FMUL(fk, P2M_PIO2_3));
  *q = k & 3;
  return r;
}
P2M_HD float p2m_sinf(float x) {
  if (p2m_isnanf(x) || p2m_fabsf(x) == p2m_inff()) return p2m_nanf();
  int q;
  float r = p2m_reduce_pio2(x, &q);
  switch (q) {
    case 0: return p2m_sin_core(r);
    case 1: return p2m_cos_core(r);
    case 2: return -p2m_sin_core(r);
    default: return -p2m_cos_core(r);
  }
}
P2M_HD float p2m_cosf(float x) {
  if (p2m_isnanf(x) || p2m_fabsf(x) == p2m_inff()) return p2m_nanf();
  int q;
  float r = p2m_reduce_pio2(x, &q);
  switch (q) {
    case 0: return p2m_cos_core(r);
    case 1: return -p2m_sin_core(r);
    case 2: return -p2m_cos_core(r);
    default: return p2m_sin_core(r);
  }
}
P2M_HD float p2m_tanf(float x) {
  if (p2m_isnanf(x) || p2m_fabsf(x) == p2m_inff()) return p2m_nanf();
  int q;
  float r = p2m_reduce_pio2(x, &q);
  float s = p2m_sin_core(r), c = p2m_cos_core(r);
  return (q & 1) ? -FDIV(c, s) : FDIV(s, c);
}
/* p2m_tanf for 0 <= x < pi/4: there the reduction is an identity (k = 0, r = x) and the
   argument tests never fire, so this is the same result bit for bit */
P2M_HD float p2m_tanf_pio4(float x) { return FDIV(p2m_sin_core(x), p2m_cos_core(x)); }

#endif /* P2M_FMATH_H */
