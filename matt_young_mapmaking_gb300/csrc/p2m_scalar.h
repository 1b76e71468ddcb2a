/*
 * p2m_scalar.h -- scalar arithmetic of the pks2map path shared by the CUDA kernels and
 * the host-side set-up code (cosmology tables).  Every routine reproduces the float /
 * double evaluation order of the reference Fortran (pks2map_src/, HEALPix 3.10) with
 * the exact-rounding macros of p2m_fmath.h, so host and device give identical bits.
 */
#ifndef P2M_SCALAR_H
#define P2M_SCALAR_H

#include "p2m_fmath.h"

#define P2M_NZTAB 10000
#define P2M_MAXMAPS 8
#define P2M_MAXTABLES 8

/* healpix_types.F90:65-73 */
#define P2M_HP_HALFPI 1.570796326794896619231321691639751442099
#define P2M_HP_PI 3.141592653589793238462643383279502884197
#define P2M_HP_TWOPI 6.283185307179586476925286766559005768394
/* cosmology.f90:8-9: the double parameter pi holds the single-precision literal */
#define P2M_COSMO_PI 3.1415927410125732421875
/* cosmology.f90:11-23 */
#define P2M_CKMS (2.99792458e10 / 1e5)

/* Background cosmology of pks2map.f90:118-128 plus the r(z), z(r) tables of
   cosmology.f90:51-105 (serial float Euler integration). */
typedef struct p2m_cosmo {
  float omegam, omegab, omegal, h, fb, rho_0, rhocrit_0, mypi;
  float drofz, dzofr;
} p2m_cosmo;

/* cosmology.f90:123-133 */
P2M_HD float p2m_dzdr(const p2m_cosmo *c, float z) {
  float zp1 = FADD(1.0f, z);
  float c3 = FMUL(FMUL(zp1, zp1), zp1);
  float s = FSQRT(FSUB(FADD(FMUL(c->omegam, c3), 1.0f), c->omegam));
  double t = DDIV((double)FMUL(c->h, 100.0f), P2M_CKMS);
  return (float)DMUL(t, (double)s);
}

/* pks2map.f90:88,118-128 and cosmology.f90:51-105; rofz/zofr receive 10000 floats */
static inline void p2m_cosmo_build(p2m_cosmo *c, float *rofz, float *zofr) {
  c->omegam = 0.25f;
  c->omegab = 0.043f;
  c->omegal = 0.75f;
  c->h = 0.7f;
  c->fb = FDIV(c->omegab, c->omegam);
  c->rho_0 = FMUL(FMUL(2.775e11f, c->omegam), FMUL(c->h, c->h));
  c->rhocrit_0 = FMUL(2.775e11f, FMUL(c->h, c->h));
  c->mypi = FMUL(4.0f, p2m_atanf(1.0f));
  c->drofz = FDIV(6.0f, (float)(P2M_NZTAB - 1));
  c->dzofr = FDIV(1.3e4f, (float)(P2M_NZTAB - 1));
  rofz[0] = 0.0f;
  for (int i = 2; i <= P2M_NZTAB; i++) {
    float z = FADD(FMUL((float)(i - 1), c->drofz), 0.0f);
    float drdz = FDIV(1.0f, p2m_dzdr(c, z));
    rofz[i - 1] = FADD(rofz[i - 2], FMUL(drdz, c->drofz));
  }
  zofr[0] = 0.0f;
  for (int i = 2; i <= P2M_NZTAB; i++) {
    float z = zofr[i - 2];
    zofr[i - 1] = FADD(zofr[i - 2], FMUL(p2m_dzdr(c, z), c->dzofr));
  }
}

/* cosmology.f90:137-181 (table minimum is 0 for both tables) */
P2M_HD float p2m_lookup(const float *tab, float dt, float x) {
  int itab = (int)FADD(FDIV(FSUB(x, 0.0f), dt), 1.0f);
  if (itab < 1) return tab[0];
  if (itab >= P2M_NZTAB) return tab[P2M_NZTAB - 1];
  float fint = FDIV(FSUB(FSUB(x, FMUL((float)(itab - 1), dt)), 0.0f), dt);
  return FADD(FMUL(FSUB(1.0f, fint), tab[itab - 1]), FMUL(fint, tab[itab]));
}

/* cosmology.f90:185-195 */
P2M_HD float p2m_rhocrit(const p2m_cosmo *c, float z) {
  float zp1 = FADD(1.0f, z);
  float c3 = FMUL(FMUL(zp1, zp1), zp1);
  return FDIV(FMUL(c->rhocrit_0, FADD(FMUL(c->omegam, c3), c->omegal)), c3);
}

/* cosmology.f90:199-214 (mixed double/float expression) */
P2M_HD float p2m_deltacrit(const p2m_cosmo *c, float z) {
  float zp1 = FADD(1.0f, z);
  float c3 = FMUL(FMUL(zp1, zp1), zp1);
  float omz = FDIV(FMUL(c->omegam, c3), FSUB(FADD(FMUL(c->omegam, c3), 1.0f), c->omegam));
  float x = FSUB(omz, 1.0f);
  double d = DSUB(DADD(DMUL(18.0, DMUL(P2M_COSMO_PI, P2M_COSMO_PI)), (double)FMUL(82.0f, x)),
                  (double)FMUL(39.0f, FMUL(x, x)));
  return (float)d;
}

/* ------------------------------------------------------------ profile table ------- */

/* Header of a make_maptable table (maptable.f90:158) plus derived log steps (:166-168).
   All tables of one painter share one header. */
typedef struct p2m_tabhdr {
  int nchit, nmht, nrt;
  float chimint, chimaxt, mhmint, mhmaxt, rmint, rmaxt;
  float dchit, dmht, drt;
  float lrmin, lcmin, lmmin; /* log(rmint), log(chimint), log(mhmint) */
  long long nelem;           /* 2*nrt*nmht*nchit */
} p2m_tabhdr;

static inline void p2m_tabhdr_derive(p2m_tabhdr *t) {
  t->dchit = FDIV(FSUB(p2m_logf(t->chimaxt), p2m_logf(t->chimint)), (float)(t->nchit - 1));
  t->drt = FDIV(FSUB(p2m_logf(t->rmaxt), p2m_logf(t->rmint)), (float)(t->nrt - 1));
  t->dmht = FDIV(FSUB(p2m_logf(t->mhmaxt), p2m_logf(t->mhmint)), (float)(t->nmht - 1));
  t->lrmin = p2m_logf(t->rmint);
  t->lcmin = p2m_logf(t->chimint);
  t->lmmin = p2m_logf(t->mhmint);
  t->nelem = 2LL * t->nrt * t->nmht * t->nchit;
}

/* Per-halo part of interpolate_table (maptable.f90:184-202): chi = rofz(z), the
   chi / mh clamps and the chi / mh indices and fractions. */
typedef struct p2m_hinterp {
  float chi_t;   /* rofz(z) before the chimint clamp */
  float fc, fm;  /* chi and mass fractions (unnormalised, as in the reference) */
  int ichi, imh; /* 1-based */
  int zero;      /* chi > chimaxt: the table returns 0 for every pixel */
} p2m_hinterp;

P2M_HD p2m_hinterp p2m_hinterp_make(const p2m_tabhdr *t, float chi_t, float mh) {
  p2m_hinterp hi;
  hi.chi_t = chi_t;
  hi.zero = chi_t > t->chimaxt;
  float chi = chi_t;
  if (chi < t->chimint) chi = FADD(t->chimint, 1e-5f);
  if (mh < t->mhmint) mh = FADD(t->mhmint, 1e-5f);
  if (mh > t->mhmaxt) mh = FSUB(t->mhmaxt, 1e-5f);
  float lc = p2m_logf(chi), lm = p2m_logf(mh);
  hi.ichi = (int)FDIV(FSUB(lc, t->lcmin), t->dchit) + 1;
  hi.imh = (int)FDIV(FSUB(lm, t->lmmin), t->dmht) + 1;
  hi.fc = FSUB(lc, FADD(t->lcmin, FMUL((float)(hi.ichi - 1), t->dchit)));
  hi.fm = FSUB(lm, FADD(t->lmmin, FMUL((float)(hi.imh - 1), t->dmht)));
  return hi;
}

/* flat column-major offset of table(profile, ir, imh, ichi); an index one past a
   dimension continues into the next slice as the unguarded Fortran read does
   (maptable.f90:204-212); offsets past the array are clamped. */
P2M_HD long long p2m_tab_off(const p2m_tabhdr *t, int profile, int ir, int imh, int ichi) {
  long long off = (long long)(profile - 1) +
                  2LL * ((long long)(ir - 1) +
                         (long long)t->nrt * ((long long)(imh - 1) + (long long)t->nmht * (ichi - 1)));
  if (off < 0) off = 0;
  if (off >= t->nelem) off = t->nelem - 1;
  return off;
}

/* the eight-corner blend of maptable.f90:204-212 for a known (ir, fr) */
P2M_HD float p2m_blend8(const float *tab, const p2m_tabhdr *t, const p2m_hinterp *hi,
                        int profile, int ir, float fr) {
  float fc = hi->fc, fm = hi->fm;
  int ichi = hi->ichi, imh = hi->imh;
  float ofr = FSUB(1.0f, fr), ofc = FSUB(1.0f, fc), ofm = FSUB(1.0f, fm);
  float v = 0.0f;
  v = FADD(v, FMUL(FMUL(FMUL(tab[p2m_tab_off(t, profile, ir, imh, ichi)], ofr), ofc), ofm));
  v = FADD(v, FMUL(FMUL(FMUL(tab[p2m_tab_off(t, profile, ir + 1, imh, ichi)], fr), ofc), ofm));
  v = FADD(v, FMUL(FMUL(FMUL(tab[p2m_tab_off(t, profile, ir, imh + 1, ichi)], ofr), fc), ofm));
  v = FADD(v, FMUL(FMUL(FMUL(tab[p2m_tab_off(t, profile, ir + 1, imh + 1, ichi)], fr), fc), ofm));
  v = FADD(v, FMUL(FMUL(FMUL(tab[p2m_tab_off(t, profile, ir, imh, ichi + 1)], ofr), ofc), fm));
  v = FADD(v, FMUL(FMUL(FMUL(tab[p2m_tab_off(t, profile, ir + 1, imh, ichi + 1)], fr), ofc), fm));
  v = FADD(v, FMUL(FMUL(FMUL(tab[p2m_tab_off(t, profile, ir, imh + 1, ichi + 1)], ofr), fc), fm));
  v = FADD(v, FMUL(FMUL(FMUL(tab[p2m_tab_off(t, profile, ir + 1, imh + 1, ichi + 1)], fr), fc), fm));
  return v;
}

/* r-direction index and fraction of maptable.f90:190,196,200 for a radius r that
   passed the rmaxt test */
P2M_HD void p2m_rindex(const p2m_tabhdr *t, float r, int *ir, float *fr) {
  if (r < t->rmint) r = FADD(t->rmint, 1e-5f);
  float lr = p2m_logf(r);
  *ir = (int)FDIV(FSUB(lr, t->lrmin), t->drt) + 1;
  *fr = FSUB(lr, FADD(t->lrmin, FMUL((float)(*ir - 1), t->drt)));
}

/* interpolate_table(theta, z, mh, profile) with the per-halo part precomputed */
P2M_HD float p2m_interp_exact(const float *tab, const p2m_tabhdr *t, const p2m_hinterp *hi,
                              float theta, int profile) {
  float r = FMUL(hi->chi_t, p2m_tanf(theta));
  if (r > t->rmaxt || hi->zero) return 0.0f;
  int ir;
  float fr;
  p2m_rindex(t, r, &ir, &fr);
  return p2m_blend8(tab, t, hi, profile, ir, fr);
}

/* ----------------------------------------------------------------- HEALPix -------- */

/* pix_tools.F90:802-836: pixels in ring, shift, and pixels north of and including it */
P2M_HD void p2m_ring_info(int nside, int ring, int *npr, int *kshift, long long *npnorth) {
  int m = nside;
  if (ring < m) m = ring;
  if (4 * nside - ring < m) m = 4 * nside - ring;
  *npr = 4 * m;
  int ks = (ring + 1) % 2;
  if (nside == 1) ks = 1 - ks;
  if (*npr < 4 * nside) ks = 1;
  *kshift = ks;
  long long n = nside;
  if (ring <= nside) {
    *npnorth = (long long)ring * (ring + 1) * 2;
  } else if (ring <= 3 * nside) {
    *npnorth = n * (n + 1) * 2 + 4 * n * (ring - nside);
  } else {
    long long ir = 4 * n - ring - 1;
    *npnorth = 12 * n * n - ir * (ir + 1) * 2;
  }
}

/* pixel_routines.F90:203-322: centre of RING pixel ipix (double precision) */
P2M_HD void p2m_pix2vec_ring(int nside, long long ipix, double v[3]) {
  long long npix = 12LL * nside * nside;
  int nl2 = 2 * nside;
  long long ncap = (long long)nl2 * (nside - 1);
  double z, sth, phi;
  if (ipix < ncap) {
    int iring = ((int)floor(DSQRT((double)(2 * ipix + 2))) + 1) / 2;
    long long iphi = ipix - 2LL * iring * (iring - 1);
    double fact2 = DMUL(DMUL(3.0, (double)nside), (double)nside);
    z = DSUB(1.0, DMUL(DDIV((double)iring, fact2), (double)iring));
    sth = DMUL((double)iring, DSQRT(DDIV(DADD(1.0, z), fact2)));
    phi = DDIV(DMUL(DADD((double)iphi, 0.5), P2M_HP_HALFPI), (double)iring);
  } else if (ipix < npix - ncap) {
    int nl4 = 4 * nside;
    long long ip = ipix - ncap;
    int iring = (int)(ip / nl4) + nside;
    long long iphi = ip & (nl4 - 1);
    double fact1 = DMUL(1.5, (double)nside);
    double fodd = DMUL(0.5, (double)((iring + nside + 1) & 1));
    z = DDIV((double)(nl2 - iring), fact1);
    sth = DSQRT(DMUL(DSUB(1.0, z), DADD(1.0, z)));
    phi = DDIV(DMUL(DADD((double)iphi, fodd), P2M_HP_HALFPI), (double)nside);
  } else {
    long long ip = npix - ipix;
    int iring = ((int)floor(DSQRT((double)(2 * ip))) + 1) / 2;
    long long iphi = 2LL * iring * (iring + 1) - ip;
    double fact2 = DMUL(DMUL(3.0, (double)nside), (double)nside);
    z = DADD(-1.0, DMUL(DDIV((double)iring, fact2), (double)iring));
    sth = DMUL((double)iring, DSQRT(DDIV(DSUB(1.0, z), fact2)));
    phi = DDIV(DMUL(DADD((double)iphi, 0.5), P2M_HP_HALFPI), (double)iring);
  }
  v[0] = DMUL(sth, cos(phi));
  v[1] = DMUL(sth, sin(phi));
  v[2] = z;
}

/* pix_tools.F90:2015-2055 */
P2M_HD double p2m_angdist(const double v1[3], const double v2[3]) {
  double sprod = DADD(DADD(DMUL(v1[0], v2[0]), DMUL(v1[1], v2[1])), DMUL(v1[2], v2[2]));
  double v3x = DSUB(DMUL(v1[1], v2[2]), DMUL(v1[2], v2[1]));
  double v3y = DSUB(DMUL(v1[2], v2[0]), DMUL(v1[0], v2[2]));
  double v3z = DSUB(DMUL(v1[0], v2[1]), DMUL(v1[1], v2[0]));
  double vprod = DSQRT(DADD(DADD(DMUL(v3x, v3x), DMUL(v3y, v3y)), DMUL(v3z, v3z)));
  return atan2(vprod, sprod);
}

/* z of ring ir as pix2vec_ring computes it (pixel_routines.F90:236,276,315) and the
   matching sin(theta); used for the per-ring constants of the disc test */
P2M_HD void p2m_ring_z_sth(int nside, int ir, double *z, double *sth) {
  if (ir < nside) {
    double fact2 = DMUL(DMUL(3.0, (double)nside), (double)nside);
    *z = DSUB(1.0, DMUL(DDIV((double)ir, fact2), (double)ir));
    *sth = DMUL((double)ir, DSQRT(DDIV(DADD(1.0, *z), fact2)));
  } else if (ir <= 3 * nside) {
    *z = DDIV((double)(2 * nside - ir), DMUL(1.5, (double)nside));
    *sth = DSQRT(DMUL(DSUB(1.0, *z), DADD(1.0, *z)));
  } else {
    int is = 4 * nside - ir;
    double fact2 = DMUL(DMUL(3.0, (double)nside), (double)nside);
    *z = DADD(-1.0, DMUL(DDIV((double)is, fact2), (double)is));
    *sth = DMUL((double)is, DSQRT(DDIV(DSUB(1.0, *z), fact2)));
  }
}

/* continuous ring coordinate of colatitude theta (rings sit at integers):
   north cap i = N sqrt(6) sin(theta/2), belt i = N (2 - 1.5 cos theta),
   south cap i = 4N - N sqrt(6) cos(theta/2) (inverse of ring2z, pix_tools.F90:535-560) */
P2M_HD float p2m_ring_coord(int nside, float theta) {
  const float cos_tc = 0.6666666667f; /* cap boundary z = 2/3 */
  float fn = (float)nside;
  float z = cosf(theta);
  if (z > cos_tc) return fn * 2.449489743f * sinf(0.5f * theta);
  if (z < -cos_tc) return 4.0f * fn - fn * 2.449489743f * cosf(0.5f * theta);
  return fn * (2.0f - 1.5f * z);
}

/* ------------------------------------------------- scramble and centre -------------- */

/* Pre-processing of pks2map.f90:162-262 (off unless set): scramble gives every halo that
   survives the radial cut a random direction; centre flips and rotates all positions so
   that the largest-RTH halo lands on the z axis.  Positions are posxyz(1..3), the first
   three floats of a record. */
typedef struct p2m_pre {
  int32_t scramble, centre;
  int32_t ntasks;        /* MPI ranks emulated: each scrambles its block (pksc.f90:51-52) */
  int32_t flip[3];       /* negate posxyz(1), posxyz(2), posxyz(3) */
  long long per_rank;    /* records per rank block */
  float ct, st, cp, sp;  /* cos, sin of rmaxtheta and rmaxphi */
} p2m_pre;

#define P2M_RANF_MASK ((1ULL << 48) - 1ULL)
/* random.f90:28-29 multiplier (373, 3707, 1442, 647) as one 48-bit number */
#define P2M_RANF_MULT (373ULL + (3707ULL << 12) + (1442ULL << 24) + (647ULL << 36))

/* low 48 bits of a * b: exact under 64-bit wrap-around */
P2M_HD unsigned long long p2m_ranf_mul(unsigned long long a, unsigned long long b) {
  return (a * b) & P2M_RANF_MASK;
}

/* Output n of the ranf stream whose seed has every digit d (pks2map.f90:164 broadcasts
   13579*(rank+1) to the four digits).  ranf (random.f90:40-57) returns the value of the
   current seed, then multiplies it by the multiplier modulo 2^48 (random.f90:264-286).
   Output 0 reads the unreduced digits; output n >= 1 is state_n / 2^48 with
   state_n = mult^n * seed (mod 2^48), found by jump-ahead. */
P2M_HD double p2m_ranf_nth(long long d, long long n) {
  if (n == 0) {
    const double fd = (double)(float)d;
    return DADD(DADD(DADD(DDIV(fd, 4096.0), DDIV(fd, 16777216.0)), DDIV(fd, 68719476736.0)),
                DDIV(fd, 281474976710656.0));
  }
  const unsigned long long ud = (unsigned long long)d;
  unsigned long long s = (ud + (ud << 12) + (ud << 24) + (ud << 36)) & P2M_RANF_MASK;
  unsigned long long a = P2M_RANF_MULT, e = (unsigned long long)n;
  while (e) { /* s = mult^n * s */
    if (e & 1ULL) s = p2m_ranf_mul(s, a);
    a = p2m_ranf_mul(a, a);
    e >>= 1;
  }
  const double s4 = (double)(s >> 36), s3 = (double)((s >> 24) & 4095ULL),
               s2 = (double)((s >> 12) & 4095ULL), s1 = (double)(s & 4095ULL);
  return DADD(DADD(DADD(DDIV(s4, 4096.0), DDIV(s3, 16777216.0)), DDIV(s2, 68719476736.0)),
              DDIV(s1, 281474976710656.0));
}

/* pks2map.f90:166-184 for the k-th surviving halo of its rank (k from 0), seed digits d */
P2M_HD void p2m_scramble_pos(long long d, long long k, float pos[3]) {
  const float xh = pos[0], yh = pos[1], zh = pos[2];
  const float chih = FSQRT(FADD(FADD(FMUL(xh, xh), FMUL(yh, yh)), FMUL(zh, zh)));
  const float muran = (float)DSUB(DMUL(2.0, p2m_ranf_nth(d, 2 * k)), 1.0);
  const float phiran = (float)DMUL((double)FMUL(2.0f, 3.14159f), p2m_ranf_nth(d, 2 * k + 1));
  const float rh = FMUL(FSQRT(FSUB(1.0f, FMUL(muran, muran))), chih);
  pos[0] = FMUL(rh, p2m_cosf(phiran));
  pos[1] = FMUL(rh, p2m_sinf(phiran));
  pos[2] = FMUL(muran, chih);
}

/* pks2map.f90:216-241: the flips, then the rotations by rmaxtheta and rmaxphi */
P2M_HD void p2m_rotate_pos(const p2m_pre *q, float pos[3]) {
  const float p1 = q->flip[0] ? -pos[0] : pos[0];
  const float p2 = q->flip[1] ? -pos[1] : pos[1];
  const float p3 = q->flip[2] ? -pos[2] : pos[2];
  float xh = FADD(FMUL(p3, q->ct), FMUL(p1, q->st));
  const float zh = FADD(FMUL(-p3, q->st), FMUL(p1, q->ct));
  const float yh = FADD(FMUL(-xh, q->sp), FMUL(p2, q->cp));
  xh = FADD(FMUL(xh, q->cp), FMUL(p2, q->sp));
  pos[2] = zh;
  pos[1] = yh;
  pos[0] = xh;
}

#endif /* P2M_SCALAR_H */
