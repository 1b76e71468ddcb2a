/*
 * p2m_oracle.c -- TEST INFRASTRUCTURE ONLY (see p2m_oracle.h).
 *
 * Plain-C restatement of the reference's pks2map path.  PARITY UNPINNED: the
 * reference has no golden vectors and cannot be built here.  Each function cites the
 * reference file:line it restates (paths relative to the reference project root).
 * Compile with -ffp-contract=off; evaluation follows the source order of the Fortran.
 */
#include "p2m_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../matt_young_mapmaking_gb300/csrc/p2m_fmath.h"

/* healpix_types.F90:65-73 */
static const double HP_HALFPI = 1.570796326794896619231321691639751442099;
static const double HP_PI = 3.141592653589793238462643383279502884197;
static const double HP_TWOPI = 6.283185307179586476925286766559005768394;
static const double HP_TWOTHIRD = 0.6666666666666666666666666666666666666666;

/* cosmology.f90:8-9: `parameter (pi = 3.14159265359)` is a default-real literal,
   so the double parameter holds its single-precision value. */
static const double COSMO_PI = 3.1415927410125732421875;
/* cosmology.f90:11-23 (c, Mpc2km as double literals; 1e2 and 1e5 are exact reals) */
static const double COSMO_C = 2.99792458e10;
static const double COSMO_CKMS = 2.99792458e10 / 1e5;

/* bbps_profile.f90:21 */
static const float BBPS_DELTA[3] = {200.0f, 500.0f, 200.0f};
/* pksc.f90:9, pks2map.f90:84, haloproject.f90:18 */
static const float DELTA_PKSC = 200.0f;
static const float MMIN = 1e13f;
static const float RMAX_DISC = 4.0f;

/* ---------------------------------------------------------------- cosmology -------- */

/* cosmology.f90:123-133: dzdr = h*100/ckms*sqrt(omegam*(1.+z)**3+1.-omegam) */
static float dzdr(const orc_cosmo *c, float z) {
  float zp1 = 1.0f + z;
  float c3 = (zp1 * zp1) * zp1;
  float s = sqrtf(((c->omegam * c3) + 1.0f) - c->omegam);
  double t = (double)(c->h * 100.0f) / COSMO_CKMS;
  return (float)(t * (double)s);
}
/* cosmology.f90:109-119 */
static float drdz(const orc_cosmo *c, float z) { return 1.0f / dzdr(c, z); }

/* pks2map.f90:88,118-132; cosmology.f90:51-105 */
void orc_cosmo_init(orc_cosmo *c) {
  c->omegam = 0.25f;
  c->omegab = 0.043f;
  c->omegal = 0.75f;
  c->h = 0.7f;
  c->fb = c->omegab / c->omegam;
  c->rho_0 = (2.775e11f * c->omegam) * (c->h * c->h);
  c->rhocrit_0 = 2.775e11f * (c->h * c->h);
  c->mypi = 4.0f * p2m_atanf(1.0f);
  /* set_rofztable */
  c->rofztable_min = 0.0f;
  c->drofztable = (6.0f - c->rofztable_min) / (float)(ORC_NZTAB - 1);
  c->rofztable[0] = 0.0f;
  for (int i = 2; i <= ORC_NZTAB; i++) {
    float z = ((float)(i - 1) * c->drofztable) + c->rofztable_min;
    c->rofztable[i - 1] = c->rofztable[i - 2] + (drdz(c, z) * c->drofztable);
  }
  /* set_zofrtable */
  c->zofrtable_min = 0.0f;
  c->dzofrtable = (1.3e4f - c->zofrtable_min) / (float)(ORC_NZTAB - 1);
  c->zofrtable[0] = 0.0f;
  for (int i = 2; i <= ORC_NZTAB; i++) {
    float z = c->zofrtable[i - 2];
    c->zofrtable[i - 1] = c->zofrtable[i - 2] + (dzdr(c, z) * c->dzofrtable);
  }
}

/* cosmology.f90:137-157 (and rofz, :161-181): linear lookup, truncated index */
static float table_lookup(const float *tab, float tmin, float dt, float x) {
  int itab = (int)(((x - tmin) / dt) + 1.0f);
  if (itab < 1) return tab[0];
  if (itab >= ORC_NZTAB) return tab[ORC_NZTAB - 1];
  float fint = ((x - ((float)(itab - 1) * dt)) - tmin) / dt;
  return ((1.0f - fint) * tab[itab - 1]) + (fint * tab[itab]);
}
float orc_zofr(const orc_cosmo *c, float r) {
  return table_lookup(c->zofrtable, c->zofrtable_min, c->dzofrtable, r);
}
float orc_rofz(const orc_cosmo *c, float z) {
  return table_lookup(c->rofztable, c->rofztable_min, c->drofztable, z);
}
/* cosmology.f90:185-195 */
float orc_rhocrit(const orc_cosmo *c, float z) {
  float zp1 = 1.0f + z;
  float c3 = (zp1 * zp1) * zp1;
  return (c->rhocrit_0 * ((c->omegam * c3) + c->omegal)) / c3;
}
/* cosmology.f90:199-214: 18*pi**2 is double (pi double), 82*x and 39*x**2 are real */
float orc_deltacrit(const orc_cosmo *c, float z) {
  float zp1 = 1.0f + z;
  float c3 = (zp1 * zp1) * zp1;
  float omegaz = (c->omegam * c3) / (((c->omegam * c3) + 1.0f) - c->omegam);
  float x = omegaz - 1.0f;
  double d = (18.0 * (COSMO_PI * COSMO_PI) + (double)(82.0f * x)) - (double)(39.0f * (x * x));
  return (float)d;
}

/* ------------------------------------------------------------------- table -------- */

/* maptable.f90:150-172 */
int orc_table_from_image(orc_table *t, const void *image, int64_t nbytes) {
  if (nbytes < 36) return -1;
  const char *b = (const char *)image;
  memcpy(&t->nchit, b + 0, 4);
  memcpy(&t->nmht, b + 4, 4);
  memcpy(&t->nrt, b + 8, 4);
  memcpy(&t->chimint, b + 12, 4);
  memcpy(&t->chimaxt, b + 16, 4);
  memcpy(&t->mhmint, b + 20, 4);
  memcpy(&t->mhmaxt, b + 24, 4);
  memcpy(&t->rmint, b + 28, 4);
  memcpy(&t->rmaxt, b + 32, 4);
  if (t->nchit < 2 || t->nmht < 2 || t->nrt < 2) return -2;
  int64_t need = 36 + 8 * (int64_t)t->nchit * t->nmht * t->nrt;
  if (nbytes < need) return -3;
  t->data = (const float *)(b + 36);
  t->dchit = (p2m_logf(t->chimaxt) - p2m_logf(t->chimint)) / (float)(t->nchit - 1);
  t->drt = (p2m_logf(t->rmaxt) - p2m_logf(t->rmint)) / (float)(t->nrt - 1);
  t->dmht = (p2m_logf(t->mhmaxt) - p2m_logf(t->mhmint)) / (float)(t->nmht - 1);
  return 0;
}

/* Fortran table(profile, ir, imh, ichi) read through its flat column-major offset.
   maptable.f90:204-212 has no upper-index guard: an index one past a dimension reads
   the next slice's first element; only a read past the whole array is clamped. */
static float tab_at(const orc_table *t, int profile, int ir, int imh, int ichi) {
  int64_t off = (int64_t)(profile - 1) +
                2 * ((int64_t)(ir - 1) + (int64_t)t->nrt * ((int64_t)(imh - 1) +
                                                              (int64_t)t->nmht * (ichi - 1)));
  int64_t n = 2 * (int64_t)t->nrt * t->nmht * t->nchit;
  if (off < 0) off = 0;
  if (off >= n) off = n - 1;
  return t->data[off];
}

/* maptable.f90:176-216, including the weight pairing of :204-212 (fc weights the
   imh+1 corner, fm the ichi+1 corner) and the in-place clamp of mh (:192-194) */
float orc_interpolate_table(const orc_cosmo *c, const orc_table *t, float theta, float z,
                            float *mh, int profile) {
  float chi = orc_rofz(c, z);
  float r = chi * p2m_tanf(theta);
  if (r > t->rmaxt || chi > t->chimaxt) return 0.0f;
  if (r < t->rmint) r = t->rmint + 1e-5f;
  if (chi < t->chimint) chi = t->chimint + 1e-5f;
  if (*mh < t->mhmint) *mh = t->mhmint + 1e-5f;
  if (*mh > t->mhmaxt) *mh = t->mhmaxt - 1e-5f;
  float lr = p2m_logf(r), lrmin = p2m_logf(t->rmint);
  float lc = p2m_logf(chi), lcmin = p2m_logf(t->chimint);
  float lm = p2m_logf(*mh), lmmin = p2m_logf(t->mhmint);
  int ir = (int)((lr - lrmin) / t->drt) + 1;
  int ichi = (int)((lc - lcmin) / t->dchit) + 1;
  int imh = (int)((lm - lmmin) / t->dmht) + 1;
  float fr = lr - (lrmin + ((float)(ir - 1) * t->drt));
  float fc = lc - (lcmin + ((float)(ichi - 1) * t->dchit));
  float fm = lm - (lmmin + ((float)(imh - 1) * t->dmht));
  float v = 0.0f;
  v = v + ((tab_at(t, profile, ir, imh, ichi) * (1.0f - fr)) * (1.0f - fc)) * (1.0f - fm);
  v = v + ((tab_at(t, profile, ir + 1, imh, ichi) * fr) * (1.0f - fc)) * (1.0f - fm);
  v = v + ((tab_at(t, profile, ir, imh + 1, ichi) * (1.0f - fr)) * fc) * (1.0f - fm);
  v = v + ((tab_at(t, profile, ir + 1, imh + 1, ichi) * fr) * fc) * (1.0f - fm);
  v = v + ((tab_at(t, profile, ir, imh, ichi + 1) * (1.0f - fr)) * (1.0f - fc)) * fm;
  v = v + ((tab_at(t, profile, ir + 1, imh, ichi + 1) * fr) * (1.0f - fc)) * fm;
  v = v + ((tab_at(t, profile, ir, imh + 1, ichi + 1) * (1.0f - fr)) * fc) * fm;
  v = v + ((tab_at(t, profile, ir + 1, imh + 1, ichi + 1) * fr) * fc) * fm;
  return v;
}

/* ----------------------------------------------------------------- HEALPix -------- */

static int fortran_nint(double x) { return (int)lround(x); } /* half away from zero */
static int fortran_modulo(int a, int n) {
  int m = a % n;
  return m < 0 ? m + n : m;
}

/* pix_tools.F90:490-533 */
int orc_ring_num(int nside, double z) {
  int iring = fortran_nint((double)nside * (2.0 - 1.5 * z));
  if (z > HP_TWOTHIRD) {
    iring = fortran_nint((double)nside * sqrt(3.0 * (1.0 - z)));
    if (iring == 0) iring = 1;
  }
  if (z < -HP_TWOTHIRD) {
    iring = fortran_nint((double)nside * sqrt(3.0 * (1.0 + z)));
    if (iring == 0) iring = 1;
    iring = 4 * nside - iring;
  }
  return iring;
}

/* pix_tools.F90:535-560 */
double orc_ring2z(int nside, int ir) {
  double fn = (double)nside;
  if (ir < nside) {
    double tmp = (double)ir;
    return 1.0 - (tmp * tmp) / ((3.0 * fn) * fn);
  } else if (ir < 3 * nside) {
    return ((double)(2 * nside - ir) * 2.0) / (3.0 * fn);
  } else {
    double tmp = (double)(4 * nside - ir);
    return -1.0 + (tmp * tmp) / ((3.0 * fn) * fn);
  }
}

/* pix_tools.F90:802-836 */
void orc_pixels_per_ring(int nside, int ring, int *npr, int *kshift, int64_t *npnorth) {
  int m = nside;
  if (ring < m) m = ring;
  if (4 * nside - ring < m) m = 4 * nside - ring;
  *npr = 4 * m;
  int ks = (ring + 1) % 2;
  if (nside == 1) ks = 1 - ks;
  if (*npr < 4 * nside) ks = 1;
  *kshift = ks;
  if (npnorth) {
    int64_t n = nside;
    if (ring <= nside) {
      *npnorth = (int64_t)ring * (ring + 1) * 2;
    } else if (ring <= 3 * nside) {
      int64_t ncap = n * (n + 1) * 2;
      *npnorth = ncap + 4 * n * (ring - nside);
    } else {
      int64_t npix = 12 * n * n;
      int64_t ir = 4 * n - ring - 1;
      *npnorth = npix - ir * (ir + 1) * 2;
    }
  }
}

/* pixel_routines.F90:203-322 (pixel centre only) */
void orc_pix2vec_ring(int nside, int64_t ipix, double v[3]) {
  int64_t npix = 12 * (int64_t)nside * nside;
  int nl2 = 2 * nside;
  int64_t ncap = (int64_t)nl2 * (nside - 1);
  double z, sth, phi;
  const double half = 0.5;
  if (ipix < ncap) {
    int iring = ((int)floor(sqrt((double)(2 * ipix + 2))) + 1) / 2; /* cheap_isqrt */
    int64_t iphi = ipix - 2 * (int64_t)iring * (iring - 1);
    double fact2 = (3.0 * nside) * nside;
    z = 1.0 - ((double)iring / fact2) * (double)iring;
    sth = (double)iring * sqrt((1.0 + z) / fact2);
    phi = (((double)iphi + half) * HP_HALFPI) / (double)iring;
  } else if (ipix < npix - ncap) {
    int nl4 = 4 * nside;
    int64_t ip = ipix - ncap;
    int iring = (int)(ip / nl4) + nside;
    int64_t iphi = ip & (nl4 - 1);
    double fact1 = 1.5 * nside;
    double fodd = half * (double)((iring + nside + 1) & 1);
    z = (double)(nl2 - iring) / fact1;
    sth = sqrt((1.0 - z) * (1.0 + z));
    phi = (((double)iphi + fodd) * HP_HALFPI) / (double)nside;
  } else {
    int64_t ip = npix - ipix;
    int iring = ((int)floor(sqrt((double)(2 * ip))) + 1) / 2;
    int64_t iphi = 2 * (int64_t)iring * (iring + 1) - ip;
    double fact2 = (3.0 * nside) * nside;
    z = -1.0 + ((double)iring / fact2) * (double)iring;
    sth = (double)iring * sqrt((1.0 - z) / fact2);
    phi = (((double)iphi + half) * HP_HALFPI) / (double)iring;
  }
  v[0] = sth * cos(phi);
  v[1] = sth * sin(phi);
  v[2] = z;
}

/* pix_tools.F90:2015-2055 */
double orc_angdist(const double v1[3], const double v2[3]) {
  double sprod = (v1[0] * v2[0] + v1[1] * v2[1]) + v1[2] * v2[2];
  double v3x = v1[1] * v2[2] - v1[2] * v2[1];
  double v3y = v1[2] * v2[0] - v1[0] * v2[2];
  double v3z = v1[0] * v2[1] - v1[1] * v2[0];
  double vprod = sqrt((v3x * v3x + v3y * v3y) + v3z * v3z);
  return atan2(vprod, sprod);
}

/* pix_tools.F90:712-760 */
static void discphirange_at_z(const double v0[3], double radius, const double *z, int nz,
                              double *dphi, double *phi0) {
  double cosang = cos(radius);
  double norm = sqrt((v0[0] * v0[0] + v0[1] * v0[1]) + v0[2] * v0[2]);
  double x0 = v0[0] / norm, y0 = v0[1] / norm, z0 = v0[2] / norm;
  *phi0 = 0.0;
  if (x0 != 0.0 || y0 != 0.0) *phi0 = atan2(y0, x0);
  double a = x0 * x0 + y0 * y0;
  for (int i = 0; i < nz; i++) {
    dphi[i] = -1000.0;
    double b = cosang - z[i] * z0;
    if (a == 0.0) {
      if (b <= 0.0) dphi[i] = HP_PI;
    } else {
      double c = 1.0 - z[i] * z[i];
      if (c < 1.0e-12) c = 1.0e-12;
      double cosdphi = b / sqrt(a * c);
      if (cosdphi < -1.0) dphi[i] = HP_PI;
      if (fabs(cosdphi) <= 1.0) dphi[i] = acos(cosdphi);
    }
  }
}

/* pixel_routines.F90:1927-2046 (inclusive = 0, nest = 0), with pix_tools.F90:762-800
   (pixels_on_edge) and pixel_routines.F90:1826-1879 (discedge2fulldisc).
   discedge2fulldisc walks rings jr_min..jr_max and reads ringphi(:, j+1) for ring
   jr_min+j, while pixels_on_edge stores only non-empty rings; when a ring inside the
   range holds no pixel centre (a "ring gap") the reference reads misaligned and
   uninitialised span data.  This restatement emits every non-empty ring with its own
   span -- the list the reference returns whenever no gap occurs -- and reports gaps. */
int64_t orc_query_disc(int nside, const double v0[3], double radius, int64_t *list,
                       int64_t cap, int *gaps) {
  if (gaps) *gaps = 0;
  if (radius < 0.0 || radius > HP_PI) return -2; /* the reference aborts */
  double norm = sqrt((v0[0] * v0[0] + v0[1] * v0[1]) + v0[2] * v0[2]);
  double z0 = v0[2] / norm;
  double rlat0 = asin(z0);
  double rlat1 = rlat0 + radius;
  double rlat2 = rlat0 - radius;
  double zmax = (rlat1 >= HP_HALFPI) ? 1.0 : sin(rlat1);
  int irmin = orc_ring_num(nside, zmax) - 1;
  if (irmin < 1) irmin = 1;
  double zmin = (rlat2 <= -HP_HALFPI) ? -1.0 : sin(rlat2);
  int irmax = orc_ring_num(nside, zmin) + 1;
  if (irmax > 4 * nside - 1) irmax = 4 * nside - 1;
  int nr = irmax - irmin + 1;
  double *ztab = (double *)malloc(sizeof(double) * (size_t)nr * 2);
  double *dphitab = ztab + nr;
  for (int iz = irmin; iz <= irmax; iz++) ztab[iz - irmin] = orc_ring2z(nside, iz);
  double phi0;
  discphirange_at_z(v0, radius, ztab, nr, dphitab, &phi0);
  int64_t nlist = 0;
  int first = -1, last = -1, nonempty = 0;
  for (int ring = irmin; ring <= irmax; ring++) {
    int npr, kshift;
    int64_t npc;
    orc_pixels_per_ring(nside, ring, &npr, &kshift, &npc);
    double dphi = dphitab[ring - irmin];
    int lo, hi;
    if (dphi >= HP_PI) {
      lo = 0;
      hi = npr - 1;
    } else if (dphi >= 0.0) {
      double shift = (double)kshift * 0.5;
      int ilo = (int)ceil(((double)npr * (phi0 - dphi)) / HP_TWOPI - shift);
      int ihi = (int)floor(((double)npr * (phi0 + dphi)) / HP_TWOPI - shift);
      if (ihi < ilo) continue;
      lo = fortran_modulo(ilo, npr);
      hi = fortran_modulo(ihi, npr);
    } else {
      continue;
    }
    if (first < 0) first = ring;
    last = ring;
    nonempty++;
    int np = fortran_modulo(hi - lo, npr) + 1;
    if (np > npr) np = npr;
    if (nlist + np > cap) {
      free(ztab);
      return -1;
    }
    for (int i = 0; i < np; i++) {
      int ip = fortran_modulo(lo + i, npr);
      list[nlist + i] = npc - npr + ip;
    }
    nlist += np;
  }
  if (gaps && nonempty > 0 && last - first + 1 != nonempty) *gaps = 1;
  free(ztab);
  return nlist;
}

/* ----------------------------------------------------------- the halo loop -------- */

typedef struct halo_state {
  float xh, yh, zh, rh, chih, mh, redshift, vh;
} halo_state;

/* pksc.f90:70-78 with the intended per-halo line-of-sight velocity (the reference's
   array expression uses posxyz(:,1), the first halo's 3-vector, and the radial cut
   at pks2map.f90:144-160 does not compact vrad). */
static float halo_vrad(const float *rec, int profile) {
  if (profile != 2) return 1.0f;
  float dot = ((rec[0] * rec[3]) + (rec[1] * rec[4])) + (rec[2] * rec[5]);
  float nrm = sqrtf(((rec[0] * rec[0]) + (rec[1] * rec[1])) + (rec[2] * rec[2]));
  float v = dot / nrm;
  return -(v / 3.e5f);
}

/* radial cut of pks2map.f90:144-160: 1 if kept.  Records with a non-finite position
   or radius are dropped (the reference's behaviour on them is undefined). */
static int halo_in_shell(const float *rec, float chihview, float cut_low, float cut_high) {
  if (!isfinite(rec[0]) || !isfinite(rec[1]) || !isfinite(rec[2]) || !isfinite(rec[6]))
    return 0;
  float xh = rec[2], yh = rec[1], zh = rec[0];
  xh = xh - chihview;
  float chih = sqrtf(((xh * xh) + (yh * yh)) + (zh * zh));
  return !(chih > cut_high || chih < cut_low);
}

/* pks2map.f90:264 and :284-298 for one kept halo; returns 0 if mass < mmin */
static int halo_prepare(const orc_cosmo *c, const orc_params *p, const float *rec,
                        halo_state *hs) {
  float rth = rec[6];
  float mass = (((4.0f / 3.0f) * c->mypi) * c->rho_0) * ((rth * rth) * rth);
  float xh = rec[2], yh = rec[1], zh = rec[0];
  float chih = sqrtf(((xh * xh) + (yh * yh)) + (zh * zh));
  float redshift = orc_zofr(c, chih);
  xh = xh - p->chihview;
  chih = sqrtf(((xh * xh) + (yh * yh)) + (zh * zh));
  float mh = sqrtf(orc_deltacrit(c, redshift) / BBPS_DELTA[p->model - 1]) * mass;
  if (mass < MMIN) return 0;
  float rh = p2m_powf((((((3.0f * mh) / 4.0f) / c->mypi) / DELTA_PKSC) / orc_rhocrit(c, redshift)),
                      1.0f / 3.0f);
  hs->xh = xh;
  hs->yh = yh;
  hs->zh = zh;
  hs->rh = rh;
  hs->chih = chih;
  hs->mh = mh;
  hs->redshift = redshift;
  return 1;
}

int orc_halo_setup(const orc_cosmo *c, const orc_params *p, const float *rec, float *out8) {
  halo_state hs;
  if (!halo_in_shell(rec, p->chihview, orc_rofz(c, p->zmin), orc_rofz(c, p->zmax))) return 0;
  if (!halo_prepare(c, p, rec, &hs)) return 0;
  out8[0] = hs.xh;
  out8[1] = hs.yh;
  out8[2] = hs.zh;
  out8[3] = hs.rh;
  out8[4] = hs.chih;
  out8[5] = hs.mh;
  out8[6] = hs.redshift;
  out8[7] = (float)((double)(RMAX_DISC * p2m_asinf(hs.rh / hs.chih)));
  return 1;
}

/* A growable log of (key, value) pairs: deposits (key = flat map index, flat-sky
   deposits as -1 - index) or pixel-set entries (key = halo, value slot unused, pix in
   aux).  Used by orc_paint_parallel to replay every thread's deposits in halo order. */
typedef struct dep_log {
  int64_t *key, *aux;
  float *val;
  int64_t n, cap;
  int err;
} dep_log;

static void log_push(dep_log *l, int64_t key, int64_t aux, float val) {
  if (l->err) return;
  if (l->n == l->cap) {
    int64_t cap = l->cap ? 2 * l->cap : (1 << 16);
    int64_t *k = (int64_t *)realloc(l->key, sizeof(int64_t) * (size_t)cap);
    if (k) l->key = k;
    int64_t *a = (int64_t *)realloc(l->aux, sizeof(int64_t) * (size_t)cap);
    if (a) l->aux = a;
    float *v = (float *)realloc(l->val, sizeof(float) * (size_t)cap);
    if (v) l->val = v;
    if (!k || !a || !v) {
      l->err = 1;
      return;
    }
    l->cap = cap;
  }
  l->key[l->n] = key;
  l->aux[l->n] = aux;
  l->val[l->n] = val;
  l->n++;
}

static void log_free(dep_log *l) {
  free(l->key);
  free(l->aux);
  free(l->val);
  memset(l, 0, sizeof(*l));
}

typedef struct paint_out {
  int fp32;
  double *hp64, *fs64;
  float *hp32, *fs32;
  int64_t hp_npix, fs_npix2;
  dep_log *log;  /* non-NULL: deposits are logged instead of added */
  dep_log *sets; /* non-NULL: HEALPix (halo, pixel) pairs are logged here */
} paint_out;

static void deposit(const paint_out *o, int hp, int map, int64_t j, float curval) {
  if (o->log) {
    log_push(o->log, hp ? (int64_t)map * o->hp_npix + j : -1 - ((int64_t)map * o->fs_npix2 + j),
             0, curval);
    return;
  }
  if (hp) {
    int64_t k = (int64_t)map * o->hp_npix + j;
    if (o->fp32) o->hp32[k] = o->hp32[k] + curval;
    else o->hp64[k] = o->hp64[k] + (double)curval;
  } else {
    int64_t k = (int64_t)map * o->fs_npix2 + j;
    if (o->fp32) o->fs32[k] = o->fs32[k] + curval;
    else o->fs64[k] = o->fs64[k] + (double)curval;
  }
}

/* haloproject.f90:83-156 (mutates x, y, z to x/chi, y/chi, z/chi) */
static void projecthalo_flatsky(const orc_cosmo *c, const orc_params *p, const orc_table *tabs,
                                halo_state *hs, const float *vmap, float fov, float dpix,
                                const paint_out *o, orc_stats *st) {
  double dtheta_halo = (double)(RMAX_DISC * p2m_asinf(hs->rh / hs->chih));
  hs->xh = hs->xh / hs->chih;
  hs->yh = hs->yh / hs->chih;
  hs->zh = hs->zh / hs->chih;
  if (p->npix_fs <= 0) return;
  if (hs->zh < 0.0f) return;
  double theta_halo = (double)p2m_asinf(hs->xh);
  double phi_halo = (double)p2m_asinf(hs->yh);
  double w = (double)1.1f * dtheta_halo;
  float thetamin = (float)(theta_halo - w), thetamax = (float)(theta_halo + w);
  float phimin = (float)(phi_halo - w), phimax = (float)(phi_halo + w);
  float hf = fov / 2.0f;
  if (thetamax < -hf || thetamin > hf) return;
  if (phimax < -hf || phimin > hf) return;
  if (thetamin <= -hf) thetamin = -hf + 1e-10f;
  if (thetamax >= hf) thetamax = hf - 1e-10f;
  if (phimin <= -hf) phimin = -hf + 1e-10f;
  if (phimax >= hf) phimax = hf - 1e-10f;
  int npix = p->npix_fs;
  int jmin = (int)((thetamin + hf) / dpix) + 1;
  if (jmin < 1) jmin = 1;
  int jmax = (int)((thetamax + hf) / dpix) + 1;
  if (jmax > npix) jmax = npix;
  int kmin = (int)((phimin + hf) / dpix) + 1;
  if (kmin < 1) kmin = 1;
  int kmax = (int)((phimax + hf) / dpix) + 1;
  if (kmax > npix) kmax = npix;
  for (int k = kmin; k <= kmax; k++) {
    float phip = -hf + (((float)k - 0.5f) * dpix);
    for (int j = jmin; j <= jmax; j++) {
      float thetap = -hf + (((float)j - 0.5f) * dpix);
      float dphi = (float)((double)phip - phi_halo);
      float dtheta = (float)((double)thetap - theta_halo);
      float angle = sqrtf((dphi * dphi) + (dtheta * dtheta));
      if ((double)angle < dtheta_halo) {
        st->fs_updates++;
        for (int m = 0; m < p->nmaps; m++) {
          float curval = vmap[m] * orc_interpolate_table(c, &tabs[p->table_id[m]], angle,
                                                         hs->redshift, &hs->mh, p->profile[m]);
          deposit(o, 0, m, (int64_t)(j - 1) + (int64_t)npix * (k - 1), curval);
        }
      }
    }
  }
}

/* haloproject.f90:38-79 (x, y, z arrive already divided by chi) */
static int projecthalo_healpix(const orc_cosmo *c, const orc_params *p, const orc_table *tabs,
                               halo_state *hs, const float *vmap, int64_t *list,
                               int64_t listcap, const paint_out *o, orc_stats *st,
                               int64_t halo_index, int64_t *set_halo, int64_t *set_pix,
                               int64_t set_cap, int64_t *set_n) {
  double dtheta_halo = (double)(RMAX_DISC * p2m_asinf(hs->rh / hs->chih));
  double v1[3];
  v1[0] = (double)(hs->zh / hs->chih);
  v1[1] = (double)(hs->yh / hs->chih);
  v1[2] = (double)(hs->xh / hs->chih);
  int gaps = 0;
  int64_t nlist = orc_query_disc(p->nside, v1, dtheta_halo, list, listcap, &gaps);
  if (nlist < 0) return (int)nlist;
  st->hp_candidates += nlist;
  st->ring_gaps += gaps;
  for (int64_t i = 0; i < nlist; i++) {
    int64_t j = list[i];
    double v2[3];
    orc_pix2vec_ring(p->nside, j, v2);
    float angle = (float)orc_angdist(v1, v2);
    if ((double)angle < dtheta_halo) {
      st->hp_updates++;
      if (o->sets) log_push(o->sets, halo_index, j, 0.0f);
      if (set_halo && *set_n < set_cap) {
        set_halo[*set_n] = halo_index;
        set_pix[*set_n] = j;
      }
      if (set_n) (*set_n)++;
      for (int m = 0; m < p->nmaps; m++) {
        float curval = vmap[m] * orc_interpolate_table(c, &tabs[p->table_id[m]], angle,
                                                       hs->redshift, &hs->mh, p->profile[m]);
        deposit(o, 1, m, j, curval);
      }
    }
  }
  return 0;
}

static int check_params(const orc_params *p, int ntables) {
  if (p->model < 1 || p->model > 3) return -10;
  if (p->nmaps < 1 || p->nmaps > ORC_MAXMAPS) return -11;
  if (p->nfloat != 7 && p->nfloat != 10) return -12;
  if (p->nside < 0 || p->nside > 8192 || (p->nside & (p->nside - 1))) return -13;
  for (int m = 0; m < p->nmaps; m++) {
    if (p->table_id[m] < 0 || p->table_id[m] >= ntables) return -14;
    if (p->profile[m] != 1 && p->profile[m] != 2) return -15;
  }
  return 0;
}

/* ------------------------------------------------------- scramble and centre -------- */

/* random.f90:264-286: c = a * b on four 12-bit digits, carries propagated, truncated to
   four digits (the digits of b may exceed 4095: pks2map seeds every digit with
   13579 * (rank + 1)) */
static void ranf_modmult(const int64_t a[4], const int64_t b[4], int64_t c[4]) {
  int64_t j1 = a[0] * b[0];
  int64_t j2 = a[0] * b[1] + a[1] * b[0];
  int64_t j3 = a[0] * b[2] + a[1] * b[1] + a[2] * b[0];
  int64_t j4 = a[0] * b[3] + a[1] * b[2] + a[2] * b[1] + a[3] * b[0];
  int64_t k1 = j1, k2 = j2 + k1 / 4096, k3 = j3 + k2 / 4096, k4 = j4 + k3 / 4096;
  c[0] = k1 % 4096;
  c[1] = k2 % 4096;
  c[2] = k3 % 4096;
  c[3] = k4 % 4096;
}

/* random.f90:40-57: the output from the current seed, then seed = multiplier * seed */
static double ranf(int64_t seed[4]) {
  static const int64_t mult[4] = {373, 3707, 1442, 647};
  double r = (((double)(float)seed[3] / 4096.0 + (double)(float)seed[2] / 16777216.0) +
              (double)(float)seed[1] / 68719476736.0) +
             (double)(float)seed[0] / 281474976710656.0;
  int64_t out[4];
  ranf_modmult(mult, seed, out);
  memcpy(seed, out, sizeof(out));
  return r;
}

/* pks2map.f90:144-262 before the halo loop: the radial cut (surv), then with scramble a
   random direction per surviving halo from its rank's ranf stream (seed 13579*(rank+1)
   in every digit, two draws per halo in rank order; :162-187), then with centre the
   flips and two rotations that put the largest-RTH halo on the z axis (:189-262).
   trec: the records with the new positions (fields 0..2 = posxyz(1..3)). */
static void preprocess(const orc_params *p, const float *recs, int64_t n, float cut_low,
                       float cut_high, float *trec, unsigned char *surv, float info[9]) {
  const int nf = p->nfloat;
  const int ntasks = p->ntasks > 1 ? p->ntasks : 1;
  const int64_t per = n > 0 ? (n - 1) / ntasks + 1 : 1;
  memcpy(trec, recs, sizeof(float) * (size_t)(n * nf));
  for (int64_t i = 0; i < n; i++)
    surv[i] = (unsigned char)halo_in_shell(recs + i * nf, p->chihview, cut_low, cut_high);
  if (p->scramble) {
    for (int r = 0; r < ntasks; r++) {
      int64_t seed[4];
      for (int k = 0; k < 4; k++) seed[k] = 13579LL * (r + 1);
      for (int64_t i = r * per; i < n && i < (r + 1) * per; i++) {
        if (!surv[i]) continue;
        float *q = trec + i * nf;
        float xh = q[0], yh = q[1], zh = q[2];
        float chih = sqrtf(((xh * xh) + (yh * yh)) + (zh * zh));
        double rnd = ranf(seed);
        float muran = (float)(2.0 * rnd - 1.0);
        rnd = ranf(seed);
        float phiran = (float)((double)(2.0f * 3.14159f) * rnd);
        float rh = sqrtf(1.0f - muran * muran) * chih;
        q[0] = rh * p2m_cosf(phiran);
        q[1] = rh * p2m_sinf(phiran);
        q[2] = muran * chih;
      }
    }
  }
  for (int k = 0; k < 9; k++) info[k] = 0.0f;
  if (!p->centre) return;
  float rthmax = -1.0f;
  for (int64_t i = 0; i < n; i++)
    if (surv[i] && recs[i * nf + 6] > rthmax) rthmax = recs[i * nf + 6];
  /* per rank: the last survivor with rth == RTHmax; then MAX over ranks per coordinate */
  float xm = -1e5f, ym = -1e5f, zm = -1e5f;
  for (int r = 0; r < ntasks; r++) {
    float xl = -1e5f, yl = -1e5f, zl = -1e5f;
    for (int64_t i = r * per; i < n && i < (r + 1) * per; i++) {
      if (!surv[i] || recs[i * nf + 6] != rthmax) continue;
      xl = trec[i * nf + 2];
      yl = trec[i * nf + 1];
      zl = trec[i * nf + 0];
    }
    if (xl > xm) xm = xl;
    if (yl > ym) ym = yl;
    if (zl > zm) zm = zl;
  }
  info[0] = rthmax;
  info[1] = sqrtf(((xm * xm) + (ym * ym)) + (zm * zm));
  info[2] = xm;
  info[3] = ym;
  info[4] = zm;
  const int f3 = xm < 0.0f, f2 = ym < 0.0f, f1 = zm < 0.0f;
  xm = fabsf(xm);
  ym = fabsf(ym);
  zm = fabsf(zm);
  float theta = p2m_asinf(zm / sqrtf((xm * xm) + (zm * zm)));
  float xml = (xm / fabsf(xm)) * sqrtf((xm * xm) + (zm * zm));
  float phi = p2m_asinf(ym / sqrtf((ym * ym) + (xml * xml)));
  float ct = p2m_cosf(theta), st = p2m_sinf(theta), cp = p2m_cosf(phi), sp = p2m_sinf(phi);
  for (int64_t i = 0; i < n; i++) {
    if (!surv[i]) continue;
    float *q = trec + i * nf;
    float p1 = f1 ? -q[0] : q[0], p2 = f2 ? -q[1] : q[1], p3 = f3 ? -q[2] : q[2];
    float xh = (p3 * ct) + (p1 * st);
    float zh = ((-p3) * st) + (p1 * ct);
    float yh = ((-xh) * sp) + (p2 * cp);
    xh = (xh * cp) + (p2 * sp);
    q[2] = zh;
    q[1] = yh;
    q[0] = xh;
  }
  for (int r = 0; r < ntasks; r++)
    for (int64_t i = r * per; i < n && i < (r + 1) * per; i++) {
      if (!surv[i] || recs[i * nf + 6] != rthmax) continue;
      const float *q = trec + i * nf;
      info[5] = sqrtf(((q[2] * q[2]) + (q[1] * q[1])) + (q[0] * q[0]));
      info[6] = q[2];
      info[7] = q[1];
      info[8] = q[0];
    }
}

/* halo loop over records [h0, h1): pks2map.f90:134-303.  With surv, the radial cut has
   been made (surv[i]) and records holds the scrambled / rotated positions, while orig
   holds the records as read (for the line-of-sight velocity). */
static int paint_range(const orc_cosmo *c, const orc_params *p, const orc_table *tabs,
                       const float *records, int64_t h0, int64_t h1, const paint_out *o,
                       orc_stats *st, int64_t *set_halo, int64_t *set_pix, int64_t set_cap,
                       int64_t *set_n, const unsigned char *surv, const float *orig) {
  float cut_low = orc_rofz(c, p->zmin), cut_high = orc_rofz(c, p->zmax);
  /* pks2map.f90:92-93: fov to radians, dpix */
  float fov = ((p->fov_deg / 360.0f) * 2.0f) * c->mypi;
  float dpix = p->npix_fs > 0 ? fov / (float)p->npix_fs : 0.0f;
  int64_t listcap = p->nside > 0 ? 12 * (int64_t)p->nside * p->nside : 1;
  int64_t *list = (int64_t *)malloc(sizeof(int64_t) * (size_t)listcap);
  if (!list) return -20;
  int rc = 0;
  for (int64_t i = h0; i < h1; i++) {
    const float *rec = records + i * p->nfloat;
    st->n_in++;
    if (surv ? !surv[i] : !halo_in_shell(rec, p->chihview, cut_low, cut_high)) continue;
    st->n_cut++;
    halo_state hs;
    if (!halo_prepare(c, p, rec, &hs)) continue;
    st->n_painted++;
    /* a scrambled halo with a NaN position (each rank's first: its seed's unreduced
       digits give a first draw above 1) counts and paints nothing */
    if (!isfinite(hs.xh) || !isfinite(hs.yh) || !isfinite(hs.zh)) continue;
    float vmap[ORC_MAXMAPS];
    const float *vrec = surv ? orig + i * p->nfloat : rec;
    for (int m = 0; m < p->nmaps; m++) vmap[m] = halo_vrad(vrec, p->profile[m]);
    projecthalo_flatsky(c, p, tabs, &hs, vmap, fov, dpix, o, st);
    if (p->nside > 0) {
      rc = projecthalo_healpix(c, p, tabs, &hs, vmap, list, listcap, o, st, i, set_halo,
                               set_pix, set_cap, set_n);
      if (rc) break;
    }
  }
  free(list);
  return rc;
}

int orc_paint(const orc_params *p, const orc_table *tables, int ntables, const float *records,
              int64_t nhalo, void *hp_out, void *fs_out, orc_stats *stats, int64_t *set_halo,
              int64_t *set_pix, int64_t set_cap, int64_t *set_n) {
  int rc = check_params(p, ntables);
  if (rc) return rc;
  orc_cosmo *c = (orc_cosmo *)malloc(sizeof(orc_cosmo));
  orc_cosmo_init(c);
  paint_out o;
  memset(&o, 0, sizeof(o));
  o.fp32 = p->fp32_accumulate;
  o.hp_npix = 12 * (int64_t)p->nside * p->nside;
  o.fs_npix2 = (int64_t)p->npix_fs * p->npix_fs;
  if (o.fp32) {
    o.hp32 = (float *)hp_out;
    o.fs32 = (float *)fs_out;
    if (o.hp32) memset(o.hp32, 0, sizeof(float) * (size_t)(o.hp_npix * p->nmaps));
    if (o.fs32) memset(o.fs32, 0, sizeof(float) * (size_t)(o.fs_npix2 * p->nmaps));
  } else {
    o.hp64 = (double *)hp_out;
    o.fs64 = (double *)fs_out;
    if (o.hp64) memset(o.hp64, 0, sizeof(double) * (size_t)(o.hp_npix * p->nmaps));
    if (o.fs64) memset(o.fs64, 0, sizeof(double) * (size_t)(o.fs_npix2 * p->nmaps));
  }
  orc_stats st;
  memset(&st, 0, sizeof(st));
  if (set_n) *set_n = 0;
  if (p->scramble || p->centre) {
    float *trec = (float *)malloc(sizeof(float) * (size_t)(nhalo * p->nfloat + 1));
    unsigned char *surv = (unsigned char *)malloc((size_t)nhalo + 1);
    if (!trec || !surv) {
      free(trec);
      free(surv);
      free(c);
      return -20;
    }
    preprocess(p, records, nhalo, orc_rofz(c, p->zmin), orc_rofz(c, p->zmax), trec, surv,
               st.centre);
    rc = paint_range(c, p, tables, trec, 0, nhalo, &o, &st, set_halo, set_pix, set_cap, set_n,
                     surv, records);
    free(trec);
    free(surv);
  } else {
    rc = paint_range(c, p, tables, records, 0, nhalo, &o, &st, set_halo, set_pix, set_cap,
                     set_n, NULL, NULL);
  }
  if (stats) *stats = st;
  free(c);
  return rc;
}

/* orc_paint in FP64 accumulation with nthreads threads, with the same result bit for bit:
   each thread runs the halo loop over a contiguous block of records and logs its deposits
   (and pixel-set pairs) instead of adding them; the logs are then replayed in thread
   order, i.e. in halo order, the adds of every map pixel in the serial loop's order
   (each replaying thread owns a contiguous range of map pixels).  For catalogues whose
   serial loop would take minutes.  set_* as orc_paint. */
int orc_paint_parallel(const orc_params *p, const orc_table *tables, int ntables,
                       const float *records, int64_t nhalo, double *hp_out, double *fs_out,
                       orc_stats *stats, int64_t *set_halo, int64_t *set_pix, int64_t set_cap,
                       int64_t *set_n, int nthreads) {
  int rc = check_params(p, ntables);
  if (rc) return rc;
  if (p->fp32_accumulate) return -16;
  if (nthreads < 1) nthreads = 1;
  orc_cosmo *c = (orc_cosmo *)malloc(sizeof(orc_cosmo));
  if (!c) return -20;
  orc_cosmo_init(c);
  const int64_t hp_npix = 12 * (int64_t)p->nside * p->nside;
  const int64_t fs_npix2 = (int64_t)p->npix_fs * p->npix_fs;
  const int64_t hp_n = hp_npix * p->nmaps, fs_n = fs_npix2 * p->nmaps;
  orc_stats st;
  memset(&st, 0, sizeof(st));
  float *trec = NULL;
  unsigned char *surv = NULL;
  const float *recs = records;
  if (p->scramble || p->centre) {
    trec = (float *)malloc(sizeof(float) * (size_t)(nhalo * p->nfloat + 1));
    surv = (unsigned char *)malloc((size_t)nhalo + 1);
    if (!trec || !surv) {
      free(trec);
      free(surv);
      free(c);
      return -20;
    }
    preprocess(p, records, nhalo, orc_rofz(c, p->zmin), orc_rofz(c, p->zmax), trec, surv,
               st.centre);
    recs = trec;
  }
  dep_log *logs = (dep_log *)calloc((size_t)nthreads, sizeof(dep_log));
  dep_log *sets = (dep_log *)calloc((size_t)nthreads, sizeof(dep_log));
  orc_stats *sts = (orc_stats *)calloc((size_t)nthreads, sizeof(orc_stats));
  int *rcs = (int *)calloc((size_t)nthreads, sizeof(int));
  if (!logs || !sets || !sts || !rcs) {
    free(logs);
    free(sets);
    free(sts);
    free(rcs);
    free(trec);
    free(surv);
    free(c);
    return -20;
  }
  int64_t per = nhalo > 0 ? (nhalo - 1) / nthreads + 1 : 0;
#pragma omp parallel num_threads(nthreads)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    int64_t h0 = per * tid, h1 = h0 + per;
    if (h1 > nhalo) h1 = nhalo;
    if (h0 < h1) {
      paint_out o;
      memset(&o, 0, sizeof(o));
      o.hp_npix = hp_npix;
      o.fs_npix2 = fs_npix2;
      o.log = &logs[tid];
      o.sets = (set_halo || set_n) ? &sets[tid] : NULL;
      rcs[tid] = paint_range(c, p, tables, recs, h0, h1, &o, &sts[tid], NULL, NULL, 0, NULL,
                             surv, surv ? records : NULL);
    }
  }
  for (int t = 0; t < nthreads; t++) {
    if (rcs[t] && !rc) rc = rcs[t];
    if ((logs[t].err || sets[t].err) && !rc) rc = -20;
  }
  if (!rc) {
    if (hp_out) memset(hp_out, 0, sizeof(double) * (size_t)(hp_n > 0 ? hp_n : 0));
    if (fs_out) memset(fs_out, 0, sizeof(double) * (size_t)(fs_n > 0 ? fs_n : 0));
    /* replay: worker w adds the logged values whose map index falls in its range */
#pragma omp parallel num_threads(nthreads)
    {
#ifdef _OPENMP
      int w = omp_get_thread_num();
#else
      int w = 0;
#endif
      int64_t hlo = hp_n * w / nthreads, hhi = hp_n * (w + 1) / nthreads;
      int64_t flo = fs_n * w / nthreads, fhi = fs_n * (w + 1) / nthreads;
      for (int t = 0; t < nthreads; t++) {
        const dep_log *l = &logs[t];
        for (int64_t i = 0; i < l->n; i++) {
          int64_t k = l->key[i];
          if (k >= 0) {
            if (k >= hlo && k < hhi && hp_out) hp_out[k] = hp_out[k] + (double)l->val[i];
          } else {
            k = -1 - k;
            if (k >= flo && k < fhi && fs_out) fs_out[k] = fs_out[k] + (double)l->val[i];
          }
        }
      }
    }
    int64_t n = 0;
    for (int t = 0; t < nthreads; t++) {
      for (int64_t i = 0; i < sets[t].n; i++, n++) {
        if (set_halo && n < set_cap) {
          set_halo[n] = sets[t].key[i];
          set_pix[n] = sets[t].aux[i];
        }
      }
    }
    if (set_n) *set_n = n;
  }
  for (int t = 0; t < nthreads; t++) {
    st.n_in += sts[t].n_in;
    st.n_cut += sts[t].n_cut;
    st.n_painted += sts[t].n_painted;
    st.hp_updates += sts[t].hp_updates;
    st.fs_updates += sts[t].fs_updates;
    st.hp_candidates += sts[t].hp_candidates;
    st.ring_gaps += sts[t].ring_gaps;
    log_free(&logs[t]);
    log_free(&sets[t]);
  }
  if (stats) *stats = st;
  free(logs);
  free(sets);
  free(sts);
  free(rcs);
  free(trec);
  free(surv);
  free(c);
  return rc;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int orc_paint_threads(const orc_params *p, const orc_table *tables, int ntables,
                      const float *records, int64_t nhalo, float *hp_out, float *fs_out,
                      int nthreads, orc_stats *stats, double t[3]) {
  int rc = check_params(p, ntables);
  if (rc) return rc;
  if (nthreads < 1) nthreads = 1;
  orc_cosmo *c = (orc_cosmo *)malloc(sizeof(orc_cosmo));
  orc_cosmo_init(c);
  int64_t hp_n = 12 * (int64_t)p->nside * p->nside * p->nmaps;
  int64_t fs_n = (int64_t)p->npix_fs * p->npix_fs * p->nmaps;
  double t0 = now_s();
  /* each "rank" owns private maps (pks2map.f90:110-115) */
  float **hpl = (float **)calloc((size_t)nthreads, sizeof(float *));
  float **fsl = (float **)calloc((size_t)nthreads, sizeof(float *));
  orc_stats *sts = (orc_stats *)calloc((size_t)nthreads, sizeof(orc_stats));
  int *rcs = (int *)calloc((size_t)nthreads, sizeof(int));
#pragma omp parallel num_threads(nthreads)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    hpl[tid] = (float *)calloc((size_t)(hp_n > 0 ? hp_n : 1), sizeof(float));
    fsl[tid] = (float *)calloc((size_t)(fs_n > 0 ? fs_n : 1), sizeof(float));
    /* `fsmapl = 0; hpmapl = 0` (pks2map.f90:278-279) writes every page of the rank's maps
       before the halo loop: done here too, so that the set-up time carries the page
       faults and the painting time is painting only */
    if (hpl[tid]) memset(hpl[tid], 0, sizeof(float) * (size_t)(hp_n > 0 ? hp_n : 1));
    if (fsl[tid]) memset(fsl[tid], 0, sizeof(float) * (size_t)(fs_n > 0 ? fs_n : 1));
  }
  double t1 = now_s();
  /* pksc.f90:51-52: nhalol = (N-1)/ntasks + 1 per rank */
  int64_t per = (nhalo - 1) / nthreads + 1;
#pragma omp parallel num_threads(nthreads)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    int64_t h0 = per * tid, h1 = h0 + per;
    if (h1 > nhalo) h1 = nhalo;
    if (h0 < h1) {
      paint_out o;
      memset(&o, 0, sizeof(o));
      o.fp32 = 1;
      o.hp32 = hpl[tid];
      o.fs32 = fsl[tid];
      o.hp_npix = 12 * (int64_t)p->nside * p->nside;
      o.fs_npix2 = (int64_t)p->npix_fs * p->npix_fs;
      rcs[tid] = paint_range(c, p, tables, records, h0, h1, &o, &sts[tid], NULL, NULL, 0, NULL,
                             NULL, NULL);
    }
  }
  double t2 = now_s();
  /* MPI_Allreduce(SUM) of the float maps (pks2map.f90:313-314), rank order */
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int64_t k = 0; k < hp_n; k++) {
    float s = 0.0f;
    for (int r = 0; r < nthreads; r++) s = s + hpl[r][k];
    if (hp_out) hp_out[k] = s;
  }
  for (int64_t k = 0; k < fs_n; k++) {
    float s = 0.0f;
    for (int r = 0; r < nthreads; r++) s = s + fsl[r][k];
    if (fs_out) fs_out[k] = s;
  }
  double t3 = now_s();
  orc_stats st;
  memset(&st, 0, sizeof(st));
  for (int r = 0; r < nthreads; r++) {
    st.n_in += sts[r].n_in;
    st.n_cut += sts[r].n_cut;
    st.n_painted += sts[r].n_painted;
    st.hp_updates += sts[r].hp_updates;
    st.fs_updates += sts[r].fs_updates;
    st.hp_candidates += sts[r].hp_candidates;
    st.ring_gaps += sts[r].ring_gaps;
    if (rcs[r]) rc = rcs[r];
    free(hpl[r]);
    free(fsl[r]);
  }
  free(hpl);
  free(fsl);
  free(sts);
  free(rcs);
  free(c);
  if (stats) *stats = st;
  if (t) {
    t[0] = t1 - t0;
    t[1] = t2 - t1;
    t[2] = t3 - t2;
  }
  return rc;
}

/* The halo loop of every "rank" over records [0, nhalo), split as pksc.f90:51-52 splits
   them, painting into caller-owned private HEALPix float maps (hp_maps[r]: nmaps * 12 *
   nside^2 floats), without allocating, zeroing or reducing them: for timing the painting
   alone over repeated samples.  HEALPix only (npix_fs must be 0). */
int orc_paint_ranks(const orc_params *p, const orc_table *tables, int ntables,
                    const float *records, int64_t nhalo, float **hp_maps, int nthreads,
                    orc_stats *stats) {
  int rc = check_params(p, ntables);
  if (rc) return rc;
  if (p->npix_fs > 0 || p->nside <= 0 || nthreads < 1) return -1;
  orc_cosmo *c = (orc_cosmo *)malloc(sizeof(orc_cosmo));
  orc_cosmo_init(c);
  orc_stats *sts = (orc_stats *)calloc((size_t)nthreads, sizeof(orc_stats));
  int *rcs = (int *)calloc((size_t)nthreads, sizeof(int));
  int64_t per = (nhalo - 1) / nthreads + 1;
#pragma omp parallel num_threads(nthreads)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    int64_t h0 = per * tid, h1 = h0 + per;
    if (h1 > nhalo) h1 = nhalo;
    if (h0 < h1) {
      paint_out o;
      memset(&o, 0, sizeof(o));
      o.fp32 = 1;
      o.hp32 = hp_maps[tid];
      o.hp_npix = 12 * (int64_t)p->nside * p->nside;
      rcs[tid] = paint_range(c, p, tables, records, h0, h1, &o, &sts[tid], NULL, NULL, 0, NULL,
                             NULL, NULL);
    }
  }
  orc_stats st;
  memset(&st, 0, sizeof(st));
  for (int r = 0; r < nthreads; r++) {
    st.n_in += sts[r].n_in;
    st.n_cut += sts[r].n_cut;
    st.n_painted += sts[r].n_painted;
    st.hp_updates += sts[r].hp_updates;
    st.hp_candidates += sts[r].hp_candidates;
    st.ring_gaps += sts[r].ring_gaps;
    if (rcs[r]) rc = rcs[r];
  }
  free(sts);
  free(rcs);
  free(c);
  if (stats) *stats = st;
  return rc;
}

/* `hpmapl = 0` (pks2map.f90:279) of every rank, each rank writing its own map */
void orc_zero_ranks(float **maps, int nranks, int64_t n) {
#pragma omp parallel for num_threads(nranks) schedule(static, 1)
  for (int r = 0; r < nranks; r++) memset(maps[r], 0, sizeof(float) * (size_t)n);
}

/* MPI_Allreduce(SUM) of the ranks' float maps in rank order (pks2map.f90:313-314) */
void orc_reduce_ranks(float **maps, int nranks, int64_t n, float *out, int nthreads) {
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int64_t k = 0; k < n; k++) {
    float s = 0.0f;
    for (int r = 0; r < nranks; r++) s = s + maps[r][k];
    out[k] = s;
  }
}

/* host evaluation of the shared float math (p2m_fmath.h) for tests:
   fn 0 log, 1 exp, 2 pow, 3 asin, 4 atan, 5 sin, 6 cos, 7 tan */
void orc_fmath_eval(int fn, const float *x, const float *y, float *out, int64_t n) {
  for (int64_t i = 0; i < n; i++) {
    float a = x[i], b = y ? y[i] : 0.0f, r;
    switch (fn) {
      case 0: r = p2m_logf(a); break;
      case 1: r = p2m_expf(a); break;
      case 2: r = p2m_powf(a, b); break;
      case 3: r = p2m_asinf(a); break;
      case 4: r = p2m_atanf(a); break;
      case 5: r = p2m_sinf(a); break;
      case 6: r = p2m_cosf(a); break;
      case 9: r = p2m_tanf_pio4(a); break;
      case 10: r = p2m_logf_normal(a); break;
      default: r = p2m_tanf(a); break;
    }
    out[i] = r;
  }
}

/* ------------------------------------------------------------- table maker -------- */

/* bbps_profile.f90:9-55 parameter tables */
static const float P0_Am[3] = {18.100f, 7.490f, 20.7f};
static const float P0_alpham[3] = {0.154f, 0.226f, -0.074f};
static const float P0_alphaz[3] = {-0.758f, -0.957f, -0.743f};
static const float xc_Am[3] = {0.497f, 0.710f, 0.438f};
static const float xc_alpham[3] = {-0.00865f, -0.0833f, 0.011f};
static const float xc_alphaz[3] = {0.731f, 0.853f, 1.01f};
static const float beta_Am[3] = {4.35f, 4.19f, 3.82f};
static const float beta_alpham[3] = {0.0393f, 0.048f, 0.0375f};
static const float beta_alphaz[3] = {0.415f, 0.615f, 0.535f};
static const float BBPS_ALPHA = 1.0f, BBPS_GAMMA = -0.3f;
static const float P0_Am_rho[3] = {1.9e-5f, 9.1e-05f, 1.5e-4f};
static const float P0_alpham_rho[3] = {0.29f, 0.10f, 0.14f};
static const float P0_alphaz_rho[3] = {-0.67f, -0.92f, -1.32f};
static const float alpha_Am_rho[3] = {0.88f, 0.69f, 0.68f};
static const float alpha_alpham_rho[3] = {-0.03f, -0.02f, -0.02f};
static const float alpha_alphaz_rho[3] = {0.20f, 0.27f, 0.29f};
static const float beta_Am_rho[3] = {3.83f, 4.43f, 6.4f};
static const float beta_alpham_rho[3] = {0.044f, 0.0035f, 0.028f};
static const float beta_alphaz_rho[3] = {-0.025f, 0.037f, -0.25f};
static const float XC_RHO = 0.5f, GAMMA_RHO = 0.2f;

/* A0*(mh/1e14)**alpham*(1+z)**alphaz (bbps_profile.f90:91,99,107,151,159,167) */
static float bbps_scaling(float A0, float alpham, float alphaz, float mh, float z) {
  return (A0 * p2m_powf(mh / 1e14f, alpham)) * p2m_powf(1.0f + z, alphaz);
}

/* integrate_profiles.f90:12-95 with bbps_profile.f90:60-180; the per-(z, mh)
   profile parameters are evaluated once (identical values to per-step evaluation) */
static float integrate_profile(const orc_cosmo *c, int model, int which, float theta,
                               float z, float mh) {
  int i = model - 1;
  const float rmax = 4.0f, ds = 1e-2f;
  float Delta = BBPS_DELTA[i];
  float chi = orc_rofz(c, z);
  double t = (double)((3.0f * mh) / 4.0f) / COSMO_PI;
  t = t / (double)Delta;
  t = t / (double)orc_rhocrit(c, z);
  float rvir = (float)pow(t, (double)(1.0f / 3.0f));
  float b = (chi * p2m_sinf(theta)) / rvir;
  if (b > rmax) return 0.0f;
  if (which == 1) {
    float P0 = bbps_scaling(P0_Am[i], P0_alpham[i], P0_alphaz[i], mh, z);
    float xc = bbps_scaling(xc_Am[i], xc_alpham[i], xc_alphaz[i], mh, z);
    float beta = bbps_scaling(beta_Am[i], beta_alpham[i], beta_alphaz[i], mh, z);
    float s0 = rmax;
    int n = (int)(s0 / ds) + 1;
    float y = 0.0f;
    for (int k = 1; k <= n; k++) {
      float s = ((float)k - 0.5f) * ds;
      float x = sqrtf((s * s) + (b * b));
      float xx = x / xc;
      float pt = (P0 * p2m_powf(xx, BBPS_GAMMA)) * p2m_powf(1.0f + p2m_powf(xx, BBPS_ALPHA), -beta);
      y = y + pt;
    }
    return y * ds;
  } else {
    float P0 = bbps_scaling(P0_Am_rho[i], P0_alpham_rho[i], P0_alphaz_rho[i], mh, z);
    float alpha_rho = bbps_scaling(alpha_Am_rho[i], alpha_alpham_rho[i], alpha_alphaz_rho[i], mh, z);
    float beta = bbps_scaling(beta_Am_rho[i], beta_alpham_rho[i], beta_alphaz_rho[i], mh, z);
    float s0 = sqrtf((rmax * rmax) - (b * b));
    int n = (int)(s0 / ds) + 1;
    float e1 = -1.0f * GAMMA_RHO;
    float e2 = (-1.0f * (beta - GAMMA_RHO)) / alpha_rho;
    float rho = 0.0f;
    for (int k = 1; k <= n; k++) {
      float s = ((float)k - 0.5f) * ds;
      float x = sqrtf((s * s) + (b * b));
      float xx = x / XC_RHO;
      float rt = (P0 * p2m_powf(xx, e1)) * p2m_powf(1.0f + p2m_powf(xx, alpha_rho), e2);
      rho = rho + rt;
    }
    rho = rho * ds;
    return 2.0f * rho;
  }
}

/* maptable.f90:25-146 (make_maptable.f90:32-43 sets the same cosmology) */
int64_t orc_make_maptable(int model, float nu, float alpha_cmb, int nchit, int nmht, int nrt,
                          void *image, int nthreads) {
  if (nchit <= 0) nchit = 100;
  if (nmht <= 0) nmht = 100;
  if (nrt <= 0) nrt = 200;
  if (model < 1 || model > 3 || nchit < 2 || nmht < 2 || nrt < 2) return -1;
  int64_t nbytes = 36 + 8 * (int64_t)nchit * nmht * nrt;
  if (!image) return nbytes;
  orc_cosmo *c = (orc_cosmo *)malloc(sizeof(orc_cosmo));
  orc_cosmo_init(c);
  /* cosmology.f90:11-38 (mp and mue are single-precision literals) */
  const double sigmat = 6.65246e-25, me = 9.109383e-28, mp = (double)1.67e-24f;
  const double msun = 1.9891e33, Mpc2km = 3.08567758e19, Mpc = 3.08567758e24,
               kpc = 3.08567758e21;
  const double H100 = 1e2 / Mpc2km;
  const float mue = 1.136f;
  const double ypermass =
      ((((((3.0 * sigmat) * (H100 * H100)) / 8.0) / COSMO_PI) / me) / (COSMO_C * COSMO_C) * msun) /
      (double)1.932f;
  const double taupersigma = (((sigmat / (double)mue) / mp) * msun / ((kpc * kpc) * kpc)) * Mpc * 1e10;
  float Delta = BBPS_DELTA[model - 1];
  float m2rfac = (float)pow(((double)(3.0f / 4.0f) / COSMO_PI) / (double)Delta, (double)(1.0f / 3.0f));
  float y0 = (float)((double)((c->fb * Delta) * (c->h * c->h)) * ypermass);
  float tau0 = (float)((taupersigma * (double)(c->h * c->h)) * (double)m2rfac);
  float x0const = 0.017612f * nu;
  float chimint = 1e2f, chimaxt = 7e3f, mhmint = 1e13f, mhmaxt = 1e16f, rmint = 1e-2f, rmaxt = 10.0f;
  float dchit = (p2m_logf(chimaxt) - p2m_logf(chimint)) / (float)(nchit - 1);
  float dmht = (p2m_logf(mhmaxt) - p2m_logf(mhmint)) / (float)(nmht - 1);
  float drt = (p2m_logf(rmaxt) - p2m_logf(rmint)) / (float)(nrt - 1);
  char *b = (char *)image;
  memcpy(b + 0, &nchit, 4);
  memcpy(b + 4, &nmht, 4);
  memcpy(b + 8, &nrt, 4);
  memcpy(b + 12, &chimint, 4);
  memcpy(b + 16, &chimaxt, 4);
  memcpy(b + 20, &mhmint, 4);
  memcpy(b + 24, &mhmaxt, 4);
  memcpy(b + 28, &rmint, 4);
  memcpy(b + 32, &rmaxt, 4);
  float *table = (float *)(b + 36);
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
  for (int i = 1; i <= nchit; i++) {
    float chit = p2m_expf(p2m_logf(chimint) + ((float)(i - 1) * dchit));
    float z = orc_zofr(c, chit);
    float zp1 = 1.0f + z;
    float zfacy = (c->omegam * ((zp1 * zp1) * zp1)) + c->omegal;
    float zfact = (1.0f / zp1) / p2m_powf(orc_rhocrit(c, z), 1.0f / 3.0f);
    float Gx = 0.0f;
    if (nu > 0.0f) {
      float x0new = x0const * p2m_powf(zp1, alpha_cmb);
      float ex = p2m_expf(x0new);
      Gx = ((x0new * (ex + 1.0f)) / (ex - 1.0f)) - 4.0f;
    }
    for (int j = 1; j <= nmht; j++) {
      float mht = p2m_expf(p2m_logf(mhmint) + ((float)(j - 1) * dmht));
      float mht3 = p2m_powf(mht, 1.0f / 3.0f);
      for (int k = 1; k <= nrt; k++) {
        float rt = p2m_expf(p2m_logf(rmint) + ((float)(k - 1) * drt));
        float theta = p2m_atanf(rt / chit);
        float y = ((y0 * mht) * zfacy) * integrate_profile(c, model, 1, theta, z, mht);
        if (nu > 0.0f) y = y * Gx;
        float tau = ((tau0 * mht3) * zfact) * integrate_profile(c, model, 2, theta, z, mht);
        int64_t off = 2 * ((int64_t)(k - 1) + (int64_t)nrt * ((int64_t)(j - 1) + (int64_t)nmht * (i - 1)));
        table[off] = y;
        table[off + 1] = tau;
      }
    }
  }
  free(c);
  return nbytes;
}

/* ------------------------------------------------------- synthetic catalogue ------- */

/* The synthetic catalogue generator of the GPU library (include/p2m_tools.h) restated for
   the CPU arms, so that they never load the product library: Philox4x32-10 (Salmon,
   Moraes, Dror and Shaw, SC 2011: ten rounds of two 32x32->64 multiplies, Weyl key
   schedule), counter = record index, two blocks per record; positions uniform in volume
   in the shell, isotropic directions, masses dN/dlnM ~ M^slope by inverse CDF, RTH from
   M = (4 pi / 3) 0.31 * 2.775e11 * 0.68^2 RTH^3, Gaussian velocities (Box-Muller),
   Lagrangian positions x - 0.01 v.  Double precision throughout, stored as float. */
static void orc_philox(const uint32_t c[4], const uint32_t k[2], uint32_t out[4]) {
  uint32_t x0 = c[0], x1 = c[1], x2 = c[2], x3 = c[3], k0 = k[0], k1 = k[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * x0, p1 = (uint64_t)0xCD9E8D57u * x2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ x1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ x3 ^ k1;
    x1 = (uint32_t)p1;
    x3 = (uint32_t)p0;
    x0 = n0;
    x2 = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = x0;
  out[1] = x1;
  out[2] = x2;
  out[3] = x3;
}

#define ORC_M_PI 3.14159265358979323846 /* the double nearest pi, as M_PI */

static double orc_u01(uint32_t x) { return ((double)x + 0.5) * (1.0 / 4294967296.0); }

int orc_generate_catalogue(uint64_t seed, int64_t first, int64_t n, int nfloat, double r_min,
                           double r_max, double m_min, double m_max, double slope,
                           double sigma_v, float *out, int nthreads) {
  if (!out || n < 0 || first < 0 || (nfloat != 7 && nfloat != 10)) return 1;
  if (!(r_min >= 0 && r_max >= r_min && m_min > 0 && m_max >= m_min && slope != 0.0)) return 1;
  const uint32_t key[2] = {(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32)};
  const double r03 = r_min * r_min * r_min, r13 = r_max * r_max * r_max;
  const double ma = pow(m_min, slope), mb = pow(m_max, slope);
  const double rth_fac = 3.0 / (4.0 * ORC_M_PI * 0.31 * 2.775e11 * 0.68 * 0.68);
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int64_t j = 0; j < n; j++) {
    uint64_t idx = (uint64_t)(first + j);
    uint32_t c0[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 0u, 0u};
    uint32_t c1[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 1u, 0u};
    uint32_t a[4], b[4];
    orc_philox(c0, key, a);
    orc_philox(c1, key, b);
    double r = cbrt(r03 + orc_u01(a[0]) * (r13 - r03));
    double mu = 2.0 * orc_u01(a[1]) - 1.0;
    double ph = 2.0 * ORC_M_PI * orc_u01(a[2]);
    double st = sqrt(fmax(0.0, 1.0 - mu * mu));
    double x = r * st * cos(ph), y = r * st * sin(ph), z = r * mu;
    double m = pow(ma + orc_u01(a[3]) * (mb - ma), 1.0 / slope);
    double rth = cbrt(rth_fac * m);
    double g1 = sqrt(-2.0 * log(orc_u01(b[0]))), t1 = 2.0 * ORC_M_PI * orc_u01(b[1]);
    double g2 = sqrt(-2.0 * log(orc_u01(b[2]))), t2 = 2.0 * ORC_M_PI * orc_u01(b[3]);
    double vx = sigma_v * g1 * cos(t1), vy = sigma_v * g1 * sin(t1), vz = sigma_v * g2 * cos(t2);
    float *o = out + j * nfloat;
    o[0] = (float)x;
    o[1] = (float)y;
    o[2] = (float)z;
    o[3] = (float)vx;
    o[4] = (float)vy;
    o[5] = (float)vz;
    o[6] = (float)rth;
    if (nfloat == 10) {
      o[7] = (float)(x - 0.01 * vx);
      o[8] = (float)(y - 0.01 * vy);
      o[9] = (float)(z - 0.01 * vz);
    }
  }
  return 0;
}

/* --------------------------------------------------------- map statistics ------- */

/* pks2map.f90:321-357 over one float map: moments sum(map**k) / n (k = 1..3, :321-327)
   and RMS sqrt(sum((map - mom1)**2) / n) (:329-334), summed in FP64 with compensation in
   pixel order (the reference's `sum` of a real array accumulates in float in a
   compiler-chosen order; the compensated sum is the value that rounding approximates); with dpdy, P(<y) (:340-357): bin
   m = int(y / dpdy_dy) + 1 with dpdy_dy = dpdy_max / ndpdy = 1e-4 / 10000 in float,
   counted in a float array (a count stops at 2^24), divided by real(n), then cumulated. */
/* Neumaier's compensated sum: s + c carries the sum of the added terms to ~2 ulp of the
   result whatever their count (a plain FP64 loop over 2e8 small map values loses ~1e-9 of
   the total to rounding) */
typedef struct nsum {
  double s, c;
} nsum;
static void nsum_add(nsum *a, double x) {
  const double t = a->s + x;
  if (fabs(a->s) >= fabs(x)) a->c += (a->s - t) + x;
  else a->c += (x - t) + a->s;
  a->s = t;
}

void orc_map_stats(const float *map, int64_t n, double mom[3], double *rms, float *dpdy) {
  nsum s1 = {0.0, 0.0}, s2 = {0.0, 0.0}, s3 = {0.0, 0.0};
  for (int64_t i = 0; i < n; i++) {
    const double x = (double)map[i];
    nsum_add(&s1, x);
    nsum_add(&s2, x * x);
    nsum_add(&s3, (x * x) * x);
  }
  mom[0] = (s1.s + s1.c) / (double)n;
  mom[1] = (s2.s + s2.c) / (double)n;
  mom[2] = (s3.s + s3.c) / (double)n;
  nsum v = {0.0, 0.0};
  for (int64_t i = 0; i < n; i++) {
    const double d = (double)map[i] - mom[0];
    nsum_add(&v, d * d);
  }
  *rms = sqrt((v.s + v.c) / (double)n);
  if (!dpdy) return;
  const int ndpdy = 10000;
  const float dy = 1e-4f / (float)ndpdy;
  for (int k = 0; k < ndpdy; k++) dpdy[k] = 0.0f;
  for (int64_t i = 0; i < n; i++) {
    const float q = map[i] / dy;
    if (!(q > -1.0f && q < (float)ndpdy)) continue; /* int() of it lies outside 0..ndpdy-1 */
    const int m = (int)q + 1;
    if (m > 0 && m <= ndpdy) dpdy[m - 1] = dpdy[m - 1] + 1.0f;
  }
  for (int k = 0; k < ndpdy; k++) dpdy[k] = dpdy[k] / (float)n;
  for (int k = 1; k < ndpdy; k++) dpdy[k] = dpdy[k - 1] + dpdy[k];
}
