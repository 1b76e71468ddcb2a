/*
 * p2m_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement (plain C) of the reference's map-making path, pks2map.  It is the
 * checker for the GPU painter: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it.  Nothing in the product links, imports or calls it.
 *
 * PARITY UNPINNED: the reference ships no tests, golden vectors or fixtures for this
 * path, its catalogue and profile tables are missing, and it cannot be compiled here
 * (Intel Fortran + MPI + cfitsio).  The restatement is pinned only by HEALPix
 * invariants and hand-derived known answers (tests/test_oracle.py).
 *
 * Evaluation rules: Fortran `real` is float and `double precision` is double; every
 * expression is evaluated in source order with the Fortran type-promotion rules; no
 * FMA contraction (-ffp-contract=off); real->integer assignment truncates; single
 * precision intrinsics (asin, log, tan, exp, atan, sin, x**y) are the shared portable
 * implementations in p2m_fmath.h (the role of the Fortran runtime's float libm);
 * double precision intrinsics are the C library's.
 */
#ifndef P2M_ORACLE_H
#define P2M_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAXMAPS 8
#define ORC_NZTAB 10000

typedef struct orc_cosmo {
  float omegam, omegab, omegal, h, fb, rho_0, rhocrit_0;
  float mypi;
  float rofztable[ORC_NZTAB], zofrtable[ORC_NZTAB];
  float drofztable, dzofrtable, rofztable_min, zofrtable_min;
} orc_cosmo;

/* one make_maptable table: header + table(2, nrt, nmht, nchit) (Fortran order) */
typedef struct orc_table {
  int32_t nchit, nmht, nrt;
  float chimint, chimaxt, mhmint, mhmaxt, rmint, rmaxt;
  float dchit, dmht, drt;
  const float *data; /* 2*nrt*nmht*nchit floats */
} orc_table;

typedef struct orc_params {
  int32_t nside;    /* HEALPix Nside; 0 = no HEALPix map */
  int32_t npix_fs;  /* flat-sky side; 0 = no flat-sky map */
  float fov_deg;    /* flat-sky field of view (degrees, as on the command line) */
  float zmin, zmax, chihview;
  int32_t model;    /* bbps model 1..3 */
  int32_t nmaps;
  int32_t profile[ORC_MAXMAPS];  /* 1 = tSZ (weight 1), 2 = kSZ (weight v_los) */
  int32_t table_id[ORC_MAXMAPS];
  int32_t fp32_accumulate;       /* 1: literal float accumulation (hpmapl += curval) */
  int32_t nfloat;                /* 7 or 10 floats per catalogue record */
  int32_t scramble, centre;      /* command-line flags of pks2map.f90:75-76 */
  int32_t ntasks;                /* MPI ranks whose streams and blocks scramble and centre
                                    follow (pksc.f90:51-52; 0 or 1: one rank) */
} orc_params;

typedef struct orc_stats {
  int64_t n_in, n_cut, n_painted;   /* records, after radial cut, after mmin cut */
  int64_t hp_updates, fs_updates;   /* (halo, pixel) pairs passing the disc test */
  int64_t hp_candidates;            /* pixels returned by query_disc */
  int64_t ring_gaps;                /* discs whose non-empty rings are not contiguous */
  float centre[9];                  /* with centre: RTHmax, then distance, x, y, z of the
                                       largest halo before and after the rotation */
} orc_stats;

/* cosmology of pks2map.f90:118-132 and cosmology.f90:51-105 */
void orc_cosmo_init(orc_cosmo *c);
float orc_zofr(const orc_cosmo *c, float r);
float orc_rofz(const orc_cosmo *c, float z);
float orc_rhocrit(const orc_cosmo *c, float z);
float orc_deltacrit(const orc_cosmo *c, float z);

/* table image: 36-byte header then the table (maptable.f90:150-172) */
int orc_table_from_image(orc_table *t, const void *image, int64_t nbytes);
float orc_interpolate_table(const orc_cosmo *c, const orc_table *t, float theta, float z,
                            float *mh, int profile);

/* HEALPix 3.10 (RING scheme) */
int orc_ring_num(int nside, double z);
double orc_ring2z(int nside, int ir);
void orc_pixels_per_ring(int nside, int ring, int *npr, int *kshift, int64_t *npnorth);
void orc_pix2vec_ring(int nside, int64_t ipix, double v[3]);
double orc_angdist(const double v1[3], const double v2[3]);
/* query_disc (non-inclusive, RING).  Returns the pixel count, or -1 if cap exceeded.
   gaps (may be NULL) is set to 1 if the disc's non-empty rings are not contiguous. */
int64_t orc_query_disc(int nside, const double v0[3], double radius, int64_t *list,
                       int64_t cap, int *gaps);

/* The pks2map halo loop (pks2map.f90:134-303) over a catalogue record array.
   hp_out: nmaps * 12*nside^2, fs_out: nmaps * npix_fs^2; double when
   fp32_accumulate == 0, float otherwise.  Set capture (may be NULL): (halo index,
   pixel) of every HEALPix deposit, in loop order.  Returns 0 or a negative error. */
int orc_paint(const orc_params *p, const orc_table *tables, int ntables, const float *records,
              int64_t nhalo, void *hp_out, void *fs_out, orc_stats *stats, int64_t *set_halo,
              int64_t *set_pix, int64_t set_cap, int64_t *set_n);

/* orc_paint in FP64 accumulation (p->fp32_accumulate = 0) on nthreads threads, with the
   same maps, stats and pixel sets bit for bit: the threads log their deposits, which are
   then added in halo order.  Returns -16 for FP32 accumulation. */
int orc_paint_parallel(const orc_params *p, const orc_table *tables, int ntables,
                       const float *records, int64_t nhalo, double *hp_out, double *fs_out,
                       orc_stats *stats, int64_t *set_halo, int64_t *set_pix, int64_t set_cap,
                       int64_t *set_n, int nthreads);

/* Same loop split over nthreads contiguous halo blocks, each painting a private float
   map, summed at the end: the reference's MPI decomposition (pksc.f90:51-66,
   pks2map.f90:313-314) with threads as ranks.  Float output only.  Times (seconds)
   of the map set-up, paint and reduction phases are returned in t[3]. */
int orc_paint_ranks(const orc_params *p, const orc_table *tables, int ntables,
                    const float *records, int64_t nhalo, float **hp_maps, int nthreads,
                    orc_stats *stats);
void orc_reduce_ranks(float **maps, int nranks, int64_t n, float *out, int nthreads);
void orc_zero_ranks(float **maps, int nranks, int64_t n);
int orc_paint_threads(const orc_params *p, const orc_table *tables, int ntables,
                      const float *records, int64_t nhalo, float *hp_out, float *fs_out,
                      int nthreads, orc_stats *stats, double t[3]);

/* make_maptable (maptable.f90:25-146): fills a table image (header + data) of
   nchit*nmht*nrt entries.  Bounds/sizes default to the reference's when <= 0.
   Returns the image size in bytes, or the size needed when image == NULL. */
int64_t orc_make_maptable(int model, float nu, float alpha_cmb, int nchit, int nmht, int nrt,
                          void *image, int nthreads);

/* shared float math evaluated on the host (fn: 0 log 1 exp 2 pow 3 asin 4 atan 5 sin
   6 cos 7 tan; y only for pow) */
void orc_fmath_eval(int fn, const float *x, const float *y, float *out, int64_t n);

/* per-halo derived quantities of the loop, for tests: returns 1 if the halo is painted */
int orc_halo_setup(const orc_cosmo *c, const orc_params *p, const float *rec, float *out8);

/* The synthetic catalogue generator of include/p2m_tools.h (p2m_generate_catalogue),
   restated so that CPU-only callers need not load the GPU library; bit-identical output
   on the same machine.  Returns 0, or 1 for bad arguments. */
int orc_generate_catalogue(uint64_t seed, int64_t first, int64_t n, int nfloat, double r_min,
                           double r_max, double m_min, double m_max, double slope,
                           double sigma_v, float *out, int nthreads);

/* pks2map.f90:321-357 over one float map: moments (k = 1..3), RMS and, with dpdy
   non-null, the cumulative P(<y) of 10000 bins. */
void orc_map_stats(const float *map, int64_t n, double mom[3], double *rms, float *dpdy);

#ifdef __cplusplus
}
#endif
#endif
