/*
 * p2m.h -- C ABI of the GB300 halo painter (drop-in for the pks2map halo loop).
 *
 * Plain C types and pointers only, so that Fortran (ISO_C_BINDING), C, C++ and Python
 * (ctypes) bind it directly.  Every entry point returns a p2m_status; nothing exits,
 * traps or prints.  A context is not thread-safe: use one per host thread.  Interface
 * it replaces (paths relative to the reference project root):
 *
 *   loadmaptable(tablefile)                  maptable.f90:150-172   -> p2m_load_table
 *   loadpksc(filein, profile)                pksc.f90:22-90         -> p2m_paint_records
 *   halo loop + projecthalo_flatsky/healpix  pks2map.f90:276-303,   -> p2m_paint_records
 *                                            haloproject.f90:38-156
 *   projecthalo_flatsky(x,y,z,r,chi,m,       pks2map.f90:300-301    -> p2m_project_halo
 *     redshift,v,profile) + _healpix(...)
 *   MPI_Allreduce of fsmap/hpmap             pks2map.f90:313-314    -> p2m_get_healpix,
 *                                                                      p2m_get_flatsky
 *   halo count / moments                     pks2map.f90:310,321-327 -> p2m_get_stats
 */
#ifndef P2M_H
#define P2M_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct p2m_ctx p2m_ctx;
typedef int32_t p2m_status;

enum {
  P2M_OK = 0,
  P2M_ERR_BADARG = 1,   /* invalid argument or configuration */
  P2M_ERR_CUDA = 2,     /* a CUDA runtime call failed */
  P2M_ERR_CAPACITY = 3, /* a work buffer overflowed (never truncated silently) */
  P2M_ERR_TIMEOUT = 4,  /* reserved (no kernel of this library waits on another) */
  P2M_ERR_IO = 5,       /* malformed table / catalogue image */
  P2M_ERR_STATE = 6,    /* call out of sequence */
  P2M_ERR_NOMEM = 7     /* device or pinned allocation failed */
};

/* precision of the per-pixel path */
enum {
  P2M_PREC_FP64 = 0,  /* plain drop-in: FP64 pixel geometry (pix2vec_ring + angdist) for
                         every candidate, FP64 accumulation */
  P2M_PREC_MIXED = 1, /* FP32 disc test and profile interpolation with an exact FP64
                         recheck near every decision boundary; compensated FP32
                         accumulation: the float maps hold the high words, the exact
                         rounding errors are summed apart and added at read-out */
  P2M_PREC_MIXED_F64 = 2, /* the same decisions; FP64 accumulation (atomic adds executed in
                             L2, not on the SM's FP64 units) */
  P2M_PREC_FIXED = 3      /* the same decisions; 64-bit fixed-point accumulation in units of
                             2^-56 (each value rounded to the unit, |pixel sum| < 128):
                             integer adds do not depend on their order, so the maps are
                             bit-identical from run to run and across launch parameters */
};

/* catalogue layouts (floats per record): 7 = x,y,z,vx,vy,vz,RTH after a 2-word header
   (pksc.f90:46-66); 10 = the same plus xL,yL,zL after a 3-word header */
enum { P2M_LAYOUT_7 = 7, P2M_LAYOUT_10 = 10 };

enum {
  P2M_FLAG_RECORD_SETS = 1, /* keep (record index, pixel) of every HEALPix deposit: up to
                               2^24 pairs, or the count in the environment variable
                               P2M_SET_CAP read by p2m_create; more is P2M_ERR_CAPACITY */
  P2M_FLAG_ALL_HALOS = 2,   /* enumerate halos whose table value is identically zero */
  P2M_FLAG_TIMING = 4,      /* record per-phase device times (p2m_get_timings) */
  P2M_FLAG_VALIDATE = 8     /* mixed precision: also run the exact path for every candidate
                               and count disagreements (p2m_stats.val_*); slow */
};

#define P2M_MAXMAPS 8

typedef struct p2m_config {
  int32_t nside;      /* HEALPix Nside (power of 2, <= 8192); 0 = no HEALPix map
                         (pks2map.f90:74, default 4096) */
  int32_t npix_fs;    /* flat-sky map side; 0 = no flat-sky map (pks2map.f90:77) */
  float fov_deg;      /* flat-sky field of view in degrees (pks2map.f90:78) */
  float zmin, zmax;   /* radial cut in redshift (pks2map.f90:73,79) */
  float chihview;     /* observer shift along x (pks2map.f90:80) */
  int32_t model;      /* profile model 1..3 (pks2map.f90:81) */
  int32_t precision;  /* P2M_PREC_* */
  int32_t nmaps;      /* maps painted per enumeration, 1..P2M_MAXMAPS */
  int32_t map_table[P2M_MAXMAPS];   /* table slot of each map */
  int32_t map_profile[P2M_MAXMAPS]; /* 1 = tSZ (weight 1), 2 = kSZ (weight -v_los/c)
                                       (pks2map.f90:82, pksc.f90:70-78) */
  int64_t max_records; /* largest record count of one paint call */
  int32_t device;      /* CUDA device ordinal */
  int32_t flags;       /* P2M_FLAG_* */
  int32_t ncones;      /* 0 or 1: one sky.  2..P2M_MAXCONES: an ensemble of independent
                          light-cones (p2m_paint_ensemble), each painted to its own copy
                          of the nmaps HEALPix maps; HEALPix only (npix_fs = 0).  No
                          counterpart in the reference, which paints one cone per run */
} p2m_config;

#define P2M_MAXCONES 4096

typedef struct p2m_stats {
  int64_t n_records;   /* records read */
  int64_t n_shell;     /* inside the radial cut (pks2map.f90:144-160) */
  int64_t n_painted;   /* passing the mass cut (pks2map.f90:296, "halos in map") */
  int64_t n_enumerated;/* halos whose discs were enumerated */
  int64_t hp_candidates; /* candidate HEALPix pixels tested */
  int64_t hp_updates;  /* (halo, pixel) pairs inside the disc */
  int64_t fs_updates;  /* flat-sky (halo, pixel) pairs inside the disc */
  int64_t n_recheck;   /* pixels decided by the exact FP64 recheck (mixed precision) */
  int64_t val_checked, val_bad_set, val_bad_index; /* P2M_FLAG_VALIDATE: candidates compared,
                          disc decisions and table indices that disagree with the exact path */
  float val_max_du;    /* largest |r-index coordinate fast - exact| seen (table cells) */
  double hp_sum[P2M_MAXMAPS]; /* sum over the HEALPix map of each map (total Y, kSZ) */
  double fs_sum[P2M_MAXMAPS];
} p2m_stats;

/* Create a painter on cfg->device; allocates device maps and work buffers. */
p2m_status p2m_create(const p2m_config *cfg, p2m_ctx **out);
void p2m_destroy(p2m_ctx *ctx);
/* Human-readable description of the last error on this context (never NULL). */
const char *p2m_last_error(const p2m_ctx *ctx);

/* Load a make_maptable table file image (36-byte header + float table(2,nrt,nmht,nchit))
   into slot 0..7.  All loaded tables must share one header. */
p2m_status p2m_load_table(p2m_ctx *ctx, int32_t slot, const void *image, int64_t nbytes);

/* Replace the r(z) and z(r) tables of cosmology.f90:51-105 (set_rofztable /
   set_zofrtable, called at pks2map.f90:131-132), which the context otherwise builds from
   the reference's hard-wired cosmology (pks2map.f90:118-128): rofz[i] = r at
   z = i * rofz_zmax / (n - 1) (Mpc), zofr[i] = z at r = i * zofr_rmax / (n - 1), both
   tables starting at 0, n = 10000 (the reference's table length); looked up as rofz/zofr
   do (cosmology.f90:137-181, linear, clamped at both ends).  They set the radial cut
   and each halo's redshift and table distance from the next paint call on.  The other
   cosmological parameters (omegam, h, rho_0: mass conversion, rhocrit, deltacrit) stay
   the reference's.  P2M_ERR_STATE while painted halos await a read-out (call it right
   after p2m_create or p2m_reset_maps). */
p2m_status p2m_set_cosmology_tables(p2m_ctx *ctx, const float *rofz, const float *zofr,
                                    int32_t n, float rofz_zmax, float zofr_rmax);

/* Zero the accumulated maps (the reference's `fsmapl=0; hpmapl=0`, pks2map.f90:278-279). */
p2m_status p2m_reset_maps(p2m_ctx *ctx);

/* Paint nrec catalogue records (nfloat = 7 or 10 floats each, header already removed)
   held in host memory: radial cut, mass, per-halo set-up and both projections, exactly
   the halo loop of pks2map.f90:134-303.  Accumulates into the context's maps.
   Where the reference aborts (query_disc on a disc radius above pi,
   pixel_routines.F90:1962, called at haloproject.f90:55) the call returns an error and
   paints none of the records of the failing ingest step (host records go in steps of
   p2m_tuning.stream_chunk; the steps before it stay painted); the context stays
   usable, and p2m_reset_maps starts over. */
p2m_status p2m_paint_records(p2m_ctx *ctx, const float *records, int64_t nrec, int32_t nfloat);
/* Page-locked host memory for catalogue records (no counterpart in the reference, whose
   loadpksc reads into an allocatable array): p2m_paint_records copies from it straight
   to the device, each step's copy overlapping the previous step's painting, where
   records in ordinary memory are first staged by the CUDA driver.  p2m_paint_records
   returns once its records are on the device, so the block can be refilled at once.
   *out = the block, or NULL and P2M_ERR_NOMEM; free it with p2m_host_free (NULL is a
   no-op). */
p2m_status p2m_host_alloc(int64_t bytes, void **out);
p2m_status p2m_host_free(void *p);
/* The pks2map command-line flags scramble and center (pks2map.f90:75-76, :162-262): 1
   gives every halo that survives the radial cut a random direction from the reference's
   ranf stream (seed 13579*(rank+1), two draws per halo in catalogue order), resp. flips
   and rotates all positions so that the largest-RTH halo lies on the z axis.  ntasks
   (1..25) is the MPI rank count whose halo blocks and streams are reproduced.  Call
   right after p2m_create or p2m_reset_maps; the whole catalogue must then come in one
   paint call. */
p2m_status p2m_set_preprocess(p2m_ctx *ctx, int32_t scramble, int32_t centre, int32_t ntasks);
/* Same with the records already in device memory (on ctx's device), ordered on the
   given cudaStream_t (NULL = the context's stream). */
p2m_status p2m_paint_records_device(p2m_ctx *ctx, const float *d_records, int64_t nrec,
                                    int32_t nfloat, void *stream);

/* Per-halo entry with the reference's by-reference arguments (bind(C) friendly):
   queues one halo whose loop quantities are already computed (pks2map.f90:284-298)
   for projecthalo_flatsky + projecthalo_healpix.  Queued halos are painted on the next
   read of a map or by p2m_flush.  x, y, z are divided by chi in place, as
   projecthalo_flatsky does to its caller's variables (haloproject.f90:97-99). */
/* Ensemble form (cfg.ncones > 1): ncones independent catalogues in one call, concatenated
   in records, cone c owning records [offsets[c], offsets[c+1]) (offsets[0] = 0,
   non-decreasing, ncones + 1 host values, ncones <= cfg.ncones).  Every cone goes through
   the halo loop of pks2map.f90:134-303 exactly as a p2m_paint_records call of its own
   would, into its own maps; all cones share one enumeration and one painting launch.
   With an ensemble, map m is ncones x 12 nside^2 floats, cone-major: p2m_get_healpix and
   the device read-outs move all cones, p2m_get_healpix_cone one.  Records painted by
   p2m_paint_records or p2m_project_halo go to cone 0. */
p2m_status p2m_paint_ensemble(p2m_ctx *ctx, const float *records, const int64_t *offsets,
                              int32_t ncones, int32_t nfloat);
p2m_status p2m_paint_ensemble_device(p2m_ctx *ctx, const float *d_records,
                                     const int64_t *offsets, int32_t ncones, int32_t nfloat,
                                     void *stream);
p2m_status p2m_get_healpix_cone(p2m_ctx *ctx, int32_t cone, int32_t map, float *out);

p2m_status p2m_project_halo(p2m_ctx *ctx, float *x, float *y, float *z, const float *r,
                            const float *chi, const float *m, const float *redshift,
                            const float *v, const int32_t *profile);
p2m_status p2m_flush(p2m_ctx *ctx);

/* Convert the accumulated map `map` to float and copy it out: host memory
   (12*nside^2 or npix_fs^2 floats, RING / column-major j-fastest order) ... */
p2m_status p2m_get_healpix(p2m_ctx *ctx, int32_t map, float *out);
p2m_status p2m_get_flatsky(p2m_ctx *ctx, int32_t map, float *out);
/* The same read-out into host memory, returning as soon as it is queued: the map is
   finished on the device and copied on a read-out stream of its own, beside whatever the
   caller does next; p2m_synchronize waits for the copies.  Pinned host memory makes the
   copy asynchronous.  Anything that would write the map's buffer before its copy is done
   (a clear after p2m_reset_maps, more painting, another read-out) waits for the copy, so
   a caller who paints the next catalogue while the maps are copied binds other buffers
   (p2m_bind_healpix_device) to the maps first.  No counterpart in the reference, which
   reads each map once at the end of its run. */
p2m_status p2m_get_healpix_async(p2m_ctx *ctx, int32_t map, float *out);
/* ... or device memory, ordered on `stream` (NULL = the context's stream).  This one
   does not wait for the device: an error the painting kernels raise is reported by the
   next call that does (the next paint call, a host read-out, p2m_get_stats or
   p2m_synchronize). */
p2m_status p2m_get_healpix_device(p2m_ctx *ctx, int32_t map, float *d_out, void *stream);
/* Make a caller-owned device buffer of 12*nside^2 floats (times ncones for an ensemble)
   the storage of HEALPix map `map`
   (the reference's hpmap allocation, pks2map.f90:113): read-outs then write it in place
   and p2m_get_healpix_device with the same pointer copies nothing.  Call right after
   p2m_create or p2m_reset_maps; NULL restores the context's own buffer. */
p2m_status p2m_bind_healpix_device(p2m_ctx *ctx, int32_t map, float *d_out);

/* Statistics of one map as a read-out delivers it (pks2map.f90:321-334): the moments
   sum(map**k) / npix, k = 1..3, and the RMS sqrt(sum((map - mom[0])**2) / npix).  The
   sums are formed on the device in float-float per thread and FP64 across threads (the
   reference's `sum` of a real array accumulates in float, in an order the compiler
   chooses; these are within its rounding of that).  No counterpart as a call in the
   reference, whose main program runs these loops over the gathered maps. */
typedef struct p2m_map_stats {
  int64_t npix;   /* pixels of the map */
  double mom[3];  /* hpmom1..3 / fsmom1..3 */
  double rms;     /* Healpix / Flatsky RMS */
} p2m_map_stats;
/* HEALPix map `map` (not an ensemble's); with dpdy non-null also the cumulative P(<y) of
   pks2map.f90:340-357 into dpdy[0..10000): bin m = int(y / 1e-8) + 1 counted in float (a
   bin stops at 2^24, as the reference's real counter does), divided by the pixel count,
   then cumulated. */
p2m_status p2m_get_healpix_stats(p2m_ctx *ctx, int32_t map, p2m_map_stats *out, float *dpdy);
p2m_status p2m_get_flatsky_stats(p2m_ctx *ctx, int32_t map, p2m_map_stats *out);

/* Write HEALPix map `map` (not an ensemble's) to the FITS file `path` as the reference's
   output_map does (pks2map.f90:381-385; an empty primary HDU, then a BINTABLE of
   1024-value float rows, NSIDE and ORDERING = 'RING' cards; see p2m_write_healpix_fits
   in p2m_tools.h for the layout): the map is converted to big-endian words on the device
   and copied out in 64 MB slices, each slice's copy overlapping the file write of the
   one before.  No host copy of the map is needed.  P2M_ERR_IO if the file cannot be
   written. */
p2m_status p2m_write_healpix_fits_device(p2m_ctx *ctx, int32_t map, const char *path);

/* Counters and map sums of everything painted since the last reset. */
p2m_status p2m_get_stats(p2m_ctx *ctx, p2m_stats *out);
/* Wait for all work queued on the context's stream. */
p2m_status p2m_synchronize(p2m_ctx *ctx);

/* (record index, RING pixel) pairs of the HEALPix deposits of the last paint call;
   requires P2M_FLAG_RECORD_SETS.  *n receives the total (may exceed cap). */
p2m_status p2m_get_pixel_sets(p2m_ctx *ctx, int64_t *rec, int64_t *pix, int64_t cap, int64_t *n);

/* Build a make_maptable table image on the GPU (maptable.f90:25-146).  Returns the
   image size in *nbytes; image may be NULL to query the size.  Sizes <= 0 take the
   reference's 100 x 100 x 200. */
p2m_status p2m_make_maptable(int32_t device, int32_t model, float nu, float alpha_cmb,
                             int32_t nchit, int32_t nmht, int32_t nrt, void *image,
                             int64_t *nbytes);

#ifdef __cplusplus
}
#endif
#endif /* P2M_H */
