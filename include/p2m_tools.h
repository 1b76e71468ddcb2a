/*
 * p2m_tools.h -- host-side tools that travel with the painter.  They have no
 * counterpart in the reference, whose input catalogues come from its halo finder
 * (hpkvd / merge_pkvd, out of scope here): they build the synthetic catalogues used
 * for tests and benchmarks.
 */
#ifndef P2M_TOOLS_H
#define P2M_TOOLS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Synthetic halo catalogue, deterministic in (seed, record index): Philox4x32-10
   with the record index as counter.  Positions uniform in volume in the shell
   [r_min, r_max] Mpc with isotropic directions; masses from dN/dlnM ~ M^slope on
   [m_min, m_max] Msun by inverse CDF; RTH = (3M / (4 pi Om 2.775e11 h^2))^(1/3) with
   Om = 0.31, h = 0.68; velocities N(0, sigma_v) km/s per axis; Lagrangian position
   x - 0.01 v.  Writes n records of nfloat (7: x,y,z,vx,vy,vz,RTH; 10: + xL,yL,zL)
   starting at record index first.  Returns 0, or 1 on bad arguments. */
int32_t p2m_generate_catalogue(uint64_t seed, int64_t first, int64_t n, int32_t nfloat,
                               double r_min, double r_max, double m_min, double m_max,
                               double slope, double sigma_v, float *out);

/* Philox4x32-10 block for (counter c[4], key k[2]) -> out[4]. */
void p2m_philox4x32(const uint32_t c[4], const uint32_t k[2], uint32_t out[4]);

/* Device time (ms) of each phase of the last paint call and of the last map read-out,
   for a context created with P2M_FLAG_TIMING: [0] cut with the per-halo set-up of
   catalogue records (one kernel), [1] set-up of p2m_project_halo batches, [2] unused
   (0: the large halos reserve their item ranges during the set-up), [3] their ring spans, [4] flat sky, [5] their candidate
   offsets, [6] HEALPix paint (both painting kernels, which run concurrently), [7] the
   large halos' painting kernel alone, [8] read-out.  Diagnostics only (the reference prints no
   timings). */
struct p2m_ctx;
int32_t p2m_get_timings(struct p2m_ctx *ctx, double *ms, int32_t n);

/* Sums (FP64 totals of float-float partial sums) of nmaps float maps of npix pixels each,
   already in device memory on the current device, written to host sums[0..nmaps).
   No counterpart in the reference (its map sums are module-array loops on the host).
   Allocates nothing: the scratch is a file-scope device array of P2M_NOALLOC_MAXMAPS
   doubles per device, cleared by the call itself on `stream` (NULL = the legacy default
   stream) before use.  For callers that may not allocate device memory (a host
   framework whose caching allocator owns the device, or a loop that cannot afford the
   device-wide synchronisation of cudaFree).  The first call on a device looks up the
   scratch address and may load the module: make it before any stream capture.  That
   address is cached per device and is not valid across a cudaDeviceReset: do not call
   this function after the device has been reset in the same process.  Calls on one
   device share the scratch, so overlapping calls race and must be serialised by the
   caller.  Synchronous: a stream under capture is refused with P2M_ERR_STATE, nothing
   queued.  nmaps > P2M_NOALLOC_MAXMAPS: P2M_ERR_CAPACITY. */
#define P2M_NOALLOC_MAXMAPS 8
int32_t p2m_map_sums_noalloc(const float *const *d_maps, int32_t nmaps, int64_t npix,
                             double *sums, void *stream);

/* Launch parameters of the sweep, chosen by p2m_autotune or set directly.  No counterpart
   in the reference, whose halo loop has no launch parameters.  The defaults are the first
   row of each field's range below; results do not depend on them (pixel sets are
   identical, map values equal up to the order of the additions). */
typedef struct p2m_tuning {
  int32_t big_rings;  /* halos spanning more rings are painted from stored (halo, ring) items
                         by the candidate-balanced kernel (0: every halo), 0..4096; 64 */
  int32_t halos_grid; /* 128-thread blocks per SM of the fused enumerate-and-paint kernel
                         (8 fit at once), 1..16; 8 */
  int32_t full_grid;  /* blocks per SM of the stored-item kernel, 1..32; 8 */
  int32_t full_chunk; /* candidates per warp chunk of the stored-item kernel, 32..65536; 1024 */
  int32_t stream_chunk; /* host records per chunk of the streamed ingest of p2m_paint_records
                           (copy of chunk k+1 overlapped with chunk k), 65536..2^26; 2^22 */
  int32_t stream_paint; /* 1: whenever a full chunk's worth of records (this call's or
                           earlier calls') awaits painting, paint it before the next chunk is
                           ingested, so that the copies overlap the painting too; 0: paint
                           at the read-out; 1 */
  int32_t halo_batch; /* halos per warp batch of the fused kernel, 1..32; 16 */
  int32_t sort_halos; /* 1: paint the halos in order of their first ring (a counting sort:
                         the set-up counts the keys, the paint scans and scatters them), so
                         that the halos in flight cover a narrow band of the maps; 0: in
                         catalogue order; 1 */
  int32_t halos_threads; /* threads per block of the fused kernel, 128 or 256 (halos_grid
                            blocks of them per SM); 128 */
  /* No table-tile field: the profile tables are read through the read-only cache
     (__ldg), not staged in shared-memory tiles.  A table is 16 MB at the reference's
     100 x 100 x 200 size and stays in L2; its loads hit L1/L2, and shared memory holds
     the fused kernel's per-warp stage instead. */
  float ms;           /* p2m_autotune: device time of one paint call with the choice */
} p2m_tuning;
int32_t p2m_get_tuning(struct p2m_ctx *ctx, p2m_tuning *out);
int32_t p2m_set_tuning(struct p2m_ctx *ctx, const p2m_tuning *t);
/* Autotuner: paints the caller's catalogue (device records, as p2m_paint_records_device)
   with candidate launch parameters and keeps the fastest.  The search is coordinate
   descent: big_rings, then the fused kernel's block size and grid, then the stored-item
   kernel's grid, then its chunk, then the painting order, then the fused kernel's
   batch.  Each candidate is timed by device events around the whole paint call
   (reset, ingest, sweep), best of `reps`.  The maps are reset before the first and after
   the last candidate.  Writes the choice to *out when out is not NULL. */
int32_t p2m_autotune(struct p2m_ctx *ctx, const float *d_records, int64_t nrec, int32_t nfloat,
                     int32_t reps, p2m_tuning *out);

/* With center: RTHmax, then the distance and x, y, z of the largest halo before and after
   the rotation (the report of pks2map.f90:205-209, :250-254); zeros otherwise. */
int32_t p2m_get_centre(struct p2m_ctx *ctx, float *out9);

/* Output files of the pks2map command line (host code, no GPU).  Each returns 0 or a
   status (P2M_ERR_BADARG, P2M_ERR_IO). */
#define P2M_NDPDY 10000
/* P(<y) of a HEALPix map, pks2map.f90:340-357: pixel counts in P2M_NDPDY bins of width
   1e-4 / P2M_NDPDY (bin int(y / width) + 1, counted in float as the reference counts, so
   a bin stops at 2^24), divided by npix and cumulated. */
int32_t p2m_dpdy(const float *map, int64_t npix, float *dpdy);
/* <out>_dp.bin: int32 P2M_NDPDY, float32 1e-4, float32 dpdy[P2M_NDPDY] (pks2map.f90:370-373) */
int32_t p2m_write_dpdy(const char *path, const float *dpdy);
/* <out>_fs.map: int32 npix, npix, float32 fov, fov (radians), float32 map[npix*npix]
   (pks2map.f90:375-379) */
int32_t p2m_write_flatsky(const char *path, const float *map, int32_t npix, float fov_rad);
/* <out>_hp.fits: empty primary HDU + BINTABLE, one column of 1024-float rows in RING
   order, NSIDE and ORDERING = 'RING' cards (pks2map.f90:381-385, HEALPix output_map) */
int32_t p2m_write_healpix_fits(const char *path, const float *map, int32_t nside);

/* Angular power spectra of painted maps, for the precision report (validation only;
   host maps in, spectra out, synchronous, device memory allocated for the call).

   p2m_cl_healpix: the spectra of RING-ordered HEALPix maps up to lmax (<= 4 nside and
   <= P2M_CL_LMAX_MAX), by the pixel-area quadrature of the HEALPix library that the
   reference vendors: map2alm without iterations and with unit ring weights
   (src/modules/External/alm_map_dd_inc.F90:2978-3224, ring_analysis and the lambda_lm
   recursion of alm_tools.F90:394-650, 1022-1097), then alm2cl (alm_map_dd_inc.F90:5347-5423).
   cl_aa[l], and with map_b, cl_ab[l] = sum_m Re a_lm conj(b_lm) / (2l+1) and cl_bb[l],
   for l = 0 .. lmax.  map_b may be NULL (cl_ab and cl_bb are then not written).

   p2m_cl_flatsky: binned periodogram of npix x npix flat-sky maps over fov_rad x fov_rad
   (the layout of p2m_get_flatsky): nbins (<= P2M_CL_MAXBINS) linear bins of ell = 2 pi |k| / fov in
   (0, ell_max], C = (fov^2 / npix^4) |FFT(map)(k)|^2 averaged over each bin's modes;
   ell_mean is the bins' mean ell and nmodes their mode counts.  The mode k = 0 and the
   Nyquist line are left out.  npix is a power of two up to 8192, or any size up to
   2048.  The reference computes no flat-sky spectrum; this one stands beside the
   HEALPix one for the 8192^2 map. */
#define P2M_CL_LMAX_MAX 16384
#define P2M_CL_MAXBINS 1024
int32_t p2m_cl_healpix(int32_t device, const float *map_a, const float *map_b, int32_t nside,
                       int32_t lmax, double *cl_aa, double *cl_ab, double *cl_bb);
int32_t p2m_cl_flatsky(int32_t device, const float *map_a, const float *map_b, int32_t npix,
                       float fov_rad, double ell_max, int32_t nbins, double *ell_mean,
                       double *cl_aa, double *cl_ab, double *cl_bb, int64_t *nmodes);

/* Self-test of the single-precision math the kernels use (fn: 0 log, 1 exp, 2 pow,
   3 asin, 4 atan, 5 sin, 6 cos, 7 tan; 8 the fixed-point sum of P2M_PREC_FIXED:
   x and y each rounded to a multiple of 2^-56, added as integers and rounded back to
   float) evaluated on the GPU over n device floats; d_y is read only for pow and 8.
   Synchronous.  Returns 0 or a CUDA error code. */
int32_t p2m_fmath_eval_device(int32_t device, int32_t fn, const float *d_x, const float *d_y,
                              float *d_out, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
