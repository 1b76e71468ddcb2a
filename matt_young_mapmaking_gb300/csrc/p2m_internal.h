/*
 * p2m_internal.h -- device data layout and kernel launchers of the halo painter.
 *
 * A paint call ingests catalogue records; the HEALPix maps are produced by a sweep when
 * they are read.  Ingest (one stream, one host round trip to size the item buffer):
 *   k_cut_setup  records -> halos inside the radial cut with mass >= mmin whose table
 *              value is not identically zero, queued in shared memory, and per queued
 *              halo the loop quantities of pks2map.f90:284-298, disc radius and centre,
 *              interpolation constants, candidate ring range, flat-sky box
 *   scan       rings of the large halos (more than big_rings rings) -> item offsets
 *   k_items    per (large halo, ring) item: FP32 superset of the ring's pixel span and
 *              the ring constants of the disc test
 *   k_paint_fs flat-sky rows (exact float sequence of the reference)
 * Sweep:
 *   k_paint_halos  the other halos, enumeration fused with painting: a warp builds the
 *              ring spans of a batch of halos in registers and paints their candidates
 *   scan + k_paint_full  the large halos' items, load-balanced over candidate pixels
 *   read-out   mixed precision: the maps hold the high words of a compensated sum and
 *              k_fold_lo adds the sparse low words; FP64 accumulation: k_finalize_full
 */
#ifndef P2M_INTERNAL_H
#define P2M_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "p2m_scalar.h"

#define P2M_STREAM_CHUNK (1LL << 22) /* host records per streamed ingest chunk */
#define P2M_BIG_RINGS 64      /* default: halos spanning more rings go through the item buffer */
#define P2M_TILE_SHIFT 5      /* compensated path: a flagged tile is 32 pixels (128 bytes) */
#define P2M_TILE_PIX (1 << P2M_TILE_SHIFT)
#define P2M_PHITAB 4096       /* grid angles 2 pi k / P2M_PHITAB of the disc-centre phi reduction */

struct DevCounters {
  /* per call (cleared before every ingest call and every paint) */
  unsigned long long n_surv, n_items, n_pix, n_fs_items, n_fs_rows;
  unsigned int next_unit, pad0;
  /* cumulative since the last reset */
  unsigned long long hp_updates, fs_updates, n_sets, n_recheck, n_shell, n_massive, n_enum,
      n_cand;
  unsigned long long val_checked, val_bad_set, val_bad_index;
  unsigned int val_max_du; /* float bits of the largest |u_fast - u_exact| */
  unsigned int err;        /* P2M_DEVERR_* raised since it was last reported */
};

enum {
  P2M_DEVERR_FS_OVERFLOW = 2,
  P2M_DEVERR_RADIUS = 4,
  P2M_DEVERR_ITEMS = 8,
  P2M_DEVERR_FIXED = 16 /* fixed-point accumulation: a value or a pixel sum out of range */
};

/* one enumerated halo */
struct HaloRec {
  float z0h, z0l, s0h, s0l, p0h, p0l; /* unit disc centre: z, sin(theta), phi / 2pi as
                                         (hi, lo) float pairs, hi + lo = the FP64 value */
  float hv[3];            /* hpvec1 of haloproject.f90:51-53 (float values) */
  float T;                /* dtheta_halo (float value), haloproject.f90:47 */
  float C_in, C_out, C_span; /* chord^2 thresholds: certainly inside / outside / span */
  float chi_t, fc, fm;    /* per-halo part of interpolate_table */
  int ichi, imh, zero;
  float w1, w2;           /* deposit weights of profile-1 and profile-2 maps */
  int cone;               /* light-cone of an ensemble: the maps' slot offset is
                             cone * 12 nside^2 (0 outside ensembles) */
  long long rec;          /* record index (over all paint calls since the reset) */
  int ir_lo, ir_hi;       /* candidate rings */
  int cbase[4];           /* table offsets of corners (imh,ichi),(imh+1,ichi),(imh,ichi+1),
                             (imh+1,ichi+1) at ir=1, profile 1; -1: clamped offsets */
  float theta_h, phi_h;   /* flat-sky centre (float values), haloproject.f90:105-106 */
  int jmin, jmax, kmin, kmax; /* flat-sky box; jmin > jmax: none */
};

/* candidate span of one ring of one disc */
static_assert(sizeof(HaloRec) == 144, "HaloRec layout");

struct RingItem {
  int halo;
  int ring_n0;               /* ring << 16 | (n0 & 0xffff) */
  int lo, count;             /* lo: unwrapped phi index of the first candidate */
  float A, B;                /* chord^2 = A + B sin^2(dphi/2) */
  float f0;                  /* x0 = (lo + kshift/2) - phi0 npr / 2pi = n0 + f0 (pixel units):
                                the k-th candidate sits at x = (n0 + k) + f0, exact integer
                                part, so x keeps full relative precision near the centre */
  float hdphi;               /* pi / npr */
  float Al, Bl, f0l, hdl;    /* low words: (A, Al), (B, Bl), (f0, f0l), (hdphi, hdl) are
                                float-float values (~44 bits) for the pixel's angle */
};
static_assert(sizeof(RingItem) == 48, "RingItem layout");

__host__ __device__ __forceinline__ int item_ring(const RingItem &it) { return it.ring_n0 >> 16; }
__host__ __device__ __forceinline__ int item_n0(const RingItem &it) {
  return (int)(short)(it.ring_n0 & 0xffff);
}

struct FsItem {
  int halo, k, jmin, count;
};

struct PaintParams {
  int nside, npix_fs, nmaps, precision, flags, nfloat, model;
  float fov, dpix, hf, cut_low, cut_high, chihview, bbps_delta;
  int map_table[P2M_MAXMAPS], map_profile[P2M_MAXMAPS];
  int any_ksz;
  float mass_fac; /* (4./3.*mypi)*rho_0 of pks2map.f90:264 */
  p2m_cosmo cosmo;
  p2m_tabhdr th;
  int ir_c;     /* r-index and fraction for r < rmint (r = rmint + 1e-5) */
  float fr_c;
  float band_u;  /* half-width of the r-index recheck band (cell units) */
  float inv_drt; /* 1 / drt of the table */
  int big_rings; /* halos spanning more rings are painted from stored items */
  const float *tables[P2M_MAXTABLES];
  /* maps 2q and 2q + 1 as one table of float2 entries (.x map 2q, .y map 2q + 1) at the
     tables' float2 index cb / 2 + ir - 1: the table itself where the pair is profiles 1
     and 2 of one table (or a lone last map of profile 1), else a gathered copy */
  const float2 *pair_tab[P2M_MAXMAPS / 2];
  const float *rofz, *zofr;
  const float4 *ringtab; /* (z hi, z lo, sin theta hi, sin theta lo) of ring i at index i */
  const float2 *ringhd;  /* pi / npr of ring i as (hi, lo) */
  const float4 *phitab;  /* (cos hi, cos lo, sin hi, sin lo) of 2 pi k / P2M_PHITAB */
  p2m_pre pre;           /* scramble / centre of the catalogue (pks2map.f90:162-262) */
  const long long *pre_ord; /* with pre: radial-cut survivors before each record */
  long long cone_npix;   /* HEALPix pixels of one cone's map (12 nside^2) */
  int halos_grid;        /* blocks per SM of k_paint_halos */
  int full_grid;         /* blocks per SM of k_paint_full */
  int full_chunk;        /* candidates per warp chunk of k_paint_full */
  int halo_batch;        /* halos per warp batch of k_paint_halos (1..32) */
  int halos_threads;     /* threads per block of k_paint_halos (128 or 256) */
  unsigned int *err_flag; /* the device error word (DevCounters::err) */
};

/* buffers of one ingest call */
struct IngestBuffers {
  const float *records;
  long long rec_base;   /* record index of records[0] */
  const long long *cone_off; /* ensemble: first record of each cone (call-local), ncones + 1 */
  int ncones;           /* 0: every record belongs to cone 0 */
  int *ring_key;        /* painting order by first ring: each halo's key (call-local) ... */
  unsigned int *ring_hist; /* ... and the keys' counts, or null when the order is not kept */
  HaloRec *halos;       /* halos[0..n_surv) of this call */
  long long halo_base;  /* global index of halos[0] */
  unsigned int *nring;  /* rings per large halo, 0 for the others */
  long long *ioff;      /* item offset per halo (call-local) */
  RingItem *items;      /* items of this call */
  FsItem *fs_items;
  long long fs_cap;
  void *fs_acc;
  long long *scan_tmp;
  DevCounters *ctr;
  long long *set_rec, *set_pix;
  long long set_cap;
};

/* buffers of one sweep */
struct SweepBuffers {
  const HaloRec *halos;
  long long n_halos;
  const RingItem *items;       /* items of the large halos */
  const long long *pix_off;    /* candidate offset of each item */
  long long n_items;
  float *out[P2M_MAXMAPS];     /* float output maps */
  void *acc;                   /* full-sky FP64 accumulator (FP64-accumulating paths) */
  float *lo;                   /* compensated path: low words, map m at lo + m * npix */
  unsigned char *tiles;        /* compensated path: 1 per tile with a nonzero low word */
  long long npix;
  DevCounters *ctr;
  long long *set_rec, *set_pix;
  long long set_cap;
  const int *order;            /* halos in painting order (sorted by first ring), or null */
};

/* launchers (p2m_kernels.cu) */
void p2m_launch_cut_setup(const PaintParams &P, const IngestBuffers &B, long long n,
                          cudaStream_t s, int nsm);
void p2m_launch_pre_flags(const PaintParams &P, const float *records, long long n,
                          unsigned int *flags, cudaStream_t s, int nsm);
void p2m_launch_pre_centre(const PaintParams &P, const float *records, long long n,
                           const unsigned int *flags, unsigned int *rthmax_bits,
                           long long *last, cudaStream_t s, int nsm);
void p2m_launch_setup_prepared(const PaintParams &P, const IngestBuffers &B, const float *prep,
                               long long n, cudaStream_t s, int nsm);
void p2m_launch_scan_u32(const unsigned int *in, const unsigned long long *n_ptr, long long *out,
                         unsigned long long *total, long long *tmp, cudaStream_t s);
void p2m_launch_items(const PaintParams &P, const IngestBuffers &B, long long n_max,
                      cudaStream_t s, int nsm);
void p2m_launch_fs(const PaintParams &P, const IngestBuffers &B, long long n_max, cudaStream_t s,
                   int nsm);
void p2m_launch_pair_table(float2 *dst, const float *ta, int pa, const float *tb, int pb,
                           long long nent, cudaStream_t s, int nsm);
void p2m_launch_item_counts(const RingItem *items, long long n, unsigned int *counts,
                            cudaStream_t s, int nsm);
void p2m_launch_paint_halos(const PaintParams &P, const SweepBuffers &W, cudaStream_t s, int nsm);
void p2m_launch_paint_full(const PaintParams &P, const SweepBuffers &W, cudaStream_t s, int nsm);
void p2m_launch_finalize_full(const PaintParams &P, const void *acc, long long npix,
                              float *const *out, int accumulate, cudaStream_t s, int nsm);
void p2m_launch_finalize_fs(const PaintParams &P, const void *acc, long long npix, float *out,
                            int map, double *sum, cudaStream_t s, int nsm);
void p2m_launch_fold_lo(const PaintParams &P, const SweepBuffers &W, cudaStream_t s, int nsm);
void p2m_launch_map_sum(const float *map, long long n, double *sum, cudaStream_t s, int nsm);
/* out[i] = the big-endian bytes of in[i] (FITS data order) */
void p2m_launch_to_big_endian(const float *in, unsigned int *out, long long n, cudaStream_t s,
                              int nsm);
/* sums[0..3) += sums of x, x^2, x^3 over the map; hist (nbins <= 12288 counters, or null)
   += the P(<y) bin counts of bin width dy */
void p2m_launch_map_stats(const float *map, long long n, double *sums, unsigned int *hist,
                          int nbins, float dy, cudaStream_t s, int nsm);
/* copies the counters into mapped host memory with the SMs' stores: no copy engine, so a
   counter read never queues behind a large read-out copy */
void p2m_launch_copy_counters(const DevCounters *d, DevCounters *h_mapped, cudaStream_t s);
/* counting sort of halos [0, n) by first ring into order[]: the set-up stored each halo's
   key and counted it; off holds the bins' first positions (the scan of the counts) and is
   consumed */
void p2m_launch_ring_scatter(const int *keys, long long n, long long *off, int *order,
                             cudaStream_t s, int nsm);
/* takes halos [0, n) of a discarded ingest back out of the first-ring counts */
void p2m_launch_ring_unhist(const int *keys, long long n, unsigned int *hist, cudaStream_t s,
                            int nsm);
struct TableConsts {
  float y0, tau0, x0const, nu, alpha;
  int model;
};
void p2m_launch_maptable(const PaintParams &P, const TableConsts &K, const p2m_tabhdr &th,
                         float *d_table, cudaStream_t s);

#endif
