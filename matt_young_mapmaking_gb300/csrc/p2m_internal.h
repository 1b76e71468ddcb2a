/*
 * p2m_internal.h -- device data layout and kernel launchers of the halo painter.
 *
 * Pipeline for one batch of catalogue records (all on one stream, no host round trip
 * inside the paint except the two capacity checks in p2m_capi.cu):
 *   k_cut      records -> indices of halos inside the shell with mass >= mmin
 *   k_setup    per halo: the loop quantities of pks2map.f90:284-298, disc radius,
 *              centre, interpolation constants, candidate ring range, flat-sky box;
 *              histogram of (halo, ring) items per ring
 *   scan       ring histogram -> ring offsets
 *   k_emit     (halo, ring) items placed in ring order; flat-sky (halo, row) items
 *   k_rings    per item: candidate pixel span of the ring (FP32 superset of the disc)
 *              and the ring constants of the disc test
 *   scan       candidate counts -> candidate offsets
 *   k_paint    per candidate pixel: disc test, profile value, deposit
 *   k_recheck  (mixed precision) exact FP64 decision for pixels near a boundary
 *   k_paint_fs flat-sky rows
 *   k_finalize accumulators -> float maps and map sums
 */
#ifndef P2M_INTERNAL_H
#define P2M_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "p2m_scalar.h"

struct DevCounters {
  unsigned long long n_records, n_shell, n_surv, n_halo, n_items, n_pix;
  unsigned long long n_fb, n_fs_items, hp_updates, fs_updates, n_sets, n_recheck;
  unsigned long long n_candidates, n_fs_rows;
  unsigned int err;
  unsigned int pad;
};

enum { P2M_DEVERR_FB_OVERFLOW = 1, P2M_DEVERR_FS_OVERFLOW = 2, P2M_DEVERR_RADIUS = 4,
       P2M_DEVERR_ITEMS = 8 };

/* one halo inside the cut, as the painter needs it */
struct HaloRec {
  double z0, sth0, phi0f; /* unit disc centre: z, sin(theta), phi / 2pi */
  float hv[3];            /* hpvec1 of haloproject.f90:51-53 (float values) */
  float T;                /* dtheta_halo (float value), haloproject.f90:47 */
  float C_in, C_out, C_span; /* chord^2 thresholds: certainly inside / outside / span */
  float chi_t, fc, fm;    /* per-halo part of interpolate_table */
  int ichi, imh, zero;
  float w1, w2;           /* deposit weights of profile-1 and profile-2 maps */
  int rec;                /* record index */
  int ir_lo, ir_hi;       /* candidate rings */
  int cbase[4];           /* table offsets of corners (imh,ichi),(imh+1,ichi),(imh,ichi+1),
                             (imh+1,ichi+1) at ir=1, profile 1; -1: use clamped offsets */
  float theta_h, phi_h;   /* flat-sky centre (float values), haloproject.f90:105-106 */
  int jmin, jmax, kmin, kmax; /* flat-sky box; jmin > jmax: none */
};

/* candidate span of one ring of one disc */
struct RingItem {
  int halo, ring, lo, count; /* lo: unwrapped phi index of the first candidate */
  float A, B;                /* chord^2 = A + B sin^2(dphi/2) */
  float x0;                  /* (lo + kshift/2) - phi0 npr / 2pi, in pixel units */
  float hdphi;               /* pi / npr */
};

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
  const float *tables[P2M_MAXTABLES];
  const float *rofz, *zofr;
  const double2 *ringtab; /* (z, sin theta) of rings 1..4N-1 at index ring */
};

struct PaintBuffers {
  const float *records;
  int *surv;
  HaloRec *halos;
  unsigned int *ring_hist, *ring_cursor;
  long long *ring_start;
  RingItem *items;
  unsigned int *counts;
  long long *pix_off;
  unsigned long long *fb; /* (item << 32 | k) */
  long long fb_cap;
  FsItem *fs_items;
  long long fs_cap;
  void *hp_acc; /* nmaps per pixel: double, or float2 (hi, lo) */
  void *fs_acc;
  long long *set_rec, *set_pix;
  long long set_cap;
  long long *scan_tmp; /* block sums */
  DevCounters *ctr;
};

/* launchers (p2m_kernels.cu) */
void p2m_launch_cut(const PaintParams &P, const PaintBuffers &B, long long n, cudaStream_t s,
                    int nsm);
void p2m_launch_setup(const PaintParams &P, const PaintBuffers &B, long long n_max,
                      cudaStream_t s, int nsm);
void p2m_launch_ring_scan(const PaintParams &P, const PaintBuffers &B, cudaStream_t s);
void p2m_launch_emit(const PaintParams &P, const PaintBuffers &B, long long n_max,
                     cudaStream_t s, int nsm);
void p2m_launch_rings(const PaintParams &P, const PaintBuffers &B, long long n_max,
                      cudaStream_t s, int nsm);
void p2m_launch_count_scan(const PaintParams &P, const PaintBuffers &B, cudaStream_t s);
void p2m_launch_paint(const PaintParams &P, const PaintBuffers &B, cudaStream_t s, int nsm);
void p2m_launch_recheck(const PaintParams &P, const PaintBuffers &B, cudaStream_t s, int nsm);
void p2m_launch_paint_fs(const PaintParams &P, const PaintBuffers &B, cudaStream_t s, int nsm);
void p2m_launch_finalize(const PaintParams &P, const void *acc, long long npix, int map,
                         float *out, double *sum, cudaStream_t s, int nsm);
void p2m_launch_prepared(const PaintParams &P, const PaintBuffers &B, const float *d_prep,
                         long long n, cudaStream_t s, int nsm);
struct TableConsts {
  float y0, tau0, x0const, nu, alpha;
  int model;
};
void p2m_launch_maptable(const PaintParams &P, const TableConsts &K, const p2m_tabhdr &th,
                         float *d_table, cudaStream_t s);

#endif
