/*
 * p2m_kernels.cu -- sm_103a kernels of the halo painter (pipeline in p2m_internal.h).
 *
 * The bulk of the halos is enumerated and painted by one fused kernel: a warp builds
 * the (halo, ring) candidate spans of a batch of halos (up to 32, in order of their
 * first ring) in registers and paints their candidate pixels 32 at a time, so no
 * per-item data goes through memory.  Halos spanning many
 * rings are load-balanced at the level of candidate pixels instead: their spans are
 * stored and prefix-summed, and each warp walks a contiguous range of the candidate
 * space.  Mixed precision accumulates into the float maps with the exact rounding
 * error of every add kept apart (compensated summation).
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>

#include "../../include/p2m_tools.h"
#include "p2m_internal.h"

#define FULL 0xffffffffu

/* ------------------------------------------------------------------ helpers ----- */

__device__ __forceinline__ void warp_count(unsigned long long *ctr, unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(ctr, v);
}

/* block-wide sum of v added to *ctr by one thread (blockDim.x <= 1024, all threads call) */
__device__ void block_count(unsigned long long *ctr, unsigned long long v) {
  __shared__ unsigned long long red[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    if (t) atomicAdd(ctr, t);
  }
}

/* *ctr += v over the warp's active lanes with one atomic; returns this lane's place
   (the old value plus the v of the active lanes below it) */
__device__ __forceinline__ unsigned long long warp_reserve(unsigned long long *ctr,
                                                           unsigned long long v) {
  const unsigned mask = __activemask();
  const int lane = threadIdx.x & 31;
  unsigned long long below = 0, tot = 0;
  for (unsigned m = mask; m;) {
    const int src = __ffs(m) - 1;
    m &= m - 1;
    const unsigned long long x = __shfl_sync(mask, v, src);
    if (src < lane) below += x;
    tot += x;
  }
  const int leader = __ffs(mask) - 1;
  unsigned long long base = 0;
  if (lane == leader && tot) base = atomicAdd(ctr, tot);
  return __shfl_sync(mask, base, leader) + below;
}

__device__ __forceinline__ bool p2m_isfinite(float x) { return fabsf(x) <= 3.4028234e38f; }

/* chord^2 of an angle a (radians): 4 sin^2(a/2); a >= pi covers the sphere */
__device__ __forceinline__ float chord2(float a) {
  if (a >= 3.14159f) return 4.5f;
  float s = sinf(0.5f * a);
  return 4.0f * s * s;
}

__device__ __forceinline__ p2m_hinterp halo_hinterp(const HaloRec &H) {
  p2m_hinterp hi;
  hi.chi_t = H.chi_t;
  hi.fc = H.fc;
  hi.fm = H.fm;
  hi.ichi = H.ichi;
  hi.imh = H.imh;
  hi.zero = H.zero;
  return hi;
}


/* ---------------------------------------------------------------- ingest: cut ----- */

#define CUT_PER_THREAD 8

/* radial cut (pks2map.f90:144-160), mass cut (:264, :296), and the table's chi bound
   (maptable.f90:184,188: chi = rofz(zofr(chi)) > chimaxt paints zeros) of one record;
   true if the record is enumerated */
/* radial cut of pks2map.f90:144-160 on a record as read */
__device__ __forceinline__ bool in_shell(const PaintParams &P, const float *r) {
  float p0 = __ldg(r + 0), p1 = __ldg(r + 1), p2 = __ldg(r + 2), rth = __ldg(r + 6);
  if (!(p2m_isfinite(p0) && p2m_isfinite(p1) && p2m_isfinite(p2) && p2m_isfinite(rth)))
    return false;
  float xh = FSUB(p2, P.chihview), yh = p1, zh = p0;
  float chih = FSQRT(FADD(FADD(FMUL(xh, xh), FMUL(yh, yh)), FMUL(zh, zh)));
  return !(chih > P.cut_high || chih < P.cut_low);
}

/* posxyz(1..3) of record i as the halo loop sees it: as read, or scrambled in its
   rank's stream and / or rotated (pks2map.f90:162-262) */
__device__ __forceinline__ void halo_position(const PaintParams &P, const float *records, long long i,
                                              float pos[3]) {
  const float *r = records + i * P.nfloat;
  pos[0] = r[0];
  pos[1] = r[1];
  pos[2] = r[2];
  if (P.pre.scramble) {
    const long long rank = i / P.pre.per_rank;
    const long long k = P.pre_ord[i] - P.pre_ord[rank * P.pre.per_rank];
    p2m_scramble_pos(13579LL * (rank + 1), k, pos);
  }
  if (P.pre.centre) p2m_rotate_pos(&P.pre, pos);
}

__device__ __forceinline__ bool cut_record(const PaintParams &P, const float *records, long long i,
                                           bool &shell, bool &massive) {
  const float *r = records + i * P.nfloat;
  shell = massive = false;
  float p0 = __ldg(r + 0), p1 = __ldg(r + 1), p2 = __ldg(r + 2), rth = __ldg(r + 6);
  if (!(p2m_isfinite(p0) && p2m_isfinite(p1) && p2m_isfinite(p2) && p2m_isfinite(rth)))
    return false;
  float xh = FSUB(p2, P.chihview), yh = p1, zh = p0;
  float chih = FSQRT(FADD(FADD(FMUL(xh, xh), FMUL(yh, yh)), FMUL(zh, zh)));
  shell = !(chih > P.cut_high || chih < P.cut_low);
  if (shell && (P.pre.scramble || P.pre.centre)) {
    /* the halo loop sees the scrambled / rotated position */
    float pos[3];
    halo_position(P, records, i, pos);
    p0 = pos[0];
    p1 = pos[1];
    p2 = pos[2];
    if (!(p2m_isfinite(p0) && p2m_isfinite(p1) && p2m_isfinite(p2))) {
      /* each rank's first scrambled halo: the seed's unreduced digits give a first draw
         above 1 and a NaN position; it counts in the mass cut and paints nothing */
      massive = !(FMUL(P.mass_fac, FMUL(FMUL(rth, rth), rth)) < 1e13f);
      return false;
    }
  }
  float mass = FMUL(P.mass_fac, FMUL(FMUL(rth, rth), rth));
  massive = shell && !(mass < 1e13f);
  bool keep = massive;
  if (massive && !(P.flags & 2)) {
    float chi0 = FSQRT(FADD(FADD(FMUL(p2, p2), FMUL(p1, p1)), FMUL(p0, p0)));
    float z = p2m_lookup(P.zofr, P.cosmo.dzofr, chi0);
    keep = !(p2m_lookup(P.rofz, P.cosmo.drofz, z) > P.th.chimaxt);
  }
  return keep;
}

/* -------------------------------------------------------------- ingest: set-up ----- */

/* float-float numbers (hi + lo, |lo| <= ulp(hi)/2) built with error-free transformations
   (Dekker / Knuth two-product and two-sum through fmaf); ~44-bit precision at FP32 cost */
struct ffloat {
  float h, l;
};

__device__ __forceinline__ ffloat ff_sq(float a) {
  const float p = __fmul_rn(a, a);
  return {p, __fmaf_rn(a, a, -p)};
}

__device__ __forceinline__ ffloat ff_norm(float s, float e) {
  const float h = __fadd_rn(s, e);
  return {h, __fsub_rn(e, __fsub_rn(h, s))};
}

__device__ __forceinline__ ffloat ff_add(ffloat x, ffloat y) {
  const float s = __fadd_rn(x.h, y.h);
  const float bb = __fsub_rn(s, x.h);
  float e = __fadd_rn(__fsub_rn(x.h, __fsub_rn(s, bb)), __fsub_rn(y.h, bb));
  e = __fadd_rn(e, __fadd_rn(x.l, y.l));
  return ff_norm(s, e);
}

/* sqrt with one Newton correction of the correctly rounded FP32 root */
__device__ __forceinline__ ffloat ff_sqrt(ffloat x) {
  const float y = __fsqrt_rn(x.h);
  const float r = __fadd_rn(__fmaf_rn(-y, y, x.h), x.l);
  return ff_norm(y, __fdiv_rn(r, __fmul_rn(2.0f, y)));
}

/* the same with the correction's quotient from the approximate division (its 2-ulp error
   is ~2^-46 of the root): the painting kernels' per-candidate form */
__device__ __forceinline__ ffloat ff_sqrt_fast(ffloat x) {
  const float y = __fsqrt_rn(x.h);
  const float r = __fadd_rn(__fmaf_rn(-y, y, x.h), x.l);
  return ff_norm(y, __fdividef(r, __fmul_rn(2.0f, y)));
}

__device__ __forceinline__ ffloat ff_mul_f(ffloat x, float y) {
  const float p = __fmul_rn(x.h, y);
  return ff_norm(p, __fmaf_rn(x.l, y, __fmaf_rn(x.h, y, -p)));
}

__device__ __forceinline__ ffloat ff_mul(ffloat x, ffloat y) {
  const float p = __fmul_rn(x.h, y.h);
  float e = __fmaf_rn(x.h, y.h, -p);
  e = __fmaf_rn(x.h, y.l, __fmaf_rn(x.l, y.h, e));
  return ff_norm(p, e);
}

/* exact sum of two floats as a float-float (Knuth's two-sum, no ordering needed) */
__device__ __forceinline__ ffloat ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

/* float-float plus float */
__device__ __forceinline__ ffloat ff_add_f(ffloat x, float y) {
  const ffloat s = ff_two_sum(x.h, y);
  return ff_norm(s.h, __fadd_rn(s.l, x.l));
}

/* square of a float-float */
__device__ __forceinline__ ffloat ff_sqr(ffloat x) {
  const float p = __fmul_rn(x.h, x.h);
  const float e = __fmaf_rn(x.h, x.h, -p);
  return ff_norm(p, __fmaf_rn(__fmul_rn(2.0f, x.h), x.l, e));
}

/* x / y with one correction of the FP32 quotient (exact remainder through fmaf) */
__device__ __forceinline__ ffloat ff_div(ffloat x, ffloat y) {
  const float q = __fdiv_rn(x.h, y.h);
  float r = __fmaf_rn(-q, y.h, x.h);
  r = __fsub_rn(__fadd_rn(r, x.l), __fmul_rn(q, y.l));
  return ff_norm(q, __fdiv_rn(r, y.h));
}

/* geometry, thresholds and interpolation constants of one halo from its loop
   quantities (pks2map.f90:284-298 outputs) */
__device__ void halo_geometry(const PaintParams &P, float xh, float yh, float zh, float rh,
                              float chih, float mh, float redshift, HaloRec &H,
                              unsigned int *err) {
  /* haloproject.f90:47 / :93 */
  float T = FMUL(4.0f, p2m_asinf(FDIV(rh, chih)));
  /* projecthalo_flatsky divides its arguments by chi in place (:97-99) */
  float xf = FDIV(xh, chih), yf = FDIV(yh, chih), zf = FDIV(zh, chih);
  /* interpolate_table per-halo part (maptable.f90:184-202) */
  float chi_t = p2m_lookup(P.rofz, P.cosmo.drofz, redshift);
  p2m_hinterp hi = p2m_hinterp_make(&P.th, chi_t, mh);
  H.T = T;
  H.chi_t = hi.chi_t;
  H.fc = hi.fc;
  H.fm = hi.fm;
  H.ichi = hi.ichi;
  H.imh = hi.imh;
  H.zero = hi.zero;
  {
    long long nrt2 = 2LL * P.th.nrt;
    const int dm[4] = {0, 1, 0, 1}, dc[4] = {0, 0, 1, 1};
    for (int c = 0; c < 4; c++) {
      long long b = 2LL * (long long)P.th.nrt *
                    ((long long)(hi.imh - 1 + dm[c]) + (long long)P.th.nmht * (hi.ichi - 1 + dc[c]));
      H.cbase[c] = (b >= 0 && b + nrt2 <= P.th.nelem) ? (int)b : -1;
    }
  }
  /* flat-sky box (haloproject.f90:101-128) */
  H.jmin = 1;
  H.jmax = 0;
  H.kmin = 1;
  H.kmax = 0;
  H.theta_h = H.phi_h = 0.0f;
  if (P.npix_fs > 0 && !(zf < 0.0f)) {
    float th = p2m_asinf(xf), ph = p2m_asinf(yf);
    double w = DMUL((double)1.1f, (double)T);
    float tmin = (float)DSUB((double)th, w), tmax = (float)DADD((double)th, w);
    float pmin = (float)DSUB((double)ph, w), pmax = (float)DADD((double)ph, w);
    float hf = P.hf;
    if (!(tmax < -hf || tmin > hf) && !(pmax < -hf || pmin > hf)) {
      if (tmin <= -hf) tmin = FADD(-hf, 1e-10f);
      if (tmax >= hf) tmax = FSUB(hf, 1e-10f);
      if (pmin <= -hf) pmin = FADD(-hf, 1e-10f);
      if (pmax >= hf) pmax = FSUB(hf, 1e-10f);
      int jmin = (int)FDIV(FADD(tmin, hf), P.dpix) + 1;
      int jmax = (int)FDIV(FADD(tmax, hf), P.dpix) + 1;
      int kmin = (int)FDIV(FADD(pmin, hf), P.dpix) + 1;
      int kmax = (int)FDIV(FADD(pmax, hf), P.dpix) + 1;
      H.jmin = max(1, jmin);
      H.jmax = min(jmax, P.npix_fs);
      H.kmin = max(1, kmin);
      H.kmax = min(kmax, P.npix_fs);
      H.theta_h = th;
      H.phi_h = ph;
    }
  }
  /* HEALPix disc (haloproject.f90:51-55) */
  H.ir_lo = 1;
  H.ir_hi = 0;
  H.z0h = H.z0l = H.s0h = H.s0l = H.p0h = H.p0l = 0.0f;
  H.C_in = H.C_out = H.C_span = 0.0f;
  if (P.nside > 0) {
    H.hv[0] = FDIV(zf, chih);
    H.hv[1] = FDIV(yf, chih);
    H.hv[2] = FDIV(xf, chih);
    if ((double)T > P2M_HP_PI || !(T >= 0.0f)) {
      atomicOr(err, (unsigned)P2M_DEVERR_RADIUS); /* query_disc aborts on radius > pi */
    } else {
      /* unit centre z = c / |v|, sin(theta) = sqrt(a^2 + b^2) / |v| in float-float (the
         squares of the float components are exact as float-float pairs); phi / 2pi from
         the FP64 atan2 */
      const float a = H.hv[0], b = H.hv[1], c = H.hv[2];
      const ffloat ss = ff_add(ff_sq(a), ff_sq(b));
      const ffloat nn = ff_add(ss, ff_sq(c));
      if (nn.h > 0.0f) {
        const ffloat nrm = ff_sqrt(nn);
        const ffloat z0 = ff_div({c, 0.0f}, nrm);
        const ffloat s0 = ss.h > 0.0f ? ff_div(ff_sqrt(ss), nrm) : ffloat{0.0f, 0.0f};
        H.z0h = z0.h;
        H.z0l = z0.l;
        H.s0h = s0.h;
        H.s0l = s0.l;
      }
      /* phi / 2pi by table-based reduction (Tang's method) in float-float: k = the grid
         angle 2 pi k / M nearest the FP32 atan2; (a, b) rotated by -2 pi k / M leaves an
         angle |d| < 8e-4 = atan(t) = t - t^3/3 (next term < 1e-16); phi / 2pi =
         k / M (exact) + d / 2pi, good to ~1e-15 */
      if (a != 0.0f || b != 0.0f) {
        const float phi1 = atan2f(b, a);
        const int k = __float2int_rn(phi1 * ((float)P2M_PHITAB / 6.28318531f));
        const float4 cs = P.phitab[k & (P2M_PHITAB - 1)];
        const ffloat cz = {cs.x, cs.y}, sz = {cs.z, cs.w};
        const ffloat ap = ff_add(ff_mul_f(cz, a), ff_mul_f(sz, b));
        const ffloat bp = ff_add(ff_mul_f(cz, b), ff_mul_f({-sz.h, -sz.l}, a));
        const ffloat t = ff_div(bp, ap);
        const float t3 = __fdiv_rn(__fmul_rn(__fmul_rn(t.h, t.h), t.h), 3.0f);
        const ffloat d = ff_add(t, {-t3, 0.0f});
        constexpr double kInv2pi = 1.0 / P2M_HP_TWOPI; /* folded at compile time */
        const ffloat inv2pi = {(float)kInv2pi, (float)(kInv2pi - (double)(float)kInv2pi)};
        const ffloat pf = ff_add({(float)k * (1.0f / (float)P2M_PHITAB), 0.0f}, ff_mul(d, inv2pi));
        H.p0h = pf.h;
        H.p0l = pf.l;
      }
      H.C_in = chord2(T * (1.0f - 2e-6f));
      H.C_out = chord2(T * (1.0f + 2e-6f));
      float tspan = T * (1.0f + 2e-5f) + 1e-6f;
      H.C_span = chord2(tspan);
      float theta0 = atan2f(H.s0h, H.z0h);
      float tmin = theta0 - tspan, tmax = theta0 + tspan;
      int n4 = 4 * P.nside;
      int lo = 1, hi_ = n4 - 1;
      if (tmin > 0.0f) lo = max(1, (int)floorf(p2m_ring_coord(P.nside, tmin)) - 1);
      if (tmax < 3.14159265f) hi_ = min(n4 - 1, (int)ceilf(p2m_ring_coord(P.nside, tmax)) + 1);
      H.ir_lo = lo;
      H.ir_hi = hi_;
    }
  }
}

__device__ __forceinline__ void store_halo(const PaintParams &P, const IngestBuffers &B, long long s,
                                           const HaloRec &H, unsigned long long &fsrows) {
  B.halos[s] = H;
  /* items are made at ingest for the large halos only; the sweep enumerates the others.
     The warp reserves its large halos' item ranges with one atomic add (with big_rings
     0, as the plain FP64 path runs, every halo is large) */
  int nr = H.ir_hi - H.ir_lo + 1;
  const unsigned big = nr > P.big_rings ? (unsigned)nr : 0u;
  B.nring[s] = big;
  const unsigned long long at = warp_reserve(&B.ctr->n_items, big);
  if (big) B.ioff[s] = (long long)at;
  if (B.ring_hist) { /* painting order by first ring */
    B.ring_key[s] = H.ir_lo;
    atomicAdd(&B.ring_hist[H.ir_lo], 1u);
  }
  if (H.jmin <= H.jmax && H.kmin <= H.kmax) fsrows += (unsigned long long)(H.kmax - H.kmin + 1);
}

/* light-cone of call-local record i: the last cone whose first record is <= i */
__device__ __forceinline__ int cone_of(const IngestBuffers &B, long long i) {
  if (B.ncones <= 1) return 0;
  int lo = 0, hi = B.ncones - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (B.cone_off[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

/* per-halo set-up of record i as halo s (pks2map.f90:264, :284-298) */
__device__ __forceinline__ void setup_record(const PaintParams &P, const IngestBuffers &B,
                                             long long s, int i, unsigned long long &fsrows) {
  {
    const float *r = B.records + (long long)i * P.nfloat;
    float pos[3];
    halo_position(P, B.records, i, pos);
    float p0 = pos[0], p1 = pos[1], p2 = pos[2], rth = r[6];
    float mass = FMUL(P.mass_fac, FMUL(FMUL(rth, rth), rth));
    float xh = p2, yh = p1, zh = p0;
    float chih = FSQRT(FADD(FADD(FMUL(xh, xh), FMUL(yh, yh)), FMUL(zh, zh)));
    float redshift = p2m_lookup(P.zofr, P.cosmo.dzofr, chih);
    xh = FSUB(xh, P.chihview);
    chih = FSQRT(FADD(FADD(FMUL(xh, xh), FMUL(yh, yh)), FMUL(zh, zh)));
    float mh = FMUL(FSQRT(FDIV(p2m_deltacrit(&P.cosmo, redshift), P.bbps_delta)), mass);
    float rh = p2m_powf(FDIV(FDIV(FDIV(FDIV(FMUL(3.0f, mh), 4.0f), P.cosmo.mypi), 200.0f),
                             p2m_rhocrit(&P.cosmo, redshift)),
                        0.333333343f);
    HaloRec H;
    H.rec = B.rec_base + i;
    H.cone = cone_of(B, i);
    H.w1 = 1.0f;
    H.w2 = 1.0f;
    if (P.any_ksz) {
      /* intended per-halo -v_los/c of pksc.f90:70-74, from the record as read */
      p0 = r[0];
      p1 = r[1];
      p2 = r[2];
      float v0 = r[3], v1 = r[4], v2 = r[5];
      float dot = FADD(FADD(FMUL(p0, v0), FMUL(p1, v1)), FMUL(p2, v2));
      float nrm = FSQRT(FADD(FADD(FMUL(p0, p0), FMUL(p1, p1)), FMUL(p2, p2)));
      H.w2 = -FDIV(FDIV(dot, nrm), 3.e5f);
    }
    halo_geometry(P, xh, yh, zh, rh, chih, mh, redshift, H, &B.ctr->err);
    store_halo(P, B, s, H, fsrows);
  }
}

#define CS_QCAP (256 + 256 * CUT_PER_THREAD)

/* The cut and the set-up in one pass: each block cuts tiles of 2048 records into a
   shared-memory queue of survivors and sets up 256 of them (one per thread) whenever the
   queue holds that many, so the FP64-heavy set-up of some warps overlaps the catalogue
   stream of others and the survivor list never goes through global memory.  Halo slots
   are reserved 256 at a time. */
__global__ void __launch_bounds__(256) k_cut_setup(PaintParams P, IngestBuffers B, long long n) {
  __shared__ int q[CS_QCAP];
  __shared__ int wsum[8];
  __shared__ int qn, tile_n;
  __shared__ long long base_s;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long nshell = 0, nmass = 0, nkeep = 0, fsrows = 0;
  if (threadIdx.x == 0) qn = 0;
  const long long tile = (long long)blockDim.x * CUT_PER_THREAD;
  for (long long t0 = (long long)blockIdx.x * tile; t0 < n; t0 += (long long)gridDim.x * tile) {
    unsigned keepbits = 0;
#pragma unroll
    for (int k = 0; k < CUT_PER_THREAD; k++) {
      long long i = t0 + (long long)k * blockDim.x + threadIdx.x;
      if (i >= n) continue;
      bool shell, massive;
      if (cut_record(P, B.records, i, shell, massive)) keepbits |= 1u << k;
      nshell += shell;
      nmass += massive;
    }
    int cnt = __popc(keepbits);
    nkeep += cnt;
    int x = cnt;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(FULL, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int w = 0; w < 8; w++) {
        int v = wsum[w];
        wsum[w] = tot;
        tot += v;
      }
      tile_n = tot;
    }
    __syncthreads();
    int pos = qn + wsum[wid] + (x - cnt);
    for (int k = 0; k < CUT_PER_THREAD; k++)
      if (keepbits & (1u << k)) q[pos++] = (int)(t0 + (long long)k * blockDim.x + threadIdx.x);
    __syncthreads();
    if (threadIdx.x == 0) qn += tile_n;
    __syncthreads();
    while (qn >= 256) {
      if (threadIdx.x == 0) base_s = (long long)atomicAdd(&B.ctr->n_surv, 256ull);
      __syncthreads();
      setup_record(P, B, base_s + threadIdx.x, q[qn - 256 + threadIdx.x], fsrows);
      __syncthreads();
      if (threadIdx.x == 0) qn -= 256;
      __syncthreads();
    }
  }
  if (qn > 0) {
    if (threadIdx.x == 0) base_s = (long long)atomicAdd(&B.ctr->n_surv, (unsigned long long)qn);
    __syncthreads();
    if ((int)threadIdx.x < qn) setup_record(P, B, base_s + threadIdx.x, q[threadIdx.x], fsrows);
  }
  block_count(&B.ctr->n_shell, nshell);
  block_count(&B.ctr->n_massive, nmass);
  block_count(&B.ctr->n_enum, nkeep);
  block_count(&B.ctr->n_fs_rows, fsrows);
}

/* per-halo set-up from already-computed loop quantities (p2m_project_halo): 9 floats
   x, y, z, r, chi, m, redshift, v, profile per halo */
__global__ void __launch_bounds__(256) k_setup_prepared(PaintParams P, IngestBuffers B,
                                                        const float *prep, long long n) {
  unsigned long long fsrows = 0;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x) {
    const float *q = prep + s * 9;
    int prof = (int)q[8];
    HaloRec H;
    H.rec = B.rec_base + s;
    H.cone = 0;
    H.w1 = prof == 1 ? q[7] : 0.0f;
    H.w2 = prof == 2 ? q[7] : 0.0f;
    halo_geometry(P, q[0], q[1], q[2], q[3], q[4], q[5], q[6], H, &B.ctr->err);
    if (H.zero && !(P.flags & 2)) { /* table value identically zero: nothing to enumerate */
      H.ir_lo = 1;
      H.ir_hi = 0;
      H.jmin = 1;
      H.jmax = 0;
    }
    store_halo(P, B, s, H, fsrows);
  }
  block_count(&B.ctr->n_fs_rows, fsrows);
  long long mine = 0;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x)
    mine++;
  block_count(&B.ctr->n_enum, (unsigned long long)mine);
}

/* --------------------------------------------------------------------- scans ----- */

#define SCAN_BLOCKS 1024

__global__ void __launch_bounds__(256) k_scan_partial(const unsigned int *in,
                                                      const unsigned long long *n_ptr,
                                                      long long *bsum) {
  long long n = (long long)*n_ptr;
  long long per = (n + SCAN_BLOCKS - 1) / SCAN_BLOCKS;
  long long lo = per * blockIdx.x, hi = min(n, lo + per);
  long long s = 0;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) s += in[i];
  __shared__ long long red[8];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(FULL, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long t = 0;
    for (int w = 0; w < 8; w++) t += red[w];
    bsum[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(1024) k_scan_top(long long *bsum, unsigned long long *total) {
  __shared__ long long sh[SCAN_BLOCKS];
  int t = threadIdx.x;
  sh[t] = bsum[t];
  __syncthreads();
  for (int o = 1; o < SCAN_BLOCKS; o <<= 1) {
    long long v = t >= o ? sh[t - o] : 0;
    __syncthreads();
    sh[t] += v;
    __syncthreads();
  }
  bsum[t] = t > 0 ? sh[t - 1] : 0;
  if (total && t == SCAN_BLOCKS - 1) *total = (unsigned long long)sh[t];
}

__global__ void __launch_bounds__(256) k_scan_apply(const unsigned int *in,
                                                    const unsigned long long *n_ptr,
                                                    const long long *bsum, long long *out) {
  long long n = (long long)*n_ptr;
  long long per = (n + SCAN_BLOCKS - 1) / SCAN_BLOCKS;
  long long lo = per * blockIdx.x, hi = min(n, lo + per);
  __shared__ long long warp_sums[8];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = bsum[blockIdx.x];
  __syncthreads();
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (long long base = lo; base < hi; base += blockDim.x) {
    long long i = base + threadIdx.x;
    long long v = i < hi ? (long long)in[i] : 0;
    long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(FULL, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    long long wofs = 0;
    for (int w = 0; w < wid; w++) wofs += warp_sums[w];
    if (i < hi) out[i] = carry + wofs + x - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += wofs + x;
    __syncthreads();
  }
}

/* --------------------------------------------------------------- ingest: items ----- */

/* a disc centre as the span construction reads it */
struct DiscGeom {
  float zh, zl, sh, sl, ph, pl, cspan;
  int irlo;
};

__device__ __forceinline__ DiscGeom geom_of(const HaloRec &H) {
  DiscGeom g;
  g.zh = H.z0h;
  g.zl = H.z0l;
  g.sh = H.s0h;
  g.sl = H.s0l;
  g.ph = H.p0h;
  g.pl = H.p0l;
  g.cspan = H.C_span;
  g.irlo = H.ir_lo;
  return g;
}

/* Candidate span of ring `ring` of a disc: every pixel centre with chord^2 <= C_span (a
   disc 2e-5 wider than dtheta) lies in [lo, lo+count).  FP32 only: the centre's z,
   sin(theta) and phi/2pi are (hi, lo) pairs like the ring table's z and sin(theta), so
   the differences lose nothing to cancellation (close hi parts subtract exactly), and
   phi0 npr / 2pi is carried as an exact two-product.  The span keeps a margin of 0.02
   pixel + 1e-5 of its half-width over the FP32 rounding of its centre (< 2e-3 pixel). */
__device__ __forceinline__ RingItem make_item(const PaintParams &P, const DiscGeom &g, int h,
                                              int ring) {
  RingItem it;
  const float4 zs = P.ringtab[ring];
  /* A = dz^2 + ds^2 and B = 4 sin(theta_ring) sin(theta_0) as float-float values: the
     ring's and the centre's (hi, lo) pairs differ without cancellation loss */
  const ffloat dzf = ff_add_f(ff_two_sum(zs.x, -g.zh), __fsub_rn(zs.y, g.zl));
  const ffloat dsf = ff_add_f(ff_two_sum(zs.z, -g.sh), __fsub_rn(zs.w, g.sl));
  const ffloat Af = ff_add(ff_sqr(dzf), ff_sqr(dsf));
  const ffloat Bf = ff_mul({zs.z, zs.w}, {__fmul_rn(4.0f, g.sh), __fmul_rn(4.0f, g.sl)});
  const float A = Af.h, Bc = Bf.h;
  int npr, kshift;
  long long npn;
  p2m_ring_info(P.nside, ring, &npr, &kshift, &npn);
  const float fn = (float)npr;
  /* q = phi0 npr / 2pi = qh + ql */
  const float qh = __fmul_rn(g.ph, fn);
  const float ql = __fmaf_rn(g.pl, fn, __fmaf_rn(g.ph, fn, -qh));
  const float sh = kshift ? 0.5f : 0.0f;
  const float cspan = g.cspan;
  int lo = 0, cnt = 0;
  bool full = false, empty = false;
  float hw = 0.0f;
  if (!(Bc > 1e-30f)) {
    if (A < cspan) full = true;
    else empty = true;
  } else {
    float t = (cspan - A) / Bc;
    if (t <= 0.0f) empty = true;
    else if (t >= 1.0f) full = true;
    else hw = asinf(sqrtf(t)) * (fn * 0.318309886f);
  }
  if (!empty) {
    const float c = __fadd_rn(__fsub_rn(qh, sh), ql); /* span centre, index units */
    if (!full) {
      const float eps = 0.02f + 1e-5f * hw;
      const float l = ceilf(c - hw - eps), hh = floorf(c + hw + eps);
      if (hh - l + 1.0f >= fn) full = true;
      else if (hh >= l) {
        lo = (int)l;
        cnt = (int)(hh - l) + 1;
      }
    }
    if (full) {
      lo = (int)ceilf(c - 0.5f * fn);
      cnt = npr;
    }
  }
  /* x0 = lo + sh - q = n0 + f0 with n0 = lo - a + rf, a = rint(qh) (qh - a exact) and rf the
     integer nearest to sh - (qh - a) - ql.  f0 = ((sh - rf) - d) - ql: sh - rf is exact and
     each subtraction rounds relative to its own result, so f0 keeps full relative precision
     however close the candidates come to the centre's longitude.  |n0| <= npr/2 + 1. */
  const float a = rintf(qh);
  const float d = __fsub_rn(qh, a);
  const float rf = rintf(__fsub_rn(__fsub_rn(sh, d), ql));
  /* f0 = ((sh - rf) - d) - ql as a float-float: sh - rf and d are exact */
  const ffloat f0f = ff_add_f(ff_two_sum(sh - rf, -d), -ql);
  const int n0 = lo - (int)a + (int)rf;
  /* pi / npr as a float-float, from the ring table */
  const float2 hdv = P.ringhd[ring];
  const ffloat hd = {hdv.x, hdv.y};
  it.halo = h;
  it.ring_n0 = (ring << 16) | (n0 & 0xffff);
  it.lo = lo;
  it.count = cnt;
  it.A = A;
  it.B = Bc;
  it.f0 = f0f.h;
  it.hdphi = hd.h;
  it.Al = Af.l;
  it.Bl = Bf.l;
  it.f0l = f0f.l;
  it.hdl = hd.l;
  return it;
}

/* warp-wide inclusive prefix sum */
__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(FULL, v, o);
    if (lane >= o) v += y;
  }
  return v;
}

/* largest lane j with key_j <= t, for keys non-decreasing over the lanes (key_0 <= t) */
__device__ __forceinline__ int warp_find(int key, int t) {
  int j = 0;
#pragma unroll
  for (int step = 16; step > 0; step >>= 1) {
    int o = __shfl_sync(FULL, key, j + step);
    if (o <= t) j += step;
  }
  return j;
}

/* one warp expands 32 consecutive halos into their (halo, ring) items, 32 items at a
   time over the warp's flattened ring list; only the large halos have rings here
   (nring 0 for the others) */
__global__ void __launch_bounds__(256) k_items(PaintParams P, IngestBuffers B) {
  const long long n = (long long)B.ctr->n_surv;
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long h0 = warp * 32; h0 < n; h0 += nwarps * 32) {
    const long long h = h0 + lane;
    const int nr = h < n ? (int)B.nring[h] : 0;
    const int rx = warp_incl_scan(nr);
    const int rel = rx - nr, total = __shfl_sync(FULL, rx, 31);
    for (int t0 = 0; t0 < total; t0 += 32) {
      const int t = t0 + lane;
      const int j = warp_find(rel, t);
      const int r = t - __shfl_sync(FULL, rel, j);
      if (t < total) {
        const long long hh = h0 + j;
        const HaloRec &H = B.halos[hh];
        B.items[B.ioff[hh] + r] = make_item(P, geom_of(H), (int)(B.halo_base + hh), H.ir_lo + r);
      }
    }
  }
}

/* ------------------------------------------------------------------ flat sky ----- */

/* appends the (halo, row) items of every halo with a flat-sky box */
__global__ void __launch_bounds__(256) k_fs_emit(PaintParams P, IngestBuffers B) {
  long long n = (long long)B.ctr->n_surv;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x) {
    const HaloRec &H = B.halos[s];
    if (H.jmin > H.jmax || H.kmin > H.kmax) continue;
    int nrow = H.kmax - H.kmin + 1;
    unsigned long long fb = atomicAdd(&B.ctr->n_fs_items, (unsigned long long)nrow);
    if ((long long)(fb + nrow) > B.fs_cap) {
      atomicOr(&B.ctr->err, (unsigned)P2M_DEVERR_FS_OVERFLOW);
      continue;
    }
    for (int t = 0; t < nrow; t++) {
      FsItem f;
      f.halo = (int)s;
      f.k = H.kmin + t;
      f.jmin = H.jmin;
      f.count = H.jmax - H.jmin + 1;
      B.fs_items[fb + t] = f;
    }
  }
}

/* the halo fields one candidate pixel needs */
struct HotHalo {
  float C_in, C_out, chi_t, fc, fm, w1, w2;
  int zc; /* bit 0: the table value is identically zero; bits 1..: the light-cone */
  int ichi, imh;
  int cb[4];
};
__device__ __forceinline__ bool hot_zero(const HotHalo &h) { return h.zc & 1; }
__device__ __forceinline__ int hot_cone(const HotHalo &h) { return h.zc >> 1; }

__device__ __forceinline__ HotHalo hot_of(const HaloRec &H) {
  HotHalo h;
  h.C_in = H.C_in;
  h.C_out = H.C_out;
  h.chi_t = H.chi_t;
  h.fc = H.fc;
  h.fm = H.fm;
  h.w1 = H.w1;
  h.w2 = H.w2;
  h.zc = (H.zero ? 1 : 0) | (H.cone << 1);
  h.ichi = H.ichi;
  h.imh = H.imh;
  for (int c = 0; c < 4; c++) h.cb[c] = H.cbase[c];
  return h;
}

/* The 64-bit fixed point of P2M_PREC_FIXED (unit 2^-56) converted with integer operations
   only: the FP64 units of this GPU run at a small fraction of the FP32 rate, and a pass
   converting every pixel of the maps through them took twice its memory time.
   float_to_fixed(v) = v 2^56 rounded to the nearest integer, ties to even (what
   __double2ll_rn((double)v * 2^56) gives for |v| < 128); fixed_to_float(q) = q 2^-56
   rounded to the nearest float, ties to even. */
__device__ __forceinline__ long long float_to_fixed(float v) {
  const unsigned int b = __float_as_uint(v);
  const int ex = (int)((b >> 23) & 0xffu);
  if (ex == 0) return 0; /* zero or subnormal: below half a unit */
  const unsigned long long m = (unsigned long long)((b & 0x7fffffu) | 0x800000u);
  const int sh = ex - 94; /* v 2^56 = m 2^sh */
  unsigned long long q;
  if (sh > 39) {
    q = 0x7fffffffffffffffull; /* |v| >= 128: outside the fixed-point range */
  } else if (sh >= 0) {
    q = m << sh;
  } else if (sh < -25) {
    q = 0; /* m 2^sh < 1/4 */
  } else {
    const int r = -sh;
    q = m >> r;
    const unsigned long long rem = m & ((1ull << r) - 1), half = 1ull << (r - 1);
    if (rem > half || (rem == half && (q & 1ull))) q++;
  }
  return (b >> 31) ? -(long long)q : (long long)q;
}
__device__ __forceinline__ float fixed_to_float(long long q) {
  if (q == 0) return 0.0f;
  const unsigned int sign = q < 0 ? 0x80000000u : 0u;
  const unsigned long long m = q < 0 ? 0ull - (unsigned long long)q : (unsigned long long)q;
  int e = 63 - __clzll((long long)m); /* m in [2^e, 2^(e+1)) */
  unsigned long long top;
  if (e > 23) {
    const int r = e - 23;
    top = m >> r;
    const unsigned long long rem = m & ((1ull << r) - 1), half = 1ull << (r - 1);
    if (rem > half || (rem == half && (top & 1ull))) top++;
    if (top >> 24) { /* rounded up to the next power of two */
      top >>= 1;
      e++;
    }
  } else {
    top = m << (23 - e);
  }
  /* q 2^-56 = 1.f 2^(e - 56): a normal float for every e in 0..64 */
  return __uint_as_float(sign | ((unsigned int)(e - 56 + 127) << 23) | (unsigned int)(top & 0x7fffffu));
}

/* the compensated deposit's second half: the exact rounding error of each map's add
   (TwoSum of its returned old value and the value) goes to that map's low word, and the
   pixel's tile is flagged when any error is nonzero */
__device__ __forceinline__ void compensate_lo(const PaintParams &P, const SweepBuffers *W,
                                              long long slot, const float *vals,
                                              const float *olds) {
  bool any = false;
#pragma unroll
  for (int m = 0; m < P2M_MAXMAPS; m++) {
    if (m >= P.nmaps || vals[m] == 0.0f) continue;
    float old = olds[m], v = vals[m];
    float sm = __fadd_rn(old, v);
    float bb = __fsub_rn(sm, old);
    float err = __fadd_rn(__fsub_rn(old, __fsub_rn(sm, bb)), __fsub_rn(v, bb));
    if (err != 0.0f) {
      atomicAdd(W->lo + (long long)m * W->npix + slot, err);
      any = true;
    }
  }
  if (any) W->tiles[slot >> P2M_TILE_SHIFT] = 1;
}

/* adds one pixel's values (nmaps of them) at slot `slot`.  ACC 0: FP64 accumulator
   (fire-and-forget red.add.f64); ACC 1: two-float (hi, lo) FP32 accumulator, hi by an
   atomic add that returns the old value, lo the exact TwoSum rounding error; ACC 2:
   compensated accumulation with the float output map as the high word, the low words
   sparse (nonzero only where an add rounded) and their tiles flagged; ACC 3: 64-bit
   fixed-point accumulator (value * 2^56 rounded to an integer, fire-and-forget).  All
   maps' adds are issued before any result is used. */
template <int ACC>
__device__ __forceinline__ void accumulate_vals(const PaintParams &P, void *acc, long long slot,
                                                const float *vals, const SweepBuffers *W) {
  if (ACC == 0) {
    double *a = (double *)acc + slot * P.nmaps;
#pragma unroll
    for (int m = 0; m < P2M_MAXMAPS; m++)
      if (m < P.nmaps && vals[m] != 0.0f) atomicAdd(a + m, (double)vals[m]);
  } else if (ACC == 2) {
    float olds[P2M_MAXMAPS];
#pragma unroll
    for (int m = 0; m < P2M_MAXMAPS; m++)
      olds[m] = (m < P.nmaps && vals[m] != 0.0f) ? atomicAdd(W->out[m] + slot, vals[m]) : 0.0f;
    compensate_lo(P, W, slot, vals, olds);
  } else if (ACC == 3) {
    /* 64-bit fixed point: integer adds are associative, so the sums do not depend on the
       order in which the atomics land */
    unsigned long long *a = (unsigned long long *)acc + slot * P.nmaps;
#pragma unroll
    for (int m = 0; m < P2M_MAXMAPS; m++)
      if (m < P.nmaps && vals[m] != 0.0f) {
        if (!(fabsf(vals[m]) < 128.0f)) atomicOr(P.err_flag, (unsigned)P2M_DEVERR_FIXED);
        atomicAdd(a + m, (unsigned long long)float_to_fixed(vals[m]));
      }
  } else {
    float *a = (float *)acc + 2 * slot * P.nmaps;
    float olds[P2M_MAXMAPS];
#pragma unroll
    for (int m = 0; m < P2M_MAXMAPS; m++)
      olds[m] = (m < P.nmaps && vals[m] != 0.0f) ? atomicAdd(a + 2 * m, vals[m]) : 0.0f;
#pragma unroll
    for (int m = 0; m < P2M_MAXMAPS; m++) {
      if (m >= P.nmaps || vals[m] == 0.0f) continue;
      float old = olds[m], v = vals[m];
      /* TwoSum: the exact rounding error of old + v, carried in the low word */
      float sm = __fadd_rn(old, v);
      float bb = __fsub_rn(sm, old);
      float err = __fadd_rn(__fsub_rn(old, __fsub_rn(sm, bb)), __fsub_rn(v, bb));
      if (err != 0.0f) atomicAdd(a + 2 * m + 1, err);
    }
  }
}

/* The eight-term blend of maptable.f90:204-212 for known (ir, fr), in the reference's
   float sequence: every product and sum rounded in source order, so that a pixel whose
   (ir, fr) equal the reference's gets the reference's value bit for bit. */
__device__ __forceinline__ float blend_pair_seq(float a0, float b0, float a1, float b1, float a2,
                                                float b2, float a3, float b3, float fr,
                                                float ofr, float fc, float ofc, float fm,
                                                float ofm) {
  float v = 0.0f;
  v = FADD(v, FMUL(FMUL(FMUL(a0, ofr), ofc), ofm));
  v = FADD(v, FMUL(FMUL(FMUL(b0, fr), ofc), ofm));
  v = FADD(v, FMUL(FMUL(FMUL(a1, ofr), fc), ofm));
  v = FADD(v, FMUL(FMUL(FMUL(b1, fr), fc), ofm));
  v = FADD(v, FMUL(FMUL(FMUL(a2, ofr), ofc), fm));
  v = FADD(v, FMUL(FMUL(FMUL(b2, fr), ofc), fm));
  v = FADD(v, FMUL(FMUL(FMUL(a3, ofr), fc), fm));
  v = FADD(v, FMUL(FMUL(FMUL(b3, fr), fc), fm));
  return v;
}

/* the four corners' rows and the r-index pair (ir, ir + 1) lie inside the table */
__device__ __forceinline__ bool fast_corners(const PaintParams &P, const HotHalo &H, int ir) {
  return H.cb[0] >= 0 && H.cb[1] >= 0 && H.cb[2] >= 0 && H.cb[3] >= 0 && ir >= 1 &&
         ir < P.th.nrt;
}

/* deposit weight of map m: 1 for tSZ (profile 1), -v_los / c for kSZ (profile 2) */
__device__ __forceinline__ float map_weight(const PaintParams &P, const HotHalo &H, int m) {
  return P.map_profile[m] == 2 ? H.w2 : H.w1;
}

/* Profile values of maps 2q and 2q + 1 at one pixel from pair table q, whose entry
   cb / 2 + ir - 1 (corner row cb) holds map 2q's table value in .x and map 2q + 1's in .y:
   both values of a (corner, r-index) entry come from one 8-byte load.  `two` false: map
   2q only (vb = 0).  Needs fast_corners. */
__device__ __forceinline__ void pair_values(const float2 *tab, const HotHalo &H, int ir,
                                            float fr, float wa, float wb, bool two, float &va,
                                            float &vb) {
  const int r = ir - 1;
  const float2 a0 = __ldg(tab + (H.cb[0] >> 1) + r), b0 = __ldg(tab + (H.cb[0] >> 1) + r + 1);
  const float2 a1 = __ldg(tab + (H.cb[1] >> 1) + r), b1 = __ldg(tab + (H.cb[1] >> 1) + r + 1);
  const float2 a2 = __ldg(tab + (H.cb[2] >> 1) + r), b2 = __ldg(tab + (H.cb[2] >> 1) + r + 1);
  const float2 a3 = __ldg(tab + (H.cb[3] >> 1) + r), b3 = __ldg(tab + (H.cb[3] >> 1) + r + 1);
  const float fc = H.fc, fm = H.fm;
  const float ofr = FSUB(1.0f, fr), ofc = FSUB(1.0f, fc), ofm = FSUB(1.0f, fm);
  va = FMUL(wa, blend_pair_seq(a0.x, b0.x, a1.x, b1.x, a2.x, b2.x, a3.x, b3.x, fr, ofr, fc,
                               ofc, fm, ofm));
  vb = two ? FMUL(wb, blend_pair_seq(a0.y, b0.y, a1.y, b1.y, a2.y, b2.y, a3.y, b3.y, fr, ofr,
                                     fc, ofc, fm, ofm))
           : 0.0f;
}

/* profile values of every map at one pixel (maptable.f90:204-212 with known ir, fr: the
   reference's float sequence), deposited at slot `slot`: through the pair tables where
   the corners lie inside the table, else (clamped corners, the last r-index) through the
   reference's clamped offsets */
template <int ACC>
__device__ __forceinline__ void deposit_maps(const PaintParams &P, const HotHalo &H, void *acc,
                                             long long slot, int ir, float fr,
                                             const SweepBuffers *W = nullptr) {
  float vals[P2M_MAXMAPS];
#pragma unroll
  for (int m = 0; m < P2M_MAXMAPS; m++) vals[m] = 0.0f;
  if (fast_corners(P, H, ir)) {
#pragma unroll
    for (int q = 0; q < P2M_MAXMAPS / 2; q++) {
      if (2 * q >= P.nmaps) continue;
      const bool two = 2 * q + 1 < P.nmaps;
      pair_values(P.pair_tab[q], H, ir, fr, map_weight(P, H, 2 * q),
                  two ? map_weight(P, H, 2 * q + 1) : 0.0f, two, vals[2 * q], vals[2 * q + 1]);
    }
  } else {
    p2m_hinterp hi;
    hi.chi_t = H.chi_t;
    hi.fc = H.fc;
    hi.fm = H.fm;
    hi.ichi = H.ichi;
    hi.imh = H.imh;
    hi.zero = hot_zero(H);
#pragma unroll
    for (int m = 0; m < P2M_MAXMAPS; m++) {
      if (m >= P.nmaps) continue;
      const int prof = P.map_profile[m];
      vals[m] = FMUL(map_weight(P, H, m),
                     p2m_blend8(P.tables[P.map_table[m]], &P.th, &hi, prof, ir, fr));
    }
  }
  accumulate_vals<ACC>(P, acc, slot, vals, W);
}

/* A compensated deposit of one or two maps split in two: the atomic adds are issued at
   once, the TwoSum of their returned old values is finished one candidate later, so the
   atomics' round trip overlaps the next candidate's decision and table reads. */
struct PendingDeposit {
  long long slot; /* -1: none */
  float v0, v1, o0, o1;
};

__device__ __forceinline__ void finish_pending(const SweepBuffers &W, PendingDeposit &d) {
  if (d.slot < 0) return;
  bool any = false;
  if (d.v0 != 0.0f) {
    const float sm = __fadd_rn(d.o0, d.v0), bb = __fsub_rn(sm, d.o0);
    const float err = __fadd_rn(__fsub_rn(d.o0, __fsub_rn(sm, bb)), __fsub_rn(d.v0, bb));
    if (err != 0.0f) {
      atomicAdd(W.lo + d.slot, err);
      any = true;
    }
  }
  if (d.v1 != 0.0f) {
    const float sm = __fadd_rn(d.o1, d.v1), bb = __fsub_rn(sm, d.o1);
    const float err = __fadd_rn(__fsub_rn(d.o1, __fsub_rn(sm, bb)), __fsub_rn(d.v1, bb));
    if (err != 0.0f) {
      atomicAdd(W.lo + W.npix + d.slot, err);
      any = true;
    }
  }
  if (any) W.tiles[d.slot >> P2M_TILE_SHIFT] = 1;
  d.slot = -1;
}

/* haloproject.f90:136-152: one warp per (halo, row); every operation is the
   reference's float sequence, so the pixel set and values are exact */
template <int PREC>
__global__ void __launch_bounds__(256) k_paint_fs(PaintParams P, IngestBuffers B) {
  long long n = (long long)min(B.ctr->n_fs_items, (unsigned long long)B.fs_cap);
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  unsigned long long nupd = 0;
  for (long long w = warp; w < n; w += nwarps) {
    FsItem f = B.fs_items[w];
    const HaloRec &H = B.halos[f.halo];
    p2m_hinterp hi = halo_hinterp(H);
    float phip = FADD(-P.hf, FMUL(FSUB((float)f.k, 0.5f), P.dpix));
    float dphi = (float)DSUB((double)phip, (double)H.phi_h);
    for (int t = lane; t < f.count; t += 32) {
      int j = f.jmin + t;
      float thetap = FADD(-P.hf, FMUL(FSUB((float)j, 0.5f), P.dpix));
      float dtheta = (float)DSUB((double)thetap, (double)H.theta_h);
      float angle = FSQRT(FADD(FMUL(dphi, dphi), FMUL(dtheta, dtheta)));
      if (angle < H.T) {
        nupd++;
        if (H.zero) continue;
        float r = FMUL(hi.chi_t, p2m_tanf(angle));
        if (r > P.th.rmaxt) continue;
        int ir;
        float fr;
        p2m_rindex(&P.th, r, &ir, &fr);
        long long pix = (long long)(j - 1) + (long long)P.npix_fs * (f.k - 1);
        deposit_maps<PREC>(P, hot_of(H), B.fs_acc, pix, ir, fr);
      }
    }
  }
  warp_count(&B.ctr->fs_updates, nupd);
}

/* ---------------------------------------------------------- sweep: the painting ----- */

/* largest g in [lo, hi) with off[g] <= p (off[lo] <= p), found by the whole warp */
__device__ __forceinline__ long long warp_upper(const long long *off, long long lo, long long hi,
                                                long long p) {
  int lane = threadIdx.x & 31;
  while (hi - lo > 32) {
    long long span = hi - lo;
    long long s = lo + (span * lane) / 32;
    bool le = off[s] <= p;
    unsigned m = __ballot_sync(FULL, le);
    int t = m ? 31 - __clz(m) : 0;
    long long nlo = lo + (span * t) / 32;
    long long nhi = t < 31 ? lo + (span * (t + 1)) / 32 : hi;
    lo = nlo;
    hi = nhi;
  }
  long long s = lo + lane;
  bool le = s < hi && off[s] <= p;
  unsigned m = __ballot_sync(FULL, le);
  return lo + (m ? 31 - __clz(m) : 0);
}

struct ExactRes {
  bool inside, zero;
  int ir;
  float fr, u;
};

/* the reference's decision and interpolation inputs for one pixel: FP64 pixel centre
   and angular distance (haloproject.f90:63-70), float interpolation (maptable.f90) */
__device__ __noinline__ ExactRes exact_eval(const PaintParams &P, const HaloRec &H, long long pix) {
  ExactRes e;
  e.inside = false;
  e.zero = false;
  e.ir = 0;
  e.fr = 0.0f;
  e.u = 0.0f;
  double v2[3], v1[3] = {(double)H.hv[0], (double)H.hv[1], (double)H.hv[2]};
  p2m_pix2vec_ring(P.nside, pix, v2);
  float angle = (float)p2m_angdist(v1, v2);
  if (!((double)angle < (double)H.T)) return e;
  e.inside = true;
  if (H.zero) {
    e.zero = true;
    return e;
  }
  float r = FMUL(H.chi_t, p2m_tanf(angle));
  if (r > P.th.rmaxt) {
    e.zero = true;
    return e;
  }
  p2m_rindex(&P.th, r, &e.ir, &e.fr);
  float rr = r < P.th.rmint ? FADD(P.th.rmint, 1e-5f) : r;
  e.u = FDIV(FSUB(p2m_logf(rr), P.th.lrmin), P.th.drt);
  return e;
}

__device__ __forceinline__ void record_set(long long *set_rec, long long *set_pix, long long cap,
                                           unsigned long long *ctr, long long rec, long long pix) {
  unsigned long long k = atomicAdd(ctr, 1ull);
  if ((long long)k < cap) {
    set_rec[k] = rec;
    set_pix[k] = pix;
  }
}

/* sin(y) - y by its Taylor series through y^15, for the half longitude offset y of a
   candidate from the disc centre: |y| < pi/2 + pi/npr <= 2.37, where the truncation stays
   below 1e-8; the result is a correction to y, so its relative rounding (a few ulp)
   costs ~y^2/6 ulp of sin(y) */
__device__ __forceinline__ float sin_minus_arg(float y) {
  const float y2 = y * y;
  float p = 1.0f / 1307674368000.0f;      /* 1/15! */
  p = fmaf(p, y2, -1.0f / 6227020800.0f); /* -1/13! */
  p = fmaf(p, y2, 1.0f / 39916800.0f);    /* 1/11! */
  p = fmaf(p, y2, -1.0f / 362880.0f);     /* -1/9! */
  p = fmaf(p, y2, 1.0f / 5040.0f);        /* 1/7! */
  p = fmaf(p, y2, -1.0f / 120.0f);        /* -1/5! */
  p = fmaf(p, y2, 1.0f / 6.0f);           /* 1/3! */
  return -y * y2 * p;                     /* -y^3 (1/3! - y^2/5! + ...) */
}

/* asin(u) - u by its series through u^15 for 0 <= u <= 1/4 (truncation < 1e-12 of u) */
__device__ __forceinline__ float asin_minus_arg(float u) {
  const float u2 = u * u;
  float p = 143.0f / 10240.0f;
  p = fmaf(p, u2, 231.0f / 13312.0f);
  p = fmaf(p, u2, 63.0f / 2816.0f);
  p = fmaf(p, u2, 35.0f / 1152.0f);
  p = fmaf(p, u2, 5.0f / 112.0f);
  p = fmaf(p, u2, 3.0f / 40.0f);
  p = fmaf(p, u2, 1.0f / 6.0f);
  return u * u2 * p;
}

/* Fast mixed-precision decision for one candidate.  Returns 0 outside, 1 inside with
   (ir, fr) or zero value, 2 when the exact path must decide.
   The chord^2 between the candidate's centre and the disc centre is formed as a
   float-float (~44 bits): c2 = A + B sin^2(y), y = x pi / npr.  Its high word decides
   against the certainly-inside / certainly-outside thresholds.  Inside, the angle
   2 asin(sqrt(c2) / 2) is carried to ~1e-11 and rounded to float, which is the
   reference's real(angdist(...)) (haloproject.f90:66) except within ~1e-11 of a rounding
   tie; from there r, log r and the table indices are the reference's float sequence
   (maptable.f90:185-202), so the pixel's value is the reference's bit for bit. */
__device__ __forceinline__ int fast_decide(const PaintParams &P, const RingItem &it,
                                           const HotHalo &H, int k, int &ir, float &fr,
                                           bool &zero_val, float &u_out) {
  const ffloat x = ff_add_f(ff_two_sum((float)(item_n0(it) + k), it.f0), it.f0l);
  const ffloat y = ff_mul(x, {it.hdphi, it.hdl});
  const ffloat sy = ff_add_f(y, sin_minus_arg(y.h));
  const ffloat c2f = ff_add({it.A, it.Al}, ff_mul({it.B, it.Bl}, ff_sqr(sy)));
  const float c2 = c2f.h;
  if (c2 >= H.C_out) return 0;
  if (c2 > H.C_in) return 2;
  zero_val = false;
  const ffloat uf = ff_sqrt_fast(c2f);
  const float u = 0.5f * uf.h;
  if (u > 0.25f) return 2; /* discs wider than ~29 degrees: the exact path */
  /* angle = 2 asin(chord / 2) = chord + 2 (asin(u) - u), u = chord / 2 */
  const ffloat ang = ff_add_f(uf, 2.0f * asin_minus_arg(u));
  const float angle = ang.h; /* hi = the float nearest hi + lo */
  const float r = FMUL(H.chi_t, p2m_tanf_pio4(angle)); /* angle <= 2 asin(1/4) < pi/4 */
  const float dr = 1e-5f;
  if (r > P.th.rmaxt * (1.0f + dr)) {
    zero_val = true;
    return 1;
  }
  if (r >= P.th.rmaxt * (1.0f - dr)) return 2;
  if (r < P.th.rmint * (1.0f - dr)) {
    ir = P.ir_c;
    fr = P.fr_c;
    u_out = -1.0f;
    return 1;
  }
  if (r <= P.th.rmint * (1.0f + dr)) return 2;
  /* the reference's log (the same float function as the exact path and the oracle):
     fr is a difference of logs that cancels to ~drt, so a cruder log's error of a few
     ulp of log r would move the value by ~1e-7 relative, and coherently over a disc */
  const float lr = p2m_logf_normal(r); /* rmint < r < rmaxt here */
  const float uu = (lr - P.th.lrmin) * P.inv_drt;
  const int iu = (int)uu;
  const float fu = uu - (float)iu;
  if (fu < P.band_u || fu > 1.0f - P.band_u || iu < 0 || iu > P.th.nrt - 2) return 2;
  ir = iu + 1;
  fr = FSUB(lr, FADD(P.th.lrmin, FMUL((float)(ir - 1), P.th.drt)));
  u_out = uu;
  return 1;
}

/* one item of a warp's 32-item window with its halo's hot fields (shared memory) */
struct CacheEnt {
  RingItem it;
  HotHalo h;
};

/* one candidate pixel (the k-th of item it, halo fields H): decision (exact or mixed)
   and deposit at map pixel pix */
template <int EXACT, int ACC>
__device__ __forceinline__ void paint_pixel(const PaintParams &P, const SweepBuffers &W,
                                            const RingItem &it, const HotHalo &H, int k,
                                            long long pix, unsigned int &nupd,
                                            unsigned int &nrc, PendingDeposit *pend = nullptr) {
  int ir = 0;
  float fr = 0.0f, u = 0.0f;
  bool zero_val = hot_zero(H);
  int d;
  if (EXACT) {
    d = 2;
  } else {
    d = fast_decide(P, it, H, k, ir, fr, zero_val, u);
    if (P.flags & 8) { /* validation: compare every fast decision with the exact path */
      ExactRes e = exact_eval(P, W.halos[it.halo], pix);
      atomicAdd(&W.ctr->val_checked, 1ull);
      if (d != 2) {
        if ((d == 1) != e.inside) atomicAdd(&W.ctr->val_bad_set, 1ull);
        else if (d == 1 && e.inside && !e.zero && !zero_val) {
          if (e.ir != ir) atomicAdd(&W.ctr->val_bad_index, 1ull);
          if (u >= 0.0f) atomicMax(&W.ctr->val_max_du, __float_as_uint(fabsf(u - e.u)));
        }
      }
    }
  }
  if (d == 0) return;
  if (d == 2) {
    if (!EXACT) nrc++;
    ExactRes e = exact_eval(P, W.halos[it.halo], pix);
    if (!e.inside) return;
    zero_val = e.zero;
    ir = e.ir;
    fr = e.fr;
  }
  nupd++;
  if (P.flags & 1)
    record_set(W.set_rec, W.set_pix, W.set_cap, &W.ctr->n_sets, W.halos[it.halo].rec, pix);
  if (zero_val || hot_zero(H)) return;
  /* the halo's cone selects its copy of the maps (always 0 outside ensembles) */
  const long long slot = pix + (long long)hot_cone(H) * P.cone_npix;
  if (!EXACT && ACC == 2 && pend && P.nmaps <= 2 && fast_corners(P, H, ir)) {
    /* one or two maps: the values from pair table 0, the adds issued now and their
       TwoSum finished one round of candidates later */
    float v0, v1;
    pair_values(P.pair_tab[0], H, ir, fr, map_weight(P, H, 0), map_weight(P, H, 1),
                P.nmaps == 2, v0, v1);
    pend->slot = slot;
    pend->v0 = v0;
    pend->v1 = v1;
    pend->o0 = v0 != 0.0f ? atomicAdd(W.out[0] + slot, v0) : 0.0f;
    pend->o1 = v1 != 0.0f ? atomicAdd(W.out[1] + slot, v1) : 0.0f;
  } else {
    deposit_maps<ACC>(P, H, W.acc, slot, ir, fr, &W);
  }
}

/* loads items g0..g0+31 (below ihi) and their halos' hot fields into the warp's cache */
__device__ __forceinline__ void fill_cache(const SweepBuffers &W, CacheEnt *cache, long long g0,
                                           long long ihi) {
  const int lane = threadIdx.x & 31;
  __syncwarp();
  long long g = g0 + lane;
  if (g < ihi) {
    RingItem it = W.items[g];
    cache[lane].it = it;
    cache[lane].h = hot_of(W.halos[it.halo]);
  }
  __syncwarp();
}

/* map pixel of the k-th candidate of item it */
__device__ __forceinline__ long long item_pixel(const PaintParams &P, const RingItem &it, int k) {
  int npr, kshift;
  long long npn;
  p2m_ring_info(P.nside, item_ring(it), &npr, &kshift, &npn);
  int iphi = it.lo + k;
  if (iphi < 0) iphi += npr;
  if (iphi >= npr) iphi -= npr;
  return npn - npr + iphi;
}

/* walk candidates [p0, p1) of items [0, ihi): one warp; EXACT 1 decides every candidate
   by the exact path, EXACT 0 by the mixed-precision path.  The 32 items around the
   current candidates, with their halos' fields, sit in the warp's shared-memory cache,
   loaded once per window. */
template <int EXACT, int ACC>
__device__ void walk_candidates(const PaintParams &P, const SweepBuffers &W, long long p0,
                                long long p1, long long ihi, unsigned int &nupd,
                                unsigned int &nrc, CacheEnt *cache) {
  const int lane = threadIdx.x & 31;
  const long long *off = W.pix_off;
  long long g0 = warp_upper(off, 0, ihi, p0);
  long long woff = (g0 + lane < ihi) ? off[g0 + lane] : (1LL << 62);
  long long wend = (g0 + 32 < ihi) ? off[g0 + 32] : (1LL << 62);
  fill_cache(W, cache, g0, ihi);
  for (long long base = p0; base < p1; base += 32) {
    long long p = base + lane;
    bool todo = p < p1;
    /* every round serves at least the lowest pending lane: <= 32 rounds */
    for (int round = 0; __any_sync(FULL, todo); round++) {
      if (round >= 64) {
        atomicOr(&W.ctr->err, (unsigned)P2M_DEVERR_ITEMS);
        return;
      }
      long long pmin = todo ? p : (1LL << 62);
      for (int o = 16; o > 0; o >>= 1) pmin = min(pmin, __shfl_xor_sync(FULL, pmin, o));
      unsigned m = __ballot_sync(FULL, woff <= pmin);
      int j0 = m ? 31 - __clz(m) : -1;
      if (j0 != 0 || pmin >= wend) {
        if (j0 < 0 || pmin >= wend) g0 = warp_upper(off, 0, ihi, pmin);
        else g0 += j0;
        woff = (g0 + lane < ihi) ? off[g0 + lane] : (1LL << 62);
        wend = (g0 + 32 < ihi) ? off[g0 + 32] : (1LL << 62);
        fill_cache(W, cache, g0, ihi);
      }
      bool here = todo && p < wend;
      int j = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        long long o = __shfl_sync(FULL, woff, j + step);
        if (o <= p) j += step;
      }
      long long ooff = __shfl_sync(FULL, woff, j);
      if (here) {
        todo = false;
        const CacheEnt &ce = cache[j];
        int k = (int)(p - ooff);
        paint_pixel<EXACT, ACC>(P, W, ce.it, ce.h, k, item_pixel(P, ce.it, k), nupd, nrc);
      }
    }
  }
}

/* the large halos' items: every warp walks 1024-candidate chunks of their candidate
   space.  EXACT 1 is the plain FP64 path, EXACT 0 the mixed path; ACC 0 deposits into the
   FP64 accumulator, ACC 2 into the maps with compensation. */
template <int EXACT, int ACC>
__global__ void __launch_bounds__(256) k_paint_full(PaintParams P, SweepBuffers W) {
  __shared__ CacheEnt s_cache[8][32];
  const long long npix_c = (long long)W.ctr->n_pix;
  if (npix_c == 0) return;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long chunk = P.full_chunk;
  CacheEnt *cache = s_cache[(threadIdx.x >> 5) & 7];
  unsigned int nupd = 0, nrc = 0;
  unsigned long long ncand = 0;
  for (long long c = warp; c * chunk < npix_c; c += nwarps) {
    long long p0 = c * chunk, p1 = min(npix_c, p0 + chunk);
    walk_candidates<EXACT, ACC>(P, W, p0, p1, W.n_items, nupd, nrc, cache);
    if ((threadIdx.x & 31) == 0) ncand += (unsigned long long)(p1 - p0);
  }
  warp_count(&W.ctr->hp_updates, nupd);
  warp_count(&W.ctr->n_recheck, nrc);
  warp_count(&W.ctr->n_cand, ncand);
}

#ifndef P2M_HALOS_CARVEOUT
/* percent of the SM's unified L1/shared memory preferred as shared: enough for eight
   blocks' 17 KB stages, the rest stays L1 for the table and halo-record loads (measured
   on GB300: the same paint time at 60 % and 70 %, 3 % slower at 50 %, 16 % slower at
   100 %) */
#define P2M_HALOS_CARVEOUT 60
#endif
#ifndef P2M_PEND_DEPTH
#define P2M_PEND_DEPTH 1 /* rounds of candidates whose atomics are in flight before their
                            TwoSum is finished (compensated path) */
#endif
/* Threads per block of k_paint_halos: 128 or 256 (p2m_tuning.halos_threads, default
   128).  The register budget allows 32 resident warps either way (8 blocks of 128 or 4
   of 256 threads, at 64 registers): 128-thread blocks measured 6 % faster painting than
   24 warps of 256-thread blocks at 80 registers, although the 64-register build spills
   a few words. */
template <int THREADS>
struct HalosBlocks {
  static constexpr int min_blocks = 1024 / THREADS; /* 32 warps (1024 threads) per SM */
};

/* per-warp shared-memory stage of the fused painter: the disc geometry and
   interpolation fields of the warp's batch of halos, and the 32 (halo, ring) items of the
   current round (structure of arrays: lanes reading different entries hit different
   banks) */
struct WarpStage {
  HotHalo hot[32];
  int hidx[32]; /* index of the staged halo in W.halos */
  float gzh[32], gzl[32], gsh[32], gsl[32], gph[32], gpl[32], gcs[32];
  int girlo[32];
  float iA[32], iB[32], if0[32], ihd[32];
  float iAl[32], iBl[32], if0l[32], ihdl[32];
  int ilo[32], in0[32], inpr[32], ij[32];
  long long irb[32]; /* RING index of the item ring's first pixel */
};

/* Enumeration fused with painting for the halos spanning at most big_rings rings.
   A warp claims a batch of halo_batch halos (consecutive in painting order), stages
   their fields and prefix-sums their ring counts; each lane builds the candidate span
   of one (halo, ring) item and stages it;
   the warp prefix-sums the spans and paints their candidates 32 at a time, each lane
   finding its item with a 32-wide search.  Nothing goes to global memory between the
   stages. */
template <int EXACT, int ACC, int THREADS>
__global__ void __launch_bounds__(THREADS, HalosBlocks<THREADS>::min_blocks)
    k_paint_halos(PaintParams P, SweepBuffers W) {
  __shared__ WarpStage s_stage[THREADS / 32];
  const int lane = threadIdx.x & 31;
  WarpStage &S = s_stage[threadIdx.x >> 5];
  const long long nh = W.n_halos;
  unsigned int nupd = 0, nrc = 0;
  unsigned long long ncand = 0;
  PendingDeposit pend[P2M_PEND_DEPTH];
#pragma unroll
  for (int q = 0; q < P2M_PEND_DEPTH; q++) {
    pend[q].slot = -1;
    pend[q].v0 = pend[q].v1 = pend[q].o0 = pend[q].o1 = 0.0f;
  }
  const int batch = P.halo_batch;
  for (;;) {
    long long h0 = 0;
    if (lane == 0) h0 = (long long)batch * (long long)atomicAdd(&W.ctr->next_unit, 1u);
    h0 = __shfl_sync(FULL, h0, 0);
    if (h0 >= nh) break;
    int nr = 0;
    __syncwarp();
    if (lane < batch && h0 + lane < nh) {
      const int hi = W.order ? W.order[h0 + lane] : (int)(h0 + lane);
      S.hidx[lane] = hi;
      const HaloRec &H = W.halos[hi];
      int r = H.ir_hi - H.ir_lo + 1;
      if (r > 0 && r <= P.big_rings) {
        nr = r;
        S.gzh[lane] = H.z0h;
        S.gzl[lane] = H.z0l;
        S.gsh[lane] = H.s0h;
        S.gsl[lane] = H.s0l;
        S.gph[lane] = H.p0h;
        S.gpl[lane] = H.p0l;
        S.gcs[lane] = H.C_span;
        S.girlo[lane] = H.ir_lo;
        S.hot[lane] = hot_of(H);
      }
    }
    const int rx = warp_incl_scan(nr);
    const int rel = rx - nr, total = __shfl_sync(FULL, rx, 31);
    for (int t0 = 0; t0 < total; t0 += 32) {
      /* item t of the batch: ring t - rel_j of halo lane j */
      const int t = t0 + lane;
      const int j = warp_find(rel, t);
      const int relj = __shfl_sync(FULL, rel, j);
      int cnt = 0;
      __syncwarp(); /* the stage's halos are written; the previous round's items are read */
      if (t < total) {
        DiscGeom g;
        g.zh = S.gzh[j];
        g.zl = S.gzl[j];
        g.sh = S.gsh[j];
        g.sl = S.gsl[j];
        g.ph = S.gph[j];
        g.pl = S.gpl[j];
        g.cspan = S.gcs[j];
        const int ring = S.girlo[j] + (t - relj);
        const RingItem it = make_item(P, g, 0, ring);
        int npr, ks;
        long long npn;
        p2m_ring_info(P.nside, ring, &npr, &ks, &npn);
        S.iA[lane] = it.A;
        S.iB[lane] = it.B;
        S.iAl[lane] = it.Al;
        S.iBl[lane] = it.Bl;
        S.if0l[lane] = it.f0l;
        S.ihdl[lane] = it.hdl;
        S.if0[lane] = it.f0;
        S.ihd[lane] = it.hdphi;
        S.ilo[lane] = it.lo;
        S.in0[lane] = it.ring_n0 & 0xffff;
        S.inpr[lane] = npr;
        S.ij[lane] = j;
        S.irb[lane] = npn - npr;
        cnt = it.count;
      }
      __syncwarp();
      const int cx = warp_incl_scan(cnt);
      const int cex = cx - cnt, ctot = __shfl_sync(FULL, cx, 31);
      for (int c0 = 0; c0 < ctot; c0 += 32) {
        const int c = c0 + lane;
        const int i = warp_find(cex, c);
        const int k = c - __shfl_sync(FULL, cex, i);
        PendingDeposit nd;
        nd.slot = -1;
        nd.v0 = nd.v1 = nd.o0 = nd.o1 = 0.0f;
        if (c < ctot) {
          RingItem ci;
          const int jj = S.ij[i];
          ci.halo = S.hidx[jj];
          ci.ring_n0 = S.in0[i];
          ci.lo = S.ilo[i];
          ci.count = 0;
          ci.A = S.iA[i];
          ci.B = S.iB[i];
          ci.Al = S.iAl[i];
          ci.Bl = S.iBl[i];
          ci.f0l = S.if0l[i];
          ci.hdl = S.ihdl[i];
          ci.f0 = S.if0[i];
          ci.hdphi = S.ihd[i];
          const int np = S.inpr[i];
          int iphi = ci.lo + k;
          if (iphi < 0) iphi += np;
          if (iphi >= np) iphi -= np;
          paint_pixel<EXACT, ACC>(P, W, ci, S.hot[jj], k, S.irb[i] + iphi, nupd, nrc,
                                  ACC == 2 ? &nd : nullptr);
        }
        if (ACC == 2) {
          /* the oldest round's adds have returned by now */
          finish_pending(W, pend[0]);
#pragma unroll
          for (int q = 0; q + 1 < P2M_PEND_DEPTH; q++) pend[q] = pend[q + 1];
          pend[P2M_PEND_DEPTH - 1] = nd;
        }
      }
      if (lane == 0) ncand += (unsigned long long)ctot;
    }
  }
  if (ACC == 2) {
#pragma unroll
    for (int q = 0; q < P2M_PEND_DEPTH; q++) finish_pending(W, pend[q]);
  }
  warp_count(&W.ctr->hp_updates, nupd);
  warp_count(&W.ctr->n_recheck, nrc);
  warp_count(&W.ctr->n_cand, ncand);
}

/* pair table of two maps: entry e = (table a's profile pa value, table b's profile pb
   value) at float2 index e of the (profile 1, profile 2) interleaved tables, for the
   nent = nelem / 2 (ir, imh, ichi) entries */
__global__ void __launch_bounds__(256) k_pair_table(float2 *__restrict__ dst,
                                                    const float *__restrict__ ta, int pa,
                                                    const float *__restrict__ tb, int pb,
                                                    long long nent) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nent;
       e += (long long)gridDim.x * blockDim.x)
    dst[e] = make_float2(ta[2 * e + (pa - 1)], tb[2 * e + (pb - 1)]);
}

void p2m_launch_pair_table(float2 *dst, const float *ta, int pa, const float *tb, int pb,
                           long long nent, cudaStream_t s, int nsm) {
  const long long need = (nent + 255) / 256;
  const int grid = (int)std::max(1LL, std::min(need, (long long)nsm * 8));
  k_pair_table<<<grid, 256, 0, s>>>(dst, ta, pa, tb, pb, nent);
}

/* candidate counts of items (input of the candidate-offset scan) */
__global__ void __launch_bounds__(256) k_item_counts(const RingItem *items, long long n,
                                                     unsigned int *counts) {
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < n;
       g += (long long)gridDim.x * blockDim.x)
    counts[g] = (unsigned)items[g].count;
}

/* FP64 accumulator -> float maps in one pass over all maps (added to the maps after the
   first sweep since the reset).  The accumulator is only read here: the caller clears it
   afterwards with a memset, because overwriting the lines that a pass has just read runs
   at a fraction of the HBM rate of a read pass followed by a separate clear (measured on
   GB300: 1.0 TB/s against 6.8 TB/s + a 7.7 TB/s memset) */
template <int FIXED>
__device__ __forceinline__ float2 acc_pair(const double *acc, long long p) {
  if (FIXED) {
    const longlong2 q = __ldcs((const longlong2 *)acc + p);
    return make_float2(fixed_to_float(q.x), fixed_to_float(q.y));
  }
  const double2 d = __ldcs((const double2 *)acc + p);
  return make_float2((float)d.x, (float)d.y);
}
template <int FIXED>
__device__ __forceinline__ float acc_one(const double *acc, long long i) {
  if (FIXED) return fixed_to_float(__ldcs((const long long *)acc + i));
  return (float)__ldcs(acc + i);
}

/* FIXED 1: the accumulator holds 64-bit fixed-point sums (unit 2^-56) */
template <int FIXED>
__global__ void __launch_bounds__(256) k_finalize_full(const double *acc, long long npix, int nmaps,
                                                       float *o0, float *o1, float *o2, float *o3,
                                                       float *o4, float *o5, float *o6, float *o7,
                                                       int accumulate) {
  float *outs[8] = {o0, o1, o2, o3, o4, o5, o6, o7};
  const long long stride = (long long)gridDim.x * blockDim.x;
  if (nmaps == 2) {
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += 4 * stride) {
      float2 a[4];
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (p + u * stride < npix) a[u] = acc_pair<FIXED>(acc, p + u * stride);
#pragma unroll
      for (int u = 0; u < 4; u++) {
        long long q = p + u * stride;
        if (q >= npix) break;
        float v0 = a[u].x, v1 = a[u].y;
        if (accumulate) {
          v0 = __fadd_rn(o0[q], v0);
          v1 = __fadd_rn(o1[q], v1);
        }
        __stcs(o0 + q, v0);
        __stcs(o1 + q, v1);
      }
    }
  } else {
    /* any other map count: the block moves 256 pixels' interleaved accumulators at a time
       through shared memory, so that the reads are linear over whole sectors and every
       thread has up to P2M_MAXMAPS loads in flight */
    __shared__ float sv[256 * P2M_MAXMAPS];
    const int t = threadIdx.x;
    for (long long base = (long long)blockIdx.x * 256; base < npix; base += (long long)gridDim.x * 256) {
      const int np = (int)(npix - base < 256 ? npix - base : 256);
      const int n = np * nmaps;
      const double *a = acc + base * nmaps;
      float r[P2M_MAXMAPS];
#pragma unroll
      for (int k = 0; k < P2M_MAXMAPS; k++)
        if (t + k * 256 < n) r[k] = acc_one<FIXED>(a, t + k * 256);
#pragma unroll
      for (int k = 0; k < P2M_MAXMAPS; k++)
        if (t + k * 256 < n) sv[t + k * 256] = r[k];
      __syncthreads();
      if (t < np)
        for (int m = 0; m < nmaps; m++) {
          float v = sv[t * nmaps + m];
          if (accumulate) v = __fadd_rn(outs[m][base + t], v);
          __stcs(outs[m] + base + t, v);
        }
      __syncthreads();
    }
  }
}

/* folds the nonzero low words of the compensated accumulation into the output maps
   (out = RN(hi + lo)) and clears them.  A warp reads the flags of 32 consecutive tiles
   and visits the flagged ones (one pixel per lane), up to four tiles with all their loads
   in flight at once for the usual two maps */
#ifndef P2M_FOLD_MINBLOCKS
/* 4 resident blocks per SM (64 registers, no spills) keep more tiles' loads in flight than
   the 3 that 80 registers allow: fold 0.136 ms instead of 0.153 ms at Nside 4096 */
#define P2M_FOLD_MINBLOCKS 4
#endif
__global__ void __launch_bounds__(256, P2M_FOLD_MINBLOCKS) k_fold_lo(SweepBuffers W, int nmaps) {
  const int lane = threadIdx.x & 31;
  const long long ntiles = (W.npix + P2M_TILE_PIX - 1) >> P2M_TILE_SHIFT;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long t0 = warp * 32; t0 < ntiles; t0 += nwarps * 32) {
    long long t = t0 + lane;
    bool dirty = t < ntiles && W.tiles[t];
    unsigned m = __ballot_sync(FULL, dirty);
    if (dirty) W.tiles[t] = 0;
    if (nmaps == 2) {
      float *lo0 = W.lo, *lo1 = W.lo + W.npix, *o0 = W.out[0], *o1 = W.out[1];
      while (m) {
        long long p[4];
        int cnt = 0;
#pragma unroll
        for (int u = 0; u < 4; u++) {
          p[u] = -1;
          if (m) {
            int b = __ffs(m) - 1;
            m &= m - 1;
            long long q = ((t0 + b) << P2M_TILE_SHIFT) + lane;
            p[u] = q < W.npix ? q : -1;
            cnt++;
          }
        }
        float l0[4], l1[4], h0[4], h1[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (u < cnt && p[u] >= 0) {
            l0[u] = lo0[p[u]];
            l1[u] = lo1[p[u]];
            h0[u] = o0[p[u]];
            h1[u] = o1[p[u]];
          }
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (u < cnt && p[u] >= 0) {
            if (l0[u] != 0.0f) {
              o0[p[u]] = __fadd_rn(h0[u], l0[u]);
              lo0[p[u]] = 0.0f;
            }
            if (l1[u] != 0.0f) {
              o1[p[u]] = __fadd_rn(h1[u], l1[u]);
              lo1[p[u]] = 0.0f;
            }
          }
      }
      continue;
    }
    while (m) {
      int b = __ffs(m) - 1;
      m &= m - 1;
      long long p = ((t0 + b) << P2M_TILE_SHIFT) + lane;
      if (p >= W.npix) continue;
      float l[P2M_MAXMAPS], h[P2M_MAXMAPS];
#pragma unroll
      for (int mp = 0; mp < P2M_MAXMAPS; mp++)
        if (mp < nmaps) l[mp] = W.lo[(long long)mp * W.npix + p];
#pragma unroll
      for (int mp = 0; mp < P2M_MAXMAPS; mp++)
        if (mp < nmaps && l[mp] != 0.0f) h[mp] = W.out[mp][p];
#pragma unroll
      for (int mp = 0; mp < P2M_MAXMAPS; mp++)
        if (mp < nmaps && l[mp] != 0.0f) {
          W.out[mp][p] = __fadd_rn(h[mp], l[mp]);
          W.lo[(long long)mp * W.npix + p] = 0.0f;
        }
    }
  }
}

/* sum over a float map: float-float (TwoSum) accumulation per thread, FP64 only for the
   per-thread totals (FP64 adds run at a small fraction of the FP32 rate here) */
__global__ void __launch_bounds__(256) k_map_sum(const float *map, long long n, double *sum) {
  float hi = 0.0f, lo = 0.0f;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const float x = map[p];
    const float sm = __fadd_rn(hi, x);
    const float bb = __fsub_rn(sm, hi);
    lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(sm, bb)), __fsub_rn(x, bb)));
    hi = sm;
  }
  double s = (double)hi + (double)lo;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(FULL, s, o);
  if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(sum, s);
}

/* The statistics of pks2map.f90:321-346 over one float map, in one pass: sums of x, x^2
   and x^3 (float-float per thread: x^2 by an exact two-product, x^3 as its float-float
   product with x; FP64 only for the per-thread totals) and, with hist, the counts of the
   P(<y) bins: m = int(x / dy) + 1 in float (:344), counted where 1 <= m <= nbins (:345).
   The bins' counters are in shared memory; lanes of a warp that fall in the same bin
   (most pixels of a y map are in bin 1) are added once by the lowest of them. */
#define P2M_STATS_THREADS 512
__global__ void __launch_bounds__(P2M_STATS_THREADS) k_map_stats(const float *map, long long n,
                                                                double *sums,
                                                                unsigned int *hist, int nbins,
                                                                float dy) {
  extern __shared__ unsigned int s_hist[];
  if (hist)
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) s_hist[b] = 0u;
  __syncthreads();
  ffloat s1 = {0.0f, 0.0f}, s2 = {0.0f, 0.0f}, s3 = {0.0f, 0.0f};
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += stride) {
    const long long p = base + threadIdx.x;
    const bool in = p < n;
    const float x = in ? map[p] : 0.0f;
    if (x != 0.0f) {
      const float q2 = __fmul_rn(x, x);
      const ffloat x2 = {q2, __fmaf_rn(x, x, -q2)};
      s1 = ff_add_f(s1, x);
      s2 = ff_add(s2, x2);
      s3 = ff_add(s3, ff_mul_f(x2, x));
    }
    if (hist) {
      int m = 0;
      if (in) {
        const float q = __fdiv_rn(x, dy);
        if (q > -1.0f && q < (float)nbins) m = (int)q + 1;
      }
      const unsigned same = __match_any_sync(FULL, m);
      if (m > 0 && lane == __ffs(same) - 1) atomicAdd(&s_hist[m - 1], (unsigned)__popc(same));
    }
  }
  double d[3] = {(double)s1.h + (double)s1.l, (double)s2.h + (double)s2.l,
                 (double)s3.h + (double)s3.l};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    for (int o = 16; o > 0; o >>= 1) d[k] += __shfl_down_sync(FULL, d[k], o);
    if (lane == 0 && d[k] != 0.0) atomicAdd(&sums[k], d[k]);
  }
  if (hist) {
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x)
      if (s_hist[b]) atomicAdd(&hist[b], s_hist[b]);
  }
}

/* flat-sky accumulator -> float map */
template <int PREC>
__global__ void __launch_bounds__(256) k_finalize_fs(const void *acc, long long npix, int nmaps, int map,
                                                     float *out, double *sum) {
  double s = 0.0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix;
       p += (long long)gridDim.x * blockDim.x) {
    float v;
    if (PREC == 0) {
      v = (float)((const double *)acc)[p * nmaps + map];
    } else if (PREC == 3) {
      v = fixed_to_float(((const long long *)acc)[p * nmaps + map]);
    } else {
      float2 a = ((const float2 *)acc)[p * nmaps + map];
      v = __fadd_rn(a.x, a.y);
    }
    out[p] = v;
    s += (double)v;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(FULL, s, o);
  if ((threadIdx.x & 31) == 0 && s != 0.0 && sum) atomicAdd(sum, s);
}

/* -------------------------------------------------------------- table maker ----- */

/* bbps_profile.f90:9-55 parameters, model-major */
__constant__ float c_bbps[18][3] = {
    {18.100f, 7.490f, 20.7f},       {0.154f, 0.226f, -0.074f},      {-0.758f, -0.957f, -0.743f},
    {0.497f, 0.710f, 0.438f},       {-0.00865f, -0.0833f, 0.011f},  {0.731f, 0.853f, 1.01f},
    {4.35f, 4.19f, 3.82f},          {0.0393f, 0.048f, 0.0375f},     {0.415f, 0.615f, 0.535f},
    {1.9e-5f, 9.1e-05f, 1.5e-4f},   {0.29f, 0.10f, 0.14f},          {-0.67f, -0.92f, -1.32f},
    {0.88f, 0.69f, 0.68f},          {-0.03f, -0.02f, -0.02f},       {0.20f, 0.27f, 0.29f},
    {3.83f, 4.43f, 6.4f},           {0.044f, 0.0035f, 0.028f},      {-0.025f, 0.037f, -0.25f}};

__device__ float bbps_scale(int row, int i, float mh, float z) {
  return FMUL(FMUL(c_bbps[row][i], p2m_powf(FDIV(mh, 1e14f), c_bbps[row + 1][i])),
              p2m_powf(FADD(1.0f, z), c_bbps[row + 2][i]));
}

/* integrate_profiles.f90:12-95 (which = 1: pressure, 2: gas density) */
__device__ float integrate_profile(const PaintParams &P, int model, int which, float theta,
                                   float z, float mh) {
  int i = model - 1;
  const float rmax = 4.0f, ds = 1e-2f;
  float Delta = (i == 1) ? 500.0f : 200.0f;
  float chi = p2m_lookup(P.rofz, P.cosmo.drofz, z);
  double t = DDIV((double)FDIV(FMUL(3.0f, mh), 4.0f), P2M_COSMO_PI);
  t = DDIV(t, (double)Delta);
  t = DDIV(t, (double)p2m_rhocrit(&P.cosmo, z));
  float rvir = (float)pow(t, (double)0.333333343f);
  float b = FDIV(FMUL(chi, p2m_sinf(theta)), rvir);
  if (b > rmax) return 0.0f;
  if (which == 1) {
    float P0 = bbps_scale(0, i, mh, z), xc = bbps_scale(3, i, mh, z), beta = bbps_scale(6, i, mh, z);
    int n = (int)FDIV(rmax, ds) + 1;
    float y = 0.0f;
    for (int k = 1; k <= n; k++) {
      float s = FMUL(FSUB((float)k, 0.5f), ds);
      float x = FSQRT(FADD(FMUL(s, s), FMUL(b, b)));
      float xx = FDIV(x, xc);
      float pt = FMUL(FMUL(P0, p2m_powf(xx, -0.3f)),
                      p2m_powf(FADD(1.0f, p2m_powf(xx, 1.0f)), -beta));
      y = FADD(y, pt);
    }
    return FMUL(y, ds);
  } else {
    float P0 = bbps_scale(9, i, mh, z), ar = bbps_scale(12, i, mh, z), beta = bbps_scale(15, i, mh, z);
    float s0 = FSQRT(FSUB(FMUL(rmax, rmax), FMUL(b, b)));
    int n = (int)FDIV(s0, ds) + 1;
    float e1 = FMUL(-1.0f, 0.2f);
    float e2 = FDIV(FMUL(-1.0f, FSUB(beta, 0.2f)), ar);
    float rho = 0.0f;
    for (int k = 1; k <= n; k++) {
      float s = FMUL(FSUB((float)k, 0.5f), ds);
      float x = FSQRT(FADD(FMUL(s, s), FMUL(b, b)));
      float xx = FDIV(x, 0.5f);
      float rt = FMUL(FMUL(P0, p2m_powf(xx, e1)), p2m_powf(FADD(1.0f, p2m_powf(xx, ar)), e2));
      rho = FADD(rho, rt);
    }
    rho = FMUL(rho, ds);
    return FMUL(2.0f, rho);
  }
}

/* maptable.f90:99-140, one thread per (chi, M, r) entry */
__global__ void __launch_bounds__(128) k_maptable(PaintParams P, TableConsts K, p2m_tabhdr th,
                                                  float *table) {
  long long n = (long long)th.nchit * th.nmht * th.nrt;
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int k = (int)(e % th.nrt) + 1;
  int j = (int)((e / th.nrt) % th.nmht) + 1;
  int i = (int)(e / ((long long)th.nrt * th.nmht)) + 1;
  float chit = p2m_expf(FADD(p2m_logf(th.chimint), FMUL((float)(i - 1), th.dchit)));
  float z = p2m_lookup(P.zofr, P.cosmo.dzofr, chit);
  float zp1 = FADD(1.0f, z);
  float zfacy = FADD(FMUL(P.cosmo.omegam, FMUL(FMUL(zp1, zp1), zp1)), P.cosmo.omegal);
  float zfact = FDIV(FDIV(1.0f, zp1), p2m_powf(p2m_rhocrit(&P.cosmo, z), 0.333333343f));
  float Gx = 0.0f;
  if (K.nu > 0.0f) {
    float x0new = FMUL(K.x0const, p2m_powf(zp1, K.alpha));
    float ex = p2m_expf(x0new);
    Gx = FSUB(FDIV(FMUL(x0new, FADD(ex, 1.0f)), FSUB(ex, 1.0f)), 4.0f);
  }
  float mht = p2m_expf(FADD(p2m_logf(th.mhmint), FMUL((float)(j - 1), th.dmht)));
  float mht3 = p2m_powf(mht, 0.333333343f);
  float rt = p2m_expf(FADD(p2m_logf(th.rmint), FMUL((float)(k - 1), th.drt)));
  float theta = p2m_atanf(FDIV(rt, chit));
  float y = FMUL(FMUL(FMUL(K.y0, mht), zfacy), integrate_profile(P, K.model, 1, theta, z, mht));
  if (K.nu > 0.0f) y = FMUL(y, Gx);
  float tau = FMUL(FMUL(FMUL(K.tau0, mht3), zfact), integrate_profile(P, K.model, 2, theta, z, mht));
  long long off = 2LL * ((long long)(k - 1) + (long long)th.nrt * ((long long)(j - 1) + (long long)th.nmht * (i - 1)));
  table[off] = y;
  table[off + 1] = tau;
}

/* ------------------------------------------------------------- math self-test ----- */

__global__ void k_fmath_eval(int fn, const float *x, const float *y, float *out, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float a = x[i], b = y ? y[i] : 0.0f, r;
  switch (fn) {
    case 0: r = p2m_logf(a); break;
    case 1: r = p2m_expf(a); break;
    case 2: r = p2m_powf(a, b); break;
    case 3: r = p2m_asinf(a); break;
    case 4: r = p2m_atanf(a); break;
    case 5: r = p2m_sinf(a); break;
    case 6: r = p2m_cosf(a); break;
    case 8: r = fixed_to_float(float_to_fixed(a) + float_to_fixed(b)); break;
    case 9: r = p2m_tanf_pio4(a); break;
    case 10: r = p2m_logf_normal(a); break;
    default: r = p2m_tanf(a); break;
  }
  out[i] = r;
}

extern "C" int32_t p2m_fmath_eval_device(int32_t device, int32_t fn, const float *d_x,
                                         const float *d_y, float *d_out, int64_t n) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return (int32_t)e;
  if (n > 0) k_fmath_eval<<<(unsigned)((n + 255) / 256), 256>>>(fn, d_x, d_y, d_out, n);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return (int32_t)e;
}

/* ---------------------------------------------------------------- launchers ----- */

static inline int grid_for(long long n, int block, int nsm, int per_sm) {
  long long g = (n + block - 1) / block;
  long long cap = (long long)nsm * per_sm;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

/* radial-cut flags of the records (input of the survivor-ordinal scan) */
__global__ void __launch_bounds__(256) k_pre_flags(PaintParams P, const float *records, long long n,
                                                   unsigned int *flags) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    flags[i] = in_shell(P, records + i * P.nfloat) ? 1u : 0u;
}

/* centre (pks2map.f90:191-210): the largest RTH among the survivors, then per rank the
   last survivor holding it */
__global__ void __launch_bounds__(256) k_pre_rthmax(PaintParams P, const float *records, long long n,
                                                    const unsigned int *flags, unsigned int *bits) {
  unsigned int mx = 0u;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float rth = records[i * P.nfloat + 6];
    if (flags[i] && rth > 0.0f) mx = max(mx, __float_as_uint(rth));
  }
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(FULL, mx, o));
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(bits, mx);
}
__global__ void __launch_bounds__(256) k_pre_last(PaintParams P, const float *records, long long n,
                                                  const unsigned int *flags,
                                                  const unsigned int *bits, long long *last) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    if (flags[i] && __float_as_uint(records[i * P.nfloat + 6]) == *bits)
      atomicMax(&last[i / P.pre.per_rank], i); /* signed: the slots start at -1 */
}

void p2m_launch_pre_flags(const PaintParams &P, const float *records, long long n,
                          unsigned int *flags, cudaStream_t s, int nsm) {
  k_pre_flags<<<grid_for(n, 256, nsm, 8), 256, 0, s>>>(P, records, n, flags);
}
void p2m_launch_pre_centre(const PaintParams &P, const float *records, long long n,
                           const unsigned int *flags, unsigned int *rthmax_bits,
                           long long *last, cudaStream_t s, int nsm) {
  k_pre_rthmax<<<grid_for(n, 256, nsm, 8), 256, 0, s>>>(P, records, n, flags, rthmax_bits);
  k_pre_last<<<grid_for(n, 256, nsm, 8), 256, 0, s>>>(P, records, n, flags, rthmax_bits, last);
}

#ifndef P2M_CUT_CARVEOUT
#define P2M_CUT_CARVEOUT -1 /* shared-memory carveout preference (percent; -1: left to the
                               CUDA runtime's choice) */
#endif
#ifndef P2M_FULL_CARVEOUT
#define P2M_FULL_CARVEOUT -1
#endif
/* sets a kernel's shared-memory carveout once per device (a bit per device ordinal;
   contexts on several host threads may race to set it, which is harmless) */
template <class K>
static void carveout_once(K kernel, int percent, std::atomic<unsigned long long> &done) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  const unsigned long long bit = 1ull << (dev & 63);
  if (done.load(std::memory_order_relaxed) & bit) return;
  if (percent >= 0)
    cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, percent);
  done.fetch_or(bit, std::memory_order_relaxed);
}

void p2m_launch_cut_setup(const PaintParams &P, const IngestBuffers &B, long long n,
                          cudaStream_t s, int nsm) {
  static std::atomic<unsigned long long> co{0};
  carveout_once(k_cut_setup, P2M_CUT_CARVEOUT, co);
  /* one resident wave: each block streams its tiles and sets up its own survivors (the
     blocks per SM, from the occupancy calculator, kept per device ordinal) */
  static std::atomic<int> resident[64];
  int dev = 0;
  cudaGetDevice(&dev);
  int per_sm = resident[dev & 63].load(std::memory_order_relaxed);
  if (per_sm < 1) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cut_setup, 256, 0) != cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
    resident[dev & 63].store(per_sm, std::memory_order_relaxed);
  }
  long long tiles = (n + 256LL * CUT_PER_THREAD - 1) / (256LL * CUT_PER_THREAD);
  long long g = std::min<long long>(tiles, (long long)nsm * per_sm);
  k_cut_setup<<<(int)std::max<long long>(g, 1), 256, 0, s>>>(P, B, n);
}
void p2m_launch_setup_prepared(const PaintParams &P, const IngestBuffers &B, const float *prep,
                               long long n, cudaStream_t s, int nsm) {
  k_setup_prepared<<<grid_for(n, 256, nsm, 8), 256, 0, s>>>(P, B, prep, n);
}
void p2m_launch_scan_u32(const unsigned int *in, const unsigned long long *n_ptr, long long *out,
                         unsigned long long *total, long long *tmp, cudaStream_t s) {
  k_scan_partial<<<SCAN_BLOCKS, 256, 0, s>>>(in, n_ptr, tmp);
  k_scan_top<<<1, SCAN_BLOCKS, 0, s>>>(tmp, total);
  k_scan_apply<<<SCAN_BLOCKS, 256, 0, s>>>(in, n_ptr, tmp, out);
}
void p2m_launch_items(const PaintParams &P, const IngestBuffers &B, long long n_max,
                      cudaStream_t s, int nsm) {
  k_items<<<grid_for(n_max, 256, nsm, 8), 256, 0, s>>>(P, B);
}
void p2m_launch_fs(const PaintParams &P, const IngestBuffers &B, long long n_max, cudaStream_t s,
                   int nsm) {
  k_fs_emit<<<grid_for(n_max, 256, nsm, 4), 256, 0, s>>>(P, B);
  if (P.precision == 1) k_paint_fs<1><<<nsm * 8, 256, 0, s>>>(P, B);
  else if (P.precision == 3) k_paint_fs<3><<<nsm * 8, 256, 0, s>>>(P, B);
  else k_paint_fs<0><<<nsm * 8, 256, 0, s>>>(P, B);
}
void p2m_launch_paint_full(const PaintParams &P, const SweepBuffers &W, cudaStream_t s, int nsm) {
  static std::atomic<unsigned long long> co0{0}, co1{0}, co2{0}, co3{0};
  carveout_once(k_paint_full<1, 0>, P2M_FULL_CARVEOUT, co1);
  carveout_once(k_paint_full<0, 2>, P2M_FULL_CARVEOUT, co2);
  carveout_once(k_paint_full<0, 3>, P2M_FULL_CARVEOUT, co3);
  carveout_once(k_paint_full<0, 0>, P2M_FULL_CARVEOUT, co0);
  const int g = nsm * P.full_grid;
  if (P.precision == 0) k_paint_full<1, 0><<<g, 256, 0, s>>>(P, W);
  else if (P.precision == 1) k_paint_full<0, 2><<<g, 256, 0, s>>>(P, W);
  else if (P.precision == 3) k_paint_full<0, 3><<<g, 256, 0, s>>>(P, W);
  else k_paint_full<0, 0><<<g, 256, 0, s>>>(P, W);
}
template <int EXACT, int ACC, int THREADS>
static void launch_paint_halos_t(const PaintParams &P, const SweepBuffers &W, cudaStream_t s,
                                 int nsm) {
  /* the shared-memory stage (19 KB per 128 threads) must not be what limits residency,
     nor take the L1 the table loads use */
  static std::atomic<unsigned long long> co{0};
  carveout_once(k_paint_halos<EXACT, ACC, THREADS>, P2M_HALOS_CARVEOUT, co);
  /* warps claim batches of halo_batch halos until none is left */
  k_paint_halos<EXACT, ACC, THREADS><<<nsm * P.halos_grid, THREADS, 0, s>>>(P, W);
}
template <int EXACT, int ACC>
static void launch_paint_halos(const PaintParams &P, const SweepBuffers &W, cudaStream_t s,
                               int nsm) {
  if (P.halos_threads == 256) launch_paint_halos_t<EXACT, ACC, 256>(P, W, s, nsm);
  else launch_paint_halos_t<EXACT, ACC, 128>(P, W, s, nsm);
}
void p2m_launch_paint_halos(const PaintParams &P, const SweepBuffers &W, cudaStream_t s, int nsm) {
  if (P.precision == 0) launch_paint_halos<1, 0>(P, W, s, nsm);
  else if (P.precision == 1) launch_paint_halos<0, 2>(P, W, s, nsm);
  else if (P.precision == 3) launch_paint_halos<0, 3>(P, W, s, nsm);
  else launch_paint_halos<0, 0>(P, W, s, nsm);
}
void p2m_launch_item_counts(const RingItem *items, long long n, unsigned int *counts,
                            cudaStream_t s, int nsm) {
  k_item_counts<<<grid_for(n, 256, nsm, 8), 256, 0, s>>>(items, n, counts);
}
void p2m_launch_fold_lo(const PaintParams &P, const SweepBuffers &W, cudaStream_t s, int nsm) {
  k_fold_lo<<<nsm * 8, 256, 0, s>>>(W, P.nmaps);
}
__global__ void k_copy_counters(const DevCounters *__restrict__ d, DevCounters *__restrict__ h) {
  const unsigned int *src = (const unsigned int *)d;
  unsigned int *dst = (unsigned int *)h;
  for (int i = threadIdx.x; i < (int)(sizeof(DevCounters) / 4); i += blockDim.x) dst[i] = src[i];
}
__global__ void k_ring_scatter(const int *__restrict__ keys, long long n,
                               long long *__restrict__ off, int *__restrict__ order) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x) {
    const unsigned long long pos = atomicAdd((unsigned long long *)&off[keys[s]], 1ull);
    order[pos] = (int)s;
  }
}
void p2m_launch_ring_scatter(const int *keys, long long n, long long *off, int *order,
                             cudaStream_t s, int nsm) {
  k_ring_scatter<<<grid_for(n, 256, nsm, 8), 256, 0, s>>>(keys, n, off, order);
}
__global__ void k_ring_unhist(const int *__restrict__ keys, long long n,
                              unsigned int *__restrict__ hist) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x)
    atomicSub(&hist[keys[s]], 1u);
}
void p2m_launch_ring_unhist(const int *keys, long long n, unsigned int *hist, cudaStream_t s,
                            int nsm) {
  k_ring_unhist<<<grid_for(n, 256, nsm, 8), 256, 0, s>>>(keys, n, hist);
}
void p2m_launch_copy_counters(const DevCounters *d, DevCounters *h_mapped, cudaStream_t s) {
  k_copy_counters<<<1, 64, 0, s>>>(d, h_mapped);
}
void p2m_launch_map_stats(const float *map, long long n, double *sums, unsigned int *hist,
                          int nbins, float dy, cudaStream_t s, int nsm) {
  /* nbins <= 12288: the counters fit the default 48 KB of dynamic shared memory */
  const size_t smem = hist ? sizeof(unsigned int) * (size_t)nbins : 0;
  k_map_stats<<<grid_for(n, P2M_STATS_THREADS, nsm, 2), P2M_STATS_THREADS, smem, s>>>(
      map, n, sums, hist, nbins, dy);
}
/* float map -> big-endian IEEE words (the byte order of FITS data) */
__global__ void __launch_bounds__(256) k_to_big_endian(const float *__restrict__ in,
                                                       unsigned int *__restrict__ out,
                                                       long long n) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x)
    out[p] = __byte_perm(__float_as_uint(in[p]), 0u, 0x0123);
}
void p2m_launch_to_big_endian(const float *in, unsigned int *out, long long n, cudaStream_t s,
                              int nsm) {
  k_to_big_endian<<<grid_for(n, 256, nsm, 8), 256, 0, s>>>(in, out, n);
}
void p2m_launch_map_sum(const float *map, long long n, double *sum, cudaStream_t s, int nsm) {
  k_map_sum<<<grid_for(n, 256, nsm, 8), 256, 0, s>>>(map, n, sum);
}
void p2m_launch_finalize_full(const PaintParams &P, const void *acc, long long npix,
                              float *const *out, int accumulate, cudaStream_t s, int nsm) {
  const int g = grid_for(npix, 256, nsm, 8);
  if (P.precision == 3)
    k_finalize_full<1><<<g, 256, 0, s>>>((const double *)acc, npix, P.nmaps, out[0], out[1], out[2],
                                         out[3], out[4], out[5], out[6], out[7], accumulate);
  else
    k_finalize_full<0><<<g, 256, 0, s>>>((const double *)acc, npix, P.nmaps, out[0], out[1], out[2],
                                         out[3], out[4], out[5], out[6], out[7], accumulate);
}
void p2m_launch_finalize_fs(const PaintParams &P, const void *acc, long long npix, float *out,
                            int map, double *sum, cudaStream_t s, int nsm) {
  int g = grid_for(npix, 256, nsm, 8);
  if (P.precision == 1) k_finalize_fs<1><<<g, 256, 0, s>>>(acc, npix, P.nmaps, map, out, sum);
  else if (P.precision == 3) k_finalize_fs<3><<<g, 256, 0, s>>>(acc, npix, P.nmaps, map, out, sum);
  else k_finalize_fs<0><<<g, 256, 0, s>>>(acc, npix, P.nmaps, map, out, sum);
}
void p2m_launch_maptable(const PaintParams &P, const TableConsts &K, const p2m_tabhdr &th,
                         float *d_table, cudaStream_t s) {
  long long n = (long long)th.nchit * th.nmht * th.nrt;
  k_maptable<<<(int)((n + 127) / 128), 128, 0, s>>>(P, K, th, d_table);
}
