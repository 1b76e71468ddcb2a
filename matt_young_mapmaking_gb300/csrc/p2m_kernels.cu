/*
 * p2m_kernels.cu -- sm_103a kernels of the halo painter (see p2m_internal.h for the
 * pipeline).  Work is balanced at the level of candidate pixels: per-ring candidate
 * spans are prefix-summed and each warp walks a fixed-size range of the candidate
 * space, locating items with a 32-wide search in registers.  Items are ordered by
 * ring, so concurrently running warps deposit into a narrow band of the RING-ordered
 * map that stays resident in L2.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "p2m_internal.h"

#define FULL 0xffffffffu

/* ------------------------------------------------------------------ helpers ----- */

/* warp-aggregated append: all 32 lanes must call; returns slot or -1 */
__device__ __forceinline__ long long warp_append(unsigned long long *ctr, bool pred) {
  unsigned m = __ballot_sync(FULL, pred);
  int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  if (m) {
    int leader = __ffs(m) - 1;
    if (lane == leader) base = atomicAdd(ctr, (unsigned long long)__popc(m));
    base = __shfl_sync(FULL, base, leader);
  }
  if (!pred) return -1;
  return (long long)(base + __popc(m & ((1u << lane) - 1u)));
}

__device__ __forceinline__ void warp_count(unsigned long long *ctr, unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(ctr, v);
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

/* --------------------------------------------------------------------- k_cut ----- */

/* radial cut (pks2map.f90:144-160) and mass cut (:264, :296) */
__global__ void __launch_bounds__(256) k_cut(PaintParams P, PaintBuffers B, long long n) {
  long long stride = (long long)gridDim.x * blockDim.x;
  int lane = threadIdx.x & 31;
  unsigned long long nshell = 0;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n;
       base += stride) {
    long long i = base + lane;
    bool shell = false, keep = false;
    if (i < n) {
      const float *r = B.records + i * P.nfloat;
      float p0 = __ldg(r + 0), p1 = __ldg(r + 1), p2 = __ldg(r + 2), rth = __ldg(r + 6);
      if (p2m_isfinite(p0) && p2m_isfinite(p1) && p2m_isfinite(p2) && p2m_isfinite(rth)) {
        float xh = FSUB(p2, P.chihview), yh = p1, zh = p0;
        float chih = FSQRT(FADD(FADD(FMUL(xh, xh), FMUL(yh, yh)), FMUL(zh, zh)));
        shell = !(chih > P.cut_high || chih < P.cut_low);
        float mass = FMUL(P.mass_fac, FMUL(FMUL(rth, rth), rth));
        keep = shell && !(mass < 1e13f);
      }
    }
    nshell += shell;
    long long slot = warp_append(&B.ctr->n_surv, keep);
    if (keep) B.surv[slot] = (int)i;
  }
  warp_count(&B.ctr->n_shell, nshell);
}

/* ------------------------------------------------------------------- k_setup ----- */

__device__ __forceinline__ int hp_nrings(const HaloRec &H) {
  return H.ir_hi >= H.ir_lo ? H.ir_hi - H.ir_lo + 1 : 0;
}

/* geometry, thresholds and interpolation constants of one halo from its loop
   quantities (pks2map.f90:284-298 outputs).  Returns false if nothing is painted. */
__device__ bool halo_geometry(const PaintParams &P, float xh, float yh, float zh, float rh,
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
  if (hi.zero && !(P.flags & 2)) return false;
  /* corner offsets for the fast blend (all corners in range for every ir < nrt) */
  {
    long long nrt2 = 2LL * P.th.nrt;
    int dm[4] = {0, 1, 0, 1}, dc[4] = {0, 0, 1, 1};
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
  if (P.nside > 0) {
    H.hv[0] = FDIV(zf, chih);
    H.hv[1] = FDIV(yf, chih);
    H.hv[2] = FDIV(xf, chih);
    if ((double)T > P2M_HP_PI || !(T >= 0.0f)) {
      atomicOr(err, (unsigned)P2M_DEVERR_RADIUS); /* query_disc aborts on radius > pi */
    } else {
      double a = (double)H.hv[0], b = (double)H.hv[1], c = (double)H.hv[2];
      double rxy = DSQRT(DADD(DMUL(a, a), DMUL(b, b)));
      double nrm = DSQRT(DADD(DADD(DMUL(a, a), DMUL(b, b)), DMUL(c, c)));
      H.z0 = DDIV(c, nrm);
      H.sth0 = DDIV(rxy, nrm);
      double phi0 = (a != 0.0 || b != 0.0) ? atan2(b, a) : 0.0;
      H.phi0f = phi0 / P2M_HP_TWOPI;
      H.C_in = chord2(T * (1.0f - 2e-6f));
      H.C_out = chord2(T * (1.0f + 2e-6f));
      float tspan = T * (1.0f + 2e-5f) + 1e-6f;
      H.C_span = chord2(tspan);
      float theta0 = atan2f((float)H.sth0, (float)H.z0);
      float tmin = theta0 - tspan, tmax = theta0 + tspan;
      int n4 = 4 * P.nside;
      int lo = 1, hi_ = n4 - 1;
      if (tmin > 0.0f) lo = max(1, (int)floorf(p2m_ring_coord(P.nside, tmin)) - 1);
      if (tmax < 3.14159265f) hi_ = min(n4 - 1, (int)ceilf(p2m_ring_coord(P.nside, tmax)) + 1);
      H.ir_lo = lo;
      H.ir_hi = hi_;
    }
  }
  return true;
}

/* per-halo set-up from a catalogue record (pks2map.f90:264, :284-298) */
__global__ void __launch_bounds__(256) k_setup(PaintParams P, PaintBuffers B) {
  long long n = (long long)B.ctr->n_surv;
  long long stride = (long long)gridDim.x * blockDim.x;
  int lane = threadIdx.x & 31;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n;
       base += stride) {
    long long s = base + lane;
    HaloRec H;
    bool keep = false;
    if (s < n) {
      int i = B.surv[s];
      const float *r = B.records + (long long)i * P.nfloat;
      float p0 = r[0], p1 = r[1], p2 = r[2], rth = r[6];
      float mass = FMUL(P.mass_fac, FMUL(FMUL(rth, rth), rth));
      float xh = p2, yh = p1, zh = p0;
      float chih = FSQRT(FADD(FADD(FMUL(xh, xh), FMUL(yh, yh)), FMUL(zh, zh)));
      float redshift = p2m_lookup(P.zofr, P.cosmo.dzofr, chih);
      xh = FSUB(xh, P.chihview);
      chih = FSQRT(FADD(FADD(FMUL(xh, xh), FMUL(yh, yh)), FMUL(zh, zh)));
      float mh = FMUL(FSQRT(FDIV(p2m_deltacrit(&P.cosmo, redshift), P.bbps_delta)), mass);
      float rh = p2m_powf(
          FDIV(FDIV(FDIV(FDIV(FMUL(3.0f, mh), 4.0f), P.cosmo.mypi), 200.0f),
               p2m_rhocrit(&P.cosmo, redshift)),
          0.333333343f);
      H.rec = i;
      H.w1 = 1.0f;
      H.w2 = 1.0f;
      if (P.any_ksz) {
        /* intended per-halo -v_los/c of pksc.f90:70-74 */
        float v0 = r[3], v1 = r[4], v2 = r[5];
        float dot = FADD(FADD(FMUL(p0, v0), FMUL(p1, v1)), FMUL(p2, v2));
        float nrm = FSQRT(FADD(FADD(FMUL(p0, p0), FMUL(p1, p1)), FMUL(p2, p2)));
        H.w2 = -FDIV(FDIV(dot, nrm), 3.e5f);
      }
      keep = halo_geometry(P, xh, yh, zh, rh, chih, mh, redshift, H, &B.ctr->err);
    }
    long long slot = warp_append(&B.ctr->n_halo, keep);
    if (keep) B.halos[slot] = H;
    warp_count(&B.ctr->n_fs_rows,
               (keep && H.jmin <= H.jmax && H.kmin <= H.kmax) ? (unsigned long long)(H.kmax - H.kmin + 1) : 0ull);
    /* ring histogram: small discs per lane, large discs by the whole warp */
    int nr = keep ? hp_nrings(H) : 0;
    bool small = nr <= 64;
    if (keep && small)
      for (int ring = H.ir_lo; ring <= H.ir_hi; ring++) atomicAdd(&B.ring_hist[ring], 1u);
    unsigned big = __ballot_sync(FULL, keep && !small);
    while (big) {
      int b = __ffs(big) - 1;
      big &= big - 1;
      int lo = __shfl_sync(FULL, H.ir_lo, b), hi = __shfl_sync(FULL, H.ir_hi, b);
      for (int ring = lo + lane; ring <= hi; ring += 32) atomicAdd(&B.ring_hist[ring], 1u);
    }
  }
}

/* per-halo set-up from already-computed loop quantities (p2m_project_halo): 9 floats
   x, y, z, r, chi, m, redshift, v, profile per halo */
__global__ void __launch_bounds__(256) k_setup_prepared(PaintParams P, PaintBuffers B,
                                                        const float *prep, long long n) {
  long long stride = (long long)gridDim.x * blockDim.x;
  int lane = threadIdx.x & 31;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n;
       base += stride) {
    long long s = base + lane;
    HaloRec H;
    bool keep = false;
    if (s < n) {
      const float *q = prep + s * 9;
      int prof = (int)q[8];
      H.rec = (int)s;
      H.w1 = prof == 1 ? q[7] : 0.0f;
      H.w2 = prof == 2 ? q[7] : 0.0f;
      keep = halo_geometry(P, q[0], q[1], q[2], q[3], q[4], q[5], q[6], H, &B.ctr->err);
    }
    long long slot = warp_append(&B.ctr->n_halo, keep);
    if (keep) B.halos[slot] = H;
    warp_count(&B.ctr->n_fs_rows,
               (keep && H.jmin <= H.jmax && H.kmin <= H.kmax) ? (unsigned long long)(H.kmax - H.kmin + 1) : 0ull);
    int nr = keep ? hp_nrings(H) : 0;
    bool small = nr <= 64;
    if (keep && small)
      for (int ring = H.ir_lo; ring <= H.ir_hi; ring++) atomicAdd(&B.ring_hist[ring], 1u);
    unsigned big = __ballot_sync(FULL, keep && !small);
    while (big) {
      int b = __ffs(big) - 1;
      big &= big - 1;
      int lo = __shfl_sync(FULL, H.ir_lo, b), hi = __shfl_sync(FULL, H.ir_hi, b);
      for (int ring = lo + lane; ring <= hi; ring += 32) atomicAdd(&B.ring_hist[ring], 1u);
    }
  }
}

/* -------------------------------------------------------------------- scans ----- */

/* exclusive scan of n (<= any) uint32 in one block; out[i] int64; *total = sum */
__global__ void __launch_bounds__(1024) k_scan_single(const unsigned int *in, long long *out,
                                                      long long n, unsigned long long *total) {
  __shared__ long long warp_sums[32];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (long long base = 0; base < n; base += blockDim.x) {
    long long i = base + threadIdx.x;
    long long v = i < n ? (long long)in[i] : 0;
    long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(FULL, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
      long long ws = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(FULL, ws, o);
        if (lane >= o) ws += y;
      }
      warp_sums[lane] = ws; /* inclusive */
    }
    __syncthreads();
    long long wofs = wid > 0 ? warp_sums[wid - 1] : 0;
    if (i < n) out[i] = carry + wofs + x - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += wofs + x;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = (unsigned long long)carry;
}

#define SCAN_BLOCKS 1024

/* block sums of counts over SCAN_BLOCKS equal ranges of [0, n) */
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

__global__ void __launch_bounds__(1024) k_scan_top(long long *bsum,
                                                   unsigned long long *total) {
  /* exclusive scan of SCAN_BLOCKS int64 in place */
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
  if (t == SCAN_BLOCKS - 1) *total = (unsigned long long)sh[t];
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

/* -------------------------------------------------------------------- k_emit ----- */

__device__ __forceinline__ void emit_item(const PaintBuffers &B, int h, int ring) {
  unsigned int k = atomicAdd(&B.ring_cursor[ring], 1u);
  long long pos = B.ring_start[ring] + k;
  RingItem it;
  it.halo = h;
  it.ring = ring;
  it.lo = 0;
  it.count = 0;
  it.A = it.B = it.x0 = it.hdphi = 0.0f;
  B.items[pos] = it;
}

/* places every (halo, ring) item at its ring's slot range; appends flat-sky rows */
__global__ void __launch_bounds__(256) k_emit(PaintParams P, PaintBuffers B) {
  long long n = (long long)B.ctr->n_halo;
  long long stride = (long long)gridDim.x * blockDim.x;
  int lane = threadIdx.x & 31;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n;
       base += stride) {
    long long h = base + lane;
    bool valid = h < n;
    int lo = 1, hi = 0;
    int jmin = 1, jmax = 0, kmin = 1, kmax = 0;
    if (valid) {
      const HaloRec &H = B.halos[h];
      lo = H.ir_lo;
      hi = H.ir_hi;
      jmin = H.jmin;
      jmax = H.jmax;
      kmin = H.kmin;
      kmax = H.kmax;
    }
    int nr = hi >= lo ? hi - lo + 1 : 0;
    bool small = nr <= 64;
    if (valid && small)
      for (int ring = lo; ring <= hi; ring++) emit_item(B, (int)h, ring);
    unsigned big = __ballot_sync(FULL, valid && !small);
    while (big) {
      int b = __ffs(big) - 1;
      big &= big - 1;
      int blo = __shfl_sync(FULL, lo, b), bhi = __shfl_sync(FULL, hi, b);
      int hb = (int)__shfl_sync(FULL, (long long)h, b);
      for (int ring = blo + lane; ring <= bhi; ring += 32) emit_item(B, hb, ring);
    }
    /* flat-sky rows */
    if (valid && jmin <= jmax && kmin <= kmax) {
      int nrow = kmax - kmin + 1;
      unsigned long long fb = atomicAdd(&B.ctr->n_fs_items, (unsigned long long)nrow);
      if ((long long)(fb + nrow) > B.fs_cap) {
        atomicOr(&B.ctr->err, (unsigned)P2M_DEVERR_FS_OVERFLOW);
      } else {
        for (int t = 0; t < nrow; t++) {
          FsItem f;
          f.halo = (int)h;
          f.k = kmin + t;
          f.jmin = jmin;
          f.count = jmax - jmin + 1;
          B.fs_items[fb + t] = f;
        }
      }
    }
  }
}

/* ------------------------------------------------------------------- k_rings ----- */

/* candidate span of one (halo, ring): every pixel centre with chord^2 <= C_span
   (a disc 2e-5 wider than dtheta) lies in [lo, lo+count); FP32 with a margin */
__global__ void __launch_bounds__(256) k_rings(PaintParams P, PaintBuffers B) {
  long long n = (long long)B.ctr->n_items;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += stride) {
    RingItem it = B.items[g];
    const HaloRec &H = B.halos[it.halo];
    double2 zs = P.ringtab[it.ring];
    double dz = zs.x - H.z0, ds = zs.y - H.sth0;
    float A = (float)(dz * dz + ds * ds);
    float Bc = (float)(4.0 * zs.y * H.sth0);
    int npr, kshift;
    long long npn;
    p2m_ring_info(P.nside, it.ring, &npr, &kshift, &npn);
    double q = H.phi0f * (double)npr;
    double sh = 0.5 * kshift;
    float cspan = H.C_span;
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
      else hw = asinf(sqrtf(t)) * ((float)npr * 0.318309886f);
    }
    if (!empty) {
      double eps = 0.02 + 1e-5 * (double)hw;
      if (!full) {
        long long l = (long long)ceil(q - sh - (double)hw - eps);
        long long h = (long long)floor(q - sh + (double)hw + eps);
        if (h - l + 1 >= npr) full = true;
        else if (h >= l) {
          lo = (int)l;
          cnt = (int)(h - l + 1);
        }
      }
      if (full) {
        lo = (int)ceil(q - sh - 0.5 * (double)npr);
        cnt = npr;
      }
    }
    it.lo = lo;
    it.count = cnt;
    it.A = A;
    it.B = Bc;
    it.x0 = (float)(((double)lo + sh) - q);
    it.hdphi = 3.14159265358979f / (float)npr;
    B.items[g] = it;
    B.counts[g] = (unsigned int)cnt;
  }
}

/* ------------------------------------------------------------------- deposit ----- */

template <int PREC>
__device__ __forceinline__ void deposit(void *acc, long long idx, float v) {
  if (PREC == 0) {
    atomicAdd((double *)acc + idx, (double)v);
  } else {
    float *a = (float *)acc + 2 * idx;
    float old = atomicAdd(a, v);
    /* TwoSum: the exact rounding error of old + v, carried in the low word */
    float s = __fadd_rn(old, v);
    float bb = __fsub_rn(s, old);
    float err = __fadd_rn(__fsub_rn(old, __fsub_rn(s, bb)), __fsub_rn(v, bb));
    if (err != 0.0f) atomicAdd(a + 1, err);
  }
}

/* profile values of every map at one pixel (maptable.f90:204-212 with known ir, fr) */
template <int PREC>
__device__ __forceinline__ void deposit_maps(const PaintParams &P, const HaloRec &H,
                                             void *acc, long long pix, int ir, float fr) {
  float ofr = FSUB(1.0f, fr), ofc = FSUB(1.0f, H.fc), ofm = FSUB(1.0f, H.fm);
  float fc = H.fc, fm = H.fm;
  bool fast = H.cbase[0] >= 0 && H.cbase[1] >= 0 && H.cbase[2] >= 0 && H.cbase[3] >= 0;
  p2m_hinterp hi = halo_hinterp(H);
  for (int m = 0; m < P.nmaps; m++) {
    int prof = P.map_profile[m];
    float w = prof == 2 ? H.w2 : H.w1;
    if (w == 0.0f) continue;
    const float *tab = P.tables[P.map_table[m]];
    float v;
    if (fast) {
      int rofs = 2 * (ir - 1) + (prof - 1);
      float t00a = __ldg(tab + H.cbase[0] + rofs), t00b = __ldg(tab + H.cbase[0] + rofs + 2);
      float t10a = __ldg(tab + H.cbase[1] + rofs), t10b = __ldg(tab + H.cbase[1] + rofs + 2);
      float t01a = __ldg(tab + H.cbase[2] + rofs), t01b = __ldg(tab + H.cbase[2] + rofs + 2);
      float t11a = __ldg(tab + H.cbase[3] + rofs), t11b = __ldg(tab + H.cbase[3] + rofs + 2);
      v = 0.0f;
      v = FADD(v, FMUL(FMUL(FMUL(t00a, ofr), ofc), ofm));
      v = FADD(v, FMUL(FMUL(FMUL(t00b, fr), ofc), ofm));
      v = FADD(v, FMUL(FMUL(FMUL(t10a, ofr), fc), ofm));
      v = FADD(v, FMUL(FMUL(FMUL(t10b, fr), fc), ofm));
      v = FADD(v, FMUL(FMUL(FMUL(t01a, ofr), ofc), fm));
      v = FADD(v, FMUL(FMUL(FMUL(t01b, fr), ofc), fm));
      v = FADD(v, FMUL(FMUL(FMUL(t11a, ofr), fc), fm));
      v = FADD(v, FMUL(FMUL(FMUL(t11b, fr), fc), fm));
    } else {
      v = p2m_blend8(tab, &P.th, &hi, prof, ir, fr);
    }
    deposit<PREC>(acc, pix * P.nmaps + m, FMUL(w, v));
  }
}

__device__ __forceinline__ void record_set(const PaintBuffers &B, const HaloRec &H, long long pix) {
  unsigned long long k = atomicAdd(&B.ctr->n_sets, 1ull);
  if ((long long)k < B.set_cap) {
    B.set_rec[k] = H.rec;
    B.set_pix[k] = pix;
  }
}

/* exact decision and deposit for one candidate: the reference's FP64 pixel centre and
   angular distance (haloproject.f90:60-73) and the float interpolation */
template <int PREC>
__device__ void paint_exact_pixel(const PaintParams &P, const PaintBuffers &B, const HaloRec &H,
                                  long long pix, unsigned long long &nupd) {
  double v2[3], v1[3] = {(double)H.hv[0], (double)H.hv[1], (double)H.hv[2]};
  p2m_pix2vec_ring(P.nside, pix, v2);
  float angle = (float)p2m_angdist(v1, v2);
  if (!((double)angle < (double)H.T)) return;
  nupd++;
  if (P.flags & 1) record_set(B, H, pix);
  if (H.zero) return;
  float r = FMUL(H.chi_t, p2m_tanf(angle));
  if (r > P.th.rmaxt) return;
  int ir;
  float fr;
  p2m_rindex(&P.th, r, &ir, &fr);
  deposit_maps<PREC>(P, H, B.hp_acc, pix, ir, fr);
}

/* ------------------------------------------------------------------- k_paint ----- */

#define PAINT_CHUNK 1024

/* largest g in [0, n) with off[g] <= p (off[0] = 0), found by the whole warp */
__device__ __forceinline__ long long warp_upper(const long long *off, long long n, long long p) {
  int lane = threadIdx.x & 31;
  long long lo = 0, hi = n;
  while (hi - lo > 32) {
    long long span = hi - lo;
    long long s = lo + (span * lane) / 32;
    bool le = off[s] <= p;
    unsigned m = __ballot_sync(FULL, le);
    int t = 31 - __clz(m); /* lane 0 always true */
    long long nlo = lo + (span * t) / 32;
    long long nhi = t < 31 ? lo + (span * (t + 1)) / 32 : hi;
    lo = nlo;
    hi = nhi;
  }
  long long s = lo + lane;
  bool le = s < hi && off[s] <= p;
  unsigned m = __ballot_sync(FULL, le);
  return lo + (31 - __clz(m));
}

template <int PREC>
__global__ void __launch_bounds__(256) k_paint(PaintParams P, PaintBuffers B) {
  const long long npix_c = (long long)B.ctr->n_pix;
  const long long nitems = (long long)B.ctr->n_items;
  if (npix_c == 0) return;
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long nchunks = (npix_c + PAINT_CHUNK - 1) / PAINT_CHUNK;
  unsigned long long nupd = 0, nfb = 0;
  for (long long c = warp; c < nchunks; c += nwarps) {
    long long p0 = c * PAINT_CHUNK, p1 = min(npix_c, p0 + PAINT_CHUNK);
    long long g0 = warp_upper(B.pix_off, nitems, p0);
    long long woff = (g0 + lane < nitems) ? B.pix_off[g0 + lane] : (1LL << 62);
    long long wend = (g0 + 32 < nitems) ? B.pix_off[g0 + 32] : (1LL << 62);
    for (long long base = p0; base < p1; base += 32) {
      long long p = base + lane;
      bool todo = p < p1;
      /* every round serves at least the lowest pending lane: <= 32 rounds */
      for (int round = 0; __any_sync(FULL, todo); round++) {
        if (round >= 64) {
          atomicOr(&B.ctr->err, (unsigned)P2M_DEVERR_ITEMS);
          break;
        }
        /* slide the 32-item window so that it starts at the item holding the lowest
           pending pixel */
        long long pmin = todo ? p : (1LL << 62);
        for (int o = 16; o > 0; o >>= 1) pmin = min(pmin, __shfl_xor_sync(FULL, pmin, o));
        unsigned m = __ballot_sync(FULL, woff <= pmin);
        int j0 = m ? 31 - __clz(m) : -1;
        if (j0 != 0 || pmin >= wend) {
          if (j0 < 0 || pmin >= wend) g0 = warp_upper(B.pix_off, nitems, pmin);
          else g0 += j0;
          woff = (g0 + lane < nitems) ? B.pix_off[g0 + lane] : (1LL << 62);
          wend = (g0 + 32 < nitems) ? B.pix_off[g0 + 32] : (1LL << 62);
        }
        bool here = todo && p < wend;
        /* item of p inside the window: binary search over lanes */
        int j = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          long long o = __shfl_sync(FULL, woff, j + step);
          if (o <= p) j += step;
        }
        long long ooff = __shfl_sync(FULL, woff, j);
        if (here) {
          todo = false;
          long long g = g0 + j;
          const RingItem &it = B.items[g];
          const HaloRec &H = B.halos[it.halo];
          int k = (int)(p - ooff);
          int npr, kshift;
          long long npn;
          p2m_ring_info(P.nside, it.ring, &npr, &kshift, &npn);
          int iphi = it.lo + k;
          if (iphi < 0) iphi += npr;
          if (iphi >= npr) iphi -= npr;
          long long pix = npn - npr + iphi;
          if (PREC == 0) {
            paint_exact_pixel<0>(P, B, H, pix, nupd);
          } else {
            float x = it.x0 + (float)k;
            float s = sinf(x * it.hdphi);
            float c2 = it.A + it.B * (s * s);
            if (c2 < H.C_out) {
              bool recheck = c2 > H.C_in;
              int ir = 0;
              float fr = 0.0f;
              bool zero_val = false;
              if (!recheck) {
                float h2 = 0.25f * c2;
                float cosd = 1.0f - 2.0f * h2;
                if (cosd < 0.05f) {
                  recheck = true;
                } else {
                  float sind = 2.0f * sqrtf(h2 * (1.0f - h2));
                  float r = H.chi_t * __fdividef(sind, cosd);
                  const float dr = 1e-5f;
                  if (r > P.th.rmaxt * (1.0f + dr)) {
                    zero_val = true;
                  } else if (r >= P.th.rmaxt * (1.0f - dr)) {
                    recheck = true;
                  } else if (r < P.th.rmint * (1.0f - dr)) {
                    ir = P.ir_c;
                    fr = P.fr_c;
                  } else if (r <= P.th.rmint * (1.0f + dr)) {
                    recheck = true;
                  } else {
                    float lr = __logf(r);
                    float u = (lr - P.th.lrmin) / P.th.drt;
                    int iu = (int)u;
                    float fu = u - (float)iu;
                    if (fu < 2e-4f || fu > 1.0f - 2e-4f || iu < 0 || iu > P.th.nrt - 2) {
                      recheck = true;
                    } else {
                      ir = iu + 1;
                      fr = FSUB(lr, FADD(P.th.lrmin, FMUL((float)(ir - 1), P.th.drt)));
                    }
                  }
                }
              }
              if (recheck) {
                unsigned long long slot = atomicAdd(&B.ctr->n_fb, 1ull);
                if ((long long)slot < B.fb_cap)
                  B.fb[slot] = ((unsigned long long)g << 32) | (unsigned int)k;
                else
                  atomicOr(&B.ctr->err, (unsigned)P2M_DEVERR_FB_OVERFLOW);
                nfb++;
              } else {
                nupd++;
                if (P.flags & 1) record_set(B, H, pix);
                if (!zero_val && !H.zero) deposit_maps<1>(P, H, B.hp_acc, pix, ir, fr);
              }
            }
          }
        }
      }
    }
  }
  warp_count(&B.ctr->hp_updates, nupd);
  warp_count(&B.ctr->n_recheck, nfb);
}

/* exact FP64 decision for the pixels the mixed-precision test could not settle */
__global__ void __launch_bounds__(256) k_recheck(PaintParams P, PaintBuffers B) {
  long long n = (long long)min(B.ctr->n_fb, (unsigned long long)B.fb_cap);
  long long stride = (long long)gridDim.x * blockDim.x;
  unsigned long long nupd = 0;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n;
       base += stride) {
    long long e = base + (threadIdx.x & 31);
    if (e < n) {
      unsigned long long v = B.fb[e];
      long long g = (long long)(v >> 32);
      int k = (int)(v & 0xffffffffu);
      const RingItem &it = B.items[g];
      const HaloRec &H = B.halos[it.halo];
      int npr, kshift;
      long long npn;
      p2m_ring_info(P.nside, it.ring, &npr, &kshift, &npn);
      int iphi = it.lo + k;
      if (iphi < 0) iphi += npr;
      if (iphi >= npr) iphi -= npr;
      paint_exact_pixel<1>(P, B, H, npn - npr + iphi, nupd);
    }
  }
  warp_count(&B.ctr->hp_updates, nupd);
}

/* ----------------------------------------------------------------- flat sky ----- */

/* haloproject.f90:136-152: one warp per (halo, row); every operation is the
   reference's float sequence, so the pixel set and values are exact */
template <int PREC>
__global__ void __launch_bounds__(256) k_paint_fs(PaintParams P, PaintBuffers B) {
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
        deposit_maps<PREC>(P, H, B.fs_acc, pix, ir, fr);
      }
    }
  }
  warp_count(&B.ctr->fs_updates, nupd);
}

/* ----------------------------------------------------------------- finalize ----- */

template <int PREC>
__global__ void __launch_bounds__(256) k_finalize(const void *acc, long long npix, int nmaps,
                                                  int map, float *out, double *sum) {
  long long stride = (long long)gridDim.x * blockDim.x;
  double s = 0.0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += stride) {
    float v;
    if (PREC == 0) {
      v = (float)__ldcs((const double *)acc + p * nmaps + map);
    } else {
      float2 a = __ldcs((const float2 *)acc + p * nmaps + map);
      v = __fadd_rn(a.x, a.y);
    }
    __stcs(out + p, v);
    s += (double)v;
  }
  __shared__ double red[8];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(FULL, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    if (sum) atomicAdd(sum, t);
  }
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

/* integrate_profiles.f90:155-238 (which = 1: pressure, 2: gas density) */
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

void p2m_launch_cut(const PaintParams &P, const PaintBuffers &B, long long n, cudaStream_t s,
                    int nsm) {
  k_cut<<<grid_for(n, 256, nsm, 8), 256, 0, s>>>(P, B, n);
}
void p2m_launch_setup(const PaintParams &P, const PaintBuffers &B, long long n_max,
                      cudaStream_t s, int nsm) {
  k_setup<<<grid_for(n_max, 256, nsm, 4), 256, 0, s>>>(P, B);
}
void p2m_launch_prepared(const PaintParams &P, const PaintBuffers &B, const float *d_prep,
                         long long n, cudaStream_t s, int nsm) {
  k_setup_prepared<<<grid_for(n, 256, nsm, 4), 256, 0, s>>>(P, B, d_prep, n);
}
void p2m_launch_ring_scan(const PaintParams &P, const PaintBuffers &B, cudaStream_t s) {
  long long n = 4LL * P.nside; /* rings 0..4N-1 (slot 0 unused) */
  k_scan_single<<<1, 1024, 0, s>>>(B.ring_hist, B.ring_start, n, &B.ctr->n_items);
}
void p2m_launch_emit(const PaintParams &P, const PaintBuffers &B, long long n_max,
                     cudaStream_t s, int nsm) {
  k_emit<<<grid_for(n_max, 256, nsm, 4), 256, 0, s>>>(P, B);
}
void p2m_launch_rings(const PaintParams &P, const PaintBuffers &B, long long n_max,
                      cudaStream_t s, int nsm) {
  k_rings<<<grid_for(n_max, 256, nsm, 8), 256, 0, s>>>(P, B);
}
void p2m_launch_count_scan(const PaintParams &P, const PaintBuffers &B, cudaStream_t s) {
  (void)P;
  k_scan_partial<<<SCAN_BLOCKS, 256, 0, s>>>(B.counts, &B.ctr->n_items, B.scan_tmp);
  k_scan_top<<<1, SCAN_BLOCKS, 0, s>>>(B.scan_tmp, &B.ctr->n_pix);
  k_scan_apply<<<SCAN_BLOCKS, 256, 0, s>>>(B.counts, &B.ctr->n_items, B.scan_tmp, B.pix_off);
}
void p2m_launch_paint(const PaintParams &P, const PaintBuffers &B, cudaStream_t s, int nsm) {
  if (P.precision == 0) k_paint<0><<<nsm * 8, 256, 0, s>>>(P, B);
  else k_paint<1><<<nsm * 8, 256, 0, s>>>(P, B);
}
void p2m_launch_recheck(const PaintParams &P, const PaintBuffers &B, cudaStream_t s, int nsm) {
  k_recheck<<<nsm * 2, 256, 0, s>>>(P, B);
}
void p2m_launch_paint_fs(const PaintParams &P, const PaintBuffers &B, cudaStream_t s, int nsm) {
  if (P.precision == 0) k_paint_fs<0><<<nsm * 8, 256, 0, s>>>(P, B);
  else k_paint_fs<1><<<nsm * 8, 256, 0, s>>>(P, B);
}
void p2m_launch_finalize(const PaintParams &P, const void *acc, long long npix, int map,
                         float *out, double *sum, cudaStream_t s, int nsm) {
  int g = grid_for(npix, 256, nsm, 8);
  if (P.precision == 0) k_finalize<0><<<g, 256, 0, s>>>(acc, npix, P.nmaps, map, out, sum);
  else k_finalize<1><<<g, 256, 0, s>>>(acc, npix, P.nmaps, map, out, sum);
}
void p2m_launch_maptable(const PaintParams &P, const TableConsts &K, const p2m_tabhdr &th,
                         float *d_table, cudaStream_t s) {
  long long n = (long long)th.nchit * th.nmht * th.nrt;
  k_maptable<<<(int)((n + 127) / 128), 128, 0, s>>>(P, K, th, d_table);
}
