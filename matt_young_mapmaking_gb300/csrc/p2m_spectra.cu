/*
 * p2m_spectra.cu -- angular power spectra of painted maps, for the precision report.
 * Validation only: nothing here is on the painting path.
 *
 * HEALPix maps (RING order): the pixel-area quadrature analysis of the HEALPix library
 * that the reference vendors, map2alm without iterations and with unit ring weights
 * (src/modules/External/alm_map_dd_inc.F90:2978-3224), followed by alm2cl (:5347-5423):
 *
 *   a_lm = (4 pi / npix) sum_rings lambda_lm(theta_r) F_r(m)
 *   F_r(m) = sum_j f_rj exp(-i m phi_rj)     (ring_analysis, alm_tools.F90:1022-1097)
 *   C_l = (Re a_l0 b_l0 + 2 sum_{m>=1} Re a_lm conj(b_lm)) / (2l + 1)
 *
 * lambda_lm is the normalised associated Legendre function.  It is computed by the
 * three-term recursion in l of HEALPix: gen_mfac (alm_tools.F90:500-522) and
 * compute_lam_mm (:559-580) start it, gen_recfac (:394-416) gives its coefficients,
 * and the loop of map2alm_sc_d runs it.  Powers of 2^100 are factored out as the
 * recursion runs, so that lambda_mm ~ sin^m(theta) neither underflows nor overflows;
 * a term whose scale is below 2^-1000 counts as zero (rescale_tab, :284-307).  Terms
 * below l_min_ylm (:882-903) are skipped as HEALPix skips them.  The ring geometry is
 * get_pixel_layout (:311-349).  The equatorial symmetry lambda_lm(pi - theta) =
 * (-1)^(l+m) lambda_lm(theta) pairs each northern ring with its southern mirror.
 *
 * GPU layout:
 *   k_ring_phases  one block per (northern ring, 256 values of m).  Both hemispheres'
 *                  rings and both maps are staged through shared memory.  Each thread
 *                  sums one m, with twiddles stepped by complex multiplication and
 *                  re-seeded from an exact integer phase index every 1024 pixels.  It
 *                  writes S = F_north + F_south and D = F_north - F_south for each map,
 *                  laid out [m][ring] so that the next kernel reads one m's rings
 *                  contiguously.
 *   k_alm          one block per m; 8 rings per thread, recursion state in registers.
 *                  Per l the warp reduces its lanes' sums, and the block's warps are
 *                  summed in shared memory 64 values of l at a time.
 *   k_alm2cl       one thread per l.
 * All arithmetic is FP64: the estimator is a diagnostic, where exactness matters more
 * than speed.
 *
 * Flat-sky maps: the periodogram of the npix x npix map over fov x fov radians, binned
 * linearly in ell = 2 pi |k| / fov.  It has no counterpart in the reference.
 *
 *   C(ell) = (fov^2 / npix^4) |FFT(map)(k)|^2, averaged over the modes of a bin
 *
 * k = 0 is left out, and so is the Nyquist line.  Both maps go through one complex FFT
 * (a + i b).  The rows are transformed by a radix-2 FFT in shared memory when npix is
 * a power of two up to 8192, or by a direct DFT for other npix up to 2048.  The columns
 * are transformed the same way after a transpose.
 */
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <vector>

#include "../../include/p2m.h"
#include "../../include/p2m_tools.h"

namespace {

#define FULL_MASK 0xffffffffu

constexpr int RP_THREADS = 256; /* values of m per k_ring_phases block */
constexpr int RP_CHUNK = 1024;  /* ring pixels staged per pass */
constexpr int ALM_THREADS = 256;
constexpr int ALM_RINGS = 8; /* rings per thread */
constexpr int ALM_GROUP = ALM_THREADS * ALM_RINGS;
constexpr int ALM_LC = 64; /* values of l per reduction chunk */
constexpr int ALM_WARPS = ALM_THREADS / 32;
constexpr int FFT_THREADS = 512;
constexpr int FFT_MAX_POW2 = 8192;
constexpr int DFT_MAX = 2048;

struct RingGeom {
  double cth, sth;
  int nph, shift; /* shift 1: pixel centres at phi = pi (2j + 1) / nph */
  long long start;
};

/* get_pixel_layout (alm_tools.F90:311-349) for northern ring ith = 1 .. 2 nside */
__device__ RingGeom ring_geom(int nside, int ith) {
  RingGeom g;
  const double n = (double)nside;
  if (ith < nside) {
    g.cth = 1.0 - ((double)ith * (double)ith) * (1.0 / (3.0 * n * n));
    g.sth = sin(2.0 * asin((double)ith * (1.0 / (sqrt(6.0) * n))));
    g.nph = 4 * ith;
    g.shift = 1;
    g.start = 2LL * ith * (ith - 1);
  } else {
    g.cth = (double)(2 * nside - ith) * (2.0 / (3.0 * n));
    g.sth = sqrt((1.0 - g.cth) * (1.0 + g.cth));
    g.nph = 4 * nside;
    g.shift = (ith + 1 - nside) & 1;
    g.start = 2LL * nside * (nside - 1) + (long long)(ith - nside) * g.nph;
  }
  return g;
}

/* 2^(100 s) for |s| <= 10, zero below (the scales that underflow) */
__device__ __forceinline__ double scale_factor(int s) {
  return (s < -10 || s > 10) ? 0.0 : ldexp(1.0, 100 * s);
}

/* F_r(m) of northern ring blockIdx.x + 1 and its mirror, for both maps */
__global__ void __launch_bounds__(RP_THREADS)
    k_ring_phases(const float *__restrict__ ma, const float *__restrict__ mb, int nside,
                  int lmax, double *__restrict__ ph) {
  __shared__ double sp[4][RP_CHUNK]; /* a north, a south, b north, b south */
  const int ith = blockIdx.x + 1;
  const int nrings = 2 * nside;
  const RingGeom g = ring_geom(nside, ith);
  const long long npix = 12LL * nside * nside;
  const long long sn = g.start, ss = npix - g.start - g.nph;
  const bool south = ith < nrings; /* the equator has no mirror */
  const int m = blockIdx.y * RP_THREADS + threadIdx.x;
  const bool act = m <= lmax;
  const int nph = g.nph, period = 2 * nph;
  /* exp(-i m phi_j) with phi_j = pi (2j + shift) / nph: phase index m (2j + shift)
     mod 2 nph, and m enters only modulo 2 nph */
  const long long mr = act ? (long long)(m % period) : 0;
  double st_s, st_c;
  sincospi((double)((2 * mr) % period) / (double)nph, &st_s, &st_c);
  const double step_r = st_c, step_i = -st_s;
  double ar[4] = {0.0, 0.0, 0.0, 0.0}, ai[4] = {0.0, 0.0, 0.0, 0.0};
  for (int j0 = 0; j0 < nph; j0 += RP_CHUNK) {
    const int nj = min(RP_CHUNK, nph - j0);
    __syncthreads();
    for (int j = threadIdx.x; j < nj; j += RP_THREADS) {
      sp[0][j] = (double)ma[sn + j0 + j];
      sp[1][j] = south ? (double)ma[ss + j0 + j] : 0.0;
      sp[2][j] = mb ? (double)mb[sn + j0 + j] : 0.0;
      sp[3][j] = (mb && south) ? (double)mb[ss + j0 + j] : 0.0;
    }
    __syncthreads();
    if (!act) continue;
    const long long k0 = (mr * (2LL * j0 + g.shift)) % period;
    double ws, wc;
    sincospi((double)k0 / (double)nph, &ws, &wc);
    double wr = wc, wi = -ws;
    for (int j = 0; j < nj; j++) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        ar[q] = fma(sp[q][j], wr, ar[q]);
        ai[q] = fma(sp[q][j], wi, ai[q]);
      }
      const double nr = wr * step_r - wi * step_i;
      wi = fma(wr, step_i, wi * step_r);
      wr = nr;
    }
  }
  if (!act) return;
  double *o = ph + ((size_t)m * nrings + (ith - 1)) * 8;
  o[0] = ar[0] + ar[1];
  o[1] = ai[0] + ai[1];
  o[2] = ar[0] - ar[1];
  o[3] = ai[0] - ai[1];
  o[4] = ar[2] + ar[3];
  o[5] = ai[2] + ai[3];
  o[6] = ar[2] - ar[3];
  o[7] = ai[2] - ai[3];
}

/* row offset of m in the packed a_lm array (l = m .. lmax) */
__host__ __device__ __forceinline__ size_t alm_row(int m, int lmax) {
  return (size_t)m * (size_t)(lmax + 1) - (size_t)m * (size_t)(m - 1) / 2;
}

/* a_lm / omega_pix of both maps for m = blockIdx.x, added into alm[(row + l - m) * 4 + c],
   c = (Re a, Im a, Re b, Im b) */
__global__ void __launch_bounds__(ALM_THREADS)
    k_alm(const double *__restrict__ ph, const double *__restrict__ mfac, int nside, int lmax,
          double *__restrict__ alm) {
  extern __shared__ double smem[];
  double *sph = smem;                 /* [ALM_GROUP][8] phases of this m */
  double *rfa = sph + ALM_GROUP * 8;  /* rf(l), l = l0 .. l0 + LC - 1 */
  double *rfb = rfa + ALM_LC;         /* 1 / rf(l - 1) */
  double *red = rfb + ALM_LC;         /* [warp][LC][4] */
  const int m = blockIdx.x;
  const int nrings = 2 * nside;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const double dm2 = (double)m * (double)m;
  const size_t row = alm_row(m, lmax);
  const double mf = mfac[m];
  for (int g0 = 0; g0 < nrings; g0 += ALM_GROUP) {
    const int ng = min(ALM_GROUP, nrings - g0);
    __syncthreads();
    const double *src = ph + ((size_t)m * nrings + g0) * 8;
    for (int i = t; i < ng * 8; i += ALM_THREADS) sph[i] = src[i];
    double cth[ALM_RINGS], lprev[ALM_RINGS], lcur[ALM_RINGS], cm[ALM_RINGS], lmm[ALM_RINGS];
    int sc[ALM_RINGS], lmin[ALM_RINGS];
    int any = 0;
#pragma unroll
    for (int k = 0; k < ALM_RINGS; k++) {
      const int r = k * ALM_THREADS + t;
      cth[k] = 0.0;
      lprev[k] = 0.0;
      lcur[k] = 0.0;
      cm[k] = 0.0;
      lmm[k] = 0.0;
      sc[k] = 0;
      lmin[k] = INT_MAX;
      if (r < ng) {
        const RingGeom gg = ring_geom(nside, g0 + r + 1);
        /* l_min_ylm: int((m - 40) / (1.35 sin theta)), at least m */
        const double v = (double)(m - 40) / (1.35 * gg.sth);
        const int lm = v > (double)lmax ? lmax + 1 : max(m, (int)v);
        if (lm <= lmax) {
          const double log2val = mf + (double)m * log(gg.sth) * (1.0 / log(2.0));
          const int s = (int)(log2val / 100.0);
          double lam_mm = exp2(log2val - 100.0 * (double)s);
          if (m & 1) lam_mm = -lam_mm;
          cth[k] = gg.cth;
          lcur[k] = 1.0; /* lambda_m / (lambda_mm scale) */
          lmm[k] = lam_mm;
          sc[k] = s;
          cm[k] = scale_factor(s) * lam_mm;
          lmin[k] = lm;
          any = 1;
        }
      }
    }
    if (!__syncthreads_or(any)) continue;
    for (int l0 = m; l0 <= lmax; l0 += ALM_LC) {
      __syncthreads();
      if (t < ALM_LC) {
        /* gen_recfac: rf(l) = sqrt((4 (l+1)^2 - 1) / ((l+1)^2 - m^2)) */
        const int l = l0 + t;
        const double f1 = (double)(l + 1) * (double)(l + 1);
        rfa[t] = sqrt((4.0 * f1 - 1.0) / (f1 - dm2));
        if (l - 1 >= m) {
          const double f0 = (double)l * (double)l;
          rfb[t] = 1.0 / sqrt((4.0 * f0 - 1.0) / (f0 - dm2));
        } else {
          rfb[t] = 0.0;
        }
      }
      __syncthreads();
      const int nl = min(ALM_LC, lmax - l0 + 1);
      for (int i = 0; i < nl; i++) {
        const int l = l0 + i;
        const int par = ((l + m) & 1) ? 2 : 0; /* S for even l + m, D for odd */
        const double ra = rfa[i], rb = rfb[i];
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
#pragma unroll
        for (int k = 0; k < ALM_RINGS; k++) {
          if (l >= lmin[k]) {
            const double lam = lcur[k] * cm[k];
            const double *p = sph + (size_t)(k * ALM_THREADS + t) * 8;
            s0 = fma(lam, p[par], s0);
            s1 = fma(lam, p[par + 1], s1);
            s2 = fma(lam, p[4 + par], s2);
            s3 = fma(lam, p[5 + par], s3);
          }
          /* lambda_{l+1} = rf(l) (cos theta lambda_l - lambda_{l-1} / rf(l-1)) */
          const double back = lprev[k] * rb;
          lprev[k] = lcur[k];
          const double nx = (cth[k] * lcur[k] - back) * ra;
          lcur[k] = nx;
          if (fabs(nx) > 0x1p100) {
            lprev[k] *= 0x1p-100;
            lcur[k] *= 0x1p-100;
            sc[k] += 1;
            cm[k] = scale_factor(sc[k]) * lmm[k];
          } else if (fabs(nx) < 0x1p-100 && nx != 0.0) {
            lprev[k] *= 0x1p100;
            lcur[k] *= 0x1p100;
            sc[k] -= 1;
            cm[k] = scale_factor(sc[k]) * lmm[k];
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          s0 += __shfl_xor_sync(FULL_MASK, s0, o);
          s1 += __shfl_xor_sync(FULL_MASK, s1, o);
          s2 += __shfl_xor_sync(FULL_MASK, s2, o);
          s3 += __shfl_xor_sync(FULL_MASK, s3, o);
        }
        if (lane == 0) {
          double *q = red + ((size_t)w * ALM_LC + i) * 4;
          q[0] = s0;
          q[1] = s1;
          q[2] = s2;
          q[3] = s3;
        }
      }
      __syncthreads();
      if (t < nl * 4) {
        const int i = t >> 2, c = t & 3;
        double s = 0.0;
        for (int ww = 0; ww < ALM_WARPS; ww++) s += red[((size_t)ww * ALM_LC + i) * 4 + c];
        alm[(row + (size_t)(l0 + i - m)) * 4 + c] += s;
      }
    }
  }
}

/* alm2cl: cl[0] a x a, cl[1] a x b, cl[2] b x b, each [lmax + 1] */
__global__ void k_alm2cl(const double *__restrict__ alm, int lmax, double omega2,
                         double *__restrict__ cl) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l > lmax) return;
  double aa = 0.0, ab = 0.0, bb = 0.0;
  for (int m = 1; m <= l; m++) {
    const double *a = alm + (alm_row(m, lmax) + (size_t)(l - m)) * 4;
    aa += a[0] * a[0] + a[1] * a[1];
    ab += a[0] * a[2] + a[1] * a[3];
    bb += a[2] * a[2] + a[3] * a[3];
  }
  const double *a0 = alm + (size_t)l * 4; /* m = 0 */
  const double inv = omega2 / (2.0 * (double)l + 1.0);
  cl[l] = (2.0 * aa + (a0[0] * a0[0] - a0[1] * a0[1])) * inv;
  cl[lmax + 1 + l] = (2.0 * ab + (a0[0] * a0[2] - a0[1] * a0[3])) * inv;
  cl[2 * (lmax + 1) + l] = (2.0 * bb + (a0[2] * a0[2] - a0[3] * a0[3])) * inv;
}

/* ------------------------------------------------------------------ flat sky ---- */

__global__ void k_fs_pack(const float *__restrict__ a, const float *__restrict__ b, long long n,
                          double2 *__restrict__ z) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    z[i] = make_double2((double)a[i], b ? (double)b[i] : 0.0);
}

/* tw[k] = exp(-2 pi i k / n), k < n / 2 */
__global__ void k_twiddles(double2 *tw, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n / 2) return;
  double s, c;
  sincospi(2.0 * (double)k / (double)n, &s, &c);
  tw[k] = make_double2(c, -s);
}

/* in-place radix-2 FFT of each row (n a power of two, n >= 4), one block per row */
__global__ void __launch_bounds__(FFT_THREADS)
    k_fft_rows(double2 *__restrict__ z, int n, int logn, const double2 *__restrict__ tw) {
  extern __shared__ double2 sz[];
  double2 *row = z + (size_t)blockIdx.x * n;
  for (int j = threadIdx.x; j < n; j += FFT_THREADS) sz[__brev((unsigned)j) >> (32 - logn)] = row[j];
  __syncthreads();
  for (int half = 1; half < n; half <<= 1) {
    const int stride = n / (2 * half);
    for (int b = threadIdx.x; b < n / 2; b += FFT_THREADS) {
      const int pos = b & (half - 1);
      const int i0 = ((b - pos) << 1) + pos, i1 = i0 + half;
      const double2 w = tw[pos * stride], u = sz[i0], v = sz[i1];
      const double vr = v.x * w.x - v.y * w.y, vi = v.x * w.y + v.y * w.x;
      sz[i0] = make_double2(u.x + vr, u.y + vi);
      sz[i1] = make_double2(u.x - vr, u.y - vi);
    }
    __syncthreads();
  }
  for (int j = threadIdx.x; j < n; j += FFT_THREADS) row[j] = sz[j];
}

/* direct DFT of each row into out (any n <= DFT_MAX), one block per row */
__global__ void __launch_bounds__(256)
    k_dft_rows(const double2 *__restrict__ z, double2 *__restrict__ out, int n) {
  extern __shared__ double2 sr[];
  const double2 *row = z + (size_t)blockIdx.x * n;
  for (int j = threadIdx.x; j < n; j += blockDim.x) sr[j] = row[j];
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)k / (double)n, &s, &c);
    const double step_r = c, step_i = -s;
    double accr = 0.0, acci = 0.0, wr = 1.0, wi = 0.0;
    for (int j = 0; j < n; j++) {
      if ((j & 63) == 0) { /* exact twiddle every 64 terms */
        sincospi(2.0 * (double)(((long long)k * j) % n) / (double)n, &s, &c);
        wr = c;
        wi = -s;
      }
      const double2 x = sr[j];
      accr += x.x * wr - x.y * wi;
      acci += x.x * wi + x.y * wr;
      const double nr = wr * step_r - wi * step_i;
      wi = wr * step_i + wi * step_r;
      wr = nr;
    }
    out[(size_t)blockIdx.x * n + k] = make_double2(accr, acci);
  }
}

__global__ void k_transpose(const double2 *__restrict__ in, double2 *__restrict__ out, int n) {
  __shared__ double2 tile[32][33];
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
  for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
    const int x = x0 + threadIdx.x, y = y0 + dy;
    if (x < n && y < n) tile[dy][threadIdx.x] = in[(size_t)y * n + x];
  }
  __syncthreads();
  for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
    const int x = y0 + threadIdx.x, y = x0 + dy;
    if (x < n && y < n) out[(size_t)y * n + x] = tile[threadIdx.x][dy];
  }
}

/* per bin: modes, sum ell, |F_a|^2, Re F_a conj F_b, |F_b|^2 over |k1|, |k2| <= kmax */
__global__ void k_fs_bins(const double2 *__restrict__ z, int n, double ell_fund, double ell_max,
                          int nbins, int kmax, double *__restrict__ acc) {
  extern __shared__ double sb[];
  for (int i = threadIdx.x; i < nbins * 5; i += blockDim.x) sb[i] = 0.0;
  __syncthreads();
  const long long side = 2LL * kmax + 1, total = side * side;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int k1 = (int)(idx / side) - kmax, k2 = (int)(idx % side) - kmax;
    if (k1 == 0 && k2 == 0) continue;
    const double ell = ell_fund * sqrt((double)k1 * k1 + (double)k2 * k2);
    if (ell > ell_max) continue;
    const int b = min((int)(ell / ell_max * nbins), nbins - 1);
    const int i1 = (k1 + n) % n, i2 = (k2 + n) % n, j1 = (n - k1) % n, j2 = (n - k2) % n;
    const double2 zk = z[(size_t)i1 * n + i2], zm = z[(size_t)j1 * n + j2];
    /* F_a = (Z(k) + conj Z(-k)) / 2, F_b = (Z(k) - conj Z(-k)) / 2i */
    const double far = 0.5 * (zk.x + zm.x), fai = 0.5 * (zk.y - zm.y);
    const double fbr = 0.5 * (zk.y + zm.y), fbi = -0.5 * (zk.x - zm.x);
    atomicAdd(&sb[b * 5 + 0], 1.0);
    atomicAdd(&sb[b * 5 + 1], ell);
    atomicAdd(&sb[b * 5 + 2], far * far + fai * fai);
    atomicAdd(&sb[b * 5 + 3], far * fbr + fai * fbi);
    atomicAdd(&sb[b * 5 + 4], fbr * fbr + fbi * fbi);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nbins * 5; i += blockDim.x)
    if (sb[i] != 0.0) atomicAdd(&acc[i], sb[i]);
}

/* device buffers released on every return path */
struct DevBufs {
  std::vector<void *> p;
  ~DevBufs() {
    for (void *q : p) cudaFree(q);
  }
  template <class T>
  cudaError_t get(T **out, size_t bytes) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes ? bytes : 1);
    if (e == cudaSuccess) p.push_back(q);
    *out = (T *)q;
    return e;
  }
};

struct DeviceScope {
  int prev = -1;
  bool ok = false;
  explicit DeviceScope(int dev) {
    if (cudaGetDevice(&prev) == cudaSuccess && cudaSetDevice(dev) == cudaSuccess) ok = true;
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

struct Stream {
  cudaStream_t s = nullptr;
  Stream() { cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking); }
  ~Stream() {
    if (s) cudaStreamDestroy(s);
  }
};

#define SP_CK(x)                                                   \
  do {                                                             \
    cudaError_t e_ = (x);                                          \
    if (e_ != cudaSuccess) {                                       \
      cudaGetLastError();                                          \
      return e_ == cudaErrorMemoryAllocation ? P2M_ERR_NOMEM : P2M_ERR_CUDA; \
    }                                                              \
  } while (0)

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) l++;
  return l;
}

}  // namespace

extern "C" {

int32_t p2m_cl_healpix(int32_t device, const float *map_a, const float *map_b, int32_t nside,
                       int32_t lmax, double *cl_aa, double *cl_ab, double *cl_bb) {
  if (!map_a || !cl_aa || !is_pow2(nside) || nside > 8192 || lmax < 0 ||
      lmax > 4 * nside || lmax > P2M_CL_LMAX_MAX)
    return P2M_ERR_BADARG;
  if (map_b && (!cl_ab || !cl_bb)) return P2M_ERR_BADARG;
  DeviceScope scope(device);
  if (!scope.ok) return P2M_ERR_CUDA;
  Stream st;
  if (!st.s) return P2M_ERR_CUDA;
  DevBufs B;
  const long long npix = 12LL * nside * nside;
  const int nrings = 2 * nside;
  const size_t nalm = alm_row(lmax + 1, lmax); /* (lmax + 1)(lmax + 2) / 2 */
  float *d_a = nullptr, *d_b = nullptr;
  double *d_ph = nullptr, *d_alm = nullptr, *d_mfac = nullptr, *d_cl = nullptr;
  SP_CK(B.get(&d_a, sizeof(float) * (size_t)npix));
  if (map_b) SP_CK(B.get(&d_b, sizeof(float) * (size_t)npix));
  SP_CK(B.get(&d_ph, sizeof(double) * 8 * (size_t)nrings * (size_t)(lmax + 1)));
  SP_CK(B.get(&d_alm, sizeof(double) * 4 * nalm));
  SP_CK(B.get(&d_mfac, sizeof(double) * (size_t)(lmax + 1)));
  SP_CK(B.get(&d_cl, sizeof(double) * 3 * (size_t)(lmax + 1)));
  /* gen_mfac: log2(prod_{k<=m} sqrt((2k+1)/(2k)) / sqrt(4 pi)) */
  std::vector<double> mfac((size_t)lmax + 1);
  {
    double f = 1.0;
    const double sq4pi_inv = 1.0 / std::sqrt(4.0 * M_PI), aln2_inv = 1.0 / std::log(2.0);
    for (int m = 0; m <= lmax; m++) {
      if (m > 0) f *= std::sqrt((double)(2 * m + 1) / (double)(2 * m));
      mfac[(size_t)m] = std::log(sq4pi_inv * f) * aln2_inv;
    }
  }
  SP_CK(cudaMemcpyAsync(d_a, map_a, sizeof(float) * (size_t)npix, cudaMemcpyHostToDevice, st.s));
  if (map_b)
    SP_CK(cudaMemcpyAsync(d_b, map_b, sizeof(float) * (size_t)npix, cudaMemcpyHostToDevice, st.s));
  SP_CK(cudaMemcpyAsync(d_mfac, mfac.data(), sizeof(double) * mfac.size(), cudaMemcpyHostToDevice,
                        st.s));
  SP_CK(cudaMemsetAsync(d_alm, 0, sizeof(double) * 4 * nalm, st.s));
  k_ring_phases<<<dim3(nrings, (lmax + RP_THREADS) / RP_THREADS), RP_THREADS, 0, st.s>>>(
      d_a, d_b, nside, lmax, d_ph);
  SP_CK(cudaGetLastError());
  const size_t smem = sizeof(double) * ((size_t)ALM_GROUP * 8 + 2 * ALM_LC +
                                        (size_t)ALM_WARPS * ALM_LC * 4);
  SP_CK(cudaFuncSetAttribute(k_alm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_alm<<<lmax + 1, ALM_THREADS, smem, st.s>>>(d_ph, d_mfac, nside, lmax, d_alm);
  SP_CK(cudaGetLastError());
  const double omega = 4.0 * M_PI / (double)npix;
  k_alm2cl<<<(lmax + 128) / 128, 128, 0, st.s>>>(d_alm, lmax, omega * omega, d_cl);
  SP_CK(cudaGetLastError());
  std::vector<double> cl(3 * (size_t)(lmax + 1));
  SP_CK(cudaMemcpyAsync(cl.data(), d_cl, sizeof(double) * cl.size(), cudaMemcpyDeviceToHost, st.s));
  SP_CK(cudaStreamSynchronize(st.s));
  const size_t nl = (size_t)lmax + 1;
  for (size_t l = 0; l < nl; l++) {
    cl_aa[l] = cl[l];
    if (map_b) {
      cl_ab[l] = cl[nl + l];
      cl_bb[l] = cl[2 * nl + l];
    }
  }
  return P2M_OK;
}

int32_t p2m_cl_flatsky(int32_t device, const float *map_a, const float *map_b, int32_t npix,
                       float fov_rad, double ell_max, int32_t nbins, double *ell_mean,
                       double *cl_aa, double *cl_ab, double *cl_bb, int64_t *nmodes) {
  if (!map_a || !ell_mean || !cl_aa || !nmodes || npix < 2 || !(fov_rad > 0.0f) ||
      !(ell_max > 0.0) || nbins < 1 || nbins > P2M_CL_MAXBINS)
    return P2M_ERR_BADARG;
  if (map_b && (!cl_ab || !cl_bb)) return P2M_ERR_BADARG;
  const bool pow2 = is_pow2(npix) && npix >= 4;
  if (pow2 ? npix > FFT_MAX_POW2 : npix > DFT_MAX) return P2M_ERR_BADARG;
  DeviceScope scope(device);
  if (!scope.ok) return P2M_ERR_CUDA;
  Stream st;
  if (!st.s) return P2M_ERR_CUDA;
  DevBufs B;
  const long long n2 = (long long)npix * npix;
  float *d_a = nullptr, *d_b = nullptr;
  double2 *z = nullptr, *z2 = nullptr, *tw = nullptr;
  double *d_acc = nullptr;
  SP_CK(B.get(&d_a, sizeof(float) * (size_t)n2));
  if (map_b) SP_CK(B.get(&d_b, sizeof(float) * (size_t)n2));
  SP_CK(B.get(&z, sizeof(double2) * (size_t)n2));
  SP_CK(B.get(&z2, sizeof(double2) * (size_t)n2));
  SP_CK(B.get(&tw, sizeof(double2) * (size_t)(npix / 2 + 1)));
  SP_CK(B.get(&d_acc, sizeof(double) * 5 * (size_t)nbins));
  SP_CK(cudaMemcpyAsync(d_a, map_a, sizeof(float) * (size_t)n2, cudaMemcpyHostToDevice, st.s));
  if (map_b)
    SP_CK(cudaMemcpyAsync(d_b, map_b, sizeof(float) * (size_t)n2, cudaMemcpyHostToDevice, st.s));
  SP_CK(cudaMemsetAsync(d_acc, 0, sizeof(double) * 5 * (size_t)nbins, st.s));
  k_fs_pack<<<(int)std::min<long long>((n2 + 255) / 256, 4096), 256, 0, st.s>>>(d_a, d_b, n2, z);
  SP_CK(cudaGetLastError());
  const dim3 tb(32, 8), tg((npix + 31) / 32, (npix + 31) / 32);
  if (pow2) {
    const int logn = ilog2(npix);
    const size_t smem = sizeof(double2) * (size_t)npix;
    SP_CK(cudaFuncSetAttribute(k_fft_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_twiddles<<<(npix / 2 + 255) / 256, 256, 0, st.s>>>(tw, npix);
    k_fft_rows<<<npix, FFT_THREADS, smem, st.s>>>(z, npix, logn, tw);
    k_transpose<<<tg, tb, 0, st.s>>>(z, z2, npix);
    k_fft_rows<<<npix, FFT_THREADS, smem, st.s>>>(z2, npix, logn, tw);
  } else {
    const size_t smem = sizeof(double2) * (size_t)npix;
    k_dft_rows<<<npix, 256, smem, st.s>>>(z, z2, npix);
    k_transpose<<<tg, tb, 0, st.s>>>(z2, z, npix);
    k_dft_rows<<<npix, 256, smem, st.s>>>(z, z2, npix);
  }
  SP_CK(cudaGetLastError());
  const double ell_fund = 2.0 * M_PI / (double)fov_rad;
  int kmax = (int)std::ceil(ell_max / ell_fund);
  kmax = std::min(kmax, npix / 2 - 1); /* the Nyquist line is left out */
  if (kmax >= 1) {
    const long long total = (2LL * kmax + 1) * (2LL * kmax + 1);
    const int grid = (int)std::min<long long>((total + 255) / 256, 1024);
    k_fs_bins<<<grid, 256, sizeof(double) * 5 * (size_t)nbins, st.s>>>(
        z2, npix, ell_fund, ell_max, nbins, kmax, d_acc);
    SP_CK(cudaGetLastError());
  }
  std::vector<double> acc(5 * (size_t)nbins);
  SP_CK(cudaMemcpyAsync(acc.data(), d_acc, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost,
                        st.s));
  SP_CK(cudaStreamSynchronize(st.s));
  const double fov = (double)fov_rad, n4 = (double)n2 * (double)n2;
  const double norm = fov * fov / n4;
  for (int b = 0; b < nbins; b++) {
    const double *q = &acc[5 * (size_t)b];
    const double cnt = q[0];
    nmodes[b] = (int64_t)cnt;
    ell_mean[b] = cnt > 0 ? q[1] / cnt : (b + 0.5) * ell_max / nbins;
    cl_aa[b] = cnt > 0 ? norm * q[2] / cnt : 0.0;
    if (map_b) {
      cl_ab[b] = cnt > 0 ? norm * q[3] / cnt : 0.0;
      cl_bb[b] = cnt > 0 ? norm * q[4] / cnt : 0.0;
    }
  }
  return P2M_OK;
}

}  // extern "C"
