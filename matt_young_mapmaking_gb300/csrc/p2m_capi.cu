/*
 * p2m_capi.cu -- the C ABI of include/p2m.h: context, device buffers, and the order of
 * kernel launches.  A paint call ingests records (one host round trip, to size the item
 * buffer); the HEALPix maps are produced by one sweep over everything ingested since the
 * last read, started by the first read of a map.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/p2m.h"
#include "../../include/p2m_tools.h"
#include "p2m_fits.h"
#include "p2m_internal.h"

enum {
  PH_CUT, PH_SETUP, PH_SCAN, PH_ITEMS, PH_FS, PH_GROUP, PH_PAINT, PH_PAINT_BIG, PH_READOUT,
  P2M_NPHASE
};

struct p2m_ctx {
  p2m_config cfg;
  int nsm = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  p2m_cosmo cosmo;
  std::vector<float> rofz_host, zofr_host;
  float *d_rofz = nullptr, *d_zofr = nullptr;
  /* map statistics: three FP64 sums and the P(<y) bin counts */
  double *d_mstat = nullptr;
  unsigned int *d_hist = nullptr;
  /* FITS writer: big-endian slices of a map on the device and in pinned host memory */
  unsigned int *d_fits[2] = {nullptr, nullptr}, *h_fits[2] = {nullptr, nullptr};
  cudaEvent_t ev_fits[2] = {nullptr, nullptr};
  float4 *d_ringtab = nullptr;
  float2 *d_ringhd = nullptr;
  float4 *d_phitab = nullptr;
  /* scramble / centre of the catalogue (pks2map.f90:162-262) */
  p2m_pre pre = {};
  unsigned int *d_pre_flags = nullptr, *d_pre_bits = nullptr;
  long long *d_pre_ord = nullptr, *d_pre_last = nullptr;
  long long cap_pre_flags = 0, cap_pre_ord = 0, cap_pre_last = 0;
  float centre_info[9] = {};
  p2m_tabhdr th;
  bool th_set = false;
  float *d_tab[P2M_MAXTABLES] = {};
  /* pair tables (PaintParams::pair_tab), set up by the first ingest after a table load:
     a gathered copy where a pair of maps is not profiles 1 and 2 of one table */
  float2 *d_pair[P2M_MAXMAPS / 2] = {};
  long long cap_pair[P2M_MAXMAPS / 2] = {};
  const float2 *pair_tab[P2M_MAXMAPS / 2] = {};
  bool pairs_ok = false;
  float band_u = 2e-4f;
  p2m_tuning tune = {P2M_BIG_RINGS, 8, 8, 1024, (int32_t)P2M_STREAM_CHUNK, 1, 16, 1, 128, 0.0f};
  /* painting order (p2m_tuning.sort_halos): counting sort by first ring */
  int *d_order = nullptr, *d_ring_key = nullptr;
  long long cap_order = 0, cap_ring_key = 0;
  unsigned int *d_ring_hist = nullptr;
  long long *d_ring_off = nullptr;
  unsigned long long *d_nbins = nullptr;
  /* outputs: hp_npix counts every cone's pixels (ncones * cone_npix) */
  long long hp_npix = 0, fs_npix = 0;
  long long cone_npix = 0;
  int ncones = 1;
  long long *d_cone_off = nullptr; /* first record of each cone of the current call */
  std::vector<long long> cone_off_host;
  float *d_out_own[P2M_MAXMAPS] = {};
  float *d_out[P2M_MAXMAPS] = {};
  double *d_acc64 = nullptr; /* full-sky FP64 accumulator (plain and FP64-accumulating paths) */
  /* compensated path: the output maps accumulate the high words; low words and their
     dirty-tile flags stay zero between sweeps */
  float *d_lo = nullptr;
  unsigned char *d_tiles = nullptr;
  bool outs_zeroed = false;
  void *d_fs_acc = nullptr;
  float *d_fs_out = nullptr;
  /* ingest state (accumulated until the next sweep) */
  HaloRec *d_halos = nullptr;
  long long cap_halos = 0, n_halos = 0;
  RingItem *d_items_raw = nullptr; /* items of the large halos */
  long long cap_items_raw = 0, n_items = 0;
  long long rec_count = 0;
  bool dirty = false, swept = false;
  bool unfolded = false; /* painted into the accumulators, read-out not yet run */
  long long pending_recs = 0; /* records ingested since the last paint */
  /* per-call buffers */
  /* streamed ingest of host records: two device staging buffers filled on a copy stream
     while the previous chunk is cut and set up */
  cudaStream_t cstream = nullptr;
  /* asynchronous read-outs (p2m_get_healpix_async): copies on their own stream; the buffer
     each map's last one reads, and the event that marks its end */
  cudaStream_t rstream = nullptr;
  cudaEvent_t ev_ready = nullptr;
  /* one guard per buffer with a read-out queued: its last copy's end; a guard is reused
     (after a host wait for its copy) when more buffers than guards are in flight */
  static const int NGUARD = 4 * P2M_MAXMAPS;
  const float *rd_buf[NGUARD] = {};
  cudaEvent_t rd_ev[NGUARD] = {};
  unsigned long long rd_seq[NGUARD] = {}, rd_clock = 0;
  float *d_stage[2] = {nullptr, nullptr};
  long long cap_stage[2] = {0, 0};
  cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_consumed[2] = {nullptr, nullptr};
  unsigned int *d_nring = nullptr;
  long long cap_nring = 0;
  long long *d_ioff = nullptr;
  long long cap_ioff = 0;
  FsItem *d_fs_items = nullptr;
  long long cap_fs = 0;
  long long *d_scan_tmp = nullptr;
  /* sweep buffers */
  unsigned int *d_counts = nullptr;
  long long cap_counts = 0;
  long long *d_pix_off = nullptr;
  long long cap_pix_off = 0;
  unsigned long long *d_nitems = nullptr;
  double *d_sums = nullptr; /* [0, MAXMAPS): HEALPix, [MAXMAPS, 2 MAXMAPS): flat sky */
  long long *d_set_rec = nullptr, *d_set_pix = nullptr;
  long long cap_set = 0;
  DevCounters *d_ctr = nullptr, *h_ctr = nullptr; /* h_ctr: mapped pinned host memory */
  DevCounters *h_ctr_dev = nullptr;                /* its device address */
  float *d_prep = nullptr;
  long long cap_prep = 0;
  std::vector<float> prep;
  long long n_records = 0;
  cudaEvent_t ev_join = nullptr, ev_back = nullptr;
  /* the compensated path's output clear runs on its own stream, beside the ingest */
  cudaStream_t zstream = nullptr;
  cudaEvent_t ev_zero_start = nullptr, ev_zero_done = nullptr;
  bool zero_pending = false;
  cudaEvent_t tev[P2M_NPHASE][2] = {};
  bool tev_used[P2M_NPHASE] = {};
};

namespace {

p2m_status fail(p2m_ctx *c, p2m_status s, const std::string &msg) {
  if (c) c->err = msg;
  return s;
}

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(ctx, P2M_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define ST(call)                    \
  do {                              \
    p2m_status st_ = (call);        \
    if (st_ != P2M_OK) return st_;  \
  } while (0)

/* grows a device buffer to at least `need` elements; keeps the first `keep` elements */
template <typename T>
cudaError_t grow(T **p, long long *cap, long long need, long long keep = 0, cudaStream_t s = 0) {
  if (need <= *cap && *p) return cudaSuccess;
  long long n = std::max(need + need / 4, (long long)1024);
  T *q = nullptr;
  cudaError_t e = cudaMalloc((void **)&q, sizeof(T) * (size_t)n);
  if (e != cudaSuccess) return e;
  if (*p && keep > 0) {
    e = cudaMemcpyAsync(q, *p, sizeof(T) * (size_t)keep, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      cudaFree(q);
      return e;
    }
  }
  if (*p) cudaFree(*p);
  *p = q;
  *cap = n;
  return cudaSuccess;
}

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

void tmark(p2m_ctx *ctx, int ph, int end, cudaStream_t s) {
  if (!(ctx->cfg.flags & P2M_FLAG_TIMING)) return;
  if (!ctx->tev[ph][end]) cudaEventCreate(&ctx->tev[ph][end]);
  cudaEventRecord(ctx->tev[ph][end], s);
  if (end) ctx->tev_used[ph] = true;
}
#define TB(ph) tmark(ctx, ph, 0, s)
#define TE(ph) tmark(ctx, ph, 1, s)

/* work queued on the context stream before a call on stream s runs first; work queued
   on the context stream after it waits for s */
void join_in(p2m_ctx *ctx, cudaStream_t s) {
  if (s == ctx->stream) return;
  cudaEventRecord(ctx->ev_join, ctx->stream);
  cudaStreamWaitEvent(s, ctx->ev_join, 0);
}
void join_out(p2m_ctx *ctx, cudaStream_t s) {
  if (s == ctx->stream) return;
  cudaEventRecord(ctx->ev_back, s);
  cudaStreamWaitEvent(ctx->stream, ctx->ev_back, 0);
}

/* per-call counters precede the cumulative ones in DevCounters */
const size_t CALL_CTR_BYTES = offsetof(DevCounters, hp_updates);

PaintParams make_params(const p2m_ctx *ctx, int nfloat) {
  PaintParams P;
  memset(&P, 0, sizeof(P));
  const p2m_config &c = ctx->cfg;
  P.nside = c.nside;
  P.npix_fs = c.npix_fs;
  P.nmaps = c.nmaps;
  P.precision = c.precision;
  P.flags = c.flags;
  P.nfloat = nfloat;
  P.model = c.model;
  P.cosmo = ctx->cosmo;
  const float mypi = ctx->cosmo.mypi;
  /* pks2map.f90:92-93 */
  P.fov = FMUL(FMUL(FDIV(c.fov_deg, 360.0f), 2.0f), mypi);
  P.dpix = c.npix_fs > 0 ? FDIV(P.fov, (float)c.npix_fs) : 0.0f;
  P.hf = FDIV(P.fov, 2.0f);
  /* pks2map.f90:134-135 */
  P.cut_low = p2m_lookup(ctx->rofz_host.data(), ctx->cosmo.drofz, c.zmin);
  P.cut_high = p2m_lookup(ctx->rofz_host.data(), ctx->cosmo.drofz, c.zmax);
  P.chihview = c.chihview;
  static const float bbps_delta[3] = {200.0f, 500.0f, 200.0f}; /* bbps_profile.f90:21 */
  P.bbps_delta = bbps_delta[c.model - 1];
  for (int m = 0; m < P2M_MAXMAPS; m++) {
    P.map_table[m] = m < c.nmaps ? c.map_table[m] : 0;
    P.map_profile[m] = m < c.nmaps ? c.map_profile[m] : 1;
    if (m < c.nmaps && c.map_profile[m] == 2) P.any_ksz = 1;
  }
  P.mass_fac = FMUL(FMUL(4.0f / 3.0f, mypi), ctx->cosmo.rho_0);
  P.th = ctx->th;
  for (int t = 0; t < P2M_MAXTABLES; t++) P.tables[t] = ctx->d_tab[t];
  for (int q = 0; q < P2M_MAXMAPS / 2; q++) P.pair_tab[q] = ctx->pair_tab[q];
  P.rofz = ctx->d_rofz;
  P.zofr = ctx->d_zofr;
  P.ringtab = ctx->d_ringtab;
  P.ringhd = ctx->d_ringhd;
  P.phitab = ctx->d_phitab;
  P.pre = ctx->pre;
  P.pre_ord = ctx->d_pre_ord;
  P.band_u = ctx->band_u;
  P.inv_drt = ctx->th_set ? 1.0f / ctx->th.drt : 0.0f;
  P.big_rings = ctx->tune.big_rings;
  P.halos_grid = ctx->tune.halos_grid;
  P.full_grid = ctx->tune.full_grid;
  P.full_chunk = ctx->tune.full_chunk;
  P.halo_batch = ctx->tune.halo_batch;
  P.halos_threads = ctx->tune.halos_threads;
  P.err_flag = &ctx->d_ctr->err;
  P.cone_npix = ctx->cone_npix;
  if (ctx->th_set) {
    float fr;
    int ir;
    p2m_rindex(&ctx->th, FMUL(ctx->th.rmint, 0.5f), &ir, &fr);
    P.ir_c = ir;
    P.fr_c = fr;
  }
  return P;
}

IngestBuffers ingest_buffers(const p2m_ctx *ctx, const float *records) {
  IngestBuffers B;
  memset(&B, 0, sizeof(B));
  B.records = records;
  B.rec_base = ctx->rec_count;
  B.halos = ctx->d_halos + ctx->n_halos;
  B.halo_base = ctx->n_halos;
  B.nring = ctx->d_nring;
  B.ioff = ctx->d_ioff;
  B.items = ctx->d_items_raw + ctx->n_items;
  B.fs_items = ctx->d_fs_items;
  B.fs_cap = ctx->cap_fs;
  B.fs_acc = ctx->d_fs_acc;
  B.scan_tmp = ctx->d_scan_tmp;
  B.ctr = ctx->d_ctr;
  B.set_rec = ctx->d_set_rec;
  B.set_pix = ctx->d_set_pix;
  B.set_cap = ctx->cap_set;
  if (ctx->tune.sort_halos && ctx->d_ring_hist) {
    B.ring_key = ctx->d_ring_key + ctx->n_halos;
    B.ring_hist = ctx->d_ring_hist;
  }
  return B;
}

/* checks that every map's table is loaded, and sets up the pair tables after a table
   load: maps 2q and 2q + 1 read their values from one table of float2 entries, the
   interleaved table itself when the pair is its profiles 1 and 2 (or a lone last map
   is its profile 1), else a copy gathered on the context's stream */
p2m_status check_tables(p2m_ctx *ctx) {
  const p2m_config &c = ctx->cfg;
  for (int m = 0; m < c.nmaps; m++)
    if (!ctx->d_tab[c.map_table[m]])
      return fail(ctx, P2M_ERR_STATE, "table slot " + std::to_string(c.map_table[m]) +
                                          " used by map " + std::to_string(m) + " is not loaded");
  if (ctx->pairs_ok) return P2M_OK;
  const long long nent = ctx->th.nelem / 2;
  for (int q = 0; q < P2M_MAXMAPS / 2; q++) {
    ctx->pair_tab[q] = nullptr;
    const int a = 2 * q, b = 2 * q + 1;
    if (a >= c.nmaps) continue;
    const int ta = c.map_table[a], pa = c.map_profile[a];
    const bool two = b < c.nmaps;
    const int tb = two ? c.map_table[b] : ta;
    const int pb = two ? c.map_profile[b] : (pa == 1 ? 2 : pa);
    if (ta == tb && pa == 1 && pb == 2) {
      ctx->pair_tab[q] = (const float2 *)ctx->d_tab[ta];
      continue;
    }
    CK(grow(&ctx->d_pair[q], &ctx->cap_pair[q], nent));
    p2m_launch_pair_table(ctx->d_pair[q], ctx->d_tab[ta], pa, ctx->d_tab[tb], pb, nent,
                          ctx->stream, ctx->nsm);
    CK(cudaGetLastError());
    ctx->pair_tab[q] = ctx->d_pair[q];
  }
  ctx->pairs_ok = true;
  return P2M_OK;
}

/* reports the device error flags in the counters last copied to host memory (after a
   wait for them); a flag stays set on the device until it is reported here, and is
   reported once: both copies are cleared */
p2m_status check_errors(p2m_ctx *ctx, cudaStream_t s) {
  const unsigned int err = ctx->h_ctr->err;
  if (err) {
    ctx->h_ctr->err = 0;
    CK(cudaMemsetAsync(&ctx->d_ctr->err, 0, sizeof(unsigned int), s));
  }
  if (err & P2M_DEVERR_RADIUS)
    return fail(ctx, P2M_ERR_BADARG, "a halo's disc radius exceeds pi (query_disc aborts)");
  if (err & P2M_DEVERR_ITEMS)
    return fail(ctx, P2M_ERR_STATE, "candidate walk exceeded its round bound (maps are incomplete)");
  if (err & P2M_DEVERR_FS_OVERFLOW)
    return fail(ctx, P2M_ERR_CAPACITY, "flat-sky row buffer overflow (maps are incomplete)");
  if (err & P2M_DEVERR_FIXED)
    return fail(ctx, P2M_ERR_CAPACITY,
                "fixed-point accumulation out of range (a value or a pixel sum of 128 or more): "
                "paint these tables with another precision");
  return P2M_OK;
}

p2m_status read_counters(p2m_ctx *ctx, cudaStream_t s) {
  p2m_launch_copy_counters(ctx->d_ctr, ctx->h_ctr_dev, s);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  return check_errors(ctx, s);
}

/* Everything after the per-halo set-up of one ingest call: item offsets, items, flat sky.
   The set-up kernel has been queued on s; n_max bounds the halo count. */
p2m_status ingest_tail(p2m_ctx *ctx, const PaintParams &P, long long n_max, cudaStream_t s) {
  IngestBuffers B = ingest_buffers(ctx, nullptr);
  /* the large halos reserved their item ranges (d_ioff, n_items) during the set-up */
  const p2m_status err = read_counters(ctx, s);
  if (err) {
    /* the call is discarded: its halos, stored past n_halos, are overwritten by the next
       call, and they leave the first-ring counts that the next sort scans */
    if (ctx->tune.sort_halos && ctx->d_ring_hist && ctx->h_ctr->n_surv > 0)
      p2m_launch_ring_unhist(ctx->d_ring_key + ctx->n_halos, (long long)ctx->h_ctr->n_surv,
                             ctx->d_ring_hist, s, ctx->nsm);
    return err;
  }
  long long n_halo = (long long)ctx->h_ctr->n_surv;
  long long n_items = P.nside > 0 ? (long long)ctx->h_ctr->n_items : 0;
  long long n_fs = (long long)ctx->h_ctr->n_fs_rows;
  (void)n_max;
  CK(grow(&ctx->d_items_raw, &ctx->cap_items_raw, ctx->n_items + std::max(n_items, 1LL),
          ctx->n_items, s));
  CK(grow(&ctx->d_fs_items, &ctx->cap_fs, std::max(n_fs, 1LL)));
  B = ingest_buffers(ctx, nullptr);
  if (n_halo > 0) {
    if (P.nside > 0 && n_items > 0) {
      TB(PH_ITEMS);
      p2m_launch_items(P, B, n_halo, s, ctx->nsm);
      TE(PH_ITEMS);
    }
    if (P.npix_fs > 0 && n_fs > 0) {
      TB(PH_FS);
      p2m_launch_fs(P, B, n_halo, s, ctx->nsm);
      TE(PH_FS);
    }
  }
  CK(cudaGetLastError());
  ctx->n_halos += n_halo;
  ctx->n_items += n_items;
  if (n_halo > 0) ctx->dirty = true;
  return P2M_OK;
}

bool compensated(const p2m_ctx *ctx) { return ctx->d_lo != nullptr; }

/* the compensated path accumulates into the output maps: clear them before the first
   paint after a reset (the buffers bound at that time).  The clear is bandwidth-bound
   and independent of the ingest, so it runs on a side stream after the work already on
   s; the sweep waits for it before painting. */
p2m_status wait_reads(p2m_ctx *ctx, cudaStream_t s);

p2m_status zero_outputs(p2m_ctx *ctx, cudaStream_t s) {
  if (!compensated(ctx) || ctx->outs_zeroed) return P2M_OK;
  CK(cudaEventRecord(ctx->ev_zero_start, s));
  CK(cudaStreamWaitEvent(ctx->zstream, ctx->ev_zero_start, 0));
  ST(wait_reads(ctx, ctx->zstream));
  for (int m = 0; m < ctx->cfg.nmaps; m++)
    CK(cudaMemsetAsync(ctx->d_out[m], 0, sizeof(float) * (size_t)ctx->hp_npix, ctx->zstream));
  CK(cudaEventRecord(ctx->ev_zero_done, ctx->zstream));
  ctx->zero_pending = true;
  ctx->outs_zeroed = true;
  return P2M_OK;
}

/* orders s after the asynchronous read-outs that may still be copying a map buffer bound
   now, so that nothing writes a map while it is being read out */
p2m_status wait_reads(p2m_ctx *ctx, cudaStream_t s) {
  for (int r = 0; r < p2m_ctx::NGUARD; r++) {
    if (!ctx->rd_buf[r]) continue;
    for (int m = 0; m < ctx->cfg.nmaps; m++)
      if (ctx->d_out[m] == ctx->rd_buf[r]) {
        CK(cudaStreamWaitEvent(s, ctx->rd_ev[r], 0));
        break;
      }
  }
  return P2M_OK;
}

/* orders s after a pending clear of the output maps */
p2m_status wait_zero(p2m_ctx *ctx, cudaStream_t s) {
  if (!ctx->zero_pending) return P2M_OK;
  CK(cudaStreamWaitEvent(s, ctx->ev_zero_done, 0));
  if (s != ctx->stream) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_zero_done, 0));
  ctx->zero_pending = false;
  return P2M_OK;
}

p2m_status begin_call(p2m_ctx *ctx, long long n, cudaStream_t s) {
  ST(zero_outputs(ctx, s));
  CK(grow(&ctx->d_nring, &ctx->cap_nring, std::max(n, 1LL)));
  CK(grow(&ctx->d_ioff, &ctx->cap_ioff, std::max(n, 1LL)));
  CK(grow(&ctx->d_halos, &ctx->cap_halos, ctx->n_halos + std::max(n, 1LL), ctx->n_halos, s));
  if (ctx->tune.sort_halos && ctx->cfg.nside > 0) {
    CK(grow(&ctx->d_ring_key, &ctx->cap_ring_key, ctx->n_halos + std::max(n, 1LL), ctx->n_halos, s));
    if (!ctx->d_ring_hist) {
      const long long nbins = 4LL * ctx->cfg.nside + 1;
      CK(cudaMalloc((void **)&ctx->d_ring_hist, sizeof(unsigned int) * (size_t)nbins));
      CK(cudaMemset(ctx->d_ring_hist, 0, sizeof(unsigned int) * (size_t)nbins));
      CK(cudaMalloc((void **)&ctx->d_ring_off, sizeof(long long) * (size_t)nbins));
      CK(cudaMalloc((void **)&ctx->d_nbins, sizeof(unsigned long long)));
      const unsigned long long nb = (unsigned long long)nbins;
      CK(cudaMemcpy(ctx->d_nbins, &nb, sizeof(nb), cudaMemcpyHostToDevice));
    }
  }
  for (int k = 0; k < P2M_NPHASE; k++) ctx->tev_used[k] = false;
  CK(cudaMemsetAsync(ctx->d_ctr, 0, CALL_CTR_BYTES, s));
  return P2M_OK;
}

p2m_status flush_prepared(p2m_ctx *ctx) {
  if (ctx->prep.empty()) return P2M_OK;
  ST(check_tables(ctx));
  cudaStream_t s = ctx->stream;
  long long n = (long long)ctx->prep.size() / 9;
  CK(grow(&ctx->d_prep, &ctx->cap_prep, (long long)ctx->prep.size()));
  CK(cudaMemcpyAsync(ctx->d_prep, ctx->prep.data(), sizeof(float) * ctx->prep.size(),
                     cudaMemcpyHostToDevice, s));
  ST(begin_call(ctx, n, s));
  PaintParams P = make_params(ctx, 7);
  IngestBuffers B = ingest_buffers(ctx, nullptr);
  /* every queued halo is enumerated: n_surv = n */
  unsigned long long nn = (unsigned long long)n;
  CK(cudaMemcpyAsync(&ctx->d_ctr->n_surv, &nn, sizeof(nn), cudaMemcpyHostToDevice, s));
  TB(PH_SETUP);
  p2m_launch_setup_prepared(P, B, ctx->d_prep, n, s, ctx->nsm);
  TE(PH_SETUP);
  CK(cudaStreamSynchronize(s)); /* nn and prep are host memory */
  ctx->prep.clear();
  ST(ingest_tail(ctx, P, n, s));
  ctx->rec_count += n;
  return P2M_OK;
}

/* scramble / centre (pks2map.f90:162-262) of the whole catalogue in d_rec: survivor
   ordinals for the rank streams, and the flips and angles that put the largest-RTH
   halo on the z axis (computed on the host with the kernels' own arithmetic) */
p2m_status preprocess(p2m_ctx *ctx, const float *d_rec, long long nrec, int nfloat,
                      cudaStream_t s) {
  p2m_pre &q = ctx->pre;
  const int ntasks = q.ntasks > 1 ? q.ntasks : 1;
  q.per_rank = nrec > 0 ? (nrec - 1) / ntasks + 1 : 1;
  q.flip[0] = q.flip[1] = q.flip[2] = 0;
  q.ct = q.cp = 1.0f;
  q.st = q.sp = 0.0f;
  const int centre = q.centre;
  q.centre = 0; /* the flags, ordinals and search see the positions before rotation */
  PaintParams P = make_params(ctx, nfloat);
  CK(grow(&ctx->d_pre_flags, &ctx->cap_pre_flags, nrec));
  CK(grow(&ctx->d_pre_ord, &ctx->cap_pre_ord, nrec));
  p2m_launch_pre_flags(P, d_rec, nrec, ctx->d_pre_flags, s, ctx->nsm);
  unsigned long long nn = (unsigned long long)nrec;
  CK(cudaMemcpyAsync(ctx->d_nitems, &nn, sizeof(nn), cudaMemcpyHostToDevice, s));
  p2m_launch_scan_u32(ctx->d_pre_flags, ctx->d_nitems, ctx->d_pre_ord, nullptr, ctx->d_scan_tmp, s);
  for (int k = 0; k < 9; k++) ctx->centre_info[k] = 0.0f;
  if (centre) {
    CK(grow(&ctx->d_pre_last, &ctx->cap_pre_last, ntasks));
    CK(cudaMemsetAsync(ctx->d_pre_last, 0xff, sizeof(long long) * (size_t)ntasks, s));
    CK(cudaMemsetAsync(ctx->d_pre_bits, 0, sizeof(unsigned int), s));
    P.pre_ord = ctx->d_pre_ord;
    p2m_launch_pre_centre(P, d_rec, nrec, ctx->d_pre_flags, ctx->d_pre_bits, ctx->d_pre_last, s,
                          ctx->nsm);
    CK(cudaGetLastError());
    std::vector<long long> last((size_t)ntasks);
    unsigned int bits = 0;
    CK(cudaMemcpyAsync(last.data(), ctx->d_pre_last, sizeof(long long) * (size_t)ntasks,
                       cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&bits, ctx->d_pre_bits, sizeof(bits), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    float rthmax;
    memcpy(&rthmax, &bits, 4);
    /* per rank the last survivor holding RTHmax, then MAX over ranks per coordinate */
    float xm = -1e5f, ym = -1e5f, zm = -1e5f;
    for (int r = 0; r < ntasks; r++) {
      if (last[(size_t)r] < 0) continue;
      const long long i = last[(size_t)r];
      float pos[3];
      CK(cudaMemcpy(pos, d_rec + i * nfloat, sizeof(pos), cudaMemcpyDeviceToHost));
      if (q.scramble) {
        long long oi = 0, ob = 0;
        CK(cudaMemcpy(&oi, ctx->d_pre_ord + i, sizeof(oi), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&ob, ctx->d_pre_ord + (long long)r * q.per_rank, sizeof(ob),
                      cudaMemcpyDeviceToHost));
        p2m_scramble_pos(13579LL * (r + 1), oi - ob, pos);
      }
      xm = std::max(xm, pos[2]);
      ym = std::max(ym, pos[1]);
      zm = std::max(zm, pos[0]);
    }
    float *info = ctx->centre_info;
    info[0] = rthmax;
    info[1] = FSQRT(FADD(FADD(FMUL(xm, xm), FMUL(ym, ym)), FMUL(zm, zm)));
    info[2] = xm;
    info[3] = ym;
    info[4] = zm;
    q.flip[2] = xm < 0.0f;
    q.flip[1] = ym < 0.0f;
    q.flip[0] = zm < 0.0f;
    xm = std::fabs(xm);
    ym = std::fabs(ym);
    zm = std::fabs(zm);
    const float theta = p2m_asinf(FDIV(zm, FSQRT(FADD(FMUL(xm, xm), FMUL(zm, zm)))));
    const float xml = FMUL(FDIV(xm, std::fabs(xm)), FSQRT(FADD(FMUL(xm, xm), FMUL(zm, zm))));
    const float phi = p2m_asinf(FDIV(ym, FSQRT(FADD(FMUL(ym, ym), FMUL(xml, xml)))));
    q.ct = p2m_cosf(theta);
    q.st = p2m_sinf(theta);
    q.cp = p2m_cosf(phi);
    q.sp = p2m_sinf(phi);
    q.centre = 1;
    /* the largest halo after the flips and rotation (pks2map.f90:245-257) */
    float after[3] = {info[4], info[3], info[2]}; /* posxyz(1..3) before them */
    p2m_rotate_pos(&q, after);
    info[5] = FSQRT(FADD(FADD(FMUL(after[2], after[2]), FMUL(after[1], after[1])),
                         FMUL(after[0], after[0])));
    info[6] = after[2];
    info[7] = after[1];
    info[8] = after[0];
  }
  CK(cudaGetLastError());
  return P2M_OK;
}

p2m_status ingest_device(p2m_ctx *ctx, const float *d_rec, long long nrec, int nfloat,
                         cudaStream_t s, int ncones = 0) {
  if (nfloat != 7 && nfloat != 10) return fail(ctx, P2M_ERR_BADARG, "nfloat must be 7 or 10");
  if (nrec < 0) return fail(ctx, P2M_ERR_BADARG, "negative record count");
  if (nrec > (1LL << 31) - 1) return fail(ctx, P2M_ERR_BADARG, "more than 2^31-1 records per call");
  ST(check_tables(ctx));
  ST(flush_prepared(ctx));
  if (nrec == 0) return P2M_OK;
  join_in(ctx, s);
  const bool pre = ctx->pre.scramble || ctx->pre.centre;
  if (pre && ctx->rec_count > 0)
    return fail(ctx, P2M_ERR_STATE,
                "with scramble or centre the catalogue must be painted in one call after a reset");
  ST(begin_call(ctx, nrec, s));
  if (pre) ST(preprocess(ctx, d_rec, nrec, nfloat, s));
  PaintParams P = make_params(ctx, nfloat);
  IngestBuffers B = ingest_buffers(ctx, d_rec);
  if (ncones > 1) {
    B.cone_off = ctx->d_cone_off;
    B.ncones = ncones;
  }
  TB(PH_CUT);
  p2m_launch_cut_setup(P, B, nrec, s, ctx->nsm);
  TE(PH_CUT);
  p2m_status st = ingest_tail(ctx, P, nrec, s);
  join_out(ctx, s);
  if (st) return st;
  ctx->rec_count += nrec;
  ctx->n_records += nrec;
  ctx->pending_recs += nrec;
  return P2M_OK;
}

SweepBuffers sweep_buffers(const p2m_ctx *ctx) {
  SweepBuffers W;
  memset(&W, 0, sizeof(W));
  W.halos = ctx->d_halos;
  W.n_halos = ctx->n_halos;
  W.items = ctx->d_items_raw;
  W.pix_off = ctx->d_pix_off;
  W.n_items = ctx->n_items;
  for (int m = 0; m < P2M_MAXMAPS; m++) W.out[m] = ctx->d_out[m];
  W.acc = ctx->d_acc64;
  W.lo = ctx->d_lo;
  W.tiles = ctx->d_tiles;
  W.npix = ctx->hp_npix;
  W.ctr = ctx->d_ctr;
  W.set_rec = ctx->d_set_rec;
  W.set_pix = ctx->d_set_pix;
  W.set_cap = ctx->cap_set;
  return W;
}

/* paints the HEALPix halos ingested since the last paint into the accumulators (the
   output maps' high words and the low words, or the FP64 accumulator); the read-out
   that turns them into maps is left to the next sweep */
p2m_status paint_pending(p2m_ctx *ctx, cudaStream_t s) {
  ST(flush_prepared(ctx));
  ST(wait_zero(ctx, s));
  if (ctx->cfg.nside <= 0) {
    ctx->dirty = false;
    return P2M_OK;
  }
  if (!ctx->dirty) return P2M_OK;
  join_in(ctx, s);
  ST(wait_reads(ctx, s));
  const long long n = ctx->n_items;
  CK(cudaMemsetAsync(ctx->d_ctr, 0, CALL_CTR_BYTES, s));
  PaintParams P = make_params(ctx, 7);
  TB(PH_GROUP);
  if (n > 0) {
    /* candidate offsets of the large halos' items */
    CK(grow(&ctx->d_counts, &ctx->cap_counts, n));
    CK(grow(&ctx->d_pix_off, &ctx->cap_pix_off, n));
    unsigned long long nn = (unsigned long long)n;
    CK(cudaMemcpyAsync(ctx->d_nitems, &nn, sizeof(nn), cudaMemcpyHostToDevice, s));
    p2m_launch_item_counts(ctx->d_items_raw, n, ctx->d_counts, s, ctx->nsm);
    p2m_launch_scan_u32(ctx->d_counts, ctx->d_nitems, ctx->d_pix_off, &ctx->d_ctr->n_pix,
                        ctx->d_scan_tmp, s);
  }
  SweepBuffers W = sweep_buffers(ctx);
  if (ctx->tune.sort_halos && ctx->d_ring_hist) {
    /* counting sort of the halos by first ring (keys and counts came from the set-up):
       the halos painted at any one time then cover a narrow band of rings, a contiguous
       stretch of each map that the L2 holds */
    const long long nbins = 4LL * ctx->cfg.nside + 1;
    CK(grow(&ctx->d_order, &ctx->cap_order, std::max(ctx->n_halos, 1LL)));
    p2m_launch_scan_u32(ctx->d_ring_hist, ctx->d_nbins, ctx->d_ring_off, nullptr, ctx->d_scan_tmp, s);
    p2m_launch_ring_scatter(ctx->d_ring_key, ctx->n_halos, ctx->d_ring_off, ctx->d_order, s, ctx->nsm);
    CK(cudaMemsetAsync(ctx->d_ring_hist, 0, sizeof(unsigned int) * (size_t)nbins, s));
    W.order = ctx->d_order;
  }
  TE(PH_GROUP);
  TB(PH_PAINT); /* the paint phase spans both painting kernels */
  if (n > 0) {
    /* the large halos' items are painted on the side stream, beside the fused kernel's
       uneven tail; the read-out waits for both */
    CK(cudaEventRecord(ctx->ev_zero_start, s));
    CK(cudaStreamWaitEvent(ctx->zstream, ctx->ev_zero_start, 0));
    tmark(ctx, PH_PAINT_BIG, 0, ctx->zstream);
    p2m_launch_paint_full(P, W, ctx->zstream, ctx->nsm);
    tmark(ctx, PH_PAINT_BIG, 1, ctx->zstream);
    CK(cudaEventRecord(ctx->ev_zero_done, ctx->zstream));
  }
  p2m_launch_paint_halos(P, W, s, ctx->nsm);
  if (n > 0) CK(cudaStreamWaitEvent(s, ctx->ev_zero_done, 0));
  TE(PH_PAINT);
  CK(cudaGetLastError());
  join_out(ctx, s);
  ctx->n_items = 0;
  ctx->n_halos = 0;
  ctx->pending_recs = 0;
  ctx->dirty = false;
  ctx->unfolded = true;
  return P2M_OK;
}

/* produces the HEALPix output maps from everything ingested since the last sweep */
p2m_status sweep(p2m_ctx *ctx, cudaStream_t s) {
  ST(paint_pending(ctx, s));
  if (ctx->cfg.nside <= 0) return P2M_OK;
  if (!ctx->unfolded) {
    if (!ctx->swept) {
      ST(wait_reads(ctx, s));
      for (int m = 0; m < ctx->cfg.nmaps; m++)
        CK(cudaMemsetAsync(ctx->d_out[m], 0, sizeof(float) * (size_t)ctx->hp_npix, s));
      ctx->swept = true;
      ctx->outs_zeroed = true;
    }
    return P2M_OK;
  }
  join_in(ctx, s);
  ST(wait_reads(ctx, s));
  PaintParams P = make_params(ctx, 7);
  SweepBuffers W = sweep_buffers(ctx);
  TB(PH_READOUT);
  if (compensated(ctx)) {
    /* fold the sparse low words into the maps and clear them */
    p2m_launch_fold_lo(P, W, s, ctx->nsm);
  } else {
    /* the read-out reads the accumulator; a memset then clears it for the next paint */
    p2m_launch_finalize_full(P, ctx->d_acc64, ctx->hp_npix, ctx->d_out, ctx->swept ? 1 : 0, s,
                             ctx->nsm);
    CK(cudaMemsetAsync(ctx->d_acc64, 0,
                       sizeof(double) * (size_t)ctx->cfg.nmaps * (size_t)ctx->hp_npix, s));
  }
  TE(PH_READOUT);
  CK(cudaGetLastError());
  /* the counters go to mapped host memory without a wait.  A device error flag raised
     by the painting is reported by the next call that waits for the device: the next
     ingest, a host read-out, the statistics or p2m_synchronize.  The fold and the FP64
     read-out leave the accumulators clear either way. */
  p2m_launch_copy_counters(ctx->d_ctr, ctx->h_ctr_dev, s);
  CK(cudaGetLastError());
  join_out(ctx, s);
  ctx->unfolded = false;
  ctx->swept = true;
  return P2M_OK;
}

}  // namespace

extern "C" {

p2m_status p2m_create(const p2m_config *cfg, p2m_ctx **out) {
  if (!cfg || !out) return P2M_ERR_BADARG;
  *out = nullptr;
  if (cfg->nside != 0 && (!is_pow2(cfg->nside) || cfg->nside > 8192)) return P2M_ERR_BADARG;
  if (cfg->npix_fs < 0 || cfg->npix_fs > 65536) return P2M_ERR_BADARG;
  if (cfg->nside == 0 && cfg->npix_fs == 0) return P2M_ERR_BADARG;
  if (cfg->model < 1 || cfg->model > 3) return P2M_ERR_BADARG;
  if (cfg->nmaps < 1 || cfg->nmaps > P2M_MAXMAPS) return P2M_ERR_BADARG;
  if (cfg->precision < P2M_PREC_FP64 || cfg->precision > P2M_PREC_FIXED) return P2M_ERR_BADARG;
  if (cfg->ncones < 0 || cfg->ncones > P2M_MAXCONES) return P2M_ERR_BADARG;
  if (cfg->ncones > 1 && (cfg->nside == 0 || cfg->npix_fs != 0)) return P2M_ERR_BADARG;
  for (int m = 0; m < cfg->nmaps; m++) {
    if (cfg->map_table[m] < 0 || cfg->map_table[m] >= P2M_MAXTABLES) return P2M_ERR_BADARG;
    if (cfg->map_profile[m] != 1 && cfg->map_profile[m] != 2) return P2M_ERR_BADARG;
  }
  p2m_ctx *ctx = new (std::nothrow) p2m_ctx();
  if (!ctx) return P2M_ERR_NOMEM;
  ctx->cfg = *cfg;
  *out = ctx;
  if (const char *e = getenv("P2M_BAND_U")) ctx->band_u = (float)atof(e);
  /* the plain FP64 path is fastest with every halo on the stored-item path, which balances
     its heavy per-candidate work over candidates; test hook: P2M_BIG_RINGS routes every
     halo through one painting path (0: stored items only) */
  if (cfg->precision == P2M_PREC_FP64) ctx->tune.big_rings = 0;
  if (const char *e = getenv("P2M_BIG_RINGS")) ctx->tune.big_rings = std::max(0, atoi(e));
  CK(cudaSetDevice(cfg->device));
  CK(cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, cfg->device));
  CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ctx->ev_back, cudaEventDisableTiming));
  CK(cudaStreamCreateWithFlags(&ctx->zstream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&ctx->ev_zero_start, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ctx->ev_zero_done, cudaEventDisableTiming));
  /* cosmology tables, built once on the host with the reference's float sequence */
  ctx->rofz_host.assign(P2M_NZTAB, 0.0f);
  ctx->zofr_host.assign(P2M_NZTAB, 0.0f);
  p2m_cosmo_build(&ctx->cosmo, ctx->rofz_host.data(), ctx->zofr_host.data());
  CK(cudaMalloc((void **)&ctx->d_rofz, sizeof(float) * P2M_NZTAB));
  CK(cudaMalloc((void **)&ctx->d_zofr, sizeof(float) * P2M_NZTAB));
  CK(cudaMemcpy(ctx->d_rofz, ctx->rofz_host.data(), sizeof(float) * P2M_NZTAB, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_zofr, ctx->zofr_host.data(), sizeof(float) * P2M_NZTAB, cudaMemcpyHostToDevice));
  if (cfg->nside > 0) {
    int nr = 4 * cfg->nside;
    /* ring z and sin(theta) (pix_tools.F90 ring2z) as (hi, lo) float pairs */
    std::vector<float4> rt((size_t)nr);
    rt[0] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
    for (int r = 1; r < nr; r++) {
      double z, sn;
      p2m_ring_z_sth(cfg->nside, r, &z, &sn);
      float zh = (float)z, sh = (float)sn;
      rt[(size_t)r] = make_float4(zh, (float)(z - (double)zh), sh, (float)(sn - (double)sh));
    }
    CK(cudaMalloc((void **)&ctx->d_ringtab, sizeof(float4) * (size_t)nr));
    CK(cudaMemcpy(ctx->d_ringtab, rt.data(), sizeof(float4) * (size_t)nr, cudaMemcpyHostToDevice));
    /* pi / npr of each ring as a (hi, lo) float pair: the candidates' longitude step */
    std::vector<float2> hd((size_t)nr);
    hd[0] = make_float2(0.0f, 0.0f);
    for (int r = 1; r < nr; r++) {
      int npr, ks;
      long long npn;
      p2m_ring_info(cfg->nside, r, &npr, &ks, &npn);
      const double v = P2M_HP_PI / (double)npr;
      const float vh = (float)v;
      hd[(size_t)r] = make_float2(vh, (float)(v - (double)vh));
    }
    CK(cudaMalloc((void **)&ctx->d_ringhd, sizeof(float2) * (size_t)nr));
    CK(cudaMemcpy(ctx->d_ringhd, hd.data(), sizeof(float2) * (size_t)nr, cudaMemcpyHostToDevice));
    /* cos and sin of the grid angles 2 pi k / M as (hi, lo) float pairs */
    std::vector<float4> pt(P2M_PHITAB);
    for (int k = 0; k < P2M_PHITAB; k++) {
      double t = P2M_HP_TWOPI * (double)k / (double)P2M_PHITAB, c = cos(t), sn = sin(t);
      float ch = (float)c, sh = (float)sn;
      pt[(size_t)k] = make_float4(ch, (float)(c - (double)ch), sh, (float)(sn - (double)sh));
    }
    CK(cudaMalloc((void **)&ctx->d_phitab, sizeof(float4) * P2M_PHITAB));
    CK(cudaMemcpy(ctx->d_phitab, pt.data(), sizeof(float4) * P2M_PHITAB, cudaMemcpyHostToDevice));
    ctx->ncones = cfg->ncones > 1 ? cfg->ncones : 1;
    ctx->cone_npix = 12LL * cfg->nside * cfg->nside;
    ctx->hp_npix = ctx->cone_npix * ctx->ncones;
    if (ctx->ncones > 1)
      CK(cudaMalloc((void **)&ctx->d_cone_off, sizeof(long long) * (size_t)(ctx->ncones + 1)));
    for (int m = 0; m < cfg->nmaps; m++) {
      CK(cudaMalloc((void **)&ctx->d_out_own[m], sizeof(float) * (size_t)ctx->hp_npix));
      ctx->d_out[m] = ctx->d_out_own[m];
    }
    if (cfg->precision == P2M_PREC_MIXED) {
      size_t lb = sizeof(float) * (size_t)cfg->nmaps * (size_t)ctx->hp_npix;
      size_t tb = (size_t)((ctx->hp_npix + P2M_TILE_PIX - 1) >> P2M_TILE_SHIFT);
      CK(cudaMalloc((void **)&ctx->d_lo, lb));
      CK(cudaMemset(ctx->d_lo, 0, lb));
      CK(cudaMalloc((void **)&ctx->d_tiles, tb));
      CK(cudaMemset(ctx->d_tiles, 0, tb));
    } else {
      size_t ab = sizeof(double) * (size_t)cfg->nmaps * (size_t)ctx->hp_npix;
      CK(cudaMalloc((void **)&ctx->d_acc64, ab));
      CK(cudaMemset(ctx->d_acc64, 0, ab));
    }
  }
  if (cfg->npix_fs > 0) {
    ctx->fs_npix = (long long)cfg->npix_fs * cfg->npix_fs;
    CK(cudaMalloc(&ctx->d_fs_acc, 8 * (size_t)cfg->nmaps * (size_t)ctx->fs_npix));
    CK(cudaMalloc((void **)&ctx->d_fs_out, sizeof(float) * (size_t)ctx->fs_npix));
  }
  CK(cudaMalloc((void **)&ctx->d_scan_tmp, sizeof(long long) * 1024));
  CK(cudaMalloc((void **)&ctx->d_ctr, sizeof(DevCounters)));
  CK(cudaHostAlloc((void **)&ctx->h_ctr, sizeof(DevCounters), cudaHostAllocMapped));
  CK(cudaHostGetDevicePointer((void **)&ctx->h_ctr_dev, ctx->h_ctr, 0));
  CK(cudaMalloc((void **)&ctx->d_nitems, sizeof(unsigned long long)));
  CK(cudaMalloc((void **)&ctx->d_pre_bits, sizeof(unsigned int)));
  CK(cudaMalloc((void **)&ctx->d_sums, sizeof(double) * 2 * P2M_MAXMAPS));
  if (cfg->flags & P2M_FLAG_RECORD_SETS) {
    /* (record, pixel) pairs kept; P2M_SET_CAP raises it for catalogues whose discs hold
       more pixels in all (16 bytes of device memory per pair) */
    ctx->cap_set = 1LL << 24;
    if (const char *e = getenv("P2M_SET_CAP")) ctx->cap_set = std::max(1LL, atoll(e));
    CK(cudaMalloc((void **)&ctx->d_set_rec, sizeof(long long) * (size_t)ctx->cap_set));
    CK(cudaMalloc((void **)&ctx->d_set_pix, sizeof(long long) * (size_t)ctx->cap_set));
  }
  long long nrec = std::max<long long>(cfg->max_records, 1024);
  CK(grow(&ctx->d_nring, &ctx->cap_nring, nrec));
  CK(grow(&ctx->d_ioff, &ctx->cap_ioff, nrec));
  CK(grow(&ctx->d_halos, &ctx->cap_halos, nrec / 4 + 1024));
  ST(p2m_reset_maps(ctx));
  CK(cudaStreamSynchronize(ctx->stream));
  return P2M_OK;
}

void p2m_destroy(p2m_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->cfg.device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->zstream) cudaStreamSynchronize(ctx->zstream);
  void *ptrs[] = {ctx->d_rofz, ctx->d_zofr, ctx->d_ringtab, ctx->d_ringhd, ctx->d_phitab, ctx->d_acc64, ctx->d_fs_acc,
                  ctx->d_fs_out, ctx->d_halos, ctx->d_items_raw,
                  ctx->d_nring, ctx->d_ioff, ctx->d_fs_items, ctx->d_scan_tmp, ctx->d_counts,
                  ctx->d_pix_off, ctx->d_nitems, ctx->d_sums, ctx->d_set_rec, ctx->d_set_pix,
                  ctx->d_ctr, ctx->d_prep, ctx->d_lo, ctx->d_tiles,
                  ctx->d_pre_flags, ctx->d_pre_bits, ctx->d_pre_ord, ctx->d_pre_last,
                  ctx->d_cone_off, ctx->d_stage[0], ctx->d_stage[1], ctx->d_order,
                  ctx->d_ring_key, ctx->d_ring_hist, ctx->d_ring_off, ctx->d_nbins,
                  ctx->d_mstat, ctx->d_hist, ctx->d_fits[0], ctx->d_fits[1]};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  for (int m = 0; m < P2M_MAXMAPS; m++)
    if (ctx->d_out_own[m]) cudaFree(ctx->d_out_own[m]);
  for (int t = 0; t < P2M_MAXTABLES; t++)
    if (ctx->d_tab[t]) cudaFree(ctx->d_tab[t]);
  for (int q = 0; q < P2M_MAXMAPS / 2; q++)
    if (ctx->d_pair[q]) cudaFree(ctx->d_pair[q]);
  if (ctx->h_ctr) cudaFreeHost(ctx->h_ctr);
  for (int b = 0; b < 2; b++) {
    if (ctx->h_fits[b]) cudaFreeHost(ctx->h_fits[b]);
    if (ctx->ev_fits[b]) cudaEventDestroy(ctx->ev_fits[b]);
  }
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->ev_back) cudaEventDestroy(ctx->ev_back);
  if (ctx->ev_zero_start) cudaEventDestroy(ctx->ev_zero_start);
  if (ctx->ev_zero_done) cudaEventDestroy(ctx->ev_zero_done);
  if (ctx->zstream) cudaStreamDestroy(ctx->zstream);
  if (ctx->cstream) {
    cudaStreamSynchronize(ctx->cstream);
    cudaStreamDestroy(ctx->cstream);
  }
  if (ctx->rstream) {
    cudaStreamSynchronize(ctx->rstream);
    cudaStreamDestroy(ctx->rstream);
  }
  if (ctx->ev_ready) cudaEventDestroy(ctx->ev_ready);
  for (int r = 0; r < p2m_ctx::NGUARD; r++)
    if (ctx->rd_ev[r]) cudaEventDestroy(ctx->rd_ev[r]);
  for (int b = 0; b < 2; b++) {
    if (ctx->ev_copied[b]) cudaEventDestroy(ctx->ev_copied[b]);
    if (ctx->ev_consumed[b]) cudaEventDestroy(ctx->ev_consumed[b]);
  }
  for (int k = 0; k < P2M_NPHASE; k++)
    for (int e = 0; e < 2; e++)
      if (ctx->tev[k][e]) cudaEventDestroy(ctx->tev[k][e]);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char *p2m_last_error(const p2m_ctx *ctx) {
  if (!ctx) return "null context";
  return ctx->err.c_str();
}

p2m_status p2m_set_cosmology_tables(p2m_ctx *ctx, const float *rofz, const float *zofr,
                                    int32_t n, float rofz_zmax, float zofr_rmax) {
  if (!ctx) return P2M_ERR_BADARG;
  if (!rofz || !zofr) return fail(ctx, P2M_ERR_BADARG, "null cosmology table");
  if (n != P2M_NZTAB)
    return fail(ctx, P2M_ERR_BADARG, "cosmology tables hold 10000 entries (cosmology.f90:60,89)");
  if (!(rofz_zmax > 0.0f && zofr_rmax > 0.0f && rofz_zmax < 1e30f && zofr_rmax < 1e30f))
    return fail(ctx, P2M_ERR_BADARG, "cosmology table ranges must be positive and finite");
  for (int i = 0; i < n; i++)
    if (!(rofz[i] == rofz[i] && zofr[i] == zofr[i]))
      return fail(ctx, P2M_ERR_BADARG, "cosmology table holds a NaN");
  if (ctx->dirty || ctx->unfolded || !ctx->prep.empty())
    return fail(ctx, P2M_ERR_STATE, "cosmology tables cannot change while painted halos await a read-out");
  CK(cudaSetDevice(ctx->cfg.device));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->rofz_host.assign(rofz, rofz + n);
  ctx->zofr_host.assign(zofr, zofr + n);
  /* drofztable, dzofrtable of cosmology.f90:61,90 (the tables start at 0) */
  ctx->cosmo.drofz = FDIV(rofz_zmax, (float)(n - 1));
  ctx->cosmo.dzofr = FDIV(zofr_rmax, (float)(n - 1));
  CK(cudaMemcpy(ctx->d_rofz, rofz, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_zofr, zofr, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice));
  return P2M_OK;
}

p2m_status p2m_load_table(p2m_ctx *ctx, int32_t slot, const void *image, int64_t nbytes) {
  if (!ctx) return P2M_ERR_BADARG;
  if (slot < 0 || slot >= P2M_MAXTABLES) return fail(ctx, P2M_ERR_BADARG, "table slot out of range");
  if (!image || nbytes < 36) return fail(ctx, P2M_ERR_IO, "table image shorter than its header");
  p2m_tabhdr t;
  memset(&t, 0, sizeof(t));
  const char *b = (const char *)image;
  memcpy(&t.nchit, b + 0, 4);
  memcpy(&t.nmht, b + 4, 4);
  memcpy(&t.nrt, b + 8, 4);
  memcpy(&t.chimint, b + 12, 4);
  memcpy(&t.chimaxt, b + 16, 4);
  memcpy(&t.mhmint, b + 20, 4);
  memcpy(&t.mhmaxt, b + 24, 4);
  memcpy(&t.rmint, b + 28, 4);
  memcpy(&t.rmaxt, b + 32, 4);
  if (t.nchit < 2 || t.nmht < 2 || t.nrt < 2 || t.nchit > 100000 || t.nmht > 100000 || t.nrt > 100000)
    return fail(ctx, P2M_ERR_IO, "table header sizes out of range");
  if (!(t.chimint > 0 && t.chimaxt > t.chimint && t.mhmint > 0 && t.mhmaxt > t.mhmint &&
        t.rmint > 0 && t.rmaxt > t.rmint))
    return fail(ctx, P2M_ERR_IO, "table header bounds invalid");
  p2m_tabhdr_derive(&t);
  if (t.nelem > (1LL << 30)) return fail(ctx, P2M_ERR_IO, "table too large");
  if (nbytes < 36 + 4 * t.nelem) return fail(ctx, P2M_ERR_IO, "table image shorter than its header says");
  if (ctx->th_set) {
    bool same = t.nchit == ctx->th.nchit && t.nmht == ctx->th.nmht && t.nrt == ctx->th.nrt &&
                t.chimint == ctx->th.chimint && t.chimaxt == ctx->th.chimaxt &&
                t.mhmint == ctx->th.mhmint && t.mhmaxt == ctx->th.mhmaxt &&
                t.rmint == ctx->th.rmint && t.rmaxt == ctx->th.rmaxt;
    int loaded = 0;
    for (int k = 0; k < P2M_MAXTABLES; k++) loaded += (ctx->d_tab[k] != nullptr && k != slot);
    if (!same && loaded) return fail(ctx, P2M_ERR_BADARG, "all tables of a context must share one header");
  }
  if (ctx->dirty || ctx->unfolded || !ctx->prep.empty())
    return fail(ctx, P2M_ERR_STATE, "tables cannot change while painted halos await a read-out");
  CK(cudaSetDevice(ctx->cfg.device));
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->d_tab[slot]) cudaFree(ctx->d_tab[slot]);
  ctx->d_tab[slot] = nullptr;
  CK(cudaMalloc((void **)&ctx->d_tab[slot], sizeof(float) * (size_t)t.nelem));
  CK(cudaMemcpy(ctx->d_tab[slot], b + 36, sizeof(float) * (size_t)t.nelem, cudaMemcpyHostToDevice));
  ctx->th = t;
  ctx->th_set = true;
  ctx->pairs_ok = false; /* the pair tables follow the tables */
  return P2M_OK;
}

p2m_status p2m_reset_maps(p2m_ctx *ctx) {
  if (!ctx) return P2M_ERR_BADARG;
  CK(cudaSetDevice(ctx->cfg.device));
  cudaStream_t s = ctx->stream;
  ctx->prep.clear();
  ctx->n_halos = 0;
  ctx->n_items = 0;
  ctx->rec_count = 0;
  ctx->n_records = 0;
  ctx->pending_recs = 0;
  ctx->dirty = false;
  ctx->swept = false;
  ctx->outs_zeroed = false;
  if (ctx->unfolded) {
    /* painted but never read out: the accumulators that stay zero between read-outs
       hold contributions */
    if (ctx->d_acc64)
      CK(cudaMemsetAsync(ctx->d_acc64, 0,
                         sizeof(double) * (size_t)ctx->cfg.nmaps * (size_t)ctx->hp_npix, s));
    if (ctx->d_lo) {
      CK(cudaMemsetAsync(ctx->d_lo, 0, sizeof(float) * (size_t)ctx->cfg.nmaps * (size_t)ctx->hp_npix, s));
      CK(cudaMemsetAsync(ctx->d_tiles, 0,
                         (size_t)((ctx->hp_npix + P2M_TILE_PIX - 1) >> P2M_TILE_SHIFT), s));
    }
    ctx->unfolded = false;
  }
  if (ctx->d_fs_acc)
    CK(cudaMemsetAsync(ctx->d_fs_acc, 0, 8 * (size_t)ctx->cfg.nmaps * (size_t)ctx->fs_npix, s));
  if (ctx->d_ring_hist)
    CK(cudaMemsetAsync(ctx->d_ring_hist, 0, sizeof(unsigned int) * (size_t)(4LL * ctx->cfg.nside + 1), s));
  CK(cudaMemsetAsync(ctx->d_ctr, 0, sizeof(DevCounters), s));
  CK(cudaMemsetAsync(ctx->d_sums, 0, sizeof(double) * 2 * P2M_MAXMAPS, s));
  return P2M_OK;
}

p2m_status p2m_set_preprocess(p2m_ctx *ctx, int32_t scramble, int32_t centre, int32_t ntasks) {
  if (!ctx) return P2M_ERR_BADARG;
  if ((scramble != 0 && scramble != 1) || (centre != 0 && centre != 1) || ntasks < 1 ||
      ntasks > 25)
    return fail(ctx, P2M_ERR_BADARG, "scramble and centre must be 0 or 1, ntasks 1..25");
  if (ctx->dirty || ctx->unfolded || ctx->rec_count > 0 || !ctx->prep.empty())
    return fail(ctx, P2M_ERR_STATE, "set the pre-processing right after p2m_reset_maps");
  if ((scramble || centre) && ctx->ncones > 1)
    return fail(ctx, P2M_ERR_BADARG, "scramble and centre act on one catalogue, not an ensemble");
  ctx->pre.scramble = scramble;
  ctx->pre.centre = centre;
  ctx->pre.ntasks = ntasks;
  return P2M_OK;
}

p2m_status upload_offsets(p2m_ctx *ctx, const int64_t *offsets, int32_t ncones, long long off,
                          long long n, cudaStream_t s);

/* Host records in chunks of at most the tuning's stream_chunk (and max_records): chunk k + 1 is
   copied on the copy stream into one of two device staging buffers while chunk k is cut
   and set up on the context's stream.  A buffer is refilled only after the chunk that
   used it has been ingested (the cut and set-up kernel is its only reader).  From pinned
   host memory the copies overlap the ingest; from pageable memory the CUDA driver stages each
   copy first.  Scramble and centre need the whole catalogue in one piece: they take a
   single chunk.  With cone offsets (ensembles) each chunk gets its own clamped table. */
p2m_status stream_host_records(p2m_ctx *ctx, const float *records, long long nrec, int nfloat,
                               const int64_t *offsets, int ncones) {
  const bool pre = ctx->pre.scramble || ctx->pre.centre;
  long long chunk = std::max<long long>(ctx->cfg.max_records, 1024);
  if (!pre) chunk = std::min<long long>(chunk, ctx->tune.stream_chunk);
  if (nrec <= 0) return P2M_OK;
  if (pre && nrec > chunk)
    return fail(ctx, P2M_ERR_CAPACITY,
                "scramble and centre need the whole catalogue in one paint call of at most "
                "max_records records");
  const long long nchunk = (nrec + chunk - 1) / chunk;
  if (!ctx->cstream) {
    CK(cudaStreamCreateWithFlags(&ctx->cstream, cudaStreamNonBlocking));
    for (int b = 0; b < 2; b++) {
      CK(cudaEventCreateWithFlags(&ctx->ev_copied[b], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ctx->ev_consumed[b], cudaEventDisableTiming));
      /* no chunk has used the buffer yet */
      CK(cudaEventRecord(ctx->ev_consumed[b], ctx->stream));
    }
  }
  const long long per = std::min(chunk, nrec) * nfloat;
  for (int b = 0; b < (nchunk > 1 ? 2 : 1); b++) {
    if (ctx->cap_stage[b] < per) {
      /* nothing may still read the old buffer */
      CK(cudaEventSynchronize(ctx->ev_consumed[b]));
      CK(grow(&ctx->d_stage[b], &ctx->cap_stage[b], per));
    }
  }
  auto issue = [&](long long k) -> p2m_status {
    const int b = (int)(k & 1);
    const long long off = k * chunk, n = std::min(chunk, nrec - off);
    CK(cudaStreamWaitEvent(ctx->cstream, ctx->ev_consumed[b], 0));
    CK(cudaMemcpyAsync(ctx->d_stage[b], records + off * nfloat, sizeof(float) * (size_t)(n * nfloat),
                       cudaMemcpyHostToDevice, ctx->cstream));
    CK(cudaEventRecord(ctx->ev_copied[b], ctx->cstream));
    return P2M_OK;
  };
  ST(issue(0));
  for (long long k = 0; k < nchunk; k++) {
    if (k + 1 < nchunk) ST(issue(k + 1));
    const int b = (int)(k & 1);
    const long long off = k * chunk, n = std::min(chunk, nrec - off);
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_copied[b], 0));
    if (offsets) ST(upload_offsets(ctx, offsets, ncones, off, n, ctx->stream));
    p2m_status st = ingest_device(ctx, ctx->d_stage[b], n, nfloat, ctx->stream, offsets ? ncones : 0);
    CK(cudaEventRecord(ctx->ev_consumed[b], ctx->stream));
    /* once a full chunk's worth of records awaits painting, paint it while the next
       chunk (of this call or the next) is copied; smaller remainders wait for the
       read-out, where one launch serves them all */
    if (!st && ctx->tune.stream_paint && ctx->pending_recs >= chunk)
      st = paint_pending(ctx, ctx->stream);
    if (st) {
      cudaStreamSynchronize(ctx->cstream);
      return st;
    }
  }
  return P2M_OK;
}

p2m_status p2m_paint_records(p2m_ctx *ctx, const float *records, int64_t nrec, int32_t nfloat) {
  if (!ctx) return P2M_ERR_BADARG;
  if (nrec > 0 && !records) return fail(ctx, P2M_ERR_BADARG, "null records");
  CK(cudaSetDevice(ctx->cfg.device));
  if (nfloat != 7 && nfloat != 10) return fail(ctx, P2M_ERR_BADARG, "nfloat must be 7 or 10");
  return stream_host_records(ctx, records, nrec, nfloat, nullptr, 0);
}

p2m_status p2m_host_alloc(int64_t bytes, void **out) {
  if (!out) return P2M_ERR_BADARG;
  *out = nullptr;
  if (bytes < 0) return P2M_ERR_BADARG;
  if (cudaHostAlloc(out, (size_t)std::max<int64_t>(bytes, 1), cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError(); /* a failed allocation leaves its error as the last error */
    *out = nullptr;
    return P2M_ERR_NOMEM;
  }
  return P2M_OK;
}

p2m_status p2m_host_free(void *p) {
  if (p && cudaFreeHost(p) != cudaSuccess) return P2M_ERR_CUDA;
  return P2M_OK;
}

p2m_status p2m_paint_records_device(p2m_ctx *ctx, const float *d_records, int64_t nrec,
                                    int32_t nfloat, void *stream) {
  if (!ctx) return P2M_ERR_BADARG;
  if (nrec > 0 && !d_records) return fail(ctx, P2M_ERR_BADARG, "null records");
  CK(cudaSetDevice(ctx->cfg.device));
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  return ingest_device(ctx, d_records, nrec, nfloat, s);
}

p2m_status check_offsets(p2m_ctx *ctx, const int64_t *offsets, int32_t ncones) {
  if (!offsets) return fail(ctx, P2M_ERR_BADARG, "null cone offsets");
  if (ncones < 1 || ncones > ctx->ncones)
    return fail(ctx, P2M_ERR_BADARG, "cone count outside 1.." + std::to_string(ctx->ncones));
  if (offsets[0] != 0) return fail(ctx, P2M_ERR_BADARG, "offsets[0] must be 0");
  for (int c = 0; c < ncones; c++)
    if (offsets[c + 1] < offsets[c]) return fail(ctx, P2M_ERR_BADARG, "offsets must not decrease");
  if (ctx->pre.scramble || ctx->pre.centre)
    return fail(ctx, P2M_ERR_STATE, "scramble and centre act on one catalogue, not an ensemble");
  return P2M_OK;
}

/* the cones' first records relative to call-local record `off`, clamped to [0, n] */
p2m_status upload_offsets(p2m_ctx *ctx, const int64_t *offsets, int32_t ncones, long long off,
                          long long n, cudaStream_t s) {
  ctx->cone_off_host.resize((size_t)ncones + 1);
  for (int c = 0; c <= ncones; c++)
    ctx->cone_off_host[(size_t)c] = std::min(std::max((long long)offsets[c] - off, 0LL), n);
  CK(cudaMemcpyAsync(ctx->d_cone_off, ctx->cone_off_host.data(),
                     sizeof(long long) * ((size_t)ncones + 1), cudaMemcpyHostToDevice, s));
  /* the host copy is reused by the next call: let this one finish reading it */
  CK(cudaStreamSynchronize(s));
  return P2M_OK;
}

p2m_status p2m_paint_ensemble(p2m_ctx *ctx, const float *records, const int64_t *offsets,
                              int32_t ncones, int32_t nfloat) {
  if (!ctx) return P2M_ERR_BADARG;
  if (ctx->ncones < 2) return fail(ctx, P2M_ERR_STATE, "the context was not created for an ensemble");
  ST(check_offsets(ctx, offsets, ncones));
  const long long nrec = offsets[ncones];
  if (nrec > 0 && !records) return fail(ctx, P2M_ERR_BADARG, "null records");
  if (nfloat != 7 && nfloat != 10) return fail(ctx, P2M_ERR_BADARG, "nfloat must be 7 or 10");
  CK(cudaSetDevice(ctx->cfg.device));
  return stream_host_records(ctx, records, nrec, nfloat, offsets, ncones);
}

p2m_status p2m_paint_ensemble_device(p2m_ctx *ctx, const float *d_records,
                                     const int64_t *offsets, int32_t ncones, int32_t nfloat,
                                     void *stream) {
  if (!ctx) return P2M_ERR_BADARG;
  if (ctx->ncones < 2) return fail(ctx, P2M_ERR_STATE, "the context was not created for an ensemble");
  ST(check_offsets(ctx, offsets, ncones));
  const long long nrec = offsets[ncones];
  if (nrec > 0 && !d_records) return fail(ctx, P2M_ERR_BADARG, "null records");
  CK(cudaSetDevice(ctx->cfg.device));
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  ST(upload_offsets(ctx, offsets, ncones, 0, nrec, s));
  return ingest_device(ctx, d_records, nrec, nfloat, s, ncones);
}

namespace {

bool tuning_ok(const p2m_tuning &t) {
  return t.big_rings >= 0 && t.big_rings <= 4096 && t.halos_grid >= 1 && t.halos_grid <= 16 &&
         t.full_grid >= 1 && t.full_grid <= 32 && t.full_chunk >= 32 && t.full_chunk <= 65536 &&
         t.stream_chunk >= 65536 && t.stream_chunk <= (1 << 26) &&
         (t.stream_paint == 0 || t.stream_paint == 1) && t.halo_batch >= 1 &&
         t.halo_batch <= 32 && (t.sort_halos == 0 || t.sort_halos == 1) &&
         (t.halos_threads == 128 || t.halos_threads == 256);
}

struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  ~EventPair() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

}  // namespace

int32_t p2m_get_tuning(p2m_ctx *ctx, p2m_tuning *out) {
  if (!ctx || !out) return P2M_ERR_BADARG;
  *out = ctx->tune;
  return P2M_OK;
}

int32_t p2m_set_tuning(p2m_ctx *ctx, const p2m_tuning *t) {
  if (!ctx || !t) return P2M_ERR_BADARG;
  if (!tuning_ok(*t)) return fail(ctx, P2M_ERR_BADARG, "tuning parameter out of range");
  if (ctx->dirty || !ctx->prep.empty())
    return fail(ctx, P2M_ERR_STATE, "change the tuning before painting or after a read-out");
  ctx->tune = *t;
  return P2M_OK;
}

int32_t p2m_autotune(p2m_ctx *ctx, const float *d_records, int64_t nrec, int32_t nfloat,
                     int32_t reps, p2m_tuning *out) {
  if (!ctx) return P2M_ERR_BADARG;
  if (!d_records || nrec < 1 || reps < 1 || reps > 100)
    return fail(ctx, P2M_ERR_BADARG, "autotune needs device records and 1..100 repetitions");
  CK(cudaSetDevice(ctx->cfg.device));
  EventPair ev;
  CK(cudaEventCreate(&ev.a));
  CK(cudaEventCreate(&ev.b));
  /* device time of one whole paint call with tuning t, best of reps */
  auto trial = [&](const p2m_tuning &t, float *ms) -> p2m_status {
    ctx->tune = t;
    float best = 3.0e38f;
    for (int r = 0; r < reps; r++) {
      ST(p2m_reset_maps(ctx));
      CK(cudaEventRecord(ev.a, ctx->stream));
      ST(ingest_device(ctx, d_records, nrec, nfloat, ctx->stream));
      ST(sweep(ctx, ctx->stream));
      CK(cudaEventRecord(ev.b, ctx->stream));
      CK(cudaEventSynchronize(ev.b));
      float e = 0.0f;
      CK(cudaEventElapsedTime(&e, ev.a, ev.b));
      best = std::min(best, e);
    }
    *ms = best;
    return P2M_OK;
  };
  static const int kBig[] = {0, 16, 32, 48, 64, 96, 128, 256};
  static const int kHalos[] = {2, 4, 6, 8, 16};
  static const int kFull[] = {2, 4, 8, 16};
  static const int kChunk[] = {256, 512, 1024, 2048, 4096};
  static const int kBatch[] = {8, 16, 32};
  static const int kSort[] = {0, 1};
  p2m_tuning best = ctx->tune;
  ST(trial(best, &best.ms));
  auto descend = [&](const int *vals, int n, int32_t p2m_tuning::*field) -> p2m_status {
    for (int i = 0; i < n; i++) {
      if (best.*field == vals[i]) continue;
      p2m_tuning t = best;
      t.*field = vals[i];
      ST(trial(t, &t.ms));
      if (t.ms < best.ms) best = t;
    }
    return P2M_OK;
  };
  p2m_status st = descend(kBig, 8, &p2m_tuning::big_rings);
  if (!st) {
    /* the other block size, with the grid that keeps the same warps per SM */
    p2m_tuning t = best;
    t.halos_threads = best.halos_threads == 128 ? 256 : 128;
    t.halos_grid = t.halos_threads == 256 ? std::max(1, best.halos_grid / 2)
                                          : std::min(16, best.halos_grid * 2);
    st = trial(t, &t.ms);
    if (!st && t.ms < best.ms) best = t;
  }
  if (!st) st = descend(kHalos, 5, &p2m_tuning::halos_grid);
  if (!st) st = descend(kFull, 4, &p2m_tuning::full_grid);
  if (!st) st = descend(kChunk, 5, &p2m_tuning::full_chunk);
  if (!st) st = descend(kSort, 2, &p2m_tuning::sort_halos);
  if (!st) st = descend(kBatch, 3, &p2m_tuning::halo_batch);
  ctx->tune = best;
  if (st) return st;
  ST(p2m_reset_maps(ctx));
  if (out) *out = best;
  return P2M_OK;
}

p2m_status p2m_get_healpix_cone(p2m_ctx *ctx, int32_t cone, int32_t map, float *out) {
  if (!ctx || !out) return P2M_ERR_BADARG;
  if (map < 0 || map >= ctx->cfg.nmaps || ctx->cfg.nside <= 0)
    return fail(ctx, P2M_ERR_BADARG, "map index out of range");
  if (cone < 0 || cone >= ctx->ncones) return fail(ctx, P2M_ERR_BADARG, "cone index out of range");
  CK(cudaSetDevice(ctx->cfg.device));
  ST(sweep(ctx, ctx->stream));
  CK(cudaMemcpyAsync(out, ctx->d_out[map] + (size_t)cone * (size_t)ctx->cone_npix,
                     sizeof(float) * (size_t)ctx->cone_npix, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return check_errors(ctx, ctx->stream);
}

p2m_status p2m_project_halo(p2m_ctx *ctx, float *x, float *y, float *z, const float *r,
                            const float *chi, const float *m, const float *redshift,
                            const float *v, const int32_t *profile) {
  if (!ctx || !x || !y || !z || !r || !chi || !m || !redshift || !v || !profile)
    return P2M_ERR_BADARG;
  if (*profile != 1 && *profile != 2) return fail(ctx, P2M_ERR_BADARG, "profile must be 1 or 2");
  float q[9] = {*x, *y, *z, *r, *chi, *m, *redshift, *v, (float)*profile};
  ctx->prep.insert(ctx->prep.end(), q, q + 9);
  /* haloproject.f90:97-99 divides the caller's x, y, z by chi */
  *x = FDIV(*x, *chi);
  *y = FDIV(*y, *chi);
  *z = FDIV(*z, *chi);
  return P2M_OK;
}

p2m_status p2m_flush(p2m_ctx *ctx) {
  if (!ctx) return P2M_ERR_BADARG;
  CK(cudaSetDevice(ctx->cfg.device));
  return sweep(ctx, ctx->stream);
}

p2m_status p2m_bind_healpix_device(p2m_ctx *ctx, int32_t map, float *d_out) {
  if (!ctx) return P2M_ERR_BADARG;
  if (map < 0 || map >= ctx->cfg.nmaps || ctx->cfg.nside <= 0)
    return fail(ctx, P2M_ERR_BADARG, "map index out of range");
  if (ctx->dirty || ctx->unfolded || ctx->swept)
    return fail(ctx, P2M_ERR_STATE, "bind output buffers right after p2m_reset_maps");
  ctx->d_out[map] = d_out ? d_out : ctx->d_out_own[map];
  ctx->outs_zeroed = false;
  return P2M_OK;
}

p2m_status p2m_get_healpix_device(p2m_ctx *ctx, int32_t map, float *d_out, void *stream) {
  if (!ctx || !d_out) return P2M_ERR_BADARG;
  if (map < 0 || map >= ctx->cfg.nmaps || ctx->cfg.nside <= 0)
    return fail(ctx, P2M_ERR_BADARG, "map index out of range");
  CK(cudaSetDevice(ctx->cfg.device));
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  ST(sweep(ctx, s));
  if (d_out != ctx->d_out[map]) {
    join_in(ctx, s);
    CK(cudaMemcpyAsync(d_out, ctx->d_out[map], sizeof(float) * (size_t)ctx->hp_npix,
                       cudaMemcpyDeviceToDevice, s));
    join_out(ctx, s);
  }
  return P2M_OK;
}

p2m_status p2m_get_healpix(p2m_ctx *ctx, int32_t map, float *out) {
  if (!ctx || !out) return P2M_ERR_BADARG;
  if (map < 0 || map >= ctx->cfg.nmaps || ctx->cfg.nside <= 0)
    return fail(ctx, P2M_ERR_BADARG, "map index out of range");
  CK(cudaSetDevice(ctx->cfg.device));
  ST(sweep(ctx, ctx->stream));
  CK(cudaMemcpyAsync(out, ctx->d_out[map], sizeof(float) * (size_t)ctx->hp_npix,
                     cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return check_errors(ctx, ctx->stream);
}

p2m_status p2m_get_healpix_async(p2m_ctx *ctx, int32_t map, float *out) {
  if (!ctx || !out) return P2M_ERR_BADARG;
  if (map < 0 || map >= ctx->cfg.nmaps || ctx->cfg.nside <= 0)
    return fail(ctx, P2M_ERR_BADARG, "map index out of range");
  CK(cudaSetDevice(ctx->cfg.device));
  ST(sweep(ctx, ctx->stream));
  if (!ctx->rstream) {
    CK(cudaStreamCreateWithFlags(&ctx->rstream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ctx->ev_ready, cudaEventDisableTiming));
    for (int r = 0; r < p2m_ctx::NGUARD; r++)
      CK(cudaEventCreateWithFlags(&ctx->rd_ev[r], cudaEventDisableTiming));
  }
  /* the guard of this buffer: its own, a free one, or the oldest after its copy is done */
  const float *buf = ctx->d_out[map];
  int g = -1;
  for (int r = 0; r < p2m_ctx::NGUARD && g < 0; r++)
    if (ctx->rd_buf[r] == buf) g = r;
  for (int r = 0; r < p2m_ctx::NGUARD && g < 0; r++)
    if (!ctx->rd_buf[r]) g = r;
  if (g < 0) {
    g = 0;
    for (int r = 1; r < p2m_ctx::NGUARD; r++)
      if (ctx->rd_seq[r] < ctx->rd_seq[g]) g = r;
    CK(cudaEventSynchronize(ctx->rd_ev[g]));
  }
  CK(cudaEventRecord(ctx->ev_ready, ctx->stream));
  CK(cudaStreamWaitEvent(ctx->rstream, ctx->ev_ready, 0));
  CK(cudaMemcpyAsync(out, buf, sizeof(float) * (size_t)ctx->hp_npix, cudaMemcpyDeviceToHost,
                     ctx->rstream));
  CK(cudaEventRecord(ctx->rd_ev[g], ctx->rstream));
  ctx->rd_buf[g] = buf;
  ctx->rd_seq[g] = ++ctx->rd_clock;
  return P2M_OK;
}

p2m_status p2m_get_flatsky(p2m_ctx *ctx, int32_t map, float *out) {
  if (!ctx || !out) return P2M_ERR_BADARG;
  if (map < 0 || map >= ctx->cfg.nmaps || ctx->cfg.npix_fs <= 0)
    return fail(ctx, P2M_ERR_BADARG, "no flat-sky map / map index out of range");
  CK(cudaSetDevice(ctx->cfg.device));
  ST(flush_prepared(ctx));
  cudaStream_t s = ctx->stream;
  PaintParams P = make_params(ctx, 7);
  double *sum = ctx->d_sums + P2M_MAXMAPS + map;
  CK(cudaMemsetAsync(sum, 0, sizeof(double), s));
  p2m_launch_finalize_fs(P, ctx->d_fs_acc, ctx->fs_npix, ctx->d_fs_out, map, sum, s, ctx->nsm);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, ctx->d_fs_out, sizeof(float) * (size_t)ctx->fs_npix,
                     cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return P2M_OK;
}

namespace {

/* moments, RMS and (dpdy non-null) P(<y) of the float map d_map (npix pixels) on the
   context's stream, pks2map.f90:321-357 */
p2m_status map_stats(p2m_ctx *ctx, const float *d_map, long long npix, p2m_map_stats *out,
                     float *dpdy) {
  cudaStream_t s = ctx->stream;
  if (!ctx->d_mstat) CK(cudaMalloc((void **)&ctx->d_mstat, sizeof(double) * 4));
  if (dpdy && !ctx->d_hist) CK(cudaMalloc((void **)&ctx->d_hist, sizeof(unsigned int) * P2M_NDPDY));
  CK(cudaMemsetAsync(ctx->d_mstat, 0, sizeof(double) * 4, s));
  if (dpdy) CK(cudaMemsetAsync(ctx->d_hist, 0, sizeof(unsigned int) * P2M_NDPDY, s));
  /* dpdy_dy = dpdy_max / ndpdy (pks2map.f90:40) */
  const float dy = FDIV(1e-4f, (float)P2M_NDPDY);
  p2m_launch_map_stats(d_map, npix, ctx->d_mstat, dpdy ? ctx->d_hist : nullptr, P2M_NDPDY, dy,
                       s, ctx->nsm);
  CK(cudaGetLastError());
  double sums[4];
  std::vector<unsigned int> h(dpdy ? P2M_NDPDY : 0);
  CK(cudaMemcpyAsync(sums, ctx->d_mstat, sizeof(double) * 4, cudaMemcpyDeviceToHost, s));
  if (dpdy)
    CK(cudaMemcpyAsync(h.data(), ctx->d_hist, sizeof(unsigned int) * P2M_NDPDY,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  ST(check_errors(ctx, s));
  const double n = (double)npix;
  out->npix = npix;
  for (int k = 0; k < 3; k++) out->mom[k] = sums[k] / n;
  /* sum((x - mom1)^2) = sum x^2 - 2 mom1 sum x + n mom1^2, in FP64 */
  const double m1 = out->mom[0];
  const double ss = sums[1] - 2.0 * m1 * sums[0] + n * m1 * m1;
  out->rms = std::sqrt(ss > 0.0 ? ss / n : 0.0);
  if (dpdy) {
    /* the reference counts in float (:345): a bin stops at 2^24 */
    for (int k = 0; k < P2M_NDPDY; k++) dpdy[k] = (float)std::min(h[k], 16777216u);
    const float norm = (float)npix;
    for (int k = 0; k < P2M_NDPDY; k++) dpdy[k] = dpdy[k] / norm;            /* :347 */
    for (int k = 1; k < P2M_NDPDY; k++) dpdy[k] = dpdy[k - 1] + dpdy[k];     /* :355-357 */
  }
  return P2M_OK;
}

}  // namespace

p2m_status p2m_get_healpix_stats(p2m_ctx *ctx, int32_t map, p2m_map_stats *out, float *dpdy) {
  if (!ctx || !out) return P2M_ERR_BADARG;
  if (map < 0 || map >= ctx->cfg.nmaps || ctx->cfg.nside <= 0)
    return fail(ctx, P2M_ERR_BADARG, "map index out of range");
  if (ctx->ncones > 1)
    return fail(ctx, P2M_ERR_BADARG, "statistics of an ensemble: read the cones out one by one");
  CK(cudaSetDevice(ctx->cfg.device));
  ST(sweep(ctx, ctx->stream));
  return map_stats(ctx, ctx->d_out[map], ctx->hp_npix, out, dpdy);
}

p2m_status p2m_get_flatsky_stats(p2m_ctx *ctx, int32_t map, p2m_map_stats *out) {
  if (!ctx || !out) return P2M_ERR_BADARG;
  if (map < 0 || map >= ctx->cfg.nmaps || ctx->cfg.npix_fs <= 0)
    return fail(ctx, P2M_ERR_BADARG, "no flat-sky map / map index out of range");
  CK(cudaSetDevice(ctx->cfg.device));
  ST(flush_prepared(ctx));
  cudaStream_t s = ctx->stream;
  PaintParams P = make_params(ctx, 7);
  double *sum = ctx->d_sums + P2M_MAXMAPS + map;
  CK(cudaMemsetAsync(sum, 0, sizeof(double), s));
  p2m_launch_finalize_fs(P, ctx->d_fs_acc, ctx->fs_npix, ctx->d_fs_out, map, sum, s, ctx->nsm);
  CK(cudaGetLastError());
  return map_stats(ctx, ctx->d_fs_out, ctx->fs_npix, out, nullptr);
}

#define P2M_FITS_SLICE (1LL << 24) /* floats per slice of the device FITS writer (64 MB) */

p2m_status p2m_write_healpix_fits_device(p2m_ctx *ctx, int32_t map, const char *path) {
  if (!ctx || !path) return P2M_ERR_BADARG;
  if (map < 0 || map >= ctx->cfg.nmaps || ctx->cfg.nside <= 0)
    return fail(ctx, P2M_ERR_BADARG, "map index out of range");
  if (ctx->ncones > 1)
    return fail(ctx, P2M_ERR_BADARG, "an ensemble's maps: read the cones out one by one");
  CK(cudaSetDevice(ctx->cfg.device));
  cudaStream_t s = ctx->stream;
  ST(sweep(ctx, s));
  const long long n = ctx->hp_npix, slice = std::min<long long>(n, P2M_FITS_SLICE);
  for (int b = 0; b < 2; b++) {
    if (!ctx->d_fits[b]) CK(cudaMalloc((void **)&ctx->d_fits[b], sizeof(unsigned int) * P2M_FITS_SLICE));
    if (!ctx->h_fits[b]) CK(cudaHostAlloc((void **)&ctx->h_fits[b], sizeof(unsigned int) * P2M_FITS_SLICE, 0));
    if (!ctx->ev_fits[b]) CK(cudaEventCreateWithFlags(&ctx->ev_fits[b], cudaEventDisableTiming));
  }
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return fail(ctx, P2M_ERR_IO, std::string("cannot open ") + path);
  bool ok = p2m_fits_put_header(fp, ctx->cfg.nside) == P2M_OK;
  /* slice k is converted and copied while slice k - 1 is written to the file (one
     writer: writes into one file from several threads measured slower, as the file
     system serialises them) */
  const long long nslice = (n + slice - 1) / slice;
  cudaError_t e = cudaSuccess;
  for (long long k = 0; k <= nslice && ok && e == cudaSuccess; k++) {
    if (k < nslice) {
      const int b = (int)(k & 1);
      const long long len = std::min(slice, n - k * slice);
      p2m_launch_to_big_endian(ctx->d_out[map] + k * slice, ctx->d_fits[b], len, s, ctx->nsm);
      e = cudaGetLastError();
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->h_fits[b], ctx->d_fits[b], sizeof(unsigned int) * (size_t)len,
                            cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_fits[b], s);
    }
    if (k > 0 && e == cudaSuccess) {
      const int b = (int)((k - 1) & 1);
      const long long len = std::min(slice, n - (k - 1) * slice);
      e = cudaEventSynchronize(ctx->ev_fits[b]);
      if (e == cudaSuccess)
        ok = std::fwrite(ctx->h_fits[b], sizeof(unsigned int), (size_t)len, fp) == (size_t)len;
    }
  }
  if (ok && e == cudaSuccess) ok = p2m_fits_put_padding(fp, ctx->cfg.nside) == P2M_OK;
  ok = (std::fclose(fp) == 0) && ok;
  if (e != cudaSuccess)
    return fail(ctx, P2M_ERR_CUDA, std::string("FITS read-out: ") + cudaGetErrorString(e));
  if (!ok) return fail(ctx, P2M_ERR_IO, std::string("cannot write ") + path);
  return check_errors(ctx, s);
}

p2m_status p2m_get_stats(p2m_ctx *ctx, p2m_stats *out) {
  if (!ctx || !out) return P2M_ERR_BADARG;
  CK(cudaSetDevice(ctx->cfg.device));
  ST(sweep(ctx, ctx->stream));
  /* sums over the HEALPix maps as they now are */
  if (ctx->cfg.nside > 0) {
    CK(cudaMemsetAsync(ctx->d_sums, 0, sizeof(double) * P2M_MAXMAPS, ctx->stream));
    for (int m = 0; m < ctx->cfg.nmaps; m++)
      p2m_launch_map_sum(ctx->d_out[m], ctx->hp_npix, ctx->d_sums + m, ctx->stream, ctx->nsm);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(ctx->stream));
  ST(check_errors(ctx, ctx->stream));
  DevCounters h;
  CK(cudaMemcpy(&h, ctx->d_ctr, sizeof(h), cudaMemcpyDeviceToHost));
  double sums[2 * P2M_MAXMAPS];
  CK(cudaMemcpy(sums, ctx->d_sums, sizeof(sums), cudaMemcpyDeviceToHost));
  memset(out, 0, sizeof(*out));
  out->n_records = ctx->n_records;
  out->n_shell = (long long)h.n_shell;
  out->n_painted = (long long)h.n_massive;
  out->n_enumerated = (long long)h.n_enum;
  out->hp_candidates = (long long)h.n_cand;
  out->hp_updates = (long long)h.hp_updates;
  out->fs_updates = (long long)h.fs_updates;
  out->n_recheck = (long long)h.n_recheck;
  out->val_checked = (long long)h.val_checked;
  out->val_bad_set = (long long)h.val_bad_set;
  out->val_bad_index = (long long)h.val_bad_index;
  float du;
  memcpy(&du, &h.val_max_du, 4);
  out->val_max_du = du;
  for (int m = 0; m < P2M_MAXMAPS; m++) {
    out->hp_sum[m] = sums[m];
    out->fs_sum[m] = sums[P2M_MAXMAPS + m];
  }
  return P2M_OK;
}

p2m_status p2m_synchronize(p2m_ctx *ctx) {
  if (!ctx) return P2M_ERR_BADARG;
  CK(cudaSetDevice(ctx->cfg.device));
  CK(cudaStreamSynchronize(ctx->zstream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->rstream) CK(cudaStreamSynchronize(ctx->rstream));
  return check_errors(ctx, ctx->stream);
}

p2m_status p2m_get_pixel_sets(p2m_ctx *ctx, int64_t *rec, int64_t *pix, int64_t cap, int64_t *n) {
  if (!ctx || !n) return P2M_ERR_BADARG;
  if (!(ctx->cfg.flags & P2M_FLAG_RECORD_SETS))
    return fail(ctx, P2M_ERR_STATE, "context was created without P2M_FLAG_RECORD_SETS");
  CK(cudaSetDevice(ctx->cfg.device));
  ST(sweep(ctx, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ST(check_errors(ctx, ctx->stream));
  DevCounters h;
  CK(cudaMemcpy(&h, ctx->d_ctr, sizeof(h), cudaMemcpyDeviceToHost));
  long long total = (long long)h.n_sets;
  *n = total;
  if (total > ctx->cap_set) return fail(ctx, P2M_ERR_CAPACITY, "pixel-set buffer overflow");
  long long k = std::min<long long>(cap, total);
  if (k > 0 && rec && pix) {
    CK(cudaMemcpy(rec, ctx->d_set_rec, sizeof(long long) * (size_t)k, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(pix, ctx->d_set_pix, sizeof(long long) * (size_t)k, cudaMemcpyDeviceToHost));
  }
  return P2M_OK;
}

int32_t p2m_get_centre(p2m_ctx *ctx, float *out9) {
  if (!ctx || !out9) return P2M_ERR_BADARG;
  for (int k = 0; k < 9; k++) out9[k] = ctx->centre_info[k];
  return P2M_OK;
}

int32_t p2m_get_timings(p2m_ctx *ctx, double *ms, int32_t n) {
  if (!ctx || !ms) return P2M_ERR_BADARG;
  if (!(ctx->cfg.flags & P2M_FLAG_TIMING))
    return fail(ctx, P2M_ERR_STATE, "context was created without P2M_FLAG_TIMING");
  CK(cudaSetDevice(ctx->cfg.device));
  for (int k = 0; k < n; k++) {
    ms[k] = 0.0;
    if (k < P2M_NPHASE && ctx->tev_used[k]) {
      float t = 0.0f;
      CK(cudaEventSynchronize(ctx->tev[k][1]));
      CK(cudaEventElapsedTime(&t, ctx->tev[k][0], ctx->tev[k][1]));
      ms[k] = (double)t;
    }
  }
  return P2M_OK;
}

p2m_status p2m_make_maptable(int32_t device, int32_t model, float nu, float alpha_cmb,
                             int32_t nchit, int32_t nmht, int32_t nrt, void *image,
                             int64_t *nbytes) {
  p2m_ctx *ctx = nullptr; /* CK needs a name; errors carry no context message */
  if (!nbytes) return P2M_ERR_BADARG;
  if (nchit <= 0) nchit = 100;
  if (nmht <= 0) nmht = 100;
  if (nrt <= 0) nrt = 200;
  if (model < 1 || model > 3 || nchit < 2 || nmht < 2 || nrt < 2) return P2M_ERR_BADARG;
  p2m_tabhdr th;
  memset(&th, 0, sizeof(th));
  th.nchit = nchit;
  th.nmht = nmht;
  th.nrt = nrt;
  th.chimint = 1e2f; /* maptable.f90:69-85 */
  th.chimaxt = 7e3f;
  th.mhmint = 1e13f;
  th.mhmaxt = 1e16f;
  th.rmint = 1e-2f;
  th.rmaxt = 10.0f;
  p2m_tabhdr_derive(&th);
  *nbytes = 36 + 4 * th.nelem;
  if (!image) return P2M_OK;
  CK(cudaSetDevice(device));
  p2m_cosmo cosmo;
  std::vector<float> rofz(P2M_NZTAB), zofr(P2M_NZTAB);
  p2m_cosmo_build(&cosmo, rofz.data(), zofr.data());
  /* maptable.f90:56-64 with cosmology.f90:11-38 constants (pi is the float literal;
     mp, mue, 1.932 and 8. are single-precision literals) */
  const double PI_D = P2M_COSMO_PI;
  const double sigmat = 6.65246e-25, me = 9.109383e-28, mp = (double)1.67e-24f, c = 2.99792458e10;
  const double msun = 1.9891e33, Mpc2km = 3.08567758e19, Mpc = 3.08567758e24, kpc = 3.08567758e21;
  const double H100 = 1e2 / Mpc2km;
  const double ypermass = ((((((3.0 * sigmat) * (H100 * H100)) / 8.0) / PI_D) / me) / (c * c) * msun) /
                          (double)1.932f;
  const double taupersigma =
      (((sigmat / (double)1.136f) / mp) * msun / ((kpc * kpc) * kpc)) * Mpc * 1e10;
  static const float bbps_delta[3] = {200.0f, 500.0f, 200.0f};
  float Delta = bbps_delta[model - 1];
  float m2rfac = (float)pow(((double)(3.0f / 4.0f) / PI_D) / (double)Delta, (double)(1.0f / 3.0f));
  TableConsts K;
  K.y0 = (float)((double)FMUL(FMUL(cosmo.fb, Delta), FMUL(cosmo.h, cosmo.h)) * ypermass);
  K.tau0 = (float)((taupersigma * (double)FMUL(cosmo.h, cosmo.h)) * (double)m2rfac);
  K.x0const = FMUL(0.017612f, nu);
  K.nu = nu;
  K.alpha = alpha_cmb;
  K.model = model;
  PaintParams P;
  memset(&P, 0, sizeof(P));
  P.cosmo = cosmo;
  float *d_rofz = nullptr, *d_zofr = nullptr, *d_tab = nullptr;
  CK(cudaMalloc((void **)&d_rofz, sizeof(float) * P2M_NZTAB));
  CK(cudaMalloc((void **)&d_zofr, sizeof(float) * P2M_NZTAB));
  CK(cudaMalloc((void **)&d_tab, sizeof(float) * (size_t)th.nelem));
  CK(cudaMemcpy(d_rofz, rofz.data(), sizeof(float) * P2M_NZTAB, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_zofr, zofr.data(), sizeof(float) * P2M_NZTAB, cudaMemcpyHostToDevice));
  P.rofz = d_rofz;
  P.zofr = d_zofr;
  p2m_launch_maptable(P, K, th, d_tab, 0);
  CK(cudaGetLastError());
  char *b = (char *)image;
  memcpy(b + 0, &th.nchit, 4);
  memcpy(b + 4, &th.nmht, 4);
  memcpy(b + 8, &th.nrt, 4);
  memcpy(b + 12, &th.chimint, 4);
  memcpy(b + 16, &th.chimaxt, 4);
  memcpy(b + 20, &th.mhmint, 4);
  memcpy(b + 24, &th.mhmaxt, 4);
  memcpy(b + 28, &th.rmint, 4);
  memcpy(b + 32, &th.rmaxt, 4);
  CK(cudaMemcpy(b + 36, d_tab, sizeof(float) * (size_t)th.nelem, cudaMemcpyDeviceToHost));
  cudaFree(d_rofz);
  cudaFree(d_zofr);
  cudaFree(d_tab);
  return P2M_OK;
}

}  // extern "C"
