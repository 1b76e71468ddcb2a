/*
 * pks2map_cli.cpp -- the pks2map command line on one GB300 (pks2map.f90:58-385).
 *
 *   pks2map <filein> <fileout> <tablefile> [<zmin> <nside> <scramble> <center> <npix>
 *           <fov> <zmax> <chihview> <model> <profile>]
 *
 * Same positional arguments and defaults as the reference (pks2map.f90:62-82; an
 * argument that is a single dot, or does not parse, takes its default, textlib.f90:33-86),
 * the same report lines, and the same output files: <fileout>_dp.bin, _fs.map, _hp.fits.
 * The halo loop runs on the GPU through the C ABI (include/p2m.h).  The environment
 * selects the precision (P2M_PRECISION = mixed | fp64 | mixed64 | fixed, default mixed) and the
 * device (P2M_DEVICE, default 0).  scramble and center follow the reference's random
 * stream and rotation; P2M_RANKS (default 1, at most 25) is the MPI rank count whose
 * halo blocks and streams they reproduce (`mpirun -np <ranks> pks2map ...`).
 *
 * The catalogue is read in steps of 4M records, each step's file read overlapping the
 * painting of the step before; the moments, RMS and P(<y) are computed on the device;
 * the FITS map is written from the device in slices whose copies overlap the file
 * write.  P2M_TIMING set in the environment prints the phase times to stderr.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <thread>
#include <vector>

#include "../../include/p2m.h"
#include "../../include/p2m_tools.h"
#include "p2m_fmath.h"
#include "p2m_pio.h"
#include "p2m_scalar.h"

namespace {

bool is_dot(const char *s) { return std::strcmp(s, ".") == 0; }

double now_s() {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* textlib.f90 i4arg / r4arg: default when absent, a single dot, or unparsable */
int i4arg(int argc, char **argv, int k, int def) {
  if (k >= argc || is_dot(argv[k])) return def;
  char *end = nullptr;
  long v = std::strtol(argv[k], &end, 10);
  if (end == argv[k] || *end) return def;
  return (int)v;
}
float r4arg(int argc, char **argv, int k, float def) {
  if (k >= argc || is_dot(argv[k])) return def;
  char *end = nullptr;
  double v = std::strtod(argv[k], &end);
  if (end == argv[k] || *end) return def;
  return (float)v;
}

bool read_file(const char *path, std::vector<char> &out) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  out.resize((size_t)(n > 0 ? n : 0));
  bool ok = n <= 0 || std::fread(out.data(), 1, (size_t)n, f) == (size_t)n;
  std::fclose(f);
  return ok;
}

int fail(const char *what, p2m_ctx *ctx = nullptr, int status = 0) {
  std::fprintf(stderr, "pks2map: %s", what);
  if (ctx) std::fprintf(stderr, ": %s", p2m_last_error(ctx));
  if (status) std::fprintf(stderr, " (status %d)", status);
  std::fprintf(stderr, "\n");
  if (ctx) p2m_destroy(ctx);
  return 1;
}

/* Fortran `1pe<w>.<d>` of a finite value: one digit before the point */
std::string fe(double v, int d) {
  char b[64];
  std::snprintf(b, sizeof b, "%.*E", d, v);
  return b;
}

/* Fortran `e10.3`: 0.ddd mantissa, right-justified in 10 columns */
std::string e103(double v) {
  char b[64];
  if (v == 0.0) {
    std::snprintf(b, sizeof b, "%10s", "0.000E+00");
    return b;
  }
  int ex = (int)std::floor(std::log10(std::fabs(v))) + 1;
  double m = std::fabs(v) / std::pow(10.0, ex);
  if (m >= 0.9995) { /* rounding to three digits carries into the exponent */
    m /= 10.0;
    ex += 1;
  }
  char body[32];
  std::snprintf(body, sizeof body, "%s0.%03dE%+03d", v < 0 ? "-" : "", (int)std::lround(m * 1000.0), ex);
  std::snprintf(b, sizeof b, "%10s", body);
  return b;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc - 1 < 3) {
    std::printf("Usage: pks2map <filein> <fileout> <tablefile> [<zmin> <nside> <scramble> "
                "<center> <npix> <fov> <zmax> <chihview> <model> <profile>]\n");
    return 0;
  }
  const char *filein = argv[1], *fileout = argv[2], *tablefile = argv[3];
  const float zmin = r4arg(argc, argv, 4, 0.0f);
  const int nside = i4arg(argc, argv, 5, 4096);
  const int scramble = i4arg(argc, argv, 6, 0);
  const int centre = i4arg(argc, argv, 7, 0);
  const int npix = i4arg(argc, argv, 8, 16);
  const float fov_deg = r4arg(argc, argv, 9, 10.0f);
  const float zmax = r4arg(argc, argv, 10, 1.25f);
  const float chihview = r4arg(argc, argv, 11, 0.0f);
  const int model = i4arg(argc, argv, 12, 1);
  const int profile = i4arg(argc, argv, 13, 1);
  if ((scramble != 0 && scramble != 1) || (centre != 0 && centre != 1))
    return fail("scramble and center must be 0 or 1");
  if (profile != 1 && profile != 2) return fail("profile must be 1 or 2");
  const int ranks = std::getenv("P2M_RANKS") ? std::atoi(std::getenv("P2M_RANKS")) : 1;

  /* pks2map.f90:88-105 (fov to radians, dpix) and its report */
  const float mypi = 4.0f * p2m_atanf(1.0f);
  const float fov = ((fov_deg / 360.0f) * 2.0f) * mypi;
  const float dpix = npix > 0 ? fov / (float)npix : 0.0f;
  const long long hpnpix = 12LL * nside * nside;
  std::printf("\n\nResolution:         %d x %d pixels (%s radians)\n", npix, npix,
              fe(dpix, 2).c_str());
  std::printf("Field of view:      %s degrees\n", fe(fov / 2.0f / mypi * 360.0f, 2).c_str());
  std::printf("Healpix Nside:      %d\nNumber of pixels:   %lld\n", nside, hpnpix);
  {
    /* pks2map.f90:134-137: cut distances from the r(z) table, printed as f4.2 Gpc */
    p2m_cosmo cosmo;
    std::vector<float> rofz(P2M_NZTAB), zofr(P2M_NZTAB);
    p2m_cosmo_build(&cosmo, rofz.data(), zofr.data());
    auto f42 = [](float v) {
      char b[16];
      if (!(v > -0.995f && v < 9.995f)) return std::string("****");
      std::snprintf(b, sizeof b, "%4.2f", v);
      return std::string(b);
    };
    std::printf("cut_low, cut_high:  %s %s Gpc\n",
                f42(p2m_lookup(rofz.data(), cosmo.drofz, zmin) / 1e3f).c_str(),
                f42(p2m_lookup(rofz.data(), cosmo.drofz, zmax) / 1e3f).c_str());
  }

  const double t_start = now_s();
  std::vector<char> table;
  if (!read_file(tablefile, table)) return fail("cannot read the table file");
  FILE *cf = std::fopen(filein, "rb");
  if (!cf) return fail("cannot read the catalogue");
  std::fseek(cf, 0, SEEK_END);
  const long long fsize = std::ftell(cf);
  std::fseek(cf, 0, SEEK_SET);
  int32_t nhalo = 0;
  if (fsize < 8 || std::fread(&nhalo, 4, 1, cf) != 1) {
    std::fclose(cf);
    return fail("cannot read the catalogue");
  }
  /* 7 floats after a 2-word header (pksc.f90:46-66) or 10 after a 3-word header */
  int nfloat = 0, hdr = 0;
  if (nhalo >= 0 && fsize == 8 + 28LL * nhalo) nfloat = 7, hdr = 8;
  else if (nhalo >= 0 && fsize == 12 + 40LL * nhalo) nfloat = 10, hdr = 12;
  if (!nfloat) {
    std::fclose(cf);
    return fail("catalogue size matches neither 8+28N nor 12+40N bytes");
  }
  std::fseek(cf, hdr, SEEK_SET);

  p2m_config cfg;
  std::memset(&cfg, 0, sizeof cfg);
  cfg.nside = nside;
  cfg.npix_fs = npix;
  cfg.fov_deg = fov_deg;
  cfg.zmin = zmin;
  cfg.zmax = zmax;
  cfg.chihview = chihview;
  cfg.model = model;
  cfg.precision = P2M_PREC_MIXED;
  if (const char *e = std::getenv("P2M_PRECISION")) {
    if (!std::strcmp(e, "fp64")) cfg.precision = P2M_PREC_FP64;
    else if (!std::strcmp(e, "mixed64")) cfg.precision = P2M_PREC_MIXED_F64;
    else if (!std::strcmp(e, "fixed")) cfg.precision = P2M_PREC_FIXED;
  }
  cfg.nmaps = 1;
  cfg.map_table[0] = 0;
  cfg.map_profile[0] = profile;
  const long long chunk = 1LL << 22; /* records per read and paint step */
  cfg.max_records = nhalo < chunk ? (nhalo > 0 ? nhalo : 1) : chunk;
  if (scramble || centre) cfg.max_records = nhalo > 0 ? nhalo : 1; /* one pass: one catalogue */
  cfg.device = std::getenv("P2M_DEVICE") ? std::atoi(std::getenv("P2M_DEVICE")) : 0;
  p2m_ctx *ctx = nullptr;
  int st = p2m_create(&cfg, &ctx);
  if (st) {
    std::fclose(cf);
    return fail("p2m_create", ctx, st);
  }
  st = p2m_load_table(ctx, 0, table.data(), (int64_t)table.size());
  if (st) {
    std::fclose(cf);
    return fail("p2m_load_table", ctx, st);
  }
  if ((st = p2m_set_preprocess(ctx, scramble, centre, ranks))) {
    std::fclose(cf);
    return fail("p2m_set_preprocess", ctx, st);
  }
  const double t_setup = now_s(); /* CUDA context, device buffers, table */
  /* the catalogue is read in steps of max_records records into two page-locked buffers
     (the copies to the device then need no staging); a reader thread reads step k + 1
     from the file, by positioned reads over several threads, while step k is painted */
  {
    const long long step = cfg.max_records;
    const long long cap = std::min<long long>(step, (long long)nhalo) * nfloat;
    float *buf[2] = {nullptr, nullptr};
    std::vector<float> plain[2]; /* if page-locked memory is refused */
    for (int b = 0; b < 2; b++) {
      void *q = nullptr;
      if (cap > 0 && p2m_host_alloc((int64_t)(sizeof(float) * (size_t)cap), &q) == P2M_OK) {
        buf[b] = (float *)q;
      } else {
        plain[b].resize((size_t)std::max<long long>(cap, 1));
        buf[b] = plain[b].data();
      }
    }
    auto release = [&]() {
      for (int b = 0; b < 2; b++)
        if (plain[b].empty()) p2m_host_free(buf[b]);
    };
    long long count[2] = {0, 0};
    bool read_ok[2] = {true, true};
    auto read_step = [&](int b, long long first) {
      const long long n = std::min<long long>(step, (long long)nhalo - first);
      count[b] = n;
      read_ok[b] = n <= 0 || p2m_pread_all(fileno(cf), buf[b], sizeof(float) * nfloat * (size_t)n,
                                           hdr + 4LL * nfloat * first);
    };
    read_step(0, 0);
    for (long long first = 0, k = 0; first < nhalo; first += step, k++) {
      const int b = (int)(k & 1);
      std::thread reader;
      if (first + step < nhalo) reader = std::thread(read_step, 1 - b, first + step);
      if (read_ok[b]) st = p2m_paint_records(ctx, buf[b], (int64_t)count[b], nfloat);
      if (reader.joinable()) reader.join();
      if (!read_ok[b] || st) {
        release();
        std::fclose(cf);
        return read_ok[b] ? fail("p2m_paint_records", ctx, st)
                          : fail("cannot read the catalogue", ctx);
      }
    }
    /* p2m_paint_records returns once its records are on the device */
    release();
  }
  std::fclose(cf);
  if (centre) {
    /* pks2map.f90:205-209 and :250-254 */
    float c[9];
    p2m_get_centre(ctx, c);
    std::printf("\nBefore rotation largest halo is at\nRTH, distance:    %s %s \nx, y, z:          %s %s %s \n\n",
                fe(c[0], 3).c_str(), fe(c[1], 3).c_str(), e103(c[2]).c_str(), e103(c[3]).c_str(),
                e103(c[4]).c_str());
    std::printf("\nAfter rotation largest halo is at\nRTH, distance:    %s %s \nx, y, z:          %s %s %s \n\n",
                fe(c[0], 3).c_str(), fe(c[5], 3).c_str(), e103(c[6]).c_str(), e103(c[7]).c_str(),
                e103(c[8]).c_str());
  }

  /* pks2map.f90:318-357: halo count, moments, RMS and mean, P(<y): on the device */
  p2m_stats stats;
  if ((st = p2m_get_stats(ctx, &stats))) return fail("p2m_get_stats", ctx, st);
  const double t_paint = now_s();
  p2m_map_stats hs, fss;
  std::memset(&hs, 0, sizeof hs);
  std::memset(&fss, 0, sizeof fss);
  std::vector<float> dpdy(P2M_NDPDY);
  if (nside > 0 && (st = p2m_get_healpix_stats(ctx, 0, &hs, dpdy.data())))
    return fail("p2m_get_healpix_stats", ctx, st);
  if (npix > 0 && (st = p2m_get_flatsky_stats(ctx, 0, &fss)))
    return fail("p2m_get_flatsky_stats", ctx, st);
  const double t_stats = now_s();
  std::printf("Number of halos in map:    %lld\n", (long long)stats.n_painted);
  std::printf("Flatsky moments:    %s %s %s \n", fe(fss.mom[0], 3).c_str(), fe(fss.mom[1], 3).c_str(),
              fe(fss.mom[2], 3).c_str());
  std::printf("Healpix moments:    %s %s %s \n", fe(hs.mom[0], 3).c_str(), fe(hs.mom[1], 3).c_str(),
              fe(hs.mom[2], 3).c_str());
  std::printf("Flatsky RMS:                %s\nFlatsky Mean:               %s\n",
              fe(fss.rms, 3).c_str(), fe(fss.mom[0], 2).c_str());
  std::printf("Healpix RMS:                %s\nHealpix Mean:               %s\n\n",
              fe(hs.rms, 3).c_str(), fe(hs.mom[0], 2).c_str());

  /* pks2map.f90:359-385: the three files */
  const std::string out = fileout;
  if (nside > 0 && (st = p2m_write_dpdy((out + "_dp.bin").c_str(), dpdy.data())))
    return fail("cannot write _dp.bin", ctx, st);
  std::vector<float> fs((size_t)npix * (size_t)npix);
  if (npix > 0 && (st = p2m_get_flatsky(ctx, 0, fs.data()))) return fail("p2m_get_flatsky", ctx, st);
  if ((st = p2m_write_flatsky((out + "_fs.map").c_str(), fs.data(), npix, fov)))
    return fail("cannot write _fs.map", ctx, st);
  if (nside > 0 && (st = p2m_write_healpix_fits_device(ctx, 0, (out + "_hp.fits").c_str())))
    return fail("cannot write _hp.fits", ctx, st);
  const double t_written = now_s();
  p2m_destroy(ctx);
  const double t_end = now_s();
  std::printf("\n");
  if (std::getenv("P2M_TIMING"))
    std::fprintf(stderr,
                 "pks2map timing: read + paint %.4f s, statistics %.4f s, writes %.4f s, "
                 "total %.4f s; of these, set-up (CUDA context, buffers, table) %.4f s and "
                 "release %.4f s\n",
                 t_paint - t_start, t_stats - t_paint, t_end - t_stats, t_end - t_start,
                 t_setup - t_start, t_end - t_written);
  return 0;
}
