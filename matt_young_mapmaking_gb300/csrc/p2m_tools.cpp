/*
 * p2m_tools.cpp -- synthetic catalogue generator (include/p2m_tools.h).
 *
 * Philox4x32-10 is the counter-based generator of Salmon, Moraes, Dror and Shaw,
 * "Parallel random numbers: as easy as 1, 2, 3" (SC 2011), restated from the paper:
 * ten rounds of two 32x32->64 multiplies with the round constants below and a Weyl
 * key schedule.  Derived quantities use double precision and are stored as float.
 */
#include <cmath>
#include <cstdint>
#include <algorithm>
#include <thread>
#include <vector>

#include "../../include/p2m_tools.h"

namespace {
const uint32_t PH_M0 = 0xD2511F53u, PH_M1 = 0xCD9E8D57u;
const uint32_t PH_W0 = 0x9E3779B9u, PH_W1 = 0xBB67AE85u;

inline double u01(uint32_t x) { return ((double)x + 0.5) * (1.0 / 4294967296.0); }

void gen_range(uint64_t seed, int64_t first, int64_t n, int32_t nfloat, double r_min,
               double r_max, double m_min, double m_max, double slope, double sigma_v,
               float *out) {
  const uint32_t key[2] = {(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32)};
  const double r03 = r_min * r_min * r_min, r13 = r_max * r_max * r_max;
  const double ma = std::pow(m_min, slope), mb = std::pow(m_max, slope);
  const double rth_fac = 3.0 / (4.0 * M_PI * 0.31 * 2.775e11 * 0.68 * 0.68);
  for (int64_t j = 0; j < n; j++) {
    uint64_t idx = (uint64_t)(first + j);
    uint32_t c0[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 0u, 0u};
    uint32_t c1[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 1u, 0u};
    uint32_t a[4], b[4];
    p2m_philox4x32(c0, key, a);
    p2m_philox4x32(c1, key, b);
    double r = std::cbrt(r03 + u01(a[0]) * (r13 - r03));
    double mu = 2.0 * u01(a[1]) - 1.0;
    double ph = 2.0 * M_PI * u01(a[2]);
    double st = std::sqrt(std::fmax(0.0, 1.0 - mu * mu));
    double x = r * st * std::cos(ph), y = r * st * std::sin(ph), z = r * mu;
    double m = std::pow(ma + u01(a[3]) * (mb - ma), 1.0 / slope);
    double rth = std::cbrt(rth_fac * m);
    /* Box-Muller: two pairs of normals */
    double g1 = std::sqrt(-2.0 * std::log(u01(b[0]))), t1 = 2.0 * M_PI * u01(b[1]);
    double g2 = std::sqrt(-2.0 * std::log(u01(b[2]))), t2 = 2.0 * M_PI * u01(b[3]);
    double vx = sigma_v * g1 * std::cos(t1), vy = sigma_v * g1 * std::sin(t1);
    double vz = sigma_v * g2 * std::cos(t2);
    float *o = out + j * nfloat;
    o[0] = (float)x;
    o[1] = (float)y;
    o[2] = (float)z;
    o[3] = (float)vx;
    o[4] = (float)vy;
    o[5] = (float)vz;
    o[6] = (float)rth;
    if (nfloat == 10) {
      o[7] = (float)(x - 0.01 * vx);
      o[8] = (float)(y - 0.01 * vy);
      o[9] = (float)(z - 0.01 * vz);
    }
  }
}
}  // namespace

extern "C" {

void p2m_philox4x32(const uint32_t c[4], const uint32_t k[2], uint32_t out[4]) {
  uint32_t x0 = c[0], x1 = c[1], x2 = c[2], x3 = c[3];
  uint32_t k0 = k[0], k1 = k[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)PH_M0 * x0, p1 = (uint64_t)PH_M1 * x2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t y0 = hi1 ^ x1 ^ k0, y1 = lo1, y2 = hi0 ^ x3 ^ k1, y3 = lo0;
    x0 = y0;
    x1 = y1;
    x2 = y2;
    x3 = y3;
    k0 += PH_W0;
    k1 += PH_W1;
  }
  out[0] = x0;
  out[1] = x1;
  out[2] = x2;
  out[3] = x3;
}

int32_t p2m_generate_catalogue(uint64_t seed, int64_t first, int64_t n, int32_t nfloat,
                               double r_min, double r_max, double m_min, double m_max,
                               double slope, double sigma_v, float *out) {
  if (!out || n < 0 || first < 0 || (nfloat != 7 && nfloat != 10)) return 1;
  if (!(r_min >= 0 && r_max >= r_min && m_min > 0 && m_max >= m_min && slope != 0.0)) return 1;
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  if (n < 65536) nt = 1;
  if (nt > 64) nt = 64;
  std::vector<std::thread> th;
  int64_t per = (n + nt - 1) / nt;
  for (unsigned t = 0; t < nt; t++) {
    int64_t lo = per * t, hi = std::min<int64_t>(n, lo + per);
    if (lo >= hi) break;
    th.emplace_back(gen_range, seed, first + lo, hi - lo, nfloat, r_min, r_max, m_min, m_max,
                    slope, sigma_v, out + lo * nfloat);
  }
  for (auto &t : th) t.join();
  return 0;
}

}  // extern "C"
