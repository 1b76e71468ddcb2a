/*
 * p2m_outputs.cpp -- the output files of pks2map (include/p2m_tools.h), host code.
 *
 *   <out>_dp.bin   int32 ndpdy, float32 dpdy_max, float32 P(<y)[ndpdy]  (pks2map.f90:366-373)
 *   <out>_fs.map   int32 npix, npix, float32 fov, fov (radians), float32 map[npix^2],
 *                  j (theta) fastest                                     (pks2map.f90:375-379)
 *   <out>_hp.fits  FITS: an empty primary HDU, then a BINTABLE with one column of
 *                  1024-element float rows holding the RING-ordered map, NSIDE and
 *                  ORDERING='RING' cards (pks2map.f90:381-385 through HEALPix
 *                  output_map / write_bintab, fits_s_inc.f90:787-960)
 *
 * The binary files follow the reference's `form='binary'` sequential writes: the values
 * back to back in host byte order, no record markers.  The FITS file is written here
 * directly (FITS 4.0: 80-byte cards, 2880-byte blocks, big-endian IEEE floats).
 */
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "../../include/p2m.h"
#include "../../include/p2m_tools.h"
#include "p2m_fits.h"

namespace {

/* pks2map.f90:39-40: `real, parameter :: dpdy_max = 1e-4, dpdy_dy = dpdy_max/ndpdy` */
const float kDpdyMax = 1e-4f;

struct File {
  FILE *f;
  explicit File(const char *path) : f(path ? std::fopen(path, "wb") : nullptr) {}
  ~File() {
    if (f) std::fclose(f);
  }
  bool put(const void *p, size_t n) { return f && std::fwrite(p, 1, n, f) == n; }
};

/* one 80-character header card */
std::string card(const std::string &text) {
  std::string c = text.substr(0, 80);
  c.resize(80, ' ');
  return c;
}
std::string card_value(const char *key, const std::string &value, const char *comment) {
  char kw[9];
  std::snprintf(kw, sizeof kw, "%-8s", key);
  std::string s = std::string(kw) + "= " + value;
  if (comment && *comment) s += " / " + std::string(comment);
  return card(s);
}
std::string fixed(long long v) {
  char b[32];
  std::snprintf(b, sizeof b, "%20lld", v);
  return b;
}
std::string logical(bool v) { return std::string(19, ' ') + (v ? "T" : "F"); }
std::string quoted(const std::string &v) {
  std::string q = "'" + v;
  while (q.size() < 9) q += ' '; /* string values are at least 8 characters */
  return q + "'";
}

/* header cards padded with blanks to whole 2880-byte blocks, after END */
bool put_header(File &f, std::vector<std::string> cards) {
  cards.push_back(card("END"));
  std::string h;
  for (auto &c : cards) h += c;
  h.resize((h.size() + 2879) / 2880 * 2880, ' ');
  return f.put(h.data(), h.size());
}

uint32_t to_big_endian(float v) {
  uint32_t u;
  std::memcpy(&u, &v, 4);
  return (u >> 24) | ((u >> 8) & 0xff00u) | ((u << 8) & 0xff0000u) | (u << 24);
}

}  // namespace

extern "C" {

int32_t p2m_dpdy(const float *map, int64_t npix, float *dpdy) {
  if (!map || !dpdy || npix <= 0) return P2M_ERR_BADARG;
  const float dy = kDpdyMax / (float)P2M_NDPDY;
  for (int k = 0; k < P2M_NDPDY; k++) dpdy[k] = 0.0f;
  /* pks2map.f90:341-346: m = int(y / dpdy_dy) + 1 (truncation toward zero), counted in
     float as the reference does, so a bin stops at 2^24 */
  for (int64_t i = 0; i < npix; i++) {
    const float q = map[i] / dy;
    if (!(q > -1.0f && q < (float)P2M_NDPDY)) continue; /* m outside 1..ndpdy */
    const int m = (int)q + 1;
    if (m > 0 && m <= P2M_NDPDY) dpdy[m - 1] = dpdy[m - 1] + 1.0f;
  }
  /* :347 normalisation, :355-357 cumulation */
  const float norm = (float)npix;
  for (int k = 0; k < P2M_NDPDY; k++) dpdy[k] = dpdy[k] / norm;
  for (int k = 1; k < P2M_NDPDY; k++) dpdy[k] = dpdy[k - 1] + dpdy[k];
  return P2M_OK;
}

int32_t p2m_write_dpdy(const char *path, const float *dpdy) {
  if (!path || !dpdy) return P2M_ERR_BADARG;
  File f(path);
  const int32_t n = P2M_NDPDY;
  const float mx = kDpdyMax;
  if (!f.put(&n, 4) || !f.put(&mx, 4) || !f.put(dpdy, sizeof(float) * P2M_NDPDY))
    return P2M_ERR_IO;
  return P2M_OK;
}

int32_t p2m_write_flatsky(const char *path, const float *map, int32_t npix, float fov_rad) {
  if (!path || (!map && npix > 0) || npix < 0) return P2M_ERR_BADARG;
  File f(path);
  if (!f.put(&npix, 4) || !f.put(&npix, 4) || !f.put(&fov_rad, 4) || !f.put(&fov_rad, 4))
    return P2M_ERR_IO;
  if (npix > 0 && !f.put(map, sizeof(float) * (size_t)npix * (size_t)npix)) return P2M_ERR_IO;
  return P2M_OK;
}

int32_t p2m_write_healpix_fits(const char *path, const float *map, int32_t nside) {
  if (!path || !map || nside < 1) return P2M_ERR_BADARG;
  const long long npix = 12LL * nside * nside;
  File f(path);
  if (!f.f) return P2M_ERR_IO;
  if (p2m_fits_put_header(f.f, nside) != P2M_OK) return P2M_ERR_IO;
  std::vector<uint32_t> buf(1 << 20);
  for (long long i0 = 0; i0 < npix; i0 += (long long)buf.size()) {
    const long long n = std::min<long long>((long long)buf.size(), npix - i0);
    for (long long k = 0; k < n; k++) buf[(size_t)k] = to_big_endian(map[i0 + k]);
    if (!f.put(buf.data(), sizeof(uint32_t) * (size_t)n)) return P2M_ERR_IO;
  }
  return p2m_fits_put_padding(f.f, nside);
}

}  // extern "C"

/* the two headers of a HEALPix FITS map (an empty primary HDU, then the BINTABLE) */
int32_t p2m_fits_put_header(FILE *fp, int32_t nside) {
  const long long npix = 12LL * nside * nside;
  /* fits_s_inc.f90:904-908: rows of 1024 values (1 for npix < 1024) */
  long long repeat = npix < 1024 ? 1 : 1024;
  if (nside > 1024 * 256) repeat = nside / 256;
  const long long nrows = npix / repeat;
  File f(nullptr);
  f.f = fp;
  char date[16];
  std::time_t now = std::time(nullptr);
  std::strftime(date, sizeof date, "%Y-%m-%d", std::gmtime(&now));
  std::vector<std::string> primary = {
      card_value("SIMPLE", logical(true), "file does conform to FITS standard"),
      card_value("BITPIX", fixed(32), "number of bits per data pixel"),
      card_value("NAXIS", fixed(0), "number of data axes"),
      card_value("EXTEND", logical(true), "FITS dataset may contain extensions"),
      card_value("DATE", quoted(date), "file creation date (YYYY-MM-DD)")};
  if (!put_header(f, primary)) return P2M_ERR_IO;
  std::string form = std::to_string(repeat) + "E";
  std::vector<std::string> ext = {
      card_value("XTENSION", quoted("BINTABLE"), "binary table extension"),
      card_value("BITPIX", fixed(8), "8-bit bytes"),
      card_value("NAXIS", fixed(2), "2-dimensional binary table"),
      card_value("NAXIS1", fixed(4 * repeat), "width of table in bytes"),
      card_value("NAXIS2", fixed(nrows), "number of rows in table"),
      card_value("PCOUNT", fixed(0), "size of special data area"),
      card_value("GCOUNT", fixed(1), "one data group (required keyword)"),
      card_value("TFIELDS", fixed(1), "number of fields in each row"),
      card_value("TTYPE1", quoted("simulation"), "label for field   1"),
      card_value("TFORM1", quoted(form), "data format of field: 4-byte REAL"),
      card_value("NSIDE", fixed(nside), "the nside of the map"),
      card_value("ORDERING", quoted("RING"), "the nside of the map")};
  const bool ok = put_header(f, ext);
  f.f = nullptr; /* the caller owns the stream */
  return ok ? P2M_OK : P2M_ERR_IO;
}

/* the zero bytes that complete the data of a map's BINTABLE to whole 2880-byte blocks */
int32_t p2m_fits_put_padding(FILE *fp, int32_t nside) {
  const long long data = 4 * 12LL * nside * nside, pad = (data + 2879) / 2880 * 2880 - data;
  std::vector<char> zeros((size_t)pad, 0);
  if (pad && std::fwrite(zeros.data(), 1, (size_t)pad, fp) != (size_t)pad) return P2M_ERR_IO;
  return P2M_OK;
}
