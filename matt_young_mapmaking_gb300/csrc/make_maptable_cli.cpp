/*
 * make_maptable_cli.cpp -- the make_maptable command line on the GPU
 * (make_maptable.f90:20-45, maptable.f90:25-146).
 *
 *   make_maptable <fileout> <model> [<frequency> <alpha_CMB>]
 *
 * Builds the 100 x 100 x 200 profile table with p2m_make_maptable (include/p2m.h) and
 * writes it in the reference's file layout: int32 nchit, nmht, nrt, float32 chimint,
 * chimaxt, mhmint, mhmaxt, rmint, rmaxt, float32 table(2, nrt, nmht, nchit).  Device from
 * P2M_DEVICE (default 0).
 */
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/p2m.h"

namespace {
bool is_dot(const char *s) { return std::strcmp(s, ".") == 0; }
int i4arg(int argc, char **argv, int k, int def) {
  if (k >= argc || is_dot(argv[k])) return def;
  char *end = nullptr;
  long v = std::strtol(argv[k], &end, 10);
  return (end == argv[k] || *end) ? def : (int)v;
}
float r4arg(int argc, char **argv, int k, float def) {
  if (k >= argc || is_dot(argv[k])) return def;
  char *end = nullptr;
  double v = std::strtod(argv[k], &end);
  return (end == argv[k] || *end) ? def : (float)v;
}
}  // namespace

int main(int argc, char **argv) {
  /* make_maptable.f90:20-23 asks for at least three arguments */
  if (argc - 1 < 3) {
    std::printf("Usage: make_maptable <fileout> <model> [<frequency> <alpha_CMB>]\n");
    return 0;
  }
  const char *fileout = argv[1];
  const int model = i4arg(argc, argv, 2, 1);
  const float nu = r4arg(argc, argv, 3, 0.0f);
  const float alpha = r4arg(argc, argv, 4, 0.0f);
  const int device = std::getenv("P2M_DEVICE") ? std::atoi(std::getenv("P2M_DEVICE")) : 0;
  std::printf("\n Making Maptable. Will take a minute\n\n");
  int64_t nbytes = 0;
  int st = p2m_make_maptable(device, model, nu, alpha, 0, 0, 0, nullptr, &nbytes);
  if (st) {
    std::fprintf(stderr, "make_maptable: status %d\n", st);
    return 1;
  }
  std::vector<char> image((size_t)nbytes);
  st = p2m_make_maptable(device, model, nu, alpha, 0, 0, 0, image.data(), &nbytes);
  if (st) {
    std::fprintf(stderr, "make_maptable: status %d\n", st);
    return 1;
  }
  FILE *f = std::fopen(fileout, "wb");
  if (!f || std::fwrite(image.data(), 1, image.size(), f) != image.size()) {
    std::fprintf(stderr, "make_maptable: cannot write %s\n", fileout);
    if (f) std::fclose(f);
    return 1;
  }
  std::fclose(f);
  return 0;
}
