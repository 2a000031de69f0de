// A C++ caller of libgbrmsd that does what a patched
// Analysis_Rms2d::Calculate_2D does: frames gathered into one
// host buffer of doubles (as GetFrame fills a Frame), one handle per process,
// one gbr_allpairs call per matrix, errors reported through gbr_last_error.
//
//   rms2d_caller <in.bin> <out.bin>
// in.bin:  int64 n_frame, int32 n_atom, int32 flags (bit 0: masses follow),
//          double xyz[n_frame][n_atom][3], double mass[n_atom] (if flagged)
// out.bin: float tri[n_frame*(n_frame-1)/2]   (fit, tensor-core precision)
//          float full[n_frame*(n_frame/2)]    (FULL: the first half of the frames
//                                               as references, the second as targets)
//          float dme[n_frame*(n_frame-1)/2]   (dme mode)
// Exit status 0 on success; the zero-mass call must fail with GBR_ERR_ZERO_MASS.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "gbrmsd.h"

static int fail(const char* what, gbr_handle* h, int rc) {
  std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, h ? gbr_last_error(h) : "");
  return 1;
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  std::FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int64_t F = 0;
  int32_t N = 0, flags = 0;
  if (std::fread(&F, 8, 1, f) != 1 || std::fread(&N, 4, 1, f) != 1 || std::fread(&flags, 4, 1, f) != 1) return 2;
  std::vector<double> xyz((size_t)F * N * 3), mass;
  if (std::fread(xyz.data(), 8, xyz.size(), f) != xyz.size()) return 2;
  if (flags & 1) {
    mass.resize(N);
    if (std::fread(mass.data(), 8, N, f) != (size_t)N) return 2;
  }
  std::fclose(f);
  const double* m = mass.empty() ? nullptr : mass.data();

  gbr_handle* h = gbr_create(0);
  if (!h) return fail("gbr_create", nullptr, -1);
  const int64_t ntri = gbr_output_count(F, F, GBR_TRI, 0, -1);
  std::vector<float> tri(ntri);
  int rc = gbr_allpairs(h, xyz.data(), nullptr, GBR_F64, F, F, N, m, m, GBR_FIT, GBR_TRI, GBR_PREC_TC, tri.data(), 0,
                        -1);
  if (rc != GBR_OK) return fail("gbr_allpairs TRI", h, rc);

  const int64_t nr = F / 2, nt = F - F / 2;
  std::vector<float> full(gbr_output_count(nr, nt, GBR_FULL, 0, -1));
  rc = gbr_allpairs(h, xyz.data(), xyz.data() + (size_t)nr * N * 3, GBR_F64, nr, nt, N, m, m, GBR_FIT, GBR_FULL,
                    GBR_PREC_TC, full.data(), 0, -1);
  if (rc != GBR_OK) return fail("gbr_allpairs FULL", h, rc);

  std::vector<float> dme(ntri);
  rc = gbr_allpairs(h, xyz.data(), nullptr, GBR_F64, F, F, N, nullptr, nullptr, GBR_DME, GBR_TRI, GBR_PREC_TC,
                    dme.data(), 0, -1);
  if (rc != GBR_OK) return fail("gbr_allpairs DME", h, rc);

  // A zero total mass is an error of the call, as Frame::RMSD reports it.
  std::vector<double> zero(N, 0.0);
  rc = gbr_allpairs(h, xyz.data(), nullptr, GBR_F64, F, F, N, zero.data(), zero.data(), GBR_FIT, GBR_TRI,
                    GBR_PREC_FP32, tri.data() /* untouched on error */, 0, -1);
  if (rc != GBR_ERR_ZERO_MASS || gbr_last_error(h)[0] == '\0') {
    std::fprintf(stderr, "zero-mass call returned %d\n", rc);
    return 1;
  }
  gbr_destroy(h);

  std::FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 2;
  std::fwrite(tri.data(), 4, tri.size(), o);
  std::fwrite(full.data(), 4, full.size(), o);
  std::fwrite(dme.data(), 4, dme.size(), o);
  std::fclose(o);
  return 0;
}
