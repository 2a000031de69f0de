// gbr_cmatrix.cu -- gbr_write_cmatrix: the clustering pairwise cache computed
// on the GPU and written straight to cpptraj's binary cluster-matrix file.
//
// File layout (version 2, as Cpptraj::Cluster::Cmatrix_Binary::WriteCmatrix
// writes it, src/Cluster/Cmatrix_Binary.cpp:141-188):
//   4 bytes  'C' 'T' 'M' 2
//   uint64   number of original frames (length of the frame-to-row map)
//   uint64   rows of the cached matrix
//   int64    sieve value (1 = no sieve, negative = random sieve)
//   float    rows*(rows-1)/2 distances in calcTriIndex order
//   char     one 'T' (sieved out) / 'F' (cached) per original frame, only
//            when the sieve value is not 1.
// The triangle is streamed (gbr_allpairs_stream): it is computed in row
// bands, each band is written to the file while the next ones compute, and
// device memory holds two bands at a time -- a cache of any size is written
// at disk speed without a host round trip per element
// (DataSet_PairwiseCache_NC::SetElement writes one element at a time in the
// reference).  GBR_DME, which is not streamed, computes the whole triangle
// in device memory and writes it in 64 MB pieces.
#include <cstdio>
#include <cstring>

#include "gbr_handle.h"

using namespace gbr;

extern "C" int gbr_write_cmatrix(gbr_handle* h, const char* path, const void* xyz, int dtype, int64_t n_frame,
                                 int32_t n_atom, const double* mass, int mode, int precision,
                                 const int32_t* frame_to_idx, int64_t n_original, int64_t sieve) {
  if (!h) return GBR_ERR_ARG;
  if (!path || !xyz) return h->fail(GBR_ERR_ARG, "cmatrix: path and xyz must not be NULL");
  if (frame_to_idx == nullptr) {
    n_original = n_frame;
    sieve = 1;
  } else {
    int64_t kept = 0;
    for (int64_t k = 0; k < n_original; ++k) {
      if (frame_to_idx[k] >= 0) {
        if (frame_to_idx[k] != kept) return h->fail(GBR_ERR_ARG, "cmatrix: frame_to_idx must number cached rows in order");
        ++kept;
      }
    }
    if (kept != n_frame) return h->fail(GBR_ERR_ARG, "cmatrix: frame_to_idx caches %lld frames, n_frame is %lld",
                                        (long long)kept, (long long)n_frame);
  }
  const int64_t n = (n_frame > 1) ? n_frame * (n_frame - 1) / 2 : 0;
  if (cudaSetDevice(h->device) != cudaSuccess) return h->cuda_fail(cudaGetLastError(), "cudaSetDevice");
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return h->fail(GBR_ERR_IO, "cmatrix: cannot open %s for writing", path);
  bool ok = true;
  const unsigned char magic[4] = {'C', 'T', 'M', 2};
  const uint64_t orig = (uint64_t)n_original, rows = (uint64_t)n_frame;
  const int64_t sv = sieve;
  ok = ok && std::fwrite(magic, 1, 4, fp) == 4;
  ok = ok && std::fwrite(&orig, sizeof orig, 1, fp) == 1;
  ok = ok && std::fwrite(&rows, sizeof rows, 1, fp) == 1;
  ok = ok && std::fwrite(&sv, sizeof sv, 1, fp) == 1;
  gbr_stats st{};
  if (ok && n > 0 && mode != GBR_DME) {
    // each band goes to the file as it arrives, in row order
    struct Sink {
      FILE* fp;
      static int write(void* user, int64_t, int64_t, const float* v, int64_t count) {
        FILE* f = static_cast<Sink*>(user)->fp;
        return std::fwrite(v, sizeof(float), (size_t)count, f) == (size_t)count ? 0 : 1;
      }
    } sink{fp};
    const int rc = gbr_allpairs_stream(h, xyz, dtype, n_frame, n_atom, mass, mode, precision, h->band_floats,
                                       &Sink::write, &sink);
    if (rc != GBR_OK) {
      std::fclose(fp);
      return rc;
    }
    st = h->stats;
  } else if (ok && n > 0) {
    if (!h->reserve_out((size_t)n)) {
      std::fclose(fp);
      return h->fail(GBR_ERR_NOMEM, "cmatrix: cannot hold %lld floats", (long long)n);
    }
    const int rc = gbr_allpairs(h, xyz, nullptr, dtype, n_frame, n_frame, n_atom, mass, mass, mode, GBR_TRI,
                                precision, h->outbuf, 0, -1);
    if (rc != GBR_OK) {
      std::fclose(fp);
      return rc;
    }
    st = h->stats;  // keep the compute call's statistics
    const size_t chunk = (size_t)16 << 20;  // floats per chunk (64 MB)
    if (!h->reserve_pinned(2 * chunk * sizeof(float))) {
      std::fclose(fp);
      return h->fail(GBR_ERR_NOMEM, "cmatrix: cannot allocate pinned staging");
    }
    float* buf[2] = {(float*)h->pinned, (float*)h->pinned + chunk};
    cudaEvent_t done[2];
    cudaEventCreateWithFlags(&done[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&done[1], cudaEventDisableTiming);
    const size_t nchunks = ((size_t)n + chunk - 1) / chunk;
    auto issue = [&](size_t k) {
      const size_t off = k * chunk, len = std::min(chunk, (size_t)n - off);
      cudaMemcpyAsync(buf[k & 1], h->outbuf + off, len * sizeof(float), cudaMemcpyDeviceToHost, h->stream);
      cudaEventRecord(done[k & 1], h->stream);
    };
    issue(0);
    for (size_t k = 0; k < nchunks && ok; ++k) {
      cudaEventSynchronize(done[k & 1]);
      if (k + 1 < nchunks) issue(k + 1);  // the other buffer was written to disk in the previous round
      const size_t off = k * chunk, len = std::min(chunk, (size_t)n - off);
      ok = std::fwrite(buf[k & 1], sizeof(float), len, fp) == len;
    }
    cudaStreamSynchronize(h->stream);
    cudaEventDestroy(done[0]);
    cudaEventDestroy(done[1]);
  }
  if (ok && sieve != 1) {
    for (int64_t k = 0; k < n_original && ok; ++k) {
      const char c = (frame_to_idx[k] == -1) ? 'T' : 'F';
      ok = std::fputc(c, fp) != EOF;
    }
  }
  if (std::fclose(fp) != 0) ok = false;
  h->stats = st;
  if (!ok) return h->fail(GBR_ERR_IO, "cmatrix: write to %s failed", path);
  return GBR_OK;
}
