// gbr_capi.cu -- the extern "C" boundary (include/gbrmsd.h) and the host-side
// orchestration of one all-pairs call:
//   stage inputs -> centre + pick references + superpose (gbr_prep.cu)
//   -> per-frame terms -> pair contraction (FP32 CUDA cores or tcgen05)
//   -> FP64 re-check of flagged pairs (gbr_exact.cu) -> results to the caller.
// It replaces the OpenMP pair loops of Analysis_Rms2d::Calculate_2D
// (src/Analysis_Rms2d.cpp:247-290) and MetricArray::calcFrameDistances
// (src/Cluster/MetricArray.cpp:777-800) as one call from the master thread.
#include <cuda_fp16.h>

#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gbrmsd.h"
#include "gbr_handle.h"
#include "gbr_internal.h"

using namespace gbr;

namespace {
constexpr int kMaxBands = 8;  // output row bands whose copies overlap the contraction
// Atom count from which the pair-of-SMs kernel uses its deep operand pipeline
// (64-atom stages x 3, measured 6-7 % faster at 1,500-3,000 atoms): below it
// the per-pair epilogue, not the operand feed, bounds the kernel, and the
// wider epilogue chunks of the shallow shape win (9 % at 1,024 atoms, 20 % at
// 500).  The deep shape's 4-frame chunks store 16-byte row segments, which
// HBM's L2 merges but the host link does not: results written straight into
// pinned host memory keep the shallow shape.
constexpr int kDeepStageAtoms = 1280;
// Below this atom count the epilogue bounds the pair kernel harder still and
// the wide-chunk shape (16-frame chunks, 3 stages: half the epilogue's named
// barriers per pair) wins: measured 4-5 % at 300 and 500 atoms, 7 % slower at
// 1,000.
constexpr int kWideChunkAtoms = 768;
int auto_tc_variant(int N) { return N >= kDeepStageAtoms ? 3 : (N < kWideChunkAtoms ? 4 : 2); }

// Whole rows of a triangle, from device memory to the caller's buffer (the
// device alias of pinned host memory, 16-byte aligned like the source): row
// i = rows[r] for r in [0, nrows), the n - 1 - i values from
// tri_index(n, i, i + 1) = n i - i (i + 1) / 2 on, the same positions in
// both.  One warp per row at a time: a scalar head up to a 16-byte boundary,
// then 16-byte pieces four at a time per lane (whole 128-byte lines per
// warp store across the host link), then the scalar tail.  The contraction
// bands run on all but kCopyFreeClusters clusters; the copy's blocks take the
// SMs left free (their shared-memory reservation, unused, keeps them from
// sharing an SM with a contraction CTA, which slowed the contraction as much
// as the overlap saved).
constexpr int kCopyFreeClusters = 4, kCopyBlocks = 2 * kCopyFreeClusters, kCopyThreads = 1024;
constexpr int kCopySmem = 64 << 10;
__global__ void __launch_bounds__(kCopyThreads) k_copy_rows(const int* rows, int64_t nrows, int64_t n,
                                                            const float* src, float* dst) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); r < nrows; r += warps) {
    const int64_t i = rows[r];
    const int64_t len = n - 1 - i, base = n * i - i * (i + 1) / 2;
    if (len <= 0) continue;
    const int64_t head = min(len, (4 - (base & 3)) & 3);
    if (lane < head) dst[base + lane] = __ldcs(src + base + lane);
    const int64_t nv = (len - head) >> 2;
    const float4* s4 = reinterpret_cast<const float4*>(src + base + head);
    float4* d4 = reinterpret_cast<float4*>(dst + base + head);
    int64_t k = lane;
    for (; k + 96 < nv; k += 128) {
      const float4 a = __ldcs(s4 + k), b = __ldcs(s4 + k + 32), c = __ldcs(s4 + k + 64), d = __ldcs(s4 + k + 96);
      d4[k] = a;
      d4[k + 32] = b;
      d4[k + 64] = c;
      d4[k + 96] = d;
    }
    for (; k < nv; k += 32) d4[k] = __ldcs(s4 + k);
    const int64_t t0 = head + 4 * nv;
    if (t0 + lane < len) dst[base + t0 + lane] = __ldcs(src + base + t0 + lane);
  }
}
// Default band of the streamed triangle: 256 Mi floats (1 GiB per device
// slot, two slots on the device and two in pinned host memory).
constexpr int64_t kDefaultBandFloats = (int64_t)1 << 28;

// A streamed TRI call: rows leave in bands of at most `band` floats, handed
// to `sink` on the host in row order.
struct RowStream {
  int64_t band;
  int32_t align;  // preferred band boundary (rows), the pair kernel's tile rows
  gbr_band_sink sink;
  void* user;
};

int allpairs_impl(gbr_handle* h, const void* ref_xyz, const void* tgt_xyz, int dtype, int64_t n_ref,
                  int64_t n_tgt, int32_t n_atom, const double* ref_mass, const double* tgt_mass, int mode,
                  int out_kind, int precision, float* out, int64_t row_begin, int64_t row_end,
                  const RowStream* rs, bool redo = false);
}

extern "C" {

int64_t gbr_row_bands(int64_t n_frame, int64_t band_floats, int32_t row_align, int64_t* cuts, int64_t max_cuts) {
  if (n_frame < 0 || band_floats < 1 || row_align < 1 || !cuts || max_cuts < 2) return -1;
  auto before = [&](int64_t r) { return r * n_frame - r * (r + 1) / 2; };  // TRI elements of rows [0, r)
  int64_t nb = 0;
  cuts[0] = 0;
  int64_t r = 0;
  while (r < n_frame) {
    const int64_t start = r;
    // whole groups of rows ending at multiples of row_align
    while (r < n_frame) {
      const int64_t g = std::min(n_frame, (r / row_align + 1) * row_align);
      if (before(g) - before(start) > band_floats) break;
      r = g;
    }
    if (r == start) {  // not even the first group fits: single rows
      while (r < n_frame && before(r + 1) - before(start) <= band_floats) ++r;
      if (r == start) return -1;  // one row alone exceeds the band
    }
    if (nb + 2 > max_cuts) return -1;
    cuts[++nb] = r;
  }
  if (nb == 0) cuts[++nb] = n_frame;
  return nb;
}

gbr_handle* gbr_create(int device) {
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  gbr_handle* h = new gbr_handle();
  h->device = device;
  if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return nullptr;
  }
  h->stream = h->own_stream;
  for (auto& e : h->ev) cudaEventCreate(&e);
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device);
  h->tc_ok = tc_supported(device);
  return h;
}

void gbr_destroy(gbr_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->ws) cudaFree(h->ws);
  if (h->ostage) cudaFree(h->ostage);
  h->release_batch();
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
}

int gbr_set_stream(gbr_handle* h, void* stream) {
  if (!h) return GBR_ERR_ARG;
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return GBR_OK;
}

const char* gbr_last_error(const gbr_handle* h) { return h ? h->err.c_str() : "null handle"; }

int gbr_get_stats(const gbr_handle* h, gbr_stats* out) {
  if (!h || !out) return GBR_ERR_ARG;
  *out = h->stats;
  return GBR_OK;
}

int gbr_set_option(gbr_handle* h, int key, double value) {
  if (!h) return GBR_ERR_ARG;
  switch (key) {
    case GBR_OPT_TAU:
      if (!(value >= 0.0)) return h->fail(GBR_ERR_ARG, "tau must be >= 0");
      h->tau = value;
      return GBR_OK;
    case GBR_OPT_MAX_REFS:
      if (value < 1 || value > kMaxRefs) return h->fail(GBR_ERR_ARG, "max_refs must be in [1, %d]", kMaxRefs);
      h->max_refs = (int)value;
      return GBR_OK;
    case GBR_OPT_TOL:
      if (!(value > 0.0)) return h->fail(GBR_ERR_ARG, "tol must be > 0");
      h->tol = value;
      return GBR_OK;
    case GBR_OPT_TIMING:
      h->timing = value != 0.0;
      return GBR_OK;
    case GBR_OPT_TC_PIPELINE:
      if (!(value == -1.0 || value == 0.0 || value == 1.0 || value == 2.0 || value == 3.0 || value == 4.0))
        return h->fail(GBR_ERR_ARG, "tc pipeline must be -1 (automatic), 0, 1, 2, 3 or 4");
      h->tc_variant = (int)value;
      return GBR_OK;
    case GBR_OPT_HOST_OUT:
      if (value != 0.0 && value != 1.0) return h->fail(GBR_ERR_ARG, "host output mode must be 0 or 1");
      h->host_out_direct = value != 0.0;
      return GBR_OK;
    case GBR_OPT_BAND_FLOATS:
      if (!(value >= 0.0 && value <= 9.0e18)) return h->fail(GBR_ERR_ARG, "band size must be >= 0");
      h->band_floats = (int64_t)value;
      return GBR_OK;
    case GBR_OPT_INPUT_OVERLAP:
      if (value != 0.0 && value != 1.0) return h->fail(GBR_ERR_ARG, "input overlap must be 0 or 1");
      h->input_overlap = value != 0.0;
      return GBR_OK;
  }
  return h->fail(GBR_ERR_ARG, "unknown option %d", key);
}

int64_t gbr_output_count(int64_t n_ref, int64_t n_tgt, int out_kind, int64_t row_begin, int64_t row_end) {
  if (out_kind == GBR_TRI) {
    if (row_end < 0 || row_end > n_ref) row_end = n_ref;
    if (row_begin < 0) row_begin = 0;
    if (row_end <= row_begin) return 0;
    auto cnt = [&](int64_t i) { return i * n_ref - (i * (i + 1)) / 2; };
    return cnt(row_end) - cnt(row_begin);
  }
  if (row_end < 0 || row_end > n_tgt) row_end = n_tgt;
  if (row_begin < 0) row_begin = 0;
  if (row_end <= row_begin) return 0;
  return (row_end - row_begin) * n_ref;
}

int gbr_allpairs(gbr_handle* h, const void* ref_xyz, const void* tgt_xyz, int dtype, int64_t n_ref,
                 int64_t n_tgt, int32_t n_atom, const double* ref_mass, const double* tgt_mass, int mode,
                 int out_kind, int precision, float* out, int64_t row_begin, int64_t row_end) {
  if (!h) return GBR_ERR_ARG;
  if (!out) return h->fail(GBR_ERR_ARG, "out is NULL");
  return allpairs_impl(h, ref_xyz, tgt_xyz, dtype, n_ref, n_tgt, n_atom, ref_mass, tgt_mass, mode, out_kind,
                       precision, out, row_begin, row_end, nullptr);
}

int gbr_allpairs_stream(gbr_handle* h, const void* xyz, int dtype, int64_t n_frame, int32_t n_atom,
                        const double* mass, int mode, int precision, int64_t band_floats, gbr_band_sink sink,
                        void* user) {
  if (!h) return GBR_ERR_ARG;
  if (!sink) return h->fail(GBR_ERR_ARG, "stream: sink is NULL");
  if (mode == GBR_DME) return h->fail(GBR_ERR_UNSUPPORTED, "stream: dme is not streamed (use row ranges)");
  RowStream rs{band_floats > 0 ? band_floats : kDefaultBandFloats, 1, sink, user};
  return allpairs_impl(h, xyz, nullptr, dtype, n_frame, n_frame, n_atom, mass, mass, mode, GBR_TRI, precision,
                       nullptr, 0, -1, &rs);
}

}  // extern "C"

namespace {
int allpairs_impl(gbr_handle* h, const void* ref_xyz, const void* tgt_xyz, int dtype, int64_t n_ref,
                  int64_t n_tgt, int32_t n_atom, const double* ref_mass, const double* tgt_mass, int mode,
                  int out_kind, int precision, float* out, int64_t row_begin, int64_t row_end,
                  const RowStream* rs, bool redo) {
  if (!h) return GBR_ERR_ARG;
  h->err.clear();
  h->stats = gbr_stats{};
  const auto t_start = std::chrono::steady_clock::now();
  if (!ref_xyz) return h->fail(GBR_ERR_ARG, "ref_xyz is NULL");
  if (!out && !rs) return h->fail(GBR_ERR_ARG, "out is NULL");
  if (dtype != GBR_F32 && dtype != GBR_F64) return h->fail(GBR_ERR_ARG, "dtype must be GBR_F32 or GBR_F64");
  if (mode != GBR_FIT && mode != GBR_NOFIT && mode != GBR_DME)
    return h->fail(GBR_ERR_ARG, "mode must be GBR_FIT, GBR_NOFIT or GBR_DME");
  if (out_kind != GBR_TRI && out_kind != GBR_FULL) return h->fail(GBR_ERR_ARG, "out_kind must be TRI or FULL");
  if (precision < GBR_PREC_FP32 || precision > GBR_PREC_FP64) return h->fail(GBR_ERR_ARG, "bad precision");
  if (n_atom < 1) return h->fail(GBR_ERR_ARG, "n_atom must be >= 1 (no atoms selected)");
  if (n_ref < 0 || n_tgt < 0) return h->fail(GBR_ERR_ARG, "negative frame count");
  if (int rc = h->check_local({ref_xyz, tgt_xyz, out}, "allpairs")) return rc;
  if (tgt_xyz == nullptr || tgt_xyz == ref_xyz) {
    tgt_xyz = nullptr;
    n_tgt = n_ref;
  }
  if (out_kind == GBR_TRI && tgt_xyz != nullptr)
    return h->fail(GBR_ERR_ARG, "GBR_TRI needs one frame set (tgt_xyz NULL)");
  if (n_ref > INT32_MAX || n_tgt > INT32_MAX) return h->fail(GBR_ERR_ARG, "frame count exceeds 2^31-1");
  const int64_t n_rows = (out_kind == GBR_TRI) ? n_ref : n_tgt;
  if (row_end < 0 || row_end > n_rows) row_end = n_rows;
  if (row_begin < 0 || row_begin > row_end) return h->fail(GBR_ERR_ARG, "bad row range [%lld, %lld)",
                                                         (long long)row_begin, (long long)row_end);
  const int64_t n_out = gbr_output_count(n_ref, n_tgt, out_kind, row_begin, row_end);
  if (mode == GBR_DME) {  // no masses, no fit: its own kernels (gbr_dme.cu)
    if (cudaSetDevice(h->device) != cudaSuccess) return h->cuda_fail(cudaGetLastError(), "cudaSetDevice");
    int rc = GBR_OK;
    if (n_out > 0)
      rc = allpairs_dme(h, ref_xyz, tgt_xyz, dtype, n_ref, n_tgt, n_atom, out_kind, precision, out, row_begin,
                        row_end, n_out);
    else
      h->stats.precision = (precision == GBR_PREC_FP64) ? GBR_PREC_FP64 : GBR_PREC_FP32;
    h->stats.ms_total =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    return rc;
  }
  if (precision == GBR_PREC_TC && !h->tc_ok)
    return h->fail(GBR_ERR_UNSUPPORTED, "tensor-core precision needs an sm_103 (GB300) device");
  if (cudaSetDevice(h->device) != cudaSuccess) return h->cuda_fail(cudaGetLastError(), "cudaSetDevice");
  cudaStream_t st = h->stream;

  // Masses: small, read them on the host whatever their memory kind.
  const int N = n_atom;
  const bool nofit = (mode == GBR_NOFIT);
  std::vector<double> w_h, wref_h;
  if (tgt_mass) {
    w_h.resize(N);
    if (!read_host_doubles(w_h.data(), tgt_mass, N)) return h->cuda_fail(cudaGetLastError(), "reading tgt_mass");
    if (ref_mass && tgt_xyz != nullptr) {
      wref_h.resize(N);
      if (!read_host_doubles(wref_h.data(), ref_mass, N)) return h->cuda_fail(cudaGetLastError(), "reading ref_mass");
    }
  }
  double Wsum = 0.0;
  if (tgt_mass) {
    for (double v : w_h) Wsum += v;
  } else {
    Wsum = (double)N;
  }
  if (Wsum < 1e-14) return h->fail(GBR_ERR_ZERO_MASS, "total mass %g is below 1e-14 (divide by zero)", Wsum);
  if (n_out == 0) {
    h->stats.precision = precision;
    return GBR_OK;
  }

  const bool ref_dev = is_device_ptr(ref_xyz);
  const bool tgt_dev = tgt_xyz ? is_device_ptr(tgt_xyz) : ref_dev;
  // Pinned host output: by default the kernels store straight into it through
  // its device alias (Grace-Blackwell's coherent host link carries the
  // contraction's ~60 GB/s of results while it runs), instead of staging the
  // triangle in HBM and copying it back in row bands afterwards.
  const bool out_on_dev = rs ? false : is_device_ptr(out);
  float* out_k = out;
  bool out_direct = false;
  if (!rs && !out_on_dev && h->host_out_direct) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, out) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer) {
      out_k = (float*)at.devicePointer;
      out_direct = true;
    } else {
      cudaGetLastError();
    }
  }
  const bool out_dev = out_on_dev || out_direct;  // kernels can write `out_k` in place
  // The kernels' results go to the host through the link as whole tile rows
  // (pinned host `out`), and `out` is filled by one copy at the end (host
  // `out` the kernels do not write in place); both may change once prep has
  // laid the frames out by reference (below).
  bool rows_to_host = out_direct;
  bool copy_back = !out_dev;
  const size_t esz = (dtype == GBR_F64) ? 8 : 4;
  const int64_t F = (tgt_xyz ? n_ref + n_tgt : n_ref);
  const int64_t tgt0 = tgt_xyz ? n_ref : 0;
  const int Np = (N + 63) / 64 * 64;
  const int Kmax = std::min<int>(h->max_refs, (int)std::max<int64_t>(F, 1));
  const bool need_planes = (precision != GBR_PREC_FP64);
  const bool tc = (precision == GBR_PREC_TC);
  const int64_t total_pairs = n_out;
  // A streamed call: TRI bands of at most rs->band floats, aligned to the
  // pair kernel's tile rows where they can be; two device slots (and two
  // pinned host slots) take turns.
  std::vector<int64_t> scuts;
  int64_t sband = 0;
  if (rs) {
    const int var = (h->tc_variant >= 0) ? h->tc_variant : auto_tc_variant(N);
    const int32_t align = tc ? tc_launch_tile_rows(var) : (need_planes ? 64 : 1);
    scuts.resize((size_t)(n_ref + 2));
    const int64_t nb = gbr_row_bands(n_ref, rs->band, align, scuts.data(), (int64_t)scuts.size());
    if (nb < 1)
      return h->fail(GBR_ERR_ARG, "stream: a band of %lld floats cannot hold one row of %lld frames",
                     (long long)rs->band, (long long)n_ref);
    scuts.resize((size_t)nb + 1);
    for (int64_t b = 0; b < nb; ++b)
      sband = std::max(sband, gbr_output_count(n_ref, n_tgt, GBR_TRI, scuts[b], scuts[b + 1]));
    sband = std::max<int64_t>(sband, 1);
    if (!h->ensure_xfer()) return h->fail(GBR_ERR_CUDA, "stream: cannot create the copy stream");
    if (!h->reserve_pinned(2 * ((size_t)sband + 4) * sizeof(float)))
      return h->fail(GBR_ERR_NOMEM, "stream: cannot allocate %.2f GB of pinned staging", 8.0 * (sband + 4) / 1e9);
  }
  const unsigned long long flag_cap =
      rs ? (unsigned long long)std::min<int64_t>(sband, 1 << 21)
         : (unsigned long long)std::min<int64_t>(total_pairs, 1 << 22);

  OutMap map{};
  map.n_ref = n_ref;
  map.tgt0 = tgt0;
  map.n_tgt = n_tgt;
  map.tri = (out_kind == GBR_TRI);
  map.row_begin = row_begin;
  map.row_end = row_end;
  map.base = (map.tri && row_begin < n_ref - 1) ? tri_index(n_ref, row_begin, row_begin + 1) : 0;
  const int64_t tc_tiles = tc ? tc_max_tiles(map) : 0;

  // ---- workspace layout (sizing pass, then carve) ----
  auto layout = [&](Arena& A, void** p) {
    p[0] = ref_dev ? nullptr : A.take<char>(esz * 3 * (size_t)N * n_ref);
    p[1] = (tgt_xyz && !tgt_dev) ? A.take<char>(esz * 3 * (size_t)N * n_tgt) : nullptr;
    p[2] = A.take<double>(N);        // w
    p[3] = A.take<double>(N);        // wref
    p[4] = A.take<double>(3 * F);    // cen
    p[5] = A.take<int64_t>(1);       // fsel
    p[6] = A.take<float>(1);         // dmax
    p[7] = A.take<float>(F);         // dist
    p[8] = A.take<int>(F);           // assign
    p[9] = A.take<double>((size_t)Kmax * 3 * N);  // refs
    p[10] = A.take<float>((size_t)Kmax * 3 * N);  // swr
    p[11] = A.take<double>(Kmax);                 // Eref
    p[12] = (need_planes && !tc) ? A.take<float>((size_t)F * 3 * Np) : nullptr;  // FP32 plane
    p[13] = A.take<float>(F);                                           // per-frame 1/scale
    p[14] = A.take<float>(F);                                           // nrm
    p[15] = A.take<float>((size_t)F * Kmax * 9);                        // P
    p[16] = A.take<float>((size_t)F * Kmax);                            // trP
    p[17] = A.take<float>((size_t)Kmax * Kmax * kRefPairStride);        // reference-pair table
    p[18] = A.take<int>(F);                                             // frames by reference
    p[19] = A.take<int>(Kmax + 1);                                      // offsets
    p[20] = A.take<int2>(rs ? 2 * flag_cap : flag_cap);                 // flagged (two slots when streamed)
    p[21] = A.take<unsigned long long>(kMaxBands);                      // counts (one per band)
    p[22] = rs ? A.take<float>(2 * (size_t)sband) : out_dev ? nullptr : A.take<float>(n_out);  // out staging
    p[23] = tc ? A.take<__half_raw>((size_t)F * 3 * Np) : nullptr;      // hi
    p[24] = tc ? A.take<__half_raw>((size_t)F * 3 * Np) : nullptr;      // lo
    p[25] = A.take<int>(2);                                             // device error, speculation flags
    p[26] = tc ? A.take<int2>(tc_tiles) : nullptr;                      // tile list
    p[27] = need_planes ? A.take<float>((size_t)Kmax * 3 * Np) : nullptr;  // reference means
    p[28] = need_planes ? A.take<float>((size_t)Kmax * 64 * 3 * Np) : nullptr;  // chunk sums
    p[29] = A.take<double>(N);                                                 // sqrt(w)
    p[30] = A.take<float>(N);                                                  // sqrt(w), FP32
    p[31] = need_planes ? A.take<char>(prep_scratch_bytes(F, N, Kmax)) : nullptr;  // prep tables
  };
  void* P[32];
  Arena sizing;
  layout(sizing, P);
  if (!h->reserve(sizing.off + 256))
    return h->fail(GBR_ERR_NOMEM, "cannot allocate %.2f GB of device workspace", (sizing.off + 256) / 1e9);
  Arena A{h->ws, 0};
  layout(A, P);

  int launches = 0;
  cudaError_t e;
  if (h->timing) cudaEventRecord(h->ev[0], st);
  // ---- stage inputs ----
  const void* d_ref = ref_dev ? ref_xyz : P[0];
  const void* d_tgt = tgt_xyz ? (tgt_dev ? tgt_xyz : P[1]) : nullptr;
  // Pinned host inputs of some size travel in chunks on the copy stream; the
  // first prep pass starts on each chunk as it lands.
  const size_t in_bytes = esz * 3 * (size_t)N * (size_t)F;
  const bool chunk_in = need_planes && (!ref_dev || (tgt_xyz && !tgt_dev)) && in_bytes >= (32u << 20) &&
                        h->ensure_xfer();
  // Pageable host input: a copy from it holds the host until it is done, so
  // the chunk copies are issued one by one from prep, each just before the
  // first pass that needs it (the passes of the earlier chunks run meanwhile).
  const bool chunk_lazy =
      chunk_in && !(is_pinned_or_device(ref_xyz) && (!tgt_xyz || is_pinned_or_device(tgt_xyz)));
  int n_chunks = 0;
  int64_t chunk_end[8];
  struct ChunkCopy {
    void* dst;
    const void* src;
    size_t bytes;
  };
  std::vector<ChunkCopy> chunk_copies;
  if (chunk_in) {
    auto plan_chunks = [&](const void* src, void* dst, int64_t set0, int64_t nf, bool dev, int parts) {
      for (int c = 0; c < parts; ++c) {
        const int64_t a = nf * c / parts, b = nf * (c + 1) / parts;
        if (b <= a) continue;
        const size_t o = esz * 3 * (size_t)N * a;
        chunk_copies.push_back({dev ? nullptr : (char*)dst + o, (const char*)src + o, esz * 3 * (size_t)N * (b - a)});
        chunk_end[n_chunks++] = set0 + b;
      }
    };
    plan_chunks(ref_xyz, P[0], 0, n_ref, ref_dev, tgt_xyz ? 4 : 8);
    if (tgt_xyz) plan_chunks(tgt_xyz, P[1], n_ref, n_tgt, tgt_dev, 4);
  } else {
    if (!ref_dev) cudaMemcpyAsync(P[0], ref_xyz, esz * 3 * (size_t)N * n_ref, cudaMemcpyDefault, st);
    if (tgt_xyz && !tgt_dev) cudaMemcpyAsync(P[1], tgt_xyz, esz * 3 * (size_t)N * n_tgt, cudaMemcpyDefault, st);
  }
  // The small copies (weights, staged tile list) go on the caller's stream
  // before the chunk copies are queued (behind them they would wait for the
  // whole input). With chunked input they leave from a tail of the handle's
  // pinned staging, past the part a single contraction launch stages its
  // tile list in, so that queueing them does not hold the host (a pageable
  // copy returns only once it is done). The staging is free: every call
  // has synchronised before it returns.
  const size_t pin_tail = ((sizeof(int2) * (size_t)std::max<int64_t>(tc_tiles, 1)) + 15) & ~size_t(15);
  const size_t pin_w = ((sizeof(double) * (size_t)N) + 15) & ~size_t(15);
  char* pin = (chunk_in && !rs && h->reserve_pinned(pin_tail + 2 * pin_w + sizeof(int2) * (size_t)tc_tiles))
                  ? (char*)h->pinned + pin_tail
                  : nullptr;
  auto put = [&](void* dst, const void* src, size_t bytes, size_t at) {
    if (pin) {
      std::memcpy(pin + at, src, bytes);
      src = pin + at;
    }
    cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
  };
  double* d_w = tgt_mass ? (double*)P[2] : nullptr;
  double* d_wref = nullptr;
  if (tgt_mass) {
    put(d_w, w_h.data(), sizeof(double) * N, 0);
    if (!wref_h.empty()) {
      d_wref = (double*)P[3];
      put(d_wref, wref_h.data(), sizeof(double) * N, pin_w);
    }
  }
  // Chunked input of one frame set, triangle into device (or mapped host)
  // memory: the contraction also runs speculatively, stage by stage.  The
  // tiles are grouped by the first chunk that completes the frames they read
  // (grouped order kept within a stage); when prep has built the operands
  // through a chunk, the tiles ready by then are launched behind it.
  const int tc_variant = (h->tc_variant >= 0) ? h->tc_variant : auto_tc_variant(N);
  // The last call of this shape needed several references: no one-reference
  // speculation (it would be thrown away).
  const bool multi_hint = h->last_multi && h->last_F == F && h->last_N == N;
  bool overlap = h->input_overlap && n_chunks > 0 && tc && map.tri && !tgt_xyz && out_dev && !multi_hint;
  int64_t stage_off[9] = {};
  if (overlap) {
    // Grouped by stage straight into the pinned staging when there is one.
    std::vector<int2>& sorted = h->tile_sorted;
    if (!pin) sorted.resize((size_t)std::max<int64_t>(tc_tiles, 1));
    int2* dst = pin ? (int2*)(pin + 2 * pin_w) : sorted.data();
    const int64_t nt = build_tiles_staged(tc_tile_grid(map, tc_variant), chunk_end, n_chunks, F, dst, tc_tiles,
                                          stage_off, h->tile_scratch);
    if (nt < 0)
      overlap = false;
    else if (nt > 0)
      cudaMemcpyAsync(P[26], dst, sizeof(int2) * nt, cudaMemcpyHostToDevice, st);
  }
  // Issues the chunk copies up to chunk c (those not issued yet) on the copy
  // stream, each followed by its event.
  int chunks_issued = 0;
  const std::function<void(int)> chunk_copy = [&](int c) {
    for (; chunks_issued <= c && chunks_issued < n_chunks; ++chunks_issued) {
      const int k = chunks_issued;
      if (k == 0) {
        cudaEventRecord(h->xev[h->kXev - 1], st);  // the copies follow earlier work on the caller's stream
        cudaStreamWaitEvent(h->xfer, h->xev[h->kXev - 1], 0);
      }
      const ChunkCopy& cc = chunk_copies[k];
      if (cc.dst) cudaMemcpyAsync(cc.dst, cc.src, cc.bytes, cudaMemcpyHostToDevice, h->xfer);
      cudaEventRecord(h->xev[k], h->xfer);
    }
  };
  if (chunk_in && !chunk_lazy) chunk_copy(n_chunks - 1);  // pinned: queued at once
  cudaMemsetAsync(P[21], 0, sizeof(unsigned long long) * kMaxBands, st);
  cudaMemsetAsync(P[25], 0, 2 * sizeof(int), st);

  map.out = out_dev ? out_k : (float*)P[22];

  PrepArgs pa{};
  pa.dtype_f64 = (dtype == GBR_F64);
  pa.ref = d_ref;
  pa.tgt = d_tgt;
  pa.n_ref = n_ref;
  pa.F = F;
  pa.N = N;
  pa.Np = Np;
  pa.nofit = nofit;
  pa.cmass_tgt = d_w;
  pa.cmass_ref = d_wref ? d_wref : d_w;
  pa.w = d_w;
  pa.Wsum = Wsum;
  pa.tau = h->tau;
  pa.max_refs = Kmax;
  pa.cen = (double*)P[4];
  pa.fsel = (int64_t*)P[5];
  pa.dmax = (float*)P[6];
  pa.dist = (float*)P[7];
  pa.assign = (int*)P[8];
  pa.refs = (double*)P[9];
  pa.swr = (float*)P[10];
  pa.Eref = (double*)P[11];
  pa.rot = nullptr;
  pa.plane = (float*)P[12];
  pa.order = (int*)P[18];
  pa.offsets = (int*)P[19];
  pa.mean = (float*)P[27];
  pa.partial = (float*)P[28];
  pa.sqw = (double*)P[29];
  pa.sqwf = (float*)P[30];
  pa.scratch = P[31];
  // With several references, a whole triangle is computed over frames laid
  // out grouped by reference (tiles then share their references, whose terms
  // the tensor-core epilogue stages per tile); outputs map back to frames.
  pa.sort_frames = (!rs && map.tri && row_begin == 0 && row_end == n_ref) ? 1 : 0;
  pa.n_chunks = n_chunks;
  // Whole input on the device and results written in place: the
  // reference-count decision stays on the device (no host round trip inside
  // prep).  A call that turns out to need several references runs again
  // (redo), from the state its first scan left in the workspace.
  pa.defer_multi = (!redo && !multi_hint && n_chunks == 0 && !rs && out_dev && Kmax > 1) ? (int*)P[25] + 1 : nullptr;
  pa.resume_scan = redo ? 1 : 0;
  for (int c = 0; c < n_chunks; ++c) {
    pa.chunk_end[c] = chunk_end[c];
    pa.chunk_ev[c] = h->xev[c];
  }
  pa.chunk_copy = chunk_lazy ? &chunk_copy : nullptr;

  ExactLaunch ex{};
  ex.dtype_f64 = pa.dtype_f64;
  ex.ref = d_ref;
  ex.tgt = d_tgt;
  ex.n_ref = n_ref;
  ex.N = N;
  ex.cen = pa.cen;
  ex.w = d_w;
  ex.Wsum = Wsum;
  ex.nofit = nofit;
  ex.tgt0 = tgt0;
  ex.map = map;

  int K = 1;
  unsigned long long nflag = 0;
  // ---- streamed bands: compute band b into device slot b & 1 while band
  // b - 1 is copied to pinned host memory and band b - 2 is handed to the
  // sink on the host ----
  using BandCompute = std::function<cudaError_t(const OutMap&, const FlagList&, int64_t)>;
  auto run_stream = [&](const BandCompute& compute) -> int {
    const int nbands = (int)scuts.size() - 1;
    float* dslot[2] = {(float*)P[22], (float*)P[22] + sband};
    float* hslot[2] = {(float*)h->pinned, (float*)h->pinned + (sband + 4)};
    unsigned long long* counts = (unsigned long long*)P[21];
    cudaEvent_t* comp = &h->xev[14];
    cudaEvent_t* copied = &h->xev[16];
    std::vector<int64_t> bcnt(nbands);
    auto drain = [&]() {
      cudaStreamSynchronize(h->xfer);
      cudaStreamSynchronize(st);
    };
    auto deliver = [&](int b) -> int {
      const int sl = b & 1;
      const cudaError_t e2 = cudaEventSynchronize(copied[sl]);
      if (e2 != cudaSuccess) return h->cuda_fail(e2, "streamed band");
      unsigned long long c = 0;
      std::memcpy(&c, hslot[sl] + sband, sizeof c);
      nflag += c;
      if (rs->sink(rs->user, scuts[b], scuts[b + 1], hslot[sl], bcnt[b]) != 0)
        return h->fail(GBR_ERR_IO, "stream: the sink stopped the call at rows [%lld, %lld)", (long long)scuts[b],
                       (long long)scuts[b + 1]);
      return GBR_OK;
    };
    for (int b = 0; b < nbands; ++b) {
      const int sl = b & 1;
      const int64_t rb = scuts[b], re = scuts[b + 1];
      bcnt[b] = gbr_output_count(n_ref, n_tgt, GBR_TRI, rb, re);
      OutMap mb = map;
      mb.row_begin = rb;
      mb.row_end = re;
      mb.base = (rb < n_ref - 1) ? tri_index(n_ref, rb, rb + 1) : 0;
      mb.out = dslot[sl];
      mb.perm = nullptr;
      if (b >= 2) cudaStreamWaitEvent(st, copied[sl], 0);  // device slot free once band b - 2 left it
      cudaMemsetAsync(counts + sl, 0, sizeof(unsigned long long), st);
      if (bcnt[b] > 0) {
        const FlagList fb{(int2*)P[20] + (size_t)sl * flag_cap, counts + sl, flag_cap};
        const cudaError_t e2 = compute(mb, fb, bcnt[b]);
        if (e2 != cudaSuccess) {
          drain();
          return h->cuda_fail(e2, "streamed band kernel");
        }
      }
      cudaEventRecord(comp[sl], st);
      if (b >= 2) {  // host slot free once the sink has taken band b - 2
        const int rc = deliver(b - 2);
        if (rc != GBR_OK) {
          drain();
          return rc;
        }
      }
      cudaStreamWaitEvent(h->xfer, comp[sl], 0);
      if (bcnt[b] > 0)
        cudaMemcpyAsync(hslot[sl], dslot[sl], sizeof(float) * bcnt[b], cudaMemcpyDeviceToHost, h->xfer);
      cudaMemcpyAsync(hslot[sl] + sband, counts + sl, sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->xfer);
      cudaEventRecord(copied[sl], h->xfer);
    }
    if (h->timing) {
      cudaEventRecord(h->ev[2], st);
      cudaEventRecord(h->ev[3], st);
    }
    for (int b = std::max(0, nbands - 2); b < nbands; ++b) {
      const int rc = deliver(b);
      if (rc != GBR_OK) {
        drain();
        return rc;
      }
    }
    int derr = 0;
    cudaMemcpyAsync(&derr, P[25], sizeof derr, cudaMemcpyDeviceToHost, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (e2 != cudaSuccess) return h->cuda_fail(e2, "streamed call");
    if (derr != 0) return h->fail(GBR_ERR_DEVICE, "pair kernel reported device error %d (bounded wait expired)", derr);
    return GBR_OK;
  };
  if (!need_planes) {
    // FP64 checking mode: centres only, then every pair directly.
    PrepArgs c = pa;
    c.centroid_only = 1;
    PrepOut po;
    if ((e = run_prep(c, po, st)) != cudaSuccess) return h->cuda_fail(e, "prep");
    launches += po.launches;
    if (h->timing) cudaEventRecord(h->ev[1], st);
    if (rs) {
      const int rc = run_stream([&](const OutMap& mb, const FlagList&, int64_t cnt) {
        ExactLaunch eb = ex;
        eb.map = mb;
        eb.list = nullptr;
        eb.count = cnt;
        ++launches;
        return run_exact(eb, st);
      });
      if (rc != GBR_OK) return rc;
    } else {
      if (h->timing) cudaEventRecord(h->ev[2], st);
      ex.list = nullptr;
      ex.count = n_out;
      if ((e = run_exact(ex, st)) != cudaSuccess) return h->cuda_fail(e, "exact kernel");
      ++launches;
    }
  } else {
    // The operand build, as run_finish does it; while chunked host input
    // lands, prep runs it speculatively for one reference (K = 1, unsorted).
    FinishArgs fa{};
    fa.prep = &pa;
    fa.plane = pa.plane;
    fa.F = F;
    fa.N = N;
    fa.Np = Np;
    fa.K = 1;
    fa.mean = pa.mean;
    fa.assign = pa.assign;
    fa.swr = pa.swr;
    fa.tc = tc;
    fa.hi = P[23];
    fa.lo = P[24];
    fa.inv_scale = (float*)P[13];
    fa.write_plane = !tc;
    fa.nrm = (float*)P[14];
    fa.P = (float*)P[15];
    fa.trP = (float*)P[16];
    fa.refs = pa.refs;
    fa.w = d_w;
    fa.nofit = nofit;
    fa.RP = (float*)P[17];
    pa.RP = fa.RP;
    // Per-frame terms as the pair kernels read them, for K references (sorted:
    // reference-grouped operand positions).
    auto make_terms = [&](int Kt, bool sorted) {
      FrameTerms t{};
      t.assign = sorted ? prep_carve(pa.scratch, F, N, Kmax).assign_pos : pa.assign;
      t.nrm = (float*)P[14];
      t.P = (float*)P[15];
      t.trP = (float*)P[16];
      t.RP = (float*)P[17];
      t.K = Kt;
      t.W = (float)Wsum;
      t.two_over_w = (float)(2.0 / (double)Wsum);
      t.tol = (float)h->tol;
      // FP32 FMA accumulation: 3-sigma random walk of half-ulp roundings (x2
      // margin), ~1.2e-7 sqrt(N) |tr D|.  Tensor memory: the FP16 hi+lo split
      // represents each product to ~2^-22 (taken coherent), and accumulation
      // measured on correlated frames behaves like truncation, about
      // eps/2 per add over 3N/16 adds: ~5.6e-9 N |tr D|, bounded with x2 margin.
      t.gem_s = tc ? 6.0e-7f : 1.2e-7f;
      t.gem_c = tc ? 1.2e-8f * (float)N : 1.2e-7f * std::sqrt((float)N);
      t.epi_coef = 8e-7f;
      t.nofit = nofit;
      return t;
    };
    // One tensor-core launch: over the tiles of map m, or (n_ready > 0) over
    // n_ready tiles already in the tile buffer from tile0 on.
    auto launch_tc = [&](const OutMap& m, const FlagList& f, const FrameTerms& t, int64_t tile0, int64_t n_ready,
                         const int* skip, int2* stage = nullptr, int cap = 0,
                         cudaStream_t on = nullptr) -> cudaError_t {
      TcLaunch L{};
      L.hi = P[23];
      L.lo = P[24];
      L.tile_buf = (int2*)P[26] + tile0;
      L.tile_cap = tc_tiles - tile0;
      L.ready_tiles = n_ready;
      L.F = F;
      L.Np = Np;
      L.N = N;
      L.tgt0 = tgt0;
      L.inv_scale = (const float*)P[13];
      L.terms = t;
      L.map = m;
      L.flags = f;
      L.dev_error = (int*)P[25];
      L.num_sms = h->num_sms;
      L.variant = tc_variant;
      // whole-row stores where the triangle lands in host memory across the
      // link; direct per-pair stores into device memory
      L.row_stores = rows_to_host ? 1 : 0;
      L.skip = skip;
      L.tile_stage = stage;
      L.cluster_cap = cap;
      return run_pairs_tc(L, on ? on : st);
    };
    // Speculative stages (see above): launched from prep through on_built.
    // Each launch exits at once if a chunk check has already seen a frame
    // farther than tau from reference 0; if the final reference count is not
    // one, everything is recomputed below.  The chunk passes run on the
    // handle's prep stream.  The stages that start within the first
    // kStageShare of the tiles go to the caller's stream, each waiting only
    // for its chunk's operands, on all but kStageFreeClusters clusters (the
    // SMs left free keep the next chunks' passes going); the rest of the
    // tiles go in one launch on every SM behind the last chunk's passes, on
    // their stream.  Measured at 10,000 x 2,000 (pinned host in and out):
    // 3.81-3.85 ms per call against 4.19-4.29 ms with the contraction after
    // the last chunk (sweep of 4-45 % of the tiles on 26-70 clusters).
    constexpr double kStageShare = 0.20;
    constexpr int kStageFreeClusters = 10;
    const bool split = overlap && h->ensure_prep_stream();
    cudaStream_t ps = split ? h->prep_stream : st;
    if (split) {
      cudaEventRecord(h->pev[h->kPev - 2], st);
      cudaStreamWaitEvent(ps, h->pev[h->kPev - 2], 0);
    }
    const int64_t n_stage_tiles = overlap ? stage_off[n_chunks] : 0;
    const int64_t stage_budget = (int64_t)(kStageShare * (double)n_stage_tiles);
    int64_t staged_end = 0;  // tiles [0, staged_end) launched in stages
    const FrameTerms terms1 = make_terms(1, false);
    int next_stage = 0;
    bool spec_terms = false;
    FlagList fl_spec{(int2*)P[20], (unsigned long long*)P[21], flag_cap};
    bool rest_launched = false;
    // The tiles no stage took, on every SM, behind the last chunk's passes
    // on their stream (not behind the stages, which may still be running),
    // queued as soon as the last chunk is built: before prep's host-side
    // reference-count check, which the speculation flag covers.
    auto launch_rest = [&]() -> cudaError_t {
      if (rest_launched || !spec_terms || staged_end >= n_stage_tiles) return cudaSuccess;
      rest_launched = true;
      ++launches;
      return launch_tc(map, fl_spec, terms1, staged_end, n_stage_tiles - staged_end, (const int*)P[25] + 1, nullptr,
                       0, ps);
    };
    std::function<cudaError_t(int64_t)> on_built = [&](int64_t built_end) -> cudaError_t {
      int c1 = next_stage;
      while (c1 < n_chunks && chunk_end[c1] <= built_end) ++c1;
      if (c1 == next_stage) return cudaSuccess;
      const int64_t t0 = stage_off[next_stage], t1 = stage_off[c1];
      next_stage = c1;
      if (t1 == t0 || t0 >= stage_budget)  // beyond the budget: the final launch
        return (c1 == n_chunks) ? launch_rest() : cudaSuccess;
      cudaError_t e2;
      if (!spec_terms) {  // reference-pair terms of reference 0, as run_finish computes them
        FinishArgs f1 = fa;
        f1.K = 1;
        f1.built = 1;
        f1.sorted = 0;
        if ((e2 = run_finish(f1, ps)) != cudaSuccess) return e2;
        spec_terms = true;
        ++launches;
        if (h->timing) cudaEventRecord(h->ev[1], ps);
      }
      if (split) {
        cudaEventRecord(h->pev[c1 - 1], ps);
        cudaStreamWaitEvent(st, h->pev[c1 - 1], 0);
      }
      e2 = launch_tc(map, fl_spec, terms1, t0, t1 - t0, (const int*)P[25] + 1, nullptr,
                     split ? -kStageFreeClusters : 0);
      staged_end = t1;
      ++launches;
      if (e2 == cudaSuccess && c1 == n_chunks) e2 = launch_rest();
      return e2;
    };
    if (overlap) {
      pa.on_built = &on_built;
      pa.spec_fail = (int*)P[25] + 1;
    }
    if (n_chunks > 0 && !multi_hint) pa.spec_build = &fa;
    PrepOut po;
    const cudaError_t ep = run_prep(pa, po, ps);
    if (chunk_in) chunk_copy(n_chunks - 1);  // every chunk issued, whatever prep did
    if ((e = ep) != cudaSuccess) return h->cuda_fail(e, "prep");
    if (overlap && po.built && (e = launch_rest()) != cudaSuccess) return h->cuda_fail(e, "pair kernel launch");
    if (split) {  // everything after prep (and the remainder) follows it on the caller's stream
      cudaEventRecord(h->pev[h->kPev - 1], ps);
      cudaStreamWaitEvent(st, h->pev[h->kPev - 1], 0);
    }
    launches += po.launches;
    K = po.K;
    // Every stage was launched by the time the last chunk was built; the
    // speculation stands when prep kept its one-reference build.
    const bool spec_done = overlap && po.built && spec_terms;
    if (overlap && !spec_done)
      cudaMemsetAsync(P[21], 0, sizeof(unsigned long long) * kMaxBands, st);  // discard speculative flags
    if (out_direct && po.sorted) {
      // A triangle over reference-sorted positions scatters its values over
      // the whole output, which the host link serves at a fraction of its
      // rate (10x slower at 50,000 x 500 with 20 references): it is computed
      // into device memory and copied back whole.
      if (!h->reserve_ostage(sizeof(float) * (size_t)n_out))
        return h->fail(GBR_ERR_NOMEM, "cannot allocate %.2f GB of device memory for the result",
                       4.0 * n_out / 1e9);
      map.out = (float*)h->ostage;
      ex.map.out = map.out;
      rows_to_host = false;
      copy_back = true;
    }
    OutMap pmap = map;  // the pair kernels' view: sorted positions when po.sorted
    if (po.sorted) pmap.perm = pa.order;
    const FrameTerms terms = make_terms(K, po.sorted != 0);
    fa.sorted = po.sorted;
    fa.K = K;
    fa.built = po.built;
    fa.skip = po.deferred ? pa.defer_multi : nullptr;
    fa.self_terms = po.self_terms;
    if (!spec_done) {
      if ((e = run_finish(fa, st)) != cudaSuccess) return h->cuda_fail(e, "finish");
      // k_build (+ k_pref with several references), k_ref_terms (unless prep wrote the one reference's)
      launches += po.built ? 1 : (K > 1 ? 3 : (po.self_terms ? 1 : 2));
    }
    // One launch of the pair kernel over the rows of map m.
    auto launch_pairs = [&](const OutMap& m, const FlagList& f, int2* stage = nullptr, int cap = 0) -> cudaError_t {
      if (tc) return launch_tc(m, f, terms, 0, 0, fa.skip, stage, cap);
      PairLaunch L{};
      L.skip = fa.skip;
      L.plane = pa.plane;
      L.Np = Np;
      L.N = N;
      L.tgt0 = tgt0;
      L.terms = terms;
      L.map = m;
      L.flags = f;
      L.tiles = make_tiles(m, 64, 64);
      return run_pairs_fp32(L, st);
    };
    if (h->timing && !spec_done) cudaEventRecord(h->ev[1], st);
    // A large result bound for pinned host memory leaves in row bands: each
    // band's pairs are computed and checked (FP64 re-check of its flagged
    // pairs, list length read on the device), then copied on the copy stream
    // while the next band computes.
    // A reference-sorted triangle bound for pinned host memory (computed into
    // device memory, see above) leaves the same way: a band of sorted rows
    // completes the caller's rows of its frames (every pair sits in the tile
    // row of its smaller position), which a copy kernel then writes whole.
    const bool sorted_to_host = out_direct && po.sorted && ((uintptr_t)out_k & 15) == 0;
    const bool band_out = !rs &&
                          ((!out_dev && !po.sorted && (size_t)n_out * sizeof(float) >= (32u << 20)) ||
                           sorted_to_host) &&
                          h->ensure_xfer();
    int derr = 0;
    if (rs) {
      // each band: its pairs, then the FP64 re-check of its flagged pairs
      // (list length read on the device; an overflowing list recomputes the band)
      const int rc = run_stream([&](const OutMap& mb, const FlagList& fb, int64_t cnt) -> cudaError_t {
        cudaError_t e2 = launch_pairs(mb, fb);
        if (e2 != cudaSuccess) return e2;
        ExactLaunch exb = ex;
        exb.map = mb;
        exb.list = fb.pairs;
        exb.count = (int64_t)fb.cap;
        exb.dev_count = fb.count;
        exb.overflow_all = 1;
        exb.map_pairs = cnt;
        launches += 2;
        return run_exact(exb, st);
      });
      if (rc != GBR_OK) return rc;
    } else if (!band_out) {
      FlagList fl{(int2*)P[20], (unsigned long long*)P[21], flag_cap};
      if (!spec_done) {
        // One contraction launch in this call: its tile list goes through the
        // handle's pinned staging, so the host queues the launch behind the
        // prep passes at once instead of waiting for them (the staging is
        // free: every call has synchronised before it returns).
        int2* stage = (tc && h->reserve_pinned(sizeof(int2) * (size_t)std::max<int64_t>(tc_tiles, 1)))
                          ? (int2*)h->pinned
                          : nullptr;
        if ((e = launch_pairs(pmap, fl, stage)) != cudaSuccess) return h->cuda_fail(e, "pair kernel launch");
        ++launches;
      }
      if (h->timing) cudaEventRecord(h->ev[2], st);
      int dflags[2] = {0, 0};  // device error, several references needed (deferred decision)
      cudaMemcpyAsync(&nflag, P[21], sizeof nflag, cudaMemcpyDeviceToHost, st);
      cudaMemcpyAsync(dflags, P[25], sizeof dflags, cudaMemcpyDeviceToHost, st);
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return h->cuda_fail(e, "pair kernel");
      derr = dflags[0];
      if (derr != 0)
        return h->fail(GBR_ERR_DEVICE, "pair kernel reported device error %d (bounded wait expired)", derr);
      if (po.deferred && dflags[1] != 0)  // every pass after the first scan did nothing
        return allpairs_impl(h, ref_xyz, tgt_xyz, dtype, n_ref, n_tgt, n_atom, ref_mass, tgt_mass, mode, out_kind,
                             precision, out, row_begin, row_end, rs, true);
      if (nflag > 0) {
        if (nflag <= flag_cap) {
          ex.list = (const int2*)P[20];
          ex.count = (int64_t)nflag;
        } else {
          ex.list = nullptr;  // too many: recompute everything exactly
          ex.count = n_out;
        }
        if ((e = run_exact(ex, st)) != cudaSuccess) return h->cuda_fail(e, "fix-up kernel");
        ++launches;
      }
      if (h->timing) cudaEventRecord(h->ev[3], st);
      if (copy_back) cudaMemcpyAsync(out, map.out, sizeof(float) * n_out, cudaMemcpyDefault, st);
    } else {
      // Band boundaries: equal pair counts, aligned to the kernel's tile rows.
      // A reference-sorted triangle is cut into equal numbers of rows instead:
      // each band's copy then moves about the same bytes (the caller's rows
      // of its frames), and the last band, the copy nothing overlaps, is no
      // larger than the others.
      const int64_t align = tc ? tc_launch_tile_rows(tc_variant) : 64;
      const int nb = kMaxBands - 2;
      std::vector<int64_t> cut{row_begin};
      const int64_t total = sorted_to_host ? row_end - row_begin : n_out;
      int64_t acc = 0;
      for (int64_t r = row_begin; r < row_end && (int)cut.size() < nb; ++r) {
        acc += sorted_to_host ? 1 : map.tri ? (n_ref - 1 - r) : n_ref;
        const int64_t r1 = r + 1;
        if (acc * nb >= total * (int64_t)cut.size() && (r1 - row_begin) % align == 0 && r1 < row_end) cut.push_back(r1);
      }
      cut.push_back(row_end);
      const int nbands = (int)cut.size() - 1;
      const unsigned long long capb = flag_cap / (unsigned long long)nbands;
      unsigned long long* counts = (unsigned long long*)P[21];
      // Band b's copy is issued after band b + 1 is queued: a copy into
      // pageable host memory holds the host until it is done, and the GPU
      // then has the next band to compute meanwhile.
      std::function<cudaError_t()> pending_copy;
      auto flush_copy = [&]() -> cudaError_t {
        cudaError_t ec = cudaSuccess;
        if (pending_copy) ec = pending_copy();
        pending_copy = nullptr;
        return ec;
      };
      for (int b = 0; b < nbands; ++b) {
        const int64_t rb = cut[b], re = cut[b + 1];
        const int64_t cnt = gbr_output_count(n_ref, n_tgt, out_kind, rb, re);
        if (cnt <= 0) continue;
        OutMap mb = sorted_to_host ? pmap : map;
        mb.row_begin = rb;
        mb.row_end = re;
        int64_t off = 0;
        if (sorted_to_host) {
          // rows of sorted positions; the stores go through the permutation to
          // the caller's positions in the whole device-side triangle
        } else if (map.tri) {
          mb.base = (rb < n_ref - 1) ? tri_index(n_ref, rb, rb + 1) : 0;
          off = mb.base - map.base;
        } else {
          off = (rb - row_begin) * n_ref;
        }
        mb.out = map.out + off;
        FlagList fb{(int2*)P[20] + (size_t)b * capb, counts + b, capb};
        if ((e = launch_pairs(mb, fb, nullptr, sorted_to_host ? -kCopyFreeClusters : 0)) != cudaSuccess)
          return h->cuda_fail(e, "pair kernel launch");
        ExactLaunch exb = ex;
        if (!sorted_to_host) exb.map = mb;  // flagged pairs are frames: the caller's map places them
        exb.list = fb.pairs;
        exb.count = (int64_t)capb;
        exb.dev_count = counts + b;
        if ((e = run_exact(exb, st)) != cudaSuccess) return h->cuda_fail(e, "fix-up kernel");
        launches += 2;
        cudaEventRecord(h->xev[8 + b], st);
        if ((e = flush_copy()) != cudaSuccess) return h->cuda_fail(e, "result copy");
        pending_copy = [&, b, rb, re, off, cnt, src = mb.out]() -> cudaError_t {
          cudaStreamWaitEvent(h->xfer, h->xev[8 + b], 0);
          if (sorted_to_host) {
            const cudaError_t ea =
                cudaFuncSetAttribute(k_copy_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, kCopySmem);
            if (ea != cudaSuccess) return ea;
            k_copy_rows<<<kCopyBlocks, kCopyThreads, kCopySmem, h->xfer>>>(pa.order + rb, re - rb, n_ref, map.out,
                                                                          out_k);
            ++launches;
            return cudaGetLastError();
          }
          return cudaMemcpyAsync(out + off, src, sizeof(float) * cnt, cudaMemcpyDeviceToHost, h->xfer);
        };
      }
      if ((e = flush_copy()) != cudaSuccess) return h->cuda_fail(e, "result copy");
      if (h->timing) {
        cudaEventRecord(h->ev[2], st);
        cudaEventRecord(h->ev[3], st);
      }
      std::vector<unsigned long long> cnts(nbands);
      cudaMemcpyAsync(cnts.data(), counts, sizeof(unsigned long long) * nbands, cudaMemcpyDeviceToHost, st);
      cudaMemcpyAsync(&derr, P[25], sizeof derr, cudaMemcpyDeviceToHost, st);
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return h->cuda_fail(e, "pair kernel");
      if (derr != 0) {
        cudaStreamSynchronize(h->xfer);
        return h->fail(GBR_ERR_DEVICE, "pair kernel reported device error %d (bounded wait expired)", derr);
      }
      bool overflow = false;
      for (int b = 0; b < nbands; ++b) {
        nflag += cnts[b];
        overflow |= cnts[b] > capb;
      }
      if (overflow) {
        // a band flagged more pairs than its list holds: recompute everything
        // exactly and send the whole result again
        cudaEventRecord(h->xev[h->kXev - 2], h->xfer);
        cudaStreamWaitEvent(st, h->xev[h->kXev - 2], 0);
        ex.list = nullptr;
        ex.count = n_out;
        if ((e = run_exact(ex, st)) != cudaSuccess) return h->cuda_fail(e, "fix-up kernel");
        ++launches;
        cudaMemcpyAsync(out, map.out, sizeof(float) * n_out, cudaMemcpyDeviceToHost, st);
        nflag = (unsigned long long)n_out;
      }
    }
  }
  if (h->timing && !need_planes) cudaEventRecord(h->ev[3], st);
  if (!rs && !need_planes && copy_back) cudaMemcpyAsync(out, map.out, sizeof(float) * n_out, cudaMemcpyDefault, st);
  if (h->xfer) {  // the copy stream's work belongs to this call
    cudaEventRecord(h->xev[h->kXev - 3], h->xfer);
    cudaStreamWaitEvent(st, h->xev[h->kXev - 3], 0);
  }
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return h->cuda_fail(e, "call");
  h->stats.pairs = n_out;
  h->stats.pairs_fixed = (int64_t)std::min<unsigned long long>(nflag, (unsigned long long)n_out);
  h->stats.n_refs = K;
  h->stats.precision = precision;
  h->stats.kernel_launches = launches;
  if (need_planes && Kmax > 1) {
    h->last_F = F;
    h->last_N = N;
    h->last_multi = (K > 1);
  }
  if (h->timing) {
    float a = 0, b = 0, c = 0;
    cudaEventElapsedTime(&a, h->ev[0], h->ev[1]);
    cudaEventElapsedTime(&b, h->ev[1], h->ev[2]);
    cudaEventElapsedTime(&c, h->ev[2], h->ev[3]);
    h->stats.ms_prep = a;
    h->stats.ms_pairs = b;
    h->stats.ms_fixup = c;
  }
  h->stats.ms_total =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  return GBR_OK;
}

}  // namespace

extern "C" {

int gbr_rmsd_backward(gbr_handle* h, const float* xyz, int64_t n_frame, int32_t n_atom, const double* mass,
                      const float* g, float* grad_xyz, float* rmsd_out) {
  if (!h) return GBR_ERR_ARG;
  h->err.clear();
  h->stats = gbr_stats{};
  const auto t_start = std::chrono::steady_clock::now();
  if (!xyz || !grad_xyz) return h->fail(GBR_ERR_ARG, "backward: xyz and grad_xyz must not be NULL");
  if (n_atom < 1) return h->fail(GBR_ERR_ARG, "n_atom must be >= 1");
  if (n_frame < 0 || n_frame > 60000) return h->fail(GBR_ERR_ARG, "backward supports 0..60000 frames");
  if (int rc = h->check_local({xyz, g, grad_xyz, rmsd_out}, "backward")) return rc;
  if (cudaSetDevice(h->device) != cudaSuccess) return h->cuda_fail(cudaGetLastError(), "cudaSetDevice");
  cudaStream_t st = h->stream;
  const int N = n_atom;
  const int64_t F = n_frame;
  std::vector<double> w_h;
  double Wsum = (double)N;
  if (mass) {
    w_h.resize(N);
    if (cudaMemcpy(w_h.data(), mass, sizeof(double) * N, cudaMemcpyDefault) != cudaSuccess)
      return h->cuda_fail(cudaGetLastError(), "reading mass");
    Wsum = 0.0;
    for (double v : w_h) Wsum += v;
  }
  if (Wsum < 1e-14) return h->fail(GBR_ERR_ZERO_MASS, "total mass %g is below 1e-14 (divide by zero)", Wsum);
  const bool xyz_dev = is_device_ptr(xyz), grad_dev = is_device_ptr(grad_xyz);
  const bool g_dev = g ? is_device_ptr(g) : false;
  const bool r_dev = rmsd_out ? is_device_ptr(rmsd_out) : false;
  const int64_t npairs = F * (F - 1) / 2;
  const int64_t ldB = (3 * F + 3) / 4 * 4;  // 16-byte rows for the GEMM's vector loads
  if (F < 2) {
    if (grad_dev) cudaMemsetAsync(grad_xyz, 0, sizeof(float) * 3 * N * F, st);
    else std::memset(grad_xyz, 0, sizeof(float) * 3 * N * F);
    cudaStreamSynchronize(st);
    return GBR_OK;
  }
  const int Np = (N + 63) / 64 * 64;
  // The pair pass (pair-of-SMs kernel, backward instantiation) and the block
  // contraction both run on the tensor cores.
  if (!h->tc_ok) return h->fail(GBR_ERR_UNSUPPORTED, "backward needs an sm_103 (GB300) device");
  const bool tc = true;
  const int64_t ldS = bwd_gemm_ld(F);
  OutMap map{};
  map.n_ref = F;
  map.n_tgt = F;
  map.tri = 1;
  map.row_begin = 0;
  map.row_end = F;
  const int64_t tc_tiles = tc ? tc_max_tiles(map) : 0;
  auto layout = [&](Arena& A, void** p) {
    p[0] = xyz_dev ? nullptr : A.take<float>((size_t)F * 3 * N);
    p[1] = A.take<double>(N);                       // w
    p[2] = A.take<double>(3 * F);                   // cen
    p[3] = A.take<int64_t>(1);                      // fsel
    p[4] = A.take<float>(1);                        // dmax
    p[5] = A.take<float>(F);                        // dist
    p[6] = A.take<int>(F);                          // assign
    p[7] = A.take<double>(3 * (size_t)N);           // refs (one)
    p[8] = A.take<float>(3 * (size_t)N);            // swr
    p[9] = A.take<double>(1);                       // Eref
    p[10] = A.take<double>(9 * (size_t)F);          // rot
    p[11] = A.take<float>((size_t)F * 3 * Np);      // plane
    p[12] = A.take<float>(F);                       // per-frame 1/scale (unused)
    p[13] = A.take<int>(F);                         // order
    p[14] = A.take<int>(2);                         // offsets
    p[15] = A.take<float>(3 * (size_t)Np);          // mean
    p[16] = A.take<float>(F);                       // nrm
    p[17] = A.take<float>(9 * (size_t)F);           // P
    p[18] = A.take<float>(F);                       // trP
    p[19] = A.take<float>(kRefPairStride);          // reference-pair table
    p[20] = A.take<float>((size_t)3 * F * ldB);     // B [3F][ldB]
    p[21] = A.take<float>(9 * (size_t)F);           // E
    p[22] = A.take<float>(F);                       // C
    p[23] = A.take<float>((size_t)3 * F * Np);      // Z
    p[24] = (g && !g_dev) ? A.take<float>(npairs) : nullptr;
    p[25] = (rmsd_out && !r_dev) ? A.take<float>(npairs) : nullptr;
    p[26] = grad_dev ? nullptr : A.take<float>((size_t)F * 3 * N);
    p[27] = A.take<unsigned long long>(1);          // flag count (unused list)
    p[28] = A.take<float>((size_t)64 * 3 * Np);     // chunk sums
    p[29] = A.take<double>(N);                      // sqrt(w)
    p[30] = A.take<float>(N);                       // sqrt(w), FP32
    p[31] = A.take<char>(prep_scratch_bytes(F, N, 1));  // prep tables
    p[32] = tc ? A.take<__half_raw>((size_t)F * 3 * Np) : nullptr;  // FP16 hi
    p[33] = tc ? A.take<__half_raw>((size_t)F * 3 * Np) : nullptr;  // FP16 lo
    p[34] = tc ? A.take<int2>(tc_tiles) : nullptr;                   // tile list
    p[35] = A.take<int>(1);                                          // device error flag
    p[36] = A.take<__half_raw>((size_t)3 * F * ldS);                 // S = B + B^T, FP16 hi
    p[37] = A.take<__half_raw>((size_t)3 * F * ldS);                 // S, FP16 lo
    p[38] = A.take<__half_raw>((size_t)Np * ldS);                    // plane transposed, FP16 hi
    p[39] = A.take<__half_raw>((size_t)Np * ldS);                    // plane transposed, FP16 lo
    p[40] = A.take<unsigned int>(2);                                 // largest |B|, |plane|
    p[41] = A.take<float>(2);                                        // split scales
    p[42] = A.take<float4>(3 * (size_t)N);                           // per-atom constants, hi + lo
  };
  void* P[43];
  Arena sizing;
  layout(sizing, P);
  if (!h->reserve(sizing.off + 256))
    return h->fail(GBR_ERR_NOMEM, "cannot allocate %.2f GB of device workspace", (sizing.off + 256) / 1e9);
  Arena A{h->ws, 0};
  layout(A, P);
  cudaError_t e;
  const float* d_xyz = xyz_dev ? xyz : (const float*)P[0];
  if (!xyz_dev) cudaMemcpyAsync(P[0], xyz, sizeof(float) * 3 * N * F, cudaMemcpyDefault, st);
  double* d_w = mass ? (double*)P[1] : nullptr;
  if (mass) cudaMemcpyAsync(d_w, w_h.data(), sizeof(double) * N, cudaMemcpyHostToDevice, st);
  const float* d_g = g ? (g_dev ? g : (const float*)P[24]) : nullptr;
  if (g && !g_dev) cudaMemcpyAsync(P[24], g, sizeof(float) * npairs, cudaMemcpyDefault, st);
  float* d_rmsd = rmsd_out ? (r_dev ? rmsd_out : (float*)P[25]) : nullptr;
  float* d_grad = grad_dev ? grad_xyz : (float*)P[26];
  if (h->timing) cudaEventRecord(h->ev[0], st);

  PrepArgs pa{};
  pa.dtype_f64 = 0;
  pa.ref = d_xyz;
  pa.n_ref = F;
  pa.F = F;
  pa.N = N;
  pa.Np = Np;
  pa.cmass_ref = pa.cmass_tgt = pa.w = d_w;
  pa.Wsum = Wsum;
  pa.tau = 1e30;
  pa.max_refs = 1;
  pa.cen = (double*)P[2];
  pa.fsel = (int64_t*)P[3];
  pa.dmax = (float*)P[4];
  pa.dist = (float*)P[5];
  pa.assign = (int*)P[6];
  pa.refs = (double*)P[7];
  pa.swr = (float*)P[8];
  pa.Eref = (double*)P[9];
  pa.rot = (double*)P[10];
  pa.plane = (float*)P[11];
  pa.order = (int*)P[13];
  pa.offsets = (int*)P[14];
  pa.mean = (float*)P[15];
  pa.partial = (float*)P[28];
  pa.sqw = (double*)P[29];
  pa.sqwf = (float*)P[30];
  pa.scratch = P[31];
  pa.RP = (float*)P[19];
  PrepOut po;
  if ((e = run_prep(pa, po, st)) != cudaSuccess) return h->cuda_fail(e, "prep");
  int launches = po.launches;
  FrameTerms terms{};
  terms.assign = pa.assign;
  terms.nrm = (float*)P[16];
  terms.P = (float*)P[17];
  terms.trP = (float*)P[18];
  terms.RP = (float*)P[19];
  terms.K = 1;
  terms.W = (float)Wsum;
  terms.two_over_w = (float)(2.0 / (double)Wsum);
  terms.tol = (float)h->tol;
  terms.gem_s = tc ? 6.0e-7f : 1.2e-7f;
  terms.gem_c = tc ? 1.2e-8f * (float)N : 1.2e-7f * std::sqrt((float)N);
  terms.epi_coef = 8e-7f;
  terms.nofit = 0;
  FinishArgs fa{};
  fa.prep = &pa;
  fa.plane = pa.plane;
  fa.F = F;
  fa.N = N;
  fa.Np = Np;
  fa.K = 1;
  fa.mean = pa.mean;
  fa.assign = pa.assign;
  fa.swr = pa.swr;
  fa.tc = tc;
  fa.hi = P[32];
  fa.lo = P[33];
  fa.write_plane = 1;  // the GEMM reads the plane (with tc: the values hi + lo represent)
  fa.inv_scale = (float*)P[12];
  fa.nrm = (float*)terms.nrm;
  fa.P = (float*)terms.P;
  fa.trP = (float*)terms.trP;
  fa.refs = pa.refs;
  fa.w = d_w;
  fa.nofit = 0;
  fa.RP = (float*)terms.RP;
  fa.self_terms = po.self_terms;
  if ((e = run_finish(fa, st)) != cudaSuccess) return h->cuda_fail(e, "finish");
  launches += po.self_terms ? 1 : 2;
  float* B = (float*)P[20];  // the pair pass writes its upper 3x3 blocks, all that is read of it
  cudaMemsetAsync(P[21], 0, sizeof(float) * 9 * F, st);
  cudaMemsetAsync(P[22], 0, sizeof(float) * F, st);
  cudaMemsetAsync(P[35], 0, sizeof(int), st);
  cudaMemsetAsync(P[40], 0, 2 * sizeof(unsigned int), st);
  if (h->timing) cudaEventRecord(h->ev[1], st);
  PairLaunch L{};
  L.bwd.B = B;
  L.bwd.ldB = ldB;
  L.bwd.E = (float*)P[21];
  L.bwd.C = (float*)P[22];
  L.bwd.g = d_g;
  L.bwd.rmsd = d_rmsd;
  L.bwd.cmax = (unsigned int*)P[40];
  L.plane = pa.plane;
  L.Np = Np;
  L.N = N;
  L.tgt0 = 0;
  L.terms = terms;
  L.map = map;
  L.flags = FlagList{nullptr, (unsigned long long*)P[27], 0};
  if (tc) {
    TcLaunch T2{};
    T2.hi = P[32];
    T2.lo = P[33];
    T2.tile_buf = P[34];
    T2.tile_cap = tc_tiles;
    T2.F = F;
    T2.Np = Np;
    T2.N = N;
    T2.tgt0 = 0;
    T2.inv_scale = (const float*)P[12];
    T2.terms = terms;
    T2.map = map;
    T2.flags = L.flags;
    T2.dev_error = (int*)P[35];
    T2.num_sms = h->num_sms;
    T2.variant = (h->tc_variant >= 2) ? h->tc_variant : (N >= kDeepStageAtoms ? 3 : 2);
    T2.bwd = &L.bwd;
    if ((e = run_pairs_tc(T2, st)) != cudaSuccess) return h->cuda_fail(e, "backward pair kernel");
  } else {
    L.tiles = make_tiles(map, 64, 64);
    if ((e = run_pairs_fp32(L, st)) != cudaSuccess) return h->cuda_fail(e, "backward pair kernel");
  }
  if (h->timing) cudaEventRecord(h->ev[2], st);
  BackwardTail T{};
  T.gemm.F = F;
  T.gemm.Np = Np;
  T.gemm.B = B;
  T.gemm.ldB = ldB;
  T.gemm.plane = pa.plane;
  T.gemm.Shi = (__half*)P[36];
  T.gemm.Slo = (__half*)P[37];
  T.gemm.Thi = (__half*)P[38];
  T.gemm.Tlo = (__half*)P[39];
  T.gemm.maxbits = (unsigned int*)P[40];
  T.gemm.scl = (float*)P[41];
  T.gemm.Z = (float*)P[23];
  T.gemm.dev_error = (int*)P[35];
  T.gemm.num_sms = h->num_sms;
  T.F = F;
  T.N = N;
  T.Np = Np;
  T.plane = pa.plane;
  T.Z = (float*)P[23];
  T.E = (float*)P[21];
  T.C = (float*)P[22];
  T.rot = pa.rot;
  T.ref0 = pa.refs;
  T.w = d_w;
  T.sqw = pa.sqw;
  T.atab = (float4*)P[42];
  T.W = Wsum;
  T.grad = d_grad;
  if ((e = run_backward_tail(T, st)) != cudaSuccess) return h->cuda_fail(e, "backward tail");
  launches += 7;
  if (h->timing) cudaEventRecord(h->ev[3], st);
  if (!grad_dev) cudaMemcpyAsync(grad_xyz, d_grad, sizeof(float) * 3 * N * F, cudaMemcpyDefault, st);
  if (rmsd_out && !r_dev) cudaMemcpyAsync(rmsd_out, d_rmsd, sizeof(float) * npairs, cudaMemcpyDefault, st);
  int derr = 0;
  cudaMemcpyAsync(&derr, P[35], sizeof derr, cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return h->cuda_fail(e, "backward");
  if (derr != 0) return h->fail(GBR_ERR_DEVICE, "pair kernel reported device error %d (bounded wait expired)", derr);
  h->stats.pairs = npairs;
  h->stats.n_refs = 1;
  h->stats.precision = tc ? GBR_PREC_TC : GBR_PREC_FP32;
  h->stats.kernel_launches = launches;
  if (h->timing) {
    float a = 0, b = 0, c = 0;
    cudaEventElapsedTime(&a, h->ev[0], h->ev[1]);
    cudaEventElapsedTime(&b, h->ev[1], h->ev[2]);
    cudaEventElapsedTime(&c, h->ev[2], h->ev[3]);
    h->stats.ms_prep = a;
    h->stats.ms_pairs = b;
    h->stats.ms_fixup = c;
  }
  h->stats.ms_total =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  return GBR_OK;
}

}  // extern "C"
