// gbr_exact.cu -- direct FP64 pair RMSD on the GPU.
//
// One warp per pair recomputes what Frame::RMSD_CenteredRef does
// (src/Frame.cpp:1137-1273): centred coordinates, E0 = 1/2 sum w(|t|^2+|r|^2)
// and the 3x3 covariance in FP64, then the largest eigenvalue (here by QCP's
// Newton iteration, the reference's alternative eigen step, src/qcprot.cpp:
// 167-246) and rms = sqrt(2(E0-lambda)/W) clamped at 0; or RMSD_NoFit
// (src/Frame.cpp:1279-1307).  It serves two purposes: the fix-up of pairs whose
// FP32/FP16 error bound exceeded the tolerance, and GBR_PREC_FP64, where it
// computes every pair (a slow checking mode).
#include "gbr_common.cuh"
#include "gbr_internal.h"

namespace gbr {

namespace {

template <typename T>
__device__ __forceinline__ const T* frame_ptr(const ExactLaunch& L, int64_t set_f) {
  const T* ref = (const T*)L.ref;
  const T* tgt = (const T*)(L.tgt ? L.tgt : L.ref);
  return (set_f < L.n_ref) ? ref + (size_t)set_f * 3 * L.N : tgt + (size_t)(set_f - L.n_ref) * 3 * L.N;
}

// Output position k of the call -> (reference frame, target frame).
__device__ __forceinline__ void pair_of(const OutMap& m, int64_t k, int64_t& i, int64_t& jt) {
  if (m.tri) {
    const int64_t n = m.n_ref;
    const int64_t g = k + m.base;  // global triangle index
    const double b = 2.0 * (double)n - 1.0;
    int64_t r = (int64_t)((b - sqrt(fmax(b * b - 8.0 * (double)g, 0.0))) * 0.5);
    auto cnt = [&](int64_t x) { return x * n - x * (x + 1) / 2; };
    if (r < 0) r = 0;
    while (r > 0 && cnt(r) > g) --r;
    while (cnt(r + 1) <= g) ++r;
    i = r;
    jt = g - cnt(r) + r + 1;
  } else {
    jt = m.row_begin + k / m.n_ref;
    i = k % m.n_ref;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_exact(ExactLaunch L) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int64_t count = L.count;
  bool use_list = L.list != nullptr;
  if (L.dev_count) {
    const unsigned long long c = *L.dev_count;
    if (L.overflow_all && c > (unsigned long long)L.count) {
      use_list = false;  // the list overflowed: every pair of the map, directly
      count = L.map_pairs;
    } else {
      count = (int64_t)min((unsigned long long)L.count, c);
    }
  }
  for (int64_t k = warp; k < count; k += nwarps) {
    int64_t i, jt;
    if (use_list) {
      const int2 p = L.list[k];
      i = p.x;
      jt = p.y;
    } else {
      pair_of(L.map, k, i, jt);
    }
    const int64_t js = L.tgt0 + jt;
    const T* xi = frame_ptr<T>(L, i);
    const T* xj = frame_ptr<T>(L, js);
    const double ci0 = L.cen[3 * i], ci1 = L.cen[3 * i + 1], ci2 = L.cen[3 * i + 2];
    const double cj0 = L.cen[3 * js], cj1 = L.cen[3 * js + 1], cj2 = L.cen[3 * js + 2];
    double v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = lane; a < L.N; a += 32) {
      const double w = L.w ? L.w[a] : 1.0;
      const double r0 = (double)xi[3 * a] - ci0, r1 = (double)xi[3 * a + 1] - ci1, r2 = (double)xi[3 * a + 2] - ci2;
      const double t0 = (double)xj[3 * a] - cj0, t1 = (double)xj[3 * a + 1] - cj1, t2 = (double)xj[3 * a + 2] - cj2;
      if (L.nofit) {
        const double d0 = r0 - t0, d1 = r1 - t1, d2 = r2 - t2;
        v[9] += w * (d0 * d0 + d1 * d1 + d2 * d2);
      } else {
        v[0] += w * t0 * r0; v[1] += w * t0 * r1; v[2] += w * t0 * r2;
        v[3] += w * t1 * r0; v[4] += w * t1 * r1; v[5] += w * t1 * r2;
        v[6] += w * t2 * r0; v[7] += w * t2 * r1; v[8] += w * t2 * r2;
        v[9] += w * (t0 * t0 + t1 * t1 + t2 * t2 + r0 * r0 + r1 * r1 + r2 * r2);
      }
    }
#pragma unroll
    for (int q = 0; q < 10; ++q)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    if (lane == 0) {
      const double Wsum = L.dWsum ? *L.dWsum : L.Wsum;
      double rms;
      if (L.nofit) {
        rms = (v[9] < 0.0) ? 0.0 : sqrt(v[9] / Wsum);
      } else {
        double R[9];
        const double E0 = 0.5 * v[9];
        const double lam = qcp_lambda_rot(v, E0, R);
        const double e = E0 - lam;
        rms = (e < 0.0) ? 0.0 : sqrt(2.0 * e / Wsum);
      }
      const int64_t idx = out_index(L.map, i, jt);
      if (idx >= 0) L.map.out[idx] = (float)rms;
    }
  }
}
}  // namespace

cudaError_t run_exact(const ExactLaunch& L, cudaStream_t st) {
  if (L.count <= 0) return cudaSuccess;
  const int64_t warps_needed = L.count;
  // With a device-side count the true length is unknown here: use a grid
  // that covers the capacity up to a few waves and loop inside.
  const int grid = (int)std::min<int64_t>((warps_needed + 7) / 8, L.dev_count ? 152 * 8 : 152 * 32);
  if (L.dev_count && L.overflow_all && L.map_pairs < 0) return cudaErrorInvalidValue;
  if (L.dtype_f64)
    k_exact<double><<<grid, 256, 0, st>>>(L);
  else
    k_exact<float><<<grid, 256, 0, st>>>(L);
  return cudaGetLastError();
}

}  // namespace gbr
