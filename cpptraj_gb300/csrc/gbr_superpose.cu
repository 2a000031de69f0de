// gbr_superpose.cu -- per-frame best fit of many frames onto one reference:
// the `rms` and `align` actions (K6).
//
// Replaces, for whole trajectories held as one frame set, the per-frame work
// of Action_Rmsd::DoAction (src/Action_Rmsd.cpp:372-395) and
// Action_Align::DoAction (src/Action_Align.cpp:85-99):
//   fit     Frame::RMSD_CenteredRef(ref, U, Trans) (src/Frame.cpp:1137-1273)
//           against the reference centred once (ReferenceAction::
//           SelectRefAtoms -> Frame::CenterOnOrigin, src/Frame.cpp:1043-1055),
//           then Frame::Trans_Rot_Trans(Trans, U, refTrans)
//           (src/Frame.h:572-581) of the frame's atoms to move;
//   nofit   Frame::RMSD_NoFit (src/Frame.cpp:1279-1307) against the
//           uncentred reference.
// One warp per frame, FP64 throughout (the arithmetic of the reference, whose
// rotation and translation outputs are compared directly): the weighted
// centre, then E0 = 1/2 sum w (|y|^2 + |r|^2) and the 3x3 covariance
// sum w y r^T of the centred frame, QCP (Theobald 2005; Liu, Agrafiotis &
// Theobald 2010) for the largest eigenvalue and the rotation, and a third
// sweep that moves the frame's move atoms.  The work is FP64-pipe bound:
// ~21 FP64 operations per atom and frame for the fit, 12 more per moved atom.
#include <vector>

#include "../../include/gbrmsd.h"
#include "gbr_common.cuh"
#include "gbr_handle.h"
#include "gbr_internal.h"

namespace gbr {
namespace {

constexpr int kSupThreads = 256;
constexpr int kSupWarps = kSupThreads / 32;

struct SupArgs {
  const double* ref;  // [N][3]: centred reference (fit) or the reference as given (nofit)
  const double* w;    // [N] target masses, nullptr = unweighted
  double W;           // sum of w (or N)
  double rc[3];       // centre of the reference (added back to moved atoms)
  int N, nofit, n_move;
  double* rmsd;       // [F] or nullptr
  double* rot;        // [F][9] or nullptr
  double* ttr;        // [F][3] or nullptr
};

template <int NV>
__device__ __forceinline__ void warp_sum_f64(double (&v)[NV]) {
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

template <typename T>
__global__ void __launch_bounds__(kSupThreads) k_superpose(const T* __restrict__ xyz, int64_t F, SupArgs a,
                                                           T* move) {
  const int lane = threadIdx.x & 31, N = a.N;
  for (int64_t f = blockIdx.x * (int64_t)kSupWarps + (threadIdx.x >> 5); f < F; f += (int64_t)gridDim.x * kSupWarps) {
    const T* x = xyz + (size_t)f * 3 * N;
    double U[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};
    double c[3] = {0.0, 0.0, 0.0};
    double rms = 0.0;
    if (a.nofit) {
      double v[1] = {0.0};
      for (int i = lane; i < N; i += 32) {
        const double wa = a.w ? a.w[i] : 1.0;
        const double d0 = a.ref[3 * i] - (double)x[3 * i], d1 = a.ref[3 * i + 1] - (double)x[3 * i + 1],
                     d2 = a.ref[3 * i + 2] - (double)x[3 * i + 2];
        v[0] += wa * (d0 * d0 + d1 * d1 + d2 * d2);
      }
      warp_sum_f64<1>(v);
      rms = (v[0] < 0.0) ? 0.0 : sqrt(v[0] / a.W);
    } else {
      double s[3] = {0.0, 0.0, 0.0};
      for (int i = lane; i < N; i += 32) {
        const double wa = a.w ? a.w[i] : 1.0;
        s[0] += (double)x[3 * i] * wa;
        s[1] += (double)x[3 * i + 1] * wa;
        s[2] += (double)x[3 * i + 2] * wa;
      }
      warp_sum_f64<3>(s);
      c[0] = s[0] / a.W;
      c[1] = s[1] / a.W;
      c[2] = s[2] / a.W;
      double v[10] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      for (int i = lane; i < N; i += 32) {
        const double wa = a.w ? a.w[i] : 1.0;
        const double y0 = (double)x[3 * i] - c[0], y1 = (double)x[3 * i + 1] - c[1], y2 = (double)x[3 * i + 2] - c[2];
        const double r0 = a.ref[3 * i], r1 = a.ref[3 * i + 1], r2 = a.ref[3 * i + 2];
        v[9] += wa * (y0 * y0 + y1 * y1 + y2 * y2 + r0 * r0 + r1 * r1 + r2 * r2);
        const double w0 = wa * y0, w1 = wa * y1, w2 = wa * y2;
        v[0] += w0 * r0; v[1] += w0 * r1; v[2] += w0 * r2;
        v[3] += w1 * r0; v[4] += w1 * r1; v[5] += w1 * r2;
        v[6] += w2 * r0; v[7] += w2 * r1; v[8] += w2 * r2;
      }
      warp_sum_f64<10>(v);
      if (lane == 0) {  // one QCP solve per frame, broadcast below
        const double E0 = 0.5 * v[9];
        const double r = E0 - qcp_lambda_rot(v, E0, U);
        rms = (r < 0.0) ? 0.0 : sqrt(2.0 * r / a.W);
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) U[k] = __shfl_sync(0xffffffffu, U[k], 0);
    }
    if (lane == 0) {
      if (a.rmsd) a.rmsd[f] = rms;
      if (a.ttr) {
        a.ttr[3 * f] = -c[0];
        a.ttr[3 * f + 1] = -c[1];
        a.ttr[3 * f + 2] = -c[2];
      }
      if (a.rot)
        for (int k = 0; k < 9; ++k) a.rot[9 * f + k] = U[k];
    }
    if (move && !a.nofit) {
      T* m = move + (size_t)f * 3 * a.n_move;
      for (int i = lane; i < a.n_move; i += 32) {
        const double p0 = (double)m[3 * i] - c[0], p1 = (double)m[3 * i + 1] - c[1], p2 = (double)m[3 * i + 2] - c[2];
        m[3 * i] = (T)(p0 * U[0] + p1 * U[1] + p2 * U[2] + a.rc[0]);
        m[3 * i + 1] = (T)(p0 * U[3] + p1 * U[4] + p2 * U[5] + a.rc[1]);
        m[3 * i + 2] = (T)(p0 * U[6] + p1 * U[7] + p2 * U[8] + a.rc[2]);
      }
    }
  }
}

}  // namespace
}  // namespace gbr

using namespace gbr;

extern "C" int gbr_superpose(gbr_handle* h, const void* ref_xyz, const void* xyz, int dtype, int64_t n_frame,
                             int32_t n_atom, const double* ref_mass, const double* mass, int mode, double* rmsd,
                             double* rot, double* tgt_trans, double* ref_trans, void* move_xyz, int32_t n_move) {
  if (!h) return GBR_ERR_ARG;
  h->err.clear();
  h->stats = gbr_stats{};
  if (!ref_xyz || !xyz) return h->fail(GBR_ERR_ARG, "ref_xyz and xyz must not be NULL");
  if (dtype != GBR_F32 && dtype != GBR_F64) return h->fail(GBR_ERR_ARG, "dtype must be GBR_F32 or GBR_F64");
  if (mode != GBR_FIT && mode != GBR_NOFIT) return h->fail(GBR_ERR_ARG, "mode must be GBR_FIT or GBR_NOFIT");
  if (n_atom < 1) return h->fail(GBR_ERR_ARG, "n_atom must be >= 1 (no atoms selected)");
  if (n_frame < 0) return h->fail(GBR_ERR_ARG, "negative frame count");
  if (!move_xyz) n_move = 0;
  if (n_move < 0) return h->fail(GBR_ERR_ARG, "negative n_move");
  if (int rc = h->check_local({ref_xyz, xyz, rmsd, rot, tgt_trans, ref_trans, move_xyz}, "superpose")) return rc;
  if (cudaSetDevice(h->device) != cudaSuccess) return h->cuda_fail(cudaGetLastError(), "cudaSetDevice");
  cudaStream_t st = h->stream;
  const int N = n_atom;
  const size_t esz = (dtype == GBR_F64) ? 8 : 4;
  const bool nofit = (mode == GBR_NOFIT);

  // Masses and the reference frame are small: read them on the host.
  std::vector<double> w_h, wr_h;
  double W = (double)N;
  if (mass) {
    w_h.resize(N);
    if (cudaMemcpy(w_h.data(), mass, sizeof(double) * N, cudaMemcpyDefault) != cudaSuccess)
      return h->cuda_fail(cudaGetLastError(), "reading mass");
    W = 0.0;
    for (double v : w_h) W += v;
  }
  if (W < 1e-14) return h->fail(GBR_ERR_ZERO_MASS, "total mass %g is below 1e-14 (divide by zero)", W);
  if (ref_mass && mass) {
    wr_h.resize(N);
    if (cudaMemcpy(wr_h.data(), ref_mass, sizeof(double) * N, cudaMemcpyDefault) != cudaSuccess)
      return h->cuda_fail(cudaGetLastError(), "reading ref_mass");
  } else {
    wr_h = w_h;
  }
  std::vector<double> ref(3 * (size_t)N);
  {
    std::vector<char> raw(esz * 3 * (size_t)N);
    if (cudaMemcpy(raw.data(), ref_xyz, raw.size(), cudaMemcpyDefault) != cudaSuccess)
      return h->cuda_fail(cudaGetLastError(), "reading ref_xyz");
    for (size_t k = 0; k < ref.size(); ++k)
      ref[k] = (dtype == GBR_F64) ? ((const double*)raw.data())[k] : (double)((const float*)raw.data())[k];
  }
  // Frame::CenterOnOrigin of the reference (mass-weighted when masses are given).
  double rc[3] = {0.0, 0.0, 0.0};
  if (!nofit) {
    double s[3] = {0.0, 0.0, 0.0}, m = 0.0;
    for (int i = 0; i < N; ++i) {
      const double wi = wr_h.empty() ? 1.0 : wr_h[i];
      s[0] += ref[3 * i] * wi;
      s[1] += ref[3 * i + 1] * wi;
      s[2] += ref[3 * i + 2] * wi;
      m += wi;
    }
    if (m < 1e-14) return h->fail(GBR_ERR_ZERO_MASS, "reference mass %g is below 1e-14 (divide by zero)", m);
    for (int p = 0; p < 3; ++p) rc[p] = s[p] / m;
    for (int i = 0; i < N; ++i)
      for (int p = 0; p < 3; ++p) ref[3 * i + p] -= rc[p];
  }
  if (ref_trans) {
    if (cudaMemcpy(ref_trans, rc, sizeof rc, cudaMemcpyDefault) != cudaSuccess)
      return h->cuda_fail(cudaGetLastError(), "writing ref_trans");
  }
  h->stats.precision = GBR_PREC_FP64;
  if (n_frame == 0) return GBR_OK;

  const bool x_dev = is_device_ptr(xyz);
  const bool mv_dev = move_xyz ? is_device_ptr(move_xyz) : true;
  const bool r_dev = rmsd ? is_device_ptr(rmsd) : true;
  const bool rot_dev = rot ? is_device_ptr(rot) : true;
  const bool t_dev = tgt_trans ? is_device_ptr(tgt_trans) : true;
  const size_t mv_bytes = esz * 3 * (size_t)n_move * n_frame;
  auto layout = [&](Arena& A, void** p) {
    p[0] = A.take<double>(3 * (size_t)N);  // reference
    p[1] = mass ? A.take<double>(N) : nullptr;
    p[2] = x_dev ? nullptr : A.take<char>(esz * 3 * (size_t)N * n_frame);
    p[3] = (move_xyz && !mv_dev) ? A.take<char>(mv_bytes) : nullptr;
    p[4] = (rmsd && !r_dev) ? A.take<double>(n_frame) : nullptr;
    p[5] = (rot && !rot_dev) ? A.take<double>(9 * (size_t)n_frame) : nullptr;
    p[6] = (tgt_trans && !t_dev) ? A.take<double>(3 * (size_t)n_frame) : nullptr;
  };
  void* P[7];
  Arena sizing;
  layout(sizing, P);
  if (!h->reserve(sizing.off + 256))
    return h->fail(GBR_ERR_NOMEM, "cannot allocate %.2f GB of device workspace", (sizing.off + 256) / 1e9);
  Arena A{h->ws, 0};
  layout(A, P);

  if (h->timing) cudaEventRecord(h->ev[0], st);
  cudaMemcpyAsync(P[0], ref.data(), sizeof(double) * 3 * N, cudaMemcpyHostToDevice, st);
  if (mass) cudaMemcpyAsync(P[1], w_h.data(), sizeof(double) * N, cudaMemcpyHostToDevice, st);
  if (!x_dev) cudaMemcpyAsync(P[2], xyz, esz * 3 * (size_t)N * n_frame, cudaMemcpyDefault, st);
  if (move_xyz && !mv_dev) cudaMemcpyAsync(P[3], move_xyz, mv_bytes, cudaMemcpyDefault, st);
  if (h->timing) cudaEventRecord(h->ev[1], st);

  SupArgs a{};
  a.ref = (const double*)P[0];
  a.w = mass ? (const double*)P[1] : nullptr;
  a.W = W;
  a.rc[0] = rc[0];
  a.rc[1] = rc[1];
  a.rc[2] = rc[2];
  a.N = N;
  a.nofit = nofit;
  a.n_move = n_move;
  a.rmsd = rmsd ? (r_dev ? rmsd : (double*)P[4]) : nullptr;
  a.rot = rot ? (rot_dev ? rot : (double*)P[5]) : nullptr;
  a.ttr = tgt_trans ? (t_dev ? tgt_trans : (double*)P[6]) : nullptr;
  void* d_move = move_xyz ? (mv_dev ? move_xyz : P[3]) : nullptr;
  const int grid = (int)std::min<int64_t>((n_frame + kSupWarps - 1) / kSupWarps, 152 * 16);
  if (dtype == GBR_F64)
    k_superpose<double><<<grid, kSupThreads, 0, st>>>((const double*)(x_dev ? xyz : P[2]), n_frame, a,
                                                      (double*)d_move);
  else
    k_superpose<float><<<grid, kSupThreads, 0, st>>>((const float*)(x_dev ? xyz : P[2]), n_frame, a,
                                                     (float*)d_move);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return h->cuda_fail(e, "superpose kernel launch");
  if (h->timing) {
    cudaEventRecord(h->ev[2], st);
    cudaEventRecord(h->ev[3], st);
  }
  if (rmsd && !r_dev) cudaMemcpyAsync(rmsd, P[4], sizeof(double) * n_frame, cudaMemcpyDeviceToHost, st);
  if (rot && !rot_dev) cudaMemcpyAsync(rot, P[5], sizeof(double) * 9 * n_frame, cudaMemcpyDeviceToHost, st);
  if (tgt_trans && !t_dev) cudaMemcpyAsync(tgt_trans, P[6], sizeof(double) * 3 * n_frame, cudaMemcpyDeviceToHost, st);
  if (move_xyz && !mv_dev) cudaMemcpyAsync(move_xyz, P[3], mv_bytes, cudaMemcpyDefault, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return h->cuda_fail(e, "superpose");
  h->stats.pairs = n_frame;
  h->stats.kernel_launches = 1;
  if (h->timing) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev[1], h->ev[2]);
    h->stats.ms_pairs = ms;
  }
  return GBR_OK;
}
