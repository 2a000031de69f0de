// gbr_centroid.cu -- cluster centroids (K7): Metric_RMS::CalculateCentroid
// (src/Cluster/Metric_RMS.cpp:86-108) for every cluster at once.
//
// The reference builds a centroid as a chain: the first member, centred
// (Frame::CenterOnOrigin), starts a running sum S; each later member is
// centred and fitted onto S by Frame::RMSD_CenteredRef(S, U, Trans)
// (src/Frame.cpp:1137-1273), rotated about the origin (Frame::Rotate,
// src/Frame.h:508-517) and added (Frame::operator+=, src/Frame.cpp:901-910);
// at the end S is divided by the member count (Frame::Divide,
// src/Frame.cpp:968-976).  No-fit sums the members as they are.  Member k's
// rotation depends on every member before it, so a cluster is one sequential
// chain: one CTA per cluster walks it, and independent clusters run on
// different SMs.
//
// One step of the chain (member k >= 1, centre c_k known):
//   sweep 1   per atom: y = x_k - c_k, the covariance sum w y S^T (9), sum w
//             |y|^2 and sum w |S|^2, and the centre sums of member k + 1 (3):
//             one block reduction of 14 values per step;
//   solve     one thread: QCP on the covariance against S / k (the
//             rotation does not depend on the scale of S; the mean keeps
//             Newton's start E0 close to the root) -> U, broadcast.  The
//             first kExactSteps steps, which set the orientation of the
//             centroid, solve in FP64 and broadcast U as FP32 hi + lo; later
//             steps solve in FP32 (a single-lane FP64 instruction costs a
//             whole warp's turn on GB300's narrow FP64 pipe: ~250 of them
//             made an FP64 solve ~8 us);
//   sweep 2   per atom: S += U y.
// FP32 frames come through a shared-memory ring (cp.async, three members
// ahead), so the chain does not wait on DRAM.  Sweep 2 of step k runs fused
// with sweep 1 of step k + 1 (one pass over the atoms per step).
// Per-atom arithmetic is FP32 (GB300's FP64 rate would make the two sweeps
// FP64-pipe bound); S is kept as an unevaluated FP32 sum hi + lo (TwoSum), so
// adding thousands of members loses nothing to rounding; the solve and the
// final division are FP64.  Fitted FP64 input frames are rounded to FP32 on
// load; no-fit sums take FP64 inputs as FP32 hi + lo.  Deviation from the
// reference's FP64 chain: ~1e-6 Angstrom in fitted centroid coordinates (FP32
// covariance sums, FP32 centring), ~1e-14 relative without fitting.
#include <vector>

#include "../../include/gbrmsd.h"
#include "gbr_common.cuh"
#include "gbr_handle.h"
#include "gbr_internal.h"

namespace gbr {
namespace {

constexpr int kChainWarps = 7;   // fitted chain: 6 sweeping warps + the solving warp
constexpr int kSolverWarp = 3;
constexpr int kRing = 8;           // staged members: k - 1, k, k + 1 in use, k + 2 .. k + 4 in flight
constexpr int kAhead = 3;          // members in flight beyond the ones in use
constexpr int kExactSteps = 32;    // chain steps solved in FP64
constexpr size_t kStageMaxBytes = 200 * 1024;
constexpr int kSumThreads = 256;   // no-fit: one thread per centroid coordinate
constexpr int kSumUnroll = 8;      // members loaded ahead per thread

struct CenArgs {
  const int32_t* members;  // frame indices, clusters back to back
  const int64_t* offsets;  // [n_cluster + 1]
  const float* w;          // [N] masses, nullptr = unweighted
  double inv_W;            // 1 / sum of w (or 1 / N)
  float inv_Wf;            // the same in FP32 (per-step centres: FP32 sums, no FP64 on the chain)
  int N;
  float2* S;               // [n_cluster][3N] running sums, hi + lo (when not in shared memory)
  double* out;             // [n_cluster][N][3]
};

__device__ __forceinline__ float2 add_hl(float2 s, float v) {
  const float hi = s.x + v;
  const float bb = hi - s.x;
  const float e = (s.x - (hi - bb)) + (v - bb);
  const float lo = s.y + e;
  const float h2 = hi + lo;  // renormalise so |lo| stays below half an ulp of hi
  return make_float2(h2, lo - (h2 - hi));
}

template <typename T>
__device__ __forceinline__ void load3(const T* x, int i, float (&v)[3]) {
  v[0] = (float)x[3 * i];
  v[1] = (float)x[3 * i + 1];
  v[2] = (float)x[3 * i + 2];
}

__device__ __forceinline__ double qnan() { return __longlong_as_double(0x7ff8000000000000LL); }

// Stages each thread's own atoms of a frame into shared memory (4-byte
// cp.async: a thread later reads exactly what it copied, so completion needs
// no barrier, only cp.async.wait_group).
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int K>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(K) : "memory"); }

// Proper rotation (row-major, FP32) of the quaternion q, in the orientation
// of qcp_lambda_rot's R.  A zero or non-finite q gives the identity.
__device__ __forceinline__ void rotation_from_quat_f32(const float qv[4], float R[9]) {
  float a0 = qv[0], a1 = qv[1], a2 = qv[2], a3 = qv[3];
  const float n2 = a0 * a0 + a1 * a1 + a2 * a2 + a3 * a3;
  if (!(n2 > 0.0f) || !isfinite(n2)) {
    a0 = 1.0f; a1 = a2 = a3 = 0.0f;
  } else {
    float inv = rsqrtf(n2);
    inv = inv * (1.5f - 0.5f * n2 * inv * inv);  // one Newton step: unit to ~1 ulp
    a0 *= inv; a1 *= inv; a2 *= inv; a3 *= inv;
  }
  const float aa = a0 * a0, bb = a1 * a1, cc = a2 * a2, dd = a3 * a3;
  R[0] = aa + bb - cc - dd;
  R[3] = 2.0f * (a1 * a2 + a0 * a3);
  R[6] = 2.0f * (a3 * a1 - a0 * a2);
  R[1] = 2.0f * (a1 * a2 - a0 * a3);
  R[4] = aa - bb + cc - dd;
  R[7] = 2.0f * (a2 * a3 + a0 * a1);
  R[2] = 2.0f * (a3 * a1 + a0 * a2);
  R[5] = 2.0f * (a2 * a3 - a0 * a1);
  R[8] = aa - bb - cc + dd;
}

// FP32 QCP for one thread on the critical path of the chain: the key matrix
// of M (A[p][q] = sum w t_p r_q) scaled by 1/E0, Newton from 1 with
// approximate divisions (the fixed point does not depend on them), and the
// largest adjugate column of K - lambda I; U in the orientation of
// qcp_lambda_rot (U t ~ r).
__device__ __forceinline__ void qcp_rot_f32(const float M[9], float E0, float U[9]) {
  const float s = __fdividef(1.0f, E0);  // a uniform scale: any rounding leaves U unchanged
  const float xx = M[0] * s, xy = M[1] * s, xz = M[2] * s, yx = M[3] * s, yy = M[4] * s,
              yz = M[5] * s, zx = M[6] * s, zy = M[7] * s, zz = M[8] * s;
  const float xx2 = xx * xx, yy2 = yy * yy, zz2 = zz * zz, xy2 = xy * xy, yz2 = yz * yz,
              xz2 = xz * xz, yx2 = yx * yx, zy2 = zy * zy, zx2 = zx * zx;
  const float c2 = -2.0f * (xx2 + yy2 + zz2 + xy2 + yx2 + xz2 + zx2 + yz2 + zy2);
  const float c1 = 8.0f * (xx * yz * zy + yy * zx * xz + zz * xy * yx - xx * yy * zz -
                           yz * zx * xy - zy * yx * xz);
  const float t1 = 2.0f * (yz * zy - yy * zz);
  const float t2 = yy2 + zz2 - xx2 + yz2 + zy2;
  const float t3 = xy2 + xz2 - yx2 - zx2;
  const float pxz = xz + zx, pyz = yz + zy, pxy = xy + yx, myz = yz - zy, mxz = xz - zx,
              mxy = xy - yx, pxx = xx + yy, mxx = xx - yy;
  const float c0 = t3 * t3 + (t2 + t1) * (t2 - t1) +
                   (-pxz * myz + mxy * (mxx - zz)) * (-mxz * pyz + mxy * (mxx + zz)) +
                   (-pxz * pyz - pxy * (pxx - zz)) * (-mxz * myz - pxy * (pxx + zz)) +
                   (pxy * pyz + pxz * (mxx + zz)) * (-mxy * myz + pxz * (pxx + zz)) +
                   (pxy * myz + mxz * (mxx - zz)) * (-mxy * pyz + mxz * (pxx - zz));
  float lam = 1.0f;
  for (int it = 0; it < 16; ++it) {
    const float l2 = lam * lam, b = (l2 + c2) * lam, a = b + c1;
    const float den = 2.0f * l2 * lam + b + a;
    if (!(den != 0.0f)) break;
    const float dl = __fdividef(a * lam + c0, den);
    lam -= dl;
    if (fabsf(dl) <= 2e-7f * fabsf(lam)) break;
  }
  const float k11 = pxx + zz - lam, k12 = myz, k13 = -mxz, k14 = mxy;
  const float k22 = mxx - zz - lam, k23 = pxy, k24 = pxz;
  const float k33 = yy - xx - zz - lam, k34 = pyz;
  const float k44 = zz - pxx - lam;
  const float a3344 = k33 * k44 - k34 * k34, a3244 = k23 * k44 - k24 * k34,
              a3243 = k23 * k34 - k24 * k33, a3143 = k13 * k34 - k14 * k33,
              a3144 = k13 * k44 - k14 * k34, a3142 = k13 * k24 - k14 * k23;
  float q[4] = {k22 * a3344 - k23 * a3244 + k24 * a3243, -k12 * a3344 + k23 * a3144 - k24 * a3143,
                k12 * a3244 - k22 * a3144 + k24 * a3142, -k12 * a3243 + k22 * a3143 - k23 * a3142};
  // All four columns, largest norm wins: a column's accuracy goes with the
  // size of the quaternion component it is proportional to.
  float bn = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  {
    float c[4] = {k12 * a3344 - k13 * a3244 + k14 * a3243, -k11 * a3344 + k13 * a3144 - k14 * a3143,
                  k11 * a3244 - k12 * a3144 + k14 * a3142, -k11 * a3243 + k12 * a3143 - k13 * a3142};
    float n = c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
    if (n > bn) { bn = n; q[0] = c[0]; q[1] = c[1]; q[2] = c[2]; q[3] = c[3]; }
    const float a1324 = k13 * k24 - k14 * k23, a1224 = k12 * k24 - k14 * k22,
                a1223 = k12 * k23 - k13 * k22, a1124 = k11 * k24 - k14 * k12,
                a1123 = k11 * k23 - k13 * k12, a1122 = k11 * k22 - k12 * k12;
    c[0] = k24 * a1324 - k34 * a1224 + k44 * a1223;
    c[1] = -k14 * a1324 + k34 * a1124 - k44 * a1123;
    c[2] = k14 * a1224 - k24 * a1124 + k44 * a1122;
    c[3] = -k14 * a1223 + k24 * a1123 - k34 * a1122;
    n = c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
    if (n > bn) { bn = n; q[0] = c[0]; q[1] = c[1]; q[2] = c[2]; q[3] = c[3]; }
    c[0] = k23 * a1324 - k33 * a1224 + k34 * a1223;
    c[1] = -k13 * a1324 + k33 * a1124 - k34 * a1123;
    c[2] = k13 * a1224 - k23 * a1124 + k34 * a1122;
    c[3] = -k13 * a1223 + k23 * a1123 - k33 * a1122;
    n = c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
    if (n > bn) { q[0] = c[0]; q[1] = c[1]; q[2] = c[2]; q[3] = c[3]; }
  }
  rotation_from_quat_f32(q, U);
}

// Warp sums of 32 values in 31 shuffles (each round keeps half of the values
// and trades the other half with the partner lane).  On return v[0] of lane
// l holds the warp's total of value index
//   16 * bit4(l) + 8 * bit3(l) + 4 * bit2(l) + 2 * bit1(l) + bit0(l).
__device__ __forceinline__ void warp_sum32(float (&v)[32], int lane) {
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    const int h = 16 >> r;  // values kept after this round
    const int o = 16 >> r;  // partner lane distance
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int j = 0; j < h; ++j) {
      const float send = up ? v[j] : v[j + h];
      const float keep = up ? v[j + h] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
}
__device__ __forceinline__ int warp_sum32_index(int lane) {
  return ((lane >> 4) & 1) * 16 + ((lane >> 3) & 1) * 8 + ((lane >> 2) & 1) * 4 + ((lane >> 1) & 1) * 2 + (lane & 1);
}

// Per-step sums of the pipelined chain (slots of red[][][32]).
constexpr int kP = 0;    // 9: sum w y_{j+1} S_j^T
constexpr int kQ = 9;    // 9: sum w y_{j+1} y_j^T
constexpr int kGy = 18;  // sum w |y_{j+1}|^2
constexpr int kGs = 19;  // sum w |S_j|^2
constexpr int kC = 20;   // 3: centre sums of member j + 2
constexpr int kNV = 23;

// Fitted centroids, one CTA per cluster: kChainWarps - 1 sweeping warps and
// one solving warp, pipelined.  With S_j the sum of members 0..j-1 (each rotated)
// and y_j member j centred, member j's rotation U_j solves the covariance
//   A_j = sum w y_j S_j^T = P_j + Q_j U_{j-1}^T,
//   P_j = sum w y_j S_{j-1}^T,  Q_j = sum w y_j y_{j-1}^T,
// because S_j = S_{j-1} + U_{j-1} y_{j-1}.  P_j and Q_j need no U_{j-1}, so
// step j's sweep (S_{j-1} += U_{j-2} y_{j-2}, then P, Q for member j + 1)
// runs while the solving warp turns A_j into U_j; then one barrier.  The
// solver keeps A_j, U_j and sum w|y_j|^2 for the next step's
//   sum w |S_{j+1}|^2 = sum w |S_j|^2 + 2 tr(U_j A_j) + sum w |y_j|^2.
// Reduction partials and the broadcast U are double-buffered by step parity.
// STAGE (FP32 frames, S and kRing frames fitting kStageMaxBytes of shared
// memory): S lives in shared memory (it is re-read every step; global stores
// do not stay in L1) and frames come through a ring of kRing shared-memory
// buffers, kAhead members issued ahead of the four in use.  Otherwise S is in
// global memory and frames are read from there.
template <typename T, bool STAGE>
__global__ void __launch_bounds__(32 * kChainWarps) k_centroid_chain(const T* __restrict__ xyz, CenArgs a) {
  extern __shared__ float4 dyn[];
  __shared__ float red[2][kChainWarps - 1][32];
  __shared__ float bc[2][18];  // U_j as FP32 hi (9) and lo (9), row-major, by step parity
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, N = a.N;
  // kChainWarps warps: the solving warp is warp kSolverWarp, alone on its
  // scheduler (warps of an SM sub-partition share warp index mod 4), so its
  // latency-bound chain does not wait for issue slots behind the sweeps; the
  // other nsw warps sweep, as sweeping warp sw.
  constexpr int nsw = kChainWarps - 1, nst = 32 * nsw;
  const bool solver = (warp == kSolverWarp);
  const int sw = warp < kSolverWarp ? warp : warp - 1;
  const int sid = 32 * sw + lane;  // sweeping thread index
  const int64_t cl = blockIdx.x;
  const int64_t o0 = a.offsets[cl], n = a.offsets[cl + 1] - o0;
  double* out = a.out + (size_t)cl * 3 * N;
  if (n <= 0) {  // the reference's centroid has no atoms
    for (int i = tid; i < 3 * N; i += blockDim.x) out[i] = qnan();
    return;
  }
  float2* S = STAGE ? (float2*)dyn : a.S + (size_t)cl * 3 * N;
  float* ring = (float*)dyn + 6 * N;  // after S (3N float2)
  const int32_t* mem = a.members + o0;
  auto frame_at = [&](int32_t f) { return xyz + (size_t)f * 3 * N; };
  auto wt = [&](int i) { return a.w ? a.w[i] : 1.0f; };
  // Copies of this thread's atoms of frame f (member k) into ring buffer
  // k % kRing: one cp.async group per member, empty past the last.
  auto stage = [&](int64_t k, int32_t f) {
    if constexpr (STAGE) {
      if (k < n) {
        const float* src = (const float*)frame_at(f);
        float* dst = ring + (size_t)(k & (kRing - 1)) * 3 * N;
        for (int i = sid; i < N; i += nst) {
          cp_async4(dst + 3 * i, src + 3 * i);
          cp_async4(dst + 3 * i + 1, src + 3 * i + 1);
          cp_async4(dst + 3 * i + 2, src + 3 * i + 2);
        }
      }
      cp_async_commit();
    }
  };
  auto get = [&](int64_t k, int i, float (&v)[3]) {
    if constexpr (STAGE) {
      const float* b = ring + (size_t)(k & (kRing - 1)) * 3 * N + 3 * i;
      v[0] = b[0]; v[1] = b[1]; v[2] = b[2];
    } else {
      load3(frame_at(mem[k]), i, v);
    }
  };
  static_assert((kRing & (kRing - 1)) == 0, "ring size is a power of two");
  static_assert(kRing >= kAhead + 4, "the ring holds members j - 1 .. j + 2 and kAhead in flight");

  // ---- prologue (sweeping warps; the solver takes part in the barriers) ----
  // Members 0 .. kAhead + 1 issued; step j issues member j + kAhead + 2, whose
  // frame index was loaded one step earlier.
  int32_t f_ahead = 0;
  if (!solver && STAGE) {
#pragma unroll
    for (int k = 0; k < kAhead + 2; ++k) stage(k, k < n ? mem[k] : 0);
    f_ahead = (kAhead + 2 < n) ? mem[kAhead + 2] : 0;
    cp_async_wait<kAhead>();  // members 0 and 1 are in
  }
  // Centres of members 0 and 1.
  {
    float v[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) v[q] = 0.0f;
    if (!solver) {
      for (int i = sid; i < N; i += nst) {
        float p[3], r[3];
        get(0, i, p);
        get(n > 1 ? 1 : 0, i, r);
        const float wi = wt(i);
        v[0] += wi * p[0]; v[1] += wi * p[1]; v[2] += wi * p[2];
        v[3] += wi * r[0]; v[4] += wi * r[1]; v[5] += wi * r[2];
      }
      warp_sum32(v, lane);
      red[1][sw][warp_sum32_index(lane)] = v[0];
    }
    __syncthreads();
  }
  // Sweeping threads keep the centres of members j - 1, j, j + 1.
  float cm1[3] = {0.0f, 0.0f, 0.0f}, c0[3], c1[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    float s0 = 0.0f, s1 = 0.0f;
    for (int w = 0; w < nsw; ++w) {
      s0 += red[1][w][q];
      s1 += red[1][w][3 + q];
    }
    c0[q] = s0 * a.inv_Wf;
    c1[q] = s1 * a.inv_Wf;
  }
  // S_1 = member 0 centred.
  if (!solver)
    for (int i = sid; i < N; i += nst) {
      float p[3];
      get(0, i, p);
#pragma unroll
      for (int q = 0; q < 3; ++q) S[3 * i + q] = make_float2(p[q] - c0[q], 0.0f);
    }
  // From here, at step j: cm1 = c_{j-1}, c0 = c_j, c1 = c_{j+1}.

  // Solver state (lane 0 of the solving warp): A_j, U_j, sum w|y_j|^2.
  float A_prev[9], Uh_prev[9], Ul_prev[9], gy_prev = 0.0f;

  // Step j = 0 .. n-1.  Sweep j: S_j from S_{j-1} (j >= 2), then the sums of
  // member j + 1.  Solve j (j >= 1): U_j from the sums of sweep j - 1.
  for (int64_t j = 0; j < n; ++j) {
    const int par = (int)(j & 1), prv = par ^ 1;
    if (solver) {
      if (j >= 1 && lane == 0) {
        // The totals of sweep j - 1: independent shared-memory loads, so
        // their latencies overlap (a shuffle gather serialises them).
        float ts[kNV];
#pragma unroll
        for (int q = 0; q < kNV; ++q) ts[q] = red[prv][0][q];
#pragma unroll
        for (int w = 1; w < nsw; ++w)
#pragma unroll
          for (int q = 0; q < kNV; ++q) ts[q] += red[prv][w][q];
        {
          float A[9];
          const float gy = ts[kGy];
          if (j <= kExactSteps) {
            // FP64 steps: A_j, sum w|S_j|^2 and the solve in FP64, U out as
            // hi + lo.  The first members' turns set the orientation of the
            // whole centroid: an FP32-rounded U (or A formed from it) would
            // turn each of them by ~1e-7 rad.
            double Ad[9], Gs;
            if (j == 1) {
#pragma unroll
              for (int q = 0; q < 9; ++q) Ad[q] = (double)ts[kP + q];  // swept against S_1 itself
              Gs = (double)ts[kGs];
            } else {
              double trUA = 0.0;
#pragma unroll
              for (int p = 0; p < 3; ++p)
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                  double acc = (double)ts[kP + 3 * p + q];
#pragma unroll
                  for (int r = 0; r < 3; ++r)
                    acc += (double)ts[kQ + 3 * p + r] * ((double)Uh_prev[3 * q + r] + (double)Ul_prev[3 * q + r]);
                  Ad[3 * p + q] = acc;
                  trUA += ((double)Uh_prev[3 * p + q] + (double)Ul_prev[3 * p + q]) * (double)A_prev[3 * q + p];
                }
              Gs = (double)ts[kGs] + 2.0 * trUA + (double)gy_prev;  // sum w |S_j|^2
            }
#pragma unroll
            for (int q = 0; q < 9; ++q) A[q] = (float)Ad[q];
            const double ik = 1.0 / (double)j;
            double U[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) Ad[q] *= ik;
            qcp_lambda_rot(Ad, 0.5 * ((double)gy + Gs * ik * ik), U);
#pragma unroll
            for (int q = 0; q < 9; ++q) {
              const float hi = (float)U[q];
              Uh_prev[q] = hi;
              Ul_prev[q] = (float)(U[q] - (double)hi);
            }
          } else {
            float trUA = 0.0f;
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
              for (int q = 0; q < 3; ++q) {
                float acc = ts[kP + 3 * p + q];
#pragma unroll
                for (int r = 0; r < 3; ++r)
                  acc = fmaf(ts[kQ + 3 * p + r], Uh_prev[3 * q + r] + Ul_prev[3 * q + r], acc);
                A[3 * p + q] = acc;
                trUA = fmaf(Uh_prev[3 * p + q] + Ul_prev[3 * p + q], A_prev[3 * q + p], trUA);
              }
            const float Gs = ts[kGs] + 2.0f * trUA + gy_prev;  // sum w |S_j|^2
            // FP32 solve: a later member moves the sum by 1/j of its own
            // weight, so its rotation error averages out.
            const float ik = __fdividef(1.0f, (float)j);
            float M[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) M[q] = A[q] * ik;
            qcp_rot_f32(M, 0.5f * (gy + Gs * ik * ik), Uh_prev);
#pragma unroll
            for (int q = 0; q < 9; ++q) Ul_prev[q] = 0.0f;
          }
#pragma unroll
          for (int q = 0; q < 9; ++q) {
            bc[par][q] = Uh_prev[q];
            bc[par][9 + q] = Ul_prev[q];
            A_prev[q] = A[q];
          }
          gy_prev = gy;
        }
      }
    } else {
      if constexpr (STAGE) {
        // Buffer (j + kAhead + 2) % kRing last held member j + kAhead + 2 -
        // kRing <= j - 2, which no later step reads.
        const int32_t f = f_ahead;
        f_ahead = (j + kAhead + 3 < n) ? mem[j + kAhead + 3] : 0;
        stage(j + kAhead + 2, f);
        cp_async_wait<kAhead>();  // members up to j + 2 are in
      }
      if (j >= 1) {  // c_{j+1} from sweep j - 1's centre sums
        cm1[0] = c0[0]; cm1[1] = c0[1]; cm1[2] = c0[2];
        c0[0] = c1[0]; c0[1] = c1[1]; c0[2] = c1[2];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          float sq = 0.0f;
          for (int w = 0; w < nsw; ++w) sq += red[prv][w][kC + q];
          c1[q] = sq * a.inv_Wf;
        }
      }
      const bool upd = (j >= 2), next = (j + 1 < n);
      float Uh[9], Ul[9];
      if (upd) {
#pragma unroll
        for (int q = 0; q < 9; ++q) {
          Uh[q] = bc[prv][q];
          Ul[q] = bc[prv][9 + q];
        }
      }
      float v[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) v[q] = 0.0f;
      if (upd || next) {
        for (int i = sid; i < N; i += nst) {
          float2 sv[3];
#pragma unroll
          for (int q = 0; q < 3; ++q) sv[q] = S[3 * i + q];
          if (upd) {  // S_j = S_{j-1} + U_{j-1} y_{j-1}
            float y[3];
            get(j - 1, i, y);
#pragma unroll
            for (int q = 0; q < 3; ++q) y[q] -= cm1[q];
#pragma unroll
            for (int p = 0; p < 3; ++p) {
              const float lo = Ul[3 * p] * y[0] + Ul[3 * p + 1] * y[1] + Ul[3 * p + 2] * y[2];
              const float r = fmaf(Uh[3 * p], y[0], fmaf(Uh[3 * p + 1], y[1], fmaf(Uh[3 * p + 2], y[2], lo)));
              sv[p] = add_hl(sv[p], r);
              S[3 * i + p] = sv[p];
            }
          }
          if (next) {
            const float wi = wt(i);
            float y1[3], y0[3], x2[3];
            get(j + 1, i, y1);
            get(j, i, y0);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
              y1[q] -= c1[q];
              y0[q] -= c0[q];
            }
#pragma unroll
            for (int p = 0; p < 3; ++p) {
              const float wy = wi * y1[p];
#pragma unroll
              for (int q = 0; q < 3; ++q) {
                v[kP + 3 * p + q] += wy * sv[q].x;
                v[kQ + 3 * p + q] += wy * y0[q];
              }
            }
            v[kGy] += wi * (y1[0] * y1[0] + y1[1] * y1[1] + y1[2] * y1[2]);
            v[kGs] += wi * (sv[0].x * sv[0].x + sv[1].x * sv[1].x + sv[2].x * sv[2].x);
            if (j + 2 < n) {
              get(j + 2, i, x2);
              v[kC] += wi * x2[0]; v[kC + 1] += wi * x2[1]; v[kC + 2] += wi * x2[2];
            }
          }
        }
      }
      warp_sum32(v, lane);
      red[par][sw][warp_sum32_index(lane)] = v[0];
    }
    // U_j and sweep j's sums published; red[prv] and bc[prv] were read.
    __syncthreads();
  }
  // The last member: S_n = S_{n-1} + U_{n-1} y_{n-1}.
  if (!solver && n >= 2) {
    const int lp = (int)((n - 1) & 1);
    float Uh[9], Ul[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      Uh[q] = bc[lp][q];
      Ul[q] = bc[lp][9 + q];
    }
    // c0 holds c_{n-1} after the last step's rotation of the centres
    for (int i = sid; i < N; i += nst) {
      float y[3];
      get(n - 1, i, y);
#pragma unroll
      for (int q = 0; q < 3; ++q) y[q] -= c0[q];
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        const float lo = Ul[3 * p] * y[0] + Ul[3 * p + 1] * y[1] + Ul[3 * p + 2] * y[2];
        const float r = fmaf(Uh[3 * p], y[0], fmaf(Uh[3 * p + 1], y[1], fmaf(Uh[3 * p + 2], y[2], lo)));
        S[3 * i + p] = add_hl(S[3 * i + p], r);
      }
    }
  }
  if constexpr (STAGE) cp_async_wait<0>();
  // The sums were written per atom (thread t: elements 3t..3t+2); they are
  // read per element below.
  __syncthreads();
  const double inv_n = 1.0 / (double)n;
  for (int i = tid; i < 3 * N; i += blockDim.x) {
    const float2 sv = S[i];
    out[i] = ((double)sv.x + (double)sv.y) * inv_n;
  }
}

// No-fit centroids: plain sums with no chain, so every coordinate of every
// cluster is its own thread (grid: clusters x coordinate blocks), members
// loaded kSumUnroll ahead.  FP64 inputs enter as FP32 hi + lo.
template <typename T>
__global__ void __launch_bounds__(kSumThreads) k_centroid_sum(const T* __restrict__ xyz, CenArgs a) {
  const int n3 = 3 * a.N;
  const int e = blockIdx.y * kSumThreads + threadIdx.x;
  const int64_t cl = blockIdx.x;
  if (e >= n3) return;
  const int64_t o0 = a.offsets[cl], n = a.offsets[cl + 1] - o0;
  double* out = a.out + (size_t)cl * n3;
  if (n <= 0) {
    out[e] = qnan();
    return;
  }
  const int32_t* mem = a.members + o0;
  float2 s = make_float2(0.0f, 0.0f);
  auto add = [&](T x) {
    const float hi = (float)x;
    s = add_hl(s, hi);
    if constexpr (sizeof(T) == 8) s = add_hl(s, (float)(x - (double)hi));
  };
  int64_t k = 0;
  for (; k + kSumUnroll <= n; k += kSumUnroll) {
    T x[kSumUnroll];
#pragma unroll
    for (int j = 0; j < kSumUnroll; ++j) x[j] = xyz[(size_t)mem[k + j] * n3 + e];
#pragma unroll
    for (int j = 0; j < kSumUnroll; ++j) add(x[j]);
  }
  for (; k < n; ++k) add(xyz[(size_t)mem[k] * n3 + e]);
  out[e] = ((double)s.x + (double)s.y) / (double)n;
}

}  // namespace
}  // namespace gbr

using namespace gbr;

extern "C" int gbr_cluster_centroids(gbr_handle* h, const void* xyz, int dtype, int64_t n_frame, int32_t n_atom,
                                     const double* mass, int mode, const int32_t* members, const int64_t* offsets,
                                     int64_t n_cluster, double* centroids) {
  if (!h) return GBR_ERR_ARG;
  h->err.clear();
  h->stats = gbr_stats{};
  if (n_cluster < 0) return h->fail(GBR_ERR_ARG, "negative cluster count");
  if (n_cluster == 0) return GBR_OK;
  if (!xyz || !offsets || !centroids) return h->fail(GBR_ERR_ARG, "xyz, offsets and centroids must not be NULL");
  if (dtype != GBR_F32 && dtype != GBR_F64) return h->fail(GBR_ERR_ARG, "dtype must be GBR_F32 or GBR_F64");
  if (mode != GBR_FIT && mode != GBR_NOFIT) return h->fail(GBR_ERR_ARG, "mode must be GBR_FIT or GBR_NOFIT");
  if (n_atom < 1) return h->fail(GBR_ERR_ARG, "n_atom must be >= 1 (no atoms selected)");
  if (n_frame < 0) return h->fail(GBR_ERR_ARG, "negative frame count");
  if (int rc = h->check_local({xyz, centroids}, "cluster_centroids")) return rc;
  if (cudaSetDevice(h->device) != cudaSuccess) return h->cuda_fail(cudaGetLastError(), "cudaSetDevice");
  cudaStream_t st = h->stream;
  const int N = n_atom;
  const size_t esz = (dtype == GBR_F64) ? 8 : 4;

  // The member lists are small: check them on the host.
  std::vector<int64_t> off(n_cluster + 1);
  if (cudaMemcpy(off.data(), offsets, sizeof(int64_t) * off.size(), cudaMemcpyDefault) != cudaSuccess)
    return h->cuda_fail(cudaGetLastError(), "reading offsets");
  if (off[0] < 0) return h->fail(GBR_ERR_ARG, "offsets[0] is negative");
  for (int64_t c = 0; c < n_cluster; ++c)
    if (off[c + 1] < off[c]) return h->fail(GBR_ERR_ARG, "offsets decrease at cluster %lld", (long long)c);
  const int64_t n_mem = off[n_cluster];
  if (n_mem > 0 && !members) return h->fail(GBR_ERR_ARG, "members must not be NULL");
  std::vector<int32_t> mem(n_mem);
  if (n_mem > 0 && cudaMemcpy(mem.data(), members, sizeof(int32_t) * n_mem, cudaMemcpyDefault) != cudaSuccess)
    return h->cuda_fail(cudaGetLastError(), "reading members");
  for (int64_t k = off[0]; k < n_mem; ++k)
    if (mem[k] < 0 || mem[k] >= n_frame)
      return h->fail(GBR_ERR_ARG, "member %lld is frame %d, outside [0, %lld)", (long long)k, mem[k],
                     (long long)n_frame);
  std::vector<float> wf;
  double W = (double)N;
  if (mass) {
    std::vector<double> w(N);
    if (cudaMemcpy(w.data(), mass, sizeof(double) * N, cudaMemcpyDefault) != cudaSuccess)
      return h->cuda_fail(cudaGetLastError(), "reading mass");
    W = 0.0;
    wf.resize(N);
    for (int i = 0; i < N; ++i) {
      W += w[i];
      wf[i] = (float)w[i];
    }
  }
  if (mode == GBR_FIT && W < 1e-14)
    return h->fail(GBR_ERR_ZERO_MASS, "total mass %g is below 1e-14 (divide by zero)", W);

  const bool x_dev = is_device_ptr(xyz);
  const bool o_dev = is_device_ptr(centroids);
  const size_t out_elems = (size_t)n_cluster * 3 * N;
  auto layout = [&](Arena& A, void** p) {
    p[0] = x_dev ? nullptr : A.take<char>(esz * 3 * (size_t)N * n_frame);
    p[1] = A.take<int64_t>(n_cluster + 1);
    p[2] = A.take<int32_t>(n_mem > 0 ? n_mem : 1);
    p[3] = mass ? A.take<float>(N) : nullptr;
    p[4] = (mode == GBR_FIT) ? A.take<float2>(out_elems) : nullptr;
    p[5] = o_dev ? nullptr : A.take<double>(out_elems);
  };
  void* P[6];
  Arena sizing;
  layout(sizing, P);
  if (!h->reserve(sizing.off + 256))
    return h->fail(GBR_ERR_NOMEM, "cannot allocate %.2f GB of device workspace", (sizing.off + 256) / 1e9);
  Arena A{h->ws, 0};
  layout(A, P);

  if (h->timing) cudaEventRecord(h->ev[0], st);
  if (!x_dev && n_frame > 0) cudaMemcpyAsync(P[0], xyz, esz * 3 * (size_t)N * n_frame, cudaMemcpyDefault, st);
  cudaMemcpyAsync(P[1], off.data(), sizeof(int64_t) * off.size(), cudaMemcpyHostToDevice, st);
  if (n_mem > 0) cudaMemcpyAsync(P[2], mem.data(), sizeof(int32_t) * n_mem, cudaMemcpyHostToDevice, st);
  if (mass) cudaMemcpyAsync(P[3], wf.data(), sizeof(float) * N, cudaMemcpyHostToDevice, st);
  if (h->timing) cudaEventRecord(h->ev[1], st);

  CenArgs a{};
  a.members = (const int32_t*)P[2];
  a.offsets = (const int64_t*)P[1];
  a.w = mass ? (const float*)P[3] : nullptr;
  a.inv_W = 1.0 / W;
  a.inv_Wf = (float)(1.0 / W);
  a.N = N;
  a.S = (float2*)P[4];
  a.out = o_dev ? centroids : (double*)P[5];
  const void* x = x_dev ? xyz : P[0];
  const unsigned grid = (unsigned)n_cluster;
  const int chain_threads = 32 * kChainWarps;
  const size_t stage_bytes = (size_t)3 * N * (sizeof(float2) + kRing * sizeof(float));
  cudaError_t e = cudaSuccess;
  if (mode == GBR_NOFIT) {
    const dim3 g(grid, (unsigned)((3 * N + kSumThreads - 1) / kSumThreads));
    if (dtype == GBR_F64)
      k_centroid_sum<double><<<g, kSumThreads, 0, st>>>((const double*)x, a);
    else
      k_centroid_sum<float><<<g, kSumThreads, 0, st>>>((const float*)x, a);
  } else if (dtype == GBR_F32 && stage_bytes <= kStageMaxBytes) {
    e = cudaFuncSetAttribute(k_centroid_chain<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)stage_bytes);
    if (e != cudaSuccess) return h->cuda_fail(e, "centroid kernel attribute");
    k_centroid_chain<float, true><<<grid, chain_threads, stage_bytes, st>>>((const float*)x, a);
  } else if (dtype == GBR_F32) {
    k_centroid_chain<float, false><<<grid, chain_threads, 0, st>>>((const float*)x, a);
  } else {
    k_centroid_chain<double, false><<<grid, chain_threads, 0, st>>>((const double*)x, a);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return h->cuda_fail(e, "centroid kernel launch");
  if (h->timing) cudaEventRecord(h->ev[2], st);
  if (!o_dev) cudaMemcpyAsync(centroids, P[5], sizeof(double) * out_elems, cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return h->cuda_fail(e, "cluster centroids");
  h->stats.pairs = n_mem;
  h->stats.kernel_launches = 1;
  h->stats.precision = GBR_PREC_FP32;
  if (h->timing) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev[1], h->ev[2]);
    h->stats.ms_pairs = ms;
  }
  return GBR_OK;
}
