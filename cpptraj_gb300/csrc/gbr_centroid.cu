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
// ahead), so the chain does not wait on DRAM.
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

constexpr int kCenThreads = 256;
constexpr int kCenWarps = kCenThreads / 32;
constexpr int kCenNV = 14;  // covariance 9, sum w|y|^2, sum w|S|^2, next centre 3
constexpr int kRing = 4;           // staged members: k, k + 1 in use, k + 2, k + 3 in flight
constexpr int kExactSteps = 32;    // chain steps solved in FP64
constexpr size_t kStageMaxBytes = 200 * 1024;
constexpr int kSumThreads = 256;   // no-fit: one thread per centroid coordinate
constexpr int kSumUnroll = 8;      // members loaded ahead per thread

struct CenArgs {
  const int32_t* members;  // frame indices, clusters back to back
  const int64_t* offsets;  // [n_cluster + 1]
  const float* w;          // [N] masses, nullptr = unweighted
  double inv_W;            // 1 / sum of w (or 1 / N)
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

// Sum of kCenNV floats over the block; the totals land in tot[] (visible to
// every thread after the call).  red: [kCenWarps][16].
__device__ __forceinline__ void block_sum_nv(float (&v)[kCenNV], float (*red)[16], float* tot) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kCenNV; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < kCenNV; ++k) red[warp][k] = v[k];
  }
  __syncthreads();
  if (warp == 0 && lane < kCenNV) {
    float s = 0.0f;
#pragma unroll
    for (int q = 0; q < kCenWarps; ++q) s += red[q][lane];
    tot[lane] = s;
  }
  __syncthreads();
}

// Warp sums of 16 values in 16 shuffles (each round keeps half of the values
// and trades the other half with the partner lane).  On return v[0] of lane
// l holds the warp's total of value index
//   8 * bit4(l) + 4 * bit3(l) + 2 * bit2(l) + bit1(l).
__device__ __forceinline__ void warp_sum16(float (&v)[16], int lane) {
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int h = 8 >> r;         // values kept after this round
    const int o = 16 >> r;        // partner lane distance
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int j = 0; j < h; ++j) {
      const float send = up ? v[j] : v[j + h];
      const float keep = up ? v[j + h] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
}

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

// Fitted centroids, one CTA per cluster.  STAGE (FP32 frames, the running
// sum and kRing frames fitting kStageMaxBytes of shared memory): S lives in
// shared memory (the sweeps re-read it every step; global stores do not stay
// in L1) and frames come through a ring of kRing shared-memory buffers,
// member k + 3 issued while member k is fitted, so the chain never waits on
// DRAM.  Otherwise S is in global memory and frames are read from there.
template <typename T, bool STAGE>
__global__ void __launch_bounds__(kCenThreads) k_centroid_chain(const T* __restrict__ xyz, CenArgs a) {
  extern __shared__ float4 dyn[];
  __shared__ float red[kCenWarps][16];
  __shared__ float tot[kCenNV];
  __shared__ float bc[21];  // U as FP32 hi (9) and lo (9) parts, row-major; centre of the next member
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, N = a.N;
  const int64_t cl = blockIdx.x;
  const int64_t o0 = a.offsets[cl], n = a.offsets[cl + 1] - o0;
  double* out = a.out + (size_t)cl * 3 * N;
  if (n <= 0) {  // the reference's centroid has no atoms
    for (int i = tid; i < 3 * N; i += kCenThreads) out[i] = qnan();
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
        for (int i = tid; i < N; i += kCenThreads) {
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

  int32_t f_ahead = 0;  // frame of member k + kRing, loaded one step before its copy is issued
  if constexpr (STAGE) {
#pragma unroll
    for (int k = 0; k < kRing; ++k) stage(k, k < n ? mem[k] : 0);
    f_ahead = (kRing < n) ? mem[kRing] : 0;
    cp_async_wait<kRing - 2>();  // members 0 and 1 are in
  }
  // Centres of members 0 and 1 (one reduction), then S = member 0 centred.
  float v[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = 0.0f;
  for (int i = tid; i < N; i += kCenThreads) {
    float p[3], r[3];
    get(0, i, p);
    get(n > 1 ? 1 : 0, i, r);
    const float wi = wt(i);
    v[0] += wi * p[0]; v[1] += wi * p[1]; v[2] += wi * p[2];
    v[11] += wi * r[0]; v[12] += wi * r[1]; v[13] += wi * r[2];
  }
  {
    float v14[kCenNV];
#pragma unroll
    for (int q = 0; q < kCenNV; ++q) v14[q] = v[q];
    block_sum_nv(v14, red, tot);
  }
  float c[3] = {(float)((double)tot[0] * a.inv_W), (float)((double)tot[1] * a.inv_W),
                (float)((double)tot[2] * a.inv_W)};
  float cn[3] = {(float)((double)tot[11] * a.inv_W), (float)((double)tot[12] * a.inv_W),
                 (float)((double)tot[13] * a.inv_W)};
  for (int i = tid; i < N; i += kCenThreads) {
    float p[3];
    get(0, i, p);
#pragma unroll
    for (int q = 0; q < 3; ++q) S[3 * i + q] = make_float2(p[q] - c[q], 0.0f);
  }
  for (int64_t k = 1; k < n; ++k) {
    c[0] = cn[0]; c[1] = cn[1]; c[2] = cn[2];
    if constexpr (STAGE) {
      // Buffer (k + kRing - 1) % kRing held member k - 1, which this thread
      // last read in the previous step.
      const int32_t f = f_ahead;
      f_ahead = (k + kRing < n) ? mem[k + kRing] : 0;
      stage(k + kRing - 1, f);
      cp_async_wait<kRing - 2>();  // members k and k + 1 are in
    }
    const bool has_next = (k + 1 < n);
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = 0.0f;
    for (int i = tid; i < N; i += kCenThreads) {
      float y[3], s[3];
      get(k, i, y);
      const float wi = wt(i);
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        y[q] -= c[q];
        s[q] = S[3 * i + q].x;
      }
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        const float wy = wi * y[p];
        v[3 * p] += wy * s[0];
        v[3 * p + 1] += wy * s[1];
        v[3 * p + 2] += wy * s[2];
      }
      v[9] += wi * (y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
      v[10] += wi * (s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
      if (has_next) {
        float r[3];
        get(k + 1, i, r);
        v[11] += wi * r[0]; v[12] += wi * r[1]; v[13] += wi * r[2];
      }
    }
    // Block totals for the solving thread only: warp sums, one barrier, and
    // warp 0 adds the warps' partials.
    warp_sum16(v, lane);
    if ((lane & 1) == 0) red[warp][((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 +
                                   ((lane >> 1) & 1)] = v[0];
    __syncthreads();
    if (warp == 0) {
      float t = 0.0f;
      if (lane < kCenNV) {
#pragma unroll
        for (int q = 0; q < kCenWarps; ++q) t += red[q][lane];
      }
      float ts[kCenNV];
#pragma unroll
      for (int q = 0; q < kCenNV; ++q) ts[q] = __shfl_sync(0xffffffffu, t, q);
      if (lane == 0) {
        if (k <= kExactSteps) {
          // FP64 solve, U out as hi + lo: the first members' turns set the
          // orientation of the whole centroid, and an FP32-rounded U would
          // turn each of them by ~1e-7 rad.
          const double ik = 1.0 / (double)k;
          double A[9], U[9];
#pragma unroll
          for (int q = 0; q < 9; ++q) A[q] = (double)ts[q] * ik;
          const double E0 = 0.5 * ((double)ts[9] + (double)ts[10] * ik * ik);
          qcp_lambda_rot(A, E0, U);
#pragma unroll
          for (int q = 0; q < 9; ++q) {
            const float hi = (float)U[q];
            bc[q] = hi;
            bc[9 + q] = (float)(U[q] - (double)hi);
          }
        } else {
          // FP32 solve: a later member moves the sum by 1/k of its own
          // weight, so its rotation error averages out.
          const float ik = __fdividef(1.0f, (float)k);
          float M[9], U[9];
#pragma unroll
          for (int q = 0; q < 9; ++q) M[q] = ts[q] * ik;
          qcp_rot_f32(M, 0.5f * (ts[9] + ts[10] * ik * ik), U);
#pragma unroll
          for (int q = 0; q < 9; ++q) {
            bc[q] = U[q];
            bc[9 + q] = 0.0f;
          }
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) bc[18 + q] = (float)((double)ts[11 + q] * a.inv_W);
      }
    }
    __syncthreads();
    float Uh[9], Ul[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      Uh[q] = bc[q];
      Ul[q] = bc[9 + q];
    }
    cn[0] = bc[18]; cn[1] = bc[19]; cn[2] = bc[20];
    for (int i = tid; i < N; i += kCenThreads) {
      float y[3];
      get(k, i, y);
#pragma unroll
      for (int q = 0; q < 3; ++q) y[q] -= c[q];
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        const float lo = Ul[3 * p] * y[0] + Ul[3 * p + 1] * y[1] + Ul[3 * p + 2] * y[2];
        const float r = fmaf(Uh[3 * p], y[0], fmaf(Uh[3 * p + 1], y[1], fmaf(Uh[3 * p + 2], y[2], lo)));
        S[3 * i + p] = add_hl(S[3 * i + p], r);
      }
    }
    // bc and red are rewritten only after the next step's first barrier,
    // which every thread reaches after reading them here.
  }
  if constexpr (STAGE) cp_async_wait<0>();
  // The sums were written per atom (thread t: elements 3t..3t+2); they are
  // read per element below.
  __syncthreads();
  const double inv_n = 1.0 / (double)n;
  for (int i = tid; i < 3 * N; i += kCenThreads) {
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
  a.N = N;
  a.S = (float2*)P[4];
  a.out = o_dev ? centroids : (double*)P[5];
  const void* x = x_dev ? xyz : P[0];
  const unsigned grid = (unsigned)n_cluster;
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
    k_centroid_chain<float, true><<<grid, kCenThreads, stage_bytes, st>>>((const float*)x, a);
  } else if (dtype == GBR_F32) {
    k_centroid_chain<float, false><<<grid, kCenThreads, 0, st>>>((const float*)x, a);
  } else {
    k_centroid_chain<double, false><<<grid, kCenThreads, 0, st>>>((const double*)x, a);
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
