// gbr_prep.cu -- per-frame passes that run before the pair contraction (K1).
//
// Every per-frame pass runs one warp per frame (8 frames per 256-thread
// block, many frames in flight per SM) with FP32 per-lane partial sums and an
// FP64 warp reduction; the per-frame 3x3 solves run on lane 0 in FP64.
//
//   k_centroid     centre of each frame: Frame::CenterOnOrigin / the target
//                  centring of Frame::RMSD_CenteredRef (src/Frame.cpp:1043-1055,
//                  1142-1171); reference frames use the reference masses.
//   k_make_ref     builds pre-alignment reference k from one frame, superposed
//                  onto an existing reference so all references share an
//                  orientation.
//   k_ref_dist     fit (or no-fit) RMSD of every frame to reference k, keeping
//                  the nearest reference per frame (greedy k-centre selection).
//   k_align        superposes every frame onto its reference with an exact FP64
//                  rotation and writes p = sqrt(w)*(R y - r) (FP32, [F][3][Np]).
//   k_ref_mean_*   mean of p over each reference's frames (two fixed-order stages).
//   k_ref_update   moves each reference to the mean of its frames.
//   k_finish       p -= mean; for the tensor path splits p into FP16 hi/lo with
//                  a per-frame power-of-two scale; n_f and P_fc from the exact
//                  operand values the contraction will read.
//   k_ref_terms    per reference pair: exact rotation U_ab, U_ab S_ba, and
//                  sum w |r_a - U_ab r_b|^2.
#include <cuda_fp16.h>

#include <vector>

#include "gbr_common.cuh"
#include "gbr_internal.h"

namespace gbr {

template <typename T>
struct FrameSrc {
  const T* ref;
  const T* tgt;
  int64_t n_ref;
  int N;
  __device__ __forceinline__ const T* frame(int64_t f) const {
    return (f < n_ref) ? ref + (size_t)f * 3 * N : tgt + (size_t)(f - n_ref) * 3 * N;
  }
};

constexpr int kPrepThreads = 256;
constexpr int kWarps = kPrepThreads / 32;

template <int NV>
__device__ __forceinline__ void warp_sum_f64(double (&v)[NV]) {
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

// Largest eigenvalue of the QCP key matrix only (Newton from E0, FP64).
__device__ inline double qcp_lambda(const double A[9], double E0) {
  const double xx = A[0], xy = A[1], xz = A[2], yx = A[3], yy = A[4], yz = A[5], zx = A[6],
               zy = A[7], zz = A[8];
  const double xx2 = xx * xx, yy2 = yy * yy, zz2 = zz * zz, xy2 = xy * xy, yz2 = yz * yz,
               xz2 = xz * xz, yx2 = yx * yx, zy2 = zy * zy, zx2 = zx * zx;
  const double c2 = -2.0 * (xx2 + yy2 + zz2 + xy2 + yx2 + xz2 + zx2 + yz2 + zy2);
  const double c1 = 8.0 * (xx * yz * zy + yy * zx * xz + zz * xy * yx - xx * yy * zz - yz * zx * xy -
                           zy * yx * xz);
  const double t1 = 2.0 * (yz * zy - yy * zz);
  const double t2 = yy2 + zz2 - xx2 + yz2 + zy2;
  const double t3 = xy2 + xz2 - yx2 - zx2;
  const double pxz = xz + zx, pyz = yz + zy, pxy = xy + yx, myz = yz - zy, mxz = xz - zx,
               mxy = xy - yx, pxx = xx + yy, mxx = xx - yy;
  const double c0 = t3 * t3 + (t2 + t1) * (t2 - t1) +
                    (-pxz * myz + mxy * (mxx - zz)) * (-mxz * pyz + mxy * (mxx + zz)) +
                    (-pxz * pyz - pxy * (pxx - zz)) * (-mxz * myz - pxy * (pxx + zz)) +
                    (pxy * pyz + pxz * (mxx + zz)) * (-mxy * myz + pxz * (pxx + zz)) +
                    (pxy * myz + mxz * (mxx - zz)) * (-mxy * pyz + mxz * (pxx - zz));
  double lam = E0;
  for (int it = 0; it < 50; ++it) {
    const double prev = lam, l2 = lam * lam, b = (l2 + c2) * lam, a = b + c1;
    const double den = 2.0 * l2 * lam + b + a;
    if (den == 0.0) break;
    lam -= (a * lam + c0) / den;
    if (fabs(lam - prev) < fabs(1e-11 * lam)) break;
  }
  return lam;
}

template <typename T>
__global__ void __launch_bounds__(kPrepThreads) k_centroid(FrameSrc<T> src, int64_t F,
                                                           const double* cmass_ref,
                                                           const double* cmass_tgt, double* cen) {
  const int lane = threadIdx.x & 31;
  for (int64_t f = blockIdx.x * (int64_t)kWarps + (threadIdx.x >> 5); f < F; f += (int64_t)gridDim.x * kWarps) {
    const T* x = src.frame(f);
    const double* m = (f < src.n_ref) ? cmass_ref : cmass_tgt;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, sm = 0.f;
    for (int a = lane; a < src.N; a += 32) {
      const float w = m ? (float)m[a] : 1.0f;
      s0 += w * (float)x[3 * a];
      s1 += w * (float)x[3 * a + 1];
      s2 += w * (float)x[3 * a + 2];
      sm += w;
    }
    double v[4] = {s0, s1, s2, sm};
    warp_sum_f64<4>(v);
    if (lane == 0) {
      double wt = m ? v[3] : (double)src.N;
      if (m && wt == 0.0) {  // zero total mass: centre at the origin, as VCenterOfMass does
        wt = 1.0;
        v[0] = v[1] = v[2] = 0.0;
      }
      cen[3 * f] = v[0] / wt;
      cen[3 * f + 1] = v[1] / wt;
      cen[3 * f + 2] = v[2] / wt;
    }
  }
}

// Reference k := frame f centred (and superposed onto reference `parent` when
// fitting and parent >= 0).  Also writes sqrt(w)*r_k in FP32 and sum w |r_k|^2.
template <typename T>
__global__ void __launch_bounds__(kPrepThreads) k_make_ref(FrameSrc<T> src, const int64_t* fsel,
                                                           const double* cen, const double* w,
                                                           const int* assign, int k, int use_parent,
                                                           int nofit, double* refs, float* swr,
                                                           double* Eref) {
  __shared__ double red[32 * 10];
  __shared__ double Rs[9];
  const int N = src.N;
  const int64_t f = *fsel;
  const T* x = src.frame(f);
  const double c0 = cen[3 * f], c1 = cen[3 * f + 1], c2 = cen[3 * f + 2];
  double* rk = refs + (size_t)k * 3 * N;
  if (threadIdx.x < 9) Rs[threadIdx.x] = (threadIdx.x % 4 == 0) ? 1.0 : 0.0;
  __syncthreads();
  const int parent = use_parent ? assign[f] : -1;
  if (!nofit && parent >= 0) {
    const double* rp = refs + (size_t)parent * 3 * N;
    double v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = threadIdx.x; a < N; a += blockDim.x) {
      const double wa = w ? w[a] : 1.0;
      const double y0 = (double)x[3 * a] - c0, y1 = (double)x[3 * a + 1] - c1, y2 = (double)x[3 * a + 2] - c2;
      const double r0 = rp[3 * a], r1 = rp[3 * a + 1], r2 = rp[3 * a + 2];
      v[0] += wa * y0 * r0; v[1] += wa * y0 * r1; v[2] += wa * y0 * r2;
      v[3] += wa * y1 * r0; v[4] += wa * y1 * r1; v[5] += wa * y1 * r2;
      v[6] += wa * y2 * r0; v[7] += wa * y2 * r1; v[8] += wa * y2 * r2;
      v[9] += wa * (y0 * y0 + y1 * y1 + y2 * y2 + r0 * r0 + r1 * r1 + r2 * r2);
    }
    block_sum_f64<10>(v, red);
    if (threadIdx.x == 0) {
      double R[9];
      qcp_lambda_rot(v, 0.5 * v[9], R);
      for (int q = 0; q < 9; ++q) Rs[q] = R[q];
    }
    __syncthreads();
  }
  double e = 0.0;
  for (int a = threadIdx.x; a < N; a += blockDim.x) {
    const double wa = w ? w[a] : 1.0;
    const double y0 = (double)x[3 * a] - c0, y1 = (double)x[3 * a + 1] - c1, y2 = (double)x[3 * a + 2] - c2;
    const double r0 = Rs[0] * y0 + Rs[1] * y1 + Rs[2] * y2;
    const double r1 = Rs[3] * y0 + Rs[4] * y1 + Rs[5] * y2;
    const double r2 = Rs[6] * y0 + Rs[7] * y1 + Rs[8] * y2;
    rk[3 * a] = r0; rk[3 * a + 1] = r1; rk[3 * a + 2] = r2;
    const double sw = sqrt(wa);
    float* s = swr + ((size_t)k * N + a) * 3;
    s[0] = (float)(sw * r0); s[1] = (float)(sw * r1); s[2] = (float)(sw * r2);
    e += wa * (r0 * r0 + r1 * r1 + r2 * r2);
  }
  double ev[1] = {e};
  block_sum_f64<1>(ev, red);
  if (threadIdx.x == 0) Eref[k] = ev[0];
}

// Distance of every frame to reference k; keeps the minimum and its index.
template <typename T>
__global__ void __launch_bounds__(kPrepThreads) k_ref_dist(FrameSrc<T> src, int64_t F, const double* cen,
                                                           const float* sqwf, double Wsum, const float* swr,
                                                           const double* Eref, int k, int nofit, float* dist,
                                                           int* assign) {
  const int N = src.N, lane = threadIdx.x & 31;
  const float* rk = swr + (size_t)k * 3 * N;  // sqrt(w) r_k
  for (int64_t f = blockIdx.x * (int64_t)kWarps + (threadIdx.x >> 5); f < F; f += (int64_t)gridDim.x * kWarps) {
    const T* x = src.frame(f);
    const float c0 = (float)cen[3 * f], c1 = (float)cen[3 * f + 1], c2 = (float)cen[3 * f + 2];
    float h[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = lane; a < N; a += 32) {
      const float sw = sqwf ? sqwf[a] : 1.0f;
      const float y0 = sw * ((float)x[3 * a] - c0), y1 = sw * ((float)x[3 * a + 1] - c1),
                  y2 = sw * ((float)x[3 * a + 2] - c2);
      const float r0 = rk[3 * a], r1 = rk[3 * a + 1], r2 = rk[3 * a + 2];
      if (nofit) {
        const float d0 = y0 - r0, d1 = y1 - r1, d2 = y2 - r2;
        h[9] += d0 * d0 + d1 * d1 + d2 * d2;
      } else {
        h[0] += y0 * r0; h[1] += y0 * r1; h[2] += y0 * r2;
        h[3] += y1 * r0; h[4] += y1 * r1; h[5] += y1 * r2;
        h[6] += y2 * r0; h[7] += y2 * r1; h[8] += y2 * r2;
        h[9] += y0 * y0 + y1 * y1 + y2 * y2;
      }
    }
    double v[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) v[q] = h[q];
    warp_sum_f64<10>(v);
    if (lane == 0) {
      double d2;
      if (nofit) {
        d2 = v[9] / Wsum;
      } else {
        const double E0 = 0.5 * (v[9] + Eref[k]);
        d2 = 2.0 * (E0 - qcp_lambda(v, E0)) / Wsum;
      }
      const float d = (float)sqrt(fmax(d2, 0.0));
      if (k == 0 || d < dist[f]) {
        dist[f] = d;
        assign[f] = k;
      }
    }
  }
}

// Single-block argmax of dist[0..F): out_val, out_idx.
__global__ void k_argmax(const float* dist, int64_t F, float* out_val, int64_t* out_idx) {
  __shared__ float sv[1024];
  __shared__ int64_t si[1024];
  float bv = -1.0f;
  int64_t bi = 0;
  for (int64_t f = threadIdx.x; f < F; f += blockDim.x) {
    const float v = dist[f];
    if (v > bv) { bv = v; bi = f; }
  }
  sv[threadIdx.x] = bv;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const float o = sv[threadIdx.x + s];
      const int64_t oi = si[threadIdx.x + s];
      if (o > sv[threadIdx.x] || (o == sv[threadIdx.x] && oi < si[threadIdx.x])) {
        sv[threadIdx.x] = o;
        si[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *out_val = sv[0];
    *out_idx = si[0];
  }
}

// Superpose every frame onto its reference (exact FP64 rotation) and write
// p = sqrt(w) * (R y - r_a) as the FP32 operand plane (zero past N).
template <typename T>
__global__ void __launch_bounds__(kPrepThreads) k_align(FrameSrc<T> src, int64_t F, int Np,
                                                        const double* cen, const float* sqwf,
                                                        const double* sqw, const double* refs,
                                                        const float* swr, const int* assign, int nofit,
                                                        double* rot, float* plane) {
  const int N = src.N, lane = threadIdx.x & 31;
  for (int64_t f = blockIdx.x * (int64_t)kWarps + (threadIdx.x >> 5); f < F; f += (int64_t)gridDim.x * kWarps) {
    const T* x = src.frame(f);
    const int a_ref = assign[f];
    const double* ra = refs + (size_t)a_ref * 3 * N;
    const float* rs = swr + (size_t)a_ref * 3 * N;
    const double c0 = cen[3 * f], c1 = cen[3 * f + 1], c2 = cen[3 * f + 2];
    double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (!nofit) {
      float h[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
      const float fc0 = (float)c0, fc1 = (float)c1, fc2 = (float)c2;
      for (int a = lane; a < N; a += 32) {
        const float sw = sqwf ? sqwf[a] : 1.0f;
        const float y0 = sw * ((float)x[3 * a] - fc0), y1 = sw * ((float)x[3 * a + 1] - fc1),
                    y2 = sw * ((float)x[3 * a + 2] - fc2);
        const float r0 = rs[3 * a], r1 = rs[3 * a + 1], r2 = rs[3 * a + 2];
        h[0] += y0 * r0; h[1] += y0 * r1; h[2] += y0 * r2;
        h[3] += y1 * r0; h[4] += y1 * r1; h[5] += y1 * r2;
        h[6] += y2 * r0; h[7] += y2 * r1; h[8] += y2 * r2;
        h[9] += y0 * y0 + y1 * y1 + y2 * y2 + r0 * r0 + r1 * r1 + r2 * r2;
      }
      double v[10];
#pragma unroll
      for (int q = 0; q < 10; ++q) v[q] = h[q];
      warp_sum_f64<10>(v);
      if (lane == 0) {
        // Any exact rotation keeps every pairwise RMSD; the optimal one only
        // makes d small.  So the eigenvector comes from FP32 QCP and the
        // rotation is built (orthogonal to FP64 rounding) from it.
        float M[9], q[4] = {1.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int k = 0; k < 9; ++k) M[k] = (float)v[k];
        const float E0 = (float)(0.5 * v[9]);
        if (E0 > 0.0f) qcp_vec_f32(M, E0, q);
        rotation_from_quat(q, R);
      }
#pragma unroll
      for (int q = 0; q < 9; ++q) R[q] = __shfl_sync(0xffffffffu, R[q], 0);
    }
    if (lane < 9 && rot) rot[9 * f + lane] = R[lane];
    float* pl = plane + (size_t)f * 3 * Np;
    for (int a = lane; a < Np; a += 32) {
      float p0 = 0.f, p1 = 0.f, p2 = 0.f;
      if (a < N) {
        const double y0 = (double)x[3 * a] - c0, y1 = (double)x[3 * a + 1] - c1, y2 = (double)x[3 * a + 2] - c2;
        const double sw = sqw ? sqw[a] : 1.0;
        p0 = (float)(sw * (R[0] * y0 + R[1] * y1 + R[2] * y2 - ra[3 * a]));
        p1 = (float)(sw * (R[3] * y0 + R[4] * y1 + R[5] * y2 - ra[3 * a + 1]));
        p2 = (float)(sw * (R[6] * y0 + R[7] * y1 + R[8] * y2 - ra[3 * a + 2]));
      }
      pl[a] = p0;
      pl[Np + a] = p1;
      pl[2 * Np + a] = p2;
    }
  }
}

// p -= mean[a(f)]; then, for the tensor path, split p into FP16 hi + lo with
// a per-frame scale s_f = 2^(14 - e), e = exponent of max |p| (so hi stays
// below 2^15), and use the value hi + lo represents from here on.  Writes
// n_f = sum |p|^2 and P_fc = sum p (sqrt(w) r_c)^T for every reference c.
__global__ void __launch_bounds__(kPrepThreads) k_finish(float* plane, int64_t F, int Np, int N, const float* mean,
                                                         const int* assign, int K, const float* swr, int tc,
                                                         __half* hi, __half* lo, float* inv_scale,
                                                         int write_plane, float* nrm, float* P, float* trP) {
  const int lane = threadIdx.x & 31;
  for (int64_t f = blockIdx.x * (int64_t)kWarps + (threadIdx.x >> 5); f < F; f += (int64_t)gridDim.x * kWarps) {
    float* pl = plane + (size_t)f * 3 * Np;
    const float* mu = mean + (size_t)assign[f] * 3 * Np;
    float scale = 1.0f, inv = 1.0f;
    if (tc) {
      float m = 0.0f;
      for (int a = lane; a < N; a += 32)
#pragma unroll
        for (int p = 0; p < 3; ++p) m = fmaxf(m, fabsf(pl[p * Np + a] - mu[p * Np + a]));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
      int e = 0;
      if (m > 0.0f) frexpf(m, &e);
      scale = ldexpf(1.0f, 14 - e);
      inv = ldexpf(1.0f, e - 14);
      if (lane == 0) inv_scale[f] = inv;
    }
    // pass over atoms: final operand values, written planes, n_f
    float n = 0.0f;
    for (int a = lane; a < Np; a += 32) {
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        float v = (a < N) ? pl[p * Np + a] - mu[p * Np + a] : 0.0f;
        if (tc) {
          const float t = v * scale;
          const __half h = __float2half_rn(t);
          const __half l = __float2half_rn(t - __half2float(h));
          hi[(size_t)f * 3 * Np + (size_t)p * Np + a] = h;
          lo[(size_t)f * 3 * Np + (size_t)p * Np + a] = l;
          v = (__half2float(h) + __half2float(l)) * inv;
        }
        if (write_plane || tc) pl[p * Np + a] = v;
        n += v * v;
      }
    }
    double nv[1] = {n};
    warp_sum_f64<1>(nv);
    if (lane == 0) nrm[f] = (float)nv[0];
    __syncwarp();
    for (int c = 0; c < K; ++c) {
      const float* rc = swr + (size_t)c * N * 3;
      float h[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int a = lane; a < N; a += 32) {
        const float p0 = pl[a], p1 = pl[Np + a], p2 = pl[2 * Np + a];
        const float r0 = rc[3 * a], r1 = rc[3 * a + 1], r2 = rc[3 * a + 2];
        h[0] += p0 * r0; h[1] += p0 * r1; h[2] += p0 * r2;
        h[3] += p1 * r0; h[4] += p1 * r1; h[5] += p1 * r2;
        h[6] += p2 * r0; h[7] += p2 * r1; h[8] += p2 * r2;
      }
      double v[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) v[q] = h[q];
      warp_sum_f64<9>(v);
      if (lane == 0) {
        float* Pf = P + ((size_t)f * K + c) * 9;
        for (int q = 0; q < 9; ++q) Pf[q] = (float)v[q];
        trP[(size_t)f * K + c] = (float)(v[0] + v[4] + v[8]);
      }
    }
  }
}

// Reference-pair table (kRefPairStride floats per b*K + a): the exact FP64
// rotation U_ab taking r_b onto r_a, SU_ab = U_ab S_ba, its antisymmetric
// combos and sum w |r_a - U_ab r_b|^2.  No-fit mode keeps U = I.
__global__ void __launch_bounds__(kPrepThreads) k_ref_terms(const double* refs, int N, int K, const double* w,
                                                            int nofit, float* RP) {
  __shared__ double red[32 * 10];
  __shared__ double Us[9];
  const int b = blockIdx.x / K, a = blockIdx.x % K;
  const double* rb = refs + (size_t)b * 3 * N;
  const double* ra = refs + (size_t)a * 3 * N;
  double v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double wa = w ? w[i] : 1.0;
    const double b0 = rb[3 * i], b1 = rb[3 * i + 1], b2 = rb[3 * i + 2];
    const double a0 = ra[3 * i], a1 = ra[3 * i + 1], a2 = ra[3 * i + 2];
    v[0] += wa * b0 * a0; v[1] += wa * b0 * a1; v[2] += wa * b0 * a2;
    v[3] += wa * b1 * a0; v[4] += wa * b1 * a1; v[5] += wa * b1 * a2;
    v[6] += wa * b2 * a0; v[7] += wa * b2 * a1; v[8] += wa * b2 * a2;
    v[9] += wa * (b0 * b0 + b1 * b1 + b2 * b2 + a0 * a0 + a1 * a1 + a2 * a2);
  }
  block_sum_f64<10>(v, red);
  if (threadIdx.x == 0) {
    double U[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (a != b && !nofit) qcp_lambda_rot(v, 0.5 * v[9], U);
    for (int k = 0; k < 9; ++k) Us[k] = U[k];
  }
  __syncthreads();
  // SS_ab = sum w |r_a - U r_b|^2, accumulated directly (no cancellation).
  double e[1] = {0.0};
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double wa = w ? w[i] : 1.0;
    const double b0 = rb[3 * i], b1 = rb[3 * i + 1], b2 = rb[3 * i + 2];
    const double d0 = ra[3 * i] - (Us[0] * b0 + Us[1] * b1 + Us[2] * b2);
    const double d1 = ra[3 * i + 1] - (Us[3] * b0 + Us[4] * b1 + Us[5] * b2);
    const double d2 = ra[3 * i + 2] - (Us[6] * b0 + Us[7] * b1 + Us[8] * b2);
    e[0] += wa * (d0 * d0 + d1 * d1 + d2 * d2);
  }
  block_sum_f64<1>(e, red);
  if (threadIdx.x == 0) {
    double SU[9];
    for (int p = 0; p < 3; ++p)
      for (int q = 0; q < 3; ++q)
        SU[p * 3 + q] = Us[p * 3] * v[q] + Us[p * 3 + 1] * v[3 + q] + Us[p * 3 + 2] * v[6 + q];
    float* o = RP + (size_t)blockIdx.x * kRefPairStride;
    for (int k = 0; k < 9; ++k) o[k] = (float)Us[k];
    for (int k = 0; k < 9; ++k) o[9 + k] = (float)SU[k];
    o[18] = (float)(SU[5] - SU[7]);
    o[19] = (float)(SU[6] - SU[2]);
    o[20] = (float)(SU[1] - SU[3]);
    o[21] = (float)((a == b) ? 0.0 : e[0]);
    o[22] = 0.f;
    o[23] = 0.f;
  }
}

__global__ void k_sqrt(const double* w, double* sqw, float* sqwf, int n) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a < n) {
    const double v = sqrt(w[a]);
    sqw[a] = v;
    sqwf[a] = (float)v;
  }
}

// Frames grouped by reference when every frame has reference 0.
__global__ void k_iota(int* order, int* offsets, int64_t F) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < F; f += (int64_t)gridDim.x * blockDim.x)
    order[f] = (int)f;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    offsets[0] = 0;
    offsets[1] = (int)F;
  }
}

// Mean of the operand plane over the frames of each reference, in two
// deterministic stages: partial sums over chunks of a reference's frame list
// (grid.y = chunk, grid.z = reference), then a fixed-order sum of the chunks.
constexpr int kMeanChunks = 64;
__global__ void k_ref_mean_partial(const float* plane, int64_t cols, const int* order, const int* offsets,
                                   float* partial) {
  const int k = blockIdx.z, ch = blockIdx.y;
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const int lo = offsets[k], hi = offsets[k + 1];
  const int per = (hi - lo + kMeanChunks - 1) / kMeanChunks;
  const int a = lo + ch * per, b = min(hi, a + per);
  float s = 0.0f;
  for (int n = a; n < b; ++n) s += plane[(size_t)order[n] * cols + c];
  partial[((size_t)k * kMeanChunks + ch) * cols + c] = s;
}
__global__ void k_ref_mean_final(const float* partial, int64_t cols, const int* offsets, float* mean) {
  const int k = blockIdx.y;
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const int cnt = offsets[k + 1] - offsets[k];
  double s = 0.0;
  for (int ch = 0; ch < kMeanChunks; ++ch) s += (double)partial[((size_t)k * kMeanChunks + ch) * cols + c];
  mean[(size_t)k * cols + c] = (cnt > 0) ? (float)(s / (double)cnt) : 0.0f;
}

// r_k += mean_k / sqrt(w) (FP64), and the derived sqrt(w) r_k, sum w |r_k|^2.
__global__ void __launch_bounds__(kPrepThreads) k_ref_update(double* refs, float* swr, double* Eref,
                                                             const float* mean, const double* w, int N, int Np) {
  __shared__ double red[32];
  const int k = blockIdx.x;
  double* r = refs + (size_t)k * 3 * N;
  const float* m = mean + (size_t)k * 3 * Np;
  double e = 0.0;
  for (int a = threadIdx.x; a < N; a += blockDim.x) {
    const double wa = w ? w[a] : 1.0;
    const double sw = sqrt(wa);
    for (int p = 0; p < 3; ++p) {
      if (sw > 0.0) r[3 * a + p] += (double)m[(size_t)p * Np + a] / sw;
      swr[((size_t)k * N + a) * 3 + p] = (float)(sw * r[3 * a + p]);
    }
    e += wa * (r[3 * a] * r[3 * a] + r[3 * a + 1] * r[3 * a + 1] + r[3 * a + 2] * r[3 * a + 2]);
  }
  double ev[1] = {e};
  block_sum_f64<1>(ev, red);
  if (threadIdx.x == 0) Eref[k] = ev[0];
}

// ---------------------------------------------------------------------------
// Host driver for the prep passes.
// ---------------------------------------------------------------------------
template <typename T>
static cudaError_t prep_impl(const PrepArgs& A, PrepOut& o, cudaStream_t st) {
  FrameSrc<T> src{(const T*)A.ref, (const T*)(A.tgt ? A.tgt : A.ref), A.n_ref, A.N};
  const int64_t F = A.F;
  const int grid = (int)std::min<int64_t>((F + kWarps - 1) / kWarps, 152 * 16);
  int launches = 0;
  if (A.nofit) {
    cudaMemsetAsync(A.cen, 0, sizeof(double) * 3 * F, st);
  } else {
    k_centroid<T><<<grid, kPrepThreads, 0, st>>>(src, F, A.cmass_ref, A.cmass_tgt, A.cen);
    ++launches;
  }
  if (A.centroid_only) {
    o.K = 0;
    o.launches = launches;
    return cudaGetLastError();
  }
  if (A.w) {
    k_sqrt<<<(A.N + 255) / 256, 256, 0, st>>>(A.w, A.sqw, A.sqwf, A.N);
    ++launches;
  }
  const float* sqwf = A.w ? A.sqwf : nullptr;
  const double* sqw = A.w ? A.sqw : nullptr;
  // Greedy k-centre choice of pre-alignment references.
  cudaMemsetAsync(A.fsel, 0, sizeof(int64_t), st);
  k_make_ref<T><<<1, kPrepThreads, 0, st>>>(src, A.fsel, A.cen, A.w, A.assign, 0, 0, A.nofit, A.refs, A.swr,
                                            A.Eref);
  if (A.max_refs > 1) {
    k_ref_dist<T><<<grid, kPrepThreads, 0, st>>>(src, F, A.cen, sqwf, A.Wsum, A.swr, A.Eref, 0, A.nofit, A.dist,
                                                 A.assign);
    ++launches;
  } else {
    cudaMemsetAsync(A.assign, 0, sizeof(int) * F, st);  // one reference: every frame uses it
  }
  ++launches;
  int K = 1;
  while (K < A.max_refs && F > 1) {
    k_argmax<<<1, 1024, 0, st>>>(A.dist, F, A.dmax, A.fsel);
    ++launches;
    float dmax = 0.0f;
    cudaMemcpyAsync(&dmax, A.dmax, sizeof(float), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    if (!(dmax > A.tau)) break;
    k_make_ref<T><<<1, kPrepThreads, 0, st>>>(src, A.fsel, A.cen, A.w, A.assign, K, 1, A.nofit, A.refs, A.swr,
                                              A.Eref);
    k_ref_dist<T><<<grid, kPrepThreads, 0, st>>>(src, F, A.cen, sqwf, A.Wsum, A.swr, A.Eref, K, A.nofit, A.dist,
                                                 A.assign);
    launches += 2;
    ++K;
  }
  o.K = K;
  k_align<T><<<grid, kPrepThreads, 0, st>>>(src, F, A.Np, A.cen, sqwf, sqw, A.refs, A.swr, A.assign, A.nofit,
                                            A.rot, A.plane);
  ++launches;
  // Refine every reference to the mean of its superposed frames: residuals
  // shrink to each frame's own fluctuation.  With several references the
  // frames are grouped by reference with a host-side counting sort.
  if (K == 1) {
    k_iota<<<(int)std::min<int64_t>((F + 255) / 256, 1024), 256, 0, st>>>(A.order, A.offsets, F);
    ++launches;
  } else {
    std::vector<int> asg(F), order(F), offsets(K + 1, 0);
    cudaMemcpyAsync(asg.data(), A.assign, sizeof(int) * F, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    for (int64_t f = 0; f < F; ++f) offsets[asg[f] + 1]++;
    for (int k = 0; k < K; ++k) offsets[k + 1] += offsets[k];
    std::vector<int> fill(offsets.begin(), offsets.end() - 1);
    for (int64_t f = 0; f < F; ++f) order[fill[asg[f]]++] = (int)f;
    cudaMemcpyAsync(A.order, order.data(), sizeof(int) * F, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(A.offsets, offsets.data(), sizeof(int) * (K + 1), cudaMemcpyHostToDevice, st);
    // the copies read host vectors that go out of scope: finish them here
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
  }
  const int64_t cols = 3 * (int64_t)A.Np;
  dim3 g1((unsigned)((cols + 255) / 256), (unsigned)kMeanChunks, (unsigned)K);
  k_ref_mean_partial<<<g1, 256, 0, st>>>(A.plane, cols, A.order, A.offsets, A.partial);
  dim3 g1b((unsigned)((cols + 255) / 256), (unsigned)K);
  k_ref_mean_final<<<g1b, 256, 0, st>>>(A.partial, cols, A.offsets, A.mean);
  k_ref_update<<<K, kPrepThreads, 0, st>>>(A.refs, A.swr, A.Eref, A.mean, A.w, A.N, A.Np);
  launches += 3;
  o.launches = launches;
  return cudaGetLastError();
}

cudaError_t run_prep(const PrepArgs& A, PrepOut& o, cudaStream_t st) {
  return A.dtype_f64 ? prep_impl<double>(A, o, st) : prep_impl<float>(A, o, st);
}

cudaError_t run_finish(const FinishArgs& A, cudaStream_t st) {
  const int grid = (int)std::min<int64_t>((A.F + kWarps - 1) / kWarps, 152 * 16);
  k_finish<<<grid, kPrepThreads, 0, st>>>(A.plane, A.F, A.Np, A.N, A.mean, A.assign, A.K, A.swr, A.tc,
                                          (__half*)A.hi, (__half*)A.lo, A.inv_scale, A.write_plane, A.nrm, A.P,
                                          A.trP);
  k_ref_terms<<<A.K * A.K, kPrepThreads, 0, st>>>(A.refs, A.N, A.K, A.w, A.nofit, A.RP);
  return cudaGetLastError();
}

}  // namespace gbr
