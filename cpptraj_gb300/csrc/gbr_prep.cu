// gbr_prep.cu -- per-frame passes that run before the pair contraction (K1).
//
//   k_centroid     centre of each frame: Frame::CenterOnOrigin / the target
//                  centring of Frame::RMSD_CenteredRef (src/Frame.cpp:1043-1055,
//                  1142-1171); reference frames use the reference masses.
//   k_make_ref     builds pre-alignment reference k from one frame, superposed
//                  onto an existing reference so all references share an
//                  orientation.
//   k_ref_dist     fit (or no-fit) RMSD of every frame to reference k, keeping
//                  the nearest reference per frame (greedy k-centre selection).
//   k_align        superposes every frame onto its reference in FP64 and writes
//                  the operand plane p = sqrt(w)*(R y - r) (FP32, [F][3][Np]).
//   k_split_f16    turns the FP32 plane into FP16 hi/lo planes ([F][4][Np],
//                  component 3 zero) for the tensor-core contraction.
//   k_frame_terms  n_f = |p_f|^2 and P_fc = sum p_f (sqrt(w) r_c)^T, computed
//                  from the exact operand values the contraction will read.
//   k_ref_terms    S_ba, its antisymmetric combos and sum w |r_a - r_b|^2.
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

template <typename T>
__global__ void __launch_bounds__(kPrepThreads) k_centroid(FrameSrc<T> src, int64_t F,
                                                           const double* cmass_ref,
                                                           const double* cmass_tgt, double* cen) {
  __shared__ double red[32 * 4];
  for (int64_t f = blockIdx.x; f < F; f += gridDim.x) {
    const T* x = src.frame(f);
    const double* m = (f < src.n_ref) ? cmass_ref : cmass_tgt;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, sm = 0.f;
    for (int a = threadIdx.x; a < src.N; a += blockDim.x) {
      const float w = m ? (float)m[a] : 1.0f;
      s0 += w * (float)x[3 * a];
      s1 += w * (float)x[3 * a + 1];
      s2 += w * (float)x[3 * a + 2];
      sm += w;
    }
    double v[4] = {s0, s1, s2, sm};
    block_sum_f64<4>(v, red);
    if (threadIdx.x == 0) {
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
                                                           const double* w, double Wsum,
                                                           const double* refs, const double* Eref, int k,
                                                           int nofit, float* dist, int* assign) {
  __shared__ double red[32 * 10];
  const int N = src.N;
  const double* rk = refs + (size_t)k * 3 * N;
  for (int64_t f = blockIdx.x; f < F; f += gridDim.x) {
    const T* x = src.frame(f);
    const float c0 = (float)cen[3 * f], c1 = (float)cen[3 * f + 1], c2 = (float)cen[3 * f + 2];
    float h[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = threadIdx.x; a < N; a += blockDim.x) {
      const float wa = w ? (float)w[a] : 1.0f;
      const float y0 = (float)x[3 * a] - c0, y1 = (float)x[3 * a + 1] - c1, y2 = (float)x[3 * a + 2] - c2;
      const float r0 = (float)rk[3 * a], r1 = (float)rk[3 * a + 1], r2 = (float)rk[3 * a + 2];
      if (nofit) {
        const float d0 = y0 - r0, d1 = y1 - r1, d2 = y2 - r2;
        h[9] += wa * (d0 * d0 + d1 * d1 + d2 * d2);
      } else {
        h[0] += wa * y0 * r0; h[1] += wa * y0 * r1; h[2] += wa * y0 * r2;
        h[3] += wa * y1 * r0; h[4] += wa * y1 * r1; h[5] += wa * y1 * r2;
        h[6] += wa * y2 * r0; h[7] += wa * y2 * r1; h[8] += wa * y2 * r2;
        h[9] += wa * (y0 * y0 + y1 * y1 + y2 * y2);
      }
    }
    double v[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) v[q] = h[q];
    block_sum_f64<10>(v, red);
    if (threadIdx.x == 0) {
      double d2;
      if (nofit) {
        d2 = v[9] / Wsum;
      } else {
        double R[9];
        const double E0 = 0.5 * (v[9] + Eref[k]);
        const double lam = qcp_lambda_rot(v, E0, R);
        d2 = 2.0 * (E0 - lam) / Wsum;
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
// p = sqrt(w) * (R y - r_a) as the FP32 operand plane.  Also tracks max |p|.
template <typename T>
__global__ void __launch_bounds__(kPrepThreads) k_align(FrameSrc<T> src, int64_t F, int Np,
                                                        const double* cen, const double* w,
                                                        const double* refs, const int* assign, int nofit,
                                                        double* rot, float* plane, unsigned* pmax_bits) {
  __shared__ double red[32 * 10];
  __shared__ double Rs[9];
  const int N = src.N;
  for (int64_t f = blockIdx.x; f < F; f += gridDim.x) {
    const T* x = src.frame(f);
    const int a_ref = assign[f];
    const double* ra = refs + (size_t)a_ref * 3 * N;
    const double c0 = cen[3 * f], c1 = cen[3 * f + 1], c2 = cen[3 * f + 2];
    if (threadIdx.x < 9) Rs[threadIdx.x] = (threadIdx.x % 4 == 0) ? 1.0 : 0.0;
    __syncthreads();
    if (!nofit) {
      float h[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int a = threadIdx.x; a < N; a += blockDim.x) {
        const float wa = w ? (float)w[a] : 1.0f;
        const float y0 = (float)((double)x[3 * a] - c0), y1 = (float)((double)x[3 * a + 1] - c1),
                    y2 = (float)((double)x[3 * a + 2] - c2);
        const float r0 = (float)ra[3 * a], r1 = (float)ra[3 * a + 1], r2 = (float)ra[3 * a + 2];
        h[0] += wa * y0 * r0; h[1] += wa * y0 * r1; h[2] += wa * y0 * r2;
        h[3] += wa * y1 * r0; h[4] += wa * y1 * r1; h[5] += wa * y1 * r2;
        h[6] += wa * y2 * r0; h[7] += wa * y2 * r1; h[8] += wa * y2 * r2;
        h[9] += wa * (y0 * y0 + y1 * y1 + y2 * y2 + r0 * r0 + r1 * r1 + r2 * r2);
      }
      double v[10];
#pragma unroll
      for (int q = 0; q < 10; ++q) v[q] = h[q];
      block_sum_f64<10>(v, red);
      if (threadIdx.x == 0) {
        double R[9];
        qcp_lambda_rot(v, 0.5 * v[9], R);
        for (int q = 0; q < 9; ++q) Rs[q] = R[q];
      }
      __syncthreads();
    }
    const double R0 = Rs[0], R1 = Rs[1], R2 = Rs[2], R3 = Rs[3], R4 = Rs[4], R5 = Rs[5], R6 = Rs[6],
                 R7 = Rs[7], R8 = Rs[8];
    if (threadIdx.x < 9 && rot) rot[9 * f + threadIdx.x] = Rs[threadIdx.x];
    float* pl = plane + (size_t)f * 3 * Np;
    float lmax = 0.0f;
    for (int a = threadIdx.x; a < Np; a += blockDim.x) {
      float p0 = 0.f, p1 = 0.f, p2 = 0.f;
      if (a < N) {
        const double y0 = (double)x[3 * a] - c0, y1 = (double)x[3 * a + 1] - c1, y2 = (double)x[3 * a + 2] - c2;
        const double sw = w ? sqrt(w[a]) : 1.0;
        p0 = (float)(sw * (R0 * y0 + R1 * y1 + R2 * y2 - ra[3 * a]));
        p1 = (float)(sw * (R3 * y0 + R4 * y1 + R5 * y2 - ra[3 * a + 1]));
        p2 = (float)(sw * (R6 * y0 + R7 * y1 + R8 * y2 - ra[3 * a + 2]));
      }
      pl[a] = p0;
      pl[Np + a] = p1;
      pl[2 * Np + a] = p2;
      lmax = fmaxf(lmax, fmaxf(fabsf(p0), fmaxf(fabsf(p1), fabsf(p2))));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
    if ((threadIdx.x & 31) == 0 && pmax_bits) atomicMax(pmax_bits, __float_as_uint(lmax));
    __syncthreads();
  }
}

// FP32 plane [F][3][Np] -> FP16 hi/lo planes [F][3][Np] scaled by `scale` (a
// power of two).  The FP32 plane is overwritten with the value hi + lo
// represents, so the per-frame terms match what the contraction reads.
__global__ void k_split_f16(float* plane, int64_t total, float scale, __half* hi, __half* lo) {
  const float inv = 1.0f / scale;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float v = plane[t] * scale;
    const __half h = __float2half_rn(v);
    const __half l = __float2half_rn(v - __half2float(h));
    hi[t] = h;
    lo[t] = l;
    plane[t] = (__half2float(h) + __half2float(l)) * inv;
  }
}

// n_f and P_fc for every frame f and reference c (from the FP32 plane).
__global__ void __launch_bounds__(kPrepThreads) k_frame_terms(const float* plane, int64_t F, int Np, int N,
                                                              const float* swr, int K, float* nrm, float* P,
                                                              float* trP) {
  __shared__ double red[32 * 10];
  for (int64_t f = blockIdx.x; f < F; f += gridDim.x) {
    const float* pl = plane + (size_t)f * 3 * Np;
    for (int c = 0; c < K; ++c) {
      const float* rc = swr + (size_t)c * N * 3;
      float h[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int a = threadIdx.x; a < N; a += blockDim.x) {
        const float p0 = pl[a], p1 = pl[Np + a], p2 = pl[2 * Np + a];
        const float r0 = rc[3 * a], r1 = rc[3 * a + 1], r2 = rc[3 * a + 2];
        h[0] += p0 * r0; h[1] += p0 * r1; h[2] += p0 * r2;
        h[3] += p1 * r0; h[4] += p1 * r1; h[5] += p1 * r2;
        h[6] += p2 * r0; h[7] += p2 * r1; h[8] += p2 * r2;
        if (c == 0) h[9] += p0 * p0 + p1 * p1 + p2 * p2;
      }
      double v[10];
#pragma unroll
      for (int q = 0; q < 10; ++q) v[q] = h[q];
      block_sum_f64<10>(v, red);
      if (threadIdx.x == 0) {
        float* Pf = P + ((size_t)f * K + c) * 9;
        for (int q = 0; q < 9; ++q) Pf[q] = (float)v[q];
        trP[(size_t)f * K + c] = (float)(v[0] + v[4] + v[8]);
        if (c == 0) nrm[f] = (float)v[9];
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

__global__ void k_absmax(const float* x, int64_t n, unsigned* out_bits) {
  float m = 0.0f;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(x[t]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out_bits, __float_as_uint(m));
}

// Mean of the operand plane over the frames of each reference:
// mean[k][c] = sum_{f in ref k} plane[f][c] / count_k, c over [0, 3*Np).
__global__ void k_ref_mean(const float* plane, int64_t cols, const int* order, const int* offsets,
                           float* mean) {
  const int k = blockIdx.y;
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const int lo = offsets[k], hi = offsets[k + 1];
  double s = 0.0;
  for (int n = lo; n < hi; ++n) s += (double)plane[(size_t)order[n] * cols + c];
  mean[(size_t)k * cols + c] = (hi > lo) ? (float)(s / (double)(hi - lo)) : 0.0f;
}

// p_f -= mean[a(f)] (the residual relative to the refined reference).
__global__ void k_shift(float* plane, int64_t F, int64_t cols, const int* assign, const float* mean) {
  const int64_t total = F * cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = t / cols, c = t - f * cols;
    plane[t] -= mean[(size_t)assign[f] * cols + c];
  }
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
  const int grid = (int)std::min<int64_t>(F, 152 * 8);
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
  // Greedy k-centre choice of pre-alignment references.
  cudaMemsetAsync(A.fsel, 0, sizeof(int64_t), st);
  k_make_ref<T><<<1, kPrepThreads, 0, st>>>(src, A.fsel, A.cen, A.w, A.assign, 0, 0, A.nofit, A.refs, A.swr,
                                            A.Eref);
  k_ref_dist<T><<<grid, kPrepThreads, 0, st>>>(src, F, A.cen, A.w, A.Wsum, A.refs, A.Eref, 0, A.nofit,
                                               A.dist, A.assign);
  launches += 2;
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
    k_ref_dist<T><<<grid, kPrepThreads, 0, st>>>(src, F, A.cen, A.w, A.Wsum, A.refs, A.Eref, K, A.nofit,
                                                 A.dist, A.assign);
    launches += 2;
    ++K;
  }
  o.K = K;
  cudaMemsetAsync(A.pmax_bits, 0, sizeof(unsigned), st);
  k_align<T><<<grid, kPrepThreads, 0, st>>>(src, F, A.Np, A.cen, A.w, A.refs, A.assign, A.nofit, A.rot,
                                            A.plane, A.pmax_bits);
  ++launches;
  // Refine every reference to the mean of its superposed frames: residuals
  // shrink to each frame's own fluctuation.  Frames are grouped by reference
  // with a host-side counting sort of the assignment.
  {
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
    const int64_t cols = 3 * (int64_t)A.Np;
    dim3 g1((unsigned)((cols + 255) / 256), (unsigned)K);
    k_ref_mean<<<g1, 256, 0, st>>>(A.plane, cols, A.order, A.offsets, A.mean);
    const int g2 = (int)std::min<int64_t>((F * cols + 255) / 256, 152 * 16);
    k_shift<<<g2, 256, 0, st>>>(A.plane, F, cols, A.assign, A.mean);
    k_ref_update<<<K, kPrepThreads, 0, st>>>(A.refs, A.swr, A.Eref, A.mean, A.w, A.N, A.Np);
    launches += 3;
    // The copies above read host vectors that go out of scope: finish them.
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
  }
  // max |p| after the shift (for the FP16 split scale)
  cudaMemsetAsync(A.pmax_bits, 0, sizeof(unsigned), st);
  {
    const int64_t total = F * 3 * (int64_t)A.Np;
    const int g3 = (int)std::min<int64_t>((total + 255) / 256, 152 * 16);
    k_absmax<<<g3, 256, 0, st>>>(A.plane, total, A.pmax_bits);
    ++launches;
  }
  o.launches = launches;
  return cudaGetLastError();
}

cudaError_t run_prep(const PrepArgs& A, PrepOut& o, cudaStream_t st) {
  return A.dtype_f64 ? prep_impl<double>(A, o, st) : prep_impl<float>(A, o, st);
}

cudaError_t run_split_f16(float* plane, int64_t F, int Np, float scale, void* hi, void* lo, cudaStream_t st) {
  const int64_t total = F * 3 * (int64_t)Np;
  const int grid = (int)std::min<int64_t>((total + 255) / 256, 152 * 16);
  k_split_f16<<<grid, 256, 0, st>>>(plane, total, scale, (__half*)hi, (__half*)lo);
  return cudaGetLastError();
}

cudaError_t run_terms(const float* plane, int64_t F, int Np, int N, const float* swr, int K, float* nrm,
                      float* P, float* trP, const double* refs, const double* w, int nofit, float* RP,
                      cudaStream_t st) {
  const int grid = (int)std::min<int64_t>(F, 152 * 8);
  k_frame_terms<<<grid, kPrepThreads, 0, st>>>(plane, F, Np, N, swr, K, nrm, P, trP);
  k_ref_terms<<<K * K, kPrepThreads, 0, st>>>(refs, N, K, w, nofit, RP);
  return cudaGetLastError();
}

}  // namespace gbr
