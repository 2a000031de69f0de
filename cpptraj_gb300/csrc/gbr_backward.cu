// gbr_backward.cu -- gradient of L = sum_{i<j} g_ij RMSD_ij with respect to
// every coordinate (K4).  cpptraj has no gradient of RMSD; this follows from
// the envelope theorem: at the optimal rotation T (taking x'_j onto x'_i)
//   dRMSD_ij/dx'_i[a] = w_a (x'_i[a] - T x'_j[a]) / (W RMSD_ij)
//   dRMSD_ij/dx'_j[a] = w_a (x'_j[a] - T^T x'_i[a]) / (W RMSD_ij)
// and centring contributes nothing because sum_a w_a (x'_i - T x'_j) = 0
// (applied explicitly in k_grad_final, which makes it hold for the computed
// centres too).
// With x'_f = r + d_f (one pre-alignment reference) and c_fh = g_fh / RMSD_fh:
//   dL/dx'_f[a] = (w_a / W) [ E_f r[a] + C_f d_f[a] - sum_h c_fh T_fh d_h[a] ]
//   E_f = sum_h c_fh (I - T_fh),  C_f = sum_h c_fh.
// The backward pair kernel (the tensor-core pair kernel's backward
// instantiation, gbr_pair_tc.cu) recomputes every RMSD and rotation and
// writes c*T blocks; the sum over h is the tensor-core
// contraction Z = (B + B^T) * plane of gbr_bwd_gemm.cu (plane = sqrt(w) d,
// FP16 hi/lo split, FP32 accumulation), and the result is rotated back into
// each frame's original orientation, dL/dx_f = R_f^T dL/dx'_f.
#include "gbr_common.cuh"
#include "gbr_internal.h"

namespace gbr {

namespace {

// Error-free transformations (Knuth's TwoSum; TwoProduct by FMA), with the
// _rn intrinsics so that no product or sum is contracted into an FMA.
__device__ __forceinline__ void ef_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void ef_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = fmaf(a, b, -p);
}

// Per-atom constants of the assembly as FP32 hi + lo pairs, from FP64:
// tab[a] = {r hi (3), r lo (3), w hi, w lo, sqrt(w) hi, sqrt(w) lo, 0, 0}.
__global__ void k_atom_split(int N, const double* r, const double* w, const double* sqw, float4* tab) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  float h[3], l[3];
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const double v = r[3 * a + p];
    h[p] = (float)v;
    l[p] = (float)(v - (double)h[p]);
  }
  const double wa = w ? w[a] : 1.0, sa = w ? sqw[a] : 1.0;
  const float wh = (float)wa, sh = (float)sa;
  tab[3 * a] = make_float4(h[0], h[1], h[2], l[0]);
  tab[3 * a + 1] = make_float4(l[1], l[2], wh, (float)(wa - (double)wh));
  tab[3 * a + 2] = make_float4(sh, (float)(sa - (double)sh), 0.f, 0.f);
}

// dL/dx_f[a] = R_f^T (J (w_a E_f r[a] + sqrt(w_a) (C_f p_f[a] - Z_f[a])) / W),
// J the centring projection g_a -> g_a - (w_a / W) sum_b g_b.  For exactly
// centred frames J changes nothing (sum_b g_b = 0 at the optimum); with the
// rounding of the computed centres it removes their first-order term, which
// is w_a-proportional, so the result is the gradient of the exactly centred
// RMSD.  One warp per frame: the first pass stores the unprojected values
// and their sum, the second projects and rotates them.
//
// The terms of the first pass are of the size of the molecule's extent and
// partly cancel, so they are combined in double-FP32 arithmetic (hi + lo
// pairs through TwoSum / TwoProduct, ~2^-44 relative) from the FP32 inputs
// and the FP64 constants split into hi + lo: as exact as FP64 arithmetic on
// the same inputs, without GB300's narrow FP64 pipe.  The sum over atoms is
// kept the same way; the projection and the rotation, which do not cancel,
// are plain FP32.
__global__ void __launch_bounds__(256) k_grad_final(int64_t F, int N, int Np, const float* E, const float* Cs,
                                                    const double* rot, const float4* tab, double iW,
                                                    const float* plane, const float* Z, float* grad) {
  const int lane = threadIdx.x & 31;
  const float iWh = (float)iW, iWl = (float)(iW - (double)iWh);
  for (int64_t f = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; f < F;
       f += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    float Ef[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Ef[k] = __ldg(E + f * 9 + k);
    const float cf = __ldg(Cs + f);
    float Ss[3] = {0.f, 0.f, 0.f}, Sc[3] = {0.f, 0.f, 0.f};
    for (int a = lane; a < N; a += 32) {
      const float4 t0 = __ldg(tab + 3 * a), t1 = __ldg(tab + 3 * a + 1), t2 = __ldg(tab + 3 * a + 2);
      const float rh[3] = {t0.x, t0.y, t0.z}, rl[3] = {t0.w, t1.x, t1.y};
      const float wh = t1.z, wl = t1.w, sh = t2.x, sl = t2.y;
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        const float* Ep = Ef + 3 * p;
        // er = E_p . r
        float es, ec, pq, eq, t;
        ef_prod(Ep[0], rh[0], es, ec);
        ef_prod(Ep[1], rh[1], pq, eq);
        ef_sum(es, pq, es, t);
        ec += t + eq;
        ef_prod(Ep[2], rh[2], pq, eq);
        ef_sum(es, pq, es, t);
        ec += t + eq;
        ec = fmaf(Ep[0], rl[0], fmaf(Ep[1], rl[1], fmaf(Ep[2], rl[2], ec)));
        // t = C_f p - Z
        const size_t row = (size_t)(3 * f + p);
        const float pl = __ldg(plane + row * Np + a), z = __ldg(Z + row * Np + a);
        float ts, tc, ps, pe;
        ef_prod(cf, pl, ps, pe);
        ef_sum(ps, -z, ts, tc);
        tc += pe;
        // u = w er + sqrt(w) t
        float a1, a2, b1, b2, us, uc;
        ef_prod(wh, es, a1, a2);
        a2 = fmaf(wh, ec, fmaf(wl, es, a2));
        ef_prod(sh, ts, b1, b2);
        b2 = fmaf(sh, tc, fmaf(sl, ts, b2));
        ef_sum(a1, b1, us, uc);
        uc += a2 + b2;
        // gp = u / W
        float g1, g2;
        ef_prod(us, iWh, g1, g2);
        g2 = fmaf(uc, iWh, fmaf(us, iWl, g2));
        float s2;
        ef_sum(g1, g2, g1, s2);  // g1: gp rounded, s2: what is left
        float e;
        ef_sum(Ss[p], g1, Ss[p], e);
        Sc[p] += e + s2;
        grad[((size_t)f * N + a) * 3 + p] = g1;
      }
    }
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float so = __shfl_xor_sync(0xffffffffu, Ss[p], o), co = __shfl_xor_sync(0xffffffffu, Sc[p], o);
        float e;
        ef_sum(Ss[p], so, Ss[p], e);
        Sc[p] += co + e;
      }
    float Sw[3];
#pragma unroll
    for (int p = 0; p < 3; ++p) Sw[p] = (Ss[p] + Sc[p]) * iWh;
    __syncwarp();
    float R[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = (float)rot[9 * f + k];
    for (int a = lane; a < N; a += 32) {
      const float wa = __ldg(tab + 3 * a + 1).z;
      float* g = grad + ((size_t)f * N + a) * 3;
      float gp[3];
#pragma unroll
      for (int p = 0; p < 3; ++p) gp[p] = fmaf(-wa, Sw[p], g[p]);
#pragma unroll
      for (int q = 0; q < 3; ++q) g[q] = fmaf(R[q], gp[0], fmaf(R[3 + q], gp[1], R[6 + q] * gp[2]));
    }
  }
}
}  // namespace

cudaError_t run_backward_tail(const BackwardTail& T, cudaStream_t st) {
  k_atom_split<<<(T.N + 127) / 128, 128, 0, st>>>(T.N, T.ref0, T.w, T.sqw, T.atab);
  cudaError_t e = run_backward_gemm(T.gemm, st);
  if (e != cudaSuccess) return e;
  const int g = (int)std::min<int64_t>((T.F + 7) / 8, 152 * 16);
  k_grad_final<<<g, 256, 0, st>>>(T.F, T.N, T.Np, T.E, T.C, T.rot, T.atab, 1.0 / T.W, T.plane, T.Z, T.grad);
  return cudaGetLastError();
}

}  // namespace gbr
