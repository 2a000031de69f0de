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

// dL/dx_f[a] = R_f^T (J (w_a E_f r[a] + sqrt(w_a) (C_f p_f[a] - Z_f[a])) / W),
// J the centring projection g_a -> g_a - (w_a / W) sum_b g_b.  For exactly
// centred frames J changes nothing (sum_b g_b = 0 at the optimum); with the
// rounding of the computed centres it removes their first-order term, which
// is w_a-proportional, so the result is the gradient of the exactly centred
// RMSD.  One warp per frame: the first pass stores the unprojected values
// and their sum, the second projects and rotates them.
__global__ void __launch_bounds__(256) k_grad_final(int64_t F, int N, int Np, const float* E, const float* Cs,
                                                    const double* rot, const double* r, const double* w,
                                                    const double* sqw, double iW, const float* plane, const float* Z,
                                                    float* grad) {
  const int lane = threadIdx.x & 31;
  for (int64_t f = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; f < F;
       f += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const float* Ef = E + f * 9;
    const double cf = Cs[f];
    double S[3] = {0.0, 0.0, 0.0};
    for (int a = lane; a < N; a += 32) {
      const double wa = w ? w[a] : 1.0;
      const double sw = w ? sqw[a] : 1.0;
      const double r0 = r[3 * a], r1 = r[3 * a + 1], r2 = r[3 * a + 2];
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        const double er = (double)Ef[p * 3] * r0 + (double)Ef[p * 3 + 1] * r1 + (double)Ef[p * 3 + 2] * r2;
        const size_t row = (size_t)(3 * f + p);
        const double gp = (wa * er + sw * (cf * (double)plane[row * Np + a] - (double)Z[row * Np + a])) * iW;
        S[p] += gp;
        grad[((size_t)f * N + a) * 3 + p] = (float)gp;
      }
    }
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) S[p] += __shfl_xor_sync(0xffffffffu, S[p], o);
    __syncwarp();
    const double* R = rot + 9 * f;
    for (int a = lane; a < N; a += 32) {
      const double wa = w ? w[a] : 1.0;
      float* g = grad + ((size_t)f * N + a) * 3;
      double gp[3];
#pragma unroll
      for (int p = 0; p < 3; ++p) gp[p] = (double)g[p] - wa * S[p] * iW;
#pragma unroll
      for (int q = 0; q < 3; ++q) g[q] = (float)(R[q] * gp[0] + R[3 + q] * gp[1] + R[6 + q] * gp[2]);
    }
  }
}
}  // namespace

cudaError_t run_backward_tail(const BackwardTail& T, cudaStream_t st) {
  cudaError_t e = run_backward_gemm(T.gemm, st);
  if (e != cudaSuccess) return e;
  const int g = (int)std::min<int64_t>((T.F + 7) / 8, 152 * 16);
  k_grad_final<<<g, 256, 0, st>>>(T.F, T.N, T.Np, T.E, T.C, T.rot, T.ref0, T.w, T.sqw, 1.0 / T.W, T.plane, T.Z,
                                  T.grad);
  return cudaGetLastError();
}

}  // namespace gbr
