// gbr_common.cuh -- shared device code of libgbrmsd: reductions, the FP64
// per-frame superposition used for pre-alignment, and the FP32 pair epilogue.
//
// Numerical scheme (why the pair kernels can run in FP32 / split FP16).
// cpptraj computes, per pair, RMSD^2 = 2*(E0 - lambda_max)/W with E0 and the
// 3x3 covariance accumulated in FP64 (src/Frame.cpp:1184-1268).  For similar
// frames E0 and lambda_max are ~W*Rg^2 while E0-lambda is ~W*RMSD^2, so the
// subtraction cancels 4-6 digits and FP32 accumulation of the raw covariance
// cannot reach 1e-4 Angstrom.  Instead every frame is first superposed (in
// FP64, exact rotation) onto its nearest of K reference structures r_k, which
// leaves RMSD unchanged, and split as x'_f = r_{a(f)} + d_f with d_f small.
// Each reference is then refined to the mean of its superposed frames, so d_f
// is of the size of the frame's own fluctuation.  For a pair (ref i, target
// j), a = a(i), b = a(j):
//     M = sum w x'_j x'_i^T = S_ba + P_ja + P_ib^T + D_ji
// with S_ba = sum w r_b r_a^T, P_fc = sum w d_f r_c^T (per frame and
// reference) and D_ji = sum w d_j d_i^T (the only per-pair contraction, on
// small numbers).  The quaternion key matrix enters through
// G = E0*I - K(M), whose smallest eigenvalue is W*RMSD^2/2.  After rotating
// the target by the exact inter-reference rotation U_ab (pair_epilogue), its
// (0,0) entry G00 = 1/2 sum w |x'_i - U_ab x'_j|^2 is assembled from small
// terms, so the smallest eigenvalue can be found in FP32 without
// cancellation: a Schur-complement (secular equation) iteration on G around
// q = (1, v), or, when the pair's relative rotation is large, QCP (Theobald
// 2005; Liu, Agrafiotis & Theobald 2010) on K(M) for the eigenvector followed
// by the Rayleigh quotient of G.  Each pair carries an
// a-priori error bound; pairs whose bound exceeds the tolerance are listed
// and recomputed directly in FP64 by gbr_exact.cu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbr {

constexpr int kMaxRefs = 64;

// --------------------------------------------------------------------------
// FP64 QCP on a 3x3 cross-covariance A[p][q] = sum w t_p r_q (target first):
// the largest eigenvalue lambda of the key matrix by Newton from E0, and the
// proper rotation R (row-major) minimising sum w |R t - r|^2.  R is the
// identity when no adjugate column of (K - lambda I) is usable.
// --------------------------------------------------------------------------
__device__ inline double qcp_lambda_rot(const double A[9], double E0, double R[9]) {
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
  // Eigenvector of the key matrix by the adjugate of (K - lam I): try each
  // column until one has a usable norm.
  const double k11 = pxx + zz - lam, k12 = myz, k13 = -mxz, k14 = mxy;
  const double k22 = mxx - zz - lam, k23 = pxy, k24 = pxz;
  const double k33 = yy - xx - zz - lam, k34 = pyz;
  const double k44 = zz - pxx - lam;
  const double K[16] = {k11, k12, k13, k14, k12, k22, k23, k24, k13, k23, k33, k34, k14, k24, k34, k44};
  double q[4] = {1.0, 0.0, 0.0, 0.0};
  double best = 0.0;
  const double scale = fabs(E0) > 0.0 ? fabs(E0) : 1.0;
  for (int col = 0; col < 4; ++col) {
    // cofactors C[r][col] for r = 0..3 of the 4x4 matrix K
    double c[4];
    for (int r = 0; r < 4; ++r) {
      int rr[3], cc[3], nr = 0, nc = 0;
      for (int k = 0; k < 4; ++k) {
        if (k != r) rr[nr++] = k;
        if (k != col) cc[nc++] = k;
      }
      const double m00 = K[rr[0] * 4 + cc[0]], m01 = K[rr[0] * 4 + cc[1]], m02 = K[rr[0] * 4 + cc[2]];
      const double m10 = K[rr[1] * 4 + cc[0]], m11 = K[rr[1] * 4 + cc[1]], m12 = K[rr[1] * 4 + cc[2]];
      const double m20 = K[rr[2] * 4 + cc[0]], m21 = K[rr[2] * 4 + cc[1]], m22 = K[rr[2] * 4 + cc[2]];
      const double det = m00 * (m11 * m22 - m12 * m21) - m01 * (m10 * m22 - m12 * m20) +
                         m02 * (m10 * m21 - m11 * m20);
      c[r] = ((r + col) & 1) ? -det : det;
    }
    const double n2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
    if (n2 > best) {
      best = n2;
      q[0] = c[0]; q[1] = c[1]; q[2] = c[2]; q[3] = c[3];
    }
    if (n2 > 1e-12 * scale * scale * scale * scale * scale * scale) break;
  }
  if (!(best > 0.0)) { q[0] = 1.0; q[1] = q[2] = q[3] = 0.0; }
  const double inv = 1.0 / sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  const double a0 = q[0] * inv, a1 = q[1] * inv, a2 = q[2] * inv, a3 = q[3] * inv;
  // Rotation of the unit quaternion, row-major, oriented so that R * t best
  // matches r (the transpose of the matrix QCP reports for this covariance).
  const double aa = a0 * a0, bb = a1 * a1, cc2 = a2 * a2, dd = a3 * a3;
  R[0] = aa + bb - cc2 - dd;
  R[3] = 2.0 * (a1 * a2 + a0 * a3);
  R[6] = 2.0 * (a3 * a1 - a0 * a2);
  R[1] = 2.0 * (a1 * a2 - a0 * a3);
  R[4] = aa - bb + cc2 - dd;
  R[7] = 2.0 * (a2 * a3 + a0 * a1);
  R[2] = 2.0 * (a3 * a1 + a0 * a2);
  R[5] = 2.0 * (a2 * a3 - a0 * a1);
  R[8] = aa - bb - cc2 + dd;
  return lam;
}

// Proper rotation (row-major, FP64) of the quaternion q, oriented as
// qcp_lambda_rot's R: R * t best matches r for the covariance QCP was given.
// q is normalised here in FP64, so R is orthogonal to FP64 rounding whatever
// precision q came from.  A zero or non-finite q gives the identity.
__device__ inline void rotation_from_quat(const float qf[4], double R[9]) {
  double a0 = qf[0], a1 = qf[1], a2 = qf[2], a3 = qf[3];
  const double n2 = a0 * a0 + a1 * a1 + a2 * a2 + a3 * a3;
  if (!(n2 > 0.0) || !isfinite(n2)) {
    a0 = 1.0; a1 = a2 = a3 = 0.0;
  } else {
    const double inv = 1.0 / sqrt(n2);
    a0 *= inv; a1 *= inv; a2 *= inv; a3 *= inv;
  }
  const double aa = a0 * a0, bb = a1 * a1, cc = a2 * a2, dd = a3 * a3;
  R[0] = aa + bb - cc - dd;
  R[3] = 2.0 * (a1 * a2 + a0 * a3);
  R[6] = 2.0 * (a3 * a1 - a0 * a2);
  R[1] = 2.0 * (a1 * a2 - a0 * a3);
  R[4] = aa - bb + cc - dd;
  R[7] = 2.0 * (a2 * a3 + a0 * a1);
  R[2] = 2.0 * (a3 * a1 + a0 * a2);
  R[5] = 2.0 * (a2 * a3 - a0 * a1);
  R[8] = aa - bb - cc + dd;
}

// --------------------------------------------------------------------------
// Per-pair data and the FP32 epilogue.
// --------------------------------------------------------------------------
// Per reference pair (index b*K + a; a = reference of the reference frame,
// b = reference of the target frame), 24 floats:
//   [0..8]   U_ab   proper rotation minimising sum w |r_a - U r_b|^2 (identity
//                   when a == b or in no-fit mode), row-major, from FP64
//   [9..17]  SU_ab  U_ab * S_ba with S_ba = sum w r_b r_a^T
//   [18..20] antisymmetric combos (yz-zy, zx-xz, xy-yx) of SU_ab, from FP64
//   [21]     SS_ab  sum w |r_a - U_ab r_b|^2
constexpr int kRefPairStride = 24;

struct FrameTerms {
  const int* assign;  // [F] reference index of each set frame
  const float* nrm;   // [F] n_f = sum |p_f|^2  (p = sqrt(w) d)
  const float* P;     // [F][K][9] P_fc[p][q] = sum p_f[p] * (sqrt(w) r_c)[q]
  const float* trP;   // [F][K]
  const float* RP;    // [K][K][kRefPairStride]
  int K;
  float W;            // total weight
  float two_over_w;   // 2 / W
  float tol;          // per-pair tolerance (Angstrom)
  // A-priori bound of the contraction error in tr D (see pair_epilogue):
  //   gem_s * sqrt(n_i n_j) + gem_c * |tr D|
  float gem_s;        // sign-random part and the FP16 split (no growth with N)
  float gem_c;        // consistently-signed accumulation, already scaled by N:
                      //   FP32 FMA (round to nearest): random walk, ~sqrt(N)
                      //   tensor memory (measured to behave like truncation): ~N
  float epi_coef;     // epilogue rounding coefficient (times the Rayleigh-quotient terms)
  int nofit;
};

// 3x3 symmetric solve by cofactors; returns det.
__device__ __forceinline__ float solve_sym3(float a00, float a01, float a02, float a11, float a12,
                                            float a22, float b0, float b1, float b2, float& x0,
                                            float& x1, float& x2, float& m2) {
  const float c00 = a11 * a22 - a12 * a12;
  const float c01 = a02 * a12 - a01 * a22;
  const float c02 = a01 * a12 - a02 * a11;
  const float c11 = a00 * a22 - a02 * a02;
  const float c12 = a01 * a02 - a00 * a12;
  const float c22 = a00 * a11 - a01 * a01;
  const float det = a00 * c00 + a01 * c01 + a02 * c02;
  // Approximate reciprocal (2 ulp): the solve only produces the trial vector
  // of a Rayleigh quotient, whose value is second order in the vector's error.
  const float id = __fdividef(1.0f, det);
  x0 = (c00 * b0 + c01 * b1 + c02 * b2) * id;
  x1 = (c01 * b0 + c11 * b1 + c12 * b2) * id;
  x2 = (c02 * b0 + c12 * b1 + c22 * b2) * id;
  m2 = c22;
  return det;
}

// FP32 QCP eigenvector of the key matrix of M (scaled by 1/E0).  When
// lam_rel is given it receives the largest eigenvalue divided by E0.
__device__ inline void qcp_vec_f32(const float M[9], float E0, float q[4], float* lam_rel = nullptr) {
  const float s = 1.0f / E0;
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
  for (int it = 0; it < 40; ++it) {
    const float l2 = lam * lam, b = (l2 + c2) * lam, a = b + c1;
    const float den = 2.0f * l2 * lam + b + a;
    if (den == 0.0f) break;
    const float dl = (a * lam + c0) / den;
    lam -= dl;
    if (fabsf(dl) <= 1e-7f * fabsf(lam)) break;
  }
  const float k11 = pxx + zz - lam, k12 = myz, k13 = -mxz, k14 = mxy;
  const float k22 = mxx - zz - lam, k23 = pxy, k24 = pxz;
  const float k33 = yy - xx - zz - lam, k34 = pyz;
  const float k44 = zz - pxx - lam;
  // Adjugate columns, largest norm wins (QCP's fallback order, all four tried).
  const float a3344 = k33 * k44 - k34 * k34, a3244 = k23 * k44 - k24 * k34,
              a3243 = k23 * k34 - k24 * k33, a3143 = k13 * k34 - k14 * k33,
              a3144 = k13 * k44 - k14 * k34, a3142 = k13 * k24 - k14 * k23;
  float best[4], bn;
  best[0] = k22 * a3344 - k23 * a3244 + k24 * a3243;
  best[1] = -k12 * a3344 + k23 * a3144 - k24 * a3143;
  best[2] = k12 * a3244 - k22 * a3144 + k24 * a3142;
  best[3] = -k12 * a3243 + k22 * a3143 - k23 * a3142;
  bn = best[0] * best[0] + best[1] * best[1] + best[2] * best[2] + best[3] * best[3];
  {
    float c[4];
    c[0] = k12 * a3344 - k13 * a3244 + k14 * a3243;
    c[1] = -k11 * a3344 + k13 * a3144 - k14 * a3143;
    c[2] = k11 * a3244 - k12 * a3144 + k14 * a3142;
    c[3] = -k11 * a3243 + k12 * a3143 - k13 * a3142;
    const float n = c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
    if (n > bn) { bn = n; best[0] = c[0]; best[1] = c[1]; best[2] = c[2]; best[3] = c[3]; }
  }
  {
    const float a1324 = k13 * k24 - k14 * k23, a1224 = k12 * k24 - k14 * k22,
                a1223 = k12 * k23 - k13 * k22, a1124 = k11 * k24 - k14 * k12,
                a1123 = k11 * k23 - k13 * k12, a1122 = k11 * k22 - k12 * k12;
    float c[4];
    c[0] = k24 * a1324 - k34 * a1224 + k44 * a1223;
    c[1] = -k14 * a1324 + k34 * a1124 - k44 * a1123;
    c[2] = k14 * a1224 - k24 * a1124 + k44 * a1122;
    c[3] = -k14 * a1223 + k24 * a1123 - k34 * a1122;
    float n = c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
    if (n > bn) { bn = n; best[0] = c[0]; best[1] = c[1]; best[2] = c[2]; best[3] = c[3]; }
    c[0] = k23 * a1324 - k33 * a1224 + k34 * a1223;
    c[1] = -k13 * a1324 + k33 * a1124 - k34 * a1123;
    c[2] = k13 * a1224 - k23 * a1124 + k34 * a1122;
    c[3] = -k13 * a1223 + k23 * a1123 - k33 * a1122;
    n = c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
    if (n > bn) { bn = n; best[0] = c[0]; best[1] = c[1]; best[2] = c[2]; best[3] = c[3]; }
  }
  if (!(bn > 0.0f)) { best[0] = 1.0f; best[1] = best[2] = best[3] = 0.0f; }
  q[0] = best[0]; q[1] = best[1]; q[2] = best[2]; q[3] = best[3];
  if (lam_rel) *lam_rel = lam;
}

// The pair epilogue.  D[pj*3+pi] = sum p_j[pj] p_i[pi] (target j first).
// Returns the RMSD (Angstrom, >= 0); sets *flag when the error bound exceeds
// the tolerance and the pair must be recomputed in FP64.
//
// With x'_i = r_a + d_i and x'_j = r_b + d_j, the pair is solved in the frame
// where target j is additionally rotated by U_ab (exact, per reference pair),
// so the remaining optimal rotation is close to the identity for every pair:
//   M'' = U_ab M = SU_ab + U_ab (P_ja + P_ib^T + D_ji)
//   G00 = 1/2 sum w |x'_i - U_ab x'_j|^2
//       = 1/2 (SS_ab + n_i + n_j) + trP_ia - <U,P_ib> - <U,P_ja^T> + trP_jb - tr(U D_ji)
// (for a == b: U = I and G00 = 1/2 (n_i + n_j) - tr D_ji).
// Everything but D_ji belongs to one frame of the pair and the pair's
// references, so it is formed once per frame and reference pair (Side) and
// the per-pair work is U D_ji, its trace and the eigen solve.
// qout (optional) receives the unit quaternion (QCP convention) of the
// optimal superposition of x'_j onto x'_i, i.e. x'_i ~ R(q)^T x'_j with R(q)
// the rotation matrix QCP builds from q; only meaningful when t.K == 1.
struct F9 {
  float v[9];
};

// One frame's share of a pair with references (a, b), U = U_ab:
//   reference frame i: Q = U P_ib^T, c = n_i/2 + trP_ia - <U, P_ib>
//   target frame j:    Q = U P_ja,   c = n_j/2 + trP_jb - <U, P_ja^T>
//   a == b:            U = I and the P terms of G00 cancel: c = n/2
// m is the sum of the magnitudes in c (for the error bound), sn = sqrt(n).
struct Side {
  float Q[9];
  float c, m, sn;
};

// Rounded operation by operation (no contraction left to the compiler), so
// that the terms formed per tile in shared memory and those formed per pair
// from global memory are the same numbers.
static __device__ __forceinline__ void side_terms(const float P[9], float n, float trPown, const float U[9],
                                                  bool same, bool ref_side, Side& s) {
  const float h = __fmul_rn(0.5f, n);
  s.sn = __fsqrt_rn(fmaxf(n, 0.0f));
  if (same) {
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = 0; q < 3; ++q) s.Q[p * 3 + q] = ref_side ? P[q * 3 + p] : P[p * 3 + q];
    s.c = h;
    s.m = h;
    return;
  }
#pragma unroll
  for (int p = 0; p < 3; ++p)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      // column q of P^T (reference side) or of P (target side)
      const float b0 = ref_side ? P[q * 3 + 0] : P[0 * 3 + q];
      const float b1 = ref_side ? P[q * 3 + 1] : P[1 * 3 + q];
      const float b2 = ref_side ? P[q * 3 + 2] : P[2 * 3 + q];
      s.Q[p * 3 + q] = __fmaf_rn(U[p * 3 + 2], b2, __fmaf_rn(U[p * 3 + 1], b1, __fmul_rn(U[p * 3], b0)));
    }
  float uP = __fmul_rn(U[0], P[0]);
#pragma unroll
  for (int k = 1; k < 9; ++k) uP = __fmaf_rn(U[k], ref_side ? P[k] : P[(k % 3) * 3 + k / 3], uP);
  s.c = __fsub_rn(__fadd_rn(h, trPown), uP);
  s.m = __fadd_rn(__fadd_rn(h, fabsf(trPown)), fabsf(uP));
}

// The reference-pair entry of (a, b) as the solver reads it (see
// kRefPairStride): U_ab, SU_ab, the antisymmetric combos and SS_ab.
struct RefPair {
  float4 v[6];
};
// From global memory (16-byte aligned entries).
static __device__ __forceinline__ void load_refpair(const float* rp, RefPair& r) {
  const float4* p = reinterpret_cast<const float4*>(rp);
#pragma unroll
  for (int k = 0; k < 6; ++k) r.v[k] = __ldg(p + k);
}
static __device__ __forceinline__ float rpv(const RefPair& r, int k) {
  const float4& q = r.v[k >> 2];
  return (k & 3) == 0 ? q.x : (k & 3) == 1 ? q.y : (k & 3) == 2 ? q.z : q.w;
}

// The solver, given D_ji as sc * Dv (Dv the contraction of the scaled
// operand planes, sc the product of the two frames' 1/scale), both sides'
// terms and the pair's reference-pair entry (in registers, from global or
// shared memory).
//
// The smallest eigenvalue of G = [[G00, g^T], [g, Gs]] is found around
// q = (1, v): with A = Gs - G00 I and mu = G00 + delta,
//   v = -(A - delta I)^-1 g,  delta = g.v.
// When A is positive definite and |delta| is below its smallest eigenvalue
// lambda, (A - delta I)^-1 = sum_k delta^k A^-(k+1).  With w0 = A^-1 g,
// w1 = A^-1 w0 and s_k = g^T A^-(k+1) g <= s0 / lambda^k, the exact delta
// solves delta = -sum_k delta^k s_k; its first-order solution
// delta0 = -s0 / (1 + s1) (s0 = g.w0, s1 = w0.w0) gives v = -(w0 + delta0 w1).
// With rho = |delta| / lambda (bounded through tr(adj A) / det A >= 1/lambda),
// the dropped terms of v are at most |w0| rho^2 / (1 - rho) and the error of
// delta0 adds |w0| rho^3 / (1 - rho); the Rayleigh quotient below turns an
// error e of v into at most tr(G) |e|^2.  This path is taken when that bound
// is negligible; otherwise the fixed-point iteration on the secular equation
// and, failing that, QCP (Theobald 2005; Liu, Agrafiotis & Theobald 2010) on
// K(M) give q.  The result is the Rayleigh quotient of G at q in either case,
// written as G00 + (2 q0 g.qv + qv^T A qv) / |q|^2 (qv = (q1, q2, q3)), whose
// terms are all small next to E0.
static __device__ __forceinline__ float pair_solve_inl(const F9 Dv, float sc, const Side& si, const Side& sj,
                                                      const RefPair& rp, bool same, const FrameTerms& t, bool* flag,
                                                      float* qout = nullptr) {
  const float* D = Dv.v;
  const float W = t.W;
  const float trD = sc * (D[0] + D[4] + D[8]);
  float Y[9], G00, g00mag;
  if (same) {
#pragma unroll
    for (int k = 0; k < 9; ++k) Y[k] = fmaf(sc, D[k], si.Q[k] + sj.Q[k]);
    G00 = (si.c + sj.c) - trD;
    g00mag = (si.m + sj.m) + fabsf(trD);
  } else {
    // sc folded into U: Y = Q_i + Q_j + (sc U) Dv
    float U[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) U[k] = sc * rpv(rp, k);
    float trUD = 0.f;
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        trUD = fmaf(U[p * 3 + q], D[q * 3 + p], trUD);
        Y[p * 3 + q] = fmaf(U[p * 3 + 2], D[6 + q],
                            fmaf(U[p * 3 + 1], D[3 + q], fmaf(U[p * 3], D[q], si.Q[p * 3 + q] + sj.Q[p * 3 + q])));
      }
    const float hs = 0.5f * rpv(rp, 21);
    G00 = hs + (si.c + sj.c) - trUD;
    g00mag = hs + (si.m + sj.m) + fabsf(trUD);
  }
  // Contraction error: products of uncorrelated residuals sum with random
  // signs (error ~ eps*sqrt(n_i n_j), independent of N), correlated ones with
  // one sign (rounding errors random-walk: ~ eps*sqrt(N)*|tr D|).
  const float gem = t.gem_s * (si.sn * sj.sn) + t.gem_c * fabsf(trD);
  if (t.nofit) {
    // RMSD_NoFit: sum w |x_i - x_j|^2 / W = 2*G00/W (references are not rotated).
    const float r = sqrtf(fmaxf(G00 * t.two_over_w, 0.0f));
    const float err = 2.0f * gem + t.epi_coef * g00mag;
    *flag = !(err <= t.tol * W * fmaxf(r, 1e-3f));
    return r;
  }
  float M[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) M[k] = rpv(rp, 9 + k) + Y[k];
  // g = G[0][1..3] = -(antisymmetric combos of M''), from the small parts.
  const float g1 = -(Y[5] - Y[7] + rpv(rp, 18));
  const float g2 = -(Y[6] - Y[2] + rpv(rp, 19));
  const float g3 = -(Y[1] - Y[3] + rpv(rp, 20));
  // A = Gs - G00 I
  const float a00 = 2.0f * (M[4] + M[8]), a11 = 2.0f * (M[0] + M[8]), a22 = 2.0f * (M[0] + M[4]);
  const float a01 = -(M[1] + M[3]), a02 = -(M[6] + M[2]), a12 = -(M[5] + M[7]);
  // Power-series solve.
  const float c00 = a11 * a22 - a12 * a12, c01 = a02 * a12 - a01 * a22, c02 = a01 * a12 - a02 * a11;
  const float c11 = a00 * a22 - a02 * a02, c12 = a01 * a02 - a00 * a12, c22 = a00 * a11 - a01 * a01;
  const float det = a00 * c00 + a01 * c01 + a02 * c02;
  const float id = __fdividef(1.0f, det);
  const float w0x = (c00 * g1 + c01 * g2 + c02 * g3) * id;
  const float w0y = (c01 * g1 + c11 * g2 + c12 * g3) * id;
  const float w0z = (c02 * g1 + c12 * g2 + c22 * g3) * id;
  const float w1x = (c00 * w0x + c01 * w0y + c02 * w0z) * id;
  const float w1y = (c01 * w0x + c11 * w0y + c12 * w0z) * id;
  const float w1z = (c02 * w0x + c12 * w0y + c22 * w0z) * id;
  const float s0 = g1 * w0x + g2 * w0y + g3 * w0z;
  const float s1 = w0x * w0x + w0y * w0y + w0z * w0z;
  const float dl = -__fdividef(s0, 1.0f + s1);
  // |delta| <= |delta0| (1 + rho^2 / (1 - rho)) <= 1.09 |delta0| while rho < 1/4.
  const float rho = 1.125f * fabsf(dl) * ((c00 + c11 + c22) * id);
  float q0 = 1.0f;
  float q1 = -(w0x + dl * w1x), q2 = -(w0y + dl * w1y), q3 = -(w0z + dl * w1z);
  // |e|^2 <= s1 rho^4 ((1 + rho) / (1 - rho))^2 <= 2.78 s1 rho^4 for rho < 1/4
  const float rho2 = rho * rho;
  const float trG = 4.0f * G00 + (a00 + a11 + a22);
  float trunc = trG * (2.78f * s1 * rho2 * rho2);
  const bool fast = (a00 > 0.0f) && (c22 > 0.0f) && (det > 0.0f) && (rho < 0.25f) && (s1 < 0.25f) &&
                    (q1 * q1 + q2 * q2 + q3 * q3 < 0.25f) && (trunc <= 0.125f * t.epi_coef * g00mag);
  if (!fast) {
    trunc = 0.0f;
    // Fixed-point iteration on the secular equation: delta = g.v(delta).
    float d = 0.f, v1 = 0.f, v2 = 0.f, v3 = 0.f, det2 = 0.f, m2 = 0.f;
    bool conv = false;
#pragma unroll 1
    for (int it = 0; it < 5; ++it) {
      det2 = solve_sym3(a00 - d, a01, a02, a11 - d, a12, a22 - d, -g1, -g2, -g3, v1, v2, v3, m2);
      const float dn = g1 * v1 + g2 * v2 + g3 * v3;
      conv = fabsf(dn - d) <= 1e-5f * fabsf(G00 + dn) + 1e-30f;
      d = dn;
      if (conv) break;
    }
    const float b00 = a00 - d;
    const bool pd = (b00 > 0.0f) && (b00 * (a11 - d) - a01 * a01 > 0.0f) && (det2 > 0.0f);
    if (conv && pd && (v1 * v1 + v2 * v2 + v3 * v3) < 0.25f) {
      q1 = v1; q2 = v2; q3 = v3;
    } else {
      float q[4];
      qcp_vec_f32(M, G00 + M[0] + M[4] + M[8], q);
      q0 = q[0]; q1 = q[1]; q2 = q[2]; q3 = q[3];
    }
  }
  const float qq = q0 * q0 + q1 * q1 + q2 * q2 + q3 * q3;
  const float iqq = __fdividef(1.0f, qq);  // qq in [1, 1.25) on the iterative paths
  const float tg = q1 * g1 + q2 * g2 + q3 * g3;
  const float d11 = a00 * q1 * q1, d22 = a11 * q2 * q2, d33 = a22 * q3 * q3;
  const float o12 = a01 * q1 * q2, o13 = a02 * q1 * q3, o23 = a12 * q2 * q3;
  const float corr = 2.0f * q0 * tg + (d11 + d22 + d33) + 2.0f * (o12 + o13 + o23);
  const float rq = G00 + corr * iqq;
  const float mag = g00mag + (2.0f * fabsf(q0) * (fabsf(q1 * g1) + fabsf(q2 * g2) + fabsf(q3 * g3)) +
                              (fabsf(d11) + fabsf(d22) + fabsf(d33)) + 2.0f * (fabsf(o12) + fabsf(o13) + fabsf(o23))) *
                                 iqq;
  const float r = sqrtf(fmaxf(rq * t.two_over_w, 0.0f));
  const float err = t.epi_coef * mag + 2.0f * gem + trunc;
  *flag = !(err <= t.tol * W * fmaxf(r, 1e-3f));
  if (qout) {
    const float inv = rsqrtf(qq);
    const float sgn = (q0 < 0.0f) ? -inv : inv;
    qout[0] = q0 * sgn; qout[1] = q1 * sgn; qout[2] = q2 * sgn; qout[3] = q3 * sgn;
  }
  return r;
}

// The same as a call: the CUDA-core kernels, whose per-thread state already
// fills the register file, keep the solver out of line.
static __device__ __noinline__ float pair_solve(const F9 Dv, const Side& si, const Side& sj, const RefPair& rp,
                                                bool same, const FrameTerms& t, bool* flag, float* qout = nullptr) {
  return pair_solve_inl(Dv, 1.0f, si, sj, rp, same, t, flag, qout);
}

// The solver's inputs for pair (i, j), every per-frame term read from
// global memory and combined with the pair's references.
struct PairIn {
  Side si, sj;
  RefPair rp;
  bool same;
};
static __device__ __forceinline__ void pair_terms(int64_t i, int64_t j, const FrameTerms& t, PairIn& in) {
  const int K = t.K;
  const int a = (K > 1) ? __ldg(t.assign + i) : 0;
  const int b = (K > 1) ? __ldg(t.assign + j) : 0;
  const bool same = (a == b);
  const float* rp = t.RP + (size_t)(b * K + a) * kRefPairStride;
  load_refpair(rp, in.rp);
  float Pib[9], Pja[9], U[9];
  const float* pib = t.P + ((size_t)i * K + b) * 9;
  const float* pja = t.P + ((size_t)j * K + a) * 9;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    Pib[k] = __ldg(pib + k);
    Pja[k] = __ldg(pja + k);
    U[k] = same ? 0.0f : rpv(in.rp, k);
  }
  const float trPia = same ? 0.0f : __ldg(t.trP + i * K + a);
  const float trPjb = same ? 0.0f : __ldg(t.trP + j * K + b);
  side_terms(Pib, __ldg(t.nrm + i), trPia, U, same, true, in.si);
  side_terms(Pja, __ldg(t.nrm + j), trPjb, U, same, false, in.sj);
  in.same = same;
}

static __device__ __forceinline__ float pair_epilogue(const float D[9], int64_t i, int64_t j, const FrameTerms& t,
                                                      bool* flag, float* qout = nullptr) {
  PairIn in;
  pair_terms(i, j, t, in);
  F9 dv;
#pragma unroll
  for (int k = 0; k < 9; ++k) dv.v[k] = D[k];
  return pair_solve(dv, in.si, in.sj, in.rp, in.same, t, flag, qout);
}

__host__ __device__ inline int64_t tri_index(int64_t n, int64_t i, int64_t j) {
  return n * i - ((i + 1) * i) / 2 + j - i - 1;
}

// Where each pair's value goes, and which pairs exist.
struct OutMap {
  float* out;
  int64_t n_ref;      // reference frames (set frames [0, n_ref))
  int64_t tgt0;       // set index of target frame 0 (0 for TRI, n_ref for FULL)
  int64_t n_tgt;
  int tri;            // 1 = triangle
  int64_t row_begin;  // TRI: ref rows; FULL: target rows
  int64_t row_end;
  int64_t base;       // TRI: tri_index of the first element of row_begin
  const int* perm;    // TRI over reference-sorted positions: position -> frame
                      // (whole triangle only; nullptr = positions are frames)
};

// i: reference frame (0..n_ref), jt: target frame (0..n_tgt).  Returns -1 if
// the pair is not part of this call's output.
__device__ __forceinline__ int64_t out_index(const OutMap& m, int64_t i, int64_t jt) {
  if (m.tri) {
    if (!(jt > i) || i < m.row_begin || i >= m.row_end || jt >= m.n_tgt) return -1;
    if (m.perm) {
      int64_t a = m.perm[i], b = m.perm[jt];
      if (a > b) {
        const int64_t c = a; a = b; b = c;
      }
      return tri_index(m.n_ref, a, b);
    }
    return tri_index(m.n_ref, i, jt) - m.base;
  }
  if (i >= m.n_ref || jt < m.row_begin || jt >= m.row_end) return -1;
  return (jt - m.row_begin) * m.n_ref + i;
}

struct FlagList {
  int2* pairs;               // (ref frame, target frame) of flagged pairs
  unsigned long long* count; // atomically incremented
  unsigned long long cap;
};

// Records a pair for the FP64 re-check, as (reference frame, target frame)
// of the caller's numbering (sorted positions mapped back through m.perm).
__device__ __forceinline__ void flag_pair(const FlagList& fl, const OutMap& m, int64_t i, int64_t jt) {
  if (m.perm) {
    int64_t a = m.perm[i], b = m.perm[jt];
    if (a > b) {
      const int64_t c = a; a = b; b = c;
    }
    i = a;
    jt = b;
  }
  const unsigned long long k = atomicAdd(fl.count, 1ull);
  if (k < fl.cap) fl.pairs[k] = make_int2((int)i, (int)jt);
}

}  // namespace gbr
