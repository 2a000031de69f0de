/*
 * rmsd_oracle.c -- CPU oracle for the all-pairs best-fit RMSD path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * library in cpptraj_gb300/csrc.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it.  The product path never calls it.
 *
 * It restates, in FP64 C, the arithmetic of cpptraj's per-pair RMSD:
 *   - Frame::RMSD_CenteredRef        src/Frame.cpp:1137-1273  (Kabsch via RR^T)
 *   - Matrix_3x3::Diagonalize        src/Matrix_3x3.cpp:110-211 (cyclic Jacobi)
 *   - Matrix_3x3::Diagonalize_Sort   src/Matrix_3x3.cpp:219-280
 *   - Frame::RMSD_NoFit              src/Frame.cpp:1279-1307
 *   - Frame::DISTRMSD                src/Frame.cpp:1313-1344 (rms2d `dme`)
 *   - Action_Rmsd / Action_Align per-frame fit, Frame::Trans_Rot_Trans
 *                                    (orc_superpose_f64)
 *   - Metric_RMS::CalculateCentroid  src/Cluster/Metric_RMS.cpp:86-108
 *                                    (orc_cluster_centroids_f64)
 *   - Frame::CenterOnOrigin          src/Frame.cpp:1043-1055, Frame.h:373-391
 *   - QCPRot::FastCalcRMSDAndRotation src/qcprot.cpp:167-246 (RMSD part) and
 *     do_quaternion_rmsd              src/QuaternionRMSD.cpp:25-120
 * and the pair loops of
 *   - Analysis_Rms2d::Calculate_2D   src/Analysis_Rms2d.cpp:196-295
 *   - MetricArray::calcFrameDistances src/Cluster/MetricArray.cpp:766-801
 * with the output index functions of Matrix<T> (src/Matrix.h:94-122).
 *
 * Parity pinning: the rms2d golden files of test/Test_2DRMS are reproduced by
 * tests/test_oracle_golden.py, and the restatement is compared with the
 * reference's own Frame code built from its sources (oracle/Makefile, target
 * "ref") on random inputs where that build is available.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Constants::SMALL (src/Constants.h:35). */
#define ORC_SMALL 1.0e-14
/* Matrix_3x3::MAX_ITERATIONS_ (src/Matrix_3x3.cpp:97). */
#define ORC_JACOBI_SWEEPS 50

enum { ORC_F32 = 0, ORC_F64 = 1 };
enum { ORC_FIT = 0, ORC_NOFIT = 1, ORC_QCP = 2, ORC_DME = 3 };
enum { ORC_TRI = 0, ORC_FULL = 1 };

/* ------------------------------------------------------------------------ */
/* Cyclic Jacobi eigen-decomposition of a symmetric 3x3 matrix.              */
/* Same sweep schedule as Matrix_3x3::Diagonalize: a threshold of            */
/* 0.2*sum|offdiag|/9 in the first three sweeps, zero afterwards; after the  */
/* fourth sweep off-diagonal entries negligible against both diagonal        */
/* entries are zeroed outright; eigenvectors accumulate as COLUMNS of v.     */
/* Returns 0 on convergence, 1 after ORC_JACOBI_SWEEPS sweeps.               */
/* ------------------------------------------------------------------------ */
static void jrot(double *m, int g, int h, double s, double tau) {
  double a = m[g], b = m[h];
  m[g] = a - s * (b + a * tau);
  m[h] = b + s * (a - b * tau);
}

static int jacobi3(const double *in, double *v, double *d) {
  double a[9];
  memcpy(a, in, sizeof a);
  for (int k = 0; k < 9; ++k) v[k] = (k % 4 == 0) ? 1.0 : 0.0;
  double base[3] = {a[0], a[4], a[8]};
  double acc[3] = {0.0, 0.0, 0.0};
  d[0] = a[0]; d[1] = a[4]; d[2] = a[8];
  for (int sweep = 0; sweep < ORC_JACOBI_SWEEPS; ++sweep) {
    double off = fabs(a[1]) + fabs(a[2]) + fabs(a[5]);
    if (off == 0.0) return 0;
    double thresh = (sweep < 3) ? 0.2 * off / 9.0 : 0.0;
    for (int p = 0; p < 2; ++p) {
      for (int q = p + 1; q < 3; ++q) {
        int pq = 3 * p + q;
        double big = 100.0 * fabs(a[pq]);
        if (sweep > 3 && fabs(d[p]) + big == fabs(d[p]) && fabs(d[q]) + big == fabs(d[q])) {
          a[pq] = 0.0;
          continue;
        }
        if (!(fabs(a[pq]) > thresh)) continue;
        double diff = d[q] - d[p];
        double t;
        if (fabs(diff) + big == fabs(diff)) {
          t = a[pq] / diff;
        } else {
          double theta = 0.5 * diff / a[pq];
          t = 1.0 / (fabs(theta) + sqrt(1.0 + theta * theta));
          if (theta < 0.0) t = -t;
        }
        double c = 1.0 / sqrt(1.0 + t * t);
        double s = t * c;
        double tau = s / (1.0 + c);
        double shift = t * a[pq];
        acc[p] -= shift; acc[q] += shift;
        d[p] -= shift;   d[q] += shift;
        a[pq] = 0.0;
        /* Rotate the remaining upper-triangle entries touched by (p,q). */
        for (int j = 0; j < p; ++j) jrot(a, 3 * j + p, 3 * j + q, s, tau);
        for (int j = p + 1; j < q; ++j) jrot(a, 3 * p + j, 3 * j + q, s, tau);
        for (int j = q + 1; j < 3; ++j) jrot(a, 3 * p + j, 3 * q + j, s, tau);
        for (int j = 0; j < 3; ++j) jrot(v, 3 * j + p, 3 * j + q, s, tau);
      }
    }
    for (int k = 0; k < 3; ++k) {
      base[k] += acc[k];
      d[k] = base[k];
      acc[k] = 0.0;
    }
  }
  return 1;
}

/* Sort eigenpairs in descending order with Diagonalize_Sort's strict-">"  */
/* tie rules; output eigenvectors as ROWS of e.                              */
static void sort_eigen(const double *v, const double *d, double *e, double *dout) {
  int i1, i2, i3;
  if (d[0] > d[1] && d[0] > d[2]) {
    if (d[1] > d[2]) { i1 = 0; i2 = 1; i3 = 2; } else { i1 = 0; i2 = 2; i3 = 1; }
  } else if (d[1] > d[0] && d[1] > d[2]) {
    if (d[0] > d[2]) { i1 = 1; i2 = 0; i3 = 2; } else { i1 = 1; i2 = 2; i3 = 0; }
  } else if (d[0] > d[1]) {
    i1 = 2; i2 = 0; i3 = 1;
  } else {
    i1 = 2; i2 = 1; i3 = 0;
  }
  int idx[3] = {i1, i2, i3};
  for (int r = 0; r < 3; ++r) {
    for (int k = 0; k < 3; ++k) e[3 * r + k] = v[3 * k + idx[r]];
    dout[r] = d[idx[r]];
  }
}

static void unit3(double *x) {
  double s = 1.0 / sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  x[0] *= s; x[1] *= s; x[2] *= s;
}

/* ------------------------------------------------------------------------ */
/* Per-pair kernels (FP64).  `ref` is already centred; `tgt` is centred here */
/* with the target masses, as Frame::RMSD_CenteredRef does.                  */
/* ------------------------------------------------------------------------ */

/* Weighted (or geometric) centre, as Frame::VCenterOfMass/VGeometricCenter. */
void orc_center(const double *x, int n, const double *mass, double *c) {
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, m = 0.0;
  for (int a = 0; a < n; ++a) {
    double w = mass ? mass[a] : 1.0;
    s0 += x[3 * a] * w; s1 += x[3 * a + 1] * w; s2 += x[3 * a + 2] * w;
    m += w;
  }
  if (mass && m == 0.0) { c[0] = c[1] = c[2] = 0.0; return; }
  c[0] = s0 / m; c[1] = s1 / m; c[2] = s2 / m;
}

/* Centre target, accumulate E0 and R[p][q] = sum w t_p r_q; return W or -1. */
static double target_moments(const double *ref, const double *tgt, int n, const double *mass,
                             double *rot, double *e0) {
  double tc[3] = {0.0, 0.0, 0.0}, W = 0.0;
  for (int a = 0; a < n; ++a) {
    double w = mass ? mass[a] : 1.0;
    tc[0] += tgt[3 * a] * w; tc[1] += tgt[3 * a + 1] * w; tc[2] += tgt[3 * a + 2] * w;
    if (mass) W += w;
  }
  if (!mass) W = (double)n;
  if (W < ORC_SMALL) return -1.0;
  tc[0] /= W; tc[1] /= W; tc[2] /= W;
  double ss = 0.0;
  for (int k = 0; k < 9; ++k) rot[k] = 0.0;
  for (int a = 0; a < n; ++a) {
    double w = mass ? mass[a] : 1.0;
    double t0 = tgt[3 * a] - tc[0], t1 = tgt[3 * a + 1] - tc[1], t2 = tgt[3 * a + 2] - tc[2];
    double r0 = ref[3 * a], r1 = ref[3 * a + 1], r2 = ref[3 * a + 2];
    ss += w * (t0 * t0 + t1 * t1 + t2 * t2 + r0 * r0 + r1 * r1 + r2 * r2);
    rot[0] += w * t0 * r0; rot[1] += w * t0 * r1; rot[2] += w * t0 * r2;
    rot[3] += w * t1 * r0; rot[4] += w * t1 * r1; rot[5] += w * t1 * r2;
    rot[6] += w * t2 * r0; rot[7] += w * t2 * r1; rot[8] += w * t2 * r2;
  }
  *e0 = 0.5 * ss;
  return W;
}

/* Kabsch RMSD of target to a centred ref (Frame::RMSD_CenteredRef); with U
 * non-NULL also the best rotation U (row-major, U y ~ r for the centred
 * target y), built as at src/Frame.cpp:1239-1250. */
static double fit_centered_ref(const double *ref, const double *tgt, int n, const double *mass, double *U) {
  double R[9], E0;
  double W = target_moments(ref, tgt, n, mass, R, &E0);
  if (W < 0.0) return -1.0;
  /* RR^T: rows of R dotted pairwise. */
  double RRt[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      RRt[3 * i + j] = R[3 * i] * R[3 * j] + R[3 * i + 1] * R[3 * j + 1] + R[3 * i + 2] * R[3 * j + 2];
  double v[9], d[3], e[9], mu[3];
  if (jacobi3(RRt, v, d)) { /* non-convergence returns 0, as the reference does */
    if (U) for (int k = 0; k < 9; ++k) U[k] = (k % 4 == 0) ? 1.0 : 0.0;
    return 0.0;
  }
  sort_eigen(v, d, e, mu);
  /* Third axis is the cross product of the first two. */
  e[6] = e[1] * e[5] - e[2] * e[4];
  e[7] = e[2] * e[3] - e[0] * e[5];
  e[8] = e[0] * e[4] - e[1] * e[3];
  double b[9];
  for (int k = 0; k < 3; ++k) {
    for (int q = 0; q < 3; ++q)
      b[3 * k + q] = e[3 * k] * R[q] + e[3 * k + 1] * R[3 + q] + e[3 * k + 2] * R[6 + q];
    unit3(b + 3 * k);
  }
  double cp[3] = {b[1] * b[5] - b[2] * b[4], b[2] * b[3] - b[0] * b[5], b[0] * b[4] - b[1] * b[3]};
  double sig3 = (cp[0] * b[6] + cp[1] * b[7] + cp[2] * b[8] < 0.0) ? -1.0 : 1.0;
  if (U) {
    b[6] = cp[0]; b[7] = cp[1]; b[8] = cp[2];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) U[3 * i + j] = e[j] * b[i] + e[3 + j] * b[3 + i] + e[6 + j] * b[6 + i];
  }
  double r = E0 - sqrt(fabs(mu[0])) - sqrt(fabs(mu[1])) - sig3 * sqrt(fabs(mu[2]));
  if (r < 0.0) return 0.0;
  return sqrt(2.0 * r / W);
}

double orc_rmsd_centered_ref(const double *ref, const double *tgt, int n, const double *mass) {
  return fit_centered_ref(ref, tgt, n, mass, NULL);
}

/* Quaternion (QCP) RMSD of target to a centred ref: Newton iteration from   */
/* E0 on the characteristic quartic of the 4x4 key matrix.                   */
double orc_rmsd_qcp(const double *ref, const double *tgt, int n, const double *mass) {
  double A[9], E0;
  double W = target_moments(ref, tgt, n, mass, A, &E0);
  if (W < 0.0) return -1.0;
  double xx = A[0], xy = A[1], xz = A[2], yx = A[3], yy = A[4], yz = A[5], zx = A[6], zy = A[7], zz = A[8];
  double xx2 = xx * xx, yy2 = yy * yy, zz2 = zz * zz, xy2 = xy * xy, yz2 = yz * yz, xz2 = xz * xz;
  double yx2 = yx * yx, zy2 = zy * zy, zx2 = zx * zx;
  double c2 = -2.0 * (xx2 + yy2 + zz2 + xy2 + yx2 + xz2 + zx2 + yz2 + zy2);
  double c1 = 8.0 * (xx * yz * zy + yy * zx * xz + zz * xy * yx - xx * yy * zz - yz * zx * xy - zy * yx * xz);
  double t1 = 2.0 * (yz * zy - yy * zz);
  double t2 = yy2 + zz2 - xx2 + yz2 + zy2;
  double t3 = xy2 + xz2 - yx2 - zx2;
  double pxz = xz + zx, pyz = yz + zy, pxy = xy + yx, myz = yz - zy, mxz = xz - zx, mxy = xy - yx;
  double pxx = xx + yy, mxx = xx - yy;
  double c0 = t3 * t3 + (t2 + t1) * (t2 - t1)
            + (-pxz * myz + mxy * (mxx - zz)) * (-mxz * pyz + mxy * (mxx + zz))
            + (-pxz * pyz - pxy * (pxx - zz)) * (-mxz * myz - pxy * (pxx + zz))
            + (pxy * pyz + pxz * (mxx + zz)) * (-mxy * myz + pxz * (pxx + zz))
            + (pxy * myz + mxz * (mxx - zz)) * (-mxy * pyz + mxz * (pxx - zz));
  double lam = E0;
  for (int it = 0; it < 50; ++it) {
    double prev = lam;
    double l2 = lam * lam;
    double b = (l2 + c2) * lam;
    double a = b + c1;
    lam -= (a * lam + c0) / (2.0 * l2 * lam + b + a);
    if (fabs(lam - prev) < fabs(1e-11 * lam)) break;
  }
  return sqrt(fabs(2.0 * (E0 - lam) / W));
}

/* RMSD without fitting (Frame::RMSD_NoFit); masses are the target's. */
double orc_rmsd_nofit(const double *ref, const double *tgt, int n, const double *mass) {
  double s = 0.0, W = 0.0;
  for (int a = 0; a < n; ++a) {
    double w = mass ? mass[a] : 1.0;
    double dx = ref[3 * a] - tgt[3 * a], dy = ref[3 * a + 1] - tgt[3 * a + 1], dz = ref[3 * a + 2] - tgt[3 * a + 2];
    W += w;
    s += w * (dx * dx + dy * dy + dz * dz);
  }
  if (W < ORC_SMALL) return -1.0;
  if (s < 0.0) return 0.0;
  return sqrt(s / W);
}

/* Distance RMSD (Frame::DISTRMSD, src/Frame.cpp:1313-1344): over atom pairs
 * a < b (a outer, b inner), the squared difference of the target's and the
 * reference's a-b distances, summed in that order; sqrt(sum / (N^2 - N)/2).
 * No masses, no centring.  N = 1 gives 0/0, as in the reference. */
double orc_rmsd_dme(const double *ref, const double *tgt, int n) {
  const double nd = (double)((n * n) - n) / 2.0;
  double sum = 0.0;
  for (int a = 0; a < n - 1; ++a) {
    for (int b = a + 1; b < n; ++b) {
      double x = tgt[3 * a] - tgt[3 * b], y = tgt[3 * a + 1] - tgt[3 * b + 1], z = tgt[3 * a + 2] - tgt[3 * b + 2];
      const double dt = sqrt(x * x + y * y + z * z);
      x = ref[3 * a] - ref[3 * b]; y = ref[3 * a + 1] - ref[3 * b + 1]; z = ref[3 * a + 2] - ref[3 * b + 2];
      const double dr = sqrt(x * x + y * y + z * z);
      const double d = dt - dr;
      sum += d * d;
    }
  }
  return sqrt(sum / nd);
}

static double pair_value(int mode, const double *R, const double *T, int n, const double *mass) {
  if (mode == ORC_FIT) return orc_rmsd_centered_ref(R, T, n, mass);
  if (mode == ORC_QCP) return orc_rmsd_qcp(R, T, n, mass);
  if (mode == ORC_DME) return orc_rmsd_dme(R, T, n);
  return orc_rmsd_nofit(R, T, n, mass);
}

/* Calculate_2D centres the reference frame for fit and qrmsd only
 * (src/Analysis_Rms2d.cpp:265-266). */
static int centres_ref(int mode) { return mode == ORC_FIT || mode == ORC_QCP; }

/* ------------------------------------------------------------------------ */
/* All-pairs driver with Calculate_2D semantics.                             */
/*   rows = reference frames (nref), columns = target frames (ntgt).         */
/*   TRI  : ref set == tgt set, pairs nref < ntgt, index calcTriIndex.       */
/*   FULL : every (nref, ntgt), index ntgt*n_ref + nref (calcFullIndex).     */
/*   Row ranges: TRI rows are reference frames, FULL rows are target frames */
/*   (the slow index); out holds exactly rows [row_begin, row_end).          */
/* ------------------------------------------------------------------------ */
int64_t orc_tri_index(int64_t n, int64_t i, int64_t j) {
  return n * i - ((i + 1) * i) / 2 + j - i - 1;
}

static void load_frame(const void *base, int dtype, int64_t f, int n, double *dst) {
  if (dtype == ORC_F64) {
    memcpy(dst, (const double *)base + (size_t)f * 3 * n, sizeof(double) * 3 * (size_t)n);
  } else {
    const float *s = (const float *)base + (size_t)f * 3 * n;
    for (int k = 0; k < 3 * n; ++k) dst[k] = (double)s[k];
  }
}

int orc_allpairs(const void *ref_xyz, const void *tgt_xyz, int dtype, int64_t n_ref, int64_t n_tgt,
                 int n_atom, const double *ref_mass, const double *tgt_mass, int mode, int out_kind,
                 float *out, int64_t row_begin, int64_t row_end, int nthreads) {
  if (n_atom < 1 || n_ref < 0 || n_tgt < 0) return 1;
  if (tgt_xyz == NULL) { tgt_xyz = ref_xyz; n_tgt = n_ref; }
  if (out_kind == ORC_TRI && n_tgt != n_ref) return 1;
  int64_t n_rows = (out_kind == ORC_TRI) ? n_ref : n_tgt;
  if (row_end < 0 || row_end > n_rows) row_end = n_rows;
  if (row_begin < 0) row_begin = 0;
  int64_t base = 0;
  if (out_kind == ORC_TRI) base = (row_begin < n_ref - 1) ? orc_tri_index(n_ref, row_begin, row_begin + 1) : 0;
  /* reference frames to visit: TRI restricts them, FULL restricts targets */
  int64_t i_begin = (out_kind == ORC_TRI) ? row_begin : 0;
  int64_t i_end = (out_kind == ORC_TRI) ? row_end : n_ref;
  int64_t j_lo = (out_kind == ORC_TRI) ? 0 : row_begin;
  int64_t j_hi = (out_kind == ORC_TRI) ? n_tgt : row_end;
  int err = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(| : err)
#endif
  {
    double *R = (double *)malloc(sizeof(double) * 3 * (size_t)n_atom);
    double *T = (double *)malloc(sizeof(double) * 3 * (size_t)n_atom);
#ifdef _OPENMP
#pragma omp for schedule(dynamic)
#endif
    for (int64_t i = i_begin; i < i_end; ++i) {
      load_frame(ref_xyz, dtype, i, n_atom, R);
      if (centres_ref(mode)) {
        double c[3];
        orc_center(R, n_atom, ref_mass, c);
        for (int a = 0; a < n_atom; ++a) {
          R[3 * a] -= c[0]; R[3 * a + 1] -= c[1]; R[3 * a + 2] -= c[2];
        }
      }
      int64_t j0 = (out_kind == ORC_TRI) ? i + 1 : j_lo;
      for (int64_t j = j0; j < j_hi; ++j) {
        load_frame(tgt_xyz, dtype, j, n_atom, T);
        const double r = pair_value(mode, R, T, n_atom, tgt_mass);
        if (r < 0.0) err |= 2;
        int64_t idx = (out_kind == ORC_TRI) ? orc_tri_index(n_ref, i, j) - base : (j - row_begin) * n_ref + i;
        out[idx] = (float)r;
      }
    }
    free(R);
    free(T);
  }
  return err;
}

/* Same pairs, returned in FP64 (for error statistics against the GPU).  */
int orc_allpairs_f64(const void *ref_xyz, const void *tgt_xyz, int dtype, int64_t n_ref, int64_t n_tgt,
                     int n_atom, const double *ref_mass, const double *tgt_mass, int mode, int out_kind,
                     double *out, int nthreads) {
  if (n_atom < 1) return 1;
  if (tgt_xyz == NULL) { tgt_xyz = ref_xyz; n_tgt = n_ref; }
  int err = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(| : err)
#endif
  {
    double *R = (double *)malloc(sizeof(double) * 3 * (size_t)n_atom);
    double *T = (double *)malloc(sizeof(double) * 3 * (size_t)n_atom);
#ifdef _OPENMP
#pragma omp for schedule(dynamic)
#endif
    for (int64_t i = 0; i < n_ref; ++i) {
      load_frame(ref_xyz, dtype, i, n_atom, R);
      if (centres_ref(mode)) {
        double c[3];
        orc_center(R, n_atom, ref_mass, c);
        for (int a = 0; a < n_atom; ++a) {
          R[3 * a] -= c[0]; R[3 * a + 1] -= c[1]; R[3 * a + 2] -= c[2];
        }
      }
      int64_t j0 = (out_kind == ORC_TRI) ? i + 1 : 0;
      for (int64_t j = j0; j < n_tgt; ++j) {
        load_frame(tgt_xyz, dtype, j, n_atom, T);
        const double r = pair_value(mode, R, T, n_atom, tgt_mass);
        if (r < 0.0) err |= 2;
        int64_t idx = (out_kind == ORC_TRI) ? orc_tri_index(n_ref, i, j) : j * n_ref + i;
        out[idx] = r;
      }
    }
    free(R);
    free(T);
  }
  return err;
}

/* Explicit pair list in FP64: out[k] = RMSD(ref=pi[k], tgt=pj[k]).  */
int orc_pairs_f64(const void *xyz, int dtype, int n_atom, const double *mass, int mode,
                  const int64_t *pi, const int64_t *pj, int64_t npairs, double *out, int nthreads) {
  int err = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(| : err)
#endif
  {
    double *R = (double *)malloc(sizeof(double) * 3 * (size_t)n_atom);
    double *T = (double *)malloc(sizeof(double) * 3 * (size_t)n_atom);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
    for (int64_t k = 0; k < npairs; ++k) {
      load_frame(xyz, dtype, pi[k], n_atom, R);
      load_frame(xyz, dtype, pj[k], n_atom, T);
      if (centres_ref(mode)) {
        double c[3];
        orc_center(R, n_atom, mass, c);
        for (int a = 0; a < n_atom; ++a) {
          R[3 * a] -= c[0]; R[3 * a + 1] -= c[1]; R[3 * a + 2] -= c[2];
        }
      }
      const double r = pair_value(mode, R, T, n_atom, mass);
      if (r < 0.0) err |= 2;
      out[k] = r;
    }
    free(R);
    free(T);
  }
  return err;
}

/* Per-frame fit of n_frame target frames onto one reference frame: the rms
 * action (Action_Rmsd::DoAction, src/Action_Rmsd.cpp:372-395) and align
 * (Action_Align::DoAction, src/Action_Align.cpp:85-99).  Fit: the reference
 * is centred (ReferenceAction::SelectRefAtoms, CenterOnOrigin; ref_trans =
 * its centre) with ref_mass (NULL => mass) when mass is given, geometrically
 * when it is not (one `mass` flag covers both frames); each frame gets RMSD_CenteredRef(ref, U, Trans)
 * with Trans = -(its centre) and, when move is given, Trans_Rot_Trans(Trans,
 * U, ref_trans) of its n_move atoms (Frame.h:572-581).  No-fit: RMSD_NoFit
 * against the uncentred reference, U = I, translations 0, nothing moved.
 * Outputs may be NULL.  move is FP64 [n_frame][n_move][3].  */
int orc_superpose_f64(const void *ref_xyz, const void *xyz, int dtype, int64_t n_frame, int n_atom,
                      const double *ref_mass, const double *mass, int mode, double *rmsd, double *rot,
                      double *tgt_trans, double *ref_trans, double *move, int n_move, int nthreads) {
  if (n_atom < 1) return 1;
  double *R = (double *)malloc(sizeof(double) * 3 * (size_t)n_atom);
  load_frame(ref_xyz, dtype, 0, n_atom, R);
  double rc[3] = {0.0, 0.0, 0.0};
  if (mode == ORC_FIT) {
    orc_center(R, n_atom, mass ? (ref_mass ? ref_mass : mass) : NULL, rc);
    for (int a = 0; a < n_atom; ++a) {
      R[3 * a] -= rc[0]; R[3 * a + 1] -= rc[1]; R[3 * a + 2] -= rc[2];
    }
  }
  if (ref_trans) { ref_trans[0] = rc[0]; ref_trans[1] = rc[1]; ref_trans[2] = rc[2]; }
  int err = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(| : err)
#endif
  {
    double *T = (double *)malloc(sizeof(double) * 3 * (size_t)n_atom);
#ifdef _OPENMP
#pragma omp for schedule(dynamic)
#endif
    for (int64_t f = 0; f < n_frame; ++f) {
      load_frame(xyz, dtype, f, n_atom, T);
      double U[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, c[3] = {0.0, 0.0, 0.0}, r;
      if (mode == ORC_FIT) {
        orc_center(T, n_atom, mass, c);
        r = fit_centered_ref(R, T, n_atom, mass, U);
      } else {
        r = orc_rmsd_nofit(R, T, n_atom, mass);
      }
      if (r < 0.0) err |= 2;
      if (rmsd) rmsd[f] = r;
      if (rot) memcpy(rot + 9 * f, U, sizeof U);
      if (tgt_trans) { tgt_trans[3 * f] = -c[0]; tgt_trans[3 * f + 1] = -c[1]; tgt_trans[3 * f + 2] = -c[2]; }
      if (move && mode == ORC_FIT) {
        double *m = move + (size_t)f * 3 * n_move;
        for (int a = 0; a < n_move; ++a) {
          const double x = m[3 * a] - c[0], y = m[3 * a + 1] - c[1], z = m[3 * a + 2] - c[2];
          m[3 * a] = x * U[0] + y * U[1] + z * U[2] + rc[0];
          m[3 * a + 1] = x * U[3] + y * U[4] + z * U[5] + rc[1];
          m[3 * a + 2] = x * U[6] + y * U[7] + z * U[8] + rc[2];
        }
      }
    }
    free(T);
  }
  free(R);
  return err;
}

/* Cluster centroids as Metric_RMS::CalculateCentroid builds them
 * (src/Cluster/Metric_RMS.cpp:86-108), one cluster per thread.  Fit: in
 * member order, the first frame centred (CenterOnOrigin) starts the running
 * sum S; every later frame is centred and fitted onto S by
 * RMSD_CenteredRef(S, U, Trans) -- S is not divided first, the rotation does
 * not depend on its scale -- rotated about the origin (Frame::Rotate,
 * src/Frame.h:508-517) and added (Frame::operator+=, src/Frame.cpp:901-910).
 * No-fit: the plain sum of the frames as given.  The centroid is S / n
 * (Frame::Divide, src/Frame.cpp:968-976).  members holds the frame indices of
 * all clusters back to back, cluster c being members[offsets[c] ..
 * offsets[c + 1]).  out: [n_cluster][n_atom][3]; an empty cluster's rows are
 * NaN (the reference leaves a frame with no atoms).  Returns 1 for a bad
 * argument (frame index out of range), 2 when a fit met a zero total mass. */
int orc_cluster_centroids_f64(const void *xyz, int dtype, int64_t n_frame, int n_atom, const double *mass,
                              int mode, const int32_t *members, const int64_t *offsets, int64_t n_cluster,
                              double *out, int nthreads) {
  if (n_atom < 1) return 1;
  for (int64_t c = 0; c < n_cluster; ++c)
    for (int64_t k = offsets[c]; k < offsets[c + 1]; ++k)
      if (members[k] < 0 || members[k] >= n_frame) return 1;
  int err = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(| : err)
#endif
  {
    double *T = (double *)malloc(sizeof(double) * 3 * (size_t)n_atom);
#ifdef _OPENMP
#pragma omp for schedule(dynamic)
#endif
    for (int64_t c = 0; c < n_cluster; ++c) {
      double *S = out + (size_t)c * 3 * n_atom;
      const int64_t n = offsets[c + 1] - offsets[c];
      if (n <= 0) {
        for (int k = 0; k < 3 * n_atom; ++k) S[k] = NAN;
        continue;
      }
      for (int64_t k = 0; k < n; ++k) {
        load_frame(xyz, dtype, members[offsets[c] + k], n_atom, T);
        double tc[3] = {0.0, 0.0, 0.0}, U[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        if (mode == ORC_FIT) {
          if (k > 0 && fit_centered_ref(S, T, n_atom, mass, U) < 0.0) err |= 2;
          orc_center(T, n_atom, mass, tc);
        }
        for (int a = 0; a < n_atom; ++a) {
          const double x = T[3 * a] - tc[0], y = T[3 * a + 1] - tc[1], z = T[3 * a + 2] - tc[2];
          const double r0 = x * U[0] + y * U[1] + z * U[2];
          const double r1 = x * U[3] + y * U[4] + z * U[5];
          const double r2 = x * U[6] + y * U[7] + z * U[8];
          if (k == 0) {
            S[3 * a] = r0; S[3 * a + 1] = r1; S[3 * a + 2] = r2;
          } else {
            S[3 * a] += r0; S[3 * a + 1] += r1; S[3 * a + 2] += r2;
          }
        }
      }
      for (int k = 0; k < 3 * n_atom; ++k) S[k] /= (double)n;
    }
    free(T);
  }
  return err;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Gradient oracle (cpptraj has no RMSD gradient; these are the checks for  */
/* gbr_rmsd_backward).  L = sum_{i<j} g_ij RMSD_ij over one frame set.       */
/* ------------------------------------------------------------------------ */

/* Optimal proper rotation R (row-major) with R*t ~ r for centred t, r, from */
/* the QCP key matrix's top eigenvector (Newton on the quartic, then the     */
/* adjugate column of largest norm).  Returns lambda.                        */
static double qcp_rotation(const double *A, double E0, double *R) {
  double xx = A[0], xy = A[1], xz = A[2], yx = A[3], yy = A[4], yz = A[5], zx = A[6], zy = A[7], zz = A[8];
  double K[16] = {xx + yy + zz, yz - zy, zx - xz, xy - yx,
                  yz - zy, xx - yy - zz, xy + yx, zx + xz,
                  zx - xz, xy + yx, -xx + yy - zz, yz + zy,
                  xy - yx, zx + xz, yz + zy, -xx - yy + zz};
  /* largest eigenvalue by Newton on det(K - l I) starting from E0 */
  double xx2 = xx * xx, yy2 = yy * yy, zz2 = zz * zz, xy2 = xy * xy, yz2 = yz * yz, xz2 = xz * xz;
  double yx2 = yx * yx, zy2 = zy * zy, zx2 = zx * zx;
  double c2 = -2.0 * (xx2 + yy2 + zz2 + xy2 + yx2 + xz2 + zx2 + yz2 + zy2);
  double c1 = 8.0 * (xx * yz * zy + yy * zx * xz + zz * xy * yx - xx * yy * zz - yz * zx * xy - zy * yx * xz);
  double t1 = 2.0 * (yz * zy - yy * zz), t2 = yy2 + zz2 - xx2 + yz2 + zy2, t3 = xy2 + xz2 - yx2 - zx2;
  double pxz = xz + zx, pyz = yz + zy, pxy = xy + yx, myz = yz - zy, mxz = xz - zx, mxy = xy - yx;
  double pxx = xx + yy, mxx = xx - yy;
  double c0 = t3 * t3 + (t2 + t1) * (t2 - t1)
            + (-pxz * myz + mxy * (mxx - zz)) * (-mxz * pyz + mxy * (mxx + zz))
            + (-pxz * pyz - pxy * (pxx - zz)) * (-mxz * myz - pxy * (pxx + zz))
            + (pxy * pyz + pxz * (mxx + zz)) * (-mxy * myz + pxz * (pxx + zz))
            + (pxy * myz + mxz * (mxx - zz)) * (-mxy * pyz + mxz * (pxx - zz));
  double lam = E0;
  for (int it = 0; it < 100; ++it) {
    double prev = lam, l2 = lam * lam, b = (l2 + c2) * lam, a = b + c1;
    double den = 2.0 * l2 * lam + b + a;
    if (den == 0.0) break;
    lam -= (a * lam + c0) / den;
    if (fabs(lam - prev) < fabs(1e-14 * lam)) break;
  }
  double q[4] = {1, 0, 0, 0}, best = -1.0;
  for (int col = 0; col < 4; ++col) {
    double c[4];
    for (int r = 0; r < 4; ++r) {
      int rr[3], cc[3], nr = 0, nc = 0;
      for (int k = 0; k < 4; ++k) {
        if (k != r) rr[nr++] = k;
        if (k != col) cc[nc++] = k;
      }
      double m[9];
      for (int u = 0; u < 3; ++u)
        for (int v = 0; v < 3; ++v) m[3 * u + v] = K[rr[u] * 4 + cc[v]] - ((rr[u] == cc[v]) ? lam : 0.0);
      double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                   m[2] * (m[3] * m[7] - m[4] * m[6]);
      c[r] = ((r + col) & 1) ? -det : det;
    }
    double n2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
    if (n2 > best) { best = n2; memcpy(q, c, sizeof q); }
  }
  double inv = 1.0 / sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  double a = q[0] * inv, b = q[1] * inv, c = q[2] * inv, d = q[3] * inv;
  /* QCP's matrix for q, transposed so that R * t ~ r */
  R[0] = a * a + b * b - c * c - d * d; R[3] = 2 * (b * c + a * d); R[6] = 2 * (d * b - a * c);
  R[1] = 2 * (b * c - a * d); R[4] = a * a - b * b + c * c - d * d; R[7] = 2 * (c * d + a * b);
  R[2] = 2 * (d * b + a * c); R[5] = 2 * (c * d - a * b); R[8] = a * a - b * b - c * c + d * d;
  return lam;
}

static void centre_copy(const float *src, int n, const double *mass, double *dst) {
  for (int k = 0; k < 3 * n; ++k) dst[k] = (double)src[k];
  double c[3];
  orc_center(dst, n, mass, c);
  for (int a = 0; a < n; ++a) { dst[3 * a] -= c[0]; dst[3 * a + 1] -= c[1]; dst[3 * a + 2] -= c[2]; }
}

/* Analytic FP64 gradient: grad[f][a][p] (double), xyz float32. */
int orc_grad_f64(const float *xyz, int64_t F, int n, const double *mass, const float *g, double *grad,
                 int nthreads) {
  double W = 0.0;
  for (int a = 0; a < n; ++a) W += mass ? mass[a] : 1.0;
  memset(grad, 0, sizeof(double) * 3 * (size_t)n * F);
  double *Y = (double *)malloc(sizeof(double) * 3 * (size_t)n * F);
  for (int64_t f = 0; f < F; ++f) centre_copy(xyz + (size_t)f * 3 * n, n, mass, Y + (size_t)f * 3 * n);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
  {
    double *acc = (double *)calloc(3 * (size_t)n * F, sizeof(double));
#ifdef _OPENMP
#pragma omp for schedule(dynamic)
#endif
    for (int64_t i = 0; i < F; ++i) {
      const double *yi = Y + (size_t)i * 3 * n;
      for (int64_t j = i + 1; j < F; ++j) {
        const double *yj = Y + (size_t)j * 3 * n;
        double A[9] = {0}, ss = 0.0;
        for (int a = 0; a < n; ++a) {
          double w = mass ? mass[a] : 1.0;
          for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q) A[3 * p + q] += w * yj[3 * a + p] * yi[3 * a + q];
          for (int p = 0; p < 3; ++p) ss += w * (yi[3 * a + p] * yi[3 * a + p] + yj[3 * a + p] * yj[3 * a + p]);
        }
        double R[9];
        qcp_rotation(A, 0.5 * ss, R);
        /* residuals e = y_i - R y_j, rmsd from them */
        double s2 = 0.0;
        for (int a = 0; a < n; ++a) {
          double w = mass ? mass[a] : 1.0;
          for (int p = 0; p < 3; ++p) {
            double e = yi[3 * a + p] - (R[3 * p] * yj[3 * a] + R[3 * p + 1] * yj[3 * a + 1] + R[3 * p + 2] * yj[3 * a + 2]);
            s2 += w * e * e;
          }
        }
        double rmsd = sqrt(s2 / W);
        if (!(rmsd > 1e-12)) continue;
        double gij = g ? (double)g[orc_tri_index(F, i, j)] : 1.0;
        double c = gij / (W * rmsd);
        double *gi = acc + (size_t)i * 3 * n, *gj = acc + (size_t)j * 3 * n;
        for (int a = 0; a < n; ++a) {
          double w = mass ? mass[a] : 1.0;
          double e[3];
          for (int p = 0; p < 3; ++p)
            e[p] = yi[3 * a + p] - (R[3 * p] * yj[3 * a] + R[3 * p + 1] * yj[3 * a + 1] + R[3 * p + 2] * yj[3 * a + 2]);
          for (int p = 0; p < 3; ++p) {
            gi[3 * a + p] += c * w * e[p];
            gj[3 * a + p] -= c * w * (R[p] * e[0] + R[3 + p] * e[1] + R[6 + p] * e[2]);
          }
        }
      }
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    for (size_t k = 0; k < 3 * (size_t)n * F; ++k) grad[k] += acc[k];
    free(acc);
  }
  free(Y);
  return 0;
}

/* Central finite difference of L with respect to xyz[f][a][p]: only the pairs */
/* containing frame f change.  All arithmetic in FP64.                          */
double orc_fd_f64(const float *xyz, int64_t F, int n, const double *mass, const float *g, int64_t f, int a,
                  int p, double h, int nthreads) {
  double total = 0.0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(+ : total)
#endif
  {
    double *R = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *T = (double *)malloc(sizeof(double) * 3 * (size_t)n);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (int64_t o = 0; o < F; ++o) {
      if (o == f) continue;
      double gw = g ? (double)g[o < f ? orc_tri_index(F, o, f) : orc_tri_index(F, f, o)] : 1.0;
      double val[2];
      for (int s = 0; s < 2; ++s) {
        for (int k = 0; k < 3 * n; ++k) R[k] = (double)xyz[(size_t)o * 3 * n + k];
        for (int k = 0; k < 3 * n; ++k) T[k] = (double)xyz[(size_t)f * 3 * n + k];
        T[3 * a + p] += (s == 0) ? h : -h;
        double c[3];
        orc_center(R, n, mass, c);
        for (int b = 0; b < n; ++b) { R[3 * b] -= c[0]; R[3 * b + 1] -= c[1]; R[3 * b + 2] -= c[2]; }
        double A[9], E0;
        double W = target_moments(R, T, n, mass, A, &E0);
        double Rm[9];
        double lam = qcp_rotation(A, E0, Rm);
        double e = E0 - lam;
        val[s] = (e < 0.0) ? 0.0 : sqrt(2.0 * e / W);
      }
      total += gw * (val[0] - val[1]) / (2.0 * h);
    }
    free(R);
    free(T);
  }
  return total;
}
