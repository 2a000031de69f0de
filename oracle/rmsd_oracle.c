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
enum { ORC_FIT = 0, ORC_NOFIT = 1, ORC_QCP = 2 };
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

/* Kabsch RMSD of target to a centred ref (Frame::RMSD_CenteredRef). */
double orc_rmsd_centered_ref(const double *ref, const double *tgt, int n, const double *mass) {
  double R[9], E0;
  double W = target_moments(ref, tgt, n, mass, R, &E0);
  if (W < 0.0) return -1.0;
  /* RR^T: rows of R dotted pairwise. */
  double RRt[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      RRt[3 * i + j] = R[3 * i] * R[3 * j] + R[3 * i + 1] * R[3 * j + 1] + R[3 * i + 2] * R[3 * j + 2];
  double v[9], d[3], e[9], mu[3];
  if (jacobi3(RRt, v, d)) return 0.0; /* non-convergence returns 0, as the reference does */
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
  double r = E0 - sqrt(fabs(mu[0])) - sqrt(fabs(mu[1])) - sig3 * sqrt(fabs(mu[2]));
  if (r < 0.0) return 0.0;
  return sqrt(2.0 * r / W);
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
      if (mode != ORC_NOFIT) {
        double c[3];
        orc_center(R, n_atom, ref_mass, c);
        for (int a = 0; a < n_atom; ++a) {
          R[3 * a] -= c[0]; R[3 * a + 1] -= c[1]; R[3 * a + 2] -= c[2];
        }
      }
      int64_t j0 = (out_kind == ORC_TRI) ? i + 1 : j_lo;
      for (int64_t j = j0; j < j_hi; ++j) {
        load_frame(tgt_xyz, dtype, j, n_atom, T);
        double r;
        if (mode == ORC_FIT) r = orc_rmsd_centered_ref(R, T, n_atom, tgt_mass);
        else if (mode == ORC_QCP) r = orc_rmsd_qcp(R, T, n_atom, tgt_mass);
        else r = orc_rmsd_nofit(R, T, n_atom, tgt_mass);
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
      if (mode != ORC_NOFIT) {
        double c[3];
        orc_center(R, n_atom, ref_mass, c);
        for (int a = 0; a < n_atom; ++a) {
          R[3 * a] -= c[0]; R[3 * a + 1] -= c[1]; R[3 * a + 2] -= c[2];
        }
      }
      int64_t j0 = (out_kind == ORC_TRI) ? i + 1 : 0;
      for (int64_t j = j0; j < n_tgt; ++j) {
        load_frame(tgt_xyz, dtype, j, n_atom, T);
        double r;
        if (mode == ORC_FIT) r = orc_rmsd_centered_ref(R, T, n_atom, tgt_mass);
        else if (mode == ORC_QCP) r = orc_rmsd_qcp(R, T, n_atom, tgt_mass);
        else r = orc_rmsd_nofit(R, T, n_atom, tgt_mass);
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
      if (mode != ORC_NOFIT) {
        double c[3];
        orc_center(R, n_atom, mass, c);
        for (int a = 0; a < n_atom; ++a) {
          R[3 * a] -= c[0]; R[3 * a + 1] -= c[1]; R[3 * a + 2] -= c[2];
        }
      }
      double r;
      if (mode == ORC_FIT) r = orc_rmsd_centered_ref(R, T, n_atom, mass);
      else if (mode == ORC_QCP) r = orc_rmsd_qcp(R, T, n_atom, mass);
      else r = orc_rmsd_nofit(R, T, n_atom, mass);
      if (r < 0.0) err |= 2;
      out[k] = r;
    }
    free(R);
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
