// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Thin C entry points over cpptraj's own Frame RMSD code, compiled from the
// reference sources by `make -C oracle ref` into oracle/_ref/.  Used to pin
// the FP64 restatement in rmsd_oracle.c and, in this container, as the
// "reference" CPU baseline.  The loops mirror
//   Analysis_Rms2d::Calculate_2D      (src/Analysis_Rms2d.cpp:247-290)  and
//   Metric_RMS::FrameDist             (src/Cluster/Metric_RMS.cpp:44-63)
// with the work itself done by Frame::RMSD_CenteredRef / RMSD_NoFit /
// QuaternionRMSD_CenteredRef.
#include <cstdint>
#include <vector>
#include "Cluster/Cframes.h"
#include "Cluster/Cmatrix_Binary.h"
#include "FileName.h"
#include "Frame.h"
#include "QuaternionRMSD.h"
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {
void fill(Frame& fr, const void* base, int dtype, int64_t f, int n) {
  double* x = fr.xAddress();
  if (dtype == 1) {
    const double* s = (const double*)base + (size_t)f * 3 * n;
    for (int k = 0; k < 3 * n; ++k) x[k] = s[k];
  } else {
    const float* s = (const float*)base + (size_t)f * 3 * n;
    for (int k = 0; k < 3 * n; ++k) x[k] = (double)s[k];
  }
}
int64_t tri(int64_t n, int64_t i, int64_t j) { return n * i - ((i + 1) * i) / 2 + j - i - 1; }
Frame make(int n, const double* mass) {
  std::vector<double> X(3 * (size_t)n, 0.0), M(n, 1.0);
  if (mass) M.assign(mass, mass + n);
  Frame f;
  f.SetupFrameXM(X, M);
  return f;
}
}  // namespace

// mode: 0 = fit (RMSD_CenteredRef), 1 = nofit, 2 = qrmsd, 3 = dme (DISTRMSD,
// reference not centred, src/Analysis_Rms2d.cpp:265-278).  Same argument meaning
// as orc_allpairs in rmsd_oracle.c.
extern "C" int ref_allpairs(const void* ref_xyz, const void* tgt_xyz, int dtype, int64_t n_ref,
                            int64_t n_tgt, int n_atom, const double* ref_mass, const double* tgt_mass,
                            int mode, int out_kind, float* out, int nthreads) {
  if (tgt_xyz == nullptr) { tgt_xyz = ref_xyz; n_tgt = n_ref; }
  bool use_mass = (tgt_mass != nullptr);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
  {
    Frame R = make(n_atom, ref_mass ? ref_mass : tgt_mass);
    Frame T = make(n_atom, tgt_mass);
#ifdef _OPENMP
#pragma omp for schedule(dynamic)
#endif
    for (int64_t i = 0; i < n_ref; ++i) {
      fill(R, ref_xyz, dtype, i, n_atom);
      if (mode == 0 || mode == 2) R.CenterOnOrigin(use_mass);
      int64_t j0 = (out_kind == 0) ? i + 1 : 0;
      for (int64_t j = j0; j < n_tgt; ++j) {
        fill(T, tgt_xyz, dtype, j, n_atom);
        double r;
        if (mode == 0) r = T.RMSD_CenteredRef(R, use_mass);
        else if (mode == 1) r = T.RMSD_NoFit(R, use_mass);
        else if (mode == 3) r = T.DISTRMSD(R);
        else r = QuaternionRMSD_CenteredRef(R, T, use_mass);
        int64_t idx = (out_kind == 0) ? tri(n_ref, i, j) : j * n_ref + i;
        out[idx] = (float)r;
      }
    }
  }
  return 0;
}

// Pair list in FP64, cluster-metric convention: frame pi[k] is the target
// ("this"), frame pj[k] is centred as the reference (Frame::RMSD).
extern "C" int ref_pairs_f64(const void* xyz, int dtype, int n_atom, const double* mass, int mode,
                             const int64_t* pi, const int64_t* pj, int64_t npairs, double* out) {
  bool use_mass = (mass != nullptr);
  Frame A = make(n_atom, mass), B = make(n_atom, mass);
  for (int64_t k = 0; k < npairs; ++k) {
    fill(A, xyz, dtype, pi[k], n_atom);
    fill(B, xyz, dtype, pj[k], n_atom);
    out[k] = (mode == 1) ? A.RMSD_NoFit(B, use_mass) : (mode == 3) ? A.DISTRMSD(B) : A.RMSD(B, use_mass);
  }
  return 0;
}

// The pairwise cache written by cpptraj's own binary cluster-matrix writer
// (Cpptraj::Cluster::Cmatrix_Binary::WriteCmatrix, src/Cluster/Cmatrix_Binary.cpp:141-188).
// frame_to_idx[k] is the cache row of original frame k, or -1 when sieved out.
extern "C" int ref_write_cmatrix(const char* path, const float* tri, const int* frame_to_idx, int64_t n_original,
                                 int64_t nrows, int sieve) {
  Cpptraj::Cluster::Cframes f2i;
  for (int64_t k = 0; k < n_original; ++k) f2i.push_back(frame_to_idx[k]);
  Cpptraj::Cluster::Cmatrix_Binary w;
  return w.WriteCmatrix(FileName(path), tri, f2i, (size_t)nrows, sieve);
}

// Per-frame fit with cpptraj's own code, as the rms/align actions run it
// (Action_Rmsd::DoAction src/Action_Rmsd.cpp:372-395, Action_Align::DoAction
// src/Action_Align.cpp:85-99): the reference centred once with CenterOnOrigin
// (ReferenceAction::SelectRefAtoms), RMSD_CenteredRef(ref, U, Trans) per frame
// and Trans_Rot_Trans(Trans, U, refTrans) of the frame's n_move atoms.  Same
// argument meaning as orc_superpose_f64 (fit only).
extern "C" int ref_superpose(const void* ref_xyz, const void* xyz, int dtype, int64_t n_frame, int n_atom,
                             const double* ref_mass, const double* mass, double* rmsd, double* rot,
                             double* tgt_trans, double* ref_trans, double* move, int n_move) {
  bool use_mass = (mass != nullptr);
  Frame R = make(n_atom, ref_mass ? ref_mass : mass);
  fill(R, ref_xyz, dtype, 0, n_atom);
  Vec3 rt = R.CenterOnOrigin(use_mass);
  for (int k = 0; k < 3; ++k) ref_trans[k] = rt[k];
  Frame T = make(n_atom, mass);
  std::vector<double> mv(3 * (size_t)n_move, 0.0), mm(n_move, 1.0);
  Frame M;
  M.SetupFrameXM(mv, mm);
  for (int64_t f = 0; f < n_frame; ++f) {
    fill(T, xyz, dtype, f, n_atom);
    Matrix_3x3 U;
    Vec3 tr;
    rmsd[f] = T.RMSD_CenteredRef(R, U, tr, use_mass);
    for (int k = 0; k < 9; ++k) rot[9 * f + k] = U[k];
    for (int k = 0; k < 3; ++k) tgt_trans[3 * f + k] = tr[k];
    if (move) {
      double* x = M.xAddress();
      double* src = move + (size_t)f * 3 * n_move;
      for (int k = 0; k < 3 * n_move; ++k) x[k] = src[k];
      M.Trans_Rot_Trans(tr, U, rt);
      for (int k = 0; k < 3 * n_move; ++k) src[k] = x[k];
    }
  }
  return 0;
}

// Cluster centroids with cpptraj's own Frame code, in the steps of
// Metric_RMS::CalculateCentroid (src/Cluster/Metric_RMS.cpp:86-108): the first
// member copied (and centred with CenterOnOrigin when fitting), each later
// member fitted onto the running sum by RMSD_CenteredRef(sum, Rot, Trans),
// rotated with Frame::Rotate and added with +=, the sum divided by the member
// count.  Same argument meaning as orc_cluster_centroids_f64 (fit = mode 0,
// nofit = mode 1); empty clusters are skipped.
extern "C" int ref_cluster_centroids(const void* xyz, int dtype, int64_t n_frame, int n_atom, const double* mass,
                                     int mode, const int32_t* members, const int64_t* offsets, int64_t n_cluster,
                                     double* out) {
  (void)n_frame;
  const bool use_mass = (mass != nullptr), nofit = (mode == 1);
  Frame frm = make(n_atom, mass);
  for (int64_t c = 0; c < n_cluster; ++c) {
    Frame cent;
    for (int64_t k = offsets[c]; k < offsets[c + 1]; ++k) {
      fill(frm, xyz, dtype, members[k], n_atom);
      if (cent.empty()) {
        cent = frm;
        if (!nofit) cent.CenterOnOrigin(use_mass);
      } else {
        if (!nofit) {
          Matrix_3x3 Rot;
          Vec3 Trans;
          frm.RMSD_CenteredRef(cent, Rot, Trans, use_mass);
          frm.Rotate(Rot);
        }
        cent += frm;
      }
    }
    const int64_t n = offsets[c + 1] - offsets[c];
    if (n <= 0) continue;
    cent.Divide((double)n);
    const double* x = cent.xAddress();
    for (int k = 0; k < 3 * n_atom; ++k) out[(size_t)c * 3 * n_atom + k] = x[k];
  }
  return 0;
}
