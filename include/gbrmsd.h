/*
 * gbrmsd.h -- C ABI of the GB300 all-pairs best-fit RMSD library (libgbrmsd.so).
 *
 * This is the drop-in boundary for cpptraj's all-pairs RMSD path.  Each entry
 * point replaces one loop of the reference:
 *
 *   gbr_allpairs      <- Analysis_Rms2d::Calculate_2D pair loop for RMS_FIT,
 *                        RMS_NOFIT and DME (src/Analysis_Rms2d.cpp:247-290), and the
 *                        Metric_RMS branch of MetricArray::calcFrameDistances
 *                        (src/Cluster/MetricArray.cpp:770-800).  The per-pair
 *                        arithmetic it reproduces is Frame::RMSD_CenteredRef
 *                        (src/Frame.cpp:1137-1273), Frame::RMSD
 *                        (src/Frame.cpp:1102-1109), Frame::RMSD_NoFit
 *                        (src/Frame.cpp:1279-1307) and Frame::DISTRMSD
 *                        (src/Frame.cpp:1313-1344).
 *   gbr_allpairs_batched <- the same loop run over many independent COORDS
 *                        sets, one rms2d per set.
 *   gbr_write_cmatrix <- the pairwise-cache fill plus Cmatrix_Binary::WriteCmatrix
 *                        (savepairdist) in one call.
 *   gbr_superpose     <- the per-frame fit of the rms / align actions
 *   gbr_cluster_centroids <- Metric_RMS::CalculateCentroid (cluster centroids)
 *                        (Action_Rmsd::DoAction, Action_Align::DoAction).
 *   gbr_rmsd_backward <- no reference counterpart (cpptraj has no gradient of
 *                        RMSD); dL/dx for L = sum_{i<j} g_ij RMSD_ij.
 *
 * Conventions (all from the reference):
 *   - Coordinates are frame-major, atom-major xyz: frame f, atom a, component
 *     p at xyz[(f*n_atom + a)*3 + p], i.e. what DataSet_Coords::GetFrame with
 *     the analysis mask (src/DataSet_Coords_CRD.cpp:142-147) gathers, stored
 *     contiguously.  dtype GBR_F32 matches COORDS sets (CompactFrameArray is
 *     float, src/CompactFrameArray.h:75-76); GBR_F64 matches `loadcrd ... prec
 *     double` FRAMES sets (src/Exec_LoadCrd.cpp:20-25).
 *   - Masses: when tgt_mass is NULL every atom weighs 1 (no `mass` keyword).
 *     Otherwise reference frames are centred with ref_mass (NULL => tgt_mass)
 *     and every sum is weighted by tgt_mass, as in Frame::CenterOnOrigin on the
 *     reference followed by RMSD_CenteredRef on the target.
 *   - Rows are reference frames (nref), columns target frames (ntgt).
 *     GBR_TRI: one set (tgt_xyz == NULL), pairs nref < ntgt, element index
 *       n*i - (i+1)*i/2 + j - i - 1 (Matrix<T>::calcTriIndex, src/Matrix.h:110-122);
 *       the layout of DataSet_MatrixFlt::AllocateTriangle and of
 *       DataSet_PairwiseCache_MEM (src/DataSet_PairwiseCache_MEM.cpp:20-41).
 *     GBR_FULL: every (nref, ntgt), index ntgt*n_ref + nref
 *       (Matrix<T>::calcFullIndex, src/Matrix.h:94-96; DataSet_MatrixFlt::Allocate2D).
 *   - Row ranges: TRI rows are reference frames; FULL rows are target frames
 *     (the slow index of calcFullIndex).  `out` receives exactly the elements
 *     of rows [row_begin, row_end) in index order, starting at out[0].  Pass
 *     row_begin = 0, row_end = -1 for the whole matrix.
 *   - Results are cast to float as SetElement does (src/Analysis_Rms2d.cpp:276).
 *     A negative E0 - lambda is clamped to 0 (src/Frame.cpp:1264-1266).
 *     Zero total mass (< 1e-14, src/Constants.h:35) is an error for the call
 *     (the reference returns -1 for the pair and prints an error).
 *   - Pointers may be host or device memory (detected per call).  Host
 *     buffers are staged through the handle's device memory.  Device
 *     buffers must be on the handle's device (GBR_ERR_ARG otherwise); masses,
 *     offsets and member lists are read once and may be on any device.
 *   - Return value: GBR_OK (0) or an error code; gbr_last_error gives text.
 *     No exception crosses the ABI.  One handle must not be used from two
 *     threads at once; separate handles are independent.
 */
#ifndef GBRMSD_H
#define GBRMSD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum gbr_status {
  GBR_OK = 0,
  GBR_ERR_ARG = 1,        /* invalid argument (sizes, null pointers, modes)   */
  GBR_ERR_CUDA = 2,       /* CUDA runtime or launch error                     */
  GBR_ERR_NOMEM = 3,      /* device workspace could not be allocated          */
  GBR_ERR_ZERO_MASS = 4,  /* total mass below 1e-14                           */
  GBR_ERR_DEVICE = 5,     /* a kernel reported a device-side error (timeout)  */
  GBR_ERR_UNSUPPORTED = 6, /* precision/mode not available on this device     */
  GBR_ERR_IO = 7           /* a file could not be opened or written           */
};

enum gbr_dtype { GBR_F32 = 0, GBR_F64 = 1 };
/* GBR_DME: distance RMSD (rms2d `dme`, Frame::DISTRMSD, src/Frame.cpp:1313-1344):
 * masses are ignored and the reference is not centred, as in the reference;
 * GBR_PREC_FP32 and GBR_PREC_TC both run the CUDA-core DME kernels (DME has no
 * tensor-core form here; gbr_stats.precision reports GBR_PREC_FP32). */
enum gbr_mode { GBR_FIT = 0, GBR_NOFIT = 1, GBR_DME = 2 };
enum gbr_out_kind { GBR_TRI = 0, GBR_FULL = 1 };
enum gbr_precision {
  GBR_PREC_FP32 = 0, /* CUDA-core FP32 contraction of pre-aligned residuals    */
  GBR_PREC_TC = 1,   /* tcgen05 tensor cores, FP16 hi+lo split of residuals     */
  GBR_PREC_FP64 = 2  /* every pair recomputed directly in FP64 (slow; checking) */
};

typedef struct gbr_handle gbr_handle;

/* Create a handle bound to CUDA device `device`; NULL on failure. */
gbr_handle *gbr_create(int device);

/* Destroy a handle and free its device memory and streams. */
void gbr_destroy(gbr_handle *h);

/* Run this handle's work on `stream` (a cudaStream_t of the handle's device,
 * or NULL to go back to the handle's own stream).  Calls still return only
 * when their results are in `out`. */
int gbr_set_stream(gbr_handle *h, void *stream);

/* Last error message of this handle ("" if none).  Valid until the next call. */
const char *gbr_last_error(const gbr_handle *h);

/* All-pairs RMSD; see the conventions above. */
int gbr_allpairs(gbr_handle *h, const void *ref_xyz, const void *tgt_xyz, int dtype,
                 int64_t n_ref, int64_t n_tgt, int32_t n_atom,
                 const double *ref_mass, const double *tgt_mass,
                 int mode, int out_kind, int precision,
                 float *out, int64_t row_begin, int64_t row_end);

/* Number of output elements gbr_allpairs writes for these arguments. */
int64_t gbr_output_count(int64_t n_ref, int64_t n_tgt, int out_kind,
                         int64_t row_begin, int64_t row_end);

/* Receives one band of a streamed triangle: the values of TRI rows
 * [row_begin, row_end) in calcTriIndex order (count floats, which start at
 * triangle index n*row_begin - (row_begin+1)*row_begin/2).  `values` is the
 * library's pinned host memory, valid until the callback returns.  Return 0
 * to go on; anything else stops the call, which then returns GBR_ERR_IO. */
typedef int (*gbr_band_sink)(void *user, int64_t row_begin, int64_t row_end, const float *values,
                             int64_t count);

/* The triangle of one frame set (GBR_TRI, as gbr_allpairs computes it) in
 * row bands of at most band_floats floats (<= 0: 2^28), for caches that do
 * not fit in device memory at once: the pairwise cache behind
 * MetricArray::CacheDistances (src/Cluster/MetricArray.cpp:722-801) with a
 * disk cache (DataSet_PairwiseCache_NC, one SetElement per pair in the
 * reference, src/DataSet_PairwiseCache_NC.h:27).  The frames are prepared
 * once; band b is computed while band b-1 is copied to the host and band b-2
 * is handed to `sink` on the calling thread, bands in row order, so device
 * memory holds the frames and two bands only.  A band must hold at least one
 * row (n_frame - 1 floats).  GBR_DME is not streamed (GBR_ERR_UNSUPPORTED);
 * an empty triangle makes no callback. */
int gbr_allpairs_stream(gbr_handle *h, const void *xyz, int dtype, int64_t n_frame, int32_t n_atom,
                        const double *mass, int mode, int precision, int64_t band_floats,
                        gbr_band_sink sink, void *user);

/* The band boundaries gbr_allpairs_stream uses: cuts[0] = 0 < cuts[1] < ...
 * < cuts[n] = n_frame with at most band_floats TRI elements per band, at
 * multiples of row_align rows where a band holds whole groups of them.
 * Returns n (the band count), or -1 when one row exceeds band_floats or
 * max_cuts (the capacity of cuts) is too small.  Host only; no device work. */
int64_t gbr_row_bands(int64_t n_frame, int64_t band_floats, int32_t row_align, int64_t *cuts,
                      int64_t max_cuts);

/* Many independent rms2d runs (GBR_TRI, one set each) in one call.  Trajectory
 * t has n_frames[t] frames of n_atoms[t] atoms at xyz[t] (GBR_F32), masses
 * mass[t] (NULL, or mass == NULL, for unweighted) and writes its triangle to
 * out[t].  All pointers of one call must be of the same kind (host or device). */
int gbr_allpairs_batched(gbr_handle *h, int32_t n_traj, const float *const *xyz,
                         const int64_t *n_frames, const int32_t *n_atoms,
                         const double *const *mass, int mode, int precision,
                         float *const *out);

/* The clustering pairwise cache of one frame set (GBR_TRI, as gbr_allpairs
 * computes it) written to `path` as cpptraj's binary cluster-matrix file,
 * version 2 -- the file `savepairdist` writes and `loadpairdist` reads
 * (Cpptraj::Cluster::Cmatrix_Binary::WriteCmatrix, src/Cluster/Cmatrix_Binary.cpp:141-188).
 * The n_frame frames are the cached ones in order.  frame_to_idx (length
 * n_original, entries -1 for sieved-out frames, else the cache row) and sieve
 * go into the header and trailer; frame_to_idx NULL means no sieve.  The
 * triangle is streamed to the file in row bands (gbr_allpairs_stream, band
 * size GBR_OPT_BAND_FLOATS), so it need not fit in device memory; GBR_DME
 * computes the whole triangle in device memory first. */
int gbr_write_cmatrix(gbr_handle *h, const char *path, const void *xyz, int dtype, int64_t n_frame,
                      int32_t n_atom, const double *mass, int mode, int precision,
                      const int32_t *frame_to_idx, int64_t n_original, int64_t sieve);

/* Gradient of L = sum_{i<j} g[tri(i,j)] * RMSD_ij (best fit, one set, GBR_F32)
 * with respect to every coordinate.  g NULL means g = 1.  grad_xyz has the
 * shape of xyz.  rmsd_out (optional, may be NULL) receives the forward TRI.
 * Pairs with RMSD == 0 contribute no gradient.  Needs an sm_103 (GB300)
 * device (GBR_ERR_UNSUPPORTED otherwise): the pair pass and the block
 * contraction (S = B + B^T times the operand plane, FP16 hi/lo operands,
 * three products, FP32 accumulation: ~2^-22 of the largest product) both
 * run on the tensor cores; at most 60,000 frames. */
int gbr_rmsd_backward(gbr_handle *h, const float *xyz, int64_t n_frame, int32_t n_atom,
                      const double *mass, const float *g, float *grad_xyz, float *rmsd_out);

/* Per-frame best fit of n_frame frames onto ONE reference frame: the `rms`
 * action (Action_Rmsd::DoAction, src/Action_Rmsd.cpp:372-395) and `align`
 * (Action_Align::DoAction, src/Action_Align.cpp:85-99) over a whole frame set.
 *   ref_xyz   the reference frame (n_atom atoms, dtype), as selected by the
 *             reference mask.  GBR_FIT centres it, as ReferenceAction does
 *             with Frame::CenterOnOrigin: mass-weighted by ref_mass (NULL =>
 *             mass) when mass is given, geometrically when mass is NULL (the
 *             action's one `mass` keyword); GBR_NOFIT uses it as given.
 *   xyz       n_frame frames of n_atom atoms (the target mask), dtype.
 *   mass      target masses weighting every sum (NULL => unweighted), as
 *             Frame::RMSD_CenteredRef / RMSD_NoFit use the target's masses.
 *   rmsd      [n_frame] RMSD_CenteredRef (fit) or RMSD_NoFit (nofit), FP64.
 *   rot       [n_frame][9] the best rotation U, row-major (U y ~ r for the
 *             centred frame y); identity for nofit.
 *   tgt_trans [n_frame][3] the frame's Trans of RMSD_CenteredRef, i.e. minus
 *             its centre (mass-weighted when mass is given); 0 for nofit.
 *   ref_trans [3] the reference's centre (ReferenceAction::RefTrans); 0 for nofit.
 *   move_xyz  [n_frame][n_move][3] of dtype, or NULL: frame f's atoms to move
 *             (align's move mask, rms's whole frame), transformed in place by
 *             Frame::Trans_Rot_Trans(tgt_trans[f], U[f], ref_trans)
 *             (src/Frame.h:572-581); untouched for nofit.
 * Any output may be NULL.  Pointers may be host or device memory.  All
 * arithmetic is FP64. */
int gbr_superpose(gbr_handle *h, const void *ref_xyz, const void *xyz, int dtype, int64_t n_frame,
                  int32_t n_atom, const double *ref_mass, const double *mass, int mode, double *rmsd,
                  double *rot, double *tgt_trans, double *ref_trans, void *move_xyz, int32_t n_move);

/* Cluster centroids as Metric_RMS::CalculateCentroid builds them
 * (src/Cluster/Metric_RMS.cpp:86-108), every cluster in one call.
 *   xyz        n_frame frames of n_atom atoms (the metric's mask), dtype.
 *   mass       masses (NULL => unweighted, the metric's useMass_ off).
 *   mode       GBR_FIT: in member order, the first member centred starts a
 *              running sum; each later member is centred, fitted onto the sum
 *              (Frame::RMSD_CenteredRef), rotated and added.  GBR_NOFIT: the
 *              plain sum of the members as given.
 *   members    frame indices (0 <= index < n_frame) of all clusters back to
 *              back, each cluster in the order the reference visits it
 *              (its Cframes list);
 *   offsets    [n_cluster + 1]: cluster c is members[offsets[c] ..
 *              offsets[c + 1]).
 *   centroids  [n_cluster][n_atom][3] FP64: the sum divided by the member
 *              count.  An empty cluster's centroid is NaN (the reference's
 *              has no atoms).
 * Pointers may be host or device memory.  Per-atom sums are FP32 with the
 * running sum kept as an FP32 hi + lo pair, the fit itself FP64: centroid
 * coordinates agree with the reference's FP64 chain to ~1e-6 Angstrom.
 * Frame indices out of range return GBR_ERR_ARG; a zero total mass with
 * GBR_FIT returns GBR_ERR_ZERO_MASS. */
int gbr_cluster_centroids(gbr_handle *h, const void *xyz, int dtype, int64_t n_frame, int32_t n_atom,
                          const double *mass, int mode, const int32_t *members, const int64_t *offsets,
                          int64_t n_cluster, double *centroids);

/* All-pairs RMSD that allocates nothing.  No counterpart in the reference:
 * cpptraj's loops allocate host frames per thread; this entry point exists for
 * callers that cannot call cudaMalloc at all -- host programs that reserve the
 * GPU's memory at start-up and serve it from their own fixed pool, and plugins
 * loaded into such a process or into one whose latency-critical streams must
 * not be stalled by the synchronisation cudaMalloc/cudaFree can cause.  It
 * computes the same triangle as
 * gbr_allpairs(..., GBR_TRI, GBR_PREC_FP64, ...) -- every pair directly in
 * FP64 -- for one frame set: xyz (dtype GBR_F32/GBR_F64), mass (NULL =
 * unweighted) and out (n_frame*(n_frame-1)/2 floats) must all be memory of
 * the current CUDA device (or managed memory), else GBR_ERR_ARG; stream may
 * be NULL (legacy default stream).  Its only scratch is a
 * fixed 32 MiB __device__ array in this library (held by every GPU that loads
 * it until the process exits): frame counts needing more (above ~1.39 million
 * frames) are rejected with GBR_ERR_NOMEM.  The first call on a device looks
 * the array's address up (make it before any stream capture).  Calls share
 * the array, so calls that overlap on the GPU race.  Returns a gbr_status;
 * there is no handle and no message text. */
int gbr_allpairs_fp64_static(const void *xyz, int dtype, int64_t n_frame, int32_t n_atom,
                             const double *mass, int mode, float *out, void *stream);

/* Per-call statistics of the last gbr_allpairs / batched / backward call. */
typedef struct gbr_stats {
  int64_t pairs;          /* pairs computed                                      */
  int64_t pairs_fixed;    /* pairs whose error bound sent them to the FP64 kernel */
  int32_t n_refs;         /* pre-alignment reference structures used             */
  int32_t precision;      /* precision actually run                              */
  int32_t kernel_launches;/* kernels launched by the call                        */
  double ms_prep;         /* device time of centring/alignment kernels (ms)      */
  double ms_pairs;        /* device time of the pair contraction kernel(s) (ms)  */
  double ms_fixup;        /* device time of the FP64 re-check kernel (ms)        */
  double ms_total;        /* wall time of the call (ms)                          */
} gbr_stats;

int gbr_get_stats(const gbr_handle *h, gbr_stats *out);

/* Tuning knobs (mostly for tests and benchmarks).  Keys:
 *   GBR_OPT_TAU          reference-selection radius in Angstrom (default 6.0)
 *   GBR_OPT_MAX_REFS     maximum pre-alignment references (1..64, default 32)
 *   GBR_OPT_TOL          per-pair error target in Angstrom (default 5e-5)
 *   GBR_OPT_TIMING       1 = record per-kernel device times in gbr_stats
 *   GBR_OPT_TC_PIPELINE  tensor-core kernel shape: 0 = one SM, 64-atom stages x 2,
 *                        1 = one SM, 32-atom stages x 4, 2 = pairs of SMs
 *                        sharing one 256-row MMA, 32-atom stages x 5,
 *                        3 = pairs of SMs, 64-atom stages x 3 with narrower
 *                        epilogue chunks, 4 = pairs of SMs, 32-atom stages x 3
 *                        with wider (16-frame) epilogue chunks; -1 (default)
 *                        = 3 from 1,280 atoms on, 4 below 768, 2 between
 *   GBR_OPT_HOST_OUT     pinned host `out` of gbr_allpairs: 1 = the kernels
 *                        store into it directly (default; a triangle over
 *                        reference-sorted frames, with several references,
 *                        is computed in device memory in row bands whose
 *                        rows are copied while the next band computes),
 *                        0 = results staged in device memory and copied back
 *                        in row bands
 *   GBR_OPT_BAND_FLOATS  band size in floats of gbr_write_cmatrix's streamed
 *                        triangle (default 2^28; at least one row)
 *   GBR_OPT_INPUT_OVERLAP  pinned host input of one frame set, triangle into
 *                        device or directly stored host memory: 1 (default) =
 *                        the contraction starts on the frames that have
 *                        landed while the rest of the input transfers (the
 *                        first tiles on part of the SMs, beside the per-chunk
 *                        preparation), 0 = it starts after the whole input is
 *                        prepared
 */
enum gbr_option { GBR_OPT_TAU = 0, GBR_OPT_MAX_REFS = 1, GBR_OPT_TOL = 2, GBR_OPT_TIMING = 3,
                  GBR_OPT_TC_PIPELINE = 4, GBR_OPT_HOST_OUT = 5, GBR_OPT_INPUT_OVERLAP = 6,
                  GBR_OPT_BAND_FLOATS = 7 };
int gbr_set_option(gbr_handle *h, int key, double value);

/* Self-test of the device-side failure detection.  No counterpart in the
 * reference (its loops run on the host).  The tensor-core pair kernels bound
 * every mbarrier wait; when a wait runs out the kernel records a site code,
 * returns normally and the call fails with GBR_ERR_DEVICE.  This runs that
 * same bounded-wait helper in a one-CTA kernel (no TMA, no MMA, no peer CTA)
 * on a barrier nothing arrives on, with a limit of limit_cycles clock cycles
 * (1000 .. 4e9).  GBR_OK means the wait gave up as designed: every thread
 * returned, the site code was recorded (*site_out, optional) and the context
 * is still usable; *waited_cycles (optional) is how long thread 0 waited. */
int gbr_selftest_bounded_wait(gbr_handle *h, int64_t limit_cycles, int32_t *site_out,
                              int64_t *waited_cycles);

#ifdef __cplusplus
}
#endif
#endif /* GBRMSD_H */
