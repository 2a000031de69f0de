// gbr_internal.h -- host-side interfaces between the C-ABI layer (gbr_capi.cu)
// and the kernel files.  Not part of the public ABI.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <functional>
#include <vector>

#include "gbr_common.cuh"
#include "gbr_tiles.h"

namespace gbr {

struct PrepArgs {
  int dtype_f64;
  const void* ref;  // device, [n_ref][N][3]
  const void* tgt;  // device or nullptr (TRI)
  int64_t n_ref;
  int64_t F;        // set frames (n_ref, or n_ref + n_tgt)
  int N, Np;
  int nofit;
  int centroid_only;        // only compute centres (FP64 checking mode)
  const double* cmass_ref;  // centring masses of reference frames (nullptr = geometric)
  const double* cmass_tgt;  // centring masses of target frames
  const double* w;          // weights (target masses) or nullptr
  double Wsum;
  double tau;
  int max_refs;
  // workspace
  double* cen;     // [F][3]
  int64_t* fsel;   // [1]
  float* dmax;     // [1]
  float* dist;     // [F]
  int* assign;     // [F]
  double* refs;    // [max_refs][N][3]
  float* swr;      // [max_refs][N][3]
  double* Eref;    // [max_refs]
  double* rot;     // [F][9] or nullptr
  float* plane;    // [F][3][Np]
  int* order;      // [F] frames grouped by reference
  int* offsets;    // [max_refs + 1]
  float* mean;     // [max_refs][3][Np]
  float* partial;  // [max_refs][64][3][Np] chunk sums for the means
  double* sqw;     // [N] sqrt of the weights
  float* sqwf;     // [N] the same in FP32
  void* scratch;   // prep_scratch_bytes(F, N, max_refs) bytes (PrepScratch)
  int sort_frames; // with several references: lay operands out grouped by reference
  // Inputs arriving in chunks (host copies overlapping the first pass):
  // frames [chunk_end[c-1], chunk_end[c]) are usable once chunk_ev[c] completes.
  int n_chunks;
  int64_t chunk_end[8];
  cudaEvent_t chunk_ev[8];
  // When non-null, called on the host just before a pass first waits on
  // chunk_ev[c], to issue chunk c's copy then (pageable host input, whose
  // copies hold the host until they are done: issued one by one between the
  // chunks' passes, each overlaps the passes of the chunks before it).
  const std::function<void(int)>* chunk_copy;
  // With chunks: the operand build for one reference (K = 1, unsorted), run
  // speculatively while the chunks land (PrepOut::built reports success).
  const struct FinishArgs* spec_build;
  // With spec_build: called on the host after each chunk's operands are
  // enqueued, with the end of the frame range [0, end) built so far (work the
  // caller enqueues there runs between the chunks' prep passes).
  const std::function<cudaError_t(int64_t)>* on_built;
  // With spec_build: an int on the device, set to 1 by the chunk checks once
  // a scanned frame is farther than tau from reference 0 (the speculation
  // will fail); work enqueued through on_built may test it.
  int* spec_fail;
  // Whole input on the device, no chunks: when non-null, the reference-count
  // decision after the first scan is left on the device.  Prep continues as
  // for one reference and every later pass of this call (prep, build, pair
  // kernel) tests this int at launch; it reads 1 once a frame is farther than
  // tau from reference 0, and then the passes do nothing and the caller
  // repeats the call with the decision on the host (PrepOut::deferred).
  int* defer_multi;
  // The second run of a deferred call: weights, reference 0 and the first
  // scan are in the workspace already (the deferred passes did nothing).
  int resume_scan;
  // Reference-pair terms [K][K][24] (optional): when one reference stays,
  // the refinement writes its terms with itself here (PrepOut::self_terms).
  float* RP;
};

// Further per-call prep buffers, carved from PrepArgs::scratch.
struct PrepScratch {
  float* cmf_ref;  // [N] centring masses of reference frames in FP32
  double* scal;    // [8] max sqrt(w), sum w, sum of reference centring masses, 0, their reciprocals
  float2* refhl;   // [Kmax][N][3] references as hi + lo floats
  double* sr;      // [Kmax][3] sum_a w_a r_k,a
  float* rmax;     // [Kmax] max_a |r_k,a|
  float4* quat;    // [F] superposition quaternion onto the assigned reference
  float* ymax;     // [F] upper bound of max_a |y_a| (centred frame)
  float* ftab;     // [F][24] rotation hi/lo (9 + 9), centre hi/lo (3 + 3)
  int* pos;        // [F] frame -> position when frames are laid out sorted by reference
  int* assign_pos; // [F] reference of the frame at each position
  float4* qscan;   // [Kmax][N] {sqrt(w) r_k, sqrt(w)} of the references as chosen (the scans read these)
  float4* qbuild;  // [Kmax][N] the same of the refined references (the operand build reads these)
  int* kstate;     // [2] k-centre choice on the device: stopped flag, index of the last reference added
  unsigned* rcount;  // k_ref_update: blocks done (one reference's self terms)
  double* rsu;       // k_ref_update: per-block sums of w r r^T (one reference)
  float* dref;       // [Kmax] k-centre round k: FP32 distances from reference k to references 0..k-1
};
size_t prep_scratch_bytes(int64_t F, int N, int Kmax);
PrepScratch prep_carve(void* base, int64_t F, int N, int Kmax);

// Last per-frame pass: shift to the refined references, optional FP16 split
// with per-frame scales, per-frame terms n/P/trP, reference-pair table.
struct FinishArgs {
  const PrepArgs* prep;  // the prep call of the same frames (sources, tables)
  int sorted;            // PrepOut::sorted of that call
  float* plane;
  int64_t F;
  int N, Np, K;
  const float* mean;
  const int* assign;
  const float* swr;
  int tc;
  void* hi;
  void* lo;
  float* inv_scale;   // [F] 1/scale per frame (tensor path)
  int write_plane;    // keep the shifted FP32 plane (FP32 pair kernel, backward)
  float* nrm;
  float* P;
  float* trP;
  const double* refs;
  const double* w;
  int nofit;
  float* RP;
  int built;          // the operands are built already (speculative prep): only the reference-pair terms
  const int* skip;    // device int or nullptr: the passes do nothing when it reads non-zero at launch
  int self_terms;     // RP holds the one reference's terms already (PrepOut::self_terms)
};
cudaError_t run_finish(const FinishArgs& A, cudaStream_t st);

struct PrepOut {
  int K = 1;
  int launches = 0;
  int sorted = 0;  // operands and per-frame terms are at sorted positions (PrepScratch::pos)
  int built = 0;   // the operands were built during prep (one reference, chunked input)
  int deferred = 0; // K = 1 was assumed and PrepArgs::defer_multi decides it on the device
  int self_terms = 0;  // one reference, and PrepArgs::RP holds its terms with itself
};

cudaError_t run_prep(const PrepArgs& A, PrepOut& o, cudaStream_t st);

}  // namespace gbr
struct gbr_handle;
namespace gbr {
// rms2d `dme` mode (gbr_dme.cu): arguments already validated by gbr_allpairs.
int allpairs_dme(gbr_handle* h, const void* ref_xyz, const void* tgt_xyz, int dtype, int64_t n_ref, int64_t n_tgt,
                 int N, int out_kind, int precision, float* out, int64_t row_begin, int64_t row_end, int64_t n_out);


// Tiles of the pair space: rows = reference frames, cols = target frames.
struct TileSpace {
  int tri;          // upper-triangle tiles only
  int64_t i0, j0;   // first reference / target frame covered
  int64_t ni, nj;   // frames covered
  int64_t ti, tj;   // tiles along i / j
  int64_t count;    // tiles launched
};

TileSpace make_tiles(const OutMap& m, int bm, int bn);

// Backward-mode outputs of the FP32 pair kernel (nullptr B = forward mode).
struct BwdArgs {
  float* B;          // [3F][3F], upper pair blocks c*T (row 3i+p, column 3j+q, i < j)
  int64_t ldB;       // row stride of B: 3F rounded up to a multiple of 4
  float* E;          // [F][9] sum_h c_fh (I - T_fh)
  float* C;          // [F]    sum_h c_fh
  const float* g;    // TRI upstream weights (nullptr = 1)
  float* rmsd;       // TRI forward values (nullptr = not stored)
  unsigned int* cmax;  // max |c| over the pairs (float bits, max-combined), a bound of max |B|
};

struct PairLaunch {
  BwdArgs bwd;
  const float* plane;  // FP32 plane [F][3][Np]
  int Np, N;
  int64_t tgt0;        // set index of target frame 0
  FrameTerms terms;
  OutMap map;
  FlagList flags;
  TileSpace tiles;
  const int* skip;     // device int or nullptr: the kernel does nothing when it reads non-zero at launch
};

cudaError_t run_pairs_fp32(const PairLaunch& L, cudaStream_t st);

// Tensor-core contraction (tcgen05).  hi/lo: FP16 planes [F][3][Np].
struct TcLaunch {
  const void* hi;
  const void* lo;
  void* tile_buf;     // device scratch for the tile list (int2)
  int64_t tile_cap;
  int64_t F;
  int Np, N;
  int64_t tgt0;
  const float* inv_scale;  // [F] per-frame 1/scale of the FP16 split
  FrameTerms terms;
  OutMap map;
  FlagList flags;
  TileSpace tiles;
  int* dev_error;    // set non-zero when a bounded wait gives up
  int num_sms;
  int variant;       // 0: 64-atom stages (128B swizzle, 2 stages); 1: 32-atom stages (64B swizzle, 4 stages);
                     // 2: pairs of SMs (cta_group::2), 32-atom stages x 5, 8-frame epilogue chunks;
                     // 3: pairs of SMs, 64-atom stages x 3, 4-frame epilogue chunks;
                     // 4: pairs of SMs, 32-atom stages x 3, 16-frame epilogue chunks, 40 reference frames per CTA
  int64_t ready_tiles;  // > 0: tile_buf already holds this many tiles (no host build or copy)
  int row_stores;       // pair kernels, triangle output: gather each tile's results and store whole rows
                        // (host memory across the link); 0: each pair stored directly (device memory)
  const int* skip;      // device int or nullptr: when it reads non-zero at launch, the kernel does nothing
  const BwdArgs* bwd;   // non-null: the backward pass (variants 2 and 3, one set, TRI, one reference)
  int cluster_cap;      // pairs of SMs: > 0 caps the persistent grid at this many clusters, < 0 leaves
                        // that many of the resident clusters free
  int2* tile_stage;     // pinned host buffer of tile_cap entries, or nullptr: the tile list is uploaded
                        // from it (the host returns at once) instead of from pageable memory (the host
                        // waits until the copy has run, i.e. until the stream's earlier work is done)
};
// Tile list of the tensor-core kernel for this map (host side).
struct TcTileInfo {
  int64_t i_base, jt_base, i_end, jt_end;
};
int64_t tc_build_tile_list(const OutMap& m, std::vector<int2>& tiles, TcTileInfo& info, int variant = 1);
// The output region and tile shape of that list (for build_tiles_staged).
TileGrid tc_tile_grid(const OutMap& m, int variant);
// Reference frames per launch tile of a tensor-core kernel shape.
int tc_launch_tile_rows(int variant);
cudaError_t run_pairs_tc(const TcLaunch& L, cudaStream_t st);
int tc_supported(int device);
int64_t tc_max_tiles(const OutMap& m);

// Backward block contraction on the tensor cores (gbr_bwd_gemm.cu):
// Z[3F][Np] = (B + B^T) * plane with both operands scaled and split into
// FP16 hi/lo.
struct BackwardGemm {
  int64_t F;
  int Np;
  const float* B;        // [3F][ldB] upper pair blocks c*T
  int64_t ldB;
  const float* plane;    // [3F][Np] sqrt(w) d
  __half* Shi;           // [3F][bwd_gemm_ld(F)] S = B + B^T, hi part
  __half* Slo;           //                      lo part
  __half* Thi;           // [Np][bwd_gemm_ld(F)] plane transposed, hi part
  __half* Tlo;           //                      lo part
  unsigned int* maxbits; // [2] bound of max |B| (set by the backward pair kernel, BwdArgs::cmax), max |plane|
  float* scl;            // [2] 1/scale of S, of the plane
  float* Z;              // [3F][Np]
  int* dev_error;        // bounded-wait error word
  int num_sms;
};
// Row stride (elements) of the split operands: 3F rounded up to the 64-wide K stage.
int64_t bwd_gemm_ld(int64_t F);
cudaError_t run_backward_gemm(const BackwardGemm& G, cudaStream_t st);

// Backward tail: Z = (B + B^T) * plane (run_backward_gemm), then assemble
// and rotate the gradient.
struct BackwardTail {
  BackwardGemm gemm;
  int64_t F;
  int N, Np;
  const float* plane;  // [F][3][Np]  (= [3F][Np])
  const float* Z;      // [3F][Np]
  const float* E;      // [F][9]
  const float* C;      // [F]
  const double* rot;   // [F][9] pre-alignment rotations
  const double* ref0;  // [N][3] the (single) pre-alignment reference
  const double* w;     // masses or nullptr
  const double* sqw;   // sqrt of the masses (when w is given)
  double W;
  float* grad;         // [F][N][3]
  float4* atab;        // [N][3] scratch: reference, weight and sqrt(weight) as FP32 hi + lo
};
cudaError_t run_backward_tail(const BackwardTail& T, cudaStream_t st);

// Direct FP64 recomputation (flagged pairs or every pair).
struct ExactLaunch {
  int dtype_f64;
  const void* ref;
  const void* tgt;
  int64_t n_ref;
  int N;
  const double* cen;  // [F][3] set-frame centres (zeros for no-fit)
  const double* w;    // target masses or nullptr
  double Wsum;
  const double* dWsum;  // non-null: the total weight is read from this device word instead of Wsum
  int nofit;
  int64_t tgt0;
  OutMap map;
  const int2* list;   // pairs (i, jt) or nullptr => every pair of the map
  int64_t count;      // pairs in list (or total pairs when list == nullptr)
  const unsigned long long* dev_count;  // non-null: the list length is read on the device,
                                        // clamped to `count` (the list capacity)
  int overflow_all;   // with dev_count: a length above the capacity recomputes every pair of the map
  int64_t map_pairs;  // pairs of the map (overflow_all)
};
cudaError_t run_exact(const ExactLaunch& L, cudaStream_t st);

}  // namespace gbr
