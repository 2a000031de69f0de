// gbr_prep.cu -- per-frame passes that run before the pair contraction (K1).
//
// GB300's FP64 rate is a small fraction of its FP32 rate, so nothing here does
// FP64 arithmetic per atom per frame.  Per-atom work is plain FP32 (the passes
// over the coordinates are bound by instruction issue, so every operation per
// atom counts).  What must not be rounded to FP32 is what acts on every atom
// of a frame alike: the rotation (kept as FP32 hi + lo of the FP64 matrix) and
// the frame centre (hi + lo of the FP64 value).  Rounding that differs from
// atom to atom -- of x - c, of the products R (x - c), of the sums -- enters
// an RMSD only through its projection on the pair's residual, about
// 2^-24 |y| / sqrt(N).  FP64 is kept for O(1)-per-frame and O(N)-per-reference
// work.
//
// Passes over the coordinates (one warp per frame, 8 frames per block):
//   k_scan<FIRST>  FIRST: the frame centre (Frame::CenterOnOrigin / the target
//                  centring of Frame::RMSD_CenteredRef, src/Frame.cpp:1043-1055,
//                  1142-1171), a bound of the centred extent, and the fit to
//                  reference 0.  Later: the fit to reference k of the greedy
//                  k-centre choice.  The fit gives the distance and the FP32
//                  QCP quaternion; a frame keeps the nearest reference.
//   k_rot          one thread per frame: exact FP64 rotation from the
//                  quaternion; it and the centre as hi/lo FP32 splits.
//   k_sample_sum   mean residual d = R y - r over the first kSample frames of
//                  each reference (fixed chunks, fixed order).
//   k_ref_update   moves each reference to that mean: residuals shrink to each
//                  frame's own fluctuation.
//   k_build        p = sqrt(w)(R (x - c) - r_a); the FP16 hi/lo split with a
//                  per-frame power-of-two scale (tensor path) or the FP32
//                  plane; n_f = |p|^2 and P_fc = sum p (sqrt(w) r_c)^T from the
//                  exact operand values the contraction reads.
//   k_ref_terms    per reference pair: exact rotation U_ab, U_ab S_ba, and
//                  sum w |r_a - U_ab r_b|^2 (O(N) per pair of references).
#include <cooperative_groups.h>
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
constexpr int kScanList = 1024;  // frames listed per block and range in a pruned k-centre scan
constexpr int kWarps = kPrepThreads / 32;
// k_scan and k_build split each frame's atom chunks over kWPF warps: a chunk
// of input (1,250 frames) then keeps twice the warps busy.  The parts' sums
// meet in shared memory in a fixed order, so every launch shape gives the
// same bits.
constexpr int kWPF = 2;
constexpr int kFPB = kWarps / kWPF;  // frames per block per round

__device__ __forceinline__ void group_sync(int grp) {
  asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(32 * kWPF) : "memory");
}
// Single-block kernels (weights, one reference, reference-pair terms) walk N
// atoms with FP64 sums; their time is the serial FP64 tail of one thread (a
// larger block measured slower).
constexpr int kOneBlockThreads = 256;
// Those kernels run as one cluster of kRefCluster CTAs (on as many SMs): each
// CTA walks every kRefCluster-th block of atoms and the sums are combined
// across the cluster in distributed shared memory (cluster_reduce_f64).
constexpr int kRefCluster = 8;

namespace cg = cooperative_groups;

// Sums of NS doubles and maxima of NM non-negative doubles over all threads
// of all CTAs of this cluster, returned to every thread, in one exchange.
// Per value: a shuffle tree per warp, then warp 0 alone combines the warps'
// results by the same tree (FP64 adds are slow on GB300: the other warps
// would only repeat them), lane k keeping value k; each CTA's result goes to
// CTA 0's `slots`, and after a cluster barrier every CTA combines the slots
// in rank order, so all CTAs see the same (deterministic) totals.  red: >=
// 32*(NS+NM) doubles, slots: >= kRefCluster*(NS+NM), bc: >= NS+NM doubles of
// this CTA's shared memory.  Every thread of every CTA of the cluster must
// call it (it contains block and cluster barriers).
template <int NS, int NM>
__device__ __forceinline__ void cluster_reduce_f64(double (&v)[NS], double (&m)[NM], double* red, double* slots,
                                                   double* bc) {
  constexpr int NV = NS + NM;
  static_assert(NV <= 32, "lane k keeps value k");
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < NS; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
#pragma unroll
    for (int k = 0; k < NM; ++k) m[k] = fmax(m[k], __shfl_xor_sync(0xffffffffu, m[k], o));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();  // `red` may still be read by an earlier reduction
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NS; ++k) red[k * 32 + warp] = v[k];
#pragma unroll
    for (int k = 0; k < NM; ++k) red[(NS + k) * 32 + warp] = m[k];
  }
  __syncthreads();
  cg::cluster_group cl = cg::this_cluster();
  const unsigned rank = cl.block_rank(), n = cl.num_blocks();
  if (warp == 0) {
    double* dst = cl.map_shared_rank(slots, 0);
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = (lane < nw) ? red[k * 32 + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_xor_sync(0xffffffffu, t, o);
        t = (k < NS) ? t + u : fmax(t, u);
      }
      if (lane == k) dst[rank * NV + k] = t;
    }
  }
  cl.sync();
  if (threadIdx.x < NV) {
    const double* src = cl.map_shared_rank(slots, 0);
    const bool is_sum = (int)threadIdx.x < NS;
    double t = 0.0;
    for (unsigned r = 0; r < n; ++r) {
      const double u = src[r * NV + threadIdx.x];
      t = is_sum ? t + u : fmax(t, u);
    }
    bc[threadIdx.x] = t;
  }
  cl.sync();  // CTA 0's slots are free again; bc is visible in this CTA
#pragma unroll
  for (int k = 0; k < NS; ++k) v[k] = bc[k];
#pragma unroll
  for (int k = 0; k < NM; ++k) m[k] = bc[NS + k];
}
constexpr int kSample = 2048;      // frames per reference that set its refined mean
constexpr int kMeanChunks = 64;    // fixed partition of those frames
constexpr int kFtab = 24;          // floats per frame in the rotation table

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

size_t prep_scratch_bytes(int64_t F, int N, int Kmax) {
  size_t b = 0;
  b += align256(sizeof(float) * N);
  b += align256(sizeof(double) * 8);
  b += align256(sizeof(float2) * (size_t)Kmax * 3 * N);
  b += align256(sizeof(double) * 3 * Kmax);
  b += align256(sizeof(float) * Kmax);
  b += align256(sizeof(float4) * F);
  b += align256(sizeof(float) * F);
  b += align256(sizeof(float) * kFtab * F);
  b += align256(sizeof(int) * F) * 2;
  b += align256(sizeof(float4) * (size_t)Kmax * N) * 2;
  b += align256(sizeof(int) * 2);
  b += align256(sizeof(unsigned));
  b += align256(sizeof(double) * 9 * (size_t)((N + 31) / 32));  // k_ref_update's blocks
  b += align256(sizeof(float) * Kmax);
  return b;
}

PrepScratch prep_carve(void* base, int64_t F, int N, int Kmax) {
  char* p = (char*)base;
  PrepScratch s;
  auto take = [&](size_t bytes) {
    char* r = p;
    p += align256(bytes);
    return (void*)r;
  };
  s.cmf_ref = (float*)take(sizeof(float) * N);
  s.scal = (double*)take(sizeof(double) * 8);
  s.refhl = (float2*)take(sizeof(float2) * (size_t)Kmax * 3 * N);
  s.sr = (double*)take(sizeof(double) * 3 * Kmax);
  s.rmax = (float*)take(sizeof(float) * Kmax);
  s.quat = (float4*)take(sizeof(float4) * F);
  s.ymax = (float*)take(sizeof(float) * F);
  s.ftab = (float*)take(sizeof(float) * kFtab * F);
  s.pos = (int*)take(sizeof(int) * F);
  s.assign_pos = (int*)take(sizeof(int) * F);
  s.qscan = (float4*)take(sizeof(float4) * (size_t)Kmax * N);
  s.qbuild = (float4*)take(sizeof(float4) * (size_t)Kmax * N);
  s.kstate = (int*)take(sizeof(int) * 2);
  s.rcount = (unsigned*)take(sizeof(unsigned));
  s.rsu = (double*)take(sizeof(double) * 9 * (size_t)((N + 31) / 32));
  s.dref = (float*)take(sizeof(float) * Kmax);
  return s;
}

template <int NV>
__device__ __forceinline__ void warp_sum_f32(float (&v)[NV]) {
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

// One atom's coordinates as FP32 hi + lo (lo = 0 for FP32 input).
__device__ __forceinline__ void load_atom(const float* x, int a, float (&h)[3], float (&l)[3]) {
  h[0] = x[3 * a]; h[1] = x[3 * a + 1]; h[2] = x[3 * a + 2];
  l[0] = l[1] = l[2] = 0.0f;
}
__device__ __forceinline__ void load_atom(const double* x, int a, float (&h)[3], float (&l)[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double v = x[3 * a + k];
    h[k] = (float)v;
    l[k] = (float)(v - (double)h[k]);
  }
}

// Staging of FP32 frames in shared memory: chunks of kChunkAtoms atoms (AoS,
// 3 floats each), from which lanes take their atoms (stride 3 floats: no bank
// conflicts).  A stage buffer holds kStage floats, 16-byte aligned.
constexpr int kChunkAtoms = 128;
constexpr int kStage = 3 * kChunkAtoms + 4;

// Coordinates of atom a as FP32 hi + lo: from the staged chunk (FP32 input)
// or from global memory (FP64 input).
__device__ __forceinline__ void fetch_atom(const float* x, const float* xs, int a, int a0, float (&h)[3],
                                           float (&l)[3]) {
  (void)x;
  const float* p = xs + 3 * (a - a0);
  h[0] = p[0]; h[1] = p[1]; h[2] = p[2];
  l[0] = l[1] = l[2] = 0.0f;
}
__device__ __forceinline__ void fetch_atom(const double* x, const float* xs, int a, int a0, float (&h)[3],
                                           float (&l)[3]) {
  (void)xs;
  (void)a0;
  load_atom(x, a, h, l);
}

// Multistage staging.  Each warp streams the chunks of all its frames --
// frames f0, f0 + stride, ... below F, chunks in atom order -- through a
// ring of kPipe shared-memory stages with cp.async
// (16-byte copies for the aligned body of a chunk, 4-byte copies for its
// unaligned head and tail, so nothing outside the frame is read).  kPipe - 1
// chunks are in flight while the warp computes on the oldest, and the stream
// runs on into the warp's next frame, so the memory latency is covered
// without holding the data in registers.  Completion is tracked with
// cp.async groups (one per chunk, empty past the last one): no spin-waits.
constexpr int kPipe = 3;

__device__ __forceinline__ void cp_async16(float* dst, const float* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Floats before the first 16-byte boundary of a chunk, and where the chunk's
// element 0 sits in its stage buffer (so that the body lands 16-byte aligned).
__device__ __forceinline__ int chunk_head(const float* src, int n) {
  const int head = (int)((16u - ((unsigned)(uintptr_t)src & 15u)) & 15u) >> 2;
  return head > n ? n : head;
}

// Warms this SM's L1 with a per-atom table every warp of the block reads:
// the block's warps start on atom 0 together, and without this each of them
// would miss on the same lines at once.  Fire and forget -- the lines land
// while the warps wait for their first staged coordinates.
__device__ __forceinline__ void prefetch_l1(const void* p, size_t bytes) {
  if (!p) return;
  const char* c = (const char*)p;
  for (size_t o = (size_t)threadIdx.x * 128; o < bytes; o += (size_t)blockDim.x * 128)
    asm volatile("prefetch.global.L1 [%0];" ::"l"(c + o));
}

template <typename T>
struct WarpPipe {
  FrameSrc<T> src;
  int64_t f_next, F, stride;  // next frame to issue, end, this warp's frame stride
  int c_next, c_lo, c_hi, issued;  // next chunk of f_next, this warp's chunks [c_lo, c_hi), chunks issued
  float* ring;                // kPipe * kStage floats, 16-byte aligned
  const int* list = nullptr;  // optional: f_next indexes a list of frames base + list[f_next]
  int64_t base = 0;
  __device__ __forceinline__ int64_t frame_at(int64_t i) const { return list ? base + list[i] : i; }

  // The warp streams chunks [c_lo, c_hi) of each of its frames (its part of
  // a frame shared by kWPF warps).
  __device__ __forceinline__ void init(const FrameSrc<T>& s, int64_t f0, int64_t f_end, int64_t str, float* buf,
                                       int lane, int lo, int hi, const int* lst = nullptr, int64_t lbase = 0) {
    src = s;
    list = lst;
    base = lbase;
    f_next = f0;
    F = f_end;
    stride = str;
    c_lo = lo;
    c_hi = hi;
    c_next = lo;
    issued = 0;
    ring = buf;
    if constexpr (sizeof(T) == 4) {
#pragma unroll
      for (int k = 0; k < kPipe - 1; ++k) issue(lane);
    }
  }
  __device__ __forceinline__ void issue(int lane) {
    if constexpr (sizeof(T) == 4) {
      if (f_next < F && c_hi > c_lo) {
        const int N = src.N, a0 = c_next * kChunkAtoms;
        const float* x = (const float*)src.frame(frame_at(f_next)) + 3 * (size_t)a0;
        const int n = 3 * (min(a0 + kChunkAtoms, N) - a0);
        const int head = chunk_head(x, n);
        const int nv = (n - head) >> 2, tail0 = head + 4 * nv;
        float* dst = ring + (issued % kPipe) * kStage + ((4 - head) & 3);
#pragma unroll
        for (int i = 0; i < (3 * kChunkAtoms / 4 + 31) / 32; ++i) {
          const int j = lane + 32 * i;
          if (j < nv) cp_async16(dst + head + 4 * j, x + head + 4 * j);
        }
        if (lane < head) cp_async4(dst + lane, x + lane);
        if (lane < n - tail0) cp_async4(dst + tail0 + lane, x + tail0 + lane);
        if (++c_next == c_hi) {
          c_next = c_lo;
          f_next += stride;
        }
      }
      cp_async_commit();
      ++issued;
    }
  }
  // body(a, a0, xs) for every atom a of frame f, the next frame of this
  // warp's stream; xs is the staged chunk holding atom a (FP32 input).
  template <class Body>
  __device__ __forceinline__ void for_each_atom(int64_t f, int lane, Body&& body) {
    const int N = src.N;
    if constexpr (sizeof(T) == 4) {
      const float* x = (const float*)src.frame(f);
      for (int c = c_lo; c < c_hi; ++c) {
        const int a0 = c * kChunkAtoms;
        const int consumed = issued - (kPipe - 1);
        cp_async_wait<kPipe - 2>();
        __syncwarp();
        const float* cx = x + 3 * (size_t)a0;
        const int n = 3 * (min(a0 + kChunkAtoms, N) - a0);
        const float* xs = ring + (consumed % kPipe) * kStage + ((4 - chunk_head(cx, n)) & 3);
        issue(lane);  // refills the stage consumed one chunk ago
#pragma unroll
        for (int kk = 0; kk < kChunkAtoms / 32; ++kk) {
          const int a = a0 + lane + 32 * kk;
          if (a < N) body(a, a0, xs);
        }
        __syncwarp();
      }
    } else {
      const int a_hi = min(c_hi * kChunkAtoms, N);
      for (int a = c_lo * kChunkAtoms + lane; a < a_hi; a += 32) body(a, 0, ring);
    }
  }
  // body(a, a0, xs, two) for the atom pairs (a, a + 1) of frame f, a even
  // (lane l takes atoms 2l and 2l + 1 of each 64); two = (a + 1 < N).  A
  // chunk holds whole pairs (kChunkAtoms is even).
  template <class Body>
  __device__ __forceinline__ void for_each_pair(int64_t f, int lane, Body&& body) {
    static_assert(kChunkAtoms % 64 == 0, "a chunk holds whole pairs of every lane");
    const int N = src.N;
    if constexpr (sizeof(T) == 4) {
      const float* x = (const float*)src.frame(f);
      for (int c = c_lo; c < c_hi; ++c) {
        const int a0 = c * kChunkAtoms;
        const int consumed = issued - (kPipe - 1);
        cp_async_wait<kPipe - 2>();
        __syncwarp();
        const float* cx = x + 3 * (size_t)a0;
        const int n = 3 * (min(a0 + kChunkAtoms, N) - a0);
        const float* xs = ring + (consumed % kPipe) * kStage + ((4 - chunk_head(cx, n)) & 3);
        issue(lane);  // refills the stage consumed one chunk ago
#pragma unroll
        for (int kk = 0; kk < kChunkAtoms / 64; ++kk) {
          const int a = a0 + 2 * lane + 64 * kk;
          if (a < N) body(a, a0, xs, a + 1 < N);
        }
        __syncwarp();
      }
    } else {
      const int a_hi = min(c_hi * kChunkAtoms, N);
      for (int a = c_lo * kChunkAtoms + 2 * lane; a < a_hi; a += 64) body(a, 0, ring, a + 1 < N);
    }
  }
  __device__ __forceinline__ void drain() {
    if constexpr (sizeof(T) == 4) cp_async_wait<0>();
  }
};

// Weights in the forms the passes read; scal = {max sqrt(w), sum w, sum of
// the reference centring masses, 0, 1 / sum w, 1 / sum of the reference
// centring masses} (a reciprocal is 0 when its sum is 0).  Run by the cluster
// that builds reference 0 (k_make_ref), at its start: atom a's sqrt(w) is
// written and then read by the same thread.
struct WeightsPass {
  const double* w;
  const double* cmass_ref;  // distinct reference centring masses or nullptr
  double* sqw;
  float* sqwf;
  float* cmf_ref;
  double* scal;
};
// This thread's atoms: writes their weight forms, adds {sum w, sum of the
// reference centring masses} into v and the largest sqrt(w) into mx.
__device__ __forceinline__ void weights_local(const WeightsPass& P, int N, double* v, double& mx) {
  const int stride = kRefCluster * blockDim.x;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += stride) {
    const double wa = P.w ? P.w[a] : 1.0;
    const double ca = P.cmass_ref ? P.cmass_ref[a] : 1.0;
    const double s = sqrt(wa);
    if (P.w) {
      P.sqw[a] = s;
      P.sqwf[a] = (float)s;
    }
    if (P.cmass_ref) P.cmf_ref[a] = (float)ca;
    mx = fmax(mx, s);
    v[0] += wa;
    v[1] += ca;
  }
}
__device__ __forceinline__ void weights_store(const WeightsPass& P, const double* v, double mx) {
  double* scal = P.scal;
  scal[0] = mx;
  scal[1] = v[0];
  scal[2] = v[1];
  scal[3] = 0.0;
  scal[4] = (v[0] != 0.0) ? 1.0 / v[0] : 0.0;
  scal[5] = (v[1] != 0.0) ? 1.0 / v[1] : 0.0;
}

// FP64-accumulated centres (the FP64 checking mode only).
template <typename T>
__global__ void __launch_bounds__(kPrepThreads) k_centroid(FrameSrc<T> src, int64_t F,
                                                           const double* cmass_ref,
                                                           const double* cmass_tgt, double* cen) {
  const int lane = threadIdx.x & 31;
  for (int64_t f = blockIdx.x * (int64_t)kWarps + (threadIdx.x >> 5); f < F; f += (int64_t)gridDim.x * kWarps) {
    const T* x = src.frame(f);
    const double* m = (f < src.n_ref) ? cmass_ref : cmass_tgt;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int a = lane; a < src.N; a += 32) {
      const double w = m ? m[a] : 1.0;
      v[0] += w * (double)x[3 * a];
      v[1] += w * (double)x[3 * a + 1];
      v[2] += w * (double)x[3 * a + 2];
      v[3] += w;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
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

// Reference k := frame *fsel centred (and, when fitting and use_parent,
// superposed onto its nearest reference with the quaternion its scan kept).
// Reference 0 is built before any centre is
// known and centres its frame itself.  Writes the FP64 reference, sqrt(w) r
// (FP32, also packed with sqrt(w) for the scans), r as hi + lo floats,
// sum w |r|^2, sum w r and max |r|.  FP64 per
// atom: one cluster of kRefCluster CTAs shares the atoms.
template <typename T>
__global__ void __cluster_dims__(kRefCluster, 1, 1) __launch_bounds__(kOneBlockThreads)
    k_make_ref(FrameSrc<T> src, const int64_t* fsel, const double* cen, const double* cmass_ref,
               const double* cmass_tgt, const double* w, const double* sqw, const int* assign, int k, int use_parent,
               int nofit, double* refs, float* swr, float2* refhl, double* Eref, double* sr, float* rmax,
               float4* qscan, const int* gate = nullptr, WeightsPass wp = WeightsPass{},
               const float4* quat = nullptr, float* dref = nullptr, double Wsum = 1.0) {
  // A gated round after the k-centre choice has stopped: every CTA of the
  // cluster reads the same word and leaves before any barrier.
  if (gate && *gate != 0) return;
  __shared__ double red[32 * 10], slots[kRefCluster * 10], bc[10];
  __shared__ double Rs[9], cs[3];
  const int N = src.N;
  const int a_first = blockIdx.x * blockDim.x + threadIdx.x, stride = kRefCluster * blockDim.x;
  const int64_t f = *fsel;
  const T* x = src.frame(f);
  if (threadIdx.x < 9) Rs[threadIdx.x] = (threadIdx.x % 4 == 0) ? 1.0 : 0.0;
  // Reference 0: the weights first (their sums travel in the same cluster
  // exchange as the frame's centre).
  double wv[2] = {0.0, 0.0}, wmx[1] = {0.0};
  if (wp.scal) weights_local(wp, N, wv, wmx[0]);
  double c0 = 0.0, c1 = 0.0, c2 = 0.0;
  if (nofit || use_parent) {
    if (!nofit) {
      c0 = cen[3 * f];
      c1 = cen[3 * f + 1];
      c2 = cen[3 * f + 2];
    }
    if (wp.scal) {
      cluster_reduce_f64<2, 1>(wv, wmx, red, slots, bc);
      if (blockIdx.x == 0 && threadIdx.x == 0) weights_store(wp, wv, wmx[0]);
    }
  } else {
    const double* m = (f < src.n_ref) ? cmass_ref : cmass_tgt;
    double v[6] = {0.0, 0.0, 0.0, 0.0, wv[0], wv[1]};
    for (int a = a_first; a < N; a += stride) {
      const double wm = m ? m[a] : 1.0;
      v[0] += wm * (double)x[3 * a];
      v[1] += wm * (double)x[3 * a + 1];
      v[2] += wm * (double)x[3 * a + 2];
      v[3] += wm;
    }
    cluster_reduce_f64<6, 1>(v, wmx, red, slots, bc);
    // one thread divides (an FP64 division is a long sequence on the FP64 pipe)
    if (threadIdx.x == 0) {
      if (wp.scal && blockIdx.x == 0) weights_store(wp, v + 4, wmx[0]);
      double wt = m ? v[3] : (double)N;
      if (m && wt == 0.0) {
        wt = 1.0;
        v[0] = v[1] = v[2] = 0.0;
      }
      cs[0] = v[0] / wt;
      cs[1] = v[1] / wt;
      cs[2] = v[2] / wt;
    }
    __syncthreads();
    c0 = cs[0];
    c1 = cs[1];
    c2 = cs[2];
  }
  __syncthreads();
  double* rk = refs + (size_t)k * 3 * N;
  // Orientation: the frame superposed onto its parent reference with the
  // quaternion its scan kept (an FP64-orthogonal rotation; any rotation
  // serves, since the rotations between references are computed exactly
  // from the references themselves).
  const int parent = use_parent ? assign[f] : -1;
  if (!nofit && parent >= 0) {
    if (threadIdx.x == 0) {
      const float4 qf = quat[f];
      const float q4[4] = {qf.x, qf.y, qf.z, qf.w};
      double R[9];
      rotation_from_quat(q4, R);
      for (int q = 0; q < 9; ++q) Rs[q] = R[q];
    }
    __syncthreads();
  }
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  double mx = 0.0;
  for (int a = a_first; a < N; a += stride) {
    const double wa = w ? w[a] : 1.0;
    const double y0 = (double)x[3 * a] - c0, y1 = (double)x[3 * a + 1] - c1, y2 = (double)x[3 * a + 2] - c2;
    double r[3] = {y0, y1, y2};  // no parent fit: R = I
    if (!nofit && parent >= 0) {
      r[0] = Rs[0] * y0 + Rs[1] * y1 + Rs[2] * y2;
      r[1] = Rs[3] * y0 + Rs[4] * y1 + Rs[5] * y2;
      r[2] = Rs[6] * y0 + Rs[7] * y1 + Rs[8] * y2;
    }
    const double sw = w ? sqw[a] : 1.0;
    float q[3];
    for (int p = 0; p < 3; ++p) {
      rk[3 * a + p] = r[p];
      q[p] = (float)(sw * r[p]);
      swr[((size_t)k * N + a) * 3 + p] = q[p];
      const float rh = (float)r[p];
      refhl[((size_t)k * N + a) * 3 + p] = make_float2(rh, (float)(r[p] - (double)rh));
      acc[1 + p] += wa * r[p];
    }
    qscan[(size_t)k * N + a] = make_float4(q[0], q[1], q[2], (float)sw);
    const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    acc[0] += wa * r2;
    mx = fmax(mx, r2);
  }
  double mxa[1] = {mx};
  cluster_reduce_f64<4, 1>(acc, mxa, red, slots, bc);
  mx = mxa[0];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    Eref[k] = acc[0];
    sr[3 * k] = acc[1];
    sr[3 * k + 1] = acc[2];
    sr[3 * k + 2] = acc[3];
    rmax[k] = (float)sqrt(mx);
  }
  if (dref) {
    // Distances from reference k to references 0..k-1, one warp each, with
    // the arithmetic of the scans (FP32 sums of sqrt(w) r, FP32 QCP): the
    // k-centre round's scan skips a frame that reference k cannot take
    // (triangle inequality).  The swr rows of reference k were written by
    // every CTA of the cluster before the cluster barriers above.
    static_assert(kRefCluster * (kOneBlockThreads / 32) >= kMaxRefs, "one warp per earlier reference");
    const int lane = threadIdx.x & 31;
    const int a = (int)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
    if (a < k) {
      const float* rk_f = swr + (size_t)k * 3 * N;
      const float* ra_f = swr + (size_t)a * 3 * N;
      float M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int i = lane; i < N; i += 32) {
        const float y0 = rk_f[3 * i], y1 = rk_f[3 * i + 1], y2 = rk_f[3 * i + 2];
        const float r0 = ra_f[3 * i], r1 = ra_f[3 * i + 1], r2 = ra_f[3 * i + 2];
        M[0] = fmaf(y0, r0, M[0]); M[1] = fmaf(y0, r1, M[1]); M[2] = fmaf(y0, r2, M[2]);
        M[3] = fmaf(y1, r0, M[3]); M[4] = fmaf(y1, r1, M[4]); M[5] = fmaf(y1, r2, M[5]);
        M[6] = fmaf(y2, r0, M[6]); M[7] = fmaf(y2, r1, M[7]); M[8] = fmaf(y2, r2, M[8]);
      }
#pragma unroll
      for (int q = 0; q < 9; ++q)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) M[q] += __shfl_xor_sync(0xffffffffu, M[q], o);
      if (lane == 0) {
        const float E0 = (float)(0.5 * (acc[0] + Eref[a]));
        float d2 = 0.0f;
        if (E0 > 0.0f) {
          float q[4], lr = 1.0f;
          qcp_vec_f32(M, E0, q, &lr);
          d2 = 2.0f * E0 * (1.0f - lr) * (float)(1.0 / Wsum);
        }
        dref[a] = sqrtf(fmaxf(d2, 0.0f));
      }
    }
  }
}

// A frame's rotation table: the FP64-orthogonal rotation of its quaternion
// and its centre, both as FP32 hi + lo (see k_rot).
__device__ __forceinline__ void write_frame_table(float* ftab, double* rot, int64_t f, const float (&q)[4],
                                                  const double (&c)[3], int nofit) {
  double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (!nofit) rotation_from_quat(q, R);
  float* o = ftab + (size_t)kFtab * f;
  for (int k = 0; k < 9; ++k) {
    const float h = (float)R[k];
    o[k] = h;
    o[9 + k] = (float)(R[k] - (double)h);
  }
  for (int k = 0; k < 3; ++k) {
    const float h = (float)c[k];
    o[18 + k] = h;
    o[21 + k] = (float)(c[k] - (double)h);
  }
  if (rot)
    for (int k = 0; k < 9; ++k) rot[9 * f + k] = R[k];
}

struct ScanArgs {
  const float* cm_ref;  // centring masses of reference frames (FP32), read when cm_ref_is_w == 0
  int cm_ref_is_w;      // reference frames centre with the fit weights (target frames always do)
  const double* scal;   // the weights' scal (k_make_ref): [1] sum w, [2] sum of reference centring masses, [4], [5] reciprocals
  const float4* q;      // [N] {sqrt(w) r_k, sqrt(w)} (the weights centre too: w = sqrt(w)^2)
  const double* sr;     // sum w r_k, [3]
  const double* Eref;   // &Eref[k]
  double Wsum;
  int k, nofit;
  const int* gate;      // non-null and non-zero at launch: the k-centre choice has stopped, the pass does nothing
  double* cen;
  float* dist;
  int* assign;
  float4* quat;
  float* ymax;
  const float* dref;    // rounds k > 0: distances from reference k to references 0..k-1 (nullptr: fit every frame)
  float margin;         // Angstrom added to the skip test for the FP32 distances
};

// FIRST: centre + extent + fit to reference 0 in one read of the frame.  The
// sums use u = x - x0 (x0 = the frame's first atom) so FP32 accumulates
// quantities of the size of the molecule, not of its absolute position:
//   c = x0 + sum cm u / sum cm
//   sum w y r^T = sum w u r^T - (c - x0) (sum w r)^T
//   sum w |y|^2 = sum w |u|^2 - 2 (c - x0).sum w u + W |c - x0|^2
// Later passes (reference k > 0) centre with the known c directly.
// Plain FP32 sums: an error d in a frame's centre moves every operand of the
// frame by the same vector, which changes a best-fit RMSD only at second
// order (|d_i - U d_j|^2 in RMSD^2), and the fit here only picks the
// pre-alignment, which any rotation serves.
template <typename T, bool FIRST>
__global__ void __launch_bounds__(kPrepThreads, 4) k_scan(FrameSrc<T> src, int64_t f_begin, int64_t F, ScanArgs s) {
  if (s.gate && *s.gate != 0) return;  // uniform over the grid: before any barrier
  __shared__ __align__(16) float sbuf[kWarps][kPipe * kStage];
  __shared__ float xpart[2][kFPB][kWPF - 1][17];  // the other parts' sums, by frame parity
  const int N = src.N, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = warp / kWPF, part = warp % kWPF;
  const bool fit = !s.nofit;
  const int64_t f_first = f_begin + blockIdx.x * (int64_t)kFPB + grp;
  const int64_t f_stride = (int64_t)gridDim.x * kFPB;
  const int nch = (N + kChunkAtoms - 1) / kChunkAtoms;
  WarpPipe<T> pipe;
  const int c_lo = part * nch / kWPF, c_hi = (part + 1) * nch / kWPF;
  {
    const size_t n4 = (size_t)N * 4;
    prefetch_l1(s.q, 4 * n4);
    if (FIRST && !s.cm_ref_is_w && f_begin < src.n_ref) prefetch_l1(s.cm_ref, n4);
  }
  // One frame: its atoms through this warp's pipe (the frame the pipe
  // streams next), the parts' sums, the per-frame tail.
  auto frame_body = [&](const int64_t f, const int it) {
    const T* x = src.frame(f);
    const bool in_ref = f < src.n_ref;
    const bool same_w = in_ref ? (s.cm_ref_is_w != 0) : true;  // centring masses = fit weights
    float o0, o1, o2;  // origin of the sums: x0 (FIRST) or the centre
    if (FIRST) {
      o0 = (float)x[0]; o1 = (float)x[1]; o2 = (float)x[2];
      if (!fit) o0 = o1 = o2 = 0.0f;
    } else {
      o0 = (float)s.cen[3 * f]; o1 = (float)s.cen[3 * f + 1]; o2 = (float)s.cen[3 * f + 2];
    }
    // v: 0-8 sum w u r^T, 9 sum w|u|^2 (fit) or sum |sqrt(w)x - sqrt(w)r|^2,
    //    10-12 sum cm u, 13-15 sum w u (weights differing from cm).
    float v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = 0.0f;
    float umax = 0.0f;  // max |u|^2
    pipe.for_each_atom(f, lane, [&](int a, int a0, const float* xs) {
      const float4 t = __ldg(s.q + a);
      const float sw = t.w, r0 = t.x, r1 = t.y, r2 = t.z;
      float xh[3], xl[3];
      fetch_atom(x, xs, a, a0, xh, xl);
      float u0 = xh[0] - o0, u1 = xh[1] - o1, u2 = xh[2] - o2;
      if constexpr (sizeof(T) == 8) {
        u0 += xl[0]; u1 += xl[1]; u2 += xl[2];
      }
      const float y0 = sw * u0, y1 = sw * u1, y2 = sw * u2;
      if (fit) {
        v[0] = fmaf(y0, r0, v[0]); v[1] = fmaf(y0, r1, v[1]); v[2] = fmaf(y0, r2, v[2]);
        v[3] = fmaf(y1, r0, v[3]); v[4] = fmaf(y1, r1, v[4]); v[5] = fmaf(y1, r2, v[5]);
        v[6] = fmaf(y2, r0, v[6]); v[7] = fmaf(y2, r1, v[7]); v[8] = fmaf(y2, r2, v[8]);
        v[9] = fmaf(y0, y0, fmaf(y1, y1, fmaf(y2, y2, v[9])));
      } else {
        const float d0 = y0 - r0, d1 = y1 - r1, d2 = y2 - r2;
        v[9] = fmaf(d0, d0, fmaf(d1, d1, fmaf(d2, d2, v[9])));
      }
      if (FIRST) {
        if (fit) {
          const float wa = sw * sw;
          const float c = same_w ? wa : __ldg(s.cm_ref + a);
          v[10] = fmaf(c, u0, v[10]); v[11] = fmaf(c, u1, v[11]); v[12] = fmaf(c, u2, v[12]);
          if (!same_w) {
            v[13] = fmaf(wa, u0, v[13]); v[14] = fmaf(wa, u1, v[14]); v[15] = fmaf(wa, u2, v[15]);
          }
        }
        umax = fmaxf(umax, fmaf(u0, u0, fmaf(u1, u1, u2 * u2)));
      }
    });
    warp_sum_f32<16>(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) umax = fmaxf(umax, __shfl_xor_sync(0xffffffffu, umax, o));
    // The frame's other parts hand their sums to part 0 (parts in order).
    if (part != 0 && lane == 0) {
      float* o = xpart[it & 1][grp][part - 1];
#pragma unroll
      for (int q = 0; q < 16; ++q) o[q] = v[q];
      o[16] = umax;
    }
    group_sync(grp);
    if (part == 0 && lane == 0) {
#pragma unroll
      for (int pp = 0; pp < kWPF - 1; ++pp) {
        const float* o = xpart[it & 1][grp][pp];
#pragma unroll
        for (int q = 0; q < 16; ++q) v[q] += o[q];
        umax = fmaxf(umax, o[16]);
      }
    }
    if (part == 0 && lane == 0) {
      // Per-frame tail, one lane.  Only the centre needs FP64 (it feeds the
      // exact superposition of the later passes); the distance to the
      // reference, E0 and the QCP input only choose the nearest reference and
      // start the FP32 QCP, so they stay in FP32 -- a warp-wide FP64
      // instruction costs the whole warp's turn on GB300's narrow FP64 pipe.
      float d2 = 0.0f;
      float q[4] = {1.0f, 0.0f, 0.0f, 0.0f};
      const float Wf = (float)s.Wsum, iWf = (float)(1.0 / s.Wsum);
      if (!fit) {
        d2 = v[9] * iWf;
        if (FIRST) {
          s.cen[3 * f] = s.cen[3 * f + 1] = s.cen[3 * f + 2] = 0.0;
          s.ymax[f] = sqrtf(umax) * (1.0f + 2e-6f);
        }
      } else {
        float del[3] = {0.0f, 0.0f, 0.0f};
        if (FIRST) {
          const double iWc = (in_ref && !s.cm_ref_is_w) ? s.scal[5] : s.scal[4];
          for (int p = 0; p < 3; ++p) {
            const double xo = (p == 0) ? o0 : (p == 1) ? o1 : o2;
            const double dd = (iWc != 0.0) ? (double)v[10 + p] * iWc : -xo;  // zero mass: origin
            s.cen[3 * f + p] = xo + dd;
            del[p] = (float)dd;
          }
          s.ymax[f] = (sqrtf(umax) + sqrtf(del[0] * del[0] + del[1] * del[1] + del[2] * del[2])) * (1.0f + 2e-6f);
        }
        float su[3], sr[3];
        for (int p = 0; p < 3; ++p) {
          su[p] = same_w ? v[10 + p] : v[13 + p];
          sr[p] = (float)s.sr[p];
        }
        float M[9];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) M[3 * i + j] = fmaf(-del[i], sr[j], v[3 * i + j]);
        const float Ey = v[9] - 2.0f * (del[0] * su[0] + del[1] * su[1] + del[2] * su[2]) +
                         Wf * (del[0] * del[0] + del[1] * del[1] + del[2] * del[2]);
        const float E0 = 0.5f * (Ey + (float)*s.Eref);
        if (E0 > 0.0f) {
          float lr = 1.0f;
          qcp_vec_f32(M, E0, q, &lr);
          d2 = 2.0f * E0 * (1.0f - lr) * iWf;
        }
      }
      const float d = sqrtf(fmaxf(d2, 0.0f));
      if (s.k == 0 || d < s.dist[f]) {
        s.dist[f] = d;
        s.assign[f] = s.k;
        s.quat[f] = make_float4(q[0], q[1], q[2], q[3]);
      }
    }
  };
  if constexpr (!FIRST) {
    if (s.dref) {
      // Rounds k > 0 with the triangle inequality: a frame at distance
      // dist from its reference a cannot come nearer to reference k than
      // D(a, k) - dist, so it keeps its assignment when D(a, k) > 2 dist
      // (plus a margin for the FP32 distances) and its fit is skipped.  Each
      // block takes a contiguous range of frames, lists the ones to fit in
      // shared memory, and its groups stream that list.
      __shared__ int flist[kScanList];
      __shared__ int fcount;
      const int64_t span = (F - f_begin + gridDim.x - 1) / gridDim.x;
      const int64_t b0 = f_begin + (int64_t)blockIdx.x * span, b1 = min(F, b0 + span);
      int it = 0;
      for (int64_t c0 = b0; c0 < b1; c0 += kScanList) {
        const int64_t c1 = min(b1, c0 + (int64_t)kScanList);
        if (threadIdx.x == 0) fcount = 0;
        __syncthreads();
        for (int64_t f = c0 + threadIdx.x; f < c1; f += kPrepThreads) {
          const float df = s.dist[f];
          const float D = s.dref[s.assign[f]];
          if (!(D > 2.0f * df + s.margin + 2e-3f * D)) flist[atomicAdd(&fcount, 1)] = (int)(f - c0);
        }
        __syncthreads();
        const int n = fcount;
        pipe.init(src, grp, n, kFPB, sbuf[warp], lane, c_lo, c_hi, flist, c0);
        for (int i = grp; i < n; i += kFPB, ++it) frame_body(c0 + flist[i], it);
        pipe.drain();
        __syncthreads();  // the list is rewritten by the next range
      }
      return;
    }
  }
  pipe.init(src, f_first, F, f_stride, sbuf[warp], lane, c_lo, c_hi);
  int it = 0;
  for (int64_t f = f_first; f < F; f += f_stride, ++it) frame_body(f, it);
  pipe.drain();
}

// Speculation check of one chunk: fail = 1 once a frame of [f0, f1) is
// farther than tau from reference 0 (the test the reference-count decision
// applies to the maximum over all frames).
__global__ void __launch_bounds__(256) k_spec_check(const float* dist, int64_t f0, int64_t f1, float tau,
                                                    int* fail) {
  bool far = false;
  for (int64_t f = f0 + threadIdx.x; f < f1; f += 256) far |= (dist[f] > tau);
  if (__syncthreads_or(far) && threadIdx.x == 0) *fail = 1;
}

// Single-block argmax of dist[0..F): out_val, out_idx (lowest index on ties).
// With multi: *multi = (max > tau), the reference-count decision on the device.
__global__ void k_argmax(const float* dist, int64_t F, float* out_val, int64_t* out_idx, float tau = 0.0f,
                         int* multi = nullptr) {
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
    if (multi) *multi = (sv[0] > tau) ? 1 : 0;
  }
}

// A round k of the k-centre choice run on the device: the argmax of
// dist[0..F); if it is farther than tau, reference k is that frame (fsel) and
// state[1] = k (k + 1 references exist); otherwise state[0] = 1 stops this
// and every later round (their k_make_ref and k_scan launches return at
// once).  state[0] != 0 on entry: an earlier round has stopped.
__global__ void k_argmax_gate(const float* dist, int64_t F, float tau, int k, float* out_val, int64_t* out_idx,
                              int* state) {
  if (state[0] != 0) return;
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
    if (sv[0] > tau) {
      *out_idx = si[0];
      state[1] = k;
    } else {
      state[0] = 1;
    }
  }
}

// One thread per frame: the exact (FP64-orthogonal) rotation of the frame's
// quaternion and the frame centre, both split into FP32 hi + lo.  No-fit:
// R = I, c = 0.  R is kept to twice FP32 precision because its rounding would
// distort every frame the same way (a shear of ~6e-8, about 1e-6 A over a
// 20 A molecule); the rounding of the products R (x - c) is independent from
// atom to atom and averages out of an RMSD.
__global__ void k_rot(int64_t f_begin, int64_t F, const float4* quat, const double* cen, int nofit, float* ftab,
                      double* rot, const int* skip = nullptr) {
  if (skip && *skip != 0) return;
  for (int64_t f = f_begin + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < F;
       f += (int64_t)gridDim.x * blockDim.x) {
    const float4 q4 = quat[f];
    const float q[4] = {q4.x, q4.y, q4.z, q4.w};
    const double c[3] = {cen[3 * f], cen[3 * f + 1], cen[3 * f + 2]};
    write_frame_table(ftab, rot, f, q, c, nofit);
  }
}

// The frame's rotation table, loaded by lanes 0-23 and shared by shuffles.
struct FrameTable {
  float Rh[9], Rl[9], ch[3], cl[3];  // rotation and centre, hi + lo
};
__device__ __forceinline__ void load_table(const float* ftab, int64_t f, int lane, FrameTable& T) {
  const float v = (lane < kFtab) ? ftab[(size_t)kFtab * f + lane] : 0.0f;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    T.Rh[k] = __shfl_sync(0xffffffffu, v, k);
    T.Rl[k] = __shfl_sync(0xffffffffu, v, 9 + k);
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    T.ch[k] = __shfl_sync(0xffffffffu, v, 18 + k);
    T.cl[k] = __shfl_sync(0xffffffffu, v, 21 + k);
  }
}

// Sum of d = R y - r_k (unweighted) over the first kSample frames of
// reference k, split into kMeanChunks fixed chunks: grid (atoms, chunk, k).
// Frames of reference k are order[offsets[k] ...] (order == nullptr: every
// frame, in index order).
template <typename T>
__global__ void __launch_bounds__(128) k_sample_sum(FrameSrc<T> src, int64_t F, int Np, const float* ftab,
                                                    const int* order, const int* offsets, const float2* refhl,
                                                    float* partial, const int* skip = nullptr) {
  if (skip && *skip != 0) return;
  const int k = blockIdx.z, ch = blockIdx.y, N = src.N;
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= Np) return;
  const int64_t lo = offsets ? offsets[k] : 0;
  const int64_t cnt = std::min<int64_t>((offsets ? (int64_t)offsets[k + 1] : F) - lo, (int64_t)kSample);
  const int64_t per = (cnt + kMeanChunks - 1) / kMeanChunks;
  const int64_t b0 = ch * per, b1 = std::min<int64_t>(cnt, b0 + per);
  // Plain FP32 (the hi parts of R, c and r): the mean only has to put the
  // reference near its frames, and every later pass takes the reference as
  // stored, whatever its last bits.
  float s[3] = {0.0f, 0.0f, 0.0f};
  if (a < N) {
    float rh[3];
    for (int p = 0; p < 3; ++p) rh[p] = refhl[((size_t)k * N + a) * 3 + p].x;
    for (int64_t n = b0; n < b1; ++n) {
      const int64_t f = order ? order[lo + n] : lo + n;
      const float* tb = ftab + (size_t)kFtab * f;
      float xh[3], xl[3];
      load_atom(src.frame(f), a, xh, xl);
      const float u0 = xh[0] - tb[18], u1 = xh[1] - tb[19], u2 = xh[2] - tb[20];
#pragma unroll
      for (int p = 0; p < 3; ++p)
        s[p] += fmaf(tb[3 * p], u0, fmaf(tb[3 * p + 1], u1, tb[3 * p + 2] * u2)) - rh[p];
    }
  }
  for (int p = 0; p < 3; ++p) partial[(((size_t)k * kMeanChunks + ch) * 3 + p) * Np + a] = s[p];
}

// r_k += mean d over its sample (FP64 over the chunk sums, fixed order), and
// the derived sqrt(w) r_k, hi/lo r_k and packed build table; grid (atoms /
// 32, reference).  rmax[k] only grows (atomicMax on the non-negative float
// bits), so it stays an upper bound of |r_k|.  Eref and sr describe the
// unrefined references and are not read after this point.
// With RP (one reference): also the reference's terms with itself, in place
// of the reference-pair pass.  Each block writes its FP64 share of
// S = sum w r r^T to `su` and counts itself done; the last block adds the
// shares in block order (so the bits do not depend on which block was last)
// and writes RP[0]: U = I, S, its antisymmetric combos, SS = 0.
struct RefUpdateArgs {
  double* refs;
  float* swr;
  float2* refhl;
  float* rmax;
  float4* qbuild;
  const double* sqw;  // sqrt(w) or nullptr
  const double* w;    // weights or nullptr (self terms)
  unsigned* count;    // [1], zero at launch (self terms)
  double* su;         // [blocks][9] (self terms)
  float* RP;          // non-null (K = 1): write the self terms
};
__global__ void __launch_bounds__(32) k_ref_update(RefUpdateArgs u, const float* partial, const int* offsets,
                                                   int64_t F, int N, int Np, const int* skip = nullptr) {
  if (skip && *skip != 0) return;
  // one warp per block: the FP64 sums of the kMeanChunks partial means are
  // spread over as many SMs as there are 32-atom groups
  const int k = blockIdx.y;
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t cnt = std::min<int64_t>((offsets ? (int64_t)(offsets[k + 1] - offsets[k]) : F), (int64_t)kSample);
  float mx = 0.0f;
  double sv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (a < N) {
    double* r = u.refs + (size_t)k * 3 * N;
    const double sw = u.sqw ? u.sqw[a] : 1.0;
    double rr[3];
    // The chunk sums in chunk order, several chunks' loads in flight at once,
    // in FP32 (four independent partial sums per coordinate): the mean only
    // has to move the reference near its frames, and every later pass reads
    // the reference as stored.  (In FP64 these adds, a warp instruction each
    // on GB300's narrow FP64 pipe, were most of this kernel's time.)
    const float* src = partial + (size_t)k * kMeanChunks * 3 * Np + a;
    float s4[4][3] = {};
#pragma unroll 8
    for (int ch = 0; ch < kMeanChunks; ++ch)
#pragma unroll
      for (int p = 0; p < 3; ++p) s4[ch & 3][p] += src[((size_t)ch * 3 + p) * Np];
    const float icnt = (cnt > 0) ? 1.0f / (float)cnt : 0.0f;
    float q[3];
    for (int p = 0; p < 3; ++p) {
      const float mean = ((s4[0][p] + s4[1][p]) + (s4[2][p] + s4[3][p])) * icnt;
      rr[p] = r[3 * a + p] + (double)mean;
      r[3 * a + p] = rr[p];
      q[p] = (float)(sw * rr[p]);
      u.swr[((size_t)k * N + a) * 3 + p] = q[p];
      const float h = (float)rr[p];
      u.refhl[((size_t)k * N + a) * 3 + p] = make_float2(h, (float)(rr[p] - (double)h));
    }
    u.qbuild[(size_t)k * N + a] = make_float4(q[0], q[1], q[2], (float)sw);
    {
      const float r0 = (float)rr[0], r1 = (float)rr[1], r2 = (float)rr[2];
      mx = sqrtf(fmaf(r0, r0, fmaf(r1, r1, r2 * r2))) * (1.0f + 1e-5f);  // an upper bound of |r|
    }
    if (u.RP) {
      const double wa = u.w ? u.w[a] : 1.0;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) sv[3 * i + j] = wa * rr[i] * rr[j];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (threadIdx.x == 0) atomicMax(reinterpret_cast<int*>(u.rmax + k), __float_as_int(mx));
  if (!u.RP) return;
#pragma unroll
  for (int q = 0; q < 9; ++q)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sv[q] += __shfl_xor_sync(0xffffffffu, sv[q], o);
  __shared__ unsigned s_last;
  if (threadIdx.x == 0) {
    for (int q = 0; q < 9; ++q) u.su[(size_t)blockIdx.x * 9 + q] = sv[q];
    __threadfence();
    s_last = (atomicAdd(u.count, 1u) == gridDim.x - 1);
  }
  __syncwarp();
  if (!s_last) return;
  __threadfence();  // the last block: every share is written
  // lane l adds the shares of blocks l, l + 32, ... (loads independent), then
  // the lanes combine in a fixed tree: the same bits whichever block is last
  double S[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (unsigned g = threadIdx.x; g < gridDim.x; g += 32)
#pragma unroll
    for (int q = 0; q < 9; ++q) S[q] += __ldcg(u.su + (size_t)g * 9 + q);
#pragma unroll
  for (int q = 0; q < 9; ++q)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) S[q] += __shfl_xor_sync(0xffffffffu, S[q], o);
  if (threadIdx.x != 0) return;
  float* o = u.RP;  // K = 1: the pair (0, 0)
  for (int q = 0; q < 9; ++q) o[q] = (q % 4 == 0) ? 1.0f : 0.0f;
  for (int q = 0; q < 9; ++q) o[9 + q] = (float)S[q];
  o[18] = (float)(S[5] - S[7]);
  o[19] = (float)(S[6] - S[2]);
  o[20] = (float)(S[1] - S[3]);
  o[21] = 0.0f;
  o[22] = 0.0f;
  o[23] = 0.0f;
}

struct BuildArgs {
  const float* ftab;
  const int* assign;
  const float* ymax;    // [F] bound of max |y|
  const float* rmax;    // [K] bound of max |r_k|
  const double* scal;   // [0] max sqrt(w)
  const float* swr;     // [K][N][3] sqrt(w) r_c
  const float4* q;      // [K][N] {sqrt(w) r_c, sqrt(w)} of the refined references
  int K, Np;
  int K_build;          // references k_build forms P against (the rest: k_pref)
  int tc;
  __half* hi;
  __half* lo;
  float* inv_scale;
  int write_plane;
  float* plane;
  float* nrm;
  float* P;
  float* trP;
  const int* pos;       // frame -> position of its operands and terms (nullptr = same)
  int* assign_pos;      // reference of the frame at each position (with pos)
  const int* skip;      // device int or nullptr: the pass does nothing when it reads non-zero
};

// Final operands, two warps per frame.  p = sqrt(w) (R_h + R_l)(x - c) - s_a
// in FP32, s_a = sqrt(w) r_a as stored (the same values P is formed with):
// u = x - c rounds relative to the centred extent, the products R u relative
// to |y|, both independently per atom.  Per atom the pass reads one 16-byte
// table entry {s_a, sqrt(w)} (the per-atom table loads, not the arithmetic,
// bounded this pass when they were four to seven separate loads).  The
// tensor path stores p*s as FP16 hi + lo, s = 2^(14 - e) with 2^e above the
// bound sqrt(w)max (max|y| + max|r_a|) >= max|p| (so |hi| < 2^15; a loose
// bound only lowers the floor of the smallest representable residual, far
// below FP32 rounding), and continues with the value hi + lo represents.
// n_f = sum |p|^2 and P_fc = sum p (sqrt(w) r_c)^T use those exact operands.
// MODE: 1 = FP16 hi/lo operands (tensor path), 2 = the FP32 plane, 3 = both.
template <typename T, int MODE>
__global__ void __launch_bounds__(kPrepThreads, 3) k_build(FrameSrc<T> src, int64_t f_begin, int64_t F,
                                                             BuildArgs b) {
  if (b.skip && *b.skip != 0) return;  // uniform over the grid: before any barrier
  constexpr bool TC = (MODE & 1) != 0, PLANE = (MODE & 2) != 0;
  __shared__ __align__(16) float sbuf[kWarps][kPipe * kStage];
  __shared__ float xpart[2][kFPB][kWPF - 1][10];  // the other parts' sums, by round parity
  const int N = src.N, Np = b.Np, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = warp / kWPF, part = warp % kWPF;
  const float sqwmax = (float)b.scal[0];
  const int64_t f_first = f_begin + blockIdx.x * (int64_t)kFPB + grp;
  const int64_t f_stride = (int64_t)gridDim.x * kFPB;
  const int nch = (N + kChunkAtoms - 1) / kChunkAtoms;
  const int c_lo = part * nch / kWPF, c_hi = (part + 1) * nch / kWPF;
  const int a_lo = c_lo * kChunkAtoms, a_hi = min(c_hi * kChunkAtoms, N);  // this part's atoms
  WarpPipe<T> pipe;
  pipe.init(src, f_first, F, f_stride, sbuf[warp], lane, c_lo, c_hi);
  // Sums of NV values over the frame's parts: part 0's lane 0 ends with the
  // total (parts added in order).
  int rnd = 0;
  auto combine = [&](float* acc, int nv) {
    if (part != 0 && lane == 0)
      for (int q = 0; q < nv; ++q) xpart[rnd & 1][grp][part - 1][q] = acc[q];
    group_sync(grp);
    if (part == 0 && lane == 0)
      for (int pp = 0; pp < kWPF - 1; ++pp)
        for (int q = 0; q < nv; ++q) acc[q] += xpart[rnd & 1][grp][pp][q];
    ++rnd;
  };
  prefetch_l1(b.q, (size_t)N * 16);  // reference 0 (the only one when K = 1)
  for (int64_t f = f_first; f < F; f += f_stride) {
    const T* x = src.frame(f);
    const int ra = b.assign[f];
    const int64_t pf = b.pos ? (int64_t)b.pos[f] : f;  // where this frame's operands go
    if (b.pos && part == 0 && lane == 0) b.assign_pos[pf] = ra;
    FrameTable Tb;
    load_table(b.ftab, f, lane, Tb);
    float scale = 1.0f, inv = 1.0f;
    if (TC) {
      const float B = sqwmax * (b.ymax[f] + b.rmax[ra]) * (1.0f + 1e-6f);
      int e = 0;
      if (B > 0.0f && isfinite(B)) frexpf(B, &e);
      e = max(-100, min(100, e));
      scale = ldexpf(1.0f, 14 - e);
      inv = ldexpf(1.0f, e - 14);
      if (part == 0 && lane == 0) b.inv_scale[pf] = inv;
    }
    const float4* qa = b.q + (size_t)ra * N;  // the frame's reference; P is formed against reference 0
    const size_t base = (size_t)pf * 3 * Np;
    float acc[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) acc[q] = 0.0f;
    // One atom's operand row p = sqrt(w) R (x - c) - s_a (s_a = sqrt(w) r_a).
    auto residual = [&](int a, int a0, const float* xs, const float4& t, float (&v)[3]) {
      float xh[3], xl[3], u[3];
      fetch_atom(x, xs, a, a0, xh, xl);
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        u[p] = xh[p] - Tb.ch[p];
        if constexpr (sizeof(T) == 8) u[p] += xl[p];
        u[p] -= Tb.cl[p];
      }
      const float sr[3] = {t.x, t.y, t.z};
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        float y = fmaf(Tb.Rl[3 * p], u[0], fmaf(Tb.Rl[3 * p + 1], u[1], Tb.Rl[3 * p + 2] * u[2]));
        y = fmaf(Tb.Rh[3 * p + 2], u[2], y);
        y = fmaf(Tb.Rh[3 * p + 1], u[1], y);
        y = fmaf(Tb.Rh[3 * p], u[0], y);
        v[p] = fmaf(t.w, y, -sr[p]);
      }
    };
    // Two consecutive atoms per lane: their operands leave as one 4-byte
    // (hi, lo) or 8-byte (plane) store per component, and the FP16 splits
    // convert two values per instruction.  A lone last atom pairs with the
    // first padding position, which holds zero.
    pipe.for_each_pair(f, lane, [&](int a, int a0, const float* xs, bool two) {
        const float4 t0 = __ldg(qa + a);
        const float4 t1 = two ? __ldg(qa + a + 1) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float v0[3], v1[3] = {0.0f, 0.0f, 0.0f};
        residual(a, a0, xs, t0, v0);
        if (two) residual(a + 1, a0, xs, t1, v1);  // (past the frame's last atom nothing is read)
#pragma unroll
        for (int p = 0; p < 3; ++p) {
          const size_t i = base + (size_t)p * Np + a;
          if (TC) {
            const float s0 = v0[p] * scale, s1 = v1[p] * scale;
            const __half2 h = __floats2half2_rn(s0, s1);
            const float2 hf = __half22float2(h);
            const __half2 l = __floats2half2_rn(s0 - hf.x, s1 - hf.y);
            const float2 lf = __half22float2(l);
            *reinterpret_cast<__half2*>(b.hi + i) = h;
            *reinterpret_cast<__half2*>(b.lo + i) = l;
            v0[p] = (hf.x + lf.x) * inv;
            v1[p] = (hf.y + lf.y) * inv;
          }
          if (PLANE) *reinterpret_cast<float2*>(b.plane + i) = make_float2(v0[p], v1[p]);
          acc[9] = fmaf(v0[p], v0[p], fmaf(v1[p], v1[p], acc[9]));
        }
        // P against reference 0 (the frame's own unless frames have several references)
        float4 c0 = t0, c1 = t1;
        if (ra != 0) {
          c0 = __ldg(b.q + a);
          c1 = two ? __ldg(b.q + a + 1) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        acc[0] = fmaf(v0[0], c0.x, fmaf(v1[0], c1.x, acc[0]));
        acc[1] = fmaf(v0[0], c0.y, fmaf(v1[0], c1.y, acc[1]));
        acc[2] = fmaf(v0[0], c0.z, fmaf(v1[0], c1.z, acc[2]));
        acc[3] = fmaf(v0[1], c0.x, fmaf(v1[1], c1.x, acc[3]));
        acc[4] = fmaf(v0[1], c0.y, fmaf(v1[1], c1.y, acc[4]));
        acc[5] = fmaf(v0[1], c0.z, fmaf(v1[1], c1.z, acc[5]));
        acc[6] = fmaf(v0[2], c0.x, fmaf(v1[2], c1.x, acc[6]));
        acc[7] = fmaf(v0[2], c0.y, fmaf(v1[2], c1.y, acc[7]));
        acc[8] = fmaf(v0[2], c0.z, fmaf(v1[2], c1.z, acc[8]));
    });
    // zero padding [N, Np), by the last part (an odd N's position N came with
    // the last atom's pair)
    for (int a = ((N + 1) & ~1) + lane; a < Np && part == kWPF - 1; a += 32) {
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        if (TC) {
          b.hi[base + (size_t)p * Np + a] = __float2half_rn(0.0f);
          b.lo[base + (size_t)p * Np + a] = __float2half_rn(0.0f);
        }
        if (PLANE) b.plane[base + (size_t)p * Np + a] = 0.0f;
      }
    }
    warp_sum_f32<10>(acc);
    combine(acc, 10);
    if (part == 0 && lane == 0) {
      b.nrm[pf] = acc[9];
      float* Pf = b.P + (size_t)pf * b.K * 9;
      for (int q = 0; q < 9; ++q) Pf[q] = acc[q];
      b.trP[(size_t)pf * b.K] = acc[0] + acc[4] + acc[8];
    }
    // P against the other references up to K_build (beyond it: k_pref after
    // this pass): read the operands back (this lane's own writes, same atom
    // mapping, this part's atoms).
    __syncwarp();
    for (int c = 1; c < b.K_build; ++c) {
      const float* rc = b.swr + (size_t)c * N * 3;
      float h9[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) h9[q] = 0.0f;
      for (int a = a_lo + lane; a < a_hi; a += 32) {
        float v[3];
#pragma unroll
        for (int p = 0; p < 3; ++p) {
          const size_t i = base + (size_t)p * Np + a;
          v[p] = TC ? (__half2float(b.hi[i]) + __half2float(b.lo[i])) * inv : b.plane[i];
        }
        const float c0 = rc[3 * a], c1 = rc[3 * a + 1], c2 = rc[3 * a + 2];
        h9[0] += v[0] * c0; h9[1] += v[0] * c1; h9[2] += v[0] * c2;
        h9[3] += v[1] * c0; h9[4] += v[1] * c1; h9[5] += v[1] * c2;
        h9[6] += v[2] * c0; h9[7] += v[2] * c1; h9[8] += v[2] * c2;
      }
      warp_sum_f32<9>(h9);
      combine(h9, 9);
      if (part == 0 && lane == 0) {
        float* Pf = b.P + ((size_t)pf * b.K + c) * 9;
        for (int q = 0; q < 9; ++q) Pf[q] = h9[q];
        b.trP[(size_t)pf * b.K + c] = h9[0] + h9[4] + h9[8];
      }
    }
  }
  pipe.drain();
}

// P_fc = sum_a p_f[a] (sqrt(w) r_c[a])^T against references c = 1 .. K-1 (c = 0
// comes with k_build), from the operands k_build wrote (the values the
// contraction reads).  A block takes 32 operand positions at a time (4 per
// warp) and walks the atoms in chunks of kPrefAtoms: the chunk of every
// reference (atom-major, the 3(K-1) values of an atom contiguous) and of the
// 32 operands is staged in shared memory, then each lane owns up to
// kPrefComb of the 3(K-1) (reference, component) columns and accumulates, for
// its warp's 4 positions, the 3 rows of each.  Per output the sum runs over
// the atoms in order.
constexpr int kPrefAtoms = 64;
constexpr int kPrefFpw = 4;   // positions per warp
constexpr int kPrefComb = 6;  // most columns per lane: 3 (K - 1) <= 32 * 6 (K <= 65)
size_t pref_smem_bytes(int K) {
  return sizeof(float) * ((size_t)kPrefAtoms * 3 * (K - 1) + 8 * kPrefFpw * 3 * kPrefAtoms + 8 * kPrefFpw * 32 * kPrefComb);
}
template <int NC>  // columns per lane: 3 (K - 1) <= 32 * NC
__global__ void __launch_bounds__(256) k_pref(BuildArgs b, int64_t F, int N) {
  extern __shared__ float ps[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int Np = b.Np, K = b.K, ncol = 3 * (K - 1);
  float* rs = ps;                                            // [kPrefAtoms][ncol]
  float* vs = rs + (size_t)kPrefAtoms * ncol;                 // [8][kPrefFpw][3][kPrefAtoms]
  float* dg = vs + 8 * kPrefFpw * 3 * kPrefAtoms;             // [8][kPrefFpw][32 * kPrefComb] diagonal terms
  float* vw = vs + warp * kPrefFpw * 3 * kPrefAtoms;
  for (int64_t g0 = (int64_t)blockIdx.x * 8 * kPrefFpw; g0 < F; g0 += (int64_t)gridDim.x * 8 * kPrefFpw) {
    const int64_t p0 = g0 + (int64_t)warp * kPrefFpw;  // this warp's first position
    float acc[kPrefFpw][NC][3];
#pragma unroll
    for (int f = 0; f < kPrefFpw; ++f)
#pragma unroll
      for (int j = 0; j < NC; ++j)
#pragma unroll
        for (int q = 0; q < 3; ++q) acc[f][j][q] = 0.0f;
    for (int a0 = 0; a0 < N; a0 += kPrefAtoms) {
      const int na = min(kPrefAtoms, N - a0);
      __syncthreads();  // the previous chunk is consumed
      for (int x = threadIdx.x; x < na * ncol; x += blockDim.x) {
        const int al = x / ncol, m = x - al * ncol;
        const int c = 1 + m / 3, qq = m - (m / 3) * 3;
        rs[x] = __ldg(b.swr + ((size_t)c * N + a0 + al) * 3 + qq);
      }
      for (int x = lane; x < kPrefFpw * 3 * kPrefAtoms; x += 32) {
        const int f = x / (3 * kPrefAtoms), r = x - f * 3 * kPrefAtoms;
        const int q = r / kPrefAtoms, al = r - q * kPrefAtoms;
        const int64_t pf = p0 + f;
        float v = 0.0f;
        if (pf < F && al < na) {
          const size_t i = (size_t)pf * 3 * Np + (size_t)q * Np + a0 + al;
          const float inv = b.tc ? b.inv_scale[pf] : 1.0f;
          v = b.tc ? (__half2float(b.hi[i]) + __half2float(b.lo[i])) * inv : b.plane[i];
        }
        vw[x] = v;
      }
      __syncthreads();
      for (int al = 0; al < na; ++al) {
        float r[NC];
#pragma unroll
        for (int j = 0; j < NC; ++j) {
          const int m = lane + 32 * j;
          r[j] = (m < ncol) ? rs[al * ncol + m] : 0.0f;
        }
#pragma unroll
        for (int f = 0; f < kPrefFpw; ++f) {
          const float v0 = vw[(f * 3 + 0) * kPrefAtoms + al], v1 = vw[(f * 3 + 1) * kPrefAtoms + al],
                      v2 = vw[(f * 3 + 2) * kPrefAtoms + al];
#pragma unroll
          for (int j = 0; j < NC; ++j) {
            acc[f][j][0] += v0 * r[j];
            acc[f][j][1] += v1 * r[j];
            acc[f][j][2] += v2 * r[j];
          }
        }
      }
    }
    // P[pf][c][q][q'] for the lane's columns m = 3 (c - 1) + q'; the diagonal
    // terms (q = q') go through shared memory for trP = P00 + P11 + P22.
    float* dw = dg + warp * kPrefFpw * 32 * kPrefComb;
#pragma unroll
    for (int f = 0; f < kPrefFpw; ++f) {
      const int64_t pf = p0 + f;
#pragma unroll
      for (int j = 0; j < NC; ++j) {
        const int m = lane + 32 * j;
        if (m < ncol) {
          const int c = 1 + m / 3, qq = m - (m / 3) * 3;
          if (pf < F) {
            float* Pf = b.P + ((size_t)pf * K + c) * 9;
            Pf[0 * 3 + qq] = acc[f][j][0];
            Pf[1 * 3 + qq] = acc[f][j][1];
            Pf[2 * 3 + qq] = acc[f][j][2];
          }
          dw[f * 32 * kPrefComb + m] = (qq == 0) ? acc[f][j][0] : (qq == 1) ? acc[f][j][1] : acc[f][j][2];
        }
      }
    }
    __syncwarp();
    for (int f = 0; f < kPrefFpw; ++f) {
      const int64_t pf = p0 + f;
      if (pf >= F) break;
      for (int c = 1 + lane; c < K; c += 32) {
        const float* d = dw + f * 32 * kPrefComb + 3 * (c - 1);
        b.trP[(size_t)pf * K + c] = d[0] + d[1] + d[2];
      }
    }
    __syncwarp();
  }
}

// Reference-pair table (kRefPairStride floats per b*K + a): the exact FP64
// rotation U_ab taking r_b onto r_a, SU_ab = U_ab S_ba, its antisymmetric
// combos and sum w |r_a - U_ab r_b|^2.  No-fit mode keeps U = I.
// One block of kRefTermThreads per reference pair: all K^2 pairs run side by
// side, each with its own FP64 solve (a cluster per pair left most of the
// GPU idle behind a few clusters' serial QCP solves).
constexpr int kRefTermThreads = 128;
template <int NV>
__device__ __forceinline__ void block_sum_f64_small(double (&v)[NV], double* red /* >= 4*NV */) {
  static_assert(kRefTermThreads == 128, "four warps");
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) red[warp * NV + k] = v[k];
  __syncthreads();
  // warps summed in a fixed order: the same totals in every thread
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = ((red[k] + red[NV + k]) + red[2 * NV + k]) + red[3 * NV + k];
  __syncthreads();
}

__global__ void __launch_bounds__(kRefTermThreads)
    k_ref_terms(const double* refs, int N, int K, const double* w, int nofit, float* RP, const int* skip) {
  if (skip && *skip != 0) return;
  __shared__ double red[4 * 10];
  __shared__ double Us[9];
  const int pair = blockIdx.x;  // one block per reference pair
  const int b = pair / K, a = pair % K;
  const double* rb = refs + (size_t)b * 3 * N;
  const double* ra = refs + (size_t)a * 3 * N;
  double v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < N; i += kRefTermThreads) {
    const double wa = w ? w[i] : 1.0;
    const double b0 = rb[3 * i], b1 = rb[3 * i + 1], b2 = rb[3 * i + 2];
    const double a0 = ra[3 * i], a1 = ra[3 * i + 1], a2 = ra[3 * i + 2];
    v[0] += wa * b0 * a0; v[1] += wa * b0 * a1; v[2] += wa * b0 * a2;
    v[3] += wa * b1 * a0; v[4] += wa * b1 * a1; v[5] += wa * b1 * a2;
    v[6] += wa * b2 * a0; v[7] += wa * b2 * a1; v[8] += wa * b2 * a2;
    v[9] += wa * (b0 * b0 + b1 * b1 + b2 * b2 + a0 * a0 + a1 * a1 + a2 * a2);
  }
  block_sum_f64_small<10>(v, red);
  if (threadIdx.x == 0) {
    double U[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (a != b && !nofit) qcp_lambda_rot(v, 0.5 * v[9], U);
    for (int k = 0; k < 9; ++k) Us[k] = U[k];
  }
  __syncthreads();
  // SS_ab = sum w |r_a - U r_b|^2, accumulated directly (no cancellation);
  // 0 for a reference with itself.
  double e[1] = {0.0};
  if (a != b) {
    for (int i = threadIdx.x; i < N; i += kRefTermThreads) {
      const double wa = w ? w[i] : 1.0;
      const double b0 = rb[3 * i], b1 = rb[3 * i + 1], b2 = rb[3 * i + 2];
      const double d0 = ra[3 * i] - (Us[0] * b0 + Us[1] * b1 + Us[2] * b2);
      const double d1 = ra[3 * i + 1] - (Us[3] * b0 + Us[4] * b1 + Us[5] * b2);
      const double d2 = ra[3 * i + 2] - (Us[6] * b0 + Us[7] * b1 + Us[8] * b2);
      e[0] += wa * (d0 * d0 + d1 * d1 + d2 * d2);
    }
    block_sum_f64_small<1>(e, red);
  }
  if (threadIdx.x == 0) {
    double SU[9];
    for (int p = 0; p < 3; ++p)
      for (int q = 0; q < 3; ++q)
        SU[p * 3 + q] = Us[p * 3] * v[q] + Us[p * 3 + 1] * v[3 + q] + Us[p * 3 + 2] * v[6 + q];
    float* o = RP + (size_t)pair * kRefPairStride;
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

// ---------------------------------------------------------------------------
// Host driver for the prep passes.
// ---------------------------------------------------------------------------
static BuildArgs build_args(const FinishArgs& fa, const PrepArgs& A, const PrepScratch& S);
// Blocks for a pass over F frames, fpb frames per block at a time: one wave
// of per_sm resident blocks on each of GB300's 152 SMs at most.  The
// cp.async-pipelined passes (k_scan, k_build; kFPB frames per block, each on
// kWPF warps) are persistent: each warp streams several frames, so the
// pipeline fills once per warp rather than once per frame.
static int prep_grid(int64_t F, int per_sm = 16, int fpb = kWarps) {
  return (int)std::min<int64_t>((F + fpb - 1) / fpb, 152 * per_sm);
}
constexpr int kScanBlocksPerSM = 4;   // k_scan: __launch_bounds__(kPrepThreads, 4)
constexpr int kBuildBlocksPerSM = 3;  // k_build: __launch_bounds__(kPrepThreads, 3)
template <typename T>
static void launch_build(int64_t f0, int64_t f1, const FrameSrc<T>& src, const BuildArgs& b, cudaStream_t st) {
  const dim3 grid(prep_grid(f1 - f0, kBuildBlocksPerSM, kFPB));
  const int mode = (b.tc ? 1 : 0) | (b.write_plane ? 2 : 0);
  if (mode == 1)
    k_build<T, 1><<<grid, kPrepThreads, 0, st>>>(src, f0, f1, b);
  else if (mode == 2)
    k_build<T, 2><<<grid, kPrepThreads, 0, st>>>(src, f0, f1, b);
  else
    k_build<T, 3><<<grid, kPrepThreads, 0, st>>>(src, f0, f1, b);
}

// k_rot: one thread per frame, FP64 throughout; small blocks spread the
// frames' FP64 work over more SMs.
constexpr int kRotThreads = 64;
static int rot_grid(int64_t frames) { return (int)std::min<int64_t>((frames + kRotThreads - 1) / kRotThreads, 4096); }

template <typename T>
static cudaError_t prep_impl(const PrepArgs& A, PrepOut& o, cudaStream_t st) {
  FrameSrc<T> src{(const T*)A.ref, (const T*)(A.tgt ? A.tgt : A.ref), A.n_ref, A.N};
  const int64_t F = A.F;
  const int N = A.N;
  const int grid = prep_grid(F);
  int launches = 0;
  if (A.centroid_only) {
    if (A.nofit) {
      cudaMemsetAsync(A.cen, 0, sizeof(double) * 3 * F, st);
    } else {
      k_centroid<T><<<grid, kPrepThreads, 0, st>>>(src, F, A.cmass_ref, A.cmass_tgt, A.cen);
      ++launches;
    }
    o.K = 0;
    o.launches = launches;
    return cudaGetLastError();
  }
  const PrepScratch S = prep_carve(A.scratch, F, N, A.max_refs);
  const bool ref_distinct = A.cmass_ref != nullptr && A.cmass_ref != A.w;
  // The reference refinement of K references (k_sample_sum, k_ref_update);
  // returns its launches.  RP (K = 1): also the reference's terms with itself.
  auto refine = [&](int K, const int* order, const int* offsets, float* RP, const int* skip) -> int {
    dim3 gs((unsigned)((A.Np + 127) / 128), (unsigned)kMeanChunks, (unsigned)K);
    k_sample_sum<T><<<gs, 128, 0, st>>>(src, F, A.Np, S.ftab, order, offsets, S.refhl, A.partial, skip);
    if (RP) cudaMemsetAsync(S.rcount, 0, sizeof(unsigned), st);
    RefUpdateArgs u{A.refs, A.swr, S.refhl, S.rmax, S.qbuild, A.w ? A.sqw : nullptr, A.w, S.rcount, S.rsu, RP};
    k_ref_update<<<dim3((unsigned)((N + 31) / 32), (unsigned)K), 32, 0, st>>>(u, A.partial, offsets, F, N, A.Np,
                                                                            skip);
    return 2;
  };
  ScanArgs sa{};
  sa.cm_ref = ref_distinct ? S.cmf_ref : nullptr;
  sa.cm_ref_is_w = !ref_distinct;
  sa.scal = S.scal;
  sa.Wsum = A.Wsum;
  sa.nofit = A.nofit;
  sa.cen = A.cen;
  sa.dist = A.dist;
  sa.assign = A.assign;
  sa.quat = S.quat;
  sa.ymax = S.ymax;
  // The weights and reference 0 from frame 0 (one launch), then centres + fit
  // to it in one pass (chunk by chunk when the frames are still arriving).
  // (resume_scan: weights, reference 0 and the first scan are in the
  // workspace from the deferred run of this call.)
  if (!A.resume_scan) {
    cudaMemsetAsync(A.fsel, 0, sizeof(int64_t), st);
    if (A.n_chunks > 0) {
      if (A.chunk_copy) (*A.chunk_copy)(0);
      cudaStreamWaitEvent(st, A.chunk_ev[0], 0);
    }
    const WeightsPass wp{A.w, ref_distinct ? A.cmass_ref : nullptr, A.sqw, A.sqwf, S.cmf_ref, S.scal};
    k_make_ref<T><<<kRefCluster, kOneBlockThreads, 0, st>>>(src, A.fsel, A.cen, A.cmass_ref, A.cmass_tgt, A.w,
                                                            A.sqw, A.assign, 0, 0, A.nofit, A.refs, A.swr, S.refhl,
                                                            A.Eref, S.sr, S.rmax, S.qscan, nullptr, wp);
    ++launches;
  }
  sa.k = 0;
  sa.q = S.qscan;  // the refinement writes qbuild: the scans always see the references as chosen
  sa.sr = S.sr;
  sa.Eref = A.Eref;
  if (A.n_chunks > 0) {
    // Frames arriving in chunks.  With spec_build, the passes after the scan
    // run speculatively for one reference as the chunks land: once the first
    // kSample frames are scanned, reference 0 is refined to their mean and
    // the operands of every scanned chunk are built.  If all frames turn out
    // within tau of reference 0, that is the final state; otherwise the
    // unrefined reference 0 is restored and the general path below runs.
    const int64_t nsample = std::min<int64_t>(F, (int64_t)kSample);
    BuildArgs bspec{};
    if (A.spec_build) bspec = build_args(*A.spec_build, A, S);
    bool refined = false;
    int64_t f0 = 0;
    for (int c = 0; c < A.n_chunks; ++c) {
      if (A.chunk_copy) (*A.chunk_copy)(c);  // (chunk 0: already issued, a no-op)
      if (c > 0) cudaStreamWaitEvent(st, A.chunk_ev[c], 0);
      const int64_t f1 = A.chunk_end[c];
      if (f1 > f0) {
        k_scan<T, true><<<prep_grid(f1 - f0, kScanBlocksPerSM, kFPB), kPrepThreads, 0, st>>>(src, f0, f1, sa);
        ++launches;
        if (A.spec_build && A.spec_fail && A.max_refs > 1 && F > 1) {
          k_spec_check<<<1, 256, 0, st>>>(A.dist, f0, f1, (float)A.tau, A.spec_fail);
          ++launches;
        }
        if (A.spec_build) {
          const int64_t b0 = refined ? f0 : 0;
          if (refined || f1 >= nsample) {
            k_rot<<<rot_grid(f1 - b0), kRotThreads, 0, st>>>(b0, f1, S.quat, A.cen, A.nofit, S.ftab, A.rot);
            ++launches;
          }
          if (!refined && f1 >= nsample) {
            launches += refine(1, nullptr, nullptr, nullptr, nullptr);
            refined = true;
          }
          if (refined) {
            launch_build<T>(b0, f1, src, bspec, st);
            ++launches;
            if (A.on_built) {
              const cudaError_t e = (*A.on_built)(f1);
              if (e != cudaSuccess) return e;
            }
          }
        }
      }
      f0 = f1;
    }
    if (A.spec_build && refined) {
      k_argmax<<<1, 1024, 0, st>>>(A.dist, F, A.dmax, A.fsel);
      ++launches;
      float dmax = 0.0f;
      cudaMemcpyAsync(&dmax, A.dmax, sizeof(float), cudaMemcpyDeviceToHost, st);
      cudaError_t e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) return e;
      if (!(dmax > A.tau) || A.max_refs == 1 || F <= 1) {
        o.K = 1;
        o.built = 1;
        o.launches = launches;
        return cudaGetLastError();
      }
      // More references are needed: rebuild the unrefined reference 0 the
      // k-centre choice below starts from (the scan results stand).
      cudaMemsetAsync(A.fsel, 0, sizeof(int64_t), st);
      k_make_ref<T><<<kRefCluster, kOneBlockThreads, 0, st>>>(src, A.fsel, A.cen, A.cmass_ref, A.cmass_tgt, A.w,
                                                              A.sqw, A.assign, 0, 0, A.nofit, A.refs, A.swr,
                                                              S.refhl, A.Eref, S.sr, S.rmax, S.qscan);
      ++launches;
    }
  } else if (!A.resume_scan) {
    k_scan<T, true><<<prep_grid(F, kScanBlocksPerSM, kFPB), kPrepThreads, 0, st>>>(src, 0, F, sa);
    ++launches;
  }
  // Greedy k-centre: add the farthest frame as a reference while it is
  // farther than tau from every reference.  The first round is decided on
  // the host (one reference is the common case and then costs no further
  // launch); once a second reference is needed, the remaining rounds are
  // queued at once, each gated on the device by the round before
  // (k_argmax_gate), so adding references costs no host round trip each.
  int K = 1;
  const int* skip = nullptr;
  if (K < A.max_refs && F > 1 && A.defer_multi && A.n_chunks == 0) {
    // The decision stays on the device: the passes below assume one
    // reference and return at once if the flag says otherwise.
    k_argmax<<<1, 1024, 0, st>>>(A.dist, F, A.dmax, A.fsel, (float)A.tau, A.defer_multi);
    ++launches;
    skip = A.defer_multi;
    o.deferred = 1;
  } else if (K < A.max_refs && F > 1) {
    k_argmax<<<1, 1024, 0, st>>>(A.dist, F, A.dmax, A.fsel);
    ++launches;
    float dmax = 0.0f;
    cudaMemcpyAsync(&dmax, A.dmax, sizeof(float), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    if (dmax > A.tau) {
      // state = {stopped, index of the last reference added}; round 1
      // repeats the host's check, which passed
      cudaMemsetAsync(S.kstate, 0, 2 * sizeof(int), st);
      for (int k = 1; k < A.max_refs; ++k) {
        k_argmax_gate<<<1, 1024, 0, st>>>(A.dist, F, (float)A.tau, k, A.dmax, A.fsel, S.kstate);
        ++launches;
        // (no-fit distances are not the fitted ones the pruning bound uses:
        // every frame is fitted then)
        float* dref = A.nofit ? nullptr : S.dref;
        k_make_ref<T><<<kRefCluster, kOneBlockThreads, 0, st>>>(src, A.fsel, A.cen, A.cmass_ref, A.cmass_tgt, A.w,
                                                                A.sqw, A.assign, k, 1, A.nofit, A.refs, A.swr,
                                                                S.refhl, A.Eref, S.sr, S.rmax, S.qscan, S.kstate,
                                                                WeightsPass{}, S.quat, dref, A.Wsum);
        ScanArgs sk = sa;
        sk.k = k;
        sk.q = S.qscan + (size_t)k * N;
        sk.sr = S.sr + 3 * k;
        sk.Eref = A.Eref + k;
        sk.gate = S.kstate;
        sk.dref = dref;
        sk.margin = 0.25f;
        k_scan<T, false><<<prep_grid(F, kScanBlocksPerSM, kFPB), kPrepThreads, 0, st>>>(src, 0, F, sk);
        launches += 2;
      }
      int kst[2] = {0, 0};
      cudaMemcpyAsync(kst, S.kstate, sizeof kst, cudaMemcpyDeviceToHost, st);
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
      K = kst[1] + 1;
    }
  }
  o.K = K;
  k_rot<<<rot_grid(F), kRotThreads, 0, st>>>(0, F, S.quat, A.cen, A.nofit, S.ftab, A.rot, skip);
  ++launches;
  // Frames grouped by reference (host counting sort) when there are several.
  const int* order = nullptr;
  const int* offsets = nullptr;
  if (K > 1) {
    std::vector<int> asg(F), ord(F), offs(K + 1, 0);
    cudaMemcpyAsync(asg.data(), A.assign, sizeof(int) * F, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    for (int64_t f = 0; f < F; ++f) offs[asg[f] + 1]++;
    for (int k = 0; k < K; ++k) offs[k + 1] += offs[k];
    std::vector<int> fill(offs.begin(), offs.end() - 1);
    for (int64_t f = 0; f < F; ++f) ord[fill[asg[f]]++] = (int)f;
    cudaMemcpyAsync(A.order, ord.data(), sizeof(int) * F, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(A.offsets, offs.data(), sizeof(int) * (K + 1), cudaMemcpyHostToDevice, st);
    std::vector<int> pos;
    if (A.sort_frames) {
      pos.resize(F);
      for (int64_t p = 0; p < F; ++p) pos[ord[p]] = (int)p;
      cudaMemcpyAsync(S.pos, pos.data(), sizeof(int) * F, cudaMemcpyHostToDevice, st);
      o.sorted = 1;
    }
    // the copies read host vectors that go out of scope: finish them here
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    order = A.order;
    offsets = A.offsets;
  }
  // One reference: the refinement also writes its terms with itself.
  float* RP = (K == 1) ? A.RP : nullptr;
  launches += refine(K, order, offsets, RP, skip);
  o.self_terms = (RP != nullptr);
  o.launches = launches;
  return cudaGetLastError();
}

cudaError_t run_prep(const PrepArgs& A, PrepOut& o, cudaStream_t st) {
  return A.dtype_f64 ? prep_impl<double>(A, o, st) : prep_impl<float>(A, o, st);
}

static BuildArgs build_args(const FinishArgs& fa, const PrepArgs& A, const PrepScratch& S) {
  BuildArgs b{};
  b.ftab = S.ftab;
  b.assign = A.assign;
  b.ymax = S.ymax;
  b.rmax = S.rmax;
  b.scal = S.scal;
  b.swr = A.swr;
  b.q = S.qbuild;
  b.K = fa.K;
  b.K_build = (fa.K > 1) ? 1 : fa.K;  // P against references 1..K-1 in k_pref
  b.Np = A.Np;
  b.tc = fa.tc;
  b.hi = (__half*)fa.hi;
  b.lo = (__half*)fa.lo;
  b.inv_scale = fa.inv_scale;
  b.write_plane = fa.write_plane || !fa.tc;
  b.plane = fa.plane;
  b.nrm = fa.nrm;
  b.P = fa.P;
  b.trP = fa.trP;
  b.pos = fa.sorted ? S.pos : nullptr;
  b.assign_pos = S.assign_pos;
  b.skip = fa.skip;
  return b;
}

template <typename T>
static cudaError_t finish_impl(const FinishArgs& fa, cudaStream_t st) {
  const PrepArgs& A = *fa.prep;
  FrameSrc<T> src{(const T*)A.ref, (const T*)(A.tgt ? A.tgt : A.ref), A.n_ref, A.N};
  const PrepScratch S = prep_carve(A.scratch, A.F, A.N, A.max_refs);
  if (!fa.built) {
    const BuildArgs b = build_args(fa, A, S);
    launch_build<T>(0, A.F, src, b, st);
    if (fa.K > 1) {
      if (3 * (fa.K - 1) > 32 * kPrefComb) return cudaErrorInvalidValue;
      const size_t sm = pref_smem_bytes(fa.K);
      const int64_t groups = (A.F + 8 * kPrefFpw - 1) / (8 * kPrefFpw);
      const unsigned grid = (unsigned)std::min<int64_t>(groups, 152 * 4);
      auto launch = [&](auto kern) -> cudaError_t {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        kern<<<grid, 256, sm, st>>>(b, A.F, A.N);
        return cudaGetLastError();
      };
      const int nc = (3 * (fa.K - 1) + 31) / 32;
      cudaError_t e = (nc <= 1)   ? launch(k_pref<1>)
                      : (nc == 2) ? launch(k_pref<2>)
                      : (nc == 3) ? launch(k_pref<3>)
                      : (nc == 4) ? launch(k_pref<4>)
                      : (nc == 5) ? launch(k_pref<5>)
                                  : launch(k_pref<6>);
      if (e != cudaSuccess) return e;
    }
  }
  if (!(fa.self_terms && fa.K == 1))
    k_ref_terms<<<fa.K * fa.K, kRefTermThreads, 0, st>>>(A.refs, A.N, fa.K, A.w, A.nofit, fa.RP, fa.skip);
  return cudaGetLastError();
}

cudaError_t run_finish(const FinishArgs& A, cudaStream_t st) {
  return A.prep->dtype_f64 ? finish_impl<double>(A, st) : finish_impl<float>(A, st);
}

}  // namespace gbr
