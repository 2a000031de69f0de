// gbr_dme.cu -- all-pairs distance RMSD, the `dme` mode of rms2d (K5).
//
// Replaces, for Analysis_Rms2d's DME mode, the pair loop of
// Analysis_Rms2d::Calculate_2D (src/Analysis_Rms2d.cpp:247-290) around
// Frame::DISTRMSD (src/Frame.cpp:1313-1344):
//     DME(ref, tgt) = sqrt( sum_{a<b} (|t_a - t_b| - |r_a - r_b|)^2 / Nd ),
//     Nd = (N^2 - N) / 2,
// with no masses and no centring of the reference (Calculate_2D centres it
// for fit and qrmsd only, :265-266).  N = 1 gives 0/0 = NaN, as there.
//
// Scheme.  For every frame the Nd intra-frame distances form a vector d_f;
// DME^2 * Nd = |d_i - d_j|^2 is a squared Euclidean distance between such
// vectors, i.e. a GEMM-shaped contraction over atom pairs.  It is evaluated
// directly -- sum of (d_i[k] - d_j[k])^2, each difference of two nearby
// values exact or nearly so -- instead of through |d_i|^2 + |d_j|^2 - 2 d_i.d_j,
// which cancels for similar frames.  Two kernels per chunk of atom pairs:
//   k_dme_dist   distance planes D[k][f] (frames contiguous per atom pair k,
//                FP32; the target set's frames in their own 64-aligned block)
//   k_dme_pairs  128 x 64 frame tiles on the CUDA cores, 8 x 4 pairs per
//                thread (64 x 64 and 4 x 4 for FP64 planes); slabs of 32
//                atom pairs staged in shared memory;
//                each slab's 32-term FP32 sum folded into a TwoSum-compensated
//                (hi, lo) accumulator, so the result is as accurate as FP64
//                accumulation of FP32-rounded distances.
// Atom pairs are processed in chunks that bound the planes (2 GB), and a
// chunk's atom pairs are split over `splits` CTAs per tile when there are
// few tiles; every (split, pair) slot is owned by one CTA, and k_dme_final
// adds the splits in a fixed order (deterministic) and takes sqrt(sum/Nd) in
// FP64.  GBR_PREC_FP64 runs the same kernels with FP64 planes and sums.
#include <cmath>
#include <vector>

#include "../../include/gbrmsd.h"
#include "gbr_common.cuh"
#include "gbr_handle.h"
#include "gbr_internal.h"

namespace gbr {
namespace {

constexpr int kDT = 64;         // target frames per tile (tile columns)
constexpr int kDKS = 32;        // atom pairs per shared-memory slab
constexpr int kDThreads = 256;  // 16 x 16 threads, MR x 4 pairs each
// Reference frames per tile (tile rows): 16 MR, MR = 8 for FP32 planes (32
// pair terms per three 16-byte shared-memory loads), 4 for FP64 planes.
template <typename P>
constexpr int dme_rows() {
  return sizeof(P) == 4 ? 128 : 64;
}
constexpr int kDistFrames = 128;
constexpr size_t kPlaneBudget = size_t(2) << 30;

// Set frame -> column of the distance planes.
struct DmeCols {
  int64_t n_ref, ref_cols;  // target frame jt sits in column ref_cols + jt
};

// Largest a with a*N - a(a+1)/2 <= k, i.e. the row of atom pair k in the
// (a outer, b inner) order; b from the remainder.
__device__ __forceinline__ void pair_of(int64_t k, int N, int& a, int& b) {
  const double m = 2.0 * N - 1.0;
  int64_t aa = (int64_t)floor((m - sqrt(fmax(m * m - 8.0 * (double)k, 0.0))) * 0.5);
  auto start = [&](int64_t r) { return r * N - r * (r + 1) / 2; };
  if (aa < 0) aa = 0;
  while (aa > 0 && start(aa) > k) --aa;
  while (start(aa + 1) <= k) ++aa;
  a = (int)aa;
  b = (int)(k - start(aa) + aa + 1);
}

template <typename T, typename P>
__device__ __forceinline__ P dist(const T* x, int a, int b) {
  if constexpr (sizeof(P) == 8) {
    const double dx = (double)x[3 * a] - (double)x[3 * b], dy = (double)x[3 * a + 1] - (double)x[3 * b + 1],
                 dz = (double)x[3 * a + 2] - (double)x[3 * b + 2];
    return sqrt(dx * dx + dy * dy + dz * dz);
  } else {
    // Each coordinate difference is rounded once (relative error 2^-24 of the
    // difference itself): the FP32 subtraction of FP32 input, or the FP64
    // difference of FP64 input rounded to FP32.
    float dx, dy, dz;
    if constexpr (sizeof(T) == 4) {
      dx = x[3 * a] - x[3 * b]; dy = x[3 * a + 1] - x[3 * b + 1]; dz = x[3 * a + 2] - x[3 * b + 2];
    } else {
      dx = (float)(x[3 * a] - x[3 * b]); dy = (float)(x[3 * a + 1] - x[3 * b + 1]);
      dz = (float)(x[3 * a + 2] - x[3 * b + 2]);
    }
    return sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
  }
}

// D[(k - k0) * Dstride + c] = |x_f[a] - x_f[b]| for atom pairs k in
// [k0, k0 + nk) and plane columns c (frame f = the column's frame); zero for
// padding columns.  grid.x: groups of kDKS atom pairs (a block walks its
// pairs in order from one inverse); grid.y: groups of 128 columns, strided.
template <typename T, typename P>
__global__ void __launch_bounds__(kDistFrames) k_dme_dist(const T* ref, const T* tgt, int64_t n_ref, int64_t n_tgt,
                                                           int N, DmeCols cols, int64_t n_cols, int64_t k0, int64_t nk,
                                                           int64_t Dstride, P* D) {
  __shared__ int ab[2];
  const int64_t kg = k0 + (int64_t)blockIdx.x * kDKS;
  if (threadIdx.x == 0) pair_of(kg, N, ab[0], ab[1]);
  __syncthreads();
  const int64_t kend = min(kg + kDKS, k0 + nk);
  for (int64_t c = (int64_t)blockIdx.y * kDistFrames + threadIdx.x; c < n_cols;
       c += (int64_t)gridDim.y * kDistFrames) {
    const T* x = nullptr;  // the frame in this column, or none (padding)
    if (c < cols.ref_cols) {
      if (c < n_ref) x = ref + (size_t)c * 3 * N;
    } else {
      const int64_t jt = c - cols.ref_cols;
      if (jt < n_tgt) x = tgt + (size_t)jt * 3 * N;
    }
    int a = ab[0], b = ab[1];
    for (int64_t k = kg; k < kend; ++k) {
      D[(size_t)(k - k0) * Dstride + c] = x ? dist<T, P>(x, a, b) : P(0);
      if (++b == N) {
        ++a;
        b = a + 1;
      }
    }
  }
}

// Four consecutive plane values (16-byte aligned for FP32, 32 for FP64).
__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&v)[4]) {
  const double2 t0 = *reinterpret_cast<const double2*>(p), t1 = *reinterpret_cast<const double2*>(p + 2);
  v[0] = t0.x; v[1] = t0.y; v[2] = t1.x; v[3] = t1.y;
}
__device__ __forceinline__ void st4(float* p, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double* p, const double (&v)[4]) {
  *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
  *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
}

__device__ __forceinline__ void two_sum_acc(float& s, float& c, float v) {
  const float t = s + v;
  const float bb = t - s;
  c += (s - (t - bb)) + (v - bb);
  s = t;
}

// Tiles (ti, tj): reference frames i0 = ti*TR .. +TR (TR = dme_rows<P>()),
// target frames j0 = tj*64 .. +64.  grid (n_tiles, splits).
// part[(split * n_out + idx)] accumulates this chunk's sum for output element
// idx: (hi, lo) for FP32, (sum, unused) for FP64.
template <typename P>
__global__ void __launch_bounds__(kDThreads, 2)
    k_dme_pairs(const P* __restrict__ D, int64_t Dstride, int64_t nk, int64_t tgt_col0, const int2* __restrict__ tiles,
                OutMap map, int64_t n_out, P* __restrict__ part, int first_chunk) {
  // Thread (ty, tx) owns rows g * 64 + ty * 4 + (0..3) for each 64-row group
  // g of the tile (MR / 4 groups) and columns tx * 4 + (0..3).
  constexpr int TR = dme_rows<P>(), MR = TR / 16;
  __shared__ __align__(16) P As[kDKS][TR];
  __shared__ __align__(16) P Bs[kDKS][kDT];
  const int2 tl = tiles[blockIdx.x];
  const int64_t i0 = (int64_t)tl.x * TR, j0 = (int64_t)tl.y * kDT;
  const int split = blockIdx.y, splits = gridDim.y;
  const int64_t nslab = (nk + kDKS - 1) / kDKS;
  const int64_t s_begin = nslab * split / splits, s_end = nslab * (split + 1) / splits;
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  P sh[MR][4], sl[MR][4];
#pragma unroll
  for (int m = 0; m < MR; ++m)
#pragma unroll
    for (int n = 0; n < 4; ++n) sh[m][n] = sl[m][n] = P(0);
  // staging: A slab kDKS x TR (TR/4 float4 per row), B slab kDKS x 64
  constexpr int AV = TR / 4;                    // 4-wide vectors per A row
  constexpr int AH = kDKS * AV / kDThreads;     // A vectors per thread
  const int lr = tid >> 4, lc = (tid & 15) * 4;  // B: slab rows lr, lr + 16; columns lc..lc+3
  for (int64_t sl_i = s_begin; sl_i < s_end; ++sl_i) {
    const int64_t kb = sl_i * kDKS;
#pragma unroll
    for (int h = 0; h < AH; ++h) {
      const int v = tid + kDThreads * h, r = v / AV, cc = (v % AV) * 4;
      P va[4] = {P(0), P(0), P(0), P(0)};
      if (kb + r < nk) ld4(D + (size_t)(kb + r) * Dstride + i0 + cc, va);
      st4(&As[r][cc], va);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = lr + 16 * h;
      P vb[4] = {P(0), P(0), P(0), P(0)};
      if (kb + r < nk) ld4(D + (size_t)(kb + r) * Dstride + tgt_col0 + j0 + lc, vb);
      st4(&Bs[r][lc], vb);
    }
    __syncthreads();
    P acc[MR][4];
#pragma unroll
    for (int m = 0; m < MR; ++m)
#pragma unroll
      for (int n = 0; n < 4; ++n) acc[m][n] = P(0);
#pragma unroll 8
    for (int kk = 0; kk < kDKS; ++kk) {
      P av[MR], bv[4];
#pragma unroll
      for (int hh = 0; hh < MR / 4; ++hh) {
        P a4[4];
        ld4(&As[kk][hh * 64 + ty * 4], a4);
#pragma unroll
        for (int t = 0; t < 4; ++t) av[4 * hh + t] = a4[t];
      }
      ld4(&Bs[kk][tx * 4], bv);
#pragma unroll
      for (int m = 0; m < MR; ++m)
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          const P d = av[m] - bv[n];
          acc[m][n] = fma(d, d, acc[m][n]);
        }
    }
#pragma unroll
    for (int m = 0; m < MR; ++m)
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        if constexpr (sizeof(P) == 4)
          two_sum_acc(sh[m][n], sl[m][n], acc[m][n]);
        else
          sh[m][n] += acc[m][n];
      }
    __syncthreads();
  }
  P* pbase = part + (size_t)split * n_out * 2;
#pragma unroll
  for (int m = 0; m < MR; ++m)
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      const int64_t idx = out_index(map, i0 + (m / 4) * 64 + ty * 4 + (m % 4), j0 + tx * 4 + n);
      if (idx < 0) continue;
      P* q = pbase + 2 * idx;
      if (first_chunk) {
        q[0] = sh[m][n];
        q[1] = sl[m][n];
      } else if constexpr (sizeof(P) == 4) {
        float hi = q[0], lo = q[1];
        two_sum_acc(hi, lo, sh[m][n]);
        lo += sl[m][n];
        q[0] = hi;
        q[1] = lo;
      } else {
        q[0] += sh[m][n];
      }
    }
}

template <typename P>
__global__ void k_dme_final(const P* __restrict__ part, int64_t n_out, int splits, double nd, float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_out; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < splits; ++k) {
      const P* q = part + ((size_t)k * n_out + i) * 2;
      s += (double)q[0] + (double)q[1];
    }
    out[i] = (float)sqrt(s / nd);
  }
}

template <typename T, typename P>
cudaError_t dme_launch(const void* d_ref, const void* d_tgt, int64_t n_ref, int64_t n_tgt, int N, const OutMap& map,
                       int64_t n_out, void* Dbuf, int64_t Dstride, int64_t n_cols, DmeCols cols, int64_t tgt_col0,
                       int64_t kc,
                       const int2* tiles, int64_t n_tiles, int splits, void* part, float* out, cudaStream_t st,
                       int& launches) {
  const int64_t Nd = (int64_t)N * (N - 1) / 2;
  const T* ref = (const T*)d_ref;
  const T* tgt = (const T*)(d_tgt ? d_tgt : d_ref);
  P* D = (P*)Dbuf;
  P* pt = (P*)part;
  if (Nd == 0) {
    cudaMemsetAsync(pt, 0, sizeof(P) * 2 * (size_t)splits * n_out, st);
  }
  for (int64_t k0 = 0, c = 0; k0 < Nd; k0 += kc, ++c) {
    const int64_t nk = std::min<int64_t>(kc, Nd - k0);
    dim3 gd((unsigned)((nk + kDKS - 1) / kDKS),
            (unsigned)std::min<int64_t>((n_cols + kDistFrames - 1) / kDistFrames, 65535));
    k_dme_dist<T, P><<<gd, kDistFrames, 0, st>>>(ref, tgt, n_ref, d_tgt ? n_tgt : 0, N, cols, n_cols, k0, nk, Dstride,
                                                D);
    dim3 gp((unsigned)n_tiles, (unsigned)splits);
    k_dme_pairs<P><<<gp, kDThreads, 0, st>>>(D, Dstride, nk, tgt_col0, tiles, map, n_out, pt, c == 0);
    launches += 2;
  }
  const int grid = (int)std::min<int64_t>((n_out + 255) / 256, 152 * 8);
  k_dme_final<P><<<grid, 256, 0, st>>>(pt, n_out, splits, (double)((int64_t)N * N - N) / 2.0, out);
  ++launches;
  return cudaGetLastError();
}

}  // namespace

int allpairs_dme(gbr_handle* h, const void* ref_xyz, const void* tgt_xyz, int dtype, int64_t n_ref, int64_t n_tgt,
                 int N, int out_kind, int precision, float* out, int64_t row_begin, int64_t row_end, int64_t n_out) {
  cudaStream_t st = h->stream;
  const bool f64 = (precision == GBR_PREC_FP64);
  const size_t psz = f64 ? 8 : 4;
  const size_t esz = (dtype == GBR_F64) ? 8 : 4;
  const bool ref_dev = is_device_ptr(ref_xyz);
  const bool tgt_dev = tgt_xyz ? is_device_ptr(tgt_xyz) : ref_dev;
  const bool out_dev = is_device_ptr(out);

  OutMap map{};
  map.n_ref = n_ref;
  map.tgt0 = tgt_xyz ? n_ref : 0;
  map.n_tgt = n_tgt;
  map.tri = (out_kind == GBR_TRI);
  map.row_begin = row_begin;
  map.row_end = row_end;
  map.base = (map.tri && row_begin < n_ref - 1) ? tri_index(n_ref, row_begin, row_begin + 1) : 0;

  // Plane columns: reference frames [0, ref_cols), target frames after them
  // (FULL), each block padded to its tile size so every tile load is aligned.
  const int64_t TR = f64 ? dme_rows<double>() : dme_rows<float>();
  DmeCols cols{n_ref, (n_ref + TR - 1) / TR * TR};
  const int64_t tgt_cols = tgt_xyz ? (n_tgt + kDT - 1) / kDT * kDT : 0;
  const int64_t n_cols = cols.ref_cols + tgt_cols;
  const int64_t tgt_col0 = tgt_xyz ? cols.ref_cols : 0;

  // Tiles of TR reference x 64 target frames covering this call's rows.
  std::vector<int2> tiles;
  const int64_t nti = (n_ref + TR - 1) / TR, ntj = (n_tgt + kDT - 1) / kDT;
  if (map.tri) {
    // a tile holds a pair of the upper triangle once its last column passes its first row
    for (int64_t ti = row_begin / TR; ti < (row_end + TR - 1) / TR; ++ti)
      for (int64_t tj = (ti * TR) / kDT; tj < ntj; ++tj) tiles.push_back(make_int2((int)ti, (int)tj));
  } else {
    for (int64_t tj = row_begin / kDT; tj < (row_end + kDT - 1) / kDT; ++tj)
      for (int64_t ti = 0; ti < nti; ++ti) tiles.push_back(make_int2((int)ti, (int)tj));
  }
  const int64_t n_tiles = (int64_t)tiles.size();
  if (n_tiles > INT32_MAX) return h->fail(GBR_ERR_ARG, "too many frame tiles");

  const int64_t Nd = (int64_t)N * (N - 1) / 2;
  int64_t kc = (int64_t)(kPlaneBudget / ((size_t)n_cols * psz)) / kDKS * kDKS;
  kc = std::max<int64_t>(kDKS, std::min<int64_t>(kc, (Nd + kDKS - 1) / kDKS * kDKS));
  const int64_t nslab_chunk = (std::min<int64_t>(kc, std::max<int64_t>(Nd, 1)) + kDKS - 1) / kDKS;
  const int64_t want = 2LL * 2 * (h->num_sms > 0 ? h->num_sms : 152);
  int splits = (int)std::max<int64_t>(1, std::min<int64_t>({(want + n_tiles - 1) / n_tiles, 64, nslab_chunk}));
  // keep the partial sums within the same 2 GB budget when the output is large
  while (splits > 1 && (size_t)splits * n_out * 2 * psz > kPlaneBudget) --splits;

  auto layout = [&](Arena& A, void** p) {
    p[0] = ref_dev ? nullptr : A.take<char>(esz * 3 * (size_t)N * n_ref);
    p[1] = (tgt_xyz && !tgt_dev) ? A.take<char>(esz * 3 * (size_t)N * n_tgt) : nullptr;
    p[2] = A.take<char>(psz * (size_t)std::min<int64_t>(kc, std::max<int64_t>(Nd, 1)) * n_cols);  // planes
    p[3] = A.take<int2>(n_tiles);
    p[4] = A.take<char>(psz * 2 * (size_t)splits * n_out);  // partial sums
    p[5] = out_dev ? nullptr : A.take<float>(n_out);
  };
  void* P[6];
  Arena sizing;
  layout(sizing, P);
  if (!h->reserve(sizing.off + 256))
    return h->fail(GBR_ERR_NOMEM, "cannot allocate %.2f GB of device workspace", (sizing.off + 256) / 1e9);
  Arena A{h->ws, 0};
  layout(A, P);

  if (h->timing) cudaEventRecord(h->ev[0], st);
  if (!ref_dev) cudaMemcpyAsync(P[0], ref_xyz, esz * 3 * (size_t)N * n_ref, cudaMemcpyDefault, st);
  if (tgt_xyz && !tgt_dev) cudaMemcpyAsync(P[1], tgt_xyz, esz * 3 * (size_t)N * n_tgt, cudaMemcpyDefault, st);
  cudaMemcpyAsync(P[3], tiles.data(), sizeof(int2) * n_tiles, cudaMemcpyHostToDevice, st);
  const void* d_ref = ref_dev ? ref_xyz : P[0];
  const void* d_tgt = tgt_xyz ? (tgt_dev ? tgt_xyz : P[1]) : nullptr;
  float* d_out = out_dev ? out : (float*)P[5];
  if (h->timing) cudaEventRecord(h->ev[1], st);

  int launches = 0;
  cudaError_t e;
  const int64_t Dstride = n_cols;
  if (dtype == GBR_F64) {
    e = f64 ? dme_launch<double, double>(d_ref, d_tgt, n_ref, n_tgt, N, map, n_out, P[2], Dstride, n_cols, cols, tgt_col0, kc,
                                         (const int2*)P[3], n_tiles, splits, P[4], d_out, st, launches)
            : dme_launch<double, float>(d_ref, d_tgt, n_ref, n_tgt, N, map, n_out, P[2], Dstride, n_cols, cols, tgt_col0, kc,
                                        (const int2*)P[3], n_tiles, splits, P[4], d_out, st, launches);
  } else {
    e = f64 ? dme_launch<float, double>(d_ref, d_tgt, n_ref, n_tgt, N, map, n_out, P[2], Dstride, n_cols, cols, tgt_col0, kc,
                                        (const int2*)P[3], n_tiles, splits, P[4], d_out, st, launches)
            : dme_launch<float, float>(d_ref, d_tgt, n_ref, n_tgt, N, map, n_out, P[2], Dstride, n_cols, cols, tgt_col0, kc,
                                       (const int2*)P[3], n_tiles, splits, P[4], d_out, st, launches);
  }
  if (e != cudaSuccess) return h->cuda_fail(e, "dme kernels");
  if (h->timing) {
    cudaEventRecord(h->ev[2], st);
    cudaEventRecord(h->ev[3], st);
  }
  if (!out_dev) cudaMemcpyAsync(out, d_out, sizeof(float) * n_out, cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return h->cuda_fail(e, "dme");
  h->stats.pairs = n_out;
  h->stats.precision = f64 ? GBR_PREC_FP64 : GBR_PREC_FP32;
  h->stats.kernel_launches = launches;
  if (h->timing) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev[1], h->ev[2]);
    h->stats.ms_pairs = ms;
  }
  return GBR_OK;
}

}  // namespace gbr
