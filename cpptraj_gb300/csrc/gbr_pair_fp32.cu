// gbr_pair_fp32.cu -- the plain FP32 CUDA-core all-pairs kernel (K3).
//
// Replaces the nested pair loop of Analysis_Rms2d::Calculate_2D
// (src/Analysis_Rms2d.cpp:252-286) and MetricArray::calcFrameDistances
// (src/Cluster/MetricArray.cpp:786-793).  A CTA owns a 64 x 64 tile of
// (reference frame, target frame) pairs.  Each of its 256 threads accumulates
// the 3x3 residual contraction D_ji = sum_a p_j[a] p_i[a]^T for 4 x 4 pairs
// in FP32 registers (144 accumulators) while cp.async double-buffers
// 32-atom slabs of the FP32 operand planes through shared memory.  The
// accumulators are then parked in shared memory and the pair epilogue
// (gbr_common.cuh) runs one pair per thread with coalesced stores straight
// into the caller's TRI / FULL matrix.
#include "gbr_common.cuh"
#include "gbr_internal.h"

namespace gbr {

namespace {
constexpr int BM = 64;        // reference frames per tile
constexpr int BN = 64;        // target frames per tile
constexpr int KC = 32;        // atoms per pipeline stage
constexpr int KCP = KC + 2;   // padded row (8-byte aligned, conflict-free LDS.64)
constexpr int THREADS = 256;
constexpr int STAGE_FLOATS = 3 * BM * KCP + 3 * BN * KCP;
constexpr int PIPE_BYTES = 2 * STAGE_FLOATS * 4;
constexpr int EPI_BYTES = BM * BN * 9 * 4;
constexpr int SMEM_BYTES = PIPE_BYTES > EPI_BYTES ? PIPE_BYTES : EPI_BYTES;

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? 8 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// Load one 32-atom slab of 64 frames x 3 components into [3][64][KCP].
__device__ __forceinline__ void load_slab(float* dst, const float* plane, int64_t f0, int64_t f_end, int Np,
                                          int k0, int tid) {
#pragma unroll
  for (int it = 0; it < (BM * 3 * KC / 2) / THREADS; ++it) {
    const int c = tid + it * THREADS;   // 8-byte chunk index
    const int row = c / (KC / 2);       // 0..191 = f_local*3 + p
    const int cc = c % (KC / 2);
    const int fl = row / 3, p = row % 3;
    const int64_t f = f0 + fl;
    const bool ok = f < f_end;
    const float* src = plane + ((size_t)(ok ? f : f0) * 3 + p) * Np + k0 + 2 * cc;
    cp_async8(dst + (p * BM + fl) * KCP + 2 * cc, src, ok);
  }
}

template <bool BWD>
__global__ void __launch_bounds__(THREADS, 1) k_pairs_fp32(PairLaunch L) {
  if (L.skip && *L.skip != 0) return;  // uniform over the grid: before any barrier
  extern __shared__ __align__(16) float smem[];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;

  // Tile coordinates.
  const TileSpace& T = L.tiles;
  int64_t ti, tj;
  const int64_t l = blockIdx.x;
  if (T.tri) {
    const double b = 2.0 * (double)T.tj + 1.0;
    int64_t t = (int64_t)((b - sqrt(b * b - 8.0 * (double)l)) * 0.5);
    auto cum = [&](int64_t x) { return x * T.tj - x * (x - 1) / 2; };
    while (t > 0 && cum(t) > l) --t;
    while (cum(t + 1) <= l) ++t;
    ti = t;
    tj = ti + (l - cum(t));
  } else {
    ti = l % T.ti;
    tj = l / T.ti;
  }
  const int64_t i0 = T.i0 + ti * BM;       // reference frames (set index == ref index)
  const int64_t jt0 = T.j0 + tj * BN;      // target frames
  const int64_t i_end = T.i0 + T.ni;
  const int64_t jt_end = T.j0 + T.nj;
  const int64_t jset0 = L.tgt0 + jt0;
  const int64_t jset_end = L.tgt0 + jt_end;

  float acc[4][4][9];
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int n = 0; n < 4; ++n)
#pragma unroll
      for (int c = 0; c < 9; ++c) acc[m][n][c] = 0.f;

  const int nk = (L.N + KC - 1) / KC;
  float* stA[2] = {smem, smem + STAGE_FLOATS};
  load_slab(stA[0], L.plane, i0, i_end, L.Np, 0, tid);
  load_slab(stA[0] + 3 * BM * KCP, L.plane, jset0, jset_end, L.Np, 0, tid);
  cp_async_commit();
  for (int kt = 0; kt < nk; ++kt) {
    if (kt + 1 < nk) {
      float* nxt = stA[(kt + 1) & 1];
      load_slab(nxt, L.plane, i0, i_end, L.Np, (kt + 1) * KC, tid);
      load_slab(nxt + 3 * BM * KCP, L.plane, jset0, jset_end, L.Np, (kt + 1) * KC, tid);
      cp_async_commit();
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const float* As = stA[kt & 1];
    const float* Bs = As + 3 * BM * KCP;
#pragma unroll 1
    for (int k = 0; k < KC; k += 2) {
      float2 a[4][3];
#pragma unroll
      for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int pi = 0; pi < 3; ++pi)
          a[m][pi] = *reinterpret_cast<const float2*>(As + (pi * BM + ty + 16 * m) * KCP + k);
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        float2 b[3];
#pragma unroll
        for (int pj = 0; pj < 3; ++pj)
          b[pj] = *reinterpret_cast<const float2*>(Bs + (pj * BN + tx + 16 * n) * KCP + k);
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
          for (int pj = 0; pj < 3; ++pj)
#pragma unroll
            for (int pi = 0; pi < 3; ++pi) {
              float s = acc[m][n][pj * 3 + pi];
              s = fmaf(a[m][pi].x, b[pj].x, s);
              s = fmaf(a[m][pi].y, b[pj].y, s);
              acc[m][n][pj * 3 + pi] = s;
            }
      }
    }
    __syncthreads();
  }

  // Park the accumulators; layout keeps the epilogue's reads conflict-free.
  const bool tri = L.map.tri;
  float* Ds = smem;
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      const int il = ty + 16 * m, jl = tx + 16 * n;
      const int slot = tri ? (il * BN + jl) : (jl * BM + il);
#pragma unroll
      for (int c = 0; c < 9; ++c) Ds[slot * 9 + c] = acc[m][n][c];
    }
  __syncthreads();

  if constexpr (!BWD) {
#pragma unroll 1
    for (int r = 0; r < (BM * BN) / THREADS; ++r) {
      const int fast = tid & 63, slow = (tid >> 6) + 4 * r;
      const int il = tri ? slow : fast, jl = tri ? fast : slow;
      const int64_t i = i0 + il, jt = jt0 + jl;
      if (i >= i_end || jt >= jt_end) continue;
      const int64_t idx = out_index(L.map, i, jt);
      if (idx < 0) continue;
      const int slot = tri ? (il * BN + jl) : (jl * BM + il);
      float D[9];
#pragma unroll
      for (int c = 0; c < 9; ++c) D[c] = Ds[slot * 9 + c];
      bool flag = false;
      const float rm = pair_epilogue(D, i, L.tgt0 + jt, L.terms, &flag);
      if (flag) flag_pair(L.flags, L.map, i, jt);
      L.map.out[idx] = rm;
    }
  } else {
    // Backward epilogue (one frame set, TRI).  For pair (i < j) with weight
    // c = g_ij / RMSD_ij and T = rotation taking x'_j onto x'_i:
    //   B[3i+p][3j+q] = c T[p][q]   (the lower block is added by transposition later)
    //   E_i += c (I - T),  E_j += c (I - T^T),  C_i += c,  C_j += c.
    // I - T comes straight from the quaternion, so it is accurate when T ~ I.
    __shared__ float Erow[BM][10], Ecol[BN][10];
    for (int k = tid; k < BM * 10; k += THREADS) (&Erow[0][0])[k] = 0.f;
    for (int k = tid; k < BN * 10; k += THREADS) (&Ecol[0][0])[k] = 0.f;
    __syncthreads();
    const BwdArgs& bw = L.bwd;
    // The 32 lanes of a warp share the reference row il (64 consecutive
    // threads per row): its E/C terms are summed across the warp before one
    // shared-memory atomic per value; each lane's column jl is its own.
#pragma unroll 1
    for (int r = 0; r < (BM * BN) / THREADS; ++r) {
      const int jl = tid & 63, il = (tid >> 6) + 4 * r;
      const int64_t i = i0 + il, j = jt0 + jl;
      float er[10];
#pragma unroll
      for (int k = 0; k < 10; ++k) er[k] = 0.f;
      const bool live = i < i_end && j < jt_end && j > i;
      if (live) {
        const int slot = il * BN + jl;
        float D[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) D[c] = Ds[slot * 9 + c];
        bool flag = false;
        float q[4];
        const float rm = pair_epilogue(D, i, j, L.terms, &flag, q);
        const int64_t t = tri_index(L.map.n_ref, i, j);
        if (bw.rmsd) bw.rmsd[t] = rm;
        const float gij = bw.g ? bw.g[t] : 1.0f;
        const float c = (rm > 1e-6f) ? gij / rm : 0.0f;
        const float a = q[0], x = q[1], y = q[2], z = q[3];
        // QCP rotation R(q) (row-major); T = R^T.
        const float R0 = a * a + x * x - y * y - z * z, R1 = 2.f * (x * y + a * z), R2 = 2.f * (z * x - a * y);
        const float R3 = 2.f * (x * y - a * z), R4 = a * a - x * x + y * y - z * z, R5 = 2.f * (y * z + a * x);
        const float R6 = 2.f * (z * x + a * y), R7 = 2.f * (y * z - a * x), R8 = a * a - x * x - y * y + z * z;
        float* Bi = bw.B + (size_t)(3 * i) * bw.ldB + 3 * j;
        Bi[0] = c * R0; Bi[1] = c * R3; Bi[2] = c * R6;
        Bi += bw.ldB;
        Bi[0] = c * R1; Bi[1] = c * R4; Bi[2] = c * R7;
        Bi += bw.ldB;
        Bi[0] = c * R2; Bi[1] = c * R5; Bi[2] = c * R8;
        const float d00 = 2.f * (y * y + z * z), d11 = 2.f * (x * x + z * z), d22 = 2.f * (x * x + y * y);
        // E_i += c (I - R^T);  E_j += c (I - R)
        er[0] = c * d00; er[1] = -c * R3; er[2] = -c * R6;
        er[3] = -c * R1; er[4] = c * d11; er[5] = -c * R7;
        er[6] = -c * R2; er[7] = -c * R5; er[8] = c * d22;
        er[9] = c;
        atomicAdd(&Ecol[jl][0], c * d00); atomicAdd(&Ecol[jl][1], -c * R1); atomicAdd(&Ecol[jl][2], -c * R2);
        atomicAdd(&Ecol[jl][3], -c * R3); atomicAdd(&Ecol[jl][4], c * d11); atomicAdd(&Ecol[jl][5], -c * R5);
        atomicAdd(&Ecol[jl][6], -c * R6); atomicAdd(&Ecol[jl][7], -c * R7); atomicAdd(&Ecol[jl][8], c * d22);
        atomicAdd(&Ecol[jl][9], c);
      }
#pragma unroll
      for (int k = 0; k < 10; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) er[k] += __shfl_xor_sync(0xffffffffu, er[k], o);
      if ((tid & 31) == 0)
#pragma unroll
        for (int k = 0; k < 10; ++k)
          if (er[k] != 0.f) atomicAdd(&Erow[il][k], er[k]);
    }
    __syncthreads();
    for (int k = tid; k < BM * 10; k += THREADS) {
      const int fl = k / 10, e = k % 10;
      const int64_t f = i0 + fl;
      const float v = Erow[fl][e];
      if (f < i_end && v != 0.f) atomicAdd(e < 9 ? &bw.E[f * 9 + e] : &bw.C[f], v);
    }
    for (int k = tid; k < BN * 10; k += THREADS) {
      const int fl = k / 10, e = k % 10;
      const int64_t f = jt0 + fl;
      const float v = Ecol[fl][e];
      if (f < jt_end && v != 0.f) atomicAdd(e < 9 ? &bw.E[f * 9 + e] : &bw.C[f], v);
    }
  }
}
}  // namespace

TileSpace make_tiles(const OutMap& m, int bm, int bn) {
  TileSpace t{};
  t.tri = m.tri;
  if (m.tri) {
    t.i0 = m.row_begin;
    t.ni = m.row_end - m.row_begin;
    t.j0 = m.row_begin;
    t.nj = m.n_tgt - m.row_begin;
  } else {
    t.i0 = 0;
    t.ni = m.n_ref;
    t.j0 = m.row_begin;
    t.nj = m.row_end - m.row_begin;
  }
  t.ti = (t.ni + bm - 1) / bm;
  t.tj = (t.nj + bn - 1) / bn;
  if (t.ni <= 0 || t.nj <= 0) {
    t.count = 0;
  } else if (m.tri) {
    // bm == bn: tiles (ti, tj) with tj >= ti.
    t.count = t.ti * t.tj - t.ti * (t.ti - 1) / 2;
  } else {
    t.count = t.ti * t.tj;
  }
  return t;
}

cudaError_t run_pairs_fp32(const PairLaunch& L, cudaStream_t st) {
  if (L.tiles.count == 0) return cudaSuccess;
  cudaError_t e;
  if (L.bwd.B) {
    e = cudaFuncSetAttribute(k_pairs_fp32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    k_pairs_fp32<true><<<(unsigned)L.tiles.count, THREADS, SMEM_BYTES, st>>>(L);
  } else {
    e = cudaFuncSetAttribute(k_pairs_fp32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    k_pairs_fp32<false><<<(unsigned)L.tiles.count, THREADS, SMEM_BYTES, st>>>(L);
  }
  return cudaGetLastError();
}

}  // namespace gbr
