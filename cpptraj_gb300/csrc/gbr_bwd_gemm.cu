// gbr_bwd_gemm.cu -- the block contraction of the backward pass on the
// tensor cores (tcgen05, sm_103a).
//
// The backward (gbr_backward.cu) needs, for every frame f and atom a,
//   Z_f[a] = sum_h c_fh T_fh d_h[a],
// i.e. Z[3F][Np] = S[3F][3F] * plane[3F][Np], where S holds the 3x3 blocks
// c_fh T_fh of every pair (written once per pair by the backward pair kernel,
// upper blocks only; S = B + B^T) and plane = sqrt(w) d the residual
// operands.  The reference has no gradient; this is the contraction the
// analytic gradient of sum_{i<j} g_ij RMSD_ij reduces to.
//
// Precision.  S and plane are scaled by powers of two (largest magnitude
// just below 2^14) and split into FP16 hi + lo; hi*hi + lo*hi + hi*lo is
// accumulated in FP32 in tensor memory, which represents every product to
// ~2^-22 of the largest one (the FP32 level the strict-FP32 GEMM gave).
//
// Operands (both K-major, K = 3F):
//   A = planeT [Np][K]  (atoms x frame components), built by k_split_planeT;
//   B = S      [3F][K]  (S is symmetric: row n of S is column n),
//       built by k_split_sym.
// The MMA computes D[atoms][Z rows] = A * B^T; the epilogue warps hold one
// atom per TMEM lane, so the stores of one Z row (atoms contiguous) are
// coalesced.
//
// Kernel shape: one CTA per SM, persistent over tiles of 128 atoms x 256 Z
// rows; per stage 64 K (128-byte rows, 128-byte swizzle) of A hi/lo and
// B hi/lo (96 KB), two stages; two 256-column FP32 accumulators in tensor
// memory so the epilogue of one tile overlaps the MMAs of the next.  Tiles
// are ordered Z-row block first, so the CTAs in flight share their B rows in
// L2.  Every mbarrier wait is bounded (gbr_mbar.cuh).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <atomic>

#include "gbr_common.cuh"
#include "gbr_internal.h"
#include "gbr_mbar.cuh"

namespace gbr {

namespace {

constexpr int GM = 128;  // atoms per tile (MMA M)
constexpr int GN = 256;  // Z rows per tile (MMA N)
constexpr int GK = 64;   // K per stage
constexpr int GSTAGES = 2;
constexpr int GA_BYTES = GM * 2 * GK;  // 16 KB
constexpr int GB_BYTES = GN * 2 * GK;  // 32 KB
constexpr int GSTAGE_BYTES = 2 * GA_BYTES + 2 * GB_BYTES;
constexpr int GEPI_WARPS = 4;
constexpr int GTHREADS = 64 + 32 * GEPI_WARPS;
constexpr int GSMEM = 1024 + GSTAGES * GSTAGE_BYTES + 256;
static_assert(GSMEM <= 232448, "backward GEMM shared memory");
constexpr uint32_t GTMEM_COLS = 512;
constexpr uint32_t GACC_STRIDE = 256;
constexpr uint32_t GSBO = 8 * 2 * GK;  // 8-row core-matrix groups of 128-byte rows
// kind::f16 instruction descriptor: D = F32, A = B = F16, both K-major,
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t GIDESC = (1u << 4) | ((uint32_t)(GN >> 3) << 17) | ((uint32_t)(GM >> 4) << 24);
// Bounded-wait site codes of this kernel (the pair kernels use 1-5 and 11-13).
constexpr int kSiteProducer = 21, kSiteMmaAcc = 22, kSiteMmaFull = 23, kSiteEpi = 24;

struct GemmParams {
  int64_t n_mt;      // atom tiles
  int64_t n_tiles;   // atom tiles x Z-row tiles
  int nk;            // K stages
  int64_t rows;      // Z rows (3F)
  int Np;            // atoms per Z row (padded)
  float* Z;          // [rows][Np]
  const float* scl;  // [2]: 1/scale of S, 1/scale of the plane
  int* err;
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// UMMA shared-memory descriptor: K-major rows of 128 bytes with the 128-byte
// swizzle, 8-row groups GSBO bytes apart, version bits 46-48 = 0b001.
__device__ __forceinline__ uint64_t gdesc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(GSBO >> 4) << 32;
  d |= 1ull << 46;
  d |= 2ull << 61;
  return d;
}

__device__ __forceinline__ void gmma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(GIDESC), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void gcommit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void gfence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void gfence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void gtmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

__global__ void __launch_bounds__(GTHREADS, 1)
    k_bwd_gemm(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
               const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl,
               const GemmParams P) {
  extern __shared__ uint8_t gsmem_raw[];
  uint8_t* smem = gsmem_raw + ((1024u - (smem_addr(gsmem_raw) & 1023u)) & 1023u);
  uint64_t* bars = (uint64_t*)(smem + GSTAGES * GSTAGE_BYTES);
  // bars: full[2] empty[2] accfull[2] accempty[2] done[1]; then the TMEM address.
  uint32_t* tmem_slot = (uint32_t*)(bars + 10);
  const uint32_t full0 = smem_addr(bars + 0), empty0 = smem_addr(bars + 2), accf0 = smem_addr(bars + 4),
                 acce0 = smem_addr(bars + 6), done = smem_addr(bars + 8);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < GSTAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf0 + 8 * b, 1);
      mbar_init(acce0 + 8 * b, GEPI_WARPS);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmAh) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmAl) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmBh) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmBl) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(GTMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  gfence_before();
  __syncthreads();
  gfence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 0;
      bool ok = true;
      int last_par[GSTAGES];
      for (int k = 0; k < GSTAGES; ++k) last_par[k] = -1;
      for (int64_t t = blockIdx.x; t < P.n_tiles && ok; t += gridDim.x) {
        const int am = (int)((t % P.n_mt) * GM);  // first atom
        const int zn = (int)((t / P.n_mt) * GN);  // first Z row
        for (int kc = 0; kc < P.nk; ++kc) {
          if (!mbar_wait(empty0 + 8 * s, ph ^ 1u, P.err, kSiteProducer)) {
            ok = false;
            break;
          }
          const uint32_t fb = full0 + 8 * s;
          mbar_expect_tx(fb, GSTAGE_BYTES);
          const uint32_t sb = smem_addr(smem + s * GSTAGE_BYTES);
          tma_load_2d(sb, &tmAh, kc * GK, am, fb);
          tma_load_2d(sb + GA_BYTES, &tmAl, kc * GK, am, fb);
          tma_load_2d(sb + 2 * GA_BYTES, &tmBh, kc * GK, zn, fb);
          tma_load_2d(sb + 2 * GA_BYTES + GB_BYTES, &tmBl, kc * GK, zn, fb);
          last_par[s] = (int)ph;
          if (++s == GSTAGES) {
            s = 0;
            ph ^= 1u;
          }
        }
      }
      // Our copies land before the CTA may exit (immediate on the normal path).
      for (int k = 0; k < GSTAGES; ++k)
        if (last_par[k] >= 0) mbar_wait_quiet(full0 + 8 * k, (uint32_t)last_par[k]);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 0, it = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < P.n_tiles && ok; t += gridDim.x, ++it) {
        const uint32_t b = it & 1u, aph = (it >> 1) & 1u;
        if (!mbar_wait(acce0 + 8 * b, aph ^ 1u, P.err, kSiteMmaAcc)) {
          ok = false;
          break;
        }
        gfence_after();
        const uint32_t d = tmem_base + b * GACC_STRIDE;
        for (int kc = 0; kc < P.nk; ++kc) {
          if (!mbar_wait(full0 + 8 * s, ph, P.err, kSiteMmaFull)) {
            ok = false;
            break;
          }
          gfence_after();
          const uint32_t sb = smem_addr(smem + s * GSTAGE_BYTES);
#pragma unroll
          for (int kk = 0; kk < GK / 16; ++kk) {
            const uint64_t ah = gdesc(sb + kk * 32), al = gdesc(sb + GA_BYTES + kk * 32);
            const uint64_t bh = gdesc(sb + 2 * GA_BYTES + kk * 32);
            const uint64_t bl = gdesc(sb + 2 * GA_BYTES + GB_BYTES + kk * 32);
            gmma(d, ah, bh, (kc | kk) != 0);
            gmma(d, al, bh, 1u);
            gmma(d, ah, bl, 1u);
          }
          gcommit(empty0 + 8 * s);  // frees the stage once these MMAs retire
          if (++s == GSTAGES) {
            s = 0;
            ph ^= 1u;
          }
        }
        if (!ok) break;
        gcommit(accf0 + 8 * b);
      }
      // Drain: every MMA issued above has retired once `done` completes.
      gcommit(done);
      mbar_wait_quiet(done, 0);
    }
  } else {
    // ---------------- epilogue: warps 2-5, one TMEM lane quadrant each ----------------
    const int q = warp & 3;
    const float zs = __ldg(P.scl) * __ldg(P.scl + 1);
    uint32_t it = 0;
    for (int64_t t = blockIdx.x; t < P.n_tiles; t += gridDim.x, ++it) {
      const uint32_t b = it & 1u, aph = (it >> 1) & 1u;
      const int a = (int)((t % P.n_mt) * GM) + 32 * q + lane;  // this lane's atom
      const int64_t zn = (t / P.n_mt) * GN;
      int ok = 0;
      if (lane == 0) ok = mbar_wait(accf0 + 8 * b, aph, P.err, kSiteEpi) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      gfence_after();
#pragma unroll 1
      for (int c = 0; c < GN / 16; ++c) {
        float v[16];
        gtmem_ld16(tmem_base + ((uint32_t)(32 * q) << 16) + b * GACC_STRIDE + c * 16, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (a < P.Np) {
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const int64_t n = zn + c * 16 + k;
            if (n < P.rows) P.Z[n * P.Np + a] = v[k] * zs;
          }
        }
      }
      // every tensor-memory read of this tile has completed: release the buffer
      gfence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acce0 + 8 * b);
    }
  }

  gfence_before();
  __syncthreads();
  gfence_after();
  if (warp == 1) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(GTMEM_COLS)
                 : "memory");
  }
}

// Largest |x| over n floats as the bits of a non-negative float (which order
// like unsigned integers), max-combined into *out.
__global__ void k_absmax(const float* __restrict__ x, int64_t n, unsigned int* out) {
  unsigned int m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, __float_as_uint(fabsf(x[i])));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m != 0) atomicMax(out, m);
}

// The power of two that brings the largest magnitude just below 2^14 (1 for
// an all-zero operand).
__device__ __forceinline__ float split_scale(unsigned int maxbits) {
  const float mx = __uint_as_float(maxbits);
  if (!(mx > 0.0f) || isinf(mx)) return 1.0f;
  int e = 0;
  frexpf(mx, &e);  // mx = m 2^e, m in [0.5, 1)
  return ldexpf(1.0f, 14 - e);
}

__device__ __forceinline__ void split_store(float v, __half* hi, __half* lo, int64_t idx) {
  const __half h = __float2half_rn(v);
  hi[idx] = h;
  lo[idx] = __float2half_rn(v - __half2float(h));
}

// S = B + B^T, scaled and split into FP16 hi/lo rows of stride ldS.  B holds
// the upper 3x3 blocks (block row i < block column j, written by the pair
// pass; nothing else of B is written or read), so
//   S[r][c] = B[r][c] for r/3 < c/3,  B[c][r] for r/3 > c/3,  0 for r/3 == c/3.
// One 64 x 64 tile of B per block (tile pairs I <= J, 32 x 8 threads, two
// columns per thread): S at (I, J) and, transposed, at (J, I).
__device__ __forceinline__ void split_store2(float v0, float v1, __half* hi, __half* lo, int64_t idx) {
  const __half2 h = __floats2half2_rn(v0, v1);
  const float2 hf = __half22float2(h);
  *reinterpret_cast<__half2*>(hi + idx) = h;
  *reinterpret_cast<__half2*>(lo + idx) = __floats2half2_rn(v0 - hf.x, v1 - hf.y);
}
__global__ void __launch_bounds__(256) k_split_sym(const float* __restrict__ B, int64_t n, int64_t ldB,
                                                   const unsigned int* maxbits, __half* Shi, __half* Slo,
                                                   int64_t ldS, float* scl) {
  __shared__ float t1[64][65];
  const float s = split_scale(*maxbits);
  if (blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0) scl[0] = 1.0f / s;
  const int64_t tiles = (n + 63) / 64;
  const int64_t l = blockIdx.x;
  const double bq = 2.0 * (double)tiles + 1.0;
  int64_t ti = (int64_t)((bq - sqrt(bq * bq - 8.0 * (double)l)) * 0.5);
  auto cum = [&](int64_t x) { return x * tiles - x * (x - 1) / 2; };
  while (ti > 0 && cum(ti) > l) --ti;
  while (cum(ti + 1) <= l) ++ti;
  const int64_t tj = ti + (l - cum(ti));
  const int x2 = 2 * threadIdx.x, y0 = threadIdx.y;
  const bool vec = ((n | ldB | ldS) & 1) == 0;  // pairs of columns stay inside rows and aligned
  for (int y = y0; y < 64; y += 8) {
    const int64_t r = ti * 64 + y, c = tj * 64 + x2;
    float v0 = 0.f, v1 = 0.f;
    if (r < n) {
      if (vec && c + 1 < n) {
        const float2 b = *reinterpret_cast<const float2*>(B + r * ldB + c);
        v0 = b.x;
        v1 = b.y;
      } else {
        if (c < n) v0 = B[r * ldB + c];
        if (c + 1 < n) v1 = B[r * ldB + c + 1];
      }
    }
    t1[y][x2] = (r / 3 < c / 3) ? v0 : 0.f;
    t1[y][x2 + 1] = (r / 3 < (c + 1) / 3) ? v1 : 0.f;
  }
  __syncthreads();
  for (int y = y0; y < 64; y += 8) {
    // (I, J): the upper entries, and on a diagonal tile the lower ones by transposition
    {
      const int64_t r = ti * 64 + y, c = tj * 64 + x2;
      float v0 = t1[y][x2], v1 = t1[y][x2 + 1];
      if (ti == tj) {
        v0 += t1[x2][y];
        v1 += t1[x2 + 1][y];
      }
      if (r < n) {
        if (vec && c + 1 < n) {
          split_store2(v0 * s, v1 * s, Shi, Slo, r * ldS + c);
        } else {
          if (c < n) split_store(v0 * s, Shi, Slo, r * ldS + c);
          if (c + 1 < n) split_store(v1 * s, Shi, Slo, r * ldS + c + 1);
        }
      }
    }
    // (J, I): the transpose
    if (ti != tj) {
      const int64_t r = tj * 64 + y, c = ti * 64 + x2;
      const float v0 = t1[x2][y], v1 = t1[x2 + 1][y];
      if (r < n) {
        if (vec && c + 1 < n) {
          split_store2(v0 * s, v1 * s, Shi, Slo, r * ldS + c);
        } else {
          if (c < n) split_store(v0 * s, Shi, Slo, r * ldS + c);
          if (c + 1 < n) split_store(v1 * s, Shi, Slo, r * ldS + c + 1);
        }
      }
    }
  }
}

// planeT[a][k] = plane[k][a] scaled and split (k < K rows of the plane,
// a < Np atoms); 32 x 32 tiles through shared memory, 32 x 8 threads.
__global__ void __launch_bounds__(256) k_split_planeT(const float* __restrict__ plane, int64_t K, int Np,
                                                      const unsigned int* maxbits, __half* Thi, __half* Tlo,
                                                      int64_t ldT, float* scl) {
  __shared__ float t[32][33];
  const float s = split_scale(*maxbits);
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) scl[1] = 1.0f / s;
  const int64_t k0 = (int64_t)blockIdx.x * 32;
  const int a0 = blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += 8) {
    const int64_t k = k0 + y;
    const int a = a0 + threadIdx.x;
    t[y][threadIdx.x] = (k < K && a < Np) ? plane[k * Np + a] : 0.f;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += 8) {
    const int a = a0 + y;
    const int64_t k = k0 + threadIdx.x;
    if (a < Np && k < K) split_store(t[threadIdx.x][y] * s, Thi, Tlo, (int64_t)a * ldT + k);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 gemm_encode_fn() {
  static std::atomic<PFN_cuTensorMapEncodeTiled_v12000> cached{nullptr};
  PFN_cuTensorMapEncodeTiled_v12000 fn = cached.load(std::memory_order_acquire);
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess) {
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
      cached.store(fn, std::memory_order_release);
    }
  }
  return fn;
}

// 2-D FP16 map over rows of `inner` elements (row stride ld elements), boxes
// of 64 elements x box_rows rows with the 128-byte swizzle; reads past
// `inner` or `rows` fill with zeros.
bool make_map_2d(CUtensorMap* m, const void* base, int64_t inner, int64_t rows, int64_t ld, int box_rows) {
  auto fn = gemm_encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)GK, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

int64_t bwd_gemm_ld(int64_t F) { return (3 * F + GK - 1) / GK * GK; }

cudaError_t run_backward_gemm(const BackwardGemm& G, cudaStream_t st) {
  const int64_t K = 3 * G.F;  // Z rows = contraction length
  const int64_t ld = bwd_gemm_ld(G.F);
  if (K <= 0) return cudaSuccess;
  // maxbits[0] (a bound of max |B|: max |c| over the pairs) comes from the
  // backward pair kernel; here the largest |plane|
  cudaError_t e = cudaMemsetAsync(G.maxbits + 1, 0, sizeof(unsigned int), st);
  if (e != cudaSuccess) return e;
  k_absmax<<<(unsigned)std::min<int64_t>(152 * 8, (K * G.Np + 255) / 256), 256, 0, st>>>(G.plane, K * G.Np,
                                                                                        G.maxbits + 1);
  const int64_t tiles = (K + 63) / 64;
  k_split_sym<<<(unsigned)(tiles * (tiles + 1) / 2), dim3(32, 8), 0, st>>>(G.B, K, G.ldB, G.maxbits, G.Shi, G.Slo,
                                                                         ld, G.scl);
  k_split_planeT<<<dim3((unsigned)((K + 31) / 32), (unsigned)((G.Np + 31) / 32)), dim3(32, 8), 0, st>>>(
      G.plane, K, G.Np, G.maxbits + 1, G.Thi, G.Tlo, ld, G.scl);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  CUtensorMap mAh, mAl, mBh, mBl;
  if (!make_map_2d(&mAh, G.Thi, K, G.Np, ld, GM) || !make_map_2d(&mAl, G.Tlo, K, G.Np, ld, GM) ||
      !make_map_2d(&mBh, G.Shi, K, K, ld, GN) || !make_map_2d(&mBl, G.Slo, K, K, ld, GN))
    return cudaErrorInvalidValue;
  GemmParams P{};
  P.n_mt = (G.Np + GM - 1) / GM;
  P.n_tiles = P.n_mt * ((K + GN - 1) / GN);
  P.nk = (int)((K + GK - 1) / GK);
  P.rows = K;
  P.Np = G.Np;
  P.Z = G.Z;
  P.scl = G.scl;
  P.err = G.dev_error;
  if ((e = cudaFuncSetAttribute(k_bwd_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, GSMEM)) != cudaSuccess)
    return e;
  const int grid = (int)std::min<int64_t>(P.n_tiles, G.num_sms > 0 ? G.num_sms : 148);
  k_bwd_gemm<<<grid, GTHREADS, GSMEM, st>>>(mAh, mAl, mBh, mBl, P);
  return cudaGetLastError();
}

}  // namespace gbr
