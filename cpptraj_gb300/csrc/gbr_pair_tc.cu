// gbr_pair_tc.cu -- tensor-core (tcgen05, sm_103a) all-pairs contraction (K2).
//
// Same job as gbr_pair_fp32.cu -- the pair loop of
// Analysis_Rms2d::Calculate_2D (src/Analysis_Rms2d.cpp:252-286) and
// MetricArray::calcFrameDistances (src/Cluster/MetricArray.cpp:786-793) --
// with the residual contraction D_ji = sum_a p_j[a] p_i[a]^T run on the
// 5th-generation tensor cores.
//
// Operands.  p = sqrt(w)*d is split into FP16 hi + lo (scaled per frame by a
// power of two, undone in the epilogue); hi*hi + lo*hi + hi*lo is accumulated
// in FP32 in tensor memory, which reproduces the products to ~2^-22 relative.  The planes are [F][3][Np]
// FP16 (atoms contiguous), so one 3-D TMA box (64 atoms, 3 components, n
// frames) lands in shared memory as (frame, component) rows of 128 bytes with
// the 128-byte swizzle the UMMA K-major descriptor expects.
//
// Tile.  A (M = 128 rows) holds 42 reference frames x 3 components (rows
// 126-127 unused); B (N = 192) holds 64 target frames x 3 components.  The
// 128 x 192 FP32 accumulator therefore contains the 3x3 block of all 42 x 64
// pairs; two accumulators (columns 0 and 256 of a 512-column TMEM allocation)
// let the epilogue of one tile overlap the MMAs of the next.
//
// Warp roles (320 threads, one persistent CTA per SM):
//   warp 0      TMA producer: 4 boxes (A hi/lo, B hi/lo) per 64-atom stage,
//               two stages in shared memory.
//   warp 1      TMEM allocation and the single MMA-issuing thread.
//   warps 2-9   epilogue: tcgen05.ld 48-column chunks, stage them through
//               shared memory, then the per-pair FP32 eigen epilogue
//               (gbr_common.cuh) and coalesced stores into TRI/FULL output.
// Every mbarrier wait is bounded (about 2 s); on expiry the kernel records
// an error code, drains its own MMAs, frees tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <atomic>
#include <vector>

#include "gbr_common.cuh"
#include "gbr_internal.h"
#include "gbr_mbar.cuh"
#include <cstring>

namespace gbr {

namespace {
constexpr int TI = 42;                 // reference frames per tile (per CTA), the default shape
constexpr int TJ = 64;                 // target frames per tile
constexpr int UM = 128;                // MMA M
constexpr int UN = 3 * TJ;             // MMA N = 192
// Pipeline configurations: KA atoms per stage, rows of 2*KA bytes with the
// matching swizzle (128 B or 64 B), STAGES stages of shared memory.
template <int KA_>
struct Pipe {
  static constexpr int KA = KA_;
  static constexpr int ROW = 2 * KA;                       // bytes per (frame, component) row
  static constexpr int STAGES = (KA == 64) ? 2 : 4;
  static constexpr int A_BYTES = UM * ROW;                 // TMA writes 126 of the 128 rows
  static constexpr int B_BYTES = UN * ROW;
  static constexpr int A_TX = 3 * TI * ROW;
  static constexpr int B_TX = UN * ROW;
  static constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr uint32_t SBO = 8 * ROW;                 // 8-row core-matrix groups
  static constexpr uint64_t LAYOUT = (KA == 64) ? 2ull : 4ull;  // SWIZZLE_128B : SWIZZLE_64B
};
constexpr int EPI_WARPS = 16;          // four groups of four warps (one per TMEM lane quadrant)
constexpr int EPI_GROUPS = EPI_WARPS / 4;
constexpr int THREADS = 64 + 32 * EPI_WARPS;
// The pair-of-SMs kernel adds one warp that stages each tile's frame terms a
// tile ahead of the epilogue.
constexpr int THREADS2 = THREADS + 32;
// Epilogue shape: CH target frames (3 CH accumulator columns) per chunk read
// from tensor memory and staged in shared memory, one staging buffer per
// group.  Wider chunks give each group more pairs per barrier (the epilogue-
// bound small-N case); narrower ones leave shared memory for deeper operand
// pipelines (large N).
template <int CH, int TI_ = TI, bool ROWS_ = true>
struct Epi {
  static constexpr int TIE = TI_;       // reference frames per CTA tile
  static constexpr int CH_TGT = CH;
  static constexpr int CH_COLS = 3 * CH;
  // Rows of the staged chunk: 16-frame chunks are written as float4s (row
  // stride 52 = 20 mod 32: the float4s of 8 consecutive rows hit distinct
  // banks); narrower ones as floats with an odd stride.
  static constexpr bool ST_VEC = (CH >= 16);
  static constexpr int ST_STRIDE = ST_VEC ? CH_COLS + 4 : CH_COLS + 1;
  static constexpr int STAGING_BYTES = 128 * ST_STRIDE * 4;
  // Result rows of one tile (pair kernels, triangle output): TI rows of TJ
  // values, padded by one chunk so the chunk writes hit 32 distinct banks.
  static constexpr int RB_STRIDE = TJ + CH;
  static constexpr int ROWBUF_BYTES = TI_ * RB_STRIDE * 4;
  // Staged frame terms (below): slots, reference-pair entry, the tile
  // (tile row, tile column, A, B), frame numbers, row bases (kernels with
  // row stores only).
  static constexpr int TERM_RP = ((TI_ + TJ) * 16 + 3) & ~3;
  static constexpr int TERM_META = TERM_RP + kRefPairStride;
  static constexpr int TERM_PERM = TERM_META + 4;
  static constexpr int TERM_ROWBASE = (TERM_PERM + TI_ + TJ + 1) & ~1;
  static constexpr int TERM_FLOATS = (TERM_ROWBASE + (ROWS_ ? 2 * (TI_ + TJ) : 0) + 3) & ~3;
};
using Epi1 = Epi<8, TI, false>;  // the one-SM kernels: 24 accumulator columns per chunk, no row stores
constexpr int STAGING_BYTES = Epi1::STAGING_BYTES;
// Per-tile frame terms staged in shared memory, two buffers.  With A the
// reference (pre-alignment) of the tile's first reference frame and B that of
// its first target frame, each frame slot holds its Side terms for a pair
// with references (A, B) (Q, c, m, sqrt n), 1/scale and its own reference, as
// four float4s: 0 = Q0..Q3, 1 = Q4..Q7, 2 = (Q8, c, m, sn), 3 = (1/scale,
// reference, -, -).  Float4 k of slot s sits at 4 s + (k ^ ((s >> 1) & 3)), so
// the k-th float4s of 8 consecutive slots fall in distinct banks.  After the
// frame slots: the reference-pair entry of (A, B) (kRefPairStride floats),
// the tile (tile row, tile column, A, B as ints), for a triangle over
// reference-sorted positions each slot's frame number (TI + TJ ints; -1
// outside the map), and the row bases below.
// Then, for the row stores of a triangle, an int64 per slot: in frame order,
// the output index of (reference slot il, target slot 0) per reference slot;
// over sorted positions, n f - f (f + 1) / 2 - f - 1 for the slot's frame f,
// so that a pair's index is the base of its smaller frame plus the larger
// frame (Epi's TERM_* offsets).
__device__ __forceinline__ int slot_f4(int s, int k) { return 4 * s + (k ^ ((s >> 1) & 3)); }
static_assert(TJ == 64, "row stores split the slot index with shifts");
template <class E>
constexpr int epi_bytes() {
  return EPI_GROUPS * E::STAGING_BYTES + 2 * E::TERM_FLOATS * 4;
}
constexpr int EPI_BYTES = epi_bytes<Epi1>();
constexpr int BAR_BYTES = 128;
constexpr int SMEM_BYTES = 1024 + 2 * (2 * UM * 128 + 2 * UN * 128) + EPI_BYTES + BAR_BYTES;
static_assert(SMEM_BYTES <= 232448, "one-SM kernel shared memory");
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t ACC_STRIDE = 256;

// Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = F16
// (bits 7-12 = 0), both K-major (bits 15-16 = 0), N >> 3 at bits 17-22,
// M >> 4 at bits 24-28.
constexpr uint32_t IDESC = (1u << 4) | ((uint32_t)(UN >> 3) << 17) | ((uint32_t)(UM >> 4) << 24);

struct TcParams {
  const int2* tiles;  // (ti, tj) per tile
  int64_t n_tiles;
  int64_t i_base;     // first reference frame of tile row 0
  int64_t jt_base;    // first target frame of tile column 0
  int64_t i_end, jt_end;
  int64_t tgt0;
  int nk;             // 64-atom stages per tile
  const float* inv_scale;  // per-frame 1/scale of the FP16 split
  FrameTerms terms;
  OutMap map;
  FlagList flags;
  int* err;
  int row_stores;  // triangle results gathered into whole tile rows before the store (pair kernels)
  const int* skip;  // non-null and non-zero at launch: the kernel returns at once
  BwdArgs bwd;      // backward instantiation: c*T blocks, row terms, forward values
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          dst),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// UMMA shared-memory descriptor: K-major, swizzled rows (128 B or 64 B),
// 8-row groups SBO bytes apart, version bits 46-48 = 0b001, layout in 61-63.
template <class PP>
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(PP::SBO >> 4) << 32;
  d |= 1ull << 46;
  d |= PP::LAYOUT << 61;
  return d;
}

__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
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
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float* v) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
#pragma unroll
  for (int k = 0; k < 4; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void named_sync(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

__device__ __forceinline__ void mbar_arrive_remote(uint32_t caddr) {
  asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(caddr) : "memory");
}

// A staged slot's Side terms (float4s 0-2) and, optionally, its 1/scale.
__device__ __forceinline__ void load_slot(const float* T, int s, Side& sd) {
  const float4* T4 = reinterpret_cast<const float4*>(T);
  const float4 v0 = T4[slot_f4(s, 0)], v1 = T4[slot_f4(s, 1)], v2 = T4[slot_f4(s, 2)];
  sd.Q[0] = v0.x; sd.Q[1] = v0.y; sd.Q[2] = v0.z; sd.Q[3] = v0.w;
  sd.Q[4] = v1.x; sd.Q[5] = v1.y; sd.Q[6] = v1.z; sd.Q[7] = v1.w;
  sd.Q[8] = v2.x; sd.c = v2.y; sd.m = v2.z; sd.sn = v2.w;
}
// The tile's reference-pair entry, staged at Trp (16-byte aligned).
__device__ __forceinline__ void load_refpair_smem(const float* Trp, RefPair& r) {
  const float4* p = reinterpret_cast<const float4*>(Trp);
#pragma unroll
  for (int k = 0; k < 6; ++k) r.v[k] = p[k];
}
__device__ __forceinline__ void load_slot(const float* T, int s, Side& sd, float& inv_scale) {
  load_slot(T, s, sd);
  inv_scale = reinterpret_cast<const float4*>(T)[slot_f4(s, 3)].x;
}

// Stages tile t's frame terms into T (one buffer of the layout above) with
// nthr threads (this one is thread tid): the tile, its references (A, B),
// each slot's Side terms against (A, B), the reference-pair entry and, for
// row stores, the frame numbers and row bases.
template <class E, bool BWD>
__device__ __forceinline__ void stage_tile_terms(const TcParams& P, float* T, int64_t t, int ti_frames, int i_off,
                                                 bool has_rowbuf, int tid, int nthr) {
  constexpr int TI = E::TIE;
  const int K = P.terms.K;
  const int2 tl = P.tiles[t];
  const int64_t i0 = P.i_base + (int64_t)tl.x * ti_frames + i_off;
  const int64_t jt0 = P.jt_base + (int64_t)tl.y * TJ;
  const int A = (K > 1 && i0 < P.i_end) ? __ldg(P.terms.assign + i0) : 0;
  const int B = (K > 1 && jt0 < P.jt_end) ? __ldg(P.terms.assign + P.tgt0 + jt0) : 0;
  const bool same_t = (A == B);
  const float* Ug = P.terms.RP + (size_t)(B * K + A) * kRefPairStride;
  float4* T4 = reinterpret_cast<float4*>(T);
  for (int sl = tid; sl < TI + TJ; sl += nthr) {
    int64_t f;
    bool valid;
    int other;
    const bool ref_side = sl < TI;
    if (ref_side) {
      f = i0 + sl;
      valid = f < P.i_end;
      other = B;
    } else {
      const int64_t jt = jt0 + (sl - TI);
      f = P.tgt0 + jt;
      valid = jt < P.jt_end;
      other = A;
    }
    float4 o0 = make_float4(0.f, 0.f, 0.f, 0.f), o1 = o0, o2 = o0, o3 = o0;
    if (valid) {
      const int own = (K > 1) ? __ldg(P.terms.assign + f) : 0;
      const float trPown = (K > 1) ? __ldg(P.terms.trP + f * K + own) : 0.0f;
      float Pv[9], U[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        Pv[k] = __ldg(P.terms.P + (f * K + other) * 9 + k);
        U[k] = same_t ? 0.0f : __ldg(Ug + k);
      }
      Side sd;
      side_terms(Pv, __ldg(P.terms.nrm + f), trPown, U, same_t, ref_side, sd);
      o0 = make_float4(sd.Q[0], sd.Q[1], sd.Q[2], sd.Q[3]);
      o1 = make_float4(sd.Q[4], sd.Q[5], sd.Q[6], sd.Q[7]);
      o2 = make_float4(sd.Q[8], sd.c, sd.m, sd.sn);
      o3 = make_float4(__ldg(P.inv_scale + f), __int_as_float(own), 0.f, 0.f);
    }
    T4[slot_f4(sl, 0)] = o0;
    T4[slot_f4(sl, 1)] = o1;
    T4[slot_f4(sl, 2)] = o2;
    T4[slot_f4(sl, 3)] = o3;
  }
  for (int x = tid; x < kRefPairStride; x += nthr) T[E::TERM_RP + x] = __ldg(Ug + x);
  if (tid == 0) {
    int* meta = reinterpret_cast<int*>(T + E::TERM_META);
    meta[0] = tl.x;
    meta[1] = tl.y;
    meta[2] = A;
    meta[3] = B;
  }
  // Row bases for every triangle a pair kernel writes (row stores or direct
  // stores); the one-SM kernels index through out_index.
  const bool rows = !BWD && has_rowbuf && P.map.tri;
  const int64_t n = P.map.n_ref;
  if (P.map.perm) {
    int* Tp = reinterpret_cast<int*>(T + E::TERM_PERM);
    int64_t* Trb = reinterpret_cast<int64_t*>(T + E::TERM_ROWBASE);
    for (int x = tid; x < TI + TJ; x += nthr) {
      int v = -1;
      if (x < TI) {
        if (i0 + x < P.i_end) v = __ldg(P.map.perm + i0 + x);
      } else {
        const int64_t jt = jt0 + (x - TI);
        if (jt < P.jt_end) v = __ldg(P.map.perm + P.tgt0 + jt);
      }
      Tp[x] = v;
      if (rows) {
        const int64_t fv = v;
        Trb[x] = n * fv - (fv + 1) * fv / 2 - fv - 1;
      }
    }
  } else if (rows) {
    // tri_index(n, i, jt0) - base for reference frame i = i0 + x
    for (int x = tid; x < TI; x += nthr) {
      const int64_t i = i0 + x;
      reinterpret_cast<int64_t*>(T + E::TERM_ROWBASE)[x] = n * i - (i + 1) * i / 2 + jt0 - i - 1 - P.map.base;
    }
  }
}

// Epilogue warps (2 .. 2 + EPI_WARPS): for tiles t0, t0 + tstep, ... wait for
// the accumulator and the tile's staged frame terms (staged here by all
// epilogue threads, or, with STAGER, by the staging warp a tile ahead: tfull
// / tempty hand the two buffers over), read the 128 x 192 FP32 block from
// tensor memory in chunks of 3 CH_TGT columns (group g takes chunks g,
// g + 4, ...), and run the per-pair solve.  The reference frames of a tile
// start at i_base + ti * ti_frames + i_off.  acce_bar is the address the
// warps arrive on when the accumulator is free (remote: CTA 0 of a pair).
// BWD (one frame set, TRI, one reference): for each pair i < j, with
// c = g_ij / RMSD_ij and T the rotation taking x'_j onto x'_i, the block
// B[3i..3i+2][3j..3j+2] = c T and the row terms E_i += c (I - T),
// E_j += c (I - T^T), C_i += c, C_j += c.  The row terms are summed across
// the warp's lanes that share a frame, then in shared memory per tile
// (rowbuf), and added to E / C once per tile.
template <class E, bool BWD = false, bool STAGER = false>
__device__ __forceinline__ void epilogue_tiles(const TcParams& P, uint32_t tmem_base, float* staging, float* terms,
                                               float* rowbuf, volatile int* okf, uint32_t accf0, uint32_t acce_bar,
                                               bool remote, int64_t t0, int64_t tstep, int ti_frames, int i_off,
                                               int warp, int lane, uint32_t tfull0 = 0, uint32_t tempty0 = 0) {
  constexpr int TI = E::TIE, TERM_RP = E::TERM_RP, TERM_PERM = E::TERM_PERM, TERM_ROWBASE = E::TERM_ROWBASE,
                TERM_FLOATS = E::TERM_FLOATS, TERM_META = E::TERM_META;
  const int e = warp - 2;
  const int g = e >> 2;
  const int q = warp & 3;               // TMEM lane quadrant this warp may access
  const int row = 32 * q + lane;        // accumulator row = (reference frame, component)
  const int tid = (e & 3) * 32 + lane;  // 0..127 within the group
  const int etid = e * 32 + lane;       // 0..511
  constexpr int CH_TGT = E::CH_TGT, CH_COLS = E::CH_COLS, ST_STRIDE = E::ST_STRIDE;
  float* st = staging + g * (128 * ST_STRIDE);
  const bool tri = P.map.tri;
  // Row stores: the pairs of a tile gather in shared memory and leave as
  // whole rows of the triangle (TJ contiguous values) instead of CH_TGT-value
  // pieces, which matters when the output is host memory across the link.
  const bool rows = !BWD && rowbuf != nullptr && tri && P.row_stores != 0;
  // Direct stores (triangle in device memory): each pair's value leaves from
  // its thread, indexed through the tile's staged row bases, with no row
  // buffer and no barrier before the stores.
  const bool direct = !BWD && rowbuf != nullptr && tri && P.row_stores == 0;
  constexpr int RB_STRIDE = E::RB_STRIDE;
  // BWD: this CTA's row terms, [TI][10] for its reference frames then
  // [TJ][10] for the tile's target frames, zero between tiles.
  float* Erow = rowbuf;
  float* Ecol = rowbuf + TI * 10;
  constexpr int kEterms = (TI + TJ) * 10;
  if constexpr (BWD) {
    static_assert(kEterms <= TI * E::RB_STRIDE, "row terms fit the row buffer");
    for (int x = etid; x < kEterms; x += EPI_WARPS * 32) rowbuf[x] = 0.0f;  // ordered by the first tile's barrier
  }
  float cmax = 0.0f;  // BWD: largest |c| this thread saw (every entry of B is at most that)
  uint32_t it = 0;
  for (int64_t t = t0; t < P.n_tiles; t += tstep, ++it) {
    const uint32_t b = it & 1u, aph = (it >> 1) & 1u;
    float* T = terms + b * TERM_FLOATS;
    // Buffer b was last read two tiles ago, before every group passed the
    // previous tile's barrier (inline staging), or is handed over by the
    // staging warp through tfull / tempty.
    if constexpr (!STAGER) stage_tile_terms<E, BWD>(P, T, t, ti_frames, i_off, rowbuf != nullptr, etid, EPI_WARPS * 32);
    // One thread waits; the verdict is shared so every thread that passes the
    // barrier behind it takes the same path.  With direct stores (no barrier
    // of all epilogue warps later in the tile) each group waits for itself,
    // so a group held up in one tile holds back only its own next tile;
    // otherwise one thread waits for all 16 warps.
    const bool group_wait = STAGER && !BWD && !rows;
    if (group_wait) {
      if (tid == 0) {
        const bool okw = mbar_wait(accf0 + 8 * b, aph, P.err, 5) && mbar_wait(tfull0 + 8 * b, aph, P.err, 15);
        okf[2 * g + b] = okw ? 1 : 0;
      }
      named_sync(1 + g, 128);
    } else {
      if (etid == 0) {
        bool okw = mbar_wait(accf0 + 8 * b, aph, P.err, 5);
        if constexpr (STAGER) okw = okw && mbar_wait(tfull0 + 8 * b, aph, P.err, 15);
        okf[b] = okw ? 1 : 0;
      }
      named_sync(1 + EPI_GROUPS, EPI_WARPS * 32);
    }
    const bool ok = okf[group_wait ? 2 * g + b : b] != 0;
    const int* meta = reinterpret_cast<const int*>(T + TERM_META);
    const int2 tl = make_int2(meta[0], meta[1]);
    const int A = meta[2], B = meta[3];
    const int64_t i0 = P.i_base + (int64_t)tl.x * ti_frames + i_off;
    const int64_t jt0 = P.jt_base + (int64_t)tl.y * TJ;
    // Tile-relative limits: reference slots [0, ilim) and target slots
    // [0, jlim) are inside the map; d0 = jt0 - i0 (a target slot jj is after
    // reference slot il iff d0 + jj > il).
    const int64_t irem = P.i_end - i0, jrem = P.jt_end - jt0;
    const int ilim = irem <= 0 ? 0 : (irem < TI ? (int)irem : TI);
    const int jlim = jrem <= 0 ? 0 : (jrem < TJ ? (int)jrem : TJ);
    const int d0 = (int)(jt0 - i0);
    if (ok) {
      tc_fence_after();
      for (int c = g; c < TJ / CH_TGT; c += EPI_GROUPS) {
        float v[CH_COLS];
        const uint32_t taddr = tmem_base + ((uint32_t)(32 * q) << 16) + b * ACC_STRIDE + c * CH_COLS;
        if constexpr (CH_COLS == 48) {
          tmem_ld16(taddr, v);
          tmem_ld16(taddr + 16, v + 16);
          tmem_ld16(taddr + 32, v + 32);
        } else if constexpr (CH_COLS == 24) {
          tmem_ld16(taddr, v);
          tmem_ld8(taddr + 16, v + 16);
        } else {
          static_assert(CH_COLS == 12, "chunks of 16, 8 or 4 target frames");
          tmem_ld4(taddr, v);
          tmem_ld4(taddr + 4, v + 4);
          tmem_ld4(taddr + 8, v + 8);
        }
        tmem_wait_ld();
        if constexpr (E::ST_VEC) {
          float4* st4 = reinterpret_cast<float4*>(st + row * ST_STRIDE);
#pragma unroll
          for (int k = 0; k < CH_COLS / 4; ++k) st4[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
        } else {
#pragma unroll
          for (int k = 0; k < CH_COLS; ++k) st[row * ST_STRIDE + k] = v[k];
        }
        named_sync(1 + g, 128);
        const int64_t jc0 = jt0 + (int64_t)c * CH_TGT;
        if constexpr (BWD) {
          // Warp-uniform trip count (the lanes meet in shuffles); pairs
          // outside the triangle contribute zero.
#pragma unroll 1
          for (int pb = 0; pb < TI * CH_TGT; pb += 128) {
            const int p = pb + tid;
            const int il = p / CH_TGT, jl = p % CH_TGT;
            const int64_t i = i0 + il, j = jc0 + jl;
            float er[10], ec[10];
#pragma unroll
            for (int k = 0; k < 10; ++k) er[k] = ec[k] = 0.0f;
            if (p < TI * CH_TGT && i < P.i_end && j < P.jt_end && j > i) {
              Side si, sj;
              float sc;
              load_slot(T, il, si, sc);
              {
                float scj;
                load_slot(T, TI + c * CH_TGT + jl, sj, scj);
                sc *= scj;
              }
              F9 D;
#pragma unroll
              for (int pj = 0; pj < 3; ++pj)
#pragma unroll
                for (int pi = 0; pi < 3; ++pi) D.v[pj * 3 + pi] = st[(3 * il + pi) * ST_STRIDE + 3 * jl + pj];
              bool flag = false;
              float qv[4];
              // K = 1: the reference-pair entry of (0, 0)
              RefPair rp;
              load_refpair_smem(T + TERM_RP, rp);
              const float rm = pair_solve_inl(D, sc, si, sj, rp, true, P.terms, &flag, qv);
              const int64_t t = tri_index(P.map.n_ref, i, j);
              if (P.bwd.rmsd) P.bwd.rmsd[t] = rm;
              const float gij = P.bwd.g ? P.bwd.g[t] : 1.0f;
              const float cw = (rm > 1e-6f) ? gij / rm : 0.0f;
              cmax = fmaxf(cmax, fabsf(cw));
              const float a = qv[0], x = qv[1], y = qv[2], z = qv[3];
              // QCP rotation R(q) (row-major); T = R^T.  I - T comes straight
              // from the quaternion, so it is accurate when T ~ I.
              const float R0 = a * a + x * x - y * y - z * z, R1 = 2.f * (x * y + a * z), R2 = 2.f * (z * x - a * y);
              const float R3 = 2.f * (x * y - a * z), R4 = a * a - x * x + y * y - z * z, R5 = 2.f * (y * z + a * x);
              const float R6 = 2.f * (z * x + a * y), R7 = 2.f * (y * z - a * x), R8 = a * a - x * x - y * y + z * z;
              float* Bi = P.bwd.B + (size_t)(3 * i) * P.bwd.ldB + 3 * j;
              Bi[0] = cw * R0; Bi[1] = cw * R3; Bi[2] = cw * R6;
              Bi += P.bwd.ldB;
              Bi[0] = cw * R1; Bi[1] = cw * R4; Bi[2] = cw * R7;
              Bi += P.bwd.ldB;
              Bi[0] = cw * R2; Bi[1] = cw * R5; Bi[2] = cw * R8;
              const float d00 = 2.f * (y * y + z * z), d11 = 2.f * (x * x + z * z), d22 = 2.f * (x * x + y * y);
              er[0] = cw * d00; er[1] = -cw * R3; er[2] = -cw * R6;
              er[3] = -cw * R1; er[4] = cw * d11; er[5] = -cw * R7;
              er[6] = -cw * R2; er[7] = -cw * R5; er[8] = cw * d22;
              er[9] = cw;
              ec[0] = cw * d00; ec[1] = -cw * R1; ec[2] = -cw * R2;
              ec[3] = -cw * R3; ec[4] = cw * d11; ec[5] = -cw * R5;
              ec[6] = -cw * R6; ec[7] = -cw * R7; ec[8] = cw * d22;
              ec[9] = cw;
            }
            // lanes of one reference frame: CH_TGT consecutive lanes; of one
            // target frame: every CH_TGT-th lane
#pragma unroll
            for (int k = 0; k < 10; ++k) {
#pragma unroll
              for (int o = 1; o < CH_TGT; o <<= 1) er[k] += __shfl_xor_sync(0xffffffffu, er[k], o);
#pragma unroll
              for (int o = CH_TGT; o < 32; o <<= 1) ec[k] += __shfl_xor_sync(0xffffffffu, ec[k], o);
            }
            if ((lane & (CH_TGT - 1)) == 0 && p < TI * CH_TGT)
#pragma unroll
              for (int k = 0; k < 10; ++k)
                if (er[k] != 0.0f) atomicAdd(&Erow[il * 10 + k], er[k]);
            if (lane < CH_TGT)
#pragma unroll
              for (int k = 0; k < 10; ++k)
                if (ec[k] != 0.0f) atomicAdd(&Ecol[(c * CH_TGT + jl) * 10 + k], ec[k]);
          }
        } else {
#pragma unroll 1
          for (int p = tid; p < TI * CH_TGT; p += 128) {
            const int il = tri ? p / CH_TGT : p % TI;
            const int jl = tri ? p % CH_TGT : p / TI;
            const int jj = c * CH_TGT + jl;  // target slot in the tile
            if (il >= ilim || jj >= jlim) continue;
            const int64_t i = i0 + il, jt = jc0 + jl;
            // A pair of this call's output?  With row stores (a triangle:
            // rows [i_base, i_end) = the map's rows, targets up to n_tgt)
            // only target > reference remains to test; the stores map it to
            // its index.
            int64_t idx = 0;
            if (rows || direct) {
              if (!(d0 + jj > il)) continue;
            } else {
              idx = out_index(P.map, i, jt);
              if (idx < 0) continue;
            }
            bool flag = false;
            // The solver's inputs from the tile's staged terms when the pair's
            // references are the tile's, else from global memory; one inlined
            // solve for both, and the same Side arithmetic, so a pair's result
            // never depends on its tile.
            const float4* T4 = reinterpret_cast<const float4*>(T);
            const int sj_slot = TI + c * CH_TGT + jl;
            const float4 i3 = T4[slot_f4(il, 3)], j3 = T4[slot_f4(sj_slot, 3)];
            Side si, sj;
            RefPair rp;
            bool same;
            float sc;
            if (__float_as_int(i3.y) == A && __float_as_int(j3.y) == B) {
              sc = i3.x * j3.x;
              load_slot(T, il, si);
              load_slot(T, sj_slot, sj);
              load_refpair_smem(T + TERM_RP, rp);
              same = (A == B);
            } else {
              sc = __ldg(P.inv_scale + i) * __ldg(P.inv_scale + P.tgt0 + jt);
              PairIn in;
              pair_terms(i, P.tgt0 + jt, P.terms, in);
              si = in.si;
              sj = in.sj;
              rp = in.rp;
              same = in.same;
            }
            F9 D;
#pragma unroll
            for (int pj = 0; pj < 3; ++pj)
#pragma unroll
              for (int pi = 0; pi < 3; ++pi) D.v[pj * 3 + pi] = st[(3 * il + pi) * ST_STRIDE + 3 * jl + pj];
            // inline: the tensor-core kernels have registers to spare
            const float r = pair_solve_inl(D, sc, si, sj, rp, same, P.terms, &flag);
            if (flag) flag_pair(P.flags, P.map, i, jt);
            if (rows) {
              rowbuf[il * RB_STRIDE + c * CH_TGT + jl] = r;
            } else if (direct) {
              const int64_t* Trb = reinterpret_cast<const int64_t*>(T + TERM_ROWBASE);
              if (P.map.perm) {
                // over sorted positions: the smaller frame's base plus the larger frame
                const int* Tp = reinterpret_cast<const int*>(T + TERM_PERM);
                const int a = Tp[il], bb = Tp[TI + jj];
                idx = (a < bb) ? Trb[il] + bb : Trb[TI + jj] + a;
              } else {
                idx = Trb[il] + jj;
              }
              P.map.out[idx] = r;
            } else {
              P.map.out[idx] = r;
            }
          }
        }
        // The group's staging buffer is written again by its next chunk: of
        // this tile, after this barrier; of the next tile, after that tile's
        // all-epilogue barrier (so none is needed after the last chunk).
        if (c + EPI_GROUPS < TJ / CH_TGT) named_sync(1 + g, 128);
      }
    }
    // Every tensor-memory read of this tile has completed (tmem_wait_ld per
    // chunk): the accumulator buffer is released before the row stores.
    tc_fence_before();
    __syncwarp();
    if (lane == 0) {
      if (remote)
        mbar_arrive_remote(acce_bar + 8 * b);
      else
        mbar_arrive(acce_bar + 8 * b);
    }
    if (!ok) break;
    if constexpr (BWD) {
      // Every group's shared-memory adds for this tile are done; the next
      // tile adds only after its own all-group barrier, past this flush.
      named_sync(1 + EPI_GROUPS, EPI_WARPS * 32);
      for (int x = etid; x < kEterms; x += EPI_WARPS * 32) {
        const float v = rowbuf[x];
        if (v == 0.0f) continue;
        rowbuf[x] = 0.0f;
        const int fl = x / 10, k = x % 10;
        const int64_t f = (fl < TI) ? i0 + fl : jt0 + (fl - TI);
        if (f < P.map.n_ref) {
          if (k < 9)
            atomicAdd(P.bwd.E + f * 9 + k, v);
          else
            atomicAdd(P.bwd.C + f, v);
        }
      }
    }
    if (rows) {
      // The next tile writes rowbuf only after its own all-group barrier,
      // which every thread reaches after these stores.
      named_sync(1 + EPI_GROUPS, EPI_WARPS * 32);
      const float* Tt = terms + b * TERM_FLOATS;  // this tile's staged frames
      const int* Tp = reinterpret_cast<const int*>(Tt + TERM_PERM);
      const int64_t* Trb = reinterpret_cast<const int64_t*>(Tt + TERM_ROWBASE);
#pragma unroll 1
      for (int x = etid; x < TI * TJ; x += EPI_WARPS * 32) {
        const int il = x >> 6, jl = x & (TJ - 1);
        // the pair loop's test: inside the map, target after reference
        if (il >= ilim || jl >= jlim || !(d0 + jl > il)) continue;
        int64_t idx;
        if (P.map.perm) {
          // out_index over sorted positions: the smaller frame's base plus
          // the larger frame
          const int a = Tp[il], bb = Tp[TI + jl];
          idx = (a < bb) ? Trb[il] + bb : Trb[TI + jl] + a;
        } else {
          idx = Trb[il] + jl;
        }
        P.map.out[idx] = rowbuf[il * RB_STRIDE + jl];
      }
    }
    if constexpr (STAGER) {
      // This warp's last read of buffer b (slots, entry, frames, row bases)
      // is done: hand it back to the staging warp.
      __syncwarp();
      if (lane == 0) mbar_arrive(tempty0 + 8 * b);
    }
  }
  if constexpr (BWD) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cmax = fmaxf(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
    if (lane == 0 && cmax > 0.0f && P.bwd.cmax) atomicMax(P.bwd.cmax, __float_as_uint(cmax));
  }
}

template <class PP>
__global__ void __launch_bounds__(THREADS, 1)
    k_pairs_tc(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
               const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl,
               const TcParams P) {
  constexpr int STAGES = PP::STAGES, KA = PP::KA, STAGE_BYTES = PP::STAGE_BYTES, A_BYTES = PP::A_BYTES,
                B_BYTES = PP::B_BYTES, A_TX = PP::A_TX, B_TX = PP::B_TX;
  if (P.skip && *P.skip != 0) return;  // a speculative launch whose speculation failed
  extern __shared__ uint8_t smem_raw[];
  // 1024-byte aligned by pointer arithmetic on the shared array itself (not
  // through an integer), so every access through it stays a shared-memory
  // access (LDS/STS), not a generic one.
  uint8_t* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  uint8_t* stage_base = smem;
  float* staging = (float*)(smem + STAGES * STAGE_BYTES);
  float* terms = (float*)(smem + STAGES * STAGE_BYTES + EPI_GROUPS * STAGING_BYTES);
  uint64_t* bars = (uint64_t*)(smem + STAGES * STAGE_BYTES + EPI_BYTES);
  // bars: full[4] empty[4] accfull[2] accempty[2] done[1]; then the TMEM address.
  uint32_t* tmem_slot = (uint32_t*)(bars + 14);
  volatile int* okf = (volatile int*)(bars + 15);  // accumulator verdicts, one per buffer
  const uint32_t full0 = smem_u32(bars + 0), empty0 = smem_u32(bars + 4), accf0 = smem_u32(bars + 8),
                 acce0 = smem_u32(bars + 10), done = smem_u32(bars + 12);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf0 + 8 * b, 1);
      mbar_init(acce0 + 8 * b, EPI_WARPS);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmAh) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmAl) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmBh) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmBl) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 0;
      bool ok = true;
      int last_par[STAGES];
      for (int k = 0; k < STAGES; ++k) last_par[k] = -1;
      for (int64_t t = blockIdx.x; t < P.n_tiles && ok; t += gridDim.x) {
        const int2 tl = P.tiles[t];
        const int iz = (int)(P.i_base + (int64_t)tl.x * TI);
        const int jz = (int)(P.tgt0 + P.jt_base + (int64_t)tl.y * TJ);
        for (int kc = 0; kc < P.nk; ++kc) {
          if (!mbar_wait(empty0 + 8 * s, ph ^ 1u, P.err, 1)) { ok = false; break; }
          const uint32_t fb = full0 + 8 * s;
          mbar_expect_tx(fb, 2 * A_TX + 2 * B_TX);
          const uint32_t sb = smem_u32(stage_base + s * STAGE_BYTES);
          tma_load_3d(sb, &tmAh, kc * KA, 0, iz, fb);
          tma_load_3d(sb + A_BYTES, &tmAl, kc * KA, 0, iz, fb);
          tma_load_3d(sb + 2 * A_BYTES, &tmBh, kc * KA, 0, jz, fb);
          tma_load_3d(sb + 2 * A_BYTES + B_BYTES, &tmBl, kc * KA, 0, jz, fb);
          last_par[s] = (int)ph;
          if (++s == STAGES) { s = 0; ph ^= 1u; }
        }
      }
      // Our copies land before the CTA may exit (immediate on the normal path).
      for (int k = 0; k < STAGES; ++k)
        if (last_par[k] >= 0) mbar_wait_quiet(full0 + 8 * k, (uint32_t)last_par[k]);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 0;
      uint32_t it = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < P.n_tiles && ok; t += gridDim.x, ++it) {
        const uint32_t b = it & 1u, aph = (it >> 1) & 1u;
        if (!mbar_wait(acce0 + 8 * b, aph ^ 1u, P.err, 2)) { ok = false; break; }
        tc_fence_after();
        const uint32_t d = tmem_base + b * ACC_STRIDE;
        for (int kc = 0; kc < P.nk; ++kc) {
          if (!mbar_wait(full0 + 8 * s, ph, P.err, 3)) { ok = false; break; }
          tc_fence_after();
          const uint32_t sb = smem_u32(stage_base + s * STAGE_BYTES);
#pragma unroll
          for (int kk = 0; kk < KA / 16; ++kk) {
            const uint64_t ah = smem_desc<PP>(sb + kk * 32), al = smem_desc<PP>(sb + A_BYTES + kk * 32);
            const uint64_t bh = smem_desc<PP>(sb + 2 * A_BYTES + kk * 32);
            const uint64_t bl = smem_desc<PP>(sb + 2 * A_BYTES + B_BYTES + kk * 32);
            umma_f16(d, ah, bh, (kc | kk) != 0);
            umma_f16(d, al, bh, 1u);
            umma_f16(d, ah, bl, 1u);
          }
          umma_commit(empty0 + 8 * s);  // frees the stage once these MMAs retire
          if (++s == STAGES) { s = 0; ph ^= 1u; }
        }
        if (!ok) break;
        umma_commit(accf0 + 8 * b);
      }
      // Drain: every MMA issued above has retired once `done` completes.
      umma_commit(done);
      mbar_wait_quiet(done, 0);
    }
  } else {
    // ---------------- epilogue ----------------
    epilogue_tiles<Epi1>(P, tmem_base, staging, terms, nullptr, okf, accf0, acce0, false, blockIdx.x, gridDim.x, TI, 0, warp,
                         lane);
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// Pair-of-SMs variant (tcgen05 cta_group::2).  A cluster of two CTAs shares
// one 256 x 192 MMA: CTA r holds reference frames i0 + 42 r .. +42 (its own
// 128-row A, rows 126-127 unused) and target frames j0 + 32 r .. +32 (half of
// B, 96 rows); the MMA issued by CTA 0 reads A from each CTA and B from both,
// and writes each CTA's 128 x 192 block into that CTA's tensor memory.  Per
// SM this halves the B bytes loaded by TMA and read from shared memory,
// which (with the three split products) is what limits the one-SM kernel.
//   full[s]  in CTA 0: both producers arrive (expect_tx of their own bytes)
//            and both CTAs' TMA copies complete_tx on it.
//   empty[s] in each CTA: CTA 0's commit arrives on both (multicast).
//   accf[b]  in each CTA: CTA 0's commit arrives on both.
//   acce[b]  in CTA 0: the epilogue warps of both CTAs arrive.
// ---------------------------------------------------------------------------
constexpr int TJH = TJ / 2;            // target frames per CTA half of B (32)
constexpr int UM2 = 256;
constexpr int UNH = 3 * TJH;           // 96 B rows per CTA
constexpr int BAR2_BYTES = 256;
// Pipeline and epilogue shape of the pair kernel: KA atoms per stage (rows of
// 2 KA bytes, 64- or 128-byte swizzle), STAGES stages, epilogue chunks of CH
// target frames.
template <int KA_, int STAGES_, int CH_, int TI_ = TI>
struct PairCfg {
  static constexpr int TIP = TI_;       // reference frames per CTA (2 TI_ per cluster tile)
  static constexpr int KA2 = KA_;
  static constexpr int ROW2 = 2 * KA_;
  static constexpr int STAGES2 = STAGES_;
  using E = Epi<CH_, TI_>;
  static constexpr int A2_BYTES = UM * ROW2;  // per CTA: 128 rows, TMA writes 126
  static constexpr int BH_BYTES = UNH * ROW2;
  static constexpr int A2_TX = 3 * TI_ * ROW2;
  static constexpr int BH_TX = UNH * ROW2;
  static constexpr int STAGE2_BYTES = 2 * A2_BYTES + 2 * BH_BYTES;
  static constexpr int EPI2_BYTES = epi_bytes<E>() + E::ROWBUF_BYTES;
  static constexpr int SMEM2_BYTES = 1024 + STAGES2 * STAGE2_BYTES + EPI2_BYTES + BAR2_BYTES;
  static constexpr uint32_t SBO = 8 * ROW2;                     // 8-row core-matrix groups
  static constexpr uint64_t LAYOUT = (KA_ == 64) ? 2ull : 4ull;  // SWIZZLE_128B : SWIZZLE_64B
  static_assert(SMEM2_BYTES <= 232448, "pair kernel shared memory");
  static_assert(STAGE2_BYTES % 1024 == 0 && A2_BYTES % 1024 == 0 && BH_BYTES % 1024 == 0, "swizzle alignment");
  static_assert(KA_ == 32 || KA_ == 64, "32- or 64-atom stages");
};
// Small N (epilogue-bound): 32-atom stages x 5, 8-frame epilogue chunks.
using PairShallow = PairCfg<32, 5, 8>;
// Large N (operand-feed bound): 64-atom stages (128-byte rows) x 3, 4-frame chunks.
using PairDeep = PairCfg<64, 3, 4>;
// Small N, wider epilogue chunks: 32-atom stages x 3, 16-frame chunks (each
// epilogue group takes one chunk per tile: half the named barriers per pair),
// 40 reference frames per CTA (rows 120-127 of A unused) so that a chunk's
// 40 x 16 pairs and a tile's 40 x 64 row stores split evenly over 128 and 512
// threads (5 each) instead of 5.25.
constexpr int TI_WIDE = 40;
using PairWide = PairCfg<32, 3, 16, TI_WIDE>;
constexpr uint32_t IDESC2 = (1u << 4) | ((uint32_t)(UN >> 3) << 17) | ((uint32_t)(UM2 >> 4) << 24);

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t mapa_rank(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Relaxed: the producer publishes no data of its own (the bytes arrive by
// TMA complete_tx); a release at cluster scope here costs about one
// round trip per stage and halves the kernel's speed.
__device__ __forceinline__ void mbar_expect_tx_remote(uint32_t caddr, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.relaxed.cluster.shared::cluster.b64 _, [%0], %1;" ::"r"(caddr), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_load_3d_pair(uint32_t dst, const CUtensorMap* map, int x, int y, int z,
                                                 uint32_t bar_caddr) {
  asm volatile(
      "cp.async.bulk.tensor.3d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
      "%4}], [%5];" ::"r"(dst),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(bar_caddr)
      : "memory");
}
__device__ __forceinline__ void umma_f16_pair(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC2), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit_pair(uint32_t bar) {
  const uint16_t mask = 0x3;
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(bar),
      "h"(mask)
      : "memory");
}
__device__ __forceinline__ void umma_commit_pair_local(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
template <class PC>
__device__ __forceinline__ uint64_t smem_desc_pair(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(PC::SBO >> 4) << 32;
  d |= 1ull << 46;
  d |= PC::LAYOUT << 61;
  return d;
}

template <class PC, bool BWD = false>
__global__ void __launch_bounds__(THREADS2, 1)
    k_pairs_tc2(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
                const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl,
                const TcParams P) {
  constexpr int TI = PC::TIP, TI2 = 2 * PC::TIP, TERM_FLOATS = PC::E::TERM_FLOATS;
  constexpr int KA2 = PC::KA2, STAGES2 = PC::STAGES2, A2_BYTES = PC::A2_BYTES, BH_BYTES = PC::BH_BYTES,
                A2_TX = PC::A2_TX, BH_TX = PC::BH_TX, STAGE2_BYTES = PC::STAGE2_BYTES,
                STAGING_BYTES = PC::E::STAGING_BYTES, EPI_BYTES = PC::EPI2_BYTES;
  // Speculative launches: every CTA reads the same flag, written by kernels
  // earlier in the stream, so both CTAs of a pair leave before any barrier.
  if (P.skip && *P.skip != 0) return;
  extern __shared__ uint8_t smem_raw[];
  // 1024-byte aligned by pointer arithmetic on the shared array itself (not
  // through an integer), so every access through it stays a shared-memory
  // access (LDS/STS), not a generic one.
  uint8_t* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  uint8_t* stage_base = smem;
  float* staging = (float*)(smem + STAGES2 * STAGE2_BYTES);
  float* terms = (float*)(smem + STAGES2 * STAGE2_BYTES + EPI_GROUPS * STAGING_BYTES);
  float* rowbuf = terms + 2 * TERM_FLOATS;
  uint64_t* bars = (uint64_t*)(smem + STAGES2 * STAGE2_BYTES + EPI_BYTES);
  // bars: full[STAGES2] empty[STAGES2] accf[2] acce[2] done; TMEM address;
  // tfull[2] tempty[2] (the staged frame terms' two buffers); verdicts.
  constexpr int kFull = 0, kEmpty = STAGES2, kAccf = 2 * STAGES2, kAcce = 2 * STAGES2 + 2, kDone = 2 * STAGES2 + 4;
  constexpr int kTfull = kDone + 3, kTempty = kDone + 5;
  static_assert((kTempty + 2) * 8 + 2 * EPI_GROUPS * 4 <= BAR2_BYTES, "barrier area");
  uint32_t* tmem_slot = (uint32_t*)(bars + kDone + 1);
  volatile int* okf = (volatile int*)(bars + kTempty + 2);  // verdicts: [group][buffer] (or [buffer])
  const uint32_t full0 = smem_u32(bars + kFull), empty0 = smem_u32(bars + kEmpty), accf0 = smem_u32(bars + kAccf),
                 acce0 = smem_u32(bars + kAcce), done = smem_u32(bars + kDone), tfull0 = smem_u32(bars + kTfull),
                 tempty0 = smem_u32(bars + kTempty);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_rank();
  const int64_t cluster = blockIdx.x >> 1, n_clusters = gridDim.x >> 1;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES2; ++s) {
      mbar_init(full0 + 8 * s, 2);   // one expect_tx arrival per CTA (used in CTA 0)
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf0 + 8 * b, 1);
      mbar_init(acce0 + 8 * b, 2 * EPI_WARPS);  // used in CTA 0
      mbar_init(tfull0 + 8 * b, 32);            // every lane of the staging warp
      mbar_init(tempty0 + 8 * b, EPI_WARPS);    // one arrival per epilogue warp
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmAh) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmAl) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmBh) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmBl) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();  // barriers of both CTAs initialised before any remote arrive
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer (both CTAs) ----------------
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 0;
      bool ok = true;
      int last_par[STAGES2];
      for (int k = 0; k < STAGES2; ++k) last_par[k] = -1;
      for (int64_t t = cluster; t < P.n_tiles && ok; t += n_clusters) {
        const int2 tl = P.tiles[t];
        const int iz = (int)(P.i_base + (int64_t)tl.x * TI2 + (int64_t)rank * TI);
        const int jz = (int)(P.tgt0 + P.jt_base + (int64_t)tl.y * TJ + (int64_t)rank * TJH);
        for (int kc = 0; kc < P.nk; ++kc) {
          if (!mbar_wait(empty0 + 8 * s, ph ^ 1u, P.err, 11)) { ok = false; break; }
          const uint32_t fb = mapa_rank(full0 + 8 * s, 0);
          if (rank == 0)
            mbar_expect_tx(full0 + 8 * s, 2 * A2_TX + 2 * BH_TX);
          else
            mbar_expect_tx_remote(fb, 2 * A2_TX + 2 * BH_TX);
          const uint32_t sb = smem_u32(stage_base + s * STAGE2_BYTES);
          tma_load_3d_pair(sb, &tmAh, kc * KA2, 0, iz, fb);
          tma_load_3d_pair(sb + A2_BYTES, &tmAl, kc * KA2, 0, iz, fb);
          tma_load_3d_pair(sb + 2 * A2_BYTES, &tmBh, kc * KA2, 0, jz, fb);
          tma_load_3d_pair(sb + 2 * A2_BYTES + BH_BYTES, &tmBl, kc * KA2, 0, jz, fb);
          last_par[s] = (int)ph;
          if (++s == STAGES2) { s = 0; ph ^= 1u; }
        }
      }
      // CTA 0 sees every copy of both CTAs complete on its full barriers.
      if (rank == 0)
        for (int k = 0; k < STAGES2; ++k)
          if (last_par[k] >= 0) mbar_wait_quiet(full0 + 8 * k, (uint32_t)last_par[k]);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer (CTA 0 only) ----------------
    if (lane == 0 && rank == 0) {
      int s = 0;
      uint32_t ph = 0;
      uint32_t it = 0;
      bool ok = true;
      for (int64_t t = cluster; t < P.n_tiles && ok; t += n_clusters, ++it) {
        const uint32_t b = it & 1u, aph = (it >> 1) & 1u;
        if (!mbar_wait(acce0 + 8 * b, aph ^ 1u, P.err, 12)) { ok = false; break; }
        tc_fence_after();
        const uint32_t d = tmem_base + b * ACC_STRIDE;
        for (int kc = 0; kc < P.nk; ++kc) {
          if (!mbar_wait(full0 + 8 * s, ph, P.err, 13)) { ok = false; break; }
          tc_fence_after();
          const uint32_t sb = smem_u32(stage_base + s * STAGE2_BYTES);
#pragma unroll
          for (int kk = 0; kk < KA2 / 16; ++kk) {
            const uint64_t ah = smem_desc_pair<PC>(sb + kk * 32), al = smem_desc_pair<PC>(sb + A2_BYTES + kk * 32);
            const uint64_t bh = smem_desc_pair<PC>(sb + 2 * A2_BYTES + kk * 32);
            const uint64_t bl = smem_desc_pair<PC>(sb + 2 * A2_BYTES + BH_BYTES + kk * 32);
            umma_f16_pair(d, ah, bh, (kc | kk) != 0);
            umma_f16_pair(d, al, bh, 1u);
            umma_f16_pair(d, ah, bl, 1u);
          }
          umma_commit_pair(empty0 + 8 * s);  // frees stage s in both CTAs
          if (++s == STAGES2) { s = 0; ph ^= 1u; }
        }
        if (!ok) break;
        umma_commit_pair(accf0 + 8 * b);
      }
      umma_commit_pair_local(done);
      mbar_wait_quiet(done, 0);
    }
  } else if (warp == 2 + EPI_WARPS) {
    // ---------------- frame-term staging (both CTAs) ----------------
    // Tile by tile, in the epilogue's order: wait until the epilogue warps
    // have released buffer b (two tiles ago), stage the tile, publish.
    uint32_t it = 0;
    for (int64_t t = cluster; t < P.n_tiles; t += n_clusters, ++it) {
      const uint32_t b = it & 1u, ph = (it >> 1) & 1u;
      if (!mbar_wait(tempty0 + 8 * b, ph ^ 1u, P.err, 16)) break;
      stage_tile_terms<typename PC::E, BWD>(P, terms + b * TERM_FLOATS, t, TI2, (int)rank * TI, true, lane, 32);
      mbar_arrive(tfull0 + 8 * b);
    }
  } else {
    // ---------------- epilogue (both CTAs) ----------------
    epilogue_tiles<typename PC::E, BWD, true>(P, tmem_base, staging, terms, rowbuf, okf, accf0, mapa_rank(acce0, 0),
                                              true, cluster, n_clusters, TI2, (int)rank * TI, warp, lane, tfull0,
                                              tempty0);
  }

  tc_fence_before();
  __syncthreads();
  cluster_sync_all();  // CTA 0's MMAs (writing both CTAs' tensor memory) have retired
  tc_fence_after();
  if (warp == 1) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(TMEM_COLS)
                 : "memory");
  }
}

// The driver's tensor-map encoder, looked up once (handles on several host
// threads may race here: the pointer is published atomically).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
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

bool make_map(CUtensorMap* m, const void* base, int64_t F, int Np, int box_frames, int ka) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3] = {(cuuint64_t)Np, 3, (cuuint64_t)F};
  cuuint64_t strides[2] = {(cuuint64_t)Np * 2, (cuuint64_t)Np * 2 * 3};
  cuuint32_t box[3] = {(cuuint32_t)ka, 3, (cuuint32_t)box_frames};
  cuuint32_t es[3] = {1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, ka == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
}  // namespace

int tc_supported(int device) {
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
  cudaGetLastError();
  return (major == 10 && minor == 3 && encode_fn() != nullptr) ? 1 : 0;
}

// The output region a tile list covers, with `rows` reference frames per
// launch tile.
static TileGrid grid_of(const OutMap& m, int rows) {
  TileGrid g{};
  if (m.tri) {
    g.i_base = m.row_begin;
    g.i_end = m.row_end;
    g.jt_base = m.row_begin;
    g.jt_end = m.n_tgt;
  } else {
    g.i_base = 0;
    g.i_end = m.n_ref;
    g.jt_base = m.row_begin;
    g.jt_end = m.row_end;
  }
  g.rows = rows;
  g.cols = TJ;
  g.tri = m.tri;
  return g;
}

// Tile list in grouped order (gbr_tiles.h).
int64_t tc_build_tiles(const OutMap& m, std::vector<int2>& tiles, int64_t& i_base, int64_t& jt_base,
                       int64_t& i_end, int64_t& jt_end, int ti_frames = TI) {
  const TileGrid g = grid_of(m, ti_frames);
  i_base = g.i_base;
  i_end = g.i_end;
  jt_base = g.jt_base;
  jt_end = g.jt_end;
  return build_tiles_grouped(g, tiles);
}

// Reference frames per CTA tile and per launch tile of each kernel shape.
static int cta_tile_rows(int variant) { return variant == 4 ? PairWide::TIP : TI; }
static int launch_tile_rows(int variant) { return variant >= 2 ? 2 * cta_tile_rows(variant) : TI; }
int tc_launch_tile_rows(int variant) { return launch_tile_rows(variant); }

int64_t tc_build_tile_list(const OutMap& m, std::vector<int2>& tiles, TcTileInfo& info, int variant) {
  return tc_build_tiles(m, tiles, info.i_base, info.jt_base, info.i_end, info.jt_end, launch_tile_rows(variant));
}

TileGrid tc_tile_grid(const OutMap& m, int variant) { return grid_of(m, launch_tile_rows(variant)); }


// Launch of the pair-of-SMs kernel: clusters of two CTAs, as many clusters
// as can be resident at once (one CTA per SM), at most one per tile.
template <class PC, bool BWD = false>
static cudaError_t launch_pair_kernel(const CUtensorMap& mAh, const CUtensorMap& mAl, const CUtensorMap& mBh,
                                      const CUtensorMap& mBl, const TcParams& P, cudaStream_t st, int cap = 0) {
  cudaError_t e =
      cudaFuncSetAttribute(k_pairs_tc2<PC, BWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, PC::SMEM2_BYTES);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(THREADS2, 1, 1);
  cfg.dynamicSmemBytes = PC::SMEM2_BYTES;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  // Resident clusters, per kernel instantiation and device (devices of one
  // process may differ in SM count); every thread computes the same value.
  constexpr int kMaxDev = 64;
  static std::atomic<int> cached_clusters[kMaxDev] = {};
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
  int max_clusters = cached_clusters[dev].load(std::memory_order_relaxed);
  if (max_clusters == 0) {
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    cfg.gridDim = dim3((unsigned)(sms & ~1), 1, 1);
    int n = 0;
    e = cudaOccupancyMaxActiveClusters(&n, k_pairs_tc2<PC, BWD>, &cfg);
    if (e != cudaSuccess) return e;
    if (n < 1) return cudaErrorInvalidConfiguration;
    max_clusters = n;
    cached_clusters[dev].store(n, std::memory_order_relaxed);
  }
  // cap > 0: at most cap clusters; cap < 0: leave -cap of the resident clusters free
  int64_t nc = std::min<int64_t>(P.n_tiles, (int64_t)max_clusters);
  if (cap > 0) nc = std::min<int64_t>(nc, cap);
  if (cap < 0) nc = std::min<int64_t>(nc, std::max<int64_t>(1, (int64_t)max_clusters + cap));
  cfg.gridDim = dim3((unsigned)(2 * nc), 1, 1);
  return cudaLaunchKernelEx(&cfg, k_pairs_tc2<PC, BWD>, mAh, mAl, mBh, mBl, P);
}

cudaError_t run_pairs_tc(const TcLaunch& L, cudaStream_t st) {
  std::vector<int2> tiles;
  int64_t i_base, jt_base, i_end, jt_end;
  int64_t n;
  cudaError_t e = cudaSuccess;
  const bool pair = (L.variant >= 2);
  const int ti_frames = launch_tile_rows(L.variant);
  if (L.ready_tiles > 0) {
    // The caller uploaded the list already (batched, graph-captured and
    // input-overlap paths).
    const TileGrid g = grid_of(L.map, ti_frames);
    i_base = g.i_base;
    jt_base = g.jt_base;
    i_end = g.i_end;
    jt_end = g.jt_end;
    n = L.ready_tiles;
  } else {
    n = tc_build_tiles(L.map, tiles, i_base, jt_base, i_end, jt_end, ti_frames);
    if (n == 0) return cudaSuccess;
    if (!L.tile_buf || n > L.tile_cap) return cudaErrorInvalidValue;
    if (L.tile_stage) {
      std::memcpy(L.tile_stage, tiles.data(), sizeof(int2) * n);
      e = cudaMemcpyAsync(L.tile_buf, L.tile_stage, sizeof(int2) * n, cudaMemcpyHostToDevice, st);
    } else {
      // From pageable memory cudaMemcpyAsync returns after the source has
      // been consumed, so `tiles` may go out of scope.
      e = cudaMemcpyAsync(L.tile_buf, tiles.data(), sizeof(int2) * n, cudaMemcpyHostToDevice, st);
    }
    if (e != cudaSuccess) return e;
  }
  const int ka = (L.variant == 0)   ? 64
                 : (L.variant == 1) ? 32
                 : (L.variant == 3) ? PairDeep::KA2
                 : (L.variant == 4) ? PairWide::KA2
                                    : PairShallow::KA2;
  const int bj = pair ? TJH : TJ;
  CUtensorMap mAh, mAl, mBh, mBl;
  const int bi = cta_tile_rows(L.variant);
  if (!make_map(&mAh, L.hi, L.F, L.Np, bi, ka) || !make_map(&mAl, L.lo, L.F, L.Np, bi, ka) ||
      !make_map(&mBh, L.hi, L.F, L.Np, bj, ka) || !make_map(&mBl, L.lo, L.F, L.Np, bj, ka))
    return cudaErrorInvalidValue;
  TcParams P{};
  P.tiles = (const int2*)L.tile_buf;
  P.n_tiles = n;
  P.i_base = i_base;
  P.jt_base = jt_base;
  P.i_end = i_end;
  P.jt_end = jt_end;
  P.tgt0 = L.tgt0;
  P.nk = (L.N + ka - 1) / ka;
  P.inv_scale = L.inv_scale;
  P.terms = L.terms;
  P.map = L.map;
  P.flags = L.flags;
  P.err = L.dev_error;
  P.row_stores = L.row_stores;
  P.skip = L.skip;
  if (L.bwd) {  // the backward instantiation exists for the pair-of-SMs kernels only
    if (!pair) return cudaErrorInvalidValue;
    P.bwd = *L.bwd;
    P.row_stores = 0;
    // (the wide-chunk shape has no backward instantiation: same stages as the shallow one)
    e = (L.variant == 3) ? launch_pair_kernel<PairDeep, true>(mAh, mAl, mBh, mBl, P, st)
                         : launch_pair_kernel<PairShallow, true>(mAh, mAl, mBh, mBl, P, st);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
  }
  if (pair) {
    e = (L.variant == 3)   ? launch_pair_kernel<PairDeep>(mAh, mAl, mBh, mBl, P, st, L.cluster_cap)
        : (L.variant == 4) ? launch_pair_kernel<PairWide>(mAh, mAl, mBh, mBl, P, st, L.cluster_cap)
                           : launch_pair_kernel<PairShallow>(mAh, mAl, mBh, mBl, P, st, L.cluster_cap);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
  }
  const int grid = (int)std::min<int64_t>(n, L.num_sms > 0 ? L.num_sms : 148);
  if (ka == 64) {
    e = cudaFuncSetAttribute(k_pairs_tc<Pipe<64>>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    k_pairs_tc<Pipe<64>><<<grid, THREADS, SMEM_BYTES, st>>>(mAh, mAl, mBh, mBl, P);
  } else {
    e = cudaFuncSetAttribute(k_pairs_tc<Pipe<32>>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    k_pairs_tc<Pipe<32>><<<grid, THREADS, SMEM_BYTES, st>>>(mAh, mAl, mBh, mBl, P);
  }
  return cudaGetLastError();
}

int64_t tc_max_tiles(const OutMap& m) {
  int64_t ni, nj;
  if (m.tri) {
    ni = m.row_end - m.row_begin;
    nj = m.n_tgt - m.row_begin;
  } else {
    ni = m.n_ref;
    nj = m.row_end - m.row_begin;
  }
  // the smallest tile of any shape (the wide one's TI_WIDE reference frames)
  return ((ni + TI_WIDE - 1) / TI_WIDE) * ((nj + TJ - 1) / TJ);
}

}  // namespace gbr
