// gbr_batch.cu -- gbr_allpairs_batched: many independent rms2d runs in one call.
//
// Each trajectory is a single-set TRI problem (as Analysis_Rms2d::Calculate_2D
// with equal masks, src/Analysis_Rms2d.cpp:196-295) with its own frame and atom
// counts.  The call
//   1. lays out one workspace slice per trajectory and uploads masses and the
//      tensor-core tile lists (through pinned staging) -- the only host work;
//   2. picks a kernel per trajectory from the autotuner table, keyed by
//      (log2 frames, log2 atoms): tcgen05 with 64- or 32-atom stages, or the
//      FP32 CUDA-core kernel (both meet the same error bound); unseen shape
//      buckets are timed once on their first trajectory;
//   3. enqueues every trajectory's passes -- centring, one pre-alignment
//      reference (no host synchronisation), operand planes, pair kernel, and an
//      FP64 fix-up whose length is read on the device -- round-robin over 8
//      streams forked from the handle's stream;
//   4. when every pointer is device memory, captures step 3 as a CUDA graph
//      and replays it while the batch signature (shapes, pointers, masses,
//      workspace) stays the same;
//   5. synchronises once and checks the device error flags and fix-up counts.
// Batched problems use one pre-alignment reference per trajectory; frames far
// from it are caught by the error bound and recomputed in FP64.
#include <cuda_fp16.h>

#include <chrono>
#include <cmath>
#include <cstring>

#include "gbr_handle.h"

using namespace gbr;

namespace {

// Kernel per trajectory: the one-SM tensor-core kernel (64- or 32-atom stages),
// the pair-of-SMs tensor-core kernel (shallow or deep stages), the FP32
// CUDA-core kernel, or FP64 for every pair.
enum Choice { kTC64 = 0, kTC32 = 1, kFP32 = 2, kFP64 = 3, kTCPairS = 4, kTCPairD = 5, kTCPairW = 6 };
bool is_tc(int c) { return c == kTC64 || c == kTC32 || c == kTCPairS || c == kTCPairD || c == kTCPairW; }
int tc_variant_of(int c) { return c == kTC64 ? 0 : c == kTC32 ? 1 : c == kTCPairS ? 2 : c == kTCPairW ? 4 : 3; }

struct Prob {
  int64_t F = 0;
  int N = 0, Np = 0;
  int choice = kFP32;
  double W = 0.0;
  bool weighted = false;
  const float* xyz = nullptr;  // caller
  float* out = nullptr;        // caller
  int64_t n_out = 0;
  unsigned long long cap = 0;
  int64_t n_tiles = 0;
  size_t tile_off = 0;         // offset of this problem's tiles in the pinned staging
  // workspace
  float* d_xyz = nullptr;
  double* d_w = nullptr;
  double* cen = nullptr;
  int64_t* fsel = nullptr;
  float* dmax = nullptr;
  float* dist = nullptr;
  int* assign = nullptr;
  double* refs = nullptr;
  float* swr = nullptr;
  double* Eref = nullptr;
  float* plane = nullptr;
  float* inv_scale = nullptr;
  float* nrm = nullptr;
  float* P = nullptr;
  float* trP = nullptr;
  float* RP = nullptr;
  int2* flags = nullptr;
  float* d_out = nullptr;
  void* hi = nullptr;
  void* lo = nullptr;
  int2* tiles = nullptr;
  float* mean = nullptr;
  float* partial = nullptr;
  double* sqw = nullptr;
  float* sqwf = nullptr;
  int* order = nullptr;
  int* offsets = nullptr;
  void* scratch = nullptr;
};

void layout_prob(Arena& A, Prob& p, bool host_in, bool host_out) {
  const size_t F = (size_t)p.F, N = (size_t)p.N, Np = (size_t)p.Np;
  const bool tc = is_tc(p.choice);
  const bool planes = (p.choice != kFP64);
  p.d_xyz = host_in ? A.take<float>(F * 3 * N) : nullptr;
  p.d_w = A.take<double>(N);
  p.cen = A.take<double>(3 * F);
  p.fsel = A.take<int64_t>(1);
  p.dmax = A.take<float>(1);
  p.dist = A.take<float>(F);
  p.assign = A.take<int>(F);
  p.refs = A.take<double>(3 * N);
  p.swr = A.take<float>(3 * N);
  p.Eref = A.take<double>(1);
  p.plane = (planes && !tc) ? A.take<float>(F * 3 * Np) : nullptr;
  p.inv_scale = A.take<float>(F);
  p.nrm = A.take<float>(F);
  p.P = A.take<float>(9 * F);
  p.trP = A.take<float>(F);
  p.RP = A.take<float>(kRefPairStride);
  p.flags = A.take<int2>(p.cap);
  p.d_out = host_out ? A.take<float>((size_t)p.n_out) : nullptr;
  p.hi = tc ? (void*)A.take<__half_raw>(F * 3 * Np) : nullptr;
  p.lo = tc ? (void*)A.take<__half_raw>(F * 3 * Np) : nullptr;
  p.tiles = tc ? A.take<int2>((size_t)p.n_tiles) : nullptr;
  p.mean = planes ? A.take<float>(3 * Np) : nullptr;
  p.partial = planes ? A.take<float>(64 * 3 * Np) : nullptr;
  p.sqw = A.take<double>(N);
  p.sqwf = A.take<float>(N);
  p.order = A.take<int>(F);
  p.offsets = A.take<int>(2);
  p.scratch = planes ? A.take<char>(prep_scratch_bytes(p.F, p.N, 1)) : nullptr;
}

OutMap tri_map(const Prob& p, float* out) {
  OutMap m{};
  m.out = out;
  m.n_ref = p.F;
  m.n_tgt = p.F;
  m.tgt0 = 0;
  m.tri = 1;
  m.row_begin = 0;
  m.row_end = p.F;
  m.base = 0;
  return m;
}

// Every pass of one problem, on one stream, with no host synchronisation.
cudaError_t enqueue_prob(gbr_handle* h, Prob& p, int mode, bool host_in, bool host_out,
                         unsigned long long* count, int* derr, cudaStream_t st, int* launches = nullptr) {
  cudaError_t e;
  int nl = 0;
  const bool nofit = (mode == GBR_NOFIT);
  if (host_in) {
    e = cudaMemcpyAsync(p.d_xyz, p.xyz, sizeof(float) * 3 * p.N * p.F, cudaMemcpyDefault, st);
    if (e != cudaSuccess) return e;
  }
  const float* xyz = host_in ? p.d_xyz : p.xyz;
  float* out = host_out ? p.d_out : p.out;
  const double* w = p.weighted ? p.d_w : nullptr;
  PrepArgs pa{};
  pa.dtype_f64 = 0;
  pa.ref = xyz;
  pa.tgt = nullptr;
  pa.n_ref = p.F;
  pa.F = p.F;
  pa.N = p.N;
  pa.Np = p.Np;
  pa.nofit = nofit;
  pa.centroid_only = (p.choice == kFP64);
  pa.cmass_ref = pa.cmass_tgt = pa.w = w;
  pa.Wsum = p.W;
  pa.tau = 1e30;
  pa.max_refs = 1;
  pa.cen = p.cen;
  pa.fsel = p.fsel;
  pa.dmax = p.dmax;
  pa.dist = p.dist;
  pa.assign = p.assign;
  pa.refs = p.refs;
  pa.swr = p.swr;
  pa.Eref = p.Eref;
  pa.rot = nullptr;
  pa.plane = p.plane;
  pa.order = p.order;
  pa.offsets = p.offsets;
  pa.mean = p.mean;
  pa.partial = p.partial;
  pa.sqw = p.sqw;
  pa.sqwf = p.sqwf;
  pa.scratch = p.scratch;
  pa.RP = p.RP;
  PrepOut po;
  if ((e = run_prep(pa, po, st)) != cudaSuccess) return e;
  nl += po.launches;
  const OutMap map = tri_map(p, out);
  ExactLaunch ex{};
  ex.dtype_f64 = 0;
  ex.ref = xyz;
  ex.tgt = nullptr;
  ex.n_ref = p.F;
  ex.N = p.N;
  ex.cen = p.cen;
  ex.w = w;
  ex.Wsum = p.W;
  ex.nofit = nofit;
  ex.tgt0 = 0;
  ex.map = map;
  if (p.choice == kFP64) {
    ex.list = nullptr;
    ex.count = p.n_out;
    e = run_exact(ex, st);
    ++nl;
  } else {
    const bool tc = (p.choice != kFP32);
    FrameTerms terms{};
    terms.assign = p.assign;
    terms.nrm = p.nrm;
    terms.P = p.P;
    terms.trP = p.trP;
    terms.RP = p.RP;
    terms.K = 1;
    terms.W = (float)p.W;
    terms.two_over_w = (float)(2.0 / (double)p.W);
    terms.tol = (float)h->tol;
    terms.gem_s = tc ? 6.0e-7f : 1.2e-7f;
    terms.gem_c = tc ? 1.2e-8f * (float)p.N : 1.2e-7f * std::sqrt((float)p.N);
    terms.epi_coef = 8e-7f;
    terms.nofit = nofit;
    FinishArgs fa{};
    fa.prep = &pa;
    fa.plane = p.plane;
    fa.F = p.F;
    fa.N = p.N;
    fa.Np = p.Np;
    fa.K = 1;
    fa.mean = p.mean;
    fa.assign = p.assign;
    fa.swr = p.swr;
    fa.tc = tc;
    fa.hi = p.hi;
    fa.lo = p.lo;
    fa.inv_scale = p.inv_scale;
    fa.write_plane = !tc;
    fa.nrm = p.nrm;
    fa.P = p.P;
    fa.trP = p.trP;
    fa.refs = p.refs;
    fa.w = w;
    fa.nofit = nofit;
    fa.RP = p.RP;
    fa.self_terms = po.self_terms;
    if ((e = run_finish(fa, st)) != cudaSuccess) return e;
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
    cudaMemsetAsync(derr, 0, sizeof(int), st);
    FlagList fl{p.flags, count, p.cap};
    if (tc) {
      TcLaunch L{};
      L.hi = p.hi;
      L.lo = p.lo;
      L.tile_buf = p.tiles;
      L.tile_cap = p.n_tiles;
      L.ready_tiles = p.n_tiles;
      L.F = p.F;
      L.Np = p.Np;
      L.N = p.N;
      L.tgt0 = 0;
      L.inv_scale = p.inv_scale;
      L.terms = terms;
      L.map = map;
      L.flags = fl;
      L.dev_error = derr;
      L.num_sms = h->num_sms;
      L.variant = tc_variant_of(p.choice);
      L.row_stores = 0;  // the triangle is in device memory (caller's or staging)
      if (p.n_tiles > 0 && (e = run_pairs_tc(L, st)) != cudaSuccess) return e;
    } else {
      PairLaunch L{};
      L.plane = p.plane;
      L.Np = p.Np;
      L.N = p.N;
      L.tgt0 = 0;
      L.terms = terms;
      L.map = map;
      L.flags = fl;
      L.tiles = make_tiles(map, 64, 64);
      if ((e = run_pairs_fp32(L, st)) != cudaSuccess) return e;
    }
    ex.list = p.flags;
    ex.count = (int64_t)p.cap;
    ex.dev_count = count;
    e = run_exact(ex, st);
    nl += po.self_terms ? 3 : 4;  // finish, reference-pair table (unless prep wrote it), pair kernel, fix-up
  }
  if (e != cudaSuccess) return e;
  if (launches) *launches += nl;
  if (host_out) e = cudaMemcpyAsync(p.out, p.d_out, sizeof(float) * p.n_out, cudaMemcpyDefault, st);
  return e;
}

int log2i(int64_t v) {
  int k = 0;
  while (v > 1) { v >>= 1; ++k; }
  return k;
}

}  // namespace

extern "C" int gbr_allpairs_batched(gbr_handle* h, int32_t n_traj, const float* const* xyz,
                                    const int64_t* n_frames, const int32_t* n_atoms,
                                    const double* const* mass, int mode, int precision, float* const* out) {
  if (!h) return GBR_ERR_ARG;
  h->err.clear();
  h->stats = gbr_stats{};
  const auto t_start = std::chrono::steady_clock::now();
  if (n_traj < 0 || (n_traj > 0 && (!xyz || !n_frames || !n_atoms || !out)))
    return h->fail(GBR_ERR_ARG, "batched: null array argument");
  if (mode != GBR_FIT && mode != GBR_NOFIT) return h->fail(GBR_ERR_ARG, "mode must be GBR_FIT or GBR_NOFIT");
  if (precision < GBR_PREC_FP32 || precision > GBR_PREC_FP64) return h->fail(GBR_ERR_ARG, "bad precision");
  if (precision == GBR_PREC_TC && !h->tc_ok)
    return h->fail(GBR_ERR_UNSUPPORTED, "tensor-core precision needs an sm_103 (GB300) device");
  if (cudaSetDevice(h->device) != cudaSuccess) return h->cuda_fail(cudaGetLastError(), "cudaSetDevice");
  if (!h->ensure_aux()) return h->fail(GBR_ERR_CUDA, "cannot create batch streams");
  cudaError_t e;

  // ---- per-problem sizes, masses, pointer kinds ----
  std::vector<Prob> probs(n_traj);
  bool host_in = false, host_out = false, any = false;
  std::vector<std::vector<double>> masses(n_traj);
  for (int t = 0; t < n_traj; ++t) {
    Prob& p = probs[t];
    p.F = n_frames[t];
    p.N = n_atoms[t];
    if (p.F < 0 || p.F > INT32_MAX) return h->fail(GBR_ERR_ARG, "trajectory %d: bad frame count", t);
    if (p.N < 1) return h->fail(GBR_ERR_ARG, "trajectory %d: n_atom must be >= 1", t);
    if (!xyz[t] || !out[t]) return h->fail(GBR_ERR_ARG, "trajectory %d: null pointer", t);
    if (int rc = h->check_local({xyz[t], out[t]}, "batched")) return rc;
    p.Np = (p.N + 63) / 64 * 64;
    p.xyz = xyz[t];
    p.out = out[t];
    p.n_out = p.F * (p.F - 1) / 2;
    const bool dev_in = is_device_ptr(xyz[t]), dev_out = is_device_ptr(out[t]);
    if (!any) {
      host_in = !dev_in;
      host_out = !dev_out;
      any = true;
    } else if (host_in == dev_in || host_out == dev_out) {
      return h->fail(GBR_ERR_ARG, "batched: all coordinate (and all output) pointers must be of one kind");
    }
    const double* m = mass ? mass[t] : nullptr;
    p.weighted = (m != nullptr);
    p.W = p.N;
    if (m) {
      masses[t].resize(p.N);
      if (cudaMemcpy(masses[t].data(), m, sizeof(double) * p.N, cudaMemcpyDefault) != cudaSuccess)
        return h->cuda_fail(cudaGetLastError(), "reading masses");
      p.W = 0.0;
      for (double v : masses[t]) p.W += v;
    }
    if (p.W < 1e-14) return h->fail(GBR_ERR_ZERO_MASS, "trajectory %d: total mass below 1e-14", t);
    p.cap = (unsigned long long)std::min<int64_t>(std::max<int64_t>(p.n_out, 1), 1 << 20);
  }

  // ---- kernel choice (autotuner table) ----
  auto candidates = [&](const Prob& p) {
    std::vector<int> c;
    if (precision == GBR_PREC_FP64) return std::vector<int>{kFP64};
    if (precision == GBR_PREC_FP32) return std::vector<int>{kFP32};
    c = {kTC32, kTC64, kFP32};
    // the pair kernel's tile holds 84 reference frames: worth timing when a
    // trajectory fills at least one such tile row
    if (p.F >= 84) {
      c.push_back(kTCPairS);
      c.push_back(kTCPairD);
      c.push_back(kTCPairW);
    }
    return c;
  };
  std::vector<int> to_tune;
  for (int t = 0; t < n_traj; ++t) {
    Prob& p = probs[t];
    auto c = candidates(p);
    if (c.size() == 1 || p.F < 2) {
      p.choice = c[0];
      continue;
    }
    auto key = std::make_pair(log2i(p.F), log2i(p.N));
    auto it = h->tuned.find(key);
    if (it != h->tuned.end()) {
      p.choice = it->second;
    } else {
      p.choice = -1;
      to_tune.push_back(t);
    }
  }

  // Tile lists (tensor-core choices) in pinned staging.
  auto plan_tiles = [&](std::vector<int2>& all) {
    all.clear();
    for (auto& p : probs) {
      p.n_tiles = 0;
      if (is_tc(p.choice)) {
        std::vector<int2> tl;
        TcTileInfo info;
        p.n_tiles = tc_build_tile_list(tri_map(p, nullptr), tl, info, tc_variant_of(p.choice));
        p.tile_off = all.size();
        all.insert(all.end(), tl.begin(), tl.end());
      }
    }
  };
  auto plan_workspace = [&]() -> int {
    Arena sizing;
    sizing.take<unsigned long long>(n_traj);
    sizing.take<int>(n_traj);
    for (auto& p : probs) layout_prob(sizing, p, host_in, host_out);
    if (!h->reserve(sizing.off + 256))
      return h->fail(GBR_ERR_NOMEM, "cannot allocate %.2f GB of device workspace", (sizing.off + 256) / 1e9);
    return GBR_OK;
  };
  unsigned long long* counts = nullptr;
  int* derrs = nullptr;
  auto carve = [&]() {
    Arena A{h->ws, 0};
    counts = A.take<unsigned long long>(n_traj);
    derrs = A.take<int>(n_traj);
    for (auto& p : probs) layout_prob(A, p, host_in, host_out);
  };
  auto upload = [&](const std::vector<int2>& tiles) -> int {
    size_t mass_doubles = 0;
    for (int t = 0; t < n_traj; ++t) mass_doubles += masses[t].size();
    const size_t bytes = sizeof(int2) * tiles.size() + sizeof(double) * mass_doubles + 64;
    if (!h->reserve_pinned(bytes)) return h->fail(GBR_ERR_NOMEM, "cannot allocate pinned staging");
    // previous uses of the staging buffer are complete: every call synchronises before returning
    std::memcpy(h->pinned, tiles.data(), sizeof(int2) * tiles.size());
    double* md = (double*)((char*)h->pinned + ((sizeof(int2) * tiles.size() + 15) & ~size_t(15)));
    size_t off = 0;
    for (int t = 0; t < n_traj; ++t) {
      Prob& p = probs[t];
      if (p.n_tiles > 0)
        cudaMemcpyAsync(p.tiles, (const int2*)h->pinned + p.tile_off, sizeof(int2) * p.n_tiles,
                        cudaMemcpyHostToDevice, h->stream);
      if (!masses[t].empty()) {
        std::memcpy(md + off, masses[t].data(), sizeof(double) * p.N);
        cudaMemcpyAsync(p.d_w, md + off, sizeof(double) * p.N, cudaMemcpyHostToDevice, h->stream);
        off += p.N;
      }
    }
    return GBR_OK;
  };

  // ---- autotune unseen shape buckets: time each candidate on one problem ----
  if (!to_tune.empty()) {
    std::map<std::pair<int, int>, int> first;
    for (int t : to_tune) first.emplace(std::make_pair(log2i(probs[t].F), log2i(probs[t].N)), t);
    for (auto& kv : first) {
      const int t = kv.second;
      float best_ms = 1e30f;
      int best = kFP32;
      for (int cand : candidates(probs[t])) {
        for (auto& p : probs) if (p.choice < 0) p.choice = kFP32;  // placeholder for sizing
        probs[t].choice = cand;
        std::vector<int2> tiles;
        plan_tiles(tiles);
        int rc = plan_workspace();
        if (rc != GBR_OK) return rc;
        carve();
        if ((rc = upload(tiles)) != GBR_OK) return rc;
        float ms = 0.0f;
        for (int rep = 0; rep < 2; ++rep) {
          cudaEventRecord(h->ev[0], h->stream);
          e = enqueue_prob(h, probs[t], mode, host_in, host_out, counts + t, derrs + t, h->stream);
          if (e != cudaSuccess) return h->cuda_fail(e, "autotune");
          cudaEventRecord(h->ev[1], h->stream);
          if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return h->cuda_fail(e, "autotune");
          cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
        }
        if (ms < best_ms) {
          best_ms = ms;
          best = cand;
        }
      }
      h->tuned[kv.first] = best;
    }
    for (int t : to_tune) probs[t].choice = h->tuned[std::make_pair(log2i(probs[t].F), log2i(probs[t].N))];
  }

  // ---- final plan, staging ----
  std::vector<int2> tiles;
  plan_tiles(tiles);
  int rc = plan_workspace();
  if (rc != GBR_OK) return rc;
  carve();
  if ((rc = upload(tiles)) != GBR_OK) return rc;

  // ---- enqueue: graph replay when the signature repeats, capture otherwise ----
  std::vector<unsigned long long> sig = {(unsigned long long)n_traj, (unsigned long long)mode,
                                         (unsigned long long)precision, (unsigned long long)(uintptr_t)h->ws,
                                         (unsigned long long)(uintptr_t)h->stream};
  for (int t = 0; t < n_traj; ++t) {
    const Prob& p = probs[t];
    unsigned long long mh = 0;
    for (double v : masses[t]) {
      unsigned long long b;
      std::memcpy(&b, &v, sizeof b);
      mh = mh * 1000003ull ^ b;
    }
    sig.insert(sig.end(), {(unsigned long long)p.F, (unsigned long long)p.N, (unsigned long long)(uintptr_t)p.xyz,
                           (unsigned long long)(uintptr_t)p.out, (unsigned long long)p.choice, mh,
                           (unsigned long long)p.weighted});
  }
  const bool graphable = !host_in && !host_out;
  int launches = 0;
  auto enqueue_all = [&](cudaStream_t origin) -> cudaError_t {
    launches = 0;
    cudaEventRecord(h->fork, origin);
    for (int s = 0; s < gbr_handle::kAux; ++s) cudaStreamWaitEvent(h->aux[s], h->fork, 0);
    for (int t = 0; t < n_traj; ++t) {
      if (probs[t].F < 2) continue;
      cudaError_t err = enqueue_prob(h, probs[t], mode, host_in, host_out, counts + t, derrs + t,
                                     h->aux[t % gbr_handle::kAux], &launches);
      if (err != cudaSuccess) return err;
    }
    for (int s = 0; s < gbr_handle::kAux; ++s) {
      cudaEventRecord(h->join[s], h->aux[s]);
      cudaStreamWaitEvent(origin, h->join[s], 0);
    }
    return cudaGetLastError();
  };
  bool used_graph = false;
  if (graphable && h->graph_exec && sig == h->graph_sig) {
    used_graph = (cudaGraphLaunch(h->graph_exec, h->stream) == cudaSuccess);
    launches = h->graph_launches;
  } else if (graphable) {
    if (h->graph_exec) {
      cudaGraphExecDestroy(h->graph_exec);
      h->graph_exec = nullptr;
      h->graph_sig.clear();
    }
    // The uploads above must land before capture starts on the same stream.
    if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return h->cuda_fail(e, "staging");
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const cudaError_t qe = enqueue_all(h->stream);
      const cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
      if (qe == cudaSuccess && ce == cudaSuccess && graph &&
          cudaGraphInstantiate(&h->graph_exec, graph, 0) == cudaSuccess) {
        h->graph_sig = sig;
        h->graph_launches = launches;
        used_graph = (cudaGraphLaunch(h->graph_exec, h->stream) == cudaSuccess);
      }
      if (graph) cudaGraphDestroy(graph);
    }
    cudaGetLastError();  // a failed capture leaves an error state: fall back to direct launches
  }
  if (!used_graph) {
    if ((e = enqueue_all(h->stream)) != cudaSuccess) return h->cuda_fail(e, "batched enqueue");
  }
  std::vector<unsigned long long> cnt(n_traj, 0);
  std::vector<int> de(n_traj, 0);
  if (n_traj > 0) {
    cudaMemcpyAsync(cnt.data(), counts, sizeof(unsigned long long) * n_traj, cudaMemcpyDeviceToHost, h->stream);
    cudaMemcpyAsync(de.data(), derrs, sizeof(int) * n_traj, cudaMemcpyDeviceToHost, h->stream);
  }
  if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return h->cuda_fail(e, "batched");
  int64_t fixed = 0, pairs = 0;
  for (int t = 0; t < n_traj; ++t) {
    Prob& p = probs[t];
    pairs += p.n_out;
    if (p.choice == kFP64 || p.F < 2) continue;
    if (de[t] != 0) return h->fail(GBR_ERR_DEVICE, "trajectory %d: pair kernel reported device error %d", t, de[t]);
    fixed += (int64_t)std::min<unsigned long long>(cnt[t], (unsigned long long)p.n_out);
    if (cnt[t] > p.cap) {
      // more flagged pairs than the list holds: recompute this trajectory exactly
      p.choice = kFP64;
      if ((e = enqueue_prob(h, p, mode, host_in, host_out, counts + t, derrs + t, h->stream)) != cudaSuccess ||
          (e = cudaStreamSynchronize(h->stream)) != cudaSuccess)
        return h->cuda_fail(e, "batched exact rerun");
    }
  }
  h->stats.pairs = pairs;
  h->stats.pairs_fixed = fixed;
  h->stats.n_refs = 1;
  h->stats.precision = precision;
  h->stats.kernel_launches = launches;
  h->last_batch_graph = used_graph;
  h->stats.ms_total =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  return GBR_OK;
}
