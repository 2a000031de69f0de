// gbr_handle.h -- the library handle and small host helpers shared by the
// C-ABI files (gbr_capi.cu, gbr_batch.cu).  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gbrmsd.h"
#include "gbr_internal.h"

namespace gbr {

// Sub-allocator over one device buffer: a sizing pass (base == nullptr)
// followed by a carving pass with the same sequence of take() calls.
struct Arena {
  char* base = nullptr;
  size_t off = 0;
  template <class T>
  T* take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
    off += n * sizeof(T);
    return p;
  }
};

inline bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

inline bool is_pinned_or_device(const void* p) {
  if (!p) return true;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type != cudaMemoryTypeUnregistered;
}

// Reads n doubles the caller passed (masses) into host memory: a plain copy
// from host memory, pinned or not, and a synchronous copy from device memory.
inline bool read_host_doubles(double* dst, const void* src, int n) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, src) != cudaSuccess) {
    cudaGetLastError();
    at.type = cudaMemoryTypeUnregistered;
  }
  if (at.type == cudaMemoryTypeUnregistered || at.type == cudaMemoryTypeHost) {
    std::memcpy(dst, src, sizeof(double) * (size_t)n);
    return true;
  }
  return cudaMemcpy(dst, src, sizeof(double) * (size_t)n, cudaMemcpyDefault) == cudaSuccess;
}

}  // namespace gbr

struct gbr_handle {
  int device = 0;
  cudaStream_t stream = nullptr;      // stream in use
  cudaStream_t own_stream = nullptr;  // created with the handle
  std::string err;
  gbr_stats stats{};
  double tau = 6.0;
  int max_refs = 32;
  // Frames and atoms of the last call whose reference count was decided,
  // and whether it needed several references: a call of the same shape then
  // decides on the host at once rather than assuming one reference on the
  // device and running again.
  int64_t last_F = -1;
  int last_N = -1;
  bool last_multi = false;
  double tol = 5e-5;
  bool timing = false;
  char* ws = nullptr;
  size_t ws_cap = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  int num_sms = 0;
  int tc_ok = 0;
  int tc_variant = -1;  // -1: pairs of SMs, stage shape chosen by atom count (see gbr_set_option)
  bool host_out_direct = true;  // kernels store into pinned host output in place
  bool input_overlap = true;    // the contraction starts on input chunks that have landed
  int64_t band_floats = 0;      // gbr_write_cmatrix's band size (0: the streaming default)
  // batched path: auxiliary streams, fork/join events, pinned staging,
  // the captured graph of the last batch signature, the autotuner table
  static constexpr int kAux = 8;
  cudaStream_t aux[kAux] = {};
  cudaEvent_t fork = nullptr, join[kAux] = {};
  void* pinned = nullptr;
  size_t pinned_cap = 0;
  std::vector<unsigned long long> graph_sig;
  // Host scratch of the input-overlap tile grouping, reused across calls.
  std::vector<int2> tile_sorted;
  std::vector<int64_t> tile_scratch;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_launches = 0;
  bool last_batch_graph = false;
  std::map<std::pair<int, int>, int> tuned;  // (log2 F, log2 N) -> kernel choice
  // device buffer for results that leave through the host (cluster-matrix files)
  float* outbuf = nullptr;
  size_t outbuf_cap = 0;
  // copies that overlap one call's compute (input chunks in, output bands out)
  cudaStream_t xfer = nullptr;
  // 0-7 input chunks, 8-13 output bands, 14-17 streamed bands (computed, copied), 21-23 joins
  static constexpr int kXev = 24;
  cudaEvent_t xev[kXev] = {};
  // Input overlap: the chunk passes run on their own stream, so that the
  // early contraction stages queued on the caller's stream (on a capped
  // number of SMs) do not hold them back; pev: one per chunk, fork, join.
  cudaStream_t prep_stream = nullptr;
  static constexpr int kPev = 16;
  cudaEvent_t pev[kPev] = {};

  int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = buf;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* where) {
    return fail(GBR_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
  }
  // GBR_ERR_ARG when a buffer the kernels access in place is device memory of
  // another GPU than this handle's (they would reach it without peer access).
  // Host and managed memory pass; NULL entries are skipped.
  int check_local(std::initializer_list<const void*> ps, const char* what) {
    for (const void* p : ps) {
      if (!p) continue;
      cudaPointerAttributes at{};
      if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        continue;
      }
      if (at.type == cudaMemoryTypeDevice && at.device != device)
        return fail(GBR_ERR_ARG, "%s: a buffer is on device %d, this handle runs on device %d", what, at.device,
                    device);
    }
    return GBR_OK;
  }
  bool reserve(size_t bytes) {
    if (bytes <= ws_cap) return true;
    if (graph_exec) {  // a captured graph points into the old workspace
      cudaGraphExecDestroy(graph_exec);
      graph_exec = nullptr;
      graph_sig.clear();
    }
    if (ws) cudaFree(ws);
    ws = nullptr;
    ws_cap = 0;
    if (cudaMalloc(&ws, bytes) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    ws_cap = bytes;
    return true;
  }
  // Device memory for a result bound for pinned host memory that the kernels
  // cannot store across the link efficiently (grown on demand, kept).
  void* ostage = nullptr;
  size_t ostage_cap = 0;
  bool reserve_ostage(size_t bytes) {
    if (bytes <= ostage_cap) return true;
    if (ostage) cudaFree(ostage);
    ostage = nullptr;
    ostage_cap = 0;
    if (cudaMalloc(&ostage, bytes) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    ostage_cap = bytes;
    return true;
  }
  bool reserve_pinned(size_t bytes) {
    if (bytes <= pinned_cap) return true;
    if (pinned) cudaFreeHost(pinned);
    pinned = nullptr;
    pinned_cap = 0;
    if (cudaHostAlloc(&pinned, bytes, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    pinned_cap = bytes;
    return true;
  }
  bool ensure_aux() {
    if (fork) return true;
    for (int s = 0; s < kAux; ++s) {
      if (cudaStreamCreateWithFlags(&aux[s], cudaStreamNonBlocking) != cudaSuccess) return false;
      if (cudaEventCreateWithFlags(&join[s], cudaEventDisableTiming) != cudaSuccess) return false;
    }
    return cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) == cudaSuccess;
  }
  bool ensure_xfer() {
    if (xfer) return true;
    if (cudaStreamCreateWithFlags(&xfer, cudaStreamNonBlocking) != cudaSuccess) {
      xfer = nullptr;
      return false;
    }
    for (auto& e : xev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return false;
    return true;
  }
  bool ensure_prep_stream() {
    if (prep_stream) return true;
    if (cudaStreamCreateWithFlags(&prep_stream, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      prep_stream = nullptr;
      return false;
    }
    for (auto& e : pev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return false;
    return true;
  }
  bool reserve_out(size_t floats) {
    if (floats <= outbuf_cap) return true;
    if (outbuf) cudaFree(outbuf);
    outbuf = nullptr;
    outbuf_cap = 0;
    if (cudaMalloc(&outbuf, floats * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    outbuf_cap = floats;
    return true;
  }
  void release_batch() {
    if (outbuf) cudaFree(outbuf);
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
    for (int s = 0; s < kAux; ++s) {
      if (aux[s]) cudaStreamDestroy(aux[s]);
      if (join[s]) cudaEventDestroy(join[s]);
    }
    if (fork) cudaEventDestroy(fork);
    if (pinned) cudaFreeHost(pinned);
    if (xfer) cudaStreamDestroy(xfer);
    for (auto& e : xev)
      if (e) cudaEventDestroy(e);
    if (prep_stream) cudaStreamDestroy(prep_stream);
    for (auto& e : pev)
      if (e) cudaEventDestroy(e);
  }
};
