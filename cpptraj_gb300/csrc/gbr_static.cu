// gbr_static.cu -- gbr_allpairs_fp64_static: all-pairs RMSD that allocates no
// memory at all.
//
// Some callers cannot call cudaMalloc: host programs (an MD engine, a
// visualiser) that reserve the GPU's memory at start-up and hand it out from
// their own fixed pool, which a library must not grow behind their back; and
// plugins loaded into such a process, or into one whose latency-critical
// streams must not be stalled by the device-wide synchronisation that
// cudaMalloc and cudaFree can cause.  For them this entry point computes the
// same upper triangle as gbr_allpairs(..., GBR_PREC_FP64) -- every pair
// directly in FP64 -- from device inputs into a device output, using as
// scratch only a file-scope __device__ array of fixed size.
//
// The scratch holds the per-frame centres (3 doubles per frame) and the total
// weight.  It is part of this library's device image, so every GPU that loads
// libgbrmsd.so holds it (kStaticScratchBytes) until the process exits.  Its
// device address is looked up once per device with cudaGetSymbolAddress, on
// the first call made with that device current; make that first call before
// any stream capture.  All calls share the one array and it keeps the last
// call's contents; everything this entry point reads from it is rewritten at
// the start of each call, so nothing has to be cleared.  Two calls whose work
// overlaps on the GPU (different streams or host threads) race on the array.
#include <mutex>

#include "../../include/gbrmsd.h"
#include "gbr_internal.h"

namespace gbr {
namespace {

constexpr size_t kStaticScratchBytes = 32u << 20;  // 32 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_static_mutex;
void* g_static_addr[kMaxDevices] = {};

// Total weight into *W (one block, fixed summation order).
__global__ void k_weight_sum(const double* mass, int n, double* W) {
  __shared__ double part[256];
  double s = 0.0;
  for (int a = threadIdx.x; a < n; a += blockDim.x) s += mass ? mass[a] : 1.0;
  part[threadIdx.x] = s;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) part[threadIdx.x] += part[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *W = part[0];
}

// True when p is device (or managed) memory that belongs to device `dev`:
// the kernels run on the current device, which cannot reach another GPU's
// memory without peer access.
bool on_device(const void* p, int dev) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeManaged) return true;
  return at.type == cudaMemoryTypeDevice && at.device == dev;
}

}  // namespace
}  // namespace gbr

using namespace gbr;

extern "C" int gbr_allpairs_fp64_static(const void* xyz, int dtype, int64_t n_frame, int32_t n_atom,
                                        const double* mass, int mode, float* out, void* stream) {
  if (!xyz || !out) return GBR_ERR_ARG;
  if (dtype != GBR_F32 && dtype != GBR_F64) return GBR_ERR_ARG;
  if (mode != GBR_FIT && mode != GBR_NOFIT) return GBR_ERR_ARG;
  if (n_atom < 1 || n_frame < 0 || n_frame > INT32_MAX) return GBR_ERR_ARG;
  // Scratch: centres [n_frame][3] doubles, then the total weight.
  const size_t need = sizeof(double) * (3 * (size_t)n_frame + 1);
  if (need > kStaticScratchBytes) return GBR_ERR_NOMEM;  // beyond the fixed scratch (~1.39M frames)
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GBR_ERR_CUDA;
  if (!on_device(xyz, dev) || !on_device(out, dev) || (mass && !on_device(mass, dev))) return GBR_ERR_ARG;
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_addr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
      if (e != cudaSuccess || p == nullptr) return GBR_ERR_CUDA;
      g_static_addr[dev] = p;
    }
    base = g_static_addr[dev];
  }
  const int64_t n_pairs = n_frame * (n_frame - 1) / 2;
  if (n_pairs == 0) return GBR_OK;
  cudaStream_t st = (cudaStream_t)stream;
  double* cen = (double*)base;
  double* dW = cen + 3 * (size_t)n_frame;
  // The total weight stays on the device: the pair kernel reads it there, and
  // the host looks at it only after the last kernel (one wait per call).
  k_weight_sum<<<1, 256, 0, st>>>(mass, n_atom, dW);

  PrepArgs pa{};
  pa.dtype_f64 = (dtype == GBR_F64);
  pa.ref = xyz;
  pa.tgt = nullptr;
  pa.n_ref = n_frame;
  pa.F = n_frame;
  pa.N = n_atom;
  pa.nofit = (mode == GBR_NOFIT);
  pa.centroid_only = 1;
  pa.cmass_ref = pa.cmass_tgt = pa.w = mass;
  pa.cen = cen;
  PrepOut po;
  if (run_prep(pa, po, st) != cudaSuccess) return GBR_ERR_CUDA;

  ExactLaunch ex{};
  ex.dtype_f64 = pa.dtype_f64;
  ex.ref = xyz;
  ex.tgt = nullptr;
  ex.n_ref = n_frame;
  ex.N = n_atom;
  ex.cen = cen;
  ex.w = mass;
  ex.dWsum = dW;
  ex.nofit = pa.nofit;
  ex.tgt0 = 0;
  OutMap map{};
  map.out = out;
  map.n_ref = n_frame;
  map.n_tgt = n_frame;
  map.tri = 1;
  map.row_begin = 0;
  map.row_end = n_frame;
  map.base = 0;
  ex.map = map;
  ex.list = nullptr;
  ex.count = n_pairs;
  if (run_exact(ex, st) != cudaSuccess) return GBR_ERR_CUDA;
  double W = 0.0;
  if (cudaMemcpyAsync(&W, dW, sizeof W, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return GBR_ERR_CUDA;
  // Zero total mass: the reference refuses the pair (src/Constants.h:35);
  // the triangle written meanwhile is not a result.
  if (W < 1e-14) return GBR_ERR_ZERO_MASS;
  return GBR_OK;
}
