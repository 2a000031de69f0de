// gbr_selftest.cu -- gbr_selftest_bounded_wait: runs the expiry path of the
// bounded mbarrier wait (gbr_mbar.cuh) that the tensor-core pair kernels use.
//
// One CTA of four warps, no TMA, no MMA and no peer CTA: thread 0 initialises
// a shared-memory mbarrier that expects one arrival, and nothing ever arrives.
// Every thread waits on it with a short cycle limit.  The first thread whose
// limit runs out records the site code; the others see the code within 256
// polls and return as well, exactly as the warps of a pair kernel do.  The
// kernel then returns normally, so the context stays usable; the host checks
// the code, that every thread came back, and how long the wait lasted.
#include "../../include/gbrmsd.h"
#include "gbr_handle.h"
#include "gbr_mbar.cuh"

namespace gbr {
namespace {

constexpr int kSelfTestThreads = 128;
constexpr int kSelfTestSite = 0x5e1f;

struct SelfTestOut {
  int err;                 // the error word the waits report into
  int returned;            // threads that came back from the wait with false
  int completed;           // threads whose wait succeeded (must stay 0)
  int pad;
  long long waited;        // cycles thread 0 spent in its wait
};

__global__ void __launch_bounds__(kSelfTestThreads) k_wait_selftest(SelfTestOut* o, long long limit) {
  __shared__ __align__(8) unsigned long long bar;
  const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) mbar_init(b, 1);
  __syncthreads();
  const long long t0 = clock64();
  const bool ok = mbar_wait(b, 0, &o->err, kSelfTestSite, limit);
  const long long dt = clock64() - t0;
  if (ok)
    atomicAdd(&o->completed, 1);
  else
    atomicAdd(&o->returned, 1);
  if (threadIdx.x == 0) o->waited = dt;
}

}  // namespace
}  // namespace gbr

using namespace gbr;

extern "C" int gbr_selftest_bounded_wait(gbr_handle* h, int64_t limit_cycles, int32_t* site_out,
                                         int64_t* waited_cycles) {
  if (!h) return GBR_ERR_ARG;
  if (limit_cycles < 1000 || limit_cycles > 4000000000LL)
    return h->fail(GBR_ERR_ARG, "limit_cycles %lld outside [1000, 4e9]", (long long)limit_cycles);
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return h->cuda_fail(e, "cudaSetDevice");
  SelfTestOut* d = nullptr;
  if ((e = cudaMalloc(&d, sizeof(SelfTestOut))) != cudaSuccess) return h->cuda_fail(e, "cudaMalloc");
  SelfTestOut o{};
  cudaStream_t st = h->stream;
  e = cudaMemsetAsync(d, 0, sizeof(SelfTestOut), st);
  if (e == cudaSuccess) {
    k_wait_selftest<<<1, kSelfTestThreads, 0, st>>>(d, (long long)limit_cycles);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&o, d, sizeof o, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d);
  if (e != cudaSuccess) return h->cuda_fail(e, "bounded-wait self-test kernel");
  if (site_out) *site_out = o.err;
  if (waited_cycles) *waited_cycles = o.waited;
  if (o.err != kSelfTestSite || o.completed != 0 || o.returned != kSelfTestThreads)
    return h->fail(GBR_ERR_DEVICE, "bounded wait self-test: code %#x, %d of %d threads returned, %d completed",
                   o.err, o.returned, kSelfTestThreads, o.completed);
  h->err.clear();
  return GBR_OK;
}
