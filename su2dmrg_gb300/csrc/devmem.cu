// Device memory of the library's plans and one-shot work lists.
//
// cudaMalloc and cudaFree synchronise the whole device, so a sweep that builds
// and drops plans at every step would stall every other solve sharing the GPU
// (and pays the synchronisation itself at every step).  Instead, plans take
// their buffers from one stream-ordered memory pool per device: an allocation
// is served on the calling thread's private set-up stream (waited for, so the
// memory is usable on any stream when dev_alloc returns), and a free is queued
// on the stream the buffer was last used on, so it is returned to the pool only
// once that stream has passed it; nothing ever waits for other streams.  Freed
// blocks stay cached in the pool up to kKeepBytes.
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>

#include "kernels.hpp"

namespace su2g {
namespace {

constexpr uint64_t kKeepBytes = 16ull << 30;  // cached free memory kept by the pool

std::mutex g_pool_mu;
std::map<int, cudaMemPool_t> g_pools;

cudaError_t device_pool(int dev, cudaMemPool_t* out) {
  std::lock_guard<std::mutex> lock(g_pool_mu);
  auto it = g_pools.find(dev);
  if (it != g_pools.end()) {
    *out = it->second;
    return cudaSuccess;
  }
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool = nullptr;
  cudaError_t e = cudaMemPoolCreate(&pool, &props);
  if (e != cudaSuccess) return e;
  uint64_t keep = kKeepBytes;
  e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  if (e != cudaSuccess) {
    cudaMemPoolDestroy(pool);
    return e;
  }
  g_pools[dev] = pool;
  *out = pool;
  return cudaSuccess;
}

}  // namespace

cudaError_t setup_stream(cudaStream_t* out) {
  // one non-blocking stream per host thread and device (never destroyed:
  // thread-local objects cannot safely call into CUDA at process exit)
  thread_local std::map<int, cudaStream_t> streams;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  auto it = streams.find(dev);
  if (it == streams.end()) {
    cudaStream_t s = nullptr;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    it = streams.emplace(dev, s).first;
  }
  *out = it->second;
  return cudaSuccess;
}

cudaError_t dev_alloc(void** p, size_t bytes) {
  *p = nullptr;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  cudaMemPool_t pool = nullptr;
  cudaStream_t st = nullptr;
  if (e == cudaSuccess) e = device_pool(dev, &pool);
  if (e == cudaSuccess) e = setup_stream(&st);
  if (e == cudaSuccess) e = cudaMallocFromPoolAsync(p, bytes ? bytes : 16, pool, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

void dev_free(void* p, cudaStream_t after) {
  if (p) cudaFreeAsync(p, after);
}

cudaError_t upload_bytes(const void* host, size_t bytes, void** dptr) {
  *dptr = nullptr;
  if (bytes == 0) return cudaSuccess;
  cudaError_t e = dev_alloc(dptr, bytes);
  cudaStream_t st = nullptr;
  if (e == cudaSuccess) e = setup_stream(&st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(*dptr, host, bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

}  // namespace su2g
