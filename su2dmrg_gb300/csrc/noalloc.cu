// Allocation-free one-shot H_eff term (su2g_hamiltonian_vector_multiplication_noalloc).
//
// Some callers of this library cannot allocate device memory at the point
// where they apply an operator term: engines that reserve their whole HBM
// budget up front and forbid later allocations, per-term calls issued from
// many host threads where cudaMalloc/cudaFree would serialise the device
// (both synchronise implicitly), and callers running inside another
// library's callbacks that must not allocate.  For them this entry point
// keeps its scratch — the intermediate blocks T = vec^T op1 and the device
// copy of the work list — in file-scope device arrays of fixed size that
// every GPU loading the library holds until the process exits.
//
// The arrays are shared by every call on a device and keep the contents of
// the last call.  Nothing needs clearing between calls: the work list is
// copied in whole, every intermediate element is written by exactly one tile
// of the first launch before the second launch reads it, and every element of
// y is written by exactly one tile of the second launch.  Each call holds a
// per-device host lock from its first copy into the arrays until its second
// launch is queued, so calls from several host threads on ONE stream queue
// whole (copy, copy, launch, launch) groups one after the other and stream
// order keeps them apart.  Calls on different streams (or devices' streams
// that overlap) still race on the arrays; the caller serialises those.
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "heff_plan.hpp"
#include "kernels.hpp"
#include "su2g.h"

namespace {

static __device__ __align__(256) double g_noalloc_scratch[SU2G_NOALLOC_SCRATCH_DOUBLES];
static __device__ __align__(256) su2g::GemmTile g_noalloc_tiles[SU2G_NOALLOC_MAX_TILES];
static __device__ __align__(256) su2g::GemmSeg g_noalloc_segs[SU2G_NOALLOC_MAX_SEGS];

struct DeviceArrays {
  bool ready = false;
  double* scratch = nullptr;
  su2g::GemmTile* tiles = nullptr;
  su2g::GemmSeg* segs = nullptr;
};

constexpr int kMaxDevices = 64;
std::mutex g_mu;
DeviceArrays g_dev[kMaxDevices];
// held by a call from its first copy into a device's arrays to its last launch
std::mutex g_call_mu[kMaxDevices];

int fail(int code, const std::string& msg) { return su2g::set_last_error(code, msg); }

// The device addresses of the file-scope arrays on the current device.  In
// host code their names are host-side stand-ins, not device addresses, so the
// addresses are looked up once per device (with that device current) and
// cached.
int device_arrays(DeviceArrays* out, int* device) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(SU2G_ECUDA, std::string("noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(SU2G_EUNSUPPORTED, "noalloc: device index beyond 63");
  std::lock_guard<std::mutex> lock(g_mu);
  DeviceArrays& d = g_dev[dev];
  if (!d.ready) {
    e = cudaGetSymbolAddress((void**)&d.scratch, g_noalloc_scratch);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&d.tiles, g_noalloc_tiles);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&d.segs, g_noalloc_segs);
    if (e != cudaSuccess)
      return fail(SU2G_ECUDA, std::string("noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    d.ready = true;
  }
  *out = d;
  *device = dev;
  return SU2G_OK;
}

}  // namespace

extern "C" int su2g_hamiltonian_vector_multiplication_noalloc(const int* vec_desc, const int* vec_flag,
                                                              const double* vec, su2g_tensor op1, su2g_tensor op2,
                                                              double* y, void* stream) {
  su2g_term term{op1, op2, 1.0};
  su2g::HeffWork w;
  std::string err;
  int rc = su2g::build_heff_work(vec_desc, vec_flag, 1, &term, nullptr, 0.0, nullptr, 0.0, &w, &err);
  if (rc) return fail(rc, "noalloc: " + err);
  if (w.psi.total > 0 && (!vec || !y)) return fail(SU2G_EINVAL, "noalloc: null vector");
  if (vec == y && vec) return fail(SU2G_EINVAL, "noalloc: vec and y must not alias");
  const size_t ntiles = w.tile1.size() + w.tile2.size();
  const size_t nsegs = w.seg1.size() + w.seg2.size();
  if (w.scratch_len > SU2G_NOALLOC_SCRATCH_DOUBLES)
    return fail(SU2G_EINVAL, "noalloc: the term needs " + std::to_string(w.scratch_len) +
                                 " doubles of intermediate blocks, more than the fixed " +
                                 std::to_string((long long)SU2G_NOALLOC_SCRATCH_DOUBLES) +
                                 "; use su2g_hamiltonian_vector_multiplication");
  if (ntiles > SU2G_NOALLOC_MAX_TILES || nsegs > SU2G_NOALLOC_MAX_SEGS)
    return fail(SU2G_EINVAL, "noalloc: the term needs " + std::to_string(ntiles) + " tiles and " +
                                 std::to_string(nsegs) + " block products, more than the fixed " +
                                 std::to_string(SU2G_NOALLOC_MAX_TILES) + " / " +
                                 std::to_string(SU2G_NOALLOC_MAX_SEGS) +
                                 "; use su2g_hamiltonian_vector_multiplication");
  DeviceArrays d;
  int dev = 0;
  rc = device_arrays(&d, &dev);
  if (rc) return rc;
  // one work list: phase-2 tiles index the segments after phase 1's
  std::vector<su2g::GemmTile> tiles(w.tile1);
  for (su2g::GemmTile t : w.tile2) {
    t.seg0 += (int)w.seg1.size();
    tiles.push_back(t);
  }
  std::vector<su2g::GemmSeg> segs(w.seg1);
  segs.insert(segs.end(), w.seg2.begin(), w.seg2.end());
  cudaStream_t st = (cudaStream_t)stream;
  // the work list is copied from host vectors freed on return: a captured
  // copy would replay from freed memory
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return fail(SU2G_EUNSUPPORTED, "noalloc: the stream is being captured; this entry point cannot be captured");
  std::lock_guard<std::mutex> call_lock(g_call_mu[dev]);
  // pageable sources: each call returns once its bytes are staged, so the
  // vectors may go out of scope afterwards
  cudaError_t e = cudaSuccess;
  if (!tiles.empty())
    e = cudaMemcpyAsync(d.tiles, tiles.data(), tiles.size() * sizeof(su2g::GemmTile), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !segs.empty())
    e = cudaMemcpyAsync(d.segs, segs.data(), segs.size() * sizeof(su2g::GemmSeg), cudaMemcpyHostToDevice, st);
  su2g::Bases b;
  b.p[su2g::kBufAbs] = 0;
  b.p[su2g::kBufPsi] = reinterpret_cast<uintptr_t>(vec);
  b.p[su2g::kBufY] = reinterpret_cast<uintptr_t>(y);
  b.p[su2g::kBufScratch] = reinterpret_cast<uintptr_t>(d.scratch);
  if (e == cudaSuccess) e = su2g::launch_gemm_f64(d.tiles, (int)w.tile1.size(), d.segs, b, st);
  if (e == cudaSuccess) e = su2g::launch_gemm_f64(d.tiles + w.tile1.size(), (int)w.tile2.size(), d.segs, b, st);
  if (e != cudaSuccess) return fail(SU2G_ECUDA, std::string("noalloc: ") + cudaGetErrorString(e));
  return SU2G_OK;
}
