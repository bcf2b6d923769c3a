// Splitting of FP64 operands into BF16 digit slices (layout in ozaki.hpp).
// One CTA per (job, row tile): a row-max pass sets the per-row exponent, then
// every thread turns 8 consecutive k of one row into S 16-byte core rows.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.hpp"
#include "ozaki.hpp"

namespace su2g {
namespace oz {
namespace {

constexpr int kPackThreads = 256;

template <int S>
__global__ void __launch_bounds__(kPackThreads) pack_kernel(const PackJob* __restrict__ jobs,
                                                            const int2* __restrict__ units, Bases bases,
                                                            uint8_t* __restrict__ packed, int* __restrict__ exps) {
  __shared__ double rmax[kPackThreads];
  __shared__ int rexp[kTM];
  __shared__ int tmax;
  const int2 u = units[blockIdx.x];
  const PackJob job = jobs[u.x];
  const int rt = u.y;
  const int RT = job.rt;
  const int r0 = rt * RT;
  const double* src = resolve(bases, job.src_buf, job.src);
  const int tid = threadIdx.x;

  // ---- per-row max |X| ----
  const int parts = kPackThreads / RT;  // 2 (RT=128) or 4 (RT=64)
  const int row = tid % RT, part = tid / RT;
  double m = 0.0;
  if (r0 + row < job.R) {
    const double* p = src + (int64_t)(r0 + row) * job.ld_r;
    for (int k = part; k < job.K; k += parts) m = fmax(m, fabs(p[(int64_t)k * job.ld_k]));
  }
  rmax[tid] = m;
  if (tid == 0) tmax = kExpZero;
  __syncthreads();
  if (tid < RT) {
    double mm = rmax[tid];
    for (int q = 1; q < parts; ++q) mm = fmax(mm, rmax[tid + q * RT]);
    mm *= fabs(job.alpha);
    // |X| 2^-e < 1/2 : e = ilogb(max) + 2
    const int e = (mm > 0.0) ? ilogb(mm) + 2 : kExpZero;
    rexp[tid] = e;
    exps[job.exp + r0 + tid] = e;
    if (e != kExpZero) atomicMax(&tmax, e);
  }
  __syncthreads();
  // the row tile's largest exponent (kExpZero for an all-zero tile)
  if (tid == 0) exps[job.texp + rt] = tmax;

  // ---- digits: one (row, 8 consecutive k) core row per thread iteration ----
  const int ncore_k = job.nkt * (kKS / 8);
  const int64_t unit_bytes = (int64_t)S * RT * kKS * 2;
  const int64_t slice_bytes = (int64_t)RT * kKS * 2;
  uint8_t* dst = packed + job.dst + (int64_t)rt * job.nkt * unit_bytes;
  for (int w = tid; w < RT * ncore_k; w += kPackThreads) {
    const int r = w % RT, kc = w / RT;
    const int e = rexp[r];
    const bool live = (r0 + r < job.R) && e != kExpZero;
    long long N[8];
    const double scale = live ? ldexp(job.alpha, kBits * S - e) : 0.0;
    const double* p = src + (int64_t)(r0 + r) * job.ld_r;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int k = kc * 8 + i;
      N[i] = (live && k < job.K) ? llrint(p[(int64_t)k * job.ld_k] * scale) : 0ll;
    }
    // balanced base-128 digits, least significant first
    __nv_bfloat16 d[S][8];
#pragma unroll
    for (int q = S - 1; q >= 1; --q) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const long long lo = ((N[i] + 64) & 127) - 64;
        N[i] = (N[i] - lo) >> kBits;
        d[q][i] = __int2bfloat16_rn((int)lo);
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) d[0][i] = __int2bfloat16_rn((int)N[i]);
    const int kt = kc / (kKS / 8), kin = kc % (kKS / 8);
    uint8_t* base = dst + (int64_t)kt * unit_bytes + (r / 8) * kSBO + kin * 128 + (r % 8) * 16;
#pragma unroll
    for (int q = 0; q < S; ++q) {
      uint4 v;
      v.x = (uint32_t)__bfloat16_as_ushort(d[q][0]) | ((uint32_t)__bfloat16_as_ushort(d[q][1]) << 16);
      v.y = (uint32_t)__bfloat16_as_ushort(d[q][2]) | ((uint32_t)__bfloat16_as_ushort(d[q][3]) << 16);
      v.z = (uint32_t)__bfloat16_as_ushort(d[q][4]) | ((uint32_t)__bfloat16_as_ushort(d[q][5]) << 16);
      v.w = (uint32_t)__bfloat16_as_ushort(d[q][6]) | ((uint32_t)__bfloat16_as_ushort(d[q][7]) << 16);
      *reinterpret_cast<uint4*>(base + q * slice_bytes) = v;
    }
  }
}

// partial tiles of a split output tile, summed in part order (deterministic)
__global__ void __launch_bounds__(256) reduce_partials(const RedTile* __restrict__ reds, Bases bases) {
  const RedTile r = reds[blockIdx.x];
  const double* P = resolve(bases, kBufScratch, r.part);
  double* C = resolve(bases, r.c_buf, r.c);
  for (int idx = threadIdx.x; idx < kTM * kTN; idx += blockDim.x) {
    const int i = idx % kTM, j = idx / kTM;
    if (i >= r.mlen || j >= r.nlen) continue;
    double s = 0.0;
    for (int p = 0; p < r.nparts; ++p) s += P[(int64_t)p * kTM * kTN + idx];
    C[(int64_t)(r.m0 + i) + (int64_t)(r.n0 + j) * r.ldc] = s;
  }
}

}  // namespace

cudaError_t launch_reduce(const RedTile* reds, int n, const Bases& bases, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  reduce_partials<<<n, 256, 0, stream>>>(reds, bases);
  return cudaGetLastError();
}

cudaError_t launch_pack(int S, const PackJob* jobs, const int2* units, int nunits, const Bases& bases,
                        uint8_t* packed, int* exps, cudaStream_t stream) {
  if (nunits <= 0) return cudaSuccess;
  switch (S) {
    case 6: pack_kernel<6><<<nunits, kPackThreads, 0, stream>>>(jobs, units, bases, packed, exps); break;
    case 7: pack_kernel<7><<<nunits, kPackThreads, 0, stream>>>(jobs, units, bases, packed, exps); break;
    case 8: pack_kernel<8><<<nunits, kPackThreads, 0, stream>>>(jobs, units, bases, packed, exps); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace oz
}  // namespace su2g
