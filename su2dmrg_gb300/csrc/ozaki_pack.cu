// Splitting of FP64 operands into BF16 digit slices (layout in ozaki.hpp), in
// two launches: the row exponents (one warp per row), then the digits (one CTA
// per row tile and 64 k).  The scaling and rounding to integers use integer
// operations only (FP64 throughput is scarce on GB300).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.hpp"
#include "ozaki.hpp"

namespace su2g {
namespace oz {
namespace {

constexpr int kPackThreads = 256;

// round(x 2^s) to the nearest integer, halves away from zero, with integer
// operations only.  The caller guarantees |x| 2^s < 2^48, so the mantissa is
// shifted right by at least five bits.
__device__ __forceinline__ long long scale_round(double x, int s) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  int E = (int)((b >> 52) & 0x7FF);
  unsigned long long M = b & 0xFFFFFFFFFFFFFull;
  if (E == 0) {
    if (M == 0) return 0;
    E = 1;  // subnormal
  } else {
    M |= 1ull << 52;
  }
  const int r = 1075 - E - s;  // |x| 2^s = M 2^-r
  unsigned long long q;
  if (r <= 0) {
    q = M << -r;  // excluded by the caller's bound; kept exact
  } else if (r > 63) {
    return 0;  // below 2^53 2^-64 < 1/2
  } else {
    q = ((M >> (r - 1)) + 1) >> 1;
  }
  return (b >> 63) ? -(long long)q : (long long)q;
}

// ilogb of a positive finite double given as its bit pattern
__device__ __forceinline__ int ilogb_bits(unsigned long long b) {
  const int E = (int)(b >> 52);
  if (E > 0) return E - 1023;
  return (63 - __clzll(b & 0xFFFFFFFFFFFFFull)) - 1074;
}

// sum_{q<S} 64 * 128^q: added to N it turns balanced digits into plain ones
template <int S>
constexpr long long kDigitBias = S == 0 ? 0 : 64ll + 128ll * kDigitBias<(S > 0 ? S - 1 : 0)>;
template <>
constexpr long long kDigitBias<0> = 0;

constexpr int kRowsPerUnit = kTM;  // row slots per unit in the row kernel (RT <= 128)
constexpr int kDigitKt = 4;        // k tiles (16 k each) per CTA of the digit kernel

// Row exponents: one warp per row of every unit, lanes along k (coalesced):
// |alpha X| 2^-e < 1/2 with e = ilogb(max |alpha X|) + 2, kExpZero for a zero row.
__global__ void __launch_bounds__(kPackThreads) pack_rows_kernel(const PackJob* __restrict__ jobs,
                                                                 const int2* __restrict__ units, int nunits,
                                                                 Bases bases, int* __restrict__ exps) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t gw = (int64_t)blockIdx.x * (kPackThreads / 32) + warp;
  const int ui = (int)(gw / kRowsPerUnit), row = (int)(gw % kRowsPerUnit);
  if (ui >= nunits) return;
  const int2 u = units[ui];
  const PackJob& job = jobs[u.x];
  if (row >= job.rt || job.rowmax >= 0) return;  // row maxima left by the producing GEMM
  const int r = u.y * job.rt + row;
  unsigned long long m = 0;  // max |x| as a bit pattern (order-preserving for |x|)
  if (r < job.R) {
    const double* p = resolve(bases, job.src_buf, job.src) + (int64_t)r * job.ld_r;
    int k = lane;
    for (; k + 96 < job.K; k += 128) {  // four loads in flight
      const unsigned long long a = __double_as_longlong(p[(int64_t)k * job.ld_k]);
      const unsigned long long b = __double_as_longlong(p[(int64_t)(k + 32) * job.ld_k]);
      const unsigned long long c = __double_as_longlong(p[(int64_t)(k + 64) * job.ld_k]);
      const unsigned long long d = __double_as_longlong(p[(int64_t)(k + 96) * job.ld_k]);
      m = max(m, max(max(a & 0x7FFFFFFFFFFFFFFFull, b & 0x7FFFFFFFFFFFFFFFull),
                     max(c & 0x7FFFFFFFFFFFFFFFull, d & 0x7FFFFFFFFFFFFFFFull)));
    }
    for (; k < job.K; k += 32)
      m = max(m, (unsigned long long)__double_as_longlong(p[(int64_t)k * job.ld_k]) & 0x7FFFFFFFFFFFFFFFull);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) {
    int e = kExpZero;
    if (m != 0) {
      if (job.alpha == 1.0 || job.alpha == -1.0) {
        e = ilogb_bits(m) + 2;
      } else {
        const double mm = __longlong_as_double((long long)m) * fabs(job.alpha);
        if (mm > 0.0) e = ilogb(mm) + 2;
      }
    }
    exps[job.exp + r] = e;
  }
}

// Digits: one CTA per (unit, kDigitKt k tiles); a warp converts 8 rows x 32 k,
// a thread one row x 8 k into S 16-byte core rows, so that a warp's stores
// fill whole 256-byte core-row groups.  The k-chunk-0 CTA also records the
// row tile's largest exponent.
template <int S>
__global__ void __launch_bounds__(kPackThreads) pack_digits_kernel(const PackJob* __restrict__ jobs,
                                                                   const int2* __restrict__ units, Bases bases,
                                                                   uint8_t* __restrict__ packed,
                                                                   int* __restrict__ exps) {
  __shared__ int rexp[kTM];
  __shared__ int tmax;
  const int2 u = units[blockIdx.x];
  const PackJob job = jobs[u.x];
  const int kt0 = blockIdx.y * kDigitKt;
  if (kt0 >= job.nkt) return;
  const int rt = u.y, RT = job.rt, r0 = rt * RT;
  const double* src = resolve(bases, job.src_buf, job.src);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) tmax = kExpZero;
  __syncthreads();
  if (tid < RT) {
    int e;
    if (job.rowmax >= 0) {  // |X| 2^-e < 1/2 from the producer's ilogb maxima
      const int v = (r0 + tid < job.R) ? exps[job.rowmax + r0 + tid] : 0;
      e = v > 0 ? v - kRowmaxBias + 2 : kExpZero;
      if (blockIdx.y == 0) exps[job.exp + r0 + tid] = e;
    } else {
      e = exps[job.exp + r0 + tid];
    }
    rexp[tid] = e;
    if (blockIdx.y == 0 && e != kExpZero) atomicMax(&tmax, e);
  }
  __syncthreads();
  if (blockIdx.y == 0 && tid == 0) exps[job.texp + rt] = tmax;

  const bool unit_alpha = job.alpha == 1.0 || job.alpha == -1.0;
  const int ncore_k = min(job.nkt - kt0, kDigitKt) * (kKS / 8);
  const int nkq = (ncore_k + 3) / 4;  // groups of 4 core columns (32 k)
  const int64_t unit_bytes = (int64_t)S * RT * kKS * 2;
  const int64_t slice_bytes = (int64_t)RT * kKS * 2;
  uint8_t* dst = packed + job.dst + ((int64_t)rt * job.nkt + kt0) * unit_bytes;
  const int r8 = lane & 7, kq = lane >> 3;
  for (int item = warp; item < (RT / 8) * nkq; item += kPackThreads / 32) {
    const int rg = item % (RT / 8), kc = (item / (RT / 8)) * 4 + kq;
    if (kc >= ncore_k) continue;
    const int r = rg * 8 + r8;
    const int e = rexp[r];
    const bool live = (r0 + r < job.R) && e != kExpZero;
    const int s = kBits * S - e;
    long long N[8];
    const double* p = src + (int64_t)(r0 + r) * job.ld_r;
    const int k0 = (kt0 * (kKS / 8) + kc) * 8;
    double xv[8];
    if (live && k0 + 8 <= job.K && job.ld_k == 1) {  // whole group along a contiguous row
      const double* q = p + k0;
#pragma unroll
      for (int i = 0; i < 8; ++i) xv[i] = q[i];
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) xv[i] = (live && k0 + i < job.K) ? p[(int64_t)(k0 + i) * job.ld_k] : 0.0;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const double x = xv[i];
      N[i] = scale_round(unit_alpha ? (job.alpha < 0 ? -x : x) : x * job.alpha, s);
    }
    // Balanced base-128 digits d_q in [-64, 63] (the leading one takes the
    // rest): N + sum_q 64 * 128^q has the plain base-128 digits d_q + 64, so
    // each digit is one shift and mask.  A digit's BF16 bits are the upper
    // half of the exact FP32 value (2^23 + u) - (2^23 + 64).
#pragma unroll
    for (int i = 0; i < 8; ++i) N[i] += kDigitBias<S>;
    const int kt = kc / (kKS / 8), kin = kc % (kKS / 8);
    uint8_t* base = dst + (int64_t)kt * unit_bytes + (r / 8) * kSBO + kin * 128 + (r % 8) * 16;
#pragma unroll
    for (int q = 0; q < S; ++q) {
      uint32_t fb[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        float f;
        if (q == 0) {  // leading digit: (N' >> 7(S-1)) - 64 in [-65, 65]
          const int u0 = (int)(N[i] >> (kBits * (S - 1))) + 1;
          f = __int_as_float(0x4B000000 + u0) - 8388673.0f;
        } else {
          const uint32_t uq = (uint32_t)(N[i] >> (kBits * (S - 1 - q))) & 127u;
          f = __int_as_float(0x4B000000 | uq) - 8388672.0f;
        }
        fb[i] = __float_as_uint(f);
      }
      uint4 v;
      v.x = __byte_perm(fb[0], fb[1], 0x7632);
      v.y = __byte_perm(fb[2], fb[3], 0x7632);
      v.z = __byte_perm(fb[4], fb[5], 0x7632);
      v.w = __byte_perm(fb[6], fb[7], 0x7632);
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

cudaError_t launch_pack(int S, const PackJob* jobs, const int2* units, int nunits, int max_nkt, bool rows_pass,
                        const Bases& bases, uint8_t* packed, int* exps, cudaStream_t stream) {
  if (nunits <= 0) return cudaSuccess;
  if (rows_pass) {
    const int64_t warps = (int64_t)nunits * kRowsPerUnit;
    const int rows_blocks = (int)((warps + kPackThreads / 32 - 1) / (kPackThreads / 32));
    pack_rows_kernel<<<rows_blocks, kPackThreads, 0, stream>>>(jobs, units, nunits, bases, exps);
  }
  const dim3 grid(nunits, (max_nkt + kDigitKt - 1) / kDigitKt);
  switch (S) {
    case 6: pack_digits_kernel<6><<<grid, kPackThreads, 0, stream>>>(jobs, units, bases, packed, exps); break;
    case 7: pack_digits_kernel<7><<<grid, kPackThreads, 0, stream>>>(jobs, units, bases, packed, exps); break;
    case 8: pack_digits_kernel<8><<<grid, kPackThreads, 0, stream>>>(jobs, units, bases, packed, exps); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace oz
}  // namespace su2g
