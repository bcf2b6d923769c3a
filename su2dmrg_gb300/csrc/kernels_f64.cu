// FP64 kernels of the hot path:
//   * gemm_f64_tiles: the block-sparse contraction engine (one CTA per output
//     tile of the work list, gemm_work.hpp), FP64 tensor-core MMA
//     (mma.sync.m8n8k4.f64) fed from shared memory;
//   * deterministic BLAS-1 (dot, axpy, scale) for the Lanczos iteration.
#include <cuda_runtime.h>

#include <cstdint>

#include "gemm_work.hpp"
#include "kernels.hpp"

namespace su2g {
namespace {

constexpr int kBK = 16;       // K per shared-memory stage
constexpr int kThreads = 128; // 4 warps, each a quadrant of the tile

__device__ __forceinline__ void dmma_m8n8k4(double (&d)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(d[0]), "+d"(d[1])
               : "d"(a), "d"(b));
}

// One TM x TN output tile: C_tile = sum_s alpha_s * op(A_s) B_s; every
// segment is accumulated on its own, scaled by its alpha and added (the
// reference scales each block product by its recoupling factor before
// summing, tensor_su2_dmrg_src.cpp:997-1004).  Warp w computes the quadrant
// (w / 2, w % 2) of (TM / 2) x (TN / 2) as FM x FN fragments of 8 x 8.
// Operands are staged K = 16 at a time in shared memory, rows padded by 4
// doubles (conflict-free fragment reads).
template <int TM, int TN>
__device__ __forceinline__ void f64_tile(const GemmTile& t, const GemmSeg* __restrict__ segs, const Bases& bases,
                                         double* __restrict__ As, double* __restrict__ Bs) {
  constexpr int FM = TM / 16, FN = TN / 16;
  constexpr int LA = TM + 4, LB = TN + 4;
  constexpr int PA = TM / 8, PB = TN / 8;  // elements each thread stages per operand per stage
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * (TM / 2), wn = (warp & 1) * (TN / 2);
  const int fr = lane >> 2, fc = lane & 3;

  double acc[FM][FN][2];
#pragma unroll
  for (int i = 0; i < FM; ++i)
#pragma unroll
    for (int j = 0; j < FN; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

  for (int s = t.seg0; s < t.seg0 + t.nseg; ++s) {
    const GemmSeg g = segs[s];
    const double* __restrict__ A = resolve(bases, g.a_buf, g.a);
    const double* __restrict__ B = resolve(bases, g.b_buf, g.b);
    double sacc[FM][FN][2];
#pragma unroll
    for (int i = 0; i < FM; ++i)
#pragma unroll
      for (int j = 0; j < FN; ++j) sacc[i][j][0] = sacc[i][j][1] = 0.0;

    for (int k0 = 0; k0 < g.K; k0 += kBK) {
      // ---- stage A (TM x 16) and B (16 x TN), zero padded ----
      if (g.transA) {  // A stored K x M: (k, m) at A[k + m*lda], contiguous in k
        const int m = tid / (kBK / PA), kb = (tid % (kBK / PA)) * PA;
        const bool mok = m < t.mlen;
        const double* src = A + (int64_t)(t.m0 + m) * g.lda + k0 + kb;
#pragma unroll
        for (int i = 0; i < PA; ++i) {
          const int k = kb + i;
          As[k * LA + m] = (mok && k0 + k < g.K) ? __ldg(src + i) : 0.0;
        }
      } else {  // A stored M x K: (m, k) at A[m + k*lda], contiguous in m
        const int k = tid >> 3, mb = (tid & 7) * PA;
        const bool kok = k0 + k < g.K;
        const double* src = A + (int64_t)(k0 + k) * g.lda + t.m0 + mb;
#pragma unroll
        for (int i = 0; i < PA; ++i) {
          const int m = mb + i;
          As[k * LA + m] = (kok && m < t.mlen) ? __ldg(src + i) : 0.0;
        }
      }
      {  // B stored K x N: (k, n) at B[k + n*ldb], contiguous in k
        const int n = tid / (kBK / PB), kb = (tid % (kBK / PB)) * PB;
        const bool nok = n < t.nlen;
        const double* src = B + (int64_t)(t.n0 + n) * g.ldb + k0 + kb;
#pragma unroll
        for (int i = 0; i < PB; ++i) {
          const int k = kb + i;
          Bs[k * LB + n] = (nok && k0 + k < g.K) ? __ldg(src + i) : 0.0;
        }
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < kBK; kk += 4) {
        double af[FM], bf[FN];
#pragma unroll
        for (int i = 0; i < FM; ++i) af[i] = As[(kk + fc) * LA + wm + i * 8 + fr];
#pragma unroll
        for (int j = 0; j < FN; ++j) bf[j] = Bs[(kk + fc) * LB + wn + j * 8 + fr];
#pragma unroll
        for (int i = 0; i < FM; ++i)
#pragma unroll
          for (int j = 0; j < FN; ++j) dmma_m8n8k4(sacc[i][j], af[i], bf[j]);
      }
      __syncthreads();
    }
    const double alpha = g.alpha;
#pragma unroll
    for (int i = 0; i < FM; ++i)
#pragma unroll
      for (int j = 0; j < FN; ++j) {
        acc[i][j][0] += alpha * sacc[i][j][0];
        acc[i][j][1] += alpha * sacc[i][j][1];
      }
  }

  double* C = resolve(bases, t.c_buf, t.c);
#pragma unroll
  for (int i = 0; i < FM; ++i) {
    const int r = wm + i * 8 + fr;
    if (r >= t.mlen) continue;
#pragma unroll
    for (int j = 0; j < FN; ++j) {
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int c = wn + j * 8 + 2 * fc + q;
        if (c < t.nlen) C[(int64_t)(t.m0 + r) + (int64_t)(t.n0 + c) * t.ldc] = acc[i][j][q];
      }
    }
  }
}

// One CTA per tile of the work list; the tile's class picks its shape (the
// branch is uniform over the CTA).
__global__ void __launch_bounds__(kThreads) gemm_f64_tiles(const GemmTile* __restrict__ tiles,
                                                           const GemmSeg* __restrict__ segs, Bases bases) {
  __shared__ double As[kBK * (kTileM + 4)];
  __shared__ double Bs[kBK * (kTileN + 4)];
  const GemmTile t = tiles[blockIdx.x];
  switch (t.cls) {
    case 1: f64_tile<64, 32>(t, segs, bases, As, Bs); break;
    case 2: f64_tile<32, 64>(t, segs, bases, As, Bs); break;
    case 3: f64_tile<32, 32>(t, segs, bases, As, Bs); break;
    default: f64_tile<64, 64>(t, segs, bases, As, Bs); break;
  }
}

// One dense product C = op(A) B in tiles of class cls, the tile and its
// segment formed from the kernel's arguments (no work list to upload): the
// same tile code, so the same sums in the same order as a work-list launch.
__global__ void __launch_bounds__(kThreads) gemm_f64_dense(int transA, int M, int N, int K, const double* A, int lda,
                                                           const double* B, int ldb, double* C, int ldc, int cls) {
  __shared__ double As[kBK * (kTileM + 4)];
  __shared__ double Bs[kBK * (kTileN + 4)];
  GemmSeg g;
  g.a = (int64_t)((uintptr_t)A / 8);
  g.b = (int64_t)((uintptr_t)B / 8);
  g.a_len = 0;
  g.b_len = 0;
  g.a_buf = g.b_buf = kBufAbs;
  g.lda = lda;
  g.ldb = ldb;
  g.K = K;
  g.transA = transA;
  g.alpha = 1.0;
  GemmTile t;
  t.c = (int64_t)((uintptr_t)C / 8);
  t.c_len = 0;
  t.c_buf = kBufAbs;
  t.ldc = ldc;
  const int tm = cls == 2 || cls == 3 ? 32 : 64, tn = cls == 1 || cls == 3 ? 32 : 64;
  t.m0 = blockIdx.x * tm;
  t.n0 = blockIdx.y * tn;
  t.mlen = min(tm, M - t.m0);
  t.nlen = min(tn, N - t.n0);
  t.seg0 = 0;
  t.nseg = 1;
  t.kwork = K;
  t.cls = cls;
  t.pad = 0;
  const Bases bases{};
  switch (cls) {
    case 1: f64_tile<64, 32>(t, &g, bases, As, Bs); break;
    case 2: f64_tile<32, 64>(t, &g, bases, As, Bs); break;
    case 3: f64_tile<32, 32>(t, &g, bases, As, Bs); break;
    default: f64_tile<64, 64>(t, &g, bases, As, Bs); break;
  }
}

}  // namespace

cudaError_t launch_gemm_f64_dense(bool transA, int M, int N, int K, const double* A, int lda, const double* B,
                                  int ldb, double* C, int ldc, int cls, cudaStream_t stream) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  if (cls < 0 || cls >= kTileClasses) return cudaErrorInvalidValue;
  const dim3 grid((M + kTileClassM[cls] - 1) / kTileClassM[cls], (N + kTileClassN[cls] - 1) / kTileClassN[cls]);
  gemm_f64_dense<<<grid, kThreads, 0, stream>>>(transA ? 1 : 0, M, N, K, A, lda, B, ldb, C, ldc, cls);
  return cudaGetLastError();
}

cudaError_t launch_gemm_f64(const GemmTile* tiles, int ntiles, const GemmSeg* segs, const Bases& bases,
                            cudaStream_t stream) {
  if (ntiles <= 0) return cudaSuccess;
  gemm_f64_tiles<<<ntiles, kThreads, 0, stream>>>(tiles, segs, bases);
  return cudaGetLastError();
}

namespace {

// ---------------------------------------------------------------- BLAS-1 --
constexpr int kRedBlocks = 512;  // fixed: the summation order never depends on the device
constexpr int kRedThreads = 256;

__device__ __forceinline__ double block_sum(double v, double* sh) {
  const int tid = threadIdx.x;
  sh[tid] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (tid < s) sh[tid] += sh[tid + s];
    __syncthreads();
  }
  return sh[0];
}

__global__ void __launch_bounds__(kRedThreads) dot_partial(const double* __restrict__ x, const double* __restrict__ y,
                                                          int64_t n, double* __restrict__ part) {
  __shared__ double sh[kRedThreads];
  double v = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v += x[i] * y[i];
  const double s = block_sum(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kRedThreads) dot_final(const double* __restrict__ part, int nparts,
                                                        double* __restrict__ out) {
  __shared__ double sh[kRedThreads];
  double v = 0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += part[i];
  const double s = block_sum(v, sh);
  if (threadIdx.x == 0) *out = s;
}

__global__ void axpy_kernel(double alpha, const double* __restrict__ x, double* __restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] += alpha * x[i];
}

__global__ void scale_kernel(double alpha, double* __restrict__ x, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= alpha;
}

}  // namespace

int reduction_scratch_doubles() { return kRedBlocks + 1; }

cudaError_t launch_dot(const double* x, const double* y, int64_t n, double* scratch, cudaStream_t stream) {
  dot_partial<<<kRedBlocks, kRedThreads, 0, stream>>>(x, y, n, scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  dot_final<<<1, kRedThreads, 0, stream>>>(scratch, kRedBlocks, scratch + kRedBlocks);
  return cudaGetLastError();
}

cudaError_t launch_dot_to(const double* x, const double* y, int64_t n, double* scratch, double* out,
                          cudaStream_t stream) {
  dot_partial<<<kRedBlocks, kRedThreads, 0, stream>>>(x, y, n, scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  dot_final<<<1, kRedThreads, 0, stream>>>(scratch, kRedBlocks, out);
  return cudaGetLastError();
}

// y -= (*c) x, the coefficient read on the device
__global__ void axpy_neg_dev_kernel(const double* __restrict__ c, const double* __restrict__ x, double* __restrict__ y,
                                    int64_t n) {
  const double a = -*c;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}

// b = sqrt(*nn), *b_out = b, x *= 1 / b
__global__ void normalize_dev_kernel(const double* __restrict__ nn, double* __restrict__ x, int64_t n,
                                     double* __restrict__ b_out) {
  const double b = sqrt(*nn);
  const double f = 1.0 / b;
  if (blockIdx.x == 0 && threadIdx.x == 0) *b_out = b;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= f;
}

cudaError_t launch_axpy_neg_dev(const double* c, const double* x, double* y, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4 * 152 * 4) blocks = 4 * 152 * 4;
  axpy_neg_dev_kernel<<<blocks, 256, 0, stream>>>(c, x, y, n);
  return cudaGetLastError();
}

cudaError_t launch_normalize_dev(const double* nn, double* x, int64_t n, double* b_out, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4 * 152 * 4) blocks = 4 * 152 * 4;
  normalize_dev_kernel<<<blocks, 256, 0, stream>>>(nn, x, n, b_out);
  return cudaGetLastError();
}

cudaError_t launch_axpy(double alpha, const double* x, double* y, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4 * 152 * 4) blocks = 4 * 152 * 4;
  axpy_kernel<<<blocks, 256, 0, stream>>>(alpha, x, y, n);
  return cudaGetLastError();
}

cudaError_t launch_scale(double alpha, double* x, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4 * 152 * 4) blocks = 4 * 152 * 4;
  scale_kernel<<<blocks, 256, 0, stream>>>(alpha, x, n);
  return cudaGetLastError();
}

}  // namespace su2g
