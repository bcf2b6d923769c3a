// Device work list of the block-sparse contraction engine.
//
// Every block product of the hot path has the form
//     C_tile = sum_s alpha_s * op(A_s) * B_s
// where B_s is stored K x N column-major and A_s is stored either K x M
// (transA = 1, the product uses A^T) or M x K (transA = 0), column-major.
// A tile is one (m0, n0) rectangle of one output block together with the
// contiguous run of segments that feed it.  Tiles are independent: each
// output element is written by exactly one tile, after all of its segments
// have been accumulated in registers, so the result does not depend on
// scheduling (no atomics, deterministic summation order).
//
// Addresses are (buffer, element offset) pairs so that one work list serves
// every application of a plan: buffer 0 holds absolute addresses (offset =
// byte address / 8, the operator blocks fixed at plan time), 1 = the input
// vector psi, 2 = the output vector y, 3 = the plan's scratch (intermediate
// blocks).  The kernels resolve them against the bases passed at launch.
#pragma once
#include <cstdint>

namespace su2g {

enum BufId : int { kBufAbs = 0, kBufPsi = 1, kBufY = 2, kBufScratch = 3, kNumBufs = 4 };

struct GemmSeg {
  int64_t a, b;   // element offsets of the A / B block origins
  int64_t a_len, b_len;  // elements of the A / B blocks (host-side bounds check)
  int a_buf, b_buf;
  int lda, ldb;
  int K;
  int transA;
  double alpha;
};

struct GemmTile {
  int64_t c;      // element offset of the C block origin
  int64_t c_len;  // elements of the C block (host-side bounds check)
  int c_buf;
  int ldc;
  int m0, n0;     // tile origin inside the block
  int mlen, nlen; // rows / columns of this tile (<= tile size)
  int seg0, nseg; // segments [seg0, seg0 + nseg)
  int64_t kwork;  // sum of K over the segments (scheduling weight)
  int cls;        // tile class (kTileClassM/N): the FP64 engine's tile shape
  int pad;
};

struct Bases {
  uintptr_t p[kNumBufs];
};

#if defined(__CUDACC__)
__host__ __device__
#endif
inline double* resolve(const Bases& b, int buf, int64_t off) {
  return reinterpret_cast<double*>(b.p[buf] + (uintptr_t)(off * 8));
}

constexpr int kTileM = 64;  // largest tile
constexpr int kTileN = 64;
// Tile classes of the FP64 engine: 64x64, 64x32, 32x64, 32x32.  Which class an
// output block uses follows its size class (a table an autotuner fills from
// measurements, tile_class_for in heff_plan.cpp).
constexpr int kTileClasses = 4;
constexpr int kTileClassM[kTileClasses] = {64, 64, 32, 32};
constexpr int kTileClassN[kTileClasses] = {64, 32, 64, 32};

}  // namespace su2g
