// Split-precision contraction engine: FP64 block products emulated with BF16
// digit slices on the tcgen05 tensor cores (the error-free splitting of
// Ozaki, Ogita, Oishi & Rump, "Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59 (2012), with integer digits and exact
// FP32 group sums).
//
// Representation.  Every operand X (R rows x K, the contraction index K) is
// scaled per row by 2^-e_r so that |X_rk| 2^-e_r < 1/2, rounded to the
// integer N_rk = rint(X_rk 2^(7S - e_r)) and written as S balanced base-128
// digits  N = sum_p d_p 2^(7(S-p)),  |d_p| <= 64 (65 for the leading digit),
// each exact in BF16.
// A product C = A B^T then is
//     C_ij = 2^(e_i + f_j - 7(S+1)) sum_{g=2}^{S+1} 2^(7(S+1-g)) G_g(i,j),
//     G_g  = sum_{p+q=g} sum_k dA_p(i,k) dB_q(j,k)
// (pairs with p+q > S+1 are dropped: they weigh below 2^-7(S+2)).  With
// |d| <= 65 and at most S <= 7 pairs per group, a group summed over 560
// values of k stays below 7 * 560 * 65^2 = 16,562,000 < 2^24 in magnitude
// (every partial sum too), so the FP32 tensor-core accumulation of one group
// over one K chunk of 560 is exact, and the chunk sums are combined in 64-bit
// integers, C = 2^(e_i + f_j - 48) sum_g 2^(48 - 7g) G_g.  The only
// rounding is in forming N (2^-48 relative to the row maximum for S = 7), in
// the dropped pairs, and in aligning products of different exponents to the
// tile's common fixed point (2^-46 of the tile's largest product).
//
// Packed operand layout (bytes), built by the pack kernel:
//   [row tile rt][k tile kt][slice p][rows RT x 16 k, tcgen05 canonical
//   no-swizzle K-major layout: 8x8 core matrices, core (r/8, k/8) at
//   (r/8)*256 + (k/8)*128, element (r%8, k%8) at (r%8)*16 + (k%8)*2]
// with RT = 128 for the A (M) role and 64 for the B (N) role, rows padded to
// RT and K padded to 16 with zeros; one int32 exponent per (padded) row.
#pragma once
#include <cstdint>

#include "gemm_work.hpp"

#if defined(__CUDACC__)
#define SU2G_HD __host__ __device__
#else
#define SU2G_HD
#endif

namespace su2g {
namespace oz {

constexpr int kBits = 7;            // bits per digit
constexpr int kTM = 128;            // tile rows (MMA M)
constexpr int kTN = 64;             // tile columns (MMA N)
constexpr int kKS = 16;             // K per packed unit and shared-memory stage (one MMA deep)
constexpr int kSBO = 8 * kKS * 2;   // bytes between 8-row core groups of a unit
constexpr int kChunkStages = 35;    // exact FP32 group sums over 35 stages = 560 k
constexpr int kStages = 4;          // shared-memory ring depth of the tile GEMM
constexpr int kExpZero = -(1 << 20);  // exponent of an all-zero row
constexpr int kFixedTop = 48;         // fixed point: group g weighs 2^(kFixedTop - 7g)
constexpr int kMaxSegs = 1024;        // segments feeding one output tile
constexpr int kTargetCtas = 4 * 152;  // phase-2 tiles are split until about this many CTAs run
constexpr int kRowmaxBias = 2048;     // row-maximum slots hold ilogb + 2048; 0 = no nonzero element

SU2G_HD constexpr int pairs(int S) { return S * (S + 1) / 2; }
SU2G_HD constexpr int a_unit_bytes(int S) { return S * kTM * kKS * 2; }
SU2G_HD constexpr int b_unit_bytes(int S) { return S * kTN * kKS * 2; }

// One FP64 operand to split: X(r, k) = alpha * src[r*ld_r + k*ld_k].
struct PackJob {
  int64_t src;       // element offset in buffer src_buf (gemm_work.hpp buffer ids)
  int src_buf;
  int R, K;
  int64_t ld_r, ld_k;
  int rt;            // 128 (A role) or 64 (B role)
  int nrt, nkt;      // row tiles, k tiles
  double alpha;
  int64_t dst;       // byte offset in the packed buffer (multiple of 1024)
  int64_t exp;       // int32 offset in the exponent buffer (nrt*rt entries)
  int64_t texp;      // int32 offset of the per-row-tile maxima (nrt entries)
  int64_t rowmax;    // int32 offset of per-row ilogb maxima left by the GEMM that
                     // produced the operand (R entries, kRowmaxBias-coded), -1: none
};

// One K segment of an output tile: both operands already packed.
struct OzSeg {
  int64_t a_unit;    // byte offset of this tile's A row tile, k tile 0
  int64_t b_unit;    // byte offset of this tile's B row tile, k tile 0
  int64_t a_exp;     // exponent index of the tile's first A row
  int64_t b_exp;     // exponent index of the tile's first B row
  int64_t a_tmax;    // exponent index of the largest exponent of the A row tile
  int nks;           // k tiles (stages) of this segment
  int pad;
};

// Sum of the partial tiles of one split output tile into its destination.
struct RedTile {
  int64_t c;         // element offset of the destination block origin
  int c_buf;
  int ldc;
  int m0, n0, mlen, nlen;
  int nparts;
  int64_t part;      // scratch offset of the first partial (kTM x kTN doubles each, ldc = kTM)
};

struct OzTile {
  int64_t c;         // element offset of the C block origin
  int c_buf;
  int ldc;
  int m0, n0, mlen, nlen;
  int seg0, nseg;
  int64_t work;      // sum of nks over the segments (scheduling weight)
  int64_t rowmax;    // phase-1 tiles: row-maximum slots of the operand this block
                     // becomes in phase 2 (its row i = columns i*rms .. of the block), -1: none
  int rms;
  int pad2;
};

}  // namespace oz
}  // namespace su2g
