// Split-precision tile GEMM on the tcgen05 tensor cores (representation in
// ozaki.hpp).  A CTA computes 128 x 64 output tiles with three roles:
//
//   warp 16, lane 0 producer: bulk-copies the packed A (S slices x 128 x 16)
//                   and B (S slices x 64 x 16) units of each K stage into a
//                   kStages-deep shared-memory ring (cp.async.bulk + mbarrier
//                   transaction counts), running ahead of the MMAs;
//   warp 17, lane 0 MMA issuer: for every digit pair (p, q) with
//                   p + q <= S + 1, D[g = p+q] += A_p B_q^T (one BF16 MMA of
//                   K = 16), one FP32 TMEM accumulator of 128 lanes x 64
//                   columns per group g; frees each stage with a commit;
//   warps 0-15      epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (tile
//                   rows) and columns 16 (w / 4) .. + 15; after every K chunk
//                   of 560 (or segment end) it reads the S group sums of its
//                   16 columns (tcgen05.ld), converts them exactly to
//                   integers, weights them by 2^(48 - 7g) and adds them,
//                   aligned to the tile's largest product exponents, into 16
//                   int64 accumulators per thread; at the end each thread
//                   scales its 16 values to FP64 and stores them.  Four warps
//                   per SM sub-partition hide the latency of these chains.
//
// Every mbarrier wait is bounded; on time-out the CTA records an error code
// in *err, drains its outstanding tensor-core work and bulk copies (bounded)
// and returns.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "kernels.hpp"
#include "ozaki.hpp"

namespace su2g {
namespace oz {
namespace {

constexpr int kEpiWarps = 16;                      // drain warps: 4 lane quarters x 4 column slices
constexpr int kEpiThreads = kEpiWarps * 32;
constexpr int kCols = kTN / (kEpiWarps / 4);         // output columns per drain thread
constexpr int kProducerWarp = kEpiWarps, kMmaWarp = kEpiWarps + 1;
constexpr int kThreads = kEpiThreads + 64;           // + producer warp + MMA warp
constexpr long long kWaitIters = 1ll << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, long long limit = kWaitIters) {
  for (long long i = 0; i < limit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}

// K-major, no swizzle: core matrices 8 rows x 16 B; LBO = 128 B between
// K-adjacent cores, SBO = kSBO = 256 B between 8-row groups (16 k per stage).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)(128 >> 4) << 16;
  d |= (uint64_t)(kSBO >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// kind::f16, BF16 x BF16 -> FP32, both K-major, M = 128, N = n
__host__ __device__ constexpr uint32_t idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTM >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(a), "l"(b), "r"(id), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// an FP32 group sum is an integer below 2^24 in magnitude: the conversion is exact
__device__ __forceinline__ int f32_to_int_exact(uint32_t bits) { return __float2int_rn(__uint_as_float(bits)); }

// Weighted sum of one column's S group sums, v = sum_g G_g 2^(34 - 7g)
// (group g weighs 2^(kFixedTop - 7(g+2))), from their FP32 bit patterns, in
// few instructions: |G_g| <= 7 * 560 * 65^2 = 16,562,000 (the exactness bound
// of a chunk), so G_1 * 128 + G_2 and G_3 * 128 + G_4 are exact in int32
// (below 129 * 16,562,000 < 2^31) and only three 64-bit shift-adds remain:
//   v = G_0 2^34 + (G_1 2^7 + G_2) 2^20 + (G_3 2^7 + G_4) 2^6 + sum_{g>=5} G_g >> (7g - 34).
template <int S>
__device__ __forceinline__ long long combine_groups(const uint32_t (&r)[S][4], int x) {
  static_assert(S >= 5 && kFixedTop == 48 && kBits == 7, "group weights 2^34, 2^27, ... assumed");
  int G[S];
#pragma unroll
  for (int gg = 0; gg < S; ++gg) G[gg] = f32_to_int_exact(r[gg][x]);
  const int Y = G[1] * 128 + G[2];
  const int X = G[3] * 128 + G[4];
  int small = 0;
#pragma unroll
  for (int gg = 5; gg < S; ++gg) small += G[gg] >> (kBits * (gg + 2) - kFixedTop);
  return ((long long)G[0] << 34) + ((long long)Y << 20) + ((long long)X << 6) + (long long)small;
}

// ilogb of a nonzero finite double given as its bit pattern (sign ignored)
__device__ __forceinline__ int ilogb_bits(unsigned long long b) {
  b &= 0x7FFFFFFFFFFFFFFFull;
  const int E = (int)(b >> 52);
  if (E > 0) return E - 1023;
  return (63 - __clzll(b & 0xFFFFFFFFFFFFFull)) - 1074;
}

// v * 2^e rounded to nearest (ties to even), built with integer operations
// only (GB300 has little FP64 throughput); equal to ldexp((double)v, e)
// whenever the result is a normal number, and computed that way otherwise.
__device__ __forceinline__ double scaled_to_double(long long v, int e) {
  if (v == 0) return 0.0;
  const unsigned long long sign = (unsigned long long)v & 0x8000000000000000ull;
  unsigned long long u = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  const int lz = __clzll(u);
  u <<= lz;                        // leading one at bit 63
  unsigned long long m = u >> 11;  // 53 significant bits, leading one at bit 52
  const unsigned rem = (unsigned)(u & 0x7FFull);
  if (rem > 0x400u || (rem == 0x400u && (m & 1ull))) ++m;
  int ex = 63 - lz + e;  // value = m 2^-52 2^ex
  if (m >> 53) {
    m >>= 1;
    ++ex;
  }
  const int biased = ex + 1023;
  if (biased <= 0 || biased >= 2047) return ldexp((double)v, e);  // subnormal or overflowing: FP64 path
  return __longlong_as_double(
      (long long)(sign | ((unsigned long long)biased << 52) | (m & 0xFFFFFFFFFFFFFull)));
}

template <int S>
struct Smem {
  static constexpr int kA = a_unit_bytes(S);
  static constexpr int kB = b_unit_bytes(S);
  static constexpr int kStage = kA + kB;
  static constexpr int kBytes = kStages * kStage + 1024;  // + alignment slack
};

// rowmax_out is the exponent buffer again: the kernel writes only its
// row-maximum region (OzWork::rowmax_base ..), which it never reads through exps.
//
// Persistent: CTA b computes tiles b, b + gridDim.x, ... (heaviest first, as
// the planner sorts them).  The producer runs ahead across tile boundaries,
// the MMAs of tile i+1 start as soon as the drain warps have read tile i's
// last chunk, and the conversion and stores of tile i overlap them.
template <int S>
__global__ void __launch_bounds__(kThreads, 1) ozaki_gemm(const OzTile* __restrict__ tiles, int ntiles,
                                                          const OzSeg* __restrict__ segs,
                                                          const uint8_t* __restrict__ packed,
                                                          const int* __restrict__ exps, int* rowmax_out,
                                                          Bases bases, int* err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t bar_full[kStages], bar_empty[kStages], bar_accf, bar_acce, bar_drain;
  __shared__ uint32_t tmem_base_sh;
  __shared__ int fmax_sh[kTN];
  __shared__ int colmax_sh[kTN];  // row maxima handed to the next pack: per tile column
  __shared__ int cshift_sh[kMaxSegs];
  __shared__ int shb_sh[kEpiWarps][kCols];  // per drain warp: column shifts of the current segment
  __shared__ int abort_sh, loaded_sh, consumed_sh;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    for (int i = 0; i < kStages; ++i) {
      mbar_init(smem_u32(&bar_full[i]), 1);
      mbar_init(smem_u32(&bar_empty[i]), 1);
    }
    mbar_init(smem_u32(&bar_accf), 1);
    mbar_init(smem_u32(&bar_acce), kEpiWarps);
    mbar_init(smem_u32(&bar_drain), 1);
    abort_sh = 0;
    loaded_sh = 0;
    consumed_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;
  volatile int* abort_v = &abort_sh;
  auto stage_a = [&](int st) { return smem_u32(smem) + (uint32_t)(st * Smem<S>::kStage); };

  if (warp == kProducerWarp) {
    // ============================ producer ============================
    if (lane == 0) {
      int loaded = 0;
      bool ok = true;
      for (int ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
        const OzTile t = tiles[ti];
        for (int s = 0; s < t.nseg && ok; ++s) {
          const OzSeg g = segs[t.seg0 + s];
          for (int ks = 0; ks < g.nks; ++ks, ++loaded) {
            const int st = loaded % kStages;
            if (*abort_v) { ok = false; break; }
            // the stage's previous contents must have been consumed by their MMAs
            if (loaded >= kStages && !mbar_wait(smem_u32(&bar_empty[st]), ((loaded / kStages) - 1) & 1)) {
              ok = false;
              break;
            }
            const uint32_t a_dst = stage_a(st), b_dst = a_dst + Smem<S>::kA;
            mbar_expect_tx(smem_u32(&bar_full[st]), Smem<S>::kStage);
            bulk_g2s(a_dst, packed + g.a_unit + (int64_t)ks * a_unit_bytes(S), Smem<S>::kA,
                     smem_u32(&bar_full[st]));
            bulk_g2s(b_dst, packed + g.b_unit + (int64_t)ks * b_unit_bytes(S), Smem<S>::kB,
                     smem_u32(&bar_full[st]));
          }
        }
      }
      if (!ok) {
        atomicExch(err, 1);
        atomicExch(&abort_sh, 1);
      }
      loaded_sh = loaded;
    }
  } else if (warp == kMmaWarp) {
    // =========================== MMA issuer ===========================
    if (lane == 0) {
      int it = 0, chunk = 0;
      bool ok = true;
      for (int ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
        const OzTile t = tiles[ti];
        for (int s = 0; s < t.nseg && ok; ++s) {
          const int nks = segs[t.seg0 + s].nks;
          for (int ks = 0; ks < nks; ++ks, ++it) {
            const int st = it % kStages;
            if (*abort_v || !mbar_wait(smem_u32(&bar_full[st]), (it / kStages) & 1)) { ok = false; break; }
            const bool first = (ks % kChunkStages) == 0;
            // a new chunk overwrites the group sums: the epilogue must have read them
            if (first && chunk > 0 && !mbar_wait(smem_u32(&bar_acce), (chunk - 1) & 1)) {
              ++it;  // this stage was waited for: it counts as consumed
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sa = stage_a(st), sb = sa + Smem<S>::kA;
            // The B digit slices lie back to back (64 rows each, same core-row
            // stride) and so do the group accumulators in TMEM (64 columns
            // each): the pairs (p, q) .. (p, q+n-1) are one MMA of N = 64 n that
            // reads B_q .. B_{q+n-1} as one 64n-row operand and adds into groups
            // p+q .. p+q+n-1.  Up to n = 4 (N = 256): 10 MMAs per stage for S = 7
            // instead of 28, and A is read once per MMA.  p = 1 touches every
            // group first, so only its MMAs start a chunk's sums from zero.
#pragma unroll
            for (int p = 1; p <= S; ++p) {
              const uint64_t ad = smem_desc(sa + (p - 1) * (kTM * kKS * 2));
              // partners of p split into MMAs of at most four slices; five
              // go as 3 + 2, not 4 + 1 (an N = 64 MMA costs more than its
              // width: 3.81 instead of 3.85 ms per D = 2000 application;
              // 6 = 3 + 3 measured no better than 4 + 2)
              const int np = S + 1 - p;
              const int n1 = np <= 4 ? np : (np == 5 ? 3 : 4);
              mma(tmem + (uint32_t)((p - 1) * kTN), ad, smem_desc(sb), idesc(kTN * n1), (first && p == 1) ? 0u : 1u);
              if (np > n1)
                mma(tmem + (uint32_t)((p - 1 + n1) * kTN), ad, smem_desc(sb + n1 * (kTN * kKS * 2)),
                    idesc(kTN * (np - n1)), (first && p == 1) ? 0u : 1u);
            }
            mma_commit(smem_u32(&bar_empty[st]));
            if ((ks % kChunkStages) == kChunkStages - 1 || ks == nks - 1) {
              mma_commit(smem_u32(&bar_accf));
              ++chunk;
            }
          }
        }
      }
      if (!ok) {
        atomicExch(err, 1);
        atomicExch(&abort_sh, 1);
      }
      consumed_sh = it;
      // drain: every MMA issued so far has completed once this commit arrives
      mma_commit(smem_u32(&bar_drain));
      if (!mbar_wait(smem_u32(&bar_drain), 0)) atomicExch(err, 2);
    }
  } else {
    // ============================ epilogue ============================
    // Every drain warp walks the same tiles, segments and chunks and takes the
    // same named barriers whatever happens: after a wait that gave up it goes
    // on without waiting or reading TMEM, so no warp is ever left at a barrier.
    const int lq = warp & 3, col0 = (warp >> 2) * kCols;
    const int row = lq * 32 + lane;  // TMEM lane == tile row
    const uint32_t lane_base = (uint32_t)(lq * 32) << 16;
    int chunk = 0;
    bool ok = true;
    for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
      const OzTile t = tiles[ti];
      // Exponent bookkeeping.  Segment s contributes 2^(eA_s(i) + eB_s(j))
      // times its digit sums; moving c_s = max_i eA_s(i) (over the tile rows)
      // from the A side to the B side leaves every product unchanged but makes
      // the tile's reference exponents emax(i) = max_s (eA_s(i) - c_s) and
      // fmax(j) = max_s (eB_s(j) + c_s) track the largest actual product scale
      // (otherwise an O(1) x O(1e-3) segment and an O(1e-3) x O(1) segment
      // would set a reference 2^10 above both).  c_s = the A row tile's largest
      // exponent, recorded by the pack kernel.
      for (int s = tid; s < t.nseg; s += kEpiThreads) {
        const int m = exps[segs[t.seg0 + s].a_tmax];
        cshift_sh[s] = (m == kExpZero) ? 0 : m;
      }
      if (tid < kTN) colmax_sh[tid] = 0;
      asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
      int emax = kExpZero;
#pragma unroll 8
      for (int s = 0; s < t.nseg; ++s) {
        const int e = exps[segs[t.seg0 + s].a_exp + row];
        if (e != kExpZero) emax = max(emax, e - cshift_sh[s]);
      }
      if (tid < kTN) {
        int f = kExpZero;
#pragma unroll 8
        for (int s = 0; s < t.nseg; ++s) {
          const int fb = exps[segs[t.seg0 + s].b_exp + tid];
          if (fb != kExpZero) f = max(f, fb + cshift_sh[s]);
        }
        fmax_sh[tid] = f;
      }
      asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
      long long acc[kCols];
#pragma unroll
      for (int j = 0; j < kCols; ++j) acc[j] = 0;
      for (int s = 0; s < t.nseg; ++s) {
        const OzSeg g = segs[t.seg0 + s];
        const int ea = exps[g.a_exp + row];
        const int cs = cshift_sh[s];
        const int sha = (ea == kExpZero) ? 1000 : emax - (ea - cs);
        // column shifts of this segment, staged per warp (no block barrier)
        __syncwarp();
        if (lane < kCols) {
          const int fj = exps[g.b_exp + col0 + lane];
          shb_sh[warp][lane] = (fj == kExpZero) ? 1000 : fmax_sh[col0 + lane] - (fj + cs);
        }
        __syncwarp();
        const int nchunks = (g.nks + kChunkStages - 1) / kChunkStages;
        for (int c = 0; c < nchunks; ++c, ++chunk) {
          if (ok && !mbar_wait(smem_u32(&bar_accf), chunk & 1)) ok = false;
          if (!ok) continue;
          tc_fence_after();
#pragma unroll
          for (int cb = 0; cb < kCols / 4; ++cb) {
            // all S group sums of 4 columns in flight, one wait
            uint32_t r[S][4];
#pragma unroll
            for (int gg = 0; gg < S; ++gg)
              tmem_ld4(tmem + lane_base + (uint32_t)(gg * kTN + col0 + cb * 4), r[gg]);
            tmem_wait_ld();
#pragma unroll
            for (int x = 0; x < 4; ++x) {
              const long long v = combine_groups<S>(r, x);
              const int j = cb * 4 + x;
              const int sh = sha + shb_sh[warp][j];
              if (sh == 0) {
                acc[j] += v;
              } else if (sh < 63) {
                acc[j] += ((v >> (sh - 1)) + 1) >> 1;  // = (v + 2^(sh-1)) >> sh: round to nearest
              }
            }
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(&bar_acce));
        }
      }
      // ---- store: C = acc * 2^(emax + fmax - kFixedTop) ----
      // A phase-1 block that becomes a phase-2 operand also leaves, per
      // operand row (block columns i*rms ..), the largest ilogb of its values,
      // so that the pack needs no pass of its own over the block.
      double* C = resolve(bases, t.c_buf, t.c);
      const int ebase = emax - kFixedTop;
      int lg[kCols];  // kRowmaxBias-coded ilogb |value|, 0 for a zero or absent value
      if (row < t.mlen) {
#pragma unroll
        for (int jj = 0; jj < kCols; ++jj) {
          const int j = col0 + jj;
          lg[jj] = 0;
          if (j < t.nlen) {
            const int f = fmax_sh[j];
            double out = 0.0;
            if (ok && emax != kExpZero && f != kExpZero) out = scaled_to_double(acc[jj], ebase + f);
            C[(int64_t)(t.m0 + row) + (int64_t)(t.n0 + j) * t.ldc] = out;
            const unsigned long long ob = (unsigned long long)__double_as_longlong(out);
            if (t.rowmax >= 0 && (ob & 0x7FFFFFFFFFFFFFFFull)) lg[jj] = ilogb_bits(ob) + kRowmaxBias;
          }
        }
      } else {
#pragma unroll
        for (int jj = 0; jj < kCols; ++jj) lg[jj] = 0;
      }
      if (t.rowmax >= 0) {  // uniform over the CTA
        // column maxima: over the warp's rows (lane jj keeps column jj), over
        // the four lane quarters (shared memory), then one global atomic per
        // column
        int mine = 0;
#pragma unroll
        for (int jj = 0; jj < kCols; ++jj) {
          const int m = (int)__reduce_max_sync(0xffffffffu, (unsigned)lg[jj]);
          if (lane == jj) mine = m;
        }
        if (lane < kCols && mine > 0) atomicMax(&colmax_sh[col0 + lane], mine);
        asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
        if (tid < t.nlen && colmax_sh[tid] > 0)
          atomicMax(&rowmax_out[t.rowmax + (t.n0 + tid) / t.rms], colmax_sh[tid]);
      }
      // the next tile's bookkeeping rewrites the shared tile state
      asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
    }
    if (!ok) {
      atomicExch(err, 3);
      atomicExch(&abort_sh, 1);
    }
  }
  tc_fence_before();
  __syncthreads();
  // bulk copies still in flight (possible only after an abort) must land
  // before the CTA exits: at most one unconsumed load per stage
  if (warp == kProducerWarp && lane == 0 && abort_sh)
    for (int i = consumed_sh; i < loaded_sh; ++i) mbar_wait(smem_u32(&bar_full[i % kStages]), (i / kStages) & 1);
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

}  // namespace

int gemm_smem_bytes(int S) {
  switch (S) {
    case 6: return Smem<6>::kBytes;
    case 7: return Smem<7>::kBytes;
    case 8: return Smem<8>::kBytes;
  }
  return 0;
}

namespace {
// The GEMM's bounded wait on an mbarrier that nothing arrives at: it must give
// up after `limit` polls and report it, leaving the context usable.
__global__ void bounded_wait_selftest_kernel(long long limit, int* timed_out) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *timed_out = mbar_wait(smem_u32(&bar), 0, limit) ? 0 : 1;
  }
}
}  // namespace

cudaError_t bounded_wait_selftest(long long limit, int* timed_out_host, cudaStream_t stream) {
  int* d = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&d, sizeof(int), stream);
  if (e != cudaSuccess) return e;
  bounded_wait_selftest_kernel<<<1, 32, 0, stream>>>(limit, d);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(timed_out_host, d, sizeof(int), cudaMemcpyDeviceToHost, stream);
  cudaFreeAsync(d, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  return e;
}

namespace {
int g_sms = 0;            // one resident CTA per SM (shared memory and TMEM): a persistent grid
bool g_prepared[9] = {};  // per S
std::mutex g_prep_mu;
}  // namespace

int ozaki_persistent_grid() {
  static std::once_flag once;
  static int grid = 152;
  std::call_once(once, [] {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
        n > 0)
      grid = n;
    else
      cudaGetLastError();  // no device here: clear the error it left
  });
  return grid;
}

cudaError_t prepare_ozaki_gemm(int S) {
  if (S != 6 && S != 7) return cudaErrorInvalidValue;
  std::lock_guard<std::mutex> lock(g_prep_mu);
  if (g_prepared[S]) return cudaSuccess;
  int dev = 0, n = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  g_sms = n > 0 ? n : 148;
  const int smem = gemm_smem_bytes(S);
  e = S == 6 ? cudaFuncSetAttribute(ozaki_gemm<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)
             : cudaFuncSetAttribute(ozaki_gemm<7>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) g_prepared[S] = true;
  return e;
}

cudaError_t launch_ozaki_gemm(int S, const OzTile* tiles, int ntiles, const OzSeg* segs, const uint8_t* packed,
                              int* exps, const Bases& bases, int* err, cudaStream_t stream) {
  if (ntiles <= 0) return cudaSuccess;
  cudaError_t e = prepare_ozaki_gemm(S);
  if (e != cudaSuccess) return e;
  const int grid = ntiles < g_sms ? ntiles : g_sms;
  const int smem = gemm_smem_bytes(S);
  if (S == 6)
    ozaki_gemm<6><<<grid, kThreads, smem, stream>>>(tiles, ntiles, segs, packed, exps, exps, bases, err);
  else
    ozaki_gemm<7><<<grid, kThreads, smem, stream>>>(tiles, ntiles, segs, packed, exps, exps, bases, err);
  return cudaGetLastError();
}

}  // namespace oz
}  // namespace su2g
