// The wave-function moves between two steps of a sweep:
//   * wavefunc_transformation (dmrg_su2_omp.cpp:1864-1876): the MPS tensor
//     next to the new centre changes which of its legs are fused into the
//     third, tensor_su2::right2left_vectran / left2right_vectran
//     (tensor_su2.cpp:749-837).  Each block keeps its numbers: its legs are
//     rotated and its CG is replaced by the canonical one of the rotated spins
//     (make_cgc), with no recoupling factor, then the directions are set to
//     (+1, +1, -1).  A rotation of the legs of a column-major block is a
//     matrix transpose: right2left sees a block as (d0 d1) x d2, left2right
//     as d0 x (d1 d2).
//   * prepare_input_vector (dmrg_su2_omp.cpp:229-254): the initial two-site
//     vector of the step, per centre spin c the product U_L,c U_R,c^T of the
//     two MPS tensors' fused-row matrices (the fuse, overlap_initial and
//     contract of the reference meet in this one product, with canonical CG
//     and factor 1).  U_R,c^T is the right2left rotation of ur's blocks, so
//     the call transposes ur once and runs the products as a work list of the
//     block-sparse engine (FP64 or split BF16).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "env_plan.hpp"
#include "kernels.hpp"
#include "su2_meta.hpp"
#include "su2g.h"

namespace {

int fail(int code, const std::string& msg) { return su2g::set_last_error(code, msg); }
int cuda_fail(cudaError_t e, const char* where) {
  return fail(e == cudaErrorMemoryAllocation ? SU2G_ENOMEM : SU2G_ECUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
      n = v;
    if (n <= 0) n = 152;
  }
  return n;
}

// one block to transpose: src rows x cols (column-major) -> dst cols x rows
struct TrItem {
  const double* src;
  double* dst;
  int rows, cols;
  int tiles_r;     // 32-row tiles along rows
  int64_t tile0;   // first global tile index of this block
};

constexpr int kTr = 32;          // tile edge
constexpr int kTrThreads = 256;  // 32 x 8

// Up to kParamItems blocks travel in the kernel's parameters (no upload);
// longer lists are copied to the device first.
constexpr int kParamItems = 160;  // 160 x 40 bytes: within the 32 KB parameter space
struct TrList {
  TrItem item[kParamItems];
};

// Global tiles are walked with a grid-stride loop; a CTA finds its block by a
// binary search of the tile prefix.  Reads are coalesced along the source
// column, writes along the destination column, through a padded 32 x 33 tile.
__device__ __forceinline__ void transpose_tiles(const TrItem* __restrict__ items, int nitems, int64_t ntiles) {
  __shared__ double tile[kTr][kTr + 1];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    int lo = 0, hi = nitems - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (items[mid].tile0 <= t) lo = mid;
      else hi = mid - 1;
    }
    const TrItem it = items[lo];
    const int64_t local = t - it.tile0;
    const int r0 = (int)(local % it.tiles_r) * kTr, c0 = (int)(local / it.tiles_r) * kTr;
    __syncthreads();  // the previous tile's reads of `tile` are done
#pragma unroll
    for (int q = 0; q < kTr; q += 8) {
      const int r = r0 + tx, c = c0 + ty + q;
      if (r < it.rows && c < it.cols) tile[ty + q][tx] = it.src[r + (int64_t)c * it.rows];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kTr; q += 8) {
      const int c = c0 + tx, r = r0 + ty + q;  // dst (c, r) at dst[c + r * cols]
      if (r < it.rows && c < it.cols) it.dst[c + (int64_t)r * it.cols] = tile[tx][ty + q];
    }
  }
}

__global__ void __launch_bounds__(kTrThreads) transpose_blocks_kernel(const TrItem* __restrict__ items, int nitems,
                                                                      int64_t ntiles) {
  transpose_tiles(items, nitems, ntiles);
}

__global__ void __launch_bounds__(kTrThreads) transpose_blocks_param_kernel(const __grid_constant__ TrList list,
                                                                            int nitems, int64_t ntiles) {
  transpose_tiles(list.item, nitems, ntiles);
}

// Runs the transposes of `items` (host list; tile0 filled here) on `st`.
cudaError_t launch_transposes(std::vector<TrItem>& items, cudaStream_t st) {
  std::vector<TrItem> live;
  int64_t ntiles = 0;
  for (TrItem it : items) {
    if (it.rows <= 0 || it.cols <= 0) continue;
    it.tiles_r = (it.rows + kTr - 1) / kTr;
    it.tile0 = ntiles;
    ntiles += (int64_t)it.tiles_r * ((it.cols + kTr - 1) / kTr);
    live.push_back(it);
  }
  if (live.empty()) return cudaSuccess;
  const int grid = (int)std::min<int64_t>(ntiles, (int64_t)sm_count() * 8);
  if ((int)live.size() <= kParamItems) {
    TrList list;
    std::copy(live.begin(), live.end(), list.item);
    transpose_blocks_param_kernel<<<grid, kTrThreads, 0, st>>>(list, (int)live.size(), ntiles);
    return cudaGetLastError();
  }
  TrItem* d_items = nullptr;
  const size_t bytes = live.size() * sizeof(TrItem);
  cudaError_t e = cudaMallocAsync((void**)&d_items, bytes, st);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(d_items, live.data(), bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    transpose_blocks_kernel<<<grid, kTrThreads, 0, st>>>(d_items, (int)live.size(), ntiles);
    e = cudaGetLastError();
  }
  // the host list must outlive the copy
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(d_items, st);
  return e;
}

// One identity placement of a fuse tensor: block rows r (< rows) carry a 1 in
// column r + shift (tensor::shift_set_identity, tensor.cpp:1411-1432).
struct OneItem {
  double* blk;
  int rows, shift;
};

__global__ void place_ones_kernel(const OneItem* __restrict__ items, int n) {
  const OneItem it = items[blockIdx.y];
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < it.rows; r += gridDim.x * blockDim.x)
    it.blk[r + (int64_t)(r + it.shift) * it.rows] = 1.0;
}

__global__ void fill_kernel(double* x, int64_t n, double v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] = v;
}

// fuse tensor of the two legs of a 2-leg desc: legs (b1, b2, fuse(b1, b2)),
// every legal block present (tensor_su2::fuse, tensor_su2.cpp:839-909)
int fuse_struct(const int* bonds_desc, su2g::Struct* out, std::string* err) {
  su2g::Struct b;
  if (!bonds_desc || !b.parse(bonds_desc, err)) return SU2G_EINVAL;
  if (b.nbond != 2) {
    *err = "two bonds expected";
    return SU2G_EINVAL;
  }
  if (b.legs[0].dir != b.legs[1].dir) {  // su2bond::fuse refuses them (su2bond.cpp:159-162)
    *err = "bonds of different directions";
    return SU2G_EINVAL;
  }
  *out = su2g::Struct();
  out->nbond = 3;
  out->locspin = 0;
  out->legs[0] = b.legs[0];
  out->legs[1] = b.legs[1];
  out->legs[2] = su2g::fuse(b.legs[0], b.legs[1]);
  out->nten = out->legs[0].n() * out->legs[1].n() * out->legs[2].n();
  out->set_layout(nullptr);
  return SU2G_OK;
}

int write_layout(const su2g::Struct& s, int* out_desc, int out_desc_cap, int* out_flag, int out_flag_cap,
                 int64_t* out_len, const char* what) {
  std::vector<int> d = {s.nbond, s.locspin};
  for (int l = 0; l < s.nbond; ++l) {
    d.push_back(s.legs[l].dir);
    d.push_back(s.legs[l].n());
    for (int a : s.legs[l].angm) d.push_back(a);
    for (int x : s.legs[l].dim) d.push_back(x);
  }
  if (!out_desc || !out_flag || (int)d.size() > out_desc_cap || s.nten > out_flag_cap)
    return fail(SU2G_EINVAL, std::string(what) + ": output arrays too small");
  std::copy(d.begin(), d.end(), out_desc);
  std::copy(s.flag.begin(), s.flag.end(), out_flag);
  if (out_len) *out_len = s.total;
  return SU2G_OK;
}

// Structure of the rotated tensor and, per stored block, its transpose.
// flag 0 = right2left (legs (0,1,2) -> (2,0,1)), 1 = left2right (-> (1,2,0)).
int vectran_struct(const su2g_tensor& u, int flag, su2g::Struct* in, su2g::Struct* out, std::string* err) {
  if (flag != 0 && flag != 1) {
    *err = "vectran: flag must be 0 (right2left) or 1 (left2right)";
    return SU2G_EINVAL;
  }
  if (!u.desc || !in->parse(u.desc, err)) {
    *err = "vectran: " + *err;
    return SU2G_EINVAL;
  }
  if (in->nbond != 3) {
    *err = "vectran: a 3-leg tensor expected";
    return SU2G_EINVAL;
  }
  in->set_layout(u.flag);
  const int shift = flag == 0 ? 1 : 2;  // old leg q -> new leg (q + shift) % 3
  *out = su2g::Struct();
  out->nbond = 3;
  out->locspin = in->locspin;
  for (int q = 0; q < 3; ++q) out->legs[(q + shift) % 3] = in->legs[q];
  out->legs[0].dir = 1;
  out->legs[1].dir = 1;
  out->legs[2].dir = -1;
  out->nten = in->nten;
  std::vector<int> f(out->nten, 0);
  for (int b = 0; b < in->nten; ++b) {
    if (!in->flag[b]) continue;
    int sec[3], ns[3];
    in->sectors(b, sec);
    for (int q = 0; q < 3; ++q) ns[(q + shift) % 3] = sec[q];
    f[out->index(ns)] = 1;
  }
  out->set_layout(f.data());
  return SU2G_OK;
}

// transposes of every stored block of `in` into its rotated place in `out`
std::vector<TrItem> vectran_items(const su2g::Struct& in, const su2g::Struct& out, int flag, const double* src,
                                  double* dst) {
  const int shift = flag == 0 ? 1 : 2;
  std::vector<TrItem> items;
  for (int b = 0; b < in.nten; ++b) {
    if (!in.flag[b]) continue;
    int sec[3], ns[3];
    in.sectors(b, sec);
    for (int q = 0; q < 3; ++q) ns[(q + shift) % 3] = sec[q];
    const int d0 = in.block_dim(b, 0), d1 = in.block_dim(b, 1), d2 = in.block_dim(b, 2);
    TrItem it{};
    it.src = src + in.offset[b];
    it.dst = dst + out.offset[out.index(ns)];
    it.rows = flag == 0 ? d0 * d1 : d0;
    it.cols = flag == 0 ? d2 : d1 * d2;
    items.push_back(it);
  }
  return items;
}

}  // namespace

extern "C" int su2g_vectran_layout(su2g_tensor u, int flag, int* out_desc, int out_desc_cap, int* out_flag,
                                   int out_flag_cap, int64_t* out_len) {
  su2g::Struct in, out;
  std::string err;
  int rc = vectran_struct(u, flag, &in, &out, &err);
  if (rc) return fail(rc, err);
  return write_layout(out, out_desc, out_desc_cap, out_flag, out_flag_cap, out_len, "vectran_layout");
}

extern "C" int su2g_vectran(su2g_tensor u, int flag, double* out, void* stream) {
  su2g::Struct in, o;
  std::string err;
  int rc = vectran_struct(u, flag, &in, &o, &err);
  if (rc) return fail(rc, err);
  if (in.total == 0) return SU2G_OK;
  if (!u.data || !out) return fail(SU2G_EINVAL, "vectran: null data");
  cudaStream_t st = (cudaStream_t)stream;
  // in place (the reference rotates uu[i] itself): transpose from a copy
  const double* src = u.data;
  double* copy = nullptr;
  cudaError_t e = cudaSuccess;
  const bool overlap = out < u.data + in.total && u.data < out + in.total;
  if (overlap) {
    e = cudaMallocAsync((void**)&copy, in.total * sizeof(double), st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(copy, u.data, in.total * sizeof(double), cudaMemcpyDeviceToDevice, st);
    src = copy;
  }
  if (e == cudaSuccess) {
    std::vector<TrItem> items = vectran_items(in, o, flag, src, out);
    e = launch_transposes(items, st);
  }
  if (copy) cudaFreeAsync(copy, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "vectran");
  return SU2G_OK;
}

extern "C" int su2g_input_vector_layout(su2g_tensor ul, su2g_tensor ur, int* out_desc, int out_desc_cap,
                                        int* out_flag, int out_flag_cap, int64_t* out_len) {
  su2g::Struct v;
  su2g::HeffWork w;
  std::string err;
  int rc = su2g::build_input_vector(ul, ur, nullptr, nullptr, &v, &w, &err);
  if (rc) return fail(rc, err);
  return write_layout(v, out_desc, out_desc_cap, out_flag, out_flag_cap, out_len, "input_vector_layout");
}

extern "C" int su2g_prepare_input_vector(su2g_tensor ul, su2g_tensor ur, double* out, int mode, void* stream) {
  su2g::Struct v, R, Rt;
  su2g::HeffWork w;
  std::string err;
  // structures first (argument errors before any device work)
  int rc = su2g::build_input_vector(ul, ur, nullptr, nullptr, &v, &w, &err);
  if (rc) return fail(rc, err);
  if (v.total == 0) return SU2G_OK;
  if (!out) return fail(SU2G_EINVAL, "prepare_input_vector: null output");
  rc = vectran_struct(ur, 0, &R, &Rt, &err);
  if (rc) return fail(rc, err);
  cudaStream_t st = (cudaStream_t)stream;
  double* urt = nullptr;  // ur's blocks transposed, at ur's own offsets
  cudaError_t e = cudaMemsetAsync(out, 0, v.total * sizeof(double), st);
  if (e == cudaSuccess && R.total > 0) e = cudaMallocAsync((void**)&urt, R.total * sizeof(double), st);
  if (e == cudaSuccess && R.total > 0) {
    std::vector<TrItem> items;
    for (int b = 0; b < R.nten; ++b) {
      if (!R.flag[b]) continue;
      TrItem it{};
      it.src = ur.data + R.offset[b];
      it.dst = urt + R.offset[b];
      it.rows = R.block_dim(b, 0) * R.block_dim(b, 1);
      it.cols = R.block_dim(b, 2);
      items.push_back(it);
    }
    e = launch_transposes(items, st);
  }
  if (e == cudaSuccess) {
    rc = su2g::build_input_vector(ul, ur, urt, out, &v, &w, &err, mode == SU2G_MODE_F64);
    if (rc) rc = fail(rc, err);
    else rc = su2g::run_work_once(std::move(w), mode, stream);
  }
  if (urt) cudaFreeAsync(urt, st);
  cudaError_t e2 = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return cuda_fail(e, "prepare_input_vector");
  return rc;
}

extern "C" int su2g_fuse_tensor_layout(const int* bonds_desc, int* out_desc, int out_desc_cap, int* out_flag,
                                       int out_flag_cap, int64_t* out_len) {
  su2g::Struct f;
  std::string err;
  if (fuse_struct(bonds_desc, &f, &err)) return fail(SU2G_EINVAL, "fuse_tensor: " + err);
  return write_layout(f, out_desc, out_desc_cap, out_flag, out_flag_cap, out_len, "fuse_tensor_layout");
}

extern "C" int su2g_fuse_tensor(const int* bonds_desc, double* out, void* stream) {
  su2g::Struct f;
  std::string err;
  if (fuse_struct(bonds_desc, &f, &err)) return fail(SU2G_EINVAL, "fuse_tensor: " + err);
  if (f.total == 0) return SU2G_OK;
  if (!out) return fail(SU2G_EINVAL, "fuse_tensor: null output");
  std::vector<OneItem> items;
  for (int b = 0; b < f.nten; ++b) {
    if (!f.flag[b]) continue;
    int sec[3];
    f.sectors(b, sec);
    const int c = f.legs[2].angm[sec[2]];
    const int r0 = su2g::fused_row(f.legs[0], f.legs[1], c, sec[0], sec[1]);
    if (r0 < 0) return fail(SU2G_EINVAL, "fuse_tensor: internal placement error");
    items.push_back(OneItem{out + f.offset[b], f.legs[0].dim[sec[0]] * f.legs[1].dim[sec[1]], r0});
  }
  cudaStream_t st = (cudaStream_t)stream;
  OneItem* d_items = nullptr;
  cudaError_t e = cudaMemsetAsync(out, 0, f.total * sizeof(double), st);
  if (e == cudaSuccess && items.size() > 65535) e = cudaErrorInvalidValue;
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_items, items.size() * sizeof(OneItem), st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(OneItem), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    int maxr = 1;
    for (const OneItem& it : items) maxr = std::max(maxr, it.rows);
    place_ones_kernel<<<dim3((maxr + 255) / 256, (unsigned)items.size()), 256, 0, st>>>(d_items, (int)items.size());
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host list must outlive the copy
  if (d_items) cudaFreeAsync(d_items, st);
  if (e != cudaSuccess) return cuda_fail(e, "fuse_tensor");
  return SU2G_OK;
}

extern "C" int su2g_initial_vector(su2g_tensor ul, su2g_tensor ur, double* out, void* stream) {
  su2g::Struct v;
  su2g::HeffWork w;
  std::string err;
  int rc = su2g::build_input_vector(ul, ur, nullptr, nullptr, &v, &w, &err);
  if (rc) return fail(rc, "initial_vector: " + err);
  if (v.total == 0) return SU2G_OK;
  if (!out) return fail(SU2G_EINVAL, "initial_vector: null output");
  cudaStream_t st = (cudaStream_t)stream;
  const int grid = (int)std::min<int64_t>((v.total + 255) / 256, (int64_t)sm_count() * 4);
  fill_kernel<<<grid, 256, 0, st>>>(out, v.total, 1.0 / std::sqrt((double)v.total));
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "initial_vector");
  return SU2G_OK;
}


// ------------------------------------------------- seeded random start vector
// tensor_su2::random_initialize_tensor (tensor_su2.cpp:2375-2393): every
// stored block filled with ran()*2 - 1 in block order, each block column-major
// (tensor::random_init, tensor.cpp:155-160), which is the packed order of the
// vector; then normalize_vector (tensor_su2.cpp:324-356) -- once inside
// random_initialize_tensor and once more by the caller (dmrg_su2_omp.cpp:80).
// ran() is the 64-bit linear congruential generator of ran.f90:2-16,
//     s <- s * 2862933555777941757 + 1013904243 (mod 2^64),
//     ran = 0.5 + (0.5 / (2^63 - 1)) * (double)(signed) s,
// element k taking the state after k + 1 steps.  Each thread jumps ahead to
// its first element (composition of the affine step, by squaring) and then
// strides by the grid with the step composed grid-size times, so the values
// are those of the sequential generator, bit for bit.
namespace {

constexpr uint64_t kLcgMul = 2862933555777941757ull;
constexpr uint64_t kLcgAdd = 1013904243ull;

// (mul, add) of the LCG applied n times
__host__ __device__ inline void lcg_power(uint64_t n, uint64_t* mul, uint64_t* add) {
  uint64_t am = 1, aa = 0;              // accumulated map x -> am x + aa
  uint64_t bm = kLcgMul, ba = kLcgAdd;  // the step applied 2^i times
  while (n) {
    if (n & 1) {
      am = am * bm;
      aa = aa * bm + ba;
    }
    ba = ba * bm + ba;
    bm = bm * bm;
    n >>= 1;
  }
  *mul = am;
  *add = aa;
}

__device__ inline double lcg_value(uint64_t s) {
  const double dmu64 = 0.5 / 9223372036854775807.0;
  const double r = __dadd_rn(0.5, __dmul_rn(dmu64, (double)(long long)s));
  return __dadd_rn(__dmul_rn(r, 2.0), -1.0);
}

__global__ void lcg_fill_kernel(double* x, int64_t n, uint64_t s0, uint64_t stride_mul, uint64_t stride_add) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  uint64_t m, a;
  lcg_power((uint64_t)t + 1, &m, &a);
  uint64_t s = m * s0 + a;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = t; k < n; k += stride) {
    x[k] = lcg_value(s);
    s = stride_mul * s + stride_add;
  }
}

// x /= sqrt(*nn), as normalize_vector divides
__global__ void div_sqrt_kernel(double* x, int64_t n, const double* nn) {
  const double nor = sqrt(*nn);
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    x[k] = __ddiv_rn(x[k], nor);
}

}  // namespace

extern "C" int su2g_random_vector(int64_t* state, double* out, int64_t n, void* stream) {
  if (!state || n < 0 || (n > 0 && !out)) return fail(SU2G_EINVAL, "random_vector: bad arguments");
  if (n == 0) return SU2G_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 4);
  uint64_t sm, sa;
  lcg_power((uint64_t)grid * 256, &sm, &sa);
  lcg_fill_kernel<<<grid, 256, 0, st>>>(out, n, (uint64_t)*state, sm, sa);
  cudaError_t e = cudaGetLastError();
  const int ns = su2g::reduction_scratch_doubles();
  double* scratch = nullptr;
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&scratch, ns * sizeof(double), st);
  for (int pass = 0; pass < 2 && e == cudaSuccess; ++pass) {  // random_initialize_tensor, then the caller
    e = su2g::launch_dot(out, out, n, scratch, st);
    if (e == cudaSuccess) {
      div_sqrt_kernel<<<grid, 256, 0, st>>>(out, n, scratch + ns - 1);
      e = cudaGetLastError();
    }
  }
  if (scratch) cudaFreeAsync(scratch, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "random_vector");
  uint64_t m, a;
  lcg_power((uint64_t)n, &m, &a);
  *state = (int64_t)(m * (uint64_t)*state + a);
  return SU2G_OK;
}
