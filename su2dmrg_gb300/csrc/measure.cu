// The centre-bond energy of a converged state (dmrg_su2::mea_enr,
// dmrg_su2_omp_mea_enr.cpp:194-242) and the block-tensor reductions it is
// made of:
//   tensor_su2::take_trace (tensor_su2.cpp:720-742): sum over the blocks of
//     equal spins of their traces (no (2j+1) weight);
//   tensor_su2::ss_inner_prod (:687-715): sum over the blocks of their
//     element overlaps, weighted by sqrt(2j_2+1)/sqrt(2j_0+1) for 3 legs;
//   tensor_su2::multiply_singular_value (:359-384): every multiplet of leg
//     `leg` scaled by its weight, the weights laid out sector by sector in
//     the leg's order.
//   mea_enr = [tr H_L + tr(W H_R W) + sum_k coef_k ss(L_k, R_k)] / sum ww^2.
// Each block's sum is one CTA with a fixed reduction tree; the block sums
// are added on the host in the reference's order, so results do not depend
// on the launch.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "kernels.hpp"
#include "su2_meta.hpp"
#include "su2g.h"

namespace {

int fail(int code, const std::string& msg) { return su2g::set_last_error(code, msg); }
int cuda_fail(cudaError_t e, const char* where) {
  return fail(e == cudaErrorMemoryAllocation ? SU2G_ENOMEM : SU2G_ECUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

// One block sum: overlap (diag == 0): sum_e a[e] b[e]; diagonal (diag = n):
// sum_i a[i (n+1)] wl[i] wr[i] (a weight pointer may be null: 1).
struct SumItem {
  const double* a;
  const double* b;
  const double* wl;
  const double* wr;
  int64_t len;
  int diag;
  int pad;
};

constexpr int kSumThreads = 256;

__global__ void __launch_bounds__(kSumThreads) block_sums_kernel(const SumItem* __restrict__ items,
                                                                 double* __restrict__ out) {
  const SumItem it = items[blockIdx.x];
  double s = 0.0;
  if (it.diag > 0) {
    for (int i = threadIdx.x; i < it.diag; i += kSumThreads) {
      double v = it.a[(int64_t)i * (it.diag + 1)];
      if (it.wl) v *= it.wl[i];
      if (it.wr) v *= it.wr[i];
      s += v;
    }
  } else {
    for (int64_t e = threadIdx.x; e < it.len; e += kSumThreads) s += it.a[e] * it.b[e];
  }
  __shared__ double red[kSumThreads];
  red[threadIdx.x] = s;
  __syncthreads();
#pragma unroll
  for (int h = kSumThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// One block to scale: x[e] *= w[index of e along leg]
struct ScaleItem {
  double* x;
  const double* w;
  int64_t len;
  int d0, d1;  // dims of legs 0, 1
  int leg;
  int pad;
};

__global__ void scale_leg_kernel(const ScaleItem* __restrict__ items) {
  const ScaleItem it = items[blockIdx.y];
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < it.len; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t k;
    if (it.leg == 0) k = e % it.d0;
    else if (it.leg == 1) k = (e / it.d0) % it.d1;
    else k = e / ((int64_t)it.d0 * it.d1);
    it.x[e] *= it.w[k];
  }
}

// uploads `items`, runs the block sums, returns them in item order
cudaError_t run_sums(const std::vector<SumItem>& items, std::vector<double>* sums, cudaStream_t st) {
  sums->assign(items.size(), 0.0);
  if (items.empty()) return cudaSuccess;
  SumItem* d_items = nullptr;
  double* d_out = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&d_items, items.size() * sizeof(SumItem), st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_out, items.size() * sizeof(double), st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(SumItem), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    block_sums_kernel<<<(unsigned)items.size(), kSumThreads, 0, st>>>(d_items, d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sums->data(), d_out, items.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (d_items) cudaFreeAsync(d_items, st);
  if (d_out) cudaFreeAsync(d_out, st);
  return e;
}

int parse(const su2g_tensor& t, su2g::Struct* s, const char* what) {
  std::string e;
  if (!t.desc || !s->parse(t.desc, &e)) return fail(SU2G_EINVAL, std::string(what) + ": " + e);
  s->set_layout(t.flag);
  if (s->total > 0 && !t.data) return fail(SU2G_EINVAL, std::string(what) + ": null data");
  return SU2G_OK;
}

bool same_legs(const su2g::Struct& a, const su2g::Struct& b) {
  if (a.nbond != b.nbond || a.locspin != b.locspin) return false;
  for (int l = 0; l < a.nbond; ++l)
    if (a.legs[l].dir != b.legs[l].dir || a.legs[l].angm != b.legs[l].angm || a.legs[l].dim != b.legs[l].dim)
      return false;
  return true;
}

int64_t block_size(const su2g::Struct& s, int b) {
  int64_t n = 1;
  for (int l = 0; l < s.nbond; ++l) n *= s.block_dim(b, l);
  return n;
}

// offset of each sector's first multiplet along a leg
std::vector<int64_t> leg_offsets(const su2g::Bond& b) {
  std::vector<int64_t> o(b.n() + 1, 0);
  for (int i = 0; i < b.n(); ++i) o[i + 1] = o[i] + b.dim[i];
  return o;
}

// trace items of a 2-leg tensor (weights wl on leg 0, wr on leg 1, may be null)
int trace_items(const su2g::Struct& s, const double* x, const double* wl, const double* wr,
                std::vector<SumItem>* items, const char* what) {
  if (s.nbond != 2) return fail(SU2G_EINVAL, std::string(what) + ": a 2-leg tensor expected");
  const std::vector<int64_t> o0 = leg_offsets(s.legs[0]), o1 = leg_offsets(s.legs[1]);
  for (int b = 0; b < s.nten; ++b) {
    if (!s.flag[b] || s.block_angm(b, 0) != s.block_angm(b, 1)) continue;
    const int n = s.block_dim(b, 0);
    if (s.block_dim(b, 1) != n) return fail(SU2G_EINVAL, std::string(what) + ": a diagonal block is not square");
    SumItem it{};
    it.a = x + s.offset[b];
    it.wl = wl ? wl + o0[s.block_sector(b, 0)] : nullptr;
    it.wr = wr ? wr + o1[s.block_sector(b, 1)] : nullptr;
    it.diag = n;
    items->push_back(it);
  }
  return SU2G_OK;
}

// overlap items of ss_inner_prod(a, b): blocks stored in a (each must be stored in b)
int overlap_items(const su2g::Struct& sa, const double* xa, const su2g::Struct& sb, const double* xb,
                  std::vector<SumItem>* items, std::vector<double>* weights, const char* what) {
  if (!same_legs(sa, sb)) return fail(SU2G_EINVAL, std::string(what) + ": operands of different structures");
  for (int b = 0; b < sa.nten; ++b) {
    if (!sa.flag[b]) continue;
    if (!sb.flag[b]) return fail(SU2G_EINVAL, std::string(what) + ": a block of the first operand is absent in the second");
    SumItem it{};
    it.a = xa + sa.offset[b];
    it.b = xb + sb.offset[b];
    it.len = block_size(sa, b);
    items->push_back(it);
    weights->push_back(sa.nbond == 3 ? std::sqrt((double)(sa.block_angm(b, 2) + 1)) /
                                           std::sqrt((double)(sa.block_angm(b, 0) + 1))
                                     : 1.0);
  }
  return SU2G_OK;
}

}  // namespace

extern "C" int su2g_take_trace(su2g_tensor t, double* out, void* stream) {
  su2g::Struct s;
  int rc = parse(t, &s, "take_trace");
  if (rc) return rc;
  if (!out) return fail(SU2G_EINVAL, "take_trace: null output");
  std::vector<SumItem> items;
  rc = trace_items(s, t.data, nullptr, nullptr, &items, "take_trace");
  if (rc) return rc;
  std::vector<double> sums;
  cudaError_t e = run_sums(items, &sums, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "take_trace");
  double r = 0;
  for (double v : sums) r += v;
  *out = r;
  return SU2G_OK;
}

extern "C" int su2g_ss_inner_prod(su2g_tensor a, su2g_tensor b, double* out, void* stream) {
  if (!out) return fail(SU2G_EINVAL, "ss_inner_prod: null output");
  if (!a.desc && !b.desc) {  // two operators never built
    *out = 0.0;
    return SU2G_OK;
  }
  su2g::Struct sa, sb;
  int rc = parse(a, &sa, "ss_inner_prod");
  if (!rc) rc = parse(b, &sb, "ss_inner_prod");
  if (rc) return rc;
  std::vector<SumItem> items;
  std::vector<double> w;
  rc = overlap_items(sa, a.data, sb, b.data, &items, &w, "ss_inner_prod");
  if (rc) return rc;
  std::vector<double> sums;
  cudaError_t e = run_sums(items, &sums, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "ss_inner_prod");
  double r = 0;
  for (size_t i = 0; i < sums.size(); ++i) r += sums[i] * w[i];
  *out = r;
  return SU2G_OK;
}

extern "C" int su2g_multiply_singular_value(const int* desc, const int* flag, double* data, int leg, const double* w,
                                            int64_t nw, void* stream) {
  su2g::Struct s;
  std::string err;
  if (!desc || !s.parse(desc, &err)) return fail(SU2G_EINVAL, "multiply_singular_value: " + err);
  s.set_layout(flag);
  if (leg < 0 || leg >= s.nbond || s.nbond > 3) return fail(SU2G_EINVAL, "multiply_singular_value: bad leg");
  const std::vector<int64_t> off = leg_offsets(s.legs[leg]);
  if (!w || nw < off.back()) return fail(SU2G_EINVAL, "multiply_singular_value: fewer weights than multiplets of the leg");
  if (s.total == 0) return SU2G_OK;
  if (!data) return fail(SU2G_EINVAL, "multiply_singular_value: null data");
  cudaStream_t st = (cudaStream_t)stream;
  double* d_w = nullptr;
  ScaleItem* d_items = nullptr;
  std::vector<ScaleItem> items;
  int64_t maxlen = 0;
  cudaError_t e = cudaMallocAsync((void**)&d_w, off.back() * sizeof(double), st);
  for (int b = 0; b < s.nten && e == cudaSuccess; ++b) {
    if (!s.flag[b]) continue;
    ScaleItem it{};
    it.x = data + s.offset[b];
    it.w = d_w + off[s.block_sector(b, leg)];
    it.len = block_size(s, b);
    it.d0 = s.block_dim(b, 0);
    it.d1 = s.nbond > 1 ? s.block_dim(b, 1) : 1;
    it.leg = leg;
    items.push_back(it);
    maxlen = std::max(maxlen, it.len);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_w, w, off.back() * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !items.empty()) {
    if (items.size() > 65535) e = cudaErrorInvalidValue;
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_items, items.size() * sizeof(ScaleItem), st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(ScaleItem), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
      const int gx = (int)std::min<int64_t>((maxlen + 255) / 256, 64);
      scale_leg_kernel<<<dim3(gx, (unsigned)items.size()), 256, 0, st>>>(d_items);
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host arrays must outlive the copies
  if (d_items) cudaFreeAsync(d_items, st);
  if (d_w) cudaFreeAsync(d_w, st);
  if (e != cudaSuccess) return cuda_fail(e, "multiply_singular_value");
  return SU2G_OK;
}

extern "C" int su2g_mea_enr(su2g_tensor hl, su2g_tensor hr, const double* ww, int64_t nww, int npairs,
                            const su2g_tensor* left, const su2g_tensor* right, const double* coef, double* energy,
                            double* parts, void* stream) {
  if (!energy || nww <= 0 || !ww || npairs < 0 || (npairs > 0 && (!left || !right || !coef)))
    return fail(SU2G_EINVAL, "mea_enr: bad arguments");
  su2g::Struct sl, sr;
  int rc = parse(hl, &sl, "mea_enr: hl");
  if (!rc) rc = parse(hr, &sr, "mea_enr: hr");
  if (rc) return rc;
  const std::vector<int64_t> o0 = leg_offsets(sr.legs[0]), o1 = leg_offsets(sr.legs[1]);
  if (sr.nbond != 2 || nww < o0.back() || nww < o1.back())
    return fail(SU2G_EINVAL, "mea_enr: fewer weights than multiplets of hr");
  cudaStream_t st = (cudaStream_t)stream;
  double* d_w = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&d_w, nww * sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_w, ww, nww * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    if (d_w) cudaFreeAsync(d_w, st);
    return cuda_fail(e, "mea_enr");
  }
  // items: the traces of hl and of W hr W, then each pair's block overlaps
  std::vector<SumItem> items;
  std::vector<double> weights;
  std::vector<int> group;  // 0: tr hl, 1: tr W hr W, 2 + k: pair k
  rc = trace_items(sl, hl.data, nullptr, nullptr, &items, "mea_enr: hl");
  group.resize(items.size(), 0);
  if (!rc) rc = trace_items(sr, hr.data, d_w, d_w, &items, "mea_enr: hr");
  group.resize(items.size(), 1);
  weights.assign(items.size(), 1.0);
  std::vector<su2g::Struct> pl(npairs), pr(npairs);
  for (int k = 0; k < npairs && !rc; ++k) {
    if (!left[k].desc && !right[k].desc) continue;  // operators never built: 0
    rc = parse(left[k], &pl[k], "mea_enr: left operator");
    if (!rc) rc = parse(right[k], &pr[k], "mea_enr: right operator");
    if (!rc) rc = overlap_items(pl[k], left[k].data, pr[k], right[k].data, &items, &weights, "mea_enr");
    group.resize(items.size(), 2 + k);
  }
  std::vector<double> sums;
  if (!rc) e = run_sums(items, &sums, st);
  cudaFreeAsync(d_w, st);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "mea_enr");
  // the reference's order: tr H_L, then tr W H_R W, then the pairs in order
  std::vector<double> g(2 + npairs, 0.0);
  for (size_t i = 0; i < sums.size(); ++i) g[group[i]] += sums[i] * weights[i];
  double pair_sum = 0.0, num = g[0];
  num += g[1];
  for (int k = 0; k < npairs; ++k) {
    num += coef[k] * g[2 + k];
    pair_sum += coef[k] * g[2 + k];
  }
  double den = 0.0;
  for (int64_t i = 0; i < nww; ++i) den += ww[i] * ww[i];
  *energy = num / den;
  if (parts) {
    parts[0] = g[0];
    parts[1] = g[1];
    parts[2] = pair_sum;
    parts[3] = den;
  }
  return SU2G_OK;
}
