// Linear combinations of block tensors of one structure, and the device-scalar
// axpy behind the excited-state projector of H_eff.
//
// out = sum_i coef_i op_i is how the reference forms the summed partner of
// each H_eff term (tmp = opr[ir][k]; tmp *= coup; op += tmp,
// dmrg_su2.cpp:588-600) and the site-step sums (hh[i] += hh2[j],
// dmrg_su2_omp.cpp:462-469).  The output holds the union of the operands'
// blocks (tensor_su2::operator+= creates missing blocks, tensor_su2.cpp:152-200);
// every element is summed in operand order, so the result does not depend on
// the launch shape.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "kernels.hpp"
#include "su2_meta.hpp"
#include "su2g.h"

namespace {

int fail(int code, const std::string& msg) { return su2g::set_last_error(code, msg); }

struct CombItem {  // one output block
  int64_t dst;     // element offset in out
  int64_t len;
  int src0, nsrc;  // range in the source list
};
struct CombSrc {
  const double* p;  // the operand's copy of this block
  double c;
};

constexpr int kCombThreads = 256;

// grid: (element chunks, one row per output block); each thread strides over its block
__global__ void __launch_bounds__(kCombThreads) combine_kernel(const CombItem* __restrict__ items,
                                                               const CombSrc* __restrict__ srcs, double* out) {
  const CombItem it = items[blockIdx.y];
  for (int64_t e = (int64_t)blockIdx.x * kCombThreads + threadIdx.x; e < it.len;
       e += (int64_t)gridDim.x * kCombThreads) {
    double acc = 0.0;
    for (int s = 0; s < it.nsrc; ++s) {
      const CombSrc q = srcs[it.src0 + s];
      acc += q.c * q.p[e];
    }
    out[it.dst + e] = acc;
  }
}

__global__ void axpy_dev_kernel(double alpha, const double* __restrict__ scale, const double* __restrict__ x,
                                double* __restrict__ y, int64_t n) {
  const double a = alpha * *scale;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}

bool same_legs(const su2g::Struct& a, const su2g::Struct& b) {
  if (a.nbond != b.nbond || a.locspin != b.locspin) return false;
  for (int l = 0; l < a.nbond; ++l)
    if (a.legs[l].dir != b.legs[l].dir || a.legs[l].angm != b.legs[l].angm || a.legs[l].dim != b.legs[l].dim)
      return false;
  return true;
}

// parses the operands; out gets their common structure with the union of blocks
int combine_struct(int n, const su2g_tensor* ops, std::vector<su2g::Struct>* in, su2g::Struct* out) {
  if (n <= 0 || !ops) return fail(SU2G_EINVAL, "operator_combine: no operands");
  in->assign(n, su2g::Struct());
  std::string e;
  for (int i = 0; i < n; ++i) {
    su2g::Struct& s = (*in)[i];
    if (!ops[i].desc || !s.parse(ops[i].desc, &e)) return fail(SU2G_EINVAL, "operator_combine: operand: " + e);
    s.set_layout(ops[i].flag);
    if (i > 0 && !same_legs(s, (*in)[0]))
      return fail(SU2G_EINVAL, "operator_combine: operands of different structures");
  }
  *out = (*in)[0];
  std::vector<int> u(out->nten, 0);
  for (const su2g::Struct& s : *in)
    for (int b = 0; b < s.nten; ++b) u[b] |= s.flag[b];
  out->set_layout(u.data());
  return SU2G_OK;
}

}  // namespace

namespace su2g {
cudaError_t launch_axpy_dev(double alpha, const double* scale, const double* x, double* y, int64_t n,
                            cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4 * 152);
  axpy_dev_kernel<<<blocks, 256, 0, stream>>>(alpha, scale, x, y, n);
  return cudaGetLastError();
}
}  // namespace su2g

extern "C" int su2g_operator_combine_layout(int n, const su2g_tensor* ops, int* out_flag, int out_flag_cap,
                                            int64_t* out_len) {
  std::vector<su2g::Struct> in;
  su2g::Struct out;
  int rc = combine_struct(n, ops, &in, &out);
  if (rc) return rc;
  if (!out_flag || out_flag_cap < out.nten) return fail(SU2G_EINVAL, "operator_combine_layout: flag array too small");
  std::copy(out.flag.begin(), out.flag.end(), out_flag);
  if (out_len) *out_len = out.total;
  return SU2G_OK;
}

extern "C" int su2g_operator_combine(int n, const su2g_tensor* ops, const double* coef, double* out, void* stream) {
  std::vector<su2g::Struct> in;
  su2g::Struct o;
  int rc = combine_struct(n, ops, &in, &o);
  if (rc) return rc;
  if (!coef || (o.total > 0 && !out)) return fail(SU2G_EINVAL, "operator_combine: null argument");
  std::vector<CombItem> items;
  std::vector<CombSrc> srcs;
  int64_t maxlen = 0;
  for (int b = 0; b < o.nten; ++b) {
    if (!o.flag[b]) continue;
    CombItem it;
    it.dst = o.offset[b];
    int64_t len = 1;
    for (int l = 0; l < o.nbond; ++l) len *= o.block_dim(b, l);
    it.len = len;
    it.src0 = (int)srcs.size();
    for (int i = 0; i < n; ++i)
      if (in[i].flag[b]) {
        if (!ops[i].data) return fail(SU2G_EINVAL, "operator_combine: missing operand data");
        srcs.push_back(CombSrc{ops[i].data + in[i].offset[b], coef[i]});
      }
    it.nsrc = (int)srcs.size() - it.src0;
    items.push_back(it);
    maxlen = std::max(maxlen, len);
  }
  if (items.empty()) return SU2G_OK;
  if (items.size() > 65535) return fail(SU2G_EUNSUPPORTED, "operator_combine: more than 65535 blocks");
  cudaStream_t st = (cudaStream_t)stream;
  CombItem* d_items = nullptr;
  CombSrc* d_srcs = nullptr;
  const size_t bi = items.size() * sizeof(CombItem), bs = std::max<size_t>(1, srcs.size()) * sizeof(CombSrc);
  cudaError_t e = cudaMallocAsync((void**)&d_items, bi, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_srcs, bs, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_items, items.data(), bi, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !srcs.empty())
    e = cudaMemcpyAsync(d_srcs, srcs.data(), srcs.size() * sizeof(CombSrc), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    const int gx = (int)std::min<int64_t>((maxlen + kCombThreads - 1) / kCombThreads, 64);
    combine_kernel<<<dim3(gx, (unsigned)items.size()), kCombThreads, 0, st>>>(d_items, d_srcs, out);
    e = cudaGetLastError();
  }
  // the host arrays must outlive the copies above
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(d_items, st);
  cudaFreeAsync(d_srcs, st);
  if (e != cudaSuccess) return fail(SU2G_ECUDA, std::string("operator_combine: ") + cudaGetErrorString(e));
  return SU2G_OK;
}
