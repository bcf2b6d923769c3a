// The H_eff plan object behind the su2g_heff_plan handle of the C ABI, shared
// by capi.cu (single plans, Lanczos) and heff_batch.cu (several plans in
// shared launches).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "heff_plan.hpp"
#include "kernels.hpp"
#include "ozaki_plan.hpp"
#include "su2g.h"

struct su2g_heff_plan {
  su2g::HeffWork work;
  int mode = SU2G_MODE_F64;
  su2g::GemmSeg* d_seg1 = nullptr;
  su2g::GemmSeg* d_seg2 = nullptr;
  su2g::GemmTile* d_tile1 = nullptr;
  su2g::GemmTile* d_tile2 = nullptr;
  double* d_scratch = nullptr;
  // split-precision work (S > 0)
  int S = 0;
  su2g::oz::OzWork oz;
  uint8_t* d_packed = nullptr;
  int* d_exps = nullptr;
  su2g::oz::PackJob* d_jobs[3] = {nullptr, nullptr, nullptr};
  int2* d_units[3] = {nullptr, nullptr, nullptr};
  su2g::oz::OzSeg* d_oseg1 = nullptr;
  su2g::oz::OzSeg* d_oseg2 = nullptr;
  su2g::oz::OzTile* d_otile1 = nullptr;
  su2g::oz::OzTile* d_otile2 = nullptr;
  su2g::oz::RedTile* d_red2 = nullptr;
  int* d_err = nullptr;
  void* d_lists = nullptr;  // one device block holding every work list above and d_err
  // Lanczos workspace (allocated on first use)
  double* d_krylov = nullptr;
  int krylov_vectors = 0;
  double* d_red = nullptr;
  // excited-state projectors y -= w (o . psi) o
  std::vector<const double*> proj_vec;
  std::vector<double> proj_w;
  double* d_proj = nullptr;  // dot scratch, reduction_scratch_doubles() per projector
  // graph-captured Lanczos steps: lanc_step[m] produces Krylov vector m
  // (matvec, orthogonalisation, normalisation), lanc_last[m] the final
  // matvec and alpha; captured on cap_stream for this plan's Krylov buffers
  std::vector<cudaGraphExec_t> lanc_step, lanc_last;
  cudaStream_t cap_stream = nullptr;
  double* d_lcoef = nullptr;  // alpha[0..), beta[0..), reorthogonalisation and norm scratch
  int lcoef_m = 0;            // largest mlanc the coefficient layout serves
  // the stream of the plan's latest work: its buffers are freed in order on it
  cudaStream_t last_st = nullptr;

  void drop_graphs() {
    for (cudaGraphExec_t g : lanc_step)
      if (g) cudaGraphExecDestroy(g);
    for (cudaGraphExec_t g : lanc_last)
      if (g) cudaGraphExecDestroy(g);
    lanc_step.clear();
    lanc_last.clear();
  }

  void release() {
    // the work lists and the error word lie in one block (d_lists)
    su2g::dev_free(d_lists, last_st);
    d_lists = nullptr;
    su2g::dev_free(d_scratch, last_st);
    su2g::dev_free(d_krylov, last_st);
    su2g::dev_free(d_red, last_st);
    su2g::dev_free(d_packed, last_st);
    su2g::dev_free(d_exps, last_st);
    for (int c = 0; c < 3; ++c) {
      d_jobs[c] = nullptr;
      d_units[c] = nullptr;
    }
    su2g::dev_free(d_proj, last_st);
    d_proj = nullptr;
    drop_graphs();
    if (cap_stream) cudaStreamDestroy(cap_stream);
    cap_stream = nullptr;
    su2g::dev_free(d_lcoef, last_st);
    d_lcoef = nullptr;
    d_seg1 = d_seg2 = nullptr;
    d_tile1 = d_tile2 = nullptr;
    d_scratch = d_krylov = d_red = nullptr;
    d_packed = nullptr;
    d_exps = d_err = nullptr;
    d_oseg1 = d_oseg2 = nullptr;
    d_otile1 = d_otile2 = nullptr;
    d_red2 = nullptr;
  }
};

namespace su2g {
// su2g_heff_apply without recording the stream as the plan's latest (for
// launches captured into graphs, whose stream is not where they run)
int heff_apply_impl(su2g_heff_plan* p, const double* psi, double* y, cudaStream_t st);
// cuda error -> status code with the library's last-error text
int cuda_status(cudaError_t e, const char* where);
// y -= w_j (o_j . psi) o_j for the plan's excited-state projectors
cudaError_t apply_projectors(su2g_heff_plan* p, const double* psi, double* y, cudaStream_t st);
}  // namespace su2g
