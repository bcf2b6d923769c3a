// Launchers of the device kernels (kernels_f64.cu and friends).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "gemm_work.hpp"

namespace su2g {

// records the calling thread's su2g_last_error() text and returns code
int set_last_error(int code, const std::string& msg);

// Device memory from a per-device stream-ordered pool (devmem.cu): usable on
// any stream when dev_alloc returns; dev_free releases it once `after` has
// passed the point of the call (pass the stream of its last use).  Neither
// synchronises the device.
cudaError_t dev_alloc(void** p, size_t bytes);
void dev_free(void* p, cudaStream_t after);
// dev_alloc + a copy of `bytes` host bytes, complete on return
cudaError_t upload_bytes(const void* host, size_t bytes, void** dptr);
// the calling thread's private non-blocking stream on the current device
cudaError_t setup_stream(cudaStream_t* out);

cudaError_t launch_gemm_f64(const GemmTile* tiles, int ntiles, const GemmSeg* segs, const Bases& bases,
                            cudaStream_t stream);
// one dense product C (M x N, ld ldc) = op(A) B with the same tile code
// (op(A) = A, M x K, or for transA A^T with A stored K x M; B stored K x N),
// tiles of class cls, the work formed from the arguments
cudaError_t launch_gemm_f64_dense(bool transA, int M, int N, int K, const double* A, int lda, const double* B,
                                  int ldb, double* C, int ldc, int cls, cudaStream_t stream);

// deterministic dot product: partial sums in scratch[0..reduction_scratch_doubles()-1),
// the result in scratch[reduction_scratch_doubles()-1]
int reduction_scratch_doubles();
cudaError_t launch_dot(const double* x, const double* y, int64_t n, double* scratch, cudaStream_t stream);
cudaError_t launch_axpy(double alpha, const double* x, double* y, int64_t n, cudaStream_t stream);
// the same reductions and updates with their scalars on the device (graph-captured Lanczos):
// *out = x . y;  y -= (*c) x;  b = sqrt(*nn), *b_out = b, x *= 1 / b
cudaError_t launch_dot_to(const double* x, const double* y, int64_t n, double* scratch, double* out,
                          cudaStream_t stream);
cudaError_t launch_axpy_neg_dev(const double* c, const double* x, double* y, int64_t n, cudaStream_t stream);
cudaError_t launch_normalize_dev(const double* nn, double* x, int64_t n, double* b_out, cudaStream_t stream);
cudaError_t launch_scale(double alpha, double* x, int64_t n, cudaStream_t stream);
// y += alpha * (*scale) * x with the scale read on the device (combine.cu)
cudaError_t launch_axpy_dev(double alpha, const double* scale, const double* x, double* y, int64_t n,
                            cudaStream_t stream);

namespace oz {
struct PackJob;
struct OzSeg;
struct OzTile;
struct RedTile;
cudaError_t launch_reduce(const RedTile* reds, int n, const Bases& bases, cudaStream_t stream);
// one-time per-process setup of the GEMM kernel (function attributes, SM count),
// done before any launch is captured into a graph
cudaError_t prepare_ozaki_gemm(int S);
// runs the GEMM's bounded mbarrier wait on a barrier nothing arrives at, with
// `limit` polls; *timed_out_host = 1 when it gave up (the expected outcome)
cudaError_t bounded_wait_selftest(long long limit, int* timed_out_host, cudaStream_t stream);
// CTAs of the persistent GEMM grid on the current device (its SM count); 152
// when no device answers (host-only planning and validation).
int ozaki_persistent_grid();
// row-exponent pass (when rows_pass) + digit pass: 1 or 2 kernels, none for nunits == 0
cudaError_t launch_pack(int S, const PackJob* jobs, const int2* units, int nunits, int max_nkt, bool rows_pass,
                        const Bases& bases, uint8_t* packed, int* exps, cudaStream_t stream);
cudaError_t launch_ozaki_gemm(int S, const OzTile* tiles, int ntiles, const OzSeg* segs, const uint8_t* packed,
                              int* exps, const Bases& bases, int* err, cudaStream_t stream);
int gemm_smem_bytes(int S);
}  // namespace oz

}  // namespace su2g
