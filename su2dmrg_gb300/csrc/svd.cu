// Truncation of a two-site vector (tensor_su2::svd, tensor_su2.cpp:1619-1758,
// with the per-sector tensor::svd of tensor.cpp:1472-1700), on the GPU:
//   * per sector, the Gram matrix of the smaller side and its FP64
//     eigendecomposition (cuSOLVER syevd in its deterministic mode,
//     eigenvalues ascending like dsyev), then the reference's refinement:
//     while more than one eigenvalue
//     lies below 0.1 of the largest of the current subspace, re-diagonalise
//     the original Gram matrix projected on that subspace;
//   * the other factor by one more product, singular values = sqrt of the
//     eigenvalues above 1e-100 of the largest, columns scaled by s^(p1-1) and
//     s^p2 (or the mirror for wide blocks);
//   * every product (Gram matrices, the refinement's projections and
//     rotations, the other factor) runs on the library's FP64 tile engine,
//     whose sums have a fixed order: the result of a truncation does not
//     depend on what else shares the GPU (a library GEMM picks its internal
//     implementation by the concurrent load, and near a cut in the rounding
//     noise that changes which multiplets are kept);
//   * the sectors are independent: each runs on its own stream, cuSOLVER
//     handle and host thread (the refinement reads eigenvalues back between
//     steps), so their eigendecompositions overlap on the GPU;
//   * on the host: all kept singular values sorted by the Shell sort of
//     sort2.f (dsort2, whose handling of equal values decides ties), the
//     largest max_dcut multiplets kept (no (2j+1) weighting), and the
//     singular values reported kept-then-discarded as the reference writes
//     them.
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "heff_plan.hpp"
#include "kernels.hpp"
#include "su2_meta.hpp"
#include "su2g.h"

namespace {

int fail(int code, const std::string& msg) { return su2g::set_last_error(code, msg); }

__global__ void scale_columns(double* a, int rows, int c0, int ncol, int ld, const double* f) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (int64_t)rows * ncol;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(idx % rows), c = (int)(idx / rows);
    a[(int64_t)(c0 + c) * ld + r] *= f[c];
  }
}

// out (cols x rows) = in^T, 32 x 32 tiles through shared memory
__global__ void transpose_kernel(const double* __restrict__ in, int rows, int cols, double* __restrict__ out) {
  __shared__ double t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int r = r0 + threadIdx.x, c = c0 + j;
    if (r < rows && c < cols) t[j][threadIdx.x] = in[(int64_t)c * rows + r];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int c = c0 + threadIdx.x, r = r0 + j;
    if (r < rows && c < cols) out[(int64_t)r * cols + c] = t[threadIdx.x][j];
  }
}

// The eigenvector sign rule of su2g::canonical_column_signs (tridiag.hpp)
// on the device: one CTA per column of the rows x cols matrix z (ld rows).
// The largest magnitude and the first index above 1e-4 of it are exact
// reductions (max, min), so the choice does not depend on the order.
__global__ void __launch_bounds__(256) canonical_signs_kernel(double* z, int rows) {
  __shared__ double smax[8];
  __shared__ int sfirst[8];
  double* col = z + (int64_t)blockIdx.x * rows;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double mx = 0;
  for (int i = threadIdx.x; i < rows; i += blockDim.x) mx = fmax(mx, fabs(col[i]));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) smax[wid] = mx;
  __syncthreads();
  mx = smax[0];
  for (int w = 1; w < 8; ++w) mx = fmax(mx, smax[w]);
  int first = rows;
  for (int i = threadIdx.x; i < rows; i += blockDim.x)
    if (fabs(col[i]) > 1e-4 * mx) {
      first = i;
      break;
    }
  for (int o = 16; o > 0; o >>= 1) first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
  if (lane == 0) sfirst[wid] = first;
  __syncthreads();
  first = sfirst[0];
  for (int w = 1; w < 8; ++w) first = min(first, sfirst[w]);
  if (first < rows && col[first] < 0)
    for (int i = threadIdx.x; i < rows; i += blockDim.x) col[i] = -col[i];
}

// Per-device resources kept across calls: lanes (one stream and one cuSOLVER
// handle each; creating a handle costs milliseconds), lent
// to a call for each sector it processes and returned after it, so calls from
// several host threads (independent solves) run at the same time; and a
// library-private memory pool whose freed blocks stay reserved (stream-ordered
// allocation without device-wide synchronisation, unlike cudaMalloc).
struct Lane {
  cudaStream_t st = nullptr;
  cusolverDnHandle_t sol = nullptr;
  cudaEvent_t done = nullptr;
};
struct DeviceRes {
  cudaMemPool_t pool = nullptr;
  std::vector<Lane> free_lanes;
};
std::mutex g_res_mutex;
std::map<int, DeviceRes> g_res;

// Lends n lanes of device dev (creating what is missing) and the pool;
// returns an error message or "".
std::string take_lanes(int dev, int n, std::vector<Lane>* out, cudaMemPool_t* pool) {
  std::lock_guard<std::mutex> lock(g_res_mutex);
  DeviceRes& r = g_res[dev];
  if (!r.pool) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    if (cudaMemPoolCreate(&r.pool, &props) != cudaSuccess) {
      r.pool = nullptr;
      return "cannot create a memory pool";
    }
    uint64_t keep = UINT64_MAX;  // freed blocks stay in the pool
    cudaMemPoolSetAttribute(r.pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  *pool = r.pool;
  out->clear();
  while ((int)out->size() < n && !r.free_lanes.empty()) {
    out->push_back(r.free_lanes.back());
    r.free_lanes.pop_back();
  }
  while ((int)out->size() < n) {
    Lane l;
    if (cudaStreamCreateWithFlags(&l.st, cudaStreamNonBlocking) != cudaSuccess) return "cannot create a stream";
    if (cudaEventCreateWithFlags(&l.done, cudaEventDisableTiming) != cudaSuccess) {
      cudaStreamDestroy(l.st);
      return "cannot create an event";
    }
    if (cusolverDnCreate(&l.sol) != CUSOLVER_STATUS_SUCCESS) {
      cudaEventDestroy(l.done);
      cudaStreamDestroy(l.st);
      return "cannot create a cuSOLVER handle";
    }
    cusolverDnSetStream(l.sol, l.st);
    // the eigensolver's deterministic mode: a truncation's result must not
    // depend on what else runs on the GPU
    if (cusolverDnSetDeterministicMode(l.sol, CUSOLVER_DETERMINISTIC_RESULTS) != CUSOLVER_STATUS_SUCCESS) {
      cusolverDnDestroy(l.sol);
      cudaEventDestroy(l.done);
      cudaStreamDestroy(l.st);
      return "cannot set the eigensolver's deterministic mode";
    }
    out->push_back(l);
  }
  return "";
}

void give_lanes(int dev, const std::vector<Lane>& lanes) {
  std::lock_guard<std::mutex> lock(g_res_mutex);
  DeviceRes& r = g_res[dev];
  r.free_lanes.insert(r.free_lanes.end(), lanes.begin(), lanes.end());
}

// Host threads that run the sectors of a call (the refinement loop reads
// eigenvalues back between its steps, so each sector needs its own thread).
// Kept across calls and grown on demand, instead of one thread per sector per
// call; never joined (the process ends with them).
class SectorThreads {
 public:
  static SectorThreads& get() {
    static SectorThreads* t = new SectorThreads();
    return *t;
  }
  // runs body(0..n-1), body(0) on the calling thread, and returns when all are done
  void run(size_t n, const std::function<void(size_t)>& body) {
    if (n == 0) return;
    struct Latch {
      std::mutex mu;
      std::condition_variable cv;
      size_t left;
    } latch;
    latch.left = n - 1;
    {
      std::lock_guard<std::mutex> lock(mu_);
      for (size_t q = 1; q < n; ++q)
        queue_.push_back([&, q] {
          body(q);
          std::lock_guard<std::mutex> l(latch.mu);
          if (--latch.left == 0) latch.cv.notify_all();
        });
      while (idle_ < queue_.size()) {  // a thread per waiting task
        std::thread(&SectorThreads::loop, this).detach();
        ++idle_;
      }
    }
    cv_.notify_all();
    body(0);
    std::unique_lock<std::mutex> l(latch.mu);
    latch.cv.wait(l, [&] { return latch.left == 0; });
  }

 private:
  void loop() {
    for (;;) {
      std::function<void()> task;
      {
        std::unique_lock<std::mutex> lock(mu_);
        cv_.wait(lock, [&] { return !queue_.empty(); });
        task = std::move(queue_.front());
        queue_.pop_front();
        --idle_;
      }
      task();
      std::lock_guard<std::mutex> lock(mu_);
      ++idle_;
    }
  }
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<std::function<void()>> queue_;
  size_t idle_ = 0;
};

// The work of one sector: its lane, its allocations (from the pool, on the
// lane's stream; released on `free_st` once the caller's stream has used
// them) and its error state.
struct Ctx {
  cudaStream_t st = nullptr;
  cudaStream_t free_st = nullptr;
  cudaMemPool_t pool = nullptr;
  cusolverDnHandle_t sol = nullptr;
  std::vector<void*> allocs;
  std::string err;
  int code = SU2G_OK;

  Ctx() = default;
  Ctx(const Ctx&) = delete;
  Ctx& operator=(const Ctx&) = delete;
  ~Ctx() {
    for (void* p : allocs) cudaFreeAsync(p, free_st);
  }
  bool ok() const { return code == SU2G_OK; }
  void set(int c, const std::string& m) {
    if (code == SU2G_OK) {
      code = c;
      err = m;
    }
  }
  double* dalloc(int64_t n) {
    void* p = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync(&p, std::max<int64_t>(n, 1) * sizeof(double), pool, st);
    if (e != cudaSuccess) {
      set(e == cudaErrorMemoryAllocation ? SU2G_ENOMEM : SU2G_ECUDA, std::string("svd: ") + cudaGetErrorString(e));
      return nullptr;
    }
    allocs.push_back(p);
    return (double*)p;
  }
  // C (M x N, ld ldc) = op(A) B with op(A) = A (M x K, ld lda) or, for
  // transA, A^T with A stored K x M; B stored K x N (ld ldb).  The library's
  // FP64 tile engine (gemm_f64_tiles): every element sums its K products in a
  // fixed order, whatever else runs on the GPU.
  void gemm(bool transA, int M, int N, int K, const double* A, int lda, const double* B, int ldb, double* C,
            int ldc) {
    if (!ok() || M == 0 || N == 0) return;
    const cudaError_t e =
        su2g::launch_gemm_f64_dense(transA, M, N, K, A, lda, B, ldb, C, ldc, su2g::tile_class_for(M, N), st);
    if (e != cudaSuccess) set(SU2G_ECUDA, std::string("svd: ") + cudaGetErrorString(e));
  }
  // out (cols x rows) = in^T (in: rows x cols, column-major)
  void transpose(const double* in, int rows, int cols, double* out) {
    if (!ok() || rows == 0 || cols == 0) return;
    const dim3 grid((cols + 31) / 32, (rows + 31) / 32);
    transpose_kernel<<<grid, dim3(32, 8), 0, st>>>(in, rows, cols, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) set(SU2G_ECUDA, std::string("svd: ") + cudaGetErrorString(e));
  }
  void copy(double* dst, const double* src, int64_t n) {
    if (!ok()) return;
    cudaError_t e = cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) set(SU2G_ECUDA, std::string("svd: ") + cudaGetErrorString(e));
  }
  // symmetric eigendecomposition in place (a: n x n, ld n), eigenvector signs
  // by the canonical rule; w: host eigenvalues
  void eigh(double* a, int n, std::vector<double>* w) {
    if (!ok()) return;
    int lwork = 0;
    double* dw = dalloc(n);
    if (!ok()) return;
    if (cusolverDnDsyevd_bufferSize(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n, a, n, dw, &lwork) !=
        CUSOLVER_STATUS_SUCCESS) {
      set(SU2G_ECUDA, "svd: syevd buffer query failed");
      return;
    }
    double* work = dalloc(lwork);
    double* dinfo = dalloc(1);
    if (!ok()) return;
    if (cusolverDnDsyevd(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n, a, n, dw, work, lwork,
                         (int*)dinfo) != CUSOLVER_STATUS_SUCCESS) {
      set(SU2G_ECUDA, "svd: syevd failed");
      return;
    }
    w->assign(n, 0.0);
    int info = 0;
    cudaError_t e = cudaMemcpyAsync(w->data(), dw, n * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && n > 0) {
      canonical_signs_kernel<<<n, 256, 0, st>>>(a, n);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) set(SU2G_ECUDA, std::string("svd: ") + cudaGetErrorString(e));
    else if (info != 0) set(SU2G_ECUDA, "svd: syevd did not converge (info " + std::to_string(info) + ")");
  }
};

// index after the last eigenvalue below tol1 of the largest (tensor.cpp:1492-1497)
int small_count(const std::vector<double>& w, int n) {
  for (int i = n - 1; i >= 0; --i)
    if (w[i] / w[n - 1] < 1.e-1) return i + 1;
  return 0;
}

struct Sector {
  int i = -1;      // leg-0 sector index
  int m = 0, n = 0;
  int dc = 0;      // singular values kept by the sector's own rule
  double* u = nullptr;  // m x dc (ld m), smallest first
  double* v = nullptr;  // n x dc (ld n)
  std::vector<double> s;  // dc values, ascending
};

// First pass of tensor::svd for one m x n block (n0 = 1): the Gram matrix of
// the smaller side and its eigendecomposition (tensor.cpp:1484-1490).
struct SectorEig {
  bool tall = true;
  int k = 0;
  // trace: host wall time of the two passes, refinement subspace sizes
  double ms_eig = 0, ms_finish = 0;
  std::vector<int> levels;
  double* G = nullptr;   // eigenvectors (k x k)
  double* A0 = nullptr;  // the Gram matrix
  std::vector<double> w;  // eigenvalues, ascending
};

void sector_eig(Ctx& c, const double* blk, int m, int n, SectorEig* e) {
  e->tall = m >= n;
  const int k = e->k = e->tall ? n : m;
  e->G = c.dalloc((int64_t)k * k);
  e->A0 = c.dalloc((int64_t)k * k);
  if (!c.ok()) return;
  if (e->tall) {
    c.gemm(true, n, n, m, blk, m, blk, m, e->G, n);  // blk^T blk
  } else {  // blk blk^T = (blk^T)^T (blk^T)
    double* bt = c.dalloc((int64_t)m * n);
    c.transpose(blk, m, n, bt);
    c.gemm(true, m, m, n, bt, n, bt, n, e->G, m);
  }
  c.copy(e->A0, e->G, (int64_t)k * k);
  c.eigh(e->G, k, &e->w);  // G now holds the eigenvectors
}

// Second pass: the reference's refinement of the small-eigenvalue subspace
// (tensor.cpp:1491-1529), then the factors.  Each refinement re-solves the
// subspace of eigenvalues below 0.1 of its largest and rotates only those
// columns, so a subspace whose largest eigenvalue is below 0.1 of lam_cut (the
// max_dcut-th largest eigenvalue over all sectors, 0 when every multiplet is
// kept or when the cut is too close to the first pass's rounding error to be
// placed) holds no multiplet the truncation keeps: refining it further changes
// neither the kept columns, their values nor the selection, and is skipped
// (its values, all discarded, stay those of the last refinement).
void sector_finish(Ctx& c, const double* blk, int m, int n, double p1, double p2, int max_dcut, double lam_cut,
                   SectorEig& e, Sector* out) {
  const bool tall = e.tall;
  const int k = e.k;
  double* G = e.G;
  std::vector<double>& w = e.w;
  if (!c.ok()) return;
  int np = small_count(w, k);
  if (np > 1 && !(lam_cut > 0 && w[np - 1] < 0.1 * lam_cut)) {
    double* ap = c.dalloc((int64_t)k * k);
    double* vp = c.dalloc((int64_t)k * k);
    double* app = c.dalloc((int64_t)k * k);
    double* vpp = c.dalloc((int64_t)k * k);
    double* tmp = c.dalloc((int64_t)k * k);
    c.copy(ap, e.A0, (int64_t)k * k);
    c.copy(vp, G, (int64_t)k * k);
    int npp = np;
    np = k;
    std::vector<double> ws;
    do {
      e.levels.push_back(npp);
      c.gemm(true, npp, np, np, vp, np, ap, np, app, npp);
      c.gemm(false, npp, npp, np, app, npp, vp, np, vpp, npp);
      c.copy(ap, vpp, (int64_t)npp * npp);
      c.eigh(vpp, npp, &ws);
      if (!c.ok()) return;
      for (int q = 0; q < npp; ++q) w[q] = ws[q];
      c.gemm(false, k, npp, npp, G, k, vpp, npp, tmp, k);
      c.copy(G, tmp, (int64_t)k * npp);
      c.copy(vp, vpp, (int64_t)npp * npp);
      const int j = small_count(ws, npp);
      np = npp;
      npp = j;
      if (npp > 1 && lam_cut > 0 && ws[npp - 1] < 0.1 * lam_cut) break;
    } while (npp > 1 && c.ok());
  }
  if (!c.ok()) return;
  double *U, *V;
  if (tall) {  // V = eigenvectors (n x n), U = blk V (m x n)
    V = G;
    U = c.dalloc((int64_t)m * n);
    c.gemm(false, m, n, n, blk, m, V, n, U, m);
  } else {  // U = eigenvectors (m x m), V = blk^T U (n x m)
    U = G;
    V = c.dalloc((int64_t)n * m);
    c.gemm(true, n, m, m, blk, m, U, m, V, n);
  }
  if (!c.ok()) return;
  // singular values above 1e-100 of the largest, scaling (tensor.cpp:1532-1567)
  const double num = w[k - 1];
  int dcut = 0;
  if (num > 1.e-100)
    for (int i = k - 1; i >= 0; --i) {
      if (w[i] / num > 1.e-100) {
        w[i] = std::sqrt(w[i]);
        ++dcut;
      } else {
        w[i] = 0;
      }
    }
  if (dcut > max_dcut) dcut = max_dcut;
  if (dcut > (tall ? m : n)) dcut = tall ? m : n;
  std::vector<double> fu(dcut), fv(dcut);
  for (int q = 0; q < dcut; ++q) {
    const double s = w[k - dcut + q];
    if (s > 0) {
      fu[q] = tall ? std::pow(s, p1 - 1.) : std::pow(s, p1);
      fv[q] = tall ? std::pow(s, p2) : std::pow(s, p2 - 1.);
    } else {
      fu[q] = fv[q] = 0.0;
    }
  }
  if (dcut > 0) {
    double* dfu = c.dalloc(dcut);
    double* dfv = c.dalloc(dcut);
    if (!c.ok()) return;
    cudaMemcpyAsync(dfu, fu.data(), dcut * sizeof(double), cudaMemcpyHostToDevice, c.st);
    cudaMemcpyAsync(dfv, fv.data(), dcut * sizeof(double), cudaMemcpyHostToDevice, c.st);
    scale_columns<<<256, 256, 0, c.st>>>(U, m, k - dcut, dcut, m, dfu);
    scale_columns<<<256, 256, 0, c.st>>>(V, n, k - dcut, dcut, n, dfv);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) c.set(SU2G_ECUDA, std::string("svd: ") + cudaGetErrorString(e));
  }
  out->m = m;
  out->n = n;
  out->dc = dcut;
  out->u = U + (int64_t)m * (k - dcut);
  out->v = V + (int64_t)n * (k - dcut);
  out->s.assign(w.begin() + (k - dcut), w.begin() + k);
}

}  // namespace

bool same_sectors(const su2g::Bond& a, const su2g::Bond& b) { return a.angm == b.angm && a.dim == b.dim; }

extern "C" int su2g_svd(const int* psi_desc, const int* psi_flag, const double* psi, const int* tu_desc, double p1,
                        const int* tv_desc, double p2, int max_dcut, int* bond, int bond_cap, double* wout,
                        int wout_cap, int* dout, double* tu, int64_t tu_cap, double* tv, int64_t tv_cap,
                        void* stream) {
  su2g::Struct P, TU, TV;
  std::string e;
  if (!psi_desc || !P.parse(psi_desc, &e)) return fail(SU2G_EINVAL, "svd: psi: " + e);
  if (P.nbond != 2) return fail(SU2G_EINVAL, "svd: psi must have 2 legs");
  if (!tu_desc || !TU.parse(tu_desc, &e) || TU.nbond != 3) return fail(SU2G_EINVAL, "svd: tu: 3-leg desc expected " + e);
  if (!tv_desc || !TV.parse(tv_desc, &e) || TV.nbond != 3) return fail(SU2G_EINVAL, "svd: tv: 3-leg desc expected " + e);
  if (!bond || !wout || !dout || max_dcut < 0) return fail(SU2G_EINVAL, "svd: bad arguments");
  // psi legs are the fused (tu leg 0, tu leg 1) and (tv leg 0, tv leg 1) (tensor_su2.cpp:1628-1634)
  if (!same_sectors(su2g::fuse(TU.legs[0], TU.legs[1]), P.legs[0]) ||
      !same_sectors(su2g::fuse(TV.legs[0], TV.legs[1]), P.legs[1]))
    return fail(SU2G_EINVAL, "svd: psi legs are not the fused legs 0, 1 of tu / tv");
  P.set_layout(psi_flag);
  if (P.total > 0 && !psi) return fail(SU2G_EINVAL, "svd: null psi");
  cudaStream_t cst = (cudaStream_t)stream;
  // SU2G_SVD_TRACE=<file>: one JSON line per call appended there (per sector:
  // m, n, Gram size, host milliseconds of the two passes, the sizes of the
  // refinement subspaces), for time breakdowns of whole sweeps
  const char* trace = std::getenv("SU2G_SVD_TRACE");
  if (trace && !*trace) trace = nullptr;
  const auto t_call = std::chrono::steady_clock::now();
  const int n0 = P.legs[0].n(), n1 = P.legs[1].n();
  // sectors in the reference's loop order: leg-0 sector, then the leg-1 sector of equal spin
  struct Job {
    int i, b, m, n;
  };
  std::vector<Job> jobs;
  for (int i = 0; i < n0; ++i)
    for (int j = 0; j < n1; ++j) {
      if (P.legs[0].angm[i] != P.legs[1].angm[j]) continue;
      const int b = i + j * n0;
      if (P.flag[b]) jobs.push_back(Job{i, b, P.legs[0].dim[i], P.legs[1].dim[j]});
    }
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return fail(SU2G_ECUDA, std::string("svd: ") + cudaGetErrorString(ce));
  std::vector<Lane> lanes;
  cudaMemPool_t pool = nullptr;
  const std::string rerr = take_lanes(dev, (int)jobs.size(), &lanes, &pool);
  if (!rerr.empty()) {
    give_lanes(dev, lanes);
    return fail(SU2G_ECUDA, "svd: " + rerr);
  }
  // the lanes go back to the device's free list when the call returns
  struct LaneReturn {
    int dev;
    const std::vector<Lane>& lanes;
    ~LaneReturn() { give_lanes(dev, lanes); }
  } lane_return{dev, lanes};
  // every sector on its own lane (stream + handles) and host thread: the
  // eigendecompositions and the refinement loops of all sectors overlap
  cudaEvent_t ready = nullptr;
  ce = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventRecord(ready, cst);
  if (ce != cudaSuccess) {
    if (ready) cudaEventDestroy(ready);
    return fail(SU2G_ECUDA, std::string("svd: ") + cudaGetErrorString(ce));
  }
  std::vector<std::unique_ptr<Ctx>> ctx(jobs.size());
  std::vector<Sector> secs(jobs.size());
  for (size_t q = 0; q < jobs.size(); ++q) {
    ctx[q].reset(new Ctx());
    Ctx& c = *ctx[q];
    c.st = lanes[q].st;
    c.free_st = cst;
    c.pool = pool;
    c.sol = lanes[q].sol;
    const cudaError_t we = cudaStreamWaitEvent(c.st, ready, 0);  // psi is written on the caller's stream
    if (we != cudaSuccess) c.set(SU2G_ECUDA, std::string("svd: ") + cudaGetErrorString(we));
  }
  // two passes over the sectors, each sector on its own host thread: the
  // eigendecompositions, then (with the global cut known) the refinements
  // and the factors
  std::vector<SectorEig> eig(jobs.size());
  double lam_cut = 0.0, lam_cut_raw = 0.0, noise_floor = 0.0;
  auto on_threads = [&](const std::function<void(size_t)>& body) { SectorThreads::get().run(jobs.size(), body); };
  on_threads([&](size_t q) {
    Ctx& c = *ctx[q];
    if (cudaSetDevice(dev) != cudaSuccess) c.set(SU2G_ECUDA, "svd: cannot select the device");
    const auto t0 = std::chrono::steady_clock::now();
    if (c.ok()) sector_eig(c, psi + P.offset[jobs[q].b], jobs[q].m, jobs[q].n, &eig[q]);
    eig[q].ms_eig = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  });
  {  // the max_dcut-th largest eigenvalue over all sectors; 0 (refine every
     // subspace, as the reference) when nothing is cut or when the cut lies
     // within 1e3 of the first pass's error k eps lambda_max of some sector,
     // where values near it are not yet known well enough to place them
    std::vector<double> all;
    double floor = 0.0;
    for (const SectorEig& e : eig) {
      const double top = e.w.empty() ? 0.0 : e.w.back();
      floor = std::max(floor, (double)e.k * 2.3e-16 * top);
      for (double v : e.w)
        if (v > 0 && v / top > 1.e-100) all.push_back(v);
    }
    if (max_dcut > 0 && (int64_t)all.size() > max_dcut) {
      std::nth_element(all.begin(), all.begin() + (max_dcut - 1), all.end(), std::greater<double>());
      lam_cut = lam_cut_raw = all[max_dcut - 1];
      if (lam_cut < 1e3 * floor) lam_cut = 0.0;
    }
    noise_floor = floor;
  }
  on_threads([&](size_t q) {
    Ctx& c = *ctx[q];
    if (cudaSetDevice(dev) != cudaSuccess) c.set(SU2G_ECUDA, "svd: cannot select the device");
    const auto t0 = std::chrono::steady_clock::now();
    if (c.ok()) {
      secs[q].i = jobs[q].i;
      sector_finish(c, psi + P.offset[jobs[q].b], jobs[q].m, jobs[q].n, p1, p2, max_dcut, lam_cut, eig[q],
                    &secs[q]);
    }
    if (trace) cudaStreamSynchronize(c.st);
    eig[q].ms_finish = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    const cudaError_t e = cudaEventRecord(lanes[q].done, c.st);
    if (e != cudaSuccess) c.set(SU2G_ECUDA, std::string("svd: ") + cudaGetErrorString(e));
  });
  // the caller's stream continues after every sector (placement copies, frees)
  for (size_t q = 0; q < jobs.size(); ++q) cudaStreamWaitEvent(cst, lanes[q].done, 0);
  cudaEventDestroy(ready);
  for (const auto& c : ctx)
    if (!c->ok()) return fail(c->code, c->err);
  // global selection of the max_dcut largest multiplets (tensor_su2.cpp:1686-1695)
  std::vector<double> ws;
  std::vector<int> is;
  for (const Sector& s : secs)
    for (int q = 0; q < s.dc; ++q) {
      ws.push_back(s.s[q]);
      is.push_back(s.i);
    }
  const int n = (int)ws.size();
  su2g::dsort2(n, ws.data(), is.data());
  std::vector<int> dim(n0, 0);
  for (int q = n - 1; q >= std::max(0, n - max_dcut); --q) ++dim[is[q]];
  // the new bond: kept sectors of psi leg 0, direction -1 (tensor_su2.cpp:1733)
  su2g::Bond nb;
  nb.dir = -1;
  for (int i = 0; i < n0; ++i)
    if (dim[i] > 0) {
      nb.angm.push_back(P.legs[0].angm[i]);
      nb.dim.push_back(dim[i]);
    }
  if (bond_cap < 1 + 2 * nb.n()) return fail(SU2G_EINVAL, "svd: bond output too small");
  bond[0] = nb.n();
  for (int q = 0; q < nb.n(); ++q) {
    bond[1 + q] = nb.angm[q];
    bond[1 + nb.n() + q] = nb.dim[q];
  }
  // kept values (per sector, ascending), then the discarded ones (tensor_su2.cpp:1706-1731)
  if (n > wout_cap) return fail(SU2G_EINVAL, "svd: wout too small (" + std::to_string(n) + " values)");
  int total_kept = 0;
  for (int d : dim) total_kept += d;
  int mk = 0, md = total_kept;
  for (const Sector& s : secs) {
    const int d = dim[s.i];
    for (int q = 0; q < d; ++q) wout[mk + q] = s.s[s.dc - d + q];
    for (int q = 0; q < s.dc - d; ++q) wout[md + q] = s.s[q];
    mk += d;
    md += s.dc - d;
  }
  *dout = md;
  // tu = fuse(tu legs 0, 1) x kept U, tv likewise with V: row ranges of the
  // kept columns, every legal block present (tensor_su2.cpp:1733-1745)
  for (int side = 0; side < 2; ++side) {
    double* out = side ? tv : tu;
    if (!out) continue;
    const su2g::Struct& T = side ? TV : TU;
    su2g::Struct O;
    O.nbond = 3;
    O.locspin = 0;
    O.legs[0] = T.legs[0];
    O.legs[1] = T.legs[1];
    O.legs[2] = nb;
    O.nten = O.legs[0].n() * O.legs[1].n() * nb.n();
    O.set_layout(nullptr);
    if (O.total > (side ? tv_cap : tu_cap))
      return fail(SU2G_EINVAL, std::string("svd: ") + (side ? "tv" : "tu") + " output too small (" +
                                   std::to_string(O.total) + " doubles)");
    for (int b = 0; b < O.nten; ++b) {
      if (!O.flag[b]) continue;
      int sec[3];
      O.sectors(b, sec);
      const int ang = nb.angm[sec[2]], d = nb.dim[sec[2]];
      const Sector* src = nullptr;
      for (const Sector& s : secs)
        if (P.legs[0].angm[s.i] == ang) src = &s;
      const int r0 = su2g::fused_row(O.legs[0], O.legs[1], ang, sec[0], sec[1]);
      const int rows = O.legs[0].dim[sec[0]] * O.legs[1].dim[sec[1]];
      if (!src || r0 < 0) return fail(SU2G_EINVAL, "svd: internal placement error");
      const int ld = side ? src->n : src->m;
      const double* col0 = (side ? src->v : src->u) + (int64_t)ld * (src->dc - d) + r0;
      const cudaError_t me = cudaMemcpy2DAsync(out + O.offset[b], rows * sizeof(double), col0,
                                               ld * sizeof(double), rows * sizeof(double), d,
                                               cudaMemcpyDeviceToDevice, cst);
      if (me != cudaSuccess) return fail(SU2G_ECUDA, std::string("svd: ") + cudaGetErrorString(me));
    }
  }
  ce = cudaStreamSynchronize(cst);
  if (ce != cudaSuccess) return fail(SU2G_ECUDA, std::string("svd: ") + cudaGetErrorString(ce));
  if (trace) {
    static std::mutex trace_mu;
    std::lock_guard<std::mutex> tl(trace_mu);
    if (FILE* f = std::fopen(trace, "a")) {
      const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_call).count();
      std::fprintf(f,
                   "{\"ms\": %.3f, \"max_dcut\": %d, \"lam_cut\": %.6e, \"lam_cut_raw\": %.6e, "
                   "\"noise_floor\": %.6e, \"kept\": %d, \"sectors\": [",
                   ms, max_dcut, lam_cut, lam_cut_raw, noise_floor, total_kept);
      for (size_t q = 0; q < jobs.size(); ++q) {
        std::fprintf(f, "%s{\"m\": %d, \"n\": %d, \"k\": %d, \"ms_eig\": %.3f, \"ms_finish\": %.3f, \"levels\": [",
                     q ? ", " : "", jobs[q].m, jobs[q].n, eig[q].k, eig[q].ms_eig, eig[q].ms_finish);
        for (size_t l = 0; l < eig[q].levels.size(); ++l) std::fprintf(f, "%s%d", l ? ", " : "", eig[q].levels[l]);
        std::fprintf(f, "]}");
      }
      std::fprintf(f, "]}\n");
      std::fclose(f);
    }
  }
  return SU2G_OK;
}
