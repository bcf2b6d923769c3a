// Several H_eff plans applied in shared launches, and their Lanczos solves run
// in lockstep (su2g_heff_batch_*).
//
// Independent DMRG solves that share the GPU (the serving loop) each reach a
// Lanczos solve at every two-site step.  At the bond dimensions of a serving
// stream one H_eff application is a few hundred small block products: a
// persistent GEMM launch over one plan leaves most SMs idle and the launch
// latency dominates.  A batch concatenates the work lists of its plans into
// one list per launch phase, so one application of every plan is the same six
// launches as one application of one plan (digit pack of psi, GEMM phase 1,
// pack of the intermediates, GEMM phase 2, split-tile sums; two GEMM launches
// in FP64 mode), with the tiles of all plans dealt together over the
// persistent grid.
//
// Addressing.  The plans' vectors lie back to back in batch vectors (plan i
// at offset off[i]), so the psi and y buffers of the merged lists are the
// batch's input and output vectors with every plan's offsets shifted by
// off[i]; every other reference (operators, the plan's scratch, packed digit
// slices and exponents) is turned into an absolute address, and the launches
// get null bases for them.
//
// Results.  Every output tile is computed by one CTA from the same segments
// in the same order whichever tiles share its launch, the split tiles are
// summed in part order and the phase-1 row maxima are maxima, so each plan's
// y is bit-identical to its own su2g_heff_apply.  The lockstep Lanczos runs,
// per plan, the same kernels on the same data in the same order as
// su2g_lanczos (lanczos_su2::lanczos1, lanczos_su2.cpp:125-195), with each
// plan's exits decided on the host exactly as there, so energies, vectors and
// matvec counts equal the solo solve's bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "plan_internal.hpp"
#include "tridiag.hpp"

namespace {

int fail(int code, const std::string& msg) { return su2g::set_last_error(code, msg); }

#define BATCH_CUDA(call)                                           \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) return su2g::cuda_status(e_, #call);    \
  } while (0)

template <class T>
cudaError_t upload(const std::vector<T>& v, T** d) {
  return su2g::upload_bytes(v.data(), v.size() * sizeof(T), (void**)d);
}

// The merged device work lists of one subset of the batch's plans.
struct Lists {
  std::vector<int> members;
  // split precision
  su2g::oz::PackJob* jobs[3] = {nullptr, nullptr, nullptr};
  int2* units[3] = {nullptr, nullptr, nullptr};
  int nunits[3] = {0, 0, 0};
  int max_nkt[3] = {0, 0, 0};
  bool rows_pass[3] = {false, false, false};
  su2g::oz::OzSeg* seg1 = nullptr;
  su2g::oz::OzSeg* seg2 = nullptr;
  su2g::oz::OzTile* tile1 = nullptr;
  su2g::oz::OzTile* tile2 = nullptr;
  int ntile1 = 0, ntile2 = 0;
  su2g::oz::RedTile* red = nullptr;
  int nred = 0;
  // FP64
  su2g::GemmSeg* fseg1 = nullptr;
  su2g::GemmSeg* fseg2 = nullptr;
  su2g::GemmTile* ftile1 = nullptr;
  su2g::GemmTile* ftile2 = nullptr;
  int nft1 = 0, nft2 = 0;

  void release(cudaStream_t st) {
    for (int c = 0; c < 3; ++c) {
      su2g::dev_free(jobs[c], st);
      su2g::dev_free(units[c], st);
    }
    for (void* p : {(void*)seg1, (void*)seg2, (void*)tile1, (void*)tile2, (void*)red, (void*)fseg1, (void*)fseg2,
                    (void*)ftile1, (void*)ftile2})
      su2g::dev_free(p, st);
  }
};

}  // namespace

struct su2g_heff_batch {
  std::vector<su2g_heff_plan*> plans;
  int S = 0;
  std::vector<int64_t> off, len;
  int64_t total = 0;
  std::map<std::vector<int>, Lists> lists;  // by member subset
  int* d_err = nullptr;
  // lockstep Lanczos: (M + 1) Krylov vectors, a work vector and a staging
  // vector, each `total` long; per plan a coefficient block and a reduction
  // scratch
  double* d_kry = nullptr;
  int kry_m = 0;
  double* d_coef = nullptr;
  double* d_red = nullptr;
  cudaStream_t last_st = nullptr;

  int coef_len() const { return 3 * (kry_m + 1) + 1; }
  double* ff(int m) { return d_kry + (int64_t)m * total; }
  double* tmpv() { return d_kry + (int64_t)(kry_m + 1) * total; }
  double* stage() { return d_kry + (int64_t)(kry_m + 2) * total; }

  void release() {
    for (auto& kv : lists) kv.second.release(last_st);
    lists.clear();
    su2g::dev_free(d_err, last_st);
    su2g::dev_free(d_kry, last_st);
    su2g::dev_free(d_coef, last_st);
    su2g::dev_free(d_red, last_st);
    d_err = nullptr;
    d_kry = d_coef = d_red = nullptr;
  }
};

namespace {

using su2g::kBufPsi;
using su2g::kBufScratch;
using su2g::kBufY;

// batch addressing of a (buffer, element offset) reference of plan i
void shift_ref(const su2g_heff_batch* B, int i, int* buf, int64_t* off) {
  if (*buf == kBufPsi || *buf == kBufY) *off += B->off[i];
  else if (*buf == kBufScratch) *off += (int64_t)((uintptr_t)B->plans[i]->d_scratch / 8);
}
int64_t packed_abs(const su2g_heff_plan* p, int64_t byte_off) { return byte_off + (int64_t)(uintptr_t)p->d_packed; }
int64_t exps_abs(const su2g_heff_plan* p, int64_t idx) {
  return idx < 0 ? idx : idx + (int64_t)((uintptr_t)p->d_exps / sizeof(int));
}

int build_lists(su2g_heff_batch* B, const std::vector<int>& members, Lists* L) {
  L->members = members;
  cudaError_t e = cudaSuccess;
  if (B->S > 0) {
    for (int c = 1; c <= 2; ++c) {
      std::vector<su2g::oz::PackJob> jobs;
      std::vector<int2> units;
      for (int i : members) {
        const su2g_heff_plan* p = B->plans[i];
        const su2g::oz::OzWork& w = p->oz;
        const int j0 = (int)jobs.size();
        for (su2g::oz::PackJob j : w.jobs[c]) {
          shift_ref(B, i, &j.src_buf, &j.src);
          j.dst = packed_abs(p, j.dst);
          j.exp = exps_abs(p, j.exp);
          j.texp = exps_abs(p, j.texp);
          j.rowmax = exps_abs(p, j.rowmax);
          jobs.push_back(j);
        }
        for (const su2g::oz::Unit& u : w.units[c]) units.push_back(make_int2(u.job + j0, u.rt));
        L->max_nkt[c] = std::max(L->max_nkt[c], w.max_nkt[c]);
        if (!w.units[c].empty()) L->rows_pass[c] = L->rows_pass[c] || w.rows_pass[c];
      }
      L->nunits[c] = (int)units.size();
      if (e == cudaSuccess) e = upload(jobs, &L->jobs[c]);
      if (e == cudaSuccess) e = upload(units, &L->units[c]);
    }
    for (int ph = 1; ph <= 2; ++ph) {
      std::vector<su2g::oz::OzSeg> segs;
      std::vector<su2g::oz::OzTile> tiles;
      for (int i : members) {
        const su2g_heff_plan* p = B->plans[i];
        const auto& ps = ph == 1 ? p->oz.seg1 : p->oz.seg2;
        const auto& pt = ph == 1 ? p->oz.tile1 : p->oz.tile2;
        const int s0 = (int)segs.size();
        for (su2g::oz::OzSeg g : ps) {
          g.a_unit = packed_abs(p, g.a_unit);
          g.b_unit = packed_abs(p, g.b_unit);
          g.a_exp = exps_abs(p, g.a_exp);
          g.b_exp = exps_abs(p, g.b_exp);
          g.a_tmax = exps_abs(p, g.a_tmax);
          segs.push_back(g);
        }
        for (su2g::oz::OzTile t : pt) {
          if (t.nseg == 0 && t.mlen == 0 && t.nlen == 0 && t.rowmax < 0) continue;  // schedule padding
          shift_ref(B, i, &t.c_buf, &t.c);
          t.seg0 += s0;
          t.rowmax = exps_abs(p, t.rowmax);
          tiles.push_back(t);
        }
      }
      su2g::oz::schedule_tiles(&tiles, segs, su2g::oz::ozaki_persistent_grid());
      if (e == cudaSuccess) e = upload(segs, ph == 1 ? &L->seg1 : &L->seg2);
      if (e == cudaSuccess) e = upload(tiles, ph == 1 ? &L->tile1 : &L->tile2);
      (ph == 1 ? L->ntile1 : L->ntile2) = (int)tiles.size();
    }
    std::vector<su2g::oz::RedTile> reds;
    for (int i : members)
      for (su2g::oz::RedTile r : B->plans[i]->oz.red2) {
        shift_ref(B, i, &r.c_buf, &r.c);
        r.part += (int64_t)((uintptr_t)B->plans[i]->d_scratch / 8);  // the partials lie in the plan's scratch
        reds.push_back(r);
      }
    L->nred = (int)reds.size();
    if (e == cudaSuccess) e = upload(reds, &L->red);
  } else {
    for (int ph = 1; ph <= 2; ++ph) {
      std::vector<su2g::GemmSeg> segs;
      std::vector<su2g::GemmTile> tiles;
      for (int i : members) {
        const su2g_heff_plan* p = B->plans[i];
        const auto& ps = ph == 1 ? p->work.seg1 : p->work.seg2;
        const auto& pt = ph == 1 ? p->work.tile1 : p->work.tile2;
        const int s0 = (int)segs.size();
        for (su2g::GemmSeg g : ps) {
          shift_ref(B, i, &g.a_buf, &g.a);
          shift_ref(B, i, &g.b_buf, &g.b);
          segs.push_back(g);
        }
        for (su2g::GemmTile t : pt) {
          shift_ref(B, i, &t.c_buf, &t.c);
          t.seg0 += s0;
          tiles.push_back(t);
        }
      }
      if (e == cudaSuccess) e = upload(segs, ph == 1 ? &L->fseg1 : &L->fseg2);
      if (e == cudaSuccess) e = upload(tiles, ph == 1 ? &L->ftile1 : &L->ftile2);
      (ph == 1 ? L->nft1 : L->nft2) = (int)tiles.size();
    }
  }
  if (e != cudaSuccess) return su2g::cuda_status(e, "heff_batch lists");
  return SU2G_OK;
}

int lists_for(su2g_heff_batch* B, const std::vector<int>& members, Lists** out) {
  auto it = B->lists.find(members);
  if (it == B->lists.end()) {
    Lists L;
    const int rc = build_lists(B, members, &L);
    if (rc) {
      L.release(B->last_st);
      return rc;
    }
    it = B->lists.emplace(members, L).first;
  }
  *out = &it->second;
  return SU2G_OK;
}

// One application of every member plan: y = H x on the members' slices of
// the batch vectors x and y.
int batch_apply(su2g_heff_batch* B, const std::vector<int>& members, const double* x, double* y, cudaStream_t st) {
  Lists* L = nullptr;
  int rc = lists_for(B, members, &L);
  if (rc) return rc;
  su2g::Bases b;
  b.p[su2g::kBufAbs] = 0;
  b.p[kBufPsi] = reinterpret_cast<uintptr_t>(x);
  b.p[kBufY] = reinterpret_cast<uintptr_t>(y);
  b.p[kBufScratch] = 0;  // scratch references are absolute in the merged lists
  if (B->S == 0) {
    BATCH_CUDA(su2g::launch_gemm_f64(L->ftile1, L->nft1, L->fseg1, b, st));
    BATCH_CUDA(su2g::launch_gemm_f64(L->ftile2, L->nft2, L->fseg2, b, st));
  } else {
    for (int i : members) {
      const su2g_heff_plan* p = B->plans[i];
      if (p->oz.rowmax_len > 0)
        BATCH_CUDA(cudaMemsetAsync(p->d_exps + p->oz.rowmax_base, 0, p->oz.rowmax_len * sizeof(int), st));
    }
    BATCH_CUDA(su2g::oz::launch_pack(B->S, L->jobs[1], L->units[1], L->nunits[1], L->max_nkt[1], L->rows_pass[1], b,
                                     nullptr, nullptr, st));
    BATCH_CUDA(su2g::oz::launch_ozaki_gemm(B->S, L->tile1, L->ntile1, L->seg1, nullptr, nullptr, b, B->d_err, st));
    BATCH_CUDA(su2g::oz::launch_pack(B->S, L->jobs[2], L->units[2], L->nunits[2], L->max_nkt[2], L->rows_pass[2], b,
                                     nullptr, nullptr, st));
    BATCH_CUDA(su2g::oz::launch_ozaki_gemm(B->S, L->tile2, L->ntile2, L->seg2, nullptr, nullptr, b, B->d_err, st));
    BATCH_CUDA(su2g::oz::launch_reduce(L->red, L->nred, b, st));
  }
  for (int i : members) {
    su2g_heff_plan* p = B->plans[i];
    if (!p->proj_vec.empty()) BATCH_CUDA(su2g::apply_projectors(p, x + B->off[i], y + B->off[i], st));
  }
  return SU2G_OK;
}

int read_status(su2g_heff_batch* B, cudaStream_t st) {
  int code = 0;
  BATCH_CUDA(cudaMemcpyAsync(&code, B->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  BATCH_CUDA(cudaMemsetAsync(B->d_err, 0, sizeof(int), st));
  BATCH_CUDA(cudaStreamSynchronize(st));
  if (code) return fail(SU2G_ETIMEOUT, "a bounded device wait gave up in a batched launch (code " +
                                           std::to_string(code) + ")");
  return SU2G_OK;
}

// ---------------------------------------------------------------- Lanczos
// The state of one plan's solve (the host side of su2g_lanczos).
struct Solve {
  int i = 0;
  int64_t n = 0;
  int mlanc = 0;
  double* psi = nullptr;  // the caller's vector: start vector in, eigenvector out
  double* coef = nullptr;
  double* red = nullptr;
  int M = 0;
  std::vector<double> aal, nnl, eig, z;
  bool active = true;
  int nmv = 0;
  double energy = 0.0;
  enum { kNone, kFinal, kEarly } pending = kNone;
  double nn = 0, pp = 0, ov = 0;  // check() scalars
  double* alpha(int j) { return coef + j; }
  double* beta(int j) { return coef + M + 1 + j; }
  double* q(int j) { return coef + 2 * (M + 1) + j; }
  double* nnd() { return coef + 3 * (M + 1); }
};

}  // namespace

extern "C" {

int su2g_heff_batch_create(su2g_heff_plan* const* plans, int n, su2g_heff_batch** out) {
  if (!out || n <= 0 || !plans) return fail(SU2G_EINVAL, "heff_batch_create: bad arguments");
  *out = nullptr;
  su2g_heff_batch* B = new su2g_heff_batch();
  for (int i = 0; i < n; ++i) {
    su2g_heff_plan* p = plans[i];
    if (!p) {
      delete B;
      return fail(SU2G_EINVAL, "heff_batch_create: null plan");
    }
    for (su2g_heff_plan* q : B->plans)
      if (q == p) {
        delete B;
        return fail(SU2G_EINVAL, "heff_batch_create: a plan appears twice");
      }
    if (i > 0 && p->S != B->S) {
      delete B;
      return fail(SU2G_EINVAL, "heff_batch_create: the plans must share one precision mode");
    }
    B->S = p->S;
    B->plans.push_back(p);
    B->off.push_back(B->total);
    B->len.push_back(p->work.psi.total);
    B->total += p->work.psi.total;
  }
  const int zero = 0;
  cudaError_t e = su2g::upload_bytes(&zero, sizeof(int), (void**)&B->d_err);
  if (e != cudaSuccess) {
    delete B;
    return su2g::cuda_status(e, "heff_batch_create");
  }
  *out = B;
  return SU2G_OK;
}

int su2g_heff_batch_destroy(su2g_heff_batch* B) {
  if (!B) return SU2G_OK;
  B->release();
  delete B;
  return SU2G_OK;
}

int su2g_heff_batch_info(const su2g_heff_batch* B, int64_t* total_len, int* nplans) {
  if (!B) return fail(SU2G_EINVAL, "heff_batch_info: null batch");
  if (total_len) *total_len = B->total;
  if (nplans) *nplans = (int)B->plans.size();
  return SU2G_OK;
}

int su2g_heff_batch_apply(su2g_heff_batch* B, const double* x, double* y, void* stream) {
  if (!B || (B->total > 0 && (!x || !y))) return fail(SU2G_EINVAL, "heff_batch_apply: bad arguments");
  if (x == y && x) return fail(SU2G_EINVAL, "heff_batch_apply: x and y must not alias");
  cudaStream_t st = (cudaStream_t)stream;
  B->last_st = st;
  std::vector<int> all(B->plans.size());
  for (size_t i = 0; i < all.size(); ++i) all[i] = (int)i;
  return batch_apply(B, all, x, y, st);
}

int su2g_heff_batch_status(su2g_heff_batch* B) {
  if (!B) return fail(SU2G_EINVAL, "heff_batch_status: null batch");
  return read_status(B, B->last_st);
}

int su2g_heff_batch_lanczos(su2g_heff_batch* B, double* const* psi, int mlanc, double* energy, int* nmatvec,
                            void* stream) {
  if (!B || !psi || !energy || mlanc < 2) return fail(SU2G_EINVAL, "heff_batch_lanczos: bad arguments");
  const int np = (int)B->plans.size();
  cudaStream_t st = (cudaStream_t)stream;
  B->last_st = st;
  std::vector<Solve> sv(np);
  int M = 0;
  for (int i = 0; i < np; ++i) {
    Solve& s = sv[i];
    s.i = i;
    s.n = B->len[i];
    if (s.n <= 0) return fail(SU2G_EINVAL, "heff_batch_lanczos: empty vector");
    if (!psi[i]) return fail(SU2G_EINVAL, "heff_batch_lanczos: null vector");
    s.psi = psi[i];
    s.mlanc = mlanc > s.n ? (int)s.n + 1 : mlanc;  // dmrg_su2.cpp:532
    M = std::max(M, s.mlanc);
  }
  const int ns = su2g::reduction_scratch_doubles();
  if (B->kry_m < M) {
    su2g::dev_free(B->d_kry, st);
    su2g::dev_free(B->d_coef, st);
    B->d_kry = B->d_coef = nullptr;
    B->kry_m = 0;
    BATCH_CUDA(su2g::dev_alloc((void**)&B->d_kry, (size_t)(M + 3) * B->total * sizeof(double)));
    B->kry_m = M;
    BATCH_CUDA(su2g::dev_alloc((void**)&B->d_coef, (size_t)np * B->coef_len() * sizeof(double)));
  }
  if (!B->d_red) BATCH_CUDA(su2g::dev_alloc((void**)&B->d_red, (size_t)np * ns * sizeof(double)));
  for (int i = 0; i < np; ++i) {
    sv[i].M = B->kry_m;
    sv[i].coef = B->d_coef + (int64_t)i * B->coef_len();
    sv[i].red = B->d_red + (int64_t)i * ns;
    sv[i].aal.assign(sv[i].mlanc, 0.0);
    sv[i].nnl.assign(sv[i].mlanc + 1, 0.0);
  }
  auto slice = [&](double* v, const Solve& s) { return v + B->off[s.i]; };
  const double tol = 1.e-6;  // lanczos_su2.cpp:128
  // ff[0] = normalised start vector (lanczos_su2.cpp:45-46)
  for (Solve& s : sv) {
    double* f0 = slice(B->ff(0), s);
    BATCH_CUDA(cudaMemcpyAsync(f0, s.psi, s.n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    BATCH_CUDA(su2g::launch_dot_to(f0, f0, s.n, s.red, s.nnd(), st));
    BATCH_CUDA(su2g::launch_normalize_dev(s.nnd(), f0, s.n, s.beta(0), st));
  }
  // host copies of the device scalars of several solves, one synchronisation
  std::vector<double> hbuf;
  auto tridiag = [](Solve& s, int m) {  // lanczos_su2::diatridiag (lanczos_su2.cpp:237-259)
    std::vector<double> d(s.aal.begin(), s.aal.begin() + m), e(m > 1 ? m - 1 : 0);
    for (int k = 0; k + 1 < m; ++k) e[k] = s.nnl[k + 1];
    su2g::tridiag_eigh(d, e, &s.eig, &s.z);
  };
  // psi = sum_j z[j] ff[j]  (lanczos_su2::compute_eigenvector, lanczos_su2.cpp:262-279)
  auto combine = [&](Solve& s, int m) -> int {
    BATCH_CUDA(cudaMemcpyAsync(s.psi, slice(B->ff(0), s), s.n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    BATCH_CUDA(su2g::launch_scale(s.z[0], s.psi, s.n, st));
    for (int j = 1; j < m; ++j) BATCH_CUDA(su2g::launch_axpy(s.z[j], slice(B->ff(j), s), s.psi, s.n, st));
    return SU2G_OK;
  };
  // lanczos_su2::check_eigenvector (lanczos_su2.cpp:320-332) for every solve
  // in `who`: normalise psi, one shared matvec, |Hv| and |<Hv,v>|/|Hv|
  auto checks = [&](const std::vector<int>& who) -> int {
    if (who.empty()) return SU2G_OK;
    hbuf.assign(2 * who.size(), 0.0);
    for (size_t k = 0; k < who.size(); ++k) {
      Solve& s = sv[who[k]];
      BATCH_CUDA(su2g::launch_dot(s.psi, s.psi, s.n, s.red, st));
      BATCH_CUDA(cudaMemcpyAsync(&hbuf[k], s.red + ns - 1, sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    BATCH_CUDA(cudaStreamSynchronize(st));
    for (size_t k = 0; k < who.size(); ++k) {
      Solve& s = sv[who[k]];
      s.nn = hbuf[k];
      BATCH_CUDA(su2g::launch_scale(1.0 / std::sqrt(s.nn), s.psi, s.n, st));
      BATCH_CUDA(cudaMemcpyAsync(slice(B->stage(), s), s.psi, s.n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      ++s.nmv;
    }
    int rc = batch_apply(B, who, B->stage(), B->tmpv(), st);
    if (rc) return rc;
    for (size_t k = 0; k < who.size(); ++k) {
      Solve& s = sv[who[k]];
      double* t = slice(B->tmpv(), s);
      BATCH_CUDA(su2g::launch_dot(t, t, s.n, s.red, st));
      BATCH_CUDA(cudaMemcpyAsync(&hbuf[2 * k], s.red + ns - 1, sizeof(double), cudaMemcpyDeviceToHost, st));
      BATCH_CUDA(su2g::launch_dot(t, s.psi, s.n, s.red, st));
      BATCH_CUDA(cudaMemcpyAsync(&hbuf[2 * k + 1], s.red + ns - 1, sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    BATCH_CUDA(cudaStreamSynchronize(st));
    for (size_t k = 0; k < who.size(); ++k) {
      Solve& s = sv[who[k]];
      s.pp = hbuf[2 * k];
      const double prod = std::sqrt(s.pp);
      s.ov = std::fabs(hbuf[2 * k + 1] / prod);
    }
    return SU2G_OK;
  };
  for (int m = 1;; ++m) {
    std::vector<int> act;
    for (const Solve& s : sv)
      if (s.active) act.push_back(s.i);
    if (act.empty()) break;
    // ff[m] = H ff[m-1] for every active solve, one set of launches
    for (int i : act) ++sv[i].nmv;
    int rc = batch_apply(B, act, B->ff(m - 1), B->ff(m), st);
    if (rc) return rc;
    for (int i : act) {
      Solve& s = sv[i];
      double* fm = slice(B->ff(m), s);
      double* fm1 = slice(B->ff(m - 1), s);
      BATCH_CUDA(su2g::launch_dot_to(fm1, fm, s.n, s.red, s.alpha(m - 1), st));
      if (m == s.mlanc) continue;  // the final matvec: alpha only (lanczos_su2.cpp:189-194)
      BATCH_CUDA(su2g::launch_axpy_neg_dev(s.alpha(m - 1), fm1, fm, s.n, st));
      if (m >= 2) {  // lanczos_su2.cpp:156-173
        BATCH_CUDA(su2g::launch_axpy_neg_dev(s.beta(m - 1), slice(B->ff(m - 2), s), fm, s.n, st));
        for (int j = 0; j < m; ++j) {
          BATCH_CUDA(su2g::launch_dot_to(fm, slice(B->ff(j), s), s.n, s.red, s.q(j), st));
          BATCH_CUDA(su2g::launch_axpy_neg_dev(s.q(j), slice(B->ff(j), s), fm, s.n, st));
        }
      }
      BATCH_CUDA(su2g::launch_dot_to(fm, fm, s.n, s.red, s.nnd(), st));
      BATCH_CUDA(su2g::launch_normalize_dev(s.nnd(), fm, s.n, s.beta(m), st));
    }
    // alpha[0..m-1], beta[1..m] of every active solve to the host
    for (int i : act) {
      Solve& s = sv[i];
      BATCH_CUDA(cudaMemcpyAsync(s.aal.data(), s.alpha(0), m * sizeof(double), cudaMemcpyDeviceToHost, st));
      BATCH_CUDA(cudaMemcpyAsync(s.nnl.data() + 1, s.beta(1), m * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    BATCH_CUDA(cudaStreamSynchronize(st));
    std::vector<int> need_check;
    for (int i : act) {
      Solve& s = sv[i];
      if (s.mlanc == 2) {  // lanczos_su2.cpp:143-154
        if (m == 1 && s.nnl[1] >= tol) continue;
        tridiag(s, m);
        if ((rc = combine(s, m))) return rc;
        s.energy = s.eig[0];
        s.active = false;
        continue;
      }
      if (m == s.mlanc) {  // the final step
        tridiag(s, m);
        if ((rc = combine(s, m))) return rc;
        s.pending = Solve::kFinal;
        need_check.push_back(i);
        continue;
      }
      if (m < 2) continue;
      tridiag(s, m);
      if (s.nnl[m] < tol) {
        if ((rc = combine(s, m))) return rc;
        s.pending = Solve::kFinal;
        need_check.push_back(i);
      } else if (m % 4 == 0) {
        if ((rc = combine(s, m))) return rc;
        s.pending = Solve::kEarly;
        need_check.push_back(i);
      }
    }
    if ((rc = checks(need_check))) return rc;
    for (int i : need_check) {
      Solve& s = sv[i];
      if (s.pending == Solve::kFinal || std::fabs(s.ov - 1.) < 1.e-8) {  // lanczos_su2.cpp:178-188
        s.energy = s.eig[0];
        s.active = false;
      }
      s.pending = Solve::kNone;
    }
  }
  for (const Solve& s : sv) {
    energy[s.i] = s.energy;
    if (nmatvec) nmatvec[s.i] = s.nmv;
  }
  BATCH_CUDA(cudaStreamSynchronize(st));
  // a bounded wait that gave up in any shared launch leaves partial products
  // in some plan's results: every result of the batch is refused
  return read_status(B, st);
}

}  // extern "C"
