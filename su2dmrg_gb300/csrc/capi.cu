// C ABI of libsu2g.so (declared in include/su2g.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "env_plan.hpp"
#include "heff_plan.hpp"
#include "kernels.hpp"
#include "ozaki_plan.hpp"
#include "plan_internal.hpp"
#include "su2_meta.hpp"
#include "su2g.h"
#include "tridiag.hpp"

namespace {
thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(e == cudaErrorMemoryAllocation ? SU2G_ENOMEM : SU2G_ECUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

#define SU2G_CUDA(call)                                 \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

template <class T>
cudaError_t upload(const std::vector<T>& v, T** dptr) {
  return su2g::upload_bytes(v.data(), v.size() * sizeof(T), (void**)dptr);
}

template <class T>
cudaError_t dalloc(T** dptr, size_t bytes) {
  return su2g::dev_alloc((void**)dptr, bytes);
}

// Host arrays gathered into one staging buffer (256-byte aligned pieces) and
// sent to the device in one allocation and one copy: a plan's work lists
// cost one transfer instead of one allocation, copy and wait each.
struct Staging {
  std::vector<uint8_t> host;
  std::vector<std::pair<void**, size_t>> slots;
  void add_bytes(const void* src, size_t n, void** slot) {
    *slot = nullptr;
    if (n == 0) return;
    const size_t off = (host.size() + 255) & ~(size_t)255;
    host.resize(off + n);
    std::memcpy(host.data() + off, src, n);
    slots.push_back({slot, off});
  }
  template <class T>
  void add(const std::vector<T>& v, T** slot) {
    add_bytes(v.data(), v.size() * sizeof(T), (void**)slot);
  }
  // with `caller`, the copy is queued on that stream (pageable source: it is
  // staged before the call returns); else on the thread's own stream, waited for
  cudaError_t send(void** base, const cudaStream_t* caller) {
    *base = nullptr;
    if (host.empty()) return cudaSuccess;
    cudaError_t e = su2g::dev_alloc(base, host.size());
    cudaStream_t st = nullptr;
    if (e == cudaSuccess) {
      if (caller) st = *caller;
      else e = su2g::setup_stream(&st);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(*base, host.data(), host.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !caller) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    for (auto& sl : slots) *sl.first = static_cast<uint8_t*>(*base) + sl.second;
    return cudaSuccess;
  }
};
}  // namespace

int su2g::set_last_error(int code, const std::string& msg) { return fail(code, msg); }


namespace {
int slices_of_mode(int mode) {
  if (mode == SU2G_MODE_F64) return 0;
  if (mode == SU2G_MODE_SPLIT_BF16) return 7;
  if (mode == SU2G_MODE_SPLIT_BF16_FAST) return 6;
  return -1;
}

su2g::Bases make_bases(const su2g_heff_plan* p, const double* psi, double* y) {
  su2g::Bases b;
  b.p[su2g::kBufAbs] = 0;
  b.p[su2g::kBufPsi] = reinterpret_cast<uintptr_t>(psi);
  b.p[su2g::kBufY] = reinterpret_cast<uintptr_t>(y);
  b.p[su2g::kBufScratch] = reinterpret_cast<uintptr_t>(p->d_scratch);
  return b;
}

// device buffers of the split-precision work, and the one-time packing of
// the operators (they stay fixed for the lifetime of the plan).  The pack
// reads the caller's operator data: with `caller` given (the one-shot work
// lists, whose operands may still be in flight on the caller's stream, such
// as transposes queued just before) it runs on that stream, ordered after
// them; without (su2g_heff_plan_create, whose operands must be complete) on
// the thread's own stream, waited for.
cudaError_t setup_split(su2g_heff_plan* p, const cudaStream_t* caller) {
  su2g::oz::OzWork& w = p->oz;
  cudaError_t e = dalloc(&p->d_packed, std::max<int64_t>(w.packed_bytes, 16));
  if (e == cudaSuccess) e = dalloc(&p->d_exps, std::max<int64_t>(w.exp_len, 1) * sizeof(int));
  if (e != cudaSuccess) return e;
  const su2g::Bases b = make_bases(p, nullptr, nullptr);
  cudaStream_t st = nullptr;
  if (caller) st = *caller;
  else e = su2g::setup_stream(&st);
  if (e == cudaSuccess)
    e = su2g::oz::launch_pack(p->S, p->d_jobs[0], p->d_units[0], (int)w.units[0].size(), w.max_nkt[0],
                              w.rows_pass[0], b, p->d_packed, p->d_exps, st);
  if (e == cudaSuccess && !caller) e = cudaStreamSynchronize(st);
  // the GEMM's one-time setup happens here, never inside a graph capture
  if (e == cudaSuccess) e = su2g::oz::prepare_ozaki_gemm(p->S);
  return e;
}
}  // namespace

extern "C" {

int su2g_version(void) { return 100; }

const char* su2g_last_error(void) { return g_err.c_str(); }

int su2g_struct_nten(const int* desc) {
  su2g::Struct s;
  std::string e;
  if (!desc || !s.parse(desc, &e)) return -1;
  return s.nten;
}

int su2g_struct_legal(const int* desc, int* legal) {
  su2g::Struct s;
  std::string e;
  if (!desc || !legal || !s.parse(desc, &e)) return -1;
  for (int i = 0; i < s.nten; ++i) legal[i] = s.legal_block(i) ? 1 : 0;
  return s.nten;
}

int64_t su2g_layout(const int* desc, const int* flag, int64_t* offsets) {
  su2g::Struct s;
  std::string e;
  if (!desc || !s.parse(desc, &e)) return -1;
  s.set_layout(flag);
  if (offsets) std::copy(s.offset.begin(), s.offset.end(), offsets);
  return s.total;
}

int su2g_bond_fuse(int n1, const int* a1, const int* d1, int n2, const int* a2, const int* d2, int* nout,
                   int* aout, int* dout) {
  if (n1 < 0 || n2 < 0 || !nout || !aout || !dout) return fail(SU2G_EINVAL, "bond_fuse: bad arguments");
  su2g::Bond b1, b2;
  b1.angm.assign(a1, a1 + n1);
  b1.dim.assign(d1, d1 + n1);
  b2.angm.assign(a2, a2 + n2);
  b2.dim.assign(d2, d2 + n2);
  su2g::Bond f = su2g::fuse(b1, b2);
  if (f.n() > 64) return fail(SU2G_EINVAL, "bond_fuse: more than 64 sectors");
  *nout = f.n();
  std::copy(f.angm.begin(), f.angm.end(), aout);
  std::copy(f.dim.begin(), f.dim.end(), dout);
  return SU2G_OK;
}

int su2g_make_cgc(int j1, int j2, int j3, double* out) {
  if (j1 < 0 || j2 < 0 || j3 < 0 || !out) return fail(SU2G_EINVAL, "make_cgc: bad arguments");
  su2g::make_cgc(j1, j2, j3, out);
  return SU2G_OK;
}

int su2g_fac_hamilt_vec(int max_angm, double* out) {
  if (max_angm <= 0 || max_angm > 64 || !out) return fail(SU2G_EINVAL, "fac_hamilt_vec: bad arguments");
  su2g::fac_hamilt_vec(max_angm, out);
  return SU2G_OK;
}

int su2g_fac_table(int table, int side, int a, int b, int c, int d, int e, double* out) {
  if (!out || table < 0 || table > 2 || (side != 0 && side != 1))
    return fail(SU2G_EINVAL, "fac_table: bad arguments");
  *out = table == 0   ? su2g::fac_operator_onsite(side, a, b, c, d, e)
         : table == 1 ? su2g::fac_operator_pairup(side, a, b, c, d, e)
                      : su2g::fac_permutation(side, a, b, c, d, e);
  return SU2G_OK;
}

int su2g_fac_operator_transformation(int side, int j, int m, int l, int i, int k, int p, double* out) {
  if (!out || side < 0 || side > 1 || j < 0 || m < 0 || l < 0 || i < 0 || k < 0 || p < 0)
    return fail(SU2G_EINVAL, "fac_operator_transformation: bad arguments");
  *out = su2g::fac_operator_transformation(side, j, m, l, i, k, p);
  return SU2G_OK;
}

}  // extern "C"

namespace {
// device side of a plan whose host work lists are built: work lists, scratch
// (intermediates + split partial tiles) and, in split mode, the packed operands
int plan_from_work(su2g::HeffWork&& work, int mode, su2g_heff_plan** plan, const cudaStream_t* caller = nullptr) {
  *plan = nullptr;
  const int S = slices_of_mode(mode);
  if (S < 0) return fail(SU2G_EINVAL, "plan_create: unknown mode");
  su2g_heff_plan* p = new su2g_heff_plan();
  p->mode = mode;
  p->S = S;
  p->work = std::move(work);
  std::string err;
  if (S > 0) {
    const int rc = su2g::oz::build_ozaki_work(p->work, S, &p->oz, &err);
    if (rc) {
      delete p;
      return fail(rc, err);
    }
  }
  // every work list of the mode and the error word (set by a bounded device
  // wait that gave up, read by su2g_heff_plan_status and every
  // result-returning caller of the plan) in one block and one copy
  Staging stage;
  const int zero = 0;
  stage.add_bytes(&zero, sizeof(int), (void**)&p->d_err);
  std::vector<int2> units[3];
  if (S == 0) {
    stage.add(p->work.seg1, &p->d_seg1);
    stage.add(p->work.seg2, &p->d_seg2);
    stage.add(p->work.tile1, &p->d_tile1);
    stage.add(p->work.tile2, &p->d_tile2);
  } else {
    const su2g::oz::OzWork& w = p->oz;
    for (int c = 0; c < 3; ++c) {
      stage.add(w.jobs[c], &p->d_jobs[c]);
      units[c].resize(w.units[c].size());
      for (size_t i = 0; i < units[c].size(); ++i) units[c][i] = make_int2(w.units[c][i].job, w.units[c][i].rt);
      stage.add(units[c], &p->d_units[c]);
    }
    stage.add(w.seg1, &p->d_oseg1);
    stage.add(w.seg2, &p->d_oseg2);
    stage.add(w.tile1, &p->d_otile1);
    stage.add(w.tile2, &p->d_otile2);
    stage.add(w.red2, &p->d_red2);
  }
  cudaError_t e = stage.send(&p->d_lists, caller);
  const int64_t scratch_doubles = p->work.scratch_len + p->oz.partial_len;
  if (e == cudaSuccess && scratch_doubles > 0) e = dalloc(&p->d_scratch, scratch_doubles * sizeof(double));
  if (e == cudaSuccess && S > 0) e = setup_split(p, caller);
  if (caller) p->last_st = *caller;
  if (e != cudaSuccess) {
    p->release();
    delete p;
    return cuda_fail(e, "plan_create");
  }
  *plan = p;
  return SU2G_OK;
}

}  // namespace

// one application of a work list on absolute addresses: build, run, wait,
// check, free
int su2g::run_work_once(HeffWork&& w, int mode, void* stream) {
  bool any = false;  // some block has a tile
  for (const auto* v : {&w.blk1, &w.blk2})
    for (const OutBlock& b : *v) any = any || (b.M > 0 && b.N > 0);
  if (!any) return SU2G_OK;
  su2g_heff_plan* p = nullptr;
  const cudaStream_t st = (cudaStream_t)stream;
  int rc = plan_from_work(std::move(w), mode, &p, &st);
  if (rc) return rc;
  rc = su2g_heff_apply(p, nullptr, nullptr, stream);
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  int code = 0;
  if (!rc && e == cudaSuccess) rc = su2g_heff_plan_status(p, &code);
  su2g_heff_plan_destroy(p);
  if (e != cudaSuccess) return cuda_fail(e, "work list");
  return rc;
}

namespace {
// one-shot environment update
int env_batch_run(su2g_tensor uu, su2g_tensor vv, int flag, int njobs, const su2g_env_job* jobs, int nslots,
                  double* const* outs, int mode, void* stream) {
  if (!outs && nslots > 0) return fail(SU2G_EINVAL, "env: missing output pointers");
  if (slices_of_mode(mode) < 0) return fail(SU2G_EINVAL, "env: unknown mode");
  su2g::HeffWork w;
  std::vector<su2g::Struct> ys;
  std::string err;
  int rc = su2g::build_env_batch(uu, vv, flag, njobs, jobs, nslots, outs, &w, &ys, &err, slices_of_mode(mode) == 0);
  if (rc) return fail(rc, err);
  return su2g::run_work_once(std::move(w), mode, stream);
}

int env_batch_layout(su2g_tensor uu, su2g_tensor vv, int flag, int njobs, const su2g_env_job* jobs, int slot,
                     int* out_desc, int out_desc_cap, int* out_flag, int out_flag_cap, int64_t* out_len) {
  su2g::HeffWork w;
  std::vector<su2g::Struct> ys;
  std::string err;
  // the jobs of the slot asked for, as a batch of one slot
  std::vector<su2g_env_job> mine;
  for (int t = 0; t < njobs && jobs; ++t)
    if (jobs[t].slot == slot) {
      mine.push_back(jobs[t]);
      mine.back().slot = 0;
    }
  if (mine.empty()) return fail(SU2G_EINVAL, "env layout: no job writes slot " + std::to_string(slot));
  int rc = su2g::build_env_batch(uu, vv, flag, (int)mine.size(), mine.data(), 1, nullptr, &w, &ys, &err);
  if (rc) return fail(rc, err);
  const su2g::Struct& y = ys[0];
  std::vector<int> d = {y.nbond, y.locspin};
  for (int l = 0; l < y.nbond; ++l) {
    d.push_back(y.legs[l].dir);
    d.push_back(y.legs[l].n());
    for (int a : y.legs[l].angm) d.push_back(a);
    for (int x : y.legs[l].dim) d.push_back(x);
  }
  if (!out_desc || !out_flag || (int)d.size() > out_desc_cap || y.nten > out_flag_cap)
    return fail(SU2G_EINVAL, "env layout: output arrays too small");
  std::copy(d.begin(), d.end(), out_desc);
  std::copy(y.flag.begin(), y.flag.end(), out_flag);
  if (out_len) *out_len = y.total;
  return SU2G_OK;
}

// overlap_transformation / operator_transformation batches: one job per operator
std::vector<su2g_env_job> transform_jobs(int kind, int nops, const su2g_tensor* ops) {
  std::vector<su2g_env_job> js(std::max(nops, 0));
  for (int t = 0; t < nops; ++t) {
    js[t] = su2g_env_job{};
    js[t].kind = kind;
    js[t].slot = t;
    js[t].coef = 1.0;
    js[t].x = ops[t];
  }
  return js;
}

int env_run(int kind, su2g_tensor uu, su2g_tensor vv, int flag, int nops, const su2g_tensor* ops, double* const* outs,
            int mode, void* stream) {
  if (nops < 0 || (nops > 0 && !ops)) return fail(SU2G_EINVAL, "env: bad operator list");
  const std::vector<su2g_env_job> js = transform_jobs(kind, nops, ops);
  return env_batch_run(uu, vv, flag, nops, js.data(), nops, outs, mode, stream);
}

int env_layout(int kind, su2g_tensor uu, su2g_tensor vv, int flag, su2g_tensor op, int* out_desc, int out_desc_cap,
               int* out_flag, int out_flag_cap, int64_t* out_len) {
  const std::vector<su2g_env_job> js = transform_jobs(kind, 1, &op);
  return env_batch_layout(uu, vv, flag, 1, js.data(), 0, out_desc, out_desc_cap, out_flag, out_flag_cap, out_len);
}
}  // namespace

extern "C" {

int su2g_heff_plan_create(const int* psi_desc, const int* psi_flag, int nterms, const su2g_term* terms,
                          const su2g_tensor* hl, double hl_coef, const su2g_tensor* hr, double hr_coef, int mode,
                          su2g_heff_plan** plan) {
  if (!plan) return fail(SU2G_EINVAL, "plan_create: null output");
  *plan = nullptr;
  if (slices_of_mode(mode) < 0) return fail(SU2G_EINVAL, "plan_create: unknown mode");
  su2g::HeffWork w;
  std::string err;
  const int rc = su2g::build_heff_work(psi_desc, psi_flag, nterms, terms, hl, hl_coef, hr, hr_coef, &w, &err,
                                       slices_of_mode(mode) == 0);
  if (rc) return fail(rc, err);
  return plan_from_work(std::move(w), mode, plan);
}

int su2g_operator_transformation_layout(su2g_tensor uu, su2g_tensor vv, int flag, su2g_tensor op, int* out_desc,
                                        int out_desc_cap, int* out_flag, int out_flag_cap, int64_t* out_len) {
  return env_layout(1, uu, vv, flag, op, out_desc, out_desc_cap, out_flag, out_flag_cap, out_len);
}

int su2g_operator_transformation(su2g_tensor uu, su2g_tensor vv, int flag, int nops, const su2g_tensor* ops,
                                 double* const* outs, int mode, void* stream) {
  return env_run(1, uu, vv, flag, nops, ops, outs, mode, stream);
}

int su2g_overlap_transformation_layout(su2g_tensor uu, su2g_tensor vv, int flag, su2g_tensor hh, int* out_desc,
                                       int out_desc_cap, int* out_flag, int out_flag_cap, int64_t* out_len) {
  return env_layout(0, uu, vv, flag, hh, out_desc, out_desc_cap, out_flag, out_flag_cap, out_len);
}

int su2g_overlap_transformation(su2g_tensor uu, su2g_tensor vv, int flag, int nops, const su2g_tensor* hhs,
                                double* const* outs, int mode, void* stream) {
  return env_run(0, uu, vv, flag, nops, hhs, outs, mode, stream);
}

int su2g_env_layout(su2g_tensor uu, su2g_tensor vv, int flag, int njobs, const su2g_env_job* jobs, int slot,
                    int* out_desc, int out_desc_cap, int* out_flag, int out_flag_cap, int64_t* out_len) {
  return env_batch_layout(uu, vv, flag, njobs, jobs, slot, out_desc, out_desc_cap, out_flag, out_flag_cap, out_len);
}

int su2g_env_run(su2g_tensor uu, su2g_tensor vv, int flag, int njobs, const su2g_env_job* jobs, int nslots,
                 double* const* outs, int mode, void* stream) {
  return env_batch_run(uu, vv, flag, njobs, jobs, nslots, outs, mode, stream);
}

int su2g_env_validate(su2g_tensor uu, su2g_tensor vv, int flag, int njobs, const su2g_env_job* jobs, int nslots,
                      int mode, double* flops, int64_t* scratch_bytes) {
  const int S = slices_of_mode(mode);
  if (S < 0) return fail(SU2G_EINVAL, "env_validate: unknown mode");
  if (nslots < 0) return fail(SU2G_EINVAL, "env_validate: bad slot count");
  // stand-in output addresses: the work list is only built and checked
  std::vector<double*> outs(std::max(nslots, 1));
  for (int s = 0; s < nslots; ++s) outs[s] = reinterpret_cast<double*>((uintptr_t)(s + 1) << 40);
  su2g::HeffWork w;
  std::vector<su2g::Struct> ys;
  std::string err;
  int rc = su2g::build_env_batch(uu, vv, flag, njobs, jobs, nslots, outs.data(), &w, &ys, &err, S == 0);
  if (rc) return fail(rc, err);
  int64_t bytes = w.scratch_len * (int64_t)sizeof(double);
  if (S > 0) {
    su2g::oz::OzWork oz;
    rc = su2g::oz::build_ozaki_work(w, S, &oz, &err);
    if (rc) return fail(rc, err);
    bytes = (w.scratch_len + oz.partial_len) * (int64_t)sizeof(double) + oz.packed_bytes +
            oz.exp_len * (int64_t)sizeof(int32_t);
  }
  if (flops) *flops = w.flops;
  if (scratch_bytes) *scratch_bytes = bytes;
  return SU2G_OK;
}

int su2g_heff_plan_validate(const int* psi_desc, const int* psi_flag, int nterms, const su2g_term* terms,
                            const su2g_tensor* hl, double hl_coef, const su2g_tensor* hr, double hr_coef, int mode,
                            double* flops, int64_t* scratch_bytes) {
  const int S = slices_of_mode(mode);
  if (S < 0) return fail(SU2G_EINVAL, "plan_validate: unknown mode");
  su2g::HeffWork w;
  std::string err;
  int rc = su2g::build_heff_work(psi_desc, psi_flag, nterms, terms, hl, hl_coef, hr, hr_coef, &w, &err, S == 0);
  if (rc) return fail(rc, err);
  int64_t bytes = w.scratch_len * (int64_t)sizeof(double);
  if (S > 0) {
    su2g::oz::OzWork oz;
    rc = su2g::oz::build_ozaki_work(w, S, &oz, &err);
    if (rc) return fail(rc, err);
    bytes += oz.packed_bytes + oz.exp_len * (int64_t)sizeof(int) + oz.partial_len * (int64_t)sizeof(double);
  }
  if (flops) *flops = w.flops;
  if (scratch_bytes) *scratch_bytes = bytes;
  return SU2G_OK;
}

}  // extern "C"

namespace {
// FNV-style digest of every field of the work lists a mode builds (the
// lists fix every sum's order, so equal digests mean bit-identical results)
struct Digest {
  uint64_t h = 1469598103934665603ull;
  void add(int64_t x) {
    h ^= (uint64_t)x;
    h *= 1099511628211ull;
    h ^= h >> 29;
  }
  void add(double x) {
    int64_t b;
    std::memcpy(&b, &x, 8);
    add(b);
  }
};

void digest_work(const su2g::HeffWork& w, const su2g::oz::OzWork* oz, Digest& d) {
  for (const auto* v : {&w.seg1, &w.seg2}) {
    d.add((int64_t)v->size());
    for (const su2g::GemmSeg& g : *v) {
      d.add(g.a), d.add((int64_t)g.a_buf), d.add(g.a_len), d.add(g.b), d.add((int64_t)g.b_buf), d.add(g.b_len);
      d.add((int64_t)g.lda), d.add((int64_t)g.ldb), d.add((int64_t)g.K), d.add((int64_t)g.transA), d.add(g.alpha);
    }
  }
  for (const auto* v : {&w.blk1, &w.blk2}) {
    d.add((int64_t)v->size());
    for (const su2g::OutBlock& b : *v) {
      d.add(b.c), d.add(b.c_len), d.add((int64_t)b.c_buf), d.add((int64_t)b.ldc), d.add((int64_t)b.M);
      d.add((int64_t)b.N), d.add((int64_t)b.seg0), d.add((int64_t)b.nseg);
    }
  }
  for (const auto* v : {&w.tile1, &w.tile2}) {
    d.add((int64_t)v->size());
    for (const su2g::GemmTile& t : *v) {
      d.add(t.c), d.add(t.c_len), d.add((int64_t)t.c_buf), d.add((int64_t)t.ldc), d.add((int64_t)t.m0);
      d.add((int64_t)t.n0), d.add((int64_t)t.mlen), d.add((int64_t)t.nlen), d.add((int64_t)t.seg0);
      d.add((int64_t)t.nseg), d.add(t.kwork), d.add((int64_t)t.cls);
    }
  }
  d.add(w.scratch_len), d.add(w.flops), d.add(w.max_k), d.add(w.psi.total);
  if (!oz) return;
  const su2g::oz::OzWork& o = *oz;
  for (const auto* v : {&o.seg1, &o.seg2}) {
    d.add((int64_t)v->size());
    for (const su2g::oz::OzSeg& z : *v) d.add(z.a_unit), d.add(z.b_unit), d.add(z.a_exp), d.add(z.b_exp), d.add(z.a_tmax), d.add((int64_t)z.nks);
  }
  for (const auto* v : {&o.tile1, &o.tile2}) {
    d.add((int64_t)v->size());
    for (const su2g::oz::OzTile& t : *v) {
      d.add(t.c), d.add((int64_t)t.c_buf), d.add((int64_t)t.ldc), d.add((int64_t)t.m0), d.add((int64_t)t.n0);
      d.add((int64_t)t.mlen), d.add((int64_t)t.nlen), d.add((int64_t)t.seg0), d.add((int64_t)t.nseg), d.add(t.work);
      d.add(t.rowmax), d.add((int64_t)t.rms);
    }
  }
  for (int c = 0; c < 3; ++c) {
    d.add((int64_t)o.jobs[c].size());
    for (const su2g::oz::PackJob& j : o.jobs[c]) {
      d.add(j.src), d.add((int64_t)j.src_buf), d.add((int64_t)j.R), d.add((int64_t)j.K), d.add(j.ld_r), d.add(j.ld_k);
      d.add((int64_t)j.rt), d.add((int64_t)j.nrt), d.add((int64_t)j.nkt), d.add(j.alpha), d.add(j.dst), d.add(j.exp);
      d.add(j.texp), d.add(j.rowmax);
    }
    d.add((int64_t)o.units[c].size());
    for (const su2g::oz::Unit& u : o.units[c]) d.add((int64_t)u.job), d.add((int64_t)u.rt);
    d.add((int64_t)o.max_nkt[c]), d.add((int64_t)o.rows_pass[c]);
  }
  d.add((int64_t)o.red2.size());
  for (const su2g::oz::RedTile& r : o.red2) {
    d.add(r.c), d.add((int64_t)r.c_buf), d.add((int64_t)r.ldc), d.add((int64_t)r.m0), d.add((int64_t)r.n0);
    d.add((int64_t)r.mlen), d.add((int64_t)r.nlen), d.add((int64_t)r.nparts), d.add(r.part);
  }
  d.add(o.packed_bytes), d.add(o.exp_len), d.add(o.rowmax_base), d.add(o.rowmax_len), d.add(o.scratch_base);
  d.add(o.partial_len);
}

int digest_of(su2g::HeffWork& w, int S, uint64_t* digest) {
  Digest d;
  std::string err;
  if (S > 0) {
    su2g::oz::OzWork oz;
    const int rc = su2g::oz::build_ozaki_work(w, S, &oz, &err);
    if (rc) return fail(rc, err);
    digest_work(w, &oz, d);
  } else {
    digest_work(w, nullptr, d);
  }
  *digest = d.h;
  return SU2G_OK;
}
}  // namespace

extern "C" {

int su2g_heff_plan_digest(const int* psi_desc, const int* psi_flag, int nterms, const su2g_term* terms,
                          const su2g_tensor* hl, double hl_coef, const su2g_tensor* hr, double hr_coef, int mode,
                          uint64_t* digest) {
  const int S = slices_of_mode(mode);
  if (S < 0 || !digest) return fail(SU2G_EINVAL, "plan_digest: bad arguments");
  su2g::HeffWork w;
  std::string err;
  const int rc = su2g::build_heff_work(psi_desc, psi_flag, nterms, terms, hl, hl_coef, hr, hr_coef, &w, &err, S == 0);
  if (rc) return fail(rc, err);
  return digest_of(w, S, digest);
}

int su2g_env_digest(su2g_tensor uu, su2g_tensor vv, int flag, int njobs, const su2g_env_job* jobs, int nslots,
                    double* const* outs, int mode, uint64_t* digest) {
  const int S = slices_of_mode(mode);
  if (S < 0 || !digest || nslots < 0 || (nslots > 0 && !outs)) return fail(SU2G_EINVAL, "env_digest: bad arguments");
  su2g::HeffWork w;
  std::vector<su2g::Struct> ys;
  std::string err;
  const int rc = su2g::build_env_batch(uu, vv, flag, njobs, jobs, nslots, outs, &w, &ys, &err, S == 0);
  if (rc) return fail(rc, err);
  return digest_of(w, S, digest);
}

int su2g_heff_plan_launches(const su2g_heff_plan* p, int* n) {
  if (!p || !n) return fail(SU2G_EINVAL, "plan_launches: bad arguments");
  int c = 0;
  if (p->S == 0) {
    c += p->work.tile1.empty() ? 0 : 1;
    c += p->work.tile2.empty() ? 0 : 1;
  } else {
    const su2g::oz::OzWork& w = p->oz;
    for (int k = 1; k <= 2; ++k)
      if (!w.units[k].empty()) c += w.rows_pass[k] ? 2 : 1;
    c += w.tile1.empty() ? 0 : 1;
    c += w.tile2.empty() ? 0 : 1;
    c += w.red2.empty() ? 0 : 1;
  }
  c += 2 * (int)p->proj_vec.size();
  *n = c;
  return SU2G_OK;
}

int su2g_selftest_bounded_wait(long long iterations, void* stream) {
  if (iterations <= 0) return fail(SU2G_EINVAL, "selftest_bounded_wait: iterations must be positive");
  int timed_out = 0;
  SU2G_CUDA(su2g::oz::bounded_wait_selftest(iterations, &timed_out, (cudaStream_t)stream));
  if (timed_out) return fail(SU2G_ETIMEOUT, "bounded wait gave up after " + std::to_string(iterations) + " polls");
  return SU2G_OK;
}

int su2g_heff_plan_status(su2g_heff_plan* p, int* code) {
  if (!p || !code) return fail(SU2G_EINVAL, "plan_status: bad arguments");
  *code = 0;
  if (!p->d_err) return SU2G_OK;
  // read after the plan's latest work, on its stream
  SU2G_CUDA(cudaMemcpyAsync(code, p->d_err, sizeof(int), cudaMemcpyDeviceToHost, p->last_st));
  SU2G_CUDA(cudaMemsetAsync(p->d_err, 0, sizeof(int), p->last_st));
  SU2G_CUDA(cudaStreamSynchronize(p->last_st));
  if (*code) return fail(SU2G_ETIMEOUT, "a bounded device wait gave up (code " + std::to_string(*code) + ")");
  return SU2G_OK;
}

int su2g_f64_tile_table(const int* m_edges, int nm, const int* n_edges, int nn, const int* cls) {
  if (nm <= 0 || nn <= 0 || !m_edges || !n_edges || !cls) return fail(SU2G_EINVAL, "f64_tile_table: bad arguments");
  if (su2g::set_tile_table(m_edges, nm, n_edges, nn, cls))
    return fail(SU2G_EINVAL, "f64_tile_table: edges must increase and classes lie in 0..3");
  return SU2G_OK;
}

int su2g_f64_tile_bench(int M, int N, int K, int nblocks, int cls, int reps, double* ms, void* stream) {
  if (M <= 0 || N <= 0 || K <= 0 || nblocks <= 0 || cls < 0 || cls >= su2g::kTileClasses || reps <= 0 || !ms)
    return fail(SU2G_EINVAL, "f64_tile_bench: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t na = (int64_t)M * K, nb = (int64_t)K * N, nc = (int64_t)M * N;
  double* buf = nullptr;
  SU2G_CUDA(dalloc(&buf, (size_t)nblocks * (na + nb + nc) * sizeof(double)));
  std::vector<su2g::GemmSeg> segs;
  std::vector<su2g::GemmTile> tiles;
  const int tm = su2g::kTileClassM[cls], tn = su2g::kTileClassN[cls];
  for (int b = 0; b < nblocks; ++b) {
    const int64_t base = (int64_t)b * (na + nb + nc);
    su2g::GemmSeg g{};
    g.a = base;
    g.b = base + na;
    g.a_len = na;
    g.b_len = nb;
    g.a_buf = g.b_buf = su2g::kBufScratch;
    g.lda = M;
    g.ldb = K;
    g.K = K;
    g.transA = 0;
    g.alpha = 1.0;
    segs.push_back(g);
    for (int m0 = 0; m0 < M; m0 += tm)
      for (int n0 = 0; n0 < N; n0 += tn) {
        su2g::GemmTile t{};
        t.c = base + na + nb;
        t.c_len = nc;
        t.c_buf = su2g::kBufScratch;
        t.ldc = M;
        t.m0 = m0;
        t.n0 = n0;
        t.mlen = std::min(tm, M - m0);
        t.nlen = std::min(tn, N - n0);
        t.seg0 = b;
        t.nseg = 1;
        t.kwork = K;
        t.cls = cls;
        tiles.push_back(t);
      }
  }
  su2g::GemmSeg* dseg = nullptr;
  su2g::GemmTile* dtile = nullptr;
  cudaError_t e = cudaMemsetAsync(buf, 0, (size_t)nblocks * (na + nb + nc) * sizeof(double), st);
  if (e == cudaSuccess) e = upload(segs, &dseg);
  if (e == cudaSuccess) e = upload(tiles, &dtile);
  su2g::Bases bases{};
  bases.p[su2g::kBufScratch] = reinterpret_cast<uintptr_t>(buf);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = su2g::launch_gemm_f64(dtile, (int)tiles.size(), dseg, bases, st);  // warm
  if (e == cudaSuccess) e = cudaEventRecord(e0, st);
  for (int r = 0; r < reps && e == cudaSuccess; ++r) e = su2g::launch_gemm_f64(dtile, (int)tiles.size(), dseg, bases, st);
  if (e == cudaSuccess) e = cudaEventRecord(e1, st);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float t = 0;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  su2g::dev_free(dseg, st);
  su2g::dev_free(dtile, st);
  su2g::dev_free(buf, st);
  if (e != cudaSuccess) return cuda_fail(e, "f64_tile_bench");
  *ms = t / reps;
  return SU2G_OK;
}

int su2g_heff_plan_mark_failed(su2g_heff_plan* p, int code) {
  if (!p || !p->d_err || code == 0) return fail(SU2G_EINVAL, "plan_mark_failed: bad arguments");
  SU2G_CUDA(cudaMemcpyAsync(p->d_err, &code, sizeof(int), cudaMemcpyHostToDevice, p->last_st));
  SU2G_CUDA(cudaStreamSynchronize(p->last_st));
  return SU2G_OK;
}

int su2g_heff_plan_info(const su2g_heff_plan* p, double* flops, int64_t* psi_len, int64_t* scratch_bytes,
                        int* ntiles) {
  if (!p) return fail(SU2G_EINVAL, "plan_info: null plan");
  if (flops) *flops = p->work.flops;
  if (psi_len) *psi_len = p->work.psi.total;
  if (scratch_bytes)
    *scratch_bytes = (p->work.scratch_len + p->oz.partial_len) * (int64_t)sizeof(double) + p->oz.packed_bytes +
                     p->oz.exp_len * (int64_t)sizeof(int);
  if (ntiles) {
    if (p->S > 0) {  // without the empty tiles that pad the persistent schedule
      int n = 0;
      for (const auto* v : {&p->oz.tile1, &p->oz.tile2})
        for (const su2g::oz::OzTile& t : *v) n += t.mlen > 0;
      *ntiles = n;
    } else {
      *ntiles = (int)(p->work.tile1.size() + p->work.tile2.size());
    }
  }
  return SU2G_OK;
}

}  // extern "C"

// y -= w_j (o_j . psi) o_j for every projector, the dot product kept on the device
cudaError_t su2g::apply_projectors(su2g_heff_plan* p, const double* psi, double* y, cudaStream_t st) {
  const int64_t n = p->work.psi.total;
  const int ns = su2g::reduction_scratch_doubles();
  for (size_t j = 0; j < p->proj_vec.size(); ++j) {
    double* scr = p->d_proj + (int64_t)j * ns;
    cudaError_t e = su2g::launch_dot(p->proj_vec[j], psi, n, scr, st);
    if (e == cudaSuccess) e = su2g::launch_axpy_dev(-p->proj_w[j], scr + ns - 1, p->proj_vec[j], y, n, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

extern "C" {

int su2g_heff_plan_add_projector(su2g_heff_plan* p, const double* o, double weight) {
  if (!p || (!o && p->work.psi.total > 0)) return fail(SU2G_EINVAL, "add_projector: bad arguments");
  const int ns = su2g::reduction_scratch_doubles();
  double* d = nullptr;
  SU2G_CUDA(dalloc(&d, (p->proj_vec.size() + 1) * ns * sizeof(double)));
  p->drop_graphs();  // captured Lanczos steps lack the new projector
  su2g::dev_free(p->d_proj, p->last_st);
  p->d_proj = d;
  p->proj_vec.push_back(o);
  p->proj_w.push_back(weight);
  return SU2G_OK;
}

}  // extern "C"

int su2g::cuda_status(cudaError_t e, const char* where) { return cuda_fail(e, where); }

int su2g::heff_apply_impl(su2g_heff_plan* p, const double* psi, double* y, cudaStream_t st) {
  const su2g::Bases b = make_bases(p, psi, y);
  if (p->S == 0) {
    SU2G_CUDA(su2g::launch_gemm_f64(p->d_tile1, (int)p->work.tile1.size(), p->d_seg1, b, st));
    SU2G_CUDA(su2g::launch_gemm_f64(p->d_tile2, (int)p->work.tile2.size(), p->d_seg2, b, st));
    SU2G_CUDA(su2g::apply_projectors(p, psi, y, st));
    return SU2G_OK;
  }
  const su2g::oz::OzWork& w = p->oz;
  // the row maxima that phase 1 leaves for the intermediates' pack start at zero
  if (w.rowmax_len > 0)
    SU2G_CUDA(cudaMemsetAsync(p->d_exps + w.rowmax_base, 0, w.rowmax_len * sizeof(int), st));
  SU2G_CUDA(su2g::oz::launch_pack(p->S, p->d_jobs[1], p->d_units[1], (int)w.units[1].size(), w.max_nkt[1], w.rows_pass[1], b, p->d_packed,
                                  p->d_exps, st));
  SU2G_CUDA(su2g::oz::launch_ozaki_gemm(p->S, p->d_otile1, (int)w.tile1.size(), p->d_oseg1, p->d_packed, p->d_exps, b,
                                        p->d_err, st));
  SU2G_CUDA(su2g::oz::launch_pack(p->S, p->d_jobs[2], p->d_units[2], (int)w.units[2].size(), w.max_nkt[2], w.rows_pass[2], b, p->d_packed,
                                  p->d_exps, st));
  SU2G_CUDA(su2g::oz::launch_ozaki_gemm(p->S, p->d_otile2, (int)w.tile2.size(), p->d_oseg2, p->d_packed, p->d_exps, b,
                                        p->d_err, st));
  SU2G_CUDA(su2g::oz::launch_reduce(p->d_red2, (int)w.red2.size(), b, st));
  SU2G_CUDA(su2g::apply_projectors(p, psi, y, st));
  return SU2G_OK;
}

extern "C" {

int su2g_heff_apply(su2g_heff_plan* p, const double* psi, double* y, void* stream) {
  if (!p) return fail(SU2G_EINVAL, "heff_apply: null plan");
  if (p->work.psi.total > 0 && (!psi || !y)) return fail(SU2G_EINVAL, "heff_apply: null vector");
  if (psi == y && psi) return fail(SU2G_EINVAL, "heff_apply: psi and y must not alias");
  p->last_st = (cudaStream_t)stream;
  return su2g::heff_apply_impl(p, psi, y, (cudaStream_t)stream);
}

int su2g_heff_apply_profile(su2g_heff_plan* p, const double* psi, double* y, void* stream, double* ms,
                            int* nlaunch) {
  if (!p || !ms || !nlaunch) return fail(SU2G_EINVAL, "apply_profile: bad arguments");
  if (psi == y && psi) return fail(SU2G_EINVAL, "apply_profile: psi and y must not alias");
  cudaStream_t st = (cudaStream_t)stream;
  p->last_st = st;
  const su2g::Bases b = make_bases(p, psi, y);
  cudaEvent_t ev[6];
  for (int i = 0; i < 6; ++i) SU2G_CUDA(cudaEventCreate(&ev[i]));
  cudaError_t e = cudaEventRecord(ev[0], st);
  int n = 0;
  if (p->S == 0) {
    if (e == cudaSuccess) e = su2g::launch_gemm_f64(p->d_tile1, (int)p->work.tile1.size(), p->d_seg1, b, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], st);
    if (e == cudaSuccess) e = su2g::launch_gemm_f64(p->d_tile2, (int)p->work.tile2.size(), p->d_seg2, b, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[2], st);
    n = 2;
  } else {
    const su2g::oz::OzWork& w = p->oz;
    if (e == cudaSuccess && w.rowmax_len > 0)
      e = cudaMemsetAsync(p->d_exps + w.rowmax_base, 0, w.rowmax_len * sizeof(int), st);
    if (e == cudaSuccess)
      e = su2g::oz::launch_pack(p->S, p->d_jobs[1], p->d_units[1], (int)w.units[1].size(), w.max_nkt[1], w.rows_pass[1], b, p->d_packed, p->d_exps,
                                st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], st);
    if (e == cudaSuccess)
      e = su2g::oz::launch_ozaki_gemm(p->S, p->d_otile1, (int)w.tile1.size(), p->d_oseg1, p->d_packed, p->d_exps, b,
                                      p->d_err, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[2], st);
    if (e == cudaSuccess)
      e = su2g::oz::launch_pack(p->S, p->d_jobs[2], p->d_units[2], (int)w.units[2].size(), w.max_nkt[2], w.rows_pass[2], b, p->d_packed, p->d_exps,
                                st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[3], st);
    if (e == cudaSuccess)
      e = su2g::oz::launch_ozaki_gemm(p->S, p->d_otile2, (int)w.tile2.size(), p->d_oseg2, p->d_packed, p->d_exps, b,
                                      p->d_err, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[4], st);
    if (e == cudaSuccess) e = su2g::oz::launch_reduce(p->d_red2, (int)w.red2.size(), b, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[5], st);
    n = 5;
  }
  if (e == cudaSuccess) e = cudaEventSynchronize(ev[n]);
  for (int i = 0; i < n && e == cudaSuccess; ++i) {
    float t = 0;
    e = cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
    ms[i] = t;
  }
  if (e == cudaSuccess && !p->proj_vec.empty()) {  // untimed: the projectors complete y
    e = su2g::apply_projectors(p, psi, y, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
  if (e != cudaSuccess) return cuda_fail(e, "apply_profile");
  *nlaunch = n;
  return SU2G_OK;
}

int su2g_heff_plan_destroy(su2g_heff_plan* p) {
  if (!p) return SU2G_OK;
  p->release();
  delete p;
  return SU2G_OK;
}

int su2g_hamiltonian_vector_multiplication(const int* vec_desc, const int* vec_flag, const double* vec,
                                           su2g_tensor op1, su2g_tensor op2, double* y, void* stream) {
  su2g_term term{op1, op2, 1.0};
  su2g_heff_plan* p = nullptr;
  int rc = su2g_heff_plan_create(vec_desc, vec_flag, 1, &term, nullptr, 0.0, nullptr, 0.0, SU2G_MODE_F64, &p);
  if (rc) return rc;
  rc = su2g_heff_apply(p, vec, y, stream);
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  su2g_heff_plan_destroy(p);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "hamiltonian_vector_multiplication");
  return SU2G_OK;
}

// ------------------------------------------------------------------ BLAS-1
int su2g_vec_dot(const double* x, const double* y, int64_t n, double* result, void* stream) {
  if (!result || n < 0) return fail(SU2G_EINVAL, "vec_dot: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  double* scratch = nullptr;
  const int ns = su2g::reduction_scratch_doubles();
  SU2G_CUDA(cudaMallocAsync((void**)&scratch, ns * sizeof(double), st));
  cudaError_t e = su2g::launch_dot(x, y, n, scratch, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(result, scratch + ns - 1, sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(scratch, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "vec_dot");
  return SU2G_OK;
}

int su2g_vec_axpy(double alpha, const double* x, double* y, int64_t n, void* stream) {
  if (n < 0) return fail(SU2G_EINVAL, "vec_axpy: bad arguments");
  SU2G_CUDA(su2g::launch_axpy(alpha, x, y, n, (cudaStream_t)stream));
  return SU2G_OK;
}

int su2g_vec_scale(double alpha, double* x, int64_t n, void* stream) {
  if (n < 0) return fail(SU2G_EINVAL, "vec_scale: bad arguments");
  SU2G_CUDA(su2g::launch_scale(alpha, x, n, (cudaStream_t)stream));
  return SU2G_OK;
}

// ----------------------------------------------------------------- Lanczos
namespace {

struct LanczosCtx {
  su2g_heff_plan* p;
  cudaStream_t st;
  int64_t n;
  int nmatvec = 0;
  double* ff(int i) { return p->d_krylov + (int64_t)i * n; }
  double* tmp() { return p->d_krylov + (int64_t)(p->krylov_vectors - 1) * n; }

  int dot(const double* x, const double* y, double* out) {
    const int ns = su2g::reduction_scratch_doubles();
    cudaError_t e = su2g::launch_dot(x, y, n, p->d_red, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, p->d_red + ns - 1, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "lanczos dot");
    return SU2G_OK;
  }
  int matvec(const double* x, double* y) {
    ++nmatvec;
    return su2g::heff_apply_impl(p, x, y, st);
  }
  int axpy(double a, const double* x, double* y) {
    cudaError_t e = su2g::launch_axpy(a, x, y, n, st);
    return e == cudaSuccess ? SU2G_OK : cuda_fail(e, "lanczos axpy");
  }
  int scale(double a, double* x) {
    cudaError_t e = su2g::launch_scale(a, x, n, st);
    return e == cudaSuccess ? SU2G_OK : cuda_fail(e, "lanczos scale");
  }
  int copy(const double* x, double* y) {
    cudaError_t e = cudaMemcpyAsync(y, x, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
    return e == cudaSuccess ? SU2G_OK : cuda_fail(e, "lanczos copy");
  }

  // ---- device-side coefficients: alpha[j], beta[j], q[j] (reorthogonalisation), nn ----
  int M() const { return p->lcoef_m; }
  double* alpha(int j) { return p->d_lcoef + j; }
  double* beta(int j) { return p->d_lcoef + M() + 1 + j; }
  double* q(int j) { return p->d_lcoef + 2 * (M() + 1) + j; }
  double* nnd() { return p->d_lcoef + 3 * (M() + 1); }

  // Enqueues the Lanczos step that produces ff[m] on stream s (lanczos_su2.cpp:136-142
  // for m = 1, :156-173 for m >= 2): matvec, alpha[m-1], the two three-term
  // updates, full reorthogonalisation against ff[0..m-1], beta[m] and the
  // normalisation -- the same kernels in the same order as the host-driven
  // sequence, with every scalar kept on the device.
  cudaError_t enqueue_step(int m, cudaStream_t s) {
    if (su2g::heff_apply_impl(p, ff(m - 1), ff(m), s) != SU2G_OK) return cudaErrorUnknown;
    cudaError_t e = su2g::launch_dot_to(ff(m - 1), ff(m), n, p->d_red, alpha(m - 1), s);
    if (e == cudaSuccess) e = su2g::launch_axpy_neg_dev(alpha(m - 1), ff(m - 1), ff(m), n, s);
    if (m >= 2) {
      if (e == cudaSuccess) e = su2g::launch_axpy_neg_dev(beta(m - 1), ff(m - 2), ff(m), n, s);
      for (int j = 0; j < m && e == cudaSuccess; ++j) {
        e = su2g::launch_dot_to(ff(m), ff(j), n, p->d_red, q(j), s);
        if (e == cudaSuccess) e = su2g::launch_axpy_neg_dev(q(j), ff(j), ff(m), n, s);
      }
    }
    if (e == cudaSuccess) e = su2g::launch_dot_to(ff(m), ff(m), n, p->d_red, nnd(), s);
    if (e == cudaSuccess) e = su2g::launch_normalize_dev(nnd(), ff(m), n, beta(m), s);
    return e;
  }
  // the final matvec and its alpha (lanczos_su2.cpp:189-194)
  cudaError_t enqueue_last(int m, cudaStream_t s) {
    if (su2g::heff_apply_impl(p, ff(m - 1), ff(m), s) != SU2G_OK) return cudaErrorUnknown;
    return su2g::launch_dot_to(ff(m - 1), ff(m), n, p->d_red, alpha(m - 1), s);
  }
  // runs a step as a CUDA graph, captured on first use
  int run_graph(bool last, int m) {
    std::vector<cudaGraphExec_t>& v = last ? p->lanc_last : p->lanc_step;
    if ((int)v.size() <= m) v.resize(m + 1, nullptr);
    if (!v[m]) {
      if (!p->cap_stream) SU2G_CUDA(cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking));
      SU2G_CUDA(cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal));
      const cudaError_t e = last ? enqueue_last(m, p->cap_stream) : enqueue_step(m, p->cap_stream);
      cudaGraph_t g = nullptr;
      const cudaError_t e2 = cudaStreamEndCapture(p->cap_stream, &g);
      if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(e != cudaSuccess ? e : e2, "lanczos graph capture");
      }
      const cudaError_t e3 = cudaGraphInstantiate(&v[m], g, 0);
      cudaGraphDestroy(g);
      if (e3 != cudaSuccess) {
        v[m] = nullptr;
        return cuda_fail(e3, "lanczos graph instantiate");
      }
    }
    ++nmatvec;
    SU2G_CUDA(cudaGraphLaunch(v[m], st));
    return SU2G_OK;
  }
  int fetch(const double* d, double* h, int count) {
    cudaError_t e = cudaMemcpyAsync(h, d, count * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? SU2G_OK : cuda_fail(e, "lanczos fetch");
  }
  // vout = sum_j z[j] ff[j]  (lanczos_su2::compute_eigenvector, lanczos_su2.cpp:262-279)
  int combine(const std::vector<double>& z, int m, double* vout) {
    int rc = copy(ff(0), vout);
    if (!rc) rc = scale(z[0], vout);
    for (int j = 1; j < m && !rc; ++j) rc = axpy(z[j], ff(j), vout);
    return rc;
  }
  // lanczos_su2::check_eigenvector (lanczos_su2.cpp:320-332): normalises v,
  // returns |Hv| and |<Hv,v>|/|Hv|
  int check(double* v, double* eig, double* olap) {
    double nn;
    int rc = dot(v, v, &nn);
    if (!rc) rc = scale(1.0 / std::sqrt(nn), v);
    if (!rc) rc = matvec(v, tmp());
    double pp = 0, ov = 0;
    if (!rc) rc = dot(tmp(), tmp(), &pp);
    if (!rc) rc = dot(tmp(), v, &ov);
    if (rc) return rc;
    const double prod = std::sqrt(pp);
    *eig = prod;
    *olap = std::fabs(ov / prod);
    return SU2G_OK;
  }
};

}  // namespace

int su2g_lanczos(su2g_heff_plan* p, double* psi, int mlanc, double* energy, int* nmatvec, void* stream) {
  if (!p || !psi || !energy || mlanc < 2) return fail(SU2G_EINVAL, "lanczos: bad arguments");
  const int64_t n = p->work.psi.total;
  if (n <= 0) return fail(SU2G_EINVAL, "lanczos: empty vector");
  if (mlanc > n) mlanc = (int)n + 1;  // dmrg_su2.cpp:532
  const int need = mlanc + 2;         // ff[0..mlanc] + one work vector
  if (p->krylov_vectors < need) {
    p->drop_graphs();  // captured with the old buffers
    su2g::dev_free(p->d_krylov, p->last_st);
    p->d_krylov = nullptr;
    p->krylov_vectors = 0;
    SU2G_CUDA(dalloc(&p->d_krylov, (size_t)need * n * sizeof(double)));
    p->krylov_vectors = need;
  }
  if (!p->d_red) SU2G_CUDA(dalloc(&p->d_red, su2g::reduction_scratch_doubles() * sizeof(double)));
  if (p->lcoef_m < mlanc) {
    p->drop_graphs();
    su2g::dev_free(p->d_lcoef, p->last_st);
    p->d_lcoef = nullptr;
    p->lcoef_m = 0;
    SU2G_CUDA(dalloc(&p->d_lcoef, (size_t)(3 * (mlanc + 1) + 1) * sizeof(double)));
    p->lcoef_m = mlanc;
  }
  p->last_st = (cudaStream_t)stream;
  LanczosCtx L{p, (cudaStream_t)stream, n};
  const double tol = 1.e-6;  // lanczos_su2.cpp:128
  std::vector<double> aal(mlanc, 0.0), nnl(mlanc + 1, 0.0), eig, z;
  int rc;
  // alpha[0..m-1] and beta[1..m] to the host (one copy each)
  auto fetch_coefs = [&](int m) -> int {
    int r = L.fetch(L.alpha(0), aal.data(), m);
    if (!r && m >= 1) r = L.fetch(L.beta(1), nnl.data() + 1, m);
    return r;
  };
  auto tridiag = [&](int m) {  // lanczos_su2::diatridiag (lanczos_su2.cpp:237-259)
    std::vector<double> d(aal.begin(), aal.begin() + m), e(m > 1 ? m - 1 : 0);
    for (int i = 0; i + 1 < m; ++i) e[i] = nnl[i + 1];
    su2g::tridiag_eigh(d, e, &eig, &z);
  };
  auto finish = [&](int m, bool do_check) -> int {
    std::vector<double> z0(z.begin(), z.begin() + m);  // ground-state column
    int r = L.combine(z0, m, psi);
    if (r) return r;
    if (do_check) {
      double ee, ov;
      r = L.check(psi, &ee, &ov);
      if (r) return r;
    }
    *energy = eig[0];
    if (nmatvec) *nmatvec = L.nmatvec;
    cudaError_t e = cudaStreamSynchronize(L.st);
    if (e != cudaSuccess) return cuda_fail(e, "lanczos");
    // a bounded wait of the split GEMM that gave up leaves partial products:
    // the result is refused, not returned
    int code = 0;
    return su2g_heff_plan_status(p, &code);
  };

  // ff[0] = normalised start vector (lanczos_su2.cpp:45-46)
  if ((rc = L.copy(psi, L.ff(0)))) return rc;
  SU2G_CUDA(su2g::launch_dot_to(L.ff(0), L.ff(0), n, p->d_red, L.nnd(), L.st));
  SU2G_CUDA(su2g::launch_normalize_dev(L.nnd(), L.ff(0), n, L.beta(0), L.st));
  // first step (lanczos_su2.cpp:136-142)
  if ((rc = L.run_graph(false, 1))) return rc;
  if (mlanc == 2) {  // lanczos_su2.cpp:143-154
    if ((rc = fetch_coefs(1))) return rc;
    if (nnl[1] < tol) {
      tridiag(1);
      return finish(1, false);
    }
    if ((rc = L.run_graph(true, 2))) return rc;
    if ((rc = fetch_coefs(2))) return rc;
    tridiag(2);
    return finish(2, false);
  }
  for (int m = 2; m < mlanc; ++m) {  // lanczos_su2.cpp:155-188
    if ((rc = L.run_graph(false, m))) return rc;
    if ((rc = fetch_coefs(m))) return rc;
    tridiag(m);
    if (nnl[m] < tol) return finish(m, true);
    if (m % 4 == 0) {
      std::vector<double> z0(z.begin(), z.begin() + m);
      if ((rc = L.combine(z0, m, psi))) return rc;
      double ee, ov;
      if ((rc = L.check(psi, &ee, &ov))) return rc;
      if (std::fabs(ov - 1.) < 1.e-8) {  // lanczos_su2.cpp:178-188
        *energy = eig[0];
        if (nmatvec) *nmatvec = L.nmatvec;
        SU2G_CUDA(cudaStreamSynchronize(L.st));
        int code = 0;
        return su2g_heff_plan_status(p, &code);
      }
    }
  }
  // final step (lanczos_su2.cpp:189-194)
  if ((rc = L.run_graph(true, mlanc))) return rc;
  if ((rc = fetch_coefs(mlanc))) return rc;
  tridiag(mlanc);
  return finish(mlanc, true);
}

}  // extern "C"
