/* Reference-side binding of libsu2g: the header a maintainer adds to the
 * SU2DMRG tree (next to tensor_su2.hpp) so that tensor_su2 objects reach the
 * C ABI of su2g.h.  It is compiled against the reference's own headers
 * (oracle/ref/build_ref.sh checks that it does); nothing in libsu2g includes
 * it.
 *
 *   Su2gView                 a tensor_su2 in the ABI's layout: host
 *                            descriptor and flags (tensor_su2.hpp:6-124,
 *                            su2struct.hpp:4-40) and a device copy of the
 *                            reduced blocks (tensor_su2::get_telement)
 *   su2g_set_result          writes a device result with a known structure
 *                            back into a tensor_su2 (set_tensor_su2 with that
 *                            structure's Clebsch-Gordan part)
 *   su2g_tensor_hamiltonian_vector_multiplication
 *                            the body of tensor_su2::hamiltonian_vector_
 *                            multiplication (tensor_su2_dmrg_src.cpp:893-1041)
 *   Su2gHeff                 the terms of one two-site step
 *                            (dmrg_su2::hamiltonian_vector_multiplication_idmrg,
 *                            dmrg_su2.cpp:543-664) as one device plan, and its
 *                            Lanczos solve in place of lanczos_su2::lanczos1
 *                            (lanczos_su2.cpp:125-195)
 *
 * Errors print the library's message and exit(0), as the reference does. */
#pragma once
#include <cuda_runtime.h>

#include <cstdlib>
#include <iostream>
#include <memory>
#include <vector>

#include "su2g.h"
#include "tensor_su2.hpp"

inline void su2g_check(int rc) {
  if (rc != SU2G_OK) {
    std::cout << "su2g error " << rc << ": " << su2g_last_error() << std::endl;
    std::exit(0);
  }
}

struct Su2gView {
  std::vector<int> desc, flag;
  double* dev = nullptr;  // the reduced blocks on the device (owned)
  int64_t len = 0;
  Su2gView() = default;
  Su2gView(const Su2gView&) = delete;
  Su2gView& operator=(const Su2gView&) = delete;
  ~Su2gView() {
    if (dev) cudaFree(dev);
  }
  su2g_tensor t() const { return su2g_tensor{desc.data(), flag.data(), dev}; }
};

// The ABI layout of t (desc: [nbond, locspin, {dir, n, 2j[n], dim[n]} per leg])
// and a device copy of its reduced blocks, queued on stream s.
inline void su2g_describe(tensor_su2& t, Su2gView& v, cudaStream_t s) {
  su2struct& c = t.get_cgc();
  v.desc = {c.get_nbond(), c.get_locspin()};
  for (int l = 0; l < c.get_nbond(); ++l) {
    v.desc.push_back(c.get_bonddir(l));
    v.desc.push_back(c.get_nmoment(l));
    for (int i = 0; i < c.get_nmoment(l); ++i) v.desc.push_back(c.get_angularmoment(l, i));
    for (int i = 0; i < c.get_nmoment(l); ++i) v.desc.push_back(c.get_bonddim(l, i));
  }
  int n1 = 0, n2 = 0;
  t.get_nelement(n1, n2);
  std::vector<double> red(n1 > 0 ? n1 : 1), cg(n2 > 0 ? n2 : 1);
  v.flag.assign(t.get_nten(), 0);
  t.get_telement(red.data(), cg.data(), v.flag.data());
  v.len = n1;
  if (cudaMalloc(&v.dev, sizeof(double) * (n1 > 0 ? n1 : 1)) != cudaSuccess) su2g_check(SU2G_ENOMEM);
  if (n1 > 0) cudaMemcpyAsync(v.dev, red.data(), sizeof(double) * n1, cudaMemcpyHostToDevice, s);
  cudaStreamSynchronize(s);  // red goes out of scope
}

// out = the device vector dev_y in the structure (and Clebsch-Gordan part) of like
inline void su2g_set_result(tensor_su2& out, tensor_su2& like, const double* dev_y, cudaStream_t s) {
  int n1 = 0, n2 = 0;
  like.get_nelement(n1, n2);
  std::vector<double> red(n1 > 0 ? n1 : 1), cg(n2 > 0 ? n2 : 1);
  std::vector<int> flag(like.get_nten(), 0);
  like.get_telement(red.data(), cg.data(), flag.data());
  if (n1 > 0) cudaMemcpyAsync(red.data(), dev_y, sizeof(double) * n1, cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  out.set_tensor_su2(like.get_cgc(), red.data(), cg.data(), flag.data());
}

// self = (op1, op2) vec, as tensor_su2::hamiltonian_vector_multiplication
inline void su2g_tensor_hamiltonian_vector_multiplication(tensor_su2& self, tensor_su2& vec, tensor_su2& op1,
                                                          tensor_su2& op2, cudaStream_t s = nullptr) {
  Su2gView v, a, b;
  su2g_describe(vec, v, s);
  su2g_describe(op1, a, s);
  su2g_describe(op2, b, s);
  double* y = nullptr;
  if (cudaMalloc(&y, sizeof(double) * (v.len > 0 ? v.len : 1)) != cudaSuccess) su2g_check(SU2G_ENOMEM);
  su2g_check(su2g_hamiltonian_vector_multiplication(v.desc.data(), v.flag.data(), v.dev, a.t(), b.t(), y, s));
  su2g_set_result(self, vec, y, s);
  cudaFree(y);
}

// The terms of one two-site step as one plan: add the (op1, op2, coef) pairs
// the engine's term loop visits (with the summed partner already formed, as
// dmrg_su2.cpp:585-600 does), the block Hamiltonians, the excited-state
// projectors; lanczos() solves with them and writes the eigenvector into vec.
class Su2gHeff {
 public:
  explicit Su2gHeff(int mode = SU2G_MODE_SPLIT_BF16, cudaStream_t s = nullptr) : mode_(mode), s_(s) {}
  ~Su2gHeff() {
    if (plan_) su2g_heff_plan_destroy(plan_);
  }
  void add_term(tensor_su2& op1, tensor_su2& op2, double coef) {
    Su2gView* a = view(op1);
    Su2gView* b = view(op2);
    pairs_.push_back({a, b, coef});
  }
  void set_blocks(tensor_su2* hl, tensor_su2* hr) {
    hl_ = hl ? view(*hl) : nullptr;
    hr_ = hr ? view(*hr) : nullptr;
  }
  void add_projector(tensor_su2& o, double weight) { proj_.push_back({view(o), weight}); }
  // lanczos_su2::lanczos1 from vec; vec receives the eigenvector; returns the eigenvalue
  double lanczos(tensor_su2& vec, int mlanc = 5, int* nmatvec = nullptr) {
    Su2gView* v = view(vec);
    std::vector<su2g_term> terms;
    for (const Pair& p : pairs_) terms.push_back(su2g_term{p.a->t(), p.b->t(), p.coef});
    su2g_tensor hl = hl_ ? hl_->t() : su2g_tensor{}, hr = hr_ ? hr_->t() : su2g_tensor{};
    su2g_check(su2g_heff_plan_create(v->desc.data(), v->flag.data(), (int)terms.size(), terms.data(),
                                     hl_ ? &hl : nullptr, 1.0, hr_ ? &hr : nullptr, 1.0, mode_, &plan_));
    for (const Proj& p : proj_) su2g_check(su2g_heff_plan_add_projector(plan_, p.o->dev, p.w));
    double e = 0.0;
    int nmv = 0;
    su2g_check(su2g_lanczos(plan_, v->dev, mlanc, &e, &nmv, s_));
    if (nmatvec) *nmatvec = nmv;
    su2g_set_result(vec, vec, v->dev, s_);
    return e;
  }

 private:
  struct Pair {
    Su2gView* a;
    Su2gView* b;
    double coef;
  };
  struct Proj {
    Su2gView* o;
    double w;
  };
  Su2gView* view(tensor_su2& t) {
    views_.emplace_back(new Su2gView());
    su2g_describe(t, *views_.back(), s_);
    return views_.back().get();
  }
  int mode_;
  cudaStream_t s_;
  su2g_heff_plan* plan_ = nullptr;
  std::vector<std::unique_ptr<Su2gView>> views_;
  std::vector<Pair> pairs_;
  std::vector<Proj> proj_;
  Su2gView* hl_ = nullptr;
  Su2gView* hr_ = nullptr;
};
