// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// A C entry layer over the reference's own objects, linked into
// oracle/_ref/libsu2ref.so by build_ref.sh.  It exists to produce golden
// fixtures (tests/golden/gen_golden.py) from the reference itself:
//   * the recoupling table fac_hamilt_vec (dmrg_su2.cpp:759-775),
//   * tensor_su2::hamiltonian_vector_multiplication on given block tensors
//     (tensor_su2_dmrg_src.cpp:893-1041),
//   * tensor_su2::contract for the spin-0 block-Hamiltonian terms
//     (tensor_su2.cpp:1255-1345, used at dmrg_su2.cpp:563-570),
//   * whole DMRG runs (do_idmrg + sweep, as main_omp.cpp:158-202 drives them).
// Block tensors cross this boundary in the reference's own checkpoint layout
// (dmrg_su2_omp.cpp:864-941): a presence flag per block, then the reduced
// blocks in mixed-radix block order (leg 0 fastest), each column-major.
// The structure travels as an int "desc":
//   [nbond, locspin, {dir, n, angm[0..n), dim[0..n)} per leg].
#include <omp.h>
#include <mkl.h>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <algorithm>
#include <vector>
#include <unistd.h>
#define private public
#include "dmrg_su2_omp.hpp"
#undef private

// Globals that main_omp.cpp:15-24 defines (main_omp.o is not linked here).
int max_dcut = 8000, myrank = 0, myrk, psize = 12, mkl = 1, comm_rank = 0, comm_size, thread,
    bdry = 2, jobid, memory_flag = 0;
double delta = 0, qdelta = 1, alpha, tau;
double t1, t2, preparetime = 0, svdtime = 0, lanczostime = 0;
dmrg_su2* chain_ptr;
tensor ***spin_op, ***cgc_coef_left, ***cgc_coef_rght, *cgc_coef_singlet, *identity;
double **spin_op_trace, *****fac_operator_onsite_left, *****fac_operator_onsite_rght,
    ******fac_operator_transformation_left, ******fac_operator_transformation_rght,
    *****fac_operator_pairup_left, *****fac_operator_pairup_rght, ***fac_hamilt_vec,
    *****fac_permutation_left, *****fac_permutation_rght, *fac_betadouble, *fac_comp_left,
    *fac_comp_rght, *fac_init_left, *fac_init_rght;
double cosk, coskminus;
double pi = M_PI;
double pi2 = pi * 2;
int nkrylov = 0, disk = 0;

namespace {
dmrg_su2* g_tables = nullptr;  // owner of the recoupling tables
tensor_su2 g_result;           // last result, read back by ref_result_*
tensor_su2 g_result_b;         // second result (tv of ref_svd)
tensor_su2* g_sel = &g_result;
tensor_su2 g_vec1, g_vec2;             // ref_idmrg_capture: psi and H_eff psi
std::vector<tensor_su2*> g_export;     // tensors exported by ref_idmrg_capture
std::vector<int> g_term_i;             // its term list (see ref_idmrg_capture)
std::vector<double> g_term_d;

void desc_to_struct(const int* desc, su2struct& s) {
  int nb = desc[0], locspin = desc[1], p = 2;
  std::vector<su2bond> bb(nb);
  for (int l = 0; l < nb; ++l) {
    int dir = desc[p], n = desc[p + 1];
    std::vector<int> ang(desc + p + 2, desc + p + 2 + n), dim(desc + p + 2 + n, desc + p + 2 + 2 * n);
    bb[l].set_su2bond(n, dir, ang.data(), dim.data());
    p += 2 + 2 * n;
  }
  s.set_su2struct(nb, locspin, bb.data());
}

// Builds a tensor_su2 from reduced blocks; the CG part of every block is the
// canonical one the engine uses: make_cgc(a0,a1,a2) for 3-leg tensors, the
// singlet for 2-leg vectors (dirs -1,-1), the identity for 2-leg scalar
// operators (dirs +1,-1).
void build_tensor(tensor_su2& t, const int* desc, const int* flag, const double* data) {
  su2struct s;
  desc_to_struct(desc, s);
  int nb = s.get_nbond(), nten = s.get_nten();
  std::vector<int> angm(nb), bdim(nb), cdim(nb);
  std::vector<double> cg;
  for (int i = 0; i < nten; ++i) {
    if (!flag[i]) continue;
    s.get_tensor_argument(i, angm.data(), bdim.data(), cdim.data());
    tensor c;
    if (nb == 3) c.make_cgc(angm[0], angm[1], angm[2]);
    else if (s.get_bonddir(0) == 1) c.make_identity(angm[0]);
    else c.make_singlet(angm[0]);
    for (int e = 0; e < c.get_nelement(); ++e) cg.push_back(c.get_telement(e));
  }
  std::vector<int> f(flag, flag + nten);
  t.set_tensor_su2(s, const_cast<double*>(data), cg.data(), f.data());
}
}  // namespace

extern "C" {

// Recoupling tables for 2j < max_angm, built exactly as the engine builds them.
int ref_setup(int nthreads, int max_angm) {
  psize = nthreads;
  omp_set_num_threads(nthreads);
  mkl_set_num_threads(1);
  if (!g_tables) {
    g_tables = new dmrg_su2();
    g_tables->physpn = 1;
    g_tables->makeup_clebsch_gordan_coefficient_tensors(max_angm);
  }
  return 0;
}

void ref_fac_hamilt_vec(int max_angm, double* out) {
  for (int i = 0; i < max_angm; ++i)
    for (int j = 0; j < max_angm; ++j)
      for (int k = 0; k < max_angm; ++k) out[(i * max_angm + j) * max_angm + k] = fac_hamilt_vec[i][j][k];
}

void ref_make_cgc(int j1, int j2, int j3, double* out) {
  tensor c;
  c.make_cgc(j1, j2, j3);
  for (int e = 0; e < c.get_nelement(); ++e) out[e] = c.get_telement(e);
}

void ref_make_singlet(int j, double* out) {
  tensor c;
  c.make_singlet(j);
  for (int e = 0; e < c.get_nelement(); ++e) out[e] = c.get_telement(e);
}

// result = hamiltonian_vector_multiplication(vec, op1, op2)
int ref_heff_term(const int* vd, const int* vf, const double* vx, const int* d1, const int* f1,
                  const double* x1, const int* d2, const int* f2, const double* x2) {
  tensor_su2 vec, op1, op2;
  build_tensor(vec, vd, vf, vx);
  build_tensor(op1, d1, f1, x1);
  build_tensor(op2, d2, f2, x2);
  g_result.hamiltonian_vector_multiplication(vec, op1, op2);
  return g_result.get_nten();
}

// result = contract(t1, i1, t2, i2)
int ref_contract(const int* da, const int* fa, const double* xa, int ia, const int* db, const int* fb,
                 const double* xb, int ib) {
  tensor_su2 a, b;
  build_tensor(a, da, fa, xa);
  build_tensor(b, db, fb, xb);
  g_result.contract(a, ia, b, ib);
  return g_result.get_nten();
}

void ref_result_sizes(int* nten, int* nele1, int* nele2) {
  *nten = g_sel->get_nten();
  g_sel->get_nelement(*nele1, *nele2);
}

void ref_result_get(int* flag, double* tele1, double* tele2) { g_sel->get_telement(tele1, tele2, flag); }

// result = operator_transformation(uu, vv, op, flag)  (tensor_su2_dmrg_src.cpp:221-402)
int ref_operator_transformation(const int* du, const int* fu, const double* xu, const int* dv, const int* fv,
                                const double* xv, const int* dop, const int* fop, const double* xop, int flag) {
  tensor_su2 uu, vv, op;
  build_tensor(uu, du, fu, xu);
  build_tensor(vv, dv, fv, xv);
  build_tensor(op, dop, fop, xop);
  g_result.operator_transformation(uu, vv, op, flag);
  return g_result.get_nten();
}

// result = overlap_transformation(uu, vv, op, flag)  (tensor_su2_dmrg_src.cpp:531-688)
int ref_overlap_transformation(const int* du, const int* fu, const double* xu, const int* dv, const int* fv,
                               const double* xv, const int* dop, const int* fop, const double* xop, int flag) {
  tensor_su2 uu, vv, op;
  build_tensor(uu, du, fu, xu);
  build_tensor(vv, dv, fv, xv);
  build_tensor(op, dop, fop, xop);
  g_result.overlap_transformation(uu, vv, op, flag);
  return g_result.get_nten();
}

// The engine's own site operators (dmrg_su2::initialize_local_operators,
// dmrg_su2.cpp:427-525): kind 0 = sigma[idx], 1 = qterm[idx], 2 = ring[idx].
static tensor_su2* site_operator(int kind, int idx) {
  static bool ready = false;
  if (!ready) {
    g_tables->initialize_local_operators();
    ready = true;
  }
  return kind == 0 ? &g_tables->sigma[idx] : kind == 1 ? &g_tables->qterm[idx] : &g_tables->ring[idx];
}

// Selects a site operator as the tensor ref_result_* read.
void ref_select_site(int kind, int idx) { g_sel = site_operator(kind, idx); }

// result = operator_initial(uu, vv, site op, flag)  (tensor_su2_dmrg_src.cpp:27-204)
// or, with an endt desc, operator_initial(uu, vv, site op, endt, flag) (:207-218)
int ref_operator_initial(const int* du, const int* fu, const double* xu, const int* dv, const int* fv,
                         const double* xv, int skind, int sidx, const int* de, const int* fe, const double* xe,
                         int flag) {
  tensor_su2 uu, vv, endt;
  build_tensor(uu, du, fu, xu);
  build_tensor(vv, dv, fv, xv);
  if (de) {
    build_tensor(endt, de, fe, xe);
    g_result.operator_initial(uu, vv, *site_operator(skind, sidx), endt, flag);
  } else {
    g_result.operator_initial(uu, vv, *site_operator(skind, sidx), flag);
  }
  g_sel = &g_result;
  return g_result.get_nten();
}

// result = operator_pairup(uu, vv, op1, site op, flag)  (tensor_su2_dmrg_src.cpp:691-890)
int ref_operator_pairup(const int* du, const int* fu, const double* xu, const int* dv, const int* fv,
                        const double* xv, const int* d1, const int* f1, const double* x1, int skind, int sidx,
                        int flag) {
  tensor_su2 uu, vv, op1;
  build_tensor(uu, du, fu, xu);
  build_tensor(vv, dv, fv, xv);
  build_tensor(op1, d1, f1, x1);
  g_result.operator_pairup(uu, vv, op1, *site_operator(skind, sidx), flag);
  g_sel = &g_result;
  return g_result.get_nten();
}

// result = permutation(uu, vv, vec, site op 1, site op 2, flag)
// (tensor_su2_hamiltonian.cpp:871-1108)
int ref_permutation(const int* du, const int* fu, const double* xu, const int* dv, const int* fv,
                    const double* xv, const int* dvec, const int* fvec, const double* xvec, int k1, int i1, int k2,
                    int i2, int flag) {
  tensor_su2 uu, vv, vec;
  build_tensor(uu, du, fu, xu);
  build_tensor(vv, dv, fv, xv);
  build_tensor(vec, dvec, fvec, xvec);
  g_result.permutation(uu, vv, vec, *site_operator(k1, i1), *site_operator(k2, i2), flag);
  g_sel = &g_result;
  return g_result.get_nten();
}

// fac_operator_onsite_{left,rght}[j][m][l][i][q], fac_operator_pairup_{left,rght}[j][i][k][m][q]
// (q = p0 + p1 * physpn2) and fac_permutation_{left,rght}[i][j][k][l][t] (dmrg_su2.cpp:776-1019)
double ref_fac_table(int table, int side, int a, int b, int c, int d, int e) {
  if (table == 0) return side == 0 ? fac_operator_onsite_left[a][b][c][d][e] : fac_operator_onsite_rght[a][b][c][d][e];
  if (table == 1) return side == 0 ? fac_operator_pairup_left[a][b][c][d][e] : fac_operator_pairup_rght[a][b][c][d][e];
  return side == 0 ? fac_permutation_left[a][b][c][d][e] : fac_permutation_rght[a][b][c][d][e];
}


// Runs do_idmrg + niter sweeps (as ref_run_dmrg), then at the last two-site
// step (il, ir) = (ns/2 - 1, ns/2) forms the engine's own input vector
// (prepare_input_vector, dmrg_su2_omp.cpp:229-254) and applies the engine's
// own hamiltonian_vector_multiplication_idmrg (dmrg_su2.cpp:543-664) to it.
// Exported tensors (ref_idmrg_select): 0 = psi, 1 = H_eff psi, 2 = hh[il],
// 3 = hh[ir], then the operators the terms name.  The term list mirrors the
// loops of hamiltonian_vector_multiplication_idmrg:
//   ints  = [nterms, per term: nl, l_idx..., nr, r_idx...]
//   dbls  = [per term: coef, l_coef..., r_coef...]
// each term being coef * hvm(psi, sum_l l_coef L_l, sum_r r_coef R_r).
// Returns the number of exported tensors.
int ref_idmrg_capture(int lx, int ly, int sec, int d, int niter, double jcoup, double qcoup, int boundary,
                      int nthreads, double* energies) {
  max_dcut = d;
  bdry = boundary;
  delta = jcoup;
  qdelta = qcoup;
  memory_flag = 0;
  psize = nthreads;
  omp_set_num_threads(nthreads);
  mkl_set_num_threads(1);
  omp_set_nested(1);
  omp_set_max_active_levels(2);
  if (ly > 1) {
    cosk = cos(0.0);
    coskminus = cosk;
  }
  dmrg_su2* c = new dmrg_su2(lx, ly, sec, 0, 0, 0);
  chain_ptr = c;
  c->set_ky(0);
  // the step eigenvalues the engine prints (dmrg_su2.cpp:539), in full
  std::streamsize prec = std::cout.precision(17);
  c->do_idmrg();
  std::cout.precision(prec);
  energies[0] = c->get_enr();
  for (int i = 0; i < niter; ++i) {
    c->sweep();
    energies[i + 1] = c->get_enr();
  }
  const int ns = c->ns, il = ns / 2 - 1, ir = ns / 2;
  c->prepare_input_vector(il, ir, g_vec1);
  c->hamiltonian_vector_multiplication_idmrg(il, ir, g_vec1, g_vec2);
  g_export = {&g_vec1, &g_vec2, &c->hh[il], &c->hh[ir]};
  g_term_i.assign(1, 0);
  g_term_d.clear();
  auto idx = [&](tensor_su2* t) {
    for (size_t q = 0; q < g_export.size(); ++q)
      if (g_export[q] == t) return (int)q;
    g_export.push_back(t);
    return (int)g_export.size() - 1;
  };
  auto term = [&](const std::vector<std::pair<tensor_su2*, double>>& l,
                  const std::vector<std::pair<tensor_su2*, double>>& r, double coef) {
    g_term_i[0]++;
    g_term_d.push_back(coef);
    g_term_i.push_back((int)l.size());
    for (auto& e : l) {
      g_term_i.push_back(idx(e.first));
      g_term_d.push_back(e.second);
    }
    g_term_i.push_back((int)r.size());
    for (auto& e : r) {
      g_term_i.push_back(idx(e.first));
      g_term_d.push_back(e.second);
    }
  };
  if (il < ns / 2) {
    for (int j = 0; j <= il; ++j) {
      std::vector<std::pair<tensor_su2*, double>> r;
      for (int k = ir; k < ns; ++k)
        if (c->hmap[j][k] > 0) r.push_back({&c->opr[ir][k], c->coup[c->hmap[j][k]]});
      if (!r.empty()) term({{&c->opr[il][j], 1.0}}, r, 1.0);
    }
  } else {
    for (int k = ir; k < ns; ++k) {
      std::vector<std::pair<tensor_su2*, double>> l;
      for (int j = 0; j <= il; ++j)
        if (c->hmap[j][k] > 0) l.push_back({&c->opr[il][j], c->coup[c->hmap[j][k]]});
      if (!l.empty()) term(l, {{&c->opr[ir][k], 1.0}}, 1.0);
    }
  }
  for (int m = 0; m < 2 * ns; ++m) {
    const int j = m % ns;
    if (il != ir - 1 || c->plqflg[il][j] != 1 || c->plqflg[ir][j] != 1) continue;
    const int* q = c->plqpos[j];
    if (il >= q[0] && ir <= q[1]) term({{&c->opr[il][q[0]], 1.0}}, {{&c->plqopr[ir][m], 1.0}}, -qdelta);
    else if (il >= q[1] && ir <= q[2]) term({{&c->plqopr[il][m], 1.0}}, {{&c->plqopr[ir][m], 1.0}}, -qdelta);
    else if (il >= q[2] && ir <= q[3]) term({{&c->plqopr[il][m], 1.0}}, {{&c->opr[ir][q[3]], 1.0}}, -qdelta);
  }
  return (int)g_export.size();
}

void ref_idmrg_select(int i) { g_sel = g_export[i]; }
int ref_idmrg_terms(int* ints, int ncap_i, double* dbls, int ncap_d) {
  if ((int)g_term_i.size() > ncap_i || (int)g_term_d.size() > ncap_d) return -1;
  std::copy(g_term_i.begin(), g_term_i.end(), ints);
  std::copy(g_term_d.begin(), g_term_d.end(), dbls);
  return (int)g_term_i.size();
}

// The initial two-site vector of a step from the MPS tensors uu[il] (ul) and
// uu[ir] (ur): the sequence of dmrg_su2::prepare_input_vector
// (dmrg_su2_omp.cpp:229-245) on the reference's own objects.
int ref_prepare_input_vector(const int* dl, const int* fl, const double* xl, const int* dr, const int* fr,
                             const double* xr) {
  tensor_su2 ul, ur, tmp1, tmp2, left, rght;
  build_tensor(ul, dl, fl, xl);
  build_tensor(ur, dr, fr, xr);
  su2bond bb[4];
  ul.get_su2bond(0, bb[0]);
  ul.get_su2bond(1, bb[1]);
  ur.get_su2bond(0, bb[2]);
  ur.get_su2bond(1, bb[3]);
  tmp1.fuse(bb[0], bb[1]);
  tmp2.fuse(bb[2], bb[3]);
  left.overlap_initial(ul, tmp1, 0);
  rght.overlap_initial(ur, tmp2, 1);
  rght.take_conjugate(0);
  g_result.contract(left, 0, rght, 0);
  g_result.makeup_input_vector();
  g_sel = &g_result;
  return g_result.get_nten();
}

// uu.right2left_vectran() (dir 0) / uu.left2right_vectran() (dir 1), the
// step of dmrg_su2::wavefunc_transformation (dmrg_su2_omp.cpp:1864-1877)
// The warm-up's initial two-site vector (dmrg_su2_omp.cpp:196-216 and
// do_idmrg :79-80): prepare_input_vector_initial's fuse / overlap_initial /
// fuse_to_singlet / contract sequence on ul = uu[il], ur = uu[ir], then
// initialize_input_vector and normalize_vector; the result is g_result.
int ref_input_vector_initial(const int* dl, const int* fl, const double* xl, const int* dr, const int* fr,
                             const double* xr) {
  tensor_su2 ul, ur, tmp1, tmp2, left, rght, tmp, tmp3;
  build_tensor(ul, dl, fl, xl);
  build_tensor(ur, dr, fr, xr);
  su2bond bb[4];
  ul.get_su2bond(0, bb[0]);
  ul.get_su2bond(1, bb[1]);
  ur.get_su2bond(0, bb[2]);
  ur.get_su2bond(1, bb[3]);
  tmp1.fuse(bb[0], bb[1]);
  tmp2.fuse(bb[2], bb[3]);
  left.overlap_initial(ul, tmp1, 0);
  rght.overlap_initial(ur, tmp2, 1);
  left.get_su2bond(0, bb[0]);
  rght.get_su2bond(0, bb[1]);
  bb[0].invert_bonddir();
  bb[1].invert_bonddir();
  tmp.fuse_to_singlet(bb[0], bb[1]);
  tmp3.contract(left, 0, tmp, 0);
  g_result.contract(tmp3, 1, rght, 0);
  g_result.makeup_input_vector();
  g_result.initialize_input_vector();
  g_result.normalize_vector();
  g_sel = &g_result;
  return 0;
}

// tensor_su2::fuse(b1, b2) (tensor_su2.cpp:839-909) of the two legs of a
// 2-leg desc; the result is g_result.
int ref_fuse_tensor(const int* bonds_desc) {
  su2struct s;
  desc_to_struct(bonds_desc, s);
  su2bond b1, b2;
  s.get_su2bond(0, b1);
  s.get_su2bond(1, b2);
  g_result.fuse(b1, b2);
  g_sel = &g_result;
  return 0;
}

int ref_vectran(const int* du, const int* fu, const double* xu, int dir) {
  build_tensor(g_result, du, fu, xu);
  if (dir == 0) g_result.right2left_vectran();
  else g_result.left2right_vectran();
  g_sel = &g_result;
  return g_result.get_nten();
}

// fac_operator_transformation_{left,rght}[j][m][l][i][k][p] (dmrg_su2.cpp:857-890)
double ref_fac_operator_transformation(int side, int j, int m, int l, int i, int k, int p) {
  return side == 0 ? fac_operator_transformation_left[j][m][l][i][k][p]
                   : fac_operator_transformation_rght[j][m][l][i][k][p];
}

// vec.svd(tu, p1, tv, p2, wout) (tensor_su2.cpp:1619-1758) with the global
// max_dcut; returns dout (entries of wout); kept[] receives the new bond's
// multiplet counts per 2j in 0..63 (tu leg 2 after the call).
int ref_svd(const int* dvec, const int* fvec, const double* xvec, const int* du, const int* fu, const double* xu,
            const int* dv, const int* fv, const double* xv, double p1, double p2, int dcut, double* wout,
            int* kept) {
  // tu, tv end up in g_result, g_result_b (tensor_su2 has no copy assignment)
  tensor_su2 vec;
  tensor_su2& tu = g_result;
  tensor_su2& tv = g_result_b;
  build_tensor(vec, dvec, fvec, xvec);
  build_tensor(tu, du, fu, xu);
  build_tensor(tv, dv, fv, xv);
  max_dcut = dcut;
  int dout = 0;
  vec.svd(tu, p1, tv, p2, dout, wout);
  for (int i = 0; i < 64; ++i) kept[i] = 0;
  for (int i = 0; i < tu.get_nmoment(2); ++i) kept[tu.get_angularmoment(2, i)] = tu.get_bonddim(2, i);
  return dout;
}

// Selects which result ref_result_* read: 0 = the last result (tu after
// ref_svd), 1 = tv after ref_svd.
void ref_select_result(int which) { g_sel = which ? &g_result_b : &g_result; }

// desc of the selected result; returns its length
int ref_result_desc(int* out) {
  su2struct& c = g_sel->get_cgc();
  int p = 0;
  out[p++] = c.get_nbond();
  out[p++] = c.get_locspin();
  for (int l = 0; l < c.get_nbond(); ++l) {
    out[p++] = c.get_bonddir(l);
    out[p++] = c.get_nmoment(l);
    for (int i = 0; i < c.get_nmoment(l); ++i) out[p++] = c.get_angularmoment(l, i);
    for (int i = 0; i < c.get_nmoment(l); ++i) out[p++] = c.get_bonddim(l, i);
  }
  return p;
}

// su2bond::fuse (su2bond.cpp:155-210); returns the sector count
int ref_fuse(int n1, const int* a1, const int* d1, int n2, const int* a2, const int* d2, int* aout, int* dout) {
  std::vector<int> x1(a1, a1 + n1), y1(d1, d1 + n1), x2(a2, a2 + n2), y2(d2, d2 + n2);
  su2bond b1, b2, f;
  b1.set_su2bond(n1, 1, x1.data(), y1.data());
  b2.set_su2bond(n2, 1, x2.data(), y2.data());
  f.fuse(b1, b2);
  for (int i = 0; i < f.get_nmoment(); ++i) {
    aout[i] = f.get_angularmoment(i);
    dout[i] = f.get_bonddim(i);
  }
  return f.get_nmoment();
}

// su2struct::get_tensor_argument legality of every block
int ref_legal(const int* desc, int* legal) {
  su2struct s;
  desc_to_struct(desc, s);
  int nb = s.get_nbond();
  std::vector<int> angm(nb), bdim(nb), cdim(nb);
  for (int i = 0; i < s.get_nten(); ++i) legal[i] = s.get_tensor_argument(i, angm.data(), bdim.data(), cdim.data());
  return s.get_nten();
}

// Runs the reference DMRG the way main_omp.cpp:158-202 does (without its
// scratch-directory creation) and returns the per-sweep energies E0-1000.
// Must be called from a scratch working directory: the engine writes its
// checkpoint files (uu-*, ww-*, enr-*) into the current directory.
// Checkpoint files written by the engine itself in directory `dir`: do_idmrg
// and niter sweeps (as ref_run_dmrg), then save_mps2 (every site, memory_flag
// 0; dmrg_su2_omp.cpp:864-941), save_enr (:1070-1097) and save_ww
// (:1154-1186).  uu[0..ns) are exported for ref_idmrg_select; *enr gets
// gs_enr[0] as written.  Returns ns, or -1 if `dir` cannot be entered.
int ref_checkpoint_write(int lx, int ly, int sec, int d, int niter, double jcoup, double qcoup, int boundary,
                         int nthreads, const char* dir, double* enr) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof cwd) || chdir(dir) != 0) return -1;
  max_dcut = d;
  bdry = boundary;
  delta = jcoup;
  qdelta = qcoup;
  memory_flag = 0;
  psize = nthreads;
  omp_set_num_threads(nthreads);
  mkl_set_num_threads(1);
  omp_set_nested(1);
  omp_set_max_active_levels(2);
  if (ly > 1) {
    cosk = cos(0.0);
    coskminus = cosk;
  }
  dmrg_su2* c = new dmrg_su2(lx, ly, sec, 0, 0, 0);
  chain_ptr = c;
  c->set_ky(0);
  // the step eigenvalues the engine prints (dmrg_su2.cpp:539), in full
  std::streamsize prec = std::cout.precision(17);
  c->do_idmrg();
  std::cout.precision(prec);
  for (int i = 0; i < niter; ++i) c->sweep();
  c->save_mps2();
  c->save_enr();
  c->save_ww();
  *enr = c->gs_enr[0];
  g_export.clear();
  for (int i = 0; i < c->ns; ++i) g_export.push_back(&c->uu[i]);
  const int ns = c->ns;
  if (chdir(cwd) != 0) return -1;
  return ns;
}

// The same files read back by the engine (read_mps, read_enr, read_ww with
// read1 = d, read2 = 0: dmrg_su2_omp.cpp:944-1151, 1188-1242) into a fresh
// engine of the same lattice.  uu[0..ns) are exported; *enr = gs_enr[0] after
// read_enr; ww[0][0..d) copied to ww_out (cap >= d).  Returns ns, -1 if `dir`
// cannot be entered, -2 if read_mps reports a missing file.
int ref_checkpoint_read(int lx, int ly, int sec, int d, const char* dir, double* enr, double* ww_out, int ww_cap) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof cwd) || chdir(dir) != 0) return -1;
  max_dcut = d;
  memory_flag = 0;
  dmrg_su2* c = new dmrg_su2(lx, ly, sec, 0, 0, 0);
  chain_ptr = c;
  c->set_ky(0);
  const bool ok = c->read_mps(d, 0);
  c->read_enr(d, 0);
  c->read_ww(d, 0);
  *enr = c->gs_enr[0];
  for (int i = 0; i < d && i < ww_cap; ++i) ww_out[i] = c->ww[0][i];
  g_export.clear();
  for (int i = 0; i < c->ns; ++i) g_export.push_back(&c->uu[i]);
  const int ns = c->ns;
  if (chdir(cwd) != 0) return -1;
  return ok ? ns : -2;
}

#ifdef SU2REF_MEA
// Built only into libsu2ref_mea.so, where the measurement variant of the
// engine (dmrg_su2_omp_mea_enr.cpp) replaces dmrg_su2_omp.cpp.
//
// The centre-bond energy of that variant on the checkpoint files in `dir`:
//   engine 1 runs what its driver runs (main_omp.cpp:164-170: read_mps,
//   read_enr, read_ww, then prepare_sweep, which ends in mea_enr,
//   dmrg_su2_omp_mea_enr.cpp:160-242); parts[4] = its gs_enr[0];
//   engine 2 builds the same environments (prepare_sweep's end tensors and
//   site-operator loop, :165-186) without calling mea_enr, so that hh[ns/2]
//   is not yet scaled, and exports hh[ns/2-1], hh[ns/2] and the operators of
//   mea_enr's pair list (ref_idmrg_select), the pairs as ints = [npairs,
//   left_idx, right_idx, ...], dbls = [coef, ...] in mea_enr's loop order
//   (where none of its plaquette cases applies, mea_enr reuses the previous
//   product, and so does the list).  parts[0..3] = tr hh[ns/2-1], tr of
//   hh[ns/2] scaled by ww on both legs, the pair sum, sum ww^2, from the
//   engine's own tensor_su2 members on engine 2's tensors; ww[0..d) to
//   ww_out.  Returns the number of exported tensors, < 0 on failure.
int ref_mea_enr(int lx, int ly, int sec, int d, double jcoup, double qcoup, int boundary, int nthreads,
                const char* dir, double* parts, double* ww_out, int ww_cap) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof cwd) || chdir(dir) != 0) return -1;
  max_dcut = d;
  bdry = boundary;
  delta = jcoup;
  qdelta = qcoup;
  memory_flag = 0;
  psize = nthreads;
  omp_set_num_threads(nthreads);
  mkl_set_num_threads(1);
  omp_set_nested(1);
  omp_set_max_active_levels(2);
  if (ly > 1) {
    cosk = cos(0.0);
    coskminus = cosk;
  }
  dmrg_su2* e1 = new dmrg_su2(lx, ly, sec, d, 0, 0);
  chain_ptr = e1;
  e1->set_ky(0);
  bool ok = e1->read_mps(d, 0);
  e1->read_enr(d, 0);
  e1->read_ww(d, 0);
  if (ok) e1->prepare_sweep();
  parts[4] = e1->gs_enr[0];
  dmrg_su2* c = new dmrg_su2(lx, ly, sec, d, 0, 0);
  chain_ptr = c;
  c->set_ky(0);
  ok = ok && c->read_mps(d, 0);
  c->read_ww(d, 0);
  if (chdir(cwd) != 0 || !ok) return -2;
  const int ns = c->ns;
  su2bond bb[4];
  int a = 0, one = 1;
  bb[0].set_su2bond(1, 1, &a, &one);
  a = c->physpn;
  bb[1].set_su2bond(1, 1, &a, &one);
  c->uu[0].fuse(bb[0], bb[1]);
  a = c->physpn;
  bb[2].set_su2bond(1, 1, &a, &one);
  a = c->totspin;
  bb[3].set_su2bond(1, 1, &a, &one);
  c->uu[ns - 1].fuse(bb[2], bb[3]);
  for (int i = 0; i < ns / 2; ++i) {
    c->prepare_site_operator_from_left(i, 0);
    c->prepare_site_operator_from_right(ns - 1 - i, 0);
  }
  const int il = ns / 2 - 1, ir = ns / 2;
  double* w = c->ww[0];
  g_export = {&c->hh[il], &c->hh[ir]};
  g_term_i.assign(1, 0);
  g_term_d.clear();
  auto idx = [&](tensor_su2* t) {
    for (size_t q = 0; q < g_export.size(); ++q)
      if (g_export[q] == t) return (int)q;
    g_export.push_back(t);
    return (int)g_export.size() - 1;
  };
  double pair_sum = 0;
  tensor_su2 *pl = nullptr, *pr = nullptr;
  auto pair = [&](tensor_su2* l, tensor_su2* r, double coef) {
    g_term_i[0]++;
    g_term_i.push_back(idx(l));
    g_term_i.push_back(idx(r));
    g_term_d.push_back(coef);
    pair_sum += coef * l->ss_inner_prod(*r);
    pl = l;
    pr = r;
  };
  for (int i = 0; i < ns / 2; ++i)
    for (int j = ns / 2; j < ns; ++j)
      if (c->hmap[i][j] != 0) pair(&c->opr[il][i], &c->opr[ir][j], c->coup[c->hmap[i][j]]);
  for (int m = 0; m < ns * 2; ++m) {
    const int j = m % ns;
    if (!(c->plqflg[il][j] && c->plqflg[ir][j])) continue;
    const int* q = c->plqpos[j];
    if (il >= q[0] && ir <= q[1]) pair(&c->opr[il][q[0]], &c->plqopr[ir][m], -qdelta);
    else if (il >= q[1] && ir <= q[2]) pair(&c->plqopr[il][m], &c->plqopr[ir][m], -qdelta);
    else if (il >= q[2] && ir <= q[3]) pair(&c->plqopr[il][m], &c->opr[ir][q[3]], -qdelta);
    else if (pl) pair(pl, pr, -qdelta);
  }
  parts[0] = c->hh[il].take_trace();
  g_result = c->hh[ir];
  g_result.multiply_singular_value(0, w);
  g_result.multiply_singular_value(1, w);
  parts[1] = g_result.take_trace();
  parts[2] = pair_sum;
  double den = 0;
  for (int i = 0; i < max_dcut; ++i) den += w[i] * w[i];
  parts[3] = den;
  for (int i = 0; i < d && i < ww_cap; ++i) ww_out[i] = w[i];
  return (int)g_export.size();
}
#endif

// tensor_su2::take_trace, ss_inner_prod and multiply_singular_value on given
// block tensors (tensor_su2.cpp:359-384, 687-742); the scaled tensor becomes
// the result (ref_result_*).
double ref_take_trace(const int* d, const int* f, const double* x) {
  build_tensor(g_result, d, f, x);
  return g_result.take_trace();
}
double ref_ss_inner_prod(const int* da, const int* fa, const double* xa, const int* db, const int* fb,
                         const double* xb) {
  tensor_su2 b;
  build_tensor(g_result, da, fa, xa);
  build_tensor(b, db, fb, xb);
  return g_result.ss_inner_prod(b);
}
int ref_multiply_singular_value(const int* d, const int* f, const double* x, int leg, const double* w) {
  build_tensor(g_result, d, f, x);
  g_result.multiply_singular_value(leg, const_cast<double*>(w));
  g_sel = &g_result;
  return 0;
}

// The engine's lattice tables and site operators (dmrg_su2.cpp:31-300,
// initialize_local_operators) for a device-side warm-up:
//   ints = [ns, physpn, totspin, hmap (ns x ns), fll (ns x ns), frr (ns x ns),
//           plqflg (ns x ns), plqpos (ns x 4)]   (row-major)
//   dbls = [coup[0..ns)]
// and exports sigma[0], sigma[1], qterm[0..8) (ref_idmrg_select 0..9).
// Returns the int count, -1 if a capacity is too small.
int ref_engine_tables(int lx, int ly, int sec, int d, double jcoup, double qcoup, int boundary, int* ints, int icap,
                      double* dbls, int dcap) {
  max_dcut = d;
  bdry = boundary;
  delta = jcoup;
  qdelta = qcoup;
  memory_flag = 0;
  if (ly > 1) {
    cosk = cos(0.0);
    coskminus = cosk;
  }
  dmrg_su2* c = new dmrg_su2(lx, ly, sec, 0, 0, 0);
  chain_ptr = c;
  c->set_ky(0);
  const int ns = c->ns;
  if (icap < 3 + 4 * ns * ns + 4 * ns || dcap < ns) return -1;
  int p = 0;
  ints[p++] = ns;
  ints[p++] = c->physpn;
  ints[p++] = c->totspin;
  for (int** t : {c->hmap, c->fll, c->frr, c->plqflg})
    for (int i = 0; i < ns; ++i)
      for (int j = 0; j < ns; ++j) ints[p++] = t[i][j];
  for (int i = 0; i < ns; ++i)
    for (int k = 0; k < 4; ++k) ints[p++] = c->plqpos[i][k];
  for (int i = 0; i < ns; ++i) dbls[i] = c->coup[i];
  g_export = {&c->sigma[0], &c->sigma[1]};
  for (int k = 0; k < 8; ++k) g_export.push_back(&c->qterm[k]);
  return p;
}

// The reference warm-up alone (do_idmrg, dmrg_su2_omp.cpp:20-95): *enr =
// gs_enr + 1000 after it (the eigenvalue of the last step), ww[0..d) its
// last truncation's singular values.
int ref_warmup(int lx, int ly, int sec, int d, double jcoup, double qcoup, int boundary, int nthreads, double* enr,
               double* ww_out, int ww_cap) {
  max_dcut = d;
  bdry = boundary;
  delta = jcoup;
  qdelta = qcoup;
  memory_flag = 0;
  psize = nthreads;
  omp_set_num_threads(nthreads);
  mkl_set_num_threads(1);
  omp_set_nested(1);
  omp_set_max_active_levels(2);
  if (ly > 1) {
    cosk = cos(0.0);
    coskminus = cosk;
  }
  dmrg_su2* c = new dmrg_su2(lx, ly, sec, 0, 0, 0);
  chain_ptr = c;
  c->set_ky(0);
  // the step eigenvalues the engine prints (dmrg_su2.cpp:539), in full
  std::streamsize prec = std::cout.precision(17);
  c->do_idmrg();
  std::cout.precision(prec);
  *enr = c->gs_enr[0] + 1000.0;
  for (int i = 0; i < d && i < ww_cap; ++i) ww_out[i] = c->ww[0][i];
  return c->ns;
}

// after ref_run_dmrg: select the engine's MPS tensor uu[i] for ref_result_desc
int ref_select_mps(int i) {
  if (!chain_ptr || i < 0 || i >= chain_ptr->ns) return -1;
  g_sel = &chain_ptr->uu[i];
  return 0;
}

int ref_run_dmrg(int lx, int ly, int sec, int d, int niter, double jcoup, double qcoup, int boundary,
                 int nthreads, double* energies) {
  max_dcut = d;
  bdry = boundary;
  delta = jcoup;
  qdelta = qcoup;
  memory_flag = 0;
  psize = nthreads;
  omp_set_num_threads(nthreads);
  mkl_set_num_threads(1);
  omp_set_nested(1);
  omp_set_max_active_levels(2);
  if (ly > 1) {
    cosk = cos(0.0);
    coskminus = cosk;
  }
  dmrg_su2* chain = new dmrg_su2(lx, ly, sec, 0, 0, 0);
  chain_ptr = chain;
  chain->set_ky(0);
  chain->do_idmrg();
  double e1 = chain->get_enr();
  energies[0] = e1;
  int n = 1;
  for (int i = 0; i < niter; ++i) {
    chain->sweep();
    double e2 = chain->get_enr();
    energies[n++] = e2;
    if (fabs(e1 - e2) < 1.e-6) break;
    e1 = e2;
  }
  return n;
}
}
