// Work lists of the environment updates on the block-product engine.
//
// Every update of a site step (dmrg_su2::prepare_site_operator_from_{left,
// right}, dmrg_su2_omp.cpp:319-825) is a sum of sandwiches
//     out(c[, s], c') += w * U(a,c)^T X(a[, s], a') V(a',c')
// over blocks of the MPS tensors uu (U) and vv (V) attached through their
// leg `flag` (the other of legs 0/1 is the spin-1/2 physical leg, multiplicity
// 1).  X is the environment operator of the job (absent for a plain
// operator_initial: then out += w U^T V), and w the product of the job's
// recoupling factor, its site-operator elements and its coefficient:
//   overlap_transformation   tensor_su2_dmrg_src.cpp:531-688   w = 1
//   operator_transformation  tensor_su2_dmrg_src.cpp:221-402   w = fac_operator_transformation
//   operator_initial         tensor_su2_dmrg_src.cpp:27-218    w = fac_operator_onsite * op
//   operator_pairup          tensor_su2_dmrg_src.cpp:691-890   w = fac_operator_pairup * op2[s]
//   permutation              tensor_su2_hamiltonian.cpp:871-1108  w = fac_permutation * <op1, op2>
// Products whose recoupling factor is below 1e-8 are skipped, and an output
// block exists when some product reaches it, as in the reference.  Phase 1
// forms T = X_s^T U once per (job, X block, U block, slice); phase 2 sums
// w T^T V (or w U^T V) per output block and slice, every tile written once.
#include "env_plan.hpp"

#include <algorithm>
#include <cmath>
#include <tuple>
#include <unordered_map>

namespace su2g {
namespace {

bool same_sectors(const Bond& a, const Bond& b) { return a.angm == b.angm && a.dim == b.dim; }
bool same_bond(const Bond& a, const Bond& b) { return a.dir == b.dir && same_sectors(a, b); }

int parse(const su2g_tensor& t, int legs, Struct* s, const char* what, std::string* err, bool need_data = true) {
  if (!t.desc) {
    *err = std::string(what) + ": missing desc";
    return SU2G_EINVAL;
  }
  std::string e;
  if (!s->parse(t.desc, &e)) {
    *err = std::string(what) + ": " + e;
    return SU2G_EINVAL;
  }
  if (legs > 0 && s->nbond != legs) {
    *err = std::string(what) + ": wrong number of legs";
    return SU2G_EINVAL;
  }
  s->set_layout(t.flag);
  if (need_data && s->total > 0 && !t.data) {
    *err = std::string(what) + ": missing data pointer";
    return SU2G_EINVAL;
  }
  return SU2G_OK;
}

int parse_dev(const su2g_tensor& t, int legs, Struct* s, uintptr_t* base, const char* what, std::string* err,
              bool need_data = true) {
  int rc = parse(t, legs, s, what, err, need_data);
  if (rc) return rc;
  *base = reinterpret_cast<uintptr_t>(t.data);
  if (*base % 8) {
    *err = std::string(what) + ": data not 8-byte aligned";
    return SU2G_EINVAL;
  }
  return SU2G_OK;
}

int64_t abs_off(uintptr_t base, int64_t elem) { return (int64_t)(base / 8) + elem; }

struct Contrib {
  int job;
  int xj;  // X block, -1: none (U^T V)
  int xs;  // X slice
  int k, l;
  int m, os;  // output block and slice
  double w;
};

// one parsed job
struct Job {
  int kind = 0, slot = 0;
  double coef = 1;
  bool has_x = false;
  Struct X, S1, S2;
  uintptr_t xb = 0;
  const double* s1 = nullptr;
  const double* s2 = nullptr;
  Struct Y;  // output structure (flags filled later)
};

int64_t block_size(const Struct& s, int b) {
  int64_t n = 1;
  for (int l = 0; l < s.nbond; ++l) n *= s.block_dim(b, l);
  return n;
}

// The stored blocks of a tensor grouped by the 2j of one leg (or of two legs),
// each group in ascending block order: the contribution loops visit exactly
// the blocks a full scan with the same tests would, in the same order,
// without scanning every block of uu and vv for every operator block.
struct Buckets {
  int w2 = 1;
  std::vector<std::vector<int>> b;
  const std::vector<int>& at(int a1, int a2 = 0) const {
    static const std::vector<int> none;
    if (a1 < 0 || a2 < 0 || a2 >= w2) return none;
    const size_t key = (size_t)a1 * w2 + a2;
    return key < b.size() ? b[key] : none;
  }
};

Buckets bucket(const Struct& s, int l1, int l2 = -1) {
  auto width = [&](int l) {
    int m = 0;
    for (int a : s.legs[l].angm) m = std::max(m, a);
    return m + 1;
  };
  Buckets r;
  r.w2 = l2 >= 0 ? width(l2) : 1;
  r.b.resize((size_t)width(l1) * r.w2);
  for (int k = 0; k < s.nten; ++k) {
    if (!s.flag[k]) continue;
    const int a1 = s.block_angm(k, l1), a2 = l2 >= 0 ? s.block_angm(k, l2) : 0;
    if (a1 >= 0 && a2 >= 0) r.b[(size_t)a1 * r.w2 + a2].push_back(k);
  }
  return r;
}

}  // namespace

int build_env_batch(const su2g_tensor& uu, const su2g_tensor& vv, int flag, int njobs, const su2g_env_job* jobs,
                    int nslots, double* const* outs, HeffWork* out, std::vector<Struct>* slot_structs,
                    std::string* err, bool fp64_tiles) {
  HeffWork& w = *out;
  w = HeffWork();
  slot_structs->clear();
  if (flag != 0 && flag != 1) {
    *err = "flag must be 0 (left) or 1 (right)";
    return SU2G_EINVAL;
  }
  if (njobs < 0 || (njobs > 0 && !jobs) || nslots < 0) {
    *err = "bad job list";
    return SU2G_EINVAL;
  }
  Struct U, V;
  uintptr_t ub = 0, vb = 0;
  int rc = parse_dev(uu, 3, &U, &ub, "uu", err);
  if (!rc) rc = parse_dev(vv, 3, &V, &vb, "vv", err);
  if (rc) return rc;
  const int pl = 1 - flag;  // physical leg
  for (const Struct* s : {&U, &V})
    for (int i = 0; i < s->legs[pl].n(); ++i)
      if (s->legs[pl].dim[i] != 1) {
        *err = "physical sectors of multiplicity other than 1 are not supported";
        return SU2G_EUNSUPPORTED;
      }
  auto fail = [&](int code, int t, const std::string& m) {
    *err = "job " + std::to_string(t) + ": " + m;
    return code;
  };
  const Buckets u_bond = bucket(U, flag), u_phys = bucket(U, pl);
  const Buckets v_bond = bucket(V, flag), v_bond_phys = bucket(V, flag, pl);
  std::vector<int> u_all;
  for (int k = 0; k < U.nten; ++k)
    if (U.flag[k]) u_all.push_back(k);

  std::vector<Job> J(njobs);
  std::vector<Contrib> cs;
  std::vector<std::vector<int>> present(nslots);
  std::vector<int> slot_owner(nslots, -1);
  for (int t = 0; t < njobs; ++t) {
    const su2g_env_job& in = jobs[t];
    Job& jb = J[t];
    jb.kind = in.kind;
    jb.slot = in.slot;
    jb.coef = in.coef;
    if (in.slot < 0 || in.slot >= nslots) return fail(SU2G_EINVAL, t, "slot out of range");
    const int kind = in.kind;
    if (kind < SU2G_ENV_OVERLAP || kind > SU2G_ENV_PERMUTATION) return fail(SU2G_EINVAL, t, "unknown kind");
    // ---- environment operator ----
    const int xlegs = (kind == SU2G_ENV_OVERLAP || kind == SU2G_ENV_INITIAL) ? 2 : 3;
    jb.has_x = in.x.desc != nullptr;
    if (!jb.has_x && kind != SU2G_ENV_INITIAL) return fail(SU2G_EINVAL, t, "missing environment operator");
    if (jb.has_x) {
      rc = parse_dev(in.x, xlegs, &jb.X, &jb.xb, "x", err);
      if (rc) return fail(rc, t, *err);
      const Bond& x0 = jb.X.legs[0];
      const Bond& xr = jb.X.legs[xlegs - 1];
      // bond checks (tensor_su2_dmrg_src.cpp:229-245, 539-555, 697-714;
      // tensor_su2_hamiltonian.cpp:879-895; operator_initial contracts endt leg
      // 0 with uu's leg, tensor_su2_dmrg_src.cpp:211-216)
      const bool dirs = kind != SU2G_ENV_INITIAL;  // the reference checks no direction for endt
      if (!same_sectors(U.legs[flag], x0) || !same_sectors(V.legs[flag], xr) ||
          (dirs && (U.legs[flag].dir != -x0.dir || V.legs[flag].dir != xr.dir)))
        return fail(SU2G_EINVAL, t, "environment operator bonds do not match uu/vv");
    } else if (!same_sectors(U.legs[flag], V.legs[flag])) {
      return fail(SU2G_EINVAL, t, "operator_initial: uu and vv bonds differ");
    }
    // ---- site operators (host) ----
    const int nsite = kind == SU2G_ENV_PERMUTATION ? 2 : (kind == SU2G_ENV_INITIAL || kind == SU2G_ENV_PAIRUP) ? 1 : 0;
    if (nsite >= 1) {
      rc = parse(in.site1, 3, &jb.S1, "site1", err);
      if (rc) return fail(rc, t, *err);
      jb.s1 = in.site1.data;
    }
    if (nsite >= 2) {
      rc = parse(in.site2, 3, &jb.S2, "site2", err);
      if (rc) return fail(rc, t, *err);
      jb.s2 = in.site2.data;
    }
    // ---- output structure: (uu leg 2, [middle], vv leg 2 inverted), locspin 0 ----
    Struct& Y = jb.Y;
    const bool three = kind == SU2G_ENV_TRANSFORM || kind == SU2G_ENV_INITIAL || kind == SU2G_ENV_PERMUTATION;
    Y.nbond = three ? 3 : 2;
    Y.locspin = 0;
    Y.legs[0] = U.legs[2];
    if (kind == SU2G_ENV_TRANSFORM) Y.legs[1] = jb.X.legs[1];
    if (kind == SU2G_ENV_INITIAL) Y.legs[1] = jb.S1.legs[1];
    if (kind == SU2G_ENV_PERMUTATION) Y.legs[1] = flag == 0 ? jb.S2.legs[1] : jb.S1.legs[2];
    Y.legs[Y.nbond - 1] = V.legs[2];
    Y.legs[Y.nbond - 1].dir = -V.legs[2].dir;
    Y.nten = 1;
    for (int l = 0; l < Y.nbond; ++l) Y.nten *= Y.legs[l].n();
    if (three)
      for (int q = 0; q < Y.legs[1].n(); ++q)
        if (kind != SU2G_ENV_TRANSFORM && Y.legs[1].dim[q] != 1)
          return fail(SU2G_EUNSUPPORTED, t, "output operator spin of multiplicity other than 1");
    const int ys = slot_owner[in.slot];
    if (ys < 0) {
      slot_owner[in.slot] = t;
      present[in.slot].assign(Y.nten, 0);
    } else {
      const Struct& Z = J[ys].Y;
      bool same = Z.nbond == Y.nbond;
      for (int l = 0; same && l < Y.nbond; ++l) same = same_bond(Z.legs[l], Y.legs[l]);
      if (!same) return fail(SU2G_EINVAL, t, "jobs of one slot produce different structures");
    }
    std::vector<int>& pres = present[in.slot];
    auto out_block = [&](int c, int s, int cp, int* m) {
      int ang[3] = {c, s, cp};
      if (Y.nbond == 2) ang[1] = cp;
      if (!legal_angm(ang, Y.nbond, 0)) return false;
      int sec[3];
      for (int q = 0; q < Y.nbond; ++q) {
        sec[q] = Y.legs[q].sector_of(ang[q]);
        if (sec[q] < 0) return false;
      }
      *m = Y.index(sec);
      return true;
    };
    auto angm_ok = [&](int a) { return a >= 0 && a < kMaxAngm; };
    const size_t c0 = cs.size();

    if (kind == SU2G_ENV_OVERLAP || kind == SU2G_ENV_TRANSFORM) {
      // reference loop order: X block, U block, V block
      const int xr = xlegs - 1;
      for (int j = 0; j < jb.X.nten; ++j) {
        if (!jb.X.flag[j]) continue;
        const int a = jb.X.block_angm(j, 0), ap = jb.X.block_angm(j, xr);
        const int s = kind == SU2G_ENV_TRANSFORM ? jb.X.block_angm(j, 1) : 0;
        const int ms = kind == SU2G_ENV_TRANSFORM ? jb.X.block_dim(j, 1) : 1;
        for (int k : u_bond.at(a)) {
          const int sig = U.block_angm(k, pl), c = U.block_angm(k, 2);
          for (int l : v_bond_phys.at(ap, sig)) {
            const int cp = V.block_angm(l, 2);
            int m;
            if (!out_block(c, s, cp, &m)) continue;
            double fac = 1.0;
            if (kind == SU2G_ENV_TRANSFORM) {
              if (!angm_ok(c) || !angm_ok(s) || !angm_ok(cp) || !angm_ok(a) || !angm_ok(ap))
                return fail(SU2G_EINVAL, t, "angular momentum beyond the recoupling table (2j > 38)");
              fac = fac_operator_transformation(flag, c, s, cp, a, ap, sig);
              if (std::fabs(fac) < 1.e-8) continue;
            }
            pres[m] = 1;
            for (int sg = 0; sg < ms; ++sg) cs.push_back(Contrib{t, j, sg, k, l, m, sg, fac});
          }
        }
      }
    } else if (kind == SU2G_ENV_INITIAL) {
      // reference loop order: site block, U block (or endt x U), V block
      const Struct& S = jb.S1;
      if (!same_sectors(U.legs[pl], S.legs[0]) || U.legs[pl].dir != -S.legs[0].dir ||
          !same_sectors(V.legs[pl], S.legs[2]) || V.legs[pl].dir != S.legs[2].dir)
        return fail(SU2G_EINVAL, t, "site operator bonds do not match uu/vv");
      const Buckets x_leg0 = jb.has_x ? bucket(jb.X, 0) : Buckets();
      const std::vector<int> no_endt{-1};
      for (int j = 0; j < S.nten; ++j) {
        if (!S.flag[j]) continue;
        if (block_size(S, j) != 1)
          return fail(SU2G_EUNSUPPORTED, t, "operator_initial needs single-element site operator blocks");
        const int sig = S.block_angm(j, 0), s = S.block_angm(j, 1), sigp = S.block_angm(j, 2);
        const double op = jb.s1[S.offset[j]];
        for (int k : u_phys.at(sig)) {
          const int a = U.block_angm(k, flag), c = U.block_angm(k, 2);
          // with endt, each U block meets the endt blocks (a, a'); a' is the
          // bond that meets vv (spin-0 endt: a' = a in 2j)
          for (int e : jb.has_x ? x_leg0.at(a) : no_endt) {
            const int ap = jb.has_x ? jb.X.block_angm(e, 1) : a;
            for (int l : v_bond_phys.at(ap, sigp)) {
              const int cp = V.block_angm(l, 2);
              int m;
              if (!out_block(c, s, cp, &m)) continue;
              if (!angm_ok(c) || !angm_ok(s) || !angm_ok(cp) || !angm_ok(ap))
                return fail(SU2G_EINVAL, t, "angular momentum beyond the recoupling table (2j > 38)");
              const double fac = fac_operator_onsite(flag, c, s, cp, ap, sig + sigp * 3);
              if (std::fabs(fac) < 1.e-8) continue;
              pres[m] = 1;
              cs.push_back(Contrib{t, jb.has_x ? e : -1, 0, k, l, m, 0, fac * op});
            }
          }
        }
      }
    } else if (kind == SU2G_ENV_PAIRUP) {
      const Struct& S = jb.S1;  // op2: (sigma, s, sigma')
      if (!same_sectors(jb.X.legs[1], S.legs[1]))
        return fail(SU2G_EINVAL, t, "operator spin legs of op1 and op2 differ");
      // reference loop order: op1 block, U block, V block, op2 block
      for (int j = 0; j < jb.X.nten; ++j) {
        if (!jb.X.flag[j]) continue;
        const int a = jb.X.block_angm(j, 0), s = jb.X.block_angm(j, 1), ap = jb.X.block_angm(j, 2);
        const int ms = jb.X.block_dim(j, 1);
        for (int k : u_bond.at(a)) {
          const int sig = U.block_angm(k, pl), c = U.block_angm(k, 2);
          for (int l : v_bond.at(ap)) {
            const int sigp = V.block_angm(l, pl), cp = V.block_angm(l, 2);
            for (int n = 0; n < S.nten; ++n) {
              if (!S.flag[n] || S.block_angm(n, 0) != sig || S.block_angm(n, 2) != sigp || S.block_angm(n, 1) != s)
                continue;
              int m;
              if (!out_block(c, 0, cp, &m)) continue;
              if (!angm_ok(c) || !angm_ok(a) || !angm_ok(ap))
                return fail(SU2G_EINVAL, t, "angular momentum beyond the recoupling table (2j > 38)");
              const double fac = fac_operator_pairup(flag, c, a, ap, s, sig + sigp * 3);
              if (std::fabs(fac) < 1.e-8) continue;
              if (block_size(S, n) != ms)
                return fail(SU2G_EINVAL, t, "site operator block does not match the operator spin multiplicity");
              pres[m] = 1;
              for (int sg = 0; sg < ms; ++sg) cs.push_back(Contrib{t, j, sg, k, l, m, 0, fac * jb.s1[S.offset[n] + sg]});
            }
          }
        }
      }
    } else {  // SU2G_ENV_PERMUTATION
      const Struct &O1 = jb.S1, &O2 = jb.S2;
      // tensor_su2_hamiltonian.cpp:896-908: the legs op1 and op2 share
      const Bond& b1 = flag == 0 ? O1.legs[2] : O1.legs[0];
      const Bond& b2 = flag == 0 ? O2.legs[2] : O2.legs[0];
      if (!same_sectors(b1, b2) || b1.dir != -b2.dir)
        return fail(SU2G_EINVAL, t, "site operators do not share a bond");
      // reference loop order: U block, vec block, V block, op1 block, op2 block
      const Buckets x_leg0 = bucket(jb.X, 0);
      for (int j : u_all) {
        const int a = U.block_angm(j, flag), sig = U.block_angm(j, pl), c = U.block_angm(j, 2);
        for (int k : x_leg0.at(a)) {
          const int s = jb.X.block_angm(k, 1), ap = jb.X.block_angm(k, 2);
          if (jb.X.block_dim(k, 1) != 1)
            return fail(SU2G_EUNSUPPORTED, t, "permutation needs an operator spin of multiplicity 1");
          for (int l : v_bond.at(ap)) {
            const int sigp = V.block_angm(l, pl), cp = V.block_angm(l, 2);
            for (int mm = 0; mm < O1.nten; ++mm) {
              if (!O1.flag[mm]) continue;
              int a4[3], a5[3];
              for (int q = 0; q < 3; ++q) a4[q] = O1.block_angm(mm, q);
              for (int nn = 0; nn < O2.nten; ++nn) {
                if (!O2.flag[nn]) continue;
                for (int q = 0; q < 3; ++q) a5[q] = O2.block_angm(nn, q);
                if ((flag == 0 && a4[2] != a5[2]) || (flag == 1 && a4[0] != a5[0])) continue;
                if ((flag == 0 && a4[1] != s) || (flag == 1 && a5[2] != s)) continue;
                if (sig != a5[flag] || sigp != a4[flag]) continue;
                const int so = flag == 0 ? a5[1] : a4[2];
                int m;
                if (!out_block(c, so, cp, &m)) continue;
                // the reference's index into the 18-entry table (C integer division)
                const int tix = flag == 0 ? a4[1] / 2 + ((a4[2] - 1) / 2) * 3 + (a5[1] / 2) * 6
                                          : a4[2] / 2 + ((a4[0] - 1) / 2) * 3 + (a5[2] / 2) * 6;
                if (tix < 0 || tix >= 18)
                  return fail(SU2G_EUNSUPPORTED, t, "site operator spins outside the permutation table");
                if (!angm_ok(a) || !angm_ok(c) || !angm_ok(ap) || !angm_ok(cp))
                  return fail(SU2G_EINVAL, t, "angular momentum beyond the recoupling table (2j > 38)");
                const double fac = fac_permutation(flag, a, c, ap, cp, tix);
                if (std::fabs(fac) < 1.e-8) continue;
                // fac1 = op1 block . op2 block (tensor::inner_prod)
                const int64_t n1 = block_size(O1, mm), n2 = block_size(O2, nn);
                if (n1 != n2) return fail(SU2G_EINVAL, t, "site operator blocks of different sizes");
                double fac1 = 0;
                for (int64_t e = 0; e < n1; ++e) fac1 += jb.s1[O1.offset[mm] + e] * jb.s2[O2.offset[nn] + e];
                pres[m] = 1;
                cs.push_back(Contrib{t, k, 0, j, l, m, 0, fac * fac1});
              }
            }
          }
        }
      }
    }
    for (size_t q = c0; q < cs.size(); ++q) cs[q].w *= jb.coef;
  }
  // slot structures
  for (int sl = 0; sl < nslots; ++sl) {
    if (slot_owner[sl] < 0) {
      *err = "slot " + std::to_string(sl) + " has no job";
      return SU2G_EINVAL;
    }
    Struct Y = J[slot_owner[sl]].Y;
    Y.set_layout(present[sl].data());
    slot_structs->push_back(Y);
  }
  if (!outs) return SU2G_OK;
  std::vector<uintptr_t> yb(nslots);
  for (int sl = 0; sl < nslots; ++sl) {
    if ((*slot_structs)[sl].total > 0 && !outs[sl]) {
      *err = "slot " + std::to_string(sl) + ": missing output pointer";
      return SU2G_EINVAL;
    }
    yb[sl] = reinterpret_cast<uintptr_t>(outs[sl]);
    if (yb[sl] % 8) {
      *err = "output not 8-byte aligned";
      return SU2G_EINVAL;
    }
  }
  // ---- phase 1: T = X_s^T U per (job, X block, U block, slice) ----
  struct TKeyHash {
    size_t operator()(const std::tuple<int, int, int>& k) const {
      const uint64_t a = (uint32_t)std::get<0>(k), b = (uint32_t)std::get<1>(k), c = (uint32_t)std::get<2>(k);
      return (size_t)((a * 0x9e3779b97f4a7c15ull) ^ (b * 0xc2b2ae3d27d4eb4full) ^ (c * 0x165667b19e3779f9ull));
    }
  };
  // (job, X block, U block) -> slice-0 T offset; lookups only (offsets follow contribution order)
  std::unordered_map<std::tuple<int, int, int>, int64_t, TKeyHash> tpos;
  for (const Contrib& c : cs) {
    if (c.xj < 0 || tpos.count({c.job, c.xj, c.k})) continue;
    const Job& jb = J[c.job];
    const int xr = jb.X.nbond - 1;
    const int A = jb.X.block_dim(c.xj, 0), Ap = jb.X.block_dim(c.xj, xr);
    const int ms = jb.X.nbond == 3 ? jb.X.block_dim(c.xj, 1) : 1;
    const int C = U.block_dim(c.k, 2);
    tpos[{c.job, c.xj, c.k}] = w.scratch_len;
    for (int sg = 0; sg < ms; ++sg) {
      GemmSeg g;
      g.a = abs_off(jb.xb, jb.X.offset[c.xj] + (int64_t)A * sg);
      g.a_buf = kBufAbs;
      g.a_len = (int64_t)A * ms * Ap - (int64_t)A * sg;
      g.b = abs_off(ub, U.offset[c.k]);
      g.b_buf = kBufAbs;
      g.b_len = (int64_t)A * C;
      g.lda = A * ms;
      g.ldb = A;
      g.K = A;
      g.transA = 1;
      g.alpha = 1.0;
      const int seg0 = (int)w.seg1.size();
      w.seg1.push_back(g);
      if (fp64_tiles) add_tiles(w.tile1, w.scratch_len, (int64_t)Ap * C, kBufScratch, Ap, Ap, C, seg0, 1, A);
      w.blk1.push_back(OutBlock{w.scratch_len, (int64_t)Ap * C, kBufScratch, Ap, Ap, C, seg0, 1});
      w.scratch_len += (int64_t)Ap * C;
      w.flops += 2.0 * A * (double)Ap * C;
      w.max_k = std::max<int64_t>(w.max_k, A);
    }
  }
  // ---- phase 2: out(c, s, c') = sum w T_s^T V (or w U^T V), per block and slice ----
  // contributions grouped by (slot, block, slice) in ascending order, each
  // group in contribution order
  using OutKey = std::tuple<int, int, int>;
  std::vector<std::pair<OutKey, int>> by_out(cs.size());
  for (int q = 0; q < (int)cs.size(); ++q) by_out[q] = {OutKey{J[cs[q].job].slot, cs[q].m, cs[q].os}, q};
  std::stable_sort(by_out.begin(), by_out.end(),
                   [](const std::pair<OutKey, int>& x, const std::pair<OutKey, int>& y) { return x.first < y.first; });
  for (size_t g0 = 0; g0 < by_out.size();) {
    size_t g1 = g0;
    while (g1 < by_out.size() && by_out[g1].first == by_out[g0].first) ++g1;
    const int sl = std::get<0>(by_out[g0].first), m = std::get<1>(by_out[g0].first), os = std::get<2>(by_out[g0].first);
    const Struct& Y = (*slot_structs)[sl];
    const int C = Y.block_dim(m, 0), Cp = Y.block_dim(m, Y.nbond - 1), ms = Y.nbond == 3 ? Y.block_dim(m, 1) : 1;
    const int seg0 = (int)w.seg2.size();
    int64_t kwork = 0;
    for (size_t gi = g0; gi < g1; ++gi) {
      const int q = by_out[gi].second;
      const Contrib& c = cs[q];
      const Job& jb = J[c.job];
      GemmSeg g;
      int K;
      if (c.xj >= 0) {
        K = jb.X.block_dim(c.xj, jb.X.nbond - 1);
        g.a = tpos[{c.job, c.xj, c.k}] + (int64_t)c.xs * K * C;
        g.a_buf = kBufScratch;
        g.a_len = (int64_t)K * C;
      } else {
        K = U.block_dim(c.k, flag);
        g.a = abs_off(ub, U.offset[c.k]);
        g.a_buf = kBufAbs;
        g.a_len = (int64_t)K * C;
      }
      g.b = abs_off(vb, V.offset[c.l]);
      g.b_buf = kBufAbs;
      g.b_len = (int64_t)K * Cp;
      g.lda = K;
      g.ldb = K;
      g.K = K;
      g.transA = 1;
      g.alpha = c.w;
      w.seg2.push_back(g);
      kwork += K;
      w.flops += 2.0 * C * (double)K * Cp;
      w.max_k = std::max<int64_t>(w.max_k, K);
    }
    const int64_t yoff = abs_off(yb[sl], Y.offset[m] + (int64_t)C * os);
    const int64_t ylen = (int64_t)C * ms * Cp - (int64_t)C * os;
    if (fp64_tiles) add_tiles(w.tile2, yoff, ylen, kBufAbs, C * ms, C, Cp, seg0, (int)w.seg2.size() - seg0, kwork);
    w.blk2.push_back(OutBlock{yoff, ylen, kBufAbs, C * ms, C, Cp, seg0, (int)w.seg2.size() - seg0});
    g0 = g1;
  }
  auto heavier = [](const GemmTile& x, const GemmTile& y) { return x.kwork > y.kwork; };
  std::stable_sort(w.tile1.begin(), w.tile1.end(), heavier);
  std::stable_sort(w.tile2.begin(), w.tile2.end(), heavier);
  return validate_heff_work(w, err);
}

int build_input_vector(const su2g_tensor& ul, const su2g_tensor& ur, const double* urt, double* out, Struct* vec,
                       HeffWork* w, std::string* err, bool fp64_tiles) {
  Struct L, R;
  uintptr_t lb = 0, rb = 0;
  int rc = parse_dev(ul, 3, &L, &lb, "input vector: ul", err, out != nullptr);
  if (!rc) rc = parse_dev(ur, 3, &R, &rb, "input vector: ur", err, out != nullptr);
  if (rc) return rc;
  // su2bond::fuse refuses legs of different directions (su2bond.cpp:159-162)
  if (L.legs[0].dir != L.legs[1].dir || R.legs[0].dir != R.legs[1].dir) {
    *err = "input vector: legs 0 and 1 of an MPS tensor have different directions";
    return SU2G_EINVAL;
  }
  // vec.contract(left, 0, rght, 0) joins the two centre bonds.  The structure
  // alone (every block of equal spins of the fused legs, makeup_input_vector)
  // does not depend on them: the warm-up's start vector joins blocks whose
  // outer bonds differ when the total spin is not 0 (fuse_to_singlet,
  // tensor_su2.cpp:1202-1247), and only its structure is used.
  if (out && !same_bond(L.legs[2], R.legs[2])) {
    *err = "input vector: ul and ur do not share their leg 2";
    return SU2G_EINVAL;
  }
  const Bond FL = fuse(L.legs[0], L.legs[1]), FR = fuse(R.legs[0], R.legs[1]);
  Struct& V = *vec;
  V = Struct();
  V.nbond = 2;
  V.locspin = 0;
  V.legs[0] = FL;
  V.legs[0].dir = L.legs[0].dir;
  V.legs[1] = FR;
  V.legs[1].dir = R.legs[0].dir;
  V.nten = FL.n() * FR.n();
  V.set_layout(nullptr);  // makeup_input_vector: every block of equal spins
  *w = HeffWork();
  if (!out) return SU2G_OK;
  const uintptr_t ob = reinterpret_cast<uintptr_t>(out), tb = reinterpret_cast<uintptr_t>(urt);
  if (ob % 8 || tb % 8 || (R.total > 0 && !urt)) {
    *err = "input vector: misaligned or missing buffer";
    return SU2G_EINVAL;
  }
  const Bond& C = L.legs[2];
  for (int k = 0; k < C.n(); ++k) {
    const int c = C.angm[k], dc = C.dim[k];
    const int i = FL.sector_of(c), j = FR.sector_of(c);
    if (i < 0 || j < 0) continue;
    const int vb = i + FL.n() * j, ldc = FL.dim[i];
    for (int r1 = 0; r1 < R.legs[1].n(); ++r1)
      for (int r0 = 0; r0 < R.legs[0].n(); ++r0) {
        const int br = r0 + R.legs[0].n() * (r1 + R.legs[1].n() * k);
        if (!R.flag[br]) continue;
        const int col = fused_row(R.legs[0], R.legs[1], c, r0, r1);
        const int nr = R.legs[0].dim[r0] * R.legs[1].dim[r1];
        for (int l1 = 0; l1 < L.legs[1].n(); ++l1)
          for (int l0 = 0; l0 < L.legs[0].n(); ++l0) {
            const int bl = l0 + L.legs[0].n() * (l1 + L.legs[1].n() * k);
            if (!L.flag[bl]) continue;
            const int row = fused_row(L.legs[0], L.legs[1], c, l0, l1);
            const int ml = L.legs[0].dim[l0] * L.legs[1].dim[l1];
            if (row < 0 || col < 0) {
              *err = "input vector: stored block outside its fused sector";
              return SU2G_EINVAL;
            }
            GemmSeg g;
            g.a = abs_off(lb, L.offset[bl]);
            g.a_buf = kBufAbs;
            g.a_len = (int64_t)ml * dc;
            g.lda = ml;
            g.transA = 0;
            g.b = abs_off(tb, R.offset[br]);
            g.b_buf = kBufAbs;
            g.b_len = (int64_t)dc * nr;
            g.ldb = dc;
            g.K = dc;
            g.alpha = 1.0;
            const int seg0 = (int)w->seg2.size();
            w->seg2.push_back(g);
            const int64_t coff = abs_off(ob, V.offset[vb] + row + (int64_t)col * ldc);
            const int64_t clen = (int64_t)(nr - 1) * ldc + ml;
            if (fp64_tiles) add_tiles(w->tile2, coff, clen, kBufAbs, ldc, ml, nr, seg0, 1, dc);
            w->blk2.push_back(OutBlock{coff, clen, kBufAbs, ldc, ml, nr, seg0, 1});
            w->flops += 2.0 * ml * (double)nr * dc;
            w->max_k = std::max<int64_t>(w->max_k, dc);
          }
      }
  }
  auto heavier = [](const GemmTile& x, const GemmTile& y) { return x.kwork > y.kwork; };
  std::stable_sort(w->tile2.begin(), w->tile2.end(), heavier);
  return validate_heff_work(*w, err);
}

}  // namespace su2g
