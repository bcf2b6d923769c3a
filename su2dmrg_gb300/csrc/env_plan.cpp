// Work lists of the environment updates on the block-product engine.
//
// tensor_su2::operator_transformation (tensor_su2_dmrg_src.cpp:221-402) and
// tensor_su2::overlap_transformation (:531-688) are sums of sandwiches
//     out(c[, s], c') += fac * U(a,c)^T X(a[, s], a') V(a',c')
// over the blocks of the MPS tensors uu (U) and vv (V) attached to the
// operator X through their leg `flag` (the other of legs 0/1 is the
// spin-1/2 physical leg, multiplicity 1; U, V share its sector).  fac is
// fac_operator_transformation_{left,rght}[c][s][c'][a][a'][sigma] for an
// operator (products below 1e-8 skipped, as the reference does) and 1 for the
// scalar block Hamiltonian.  Phase 1 forms T = X_s^T U (a' x c) once per
// (X block, U block, s slice); phase 2 accumulates out = sum fac T^T V per
// output block, all tiles written once.
#include "env_plan.hpp"

#include <algorithm>
#include <cmath>
#include <map>
#include <tuple>

namespace su2g {
namespace {

bool same_sectors(const Bond& a, const Bond& b) { return a.angm == b.angm && a.dim == b.dim; }

int parse(const su2g_tensor& t, int legs, Struct* s, uintptr_t* base, const char* what, std::string* err) {
  if (!t.desc) {
    *err = std::string(what) + ": missing desc";
    return SU2G_EINVAL;
  }
  std::string e;
  if (!s->parse(t.desc, &e)) {
    *err = std::string(what) + ": " + e;
    return SU2G_EINVAL;
  }
  if (s->nbond != legs) {
    *err = std::string(what) + ": wrong number of legs";
    return SU2G_EINVAL;
  }
  s->set_layout(t.flag);
  *base = reinterpret_cast<uintptr_t>(t.data);
  if (s->total > 0 && !t.data) {
    *err = std::string(what) + ": missing data pointer";
    return SU2G_EINVAL;
  }
  if (*base % 8) {
    *err = std::string(what) + ": data not 8-byte aligned";
    return SU2G_EINVAL;
  }
  return SU2G_OK;
}

int64_t abs_off(uintptr_t base, int64_t elem) { return (int64_t)(base / 8) + elem; }

void add_tiles(std::vector<GemmTile>& tiles, int64_t c_off, int64_t c_len, int c_buf, int ldc, int M, int N, int seg0,
               int nseg, int64_t kwork) {
  for (int m0 = 0; m0 < M; m0 += kTileM)
    for (int n0 = 0; n0 < N; n0 += kTileN) {
      GemmTile t;
      t.c = c_off;
      t.c_len = c_len;
      t.c_buf = c_buf;
      t.ldc = ldc;
      t.m0 = m0;
      t.n0 = n0;
      t.mlen = std::min(kTileM, M - m0);
      t.nlen = std::min(kTileN, N - n0);
      t.seg0 = seg0;
      t.nseg = nseg;
      t.kwork = kwork;
      tiles.push_back(t);
    }
}

}  // namespace

int build_env_work(int kind, const su2g_tensor& uu, const su2g_tensor& vv, int flag, int nops, const su2g_tensor* ops,
                   double* const* outs, HeffWork* out, std::vector<Struct>* out_structs, std::string* err) {
  HeffWork& w = *out;
  w = HeffWork();
  out_structs->clear();
  if (kind != 0 && kind != 1) {
    *err = "unknown transformation kind";
    return SU2G_EINVAL;
  }
  if (flag != 0 && flag != 1) {
    *err = "flag must be 0 (left) or 1 (right)";
    return SU2G_EINVAL;
  }
  if (nops < 0 || (nops > 0 && !ops)) {
    *err = "bad operator list";
    return SU2G_EINVAL;
  }
  Struct U, V;
  uintptr_t ub = 0, vb = 0;
  int rc = parse(uu, 3, &U, &ub, "uu", err);
  if (!rc) rc = parse(vv, 3, &V, &vb, "vv", err);
  if (rc) return rc;
  const int pl = 1 - flag;  // physical leg
  for (int i = 0; i < U.legs[pl].n(); ++i)
    if (U.legs[pl].dim[i] != 1) {
      *err = "physical sectors of multiplicity other than 1 are not supported";
      return SU2G_EUNSUPPORTED;
    }
  for (int i = 0; i < V.legs[pl].n(); ++i)
    if (V.legs[pl].dim[i] != 1) {
      *err = "physical sectors of multiplicity other than 1 are not supported";
      return SU2G_EUNSUPPORTED;
    }
  const int xlegs = kind ? 3 : 2;
  const int xr = xlegs - 1;  // leg of X contracted with V
  for (int t = 0; t < nops; ++t) {
    Struct X;
    uintptr_t xb = 0;
    rc = parse(ops[t], xlegs, &X, &xb, kind ? "op" : "hh", err);
    if (rc) return rc;
    // bond checks of tensor_su2_dmrg_src.cpp:229-245 / 539-555
    if (!same_sectors(U.legs[flag], X.legs[0]) || U.legs[flag].dir != -X.legs[0].dir ||
        !same_sectors(V.legs[flag], X.legs[xr]) || V.legs[flag].dir != X.legs[xr].dir) {
      *err = "operator " + std::to_string(t) + ": bonds do not match uu/vv";
      return SU2G_EINVAL;
    }
    // output structure (uu leg 2[, op leg 1], vv leg 2 inverted), locspin 0
    Struct Y;
    Y.nbond = xlegs;
    Y.locspin = 0;
    Y.legs[0] = U.legs[2];
    if (kind) Y.legs[1] = X.legs[1];
    Y.legs[xlegs - 1] = V.legs[2];
    Y.legs[xlegs - 1].dir = -V.legs[2].dir;
    Y.nten = 1;
    for (int l = 0; l < Y.nbond; ++l) Y.nten *= Y.legs[l].n();

    // ---- contributions (the reference's loop order: X block, U block, V block) ----
    struct Contrib {
      int j, k, l, m;
      double fac;
    };
    std::vector<Contrib> cs;
    std::vector<int> present(Y.nten, 0);
    for (int j = 0; j < X.nten; ++j) {
      if (!X.flag[j]) continue;
      const int a = X.block_angm(j, 0), ap = X.block_angm(j, xr), s = kind ? X.block_angm(j, 1) : 0;
      for (int k = 0; k < U.nten; ++k) {
        if (!U.flag[k] || U.block_angm(k, flag) != a) continue;
        const int sig = U.block_angm(k, pl), c = U.block_angm(k, 2);
        for (int l = 0; l < V.nten; ++l) {
          if (!V.flag[l] || V.block_angm(l, flag) != ap || V.block_angm(l, pl) != sig) continue;
          const int cp = V.block_angm(l, 2);
          int oang[3] = {c, kind ? s : cp, cp};
          if (!legal_angm(oang, xlegs, 0)) continue;
          int osec[3];
          bool ok = true;
          for (int q = 0; q < xlegs; ++q) {
            osec[q] = Y.legs[q].sector_of(oang[q]);
            if (osec[q] < 0) ok = false;
          }
          if (!ok) continue;
          double fac = 1.0;
          if (kind) {
            if (c >= kMaxAngm || s >= kMaxAngm || cp >= kMaxAngm || a >= kMaxAngm || ap >= kMaxAngm) {
              *err = "angular momentum beyond the recoupling table (2j >= 25)";
              return SU2G_EINVAL;
            }
            fac = fac_operator_transformation(flag, c, s, cp, a, ap, sig);
            if (std::fabs(fac) < 1.e-8) continue;
          }
          const int m = Y.index(osec);
          present[m] = 1;
          cs.push_back(Contrib{j, k, l, m, fac});
        }
      }
    }
    Y.set_layout(present.data());
    out_structs->push_back(Y);
    if (!outs) continue;  // layout only
    if (Y.total > 0 && !outs[t]) {
      *err = "operator " + std::to_string(t) + ": missing output pointer";
      return SU2G_EINVAL;
    }
    const uintptr_t yb = reinterpret_cast<uintptr_t>(outs[t]);
    if (yb % 8) {
      *err = "output not 8-byte aligned";
      return SU2G_EINVAL;
    }
    // ---- phase 1: T = X_s^T U per (X block, U block, s slice) ----
    std::map<std::pair<int, int>, int64_t> tpos;  // (j, k) -> scratch offset of the slice-0 T
    for (const Contrib& c : cs) {
      if (tpos.count({c.j, c.k})) continue;
      const int A = X.block_dim(c.j, 0), Ap = X.block_dim(c.j, xr), ms = kind ? X.block_dim(c.j, 1) : 1;
      const int C = U.block_dim(c.k, 2);
      tpos[{c.j, c.k}] = w.scratch_len;
      for (int sg = 0; sg < ms; ++sg) {
        GemmSeg g;
        g.a = abs_off(xb, X.offset[c.j] + (int64_t)A * sg);
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
        add_tiles(w.tile1, w.scratch_len, (int64_t)Ap * C, kBufScratch, Ap, Ap, C, seg0, 1, A);
        w.blk1.push_back(OutBlock{w.scratch_len, (int64_t)Ap * C, kBufScratch, Ap, Ap, C, seg0, 1});
        w.scratch_len += (int64_t)Ap * C;
        w.flops += 2.0 * A * (double)Ap * C;
        w.max_k = std::max<int64_t>(w.max_k, A);
      }
    }
    // ---- phase 2: out(c, s, c') = sum fac T_s^T V, per output block and slice ----
    for (int m = 0; m < Y.nten; ++m) {
      if (!Y.flag[m]) continue;
      const int C = Y.block_dim(m, 0), Cp = Y.block_dim(m, xlegs - 1), ms = kind ? Y.block_dim(m, 1) : 1;
      for (int sg = 0; sg < ms; ++sg) {
        const int seg0 = (int)w.seg2.size();
        int64_t kwork = 0;
        for (const Contrib& c : cs) {
          if (c.m != m) continue;
          const int Ap = X.block_dim(c.j, xr);
          GemmSeg g;
          g.a = tpos[{c.j, c.k}] + (int64_t)sg * Ap * C;
          g.a_buf = kBufScratch;
          g.a_len = (int64_t)Ap * C;
          g.b = abs_off(vb, V.offset[c.l]);
          g.b_buf = kBufAbs;
          g.b_len = (int64_t)Ap * Cp;
          g.lda = Ap;
          g.ldb = Ap;
          g.K = Ap;
          g.transA = 1;
          g.alpha = c.fac;
          w.seg2.push_back(g);
          kwork += Ap;
          w.flops += 2.0 * C * (double)Ap * Cp;
          w.max_k = std::max<int64_t>(w.max_k, Ap);
        }
        const int64_t yoff = abs_off(yb, Y.offset[m] + (int64_t)C * sg);
        const int64_t ylen = (int64_t)C * ms * Cp - (int64_t)C * sg;
        add_tiles(w.tile2, yoff, ylen, kBufAbs, C * ms, C, Cp, seg0, (int)w.seg2.size() - seg0, kwork);
        w.blk2.push_back(OutBlock{yoff, ylen, kBufAbs, C * ms, C, Cp, seg0, (int)w.seg2.size() - seg0});
      }
    }
  }
  if (!outs) return SU2G_OK;
  auto heavier = [](const GemmTile& x, const GemmTile& y) { return x.kwork > y.kwork; };
  std::stable_sort(w.tile1.begin(), w.tile1.end(), heavier);
  std::stable_sort(w.tile2.begin(), w.tile2.end(), heavier);
  return validate_heff_work(w, err);
}

}  // namespace su2g
