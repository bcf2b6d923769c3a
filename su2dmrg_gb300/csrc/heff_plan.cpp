// Host-side construction of the H_eff work list; see heff_plan.hpp.
#include "heff_plan.hpp"

#include <algorithm>
#include <mutex>
#include <cmath>
#include <cstdio>

namespace su2g {
namespace {

bool same_sectors(const Bond& a, const Bond& b) { return a.angm == b.angm && a.dim == b.dim; }

struct Op {
  Struct s;
  uintptr_t base = 0;  // device address of the packed data
};

int parse_tensor(const su2g_tensor& t, int want_legs, Op* op, const char* what, std::string* err) {
  if (!t.desc) {
    *err = std::string(what) + ": missing desc";
    return SU2G_EINVAL;
  }
  std::string e;
  if (!op->s.parse(t.desc, &e)) {
    *err = std::string(what) + ": " + e;
    return SU2G_EINVAL;
  }
  if (want_legs > 0 && op->s.nbond != want_legs) {
    *err = std::string(what) + ": wrong number of legs";
    return SU2G_EINVAL;
  }
  op->s.set_layout(t.flag);
  if (op->s.total > 0 && !t.data) {
    *err = std::string(what) + ": missing data pointer";
    return SU2G_EINVAL;
  }
  op->base = reinterpret_cast<uintptr_t>(t.data);
  if (op->base % 8 != 0) {
    *err = std::string(what) + ": data not 8-byte aligned";
    return SU2G_EINVAL;
  }
  return SU2G_OK;
}

int64_t abs_off(uintptr_t base, int64_t elem_off) { return (int64_t)(base / 8) + elem_off; }

}  // namespace

// ---- tile classes by block size (filled by the autotuner; default 64 x 64) ----
namespace {
std::mutex g_tile_mu;
std::vector<int> g_tile_m_edges, g_tile_n_edges, g_tile_cls;  // buckets: size <= edge
}  // namespace

int set_tile_table(const int* m_edges, int nm, const int* n_edges, int nn, const int* cls) {
  std::vector<int> me(m_edges, m_edges + nm), ne(n_edges, n_edges + nn), c(cls, cls + (size_t)nm * nn);
  for (int v : c)
    if (v < 0 || v >= kTileClasses) return SU2G_EINVAL;
  for (int i = 1; i < nm; ++i)
    if (me[i] <= me[i - 1]) return SU2G_EINVAL;
  for (int i = 1; i < nn; ++i)
    if (ne[i] <= ne[i - 1]) return SU2G_EINVAL;
  std::lock_guard<std::mutex> lock(g_tile_mu);
  g_tile_m_edges.swap(me);
  g_tile_n_edges.swap(ne);
  g_tile_cls.swap(c);
  return SU2G_OK;
}

int tile_class_for(int M, int N) {
  std::lock_guard<std::mutex> lock(g_tile_mu);
  if (g_tile_cls.empty()) return 0;
  auto bucket = [](const std::vector<int>& edges, int v) {
    int b = 0;
    while (b + 1 < (int)edges.size() && v > edges[b]) ++b;
    return b;
  };
  return g_tile_cls[(size_t)bucket(g_tile_m_edges, M) * g_tile_n_edges.size() + bucket(g_tile_n_edges, N)];
}

void add_tiles(std::vector<GemmTile>& tiles, int64_t c_off, int64_t c_len, int c_buf, int ldc, int M, int N,
               int seg0, int nseg, int64_t kwork) {
  const int cls = tile_class_for(M, N);
  const int tm = kTileClassM[cls], tn = kTileClassN[cls];
  for (int m0 = 0; m0 < M; m0 += tm)
    for (int n0 = 0; n0 < N; n0 += tn) {
      GemmTile t{};
      t.c = c_off;
      t.c_len = c_len;
      t.c_buf = c_buf;
      t.ldc = ldc;
      t.m0 = m0;
      t.n0 = n0;
      t.mlen = std::min(tm, M - m0);
      t.nlen = std::min(tn, N - n0);
      t.seg0 = seg0;
      t.nseg = nseg;
      t.kwork = kwork;
      t.cls = cls;
      tiles.push_back(t);
    }
}

int build_heff_work(const int* psi_desc, const int* psi_flag, int nterms, const su2g_term* terms,
                    const su2g_tensor* hl, double hl_coef, const su2g_tensor* hr, double hr_coef, HeffWork* out,
                    std::string* err, bool fp64_tiles) {
  HeffWork& w = *out;
  w = HeffWork();
  if (!psi_desc) {
    *err = "psi: missing desc";
    return SU2G_EINVAL;
  }
  if (!w.psi.parse(psi_desc, err)) return SU2G_EINVAL;
  if (w.psi.nbond != 2 || w.psi.locspin != 0) {
    *err = "psi must have 2 legs and locspin 0";
    return SU2G_EINVAL;
  }
  w.psi.set_layout(psi_flag);
  const Struct& P = w.psi;
  if (nterms < 0 || (nterms > 0 && !terms)) {
    *err = "bad term list";
    return SU2G_EINVAL;
  }

  std::vector<Op> op1(nterms), op2(nterms);
  std::vector<char> scalar_pair(nterms, 0);
  for (int t = 0; t < nterms; ++t) {
    int rc = parse_tensor(terms[t].op1, 0, &op1[t], "op1", err);
    if (rc) return rc;
    rc = parse_tensor(terms[t].op2, 0, &op2[t], "op2", err);
    if (rc) return rc;
    if (op1[t].s.nbond == 2 && op2[t].s.nbond == 2) {
      // two scalar operators: contract(contract(op1, 0, vec, 0), 1, op2, 0),
      // tensor_su2_dmrg_src.cpp:902-906, i.e. L^T psi R per sector with no
      // recoupling factor; carried as 3-leg operators whose middle leg is one
      // spin-0 multiplet (the same packed layout)
      scalar_pair[t] = 1;
      for (Op* o : {&op1[t], &op2[t]}) {
        Struct& x = o->s;
        x.legs[2] = x.legs[1];
        x.legs[1] = Bond();
        x.legs[1].dir = 1;
        x.legs[1].angm = {0};
        x.legs[1].dim = {1};
        x.nbond = 3;
      }
    } else if (op1[t].s.nbond != 3 || op2[t].s.nbond != 3) {
      *err = "term " + std::to_string(t) + ": operators need 3 legs each (or 2 legs each)";
      return SU2G_EINVAL;
    }
    const Struct &s1 = op1[t].s, &s2 = op2[t].s;
    // bond checks of tensor_su2_dmrg_src.cpp:908-921 plus the output legs
    // matching psi (the result is accumulated into psi-shaped vectors)
    if (!same_sectors(s1.legs[0], P.legs[0]) || s1.legs[0].dir != -P.legs[0].dir ||
        !same_sectors(s2.legs[0], P.legs[1]) || s2.legs[0].dir != -P.legs[1].dir ||
        !same_sectors(s1.legs[1], s2.legs[1]) || s1.legs[1].dir != s2.legs[1].dir) {
      *err = "term " + std::to_string(t) + ": operator bonds do not match psi";
      return SU2G_EINVAL;
    }
    if (!same_sectors(s1.legs[2], P.legs[0]) || s1.legs[2].dir != P.legs[0].dir ||
        !same_sectors(s2.legs[2], P.legs[1]) || s2.legs[2].dir != P.legs[1].dir) {
      *err = "term " + std::to_string(t) + ": output legs differ from psi's";
      return SU2G_EINVAL;
    }
  }
  Op h[2];
  const su2g_tensor* hs[2] = {hl, hr};
  for (int side = 0; side < 2; ++side) {
    if (!hs[side]) continue;
    int rc = parse_tensor(*hs[side], 2, &h[side], side ? "hr" : "hl", err);
    if (rc) return rc;
    const Struct& s = h[side].s;
    const Bond& pb = P.legs[side];
    if (!same_sectors(s.legs[0], pb) || s.legs[0].dir != -pb.dir || !same_sectors(s.legs[1], pb) ||
        s.legs[1].dir != pb.dir) {
      *err = std::string(side ? "hr" : "hl") + ": bonds do not match psi";
      return SU2G_EINVAL;
    }
  }

  auto fac_of = [&](int ja, int s, int jc, double* f) -> bool {
    if (ja >= kMaxAngm || s >= kMaxAngm || jc >= kMaxAngm) return false;
    *f = fac_hamilt_vec_at(ja, s, jc);
    return true;
  };

  // ---- phase 1: intermediate blocks T = psi^T op1 ----
  struct TBlock {
    int t, k, j;
    int64_t off;
    int a, b, ms, c;
    int ja, jb, s, jc;
    double fac;
  };
  std::vector<TBlock> tb;
  for (int t = 0; t < nterms; ++t) {
    const Struct &s1 = op1[t].s, &s2 = op2[t].s;
    for (int j = 0; j < s1.nten; ++j) {
      if (!s1.flag[j]) continue;
      const int ja = s1.block_angm(j, 0), s = s1.block_angm(j, 1), jc = s1.block_angm(j, 2);
      const int a = s1.block_dim(j, 0), ms = s1.block_dim(j, 1), c = s1.block_dim(j, 2);
      for (int k = 0; k < P.nten; ++k) {
        if (!P.flag[k] || P.block_angm(k, 0) != ja) continue;
        const int jb = P.block_angm(k, 1), b = P.block_dim(k, 1);
        // does this step1 block reach a stored output block through op2?
        bool used = false;
        double f = 0;
        for (int l = 0; l < s2.nten && !used; ++l) {
          if (!s2.flag[l] || s2.block_angm(l, 0) != jb || s2.block_angm(l, 1) != s) continue;
          const int jd = s2.block_angm(l, 2);
          const int oa[2] = {jc, jd};
          if (!legal_angm(oa, 2, 0)) continue;
          if (scalar_pair[t]) {
            f = 1.0;
          } else if (!fac_of(ja, s, jc, &f)) {
            *err = "angular momentum beyond the recoupling table (2j > 38)";
            return SU2G_EINVAL;
          }
          if (std::fabs(f) < 1.e-12) continue;
          const int sec[2] = {P.legs[0].sector_of(jc), P.legs[1].sector_of(jd)};
          if (sec[0] < 0 || sec[1] < 0 || !P.flag[P.index(sec)]) {
            *err = "a term reaches an output block that psi's layout does not store";
            return SU2G_EINVAL;
          }
          used = true;
        }
        if (!used || a == 0 || b == 0 || ms == 0 || c == 0) continue;  // zero-size products add nothing
        TBlock T{t, k, j, w.scratch_len, a, b, ms, c, ja, jb, s, jc, f};
        tb.push_back(T);
        GemmSeg g;
        g.a = P.offset[k];
        g.a_buf = kBufPsi;
        g.b = abs_off(op1[t].base, s1.offset[j]);
        g.b_buf = kBufAbs;
        g.a_len = (int64_t)a * b;
        g.b_len = (int64_t)a * ms * c;
        g.lda = a;
        g.ldb = a;
        g.K = a;
        g.transA = 1;
        g.alpha = 1.0;
        const int seg0 = (int)w.seg1.size();
        w.seg1.push_back(g);
        if (fp64_tiles) add_tiles(w.tile1, T.off, (int64_t)b * ms * c, kBufScratch, b, b, ms * c, seg0, 1, a);
        w.blk1.push_back(OutBlock{T.off, (int64_t)b * ms * c, kBufScratch, b, b, ms * c, seg0, 1});
        w.scratch_len += (int64_t)b * ms * c;
        w.flops += 2.0 * a * b * (double)ms * c;
        w.max_k = std::max<int64_t>(w.max_k, a);
      }
    }
  }

  // ---- phase 2: output blocks ----
  for (int m = 0; m < P.nten; ++m) {
    if (!P.flag[m]) continue;
    const int jc = P.block_angm(m, 0), jd = P.block_angm(m, 1);
    const int c = P.block_dim(m, 0), d = P.block_dim(m, 1);
    const int seg0 = (int)w.seg2.size();
    int64_t kwork = 0;
    if (hl) {  // Y(jc,jd) += hl_coef * H_L(ja,jc)^T psi(ja,jd)
      const Struct& s = h[0].s;
      for (int l = 0; l < s.nten; ++l) {
        if (!s.flag[l] || s.block_angm(l, 1) != jc) continue;
        const int ja = s.block_angm(l, 0), a = s.block_dim(l, 0);
        const int sec[2] = {P.legs[0].sector_of(ja), P.legs[1].sector_of(jd)};
        if (sec[0] < 0 || !P.flag[P.index(sec)] || a == 0) continue;
        const int k = P.index(sec);
        GemmSeg g;
        g.a = abs_off(h[0].base, s.offset[l]);
        g.a_buf = kBufAbs;
        g.b = P.offset[k];
        g.b_buf = kBufPsi;
        g.a_len = (int64_t)a * c;
        g.b_len = (int64_t)a * d;
        g.lda = a;
        g.ldb = a;
        g.K = a;
        g.transA = 1;
        g.alpha = hl_coef;
        w.seg2.push_back(g);
        kwork += a;
        w.flops += 2.0 * c * (double)a * d;
        w.max_k = std::max<int64_t>(w.max_k, a);
      }
    }
    if (hr) {  // Y(jc,jd) += hr_coef * psi(jc,jb) H_R(jb,jd)
      const Struct& s = h[1].s;
      for (int l = 0; l < s.nten; ++l) {
        if (!s.flag[l] || s.block_angm(l, 1) != jd) continue;
        const int jb = s.block_angm(l, 0), b = s.block_dim(l, 0);
        const int sec[2] = {P.legs[0].sector_of(jc), P.legs[1].sector_of(jb)};
        if (sec[1] < 0 || !P.flag[P.index(sec)] || b == 0) continue;
        const int k = P.index(sec);
        GemmSeg g;
        g.a = P.offset[k];
        g.a_buf = kBufPsi;
        g.b = abs_off(h[1].base, s.offset[l]);
        g.b_buf = kBufAbs;
        g.a_len = (int64_t)c * b;
        g.b_len = (int64_t)b * d;
        g.lda = c;
        g.ldb = b;
        g.K = b;
        g.transA = 0;
        g.alpha = hr_coef;
        w.seg2.push_back(g);
        kwork += b;
        w.flops += 2.0 * c * (double)b * d;
        w.max_k = std::max<int64_t>(w.max_k, b);
      }
    }
    // spin-1 (and any other operator-spin) terms, in term order
    for (const TBlock& T : tb) {
      if (T.jc != jc) continue;
      const Struct& s2 = op2[T.t].s;
      for (int l = 0; l < s2.nten; ++l) {
        if (!s2.flag[l] || s2.block_angm(l, 0) != T.jb || s2.block_angm(l, 1) != T.s || s2.block_angm(l, 2) != jd)
          continue;
        GemmSeg g;
        g.a = T.off;
        g.a_buf = kBufScratch;
        g.b = abs_off(op2[T.t].base, s2.offset[l]);
        g.b_buf = kBufAbs;
        g.a_len = (int64_t)T.b * T.ms * T.c;
        g.b_len = (int64_t)T.b * T.ms * d;
        g.lda = T.b * T.ms;
        g.ldb = T.b * T.ms;
        g.K = T.b * T.ms;
        g.transA = 1;
        g.alpha = terms[T.t].coef * T.fac;
        w.seg2.push_back(g);
        kwork += g.K;
        w.flops += 2.0 * c * (double)g.K * d;
        w.max_k = std::max<int64_t>(w.max_k, g.K);
      }
    }
    if (fp64_tiles)
      add_tiles(w.tile2, P.offset[m], (int64_t)c * d, kBufY, c, c, d, seg0, (int)w.seg2.size() - seg0, kwork);
    w.blk2.push_back(OutBlock{P.offset[m], (int64_t)c * d, kBufY, c, c, d, seg0, (int)w.seg2.size() - seg0});
  }

  // heaviest tiles first: the block scheduler then approximates LPT order
  auto heavier = [](const GemmTile& x, const GemmTile& y) { return x.kwork > y.kwork; };
  std::stable_sort(w.tile1.begin(), w.tile1.end(), heavier);
  std::stable_sort(w.tile2.begin(), w.tile2.end(), heavier);
  return validate_heff_work(w, err);
}

namespace {
bool within(int64_t off, int64_t len, int buf, const HeffWork& w) {
  if (off < 0 || len < 0) return false;
  if (buf == kBufPsi || buf == kBufY) return off + len <= w.psi.total;
  if (buf == kBufScratch) return off + len <= w.scratch_len;
  return buf == kBufAbs;
}

// largest element index read from an operand stored with leading dimension
// ld: rows [r0, r0+nr) x columns [c0, c0+nc)
int64_t last_index(int64_t r0, int64_t nr, int64_t c0, int64_t nc, int64_t ld) {
  return (r0 + nr - 1) + (c0 + nc - 1) * ld;
}

int check_list(const std::vector<GemmTile>& tiles, const std::vector<GemmSeg>& segs, const HeffWork& w,
               const char* phase, std::string* err) {
  for (const GemmTile& t : tiles) {
    if (t.cls < 0 || t.cls >= kTileClasses || t.mlen <= 0 || t.nlen <= 0 || t.mlen > kTileClassM[t.cls] ||
        t.nlen > kTileClassN[t.cls] || t.m0 < 0 || t.n0 < 0 ||
        !within(t.c, t.c_len, t.c_buf, w) || last_index(t.m0, t.mlen, t.n0, t.nlen, t.ldc) >= t.c_len ||
        t.ldc < t.m0 + t.mlen || t.seg0 < 0 || t.nseg < 0 || t.seg0 + t.nseg > (int)segs.size()) {
      *err = std::string(phase) + ": tile out of bounds";
      return SU2G_EINVAL;
    }
    for (int s = t.seg0; s < t.seg0 + t.nseg; ++s) {
      const GemmSeg& g = segs[s];
      if (g.K <= 0 || !within(g.a, g.a_len, g.a_buf, w) || !within(g.b, g.b_len, g.b_buf, w)) {
        *err = std::string(phase) + ": segment out of bounds";
        return SU2G_EINVAL;
      }
      const int64_t alast = g.transA ? last_index(0, g.K, t.m0, t.mlen, g.lda) : last_index(t.m0, t.mlen, 0, g.K, g.lda);
      const int64_t blast = last_index(0, g.K, t.n0, t.nlen, g.ldb);
      const bool lda_ok = g.transA ? g.lda >= g.K : g.lda >= t.m0 + t.mlen;
      if (alast >= g.a_len || blast >= g.b_len || !lda_ok || g.ldb < g.K) {
        *err = std::string(phase) + ": operand access beyond its block";
        return SU2G_EINVAL;
      }
    }
  }
  return SU2G_OK;
}

// every output block (M x N, leading dimension ldc) and every product it sums:
// the accesses of all its tiles, whichever engine cuts them (a block's tiles
// reach its first and last rows and columns, and no further)
int check_blocks(const std::vector<OutBlock>& blks, const std::vector<GemmSeg>& segs, const HeffWork& w,
                 const char* phase, std::string* err) {
  for (const OutBlock& b : blks) {
    if (b.M <= 0 || b.N <= 0) continue;  // no tile
    if (!within(b.c, b.c_len, b.c_buf, w) || last_index(0, b.M, 0, b.N, b.ldc) >= b.c_len || b.ldc < b.M ||
        b.seg0 < 0 || b.nseg < 0 || b.seg0 + b.nseg > (int)segs.size()) {
      *err = std::string(phase) + ": block out of bounds";
      return SU2G_EINVAL;
    }
    for (int s = b.seg0; s < b.seg0 + b.nseg; ++s) {
      const GemmSeg& g = segs[s];
      if (g.K <= 0 || !within(g.a, g.a_len, g.a_buf, w) || !within(g.b, g.b_len, g.b_buf, w)) {
        *err = std::string(phase) + ": segment out of bounds";
        return SU2G_EINVAL;
      }
      const int64_t alast = g.transA ? last_index(0, g.K, 0, b.M, g.lda) : last_index(0, b.M, 0, g.K, g.lda);
      const int64_t blast = last_index(0, g.K, 0, b.N, g.ldb);
      const bool lda_ok = g.transA ? g.lda >= g.K : g.lda >= b.M;
      if (alast >= g.a_len || blast >= g.b_len || !lda_ok || g.ldb < g.K) {
        *err = std::string(phase) + ": operand access beyond its block";
        return SU2G_EINVAL;
      }
    }
  }
  return SU2G_OK;
}
}  // namespace

int validate_heff_work(const HeffWork& w, std::string* err) {
  int rc = check_blocks(w.blk1, w.seg1, w, "phase 1", err);
  if (!rc) rc = check_blocks(w.blk2, w.seg2, w, "phase 2", err);
  if (!rc) rc = check_list(w.tile1, w.seg1, w, "phase 1", err);
  if (!rc) rc = check_list(w.tile2, w.seg2, w, "phase 2", err);
  if (rc) return rc;
  // the output blocks cover y exactly (each element written once; the FP64
  // tiles partition the blocks)
  int64_t written = 0;
  for (const OutBlock& b : w.blk2)
    if (b.c_buf == kBufY && b.M > 0 && b.N > 0) written += (int64_t)b.M * b.N;
  if (written != w.psi.total) {
    *err = "phase 2 tiles do not cover y exactly";
    return SU2G_EINVAL;
  }
  return SU2G_OK;
}

}  // namespace su2g
