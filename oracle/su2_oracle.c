/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, CPU restatement of the reference SU2DMRG hot path, used as the
 * checker for the GPU library: only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load it, and never as the thing measured or
 * shipped.  Every function cites the reference code it follows.
 *
 * Parity pinning: tests/golden/ holds fixtures produced by the reference
 * itself (built by oracle/ref/build_ref.sh); tests/test_oracle_golden.py checks
 * this file against them before any GPU result is compared to it.
 *
 * Data model (the reference's checkpoint layout, dmrg_su2_omp.cpp:864-941):
 *   desc  = [nbond, locspin, {dir, n, angm[0..n), dim[0..n)} per leg]
 *           angm = 2j of each sector (ascending), dim = multiplet count.
 *   flag  = one int per block (mixed-radix block index, leg 0 fastest).
 *   data  = the present blocks in block order, each a column-major array of
 *           multiplet dims (leg 0 fastest).
 *
 * Floating point: compile with -ffp-contract=off so that the recoupling table
 * arithmetic is the same operation sequence as the reference build.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MAXLEG 4
#define OR_MAXSEC 64
#define OR_FUSE_CAP 38 /* su2bond.cpp:177,231,291 */

/* ----------------------------------------------------------------------- */
/* BLAS entry point (Fortran ABI), supplied by the caller at run time.      */
/* ----------------------------------------------------------------------- */
typedef void (*dgemm_fn)(const char*, const char*, const int*, const int*, const int*, const double*,
                         const double*, const int*, const double*, const int*, const double*, double*,
                         const int*);
static dgemm_fn g_dgemm = 0;
void or_set_dgemm(void* fn) { g_dgemm = (dgemm_fn)fn; }

/* ----------------------------------------------------------------------- */
/* Structure parsing                                                       */
/* ----------------------------------------------------------------------- */
typedef struct {
  int nbond, locspin, nten;
  int dir[OR_MAXLEG], n[OR_MAXLEG];
  int angm[OR_MAXLEG][OR_MAXSEC], dim[OR_MAXLEG][OR_MAXSEC];
} or_struct;

static int parse_desc(const int* d, or_struct* s) {
  s->nbond = d[0];
  s->locspin = d[1];
  if (s->nbond < 1 || s->nbond > OR_MAXLEG) return -1;
  int p = 2;
  s->nten = 1;
  for (int l = 0; l < s->nbond; ++l) {
    s->dir[l] = d[p];
    s->n[l] = d[p + 1];
    if (s->n[l] < 0 || s->n[l] > OR_MAXSEC) return -1;
    for (int i = 0; i < s->n[l]; ++i) {
      s->angm[l][i] = d[p + 2 + i];
      s->dim[l][i] = d[p + 2 + s->n[l] + i];
    }
    p += 2 + 2 * s->n[l];
    s->nten *= s->n[l];
  }
  return 0;
}

/* su2bond::fuse restricted to the angular-momentum set (su2bond.cpp:155-210):
 * all k in |m1-m2| .. min(m1+m2, 38) step 2 for every pair. */
static int fuse_set(const int* a, int na, const int* b, int nb, int* out) {
  int num = 0;
  for (int i = 0; i < na; ++i)
    for (int j = 0; j < nb; ++j) {
      int ks = abs(a[i] - b[j]), ke = abs(a[i] + b[j]);
      if (ke > OR_FUSE_CAP) ke = OR_FUSE_CAP;
      for (int k = ks; k <= ke; k += 2) {
        int seen = 0;
        for (int l = 0; l < num; ++l)
          if (out[l] == k) { seen = 1; break; }
        if (!seen) out[num++] = k;
      }
    }
  return num;
}

/* su2struct::check_angularmoments / get_tensor_argument (su2struct.cpp:264-332):
 * a block is legal when locspin is reachable by fusing its sector spins left
 * to right. */
static int legal_angm(const int* angm, int nbond, int locspin) {
  if (nbond == 1) return angm[0] == locspin;
  int cur[64], nxt[64], ncur = 1;
  cur[0] = angm[0];
  for (int l = 1; l < nbond; ++l) {
    ncur = fuse_set(cur, ncur, &angm[l], 1, nxt);
    memcpy(cur, nxt, sizeof(int) * ncur);
  }
  for (int i = 0; i < ncur; ++i)
    if (cur[i] == locspin) return 1;
  return 0;
}

/* block index -> per-leg sector indices (su2struct.cpp:272-278) */
static void block_sectors(const or_struct* s, int idx, int* sec) {
  for (int l = 0; l < s->nbond; ++l) {
    sec[l] = idx % s->n[l];
    idx /= s->n[l];
  }
}

static int block_index(const or_struct* s, const int* sec) { /* su2struct.cpp:254-258 */
  int i0 = 0;
  for (int l = s->nbond - 1; l >= 0; --l) i0 = i0 * s->n[l] + sec[l];
  return i0;
}

static int sector_of(const or_struct* s, int leg, int angm) { /* su2struct.cpp:228-240 */
  for (int i = 0; i < s->n[leg]; ++i)
    if (s->angm[leg][i] == angm) return i;
  return -1;
}

int or_nten(const int* desc) {
  or_struct s;
  if (parse_desc(desc, &s)) return -1;
  return s.nten;
}

/* legal[i] = 1 if block i passes the reference's legality test */
int or_legal_blocks(const int* desc, int* legal) {
  or_struct s;
  if (parse_desc(desc, &s)) return -1;
  int sec[OR_MAXLEG], angm[OR_MAXLEG];
  for (int i = 0; i < s.nten; ++i) {
    block_sectors(&s, i, sec);
    for (int l = 0; l < s.nbond; ++l) angm[l] = s.angm[l][sec[l]];
    legal[i] = legal_angm(angm, s.nbond, s.locspin);
  }
  return s.nten;
}

/* offsets (in doubles) of present blocks in the packed layout; -1 if absent */
int64_t or_offsets(const int* desc, const int* flag, int64_t* off) {
  or_struct s;
  if (parse_desc(desc, &s)) return -1;
  int sec[OR_MAXLEG];
  int64_t pos = 0;
  for (int i = 0; i < s.nten; ++i) {
    if (!flag[i]) { off[i] = -1; continue; }
    block_sectors(&s, i, sec);
    int64_t sz = 1;
    for (int l = 0; l < s.nbond; ++l) sz *= s.dim[l][sec[l]];
    off[i] = pos;
    pos += sz;
  }
  return pos;
}

/* su2bond::fuse with multiplicities (su2bond.cpp:155-210), the result sorted
 * ascending like isort2_ does.  Returns the sector count. */
int or_fuse(int n1, const int* a1, const int* d1, int n2, const int* a2, const int* d2, int* aout, int* dout) {
  int num = 0;
  for (int i = 0; i < n1; ++i)
    for (int j = 0; j < n2; ++j) {
      int ks = abs(a1[i] - a2[j]), ke = abs(a1[i] + a2[j]);
      if (ke > OR_FUSE_CAP) ke = OR_FUSE_CAP;
      for (int k = ks; k <= ke; k += 2) {
        int l;
        for (l = 0; l < num; ++l)
          if (aout[l] == k) { dout[l] += d1[i] * d2[j]; break; }
        if (l == num) { aout[num] = k; dout[num] = d1[i] * d2[j]; ++num; }
      }
    }
  /* insertion sort is enough for <= 64 entries; keys are distinct */
  for (int i = 1; i < num; ++i)
    for (int j = i; j > 0 && aout[j - 1] > aout[j]; --j) {
      int t = aout[j]; aout[j] = aout[j - 1]; aout[j - 1] = t;
      t = dout[j]; dout[j] = dout[j - 1]; dout[j - 1] = t;
    }
  return num;
}

/* ----------------------------------------------------------------------- */
/* Clebsch-Gordan tensors and the H_eff recoupling table                    */
/* ----------------------------------------------------------------------- */
double or_factorial(int n) { /* tensor.cpp:1410-1420 */
  double f = 1;
  if (n == 0 || n == 1) return 1;
  for (int i = 2; i <= n; ++i) f *= (double)i;
  return f;
}

/* tensor::make_cgc (tensor.cpp:1353-1407), Racah's formula with j as 2j;
 * out has (j1+1)(j2+1)(j3+1) entries, column-major. */
void or_make_cgc(int j1, int j2, int j3, double* out) {
  int n0 = j1 + 1, n1 = j2 + 1, n2 = j3 + 1;
  for (int i = 0; i < n0 * n1 * n2; ++i) out[i] = 0;
  double fac1 = sqrt((double)(j3 + 1) * or_factorial((j3 + j1 - j2) / 2) * or_factorial((j3 - j1 + j2) / 2) *
                     or_factorial((j1 + j2 - j3) / 2) / or_factorial((j1 + j2 + j3) / 2 + 1));
  for (int i = 0; i < n0; ++i) {
    int m1 = 2 * i - j1;
    double f1 = or_factorial((j1 + m1) / 2) * or_factorial((j1 - m1) / 2);
    for (int j = 0; j < n1; ++j) {
      int m2 = 2 * j - j2;
      double f2 = or_factorial((j2 + m2) / 2) * or_factorial((j2 - m2) / 2);
      for (int k = 0; k < n2; ++k) {
        int m3 = 2 * k - j3;
        double f3 = or_factorial((j3 + m3) / 2) * or_factorial((j3 - m3) / 2);
        if (m1 + m2 - m3 != 0) continue;
        double fac2 = sqrt(f1 * f2 * f3);
        int k1 = (j1 + j2 - j3) / 2, k2 = (j1 - m1) / 2, k3 = (j2 + m2) / 2;
        int k4 = (j3 - j2 + m1) / 2, k5 = (j3 - j1 - m2) / 2, kmax = (j1 + j2 + j3) / 2;
        double sumk = 0;
        for (int k0 = 0; k0 <= kmax; ++k0) {
          if (k1 - k0 >= 0 && k2 - k0 >= 0 && k3 - k0 >= 0 && k4 + k0 >= 0 && k5 + k0 >= 0) {
            double sgn = (k0 % 2 == 0) ? 1 : -1;
            sumk += sgn / (or_factorial(k0) * or_factorial(k1 - k0) * or_factorial(k2 - k0) * or_factorial(k3 - k0) *
                           or_factorial(k4 + k0) * or_factorial(k5 + k0));
          }
        }
        out[i + j * n0 + k * n0 * n1] = fac1 * fac2 * sumk;
      }
    }
  }
}

/* tensor::make_singlet (tensor.cpp:1327-1350): S[i][j] = (-1)^((jj-m1)/2)/sqrt(jj+1) for m1+m2=0 */
void or_make_singlet(int jj, double* out) {
  int n = jj + 1;
  for (int i = 0; i < n * n; ++i) out[i] = 0;
  for (int i = 0; i < n; ++i) {
    int m1 = 2 * i - jj;
    int j = n - 1 - i; /* m2 = -m1 */
    int sgn = (((jj - m1) / 2) % 2 == 0) ? 1 : -1;
    out[i + j * n] = sgn / sqrt((double)(jj + 1));
  }
}

/* fac_hamilt_vec[i][j][k] (dmrg_su2.cpp:759-766):
 *   T = C_ijk contracted on each leg with the singlet of that leg's spin,
 *   fac = <C_ijk, T> * sqrt(j+1).
 * Each singlet has one nonzero per row, so every entry of T is one product
 * chain ((C*S_i)*S_j)*S_k, formed in that order; the inner product runs over
 * entries in column-major order.  out is [max_angm]^3, k fastest. */
void or_fac_hamilt_vec(int max_angm, double* out) {
  memset(out, 0, sizeof(double) * max_angm * max_angm * max_angm);
  for (int i = 0; i < max_angm; ++i)
    for (int j = 0; j < max_angm; ++j)
      for (int k = 0; k < max_angm; ++k) {
        if (!(k >= abs(i - j) && k <= abs(i + j) && (i % 2 == k % 2))) continue;
        int n0 = i + 1, n1 = j + 1, n2 = k + 1, ne = n0 * n1 * n2;
        double* c = (double*)malloc(sizeof(double) * ne);
        or_make_cgc(i, j, k, c);
        double prod = 0;
        for (int e = 0; e < ne; ++e) {
          int a = e % n0, b = (e / n0) % n1, cc = e / (n0 * n1);
          /* T[a,b,cc] = C[abar,bbar,ccbar] * S_i[a,abar] * S_j[b,bbar] * S_k[cc,ccbar] */
          int ab = n0 - 1 - a, bb = n1 - 1 - b, cb = n2 - 1 - cc;
          int ma = 2 * a - i, mb = 2 * b - j, mc = 2 * cc - k;
          double Si = ((((i - ma) / 2) % 2 == 0) ? 1 : -1) / sqrt((double)(i + 1));
          double Sj = ((((j - mb) / 2) % 2 == 0) ? 1 : -1) / sqrt((double)(j + 1));
          double Sk = ((((k - mc) / 2) % 2 == 0) ? 1 : -1) / sqrt((double)(k + 1));
          double t = c[ab + bb * n0 + cb * n0 * n1] * Si;
          t = t * Sj;
          t = t * Sk;
          prod += c[e] * t;
        }
        out[(i * max_angm + j) * max_angm + k] = prod * sqrt((double)(j + 1));
        free(c);
      }
}

/* ----------------------------------------------------------------------- */
/* H_eff terms                                                             */
/* ----------------------------------------------------------------------- */
static void gemm(char ta, char tb, int m, int n, int k, double alpha, const double* a, int lda, const double* b,
                 int ldb, double beta, double* c, int ldc) {
  if (m == 0 || n == 0) return;
  if (g_dgemm) {
    g_dgemm(&ta, &tb, &m, &n, &k, &alpha, a, &lda, b, &ldb, &beta, c, &ldc);
    return;
  }
  /* reference loop when no BLAS was supplied (small test cases only) */
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double s = 0;
      for (int p = 0; p < k; ++p) {
        double x = (ta == 'N') ? a[i + (int64_t)p * lda] : a[p + (int64_t)i * lda];
        double y = (tb == 'N') ? b[p + (int64_t)j * ldb] : b[j + (int64_t)p * ldb];
        s += x * y;
      }
      double* cij = &c[i + (int64_t)j * ldc];
      *cij = alpha * s + (beta == 0 ? 0 : beta * *cij);
    }
}

typedef struct {
  or_struct s;
  const int* flag;
  const double* data;
  int64_t* off;
} or_tensor;

static int tensor_open(or_tensor* t, const int* desc, const int* flag, const double* data) {
  if (parse_desc(desc, &t->s)) return -1;
  t->flag = flag;
  t->data = data;
  t->off = (int64_t*)malloc(sizeof(int64_t) * (t->s.nten > 0 ? t->s.nten : 1));
  or_offsets(desc, flag, t->off);
  return 0;
}
static void tensor_close(or_tensor* t) { free(t->off); }

/* One H_eff term, tensor_su2::hamiltonian_vector_multiplication
 * (tensor_su2_dmrg_src.cpp:893-1041) for 3-leg op1/op2:
 *   for every vec block (ja,jb), op1 block (ja,s,jc), op2 block (jb,s,jd)
 *   with (jc,jd) a legal block of the output (2-leg, locspin 0):
 *     step1 = vec^T op1                      (tensor.cpp:521-583, i1=i2=0)
 *     Y(jc,jd) += coef * fac_hamilt_vec[ja][s][jc] * step1^T op2
 *                                            (tensor_dmrg_src.cpp:536-575)
 *   terms with |fac| < 1e-12 are skipped (tensor_su2_dmrg_src.cpp:996).
 * y uses the layout (ydesc, yflag); blocks the term reaches must be present.
 * nthreads > 1 parallelises over (vec block, op1 block) pairs with a private
 * output copy per thread, reduced in thread order. */
int or_heff_term(const int* vd, const int* vf, const double* vx, const int* d1, const int* f1, const double* x1,
                 const int* d2, const int* f2, const double* x2, const int* yd, const int* yf, double* y,
                 double coef, const double* fac, int max_angm) {
  or_tensor v, o1, o2, out;
  if (tensor_open(&v, vd, vf, vx) || tensor_open(&o1, d1, f1, x1) || tensor_open(&o2, d2, f2, x2) ||
      tensor_open(&out, yd, yf, y))
    return -1;
  int rc = 0;
  int np = v.s.nten * o1.s.nten;
  for (int pidx = 0; pidx < np && rc == 0; ++pidx) {
    int j = pidx % o1.s.nten, k = (pidx / o1.s.nten) % v.s.nten;
    if (!o1.flag[j] || !v.flag[k]) continue;
    int s1[OR_MAXLEG], sv[OR_MAXLEG], a1[3], av[2];
    block_sectors(&o1.s, j, s1);
    block_sectors(&v.s, k, sv);
    for (int l = 0; l < 3; ++l) a1[l] = o1.s.angm[l][s1[l]];
    for (int l = 0; l < 2; ++l) av[l] = v.s.angm[l][sv[l]];
    if (a1[0] != av[0]) continue;
    int va = v.s.dim[0][sv[0]], vb = v.s.dim[1][sv[1]];
    int oa = o1.s.dim[0][s1[0]], os = o1.s.dim[1][s1[1]], oc = o1.s.dim[2][s1[2]];
    if (oa != va) { rc = -2; break; }
    double* step1 = (double*)malloc(sizeof(double) * (size_t)vb * os * oc);
    /* step1 (vb x os*oc) = vec^T (vb x va) * op1 (va x os*oc) */
    gemm('T', 'N', vb, os * oc, va, 1.0, v.data + v.off[k], va, o1.data + o1.off[j], va, 0.0, step1, vb);
    for (int l = 0; l < o2.s.nten; ++l) {
      if (!o2.flag[l]) continue;
      int s3[OR_MAXLEG], a3[3];
      block_sectors(&o2.s, l, s3);
      for (int q = 0; q < 3; ++q) a3[q] = o2.s.angm[q][s3[q]];
      if (a3[0] != av[1] || a1[1] != a3[1]) continue;
      int oangm[2] = {a1[2], a3[2]};
      if (!legal_angm(oangm, 2, out.s.locspin)) continue;
      int os0 = sector_of(&out.s, 0, a1[2]), os1 = sector_of(&out.s, 1, a3[2]);
      if (os0 < 0 || os1 < 0) continue;
      if (a1[0] >= max_angm || a1[1] >= max_angm || a1[2] >= max_angm) { rc = -3; break; }
      double f = fac[(a1[0] * max_angm + a1[1]) * max_angm + a1[2]];
      if (fabs(f) < 1.e-12) continue;
      int osec[2] = {os0, os1};
      int m = block_index(&out.s, osec);
      if (!out.flag[m]) { rc = -4; break; }
      int rb = o2.s.dim[0][s3[0]], rs = o2.s.dim[1][s3[1]], rd = o2.s.dim[2][s3[2]];
      if (rb != vb || rs != os) { rc = -2; break; }
      /* Y (oc x rd) += coef*f * step1^T ((vb*os) x oc)^T * op2 ((vb*os) x rd) */
      gemm('T', 'N', oc, rd, vb * os, coef * f, step1, vb * os, o2.data + o2.off[l], vb * os, 1.0, y + out.off[m], oc);
    }
    free(step1);
  }
  tensor_close(&v);
  tensor_close(&o1);
  tensor_close(&o2);
  tensor_close(&out);
  return rc;
}

/* Spin-0 block-Hamiltonian terms (dmrg_su2.cpp:558-570 via tensor_su2::contract,
 * tensor_su2.cpp:1255-1345), for scalar operators with identity CG:
 *   side 0:  Y(j,j') += coef * H(j,j)^T vec(j,j')    (contract(hh[il],0,vec,0))
 *   side 1:  Y(j,j') += coef * vec(j,j') H(j',j')    (contract(vec,1,hh[ir],0)) */
int or_heff_spin0(int side, const int* hd, const int* hf, const double* hx, const int* vd, const int* vf,
                  const double* vx, const int* yd, const int* yf, double* y, double coef) {
  or_tensor h, v, out;
  if (tensor_open(&h, hd, hf, hx) || tensor_open(&v, vd, vf, vx) || tensor_open(&out, yd, yf, y)) return -1;
  int rc = 0;
  for (int k = 0; k < v.s.nten && rc == 0; ++k) {
    if (!v.flag[k]) continue;
    int sv[2];
    block_sectors(&v.s, k, sv);
    int ja = v.s.angm[0][sv[0]], jb = v.s.angm[1][sv[1]];
    int va = v.s.dim[0][sv[0]], vb = v.s.dim[1][sv[1]];
    int jc = side == 0 ? ja : jb;
    for (int l = 0; l < h.s.nten; ++l) {
      if (!h.flag[l]) continue;
      int sh[2];
      block_sectors(&h.s, l, sh);
      if (h.s.angm[0][sh[0]] != jc) continue;
      int jo = h.s.angm[1][sh[1]];
      int ho = h.s.dim[1][sh[1]], hi = h.s.dim[0][sh[0]];
      int oang[2] = {side == 0 ? jo : ja, side == 0 ? jb : jo};
      if (!legal_angm(oang, 2, out.s.locspin)) continue;
      int osec[2] = {sector_of(&out.s, 0, oang[0]), sector_of(&out.s, 1, oang[1])};
      if (osec[0] < 0 || osec[1] < 0) continue;
      int m = block_index(&out.s, osec);
      if (!out.flag[m]) { rc = -4; break; }
      if (side == 0) { /* (ho x vb) += H^T (hi x ho)^T * vec (va x vb) */
        if (hi != va) { rc = -2; break; }
        gemm('T', 'N', ho, vb, va, coef, h.data + h.off[l], hi, v.data + v.off[k], va, 1.0, y + out.off[m], ho);
      } else { /* (va x ho) += vec (va x vb) * H (hi x ho) */
        if (hi != vb) { rc = -2; break; }
        gemm('N', 'N', va, ho, vb, coef, v.data + v.off[k], va, h.data + h.off[l], hi, 1.0, y + out.off[m], va);
      }
    }
  }
  tensor_close(&h);
  tensor_close(&v);
  tensor_close(&out);
  return rc;
}

/* ----------------------------------------------------------------------- */
/* Environment updates                                                     */
/* ----------------------------------------------------------------------- */

/* tensor::is_proportional_to (tensor.cpp:1231-1269) */
static int or_proportional(const double* t, const double* ref, int n, double* ratio) {
  const double tol = 1.e-12;
  int zero = 1;
  for (int e = 0; e < n; ++e)
    if (fabs(t[e]) > tol) zero = 0;
  if (zero) { *ratio = 0; return 1; }
  int pos = 0;
  double mx = 0;
  for (int e = 0; e < n; ++e)
    if (fabs(ref[e]) > mx) { pos = e; mx = fabs(ref[e]); }
  if (mx <= tol) return 0;
  double rat = t[pos] / ref[pos];
  for (int e = 0; e < n; ++e) {
    int a = fabs(t[e]) <= tol, b = fabs(ref[e]) <= tol;
    if (a && b) continue;
    if (a != b) return 0;
    if (fabs(t[e] / ref[e] - rat) > tol) return 0;
  }
  *ratio = rat;
  return 1;
}

/* fac_operator_transformation_{left,rght}[j][m][l][i][k][p] (dmrg_su2.cpp:857-890):
 * contract_dmrg_operator_transformation (tensor_dmrg_src.cpp:104-166) of
 * three CG tensors compared with make_cgc(j,m,l). */
double or_fac_operator_transformation(int side, int j, int m, int l, int i, int k, int p) {
  if (p < 0 || p > 2 || m < 0 || m > 6 || m % 2) return 0;
  if (!(j >= abs(i - p) && j <= i + p && l >= abs(k - p) && l <= k + p)) return 0;
  if (!(k >= abs(i - m) && k <= i + m && k % 2 == i % 2 && l >= abs(j - m) && l <= j + m && j % 2 == l % 2)) return 0;
  int ni = i + 1, nj = j + 1, nk = k + 1, nl = l + 1, nm = m + 1, np = p + 1;
  double* c1 = (double*)malloc(sizeof(double) * ni * np * nj);
  double* c2 = (double*)malloc(sizeof(double) * nk * np * nl);
  double* c3 = (double*)malloc(sizeof(double) * ni * nm * nk);
  double* ref = (double*)malloc(sizeof(double) * nj * nm * nl);
  double* t = (double*)calloc(nj * nm * nl, sizeof(double));
  if (side == 0) { or_make_cgc(i, p, j, c1); or_make_cgc(k, p, l, c2); }
  else { or_make_cgc(p, i, j, c1); or_make_cgc(p, k, l, c2); }
  or_make_cgc(i, m, k, c3);
  or_make_cgc(j, m, l, ref);
  for (int a = 0; a < ni; ++a)
    for (int b = 0; b < nk; ++b)
      for (int mm = 0; mm < nm; ++mm) {
        double x3 = c3[a + ni * (mm + nm * b)];
        if (x3 == 0) continue;
        for (int pp = 0; pp < np; ++pp)
          for (int jj = 0; jj < nj; ++jj) {
            double x1 = side == 0 ? c1[a + ni * (pp + np * jj)] : c1[pp + np * (a + ni * jj)];
            if (x1 == 0) continue;
            for (int ll = 0; ll < nl; ++ll) {
              double x2 = side == 0 ? c2[b + nk * (pp + np * ll)] : c2[pp + np * (b + nk * ll)];
              t[jj + nj * (mm + nm * ll)] += x1 * x3 * x2;
            }
          }
      }
  double rat = 0;
  if (!or_proportional(t, ref, nj * nm * nl, &rat)) rat = 0;
  free(c1); free(c2); free(c3); free(ref); free(t);
  return rat;
}

/* tensor_su2::operator_transformation (kind 1, tensor_su2_dmrg_src.cpp:221-402)
 * and tensor_su2::overlap_transformation (kind 0, :531-688):
 *   out(c[, s], c') += fac * sum_p sum_{a,a'} uu(a,p,c) op(a[, s], a') vv(a',p,c')
 * for uu/vv blocks that share the physical sector p and are attached to the
 * op through leg `flag` (the other of legs 0/1 is physical), fac from the
 * transformation table (kind 1, entries below 1e-8 skipped) or 1 (kind 0).
 * The output structure is (uu leg 2[, op leg 1], vv leg 2 inverted); with
 * yout == NULL only the presence flags fout are computed (a block exists where
 * at least one product lands, as in the reference); otherwise yout receives
 * the blocks in the layout of fout. */
int or_env_transform(int kind, const int* du, const int* fu, const double* xu, const int* dv, const int* fv,
                     const double* xv, const int* dop, const int* fop, const double* xop, int flag, const int* dout,
                     int* fout, double* yout) {
  or_tensor u, v, o;
  or_struct so;
  if (tensor_open(&u, du, fu, xu) || tensor_open(&v, dv, fv, xv) || tensor_open(&o, dop, fop, xop)) return -1;
  if (parse_desc(dout, &so)) return -1;
  int64_t* yoff = (int64_t*)malloc(sizeof(int64_t) * so.nten);
  if (yout) or_offsets(dout, fout, yoff);
  else for (int i = 0; i < so.nten; ++i) fout[i] = 0;
  const int pl = 1 - flag; /* physical leg of uu/vv */
  int rc = 0;
  for (int j = 0; j < o.s.nten && !rc; ++j) {
    if (!o.flag[j]) continue;
    int so_[OR_MAXLEG], ao[3];
    block_sectors(&o.s, j, so_);
    for (int q = 0; q < o.s.nbond; ++q) ao[q] = o.s.angm[q][so_[q]];
    const int A = o.s.dim[0][so_[0]];
    const int ms = kind ? o.s.dim[1][so_[1]] : 1;
    const int Ap = o.s.dim[kind ? 2 : 1][so_[kind ? 2 : 1]];
    const int a = ao[0], ap = ao[kind ? 2 : 1], s = kind ? ao[1] : 0;
    for (int k = 0; k < u.s.nten && !rc; ++k) {
      if (!u.flag[k]) continue;
      int su[OR_MAXLEG];
      block_sectors(&u.s, k, su);
      if (u.s.angm[flag][su[flag]] != a) continue;
      const int sig = u.s.angm[pl][su[pl]], c = u.s.angm[2][su[2]];
      const int P = u.s.dim[pl][su[pl]], C = u.s.dim[2][su[2]];
      for (int l = 0; l < v.s.nten && !rc; ++l) {
        if (!v.flag[l]) continue;
        int sv[OR_MAXLEG];
        block_sectors(&v.s, l, sv);
        if (v.s.angm[flag][sv[flag]] != ap || v.s.angm[pl][sv[pl]] != sig) continue;
        const int cp = v.s.angm[2][sv[2]], Cp = v.s.dim[2][sv[2]];
        int oang[3], osec[3];
        if (kind) { oang[0] = c; oang[1] = s; oang[2] = cp; }
        else { oang[0] = c; oang[1] = cp; }
        if (!legal_angm(oang, kind ? 3 : 2, 0)) continue;
        int missing = 0;
        for (int q = 0; q < (kind ? 3 : 2); ++q) {
          osec[q] = sector_of(&so, q, oang[q]);
          if (osec[q] < 0) missing = 1;
        }
        if (missing) continue;
        double fac = 1.0;
        if (kind) {
          fac = flag == 0 ? or_fac_operator_transformation(0, c, s, cp, a, ap, sig)
                          : or_fac_operator_transformation(1, c, s, cp, a, ap, sig);
          if (fabs(fac) < 1.e-8) continue;
        }
        const int m = block_index(&so, osec);
        if (!yout) { fout[m] = 1; continue; }
        if (!fout[m]) { rc = -4; break; }
        const double* U = u.data + u.off[k];
        const double* V = v.data + v.off[l];
        const double* O = o.data + o.off[j];
        double* Y = yout + yoff[m];
        for (int p = 0; p < P; ++p)
          for (int sg = 0; sg < ms; ++sg)
            for (int cc = 0; cc < C; ++cc)
              for (int ccp = 0; ccp < Cp; ++ccp) {
                double acc = 0;
                for (int aa = 0; aa < A; ++aa) {
                  double uv = flag == 0 ? U[aa + A * (p + P * cc)] : U[p + P * (aa + A * cc)];
                  if (uv == 0) continue;
                  double inner = 0;
                  for (int aap = 0; aap < Ap; ++aap) {
                    double vv_ = flag == 0 ? V[aap + Ap * (p + P * ccp)] : V[p + P * (aap + Ap * ccp)];
                    inner += O[aa + A * (sg + ms * aap)] * vv_;
                  }
                  acc += uv * inner;
                }
                Y[cc + C * (sg + ms * ccp)] += fac * acc;
              }
      }
    }
  }
  free(yoff);
  tensor_close(&u);
  tensor_close(&v);
  tensor_close(&o);
  return rc;
}
