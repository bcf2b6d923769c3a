// Host-side SU(2) bookkeeping; see su2_meta.hpp for the reference map.
// Built with -ffp-contract=off: the table arithmetic must not be fused into
// multiply-adds, so the same operation sequence gives the same bits on every
// host architecture.
#include "su2_meta.hpp"

#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <utility>

namespace su2g {

bool Struct::parse(const int* d, std::string* err) {
  nbond = d[0];
  locspin = d[1];
  if (nbond < 1 || nbond > kMaxLegs) {
    if (err) *err = "nbond out of range";
    return false;
  }
  if (locspin < 0) {
    if (err) *err = "negative locspin";
    return false;
  }
  int p = 2;
  nten = 1;
  for (int l = 0; l < nbond; ++l) {
    Bond& b = legs[l];
    b.dir = d[p];
    int n = d[p + 1];
    if (n < 1 || n > 64) {
      if (err) *err = "sector count out of range";
      return false;
    }
    b.angm.assign(d + p + 2, d + p + 2 + n);
    b.dim.assign(d + p + 2 + n, d + p + 2 + 2 * n);
    for (int i = 0; i < n; ++i) {
      if (b.angm[i] < 0 || b.dim[i] < 0 || (i > 0 && b.angm[i] <= b.angm[i - 1])) {
        if (err) *err = "sector list must be ascending 2j with non-negative dims";
        return false;
      }
    }
    p += 2 + 2 * n;
    nten *= n;
  }
  return true;
}

bool legal_angm(const int* angm, int n, int locspin) {
  if (n == 1) return angm[0] == locspin;  // su2struct.cpp:279-280
  // sequential fusion of single-sector bonds (su2struct.cpp:281-296)
  int cur[kFuseCap + 2], nxt[kFuseCap + 2];
  int ncur = 1;
  cur[0] = angm[0];
  for (int l = 1; l < n; ++l) {
    int nn = 0;
    for (int i = 0; i < ncur; ++i) {
      int ks = std::abs(cur[i] - angm[l]), ke = std::abs(cur[i] + angm[l]);
      if (ke > kFuseCap) ke = kFuseCap;
      for (int k = ks; k <= ke; k += 2) {
        bool seen = false;
        for (int q = 0; q < nn; ++q)
          if (nxt[q] == k) { seen = true; break; }
        if (!seen) nxt[nn++] = k;
      }
    }
    ncur = nn;
    for (int i = 0; i < ncur; ++i) cur[i] = nxt[i];
  }
  for (int i = 0; i < ncur; ++i)
    if (cur[i] == locspin) return true;
  return false;
}

bool Struct::legal_block(int idx) const {
  int sec[kMaxLegs], a[kMaxLegs];
  sectors(idx, sec);
  for (int l = 0; l < nbond; ++l) a[l] = legs[l].angm[sec[l]];
  return legal_angm(a, nbond, locspin);
}

void Struct::set_layout(const int* flags) {
  flag.assign(nten, 0);
  offset.assign(nten, -1);
  total = 0;
  int sec[kMaxLegs];
  for (int i = 0; i < nten; ++i) {
    flag[i] = flags ? (flags[i] != 0) : (legal_block(i) ? 1 : 0);
    if (!flag[i]) continue;
    sectors(i, sec);
    int64_t sz = 1;
    for (int l = 0; l < nbond; ++l) sz *= legs[l].dim[sec[l]];
    offset[i] = total;
    total += sz;
  }
}

Bond fuse(const Bond& b1, const Bond& b2) {
  Bond out;
  out.dir = -b1.dir;
  for (int i = 0; i < b1.n(); ++i)
    for (int j = 0; j < b2.n(); ++j) {
      int ks = std::abs(b1.angm[i] - b2.angm[j]), ke = std::abs(b1.angm[i] + b2.angm[j]);
      if (ke > kFuseCap) ke = kFuseCap;
      for (int k = ks; k <= ke; k += 2) {
        int s = out.sector_of(k);
        if (s >= 0) {
          out.dim[s] += b1.dim[i] * b2.dim[j];
        } else {
          out.angm.push_back(k);
          out.dim.push_back(b1.dim[i] * b2.dim[j]);
        }
      }
    }
  // ascending by 2j (keys are distinct, so any correct sort gives isort2_'s order)
  for (int i = 1; i < out.n(); ++i)
    for (int j = i; j > 0 && out.angm[j - 1] > out.angm[j]; --j) {
      std::swap(out.angm[j - 1], out.angm[j]);
      std::swap(out.dim[j - 1], out.dim[j]);
    }
  return out;
}

double factorial(int n) {
  double f = 1;
  if (n == 0 || n == 1) return 1;
  for (int i = 2; i <= n; ++i) f *= (double)i;
  return f;
}

void make_cgc(int j1, int j2, int j3, double* out) {
  const int n0 = j1 + 1, n1 = j2 + 1, n2 = j3 + 1;
  for (int i = 0; i < n0 * n1 * n2; ++i) out[i] = 0;
  const double fac1 = std::sqrt((double)(j3 + 1) * factorial((j3 + j1 - j2) / 2) * factorial((j3 - j1 + j2) / 2) *
                                factorial((j1 + j2 - j3) / 2) / factorial((j1 + j2 + j3) / 2 + 1));
  for (int i = 0; i < n0; ++i) {
    const int m1 = 2 * i - j1;
    const double f1 = factorial((j1 + m1) / 2) * factorial((j1 - m1) / 2);
    for (int j = 0; j < n1; ++j) {
      const int m2 = 2 * j - j2;
      const double f2 = factorial((j2 + m2) / 2) * factorial((j2 - m2) / 2);
      for (int k = 0; k < n2; ++k) {
        const int m3 = 2 * k - j3;
        if (m1 + m2 - m3 != 0) continue;
        const double f3 = factorial((j3 + m3) / 2) * factorial((j3 - m3) / 2);
        const double fac2 = std::sqrt(f1 * f2 * f3);
        const int k1 = (j1 + j2 - j3) / 2, k2 = (j1 - m1) / 2, k3 = (j2 + m2) / 2;
        const int k4 = (j3 - j2 + m1) / 2, k5 = (j3 - j1 - m2) / 2, kmax = (j1 + j2 + j3) / 2;
        double sumk = 0;
        for (int k0 = 0; k0 <= kmax; ++k0) {
          if (k1 - k0 >= 0 && k2 - k0 >= 0 && k3 - k0 >= 0 && k4 + k0 >= 0 && k5 + k0 >= 0) {
            const double sgn = (k0 % 2 == 0) ? 1 : -1;
            sumk += sgn / (factorial(k0) * factorial(k1 - k0) * factorial(k2 - k0) * factorial(k3 - k0) *
                           factorial(k4 + k0) * factorial(k5 + k0));
          }
        }
        out[i + j * n0 + k * n0 * n1] = fac1 * fac2 * sumk;
      }
    }
  }
}

// Singlet entry S_jj[row, m=-m_row] = (-1)^((jj - m_row)/2) / sqrt(jj+1)
// (tensor.cpp:1339-1347); the integer sign is converted before the divide.
static inline double singlet_entry(int jj, int row) {
  const int m = 2 * row - jj;
  const int sgn = (((jj - m) / 2) % 2 == 0) ? 1 : -1;
  return sgn / std::sqrt((double)(jj + 1));
}

namespace {
bool hv_triangle(int i, int j, int k) { return k >= std::abs(i - j) && k <= std::abs(i + j) && (i % 2 == k % 2); }

// one entry: <C, C contracted with the singlet on every leg> * sqrt(j+1);
// each contracted entry is the product chain ((C*S_i)*S_j)*S_k
double fac_hamilt_vec_entry(int i, int j, int k, std::vector<double>& c) {
  const int n0 = i + 1, n1 = j + 1, n2 = k + 1, ne = n0 * n1 * n2;
  c.assign(ne, 0.0);
  make_cgc(i, j, k, c.data());
  double prod = 0;
  for (int e = 0; e < ne; ++e) {
    const int a = e % n0, b = (e / n0) % n1, cc = e / (n0 * n1);
    const int abar = n0 - 1 - a, bbar = n1 - 1 - b, cbar = n2 - 1 - cc;
    double t = c[abar + bbar * n0 + cbar * n0 * n1] * singlet_entry(i, a);
    t = t * singlet_entry(j, b);
    t = t * singlet_entry(k, cc);
    prod += c[e] * t;
  }
  return prod * std::sqrt((double)(j + 1));
}
}  // namespace

void fac_hamilt_vec(int m, double* out) {
  for (int i = 0; i < m * m * m; ++i) out[i] = 0;
  std::vector<double> c;
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j)
      for (int k = 0; k < m; ++k)
        if (hv_triangle(i, j, k)) out[(i * m + j) * m + k] = fac_hamilt_vec_entry(i, j, k, c);
}

double fac_hamilt_vec_at(int i, int j, int k) {
  constexpr int m = kMaxAngm;
  static std::vector<double> table((size_t)m * m * m, 0.0);
  static std::once_flag once[m];
  if (i < 0 || j < 0 || k < 0 || i >= m || j >= m || k >= m) return 0.0;
  std::call_once(once[j], [j] {
    std::vector<double> c;
    for (int a = 0; a < m; ++a)
      for (int b = 0; b < m; ++b)
        if (hv_triangle(a, j, b)) table[((size_t)a * m + j) * m + b] = fac_hamilt_vec_entry(a, j, b, c);
  });
  return table[((size_t)i * m + j) * m + k];
}

namespace {

// the conditions under which dmrg_su2.cpp:867-876 fills an entry
bool optrans_defined(int j, int m, int l, int i, int k, int p) {
  if (p < 0 || p > 2 || m < 0 || m > 6 || (m % 2) != 0) return false;
  if (!(j >= std::abs(i - p) && j <= i + p)) return false;
  if (!(l >= std::abs(k - p) && l <= k + p)) return false;
  return k >= std::abs(i - m) && k <= i + m && (k % 2 == i % 2) && l >= std::abs(j - m) && l <= j + m &&
         (j % 2 == l % 2);
}

// tensor::is_proportional_to (tensor.cpp:1231-1269): t = ratio * ref
bool proportional(const std::vector<double>& t, const std::vector<double>& ref, double* ratio) {
  const double tol = 1.e-12;
  bool zero = true;
  for (double v : t)
    if (std::fabs(v) > tol) zero = false;
  if (zero) {
    *ratio = 0;
    return true;
  }
  size_t pos = 0;
  double mx = 0;
  for (size_t e = 0; e < ref.size(); ++e)
    if (std::fabs(ref[e]) > mx) {
      pos = e;
      mx = std::fabs(ref[e]);
    }
  if (mx <= tol) return false;
  const double rat = t[pos] / ref[pos];
  for (size_t e = 0; e < t.size(); ++e) {
    const bool a = std::fabs(t[e]) <= tol, b = std::fabs(ref[e]) <= tol;
    if (a && b) continue;
    if (a != b) return false;
    if (std::fabs(t[e] / ref[e] - rat) > tol) return false;
  }
  *ratio = rat;
  return true;
}

double compute_optrans(int side, int j, int m, int l, int i, int k, int p) {
  // side 0: T[jj,mm,ll] = sum C(i,p,j)[ii,pp,jj] C(i,m,k)[ii,mm,kk] C(k,p,l)[kk,pp,ll]
  // side 1: T[jj,mm,ll] = sum C(p,i,j)[pp,ii,jj] C(i,m,k)[ii,mm,kk] C(p,k,l)[pp,kk,ll]
  const int ni = i + 1, nj = j + 1, nk = k + 1, nl = l + 1, nm = m + 1, np = p + 1;
  std::vector<double> c1(ni * np * nj), c2(nk * np * nl), c3(ni * nm * nk), ref(nj * nm * nl), t(nj * nm * nl, 0.0);
  if (side == 0) {
    make_cgc(i, p, j, c1.data());
    make_cgc(k, p, l, c2.data());
  } else {
    make_cgc(p, i, j, c1.data());
    make_cgc(p, k, l, c2.data());
  }
  make_cgc(i, m, k, c3.data());
  make_cgc(j, m, l, ref.data());
  for (int jj = 0; jj < nj; ++jj)
    for (int mm = 0; mm < nm; ++mm)
      for (int ll = 0; ll < nl; ++ll) {
        double sum = 0;
        for (int ii = 0; ii < ni; ++ii)
          for (int kk = 0; kk < nk; ++kk) {
            const double x3 = c3[ii + ni * (mm + nm * kk)];
            if (x3 == 0) continue;
            for (int pp = 0; pp < np; ++pp) {
              const double x1 = side == 0 ? c1[ii + ni * (pp + np * jj)] : c1[pp + np * (ii + ni * jj)];
              const double x2 = side == 0 ? c2[kk + nk * (pp + np * ll)] : c2[pp + np * (kk + nk * ll)];
              sum += x1 * x3 * x2;
            }
          }
        t[jj + nj * (mm + nm * ll)] = sum;
      }
  double ratio = 0;
  if (!proportional(t, ref, &ratio)) return 0.0;
  return ratio;
}

}  // namespace

double fac_operator_transformation(int side, int j, int m, int l, int i, int k, int p) {
  if (!optrans_defined(j, m, l, i, k, p) || j >= kMaxAngm || l >= kMaxAngm || i >= kMaxAngm || k >= kMaxAngm)
    return 0.0;
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int, int, int, int>, double> cache;
  const auto key = std::make_tuple(side, j, m, l, i, k, p);
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  const double v = compute_optrans(side, j, m, l, i, k, p);
  std::lock_guard<std::mutex> lock(mu);
  cache[key] = v;
  return v;
}

void make_singlet(int j, double* out) {
  const int n = j + 1;
  for (int e = 0; e < n * n; ++e) out[e] = 0;
  for (int r = 0; r < n; ++r) out[r + n * (n - 1 - r)] = singlet_entry(j, r);
}

namespace {

// dense CG block C(j1, j2, j3) as a column-major array
struct Cg {
  int n0, n1, n2;
  std::vector<double> v;
  Cg(int a, int b, int c) : n0(a + 1), n1(b + 1), n2(c + 1), v((size_t)(a + 1) * (b + 1) * (c + 1)) {
    make_cgc(a, b, c, v.data());
  }
  double operator()(int x, int y, int z) const { return v[x + n0 * (y + n1 * z)]; }
};

bool tri(int a, int b, int c) { return c >= std::abs(a - b) && c <= a + b; }

template <class F>
double cached(int table, int side, int a, int b, int c, int d, int e, F compute) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int, int, int, int>, double> cache;
  const auto key = std::make_tuple(table, side, a, b, c, d, e);
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  const double v = compute();
  std::lock_guard<std::mutex> lock(mu);
  cache[key] = v;
  return v;
}

// tensor::contract_dmrg_operator_initial (tensor_dmrg_src.cpp:69-101) of the
// table loop at dmrg_su2.cpp:804-833:
//   side 0  T[j,m,l] = sum C(i,p0,j)[i,q0,j] C(p0,m,p1)[q0,m,q1] C(i,p1,l)[i,q1,l]
//   side 1  T[j,m,l] = sum C(p0,i,j)[q0,i,j] C(p0,m,p1)[q0,m,q1] C(p1,i,l)[q1,i,l]
double compute_onsite(int side, int j, int m, int l, int i, int p0, int p1) {
  const Cg u = side ? Cg(p0, i, j) : Cg(i, p0, j);
  const Cg v = side ? Cg(p1, i, l) : Cg(i, p1, l);
  const Cg o(p0, m, p1), ref(j, m, l);
  std::vector<double> t(ref.v.size(), 0.0);
  for (int jj = 0; jj <= j; ++jj)
    for (int mm = 0; mm <= m; ++mm)
      for (int ll = 0; ll <= l; ++ll) {
        double sum = 0;
        for (int ii = 0; ii <= i; ++ii)
          for (int q0 = 0; q0 <= p0; ++q0) {
            const double x = side ? u(q0, ii, jj) : u(ii, q0, jj);
            if (x == 0) continue;
            for (int q1 = 0; q1 <= p1; ++q1) sum += x * o(q0, mm, q1) * (side ? v(q1, ii, ll) : v(ii, q1, ll));
          }
        t[jj + (j + 1) * (mm + (m + 1) * ll)] = sum;
      }
  double r = 0;
  return proportional(t, ref.v, &r) ? r : 0.0;
}

// tensor::contract_dmrg_operator_pairup (tensor_dmrg_src.cpp:169-211) of the
// table loop at dmrg_su2.cpp:920-943, with the site factor
// w[q0,n,q1] = sqrt(m+1) sum_mm C(p0,m,p1)[q0,mm,q1] S_m[n,mm]:
//   side 0  T[j,l] = sum C(i,p0,j)[i,q0,j] C(i,m,k)[i,n,k] w[q0,n,q1] C(k,p1,l)[k,q1,l]
//   side 1  T[j,l] = sum C(p0,i,j)[q0,i,j] C(i,m,k)[i,n,k] w[q0,n,q1] C(p1,k,l)[q1,k,l]
// compared with the identity (l = j).
double compute_pairup(int side, int j, int i, int k, int m, int p0, int p1) {
  const int l = j;
  const Cg u = side ? Cg(p0, i, j) : Cg(i, p0, j);
  const Cg v = side ? Cg(p1, k, l) : Cg(k, p1, l);
  const Cg o(p0, m, p1), op(i, m, k);
  std::vector<double> sg((size_t)(m + 1) * (m + 1));
  make_singlet(m, sg.data());
  const int n0 = p0 + 1, nm = m + 1, n1 = p1 + 1;
  std::vector<double> w((size_t)n0 * nm * n1, 0.0);
  for (int q0 = 0; q0 < n0; ++q0)
    for (int n = 0; n < nm; ++n)
      for (int q1 = 0; q1 < n1; ++q1) {
        double s = 0;
        for (int mm = 0; mm < nm; ++mm) s += o(q0, mm, q1) * sg[n + nm * mm];
        w[q0 + n0 * (n + nm * q1)] = s * std::sqrt((double)(m + 1));
      }
  // e[jj, n, kk, q1] = sum_ii,q0 u[ii,q0,jj] C(i,m,k)[ii,n,kk] w[q0,n,q1]
  std::vector<double> t((size_t)(j + 1) * (l + 1), 0.0), ident((size_t)(j + 1) * (j + 1), 0.0);
  for (int e = 0; e <= j; ++e) ident[e + (j + 1) * e] = 1.0;
  for (int jj = 0; jj <= j; ++jj)
    for (int ll = 0; ll <= l; ++ll) {
      double sum = 0;
      for (int ii = 0; ii <= i; ++ii)
        for (int q0 = 0; q0 < n0; ++q0) {
          const double x = side ? u(q0, ii, jj) : u(ii, q0, jj);
          if (x == 0) continue;
          for (int n = 0; n < nm; ++n)
            for (int kk = 0; kk <= k; ++kk) {
              const double y = op(ii, n, kk);
              if (y == 0) continue;
              for (int q1 = 0; q1 < n1; ++q1)
                sum += x * y * w[q0 + n0 * (n + nm * q1)] * (side ? v(q1, kk, ll) : v(kk, q1, ll));
            }
        }
      t[jj + (j + 1) * ll] = sum;
    }
  double r = 0;
  return proportional(t, ident, &r) ? r : 0.0;
}

// tensor::contract_dmrg_permutation (tensor_dmrg_src.cpp:476-533) of the
// table loop at dmrg_su2.cpp:974-1017 (spin-1/2 sites, P = 1), with
// (a1, a2, a3) decoded from t as a1 = 2 (t % 3), a2 = 2 ((t / 3) % 2) + 1,
// a3 = 2 ((t / 6) % 3):
//   side 0  T[j,x,l] = sum C(i,P,j)[i,q,j] C(P,a3,a2)[q,x,y] C(i,a1,k)[i,a,k] C(P,a1,a2)[p,a,y] C(k,P,l)[k,p,l]
//           compared with C(j,a3,l)
//   side 1  T[j,a,l] = sum C(P,i,j)[q,i,j] C(a2,P,a3)[y,q,x] C(i,a3,k)[i,x,k] C(a2,P,a1)[y,p,a] C(P,k,l)[p,k,l]
//           compared with C(j,a1,l)
double compute_permutation(int side, int i, int j, int k, int l, int t) {
  const int P = 1;
  const int a1 = (t % 3) * 2, a2 = ((t / 3) % 2) * 2 + 1, a3 = ((t / 6) % 3) * 2;
  if (!(tri(a1, P, a2) && tri(a2, P, a3))) return 0.0;
  if (i % 2 != k % 2 || j % 2 != l % 2) return 0.0;
  const int s_in = side ? a3 : a1;   // spin carried by the operator between i and k
  const int s_out = side ? a1 : a3;  // spin of the result between j and l
  if (!tri(s_in, i, k) || !tri(s_out, j, l)) return 0.0;
  const Cg u = side ? Cg(P, i, j) : Cg(i, P, j);
  const Cg v = side ? Cg(P, k, l) : Cg(k, P, l);
  const Cg vec(i, s_in, k), ref(j, s_out, l);
  // site factors: side 0 fu = C(P,a3,a2)[q,x,y], fv = C(P,a1,a2)[p,a,y];
  //               side 1 fu = C(a2,P,a3)[y,q,x], fv = C(a2,P,a1)[y,p,a]
  const Cg fu = side ? Cg(a2, P, a3) : Cg(P, a3, a2);
  const Cg fv = side ? Cg(a2, P, a1) : Cg(P, a1, a2);
  const int ny = a2 + 1, nq = P + 1, nx = s_out + 1, na = s_in + 1;
  std::vector<double> tt(ref.v.size(), 0.0);
  if (side == 0) {
    // vec couples to the v-side factor: b[ii,y,ll] = sum_a,kk,p vec[ii,a,kk] fv[p,a,y] v[kk,p,ll]
    std::vector<double> b((size_t)(i + 1) * ny * (l + 1), 0.0);
    for (int ii = 0; ii <= i; ++ii)
      for (int y = 0; y < ny; ++y)
        for (int ll = 0; ll <= l; ++ll) {
          double s = 0;
          for (int a = 0; a < na; ++a)
            for (int kk = 0; kk <= k; ++kk) {
              const double z = vec(ii, a, kk);
              if (z == 0) continue;
              for (int p = 0; p < nq; ++p) s += z * fv(p, a, y) * v(kk, p, ll);
            }
          b[ii + (i + 1) * (y + ny * ll)] = s;
        }
    // T[jj,x,ll] = sum_ii,q,y u[ii,q,jj] fu[q,x,y] b[ii,y,ll]
    for (int jj = 0; jj <= j; ++jj)
      for (int x = 0; x < nx; ++x)
        for (int ll = 0; ll <= l; ++ll) {
          double s = 0;
          for (int ii = 0; ii <= i; ++ii)
            for (int q = 0; q < nq; ++q) {
              const double z = u(ii, q, jj);
              if (z == 0) continue;
              for (int y = 0; y < ny; ++y) s += z * fu(q, x, y) * b[ii + (i + 1) * (y + ny * ll)];
            }
          tt[jj + (j + 1) * (x + nx * ll)] = s;
        }
  } else {
    // vec couples to the u-side factor: h[y,kk,jj] = sum_ii,q,x u[q,ii,jj] fu[y,q,x] vec[ii,x,kk]
    std::vector<double> h((size_t)ny * (k + 1) * (j + 1), 0.0);
    for (int y = 0; y < ny; ++y)
      for (int kk = 0; kk <= k; ++kk)
        for (int jj = 0; jj <= j; ++jj) {
          double s = 0;
          for (int ii = 0; ii <= i; ++ii)
            for (int q = 0; q < nq; ++q) {
              const double z = u(q, ii, jj);
              if (z == 0) continue;
              for (int x = 0; x < na; ++x) s += z * fu(y, q, x) * vec(ii, x, kk);
            }
          h[y + ny * (kk + (k + 1) * jj)] = s;
        }
    // T[jj,a,ll] = sum_y,kk,p h[y,kk,jj] fv[y,p,a] v[p,kk,ll]
    for (int jj = 0; jj <= j; ++jj)
      for (int a = 0; a < nx; ++a)
        for (int ll = 0; ll <= l; ++ll) {
          double s = 0;
          for (int y = 0; y < ny; ++y)
            for (int kk = 0; kk <= k; ++kk) {
              const double z = h[y + ny * (kk + (k + 1) * jj)];
              if (z == 0) continue;
              for (int p = 0; p < nq; ++p) s += z * fv(y, p, a) * v(p, kk, ll);
            }
          tt[jj + (j + 1) * (a + nx * ll)] = s;
        }
  }
  double r = 0;
  return proportional(tt, ref.v, &r) ? r : 0.0;
}

bool in_table(int x) { return x >= 0 && x < kMaxAngm; }

}  // namespace

double fac_operator_onsite(int side, int j, int m, int l, int i, int q) {
  const int p0 = q % 3, p1 = q / 3;
  if (q < 0 || q >= 9 || m < 0 || m > 6 || m % 2 || !in_table(j) || !in_table(l) || !in_table(i)) return 0.0;
  if (!tri(i, p0, j) || !tri(i, p1, l) || !tri(j, m, l) || j % 2 != l % 2 || !tri(p0, m, p1)) return 0.0;
  return cached(0, side, j, m, l, i, q, [&] { return compute_onsite(side, j, m, l, i, p0, p1); });
}

double fac_operator_pairup(int side, int j, int i, int k, int m, int q) {
  const int p0 = q % 3, p1 = q / 3;
  if (q < 0 || q >= 9 || m < 0 || m > 6 || m % 2 || !in_table(j) || !in_table(i) || !in_table(k)) return 0.0;
  if (!tri(i, p0, j) || !tri(k, p1, j) || !tri(i, m, k) || !tri(p0, m, p1)) return 0.0;
  return cached(1, side, j, i, k, m, q, [&] { return compute_pairup(side, j, i, k, m, p0, p1); });
}

double fac_permutation(int side, int i, int j, int k, int l, int t) {
  if (t < 0 || t >= 18 || !in_table(i) || !in_table(j) || !in_table(k) || !in_table(l)) return 0.0;
  if (!tri(i, 1, j) || !tri(k, 1, l)) return 0.0;
  return cached(2, side, i, j, k, l, t, [&] { return compute_permutation(side, i, j, k, l, t); });
}

void dsort2(int n, double* key, int* tag) {
  for (int gap = n / 2; gap > 0; gap /= 2)
    for (int i = gap; i < n; ++i)
      for (int j = i - gap; j >= 0 && key[j] > key[j + gap]; j -= gap) {
        std::swap(key[j], key[j + gap]);
        std::swap(tag[j], tag[j + gap]);
      }
}

int fused_row(const Bond& b0, const Bond& b1, int c, int j0, int j1) {
  int pos = 0;
  for (int q1 = 0; q1 < b1.n(); ++q1)
    for (int q0 = 0; q0 < b0.n(); ++q0) {
      const int a = b0.angm[q0], s = b1.angm[q1];
      if (c < std::abs(a - s) || c > a + s || (a + s - c) % 2) continue;
      if (q0 == j0 && q1 == j1) return pos;
      pos += b0.dim[q0] * b1.dim[q1];
    }
  return -1;
}

}  // namespace su2g
