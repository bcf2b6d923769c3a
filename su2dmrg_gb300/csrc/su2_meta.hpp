// Host-side SU(2) symmetry bookkeeping: bonds, block structures, block
// layout, Clebsch-Gordan tensors and recoupling tables.
//
// Integer metadata follows the reference exactly (bit-exact by construction):
//   su2bond::fuse                      su2bond.cpp:155-210 (2j capped at 38)
//   su2struct block index (mixed radix, leg 0 fastest)  su2struct.cpp:243-302
//   block legality (sequential fusion contains locspin) su2struct.cpp:305-332
// FP64 tables follow the reference's operation sequence:
//   tensor::make_cgc                   tensor.cpp:1353-1407
//   fac_hamilt_vec                     dmrg_su2.cpp:759-766
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace su2g {

constexpr int kMaxLegs = 4;
constexpr int kFuseCap = 38;   // su2bond.cpp:177
// The engine's recoupling arrays hold 2j < 25 (max_angm, dmrg_su2.cpp:46),
// while su2bond::fuse lets bonds reach 2j = 38; a run whose bonds pass 2j = 24
// (a large-D warm-up keeps high-spin multiplets until D binds) reads outside
// the engine's arrays.  The coefficients here are computed on demand from the
// Clebsch-Gordan contractions, so they extend to the fuse cap.
constexpr int kMaxAngm = kFuseCap + 1;

struct Bond {
  int dir = 1;
  std::vector<int> angm;  // 2j per sector, ascending
  std::vector<int> dim;   // multiplet count per sector
  int n() const { return (int)angm.size(); }
  int sector_of(int a) const {
    for (int i = 0; i < n(); ++i)
      if (angm[i] == a) return i;
    return -1;
  }
};

// The block structure of one tensor (su2struct) with its presence flags and
// the packed layout of the present blocks.
struct Struct {
  int nbond = 0, locspin = 0, nten = 0;
  Bond legs[kMaxLegs];
  std::vector<int> flag;        // 1 = block stored
  std::vector<int64_t> offset;  // doubles from the start of the packed data, -1 if absent
  int64_t total = 0;            // doubles in the packed data

  // desc = [nbond, locspin, {dir, n, angm[n], dim[n]} per leg]
  bool parse(const int* desc, std::string* err);
  // flags + offsets; flag == nullptr means "every legal block is present"
  void set_layout(const int* flags);
  void sectors(int idx, int* sec) const {
    for (int l = 0; l < nbond; ++l) {
      sec[l] = idx % legs[l].n();
      idx /= legs[l].n();
    }
  }
  int index(const int* sec) const {
    int i0 = 0;
    for (int l = nbond - 1; l >= 0; --l) i0 = i0 * legs[l].n() + sec[l];
    return i0;
  }
  bool legal_block(int idx) const;
  int block_sector(int idx, int leg) const {
    for (int l = 0; l < leg; ++l) idx /= legs[l].n();
    return idx % legs[leg].n();
  }
  int block_dim(int idx, int leg) const { return legs[leg].dim[block_sector(idx, leg)]; }
  int block_angm(int idx, int leg) const { return legs[leg].angm[block_sector(idx, leg)]; }
};

// true when `locspin` is reachable by fusing angm[0..n) left to right
bool legal_angm(const int* angm, int n, int locspin);

// su2bond::fuse with multiplicities; the result is sorted ascending and has
// direction -b1.dir (su2bond.cpp:207).
Bond fuse(const Bond& b1, const Bond& b2);

double factorial(int n);
void make_cgc(int j1, int j2, int j3, double* out);
// fac_hamilt_vec[i][j][k] stored at (i*m + j)*m + k, m = max_angm
void fac_hamilt_vec(int max_angm, double* out);
// fac_hamilt_vec[i][j][k] for 2j < kMaxAngm: the slab of one operator spin j
// is computed on first use (the same arithmetic as fac_hamilt_vec) and cached
double fac_hamilt_vec_at(int i, int j, int k);

// fac_operator_transformation_{left (side 0), rght (side 1)}[j][m][l][i][k][p]
// of dmrg_su2.cpp:857-890: the ratio between the three-CG contraction of
// tensor::contract_dmrg_operator_transformation and make_cgc(j, m, l), taken
// at the largest entry of the latter (tensor::is_proportional_to,
// tensor.cpp:1231-1269); 0 where the reference leaves the entry unset.
// Entries are computed on first use and cached (thread safe).
double fac_operator_transformation(int side, int j, int m, int l, int i, int k, int p);

// The site-update tables of dmrg_su2.cpp:776-1019, same conventions (first
// use computes, later uses read a thread-safe cache; 0 where the reference
// leaves an entry unset):
//   fac_operator_onsite_{left,rght}[j][m][l][i][p0 + 3 p1]
//   fac_operator_pairup_{left,rght}[j][i][k][m][p0 + 3 p1]
//   fac_permutation_{left,rght}[i][j][k][l][t]  (spin-1/2 sites, t < 18)
double fac_operator_onsite(int side, int j, int m, int l, int i, int q);
double fac_operator_pairup(int side, int j, int i, int k, int m, int q);
double fac_permutation(int side, int i, int j, int k, int l, int t);
// First row of the (b0 sector j0, b1 sector j1) sub-block inside the fused
// sector 2j = c of fuse(b0, b1), in the order tensor_su2::fuse places them
// (tensor_su2.cpp:878-900): b1 sectors outer, b0 sectors inner, dim0 * dim1
// rows each (b0 fastest); -1 if the pair does not reach c.
int fused_row(const Bond& b0, const Bond& b1, int c, int j0, int j1);

// tensor::make_singlet (tensor.cpp:1331-1350), (j+1) x (j+1) column-major
void make_singlet(int j, double* out);

// Ascending Shell sort of key[0..n) (gaps n/2, n/4, ..., 1, exchange inner
// loop), carrying tag[] along: the dsort2 of sort2.f:76-108.  Equal keys end
// up in the order this exchange sequence leaves them, which decides which of
// two degenerate multiplets the truncation keeps.
void dsort2(int n, double* key, int* tag);

}  // namespace su2g
