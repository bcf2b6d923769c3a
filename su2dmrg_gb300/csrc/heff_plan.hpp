// Host-side construction of the H_eff work list (two launch phases).
//
// Phase 1, one intermediate block per (term t, psi block (ja,jb), op1 block
// (ja,s,jc)) that reaches a stored output block:
//     T = psi(ja,jb)^T * op1(ja,s,jc)            (jb x s_dim*jc) in scratch
// which is step1 of tensor_su2_dmrg_src.cpp:986 (tensor.cpp:521-583, i1=i2=0).
// Phase 2, one tile list per output block (jc,jd):
//     Y = hl_coef * H_L(ja,jc)^T psi(ja,jd)      (tensor_su2.cpp:1255-1345,
//       + hr_coef * psi(jc,jb) H_R(jb,jd)         dmrg_su2.cpp:563-570)
//       + sum coef_t * fac_hamilt_vec[ja][s][jc] * T^T * op2(jb,s,jd)
// where the last product is contract_dmrg_hamiltonian_vector_multiplication
// (tensor_dmrg_src.cpp:536-575) with the factor and the 1e-12 skip of
// tensor_su2_dmrg_src.cpp:995-996.  T viewed as (jb*s_dim) x jc contracts the
// operator-spin multiplicity together with jb, as the reference does.
#pragma once
#include <string>
#include <vector>

#include "gemm_work.hpp"
#include "su2_meta.hpp"
#include "su2g.h"

namespace su2g {

// One output block of a phase and the contiguous run of block products
// (GemmSeg, each over its full K) that feed it.
struct OutBlock {
  int64_t c;
  int64_t c_len;
  int c_buf;
  int ldc;
  int M, N;
  int seg0, nseg;
};

// Tile classes by output-block size (see kTileClassM/N): the table maps size
// buckets (M <= m_edges[i], N <= n_edges[j], the last bucket open-ended) to a
// class; without a table every block uses 64 x 64 tiles.
int set_tile_table(const int* m_edges, int nm, const int* n_edges, int nn, const int* cls);
int tile_class_for(int M, int N);
// the FP64 tiles of one M x N output block, in the class its size selects
void add_tiles(std::vector<GemmTile>& tiles, int64_t c_off, int64_t c_len, int c_buf, int ldc, int M, int N,
               int seg0, int nseg, int64_t kwork);

struct HeffWork {
  Struct psi;  // layout of psi and y
  std::vector<GemmSeg> seg1, seg2;
  std::vector<OutBlock> blk1, blk2;
  std::vector<GemmTile> tile1, tile2;
  int64_t scratch_len = 0;  // doubles of intermediate blocks
  double flops = 0;         // algorithmic FLOPs of one application
  int64_t max_k = 0;        // largest segment K
};

// Returns SU2G_OK or SU2G_EINVAL with *err set.  fp64_tiles: also cut the
// blocks into the FP64 engine's tiles (the split engine plans its own tiles
// from the blocks and products).
int build_heff_work(const int* psi_desc, const int* psi_flag, int nterms, const su2g_term* terms,
                    const su2g_tensor* hl, double hl_coef, const su2g_tensor* hr, double hr_coef, HeffWork* out,
                    std::string* err, bool fp64_tiles = true);

// Checks every element access the kernels will make against the extent of
// the block it belongs to (and the block against its buffer for psi, y and
// scratch): every output block with every product it sums, and every FP64
// tile when they were built.  Returns SU2G_OK or SU2G_EINVAL with *err set.
int validate_heff_work(const HeffWork& w, std::string* err);

}  // namespace su2g
