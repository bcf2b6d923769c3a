// Environment-update work lists (see env_plan.cpp).
#pragma once
#include <string>
#include <vector>

#include "heff_plan.hpp"

namespace su2g {

// A batch of environment updates sharing the MPS tensors uu, vv and the side
// `flag`: jobs of kinds SU2G_ENV_* (include/su2g.h), each adding its result
// (times job.coef) to output slot job.slot.  Outputs of one slot share one
// structure; its presence flags are the union of the blocks the slot's jobs
// reach.  outs == nullptr builds only the slot structures.  Device inputs
// and outputs are absolute addresses (buffer kBufAbs); site operators are
// read on the host.
int build_env_batch(const su2g_tensor& uu, const su2g_tensor& vv, int flag, int njobs, const su2g_env_job* jobs,
                    int nslots, double* const* outs, HeffWork* out, std::vector<Struct>* slot_structs,
                    std::string* err, bool fp64_tiles = true);

// The initial two-site vector of a step (dmrg_su2::prepare_input_vector,
// dmrg_su2_omp.cpp:229-254) from ul = uu[il] and ur = uu[ir]: *vec gets the
// output structure (fused legs, every equal-spin block present); with
// out != nullptr, *w gets one product per pair of stored (ul, ur) blocks of
// one centre spin, out_sub = ul_blk * urt_blk, written into its rows and
// columns of the output block.  urt holds ur's blocks transposed (d_c x
// rows, at ur's offsets).  Output elements no product reaches are not
// written (the caller zeroes them).
int build_input_vector(const su2g_tensor& ul, const su2g_tensor& ur, const double* urt, double* out, Struct* vec,
                       HeffWork* w, std::string* err, bool fp64_tiles = true);

// Runs a work list on absolute addresses once (plan, apply, wait, status,
// release); SU2G_OK at once for an empty list.
int run_work_once(HeffWork&& w, int mode, void* stream);

}  // namespace su2g
