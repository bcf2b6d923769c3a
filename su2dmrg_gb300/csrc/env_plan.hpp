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
                    std::string* err);

}  // namespace su2g
