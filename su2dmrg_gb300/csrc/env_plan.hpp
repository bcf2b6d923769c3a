// Environment-update work lists (see env_plan.cpp).
#pragma once
#include <string>
#include <vector>

#include "heff_plan.hpp"

namespace su2g {

// kind 1: operator_transformation (3-leg operators), kind 0:
// overlap_transformation (2-leg scalar operators).  outs == nullptr builds only
// the output structures (presence flags = blocks reached by a product).
// Inputs and outputs are absolute device addresses (buffer kBufAbs).
int build_env_work(int kind, const su2g_tensor& uu, const su2g_tensor& vv, int flag, int nops, const su2g_tensor* ops,
                   double* const* outs, HeffWork* out, std::vector<Struct>* out_structs, std::string* err);

}  // namespace su2g
