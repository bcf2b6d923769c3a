// Split-precision work list (see ozaki.hpp for the representation).
#pragma once
#include <string>
#include <vector>

#include "heff_plan.hpp"
#include "ozaki.hpp"

namespace su2g {
namespace oz {

struct Unit {  // one CTA of the pack kernel; same layout as int2
  int job, rt;
};

struct OzWork {
  int S = 7;
  // pack jobs by source: 0 = operators (packed once at plan creation),
  // 1 = blocks of psi (packed at the start of every application),
  // 2 = phase-1 intermediates (packed between the two phases)
  std::vector<PackJob> jobs[3];
  std::vector<Unit> units[3];
  int max_nkt[3] = {0, 0, 0};  // largest k-tile count of a job of each class
  bool rows_pass[3] = {true, true, true};  // some job of the class needs the row-exponent pass
  std::vector<OzSeg> seg1, seg2;
  std::vector<OzTile> tile1, tile2;
  std::vector<RedTile> red2;  // phase-2 tiles split across CTAs: fixed-order sums
  int64_t packed_bytes = 0;   // bytes of all packed operands
  int64_t exp_len = 0;        // int32 row exponents of all packed operands
  int64_t rowmax_base = 0;    // the row-maximum slots: exps[rowmax_base, + rowmax_len),
  int64_t rowmax_len = 0;     // zeroed before phase 1 of every application
  int64_t scratch_base = 0;   // doubles of the plan scratch before the partial tiles
  int64_t partial_len = 0;    // doubles of partial tiles after scratch_base
};

// The operand that is not an operator (psi or an intermediate) carries no
// scale factor: a product's alpha is folded into its operator operand.
int build_ozaki_work(const HeffWork& hw, int S, OzWork* out, std::string* err);
// The static schedule of the persistent GEMM over `grid` CTAs: tiles dealt
// longest first to the least-loaded CTA and laid out so that CTA b walks
// b, b + grid, ...; empty tiles pad the walks.
void schedule_tiles(std::vector<OzTile>* tiles, const std::vector<OzSeg>& segs, int grid);
int validate_ozaki_work(const OzWork& w, std::string* err);

}  // namespace oz
}  // namespace su2g
