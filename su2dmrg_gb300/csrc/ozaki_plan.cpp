// Host-side construction of the split-precision work: pack jobs (one per
// distinct operand view, deduplicated) and the 128 x 64 output tiles with their
// segments, derived from the block-level products of the H_eff work list.
#include "ozaki_plan.hpp"

#include "kernels.hpp"

#include <algorithm>
#include <cstring>
#include <tuple>
#include <unordered_map>

namespace su2g {
namespace oz {
namespace {

using Key = std::tuple<int, int64_t, int64_t, int64_t, int, int, int, uint64_t>;

struct KeyHash {
  size_t operator()(const Key& k) const {
    uint64_t h = 0x9e3779b97f4a7c15ull;
    auto mix = [&](uint64_t x) { h ^= x + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2); };
    mix((uint64_t)std::get<0>(k));
    mix((uint64_t)std::get<1>(k));
    mix((uint64_t)std::get<2>(k));
    mix((uint64_t)std::get<3>(k));
    mix((uint64_t)std::get<4>(k));
    mix((uint64_t)std::get<5>(k));
    mix((uint64_t)std::get<6>(k));
    mix(std::get<7>(k));
    return (size_t)h;
  }
};

struct Builder {
  int S;
  OzWork* w;
  // key -> (class, job index); lookups only: jobs are numbered in order of first use
  std::unordered_map<Key, std::pair<int, int>, KeyHash> index;
  std::vector<PackJob>* lists[3];

  // class 0 = operator (packed once), 1 = from psi, 2 = from the phase-1 intermediates
  int job(int src_buf, int64_t src, int64_t ld_r, int64_t ld_k, int R, int K, int rt, double alpha) {
    uint64_t abits;
    std::memcpy(&abits, &alpha, 8);
    const Key key{src_buf, src, ld_r, ld_k, R, K, rt, abits};
    auto it = index.find(key);
    const int cls = src_buf == kBufAbs ? 0 : (src_buf == kBufPsi ? 1 : 2);
    if (it != index.end()) return it->second.second;
    PackJob j;
    j.src = src;
    j.src_buf = src_buf;
    j.R = R;
    j.K = K;
    j.ld_r = ld_r;
    j.ld_k = ld_k;
    j.rt = rt;
    j.nrt = (R + rt - 1) / rt;
    j.nkt = (K + kKS - 1) / kKS;
    j.alpha = alpha;
    j.dst = w->packed_bytes;
    j.exp = w->exp_len;
    j.texp = w->exp_len + (int64_t)j.nrt * rt;
    j.rowmax = -1;
    w->packed_bytes += (int64_t)j.nrt * j.nkt * S * rt * kKS * 2;
    w->exp_len += (int64_t)j.nrt * rt + j.nrt;
    lists[cls]->push_back(j);
    const int id = (int)lists[cls]->size() - 1;
    index[key] = {cls, id};
    return id;
  }
  const PackJob& get(int src_buf, int id) {
    const int cls = src_buf == kBufAbs ? 0 : (src_buf == kBufPsi ? 1 : 2);
    return (*lists[cls])[id];
  }
};

// The exact combination of a tile's group sums holds at most 2^17 contracted
// values (and kMaxSegs products) per output tile.  A phase-2 block fed by more
// (many terms at large D) is computed as partial tiles over runs of its
// products, each within the bounds, written into scratch and summed in run
// order by the reduction (RedTile), as the split tiles are.
constexpr int64_t kMaxKPerTile = (int64_t)1 << 17;

int build_phase(Builder& B, const std::vector<GemmSeg>& segs, const std::vector<OutBlock>& blks,
                std::vector<OzSeg>* oseg, std::vector<OzTile>* otile, std::string* err, bool may_split) {
  const int S = B.S;
  for (const OutBlock& ob : blks) {
    // pack jobs of every product of this block
    std::vector<std::pair<int, int>> ids;  // (A job, B job) indices
    std::vector<std::pair<int, int>> bufs;
    for (int s = ob.seg0; s < ob.seg0 + ob.nseg; ++s) {
      const GemmSeg& g = segs[s];
      double aa = 1.0, ab = 1.0;
      if (g.alpha != 1.0) {
        if (g.b_buf == kBufAbs) ab = g.alpha;
        else if (g.a_buf == kBufAbs) aa = g.alpha;
        else {
          *err = "split mode: a scaled product needs one operator operand";
          return SU2G_EUNSUPPORTED;
        }
      }
      const int64_t a_ldr = g.transA ? g.lda : 1, a_ldk = g.transA ? 1 : g.lda;
      const int ja = B.job(g.a_buf, g.a, a_ldr, a_ldk, ob.M, g.K, kTM, aa);
      const int jb = B.job(g.b_buf, g.b, g.ldb, 1, ob.N, g.K, kTN, ab);
      ids.push_back({ja, jb});
      bufs.push_back({g.a_buf, g.b_buf});
    }
    // runs of products within the bounds of one tile (one run: the whole
    // block, also when no product reaches it)
    std::vector<std::pair<int, int>> runs;  // (first product, count) relative to ob.seg0
    {
      int r0 = 0;
      int64_t k = 0;
      for (int s = 0; s < ob.nseg; ++s) {
        const int64_t ks = segs[ob.seg0 + s].K;
        if (ks >= kMaxKPerTile) {
          *err = "split mode: one product contracts 2^17 values or more";
          return SU2G_EUNSUPPORTED;
        }
        if (s > r0 && (k + ks >= kMaxKPerTile || s - r0 >= kMaxSegs)) {
          runs.push_back({r0, s - r0});
          r0 = s;
          k = 0;
        }
        k += ks;
      }
      runs.push_back({r0, ob.nseg - r0});  // a block no product reaches: one tile of zeros
    }
    if (runs.size() > 1 && !may_split) {
      *err = "split mode: more than 2^17 contracted values or 1024 products feed one intermediate block";
      return SU2G_EUNSUPPORTED;
    }
    for (int m0 = 0; m0 < ob.M; m0 += kTM)
      for (int n0 = 0; n0 < ob.N; n0 += kTN) {
        RedTile r{};
        const bool parts = runs.size() > 1;
        if (parts) {
          r.c = ob.c;
          r.c_buf = ob.c_buf;
          r.ldc = ob.ldc;
          r.m0 = m0;
          r.n0 = n0;
          r.mlen = std::min(kTM, ob.M - m0);
          r.nlen = std::min(kTN, ob.N - n0);
          r.part = B.w->scratch_base + B.w->partial_len;
          r.nparts = (int)runs.size();
        }
        for (const auto& run : runs) {
          OzTile t;
          t.c = ob.c;
          t.c_buf = ob.c_buf;
          t.ldc = ob.ldc;
          t.m0 = m0;
          t.n0 = n0;
          t.mlen = std::min(kTM, ob.M - m0);
          t.nlen = std::min(kTN, ob.N - n0);
          if (parts) {  // a partial tile of the scratch (kTM x kTN, column-major)
            t.c = B.w->scratch_base + B.w->partial_len;
            t.c_buf = kBufScratch;
            t.ldc = kTM;
            t.m0 = 0;
            t.n0 = 0;
            B.w->partial_len += (int64_t)kTM * kTN;
          }
          t.seg0 = (int)oseg->size();
          t.nseg = run.second;
          t.work = 0;
          t.rowmax = -1;
          t.rms = 1;
          t.pad2 = 0;
          for (int s = run.first; s < run.first + run.second; ++s) {
            const PackJob& a = B.get(bufs[s].first, ids[s].first);
            const PackJob& b = B.get(bufs[s].second, ids[s].second);
            OzSeg z;
            z.a_unit = a.dst + (int64_t)(m0 / kTM) * a.nkt * a_unit_bytes(S);
            z.b_unit = b.dst + (int64_t)(n0 / kTN) * b.nkt * b_unit_bytes(S);
            z.a_exp = a.exp + m0;
            z.b_exp = b.exp + n0;
            z.a_tmax = a.texp + m0 / kTM;
            z.nks = a.nkt;
            z.pad = 0;
            t.work += z.nks;
            oseg->push_back(z);
          }
          otile->push_back(t);
        }
        if (parts) B.w->red2.push_back(r);
      }
  }
  return SU2G_OK;
}

// Phase-2 tiles feed on many segments, but there may be fewer tiles than SMs:
// split the segment run of each tile into parts of about equal work, each part
// a CTA writing a partial tile into scratch, summed afterwards in part order.
void split_phase2(OzWork& w) {
  const int ntiles = (int)w.tile2.size();
  if (ntiles == 0 || ntiles >= kTargetCtas) return;
  const int want = (kTargetCtas + ntiles - 1) / ntiles;
  std::vector<OzTile> out;
  for (const OzTile& t : w.tile2) {
    const int parts = t.c_buf == kBufScratch ? 1 : std::min(want, t.nseg);  // partial tiles stay whole
    if (parts <= 1) {
      out.push_back(t);
      continue;
    }
    RedTile r;
    r.c = t.c;
    r.c_buf = t.c_buf;
    r.ldc = t.ldc;
    r.m0 = t.m0;
    r.n0 = t.n0;
    r.mlen = t.mlen;
    r.nlen = t.nlen;
    r.part = w.scratch_base + w.partial_len;
    r.nparts = 0;
    // cut the run where the cumulative work crosses multiples of work/parts
    int64_t done = 0;
    int s0 = t.seg0;
    for (int s = t.seg0; s < t.seg0 + t.nseg; ++s) {
      done += w.seg2[s].nks;
      const bool cut = done * parts >= (int64_t)(r.nparts + 1) * t.work || s == t.seg0 + t.nseg - 1;
      if (!cut) continue;
      OzTile p = t;
      p.c = w.scratch_base + w.partial_len;
      p.c_buf = kBufScratch;
      p.ldc = kTM;
      p.m0 = 0;
      p.n0 = 0;
      p.seg0 = s0;
      p.nseg = s + 1 - s0;
      p.work = 0;
      for (int q = s0; q <= s; ++q) p.work += w.seg2[q].nks;
      out.push_back(p);
      w.partial_len += (int64_t)kTM * kTN;
      ++r.nparts;
      s0 = s + 1;
    }
    if (r.nparts < 2) {  // one segment carries nearly all the work: keep the tile whole
      out.pop_back();
      w.partial_len -= (int64_t)kTM * kTN;
      out.push_back(t);
      continue;
    }
    w.red2.push_back(r);
  }
  w.tile2.swap(out);
}

}  // namespace

// Static schedule of the persistent GEMM, whose CTA b walks the tiles b, b +
// G, b + 2G, ... (G = grid).  Each tile's cost in stage units counts its
// stages, one drain of the TMEM group sums per chunk (about five stages of
// MMA time) and its store (about four); tiles are dealt longest first to the
// least-loaded CTA, then laid out so that the walk of CTA b visits exactly
// its own tiles, heaviest first.  CTAs with fewer tiles meet empty tiles (no
// segments, no rows) at the end of their walk.
void schedule_tiles(std::vector<OzTile>* tiles, const std::vector<OzSeg>& segs, int grid) {
  const int n = (int)tiles->size();
  auto heavier = [](const OzTile& x, const OzTile& y) { return x.work > y.work; };
  if (n <= grid || grid <= 0) {
    std::stable_sort(tiles->begin(), tiles->end(), heavier);
    return;
  }
  std::vector<int64_t> cost(n);
  for (int i = 0; i < n; ++i) {
    const OzTile& t = (*tiles)[i];
    int64_t c = 4;
    for (int s = t.seg0; s < t.seg0 + t.nseg; ++s)
      c += segs[s].nks + 5 * ((segs[s].nks + kChunkStages - 1) / kChunkStages);
    cost[i] = c;
  }
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  // Longest first to the least-loaded CTA (the lower CTA on equal loads): a
  // binary min-heap on (load, cta), whose top takes each tile's cost and
  // sinks; every (load, cta) key is distinct, so the choices are those of any
  // exact min-queue.
  std::vector<std::pair<int64_t, int>> heap(grid);  // (load, cta)
  for (int b = 0; b < grid; ++b) heap[b] = {0, b};
  std::vector<int> count(grid, 0);
  std::vector<int64_t> slot(n);  // position of tile i in the schedule: cta + k * grid
  for (int i : order) {
    const int b = heap[0].second;
    slot[i] = b + (int64_t)count[b]++ * grid;
    heap[0].first += cost[i];
    for (int p = 0;;) {  // sink the top
      const int l = 2 * p + 1, r = l + 1;
      int m = p;
      if (l < grid && heap[l] < heap[m]) m = l;
      if (r < grid && heap[r] < heap[m]) m = r;
      if (m == p) break;
      std::swap(heap[p], heap[m]);
      p = m;
    }
  }
  int kmax = 0;
  for (int c : count) kmax = std::max(kmax, c);
  OzTile pad{};
  pad.c_buf = kBufAbs;
  pad.ldc = 1;
  pad.rowmax = -1;
  pad.rms = 1;
  std::vector<OzTile> out((size_t)grid * kmax, pad);
  for (int i = 0; i < n; ++i) out[slot[i]] = (*tiles)[i];
  tiles->swap(out);
}

int build_ozaki_work(const HeffWork& hw, int S, OzWork* out, std::string* err) {
  OzWork& w = *out;
  w = OzWork();
  w.S = S;
  w.scratch_base = hw.scratch_len;
  Builder B;
  B.S = S;
  B.w = &w;
  B.lists[0] = &w.jobs[0];
  B.lists[1] = &w.jobs[1];
  B.lists[2] = &w.jobs[2];
  int rc = build_phase(B, hw.seg1, hw.blk1, &w.seg1, &w.tile1, err, false);
  if (rc) return rc;
  rc = build_phase(B, hw.seg2, hw.blk2, &w.seg2, &w.tile2, err, true);
  if (rc) return rc;
  // Phase-1 outputs become phase-2 operands: when a phase-1 block feeds exactly
  // one unit-scaled pack job as its rows (row i = block columns i*rms ..
  // (i+1)*rms - 1, all block rows), the phase-1 tiles leave the row maxima
  // and the pack skips its own pass over the block.
  {
    std::unordered_map<int64_t, std::vector<int>> by_src;
    for (int j = 0; j < (int)w.jobs[2].size(); ++j)
      if (w.jobs[2][j].src_buf == kBufScratch) by_src[w.jobs[2][j].src].push_back(j);
    w.rowmax_base = w.exp_len;
    std::unordered_map<int64_t, std::pair<int64_t, int>> slots;  // block origin -> (slots, rms)
    for (const OutBlock& ob : hw.blk1) {
      auto it = by_src.find(ob.c);
      if (ob.c_buf != kBufScratch || it == by_src.end() || it->second.size() != 1) continue;
      PackJob& j = w.jobs[2][it->second[0]];
      if (j.alpha != 1.0 || j.ld_k != 1 || j.R <= 0 || ob.N % j.R != 0) continue;
      const int rms = ob.N / j.R;
      if (j.ld_r != (int64_t)ob.ldc * rms || j.K != ob.M * rms || ob.ldc != ob.M) continue;
      j.rowmax = w.exp_len;
      w.exp_len += j.R;
      slots[ob.c] = {j.rowmax, rms};
    }
    w.rowmax_len = w.exp_len - w.rowmax_base;
    for (OzTile& t : w.tile1) {
      auto it = slots.find(t.c);
      if (it == slots.end()) continue;
      t.rowmax = it->second.first;
      t.rms = it->second.second;
    }
  }
  split_phase2(w);
  const int grid = ozaki_persistent_grid();
  schedule_tiles(&w.tile1, w.seg1, grid);
  schedule_tiles(&w.tile2, w.seg2, grid);
  for (int c = 0; c < 3; ++c) {
    w.units[c].clear();
    w.max_nkt[c] = 0;
    w.rows_pass[c] = false;
    for (int j = 0; j < (int)w.jobs[c].size(); ++j) {
      w.max_nkt[c] = std::max(w.max_nkt[c], w.jobs[c][j].nkt);
      if (w.jobs[c][j].rowmax < 0) w.rows_pass[c] = true;
      for (int r = 0; r < w.jobs[c][j].nrt; ++r) w.units[c].push_back(Unit{j, r});
    }
  }
  return validate_ozaki_work(w, err);
}

int validate_ozaki_work(const OzWork& w, std::string* err) {
  for (int c = 0; c < 3; ++c)
    for (const PackJob& j : w.jobs[c]) {
      const int64_t bytes = (int64_t)j.nrt * j.nkt * w.S * j.rt * kKS * 2;
      if (j.dst < 0 || j.dst % 1024 || j.dst + bytes > w.packed_bytes || j.exp < 0 ||
          j.exp + (int64_t)j.nrt * j.rt > w.exp_len || j.texp < 0 || j.texp + j.nrt > w.exp_len ||
          (j.rowmax >= 0 && (j.rowmax < w.rowmax_base || j.rowmax + j.R > w.rowmax_base + w.rowmax_len)) || j.R <= 0 ||
          j.K <= 0 || (j.rt != kTM && j.rt != kTN)) {
        *err = "split mode: pack job out of bounds";
        return SU2G_EINVAL;
      }
    }
  auto check = [&](const std::vector<OzTile>& tiles, const std::vector<OzSeg>& segs) -> bool {
    for (const OzTile& t : tiles) {
      if (t.nseg == 0 && t.mlen == 0 && t.nlen == 0 && t.rowmax < 0) continue;  // schedule padding
      if (t.seg0 < 0 || t.nseg < 0 || t.seg0 + t.nseg > (int)segs.size() || t.mlen <= 0 || t.mlen > kTM ||
          t.nlen <= 0 || t.nlen > kTN || t.ldc < t.m0 + t.mlen)
        return false;
      if (t.rowmax >= 0 && (t.rms <= 0 || t.rowmax < w.rowmax_base ||
                            t.rowmax + (t.n0 + t.nlen - 1) / t.rms >= w.rowmax_base + w.rowmax_len))
        return false;
      for (int s = t.seg0; s < t.seg0 + t.nseg; ++s) {
        const OzSeg& z = segs[s];
        if (z.nks <= 0 || z.a_unit < 0 || z.b_unit < 0 ||
            z.a_unit + (int64_t)z.nks * a_unit_bytes(w.S) > w.packed_bytes ||
            z.b_unit + (int64_t)z.nks * b_unit_bytes(w.S) > w.packed_bytes || z.a_unit % 1024 || z.b_unit % 1024 ||
            z.a_exp < 0 || z.a_exp + kTM > w.exp_len || z.b_exp < 0 || z.b_exp + kTN > w.exp_len ||
            z.a_tmax < 0 || z.a_tmax >= w.exp_len)
          return false;
      }
    }
    return true;
  };
  if (!check(w.tile1, w.seg1) || !check(w.tile2, w.seg2)) {
    *err = "split mode: tile segment out of bounds";
    return SU2G_EINVAL;
  }
  const int64_t scratch_end = w.scratch_base + w.partial_len;
  for (const OzTile& t : w.tile2)
    if (t.c_buf == kBufScratch && (t.c < w.scratch_base || t.c + (int64_t)kTM * kTN > scratch_end)) {
      *err = "split mode: partial tile out of bounds";
      return SU2G_EINVAL;
    }
  for (const RedTile& r : w.red2)
    if (r.nparts < 2 || r.part < w.scratch_base || r.part + (int64_t)r.nparts * kTM * kTN > scratch_end ||
        r.mlen <= 0 || r.mlen > kTM || r.nlen <= 0 || r.nlen > kTN || r.ldc < r.m0 + r.mlen) {
      *err = "split mode: partial sum out of bounds";
      return SU2G_EINVAL;
    }
  return SU2G_OK;
}

}  // namespace oz
}  // namespace su2g
