// Launch shapes of the iteration graph and the autotuner's per-class cache.
//
// A launch shape picks how one DCFR iteration is launched: the plan (0:
// staged, terminal groups on side streams; 2: fused backward levels) and,
// for each kind of level launch, the grid: one CTA per task (cap 0), or a
// persistent grid of `cap` x SM-count CTAs that stride over the level's
// (spot, node-range) tasks. The kernels compute every task the same way in
// either form, so a shape changes timing only, never a row.
//
// Engine::autotune times candidate shapes on the tree and keeps the
// fastest; the choice is cached per tree-size class (widest combo list,
// size of the row table) in memory and, unless PPS_GB_TUNE_FILE is "off",
// in a small text file (PPS_GB_TUNE_FILE, else $XDG_CACHE_HOME or
// $HOME/.cache, file pps_gb/launch_shapes), so later solvers and processes
// of the same class skip the timing. Batches (forest.cu) take the cached
// shape of their class, or the default.
#pragma once

#include <cstdint>
#include <string>

namespace pps {
namespace gb {

struct LaunchShape {
  int plan = 0;    // 0 staged, 2 fused backward levels
  int fwdCap = 0;  // forward level grids: 0 one CTA per task, else cap x SMs
  int bwdCap = 0;  // backward level grids
  int sdCap = 0;   // showdown group grids
  int fdCap = 0;   // fold group grids
  bool operator==(const LaunchShape& o) const {
    return plan == o.plan && fwdCap == o.fwdCap && bwdCap == o.bwdCap && sdCap == o.sdCap &&
           fdCap == o.fdCap;
  }
};

// Tree-size class: the widest combo list (<= 511, <= 1023, wider: the
// terminal CTA width) and log2 of the row table's bytes.
struct TuneKey {
  int widthClass = 0;
  int sizeClass = 0;
};
TuneKey tuneKeyOf(int maxN, int64_t rowBytes);

bool lookupShape(const TuneKey& k, LaunchShape* out);
void storeShape(const TuneKey& k, const LaunchShape& s, double msPerIteration);
std::string shapeText(const LaunchShape& s);

// Grid of a launch with `count` tasks under a cap in SM multiples.
unsigned cappedGrid(unsigned grid, int capSms);

}  // namespace gb
}  // namespace pps
