// Forest: many compiled spots resident on one GPU and iterated together.
//
// Each admitted spot's layout is relocated into shared pools (one device
// array per table kind, the base pointers the level kernels take), so one
// level launch covers that depth of every spot and one captured graph runs
// a DCFR iteration of all of them. Each spot keeps its own iteration
// counter (its slot, stored in node meta bits 16-31) and its own rows;
// nothing is shared between spots, so a spot's rows do not depend on which
// other spots are resident. Pool ranges are handed out first-fit and freed
// when a spot retires. Each pool is a fixed virtual address range: memory
// is mapped at its end when a range does not fit and unmapped when the top
// falls, so pools never move and growing never copies.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

#include "compiler.h"
#include "gpu_cfr.h"
#include "layout.h"

namespace pps {
namespace gb {

struct CompiledSpot {
  Tree tree;
  HostLayout layout;
  double pairMass = 0.0;  // Z of the value walks (both ranges, blockers)
  size_t bytes = 0;       // device bytes the spot occupies in a forest
};

// Compiles a spot for a forest (host only; throws Error).
std::unique_ptr<CompiledSpot> compileSpot(const gpu::PostflopSpot& spot,
                                          const gpu::StreetBetConfigs& cfgs, bool perStreet);
double pairMassOf(const Tree& t);

class Forest {
 public:
  // coef: the DCFR schedule, 3 floats (pos, neg, avg) per iteration index;
  // a spot runs at most coef.size() / 3 iterations. maxBytes bounds every
  // pool (each reserves that much address space up front).
  Forest(const std::vector<float>& coef, size_t maxBytes);
  ~Forest();
  Forest(const Forest&) = delete;
  Forest& operator=(const Forest&) = delete;

  // Places a compiled spot (rows zeroed, counter 0) and returns its slot,
  // taking ownership; returns -1 (spot untouched) when the forest's device
  // bytes would exceed `budget`.
  int admit(std::unique_ptr<CompiledSpot>& s, size_t budget);
  // Frees the spot's ranges and returns it (trim() gives the memory back).
  std::unique_ptr<CompiledSpot> retire(int slot);
  // Unmaps pool memory above the pools' tops (waits for queued work).
  void trim();
  std::vector<int> slots() const;  // resident slots, ascending
  const CompiledSpot& spot(int slot) const;
  int iterations(int slot) const;
  int maxIterations() const;

  // Enqueues n DCFR iterations of every resident spot.
  void iterate(int n);
  // Device time of the last iterate() (CUDA events; waits for it).
  double lastIterateMs();
  // One FP64 walk (kModeEV or kModeBR) of traverser tr over `slots`;
  // returns each spot's root value divided by its pair mass (chips).
  std::vector<double> walkValues(const std::vector<int>& slots, int tr, int mode);
  // The same values from an f32 walk (a screen: rounding of the f32 rows,
  // about 1e-6 of the values).
  std::vector<double> walkValuesF32(const std::vector<int>& slots, int tr, int mode);
  // Cumulative strategy rows of each spot's root decide node (na x n,
  // dense; empty where the root is not a decision), copied in one batch.
  std::vector<std::vector<float>> rootRows(const std::vector<int>& slots);
  void sync();

  size_t deviceBytes() const;  // pool capacity
  size_t usedBytes() const;    // sum of resident spots' footprints
  int captures() const;        // iteration graphs captured so far
  int launchesPerIteration() const;

  struct Dev;

 private:
  std::unique_ptr<Dev> d_;
  template <typename T>
  std::vector<double> walk(const std::vector<int>& slots, int tr, int mode);
};

}  // namespace gb
}  // namespace pps
