// Device engine of one compiled spot: buffers, the per-iteration CUDA
// graph, and the FP64 value / best-response walks. Host-facing types only
// (no CUDA headers) so that plain C++ translation units can use it.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "compiler.h"
#include "layout.h"
#include "tune.h"

namespace pps {
namespace gb {

class Engine {
 public:
  Engine(const Tree& t, HostLayout&& layout);
  ~Engine();
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  // Zeroes regret and strategy rows and the iteration counter.
  void zeroRows();
  // Uploads the discount table (3 floats per iteration index, covering
  // [0, entries)) and sets the device iteration counter.
  void setSchedule(const std::vector<float>& coef, int counter);
  void setCounter(int counter);
  // Enqueues n iterations (graph replays); returns without waiting.
  void iterate(int n);
  void sync();
  void checkDeviceError();
  // Diagnostic of the bounded device waits: one warp waits on its barrier
  // for a copy that is never issued, `spins` polls a round; its give-up
  // path sets this engine's error word, and checkDeviceError throws.
  void probeBoundedWait(int spins);
  // Runs one FP64 walk (mode 1 = average-strategy EV, 2 = best response)
  // for traverser tr and waits for it; rows stay readable afterwards.
  void walk(int tr, int mode);
  // The same walk restricted to what node u's rows depend on: the forward
  // path from the root to u (each opponent decide ancestor's chunks, each
  // chance ancestor's branch toward u) and u's subtree (forward and
  // backward). u's rows and its descendants' come out exactly as after
  // walk(); other rows are stale. Node ids are DFS pre-order, so a subtree
  // is the id range [u, subtreeEnd(u)).
  void walkFrom(int tr, int mode, int u);
  // Rows of the last walk (double): the traverser's value row at `node`
  // (n_tr entries) and the opponent reach row of layout tr (n_opp entries).
  std::vector<double> walkCfv(int node, int tr) const;
  std::vector<double> walkReach(int node, int tr) const;
  // Regret (which = 0) or strategy (1) rows in the reference's dense
  // layout (decide nodes in node order, na x n, action-major).
  std::vector<float> denseRows(int which) const;
  void setDenseRows(int which, const std::vector<float>& dense);
  // The same rows as 16-bit codes (dense order) with one scale per action
  // row (rowcodec.h), coded and decoded on the device.
  void packRows(int which, std::vector<uint16_t>& codes, std::vector<float>& scales) const;
  void unpackRows(int which, const std::vector<uint16_t>& codes,
                  const std::vector<float>& scales);
  int64_t actionRows() const;
  // One decide node's strategy rows (na x n, dense).
  std::vector<float> nodeRows(int which, int node) const;

  // Benchmark helpers (see pps_gb_time_iterations / pps_gb_profile).
  double timeIterations(int n);
  struct KernelStat {
    std::string name;
    int64_t launches = 0;
    double ms = 0.0;
    double bytes = 0.0;
  };
  std::vector<KernelStat> profile(int n, bool splitKinds = false);
  int64_t h2dBytes() const { return h2d_; }
  int64_t d2hBytes() const { return d2h_; }

  // Selects the iteration graph's terminal kernels: 0 = groups of four
  // nodes of one level and board state (default); 1 = one CTA per node.
  // Recaptures on change.
  void setEngineKind(int kind);
  // Picks the faster of the staged (0) and fused (2) plans for this tree by
  // timing a few graph replays of each, then zeroes the rows and the
  // counter (both plans compute identical rows). A no-op once tuned, after
  // setEngineKind, and where the fused plan does not apply.
  void autotune();
  // Sets the launch shape (plan and level / group grids, tune.h) and turns
  // the autotuner off; recaptures.
  void setShape(const LaunchShape& s);
  LaunchShape shape() const;
  int engineKind() const { return engineKind_; }
  // Compensated (two-float) cumulative-strategy sums: the strategy rows get
  // a row of low words (allocated on first use, zeroed when turned on; the
  // current sums become their high words) and the update carries its
  // rounding errors there. Off by default; recaptures on change.
  void setCompensated(bool on);
  bool compensated() const { return comp_; }
  int launchesPerIteration() const { return launchesPerIter_; }
  size_t deviceBytes() const { return deviceBytes_; }
  // The stream every launch of this engine is issued on.
  void* stream() const;

  struct Dev;  // device-side state (engine.cu)

 private:
  const Tree& t_;
  HostLayout L_;
  std::unique_ptr<Dev> d_;
  int engineKind_ = 0;
  std::vector<int> subEnd_;  // per node: one past the last id of its subtree (walkFrom)
  bool tuned_ = false;
  bool comp_ = false;
  int launchesPerIter_ = 0;
  size_t deviceBytes_ = 0;
  mutable int64_t h2d_ = 0, d2h_ = 0;
  void capture();
  double timeShape(const LaunchShape& s, int n);
  void buildPlans();
  double taskBytes(int task, int tr, bool fwd) const;
  void ensureWalkBuffers();
};

}  // namespace gb
}  // namespace pps
