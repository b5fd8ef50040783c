// Solver core behind the C ABI: one compiled spot, its device engine and
// the reference's solve / query / file semantics (cuda/gpu_cfr.cu:
// 1829-2853). Errors are thrown as gb::Error.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "compiler.h"
#include "engine.h"
#include "gpu_cfr.h"

namespace pps {
namespace gb {

// DCFR-family schedule: gamma 3 with the cumulative strategy reset at
// powers of 4 ("dcfr", the reference's, cuda/gpu_cfr.cu:598-610), its
// gamma-2 / no-reset variants, or HS-DCFR(30) ("hs30", 587-597).
struct Schedule {
  bool hs30 = false;
  double gamma = 3.0;
  bool resetPow4 = true;
  static bool parse(const std::string& algo, Schedule& out);
  // (pos, neg, avg) for iteration index t of a planned `iters`.
  void coefs(int t, int iters, double out[3]) const;
};

// Range-weighted average action frequencies of a decide node whose rows
// (na x nC, dense, cumulative strategy) belong to combos weighted w.
std::vector<double> aggregate(const std::vector<float>& rows, int na, int nC,
                              const std::vector<double>& w);

class SolverCore {
 public:
  SolverCore(const gpu::PostflopSpot& spot, const gpu::StreetBetConfigs& cfgs,
             bool perStreet);
  static std::unique_ptr<SolverCore> load(const std::string& path);

  void solve(int iterations, const std::string& algo, double target);
  void continueSolve(int iterations, double target);
  void reset();
  pf::NodeStats stats();
  std::vector<double> rootStrategy();
  std::vector<double> nodeStrategy(int decideIdx);
  gpu::DecideNodeInfo decideNode(int decideIdx) const;
  gpu::ComboStrategy comboStrategy(int decideIdx);
  gpu::ComboEv rootEvPerCombo();
  gpu::NodeEv nodeEv(int decideIdx);
  gpu::RunoutSummary runoutSummary(int decideIdx, int actionIdx);
  std::vector<uint8_t> playerCards(int player) const;
  int numBaseCombos(int player) const;
  std::vector<double> playerWeights(int player) const;
  gpu::TreeStructure treeStructure() const;
  // compressed: rows as 16-bit codes with per-action-row scales (file
  // versions 3 / 4); otherwise f32 rows (versions 1 / 2).
  void save(const std::string& path, bool compressed = false) const;
  void debugDump();
  // Benchmark helpers: n more iterations continuing the DCFR schedule
  // (CUDA-event timed / profiled launch by launch).
  double timeIterations(int n);
  void probeBoundedWait(int spins);
  std::vector<Engine::KernelStat> profile(int n, bool splitKinds);
  // Root value (chips) of one FP64 walk; fills the traverser's root row.
  double walkValue(int tr, int mode, std::vector<double>* rootRow);

  const Tree& tree() const { return tree_; }
  Engine* engine() { return eng_.get(); }
  int iterationsRun() const { return iterationsRun_; }
  int64_t totalIterations() const { return totalIters_; }
  bool empty() const { return tree_.empty; }

 private:
  Tree tree_;
  std::unique_ptr<Engine> eng_;
  int iterationsRun_ = 0;
  int64_t totalIters_ = 0;
  std::string lastAlgo_;
  Schedule sched_;

  double pairMass() const;
  void replayChunks(int iterations, double target);
  double explNow();
  void checkDecide(int decideIdx) const;
  void extendSchedule(int n);
  void requireEngine() const;
};

}  // namespace gb
}  // namespace pps
