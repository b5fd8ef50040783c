#pragma once
// GB300-native heads-up postflop DCFR solver: C++ drop-in for the
// reference's cuda/gpu_cfr.h:35-264 (same namespace, types and method
// signatures), so reference callers such as tools/gpu_pfflop.cu and
// python/pps_native.cpp compile against this header unchanged.
//
// Behind it: a host tree compiler emitting flat node arrays and per-board
// tables, and hand-written sm_103a kernels run one DCFR iteration per CUDA
// graph replay. The class is a thin wrapper over the C ABI in pps_gb.h.
#include <cstdint>
#include <string>
#include <vector>

#include "postflop_cfr.h"
#include "range.h"

namespace pps {
namespace gpu {

struct PostflopSpot {
  Card board[5] = {0, 0, 0, 0, 0};
  int nBoard = 0;  // 3, 4 or 5
  Range oop;       // player 0, out of position
  Range ip;        // player 1, in position
  int64_t pot = 0;
  int64_t stack = 0;
};

// Per-street bet abstraction (extension; the reference has one BetConfig
// for every street). street[k] applies where the board has 3 + k cards.
struct StreetBetConfigs {
  pf::BetConfig street[3];
};

// One labeled action of a decide node: amount is the street-level total
// contribution for Bet/Raise/AllIn, 0 otherwise.
struct ActionLabel {
  pf::ActionKind kind = pf::ActionKind::Check;
  int64_t amount = 0;
};

struct DecideNodeInfo {
  int nodeId = 0;   // global tree index
  int player = 0;   // 0 = OOP, 1 = IP
  int depth = 0;
  int nBoard = 0;
  int nCombos = 0;  // the deciding player's combos here
  std::vector<ActionLabel> actions;
  std::vector<int> children;  // node id per action
};

// Per-combo average strategy of a decide node; freqs is action-major
// (freqs[a * combos.size() + c]); combos index the decider's base list.
struct ComboStrategy {
  std::vector<ActionLabel> actions;
  std::vector<int> combos;
  std::vector<double> freqs;
};

// Per-combo root EVs (chips) vs the average strategy; mass[p] is the
// opponent weight valid against each combo (the per-combo normalizer).
struct ComboEv {
  std::vector<int> combos[2];
  std::vector<double> ev[2];
  std::vector<double> mass[2];
};

// Node kinds: 0 decide, 1 showdown, 2 fold, 3 chance; CSR children; 5
// board card slots per node (0 where undealt).
struct TreeStructure {
  std::vector<uint8_t> kinds;
  std::vector<int> childBase;
  std::vector<int> children;
  std::vector<uint8_t> boards;
};

struct NodeEv {
  struct Side {
    std::vector<int> combos;
    std::vector<double> ev;
    std::vector<double> mass;
    double aggEv = 0.0;
  };
  struct ActionEv {
    std::vector<double> perCombo;
    double aggEv = 0.0;
  };
  int decider = 0;
  std::vector<ActionLabel> actions;
  std::vector<ActionEv> actionEv;
  Side side[2];
};

struct RunoutSummary {
  struct Branch {
    int card = 0;
    int nextDecide = -1;
    std::vector<double> freq;
    double aggEv[2] = {0.0, 0.0};
  };
  int decider = 0;
  std::vector<ActionLabel> actions;
  std::vector<Branch> branches;
};

class GpuPostflopSolver {
 public:
  // Compiles the spot (tree build + upload to the device).
  GpuPostflopSolver(const PostflopSpot& spot, const pf::BetConfig& cfg);
  // Extension: a separate bet abstraction per street.
  GpuPostflopSolver(const PostflopSpot& spot, const StreetBetConfigs& cfgs);
  // Loads a solution file written by save().
  explicit GpuPostflopSolver(const std::string& solutionPath);
  ~GpuPostflopSolver();
  GpuPostflopSolver(const GpuPostflopSolver&) = delete;
  GpuPostflopSolver& operator=(const GpuPostflopSolver&) = delete;

  // Up to `iterations` DCFR iterations ("dcfr", "hs30"; schedule variants
  // "dcfr-g2", "dcfr-noreset", "dcfr-g2-noreset"). target > 0 stops once
  // the exploitability (checked every 128 iterations) is <= target. A
  // fresh solve zeroes the rows and restarts the schedule.
  void solve(int iterations, const std::string& algo, double target = -1.0);
  // Continues a DCFR-family solve where it stopped.
  void continueSolve(int iterations, double target = -1.0);
  void reset();

  int iterationsRun() const { return iterationsRun_; }
  int64_t totalIterations() const { return totalIters_; }

  pf::NodeStats stats();
  std::vector<double> rootStrategy();
  std::vector<double> nodeStrategy(int decideIdx);
  int numDecideNodes() const;
  DecideNodeInfo decideNode(int decideIdx) const;
  ComboStrategy comboStrategy(int decideIdx);
  ComboEv rootEvPerCombo();
  NodeEv nodeEv(int decideIdx);
  RunoutSummary runoutSummary(int decideIdx, int actionIdx);
  std::vector<uint8_t> playerCards(int player) const;
  int numBaseCombos(int player) const;
  std::vector<double> playerWeights(int player) const;
  TreeStructure treeStructure() const;

  int numNodes() const { return numNodes_; }
  int maxDepth() const { return maxDepth_; }

  void save(const std::string& path) const;
  // Extension: the same file with compressed rows (16-bit codes, one scale
  // per action row); the path constructor reads both.
  void saveCompressed(const std::string& path) const;
  // Debug: non-finite counts of the regret and strategy rows (stderr).
  void debugDump();

  // The C-ABI handle (pps_gb_solver*) this object wraps.
  void* handle() const;

 private:
  struct Impl;
  Impl* impl_ = nullptr;
  int numNodes_ = 0;
  int maxDepth_ = 0;
  int iterationsRun_ = 0;
  int64_t totalIters_ = 0;
  void refresh();
};

}  // namespace gpu
}  // namespace pps
