// Host tree compiler: spot + bet abstraction -> flat tree.
//
// Node numbering, node fields and action sets are those of the reference
// compiler (cuda/gpu_cfr.cu:1116-1326: DFS pre-order, fold nodes created
// inline, dead-street rule, chance over the undealt cards). Internally the
// per-node combo lists are not copied per node: every node points at a
// BoardState (the spot board plus the cards dealt so far), and each state
// owns its two compact combo lists once. exportReference() re-derives the
// reference's own per-node layout for the bit-exact gate.
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "gpu_cfr.h"
#include "postflop_cfr.h"

namespace pps {
namespace gb {

enum NodeKind : uint8_t { kDecide = 0, kShowdown = 1, kFold = 2, kChance = 3 };
constexpr int kMaxActions = 32;

// Error raised by the compiler and engine; `code` is a PPS_GB_E_* value.
struct Error {
  int code;
  std::string msg;
};

struct Node {
  uint8_t kind = kDecide;
  uint8_t player = 0;   // decide: the actor
  uint8_t foldBy = 0;   // fold: who folded
  uint8_t na = 0;       // decide: actions; chance: 0 (see nChildren)
  int depth = 0;
  int parent = -1;
  int state = 0;        // BoardState index
  int childBase = 0;    // into Tree::children
  int nChildren = 0;
  int actBase = 0;      // decide: into Tree::actions
  int64_t potBase = 0, sc0 = 0, sc1 = 0, pc0 = 0, pc1 = 0;
};

struct BoardState {
  int parent = -1;  // state this one was dealt from (-1: the spot board)
  int dealt = -1;   // card dealt from the parent state
  int nBoard = 0;
  uint8_t board[5] = {0, 0, 0, 0, 0};
  std::vector<uint16_t> list[2];  // base combo slots alive here, ascending
  int riverIndex = -1;            // index among nBoard == 5 states
};

struct Side {
  int n = 0;
  std::vector<uint8_t> cards;   // 2 per base slot
  std::vector<double> w;        // base weights (positive)
  std::vector<int> sameOther;   // base slot -> identical slot on the other side
};

struct Tree {
  gpu::PostflopSpot spot;
  gpu::StreetBetConfigs cfgs;
  bool perStreet = false;
  bool empty = false;
  Side side[2];
  std::vector<Node> nodes;
  std::vector<int> children;
  std::vector<pf::TreeAction> actions;
  std::vector<BoardState> states;
  std::vector<int> decideNodes;  // decide node ids in node order
  int maxDepth = 0;
  int maxNa = 1;
  int64_t rowTotal = 0;          // reference regTotal: sum na * nTr

  int n(int node, int p) const {
    return (int)states[nodes[node].state].list[p].size();
  }
  const pf::BetConfig& cfgFor(int nBoard) const {
    return cfgs.street[nBoard - 3];
  }
};

// Throws Error (PPS_GB_E_ARG / PPS_GB_E_TOO_WIDE).
Tree compileTree(const gpu::PostflopSpot& spot,
                 const gpu::StreetBetConfigs& cfgs, bool perStreet);

// Strength key of every base combo of side p on a 5-card board.
std::vector<uint64_t> strengthKeys(const Tree& t, int p, const uint8_t b5[5]);

using ArraySink = std::function<void(const char* name, char dtype,
                                     const void* data, int64_t count)>;
// Emits the reference compiler's artifacts (names as in its Impl, cuda/
// gpu_cfr.cu:625-698) in the reference's own layout.
void exportReference(const Tree& t, const ArraySink& sink);

}  // namespace gb
}  // namespace pps
