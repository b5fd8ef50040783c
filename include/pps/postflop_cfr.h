#pragma once
// Bet-tree abstraction (drop-in for the reference's src/postflop_cfr.h:1-63).
//
// betActions lists the actions of one betting state: pot-relative bets
// (sized on the call-inclusive pot), raises as multiples of the previous
// bet, an optional explicit all-in and geometric size, the min-raise floor,
// the add/force all-in thresholds and the merge of nearby sizes. The tree
// compiler passes the behind-stack remaining at the start of the street.
#include <cstdint>
#include <string>
#include <vector>

namespace pps {
namespace pf {

enum class ActionKind : uint8_t { Fold, Check, Call, Bet, Raise, AllIn };

struct TreeAction {
  ActionKind kind;
  int64_t amount = 0;  // street-level total contribution (Bet/Raise/AllIn)
};

struct BetConfig {
  // Bet sizes as fractions of the call-inclusive pot; raises as multiples
  // of the previous bet. betAllIn adds an all-in to every unopened street;
  // betGeometric adds the geometric size ((2*SPR+1)^(1/streets)-1)/2.
  std::vector<double> betFracs = {0.5, 0.75, 1.0};
  std::vector<double> raiseMults = {2.5, 3.0};
  bool betAllIn = false;
  bool betGeometric = false;
  // Max non-all-in bet/raise actions per street (0 = unlimited).
  int maxRaises = 0;
  double addAllinThreshold = 1.5;
  double forceAllinThreshold = 0.15;
  double mergingThreshold = 0.1;
};

// contributions (sc0, sc1) on the current street, potBase = the pot before
// this street's chips, stack = the behind-stack at the start of the street,
// numBets = bet/raise actions already made this street, numStreets = the
// streets left including this one (geometric sizing).
std::vector<TreeAction> betActions(int64_t potBase, int64_t stack,
                                   const BetConfig& cfg, int64_t sc0,
                                   int64_t sc1, int actor, bool afterAllin,
                                   int numBets = 0, int numStreets = 1);

// Result of a solve; values in chips. ev0 + ev1 is the starting pot.
struct NodeStats {
  double ev0 = 0.0;      // average-strategy value for OOP
  double ev1 = 0.0;      // average-strategy value for IP
  double expl = 0.0;     // exploitability: (BR0 + BR1 - pot) / 2
  int64_t pairMass = 0;  // disjoint weighted combo-pair mass x 2^20
};

}  // namespace pf
}  // namespace pps
