// Bet abstraction: the action list of one betting state.
//
// Same integer semantics as the reference's pf::betActions
// (src/postflop_cfr.cpp:18-152), which mirrors postflop-solver's
// action_tree.rs: the node and action sets of the compiled tree must match
// the reference's exactly, so the rounding (llround), thresholds, sort
// orders and the 1e-12 merge epsilon are the same. Structure: candidate
// generation, clamp/force-all-in, canonical sort+unique, merge.
#include <algorithm>
#include <cmath>
#include <cstdint>

#include "postflop_cfr.h"

namespace pps {
namespace pf {

namespace {

int64_t roundChips(double x) { return (int64_t)std::llround(x); }

bool byKindThenAmount(const TreeAction& x, const TreeAction& y) {
  return x.kind != y.kind ? x.kind < y.kind : x.amount < y.amount;
}

bool isWager(ActionKind k) {
  return k == ActionKind::Bet || k == ActionKind::Raise ||
         k == ActionKind::AllIn;
}

}  // namespace

std::vector<TreeAction> betActions(int64_t potBase, int64_t stack,
                                   const BetConfig& cfg, int64_t sc0,
                                   int64_t sc1, int actor, bool afterAllin,
                                   int numBets, int numStreets) {
  const int64_t mine = actor == 0 ? sc0 : sc1;
  const int64_t theirs = actor == 0 ? sc1 : sc0;
  const int64_t prev = std::max(sc0, sc1);
  const int64_t toCall = theirs > mine ? theirs - mine : 0;
  // Pot after the actor calls: the base every size refers to.
  const int64_t pot = potBase + 2 * (mine + toCall);
  const int64_t theirLeft = stack - theirs;
  const int64_t cap = theirLeft + prev;  // all-in street total
  int64_t floorAmt = std::max<int64_t>(prev + toCall, 1);
  if (floorAmt > cap) floorAmt = cap;
  const bool mayWager = cfg.maxRaises <= 0 || numBets < cfg.maxRaises;

  std::vector<TreeAction> acts;
  if (toCall == 0) {
    acts.push_back({ActionKind::Check, 0});
    if (mayWager) {
      for (double f : cfg.betFracs)
        acts.push_back({ActionKind::Bet, roundChips(f * (double)pot)});
      if (cfg.betGeometric && numStreets > 0 && pot > 0) {
        const double spr = (double)theirLeft / (double)pot;
        const double ratio =
            (std::pow(2.0 * spr + 1.0, 1.0 / numStreets) - 1.0) / 2.0;
        acts.push_back({ActionKind::Bet, roundChips(ratio * (double)pot)});
      }
    }
    if (cfg.betAllIn || cap <= roundChips(cfg.addAllinThreshold * (double)pot))
      acts.push_back({ActionKind::AllIn, cap});
  } else {
    acts.push_back({ActionKind::Fold, 0});
    acts.push_back({ActionKind::Call, 0});
    if (!afterAllin) {
      if (mayWager)
        for (double m : cfg.raiseMults)
          acts.push_back({ActionKind::Raise, roundChips(m * (double)prev)});
      if (cap <= prev + roundChips(cfg.addAllinThreshold * (double)pot))
        acts.push_back({ActionKind::AllIn, cap});
    }
  }

  // Clamp sized wagers into [floor, cap]; a wager leaving less than the
  // force threshold of the resulting pot behind becomes the all-in.
  for (TreeAction& a : acts) {
    if (a.kind != ActionKind::Bet && a.kind != ActionKind::Raise) continue;
    const int64_t amt = std::min(std::max(a.amount, floorAmt), cap);
    const int64_t potAfter = pot + 2 * (amt - prev);
    if (cap <= amt + roundChips((double)potAfter * cfg.forceAllinThreshold))
      a = {ActionKind::AllIn, cap};
    else
      a.amount = amt;
  }

  std::sort(acts.begin(), acts.end(), byKindThenAmount);
  acts.erase(std::unique(acts.begin(), acts.end(),
                         [](const TreeAction& x, const TreeAction& y) {
                           return x.kind == y.kind && x.amount == y.amount;
                         }),
             acts.end());
  if (cfg.mergingThreshold <= 0) return acts;

  // Merge: walk the wagers from the largest down and keep one only when its
  // pot ratio is clearly below the last kept one's merge window.
  std::vector<TreeAction> passive, wagers;
  for (const TreeAction& a : acts) (isWager(a.kind) ? wagers : passive).push_back(a);
  std::sort(wagers.begin(), wagers.end(),
            [](const TreeAction& x, const TreeAction& y) {
              return x.amount != y.amount ? x.amount > y.amount : x.kind < y.kind;
            });
  const double mt = cfg.mergingThreshold;
  std::vector<TreeAction> kept;
  int64_t lastKept = INT64_MAX;
  for (const TreeAction& a : wagers) {
    const double ratio = (double)(a.amount - prev) / (double)pot;
    const double lastRatio = (double)(lastKept - prev) / (double)pot;
    const double window = (lastRatio - mt) / (1.0 + mt);
    if (ratio < window * (1.0 - 1e-12)) {
      kept.push_back(a);
      lastKept = a.amount;
    }
  }
  std::sort(passive.begin(), passive.end(), byKindThenAmount);
  std::vector<TreeAction> out(passive);
  out.insert(out.end(), kept.rbegin(), kept.rend());
  return out;
}

}  // namespace pf
}  // namespace pps
