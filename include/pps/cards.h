#pragma once
// Card representation and best-5 hand evaluation (drop-in for the
// reference's src/cards.h:1-38: same names, card ids and HandValue order).
//
// Card is uint8_t in [0, 52): suit = card / 13 (0..3 = c, d, h, s),
// rank = card % 13 (0 = deuce .. 12 = ace).
#include <array>
#include <cstdint>
#include <string>

namespace pps {

using Card = uint8_t;
constexpr int kNumCards = 52;

inline int rankOf(Card c) { return c % 13; }
inline int suitOf(Card c) { return c / 13; }

// Two-character text ("Ah", "Tc").
std::string cardName(Card c);

// Best-5 hand value from n cards (5 <= n <= 7). category: 8 straight
// flush, 7 quads, 6 full house, 5 flush, 4 straight, 3 trips, 2 two pair,
// 1 pair, 0 high card. tiebreak holds the deciding ranks, most significant
// first (unused trailing slots 0). Higher compares better; equal values
// split the pot.
struct HandValue {
  int category = 0;
  std::array<int, 5> tiebreak{};
  bool operator<(const HandValue& o) const;
  bool operator==(const HandValue& o) const;
};

HandValue evaluateN(const Card* cards, int n);
HandValue evaluate7(const Card* cards);

// Total-order strength key of a HandValue: category, then the 5 tiebreaks,
// packed base 13 (the sort key the reference compiler orders river combos
// by, cuda/gpu_cfr.cu:616-621).
uint64_t handKey(const HandValue& v);

}  // namespace pps
