#pragma once
// Weighted hand ranges over the 1326 hole-card combos (drop-in for the
// reference's src/range.h:1-46: same combo order, names and parser syntax).
#include <cstdint>
#include <string>

#include "cards.h"

namespace pps {

constexpr int kCombos = 1326;

// Combo i is the card pair (a < b); combos are enumerated in ascending
// (a, b) order: (0,1), (0,2), ..., (50,51).
void comboCards(int i, uint8_t& a, uint8_t& b);

// Index of the combo {a, b} (a != b), order-independent; -1 if a == b or
// either card is out of range.
int comboIndex(uint8_t a, uint8_t b);

struct Range {
  double w[kCombos];
  Range();              // all zeros
  static Range ones();  // every combo weight 1
  double total() const;
  void normalize();     // weights sum to 1 (no-op on an empty range)
  void filterBoard(const Card* board, int n);  // zero combos using a board card
};

// Parses the postflop-solver range syntax subset: pairs "TT", suited "AKs",
// offsuit "AKo", bare "AK" (both), "+" ranges ("TT+", "A9s+", "T9s+"),
// dash ranges ("55-22", "A5s-A2s", "KQo-JTo") and ":weight" suffixes.
// Throws std::runtime_error on anything else.
Range parseRange(const std::string& s);

// '2'..'9','T','J','Q','K','A' -> 0..12, else -1.
int rankFromChar(char c);

}  // namespace pps
