// Cards, 7-card evaluation, combo space and the range parser.
//
// Drop-in semantics of the reference's src/cards.cpp:30-165 (evaluateN),
// src/range.cpp:10-251 (combo order, parser) and the strength key of
// cuda/gpu_cfr.cu:616-621. The evaluator here keeps one 13-bit rank mask
// per suit plus rank and suit counts, and finds straights with a
// shifted-AND run test. Its HandValue (category plus 5 tiebreak ranks)
// follows the reference's conventions exactly, because the compiler's
// strength order must match the reference bit for bit.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>

#include "cards.h"
#include "range.h"

namespace pps {

std::string cardName(Card c) {
  static const char kRanks[] = "23456789TJQKA";
  static const char kSuits[] = "cdhs";
  if (c >= kNumCards) return "??";
  return std::string{kRanks[rankOf(c)], kSuits[suitOf(c)]};
}

bool HandValue::operator<(const HandValue& o) const {
  if (category != o.category) return category < o.category;
  return tiebreak < o.tiebreak;  // lexicographic over the 5 ranks
}

bool HandValue::operator==(const HandValue& o) const {
  return category == o.category && tiebreak == o.tiebreak;
}

namespace {

// Highest straight in a 13-bit rank mask (ace plays low too); -1 if none.
// Returns the rank of the straight's top card.
int topOfStraight(unsigned mask) {
  const unsigned s = (mask << 1) | ((mask >> 12) & 1u);  // bit r+1 = rank r
  const unsigned run = s & (s >> 1) & (s >> 2) & (s >> 3) & (s >> 4);
  if (!run) return -1;
  const int low = 31 - __builtin_clz(run);  // lowest card of the top run
  return low + 3;                           // its top card, unshifted
}

// Fills v.tiebreak[from..] with the highest ranks of `mask`, skipping the
// ranks in `skip`, until `count` ranks are placed.
void fillKickers(HandValue& v, int from, int count, unsigned mask,
                 unsigned skip) {
  int slot = from;
  for (int r = 12; r >= 0 && slot < from + count; --r)
    if ((mask >> r) & 1u && !((skip >> r) & 1u)) v.tiebreak[slot++] = r;
}

}  // namespace

HandValue evaluateN(const Card* cards, int n) {
  // Counts keep multiplicity: the compiler also ranks combos that hold a
  // dealt card (they are blocked there, but the reference's strength
  // tables order them too, src/cards.cpp:33-44), so a repeated card must
  // count twice exactly as in the reference.
  unsigned suitMask[4] = {0, 0, 0, 0};
  int suitCount[4] = {0, 0, 0, 0};
  int rankCount[13] = {0};
  for (int i = 0; i < n; ++i) {
    suitMask[suitOf(cards[i])] |= 1u << rankOf(cards[i]);
    ++suitCount[suitOf(cards[i])];
    ++rankCount[rankOf(cards[i])];
  }
  const unsigned any = suitMask[0] | suitMask[1] | suitMask[2] | suitMask[3];

  HandValue v;
  for (int s = 0; s < 4; ++s) {
    if (suitCount[s] < 5) continue;
    const int sf = topOfStraight(suitMask[s]);
    if (sf >= 0) {
      v.category = 8;
      v.tiebreak[0] = sf;
    } else {
      v.category = 5;
      fillKickers(v, 0, 5, suitMask[s], 0);
    }
    return v;
  }

  int quad = -1, tripHi = -1, tripLo = -1;
  int pairRanks[4] = {-1, -1, -1, -1};
  int nPairs = 0;
  for (int r = 12; r >= 0; --r) {
    if (rankCount[r] == 4) {
      quad = r;
    } else if (rankCount[r] == 3) {
      if (tripHi < 0) tripHi = r;
      tripLo = r;
    } else if (rankCount[r] == 2 && nPairs < 4) {
      pairRanks[nPairs++] = r;
    }
  }
  if (tripLo == tripHi) tripLo = -1;

  if (quad >= 0) {
    v.category = 7;
    v.tiebreak[0] = quad;
    fillKickers(v, 1, 1, any, 1u << quad);
    return v;
  }
  if (tripHi >= 0 && (nPairs > 0 || tripLo >= 0)) {
    v.category = 6;
    v.tiebreak[0] = tripHi;
    v.tiebreak[1] = std::max(nPairs > 0 ? pairRanks[0] : -1, tripLo);
    return v;
  }
  const int st = topOfStraight(any);
  if (st >= 0) {
    v.category = 4;
    v.tiebreak[0] = st;
    return v;
  }
  if (tripHi >= 0) {
    v.category = 3;
    v.tiebreak[0] = tripHi;
    fillKickers(v, 1, 2, any, 1u << tripHi);
    return v;
  }
  if (nPairs >= 2) {
    v.category = 2;
    v.tiebreak[0] = pairRanks[0];
    v.tiebreak[1] = pairRanks[1];
    fillKickers(v, 2, 1, any, (1u << pairRanks[0]) | (1u << pairRanks[1]));
    return v;
  }
  if (nPairs == 1) {
    // One pair ranks by FOUR kickers in the reference (src/cards.cpp:
    // 145-151), one more than a 5-card hand plays; the strength order
    // (and so the showdown tie classes) must follow it to stay bit-exact.
    v.category = 1;
    v.tiebreak[0] = pairRanks[0];
    fillKickers(v, 1, 4, any, 1u << pairRanks[0]);
    return v;
  }
  // High card: slots a short rank set cannot fill stay -1, as in the
  // reference (only reachable with a repeated card).
  v.category = 0;
  v.tiebreak = {-1, -1, -1, -1, -1};
  unsigned singles = 0;
  for (int r = 0; r < 13; ++r)
    if (rankCount[r] > 0) singles |= 1u << r;
  fillKickers(v, 0, 5, singles, 0);
  return v;
}

HandValue evaluate7(const Card* cards) { return evaluateN(cards, 7); }

uint64_t handKey(const HandValue& v) {
  uint64_t key = (uint64_t)v.category;
  for (int i = 0; i < 5; ++i) key = key * 13 + (uint64_t)v.tiebreak[i];
  return key;
}

// ---------------------------------------------------------------------------
// Combo space: combo i <-> (a < b), ascending (a, b).
// ---------------------------------------------------------------------------

namespace {
int comboStart(int a) { return a * (103 - a) / 2; }  // first combo with card a
}  // namespace

void comboCards(int i, uint8_t& a, uint8_t& b) {
  int lo = 0;
  while (lo < 50 && comboStart(lo + 1) <= i) ++lo;
  a = (uint8_t)lo;
  b = (uint8_t)(i - comboStart(lo) + lo + 1);
}

int comboIndex(uint8_t a, uint8_t b) {
  if (a == b || a >= kNumCards || b >= kNumCards) return -1;
  if (a > b) std::swap(a, b);
  return comboStart(a) + (b - a - 1);
}

Range::Range() { std::fill(w, w + kCombos, 0.0); }

Range Range::ones() {
  Range r;
  std::fill(r.w, r.w + kCombos, 1.0);
  return r;
}

double Range::total() const {
  double s = 0.0;
  for (double x : w) s += x;
  return s;
}

void Range::normalize() {
  const double s = total();
  if (s > 0)
    for (double& x : w) x /= s;
}

void Range::filterBoard(const Card* board, int n) {
  uint64_t used = 0;
  for (int i = 0; i < n; ++i) used |= 1ull << board[i];
  for (int i = 0; i < kCombos; ++i) {
    uint8_t a, b;
    comboCards(i, a, b);
    if ((used >> a) & 1ull || (used >> b) & 1ull) w[i] = 0.0;
  }
}

int rankFromChar(char c) {
  static const char kRanks[] = "23456789TJQKA";
  for (int r = 0; r < 13; ++r)
    if (kRanks[r] == c) return r;
  return -1;
}

// ---------------------------------------------------------------------------
// Range parser (syntax of src/range.h:34-41, semantics of
// src/range.cpp:176-251): weights add up across tokens.
// ---------------------------------------------------------------------------

namespace {

struct HandClass {
  int hi = -1, lo = -1;
  char kind = 'p';  // 'p' pair, 's' suited, 'o' offsuit, 'a' suited+offsuit
  double weight = 1.0;
};

[[noreturn]] void badToken(const std::string& what, const std::string& tok) {
  throw std::runtime_error(what + ": " + tok);
}

HandClass parseHandClass(const std::string& token) {
  HandClass c;
  std::string t = token;
  const size_t colon = t.find(':');
  if (colon != std::string::npos) {
    const std::string ws = t.substr(colon + 1);
    char* end = nullptr;
    c.weight = std::strtod(ws.c_str(), &end);
    if (ws.empty() || end == ws.c_str()) badToken("bad range weight", token);
    t.resize(colon);
  }
  if (t.size() < 2) badToken("bad range token", token);
  const int r1 = rankFromChar(t[0]), r2 = rankFromChar(t[1]);
  if (r1 < 0 || r2 < 0) badToken("bad range token", token);
  c.hi = std::max(r1, r2);
  c.lo = std::min(r1, r2);
  if (t.size() == 2) {
    c.kind = r1 == r2 ? 'p' : 'a';
    return c;
  }
  if (t.size() == 3 && r1 != r2 && (t[2] == 's' || t[2] == 'o')) {
    c.kind = t[2];
    return c;
  }
  badToken("bad range token", token);
}

void addClass(Range& r, int hi, int lo, char kind, double weight) {
  auto add = [&](int a, int b) {
    if (a != b) r.w[comboIndex((uint8_t)a, (uint8_t)b)] += weight;
  };
  switch (kind) {
    case 'a':
      addClass(r, hi, lo, 's', weight);
      addClass(r, hi, lo, 'o', weight);
      break;
    case 'p':
      for (int s1 = 0; s1 < 4; ++s1)
        for (int s2 = s1 + 1; s2 < 4; ++s2) add(s1 * 13 + hi, s2 * 13 + hi);
      break;
    case 's':
      for (int s = 0; s < 4; ++s) add(s * 13 + hi, s * 13 + lo);
      break;
    default:  // offsuit
      for (int s1 = 0; s1 < 4; ++s1)
        for (int s2 = 0; s2 < 4; ++s2)
          if (s1 != s2) add(s1 * 13 + hi, s2 * 13 + lo);
  }
}

// The class sharing `c`'s gap whose top rank is `hi`.
void addSlid(Range& r, const HandClass& c, int hi) {
  if (c.kind == 'p') addClass(r, hi, hi, 'p', c.weight);
  else addClass(r, hi, hi - (c.hi - c.lo), c.kind, c.weight);
}

std::string trimmed(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && s[a] == ' ') ++a;
  while (b > a && s[b - 1] == ' ') --b;
  return s.substr(a, b - a);
}

}  // namespace

Range parseRange(const std::string& text) {
  Range r;
  size_t pos = 0;
  while (pos <= text.size()) {
    size_t comma = text.find(',', pos);
    if (comma == std::string::npos) comma = text.size();
    std::string tok = trimmed(text.substr(pos, comma - pos));
    pos = comma + 1;
    if (tok.empty()) continue;

    const bool plus = tok.back() == '+';
    if (plus) tok.pop_back();
    const size_t dash = tok.find('-');
    if (!plus && dash != std::string::npos) {
      const HandClass a = parseHandClass(tok.substr(0, dash));
      const HandClass b = parseHandClass(tok.substr(dash + 1));
      if (a.kind != b.kind) badToken("range dash mismatch", tok);
      if (a.hi - a.lo == b.hi - b.lo) {
        if (a.hi < b.hi) badToken("range must be descending", tok);
        for (int hi = b.hi; hi <= a.hi; ++hi) addSlid(r, a, hi);
      } else if (a.hi == b.hi) {
        if (a.lo < b.lo) badToken("range must be descending", tok);
        if (a.kind == 'p') badToken("pair dash needs same gap", tok);
        for (int lo = b.lo; lo <= a.lo; ++lo) addClass(r, a.hi, lo, a.kind, a.weight);
      } else {
        badToken("invalid range", tok);
      }
      continue;
    }
    const HandClass c = parseHandClass(tok);
    if (!plus) {
      addClass(r, c.hi, c.lo, c.kind, c.weight);
    } else if (c.hi - c.lo <= 1) {
      for (int hi = c.hi; hi <= 12; ++hi) addSlid(r, c, hi);
    } else {
      for (int lo = c.lo; lo < c.hi; ++lo) addClass(r, c.hi, lo, c.kind, c.weight);
    }
  }
  return r;
}

}  // namespace pps
