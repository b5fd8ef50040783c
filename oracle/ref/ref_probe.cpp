// ref_probe: runs REFERENCE host functions on inputs read from stdin.
//
// TEST INFRASTRUCTURE ONLY (golden-fixture generator), built by
// oracle/ref/build_ref.sh into oracle/_ref/.
//
//   ref_probe eval   lines "c0 .. c6"  -> strength key per line: the
//                    reference evaluator (src/cards.cpp:30-165) packed as
//                    the reference engine packs it (cuda/gpu_cfr.cu:616-621)
//   ref_probe bet    lines "potBase stack sc0 sc1 actor afterAllin numBets
//                    numStreets allin geo maxRaises addT forceT mergeT nb nr
//                    b1..bnb r1..rnr" -> "n k0 a0 k1 a1 ..." from
//                    pf::betActions (src/postflop_cfr.cpp:18-152)
//   ref_probe range  lines "<range text>" -> 1326 weights from parseRange
//                    (src/range.cpp:176-251), or "ERR" if it throws
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "cards.h"
#include "postflop_cfr.h"
#include "range.h"

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: ref_probe eval|bet|range < input\n");
    return 2;
  }
  const std::string mode = argv[1];
  std::string line;
  while (std::getline(std::cin, line)) {
    if (mode == "eval") {
      int c[7];
      if (std::sscanf(line.c_str(), "%d %d %d %d %d %d %d", &c[0], &c[1],
                      &c[2], &c[3], &c[4], &c[5], &c[6]) != 7)
        continue;
      pps::Card cards[7];
      for (int i = 0; i < 7; ++i) cards[i] = (pps::Card)c[i];
      const pps::HandValue v = pps::evaluate7(cards);
      uint64_t key = (uint64_t)v.category;
      for (int i = 0; i < 5; ++i) key = key * 13 + (uint64_t)v.tiebreak[i];
      std::printf("%llu\n", (unsigned long long)key);
    } else if (mode == "bet") {
      long long potBase, stack, sc0, sc1;
      int actor, afterAllin, numBets, numStreets, allin, geo, maxRaises, nb, nr;
      double addT, forceT, mergeT;
      const char* p = line.c_str();
      int used = 0;
      if (std::sscanf(p, "%lld %lld %lld %lld %d %d %d %d %d %d %d %lf %lf %lf %d %d%n",
                      &potBase, &stack, &sc0, &sc1, &actor, &afterAllin,
                      &numBets, &numStreets, &allin, &geo, &maxRaises, &addT,
                      &forceT, &mergeT, &nb, &nr, &used) != 16)
        continue;
      p += used;
      pps::pf::BetConfig cfg;
      cfg.betFracs.clear();
      cfg.raiseMults.clear();
      for (int i = 0; i < nb + nr; ++i) {
        double x;
        std::sscanf(p, "%lf%n", &x, &used);
        p += used;
        (i < nb ? cfg.betFracs : cfg.raiseMults).push_back(x);
      }
      cfg.betAllIn = allin != 0;
      cfg.betGeometric = geo != 0;
      cfg.maxRaises = maxRaises;
      cfg.addAllinThreshold = addT;
      cfg.forceAllinThreshold = forceT;
      cfg.mergingThreshold = mergeT;
      const auto acts = pps::pf::betActions(potBase, stack, cfg, sc0, sc1,
                                            actor, afterAllin != 0, numBets,
                                            numStreets);
      std::printf("%zu", acts.size());
      for (const auto& a : acts)
        std::printf(" %d %lld", (int)a.kind, (long long)a.amount);
      std::printf("\n");
    } else if (mode == "range") {
      try {
        const pps::Range r = pps::parseRange(line);
        for (int i = 0; i < pps::kCombos; ++i)
          std::printf(i ? " %.17g" : "%.17g", r.w[i]);
        std::printf("\n");
      } catch (...) {
        std::printf("ERR\n");
      }
    }
  }
  return 0;
}
