// gpu_pfflop: command-line driver with the reference CLI's protocol
// (tools/gpu_pfflop.cu:5-206), so the reference's gate and bench scripts
// can drive this solver unchanged.
//
//   gpu_pfflop postflop <board> <oop_range> <ip_range> <pot> <stack>
//             <bets> <raises> <iters> [--algo dcfr|hs30] [--root]
//             [--strat <decide_idx>] [--target <chips>] [--max-raises <n>]
//
// stdout: ROOTSTRAT / STRAT <i> (when asked), then EV 0, EV 1,
// EXPLOITABILITY. stderr: the reference's timing lines.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpu_cfr.h"
#include "postflop_cfr.h"
#include "range.h"

using namespace pps;

namespace {

// Card id of a rank and suit character (either case), -1 for a bad rank,
// -2 for a bad suit (the rank is checked first, as the reference does).
int cardOf(char r, char s) {
  const int rank = rankFromChar((char)std::toupper((unsigned char)r));
  if (rank < 0) return -1;
  const char* suits = "cdhs";
  const char* sp = s ? std::strchr(suits, std::tolower((unsigned char)s)) : nullptr;
  if (!sp) return -2;
  return (int)(sp - suits) * 13 + rank;
}

std::vector<std::string> split(const std::string& s) {
  std::vector<std::string> out;
  size_t a = 0;
  while (a <= s.size()) {
    size_t e = s.find(',', a);
    if (e == std::string::npos) e = s.size();
    if (e > a) out.push_back(s.substr(a, e - a));
    a = e + 1;
  }
  return out;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 10 || (std::strcmp(argv[1], "postflop") != 0 && std::strcmp(argv[1], "river") != 0)) {
    std::fprintf(stderr,
                 "usage: gpu_pfflop postflop <board> <oop_range> <ip_range> <pot> <stack> "
                 "<bets> <raises> <iters> [--algo dcfr|hs30] [--root] [--strat <decide_idx>] "
                 "[--target <chips>] [--max-raises <n>]\n"
                 "  board: 3, 4 or 5 cards (flop / turn / river)\n");
    return 2;
  }
  try {
    const std::string board = argv[2];
    if (board.size() != 6 && board.size() != 8 && board.size() != 10) {
      std::fprintf(stderr, "board must be 3, 4 or 5 cards\n");
      return 2;
    }
    gpu::PostflopSpot spot;
    spot.nBoard = (int)board.size() / 2;
    for (int i = 0; i < spot.nBoard; ++i) {
      const int c = cardOf(board[2 * i], board[2 * i + 1]);
      if (c < 0) {  // the reference's messages (tools/gpu_pfflop.cu:44, 52)
        if (c == -1) std::fprintf(stderr, "bad card rank '%c'\n", board[2 * i]);
        else std::fprintf(stderr, "bad card suit '%c'\n", board[2 * i + 1]);
        return 2;
      }
      spot.board[i] = (Card)c;
    }
    spot.oop = parseRange(argv[3]);
    spot.ip = parseRange(argv[4]);
    spot.pot = std::stoll(argv[5]);
    spot.stack = std::stoll(argv[6]);
    pf::BetConfig cfg;
    cfg.betFracs.clear();
    cfg.raiseMults.clear();
    for (const std::string& tok : split(argv[7])) {
      if (tok == "a" || tok == "A" || tok == "allin") cfg.betAllIn = true;
      else if (tok == "e" || tok == "E" || tok == "geo") cfg.betGeometric = true;
      else {
        try {
          cfg.betFracs.push_back(std::stod(tok));
        } catch (const std::exception&) {  // the reference's message and status
          std::fprintf(stderr, "bad bet sizes '%s' (use fractions and/or 'a')\n", argv[7]);
          return 2;
        }
      }
    }
    for (const std::string& tok : split(argv[8])) cfg.raiseMults.push_back(std::stod(tok));
    int iters = std::stoi(argv[9]);
    std::string algo = "dcfr";
    bool rootStrat = false;
    int stratNode = -1;
    double target = -1.0;
    for (int i = 10; i < argc; ++i) {
      if (!std::strcmp(argv[i], "--algo") && i + 1 < argc) algo = argv[++i];
      else if (!std::strcmp(argv[i], "--root")) rootStrat = true;
      else if (!std::strcmp(argv[i], "--target") && i + 1 < argc) {
        target = std::stod(argv[++i]);
        if (iters < 100000) iters = 100000;  // the target decides; iters is a cap
      } else if (!std::strcmp(argv[i], "--max-raises") && i + 1 < argc)
        cfg.maxRaises = std::atoi(argv[++i]);
      else if (!std::strcmp(argv[i], "--strat") && i + 1 < argc)
        stratNode = std::atoi(argv[++i]);
    }

    const auto w0 = std::chrono::steady_clock::now();
    gpu::GpuPostflopSolver solver(spot, cfg);
    const auto w1 = std::chrono::steady_clock::now();
    std::fprintf(stderr, "gpu_cfr: nodes=%d depth=%d board=%d cards\n", solver.numNodes(),
                 solver.maxDepth(), spot.nBoard);
    std::fprintf(stderr, "gpu_cfr: compile %.1f ms\n",
                 std::chrono::duration<double, std::milli>(w1 - w0).count());
    const auto s0 = std::chrono::steady_clock::now();
    solver.solve(iters, algo, target);
    const auto s1 = std::chrono::steady_clock::now();
    const double ms = std::chrono::duration<double, std::milli>(s1 - s0).count();
    std::fprintf(stderr, "gpu_cfr: %d iters in %.1f ms (%.0f iters/s)\n", solver.iterationsRun(),
                 ms, ms > 0 ? solver.iterationsRun() / (ms / 1000.0) : 0.0);
    if (target > 0.0)
      std::fprintf(stderr, "gpu_cfr: target %.4f reached at %d iters\n", target,
                   solver.iterationsRun());
    if (std::getenv("GPU_CFR_DEBUG")) solver.debugDump();
    const auto t0 = std::chrono::steady_clock::now();
    if (rootStrat) {
      std::printf("ROOTSTRAT");
      for (double f : solver.rootStrategy()) std::printf(" %.6f", f);
      std::printf("\n");
    }
    if (stratNode >= 0) {
      std::printf("STRAT %d", stratNode);
      for (double f : solver.nodeStrategy(stratNode)) std::printf(" %.6f", f);
      std::printf("\n");
    }
    const pf::NodeStats st = solver.stats();
    const auto t1 = std::chrono::steady_clock::now();
    std::fprintf(stderr, "gpu_cfr: stats walk %.1f ms\n",
                 std::chrono::duration<double, std::milli>(t1 - t0).count());
    std::printf("EV 0 %.6f\n", st.ev0);
    std::printf("EV 1 %.6f\n", st.ev1);
    std::printf("EXPLOITABILITY %.6f\n", st.expl);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "gpu_pfflop: %s\n", e.what());
    return 1;
  }
  return 0;
}
