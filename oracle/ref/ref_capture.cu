// ref_capture: runs the REFERENCE engine's own tree compiler on the host
// and dumps every integer artifact it produces.
//
// TEST INFRASTRUCTURE ONLY (golden-fixture generator). It is compiled by
// oracle/ref/build_ref.sh from the reference sources where they lie
// (cuda/gpu_cfr.cu, src/postflop_cfr.cpp, src/cards.cpp, src/range.cpp,
// src/common.cpp) and linked against oracle/ref/cuda_host_stub.cpp with
// `-cudart none`, so GpuPostflopSolver's constructor (cuda/gpu_cfr.cu:1829,
// init at 1331-1827) runs entirely in host memory. The reference's private
// Impl is opened with `#define private public` so its arrays can be read.
//
//   ref_capture <out.bin> <board> <oop> <ip> <pot> <stack> <bets> <raises>
//               <maxRaises>
//   ref_capture --save <out.pps> <iterations> <board> <oop> <ip> <pot> <stack>
//               <bets> <raises> <maxRaises>
//       the reference's own save() (cuda/gpu_cfr.cu:2743-2785) of the spot
//       with rows set to a fixed pattern (savePattern) and the iteration
//       count given: a "PPS1" version-1 solution file written by the
//       reference, for the file-format golden test
//   ref_capture --load <in.pps> <out.bin>
//       the reference's load constructor (cuda/gpu_cfr.cu:2787-2853) on a
//       solution file, dumping the rows and scalars it read back
//
// <oop>/<ip>: a range string (reference syntax, src/range.h:34-41) or
// "@path" to 1326 little-endian float64 combo weights.
// <bets>: comma list of pot fractions plus "a" (all-in) / "e" (geometric),
// parsed like tools/gpu_pfflop.cu:70-97.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#define private public
#include "gpu_cfr.h"
#undef private
#include "gpu_cfr.cu"

extern "C" size_t refStubAllocSize(const void* p);

using namespace pps;

namespace {

struct Dump {
  FILE* f = nullptr;
  uint32_t count = 0;
  long countPos = 0;
  explicit Dump(const char* path) {
    f = std::fopen(path, "wb");
    if (!f) {
      std::perror(path);
      std::exit(2);
    }
    std::fwrite("PPSDUMP1", 1, 8, f);
    countPos = std::ftell(f);
    std::fwrite(&count, 4, 1, f);
  }
  void raw(const char* name, char dtype, size_t elem, const void* p,
           uint64_t n) {
    uint16_t len = (uint16_t)std::strlen(name);
    std::fwrite(&len, 2, 1, f);
    std::fwrite(name, 1, len, f);
    std::fwrite(&dtype, 1, 1, f);
    std::fwrite(&n, 8, 1, f);
    if (n) std::fwrite(p, elem, n, f);
    ++count;
  }
  // A device block: its length comes from the stub's allocation table.
  template <typename T>
  void dev(const char* name, char dtype, const T* p) {
    const uint64_t n = p ? refStubAllocSize(p) / sizeof(T) : 0;
    raw(name, dtype, sizeof(T), p, n);
  }
  template <typename T>
  void vec(const char* name, char dtype, const std::vector<T>& v) {
    raw(name, dtype, sizeof(T), v.data(), v.size());
  }
  void scalar(const char* name, int64_t v) { raw(name, 'q', 8, &v, 1); }
  ~Dump() {
    std::fseek(f, countPos, SEEK_SET);
    std::fwrite(&count, 4, 1, f);
    std::fclose(f);
  }
};

Card cardFromText(const std::string& s, int i) {
  const char* ranks = "23456789TJQKA";
  const char* suits = "cdhs";
  const char* r = std::strchr(ranks, std::toupper(s[2 * i]));
  const char* su = std::strchr(suits, std::tolower(s[2 * i + 1]));
  if (!r || !su) {
    std::fprintf(stderr, "bad card in '%s'\n", s.c_str());
    std::exit(2);
  }
  return (Card)((su - suits) * 13 + (r - ranks));
}

Range rangeFromSpec(const std::string& spec) {
  if (!spec.empty() && spec[0] == '@') {
    Range r;
    FILE* f = std::fopen(spec.c_str() + 1, "rb");
    if (!f || std::fread(r.w, sizeof(double), kCombos, f) != (size_t)kCombos) {
      std::fprintf(stderr, "cannot read weights %s\n", spec.c_str() + 1);
      std::exit(2);
    }
    std::fclose(f);
    return r;
  }
  return parseRange(spec);
}

void parseBets(const std::string& s, pf::BetConfig& cfg) {
  size_t start = 0;
  while (start <= s.size()) {
    size_t end = s.find(',', start);
    std::string tok = end == std::string::npos ? s.substr(start)
                                               : s.substr(start, end - start);
    if (!tok.empty()) {
      if (tok == "a") cfg.betAllIn = true;
      else if (tok == "e") cfg.betGeometric = true;
      else cfg.betFracs.push_back(std::stod(tok));
    }
    if (end == std::string::npos) break;
    start = end + 1;
  }
}

std::vector<double> parseList(const std::string& s) {
  std::vector<double> out;
  size_t start = 0;
  while (start <= s.size()) {
    size_t end = s.find(',', start);
    std::string tok = end == std::string::npos ? s.substr(start)
                                               : s.substr(start, end - start);
    if (!tok.empty()) out.push_back(std::stod(tok));
    if (end == std::string::npos) break;
    start = end + 1;
  }
  return out;
}

}  // namespace

// Deterministic row contents for the file-format golden: regrets of both
// signs, strategy sums >= 0 (the test reproduces them from the index).
float savePattern(int which, uint32_t i) {
  if (which == 0) return (float)((int)((i * 2654435761u) % 20001u) - 10000) / 64.0f;
  return (float)((i * 40503u) % 1000u) / 8.0f;
}

int saveMode(int argc, char** argv) {
  // --save <out.pps> <iterations> <board> <oop> <ip> <pot> <stack> <bets> <raises> <maxRaises>
  if (argc != 12) return 2;
  gpu::PostflopSpot spot;
  const std::string board = argv[4];
  spot.nBoard = (int)board.size() / 2;
  for (int i = 0; i < spot.nBoard; ++i) spot.board[i] = cardFromText(board, i);
  spot.oop = rangeFromSpec(argv[5]);
  spot.ip = rangeFromSpec(argv[6]);
  spot.pot = std::stoll(argv[7]);
  spot.stack = std::stoll(argv[8]);
  pf::BetConfig cfg;
  cfg.betFracs.clear();
  parseBets(argv[9], cfg);
  cfg.raiseMults = parseList(argv[10]);
  cfg.maxRaises = std::atoi(argv[11]);
  gpu::GpuPostflopSolver solver(spot, cfg);
  auto* I = solver.impl_;
  for (size_t i = 0; i < I->regTotal; ++i) {
    I->dRegret[i] = savePattern(0, (uint32_t)i);
    I->dStrat[i] = savePattern(1, (uint32_t)i);
  }
  solver.totalIters_ = std::atoll(argv[3]);
  I->lastAlgo = "dcfr";
  solver.save(argv[2]);
  std::fprintf(stderr, "ref_capture --save: nodes=%d regTotal=%zu -> %s\n", I->numNodes,
               I->regTotal, argv[2]);
  return 0;
}

int loadMode(int argc, char** argv) {
  // --load <in.pps> <out.bin>
  if (argc != 4) return 2;
  gpu::GpuPostflopSolver solver{std::string(argv[2])};
  auto* I = solver.impl_;
  Dump d(argv[3]);
  d.scalar("numNodes", I->numNodes);
  d.scalar("regTotal", (int64_t)I->regTotal);
  d.scalar("totalIterations", (int64_t)solver.totalIters_);
  d.raw("regret", 'f', sizeof(float), I->dRegret, I->regTotal);
  d.raw("strat", 'f', sizeof(float), I->dStrat, I->regTotal);
  int counter = 0;
  std::memcpy(&counter, I->dCounter, sizeof(int));
  d.scalar("counter", counter);
  return 0;
}

// `ref_capture --treebuf`: the reference kernels' argument block, TreeBuf
// (cuda/gpu_cfr.cu:132-201), as "name offset" lines plus "sizeof N".
int printTreeBuf() {
  using TB = gpu::TreeBuf;
#define M(f) std::printf("%s %zu\n", #f, offsetof(TB, f));
  M(regret) M(regretRW) M(strat) M(stratRW) M(regOff) M(strOff) M(na) M(player)
  M(foldBy) M(childFlat) M(childBase) M(kind) M(boardId) M(nC0) M(nC1) M(comboOff0)
  M(comboOff1) M(comboId) M(reachOff) M(cfvOff) M(sc0) M(sc1) M(potBase) M(reach)
  M(reachRW) M(cfv) M(cfvRW) M(nBranch) M(chanceQ) M(pc0) M(pc1) M(runOffOff)
  M(runOff) M(ctap) M(ctapBase) M(expOffOff) M(expOff) M(expIdx) M(expIdxBase)
  M(cards0) M(cards1) M(sameOther0) M(sameOther1) M(brOppSortedOff) M(brOppSorted)
  M(brLessOff) M(brLessEnd) M(brTieEnd) M(brCardPosOff) M(brCardPosIdx)
  M(brRevSortedOff) M(brRevSorted) M(foldSonOff) M(foldSon) M(n0Base) M(n1Base) M(pot)
#undef M
  std::printf("sizeof %zu\n", sizeof(TB));
  return 0;
}

int main(int argc, char** argv) {
  if (argc == 2 && std::strcmp(argv[1], "--treebuf") == 0) return printTreeBuf();
  if (argc >= 2 && std::strcmp(argv[1], "--save") == 0) return saveMode(argc, argv);
  if (argc >= 2 && std::strcmp(argv[1], "--load") == 0) return loadMode(argc, argv);
  if (argc != 10) {
    std::fprintf(stderr,
                 "usage: ref_capture <out.bin> <board> <oop> <ip> <pot> "
                 "<stack> <bets> <raises> <maxRaises>\n");
    return 2;
  }
  const std::string board = argv[2];
  gpu::PostflopSpot spot;
  spot.nBoard = (int)board.size() / 2;
  for (int i = 0; i < spot.nBoard; ++i) spot.board[i] = cardFromText(board, i);
  spot.oop = rangeFromSpec(argv[3]);
  spot.ip = rangeFromSpec(argv[4]);
  spot.pot = std::stoll(argv[5]);
  spot.stack = std::stoll(argv[6]);
  pf::BetConfig cfg;
  cfg.betFracs.clear();
  parseBets(argv[7], cfg);
  cfg.raiseMults = parseList(argv[8]);
  cfg.maxRaises = std::atoi(argv[9]);

  auto t0 = std::chrono::steady_clock::now();
  gpu::GpuPostflopSolver solver(spot, cfg);
  auto t1 = std::chrono::steady_clock::now();
  auto* I = solver.impl_;
  std::fprintf(stderr, "ref_capture: nodes=%d depth=%d n0=%d n1=%d "
               "regTotal=%zu (%.1f ms)\n", I->numNodes, I->maxDepth,
               I->n0Base, I->n1Base, I->regTotal,
               std::chrono::duration<double, std::milli>(t1 - t0).count());

  Dump d(argv[1]);
  d.scalar("numNodes", I->numNodes);
  d.scalar("maxDepth", I->maxDepth);
  d.scalar("n0Base", I->n0Base);
  d.scalar("n1Base", I->n1Base);
  d.scalar("maxNa", I->maxNa);
  d.scalar("regTotal", (int64_t)I->regTotal);
  d.scalar("reachTotal", (int64_t)I->reachTotal);
  d.scalar("reachTotal0", (int64_t)I->reachTotal0);
  d.scalar("reachTotal1", (int64_t)I->reachTotal1);
  d.scalar("empty", I->empty ? 1 : 0);
  if (I->empty) return 0;

  d.dev("kind", 'i', I->dKind);
  d.dev("player", 'i', I->dPlayer);
  d.dev("foldBy", 'i', I->dFoldBy);
  d.dev("na", 'i', I->dNa);
  d.dev("childBase", 'i', I->dChildBase);
  d.dev("childFlat", 'i', I->dChildFlat);
  d.dev("boardId", 'i', I->dBoardId);
  d.dev("nC0", 'i', I->dNC0);
  d.dev("nC1", 'i', I->dNC1);
  d.dev("comboOff0", 'i', I->dComboOff0);
  d.dev("comboOff1", 'i', I->dComboOff1);
  d.dev("comboId", 'i', I->dComboId);
  d.dev("reachOff0", 'i', I->dReachOff0);
  d.dev("reachOff1", 'i', I->dReachOff1);
  d.dev("cfvOff", 'i', I->dCfvOff);
  d.dev("regOff", 'i', I->dRegOff);
  d.dev("sc0", 'q', I->dSc0);
  d.dev("sc1", 'q', I->dSc1);
  d.dev("potBase", 'q', I->dPotBase);
  d.dev("pc0", 'q', I->dPc0);
  d.dev("pc1", 'q', I->dPc1);
  d.dev("nBranch", 'i', I->dNBranch);
  d.dev("chanceQ", 'i', I->dChanceQ);
  d.dev("runOffOff", 'i', I->dRunOffOff);
  d.dev("runOff", 'i', I->dRunOff);
  d.dev("ctapBase", 'i', I->dCtapBase);
  d.dev("ctap", 'i', I->dCtap);
  d.dev("expOffOff", 'i', I->dExpOffOff);
  d.dev("expIdxBase", 'i', I->dExpIdxBase);
  d.dev("expOff", 'i', I->dExpOff);
  d.dev("expIdx", 'i', I->dExpIdx);
  d.dev("w0", 'f', I->dW0);
  d.dev("w1", 'f', I->dW1);
  d.dev("cards0", 'B', I->dCards0);
  d.dev("cards1", 'B', I->dCards1);
  d.dev("sameOther0", 'i', I->dSameOther0);
  d.dev("sameOther1", 'i', I->dSameOther1);
  d.dev("brOppSortedOff", 'i', I->dBrOppSortedOff);
  d.dev("brOppSorted", 'i', I->dBrOppSorted);
  d.dev("brLessOff", 'i', I->dBrLessOff);
  d.dev("brLessEnd", 'i', I->dBrLessEnd);
  d.dev("brTieEnd", 'i', I->dBrTieEnd);
  d.dev("brCardPosOff", 'i', I->dBrCardPosOff);
  d.dev("brCardPosIdx", 'i', I->dBrCardPosIdx);
  d.dev("brRevSortedOff", 'i', I->dBrRevSortedOff);
  d.dev("brRevSorted", 'i', I->dBrRevSorted);
  d.dev("foldSonOff", 'i', I->dFoldSonOff);
  d.dev("foldSon", 'i', I->dFoldSon);
  d.vec("w0d", 'd', I->w0);
  d.vec("w1d", 'd', I->w1);
  d.vec("nodeBoard", 'B', I->hNodeBoard);

  // Depth lists, flattened with per-depth counts.
  std::vector<int> decideFlat, chanceFlat, bwdFlat, brOffFlat;
  for (size_t dd = 0; dd < I->decideCount.size(); ++dd) {
    auto app = [](std::vector<int>& out, const int* p, int n) {
      for (int i = 0; i < n; ++i) out.push_back(p[i]);
    };
    app(decideFlat, I->dDecideList[dd], I->decideCount[dd]);
    app(chanceFlat, I->dChanceList[dd], I->chanceCount[dd]);
    app(bwdFlat, I->dBwdList[dd], I->bwdCount[dd]);
    app(brOffFlat, I->dChanceBrOff[dd], I->chanceCount[dd] + 1);
  }
  d.vec("decideCount", 'i', I->decideCount);
  d.vec("chanceCount", 'i', I->chanceCount);
  d.vec("bwdCount", 'i', I->bwdCount);
  d.vec("chanceBrTotal", 'i', I->chanceBrTotal);
  d.vec("decideList", 'i', decideFlat);
  d.vec("chanceList", 'i', chanceFlat);
  d.vec("bwdList", 'i', bwdFlat);
  d.vec("chanceBrOff", 'i', brOffFlat);

  std::vector<int> meta;
  for (const auto& m : I->decideMeta) {
    const int row[8] = {m.regOff, m.na, m.player, m.nC,
                        m.depth, m.nBoard, m.nodeId, m.actBase};
    meta.insert(meta.end(), row, row + 8);
  }
  d.vec("decideMeta", 'i', meta);
  std::vector<uint8_t> actKind;
  std::vector<int64_t> actAmount;
  for (const auto& a : I->actFlat) {
    actKind.push_back((uint8_t)a.kind);
    actAmount.push_back(a.amount);
  }
  d.vec("actKind", 'B', actKind);
  d.vec("actAmount", 'q', actAmount);
  return 0;
}
