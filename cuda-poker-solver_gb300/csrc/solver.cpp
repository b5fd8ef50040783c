// Solver core (see solver.h). Solve loop, stats, queries and the "PPS1"
// solution file follow the reference's observable behaviour
// (cuda/gpu_cfr.cu:1829-2853); the compute runs in the Engine.
#include "solver.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>

#include "pps_gb.h"

namespace pps {
namespace gb {

// ---------------------------------------------------------------------------
// Schedule.
// ---------------------------------------------------------------------------

bool Schedule::parse(const std::string& algo, Schedule& out) {
  Schedule s;
  if (algo == "hs30") s.hs30 = true;
  else if (algo == "dcfr") {}
  else if (algo == "dcfr-g2") s.gamma = 2.0;
  else if (algo == "dcfr-noreset") s.resetPow4 = false;
  else if (algo == "dcfr-g2-noreset") { s.gamma = 2.0; s.resetPow4 = false; }
  else return false;
  out = s;
  return true;
}

void Schedule::coefs(int t, int iters, double out[3]) const {
  if (hs30) {
    // HS-DCFR(30): alpha = 1 + 3t/n, beta = -1 - 2t/n, gamma = 30 - 5t/n
    // with t counted from 1 (arXiv 2404.09097, eq. 4).
    const double n = (double)iters, tt = (double)(t + 1);
    const double pa = std::pow(tt, 1.0 + 3.0 * tt / n);
    const double pb = std::pow(tt, -1.0 - 2.0 * tt / n);
    out[0] = pa / (pa + 1.0);
    out[1] = pb / (pb + 1.0);
    out[2] = std::pow(tt / (tt + 1.0), 30.0 - 5.0 * tt / n);
    return;
  }
  // DCFR: positive regrets weighted ta^1.5 / (ta^1.5 + 1) with ta = t - 1,
  // negative regrets halved, the average strategy weighted ((t-k)/(t-k+1))^
  // gamma where k is the largest power of 4 <= t (0 without the reset).
  const double ta = (double)std::max(t - 1, 0);
  const double pa = ta * std::sqrt(ta);
  int k = 0;
  if (resetPow4 && t > 0) {
    k = 1;
    while ((int64_t)k * 4 <= t) k *= 4;
  }
  const double tg = (double)(t - k);
  out[0] = pa / (pa + 1.0);
  out[1] = 0.5;
  out[2] = std::pow(tg / (tg + 1.0), gamma);
}

// ---------------------------------------------------------------------------
// Construction and the solve loop.
// ---------------------------------------------------------------------------

SolverCore::SolverCore(const gpu::PostflopSpot& spot,
                       const gpu::StreetBetConfigs& cfgs, bool perStreet)
    : tree_(compileTree(spot, cfgs, perStreet)) {
  if (!tree_.empty) eng_.reset(new Engine(tree_, buildLayout(tree_)));
}

void SolverCore::requireEngine() const {
  if (!eng_) throw Error{PPS_GB_E_STATE, "solver compiled to empty ranges"};
}

void SolverCore::checkDecide(int decideIdx) const {
  if (decideIdx < 0 || decideIdx >= (int)tree_.decideNodes.size())
    throw Error{PPS_GB_E_INDEX, "decide node index " + std::to_string(decideIdx) +
                                    " out of range (" +
                                    std::to_string(tree_.decideNodes.size()) +
                                    " decide nodes)"};
}

void SolverCore::reset() {
  iterationsRun_ = 0;
  totalIters_ = 0;
  if (eng_) eng_->zeroRows();
}

void SolverCore::replayChunks(int iterations, double target) {
  const int chunk = 128;
  int done = 0;
  while (done < iterations) {
    const int n = std::min(chunk, iterations - done);
    eng_->iterate(n);
    done += n;
    iterationsRun_ = done;
    totalIters_ += n;
    if (target > 0.0 && done < iterations && explNow() <= target) break;
  }
  eng_->sync();
}

void SolverCore::solve(int iterations, const std::string& algo, double target) {
  iterationsRun_ = 0;
  if (tree_.empty) return;
  Schedule s;
  if (!Schedule::parse(algo, s))
    throw Error{PPS_GB_E_ARG, "unknown algo '" + algo + "' (expected dcfr or hs30)"};
  reset();
  if (iterations <= 0) return;
  lastAlgo_ = algo;
  sched_ = s;
  std::vector<float> tab((size_t)iterations * 3);
  for (int t = 0; t < iterations; ++t) {
    double c[3];
    s.coefs(t, iterations, c);
    for (int k = 0; k < 3; ++k) tab[(size_t)t * 3 + k] = (float)c[k];
  }
  eng_->setSchedule(tab, 0);
  if (iterations >= 32) eng_->autotune();
  replayChunks(iterations, target);
}

void SolverCore::continueSolve(int iterations, double target) {
  iterationsRun_ = 0;
  if (tree_.empty) return;
  if (totalIters_ == 0)
    throw Error{PPS_GB_E_STATE, "continueSolve: no prior solve() to continue"};
  if (sched_.hs30)
    throw Error{PPS_GB_E_STATE,
                "continueSolve: the last solve used '" + lastAlgo_ +
                    "', whose schedule depends on the planned iteration count; "
                    "continuation is defined for DCFR only"};
  if (iterations <= 0) return;
  const int64_t t0 = totalIters_, tEnd = t0 + iterations;
  if (tEnd > (int64_t)std::numeric_limits<int>::max())
    throw Error{PPS_GB_E_ARG, "continueSolve: schedule index overflow"};
  // The device indexes the table by the absolute iteration counter, so it
  // spans [0, t0 + n); entries below t0 are never read again.
  std::vector<float> tab((size_t)tEnd * 3);
  double c0[3];
  sched_.coefs((int)t0, (int)tEnd, c0);
  for (int64_t t = 0; t < tEnd; ++t) {
    double c[3];
    if (t < t0) std::memcpy(c, c0, sizeof(c));
    else sched_.coefs((int)t, (int)tEnd, c);
    for (int k = 0; k < 3; ++k) tab[(size_t)t * 3 + k] = (float)c[k];
  }
  eng_->setSchedule(tab, (int)t0);
  replayChunks(iterations, target);
}

// Makes the device schedule cover the next n iterations (benchmarks run
// past a planned solve; DCFR needs only the absolute index).
void SolverCore::extendSchedule(int n) {
  requireEngine();
  if (lastAlgo_.empty() || sched_.hs30) {
    lastAlgo_ = "dcfr";
    sched_ = Schedule{};
  }
  const int64_t t0 = totalIters_, tEnd = t0 + n;
  if (tEnd > (int64_t)std::numeric_limits<int>::max())
    throw Error{PPS_GB_E_ARG, "schedule index overflow"};
  std::vector<float> tab((size_t)tEnd * 3);
  for (int64_t t = 0; t < tEnd; ++t) {
    double c[3];
    sched_.coefs((int)t, (int)tEnd, c);
    for (int k = 0; k < 3; ++k) tab[(size_t)t * 3 + k] = (float)c[k];
  }
  eng_->setSchedule(tab, (int)t0);
}

void SolverCore::probeBoundedWait(int spins) { eng_->probeBoundedWait(spins); }

double SolverCore::timeIterations(int n) {
  extendSchedule(n);
  const double ms = eng_->timeIterations(n);
  totalIters_ += n;
  iterationsRun_ = n;
  return ms;
}

std::vector<Engine::KernelStat> SolverCore::profile(int n, bool splitKinds) {
  extendSchedule(n);
  auto out = eng_->profile(n, splitKinds);
  totalIters_ += n;
  iterationsRun_ = n;
  return out;
}

// ---------------------------------------------------------------------------
// Walks and stats.
// ---------------------------------------------------------------------------

double SolverCore::pairMass() const {
  const Side& s0 = tree_.side[0];
  const Side& s1 = tree_.side[1];
  double total1 = 0.0, cardSum[52] = {0.0};
  for (int j = 0; j < s1.n; ++j) {
    total1 += s1.w[j];
    cardSum[s1.cards[2 * j]] += s1.w[j];
    cardSum[s1.cards[2 * j + 1]] += s1.w[j];
  }
  double Z = 0.0;
  for (int i = 0; i < s0.n; ++i) {
    double w = total1 - cardSum[s0.cards[2 * i]] - cardSum[s0.cards[2 * i + 1]];
    if (s0.sameOther[i] >= 0) w += s1.w[s0.sameOther[i]];
    if (w > 0.0) Z += s0.w[i] * w;
  }
  return Z;
}

double SolverCore::walkValue(int tr, int mode, std::vector<double>* rootRow) {
  requireEngine();
  eng_->walk(tr, mode);
  std::vector<double> cfv = eng_->walkCfv(0, tr);
  double v = 0.0;
  for (size_t i = 0; i < cfv.size(); ++i) v += tree_.side[tr].w[i] * cfv[i];
  if (rootRow) *rootRow = cfv;
  const double Z = pairMass();
  return Z > 0.0 ? v / Z : 0.0;
}

double SolverCore::explNow() {
  const double v0 = walkValue(0, kModeBR, nullptr);
  const double v1 = walkValue(1, kModeBR, nullptr);
  return (v0 + v1 - (double)tree_.spot.pot) / 2.0;
}

pf::NodeStats SolverCore::stats() {
  pf::NodeStats st{};
  if (tree_.empty) return st;
  const double Z = pairMass();
  if (Z <= 0.0) return st;
  // Debug hook of the reference (cuda/gpu_cfr.cu:2066-2097): seed the
  // average-strategy rows with a fixed profile to check the value walk
  // against known answers. Modes select which decide nodes are seeded.
  if (const char* sm = std::getenv("GPU_CFR_SEED_STRAT")) {
    const int mode = std::atoi(sm);
    std::vector<float> rows((size_t)tree_.rowTotal, 0.0f);
    size_t off = 0;
    for (size_t mi = 0; mi < tree_.decideNodes.size(); ++mi) {
      const Node& nd = tree_.nodes[tree_.decideNodes[mi]];
      const int nC = tree_.n(tree_.decideNodes[mi], nd.player);
      const size_t base = off;
      off += (size_t)nd.na * nC;
      const bool turnNode = nd.depth <= 2;
      bool seed = nd.na >= 2;
      switch (mode) {
        case 2: seed &= turnNode; break;
        case 3: seed &= !turnNode; break;
        case 4: seed &= nd.depth == 0; break;
        case 5: seed &= nd.depth == 1; break;
        case 6: seed &= nd.depth == 2; break;
        case 7: seed &= mi == 1; break;
        case 8: seed &= mi == 2; break;
        case 9: seed &= nd.depth == 1 && mi != 1; break;
        default: break;
      }
      if (!seed) continue;
      for (int c = 0; c < nC; ++c) {
        const float p0 = (float)(0.15 + 0.7 * ((c % 8) / 7.0));
        rows[base + c] = p0;
        rows[base + (size_t)nC + c] = 1.0f - p0;
      }
    }
    eng_->setDenseRows(1, rows);
    std::fprintf(stderr, "seeded strat rows (mode %d)\n", mode);
  }
  st.ev0 = walkValue(0, kModeEV, nullptr);
  st.ev1 = walkValue(1, kModeEV, nullptr);
  const double v0 = walkValue(0, kModeBR, nullptr);
  const double v1 = walkValue(1, kModeBR, nullptr);
  st.expl = (v0 + v1 - (double)tree_.spot.pot) / 2.0;
  st.pairMass = (int64_t)(Z * (double)(1LL << 20));
  return st;
}

// ---------------------------------------------------------------------------
// Strategy queries.
// ---------------------------------------------------------------------------

// Range-weighted average frequencies over a first-street node's rows.
std::vector<double> aggregate(const std::vector<float>& rows, int na, int nC,
                              const std::vector<double>& w) {
  std::vector<double> freq(na, 0.0), tot(nC, 0.0);
  double z = 0.0;
  for (int c = 0; c < nC; ++c) {
    for (int a = 0; a < na; ++a) tot[c] += rows[(size_t)a * nC + c];
    z += w[c];
  }
  if (z <= 0.0) return freq;
  const double uniform = 1.0 / na;
  for (int a = 0; a < na; ++a) {
    double acc = 0.0;
    for (int c = 0; c < nC; ++c)
      acc += w[c] * (tot[c] > 0.0 ? rows[(size_t)a * nC + c] / tot[c] : uniform);
    freq[a] = acc / z;
  }
  return freq;
}

namespace {

gpu::ActionLabel label(const pf::TreeAction& a) { return {a.kind, a.amount}; }

int slotIn(const std::vector<uint16_t>& list, int base) {
  auto it = std::lower_bound(list.begin(), list.end(), (uint16_t)base);
  return it != list.end() && *it == base ? (int)(it - list.begin()) : -1;
}

}  // namespace

std::vector<double> SolverCore::rootStrategy() {
  if (tree_.empty) return {};
  const Node& root = tree_.nodes[0];
  return aggregate(eng_->nodeRows(1, 0), root.na, tree_.n(0, 0), tree_.side[0].w);
}

std::vector<double> SolverCore::nodeStrategy(int decideIdx) {
  if (tree_.empty || decideIdx < 0 || decideIdx >= (int)tree_.decideNodes.size())
    return {};
  const int u = tree_.decideNodes[decideIdx];
  const Node& nd = tree_.nodes[u];
  // Only first-street nodes carry the base lists, where the range weights
  // are the exact reach weights.
  if (tree_.states[nd.state].nBoard != tree_.spot.nBoard) return {};
  return aggregate(eng_->nodeRows(1, u), nd.na, tree_.n(u, nd.player),
                   tree_.side[nd.player].w);
}

gpu::DecideNodeInfo SolverCore::decideNode(int decideIdx) const {
  checkDecide(decideIdx);
  const int u = tree_.decideNodes[decideIdx];
  const Node& nd = tree_.nodes[u];
  gpu::DecideNodeInfo out;
  out.nodeId = u;
  out.player = nd.player;
  out.depth = nd.depth;
  out.nBoard = tree_.states[nd.state].nBoard;
  out.nCombos = tree_.n(u, nd.player);
  for (int a = 0; a < nd.na; ++a) {
    out.actions.push_back(label(tree_.actions[nd.actBase + a]));
    out.children.push_back(tree_.children[nd.childBase + a]);
  }
  return out;
}

gpu::ComboStrategy SolverCore::comboStrategy(int decideIdx) {
  requireEngine();
  checkDecide(decideIdx);
  const int u = tree_.decideNodes[decideIdx];
  const Node& nd = tree_.nodes[u];
  const auto& list = tree_.states[nd.state].list[nd.player];
  const int nC = (int)list.size(), na = nd.na;
  gpu::ComboStrategy out;
  for (int a = 0; a < na; ++a) out.actions.push_back(label(tree_.actions[nd.actBase + a]));
  out.combos.assign(list.begin(), list.end());
  const std::vector<float> rows = eng_->nodeRows(1, u);
  out.freqs.assign((size_t)na * nC, 0.0);
  const double uniform = na > 0 ? 1.0 / na : 0.0;
  for (int c = 0; c < nC; ++c) {
    double s = 0.0;
    for (int a = 0; a < na; ++a) s += rows[(size_t)a * nC + c];
    for (int a = 0; a < na; ++a)
      out.freqs[(size_t)a * nC + c] = s > 0.0 ? (double)rows[(size_t)a * nC + c] / s : uniform;
  }
  return out;
}

// ---------------------------------------------------------------------------
// Value queries (one FP64 EV walk per player; cuda/gpu_cfr.cu:2185-2684).
// ---------------------------------------------------------------------------

gpu::ComboEv SolverCore::rootEvPerCombo() {
  gpu::ComboEv out;
  if (tree_.empty) return out;
  for (int tr = 0; tr < 2; ++tr) {
    eng_->walk(tr, kModeEV);
    const std::vector<double> cfv = eng_->walkCfv(0, tr);
    const Side& self = tree_.side[tr];
    const Side& opp = tree_.side[1 - tr];
    double cardSum[52] = {0.0}, totalOpp = 0.0;
    for (int j = 0; j < opp.n; ++j) {
      totalOpp += opp.w[j];
      cardSum[opp.cards[2 * j]] += opp.w[j];
      cardSum[opp.cards[2 * j + 1]] += opp.w[j];
    }
    const int n = self.n;
    out.combos[tr].resize(n);
    out.ev[tr].resize(n);
    out.mass[tr].resize(n);
    for (int i = 0; i < n; ++i) {
      out.combos[tr][i] = i;
      double mass = totalOpp - cardSum[self.cards[2 * i]] - cardSum[self.cards[2 * i + 1]];
      if (self.sameOther[i] >= 0) mass += opp.w[self.sameOther[i]];
      out.mass[tr][i] = mass;
      out.ev[tr][i] = mass > 0.0 ? cfv[i] / mass : 0.0;
    }
  }
  return out;
}

gpu::NodeEv SolverCore::nodeEv(int decideIdx) {
  requireEngine();
  checkDecide(decideIdx);
  const int u = tree_.decideNodes[decideIdx];
  const Node& nd = tree_.nodes[u];
  const BoardState& st = tree_.states[nd.state];
  const int na = nd.na, dec = nd.player;
  gpu::NodeEv out;
  out.decider = dec;
  for (int a = 0; a < na; ++a) out.actions.push_back(label(tree_.actions[nd.actBase + a]));
  out.actionEv.assign(na, {});
  const std::vector<float> srows = eng_->nodeRows(1, u);

  for (int tr = 0; tr < 2; ++tr) {
    eng_->walkFrom(tr, kModeEV, u);  // rows of u and its children
    gpu::NodeEv::Side& S = out.side[tr];
    const auto& list = st.list[tr];
    const auto& olist = st.list[1 - tr];
    const int nC = (int)list.size();
    S.combos.assign(list.begin(), list.end());
    S.ev.assign(nC, 0.0);
    S.mass.assign(nC, 0.0);
    const Side& self = tree_.side[tr];
    const Side& opp = tree_.side[1 - tr];
    // Opponent reach at u (layout tr) -> per-combo mass with the same card
    // removal as the terminal kernels.
    const std::vector<double> reach = eng_->walkReach(u, tr);
    double cardSum[52] = {0.0}, tot = 0.0;
    for (size_t j = 0; j < olist.size(); ++j) {
      tot += reach[j];
      cardSum[opp.cards[2 * olist[j]]] += reach[j];
      cardSum[opp.cards[2 * olist[j] + 1]] += reach[j];
    }
    for (int i = 0; i < nC; ++i) {
      const int b = list[i];
      double mass = tot - cardSum[self.cards[2 * b]] - cardSum[self.cards[2 * b + 1]];
      const int so = self.sameOther[b];
      if (so >= 0) {
        const int slot = slotIn(olist, so);
        if (slot >= 0) mass += reach[slot];
      }
      S.mass[i] = mass;
    }
    const std::vector<double> row = eng_->walkCfv(u, tr);
    for (int i = 0; i < nC; ++i) S.ev[i] = S.mass[i] > 0.0 ? row[i] / S.mass[i] : 0.0;

    if (tr == dec) {
      for (int a = 0; a < na; ++a) {
        const int ch = tree_.children[nd.childBase + a];
        const bool chance = tree_.nodes[ch].kind == kChance;
        const auto& clist = tree_.states[tree_.nodes[ch].state].list[tr];
        const std::vector<double> crow = eng_->walkCfv(ch, tr);
        auto& pc = out.actionEv[a].perCombo;
        pc.assign(nC, 0.0);
        for (int i = 0; i < nC; ++i) {
          if (S.mass[i] <= 0.0) continue;
          const int slot = chance ? slotIn(clist, S.combos[i]) : i;
          if (slot >= 0) pc[i] = crow[slot] / S.mass[i];
        }
        double num = 0, den = 0, num0 = 0, den0 = 0;
        for (int i = 0; i < nC; ++i) {
          const double mass = S.mass[i];
          if (mass <= 0.0) continue;
          double s = 0.0;
          for (int a2 = 0; a2 < na; ++a2) s += srows[(size_t)a2 * nC + i];
          const double wb = self.w[S.combos[i]] * mass;
          num0 += wb * pc[i];
          den0 += wb;
          if (s <= 0.0) continue;
          const double wt = wb * (double)srows[(size_t)a * nC + i] / s;
          num += wt * pc[i];
          den += wt;
        }
        out.actionEv[a].aggEv = den > 0.0 ? num / den : (den0 > 0.0 ? num0 / den0 : 0.0);
      }
      for (int i = 0; i < nC; ++i) {
        double s = 0.0;
        for (int a = 0; a < na; ++a) s += srows[(size_t)a * nC + i];
        if (s <= 0.0) continue;
        double ev = 0.0;
        for (int a = 0; a < na; ++a)
          ev += (double)srows[(size_t)a * nC + i] / s * out.actionEv[a].perCombo[i];
        S.ev[i] = ev;
      }
    }
    double num = 0.0, den = 0.0;
    for (int i = 0; i < nC; ++i) {
      if (S.mass[i] <= 0.0) continue;
      const double wt = self.w[S.combos[i]] * S.mass[i];
      num += wt * S.ev[i];
      den += wt;
    }
    S.aggEv = den > 0.0 ? num / den : 0.0;
  }
  return out;
}

gpu::RunoutSummary SolverCore::runoutSummary(int decideIdx, int actionIdx) {
  requireEngine();
  checkDecide(decideIdx);
  const int u = tree_.decideNodes[decideIdx];
  const Node& nd = tree_.nodes[u];
  if (actionIdx < 0 || actionIdx >= nd.na)
    throw Error{PPS_GB_E_INDEX, "action index " + std::to_string(actionIdx) + " out of range"};
  const int ch = tree_.children[nd.childBase + actionIdx];
  if (tree_.nodes[ch].kind != kChance)
    throw Error{PPS_GB_E_ARG, "action does not lead to a deal"};
  std::vector<int> metaOf(tree_.nodes.size(), -1);
  for (size_t i = 0; i < tree_.decideNodes.size(); ++i) metaOf[tree_.decideNodes[i]] = (int)i;
  // First decide node below a branch (breadth-first through further deals).
  auto firstDecide = [&](int start) {
    if (tree_.nodes[start].kind == kDecide) return start;
    std::vector<int> q{start};
    for (size_t qi = 0; qi < q.size(); ++qi) {
      const Node& x = tree_.nodes[q[qi]];
      for (int k = 0; k < x.nChildren; ++k) {
        const int c = tree_.children[x.childBase + k];
        if (tree_.nodes[c].kind == kDecide) return c;
        if (tree_.nodes[c].kind == kChance) q.push_back(c);
      }
    }
    return -1;
  };
  const Node& cn = tree_.nodes[ch];
  gpu::RunoutSummary out;
  out.branches.resize(cn.nChildren);
  int firstIdx = -1;
  for (int br = 0; br < cn.nChildren; ++br) {
    const int bc = tree_.children[cn.childBase + br];
    out.branches[br].card = tree_.states[tree_.nodes[bc].state].dealt;
    const int fd = firstDecide(bc);
    if (fd >= 0) {
      out.branches[br].nextDecide = metaOf[fd];
      if (firstIdx < 0) firstIdx = metaOf[fd];
    }
  }
  if (firstIdx < 0) return out;
  const Node& fm = tree_.nodes[tree_.decideNodes[firstIdx]];
  out.decider = fm.player;
  for (int a = 0; a < fm.na; ++a) out.actions.push_back(label(tree_.actions[fm.actBase + a]));

  for (int tr = 0; tr < 2; ++tr) {
    eng_->walkFrom(tr, kModeEV, ch);  // rows below the deal
    const Side& self = tree_.side[tr];
    const Side& opp = tree_.side[1 - tr];
    for (int br = 0; br < cn.nChildren; ++br) {
      const int bi = out.branches[br].nextDecide;
      if (bi < 0) continue;
      const int f = tree_.decideNodes[bi];
      const Node& bm = tree_.nodes[f];
      const BoardState& st = tree_.states[bm.state];
      const auto& list = st.list[tr];
      const auto& olist = st.list[1 - tr];
      const int nC = (int)list.size();
      const std::vector<double> reach = eng_->walkReach(f, tr);
      double cardSum[52] = {0.0}, tot = 0.0;
      for (size_t j = 0; j < olist.size(); ++j) {
        tot += reach[j];
        cardSum[opp.cards[2 * olist[j]]] += reach[j];
        cardSum[opp.cards[2 * olist[j] + 1]] += reach[j];
      }
      std::vector<double> mass(nC, 0.0);
      for (int i = 0; i < nC; ++i) {
        const int b = list[i];
        double mm = tot - cardSum[self.cards[2 * b]] - cardSum[self.cards[2 * b + 1]];
        const int so = self.sameOther[b];
        if (so >= 0) {
          const int slot = slotIn(olist, so);
          if (slot >= 0) mm += reach[slot];
        }
        mass[i] = mm;
      }
      const std::vector<double> row = eng_->walkCfv(f, tr);
      double num = 0.0, den = 0.0;
      for (int i = 0; i < nC; ++i) {
        if (mass[i] <= 0.0) continue;
        const double wt = self.w[list[i]] * mass[i];
        num += wt * row[i] / mass[i];
        den += wt;
      }
      out.branches[br].aggEv[tr] = den > 0.0 ? num / den : 0.0;
      // This walk's reach row is the decider's own reach when the decider
      // is the opponent of tr: aggregate its strategy over it.
      if (bm.player != tr && bm.na == (int)out.actions.size()) {
        const int nDec = (int)olist.size();
        const std::vector<float> sr = eng_->nodeRows(1, f);
        std::vector<double>& freq = out.branches[br].freq;
        freq.assign(bm.na, 0.0);
        double z = 0.0;
        for (int c = 0; c < nDec; ++c) {
          double s = 0.0;
          for (int a = 0; a < bm.na; ++a) s += sr[(size_t)a * nDec + c];
          if (s <= 0.0) continue;
          z += reach[c];
          for (int a = 0; a < bm.na; ++a) freq[a] += reach[c] * (double)sr[(size_t)a * nDec + c] / s;
        }
        if (z > 0.0)
          for (int a = 0; a < bm.na; ++a) freq[a] /= z;
      }
    }
  }
  return out;
}

// ---------------------------------------------------------------------------
// Introspection.
// ---------------------------------------------------------------------------

std::vector<uint8_t> SolverCore::playerCards(int player) const {
  if (player < 0 || player > 1) throw Error{PPS_GB_E_INDEX, "player must be 0 (OOP) or 1 (IP)"};
  return tree_.side[player].cards;
}

int SolverCore::numBaseCombos(int player) const {
  if (player < 0 || player > 1) throw Error{PPS_GB_E_INDEX, "player must be 0 (OOP) or 1 (IP)"};
  return tree_.side[player].n;
}

std::vector<double> SolverCore::playerWeights(int player) const {
  if (player < 0 || player > 1) throw Error{PPS_GB_E_INDEX, "player must be 0 (OOP) or 1 (IP)"};
  return tree_.side[player].w;
}

gpu::TreeStructure SolverCore::treeStructure() const {
  gpu::TreeStructure t;
  for (const Node& nd : tree_.nodes) {
    t.kinds.push_back(nd.kind);
    t.childBase.push_back(nd.childBase);
    const BoardState& st = tree_.states[nd.state];
    for (int i = 0; i < 5; ++i) t.boards.push_back(i < st.nBoard ? st.board[i] : 0);
  }
  t.children = tree_.children;
  return t;
}

void SolverCore::debugDump() {
  if (!eng_) return;
  for (int which = 1; which >= 0; --which) {
    const std::vector<float> rows = eng_->denseRows(which);
    long long bad = 0;
    for (float v : rows) bad += !std::isfinite(v);
    std::fprintf(stderr, "%s nonfinite=%lld of %zu\n", which ? "strat" : "regret", bad,
                 rows.size());
  }
}

// ---------------------------------------------------------------------------
// "PPS1" solution files (cuda/gpu_cfr.cu:2686-2853). Version 1 holds one
// bet config; version 2 (per-street configs, no reference counterpart)
// holds three in the same field order. Versions 3 and 4 (no reference
// counterpart) are 1 and 2 with compressed rows: after the row count, the
// number of action rows, then for the regrets and then the strategy one
// f32 scale per action row followed by one 16-bit code per entry
// (rowcodec.h), about half the size of the f32 rows.
// ---------------------------------------------------------------------------

namespace {
constexpr uint32_t kMagic = 0x31535050;  // "PPS1"

struct Writer {
  FILE* f;
  const std::string& path;
  void put(const void* p, size_t n) {
    if (std::fwrite(p, 1, n, f) != n) throw Error{PPS_GB_E_IO, "write failed: " + path};
  }
  template <typename T>
  void val(T v) { put(&v, sizeof(T)); }
  void doubles(const std::vector<double>& v) {
    val<int32_t>((int32_t)v.size());
    put(v.data(), v.size() * sizeof(double));
  }
  void cfg(const pf::BetConfig& c) {
    doubles(c.betFracs);
    doubles(c.raiseMults);
    val<int8_t>((int8_t)c.betAllIn);
    val<int8_t>((int8_t)c.betGeometric);
    val<int32_t>(c.maxRaises);
    val<double>(c.addAllinThreshold);
    val<double>(c.forceAllinThreshold);
    val<double>(c.mergingThreshold);
  }
};

struct Reader {
  FILE* f = nullptr;
  std::string path;
  explicit Reader(const std::string& p) : path(p) {
    f = std::fopen(p.c_str(), "rb");
    if (!f) throw Error{PPS_GB_E_IO, "cannot open solution file: " + p};
  }
  ~Reader() {
    if (f) std::fclose(f);
  }
  void get(void* p, size_t n) {
    if (std::fread(p, 1, n, f) != n)
      throw Error{PPS_GB_E_FORMAT, "solution file truncated: " + path};
  }
  template <typename T>
  T val() {
    T v;
    get(&v, sizeof(T));
    return v;
  }
  std::vector<double> doubles() {
    const int32_t n = val<int32_t>();
    if (n < 0 || n > (1 << 24))
      throw Error{PPS_GB_E_FORMAT, "solution file corrupt: bad length: " + path};
    std::vector<double> v((size_t)n);
    get(v.data(), v.size() * sizeof(double));
    return v;
  }
  pf::BetConfig cfg() {
    pf::BetConfig c;
    c.betFracs = doubles();
    c.raiseMults = doubles();
    c.betAllIn = val<int8_t>() != 0;
    c.betGeometric = val<int8_t>() != 0;
    c.maxRaises = val<int32_t>();
    c.addAllinThreshold = val<double>();
    c.forceAllinThreshold = val<double>();
    c.mergingThreshold = val<double>();
    return c;
  }
};
}  // namespace

void SolverCore::save(const std::string& path, bool compressed) const {
  if (!eng_) throw Error{PPS_GB_E_STATE, "cannot save an empty solver"};
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw Error{PPS_GB_E_IO, "cannot open for writing: " + path};
  try {
    Writer w{f, path};
    const gpu::PostflopSpot& sp = tree_.spot;
    w.val<uint32_t>(kMagic);
    w.val<uint32_t>((tree_.perStreet ? 2u : 1u) + (compressed ? 2u : 0u));
    w.val<int32_t>(sp.nBoard);
    w.put(sp.board, sizeof(sp.board));
    w.val<int64_t>(sp.pot);
    w.val<int64_t>(sp.stack);
    w.put(sp.oop.w, sizeof(sp.oop.w));
    w.put(sp.ip.w, sizeof(sp.ip.w));
    if (tree_.perStreet)
      for (int k = 0; k < 3; ++k) w.cfg(tree_.cfgs.street[k]);
    else
      w.cfg(tree_.cfgs.street[0]);
    w.val<int64_t>((int64_t)tree_.nodes.size());
    w.val<int64_t>(totalIters_);
    w.val<int32_t>((int32_t)lastAlgo_.size());
    w.put(lastAlgo_.data(), lastAlgo_.size());
    w.val<int64_t>(tree_.rowTotal);
    if (compressed) {
      w.val<int64_t>(eng_->actionRows());
      for (int which = 0; which < 2; ++which) {
        std::vector<uint16_t> codes;
        std::vector<float> scales;
        eng_->packRows(which, codes, scales);
        w.put(scales.data(), scales.size() * sizeof(float));
        w.put(codes.data(), codes.size() * sizeof(uint16_t));
      }
    } else {
      const std::vector<float> reg = eng_->denseRows(0), str = eng_->denseRows(1);
      w.put(reg.data(), reg.size() * sizeof(float));
      w.put(str.data(), str.size() * sizeof(float));
    }
    if (std::fflush(f) != 0) throw Error{PPS_GB_E_IO, "write failed: " + path};
  } catch (...) {
    std::fclose(f);
    throw;
  }
  std::fclose(f);
}

std::unique_ptr<SolverCore> SolverCore::load(const std::string& path) {
  Reader r(path);
  if (r.val<uint32_t>() != kMagic)
    throw Error{PPS_GB_E_FORMAT, "not a solution file: " + path};
  const uint32_t ver = r.val<uint32_t>();
  if (ver < 1 || ver > 4)
    throw Error{PPS_GB_E_FORMAT, "solution file version " + std::to_string(ver) +
                                     " unsupported (expected 1 to 4): " + path};
  const bool perStreet = ver == 2 || ver == 4, compressed = ver >= 3;
  gpu::PostflopSpot spot;
  spot.nBoard = r.val<int32_t>();
  if (spot.nBoard < 3 || spot.nBoard > 5)
    throw Error{PPS_GB_E_FORMAT, "solution file corrupt: bad board size"};
  r.get(spot.board, sizeof(spot.board));
  spot.pot = r.val<int64_t>();
  spot.stack = r.val<int64_t>();
  r.get(spot.oop.w, sizeof(spot.oop.w));
  r.get(spot.ip.w, sizeof(spot.ip.w));
  gpu::StreetBetConfigs cfgs;
  if (perStreet) {
    for (int k = 0; k < 3; ++k) cfgs.street[k] = r.cfg();
  } else {
    cfgs.street[0] = r.cfg();
    cfgs.street[1] = cfgs.street[2] = cfgs.street[0];
  }
  r.val<int64_t>();  // node count (informational; the row table validates)
  const int64_t savedIters = r.val<int64_t>();
  const int32_t algoLen = r.val<int32_t>();
  if (algoLen < 0 || algoLen > 15)
    throw Error{PPS_GB_E_FORMAT, "solution file corrupt: bad algo length"};
  std::string algo((size_t)algoLen, '\0');
  r.get(&algo[0], (size_t)algoLen);
  Schedule sched;
  if (!Schedule::parse(algo, sched))
    throw Error{PPS_GB_E_FORMAT, "solution file corrupt: unknown algo '" + algo + "'"};
  std::unique_ptr<SolverCore> s(new SolverCore(spot, cfgs, perStreet));
  if (s->tree_.empty)
    throw Error{PPS_GB_E_FORMAT,
                "solution spot compiled to an empty solver (empty or fully "
                "board-blocked range)"};
  const int64_t rowTotal = r.val<int64_t>();
  if (rowTotal != s->tree_.rowTotal)
    throw Error{PPS_GB_E_FORMAT,
                "solution file does not match this engine's compiled tree (row table " +
                    std::to_string(rowTotal) + " vs " + std::to_string(s->tree_.rowTotal) +
                    " - different engine version or spot semantics)"};
  if (savedIters < 0 || savedIters > std::numeric_limits<int>::max())
    throw Error{PPS_GB_E_FORMAT, "solution file corrupt: bad iteration count"};
  if (compressed) {
    const int64_t nRows = r.val<int64_t>();
    if (nRows != s->eng_->actionRows())
      throw Error{PPS_GB_E_FORMAT, "solution file corrupt: action row count " +
                                       std::to_string(nRows) + " vs " +
                                       std::to_string(s->eng_->actionRows())};
    for (int which = 0; which < 2; ++which) {
      std::vector<float> scales((size_t)nRows);
      std::vector<uint16_t> codes((size_t)rowTotal);
      r.get(scales.data(), scales.size() * sizeof(float));
      r.get(codes.data(), codes.size() * sizeof(uint16_t));
      for (float m : scales)
        if (!(m >= 0.f) || !std::isfinite(m))
          throw Error{PPS_GB_E_FORMAT, "solution file corrupt: bad row scale"};
      s->eng_->unpackRows(which, codes, scales);
    }
  } else {
    std::vector<float> reg((size_t)rowTotal), str((size_t)rowTotal);
    r.get(reg.data(), reg.size() * sizeof(float));
    r.get(str.data(), str.size() * sizeof(float));
    s->eng_->setDenseRows(0, reg);
    s->eng_->setDenseRows(1, str);
  }
  s->eng_->setCounter((int)savedIters);
  s->lastAlgo_ = algo;
  s->sched_ = sched;
  s->totalIters_ = savedIters;
  return s;
}

}  // namespace gb
}  // namespace pps
