// CPU ORACLE - test infrastructure only.
//
// A plain recursive restatement of the reference's DCFR solve for one
// postflop spot. The GPU solver is tested against it (tests/), and it backs the
// smoke check (__graft_entry__.smoke) and the CPU baseline leg of
// bench.py; no product code links or calls it.
//
// What it restates (reference file:line):
//   hand strength        src/cards.cpp:30-165 (incl. its 4-kicker pair rule)
//   bet abstraction      src/postflop_cfr.cpp:18-152
//   tree shape           cuda/gpu_cfr.cu:1116-1326 (DFS pre-order, inline
//                        folds, dead street, chance over undealt cards)
//   iteration order      cuda/gpu_cfr.cu:856-857 (alternating half-steps)
//   forward strategy     cuda/gpu_cfr.cu:240-263 (RM+ / average strategy)
//   chance weight        cuda/gpu_cfr.cu:281 (1 / (52 - nBoard - 4))
//   showdown payoffs     cuda/gpu_cfr.cu:355-405
//   fold payoffs         cuda/gpu_cfr.cu:433-454
//   DCFR update          cuda/gpu_cfr.cu:479-523 (sigma from pre-update
//                        regrets)
//   chance backward      cuda/gpu_cfr.cu:542-554
//   schedule             cuda/gpu_cfr.cu:585-614
//   value / BR walks, Z  cuda/gpu_cfr.cu:871-923, 2042-2105
//
// The formulation is deliberately different from the GPU kernels: the
// half-step is one depth-first recursion (reach flows down, values flow
// up), the showdown is a two-pass sweep over strength-sorted combos with
// running per-card sums, and every row is an ordinary std::vector. R is the
// arithmetic type (float mirrors the reference's precision class, double
// gives the FP64 column).
//
// Rows use the reference's dense layout (decide nodes in node order, each
// na x n action-major), so tests compare them with the GPU's rows 1:1.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Cards and strength (reference rules, plain arrays).
// ---------------------------------------------------------------------------

int straightTop(int mask) {
  int m = (mask << 1) | ((mask >> 12) & 1);
  for (int hi = 13; hi >= 4; --hi) {
    int run = 1;
    for (int j = 0; j < 5; ++j)
      if (!((m >> (hi - j)) & 1)) run = 0;
    if (run) return hi - 1;
  }
  return -1;
}

uint64_t strength7(const int* cards) {
  int rc[13] = {0}, sc[4] = {0}, sm[4] = {0}, any = 0;
  for (int i = 0; i < 7; ++i) {
    rc[cards[i] % 13]++;
    sc[cards[i] / 13]++;
    sm[cards[i] / 13] |= 1 << (cards[i] % 13);
    any |= 1 << (cards[i] % 13);
  }
  int cat = 0, tb[5] = {0, 0, 0, 0, 0};
  auto kick = [&](int from, int count, int mask, int skip) {
    int k = from;
    for (int r = 12; r >= 0 && k < from + count; --r)
      if (((mask >> r) & 1) && !((skip >> r) & 1)) tb[k++] = r;
  };
  int flushSuit = -1;
  for (int s = 0; s < 4; ++s)
    if (sc[s] >= 5) flushSuit = s;
  int quad = -1, t1 = -1, t2 = -1, pairs[3] = {-1, -1, -1}, np = 0;
  for (int r = 12; r >= 0; --r) {
    if (rc[r] == 4) quad = r;
    else if (rc[r] == 3) { if (t1 < 0) t1 = r; else t2 = r; }
    else if (rc[r] == 2 && np < 3) pairs[np++] = r;
  }
  if (flushSuit >= 0) {
    const int sf = straightTop(sm[flushSuit]);
    if (sf >= 0) { cat = 8; tb[0] = sf; }
    else { cat = 5; kick(0, 5, sm[flushSuit], 0); }
  } else if (quad >= 0) {
    cat = 7; tb[0] = quad; kick(1, 1, any, 1 << quad);
  } else if (t1 >= 0 && (np > 0 || t2 >= 0)) {
    cat = 6; tb[0] = t1; tb[1] = std::max(np > 0 ? pairs[0] : -1, t2);
  } else if (straightTop(any) >= 0) {
    cat = 4; tb[0] = straightTop(any);
  } else if (t1 >= 0) {
    cat = 3; tb[0] = t1; kick(1, 2, any, 1 << t1);
  } else if (np >= 2) {
    cat = 2; tb[0] = pairs[0]; tb[1] = pairs[1];
    kick(2, 1, any, (1 << pairs[0]) | (1 << pairs[1]));
  } else if (np == 1) {
    cat = 1; tb[0] = pairs[0]; kick(1, 4, any, 1 << pairs[0]);
  } else {
    kick(0, 5, any, 0);
  }
  uint64_t key = (uint64_t)cat;
  for (int i = 0; i < 5; ++i) key = key * 13 + (uint64_t)tb[i];
  return key;
}

// ---------------------------------------------------------------------------
// Bet abstraction (reference src/postflop_cfr.cpp:18-152).
// ---------------------------------------------------------------------------

enum { kFold = 0, kCheck = 1, kCall = 2, kBet = 3, kRaise = 4, kAllIn = 5 };

struct Cfg {
  std::vector<double> bets, raises;
  bool allin = false, geo = false;
  int maxRaises = 0;
  double addT = 1.5, forceT = 0.15, mergeT = 0.1;
};

struct Act {
  int kind;
  int64_t amt;
};

int64_t rnd(double x) { return (int64_t)std::llround(x); }

std::vector<Act> actionsOf(int64_t potBase, int64_t stack, const Cfg& c, int64_t sc0, int64_t sc1,
                           int actor, bool afterAllin, int numBets, int streets) {
  const int64_t my = actor == 0 ? sc0 : sc1, op = actor == 0 ? sc1 : sc0;
  const int64_t prev = sc0 > sc1 ? sc0 : sc1;
  const int64_t call = my < op ? op - my : 0;
  const int64_t pot = potBase + 2 * (my + call);
  const int64_t maxA = stack - op + prev;
  int64_t minA = prev + call;
  if (minA < 1) minA = 1;
  if (minA > maxA) minA = maxA;
  const bool canRaise = c.maxRaises <= 0 || numBets < c.maxRaises;
  std::vector<Act> v;
  if (call == 0) {
    v.push_back({kCheck, 0});
    if (canRaise) {
      for (double f : c.bets) v.push_back({kBet, rnd(f * (double)pot)});
      if (c.geo && streets > 0 && pot > 0) {
        const double spr = (double)(stack - op) / (double)pot;
        const double ratio = (std::pow(2.0 * spr + 1.0, 1.0 / streets) - 1.0) / 2.0;
        v.push_back({kBet, rnd(ratio * (double)pot)});
      }
    }
    if (c.allin || maxA <= rnd(c.addT * (double)pot)) v.push_back({kAllIn, maxA});
  } else {
    v.push_back({kFold, 0});
    v.push_back({kCall, 0});
    if (!afterAllin) {
      if (canRaise)
        for (double m : c.raises) v.push_back({kRaise, rnd(m * (double)prev)});
      if (maxA <= prev + rnd(c.addT * (double)pot)) v.push_back({kAllIn, maxA});
    }
  }
  for (Act& a : v) {
    if (a.kind != kBet && a.kind != kRaise) continue;
    int64_t x = a.amt < minA ? minA : a.amt;
    if (x > maxA) x = maxA;
    if (maxA <= x + rnd((double)(pot + 2 * (x - prev)) * c.forceT)) a = {kAllIn, maxA};
    else a.amt = x;
  }
  std::sort(v.begin(), v.end(), [](const Act& a, const Act& b) {
    return a.kind != b.kind ? a.kind < b.kind : a.amt < b.amt;
  });
  v.erase(std::unique(v.begin(), v.end(),
                      [](const Act& a, const Act& b) { return a.kind == b.kind && a.amt == b.amt; }),
          v.end());
  if (c.mergeT > 0) {
    std::vector<Act> wag, rest, kept;
    for (const Act& a : v) (a.kind >= kBet ? wag : rest).push_back(a);
    std::sort(wag.begin(), wag.end(), [](const Act& a, const Act& b) {
      return a.amt != b.amt ? a.amt > b.amt : a.kind < b.kind;
    });
    int64_t cur = INT64_MAX;
    for (const Act& a : wag) {
      const double r = (double)(a.amt - prev) / (double)pot;
      const double cr = (double)(cur - prev) / (double)pot;
      if (r < (cr - c.mergeT) / (1.0 + c.mergeT) * (1.0 - 1e-12)) {
        kept.push_back(a);
        cur = a.amt;
      }
    }
    std::sort(rest.begin(), rest.end(), [](const Act& a, const Act& b) {
      return a.kind != b.kind ? a.kind < b.kind : a.amt < b.amt;
    });
    v = rest;
    v.insert(v.end(), kept.rbegin(), kept.rend());
  }
  return v;
}

// ---------------------------------------------------------------------------
// Tree.
// ---------------------------------------------------------------------------

struct Combo {
  int a, b;
  double w;
};

using List = std::shared_ptr<std::vector<int>>;  // base indices, ascending
using Keys = std::shared_ptr<std::vector<uint64_t>>;

enum { kDecide = 0, kShow = 1, kFoldN = 2, kChance = 3 };

struct ONode {
  int kind = kDecide, player = 0, foldBy = 0;
  int nBoard = 0;
  int board[5] = {0, 0, 0, 0, 0};
  int64_t potBase = 0, sc0 = 0, sc1 = 0, pc0 = 0, pc1 = 0;
  List list[2];
  Keys keys[2];           // river nodes: strength per base combo
  std::vector<int> kids;  // children node ids
  std::vector<int> dealt; // chance: card per branch
  int64_t rowOff = -1;    // decide: offset in the dense row table
  int na = 0;
  int actBase = 0;        // decide: first action in Spot::acts
};

struct Spot {
  std::vector<Combo> side[2];
  std::vector<int> same[2];  // base -> identical base on the other side
  int64_t pot = 0, stack = 0;
  Cfg cfg[3];
  std::vector<ONode> nodes;
  std::vector<Act> acts;  // every decide node's actions, in node order
  int64_t rowTotal = 0;
  int nBoard0 = 0;

  bool holds(int p, int base, int card) const {
    return side[p][base].a == card || side[p][base].b == card;
  }

  int build(const int* board, int nBoard, int64_t potBase, int64_t sc0, int64_t sc1, int actor,
            bool afterAllin, bool closed, int64_t pc0, int64_t pc1, int numBets, const List* lists,
            const Keys* keys) {
    const int id = (int)nodes.size();
    nodes.emplace_back();
    {
      ONode& n = nodes[id];
      n.nBoard = nBoard;
      for (int i = 0; i < nBoard; ++i) n.board[i] = board[i];
      n.potBase = potBase;
      n.sc0 = sc0;
      n.sc1 = sc1;
      n.pc0 = pc0;
      n.pc1 = pc1;
      for (int p = 0; p < 2; ++p) {
        n.list[p] = lists[p];
        n.keys[p] = keys[p];
      }
    }
    if (!closed && stack - pc0 <= 0) closed = true;
    if (closed) {
      if (nBoard == 5) {
        nodes[id].kind = kShow;
        return id;
      }
      nodes[id].kind = kChance;
      for (int c = 0; c < 52; ++c) {
        bool on = false;
        for (int i = 0; i < nBoard; ++i) on |= board[i] == c;
        if (on) continue;
        int nb[5];
        for (int i = 0; i < nBoard; ++i) nb[i] = board[i];
        nb[nBoard] = c;
        List cl[2];
        Keys ck[2];
        for (int p = 0; p < 2; ++p) {
          cl[p] = std::make_shared<std::vector<int>>();
          for (int b : *lists[p])
            if (!holds(p, b, c)) cl[p]->push_back(b);
          if (nBoard + 1 == 5) {
            ck[p] = std::make_shared<std::vector<uint64_t>>(side[p].size(), 0);
            for (int b : *cl[p]) {
              const int seven[7] = {side[p][b].a, side[p][b].b, nb[0], nb[1], nb[2], nb[3], nb[4]};
              (*ck[p])[b] = strength7(seven);
            }
          }
        }
        const int kid = build(nb, nBoard + 1, potBase + sc0 + sc1, 0, 0, 0, false, false,
                              pc0 + sc0, pc1 + sc1, 0, cl, ck);
        nodes[id].kids.push_back(kid);
        nodes[id].dealt.push_back(c);
      }
      return id;
    }
    const std::vector<Act> acts = actionsOf(potBase, stack - pc0, cfg[nBoard - 3], sc0, sc1,
                                            actor, afterAllin, numBets, 6 - nBoard);
    nodes[id].kind = kDecide;
    nodes[id].player = actor;
    nodes[id].na = (int)acts.size();
    nodes[id].actBase = (int)this->acts.size();
    this->acts.insert(this->acts.end(), acts.begin(), acts.end());
    for (const Act& a : acts) {
      int64_t n0 = sc0, n1 = sc1;
      bool after = afterAllin, ends = false;
      int kid = -1;
      if (a.kind == kCheck) {
        if (actor == 0)
          kid = build(board, nBoard, potBase, sc0, sc1, 1, afterAllin, false, pc0, pc1, numBets,
                      lists, keys);
        else
          ends = true;
      } else if (a.kind == kFold) {
        kid = (int)nodes.size();
        nodes.emplace_back();
        ONode& f = nodes[kid];
        f.kind = kFoldN;
        f.foldBy = actor;
        f.nBoard = nBoard;
        for (int i = 0; i < nBoard; ++i) f.board[i] = board[i];
        f.potBase = potBase;
        f.sc0 = sc0;
        f.sc1 = sc1;
        f.pc0 = pc0;
        f.pc1 = pc1;
        for (int p = 0; p < 2; ++p) {
          f.list[p] = lists[p];
          f.keys[p] = keys[p];
        }
      } else if (a.kind == kCall) {
        (actor == 0 ? n0 : n1) = sc0 > sc1 ? sc0 : sc1;
        ends = true;
      } else {
        if (a.kind == kAllIn) after = true;
        (actor == 0 ? n0 : n1) = a.amt;
      }
      if (ends)
        kid = build(board, nBoard, potBase, n0, n1, 0, false, true, pc0, pc1, 0, lists, keys);
      else if (kid < 0)
        kid = build(board, nBoard, potBase, n0, n1, actor ^ 1, after, false, pc0, pc1,
                    a.kind == kCheck ? numBets : numBets + 1, lists, keys);
      nodes[id].kids.push_back(kid);
    }
    return id;
  }

  void assignRows() {
    rowTotal = 0;
    for (ONode& n : nodes)
      if (n.kind == kDecide) {
        n.rowOff = rowTotal;
        rowTotal += (int64_t)n.na * (int64_t)n.list[n.player]->size();
      }
  }
};

// ---------------------------------------------------------------------------
// DCFR over the tree.
// ---------------------------------------------------------------------------

struct Coef {
  double pos, neg, avg;
};

Coef schedule(int kind, int t, int iters) {
  // kind: 0 dcfr (gamma 3, reset at powers of 4), 1 hs30, 2 gamma 2,
  // 3 no reset, 4 gamma 2 no reset.
  if (kind == 1) {
    const double n = iters, tt = t + 1;
    const double pa = std::pow(tt, 1.0 + 3.0 * tt / n), pb = std::pow(tt, -1.0 - 2.0 * tt / n);
    return {pa / (pa + 1.0), pb / (pb + 1.0), std::pow(tt / (tt + 1.0), 30.0 - 5.0 * tt / n)};
  }
  const double gamma = (kind == 2 || kind == 4) ? 2.0 : 3.0;
  const bool reset = kind != 3 && kind != 4;
  const double ta = t > 1 ? t - 1 : 0;
  const double pa = std::pow(ta, 1.5);
  double k = 0;
  if (reset && t > 0) {
    k = 1;
    while (k * 4 <= t) k *= 4;
  }
  const double tg = t - k;
  return {pa / (pa + 1.0), 0.5, std::pow(tg / (tg + 1.0), gamma)};
}

template <typename R>
struct Solver {
  Spot sp;
  std::vector<float> regret, strat;  // dense rows (the reference's f32 storage)
  std::vector<double> regretD, stratD;  // f64 mode storage
  bool f64 = false;

  double rowGet(const std::vector<float>& f, const std::vector<double>& d, int64_t i) const {
    return f64 ? d[i] : (double)f[i];
  }

  // Traverser values of node u given the opponent reach row (aligned with
  // the node's opponent list). mode 0: CFR update, 1: EV, 2: BR.
  std::vector<R> walk(int u, int tr, const std::vector<R>& reach, int mode, const R* coef) {
    const ONode& n = sp.nodes[u];
    const int opp = 1 - tr;
    const std::vector<int>& lt = *n.list[tr];
    const std::vector<int>& lo = *n.list[opp];
    const int nt = (int)lt.size(), no = (int)lo.size();
    std::vector<R> out(nt, R(0));
    if (n.kind == kFoldN) {
      R cs[52] = {}, tot = R(0);
      for (int j = 0; j < no; ++j) {
        tot += reach[j];
        cs[sp.side[opp][lo[j]].a] += reach[j];
        cs[sp.side[opp][lo[j]].b] += reach[j];
      }
      const int fb = n.foldBy;
      const int64_t sc = fb == 0 ? n.sc0 : n.sc1;
      const int64_t pcF = fb == 0 ? n.pc0 : n.pc1;
      const int64_t pcT = tr == 0 ? n.pc0 : n.pc1;
      const R v = tr == fb ? -((R)sc + (R)pcF) : ((R)(n.potBase + sc) - (R)pcT);
      for (int i = 0; i < nt; ++i) {
        const Combo& c = sp.side[tr][lt[i]];
        R w = tot - cs[c.a] - cs[c.b];
        const int so = sp.same[tr][lt[i]];
        if (so >= 0) {
          auto it = std::lower_bound(lo.begin(), lo.end(), so);
          if (it != lo.end() && *it == so) w += reach[it - lo.begin()];
        }
        if (w < R(0)) w = R(0);
        out[i] = w * v;
      }
      return out;
    }
    if (n.kind == kShow) {
      const std::vector<uint64_t>& kt = *n.keys[tr];
      const std::vector<uint64_t>& ko = *n.keys[opp];
      std::vector<int> ordO(no), ordT(nt);
      for (int j = 0; j < no; ++j) ordO[j] = j;
      for (int i = 0; i < nt; ++i) ordT[i] = i;
      std::stable_sort(ordO.begin(), ordO.end(),
                       [&](int x, int y) { return ko[lo[x]] < ko[lo[y]]; });
      std::stable_sort(ordT.begin(), ordT.end(),
                       [&](int x, int y) { return kt[lt[x]] < kt[lt[y]]; });
      std::vector<R> beat(nt), lose(nt);
      // Ascending sweep: opponents strictly weaker than each traverser combo.
      {
        R tot = R(0), cs[52] = {};
        int j = 0;
        for (int ii = 0; ii < nt; ++ii) {
          const int i = ordT[ii];
          const uint64_t s = kt[lt[i]];
          while (j < no && ko[lo[ordO[j]]] < s) {
            const int o = ordO[j++];
            tot += reach[o];
            cs[sp.side[opp][lo[o]].a] += reach[o];
            cs[sp.side[opp][lo[o]].b] += reach[o];
          }
          const Combo& c = sp.side[tr][lt[i]];
          beat[i] = tot - cs[c.a] - cs[c.b];
        }
      }
      // Descending sweep: opponents strictly stronger.
      {
        R tot = R(0), cs[52] = {};
        int j = no - 1;
        for (int ii = nt - 1; ii >= 0; --ii) {
          const int i = ordT[ii];
          const uint64_t s = kt[lt[i]];
          while (j >= 0 && ko[lo[ordO[j]]] > s) {
            const int o = ordO[j--];
            tot += reach[o];
            cs[sp.side[opp][lo[o]].a] += reach[o];
            cs[sp.side[opp][lo[o]].b] += reach[o];
          }
          const Combo& c = sp.side[tr][lt[i]];
          lose[i] = tot - cs[c.a] - cs[c.b];
        }
      }
      R all = R(0), csAll[52] = {};
      for (int j = 0; j < no; ++j) {
        all += reach[j];
        csAll[sp.side[opp][lo[j]].a] += reach[j];
        csAll[sp.side[opp][lo[j]].b] += reach[j];
      }
      const int64_t d = n.sc0 > n.sc1 ? n.sc0 - n.sc1 : n.sc1 - n.sc0;
      const R total = (R)(n.potBase + n.sc0 + n.sc1 - d);
      const R mine = (R)((tr == 0 ? n.sc0 : n.sc1) + (tr == 0 ? n.pc0 : n.pc1));
      const R winV = total - mine, tieV = total * R(0.5) - mine, loseV = -mine;
      for (int i = 0; i < nt; ++i) {
        const Combo& c = sp.side[tr][lt[i]];
        R valid = all - csAll[c.a] - csAll[c.b];
        const int so = sp.same[tr][lt[i]];
        if (so >= 0) {
          auto it = std::lower_bound(lo.begin(), lo.end(), so);
          if (it != lo.end() && *it == so) valid += reach[it - lo.begin()];
        }
        R b = beat[i] > R(0) ? beat[i] : R(0);
        R l = lose[i] > R(0) ? lose[i] : R(0);
        R tie = valid - b - l;
        if (tie < R(0)) tie = R(0);
        out[i] = b * winV + tie * tieV + l * loseV;
      }
      return out;
    }
    if (n.kind == kChance) {
      const R inv = R(1) / R(52 - n.nBoard - 4);
      const int nb = (int)n.kids.size();
      std::vector<std::vector<R>> childVals(nb);
      std::vector<std::vector<int>> childPos(nb);
      auto branch = [&](int b) {
        const ONode& ch = sp.nodes[n.kids[b]];
        const std::vector<int>& clo = *ch.list[opp];
        std::vector<R> cr(clo.size());
        size_t j = 0;
        for (size_t k = 0; k < clo.size(); ++k) {
          while (lo[j] != clo[k]) ++j;
          cr[k] = reach[j] * inv;
        }
        childVals[b] = walk(n.kids[b], tr, cr, mode, coef);
      };
#ifdef _OPENMP
      if (!omp_in_parallel()) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int b = 0; b < nb; ++b) branch(b);
      } else
#endif
        for (int b = 0; b < nb; ++b) branch(b);
      for (int b = 0; b < nb; ++b) {
        const std::vector<int>& clt = *sp.nodes[n.kids[b]].list[tr];
        size_t k = 0;
        for (int i = 0; i < nt && k < clt.size(); ++i)
          if (lt[i] == clt[k]) out[i] += childVals[b][k++];
      }
      return out;
    }
    // Decide node.
    const int na = n.na;
    const int actor = n.player;
    const bool useAvg = mode != 0;
    auto rowAt = [&](int a, int c, int nc) -> double {
      const int64_t i = n.rowOff + (int64_t)a * nc + c;
      return useAvg ? rowGet(strat, stratD, i) : rowGet(regret, regretD, i);
    };
    if (actor != tr) {
      std::vector<R> sig((size_t)na * no);
      for (int c = 0; c < no; ++c) {
        R acc = R(0);
        for (int a = 0; a < na; ++a) {
          const R x = (R)rowAt(a, c, no);
          acc += useAvg ? x : (x > R(0) ? x : R(0));
        }
        for (int a = 0; a < na; ++a) {
          const R x = (R)rowAt(a, c, no);
          R s;
          if (useAvg) s = acc > R(0) ? x / acc : R(1) / R(na);
          else s = acc > R(0) ? (x > R(0) ? x / acc : R(0)) : R(1) / R(na);
          sig[(size_t)a * no + c] = s;
        }
      }
      for (int a = 0; a < na; ++a) {
        std::vector<R> cr(no);
        for (int c = 0; c < no; ++c) cr[c] = reach[c] * sig[(size_t)a * no + c];
        const std::vector<R> v = walk(n.kids[a], tr, cr, mode, coef);
        for (int i = 0; i < nt; ++i) out[i] += v[i];
      }
      return out;
    }
    std::vector<std::vector<R>> cv(na);
    for (int a = 0; a < na; ++a) cv[a] = walk(n.kids[a], tr, reach, mode, coef);
    for (int c = 0; c < nt; ++c) {
      if (mode == 2) {
        R best = R(-1e30);
        for (int a = 0; a < na; ++a) best = cv[a][c] > best ? cv[a][c] : best;
        out[c] = best;
        continue;
      }
      R acc = R(0);
      R sig[64];
      for (int a = 0; a < na; ++a) {
        const R x = (R)rowAt(a, c, nt);
        sig[a] = x;
        acc += useAvg ? x : (x > R(0) ? x : R(0));
      }
      R val = R(0);
      for (int a = 0; a < na; ++a) {
        const R x = sig[a];
        R s;
        if (useAvg) s = acc > R(0) ? x / acc : R(1) / R(na);
        else s = acc > R(0) ? (x > R(0) ? x / acc : R(0)) : R(1) / R(na);
        sig[a] = s;
        val += s * cv[a][c];
      }
      out[c] = val;
      if (mode != 0) continue;
      for (int a = 0; a < na; ++a) {
        const int64_t i = n.rowOff + (int64_t)a * nt + c;
        if (f64) {
          const double r0 = regretD[i];
          stratD[i] = stratD[i] * (double)coef[2] + (double)sig[a];
          regretD[i] = r0 * (r0 >= 0.0 ? (double)coef[0] : (double)coef[1]) +
                       (double)(cv[a][c] - val);
        } else {
          const float r0 = regret[i];
          strat[i] = strat[i] * (float)coef[2] + (float)sig[a];
          regret[i] = r0 * (r0 >= 0.0f ? (float)coef[0] : (float)coef[1]) +
                      (float)(cv[a][c] - val);
        }
      }
    }
    return out;
  }

  std::vector<R> rootReach(int tr) const {
    std::vector<R> r;
    for (const Combo& c : sp.side[1 - tr]) r.push_back((R)c.w);
    return r;
  }
};

struct Handle {
  int precision = 32;
  Solver<float> s32;
  Solver<double> s64;
  Spot& spot() { return precision == 32 ? s32.sp : s64.sp; }
};

double pairMass(const Spot& sp) {
  double t1 = 0, cs[52] = {0};
  for (const Combo& c : sp.side[1]) {
    t1 += c.w;
    cs[c.a] += c.w;
    cs[c.b] += c.w;
  }
  double Z = 0;
  for (size_t i = 0; i < sp.side[0].size(); ++i) {
    const Combo& c = sp.side[0][i];
    double w = t1 - cs[c.a] - cs[c.b];
    if (sp.same[0][i] >= 0) w += sp.side[1][sp.same[0][i]].w;
    if (w > 0) Z += c.w * w;
  }
  return Z;
}

// ---------------------------------------------------------------------------
// The reference's device layout, restated from this file's tree: the
// arrays GpuPostflopSolver's init() uploads (cuda/gpu_cfr.cu:1363-1827),
// under the names of its TreeBuf / Impl members, so that the reference's
// own kernels can run a spot with no product code in the path. The tests
// pin every array against the reference's init() run on a host CUDA stub.
// ---------------------------------------------------------------------------

using Sink = void (*)(void* user, const char* name, char dtype, const void* data, int64_t n);

struct RefExport {
  const Spot& sp;
  Sink sink;
  void* user;
  std::vector<int> comboOff[2], comboId, runOffOff, runOff, ctapBase, ctap, expOffOff,
      expIdxBase, expOff, expIdx;

  void ints(const char* name, const std::vector<int>& v) { sink(user, name, 'i', v.data(), (int64_t)v.size()); }
  void longs(const char* name, const std::vector<int64_t>& v) {
    sink(user, name, 'q', v.data(), (int64_t)v.size());
  }
  void scalar(const char* name, int64_t v) { sink(user, name, 'q', &v, 1); }

  // Node-local slot in the parent's list of each child-list entry.
  static std::vector<int> parentSlots(const std::vector<int>& parent, const std::vector<int>& child) {
    std::vector<int> out;
    size_t i = 0;
    for (int b : child) {
      while (parent[i] != b) ++i;
      out.push_back((int)i);
    }
    return out;
  }

  // Combo lists and chance maps in the order the reference's recursion
  // appends them (cuda/gpu_cfr.cu:1197-1245): a chance node reserves its
  // runOff section, appends each branch's child lists right before
  // building that child, and writes its ctap / expOff / expIdx sections
  // after all children.
  void lists(int u, int off0, int off1) {
    const ONode& n = sp.nodes[u];
    comboOff[0][u] = off0;
    comboOff[1][u] = off1;
    if (n.kind != kChance) {
      for (int k : n.kids) lists(k, off0, off1);
      return;
    }
    const int nb = (int)n.kids.size();
    runOffOff[u] = (int)runOff.size();
    runOff.resize(runOff.size() + 2 * (nb + 1), 0);
    for (int k : n.kids) {
      const ONode& c = sp.nodes[k];
      const int c0 = (int)comboId.size();
      comboId.insert(comboId.end(), c.list[0]->begin(), c.list[0]->end());
      const int c1 = (int)comboId.size();
      comboId.insert(comboId.end(), c.list[1]->begin(), c.list[1]->end());
      lists(k, c0, c1);
    }
    ctapBase[u] = (int)ctap.size();
    for (int p = 0; p < 2; ++p) {
      const int base = runOffOff[u] + p * (nb + 1);
      int total = 0;
      for (int br = 0; br < nb; ++br) {
        runOff[base + br] = total;
        for (int j : parentSlots(*n.list[p], *sp.nodes[n.kids[br]].list[p])) {
          ctap.push_back(j);
          ++total;
        }
      }
      runOff[base + nb] = total;
    }
    expOffOff[u] = (int)expOff.size();
    expIdxBase[u] = (int)expIdx.size();
    for (int p = 0; p < 2; ++p) {
      std::vector<std::vector<int>> perSlot(n.list[p]->size());
      for (int br = 0; br < nb; ++br) {
        const auto par = parentSlots(*n.list[p], *sp.nodes[n.kids[br]].list[p]);
        for (int j = 0; j < (int)par.size(); ++j) perSlot[par[j]].push_back(br * 4096 + j);
      }
      int cnt = 0;
      for (const auto& v : perSlot) {
        expOff.push_back(cnt);
        expIdx.insert(expIdx.end(), v.begin(), v.end());
        cnt += (int)v.size();
      }
      expOff.push_back(cnt);
    }
  }

  void run() {
    const int N = (int)sp.nodes.size();
    std::vector<int> parent(N, -1), depth(N, 0);
    for (int u = 0; u < N; ++u)
      for (int k : sp.nodes[u].kids) {
        parent[k] = u;
        depth[k] = depth[u] + 1;
      }
    int maxDepth = 0, maxNa = 0;
    for (int u = 0; u < N; ++u) {
      maxDepth = std::max(maxDepth, depth[u]);
      maxNa = std::max(maxNa, sp.nodes[u].na);
    }
    const int n0 = (int)sp.side[0].size(), n1 = (int)sp.side[1].size();
    scalar("numNodes", N);
    scalar("maxDepth", maxDepth);
    scalar("n0Base", n0);
    scalar("n1Base", n1);
    scalar("maxNa", maxNa);
    scalar("regTotal", sp.rowTotal);

    for (int p = 0; p < 2; ++p) comboOff[p].assign(N, 0);
    runOffOff.assign(N, 0);
    ctapBase.assign(N, 0);
    expOffOff.assign(N, 0);
    expIdxBase.assign(N, 0);
    for (int p = 0; p < 2; ++p)
      for (int i = 0; i < (int)sp.side[p].size(); ++i) comboId.push_back(i);
    lists(0, 0, n0);

    std::vector<int> kind(N), player(N), foldBy(N), na(N), childBase(N), childFlat, boardId(N, 0),
        nC0(N), nC1(N), regOff(N, 0), cfvOff(N), reachOff0(N), reachOff1(N), nBranch(N),
        chanceQ(N);
    std::vector<int64_t> sc0(N), sc1(N), potBase(N), pc0(N), pc1(N);
    std::vector<uint8_t> nodeBoard((size_t)N * 5, 0);
    std::vector<std::vector<int>> boards;  // showdown boards, first seen
    std::vector<int> boardNode;
    int64_t reachTotal = 0, reachTotal0 = 0, reachTotal1 = 0, regTotal = 0;
    for (int u = 0; u < N; ++u) {
      const ONode& n = sp.nodes[u];
      kind[u] = n.kind;
      player[u] = n.kind == kDecide ? n.player : 0;
      foldBy[u] = n.kind == kFoldN ? n.foldBy : 0;
      na[u] = n.kind == kDecide ? n.na : 0;
      childBase[u] = (int)childFlat.size();
      childFlat.insert(childFlat.end(), n.kids.begin(), n.kids.end());
      nC0[u] = (int)n.list[0]->size();
      nC1[u] = (int)n.list[1]->size();
      sc0[u] = n.sc0;
      sc1[u] = n.sc1;
      potBase[u] = n.potBase;
      pc0[u] = n.pc0;
      pc1[u] = n.pc1;
      nBranch[u] = n.kind == kChance ? (int)n.kids.size() : 0;
      chanceQ[u] = 52 - n.nBoard - 4;
      for (int i = 0; i < n.nBoard; ++i) nodeBoard[(size_t)u * 5 + i] = (uint8_t)n.board[i];
      if (n.kind == kShow) {
        const std::vector<int> key(n.board, n.board + 5);
        int id = -1;
        for (size_t b = 0; b < boards.size(); ++b)
          if (boards[b] == key) id = (int)b;
        if (id < 0) {
          id = (int)boards.size();
          boards.push_back(key);
          boardNode.push_back(u);
        }
        boardId[u] = id;
      }
      const int row = std::max(nC0[u], nC1[u]);
      cfvOff[u] = (int)reachTotal;
      reachTotal += row;
      if (n.kind == kDecide) {
        regOff[u] = (int)regTotal;
        regTotal += (int64_t)n.na * (n.player == 0 ? nC0[u] : nC1[u]);
      }
      // Rows under a decide node of the layout's traverser alias the
      // parent's row (cuda/gpu_cfr.cu:1491-1514).
      const int par = parent[u];
      const bool parDecide = par >= 0 && sp.nodes[par].kind == kDecide;
      if (parDecide && sp.nodes[par].player == 0) reachOff0[u] = reachOff0[par];
      else { reachOff0[u] = (int)reachTotal0; reachTotal0 += row; }
      if (parDecide && sp.nodes[par].player == 1) reachOff1[u] = reachOff1[par];
      else { reachOff1[u] = (int)reachTotal1; reachTotal1 += row; }
    }
    scalar("reachTotal", reachTotal);
    scalar("reachTotal0", reachTotal0);
    scalar("reachTotal1", reachTotal1);
    scalar("empty", 0);
    ints("kind", kind);
    ints("player", player);
    ints("foldBy", foldBy);
    ints("na", na);
    ints("childBase", childBase);
    ints("childFlat", childFlat);
    ints("boardId", boardId);
    ints("nC0", nC0);
    ints("nC1", nC1);
    ints("comboOff0", comboOff[0]);
    ints("comboOff1", comboOff[1]);
    ints("comboId", comboId);
    ints("reachOff0", reachOff0);
    ints("reachOff1", reachOff1);
    ints("cfvOff", cfvOff);
    ints("regOff", regOff);
    longs("sc0", sc0);
    longs("sc1", sc1);
    longs("potBase", potBase);
    longs("pc0", pc0);
    longs("pc1", pc1);
    ints("nBranch", nBranch);
    ints("chanceQ", chanceQ);
    ints("runOffOff", runOffOff);
    ints("runOff", runOff);
    ints("ctapBase", ctapBase);
    ints("ctap", ctap);
    ints("expOffOff", expOffOff);
    ints("expIdxBase", expIdxBase);
    ints("expOff", expOff);
    ints("expIdx", expIdx);
    for (int p = 0; p < 2; ++p) {
      std::vector<float> wf;
      std::vector<uint8_t> cards;
      for (const Combo& c : sp.side[p]) {
        wf.push_back((float)c.w);
        cards.push_back((uint8_t)c.a);
        cards.push_back((uint8_t)c.b);
      }
      sink(user, p == 0 ? "w0" : "w1", 'f', wf.data(), (int64_t)wf.size());
      sink(user, p == 0 ? "cards0" : "cards1", 'B', cards.data(), (int64_t)cards.size());
      ints(p == 0 ? "sameOther0" : "sameOther1", sp.same[p]);
    }

    // Strength tables per (showdown board, traverser) over the full base
    // lists (cuda/gpu_cfr.cu:1594-1703): opponent combos stable-sorted by
    // strength, less / tie ends per traverser combo, the sorted positions
    // holding each card, and sorted position -> the board's node-local slot.
    const int nTables = (int)boards.size() * 2;
    std::vector<int> oppSortedOff(nTables + 1, 0), oppSorted, lessOff(nTables + 1, 0), lessEnd,
        tieEnd, cardPosOff(nTables * 53 + 1, 0), cardPosIdx, revSortedOff(nTables + 1, 0),
        revSorted;
    for (int bid = 0; bid < (int)boards.size(); ++bid) {
      const ONode& bn = sp.nodes[boardNode[bid]];
      std::vector<uint64_t> key[2];
      for (int p = 0; p < 2; ++p)
        for (const Combo& c : sp.side[p]) {
          const int seven[7] = {c.a, c.b, bn.board[0], bn.board[1], bn.board[2], bn.board[3],
                                bn.board[4]};
          key[p].push_back(strength7(seven));
        }
      for (int tr = 0; tr < 2; ++tr) {
        const int ti = bid * 2 + tr, opp = 1 - tr;
        const int no = (int)sp.side[opp].size();
        std::vector<int> ord(no);
        for (int i = 0; i < no; ++i) ord[i] = i;
        std::stable_sort(ord.begin(), ord.end(),
                         [&](int x, int y) { return key[opp][x] < key[opp][y]; });
        oppSortedOff[ti] = (int)oppSorted.size();
        oppSorted.insert(oppSorted.end(), ord.begin(), ord.end());
        std::vector<int> local(no, -1);
        const std::vector<int>& lo = *bn.list[opp];
        for (size_t j = 0; j < lo.size(); ++j) local[lo[j]] = (int)j;
        revSortedOff[ti] = (int)revSorted.size();
        for (int k = 0; k < no; ++k) revSorted.push_back(local[ord[k]]);
        lessOff[ti] = (int)lessEnd.size();
        for (size_t i = 0; i < sp.side[tr].size(); ++i) {
          const uint64_t v = key[tr][i];
          int lo2 = 0, hi2 = no;
          while (lo2 < hi2) {  // first position not weaker
            const int m = (lo2 + hi2) / 2;
            if (key[opp][ord[m]] < v) lo2 = m + 1; else hi2 = m;
          }
          int lo3 = lo2, hi3 = no;
          while (lo3 < hi3) {  // first position stronger
            const int m = (lo3 + hi3) / 2;
            if (key[opp][ord[m]] <= v) lo3 = m + 1; else hi3 = m;
          }
          lessEnd.push_back(lo2);
          tieEnd.push_back(lo3);
        }
        const int cpo = ti * 53;
        cardPosOff[cpo] = (int)cardPosIdx.size();
        for (int c = 0; c < 52; ++c) {
          cardPosOff[cpo + c + 1] = cardPosOff[cpo + c];
          for (int pos = 0; pos < no; ++pos) {
            const Combo& cb = sp.side[opp][ord[pos]];
            if (cb.a == c || cb.b == c) {
              cardPosIdx.push_back(pos);
              ++cardPosOff[cpo + c + 1];
            }
          }
        }
      }
    }
    ints("brOppSortedOff", oppSortedOff);
    ints("brOppSorted", oppSorted);
    ints("brLessOff", lessOff);
    ints("brLessEnd", lessEnd);
    ints("brTieEnd", tieEnd);
    ints("brCardPosOff", cardPosOff);
    ints("brCardPosIdx", cardPosIdx);
    ints("brRevSortedOff", revSortedOff);
    ints("brRevSorted", revSorted);

    // Fold nodes: per traverser combo, the node-local slot of the identical
    // combo in the opponent's list (cuda/gpu_cfr.cu:1754-1786).
    std::vector<int> foldSonOff(N, 0), foldSon;
    for (int u = 0; u < N; ++u) {
      const ONode& n = sp.nodes[u];
      if (n.kind != kFoldN) continue;
      foldSonOff[u] = (int)foldSon.size();
      for (int p = 0; p < 2; ++p) {
        std::vector<int> local(sp.side[1 - p].size(), -1);
        const std::vector<int>& lo = *n.list[1 - p];
        for (size_t j = 0; j < lo.size(); ++j) local[lo[j]] = (int)j;
        for (int b : *n.list[p]) {
          const int so = sp.same[p][b];
          foldSon.push_back(so >= 0 ? local[so] : -1);
        }
      }
    }
    ints("foldSonOff", foldSonOff);
    ints("foldSon", foldSon);
    std::vector<double> wd[2];
    for (int p = 0; p < 2; ++p)
      for (const Combo& c : sp.side[p]) wd[p].push_back(c.w);
    sink(user, "w0d", 'd', wd[0].data(), (int64_t)wd[0].size());
    sink(user, "w1d", 'd', wd[1].data(), (int64_t)wd[1].size());
    sink(user, "nodeBoard", 'B', nodeBoard.data(), (int64_t)nodeBoard.size());

    // Per-depth node lists and chance-branch prefixes (cuda/gpu_cfr.cu:1377-1421).
    const int D = maxDepth + 1;
    std::vector<int> decideCount(D, 0), chanceCount(D, 0), bwdCount(D, 0), chanceBrTotal(D, 0),
        decideList, chanceList, bwdList, chanceBrOff;
    std::vector<std::vector<int>> dl(D), cl(D), bl(D);
    for (int u = 0; u < N; ++u) {
      bl[depth[u]].push_back(u);
      if (sp.nodes[u].kind == kDecide) dl[depth[u]].push_back(u);
      if (sp.nodes[u].kind == kChance) cl[depth[u]].push_back(u);
    }
    for (int d = 0; d < D; ++d) {
      decideCount[d] = (int)dl[d].size();
      chanceCount[d] = (int)cl[d].size();
      bwdCount[d] = (int)bl[d].size();
      decideList.insert(decideList.end(), dl[d].begin(), dl[d].end());
      chanceList.insert(chanceList.end(), cl[d].begin(), cl[d].end());
      bwdList.insert(bwdList.end(), bl[d].begin(), bl[d].end());
      int acc = 0;
      chanceBrOff.push_back(0);
      for (int u : cl[d]) {
        acc += (int)sp.nodes[u].kids.size();
        chanceBrOff.push_back(acc);
      }
      chanceBrTotal[d] = acc;
    }
    ints("decideCount", decideCount);
    ints("chanceCount", chanceCount);
    ints("bwdCount", bwdCount);
    ints("chanceBrTotal", chanceBrTotal);
    ints("decideList", decideList);
    ints("chanceList", chanceList);
    ints("bwdList", bwdList);
    ints("chanceBrOff", chanceBrOff);

    std::vector<int> meta;
    for (int u = 0; u < N; ++u) {
      const ONode& n = sp.nodes[u];
      if (n.kind != kDecide) continue;
      const int row[8] = {regOff[u], n.na, n.player, n.player == 0 ? nC0[u] : nC1[u],
                          depth[u], n.nBoard, u, n.actBase};
      meta.insert(meta.end(), row, row + 8);
    }
    ints("decideMeta", meta);
    std::vector<uint8_t> actKind;
    std::vector<int64_t> actAmount;
    for (const Act& a : sp.acts) {
      actKind.push_back((uint8_t)a.kind);
      actAmount.push_back(a.amt);
    }
    sink(user, "actKind", 'B', actKind.data(), (int64_t)actKind.size());
    longs("actAmount", actAmount);
  }
};

}  // namespace

extern "C" {

struct orc_cfg {
  double bets[16];
  int n_bets;
  double raises[16];
  int n_raises;
  int allin, geo, max_raises;
  double add_t, force_t, merge_t;
};

// Builds the spot. w0/w1: 1326 combo weights; combos touching the board or
// with weight <= 0 are dropped (cuda/gpu_cfr.cu:1059-1076). precision 32
// or 64. Returns NULL if either side is empty.
void* orc_create(const uint8_t* board, int nBoard, const double* w0, const double* w1,
                 int64_t pot, int64_t stack, const orc_cfg* cfgs, int nCfgs, int precision) {
  auto* h = new Handle();
  h->precision = precision;
  Spot& sp = h->spot();
  sp.pot = pot;
  sp.stack = stack;
  sp.nBoard0 = nBoard;
  for (int k = 0; k < 3; ++k) {
    const orc_cfg& c = cfgs[nCfgs == 3 ? k : 0];
    Cfg& o = sp.cfg[k];
    o.bets.assign(c.bets, c.bets + c.n_bets);
    o.raises.assign(c.raises, c.raises + c.n_raises);
    o.allin = c.allin != 0;
    o.geo = c.geo != 0;
    o.maxRaises = c.max_raises;
    o.addT = c.add_t;
    o.forceT = c.force_t;
    o.mergeT = c.merge_t;
  }
  int idx = 0;
  int slot[2][52][52];
  std::memset(slot, -1, sizeof(slot));
  for (int a = 0; a < 52; ++a)
    for (int b = a + 1; b < 52; ++b, ++idx) {
      bool blocked = false;
      for (int i = 0; i < nBoard; ++i) blocked |= board[i] == a || board[i] == b;
      if (blocked) continue;
      if (w0[idx] > 0) {
        slot[0][a][b] = (int)sp.side[0].size();
        sp.side[0].push_back({a, b, w0[idx]});
      }
      if (w1[idx] > 0) {
        slot[1][a][b] = (int)sp.side[1].size();
        sp.side[1].push_back({a, b, w1[idx]});
      }
    }
  if (sp.side[0].empty() || sp.side[1].empty()) {
    delete h;
    return nullptr;
  }
  for (int p = 0; p < 2; ++p)
    for (const Combo& c : sp.side[p]) sp.same[p].push_back(slot[1 - p][c.a][c.b]);
  List lists[2];
  Keys keys[2];
  int bd[5] = {0, 0, 0, 0, 0};
  for (int i = 0; i < nBoard; ++i) bd[i] = board[i];
  for (int p = 0; p < 2; ++p) {
    lists[p] = std::make_shared<std::vector<int>>();
    for (int i = 0; i < (int)sp.side[p].size(); ++i) lists[p]->push_back(i);
    if (nBoard == 5) {
      keys[p] = std::make_shared<std::vector<uint64_t>>();
      for (const Combo& c : sp.side[p]) {
        const int seven[7] = {c.a, c.b, bd[0], bd[1], bd[2], bd[3], bd[4]};
        keys[p]->push_back(strength7(seven));
      }
    }
  }
  sp.build(bd, nBoard, pot, 0, 0, 0, false, false, 0, 0, 0, lists, keys);
  sp.assignRows();
  if (precision == 32) {
    h->s32.regret.assign(sp.rowTotal, 0.0f);
    h->s32.strat.assign(sp.rowTotal, 0.0f);
  } else {
    h->s64.f64 = true;
    h->s64.regretD.assign(sp.rowTotal, 0.0);
    h->s64.stratD.assign(sp.rowTotal, 0.0);
  }
  return h;
}

void orc_destroy(void* p) { delete (Handle*)p; }

// The reference's device layout of the spot (RefExport), array by array.
void orc_export(void* p, Sink sink, void* user) {
  RefExport e{((Handle*)p)->spot(), sink, user};
  e.run();
}
int orc_num_nodes(void* p) { return (int)((Handle*)p)->spot().nodes.size(); }
int64_t orc_row_total(void* p) { return ((Handle*)p)->spot().rowTotal; }

void orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// Runs n DCFR iterations with absolute indices t0 .. t0+n-1 of a schedule
// planned for `planned` iterations. The f32 mode rounds each coefficient to
// float, as the reference's device table does (cuda/gpu_cfr.cu:1887-1893).
void orc_iterate(void* p, int t0, int n, int planned, int sched) {
  Handle* h = (Handle*)p;
  for (int t = t0; t < t0 + n; ++t) {
    const Coef c = schedule(sched, t, planned);
    if (h->precision == 32) {
      const float cf[3] = {(float)c.pos, (float)c.neg, (float)c.avg};
      for (int tr = 0; tr < 2; ++tr) h->s32.walk(0, tr, h->s32.rootReach(tr), 0, cf);
    } else {
      const double cd[3] = {c.pos, c.neg, c.avg};
      for (int tr = 0; tr < 2; ++tr) h->s64.walk(0, tr, h->s64.rootReach(tr), 0, cd);
    }
  }
}

// Value walk in f64 over the current rows (mode 1 = EV vs the average
// strategy, 2 = best response): root value in chips; rootRow (optional)
// gets the traverser's per-combo root values.
double orc_value(void* p, int tr, int mode, double* rootRow) {
  Handle* h = (Handle*)p;
  Solver<double> w;
  w.sp = h->spot();
  w.f64 = true;
  if (h->precision == 32) {
    w.regretD.assign(h->s32.regret.begin(), h->s32.regret.end());
    w.stratD.assign(h->s32.strat.begin(), h->s32.strat.end());
  } else {
    w.regretD = h->s64.regretD;
    w.stratD = h->s64.stratD;
  }
  const double zero[3] = {0, 0, 0};
  const std::vector<double> v = w.walk(0, tr, w.rootReach(tr), mode, zero);
  double s = 0;
  for (size_t i = 0; i < v.size(); ++i) {
    s += w.sp.side[tr][i].w * v[i];
    if (rootRow) rootRow[i] = v[i];
  }
  const double Z = pairMass(w.sp);
  return Z > 0 ? s / Z : 0.0;
}

void orc_rows(void* p, int which, float* out) {
  Handle* h = (Handle*)p;
  if (h->precision == 32) {
    const std::vector<float>& v = which == 0 ? h->s32.regret : h->s32.strat;
    std::copy(v.begin(), v.end(), out);
  } else {
    const std::vector<double>& v = which == 0 ? h->s64.regretD : h->s64.stratD;
    for (size_t i = 0; i < v.size(); ++i) out[i] = (float)v[i];
  }
}

void orc_set_rows(void* p, int which, const float* in) {
  Handle* h = (Handle*)p;
  const int64_t n = h->spot().rowTotal;
  if (h->precision == 32) {
    std::vector<float>& v = which == 0 ? h->s32.regret : h->s32.strat;
    std::copy(in, in + n, v.begin());
  } else {
    std::vector<double>& v = which == 0 ? h->s64.regretD : h->s64.stratD;
    for (int64_t i = 0; i < n; ++i) v[i] = in[i];
  }
}

double orc_pair_mass(void* p) { return pairMass(((Handle*)p)->spot()); }

// Strength key of one 7-card hand (reference packing).
uint64_t orc_strength7(const uint8_t* c) {
  const int k[7] = {c[0], c[1], c[2], c[3], c[4], c[5], c[6]};
  return strength7(k);
}

// Bet abstraction of one state; returns the action count, kinds/amounts in
// out (room for 64).
int orc_actions(int64_t potBase, int64_t stack, const orc_cfg* c, int64_t sc0, int64_t sc1,
                int actor, int afterAllin, int numBets, int streets, int* kinds,
                int64_t* amounts) {
  Cfg o;
  o.bets.assign(c->bets, c->bets + c->n_bets);
  o.raises.assign(c->raises, c->raises + c->n_raises);
  o.allin = c->allin != 0;
  o.geo = c->geo != 0;
  o.maxRaises = c->max_raises;
  o.addT = c->add_t;
  o.forceT = c->force_t;
  o.mergeT = c->merge_t;
  const std::vector<Act> v =
      actionsOf(potBase, stack, o, sc0, sc1, actor, afterAllin != 0, numBets, streets);
  for (size_t i = 0; i < v.size() && i < 64; ++i) {
    kinds[i] = v[i].kind;
    amounts[i] = v[i].amt;
  }
  return (int)v.size();
}

}  // extern "C"
