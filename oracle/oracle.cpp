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
};

struct Spot {
  std::vector<Combo> side[2];
  std::vector<int> same[2];  // base -> identical base on the other side
  int64_t pot = 0, stack = 0;
  Cfg cfg[3];
  std::vector<ONode> nodes;
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
