// Host tree compiler (see compiler.h).
#include "compiler.h"

#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>
#include <utility>

#include "pps_gb.h"

namespace pps {
namespace gb {

namespace {

class Builder {
 public:
  explicit Builder(Tree& t) : t_(t) {}

  // Node creation mirrors the recursion of cuda/gpu_cfr.cu:1116-1326:
  // the node is numbered before its children (pre-order) and fold nodes
  // are created inline by their decide parent.
  int build(int state, int64_t potBase, int64_t sc0, int64_t sc1, int actor,
            bool afterAllin, bool closed, int depth, int64_t pc0, int64_t pc1,
            int numBets, int parent) {
    const int idx = newNode(state, potBase, sc0, sc1, pc0, pc1, depth, parent);
    const int64_t stack = t_.spot.stack;
    // Nothing behind after the earlier streets: the street is dead.
    if (!closed && stack - pc0 <= 0) closed = true;
    const int nBoard = t_.states[state].nBoard;

    if (closed) {
      if (nBoard == 5) {
        t_.nodes[idx].kind = kShowdown;
        return idx;
      }
      t_.nodes[idx].kind = kChance;
      uint64_t onBoard = 0;
      for (int i = 0; i < nBoard; ++i) onBoard |= 1ull << t_.states[state].board[i];
      int kids[52];
      int nk = 0;
      for (int c = 0; c < 52; ++c) {
        if ((onBoard >> c) & 1ull) continue;
        const int cs = childState(state, c);
        kids[nk++] = build(cs, potBase + sc0 + sc1, 0, 0, 0, false, false, depth + 1,
                           pc0 + sc0, pc1 + sc1, 0, idx);
      }
      setKids(idx, kids, nk);
      return idx;
    }

    const std::vector<pf::TreeAction>& acts =
        actionsFor(potBase, stack - pc0, nBoard, sc0, sc1, actor, afterAllin, numBets);
    {
      Node& nd = t_.nodes[idx];
      nd.kind = kDecide;
      nd.player = (uint8_t)actor;
      nd.na = (uint8_t)acts.size();
      nd.actBase = (int)t_.actions.size();
    }
    t_.maxNa = std::max<int>(t_.maxNa, (int)acts.size());
    t_.actions.insert(t_.actions.end(), acts.begin(), acts.end());

    int kids[kMaxActions];
    int nk = 0;
    for (const pf::TreeAction& act : acts) {
      int64_t nsc0 = sc0, nsc1 = sc1;
      bool nAfterAllin = afterAllin;
      bool streetEnds = false;
      int child = -1;
      switch (act.kind) {
        case pf::ActionKind::Check:
          if (actor == 0)
            child = build(state, potBase, sc0, sc1, 1, afterAllin, false,
                          depth + 1, pc0, pc1, numBets, idx);
          else
            streetEnds = true;  // IP checks behind
          break;
        case pf::ActionKind::Fold: {
          child = newNode(state, potBase, sc0, sc1, pc0, pc1, depth + 1, idx);
          t_.nodes[child].kind = kFold;
          t_.nodes[child].foldBy = (uint8_t)actor;
          break;
        }
        case pf::ActionKind::Call:
          (actor == 0 ? nsc0 : nsc1) = std::max(sc0, sc1);
          streetEnds = true;
          break;
        default:  // Bet, Raise, AllIn
          if (act.kind == pf::ActionKind::AllIn) nAfterAllin = true;
          (actor == 0 ? nsc0 : nsc1) = act.amount;
          break;
      }
      if (streetEnds)
        child = build(state, potBase, nsc0, nsc1, 0, false, true, depth + 1,
                      pc0, pc1, 0, idx);
      else if (child < 0)
        child = build(state, potBase, nsc0, nsc1, actor ^ 1, nAfterAllin,
                      false, depth + 1, pc0, pc1,
                      act.kind == pf::ActionKind::Check ? numBets : numBets + 1,
                      idx);
      kids[nk++] = child;
    }
    setKids(idx, kids, nk);
    return idx;
  }

  // The number of nodes build() creates from the same arguments, so the
  // node arrays are sized once (a runout's subtree depends only on the
  // betting state, so equal states are counted once). Any mismatch would
  // only cost growth; the tree itself comes from build().
  int64_t count(int nBoard, int64_t potBase, int64_t sc0, int64_t sc1, int actor,
                bool afterAllin, bool closed, int64_t pc0, int64_t pc1, int numBets) {
    const int64_t stack = t_.spot.stack;
    if (!closed && stack - pc0 <= 0) closed = true;
    const auto key = std::make_tuple(nBoard, potBase, sc0, sc1, actor, afterAllin, closed, pc0,
                                     pc1, numBets);
    auto it = counts_.find(key);
    if (it != counts_.end()) return it->second;
    int64_t n = 1;
    if (closed) {
      if (nBoard < 5)
        n += (int64_t)(52 - nBoard) * count(nBoard + 1, potBase + sc0 + sc1, 0, 0, 0, false,
                                            false, pc0 + sc0, pc1 + sc1, 0);
    } else {
      const std::vector<pf::TreeAction>& acts =
          actionsFor(potBase, stack - pc0, nBoard, sc0, sc1, actor, afterAllin, numBets);
      for (const pf::TreeAction& act : acts) {
        int64_t nsc0 = sc0, nsc1 = sc1;
        switch (act.kind) {
          case pf::ActionKind::Check:
            n += actor == 0 ? count(nBoard, potBase, sc0, sc1, 1, afterAllin, false, pc0, pc1,
                                    numBets)
                            : count(nBoard, potBase, sc0, sc1, 0, false, true, pc0, pc1, 0);
            break;
          case pf::ActionKind::Fold:
            n += 1;
            break;
          case pf::ActionKind::Call:
            (actor == 0 ? nsc0 : nsc1) = std::max(sc0, sc1);
            n += count(nBoard, potBase, nsc0, nsc1, 0, false, true, pc0, pc1, 0);
            break;
          default:
            (actor == 0 ? nsc0 : nsc1) = act.amount;
            n += count(nBoard, potBase, nsc0, nsc1, actor ^ 1,
                       afterAllin || act.kind == pf::ActionKind::AllIn, false, pc0, pc1,
                       numBets + 1);
            break;
        }
      }
    }
    counts_.emplace(key, n);
    return n;
  }

  void reserve(int64_t nodes) {
    if (nodes <= 0 || nodes > (int64_t)1 << 31) return;
    t_.nodes.reserve((size_t)nodes);
    kidOff_.reserve((size_t)nodes);
    kidCnt_.reserve((size_t)nodes);
    kidFlat_.reserve((size_t)nodes);
  }

  void flattenChildren() {
    t_.children.clear();
    t_.children.reserve(kidFlat_.size());
    for (size_t u = 0; u < t_.nodes.size(); ++u) {
      t_.nodes[u].childBase = (int)t_.children.size();
      t_.nodes[u].nChildren = kidCnt_[u];
      t_.children.insert(t_.children.end(), kidFlat_.begin() + kidOff_[u],
                         kidFlat_.begin() + kidOff_[u] + kidCnt_[u]);
    }
  }

 private:
  // The action list of a betting state. The same states recur under every
  // runout, so each distinct argument tuple is computed once.
  struct ActKey {
    int64_t potBase, stack, sc0, sc1;
    int nBoard, actor, numBets;
    bool afterAllin;
    bool operator<(const ActKey& o) const {
      return std::tie(potBase, stack, sc0, sc1, nBoard, actor, numBets, afterAllin) <
             std::tie(o.potBase, o.stack, o.sc0, o.sc1, o.nBoard, o.actor, o.numBets,
                      o.afterAllin);
    }
  };
  const std::vector<pf::TreeAction>& actionsFor(int64_t potBase, int64_t stack, int nBoard,
                                                int64_t sc0, int64_t sc1, int actor,
                                                bool afterAllin, int numBets) {
    const ActKey key{potBase, stack, sc0, sc1, nBoard, actor, numBets, afterAllin};
    auto it = acts_.find(key);
    if (it != acts_.end()) return it->second;
    std::vector<pf::TreeAction> acts = pf::betActions(
        potBase, stack, t_.cfgFor(nBoard), sc0, sc1, actor, afterAllin, numBets, 6 - nBoard);
    if ((int)acts.size() > kMaxActions)
      throw Error{PPS_GB_E_TOO_WIDE,
                  "bet config too wide (max actions " +
                      std::to_string(acts.size()) + " > " +
                      std::to_string(kMaxActions) + ")"};
    return acts_.emplace(key, std::move(acts)).first->second;
  }

  // Children are recorded when a node's subtree is complete (post-order)
  // and put back in node order by flattenChildren.
  void setKids(int idx, const int* kids, int nk) {
    kidOff_[idx] = (int64_t)kidFlat_.size();
    kidCnt_[idx] = nk;
    kidFlat_.insert(kidFlat_.end(), kids, kids + nk);
  }

  Tree& t_;
  std::vector<int> kidFlat_, kidCnt_;
  std::vector<int64_t> kidOff_;
  std::map<ActKey, std::vector<pf::TreeAction>> acts_;
  std::map<std::tuple<int, int64_t, int64_t, int64_t, int, bool, bool, int64_t, int64_t, int>,
           int64_t>
      counts_;
  std::vector<int> dealt_;  // [state * 52 + card] -> dealt state, or -1
  int rivers_ = -1;         // river states so far (counted on first use)

  int newNode(int state, int64_t potBase, int64_t sc0, int64_t sc1,
              int64_t pc0, int64_t pc1, int depth, int parent) {
    Node nd;
    nd.state = state;
    nd.potBase = potBase;
    nd.sc0 = sc0;
    nd.sc1 = sc1;
    nd.pc0 = pc0;
    nd.pc1 = pc1;
    nd.depth = depth;
    nd.parent = parent;
    t_.nodes.push_back(nd);
    kidOff_.push_back(0);
    kidCnt_.push_back(0);
    return (int)t_.nodes.size() - 1;
  }

  // The state reached by dealing `card` from state `ps` (interned): its
  // lists are the parent's minus every combo holding the card.
  int childState(int ps, int card) {
    const size_t key = (size_t)ps * 52 + (size_t)card;
    if (dealt_.size() < t_.states.size() * 52) dealt_.resize(t_.states.size() * 52, -1);
    if (dealt_[key] >= 0) return dealt_[key];
    BoardState s;
    s.parent = ps;
    s.dealt = card;
    s.nBoard = t_.states[ps].nBoard + 1;
    std::memcpy(s.board, t_.states[ps].board, 5);
    s.board[s.nBoard - 1] = (uint8_t)card;
    for (int p = 0; p < 2; ++p) {
      const Side& sd = t_.side[p];
      for (uint16_t slot : t_.states[ps].list[p])
        if (sd.cards[2 * slot] != card && sd.cards[2 * slot + 1] != card)
          s.list[p].push_back(slot);
    }
    if (s.nBoard == 5) {
      if (rivers_ < 0) {
        rivers_ = 0;
        for (const BoardState& o : t_.states) rivers_ += o.nBoard == 5;
      }
      s.riverIndex = rivers_++;
    }
    t_.states.push_back(std::move(s));
    const int id = (int)t_.states.size() - 1;
    dealt_[key] = id;
    return id;
  }
};

}  // namespace

Tree compileTree(const gpu::PostflopSpot& spot,
                 const gpu::StreetBetConfigs& cfgs, bool perStreet) {
  if (spot.nBoard < 3 || spot.nBoard > 5)
    throw Error{PPS_GB_E_ARG, "board must be 3, 4 or 5 cards"};
  uint64_t used = 0;
  for (int i = 0; i < spot.nBoard; ++i) {
    if (spot.board[i] >= 52) throw Error{PPS_GB_E_ARG, "bad board card id"};
    if ((used >> spot.board[i]) & 1ull)
      throw Error{PPS_GB_E_ARG, "duplicate board card"};
    used |= 1ull << spot.board[i];
  }
  for (int k = 0; k < 3; ++k)
    if ((int)cfgs.street[k].betFracs.size() > PPS_GB_MAX_SIZES ||
        (int)cfgs.street[k].raiseMults.size() > PPS_GB_MAX_SIZES)
      throw Error{PPS_GB_E_ARG, "too many bet or raise sizes"};

  Tree t;
  t.spot = spot;
  t.cfgs = cfgs;
  t.perStreet = perStreet;
  // Base lists: combo order (a < b ascending), board-blocked and
  // non-positive weights dropped (cuda/gpu_cfr.cu:1059-1076).
  for (int p = 0; p < 2; ++p) {
    const Range& r = p == 0 ? spot.oop : spot.ip;
    Side& sd = t.side[p];
    for (int i = 0; i < kCombos; ++i) {
      uint8_t a, b;
      comboCards(i, a, b);
      if ((used >> a) & 1ull || (used >> b) & 1ull || !(r.w[i] > 0.0)) continue;
      sd.cards.push_back(a);
      sd.cards.push_back(b);
      sd.w.push_back(r.w[i]);
      ++sd.n;
    }
  }
  for (int p = 0; p < 2; ++p) {
    std::vector<int> slotOf(kCombos, -1);
    const Side& o = t.side[1 - p];
    for (int j = 0; j < o.n; ++j) slotOf[comboIndex(o.cards[2 * j], o.cards[2 * j + 1])] = j;
    Side& sd = t.side[p];
    sd.sameOther.resize(sd.n);
    for (int i = 0; i < sd.n; ++i)
      sd.sameOther[i] = slotOf[comboIndex(sd.cards[2 * i], sd.cards[2 * i + 1])];
  }
  if (t.side[0].n == 0 || t.side[1].n == 0) {
    t.empty = true;
    return t;
  }

  BoardState root;
  root.nBoard = spot.nBoard;
  std::memcpy(root.board, spot.board, 5);
  for (int i = spot.nBoard; i < 5; ++i) root.board[i] = 0;
  for (int p = 0; p < 2; ++p)
    for (int i = 0; i < t.side[p].n; ++i) root.list[p].push_back((uint16_t)i);
  if (root.nBoard == 5) root.riverIndex = 0;
  t.states.push_back(std::move(root));

  Builder b(t);
  b.reserve(b.count(spot.nBoard, spot.pot, 0, 0, 0, false, false, 0, 0, 0));
  b.build(0, spot.pot, 0, 0, 0, false, false, 0, 0, 0, 0, -1);
  b.flattenChildren();

  for (size_t u = 0; u < t.nodes.size(); ++u) {
    const Node& nd = t.nodes[u];
    t.maxDepth = std::max(t.maxDepth, nd.depth);
    if (nd.kind == kDecide) {
      t.decideNodes.push_back((int)u);
      t.rowTotal += (int64_t)nd.na * t.n((int)u, nd.player);
    }
  }
  return t;
}

std::vector<uint64_t> strengthKeys(const Tree& t, int p, const uint8_t b5[5]) {
  const Side& sd = t.side[p];
  std::vector<uint64_t> keys(sd.n);
  Card seven[7];
  for (int i = 0; i < 5; ++i) seven[2 + i] = b5[i];
  for (int i = 0; i < sd.n; ++i) {
    seven[0] = sd.cards[2 * i];
    seven[1] = sd.cards[2 * i + 1];
    keys[i] = handKey(evaluateN(seven, 7));
  }
  return keys;
}

// ---------------------------------------------------------------------------
// Reference-layout export.
// ---------------------------------------------------------------------------

namespace {

struct RefLayout {
  const Tree& t;
  std::vector<int> comboOff[2], comboId;
  std::vector<int> runOffOff, runOff, ctapBase, ctap;
  std::vector<int> expOffOff, expIdxBase, expOff, expIdx;

  explicit RefLayout(const Tree& tree) : t(tree) {
    const size_t N = t.nodes.size();
    for (int p = 0; p < 2; ++p) comboOff[p].assign(N, 0);
    runOffOff.assign(N, 0);
    ctapBase.assign(N, 0);
    expOffOff.assign(N, 0);
    expIdxBase.assign(N, 0);
    // Root lists are the identity base lists, side 0 then side 1.
    for (int p = 0; p < 2; ++p)
      for (int i = 0; i < t.side[p].n; ++i) comboId.push_back(i);
    walk(0, 0, t.side[0].n);
  }

  // Appends happen at the same moments as in the reference recursion:
  // runOff sections are reserved before a chance node's children,
  // each branch's child lists are appended right before that child is
  // built, and ctap/expOff/expIdx sections after all children.
  void walk(int u, int off0, int off1) {
    const Node& nd = t.nodes[u];
    comboOff[0][u] = off0;
    comboOff[1][u] = off1;
    if (nd.kind != kChance) {
      for (int k = 0; k < nd.nChildren; ++k)
        walk(t.children[nd.childBase + k], off0, off1);
      return;
    }
    const int nb = nd.nChildren;
    runOffOff[u] = (int)runOff.size();
    runOff.resize(runOff.size() + 2 * (nb + 1), 0);
    const BoardState& ps = t.states[nd.state];
    for (int br = 0; br < nb; ++br) {
      const int ch = t.children[nd.childBase + br];
      const BoardState& cs = t.states[t.nodes[ch].state];
      const int c0 = (int)comboId.size();
      comboId.insert(comboId.end(), cs.list[0].begin(), cs.list[0].end());
      const int c1 = (int)comboId.size();
      comboId.insert(comboId.end(), cs.list[1].begin(), cs.list[1].end());
      walk(ch, c0, c1);
    }
    ctapBase[u] = (int)ctap.size();
    for (int p = 0; p < 2; ++p) {
      const int base = runOffOff[u] + p * (nb + 1);
      int total = 0;
      for (int br = 0; br < nb; ++br) {
        runOff[base + br] = total;
        const int ch = t.children[nd.childBase + br];
        for (int j : parentSlots(ps, t.states[t.nodes[ch].state], p)) {
          ctap.push_back(j);
          ++total;
        }
      }
      runOff[base + nb] = total;
    }
    expOffOff[u] = (int)expOff.size();
    expIdxBase[u] = (int)expIdx.size();
    for (int p = 0; p < 2; ++p) {
      const int parentN = (int)ps.list[p].size();
      std::vector<std::vector<int>> perSlot(parentN);
      for (int br = 0; br < nb; ++br) {
        const int ch = t.children[nd.childBase + br];
        const auto par = parentSlots(ps, t.states[t.nodes[ch].state], p);
        for (int j = 0; j < (int)par.size(); ++j)
          perSlot[par[j]].push_back(br * 4096 + j);
      }
      int cnt = 0;
      for (int s = 0; s < parentN; ++s) {
        expOff.push_back(cnt);
        for (int e : perSlot[s]) expIdx.push_back(e);
        cnt += (int)perSlot[s].size();
      }
      expOff.push_back(cnt);
    }
  }

  // Parent node-local slot of each child-list entry.
  static std::vector<int> parentSlots(const BoardState& ps,
                                      const BoardState& cs, int p) {
    std::vector<int> out;
    size_t i = 0;
    for (uint16_t base : cs.list[p]) {
      while (ps.list[p][i] != base) ++i;
      out.push_back((int)i);
    }
    return out;
  }
};

}  // namespace

void exportReference(const Tree& t, const ArraySink& sink) {
  auto scalar = [&](const char* name, int64_t v) { sink(name, 'q', &v, 1); };
  auto ints = [&](const char* name, const std::vector<int>& v) {
    sink(name, 'i', v.data(), (int64_t)v.size());
  };
  auto longs = [&](const char* name, const std::vector<int64_t>& v) {
    sink(name, 'q', v.data(), (int64_t)v.size());
  };
  const int N = (int)t.nodes.size();
  scalar("numNodes", N);
  scalar("maxDepth", t.maxDepth);
  scalar("n0Base", t.side[0].n);
  scalar("n1Base", t.side[1].n);
  scalar("maxNa", t.maxNa);
  scalar("regTotal", t.rowTotal);
  if (t.empty) {
    scalar("reachTotal", 0);
    scalar("reachTotal0", 0);
    scalar("reachTotal1", 0);
    scalar("empty", 1);
    return;
  }

  RefLayout L(t);
  std::vector<int> kind(N), player(N), foldBy(N), na(N), childBase(N),
      boardId(N), nC0(N), nC1(N), regOff(N), cfvOff(N), reachOff0(N),
      reachOff1(N), nBranch(N), chanceQ(N);
  std::vector<int64_t> sc0(N), sc1(N), potBase(N), pc0(N), pc1(N);
  std::vector<uint8_t> nodeBoard((size_t)N * 5, 0);
  std::map<std::vector<uint8_t>, int> boards;  // showdown boards, first seen
  std::vector<int> boardState;                 // board id -> state
  int64_t reachTotal = 0, reachTotal0 = 0, reachTotal1 = 0, regTotal = 0;
  for (int u = 0; u < N; ++u) {
    const Node& nd = t.nodes[u];
    const BoardState& st = t.states[nd.state];
    kind[u] = nd.kind;
    player[u] = nd.kind == kDecide ? nd.player : 0;
    foldBy[u] = nd.kind == kFold ? nd.foldBy : 0;
    na[u] = nd.kind == kDecide ? nd.na : 0;
    childBase[u] = nd.childBase;
    nC0[u] = (int)st.list[0].size();
    nC1[u] = (int)st.list[1].size();
    sc0[u] = nd.sc0;
    sc1[u] = nd.sc1;
    potBase[u] = nd.potBase;
    pc0[u] = nd.pc0;
    pc1[u] = nd.pc1;
    nBranch[u] = nd.kind == kChance ? nd.nChildren : 0;
    chanceQ[u] = 52 - st.nBoard - 4;
    for (int i = 0; i < st.nBoard; ++i) nodeBoard[(size_t)u * 5 + i] = st.board[i];
    if (nd.kind == kShowdown) {
      std::vector<uint8_t> key(st.board, st.board + 5);
      auto it = boards.find(key);
      if (it == boards.end()) {
        it = boards.emplace(key, (int)boards.size()).first;
        boardState.push_back(nd.state);
      }
      boardId[u] = it->second;
    }
    const int row = std::max(nC0[u], nC1[u]);
    cfvOff[u] = (int)reachTotal;
    reachTotal += row;
    if (nd.kind == kDecide) {
      regOff[u] = (int)regTotal;
      regTotal += (int64_t)nd.na * (nd.player == 0 ? nC0[u] : nC1[u]);
    }
    // Reach rows alias the parent's row under a decide node of the layout's
    // traverser (cuda/gpu_cfr.cu:1491-1514).
    const int par = nd.parent;
    const bool parDecide = par >= 0 && t.nodes[par].kind == kDecide;
    if (parDecide && t.nodes[par].player == 0) reachOff0[u] = reachOff0[par];
    else { reachOff0[u] = (int)reachTotal0; reachTotal0 += row; }
    if (parDecide && t.nodes[par].player == 1) reachOff1[u] = reachOff1[par];
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
  ints("childFlat", t.children);
  ints("boardId", boardId);
  ints("nC0", nC0);
  ints("nC1", nC1);
  ints("comboOff0", L.comboOff[0]);
  ints("comboOff1", L.comboOff[1]);
  ints("comboId", L.comboId);
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
  ints("runOffOff", L.runOffOff);
  ints("runOff", L.runOff);
  ints("ctapBase", L.ctapBase);
  ints("ctap", L.ctap);
  ints("expOffOff", L.expOffOff);
  ints("expIdxBase", L.expIdxBase);
  ints("expOff", L.expOff);
  ints("expIdx", L.expIdx);
  for (int p = 0; p < 2; ++p) {
    std::vector<float> wf(t.side[p].w.begin(), t.side[p].w.end());
    sink(p == 0 ? "w0" : "w1", 'f', wf.data(), (int64_t)wf.size());
    sink(p == 0 ? "cards0" : "cards1", 'B', t.side[p].cards.data(),
         (int64_t)t.side[p].cards.size());
    ints(p == 0 ? "sameOther0" : "sameOther1", t.side[p].sameOther);
  }

  // Strength tables per (showdown board, traverser) over the full base
  // lists (cuda/gpu_cfr.cu:1594-1703).
  const int nTables = (int)boards.size() * 2;
  std::vector<int> oppSortedOff(nTables + 1, 0), oppSorted, lessOff(nTables + 1, 0),
      lessEnd, tieEnd, cardPosOff(nTables * 53 + 1, 0), cardPosIdx,
      revSortedOff(nTables + 1, 0), revSorted;
  for (int bid = 0; bid < (int)boards.size(); ++bid) {
    const BoardState& st = t.states[boardState[bid]];
    std::vector<uint64_t> key[2] = {strengthKeys(t, 0, st.board),
                                    strengthKeys(t, 1, st.board)};
    for (int tr = 0; tr < 2; ++tr) {
      const int ti = bid * 2 + tr, opp = 1 - tr;
      const Side& so = t.side[opp];
      std::vector<int> ord(so.n);
      for (int i = 0; i < so.n; ++i) ord[i] = i;
      std::stable_sort(ord.begin(), ord.end(),
                       [&](int x, int y) { return key[opp][x] < key[opp][y]; });
      oppSortedOff[ti] = (int)oppSorted.size();
      oppSorted.insert(oppSorted.end(), ord.begin(), ord.end());
      // Node-local slot of each base slot in this board's opponent list.
      std::vector<int> local(so.n, -1);
      for (size_t j = 0; j < st.list[opp].size(); ++j) local[st.list[opp][j]] = (int)j;
      revSortedOff[ti] = (int)revSorted.size();
      for (int k = 0; k < so.n; ++k) revSorted.push_back(local[ord[k]]);
      lessOff[ti] = (int)lessEnd.size();
      for (int i = 0; i < t.side[tr].n; ++i) {
        const uint64_t s = key[tr][i];
        auto lo = std::lower_bound(ord.begin(), ord.end(), s,
                                   [&](int o, uint64_t v) { return key[opp][o] < v; });
        auto hi = std::upper_bound(lo, ord.end(), s,
                                   [&](uint64_t v, int o) { return v < key[opp][o]; });
        lessEnd.push_back((int)(lo - ord.begin()));
        tieEnd.push_back((int)(hi - ord.begin()));
      }
      const int cpo = ti * 53;
      cardPosOff[cpo] = (int)cardPosIdx.size();
      for (int c = 0; c < 52; ++c) {
        cardPosOff[cpo + c + 1] = cardPosOff[cpo + c];
        for (int pos = 0; pos < so.n; ++pos) {
          const int o = ord[pos];
          if (so.cards[2 * o] == c || so.cards[2 * o + 1] == c) {
            cardPosIdx.push_back(pos);
            ++cardPosOff[cpo + c + 1];
          }
        }
      }
    }
  }
  // The reference leaves the trailing slots of these offset tables at 0.
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
  // combo in the opponent list (cuda/gpu_cfr.cu:1754-1786).
  std::vector<int> foldSonOff(N, 0), foldSon;
  for (int u = 0; u < N; ++u) {
    if (t.nodes[u].kind != kFold) continue;
    foldSonOff[u] = (int)foldSon.size();
    const BoardState& st = t.states[t.nodes[u].state];
    for (int p = 0; p < 2; ++p) {
      std::vector<int> local(t.side[1 - p].n, -1);
      for (size_t j = 0; j < st.list[1 - p].size(); ++j) local[st.list[1 - p][j]] = (int)j;
      for (uint16_t base : st.list[p]) {
        const int so = t.side[p].sameOther[base];
        foldSon.push_back(so >= 0 ? local[so] : -1);
      }
    }
  }
  ints("foldSonOff", foldSonOff);
  ints("foldSon", foldSon);
  std::vector<double> w0(t.side[0].w), w1(t.side[1].w);
  sink("w0d", 'd', w0.data(), (int64_t)w0.size());
  sink("w1d", 'd', w1.data(), (int64_t)w1.size());
  sink("nodeBoard", 'B', nodeBoard.data(), (int64_t)nodeBoard.size());

  // Depth lists (cuda/gpu_cfr.cu:1377-1421).
  const int D = t.maxDepth + 1;
  std::vector<int> decideCount(D, 0), chanceCount(D, 0), bwdCount(D, 0),
      chanceBrTotal(D, 0), decideList, chanceList, bwdList, chanceBrOff;
  std::vector<std::vector<int>> dl(D), cl(D), bl(D);
  for (int u = 0; u < N; ++u) {
    const Node& nd = t.nodes[u];
    bl[nd.depth].push_back(u);
    if (nd.kind == kDecide) dl[nd.depth].push_back(u);
    if (nd.kind == kChance) cl[nd.depth].push_back(u);
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
      acc += t.nodes[u].nChildren;
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
  for (int u : t.decideNodes) {
    const Node& nd = t.nodes[u];
    const int row[8] = {regOff[u], nd.na, nd.player, nd.player == 0 ? nC0[u] : nC1[u],
                        nd.depth, t.states[nd.state].nBoard, u, nd.actBase};
    meta.insert(meta.end(), row, row + 8);
  }
  ints("decideMeta", meta);
  std::vector<uint8_t> actKind;
  std::vector<int64_t> actAmount;
  for (const auto& a : t.actions) {
    actKind.push_back((uint8_t)a.kind);
    actAmount.push_back(a.amount);
  }
  sink("actKind", 'B', actKind.data(), (int64_t)actKind.size());
  longs("actAmount", actAmount);
}

}  // namespace gb
}  // namespace pps
