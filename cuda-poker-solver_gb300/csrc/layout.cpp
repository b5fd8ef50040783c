// Device layout builder (see layout.h).
#include "layout.h"

#include <algorithm>
#include <atomic>
#include <exception>
#include <map>
#include <mutex>
#include <numeric>
#include <stdexcept>
#include <thread>

#include "pps_gb.h"

namespace pps {
namespace gb {

namespace {

// Tables that kernels stage into shared memory start on a 16-byte boundary
// so they can be copied with 16-byte vector loads (and a copy that rounds
// the table up to whole 16-byte chunks stays inside the pool).
void alignU16(std::vector<uint16_t>& pool) {
  while (pool.size() % 8) pool.push_back(0);
}
void alignI16(std::vector<int16_t>& pool) {
  while (pool.size() % 8) pool.push_back(0);
}
void alignU8(std::vector<uint8_t>& pool) {
  while (pool.size() % 16) pool.push_back(0);
}

int appendU16(std::vector<uint16_t>& pool, const std::vector<int>& v) {
  const int off = (int)pool.size();
  for (int x : v) pool.push_back((uint16_t)x);
  return off;
}

int appendI16(std::vector<int16_t>& pool, const std::vector<int>& v) {
  const int off = (int)pool.size();
  for (int x : v) pool.push_back((int16_t)x);
  return off;
}

// Slot of base combo `base` in an ascending list, or -1.
int slotOf(const std::vector<uint16_t>& list, int base) {
  auto it = std::lower_bound(list.begin(), list.end(), (uint16_t)base);
  return it != list.end() && *it == base ? (int)(it - list.begin()) : -1;
}

// One board state's tables (see StateDev), before they go into the pools.
struct StateParts {
  std::vector<uint8_t> cards[2];
  std::vector<int> starts[2], entries[2], same[2], up[2], down[2];
  int maxCardSeg = 0;
  std::vector<int> ord[2], segStart[2], segSlot[2];  // river states
  std::vector<ShowdownInfo> info[2];
};

// Reorders one traverser's showdown entries within each kSdWindow-entry
// window (the combos one warp evaluates together). A float4 gather from shared memory is
// served a quarter warp (eight lanes) at a time, and lanes whose indices
// fall in one 16-byte bank group (index mod 8) at different addresses are
// served one after another: list order puts about two such collisions in
// every quarter warp and gather. The window's entries are dealt to its
// quarter warps greedily (each slot takes the remaining entry that adds the
// fewest collisions over the loop's ten gathers, the lowest index on ties),
// and z bits 24-28 record each entry's offset in list order.
void spreadShowdownBanks(std::vector<ShowdownInfo>& info) {
  constexpr int kG = 10;
  const int n = (int)info.size();
  for (int w0 = 0; w0 < n; w0 += kSdWindow) {
    const int m = std::min(kSdWindow, n - w0);
    int A[kSdWindow][kG];
    for (int k = 0; k < m; ++k) {
      const ShowdownInfo& f = info[w0 + k];
      const int sHi = (int)((f.x >> 24) | ((f.y >> 16) & 0xf00));
      const int v[kG] = {(int)(f.x & 0xfff), (int)((f.x >> 12) & 0xfff), (int)(f.y & 0xfff),
                         (int)((f.y >> 12) & 0xfff), (int)(f.z & 0xfff), (int)((f.z >> 12) & 0xfff),
                         sHi, sHi - 1 - (int)((f.w >> 28) & 1), (int)(f.w & 0x7ff),
                         (int)((f.w >> 11) & 0x7ff)};
      std::copy(v, v + kG, A[k]);
    }
    bool used[kSdWindow] = {};
    ShowdownInfo out[kSdWindow];
    int pos = 0;
    for (int q0 = 0; q0 < m; q0 += 8) {
      // Per gather: the quarter warp's distinct indices and, per bank group,
      // how many of them it holds.
      int addr[kG][8], na[kG] = {}, cnt[kG][8] = {}, top[kG] = {};
      for (int s = 0; s < std::min(8, m - q0); ++s) {
        int best = -1, bestCost = 1 << 30;
        for (int k = 0; k < m; ++k) {
          if (used[k]) continue;
          int cost = 0;
          for (int g = 0; g < kG; ++g) {
            const int a = A[k][g];
            bool dup = false;
            for (int j = 0; j < na[g]; ++j) dup |= addr[g][j] == a;
            if (!dup && cnt[g][a & 7] + 1 > top[g]) ++cost;
          }
          if (cost < bestCost) {
            bestCost = cost;
            best = k;
          }
        }
        used[best] = true;
        for (int g = 0; g < kG; ++g) {
          const int a = A[best][g];
          bool dup = false;
          for (int j = 0; j < na[g]; ++j) dup |= addr[g][j] == a;
          if (dup) continue;
          addr[g][na[g]++] = a;
          top[g] = std::max(top[g], ++cnt[g][a & 7]);
        }
        out[pos] = info[w0 + best];
        out[pos].z |= (uint32_t)best << 24;
        ++pos;
      }
    }
    std::copy(out, out + m, info.begin() + w0);
  }
}

void buildStateParts(const Tree& t, int s, StateParts& P) {
  const BoardState& st = t.states[s];
  for (int p = 0; p < 2; ++p) {
    const Side& side = t.side[p];
    const auto& list = st.list[p];
    const int n = (int)list.size();
    P.cards[p].reserve(2 * (size_t)n);
    for (uint16_t b : list) {
      P.cards[p].push_back(side.cards[2 * b]);
      P.cards[p].push_back(side.cards[2 * b + 1]);
    }
    // Card segments: per card, the slots holding it in ascending order
    // (one counting pass, one filling pass).
    std::vector<int> count(52, 0);
    for (int j = 0; j < n; ++j) {
      ++count[side.cards[2 * list[j]]];
      ++count[side.cards[2 * list[j] + 1]];
    }
    std::vector<int>& starts = P.starts[p];
    starts.assign(53, 0);
    for (int c = 0; c < 52; ++c) {
      starts[c + 1] = starts[c] + count[c];
      P.maxCardSeg = std::max(P.maxCardSeg, count[c]);
    }
    P.entries[p].assign(starts[52], 0);
    std::vector<int> fill(starts.begin(), starts.begin() + 52);
    for (int j = 0; j < n; ++j) {
      P.entries[p][fill[side.cards[2 * list[j]]]++] = j;
      P.entries[p][fill[side.cards[2 * list[j] + 1]]++] = j;
    }
    P.same[p].assign(n, -1);
    for (int j = 0; j < n; ++j) {
      const int so = side.sameOther[list[j]];
      if (so >= 0) P.same[p][j] = slotOf(st.list[1 - p], so);
    }
    if (st.parent >= 0) {
      const auto& plist = t.states[st.parent].list[p];
      std::vector<int>& up = P.up[p];
      std::vector<int>& down = P.down[p];
      up.assign(n, 0);
      down.assign(plist.size(), -1);
      size_t i = 0;
      for (int j = 0; j < n; ++j) {
        while (plist[i] != list[j]) ++i;
        up[j] = (int)i;
        down[i] = j;
      }
    }
  }
  if (st.nBoard != 5) return;

  // River strength tables over this state's own lists.
  std::vector<uint64_t> keyBase[2] = {strengthKeys(t, 0, st.board),
                                      strengthKeys(t, 1, st.board)};
  for (int tr = 0; tr < 2; ++tr) {
    const int opp = 1 - tr;
    const auto& ol = st.list[opp];
    const auto& tl = st.list[tr];
    const int no = (int)ol.size();
    std::vector<int>& ord = P.ord[tr];
    ord.resize(no);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
      return keyBase[opp][ol[a]] < keyBase[opp][ol[b]];
    });
    std::vector<uint64_t> sortedKey(no);
    std::vector<int> posOfSlot(no);  // opponent slot -> sorted position
    for (int k = 0; k < no; ++k) {
      sortedKey[k] = keyBase[opp][ol[ord[k]]];
      posOfSlot[ord[k]] = k;
    }
    std::vector<int>& segStart = P.segStart[tr];
    std::vector<int>& segSlot = P.segSlot[tr];
    segStart.assign(53, 0);
    std::vector<std::vector<int>> posOfCard(52);
    for (int k = 0; k < no; ++k) {
      const int b = ol[ord[k]];
      posOfCard[t.side[opp].cards[2 * b]].push_back(k);
      posOfCard[t.side[opp].cards[2 * b + 1]].push_back(k);
    }
    for (int c = 0; c < 52; ++c) {
      segStart[c] = (int)segSlot.size();
      for (int k : posOfCard[c]) segSlot.push_back(ord[k]);
    }
    segStart[52] = (int)segSlot.size();
    P.info[tr].reserve(tl.size());
    for (int i = 0; i < (int)tl.size(); ++i) {
      const int b = tl[i];
      const uint64_t key = keyBase[tr][b];
      const int le = (int)(std::lower_bound(sortedKey.begin(), sortedKey.end(), key) -
                           sortedKey.begin());
      const int te = (int)(std::upper_bound(sortedKey.begin(), sortedKey.end(), key) -
                           sortedKey.begin());
      const int c1 = t.side[tr].cards[2 * b], c2 = t.side[tr].cards[2 * b + 1];
      auto below = [&](int c, int pos) {
        const auto& v = posOfCard[c];
        return (int)(std::lower_bound(v.begin(), v.end(), pos) - v.begin());
      };
      const int so = t.side[tr].sameOther[b];
      const int same = so >= 0 ? slotOf(ol, so) : -1;
      const int len1 = (int)posOfCard[c1].size(), len2 = (int)posOfCard[c2].size();
      // The identical combo's entry in card c1's segment (it holds c1), plus
      // one; 0: none.
      int ks1 = 0;
      if (same >= 0) {
        const auto& v = posOfCard[c1];
        ks1 = (int)(std::lower_bound(v.begin(), v.end(), posOfSlot[same]) - v.begin()) + 1;
      }
      // Segment prefix runs: card c's run starts at seg[c] + c (one more
      // entry than the segment); the kernels address entry k of the
      // concatenated runs at pad8(k).
      const int a1 = segStart[c1] + c1, a2 = segStart[c2] + c2;
      const int x1le = pad8(a1 + below(c1, le)), x1te = pad8(a1 + below(c1, te));
      const int x1end = pad8(a1 + len1);
      const int x2le = pad8(a2 + below(c2, le)), x2te = pad8(a2 + below(c2, te));
      const int x2end = pad8(a2 + len2);
      // The identical combo: the step of card c1's run at its entry (prefix
      // after it minus prefix before it); without one, two in-range
      // entries that the kernels read and discard.
      const int sHi = ks1 > 0 ? pad8(a1 + ks1) : 2;
      const int sStep = ks1 > 0 ? sHi - pad8(a1 + ks1 - 1) : 1;
      const int pLe = pad8(le), pTe = pad8(te);
      if (x1end >= 4096 || x2end >= 4096 || sHi >= 4096 || pTe >= 2048 || (te >> 8) >= 8)
        throw Error{PPS_GB_E_FORMAT, "showdown table entry out of range"};
      ShowdownInfo info;
      info.x = (uint32_t)x1le | ((uint32_t)x1te << 12) | ((uint32_t)(sHi & 0xff) << 24);
      info.y = (uint32_t)x1end | ((uint32_t)x2le << 12) | ((uint32_t)(sHi >> 8) << 24);
      info.z = (uint32_t)x2te | ((uint32_t)x2end << 12);
      info.w = (uint32_t)pLe | ((uint32_t)pTe << 11) | ((uint32_t)(le >> 8) << 22) |
               ((uint32_t)(te >> 8) << 25) | ((uint32_t)(sStep - 1) << 28) |
               ((uint32_t)(ks1 > 0) << 29);
      P.info[tr].push_back(info);
    }
    spreadShowdownBanks(P.info[tr]);
  }
}

// Helper threads running across all parallelFor calls of the process: a
// call borrows only the cores that others leave, so that many concurrent
// compiles (a batch's compile workers) do not oversubscribe the host.
std::atomic<int> gHelpers{0};

// Runs f(0 .. n-1) on the calling thread and up to 15 helpers; the first
// exception is rethrown after every thread has finished.
template <typename F>
void parallelFor(int n, F&& f) {
  const unsigned hwu = std::thread::hardware_concurrency();
  const int hw = hwu ? (int)hwu : 1;
  const int want = std::min(n, std::min(hw, 16)) - 1;
  int got = 0;
  if (want > 0) {
    int cur = gHelpers.load();
    do {
      got = std::max(0, std::min(want, hw - 1 - cur));
    } while (got > 0 && !gHelpers.compare_exchange_weak(cur, cur + got));
  }
  if (got == 0) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  const int nt = got + 1;
  std::atomic<int> next{0};
  std::exception_ptr err;
  std::mutex m;
  auto work = [&] {
    try {
      for (int i = next++; i < n; i = next++) f(i);
    } catch (...) {
      std::lock_guard<std::mutex> lock(m);
      if (!err) err = std::current_exception();
      next = n;
    }
  };
  std::vector<std::thread> pool;
  try {
    for (int k = 1; k < nt; ++k) pool.emplace_back(work);
  } catch (...) {  // no thread could be started: the caller does the rest
  }
  work();
  for (std::thread& th : pool) th.join();
  gHelpers -= got;
  if (err) std::rethrow_exception(err);
}

}  // namespace

namespace {

// The staged plan's backward levels (layout.h). Per traverser tr:
//   - an opponent decide node whose parent is one of tr's decide nodes is
//     "folded into" the parent: its value row (the sum of its children's)
//     is computed by the parent's records, chunk by chunk, right before the
//     parent uses it, so it needs no level of its own;
//   - every other node with backward work (tr's decide nodes, chance nodes,
//     opponent decide nodes under a chance node) sits at a level below all
//     the levels that read its row (see the work depth below);
//   - an opponent decide node at the root does no work (its value is read
//     by nothing in the iteration).
// The records of a traverser node with folded-in children are new: [regret
// row, value row, n | na << 16 | 1 << 24 | 1 << 25, chunk, child rows[na],
// P, then P times (child value row, m, its m children's value rows)]; other
// nodes' records are copies of their depth-list records. Each level's
// records lie together in the pool (by size class, see below).
void buildBackwardLevels(const Tree& t, HostLayout& L,
                         const std::vector<uint32_t> (&firstRec)[2],
                         const std::vector<std::vector<uint32_t>> (&chanceRecs)[2]) {
  const int N = (int)t.nodes.size();
  auto child = [&](int u, int a) { return t.children[t.nodes[u].childBase + a]; };
  auto terminal = [&](int u) {
    return t.nodes[u].kind == kShowdown || t.nodes[u].kind == kFold;
  };
  auto chunks = [](int n) { return (int)((quads(n) + kRecQuads - 1) / kRecQuads); };
  auto recWords = [](int na) { return (size_t)(4 + na + 3) / 4 * 4; };
  // Each level's records: their words end to end, and where each starts.
  // The traversers' levels are built in parallel (they read the pool and
  // write only their own lists); their records go into the pool after, in
  // traverser order.
  std::vector<std::vector<uint32_t>> pendWordsOf[2], pendStartOf[2];
  parallelFor(2, [&](int tr) {
    auto opponent = [&](int u) {
      return t.nodes[u].kind == kDecide && t.nodes[u].player != tr;
    };
    auto foldedIn = [&](int u) {
      const int p = t.nodes[u].parent;
      return opponent(u) && p >= 0 && t.nodes[p].kind == kDecide && t.nodes[p].player == tr;
    };
    auto works = [&](int u) {
      if (terminal(u) || foldedIn(u)) return false;
      return !(opponent(u) && t.nodes[u].parent < 0);
    };
    // Levels as late as possible: a node's work depth is the number of
    // working ancestors (through folded-in children), and level = deepest
    // work depth - its own, so each level holds the nodes of one work depth
    // and reads the terminals of the depths just below them: the backward
    // pass starts on the deepest nodes while shallower terminal groups are
    // still running.
    std::vector<int> wd(N, -1), h(N, -1);
    std::vector<uint64_t> need(N, 0);
    int maxWd = -1;
    for (int u = 0; u < N; ++u) {  // parents first (DFS pre-order)
      int up = -1;
      for (int p = t.nodes[u].parent; p >= 0; p = t.nodes[p].parent)
        if (works(p)) {
          up = wd[p];
          break;
        }
      if (!works(u)) continue;
      wd[u] = up + 1;
      maxWd = std::max(maxWd, wd[u]);
    }
    const int H = maxWd + 1;
    for (int u = 0; u < N; ++u) {
      if (!works(u)) continue;
      h[u] = maxWd - wd[u];
      uint64_t nd = 0;
      auto input = [&](int k) {
        if (terminal(k)) nd |= (uint64_t)1 << t.nodes[k].depth;
      };
      for (int a = 0; a < t.nodes[u].nChildren; ++a) {
        const int k = child(u, a);
        if (foldedIn(k))
          for (int b = 0; b < t.nodes[k].nChildren; ++b) input(child(k, b));
        else
          input(k);
      }
      need[u] = nd;
    }
    if (t.maxDepth >= 64) throw Error{PPS_GB_E_ARG, "tree deeper than 64 levels"};
    L.bwdRecsH[tr].assign(H, {});
    L.bwdChanceRecsH[tr].assign(H, {});
    L.bwdTasksH[tr].assign(H, {});
    L.bwdNeed[tr].assign(H, 0);
    L.levelRecs[tr].clear();
    std::vector<std::vector<uint32_t>>& pendWords = pendWordsOf[tr];
    std::vector<std::vector<uint32_t>>& pendStart = pendStartOf[tr];
    pendWords.assign(H, {});
    pendStart.assign(H, {});
    for (int u = 0; u < N; ++u) {
      if (h[u] < 0) continue;
      const Node& nd = t.nodes[u];
      const int lv = h[u];
      L.bwdNeed[tr][lv] |= need[u];
      if (nd.kind == kChance) {
        for (uint32_t off : chanceRecs[tr][u]) L.bwdChanceRecsH[tr][lv].push_back(off);
        for (int c = 0; c < (int)(quads(t.n(u, tr)) * 4 + kChanceChunk - 1) / kChanceChunk; ++c)
          L.bwdTasksH[tr][lv].push_back(makeTask(kTaskChance, c, u));
        continue;
      }
      const int n = t.n(u, tr), nc = chunks(n);
      for (int c = 0; c < (n + 4 * kChunkQuads - 1) / (4 * kChunkQuads); ++c)
        L.bwdTasksH[tr][lv].push_back(makeTask(kTaskDecide, c, u));
      bool folds = false;
      for (int a = 0; a < nd.na; ++a) folds |= foldedIn(child(u, a));
      std::vector<uint32_t>& pw = pendWords[lv];
      if (!folds) {  // copies of the depth-list records
        const uint32_t stride = (uint32_t)(recWords(nd.na) / 4);
        for (int c = 0; c < nc; ++c) {
          const size_t at = (size_t)(firstRec[tr][u] + (uint32_t)c * stride) * 4;
          pendStart[lv].push_back((uint32_t)pw.size());
          pw.insert(pw.end(), L.recPool.begin() + at, L.recPool.begin() + at + 4 + nd.na);
        }
        continue;
      }
      for (int a = 0; a < nd.na; ++a) {  // the folded-in children's work (byte model)
        const int k = child(u, a);
        if (foldedIn(k))
          for (int c = 0; c < (n + 4 * kChunkQuads - 1) / (4 * kChunkQuads); ++c)
            L.bwdTasksH[tr][lv].push_back(makeTask(kTaskDecide, c, k));
      }
      for (int c = 0; c < nc; ++c) {
        pendStart[lv].push_back((uint32_t)pw.size());
        pw.push_back(L.nodes[u].regQ);
        pw.push_back(L.rows[u].cfvQ);
        pw.push_back((uint32_t)n | ((uint32_t)nd.na << 16) | (1u << 24) | (1u << 25));
        pw.push_back((uint32_t)c);
        int P = 0;
        for (int a = 0; a < nd.na; ++a) {
          pw.push_back(L.rows[child(u, a)].cfvQ);
          P += foldedIn(child(u, a)) ? 1 : 0;
        }
        pw.push_back((uint32_t)P);
        for (int a = 0; a < nd.na; ++a) {
          const int k = child(u, a);
          if (!foldedIn(k)) continue;
          pw.push_back(L.rows[k].cfvQ);
          pw.push_back((uint32_t)t.nodes[k].nChildren);
          for (int b = 0; b < t.nodes[k].nChildren; ++b) pw.push_back(L.rows[child(k, b)].cfvQ);
        }
      }
    }
  });
  for (int tr = 0; tr < 2; ++tr) {
    const int H = (int)pendWordsOf[tr].size();
    // A level's records lie together, grouped by size class (16-byte units
    // rounded up to a power of two, at least two; the largest class first,
    // so the records with the most work start first and the level's tail is
    // short), each padded to its class: the level's offsets form a few
    // arithmetic runs, from which a kernel computes a record's offset
    // instead of loading it.
    while (L.recPool.size() % 4) L.recPool.push_back(0);
    constexpr int kClasses = 16;  // class c: 2 << c units
    for (int lv = 0; lv < H; ++lv) {
      const std::vector<uint32_t>& pw = pendWordsOf[tr][lv];
      std::vector<uint32_t>& ps = pendStartOf[tr][lv];
      const size_t nr = ps.size();
      ps.push_back((uint32_t)pw.size());
      std::vector<uint8_t> cls(nr);
      size_t count[kClasses] = {}, words = 0;
      for (size_t i = 0; i < nr; ++i) {
        int c = 0;
        while (c + 1 < kClasses && (size_t)(8u << c) < ps[i + 1] - ps[i]) ++c;
        cls[i] = (uint8_t)c;
        ++count[c];
        words += (size_t)(8u << c);
      }
      L.recPool.reserve(L.recPool.size() + words);
      L.bwdRecsH[tr][lv].reserve(nr);
      for (int c = kClasses - 1; c >= 0; --c) {
        if (!count[c]) continue;
        for (size_t i = 0; i < nr; ++i) {
          if (cls[i] != c) continue;
          const uint32_t off = (uint32_t)(L.recPool.size() / 4);
          L.recPool.insert(L.recPool.end(), pw.begin() + ps[i], pw.begin() + ps[i + 1]);
          L.recPool.resize((size_t)off * 4 + (8u << c), 0u);
          L.bwdRecsH[tr][lv].push_back(off);
          L.levelRecs[tr].push_back(off);
        }
      }
    }
  }
}

}  // namespace

HostLayout buildLayout(const Tree& t) {
  HostLayout L;
  const int N = (int)t.nodes.size();
  const int S = (int)t.states.size();

  // ---- board-state tables ----
  // States are independent: their tables are built in parallel, then
  // appended to the pools in state order (the same bytes as a serial build).
  std::vector<StateParts> parts(S);
  parallelFor(S, [&](int s) { buildStateParts(t, s, parts[s]); });
  size_t nU8 = 0, nU16 = 0, nI16 = 0, nSd = 0;
  for (const StateParts& P : parts)
    for (int p = 0; p < 2; ++p) {
      nU8 += P.cards[p].size() + 16;
      nU16 += P.starts[p].size() + P.entries[p].size() + P.up[p].size() + P.ord[p].size() +
              P.segStart[p].size() + P.segSlot[p].size() + 16;  // + alignment
      nI16 += P.same[p].size() + P.down[p].size() + 8;
      nSd += P.info[p].size();
    }
  L.poolU8.reserve(L.poolU8.size() + nU8);
  L.poolU16.reserve(L.poolU16.size() + nU16);
  L.poolI16.reserve(L.poolI16.size() + nI16);
  L.poolSd.reserve(L.poolSd.size() + nSd);
  L.states.resize(S);
  for (int s = 0; s < S; ++s) {
    const BoardState& st = t.states[s];
    const StateParts& P = parts[s];
    StateDev& sd = L.states[s];
    for (int p = 0; p < 2; ++p) {
      const int n = (int)st.list[p].size();
      sd.n[p] = n;
      L.maxN = std::max(L.maxN, n);
      alignU8(L.poolU8);
      sd.cardsOff[p] = (int)L.poolU8.size();
      L.poolU8.insert(L.poolU8.end(), P.cards[p].begin(), P.cards[p].end());
      alignU16(L.poolU16);
      sd.csrOff[p] = appendU16(L.poolU16, P.starts[p]);
      appendU16(L.poolU16, P.entries[p]);
      alignI16(L.poolI16);
      sd.sameOff[p] = appendI16(L.poolI16, P.same[p]);
      sd.upOff[p] = sd.downOff[p] = -1;
      if (st.parent >= 0) {
        sd.upOff[p] = appendU16(L.poolU16, P.up[p]);
        sd.downOff[p] = appendI16(L.poolI16, P.down[p]);
      }
      sd.sdOff[p] = sd.sdInfoOff[p] = -1;
    }
    L.maxCardSeg = std::max(L.maxCardSeg, P.maxCardSeg);
    if (st.nBoard != 5) continue;
    for (int tr = 0; tr < 2; ++tr) {
      alignU16(L.poolU16);
      sd.sdOff[tr] = appendU16(L.poolU16, P.ord[tr]);
      appendU16(L.poolU16, P.segStart[tr]);
      appendU16(L.poolU16, P.segSlot[tr]);
      sd.sdInfoOff[tr] = (int)L.poolSd.size();
      L.poolSd.insert(L.poolSd.end(), P.info[tr].begin(), P.info[tr].end());
    }
  }
  // The showdown kernel scans one card segment per warp, two entries per
  // lane plus the total slot: at most 63 entries (a card pairs with <= 51).
  if (L.maxCardSeg > 63)
    throw Error{PPS_GB_E_ARG, "card segment longer than 63 combos"};

  // ---- nodes, rows, payoffs ----
  L.nodes.resize(N);
  L.rows.resize(N);
  L.termVal.assign((size_t)N * 8, 0.0f);
  L.children = t.children;
  uint64_t regQ = 0, cfvQ = 0, reachQ[2] = {0, 0};
  for (int u = 0; u < N; ++u) {
    const Node& nd = t.nodes[u];
    const int n0 = t.n(u, 0), n1 = t.n(u, 1);
    NodeDev& dv = L.nodes[u];
    dv.meta = packNode(nd.kind, nd.player, nd.foldBy,
                       nd.kind == kDecide ? nd.na : nd.kind == kChance ? nd.nChildren : 0);
    dv.state = nd.state;
    dv.childBase = nd.childBase;
    dv.regQ = 0;
    if (nd.kind == kDecide) {
      dv.regQ = (uint32_t)regQ;
      regQ += (uint64_t)nd.na * quads(nd.player == 0 ? n0 : n1);
    }
    RowDev& rw = L.rows[u];
    rw.cfvQ = (uint32_t)cfvQ;
    cfvQ += quads(std::max(n0, n1));
    for (int tr = 0; tr < 2; ++tr) {
      const int par = nd.parent;
      if (par >= 0 && t.nodes[par].kind == kDecide && t.nodes[par].player == tr) {
        rw.reachQ[tr] = L.rows[par].reachQ[tr];
      } else {
        rw.reachQ[tr] = (uint32_t)reachQ[tr];
        reachQ[tr] += quads(tr == 0 ? n1 : n0);
      }
    }
    const int nBoard = t.states[nd.state].nBoard;
    rw.chanceQ = 52 - nBoard - 4;
    if (regQ > 0xffffffffull || cfvQ > 0xffffffffull || reachQ[0] > 0xffffffffull ||
        reachQ[1] > 0xffffffffull)
      throw Error{PPS_GB_E_MEMORY, "tree too large for 32-bit row offsets"};
    // Terminal payoffs from the root baseline, computed in float exactly as
    // the reference's terminal kernels do (cuda/gpu_cfr.cu:356-364, 433-439).
    for (int tr = 0; tr < 2; ++tr) {
      float* tv = &L.termVal[((size_t)u * 2 + tr) * 4];
      const int64_t scTr = tr == 0 ? nd.sc0 : nd.sc1;
      const int64_t pcTr = tr == 0 ? nd.pc0 : nd.pc1;
      if (nd.kind == kShowdown) {
        const int64_t diff = nd.sc0 > nd.sc1 ? nd.sc0 - nd.sc1 : nd.sc1 - nd.sc0;
        const float totalPot = (float)(nd.potBase + nd.sc0 + nd.sc1 - diff);
        const float mySc = (float)(scTr + pcTr);
        tv[0] = totalPot - mySc;
        tv[1] = totalPot * 0.5f - mySc;
        tv[2] = -mySc;
      } else if (nd.kind == kFold) {
        const int fb = nd.foldBy;
        const int64_t scF = fb == 0 ? nd.sc0 : nd.sc1;
        const int64_t pcF = fb == 0 ? nd.pc0 : nd.pc1;
        tv[0] = tr == fb ? -((float)scF + (float)pcF)
                         : ((float)(nd.potBase + scF) - (float)pcTr);
      }
    }
  }
  L.regQuads = regQ;
  L.cfvQuads = cfvQ;
  L.reachQuads[0] = reachQ[0];
  L.reachQuads[1] = reachQ[1];

  // ---- warp task lists (per traverser) and terminal groups ----
  // Three independent jobs, each writing only its own lists.
  const int D = t.maxDepth + 1;
  auto taskLists = [&](int tr) {
    L.fwdTasks[tr].assign(D, {});
    L.bwdTasks[tr].assign(D, {});
    std::vector<std::vector<int>> sd(D), fd(D), ch(D), dc(D);
    for (int u = 0; u < N; ++u) {
      const Node& nd = t.nodes[u];
      const int chunksTr = (int)((quads(t.n(u, tr)) + kChunkQuads - 1) / kChunkQuads);
      switch (nd.kind) {
        case kShowdown: sd[nd.depth].push_back(makeTask(kTaskShowdown, 0, u)); break;
        case kFold: fd[nd.depth].push_back(makeTask(kTaskFold, 0, u)); break;
        case kChance:
          for (int c = 0; c < (int)(quads(t.n(u, tr)) * 4 + kChanceChunk - 1) / kChanceChunk; ++c)
            ch[nd.depth].push_back(makeTask(kTaskChance, c, u));
          for (int br = 0; br < nd.nChildren; ++br)
            L.fwdTasks[tr][nd.depth].push_back(makeTask(kTaskChance, br, u));
          break;
        default: {
          for (int c = 0; c < chunksTr; ++c) dc[nd.depth].push_back(makeTask(kTaskDecide, c, u));
          if (nd.player != tr) {
            const int chunksOpp =
                (int)((quads(t.n(u, 1 - tr)) + kChunkQuads - 1) / kChunkQuads);
            for (int c = 0; c < chunksOpp; ++c)
              L.fwdTasks[tr][nd.depth].push_back(makeTask(kTaskDecide, c, u));
          }
        }
      }
    }
    for (int d = 0; d < D; ++d) {
      auto& b = L.bwdTasks[tr][d];
      for (auto* v : {&sd[d], &fd[d], &ch[d], &dc[d]}) b.insert(b.end(), v->begin(), v->end());
      L.innerTasks[tr].push_back(ch[d]);
      L.innerTasks[tr].back().insert(L.innerTasks[tr].back().end(), dc[d].begin(), dc[d].end());
    }
  };
  // Terminal groups: per depth, the showdown (then fold) nodes of one board
  // state in fours, in node order (the same groups serve both traversers).
  auto termGroups = [&] {
    L.sdGroupTasks.assign(D, {});
    L.fdGroupTasks.assign(D, {});
    for (int kind : {(int)kShowdown, (int)kFold}) {
      std::vector<std::vector<std::vector<int>>> byState(D, std::vector<std::vector<int>>(S));
      for (int u = 0; u < N; ++u)
        if (t.nodes[u].kind == kind) byState[t.nodes[u].depth][t.nodes[u].state].push_back(u);
      for (int d = 0; d < D; ++d)
        for (int s = 0; s < S; ++s) {
          const auto& v = byState[d][s];
          for (size_t i = 0; i < v.size(); i += 4) {
            TermGroup g{{-1, -1, -1, -1}};
            for (size_t k = 0; k < 4 && i + k < v.size(); ++k) g.node[k] = v[i + k];
            const int task = makeTask(kind == kShowdown ? kTaskShowdown : kTaskFold, 0,
                                      (int)L.groups.size());
            (kind == kShowdown ? L.sdGroupTasks : L.fdGroupTasks)[d].push_back(task);
            L.groups.push_back(g);
          }
        }
    }
  };
  parallelFor(3, [&](int job) {
    if (job < 2) taskLists(job);
    else termGroups();
  });
  // Group records: what each traverser's group kernels read of the nodes,
  // their state and their rows (layout.h GroupRec).
  L.groupRecs.assign(L.groups.size() * 2, GroupRec{});
  for (size_t gi = 0; gi < L.groups.size(); ++gi) {
    const TermGroup& g = L.groups[gi];
    const int kind = t.nodes[g.node[0]].kind == kShowdown ? kTaskShowdown : kTaskFold;
    const StateDev& st = L.states[L.nodes[g.node[0]].state];
    for (int tr = 0; tr < 2; ++tr) {
      GroupRec& r = L.groupRecs[gi * 2 + tr];
      const int opp = 1 - tr;
      r.no = st.n[opp];
      r.nt = st.n[tr];
      r.kind = kind;
      if (kind == kTaskShowdown) {
        r.tabOff = st.sdOff[tr];
        r.infoOff = st.sdInfoOff[tr];
        r.sameOff = -1;
      } else {
        r.tabOff = st.csrOff[opp];
        r.infoOff = st.cardsOff[tr];
        r.sameOff = st.sameOff[tr];
      }
      for (int k = 0; k < 4; ++k) {
        const int u = g.node[k];
        if (u < 0) continue;
        r.mask |= 1 << k;
        r.reachQ[k] = L.rows[u].reachQ[tr];
        r.cfvQ[k] = L.rows[u].cfvQ;
        for (int j = 0; j < 4; ++j) r.val[k][j] = L.termVal[((size_t)u * 2 + tr) * 4 + j];
      }
    }
  }
  // Forward levels (see layout.h): level of a forward-working node = one
  // more than its nearest forward-working ancestor's (0 without one); the
  // nodes are in DFS pre-order, so parents come first.
  std::vector<int> fwdLevel[2];
  int F[2] = {0, 0};
  for (int tr = 0; tr < 2; ++tr) {
    std::vector<int>& lev = fwdLevel[tr];
    std::vector<int> writer(N, -1);  // level of the task that wrote u's reach row
    lev.assign(N, -1);
    for (int u = 0; u < N; ++u) {
      const Node& nd = t.nodes[u];
      const int par = nd.parent;
      if (par >= 0) {
        const Node& pn = t.nodes[par];
        const bool parWorks = pn.kind == kChance || (pn.kind == kDecide && pn.player != tr);
        writer[u] = parWorks ? lev[par] : writer[par];
      }
      const bool works = nd.kind == kChance || (nd.kind == kDecide && nd.player != tr);
      if (works) {
        lev[u] = writer[u] + 1;
        F[tr] = std::max(F[tr], lev[u] + 1);
      }
    }
    L.termAfter[tr].assign(D, -1);
    for (int u = 0; u < N; ++u)
      if (t.nodes[u].kind == kShowdown || t.nodes[u].kind == kFold)
        L.termAfter[tr][t.nodes[u].depth] =
            std::max(L.termAfter[tr][t.nodes[u].depth], writer[u]);
  }
  // Decide records and chance word lists of the default iteration.
  for (int tr = 0; tr < 2; ++tr) {
    L.bwdRecs[tr].assign(D, {});
    L.fwdRecs[tr].assign(F[tr], {});
    L.bwdChance[tr].assign(D, {});
    L.fwdChance[tr].assign(F[tr], {});
    L.fwdDecide[tr].assign(F[tr], {});
    for (int d = 0; d < D; ++d) {
      for (int w : L.bwdTasks[tr][d])
        if ((w & 3) == kTaskChance) L.bwdChance[tr][d].push_back(w);
      for (int w : L.fwdTasks[tr][d]) {
        const int lv = fwdLevel[tr][(int)((unsigned)w >> 8)];
        ((w & 3) == kTaskChance ? L.fwdChance : L.fwdDecide)[tr][lv].push_back(w);
      }
    }
  }
  // Decide records: [own regret row, value or reach row, n | na << 16 |
  // own << 24, chunk, child rows[na]], padded to 16 bytes. One pass counts
  // them, one writes them into the pool sized once.
  auto recWords = [](int na) { return (size_t)(4 + na + 3) / 4 * 4; };
  auto chunksOf = [](int n) { return (int)((quads(n) + kRecQuads - 1) / kRecQuads); };
  // Forward records lie apart from the backward ones: per traverser and
  // forward level, in node order, each padded to the level's largest record,
  // so a level's records sit at one stride from its first (a kernel can
  // compute a record's offset from its index).
  size_t words = L.recPool.size();
  std::vector<size_t> nBwd[2] = {std::vector<size_t>(D, 0), std::vector<size_t>(D, 0)};
  std::vector<std::vector<int>> fwdNodes[2];  // per forward level: its nodes
  std::vector<size_t> fwdSpan[2];              // per forward level: words a record
  for (int tr = 0; tr < 2; ++tr) {
    fwdNodes[tr].assign(F[tr], {});
    fwdSpan[tr].assign(F[tr], 0);
  }
  for (int u = 0; u < N; ++u) {
    const Node& nd = t.nodes[u];
    if (nd.kind != kDecide) continue;
    for (int tr = 0; tr < 2; ++tr) {
      const int cb = chunksOf(t.n(u, tr));
      nBwd[tr][nd.depth] += cb;
      words += cb * recWords(nd.na);
      if (nd.player == tr) continue;
      const int lv = fwdLevel[tr][u];
      fwdNodes[tr][lv].push_back(u);
      fwdSpan[tr][lv] = std::max(fwdSpan[tr][lv], recWords(nd.na));
    }
  }
  for (int tr = 0; tr < 2; ++tr)
    for (int lv = 0; lv < F[tr]; ++lv) {
      size_t nf = 0;
      for (int u : fwdNodes[tr][lv]) nf += chunksOf(t.n(u, 1 - tr));
      L.fwdRecs[tr][lv].reserve(nf);
      words += nf * fwdSpan[tr][lv];
    }
  for (int tr = 0; tr < 2; ++tr)
    for (int d = 0; d < D; ++d) L.bwdRecs[tr][d].reserve(nBwd[tr][d]);
  size_t w = L.recPool.size();
  L.recPool.resize(words, 0u);
  std::vector<uint32_t> kids;
  auto addRecord = [&](uint32_t regQ, uint32_t rowQ, int n, int na, int own, int chunk,
                       size_t span) {
    const uint32_t off = (uint32_t)(w / 4);
    uint32_t* r = L.recPool.data() + w;
    r[0] = regQ;
    r[1] = rowQ;
    r[2] = (uint32_t)n | ((uint32_t)na << 16) | ((uint32_t)own << 24);
    r[3] = (uint32_t)chunk;
    for (int a = 0; a < na; ++a) r[4 + a] = kids[a];
    w += span;
    return off;
  };
  std::vector<uint32_t> bwdRecFirst[2] = {std::vector<uint32_t>(N, 0),
                                          std::vector<uint32_t>(N, 0)};
  for (int u = 0; u < N; ++u) {
    const Node& nd = t.nodes[u];
    if (nd.kind != kDecide) continue;
    kids.resize(nd.na);
    for (int tr = 0; tr < 2; ++tr) {
      for (int a = 0; a < nd.na; ++a) kids[a] = L.rows[t.children[nd.childBase + a]].cfvQ;
      const int nTr = t.n(u, tr);
      bwdRecFirst[tr][u] = (uint32_t)(w / 4);
      for (int c = 0, cb = chunksOf(nTr); c < cb; ++c)
        L.bwdRecs[tr][nd.depth].push_back(addRecord(L.nodes[u].regQ, L.rows[u].cfvQ, nTr, nd.na,
                                                    nd.player == tr, c, recWords(nd.na)));
    }
  }
  for (int tr = 0; tr < 2; ++tr)
    for (int lv = 0; lv < F[tr]; ++lv)
      for (int u : fwdNodes[tr][lv]) {
        const Node& nd = t.nodes[u];
        kids.resize(nd.na);
        for (int a = 0; a < nd.na; ++a)
          kids[a] = L.rows[t.children[nd.childBase + a]].reachQ[tr];
        const int nOpp = t.n(u, 1 - tr);
        for (int c = 0, cf = chunksOf(nOpp); c < cf; ++c)
          L.fwdRecs[tr][lv].push_back(addRecord(L.nodes[u].regQ, L.rows[u].reachQ[tr], nOpp,
                                                nd.na, 0, c, fwdSpan[tr][lv]));
      }
  // Chance records: every row and table address a chance task needs, so a
  // CTA reaches its data in two dependent loads.
  //   forward, per branch: [parent reach row, child reach row (quads, the
  //     traverser's layout), child -> parent slot map (u16 pool), n_child |
  //     chanceQ << 16]
  //   backward, per 128-combo chunk: [value row, n | branches << 16, chunk,
  //     branch table (16-byte units)]; the table holds per branch [child
  //     value row, parent -> child slot map (i16 pool)], once per node.
  std::vector<std::vector<uint32_t>> chanceRecsOf[2] = {
      std::vector<std::vector<uint32_t>>(N), std::vector<std::vector<uint32_t>>(N)};
  for (int tr = 0; tr < 2; ++tr) {
    const int opp = 1 - tr;
    L.bwdChanceRecs[tr].assign(D, {});
    L.chanceTables[tr].clear();
    std::map<int, uint32_t> table;  // node -> its branch table
    L.fwdChanceRecs[tr].assign(F[tr], {});
    for (int lv = 0; lv < F[tr]; ++lv)
      for (int w : L.fwdChance[tr][lv]) {
        const int u = (int)((unsigned)w >> 8), br = (w >> 2) & 63;
        const int ch = t.children[t.nodes[u].childBase + br];
        const StateDev& cs = L.states[t.nodes[ch].state];
        const uint32_t off = (uint32_t)(L.recPool.size() / 4);
        L.recPool.push_back(L.rows[u].reachQ[tr]);
        L.recPool.push_back(L.rows[ch].reachQ[tr]);
        L.recPool.push_back((uint32_t)cs.upOff[opp]);
        L.recPool.push_back((uint32_t)cs.n[opp] | ((uint32_t)L.rows[u].chanceQ << 16));
        L.fwdChanceRecs[tr][lv].push_back(off);
      }
    for (int d = 0; d < D; ++d) {
      for (int w : L.bwdChance[tr][d]) {
        const int u = (int)((unsigned)w >> 8), chunk = (w >> 2) & 63;
        const Node& nd = t.nodes[u];
        auto it = table.find(u);
        if (it == table.end()) {
          // The record kernels hold one slot column per branch (64 at most).
          if (nd.nChildren > 64) throw Error{PPS_GB_E_ARG, "chance node with more than 64 branches"};
          const uint32_t toff = (uint32_t)(L.recPool.size() / 4);
          for (int b = 0; b < nd.nChildren; ++b) {
            const int ch = t.children[nd.childBase + b];
            L.recPool.push_back(L.rows[ch].cfvQ);
            L.recPool.push_back((uint32_t)L.states[t.nodes[ch].state].downOff[tr]);
          }
          while (L.recPool.size() % 4) L.recPool.push_back(0);
          it = table.emplace(u, toff).first;
          L.chanceTables[tr].push_back({toff, nd.nChildren});
        }
        const uint32_t off = (uint32_t)(L.recPool.size() / 4);
        L.recPool.push_back(L.rows[u].cfvQ);
        L.recPool.push_back((uint32_t)L.states[nd.state].n[tr] | ((uint32_t)nd.nChildren << 16));
        L.recPool.push_back((uint32_t)chunk);
        L.recPool.push_back(it->second);
        L.bwdChanceRecs[tr][d].push_back(off);
        chanceRecsOf[tr][u].push_back(off);
      }
    }
  }
  buildBackwardLevels(t, L, bwdRecFirst, chanceRecsOf);
  if (N >= (1 << 24)) throw Error{PPS_GB_E_MEMORY, "tree too large for 24-bit task node ids"};
  alignU16(L.poolU16);
  alignI16(L.poolI16);
  alignU8(L.poolU8);
  return L;
}

namespace {

struct Fnv {
  uint64_t h = 1469598103934665603ull;
  void bytes(const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) {
      h ^= b[i];
      h *= 1099511628211ull;
    }
  }
  template <typename T>
  void vec(const std::vector<T>& v) {
    const uint64_t n = v.size();
    bytes(&n, sizeof n);
    if (n) bytes(v.data(), n * sizeof(T));
  }
  template <typename T>
  void vecs(const std::vector<std::vector<T>>& v) {
    const uint64_t n = v.size();
    bytes(&n, sizeof n);
    for (const auto& x : v) vec(x);
  }
};

}  // namespace

uint64_t layoutDigest(const HostLayout& L) {
  Fnv f;
  f.vec(L.nodes);
  f.vec(L.rows);
  f.vec(L.termVal);
  f.vec(L.children);
  f.vec(L.states);
  f.vec(L.poolU8);
  f.vec(L.poolU16);
  f.vec(L.poolI16);
  f.vec(L.poolSd);
  f.bytes(&L.regQuads, sizeof L.regQuads);
  f.bytes(&L.cfvQuads, sizeof L.cfvQuads);
  f.bytes(L.reachQuads, sizeof L.reachQuads);
  for (int tr = 0; tr < 2; ++tr) {
    f.vecs(L.fwdTasks[tr]);
    f.vecs(L.bwdTasks[tr]);
    f.vecs(L.innerTasks[tr]);
  }
  f.vec(L.groups);
  f.vec(L.groupRecs);
  f.vecs(L.sdGroupTasks);
  f.vecs(L.fdGroupTasks);
  f.vec(L.recPool);
  for (int tr = 0; tr < 2; ++tr) {
    f.vecs(L.bwdRecs[tr]);
    f.vecs(L.fwdRecs[tr]);
    f.vecs(L.fwdChanceRecs[tr]);
    f.vecs(L.bwdChanceRecs[tr]);
    for (const auto& c : L.chanceTables[tr]) {
      f.bytes(&c.first, sizeof c.first);
      f.bytes(&c.second, sizeof c.second);
    }
    f.vecs(L.bwdChance[tr]);
    f.vecs(L.fwdChance[tr]);
    f.vecs(L.fwdDecide[tr]);
    f.vec(L.termAfter[tr]);
    f.vecs(L.bwdRecsH[tr]);
    f.vecs(L.bwdChanceRecsH[tr]);
    f.vecs(L.bwdTasksH[tr]);
    f.vec(L.bwdNeed[tr]);
    f.vec(L.levelRecs[tr]);
  }
  f.bytes(&L.maxN, sizeof L.maxN);
  f.bytes(&L.maxCardSeg, sizeof L.maxCardSeg);
  return f.h;
}

}  // namespace gb
}  // namespace pps
