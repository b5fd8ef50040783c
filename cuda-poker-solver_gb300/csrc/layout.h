// Device data layout of one compiled spot (built on the host, uploaded by
// the engine).
//
// Rows. Every per-combo row (regret, strategy, reach, counterfactual value)
// starts on a 16-byte boundary and is padded to a multiple of 4 entries,
// so kernels move whole float4 (double2x2) quads; offsets are stored in
// quad units. Regret and strategy rows of a decide node are na rows of
// pad4(n_actor) entries, action-major (the reference's [a][c] order,
// cuda/gpu_cfr.cu:1476-1481, plus padding). Reach rows exist per traverser
// layout and alias the parent's row under the traverser's own decide nodes
// (the reference's pass-through aliasing, cuda/gpu_cfr.cu:1491-1514).
//
// Board states. Combo lists and every table derived from them (cards per
// list slot, card->slot lists, identical-combo maps, chance slot maps and
// the river strength tables) exist once per BoardState, not per node.
#pragma once

#include <cstdint>
#include <vector>

#include "compiler.h"

namespace pps {
namespace gb {

// Half-step modes: a DCFR iteration, an average-strategy value walk, a
// best-response walk.
enum WalkMode : int { kModeCFR = 0, kModeEV = 1, kModeBR = 2 };

// Packed node word: kind (bits 0-1), player (bit 2), foldBy (bit 3),
// na or branch count (bits 8-15); a forest stores the spot's slot in bits
// 16-31 (its iteration counter).
inline int packNode(int kind, int player, int foldBy, int na) {
  return kind | (player << 2) | (foldBy << 3) | (na << 8);
}

// Warp task word: kind (bits 0-1), sub = quad chunk or chance branch (bits
// 2-7), node (bits 8-31).
enum TaskKind : int { kTaskDecide = 0, kTaskChance = 1, kTaskFold = 2, kTaskShowdown = 3 };
constexpr int kChunkQuads = 128;   // row quads per decide task
constexpr int kRecQuads = 32;      // row quads per decide record (one warp)
constexpr int kChanceChunk = 128;  // combos per backward chance task
inline int makeTask(int kind, int sub, int node) { return kind | (sub << 2) | (node << 8); }

struct alignas(16) NodeDev {
  int meta;         // packNode(...)
  int state;        // BoardState index
  int childBase;    // into children[]
  uint32_t regQ;    // decide: regret/strategy row start (quads)
};

struct alignas(16) RowDev {
  uint32_t reachQ[2];  // reach row start per traverser layout (quads)
  uint32_t cfvQ;       // counterfactual-value row start (quads)
  int chanceQ;         // 52 - nBoard - 4: pair-conditional deal count
};

// Per board state, per side p (0/1); offsets index the pools below, -1 if
// the table does not exist for this state.
struct alignas(16) StateDev {
  int n[2];         // list sizes
  int cardsOff[2];  // u8 pool: 2 cards per list slot
  int csrOff[2];    // u16 pool: 53 segment starts, then the slots holding
                    // each card (card-major, ascending)
  int sameOff[2];   // i16 pool: slot of the identical combo in the other
                    // side's list, or -1
  int upOff[2];     // u16 pool: child slot -> parent slot (dealt states)
  int downOff[2];   // i16 pool: parent slot -> child slot or -1
  int sdOff[2];     // river states, per traverser tr: u16 pool holding
                    // ord[n_opp] (opponent slots, weakest first), 53
                    // card-segment starts, then per card (in strength
                    // order) the slots of the opponent combos holding it
  int sdInfoOff[2]; // river states, per traverser: u32x4 pool, one entry
                    // per traverser slot (see showdownInfo)
};

#ifdef __CUDACC__
#define PPS_HD __host__ __device__
#else
#define PPS_HD
#endif
// Padded float4 arrays of the terminal kernels: entry k lives at pad8(k),
// one padding entry after every eight, so that eight threads writing eight
// consecutive entries each hit eight different bank groups. unpad8 inverts
// it on the entries pad8 produces.
PPS_HD inline int pad8(int k) { return k + (k >> 3); }
PPS_HD inline int unpad8(int p) { return p - p / 9; }

// Showdown entry of one traverser combo (cards c1, c2), as shared-memory
// indices of the kernels' padded arrays. The opponents strictly weaker /
// weaker-or-equal end at sorted positions le / te; card cX's prefix run
// (one entry more than its segment of the strength order) starts at entry
// aX = seg[cX] + cX of the concatenated runs, and kXle / kXte count its
// entries below le / te. Fields:
//   x = pad8(a1 + k1le) | pad8(a1 + k1te) << 12 | (sHi & 0xff) << 24
//   y = pad8(a1 + len1) | pad8(a2 + k2le) << 12 | (sHi >> 8) << 24
//   z = pad8(a2 + k2te) | pad8(a2 + len2) << 12 | (i % kSdWindow) << 24
//   w = pad8(le) | pad8(te) << 11 | (le >> 8) << 22 | (te >> 8) << 25 |
//       (step - 1) << 28 | hasSame << 29
// The identical combo's reach is the step of card c1's run at its entry:
// run[sHi] - run[sHi - step] (step 1, or 2 across a padding entry), where
// hasSame is set; otherwise sHi = 2, step 1, read and discarded.
// Entries are reordered within each kSdWindow-entry window (one warp's
// combos) to spread every quarter warp's indices over the shared-memory bank
// groups: entry k belongs to traverser combo
// i = (k & ~(kSdWindow - 1)) | (z >> 24 & (kSdWindow - 1)).
constexpr int kSdWindow = 32;
struct alignas(16) ShowdownInfo {
  uint32_t x, y, z, w;
};
PPS_HD inline int showdownCombo(int k, const ShowdownInfo& f) {
  return (k & ~(kSdWindow - 1)) | (int)((f.z >> 24) & (kSdWindow - 1));
}

// Four terminal nodes (showdown or fold) of one depth and one board state,
// evaluated together (-1: no node).
struct alignas(16) TermGroup {
  int node[4];
};

// A terminal group as one traverser's kernels read it: the state's list
// sizes and table offsets, the four nodes' rows and payoffs, so that a group
// CTA reaches its tables and rows one dependent load after its task word
// (instead of group -> node -> state -> tables and node -> row -> data).
// Records are stored per group and traverser, at 2 group + tr.
struct alignas(16) GroupRec {
  int no, nt;          // opponent / traverser list sizes
  int tabOff;          // u16 pool: showdown sdOff[tr]; fold csrOff[opp]
  int infoOff;         // showdown: sdInfoOff[tr] (showdown pool); fold: cardsOff[tr] (u8 pool)
  int sameOff;         // fold: sameOff[tr] (i16 pool); showdown: -1
  int mask;            // bit k: node slot k holds a node
  int kind;            // kTaskShowdown or kTaskFold
  int pad;
  uint32_t reachQ[4];  // opponent reach row of each node, in tr's layout (quads)
  uint32_t cfvQ[4];    // value rows (quads)
  float val[4][4];     // payoffs per node: showdown (win, tie, lose, 0), fold (v, 0, 0, 0)
};
static_assert(sizeof(GroupRec) == 128, "group records are one 128-byte line");

struct HostLayout {
  std::vector<NodeDev> nodes;
  std::vector<RowDev> rows;
  std::vector<float> termVal;  // 4 per (node, traverser): showdown
                               // (win, tie, lose, 0); fold (v, 0, 0, 0)
  std::vector<int> children;
  std::vector<StateDev> states;
  std::vector<uint8_t> poolU8;
  std::vector<uint16_t> poolU16;
  std::vector<int16_t> poolI16;
  std::vector<ShowdownInfo> poolSd;
  uint64_t regQuads = 0;          // regret (= strategy) pool size
  uint64_t cfvQuads = 0;
  uint64_t reachQuads[2] = {0, 0};
  // Warp task lists (kernels.cuh task words) per traverser and depth:
  // forward = the opponent's decide nodes in 128-quad chunks plus one task
  // per chance branch; backward = showdowns, folds, chance chunks, decide
  // chunks (longest tasks first).
  std::vector<std::vector<int>> fwdTasks[2], bwdTasks[2];
  // The f32 iteration's backward lists: terminal group tasks per depth
  // (node field = index into `groups`; the same for both traversers) and
  // the chance + decide tasks per traverser and depth.
  std::vector<TermGroup> groups;
  std::vector<GroupRec> groupRecs;  // per group and traverser, at 2 group + tr
  std::vector<std::vector<int>> sdGroupTasks, fdGroupTasks;
  std::vector<std::vector<int>> innerTasks[2];
  // Decide records (decide.cuh) of the default iteration: the pool, per
  // traverser and depth the backward record offsets (16-byte units), and
  // per traverser and FORWARD LEVEL the forward ones. A forward task (an
  // opponent decide node's chunk, a chance branch) reads the reach row that
  // its node's nearest forward-working ancestor wrote (the traverser's own
  // decide nodes pass rows through unchanged), so its level is one more
  // than that ancestor's: a chain of opponent and chance nodes, about half
  // the depth. fwdDecide / fwdChance hold the same tasks as task words
  // (byte model); termAfter[tr][d] is the forward level after which every
  // reach row that depth d's terminal nodes read is written (-1: at the
  // start of the half-step).
  std::vector<uint32_t> recPool;
  std::vector<std::vector<uint32_t>> bwdRecs[2], fwdRecs[2];
  // Chance records in the same pool (decide.cuh): forward one per branch,
  // backward one per 128-combo chunk pointing at a per-node branch table.
  std::vector<std::vector<uint32_t>> fwdChanceRecs[2], bwdChanceRecs[2];
  // Branch tables: offset (16-byte units) and branch count.
  std::vector<std::pair<uint32_t, int>> chanceTables[2];
  std::vector<std::vector<int>> bwdChance[2], fwdChance[2], fwdDecide[2];
  std::vector<int> termAfter[2];
  // The staged plan's backward lists per traverser and LEVEL (see
  // buildBackwardLevels in layout.cpp): a traverser decide node's records
  // also compute the value rows of its opponent children, so those need no
  // level; decide and chance record offsets, the same work as task words
  // (byte model), per level the depths of the terminal nodes it reads (bit
  // d), and every record of the levels (their own copies, grouped by size
  // class: relocated on their own).
  std::vector<std::vector<uint32_t>> bwdRecsH[2], bwdChanceRecsH[2];
  std::vector<std::vector<int>> bwdTasksH[2];
  std::vector<uint64_t> bwdNeed[2];
  std::vector<uint32_t> levelRecs[2];
  int maxN = 0;        // largest list size (either side)
  int maxCardSeg = 0;  // longest card segment of any list
};

HostLayout buildLayout(const Tree& t);

// FNV-1a digest of every array and scalar of a layout, in a fixed order
// (tests pin layouts with it: equal digests, byte-identical layouts).
uint64_t layoutDigest(const HostLayout& L);

inline uint32_t quads(int n) { return (uint32_t)((n + 3) / 4); }

}  // namespace gb
}  // namespace pps
