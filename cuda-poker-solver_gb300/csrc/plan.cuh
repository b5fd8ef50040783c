// Launch plans shared by the single-spot engine and the forest: a DCFR
// iteration is a list of level launches (kernel, task list, traverser,
// algorithmic bytes), issued on a main stream with independent pairs forked
// onto a side stream (graph branches when captured).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "compiler.h"
#include "kernels.cuh"
#include "decide.cuh"
#include "pps_gb.h"
#include "terminal.cuh"
#include "tune.h"

namespace pps {
namespace gb {

#define GB_CK(call)                                                          \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      throw Error{e_ == cudaErrorMemoryAllocation ? PPS_GB_E_MEMORY          \
                                                  : PPS_GB_E_CUDA,           \
                  std::string("CUDA error: ") + cudaGetErrorString(e_) +     \
                      " (" #call ")"};                                       \
  } while (0)

struct ListRef {
  int off = 0, count = 0;
};

enum LaunchKind { kFwd, kBwdTerm, kBwdInt, kSdGroup, kFdGroup, kFwdMix, kBwdMix, kCounter,
                  kBwdFused };
inline const char* launchName(LaunchKind k) {
  static const char* names[] = {"fwd_level", "bwd_terminal", "bwd_interior", "bwd_showdown",
                                "bwd_fold",  "fwd_level",    "bwd_interior", "counter",
                                "bwd_level"};
  return names[k];
}

struct Launch {
  LaunchKind kind;
  int tr;
  ListRef list;
  double bytes;           // algorithmic bytes of this launch (f32 rows)
  bool withNext = false;  // independent of the next launch: run both at once
  ListRef list2{};        // kFwdMix / kBwdMix / kBwdFused: chance records (list: decide records)
  ListRef list3{}, list4{};  // kBwdFused: the showdown and fold group tasks
  double bytes2 = 0.0;    // list2's share of bytes (profile split)
  bool late = false;      // kFwdMix: late triggers (the fused plan)
  bool early = false;     // kFwdMix: regret copies before the wait (first half-step only)
  bool termWait = false;  // kBwdFused: its terminal groups wait for the previous grid
  // kSdGroup / kFdGroup: the list's groups are groupBase, groupBase + 1, ...
  // (one spot's layout): the kernels take a CTA's record from its task
  // index instead of loading the task word first. -1: read the list.
  int groupBase = -1;
  // kFwdMix: the list's records are recBase + k recStride (16-byte units;
  // one spot's layout), so the kernel computes a record's offset from its
  // index instead of loading it. -1: read the list.
  long long recBase = -1;
  uint32_t recStride = 0;
  long long chBase = -1;  // kFwdMix: the same for the chance records (list2)
  uint32_t chStride = 0;
  // kBwdMix: the level's records as arithmetic runs (one spot's layout),
  // used instead of the list when runsOn.
  bool runsOn = false;
  RecRuns runs{};
};

// What the level launches of a plan read: the tree, the f32 rows, the
// concatenated task lists, the per-spot counters.
struct PlanArgs {
  DevTree tree;
  DevRows<float> rows;
  const int* tasks;
  int* counter;
  int spots;    // counters advanced per iteration
  int maxN;     // largest combo list (shared scratch layout)
  size_t smem;  // bwdScratchBytes<float>(maxN)
  const GroupRec* groups;  // terminal group records (2 group + traverser)
  size_t smemSd, smemFd;  // sdGroupSmem / fdGroupSmem(maxN)
  const uint32_t* recs;      // decide record pool
  const uint32_t* recTasks;  // record offsets (the record and chance lists index these)
  LaunchShape shape{};       // grids of the level and group launches (tune.h)
};

inline unsigned gridOf(int count) { return (unsigned)std::min(count, 1 << 20); }

// One CFR-mode launch of the plan on stream s. Internal linkage, like the
// kernels it launches that have no template parameter: each translation
// unit launches (and sets the shared-memory limit of) its own copy.
static inline void issueLaunch(const PlanArgs& a, const Launch& l, cudaStream_t s) {
  const unsigned g = gridOf(l.list.count);
  const int* tk = a.tasks + l.list.off;
  switch (l.kind) {
    case kFwd:
      fwdLevelK<float><<<g, kThreads, 0, s>>>(a.tree, a.rows, tk, l.list.count, l.tr, 0);
      break;
    case kBwdTerm:
      bwdTerminalK<float><<<g, kThreads, a.smem, s>>>(a.tree, a.rows, tk, l.list.count, l.tr,
                                                      a.maxN);
      break;
    case kBwdInt:
      bwdInteriorK<float><<<g, kThreads, 0, s>>>(a.tree, a.rows, tk, l.list.count, l.tr,
                                                 kModeCFR);
      break;
    case kSdGroup:
      launchSdGroups(cappedGrid(g, a.shape.sdCap), a.smemSd, s, a.tree, a.rows,
                     l.groupBase >= 0 ? a.groups + 2 * (size_t)l.groupBase : a.groups,
                     l.groupBase >= 0 ? nullptr : tk, l.list.count, l.tr, a.maxN);
      break;
    case kFdGroup:
      launchFdGroups(cappedGrid(g, a.shape.fdCap), a.smemFd, s, a.tree, a.rows,
                     l.groupBase >= 0 ? a.groups + 2 * (size_t)l.groupBase : a.groups,
                     l.groupBase >= 0 ? nullptr : tk, l.list.count, l.tr, a.maxN);
      break;
    case kBwdFused: {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(cappedGrid(gridOf(recordCtas(l.list.count) + l.list2.count +
                                           l.list3.count + l.list4.count),
                                    a.shape.bwdCap));
      cfg.blockDim = dim3(kThreads);
      cfg.dynamicSmemBytes = fusedLevelSmem(a.maxN);
      cfg.stream = s;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      attr[0].val.programmaticStreamSerializationAllowed = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      GB_CK(cudaLaunchKernelEx(&cfg, bwdLevelFusedK, a.tree, a.rows, a.recs,
                               a.recTasks + l.list.off, l.list.count, a.recTasks + l.list2.off,
                               l.list2.count, a.groups, a.tasks + l.list3.off, l.list3.count,
                               a.tasks + l.list4.off, l.list4.count, l.tr, a.maxN,
                               l.termWait ? 1 : 0));
      break;
    }
    case kFwdMix:
    case kBwdMix: {
      // Programmatic dependent launch: the grid may start while the
      // previous kernel in the stream drains (the kernels wait for it
      // before touching rows).
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(cappedGrid(gridOf(recordCtas(l.list.count) + l.list2.count),
                                    l.kind == kFwdMix ? a.shape.fwdCap : a.shape.bwdCap));
      cfg.blockDim = dim3(kThreads);
      cfg.dynamicSmemBytes = l.kind == kFwdMix ? fwdStageBytes() : bwdStageBytes();
      cfg.stream = s;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      attr[0].val.programmaticStreamSerializationAllowed = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      const uint32_t* rt = a.recTasks + l.list.off;
      const uint32_t* ch = a.recTasks + l.list2.off;  // chance record offsets
      if (l.kind == kFwdMix)
        GB_CK(cudaLaunchKernelEx(&cfg, fwdLevelMixK, a.tree, a.rows, a.recs,
                                 l.recBase >= 0 ? nullptr : rt, l.list.count,
                                 l.chBase >= 0 ? nullptr : ch, l.list2.count, l.tr,
                                 l.late ? 1 : 0, l.early ? 1 : 0,
                                 (uint32_t)(l.recBase >= 0 ? l.recBase : 0), l.recStride,
                                 (uint32_t)(l.chBase >= 0 ? l.chBase : 0), l.chStride));
      else
        GB_CK(cudaLaunchKernelEx(&cfg, bwdLevelMixK, a.tree, a.rows, a.recs,
                                 l.runsOn ? nullptr : rt, l.list.count, ch, l.list2.count, l.tr,
                                 l.runs));
      break;
    }
    case kCounter:
      advanceCounterK<<<(a.spots + 255) / 256, 256, 0, s>>>(a.counter, a.spots);
      break;
  }
}

// Streams and events of a plan with up to kSides + 1 concurrent branches.
constexpr int kTermRot = 4;  // side streams per terminal kind, used in turn by depth
constexpr int kSides = 1 + 2 * kTermRot;
struct Branches {
  cudaStream_t main = nullptr, side[kSides] = {};
  cudaEvent_t fork = nullptr, join[kSides] = {};
  void create(cudaStream_t mainStream) {
    main = mainStream;
    GB_CK(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    for (int k = 0; k < kSides; ++k) {
      GB_CK(cudaStreamCreateWithFlags(&side[k], cudaStreamNonBlocking));
      GB_CK(cudaEventCreateWithFlags(&join[k], cudaEventDisableTiming));
    }
  }
  void destroy() {
    if (fork) cudaEventDestroy(fork);
    for (int k = 0; k < kSides; ++k) {
      if (side[k]) cudaStreamDestroy(side[k]);
      if (join[k]) cudaEventDestroy(join[k]);
    }
  }
};

// Issues a plan; a run of launches chained by withNext runs concurrently:
// the first on the main stream, the others on side streams forked from it
// and joined back (graph branches under capture). `one` issues a single
// launch on a stream.
template <typename IssueOne>
void issuePlan(const std::vector<Launch>& P, const Branches& b, IssueOne&& one) {
  for (size_t i = 0; i < P.size();) {
    size_t j = i;
    while (j + 1 < P.size() && P[j].withNext && (int)(j - i) < kSides) ++j;
    if (j == i) {
      one(P[i], b.main);
      ++i;
      continue;
    }
    GB_CK(cudaEventRecord(b.fork, b.main));
    for (size_t k = i + 1; k <= j; ++k) GB_CK(cudaStreamWaitEvent(b.side[k - i - 1], b.fork, 0));
    one(P[i], b.main);
    for (size_t k = i + 1; k <= j; ++k) one(P[k], b.side[k - i - 1]);
    for (size_t k = i + 1; k <= j; ++k) {
      GB_CK(cudaEventRecord(b.join[k - i - 1], b.side[k - i - 1]));
      GB_CK(cudaStreamWaitEvent(b.main, b.join[k - i - 1], 0));
    }
    i = j + 1;
  }
}

// The default iteration as a staged plan: per traverser half-step and
// depth, the forward launches (run together), the showdown and fold group
// launches, and the backward interior launches (run together). Terminal
// values depend only on reach rows, so a depth's terminal groups start as
// soon as the forward level that wrote their reach rows is done, on their
// own streams, beside the rest of the forward pass; a backward level waits
// only for the terminals one depth below it.
struct HalfStep {
  std::vector<std::vector<Launch>> fwd;  // per forward level (layout.h)
  // Backward launches per level (layout.h), deepest first; bwdNeed
  // per level: the depths (bit d) of the terminal groups its nodes read.
  // Without bwdNeed, per depth, deepest first (each waiting for the
  // terminals one depth below).
  std::vector<std::vector<Launch>> bwd;
  std::vector<uint64_t> bwdNeed;
  std::vector<Launch> sd, fd;            // per depth (count 0: none)
  // Per depth: the forward level after which its terminal groups may
  // start (-1: at the start of the half-step).
  std::vector<int> termAfter;
};
struct StagedPlan {
  HalfStep half[2];
  Launch counter{kCounter, 0, ListRef{}, 0.0};
  // Every launch in an order that respects the dependencies (profile pass).
  std::vector<Launch> flat() const {
    std::vector<Launch> out;
    for (const HalfStep& h : half) {
      for (const auto& set : h.fwd) out.insert(out.end(), set.begin(), set.end());
      for (size_t d = 0; d < h.sd.size(); ++d) {
        if (h.sd[d].list.count) out.push_back(h.sd[d]);
        if (h.fd[d].list.count) out.push_back(h.fd[d]);
      }
      if (!h.bwdNeed.empty())
        for (const auto& set : h.bwd) out.insert(out.end(), set.begin(), set.end());
      else
        for (size_t d = h.bwd.size(); d-- > 0;)
          out.insert(out.end(), h.bwd[d].begin(), h.bwd[d].end());
    }
    out.push_back(counter);
    for (Launch& l : out) l.withNext = false;
    return out;
  }
};

struct StagedEvents {
  cudaEvent_t start = nullptr, lfork = nullptr, ljoin = nullptr;
  std::vector<cudaEvent_t> fwd, sd, fd;
  void ensure(int D) {
    auto mk = [](cudaEvent_t& e) {
      if (!e) GB_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    };
    mk(start);
    mk(lfork);
    mk(ljoin);
    for (auto* v : {&fwd, &sd, &fd}) {
      while ((int)v->size() < D) v->push_back(nullptr);
      for (auto& e : *v) mk(e);
    }
  }
  void destroy() {
    for (cudaEvent_t e : {start, lfork, ljoin})
      if (e) cudaEventDestroy(e);
    for (auto* v : {&fwd, &sd, &fd})
      for (cudaEvent_t e : *v)
        if (e) cudaEventDestroy(e);
    start = lfork = ljoin = nullptr;
    fwd.clear();
    sd.clear();
    fd.clear();
  }
};

// Issues a staged plan: main stream b.main, level partner b.side[0], the
// showdown and fold groups of depth d on b.side[1 + 2 (d mod kTermRot)] and
// the stream after it. Streams used in turn let the groups of consecutive
// depths run at once: a depth's groups wait for the forward level that
// wrote their reach rows, not for the previous depth's groups.
template <typename IssueOne>
void issueStaged(const StagedPlan& P, const Branches& b, StagedEvents& ev, IssueOne&& one) {
  auto issueSet = [&](const std::vector<Launch>& set) {
    if (set.empty()) return;
    if (set.size() == 1) {
      one(set[0], b.main);
      return;
    }
    GB_CK(cudaEventRecord(ev.lfork, b.main));
    GB_CK(cudaStreamWaitEvent(b.side[0], ev.lfork, 0));
    one(set[0], b.main);
    for (size_t k = 1; k < set.size(); ++k) one(set[k], b.side[0]);
    GB_CK(cudaEventRecord(ev.ljoin, b.side[0]));
    GB_CK(cudaStreamWaitEvent(b.main, ev.ljoin, 0));
  };
  for (const HalfStep& h : P.half) {
    const int D = (int)h.sd.size(), F = (int)h.fwd.size();
    ev.ensure(std::max(D, F));
    GB_CK(cudaEventRecord(ev.start, b.main));
    std::vector<char> sdOpen(D, 0), fdOpen(D, 0);
    auto startTerminals = [&](int d, int after) {  // depth d's reach rows are written
      for (int k = 0; k < 2; ++k) {
        const Launch& l = k == 0 ? h.sd[d] : h.fd[d];
        if (!l.list.count) continue;
        cudaStream_t s = b.side[1 + 2 * (d % kTermRot) + k];
        GB_CK(cudaStreamWaitEvent(s, after < 0 ? ev.start : ev.fwd[after], 0));
        one(l, s);
        GB_CK(cudaEventRecord(k == 0 ? ev.sd[d] : ev.fd[d], s));
        (k == 0 ? sdOpen : fdOpen)[d] = 1;
      }
    };
    auto joinTerminals = [&](int d) {
      if (d >= D) return;
      if (sdOpen[d]) GB_CK(cudaStreamWaitEvent(b.main, ev.sd[d], 0));
      if (fdOpen[d]) GB_CK(cudaStreamWaitEvent(b.main, ev.fd[d], 0));
      sdOpen[d] = fdOpen[d] = 0;
    };
    // A depth whose terminals need a level past the last one that launches
    // (none does, but keep every depth covered) starts after the last.
    auto afterOf = [&](int d) {
      const int a = d < (int)h.termAfter.size() ? h.termAfter[d] : F - 1;
      return std::min(a, F - 1);
    };
    for (int d = 0; d < D; ++d)
      if (afterOf(d) < 0) startTerminals(d, -1);
    for (int lv = 0; lv < F; ++lv) {
      issueSet(h.fwd[lv]);
      GB_CK(cudaEventRecord(ev.fwd[lv], b.main));
      for (int d = 0; d < D; ++d)
        if (afterOf(d) == lv) startTerminals(d, lv);
    }
    if (!h.bwdNeed.empty()) {
      for (size_t lv = 0; lv < h.bwd.size(); ++lv) {
        for (int d = 0; d < D && d < 64; ++d)
          if ((h.bwdNeed[lv] >> d) & 1) joinTerminals(d);
        issueSet(h.bwd[lv]);
      }
    } else {
      for (int d = D - 1; d >= 0; --d) {
        joinTerminals(d + 1);
        issueSet(h.bwd[d]);
      }
    }
    for (int d = 0; d < D; ++d) joinTerminals(d);
  }
  one(P.counter, b.main);
}

// Splits a backward level list (sorted showdown, fold, chance, decide) into
// its terminal head and interior tail.
inline int terminalCount(const std::vector<int>& v) {
  int nt = 0;
  while (nt < (int)v.size() && (v[nt] & 3) >= 2) ++nt;
  return nt;
}

// Raises the dynamic shared-memory limit of a kernel to at least `bytes`
// (never lowers it: graphs captured earlier keep their launch sizes valid).
void raiseSmemLimit(const void* kernel, size_t bytes);

}  // namespace gb
}  // namespace pps
