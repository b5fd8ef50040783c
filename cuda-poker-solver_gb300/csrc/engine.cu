// Device engine (see engine.h): uploads the layout, captures one DCFR
// iteration (two alternating half-steps plus the counter bump, the
// reference's captureGraph, cuda/gpu_cfr.cu:844-868) as a CUDA graph, and
// runs the FP64 walks.
//
// An iteration is described once as a launch plan (kernel, task list,
// traverser, algorithmic bytes); graph capture and the profile pass replay
// the plan.
#include "engine.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "kernels.cuh"
#include "plan.cuh"
#include "rowcodec.h"
#include "terminal.cuh"
#include "tune.h"
#include "pps_gb.h"

namespace pps {
namespace gb {

void raiseSmemLimit(const void* kernel, size_t bytes) {
  static std::mutex m;
  static std::map<const void*, size_t> limit;
  std::lock_guard<std::mutex> lock(m);
  size_t& cur = limit[kernel];
  if (bytes <= cur) return;
  GB_CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
}

namespace {

template <typename V>
V* alloc(size_t count, size_t& bytes) {
  V* p = nullptr;
  GB_CK(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(V)));
  bytes += std::max<size_t>(count, 1) * sizeof(V);
  return p;
}

// A record list at one stride from its first record: {first, stride}, else
// {-1, 0} (a layout places each forward level's decide records so, and its
// chance records one after another).
std::pair<long long, uint32_t> strided(const std::vector<uint32_t>& offs) {
  if (offs.empty()) return {-1, 0};
  const uint32_t d = offs.size() > 1 ? offs[1] - offs[0] : 0;
  for (size_t k = 0; k < offs.size(); ++k)
    if (offs[k] != offs[0] + (uint32_t)k * d) return {-1, 0};
  return {(long long)offs[0], d};
}

// A record list as at most four arithmetic runs (a layout groups each
// backward level's records by size class); false if it needs more.
bool recRuns(const std::vector<uint32_t>& offs, RecRuns& R) {
  if (offs.empty()) return false;
  size_t i = 0;
  int j = 0;
  while (i < offs.size()) {
    if (j == 4) return false;
    const uint32_t st = i + 1 < offs.size() ? offs[i + 1] - offs[i] : 0;
    size_t e = i + 1;
    while (e < offs.size() && offs[e] == offs[i] + (uint32_t)(e - i) * st) ++e;
    R.base[j] = offs[i];
    R.stride[j] = st;
    R.end[j] = (uint32_t)e;
    ++j;
    i = e;
  }
  for (; j < 4; ++j) {
    R.base[j] = R.stride[j] = 0;
    R.end[j] = 0xffffffffu;
  }
  return true;
}

// First group of a group task list whose groups are consecutive (a layout
// appends each depth's groups together), else -1.
int consecutiveGroups(const std::vector<int>& tasks) {
  if (tasks.empty()) return -1;
  const int g0 = (int)((unsigned)tasks[0] >> 8);
  for (size_t i = 0; i < tasks.size(); ++i)
    if ((int)((unsigned)tasks[i] >> 8) != g0 + (int)i) return -1;
  return g0;
}

}  // namespace

struct Engine::Dev {
  cudaStream_t stream = nullptr;
  Branches br;  // main = stream, plus the side branch
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void*> owned;
  DevTree tree{};
  DevRows<float> rowsF{};
  DevRows<double> rowsD{};
  float* coef = nullptr;
  size_t coefCap = 0;  // iterations the coef table holds
  int* counter = nullptr;
  int* tasks = nullptr;
  std::vector<int> hostTasks;  // host copy of the concatenated task lists
  int* qTasks = nullptr;       // walkFrom's task lists (grown on demand)
  size_t qCap = 0;
  std::vector<ListRef> fwd[2], bwd[2];
  std::vector<ListRef> sdG, fdG, inner[2];  // the group plan's backward lists
  std::vector<ListRef> bCh[2], fCh[2];       // its chance word lists
  std::vector<ListRef> bRec[2], fRec[2];     // its decide record lists (into recTasks)
  std::vector<ListRef> bRecH[2], bChH[2];    // backward per level (the staged plan)
  GroupRec* groups = nullptr;
  uint32_t* recs = nullptr;
  uint32_t* recTasks = nullptr;
  float* stratLo = nullptr;  // low words of the strategy rows (compensated sums)
  std::vector<Launch> plan[3];  // per engine kind: one iteration (kind 0 flattened)
  StagedPlan staged;           // kind 0 as captured
  StagedEvents sev;
  bool walkReady = false;
  LaunchShape shape;  // grids of the captured iteration (tune.h)
  int maxN = 0;
  size_t smemF = 0, smemD = 0;

  template <typename P>
  P* own(P* p) {
    owned.push_back((void*)p);
    return p;
  }
};

namespace {

template <typename V>
V* upload(Engine::Dev& d, const std::vector<V>& v, size_t& bytes, int64_t& h2d) {
  if (v.empty()) return nullptr;
  V* p = nullptr;
  GB_CK(cudaMalloc(&p, v.size() * sizeof(V)));
  GB_CK(cudaMemcpy(p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice));
  bytes += v.size() * sizeof(V);
  h2d += (int64_t)(v.size() * sizeof(V));
  return d.own(p);
}

PlanArgs planArgs(const Engine::Dev& d) {
  return PlanArgs{d.tree,   d.rowsF, d.tasks, d.counter, 1, d.maxN, d.smemF, d.groups,
                  sdGroupSmem(d.maxN), fdGroupSmem(d.maxN), d.recs, d.recTasks, d.shape};
}

// Issues one planned launch (CFR mode, f32 rows) on stream s.
void issue(Engine::Dev& d, const Launch& l, cudaStream_t s) {
  issueLaunch(planArgs(d), l, s);
}

}  // namespace

Engine::Engine(const Tree& t, HostLayout&& layout)
    : t_(t), L_(std::move(layout)), d_(new Dev()) {
  Dev& d = *d_;
  size_t& B = deviceBytes_;
  GB_CK(cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking));
  d.br.create(d.stream);
  d.tree.nodes = upload(d, L_.nodes, B, h2d_);
  d.tree.rows = upload(d, L_.rows, B, h2d_);
  d.tree.termVal = upload(d, L_.termVal, B, h2d_);
  d.tree.children = upload(d, L_.children, B, h2d_);
  d.tree.states = upload(d, L_.states, B, h2d_);
  d.tree.poolU8 = upload(d, L_.poolU8, B, h2d_);
  d.tree.poolU16 = upload(d, L_.poolU16, B, h2d_);
  d.tree.poolI16 = upload(d, L_.poolI16, B, h2d_);
  d.tree.poolSd = upload(d, L_.poolSd, B, h2d_);
  d.tree.regret = d.own(alloc<float>(L_.regQuads * 4, B));
  d.tree.strat = d.own(alloc<float>(L_.regQuads * 4, B));
  d.rowsF.cfv = d.own(alloc<float>(L_.cfvQuads * 4, B));
  for (int tr = 0; tr < 2; ++tr)
    d.rowsF.reach[tr] = d.own(alloc<float>(L_.reachQuads[tr] * 4, B));
  d.counter = d.own(alloc<int>(1, B));
  d.coefCap = 1024;
  d.coef = d.own(alloc<float>(d.coefCap * 3, B));
  d.tree.counter = d.counter;
  d.tree.coef = d.coef;
  d.tree.err = d.own(alloc<int>(1, B));
  GB_CK(cudaMemset(d.tree.err, 0, sizeof(int)));

  // Root reach rows: the opponent's range weights (padding zero).
  for (int tr = 0; tr < 2; ++tr) {
    const Side& opp = t_.side[1 - tr];
    std::vector<float> row(quads(opp.n) * 4, 0.0f);
    for (int j = 0; j < opp.n; ++j) row[j] = (float)opp.w[j];
    GB_CK(cudaMemcpy(d.rowsF.reach[tr], row.data(), row.size() * sizeof(float),
                     cudaMemcpyHostToDevice));
    h2d_ += (int64_t)(row.size() * sizeof(float));
  }

  // Task lists, concatenated.
  std::vector<int> all;
  auto addList = [&](const std::vector<int>& v) {
    ListRef r{(int)all.size(), (int)v.size()};
    all.insert(all.end(), v.begin(), v.end());
    return r;
  };
  const int D = (int)L_.bwdTasks[0].size();
  for (int tr = 0; tr < 2; ++tr)
    for (int dd = 0; dd < D; ++dd) {
      d.fwd[tr].push_back(addList(L_.fwdTasks[tr][dd]));
      d.bwd[tr].push_back(addList(L_.bwdTasks[tr][dd]));
      d.inner[tr].push_back(addList(L_.innerTasks[tr][dd]));
    }
  for (int dd = 0; dd < D; ++dd) {
    d.sdG.push_back(addList(L_.sdGroupTasks[dd]));
    d.fdG.push_back(addList(L_.fdGroupTasks[dd]));
  }
  std::vector<uint32_t> recTasks;
  auto addRecs = [&](const std::vector<uint32_t>& v, std::vector<ListRef>& dst) {
    dst.push_back(ListRef{(int)recTasks.size(), (int)v.size()});
    recTasks.insert(recTasks.end(), v.begin(), v.end());
  };
  for (int tr = 0; tr < 2; ++tr) {
    for (int dd = 0; dd < D; ++dd) {  // backward: per depth
      addRecs(L_.bwdRecs[tr][dd], d.bRec[tr]);
      addRecs(L_.bwdChanceRecs[tr][dd], d.bCh[tr]);
    }
    for (size_t lv = 0; lv < L_.fwdRecs[tr].size(); ++lv) {  // forward: per level
      addRecs(L_.fwdRecs[tr][lv], d.fRec[tr]);
      addRecs(L_.fwdChanceRecs[tr][lv], d.fCh[tr]);
    }
    for (size_t lv = 0; lv < L_.bwdRecsH[tr].size(); ++lv) {  // backward: per level
      addRecs(L_.bwdRecsH[tr][lv], d.bRecH[tr]);
      addRecs(L_.bwdChanceRecsH[tr][lv], d.bChH[tr]);
    }
  }
  d.recs = upload(d, L_.recPool, B, h2d_);
  d.recTasks = upload(d, recTasks, B, h2d_);
  d.tasks = upload(d, all, B, h2d_);
  d.hostTasks = all;
  d.groups = reinterpret_cast<GroupRec*>(upload(d, L_.groupRecs, B, h2d_));

  d.maxN = L_.maxN;
  d.smemF = bwdScratchBytes<float>(d.maxN);
  d.smemD = bwdScratchBytes<double>(d.maxN);
  raiseSmemLimit((const void*)bwdLevelK<float>, d.smemF);
  raiseSmemLimit((const void*)bwdLevelK<double>, d.smemD);
  raiseSmemLimit((const void*)bwdTerminalK<float>, d.smemF);
  raiseGroupSmem(d.maxN);
  buildPlans();
  engineKind_ = 0;
  zeroRows();
}

Engine::~Engine() {
  if (!d_) return;
  if (d_->qTasks) cudaFree(d_->qTasks);
  if (d_->exec) cudaGraphExecDestroy(d_->exec);
  if (d_->graph) cudaGraphDestroy(d_->graph);
  if (d_->stream) cudaStreamSynchronize(d_->stream);
  for (void* p : d_->owned) cudaFree(p);
  if (d_->stream) cudaStreamDestroy(d_->stream);
  d_->br.destroy();
  d_->sev.destroy();
}

void* Engine::stream() const { return (void*)d_->stream; }

// Algorithmic f32 row bytes of one task: every row the task must read or
// write once (index tables excluded).
double Engine::taskBytes(int task, int tr, bool fwd) const {
  const Tree& t = t_;
  const int u = (int)((unsigned)task >> 8), sub = (task >> 2) & 63, kind = task & 3;
  const Node& nd = t.nodes[u];
  auto share = [&](int n) {  // the quads of this task's chunk
    const int q = (int)quads(n), q0 = sub * kChunkQuads, q1 = std::min(q, q0 + kChunkQuads);
    return std::max(0, q1 - q0) * 4.0 * n / std::max(4 * q, 1);
  };
  if (fwd) {
    if (kind == kTaskChance) {
      const int ch = t.children[nd.childBase + sub];
      return 4.0 * t.n(ch, 1 - tr) + 4.0 * t.n(u, 1 - tr) / nd.nChildren;
    }
    return 4.0 * share(t.n(u, 1 - tr)) * (1 + 2.0 * nd.na);
  }
  switch (kind) {
    case kTaskShowdown:
    case kTaskFold:
      return 4.0 * (t.n(u, 1 - tr) + t.n(u, tr));
    case kTaskChance: {
      double kids = 0;
      for (int k = 0; k < nd.nChildren; ++k) kids += t.n(t.children[nd.childBase + k], tr);
      const int n = t.n(u, tr);
      const int e = std::max(0, std::min(n, (sub + 1) * kChanceChunk) - sub * kChanceChunk);
      return 4.0 * e * (1.0 + kids / std::max(n, 1));
    }
    default:
      // Traverser's node: regret and strategy rows read and written, child
      // values read, own value written (plus the strategy's low words read
      // and written with compensated sums).
      return nd.player == tr ? 4.0 * share(t.n(u, tr)) * ((comp_ ? 7.0 : 5.0) * nd.na + 1)
                             : 4.0 * share(t.n(u, tr)) * (nd.na + 1.0);
  }
}

// Plans of one iteration. Kind 0 (default): the staged plan of plan.cuh
// (decide records and chance tasks per level; showdown / fold groups of a
// depth started once its reach rows are written). Kind 1: per level, one
// CTA per terminal node (bwdTerminalK) beside the node-based interior
// tasks (bwdInteriorK), the arithmetic of the walks.
void Engine::buildPlans() {
  Dev& d = *d_;
  auto listBytes = [&](const std::vector<int>& v, int tr, bool fwd) {
    double b = 0;
    for (int task : v) b += taskBytes(task, tr, fwd);
    return b;
  };
  auto kindOnly = [](const std::vector<int>& v, int kind) {
    std::vector<int> out;
    for (int w : v)
      if ((w & 3) == kind) out.push_back(w);
    return out;
  };
  auto groupBytes = [&](const std::vector<int>& v, int tr) {
    double b = 0;
    for (int task : v) {
      const TermGroup& g = L_.groups[(unsigned)task >> 8];
      for (int k = 0; k < 4; ++k)
        if (g.node[k] >= 0) b += taskBytes(makeTask(task & 3, 0, g.node[k]), tr, false);
    }
    return b;
  };
  // Kind 0: the staged plan (decide records, chance words, terminal groups
  // started right after the forward level that wrote their reach rows).
  const int D = (int)d.fwd[0].size();
  for (int tr = 0; tr < 2; ++tr) {
    HalfStep& h = d.staged.half[tr];
    const int F = (int)d.fRec[tr].size();
    h.fwd.assign(F, {});
    h.bwd.assign(D, {});
    h.sd.assign(D, Launch{kSdGroup, tr, ListRef{}, 0.0});
    h.fd.assign(D, Launch{kFdGroup, tr, ListRef{}, 0.0});
    h.termAfter = L_.termAfter[tr];
    for (int lv = 0; lv < F; ++lv) {
      if (d.fRec[tr][lv].count || d.fCh[tr][lv].count) {
        Launch l{kFwdMix, tr, d.fRec[tr][lv],
                 listBytes(L_.fwdDecide[tr][lv], tr, true) +
                     listBytes(L_.fwdChance[tr][lv], tr, true)};
        l.list2 = d.fCh[tr][lv];
        l.bytes2 = listBytes(L_.fwdChance[tr][lv], tr, true);
        l.early = tr == 0;  // the first half-step of the iteration
        const auto st = strided(L_.fwdRecs[tr][lv]), sc = strided(L_.fwdChanceRecs[tr][lv]);
        l.recBase = st.first;
        l.recStride = st.second;
        l.chBase = sc.first;
        l.chStride = sc.second;
        h.fwd[lv].push_back(l);
      }
    }
    for (int dd = 0; dd < D; ++dd) {
      if (d.sdG[dd].count) {
        h.sd[dd] = {kSdGroup, tr, d.sdG[dd], groupBytes(L_.sdGroupTasks[dd], tr)};
        h.sd[dd].groupBase = consecutiveGroups(L_.sdGroupTasks[dd]);
      }
      if (d.fdG[dd].count) {
        h.fd[dd] = {kFdGroup, tr, d.fdG[dd], groupBytes(L_.fdGroupTasks[dd], tr)};
        h.fd[dd].groupBase = consecutiveGroups(L_.fdGroupTasks[dd]);
      }
    }
    // Backward per level (layout.h): each launch waits for the
    // terminal depths its nodes read.
    const int H = (int)d.bRecH[tr].size();
    h.bwd.assign(H, {});
    h.bwdNeed = L_.bwdNeed[tr];
    for (int lv = 0; lv < H; ++lv) {
      if (!d.bRecH[tr][lv].count && !d.bChH[tr][lv].count) continue;
      Launch l{kBwdMix, tr, d.bRecH[tr][lv], listBytes(L_.bwdTasksH[tr][lv], tr, false)};
      l.list2 = d.bChH[tr][lv];
      l.bytes2 = listBytes(kindOnly(L_.bwdTasksH[tr][lv], kTaskChance), tr, false);
      l.runsOn = recRuns(L_.bwdRecsH[tr][lv], l.runs);
      h.bwd[lv].push_back(l);
    }
  }
  d.plan[0] = d.staged.flat();
  d.sev.ensure(D);  // events exist before any capture
  // Kind 1: per level, one CTA per terminal node beside the interior tasks.
  std::vector<Launch>& P = d.plan[1];
  P.clear();
  for (int tr = 0; tr < 2; ++tr) {
    for (int dd = 0; dd < D; ++dd)
      if (d.fwd[tr][dd].count)
        P.push_back({kFwd, tr, d.fwd[tr][dd], listBytes(L_.fwdTasks[tr][dd], tr, true)});
    for (int dd = D - 1; dd >= 0; --dd) {
      std::vector<Launch> set;
      const std::vector<int>& v = L_.bwdTasks[tr][dd];
      const int nt = terminalCount(v);
      if (nt)
        set.push_back({kBwdTerm, tr, ListRef{d.bwd[tr][dd].off, nt},
                       listBytes(std::vector<int>(v.begin(), v.begin() + nt), tr, false)});
      if (d.inner[tr][dd].count)
        set.push_back({kBwdInt, tr, d.inner[tr][dd], listBytes(L_.innerTasks[tr][dd], tr, false)});
      for (size_t k = 0; k + 1 < set.size(); ++k) set[k].withNext = true;
      P.insert(P.end(), set.begin(), set.end());
    }
  }
  P.push_back({kCounter, 0, ListRef{}, 0.0});
  // Kind 2 (narrow ranges): the staged plan's forward levels, then one
  // fused launch per backward level (records, chance, showdown and fold
  // groups of that depth), all on one stream.
  std::vector<Launch>& F = d.plan[2];
  F.clear();
  if (d.maxN <= kFusedMaxN) {
    for (int tr = 0; tr < 2; ++tr) {
      const HalfStep& h = d.staged.half[tr];
      for (const auto& set : h.fwd)
        for (Launch l : set) {
          l.late = true;
          F.push_back(l);
        }
      bool first = true;
      for (int dd = D - 1; dd >= 0; --dd) {
        Launch l{kBwdFused, tr, d.bRec[tr][dd], 0.0};
        l.termWait = first;
        l.list2 = d.bCh[tr][dd];
        l.list3 = d.sdG[dd];
        l.list4 = d.fdG[dd];
        if (!l.list.count && !l.list2.count && !l.list3.count && !l.list4.count) continue;
        l.bytes = listBytes(kindOnly(L_.bwdTasks[tr][dd], kTaskDecide), tr, false) +
                  listBytes(L_.bwdChance[tr][dd], tr, false) + h.sd[dd].bytes + h.fd[dd].bytes;
        F.push_back(l);
        first = false;
      }
    }
    F.push_back({kCounter, 0, ListRef{}, 0.0});
  }
}

void Engine::setCompensated(bool on) {
  Dev& d = *d_;
  if (on == comp_) return;
  GB_CK(cudaStreamSynchronize(d.stream));
  if (on) {
    if (!d.stratLo) d.stratLo = d.own(alloc<float>(L_.regQuads * 4, deviceBytes_));
    GB_CK(cudaMemsetAsync(d.stratLo, 0, L_.regQuads * 16, d.stream));
    GB_CK(cudaStreamSynchronize(d.stream));
  }
  d.tree.stratLo = on ? d.stratLo : nullptr;
  comp_ = on;
  buildPlans();  // the byte model counts the low words
  if (d.exec) {  // the captured kernels hold the old tree arguments
    cudaGraphExecDestroy(d.exec);
    cudaGraphDestroy(d.graph);
    d.exec = nullptr;
    d.graph = nullptr;
  }
}

void Engine::zeroRows() {
  Dev& d = *d_;
  GB_CK(cudaMemsetAsync(d.tree.regret, 0, L_.regQuads * 16, d.stream));
  GB_CK(cudaMemsetAsync(d.tree.strat, 0, L_.regQuads * 16, d.stream));
  if (d.tree.stratLo) GB_CK(cudaMemsetAsync(d.tree.stratLo, 0, L_.regQuads * 16, d.stream));
  GB_CK(cudaMemsetAsync(d.counter, 0, sizeof(int), d.stream));
  GB_CK(cudaStreamSynchronize(d.stream));
}

void Engine::setSchedule(const std::vector<float>& coef, int counter) {
  Dev& d = *d_;
  const size_t entries = coef.size() / 3;
  if (entries > d.coefCap) {
    GB_CK(cudaStreamSynchronize(d.stream));
    float* fresh = nullptr;
    const size_t cap = std::max(entries, d.coefCap * 2);
    GB_CK(cudaMalloc(&fresh, cap * 3 * sizeof(float)));
    for (auto& p : d.owned)
      if (p == (void*)d.coef) p = (void*)fresh;
    cudaFree(d.coef);
    deviceBytes_ += (cap - d.coefCap) * 3 * sizeof(float);
    d.coef = fresh;
    d.coefCap = cap;
    d.tree.coef = fresh;
    if (d.exec) {  // the captured kernels hold the old table address
      cudaGraphExecDestroy(d.exec);
      cudaGraphDestroy(d.graph);
      d.exec = nullptr;
      d.graph = nullptr;
    }
  }
  GB_CK(cudaMemcpyAsync(d.coef, coef.data(), coef.size() * sizeof(float),
                        cudaMemcpyHostToDevice, d.stream));
  h2d_ += (int64_t)(coef.size() * sizeof(float));
  setCounter(counter);
}

void Engine::setCounter(int counter) {
  Dev& d = *d_;
  GB_CK(cudaMemcpyAsync(d.counter, &counter, sizeof(int), cudaMemcpyHostToDevice,
                        d.stream));
  GB_CK(cudaStreamSynchronize(d.stream));
}

void Engine::capture() {
  Dev& d = *d_;
  if (d.exec) {
    cudaGraphExecDestroy(d.exec);
    cudaGraphDestroy(d.graph);
    d.exec = nullptr;
    d.graph = nullptr;
  }
  const std::vector<Launch>& P = d.plan[engineKind_];
  GB_CK(cudaStreamBeginCapture(d.stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t launchErr = cudaSuccess;
  auto one = [&](const Launch& l, cudaStream_t s) { issue(d, l, s); };
  if (engineKind_ == 0) issueStaged(d.staged, d.br, d.sev, one);
  else issuePlan(P, d.br, one);
  launchErr = cudaGetLastError();
  cudaGraph_t g = nullptr;
  const cudaError_t endErr = cudaStreamEndCapture(d.stream, &g);
  if (launchErr != cudaSuccess || endErr != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    GB_CK(launchErr);
    GB_CK(endErr);
  }
  d.graph = g;
  GB_CK(cudaGraphInstantiate(&d.exec, d.graph, 0));
  launchesPerIter_ = (int)P.size();
}

void Engine::setEngineKind(int kind) {
  if (kind == 2 && d_->plan[2].empty())
    throw Error{PPS_GB_E_ARG, "engine 2 (fused levels) needs lists of at most " +
                                  std::to_string(kFusedMaxN) + " combos"};
  tuned_ = true;
  const int k = kind == 1 || kind == 2 ? kind : 0;
  if (k == engineKind_ && d_->exec) return;
  engineKind_ = k;
  d_->shape.plan = k == 2 ? 2 : 0;
  capture();
}

void Engine::setShape(const LaunchShape& s) {
  if (s.plan != 0 && s.plan != 2) throw Error{PPS_GB_E_ARG, "launch shape: plan must be 0 or 2"};
  if (s.plan == 2 && d_->plan[2].empty())
    throw Error{PPS_GB_E_ARG, "engine 2 (fused levels) needs lists of at most " +
                                  std::to_string(kFusedMaxN) + " combos"};
  for (int c : {s.fwdCap, s.bwdCap, s.sdCap, s.fdCap})
    if (c < 0 || c > 64) throw Error{PPS_GB_E_ARG, "launch shape: caps must be 0..64"};
  tuned_ = true;
  d_->shape = s;
  engineKind_ = s.plan;
  capture();
}

LaunchShape Engine::shape() const { return d_->shape; }

// Times `shape` on this tree: capture, one warm-up replay, then `n` timed
// replays from iteration 0 of the schedule (the counter is reset first, so
// no replay reads past the table).
double Engine::timeShape(const LaunchShape& s, int n) {
  d_->shape = s;
  engineKind_ = s.plan;
  capture();
  setCounter(0);
  iterate(1);
  // The faster of two timings (a single short one is noisy against the 1%
  // margin below).
  const double a = timeIterations(n), b = timeIterations(n);
  return (a < b ? a : b) / n;
}

// Picks the launch shape of this tree: the cached one of its size class,
// else the fastest candidate by timing: the plan, then the showdown and
// fold grids together (every pair of caps, since their gains add: on the
// 48,255-node turn, 1 and 1 beat either alone), then the forward and
// backward grids, each candidate taking over only when it is at least 1%
// faster. The choice is cached for the class;
// the rows and the counter are zeroed afterwards (shapes compute identical
// rows).
void Engine::autotune() {
  if (tuned_) return;
  tuned_ = true;
  const TuneKey key = tuneKeyOf(d_->maxN, (int64_t)L_.regQuads * 16);
  LaunchShape cached;
  if (lookupShape(key, &cached) && (cached.plan == 0 || !d_->plan[2].empty())) {
    d_->shape = cached;
    engineKind_ = cached.plan;
    capture();
    return;
  }
  const int n = 4;
  LaunchShape best = d_->shape;
  best.plan = 0;
  double bestMs = timeShape(best, n);
  auto consider = [&](LaunchShape c) {
    if (c == best) return;
    const double ms = timeShape(c, n);
    if (ms < 0.99 * bestMs) {
      best = c;
      bestMs = ms;
    }
  };
  if (!d_->plan[2].empty()) {
    LaunchShape c = best;
    c.plan = 2;
    consider(c);
  }
  if (best.plan == 0) {
    const LaunchShape base = best;
    for (int sd : {0, 1, 2})
      for (int fd : {0, 1, 3}) {
        LaunchShape c = base;
        c.sdCap = sd;
        c.fdCap = fd;
        consider(c);
      }
  }
  for (int cap : {16}) {
    LaunchShape c = best;
    c.fwdCap = cap;
    consider(c);
    c = best;
    c.bwdCap = cap;
    consider(c);
  }
  if (!(d_->shape == best)) {
    d_->shape = best;
    engineKind_ = best.plan;
    capture();
  }
  storeShape(key, best, bestMs);
  zeroRows();
}

void Engine::iterate(int n) {
  Dev& d = *d_;
  if (!d.exec) capture();
  for (int i = 0; i < n; ++i) GB_CK(cudaGraphLaunch(d.exec, d.stream));
}

void Engine::sync() {
  GB_CK(cudaStreamSynchronize(d_->stream));
  checkDeviceError();
}

// One warp expects 16 bytes on its barrier that no copy delivers, and waits
// with the records' bounded wait and give-up path (warpCopiesLanded).
static __global__ void boundedWaitProbeK(int* err, int spins) {
  __shared__ unsigned long long bar;
  const int lane = (int)threadIdx.x & 31;
  if (lane == 0) {
    barInit(&bar);
    barExpect(&bar, 16);
  }
  __syncwarp();
  warpCopiesLanded(&bar, 0, err, lane, spins);
}

void Engine::probeBoundedWait(int spins) {
  boundedWaitProbeK<<<1, 32, 0, d_->stream>>>(d_->tree.err, spins);
  GB_CK(cudaGetLastError());
  GB_CK(cudaStreamSynchronize(d_->stream));
  checkDeviceError();
}

// A bounded wait in a kernel gave up (its results are not valid).
void Engine::checkDeviceError() {
  int e = 0;
  GB_CK(cudaMemcpy(&e, d_->tree.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    GB_CK(cudaMemset(d_->tree.err, 0, sizeof(int)));
    throw Error{PPS_GB_E_CUDA, "a device wait timed out (bulk copy never completed)"};
  }
}

double Engine::timeIterations(int n) {
  Dev& d = *d_;
  if (!d.exec) capture();
  cudaEvent_t a, b;
  GB_CK(cudaEventCreate(&a));
  GB_CK(cudaEventCreate(&b));
  GB_CK(cudaEventRecord(a, d.stream));
  iterate(n);
  GB_CK(cudaEventRecord(b, d.stream));
  GB_CK(cudaEventSynchronize(b));
  float ms = 0.0f;
  GB_CK(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  checkDeviceError();
  return ms;
}

std::vector<Engine::KernelStat> Engine::profile(int n, bool splitKinds) {
  Dev& d = *d_;
  // With splitKinds, each backward level launch is issued as one launch per
  // task kind (the lists are sorted by kind), attributing time per kind.
  static const char* kKindName[] = {"bwd_decide", "bwd_chance", "bwd_fold", "bwd_showdown"};
  std::vector<std::pair<Launch, std::string>> P;
  for (const Launch& l : d.plan[engineKind_]) {
    if (splitKinds && (l.kind == kFwdMix || l.kind == kBwdMix)) {
      // The level's records and chance records as two launches of the
      // same kernel.
      const bool fwd = l.kind == kFwdMix;
      if (l.list.count) {
        Launch r = l;
        r.list2 = ListRef{};
        r.bytes = l.bytes - l.bytes2;
        P.push_back({r, fwd ? "fwd_decide" : "bwd_decide"});
      }
      if (l.list2.count) {
        Launch c = l;
        c.list = ListRef{};
        c.bytes = l.bytes2;
        P.push_back({c, fwd ? "fwd_chance" : "bwd_chance"});
      }
      continue;
    }
    const bool bwd = l.kind == kBwdTerm || l.kind == kBwdInt;
    if (!bwd || !splitKinds) {
      P.push_back({l, launchName(l.kind)});
      continue;
    }
    int i = l.list.off;
    const int end = l.list.off + l.list.count;
    while (i < end) {
      const int kind = d.hostTasks[i] & 3;
      int j = i;
      double bytes = 0;
      while (j < end && (d.hostTasks[j] & 3) == kind) bytes += taskBytes(d.hostTasks[j++], l.tr, false);
      P.push_back({Launch{l.kind, l.tr, ListRef{i, j - i}, bytes}, kKindName[kind]});
      i = j;
    }
  }
  std::vector<cudaEvent_t> ev(2 * P.size() * (size_t)n);
  for (auto& e : ev) GB_CK(cudaEventCreate(&e));
  size_t k = 0;
  for (int it = 0; it < n; ++it)
    for (const auto& pl : P) {
      GB_CK(cudaEventRecord(ev[k++], d.stream));
      issue(d, pl.first, d.stream);
      GB_CK(cudaGetLastError());
      GB_CK(cudaEventRecord(ev[k++], d.stream));
    }
  GB_CK(cudaStreamSynchronize(d.stream));
  std::vector<KernelStat> out;
  k = 0;
  for (int it = 0; it < n; ++it)
    for (const auto& pl : P) {
      float ms = 0.0f;
      GB_CK(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
      k += 2;
      auto it2 = std::find_if(out.begin(), out.end(),
                              [&](const KernelStat& s) { return s.name == pl.second; });
      if (it2 == out.end()) {
        out.push_back(KernelStat{pl.second});
        it2 = out.end() - 1;
      }
      it2->launches += 1;
      it2->ms += ms;
      it2->bytes += pl.first.bytes;
    }
  for (auto& e : ev) cudaEventDestroy(e);
  out.erase(std::remove_if(out.begin(), out.end(),
                           [](const KernelStat& s) { return s.launches == 0; }),
            out.end());
  return out;
}

void Engine::ensureWalkBuffers() {
  Dev& d = *d_;
  if (d.walkReady) return;
  size_t& B = deviceBytes_;
  d.rowsD.cfv = d.own(alloc<double>(L_.cfvQuads * 4, B));
  for (int tr = 0; tr < 2; ++tr) {
    d.rowsD.reach[tr] = d.own(alloc<double>(L_.reachQuads[tr] * 4, B));
    const Side& opp = t_.side[1 - tr];
    std::vector<double> row(quads(opp.n) * 4, 0.0);
    for (int j = 0; j < opp.n; ++j) row[j] = opp.w[j];
    GB_CK(cudaMemcpy(d.rowsD.reach[tr], row.data(), row.size() * sizeof(double),
                     cudaMemcpyHostToDevice));
    h2d_ += (int64_t)(row.size() * sizeof(double));
  }
  d.walkReady = true;
}

void Engine::walk(int tr, int mode) {
  Dev& d = *d_;
  ensureWalkBuffers();
  const int D = (int)d.fwd[tr].size();
  for (int dd = 0; dd < D; ++dd) {
    const ListRef a = d.fwd[tr][dd];
    if (a.count)
      fwdLevelK<double><<<gridOf(a.count), kThreads, 0, d.stream>>>(
          d.tree, d.rowsD, d.tasks + a.off, a.count, tr, 1);
  }
  for (int dd = D - 1; dd >= 0; --dd) {
    const ListRef b = d.bwd[tr][dd];
    if (b.count)
      bwdLevelK<double><<<gridOf(b.count), kThreads, d.smemD, d.stream>>>(
          d.tree, d.rowsD, d.tasks + b.off, b.count, tr, mode, d.maxN);
  }
  GB_CK(cudaGetLastError());
  GB_CK(cudaStreamSynchronize(d.stream));
}

void Engine::walkFrom(int tr, int mode, int u) {
  Dev& d = *d_;
  const int N = (int)t_.nodes.size();
  if (subEnd_.empty()) {
    // One past each subtree's last id; -1 marks a tree whose subtrees are
    // not contiguous id ranges (walkFrom then walks the whole tree).
    subEnd_.assign(N, 0);
    std::vector<int> size(N, 1);
    bool ok = true;
    for (int v = N - 1; v >= 0; --v) {
      const Node& nd = t_.nodes[v];
      int end = v + 1;
      for (int k = 0; k < nd.nChildren; ++k) {
        const int c = t_.children[nd.childBase + k];
        if (c <= v) ok = false;
        size[v] += size[c];
        end = std::max(end, subEnd_[c]);
      }
      subEnd_[v] = end;
      if (end - v != size[v]) ok = false;
    }
    if (!ok) subEnd_.assign(N, -1);
  }
  // PPS_GB_QUERY_FULL_WALKS (tests): walk the whole tree instead.
  if (u <= 0 || u >= N || subEnd_[u] < 0 || std::getenv("PPS_GB_QUERY_FULL_WALKS")) {
    walk(tr, mode);
    return;
  }
  ensureWalkBuffers();
  // Ancestors of u and the child index toward u at each.
  std::map<int, int> toward;
  for (int c = u, p = t_.nodes[u].parent; p >= 0; c = p, p = t_.nodes[p].parent) {
    const Node& pn = t_.nodes[p];
    for (int k = 0; k < pn.nChildren; ++k)
      if (t_.children[pn.childBase + k] == c) toward[p] = k;
  }
  const int end = subEnd_[u];
  const int D = (int)L_.fwdTasks[tr].size();
  std::vector<int> all;
  std::vector<ListRef> fwd(D), bwd(D);
  for (int dd = 0; dd < D; ++dd) {
    fwd[dd].off = (int)all.size();
    for (int w : L_.fwdTasks[tr][dd]) {
      const int v = (int)((unsigned)w >> 8);
      bool keep = v >= u && v < end;
      if (!keep) {
        auto it = toward.find(v);
        keep = it != toward.end() && ((w & 3) != kTaskChance || ((w >> 2) & 63) == it->second);
      }
      if (keep) all.push_back(w);
    }
    fwd[dd].count = (int)all.size() - fwd[dd].off;
  }
  for (int dd = 0; dd < D; ++dd) {
    bwd[dd].off = (int)all.size();
    for (int w : L_.bwdTasks[tr][dd]) {
      const int v = (int)((unsigned)w >> 8);
      if (v >= u && v < end) all.push_back(w);
    }
    bwd[dd].count = (int)all.size() - bwd[dd].off;
  }
  if (all.empty()) return;
  if (all.size() > d.qCap) {
    if (d.qTasks) cudaFree(d.qTasks);
    d.qTasks = nullptr;
    d.qCap = 0;
    GB_CK(cudaMalloc(&d.qTasks, all.size() * sizeof(int)));
    d.qCap = all.size();
  }
  GB_CK(cudaMemcpyAsync(d.qTasks, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice,
                        d.stream));
  h2d_ += (int64_t)(all.size() * sizeof(int));
  for (int dd = 0; dd < D; ++dd)
    if (fwd[dd].count)
      fwdLevelK<double><<<gridOf(fwd[dd].count), kThreads, 0, d.stream>>>(
          d.tree, d.rowsD, d.qTasks + fwd[dd].off, fwd[dd].count, tr, 1);
  for (int dd = D - 1; dd >= 0; --dd)
    if (bwd[dd].count)
      bwdLevelK<double><<<gridOf(bwd[dd].count), kThreads, d.smemD, d.stream>>>(
          d.tree, d.rowsD, d.qTasks + bwd[dd].off, bwd[dd].count, tr, mode, d.maxN);
  GB_CK(cudaGetLastError());
  GB_CK(cudaStreamSynchronize(d.stream));
}

std::vector<double> Engine::walkCfv(int node, int tr) const {
  const int n = t_.n(node, tr);
  std::vector<double> out(n);
  if (n)
    GB_CK(cudaMemcpy(out.data(), d_->rowsD.cfv + (size_t)L_.rows[node].cfvQ * 4,
                     n * sizeof(double), cudaMemcpyDeviceToHost));
  d2h_ += (int64_t)n * 8;
  return out;
}

std::vector<double> Engine::walkReach(int node, int tr) const {
  const int n = t_.n(node, 1 - tr);
  std::vector<double> out(n);
  if (n)
    GB_CK(cudaMemcpy(out.data(), d_->rowsD.reach[tr] + (size_t)L_.rows[node].reachQ[tr] * 4,
                     n * sizeof(double), cudaMemcpyDeviceToHost));
  d2h_ += (int64_t)n * 8;
  return out;
}

std::vector<float> Engine::denseRows(int which) const {
  std::vector<float> padded(L_.regQuads * 4);
  GB_CK(cudaStreamSynchronize(d_->stream));
  if (!padded.empty())
    GB_CK(cudaMemcpy(padded.data(), which == 0 ? d_->tree.regret : d_->tree.strat,
                     padded.size() * sizeof(float), cudaMemcpyDeviceToHost));
  d2h_ += (int64_t)(padded.size() * sizeof(float));
  std::vector<float> dense;
  dense.reserve((size_t)t_.rowTotal);
  for (int u : t_.decideNodes) {
    const Node& nd = t_.nodes[u];
    const int n = t_.n(u, nd.player);
    const size_t base = (size_t)L_.nodes[u].regQ * 4, stride = quads(n) * 4;
    for (int a = 0; a < nd.na; ++a)
      dense.insert(dense.end(), padded.begin() + base + a * stride,
                   padded.begin() + base + a * stride + n);
  }
  return dense;
}

void Engine::setDenseRows(int which, const std::vector<float>& dense) {
  if ((int64_t)dense.size() != t_.rowTotal)
    throw Error{PPS_GB_E_ARG, "row table size mismatch"};
  std::vector<float> padded(L_.regQuads * 4, 0.0f);
  size_t k = 0;
  for (int u : t_.decideNodes) {
    const Node& nd = t_.nodes[u];
    const int n = t_.n(u, nd.player);
    const size_t base = (size_t)L_.nodes[u].regQ * 4, stride = quads(n) * 4;
    for (int a = 0; a < nd.na; ++a)
      for (int c = 0; c < n; ++c) padded[base + a * stride + c] = dense[k++];
  }
  GB_CK(cudaStreamSynchronize(d_->stream));
  if (!padded.empty())
    GB_CK(cudaMemcpy(which == 0 ? d_->tree.regret : d_->tree.strat, padded.data(),
                     padded.size() * sizeof(float), cudaMemcpyHostToDevice));
  h2d_ += (int64_t)(padded.size() * sizeof(float));
  // New strategy sums carry no low words.
  if (which == 1 && d_->tree.stratLo && L_.regQuads)
    GB_CK(cudaMemset(d_->tree.stratLo, 0, L_.regQuads * 16));
}

namespace {
// Action rows of the decide nodes in dense order: padded device offset,
// dense offset, length.
std::vector<RowRef> actionRowTable(const Tree& t, const HostLayout& L) {
  std::vector<RowRef> tab;
  int64_t dst = 0;
  for (int u : t.decideNodes) {
    const Node& nd = t.nodes[u];
    const int n = t.n(u, nd.player);
    const int64_t base = (int64_t)L.nodes[u].regQ * 4, stride = (int64_t)quads(n) * 4;
    for (int a = 0; a < nd.na; ++a) {
      tab.push_back(RowRef{base + a * stride, dst, n, 0});
      dst += n;
    }
  }
  return tab;
}
}  // namespace

int64_t Engine::actionRows() const {
  int64_t k = 0;
  for (int u : t_.decideNodes) k += t_.nodes[u].na;
  return k;
}

void Engine::packRows(int which, std::vector<uint16_t>& codes,
                      std::vector<float>& scales) const {
  GB_CK(cudaStreamSynchronize(d_->stream));
  gb::packRows(which == 0 ? d_->tree.regret : d_->tree.strat, actionRowTable(t_, L_),
               t_.rowTotal, which == 0, d_->stream, codes, scales);
  d2h_ += (int64_t)(codes.size() * sizeof(uint16_t) + scales.size() * sizeof(float));
}

void Engine::unpackRows(int which, const std::vector<uint16_t>& codes,
                        const std::vector<float>& scales) {
  if ((int64_t)codes.size() != t_.rowTotal || (int64_t)scales.size() != actionRows())
    throw Error{PPS_GB_E_ARG, "compressed row table size mismatch"};
  float* rows = which == 0 ? d_->tree.regret : d_->tree.strat;
  GB_CK(cudaStreamSynchronize(d_->stream));
  if (L_.regQuads)
    GB_CK(cudaMemsetAsync(rows, 0, (size_t)L_.regQuads * 4 * sizeof(float), d_->stream));
  gb::unpackRows(rows, actionRowTable(t_, L_), which == 0, codes, scales, d_->stream);
  h2d_ += (int64_t)(codes.size() * sizeof(uint16_t) + scales.size() * sizeof(float));
  if (which == 1 && d_->tree.stratLo && L_.regQuads)
    GB_CK(cudaMemsetAsync(d_->tree.stratLo, 0, L_.regQuads * 16, d_->stream));
}

std::vector<float> Engine::nodeRows(int which, int node) const {
  const Node& nd = t_.nodes[node];
  const int n = t_.n(node, nd.player);
  const size_t stride = quads(n) * 4;
  std::vector<float> padded(stride * nd.na), out((size_t)n * nd.na);
  GB_CK(cudaStreamSynchronize(d_->stream));
  if (!padded.empty())
    GB_CK(cudaMemcpy(padded.data(),
                     (which == 0 ? d_->tree.regret : d_->tree.strat) +
                         (size_t)L_.nodes[node].regQ * 4,
                     padded.size() * sizeof(float), cudaMemcpyDeviceToHost));
  d2h_ += (int64_t)(padded.size() * sizeof(float));
  for (int a = 0; a < nd.na; ++a)
    std::copy(padded.begin() + a * stride, padded.begin() + a * stride + n,
              out.begin() + (size_t)a * n);
  return out;
}

}  // namespace gb
}  // namespace pps
