// Device engine (see engine.h): uploads the layout, captures one DCFR
// iteration (two alternating half-steps plus the counter bump, the
// reference's captureGraph, cuda/gpu_cfr.cu:844-868) as a CUDA graph, and
// runs the FP64 walks.
#include "engine.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "kernels.cuh"
#include "leaf_kernel.cuh"
#include "pps_gb.h"

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

namespace {

template <typename V>
V* upload(const std::vector<V>& v, size_t& bytes) {
  if (v.empty()) return nullptr;
  V* p = nullptr;
  GB_CK(cudaMalloc(&p, v.size() * sizeof(V)));
  GB_CK(cudaMemcpy(p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice));
  bytes += v.size() * sizeof(V);
  return p;
}

template <typename V>
V* alloc(size_t count, size_t& bytes) {
  V* p = nullptr;
  GB_CK(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(V)));
  bytes += std::max<size_t>(count, 1) * sizeof(V);
  return p;
}

}  // namespace

struct Engine::Dev {
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void*> owned;
  DevTree tree{};
  DevRows<float> rowsF{};
  DevRows<double> rowsD{};
  float* coef = nullptr;
  size_t coefCap = 0;  // iterations the coef table holds
  int* counter = nullptr;
  int* lists = nullptr;
  std::vector<ListRef> fwdDecide[2], fwdChance[2], bwd;
  LeafPlan leaf;       // fused leaf-street plan (empty if not applicable)
  bool walkReady = false;

  template <typename P>
  P* own(P* p) {
    owned.push_back((void*)p);
    return p;
  }
};

Engine::Engine(const Tree& t, HostLayout&& layout)
    : t_(t), L_(std::move(layout)), d_(new Dev()) {
  Dev& d = *d_;
  size_t& B = deviceBytes_;
  GB_CK(cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking));
  d.tree.nodes = d.own(upload(L_.nodes, B));
  d.tree.rows = d.own(upload(L_.rows, B));
  d.tree.termVal = d.own(upload(L_.termVal, B));
  d.tree.children = d.own(upload(L_.children, B));
  d.tree.states = d.own(upload(L_.states, B));
  d.tree.poolU8 = d.own(upload(L_.poolU8, B));
  d.tree.poolU16 = d.own(upload(L_.poolU16, B));
  d.tree.poolI16 = d.own(upload(L_.poolI16, B));
  d.tree.poolSd = d.own(upload(L_.poolSd, B));
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

  // Root reach rows: the opponent's range weights (padding zero).
  for (int tr = 0; tr < 2; ++tr) {
    const Side& opp = t_.side[1 - tr];
    std::vector<float> row(quads(opp.n) * 4, 0.0f);
    for (int j = 0; j < opp.n; ++j) row[j] = (float)opp.w[j];
    GB_CK(cudaMemcpy(d.rowsF.reach[tr], row.data(), row.size() * sizeof(float),
                     cudaMemcpyHostToDevice));
  }

  // Work lists, concatenated.
  std::vector<int> all;
  auto addList = [&](const std::vector<int>& v) {
    ListRef r{(int)all.size(), (int)v.size()};
    all.insert(all.end(), v.begin(), v.end());
    return r;
  };
  const int D = (int)L_.bwd.size();
  for (int tr = 0; tr < 2; ++tr)
    for (int dd = 0; dd < D; ++dd) {
      d.fwdDecide[tr].push_back(addList(L_.fwdDecide[tr][dd]));
      d.fwdChance[tr].push_back(addList(L_.fwdChance[tr][dd]));
    }
  for (int dd = 0; dd < D; ++dd) d.bwd.push_back(addList(L_.bwd[dd]));
  d.leaf = planLeaf(t_, L_, all);
  d.lists = d.own(upload(all, B));
  if (d.leaf.ok) d.leaf.scratch = d.own(alloc<float>(d.leaf.scratchFloats, B));

  GB_CK(cudaFuncSetAttribute(bwdK<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bwdSmemBytes<float>(L_.maxN)));
  GB_CK(cudaFuncSetAttribute(bwdK<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bwdSmemBytes<double>(L_.maxN)));
  if (d.leaf.ok)
    GB_CK(cudaFuncSetAttribute(leafK, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)d.leaf.smemBytes));
  engineKind_ = d.leaf.ok ? 1 : 0;
  zeroRows();
}

Engine::~Engine() {
  if (!d_) return;
  if (d_->exec) cudaGraphExecDestroy(d_->exec);
  if (d_->graph) cudaGraphDestroy(d_->graph);
  if (d_->stream) cudaStreamSynchronize(d_->stream);
  for (void* p : d_->owned) cudaFree(p);
  if (d_->stream) cudaStreamDestroy(d_->stream);
}

void* Engine::stream() const { return (void*)d_->stream; }

void Engine::zeroRows() {
  Dev& d = *d_;
  GB_CK(cudaMemsetAsync(d.tree.regret, 0, L_.regQuads * 16, d.stream));
  GB_CK(cudaMemsetAsync(d.tree.strat, 0, L_.regQuads * 16, d.stream));
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
  setCounter(counter);
}

void Engine::setCounter(int counter) {
  Dev& d = *d_;
  GB_CK(cudaMemcpyAsync(d.counter, &counter, sizeof(int), cudaMemcpyHostToDevice,
                        d.stream));
  GB_CK(cudaStreamSynchronize(d.stream));
}

namespace {

template <typename T>
int halfStep(Engine::Dev& d, const DevRows<T>& rows, int D, int tr, int mode,
             int sigSrc, size_t smem) {
  int launches = 0;
  auto grid = [](int count) { return (unsigned)std::min(count, 65535); };
  for (int dd = 0; dd < D; ++dd) {
    const ListRef a = d.fwdDecide[tr][dd], c = d.fwdChance[tr][dd];
    if (a.count) {
      fwdDecideK<T><<<grid(a.count), kThreads, 0, d.stream>>>(
          d.tree, rows, d.lists + a.off, a.count, tr, sigSrc);
      ++launches;
    }
    if (c.count) {
      fwdChanceK<T><<<grid(c.count), kThreads, 0, d.stream>>>(
          d.tree, rows, d.lists + c.off, c.count, tr);
      ++launches;
    }
  }
  for (int dd = D - 1; dd >= 0; --dd) {
    const ListRef b = d.bwd[dd];
    if (!b.count) continue;
    bwdK<T><<<grid(b.count), kThreads, smem, d.stream>>>(d.tree, rows, d.lists + b.off,
                                                          b.count, tr, mode);
    ++launches;
  }
  GB_CK(cudaGetLastError());
  return launches;
}

}  // namespace

// Fused variant of one half-step: depth-level launches above the leaf
// street, one persistent launch for every leaf subtree, depth-level below.
static int halfStepLeaf(Engine::Dev& d, int D, int tr, size_t smem) {
  int launches = 0;
  auto grid = [](int count) { return (unsigned)std::min(count, 65535); };
  const LeafPlan& lp = d.leaf;
  for (int dd = 0; dd < lp.rootDepthMin; ++dd) {
    const ListRef a = d.fwdDecide[tr][dd], c = d.fwdChance[tr][dd];
    if (a.count) {
      fwdDecideK<float><<<grid(a.count), kThreads, 0, d.stream>>>(
          d.tree, d.rowsF, d.lists + a.off, a.count, tr, 0);
      ++launches;
    }
    if (c.count) {
      fwdChanceK<float><<<grid(c.count), kThreads, 0, d.stream>>>(
          d.tree, d.rowsF, d.lists + c.off, c.count, tr);
      ++launches;
    }
  }
  launches += launchLeaf(lp, d.tree, d.rowsF, d.lists, tr, d.stream);
  for (int dd = lp.rootDepthMin - 1; dd >= 0; --dd) {
    const ListRef b = lp.upperBwd[dd];
    if (!b.count) continue;
    bwdK<float><<<grid(b.count), kThreads, smem, d.stream>>>(
        d.tree, d.rowsF, d.lists + b.off, b.count, tr, kModeCFR);
    ++launches;
  }
  GB_CK(cudaGetLastError());
  return launches;
}

void Engine::capture() {
  Dev& d = *d_;
  if (d.exec) {
    cudaGraphExecDestroy(d.exec);
    cudaGraphDestroy(d.graph);
    d.exec = nullptr;
    d.graph = nullptr;
  }
  const int D = (int)L_.bwd.size();
  const size_t smem = bwdSmemBytes<float>(L_.maxN);
  GB_CK(cudaStreamBeginCapture(d.stream, cudaStreamCaptureModeThreadLocal));
  int launches = 0;
  try {
    for (int tr = 0; tr < 2; ++tr)
      launches += engineKind_ == 1 && d.leaf.ok
                      ? halfStepLeaf(d, D, tr, smem)
                      : halfStep<float>(d, d.rowsF, D, tr, kModeCFR, 0, smem);
    advanceCounterK<<<1, 32, 0, d.stream>>>(d.counter);
    ++launches;
  } catch (...) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(d.stream, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  GB_CK(cudaStreamEndCapture(d.stream, &d.graph));
  GB_CK(cudaGraphInstantiate(&d.exec, d.graph, 0));
  launchesPerIter_ = launches;
}

void Engine::setEngineKind(int kind) {
  const int k = kind == 1 && d_->leaf.ok ? 1 : 0;
  if (k == engineKind_ && d_->exec) return;
  engineKind_ = k;
  capture();
}

void Engine::iterate(int n) {
  Dev& d = *d_;
  if (!d.exec) capture();
  for (int i = 0; i < n; ++i) GB_CK(cudaGraphLaunch(d.exec, d.stream));
}

void Engine::sync() { GB_CK(cudaStreamSynchronize(d_->stream)); }

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
  }
  d.walkReady = true;
}

void Engine::walk(int tr, int mode) {
  Dev& d = *d_;
  ensureWalkBuffers();
  halfStep<double>(d, d.rowsD, (int)L_.bwd.size(), tr, mode, 1,
                   bwdSmemBytes<double>(L_.maxN));
  GB_CK(cudaStreamSynchronize(d.stream));
}

std::vector<double> Engine::walkCfv(int node, int tr) const {
  const int n = t_.n(node, tr);
  std::vector<double> out(n);
  if (n)
    GB_CK(cudaMemcpy(out.data(), d_->rowsD.cfv + (size_t)L_.rows[node].cfvQ * 4,
                     n * sizeof(double), cudaMemcpyDeviceToHost));
  return out;
}

std::vector<double> Engine::walkReach(int node, int tr) const {
  const int n = t_.n(node, 1 - tr);
  std::vector<double> out(n);
  if (n)
    GB_CK(cudaMemcpy(out.data(), d_->rowsD.reach[tr] + (size_t)L_.rows[node].reachQ[tr] * 4,
                     n * sizeof(double), cudaMemcpyDeviceToHost));
  return out;
}

std::vector<float> Engine::denseRows(int which) const {
  std::vector<float> padded(L_.regQuads * 4);
  GB_CK(cudaStreamSynchronize(d_->stream));
  if (!padded.empty())
    GB_CK(cudaMemcpy(padded.data(), which == 0 ? d_->tree.regret : d_->tree.strat,
                     padded.size() * sizeof(float), cudaMemcpyDeviceToHost));
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
  for (int a = 0; a < nd.na; ++a)
    std::copy(padded.begin() + a * stride, padded.begin() + a * stride + n,
              out.begin() + (size_t)a * n);
  return out;
}

}  // namespace gb
}  // namespace pps
