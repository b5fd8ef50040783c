// No-allocation DCFR solve over caller-owned rows (pps_gb_solve_noalloc in
// include/pps_gb.h).
//
// For callers that cannot call cudaMalloc (their device memory belongs to
// another allocator, or they must avoid cudaMalloc's implicit
// synchronization): the caller passes its regret and strategy rows; every
// other device buffer of the solve - tree tables, task lists, reach and
// value rows, the schedule - is carved out of gNoAllocScratch, one
// file-scope static device array of PPS_GB_NOALLOC_SCRATCH_BYTES. Nothing
// here allocates device memory.
//
// Host code never dereferences or passes gNoAllocScratch itself: on the
// host that name is a stand-in, not a device address. Its device address is
// looked up once per device with cudaGetSymbolAddress (with that device
// current) and kept, keyed on the device's current context: after a
// cudaDeviceReset the next call finds a new context and looks the address
// up again. The first call on a device (and the first after a reset) does
// this set-up, so it should come before any stream capture. All calls share
// the array and leave their contents in it; every buffer a call reads is
// written by that call first (or cleared), and calls that overlap on a GPU
// race on it.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "compiler.h"
#include "kernels.cuh"
#include "layout.h"
#include "noalloc.h"
#include "plan.cuh"
#include "pps_gb.h"
#include "solver.h"

namespace pps {
namespace gb {

static __device__ __align__(256) unsigned char gNoAllocScratch[PPS_GB_NOALLOC_SCRATCH_BYTES];

namespace {

#define NA_CK(call)                                                          \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      throw Error{PPS_GB_E_CUDA, std::string("CUDA error: ") +               \
                                     cudaGetErrorString(e_) + " (" #call ")"}; \
  } while (0)

constexpr int kMaxDevices = 128;
std::mutex gSetupMutex;
struct ScratchAddr {
  CUcontext ctx = nullptr;      // the context the address belongs to
  unsigned char* ptr = nullptr; // gNoAllocScratch's device address there
};
ScratchAddr gScratchOnDevice[kMaxDevices];

// The driver's cuCtxGetCurrent, looked up through the runtime (the library
// does not link the driver library directly).
decltype(&::cuCtxGetCurrent) ctxGetCurrent() {
  static const decltype(&::cuCtxGetCurrent) fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<decltype(&::cuCtxGetCurrent)>(p);
  }();
  return fn;
}

CUcontext currentContext() {
  const auto get = ctxGetCurrent();
  if (!get) throw Error{PPS_GB_E_CUDA, "driver entry point missing: cuCtxGetCurrent"};
  CUcontext ctx = nullptr;
  if (get(&ctx) != CUDA_SUCCESS) throw Error{PPS_GB_E_CUDA, "cuCtxGetCurrent failed"};
  return ctx;
}

// Device address of gNoAllocScratch on the current device, looked up once
// per device and context (cudaGetSymbolAddress also makes the device's
// primary context current on the first call).
unsigned char* scratchBase() {
  int dev = 0;
  NA_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) throw Error{PPS_GB_E_CUDA, "device index out of range"};
  const CUcontext ctx = currentContext();
  std::lock_guard<std::mutex> lock(gSetupMutex);
  ScratchAddr& a = gScratchOnDevice[dev];
  if (!a.ptr || !ctx || a.ctx != ctx) {
    void* p = nullptr;
    NA_CK(cudaGetSymbolAddress(&p, gNoAllocScratch));
    a.ptr = static_cast<unsigned char*>(p);
    a.ctx = currentContext();
  }
  return a.ptr;
}

// Per decide node: where its rows sit in the caller's dense layout and in
// the padded scratch layout.
struct RowMap {
  int dense;     // first dense entry
  uint32_t padQ; // first padded quad
  int na;
  int n;
};

// Copies rows between the caller's dense layout and the padded layout the
// kernels use (toPadded: dense -> padded); padding lanes are left as set.
__global__ void repackK(const RowMap* __restrict__ map, int count, const float* src, float* dst,
                        int toPadded) {
  for (int k = blockIdx.x; k < count; k += gridDim.x) {
    const RowMap m = map[k];
    const int stride = quadsOf(m.n) * 4;
    for (int e = threadIdx.x; e < m.na * m.n; e += blockDim.x) {
      const int a = e / m.n, c = e - a * m.n;
      const size_t pad = (size_t)m.padQ * 4 + (size_t)a * stride + c;
      const size_t dense = (size_t)m.dense + e;
      if (toPadded) dst[pad] = src[dense];
      else dst[dense] = src[pad];
    }
  }
}

struct Arena {
  size_t used = 0;
  size_t take(size_t bytes) {
    const size_t off = used;
    used += (bytes + 255) / 256 * 256;
    return off;
  }
};

}  // namespace

int64_t noallocSolve(const gpu::PostflopSpot& spot, const pf::BetConfig& cfg, float* dRegret,
                     float* dStrat, int64_t rowCapacity, int firstIteration, int iterations,
                     cudaStream_t stream, int64_t* needRows) {
  if (firstIteration < 0 || iterations < 0 ||
      (int64_t)firstIteration + iterations > (int64_t)INT_MAX)
    throw Error{PPS_GB_E_ARG, "bad iteration range"};
  // An error left pending by the caller's own earlier CUDA work is reported
  // as such (and left pending), not as a failure of this solve.
  {
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess)
      throw Error{PPS_GB_E_CUDA, std::string("a CUDA error was pending before this call: ") +
                                     cudaGetErrorString(pending)};
  }
  gpu::StreetBetConfigs cfgs;
  cfgs.street[0] = cfgs.street[1] = cfgs.street[2] = cfg;
  const Tree t = compileTree(spot, cfgs, false);
  if (t.empty) throw Error{PPS_GB_E_STATE, "solver compiled to empty ranges"};
  if (needRows) *needRows = t.rowTotal;  // also on the errors below: a size query
  if (t.rowTotal > (int64_t)INT_MAX) throw Error{PPS_GB_E_BUDGET, "row table too large"};
  if (t.rowTotal > 0 && (!dRegret || !dStrat)) throw Error{PPS_GB_E_ARG, "null row buffer"};
  if (rowCapacity < t.rowTotal)
    throw Error{PPS_GB_E_ARG, "row buffers hold " + std::to_string(rowCapacity) +
                                  " floats; the spot needs " + std::to_string(t.rowTotal)};
  const HostLayout L = buildLayout(t);

  // Task lists of the default iteration (the engine's kind 0: forward
  // levels, then per backward level the showdown groups, the fold groups and
  // the interior tasks) and the row map.
  std::vector<int> tasks;
  const int D = (int)L.bwdTasks[0].size();
  std::vector<std::pair<int, int>> fwd[2], sdG, fdG, inner[2];
  auto add = [&](const std::vector<int>& v) {
    const std::pair<int, int> r{(int)tasks.size(), (int)v.size()};
    tasks.insert(tasks.end(), v.begin(), v.end());
    return r;
  };
  for (int d = 0; d < D; ++d) {
    sdG.push_back(add(L.sdGroupTasks[d]));
    fdG.push_back(add(L.fdGroupTasks[d]));
    for (int tr = 0; tr < 2; ++tr) {
      fwd[tr].push_back(add(L.fwdTasks[tr][d]));
      inner[tr].push_back(add(L.innerTasks[tr][d]));
    }
  }
  std::vector<RowMap> rowMap;
  int dense = 0;
  for (int u : t.decideNodes) {
    const Node& nd = t.nodes[u];
    const int n = t.n(u, nd.player);
    rowMap.push_back({dense, L.nodes[u].regQ, nd.na, n});
    dense += nd.na * n;
  }
  // The schedule window of this call only: the device counter starts at 0
  // and entry k holds the coefficients of absolute iteration
  // firstIteration + k (the DCFR coefficients depend on the absolute index
  // alone), so a continuation far into a solve costs no more than its own
  // iterations.
  std::vector<float> coef((size_t)iterations * 3 + 3, 0.0f);
  Schedule sched;
  for (int k = 0; k < iterations; ++k) {
    double c[3];
    sched.coefs(firstIteration + k, firstIteration + iterations, c);
    for (int j = 0; j < 3; ++j) coef[(size_t)k * 3 + j] = (float)c[j];
  }
  const int counterStart = 0;
  std::vector<float> rootReach[2];
  for (int tr = 0; tr < 2; ++tr) {
    const Side& opp = t.side[1 - tr];
    rootReach[tr].assign(quads(opp.n) * 4, 0.0f);
    for (int j = 0; j < opp.n; ++j) rootReach[tr][j] = (float)opp.w[j];
  }

  // Scratch plan.
  Arena A;
  auto bytesOf = [](const auto& v) { return v.size() * sizeof(v[0]); };
  const size_t oNodes = A.take(bytesOf(L.nodes)), oRows = A.take(bytesOf(L.rows)),
               oTerm = A.take(bytesOf(L.termVal)), oKids = A.take(bytesOf(L.children)),
               oStates = A.take(bytesOf(L.states)), oU8 = A.take(bytesOf(L.poolU8)),
               oU16 = A.take(bytesOf(L.poolU16)), oI16 = A.take(bytesOf(L.poolI16)),
               oSd = A.take(bytesOf(L.poolSd)), oTasks = A.take(bytesOf(tasks)),
               oGroups = A.take(bytesOf(L.groupRecs)),
               oMap = A.take(bytesOf(rowMap)), oReg = A.take(L.regQuads * 16),
               oStr = A.take(L.regQuads * 16), oCfv = A.take(L.cfvQuads * 16),
               oReach0 = A.take(L.reachQuads[0] * 16), oReach1 = A.take(L.reachQuads[1] * 16),
               oCoef = A.take(bytesOf(coef)), oCounter = A.take(sizeof(int));
  if (A.used > (size_t)PPS_GB_NOALLOC_SCRATCH_BYTES)
    throw Error{PPS_GB_E_BUDGET,
                "spot and iteration window need " + std::to_string(A.used) +
                    " bytes of scratch (of which the schedule of " + std::to_string(iterations) +
                    " iterations takes " + std::to_string(bytesOf(coef)) +
                    "); the static scratch holds " +
                    std::to_string((size_t)PPS_GB_NOALLOC_SCRATCH_BYTES)};

  unsigned char* base = scratchBase();
  auto put = [&](size_t off, const auto& v) {
    if (!v.empty())
      NA_CK(cudaMemcpyAsync(base + off, v.data(), bytesOf(v), cudaMemcpyHostToDevice, stream));
  };
  put(oNodes, L.nodes);
  put(oRows, L.rows);
  put(oTerm, L.termVal);
  put(oKids, L.children);
  put(oStates, L.states);
  put(oU8, L.poolU8);
  put(oU16, L.poolU16);
  put(oI16, L.poolI16);
  put(oSd, L.poolSd);
  put(oTasks, tasks);
  put(oGroups, L.groupRecs);
  put(oMap, rowMap);
  put(oCoef, coef);
  put(oReach0, rootReach[0]);
  put(oReach1, rootReach[1]);
  NA_CK(cudaMemcpyAsync(base + oCounter, &counterStart, sizeof(int), cudaMemcpyHostToDevice,
                        stream));
  // Padded rows start from zero (padding lanes must stay zero), then take
  // the caller's values.
  NA_CK(cudaMemsetAsync(base + oReg, 0, L.regQuads * 16, stream));
  NA_CK(cudaMemsetAsync(base + oStr, 0, L.regQuads * 16, stream));
  float* reg = reinterpret_cast<float*>(base + oReg);
  float* str = reinterpret_cast<float*>(base + oStr);
  const RowMap* map = reinterpret_cast<const RowMap*>(base + oMap);
  // A spot without decide nodes (a zero behind-stack makes the root a
  // showdown or chance node) has no rows to move.
  const int nMap = (int)rowMap.size();
  const unsigned gMap = (unsigned)std::min(nMap, 1 << 20);
  if (nMap > 0) {
    repackK<<<gMap, 128, 0, stream>>>(map, nMap, dRegret, reg, 1);
    repackK<<<gMap, 128, 0, stream>>>(map, nMap, dStrat, str, 1);
  }

  DevTree tree{};
  tree.nodes = reinterpret_cast<const NodeDev*>(base + oNodes);
  tree.rows = reinterpret_cast<const RowDev*>(base + oRows);
  tree.termVal = reinterpret_cast<const float*>(base + oTerm);
  tree.children = reinterpret_cast<const int*>(base + oKids);
  tree.states = reinterpret_cast<const StateDev*>(base + oStates);
  tree.poolU8 = base + oU8;
  tree.poolU16 = reinterpret_cast<const uint16_t*>(base + oU16);
  tree.poolI16 = reinterpret_cast<const int16_t*>(base + oI16);
  tree.poolSd = reinterpret_cast<const ShowdownInfo*>(base + oSd);
  tree.regret = reg;
  tree.strat = str;
  tree.coef = reinterpret_cast<const float*>(base + oCoef);
  int* counter = reinterpret_cast<int*>(base + oCounter);
  tree.counter = counter;
  DevRows<float> rows{};
  rows.reach[0] = reinterpret_cast<float*>(base + oReach0);
  rows.reach[1] = reinterpret_cast<float*>(base + oReach1);
  rows.cfv = reinterpret_cast<float*>(base + oCfv);
  const int* dTasks = reinterpret_cast<const int*>(base + oTasks);

  const GroupRec* groups = reinterpret_cast<const GroupRec*>(base + oGroups);
  const size_t smemSd = sdGroupSmem(L.maxN), smemFd = fdGroupSmem(L.maxN);
  raiseGroupSmem(L.maxN);
  auto grid = [](int count) { return (unsigned)std::min(count, 1 << 20); };
  for (int it = 0; it < iterations; ++it) {
    for (int tr = 0; tr < 2; ++tr) {
      for (int d = 0; d < D; ++d)
        if (fwd[tr][d].second)
          fwdLevelK<float><<<grid(fwd[tr][d].second), kThreads, 0, stream>>>(
              tree, rows, dTasks + fwd[tr][d].first, fwd[tr][d].second, tr, 0);
      for (int d = D - 1; d >= 0; --d) {
        if (sdG[d].second)
          launchSdGroups(grid(sdG[d].second), smemSd, stream, tree, rows, groups,
                         dTasks + sdG[d].first, sdG[d].second, tr, L.maxN);
        if (fdG[d].second)
          launchFdGroups(grid(fdG[d].second), smemFd, stream, tree, rows, groups,
                         dTasks + fdG[d].first, fdG[d].second, tr, L.maxN);
        if (inner[tr][d].second)
          bwdInteriorK<float><<<grid(inner[tr][d].second), kThreads, 0, stream>>>(
              tree, rows, dTasks + inner[tr][d].first, inner[tr][d].second, tr, kModeCFR);
      }
    }
    advanceCounterK<<<1, 32, 0, stream>>>(counter, 1);
    NA_CK(cudaGetLastError());
  }
  if (nMap > 0) {
    repackK<<<gMap, 128, 0, stream>>>(map, nMap, reg, dRegret, 0);
    repackK<<<gMap, 128, 0, stream>>>(map, nMap, str, dStrat, 0);
  }
  NA_CK(cudaGetLastError());
  NA_CK(cudaStreamSynchronize(stream));
  return t.rowTotal;
}

}  // namespace gb
}  // namespace pps
