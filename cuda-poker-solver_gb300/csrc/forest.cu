// Forest (see forest.h): shared device pools, relocation of spot layouts,
// the all-spots iteration graph and the FP64 check walks.
#include "forest.h"

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <type_traits>

#include "kernels.cuh"
#include "plan.cuh"
#include "tune.h"
#include "pps_gb.h"

namespace pps {
namespace gb {

double pairMassOf(const Tree& t) {
  const Side& s0 = t.side[0];
  const Side& s1 = t.side[1];
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

namespace {

// Pools. A region is one index space (node ids, row quads, ...); arrays
// are the device buffers indexed by it.
enum Region { rNode, rChild, rState, rU8, rU16, rI16, rSd, rReg, rCfv, rReach0, rReach1, rW,
              rGroup, rRec, kRegions };
// Allocation granule per region, in entries: every range starts on a
// 16-byte boundary (u16 tables are staged with 16-byte loads; decide
// records are addressed in 16-byte units).
constexpr size_t kGranule[kRegions] = {1, 4, 1, 16, 8, 8, 1, 1, 1, 1, 1, 2, 1, 4};

enum Array { aNodes, aRows, aTerm, aChild, aState, aU8, aU16, aI16, aSd, aReg, aStr, aCfvF,
             aCfvD, aReachF0, aReachD0, aReachF1, aReachD1, aW, aGroups, aRecs, kArrays };
struct ArrayDef {
  Region region;
  size_t entryBytes;
};
const ArrayDef kArray[kArrays] = {
    {rNode, sizeof(NodeDev)}, {rNode, sizeof(RowDev)}, {rNode, 8 * sizeof(float)},
    {rChild, sizeof(int)},    {rState, sizeof(StateDev)}, {rU8, 1},
    {rU16, 2},                {rI16, 2},                  {rSd, sizeof(ShowdownInfo)},
    {rReg, 16},               {rReg, 16},                 {rCfv, 16},
    {rCfv, 32},               {rReach0, 16},              {rReach0, 32},
    {rReach1, 16},            {rReach1, 32},              {rW, 8},
    {rGroup, 2 * sizeof(GroupRec)}, {rRec, sizeof(uint32_t)}};

size_t roundUp(size_t n, size_t g) { return (n + g - 1) / g * g; }

void regionSizes(const Tree& t, const HostLayout& L, size_t out[kRegions]) {
  out[rNode] = L.nodes.size();
  out[rChild] = L.children.size();
  out[rState] = L.states.size();
  out[rU8] = L.poolU8.size();
  out[rU16] = L.poolU16.size();
  out[rI16] = L.poolI16.size();
  out[rSd] = L.poolSd.size();
  out[rReg] = L.regQuads;
  out[rCfv] = L.cfvQuads;
  out[rReach0] = L.reachQuads[0];
  out[rReach1] = L.reachQuads[1];
  out[rW] = (size_t)t.side[0].n + (size_t)t.side[1].n;  // w0 then w1
  out[rGroup] = L.groups.size();
  out[rRec] = L.recPool.size();
}

size_t footprintOf(const Tree& t, const HostLayout& L) {
  size_t sz[kRegions];
  regionSizes(t, L, sz);
  size_t bytes = 0;
  for (int a = 0; a < kArrays; ++a) {
    const Region r = kArray[a].region;
    bytes += roundUp(sz[r], kGranule[r]) * kArray[a].entryBytes;
  }
  return bytes;
}

// First-fit range allocator over one index space: holes by offset, a bump
// pointer at the top; ranges are multiples of the region's granule.
class RangeAlloc {
 public:
  size_t alloc(size_t n, size_t g) {
    n = roundUp(n, g);
    if (n == 0) return 0;
    for (auto it = holes_.begin(); it != holes_.end(); ++it) {
      if (it->second < n) continue;
      const size_t off = it->first, rest = it->second - n;
      holes_.erase(it);
      if (rest) holes_[off + n] = rest;
      return off;
    }
    const size_t off = top_;
    top_ += n;
    return off;
  }
  void release(size_t off, size_t n, size_t g) {
    n = roundUp(n, g);
    if (n == 0) return;
    auto next = holes_.lower_bound(off);
    if (next != holes_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        off = prev->first;
        n += prev->second;
        holes_.erase(prev);
      }
    }
    if (next != holes_.end() && off + n == next->first) {
      n += next->second;
      holes_.erase(next);
    }
    if (off + n == top_) {
      top_ = off;
      // A hole may now end at the new top.
      if (!holes_.empty()) {
        auto last = std::prev(holes_.end());
        if (last->first + last->second == top_) {
          top_ = last->first;
          holes_.erase(last);
        }
      }
    } else {
      holes_[off] = n;
    }
  }
  size_t top() const { return top_; }

 private:
  std::map<size_t, size_t> holes_;
  size_t top_ = 0;
};

// Driver virtual-memory entry points, looked up through the runtime (the
// library does not link the driver library directly).
struct DriverVmm {
  decltype(&::cuMemGetAllocationGranularity) granularity = nullptr;
  decltype(&::cuMemAddressReserve) reserve = nullptr;
  decltype(&::cuMemAddressFree) addressFree = nullptr;
  decltype(&::cuMemCreate) create = nullptr;
  decltype(&::cuMemRelease) release = nullptr;
  decltype(&::cuMemMap) map = nullptr;
  decltype(&::cuMemUnmap) unmap = nullptr;
  decltype(&::cuMemSetAccess) setAccess = nullptr;
};

const DriverVmm& vmm() {
  static const DriverVmm v = [] {
    DriverVmm d;
    auto get = [](const char* name, auto& fn) {
      cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
      void* p = nullptr;
      GB_CK(cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q));
      if (q != cudaDriverEntryPointSuccess || !p)
        throw Error{PPS_GB_E_CUDA, std::string("driver entry point missing: ") + name};
      fn = reinterpret_cast<std::remove_reference_t<decltype(fn)>>(p);
    };
    get("cuMemGetAllocationGranularity", d.granularity);
    get("cuMemAddressReserve", d.reserve);
    get("cuMemAddressFree", d.addressFree);
    get("cuMemCreate", d.create);
    get("cuMemRelease", d.release);
    get("cuMemMap", d.map);
    get("cuMemUnmap", d.unmap);
    get("cuMemSetAccess", d.setAccess);
    return d;
  }();
  return v;
}

void cuCheck(CUresult r, const char* what) {
  if (r != CUDA_SUCCESS)
    throw Error{r == CUDA_ERROR_OUT_OF_MEMORY ? PPS_GB_E_MEMORY : PPS_GB_E_CUDA,
                std::string("CUDA driver error ") + std::to_string((int)r) + " (" + what + ")"};
}

// A device array at a fixed virtual address range: physical memory is
// mapped at its end as the array grows and unmapped as it shrinks, so the
// base pointer never moves and growing copies nothing.
struct VmArray {
  CUdeviceptr base = 0;
  size_t reserved = 0, mapped = 0;
  std::vector<std::pair<CUmemGenericAllocationHandle, size_t>> chunks;  // address order
};

struct RootInfo {
  uint32_t cfvQ;  // root value row (quads)
  int wOff;       // traverser weights in the weight pool
  int n;          // traverser combos
  int pad;
};

// Root value of each listed spot: sum_j w[j] * cfv[j] in a fixed order
// (one CTA per spot, strided partial sums, then a tree reduction).
template <typename T>
__global__ void __launch_bounds__(128) rootValueK(const T* __restrict__ cfv,
                                                  const double* __restrict__ w,
                                                  const RootInfo* __restrict__ info,
                                                  double* __restrict__ out) {
  __shared__ double part[128];
  const RootInfo r = info[blockIdx.x];
  double acc = 0.0;
  for (int j = threadIdx.x; j < r.n; j += blockDim.x)
    acc += w[r.wOff + j] * (double)cfv[(size_t)r.cfvQ * 4 + j];
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 64; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = part[0];
}

template <typename V>
void ensureBuf(V*& p, size_t& cap, size_t need) {
  if (need <= cap) return;
  const size_t n = std::max(need, cap + cap / 2);
  if (p) GB_CK(cudaFree(p));
  p = nullptr;
  GB_CK(cudaMalloc(&p, n * sizeof(V)));
  cap = n;
}

}  // namespace

std::unique_ptr<CompiledSpot> compileSpot(const gpu::PostflopSpot& spot,
                                          const gpu::StreetBetConfigs& cfgs, bool perStreet) {
  std::unique_ptr<CompiledSpot> s(new CompiledSpot);
  s->tree = compileTree(spot, cfgs, perStreet);
  if (!s->tree.empty) {
    s->layout = buildLayout(s->tree);
    s->pairMass = pairMassOf(s->tree);
    s->bytes = footprintOf(s->tree, s->layout);
  }
  return s;
}

struct SlotRec {
  std::unique_ptr<CompiledSpot> spot;
  size_t off[kRegions] = {};
  size_t size[kRegions] = {};
  int iters = 0;
  uint32_t rootCfvQ = 0, rootRegQ = 0;
  int depth = 0;
  // Task lists per traverser and depth, node ids relocated; backward lists
  // keep the layout's order (terminal tasks first). The iteration uses the
  // terminal group lists (group ids relocated) and the interior lists.
  std::vector<std::vector<int>> fwd[2], bwd[2], inner[2];
  std::vector<std::vector<int>> sdG, fdG;
  std::vector<std::vector<uint32_t>> bCh[2], fCh[2];  // chance record offsets, relocated
  std::vector<std::vector<uint32_t>> bRec[2], fRec[2];  // record offsets, relocated
  // fRec / fCh are per forward level (layout.h); termAfter[tr][d]: the
  // forward level after which depth d's terminal reach rows are written.
  std::vector<int> termAfter[2];
  // Backward per level (layout.h): records, chance records, and the
  // terminal depths each level reads.
  std::vector<std::vector<uint32_t>> bRecH[2], bChH[2];
  std::vector<uint64_t> bNeed[2];
};

struct Forest::Dev {
  cudaStream_t stream = nullptr;
  Branches br;
  cudaEvent_t evA = nullptr, evB = nullptr;  // around the last iterate()
  bool timed = false;
  RangeAlloc regions[kRegions];
  VmArray va[kArrays];
  void* arr[kArrays] = {};  // va[a].base
  int device = 0;
  size_t gran = 0;          // physical mapping granularity
  float* coef = nullptr;
  int coefEntries = 0;
  int* counter = nullptr;
  size_t counterCap = 0;
  int* err = nullptr;  // device error word (a bounded wait gave up)
  std::vector<int> freeSlots;
  int nextSlot = 0;
  std::map<int, SlotRec> live;
  size_t used = 0;
  // Iteration graph.
  int* tasks = nullptr;
  size_t tasksCap = 0;
  uint32_t* recTasks = nullptr;
  size_t recTasksCap = 0;
  std::vector<Launch> plan;  // the staged plan, flattened
  StagedPlan staged;
  StagedEvents sev;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool dirty = true;
  int captures = 0;
  // Walk scratch.
  int* wTasks = nullptr;
  size_t wTasksCap = 0;
  RootInfo* info = nullptr;
  size_t infoCap = 0;
  double* vals = nullptr;
  size_t valsCap = 0;

  template <typename V>
  V* at(int a, size_t entry) const {
    return reinterpret_cast<V*>(static_cast<char*>(arr[a]) + entry * kArray[a].entryBytes);
  }
  DevTree tree() const {
    DevTree t{};
    t.nodes = static_cast<const NodeDev*>(arr[aNodes]);
    t.rows = static_cast<const RowDev*>(arr[aRows]);
    t.termVal = static_cast<const float*>(arr[aTerm]);
    t.children = static_cast<const int*>(arr[aChild]);
    t.states = static_cast<const StateDev*>(arr[aState]);
    t.poolU8 = static_cast<const uint8_t*>(arr[aU8]);
    t.poolU16 = static_cast<const uint16_t*>(arr[aU16]);
    t.poolI16 = static_cast<const int16_t*>(arr[aI16]);
    t.poolSd = static_cast<const ShowdownInfo*>(arr[aSd]);
    t.regret = static_cast<float*>(arr[aReg]);
    t.strat = static_cast<float*>(arr[aStr]);
    t.coef = coef;
    t.counter = counter;
    t.err = err;
    return t;
  }
  template <typename T>
  DevRows<T> rows(int fArr0, int fArr1, int cArr) const {
    DevRows<T> r{};
    r.reach[0] = static_cast<T*>(arr[fArr0]);
    r.reach[1] = static_cast<T*>(arr[fArr1]);
    r.cfv = static_cast<T*>(arr[cArr]);
    return r;
  }
  void dropGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    dirty = true;
  }
  // Bytes array a maps when its region's top is `top` entries.
  size_t mappedFor(int a, size_t top) const {
    return roundUp(top * kArray[a].entryBytes, gran);
  }
  // Maps physical memory so array a covers its region.
  void grow(int a) {
    VmArray& v = va[a];
    const size_t need = mappedFor(a, regions[kArray[a].region].top());
    if (need <= v.mapped) return;
    if (need > v.reserved) throw Error{PPS_GB_E_BUDGET, "forest: pool address range exhausted"};
    const DriverVmm& dv = vmm();
    const size_t add = need - v.mapped;
    CUmemAllocationProp prop{};
    prop.type = CU_MEM_ALLOCATION_TYPE_PINNED;
    prop.location.type = CU_MEM_LOCATION_TYPE_DEVICE;
    prop.location.id = device;
    CUmemGenericAllocationHandle h = 0;
    cuCheck(dv.create(&h, add, &prop, 0), "cuMemCreate");
    CUresult r = dv.map(v.base + v.mapped, add, 0, h, 0);
    if (r != CUDA_SUCCESS) {
      dv.release(h);
      cuCheck(r, "cuMemMap");
    }
    CUmemAccessDesc acc{};
    acc.location = prop.location;
    acc.flags = CU_MEM_ACCESS_FLAGS_PROT_READWRITE;
    r = dv.setAccess(v.base + v.mapped, add, &acc, 1);
    if (r != CUDA_SUCCESS) {
      dv.unmap(v.base + v.mapped, add);
      dv.release(h);
      cuCheck(r, "cuMemSetAccess");
    }
    v.chunks.emplace_back(h, add);
    v.mapped = need;
  }
  // Unmaps whole trailing chunks above array a's region top (the stream is
  // idle: callers synchronize first).
  void trim(int a) {
    VmArray& v = va[a];
    const size_t need = mappedFor(a, regions[kArray[a].region].top());
    const DriverVmm& dv = vmm();
    while (!v.chunks.empty() && v.mapped - v.chunks.back().second >= need) {
      const auto c = v.chunks.back();
      v.mapped -= c.second;
      cuCheck(dv.unmap(v.base + v.mapped, c.second), "cuMemUnmap");
      cuCheck(dv.release(c.first), "cuMemRelease");
      v.chunks.pop_back();
    }
  }
  size_t mappedBytes() const {
    size_t b = 0;
    for (const VmArray& v : va) b += v.mapped;
    return b;
  }
  int maxN(const std::vector<int>& slots) const {
    int m = 1;
    for (int s : slots) m = std::max(m, live.at(s).spot->layout.maxN);
    return m;
  }
};

Forest::Forest(const std::vector<float>& coef, size_t maxBytes) : d_(new Dev()) {
  Dev& d = *d_;
  GB_CK(cudaGetDevice(&d.device));
  const DriverVmm& dv = vmm();
  CUmemAllocationProp prop{};
  prop.type = CU_MEM_ALLOCATION_TYPE_PINNED;
  prop.location.type = CU_MEM_LOCATION_TYPE_DEVICE;
  prop.location.id = d.device;
  cuCheck(dv.granularity(&d.gran, &prop, CU_MEM_ALLOC_GRANULARITY_MINIMUM),
          "cuMemGetAllocationGranularity");
  // Every pool may grow to the whole budget: reserve that much address
  // space per array (address space only; memory is mapped on growth).
  const size_t reserve = roundUp(std::max(maxBytes, d.gran), d.gran);
  for (int a = 0; a < kArrays; ++a) {
    cuCheck(dv.reserve(&d.va[a].base, reserve, 0, 0, 0), "cuMemAddressReserve");
    d.va[a].reserved = reserve;
    d.arr[a] = reinterpret_cast<void*>(d.va[a].base);
  }
  GB_CK(cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking));
  GB_CK(cudaMalloc(&d.err, sizeof(int)));
  GB_CK(cudaMemset(d.err, 0, sizeof(int)));
  d.br.create(d.stream);
  GB_CK(cudaEventCreate(&d.evA));
  GB_CK(cudaEventCreate(&d.evB));
  d.coefEntries = (int)(coef.size() / 3);
  GB_CK(cudaMalloc(&d.coef, std::max<size_t>(coef.size(), 3) * sizeof(float)));
  if (!coef.empty())
    GB_CK(cudaMemcpy(d.coef, coef.data(), coef.size() * sizeof(float), cudaMemcpyHostToDevice));
}

Forest::~Forest() {
  if (!d_) return;
  Dev& d = *d_;
  if (d.stream) cudaStreamSynchronize(d.stream);
  if (d.exec) cudaGraphExecDestroy(d.exec);
  if (d.graph) cudaGraphDestroy(d.graph);
  const DriverVmm& dv = vmm();
  for (VmArray& v : d.va) {
    size_t at = 0;
    for (const auto& c : v.chunks) {
      dv.unmap(v.base + at, c.second);
      dv.release(c.first);
      at += c.second;
    }
    if (v.base) dv.addressFree(v.base, v.reserved);
  }
  cudaFree(d.coef);
  cudaFree(d.counter);
  cudaFree(d.tasks);
  cudaFree(d.recTasks);
  cudaFree(d.err);
  cudaFree(d.wTasks);
  cudaFree(d.info);
  cudaFree(d.vals);
  d.br.destroy();
  d.sev.destroy();
  if (d.evA) cudaEventDestroy(d.evA);
  if (d.evB) cudaEventDestroy(d.evB);
  if (d.stream) cudaStreamDestroy(d.stream);
}

int Forest::admit(std::unique_ptr<CompiledSpot>& s, size_t budget) {
  Dev& d = *d_;
  if (!s || s->tree.empty) throw Error{PPS_GB_E_ARG, "forest: spot compiled to empty ranges"};
  const Tree& t = s->tree;
  HostLayout& L = s->layout;
  int slot;
  if (!d.freeSlots.empty()) {
    slot = d.freeSlots.back();
    d.freeSlots.pop_back();
  } else {
    if (d.nextSlot > 0xffff) throw Error{PPS_GB_E_BUDGET, "forest: more than 65536 spots"};
    slot = d.nextSlot++;
  }
  SlotRec rec;
  regionSizes(t, L, rec.size);
  for (int r = 0; r < kRegions; ++r) rec.off[r] = d.regions[r].alloc(rec.size[r], kGranule[r]);
  const size_t N = rec.size[rNode];
  // Index widths: 24-bit task node ids, 32-bit row quads, 31-bit pools.
  bool fits = rec.off[rNode] + N < ((size_t)1 << 24);
  for (int r : {rReg, rCfv, rReach0, rReach1})
    fits = fits && rec.off[r] + rec.size[r] <= 0xffffffffull;
  for (int r : {rChild, rState, rU8, rU16, rI16, rSd, rW, rGroup, rRec})
    fits = fits && rec.off[r] + rec.size[r] < ((size_t)1 << 31);
  if (!fits) {
    for (int r = 0; r < kRegions; ++r) d.regions[r].release(rec.off[r], rec.size[r], kGranule[r]);
    d.freeSlots.push_back(slot);
    throw Error{PPS_GB_E_BUDGET, "forest: resident spots exceed the 32-bit row / 24-bit node "
                                 "index space"};
  }
  // Device bytes once the pools cover the new ranges (plus the small
  // fixed buffers): the spot waits while that exceeds the budget.
  size_t after = deviceBytes() - d.mappedBytes();
  for (int a = 0; a < kArrays; ++a)
    after += std::max(d.va[a].mapped, d.mappedFor(a, d.regions[kArray[a].region].top()));
  if (after > budget) {
    for (int r = 0; r < kRegions; ++r) d.regions[r].release(rec.off[r], rec.size[r], kGranule[r]);
    d.freeSlots.push_back(slot);
    return -1;
  }
  for (int a = 0; a < kArrays; ++a) d.grow(a);
  if ((size_t)slot >= d.counterCap) {
    const size_t cap = std::max<size_t>(64, (size_t)slot * 2);
    int* p = nullptr;
    GB_CK(cudaMalloc(&p, cap * sizeof(int)));
    GB_CK(cudaMemsetAsync(p, 0, cap * sizeof(int), d.stream));
    if (d.counter) {
      GB_CK(cudaMemcpyAsync(p, d.counter, d.counterCap * sizeof(int), cudaMemcpyDeviceToDevice,
                            d.stream));
      GB_CK(cudaStreamSynchronize(d.stream));
      GB_CK(cudaFree(d.counter));
    }
    d.counter = p;
    d.counterCap = cap;
    d.dropGraph();
  }

  // Relocate the layout into the pools.
  const size_t* off = rec.off;
  for (NodeDev& nd : L.nodes) {
    nd.meta = (int)(((unsigned)nd.meta & 0xffffu) | ((unsigned)slot << 16));
    nd.state += (int)off[rState];
    nd.childBase += (int)off[rChild];
    nd.regQ += (uint32_t)off[rReg];
  }
  for (RowDev& rw : L.rows) {
    rw.reachQ[0] += (uint32_t)off[rReach0];
    rw.reachQ[1] += (uint32_t)off[rReach1];
    rw.cfvQ += (uint32_t)off[rCfv];
  }
  for (int& c : L.children) c += (int)off[rNode];
  auto shift = [](int& v, size_t by) {
    if (v >= 0) v += (int)by;
  };
  for (StateDev& st : L.states)
    for (int p = 0; p < 2; ++p) {
      shift(st.cardsOff[p], off[rU8]);
      shift(st.csrOff[p], off[rU16]);
      shift(st.sameOff[p], off[rI16]);
      shift(st.upOff[p], off[rU16]);
      shift(st.downOff[p], off[rI16]);
      shift(st.sdOff[p], off[rU16]);
      shift(st.sdInfoOff[p], off[rSd]);
    }
  auto put = [&](int a, size_t entry, const void* src, size_t bytes) {
    if (bytes)
      GB_CK(cudaMemcpyAsync(d.at<char>(a, entry), src, bytes, cudaMemcpyHostToDevice, d.stream));
  };
  put(aNodes, off[rNode], L.nodes.data(), L.nodes.size() * sizeof(NodeDev));
  put(aRows, off[rNode], L.rows.data(), L.rows.size() * sizeof(RowDev));
  put(aTerm, off[rNode], L.termVal.data(), L.termVal.size() * sizeof(float));
  put(aChild, off[rChild], L.children.data(), L.children.size() * sizeof(int));
  put(aState, off[rState], L.states.data(), L.states.size() * sizeof(StateDev));
  put(aU8, off[rU8], L.poolU8.data(), L.poolU8.size());
  put(aU16, off[rU16], L.poolU16.data(), L.poolU16.size() * 2);
  put(aI16, off[rI16], L.poolI16.data(), L.poolI16.size() * 2);
  put(aSd, off[rSd], L.poolSd.data(), L.poolSd.size() * sizeof(ShowdownInfo));
  // Group records (two per group, one per traverser): table offsets into
  // the pools, the nodes' rows.
  for (size_t k = 0; k < L.groupRecs.size(); ++k) {
    GroupRec& g = L.groupRecs[k];
    const int tr = (int)(k & 1);
    g.tabOff += (int)off[rU16];
    if (g.kind == kTaskShowdown) {
      g.infoOff += (int)off[rSd];
    } else {
      g.infoOff += (int)off[rU8];
      g.sameOff += (int)off[rI16];
    }
    for (int j = 0; j < 4; ++j)
      if ((g.mask >> j) & 1) {
        g.reachQ[j] += (uint32_t)off[tr ? rReach1 : rReach0];
        g.cfvQ[j] += (uint32_t)off[rCfv];
      }
  }
  put(aGroups, off[rGroup], L.groupRecs.data(), L.groupRecs.size() * sizeof(GroupRec));
  // Decide records: row offsets into the pools, the spot's counter slot.
  for (int tr = 0; tr < 2; ++tr)
    for (int fwd = 0; fwd < 2; ++fwd) {
      const uint32_t rowOff = (uint32_t)(fwd ? off[tr ? rReach1 : rReach0] : off[rCfv]);
      for (const auto& v : fwd ? L.fwdRecs[tr] : L.bwdRecs[tr])
        for (uint32_t o : v) {
          uint32_t* r = &L.recPool[(size_t)o * 4];
          const int na = (int)((r[2] >> 16) & 0xff);
          r[0] += (uint32_t)off[rReg];
          r[1] += rowOff;
          r[3] = (r[3] & 0xffffu) | ((uint32_t)slot << 16);
          for (int a = 0; a < na; ++a) r[4 + a] += rowOff;
        }
    }
  // The backward levels' own records: the header rows, the child rows and,
  // where there are folded-in children (header bit 25), every folded-in row
  // list.
  for (int tr = 0; tr < 2; ++tr)
    for (uint32_t o : L.levelRecs[tr]) {
      uint32_t* r = &L.recPool[(size_t)o * 4];
      const int na = (int)((r[2] >> 16) & 0xff);
      const uint32_t cfv = (uint32_t)off[rCfv];
      r[0] += (uint32_t)off[rReg];
      r[1] += cfv;
      r[3] = (r[3] & 0xffffu) | ((uint32_t)slot << 16);
      for (int a = 0; a < na; ++a) r[4 + a] += cfv;
      if (!((r[2] >> 25) & 1)) continue;
      uint32_t* p = r + 4 + na;
      const int P = (int)*p++;
      for (int e = 0; e < P; ++e) {
        p[0] += cfv;
        const int m = (int)p[1];
        for (int b = 0; b < m; ++b) p[2 + b] += cfv;
        p += 2 + m;
      }
    }
  // Chance records and their branch tables: rows, maps, table offsets.
  const uint32_t recShift16 = (uint32_t)(off[rRec] / 4);
  for (int tr = 0; tr < 2; ++tr) {
    const uint32_t reachOff = (uint32_t)off[tr ? rReach1 : rReach0];
    for (const auto& v : L.fwdChanceRecs[tr])
      for (uint32_t o : v) {
        uint32_t* r = &L.recPool[(size_t)o * 4];
        r[0] += reachOff;
        r[1] += reachOff;
        r[2] += (uint32_t)off[rU16];
      }
    for (const auto& v : L.bwdChanceRecs[tr])
      for (uint32_t o : v) {
        uint32_t* r = &L.recPool[(size_t)o * 4];
        r[0] += (uint32_t)off[rCfv];
        r[3] += recShift16;
      }
  }
  for (int tr = 0; tr < 2; ++tr)
    for (const auto& tb : L.chanceTables[tr]) {
      uint32_t* e = &L.recPool[(size_t)tb.first * 4];
      for (int b = 0; b < tb.second; ++b) {
        e[2 * b] += (uint32_t)off[rCfv];
        e[2 * b + 1] += (uint32_t)off[rI16];
      }
    }
  put(aRecs, off[rRec], L.recPool.data(), L.recPool.size() * sizeof(uint32_t));
  for (int a : {aReg, aStr, aCfvF, aCfvD, aReachF0, aReachD0, aReachF1, aReachD1}) {
    const Region r = kArray[a].region;
    const size_t bytes = rec.size[r] * kArray[a].entryBytes;
    if (bytes) GB_CK(cudaMemsetAsync(d.at<char>(a, off[r]), 0, bytes, d.stream));
  }
  // Root reach rows (the opponent's weights) and the weight rows.
  std::vector<double> w(t.side[0].w);
  w.insert(w.end(), t.side[1].w.begin(), t.side[1].w.end());
  put(aW, off[rW], w.data(), w.size() * sizeof(double));
  for (int tr = 0; tr < 2; ++tr) {
    const Side& opp = t.side[1 - tr];
    std::vector<float> rf(opp.w.begin(), opp.w.end());
    const size_t q = L.rows[0].reachQ[tr];
    put(tr ? aReachF1 : aReachF0, q, rf.data(), rf.size() * sizeof(float));
    put(tr ? aReachD1 : aReachD0, q, opp.w.data(), opp.w.size() * sizeof(double));
  }
  GB_CK(cudaMemsetAsync(d.counter + slot, 0, sizeof(int), d.stream));

  rec.rootCfvQ = L.rows[0].cfvQ;
  rec.rootRegQ = L.nodes[0].regQ;
  rec.depth = (int)L.fwdTasks[0].size();
  const unsigned nodeShift = (unsigned)off[rNode] << 8;
  for (int tr = 0; tr < 2; ++tr) {
    rec.fwd[tr] = std::move(L.fwdTasks[tr]);
    rec.bwd[tr] = std::move(L.bwdTasks[tr]);
    rec.inner[tr] = std::move(L.innerTasks[tr]);
    for (auto* lists : {&rec.fwd[tr], &rec.bwd[tr], &rec.inner[tr]})
      for (auto& v : *lists)
        for (int& task : v) task = (int)((unsigned)task + nodeShift);
  }
  const uint32_t recShift = (uint32_t)(off[rRec] / 4);
  for (int tr = 0; tr < 2; ++tr) {
    rec.bRec[tr] = std::move(L.bwdRecs[tr]);
    rec.fRec[tr] = std::move(L.fwdRecs[tr]);
    rec.bCh[tr] = std::move(L.bwdChanceRecs[tr]);
    rec.fCh[tr] = std::move(L.fwdChanceRecs[tr]);
    rec.termAfter[tr] = L.termAfter[tr];
    rec.bRecH[tr] = std::move(L.bwdRecsH[tr]);
    rec.bChH[tr] = std::move(L.bwdChanceRecsH[tr]);
    rec.bNeed[tr] = L.bwdNeed[tr];
    for (auto* lists : {&rec.bRec[tr], &rec.fRec[tr], &rec.bCh[tr], &rec.fCh[tr], &rec.bRecH[tr],
                        &rec.bChH[tr]})
      for (auto& v : *lists)
        for (uint32_t& o : v) o += recShift;
  }
  const unsigned groupShift = (unsigned)off[rGroup] << 8;
  rec.sdG = std::move(L.sdGroupTasks);
  rec.fdG = std::move(L.fdGroupTasks);
  for (auto* lists : {&rec.sdG, &rec.fdG})
    for (auto& v : *lists)
      for (int& task : v) task = (int)((unsigned)task + groupShift);
  // The host tables are on the device now; keep only what queries need.
  GB_CK(cudaStreamSynchronize(d.stream));
  L.termVal = {};
  L.children = {};
  L.poolU8 = {};
  L.poolU16 = {};
  L.poolI16 = {};
  L.poolSd = {};
  L.states = {};
  L.groups = {};
  L.groupRecs = {};
  L.recPool = {};
  d.used += s->bytes;
  rec.spot = std::move(s);
  d.live[slot] = std::move(rec);
  d.dirty = true;
  return slot;
}

std::unique_ptr<CompiledSpot> Forest::retire(int slot) {
  Dev& d = *d_;
  auto it = d.live.find(slot);
  if (it == d.live.end()) throw Error{PPS_GB_E_INDEX, "forest: no spot in slot"};
  SlotRec& rec = it->second;
  for (int r = 0; r < kRegions; ++r) d.regions[r].release(rec.off[r], rec.size[r], kGranule[r]);
  std::unique_ptr<CompiledSpot> s = std::move(rec.spot);
  d.used -= s->bytes;
  d.live.erase(it);
  d.freeSlots.push_back(slot);
  d.dirty = true;
  return s;
}

std::vector<int> Forest::slots() const {
  std::vector<int> out;
  for (const auto& kv : d_->live) out.push_back(kv.first);
  return out;
}

const CompiledSpot& Forest::spot(int slot) const { return *d_->live.at(slot).spot; }
int Forest::iterations(int slot) const { return d_->live.at(slot).iters; }
int Forest::maxIterations() const { return d_->coefEntries; }

namespace {

// Concatenates the listed spots' task lists: per traverser, forward lists
// per depth and backward lists per depth (terminal head, interior tail
// when `split`). Returns the refs into `all`.
struct Lists {
  std::vector<int> all;
  std::vector<uint32_t> recs;  // record offsets
  std::vector<ListRef> fwd[2], bwd[2], fCh[2], bCh[2], fRec[2], bRec[2], sdG, fdG;
  std::vector<int> termAfter[2];  // per depth: the latest of the spots' levels
  std::vector<ListRef> bRecH[2], bChH[2];  // backward per level
  std::vector<uint64_t> bNeed[2];          // per level: the union of the spots' masks
};

Lists gather(const std::map<int, SlotRec>& live, const std::vector<int>& slots, bool iteration) {
  Lists out;
  int D = 0;
  for (int s : slots) D = std::max(D, live.at(s).depth);
  auto cat = [&](auto pick) {
    const int b = (int)out.all.size();
    for (int s : slots) {
      const std::vector<int>* v = pick(live.at(s));
      if (v) out.all.insert(out.all.end(), v->begin(), v->end());
    }
    return ListRef{b, (int)out.all.size() - b};
  };
  auto at = [](const std::vector<std::vector<int>>& lists, int dd) {
    return dd < (int)lists.size() ? &lists[dd] : nullptr;
  };
  auto catRec = [&](auto pick) {
    const int b = (int)out.recs.size();
    for (int s : slots) {
      const std::vector<uint32_t>* v = pick(live.at(s));
      if (v) out.recs.insert(out.recs.end(), v->begin(), v->end());
    }
    return ListRef{b, (int)out.recs.size() - b};
  };
  auto atR = [](const std::vector<std::vector<uint32_t>>& lists, int dd) {
    return dd < (int)lists.size() ? &lists[dd] : nullptr;
  };
  for (int tr = 0; tr < 2; ++tr) {
    if (iteration) {
      // Forward levels: a spot's level l tasks depend only on its own
      // levels below l, so the spots' levels merge by index.
      int F = 0;
      for (int s : slots) F = std::max(F, (int)live.at(s).fRec[tr].size());
      for (int lv = 0; lv < F; ++lv) {
        out.fCh[tr].push_back(catRec([&](const SlotRec& r) { return atR(r.fCh[tr], lv); }));
        out.fRec[tr].push_back(catRec([&](const SlotRec& r) { return atR(r.fRec[tr], lv); }));
      }
      out.termAfter[tr].assign(D, -1);
      for (int s : slots) {
        const std::vector<int>& ta = live.at(s).termAfter[tr];
        for (int dd = 0; dd < D && dd < (int)ta.size(); ++dd)
          out.termAfter[tr][dd] = std::max(out.termAfter[tr][dd], ta[dd]);
      }
      // Backward levels merge by index too: each spot's level l reads only
      // its own levels below l.
      int H = 0;
      for (int s : slots) H = std::max(H, (int)live.at(s).bRecH[tr].size());
      out.bNeed[tr].assign(H, 0);
      for (int lv = 0; lv < H; ++lv) {
        out.bRecH[tr].push_back(catRec([&](const SlotRec& r) { return atR(r.bRecH[tr], lv); }));
        out.bChH[tr].push_back(catRec([&](const SlotRec& r) { return atR(r.bChH[tr], lv); }));
        for (int s : slots) {
          const std::vector<uint64_t>& nd = live.at(s).bNeed[tr];
          if (lv < (int)nd.size()) out.bNeed[tr][lv] |= nd[lv];
        }
      }
    }
    for (int dd = 0; dd < D; ++dd) {
      if (iteration) {
        out.bCh[tr].push_back(catRec([&](const SlotRec& r) { return atR(r.bCh[tr], dd); }));
        out.bRec[tr].push_back(catRec([&](const SlotRec& r) { return atR(r.bRec[tr], dd); }));
      } else {
        out.fwd[tr].push_back(cat([&](const SlotRec& r) { return at(r.fwd[tr], dd); }));
        out.bwd[tr].push_back(cat([&](const SlotRec& r) { return at(r.bwd[tr], dd); }));
      }
    }
  }
  if (iteration)
    for (int dd = 0; dd < D; ++dd) {
      out.sdG.push_back(cat([&](const SlotRec& r) { return at(r.sdG, dd); }));
      out.fdG.push_back(cat([&](const SlotRec& r) { return at(r.fdG, dd); }));
    }
  return out;
}

}  // namespace

void Forest::iterate(int n) {
  Dev& d = *d_;
  if (d.live.empty() || n <= 0) return;
  for (const auto& kv : d.live)
    if (kv.second.iters + n > d.coefEntries)
      throw Error{PPS_GB_E_STATE, "forest: a spot would run past the schedule table"};
  if (d.dirty || !d.exec) {
    d.dropGraph();
    const std::vector<int> all = slots();
    Lists ls = gather(d.live, all, true);
    ensureBuf(d.tasks, d.tasksCap, std::max<size_t>(ls.all.size(), 1));
    if (!ls.all.empty())
      GB_CK(cudaMemcpyAsync(d.tasks, ls.all.data(), ls.all.size() * sizeof(int),
                            cudaMemcpyHostToDevice, d.stream));
    ensureBuf(d.recTasks, d.recTasksCap, std::max<size_t>(ls.recs.size(), 1));
    if (!ls.recs.empty())
      GB_CK(cudaMemcpyAsync(d.recTasks, ls.recs.data(), ls.recs.size() * sizeof(uint32_t),
                            cudaMemcpyHostToDevice, d.stream));
    for (int tr = 0; tr < 2; ++tr) {
      const int D = (int)ls.bRec[tr].size();
      HalfStep& h = d.staged.half[tr];
      const int F = (int)ls.fRec[tr].size();
      h.fwd.assign(F, {});
      h.bwd.assign(D, {});
      h.sd.assign(D, Launch{kSdGroup, tr, ListRef{}, 0.0});
      h.fd.assign(D, Launch{kFdGroup, tr, ListRef{}, 0.0});
      h.termAfter = ls.termAfter[tr];
      for (int lv = 0; lv < F; ++lv)
        if (ls.fRec[tr][lv].count || ls.fCh[tr][lv].count) {
          Launch l{kFwdMix, tr, ls.fRec[tr][lv], 0.0};
          l.list2 = ls.fCh[tr][lv];
          l.early = tr == 0;  // the first half-step of the iteration
          h.fwd[lv].push_back(l);
        }
      for (int dd = 0; dd < D; ++dd) {
        if (ls.sdG[dd].count) h.sd[dd] = {kSdGroup, tr, ls.sdG[dd], 0.0};
        if (ls.fdG[dd].count) h.fd[dd] = {kFdGroup, tr, ls.fdG[dd], 0.0};
      }
      const int H = (int)ls.bRecH[tr].size();
      h.bwd.assign(H, {});
      h.bwdNeed = ls.bNeed[tr];
      for (int lv = 0; lv < H; ++lv)
        if (ls.bRecH[tr][lv].count || ls.bChH[tr][lv].count) {
          Launch l{kBwdMix, tr, ls.bRecH[tr][lv], 0.0};
          l.list2 = ls.bChH[tr][lv];
          h.bwd[lv].push_back(l);
        }
    }
    d.staged.counter = Launch{kCounter, 0, ListRef{}, 0.0};
    d.plan = d.staged.flat();
    d.sev.ensure((int)std::max(d.staged.half[0].fwd.size(), d.staged.half[1].fwd.size()));
    const int maxN = d.maxN(all);
    const size_t smemSd = sdGroupSmem(maxN), smemFd = fdGroupSmem(maxN);
    raiseGroupSmem(maxN);
    // The launch shape the autotuner cached for this size class (tune.h);
    // the forest always runs the staged plan.
    LaunchShape shape;
    {
      int64_t rowBytes = 0;
      for (const auto& kv : d.live) rowBytes += (int64_t)kv.second.spot->layout.regQuads * 16;
      if (lookupShape(tuneKeyOf(maxN, rowBytes), &shape)) shape.plan = 0;
      else shape = LaunchShape{};
    }
    const PlanArgs args{d.tree(), d.rows<float>(aReachF0, aReachF1, aCfvF), d.tasks, d.counter,
                        (int)d.counterCap, maxN, bwdScratchBytes<float>(maxN),
                        static_cast<const GroupRec*>(d.arr[aGroups]), smemSd, smemFd,
                        static_cast<const uint32_t*>(d.arr[aRecs]), d.recTasks, shape};
    GB_CK(cudaStreamBeginCapture(d.stream, cudaStreamCaptureModeThreadLocal));
    issueStaged(d.staged, d.br, d.sev,
                [&](const Launch& l, cudaStream_t s) { issueLaunch(args, l, s); });
    const cudaError_t launchErr = cudaGetLastError();
    cudaGraph_t g = nullptr;
    const cudaError_t endErr = cudaStreamEndCapture(d.stream, &g);
    if (launchErr != cudaSuccess || endErr != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      GB_CK(launchErr);
      GB_CK(endErr);
    }
    d.graph = g;
    GB_CK(cudaGraphInstantiate(&d.exec, d.graph, 0));
    d.dirty = false;
    ++d.captures;
  }
  GB_CK(cudaEventRecord(d.evA, d.stream));
  for (int i = 0; i < n; ++i) GB_CK(cudaGraphLaunch(d.exec, d.stream));
  GB_CK(cudaEventRecord(d.evB, d.stream));
  d.timed = true;
  for (auto& kv : d.live) kv.second.iters += n;
}

double Forest::lastIterateMs() {
  Dev& d = *d_;
  if (!d.timed) return 0.0;
  GB_CK(cudaEventSynchronize(d.evB));
  float ms = 0.0f;
  GB_CK(cudaEventElapsedTime(&ms, d.evA, d.evB));
  int e = 0;
  GB_CK(cudaMemcpy(&e, d.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    GB_CK(cudaMemset(d.err, 0, sizeof(int)));
    throw Error{PPS_GB_E_CUDA, "forest: a device wait timed out (bulk copy never completed)"};
  }
  return ms;
}

std::vector<double> Forest::walkValues(const std::vector<int>& slots, int tr, int mode) {
  return walk<double>(slots, tr, mode);
}

// The same walk with f32 rows: the iteration's own reach and value rows
// serve as its scratch (every iteration rewrites them before reading).
std::vector<double> Forest::walkValuesF32(const std::vector<int>& slots, int tr, int mode) {
  return walk<float>(slots, tr, mode);
}

template <typename T>
std::vector<double> Forest::walk(const std::vector<int>& slots, int tr, int mode) {
  Dev& d = *d_;
  std::vector<double> out(slots.size(), 0.0);
  if (slots.empty()) return out;
  Lists ls = gather(d.live, slots, false);
  ensureBuf(d.wTasks, d.wTasksCap, std::max<size_t>(ls.all.size(), 1));
  if (!ls.all.empty())
    GB_CK(cudaMemcpyAsync(d.wTasks, ls.all.data(), ls.all.size() * sizeof(int),
                          cudaMemcpyHostToDevice, d.stream));
  const int maxN = d.maxN(slots);
  const size_t smem = bwdScratchBytes<T>(maxN);
  raiseSmemLimit((const void*)bwdLevelK<T>, smem);
  const DevTree tree = d.tree();
  const bool f64 = sizeof(T) == 8;
  const DevRows<T> rows = f64 ? d.rows<T>(aReachD0, aReachD1, aCfvD)
                              : d.rows<T>(aReachF0, aReachF1, aCfvF);
  const int D = (int)ls.fwd[tr].size();
  for (int dd = 0; dd < D; ++dd) {
    const ListRef a = ls.fwd[tr][dd];
    if (a.count)
      fwdLevelK<T><<<gridOf(a.count), kThreads, 0, d.stream>>>(tree, rows, d.wTasks + a.off,
                                                              a.count, tr, 1);
  }
  for (int dd = D - 1; dd >= 0; --dd) {
    const ListRef b = ls.bwd[tr][dd];
    if (b.count)
      bwdLevelK<T><<<gridOf(b.count), kThreads, smem, d.stream>>>(
          tree, rows, d.wTasks + b.off, b.count, tr, mode, maxN);
  }
  std::vector<RootInfo> info(slots.size());
  for (size_t i = 0; i < slots.size(); ++i) {
    const SlotRec& r = d.live.at(slots[i]);
    info[i].cfvQ = r.rootCfvQ;
    info[i].wOff = (int)r.off[rW] + (tr == 0 ? 0 : r.spot->tree.side[0].n);
    info[i].n = r.spot->tree.side[tr].n;
    info[i].pad = 0;
  }
  ensureBuf(d.info, d.infoCap, info.size());
  ensureBuf(d.vals, d.valsCap, info.size());
  GB_CK(cudaMemcpyAsync(d.info, info.data(), info.size() * sizeof(RootInfo),
                        cudaMemcpyHostToDevice, d.stream));
  rootValueK<T><<<(unsigned)info.size(), 128, 0, d.stream>>>(
      static_cast<const T*>(d.arr[f64 ? aCfvD : aCfvF]), static_cast<const double*>(d.arr[aW]),
      d.info, d.vals);
  GB_CK(cudaGetLastError());
  GB_CK(cudaMemcpyAsync(out.data(), d.vals, out.size() * sizeof(double), cudaMemcpyDeviceToHost,
                        d.stream));
  GB_CK(cudaStreamSynchronize(d.stream));
  for (size_t i = 0; i < slots.size(); ++i) {
    const double Z = d.live.at(slots[i]).spot->pairMass;
    out[i] = Z > 0.0 ? out[i] / Z : 0.0;
  }
  return out;
}

std::vector<std::vector<float>> Forest::rootRows(const std::vector<int>& slots) {
  Dev& d = *d_;
  // One host staging buffer, every copy queued, one wait.
  std::vector<size_t> at(slots.size() + 1, 0);
  for (size_t k = 0; k < slots.size(); ++k) {
    const Tree& t = d.live.at(slots[k]).spot->tree;
    const Node& root = t.nodes[0];
    at[k + 1] = at[k] + (root.kind == kDecide ? quads(t.n(0, root.player)) * 4 * root.na : 0);
  }
  std::vector<float> staged(std::max<size_t>(at.back(), 1));
  for (size_t k = 0; k < slots.size(); ++k)
    if (at[k + 1] > at[k])
      GB_CK(cudaMemcpyAsync(staged.data() + at[k], d.at<float>(aStr, d.live.at(slots[k]).rootRegQ),
                            (at[k + 1] - at[k]) * sizeof(float), cudaMemcpyDeviceToHost,
                            d.stream));
  GB_CK(cudaStreamSynchronize(d.stream));
  std::vector<std::vector<float>> out(slots.size());
  for (size_t k = 0; k < slots.size(); ++k) {
    if (at[k + 1] == at[k]) continue;
    const Tree& t = d.live.at(slots[k]).spot->tree;
    const Node& root = t.nodes[0];
    const int n = t.n(0, root.player);
    const size_t stride = quads(n) * 4;
    out[k].resize((size_t)n * root.na);
    for (int a = 0; a < root.na; ++a)
      std::copy(staged.begin() + at[k] + a * stride, staged.begin() + at[k] + a * stride + n,
                out[k].begin() + (size_t)a * n);
  }
  return out;
}

void Forest::trim() {
  Dev& d = *d_;
  GB_CK(cudaStreamSynchronize(d.stream));
  for (int a = 0; a < kArrays; ++a) d.trim(a);
}

void Forest::sync() { GB_CK(cudaStreamSynchronize(d_->stream)); }

size_t Forest::deviceBytes() const {
  const Dev& d = *d_;
  size_t b = (size_t)d.coefEntries * 3 * sizeof(float) + d.counterCap * sizeof(int) +
             d.tasksCap * sizeof(int) + d.recTasksCap * sizeof(uint32_t) +
             d.wTasksCap * sizeof(int) +
             d.infoCap * sizeof(RootInfo) + d.valsCap * sizeof(double);
  return b + d.mappedBytes();
}

size_t Forest::usedBytes() const { return d_->used; }
int Forest::captures() const { return d_->captures; }
int Forest::launchesPerIteration() const { return (int)d_->plan.size(); }

}  // namespace gb
}  // namespace pps
