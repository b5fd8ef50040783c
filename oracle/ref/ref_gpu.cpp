// Runs the REFERENCE's own GPU kernels (cuda/gpu_cfr.cu: fwdLevelK,
// bwdDepthK, advanceCounterK), compiled from its source into a fatbin by
// oracle/ref/build_ref.sh, on the GB300. TEST AND MEASUREMENT
// INFRASTRUCTURE ONLY: the GPU parity tests use it as a second checker
// (the reference's iteration itself, on the same inputs), and the bench's
// reference leg times it beside the CPU port. No product code links it.
//
// The host side restates the reference's: the device arrays are the
// reference layout exported by the product compiler (bit-exact against the
// reference's own init(), cuda/gpu_cfr.cu:1331-1827, by the compiler
// tests); the kernel argument block mirrors TreeBuf (cuda/gpu_cfr.cu:
// 132-201); one CUDA graph per iteration is captured as captureGraph does
// (cuda/gpu_cfr.cu:843-868): halfStep(0), halfStep(1), advanceCounterK,
// each halfStep = one fwdLevelK per depth 0..D with decide or chance nodes
// and one bwdDepthK per non-empty depth D..0 (cuda/gpu_cfr.cu:797-829),
// 128 threads a block, 2 * max(n0Base, n1Base) floats of dynamic shared
// memory for the backward launches. The schedule is the reference's
// discountCoefs (cuda/gpu_cfr.cu:585-614), "dcfr" only.
//
// Before the first launch every kernel's parameter list is read back from
// the loaded module (cuFuncGetParamInfo) and compared with the argument
// block built here; on any difference nothing is launched.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace {

thread_local std::string g_err;

struct Fail : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define RT(x)                                                                       \
  do {                                                                              \
    cudaError_t e_ = (x);                                                           \
    if (e_ != cudaSuccess)                                                          \
      throw Fail(std::string(#x) + ": " + cudaGetErrorString(e_));                  \
  } while (0)
#define DRV(x)                                                                      \
  do {                                                                              \
    CUresult r_ = (x);                                                              \
    if (r_ != CUDA_SUCCESS)                                                         \
      throw Fail(std::string(#x) + ": driver error " + std::to_string((int)r_));    \
  } while (0)

// Driver entry points, looked up through the runtime so that the library
// loads (for the layout check) where no driver is installed.
struct Driver {
  decltype(&::cuModuleLoad) moduleLoad = nullptr;
  decltype(&::cuModuleUnload) moduleUnload = nullptr;
  decltype(&::cuModuleGetFunctionCount) functionCount = nullptr;
  decltype(&::cuModuleEnumerateFunctions) enumerateFunctions = nullptr;
  decltype(&::cuFuncGetName) funcName = nullptr;
  decltype(&::cuFuncGetParamInfo) paramInfo = nullptr;
  decltype(&::cuLaunchKernel) launchKernel = nullptr;
};

const Driver& drv() {
  static Driver d;
  static bool loaded = false;
  if (loaded) return d;
  auto get = [](const char* name, auto& fn) {
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    void* p = nullptr;
    RT(cudaGetDriverEntryPointByVersion(name, &p, 12040, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p)
      throw Fail(std::string("driver entry point missing: ") + name);
    fn = reinterpret_cast<std::remove_reference_t<decltype(fn)>>(p);
  };
  get("cuModuleLoad", d.moduleLoad);
  get("cuModuleUnload", d.moduleUnload);
  get("cuModuleGetFunctionCount", d.functionCount);
  get("cuModuleEnumerateFunctions", d.enumerateFunctions);
  get("cuFuncGetName", d.funcName);
  get("cuFuncGetParamInfo", d.paramInfo);
  get("cuLaunchKernel", d.launchKernel);
  loaded = true;
  return d;
}

// TreeBuf's members in declaration order (cuda/gpu_cfr.cu:132-201): 54
// pointers, then int n0Base, int n1Base, int64_t pot.
enum Slot {
  sRegret, sRegretRW, sStrat, sStratRW, sRegOff, sStrOff, sNa, sPlayer, sFoldBy,
  sChildFlat, sChildBase, sKind, sBoardId, sNC0, sNC1, sComboOff0, sComboOff1,
  sComboId, sReachOff, sCfvOff, sSc0, sSc1, sPotBase, sReach, sReachRW, sCfv,
  sCfvRW, sNBranch, sChanceQ, sPc0, sPc1, sRunOffOff, sRunOff, sCtap, sCtapBase,
  sExpOffOff, sExpOff, sExpIdx, sExpIdxBase, sCards0, sCards1, sSameOther0,
  sSameOther1, sBrOppSortedOff, sBrOppSorted, sBrLessOff, sBrLessEnd, sBrTieEnd,
  sBrCardPosOff, sBrCardPosIdx, sBrRevSortedOff, sBrRevSorted, sFoldSonOff,
  sFoldSon, kSlots
};

struct TreeArgs {
  const void* p[kSlots];
  int n0Base, n1Base;
  int64_t pot;
};
static_assert(sizeof(TreeArgs) == 448, "TreeBuf is 54 pointers + 2 ints + 1 int64");

// Export array name of each table slot (the reference's d* array it holds).
struct TableName {
  Slot slot;
  const char* name;
};
const TableName kTables[] = {
    {sRegOff, "regOff"},       {sStrOff, "regOff"},         {sNa, "na"},
    {sPlayer, "player"},       {sFoldBy, "foldBy"},         {sChildFlat, "childFlat"},
    {sChildBase, "childBase"}, {sKind, "kind"},             {sBoardId, "boardId"},
    {sNC0, "nC0"},             {sNC1, "nC1"},               {sComboOff0, "comboOff0"},
    {sComboOff1, "comboOff1"}, {sComboId, "comboId"},       {sCfvOff, "cfvOff"},
    {sSc0, "sc0"},             {sSc1, "sc1"},               {sPotBase, "potBase"},
    {sNBranch, "nBranch"},     {sChanceQ, "chanceQ"},       {sPc0, "pc0"},
    {sPc1, "pc1"},             {sRunOffOff, "runOffOff"},   {sRunOff, "runOff"},
    {sCtap, "ctap"},           {sCtapBase, "ctapBase"},     {sExpOffOff, "expOffOff"},
    {sExpOff, "expOff"},       {sExpIdx, "expIdx"},         {sExpIdxBase, "expIdxBase"},
    {sCards0, "cards0"},       {sCards1, "cards1"},         {sSameOther0, "sameOther0"},
    {sSameOther1, "sameOther1"}, {sBrOppSortedOff, "brOppSortedOff"},
    {sBrOppSorted, "brOppSorted"}, {sBrLessOff, "brLessOff"}, {sBrLessEnd, "brLessEnd"},
    {sBrTieEnd, "brTieEnd"},   {sBrCardPosOff, "brCardPosOff"},
    {sBrCardPosIdx, "brCardPosIdx"}, {sBrRevSortedOff, "brRevSortedOff"},
    {sBrRevSorted, "brRevSorted"}, {sFoldSonOff, "foldSonOff"}, {sFoldSon, "foldSon"},
};

struct HostArray {
  const void* data;
  int64_t count;
  int elem;
};

constexpr int kThreads = 128;  // cuda/gpu_cfr.cu:40

// cuda/gpu_cfr.cu:585-614, algo "dcfr": positive regrets weighted
// pa / (pa + 1) with pa = ta * sqrt(ta), ta = max(t - 1, 0); negative ones
// 0.5; the average strategy ((t-k)/(t-k+1))^3 with k the largest power of 4
// <= t (0 at t = 0); computed in double, stored f32.
void dcfrCoefs(int t, double out[3]) {
  const double ta = (double)std::max(t - 1, 0);
  const double pa = ta * std::sqrt(ta);
  int64_t k = 0;
  if (t > 0) {
    k = 1;
    while (k * 4 <= t) k *= 4;
  }
  const double tg = (double)(t - k);
  out[0] = pa / (pa + 1.0);
  out[1] = 0.5;
  out[2] = std::pow(tg / (tg + 1.0), 3.0);
}

struct Runner {
  int dev = 0;
  CUmodule mod = nullptr;
  CUfunction fFwd = nullptr, fBwd = nullptr, fAdv = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void*> allocs;
  TreeArgs base{};
  float* regret = nullptr;
  float* strat = nullptr;
  float* reach[2] = {nullptr, nullptr};
  const void* reachOff[2] = {nullptr, nullptr};
  float* coef = nullptr;
  int coefCap = 0;
  int* counter = nullptr;
  int64_t regTotal = 0;
  int maxDepth = 0, maxBase = 0;
  std::vector<int> decideCount, chanceCount, bwdCount, chanceBrTotal;
  std::vector<const int*> decideList, chanceList, bwdList, chanceBrOff;
  bool empty = false;

  ~Runner() {
    if (exec) cudaGraphExecDestroy(exec);
    for (void* p : allocs) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
    if (mod) drv().moduleUnload(mod);
  }

  void* upload(const HostArray& a) {
    const size_t bytes = (size_t)a.count * a.elem;
    void* d = nullptr;
    RT(cudaMalloc(&d, std::max<size_t>(bytes, 16)));
    allocs.push_back(d);
    RT(cudaMemset(d, 0, std::max<size_t>(bytes, 16)));
    if (bytes) RT(cudaMemcpy(d, a.data, bytes, cudaMemcpyHostToDevice));
    return d;
  }
  void* zeros(int64_t count, int elem) {
    const size_t bytes = std::max<size_t>((size_t)count * elem, 16);
    void* d = nullptr;
    RT(cudaMalloc(&d, bytes));
    allocs.push_back(d);
    RT(cudaMemset(d, 0, bytes));
    return d;
  }

  // Finds the one function whose (mangled) name holds `key` and checks
  // its parameter sizes.
  CUfunction kernel(const std::vector<CUfunction>& fs, const char* key,
                    const std::vector<size_t>& sizes) {
    CUfunction found = nullptr;
    for (CUfunction f : fs) {
      const char* nm = nullptr;
      DRV(drv().funcName(&nm, f));
      if (nm && std::strstr(nm, key)) {
        if (found) throw Fail(std::string("two kernels match ") + key);
        found = f;
      }
    }
    if (!found) throw Fail(std::string("kernel not in the module: ") + key);
    for (size_t i = 0; i < sizes.size(); ++i) {
      size_t off = 0, sz = 0;
      DRV(drv().paramInfo(found, i, &off, &sz));
      if (sz != sizes[i])
        throw Fail(std::string(key) + ": parameter " + std::to_string(i) + " is " +
                   std::to_string(sz) + " bytes, expected " + std::to_string(sizes[i]));
    }
    size_t off = 0, sz = 0;
    if (drv().paramInfo(found, sizes.size(), &off, &sz) == CUDA_SUCCESS)
      throw Fail(std::string(key) + ": more parameters than expected");
    return found;
  }

  void loadModule(const char* fatbin) {
    RT(cudaSetDevice(dev));
    RT(cudaFree(nullptr));  // the primary context, current on this thread
    DRV(drv().moduleLoad(&mod, fatbin));
    unsigned n = 0;
    DRV(drv().functionCount(&n, mod));
    std::vector<CUfunction> fs(n);
    if (n) DRV(drv().enumerateFunctions(fs.data(), n, mod));
    const size_t P = sizeof(void*), I = sizeof(int), T = sizeof(TreeArgs);
    // fwdLevelK(dlist, nD, clist, nC, gy, cBrOff, tr, sigSrc, TreeBuf)
    fFwd = kernel(fs, "9fwdLevelK", {P, I, P, I, I, P, I, I, T});
    // bwdDepthK(nodes, count, tr, mode, coefTab, counter, kindMask, TreeBuf)
    fBwd = kernel(fs, "9bwdDepthK", {P, I, I, I, P, P, I, T});
    // advanceCounterK(counter)
    fAdv = kernel(fs, "15advanceCounterK", {P});
  }

  void build(const std::map<std::string, HostArray>& arr, int64_t pot) {
    auto get = [&](const char* name) -> const HostArray& {
      auto it = arr.find(name);
      if (it == arr.end()) throw Fail(std::string("missing array ") + name);
      return it->second;
    };
    auto scalar = [&](const char* name) -> int64_t {
      const HostArray& a = get(name);
      if (a.count != 1 || a.elem != 8) throw Fail(std::string("bad scalar ") + name);
      return *static_cast<const int64_t*>(a.data);
    };
    empty = scalar("empty") != 0;
    if (empty) return;
    maxDepth = (int)scalar("maxDepth");
    base.n0Base = (int)scalar("n0Base");
    base.n1Base = (int)scalar("n1Base");
    base.pot = pot;
    maxBase = std::max(base.n0Base, base.n1Base);
    regTotal = scalar("regTotal");
    for (const TableName& t : kTables) base.p[t.slot] = upload(get(t.name));
    reachOff[0] = upload(get("reachOff0"));
    reachOff[1] = upload(get("reachOff1"));
    regret = static_cast<float*>(zeros(regTotal, 4));
    strat = static_cast<float*>(zeros(regTotal, 4));
    float* cfv = static_cast<float*>(zeros(scalar("reachTotal"), 4));
    reach[0] = static_cast<float*>(zeros(scalar("reachTotal0"), 4));
    reach[1] = static_cast<float*>(zeros(scalar("reachTotal1"), 4));
    // Root row of each traverser's reach layout = the opponent's weights
    // (cuda/gpu_cfr.cu:1578-1584).
    const HostArray& w0 = get("w0");
    const HostArray& w1 = get("w1");
    RT(cudaMemcpy(reach[0], w1.data, (size_t)w1.count * 4, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(reach[1], w0.data, (size_t)w0.count * 4, cudaMemcpyHostToDevice));
    base.p[sRegret] = regret;
    base.p[sRegretRW] = regret;
    base.p[sStrat] = strat;
    base.p[sStratRW] = strat;
    base.p[sCfv] = cfv;
    base.p[sCfvRW] = cfv;
    counter = static_cast<int*>(zeros(1, 4));
    for (int i = 0; i < kSlots; ++i)
      if (!base.p[i] && i != sReachOff && i != sReach && i != sReachRW)
        throw Fail("argument slot " + std::to_string(i) + " left empty");

    // Per-depth lists (cuda/gpu_cfr.cu:1377-1421), concatenated by depth.
    const int D = maxDepth + 1;
    auto ints = [&](const char* name) {
      const HostArray& a = get(name);
      if (a.elem != 4) throw Fail(std::string("bad int array ") + name);
      const int* p = static_cast<const int*>(a.data);
      return std::vector<int>(p, p + a.count);
    };
    decideCount = ints("decideCount");
    chanceCount = ints("chanceCount");
    bwdCount = ints("bwdCount");
    chanceBrTotal = ints("chanceBrTotal");
    if ((int)decideCount.size() != D || (int)chanceCount.size() != D ||
        (int)bwdCount.size() != D || (int)chanceBrTotal.size() != D)
      throw Fail("depth tables do not match maxDepth");
    const int* dl = static_cast<const int*>(upload(get("decideList")));
    const int* cl = static_cast<const int*>(upload(get("chanceList")));
    const int* bl = static_cast<const int*>(upload(get("bwdList")));
    const int* bo = static_cast<const int*>(upload(get("chanceBrOff")));
    int64_t od = 0, oc = 0, ob = 0, oo = 0;
    for (int d = 0; d < D; ++d) {
      decideList.push_back(dl + od);
      chanceList.push_back(cl + oc);
      bwdList.push_back(bl + ob);
      chanceBrOff.push_back(bo + oo);
      od += decideCount[d];
      oc += chanceCount[d];
      ob += bwdCount[d];
      oo += chanceCount[d] + 1;
    }
    if (od != get("decideList").count || oc != get("chanceList").count ||
        ob != get("bwdList").count || oo != get("chanceBrOff").count)
      throw Fail("depth lists do not match their counts");
    RT(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  }

  void launch(CUfunction f, unsigned grid, unsigned smem, void** args) {
    DRV(drv().launchKernel(f, grid, 1, 1, kThreads, 1, 1, smem, (CUstream)stream, args, nullptr));
  }

  // cuda/gpu_cfr.cu:797-829, CFR mode (sigSrc 0).
  void halfStep(int tr) {
    TreeArgs b = base;
    b.p[sReachOff] = reachOff[tr];
    b.p[sReach] = reach[tr];
    b.p[sReachRW] = reach[tr];
    const int gy = (maxBase + kThreads - 1) / kThreads;
    const unsigned smem = (unsigned)(2 * maxBase * sizeof(float));
    int sigSrc = 0, mode = 0, kindMask = -1;
    for (int d = 0; d <= maxDepth; ++d) {
      int nD = decideCount[d], nC = chanceCount[d];
      if (nD == 0 && nC == 0) continue;
      const unsigned g = (unsigned)(nD * gy + chanceBrTotal[d]);
      const int* dlp = decideList[d];
      const int* clp = chanceList[d];
      const int* bop = chanceBrOff[d];
      int gyv = gy, trv = tr;
      void* args[] = {&dlp, &nD, &clp, &nC, &gyv, &bop, &trv, &sigSrc, &b};
      launch(fFwd, g, 0, args);
    }
    for (int d = maxDepth; d >= 0; --d) {
      int cnt = bwdCount[d];
      if (cnt <= 0) continue;
      const int* blp = bwdList[d];
      const float* cp = coef;
      const int* ctr = counter;
      int trv = tr;
      void* args[] = {&blp, &cnt, &trv, &mode, &cp, &ctr, &kindMask, &b};
      launch(fBwd, (unsigned)cnt, smem, args);
    }
  }

  void capture() {
    if (exec) {
      cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
    cudaGraph_t g = nullptr;
    RT(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    try {
      halfStep(0);
      halfStep(1);
      int* ctr = counter;
      void* args[] = {&ctr};
      DRV(drv().launchKernel(fAdv, 1, 1, 1, 1, 1, 1, 0, (CUstream)stream, args, nullptr));
    } catch (...) {
      cudaStreamEndCapture(stream, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    RT(cudaStreamEndCapture(stream, &g));
    const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    RT(e);
  }

  // Resets the rows and the counter and loads the schedule of an
  // `iterations`-long solve (cuda/gpu_cfr.cu:1842-1893).
  void prepare(int iterations) {
    if (iterations > coefCap) {
      if (coef) {
        RT(cudaFree(coef));
        allocs.erase(std::find(allocs.begin(), allocs.end(), (void*)coef));
      }
      coefCap = std::max(iterations, 2 * coefCap);
      RT(cudaMalloc(&coef, (size_t)coefCap * 3 * sizeof(float)));
      allocs.push_back(coef);
      capture();
    } else if (!exec) {
      capture();
    }
    std::vector<float> tab((size_t)iterations * 3);
    for (int t = 0; t < iterations; ++t) {
      double c[3];
      dcfrCoefs(t, c);
      for (int k = 0; k < 3; ++k) tab[(size_t)t * 3 + k] = (float)c[k];
    }
    RT(cudaMemcpy(coef, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice));
    RT(cudaMemsetAsync(regret, 0, (size_t)regTotal * 4, stream));
    RT(cudaMemsetAsync(strat, 0, (size_t)regTotal * 4, stream));
    RT(cudaMemsetAsync(counter, 0, 4, stream));
    RT(cudaStreamSynchronize(stream));
  }

  void replay(int n) {
    for (int i = 0; i < n; ++i) RT(cudaGraphLaunch(exec, stream));
  }
};

int fail(const char* what) {
  g_err = what;
  return 1;
}

}  // namespace

extern "C" {

const char* refgpu_last_error() { return g_err.c_str(); }

// Builds the reference's device arrays from the exported layout (names,
// element sizes, counts and host pointers of every array the product
// compiler's reference export yields) and loads the kernels from `fatbin`.
int refgpu_create(const char* fatbin, int n, const char* const* names,
                  const void* const* data, const int64_t* counts, const int* elems,
                  int64_t pot, void** out) {
  *out = nullptr;
  Runner* r = new Runner();
  try {
    std::map<std::string, HostArray> arr;
    for (int i = 0; i < n; ++i) arr[names[i]] = HostArray{data[i], counts[i], elems[i]};
    r->loadModule(fatbin);
    r->build(arr, pot);
  } catch (const std::exception& e) {
    delete r;
    return fail(e.what());
  }
  *out = r;
  return 0;
}

void refgpu_destroy(void* h) { delete static_cast<Runner*>(h); }

// Runs a fresh `iterations`-iteration solve (the reference's solve()
// without a target): reset, schedule, graph replays, synchronize.
int refgpu_solve(void* h, int iterations) {
  Runner* r = static_cast<Runner*>(h);
  try {
    if (r->empty || iterations <= 0) return 0;
    r->prepare(iterations);
    r->replay(iterations);
    RT(cudaStreamSynchronize(r->stream));
  } catch (const std::exception& e) {
    return fail(e.what());
  }
  return 0;
}

// Milliseconds per iteration: a fresh solve of warmup + iterations graph
// replays, the last `iterations` timed with CUDA events on the solver's
// stream.
int refgpu_time(void* h, int warmup, int iterations, double* msPerIter) {
  Runner* r = static_cast<Runner*>(h);
  *msPerIter = 0.0;
  try {
    if (r->empty || iterations <= 0) return 0;
    r->prepare(warmup + iterations);
    r->replay(warmup);
    cudaEvent_t a, b;
    RT(cudaEventCreate(&a));
    RT(cudaEventCreate(&b));
    RT(cudaStreamSynchronize(r->stream));
    RT(cudaEventRecord(a, r->stream));
    r->replay(iterations);
    RT(cudaEventRecord(b, r->stream));
    RT(cudaEventSynchronize(b));
    float ms = 0.f;
    RT(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *msPerIter = (double)ms / iterations;
  } catch (const std::exception& e) {
    return fail(e.what());
  }
  return 0;
}

// Copies the cumulative regret (which 0) or strategy (which 1) rows,
// regTotal floats in the reference's regOff layout.
int refgpu_rows(void* h, int which, float* out, int64_t cap) {
  Runner* r = static_cast<Runner*>(h);
  try {
    if (r->empty) return 0;
    if (cap < r->regTotal) throw Fail("row buffer too small");
    RT(cudaMemcpy(out, which == 0 ? r->regret : r->strat, (size_t)r->regTotal * 4,
                  cudaMemcpyDeviceToHost));
  } catch (const std::exception& e) {
    return fail(e.what());
  }
  return 0;
}

int64_t refgpu_row_total(void* h) { return static_cast<Runner*>(h)->regTotal; }

// The kernel argument block as built here: TreeBuf member names in slot
// order with their byte offsets; returns the member count and the block
// size in *size (checked against the reference's own struct by a test).
int refgpu_args_layout(const char** names, int64_t* offsets, int cap, int64_t* size) {
  static const char* const kNames[] = {
      "regret", "regretRW", "strat", "stratRW", "regOff", "strOff", "na", "player",
      "foldBy", "childFlat", "childBase", "kind", "boardId", "nC0", "nC1", "comboOff0",
      "comboOff1", "comboId", "reachOff", "cfvOff", "sc0", "sc1", "potBase", "reach",
      "reachRW", "cfv", "cfvRW", "nBranch", "chanceQ", "pc0", "pc1", "runOffOff",
      "runOff", "ctap", "ctapBase", "expOffOff", "expOff", "expIdx", "expIdxBase",
      "cards0", "cards1", "sameOther0", "sameOther1", "brOppSortedOff", "brOppSorted",
      "brLessOff", "brLessEnd", "brTieEnd", "brCardPosOff", "brCardPosIdx",
      "brRevSortedOff", "brRevSorted", "foldSonOff", "foldSon"};
  static_assert(sizeof(kNames) / sizeof(kNames[0]) == kSlots, "one name per slot");
  const int n = kSlots + 3;
  for (int i = 0; i < n && i < cap; ++i) {
    if (i < kSlots) {
      names[i] = kNames[i];
      offsets[i] = (int64_t)(i * sizeof(void*));
    } else {
      static const char* const tail[] = {"n0Base", "n1Base", "pot"};
      names[i] = tail[i - kSlots];
      offsets[i] = i == kSlots ? (int64_t)offsetof(TreeArgs, n0Base)
                   : i == kSlots + 1 ? (int64_t)offsetof(TreeArgs, n1Base)
                                     : (int64_t)offsetof(TreeArgs, pot);
    }
  }
  *size = (int64_t)sizeof(TreeArgs);
  return n;
}

}  // extern "C"
