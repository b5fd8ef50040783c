// Batched and served solving: a request queue in front of a Forest.
//
// submit() hands a spot to a pool of compile threads; compiled spots wait
// in ticket order and are admitted into the forest while the device memory
// the forest maps stays within the HBM budget. A driver
// (run() on the caller's thread, or the thread start() launches) repeats
// epochs: admit, run DCFR iterations of every resident spot in one graph
// until the next spot is due for a check, run the FP64 best-response walks
// of the spots that are due, and retire each spot whose exploitability
// reached its target (or whose iteration cap was reached) after its FP64
// EV walks. Spots admitted while others are resident share the same
// launches, so work of requests that arrive at different times overlaps on
// the device.
//
// Check schedule (per spot, counted from its admission, in steps of
// kCheckStep iterations). Adaptive (default): the first check after
// min(32, checkEvery) iterations; after a check at t with exploitability e
// above the target, the next one where e ~ 1/t^2 would meet the target,
// t * sqrt(e / target), but at least kCheckStep and at most checkEvery
// iterations later. Fixed: every checkEvery iterations. A spot's schedule
// depends only on its own exploitability values, and its rows on nothing
// but its own inputs, so a result does not depend on which other spots
// were resident.
#pragma once

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "forest.h"
#include "gpu_cfr.h"
#include "postflop_cfr.h"

namespace pps {
namespace gb {

constexpr int kCheckStep = 16;  // check granularity (iterations)

struct BatchConfig {
  int64_t budget = 0;        // device bytes for resident spots (0: 80% of free memory)
  int checkEvery = 64;       // most iterations between two checks of a spot
  bool fixedChecks = false;  // check every checkEvery iterations (no prediction)
  int maxIterations = 4096;  // per spot, rounded up to a multiple of kCheckStep
  int threads = 0;           // compile threads (0: hardware threads, at most 16)
  std::string algo = "dcfr";
};

struct BatchResult {
  int64_t ticket = 0;
  int status = 0;  // PPS_GB_OK or a PPS_GB_E_* code
  std::string error;
  bool converged = false;
  int iterations = 0;
  double ev0 = 0.0, ev1 = 0.0, expl = 0.0, target = 0.0;
  int64_t pairMass = 0;
  double submitMs = 0.0, admitMs = 0.0, finishMs = 0.0;
  int numNodes = 0;
  size_t deviceBytes = 0;
  std::vector<pf::TreeAction> rootActions;
  std::vector<double> rootFreqs;
  int rootCombos = 0;
  std::vector<float> rootRows;  // na x n cumulative root strategy rows
};

struct BatchInfo {
  int64_t submitted = 0, compiling = 0, waiting = 0, active = 0, done = 0, failed = 0;
  int64_t usedBytes = 0, deviceBytes = 0, budget = 0;
  int64_t epochs = 0, spotIterations = 0, captures = 0, peakActive = 0, peakUsed = 0;
  int checkEvery = 0, maxIterations = 0;
  int64_t checks = 0;  // spot checks (best-response walk pairs per spot)
  double admitMs = 0.0, iterateMs = 0.0, checkMs = 0.0, retireMs = 0.0, idleMs = 0.0;
};

class BatchServer {
 public:
  explicit BatchServer(const BatchConfig& cfg);
  ~BatchServer();
  BatchServer(const BatchServer&) = delete;
  BatchServer& operator=(const BatchServer&) = delete;

  // Queues a spot; target = exploitability in chips (<= 0: run to the cap).
  int64_t submit(const gpu::PostflopSpot& spot, const gpu::StreetBetConfigs& cfgs,
                 bool perStreet, double target);
  void setBudget(int64_t bytes);
  // Drives epochs on the calling thread until every submitted request has
  // finished; false if timeoutS (> 0) passed first.
  bool run(double timeoutS);
  void start();
  void stop();
  // True (and *out filled) once the request finished.
  bool poll(int64_t ticket, BatchResult* out) const;
  bool wait(int64_t ticket, double timeoutS, BatchResult* out);
  // Finished results not collected before, in ticket order (at most max).
  std::vector<BatchResult> collect(size_t max);
  BatchInfo info() const;
  double nowMs() const;

 private:
  enum ReqState { kCompiling, kWaiting, kActive, kDone };
  struct Request {
    ReqState state = kCompiling;
    gpu::PostflopSpot spot;
    gpu::StreetBetConfigs cfgs;
    bool perStreet = false;
    double target = 0.0;
    BatchResult result;
  };

  BatchConfig cfg_;
  int device_ = 0;
  std::unique_ptr<Forest> forest_;
  std::chrono::steady_clock::time_point t0_;

  mutable std::mutex m_;
  std::condition_variable cvCompile_, cvReady_, cvDone_;
  std::map<int64_t, Request> reqs_;
  std::vector<int64_t> compileQueue_;  // FIFO of tickets to compile
  size_t compileHead_ = 0;
  std::map<int64_t, std::unique_ptr<CompiledSpot>> ready_;
  // Device bytes of the compiled spots waiting for admission. Compile
  // threads pause while it exceeds twice the HBM budget: spots beyond that
  // cannot be admitted soon, and each holds its host tables meanwhile
  // (~50 MB for a 48,255-node turn), so a long queue of requests would
  // otherwise grow host memory without bound.
  int64_t readyBytes_ = 0;
  std::map<int, int64_t> slotTicket_;
  std::map<int, int> nextCheck_;  // slot -> iteration count of its next check
  int64_t nextTicket_ = 1;
  int64_t budget_ = 0;
  int64_t pending_ = 0;  // submitted, not finished
  BatchInfo stats_;
  bool closing_ = false;
  std::vector<std::thread> compilers_;

  std::mutex driverMutex_;  // one driver at a time
  std::thread serveThread_;
  std::atomic<bool> serving_{false};

  void compileLoop();
  bool epoch();  // one admission / iterate / check / retire round
  void finish(int64_t ticket, BatchResult&& r);
};

}  // namespace gb
}  // namespace pps
