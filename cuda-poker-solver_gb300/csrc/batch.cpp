// Batched and served solving (see batch.h).
#include "batch.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>

#include "layout.h"
#include "pps_gb.h"
#include "solver.h"

namespace pps {
namespace gb {

namespace {

void cudaCheck(cudaError_t e, const char* what) {
  if (e != cudaSuccess)
    throw Error{e == cudaErrorMemoryAllocation ? PPS_GB_E_MEMORY : PPS_GB_E_CUDA,
                std::string("CUDA error: ") + cudaGetErrorString(e) + " (" + what + ")"};
}

std::vector<float> scheduleTable(const Schedule& s, int entries) {
  std::vector<float> tab((size_t)entries * 3);
  for (int t = 0; t < entries; ++t) {
    double c[3];
    s.coefs(t, entries, c);
    for (int k = 0; k < 3; ++k) tab[(size_t)t * 3 + k] = (float)c[k];
  }
  return tab;
}

}  // namespace

BatchServer::BatchServer(const BatchConfig& cfg) : cfg_(cfg), t0_(std::chrono::steady_clock::now()) {
  Schedule s;
  if (!Schedule::parse(cfg_.algo, s) || s.hs30)
    throw Error{PPS_GB_E_ARG, "batch: algo must be a DCFR schedule (dcfr, dcfr-g2, "
                              "dcfr-noreset, dcfr-g2-noreset), got '" + cfg_.algo + "'"};
  if (cfg_.checkEvery <= 0) cfg_.checkEvery = 64;
  cfg_.checkEvery = (cfg_.checkEvery + kCheckStep - 1) / kCheckStep * kCheckStep;
  if (cfg_.maxIterations <= 0) cfg_.maxIterations = 4096;
  cfg_.maxIterations = (cfg_.maxIterations + kCheckStep - 1) / kCheckStep * kCheckStep;
  cudaCheck(cudaGetDevice(&device_), "cudaGetDevice");
  budget_ = cfg_.budget;
  if (budget_ <= 0) {
    size_t freeB = 0, totalB = 0;
    cudaCheck(cudaMemGetInfo(&freeB, &totalB), "cudaMemGetInfo");
    budget_ = (int64_t)(0.8 * (double)freeB);
  }
  size_t freeB = 0, totalB = 0;
  cudaCheck(cudaMemGetInfo(&freeB, &totalB), "cudaMemGetInfo");
  forest_.reset(new Forest(scheduleTable(s, cfg_.maxIterations),
                           std::max<size_t>(totalB, (size_t)std::max<int64_t>(budget_, 0))));
  stats_.checkEvery = cfg_.checkEvery;
  stats_.maxIterations = cfg_.maxIterations;
  int n = cfg_.threads;
  if (n <= 0) n = std::min(16, std::max(1, (int)std::thread::hardware_concurrency()));
  for (int i = 0; i < n; ++i) compilers_.emplace_back([this] { compileLoop(); });
}

BatchServer::~BatchServer() {
  stop();
  {
    std::lock_guard<std::mutex> lock(m_);
    closing_ = true;
  }
  cvCompile_.notify_all();
  for (auto& t : compilers_) t.join();
}

double BatchServer::nowMs() const {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0_)
      .count();
}

int64_t BatchServer::submit(const gpu::PostflopSpot& spot, const gpu::StreetBetConfigs& cfgs,
                            bool perStreet, double target) {
  std::lock_guard<std::mutex> lock(m_);
  const int64_t ticket = nextTicket_++;
  Request& r = reqs_[ticket];
  r.spot = spot;
  r.cfgs = cfgs;
  r.perStreet = perStreet;
  r.target = target;
  r.result.ticket = ticket;
  r.result.target = target;
  r.result.submitMs = nowMs();
  compileQueue_.push_back(ticket);
  ++pending_;
  ++stats_.submitted;
  ++stats_.compiling;
  cvCompile_.notify_one();
  return ticket;
}

void BatchServer::setBudget(int64_t bytes) {
  {
    std::lock_guard<std::mutex> lock(m_);
    budget_ = bytes;
  }
  cvCompile_.notify_all();  // the compile-ahead limit follows the budget
}

void BatchServer::compileLoop() {
  for (;;) {
    int64_t ticket;
    gpu::PostflopSpot spot;
    gpu::StreetBetConfigs cfgs;
    bool perStreet;
    {
      std::unique_lock<std::mutex> lock(m_);
      cvCompile_.wait(lock, [&] {
        return closing_ || (compileHead_ < compileQueue_.size() &&
                            (ready_.empty() || budget_ <= 0 || readyBytes_ <= 2 * budget_));
      });
      if (closing_) return;
      ticket = compileQueue_[compileHead_++];
      if (compileHead_ == compileQueue_.size()) {
        compileQueue_.clear();
        compileHead_ = 0;
      }
      const Request& r = reqs_.at(ticket);
      spot = r.spot;
      cfgs = r.cfgs;
      perStreet = r.perStreet;
    }
    std::unique_ptr<CompiledSpot> cs;
    int code = PPS_GB_OK;
    std::string msg;
    try {
      cs = compileSpot(spot, cfgs, perStreet);
    } catch (const Error& e) {
      code = e.code;
      msg = e.msg;
    } catch (const std::exception& e) {
      code = PPS_GB_E_MEMORY;
      msg = e.what();
    }
    std::unique_lock<std::mutex> lock(m_);
    --stats_.compiling;
    Request& r = reqs_.at(ticket);
    if (code != PPS_GB_OK || cs->tree.empty) {
      // Failed compiles and empty ranges finish at once (empty: zero stats,
      // as a lone solver reports).
      BatchResult res = r.result;
      res.status = code;
      res.error = msg;
      res.admitMs = res.finishMs = nowMs();
      if (code == PPS_GB_OK) res.converged = true;
      lock.unlock();
      finish(ticket, std::move(res));
      continue;
    }
    r.result.numNodes = (int)cs->tree.nodes.size();
    r.result.deviceBytes = cs->bytes;
    r.state = kWaiting;
    ++stats_.waiting;
    readyBytes_ += (int64_t)cs->bytes;
    ready_[ticket] = std::move(cs);
    cvReady_.notify_all();
  }
}

void BatchServer::finish(int64_t ticket, BatchResult&& r) {
  std::lock_guard<std::mutex> lock(m_);
  Request& q = reqs_.at(ticket);
  q.state = kDone;
  if (r.status != PPS_GB_OK) ++stats_.failed;
  ++stats_.done;
  q.result = std::move(r);
  --pending_;
  cvDone_.notify_all();
}

bool BatchServer::epoch() {
  Forest& F = *forest_;
  const double tStart = nowMs();
  // Admission in ticket order while the forest's device bytes stay within
  // the budget; a spot that does not fit waits (or fails if it cannot fit
  // even alone).
  bool admitted = false;
  for (;;) {
    int64_t ticket;
    std::unique_ptr<CompiledSpot> cs;
    int64_t budget;
    {
      std::lock_guard<std::mutex> lock(m_);
      if (ready_.empty()) break;
      auto it = ready_.begin();
      ticket = it->first;
      cs = std::move(it->second);
      ready_.erase(it);
      readyBytes_ -= (int64_t)cs->bytes;
      budget = budget_;
    }
    int slot = -1;
    int code = PPS_GB_OK;
    std::string msg;
    try {
      slot = F.admit(cs, budget > 0 ? (size_t)budget : 0);
    } catch (const Error& e) {
      code = e.code;
      msg = e.msg;
    }
    if (code == PPS_GB_OK && slot < 0 && F.slots().empty()) {
      code = PPS_GB_E_BUDGET;
      msg = "spot needs " + std::to_string(cs->bytes) + " device bytes, budget is " +
            std::to_string(budget);
    }
    std::unique_lock<std::mutex> lock(m_);
    if (code == PPS_GB_OK && slot < 0) {
      readyBytes_ += (int64_t)cs->bytes;
      ready_[ticket] = std::move(cs);  // waits for memory to free up
      break;
    }
    --stats_.waiting;
    cvCompile_.notify_all();  // the waiting queue shrank
    if (code != PPS_GB_OK) {
      BatchResult res = reqs_.at(ticket).result;
      res.status = code;
      res.error = msg;
      res.admitMs = res.finishMs = nowMs();
      lock.unlock();
      finish(ticket, std::move(res));
      continue;
    }
    slotTicket_[slot] = ticket;
    Request& q = reqs_.at(ticket);
    q.state = kActive;
    q.result.admitMs = nowMs();
    ++stats_.active;
    admitted = true;
  }
  const std::vector<int> slots = F.slots();
  const double tAdmitted = nowMs();
  {
    std::lock_guard<std::mutex> lock(m_);
    stats_.admitMs += tAdmitted - tStart;
    stats_.peakActive = std::max<int64_t>(stats_.peakActive, (int64_t)slots.size());
    stats_.usedBytes = (int64_t)F.usedBytes();
    stats_.peakUsed = std::max(stats_.peakUsed, stats_.usedBytes);
    stats_.deviceBytes = (int64_t)F.deviceBytes();
  }
  if (slots.empty()) return admitted;

  // Iterate until the first resident spot is due (every count and due
  // point is a multiple of kCheckStep, so no spot passes its check point).
  const int first = cfg_.fixedChecks ? cfg_.checkEvery : std::min(32, cfg_.checkEvery);
  int n = cfg_.maxIterations;
  for (int slot : slots) {
    auto it = nextCheck_.find(slot);
    if (it == nextCheck_.end()) it = nextCheck_.emplace(slot, first).first;
    it->second = std::min(it->second, cfg_.maxIterations);
    n = std::min(n, it->second - F.iterations(slot));
  }
  n = std::max(n, kCheckStep);
  F.iterate(n);
  // Wait for the replays here, so that the check time below covers the
  // walks alone (the replays are timed on the device).
  const double iterMs = F.lastIterateMs();
  const double tIterated = nowMs();
  std::vector<int> due;
  for (int slot : slots)
    if (F.iterations(slot) >= nextCheck_.at(slot)) due.push_back(slot);
  // Exploitability of each due spot: an f32 best-response walk screens
  // first; a spot whose f32 value is within kScreen of its target (or that
  // has reached max_iterations) is walked again in FP64, and only the FP64
  // value retires it. The f32 value of the others only places their next
  // check. (f32 rounding moves the value by ~1e-6 of the pot, far inside
  // the factor.)
  constexpr double kScreen = 1.5;
  std::vector<double> expl(due.size(), 0.0), target(due.size(), 0.0);
  std::vector<char> exact(due.size(), 0);
  {
    const std::vector<double> s0 = F.walkValuesF32(due, 0, kModeBR);
    const std::vector<double> s1 = F.walkValuesF32(due, 1, kModeBR);
    std::vector<int> close;
    std::vector<size_t> closeAt;
    for (size_t i = 0; i < due.size(); ++i) {
      const int slot = due[i];
      expl[i] = (s0[i] + s1[i] - (double)F.spot(slot).tree.spot.pot) / 2.0;
      {
        std::lock_guard<std::mutex> lock(m_);
        target[i] = reqs_.at(slotTicket_.at(slot)).target;
      }
      if ((target[i] > 0.0 && expl[i] <= kScreen * target[i]) ||
          F.iterations(slot) >= cfg_.maxIterations) {
        close.push_back(slot);
        closeAt.push_back(i);
      }
    }
    const std::vector<double> br0 = F.walkValues(close, 0, kModeBR);
    const std::vector<double> br1 = F.walkValues(close, 1, kModeBR);
    for (size_t k = 0; k < close.size(); ++k) {
      const size_t i = closeAt[k];
      expl[i] = (br0[k] + br1[k] - (double)F.spot(close[k]).tree.spot.pot) / 2.0;
      exact[i] = 1;
    }
  }
  std::vector<int> done;
  std::vector<double> doneExpl;
  for (size_t i = 0; i < due.size(); ++i) {
    const int slot = due[i];
    const int t = F.iterations(slot);
    if (exact[i] && ((target[i] > 0.0 && expl[i] <= target[i]) || t >= cfg_.maxIterations)) {
      done.push_back(slot);
      doneExpl.push_back(expl[i]);
      continue;
    }
    int step = cfg_.checkEvery;
    if (!cfg_.fixedChecks && target[i] > 0.0 && expl[i] > 0.0) {
      const double want = (double)t * std::sqrt(expl[i] / target[i]) - (double)t;
      const int s = (int)std::ceil(std::max(want, 1.0) / kCheckStep) * kCheckStep;
      step = std::min(cfg_.checkEvery, std::max(kCheckStep, s));
    }
    nextCheck_[slot] = t + step;
  }
  const double tChecked = nowMs();
  {
    std::lock_guard<std::mutex> lock(m_);
    ++stats_.epochs;
    stats_.spotIterations += (int64_t)slots.size() * n;
    stats_.checks += (int64_t)due.size();
    stats_.captures = F.captures();
    stats_.iterateMs += iterMs;
    stats_.checkMs += tChecked - tIterated;
  }
  if (done.empty()) return true;

  const std::vector<double> ev0 = F.walkValues(done, 0, kModeEV);
  const std::vector<double> ev1 = F.walkValues(done, 1, kModeEV);
  std::vector<std::vector<float>> rootRows = F.rootRows(done);
  for (size_t i = 0; i < done.size(); ++i) {
    const int slot = done[i];
    BatchResult res;
    int64_t ticket;
    {
      std::lock_guard<std::mutex> lock(m_);
      ticket = slotTicket_.at(slot);
      res = reqs_.at(ticket).result;
    }
    const CompiledSpot& cs = F.spot(slot);
    const Tree& t = cs.tree;
    res.status = PPS_GB_OK;
    res.iterations = F.iterations(slot);
    res.expl = doneExpl[i];
    res.converged = res.target > 0.0 && res.expl <= res.target;
    res.ev0 = ev0[i];
    res.ev1 = ev1[i];
    res.pairMass = (int64_t)(cs.pairMass * (double)(1LL << 20));
    const Node& root = t.nodes[0];
    if (root.kind == kDecide) {
      res.rootRows = std::move(rootRows[i]);
      res.rootCombos = t.n(0, root.player);
      res.rootFreqs = aggregate(res.rootRows, root.na, res.rootCombos, t.side[root.player].w);
      res.rootActions.assign(t.actions.begin() + root.actBase,
                             t.actions.begin() + root.actBase + root.na);
    }
    F.retire(slot);
    nextCheck_.erase(slot);
    res.finishMs = nowMs();
    {
      std::lock_guard<std::mutex> lock(m_);
      slotTicket_.erase(slot);
      --stats_.active;
      stats_.usedBytes = (int64_t)F.usedBytes();
    }
    finish(ticket, std::move(res));
  }
  F.trim();
  std::lock_guard<std::mutex> lock(m_);
  stats_.retireMs += nowMs() - tChecked;
  stats_.deviceBytes = (int64_t)F.deviceBytes();
  return true;
}

bool BatchServer::run(double timeoutS) {
  std::unique_lock<std::mutex> driver(driverMutex_, std::try_to_lock);
  if (!driver.owns_lock() || serving_)
    throw Error{PPS_GB_E_STATE, "batch: another driver (run or the serve thread) is active"};
  cudaCheck(cudaSetDevice(device_), "cudaSetDevice");
  const double deadline = timeoutS > 0.0 ? nowMs() + 1000.0 * timeoutS : 0.0;
  for (;;) {
    {
      std::lock_guard<std::mutex> lock(m_);
      if (pending_ == 0) return true;
    }
    if (deadline > 0.0 && nowMs() > deadline) return false;
    if (!epoch()) {
      // Nothing resident: wait for a compile to finish.
      const double t = nowMs();
      std::unique_lock<std::mutex> lock(m_);
      cvReady_.wait_for(lock, std::chrono::milliseconds(20),
                        [&] { return !ready_.empty() || pending_ == 0; });
      stats_.idleMs += nowMs() - t;
    }
  }
}

void BatchServer::start() {
  if (serving_.exchange(true)) return;
  serveThread_ = std::thread([this] {
    std::lock_guard<std::mutex> driver(driverMutex_);
    try {
      cudaCheck(cudaSetDevice(device_), "cudaSetDevice");
      while (serving_) {
        if (!epoch()) {
          const double t = nowMs();
          std::unique_lock<std::mutex> lock(m_);
          cvReady_.wait_for(lock, std::chrono::milliseconds(5),
                            [&] { return !ready_.empty() || !serving_; });
          stats_.idleMs += nowMs() - t;
        }
      }
    } catch (const Error& e) {
      // A device error ends serving: fail everything still pending.
      std::lock_guard<std::mutex> lock(m_);
      for (auto& kv : reqs_)
        if (kv.second.state != kDone) {
          kv.second.state = kDone;
          kv.second.result.status = e.code;
          kv.second.result.error = e.msg;
          ++stats_.failed;
          ++stats_.done;
          --pending_;
        }
      serving_ = false;
      cvDone_.notify_all();
    }
  });
}

void BatchServer::stop() {
  serving_ = false;
  cvReady_.notify_all();
  if (serveThread_.joinable()) serveThread_.join();
}

bool BatchServer::poll(int64_t ticket, BatchResult* out) const {
  std::lock_guard<std::mutex> lock(m_);
  auto it = reqs_.find(ticket);
  if (it == reqs_.end()) throw Error{PPS_GB_E_INDEX, "batch: unknown or collected ticket"};
  if (it->second.state != kDone) return false;
  if (out) *out = it->second.result;
  return true;
}

bool BatchServer::wait(int64_t ticket, double timeoutS, BatchResult* out) {
  std::unique_lock<std::mutex> lock(m_);
  auto done = [&] {
    auto it = reqs_.find(ticket);
    return it == reqs_.end() || it->second.state == kDone;
  };
  if (timeoutS > 0.0)
    cvDone_.wait_for(lock, std::chrono::duration<double>(timeoutS), done);
  else
    cvDone_.wait(lock, done);
  auto it = reqs_.find(ticket);
  if (it == reqs_.end()) throw Error{PPS_GB_E_INDEX, "batch: unknown or collected ticket"};
  if (it->second.state != kDone) return false;
  if (out) *out = it->second.result;
  return true;
}

std::vector<BatchResult> BatchServer::collect(size_t max) {
  std::lock_guard<std::mutex> lock(m_);
  std::vector<BatchResult> out;
  for (auto it = reqs_.begin(); it != reqs_.end() && out.size() < max;) {
    if (it->second.state == kDone) {
      out.push_back(std::move(it->second.result));
      it = reqs_.erase(it);
    } else {
      ++it;
    }
  }
  return out;
}

BatchInfo BatchServer::info() const {
  std::lock_guard<std::mutex> lock(m_);
  BatchInfo b = stats_;
  b.budget = budget_;
  return b;
}

}  // namespace gb
}  // namespace pps
