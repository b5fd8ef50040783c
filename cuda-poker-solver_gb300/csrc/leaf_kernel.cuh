// Fused leaf-street iteration kernel: plan + launch interface.
// (Not applicable yet: the plan reports ok = false and the engine runs the
// depth-level kernels.)
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <vector>

#include "compiler.h"
#include "kernels.cuh"
#include "layout.h"
#include "plan.cuh"

namespace pps {
namespace gb {

struct LeafPlan {
  bool ok = false;
  // Level task lists of the nodes above the leaf street, per traverser.
  std::vector<std::vector<int>> fwdTasks[2], bwdTasks[2];
  std::vector<ListRef> fwd[2], bwd[2];
  double algoBytes[2] = {0.0, 0.0};  // per traverser launch
};

inline LeafPlan planLeaf(const Tree&, const HostLayout&, std::vector<int>&) { return LeafPlan{}; }

inline void finishLeaf(LeafPlan&, const int*, const std::function<float*(size_t)>&) {}

inline cudaError_t prepareLeaf(LeafPlan&) { return cudaSuccess; }

inline void launchLeaf(const LeafPlan&, const DevTree&, const DevRows<float>&, int,
                       cudaStream_t) {}

}  // namespace gb
}  // namespace pps
