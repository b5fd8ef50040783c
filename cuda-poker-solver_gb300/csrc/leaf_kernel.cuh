// Fused leaf-street iteration kernel (plan + launch). Placeholder plan:
// not applicable, so the engine uses the depth-level kernels only.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "compiler.h"
#include "kernels.cuh"
#include "layout.h"

namespace pps {
namespace gb {

struct ListRef {
  int off = 0, count = 0;
};

struct LeafPlan {
  bool ok = false;
  int rootDepthMin = 0;
  std::vector<ListRef> upperBwd;
  float* scratch = nullptr;
  size_t scratchFloats = 0;
  size_t smemBytes = 0;
};

__global__ void leafK() {}

inline LeafPlan planLeaf(const Tree&, const HostLayout&, std::vector<int>&) {
  return LeafPlan{};
}

inline int launchLeaf(const LeafPlan&, const DevTree&, const DevRows<float>&,
                      const int*, int, cudaStream_t) {
  return 0;
}

}  // namespace gb
}  // namespace pps
