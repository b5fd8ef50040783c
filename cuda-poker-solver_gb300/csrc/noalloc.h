// No-allocation DCFR solve over caller-owned rows (noalloc.cu); backs
// pps_gb_solve_noalloc. Throws gb::Error.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gpu_cfr.h"

namespace pps {
namespace gb {

// Runs `iterations` DCFR iterations (absolute indices firstIteration ..)
// over the caller's dense regret/strategy rows; returns the row count.
int64_t noallocSolve(const gpu::PostflopSpot& spot, const pf::BetConfig& cfg, float* dRegret,
                     float* dStrat, int64_t rowCapacity, int firstIteration, int iterations,
                     cudaStream_t stream);

}  // namespace gb
}  // namespace pps
