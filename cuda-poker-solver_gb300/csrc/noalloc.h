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
// *needRows (if given) receives the row count as soon as the spot is
// compiled, so it is set on the capacity and budget errors too.
int64_t noallocSolve(const gpu::PostflopSpot& spot, const pf::BetConfig& cfg, float* dRegret,
                     float* dStrat, int64_t rowCapacity, int firstIteration, int iterations,
                     cudaStream_t stream, int64_t* needRows);

}  // namespace gb
}  // namespace pps
