// Compressed solution rows: each action row (one decide node's row of one
// action, n combos) is stored as 16-bit codes with one f32 scale, the
// row's largest magnitude. Regret rows use signed codes (x = code * m /
// 32767), strategy rows unsigned ones (x = code * m / 65535), so an entry
// is off by at most half a step of its row's scale. The codes are made and
// read on the device; only codes and scales cross to the host.
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace pps {
namespace gb {

// One action row: its first entry in the padded device rows (floats), its
// first entry in the dense layout (the file's order), its length.
struct RowRef {
  int64_t src;
  int64_t dst;
  int32_t n;
  int32_t pad;
};

// Codes of `dense` entries (the dense layout) and one scale per row.
void packRows(const float* dRows, const std::vector<RowRef>& table, int64_t dense,
              bool signedRows, cudaStream_t s, std::vector<uint16_t>& codes,
              std::vector<float>& scales);

// Writes the decoded rows into the padded device rows (entries the table
// does not cover are left as they are).
void unpackRows(float* dRows, const std::vector<RowRef>& table, bool signedRows,
                const std::vector<uint16_t>& codes, const std::vector<float>& scales,
                cudaStream_t s);

}  // namespace gb
}  // namespace pps
