// Compressed solution rows (see rowcodec.h): one warp per action row finds
// the row's largest magnitude (a fixed xor tree, so the scale does not
// depend on scheduling) and converts the row to 16-bit codes; decoding is
// the same walk backwards. Both are HBM-bound streams over the rows.
#include "rowcodec.h"

#include <string>

#include "plan.cuh"

namespace pps {
namespace gb {

namespace {

constexpr int kCodecWarps = 8;  // rows per CTA

__global__ void __launch_bounds__(32 * kCodecWarps)
packRowsK(const float* __restrict__ rows, const RowRef* __restrict__ tab, int nRows, int sgn,
          uint16_t* __restrict__ codes, float* __restrict__ scales) {
  const int w = blockIdx.x * kCodecWarps + (int)(threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= nRows) return;
  const RowRef r = tab[w];
  const float* x = rows + r.src;
  float m = 0.f;
  for (int c = lane; c < r.n; c += 32) m = fmaxf(m, fabsf(x[c]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) scales[w] = m;
  const float q = sgn ? 32767.f : 65535.f;
  const float k = m > 0.f ? q / m : 0.f;
  const int lo = sgn ? -32767 : 0, hi = sgn ? 32767 : 65535;
  uint16_t* out = codes + r.dst;
  for (int c = lane; c < r.n; c += 32) {
    int v = __float2int_rn(x[c] * k);
    v = v < lo ? lo : (v > hi ? hi : v);
    out[c] = (uint16_t)(v & 0xffff);
  }
}

__global__ void __launch_bounds__(32 * kCodecWarps)
unpackRowsK(float* __restrict__ rows, const RowRef* __restrict__ tab, int nRows, int sgn,
            const uint16_t* __restrict__ codes, const float* __restrict__ scales) {
  const int w = blockIdx.x * kCodecWarps + (int)(threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= nRows) return;
  const RowRef r = tab[w];
  const float step = scales[w] / (sgn ? 32767.f : 65535.f);
  const uint16_t* in = codes + r.dst;
  float* x = rows + r.src;
  for (int c = lane; c < r.n; c += 32) {
    const float v = sgn ? (float)(int16_t)in[c] : (float)in[c];
    x[c] = v * step;
  }
}

// Device scratch of one codec call, released on every path.
struct CodecScratch {
  void* p[3] = {nullptr, nullptr, nullptr};
  ~CodecScratch() {
    for (void* q : p)
      if (q) cudaFree(q);
  }
};

unsigned codecGrid(size_t rows) { return (unsigned)((rows + kCodecWarps - 1) / kCodecWarps); }

}  // namespace

void packRows(const float* dRows, const std::vector<RowRef>& table, int64_t dense,
              bool signedRows, cudaStream_t s, std::vector<uint16_t>& codes,
              std::vector<float>& scales) {
  codes.assign((size_t)dense, 0);
  scales.assign(table.size(), 0.f);
  if (table.empty()) return;
  if (table.size() > (size_t)(1 << 30)) throw Error{PPS_GB_E_MEMORY, "row table too large"};
  CodecScratch m;
  GB_CK(cudaMalloc(&m.p[0], table.size() * sizeof(RowRef)));
  GB_CK(cudaMalloc(&m.p[1], (size_t)dense * sizeof(uint16_t)));
  GB_CK(cudaMalloc(&m.p[2], table.size() * sizeof(float)));
  GB_CK(cudaMemcpyAsync(m.p[0], table.data(), table.size() * sizeof(RowRef),
                        cudaMemcpyHostToDevice, s));
  packRowsK<<<codecGrid(table.size()), 32 * kCodecWarps, 0, s>>>(
      dRows, static_cast<const RowRef*>(m.p[0]), (int)table.size(), signedRows ? 1 : 0,
      static_cast<uint16_t*>(m.p[1]), static_cast<float*>(m.p[2]));
  GB_CK(cudaGetLastError());
  GB_CK(cudaMemcpyAsync(codes.data(), m.p[1], (size_t)dense * sizeof(uint16_t),
                        cudaMemcpyDeviceToHost, s));
  GB_CK(cudaMemcpyAsync(scales.data(), m.p[2], table.size() * sizeof(float),
                        cudaMemcpyDeviceToHost, s));
  GB_CK(cudaStreamSynchronize(s));
}

void unpackRows(float* dRows, const std::vector<RowRef>& table, bool signedRows,
                const std::vector<uint16_t>& codes, const std::vector<float>& scales,
                cudaStream_t s) {
  if (table.empty()) return;
  if (scales.size() != table.size()) throw Error{PPS_GB_E_ARG, "one scale per row expected"};
  for (const RowRef& r : table)
    if (r.n < 0 || r.dst < 0 || r.dst + r.n > (int64_t)codes.size())
      throw Error{PPS_GB_E_ARG, "row table does not match the codes"};
  CodecScratch m;
  GB_CK(cudaMalloc(&m.p[0], table.size() * sizeof(RowRef)));
  GB_CK(cudaMalloc(&m.p[1], codes.size() * sizeof(uint16_t)));
  GB_CK(cudaMalloc(&m.p[2], scales.size() * sizeof(float)));
  GB_CK(cudaMemcpyAsync(m.p[0], table.data(), table.size() * sizeof(RowRef),
                        cudaMemcpyHostToDevice, s));
  GB_CK(cudaMemcpyAsync(m.p[1], codes.data(), codes.size() * sizeof(uint16_t),
                        cudaMemcpyHostToDevice, s));
  GB_CK(cudaMemcpyAsync(m.p[2], scales.data(), scales.size() * sizeof(float),
                        cudaMemcpyHostToDevice, s));
  unpackRowsK<<<codecGrid(table.size()), 32 * kCodecWarps, 0, s>>>(
      dRows, static_cast<const RowRef*>(m.p[0]), (int)table.size(), signedRows ? 1 : 0,
      static_cast<const uint16_t*>(m.p[1]), static_cast<const float*>(m.p[2]));
  GB_CK(cudaGetLastError());
  GB_CK(cudaStreamSynchronize(s));
}

}  // namespace gb
}  // namespace pps
