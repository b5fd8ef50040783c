// Depth-level DCFR kernels for sm_103a.
//
// One DCFR half-step for traverser tr (the reference's halfStep,
// cuda/gpu_cfr.cu:797-828) is a top-down forward pass (fwdLevelK per depth:
// opponent reach times the opponent's strategy; chance compaction) and a
// bottom-up backward pass (bwdLevelK per depth: showdown, fold, chance sum,
// decide value and the DCFR regret/strategy update).
//
// Work is split into warp-sized tasks, one 32-bit task word each:
//   bits 0-1 kind, bits 2-7 sub (quad chunk or chance branch), bits 8-31 node.
// Forward kinds: 0 = decide chunk (128 row quads), 1 = chance branch.
// Backward kinds: 0 = decide chunk, 1 = chance chunk (128 quads),
// 2 = fold node, 3 = showdown node (one warp per terminal node). A CTA is
// kWarps warps; each warp takes tasks independently, so there is no
// block-wide barrier on the hot path.
//
// Rows are 16-byte-aligned quads (4 floats or 4 doubles) with zero padding.
// T is the value type of reach and cfv rows: float for CFR iterations,
// double for the value / best-response walks; regret and strategy rows are
// always float. No atomics: every sum has a fixed order (deterministic).
#pragma once

#include <cstdint>

#include "layout.h"

namespace pps {
namespace gb {

constexpr int kWarps = 4;              // warps per CTA
constexpr int kThreads = kWarps * 32;  // threads per CTA
constexpr int kRegNa = 8;              // actions kept in registers

struct DevTree {
  const NodeDev* nodes;
  const RowDev* rows;
  const float* termVal;
  const int* children;
  const StateDev* states;
  const uint8_t* poolU8;
  const uint16_t* poolU16;
  const int16_t* poolI16;
  const ShowdownInfo* poolSd;
  float* regret;
  float* strat;
  const float* coef;     // 3 floats per iteration: pos, neg, avg
  const int* counter;    // current iteration index
};

template <typename T>
struct DevRows {
  T* reach[2];
  T* cfv;
};

__device__ __forceinline__ int nodeKind(int meta) { return meta & 3; }
__device__ __forceinline__ int nodePlayer(int meta) { return (meta >> 2) & 1; }
__device__ __forceinline__ int nodeCount(int meta) { return (meta >> 8) & 0xff; }
__device__ __forceinline__ int quadsOf(int n) { return (n + 3) >> 2; }

// ---- quad load/store ----
__device__ __forceinline__ void ldq(const float* p, float (&x)[4]) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
}
__device__ __forceinline__ void stq(float* p, const float (&x)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(x[0], x[1], x[2], x[3]);
}
__device__ __forceinline__ void ldq(const double* p, double (&x)[4]) {
  const double2 a = reinterpret_cast<const double2*>(p)[0];
  const double2 b = reinterpret_cast<const double2*>(p)[1];
  x[0] = a.x; x[1] = a.y; x[2] = b.x; x[3] = b.y;
}
__device__ __forceinline__ void stq(double* p, const double (&x)[4]) {
  reinterpret_cast<double2*>(p)[0] = make_double2(x[0], x[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(x[2], x[3]);
}
template <typename T>
__device__ __forceinline__ void ldqf(const float* p, T (&x)[4]) {
  float f[4];
  ldq(p, f);
  for (int l = 0; l < 4; ++l) x[l] = (T)f[l];
}

// Strategy of one combo from its action rows: regret matching+ over the
// cumulative regrets (sigSrc 0) or the normalized average strategy
// (sigSrc 1); the reference's arithmetic, cuda/gpu_cfr.cu:245-262.
template <typename T>
__device__ __forceinline__ T sigmaOf(T x, T acc, T uniform, int sigSrc) {
  if (sigSrc == 0) return acc > T(0) ? (x > T(0) ? x / acc : T(0)) : uniform;
  return acc > T(0) ? x / acc : uniform;
}
template <typename T>
__device__ __forceinline__ T sigmaMass(T x, int sigSrc) {
  return sigSrc == 0 ? (x > T(0) ? x : T(0)) : x;
}

template <typename T>
__device__ __forceinline__ T warpSum(T v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

template <typename T>
__device__ __forceinline__ T warpInclScan(T v, int lane) {
  for (int off = 1; off < 32; off <<= 1) {
    const T u = __shfl_up_sync(0xffffffffu, v, off);
    if (lane >= off) v += u;
  }
  return v;
}

// Error-free a + b = s + e (Knuth TwoSum).
template <typename T>
__device__ __forceinline__ void twoSum(T a, T b, T& s, T& e) {
  s = a + b;
  const T bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (hi, lo) += b, renormalized (compensated accumulation).
template <typename T>
__device__ __forceinline__ void addComp(T& hi, T& lo, T b) {
  T s, e;
  twoSum(hi, b, s, e);
  e += lo;
  hi = s + e;
  lo = e - (hi - s);
}

// ---------------------------------------------------------------------------
// Forward pass (one launch per depth level).
// ---------------------------------------------------------------------------

template <typename T>
__device__ void fwdDecideChunk(const DevTree& t, const DevRows<T>& rows, int u, int chunk,
                               int tr, int sigSrc, int lane) {
  const NodeDev nd = t.nodes[u];
  const int na = nodeCount(nd.meta);
  const int n = t.states[nd.state].n[1 - tr];
  const int nq = quadsOf(n);
  const float* src = (sigSrc == 0 ? t.regret : t.strat) + (size_t)nd.regQ * 4;
  const T* r = rows.reach[tr] + (size_t)t.rows[u].reachQ[tr] * 4;
  const int* kids = t.children + nd.childBase;
  const T uniform = T(1) / T(na);
  const int q1 = min(nq, (chunk + 1) * kChunkQuads);
  for (int q = chunk * kChunkQuads + lane; q < q1; q += 32) {
    T rr[4], acc[4] = {T(0), T(0), T(0), T(0)};
    ldq(r + 4 * q, rr);
    if (na <= kRegNa) {
      T x[kRegNa][4];
#pragma unroll
      for (int a = 0; a < kRegNa; ++a)
        if (a < na) {
          ldqf(src + ((size_t)a * nq + q) * 4, x[a]);
          for (int l = 0; l < 4; ++l) acc[l] += sigmaMass(x[a][l], sigSrc);
        }
#pragma unroll
      for (int a = 0; a < kRegNa; ++a)
        if (a < na) {
          T out[4];
          for (int l = 0; l < 4; ++l)
            out[l] = 4 * q + l < n ? rr[l] * sigmaOf(x[a][l], acc[l], uniform, sigSrc) : T(0);
          stq(rows.reach[tr] + (size_t)t.rows[kids[a]].reachQ[tr] * 4 + 4 * q, out);
        }
    } else {
      for (int a = 0; a < na; ++a) {
        T x[4];
        ldqf(src + ((size_t)a * nq + q) * 4, x);
        for (int l = 0; l < 4; ++l) acc[l] += sigmaMass(x[l], sigSrc);
      }
      for (int a = 0; a < na; ++a) {
        T x[4], out[4];
        ldqf(src + ((size_t)a * nq + q) * 4, x);
        for (int l = 0; l < 4; ++l)
          out[l] = 4 * q + l < n ? rr[l] * sigmaOf(x[l], acc[l], uniform, sigSrc) : T(0);
        stq(rows.reach[tr] + (size_t)t.rows[kids[a]].reachQ[tr] * 4 + 4 * q, out);
      }
    }
  }
}

// Chance branch: the child's opponent reach row is the parent's, compacted
// through the child's slot map and scaled by the pair-conditional deal
// probability 1 / (52 - nBoard - 4) (cuda/gpu_cfr.cu:276-293).
template <typename T>
__device__ void fwdChanceBranch(const DevTree& t, const DevRows<T>& rows, int u, int br,
                                int tr, int lane) {
  const int opp = 1 - tr;
  const int child = t.children[t.nodes[u].childBase + br];
  const StateDev& cs = t.states[t.nodes[child].state];
  const int nc = cs.n[opp];
  const uint16_t* up = t.poolU16 + cs.upOff[opp];
  const RowDev ru = t.rows[u];
  const T inv = T(1) / T(ru.chanceQ);
  const T* pr = rows.reach[tr] + (size_t)ru.reachQ[tr] * 4;
  T* cr = rows.reach[tr] + (size_t)t.rows[child].reachQ[tr] * 4;
  for (int q = lane; q < quadsOf(nc); q += 32) {
    T out[4];
    for (int l = 0; l < 4; ++l) {
      const int j = 4 * q + l;
      out[l] = j < nc ? pr[up[j]] * inv : T(0);
    }
    stq(cr + 4 * q, out);
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
fwdLevelK(DevTree t, DevRows<T> rows, const int* __restrict__ tasks, int count, int tr,
          int sigSrc) {
  const int lane = threadIdx.x & 31;
  for (int i = blockIdx.x * kWarps + (threadIdx.x >> 5); i < count; i += gridDim.x * kWarps) {
    const int w = tasks[i];
    const int node = w >> 8, sub = (w >> 2) & 63;
    if ((w & 3) == kTaskDecide) fwdDecideChunk<T>(t, rows, node, sub, tr, sigSrc, lane);
    else fwdChanceBranch<T>(t, rows, node, sub, tr, lane);
  }
}

// ---------------------------------------------------------------------------
// Backward pass (one launch per depth level).
// ---------------------------------------------------------------------------

// Per-warp shared scratch of the terminal tasks, for lists of up to maxN
// combos: s_local [maxN + 32], block prefix pairs bh/bl [maxN/32 + 2] each,
// card-segment scans X [2 maxN + 52], segment starts [53].
template <typename T>
struct WarpScratch {
  T* sl;
  T* bh;
  T* bl;
  T* X;
  int* seg;
};

__host__ __device__ inline int scratchBlocks(int maxN) { return maxN / 32 + 2; }

template <typename T>
__host__ __device__ inline size_t warpScratchBytes(int maxN) {
  const size_t elems = (size_t)(maxN + 32) + 2 * (size_t)scratchBlocks(maxN) +
                       2 * (size_t)maxN + 52;
  return ((elems * sizeof(T) + 53 * sizeof(int)) + 15) / 16 * 16;
}

template <typename T>
__device__ WarpScratch<T> warpScratch(unsigned char* smem, int warp, int maxN) {
  unsigned char* base = smem + (size_t)warp * warpScratchBytes<T>(maxN);
  WarpScratch<T> s;
  s.sl = reinterpret_cast<T*>(base);
  s.bh = s.sl + maxN + 32;
  s.bl = s.bh + scratchBlocks(maxN);
  s.X = s.bl + scratchBlocks(maxN);
  s.seg = reinterpret_cast<int*>(s.X + 2 * maxN + 52);
  return s;
}

// Showdown (one warp per node): combo i wins against opponents strictly
// weaker, ties the equal band, loses to the rest (payoffs as
// cuda/gpu_cfr.cu:356-406). Band masses come from an exclusive prefix of the
// strength-sorted opponent reach, kept as a compensated (hi, lo) prefix per
// 32-entry block plus a block-local offset. Opponents sharing a card with i
// are removed with per-card exclusive scans (X) at precomputed counts; the
// identical combo (in the tie band, removed twice) is added back once.
template <typename T>
__device__ void showdownTask(const DevTree& t, const DevRows<T>& rows, int u, int tr,
                             int lane, const WarpScratch<T>& ws) {
  const NodeDev nd = t.nodes[u];
  const StateDev& st = t.states[nd.state];
  const int opp = 1 - tr;
  const int no = st.n[opp], nt = st.n[tr];
  const uint16_t* ord = t.poolU16 + st.sdOff[tr];
  const uint16_t* segStart = ord + no;
  const uint16_t* segSlot = segStart + 53;
  const ShowdownInfo* info = t.poolSd + st.sdInfoOff[tr];
  const RowDev ru = t.rows[u];
  const T* r = rows.reach[tr] + (size_t)ru.reachQ[tr] * 4;

  for (int c = lane; c < 53; c += 32) ws.seg[c] = segStart[c];
  // Sorted prefix: 32-entry blocks, block prefixes accumulated compensated.
  T runHi = T(0), runLo = T(0);
  for (int b = 0; b <= (no >> 5); ++b) {
    const int k = (b << 5) + lane;
    const T v = k < no ? r[ord[k]] : T(0);
    const T incl = warpInclScan(v, lane);
    T excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = T(0);
    ws.sl[k] = excl;
    if (lane == 0) {
      ws.bh[b] = runHi;
      ws.bl[b] = runLo;
    }
    addComp(runHi, runLo, __shfl_sync(0xffffffffu, incl, 31));
  }
  __syncwarp();
  // Card segments: X[seg[c] + c + k] = reach of the first k entries.
  for (int c = 0; c < 52; ++c) {
    const int s0 = ws.seg[c], len = ws.seg[c + 1] - s0;
    T* xo = ws.X + s0 + c;
    const int e0 = 2 * lane, e1 = e0 + 1;
    const T v0 = e0 < len ? r[segSlot[s0 + e0]] : T(0);
    const T v1 = e1 < len ? r[segSlot[s0 + e1]] : T(0);
    const T incl = warpInclScan(v0 + v1, lane);
    const T excl = incl - (v0 + v1);
    if (e0 <= len) xo[e0] = excl;
    if (e1 <= len) xo[e1] = excl + v0;
  }
  __syncwarp();

  const float* tv = t.termVal + ((size_t)u * 2 + tr) * 4;
  const T winV = (T)tv[0], tieV = (T)tv[1], loseV = (T)tv[2];
  T* out = rows.cfv + (size_t)ru.cfvQ * 4;
  const int nt4 = quadsOf(nt) * 4;
  const int bn = no >> 5;
  for (int i = lane; i < nt4; i += 32) {
    if (i >= nt) {
      out[i] = T(0);
      continue;
    }
    const ShowdownInfo f = info[i];
    const int le = f.x & 0xffff, te = f.x >> 16;
    const int c1 = f.y & 0xff, c2 = (f.y >> 8) & 0xff;
    const int a1 = ws.seg[c1] + c1, a2 = ws.seg[c2] + c2;
    const int len1 = ws.seg[c1 + 1] - ws.seg[c1], len2 = ws.seg[c2 + 1] - ws.seg[c2];
    const T x1le = ws.X[a1 + ((f.y >> 16) & 0xff)], x1te = ws.X[a1 + (f.y >> 24)];
    const T x2le = ws.X[a2 + (f.z & 0xff)], x2te = ws.X[a2 + ((f.z >> 8) & 0xff)];
    const int same = (int)(f.z >> 16) - 1;
    const T sameR = same >= 0 ? r[same] : T(0);
    const int bl = le >> 5, bt = te >> 5;
    const T below = ws.bh[bl] + (ws.bl[bl] + ws.sl[le]);
    const T band = (ws.bh[bt] - ws.bh[bl]) + (ws.bl[bt] - ws.bl[bl]) + (ws.sl[te] - ws.sl[le]);
    const T above = (ws.bh[bn] - ws.bh[bt]) + (ws.bl[bn] - ws.bl[bt]) + (ws.sl[no] - ws.sl[te]);
    T lm = below - x1le - x2le;
    T tm = band - (x1te - x1le) - (x2te - x2le) + sameR;
    T gm = above - (ws.X[a1 + len1] - x1te) - (ws.X[a2 + len2] - x2te);
    lm = lm > T(0) ? lm : T(0);
    tm = tm > T(0) ? tm : T(0);
    gm = gm > T(0) ? gm : T(0);
    out[i] = lm * winV + tm * tieV + gm * loseV;
  }
  __syncwarp();
}

// Fold (one warp per node): every opponent combo not sharing a card with i
// pays (cuda/gpu_cfr.cu:409-455); per-card sums over the card lists, one
// card per lane, fixed order (no atomics).
template <typename T>
__device__ void foldTask(const DevTree& t, const DevRows<T>& rows, int u, int tr, int lane,
                         const WarpScratch<T>& ws) {
  const NodeDev nd = t.nodes[u];
  const StateDev& st = t.states[nd.state];
  const int opp = 1 - tr;
  const int no = st.n[opp], nt = st.n[tr];
  const RowDev ru = t.rows[u];
  const T* r = rows.reach[tr] + (size_t)ru.reachQ[tr] * 4;
  const uint16_t* csr = t.poolU16 + st.csrOff[opp];
  T* cs = ws.X;  // [52]
  for (int c = lane; c < 52; c += 32) {
    const int s0 = csr[c], s1 = csr[c + 1];
    T a0 = T(0), a1 = T(0);
    int e = s0;
    for (; e + 1 < s1; e += 2) {
      a0 += r[csr[53 + e]];
      a1 += r[csr[54 + e]];
    }
    if (e < s1) a0 += r[csr[53 + e]];
    cs[c] = a0 + a1;
  }
  T part = T(0);
  for (int j = lane; j < no; j += 32) part += r[j];
  const T tot = warpSum(part);
  __syncwarp();
  const T v = (T)t.termVal[((size_t)u * 2 + tr) * 4];
  const uint8_t* cards = t.poolU8 + st.cardsOff[tr];
  const int16_t* same = t.poolI16 + st.sameOff[tr];
  T* out = rows.cfv + (size_t)ru.cfvQ * 4;
  const int nt4 = quadsOf(nt) * 4;
  for (int i = lane; i < nt4; i += 32) {
    if (i >= nt) {
      out[i] = T(0);
      continue;
    }
    T w = tot - cs[cards[2 * i]] - cs[cards[2 * i + 1]];
    const int s = same[i];
    if (s >= 0) w += r[s];
    if (w < T(0)) w = T(0);
    out[i] = w * v;
  }
  __syncwarp();
}

// Chance chunk: the parent's value of combo i sums the children's values
// over the branches it survives, in branch order (cuda/gpu_cfr.cu:529-555).
template <typename T>
__device__ void chanceChunk(const DevTree& t, const DevRows<T>& rows, int u, int chunk,
                            int tr, int lane) {
  const NodeDev nd = t.nodes[u];
  const int nb = nodeCount(nd.meta);
  const int nt = t.states[nd.state].n[tr];
  T* out = rows.cfv + (size_t)t.rows[u].cfvQ * 4;
  const int i0 = chunk * kChunkQuads * 4;
  const int i1 = min(quadsOf(nt) * 4, i0 + kChunkQuads * 4);
  for (int i = i0 + lane; i < i1; i += 32) {
    T v = T(0);
    if (i < nt)
      for (int b = 0; b < nb; ++b) {
        const int ch = t.children[nd.childBase + b];
        const int k = t.poolI16[t.states[t.nodes[ch].state].downOff[tr] + i];
        if (k >= 0) v += rows.cfv[(size_t)t.rows[ch].cfvQ * 4 + k];
      }
    out[i] = v;
  }
}

// Decide chunk. Opponent node: the traverser's value sums the children.
// Traverser node, CFR: regret-matching+ strategy from the pre-update
// regrets, the node value, then the DCFR update (cuda/gpu_cfr.cu:479-523)
//   strat = strat * avg + sigma
//   regret = regret * (regret >= 0 ? pos : neg) + (cfv_a - value).
// EV: the average strategy's value. BR: the best action's value.
template <typename T>
__device__ void decideChunk(const DevTree& t, const DevRows<T>& rows, int u, int chunk, int tr,
                            int mode, int lane) {
  const NodeDev nd = t.nodes[u];
  const int na = nodeCount(nd.meta);
  const int n = t.states[nd.state].n[tr];
  const int nq = quadsOf(n);
  const int* kids = t.children + nd.childBase;
  T* out = rows.cfv + (size_t)t.rows[u].cfvQ * 4;
  const int q1 = min(nq, (chunk + 1) * kChunkQuads);
  if (nodePlayer(nd.meta) != tr || mode == kModeBR) {
    const bool best = nodePlayer(nd.meta) == tr;
    for (int q = chunk * kChunkQuads + lane; q < q1; q += 32) {
      T v[4];
      for (int l = 0; l < 4; ++l) v[l] = best ? T(-1e30) : T(0);
      for (int a = 0; a < na; ++a) {
        T c[4];
        ldq(rows.cfv + (size_t)t.rows[kids[a]].cfvQ * 4 + 4 * q, c);
        for (int l = 0; l < 4; ++l) v[l] = best ? (c[l] > v[l] ? c[l] : v[l]) : v[l] + c[l];
      }
      for (int l = 0; l < 4; ++l)
        if (4 * q + l >= n) v[l] = T(0);
      stq(out + 4 * q, v);
    }
    return;
  }
  float* reg = t.regret + (size_t)nd.regQ * 4;
  float* str = t.strat + (size_t)nd.regQ * 4;
  const float* src = mode == kModeCFR ? reg : str;
  const int sigSrc = mode == kModeCFR ? 0 : 1;
  const T uniform = T(1) / T(na);
  float pos = 0.f, neg = 0.f, avg = 0.f;
  if (mode == kModeCFR) {
    const float* c = t.coef + (size_t)(*t.counter) * 3;
    pos = c[0];
    neg = c[1];
    avg = c[2];
  }
  for (int q = chunk * kChunkQuads + lane; q < q1; q += 32) {
    bool live[4];
    for (int l = 0; l < 4; ++l) live[l] = 4 * q + l < n;
    T val[4] = {T(0), T(0), T(0), T(0)}, acc[4] = {T(0), T(0), T(0), T(0)};
    if (na <= kRegNa) {
      T x[kRegNa][4], cv[kRegNa][4];
#pragma unroll
      for (int a = 0; a < kRegNa; ++a)
        if (a < na) {
          ldqf(src + ((size_t)a * nq + q) * 4, x[a]);
          ldq(rows.cfv + (size_t)t.rows[kids[a]].cfvQ * 4 + 4 * q, cv[a]);
          for (int l = 0; l < 4; ++l) acc[l] += sigmaMass(x[a][l], sigSrc);
        }
#pragma unroll
      for (int a = 0; a < kRegNa; ++a)
        if (a < na)
          for (int l = 0; l < 4; ++l) {
            x[a][l] = live[l] ? sigmaOf(x[a][l], acc[l], uniform, sigSrc) : T(0);
            val[l] += x[a][l] * cv[a][l];
          }
      stq(out + 4 * q, val);
      if (mode != kModeCFR) continue;
#pragma unroll
      for (int a = 0; a < kRegNa; ++a)
        if (a < na) {
          float rg[4], sg[4];
          const size_t o = ((size_t)a * nq + q) * 4;
          ldq(reg + o, rg);
          ldq(str + o, sg);
          for (int l = 0; l < 4; ++l) {
            sg[l] = sg[l] * avg + (float)x[a][l];
            rg[l] = rg[l] * (rg[l] >= 0.0f ? pos : neg) + (float)(cv[a][l] - val[l]);
          }
          stq(str + o, sg);
          stq(reg + o, rg);
        }
    } else {
      for (int a = 0; a < na; ++a) {
        T x[4];
        ldqf(src + ((size_t)a * nq + q) * 4, x);
        for (int l = 0; l < 4; ++l) acc[l] += sigmaMass(x[l], sigSrc);
      }
      for (int a = 0; a < na; ++a) {
        T x[4], c[4];
        ldqf(src + ((size_t)a * nq + q) * 4, x);
        ldq(rows.cfv + (size_t)t.rows[kids[a]].cfvQ * 4 + 4 * q, c);
        for (int l = 0; l < 4; ++l)
          val[l] += (live[l] ? sigmaOf(x[l], acc[l], uniform, sigSrc) : T(0)) * c[l];
      }
      stq(out + 4 * q, val);
      if (mode != kModeCFR) continue;
      for (int a = 0; a < na; ++a) {
        float rg[4], sg[4];
        T c[4];
        const size_t o = ((size_t)a * nq + q) * 4;
        ldq(reg + o, rg);
        ldq(str + o, sg);
        ldq(rows.cfv + (size_t)t.rows[kids[a]].cfvQ * 4 + 4 * q, c);
        for (int l = 0; l < 4; ++l) {
          const T s = live[l] ? sigmaOf((T)rg[l], acc[l], uniform, 0) : T(0);
          sg[l] = sg[l] * avg + (float)s;
          rg[l] = rg[l] * (rg[l] >= 0.0f ? pos : neg) + (float)(c[l] - val[l]);
        }
        stq(str + o, sg);
        stq(reg + o, rg);
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
bwdLevelK(DevTree t, DevRows<T> rows, const int* __restrict__ tasks, int count, int tr,
          int mode, int maxN) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const WarpScratch<T> ws = warpScratch<T>(smem, warp, maxN);
  for (int i = blockIdx.x * kWarps + warp; i < count; i += gridDim.x * kWarps) {
    const int w = tasks[i];
    const int node = w >> 8, sub = (w >> 2) & 63;
    switch (w & 3) {
      case kTaskShowdown: showdownTask<T>(t, rows, node, tr, lane, ws); break;
      case kTaskFold: foldTask<T>(t, rows, node, tr, lane, ws); break;
      case kTaskChance: chanceChunk<T>(t, rows, node, sub, tr, lane); break;
      default: decideChunk<T>(t, rows, node, sub, tr, mode, lane);
    }
  }
}

__global__ void advanceCounterK(int* counter) {
  if (threadIdx.x == 0 && blockIdx.x == 0) ++(*counter);
}

}  // namespace gb
}  // namespace pps
