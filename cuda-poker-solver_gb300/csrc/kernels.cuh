// Depth-level DCFR kernels for sm_103a.
//
// One DCFR half-step for traverser tr (the reference's halfStep,
// cuda/gpu_cfr.cu:797-828) is a top-down forward pass (fwdLevelK per depth:
// opponent reach times the opponent's strategy; chance compaction) and a
// bottom-up backward pass (bwdLevelK per depth: showdown, fold, chance sum,
// decide value and the DCFR regret/strategy update).
//
// Work is split into CTA-sized tasks, one 32-bit task word each:
//   bits 0-1 kind, bits 2-7 sub (quad chunk or chance branch), bits 8-31 node.
// Forward kinds: 0 = decide chunk (128 row quads, one thread per quad),
// 1 = chance branch. Backward kinds: 0 = decide chunk, 1 = chance chunk,
// 2 = fold node, 3 = showdown node. Task lists put the long terminal tasks
// first. Registers are capped (launch bounds) so that at least 6 CTAs of
// 128 threads share an SM; the terminal tasks' scratch (one reach row plus
// prefix arrays, ~19 KB at 1128 combos) fits that budget.
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

constexpr int kThreads = 128;  // threads per CTA
constexpr int kRegNa = 6;      // actions kept in registers by the decide update

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
  float* stratLo;        // compensated strategy sums: the low words of the
                         // strategy rows (same layout), or nullptr for the
                         // plain f32 sums
  const float* coef;     // 3 floats per iteration: pos, neg, avg
  const int* counter;    // current iteration index, per spot (node meta
                         // bits 16-31; a lone spot is spot 0)
  int* err;              // device error word: a bounded wait gave up (0: none)
};

template <typename T>
struct DevRows {
  T* reach[2];
  T* cfv;
};

__device__ __forceinline__ int nodeKind(int meta) { return meta & 3; }
__device__ __forceinline__ int nodePlayer(int meta) { return (meta >> 2) & 1; }
__device__ __forceinline__ int nodeCount(int meta) { return (meta >> 8) & 0xff; }
__device__ __forceinline__ int nodeSpot(int meta) { return (int)((unsigned)meta >> 16); }
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
// The walks (T = double) normalize with one reciprocal per combo and a
// product per action: an FP64 division is a multi-instruction sequence,
// and GB300's FP64 pipe is what bounds the walks. The f32 iteration keeps
// the reference's x / acc per action (sigmaScale is then unused).
template <typename T>
__device__ __forceinline__ T sigmaScale(T acc) {
  if constexpr (sizeof(T) == 8) return acc > T(0) ? T(1) / acc : T(0);
  else return acc;
}
template <typename T>
__device__ __forceinline__ T sigmaOfScaled(T x, T acc, T scale, T uniform, int sigSrc) {
  if constexpr (sizeof(T) == 8) {
    if (!(acc > T(0))) return uniform;
    return (sigSrc == 0 ? (x > T(0) ? x : T(0)) : x) * scale;
  } else {
    return sigmaOf(x, acc, uniform, sigSrc);
  }
}

// Cumulative-strategy update s <- s * avg + sigma (the reference's
// cuda/gpu_cfr.cu:512-523). Plain: one f32 fma. Compensated: s is carried
// as an unevaluated sum hi + lo of two floats; the rounding error of the
// product (from an fma) and of the sum (Knuth's two-sum) go into lo, and
// the pair is renormalized (Dekker's fast two-sum) so that hi stays the
// sum rounded to f32 - every reader of the strategy rows reads hi alone.
// The _rn intrinsics keep the compiler from contracting the steps.
__device__ __forceinline__ void stratComp(float& hi, float& lo, float avg, float sigma) {
  const float p = __fmul_rn(hi, avg);
  const float ep = __fmaf_rn(hi, avg, -p);
  const float t = __fadd_rn(p, sigma);
  const float bb = __fsub_rn(t, p);
  const float es = __fadd_rn(__fsub_rn(p, __fsub_rn(t, bb)), __fsub_rn(sigma, bb));
  const float l = __fmaf_rn(lo, avg, __fadd_rn(ep, es));
  hi = __fadd_rn(t, l);
  lo = __fsub_rn(l, __fsub_rn(hi, t));
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

// (hi, lo) += (bh, bl), renormalized (double-word addition).
template <typename T>
__device__ __forceinline__ void addPair(T& hi, T& lo, T bh, T bl) {
  T s, e;
  twoSum(hi, bh, s, e);
  e += lo + bl;
  hi = s + e;
  lo = e - (hi - s);
}

// ---------------------------------------------------------------------------
// Forward pass (one launch per depth level; one CTA per task).
// ---------------------------------------------------------------------------

// Opponent decide chunk: child reach = reach x sigma_a, one thread per quad.
template <typename T>
__device__ void fwdDecideChunk(const DevTree& t, const DevRows<T>& rows, int u, int chunk,
                               int tr, int sigSrc) {
  const NodeDev nd = t.nodes[u];
  const int na = nodeCount(nd.meta);
  const int n = t.states[nd.state].n[1 - tr];
  const int nq = quadsOf(n);
  const int q = chunk * kChunkQuads + (int)threadIdx.x;
  if (q >= nq) return;
  const float* src = (sigSrc == 0 ? t.regret : t.strat) + (size_t)nd.regQ * 4;
  const T* r = rows.reach[tr] + (size_t)t.rows[u].reachQ[tr] * 4;
  const int* kids = t.children + nd.childBase;
  const T uniform = T(1) / T(na);
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
    T sc[4];
    for (int l = 0; l < 4; ++l) sc[l] = sigmaScale(acc[l]);
#pragma unroll
    for (int a = 0; a < kRegNa; ++a)
      if (a < na) {
        T out[4];
        for (int l = 0; l < 4; ++l)
          out[l] = 4 * q + l < n ? rr[l] * sigmaOfScaled(x[a][l], acc[l], sc[l], uniform, sigSrc)
                                 : T(0);
        stq(rows.reach[tr] + (size_t)t.rows[kids[a]].reachQ[tr] * 4 + 4 * q, out);
      }
    return;
  }
  for (int a = 0; a < na; ++a) {
    T x[4];
    ldqf(src + ((size_t)a * nq + q) * 4, x);
    for (int l = 0; l < 4; ++l) acc[l] += sigmaMass(x[l], sigSrc);
  }
  T sc[4];
  for (int l = 0; l < 4; ++l) sc[l] = sigmaScale(acc[l]);
  for (int a = 0; a < na; ++a) {
    T x[4], out[4];
    ldqf(src + ((size_t)a * nq + q) * 4, x);
    for (int l = 0; l < 4; ++l)
      out[l] = 4 * q + l < n ? rr[l] * sigmaOfScaled(x[l], acc[l], sc[l], uniform, sigSrc)
                             : T(0);
    stq(rows.reach[tr] + (size_t)t.rows[kids[a]].reachQ[tr] * 4 + 4 * q, out);
  }
}

// Chance branch: the child's opponent reach row is the parent's, compacted
// through the child's slot map and scaled by the pair-conditional deal
// probability 1 / (52 - nBoard - 4) (cuda/gpu_cfr.cu:276-293).
template <typename T>
__device__ void fwdChanceBranch(const DevTree& t, const DevRows<T>& rows, int u, int br,
                                int tr) {
  const int opp = 1 - tr;
  const int child = t.children[t.nodes[u].childBase + br];
  const StateDev& cs = t.states[t.nodes[child].state];
  const int nc = cs.n[opp];
  const uint16_t* up = t.poolU16 + cs.upOff[opp];
  const RowDev ru = t.rows[u];
  const T inv = T(1) / T(ru.chanceQ);
  const T* pr = rows.reach[tr] + (size_t)ru.reachQ[tr] * 4;
  T* cr = rows.reach[tr] + (size_t)t.rows[child].reachQ[tr] * 4;
  for (int q = threadIdx.x; q < quadsOf(nc); q += blockDim.x) {
    T out[4];
    for (int l = 0; l < 4; ++l) {
      const int j = 4 * q + l;
      out[l] = j < nc ? pr[up[j]] * inv : T(0);
    }
    stq(cr + 4 * q, out);
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 6)
fwdLevelK(DevTree t, DevRows<T> rows, const int* __restrict__ tasks, int count, int tr,
          int sigSrc) {
  for (int i = blockIdx.x; i < count; i += gridDim.x) {
    const int w = tasks[i];
    const int node = (int)((unsigned)w >> 8), sub = (w >> 2) & 63;
    if ((w & 3) == kTaskDecide) fwdDecideChunk<T>(t, rows, node, sub, tr, sigSrc);
    else fwdChanceBranch<T>(t, rows, node, sub, tr);
  }
}

// ---------------------------------------------------------------------------
// Backward pass (one launch per depth level; one CTA per task).
// ---------------------------------------------------------------------------

// Shared scratch of the terminal tasks for lists of up to maxN combos:
// staged reach rs [4 quads(maxN)], block-local exclusive prefixes
// sl [maxN + 32], compensated block prefixes bh/bl [maxN/32 + 2] each,
// card-segment scans X [2 maxN + 52], and the node's staged u16 index
// table tab [3 maxN + 64] (showdown: order, segment starts, segment slots;
// fold: card lists).
__host__ __device__ inline int scratchBlocks(int maxN) { return maxN / 32 + 2; }
__host__ __device__ inline int scratchTab(int maxN) { return (3 * maxN + 53 + 7) / 8 * 8 + 8; }

// Chance tasks keep 64 row pointers and 64 slot-map pointers at the start of
// the same scratch (a chance node has at most 49 branches).
constexpr size_t kChanceScratchBytes = 2 * 64 * sizeof(void*);

template <typename T>
__host__ __device__ inline size_t bwdScratchBytes(int maxN) {
  const size_t elems = 4 * (size_t)((maxN + 3) / 4) + (size_t)(maxN + 32) +
                       2 * (size_t)scratchBlocks(maxN) + 2 * (size_t)maxN + 52;
  const size_t valBytes = (elems * sizeof(T) + 15) / 16 * 16;
  const size_t total = valBytes + (size_t)scratchTab(maxN) * sizeof(uint16_t);
  return total > kChanceScratchBytes ? total : kChanceScratchBytes;
}

template <typename T>
struct Scratch {
  T* rs;
  T* sl;
  T* bh;
  T* bl;
  T* X;
  uint16_t* tab;
};

template <typename T>
__device__ Scratch<T> scratchOf(unsigned char* smem, int maxN) {
  Scratch<T> s;
  s.rs = reinterpret_cast<T*>(smem);
  s.sl = s.rs + 4 * ((maxN + 3) / 4);
  s.bh = s.sl + maxN + 32;
  s.bl = s.bh + scratchBlocks(maxN);
  s.X = s.bl + scratchBlocks(maxN);
  const size_t elems = 4 * (size_t)((maxN + 3) / 4) + (size_t)(maxN + 32) +
                       2 * (size_t)scratchBlocks(maxN) + 2 * (size_t)maxN + 52;
  s.tab = reinterpret_cast<uint16_t*>(smem + (elems * sizeof(T) + 15) / 16 * 16);
  return s;
}

// Copies n u16 table entries (16-byte aligned in the pool, which is padded
// to a multiple of 8 entries) into shared memory with 16-byte loads.
__device__ __forceinline__ void stageTab(uint16_t* dst, const uint16_t* src, int n) {
  const uint4* s4 = reinterpret_cast<const uint4*>(src);
  uint4* d4 = reinterpret_cast<uint4*>(dst);
  for (int k = threadIdx.x; k < (n + 7) / 8; k += blockDim.x) d4[k] = s4[k];
}

// Stages row r (n entries, quad padded) into shared memory.
template <typename T>
__device__ __forceinline__ void stageRow(T* dst, const T* r, int n) {
  for (int q = threadIdx.x; q < quadsOf(n); q += blockDim.x) {
    T x[4];
    ldq(r + 4 * q, x);
    for (int l = 0; l < 4; ++l) dst[4 * q + l] = x[l];
  }
}

// Showdown (one CTA per node): combo i wins against opponents strictly
// weaker, ties the equal band, loses to the rest (payoffs as
// cuda/gpu_cfr.cu:356-406). Band masses come from an exclusive prefix of the
// strength-sorted opponent reach: block-local prefixes of 32 entries plus a
// compensated (hi, lo) prefix of the block totals. Opponents sharing a card
// with i are removed with per-card exclusive scans (X) read at precomputed
// counts; the identical combo (in the tie band, removed twice) is added
// back once.
template <typename T>
__device__ void showdownNode(const DevTree& t, const DevRows<T>& rows, int u, int tr,
                             const Scratch<T>& ws) {
  const NodeDev nd = t.nodes[u];
  const StateDev& st = t.states[nd.state];
  const int opp = 1 - tr;
  const int no = st.n[opp], nt = st.n[tr];
  const uint16_t* ord = ws.tab;
  const uint16_t* seg = ord + no;
  const uint16_t* segSlot = seg + 53;
  const ShowdownInfo* info = t.poolSd + st.sdInfoOff[tr];
  const int16_t* sameTab = t.poolI16 + st.sameOff[tr];  // identical combo's opponent slot
  const RowDev ru = t.rows[u];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;

  stageRow(ws.rs, rows.reach[tr] + (size_t)ru.reachQ[tr] * 4, no);
  stageTab(ws.tab, t.poolU16 + st.sdOff[tr], 3 * no + 53);
  __syncthreads();
  // Block-local prefixes of the sorted reach; block totals into bh.
  const int nb = (no >> 5) + 1;
  for (int b = warp; b < nb; b += nw) {
    const int k = (b << 5) + lane;
    const T v = k < no ? ws.rs[ord[k]] : T(0);
    const T incl = warpInclScan(v, lane);
    T excl = __shfl_up_sync(0xffffffffu, incl, 1);
    ws.sl[k] = lane == 0 ? T(0) : excl;
    if (lane == 31) ws.bh[b] = incl;
  }
  // Card segments: X[seg[c] + c + k] = reach of the first k entries.
  for (int c = warp; c < 52; c += nw) {
    const int s0 = seg[c], len = seg[c + 1] - s0;
    T* xo = ws.X + s0 + c;
    const int e0 = 2 * lane, e1 = e0 + 1;
    const T v0 = e0 < len ? ws.rs[segSlot[s0 + e0]] : T(0);
    const T v1 = e1 < len ? ws.rs[segSlot[s0 + e1]] : T(0);
    const T incl = warpInclScan(v0 + v1, lane);
    const T excl = incl - (v0 + v1);
    if (e0 <= len) xo[e0] = excl;
    if (e1 <= len) xo[e1] = excl + v0;
  }
  __syncthreads();
  // Compensated exclusive prefix of the block totals (nb <= 64: two blocks
  // per lane of warp 0). In FP64 (the walks) a plain prefix is exact enough
  // and spares the FP64 pipe.
  if (warp == 0 && sizeof(T) == 8) {
    const int b0 = 2 * lane, b1 = b0 + 1;
    const T t0 = b0 < nb ? ws.bh[b0] : T(0), t1 = b1 < nb ? ws.bh[b1] : T(0);
    const T incl = warpInclScan(t0 + t1, lane);
    T e = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) e = T(0);
    if (b0 < nb) {
      ws.bh[b0] = e;
      ws.bl[b0] = T(0);
    }
    if (b1 < nb) {
      ws.bh[b1] = e + t0;
      ws.bl[b1] = T(0);
    }
  } else if (warp == 0) {
    const int b0 = 2 * lane, b1 = b0 + 1;
    const T t0 = b0 < nb ? ws.bh[b0] : T(0), t1 = b1 < nb ? ws.bh[b1] : T(0);
    T hi = t0, lo = T(0);
    addComp(hi, lo, t1);
    for (int off = 1; off < 32; off <<= 1) {
      const T oh = __shfl_up_sync(0xffffffffu, hi, off);
      const T ol = __shfl_up_sync(0xffffffffu, lo, off);
      if (lane >= off) {
        T h = oh, l = ol;
        addPair(h, l, hi, lo);
        hi = h;
        lo = l;
      }
    }
    T eh = __shfl_up_sync(0xffffffffu, hi, 1), el = __shfl_up_sync(0xffffffffu, lo, 1);
    if (lane == 0) eh = el = T(0);
    if (b0 < nb) {
      ws.bh[b0] = eh;
      ws.bl[b0] = el;
    }
    addComp(eh, el, t0);
    if (b1 < nb) {
      ws.bh[b1] = eh;
      ws.bl[b1] = el;
    }
  }
  __syncthreads();

  const float* tv = t.termVal + ((size_t)u * 2 + tr) * 4;
  const T winV = (T)tv[0], tieV = (T)tv[1], loseV = (T)tv[2];
  T* out = rows.cfv + (size_t)ru.cfvQ * 4;
  const int nt4 = quadsOf(nt) * 4;
  const int bn = no >> 5;
  // Four combos per thread per round: their table entries are loaded first
  // so the loads overlap.
  for (int k0 = threadIdx.x; k0 < nt4; k0 += 4 * blockDim.x) {
    ShowdownInfo fs[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = k0 + j * blockDim.x;
      if (k < nt) fs[j] = info[k];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
    const int k = k0 + j * blockDim.x;
    if (k >= nt4) break;
    if (k >= nt) {
      out[k] = T(0);
      continue;
    }
    // The entry holds the group kernels' padded indices and its combo's
    // offset in its window (layout.h); this kernel's arrays are
    // unpadded.
    const ShowdownInfo f = fs[j];
    const int i = showdownCombo(k, f);
    const int le = unpad8((int)(f.w & 0x7ff)), te = unpad8((int)((f.w >> 11) & 0x7ff));
    const T x1le = ws.X[unpad8((int)(f.x & 0xfff))], x1te = ws.X[unpad8((int)((f.x >> 12) & 0xfff))];
    const T x1end = ws.X[unpad8((int)(f.y & 0xfff))], x2le = ws.X[unpad8((int)((f.y >> 12) & 0xfff))];
    const T x2te = ws.X[unpad8((int)(f.z & 0xfff))], x2end = ws.X[unpad8((int)((f.z >> 12) & 0xfff))];
    const int same = sameTab[i];
    const T sameR = same >= 0 ? ws.rs[same] : T(0);
    const int bl = le >> 5, bt = te >> 5;
    T below, band, above;
    if constexpr (sizeof(T) == 8) {  // plain FP64 prefixes (bl is zero)
      const T ple = ws.bh[bl] + ws.sl[le], pte = ws.bh[bt] + ws.sl[te];
      below = ple;
      band = pte - ple;
      above = (ws.bh[bn] + ws.sl[no]) - pte;
    } else {
      below = ws.bh[bl] + (ws.bl[bl] + ws.sl[le]);
      band = (ws.bh[bt] - ws.bh[bl]) + (ws.bl[bt] - ws.bl[bl]) + (ws.sl[te] - ws.sl[le]);
      above = (ws.bh[bn] - ws.bh[bt]) + (ws.bl[bn] - ws.bl[bt]) + (ws.sl[no] - ws.sl[te]);
    }
    T lm = below - x1le - x2le;
    T tm = band - (x1te - x1le) - (x2te - x2le) + sameR;
    T gm = above - (x1end - x1te) - (x2end - x2te);
    lm = lm > T(0) ? lm : T(0);
    tm = tm > T(0) ? tm : T(0);
    gm = gm > T(0) ? gm : T(0);
    out[i] = lm * winV + tm * tieV + gm * loseV;
    }
  }
}

// Fold (one CTA per node): every opponent combo not sharing a card with i
// pays (cuda/gpu_cfr.cu:409-455); per-card sums over the card lists, one
// card per thread, and a fixed-order total (no atomics).
template <typename T>
__device__ void foldNode(const DevTree& t, const DevRows<T>& rows, int u, int tr,
                         const Scratch<T>& ws) {
  const NodeDev nd = t.nodes[u];
  const StateDev& st = t.states[nd.state];
  const int opp = 1 - tr;
  const int no = st.n[opp], nt = st.n[tr];
  const RowDev ru = t.rows[u];
  const uint16_t* csr = ws.tab;
  stageRow(ws.rs, rows.reach[tr] + (size_t)ru.reachQ[tr] * 4, no);
  stageTab(ws.tab, t.poolU16 + st.csrOff[opp], 53 + 2 * no);
  __syncthreads();
  T* cs = ws.X;  // [52], then the total at [52]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // One warp per card: lanes sum the card's list entries, then a fixed
  // shuffle tree (card lists hold at most 51 combos: two entries per lane).
  for (int c = warp; c < 52; c += nw) {
    const int s0 = csr[c], s1 = csr[c + 1];
    T a = T(0);
    for (int e = s0 + lane; e < s1; e += 32) a += ws.rs[csr[53 + e]];
    a = warpSum(a);
    if (lane == 0) cs[c] = a;
  }
  if (warp == nw - 1) {
    T part = T(0);
    for (int j = lane; j < no; j += 32) part += ws.rs[j];
    part = warpSum(part);
    if (lane == 0) cs[52] = part;
  }
  __syncthreads();
  const T tot = cs[52];
  const T v = (T)t.termVal[((size_t)u * 2 + tr) * 4];
  // Card pairs as one u16 per combo (cardsOff is even).
  const uint16_t* cards = reinterpret_cast<const uint16_t*>(t.poolU8 + st.cardsOff[tr]);
  const int16_t* same = t.poolI16 + st.sameOff[tr];
  T* out = rows.cfv + (size_t)ru.cfvQ * 4;
  const int nt4 = quadsOf(nt) * 4;
  for (int i0 = threadIdx.x; i0 < nt4; i0 += 4 * blockDim.x) {
    int cp[4], sm[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int i = i0 + j * blockDim.x;
      cp[j] = i < nt ? cards[i] : 0;
      sm[j] = i < nt ? same[i] : -1;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int i = i0 + j * blockDim.x;
      if (i >= nt4) break;
      if (i >= nt) {
        out[i] = T(0);
        continue;
      }
      T w = tot - cs[cp[j] & 0xff] - cs[cp[j] >> 8];
      if (sm[j] >= 0) w += ws.rs[sm[j]];
      if (w < T(0)) w = T(0);
      out[i] = w * v;
    }
  }
}

// Chance chunk: the parent's value of combo i sums the children's values
// over the branches it survives, in branch order (cuda/gpu_cfr.cu:529-555).
// One thread per parent combo (kChanceChunk combos per task); each branch's
// value row and slot map are resolved once per CTA into shared memory, and
// the per-branch loads go out in batches of 8 independent loads.
template <typename T>
__device__ void chanceChunk(const DevTree& t, const DevRows<T>& rows, int u, int chunk,
                            int tr, unsigned char* smem) {
  const NodeDev nd = t.nodes[u];
  const int nb = nodeCount(nd.meta);
  const int nt = t.states[nd.state].n[tr];
  const T** rowOf = reinterpret_cast<const T**>(smem);
  const int16_t** downOf = reinterpret_cast<const int16_t**>(smem + 64 * sizeof(void*));
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const int ch = t.children[nd.childBase + b];
    rowOf[b] = rows.cfv + (size_t)t.rows[ch].cfvQ * 4;
    downOf[b] = t.poolI16 + t.states[t.nodes[ch].state].downOff[tr];
  }
  __syncthreads();
  T* out = rows.cfv + (size_t)t.rows[u].cfvQ * 4;
  const int i = chunk * kChanceChunk + (int)threadIdx.x;
  if (i >= quadsOf(nt) * 4) return;
  T v = T(0);
  if (i < nt) {
    for (int b0 = 0; b0 < nb; b0 += 8) {
      int k[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) k[j] = b0 + j < nb ? downOf[b0 + j][i] : -1;
      T x[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) x[j] = k[j] >= 0 ? rowOf[b0 + j][k[j]] : T(0);
#pragma unroll
      for (int j = 0; j < 8; ++j) v += x[j];
    }
  }
  out[i] = v;
}

// Decide chunk, one thread per quad. Opponent node: the traverser's value
// sums the children. Traverser node, CFR: regret-matching+ strategy from
// the pre-update regrets, the node value, then the DCFR update
// (cuda/gpu_cfr.cu:479-523)
//   strat = strat * avg + sigma
//   regret = regret * (regret >= 0 ? pos : neg) + (cfv_a - value).
// EV: the average strategy's value. BR: the best action's value.
template <typename T>
__device__ void decideChunk(const DevTree& t, const DevRows<T>& rows, int u, int chunk, int tr,
                            int mode) {
  const NodeDev nd = t.nodes[u];
  const int na = nodeCount(nd.meta);
  const int n = t.states[nd.state].n[tr];
  const int nq = quadsOf(n);
  const int q = chunk * kChunkQuads + (int)threadIdx.x;
  if (q >= nq) return;
  const int* kids = t.children + nd.childBase;
  T* out = rows.cfv + (size_t)t.rows[u].cfvQ * 4;
  bool live[4];
  for (int l = 0; l < 4; ++l) live[l] = 4 * q + l < n;
  if (nodePlayer(nd.meta) != tr || mode == kModeBR) {
    const bool best = nodePlayer(nd.meta) == tr;
    T v[4];
    for (int l = 0; l < 4; ++l) v[l] = best ? T(-1e30) : T(0);
    for (int a = 0; a < na; ++a) {
      T c[4];
      ldq(rows.cfv + (size_t)t.rows[kids[a]].cfvQ * 4 + 4 * q, c);
      for (int l = 0; l < 4; ++l) v[l] = best ? (c[l] > v[l] ? c[l] : v[l]) : v[l] + c[l];
    }
    for (int l = 0; l < 4; ++l)
      if (!live[l]) v[l] = T(0);
    stq(out + 4 * q, v);
    return;
  }
  float* reg = t.regret + (size_t)nd.regQ * 4;
  float* str = t.strat + (size_t)nd.regQ * 4;
  const float* src = mode == kModeCFR ? reg : str;
  const int sigSrc = mode == kModeCFR ? 0 : 1;
  const T uniform = T(1) / T(na);
  float pos = 0.f, neg = 0.f, avg = 0.f;
  if (mode == kModeCFR) {
    const float* c = t.coef + (size_t)t.counter[nodeSpot(nd.meta)] * 3;
    pos = c[0];
    neg = c[1];
    avg = c[2];
  }
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
    T sc[4];
    for (int l = 0; l < 4; ++l) sc[l] = sigmaScale(acc[l]);
#pragma unroll
    for (int a = 0; a < kRegNa; ++a)
      if (a < na)
        for (int l = 0; l < 4; ++l) {
          x[a][l] = live[l] ? sigmaOfScaled(x[a][l], acc[l], sc[l], uniform, sigSrc) : T(0);
          val[l] += x[a][l] * cv[a][l];
        }
    stq(out + 4 * q, val);
    if (mode != kModeCFR) return;
    float* strLo = t.stratLo ? t.stratLo + (size_t)nd.regQ * 4 : nullptr;
#pragma unroll
    for (int a = 0; a < kRegNa; ++a)
      if (a < na) {
        float rg[4], sg[4], lo[4];
        const size_t o = ((size_t)a * nq + q) * 4;
        ldq(reg + o, rg);
        ldq(str + o, sg);
        if (strLo) {
          ldq(strLo + o, lo);
          for (int l = 0; l < 4; ++l) stratComp(sg[l], lo[l], avg, (float)x[a][l]);
          stq(strLo + o, lo);
        } else {
          for (int l = 0; l < 4; ++l) sg[l] = sg[l] * avg + (float)x[a][l];
        }
        for (int l = 0; l < 4; ++l)
          rg[l] = rg[l] * (rg[l] >= 0.0f ? pos : neg) + (float)(cv[a][l] - val[l]);
        stq(str + o, sg);
        stq(reg + o, rg);
      }
    return;
  }
  for (int a = 0; a < na; ++a) {
    T x[4];
    ldqf(src + ((size_t)a * nq + q) * 4, x);
    for (int l = 0; l < 4; ++l) acc[l] += sigmaMass(x[l], sigSrc);
  }
  T sc[4];
  for (int l = 0; l < 4; ++l) sc[l] = sigmaScale(acc[l]);
  for (int a = 0; a < na; ++a) {
    T x[4], c[4];
    ldqf(src + ((size_t)a * nq + q) * 4, x);
    ldq(rows.cfv + (size_t)t.rows[kids[a]].cfvQ * 4 + 4 * q, c);
    for (int l = 0; l < 4; ++l)
      val[l] += (live[l] ? sigmaOfScaled(x[l], acc[l], sc[l], uniform, sigSrc) : T(0)) * c[l];
  }
  stq(out + 4 * q, val);
  if (mode != kModeCFR) return;
  float* strLo = t.stratLo ? t.stratLo + (size_t)nd.regQ * 4 : nullptr;
  for (int a = 0; a < na; ++a) {
    float rg[4], sg[4], lo[4] = {0.f, 0.f, 0.f, 0.f};
    T c[4];
    const size_t o = ((size_t)a * nq + q) * 4;
    ldq(reg + o, rg);
    ldq(str + o, sg);
    if (strLo) ldq(strLo + o, lo);
    ldq(rows.cfv + (size_t)t.rows[kids[a]].cfvQ * 4 + 4 * q, c);
    for (int l = 0; l < 4; ++l) {
      const T s = live[l] ? sigmaOf((T)rg[l], acc[l], uniform, 0) : T(0);
      if (strLo) stratComp(sg[l], lo[l], avg, (float)s);
      else sg[l] = sg[l] * avg + (float)s;
      rg[l] = rg[l] * (rg[l] >= 0.0f ? pos : neg) + (float)(c[l] - val[l]);
    }
    stq(str + o, sg);
    if (strLo) stq(strLo + o, lo);
    stq(reg + o, rg);
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 6)
bwdLevelK(DevTree t, DevRows<T> rows, const int* __restrict__ tasks, int count, int tr,
          int mode, int maxN) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Scratch<T> ws = scratchOf<T>(smem, maxN);
  for (int i = blockIdx.x; i < count; i += gridDim.x) {
    const int w = tasks[i];
    const int node = (int)((unsigned)w >> 8), sub = (w >> 2) & 63;
    switch (w & 3) {
      case kTaskShowdown: showdownNode<T>(t, rows, node, tr, ws); break;
      case kTaskFold: foldNode<T>(t, rows, node, tr, ws); break;
      case kTaskChance: chanceChunk<T>(t, rows, node, sub, tr, smem); break;
      default: decideChunk<T>(t, rows, node, sub, tr, mode);
    }
    __syncthreads();  // the next task reuses the shared scratch
  }
}

// The same level split in two: terminal tasks (showdown, fold: shared
// scratch, 6 CTAs per SM) and interior tasks (decide, chance: 1 KB of
// shared memory, 8 CTAs per SM, memory-latency bound). The two halves of a
// level are independent and run concurrently (graph branches); the
// per-node arithmetic is bwdLevelK's.
template <typename T>
__global__ void __launch_bounds__(kThreads, 6)
bwdTerminalK(DevTree t, DevRows<T> rows, const int* __restrict__ tasks, int count, int tr,
             int maxN) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Scratch<T> ws = scratchOf<T>(smem, maxN);
  for (int i = blockIdx.x; i < count; i += gridDim.x) {
    const int w = tasks[i];
    if ((w & 3) == kTaskShowdown) showdownNode<T>(t, rows, (int)((unsigned)w >> 8), tr, ws);
    else foldNode<T>(t, rows, (int)((unsigned)w >> 8), tr, ws);
    __syncthreads();
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 8)
bwdInteriorK(DevTree t, DevRows<T> rows, const int* __restrict__ tasks, int count, int tr,
             int mode) {
  __shared__ __align__(16) unsigned char smem[kChanceScratchBytes];
  for (int i = blockIdx.x; i < count; i += gridDim.x) {
    const int w = tasks[i];
    const int node = (int)((unsigned)w >> 8), sub = (w >> 2) & 63;
    if ((w & 3) == kTaskChance) chanceChunk<T>(t, rows, node, sub, tr, smem);
    else decideChunk<T>(t, rows, node, sub, tr, mode);
    __syncthreads();
  }
}

// Internal linkage: this header is included by more than one translation unit.
static __global__ void advanceCounterK(int* counter, int spots) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < spots; i += gridDim.x * blockDim.x)
    ++counter[i];
}

}  // namespace gb
}  // namespace pps
