// Depth-level DCFR kernels for sm_103a.
//
// One DCFR half-step for traverser tr (the reference's halfStep,
// cuda/gpu_cfr.cu:797-828) is a top-down forward pass (fwdDecideK /
// fwdChanceK per depth: opponent reach times the opponent's strategy;
// chance compaction) and a bottom-up backward pass (bwdK per depth, one
// CTA per node dispatched on kind: showdown, fold, chance sum, decide
// value and the DCFR regret/strategy update).
//
// Rows are processed as 16-byte quads (4 floats or 4 doubles), padded
// lanes hold zero. T is the value type of the reach and cfv rows: float
// for CFR iterations, double for the value / best-response walks. Regret
// and strategy rows are always float.
//
// Everything is deterministic: no atomics; every sum has a fixed order.
#pragma once

#include <cstdint>

#include "layout.h"

namespace pps {
namespace gb {

constexpr int kThreads = 128;
constexpr int kRegNa = 8;  // actions kept in registers by the decide update

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
__device__ __forceinline__ int nodeFoldBy(int meta) { return (meta >> 3) & 1; }
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
// Strategy/regret quads converted to the walk type.
template <typename T>
__device__ __forceinline__ void ldqf(const float* p, T (&x)[4]) {
  float f[4];
  ldq(p, f);
  for (int l = 0; l < 4; ++l) x[l] = (T)f[l];
}

// Strategy of one combo lane from its action rows: regret matching+ over
// cumulative regrets (sigSrc 0) or the normalized average strategy
// (sigSrc 1). Same arithmetic as the reference (cuda/gpu_cfr.cu:245-262).
template <typename T>
__device__ __forceinline__ T sigmaOf(T x, T acc, T uniform, int sigSrc) {
  if (sigSrc == 0) return acc > T(0) ? (x > T(0) ? x / acc : T(0)) : uniform;
  return acc > T(0) ? x / acc : uniform;
}

// ---------------------------------------------------------------------------
// Forward pass.
// ---------------------------------------------------------------------------

// Opponent decide nodes at one depth: child reach = reach x sigma_a.
template <typename T>
__global__ void __launch_bounds__(kThreads)
fwdDecideK(DevTree t, DevRows<T> rows, const int* __restrict__ items, int count,
           int tr, int sigSrc) {
  for (int it = blockIdx.x; it < count; it += gridDim.x) {
    const int u = items[it];
    const NodeDev nd = t.nodes[u];
    const int na = nodeCount(nd.meta);
    const int opp = 1 - tr;
    const int n = t.states[nd.state].n[opp];
    const int nq = quadsOf(n);
    const float* src = (sigSrc == 0 ? t.regret : t.strat) + (size_t)nd.regQ * 4;
    const T* r = rows.reach[tr] + (size_t)t.rows[u].reachQ[tr] * 4;
    const int* kids = t.children + nd.childBase;
    const T uniform = T(1) / T(na);
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
      T rr[4], acc[4] = {T(0), T(0), T(0), T(0)};
      ldq(r + 4 * q, rr);
      for (int a = 0; a < na; ++a) {
        T x[4];
        ldqf(src + ((size_t)a * nq + q) * 4, x);
        for (int l = 0; l < 4; ++l) acc[l] += sigSrc == 0 ? (x[l] > T(0) ? x[l] : T(0)) : x[l];
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

// Chance branches at one depth: the child's opponent reach row is the
// parent's, compacted through the child's slot map and scaled by the
// pair-conditional deal probability 1 / (52 - nBoard - 4)
// (cuda/gpu_cfr.cu:276-293).
template <typename T>
__global__ void __launch_bounds__(kThreads)
fwdChanceK(DevTree t, DevRows<T> rows, const int* __restrict__ items, int count,
           int tr) {
  for (int it = blockIdx.x; it < count; it += gridDim.x) {
    const int item = items[it];
    const int u = item >> 6, br = item & 63;
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
}

// ---------------------------------------------------------------------------
// Block helpers.
// ---------------------------------------------------------------------------

// Error-free transformation a + b = s + e (Knuth TwoSum).
template <typename T>
__device__ __forceinline__ void twoSum(T a, T b, T& s, T& e) {
  s = a + b;
  const T bb = s - a;
  e = (a - (s - bb)) + (b - bb);
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

// Compensated exclusive scan of src[0..n) into (hi, lo)[0..n], entry k the
// sum of src[0..k); entry n the total. Each thread owns a contiguous chunk.
template <typename T>
__device__ void blockScanExclPair(const T* src, T* hi, T* lo, int n) {
  __shared__ T wHi[32], wLo[32];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int chunk = (n + nthr - 1) / nthr;
  const int b = min(tid * chunk, n), e = min(b + chunk, n);
  T sh = T(0), sl = T(0);
  for (int k = b; k < e; ++k) addPair(sh, sl, src[k], T(0));
  // Inclusive warp scan of the chunk sums.
  const int lane = tid & 31, warp = tid >> 5;
  T ih = sh, il = sl;
  for (int off = 1; off < 32; off <<= 1) {
    const T oh = __shfl_up_sync(0xffffffffu, ih, off);
    const T ol = __shfl_up_sync(0xffffffffu, il, off);
    if (lane >= off) {
      T h = oh, l = ol;
      addPair(h, l, ih, il);
      ih = h;
      il = l;
    }
  }
  if (lane == 31) {
    wHi[warp] = ih;
    wLo[warp] = il;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = (nthr + 31) >> 5;
    T h = lane < nw ? wHi[lane] : T(0), l = lane < nw ? wLo[lane] : T(0);
    for (int off = 1; off < 32; off <<= 1) {
      const T oh = __shfl_up_sync(0xffffffffu, h, off);
      const T ol = __shfl_up_sync(0xffffffffu, l, off);
      if (lane >= off) {
        T hh = oh, ll = ol;
        addPair(hh, ll, h, l);
        h = hh;
        l = ll;
      }
    }
    if (lane < nw) {
      wHi[lane] = h;
      wLo[lane] = l;
    }
  }
  __syncthreads();
  // Exclusive prefix of this thread's chunk start.
  T ph = warp > 0 ? wHi[warp - 1] : T(0), pl = warp > 0 ? wLo[warp - 1] : T(0);
  {
    T xh = __shfl_up_sync(0xffffffffu, ih, 1), xl = __shfl_up_sync(0xffffffffu, il, 1);
    if (lane > 0) addPair(ph, pl, xh, xl);
  }
  for (int k = b; k < e; ++k) {
    hi[k] = ph;
    lo[k] = pl;
    addPair(ph, pl, src[k], T(0));
  }
  if (e == n && b < e) {  // exactly one thread owns the last entry
    hi[n] = ph;
    lo[n] = pl;
  }
  if (n == 0 && tid == 0) {
    hi[0] = T(0);
    lo[0] = T(0);
  }
  __syncthreads();
}

// Deterministic block sum (fixed order: strided per thread, shuffle tree,
// warps in order).
template <typename T>
__device__ T blockSum(const T* v, int n) {
  __shared__ T part[32];
  T s = T(0);
  for (int k = threadIdx.x; k < n; k += blockDim.x) s += v[k];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) part[warp] = s;
  __syncthreads();
  T tot = T(0);
  const int nw = (blockDim.x + 31) >> 5;
  for (int w = 0; w < nw; ++w) tot += part[w];
  __syncthreads();
  return tot;
}

// ---------------------------------------------------------------------------
// Backward node handlers.
// ---------------------------------------------------------------------------

// Showdown: traverser combo i wins against opponents strictly weaker, ties
// the equal band, loses to the rest; opponents sharing a card with i are
// removed per card from each band using exclusive scans of the card
// segments (O(1) per combo), the identical combo (in the tie band, removed
// twice) is added back once. Payoffs as cuda/gpu_cfr.cu:356-406.
template <typename T>
__device__ void showdownNode(const DevTree& t, const DevRows<T>& rows, int u,
                             const NodeDev& nd, int tr, unsigned char* smem) {
  const int opp = 1 - tr;
  const StateDev& st = t.states[nd.state];
  const int no = st.n[opp], nt = st.n[tr];
  const uint16_t* ord = t.poolU16 + st.sdOff[tr];
  const uint16_t* seg = ord + no;
  const uint16_t* segPos = seg + 53;
  const ShowdownInfo* info = t.poolSd + st.sdInfoOff[tr];
  const RowDev ru = t.rows[u];
  const T* r = rows.reach[tr] + (size_t)ru.reachQ[tr] * 4;
  T* sr = reinterpret_cast<T*>(smem);   // sorted reach [no]
  T* sHi = sr + no;                     // [no + 1]
  T* sLo = sHi + no + 1;                // [no + 1]
  T* X = sLo + no + 1;                  // [2 no + 52]
  int* segS = reinterpret_cast<int*>(X + 2 * no + 52);  // [53]

  for (int k = threadIdx.x; k < no; k += blockDim.x) sr[k] = r[ord[k]];
  for (int c = threadIdx.x; c < 53; c += blockDim.x) segS[c] = seg[c];
  __syncthreads();
  blockScanExclPair(sr, sHi, sLo, no);

  // Per-card exclusive scans: warp w owns cards w, w + nWarps, ...
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  for (int c = warp; c < 52; c += nw) {
    const int s0 = segS[c], len = segS[c + 1] - s0;
    T* out = X + s0 + c;
    const int e0 = 2 * lane, e1 = 2 * lane + 1;
    const T v0 = e0 < len ? sr[segPos[s0 + e0]] : T(0);
    const T v1 = e1 < len ? sr[segPos[s0 + e1]] : T(0);
    T incl = v0 + v1;
    for (int off = 1; off < 32; off <<= 1) {
      const T o = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += o;
    }
    const T excl = incl - (v0 + v1);
    if (e0 <= len) out[e0] = excl;
    if (e1 <= len) out[e1] = excl + v0;
  }
  __syncthreads();

  const float* tv = t.termVal + ((size_t)u * 2 + tr) * 4;
  const T winV = (T)tv[0], tieV = (T)tv[1], loseV = (T)tv[2];
  T* out = rows.cfv + (size_t)ru.cfvQ * 4;
  const int nq4 = quadsOf(nt) * 4;
  for (int i = threadIdx.x; i < nq4; i += blockDim.x) {
    if (i >= nt) {
      out[i] = T(0);
      continue;
    }
    const ShowdownInfo f = info[i];
    const int le = f.x & 0xffff, te = f.x >> 16;
    const int c1 = f.y & 0xff, c2 = (f.y >> 8) & 0xff;
    const int a1 = segS[c1] + c1, a2 = segS[c2] + c2;
    const int len1 = segS[c1 + 1] - segS[c1], len2 = segS[c2 + 1] - segS[c2];
    const T x1le = X[a1 + ((f.y >> 16) & 0xff)], x1te = X[a1 + (f.y >> 24)];
    const T x2le = X[a2 + (f.z & 0xff)], x2te = X[a2 + ((f.z >> 8) & 0xff)];
    const int same = (int)(f.z >> 16) - 1;
    const T sameR = same >= 0 ? r[same] : T(0);
    // Band masses from the compensated prefix pairs.
    const T below = sHi[le] + sLo[le];
    const T band = (sHi[te] - sHi[le]) + (sLo[te] - sLo[le]);
    const T above = (sHi[no] - sHi[te]) + (sLo[no] - sLo[te]);
    T lm = below - x1le - x2le;
    T tm = band - (x1te - x1le) - (x2te - x2le) + sameR;
    T gm = above - (X[a1 + len1] - x1te) - (X[a2 + len2] - x2te);
    lm = lm > T(0) ? lm : T(0);
    tm = tm > T(0) ? tm : T(0);
    gm = gm > T(0) ? gm : T(0);
    out[i] = lm * winV + tm * tieV + gm * loseV;
  }
}

// Fold: every opponent combo not sharing a card with i pays; per-card sums
// come from the card segments (no atomics). cuda/gpu_cfr.cu:409-455.
template <typename T>
__device__ void foldNode(const DevTree& t, const DevRows<T>& rows, int u,
                         const NodeDev& nd, int tr, unsigned char* smem) {
  const int opp = 1 - tr;
  const StateDev& st = t.states[nd.state];
  const int no = st.n[opp], nt = st.n[tr];
  const RowDev ru = t.rows[u];
  const T* r = rows.reach[tr] + (size_t)ru.reachQ[tr] * 4;
  const uint16_t* csr = t.poolU16 + st.csrOff[opp];
  T* cs = reinterpret_cast<T*>(smem);  // [52]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  for (int c = warp; c < 52; c += nw) {
    const int s0 = csr[c], s1 = csr[c + 1];
    T s = T(0);
    for (int e = s0 + lane; e < s1; e += 32) s += r[csr[53 + e]];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) cs[c] = s;
  }
  const T tot = blockSum(r, no);  // also orders the cs[] writes
  const T v = (T)t.termVal[((size_t)u * 2 + tr) * 4];
  const uint8_t* cards = t.poolU8 + st.cardsOff[tr];
  const int16_t* same = t.poolI16 + st.sameOff[tr];
  T* out = rows.cfv + (size_t)ru.cfvQ * 4;
  const int nq4 = quadsOf(nt) * 4;
  for (int i = threadIdx.x; i < nq4; i += blockDim.x) {
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
}

// Chance: parent value of combo i sums the children's values over the
// branches it survives (cuda/gpu_cfr.cu:529-555), branches in order.
template <typename T>
__device__ void chanceNode(const DevTree& t, const DevRows<T>& rows, int u,
                           const NodeDev& nd, int tr, unsigned char* smem) {
  const int nb = nodeCount(nd.meta);
  const StateDev& st = t.states[nd.state];
  const int nt = st.n[tr];
  const T** rowp = reinterpret_cast<const T**>(smem);
  const int16_t** down = reinterpret_cast<const int16_t**>(smem + 64 * sizeof(void*));
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const int ch = t.children[nd.childBase + b];
    rowp[b] = rows.cfv + (size_t)t.rows[ch].cfvQ * 4;
    down[b] = t.poolI16 + t.states[t.nodes[ch].state].downOff[tr];
  }
  __syncthreads();
  T* out = rows.cfv + (size_t)t.rows[u].cfvQ * 4;
  const int nq4 = quadsOf(nt) * 4;
  for (int i = threadIdx.x; i < nq4; i += blockDim.x) {
    T v = T(0);
    if (i < nt)
      for (int b = 0; b < nb; ++b) {
        const int k = down[b][i];
        if (k >= 0) v += rowp[b][k];
      }
    out[i] = v;
  }
}

// Decide node of the opponent: the traverser's value sums the children.
template <typename T>
__device__ void decideOpponent(const DevTree& t, const DevRows<T>& rows, int u,
                               const NodeDev& nd, int tr) {
  const int na = nodeCount(nd.meta);
  const int nq = quadsOf(t.states[nd.state].n[tr]);
  const int* kids = t.children + nd.childBase;
  T* out = rows.cfv + (size_t)t.rows[u].cfvQ * 4;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    T v[4] = {T(0), T(0), T(0), T(0)};
    for (int a = 0; a < na; ++a) {
      T c[4];
      ldq(rows.cfv + (size_t)t.rows[kids[a]].cfvQ * 4 + 4 * q, c);
      for (int l = 0; l < 4; ++l) v[l] += c[l];
    }
    stq(out + 4 * q, v);
  }
}

// Decide node of the traverser. CFR: regret-matching+ strategy from the
// pre-update regrets, node value, then the DCFR update
//   strat = strat * avg + sigma;  regret = regret * (regret >= 0 ? pos : neg)
//   + (cfv_a - value)                      (cuda/gpu_cfr.cu:479-523).
// EV: the average strategy's value. BR: the best action's value.
template <typename T>
__device__ void decideTraverser(const DevTree& t, const DevRows<T>& rows, int u,
                                const NodeDev& nd, int tr, int mode) {
  const int na = nodeCount(nd.meta);
  const int n = t.states[nd.state].n[tr];
  const int nq = quadsOf(n);
  const int* kids = t.children + nd.childBase;
  float* reg = t.regret + (size_t)nd.regQ * 4;
  float* str = t.strat + (size_t)nd.regQ * 4;
  const float* src = mode == kModeCFR ? reg : str;
  T* out = rows.cfv + (size_t)t.rows[u].cfvQ * 4;
  const T uniform = T(1) / T(na);
  float pos = 0.f, neg = 0.f, avg = 0.f;
  if (mode == kModeCFR) {
    const float* c = t.coef + (size_t)(*t.counter) * 3;
    pos = c[0];
    neg = c[1];
    avg = c[2];
  }
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    bool live[4];
    for (int l = 0; l < 4; ++l) live[l] = 4 * q + l < n;
    T val[4] = {T(0), T(0), T(0), T(0)};
    if (mode == kModeBR) {
      for (int l = 0; l < 4; ++l) val[l] = T(-1e30);
      for (int a = 0; a < na; ++a) {
        T c[4];
        ldq(rows.cfv + (size_t)t.rows[kids[a]].cfvQ * 4 + 4 * q, c);
        for (int l = 0; l < 4; ++l) val[l] = c[l] > val[l] ? c[l] : val[l];
      }
      for (int l = 0; l < 4; ++l) val[l] = live[l] ? val[l] : T(0);
      stq(out + 4 * q, val);
      continue;
    }
    const int sigSrc = mode == kModeCFR ? 0 : 1;
    T acc[4] = {T(0), T(0), T(0), T(0)};
    if (na <= kRegNa) {
      T x[kRegNa][4], cv[kRegNa][4];
#pragma unroll
      for (int a = 0; a < kRegNa; ++a) {
        if (a < na) {
          ldqf(src + ((size_t)a * nq + q) * 4, x[a]);
          ldq(rows.cfv + (size_t)t.rows[kids[a]].cfvQ * 4 + 4 * q, cv[a]);
          for (int l = 0; l < 4; ++l)
            acc[l] += sigSrc == 0 ? (x[a][l] > T(0) ? x[a][l] : T(0)) : x[a][l];
        }
      }
#pragma unroll
      for (int a = 0; a < kRegNa; ++a) {
        if (a < na) {
          for (int l = 0; l < 4; ++l) {
            x[a][l] = live[l] ? sigmaOf(x[a][l], acc[l], uniform, sigSrc) : T(0);
            val[l] += x[a][l] * cv[a][l];
          }
        }
      }
      stq(out + 4 * q, val);
      if (mode != kModeCFR) continue;
#pragma unroll
      for (int a = 0; a < kRegNa; ++a) {
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
      }
    } else {
      for (int a = 0; a < na; ++a) {
        T x[4];
        ldqf(src + ((size_t)a * nq + q) * 4, x);
        for (int l = 0; l < 4; ++l) acc[l] += sigSrc == 0 ? (x[l] > T(0) ? x[l] : T(0)) : x[l];
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

// One CTA per node of a depth level, dispatched on kind.
template <typename T>
__global__ void __launch_bounds__(kThreads)
bwdK(DevTree t, DevRows<T> rows, const int* __restrict__ items, int count, int tr,
     int mode) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int it = blockIdx.x; it < count; it += gridDim.x) {
    const int u = items[it];
    const NodeDev nd = t.nodes[u];
    switch (nodeKind(nd.meta)) {
      case kShowdown: showdownNode<T>(t, rows, u, nd, tr, smem); break;
      case kFold: foldNode<T>(t, rows, u, nd, tr, smem); break;
      case kChance: chanceNode<T>(t, rows, u, nd, tr, smem); break;
      default:
        if (nodePlayer(nd.meta) == tr) decideTraverser<T>(t, rows, u, nd, tr, mode);
        else decideOpponent<T>(t, rows, u, nd, tr);
    }
    __syncthreads();
  }
}

__global__ void advanceCounterK(int* counter) {
  if (threadIdx.x == 0 && blockIdx.x == 0) ++(*counter);
}

// Shared memory the backward kernel needs for lists of up to maxN combos.
template <typename T>
inline size_t bwdSmemBytes(int maxN) {
  const size_t sd = sizeof(T) * ((size_t)maxN + 2 * ((size_t)maxN + 1) + 2 * (size_t)maxN + 52) +
                    53 * sizeof(int);
  const size_t ch = 128 * sizeof(void*);
  return sd > ch ? sd : ch;
}

}  // namespace gb
}  // namespace pps
