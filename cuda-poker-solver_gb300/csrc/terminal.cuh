// Terminal groups: the showdown and fold nodes of one depth level and one
// board state, taken four at a time (the f32 DCFR iteration).
//
// The four nodes share the state's tables (strength order, card segments,
// card lists, showdown entries), so a CTA stages those once and runs the
// four nodes' arithmetic side by side as float4 lanes: reach rows are staged
// transposed (entry j of the four rows is one float4), every scan and
// gather moves float4s, and each table entry is decoded once for all four
// nodes. The per-node formulas are those of showdownNode / foldNode
// (kernels.cuh; the reference's cuda/gpu_cfr.cu:355-406 and 433-454):
//   showdown: win / tie / lose masses from an exclusive prefix of the
//     strength-sorted opponent reach (warp blocks of 256 positions, block
//     totals accumulated compensated, as (hi, lo) pairs, the lo word
//     folded into the block's position prefixes), minus the
//     opponents holding either card (per-card segment prefixes X read at
//     precomputed counts), plus the identical combo once in the tie band;
//   fold: (total - card sums of both cards + identical combo) x payoff,
//     card sums in a fixed order (no atomics); the total is half the sum
//     of the 52 card sums (each combo holds two cards).
#pragma once

#include "decide.cuh"
#include "kernels.cuh"

namespace pps {
namespace gb {

constexpr int kTermThreads = 256;

// ---- float4 lane arithmetic ----
// Each float4 operation is two packed f32x2 instructions (sm_100+), the
// lanes rounded exactly as four scalar operations would be; a - b is
// fma(b, -1, a), which rounds once, as a subtraction does.
__device__ __forceinline__ float2 lanesXY(float4 a) { return make_float2(a.x, a.y); }
__device__ __forceinline__ float2 lanesZW(float4 a) { return make_float2(a.z, a.w); }
__device__ __forceinline__ float4 lanes4(float2 xy, float2 zw) {
  return make_float4(xy.x, xy.y, zw.x, zw.y);
}
__device__ __forceinline__ float4 operator+(float4 a, float4 b) {
  return lanes4(__fadd2_rn(lanesXY(a), lanesXY(b)), __fadd2_rn(lanesZW(a), lanesZW(b)));
}
__device__ __forceinline__ float4 operator-(float4 a, float4 b) {
  const float2 m1 = make_float2(-1.f, -1.f);
  return lanes4(__ffma2_rn(lanesXY(b), m1, lanesXY(a)), __ffma2_rn(lanesZW(b), m1, lanesZW(a)));
}
// a * b + c per lane (one rounding).
__device__ __forceinline__ float4 fma4(float4 a, float4 b, float4 c) {
  return lanes4(__ffma2_rn(lanesXY(a), lanesXY(b), lanesXY(c)),
                __ffma2_rn(lanesZW(a), lanesZW(b), lanesZW(c)));
}
__device__ __forceinline__ float4 mul4(float4 a, float4 b) {
  return lanes4(__fmul2_rn(lanesXY(a), lanesXY(b)), __fmul2_rn(lanesZW(a), lanesZW(b)));
}
__device__ __forceinline__ float4& operator+=(float4& a, float4 b) { return a = a + b; }
__device__ __forceinline__ float4 max0(float4 a) {
  return make_float4(a.x > 0.f ? a.x : 0.f, a.y > 0.f ? a.y : 0.f, a.z > 0.f ? a.z : 0.f,
                     a.w > 0.f ? a.w : 0.f);
}
__device__ __forceinline__ float4 zero4() { return make_float4(0.f, 0.f, 0.f, 0.f); }
__device__ __forceinline__ float4 shflUp4(float4 v, int off, int width = 32) {
  return make_float4(__shfl_up_sync(0xffffffffu, v.x, off, width),
                     __shfl_up_sync(0xffffffffu, v.y, off, width),
                     __shfl_up_sync(0xffffffffu, v.z, off, width),
                     __shfl_up_sync(0xffffffffu, v.w, off, width));
}
__device__ __forceinline__ float4 shflXor4(float4 v, int mask, int width = 32) {
  return make_float4(__shfl_xor_sync(0xffffffffu, v.x, mask, width),
                     __shfl_xor_sync(0xffffffffu, v.y, mask, width),
                     __shfl_xor_sync(0xffffffffu, v.z, mask, width),
                     __shfl_xor_sync(0xffffffffu, v.w, mask, width));
}
__device__ __forceinline__ float comp4(float4 v, int g) {
  return g == 0 ? v.x : g == 1 ? v.y : g == 2 ? v.z : v.w;
}

// The group record as the kernels read it: every thread loads the header
// (list sizes, table offsets) and the reach rows, which the staging needs,
// in one round trip after the task word; threads 0-7 copy the whole record
// to shared memory on the way, and what is read after the first barrier
// (value rows, payoffs, the showdown table offset) comes from that copy
// instead of occupying registers through the table builds.
struct GroupHead {
  int no, nt, tabOff, infoOff, sameOff, mask;
  uint4 reachQ;
};
static __device__ __forceinline__ GroupHead loadGroupHead(const GroupRec* g, GroupRec* copy) {
  const uint4* w = reinterpret_cast<const uint4*>(g);
  const uint4 h0 = w[0], h1 = w[1];
  GroupHead h;
  h.no = (int)h0.x;
  h.nt = (int)h0.y;
  h.tabOff = (int)h0.z;
  h.infoOff = (int)h0.w;
  h.sameOff = (int)h1.x;
  h.mask = (int)h1.y;
  h.reachQ = w[2];
  if (threadIdx.x < sizeof(GroupRec) / 16)
    reinterpret_cast<uint4*>(copy)[threadIdx.x] = w[threadIdx.x];
  return h;
}
static __device__ __forceinline__ uint4 cfvQOf(const GroupRec* c) {
  return *reinterpret_cast<const uint4*>(c->cfvQ);
}
static __device__ __forceinline__ float4 valOf(const GroupRec* c, int k) {
  return *reinterpret_cast<const float4*>(c->val[k]);
}

// ---- shared-memory layout of a group task (maxN: largest list) ----
// The sorted prefix gives each thread kSpan consecutive positions, so one
// pass of kTermThreads threads covers every list (kSpan * 256 >= 1327), and
// narrower CTAs cover narrower lists (termThreadsFor); a warp's 256
// positions form one compensation block.
constexpr int kSpan = 8;
constexpr int kSpanShift = 8;  // log2(32 * kSpan): position -> warp block
static_assert(kSpanShift == 8, "showdown entries carry position >> 8 as the warp block (layout.h)");
__host__ __device__ inline int groupTabEntries(int maxN) { return (3 * maxN + 53 + 7) / 8 * 8; }
// The float4 arrays below are padded with one entry after every 8 (entry k
// lives at pad8(k)): a thread's 8 consecutive positions, and the 8 lanes
// of a card segment, then fall in 8 different bank groups when they write
// at stride 8, instead of 8-way conflicts on one bank group (ncu counted
// conflicts as 62% of the showdown kernel's shared-memory wavefronts).
__host__ __device__ inline int groupPrefixEntries(int maxN) { return pad8(maxN + kSpan) + 1; }
__host__ __device__ inline int groupXEntries(int maxN) { return pad8(2 * maxN + 52) + 1; }
__host__ __device__ inline int groupRowEntries(int maxN) { return pad8(4 * ((maxN + 3) / 4)) + 1; }
constexpr int kGroupBlocks = kTermThreads / 32 + 1;  // warp blocks + the total

// Showdown groups: tab | P4 | X4 | W4 | BH | record copy. The P4 region
// first holds the staged (transposed, unsorted) reach rows, then the sorted
// prefixes.
__host__ __device__ inline size_t sdGroupSmem(int maxN) {
  return (size_t)groupTabEntries(maxN) * 2 +
         16 * ((size_t)groupPrefixEntries(maxN) + groupXEntries(maxN) + 2 * kGroupBlocks) +
         sizeof(GroupRec);
}
// Fold groups: tab | rs4 | cs4[53] | card pairs (u16) | identical-combo
// slots (i16) | group tail.
// The fold's table (53 segment starts, then the card lists) is shorter than
// the showdown's.
__host__ __device__ inline int foldTabEntries(int maxN) { return (2 * maxN + 53 + 7) / 8 * 8; }
__host__ __device__ inline size_t fdGroupSmem(int maxN) {
  return (size_t)foldTabEntries(maxN) * 2 + 16 * ((size_t)groupRowEntries(maxN) + 53) +
         (size_t)4 * ((maxN + 7) / 8 * 8) + sizeof(GroupRec);
}

// Stages the group's opponent reach rows transposed: rs4[pad8(j)] holds
// entry j of the four rows (0 for an absent node).
static __device__ __forceinline__ void stageRows4(float4* rs4, const DevRows<float>& rows,
                                                  int mask, uint4 reachQ, int tr, int no) {
  const uint32_t q[4] = {reachQ.x, reachQ.y, reachQ.z, reachQ.w};
  const float* r[4];
#pragma unroll
  for (int g = 0; g < 4; ++g)
    r[g] = (mask >> g) & 1 ? rows.reach[tr] + (size_t)q[g] * 4 : nullptr;
  // Read-only loads: the compiler may issue a thread's next quad before
  // the shared-memory stores of this one.
  for (int q = threadIdx.x; q < quadsOf(no); q += blockDim.x) {
    float4 v[4];
#pragma unroll
    for (int g = 0; g < 4; ++g)
      v[g] = r[g] ? __ldg(reinterpret_cast<const float4*>(r[g] + 4 * q)) : zero4();
    float4* d = rs4 + pad8(4 * q);  // the quad's 4 entries share one pad block
    d[0] = make_float4(v[0].x, v[1].x, v[2].x, v[3].x);
    d[1] = make_float4(v[0].y, v[1].y, v[2].y, v[3].y);
    d[2] = make_float4(v[0].z, v[1].z, v[2].z, v[3].z);
    d[3] = make_float4(v[0].w, v[1].w, v[2].w, v[3].w);
  }
}

// Starts asynchronous copies (cp.async, 16 bytes each) of a 16-byte aligned
// table of n16 chunks into shared memory; they land while the thread loads
// the reach rows, and stageDone waits for them.
static __device__ __forceinline__ void stageChunksAsync(void* dst, const void* src, int n16) {
  for (int k = threadIdx.x; k < n16; k += blockDim.x) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(reinterpret_cast<uint4*>(dst) + k);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s),
                 "l"(reinterpret_cast<const uint4*>(src) + k)
                 : "memory");
  }
}
static __device__ __forceinline__ void stageDone() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Value rows of the group's nodes (nullptr for an absent node).
static __device__ __forceinline__ void outRows4(float* (&out)[4], const DevRows<float>& rows,
                                                int mask, uint4 cfvQ) {
  const uint32_t q[4] = {cfvQ.x, cfvQ.y, cfvQ.z, cfvQ.w};
#pragma unroll
  for (int g = 0; g < 4; ++g) out[g] = (mask >> g) & 1 ? rows.cfv + (size_t)q[g] * 4 : nullptr;
}


static __device__ __forceinline__ void storeOut4(float* const (&out)[4], int i, float4 c) {
  if (out[0]) out[0][i] = c.x;
  if (out[1]) out[1][i] = c.y;
  if (out[2]) out[2][i] = c.z;
  if (out[3]) out[3][i] = c.w;
}

static __device__ void showdownGroup(const DevTree& t, const DevRows<float>& rows,
                                     const GroupRec* grec, int tr, unsigned char* smem, int maxN) {
  uint16_t* tab = reinterpret_cast<uint16_t*>(smem);
  float4* P4 = reinterpret_cast<float4*>(smem + (size_t)groupTabEntries(maxN) * 2);
  float4* rs4 = P4;  // staged rows until the prefixes replace them
  float4* X4 = P4 + groupPrefixEntries(maxN);
  float4* W4 = X4 + groupXEntries(maxN);
  float4* BH4 = W4 + kGroupBlocks;  // per warp block: the hi word of its offset
  GroupRec* rc = reinterpret_cast<GroupRec*>(W4 + 2 * kGroupBlocks);
  {
    const GroupHead gh = loadGroupHead(grec, rc);
    stageChunksAsync(tab, t.poolU16 + gh.tabOff, (3 * gh.no + 53 + 7) / 8);
    stageRows4(rs4, rows, gh.mask, gh.reachQ, tr, gh.no);
    stageDone();
  }
  __syncthreads();
  // From here on the record's words come from the shared copy.
  const int no = rc->no, nt = rc->nt;
  const uint16_t* ord = tab;
  const uint16_t* seg = ord + no;
  const uint16_t* segSlot = seg + 53;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;

  // Card segments, four cards per warp (8 lanes x 8 entries per card):
  // X4[pad8(seg[c] + c + k)] = reach of the card's first k entries, k = 0..len.
  for (int cb = warp * 4; cb < 52; cb += nw * 4) {
    const int c = cb + (lane >> 3), sub = lane & 7;
    const int s0 = seg[c], len = seg[c + 1] - s0;
    float4 pre[8];
    float4 run = zero4();
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int e = sub * 8 + j;
      pre[j] = run;
      if (e < len) run += rs4[pad8(segSlot[s0 + e])];
    }
    float4 incl = run;
#pragma unroll
    for (int off = 1; off < 8; off <<= 1) {
      const float4 x = shflUp4(incl, off, 8);
      if (sub >= off) incl += x;
    }
    float4 base = shflUp4(incl, 1, 8);
    if (sub == 0) base = zero4();
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int e = sub * 8 + j;
      if (e <= len) X4[pad8(s0 + c + e)] = base + pre[j];
    }
  }
  // Exclusive prefixes of the strength-sorted reach in one pass: thread t
  // takes positions [8t, 8t + 8); lane totals are scanned within the warp
  // (uncompensated within a warp's 256 positions) and the warp totals go
  // to W4 for the compensated pass below. The prefixes stay in registers
  // until every thread has read the staged rows they replace.
  const int nbw = (no >> kSpanShift) + 1;  // warp blocks covering 0..no
  const int k0 = threadIdx.x * kSpan;
  const bool mine = warp < nbw && k0 <= no;
  float4 pre[kSpan], ex = zero4();
  if (warp < nbw) {
    float4 v[kSpan];
    const uint4 o8 = mine && k0 < no ? *reinterpret_cast<const uint4*>(ord + k0) : make_uint4(0, 0, 0, 0);
    const uint16_t* o = reinterpret_cast<const uint16_t*>(&o8);
#pragma unroll
    for (int j = 0; j < kSpan; ++j) v[j] = k0 + j < no ? rs4[pad8(o[j])] : zero4();
    float4 run = zero4();
#pragma unroll
    for (int j = 0; j < kSpan; ++j) {
      pre[j] = run;
      run += v[j];
    }
    float4 incl = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const float4 x = shflUp4(incl, off);
      if (lane >= off) incl += x;
    }
    ex = shflUp4(incl, 1);
    if (lane == 0) ex = zero4();
    if (lane == 31) W4[warp] = incl;
  }
  __syncthreads();
  // Compensated exclusive prefix of the warp-block totals: every thread
  // of a block computes its own block's (hi, lo) offset, in the same order
  // as every other, and stores its positions as Q = lo + P (the low word
  // folded into the block-local prefix); the block's hi goes to BH.
  if (mine) {
    float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
    for (int b = 0; b < warp; ++b) {
      const float4 w = W4[b];
      addComp(hi[0], lo[0], w.x);
      addComp(hi[1], lo[1], w.y);
      addComp(hi[2], lo[2], w.z);
      addComp(hi[3], lo[3], w.w);
    }
    const float4 bl = make_float4(lo[0], lo[1], lo[2], lo[3]);
#pragma unroll
    for (int j = 0; j < kSpan; ++j) P4[pad8(k0 + j)] = bl + (ex + pre[j]);
    if (lane == 0) BH4[warp] = make_float4(hi[0], hi[1], hi[2], hi[3]);
  }
  __syncthreads();

  // Payoffs of the four nodes (zero for an absent node: the record's
  // padding slots hold zeros).
  const float4 v0 = valOf(rc, 0), v1 = valOf(rc, 1), v2 = valOf(rc, 2), v3 = valOf(rc, 3);
  const float4 win4 = make_float4(v0.x, v1.x, v2.x, v3.x);
  const float4 tie4 = make_float4(v0.y, v1.y, v2.y, v3.y);
  const float4 lose4 = make_float4(v0.z, v1.z, v2.z, v3.z);
  const ShowdownInfo* info = t.poolSd + rc->infoOff;
  const int bn = no >> kSpanShift;
  const float4 TH = BH4[bn], QT = P4[pad8(no)];
  float* out[4];
  outRows4(out, rows, rc->mask, cfvQOf(rc));
  const int nt4 = quadsOf(nt) * 4;
#pragma unroll 3
  for (int k = threadIdx.x; k < nt4; k += blockDim.x) {
    if (k >= nt) {
      storeOut4(out, k, zero4());
      continue;
    }
    // The entry holds the shared-memory indices themselves and its combo's
    // offset in its warp window (layout.h).
    const ShowdownInfo f = info[k];
    const int i = showdownCombo(k, f);
    const float4 x1le = X4[f.x & 0xfff], x1te = X4[(f.x >> 12) & 0xfff];
    const float4 x1end = X4[f.y & 0xfff], x2le = X4[(f.y >> 12) & 0xfff];
    const float4 x2te = X4[f.z & 0xfff], x2end = X4[(f.z >> 12) & 0xfff];
    // The identical combo's reach: its step in card c1's segment prefix
    // (exact up to the rounding of that prefix, a few units in the last
    // place of a sum of at most 51 entries).
    const int sHi = (int)((f.x >> 24) | ((f.y >> 16) & 0xf00));
    const int sLo = sHi - 1 - (int)((f.w >> 28) & 1);
    float4 sameR = X4[sHi] - X4[sLo];
    if (!((f.w >> 29) & 1)) sameR = zero4();
    const float4 bhl = BH4[(f.w >> 22) & 7], bht = BH4[(f.w >> 25) & 7];
    const float4 qle = P4[f.w & 0x7ff], qte = P4[(f.w >> 11) & 0x7ff];
    const float4 below = bhl + qle;
    const float4 band = (bht - bhl) + (qte - qle);
    const float4 above = (TH - bht) + (QT - qte);
    const float4 lm = max0(below - x1le - x2le);
    const float4 tm = max0(band - (x1te - x1le) - (x2te - x2le) + sameR);
    const float4 gm = max0(above - (x1end - x1te) - (x2end - x2te));
    const float4 c = fma4(gm, lose4, fma4(tm, tie4, mul4(lm, win4)));
    storeOut4(out, i, c);
  }
}

static __device__ void foldGroup(const DevTree& t, const DevRows<float>& rows, const GroupRec* grec,
                                 int tr, unsigned char* smem, int maxN) {
  uint16_t* csr = reinterpret_cast<uint16_t*>(smem);
  float4* rs4 = reinterpret_cast<float4*>(smem + (size_t)foldTabEntries(maxN) * 2);
  float4* cs4 = rs4 + groupRowEntries(maxN);  // [52] card sums, [52] total
  uint16_t* cardsS = reinterpret_cast<uint16_t*>(cs4 + 53);
  int16_t* sameS = reinterpret_cast<int16_t*>(cardsS + (maxN + 7) / 8 * 8);
  GroupRec* rc = reinterpret_cast<GroupRec*>(sameS + (maxN + 7) / 8 * 8);
  const GroupHead gh = loadGroupHead(grec, rc);
  const int no = gh.no, nt = gh.nt;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;

  // The opponent's card lists, the traverser's card pairs (u16 each) and
  // identical-combo slots: 16-byte aligned tables copied in whole chunks.
  stageChunksAsync(csr, t.poolU16 + gh.tabOff, (53 + 2 * no + 7) / 8);
  stageChunksAsync(cardsS, t.poolU8 + gh.infoOff, (nt + 7) / 8);
  stageChunksAsync(sameS, t.poolI16 + gh.sameOff, (nt + 7) / 8);
  stageRows4(rs4, rows, gh.mask, gh.reachQ, tr, no);
  stageDone();
  __syncthreads();
  // Card sums, four cards per warp (8 lanes x 8 entries, then a fixed
  // xor tree over the 8 lanes).
  for (int cb = warp * 4; cb < 52; cb += nw * 4) {
    const int c = cb + (lane >> 3), sub = lane & 7;
    const int s0 = csr[c], len = csr[c + 1] - s0;
    float4 a = zero4();
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int e = sub * 8 + j;
      if (e < len) a += rs4[pad8(csr[53 + s0 + e])];
    }
#pragma unroll
    for (int m = 4; m > 0; m >>= 1) a += shflXor4(a, m, 8);
    if (sub == 0) cs4[c] = a;
  }
  __syncthreads();
  // Total: every combo holds two cards, so it is half the 52 card sums'
  // total (warp 0: card pairs c, c + 26, then a fixed xor tree).
  if (warp == 0) {
    float4 a = lane < 26 ? cs4[lane] + cs4[lane + 26] : zero4();
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) a += shflXor4(a, m);
    if (lane == 0) cs4[52] = make_float4(0.5f * a.x, 0.5f * a.y, 0.5f * a.z, 0.5f * a.w);
  }
  __syncthreads();
  const float4 tot = cs4[52];
  const float4 pay = make_float4(rc->val[0][0], rc->val[1][0], rc->val[2][0], rc->val[3][0]);
  float* out[4];
  outRows4(out, rows, rc->mask, cfvQOf(rc));
  const int nt4 = quadsOf(nt) * 4;
#pragma unroll 2
  for (int i = threadIdx.x; i < nt4; i += blockDim.x) {
    if (i >= nt) {
      storeOut4(out, i, zero4());
      continue;
    }
    const int cp = cardsS[i], sm = sameS[i];
    float4 w = tot - cs4[cp & 0xff] - cs4[cp >> 8];
    if (sm >= 0) w += rs4[pad8(sm)];
    w = max0(w);
    storeOut4(out, i, mul4(w, pay));
  }
}

// One CTA per group task: task word kind 3 (showdown) or 2 (fold), node
// field = index into the group table (four node ids, -1 for none). One
// kernel per kind (the showdown tables need 4x the shared memory and more
// registers; folds fit more CTAs per SM). Internal linkage: this header is
// included by more than one translation unit, each keeping its own copy.
//
// The CTA has kT threads, the fewest whose sorted-prefix pass (kSpan
// positions a thread) covers positions 0..maxN: narrow ranges (lists of up
// to 511 combos) take 64-thread CTAs, so a level's groups fit the GPU in
// one wave instead of holding idle threads.
__host__ __device__ constexpr int termThreadsFor(int maxN) {
  return maxN + 1 <= kSpan * 64 ? 64 : maxN + 1 <= kSpan * 128 ? 128 : kTermThreads;
}
constexpr int sdMinBlocks(int kT) { return 3 * kTermThreads / kT; }
// Seven 256-thread fold CTAs per SM (32 registers, 29.7 KB of shared memory
// on the full-range lists): +0.6% on the 48,255-node turn and +0.7% on the
// 6,333-node one over six (40 registers), +1.0% for six over five before.
// The narrower instances stay at the five-CTA register budget, which
// measured faster on the narrow-range spots.
constexpr int fdMinBlocks(int kT) { return (kT == kTermThreads ? 7 : 5) * kTermThreads / kT; }

// Group record of task i: from the task word's node field, or, for a list
// of consecutive groups (tasks null, groups at its first), the i-th.
static __device__ __forceinline__ const GroupRec* groupOf(const GroupRec* groups,
                                                          const int* tasks, int i, int tr) {
  return groups + 2 * (tasks ? (unsigned)tasks[i] >> 8 : (unsigned)i) + tr;
}

template <int kT>
static __global__ void __launch_bounds__(kT, sdMinBlocks(kT))
sdGroupK(DevTree t, DevRows<float> rows, const GroupRec* __restrict__ groups,
         const int* __restrict__ tasks, int count, int tr, int maxN) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int i = blockIdx.x; i < count; i += gridDim.x) {
    showdownGroup(t, rows, groupOf(groups, tasks, i, tr), tr, smem, maxN);
    __syncthreads();  // the next task reuses the shared memory
  }
}

template <int kT>
static __global__ void __launch_bounds__(kT, fdMinBlocks(kT))
fdGroupK(DevTree t, DevRows<float> rows, const GroupRec* __restrict__ groups,
         const int* __restrict__ tasks, int count, int tr, int maxN) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int i = blockIdx.x; i < count; i += gridDim.x) {
    foldGroup(t, rows, groupOf(groups, tasks, i, tr), tr, smem, maxN);
    __syncthreads();
  }
}

// Backward level of the fused plan (engine kind 2, narrow ranges: lists of
// up to 1023 combos): one launch per level covers the level's decide
// records (four per CTA), chance tasks, showdown groups and fold groups,
// chained to the previous level by programmatic dependent launch, so the
// iteration runs on one stream with no cross-stream joins. The group CTAs
// have kThreads (128) threads. Dynamic shared memory: fusedLevelSmem(maxN).
//
// Every kernel of the fused plan lets the next grid launch only after its
// own wait has returned ("late" triggers), so a grid that has launched
// implies that the grid two places before it has completed. Terminal
// groups read only reach rows, written by the forward pass, and write
// value rows that nothing in the previous grid touches; so, except in the
// first backward launch of a half-step (termWait: its reach rows come from
// the grid just before), they start without waiting and run under the
// previous level's tail. They wait as well where the launch has no record
// or chance CTA, so that the late-trigger chain is never broken.
__host__ __device__ inline size_t fusedLevelSmem(int maxN) {
  size_t s = sdGroupSmem(maxN);
  if (fdGroupSmem(maxN) > s) s = fdGroupSmem(maxN);
  return s > bwdStageBytes() ? s : bwdStageBytes();
}
constexpr int kFusedMaxN = kSpan * kThreads - 1;  // widest list of a 128-thread group

static __global__ void __launch_bounds__(kThreads, 6)
bwdLevelFusedK(DevTree t, DevRows<float> rows, const uint32_t* __restrict__ recs,
               const uint32_t* __restrict__ recTasks, int nRec, const uint32_t* __restrict__ chance,
               int nCh, const GroupRec* __restrict__ groups, const int* __restrict__ sd, int nSd,
               const int* __restrict__ fd, int nFd, int tr, int maxN, int termWait) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = (int)threadIdx.x & 31;
  const int e1 = recordCtas(nRec), e2 = e1 + nCh, e3 = e2 + nSd, e4 = e3 + nFd;
  const bool groupsWait = termWait || e2 == 0;
  bool waited = false;
  for (int i = blockIdx.x; i < e4; i += gridDim.x) {
    if (i != (int)blockIdx.x) __syncthreads();  // shared memory of the last task
    if (i < e1) {
      const int k = i * kRecWarps + (int)(threadIdx.x >> 5);
      if (k < nRec) {
        const DecRec r = loadRec(recs, recTasks[k]);
        decideRecordOwnRows(t, r, lane, reinterpret_cast<float4*>(smem));
        pdlWait();
        waited = true;
        decideRecordStaged(t, rows, r, lane, reinterpret_cast<float4*>(smem));
      }
    } else if (i < e2) {
      const uint4 h = loadChanceHeader(recs, chance[i - e1]);
      chanceRecordTables(t, rows, recs, h, smem);
      __syncthreads();
      chanceRecordSlots(h, smem);
      pdlWait();
      waited = true;
      chanceRecordSum(rows, h, smem);
      __syncthreads();  // the next task reuses the shared memory
    } else {
      const bool show = i < e3;
      const GroupRec* g = groups + 2 * ((unsigned)(show ? sd[i - e2] : fd[i - e3]) >> 8) + tr;
      if (groupsWait) {
        pdlWait();
        waited = true;
      }
      pdlTrigger();
      if (show) showdownGroup(t, rows, g, tr, smem, maxN);
      else foldGroup(t, rows, g, tr, smem, maxN);
      __syncthreads();
      continue;
    }
    if (waited) pdlTrigger();
  }
  if (!waited) {  // idle warps of a record CTA
    pdlWait();
    pdlTrigger();
  }
}

void raiseSmemLimit(const void* kernel, size_t bytes);

// Launches one level's showdown (fold) groups with the CTA size of maxN.
static inline void launchSdGroups(unsigned grid, size_t smem, cudaStream_t s, const DevTree& t,
                                  const DevRows<float>& rows, const GroupRec* groups,
                                  const int* tasks, int count, int tr, int maxN) {
  switch (termThreadsFor(maxN)) {
    case 64: sdGroupK<64><<<grid, 64, smem, s>>>(t, rows, groups, tasks, count, tr, maxN); break;
    case 128: sdGroupK<128><<<grid, 128, smem, s>>>(t, rows, groups, tasks, count, tr, maxN); break;
    default:
      sdGroupK<kTermThreads><<<grid, kTermThreads, smem, s>>>(t, rows, groups, tasks, count, tr,
                                                             maxN);
  }
}
static inline void launchFdGroups(unsigned grid, size_t smem, cudaStream_t s, const DevTree& t,
                                  const DevRows<float>& rows, const GroupRec* groups,
                                  const int* tasks, int count, int tr, int maxN) {
  switch (termThreadsFor(maxN)) {
    case 64: fdGroupK<64><<<grid, 64, smem, s>>>(t, rows, groups, tasks, count, tr, maxN); break;
    case 128: fdGroupK<128><<<grid, 128, smem, s>>>(t, rows, groups, tasks, count, tr, maxN); break;
    default:
      fdGroupK<kTermThreads><<<grid, kTermThreads, smem, s>>>(t, rows, groups, tasks, count, tr,
                                                             maxN);
  }
}
// Opens the dynamic shared memory the group kernels of maxN need (every CTA
// size: the translation unit's own copies).
static inline void raiseGroupSmem(int maxN) {
  const size_t sd = sdGroupSmem(maxN), fd = fdGroupSmem(maxN);
  raiseSmemLimit((const void*)sdGroupK<64>, sd);
  raiseSmemLimit((const void*)sdGroupK<128>, sd);
  raiseSmemLimit((const void*)sdGroupK<kTermThreads>, sd);
  raiseSmemLimit((const void*)fdGroupK<64>, fd);
  raiseSmemLimit((const void*)fdGroupK<128>, fd);
  raiseSmemLimit((const void*)fdGroupK<kTermThreads>, fd);
  if (maxN <= kFusedMaxN) raiseSmemLimit((const void*)bwdLevelFusedK, fusedLevelSmem(maxN));
}

}  // namespace gb
}  // namespace pps
