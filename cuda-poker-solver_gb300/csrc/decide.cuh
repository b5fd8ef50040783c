// Decide records: the f32 DCFR iteration's decide-node tasks with every row
// address resolved on the host.
//
// A node-based task (kernels.cuh) reaches its rows through a chain of
// dependent loads (task -> node -> state / children / own row -> each
// child's row -> data); at four or five round trips of device memory
// latency per task this chain, not bandwidth, bounds the level launches.
// A record holds the addresses themselves, so a CTA loads its task offset,
// then the record (one cache line for up to 12 actions), then the data.
//
// Record layout (uint32 words, 16-byte aligned; task lists hold record
// offsets in 16-byte units):
//   [0] regQ   regret / strategy rows of the node (quads)
//   [1] rowQ   backward: the node's value row; forward: its reach row in
//              the traverser's layout (quads)
//   [2] n | na << 16 | own << 24   combos of the row's side, actions,
//              own = 1 when the traverser acts (backward update)
//   [3] chunk | spot << 16         quad chunk (kRecQuads quads: one warp's
//              lanes), spot slot
//   [4 + a]    action a's child row: backward its value row, forward its
//              reach row in the traverser's layout (quads)
// The arithmetic is decideChunk's / fwdDecideChunk's (the reference's
// cuda/gpu_cfr.cu:240-263 and 479-523).
#pragma once

#include "kernels.cuh"

namespace pps {
namespace gb {

__host__ __device__ inline int recordWords(int na) { return (4 + na + 3) / 4 * 4; }

// Regret matching+ with one reciprocal per combo: sigma_a = max(x_a, 0) /
// acc (the reference's cuda/gpu_cfr.cu:245-262 and 479-500), uniform where
// acc = 0. The quotient comes from r = RN(1 / acc), computed once per
// combo, and one correction step (Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990): q0 = RN(x r), e = RN(x - q0 acc) exactly by an fma, q = RN(q0 +
// e r). With r the correctly rounded reciprocal and no overflow or
// underflow on the way (0 < x <= acc, regrets far from both limits), q is
// the correctly rounded quotient: the same sigma as a division, bit for
// bit, for three instructions instead of a division per action.
__device__ __forceinline__ float rmInv(float acc) { return acc > 0.f ? __frcp_rn(acc) : 0.f; }
__device__ __forceinline__ float rmSigma(float x, float acc, float inv, float uniform) {
  if (!(acc > 0.f)) return uniform;
  if (!(x > 0.f)) return 0.f;
  const float q0 = __fmul_rn(x, inv);
  const float e = __fmaf_rn(-q0, acc, x);
  return __fmaf_rn(e, inv, q0);
}

// rmSigma for two lanes: the quotient of both by packed f32x2 instructions
// (each lane rounded exactly as the scalar form rounds it; x - q0 acc as
// q0 (-acc) + x, the same single rounding), then each lane's cases.
__device__ __forceinline__ float2 rmSigma2(float2 x, float2 acc, float2 negAcc, float2 inv,
                                           float uniform) {
  const float2 q0 = __fmul2_rn(x, inv);
  const float2 e = __ffma2_rn(q0, negAcc, x);
  const float2 q = __ffma2_rn(e, inv, q0);
  float2 s;
  s.x = !(acc.x > 0.f) ? uniform : !(x.x > 0.f) ? 0.f : q.x;
  s.y = !(acc.y > 0.f) ? uniform : !(x.y > 0.f) ? 0.f : q.y;
  return s;
}

// DCFR coefficients of the iteration and the uniform strategy of the node.
struct RecCoef {
  float pos, neg, avg, uniform;
};
// One traverser decide record's update, a lane's four combos as two f32x2
// pairs: regret matching, the node value, then per action the strategy sums
// and the regrets, by the formulas of the per-node form (kernels.cuh
// decideChunk; the reference's cuda/gpu_cfr.cu:479-523), each lane rounded
// as the scalar operation would round it. RQ(a),
// SQ(a), CQ(a) give the lane's regret, strategy and child value quads of
// action a (a shared-memory stage or the global rows).
template <typename RQ, typename SQ, typename CQ>
__device__ __forceinline__ void recordUpdatePackedBy(RQ Rq, SQ Sq, CQ Cq, int na,
                                                     const bool (&live)[4], RecCoef k,
                                                     float* out, float* reg, float* str,
                                                     float* strLo, int nq, int q) {
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int a = 0; a < na; ++a) {
    const float4 x = Rq(a);
    acc[0] += x.x > 0.f ? x.x : 0.f;
    acc[1] += x.y > 0.f ? x.y : 0.f;
    acc[2] += x.z > 0.f ? x.z : 0.f;
    acc[3] += x.w > 0.f ? x.w : 0.f;
  }
  const float2 A0 = make_float2(acc[0], acc[1]), A1 = make_float2(acc[2], acc[3]);
  const float2 N0 = make_float2(-acc[0], -acc[1]), N1 = make_float2(-acc[2], -acc[3]);
  const float2 I0 = make_float2(rmInv(acc[0]), rmInv(acc[1]));
  const float2 I1 = make_float2(rmInv(acc[2]), rmInv(acc[3]));
  auto sigma = [&](const float4& x, float2& s0, float2& s1) {
    s0 = rmSigma2(make_float2(x.x, x.y), A0, N0, I0, k.uniform);
    s1 = rmSigma2(make_float2(x.z, x.w), A1, N1, I1, k.uniform);
    if (!live[0]) s0.x = 0.f;
    if (!live[1]) s0.y = 0.f;
    if (!live[2]) s1.x = 0.f;
    if (!live[3]) s1.y = 0.f;
  };
  float2 V0 = make_float2(0.f, 0.f), V1 = make_float2(0.f, 0.f);
  for (int a = 0; a < na; ++a) {
    float2 s0, s1;
    sigma(Rq(a), s0, s1);
    const float4 c = Cq(a);
    V0 = __ffma2_rn(s0, make_float2(c.x, c.y), V0);
    V1 = __ffma2_rn(s1, make_float2(c.z, c.w), V1);
  }
  *reinterpret_cast<float4*>(out + 4 * q) = make_float4(V0.x, V0.y, V1.x, V1.y);
  const float2 NV0 = make_float2(-V0.x, -V0.y), NV1 = make_float2(-V1.x, -V1.y);
  const float2 avg2 = make_float2(k.avg, k.avg);
  for (int a = 0; a < na; ++a) {
    const size_t o = ((size_t)a * nq + q) * 4;
    const float4 rg = Rq(a), sg = Sq(a), c = Cq(a);
    float2 s0, s1;
    sigma(rg, s0, s1);
    float4 sgo;
    if (strLo) {
      float sv[4] = {sg.x, sg.y, sg.z, sg.w}, lo[4];
      ldq(strLo + o, lo);
      const float sl[4] = {s0.x, s0.y, s1.x, s1.y};
      for (int l = 0; l < 4; ++l) stratComp(sv[l], lo[l], k.avg, sl[l]);
      stq(strLo + o, lo);
      sgo = make_float4(sv[0], sv[1], sv[2], sv[3]);
    } else {
      const float2 g0 = __ffma2_rn(make_float2(sg.x, sg.y), avg2, s0);
      const float2 g1 = __ffma2_rn(make_float2(sg.z, sg.w), avg2, s1);
      sgo = make_float4(g0.x, g0.y, g1.x, g1.y);
    }
    const float2 d0 = __fadd2_rn(make_float2(c.x, c.y), NV0);
    const float2 d1 = __fadd2_rn(make_float2(c.z, c.w), NV1);
    const float2 f0 = make_float2(rg.x >= 0.f ? k.pos : k.neg, rg.y >= 0.f ? k.pos : k.neg);
    const float2 f1 = make_float2(rg.z >= 0.f ? k.pos : k.neg, rg.w >= 0.f ? k.pos : k.neg);
    const float2 r0 = __ffma2_rn(make_float2(rg.x, rg.y), f0, d0);
    const float2 r1 = __ffma2_rn(make_float2(rg.z, rg.w), f1, d1);
    *reinterpret_cast<float4*>(str + o) = sgo;
    *reinterpret_cast<float4*>(reg + o) = make_float4(r0.x, r0.y, r1.x, r1.y);
  }
}

// The update from the record's shared-memory stage: entry a of the lane at
// R[a * stride], S[a * stride], C[a * stride].
__device__ __forceinline__ void recordUpdatePacked(const float4* R, const float4* S,
                                                   const float4* C, int stride, int na,
                                                   const bool (&live)[4], RecCoef k,
                                                   float* out, float* reg, float* str,
                                                   float* strLo, int nq, int q) {
  recordUpdatePackedBy([&](int a) { return R[a * stride]; }, [&](int a) { return S[a * stride]; },
                       [&](int a) { return C[a * stride]; }, na, live, k, out, reg, str, strLo,
                       nq, q);
}

struct DecRec {
  uint32_t regQ, rowQ;
  int n, na, own, chunk, spot;
  const uint32_t* kid;
  const uint32_t* pre;  // folded-in children (header bit 25), else nullptr
};

// A level's record offsets as up to four arithmetic runs (records grouped
// by size class): run j covers the indices [end[j - 1], end[j]) at base[j] +
// (k - end[j - 1]) stride[j] (16-byte units).
struct RecRuns {
  uint32_t end[4], base[4], stride[4];
};
// Offset of record k: from the level's offset list, or (list null) from
// its runs.
__device__ __forceinline__ uint32_t recOffset(const uint32_t* __restrict__ recTasks,
                                              const RecRuns& R, int k) {
  if (recTasks) return recTasks[k];
  const uint32_t u = (uint32_t)k;
  if (u < R.end[0]) return R.base[0] + u * R.stride[0];
  if (u < R.end[1]) return R.base[1] + (u - R.end[0]) * R.stride[1];
  if (u < R.end[2]) return R.base[2] + (u - R.end[1]) * R.stride[2];
  return R.base[3] + (u - R.end[2]) * R.stride[3];
}

__device__ __forceinline__ DecRec loadRec(const uint32_t* __restrict__ recs, uint32_t off16) {
  const uint32_t* r = recs + (size_t)off16 * 4;
  const uint4 h = *reinterpret_cast<const uint4*>(r);
  DecRec d;
  d.regQ = h.x;
  d.rowQ = h.y;
  d.n = (int)(h.z & 0xffff);
  d.na = (int)((h.z >> 16) & 0xff);
  d.own = (int)((h.z >> 24) & 1);
  d.chunk = (int)(h.w & 0xffff);
  d.spot = (int)(h.w >> 16);
  d.kid = r + 4;
  d.pre = (h.z >> 25) & 1 ? r + 4 + d.na : nullptr;
  return d;
}

// Folded-in children of a traverser record (layout.cpp, buildBackwardLevels):
// for each, the lane's quad of its value row = the sum of its children's,
// in action order, padding lanes zero - exactly what that child's own
// record computes (the opponent branch of decideRecord) - written before
// the record reads its children's rows. Each lane writes only its own
// quad; the caller orders the writes before reads by other lanes or by the
// bulk-copy engine.
__device__ __forceinline__ void recordFoldedChildren(const DevRows<float>& rows, const DecRec& r,
                                                     int lane) {
  if (!r.pre) return;
  const int nq = quadsOf(r.n);
  const int q = r.chunk * kRecQuads + lane;
  const uint32_t* p = r.pre;
  const int P = (int)p[0];
  ++p;
  for (int e = 0; e < P; ++e) {
    const uint32_t row = p[0];
    const int m = (int)p[1];
    p += 2;
    if (q < nq) {
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      for (int b = 0; b < m; ++b) {
        float c[4];
        ldq(rows.cfv + (size_t)p[b] * 4 + 4 * q, c);
        for (int l = 0; l < 4; ++l) v[l] += c[l];
      }
      for (int l = 0; l < 4; ++l)
        if (4 * q + l >= r.n) v[l] = 0.f;
      stq(rows.cfv + (size_t)row * 4 + 4 * q, v);
    }
    p += m;
  }
  // The rows just written are read next by copies of the async proxy (bulk
  // and cp.async staging) and by other lanes.
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Asks for the low words of a record's strategy rows ahead of the update
// (an L2 hint, no data): they are read only there, by plain loads.
__device__ __forceinline__ void prefetchStratLo(const DevTree& t, const DecRec& r, int q, int nq) {
  if (!t.stratLo) return;
  const float* lo = t.stratLo + (size_t)r.regQ * 4;
  for (int a = 0; a < r.na; ++a)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(lo + ((size_t)a * nq + q) * 4));
}

// Actions of a record staged in shared memory (larger records stream).
constexpr int kAsyncNa = 4;

__device__ __forceinline__ void cpAsync16(float4* smem, const float* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cpAsyncWaitAll() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}
__device__ __forceinline__ void ld4s(const float4* p, float (&x)[4]) {
  const float4 v = *p;
  x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
}

// recordFoldedChildren through free stage entries of the record: per
// folded-in child, the lane's quads of up to `slots` of its children are
// copied with cp.async (all in flight at once, no registers held) and
// summed from the stage in the children's order, so a child costs one
// memory round trip per `slots` grandchildren instead of one per
// grandchild. Entry j of the lane lives at C[j * stride + slot]; each
// thread reads back only its own entries. The sums are bitwise those of
// recordFoldedChildren.
__device__ __forceinline__ void recordFoldedChildrenStaged(const DevRows<float>& rows,
                                                           const DecRec& r, int lane, float4* C,
                                                           int stride, int slot, int slots) {
  if (!r.pre) return;
  const int nq = quadsOf(r.n);
  const int q = r.chunk * kRecQuads + lane;
  const uint32_t* p = r.pre;
  const int P = (int)p[0];
  ++p;
  for (int e = 0; e < P; ++e) {
    const uint32_t row = p[0];
    const int m = (int)p[1];
    p += 2;
    if (q < nq) {
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      for (int b0 = 0; b0 < m; b0 += slots) {
        const int k = m - b0 < slots ? m - b0 : slots;
        for (int j = 0; j < k; ++j)
          cpAsync16(&C[j * stride + slot], rows.cfv + (size_t)p[b0 + j] * 4 + 4 * q);
        cpAsyncWaitAll();
        for (int j = 0; j < k; ++j) {
          float c[4];
          ld4s(&C[j * stride + slot], c);
          for (int l = 0; l < 4; ++l) v[l] += c[l];
        }
      }
      for (int l = 0; l < 4; ++l)
        if (4 * q + l >= r.n) v[l] = 0.f;
      stq(rows.cfv + (size_t)row * 4 + 4 * q, v);
    }
    p += m;
  }
  // The rows just written are read next by copies of the async proxy (bulk
  // and cp.async staging) and by other lanes.
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Backward decide record (CFR mode, f32 rows), one warp: lane = quad.
// With a stage (the record's unused shared-memory segments: `slots`
// entries per lane at stage[j * stride + slot]), its folded-in children are
// summed through it.
__device__ __forceinline__ void decideRecord(const DevTree& t, const DevRows<float>& rows,
                                             const DecRec& r, int lane, float4* stage = nullptr,
                                             int stride = 0, int slot = 0, int slots = 0) {
  if (stage) recordFoldedChildrenStaged(rows, r, lane, stage, stride, slot, slots);
  else recordFoldedChildren(rows, r, lane);  // this lane reads back only its own quads
  const int nq = quadsOf(r.n);
  const int q = r.chunk * kRecQuads + lane;
  if (q >= nq) return;
  float* out = rows.cfv + (size_t)r.rowQ * 4;
  bool live[4];
  for (int l = 0; l < 4; ++l) live[l] = 4 * q + l < r.n;
  const int na = r.na;
  if (!r.own) {
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    for (int a = 0; a < na; ++a) {
      float c[4];
      ldq(rows.cfv + (size_t)r.kid[a] * 4 + 4 * q, c);
      for (int l = 0; l < 4; ++l) v[l] += c[l];
    }
    for (int l = 0; l < 4; ++l)
      if (!live[l]) v[l] = 0.f;
    stq(out + 4 * q, v);
    return;
  }
  float* reg = t.regret + (size_t)r.regQ * 4;
  float* str = t.strat + (size_t)r.regQ * 4;
  const float* c3 = t.coef + (size_t)t.counter[r.spot] * 3;
  const float pos = c3[0], neg = c3[1], avg = c3[2];
  const float uniform = 1.f / (float)na;
  // The children's value rows and the strategy rows are needed only after
  // the regret pass: start fetching them into L2 now (a hint, no data).
  for (int a = 0; a < na; ++a) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(rows.cfv + (size_t)r.kid[a] * 4 + 4 * q));
    asm volatile("prefetch.global.L2 [%0];" ::"l"(str + ((size_t)a * nq + q) * 4));
  }
  prefetchStratLo(t, r, q, nq);
  // Streaming form: a row is reloaded (a cache hit) instead of held in
  // registers; the launches are bound by memory latency, not by
  // instruction count. The arithmetic is the staged records' (packed).
  const uint32_t* kid = r.kid;
  const float* cfv = rows.cfv;
  const RecCoef kc{pos, neg, avg, uniform};
  recordUpdatePackedBy(
      [&](int a) { return *reinterpret_cast<const float4*>(reg + ((size_t)a * nq + q) * 4); },
      [&](int a) { return *reinterpret_cast<const float4*>(str + ((size_t)a * nq + q) * 4); },
      [&](int a) { return *reinterpret_cast<const float4*>(cfv + (size_t)kid[a] * 4 + 4 * q); },
      na, live, kc, out, reg, str, t.stratLo ? t.stratLo + (size_t)r.regQ * 4 : nullptr, nq, q);
}

// Forward decide record (opponent node, CFR mode): child reach = reach x
// sigma_a from the regrets (regret matching+).
// Forward record arithmetic (the staged and streaming forms): child reach
// = reach x sigma_a, two lanes per packed f32x2 instruction (each rounded
// as the scalar form rounds it). RQ(a): the lane's regret quad of action a.
template <typename RQ>
__device__ __forceinline__ void fwdRecordPackedBy(RQ Rq, float4 rr, int na, const DecRec& r,
                                                  int tr, const DevRows<float>& rows, int q) {
  const float uniform = 1.f / (float)na;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int a = 0; a < na; ++a) {
    const float4 x = Rq(a);
    acc[0] += x.x > 0.f ? x.x : 0.f;
    acc[1] += x.y > 0.f ? x.y : 0.f;
    acc[2] += x.z > 0.f ? x.z : 0.f;
    acc[3] += x.w > 0.f ? x.w : 0.f;
  }
  const float2 A0 = make_float2(acc[0], acc[1]), A1 = make_float2(acc[2], acc[3]);
  const float2 N0 = make_float2(-acc[0], -acc[1]), N1 = make_float2(-acc[2], -acc[3]);
  const float2 I0 = make_float2(rmInv(acc[0]), rmInv(acc[1]));
  const float2 I1 = make_float2(rmInv(acc[2]), rmInv(acc[3]));
  const float2 rr0 = make_float2(rr.x, rr.y), rr1 = make_float2(rr.z, rr.w);
  for (int a = 0; a < na; ++a) {
    const float4 x = Rq(a);
    float2 o0 = __fmul2_rn(rr0, rmSigma2(make_float2(x.x, x.y), A0, N0, I0, uniform));
    float2 o1 = __fmul2_rn(rr1, rmSigma2(make_float2(x.z, x.w), A1, N1, I1, uniform));
    if (4 * q + 0 >= r.n) o0.x = 0.f;
    if (4 * q + 1 >= r.n) o0.y = 0.f;
    if (4 * q + 2 >= r.n) o1.x = 0.f;
    if (4 * q + 3 >= r.n) o1.y = 0.f;
    *reinterpret_cast<float4*>(rows.reach[tr] + (size_t)r.kid[a] * 4 + 4 * q) =
        make_float4(o0.x, o0.y, o1.x, o1.y);
  }
}

__device__ __forceinline__ void fwdDecideRecord(const DevTree& t, const DevRows<float>& rows,
                                                int tr, const DecRec& r, int lane) {
  const int nq = quadsOf(r.n);
  const int q = r.chunk * kRecQuads + lane;
  if (q >= nq) return;
  const int na = r.na;
  const float* src = t.regret + (size_t)r.regQ * 4;
  // Every action's regret quad requested at once (L1 hints), then read in
  // the regret-matching order.
  for (int a = 0; a < na; ++a)
    asm volatile("prefetch.global.L1 [%0];" ::"l"(src + ((size_t)a * nq + q) * 4));
  const float4 rr = *reinterpret_cast<const float4*>(rows.reach[tr] + (size_t)r.rowQ * 4 + 4 * q);
  fwdRecordPackedBy(
      [&](int a) { return *reinterpret_cast<const float4*>(src + ((size_t)a * nq + q) * 4); }, rr,
      na, r, tr, rows, q);
}

// ---------------------------------------------------------------------------
// Staged records: every row quad a thread needs (the children's value
// quads, and for the traverser's own node its regret and strategy quads;
// forward: its reach quad and regret quads) is requested at once with
// cp.async into shared memory, so a record costs one memory round trip
// instead of three dependent ones, and the data in flight holds no
// registers. Each thread reads back only what it copied (cp.async.wait_group
// waits for the thread's own copies: nothing to spin on). Records with more
// than kAsyncNa actions (8% of the row bytes of the 48,255-node turn spot)
// use the streaming form.
// Layout: [row kind][action][thread] float4, conflict-free.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr size_t recStageBytes() {
  return (size_t)3 * kAsyncNa * kThreads * sizeof(float4);
}


// Backward decide record, staged, first part: the copies of the regret and
// strategy rows of the traverser's own node (nothing for another node or a
// record that is not staged). Those rows are written only by the backward
// pass of this level in an earlier iteration, so the copies may go out
// before the wait for the previous level.
__device__ __forceinline__ void decideRecordOwnRows(const DevTree& t, const DecRec& r, int lane,
                                                    float4* stage) {
  const int na = r.na;
  if (na > kAsyncNa || !r.own) return;
  const int nq = quadsOf(r.n);
  const int q = r.chunk * kRecQuads + lane;
  if (q >= nq) return;
  const int tid = (int)threadIdx.x;
  float4* R = stage + kAsyncNa * kThreads;
  float4* S = R + kAsyncNa * kThreads;
  const float* reg = t.regret + (size_t)r.regQ * 4;
  const float* str = t.strat + (size_t)r.regQ * 4;
  for (int a = 0; a < na; ++a) {
    const size_t o = ((size_t)a * nq + q) * 4;
    cpAsync16(&R[a * kThreads + tid], reg + o);
    cpAsync16(&S[a * kThreads + tid], str + o);
  }
  prefetchStratLo(t, r, q, nq);
}

// Backward decide record, staged (same arithmetic and order as
// decideRecord), after decideRecordOwnRows and the wait for the previous
// level: the child value copies, then the update.
__device__ __forceinline__ void decideRecordStaged(const DevTree& t, const DevRows<float>& rows,
                                                   const DecRec& r, int lane, float4* stage) {
  const int na = r.na;
  const int tid = (int)threadIdx.x;
  if (na > kAsyncNa) {  // streams; its stage entries are free
    decideRecord(t, rows, r, lane, stage, kThreads, tid, 3 * kAsyncNa);
    return;
  }
  recordFoldedChildrenStaged(rows, r, lane, stage, kThreads, tid, kAsyncNa);
  const int nq = quadsOf(r.n);
  const int q = r.chunk * kRecQuads + lane;
  if (q >= nq) return;
  float4* C = stage;
  float4* R = stage + kAsyncNa * kThreads;
  float4* S = R + kAsyncNa * kThreads;
  for (int a = 0; a < na; ++a)
    cpAsync16(&C[a * kThreads + tid], rows.cfv + (size_t)r.kid[a] * 4 + 4 * q);
  float* out = rows.cfv + (size_t)r.rowQ * 4;
  bool live[4];
  for (int l = 0; l < 4; ++l) live[l] = 4 * q + l < r.n;
  if (!r.own) {
    cpAsyncWaitAll();
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    for (int a = 0; a < na; ++a) {
      float c[4];
      ld4s(&C[a * kThreads + tid], c);
      for (int l = 0; l < 4; ++l) v[l] += c[l];
    }
    for (int l = 0; l < 4; ++l)
      if (!live[l]) v[l] = 0.f;
    stq(out + 4 * q, v);
    return;
  }
  float* reg = t.regret + (size_t)r.regQ * 4;
  float* str = t.strat + (size_t)r.regQ * 4;
  const float* c3 = t.coef + (size_t)t.counter[r.spot] * 3;
  const RecCoef kc{c3[0], c3[1], c3[2], 1.f / (float)na};
  cpAsyncWaitAll();
  recordUpdatePacked(R + tid, S + tid, C + tid, kThreads, na, live, kc, out, reg, str,
                     t.stratLo ? t.stratLo + (size_t)r.regQ * 4 : nullptr, nq, q);
}

// Forward decide record, first part: the copies of the node's regret rows
// into the staging buffer (a no-op for records that are not staged).
__device__ __forceinline__ void fwdRecordRegrets(const DevTree& t, const DecRec& r, int lane,
                                                 float4* stage) {
  const int na = r.na;
  if (na > kAsyncNa) return;
  const int nq = quadsOf(r.n);
  const int q = r.chunk * kRecQuads + lane;
  if (q >= nq) return;
  float4* R = stage + kThreads;  // [action][thread]
  const float* src = t.regret + (size_t)r.regQ * 4;
  for (int a = 0; a < na; ++a)
    cpAsync16(&R[a * kThreads + (int)threadIdx.x], src + ((size_t)a * nq + q) * 4);
}

// Forward decide record, staged (same arithmetic and order as
// fwdDecideRecord). regretsIssued: fwdRecordRegrets already ran for this
// record.
__device__ __forceinline__ void fwdDecideRecordStaged(const DevTree& t, const DevRows<float>& rows,
                                                      int tr, const DecRec& r, int lane,
                                                      float4* stage, bool regretsIssued) {
  const int na = r.na;
  if (na > kAsyncNa) {
    fwdDecideRecord(t, rows, tr, r, lane);
    return;
  }
  const int nq = quadsOf(r.n);
  const int q = r.chunk * kRecQuads + lane;
  if (q >= nq) return;
  const int tid = (int)threadIdx.x;
  float4* RR = stage;                     // [thread]
  float4* R = stage + kThreads;           // [action][thread]
  cpAsync16(&RR[tid], rows.reach[tr] + (size_t)r.rowQ * 4 + 4 * q);
  if (!regretsIssued) fwdRecordRegrets(t, r, lane, stage);
  cpAsyncWaitAll();
  fwdRecordPackedBy([&](int a) { return R[a * kThreads + tid]; }, RR[tid], na, r, tr, rows, q);
}

// ---------------------------------------------------------------------------
// Backward records staged by the bulk-copy engine: lane 0 of the warp asks
// for every row segment of its record (up to 32 quads of each child value
// row, and for the traverser's own node of each regret and strategy row)
// with cp.async.bulk, counted on the warp's mbarrier; the lanes wait on the
// barrier and compute from shared memory as decideRecordStaged does. The
// wait is bounded: after kBarSpins polls the warp drains, records an error
// in the device error word and leaves the record, so a wait can never hang;
// that warp's later records (persistent grids) skip their copies.
// Layout per warp: [row kind][action][32 quads], contiguous segments.
//
// The record waits for the previous level itself (griddepcontrol.wait),
// between its two groups of copies. The regret and strategy rows of the
// traverser's own node are written by this pass at this level only, in an
// earlier iteration, and every iteration ends with a launch that has no
// programmatic dependency (advanceCounterK), so those writes are complete
// when the record starts: their copies go out before the wait and overlap
// the previous level's tail. The child value rows are the previous level's
// output: their copies go out after the wait.
// ---------------------------------------------------------------------------
constexpr int kBarSpins = 1 << 16;
// Rounds of kBarSpins polls that a warp whose wait ran out spends draining
// its own copies before it leaves the record.
constexpr int kDrainRounds = 4;

__device__ __forceinline__ void pdlTrigger() { asm volatile("griddepcontrol.launch_dependents;"); }
__device__ __forceinline__ void pdlWait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void barInit(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smemAddr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void barExpect(unsigned long long* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulkLoad(void* dst, const float* src, uint32_t bytes,
                                         unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smemAddr(dst)),
      "l"(src), "r"(bytes), "r"(smemAddr(bar))
      : "memory");
}
// True once the barrier's phase `parity` completed; false after kBarSpins
// polls (each poll may itself wait a little: try_wait has a time limit).
__device__ __forceinline__ bool barWait(unsigned long long* bar, uint32_t parity,
                                        int spins = kBarSpins) {
  for (int i = 0; i < spins; ++i) {
    uint32_t done = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smemAddr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// A warp's wait for the copies it issued on its barrier, bounded: true once
// they landed (every lane agrees). Otherwise it drains - waits for the same
// copies for up to kDrainRounds more rounds, so that the CTA does not leave
// with asynchronous writes into its shared memory in flight - sets the
// device error word (bit 1: the wait ran out; bit 2 as well: the drain ran
// out too, and the copies may outlive the CTA) and returns false.
__device__ __forceinline__ bool warpCopiesLanded(unsigned long long* bar, uint32_t parity, int* err,
                                                 int lane, int spins = kBarSpins) {
  if (__all_sync(0xffffffffu, barWait(bar, parity, spins))) return true;
  bool drained = false;
  for (int k = 0; k < kDrainRounds && !drained; ++k) drained = barWait(bar, parity, spins);
  if (lane == 0 && err) atomicOr(err, drained ? 1 : 3);
  return false;
}

// stage: this warp's segments; bar: this warp's barrier; phase: the
// barrier's next parity (flipped here).
__device__ __forceinline__ void decideRecordBulk(const DevTree& t, const DevRows<float>& rows,
                                                 const DecRec& r, int lane, float4* stage,
                                                 unsigned long long* bar, uint32_t& phase,
                                                 bool& broken) {
  const int na = r.na;
  if (na > kAsyncNa) {  // streams; the warp's stage is free
    pdlWait();
    decideRecord(t, rows, r, lane, stage, kRecQuads, lane, 3 * kAsyncNa);
    return;
  }
  const int nq = quadsOf(r.n);
  const int q0 = r.chunk * kRecQuads;
  const int segQ = nq - q0 < kRecQuads ? nq - q0 : kRecQuads;  // >= 1: the record exists
  const uint32_t segBytes = (uint32_t)segQ * 16u;
  float4* C = stage;
  float4* R = stage + kAsyncNa * kRecQuads;
  float4* S = R + kAsyncNa * kRecQuads;
  float* reg = t.regret + (size_t)r.regQ * 4;
  float* str = t.strat + (size_t)r.regQ * 4;
  // A warp whose barrier wait gave up on an earlier record issues no more
  // copies (its barrier may still count that record's); warp-uniform.
  if (broken) return;
  __syncwarp();  // the lanes' reads of the last record's segments are done
  if (lane == 0) {
    // Earlier reads of the stage (generic proxy) before the copies (async proxy).
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    barExpect(bar, segBytes * (uint32_t)(r.own ? 3 * na : na));
    if (r.own)
      for (int a = 0; a < na; ++a) {
        const size_t o = ((size_t)a * nq + q0) * 4;
        bulkLoad(&R[a * kRecQuads], reg + o, segBytes, bar);
        bulkLoad(&S[a * kRecQuads], str + o, segBytes, bar);
      }
  }
  if (r.own && q0 + lane < nq) prefetchStratLo(t, r, q0 + lane, nq);
  pdlWait();
  if (r.pre) {  // folded-in children: every lane's quads written before lane 0's copies
    recordFoldedChildrenStaged(rows, r, lane, C, kRecQuads, lane, kAsyncNa);
    __syncwarp();
    // The lanes' reads of C (generic proxy) before the child copies into it
    // (async proxy).
    if (lane == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (lane == 0)
    for (int a = 0; a < na; ++a)
      bulkLoad(&C[a * kRecQuads], rows.cfv + ((size_t)r.kid[a] + q0) * 4, segBytes, bar);
  const uint32_t parity = phase;
  phase ^= 1u;
  if (!warpCopiesLanded(bar, parity, t.err, lane)) {
    // The host discards the launch's results.
    broken = true;
    return;
  }
  const int q = q0 + lane;
  if (q >= nq) return;
  float* out = rows.cfv + (size_t)r.rowQ * 4;
  bool live[4];
  for (int l = 0; l < 4; ++l) live[l] = 4 * q + l < r.n;
  if (!r.own) {
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    for (int a = 0; a < na; ++a) {
      float c[4];
      ld4s(&C[a * kRecQuads + lane], c);
      for (int l = 0; l < 4; ++l) v[l] += c[l];
    }
    for (int l = 0; l < 4; ++l)
      if (!live[l]) v[l] = 0.f;
    stq(out + 4 * q, v);
    return;
  }
  const float* c3 = t.coef + (size_t)t.counter[r.spot] * 3;
  const RecCoef kc{c3[0], c3[1], c3[2], 1.f / (float)na};
  recordUpdatePacked(R + lane, S + lane, C + lane, kRecQuads, na, live, kc, out, reg, str,
                     t.stratLo ? t.stratLo + (size_t)r.regQ * 4 : nullptr, nq, q);
}

// ---------------------------------------------------------------------------
// Chance records (layout.cpp): the arithmetic of fwdChanceBranch /
// chanceChunk (kernels.cuh) with every address resolved on the host. The
// record header is static data, read before the kernel waits for the
// previous grid.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 loadChanceHeader(const uint32_t* __restrict__ recs,
                                                  uint32_t off16) {
  return *reinterpret_cast<const uint4*>(recs + (size_t)off16 * 4);
}

// Forward: child reach = parent reach through the child -> parent slot map,
// scaled by 1 / chanceQ (cuda/gpu_cfr.cu:276-293). The slot map is static:
// before the wait for the previous level, each thread copies its own
// entries of it into shared memory (fwdChanceSlots); after the wait, one
// dependent load per entry remains.
__device__ __forceinline__ bool fwdChanceStaged(uint4 h, size_t stageBytes) {
  return (size_t)quadsOf((int)(h.w & 0xffff)) * 4 * sizeof(uint16_t) <= stageBytes;
}
// Thread t copies the entries of the quads it writes in fwdChanceRecord
// (quads t, t + blockDim.x, ...), so it reads back only its own copies.
__device__ __forceinline__ void fwdChanceSlots(const DevTree& t, uint4 h, uint16_t* upS) {
  const int nc = (int)(h.w & 0xffff);
  const uint16_t* up = t.poolU16 + h.z;
  for (int q = threadIdx.x; q < quadsOf(nc); q += blockDim.x) {
    uint16_t v[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) v[l] = 4 * q + l < nc ? up[4 * q + l] : (uint16_t)0;
#pragma unroll
    for (int l = 0; l < 4; ++l)
      if (4 * q + l < nc) upS[4 * q + l] = v[l];
  }
}
__device__ __forceinline__ void fwdChanceRecord(const DevTree& t, const DevRows<float>& rows,
                                                int tr, uint4 h, const uint16_t* upS) {
  const int nc = (int)(h.w & 0xffff);
  const float inv = 1.f / (float)(h.w >> 16);
  const uint16_t* up = upS ? upS : t.poolU16 + h.z;
  const float* pr = rows.reach[tr] + (size_t)h.x * 4;
  float* cr = rows.reach[tr] + (size_t)h.y * 4;
  for (int q = threadIdx.x; q < quadsOf(nc); q += blockDim.x) {
    float out[4];
    for (int l = 0; l < 4; ++l) {
      const int j = 4 * q + l;
      out[l] = j < nc ? pr[up[j]] * inv : 0.f;
    }
    stq(cr + 4 * q, out);
  }
}

// Backward, first part (static data, before the wait): the branch table
// into shared memory (child value rows and parent -> child slot maps).
// Layout: rowOf[64] | downOf[64] | slot[64][kChanceChunk] (int16).
constexpr int kChanceMaxBranches = 64;  // a chance node has at most 49 branches
constexpr size_t kChanceStageBytes =
    kChanceScratchBytes + (size_t)kChanceMaxBranches * kChanceChunk * sizeof(int16_t);
__device__ __forceinline__ void chanceRecordTables(const DevTree& t, const DevRows<float>& rows,
                                                   const uint32_t* __restrict__ recs, uint4 h,
                                                   unsigned char* smem) {
  const int nb = (int)(h.y >> 16);
  const uint32_t* tab = recs + (size_t)h.w * 4;
  const float** rowOf = reinterpret_cast<const float**>(smem);
  const int16_t** downOf = reinterpret_cast<const int16_t**>(smem + 64 * sizeof(void*));
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    rowOf[b] = rows.cfv + (size_t)tab[2 * b] * 4;
    downOf[b] = t.poolI16 + tab[2 * b + 1];
  }
}

// Backward, second part (static data, after a __syncthreads, still before
// the wait): each thread's slot in every branch's child row, slot[b][thread]
// (-1: the branch blocks the combo). A thread reads back only its own
// column.
__device__ __forceinline__ void chanceRecordSlots(uint4 h, unsigned char* smem) {
  const int n = (int)(h.y & 0xffff), nb = (int)(h.y >> 16);
  const int16_t* const* downOf =
      reinterpret_cast<const int16_t* const*>(smem + 64 * sizeof(void*));
  int16_t* slot = reinterpret_cast<int16_t*>(smem + kChanceScratchBytes);
  const int i = (int)h.z * kChanceChunk + (int)threadIdx.x;
  if (i >= n) return;
  for (int b0 = 0; b0 < nb; b0 += 16) {  // 16 loads in flight, then their stores
    int16_t v[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = b0 + j < nb ? downOf[b0 + j][i] : (int16_t)-1;
#pragma unroll
    for (int j = 0; j < 16; ++j)
      if (b0 + j < nb) slot[(b0 + j) * kChanceChunk + threadIdx.x] = v[j];
  }
}

// Backward, last part (after the wait): parent value of one 128-combo
// chunk = sum over the branches in branch order (cuda/gpu_cfr.cu:542-554),
// 16 branch loads in flight per thread.
constexpr int kChanceBatch = 24;
__device__ __forceinline__ void chanceRecordSum(const DevRows<float>& rows, uint4 h,
                                                const unsigned char* smem) {
  const int n = (int)(h.y & 0xffff), nb = (int)(h.y >> 16);
  const float* const* rowOf = reinterpret_cast<const float* const*>(smem);
  const int16_t* slot = reinterpret_cast<const int16_t*>(smem + kChanceScratchBytes);
  float* out = rows.cfv + (size_t)h.x * 4;
  const int i = (int)h.z * kChanceChunk + (int)threadIdx.x;
  if (i >= quadsOf(n) * 4) return;
  float v = 0.f;
  if (i < n) {
    for (int b0 = 0; b0 < nb; b0 += kChanceBatch) {
      float x[kChanceBatch];
#pragma unroll
      for (int j = 0; j < kChanceBatch; ++j) {
        const int k = b0 + j < nb ? slot[(b0 + j) * kChanceChunk + threadIdx.x] : -1;
        x[j] = k >= 0 ? rowOf[b0 + j][k] : 0.f;
      }
#pragma unroll
      for (int j = 0; j < kChanceBatch; ++j) v += x[j];
    }
  }
  out[i] = v;
}

// One warp per record, kRecWarps records per CTA. A warp's records are
// independent of its CTA's other warps: no barrier.
constexpr int kRecWarps = kThreads / 32;
__host__ __device__ inline int recordCtas(int records) {
  return (records + kRecWarps - 1) / kRecWarps;
}

// Dynamic shared memory of the record kernels: the staging buffers
// (forward: one reach quad and kAsyncNa regret quads per thread).
__host__ __device__ constexpr size_t fwdStageBytes() {
  return (size_t)(1 + kAsyncNa) * kThreads * sizeof(float4);
}
// Backward: the staging buffers (records, or a chance chunk's tables),
// then one mbarrier per warp.
__host__ __device__ constexpr size_t bwdStageBytes() {
  return (recStageBytes() > kChanceStageBytes ? recStageBytes() : kChanceStageBytes) +
         kRecWarps * sizeof(unsigned long long);
}

// ---------------------------------------------------------------------------
// Level kernels of the default iteration: one launch per level and pass
// covering the level's chance records and decide records (CTA i < nCh: one
// chance record, started first because its chain of loads is the longest;
// else one decide record per warp),
// launched with programmatic dependent
// launch so consecutive levels overlap: each CTA lets the next level's grid
// start (launch_dependents), loads its record (static data), then waits
// until the previous level's grid has finished and its writes are visible
// (griddepcontrol.wait) before touching rows. Without a programmatic
// dependency the wait returns at once. A backward decide record also asks
// for its own node's regret and strategy rows before the wait
// (decideRecordBulk).
// ---------------------------------------------------------------------------

// late: each CTA lets the next grid launch only once its own wait has
// returned (so a grid that has launched implies that the grid two places
// before it has completed; the fused plan relies on that), instead of at
// its start.
// recTasks (chance) null: the level's records are recBase + k recStride
// (chBase + i chStride; 16-byte units), at one stride from the first.
// early: the records ask for their regret rows before the wait. Only for
// the first half-step of an iteration (traverser 0): the regrets it reads
// are the other player's, written by the second half-step of an earlier
// iteration, and every iteration ends with a launch that has no
// programmatic dependency (advanceCounterK). The second half-step reads
// regrets that the first one has just written.
static __global__ void __launch_bounds__(kThreads, 10)
fwdLevelMixK(DevTree t, DevRows<float> rows, const uint32_t* __restrict__ recs,
             const uint32_t* __restrict__ recTasks, int nRec, const uint32_t* __restrict__ chance,
             int nCh, int tr, int late, int early, uint32_t recBase, uint32_t recStride,
             uint32_t chBase, uint32_t chStride) {
  extern __shared__ __align__(16) unsigned char smem[];
  float4* stage = reinterpret_cast<float4*>(smem);
  if (!late) pdlTrigger();
  const int nRc = recordCtas(nRec), lane = (int)threadIdx.x & 31;
  bool waited = false;
  for (int i = blockIdx.x; i < nCh + nRc; i += gridDim.x) {
    // A CTA that runs more than one task (grids past 2^20 CTAs) must not
    // overwrite shared memory that its threads still read for the last one.
    if (i != (int)blockIdx.x) __syncthreads();
    if (i >= nCh) {
      const int k = (i - nCh) * kRecWarps + (int)(threadIdx.x >> 5);
      if (k >= nRec) continue;
      const DecRec r = loadRec(recs, recTasks ? recTasks[k] : recBase + (uint32_t)k * recStride);
      if (early) fwdRecordRegrets(t, r, lane, stage);
      pdlWait();
      waited = true;
      fwdDecideRecordStaged(t, rows, tr, r, lane, stage, early != 0);
    } else {
      const uint4 h = loadChanceHeader(recs, chance ? chance[i] : chBase + (uint32_t)i * chStride);
      const bool st = fwdChanceStaged(h, fwdStageBytes());
      uint16_t* upS = reinterpret_cast<uint16_t*>(smem);
      if (st) fwdChanceSlots(t, h, upS);
      pdlWait();
      waited = true;
      fwdChanceRecord(t, rows, tr, h, st ? upS : nullptr);
    }
    if (late) pdlTrigger();
  }
  if (late && !waited) {  // an idle warp of a record CTA
    pdlWait();
    pdlTrigger();
  }
}

static __global__ void __launch_bounds__(kThreads, 8)
bwdLevelMixK(DevTree t, DevRows<float> rows, const uint32_t* __restrict__ recs,
             const uint32_t* __restrict__ recTasks, int nRec, const uint32_t* __restrict__ chance,
             int nCh, int tr, RecRuns runs) {
  extern __shared__ __align__(16) unsigned char smem[];  // bwdStageBytes()
  pdlTrigger();
  const int nRc = recordCtas(nRec), lane = (int)threadIdx.x & 31;
  const int warp = (int)(threadIdx.x >> 5);
  unsigned long long* bar =
      reinterpret_cast<unsigned long long*>(smem + bwdStageBytes()) - kRecWarps + warp;
  if (lane == 0) barInit(bar);
  __syncwarp();
  uint32_t phase = 0;
  bool broken = false;
  for (int i = blockIdx.x; i < nCh + nRc; i += gridDim.x) {
    // A CTA that runs more than one task (grids past 2^20 CTAs) must not
    // overwrite shared memory that its warps still read for the last one.
    if (i != (int)blockIdx.x) __syncthreads();
    if (i >= nCh) {
      const int k = (i - nCh) * kRecWarps + (int)(threadIdx.x >> 5);
      if (k >= nRec) continue;
      const DecRec r = loadRec(recs, recOffset(recTasks, runs, k));
      decideRecordBulk(t, rows, r, lane,  // waits for the previous level itself
                       reinterpret_cast<float4*>(smem) + warp * 3 * kAsyncNa * kRecQuads, bar,
                       phase, broken);
    } else {
      const uint4 h = loadChanceHeader(recs, chance[i]);
      chanceRecordTables(t, rows, recs, h, smem);
      __syncthreads();
      chanceRecordSlots(h, smem);
      pdlWait();
      chanceRecordSum(rows, h, smem);
      __syncthreads();  // the next chance task reuses the pointer tables
    }
  }
}

}  // namespace gb
}  // namespace pps
