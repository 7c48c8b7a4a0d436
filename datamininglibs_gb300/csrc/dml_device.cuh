// Device numerics shared by the fit and predict kernels.
//
// Every floating-point step that decides a split is written with explicit
// round-to-nearest intrinsics (no contraction, fixed order) so that the gains
// are bit-identical to a host computation that performs the same operations
// one at a time.  The recipes:
//   * Philox4x32-10 counter-based RNG (Salmon, Moraes, Dror, Shaw, SC'11)
//   * entropy gain (bits) of a 2 x C table, restating lib_ensembles/source/
//     gpudte.cu:70-117, evaluated as float-float sums of an n*ln(n) table
//   * variance gain nL*nR*(mL-mR)^2/(nL+nR) (lib_ensembles/source/gpuert.cu:
//     363-378) from exact 64-bit fixed-point target sums, in float-float
#pragma once
#include <cfloat>
#include <cstdint>

#include "dml_internal.h"

namespace dml {

// ------------------------------------------------------------------ Philox
struct U4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                            uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t h0 = __umulhi(0xD2511F53u, c0), l0 = 0xD2511F53u * c0;
    uint32_t h1 = __umulhi(0xCD9E8D57u, c2), l1 = 0xCD9E8D57u * c2;
    uint32_t n0 = h1 ^ c1 ^ k0;
    uint32_t n2 = h0 ^ c3 ^ k1;
    c0 = n0;
    c1 = l1;
    c2 = n2;
    c3 = l0;
  }
  return U4{c0, c1, c2, c3};
}

enum : uint32_t { kTagFeature = 1, kTagSample = 2, kTagBoot = 3, kTagBalanced = 4, kTagPermute = 5 };

// Draw keys: counter = {a, b, tree, tag<<24 | depth}, key = seed.
__device__ __forceinline__ U4 keyed(uint64_t seed, uint32_t tag, uint32_t depth,
                                    uint32_t tree, uint32_t a, uint32_t b) {
  return philox4x32_10(a, b, tree, (tag << 24) | (depth & 0xFFFFFFu), (uint32_t)seed,
                       (uint32_t)(seed >> 32));
}

__device__ __forceinline__ uint32_t pick(const U4& v, int i) {
  return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}

// ----------------------------------------------------------- float helpers
__device__ __forceinline__ uint32_t orderable(float x) {
  uint32_t u = __float_as_uint(x);
  if ((u << 1) == 0) u = 0;  // -0 and +0 are one value
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float from_orderable(uint32_t k) {
  uint32_t u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
  return __uint_as_float(u);
}
__device__ __forceinline__ bool goes_left(float x, float thr) {
  return x == -FLT_MAX || x < thr;
}
// Threshold between two sorted distinct values a < b: their midpoint, or b
// where the midpoint rounds onto a (or overflows), so that {x < thr} is
// exactly the set of values <= a.
__device__ __forceinline__ float midpoint_threshold(float a, float b) {
  float m = __fdiv_rn(__fadd_rn(a, b), 2.0f);
  return (a < m && m <= b) ? m : b;
}

// ------------------------------------------------------------ float-float
struct ff {
  float hi, lo;
};
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return ff{s, e};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  float s = __fadd_rn(a.hi, b.hi);
  float bb = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s, e);
}
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff{-b.hi, -b.lo}); }
__device__ __forceinline__ ff ff_from_i64(long long x) {
  float hi = __ll2float_rn(x);
  long long r = x - __float2ll_rz(hi);
  return ff{hi, __ll2float_rn(r)};
}
__device__ __forceinline__ ff ff_div_f(ff a, float b) {
  float q1 = __fdiv_rn(a.hi, b);
  float p = __fmul_rn(q1, b);
  float pe = __fmaf_rn(q1, b, -p);
  ff r = ff_add(a, ff{-p, -pe});
  float q2 = __fdiv_rn(r.hi, b);
  return fast_two_sum(q1, q2);
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  float p = __fmul_rn(a.hi, b.hi);
  float pe = __fmaf_rn(a.hi, b.hi, -p);
  float t1 = __fmul_rn(a.hi, b.lo);
  float t2 = __fmul_rn(a.lo, b.hi);
  pe = __fadd_rn(pe, __fadd_rn(t1, t2));
  return fast_two_sum(p, pe);
}
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
  float p = __fmul_rn(a.hi, b);
  float pe = __fmaf_rn(a.hi, b, -p);
  pe = __fadd_rn(pe, __fmul_rn(a.lo, b));
  return fast_two_sum(p, pe);
}
__device__ __forceinline__ float pow2f(int e) { return __uint_as_float((uint32_t)(e + 127) << 23); }
__device__ __forceinline__ float scale_pow2(float g, int e) {
  while (e < -126) {
    g = __fmul_rn(g, pow2f(-126));
    e += 126;
  }
  while (e > 127) {
    g = __fmul_rn(g, pow2f(127));
    e -= 127;
  }
  return __fmul_rn(g, pow2f(e));
}
__device__ __forceinline__ double pow2d(int e) {
  return __longlong_as_double((long long)(e + 1023) << 52);
}

constexpr float kLn2f = 0.693147182464599609375f;
constexpr float kSensible = 0.001f;  // gain > 1e-3 (double) <=> gain >= 0.001f

// Entropy terms in fixed point: H[n] = round(n ln n * 2^28) as int64 (built on
// the host, the same table as the oracle's), so P and Q below are exact integer
// sums in any order.  n < 2^27 keeps every sum below 2^63.
constexpr float kHScale = 1.0f / 268435456.0f;  // 2^-28, exact

// Prior numerator h(n) - sum_c h(N_c) of a node.
template <class CountFn>
__device__ __forceinline__ long long entropy_prior(const long long* H, long long n, int C,
                                                   CountFn cnt) {
  long long P = __ldg(H + n);
  for (int c = 0; c < C; ++c) P -= __ldg(H + cnt(c));
  return P;
}

// Gain in bits from the exact numerator D = P - Q of a node of n rows: the
// float conversion of D, an exact power-of-two scale, n * ln2 and one division,
// each rounded to nearest, as the oracle does.
__device__ __forceinline__ float gain_from_numerator(long long D, long long n) {
  const float num = __fmul_rn(__ll2float_rn(D), kHScale);
  const float den = __fmul_rn(__ll2float_rn(n), kLn2f);
  return __fdiv_rn(num, den);
}

// Entropy gain in bits of the split with left class counts L(c), node counts
// Ntot(c): Q = h(nL) + h(nR) - sum_c (h(L_c) + h(N_c - L_c)).
template <class LeftFn, class TotFn>
__device__ __forceinline__ float entropy_gain(const long long* H, long long P, int C,
                                              long long nL, long long nR, LeftFn L,
                                              TotFn Ntot) {
  long long Q = __ldg(H + nL) + __ldg(H + nR);
  for (int c = 0; c < C; ++c) {
    const long long l = L(c);
    Q -= __ldg(H + l) + __ldg(H + (Ntot(c) - l));
  }
  return gain_from_numerator(P - Q, nL + nR);
}

// Q of a split with the class loop unrolled to a compile-time bound CMAX >= C,
// so that per-class counts held in registers are read without index
// arithmetic.  The split's gain numerator is P - Q.
template <int CMAX, class LeftFn, class TotFn>
__device__ __forceinline__ long long entropy_q_u(const long long* H, int C, long long nL,
                                                 long long nR, LeftFn L, TotFn Ntot) {
  long long Q = __ldg(H + nL) + __ldg(H + nR);
#pragma unroll
  for (int c = 0; c < CMAX; ++c)
    if (c < C) {
      const long long l = L(c);
      Q -= __ldg(H + l) + __ldg(H + (Ntot(c) - l));
    }
  return Q;
}

template <int CMAX, class LeftFn, class TotFn>
__device__ __forceinline__ float entropy_gain_u(const long long* H, long long P, int C,
                                                long long nL, long long nR, LeftFn L,
                                                TotFn Ntot) {
  return gain_from_numerator(P - entropy_q_u<CMAX>(H, C, nL, nR, L, Ntot), nL + nR);
}

// Change of Q when one entry of class c and weight w moves from the right side
// (nR rows, Rc of class c) to the left (nL rows, Lc of class c).  Integer
// terms, so Q kept this way equals Q recomputed.
__device__ __forceinline__ long long entropy_q_move(const long long* H, long long nL,
                                                    long long nR, long long Lc, long long Rc,
                                                    long long w) {
  return (__ldg(H + nL + w) - __ldg(H + nL)) + (__ldg(H + nR - w) - __ldg(H + nR)) -
         (__ldg(H + Lc + w) - __ldg(H + Lc)) - (__ldg(H + Rc - w) - __ldg(H + Rc));
}

// For numerators d > dtop of one node: false when gain_from_numerator(d) is
// certainly above gain_from_numerator(dtop).  The int64 -> float conversion
// and the two rounded operations that follow move a value by at most 2^-24
// relative each, so numerators more than 2^-21 apart (relative to the larger
// magnitude) give different gains; only closer ones need their gains compared.
__device__ __forceinline__ bool gain_may_tie(long long d, long long dtop) {
  const unsigned long long ad = d < 0 ? 0ull - (unsigned long long)d : (unsigned long long)d;
  const unsigned long long at =
      dtop < 0 ? 0ull - (unsigned long long)dtop : (unsigned long long)dtop;
  const unsigned long long mx = ad > at ? ad : at;
  return (unsigned long long)(d - dtop) <= (mx >> 21);
}

// Best boundary of one thread that offers its positions in increasing order:
// the first position of the highest gain, found on exact gain numerators of
// one node (n rows).  The gain is monotone in the numerator, so a numerator
// that does not exceed the highest one seen cannot win; a float gain is
// computed only when two numerators are close enough to round to the same one.
// The best gain is always the gain of `top`.
struct NumBest {
  long long top;
  int p;  // -1 before the first offer
  __device__ __forceinline__ void init() {
    p = -1;
    top = 0;
  }
  // True when `pos` becomes the best position.
  __device__ __forceinline__ bool offer(long long d, int pos, long long n) {
    if (p < 0) {
      p = pos;
      top = d;
      return true;
    }
    if (d <= top) return false;
    const bool take =
        !gain_may_tie(d, top) || gain_from_numerator(d, n) > gain_from_numerator(top, n);
    top = d;
    if (take) p = pos;
    return take;
  }
  __device__ __forceinline__ float gain(long long n) const {
    return p < 0 ? -FLT_MAX : gain_from_numerator(top, n);
  }
};

__device__ __forceinline__ float variance_gain(long long nL, long long SL, long long nR,
                                               long long SR, int S) {
  ff mL = ff_div_f(ff_from_i64(SL), __ll2float_rn(nL));
  ff mR = ff_div_f(ff_from_i64(SR), __ll2float_rn(nR));
  ff d = ff_sub(mL, mR);
  ff d2 = ff_mul(d, d);
  float w = __fdiv_rn(__fmul_rn(__ll2float_rn(nL), __ll2float_rn(nR)), __ll2float_rn(nL + nR));
  float g = ff_mul_f(d2, w).hi;
  return scale_pow2(g, -2 * S);
}

// Bounds lo <= variance_gain(nL, SL, nR, SR, S) <= hi from a few float
// operations, so that a scan evaluates the float-float gain only where it can
// reach the best.  With a = float(nL), b = float(nR) (the values variance_gain
// divides by), the mean difference is (SL b - SR a) / (a b); its float
// numerator is within 3.001 * 2^-24 * A of the exact one, A = |SL| b + |SR| a,
// and variance_gain's own difference within 2^-43 A / (a b).  The margin
// e = 2^-20 A covers both and __fdividef's 2 ulp; the last factor 1 +- 2^-16
// covers the remaining roundings (a dozen at 2^-24 each).  rc = 1 / float(n)
// rounded, p2 = 2^(-2S) (-2S in [-124, 120]: one exact scaling, monotone as in
// variance_gain).  No overflow: a side's mean is at most 2^(61 - ceil(log2 N))
// in magnitude, so hi stays below 2^128.  Requires nL, nR >= 1.
__device__ __forceinline__ void variance_gain_bounds(int nL, long long SL, int nR, long long SR,
                                                     float rc, float p2, float& lo, float& hi) {
  const float a = __int2float_rn(nL), b = __int2float_rn(nR);
  const float t1 = __fmul_rn(__ll2float_rn(SL), b);
  const float t2 = __fmul_rn(__ll2float_rn(SR), a);
  const float d = fabsf(__fsub_rn(t1, t2));
  const float e = __fmul_rn(__fadd_rn(fabsf(t1), fabsf(t2)), 0x1p-20f);
  const float ab = __fmul_rn(a, b);
  const float w = __fmul_rn(ab, rc);
  const float du = __fdividef(__fadd_rn(d, e), ab);
  const float dl = __fdividef(fmaxf(__fsub_rn(d, e), 0.0f), ab);
  hi = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(du, du), w), 0x1.0001p0f), p2);
  lo = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(dl, dl), w), 0x1.fffep-1f), p2);
}

// A regression entry's fixed-point target q and weight w in one word,
// q * 2^wb + w with wb the bit length of N.  Lossless: a tree draws N rows, so
// 0 <= w <= N < 2^wb, and the target scale keeps |q| <= 2^(61 - ceil(log2 N))
// <= 2^(62 - wb), so |q * 2^wb| <= 2^62.
__device__ __forceinline__ int qw_bits(long long N) { return 64 - __clzll(N); }
__device__ __forceinline__ long long qw_pack(long long q, int w, int wb) {
  return q * (1ll << wb) + w;
}
__device__ __forceinline__ int qw_weight(long long x, int wb) {
  return (int)(x & ((1ll << wb) - 1));
}
__device__ __forceinline__ long long qw_target(long long x, int wb) { return x >> wb; }

// Walks trees t0 .. t0+W-1 for one row in lockstep, so that W independent
// node loads are in flight at a time; x(f) reads the row's value of feature f.
// leaf[k] receives tree t0+k's leaf (predict layout, PNode).
template <int W, class XFn>
__device__ __forceinline__ void walk_trees(const PNode* __restrict__ nodes, int t0, XFn x,
                                           int4 (&leaf)[W]) {
#pragma unroll
  for (int k = 0; k < W; ++k) leaf[k] = __ldg(reinterpret_cast<const int4*>(nodes) + t0 + k);
  bool more = true;
  while (more) {
    more = false;
#pragma unroll
    for (int k = 0; k < W; ++k)
      if (leaf[k].x >= 0) {
        const int nx = goes_left(x(leaf[k].y), __int_as_float(leaf[k].z)) ? leaf[k].x
                                                                           : leaf[k].x + 1;
        leaf[k] = __ldg(reinterpret_cast<const int4*>(nodes) + nx);
        more |= leaf[k].x >= 0;
      }
  }
}

// Candidate order: valid first, then higher gain, lower feature, lower threshold.
__device__ __forceinline__ bool cand_better(bool va, float ga, int fa, float ta, bool vb,
                                            float gb, int fb, float tb) {
  if (va != vb) return va;
  if (ga != gb) return ga > gb;
  if (fa != fb) return fa < fb;
  return ta < tb;
}

}  // namespace dml
