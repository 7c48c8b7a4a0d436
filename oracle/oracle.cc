// ORACLE — test infrastructure only.
//
// A CPU restatement of the reference's random-forest / extremely-randomized-
// trees fit and predict path (novelari/DataminingLibs, lib_ensembles).  It is
// the correctness checker for the CUDA engine in datamininglibs_gb300/ and the
// timed CPU baseline in bench.py.  Nothing in the product links, loads or calls
// this file; only tests/, __graft_entry__.smoke() and bench.py's CPU legs do.
//
// It restates (file:line in the reference project):
//   - ERT node search: lib_ensembles/source/gpuert.cu:119-247 (try loop,
//     10-sample-mean threshold), :275-326 (2xC histogram, entropy gain,
//     -FLT_MAX for an empty side), :328-381 (variance gain)
//   - RF node search: lib_ensembles/source/gpurf.cu:131-259 (try loop),
//     :440-616 (sort by feature value), :618-768 (best boundary, midpoint
//     threshold), :770-917 (variance boundary scan, restated on targets)
//   - entropy in bits: lib_ensembles/source/gpudte.cu:70-117
//   - leaf rule and node payload: lib_ensembles/source/gpudte.cu:156-309
//   - predict traversal, missing-value rule and vote: gpudte.cu:311-359
//   - default K = round(ln F) + 1: lib_ensembles/source/gpudte_algorithm.cc:579-580
//   - Classify node layout {child_start, child_count, probability_start,
//     attribute, split_point}: lib_ensembles/source/gpudte_algorithm_shared.h:82-90
//   - level-by-level node-array assembly: gpudte_algorithm.cc:46-92
//
// Where the reference is nondeterministic or defective the oracle implements
// the corrected, deterministic behaviour that the CUDA engine also implements:
//   * all randomness from Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)
//     keyed by (seed, tree, depth, node-in-level, try, draw) instead of
//     1024 shared cuRAND MRG32k3a states (gpurf.cu:104-112, gpuert.cu:128-130)
//   * stable partitions and a level-major, tree-major, parent-ordered node
//     array instead of atomic order (gpudte.cu:215-232, 259-266)
//   * RF gain of the split {x < thr} vs {x >= thr} at every boundary between
//     distinct values (fixes the race and off-by-one at gpurf.cu:624-694,
//     679-682, 727-744); variance on targets, not feature values
//     (gpurf.cu:786-794)
//   * regression leaf value = node mean (gpudte.cu:294-301)
//   * gain ties broken by the lowest (feature, threshold)
//   * entropy evaluated from an n*ln(n) table in int64 fixed point
//     (round(n ln n * 2^28)), so that the gain numerators are exact integer
//     sums and the CPU and GPU produce identical FP32 gains; an independent
//     FP64 gain is kept beside it for the tolerance check
//
// Build: oracle/Makefile (g++ -O2 -fopenmp -ffp-contract=off).

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- Philox4x32-10
struct W4 {
  uint32_t v[4];
};

inline void mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

W4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                 uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += W0;
      k1 += W1;
    }
    uint32_t h0, l0, h1, l1;
    mulhilo(M0, c0, &h0, &l0);
    mulhilo(M1, c2, &h1, &l1);
    uint32_t n0 = h1 ^ c1 ^ k0;
    uint32_t n2 = h0 ^ c3 ^ k1;
    c0 = n0;
    c1 = l1;
    c2 = n2;
    c3 = l0;
  }
  W4 o;
  o.v[0] = c0;
  o.v[1] = c1;
  o.v[2] = c2;
  o.v[3] = c3;
  return o;
}

enum : uint32_t { kTagFeature = 1, kTagSample = 2, kTagBoot = 3, kTagBalanced = 4, kTagPermute = 5 };

inline W4 keyed(uint64_t seed, uint32_t tag, uint32_t depth, uint32_t tree,
                uint32_t a, uint32_t b) {
  return philox4x32_10(a, b, tree, (tag << 24) | (depth & 0xFFFFFFu),
                       (uint32_t)seed, (uint32_t)(seed >> 32));
}

// --------------------------------------------------------- n*ln(n) table recipe
// ln(x) for x >= 1 from x = m * 2^e, m in [sqrt(1/2), sqrt(2)), and
// ln(m) = 2*atanh(z), z = (m-1)/(m+1), summed as the odd power series.  Only
// IEEE double +,-,*,/ and frexp are used, in a fixed order, so the table is
// bit-identical on every host.
const double kLn2d = 0.6931471805599453094;
double table_ln(double x) {
  int e = 0;
  double m = std::frexp(x, &e);
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e = e - 1;
  }
  double z = (m - 1.0) / (m + 1.0);
  double z2 = z * z;
  double term = z;
  double sum = 0.0;
  for (int k = 0; k < 13; ++k) {
    sum = sum + term / (double)(2 * k + 1);
    term = term * z2;
  }
  return 2.0 * sum + (double)e * kLn2d;
}

struct FF {
  float hi, lo;
};

// Entropy terms n ln n in fixed point: H[n] = round(n ln n * 2^28) (ldexp is
// exact, llrint rounds to nearest even), so the sums of a gain (the prior
// P = H[n] - sum_c H[N_c] and Q = H[nL] + H[nR] - sum_c (H[L_c] + H[R_c]),
// gpudte.cu:76-117 restated) are exact integers; n < 2^27 keeps them below 2^63.
std::vector<int64_t> build_nlogn_table(int64_t nmax) {
  std::vector<int64_t> t((size_t)nmax + 1);
  for (int64_t n = 0; n <= nmax; ++n)
    t[n] = n < 2 ? 0 : std::llrint(std::ldexp((double)n * table_ln((double)n), 28));
  return t;
}
const float kHScale = 1.0f / 268435456.0f;  // 2^-28, exact


// ------------------------------------------------------ float-float arithmetic
inline FF fast_two_sum(float a, float b) {
  float s = a + b;
  float e = b - (s - a);
  return FF{s, e};
}
inline FF ff_add(FF a, FF b) {
  float s = a.hi + b.hi;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e = e + (a.lo + b.lo);
  return fast_two_sum(s, e);
}
inline FF ff_neg(FF a) { return FF{-a.hi, -a.lo}; }
inline FF ff_sub(FF a, FF b) { return ff_add(a, ff_neg(b)); }
inline FF ff_from_i64(int64_t x) {
  float hi = (float)x;
  int64_t r = x - (int64_t)hi;
  float lo = (float)r;
  return FF{hi, lo};
}
inline FF ff_div_f(FF a, float b) {
  float q1 = a.hi / b;
  float p = q1 * b;
  float pe = std::fmaf(q1, b, -p);
  FF r = ff_add(a, FF{-p, -pe});
  float q2 = r.hi / b;
  return fast_two_sum(q1, q2);
}
inline FF ff_mul(FF a, FF b) {
  float p = a.hi * b.hi;
  float pe = std::fmaf(a.hi, b.hi, -p);
  float t1 = a.hi * b.lo;
  float t2 = a.lo * b.hi;
  pe = pe + (t1 + t2);
  return fast_two_sum(p, pe);
}
inline FF ff_mul_f(FF a, float b) {
  float p = a.hi * b;
  float pe = std::fmaf(a.hi, b, -p);
  pe = pe + a.lo * b;
  return fast_two_sum(p, pe);
}
inline float pow2f(int e) {  // exact 2^e for e in [-126, 127]
  uint32_t bits = (uint32_t)(e + 127) << 23;
  float f;
  std::memcpy(&f, &bits, 4);
  return f;
}
inline float scale_pow2(float g, int e) {
  while (e < -126) {
    g = g * pow2f(-126);
    e += 126;
  }
  while (e > 127) {
    g = g * pow2f(127);
    e -= 127;
  }
  return g * pow2f(e);
}
inline double pow2d(int e) {  // exact 2^e for e in [-1022, 1023]
  uint64_t bits = (uint64_t)(e + 1023) << 52;
  double d;
  std::memcpy(&d, &bits, 8);
  return d;
}

const float kLn2f = 0.693147182464599609375f;
// Gain in bits from the exact numerator D = P - Q of a node of n rows: three
// float roundings (the conversion of D, n * ln2, the division); the power-of-two
// scale is exact.
inline float gain_from_numerator(int64_t D, int64_t n) {
  const float num = (float)D * kHScale;
  const float den = (float)n * kLn2f;
  return num / den;
}

const float kSensible = 0.001f;  // g > 1e-3 (double) <=> g >= 0.001f (float)

// -------------------------------------------------------------- the problem
struct Problem {
  int algo;  // 0 RF (bootstrap), 1 ERT (no bootstrap)
  int task;  // 0 classification, 1 regression
  int n_trees, K, max_depth, min_node_size, min_leaf, n_classes;
  uint64_t seed;
  int64_t N;
  int F;
  int tree_offset;  // RNG key of tree 0
  int balanced;     // RF classification: per-class bootstrap (easy ensemble)
  const float* X;  // feature-major [F*N]
  const float* y;  // [N]
};

// Rows of each class in ascending order (the balanced bootstrap draws from them).
std::vector<std::vector<int32_t>> class_rows(const float* y, int64_t N, int C) {
  std::vector<std::vector<int32_t>> r((size_t)C);
  for (int64_t i = 0; i < N; ++i) r[(size_t)y[i]].push_back((int32_t)i);
  return r;
}

// Bootstrap multiplicities of one tree.  Plain (gpurf.cu:101-113 with keyed
// draws): draw i in [0, N) picks row (word i&3 of Philox(seed; i>>2, i>>34,
// tree, kTagBoot)) % N.  Balanced, the reference's easy ensemble
// (gpurf.cu:73-100): for every class c with rows, N / C draws
// i = c * (N / C) + j pick rows of c uniformly (kTagBalanced); empty classes
// draw nothing.
std::vector<int32_t> bag_counts(const Problem& p, int tree,
                                const std::vector<std::vector<int32_t>>* rows) {
  const int64_t N = p.N;
  std::vector<int32_t> w((size_t)N, 0);
  const uint32_t key = (uint32_t)(tree + p.tree_offset);
  if (!p.balanced) {
    for (int64_t i = 0; i < N; ++i) {
      W4 r = keyed(p.seed, kTagBoot, 0, key, (uint32_t)(i >> 2), (uint32_t)(i >> 34));
      w[r.v[i & 3] % (uint32_t)N] += 1;
    }
    return w;
  }
  const int64_t m = N / p.n_classes;
  for (int64_t i = 0; i < (int64_t)p.n_classes * m; ++i) {
    const std::vector<int32_t>& rc = (*rows)[(size_t)(i / m)];
    if (rc.empty()) continue;
    W4 r = keyed(p.seed, kTagBalanced, 0, key, (uint32_t)(i >> 2), (uint32_t)(i >> 34));
    w[rc[r.v[i & 3] % (uint32_t)rc.size()]] += 1;
  }
  return w;
}

struct NodeOut {
  int is_leaf;
  int attr;
  float thr;
  float gain32;
  double gain64;
  std::vector<int64_t> counts;  // classification leaf payload (weighted)
  float value;                  // regression leaf value
};

struct TreeOut {
  std::vector<std::vector<NodeOut>> levels;
};

struct Forest {
  int task, C, F, n_trees;
  std::vector<int32_t> node_array;  // 5 ints per node (split_point stored as bits)
  std::vector<float> probs;
  std::vector<float> gains32;       // per node in node-array order (NaN for leaves)
  std::vector<double> gains64;
  std::vector<int32_t> depth;       // per node
};

inline uint32_t orderable(float x) {
  if (x == 0.0f) x = 0.0f;  // -0 and +0 are one value
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

inline bool goes_left(float x, float thr) { return x == -FLT_MAX || x < thr; }

struct Cand {
  bool valid;
  float gain;
  int f;
  float thr;
  double gain64;
};

// total order: valid first, higher gain, lower feature, lower threshold
inline bool better(const Cand& a, const Cand& b) {
  if (a.valid != b.valid) return a.valid;
  if (a.gain != b.gain) return a.gain > b.gain;
  if (a.f != b.f) return a.f < b.f;
  return a.thr < b.thr;
}

struct Ctx {
  const Problem* p;
  const std::vector<int64_t>* H;
  std::vector<int32_t> lab;  // classification labels
  std::vector<int64_t> q;    // regression targets, fixed point 2^-S
  int S;
  std::vector<std::vector<int32_t>> class_rows;  // balanced bootstrap
};

double h64(double x) { return x <= 1.0 ? 0.0 : x * std::log(x); }

float entropy_gain(const Ctx& cx, int64_t P, const int64_t* L, const int64_t* R,
                   int C, int64_t nL, int64_t nR, double* g64,
                   const int64_t* Ntot) {
  const std::vector<int64_t>& H = *cx.H;
  int64_t Q = H[nL] + H[nR];
  for (int c = 0; c < C; ++c) Q -= H[L[c]] + H[R[c]];
  int64_t n = nL + nR;
  float g = gain_from_numerator(P - Q, n);
  if (g64) {
    double num = h64((double)n) - h64((double)nL) - h64((double)nR);
    for (int c = 0; c < C; ++c)
      num += -h64((double)Ntot[c]) + h64((double)L[c]) + h64((double)R[c]);
    *g64 = num / ((double)n * std::log(2.0));
  }
  return g;
}

float variance_gain(int64_t nL, int64_t SL, int64_t nR, int64_t SR, int S,
                    double* g64) {
  FF mL = ff_div_f(ff_from_i64(SL), (float)nL);
  FF mR = ff_div_f(ff_from_i64(SR), (float)nR);
  FF d = ff_sub(mL, mR);
  FF d2 = ff_mul(d, d);
  float w = ((float)nL * (float)nR) / (float)(nL + nR);
  float g = ff_mul_f(d2, w).hi;
  g = scale_pow2(g, -2 * S);
  if (g64) {
    long double sl = (long double)SL, sr = (long double)SR;
    long double ml = sl / (long double)nL, mr = sr / (long double)nR;
    long double dd = ml - mr;
    long double v = (long double)nL * (long double)nR * dd * dd /
                    (long double)(nL + nR);
    *g64 = (double)(v * (long double)pow2d(-2 * S));
  }
  return g;
}

struct Entry {
  int32_t row;
  int32_t w;
};

struct OpenNode {
  int64_t ebeg, ecnt;  // entries [ebeg, ebeg+ecnt) of the tree's entry list
  int64_t n;           // weighted count
  std::vector<int64_t> counts;
  int64_t sum;  // regression: sum of q*w
};

// Evaluate one try.  Returns the candidate.
Cand eval_try(const Ctx& cx, const std::vector<Entry>& E, const OpenNode& nd,
              int tree, int depth, int idx, int tr, int f, int64_t P,
              std::vector<std::pair<uint32_t, int32_t>>& sortbuf) {
  const Problem& p = *cx.p;
  const int C = p.n_classes;
  const float* xf = p.X + (int64_t)f * p.N;
  Cand cand{false, -FLT_MAX, f, 0.0f, -DBL_MAX};
  const int64_t m = nd.ecnt;
  if (p.algo == 1) {
    // ERT: threshold = mean of 10 node values drawn with replacement
    float acc = 0.0f;
    for (int s = 0; s < 10; ++s) {
      W4 w = keyed(p.seed, kTagSample, (uint32_t)depth, (uint32_t)(tree + p.tree_offset),
                   (uint32_t)idx, (uint32_t)(tr * 3 + s / 4));
      int64_t pos = (int64_t)(w.v[s % 4] % (uint32_t)m);
      acc = acc + xf[E[nd.ebeg + pos].row];
    }
    float thr = acc / 10.0f;
    cand.thr = thr;
    if (p.task == 0) {
      std::vector<int64_t> L(C, 0), R(C, 0);
      int64_t nL = 0, nR = 0;
      for (int64_t i = 0; i < m; ++i) {
        const Entry& e = E[nd.ebeg + i];
        int k = cx.lab[e.row];
        if (goes_left(xf[e.row], thr)) {
          L[k] += e.w;
          nL += e.w;
        } else {
          R[k] += e.w;
          nR += e.w;
        }
      }
      if (nL >= p.min_leaf && nR >= p.min_leaf && nL > 0 && nR > 0) {
        cand.valid = true;
        cand.gain = entropy_gain(cx, P, L.data(), R.data(), C, nL, nR,
                                 &cand.gain64, nd.counts.data());
      }
    } else {
      int64_t nL = 0, nR = 0, SL = 0, SR = 0;
      for (int64_t i = 0; i < m; ++i) {
        const Entry& e = E[nd.ebeg + i];
        if (goes_left(xf[e.row], thr)) {
          nL += e.w;
          SL += cx.q[e.row] * e.w;
        } else {
          nR += e.w;
          SR += cx.q[e.row] * e.w;
        }
      }
      if (nL >= p.min_leaf && nR >= p.min_leaf && nL > 0 && nR > 0) {
        cand.valid = true;
        cand.gain = variance_gain(nL, SL, nR, SR, cx.S, &cand.gain64);
      }
    }
    return cand;
  }
  // RF: exact best boundary between distinct values
  sortbuf.resize((size_t)m);
  for (int64_t i = 0; i < m; ++i)
    sortbuf[i] = std::make_pair(orderable(xf[E[nd.ebeg + i].row]), (int32_t)i);
  std::sort(sortbuf.begin(), sortbuf.end());
  std::vector<int64_t> L(C, 0), R(C, 0);
  int64_t nL = 0, SL = 0;
  bool have = false;
  float bestg = 0.0f;
  int64_t bestp = -1;
  double bestg64 = 0.0;
  for (int64_t pos = 1; pos < m; ++pos) {
    const Entry& ep = E[nd.ebeg + sortbuf[pos - 1].second];
    if (p.task == 0)
      L[cx.lab[ep.row]] += ep.w;
    else
      SL += cx.q[ep.row] * ep.w;
    nL += ep.w;
    float xa = xf[ep.row];
    float xb = xf[E[nd.ebeg + sortbuf[pos].second].row];
    if (!(xa < xb)) continue;
    int64_t nR = nd.n - nL;
    if (nL < p.min_leaf || nR < p.min_leaf) continue;
    float g;
    double g64;
    if (p.task == 0) {
      for (int c = 0; c < C; ++c) R[c] = nd.counts[c] - L[c];
      g = entropy_gain(cx, P, L.data(), R.data(), C, nL, nR, &g64,
                       nd.counts.data());
    } else {
      g = variance_gain(nL, SL, nR, nd.sum - SL, cx.S, &g64);
    }
    if (!have || g > bestg) {
      have = true;
      bestg = g;
      bestp = pos;
      bestg64 = g64;
    }
  }
  if (have) {
    float xa = xf[E[nd.ebeg + sortbuf[bestp - 1].second].row];
    float xb = xf[E[nd.ebeg + sortbuf[bestp].second].row];
    float mid = (xa + xb) / 2.0f;
    float thr = (xa < mid && mid <= xb) ? mid : xb;
    cand.valid = true;
    cand.gain = bestg;
    cand.thr = thr;
    cand.gain64 = bestg64;
  }
  return cand;
}

// Stable partition of a node's entries (gpudte.cu:205-232, made stable):
// left = {x == -FLT_MAX or x < thr} in entry order, then right in entry order.
// Fills the children's entry ranges (relative to the node) and their weighted
// class counts / target sums (gpudte.cu:168-201).
void split_entries(const Entry* in, int64_t m, const float* xf, float thr,
                   int task, int C, const int32_t* lab, const int64_t* q,
                   Entry* out, OpenNode* l, OpenNode* r) {
  l->counts.assign(C, 0);
  r->counts.assign(C, 0);
  l->n = r->n = 0;
  l->sum = r->sum = 0;
  int64_t nl = 0;
  for (int64_t i = 0; i < m; ++i)
    if (goes_left(xf[in[i].row], thr)) ++nl;
  int64_t wl = 0, wr = nl;
  for (int64_t i = 0; i < m; ++i) {
    const Entry& e = in[i];
    bool left = goes_left(xf[e.row], thr);
    OpenNode* ch = left ? l : r;
    out[left ? wl++ : wr++] = e;
    ch->n += e.w;
    if (task == 0)
      ch->counts[lab[e.row]] += e.w;
    else
      ch->sum += q[e.row] * e.w;
  }
  l->ebeg = 0;
  l->ecnt = nl;
  r->ebeg = nl;
  r->ecnt = m - nl;
}

// Leaf rule (gpudte.cu:253-257): a node is a leaf when it holds at most
// min_node_size rows, is at max_depth, or no try gave two non-empty sides.
bool is_leaf_rule(int64_t n, int depth, int min_node_size, int max_depth,
                  bool valid_split) {
  return n <= min_node_size || depth >= max_depth || !valid_split;
}

// One node of a level: search, leaf rule, partition.  Writes its output and,
// for a split, its two children into ch[0..1] (has_children set).
void fit_node(const Ctx& cx, int tree, int depth, size_t idx, OpenNode& nd,
              std::vector<Entry>& E, std::vector<Entry>& E2, NodeOut& no,
              OpenNode* ch, bool* has_children,
              std::vector<std::pair<uint32_t, int32_t>>& sortbuf) {
  const Problem& p = *cx.p;
  const int C = p.n_classes;
  const int64_t N = p.N;
  *has_children = false;
  no.is_leaf = 1;
  no.attr = -1;
  no.thr = -1.0f;
  no.gain32 = NAN;
  no.gain64 = NAN;
  Cand best{false, -FLT_MAX, -1, 0.0f, 0.0};
  if (nd.n > p.min_node_size && depth < p.max_depth) {
    int64_t P = 0;
    if (p.task == 0) {
      P = (*cx.H)[nd.n];
      for (int c = 0; c < C; ++c) P -= (*cx.H)[nd.counts[c]];
    }
    // try loop: gpuert.cu:144-149 / gpurf.cu:177-182
    int K = p.K, F = p.F;
    int n_mand = K < F ? K : F;
    int n_opt = K < F ? std::min(F - K, 10) : 0;
    int tr = 0;
    for (; tr < n_mand; ++tr) {
      W4 w = keyed(p.seed, kTagFeature, (uint32_t)depth, (uint32_t)(tree + p.tree_offset),
                   (uint32_t)idx, (uint32_t)tr);
      int f = (int)(w.v[0] % (uint32_t)F);
      Cand c = eval_try(cx, E, nd, tree, depth, (int)idx, tr, f, P, sortbuf);
      if (tr == 0 || better(c, best)) best = c;
    }
    if (!(best.valid && best.gain >= kSensible)) {
      for (int j = 0; j < n_opt; ++j, ++tr) {
        W4 w = keyed(p.seed, kTagFeature, (uint32_t)depth, (uint32_t)(tree + p.tree_offset),
                     (uint32_t)idx, (uint32_t)tr);
        int f = (int)(w.v[0] % (uint32_t)F);
        Cand c = eval_try(cx, E, nd, tree, depth, (int)idx, tr, f, P, sortbuf);
        if (better(c, best)) best = c;
        if (c.valid && c.gain >= kSensible) break;
      }
    }
  }
  if (is_leaf_rule(nd.n, depth, p.min_node_size, p.max_depth, best.valid)) {
    // leaf: payload = node class counts / node mean
    if (p.task == 0)
      no.counts = nd.counts;
    else
      no.value = (float)(((double)nd.sum * pow2d(-cx.S)) / (double)nd.n);
    return;
  }
  // internal node: stable partition into children (left, right)
  no.is_leaf = 0;
  no.attr = best.f;
  no.thr = best.thr;
  no.gain32 = best.gain;
  no.gain64 = best.gain64;
  split_entries(E.data() + nd.ebeg, nd.ecnt, p.X + (int64_t)best.f * N, best.thr,
                p.task, C, cx.lab.data(), cx.q.data(), E2.data() + nd.ebeg, &ch[0],
                &ch[1]);
  ch[0].ebeg += nd.ebeg;
  ch[1].ebeg += nd.ebeg;
  *has_children = true;
}

// Level-wise build of one tree.  With par_nodes the nodes of a level are
// spread over OpenMP threads (each node owns its entry range and its output
// slots, so the result does not depend on the thread count).
void fit_tree(const Ctx& cx, int tree, TreeOut& out, bool par_nodes, int threads) {
  const Problem& p = *cx.p;
  const int C = p.n_classes;
  const int64_t N = p.N;
  std::vector<Entry> E, E2;
  // root entries: bootstrap multiplicities (RF) or every row once (ERT)
  if (p.algo == 0) {
    std::vector<int32_t> w = bag_counts(p, tree, &cx.class_rows);
    for (int64_t i = 0; i < N; ++i)
      if (w[i] > 0) E.push_back(Entry{(int32_t)i, w[i]});
  } else {
    E.resize((size_t)N);
    for (int64_t i = 0; i < N; ++i) E[i] = Entry{(int32_t)i, 1};
  }
  E2.resize(E.size());
  std::vector<OpenNode> cur(1), nxt;
  cur[0].ebeg = 0;
  cur[0].ecnt = (int64_t)E.size();
  cur[0].n = 0;
  cur[0].counts.assign(C, 0);
  cur[0].sum = 0;
  for (const Entry& e : E) {
    cur[0].n += e.w;
    if (p.task == 0)
      cur[0].counts[cx.lab[e.row]] += e.w;
    else
      cur[0].sum += cx.q[e.row] * e.w;
  }
  for (int depth = 0; !cur.empty(); ++depth) {
    out.levels.emplace_back();
    std::vector<NodeOut>& lv = out.levels.back();
    const size_t n = cur.size();
    lv.resize(n);
    std::vector<OpenNode> kids(2 * n);
    std::vector<char> has(n, 0);
#ifdef _OPENMP
#pragma omp parallel num_threads(par_nodes ? threads : 1)
#endif
    {
      std::vector<std::pair<uint32_t, int32_t>> sortbuf;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
      for (long long idx = 0; idx < (long long)n; ++idx) {
        bool h = false;
        fit_node(cx, tree, depth, (size_t)idx, cur[idx], E, E2, lv[idx], &kids[2 * idx],
                 &h, sortbuf);
        has[idx] = h;
      }
    }
    nxt.clear();
    for (size_t idx = 0; idx < n; ++idx)
      if (has[idx]) {
        nxt.push_back(std::move(kids[2 * idx]));
        nxt.push_back(std::move(kids[2 * idx + 1]));
      }
    // entries of split nodes were rewritten into E2; copy them back in place
    for (const OpenNode& ch : nxt)
      std::copy(E2.begin() + ch.ebeg, E2.begin() + ch.ebeg + ch.ecnt,
                E.begin() + ch.ebeg);
    cur.swap(nxt);
  }
}

int quant_scale(const float* y, int64_t N) {
  float mx = 0.0f;
  for (int64_t i = 0; i < N; ++i) mx = std::max(mx, std::fabs(y[i]));
  if (mx == 0.0f) return 0;
  int ey = std::ilogb(mx) + 1;
  int en = 0;
  while (((int64_t)1 << en) < N) ++en;
  int S = 61 - ey - en;
  if (S > 62) S = 62;
  if (S < -60) S = -60;
  return S;
}

}  // namespace

extern "C" {

typedef struct {
  int32_t algo, task, n_trees, K, max_depth, min_node_size, min_leaf,
      n_classes;
  uint64_t seed;
  int64_t n_rows;
  int32_t n_features, threads;
  const float* samples;
  const float* targets;
  int32_t tree_offset, balanced;
} oracle_desc;

// Philox4x32-10 known-answer access for tests.
void oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  W4 w = philox4x32_10(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = w.v[i];
}

void oracle_nlogn_table(int64_t nmax, int64_t* out) {
  std::vector<int64_t> t = build_nlogn_table(nmax);
  std::memcpy(out, t.data(), sizeof(int64_t) * (size_t)(nmax + 1));
}

// Entropy gain (bits) of a 2 x C count table, FP32 (table-based) and FP64.
float oracle_entropy_gain(const int64_t* L, const int64_t* R, int C,
                          double* g64) {
  int64_t nL = 0, nR = 0;
  std::vector<int64_t> Nt(C);
  for (int c = 0; c < C; ++c) {
    nL += L[c];
    nR += R[c];
    Nt[c] = L[c] + R[c];
  }
  std::vector<int64_t> H = build_nlogn_table(nL + nR);
  Ctx cx;
  cx.H = &H;
  cx.p = nullptr;
  cx.S = 0;
  int64_t P = H[nL + nR];
  for (int c = 0; c < C; ++c) P -= H[Nt[c]];
  return entropy_gain(cx, P, L, R, C, nL, nR, g64, Nt.data());
}

float oracle_variance_gain(int64_t nL, int64_t SL, int64_t nR, int64_t SR,
                           int S, double* g64) {
  return variance_gain(nL, SL, nR, SR, S, g64);
}

int oracle_quant_scale(const float* y, int64_t N) { return quant_scale(y, N); }

// The oracle's node split step on one classification node with unit weights:
// leaf rule, then the stable partition.  Returns 1 for a leaf.
int oracle_split_node(const int32_t* rows, int64_t m, const float* xf, float thr,
                      const float* y, int C, int depth, int max_depth,
                      int min_node_size, int32_t* rows_out, int64_t* child_n,
                      int64_t* counts_out) {
  std::vector<Entry> in((size_t)m), out((size_t)m);
  std::vector<int32_t> lab;
  int32_t mx = 0;
  for (int64_t i = 0; i < m; ++i) mx = std::max(mx, rows[i]);
  lab.assign((size_t)mx + 1, 0);
  for (int64_t i = 0; i < m; ++i) {
    in[i] = Entry{rows[i], 1};
    lab[rows[i]] = (int32_t)y[rows[i]];
  }
  OpenNode l, r;
  split_entries(in.data(), m, xf, thr, 0, C, lab.data(), nullptr, out.data(),
                &l, &r);
  bool valid = l.n > 0 && r.n > 0;
  for (int c = 0; c < C; ++c) counts_out[c] = l.counts[c] + r.counts[c];
  if (is_leaf_rule(m, depth, min_node_size, max_depth, valid)) {
    child_n[0] = child_n[1] = 0;
    return 1;
  }
  for (int64_t i = 0; i < m; ++i) rows_out[i] = out[i].row;
  child_n[0] = l.n;
  child_n[1] = r.n;
  return 0;
}

void* oracle_fit(const oracle_desc* d) {
  Problem p;
  p.algo = d->algo;
  p.task = d->task;
  p.n_trees = d->n_trees;
  p.F = d->n_features;
  p.K = d->K > 0 ? d->K : (int)std::round(std::log((double)d->n_features)) + 1;
  p.max_depth = d->max_depth;
  p.min_node_size = d->min_node_size;
  p.min_leaf = d->min_leaf < 1 ? 1 : d->min_leaf;
  p.n_classes = d->task == 0 ? d->n_classes : 1;
  p.seed = d->seed;
  p.N = d->n_rows;
  p.X = d->samples;
  p.y = d->targets;
  p.tree_offset = d->tree_offset;
  p.balanced = d->balanced;
  Ctx cx;
  cx.p = &p;
  if (p.balanced) cx.class_rows = class_rows(p.y, p.N, p.n_classes);
  std::vector<int64_t> H;
  if (p.task == 0) {
    H = build_nlogn_table(p.N);
    cx.lab.resize((size_t)p.N);
    for (int64_t i = 0; i < p.N; ++i) cx.lab[i] = (int32_t)p.y[i];
    cx.S = 0;
  } else {
    cx.S = quant_scale(p.y, p.N);
    cx.q.resize((size_t)p.N);
    double sc = pow2d(cx.S);
    for (int64_t i = 0; i < p.N; ++i)
      cx.q[i] = (int64_t)std::llrint((double)p.y[i] * sc);
  }
  cx.H = &H;
  std::vector<TreeOut> trees((size_t)p.n_trees);
  int th = 1;
#ifdef _OPENMP
  th = d->threads > 0 ? d->threads : omp_get_max_threads();
#endif
  if (p.n_trees >= th) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(th)
#endif
    for (int t = 0; t < p.n_trees; ++t) fit_tree(cx, t, trees[t], false, 1);
  } else {
    for (int t = 0; t < p.n_trees; ++t) fit_tree(cx, t, trees[t], true, th);
  }

  // level-major, tree-major assembly (gpudte_algorithm.cc:46-92 with a
  // deterministic order): roots 0..T-1, then level 1 of every tree, ...
  Forest* fo = new Forest();
  fo->task = p.task;
  fo->C = p.task == 0 ? p.n_classes : 1;
  fo->F = p.F;
  fo->n_trees = p.n_trees;
  size_t maxd = 0;
  for (auto& t : trees) maxd = std::max(maxd, t.levels.size());
  std::vector<int64_t> level_base(maxd + 1, 0);
  std::vector<std::vector<int64_t>> tree_off(maxd);  // offset of tree in level
  for (size_t d = 0; d < maxd; ++d) {
    tree_off[d].resize(p.n_trees);
    int64_t off = 0;
    for (int t = 0; t < p.n_trees; ++t) {
      tree_off[d][t] = off;
      if (d < trees[t].levels.size()) off += (int64_t)trees[t].levels[d].size();
    }
    level_base[d + 1] = level_base[d] + off;
  }
  int64_t total = level_base[maxd];
  fo->node_array.assign((size_t)total * 5, 0);
  fo->gains32.assign((size_t)total, NAN);
  fo->gains64.assign((size_t)total, NAN);
  fo->depth.assign((size_t)total, 0);
  std::vector<int64_t> leaf_rank((size_t)total, -1);
  // child positions: the children of split node j (in tree order) at level d
  // are the next level's entries 2*s, 2*s+1 where s counts earlier splits
  for (size_t d = 0; d < maxd; ++d) {
    for (int t = 0; t < p.n_trees; ++t) {
      if (d >= trees[t].levels.size()) continue;
      const std::vector<NodeOut>& lv = trees[t].levels[d];
      int64_t splits = 0;
      for (size_t j = 0; j < lv.size(); ++j) {
        int64_t gi = level_base[d] + tree_off[d][t] + (int64_t)j;
        int32_t* rec = &fo->node_array[(size_t)gi * 5];
        fo->depth[gi] = (int32_t)d;
        if (lv[j].is_leaf) {
          rec[0] = -1;
          rec[1] = 0;
          rec[2] = 0;  // probability_start assigned below
          rec[3] = -1;
          float m1 = -1.0f;
          std::memcpy(&rec[4], &m1, 4);
        } else {
          int64_t cs = level_base[d + 1] + tree_off[d + 1][t] + 2 * splits;
          ++splits;
          rec[0] = (int32_t)cs;
          rec[1] = 2;
          rec[2] = -1;
          rec[3] = lv[j].attr;
          std::memcpy(&rec[4], &lv[j].thr, 4);
          fo->gains32[gi] = lv[j].gain32;
          fo->gains64[gi] = lv[j].gain64;
        }
      }
    }
  }
  // leaf payloads in node-array order
  for (size_t d = 0; d < maxd; ++d)
    for (int t = 0; t < p.n_trees; ++t) {
      if (d >= trees[t].levels.size()) continue;
      const std::vector<NodeOut>& lv = trees[t].levels[d];
      for (size_t j = 0; j < lv.size(); ++j) {
        if (!lv[j].is_leaf) continue;
        int64_t gi = level_base[d] + tree_off[d][t] + (int64_t)j;
        fo->node_array[(size_t)gi * 5 + 2] = (int32_t)fo->probs.size();
        if (p.task == 0)
          for (int c = 0; c < fo->C; ++c)
            fo->probs.push_back((float)lv[j].counts[c]);
        else
          fo->probs.push_back(lv[j].value);
      }
    }
  return fo;
}

void oracle_forest_sizes(void* h, int64_t* n_nodes, int64_t* n_probs) {
  Forest* f = (Forest*)h;
  *n_nodes = (int64_t)(f->node_array.size() / 5);
  *n_probs = (int64_t)f->probs.size();
}

void oracle_forest_export(void* h, int32_t* nodes, float* probs, float* g32,
                          double* g64, int32_t* depth) {
  Forest* f = (Forest*)h;
  std::memcpy(nodes, f->node_array.data(), f->node_array.size() * 4);
  std::memcpy(probs, f->probs.data(), f->probs.size() * 4);
  if (g32) std::memcpy(g32, f->gains32.data(), f->gains32.size() * 4);
  if (g64) std::memcpy(g64, f->gains64.data(), f->gains64.size() * 8);
  if (depth) std::memcpy(depth, f->depth.data(), f->depth.size() * 4);
}

void oracle_forest_free(void* h) { delete (Forest*)h; }

// Predict with a model in the reference's Classify layout (5 x int32 per
// node, split_point as float bits).  gpudte.cu:311-359: walk each tree, go
// left on a missing value (-FLT_MAX) or x < split_point; classification votes
// for the first class with the strictly largest leaf count; regression sums
// the tree outputs (in tree order).
void oracle_predict(const int32_t* nodes, const float* probs, int n_trees,
                    int C, int task, const float* X, int64_t N, float* out,
                    int threads) {
  int64_t width = task == 0 ? C : 1;
  std::memset(out, 0, sizeof(float) * (size_t)(N * width));
#ifdef _OPENMP
  int th = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(th)
#endif
  for (int64_t i = 0; i < N; ++i) {
    for (int t = 0; t < n_trees; ++t) {
      const int32_t* nd = nodes + (size_t)t * 5;
      while (nd[1] > 0) {
        float thr;
        std::memcpy(&thr, &nd[4], 4);
        float x = X[(int64_t)nd[3] * N + i];
        int64_t nx = goes_left(x, thr) ? nd[0] : nd[0] + 1;
        nd = nodes + (size_t)nx * 5;
      }
      const float* pr = probs + nd[2];
      if (task == 0) {
        int sel = 0;
        float mx = 0.0f;
        for (int c = 0; c < C; ++c)
          if (pr[c] > mx) {
            mx = pr[c];
            sel = c;
          }
        out[i * C + sel] += 1.0f;
      } else {
        out[i] = out[i] + pr[0];
      }
    }
  }
}

// Fixed-shape sum of v[0..n), the engine's order: block b of 256 threads
// covers [4096 b, 4096 (b+1)), thread j adds items j, j+256, ... in order, then
// a halving tree (w = 128 .. 1) over the block; the block sums are summed the
// same way by one block (thread j adds items j, j+256, ...).
static double tree256(std::vector<double>& sm) {
  for (int w = 128; w > 0; w >>= 1)
    for (int j = 0; j < w; ++j) sm[j] = sm[j] + sm[j + w];
  return sm[0];
}
static double fixed_sum(const double* v, int64_t n) {
  const int64_t nblk = (n + 4095) / 4096;
  std::vector<double> part((size_t)nblk), sm(256);
  for (int64_t b = 0; b < nblk; ++b) {
    for (int j = 0; j < 256; ++j) {
      double s = 0.0;
      for (int k = 0; k < 16; ++k) {
        int64_t i = b * 4096 + j + (int64_t)k * 256;
        if (i < n) s = s + v[i];
      }
      sm[j] = s;
    }
    part[b] = tree256(sm);
  }
  for (int j = 0; j < 256; ++j) {
    double s = 0.0;
    for (int64_t i = j; i < nblk; i += 256) s = s + part[i];
    sm[j] = s;
  }
  return tree256(sm);
}

// Out-of-bag estimate (gpurf.cu:290-359) and the permutation run of one
// feature (gpurf.cu:361-438), restated: every (tree, row) pair whose row is
// out of the tree's bag walks the tree; with perm_feature >= 0, nodes that
// split on it read row Philox(seed; row, row>>32, tree, kTagPermute | depth =
// feature).x % N instead.  Per row: pairs, correct pairs (classification) or
// sum of squared errors in tree order (regression), whether the row has a
// pair, and whether its out-of-bag vote is right (or the squared error of its
// mean out-of-bag output).  out[0..3] are the fixed-order sums of the four.
void oracle_oob(const oracle_desc* d, const int32_t* nodes, const float* probs,
                int perm_feature, double out[4]) {
  Problem p;
  p.algo = 0;
  p.task = d->task;
  p.n_trees = d->n_trees;
  p.n_classes = d->task == 0 ? d->n_classes : 1;
  p.seed = d->seed;
  p.N = d->n_rows;
  p.F = d->n_features;
  p.X = d->samples;
  p.y = d->targets;
  p.tree_offset = d->tree_offset;
  p.balanced = d->balanced;
  const int64_t N = p.N;
  const int C = p.n_classes;
  std::vector<std::vector<int32_t>> rows;
  if (p.balanced) rows = class_rows(p.y, N, C);
  std::vector<std::vector<int32_t>> bags((size_t)p.n_trees);
  for (int t = 0; t < p.n_trees; ++t) bags[t] = bag_counts(p, t, &rows);
  std::vector<double> acc((size_t)(4 * N), 0.0);
  for (int64_t i = 0; i < N; ++i) {
    int64_t pairs = 0, correct = 0;
    double se = 0.0, vsum = 0.0;
    std::vector<int64_t> votes((size_t)C, 0);
    const float target = p.y[i];
    for (int t = 0; t < p.n_trees; ++t) {
      if (bags[t][i] > 0) continue;
      int64_t prow = i;
      if (perm_feature >= 0) {
        W4 r = keyed(p.seed, kTagPermute, (uint32_t)perm_feature,
                     (uint32_t)(t + p.tree_offset), (uint32_t)i, (uint32_t)(i >> 32));
        prow = r.v[0] % (uint32_t)N;
      }
      const int32_t* nd = nodes + (size_t)t * 5;
      while (nd[1] > 0) {
        float thr;
        std::memcpy(&thr, &nd[4], 4);
        const int64_t r = nd[3] == perm_feature ? prow : i;
        const float x = p.X[(int64_t)nd[3] * N + r];
        nd = nodes + (size_t)(goes_left(x, thr) ? nd[0] : nd[0] + 1) * 5;
      }
      const float* pr = probs + nd[2];
      ++pairs;
      if (p.task == 0) {
        int sel = 0;
        float mx = 0.0f;
        for (int c = 0; c < C; ++c)
          if (pr[c] > mx) {
            mx = pr[c];
            sel = c;
          }
        correct += sel == (int)target;
        votes[sel] += 1;
      } else {
        const double v = (double)pr[0];
        const double e = (double)target - v;
        se = se + e * e;
        vsum = vsum + v;
      }
    }
    acc[i] = (double)pairs;
    acc[N + i] = p.task == 0 ? (double)correct : se;
    acc[2 * N + i] = pairs > 0 ? 1.0 : 0.0;
    double ens = 0.0;
    if (pairs > 0) {
      if (p.task == 0) {
        int sel = 0;
        int64_t mx = 0;
        for (int c = 0; c < C; ++c)
          if (votes[c] > mx) {
            mx = votes[c];
            sel = c;
          }
        ens = sel == (int)target ? 1.0 : 0.0;
      } else {
        const double e = (double)target - vsum / (double)pairs;
        ens = e * e;
      }
    }
    acc[3 * N + i] = ens;
  }
  for (int k = 0; k < 4; ++k) out[k] = fixed_sum(acc.data() + (size_t)k * N, N);
}

}  // extern "C"
