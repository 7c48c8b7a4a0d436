// Internal structures shared by the fit/predict host drivers and kernels.
#pragma once
#include <cstdint>

namespace dml {

constexpr int kMaxClasses = 32;
constexpr int kMaxTries = 64;  // mandatory + optional tries evaluated per node

// Resident CTAs per SM of the big-node item kernel: four (64 registers) for 3
// to 16 classes, where the extra warps more than pay for the spills; three
// (80 registers) for one packed word (two classes, or regression, whose
// boundary scan keeps more per thread: four measured 3% slower there); two for
// wider class counts.
constexpr int big_ctas_per_sm(int cw) { return cw == 1 ? 3 : cw <= 8 ? 4 : 2; }

// Resident CTAs per SM of the shared-memory search kernel (80 registers and
// 59 KB of shared memory at the default cap of 2048 entries).
constexpr int smem_ctas_per_sm(int cw) { return cw <= 8 ? 3 : 2; }

// One forest of a fit batch (device-visible copy).
struct ProbDesc {
  const float* X;          // feature-major [F * N]
  const int32_t* lab;      // classification labels [N]
  const long long* q;      // regression targets, fixed point 2^-S [N]
  long long N;
  int F, C, K, n_mand, n_opt;
  int max_depth, min_node_size, min_leaf;
  int algo, task, S;
  unsigned long long seed;
  int n_trees;
  int tree0;               // global index of tree 0 of this forest in the batch
  long long ent0;          // entry slot of tree 0; tree t owns [ent0 + t*N, +N)
  int tree_key0;           // RNG tree key of tree 0 (trees sharded across calls)
  int balanced;            // RF classification: per-class bootstrap (easy ensemble)
  long long bal_m;         // draws per class: N / C
  const int* class_rows;   // rows of class c at [class_off[c], class_off[c+1]), ascending
  const long long* class_off;
  const uint32_t* rank;    // RF: dense value ranks [F * N] (null: sort raw keys)
  const float* vals;       // RF: value of each rank [F * N]
};

// An open node of the current level.  Levels are stored forest-major,
// tree-major, parent-ordered (left before right).
struct LNode {
  int prob, tree, idx, depth;
  int tstart, fstart, fend, ecnt;  // level positions: tree's / forest's first node, forest end
  long long ebeg;                  // first entry slot
  int n, pad;                      // weighted row count
  long long sum;                   // regression: sum of q * w
};

// Result of a node's search + split.
struct NodeRes {
  int split, f;
  float thr, gain;
  int nl_e, nl;      // entries / weighted rows going left
  long long suml;    // regression: left sum of q * w
};

// Node of the reference's model layout (gpudte_algorithm_shared.h:82-90).
struct ClassifyNode {
  int child_start, child_count, probability_start, attribute;
  float split_point;
};
static_assert(sizeof(ClassifyNode) == 20, "Classify node is 20 bytes");

// Predict layout: one 16-byte load per node.  Internal: {child_start,
// attribute, split bits, 0}; leaf: {-1, voted class, value bits, 0}.
struct PNode {
  int a, b;
  float t;
  int pad;
};

// Compact predict layout for bulk prediction, one 8-byte load per node, same
// node indices as PNode.  Internal: w = (offset of the children from the node
// << fbits) | feature; leaf: w = (voted class << fbits) | 2^fbits - 1; t = the
// split point or the regression leaf value.  Built when every feature and
// child offset fits (fbits = bits of the feature count).
struct PNode8 {
  uint32_t w;
  float t;
};

// Per-level, per-forest segment of the level list (for the final gather).
struct Seg {
  long long node_pos;   // position in the node log
  int node_cnt;
  int pad;
  long long leaf_rank;  // first leaf rank in the probability log
  long long leaf_cnt;
};

}  // namespace dml
