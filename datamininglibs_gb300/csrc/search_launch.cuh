// Launch of the split-search kernels of one node class, instantiated per
// packed class-count width CW in search_cw*.cu (compiled in parallel).
#pragma once
#include "engine.h"
#include "level_kernels.cuh"
#include "big_rf.cuh"
#include "ert_warp.cuh"

namespace dml {

constexpr int kBlock = 256;
constexpr int kSmemCap = kSearchSmemCap;  // RF nodes up to this many entries fit shared memory

template <int CW>
void launch_search_cw(int q, const LevelArgs& a, int count, cudaStream_t s);
// Both phases of the big-node path (per-try items, decide + partition).
template <int CW>
void launch_big_cw(BigArgs b, int phase, int grid, int decide_grid, int tries, cudaStream_t s);

#ifdef DML_SEARCH_CW
// cudaFuncSetAttribute acts on the current device only, and fits run on
// whatever device the calling thread selects, so the shared-memory limit of the
// CTA kernel is raised before each of its launches (one per level, a host call
// of about a microsecond) rather than once per process.
template <int CW>
static void set_smem_attrs() {
  DML_CK(cudaFuncSetAttribute(k_rf_smem<CW, kSmemCap>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              kSmemCap * 24));
}

template <int CW>
void launch_search_cw(int q, const LevelArgs& a, int count, cudaStream_t s) {
  LevelArgs b = a;
  b.nwork = count;
  const int wblocks = std::max(1, std::min((count + 7) / 8, 1 << 20));
  if (q == kQWarp) {
    k_group_nodes<CW, 32><<<wblocks, 256, 0, s>>>(b);
  } else if (q == kQG16) {
    k_group_nodes<CW, 16><<<std::max(1, std::min((count + 15) / 16, 1 << 20)), 256, 0, s>>>(b);
  } else if (q == kQG8) {
    k_group_nodes<CW, 8><<<std::max(1, std::min((count + 31) / 32, 1 << 20)), 256, 0, s>>>(b);
  } else if (q == kQRfW2) {
    k_warp_rf<2, CW><<<wblocks, 256, 0, s>>>(b);
  } else if (q == kQRfW4) {
    k_warp_rf<4, CW><<<wblocks, 256, 0, s>>>(b);
  } else if (q == kQRfW8) {
    k_warp_rf<8, CW><<<wblocks, 256, 0, s>>>(b);
  } else if (q == kQRfW16) {
    constexpr int wpb = warp_rf_wpb<16>();
    k_warp_rf<16, CW><<<std::max(1, std::min((count + wpb - 1) / wpb, 1 << 20)), 32 * wpb, 0, s>>>(b);
  } else if (q == kQErtW) {
    k_ert_warp<8><<<wblocks, 256, 0, s>>>(b);
  } else if (q == kQErt) {
    k_ert_cta<kBlock><<<std::min(count, 1 << 20), kBlock, 0, s>>>(b);
  } else {
    set_smem_attrs<CW>();
    k_rf_smem<CW, kSmemCap><<<std::min(count, 1 << 20), kBlock, (size_t)b.smem_cap * 24, s>>>(b);
  }
  DML_CK(cudaGetLastError());
}

template <int CW>
void launch_big_cw(BigArgs b, int phase, int grid, int decide_grid, int tries, cudaStream_t s) {
  b.phase = phase;
  b.tries_per_node = tries;
  if (phase == 1) k_big_pack<CW><<<decide_grid, kBigBlock, 0, s>>>(b);
  k_rf_big_items<CW><<<grid, kBigBlock, 0, s>>>(b);
  k_rf_big_decide<CW><<<decide_grid, kBigBlock, 0, s>>>(b);
  DML_CK(cudaGetLastError());
}

#endif

}  // namespace dml
