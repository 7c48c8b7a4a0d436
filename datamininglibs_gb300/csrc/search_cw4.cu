// Split-search kernels instantiated for 4 packed class-count word(s).
#define DML_SEARCH_CW 1
#include "search_launch.cuh"

namespace dml {
template void launch_search_cw<4>(int, const LevelArgs&, int, cudaStream_t);
template void launch_big_cw<4>(BigArgs, int, int, int, int, cudaStream_t);
}  // namespace dml
