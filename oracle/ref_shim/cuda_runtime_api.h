// Minimal host stand-in for the CUDA runtime API names the reference's
// device-code files mention (oracle pinning harness only).
#pragma once
#include <cstddef>
#include <cstring>
typedef enum cudaError_enum_rt { cudaSuccess = 0 } cudaError_t;
enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2
};
template <class S>
inline cudaError_t cudaMemcpyToSymbol(S& sym, const void* src, size_t n,
                                      size_t off = 0,
                                      cudaMemcpyKind = cudaMemcpyHostToDevice) {
  std::memcpy((char*)&sym + off, src, n);
  return cudaSuccess;
}
