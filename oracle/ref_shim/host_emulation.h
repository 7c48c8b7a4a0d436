// Host emulation of the CUDA builtins used by the reference's device code, so
// that its device functions can be compiled by g++ as host code and run with
// one thread per block (blockDim.x == 1).  Part of the oracle's pinning
// harness (test infrastructure); never linked into the product.
#pragma once
#include <cstring>
#include <math.h>  // the float overloads of log() that device code sees
#define __device__
#define __host__
#define __global__
#define __constant__
#define __shared__ static
#define __forceinline__ inline

struct EmuDim3 {
  unsigned x, y, z;
};
extern EmuDim3 threadIdx, blockIdx, blockDim, gridDim;

inline void __syncthreads() {}
inline float atomicAdd(float* a, float v) {
  float o = *a;
  *a = o + v;
  return o;
}
inline int atomicAdd(int* a, int v) {
  int o = *a;
  *a = o + v;
  return o;
}
inline unsigned atomicAdd(unsigned* a, unsigned v) {
  unsigned o = *a;
  *a = o + v;
  return o;
}
inline unsigned long long atomicCAS(unsigned long long* a, unsigned long long c,
                                    unsigned long long v) {
  unsigned long long o = *a;
  if (o == c) *a = v;
  return o;
}
inline long long __double_as_longlong(double d) {
  long long r;
  std::memcpy(&r, &d, 8);
  return r;
}
inline double __longlong_as_double(long long l) {
  double r;
  std::memcpy(&r, &l, 8);
  return r;
}
