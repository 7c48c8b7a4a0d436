// The engine's Philox4x32-10 (dml_device.cuh, written from Salmon et al.,
// SC'11) against cuRAND's Philox4_32_10 generator on the same counters and
// keys.  cuRAND's state for (seed, subsequence, offset) sits at counter
// {offset/4 (64-bit), subsequence (64-bit)} with key = seed, and curand4()
// returns the block of that counter, so for counter {c0, c1, c2, c3}:
//   curand_init(seed, c2 | c3 << 32, 4 * (c0 | c1 << 32), &st); curand4(&st)
// (for c1 < 2^30, where the offset fits 64 bits)
// Prints the number of mismatching words; exit status 0 when there are none.
#include <cstdio>
#include <cstdlib>

#include <curand_kernel.h>

#include "dml_device.cuh"

__global__ void k_compare(const uint4* ctr, const unsigned long long* seed, int n,
                          unsigned* mismatches) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint4 c = ctr[i];
  const unsigned long long k = seed[i];
  curandStatePhilox4_32_10_t st;
  curand_init(k, (unsigned long long)c.z | ((unsigned long long)c.w << 32),
              4ull * ((unsigned long long)c.x | ((unsigned long long)c.y << 32)), &st);
  const uint4 r = curand4(&st);
  const dml::U4 m = dml::philox4x32_10(c.x, c.y, c.z, c.w, (uint32_t)k, (uint32_t)(k >> 32));
  const unsigned bad = (r.x != m.x) + (r.y != m.y) + (r.z != m.z) + (r.w != m.w);
  if (bad) atomicAdd(mismatches, bad);
}

int main() {
  const int n = 1 << 16;
  uint4* hc = (uint4*)malloc(sizeof(uint4) * n);
  unsigned long long* hs = (unsigned long long*)malloc(sizeof(unsigned long long) * n);
  unsigned long long x = 0x9E3779B97F4A7C15ull;
  auto next = [&]() {  // splitmix64 for varied counters and keys
    x += 0x9E3779B97F4A7C15ull;
    unsigned long long z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  for (int i = 0; i < n; ++i) {
    const unsigned long long a = next(), b = next();
    // the engine's draws: small counters, tag << 24 | depth in the last word
    if (i % 2 == 0)
      hc[i] = make_uint4((unsigned)(a % 100000), (unsigned)(a >> 60), (unsigned)(b % 4096),
                         (3u << 24) | (unsigned)(b >> 59));
    else  // c1 < 2^30 so that the offset 4 * (c0 | c1 << 32) fits 64 bits
      hc[i] = make_uint4((unsigned)a, (unsigned)(a >> 34), (unsigned)b, (unsigned)(b >> 32));
    hs[i] = i % 3 == 0 ? (unsigned long long)(i % 7) : next();
  }
  uint4* dc;
  unsigned long long* ds;
  unsigned* dm;
  cudaMalloc(&dc, sizeof(uint4) * n);
  cudaMalloc(&ds, sizeof(unsigned long long) * n);
  cudaMalloc(&dm, sizeof(unsigned));
  cudaMemcpy(dc, hc, sizeof(uint4) * n, cudaMemcpyHostToDevice);
  cudaMemcpy(ds, hs, sizeof(unsigned long long) * n, cudaMemcpyHostToDevice);
  cudaMemset(dm, 0, sizeof(unsigned));
  k_compare<<<(n + 255) / 256, 256>>>(dc, ds, n, dm);
  unsigned bad = 0;
  const cudaError_t e = cudaMemcpy(&bad, dm, sizeof(unsigned), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    printf("cuda error: %s\n", cudaGetErrorString(e));
    return 2;
  }
  printf("compared %d blocks of 4 words, mismatching words: %u\n", n, bad);
  return bad == 0 ? 0 : 1;
}
