// Type name only: the reference's gpudte.cu includes this header but draws no
// random numbers (oracle pinning harness only).
#pragma once
struct curandStateMRG32k3a {
  unsigned s[8];
};
