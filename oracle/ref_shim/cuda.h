// Minimal host stand-in for CUDA driver API type names (oracle pinning harness only).
#pragma once
typedef void* CUcontext;
typedef void* CUstream;
typedef enum cudaError_enum_drv { CUDA_SUCCESS = 0 } CUresult;
typedef int CUdevice;
typedef unsigned long long CUdeviceptr;
