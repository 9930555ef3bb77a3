// Host stand-ins for the CUDA runtime names used by the reference's
// src/demag_cu.cu, so that the unmodified file compiles with g++ and its host
// function ktensorcpu::ktensorCPU and its kernel calHexchangeKernel run on the
// CPU.  TEST INFRASTRUCTURE ONLY (the oracle/_ref build of oracle/build_ref.py).
//
// - __global__ / __device__ vanish, so kernels become plain host functions;
// - threadIdx, blockIdx, blockDim, gridDim are file-scope variables that the
//   driver in oracle/ref_shim.cpp sets before each emulated thread's call;
// - cudaMemcpy is a host memcpy (ktensorCPU ends with copies "to the device",
//   src/demag_cu.cu:240-244; here the "device" buffers are host arrays).
#pragma once
#include <cmath>
#include <cstdio>
#include <cstring>

#define __global__
#define __device__
#define __host__

struct float2 { float x, y; };
struct double2 { double x, y; };
struct uint3 { unsigned int x, y, z; };
struct dim3 { unsigned int x, y, z; };

static uint3 threadIdx, blockIdx;
static dim3 blockDim, gridDim;

enum cudaError_t { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2 };

static inline cudaError_t cudaMemcpy(void* dst, const void* src, size_t bytes, cudaMemcpyKind) {
  std::memcpy(dst, src, bytes);
  return cudaSuccess;
}
