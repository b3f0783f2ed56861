/* CPU-only stand-in for the CUDA runtime calls the reference's MPM core makes
 * at construction (material_point_method.hpp:121-128,149-156,
 * material_point_method.cpp:144-154).  Allocation "succeeds" with a null device
 * pointer; nothing is ever launched because the only caller, precalculateWeights
 * (material_point_method.cpp:65-76), is never called by the oracle harness. */
#pragma once
#include <cstddef>
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
enum cudaError { cudaSuccess = 0, cudaErrorUnknown = 999 };
typedef cudaError cudaError_t;
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1,
                      cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };
inline cudaError_t cudaMalloc(void** p, std::size_t) { *p = nullptr; return cudaSuccess; }
inline cudaError_t cudaFree(void*) { return cudaSuccess; }
inline cudaError_t cudaMemcpy(void*, const void*, std::size_t, cudaMemcpyKind) { return cudaSuccess; }
inline cudaError_t cudaMemset(void*, int, std::size_t) { return cudaSuccess; }
inline cudaError_t cudaMemcpyToSymbol(const void*, const void*, std::size_t, std::size_t = 0,
                                      cudaMemcpyKind = cudaMemcpyHostToDevice) { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline const char* cudaGetErrorString(cudaError_t) { return "no device (CPU oracle build)"; }
