/*
 * shim.h - lets the reference's CUDA kernel sources compile as plain C++ for the CPU, so that
 * the oracle can be checked against the reference's own code.  TEST INFRASTRUCTURE ONLY.
 *
 * Execution model: a kernel is an ordinary function; ref_harness.cpp runs it once per thread
 * index, blocks and threads in ascending order, one at a time.  Atomics are therefore plain
 * read-modify-writes, and every order-dependent kernel behaves as if its threads ran in
 * ascending global index order.  __syncthreads is a no-op, so kernels that need it
 * (block-level histograms) must not be run; the hot-path kernels do not use it.
 */
#ifndef REF_SHIM_H
#define REF_SHIM_H
#define __CUDACC__ 1
#include <math.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>
#include <stdint.h>
#include <cmath>
#include <algorithm>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__
#define __forceinline__ inline
#define __noinline__

struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct int2 { int x, y; };
struct uint3 { unsigned int x, y, z; };
struct dim3 { unsigned int x = 1, y = 1, z = 1; };
inline float2 make_float2(float x, float y) { return {x, y}; }
inline float3 make_float3(float x, float y, float z) { return {x, y, z}; }
inline float4 make_float4(float x, float y, float z, float w) { return {x, y, z, w}; }
inline int2 make_int2(int x, int y) { return {x, y}; }

extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;
inline void __syncthreads() {}

/* sequential atomics */
template <class T, class U> inline T atomicAdd(T *a, U v) { T o = *a; *a = (T)(o + v); return o; }
template <class T, class U> inline T atomicOr(T *a, U v) { T o = *a; *a = (T)(o | v); return o; }
template <class T> inline T atomicMin(T *a, T v) { T o = *a; *a = v < o ? v : o; return o; }
template <class T> inline T atomicMax(T *a, T v) { T o = *a; *a = v > o ? v : o; return o; }
template <class T> inline T atomicExch(T *a, T v) { T o = *a; *a = v; return o; }
template <class T> inline T atomicCAS(T *a, T cmp, T v) { T o = *a; if (o == cmp) *a = v; return o; }

inline float __saturatef(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
inline float max(float a, float b) { return fmaxf(a, b); }
inline float min(float a, float b) { return fminf(a, b); }
inline double max(double a, double b) { return fmax(a, b); }
inline double min(double a, double b) { return fmin(a, b); }

/* host runtime API: declarations and inert stand-ins (the harness never allocates through them) */
typedef int cudaError_t;
typedef cudaError_t cudaError;
enum { cudaSuccess = 0 };
typedef struct CUstream_st *cudaStream_t;
typedef struct cudaArray *cudaArray_t;
struct cudaGraphicsResource;
typedef struct cudaGraphicsResource *cudaGraphicsResource_t;
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost,
                      cudaMemcpyDeviceToDevice, cudaMemcpyDefault };
inline const char *cudaGetErrorString(cudaError_t) { return "shim"; }
inline cudaError_t cudaGetLastError() { return 0; }
inline cudaError_t cudaDeviceSynchronize() { return 0; }
template <class T> inline cudaError_t cudaMalloc(T **p, size_t n) { *p = (T *)calloc(1, n); return 0; }
template <class T> inline cudaError_t cudaMallocAsync(T **p, size_t n, cudaStream_t) { *p = (T *)calloc(1, n); return 0; }
inline cudaError_t cudaFree(void *p) { free(p); return 0; }
inline cudaError_t cudaFreeAsync(void *p, cudaStream_t) { free(p); return 0; }
inline cudaError_t cudaMemset(void *p, int v, size_t n) { memset(p, v, n); return 0; }
inline cudaError_t cudaMemsetAsync(void *p, int v, size_t n, cudaStream_t = nullptr) { memset(p, v, n); return 0; }
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { memcpy(d, s, n); return 0; }
inline cudaError_t cudaMemcpyAsync(void *d, const void *s, size_t n, cudaMemcpyKind, cudaStream_t = nullptr) { memcpy(d, s, n); return 0; }
template <class T> inline cudaError_t cudaMemcpyToSymbol(T &sym, const void *src, size_t n) { memcpy(&sym, src, n); return 0; }
#endif
