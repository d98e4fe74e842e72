/*
 * shim.h — lets the reference's .cu sources compile as host C++ for the
 * validation harness.  TEST INFRASTRUCTURE ONLY.
 *
 * CUDA qualifiers become nothing (or 'static' for __shared__ inside the
 * Smith-Waterman kernel, so that one CPU "block" of fibers shares them);
 * threadIdx/blockIdx/blockDim are globals set by the fiber scheduler;
 * __syncthreads() yields to the next fiber.  Device memory is host memory:
 * cudaMalloc returns zeroed memory with 64 KB of zeroed slack after it (so
 * reads just past an allocation see 0), cudaMemcpy and cudaMemcpyToSymbol
 * copy, cudaFree frees.
 *
 * REF_L13 (lookupTable13.cu): the block's __shared__ variables go to the
 * section ref13shr, which the harness zeroes before every block, calloc
 * leaves room for the one-past-the-end write of lookupTable13Create, and
 * the file's __constant__ tables get names of their own (constant memory
 * is per module in CUDA; lookupTable5.cu defines the same names).
 */
#ifndef REF_SHIM_H_
#define REF_SHIM_H_
#include <ctype.h>
#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "common.h"
#undef TMP_DIR
#define TMP_DIR REF_TMP_DIR

#define __global__
#define __device__
#define __host__
#define __constant__
#if defined(REF_L13)
#define __shared__ static __attribute__((section("ref13shr")))
static inline void *ref13_calloc(size_t n, size_t sz) { return calloc(n + 1024, sz); }
#define calloc ref13_calloc
/* __constant__ arrays are per module in CUDA; lookupTable5.cu has its own */
#define hashCodes_gpu ref13_hashCodes_gpu
#define powerVals_gpu ref13_powerVals_gpu
#elif defined(REF_SHARED_STATIC)
#define __shared__ static
/* the kernel file defines its own toupper; keep libc's declaration apart */
#define toupper ref_sw_toupper
#else
#define __shared__
#endif

#ifdef REF_ALIGN
/* align.cu: device queries answered for one device, rand() pinned to 0 */
extern "C" int ref_rand_zero(void);
#define rand ref_rand_zero
#endif

#ifdef REF_PIN_RAND
/* array.cu: rand() -> a counter 0, 1, 2, ... reset before each call of
 * interest, which pins mapHits6's random picks to the first clusters */
extern "C" int ref_rand(void);
#define rand ref_rand
#endif

/* device-side min/max that CUDA provides */
static inline int max(int a, int b) { return a > b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }
static inline short max(short a, short b) { return a > b ? a : b; }
static inline long long max(long long a, long long b) { return a > b ? a : b; }
static inline short min(short a, short b) { return a < b ? a : b; }

struct ref_dim3 {
  unsigned int x, y, z;
};
extern struct ref_dim3 threadIdx, blockIdx, blockDim, gridDim;
void __syncthreads(void);

typedef int cudaError_t;
typedef struct ref_dim3 dim3;
/* the device align.cu sizes its batches from: ref_device_mem bytes */
extern long long ref_device_mem;
struct cudaDeviceProp {
  size_t totalGlobalMem;
  int maxGridSize[3];
  int regsPerBlock;
  int maxThreadsPerBlock;
  size_t sharedMemPerBlock;
};
static inline cudaError_t cudaGetDeviceProperties(struct cudaDeviceProp *p, int) {
  memset(p, 0, sizeof(*p));
  p->totalGlobalMem = (size_t)ref_device_mem;
  p->maxGridSize[0] = 2147483647;
  p->regsPerBlock = 65536;
  p->maxThreadsPerBlock = 1024;
  p->sharedMemPerBlock = 49152;
  return 0;
}
static inline cudaError_t cudaGetDevice(int *d) { *d = 0; return 0; }
static inline cudaError_t cudaGetDeviceCount(int *n) { *n = 1; return 0; }
static inline cudaError_t cudaSetDevice(int) { return 0; }
enum cudaMemcpyKind {
  cudaMemcpyHostToHost,
  cudaMemcpyHostToDevice,
  cudaMemcpyDeviceToHost,
  cudaMemcpyDeviceToDevice
};
#define cudaSuccess 0
cudaError_t cudaGetLastError(void);
const char *cudaGetErrorString(cudaError_t);
cudaError_t cudaMalloc(void **, size_t);
cudaError_t cudaFree(void *);
cudaError_t cudaMemcpy(void *, const void *, size_t, enum cudaMemcpyKind);
cudaError_t cudaMemset(void *, int, size_t);
template <class T>
cudaError_t cudaMemcpyToSymbol(const T &sym, const void *src, size_t n, size_t off = 0,
                               enum cudaMemcpyKind = cudaMemcpyHostToDevice) {
  memcpy((char *)&sym + off, src, n);
  return 0;
}
#endif
