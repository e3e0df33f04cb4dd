/*
 * cuda_host_shim.h -- lets the reference's CUDA sources compile as host C++.
 *
 * TEST INFRASTRUCTURE ONLY: used by oracle/build_ref.py to build the
 * reference's own kernels (rupertnash/gpu-swimmers, lbswim/liblbswim/*.cu) for
 * the CPU, so the oracle restatement can be pinned against them.  Kernel
 * launches are rewritten by build_ref.py into ref_launch(grid, block, body),
 * which runs every block (OpenMP) and every thread of the block in turn.  The
 * reference kernels use no __syncthreads or shared memory, so running the
 * threads of a block one after another is a valid schedule.
 */
#ifndef CUDA_HOST_SHIM_H
#define CUDA_HOST_SHIM_H

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>

#define __global__
#define __device__
#define __host__
#define __constant__

struct dim3 {
  unsigned int x, y, z;
  dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};

static thread_local dim3 threadIdx(0, 0, 0);
static thread_local dim3 blockIdx(0, 0, 0);
static thread_local dim3 blockDim(1, 1, 1);
static thread_local dim3 gridDim(1, 1, 1);

typedef int cudaError;
typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3
};

static inline const char* cudaGetErrorString(int) { return "host shim"; }
template <typename T>
static inline int cudaMalloc(T** p, size_t bytes) {
  *p = (T*)calloc(bytes ? bytes : 1, 1);
  return *p ? 0 : 2;
}
static inline int cudaFree(void* p) {
  free(p);
  return 0;
}
static inline int cudaMemcpy(void* dst, const void* src, size_t bytes, int) {
  memcpy(dst, src, bytes);
  return 0;
}
static inline int cudaDeviceSynchronize() { return 0; }

static inline unsigned long long atomicCAS(unsigned long long* addr, unsigned long long compare,
                                           unsigned long long val) {
  unsigned long long expected = compare;
  __atomic_compare_exchange_n(addr, &expected, val, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
  return expected;
}
static inline long long __double_as_longlong(double d) {
  long long r;
  memcpy(&r, &d, sizeof r);
  return r;
}
static inline double __longlong_as_double(long long l) {
  double r;
  memcpy(&r, &l, sizeof r);
  return r;
}

int ref_shim_threads();

template <typename F>
static void ref_launch(dim3 grid, dim3 block, F body) {
  const long nb = (long)grid.x * grid.y * grid.z;
#pragma omp parallel for schedule(dynamic) num_threads(ref_shim_threads())
  for (long b = 0; b < nb; b++) {
    gridDim = grid;
    blockDim = block;
    blockIdx = dim3((unsigned)(b % grid.x), (unsigned)((b / grid.x) % grid.y),
                    (unsigned)(b / ((long)grid.x * grid.y)));
    for (unsigned tz = 0; tz < block.z; tz++)
      for (unsigned ty = 0; ty < block.y; ty++)
        for (unsigned tx = 0; tx < block.x; tx++) {
          threadIdx = dim3(tx, ty, tz);
          body();
        }
  }
}
template <typename F>
static void ref_launch(int grid, int block, F body) {
  ref_launch(dim3((unsigned)grid), dim3((unsigned)block), body);
}

#endif
