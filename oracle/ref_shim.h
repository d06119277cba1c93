/*
 * ref_shim.h -- lets the reference's CUDA kernel source compile as plain C++
 * on the host (TEST INFRASTRUCTURE: used only to build oracle/_ref, the
 * checker that pins the RC restatement in kvtomo_oracle.c).
 *
 * The reference kernels (Projector.cu, the __device__/__global__ functions
 * only) are compiled once per ray / voxel with blockDim = (1,1,1) and the
 * ray or voxel index placed in a thread-local blockIdx.
 */
#pragma once
#include <cmath>
#include <cstdio>

#define __global__
#define __device__
#define __host__
#define __forceinline inline

struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};
struct float2 { float x, y; };
struct float3 { float x, y, z; };

extern thread_local dim3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 threadIdx;

using std::fabs;
using std::fmax;
using std::fmin;
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }
