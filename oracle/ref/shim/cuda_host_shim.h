/*
 * cuda_host_shim.h -- lets the reference's kernel sources compile as plain
 * host C++ (TEST INFRASTRUCTURE ONLY, used to pin the oracle).
 *
 * The reference kernels use one thread per item, no shared memory, no
 * atomics and no synchronisation, so running each "thread" as one iteration
 * of a host loop is exact.  blockIdx/threadIdx/blockDim are thread-local so
 * the host loop may be OpenMP-parallel.
 */
#pragma once
#include <cmath>
#include <cstdio>
#include <array>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __forceinline__ inline

struct shim_dim3 { unsigned int x, y, z; };
extern thread_local shim_dim3 blockIdx, threadIdx, blockDim, gridDim;

/* round-down conversion used by getPBCCellIndex */
inline long long __double2ll_rd(double x) { return (long long)std::floor(x); }
