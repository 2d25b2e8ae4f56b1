// Shared device/host helpers of libopyx (GB300, sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "opyx.h"

#define OPYX_HD __host__ __device__ __forceinline__
#define OPYX_D __device__ __forceinline__

namespace opyx {

// 152 SMs on GB300; grids of grid-stride kernels are sized in multiples of
// this (re-read from the device at first use).
int sm_count();

// Grid size for a grid-stride loop over n items with `block` threads.
inline unsigned grid_for(int64_t n, int block, int per_sm = 8) {
  int64_t want = (n + block - 1) / block;
  int64_t cap = (int64_t)sm_count() * per_sm;
  if (want < 1) want = 1;
  return (unsigned)(want < cap ? want : cap);
}

inline int check_launch() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? OPYX_OK : OPYX_ERR_LAUNCH;
}

#define OPYX_CHECK_LAUNCH() do { int _s = ::opyx::check_launch(); if (_s) return _s; } while (0)

// Dispatch on the run-time dtype code to a templated callable.
#define OPYX_DISPATCH(dtype, T, ...)                                   \
  do {                                                                 \
    if ((dtype) == OPYX_F32) { using T = float; __VA_ARGS__; }         \
    else if ((dtype) == OPYX_F64) { using T = double; __VA_ARGS__; }   \
    else return OPYX_ERR_ARG;                                          \
  } while (0)

template <typename T> OPYX_D T ld(const T* p) { return __ldg(p); }

// ---------------------------------------------------------------------------
// Deterministic FP64 reductions.
//
// Each block reduces NV values (sum or max) to one partial per value with
// warp shuffles, writes the partials to `partials[v*nblocks + block]`, and the
// last block to arrive (atomic ticket) folds all partials in block order and
// hands the NV totals to `finish`.  The ticket is reset by that last block, so
// a reduction buffer can be reused by the next launch on the same stream.
// ---------------------------------------------------------------------------

enum RedOp { RED_SUM = 0, RED_MAX = 1 };

OPYX_D double red_apply(int op, double a, double b) {
  return op == RED_MAX ? fmax(a, b) : a + b;
}

OPYX_D double warp_reduce(int op, double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = red_apply(op, v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block size must be a multiple of 32 and at most 1024.
template <int NV, typename Finish>
__device__ void block_reduce_and_finish(double (&vals)[NV], const int (&ops)[NV],
                                        double* partials, unsigned* ticket,
                                        Finish finish) {
  __shared__ double s_warp[32][NV];
  __shared__ bool s_last;
  // linear thread / block ids: blocks and grids may be 2-D or 3-D
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
  const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
  const int lane = tid & 31, warp = tid >> 5;
  const int nwarps = (nthreads + 31) >> 5;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    double r = warp_reduce(ops[v], vals[v]);
    if (lane == 0) s_warp[warp][v] = r;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double r = lane < nwarps ? s_warp[lane][v] : (ops[v] == RED_MAX ? -INFINITY : 0.0);
      r = warp_reduce(ops[v], r);
      if (lane == 0) partials[(size_t)v * nblocks + bid] = r;
    }
    if (lane == 0) {
      __threadfence();
      unsigned t = atomicAdd(ticket, 1u);
      s_last = (t == nblocks - 1);
    }
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // Last block: fold partials in fixed block order (deterministic).
  double tot[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    double r = ops[v] == RED_MAX ? -INFINITY : 0.0;
    for (unsigned b = tid; b < nblocks; b += nthreads)
      r = red_apply(ops[v], r, ((volatile double*)partials)[(size_t)v * nblocks + b]);
    r = warp_reduce(ops[v], r);
    __syncwarp();
    if (lane == 0) s_warp[warp][v] = r;
  }
  __syncthreads();
  if (tid == 0) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double r = ops[v] == RED_MAX ? -INFINITY : 0.0;
      for (int w = 0; w < nwarps; ++w) r = red_apply(ops[v], r, s_warp[w][v]);
      tot[v] = r;
    }
    *ticket = 0u;
    finish(tot);
  }
}

}  // namespace opyx
