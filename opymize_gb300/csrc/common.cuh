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
// Programmatic dependent launch.  A kernel launched by launch_chained may be
// scheduled while the kernel before it on the stream drains (its CTAs take
// the SM slots that the earlier kernel's CTAs free); they set up shared
// memory, then call chain_wait() before their first global memory access
// (read or write), which returns once that kernel has completed and its
// writes are visible.  The dependents of a chained kernel are released as its
// CTAs exit: releasing them at the start (griddepcontrol.launch_dependents)
// measured slower inside CUDA graphs (1000 sweeps of 1024^2: 10.3 ms against
// 9.2 ms released at exit and 9.5 ms launched plainly).  For a kernel launched
// plainly chain_wait() is a no-op.
// ---------------------------------------------------------------------------

#ifndef OPYX_CHAIN
#define OPYX_CHAIN 1   // 0: chained kernels are launched plainly
#endif

OPYX_D void chain_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... Params, typename... Args>
inline void launch_chained(void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem,
                           cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = OPYX_CHAIN ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, args...);
}

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

// The last block's part of the reductions below: fold the NV partials of
// every block in fixed block order (deterministic) and hand the totals to
// `finish` (thread 0).  Each thread adds its strided share b = tid,
// tid + nthreads, ... in that order; the L2 loads of four shares of every
// value are issued before their adds (one L2 round trip per four shares
// instead of one per partial: with ~1500 blocks the serial chain of loads
// cost ~35 us).
template <int NV, typename Finish>
__device__ void fold_partials_and_finish(const int (&ops)[NV], const double* partials,
                                         unsigned* ticket, unsigned nblocks, int tid,
                                         int nthreads, double (*s_warp)[NV], Finish finish) {
  const int lane = tid & 31, warp = tid >> 5;
  const int nwarps = (nthreads + 31) >> 5;
  double tot[NV];
  double acc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) acc[v] = ops[v] == RED_MAX ? -INFINITY : 0.0;
  constexpr int kFoldLoads = 4;
  for (unsigned b0 = tid; b0 < nblocks; b0 += kFoldLoads * nthreads) {
    double t[NV][kFoldLoads];
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
      for (int j = 0; j < kFoldLoads; ++j) {
        const unsigned b = b0 + j * nthreads;
        t[v][j] = b < nblocks ? __ldcg(partials + (size_t)v * nblocks + b) : 0.0;
      }
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
      for (int j = 0; j < kFoldLoads; ++j)
        if (b0 + j * nthreads < nblocks) acc[v] = red_apply(ops[v], acc[v], t[v][j]);
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double r = warp_reduce(ops[v], acc[v]);
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
  fold_partials_and_finish<NV>(ops, partials, ticket, nblocks, tid, nthreads, s_warp, finish);
}

// ---------------------------------------------------------------------------
// Double-float sums: a value as an unevaluated FP32 pair hi + lo (about 48
// significant bits), added by Knuth's TwoSum (the rounding error of hi + hi'
// recovered exactly) and renormalised.  Within blocks the gap sums are
// carried this way instead of in FP64, whose pipe on this GPU is narrow: a
// block reduction of five FP64 values per warp cost ~14 us per sweep over a
// 2048^2 image (912 blocks ending together).
// ---------------------------------------------------------------------------

struct DF {
  float hi, lo;
};

OPYX_D DF df_add(DF a, DF b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb);
  const float lo = (a.lo + b.lo) + e;
  const float h = s + lo;
  return {h, lo - (h - s)};
}

OPYX_D DF warp_sum_df(DF v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const DF w = {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = df_add(v, w);
  }
  return v;
}

OPYX_D float warp_max_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Arrival of a block at a reduction whose last block folds the partials:
// `tickets` holds 1 + kTicketGroups zeroed counters.  Blocks count in
// kTicketGroups groups (bid % kTicketGroups) and the last of each group in
// tickets[0], so no counter takes more than ~nblocks / 32 atomics (one
// counter for ~900 blocks, as the sweep's grid has, cost several us of
// serialised atomics at the end of the kernel).  Called by one thread per
// block after its partials are written; true for the last block overall,
// which then resets every counter.
constexpr int kTicketGroups = 32;

OPYX_D bool arrive_grouped(unsigned* tickets, unsigned bid, unsigned nblocks) {
  const unsigned ng = nblocks < (unsigned)kTicketGroups ? nblocks : (unsigned)kTicketGroups;
  const unsigned g = bid % ng;
  const unsigned in_g = nblocks / ng + (g < nblocks % ng ? 1u : 0u);
  __threadfence();
  if (atomicAdd(&tickets[1 + g], 1u) != in_g - 1) return false;
  __threadfence();
  if (atomicAdd(&tickets[0], 1u) != ng - 1) return false;
  __threadfence();
  for (unsigned j = 0; j <= ng; ++j) tickets[j] = 0u;
  return true;
}

// As block_reduce_and_finish for NS sums given as double-float pairs and one
// maximum given in FP32: each block's partials (sums, then the max) are
// stored as FP32 pairs (hi, lo) in the `partials` buffer, and the last block
// folds them in double-float as well, in fixed block order; only the NS + 1
// totals handed to `finish` are FP64 (double(hi) + double(lo)).  An FP64
// fold of ~900 blocks' partials by the last block cost ~9 us at the end of
// the kernel.  `ticket` points to 1 + kTicketGroups zeroed counters
// (arrive_grouped).
template <int NS, typename Finish>
__device__ void block_reduce_df_and_finish(const DF (&sums)[NS], float mx, double* partials,
                                           unsigned* ticket, Finish finish) {
  constexpr int NV = NS + 1;
  __shared__ DF s_df[32][NS];
  __shared__ float s_mx[32];
  __shared__ bool s_last;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
  const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
  const int lane = tid & 31, warp = tid >> 5;
  const int nwarps = (nthreads + 31) >> 5;
  float2* part = reinterpret_cast<float2*>(partials);
  // this block's totals -> one partial per value
#pragma unroll
  for (int v = 0; v < NS; ++v) {
    const DF r = warp_sum_df(sums[v]);
    if (lane == 0) s_df[warp][v] = r;
  }
  const float m = warp_max_f(mx);
  if (lane == 0) s_mx[warp] = m;
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int v = 0; v < NS; ++v) {
      const DF r = warp_sum_df(lane < nwarps ? s_df[lane][v] : DF{0.f, 0.f});
      if (lane == 0) part[(size_t)v * nblocks + bid] = make_float2(r.hi, r.lo);
    }
    const float mb = warp_max_f(lane < nwarps ? s_mx[lane] : -INFINITY);
    if (lane == 0) {
      part[(size_t)NS * nblocks + bid] = make_float2(mb, 0.f);
      s_last = arrive_grouped(ticket, bid, nblocks);
    }
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // last block: each thread folds its strided share b = tid, tid + nthreads,
  // ... in that order, with the L2 loads of four shares issued before their adds
  DF acc[NS];
  float amx = -INFINITY;
#pragma unroll
  for (int v = 0; v < NS; ++v) acc[v] = DF{0.f, 0.f};
  constexpr int kFoldLoads = 4;
  for (unsigned b0 = tid; b0 < nblocks; b0 += kFoldLoads * nthreads) {
    float2 t[NV][kFoldLoads];
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
      for (int j = 0; j < kFoldLoads; ++j) {
        const unsigned b = b0 + j * nthreads;
        t[v][j] = b < nblocks ? __ldcg(part + (size_t)v * nblocks + b) : make_float2(0.f, 0.f);
      }
#pragma unroll
    for (int j = 0; j < kFoldLoads; ++j) {
      if (b0 + j * nthreads >= nblocks) break;
#pragma unroll
      for (int v = 0; v < NS; ++v) acc[v] = df_add(acc[v], DF{t[v][j].x, t[v][j].y});
      amx = fmaxf(amx, t[NS][j].x);
    }
  }
  __syncthreads();   // s_df, s_mx of this block's own partial are read
#pragma unroll
  for (int v = 0; v < NS; ++v) {
    const DF r = warp_sum_df(acc[v]);
    if (lane == 0) s_df[warp][v] = r;
  }
  const float wm = warp_max_f(amx);
  if (lane == 0) s_mx[warp] = wm;
  __syncthreads();
  if (warp == 0) {
    double tot[NV];
#pragma unroll
    for (int v = 0; v < NS; ++v) {
      const DF r = warp_sum_df(lane < nwarps ? s_df[lane][v] : DF{0.f, 0.f});
      tot[v] = (double)r.hi + (double)r.lo;
    }
    tot[NS] = (double)warp_max_f(lane < nwarps ? s_mx[lane] : -INFINITY);
    if (lane == 0) finish(tot);
  }
}

}  // namespace opyx
