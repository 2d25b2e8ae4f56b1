// Kernels of the learned warm start: a U-Net on NHWC bf16 activations whose
// 3x3 convolutions run on the tcgen05 tensor cores, plus the elementwise,
// pooling, loss and optimiser kernels around them.
//
// Convolution as an implicit GEMM: the output tile is 128 pixels (one or
// more whole image rows of a level: 128 / min(W, 128) rows of min(W, 128)
// pixels) x Cout channels.  For each of the 9 taps and each 32-channel chunk
// of the input, a TMA tiled copy brings the 128 shifted input pixels (rows
// of 64 bytes; out-of-image coordinates are filled with zeros, which is the
// convolution's zero padding) and the tap's Cout x 32 weight block into a
// shared-memory stage; one elected thread issues two K = 16 tcgen05 MMAs per
// stage into a TMEM accumulator of Cout FP32 columns.  Warp roles (192
// threads): warp 0 produces (TMA), warp 1 issues the MMAs and owns the TMEM
// allocation, warps 2-5 drain the accumulator (tcgen05.ld, 32 lanes each)
// through the epilogue.
//
// Weight gradient as an implicit GEMM with the pixel axis as K:
// dW[tap][co][ci] = sum_p x[p + off(tap), ci] * dy[p, co].  Both operands
// are read in their natural NHWC layout, which for this product is
// MN-major (channels contiguous, pixels along K); a CTA covers 128
// accumulator rows (one tap and 128 input channels, or several taps of a
// narrower input) and a contiguous range of pixel tiles and writes an FP32
// partial that a second kernel sums over the ranges in a fixed order.
#include <cuda.h>
#include <cuda_bf16.h>

#include "common.cuh"
#include "tc.cuh"

namespace opyx {
namespace net {

using bf16 = __nv_bfloat16;
constexpr int kTileM = 128;      // pixels per tile
constexpr int kChunk = 32;       // channels per stage (64-byte rows)
constexpr int kConvStages = 4;
constexpr int kConvThreads = 192;

struct ConvArgs {
  int32_t B, H, W, Wt, Ht;       // Wt x Ht pixels per tile (Wt * Ht = 128)
  int32_t cin, in_off, kchunks;  // input channels read, first channel, cin / 32
  int32_t cout, out_stride, out_off;
  int32_t epilogue, accumulate;
  const float* bias;
  void* y;
  void* z;
  unsigned* fault;
};

OPYX_D float gelu(float z) {
  // tanh form of GELU: 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3)))
  const float u = 0.7978845608028654f * (z + 0.044715f * z * z * z);
  return 0.5f * z * (1.f + tanhf(u));
}

OPYX_D float gelu_grad(float z) {
  const float z2 = z * z;
  const float u = 0.7978845608028654f * (z + 0.044715f * z2 * z);
  const float t = tanhf(u);
  const float du = 0.7978845608028654f * (1.f + 3.f * 0.044715f * z2);
  return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * du;
}

OPYX_D void flag_fault(unsigned* f) {
  if (f) atomicExch(f, 1u);
}

// Pixel tile t of a level: image n, first row y0, first column x0.
OPYX_D void tile_origin(const ConvArgs& p, int t, int* n, int* y0, int* x0) {
  const int per_row = p.W / p.Wt;
  const int per_img = (p.H / p.Ht) * per_row;
  *n = t / per_img;
  const int r = t % per_img;
  *y0 = (r / per_row) * p.Ht;
  *x0 = (r % per_row) * p.Wt;
}

template <int N>
struct ConvSmem {
  static constexpr int A = kTileM * kChunk * 2;   // 8 KB
  static constexpr int Bb = N * kChunk * 2;       // N x 64 bytes
  static constexpr int STAGE = A + Bb;            // multiple of 1024
  static constexpr int bytes = kConvStages * STAGE + 1024;   // + alignment slack
  static constexpr int cols = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
};

template <int N>
__global__ void __launch_bounds__(kConvThreads, 1)
k_conv3x3(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap wmap,
          const ConvArgs p) {
  using S = ConvSmem<N>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[kConvStages], empty[kConvStages], accf;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int n, y0, x0;
  tile_origin(p, blockIdx.x, &n, &y0, &x0);
  const int co0 = blockIdx.y * N;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kConvStages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(&accf, 1);
    tc::mbar_fence_init();
    tc::prefetch_map(&xmap);
    tc::prefetch_map(&wmap);
  }
  if (warp == 1) {
    tc::tmem_alloc(&tmem_base, S::cols);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const int KS = 9 * p.kchunks;
  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int ks = 0; ks < KS; ++ks) {
        const int s = ks % kConvStages;
        if (ks >= kConvStages && !tc::mbar_wait(&empty[s], ((ks / kConvStages) - 1) & 1)) {
          flag_fault(p.fault);
          break;
        }
        const int tap = ks / p.kchunks, ch = ks % p.kchunks;
        uint8_t* st = sm + s * S::STAGE;
        tc::mbar_expect_tx(&full[s], S::STAGE);
        tc::tma_load_4d(st, &xmap, p.in_off + ch * kChunk, x0 + tap % 3 - 1, y0 + tap / 3 - 1, n,
                        &full[s]);
        tc::tma_load_3d(st + S::A, &wmap, ch * kChunk, co0, tap, &full[s]);
        issued = ks + 1;
      }
      // copies still in flight land before the CTA leaves (bounded)
      for (int ks = issued - kConvStages > 0 ? issued - kConvStages : 0; ks < issued; ++ks)
        tc::mbar_wait(&full[ks % kConvStages], (ks / kConvStages) & 1);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t id = tc::idesc_bf16(kTileM, N);
      bool ok = true;
      for (int ks = 0; ks < KS && ok; ++ks) {
        const int s = ks % kConvStages;
        if (!tc::mbar_wait(&full[s], (ks / kConvStages) & 1)) {
          flag_fault(p.fault);
          ok = false;
          break;
        }
        tc::fence_after_sync();
        const uint8_t* st = sm + s * S::STAGE;
        const uint64_t ad = tc::sdesc_sw64(st, 16, 512);
        const uint64_t bd = tc::sdesc_sw64(st + S::A, 16, 512);
#pragma unroll
        for (int k = 0; k < 2; ++k)   // K = 16 slices: +32 bytes inside the 64-byte rows
          tc::mma_bf16(tmem, ad + 2 * k, bd + 2 * k, id, ks > 0 || k > 0);
        tc::mma_commit(&empty[s]);
      }
      tc::mma_commit(&accf);
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32 * (w % 4) .. + 31 = tile rows
    const int q = warp & 3;
    const int row = q * 32 + lane;
    const bool ok = tc::mbar_wait(&accf, 0);
    if (!ok) flag_fault(p.fault);
    tc::fence_after_sync();
    const int64_t pix = (((int64_t)n * p.H + y0 + row / p.Wt) * p.W) + x0 + row % p.Wt;
#pragma unroll 1
    for (int c = 0; c < N; c += 16) {
      uint32_t r[16];
      tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c, r);
      tc::tmem_wait_ld();
      if (!ok) continue;
      float v[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]) + (p.bias ? p.bias[co0 + c + j] : 0.f);
      const int64_t o = pix * p.out_stride + p.out_off + co0 + c;
      if (p.epilogue == OPYX_CONV_F32) {
        float* y = (float*)p.y + o;
        if (p.accumulate) {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] += y[j];
        }
#pragma unroll
        for (int j = 0; j < 16; j += 4) *(float4*)(y + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
      } else {
        __align__(16) bf16 a[16];
        if (p.epilogue == OPYX_CONV_GELU) {
          if (p.z) {
            __align__(16) bf16 zz[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) zz[j] = __float2bfloat16(v[j]);
            bf16* zp = (bf16*)p.z + pix * p.cout + co0 + c;
            *(uint4*)zp = *(const uint4*)zz;
            *(uint4*)(zp + 8) = *(const uint4*)(zz + 8);
          }
#pragma unroll
          for (int j = 0; j < 16; ++j) a[j] = __float2bfloat16(gelu(v[j]));
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) a[j] = __float2bfloat16(v[j]);
        }
        bf16* y = (bf16*)p.y + o;
        *(uint4*)y = *(const uint4*)a;
        *(uint4*)(y + 8) = *(const uint4*)(a + 8);
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, S::cols);
  }
}

// ------------------------------------------------------------ weight grad
// The 128 rows of a CTA's accumulator are four 32-channel blocks of the
// input; with fewer than 128 input channels each block takes another tap
// (taps_per_group = 128 / cin: 4 taps at 32 channels, 2 at 64), so no MMA
// row is wasted on channels that do not exist.  Stages by accumulator width:
// as many as fit in 200 KB of shared memory (5, 4, 3 for N = 32, 64, 128).
template <int N>
struct WgSmem {
  static constexpr int BLK = kTileM * kChunk * 2;      // 128 pixels x 32 channels: 8 KB
  static constexpr int A = 4 * BLK;                    // 4 blocks of 32 input channels
  static constexpr int Bb = (N / kChunk) * BLK;        // N output channels
  static constexpr int STAGE = A + Bb;
  static constexpr int stages = N == 32 ? 5 : N == 64 ? 4 : 3;
  static constexpr int bytes = stages * STAGE + 1024;
  static constexpr int cols = N <= 32 ? 32 : N <= 64 ? 64 : 128;
};

struct WgArgs {
  int32_t B, H, W, Wt, Ht;
  int32_t cin, in_off, cout;
  int32_t tpg, ngroups;           // taps per group, tap groups
  int32_t tiles, tiles_per_cta;   // pixel tiles in total / per CTA
  float* ws;                      // [split][9][cin][cout]
  unsigned* fault;
};

// Tap and first input channel of accumulator block b (0..3) for tap group
// `grp` and channel tile mt; false if the block holds nothing.
OPYX_D bool wg_block(const WgArgs& p, int grp, int mt, int b, int* tap, int* c0) {
  if (p.tpg > 1) {
    const int per = p.cin / kChunk;            // blocks per tap
    *tap = grp * p.tpg + b / per;
    *c0 = (b % per) * kChunk;
    return *tap < 9;
  }
  *tap = grp;
  *c0 = (mt * 4 + b) * kChunk;
  return *c0 < p.cin;
}

template <int N>
__global__ void __launch_bounds__(kConvThreads, 1)
k_conv3x3_wgrad(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap dmap,
                const WgArgs p) {
  using S = WgSmem<N>;
  constexpr int NS = S::stages;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[NS], empty[NS], accf;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int grp = blockIdx.x % p.ngroups, split = blockIdx.x / p.ngroups, mt = blockIdx.y;
  const int t0 = split * p.tiles_per_cta;
  const int t1 = t0 + p.tiles_per_cta < p.tiles ? t0 + p.tiles_per_cta : p.tiles;
  int nblk = 0;
  for (int b = 0; b < 4; ++b) {
    int tp, c0;
    nblk += wg_block(p, grp, mt, b, &tp, &c0) ? 1 : 0;
  }
  const unsigned stage_bytes = (unsigned)((nblk + N / kChunk) * S::BLK);
  ConvArgs g{};
  g.B = p.B; g.H = p.H; g.W = p.W; g.Wt = p.Wt; g.Ht = p.Ht;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(&accf, 1);
    tc::mbar_fence_init();
    tc::prefetch_map(&xmap);
    tc::prefetch_map(&dmap);
  }
  if (warp == 1) {
    tc::tmem_alloc(&tmem_base, S::cols);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const int KS = t1 > t0 ? t1 - t0 : 0;
  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int ks = 0; ks < KS; ++ks) {
        const int s = ks % NS;
        if (ks >= NS && !tc::mbar_wait(&empty[s], ((ks / NS) - 1) & 1)) {
          flag_fault(p.fault);
          break;
        }
        int n, y0, x0;
        tile_origin(g, t0 + ks, &n, &y0, &x0);
        uint8_t* st = sm + s * S::STAGE;
        tc::mbar_expect_tx(&full[s], stage_bytes);
        for (int b = 0; b < 4; ++b) {
          int tp, c0;
          if (wg_block(p, grp, mt, b, &tp, &c0))
            tc::tma_load_4d(st + b * S::BLK, &xmap, p.in_off + c0, x0 + tp % 3 - 1, y0 + tp / 3 - 1,
                            n, &full[s]);
        }
        for (int b = 0; b < N / kChunk; ++b)
          tc::tma_load_4d(st + S::A + b * S::BLK, &dmap, b * kChunk, x0, y0, n, &full[s]);
        issued = ks + 1;
      }
      for (int ks = issued - NS > 0 ? issued - NS : 0; ks < issued; ++ks)
        tc::mbar_wait(&full[ks % NS], (ks / NS) & 1);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t id = tc::idesc_bf16(kTileM, N, 1, 1);
      for (int ks = 0; ks < KS; ++ks) {
        const int s = ks % NS;
        if (!tc::mbar_wait(&full[s], (ks / NS) & 1)) {
          flag_fault(p.fault);
          break;
        }
        tc::fence_after_sync();
        const uint8_t* st = sm + s * S::STAGE;
#pragma unroll
        for (int k = 0; k < kTileM / 16; ++k) {   // 16 pixel rows = two 512-byte groups
          const uint64_t ad = tc::sdesc_sw64(st + k * 1024, S::BLK, 512);
          const uint64_t bd = tc::sdesc_sw64(st + S::A + k * 1024, S::BLK, 512);
          tc::mma_bf16(tmem, ad, bd, id, ks > 0 || k > 0);
        }
        tc::mma_commit(&empty[s]);
      }
      tc::mma_commit(&accf);
    }
  } else {
    const int q = warp & 3;                 // accumulator rows 32 q .. 32 q + 31 = block q
    const bool ok = tc::mbar_wait(&accf, 0);
    if (!ok) flag_fault(p.fault);
    tc::fence_after_sync();
    int tp = 0, c0 = 0;
    const bool live = wg_block(p, grp, mt, q, &tp, &c0);
    float* out = p.ws + ((((int64_t)split * 9 + tp) * p.cin) + c0 + lane) * p.cout;
#pragma unroll 1
    for (int c = 0; c < N; c += 16) {
      uint32_t r[16];
      tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c, r);
      tc::tmem_wait_ld();
      if (!live) continue;
      float v[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = (ok && KS > 0) ? __uint_as_float(r[j]) : 0.f;
#pragma unroll
      for (int j = 0; j < 16; j += 4)
        *(float4*)(out + c + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, S::cols);
  }
}

// dw[tap][co][ci] = sum over splits of ws[split][tap][ci][co] (fixed order).
__global__ void k_wgrad_reduce(const float* __restrict__ ws, int splits, int cin, int cout,
                               float* __restrict__ dw, int accumulate) {
  const int64_t total = (int64_t)9 * cout * cin;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int ci = (int)(i % cin);
    const int co = (int)((i / cin) % cout);
    const int tap = (int)(i / ((int64_t)cin * cout));
    const int64_t off = ((int64_t)tap * cin + ci) * cout + co;
    float sum = 0.f;
    for (int k = 0; k < splits; ++k) sum += ws[k * total + off];
    dw[i] = accumulate ? dw[i] + sum : sum;
  }
}

// ------------------------------------------------------------ elementwise
// dz = da * gelu'(z) (bf16), per-block column sums of dz for the bias grad.
__global__ void k_gelu_bwd(int64_t npix, int C, const float* __restrict__ da, int da_stride,
                           int da_off, const bf16* __restrict__ z, bf16* __restrict__ dz,
                           float* __restrict__ colpart) {
  extern __shared__ float red[];   // blockDim.x floats
  const int c = threadIdx.x % C;
  const int lanes = blockDim.x / C * C;   // threads in use (a multiple of C)
  float acc = 0.f;
  if ((int)threadIdx.x < lanes) {
    const int pr = threadIdx.x / C, ppb = blockDim.x / C;
    for (int64_t p = (int64_t)blockIdx.x * ppb + pr; p < npix; p += (int64_t)gridDim.x * ppb) {
      const float g = da[p * da_stride + da_off + c] * gelu_grad(__bfloat162float(z[p * C + c]));
      const bf16 gb = __float2bfloat16(g);
      dz[p * C + c] = gb;
      acc += __bfloat162float(gb);
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  if ((int)threadIdx.x < C) {
    float s = 0.f;
    for (int t = threadIdx.x; t < lanes; t += C) s += red[t];
    colpart[(int64_t)blockIdx.x * C + threadIdx.x] = s;
  }
}

// ---- vectorised versions (8 bf16 or 4 fp32 channels per thread; channel
// counts, strides and offsets multiples of 8, 16-byte aligned pointers)
struct alignas(16) bf8 { bf16 v[8]; };

__global__ void k_gelu_bwd8(int64_t npix, int C, const float* __restrict__ da, int da_stride,
                            int da_off, const bf16* __restrict__ z, bf16* __restrict__ dz,
                            float* __restrict__ colpart) {
  extern __shared__ float red8[];   // blockDim.x * 8 floats
  const int G = C / 8, ppb = (int)blockDim.x / G;
  const int g = threadIdx.x % G, pl = threadIdx.x / G;
  float acc[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j] = 0.f;
  if (pl < ppb) {
    for (int64_t p = (int64_t)blockIdx.x * ppb + pl; p < npix; p += (int64_t)gridDim.x * ppb) {
      const float4* ap = reinterpret_cast<const float4*>(da + p * da_stride + da_off + 8 * g);
      const float4 a0 = ap[0], a1 = ap[1];
      const bf8 zz = *reinterpret_cast<const bf8*>(z + p * C + 8 * g);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      bf8 out;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        out.v[j] = __float2bfloat16(av[j] * gelu_grad(__bfloat162float(zz.v[j])));
        acc[j] += __bfloat162float(out.v[j]);
      }
      *reinterpret_cast<bf8*>(dz + p * C + 8 * g) = out;
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) red8[threadIdx.x * 8 + j] = acc[j];
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    float sum = 0.f;
    for (int q = 0; q < ppb; ++q) sum += red8[(q * G + c / 8) * 8 + (c & 7)];
    colpart[(int64_t)blockIdx.x * C + c] = sum;
  }
}

// Column sums of per-block partials: one CTA per column, a fixed order.
__global__ void k_colsum_par(const float* __restrict__ part, int nblk, int C, float* __restrict__ out,
                             int accumulate) {
  const int c = blockIdx.x;
  float sum = 0.f;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) sum += part[(int64_t)b * C + c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
  __shared__ float wsum[32];
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[w];
    out[c] = accumulate ? out[c] + t : t;
  }
}

__global__ void k_pool2_8(int B, int H, int W, int C, const bf16* __restrict__ x, int xs, int xo,
                          bf16* __restrict__ y) {
  const int h = H / 2, w = W / 2, G = C / 8;
  const int64_t total = (int64_t)B * h * w * G;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int g = (int)(i % G);
    const int64_t pp = i / G;
    const int xx = (int)(pp % w), yy = (int)((pp / w) % h);
    const int64_t n = pp / ((int64_t)w * h);
    const int64_t b0 = (n * H + 2 * yy) * W + 2 * xx;
    const bf8 v0 = *reinterpret_cast<const bf8*>(x + b0 * xs + xo + 8 * g);
    const bf8 v1 = *reinterpret_cast<const bf8*>(x + (b0 + 1) * xs + xo + 8 * g);
    const bf8 v2 = *reinterpret_cast<const bf8*>(x + (b0 + W) * xs + xo + 8 * g);
    const bf8 v3 = *reinterpret_cast<const bf8*>(x + (b0 + W + 1) * xs + xo + 8 * g);
    bf8 out;
#pragma unroll
    for (int j = 0; j < 8; ++j)
      out.v[j] = __float2bfloat16(0.25f * (__bfloat162float(v0.v[j]) + __bfloat162float(v1.v[j]) +
                                           __bfloat162float(v2.v[j]) + __bfloat162float(v3.v[j])));
    *reinterpret_cast<bf8*>(y + pp * C + 8 * g) = out;
  }
}

__global__ void k_pool2_bwd4(int B, int H, int W, int C, const float* __restrict__ dy,
                             float* __restrict__ dx, int dxs, int dxo, int accumulate) {
  const int h = H / 2, w = W / 2, G = C / 4;
  const int64_t total = (int64_t)B * H * W * G;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int g = (int)(i % G);
    const int64_t pp = i / G;
    const int xx = (int)(pp % W), yy = (int)((pp / W) % H);
    const int64_t n = pp / ((int64_t)W * H);
    float4 v = *reinterpret_cast<const float4*>(dy + ((n * h + yy / 2) * w + xx / 2) * C + 4 * g);
    v.x *= 0.25f; v.y *= 0.25f; v.z *= 0.25f; v.w *= 0.25f;
    float4* d = reinterpret_cast<float4*>(dx + pp * dxs + dxo + 4 * g);
    if (accumulate) {
      const float4 o = *d;
      v.x += o.x; v.y += o.y; v.z += o.z; v.w += o.w;
    }
    *d = v;
  }
}

__global__ void k_up2_8(int B, int h, int w, int C, const bf16* __restrict__ x, bf16* __restrict__ y,
                        int ys, int yo) {
  const int H = 2 * h, W = 2 * w, G = C / 8;
  const int64_t total = (int64_t)B * H * W * G;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int g = (int)(i % G);
    const int64_t pp = i / G;
    const int xx = (int)(pp % W), yy = (int)((pp / W) % H);
    const int64_t n = pp / ((int64_t)W * H);
    *reinterpret_cast<bf8*>(y + pp * ys + yo + 8 * g) =
        *reinterpret_cast<const bf8*>(x + ((n * h + yy / 2) * w + xx / 2) * C + 8 * g);
  }
}

__global__ void k_up2_bwd4(int B, int h, int w, int C, const float* __restrict__ dy, int dys, int dyo,
                           float* __restrict__ dx) {
  const int H = 2 * h, W = 2 * w, G = C / 4;
  const int64_t total = (int64_t)B * h * w * G;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int g = (int)(i % G);
    const int64_t pp = i / G;
    const int xx = (int)(pp % w), yy = (int)((pp / w) % h);
    const int64_t n = pp / ((int64_t)w * h);
    const int64_t b0 = (n * H + 2 * yy) * W + 2 * xx;
    const float4 a = *reinterpret_cast<const float4*>(dy + b0 * dys + dyo + 4 * g);
    const float4 b = *reinterpret_cast<const float4*>(dy + (b0 + 1) * dys + dyo + 4 * g);
    const float4 c = *reinterpret_cast<const float4*>(dy + (b0 + W) * dys + dyo + 4 * g);
    const float4 d = *reinterpret_cast<const float4*>(dy + (b0 + W + 1) * dys + dyo + 4 * g);
    *reinterpret_cast<float4*>(dx + pp * C + 4 * g) =
        make_float4(a.x + b.x + c.x + d.x, a.y + b.y + c.y + d.y, a.z + b.z + c.z + d.z,
                    a.w + b.w + c.w + d.w);
  }
}

// Head parameter grads from the per-block partials, summed in block order.
__global__ void k_head_fold(const float* __restrict__ part, int nblk, int np, float* __restrict__ dw,
                            float* __restrict__ db) {
  const int i = threadIdx.x;
  if (i >= np) return;
  float s = 0.f;
  for (int b = 0; b < nblk; ++b) s += part[(int64_t)b * np + i];
  if (i < np - 3) dw[i] = s;
  else db[i - (np - 3)] = s;
}

// 2x2 average pooling of a channel slice (bf16 -> bf16, dense output).
__global__ void k_pool2(int B, int H, int W, int C, const bf16* __restrict__ x, int xs, int xo,
                        bf16* __restrict__ y) {
  const int h = H / 2, w = W / 2;
  const int64_t total = (int64_t)B * h * w * C;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const int64_t pp = i / C;
    const int xx = (int)(pp % w), yy = (int)((pp / w) % h);
    const int64_t n = pp / ((int64_t)w * h);
    const int64_t b0 = ((n * H + 2 * yy) * W + 2 * xx);
    const float s = __bfloat162float(x[b0 * xs + xo + c]) + __bfloat162float(x[(b0 + 1) * xs + xo + c]) +
                    __bfloat162float(x[(b0 + W) * xs + xo + c]) +
                    __bfloat162float(x[(b0 + W + 1) * xs + xo + c]);
    y[i] = __float2bfloat16(0.25f * s);
  }
}

// dx[slice] (+)= dy / 4 spread over each 2x2 block (fp32).
__global__ void k_pool2_bwd(int B, int H, int W, int C, const float* __restrict__ dy,
                            float* __restrict__ dx, int dxs, int dxo, int accumulate) {
  const int64_t total = (int64_t)B * H * W * C;
  const int h = H / 2, w = W / 2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const int64_t pp = i / C;
    const int xx = (int)(pp % W), yy = (int)((pp / W) % H);
    const int64_t n = pp / ((int64_t)W * H);
    const float g = 0.25f * dy[((n * h + yy / 2) * w + xx / 2) * C + c];
    float* d = dx + pp * dxs + dxo + c;
    *d = accumulate ? *d + g : g;
  }
}

// Nearest 2x upsampling of a dense bf16 tensor into a channel slice.
__global__ void k_up2(int B, int h, int w, int C, const bf16* __restrict__ x, bf16* __restrict__ y,
                      int ys, int yo) {
  const int H = 2 * h, W = 2 * w;
  const int64_t total = (int64_t)B * H * W * C;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const int64_t pp = i / C;
    const int xx = (int)(pp % W), yy = (int)((pp / W) % H);
    const int64_t n = pp / ((int64_t)W * H);
    y[pp * ys + yo + c] = x[((n * h + yy / 2) * w + xx / 2) * C + c];
  }
}

// dx = sum of the 2x2 block of a channel slice of dy (fp32, dense dx).
__global__ void k_up2_bwd(int B, int h, int w, int C, const float* __restrict__ dy, int dys, int dyo,
                          float* __restrict__ dx) {
  const int H = 2 * h, W = 2 * w;
  const int64_t total = (int64_t)B * h * w * C;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const int64_t pp = i / C;
    const int xx = (int)(pp % w), yy = (int)((pp / w) % h);
    const int64_t n = pp / ((int64_t)w * h);
    const int64_t b0 = (n * H + 2 * yy) * W + 2 * xx;
    dx[i] = dy[b0 * dys + dyo + c] + dy[(b0 + 1) * dys + dyo + c] + dy[(b0 + W) * dys + dyo + c] +
            dy[(b0 + W + 1) * dys + dyo + c];
  }
}

// Network input: channel 0 = f, channel 1 = lambda of the pixel's image,
// channels 2..31 = 0 (bf16, 32 channels).
__global__ void k_pack_input(int B, int64_t hw, const float* __restrict__ f,
                             const float* __restrict__ lam, float lam_scale, bf16* __restrict__ x) {
  const int64_t total = (int64_t)B * hw * 32;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i & 31);
    const int64_t pp = i >> 5;
    float v = 0.f;
    if (c == 0) v = f[pp];
    else if (c == 1) v = lam[pp / hw] * lam_scale;
    x[i] = __float2bfloat16(v);
  }
}

// Network input of the restart mode: f, lambda * lam_scale, the current
// iterate as x - f and y / lambda (2 channels), zeros up to 32.
__global__ void k_pack_input_state(int B, int64_t hw, const float* __restrict__ f,
                                   const float* __restrict__ lam, float lam_scale,
                                   const float* __restrict__ xb, const float* __restrict__ yb,
                                   bf16* __restrict__ x) {
  const int64_t total = (int64_t)B * hw * 32;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i & 31);
    const int64_t pp = i >> 5;
    const float l = lam[pp / hw];
    float v = 0.f;
    if (c == 0) v = f[pp];
    else if (c == 1) v = l * lam_scale;
    else if (c == 2) v = xb[pp] - f[pp];
    else if (c == 3) v = yb[2 * pp] / l;
    else if (c == 4) v = yb[2 * pp + 1] / l;
    x[i] = __float2bfloat16(v);
  }
}

// Head: 1x1 convolution of the last 32-channel activation to K outputs (fp32).
template <int K>
__global__ void k_head(int64_t npix, const bf16* __restrict__ a, const float* __restrict__ w,
                       const float* __restrict__ b, float* __restrict__ out) {
  __shared__ float sw[K * 32 + K];
  for (int i = threadIdx.x; i < K * 32; i += blockDim.x) sw[i] = w[i];
  if (threadIdx.x < K) sw[K * 32 + threadIdx.x] = b[threadIdx.x];
  __syncthreads();
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npix;
       p += (int64_t)gridDim.x * blockDim.x) {
    float v[32];
    const uint4* ap = (const uint4*)(a + p * 32);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint4 u = ap[j];
      const bf16* e = (const bf16*)&u;
#pragma unroll
      for (int t = 0; t < 8; ++t) v[8 * j + t] = __bfloat162float(e[t]);
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      float s = sw[K * 32 + k];
#pragma unroll
      for (int c = 0; c < 32; ++c) s += sw[k * 32 + c] * v[c];
      out[p * K + k] = s;
    }
  }
}

// Head backward: da[p, c] = sum_k dout[p, k] w[k, c]; per-block partials of
// dW[k, c] = sum_p dout[p, k] a[p, c] and db[k] = sum_p dout[p, k].
template <int K>
__global__ void k_head_bwd(int64_t npix, const bf16* __restrict__ a, const float* __restrict__ w,
                           const float* __restrict__ dout, float* __restrict__ da,
                           float* __restrict__ part) {
  constexpr int NP = K * 32 + K;
  __shared__ float sw[K * 32];
  __shared__ float red[NP];
  for (int i = threadIdx.x; i < K * 32; i += blockDim.x) sw[i] = w[i];
  for (int i = threadIdx.x; i < NP; i += blockDim.x) red[i] = 0.f;
  __syncthreads();
  float gw[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) gw[i] = 0.f;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npix;
       p += (int64_t)gridDim.x * blockDim.x) {
    float v[32], g[K];
    const uint4* ap = (const uint4*)(a + p * 32);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint4 u = ap[j];
      const bf16* e = (const bf16*)&u;
#pragma unroll
      for (int t = 0; t < 8; ++t) v[8 * j + t] = __bfloat162float(e[t]);
    }
#pragma unroll
    for (int k = 0; k < K; ++k) g[k] = dout[p * K + k];
#pragma unroll
    for (int c = 0; c < 32; ++c) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        s += g[k] * sw[k * 32 + c];
        gw[k * 32 + c] += g[k] * v[c];
      }
      da[p * 32 + c] = s;
    }
#pragma unroll
    for (int k = 0; k < K; ++k) gw[K * 32 + k] += g[k];
  }
  // block reduction in a fixed order: warp shuffles, then warps in order
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    float s = gw[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    gw[i] = s;
  }
  __shared__ float wred[8][NP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int i = 0; i < NP; ++i) wred[warp][i] = gw[i];
  __syncthreads();
  for (int i = threadIdx.x; i < NP; i += blockDim.x) {
    float s = 0.f;
    for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2) s += wred[w2][i];
    part[(int64_t)blockIdx.x * NP + i] = s;
  }
}

// Weighted squared error of the head output against the targets:
// loss partial per block (FP64), grad = 2 wgt (pred - target) / count.
__global__ void k_mse(int64_t n, int K, const float* __restrict__ pred, const float* __restrict__ tgt,
                      const float* __restrict__ wk, double inv_count, float* __restrict__ grad,
                      double* __restrict__ part) {
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float wt = wk[i % K];
    const float d = pred[i] - tgt[i];
    acc += (double)(wt * d * d);
    grad[i] = (float)(2.0 * inv_count) * wt * d;
  }
  acc = warp_reduce(RED_SUM, acc);
  __shared__ double wr[32];
  if ((threadIdx.x & 31) == 0) wr[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2) s += wr[w2];
    part[blockIdx.x] = s * inv_count;
  }
}

// Warm-start loss.  Head outputs per pixel: o0 = x - f, (o1, o2) = y / lambda
// (components along rows and columns).  With e = o[1:3] - t[1:3] and the
// divergence d = div(e) adjoint to the forward gradient (div v =
// sum_t v_t[i] [c_t < n_t - 1] - v_t[i - s_t] [c_t > 0]), the loss is
//   (1/n) sum_i  w_x (o0 - t0)^2 + w_div (lambda d)^2 + w_u |e|^2 :
// the dual enters through lambda div(y / lambda) = div y, which is what the
// duality gap sees (at the optimum x - f = div y), while y itself is only
// determined up to divergence-free fields where x is flat.
// A fourth term weights the low frequencies, where PDHG converges slowly:
// with R = 8x8 block means of the primal error and of lambda d,
//   w_p (4096 / n) sum_blocks (Rx^2 + Rd^2)
// (white-noise errors weigh as in the pixel terms, smooth ones 64 times more).
OPYX_D float warm_div(int H, int W, const float* out, const float* tgt, int64_t i, int x, int y) {
  float d = 0.f;
  if (y < H - 1) d += out[3 * i + 1] - tgt[3 * i + 1];
  if (y > 0) d -= out[3 * (i - W) + 1] - tgt[3 * (i - W) + 1];
  if (x < W - 1) d += out[3 * i + 2] - tgt[3 * i + 2];
  if (x > 0) d -= out[3 * (i - 1) + 2] - tgt[3 * (i - 1) + 2];
  return d;
}

__global__ void k_warm_pool(int B, int H, int W, const float* __restrict__ out,
                            const float* __restrict__ tgt, const float* __restrict__ lam,
                            float* __restrict__ pooled) {
  const int hb = H / 8, wb = W / 8;
  const int64_t total = (int64_t)B * hb * wb;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int bx = (int)(k % wb), by = (int)((k / wb) % hb);
    const int64_t n = k / ((int64_t)hb * wb);
    const float l = lam[n];
    float rx = 0.f, rd = 0.f;
    for (int yy = 8 * by; yy < 8 * by + 8; ++yy)
      for (int xx = 8 * bx; xx < 8 * bx + 8; ++xx) {
        const int64_t i = (n * H + yy) * W + xx;
        rx += out[3 * i] - tgt[3 * i];
        rd += l * warm_div(H, W, out, tgt, i, xx, yy);
      }
    pooled[2 * k] = rx * (1.f / 64.f);
    pooled[2 * k + 1] = rd * (1.f / 64.f);
  }
}

// Pass 1: c = 2 w_div lambda^2 d / n (+ the pooled term's share) into `scr`,
// loss partials per block.
__global__ void k_warm_loss1(int B, int H, int W, const float* __restrict__ out,
                             const float* __restrict__ tgt, const float* __restrict__ lam, float w_x,
                             float w_div, float w_u, float w_p, double inv_n,
                             const float* __restrict__ pooled, float* __restrict__ scr,
                             double* __restrict__ part) {
  const int64_t total = (int64_t)B * H * W;
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % W), y = (int)((i / W) % H);
    const float l = lam[i / ((int64_t)H * W)];
    const float r0 = out[3 * i] - tgt[3 * i];
    const float e0 = out[3 * i + 1] - tgt[3 * i + 1], e1 = out[3 * i + 2] - tgt[3 * i + 2];
    const float d = warm_div(H, W, out, tgt, i, x, y);
    const float ld = l * d;
    acc += (double)(w_x * r0 * r0 + w_div * ld * ld + w_u * (e0 * e0 + e1 * e1));
    float c = (float)(2.0 * inv_n) * w_div * l * ld;
    if (w_p != 0.f) {
      const int64_t k = ((i / ((int64_t)H * W)) * (H / 8) + y / 8) * (W / 8) + x / 8;
      const float rd = pooled[2 * k + 1];
      c += (float)(128.0 * inv_n) * w_p * l * rd;
      if ((x & 7) == 0 && (y & 7) == 0) {
        const float rx = pooled[2 * k];
        acc += (double)(4096.f * w_p * (rx * rx + rd * rd));
      }
    }
    scr[i] = c;
  }
  acc = warp_reduce(RED_SUM, acc);
  __shared__ double wr[32];
  if ((threadIdx.x & 31) == 0) wr[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2) s += wr[w2];
    part[blockIdx.x] = s * inv_n;
  }
}

// Pass 2: grad o0 = 2 w_x r0 / n; grad e_t = 2 w_u e_t / n + (div^T c)_t,
// where div^T c = c[i] - c[i + s_t] if i + s_t is inside the image, else 0
// (minus the forward gradient of c): the adjoint of the sum above.
__global__ void k_warm_loss2(int B, int H, int W, const float* __restrict__ out,
                             const float* __restrict__ tgt, float w_x, float w_u, float w_p,
                             double inv_n, const float* __restrict__ pooled,
                             const float* __restrict__ scr, float* __restrict__ grad) {
  const int64_t total = (int64_t)B * H * W;
  const float s2 = (float)(2.0 * inv_n);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % W), y = (int)((i / W) % H);
    const float c = scr[i];
    // d_j depends on e0[i] with +1 (j = i, y < H-1) and -1 (j = i + W, y+1 > 0)
    float g0 = 0.f, g1 = 0.f;
    if (y < H - 1) g0 = c - scr[i + W];
    if (x < W - 1) g1 = c - scr[i + 1];
    float gx = s2 * w_x * (out[3 * i] - tgt[3 * i]);
    if (w_p != 0.f) {
      const int64_t k = ((i / ((int64_t)H * W)) * (H / 8) + y / 8) * (W / 8) + x / 8;
      gx += (float)(128.0 * inv_n) * w_p * pooled[2 * k];
    }
    grad[3 * i] = gx;
    grad[3 * i + 1] = s2 * w_u * (out[3 * i + 1] - tgt[3 * i + 1]) + g0;
    grad[3 * i + 2] = s2 * w_u * (out[3 * i + 2] - tgt[3 * i + 2]) + g1;
  }
}

// Proposal: x0 = f + o0, y0 = lambda * (o1, o2) / max(1, |(o1, o2)|).
__global__ void k_warm_unpack(int64_t npix, int64_t hw, const float* __restrict__ f,
                              const float* __restrict__ lam, const float* __restrict__ out,
                              float* __restrict__ x0, float* __restrict__ y0) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npix;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float l = lam[i / hw];
    x0[i] = f[i] + out[3 * i];
    const float u0 = out[3 * i + 1], u1 = out[3 * i + 2];
    const float n = sqrtf(u0 * u0 + u1 * u1);
    const float s = l / (n > 1.f ? n : 1.f);
    y0[2 * i] = s * u0;
    y0[2 * i + 1] = s * u1;
  }
}

// Correction of a PDHG iterate: x0 = xb + o0, y0 = lambda * proj(yb / lambda + o12)
// onto the unit ball (xb (n), yb (n, 2) the iterate the network saw).
__global__ void k_warm_unpack_rel(int64_t npix, int64_t hw, const float* __restrict__ xb,
                                  const float* __restrict__ yb, const float* __restrict__ lam,
                                  const float* __restrict__ out, float* __restrict__ x0,
                                  float* __restrict__ y0) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npix;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float l = lam[i / hw];
    x0[i] = xb[i] + out[3 * i];
    const float u0 = yb[2 * i] / l + out[3 * i + 1], u1 = yb[2 * i + 1] / l + out[3 * i + 2];
    const float n = sqrtf(u0 * u0 + u1 * u1);
    const float s = l / (n > 1.f ? n : 1.f);
    y0[2 * i] = s * u0;
    y0[2 * i + 1] = s * u1;
  }
}

// Adam (Kingma & Ba 2015) on FP32 master weights; optionally refreshes the
// bf16 copy used by the forward convolutions and the tap-flipped,
// in/out-transposed bf16 copy used by the input-gradient convolutions.
__global__ void k_adam(int64_t n, float* __restrict__ w, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2,
                       float eps, float c1, float c2, bf16* __restrict__ wb, bf16* __restrict__ wt,
                       int cin, int cout) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
    if (wt) {
      // w[tap][co][ci] -> wt[8 - tap][ci][co]
      const int ci = (int)(i % cin), co = (int)((i / cin) % cout), tap = (int)(i / ((int64_t)cin * cout));
      wt[((int64_t)(8 - tap) * cin + ci) * cout + co] = __float2bfloat16(wi);
    }
  }
}

__global__ void k_conv_weights(int64_t n, const float* __restrict__ w, bf16* __restrict__ wb,
                               bf16* __restrict__ wt, int cin, int cout) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float wi = w[i];
    if (wb) wb[i] = __float2bfloat16(wi);
    if (wt) {
      const int ci = (int)(i % cin), co = (int)((i / cin) % cout), tap = (int)(i / ((int64_t)cin * cout));
      wt[((int64_t)(8 - tap) * cin + ci) * cout + co] = __float2bfloat16(wi);
    }
  }
}

// ------------------------------------------------------------ host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

// NHWC bf16 activation map: dims {stride, W, H, B}, box {32, Wt, Ht, 1}.
static int act_map(CUtensorMap* m, const void* base, int B, int H, int W, int stride, int Wt, int Ht) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return OPYX_ERR_LAUNCH;
  const cuuint64_t dims[4] = {(cuuint64_t)stride, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
  const cuuint64_t strides[3] = {(cuuint64_t)stride * 2, (cuuint64_t)stride * 2 * W,
                                 (cuuint64_t)stride * 2 * W * H};
  const cuuint32_t box[4] = {(cuuint32_t)kChunk, (cuuint32_t)Wt, (cuuint32_t)Ht, 1};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box,
                   es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? OPYX_OK : OPYX_ERR_ARG;
}

// Weights [9][cout][cin] bf16: dims {cin, cout, 9}, box {32, N, 1}.
static int w_map(CUtensorMap* m, const void* base, int cin, int cout, int N) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return OPYX_ERR_LAUNCH;
  const cuuint64_t dims[3] = {(cuuint64_t)cin, (cuuint64_t)cout, 9};
  const cuuint64_t strides[2] = {(cuuint64_t)cin * 2, (cuuint64_t)cin * 2 * cout};
  const cuuint32_t box[3] = {(cuuint32_t)kChunk, (cuuint32_t)N, 1};
  const cuuint32_t es[3] = {1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box,
                   es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? OPYX_OK : OPYX_ERR_ARG;
}

static bool al16(const void* p) { return ((uintptr_t)p & 15) == 0; }

static int tile_shape(int H, int W, int* Wt, int* Ht) {
  const int wt = W < kTileM ? W : kTileM;
  if (wt <= 0 || kTileM % wt || W % wt) return OPYX_ERR_UNSUPPORTED;
  const int ht = kTileM / wt;
  if (H % ht) return OPYX_ERR_UNSUPPORTED;
  *Wt = wt;
  *Ht = ht;
  return OPYX_OK;
}

static int conv_check(const opyx_conv3x3_desc* d) {
  if (!d || !d->x || !d->w || !d->y) return OPYX_ERR_ARG;
  if (d->batch < 1 || d->height < 1 || d->width < 1) return OPYX_ERR_ARG;
  if (d->in_channels < kChunk || d->in_channels % kChunk || d->in_stride % 8 || d->in_offset % 8 ||
      d->in_offset < 0 || d->in_offset + d->in_channels > d->in_stride)
    return OPYX_ERR_ARG;
  if (d->out_stride % 8 || d->out_offset % 8 || d->out_offset < 0 ||
      d->out_offset + d->out_channels > d->out_stride)
    return OPYX_ERR_ARG;
  if (!al16(d->x) || !al16(d->w) || !al16(d->y) || (d->z && !al16(d->z))) return OPYX_ERR_ARG;
  if (d->epilogue < OPYX_CONV_GELU || d->epilogue > OPYX_CONV_BF16) return OPYX_ERR_ARG;
  return OPYX_OK;
}

template <int N>
static int launch_conv(const CUtensorMap& xm, const CUtensorMap& wm, const ConvArgs& a, int tiles,
                       int ntiles, cudaStream_t s) {
  const int smem = ConvSmem<N>::bytes;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_conv3x3<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
      return OPYX_ERR_LAUNCH;
    attr = true;
  }
  k_conv3x3<N><<<dim3(tiles, ntiles), kConvThreads, smem, s>>>(xm, wm, a);
  return check_launch();
}

template <int N>
static int launch_wgrad(const CUtensorMap& xm, const CUtensorMap& dm, const WgArgs& a, int ctas,
                        int mtiles, cudaStream_t s) {
  const int smem = WgSmem<N>::bytes;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_conv3x3_wgrad<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
        cudaSuccess)
      return OPYX_ERR_LAUNCH;
    attr = true;
  }
  k_conv3x3_wgrad<N><<<dim3(ctas, mtiles), kConvThreads, smem, s>>>(xm, dm, a);
  return check_launch();
}

// The network kernels' sticky fault flag: a static device word (no
// allocation), one per GPU that loads the library.
__device__ unsigned g_net_fault;

static unsigned* fault_word() {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_net_fault) != cudaSuccess) return nullptr;
  return (unsigned*)p;
}

// Pixel-tile ranges of the weight gradient: about two waves of CTAs.
static void wgrad_groups(int cin, int* tpg, int* ngroups, int* mtiles) {
  *tpg = (cin < kTileM && kTileM % cin == 0) ? kTileM / cin : 1;
  *ngroups = (9 + *tpg - 1) / *tpg;
  *mtiles = *tpg > 1 ? 1 : (cin + kTileM - 1) / kTileM;
}

static int wgrad_splits(int tiles, int cta_per_split) {
  int want = (2 * sm_count() + cta_per_split - 1) / cta_per_split;
  if (want < 1) want = 1;
  if (want > tiles) want = tiles;
  return want;
}

}  // namespace net
}  // namespace opyx

using namespace opyx;
using namespace opyx::net;

extern "C" {

int opyx_conv3x3(const opyx_conv3x3_desc* d, void* stream) {
  int st = conv_check(d);
  if (st) return st;
  const int N = d->out_channels;
  if (N != 32 && N != 64 && N != 128 && N != 256) return OPYX_ERR_UNSUPPORTED;
  if (d->epilogue == OPYX_CONV_GELU && d->z && d->out_channels % 16) return OPYX_ERR_ARG;
  int Wt, Ht;
  if ((st = tile_shape(d->height, d->width, &Wt, &Ht))) return st;
  CUtensorMap xm, wm;
  if ((st = act_map(&xm, d->x, d->batch, d->height, d->width, d->in_stride, Wt, Ht))) return st;
  if ((st = w_map(&wm, d->w, d->in_channels, d->out_channels, N))) return st;
  ConvArgs a{};
  a.B = d->batch; a.H = d->height; a.W = d->width; a.Wt = Wt; a.Ht = Ht;
  a.cin = d->in_channels; a.in_off = d->in_offset; a.kchunks = d->in_channels / kChunk;
  a.cout = d->out_channels; a.out_stride = d->out_stride; a.out_off = d->out_offset;
  a.epilogue = d->epilogue; a.accumulate = d->accumulate;
  a.bias = d->bias; a.y = d->y; a.z = d->z;
  a.fault = fault_word();
  const int64_t tiles = (int64_t)d->batch * d->height * d->width / kTileM;
  if (tiles > INT32_MAX) return OPYX_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  switch (N) {
    case 32: return launch_conv<32>(xm, wm, a, (int)tiles, 1, s);
    case 64: return launch_conv<64>(xm, wm, a, (int)tiles, 1, s);
    case 128: return launch_conv<128>(xm, wm, a, (int)tiles, 1, s);
    default: return launch_conv<256>(xm, wm, a, (int)tiles, 1, s);
  }
}

size_t opyx_conv3x3_wgrad_workspace(const opyx_conv3x3_desc* d) {
  if (conv_check(d)) return 0;
  const int64_t tiles = (int64_t)d->batch * d->height * d->width / kTileM;
  int tpg, ngroups, mtiles;
  wgrad_groups(d->in_channels, &tpg, &ngroups, &mtiles);
  const int splits = wgrad_splits((int)tiles, ngroups * mtiles);
  return (size_t)splits * 9 * d->in_channels * d->out_channels * sizeof(float);
}

int opyx_conv3x3_wgrad(const opyx_conv3x3_desc* d, const void* dy, float* dw, int accumulate,
                       void* ws, size_t ws_bytes, void* stream) {
  int st = conv_check(d);
  if (st) return st;
  if (!dy || !dw || !ws || !al16(dy) || !al16(ws)) return OPYX_ERR_ARG;
  const int N = d->out_channels;
  if (N != 32 && N != 64 && N != 128) return OPYX_ERR_UNSUPPORTED;
  int Wt, Ht;
  if ((st = tile_shape(d->height, d->width, &Wt, &Ht))) return st;
  const int64_t tiles = (int64_t)d->batch * d->height * d->width / kTileM;
  if (tiles > INT32_MAX) return OPYX_ERR_UNSUPPORTED;
  int tpg, ngroups, mtiles;
  wgrad_groups(d->in_channels, &tpg, &ngroups, &mtiles);
  const int splits = wgrad_splits((int)tiles, ngroups * mtiles);
  if (ws_bytes < opyx_conv3x3_wgrad_workspace(d)) return OPYX_ERR_WORKSPACE;
  CUtensorMap xm, dm;
  if ((st = act_map(&xm, d->x, d->batch, d->height, d->width, d->in_stride, Wt, Ht))) return st;
  if ((st = act_map(&dm, dy, d->batch, d->height, d->width, N, Wt, Ht))) return st;
  WgArgs a{};
  a.B = d->batch; a.H = d->height; a.W = d->width; a.Wt = Wt; a.Ht = Ht;
  a.cin = d->in_channels; a.in_off = d->in_offset; a.cout = N;
  a.tpg = tpg; a.ngroups = ngroups;
  a.tiles = (int)tiles;
  a.tiles_per_cta = (int)((tiles + splits - 1) / splits);
  a.ws = (float*)ws;
  a.fault = fault_word();
  cudaStream_t s = (cudaStream_t)stream;
  switch (N) {
    case 32: st = launch_wgrad<32>(xm, dm, a, ngroups * splits, mtiles, s); break;
    case 64: st = launch_wgrad<64>(xm, dm, a, ngroups * splits, mtiles, s); break;
    default: st = launch_wgrad<128>(xm, dm, a, ngroups * splits, mtiles, s); break;
  }
  if (st) return st;
  const int64_t total = (int64_t)9 * N * d->in_channels;
  k_wgrad_reduce<<<grid_for(total, 256), 256, 0, s>>>((const float*)ws, splits, d->in_channels, N, dw,
                                                      accumulate);
  return check_launch();
}

int opyx_net_fault(unsigned* out) {
  if (!out) return OPYX_ERR_ARG;
  unsigned* f = fault_word();
  if (!f) return OPYX_ERR_LAUNCH;
  if (cudaMemcpy(out, f, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return OPYX_ERR_LAUNCH;
  return OPYX_OK;
}

size_t opyx_gelu_bwd_workspace(int64_t npix, int C) {
  (void)npix;
  return (size_t)sm_count() * 4 * C * sizeof(float);
}

int opyx_gelu_bwd(int64_t npix, int C, const float* da, int da_stride, int da_off, const void* z,
                  void* dz, float* dbias, int accumulate, void* ws, size_t ws_bytes, void* stream) {
  if (npix < 0 || C < 1 || C > 256 || !da || !z || !dz || !dbias || !ws || da_stride < C ||
      da_off < 0 || da_off + C > da_stride)
    return OPYX_ERR_ARG;
  if (ws_bytes < opyx_gelu_bwd_workspace(npix, C)) return OPYX_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const int nblk = sm_count() * 4;
  if (C % 8 == 0 && 256 % (C / 8) == 0 && da_stride % 4 == 0 && da_off % 4 == 0 && al16(da) &&
      al16(z) && al16(dz)) {
    k_gelu_bwd8<<<nblk, 256, 256 * 8 * sizeof(float), s>>>(npix, C, da, da_stride, da_off,
                                                           (const bf16*)z, (bf16*)dz, (float*)ws);
  } else {
    const int threads = 256 / C * C;
    k_gelu_bwd<<<nblk, threads, threads * sizeof(float), s>>>(npix, C, da, da_stride, da_off,
                                                              (const bf16*)z, (bf16*)dz, (float*)ws);
  }
  OPYX_CHECK_LAUNCH();
  k_colsum_par<<<C, 256, 0, s>>>((const float*)ws, nblk, C, dbias, accumulate);
  return check_launch();
}

int opyx_pool2(int B, int H, int W, int C, const void* x, int xs, int xo, void* y, void* stream) {
  if (B < 1 || H < 2 || W < 2 || (H | W) & 1 || C < 1 || !x || !y || xo < 0 || xo + C > xs)
    return OPYX_ERR_ARG;
  const int64_t total = (int64_t)B * (H / 2) * (W / 2) * C;
  if (C % 8 == 0 && xs % 8 == 0 && xo % 8 == 0 && al16(x) && al16(y))
    k_pool2_8<<<grid_for(total / 8, 256), 256, 0, (cudaStream_t)stream>>>(B, H, W, C, (const bf16*)x,
                                                                           xs, xo, (bf16*)y);
  else
    k_pool2<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(B, H, W, C, (const bf16*)x, xs, xo,
                                                                     (bf16*)y);
  return check_launch();
}

int opyx_pool2_bwd(int B, int H, int W, int C, const float* dy, float* dx, int dxs, int dxo,
                   int accumulate, void* stream) {
  if (B < 1 || H < 2 || W < 2 || (H | W) & 1 || C < 1 || !dy || !dx || dxo < 0 || dxo + C > dxs)
    return OPYX_ERR_ARG;
  const int64_t total = (int64_t)B * H * W * C;
  if (C % 4 == 0 && dxs % 4 == 0 && dxo % 4 == 0 && al16(dy) && al16(dx))
    k_pool2_bwd4<<<grid_for(total / 4, 256), 256, 0, (cudaStream_t)stream>>>(B, H, W, C, dy, dx, dxs,
                                                                               dxo, accumulate);
  else
    k_pool2_bwd<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(B, H, W, C, dy, dx, dxs, dxo,
                                                                         accumulate);
  return check_launch();
}

int opyx_up2(int B, int h, int w, int C, const void* x, void* y, int ys, int yo, void* stream) {
  if (B < 1 || h < 1 || w < 1 || C < 1 || !x || !y || yo < 0 || yo + C > ys) return OPYX_ERR_ARG;
  const int64_t total = (int64_t)B * 4 * h * w * C;
  if (C % 8 == 0 && ys % 8 == 0 && yo % 8 == 0 && al16(x) && al16(y))
    k_up2_8<<<grid_for(total / 8, 256), 256, 0, (cudaStream_t)stream>>>(B, h, w, C, (const bf16*)x,
                                                                         (bf16*)y, ys, yo);
  else
    k_up2<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(B, h, w, C, (const bf16*)x, (bf16*)y,
                                                                  ys, yo);
  return check_launch();
}

int opyx_up2_bwd(int B, int h, int w, int C, const float* dy, int dys, int dyo, float* dx,
                 void* stream) {
  if (B < 1 || h < 1 || w < 1 || C < 1 || !dy || !dx || dyo < 0 || dyo + C > dys) return OPYX_ERR_ARG;
  const int64_t total = (int64_t)B * h * w * C;
  if (C % 4 == 0 && dys % 4 == 0 && dyo % 4 == 0 && al16(dy) && al16(dx))
    k_up2_bwd4<<<grid_for(total / 4, 256), 256, 0, (cudaStream_t)stream>>>(B, h, w, C, dy, dys, dyo,
                                                                             dx);
  else
    k_up2_bwd<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(B, h, w, C, dy, dys, dyo, dx);
  return check_launch();
}

int opyx_pack_input(int B, int64_t hw, const float* f, const float* lam, double lam_scale, void* x,
                    void* stream) {
  if (B < 1 || hw < 1 || !f || !lam || !x || !al16(x)) return OPYX_ERR_ARG;
  const int64_t total = (int64_t)B * hw * 32;
  k_pack_input<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(B, hw, f, lam, (float)lam_scale,
                                                                       (bf16*)x);
  return check_launch();
}

int opyx_pack_input_state(int B, int64_t hw, const float* f, const float* lam, double lam_scale,
                          const float* xb, const float* yb, void* x, void* stream) {
  if (B < 1 || hw < 1 || !f || !lam || !xb || !yb || !x || !al16(x)) return OPYX_ERR_ARG;
  const int64_t total = (int64_t)B * hw * 32;
  k_pack_input_state<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(
      B, hw, f, lam, (float)lam_scale, xb, yb, (bf16*)x);
  return check_launch();
}

int opyx_head(int64_t npix, int K, const void* a, const float* w, const float* b, float* out,
              void* stream) {
  if (npix < 1 || K != 3 || !a || !w || !b || !out || !al16(a)) return OPYX_ERR_ARG;
  k_head<3><<<grid_for(npix, 256), 256, 0, (cudaStream_t)stream>>>(npix, (const bf16*)a, w, b, out);
  return check_launch();
}

size_t opyx_head_bwd_workspace(int64_t npix, int K) {
  (void)npix;
  return (size_t)sm_count() * 2 * (K * 32 + K) * sizeof(float);
}

int opyx_head_bwd(int64_t npix, int K, const void* a, const float* w, const float* dout, float* da,
                  float* dw, float* db, void* ws, size_t ws_bytes, void* stream) {
  if (npix < 1 || K != 3 || !a || !w || !dout || !da || !dw || !db || !ws || !al16(a))
    return OPYX_ERR_ARG;
  if (ws_bytes < opyx_head_bwd_workspace(npix, K)) return OPYX_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const int nblk = sm_count() * 2;
  constexpr int NP = 3 * 32 + 3;
  k_head_bwd<3><<<nblk, 256, 0, s>>>(npix, (const bf16*)a, w, dout, da, (float*)ws);
  OPYX_CHECK_LAUNCH();
  // the first 96 sums are dW[k][c], the last 3 db[k]
  k_head_fold<<<1, 128, 0, s>>>((const float*)ws, nblk, NP, dw, db);
  return check_launch();
}

int opyx_mse(int64_t n, int K, const float* pred, const float* tgt, const float* wk, float* grad,
             double* partials, int nparts, void* stream) {
  if (n < 1 || K < 1 || !pred || !tgt || !wk || !grad || !partials || nparts < 1) return OPYX_ERR_ARG;
  k_mse<<<nparts, 256, 0, (cudaStream_t)stream>>>(n, K, pred, tgt, wk, 1.0 / (double)n, grad, partials);
  return check_launch();
}

int opyx_warm_loss(int B, int H, int W, const float* out, const float* tgt, const float* lam,
                   double w_x, double w_div, double w_u, double w_pool, float* grad, float* scratch,
                   double* partials, int nparts, void* stream) {
  if (B < 1 || H < 2 || W < 2 || !out || !tgt || !lam || !grad || !scratch || !partials || nparts < 1)
    return OPYX_ERR_ARG;
  if (w_pool != 0.0 && (H % 8 || W % 8)) return OPYX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const double inv_n = 1.0 / ((double)B * H * W);
  const int64_t total = (int64_t)B * H * W;
  float* pooled = scratch + total;
  if (w_pool != 0.0) {
    const int64_t nb = total / 64;
    k_warm_pool<<<grid_for(nb, 256), 256, 0, s>>>(B, H, W, out, tgt, lam, pooled);
    OPYX_CHECK_LAUNCH();
  }
  k_warm_loss1<<<nparts, 256, 0, s>>>(B, H, W, out, tgt, lam, (float)w_x, (float)w_div, (float)w_u,
                                      (float)w_pool, inv_n, pooled, scratch, partials);
  OPYX_CHECK_LAUNCH();
  k_warm_loss2<<<grid_for(total, 256), 256, 0, s>>>(B, H, W, out, tgt, (float)w_x, (float)w_u,
                                                    (float)w_pool, inv_n, pooled, scratch, grad);
  return check_launch();
}

int opyx_warm_unpack(int B, int64_t hw, const float* f, const float* lam, const float* out, float* x0,
                     float* y0, void* stream) {
  if (B < 1 || hw < 1 || !f || !lam || !out || !x0 || !y0) return OPYX_ERR_ARG;
  const int64_t n = (int64_t)B * hw;
  k_warm_unpack<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, hw, f, lam, out, x0, y0);
  return check_launch();
}

int opyx_warm_unpack_rel(int B, int64_t hw, const float* xb, const float* yb, const float* lam,
                         const float* out, float* x0, float* y0, void* stream) {
  if (B < 1 || hw < 1 || !xb || !yb || !lam || !out || !x0 || !y0) return OPYX_ERR_ARG;
  const int64_t n = (int64_t)B * hw;
  k_warm_unpack_rel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, hw, xb, yb, lam, out, x0, y0);
  return check_launch();
}

int opyx_adam(int64_t n, float* w, const float* g, float* m, float* v, double lr, double b1, double b2,
              double eps, int step, void* wb, void* wt, int cin, int cout, void* stream) {
  if (n < 1 || !w || !g || !m || !v || step < 1) return OPYX_ERR_ARG;
  if (wt && (cin < 1 || cout < 1 || (int64_t)9 * cin * cout != n)) return OPYX_ERR_ARG;
  const float c1 = (float)(1.0 - pow(b1, step)), c2 = (float)(1.0 - pow(b2, step));
  k_adam<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, w, g, m, v, (float)lr, (float)b1,
                                                             (float)b2, (float)eps, c1, c2, (bf16*)wb,
                                                             (bf16*)wt, cin, cout);
  return check_launch();
}

int opyx_conv_weights(int cin, int cout, const float* w, void* wb, void* wt, void* stream) {
  if (cin < 1 || cout < 1 || !w) return OPYX_ERR_ARG;
  const int64_t n = (int64_t)9 * cin * cout;
  k_conv_weights<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, w, (bf16*)wb, (bf16*)wt, cin,
                                                                     cout);
  return check_launch();
}

}  // extern "C"
