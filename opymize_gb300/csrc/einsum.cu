// Per-pixel small matrix products (MatrixMult, MatrixMultR, batched and
// tangled variants, diagonal scaling) and the label gather / scatter of the
// indexed operators.  One thread per output element.
//
// Two GB300 costs shape these kernels:
//  * The coefficient tables arrive in FP64 (the reference keeps them in
//    float64).  Converting an FP64 value is an FP64-pipe instruction, and that
//    pipe retires about two lanes per clock per SM on GB300, so a conversion
//    per use made the FP32 label scatter of a 512^2 x 16-label problem take
//    0.5 ms.  Each CTA converts its table once into shared memory in the
//    compute type (tables up to kTabBytes; larger ones are read and converted
//    per use).
//  * The output index is split into its coordinates by division.  64-bit
//    division by a run-time value is a long emulated sequence; below 2^31
//    outputs the kernels divide by multiply-high and shift (FastDiv).
#include "common.cuh"

namespace opyx {

constexpr int kEinThreads = 256;
constexpr int kTabBytes = 32 * 1024;

// Division by a run-time constant d >= 1 for numerators n < 2^31 with one
// multiply-high, one add and one shift (Granlund & Montgomery, "Division by
// Invariant Integers using Multiplication", PLDI 1994, Theorem 4.2): with
// l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1 (< 2^32),
// floor(n / d) = (umulhi(m, n) + n) >> l; the sum stays below 2^32 because
// umulhi(m, n) <= n < 2^31.
struct FastDiv {
  unsigned m, l;
  OPYX_D unsigned div(unsigned n) const { return (__umulhi(m, n) + n) >> l; }
};

inline FastDiv make_fastdiv(int64_t d) {
  unsigned l = 0;
  while (((int64_t)1 << l) < d) ++l;
  const uint64_t m = (((((uint64_t)1 << l) - (uint64_t)d) << 32) / (uint64_t)d) + 1;
  return FastDiv{(unsigned)m, l};
}

// Index arithmetic of one launch: 32-bit with FastDiv when every output
// index fits in 31 bits, else 64-bit with plain division.
template <typename I> struct Div;
template <> struct Div<unsigned> {
  FastDiv f;
  static Div make(int64_t d) { return Div{make_fastdiv(d)}; }
  OPYX_D unsigned operator()(unsigned n) const { return f.div(n); }
};
template <> struct Div<int64_t> {
  int64_t d;
  static Div make(int64_t d) { return Div{d}; }
  OPYX_D int64_t operator()(int64_t n) const { return n / d; }
};

#define EIN_LOOP(I, o, total)                                                  \
  for (I o = (I)(blockIdx.x * blockDim.x + threadIdx.x); o < (I)(total);        \
       o += (I)(gridDim.x * blockDim.x))

// The coefficient table in the compute type: a per-CTA copy in shared memory
// when the launch staged it, else the FP64 table read and converted per use.
template <typename T>
struct Coef {
  const T* s;
  const double* g;
  OPYX_D T operator[](int64_t k) const { return s ? s[k] : (T)__ldg(g + k); }
};

template <typename T>
OPYX_D T* ein_smem() {
  extern __shared__ __align__(16) unsigned char ein_raw[];
  return reinterpret_cast<T*>(ein_raw);
}

// ntab > 0: convert A[0, ntab) into shared memory (every thread of the CTA
// takes part; called before any thread may leave the kernel).
template <typename T>
OPYX_D Coef<T> stage_coef(const double* __restrict__ A, int ntab) {
  T* s = ein_smem<T>();
  for (int k = threadIdx.x; k < ntab; k += blockDim.x) s[k] = (T)__ldg(A + k);
  __syncthreads();
  return Coef<T>{ntab > 0 ? s : nullptr, A};
}

// y_ji = sum_k A_jk x_ki  (A (J,K); trans: A (K,J))
template <typename T, typename I>
__global__ void __launch_bounds__(kEinThreads)
k_matrixmult(I N, int J, int K, const double* __restrict__ A, int ntab, int trans,
             Div<I> divN, const T* __restrict__ x, T* __restrict__ y, int add) {
  const Coef<T> c = stage_coef<T>(A, ntab);
  EIN_LOOP(I, o, (int64_t)J * N) {
    const I jj = divN(o);
    const int j = (int)jj;
    const I i = o - jj * N;
    T acc = T(0);
    for (int k = 0; k < K; ++k)
      acc += c[trans ? (int64_t)k * J + j : (int64_t)j * K + k] * x[(int64_t)k * N + i];
    y[o] = add ? y[o] + acc : acc;
  }
}

// y_ij = sum_k x_ik A_kj  (A (K,J); trans: A (J,K))
template <typename T, typename I>
__global__ void __launch_bounds__(kEinThreads)
k_matrixmultr(I N, int K, int J, const double* __restrict__ A, int ntab, int trans,
              Div<I> divJ, const T* __restrict__ x, T* __restrict__ y, int add) {
  const Coef<T> c = stage_coef<T>(A, ntab);
  EIN_LOOP(I, o, (int64_t)N * J) {
    const I i = divJ(o);
    const int j = (int)(o - i * (I)J);
    const T* xi = x + (int64_t)i * K;
    T acc = T(0);
    for (int k = 0; k < K; ++k)
      acc += xi[k] * c[trans ? (int64_t)j * K + k : (int64_t)k * J + j];
    y[o] = add ? y[o] + acc : acc;
  }
}

// y_jlk = sum_m x_jlm A_jmk  (A (J,M,K); trans: A (J,K,M))
template <typename T, typename I>
__global__ void __launch_bounds__(kEinThreads)
k_mmr_batched(int J, I L, int M, int K, const double* __restrict__ A, int ntab, int trans,
              Div<I> divK, Div<I> divL, const T* __restrict__ x, T* __restrict__ y, int add) {
  const Coef<T> c = stage_coef<T>(A, ntab);
  EIN_LOOP(I, o, (int64_t)J * L * K) {
    const I jl = divK(o);
    const int k = (int)(o - jl * (I)K);
    const I jj = divL(jl);
    const int j = (int)jj;
    const T* xjl = x + (int64_t)jl * M;
    const int64_t a0 = (int64_t)j * M * K;
    T acc = T(0);
    for (int m = 0; m < M; ++m)
      acc += xjl[m] * c[a0 + (trans ? (int64_t)k * M + m : (int64_t)m * K + k)];
    y[o] = add ? y[o] + acc : acc;
  }
}

// y_mik = sum_jl x_jil A_jlmk  (A (J,L,M,K); trans: A (M,K,J,L))
template <typename T, typename I>
__global__ void __launch_bounds__(kEinThreads)
k_tangled(int J, I N, int L, int M, int K, const double* __restrict__ A, int ntab, int trans,
          Div<I> divK, Div<I> divN, const T* __restrict__ x, T* __restrict__ y, int add) {
  const Coef<T> c = stage_coef<T>(A, ntab);
  const int MK = M * K;
  EIN_LOOP(I, o, (int64_t)M * N * K) {
    const I mi = divK(o);
    const int k = (int)(o - mi * (I)K);
    const I mm = divN(mi);
    const I i = mi - mm * N;
    const int mk = (int)mm * K + k;
    T acc = T(0);
    for (int j = 0; j < J; ++j) {
      const T* xji = x + ((int64_t)j * N + i) * L;
      for (int l = 0; l < L; ++l)
        acc += xji[l] * c[trans ? (int64_t)mk * J * L + j * L + l
                                : ((int64_t)j * L + l) * MK + mk];
    }
    y[o] = add ? y[o] + acc : acc;
  }
}

template <typename T, typename I>
__global__ void __launch_bounds__(kEinThreads)
k_diag_mmr(I N, int K, const double* __restrict__ A, int ntab, Div<I> divK,
           const T* __restrict__ x, T* __restrict__ y, int add) {
  const Coef<T> c = stage_coef<T>(A, ntab);
  EIN_LOOP(I, o, (int64_t)N * K) {
    const int k = (int)(o - divK(o) * (I)K);
    const T v = x[o] * c[k];
    y[o] = add ? y[o] + v : v;
  }
}

// y[j,i,m] = -sum_l B[j,m,l] x[i,P[j,l]]
template <typename T, typename I>
__global__ void __launch_bounds__(kEinThreads)
k_indexedmult(int J, I N, int M, int L, int K, const double* __restrict__ B, int ntab,
              const int64_t* __restrict__ P, Div<I> divM, Div<I> divN,
              const T* __restrict__ x, T* __restrict__ y, int add) {
  const Coef<T> c = stage_coef<T>(B, ntab);
  EIN_LOOP(I, o, (int64_t)J * N * M) {
    const I ji = divM(o);
    const int m = (int)(o - ji * (I)M);
    const I jj = divN(ji);
    const int j = (int)jj;
    const I i = ji - jj * N;
    T acc = T(0);
    for (int l = 0; l < L; ++l) {
      const int64_t pk = __ldg(P + (int64_t)j * L + l);
      if (pk < 0 || pk >= K) continue;  // the host validates P; never read out of range
      acc -= c[((int64_t)j * M + m) * L + l] * x[(int64_t)i * K + pk];
    }
    y[o] = add ? y[o] + acc : acc;
  }
}

// Per-CTA lists of the (j, l) with P[j, l] = k for every label k, in
// ascending (j, l): offsets off[0..K] and entries (j << 16) | l.  Every
// thread of the CTA takes part.
OPYX_D void label_lists(const int64_t* __restrict__ P, int JL, int L, int K, int* off,
                        int* ent) {
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    int cnt = 0;
    for (int e = 0; e < JL; ++e) cnt += (int)(__ldg(P + e) == k);
    off[k + 1] = cnt;
  }
  if (threadIdx.x == 0) off[0] = 0;
  __syncthreads();
  if (threadIdx.x < 32) {           // inclusive scan of the counts, 32 at a time
    int carry = 0;
    for (int b = 0; b < K; b += 32) {
      const int lane = threadIdx.x, k = b + lane;
      int v = k < K ? off[k + 1] : 0;
#pragma unroll
      for (int s = 1; s < 32; s <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, s);
        if (lane >= s) v += u;
      }
      if (k < K) off[k + 1] = v + carry;
      carry += __shfl_sync(0xffffffffu, v, 31);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    int q = off[k];
    for (int e = 0; e < JL; ++e)
      if (__ldg(P + e) == k) {
        const int j = e / L;
        ent[q++] = (j << 16) | (e - j * L);
      }
  }
  __syncthreads();
}

// y[i,k] = -sum_{j,l: P[j,l]=k} sum_m B[j,m,l] x[j,i,m]: one thread per
// output (i,k), so no two threads write the same element.  Staged launches
// also build, per CTA, the list of the (j,l) with P[j,l] = k for every label
// (ascending (j,l), the order of the unstaged loop): a thread then visits its
// label's entries only, instead of testing all J*L.
template <typename T, typename I>
__global__ void __launch_bounds__(kEinThreads)
k_indexedmult_adj(int J, I N, int M, int L, int K, const double* __restrict__ B, int ntab,
                  const int64_t* __restrict__ P, Div<I> divK, const T* __restrict__ x,
                  T* __restrict__ y, int add) {
  const Coef<T> c = stage_coef<T>(B, ntab);
  const int JL = J * L;
  int* off = reinterpret_cast<int*>(ein_smem<T>() + ntab);   // K + 1 list offsets
  int* ent = off + K + 1;                                    // JL entries, (j << 16) | l
  if (ntab > 0) label_lists(P, JL, L, K, off, ent);
  EIN_LOOP(I, o, (int64_t)N * K) {
    const I i = divK(o);
    const int k = (int)(o - i * (I)K);
    T acc = T(0);
    if (ntab > 0) {
      const int q1 = off[k + 1];
      for (int q = off[k]; q < q1; ++q) {
        const int j = ent[q] >> 16, l = ent[q] & 0xffff;
        const T* xji = x + ((int64_t)j * N + i) * M;
        for (int m = 0; m < M; ++m) acc -= c[((int64_t)j * M + m) * L + l] * xji[m];
      }
    } else {
      for (int j = 0; j < J; ++j) {
        for (int l = 0; l < L; ++l) {
          if (__ldg(P + (int64_t)j * L + l) != k) continue;
          const T* xji = x + ((int64_t)j * N + i) * M;
          for (int m = 0; m < M; ++m) acc -= c[((int64_t)j * M + m) * L + l] * xji[m];
        }
      }
    }
    y[o] = add ? y[o] + acc : acc;
  }
}

// ---------------------------------------------------------------------------
// Tiled forms.  The per-output kernels above read rows of K labels with a
// stride of K values between neighbouring threads (the gather) or write them
// so (the scatter, MatrixMultR); one warp-wide access then touches up to 32
// sectors for 128 useful bytes.  The tiled kernels move a tile of kTilePx
// pixels through shared memory instead: the rows in (gather, MatrixMultR) or
// the rows out (scatter) are copied as one contiguous, coalesced block, with a
// row pitch of K + 1 values so that column accesses in shared memory are free
// of bank conflicts.  Each output is the same sum, in the same order, as in
// the per-output kernels.
// ---------------------------------------------------------------------------

constexpr int kTilePx = kEinThreads;
constexpr int kTileSmemMax = 48 * 1024;

// Offset (in T) of the tile after `bytes` of tables, rounded up to 16 bytes.
template <typename T>
inline int64_t tile_offset(int64_t bytes) {
  return ((bytes + 15) / 16 * 16) / (int64_t)sizeof(T);
}

// rows [p0, p0 + np) of a row-major (*, K) array into xs with pitch K + 1
template <typename T>
OPYX_D void stage_rows(const T* __restrict__ x, int64_t p0, int np, int K, FastDiv divK,
                       T* __restrict__ xs) {
  const T* src = x + p0 * K;
  const int n = np * K;
#pragma unroll 4
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const int p = (int)divK.div((unsigned)e);
    xs[p * (K + 1) + (e - p * K)] = src[e];
  }
}

// y_ij = sum_k x_ik A_kj over a tile of rows (as k_matrixmultr)
template <typename T>
__global__ void __launch_bounds__(kEinThreads)
k_matrixmultr_tile(int64_t N, int K, int J, const double* __restrict__ A, int ntab, int trans,
                   int64_t tile_off, FastDiv divK, FastDiv divJ, const T* __restrict__ x,
                   T* __restrict__ y, int add) {
  const Coef<T> c = stage_coef<T>(A, ntab);
  T* xs = ein_smem<T>() + tile_off;
  for (int64_t p0 = blockIdx.x * (int64_t)kTilePx; p0 < N; p0 += (int64_t)gridDim.x * kTilePx) {
    const int np = (int)(N - p0 < kTilePx ? N - p0 : kTilePx);
    stage_rows(x, p0, np, K, divK, xs);
    __syncthreads();
    T* yt = y + p0 * J;
    const int n = np * J;
#pragma unroll 4
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
      const int p = (int)divJ.div((unsigned)e);
      const int j = e - p * J;
      const T* xp = xs + p * (K + 1);
      T acc = T(0);
      for (int k = 0; k < K; ++k) acc += xp[k] * c[trans ? j * K + k : k * J + j];
      yt[e] = add ? yt[e] + acc : acc;
    }
    __syncthreads();
  }
}

// y[j,i,m] = -sum_l B[j,m,l] x[i,P[j,l]] over a tile of pixels (as k_indexedmult)
template <typename T>
__global__ void __launch_bounds__(kEinThreads)
k_indexedmult_tile(int J, int64_t N, int M, int L, int K, const double* __restrict__ B,
                   int ntab, const int64_t* __restrict__ P, int64_t tile_off, FastDiv divK,
                   FastDiv divM, const T* __restrict__ x, T* __restrict__ y, int add) {
  const Coef<T> c = stage_coef<T>(B, ntab);
  int* ps = reinterpret_cast<int*>(ein_smem<T>() + ntab);    // P as int, -1 out of range
  for (int e = threadIdx.x; e < J * L; e += blockDim.x) {
    const int64_t pk = __ldg(P + e);
    ps[e] = pk < 0 || pk >= K ? -1 : (int)pk;   // the host validates P; never read out of range
  }
  T* xs = ein_smem<T>() + tile_off;
  for (int64_t p0 = blockIdx.x * (int64_t)kTilePx; p0 < N; p0 += (int64_t)gridDim.x * kTilePx) {
    const int np = (int)(N - p0 < kTilePx ? N - p0 : kTilePx);
    stage_rows(x, p0, np, K, divK, xs);
    __syncthreads();
    const int n = np * M;
    for (int j = 0; j < J; ++j) {
      T* yt = y + ((int64_t)j * N + p0) * M;
#pragma unroll 2
      for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int p = (int)divM.div((unsigned)e);
        const int m = e - p * M;
        const T* xp = xs + p * (K + 1);
        T acc = T(0);
        for (int l = 0; l < L; ++l) {
          const int pk = ps[j * L + l];
          if (pk < 0) continue;
          acc -= c[((int64_t)j * M + m) * L + l] * xp[pk];
        }
        yt[e] = add ? yt[e] + acc : acc;
      }
    }
    __syncthreads();
  }
}

// y[i,k] = -sum_{j,l: P[j,l]=k} sum_m B[j,m,l] x[j,i,m] over a tile of
// pixels (as k_indexedmult_adj): thread t sums every label of pixel p0 + t,
// reading x[j, i, :] coalesced across the warp, into a tile that leaves as one
// contiguous block.
template <typename T>
__global__ void __launch_bounds__(kEinThreads)
k_indexedmult_adj_tile(int J, int64_t N, int M, int L, int K, const double* __restrict__ B,
                       int ntab, const int64_t* __restrict__ P, int64_t tile_off, FastDiv divK,
                       const T* __restrict__ x, T* __restrict__ y, int add) {
  const Coef<T> c = stage_coef<T>(B, ntab);
  int* off = reinterpret_cast<int*>(ein_smem<T>() + ntab);
  int* ent = off + K + 1;
  label_lists(P, J * L, L, K, off, ent);
  T* ts = ein_smem<T>() + tile_off;
  for (int64_t p0 = blockIdx.x * (int64_t)kTilePx; p0 < N; p0 += (int64_t)gridDim.x * kTilePx) {
    const int np = (int)(N - p0 < kTilePx ? N - p0 : kTilePx);
    const int p = threadIdx.x;
    if (p < np) {
      const int64_t i = p0 + p;
      for (int k = 0; k < K; ++k) {
        T acc = T(0);
        const int q1 = off[k + 1];
        for (int q = off[k]; q < q1; ++q) {
          const int j = ent[q] >> 16, l = ent[q] & 0xffff;
          const T* xji = x + ((int64_t)j * N + i) * M;
          for (int m = 0; m < M; ++m) acc -= c[((int64_t)j * M + m) * L + l] * xji[m];
        }
        ts[p * (K + 1) + k] = acc;
      }
    }
    __syncthreads();
    T* yt = y + p0 * K;
    const int n = np * K;
#pragma unroll 4
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
      const int q = (int)divK.div((unsigned)e);
      const T v = ts[q * (K + 1) + (e - q * K)];
      yt[e] = add ? yt[e] + v : v;
    }
    __syncthreads();
  }
}

// Entries of a table staged in shared memory (0: read from global memory).
template <typename T>
inline int tab_entries(int64_t n, int64_t extra_bytes = 0) {
  return n > 0 && n * (int64_t)sizeof(T) + extra_bytes <= kTabBytes ? (int)n : 0;
}

// Launch `kern` over `total` outputs with 32-bit indices when they fit.
#define EIN_LAUNCH(total, ntab_expr, extra, KERNEL, ...)                              \
  do {                                                                                \
    if ((total) == 0) return OPYX_OK;                                                 \
    OPYX_DISPATCH(dtype, T, {                                                         \
      const int ntab = (ntab_expr);                                                   \
      const size_t smem = ntab ? (size_t)ntab * sizeof(T) + (size_t)(extra) : 0;      \
      const unsigned grid = grid_for((total), kEinThreads);                           \
      cudaStream_t s = (cudaStream_t)stream;                                          \
      if ((total) < ((int64_t)1 << 31)) {                                             \
        using I = unsigned;                                                           \
        KERNEL<T, I><<<grid, kEinThreads, smem, s>>>(__VA_ARGS__);                    \
      } else {                                                                        \
        using I = int64_t;                                                            \
        KERNEL<T, I><<<grid, kEinThreads, smem, s>>>(__VA_ARGS__);                    \
      }                                                                               \
    });                                                                               \
    return check_launch();                                                            \
  } while (0)

}  // namespace opyx

using namespace opyx;

extern "C" {

int opyx_matrixmult(int dtype, int64_t N, int J, int K, const double* A, int trans,
                    const void* x, void* y, int add, void* stream) {
  if (N < 0 || J < 0 || K < 0 || !A || !x || !y) return OPYX_ERR_ARG;
  EIN_LAUNCH((int64_t)J * N, tab_entries<T>((int64_t)J * K), 0, k_matrixmult,
             (I)N, J, K, A, ntab, trans, Div<I>::make(N > 0 ? N : 1), (const T*)x, (T*)y, add);
}

int opyx_matrixmultr(int dtype, int64_t N, int K, int J, const double* A, int trans,
                     const void* x, void* y, int add, void* stream) {
  if (N < 0 || J < 0 || K < 0 || !A || !x || !y) return OPYX_ERR_ARG;
  if (N > 0) {
    OPYX_DISPATCH(dtype, T, {
      const int ntab = tab_entries<T>((int64_t)K * J);
      const int64_t toff = tile_offset<T>((int64_t)ntab * sizeof(T));
      const int64_t smem = (toff + (int64_t)kTilePx * (K + 1)) * (int64_t)sizeof(T);
      if (ntab > 0 && smem <= kTileSmemMax) {
        k_matrixmultr_tile<T><<<grid_for(N, kTilePx), kEinThreads, smem, (cudaStream_t)stream>>>(
            N, K, J, A, ntab, trans, toff, make_fastdiv(K), make_fastdiv(J), (const T*)x,
            (T*)y, add);
        return check_launch();
      }
    });
  }
  EIN_LAUNCH(N * J, tab_entries<T>((int64_t)K * J), 0, k_matrixmultr,
             (I)N, K, J, A, ntab, trans, Div<I>::make(J > 0 ? J : 1), (const T*)x, (T*)y, add);
}

int opyx_matrixmultr_batched(int dtype, int J, int64_t L, int M, int K, const double* A,
                             int trans, const void* x, void* y, int add, void* stream) {
  if (J < 0 || L < 0 || M < 0 || K < 0 || !A || !x || !y) return OPYX_ERR_ARG;
  EIN_LAUNCH((int64_t)J * L * K, tab_entries<T>((int64_t)J * M * K), 0, k_mmr_batched,
             J, (I)L, M, K, A, ntab, trans, Div<I>::make(K > 0 ? K : 1),
             Div<I>::make(L > 0 ? L : 1), (const T*)x, (T*)y, add);
}

int opyx_tangled_matrixmultr(int dtype, int J, int64_t N, int L, int M, int K,
                             const double* A, int trans, const void* x, void* y, int add,
                             void* stream) {
  if (J < 0 || N < 0 || L < 0 || M < 0 || K < 0 || !A || !x || !y) return OPYX_ERR_ARG;
  EIN_LAUNCH((int64_t)M * N * K, tab_entries<T>((int64_t)J * L * M * K), 0, k_tangled,
             J, (I)N, L, M, K, A, ntab, trans, Div<I>::make(K > 0 ? K : 1),
             Div<I>::make(N > 0 ? N : 1), (const T*)x, (T*)y, add);
}

int opyx_diag_matrixmultr(int dtype, int64_t N, int K, const double* A, const void* x,
                          void* y, int add, void* stream) {
  if (N < 0 || K < 0 || !A || !x || !y) return OPYX_ERR_ARG;
  EIN_LAUNCH(N * K, tab_entries<T>(K), 0, k_diag_mmr,
             (I)N, K, A, ntab, Div<I>::make(K > 0 ? K : 1), (const T*)x, (T*)y, add);
}

int opyx_indexedmult(int dtype, int J, int64_t N, int M, int L, int K, const double* B,
                     const int64_t* P, const void* x, void* y, int add, void* stream) {
  if (J < 0 || N < 0 || M < 0 || L < 0 || K < 1 || !B || !P || !x || !y) return OPYX_ERR_ARG;
  if (N > 0 && J > 0 && M > 0 && L > 0) {
    OPYX_DISPATCH(dtype, T, {
      const int64_t ps = (int64_t)J * L * (int64_t)sizeof(int);
      const int ntab = tab_entries<T>((int64_t)J * M * L, ps);
      const int64_t toff = tile_offset<T>((int64_t)ntab * sizeof(T) + ps);
      const int64_t smem = (toff + (int64_t)kTilePx * (K + 1)) * (int64_t)sizeof(T);
      if (ntab > 0 && smem <= kTileSmemMax) {
        k_indexedmult_tile<T><<<grid_for(N, kTilePx), kEinThreads, smem, (cudaStream_t)stream>>>(
            J, N, M, L, K, B, ntab, P, toff, make_fastdiv(K), make_fastdiv(M), (const T*)x,
            (T*)y, add);
        return check_launch();
      }
    });
  }
  EIN_LAUNCH((int64_t)J * N * M, tab_entries<T>((int64_t)J * M * L), 0, k_indexedmult,
             J, (I)N, M, L, K, B, ntab, P, Div<I>::make(M > 0 ? M : 1),
             Div<I>::make(N > 0 ? N : 1), (const T*)x, (T*)y, add);
}

int opyx_indexedmult_adj(int dtype, int J, int64_t N, int M, int L, int K, const double* B,
                         const int64_t* P, const void* x, void* y, int add, void* stream) {
  if (J < 0 || N < 0 || M < 0 || L < 0 || K < 1 || !B || !P || !x || !y) return OPYX_ERR_ARG;
  // the label lists pack (j, l) into 16 bits each; their offsets and entries
  // follow the table in shared memory
  const int64_t lists = ((int64_t)K + 1 + (int64_t)J * L) * (int64_t)sizeof(int);
  // (each thread of the CTA's prologue scans all J*L indices for its labels)
  const int64_t JL = (int64_t)J * L;
  const bool listable = J < 32768 && L < 65536 && JL <= 4096 && K <= 4096 &&
                        ((int64_t)K + kEinThreads - 1) / kEinThreads * JL <= 4096;
  if (listable && N > 0 && J * M * L > 0) {
    OPYX_DISPATCH(dtype, T, {
      const int ntab = tab_entries<T>((int64_t)J * M * L, lists);
      const int64_t toff = tile_offset<T>((int64_t)ntab * sizeof(T) + lists);
      const int64_t smem = (toff + (int64_t)kTilePx * (K + 1)) * (int64_t)sizeof(T);
      if (ntab > 0 && smem <= kTileSmemMax) {
        k_indexedmult_adj_tile<T><<<grid_for(N, kTilePx), kEinThreads, smem,
                                    (cudaStream_t)stream>>>(J, N, M, L, K, B, ntab, P, toff,
                                                            make_fastdiv(K), (const T*)x, (T*)y,
                                                            add);
        return check_launch();
      }
    });
  }
  EIN_LAUNCH(N * K, listable && J * M * L > 0 ? tab_entries<T>((int64_t)J * M * L, lists) : 0,
             lists, k_indexedmult_adj, J, (I)N, M, L, K, B, ntab, P,
             Div<I>::make(K), (const T*)x, (T*)y, add);
}

}  // extern "C"
