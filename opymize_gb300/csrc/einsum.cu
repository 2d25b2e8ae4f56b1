// Per-pixel small matrix products (MatrixMult, MatrixMultR, batched and
// tangled variants, diagonal scaling) and the label gather / scatter of the
// indexed operators.  One thread per output element; the small matrices stay
// in L1 through __ldg.
#include "common.cuh"

namespace opyx {

#define GRID_STRIDE(o, total) \
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < (total); \
       o += (int64_t)gridDim.x * blockDim.x)

// y_ji = sum_k A_jk x_ki  (A (J,K); trans: A (K,J))
template <typename T>
__global__ void k_matrixmult(int64_t N, int J, int K, const double* __restrict__ A, int trans,
                             const T* __restrict__ x, T* __restrict__ y, int add) {
  GRID_STRIDE(o, (int64_t)J * N) {
    const int j = (int)(o / N);
    const int64_t i = o % N;
    T acc = T(0);
    for (int k = 0; k < K; ++k) {
      const double a = trans ? __ldg(A + (int64_t)k * J + j) : __ldg(A + (int64_t)j * K + k);
      acc += (T)a * x[(int64_t)k * N + i];
    }
    y[o] = add ? y[o] + acc : acc;
  }
}

// y_ij = sum_k x_ik A_kj  (A (K,J); trans: A (J,K))
template <typename T>
__global__ void k_matrixmultr(int64_t N, int K, int J, const double* __restrict__ A, int trans,
                              const T* __restrict__ x, T* __restrict__ y, int add) {
  GRID_STRIDE(o, N * J) {
    const int j = (int)(o % J);
    const int64_t i = o / J;
    const T* xi = x + i * K;
    T acc = T(0);
    for (int k = 0; k < K; ++k) {
      const double a = trans ? __ldg(A + (int64_t)j * K + k) : __ldg(A + (int64_t)k * J + j);
      acc += xi[k] * (T)a;
    }
    y[o] = add ? y[o] + acc : acc;
  }
}

// y_jlk = sum_m x_jlm A_jmk  (A (J,M,K); trans: A (J,K,M))
template <typename T>
__global__ void k_mmr_batched(int J, int64_t L, int M, int K, const double* __restrict__ A,
                              int trans, const T* __restrict__ x, T* __restrict__ y, int add) {
  GRID_STRIDE(o, (int64_t)J * L * K) {
    const int k = (int)(o % K);
    const int64_t l = (o / K) % L;
    const int j = (int)(o / (K * L));
    const T* xjl = x + ((int64_t)j * L + l) * M;
    const double* Aj = A + (int64_t)j * M * K;
    T acc = T(0);
    for (int m = 0; m < M; ++m) {
      const double a = trans ? __ldg(Aj + (int64_t)k * M + m) : __ldg(Aj + (int64_t)m * K + k);
      acc += xjl[m] * (T)a;
    }
    y[o] = add ? y[o] + acc : acc;
  }
}

// y_mik = sum_jl x_jil A_jlmk  (A (J,L,M,K); trans: A (M,K,J,L))
template <typename T>
__global__ void k_tangled(int J, int64_t N, int L, int M, int K, const double* __restrict__ A,
                          int trans, const T* __restrict__ x, T* __restrict__ y, int add) {
  const int MK = M * K;
  GRID_STRIDE(o, (int64_t)M * N * K) {
    const int k = (int)(o % K);
    const int64_t i = (o / K) % N;
    const int m = (int)(o / (K * N));
    const int mk = m * K + k;
    T acc = T(0);
    for (int j = 0; j < J; ++j) {
      const T* xji = x + ((int64_t)j * N + i) * L;
      for (int l = 0; l < L; ++l) {
        const double a = trans ? __ldg(A + (int64_t)mk * J * L + j * L + l)
                               : __ldg(A + ((int64_t)j * L + l) * MK + mk);
        acc += xji[l] * (T)a;
      }
    }
    y[o] = add ? y[o] + acc : acc;
  }
}

template <typename T>
__global__ void k_diag_mmr(int64_t N, int K, const double* __restrict__ A,
                           const T* __restrict__ x, T* __restrict__ y, int add) {
  GRID_STRIDE(o, N * K) {
    const T v = x[o] * (T)__ldg(A + (int)(o % K));
    y[o] = add ? y[o] + v : v;
  }
}

// y[j,i,m] = -sum_l B[j,m,l] x[i,P[j,l]]
template <typename T>
__global__ void k_indexedmult(int J, int64_t N, int M, int L, int K, const double* __restrict__ B,
                              const int64_t* __restrict__ P, const T* __restrict__ x,
                              T* __restrict__ y, int add) {
  GRID_STRIDE(o, (int64_t)J * N * M) {
    const int m = (int)(o % M);
    const int64_t i = (o / M) % N;
    const int j = (int)(o / (M * N));
    T acc = T(0);
    for (int l = 0; l < L; ++l) {
      const int64_t pk = __ldg(P + (int64_t)j * L + l);
      if (pk < 0 || pk >= K) continue;  // the host validates P; never read out of range
      acc -= (T)__ldg(B + ((int64_t)j * M + m) * L + l) * x[i * K + pk];
    }
    y[o] = add ? y[o] + acc : acc;
  }
}

// y[i,k] = -sum_{j,l: P[j,l]=k} sum_m B[j,m,l] x[j,i,m]: one thread per
// output (i,k) gathers every (j,l) that maps to label k, so no two threads
// write the same element.
template <typename T>
__global__ void k_indexedmult_adj(int J, int64_t N, int M, int L, int K,
                                  const double* __restrict__ B, const int64_t* __restrict__ P,
                                  const T* __restrict__ x, T* __restrict__ y, int add) {
  GRID_STRIDE(o, N * K) {
    const int k = (int)(o % K);
    const int64_t i = o / K;
    T acc = T(0);
    for (int j = 0; j < J; ++j) {
      for (int l = 0; l < L; ++l) {
        if (__ldg(P + (int64_t)j * L + l) != k) continue;
        const T* xji = x + ((int64_t)j * N + i) * M;
        for (int m = 0; m < M; ++m) acc -= (T)__ldg(B + ((int64_t)j * M + m) * L + l) * xji[m];
      }
    }
    y[o] = add ? y[o] + acc : acc;
  }
}

}  // namespace opyx

using namespace opyx;

#define LAUNCH(kernel, n, ...)                                                  \
  do {                                                                          \
    if ((n) == 0) return OPYX_OK;                                               \
    OPYX_DISPATCH(dtype, T, (kernel<T><<<grid_for((n), 256), 256, 0,            \
                                         (cudaStream_t)stream>>>(__VA_ARGS__))); \
    return check_launch();                                                      \
  } while (0)

extern "C" {

int opyx_matrixmult(int dtype, int64_t N, int J, int K, const double* A, int trans,
                    const void* x, void* y, int add, void* stream) {
  if (N < 0 || J < 0 || K < 0 || !A || !x || !y) return OPYX_ERR_ARG;
  LAUNCH(k_matrixmult, (int64_t)J * N, N, J, K, A, trans, (const T*)x, (T*)y, add);
}

int opyx_matrixmultr(int dtype, int64_t N, int K, int J, const double* A, int trans,
                     const void* x, void* y, int add, void* stream) {
  if (N < 0 || J < 0 || K < 0 || !A || !x || !y) return OPYX_ERR_ARG;
  LAUNCH(k_matrixmultr, N * J, N, K, J, A, trans, (const T*)x, (T*)y, add);
}

int opyx_matrixmultr_batched(int dtype, int J, int64_t L, int M, int K, const double* A,
                             int trans, const void* x, void* y, int add, void* stream) {
  if (J < 0 || L < 0 || M < 0 || K < 0 || !A || !x || !y) return OPYX_ERR_ARG;
  LAUNCH(k_mmr_batched, (int64_t)J * L * K, J, L, M, K, A, trans, (const T*)x, (T*)y, add);
}

int opyx_tangled_matrixmultr(int dtype, int J, int64_t N, int L, int M, int K,
                             const double* A, int trans, const void* x, void* y, int add,
                             void* stream) {
  if (J < 0 || N < 0 || L < 0 || M < 0 || K < 0 || !A || !x || !y) return OPYX_ERR_ARG;
  LAUNCH(k_tangled, (int64_t)M * N * K, J, N, L, M, K, A, trans, (const T*)x, (T*)y, add);
}

int opyx_diag_matrixmultr(int dtype, int64_t N, int K, const double* A, const void* x,
                          void* y, int add, void* stream) {
  if (N < 0 || K < 0 || !A || !x || !y) return OPYX_ERR_ARG;
  LAUNCH(k_diag_mmr, N * K, N, K, A, (const T*)x, (T*)y, add);
}

int opyx_indexedmult(int dtype, int J, int64_t N, int M, int L, int K, const double* B,
                     const int64_t* P, const void* x, void* y, int add, void* stream) {
  if (J < 0 || N < 0 || M < 0 || L < 0 || K < 1 || !B || !P || !x || !y) return OPYX_ERR_ARG;
  LAUNCH(k_indexedmult, (int64_t)J * N * M, J, N, M, L, K, B, P, (const T*)x, (T*)y, add);
}

int opyx_indexedmult_adj(int dtype, int J, int64_t N, int M, int L, int K, const double* B,
                         const int64_t* P, const void* x, void* y, int add, void* stream) {
  if (J < 0 || N < 0 || M < 0 || L < 0 || K < 1 || !B || !P || !x || !y) return OPYX_ERR_ARG;
  LAUNCH(k_indexedmult_adj, N * K, J, N, M, L, K, B, P, (const T*)x, (T*)y, add);
}

}  // extern "C"
