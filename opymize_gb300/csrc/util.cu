// Library-wide utilities: status strings, SM count, fill / axpby /
// broadcast kernels and FP64 norms.
#include "common.cuh"

namespace opyx {

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (cached[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    cached[dev] = n;
  }
  return cached[dev];
}

template <typename T>
__global__ void k_fill(T* y, int64_t n, T v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = v;
}

template <typename T>
__global__ void k_axpby(int64_t n, T a, const T* __restrict__ x, T b, T* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    T r = a * x[i];
    if (b != T(0)) r += b * y[i];
    y[i] = r;
  }
}

template <typename T>
__global__ void k_abs(int64_t n, const T* __restrict__ x, T* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = x[i] < T(0) ? -x[i] : x[i];
}

template <typename S, typename D>
__global__ void k_cast(int64_t n, const S* __restrict__ x, D* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (D)x[i];
}

template <typename T>
__global__ void k_recip_positive(int64_t n, T* __restrict__ x, double eps) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if ((double)x[i] > eps) x[i] = T(1) / x[i];
}

template <typename T>
__global__ void k_broadcast_mid(const double* __restrict__ pat, int64_t outer, int64_t N,
                                int64_t inner, T* __restrict__ y, int add) {
  const int64_t total = outer * N * inner;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i % inner;
    int64_t o = i / (inner * N);
    T v = (T)pat[o * inner + r];
    y[i] = add ? y[i] + v : v;
  }
}

constexpr int kRedBlocks = 1024;   // upper bound of reduction grids
constexpr int kRedThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kRedThreads)
k_norms(int64_t n, const T* __restrict__ x, double* out, double* partials, unsigned* ticket) {
  double s = 0.0, m = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = (double)x[i];
    s += v * v;
    m = fmax(m, fabs(v));
  }
  double vals[2] = {s, m};
  const int ops[2] = {RED_SUM, RED_MAX};
  block_reduce_and_finish<2>(vals, ops, partials, ticket, [&](double* tot) {
    out[0] = tot[0];
    out[1] = tot[1];
  });
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads)
k_dot(int64_t n, const T* __restrict__ x, const T* __restrict__ y, double* out, double* partials,
      unsigned* ticket) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s += (double)x[i] * (double)y[i];
  double vals[1] = {s};
  const int ops[1] = {RED_SUM};
  block_reduce_and_finish<1>(vals, ops, partials, ticket, [&](double* tot) { out[0] = tot[0]; });
}

}  // namespace opyx

using namespace opyx;

extern "C" {

int opyx_version(void) { return 10000; }

const char* opyx_status_string(int s) {
  switch (s) {
    case OPYX_OK: return "ok";
    case OPYX_ERR_ARG: return "invalid argument (shape, size, pointer or enum)";
    case OPYX_ERR_LAUNCH: return "CUDA launch or runtime error";
    case OPYX_ERR_UNSUPPORTED: return "unsupported by this build";
    case OPYX_ERR_WORKSPACE: return "workspace too small or misaligned";
    case OPYX_ERR_NOT_CONVERGED: return "iterative device routine hit its iteration bound";
    case OPYX_ERR_SCRATCH_LIMIT:
      return "problem larger than the static scratch of the allocation-free entry point";
    default: return "unknown status";
  }
}

int opyx_sm_count(void) { return sm_count(); }

int opyx_fill(int dtype, void* y, int64_t n, double value, void* stream) {
  if (n < 0 || (n > 0 && !y)) return OPYX_ERR_ARG;
  if (n == 0) return OPYX_OK;
  OPYX_DISPATCH(dtype, T, (k_fill<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                              (T*)y, n, (T)value)));
  return check_launch();
}

int opyx_axpby(int dtype, int64_t n, double a, const void* x, double b, void* y,
               void* stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return OPYX_ERR_ARG;
  if (n == 0) return OPYX_OK;
  OPYX_DISPATCH(dtype, T, (k_axpby<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                              n, (T)a, (const T*)x, (T)b, (T*)y)));
  return check_launch();
}

int opyx_abs(int dtype, int64_t n, const void* x, void* y, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return OPYX_ERR_ARG;
  if (n == 0) return OPYX_OK;
  OPYX_DISPATCH(dtype, T, (k_abs<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                              n, (const T*)x, (T*)y)));
  return check_launch();
}

int opyx_cast(int src_dtype, int dst_dtype, int64_t n, const void* x, void* y, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return OPYX_ERR_ARG;
  if (n == 0) return OPYX_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned g = grid_for(n, 256);
  if (src_dtype == OPYX_F64 && dst_dtype == OPYX_F32)
    k_cast<double, float><<<g, 256, 0, s>>>(n, (const double*)x, (float*)y);
  else if (src_dtype == OPYX_F32 && dst_dtype == OPYX_F64)
    k_cast<float, double><<<g, 256, 0, s>>>(n, (const float*)x, (double*)y);
  else if (src_dtype == dst_dtype && (src_dtype == OPYX_F32 || src_dtype == OPYX_F64))
    return cudaMemcpyAsync(y, x, (size_t)n * (src_dtype == OPYX_F32 ? 4 : 8),
                           cudaMemcpyDeviceToDevice, s) == cudaSuccess ? OPYX_OK : OPYX_ERR_LAUNCH;
  else
    return OPYX_ERR_ARG;
  return check_launch();
}

int opyx_recip_positive(int dtype, int64_t n, void* x, double eps, void* stream) {
  if (n < 0 || (n > 0 && !x)) return OPYX_ERR_ARG;
  if (n == 0) return OPYX_OK;
  OPYX_DISPATCH(dtype, T, (k_recip_positive<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                              n, (T*)x, eps)));
  return check_launch();
}

int opyx_broadcast_mid(int dtype, const double* pat, int64_t outer, int64_t N,
                       int64_t inner, void* y, int add, void* stream) {
  if (outer < 0 || N < 0 || inner < 0) return OPYX_ERR_ARG;
  int64_t n = outer * N * inner;
  if (n == 0) return OPYX_OK;
  if (!pat || !y) return OPYX_ERR_ARG;
  OPYX_DISPATCH(dtype, T, (k_broadcast_mid<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                              pat, outer, N, inner, (T*)y, add)));
  return check_launch();
}

size_t opyx_reduce_workspace_size(void) {
  // partials for up to 8 values per block + ticket, 256-byte aligned
  return (size_t)kRedBlocks * 8 * sizeof(double) + 256;
}

int opyx_norms(int dtype, int64_t n, const void* x, double* out, void* ws, void* stream) {
  if (n < 0 || !out || !ws || (n > 0 && !x)) return OPYX_ERR_ARG;
  if (((uintptr_t)ws) & 7) return OPYX_ERR_WORKSPACE;
  double* partials = (double*)ws;
  unsigned* ticket = (unsigned*)((char*)ws + (size_t)kRedBlocks * 8 * sizeof(double));
  unsigned g = grid_for(n, kRedThreads, 4);
  if (g > (unsigned)kRedBlocks) g = kRedBlocks;
  OPYX_DISPATCH(dtype, T, (k_norms<T><<<g, kRedThreads, 0, (cudaStream_t)stream>>>(
                              n, (const T*)x, out, partials, ticket)));
  return check_launch();
}

int opyx_dot(int dtype, int64_t n, const void* x, const void* y, double* out, void* ws, void* stream) {
  if (n < 0 || !out || !ws || (n > 0 && (!x || !y))) return OPYX_ERR_ARG;
  if (((uintptr_t)ws) & 7) return OPYX_ERR_WORKSPACE;
  double* partials = (double*)ws;
  unsigned* ticket = (unsigned*)((char*)ws + (size_t)kRedBlocks * 8 * sizeof(double));
  unsigned g = grid_for(n, kRedThreads, 4);
  if (g > (unsigned)kRedBlocks) g = kRedBlocks;
  OPYX_DISPATCH(dtype, T, (k_dot<T><<<g, kRedThreads, 0, (cudaStream_t)stream>>>(
                              n, (const T*)x, (const T*)y, out, partials, ticket)));
  return check_launch();
}

}  // extern "C"
