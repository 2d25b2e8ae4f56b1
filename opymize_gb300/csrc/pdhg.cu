// Generic PDHG step kernels (any LinOp / prox composition): primal and dual
// steps, the FP64 residual reductions of the adaptive step rule and the
// on-device step-size update (opymize/solvers/pdhg.py:46-187).
#include "common.cuh"
#include "prox_dev.cuh"

namespace opyx {

#define GRID_STRIDE(o, total) \
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < (total); \
       o += (int64_t)gridDim.x * blockDim.x)

template <typename T>
__global__ void k_take_step(int64_t n, T* __restrict__ zkp1, const T* __restrict__ zk, T dir,
                            StepT<T> step, const T* __restrict__ zg) {
  step.load();
  GRID_STRIDE(i, n) zkp1[i] = zk[i] + dir * step.at(i) * zg[i];
}

template <typename T>
__global__ void k_dual_step(int64_t n, T* __restrict__ ykp1, const T* __restrict__ yk,
                            StepT<T> sigma, T theta, const T* __restrict__ ygkp1,
                            const T* __restrict__ ygk) {
  sigma.load();
  GRID_STRIDE(i, n) {
    const T ybar = (T(1) + theta) * ygkp1[i] - theta * ygk[i];
    ykp1[i] = yk[i] + sigma.at(i) * ybar;
  }
}

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 1024;

template <typename T>
__global__ void __launch_bounds__(kRedThreads)
k_residual_pair(int64_t n, StepT<T> a, const T* __restrict__ zk, const T* __restrict__ zkp1,
                T b, const T* __restrict__ zgk, T c1, T c2, const T* __restrict__ zgkp1,
                double* out, double* partials, unsigned* ticket) {
  a.load();
  double s1 = 0.0, s2 = 0.0;
  GRID_STRIDE(i, n) {
    const T base = (zk[i] - zkp1[i]) / a.at(i) - b * zgk[i];
    const double r1 = (double)(base + c1 * zgkp1[i]);
    const double r2 = (double)(base + c2 * zgkp1[i]);
    s1 += r1 * r1;
    s2 += r2 * r2;
  }
  double vals[2] = {s1, s2};
  const int ops[2] = {RED_SUM, RED_SUM};
  block_reduce_and_finish<2>(vals, ops, partials, ticket, [&](double* tot) {
    out[0] += tot[0];
    out[1] += tot[1];
  });
}

__global__ void k_adaptive_update(opyx_adaptive_state* st) {
  if (threadIdx.x == 0 && blockIdx.x == 0) adaptive_rule(st);
}

}  // namespace opyx

using namespace opyx;

extern "C" {

int opyx_take_step(int dtype, int64_t n, void* zkp1, const void* zk, int direction,
                   opyx_step step, const void* zgrad, void* stream) {
  if (n < 0 || (n > 0 && (!zkp1 || !zk || !zgrad))) return OPYX_ERR_ARG;
  if (n == 0) return OPYX_OK;
  OPYX_DISPATCH(dtype, T, (k_take_step<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                              n, (T*)zkp1, (const T*)zk, (T)direction, StepT<T>(step),
                              (const T*)zgrad)));
  return check_launch();
}

int opyx_dual_step(int dtype, int64_t n, void* ykp1, const void* yk, opyx_step sigma,
                   double theta, const void* ygkp1, const void* ygk, void* stream) {
  if (n < 0 || (n > 0 && (!ykp1 || !yk || !ygkp1 || !ygk))) return OPYX_ERR_ARG;
  if (n == 0) return OPYX_OK;
  OPYX_DISPATCH(dtype, T, (k_dual_step<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                              n, (T*)ykp1, (const T*)yk, StepT<T>(sigma), (T)theta,
                              (const T*)ygkp1, (const T*)ygk)));
  return check_launch();
}

int opyx_residual_pair(int dtype, int64_t n, opyx_step a, const void* zk, const void* zkp1,
                       double b, const void* zgk, double c1, double c2, const void* zgkp1,
                       double* out, void* ws, void* stream) {
  if (n < 0 || !out || !ws || (n > 0 && (!zk || !zkp1 || !zgk || !zgkp1))) return OPYX_ERR_ARG;
  if (((uintptr_t)ws) & 7) return OPYX_ERR_WORKSPACE;
  double* partials = (double*)ws;
  unsigned* ticket = (unsigned*)((char*)ws + (size_t)kRedBlocks * 8 * sizeof(double));
  unsigned g = grid_for(n, kRedThreads, 4);
  if (g > (unsigned)kRedBlocks) g = kRedBlocks;
  OPYX_DISPATCH(dtype, T, (k_residual_pair<T><<<g, kRedThreads, 0, (cudaStream_t)stream>>>(
                              n, StepT<T>(a), (const T*)zk, (const T*)zkp1, (T)b,
                              (const T*)zgk, (T)c1, (T)c2, (const T*)zgkp1, out, partials,
                              ticket)));
  return check_launch();
}

int opyx_adaptive_update(opyx_adaptive_state* st, void* stream) {
  if (!st) return OPYX_ERR_ARG;
  k_adaptive_update<<<1, 32, 0, (cudaStream_t)stream>>>(st);
  return check_launch();
}

}  // extern "C"
