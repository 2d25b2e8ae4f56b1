// Prox / projection maps of the functionals on the PDHG path (generic path):
// affine shift-scale, SSD prox, positive / negative parts, constraints,
// l1-norm ball projections (Frobenius, spectral 2xM), Huber conjugate prox and
// the quadratic-epigraph projection with its FP64 cubic root-solve.
#include "common.cuh"
#include "prox_dev.cuh"

namespace opyx {

#define GRID_STRIDE(o, total) \
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < (total); \
       o += (int64_t)gridDim.x * blockDim.x)

template <typename T>
__global__ void k_shiftscale(int64_t n, const T* __restrict__ av, T a, const T* __restrict__ bv,
                             T b, const T* __restrict__ sv, T s, const T* __restrict__ x,
                             T* __restrict__ y, int add) {
  GRID_STRIDE(i, n) {
    const T ai = av ? av[i] : a;
    const T bi = bv ? bv[i] : b;
    const T si = sv ? sv[i] : s;
    const T v = ai * (x[i] + bi * si);
    y[i] = add ? y[i] + v : v;
  }
}

// y = a*(x - tau*c): prox of tau*(b + <c, x>) (masked by a)
template <typename T>
__global__ void k_affine_prox(int64_t n, const T* __restrict__ av, T a, const T* __restrict__ cv,
                              T c, StepT<T> tau, const T* __restrict__ x, T* __restrict__ y) {
  tau.load();
  GRID_STRIDE(i, n) {
    const T ai = av ? av[i] : a;
    const T ci = cv ? cv[i] : c;
    y[i] = ai * (x[i] - tau.at(i) * ci);
  }
}

template <typename T>
__global__ void k_ssd_prox(int64_t N, int C, const T* __restrict__ f, const double* __restrict__ vol,
                           const uint8_t* __restrict__ mask, StepT<T> tau,
                           const T* __restrict__ x, T* __restrict__ y) {
  tau.load();
  GRID_STRIDE(o, N * C) {
    const int k = (int)(o % C);
    const int64_t i = o / C;
    T v = x[o];
    if (!mask || mask[i]) {
      const T tv = tau.at(o) * (T)(vol ? __ldg(vol + k) : 1.0);
      v = ssd_prox_value(v, f[o], tv);
    }
    y[o] = v;
  }
}

template <typename T>
__global__ void k_posneg(int64_t n, int neg, const T* __restrict__ x, T* __restrict__ y, int add) {
  GRID_STRIDE(i, n) {
    const T xi = x[i];
    const T v = neg ? (xi > T(0) ? T(0) : xi) : (xi < T(0) ? T(0) : xi);
    y[i] = add ? y[i] + v : v;
  }
}

template <typename T>
__global__ void k_constrain(int64_t N, int M, const uint8_t* __restrict__ mask,
                            const T* __restrict__ c, const T* __restrict__ x, T* __restrict__ y,
                            int add) {
  GRID_STRIDE(o, N * M) {
    const T v = mask[o / M] ? c[o] : x[o];
    y[o] = add ? y[o] + v : v;
  }
}

template <typename T>
__global__ void k_l1proj(int64_t N, int M1, int M2, T lbd, int spectral, T* __restrict__ x) {
  GRID_STRIDE(i, N) {
    T* xi = x + i * (int64_t)(M1 * M2);
    if (spectral && M1 != 1 && M2 != 1)
      spectral_proj_2xm(xi, M1, M2, lbd);
    else
      frob_proj(xi, M1 * M2, lbd);
  }
}

template <typename T>
__global__ void k_huber_conj(int64_t N, int m, T lbd, T alpha, StepT<T> sigma, T* __restrict__ x) {
  sigma.load();
  GRID_STRIDE(i, N) {
    T* xi = x + i * (int64_t)m;
    for (int j = 0; j < m; ++j) xi[j] /= T(1) + sigma.at(i * (int64_t)m + j) * alpha / lbd;
    frob_proj(xi, m, lbd);
  }
}

template <typename T>
__global__ void k_quadepi(int64_t N, int M, double alph, const T* __restrict__ shift,
                          double lbd, T* __restrict__ x) {
  GRID_STRIDE(i, N) {
    T* xi = x + i * (int64_t)(M + 1);
    quadepi_proj(xi, M, alph, shift ? shift + i * (int64_t)(M + 1) : nullptr, lbd);
  }
}

}  // namespace opyx

using namespace opyx;

// Projection onto the Frobenius lbd-ball of each group of M values, in
// place, recording the Jacobian of the map at x (L1NormsProj with
// jacobian=True and L12ProjJacobian.update, opymize/operators/proj.py:
// 206-226, :244-252): outside the ball n = x/|x| and s = lbd/|x|, inside
// n = 0 and s = 1, so that J v = s (v - <n, v> n) is the identity there.
// The arithmetic is that of norm_projection (proj.py:99-108): the
// reciprocal norm, then two scalings.
template <typename T>
__global__ void k_l1proj_jac(int64_t N, int M, T lbd, T* __restrict__ x, T* __restrict__ xn,
                             T* __restrict__ s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x) {
    T* g = x + i * M;
    T* nn = xn + i * M;
    T sq = T(0);
    for (int k = 0; k < M; ++k) sq += g[k] * g[k];
    const T nrm = sqrt(sq);
    if (nrm > lbd) {
      const T rec = T(1) / nrm;
      for (int k = 0; k < M; ++k) {
        nn[k] = g[k] * rec;
        g[k] = g[k] * rec * lbd;
      }
      s[i] = lbd * rec;
    } else {
      for (int k = 0; k < M; ++k) nn[k] = T(0);
      s[i] = T(1);
    }
  }
}

// y (+)= s_i (x_i - <n_i, x_i> n_i) per group (L12ProjJacobian._call_cpu,
// proj.py:254-276: y = n; y *= -<n, x>; y += x; y *= s).
template <typename T>
__global__ void k_l12_jac_apply(int64_t N, int M, const T* __restrict__ xn, const T* __restrict__ s,
                                const T* __restrict__ x, T* __restrict__ y, int add) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T* nn = xn + i * M;
    const T* xv = x + i * M;
    T d = T(0);
    for (int k = 0; k < M; ++k) d += nn[k] * xv[k];
    const T si = s[i];
    for (int k = 0; k < M; ++k) {
      const T v = (nn[k] * (-d) + xv[k]) * si;
      y[i * M + k] = add ? y[i * M + k] + v : v;
    }
  }
}

#define LAUNCH(kernel, n, ...)                                                  \
  do {                                                                          \
    if ((n) == 0) return OPYX_OK;                                               \
    OPYX_DISPATCH(dtype, T, (kernel<T><<<grid_for((n), 256), 256, 0,            \
                                         (cudaStream_t)stream>>>(__VA_ARGS__))); \
    return check_launch();                                                      \
  } while (0)

extern "C" {

int opyx_shiftscale(int dtype, int64_t n, const void* a_vec, double a, const void* b_vec,
                    double b, const void* shift_vec, double shift, const void* x, void* y,
                    int add, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return OPYX_ERR_ARG;
  LAUNCH(k_shiftscale, n, n, (const T*)a_vec, (T)a, (const T*)b_vec, (T)b,
         (const T*)shift_vec, (T)shift, (const T*)x, (T*)y, add);
}

int opyx_affine_prox(int dtype, int64_t n, const void* a_vec, double a, const void* c_vec,
                     double c, opyx_step tau, const void* x, void* y, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return OPYX_ERR_ARG;
  LAUNCH(k_affine_prox, n, n, (const T*)a_vec, (T)a, (const T*)c_vec, (T)c, StepT<T>(tau),
         (const T*)x, (T*)y);
}

int opyx_ssd_prox(int dtype, int64_t N, int C, const void* f, const double* vol,
                  const uint8_t* mask, opyx_step tau, const void* x, void* y, void* stream) {
  if (N < 0 || C < 1 || (N > 0 && (!f || !x || !y))) return OPYX_ERR_ARG;
  LAUNCH(k_ssd_prox, N * C, N, C, (const T*)f, vol, mask, StepT<T>(tau), (const T*)x, (T*)y);
}

int opyx_posproj(int dtype, int64_t n, const void* x, void* y, int add, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return OPYX_ERR_ARG;
  LAUNCH(k_posneg, n, n, 0, (const T*)x, (T*)y, add);
}

int opyx_negproj(int dtype, int64_t n, const void* x, void* y, int add, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return OPYX_ERR_ARG;
  LAUNCH(k_posneg, n, n, 1, (const T*)x, (T*)y, add);
}

int opyx_constrain(int dtype, int64_t N, int M, const uint8_t* mask, const void* c,
                   const void* x, void* y, int add, void* stream) {
  if (N < 0 || M < 1 || (N > 0 && (!mask || !c || !x || !y))) return OPYX_ERR_ARG;
  LAUNCH(k_constrain, N * M, N, M, mask, (const T*)c, (const T*)x, (T*)y, add);
}

int opyx_l1normsproj(int dtype, int64_t N, int M1, int M2, double lbd, int matrixnorm,
                     void* x, void* stream) {
  if (N < 0 || M1 < 1 || M2 < 1 || (N > 0 && !x)) return OPYX_ERR_ARG;
  if (matrixnorm != OPYX_NORM_FROBENIUS && matrixnorm != OPYX_NORM_SPECTRAL) return OPYX_ERR_ARG;
  if (matrixnorm == OPYX_NORM_SPECTRAL && M1 != 1 && M2 != 1 && M1 != 2 && M2 != 2)
    return OPYX_ERR_UNSUPPORTED;
  LAUNCH(k_l1proj, N, N, M1, M2, (T)lbd, matrixnorm == OPYX_NORM_SPECTRAL, (T*)x);
}

int opyx_l1normsproj_jac(int dtype, int64_t N, int M, double lbd, void* x, void* xn, void* s,
                         void* stream) {
  if (N < 0 || M < 1 || !(lbd > 0) || (N > 0 && (!x || !xn || !s))) return OPYX_ERR_ARG;
  LAUNCH(k_l1proj_jac, N, N, M, (T)lbd, (T*)x, (T*)xn, (T*)s);
}

int opyx_l12proj_jacobian(int dtype, int64_t N, int M, const void* xn, const void* s, const void* x,
                          void* y, int add, void* stream) {
  if (N < 0 || M < 1 || (N > 0 && (!xn || !s || !x || !y))) return OPYX_ERR_ARG;
  LAUNCH(k_l12_jac_apply, N, N, M, (const T*)xn, (const T*)s, (const T*)x, (T*)y, add);
}

int opyx_huber_conj_prox(int dtype, int64_t N, int m, double lbd, double alpha,
                         opyx_step sigma, void* x, void* stream) {
  if (N < 0 || m < 1 || !(lbd > 0) || alpha < 0 || (N > 0 && !x)) return OPYX_ERR_ARG;
  LAUNCH(k_huber_conj, N, N, m, (T)lbd, (T)alpha, StepT<T>(sigma), (T*)x);
}

int opyx_quadepiproj(int dtype, int64_t N, int M, double alph, const void* shift, double lbd,
                     void* x, void* stream) {
  if (N < 0 || M < 1 || M > OPYX_QUADEPI_MAX_M || !(alph > 0) || !(lbd > 0) || (N > 0 && !x))
    return OPYX_ERR_ARG;
  LAUNCH(k_quadepi, N, N, M, alph, (const T*)shift, lbd, (T*)x);
}

}  // extern "C"
