// Values and infeasibilities of the functionals on the PDHG path, reduced in
// FP64 on the device -- the ingredients of the primal-dual gap
// (opymize/solvers/pdhg.py:23-44), which the reference evaluates in numpy on
// the host after copying every iterate back.
#include "common.cuh"
#include "prox_dev.cuh"

namespace opyx {

constexpr int kFctThreads = 256;
constexpr int kFctBlocks = 1024;

// singular values of a per-group matrix with one side of length 2, read in
// the (M2 x M1) row-major order of spectral_proj_2xm
template <typename T>
OPYX_D void sv2(const T* xi, int M1, int M2, double* smax, double* smin) {
  const bool pairs = M1 <= M2;
  const int R = pairs ? M2 : M1;
  const int st1 = pairs ? 2 : 1, st2 = pairs ? 1 : M1;
  double C11 = 0, C12 = 0, C22 = 0;
  for (int r = 0; r < R; ++r) {
    const double a = (double)xi[r * st1], b = (double)xi[r * st1 + st2];
    C11 += a * a;
    C12 += a * b;
    C22 += b * b;
  }
  const double tr = C11 + C22;
  const double d = sqrt(fmax(0.0, 0.25 * tr * tr - (C11 * C22 - C12 * C12)));
  *smax = sqrt(fmax(0.0, 0.5 * tr + d));
  *smin = sqrt(fmax(0.0, 0.5 * tr - d));
}

template <typename T>
OPYX_D double group_norm(const T* xi, int M1, int M2, int spectral, int nuclear) {
  if ((spectral || nuclear) && M1 != 1 && M2 != 1) {
    double smax, smin;
    sv2(xi, M1, M2, &smax, &smin);
    return nuclear ? smax + smin : smax;
  }
  double s = 0.0;
  for (int j = 0; j < M1 * M2; ++j) s += (double)xi[j] * (double)xi[j];
  return sqrt(s);
}

template <typename T>
__global__ void __launch_bounds__(kFctThreads)
k_fct_eval(opyx_fct f, const T* __restrict__ x, double* out, double* partials, unsigned* ticket) {
  const int m = f.m1 * f.m2;
  const T* v0 = (const T*)f.v0;
  const T* v1 = (const T*)f.v1;
  double val = 0.0, infA = 0.0, infB = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < f.ngroups;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T* xi = x + i * m;
    switch (f.kind) {
      case OPYX_FCT_SSD: {
        if (f.mask && !f.mask[i]) break;
        for (int k = 0; k < m; ++k) {
          const double d = (double)xi[k] - (double)v0[i * m + k];
          val += 0.5 * (f.vol ? f.vol[k] : 1.0) * d * d;
        }
        break;
      }
      case OPYX_FCT_L1NORMS:
        val += group_norm(xi, f.m1, f.m2, 0, f.matrixnorm == OPYX_NORM_SPECTRAL);
        break;
      case OPYX_FCT_L1NORMS_CONJ:
        infA = fmax(infA, group_norm(xi, f.m1, f.m2, f.matrixnorm == OPYX_NORM_SPECTRAL, 0) - f.lbd);
        break;
      case OPYX_FCT_HUBER: {
        const double r = group_norm(xi, f.m1, f.m2, 0, 0);
        val += r <= f.alpha ? 0.5 * r * r / f.alpha : r - 0.5 * f.alpha;
        break;
      }
      case OPYX_FCT_HUBER_CONJ: {
        const double r = group_norm(xi, f.m1, f.m2, 0, 0);
        val += r * r;
        infA = fmax(infA, r - f.lbd);
        break;
      }
      case OPYX_FCT_QUADEPI_IND: {
        double fx = v1 ? (double)v1[i] : 0.0;
        for (int k = 0; k < m - 1; ++k) {
          const double xk = (double)xi[k];
          fx += 0.5 * f.a * xk * xk + (v0 ? (double)v0[i * (m - 1) + k] : 0.0) * xk;
        }
        infA = fmax(infA, fx - (double)xi[m - 1]);
        break;
      }
      case OPYX_FCT_QUADEPI_SUPP: {
        const double xl = (double)xi[m - 1];
        if (xl < -1e-8) {
          const double x2 = -xl;
          double s = 0.0;
          for (int k = 0; k < m - 1; ++k) {
            const double xk = (double)xi[k];
            s += 0.5 * f.a * xk * xk / x2 + (v0 ? (double)v0[i * (m - 1) + k] : 0.0) * xk;
          }
          val += s + x2 * (v1 ? (double)v1[i] : 0.0);
        } else {
          infA = fmax(infA, fabs(xl));
        }
        break;
      }
      case OPYX_FCT_HUBER_PERSP: {
        double n2 = 0.0;
        for (int k = 0; k < m - 1; ++k) n2 += (double)xi[k] * (double)xi[k];
        const double n = sqrt(n2), x2 = -(double)xi[m - 1];
        if (n < f.alpha * x2) val += 0.5 / f.alpha * n2 / x2;
        else if (x2 > -1e-4) val += n - x2 * f.alpha / 2;
        infA = fmax(infA, -x2);
        break;
      }
      case OPYX_FCT_TRUNCQUAD_IND: {
        double n2 = 0.0;
        for (int k = 0; k < m - 1; ++k) n2 += (double)xi[k] * (double)xi[k];
        const double n = sqrt(n2);
        infA = fmax(infA, n - f.lbd);
        const double mn = fmin(f.lbd, n);
        infB = fmax(infB, 0.5 * f.alpha * mn * mn - (double)xi[m - 1]);
        break;
      }
      case OPYX_FCT_POSITIVITY:
        for (int k = 0; k < m; ++k) infA = fmax(infA, -(double)xi[k]);
        break;
      case OPYX_FCT_NEGATIVITY:
        for (int k = 0; k < m; ++k) infA = fmax(infA, (double)xi[k]);
        break;
      case OPYX_FCT_AFFINE:
        for (int k = 0; k < m; ++k)
          val += (v0 ? (double)v0[i * m + k] : f.scalar1) * (double)xi[k];
        break;
      case OPYX_FCT_INDICATOR:
        for (int k = 0; k < m; ++k)
          infA = fmax(infA, fabs((double)xi[k] - (v0 ? (double)v0[i * m + k] : f.scalar1)));
        break;
      case OPYX_FCT_CONSTRAIN:
        if (f.mask[i])
          for (int k = 0; k < m; ++k)
            infA = fmax(infA, fabs((double)xi[k] - (double)v0[i * m + k]));
        break;
      case OPYX_FCT_MASKED_AFFINE:
        if (f.mask[i]) {
          for (int k = 0; k < m; ++k) val += (double)v0[i * m + k] * (double)xi[k];
        } else {
          for (int k = 0; k < m; ++k) infA = fmax(infA, fabs((double)xi[k]));
        }
        break;
      default:
        break;
    }
  }
  double vals[3] = {val, infA, infB};
  const int ops[3] = {RED_SUM, RED_MAX, RED_MAX};
  block_reduce_and_finish<3>(vals, ops, partials, ticket, [&](double* tot) {
    double v = tot[0], inf = fmax(0.0, tot[1]);
    switch (f.kind) {
      case OPYX_FCT_SSD: v += f.scalar0; break;
      case OPYX_FCT_L1NORMS: case OPYX_FCT_HUBER: v *= f.lbd; break;
      case OPYX_FCT_L1NORMS_CONJ: v = 0.0; break;
      case OPYX_FCT_HUBER_CONJ: v *= 0.5 * f.alpha / f.lbd; break;
      case OPYX_FCT_HUBER_PERSP: v *= f.lbd; break;
      case OPYX_FCT_TRUNCQUAD_IND: inf += fmax(0.0, tot[2]); break;
      case OPYX_FCT_AFFINE: v += f.scalar0; break;
      case OPYX_FCT_INDICATOR: v = f.scalar0; break;
      default: break;
    }
    out[0] = v;
    out[1] = inf;
  });
}

}  // namespace opyx

using namespace opyx;

extern "C" {

int opyx_fct_eval(const opyx_fct* f, int dtype, const void* x, double* out, void* ws,
                  void* stream) {
  if (!f || !out || !ws || f->ngroups < 0 || f->m1 < 1 || f->m2 < 1) return OPYX_ERR_ARG;
  if (f->ngroups > 0 && !x) return OPYX_ERR_ARG;
  if (f->kind < OPYX_FCT_SSD || f->kind > OPYX_FCT_MASKED_AFFINE) return OPYX_ERR_ARG;
  if ((f->kind == OPYX_FCT_SSD || f->kind == OPYX_FCT_CONSTRAIN ||
       f->kind == OPYX_FCT_MASKED_AFFINE) && !f->v0) return OPYX_ERR_ARG;
  if ((f->kind == OPYX_FCT_CONSTRAIN || f->kind == OPYX_FCT_MASKED_AFFINE) && !f->mask)
    return OPYX_ERR_ARG;
  if (((uintptr_t)ws) & 7) return OPYX_ERR_WORKSPACE;
  double* partials = (double*)ws;
  unsigned* ticket = (unsigned*)((char*)ws + (size_t)kFctBlocks * 8 * sizeof(double));
  unsigned g = grid_for(f->ngroups > 0 ? f->ngroups : 1, kFctThreads, 4);
  if (g > (unsigned)kFctBlocks) g = kFctBlocks;
  OPYX_DISPATCH(dtype, T, (k_fct_eval<T><<<g, kFctThreads, 0, (cudaStream_t)stream>>>(
                              *f, (const T*)x, out, partials, ticket)));
  return check_launch();
}

}  // extern "C"
