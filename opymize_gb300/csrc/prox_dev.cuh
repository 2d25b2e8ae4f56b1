// Device-side prox building blocks shared by the generic kernels (prox.cu)
// and the fused PDHG passes.
#pragma once

#include "common.cuh"

#define OPYX_QUADEPI_MAX_M 32

namespace opyx {

// Step size: per-element vector, device scalar (adaptive) or constant.
template <typename T>
struct StepT {
  const T* vec;
  const double* dev;
  T value;
  __host__ StepT(const opyx_step& s) : vec((const T*)s.vec), dev(s.dev), value((T)s.value) {}
  OPYX_D T at(int64_t i) const { return vec ? vec[i] : (dev ? (T)__ldg(dev) : value); }
  // Read a device scalar once per thread: the conversion from FP64 is an
  // FP64-pipe instruction, far too slow on GB300 to repeat per element.
  OPYX_D void load() {
    if (!vec && dev) {
      value = (T)__ldg(dev);
      dev = nullptr;
    }
  }
};

// SSD prox of one value with t = tau*vol: a*(x + t*f), a = 1/(1 + t)
// (ShiftScaleOp with the arrays of SSD.prox, functionals/quad.py:45-55).
template <typename T>
OPYX_D T ssd_prox_value(T x, T f, T t) {
  const T a = T(1) / (T(1) + t);
  return a * (x + t * f);
}

// Projection of m values onto the Frobenius ball of radius lbd
// (operators/proj.cu:34-44).
template <typename T>
OPYX_D void frob_proj(T* xi, int m, T lbd) {
  T nrm = T(0);
  for (int j = 0; j < m; ++j) nrm += xi[j] * xi[j];
  if (nrm > lbd * lbd) {
    const T s = lbd / sqrt(nrm);
    for (int j = 0; j < m; ++j) xi[j] *= s;
  }
}

// Projection onto the spectral-norm ball of a per-pixel matrix with one side
// of length 2 (operators/proj.cu:45-105).  The buffer is read as the
// (M2 x M1) row-major matrix -- the (D, C) memory order of the gradient
// output when M = (C, D) -- i.e. as R rows of 2 values: (x[2r], x[2r+1]) for
// M1 == 2, or (x[r], x[M1+r]) for M2 == 2.  Eigen-decomposition of the 2x2
// Gram matrix in closed form; singular values are clipped at lbd.
template <typename T>
OPYX_D void spectral_proj_2xm(T* xi, int M1, int M2, T lbd) {
  const bool pairs = M1 <= M2;            // M1 == 2
  const int R = pairs ? M2 : M1;
  const int st1 = pairs ? 2 : 1, st2 = pairs ? 1 : M1;
  T C11 = 0, C12 = 0, C22 = 0;
  for (int r = 0; r < R; ++r) {
    const T a = xi[r * st1], b = xi[r * st1 + st2];
    C11 += a * a;
    C12 += a * b;
    C22 += b * b;
  }
  const T tr = C11 + C22;
  const T d = sqrt(fmax(T(0), T(0.25) * tr * tr - (C11 * C22 - C12 * C12)));
  const T lmax = fmax(T(0), T(0.5) * tr + d);
  const T lmin = fmax(T(0), T(0.5) * tr - d);
  const T smax = sqrt(lmax), smin = sqrt(lmin);
  if (!(smax > lbd)) return;
  T V11, V12, V21, V22;
  if (C12 == T(0)) {
    if (C11 >= C22) { V11 = 1; V12 = 0; V21 = 0; V22 = 1; }
    else { V11 = 0; V12 = 1; V21 = 1; V22 = 0; }
  } else {
    V11 = C12; V12 = C12;
    V21 = lmax - C11; V22 = lmin - C11;
    T n1 = hypot(V11, V21), n2 = hypot(V12, V22);
    V11 /= n1; V21 /= n1; V12 /= n2; V22 /= n2;
  }
  const T s1 = fmin(smax, lbd) / smax;
  const T s2 = smin > T(0) ? fmin(smin, lbd) / smin : T(0);
  const T M11 = s1 * V11 * V11 + s2 * V12 * V12;
  const T M12 = s1 * V11 * V21 + s2 * V12 * V22;
  const T M21 = s1 * V21 * V11 + s2 * V22 * V12;
  const T M22 = s1 * V21 * V21 + s2 * V22 * V22;
  for (int r = 0; r < R; ++r) {
    const T a = xi[r * st1], b = xi[r * st1 + st2];
    xi[r * st1] = a * M11 + b * M21;
    xi[r * st1 + st2] = a * M12 + b * M22;
  }
}

// Real root of x^3 + a x + b = 0 in FP64 (operators/proj.cu:111-139):
// cbrt(-b) for a == 0, the trigonometric form when Q^3 + R^2 <= 0, Cardano
// otherwise.  The acos argument is clipped to [-1, 1] so that rounding at
// Q^3 + R^2 ~ 0 cannot produce NaN.
OPYX_D double solve_reduced_monic_cubic(double a, double b) {
  if (a == 0.0) return b == 0.0 ? 0.0 : cbrt(-b);
  if (b == 0.0 && a > 0.0) return 0.0;
  const double Q = a / 3.0, R = -b / 2.0;
  const double Q3 = Q * Q * Q;
  const double D = Q3 + R * R;
  if (D <= 0.0) {
    const double c = fmin(1.0, fmax(-1.0, R / sqrt(-Q3)));
    return 2.0 * sqrt(-Q) * cos(acos(c) / 3.0);
  }
  double AD = cbrt(fabs(R) + sqrt(D));
  if (R < 0.0) AD = -AD;
  return AD - Q / AD;
}

// Projection of (x1, x2) in R^M x R onto epi(0.5*alph*|x1 - s1|^2 + s2),
// truncated at |x1 - s1| <= lbd when lbd is finite (operators/proj.cu:141-219).
// Computed in FP64 whatever T is.
template <typename T>
OPYX_D void quadepi_proj(T* xi, int M, double alph, const T* shift, double lbd) {
  double v[OPYX_QUADEPI_MAX_M + 1];
  for (int j = 0; j <= M; ++j) v[j] = (double)xi[j] - (shift ? (double)shift[j] : 0.0);
  double& x2 = v[M];
  double nsq = 0.0;
  for (int j = 0; j < M; ++j) nsq += v[j] * v[j];
  if (nsq > 0.0) {
    double n = sqrt(nsq);
    bool done = false;
    if (isfinite(lbd)) {
      const double l = -n / (lbd * alph) + 0.5 * alph * lbd * lbd + 1.0 / alph;
      if (l <= x2) {
        if (n > lbd) {
          const double s = lbd / n;
          for (int j = 0; j < M; ++j) v[j] *= s;
          const double l2 = 0.5 * alph * lbd * lbd;
          if (l2 > x2) x2 = l2;
        }
        done = true;
      }
    }
    if (!done && 0.5 * alph * nsq > x2) {
      const double l = 2.0 / (alph * alph);
      const double yn = solve_reduced_monic_cubic(l * (1.0 - x2 * alph), -l * n);
      const double s = yn / n;
      for (int j = 0; j < M; ++j) v[j] *= s;
      x2 = 0.5 * alph * yn * yn;
    }
  } else if (x2 < 0.0) {
    x2 = 0.0;
  }
  for (int j = 0; j <= M; ++j) xi[j] = (T)(v[j] + (shift ? (double)shift[j] : 0.0));
}

// Adaptive step rule (opymize/solvers/pdhg.py:156-183) applied to the
// squared residual norms accumulated in st->sums, which it then clears.
OPYX_D void adaptive_rule(opyx_adaptive_state* st) {
  const double resp = sqrt(st->sums[0]), gp = sqrt(st->sums[1]);
  const double resd = sqrt(st->sums[2]), gd = sqrt(st->sums[3]);
  const double epsp = sqrt(st->xsize) * st->eps[0] + st->eps[1] * gp;
  const double epsd = sqrt(st->ysize) * st->eps[2] + st->eps[3] * gd;
  const double scale = epsp / epsd;
  if (resp > scale * resd * st->Delta) {
    st->tau /= 1.0 - st->alpha;
    st->sigma *= 1.0 - st->alpha;
    st->alpha *= st->eta;
  }
  if (resp < scale * resd / st->Delta) {
    st->tau *= 1.0 - st->alpha;
    st->sigma /= 1.0 - st->alpha;
    st->alpha *= st->eta;
  }
  st->resp = resp;
  st->resd = resd;
  st->epsp = epsp;
  st->epsd = epsd;
  for (int j = 0; j < 4; ++j) st->sums[j] = 0.0;
}

}  // namespace opyx
