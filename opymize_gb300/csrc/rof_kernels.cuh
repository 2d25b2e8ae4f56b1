// Fused PDHG passes for ROF-type problems
//
//     min_x  G(x) + F(Ax),  G = SSD (0.5*sum_mask vol_k (x - f)^2 + shift),
//                           F = lbd*sum_i |(Ax)_i|_F  or its Huber smoothing,
//                           A = forward-difference gradient (Neumann).
//
// One PDHG iteration of the reference (opymize/solvers/pdhg.py:124-187) is
// two passes over HBM:
//
//   pass A (primal): x_{k+1} = prox_tauG(x_k - tau*A^T y_k)   (A^T y on the fly)
//                    xbar    = (1+theta)*x_{k+1} - theta*x_k
//   pass B (dual):   y_{k+1} = prox_sigmaF*(y_k + sigma*A xbar) (A xbar on the fly)
//
// A xbar equals the reference's overrelaxed (1+theta)*A x_{k+1} - theta*A x_k by
// linearity.  Adaptive steps add a third pass (R) that stores A^T y_{k+1} and
// reduces the primal residual; the last block of R applies the step rule on
// the device, so no iteration waits for the host.
//
// Layout (pixel-major, as the reference's Variables): x, xbar, f are (N, C),
// y is (N, D, C).  Threads map to pixels: threadIdx.x / blockIdx.x run along
// the contiguous last axis, blockIdx.y (grid-stride) over the flattened
// remaining axes, so every load and store of a warp is one contiguous run.
#pragma once

#include "common.cuh"
#include "prox_dev.cuh"

namespace opyx {
namespace rof {

struct Geo {
  int64_t N;          // pixels
  int64_t nl;         // length of the last (contiguous) axis
  int64_t rows;       // N / nl
  int64_t n[3];       // dims (n[0..D-1])
  int64_t s[3];       // strides in pixels
  double invh[3];
  double w[OPYX_ROF_MAX_C];
  double vol[OPYX_ROF_MAX_C];
  double lbd, huber, theta;
  int steps;
};

// Per-launch constants, by value.
template <typename T>
struct Args {
  T* x;
  T* xbar;
  T* y;
  const T* f;
  const uint8_t* mask;
  T* xgrad;
  T* gp;
  opyx_adaptive_state* st;
  double* partials;
  unsigned* ticket;
  opyx_rof_info* info;
  double tau, sigma;  // constant steps
};

// Coordinates of pixel (row r, column q): c[D-1] = q, the others from r.
template <int D>
OPYX_D void coords(const Geo& g, int64_t r, int64_t q, int64_t* c) {
  c[D - 1] = q;
  if (D == 2) c[0] = r;
  if (D == 3) { c[1] = r % g.n[1]; c[0] = r / g.n[1]; }
}

// Analytic diagonal preconditioners of the forward gradient
// (pdhg.py:191-204 with the rowwise l1 norms of diffopn):
//   sigma_{i,t,k} = 1/(2|w_k|/h_t) on inner rows, 0 on the far boundary;
//   tau_{i,k}     = 1/(|w_k| sum_t ([c_t < n_t-1] + [c_t > 0]) / h_t).
template <int D>
OPYX_D double precond_sigma(const Geo& g, const int64_t* c, int t, int k) {
  if (c[t] >= g.n[t] - 1) return 0.0;
  const double rs = 2.0 * fabs(g.w[k]) * g.invh[t];
  return rs > 2.220446049250313e-16 ? 1.0 / rs : 0.0;
}

template <int D>
OPYX_D double precond_tau(const Geo& g, const int64_t* c, int k) {
  double cs = 0.0;
#pragma unroll
  for (int t = 0; t < D; ++t)
    cs += fabs(g.w[k]) * g.invh[t] * (double)((c[t] < g.n[t] - 1) + (c[t] > 0));
  return cs > 2.220446049250313e-16 ? 1.0 / cs : 0.0;
}

// (A^T y)_i = w_k * sum_t (-y[i,t,k]/h_t [c_t < n_t-1] + y[i-s_t,t,k]/h_t [c_t > 0])
// (divergence, diff.cu:114-123).
template <typename T, int D, int C>
OPYX_D void div_at(const Geo& g, const T* __restrict__ y, int64_t i, const int64_t* c,
                   T (&out)[C]) {
#pragma unroll
  for (int k = 0; k < C; ++k) out[k] = T(0);
#pragma unroll
  for (int t = 0; t < D; ++t) {
    const T ih = (T)g.invh[t];
    if (c[t] < g.n[t] - 1) {
#pragma unroll
      for (int k = 0; k < C; ++k) out[k] -= y[(i * D + t) * C + k] * ih;
    }
    if (c[t] > 0) {
      const int64_t j = i - g.s[t];
#pragma unroll
      for (int k = 0; k < C; ++k) out[k] += y[(j * D + t) * C + k] * ih;
    }
  }
#pragma unroll
  for (int k = 0; k < C; ++k) out[k] *= (T)g.w[k];
}

// (A v)_{i,t,k} = w_k/h_t (v[i+s_t,k] - v[i,k]) if c_t < n_t-1 else 0
// (gradient, diff.cu:64-74).
template <typename T, int D, int C>
OPYX_D void grad_at(const Geo& g, const T* __restrict__ v, int64_t i, const int64_t* c,
                    T (&out)[D * C]) {
  T vi[C];
#pragma unroll
  for (int k = 0; k < C; ++k) vi[k] = v[i * C + k];
#pragma unroll
  for (int t = 0; t < D; ++t) {
    if (c[t] < g.n[t] - 1) {
      const int64_t j = i + g.s[t];
#pragma unroll
      for (int k = 0; k < C; ++k) out[t * C + k] = (T)(g.w[k] * g.invh[t]) * (v[j * C + k] - vi[k]);
    } else {
#pragma unroll
      for (int k = 0; k < C; ++k) out[t * C + k] = T(0);
    }
  }
}

// prox of sigma*F*: optional Huber shrink y/(1 + sigma*alpha/lbd), then the
// projection of the D*C group onto the Frobenius ball of radius lbd.
template <typename T, int M>
OPYX_D void fconj_prox(const Geo& g, T (&yv)[M], const T (&sig)[M]) {
  if (g.huber > 0) {
#pragma unroll
    for (int j = 0; j < M; ++j) yv[j] /= T(1) + sig[j] * (T)(g.huber / g.lbd);
  }
  frob_proj(yv, M, (T)g.lbd);
}

template <typename T>
OPYX_D T tau_const(const Args<T>& a, const Geo& g) {
  return g.steps == OPYX_STEPS_ADAPTIVE ? (T)__ldg(&a.st->tau) : (T)a.tau;
}
template <typename T>
OPYX_D T sigma_const(const Args<T>& a, const Geo& g) {
  return g.steps == OPYX_STEPS_ADAPTIVE ? (T)__ldg(&a.st->sigma) : (T)a.sigma;
}

// Grid-stride over rows (y) and columns (x): every (r, q) pixel is visited
// exactly once whatever the grid shape.
#define ROF_PIXEL_LOOP                                                         \
  for (int64_t r = blockIdx.y * (int64_t)blockDim.y + threadIdx.y; r < g.rows;   \
       r += (int64_t)gridDim.y * blockDim.y)                                    \
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < g.nl;   \
         q += (int64_t)gridDim.x * blockDim.x)

// ---------------------------------------------------------------- pass A
// ADAPT = 0: reads y (neighbours), x, f; writes x, xbar.
// ADAPT = 1: reads xgrad (stored A^T y_k), x, f; writes x, xbar and
//            gp = (x_k - x_{k+1})/tau - A^T y_k; reduces |gp|^2 into sums[1].
template <typename T, int D, int C, int ADAPT>
__global__ void __launch_bounds__(256) k_passA(Geo g, Args<T> a) {
  double acc = 0.0;
  const T tau_c = tau_const(a, g);
  ROF_PIXEL_LOOP {
    const int64_t i = r * g.nl + q;
    int64_t c[3];
    coords<D>(g, r, q, c);
    T div[C];
    if (ADAPT) {
#pragma unroll
      for (int k = 0; k < C; ++k) div[k] = a.xgrad[i * C + k];
    } else {
      div_at<T, D, C>(g, a.y, i, c, div);
    }
    const bool on = !a.mask || a.mask[i];
#pragma unroll
    for (int k = 0; k < C; ++k) {
      const T tau = g.steps == OPYX_STEPS_PRECOND ? (T)precond_tau<D>(g, c, k) : tau_c;
      const T xo = a.x[i * C + k];
      T xn = xo - tau * div[k];
      if (on) xn = ssd_prox_value(xn, a.f[i * C + k], tau * (T)g.vol[k]);
      a.x[i * C + k] = xn;
      a.xbar[i * C + k] = (T)(1.0 + g.theta) * xn - (T)g.theta * xo;
      if (ADAPT) {
        const T gpk = (xo - xn) / tau - div[k];
        a.gp[i * C + k] = gpk;
        acc += (double)gpk * (double)gpk;
      }
    }
  }
  if (ADAPT) {
    double vals[1] = {acc};
    const int ops[1] = {RED_SUM};
    opyx_adaptive_state* st = a.st;
    block_reduce_and_finish<1>(vals, ops, a.partials, a.ticket,
                               [&](double* tot) { st->sums[1] = tot[0]; });
  }
}

// ---------------------------------------------------------------- pass B
// ADAPT = 0: reads xbar (neighbours), y; writes y.
// ADAPT = 1: also reads x = x_{k+1} (neighbours) and reduces
//            |r_d|^2 = |(y_k - y_{k+1})/sigma - theta*A x_k + theta*A x_{k+1}|^2 and
//            |g_d|^2 = |(y_k - y_{k+1})/sigma - theta*A x_k + (theta+1)*A x_{k+1}|^2
//            into sums[2], sums[3]  (pdhg.py:157-162).
template <typename T, int D, int C, int ADAPT>
__global__ void __launch_bounds__(256) k_passB(Geo g, Args<T> a) {
  constexpr int M = D * C;
  double acc_r = 0.0, acc_g = 0.0;
  const T sig_c = sigma_const(a, g);
  ROF_PIXEL_LOOP {
    const int64_t i = r * g.nl + q;
    int64_t c[3];
    coords<D>(g, r, q, c);
    T gb[M], yv[M], yo[M], sig[M];
    grad_at<T, D, C>(g, a.xbar, i, c, gb);
#pragma unroll
    for (int t = 0; t < D; ++t) {
#pragma unroll
      for (int k = 0; k < C; ++k) {
        sig[t * C + k] = g.steps == OPYX_STEPS_PRECOND ? (T)precond_sigma<D>(g, c, t, k) : sig_c;
      }
    }
#pragma unroll
    for (int j = 0; j < M; ++j) {
      yo[j] = a.y[i * M + j];
      yv[j] = yo[j] + sig[j] * gb[j];
    }
    fconj_prox<T, M>(g, yv, sig);
#pragma unroll
    for (int j = 0; j < M; ++j) a.y[i * M + j] = yv[j];
    if (ADAPT) {
      T gn[M];
      grad_at<T, D, C>(g, a.x, i, c, gn);
      const T th = (T)g.theta;
#pragma unroll
      for (int j = 0; j < M; ++j) {
        // A x_k from xbar = (1+theta) x_{k+1} - theta x_k
        const T axk = ((T(1) + th) * gn[j] - gb[j]) / th;
        const T base = (yo[j] - yv[j]) / sig[j] - th * axk;
        const double rr = (double)(base + th * gn[j]);
        const double gg = (double)(base + (th + T(1)) * gn[j]);
        acc_r += rr * rr;
        acc_g += gg * gg;
      }
    }
  }
  if (ADAPT) {
    double vals[2] = {acc_r, acc_g};
    const int ops[2] = {RED_SUM, RED_SUM};
    opyx_adaptive_state* st = a.st;
    block_reduce_and_finish<2>(vals, ops, a.partials, a.ticket, [&](double* tot) {
      st->sums[2] = tot[0];
      st->sums[3] = tot[1];
    });
  }
}

// ---------------------------------------------------------------- pass R
// Adaptive only: xgrad = A^T y_{k+1}; RESID = 1 also reduces
// |r_p|^2 = |gp + A^T y_{k+1}|^2 into sums[0] and applies the step rule.
template <typename T, int D, int C, int RESID>
__global__ void __launch_bounds__(256) k_passR(Geo g, Args<T> a) {
  double acc = 0.0;
  ROF_PIXEL_LOOP {
    const int64_t i = r * g.nl + q;
    int64_t c[3];
    coords<D>(g, r, q, c);
    T div[C];
    div_at<T, D, C>(g, a.y, i, c, div);
#pragma unroll
    for (int k = 0; k < C; ++k) {
      a.xgrad[i * C + k] = div[k];
      if (RESID) {
        const double rp = (double)(a.gp[i * C + k] + div[k]);
        acc += rp * rp;
      }
    }
  }
  if (RESID) {
    double vals[1] = {acc};
    const int ops[1] = {RED_SUM};
    opyx_adaptive_state* st = a.st;
    block_reduce_and_finish<1>(vals, ops, a.partials, a.ticket, [&](double* tot) {
      st->sums[0] = tot[0];
      adaptive_rule(st);
    });
  }
}

// ---------------------------------------------------------------- gap
// objp = G(x) + F(Ax), objd = -G*(-A^T y) - F*(y) (pdhg.py:23-44) with FP64
// accumulation.  G*(-a) is expanded as sum_mask (a^2/(2 vol) - f a) - shift,
// the reference's conjugate SSD (functionals/quad.py:18-24) without the
// cancellation of its two large sums.
template <typename T, int D, int C>
__global__ void __launch_bounds__(256) k_gap(Geo g, Args<T> a, double ssd_shift) {
  constexpr int M = D * C;
  double sG = 0.0, sF = 0.0, sGs = 0.0, sFs = 0.0, inf = 0.0;
  ROF_PIXEL_LOOP {
    const int64_t i = r * g.nl + q;
    int64_t c[3];
    coords<D>(g, r, q, c);
    T ax[M], div[C];
    grad_at<T, D, C>(g, a.x, i, c, ax);
    div_at<T, D, C>(g, a.y, i, c, div);
    const bool on = !a.mask || a.mask[i];
    if (on) {
#pragma unroll
      for (int k = 0; k < C; ++k) {
        const double d = (double)a.x[i * C + k] - (double)a.f[i * C + k];
        sG += 0.5 * g.vol[k] * d * d;
        const double ak = (double)div[k];
        sGs += ak * ak / (2.0 * g.vol[k]) - (double)a.f[i * C + k] * ak;
      }
    }
    double n2 = 0.0, y2 = 0.0;
#pragma unroll
    for (int j = 0; j < M; ++j) {
      n2 += (double)ax[j] * (double)ax[j];
      const double yj = (double)a.y[i * M + j];
      y2 += yj * yj;
    }
    const double nrm = sqrt(n2);
    if (g.huber > 0)
      sF += nrm <= g.huber ? 0.5 * n2 / g.huber : nrm - 0.5 * g.huber;
    else
      sF += nrm;
    sFs += y2;
    inf = fmax(inf, sqrt(y2) - g.lbd);
  }
  double vals[5] = {sG, sF, sGs, sFs, inf};
  const int ops[5] = {RED_SUM, RED_SUM, RED_SUM, RED_SUM, RED_MAX};
  opyx_rof_info* info = a.info;
  const opyx_adaptive_state* st = a.st;
  block_reduce_and_finish<5>(vals, ops, a.partials, a.ticket, [&](double* tot) {
    const double Gx = tot[0] + ssd_shift;
    const double FAx = g.lbd * tot[1];
    const double Gs = tot[2] - ssd_shift;
    const double Fs = g.huber > 0 ? 0.5 * g.huber / g.lbd * tot[3] : 0.0;
    info->objp = Gx + FAx;
    info->objd = -Gs - Fs;
    info->infeasp = 0.0;
    info->infeasd = fmax(0.0, tot[4]);
    info->gap = info->objp - info->objd;
    info->relgap = info->gap / fmax(2.220446049250313e-16, fabs(info->objd));
    info->tau = st->tau;
    info->sigma = st->sigma;
    info->alpha = st->alpha;
    info->resp = st->resp;
    info->resd = st->resd;
    info->epsp = st->epsp;
    info->epsd = st->epsd;
  });
}

}  // namespace rof
}  // namespace opyx
