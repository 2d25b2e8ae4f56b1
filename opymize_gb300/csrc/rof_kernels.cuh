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

// Problem geometry and coefficients.  Everything a kernel touches per pixel
// is precomputed on the host in the iterate type T, so FP32 kernels do no
// FP64 arithmetic outside the gap reductions.
template <typename T>
struct Geo {
  int64_t N;          // pixels
  int64_t nl;         // length of the last (contiguous) axis
  int64_t rows;       // N / nl
  int64_t n[3];       // dims (n[0..D-1])
  int64_t s[3];       // strides in pixels
  T invh[3];                          // 1/h_t
  T coef[3][OPYX_ROF_MAX_C];          // w_k/h_t
  T absc[3][OPYX_ROF_MAX_C];          // |w_k|/h_t (preconditioner sums)
  T sig_pre[3][OPYX_ROF_MAX_C];       // h_t/(2|w_k|): sigma of inner rows
  T w[OPYX_ROF_MAX_C];
  T vol[OPYX_ROF_MAX_C];
  T half_rvol[OPYX_ROF_MAX_C];        // 1/(2 vol_k)
  T lbd, lbd2, hub_ratio, theta, theta1;
  T huber, half_huber, half_rhuber;   // alpha, alpha/2, 1/(2 alpha)
  // Preconditioned steps depend on a pixel only through how many neighbours
  // it has along each axis (0, 1 or 2): index cb = n_last + 3 n_row + 9 n_z.
  T tau_tab[27][OPYX_ROF_MAX_C];      // tau = 1/colsum
  T a_tab[27][OPYX_ROF_MAX_C];        // 1/(1 + tau vol): SSD prox scale
  T tv_tab[27][OPYX_ROF_MAX_C];       // tau vol
  T hub_pre[3][OPYX_ROF_MAX_C];       // 1/(1 + sigma_pre alpha/lbd) on inner rows
  double lbd_d, huber_d;
  double term_relgap, term_infeas;    // device-side stop test (term_mode)
  int steps;
  int term_mode;
  bool use_huber;
};

// Neighbour-count index of the preconditioner tables for a pixel with
// coordinates c (scalar kernels).
template <typename T, int D>
OPYX_D int combo_of(const Geo<T>& g, const int64_t* c) {
  int cb = (int)((c[D - 1] < g.n[D - 1] - 1) + (c[D - 1] > 0));
  if (D >= 2) cb += 3 * (int)((c[D - 2] < g.n[D - 2] - 1) + (c[D - 2] > 0));
  if (D == 3) cb += 9 * (int)((c[0] < g.n[0] - 1) + (c[0] > 0));
  return cb;
}

// Primal step coefficients for constant / adaptive steps, computed once per
// thread: tau, 1/(1 + tau vol_k), tau vol_k.
template <typename T, int C>
struct PrimalCoefs {
  T tau, a[C], tv[C];
  OPYX_D PrimalCoefs(const Geo<T>& g, T t) {
    tau = t;
#pragma unroll
    for (int k = 0; k < C; ++k) {
      tv[k] = t * g.vol[k];
      a[k] = T(1) / (T(1) + tv[k]);
    }
  }
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
  T* x2;   // single-sweep iterations: targets of x and y (ping-pong)
  T* y2;
  opyx_adaptive_state* st;
  double* partials;
  unsigned* ticket;
  opyx_rof_info* info;
  double tau, sigma;  // constant steps
};

// Every fused kernel returns at once once the stop test has passed, so a
// host may queue iterations beyond its next check without changing the
// result.  The flag is written only by the last block of a gap kernel, never
// while another kernel of the same solve runs, so all threads of a launch
// read the same value.
template <typename T>
OPYX_D bool stopped(const Args<T>& a) {
  return a.info->done != 0.0;
}

// Objectives of the gap kernels from the block-reduced sums
// tot = {sum G-terms, sum |Ax|, sum G*-terms, sum |y|^2, max(|y| - lbd)}
// (pdhg.py:23-44), the step state, the check counter and the stop test of
// the reference's solve loop (pdhg.py:290-305).
template <typename T>
OPYX_D void write_info(const Geo<T>& g, const Args<T>& a, const double* tot, double ssd_shift) {
  opyx_rof_info* info = a.info;
  const opyx_adaptive_state* st = a.st;
  const double Gx = tot[0] + ssd_shift;
  const double FAx = g.lbd_d * tot[1];
  const double Gs = tot[2] - ssd_shift;
  const double Fs = g.use_huber ? 0.5 * g.huber_d / g.lbd_d * tot[3] : 0.0;
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
  info->checks += 1.0;
  bool stop = false;
  if (g.term_mode == 1)
    stop = fabs(info->relgap) < g.term_relgap &&
           fmax(info->infeasp, info->infeasd) < g.term_infeas;
  else if (g.term_mode == 2)
    stop = st->resp < st->epsp && st->resd < st->epsd;
  if (stop) info->done = 1.0;
}

// Coordinates of pixel (row r, column q): c[D-1] = q, the others from r.
template <typename T, int D>
OPYX_D void coords(const Geo<T>& g, int64_t r, int64_t q, int64_t* c) {
  c[D - 1] = q;
  if (D == 2) c[0] = r;
  if (D == 3) { c[1] = r % g.n[1]; c[0] = r / g.n[1]; }
}

// Analytic diagonal preconditioners of the forward gradient
// (pdhg.py:191-204 with the rowwise l1 norms of diffopn):
//   sigma_{i,t,k} = 1/(2|w_k|/h_t) on inner rows, 0 on the far boundary;
//   tau_{i,k}     = 1/(sum_t |w_k|/h_t ([c_t < n_t-1] + [c_t > 0])).
template <typename T, int D>
OPYX_D T precond_sigma(const Geo<T>& g, const int64_t* c, int t, int k) {
  return c[t] < g.n[t] - 1 ? g.sig_pre[t][k] : T(0);
}

template <typename T, int D>
OPYX_D T precond_tau(const Geo<T>& g, const int64_t* c, int k) {
  T cs = T(0);
#pragma unroll
  for (int t = 0; t < D; ++t)
    cs += g.absc[t][k] * (T)((c[t] < g.n[t] - 1) + (c[t] > 0));
  return cs > T(2.220446049250313e-16) ? T(1) / cs : T(0);
}

// (A^T y)_i = w_k * sum_t (-y[i,t,k]/h_t [c_t < n_t-1] + y[i-s_t,t,k]/h_t [c_t > 0])
// (divergence, diff.cu:114-123).
template <typename T, int D, int C>
OPYX_D void div_at(const Geo<T>& g, const T* __restrict__ y, int64_t i, const int64_t* c,
                   T (&out)[C]) {
#pragma unroll
  for (int k = 0; k < C; ++k) out[k] = T(0);
#pragma unroll
  for (int t = 0; t < D; ++t) {
    const T ih = g.invh[t];
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
  for (int k = 0; k < C; ++k) out[k] *= g.w[k];
}

// (A v)_{i,t,k} = w_k/h_t (v[i+s_t,k] - v[i,k]) if c_t < n_t-1 else 0
// (gradient, diff.cu:64-74).
template <typename T, int D, int C>
OPYX_D void grad_at(const Geo<T>& g, const T* __restrict__ v, int64_t i, const int64_t* c,
                    T (&out)[D * C]) {
  T vi[C];
#pragma unroll
  for (int k = 0; k < C; ++k) vi[k] = v[i * C + k];
#pragma unroll
  for (int t = 0; t < D; ++t) {
    if (c[t] < g.n[t] - 1) {
      const int64_t j = i + g.s[t];
#pragma unroll
      for (int k = 0; k < C; ++k) out[t * C + k] = g.coef[t][k] * (v[j * C + k] - vi[k]);
    } else {
#pragma unroll
      for (int k = 0; k < C; ++k) out[t * C + k] = T(0);
    }
  }
}

// prox of sigma*F*: optional Huber shrink y/(1 + sigma*alpha/lbd), then the
// projection of the D*C group onto the Frobenius ball of radius lbd.
// hf[j] = 1/(1 + sigma_j alpha/lbd), precomputed (Geo::hub_pre, or once per
// thread for constant steps).
template <typename T, int M>
OPYX_D void fconj_prox(const Geo<T>& g, T (&yv)[M], const T (&hf)[M]) {
  if (g.use_huber) {
#pragma unroll
    for (int j = 0; j < M; ++j) yv[j] *= hf[j];
  }
  T nrm = T(0);
#pragma unroll
  for (int j = 0; j < M; ++j) nrm += yv[j] * yv[j];
  if (nrm > g.lbd2) {
    const T sc = g.lbd / sqrt(nrm);
#pragma unroll
    for (int j = 0; j < M; ++j) yv[j] *= sc;
  }
}

template <typename T>
OPYX_D T tau_const(const Args<T>& a, const Geo<T>& g) {
  return g.steps == OPYX_STEPS_ADAPTIVE ? (T)__ldg(&a.st->tau) : (T)a.tau;
}
template <typename T>
OPYX_D T sigma_const(const Args<T>& a, const Geo<T>& g) {
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
__global__ void __launch_bounds__(256) k_passA(Geo<T> g, Args<T> a) {
  if (stopped(a)) return;
  double acc = 0.0;
  const PrimalCoefs<T, C> pc(g, tau_const(a, g));
  const bool pre = g.steps == OPYX_STEPS_PRECOND;
  ROF_PIXEL_LOOP {
    const int64_t i = r * g.nl + q;
    int64_t c[3];
    coords<T, D>(g, r, q, c);
    T div[C];
    if (ADAPT) {
#pragma unroll
      for (int k = 0; k < C; ++k) div[k] = a.xgrad[i * C + k];
    } else {
      div_at<T, D, C>(g, a.y, i, c, div);
    }
    const bool on = !a.mask || a.mask[i];
    const int cb = pre ? combo_of<T, D>(g, c) : 0;
#pragma unroll
    for (int k = 0; k < C; ++k) {
      const T tau = pre ? g.tau_tab[cb][k] : pc.tau;
      const T xo = a.x[i * C + k];
      T xn = xo - tau * div[k];
      if (on) xn = (pre ? g.a_tab[cb][k] : pc.a[k]) *
                   (xn + (pre ? g.tv_tab[cb][k] : pc.tv[k]) * a.f[i * C + k]);
      a.x[i * C + k] = xn;
      a.xbar[i * C + k] = g.theta1 * xn - g.theta * xo;
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
__global__ void __launch_bounds__(256) k_passB(Geo<T> g, Args<T> a) {
  if (stopped(a)) return;
  constexpr int M = D * C;
  double acc_r = 0.0, acc_g = 0.0;
  const T sig_c = sigma_const(a, g);
  const T hub_c = T(1) / (T(1) + sig_c * g.hub_ratio);
  const bool pre = g.steps == OPYX_STEPS_PRECOND;
  ROF_PIXEL_LOOP {
    const int64_t i = r * g.nl + q;
    int64_t c[3];
    coords<T, D>(g, r, q, c);
    T gb[M], yv[M], yo[M], sig[M], hf[M];
    grad_at<T, D, C>(g, a.xbar, i, c, gb);
#pragma unroll
    for (int t = 0; t < D; ++t) {
      const bool inner = c[t] < g.n[t] - 1;
#pragma unroll
      for (int k = 0; k < C; ++k) {
        sig[t * C + k] = pre ? (inner ? g.sig_pre[t][k] : T(0)) : sig_c;
        hf[t * C + k] = pre ? (inner ? g.hub_pre[t][k] : T(1)) : hub_c;
      }
    }
#pragma unroll
    for (int j = 0; j < M; ++j) {
      yo[j] = a.y[i * M + j];
      yv[j] = yo[j] + sig[j] * gb[j];
    }
    fconj_prox<T, M>(g, yv, hf);
#pragma unroll
    for (int j = 0; j < M; ++j) a.y[i * M + j] = yv[j];
    if (ADAPT) {
      T gn[M];
      grad_at<T, D, C>(g, a.x, i, c, gn);
      const T th = g.theta;
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
__global__ void __launch_bounds__(256) k_passR(Geo<T> g, Args<T> a) {
  if (stopped(a)) return;
  double acc = 0.0;
  ROF_PIXEL_LOOP {
    const int64_t i = r * g.nl + q;
    int64_t c[3];
    coords<T, D>(g, r, q, c);
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
__global__ void __launch_bounds__(256) k_gap(Geo<T> g, Args<T> a, double ssd_shift) {
  if (stopped(a)) return;
  constexpr int M = D * C;
  double sG = 0.0, sF = 0.0, sGs = 0.0, sFs = 0.0, inf = 0.0;
  ROF_PIXEL_LOOP {
    const int64_t i = r * g.nl + q;
    int64_t c[3];
    coords<T, D>(g, r, q, c);
    T ax[M], div[C];
    grad_at<T, D, C>(g, a.x, i, c, ax);
    div_at<T, D, C>(g, a.y, i, c, div);
    const bool on = !a.mask || a.mask[i];
    if (on) {
      T pg = T(0), ps = T(0);
#pragma unroll
      for (int k = 0; k < C; ++k) {
        const T fk = a.f[i * C + k];
        const T d = a.x[i * C + k] - fk;
        pg += g.vol[k] * d * d;
        ps += div[k] * div[k] * g.half_rvol[k] - fk * div[k];
      }
      sG += 0.5 * (double)pg;
      sGs += (double)ps;
    }
    T n2 = T(0), y2 = T(0);
#pragma unroll
    for (int j = 0; j < M; ++j) {
      n2 += ax[j] * ax[j];
      const T yj = a.y[i * M + j];
      y2 += yj * yj;
    }
    const T nrm = sqrt(n2);
    T fv;
    if (g.use_huber)
      fv = nrm <= g.huber ? n2 * g.half_rhuber : nrm - g.half_huber;
    else
      fv = nrm;
    sF += (double)fv;
    sFs += (double)y2;
    inf = fmax(inf, (double)(sqrt(y2) - g.lbd));
  }
  double vals[5] = {sG, sF, sGs, sFs, inf};
  const int ops[5] = {RED_SUM, RED_SUM, RED_SUM, RED_SUM, RED_MAX};
  block_reduce_and_finish<5>(vals, ops, a.partials, a.ticket, [&](double* tot) {
    write_info(g, a, tot, ssd_shift);
  });
}

}  // namespace rof
}  // namespace opyx
