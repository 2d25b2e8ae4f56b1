// Fused PDHG iteration of the sublabel-lifted scalar model (the block system
// that opymize_gb300/tools/lifting.py assembles from the reference's own
// operators), in two passes over HBM instead of the generic path's ~22
// operator launches per iteration.
//
//   primal x = (u [N, L], gamma [N], mu [L-1, N, 2])
//   dual   y = (q [N, L], e [N], p [N, 2], s [N], z [L-1, N, 2])
//   A x    = (u + IndexedMultAdj(mu), <t, u> - gamma, grad gamma, <1, u>, mu)
//   G      = PositivityFct(u) + 0(gamma) + 0(mu)
//   F*     = 0 (q), 0 (e), indicator |p_i| <= lbd, <1, s>, EpigraphInd (z)
//
// The reference iterates such a model with its generic operators and
// kernels (PDHG.iteration_step, opymize/solvers/pdhg.py:124-187, over
// BlockOp / IndexedMultAdj / MatrixMultR / ScaleOp / GradientOp and the
// prox operators of the functionals above).  Here:
//
//   pass A (one thread per pixel): A^T y_k at the pixel (only the gamma row
//     is a stencil: -div p needs p of the left and upper neighbours),
//     x_{k+1} = prox_tauG(x_k - tau A^T y_k), xbar = (1 + theta) x_{k+1} -
//     theta x_k; writes x_{k+1} and xbar.
//   pass B: A xbar at the pixel (grad gammabar needs the right and lower
//     neighbours), y_{k+1} = prox_sigmaF*(y_k + sigma A xbar): q, e unchanged
//     by the prox, p projected onto the lbd-ball, s - sigma, and every
//     interval's (slope, offset) pair z projected onto its epigraph by the
//     direct one-dimensional method (epi1_dev.cuh).
//
// y_k + sigma A xbar equals the reference's y_k + sigma ((1 + theta) A x_{k+1}
// - theta A x_k) up to rounding.  Steps: preconditioned (per label, per
// interval and per component the same for every pixel; gamma's tau and p's
// sigma depend on the pixel's neighbours and are read per pixel) or
// constant.
#include "common.cuh"
#include "epi1_dev.cuh"
#include "prox_dev.cuh"

#define SUB_GRID_STRIDE(i, n)                                                         \
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n);          \
       i += (int64_t)gridDim.x * blockDim.x)

namespace opyx {
namespace sub {

constexpr int kLmax = 32;
constexpr int kThreads = 128;

template <typename T>
struct Args {
  int64_t N, H, W;
  int L, nsub;                     // labels; points per interval (<= 16)
  const T* xk;                     // x_k
  T* xkp1;                         // x_{k+1}
  T* xbar;
  const T* yk;
  T* ykp1;
  T t[kLmax];                      // label positions (MatrixMultR into e)
  T B[kLmax - 1][2][2];            // IndexedMult coefficients B[j][m][k], P[j] = (j, j + 1)
  T tau_u[kLmax], tau_mu[kLmax - 1][2];
  T sig_q[kLmax], sig_z[kLmax - 1][2];
  T sig_e, sig_s;
  const T* tau_g;                  // per pixel (N), or NULL: tau_g0
  const T* sig_p;                  // per pixel (N, 2), or NULL: sig_p0
  T tau_g0, sig_p0;
  T lbd, theta;
  const T* v;                      // (npoints,) sample points
  const T* bt;                     // (npoints, N) the data term at the points
  const uint8_t* It;               // (npoints, N) point masks, or NULL (all set)
  const int64_t* J;                // (L - 1, nsub) points of every interval
  int sorted;                      // perm orders each interval's points by increasing,
  uint8_t perm[kLmax - 1][16];     // distinct v (the projection then skips its sort)
  int use_inv;                     // sorted with at most 8 points: inv holds per interval
  T inv[kLmax - 1][36];            // 1/(v_k - v_m) (28 pairs) and 1/(1 + v_k^2) (8)
  uint8_t* hull;                   // (L - 1, N) live lines of every instance (sorted order), or NULL
};

// A pixel's L label values (L <= LT) between registers and memory: 128-bit
// accesses when FP32 and L a multiple of 4 (rows are then 16-byte aligned).
template <typename T, int LT>
OPYX_D void ld_labels(T (&d)[LT], const T* p, int L) {
  if (sizeof(T) == 4 && (L & 3) == 0) {
#pragma unroll
    for (int l = 0; l < LT; l += 4) {
      if (l >= L) { d[l] = d[l + 1] = d[l + 2] = d[l + 3] = T(0); continue; }
      const float4 v = *reinterpret_cast<const float4*>(p + l);
      d[l] = v.x; d[l + 1] = v.y; d[l + 2] = v.z; d[l + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int l = 0; l < LT; ++l) d[l] = l < L ? p[l] : T(0);
  }
}
template <typename T, int LT>
OPYX_D void st_labels(T* p, const T (&d)[LT], int L) {
  if (sizeof(T) == 4 && (L & 3) == 0) {
#pragma unroll
    for (int l = 0; l < LT; l += 4) {
      if (l >= L) break;
      *reinterpret_cast<float4*>(p + l) = make_float4(d[l], d[l + 1], d[l + 2], d[l + 3]);
    }
  } else {
#pragma unroll
    for (int l = 0; l < LT; ++l) {
      if (l >= L) break;
      p[l] = d[l];
    }
  }
}

// ---- pass A (L labels, LT >= L the compile-time capacity)
template <typename T, int LT>
__global__ void __launch_bounds__(kThreads, 4) k_pass_a(Args<T> a) {
  const int64_t N = a.N, W = a.W;
  const int L = a.L;
  const T* u_k = a.xk;
  const T* g_k = a.xk + N * L;
  const T* mu_k = a.xk + N * L + N;
  const T* q_k = a.yk;
  const T* e_k = a.yk + N * L;
  const T* p_k = a.yk + N * L + N;
  const T* s_k = a.yk + N * L + 3 * N;
  const T* z_k = a.yk + N * L + 4 * N;
  const T th = a.theta, th1 = T(1) + a.theta;
  SUB_GRID_STRIDE(i, N) {
    const int64_t r = i / W, c = i - r * W;
    T q[LT], uo[LT], un[LT], ub[LT];
    ld_labels(q, q_k + i * L, L);
    ld_labels(uo, u_k + i * L, L);
    const T e = e_k[i], s = s_k[i];
    // u: A^T y = q + t e + 1 s (the blocks of the u column in row order)
#pragma unroll
    for (int l = 0; l < LT; ++l) {
      T xg = q[l];
      xg += a.t[l] * e;
      xg += T(1) * s;
      T v = uo[l] + (-a.tau_u[l]) * xg;
      v = v < T(0) ? T(0) : v;
      un[l] = v;
      ub[l] = th1 * v - th * uo[l];
    }
    st_labels(a.xkp1 + i * L, un, L);
    st_labels(a.xbar + i * L, ub, L);
    // gamma: A^T y = -e - div p (forward differences, h = 1)
    {
      T acc = T(0);
      if (r < a.H - 1) acc -= p_k[i * 2];
      if (r > 0) acc += p_k[(i - W) * 2];
      if (c < W - 1) acc -= p_k[i * 2 + 1];
      if (c > 0) acc += p_k[(i - 1) * 2 + 1];
      T xg = T(-1) * e;
      xg += acc;
      const T go = g_k[i];
      const T tg = a.tau_g ? a.tau_g[i] : a.tau_g0;
      const T gn = go + (-tg) * xg;
      a.xkp1[N * L + i] = gn;
      a.xbar[N * L + i] = th1 * gn - th * go;
    }
    // mu: A^T y = IndexedMult(q) + z, IndexedMult(q)[j, m] = -sum_k B[j][m][k] q[j + k]
#pragma unroll
    for (int j = 0; j < LT - 1; ++j) {
      if (j >= L - 1) break;
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        const int64_t o = (j * N + i) * 2 + m;
        T xg = -(a.B[j][m][0] * q[j] + a.B[j][m][1] * q[j + 1]);
        xg += z_k[o];
        const T mo = mu_k[o];
        const T mn = mo + (-a.tau_mu[j][m]) * xg;
        a.xkp1[N * L + N + o] = mn;
        a.xbar[N * L + N + o] = th1 * mn - th * mo;
      }
    }
  }
}

// The z block of interval j at pixel i: (slope, offset) moved by sigma
// mubar and projected onto the epigraph of the interval's piecewise-linear
// data term (project1 over the interval's points, in increasing slope).
template <typename T, int NS, bool SORTED>
OPYX_D void z_project(const Args<T>& a, int j, int64_t i) {
  const int64_t N = a.N, L = a.L;
  const T* mub = a.xbar + N * L + N;
  const T* z_k = a.yk + N * L + 4 * N;
  T* z_n = a.ykp1 + N * L + 4 * N;
  T cv[NS], cb[NS];
  bool on[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    const bool used = k < a.nsub;
    const int kk = SORTED ? a.perm[j][k] : k;
    const int64_t l = used ? a.J[j * a.nsub + kk] : 0;
    on[k] = used && (!a.It || a.It[l * N + i] != 0);
    cv[k] = on[k] ? a.v[l] : T(0);
    cb[k] = on[k] ? a.bt[l * N + i] : T(0);
  }
  const int64_t o = (j * N + i) * 2;
  const T s0 = z_k[o] + a.sig_z[j][0] * mub[o];
  const T t0 = z_k[o + 1] + a.sig_z[j][1] * mub[o + 1];
  T ys, yt;
  epi::project1<T, NS, SORTED>(cv, cb, on, s0, t0, ys, yt,
                               NS == 8 && a.use_inv ? a.inv[j] : nullptr);
  z_n[o] = ys;
  z_n[o + 1] = yt;
}

// The z block of interval j at pixel i with the instance's live lines known
// (hull): only they are read, and the scan visits only them.
template <typename T, int NS>
OPYX_D void z_project_live(const Args<T>& a, int j, int64_t i) {
  const int64_t N = a.N, L = a.L;
  const T* mub = a.xbar + N * L + N;
  const T* z_k = a.yk + N * L + 4 * N;
  T* z_n = a.ykp1 + N * L + 4 * N;
  const unsigned live = a.hull[j * N + i];
  T cv[NS], cb[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    const bool on = (live >> k) & 1u;
    const int64_t l = on ? a.J[j * a.nsub + a.perm[j][k]] : 0;
    cv[k] = on ? a.v[l] : T(0);
    cb[k] = on ? a.bt[l * N + i] : T(0);
  }
  const int64_t o = (j * N + i) * 2;
  const T s0 = z_k[o] + a.sig_z[j][0] * mub[o];
  const T t0 = z_k[o + 1] + a.sig_z[j][1] * mub[o + 1];
  T ys, yt;
  epi::project1_live<T, NS>(cv, cb, live, s0, t0, ys, yt);
  z_n[o] = ys;
  z_n[o + 1] = yt;
}

// The live lines of every (interval, pixel) instance, once per solve (the
// data term is fixed): bit k for the k-th point in increasing slope.
template <typename T, int NS>
__global__ void __launch_bounds__(kThreads) k_hull(Args<T> a) {
  const int j = (int)blockIdx.y;
  SUB_GRID_STRIDE(i, a.N) {
    T cv[NS], cb[NS];
    bool on[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const bool used = k < a.nsub;
      const int64_t l = used ? a.J[j * a.nsub + a.perm[j][k]] : 0;
      on[k] = used && (!a.It || a.It[l * a.N + i] != 0);
      cv[k] = on[k] ? a.v[l] : T(0);
      cb[k] = on[k] ? a.bt[l * a.N + i] : T(0);
    }
    a.hull[j * a.N + i] = (uint8_t)epi::live_mask1<T, NS>(cv, cb, on);
  }
}

// ---- pass B, z blocks: blockIdx.y = j the interval (a kernel of its own:
// far fewer registers than the pixel part, so twice the resident warps for
// this compute-bound part)
template <typename T, int NS, bool SORTED>
__global__ void __launch_bounds__(kThreads, 8) k_pass_z(Args<T> a) {
  const int j = (int)blockIdx.y;
  if (SORTED && a.hull) {
    SUB_GRID_STRIDE(i, a.N) z_project_live<T, NS>(a, j, i);
  } else {
    SUB_GRID_STRIDE(i, a.N) z_project<T, NS, SORTED>(a, j, i);
  }
}

// ---- pass B, the q, e, p, s blocks of every pixel
template <typename T, int LT>
__global__ void __launch_bounds__(kThreads, 4) k_pass_b(Args<T> a) {
  const int64_t N = a.N, W = a.W;
  const int L = a.L;
  const T* ub = a.xbar;
  const T* gb = a.xbar + N * L;
  const T* mub = a.xbar + N * L + N;
  const T* q_k = a.yk;
  const T* e_k = a.yk + N * L;
  const T* p_k = a.yk + N * L + N;
  const T* s_k = a.yk + N * L + 3 * N;
  T* q_n = a.ykp1;
  T* e_n = a.ykp1 + N * L;
  T* p_n = a.ykp1 + N * L + N;
  T* s_n = a.ykp1 + N * L + 3 * N;
  SUB_GRID_STRIDE(i, N) {
    const int64_t r = i / W, c = i - r * W;
    T u[LT];
    ld_labels(u, ub + i * L, L);
    // q: u + IndexedMultAdj(mu), IndexedMultAdj(mu)[l] -= sum_m B[j][m][k] mu[j][m], l = j + k
    {
      T ax[LT];
#pragma unroll
      for (int l = 0; l < LT; ++l) ax[l] = u[l];
#pragma unroll
      for (int j = 0; j < LT - 1; ++j) {
        if (j >= L - 1) break;
        const T m0 = mub[(j * N + i) * 2], m1 = mub[(j * N + i) * 2 + 1];
#pragma unroll
        for (int k = 0; k < 2; ++k) ax[j + k] -= a.B[j][0][k] * m0 + a.B[j][1][k] * m1;
      }
      T qo[LT];
      ld_labels(qo, q_k + i * L, L);
#pragma unroll
      for (int l = 0; l < LT; ++l) ax[l] = qo[l] + a.sig_q[l] * ax[l];
      st_labels(q_n + i * L, ax, L);
    }
    // e: <t, u> - gamma
    const T g0 = gb[i];
    {
      T ax = T(0);
#pragma unroll
      for (int l = 0; l < LT; ++l) {
        if (l >= L) break;
        ax += u[l] * a.t[l];
      }
      ax += T(-1) * g0;
      e_n[i] = e_k[i] + a.sig_e * ax;
    }
    // p: grad gamma, projected onto the lbd-ball
    {
      const T gd = r < a.H - 1 ? gb[i + W] - g0 : T(0);
      const T gr = c < W - 1 ? gb[i + 1] - g0 : T(0);
      const T sp0 = a.sig_p ? a.sig_p[i * 2] : a.sig_p0;
      const T sp1 = a.sig_p ? a.sig_p[i * 2 + 1] : a.sig_p0;
      T pv[2] = {p_k[i * 2] + sp0 * gd, p_k[i * 2 + 1] + sp1 * gr};
      frob_proj(pv, 2, a.lbd);
      p_n[i * 2] = pv[0];
      p_n[i * 2 + 1] = pv[1];
    }
    // s: <1, u>, prox of <1, s>: s - sigma
    {
      T ax = T(0);
#pragma unroll
      for (int l = 0; l < LT; ++l) {
        if (l >= L) break;
        ax += u[l];
      }
      const T sv = s_k[i] + a.sig_s * ax;
      s_n[i] = sv - a.sig_s * T(1);
    }
  }
}

template <typename T, int LT>
static int launch_l(const Args<T>& a, int which, cudaStream_t s) {
  const unsigned g = grid_for(a.N, kThreads, 8);
  if (which == 0) {
    k_pass_a<T, LT><<<g, kThreads, 0, s>>>(a);
    return check_launch();
  }
  if (which == 2) {   // the instances' live lines, into a.hull
    const dim3 grid(g, (unsigned)(a.L - 1), 1);
    if (a.nsub <= 8) k_hull<T, 8><<<grid, kThreads, 0, s>>>(a);
    else k_hull<T, 16><<<grid, kThreads, 0, s>>>(a);
    return check_launch();
  }
  k_pass_b<T, LT><<<g, kThreads, 0, s>>>(a);
  int st = check_launch();
  if (st) return st;
  const dim3 grid(g, (unsigned)(a.L - 1), 1);   // every interval's z blocks
  if (a.nsub <= 8) {
    if (a.sorted) k_pass_z<T, 8, true><<<grid, kThreads, 0, s>>>(a);
    else k_pass_z<T, 8, false><<<grid, kThreads, 0, s>>>(a);
  } else {
    if (a.sorted) k_pass_z<T, 16, true><<<grid, kThreads, 0, s>>>(a);
    else k_pass_z<T, 16, false><<<grid, kThreads, 0, s>>>(a);
  }
  return check_launch();
}

template <typename T>
static int launch(const opyx_sublabel* d, int which, cudaStream_t s) {
  Args<T> a;
  memset(&a, 0, sizeof(a));
  a.N = d->H * d->W;
  a.H = d->H;
  a.W = d->W;
  a.L = d->L;
  a.nsub = d->nsub;
  a.xk = (const T*)d->xk;
  a.xkp1 = (T*)d->xkp1;
  a.xbar = (T*)d->xbar;
  a.yk = (const T*)d->yk;
  a.ykp1 = (T*)d->ykp1;
  const int L = d->L;
  for (int l = 0; l < L; ++l) {
    a.t[l] = (T)d->t[l];
    a.tau_u[l] = (T)d->tau_u[l];
    a.sig_q[l] = (T)d->sig_q[l];
  }
  for (int j = 0; j < L - 1; ++j)
    for (int m = 0; m < 2; ++m) {
      for (int k = 0; k < 2; ++k) a.B[j][m][k] = (T)d->B[(j * 2 + m) * 2 + k];
      a.tau_mu[j][m] = (T)d->tau_mu[j * 2 + m];
      a.sig_z[j][m] = (T)d->sig_z[j * 2 + m];
    }
  a.sig_e = (T)d->sig_e;
  a.sig_s = (T)d->sig_s;
  a.tau_g = (const T*)d->tau_g;
  a.sig_p = (const T*)d->sig_p;
  a.tau_g0 = (T)d->tau_g0;
  a.sig_p0 = (T)d->sig_p0;
  a.lbd = (T)d->lbd;
  a.theta = (T)d->theta;
  a.v = (const T*)d->v;
  a.bt = (const T*)d->bt;
  a.It = d->It;
  a.J = d->J;
  a.sorted = d->sorted;
  a.hull = d->hull;
  // reciprocals of the sorted points' slope differences (one interval's
  // points are shared by every pixel): the projection multiplies
  a.use_inv = d->sorted && d->nsub <= 8;
  if (a.use_inv) {
    for (int j = 0; j < L - 1; ++j) {
      double vs[8];
      for (int k = 0; k < 8; ++k) vs[k] = k < d->nsub ? d->vsorted[j * 16 + k] : 0.0;
      int idx = 0;
      for (int m = 0; m < 8; ++m)
        for (int k = m + 1; k < 8; ++k, ++idx)
          a.inv[j][idx] = (T)(k < d->nsub && m < d->nsub ? 1.0 / (vs[k] - vs[m]) : 0.0);
      for (int k = 0; k < 8; ++k) a.inv[j][28 + k] = (T)(1.0 / (1.0 + vs[k] * vs[k]));
    }
  }
  for (int j = 0; j < L - 1; ++j)
    for (int k = 0; k < 16; ++k) a.perm[j][k] = d->perm[j * 16 + k];
  if (L <= 8) return launch_l<T, 8>(a, which, s);
  if (L <= 16) return launch_l<T, 16>(a, which, s);
  return launch_l<T, 32>(a, which, s);
}

}  // namespace sub
}  // namespace opyx

using namespace opyx;

extern "C" int opyx_sublabel_pass(const opyx_sublabel* d, int which, void* stream) {
  if (!d || which < 0 || which > 2) return OPYX_ERR_ARG;
  if (which == 2 && (!d->hull || !d->sorted)) return OPYX_ERR_ARG;
  if (d->H < 1 || d->W < 1 || d->nsub < 2 || d->nsub > 16) return OPYX_ERR_ARG;
  if (d->L < 2 || d->L > 32) return OPYX_ERR_UNSUPPORTED;
  if (which < 2 && (!d->xk || !d->xbar || !d->yk || (which == 0 && !d->xkp1) ||
                    (which == 1 && !d->ykp1)))
    return OPYX_ERR_ARG;
  if (which >= 1 && (!d->v || !d->bt || !d->J)) return OPYX_ERR_ARG;
  if (d->sorted)
    for (int j = 0; j < d->L - 1; ++j)
      for (int k = 0; k < d->nsub; ++k)
        if (d->perm[j * 16 + k] >= d->nsub) return OPYX_ERR_ARG;
  if (d->dtype == OPYX_F32) return sub::launch<float>(d, which, (cudaStream_t)stream);
  if (d->dtype == OPYX_F64) return sub::launch<double>(d, which, (cudaStream_t)stream);
  return OPYX_ERR_ARG;
}
