// Vectorised FP32 versions of the fused ROF passes (constant and
// preconditioned steps) and of the gap kernel.
//
// Thread tile: a "quad" of 4 consecutive pixels along the contiguous last
// axis, for R consecutive rows (a row = all pixels with the same coordinates
// in the other axes).  Per pixel the arrays hold C (x, xbar, f) or D*C (y)
// floats, so a quad is C or D*C float4 -- every global access is a 128-bit
// load or store of a contiguous, 16-byte aligned run (requires the last axis
// to be a multiple of 4).  Neighbours:
//   * along the last axis: the next / previous pixel of the quad, or the
//     adjacent lane's quad through a warp shuffle (the warp's edge lanes load
//     it from memory);
//   * along axis D-2: the next / previous row, carried in registers while the
//     thread slides down its R rows;
//   * along axis 0 for D = 3: a load of the quad one plane away (an L2 hit:
//     that plane is the current plane of other blocks in flight).
#pragma once

#include "rof_kernels.cuh"

namespace opyx {
namespace rof {

constexpr int kVecThreads = 128;

template <int NF>
OPYX_D void ldv(float (&d)[NF], const float* __restrict__ p) {
  static_assert(NF % 4 == 0, "whole float4s");
  const float4* s = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int j = 0; j < NF / 4; ++j) {
    const float4 v = s[j];
    d[4 * j] = v.x;
    d[4 * j + 1] = v.y;
    d[4 * j + 2] = v.z;
    d[4 * j + 3] = v.w;
  }
}

template <int NF>
OPYX_D void stv(float* __restrict__ p, const float (&d)[NF]) {
  static_assert(NF % 4 == 0, "whole float4s");
  float4* s = reinterpret_cast<float4*>(p);
#pragma unroll
  for (int j = 0; j < NF / 4; ++j) s[j] = make_float4(d[4 * j], d[4 * j + 1], d[4 * j + 2], d[4 * j + 3]);
}

template <int NF>
OPYX_D void zero(float (&d)[NF]) {
#pragma unroll
  for (int j = 0; j < NF; ++j) d[j] = 0.f;
}

// Row coordinates: crow along axis D-2, cz along axis 0 (D = 3).
template <int D>
OPYX_D void row_coords(const Geo<float>& g, int64_t r, int64_t* crow, int64_t* cz) {
  if (D == 1) { *crow = 0; *cz = 0; }
  if (D == 2) { *crow = r; *cz = 0; }
  if (D == 3) { *crow = r % g.n[1]; *cz = r / g.n[1]; }
}

// ------------------------------------------------------------------ pass B
// y <- prox_{sigma F*}(y + sigma * A xbar) for R rows of one quad.
template <int D, int C>
__global__ void __launch_bounds__(kVecThreads) k_passB_v(Geo<float> g, Args<float> a, int R) {
  if (stopped(a)) return;
  constexpr int M = D * C;
  const int64_t Q = g.nl >> 2;
  const int64_t quad = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool act = quad < Q;
  const int64_t q0 = quad * 4;
  const int lane = threadIdx.x & 31;
  const bool pre = g.steps == OPYX_STEPS_PRECOND;
  const float sig_c = (float)a.sigma;
  const float hub_c = 1.f / (1.f + sig_c * g.hub_ratio);
  for (int64_t r0 = blockIdx.y * (int64_t)R; r0 < g.rows; r0 += (int64_t)gridDim.y * R) {
    const int64_t rend = r0 + R < g.rows ? r0 + R : g.rows;
    float xc[4 * C];
    if (act) ldv(xc, a.xbar + (r0 * g.nl + q0) * C); else zero(xc);
    for (int64_t r = r0; r < rend; ++r) {
      const int64_t i0 = r * g.nl + q0;
      int64_t crow, cz;
      row_coords<D>(g, r, &crow, &cz);
      float xn[4 * C], xz[4 * C];
      if (act && r + 1 < g.rows) ldv(xn, a.xbar + (i0 + g.nl) * C); else zero(xn);
      const bool has_next = D >= 2 && crow < g.n[D - 2] - 1;
      const bool has_z = D == 3 && cz < g.n[0] - 1;
      if (D == 3) { if (act && has_z) ldv(xz, a.xbar + (i0 + g.s[0]) * C); else zero(xz); }
      float xr[C];
#pragma unroll
      for (int k = 0; k < C; ++k) xr[k] = __shfl_down_sync(0xffffffffu, xc[k], 1);
      if (lane == 31 && act && q0 + 4 < g.nl) {
#pragma unroll
        for (int k = 0; k < C; ++k) xr[k] = a.xbar[(i0 + 4) * C + k];
      }
      float yv[4 * M];
      if (act) ldv(yv, a.y + i0 * M); else zero(yv);
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        const bool inx = q0 + p < g.nl - 1;
        float hf[M];
#pragma unroll
        for (int k = 0; k < C; ++k) {
          const float xk = xc[p * C + k];
          const float nb = p < 3 ? xc[(p + 1) * C + k] : xr[k];
          const float gl = inx ? g.coef[D - 1][k] * (nb - xk) : 0.f;
          yv[p * M + (D - 1) * C + k] += (pre ? (inx ? g.sig_pre[D - 1][k] : 0.f) : sig_c) * gl;
          hf[(D - 1) * C + k] = pre ? (inx ? g.hub_pre[D - 1][k] : 1.f) : hub_c;
          if (D >= 2) {
            const float gr = has_next ? g.coef[D - 2][k] * (xn[p * C + k] - xk) : 0.f;
            yv[p * M + (D - 2) * C + k] +=
                (pre ? (has_next ? g.sig_pre[D - 2][k] : 0.f) : sig_c) * gr;
            hf[(D - 2) * C + k] = pre ? (has_next ? g.hub_pre[D - 2][k] : 1.f) : hub_c;
          }
          if (D == 3) {
            const float gz = has_z ? g.coef[0][k] * (xz[p * C + k] - xk) : 0.f;
            yv[p * M + k] += (pre ? (has_z ? g.sig_pre[0][k] : 0.f) : sig_c) * gz;
            hf[k] = pre ? (has_z ? g.hub_pre[0][k] : 1.f) : hub_c;
          }
        }
        if (g.use_huber) {
#pragma unroll
          for (int j = 0; j < M; ++j) yv[p * M + j] *= hf[j];
        }
        float n2 = 0.f;
#pragma unroll
        for (int j = 0; j < M; ++j) n2 += yv[p * M + j] * yv[p * M + j];
        if (n2 > g.lbd2) {
          const float sc = g.lbd * rsqrtf(n2);   // 2-ulp reciprocal square root
#pragma unroll
          for (int j = 0; j < M; ++j) yv[p * M + j] *= sc;
        }
      }
      if (act) stv(a.y + i0 * M, yv);
#pragma unroll
      for (int j = 0; j < 4 * C; ++j) xc[j] = xn[j];
    }
  }
}

// Divergence of y at the 4 pixels of a quad: the row's own y (yv), the
// previous pixel's last-axis component (yl, from the neighbouring lane), the
// axis D-2 component of the row above (yup) and, for D = 3, the axis-0
// component one plane back (yz).
template <int D, int C>
OPYX_D void quad_div(const Geo<float>& g, int64_t q0, int64_t crow, int64_t cz,
                     const float (&yv)[4 * D * C], const float (&yl)[C],
                     const float (&yup)[4 * C], const float (&yz)[4 * C],
                     float (&dv)[4 * C]) {
  constexpr int M = D * C;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int64_t cl = q0 + p;
#pragma unroll
    for (int k = 0; k < C; ++k) {
      float s = 0.f;
      const float ihl = g.invh[D - 1];
      if (cl < g.nl - 1) s -= yv[p * M + (D - 1) * C + k] * ihl;
      if (cl > 0) s += (p > 0 ? yv[(p - 1) * M + (D - 1) * C + k] : yl[k]) * ihl;
      if (D >= 2) {
        const float ihr = g.invh[D - 2];
        if (crow < g.n[D - 2] - 1) s -= yv[p * M + (D - 2) * C + k] * ihr;
        if (crow > 0) s += yup[p * C + k] * ihr;
      }
      if (D == 3) {
        const float ihz = g.invh[0];
        if (cz < g.n[0] - 1) s -= yv[p * M + k] * ihz;
        if (cz > 0) s += yz[p * C + k] * ihz;
      }
      dv[p * C + k] = g.w[k] * s;
    }
  }
}

// Loads of the backward neighbours needed by quad_div.
template <int D, int C>
OPYX_D void quad_back(const Geo<float>& g, const float* __restrict__ y, bool act, int lane,
                      int64_t i0, int64_t q0, int64_t cz, const float (&yv)[4 * D * C],
                      float (&yl)[C], float (&yz)[4 * C]) {
  constexpr int M = D * C;
#pragma unroll
  for (int k = 0; k < C; ++k) yl[k] = __shfl_up_sync(0xffffffffu, yv[3 * M + (D - 1) * C + k], 1);
  if (lane == 0 && act && q0 > 0) {
#pragma unroll
    for (int k = 0; k < C; ++k) yl[k] = y[(i0 - 1) * M + (D - 1) * C + k];
  }
  if (D == 3) {
    if (act && cz > 0) {
      float tmp[4 * M];
      ldv(tmp, y + (i0 - g.s[0]) * M);
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int k = 0; k < C; ++k) yz[p * C + k] = tmp[p * M + k];
    } else {
      zero(yz);
    }
  }
}

// Index of the preconditioner tables for the pixel at last-axis coordinate
// cl in a row with coordinates (crow, cz).
template <int D>
OPYX_D int quad_combo(const Geo<float>& g, int64_t cl, int64_t crow, int64_t cz) {
  int cb = (int)((cl < g.nl - 1) + (cl > 0));
  if (D >= 2) cb += 3 * (int)((crow < g.n[D - 2] - 1) + (crow > 0));
  if (D == 3) cb += 9 * (int)((cz < g.n[0] - 1) + (cz > 0));
  return cb;
}

// ------------------------------------------------------------------ pass A
// x <- prox_{tau G}(x - tau A^T y), xbar <- (1+theta) x_new - theta x_old.
template <int D, int C>
__global__ void __launch_bounds__(kVecThreads) k_passA_v(Geo<float> g, Args<float> a, int R) {
  if (stopped(a)) return;
  constexpr int M = D * C;
  const int64_t Q = g.nl >> 2;
  const int64_t quad = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool act = quad < Q;
  const int64_t q0 = quad * 4;
  const int lane = threadIdx.x & 31;
  const bool pre = g.steps == OPYX_STEPS_PRECOND;
  const PrimalCoefs<float, C> pc(g, (float)a.tau);
  for (int64_t r0 = blockIdx.y * (int64_t)R; r0 < g.rows; r0 += (int64_t)gridDim.y * R) {
    const int64_t rend = r0 + R < g.rows ? r0 + R : g.rows;
    float yup[4 * C];
    zero(yup);
    if (D >= 2 && act && r0 > 0) {
      float tmp[4 * M];
      ldv(tmp, a.y + ((r0 - 1) * g.nl + q0) * M);
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int k = 0; k < C; ++k) yup[p * C + k] = tmp[p * M + (D - 2) * C + k];
    }
    for (int64_t r = r0; r < rend; ++r) {
      const int64_t i0 = r * g.nl + q0;
      int64_t crow, cz;
      row_coords<D>(g, r, &crow, &cz);
      float yv[4 * M];
      if (act) ldv(yv, a.y + i0 * M); else zero(yv);
      float yl[C], yz[4 * C];
      quad_back<D, C>(g, a.y, act, lane, i0, q0, cz, yv, yl, yz);
      float dv[4 * C];
      quad_div<D, C>(g, q0, crow, cz, yv, yl, yup, yz, dv);
      if (act) {
        float xo[4 * C], fv[4 * C], xn[4 * C], xb[4 * C];
        ldv(xo, a.x + i0 * C);
        ldv(fv, a.f + i0 * C);
        unsigned mk = 0xffffffffu;
        if (a.mask) mk = *reinterpret_cast<const unsigned*>(a.mask + i0);
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          const bool on = (mk >> (8 * p)) & 0xffu;
          const int cb = pre ? quad_combo<D>(g, q0 + p, crow, cz) : 0;
#pragma unroll
          for (int k = 0; k < C; ++k) {
            const float tau = pre ? g.tau_tab[cb][k] : pc.tau;
            float v = xo[p * C + k] - tau * dv[p * C + k];
            if (on) v = (pre ? g.a_tab[cb][k] : pc.a[k]) *
                        (v + (pre ? g.tv_tab[cb][k] : pc.tv[k]) * fv[p * C + k]);
            xn[p * C + k] = v;
            xb[p * C + k] = g.theta1 * v - g.theta * xo[p * C + k];
          }
        }
        stv(a.x + i0 * C, xn);
        stv(a.xbar + i0 * C, xb);
      }
      if (D >= 2) {
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
          for (int k = 0; k < C; ++k) yup[p * C + k] = yv[p * M + (D - 2) * C + k];
      }
    }
  }
}

// ------------------------------------------------------------------ gap
// Same sums as k_gap; per-thread partials are accumulated in FP32 over the
// thread's quads and rows and folded in FP64 across threads and blocks.
template <int D, int C>
__global__ void __launch_bounds__(kVecThreads) k_gap_v(Geo<float> g, Args<float> a, int R,
                                                       double ssd_shift) {
  if (stopped(a)) return;
  constexpr int M = D * C;
  const int64_t Q = g.nl >> 2;
  const int64_t quad = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool act = quad < Q;
  const int64_t q0 = quad * 4;
  const int lane = threadIdx.x & 31;
  double sG = 0.0, sF = 0.0, sGs = 0.0, sFs = 0.0, inf = 0.0;
  for (int64_t r0 = blockIdx.y * (int64_t)R; r0 < g.rows; r0 += (int64_t)gridDim.y * R) {
    const int64_t rend = r0 + R < g.rows ? r0 + R : g.rows;
    float pG = 0.f, pF = 0.f, pGs = 0.f, pFs = 0.f, pinf = -INFINITY;
    float yup[4 * C];
    zero(yup);
    if (D >= 2 && act && r0 > 0) {
      float tmp[4 * M];
      ldv(tmp, a.y + ((r0 - 1) * g.nl + q0) * M);
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int k = 0; k < C; ++k) yup[p * C + k] = tmp[p * M + (D - 2) * C + k];
    }
    float xc[4 * C];
    if (act) ldv(xc, a.x + (r0 * g.nl + q0) * C); else zero(xc);
    for (int64_t r = r0; r < rend; ++r) {
      const int64_t i0 = r * g.nl + q0;
      int64_t crow, cz;
      row_coords<D>(g, r, &crow, &cz);
      // dual side: A^T y and y
      float yv[4 * M];
      if (act) ldv(yv, a.y + i0 * M); else zero(yv);
      float yl[C], yz[4 * C];
      quad_back<D, C>(g, a.y, act, lane, i0, q0, cz, yv, yl, yz);
      float dv[4 * C];
      quad_div<D, C>(g, q0, crow, cz, yv, yl, yup, yz, dv);
      // primal side: A x
      float xn[4 * C], xz[4 * C];
      if (act && r + 1 < g.rows) ldv(xn, a.x + (i0 + g.nl) * C); else zero(xn);
      const bool has_next = D >= 2 && crow < g.n[D - 2] - 1;
      const bool has_z = D == 3 && cz < g.n[0] - 1;
      if (D == 3) { if (act && has_z) ldv(xz, a.x + (i0 + g.s[0]) * C); else zero(xz); }
      float xr[C];
#pragma unroll
      for (int k = 0; k < C; ++k) xr[k] = __shfl_down_sync(0xffffffffu, xc[k], 1);
      if (lane == 31 && act && q0 + 4 < g.nl) {
#pragma unroll
        for (int k = 0; k < C; ++k) xr[k] = a.x[(i0 + 4) * C + k];
      }
      if (act) {
        float fv[4 * C];
        ldv(fv, a.f + i0 * C);
        unsigned mk = 0xffffffffu;
        if (a.mask) mk = *reinterpret_cast<const unsigned*>(a.mask + i0);
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          const bool on = (mk >> (8 * p)) & 0xffu;
          const bool inx = q0 + p < g.nl - 1;
          float n2 = 0.f, y2 = 0.f;
#pragma unroll
          for (int k = 0; k < C; ++k) {
            const float xk = xc[p * C + k], fk = fv[p * C + k], ak = dv[p * C + k];
            if (on) {
              const float d = xk - fk;
              pG += g.vol[k] * d * d;
              pGs += ak * ak * g.half_rvol[k] - fk * ak;
            }
            const float nb = p < 3 ? xc[(p + 1) * C + k] : xr[k];
            const float gl = inx ? g.coef[D - 1][k] * (nb - xk) : 0.f;
            n2 += gl * gl;
            if (D >= 2) {
              const float gr = has_next ? g.coef[D - 2][k] * (xn[p * C + k] - xk) : 0.f;
              n2 += gr * gr;
            }
            if (D == 3) {
              const float gz = has_z ? g.coef[0][k] * (xz[p * C + k] - xk) : 0.f;
              n2 += gz * gz;
            }
          }
#pragma unroll
          for (int j = 0; j < M; ++j) y2 += yv[p * M + j] * yv[p * M + j];
          const float nrm = sqrtf(n2);
          pF += g.use_huber ? (nrm <= g.huber ? n2 * g.half_rhuber : nrm - g.half_huber) : nrm;
          pFs += y2;
          pinf = fmaxf(pinf, sqrtf(y2) - g.lbd);
        }
      }
      if (D >= 2) {
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
          for (int k = 0; k < C; ++k) yup[p * C + k] = yv[p * M + (D - 2) * C + k];
      }
#pragma unroll
      for (int j = 0; j < 4 * C; ++j) xc[j] = xn[j];
    }
    sG += 0.5 * (double)pG;
    sF += (double)pF;
    sGs += (double)pGs;
    sFs += (double)pFs;
    inf = fmax(inf, (double)pinf);
  }
  double vals[5] = {sG, sF, sGs, sFs, inf};
  const int ops[5] = {RED_SUM, RED_SUM, RED_SUM, RED_SUM, RED_MAX};
  block_reduce_and_finish<5>(vals, ops, a.partials, a.ticket, [&](double* tot) {
    write_info(g, a, tot, ssd_shift);
  });
}

}  // namespace rof
}  // namespace opyx
