// One PDHG iteration of the 2-D fused ROF path for ONE channel, streamed
// through the registers of one warp: the body of the persistent batched
// solve (rof.cu, k_batch_persist).
//
// The iteration is that of k_sweep (rof_sweep.cuh): at row step r, pass A
// on row r (x_{k+1}[r], xbar[r] from y_k rows r-1, r and x_k[r], f[r]) and
// pass B on row r-1 (y_{k+1}[r-1] from xbar rows r-1, r and y_k[r-1]),
// reading (x, y) and writing (x2, y2), with the halo row after the run and
// the halo pixel right of the warp's range recomputed.  The per-pixel
// arithmetic is that of k_passA_p / k_passB_p, so the results are
// bit-identical to the two passes and to the single-image sweep.
//
// A warp owns a strip of 128 pixels (4 per lane) and a run of rows, and
// needs nothing from other warps: the rows arrive by 128-bit loads straight
// into registers, two rows ahead of their use (one row ahead: 0.82 against
// 0.76 ms per iteration of the 512-instance batch); y_k and xbar of the previous
// row stay in registers; neighbours along the row come by warp shuffles,
// and only lane 0 (the y value left of the strip) and lane 31 (pass A of
// the pixel right of it, for pass B's neighbour) load a few scalars more.
// x_{k+1} and y_{k+1} leave by 128-bit stores.  With no shared memory and no
// block barrier a warp can take any work item, which is what a batch of
// instances of uneven sizes needs; on small images (1024^2) this body ran
// an iteration in 10.3 us against 12.4 us for the shared-memory sweep.
// Quads away from the image border take a path with the border tests
// resolved and the preconditioner coefficients in registers.
#pragma once

#include "rof_sweep.cuh"

namespace opyx {
namespace rof {

// Step coefficients of the interior pixels, held in registers.
struct Coef1 {
  float tau, a, tv;            // primal step, SSD prox scale, tau * vol
  float sig_l, sig_r;          // dual steps along the row / across rows
  float hub_l, hub_r;          // Huber scales of the dual
};

OPYX_D Coef1 interior_coef(const Geo<float>& g, bool pre, const PrimalCoefs<float, 1>& pc,
                           float sig_c, float hub_c) {
  Coef1 c;
  c.tau = pre ? g.tau_tab[8][0] : pc.tau;
  c.a = pre ? g.a_tab[8][0] : pc.a[0];
  c.tv = pre ? g.tv_tab[8][0] : pc.tv[0];
  c.sig_l = pre ? g.sig_pre[1][0] : sig_c;
  c.sig_r = pre ? g.sig_pre[0][0] : sig_c;
  c.hub_l = pre ? g.hub_pre[1][0] : hub_c;
  c.hub_r = pre ? g.hub_pre[0][0] : hub_c;
  return c;
}

// Pass A of pixel q of row r (as k_passA_p with C = 1, D = 2): yc1 = y_k[r]
// component along the row at q, yl1 = the same at q - 1, yc0 = y_k[r]
// across rows at q, yu0 = y_k[r - 1] across rows at q; `on` = the SSD term
// applies (mask).  FAST: q is not on the image border and r has rows above
// and below (cb = 8).
template <bool FAST>
OPYX_D void pass_a1(const Geo<float>& g, bool pre, const PrimalCoefs<float, 1>& pc,
                    const Coef1& ci, int64_t q, bool on, bool has_up, bool has_dn, float yc1,
                    float yl1, float yc0, float yu0, float xo, float fq, float& xn, float& xb) {
  float s = 0.f;
  const float ihl = g.invh[1];
  if (FAST || q < g.nl - 1) s -= yc1 * ihl;
  if (FAST || q > 0) s += yl1 * ihl;
  const float ihr = g.invh[0];
  if (FAST || has_dn) s -= yc0 * ihr;
  if (FAST || has_up) s += yu0 * ihr;
  const float dv = g.w[0] * s;
  float v;
  if (FAST) {
    v = xo - ci.tau * dv;
    if (on) v = ci.a * (v + ci.tv * fq);
  } else {
    const int cb = (int)((q < g.nl - 1) + (q > 0)) + 3 * (int)(has_dn + has_up);
    const float tau = pre ? g.tau_tab[cb][0] : pc.tau;
    v = xo - tau * dv;
    if (on) v = (pre ? g.a_tab[cb][0] : pc.a[0]) * (v + (pre ? g.tv_tab[cb][0] : pc.tv[0]) * fq);
  }
  xn = v;
  xb = g.theta1 * v - g.theta * xo;
}

// Pass B of pixel q of row rb (as k_passB_p with C = 1, D = 2): xk = xbar[rb]
// at q, nb = xbar[rb] at q + 1, xn = xbar[rb + 1] at q; (y0, y1) = y_k[rb]
// at q across / along rows, updated in place to y_{k+1}.
template <bool FAST>
OPYX_D void pass_b1(const Geo<float>& g, bool pre, float sig_c, float hub_c, const Coef1& ci,
                    int64_t q, bool has_next, float xk, float nb, float xn, float& y0, float& y1) {
  const bool inx = FAST || q < g.nl - 1;
  const bool hn = FAST || has_next;
  const float gl = inx ? g.coef[1][0] * (nb - xk) : 0.f;
  float hf1, hf0;
  if (FAST) {
    y1 += ci.sig_l * gl;
    hf1 = ci.hub_l;
  } else {
    y1 += (pre ? (inx ? g.sig_pre[1][0] : 0.f) : sig_c) * gl;
    hf1 = pre ? (inx ? g.hub_pre[1][0] : 1.f) : hub_c;
  }
  const float gr = hn ? g.coef[0][0] * (xn - xk) : 0.f;
  if (FAST) {
    y0 += ci.sig_r * gr;
    hf0 = ci.hub_r;
  } else {
    y0 += (pre ? (hn ? g.sig_pre[0][0] : 0.f) : sig_c) * gr;
    hf0 = pre ? (hn ? g.hub_pre[0][0] : 1.f) : hub_c;
  }
  if (g.use_huber) {
    y0 *= hf0;
    y1 *= hf1;
  }
  float n2 = 0.f;
  n2 += y0 * y0;
  n2 += y1 * y1;
  if (n2 > g.lbd2) {
    const float sc = g.lbd * rsqrtf(n2);
    y0 *= sc;
    y1 *= sc;
  }
}

// The data of one row for one lane: its quad of y_k (4 x 2), x_k, f and
// mask bytes; lane 0's y_k (along the row) left of its quad; lane 31's halo
// pixel right of it (y_k both components, x_k, f, mask).
struct Row1 {
  float4 y01, y23, xv, fv;
  unsigned mk;
  float yl, hy0, hy1, hx, hf;
  unsigned hm;
};

// Iterates are read through L2 (ld.global.cg): in a persistent kernel other
// SMs rewrite them between iterations, and L1 is not coherent across SMs.
// f and the mask do not change and may be cached in L1.
OPYX_D float4 ldcg4(const float* p) { return __ldcg(reinterpret_cast<const float4*>(p)); }
OPYX_D float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
OPYX_D void stg4(float* p, float a0, float a1, float a2, float a3) {
  *reinterpret_cast<float4*>(p) = make_float4(a0, a1, a2, a3);
}

// Row r (none if r is outside [0, rows)) for the lane whose quad starts at
// q0; act: the quad lies in the image.
template <bool MASK>
OPYX_D Row1 load_row1(const Geo<float>& g, const Args<float>& a, int64_t r, int64_t q0, bool act,
                      int lane) {
  Row1 d;
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  d.y01 = d.y23 = d.xv = d.fv = z;
  d.mk = 0xffffffffu;
  d.yl = d.hy0 = d.hy1 = d.hx = d.hf = 0.f;
  d.hm = 1u;
  if (r < 0 || r >= g.rows) return d;
  const int64_t i0 = r * g.nl + q0;
  if (act) {
    d.y01 = ldcg4(a.y + i0 * 2);
    d.y23 = ldcg4(a.y + i0 * 2 + 4);
    d.xv = ldcg4(a.x + i0);
    d.fv = ldg4(a.f + i0);
    if (MASK) d.mk = __ldg(reinterpret_cast<const unsigned*>(a.mask + i0));
  }
  if (lane == 0 && act && q0 > 0) d.yl = __ldcg(a.y + i0 * 2 - 1);
  if (lane == 31 && q0 + 4 < g.nl) {
    const float2 h = __ldcg(reinterpret_cast<const float2*>(a.y + (i0 + 4) * 2));
    d.hy0 = h.x;
    d.hy1 = h.y;
    d.hx = __ldcg(a.x + i0 + 4);
    d.hf = __ldg(a.f + i0 + 4);
    if (MASK) d.hm = __ldg(a.mask + i0 + 4);
  }
  return d;
}

// One iteration on rows [r0, r1) of the strip of 128 pixels starting at
// q_beg (clipped to the image), by one warp: lane l owns the quad at
// q_beg + 4 l.  Reads a.x, a.y, a.f; writes a.x2, a.y2.  MASK: a.mask is
// set (else the SSD term applies everywhere).
#ifndef OPYX_STRIP_PF
#define OPYX_STRIP_PF 2
#endif
constexpr int kStripPF = OPYX_STRIP_PF;   // rows each lane has in flight

template <bool PRE, bool MASK>
OPYX_D void sweep_strip1(const Geo<float>& g, const Args<float>& a, int64_t q_beg, int64_t r0,
                         int64_t r1) {
  const int lane = threadIdx.x & 31;
  const int64_t q0 = q_beg + 4 * lane;
  const bool act = q0 < g.nl;   // whole quads: the last axis is a multiple of 4
  const int64_t rl = r1 < g.rows ? r1 : r1 - 1;   // last row whose pass A runs here
  constexpr bool pre = PRE;
  const PrimalCoefs<float, 1> pc(g, (float)a.tau);
  const float sig_c = (float)a.sigma;
  const float hub_c = 1.f / (1.f + sig_c * g.hub_ratio);
  const Coef1 ci = interior_coef(g, pre, pc, sig_c, hub_c);
  const bool qin = q0 > 0 && q0 + 4 < g.nl;   // the quad and its right neighbour inside
  float py0[4], py1[4], pxb[4], phb = 0.f, phy0;
  {
    // y_k of the row above the run (across rows) for pass A of its first row
    const Row1 u = load_row1<MASK>(g, a, r0 - 1, q0, act, lane);
    py0[0] = u.y01.x; py0[1] = u.y01.z; py0[2] = u.y23.x; py0[3] = u.y23.z;
    py1[0] = u.y01.y; py1[1] = u.y01.w; py1[2] = u.y23.y; py1[3] = u.y23.w;
    phy0 = u.hy0;
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) pxb[p] = 0.f;
  Row1 cur = load_row1<MASK>(g, a, r0, q0, act, lane);
  Row1 nx2 = load_row1<MASK>(g, a, kStripPF > 1 && r0 + 1 <= rl ? r0 + 1 : -1, q0, act, lane);
  for (int64_t r = r0; r <= r1; ++r) {
    const Row1 nxt = kStripPF > 1 ? nx2
                                  : load_row1<MASK>(g, a, r + 1 <= rl ? r + 1 : -1, q0, act, lane);
    if (kStripPF > 1) nx2 = load_row1<MASK>(g, a, r + 2 <= rl ? r + 2 : -1, q0, act, lane);
    const bool has_up = r > 0, has_dn = r < g.rows - 1;
    const float cy0[4] = {cur.y01.x, cur.y01.z, cur.y23.x, cur.y23.z};
    const float cy1[4] = {cur.y01.y, cur.y01.w, cur.y23.y, cur.y23.w};
    float cxb[4] = {0.f, 0.f, 0.f, 0.f}, chb = 0.f;
    if (r <= rl) {
      // ---- pass A of row r
      const float xo[4] = {cur.xv.x, cur.xv.y, cur.xv.z, cur.xv.w};
      const float fq[4] = {cur.fv.x, cur.fv.y, cur.fv.z, cur.fv.w};
      const float up1 = __shfl_up_sync(0xffffffffu, cy1[3], 1);
      const float yl0 = lane ? up1 : cur.yl;
      float xn[4];
      if (qin && has_up && has_dn) {
#pragma unroll
        for (int p = 0; p < 4; ++p)
          pass_a1<true>(g, pre, pc, ci, q0 + p, !MASK || ((cur.mk >> (8 * p)) & 0xffu) != 0, has_up,
                        has_dn, cy1[p], p > 0 ? cy1[p - 1] : yl0, cy0[p], py0[p], xo[p], fq[p],
                        xn[p], cxb[p]);
      } else {
#pragma unroll
        for (int p = 0; p < 4; ++p)
          pass_a1<false>(g, pre, pc, ci, q0 + p,
                         !MASK || q0 + p >= g.nl || ((cur.mk >> (8 * p)) & 0xffu) != 0, has_up, has_dn,
                         cy1[p], p > 0 ? cy1[p - 1] : yl0, cy0[p], py0[p], xo[p], fq[p], xn[p],
                         cxb[p]);
      }
      if (lane == 31) {
        float hxn;
        pass_a1<false>(g, pre, pc, ci, q0 + 4, !MASK || q0 + 4 >= g.nl || cur.hm != 0, has_up, has_dn,
                       cur.hy1, cy1[3], cur.hy0, phy0, cur.hx, cur.hf, hxn, chb);
      }
      if (r < r1 && act) stg4(a.x2 + r * g.nl + q0, xn[0], xn[1], xn[2], xn[3]);
    }
    // ---- pass B of row r - 1
    if (r > r0) {
      const bool has_next = r - 1 < g.rows - 1;
      const float dn = __shfl_down_sync(0xffffffffu, pxb[0], 1);
      const float xr = lane == 31 ? phb : dn;
      if (qin && has_next) {
#pragma unroll
        for (int p = 0; p < 4; ++p)
          pass_b1<true>(g, pre, sig_c, hub_c, ci, q0 + p, has_next, pxb[p],
                        p < 3 ? pxb[p + 1] : xr, cxb[p], py0[p], py1[p]);
      } else {
#pragma unroll
        for (int p = 0; p < 4; ++p)
          pass_b1<false>(g, pre, sig_c, hub_c, ci, q0 + p, has_next, pxb[p],
                         p < 3 ? pxb[p + 1] : xr, cxb[p], py0[p], py1[p]);
      }
      if (act) {
        float* yo = a.y2 + ((r - 1) * g.nl + q0) * 2;
        stg4(yo, py0[0], py1[0], py0[1], py1[1]);
        stg4(yo + 4, py0[2], py1[2], py0[3], py1[3]);
      }
    }
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      py0[p] = cy0[p];
      py1[p] = cy1[p];
      pxb[p] = cxb[p];
    }
    phb = chb;
    phy0 = cur.hy0;
    cur = nxt;
  }
}

}  // namespace rof
}  // namespace opyx
