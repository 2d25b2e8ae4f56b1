// One PDHG iteration of the 2-D fused ROF path in a single sweep over HBM.
//
// The two-pass iteration (rof_pipe.cuh) writes xbar in pass A and reads it
// back in pass B.  Here one CTA streams its rows once and does both: at row
// step r it runs pass A on row r (x_{k+1}[r] and xbar[r] from y_k rows r-1,
// r and x_k[r], f[r]) and then pass B on row r-1 (y_{k+1}[r-1] from xbar rows
// r-1, r and y_k[r-1]).  xbar never leaves shared memory, so an iteration
// moves 4*N*(3C + 2K) bytes instead of 4*N*(5C + 3K) (2048^2 x 3: 352 MB
// instead of 554 MB).
//
// Pass A of row r reads y_k[r-1], which the CTA owning the rows above writes
// as y_{k+1}[r-1]; pass B of a CTA's last row needs xbar of the first row of
// the CTA below, computed from x_k and y_k there.  So the sweep reads
// (x, y) and writes (x2, y2) -- ping-pong buffers the host swaps every
// iteration -- and each CTA recomputes pass A of the row after its run (and
// of the first pixel past its tile's right edge) for the xbar halo, without
// storing it: about 1/RB extra reads, no race.  The arithmetic of every pixel
// is that of k_passA_p / k_passB_p, so results are bit-identical to the two
// passes.
//
// Shared memory per CTA (TW = 512): y ring 3 x (TW+8) x K (4-pixel halo
// both sides), x and f rings 2 x (TW+4) x C (right halo), xbar 2 x (TW+4) x C.
// Requirements as rof_pipe.cuh (checked on the host); 2-D only (the
// neighbour one plane away in 3-D would need a plane of xbar on chip).
#pragma once

#include "rof_pipe.cuh"

namespace opyx {
namespace rof {

template <int C>
struct SweepSmem {
  static constexpr int M = 2 * C;
  static constexpr int X4 = (kPipeTW + 4) * C;   // right halo
  static constexpr int Y44 = (kPipeTW + 8) * M;  // 4-pixel halo on both sides
  static constexpr int bytes = 4 * (3 * Y44 + 2 * X4 + 2 * X4 + 2 * X4);
};

// Pixels per thread of the sweep: 2 (256 threads per 512-pixel tile), twice
// the resident warps of 4-pixel quads at the same shared memory per pixel --
// the sweep does both passes' arithmetic per byte and is latency-bound.
constexpr int kSweepP = 2;
constexpr int kSweepThreads = kPipeTW / kSweepP;

// Shared <-> register moves of NF consecutive floats: 128-bit when NF is a
// multiple of 4 (then the address is 16-byte aligned), 64-bit when it is
// even (8-byte aligned), else one float at a time.
template <int NF>
OPYX_D void lds(float (&d)[NF], const float* __restrict__ p) {
  if (NF % 4 == 0) {
#pragma unroll
    for (int j = 0; j < NF / 4; ++j) {
      const float4 v = reinterpret_cast<const float4*>(p)[j];
      d[4 * j] = v.x; d[4 * j + 1] = v.y; d[4 * j + 2] = v.z; d[4 * j + 3] = v.w;
    }
  } else if (NF % 2 == 0) {
#pragma unroll
    for (int j = 0; j < NF / 2; ++j) {
      const float2 v = reinterpret_cast<const float2*>(p)[j];
      d[2 * j] = v.x; d[2 * j + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < NF; ++j) d[j] = p[j];
  }
}
template <int NF>
OPYX_D void sts(float* __restrict__ p, const float (&d)[NF]) {
  if (NF % 4 == 0) {
#pragma unroll
    for (int j = 0; j < NF / 4; ++j)
      reinterpret_cast<float4*>(p)[j] = make_float4(d[4 * j], d[4 * j + 1], d[4 * j + 2], d[4 * j + 3]);
  } else if (NF % 2 == 0) {
#pragma unroll
    for (int j = 0; j < NF / 2; ++j)
      reinterpret_cast<float2*>(p)[j] = make_float2(d[2 * j], d[2 * j + 1]);
  } else {
#pragma unroll
    for (int j = 0; j < NF; ++j) p[j] = d[j];
  }
}

// Pass A of NP consecutive pixels from local pixel lp (0..TW) of row r:
// x_{k+1} (into qx) and xbar (into qb), as k_passA_p.
template <int C, int NP>
OPYX_D void sweep_a(const Geo<float>& g, const Args<float>& a, const PrimalCoefs<float, C>& pc,
                    bool pre, const float* yc, const float* yu, const float* xv, const float* fv,
                    int64_t r, int64_t q_beg, int lp, float (&qx)[NP * C], float (&qb)[NP * C]) {
  constexpr int D = 2, M = D * C;
  const bool has_up = r > 0, has_dn = r < g.rows - 1;
  const int64_t qt = q_beg + lp;
  float qy[NP * M], qu[NP * M], qf[NP * C], yl[C];
  lds(qy, yc + (lp + 4) * M);
  lds(qu, yu + (lp + 4) * M);
  lds(qx, xv + lp * C);
  lds(qf, fv + lp * C);
#pragma unroll
  for (int k2 = 0; k2 < C; ++k2) yl[k2] = yc[(lp + 3) * M + (D - 1) * C + k2];
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    const int64_t q = qt + p;
    const bool on = !a.mask || q >= g.nl || a.mask[r * g.nl + q];
    const int cb = (int)((q < g.nl - 1) + (q > 0)) + 3 * (int)(has_dn + has_up);
#pragma unroll
    for (int k2 = 0; k2 < C; ++k2) {
      float s = 0.f;
      const float ihl = g.invh[D - 1];
      if (q < g.nl - 1) s -= qy[p * M + (D - 1) * C + k2] * ihl;
      if (q > 0) s += (p > 0 ? qy[(p - 1) * M + (D - 1) * C + k2] : yl[k2]) * ihl;
      const float ihr = g.invh[D - 2];
      if (has_dn) s -= qy[p * M + (D - 2) * C + k2] * ihr;
      if (has_up) s += qu[p * M + (D - 2) * C + k2] * ihr;
      const float dv = g.w[k2] * s;
      const float tau = pre ? g.tau_tab[cb][k2] : pc.tau;
      const float xo = qx[p * C + k2];
      float v = xo - tau * dv;
      if (on) v = (pre ? g.a_tab[cb][k2] : pc.a[k2]) *
                  (v + (pre ? g.tv_tab[cb][k2] : pc.tv[k2]) * qf[p * C + k2]);
      qx[p * C + k2] = v;
      qb[p * C + k2] = g.theta1 * v - g.theta * xo;
    }
  }
}

template <int C>
__global__ void __launch_bounds__(kSweepThreads, 3) k_sweep(Geo<float> g, Args<float> a, int RB) {
  if (stopped(a)) return;
  using S = SweepSmem<C>;
  constexpr int D = 2, M = D * C, P = kSweepP, NT = kSweepThreads;
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  float* ys = sm;                          // 3 x Y44: row q in slot (q - r0 + 1) % 3
  float* xs = ys + 3 * S::Y44;             // 2 x X4 : x_k, then x_{k+1}
  float* fs = xs + 2 * S::X4;              // 2 x X4
  float* bs = fs + 2 * S::X4;              // 2 x X4 : xbar rows, slot (q - r0) & 1
  const int64_t q_beg = blockIdx.x * (int64_t)kPipeTW;
  const int lp0 = threadIdx.x * P;
  const bool halo = threadIdx.x == NT - 1;   // also computes xbar at pixel TW
  const bool pre = g.steps == OPYX_STEPS_PRECOND;
  const PrimalCoefs<float, C> pc(g, (float)a.tau);
  const float sig_c = (float)a.sigma;
  const float hub_c = 1.f / (1.f + sig_c * g.hub_ratio);
  for (int64_t r0 = blockIdx.y * (int64_t)RB; r0 < g.rows; r0 += (int64_t)gridDim.y * RB) {
    const int64_t r1 = r0 + RB < g.rows ? r0 + RB : g.rows;
    const int64_t rl = r1 < g.rows ? r1 : r1 - 1;   // last row whose pass A runs here
    copy_row<M, 4, 4, NT>(ys, a.y, g, r0 - 1, q_beg);
    copy_row<M, 4, 4, NT>(ys + S::Y44, a.y, g, r0, q_beg);
    copy_row<C, 0, 4, NT>(xs, a.x, g, r0, q_beg);
    copy_row<C, 0, 4, NT>(fs, a.f, g, r0, q_beg);
    cp_commit();
    for (int64_t r = r0; r <= r1; ++r) {
      const int k = (int)(r - r0);
      const bool run_a = r <= rl;
      const bool more = r + 1 <= rl;
      copy_row<M, 4, 4, NT>(ys + ((k + 2) % 3) * S::Y44, a.y, g, r + 1, q_beg, more);
      copy_row<C, 0, 4, NT>(xs + ((k + 1) & 1) * S::X4, a.x, g, r + 1, q_beg, more);
      copy_row<C, 0, 4, NT>(fs + ((k + 1) & 1) * S::X4, a.f, g, r + 1, q_beg, more);
      cp_commit();
      cp_wait<1>();
      __syncthreads();
      const float* yc = ys + ((k + 1) % 3) * S::Y44;    // y_k row r
      float* yu = ys + (k % 3) * S::Y44;                // y_k row r - 1
      float* xv = xs + (k & 1) * S::X4;
      const float* fv = fs + (k & 1) * S::X4;
      float* bc = bs + (k & 1) * S::X4;                 // xbar row r
      const float* bu = bs + ((k + 1) & 1) * S::X4;     // xbar row r - 1
      // ---- pass A, row r (and xbar at the first pixel past the tile)
      if (run_a) {
        float qx[P * C], qb[P * C];
        sweep_a<C, P>(g, a, pc, pre, yc, yu, xv, fv, r, q_beg, lp0, qx, qb);
        float hb[C];
        if (halo) {
          float hx[C];
          sweep_a<C, 1>(g, a, pc, pre, yc, yu, xv, fv, r, q_beg, kPipeTW, hx, hb);
        }
        __syncthreads();   // every thread has read the x_k values it needs
        sts(xv + lp0 * C, qx);
        sts(bc + lp0 * C, qb);
        if (halo) {
#pragma unroll
          for (int k2 = 0; k2 < C; ++k2) bc[kPipeTW * C + k2] = hb[k2];
        }
      }
      __syncthreads();
      if (r < r1) store_row<C, 0, NT>(a.x2, xv, g, r, q_beg);
      // ---- pass B, row r - 1 (as k_passB_p), in place in its y slot
      if (r > r0) {
        const int64_t rb = r - 1;
        const bool has_next = rb < g.rows - 1;
        float qx[P * C], qn[P * C], qy[P * M], xr[C];
        lds(qx, bu + lp0 * C);
        lds(qn, bc + lp0 * C);
        lds(qy, yu + (lp0 + 4) * M);
#pragma unroll
        for (int k2 = 0; k2 < C; ++k2) xr[k2] = bu[(lp0 + P) * C + k2];
#pragma unroll
        for (int p = 0; p < P; ++p) {
          const int64_t q = q_beg + lp0 + p;
          const bool inx = q < g.nl - 1;
          float hf[M];
#pragma unroll
          for (int k2 = 0; k2 < C; ++k2) {
            const float xk = qx[p * C + k2];
            const float nb = p < P - 1 ? qx[(p + 1) * C + k2] : xr[k2];
            const float gl = inx ? g.coef[D - 1][k2] * (nb - xk) : 0.f;
            qy[p * M + (D - 1) * C + k2] += (pre ? (inx ? g.sig_pre[D - 1][k2] : 0.f) : sig_c) * gl;
            hf[(D - 1) * C + k2] = pre ? (inx ? g.hub_pre[D - 1][k2] : 1.f) : hub_c;
            const float gr = has_next ? g.coef[D - 2][k2] * (qn[p * C + k2] - xk) : 0.f;
            qy[p * M + (D - 2) * C + k2] +=
                (pre ? (has_next ? g.sig_pre[D - 2][k2] : 0.f) : sig_c) * gr;
            hf[(D - 2) * C + k2] = pre ? (has_next ? g.hub_pre[D - 2][k2] : 1.f) : hub_c;
          }
          if (g.use_huber) {
#pragma unroll
            for (int j = 0; j < M; ++j) qy[p * M + j] *= hf[j];
          }
          float n2 = 0.f;
#pragma unroll
          for (int j = 0; j < M; ++j) n2 += qy[p * M + j] * qy[p * M + j];
          if (n2 > g.lbd2) {
            const float sc = g.lbd * rsqrtf(n2);
#pragma unroll
            for (int j = 0; j < M; ++j) qy[p * M + j] *= sc;
          }
        }
        sts(yu + (lp0 + 4) * M, qy);
        __syncthreads();
        store_row<M, 4, NT>(a.y2, yu, g, rb, q_beg);
      }
      __syncthreads();
    }
    cp_wait<0>();
    __syncthreads();
  }
}

}  // namespace rof
}  // namespace opyx
