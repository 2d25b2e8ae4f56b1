// Row-streaming FP32 kernels of the fused ROF passes and gap, with the
// global->shared traffic in asynchronous copies (cp.async, 16 bytes per
// instruction, zero-fill outside the image).
//
// A CTA owns a tile of TW pixels along the contiguous last axis and a run
// of RB consecutive rows (row = all pixels with equal coordinates in the
// other axes).  Each array it reads streams through a small ring of row
// slots in shared memory: while the CTA computes row r, the copies of the
// rows it needs next are already in flight, so memory stays busy without
// holding data in registers.  Results go back to shared memory and leave in
// coalesced 128-bit stores (each warp instruction covers 512 contiguous
// bytes).  Neighbours along the last axis are read from the slot (slots carry
// a 4-pixel halo), neighbours along axis D-2 are the adjacent row slots, and
// for D = 3 the rows one plane away stream through rings of their own.
//
// All waits are cp.async.wait_group (hardware completion of this thread's
// own copies); there is no spin loop.  Requirements (checked on the host):
// last axis a multiple of 4, 16-byte aligned arrays, 4-byte aligned mask.
#pragma once

#include "rof_kernels.cuh"

namespace opyx {
namespace rof {

constexpr int kPipeTW = 512;               // tile width in pixels
constexpr int kPipeThreads = kPipeTW / 4;  // 4 pixels per thread

OPYX_D void cp_async16(void* sdst, const void* gsrc, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
  const int n = valid ? 16 : 0;   // 0: zero-fill, the source is not read
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gsrc), "r"(n)
               : "memory");
}
OPYX_D void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
OPYX_D void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Cooperative copy of row `r` of an array with E floats per pixel into a slot
// holding pixels [q_beg - HL, q_beg + TW + HR).  Chunks outside the row or
// outside [0, rows) are zero-filled; `need` = false (a row past the end of
// the CTA's run) issues nothing.
template <int E, int HL, int HR, int NT = kPipeThreads, int TW = kPipeTW>
OPYX_D void copy_row(float* slot, const float* __restrict__ arr, const Geo<float>& g, int64_t r,
                     int64_t q_beg, bool need = true) {
  if (!need) return;
  constexpr int NPX = TW + HL + HR;
  constexpr int NCH = NPX * E / 4;
  const bool rv = r >= 0 && r < g.rows;
  const int64_t row_f0 = (rv ? r : 0) * g.nl * E;        // float offset of the row
  const int64_t f0 = (q_beg - HL) * E;                    // float offset of the slot in the row
  const int64_t fmax = g.nl * E;
  for (int c = threadIdx.x; c < NCH; c += NT) {
    const int64_t fo = f0 + (int64_t)c * 4;
    const bool valid = rv && fo >= 0 && fo + 4 <= fmax;
    cp_async16(slot + c * 4, arr + row_f0 + (valid ? fo : 0), valid);
  }
}

// Cooperative coalesced store of the first TW pixels (after HL halo pixels)
// of a slot to row r.
template <int E, int HL, int NT = kPipeThreads, int TW = kPipeTW>
OPYX_D void store_row(float* __restrict__ arr, const float* slot, const Geo<float>& g, int64_t r,
                      int64_t q_beg) {
  constexpr int NCH = TW * E / 4;
  const int64_t f0 = q_beg * E;
  const int64_t fmax = g.nl * E;
  float* row = arr + r * g.nl * E;
  const float4* s = reinterpret_cast<const float4*>(slot + HL * E);
  for (int c = threadIdx.x; c < NCH; c += NT) {
    const int64_t fo = f0 + (int64_t)c * 4;
    if (fo + 4 <= fmax) *reinterpret_cast<float4*>(row + fo) = s[c];
  }
}

template <int D>
OPYX_D void pipe_row_coords(const Geo<float>& g, int64_t r, int64_t* crow, int64_t* cz) {
  if (D == 2) { *crow = r; *cz = 0; }
  if (D == 3) { *crow = r % g.n[1]; *cz = r / g.n[1]; }
}

// Shared-memory sizes (bytes) of the three kernels.
template <int D, int C, int TW = kPipeTW>
struct PipeSmem {
  static constexpr int M = D * C;
  static constexpr int X4 = (TW + 4) * C;   // floats of a slot with a 4-pixel halo
  static constexpr int Y4 = (TW + 4) * M;
  static constexpr int X0 = TW * C;
  static constexpr int Y0 = TW * M;
  // pass B: xbar ring 3 (halo right), y ring 2, [xbar plane ring 2]
  static constexpr int B = 4 * (3 * X4 + 2 * Y0 + (D == 3 ? 2 * X0 : 0));
  // pass A: y ring 3 (halo left), x ring 2, f ring 2, xbar out, [y plane ring 2]
  static constexpr int A = 4 * (3 * Y4 + 2 * X0 + 2 * X0 + X0 + (D == 3 ? 2 * Y0 : 0));
  // gap: x ring 3 (halo right), y ring 3 (halo left), f ring 2, [x, y plane rings]
  static constexpr int G = 4 * (3 * X4 + 3 * Y4 + 2 * X0 + (D == 3 ? 2 * X0 + 2 * Y0 : 0));
};

// ------------------------------------------------------------------ pass B
template <int D, int C, int TW = kPipeTW>
__global__ void __launch_bounds__(TW / 4) k_passB_p(Geo<float> g, Args<float> a, int RB) {
  if (stopped(a)) return;
  using S = PipeSmem<D, C, TW>;
  constexpr int NT = TW / 4;
  constexpr int M = D * C;
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  float* xs = sm;                          // 3 x X4
  float* ys = xs + 3 * S::X4;              // 2 x Y0
  float* zs = ys + 2 * S::Y0;              // 2 x X0 (D = 3)
  const int64_t q_beg = blockIdx.x * (int64_t)TW;
  const int lp0 = threadIdx.x * 4;         // first local pixel of this thread
  const bool pre = g.steps == OPYX_STEPS_PRECOND;
  const float sig_c = (float)a.sigma;
  const float hub_c = 1.f / (1.f + sig_c * g.hub_ratio);
  const int64_t nplane = D == 3 ? g.n[1] : 0;  // rows per plane
  for (int64_t r0 = blockIdx.y * (int64_t)RB; r0 < g.rows; r0 += (int64_t)gridDim.y * RB) {
    const int64_t r1 = r0 + RB < g.rows ? r0 + RB : g.rows;
    copy_row<C, 0, 4, NT, TW>(xs, a.xbar, g, r0, q_beg);
    copy_row<C, 0, 4, NT, TW>(xs + S::X4, a.xbar, g, r0 + 1, q_beg);
    copy_row<M, 0, 0, NT, TW>(ys, a.y, g, r0, q_beg);
    if (D == 3) copy_row<C, 0, 0, NT, TW>(zs, a.xbar, g, r0 + nplane, q_beg);
    cp_commit();
    for (int64_t r = r0; r < r1; ++r) {
      const int k = (int)(r - r0);
      // prefetch the rows of the next step
      copy_row<C, 0, 4, NT, TW>(xs + ((k + 2) % 3) * S::X4, a.xbar, g, r + 2, q_beg, r + 2 <= r1);
      copy_row<M, 0, 0, NT, TW>(ys + ((k + 1) & 1) * S::Y0, a.y, g, r + 1, q_beg, r + 1 < r1);
      if (D == 3)
        copy_row<C, 0, 0, NT, TW>(zs + ((k + 1) & 1) * S::X0, a.xbar, g, r + 1 + nplane, q_beg, r + 1 < r1);
      cp_commit();
      cp_wait<1>();
      __syncthreads();
      const float* xc = xs + (k % 3) * S::X4;
      const float* xn = xs + ((k + 1) % 3) * S::X4;
      float* yv = ys + (k & 1) * S::Y0;
      const float* xz = zs + (k & 1) * S::X0;
      int64_t crow, cz;
      pipe_row_coords<D>(g, r, &crow, &cz);
      const bool has_next = crow < g.n[D - 2] - 1;
      const bool has_z = D == 3 && cz < g.n[0] - 1;
      // this thread's quad, pulled from the slots with 128-bit shared loads
      float qx[4 * C], qn[4 * C], qz[4 * C], qy[4 * M], xr[C];
      ldv(qx, xc + lp0 * C);
      ldv(qn, xn + lp0 * C);
      if (D == 3) ldv(qz, xz + lp0 * C);
      ldv(qy, yv + lp0 * M);
#pragma unroll
      for (int k2 = 0; k2 < C; ++k2) xr[k2] = xc[(lp0 + 4) * C + k2];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        const int64_t q = q_beg + lp0 + p;
        const bool inx = q < g.nl - 1;
        float hf[M];
#pragma unroll
        for (int k2 = 0; k2 < C; ++k2) {
          const float xk = qx[p * C + k2];
          const float nb = p < 3 ? qx[(p + 1) * C + k2] : xr[k2];
          const float gl = inx ? g.coef[D - 1][k2] * (nb - xk) : 0.f;
          qy[p * M + (D - 1) * C + k2] += (pre ? (inx ? g.sig_pre[D - 1][k2] : 0.f) : sig_c) * gl;
          hf[(D - 1) * C + k2] = pre ? (inx ? g.hub_pre[D - 1][k2] : 1.f) : hub_c;
          const float gr = has_next ? g.coef[D - 2][k2] * (qn[p * C + k2] - xk) : 0.f;
          qy[p * M + (D - 2) * C + k2] +=
              (pre ? (has_next ? g.sig_pre[D - 2][k2] : 0.f) : sig_c) * gr;
          hf[(D - 2) * C + k2] = pre ? (has_next ? g.hub_pre[D - 2][k2] : 1.f) : hub_c;
          if (D == 3) {
            const float gz = has_z ? g.coef[0][k2] * (qz[p * C + k2] - xk) : 0.f;
            qy[p * M + k2] += (pre ? (has_z ? g.sig_pre[0][k2] : 0.f) : sig_c) * gz;
            hf[k2] = pre ? (has_z ? g.hub_pre[0][k2] : 1.f) : hub_c;
          }
        }
        if (g.use_huber) {
#pragma unroll
          for (int j = 0; j < M; ++j) qy[p * M + j] *= hf[j];
        }
        float n2 = 0.f;
#pragma unroll
        for (int j = 0; j < M; ++j) n2 += qy[p * M + j] * qy[p * M + j];
        if (n2 > g.lbd2) {
          const float sc = g.lbd * rsqrtf(n2);   // 2-ulp reciprocal square root
#pragma unroll
          for (int j = 0; j < M; ++j) qy[p * M + j] *= sc;
        }
      }
      stv(yv + lp0 * M, qy);
      __syncthreads();
      store_row<M, 0, NT, TW>(a.y, yv, g, r, q_beg);
      __syncthreads();
    }
    cp_wait<0>();
    __syncthreads();
  }
}

// ------------------------------------------------------------------ pass A
template <int D, int C, int TW = kPipeTW>
__global__ void __launch_bounds__(TW / 4) k_passA_p(Geo<float> g, Args<float> a, int RB) {
  if (stopped(a)) return;
  using S = PipeSmem<D, C, TW>;
  constexpr int NT = TW / 4;
  constexpr int M = D * C;
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  float* ys = sm;                          // 3 x Y4 (halo left: local pixel = lp + 4)
  float* xs = ys + 3 * S::Y4;              // 2 x X0
  float* fs = xs + 2 * S::X0;              // 2 x X0
  float* bs = fs + 2 * S::X0;              // 1 x X0 (xbar out)
  float* zs = bs + S::X0;                  // 2 x Y0 (D = 3: y one plane back)
  const int64_t q_beg = blockIdx.x * (int64_t)TW;
  const int lp0 = threadIdx.x * 4;
  const bool pre = g.steps == OPYX_STEPS_PRECOND;
  const PrimalCoefs<float, C> pc(g, (float)a.tau);
  const int64_t nplane = D == 3 ? g.n[1] : 0;
  for (int64_t r0 = blockIdx.y * (int64_t)RB; r0 < g.rows; r0 += (int64_t)gridDim.y * RB) {
    const int64_t r1 = r0 + RB < g.rows ? r0 + RB : g.rows;
    // y slot of row r is ((r - r0 + 1) % 3): row r0 - 1 -> 0, r0 -> 1, r0 + 1 -> 2
    copy_row<M, 4, 0, NT, TW>(ys, a.y, g, r0 - 1, q_beg);
    copy_row<M, 4, 0, NT, TW>(ys + S::Y4, a.y, g, r0, q_beg);
    copy_row<C, 0, 0, NT, TW>(xs, a.x, g, r0, q_beg);
    copy_row<C, 0, 0, NT, TW>(fs, a.f, g, r0, q_beg);
    if (D == 3) copy_row<M, 0, 0, NT, TW>(zs, a.y, g, r0 - nplane, q_beg);
    cp_commit();
    for (int64_t r = r0; r < r1; ++r) {
      const int k = (int)(r - r0);
      const bool more = r + 1 < r1;
      copy_row<M, 4, 0, NT, TW>(ys + ((k + 2) % 3) * S::Y4, a.y, g, r + 1, q_beg, more);
      copy_row<C, 0, 0, NT, TW>(xs + ((k + 1) & 1) * S::X0, a.x, g, r + 1, q_beg, more);
      copy_row<C, 0, 0, NT, TW>(fs + ((k + 1) & 1) * S::X0, a.f, g, r + 1, q_beg, more);
      if (D == 3) copy_row<M, 0, 0, NT, TW>(zs + ((k + 1) & 1) * S::Y0, a.y, g, r + 1 - nplane, q_beg, more);
      cp_commit();
      cp_wait<1>();
      __syncthreads();
      const float* yc = ys + ((k + 1) % 3) * S::Y4;     // row r
      const float* yu = ys + (k % 3) * S::Y4;           // row r - 1
      float* xv = xs + (k & 1) * S::X0;
      const float* fv = fs + (k & 1) * S::X0;
      const float* yz = zs + (k & 1) * S::Y0;
      int64_t crow, cz;
      pipe_row_coords<D>(g, r, &crow, &cz);
      const bool has_up = crow > 0, has_dn = crow < g.n[D - 2] - 1;
      const bool has_zb = D == 3 && cz > 0, has_zf = D == 3 && cz < g.n[0] - 1;
      unsigned mk = 0xffffffffu;
      const int64_t qt = q_beg + lp0;
      if (a.mask && qt < g.nl) mk = *reinterpret_cast<const unsigned*>(a.mask + r * g.nl + qt);
      // this thread's quad (y slots carry 4 halo pixels on the left)
      float qy[4 * M], qu[4 * M], qx[4 * C], qf[4 * C], qb[4 * C], yl[C];
      ldv(qy, yc + (lp0 + 4) * M);
      ldv(qu, yu + (lp0 + 4) * M);
      ldv(qx, xv + lp0 * C);
      ldv(qf, fv + lp0 * C);
#pragma unroll
      for (int k2 = 0; k2 < C; ++k2) yl[k2] = yc[(lp0 + 3) * M + (D - 1) * C + k2];
      float qz[4 * M];
      if (D == 3) ldv(qz, yz + lp0 * M);
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        const int64_t q = q_beg + lp0 + p;
        const bool on = (mk >> (8 * p)) & 0xffu;
        const int cb = (int)((q < g.nl - 1) + (q > 0)) + 3 * (int)(has_dn + has_up) +
                       (D == 3 ? 9 * (int)(has_zf + has_zb) : 0);
#pragma unroll
        for (int k2 = 0; k2 < C; ++k2) {
          float s = 0.f;
          const float ihl = g.invh[D - 1];
          if (q < g.nl - 1) s -= qy[p * M + (D - 1) * C + k2] * ihl;
          if (q > 0) s += (p > 0 ? qy[(p - 1) * M + (D - 1) * C + k2] : yl[k2]) * ihl;
          const float ihr = g.invh[D - 2];
          if (has_dn) s -= qy[p * M + (D - 2) * C + k2] * ihr;
          if (has_up) s += qu[p * M + (D - 2) * C + k2] * ihr;
          if (D == 3) {
            const float ihz = g.invh[0];
            if (has_zf) s -= qy[p * M + k2] * ihz;
            if (has_zb) s += qz[p * M + k2] * ihz;
          }
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
      stv(xv + lp0 * C, qx);
      stv(bs + lp0 * C, qb);
      __syncthreads();
      store_row<C, 0, NT, TW>(a.x, xv, g, r, q_beg);
      store_row<C, 0, NT, TW>(a.xbar, bs, g, r, q_beg);
      __syncthreads();
    }
    cp_wait<0>();
    __syncthreads();
  }
}

// ------------------------------------------------------------------ gap
// The sums of k_gap; FP32 partials per thread over its pixels and rows,
// double-float pairs across runs and threads, FP64 across blocks.
template <int D, int C, int TW = kPipeTW>
__global__ void __launch_bounds__(TW / 4) k_gap_p(Geo<float> g, Args<float> a, int RB,
                                                        double ssd_shift) {
  if (stopped(a)) return;
  using S = PipeSmem<D, C, TW>;
  constexpr int NT = TW / 4;
  constexpr int M = D * C;
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  float* xs = sm;                          // 3 x X4 (halo right)
  float* ys = xs + 3 * S::X4;              // 3 x Y4 (halo left)
  float* fs = ys + 3 * S::Y4;              // 2 x X0
  float* xzs = fs + 2 * S::X0;             // 2 x X0 (D = 3: x one plane forward)
  float* yzs = xzs + 2 * S::X0;            // 2 x Y0 (D = 3: y one plane back)
  const int64_t q_beg = blockIdx.x * (int64_t)TW;
  const int lp0 = threadIdx.x * 4;
  const int64_t nplane = D == 3 ? g.n[1] : 0;
  DF sum[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};   // runs so far
  float inf = 0.f;
  for (int64_t r0 = blockIdx.y * (int64_t)RB; r0 < g.rows; r0 += (int64_t)gridDim.y * RB) {
    const int64_t r1 = r0 + RB < g.rows ? r0 + RB : g.rows;
    float pG = 0.f, pF = 0.f, pGs = 0.f, pFs = 0.f, pinf = -INFINITY;
    // x slot of row r: (r - r0) % 3; y slot of row r: (r - r0 + 1) % 3
    copy_row<C, 0, 4, NT, TW>(xs, a.x, g, r0, q_beg);
    copy_row<C, 0, 4, NT, TW>(xs + S::X4, a.x, g, r0 + 1, q_beg);
    copy_row<M, 4, 0, NT, TW>(ys, a.y, g, r0 - 1, q_beg);
    copy_row<M, 4, 0, NT, TW>(ys + S::Y4, a.y, g, r0, q_beg);
    copy_row<C, 0, 0, NT, TW>(fs, a.f, g, r0, q_beg);
    if (D == 3) {
      copy_row<C, 0, 0, NT, TW>(xzs, a.x, g, r0 + nplane, q_beg);
      copy_row<M, 0, 0, NT, TW>(yzs, a.y, g, r0 - nplane, q_beg);
    }
    cp_commit();
    for (int64_t r = r0; r < r1; ++r) {
      const int k = (int)(r - r0);
      const bool more = r + 1 < r1;
      copy_row<C, 0, 4, NT, TW>(xs + ((k + 2) % 3) * S::X4, a.x, g, r + 2, q_beg, r + 2 <= r1);
      copy_row<M, 4, 0, NT, TW>(ys + ((k + 2) % 3) * S::Y4, a.y, g, r + 1, q_beg, more);
      copy_row<C, 0, 0, NT, TW>(fs + ((k + 1) & 1) * S::X0, a.f, g, r + 1, q_beg, more);
      if (D == 3) {
        copy_row<C, 0, 0, NT, TW>(xzs + ((k + 1) & 1) * S::X0, a.x, g, r + 1 + nplane, q_beg, more);
        copy_row<M, 0, 0, NT, TW>(yzs + ((k + 1) & 1) * S::Y0, a.y, g, r + 1 - nplane, q_beg, more);
      }
      cp_commit();
      cp_wait<1>();
      __syncthreads();
      const float* xc = xs + (k % 3) * S::X4;
      const float* xn = xs + ((k + 1) % 3) * S::X4;
      const float* yc = ys + ((k + 1) % 3) * S::Y4;
      const float* yu = ys + (k % 3) * S::Y4;
      const float* fv = fs + (k & 1) * S::X0;
      const float* xz = xzs + (k & 1) * S::X0;
      const float* yz = yzs + (k & 1) * S::Y0;
      int64_t crow, cz;
      pipe_row_coords<D>(g, r, &crow, &cz);
      const bool has_up = crow > 0, has_dn = crow < g.n[D - 2] - 1;
      const bool has_zb = D == 3 && cz > 0, has_zf = D == 3 && cz < g.n[0] - 1;
      unsigned mk = 0xffffffffu;
      const int64_t qt = q_beg + lp0;
      if (a.mask && qt < g.nl) mk = *reinterpret_cast<const unsigned*>(a.mask + r * g.nl + qt);
      // this thread's quad from the slots (128-bit shared loads)
      float qx[4 * C], qn[4 * C], qf[4 * C], qy[4 * M], qu[4 * M], xr[C], yl[C];
      float qxz[4 * C], qyz[4 * M];
      ldv(qx, xc + lp0 * C);
      ldv(qn, xn + lp0 * C);
      ldv(qf, fv + lp0 * C);
      ldv(qy, yc + (lp0 + 4) * M);
      ldv(qu, yu + (lp0 + 4) * M);
      if (D == 3) {
        ldv(qxz, xz + lp0 * C);
        ldv(qyz, yz + lp0 * M);
      }
#pragma unroll
      for (int k2 = 0; k2 < C; ++k2) {
        xr[k2] = xc[(lp0 + 4) * C + k2];
        yl[k2] = yc[(lp0 + 3) * M + (D - 1) * C + k2];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        const int64_t q = q_beg + lp0 + p;
        if (q >= g.nl) continue;
        const bool on = (mk >> (8 * p)) & 0xffu;
        const bool inx = q < g.nl - 1;
        float n2 = 0.f, y2 = 0.f;
#pragma unroll
        for (int k2 = 0; k2 < C; ++k2) {
          const float xk = qx[p * C + k2], fk = qf[p * C + k2];
          // A^T y
          float s = 0.f;
          const float ihl = g.invh[D - 1], ihr = g.invh[D - 2];
          if (inx) s -= qy[p * M + (D - 1) * C + k2] * ihl;
          if (q > 0) s += (p > 0 ? qy[(p - 1) * M + (D - 1) * C + k2] : yl[k2]) * ihl;
          if (has_dn) s -= qy[p * M + (D - 2) * C + k2] * ihr;
          if (has_up) s += qu[p * M + (D - 2) * C + k2] * ihr;
          if (D == 3) {
            const float ihz = g.invh[0];
            if (has_zf) s -= qy[p * M + k2] * ihz;
            if (has_zb) s += qyz[p * M + k2] * ihz;
          }
          const float ak = g.w[k2] * s;
          if (on) {
            const float d = xk - fk;
            pG += g.vol[k2] * d * d;
            pGs += ak * ak * g.half_rvol[k2] - fk * ak;
          }
          // A x
          const float nb = p < 3 ? qx[(p + 1) * C + k2] : xr[k2];
          const float gl = inx ? g.coef[D - 1][k2] * (nb - xk) : 0.f;
          const float gr = has_dn ? g.coef[D - 2][k2] * (qn[p * C + k2] - xk) : 0.f;
          n2 += gl * gl + gr * gr;
          if (D == 3) {
            const float gz = has_zf ? g.coef[0][k2] * (qxz[p * C + k2] - xk) : 0.f;
            n2 += gz * gz;
          }
        }
#pragma unroll
        for (int j = 0; j < M; ++j) y2 += qy[p * M + j] * qy[p * M + j];
        const float nrm = sqrtf(n2);
        pF += g.use_huber ? (nrm <= g.huber ? n2 * g.half_rhuber : nrm - g.half_huber) : nrm;
        pFs += y2;
        pinf = fmaxf(pinf, sqrtf(y2) - g.lbd);
      }
      __syncthreads();
    }
    cp_wait<0>();
    __syncthreads();
    sum[0] = df_add(sum[0], DF{0.5f * pG, 0.f});
    sum[1] = df_add(sum[1], DF{pF, 0.f});
    sum[2] = df_add(sum[2], DF{pGs, 0.f});
    sum[3] = df_add(sum[3], DF{pFs, 0.f});
    inf = fmaxf(inf, pinf);
  }
  block_reduce_df_and_finish<4>(sum, inf, a.partials, a.ticket, [&](double* tot) {
    write_info(g, a, tot, ssd_shift);
  });
}

}  // namespace rof
}  // namespace opyx
