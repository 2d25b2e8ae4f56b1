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
// Rows move in and out as 1-D bulk asynchronous copies (TMA) issued by one
// thread: loads complete on an mbarrier (two, alternating per stage; every
// wait is bounded and a timeout sets info->fault and ends the kernel),
// stores are bulk groups drained before their slot is refilled.  The other
// threads only compute.  Shared memory per CTA (TW = 512): y ring 3 x (TW+8)
// x K (4-pixel halo both sides), x and f rings 2 x (TW+4) x C (right halo),
// xbar 2 x (TW+4) x C.
// Requirements as rof_pipe.cuh (checked on the host); 2-D only (the
// neighbour one plane away in 3-D would need a plane of xbar on chip).
#pragma once

#include "rof_pipe.cuh"

namespace opyx {
namespace rof {

// Rows of prefetch (DP): the bulk load of row r + DP is issued when row r
// is computed.  One channel's row steps are short, so two rows keep DRAM
// latency hidden; three or four channels keep one (their rings would cost an
// SM one of its three CTAs).
constexpr int sweep_depth(int C) { return C <= 2 ? 2 : 1; }
constexpr int kSweepMaxBars = 3;   // mbarriers per CTA: DP + 1 stages in flight

template <int C, int TW = kPipeTW, int DP = 1>
struct SweepSmem {
  static constexpr int M = 2 * C;
  static constexpr int X4 = (TW + 4) * C;   // right halo
  static constexpr int Y44 = (TW + 8) * M;  // 4-pixel halo on both sides
  static constexpr int NY = DP + 2;         // y rows r-1 .. r+DP
  static constexpr int NX = DP + 1;         // x, f rows r .. r+DP
  static constexpr int bytes = 4 * (NY * Y44 + NX * X4 + NX * X4 + 2 * X4);
};

// Pixels per thread of the sweep: 2 (256 threads per 512-pixel tile), twice
// the resident warps of 4-pixel quads at the same shared memory per pixel --
// the sweep does both passes' arithmetic per byte and is latency-bound.
constexpr int kSweepP = 2;
constexpr int kSweepThreads = kPipeTW / kSweepP;   // of a 512-pixel tile

// Pixels per thread by channel count: one channel does a third of the
// arithmetic per row step of three, so its CTAs are made smaller (4 pixels
// per thread) and twice as many of them overlap their row pipelines on an SM.
constexpr int sweep_p(int C) { return C == 1 ? 4 : kSweepP; }
// Resident CTAs per SM the register budget is fitted to.
constexpr int sweep_min_blocks(int TW, int P) {
  return (P == 4 ? 6 : 3) * kPipeTW / TW > 32 ? 32 : (P == 4 ? 6 : 3) * kPipeTW / TW;
}

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
// WARP: called by all 32 lanes of a warp on consecutive pixel groups (the
// left neighbour's y comes from the lane below by a shuffle; lane 0 reads
// shared memory), else by a single thread (the halo pixel).
template <int C, int NP, bool WARP = true>
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
  if (WARP) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k2 = 0; k2 < C; ++k2) {
      const float up = __shfl_up_sync(0xffffffffu, qy[(NP - 1) * M + (D - 1) * C + k2], 1);
      yl[k2] = lane ? up : yc[(lp + 3) * M + (D - 1) * C + k2];
    }
  } else {
#pragma unroll
    for (int k2 = 0; k2 < C; ++k2) yl[k2] = yc[(lp + 3) * M + (D - 1) * C + k2];
  }
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

// ---- bulk asynchronous copies (TMA, 1-D) and their mbarriers
constexpr int kMbarSpin = 1 << 22;   // bound on mbarrier polls (each may suspend)

OPYX_D unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
OPYX_D void mbar_init(uint64_t* m, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}
OPYX_D void mbar_arrive_expect(uint64_t* m, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)),
               "r"(bytes) : "memory");
}
OPYX_D bool mbar_try(uint64_t* m, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(smem_u32(m)), "r"(parity) : "memory");
  return ok != 0;
}
// Bounded wait for the phase of parity `parity`; false if the bound ran out.
OPYX_D bool mbar_wait(uint64_t* m, unsigned parity) {
  for (int i = 0; i < kMbarSpin; ++i)
    if (mbar_try(m, parity)) return true;
  return false;
}
OPYX_D void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* m) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(m)) : "memory");
}
OPYX_D void bulk_store(void* dst, const void* src, unsigned bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
               "r"(smem_u32(src)), "r"(bytes) : "memory");
}
OPYX_D void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
OPYX_D void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
OPYX_D void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
OPYX_D void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// The in-image part of row r for a slot holding pixels [q_beg - HL,
// q_beg + TW + HR): bytes (0 if the row is outside the image), the first
// pixel's offset in the slot and its index in the array.  Slot pixels
// outside the image are left as they are: every use of them in the sweep is
// masked by the boundary tests.  Sizes and addresses are multiples of 16
// bytes because the last axis is a multiple of 4 and the arrays 16-byte
// aligned (checked on the host).
template <int E, int HL, int HR, int TW>
OPYX_D unsigned row_span(const Geo<float>& g, int64_t r, int64_t q_beg, int* off_px,
                         int64_t* src_px) {
  if (r < 0 || r >= g.rows) return 0u;
  const int64_t lo_slot = q_beg - HL;
  const int64_t lo = lo_slot > 0 ? lo_slot : 0;
  const int64_t hi_slot = q_beg + TW + HR;
  const int64_t hi = hi_slot < g.nl ? hi_slot : g.nl;
  if (hi <= lo) return 0u;
  *off_px = (int)(lo - lo_slot);
  *src_px = r * g.nl + lo;
  return (unsigned)((hi - lo) * E * 4);
}

// Thread 0: announce and issue the copies of one stage (rows for y, x, f).
template <int C, int TW>
OPYX_D void issue_stage(const Geo<float>& g, const Args<float>& a, int64_t q_beg, uint64_t* m,
                        float* ys0, int64_t ry0, float* ys1, int64_t ry1, float* xsl, float* fsl,
                        int64_t rx) {
  constexpr int M = 2 * C;
  int oy0 = 0, oy1 = 0, ox = 0, of = 0;
  int64_t sy0 = 0, sy1 = 0, sx = 0, sf = 0;
  const unsigned by0 = ys0 ? row_span<M, 4, 4, TW>(g, ry0, q_beg, &oy0, &sy0) : 0u;
  const unsigned by1 = ys1 ? row_span<M, 4, 4, TW>(g, ry1, q_beg, &oy1, &sy1) : 0u;
  const unsigned bx = row_span<C, 0, 4, TW>(g, rx, q_beg, &ox, &sx);
  const unsigned bf = row_span<C, 0, 4, TW>(g, rx, q_beg, &of, &sf);
  mbar_arrive_expect(m, by0 + by1 + bx + bf);
  if (by0) bulk_load(ys0 + oy0 * M, a.y + sy0 * M, by0, m);
  if (by1) bulk_load(ys1 + oy1 * M, a.y + sy1 * M, by1, m);
  if (bx) bulk_load(xsl + ox * C, a.x + sx * C, bx, m);
  if (bf) bulk_load(fsl + of * C, a.f + sf * C, bf, m);
}

// Thread 0: store the pixels [q_beg, min(q_beg + TW, q_end)) of a slot
// (after HL halo pixels) to row r.
template <int E, int HL, int TW>
OPYX_D void store_span(float* arr, const float* slot, const Geo<float>& g, int64_t r,
                       int64_t q_beg, int64_t q_end) {
  const int64_t lim = q_end < g.nl ? q_end : g.nl;
  const int64_t hi = q_beg + TW < lim ? q_beg + TW : lim;
  if (hi <= q_beg) return;
  fence_proxy_async();   // the threads' shared-memory writes, before the copy reads them
  bulk_store(arr + (r * g.nl + q_beg) * E, slot + HL * E, (unsigned)((hi - q_beg) * E * 4));
  bulk_commit();
}

// The primal-dual gap of the state a sweep starts from (x_k, y_k), summed
// from the rows the sweep has in shared memory anyway: at row step r the
// terms of row r that need only rows r - 1 and r (G(x), G*(-A^T y), |y|^2,
// the infeasibility, the horizontal part of |A x|^2), and the vertical part of
// row r - 1 from x_k of rows r - 1 (kept in registers) and r.  The per-pixel
// arithmetic is that of k_gap_p; FP32 sums per thread over its run,
// double-float pairs across runs, threads and CTAs (the last CTA folds them
// and runs the stop test).
template <int C, int P>
struct SweepGap {
  float pG = 0.f, pF = 0.f, pGs = 0.f, pFs = 0.f, pinf = -INFINITY;   // this run
  DF sum[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};      // runs so far
  float xp[P * C];   // x_k of the previous row at this thread's pixels
  float hp[P];       // horizontal |A x|^2 of the previous row
  OPYX_D void fold_run() {
    sum[0] = df_add(sum[0], DF{0.5f * pG, 0.f});
    sum[1] = df_add(sum[1], DF{pF, 0.f});
    sum[2] = df_add(sum[2], DF{pGs, 0.f});
    sum[3] = df_add(sum[3], DF{pFs, 0.f});
    pG = pF = pGs = pFs = 0.f;
  }
};

// Square root for the gap sums: the hardware approximation (sqrt.approx.f32),
// whose error is of the order of the FP32 rounding the sums carry anyway (the
// gap parity tests bound the effect); the IEEE-rounded sqrtf takes several
// more instructions per call, two calls per pixel.
OPYX_D float gap_sqrt(float v) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}

// |A x|^2 of pixel p of the previous row is complete: its F term.
template <int C, int P>
OPYX_D void gap_f_term(const Geo<float>& g, SweepGap<C, P>& acc, float n2) {
  const float nrm = gap_sqrt(n2);
  acc.pF += g.use_huber ? (nrm <= g.huber ? n2 * g.half_rhuber : nrm - g.half_huber) : nrm;
}

// Row step r of a run [r0, r1) with x_k row r in `xv` (not yet overwritten
// by x_{k+1}), y_k rows r and r - 1 in `yc`, `yu`, f row r in `fv`; called
// by every thread of the CTA (warp shuffles).  Finishes row r - 1 (r > r0)
// and, for r < r1, sums the terms of row r.  Pixel tests in tile-local
// 32-bit indices: nq pixels of the tile lie in the image, the first lx have a
// right neighbour.
template <int C, int P>
OPYX_D void gap_row(const Geo<float>& g, const Args<float>& a, const float* yc, const float* yu,
                    const float* xv, const float* fv, int64_t r, int64_t r0, int64_t r1,
                    int64_t q_beg, int lp0, int nq, int lx, SweepGap<C, P>& acc) {
  constexpr int D = 2, M = D * C;
  const int lane = threadIdx.x & 31;
  float qx[P * C], xr[C];
  lds(qx, xv + lp0 * C);
#pragma unroll
  for (int k2 = 0; k2 < C; ++k2) {
    const float dn = __shfl_down_sync(0xffffffffu, qx[k2], 1);
    xr[k2] = lane < 31 ? dn : xv[(lp0 + P) * C + k2];
  }
  if (r > r0) {
    // row r - 1 has row r below it
#pragma unroll
    for (int p = 0; p < P; ++p) {
      float n2 = acc.hp[p];
#pragma unroll
      for (int k2 = 0; k2 < C; ++k2) {
        const float gr = g.coef[D - 2][k2] * (qx[p * C + k2] - acc.xp[p * C + k2]);
        n2 = fmaf(gr, gr, n2);
      }
      if (lp0 + p < nq) gap_f_term(g, acc, n2);
    }
  }
  if (r >= r1) return;
  float qy[P * M], qu[P * M], qf[P * C], yl[C];
  lds(qy, yc + (lp0 + 4) * M);
  lds(qu, yu + (lp0 + 4) * M);
  lds(qf, fv + lp0 * C);
#pragma unroll
  for (int k2 = 0; k2 < C; ++k2) {
    const float up = __shfl_up_sync(0xffffffffu, qy[(P - 1) * M + (D - 1) * C + k2], 1);
    yl[k2] = lane ? up : yc[(lp0 + 3) * M + (D - 1) * C + k2];
  }
  const bool has_up = r > 0, has_dn = r < g.rows - 1;
  const uint8_t* mrow = a.mask ? a.mask + r * g.nl + q_beg : nullptr;
#pragma unroll
  for (int p = 0; p < P; ++p) {
    const int lq = lp0 + p;
    const bool in = lq < nq, inx = lq < lx, has_l = q_beg + lq > 0;
    const bool on = in && (!mrow || mrow[lq]);
    float h2 = 0.f, y2 = 0.f;
#pragma unroll
    for (int k2 = 0; k2 < C; ++k2) {
      const float xk = qx[p * C + k2], fk = qf[p * C + k2];
      const float ihl = g.invh[D - 1], ihr = g.invh[D - 2];
      float s = inx ? -qy[p * M + (D - 1) * C + k2] * ihl : 0.f;
      if (has_l) s = fmaf(p > 0 ? qy[(p - 1) * M + (D - 1) * C + k2] : yl[k2], ihl, s);
      if (has_dn) s = fmaf(-qy[p * M + (D - 2) * C + k2], ihr, s);
      if (has_up) s = fmaf(qu[p * M + (D - 2) * C + k2], ihr, s);
      const float ak = g.w[k2] * s;
      if (on) {
        const float d = xk - fk;
        acc.pG = fmaf(g.vol[k2] * d, d, acc.pG);
        acc.pGs = fmaf(ak, fmaf(ak, g.half_rvol[k2], -fk), acc.pGs);
      }
      const float nb = p < P - 1 ? qx[(p + 1) * C + k2] : xr[k2];
      const float gl = inx ? g.coef[D - 1][k2] * (nb - xk) : 0.f;
      h2 = fmaf(gl, gl, h2);
    }
#pragma unroll
    for (int j = 0; j < M; ++j) y2 = fmaf(qy[p * M + j], qy[p * M + j], y2);
    if (in) {
      acc.pFs += y2;
      acc.pinf = fmaxf(acc.pinf, gap_sqrt(y2) - g.lbd);
      if (!has_dn) gap_f_term(g, acc, h2);   // the last row of the image: no vertical part
    }
    acc.hp[p] = h2;
  }
#pragma unroll
  for (int j = 0; j < P * C; ++j) acc.xp[j] = qx[j];
}

// One run of rows [r0, r1) of the column tile [q_beg, q_end) (at most TW
// pixels): the body of the sweep, shared by the single-instance and the
// batched kernels.  Pixels of the slot past q_end are computed from the
// loaded rows but not stored (their own tile stores them).  `st` counts the
// stages this CTA has issued on its mbarriers.  Returns false if a copy did
// not arrive within the wait bound (info->fault is then set).
// GAP: also sum the gap of the state it starts from into *gap (single-image
// tiles only: q_end = g.nl).
template <int C, int TW, int P, int DP, bool GAP = false>
OPYX_D bool sweep_rows(const Geo<float>& g, const Args<float>& a, int64_t q_beg, int64_t q_end,
                       int64_t r0, int64_t r1, uint64_t* mbar, unsigned& st, float* sm,
                       SweepGap<C, P>* gap = nullptr) {
  using S = SweepSmem<C, TW, DP>;
  constexpr int D = 2, M = D * C, NT = TW / P, NB = DP + 1;
  float* ys = sm;                          // NY x Y44: row q in slot (q - r0 + 1) % NY
  float* xs = ys + S::NY * S::Y44;         // NX x X4 : x_k, then x_{k+1}; row q in (q - r0) % NX
  float* fs = xs + S::NX * S::X4;          // NX x X4
  float* bs = fs + S::NX * S::X4;          // 2 x X4 : xbar rows, slot (q - r0) & 1
  const int lp0 = threadIdx.x * P;
  const bool lead = threadIdx.x == 0;        // issues the bulk copies
  const bool halo = threadIdx.x == NT - 1;   // also computes xbar at pixel TW
  const bool pre = g.steps == OPYX_STEPS_PRECOND;
  const PrimalCoefs<float, C> pc(g, (float)a.tau);
  const float sig_c = (float)a.sigma;
  const float hub_c = 1.f / (1.f + sig_c * g.hub_ratio);
  const int64_t rl = r1 < g.rows ? r1 : r1 - 1;   // last row whose pass A runs here
  // pixels of the tile in the image / with a right neighbour (gap sums)
  const int gap_nq = (int)(g.nl - q_beg < TW ? g.nl - q_beg : TW);
  const int gap_lx = (int)(g.nl - 1 - q_beg < TW ? g.nl - 1 - q_beg : TW);
  // stage of row q (r0 <= q <= rl) is base + (q - r0), on mbar[stage % NB]
  const unsigned base = st;
  if (lead) {
    bulk_wait_read_all();
    fence_proxy_async();
    for (int64_t q = r0; q <= rl && q < r0 + DP; ++q) {
      const unsigned sq = base + (unsigned)(q - r0);
      const int kq = (int)(q - r0);
      issue_stage<C, TW>(g, a, q_beg, &mbar[sq % NB], q == r0 ? ys : nullptr, r0 - 1,
                         ys + ((kq + 1) % S::NY) * S::Y44, q, xs + (kq % S::NX) * S::X4,
                         fs + (kq % S::NX) * S::X4, q);
    }
  }
  for (int64_t r = r0; r <= r1; ++r) {
    const int k = (int)(r - r0);
    const bool run_a = r <= rl;
    const int64_t rn = r + DP;                 // row whose copies start now
    if (rn <= rl && lead) {
      bulk_wait_read_all();   // stores still reading the slots about to be refilled
      fence_proxy_async();
      const int kn = (int)(rn - r0);
      issue_stage<C, TW>(g, a, q_beg, &mbar[(base + (unsigned)kn) % NB], nullptr, 0,
                         ys + ((kn + 1) % S::NY) * S::Y44, rn, xs + (kn % S::NX) * S::X4,
                         fs + (kn % S::NX) * S::X4, rn);
    }
    const unsigned cur = base + (unsigned)k;
    bool ok = true;
    if (run_a) ok = mbar_wait(&mbar[cur % NB], (cur / NB) & 1u);
    if (__syncthreads_or(!ok)) {
      // a copy did not arrive within the bound: flag it, give the copies
      // in flight a bounded chance to land, and leave
      if (lead) {
        a.info->fault = 1.0;
        a.info->done = 1.0;
        for (int64_t q = r; q <= rl && q <= rn; ++q) {   // every stage still in flight
          const unsigned sq = base + (unsigned)(q - r0);
          mbar_wait(&mbar[sq % NB], (sq / NB) & 1u);
        }
        bulk_wait_all();
      }
      return false;
    }
    const float* yc = ys + ((k + 1) % S::NY) * S::Y44;    // y_k row r
    float* yu = ys + (k % S::NY) * S::Y44;                // y_k row r - 1
    float* xv = xs + (k % S::NX) * S::X4;
    const float* fv = fs + (k % S::NX) * S::X4;
    float* bc = bs + (k & 1) * S::X4;                     // xbar row r
    const float* bu = bs + ((k + 1) & 1) * S::X4;         // xbar row r - 1
    // ---- pass A, row r (and xbar at the first pixel past the tile)
    if (run_a) {
      // (both read shared memory only; the gap first, so that its arrays
      // and pass A's are not live at once)
      if (GAP) gap_row<C, P>(g, a, yc, yu, xv, fv, r, r0, r1, q_beg, lp0, gap_nq, gap_lx, *gap);
      float qx[P * C], qb[P * C];
      sweep_a<C, P>(g, a, pc, pre, yc, yu, xv, fv, r, q_beg, lp0, qx, qb);
      float hb[C];
      if (halo) {
        float hx[C];
        sweep_a<C, 1, false>(g, a, pc, pre, yc, yu, xv, fv, r, q_beg, TW, hx, hb);
      }
      __syncthreads();   // every thread has read the x_k values it needs
      sts(xv + lp0 * C, qx);
      sts(bc + lp0 * C, qb);
      if (halo) {
#pragma unroll
        for (int k2 = 0; k2 < C; ++k2) bc[TW * C + k2] = hb[k2];
      }
    }
    __syncthreads();
    if (lead && r < r1) store_span<C, 0, TW>(a.x2, xv, g, r, q_beg, q_end);
    // ---- pass B, row r - 1 (as k_passB_p), in place in its y slot
    if (r > r0) {
      const int64_t rb = r - 1;
      const bool has_next = rb < g.rows - 1;
      float qx[P * C], qn[P * C], qy[P * M], xr[C];
      lds(qx, bu + lp0 * C);
      lds(qn, bc + lp0 * C);
      lds(qy, yu + (lp0 + 4) * M);
      {
        // right neighbour's xbar from the lane above; lane 31 reads shared
        // memory (for the CTA's last thread: the halo pixel)
        const int lane = threadIdx.x & 31;
#pragma unroll
        for (int k2 = 0; k2 < C; ++k2) {
          const float dn = __shfl_down_sync(0xffffffffu, qx[k2], 1);
          xr[k2] = lane < 31 ? dn : bu[(lp0 + P) * C + k2];
        }
      }
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
      if (lead) store_span<M, 4, TW>(a.y2, yu, g, rb, q_beg, q_end);
    }
    __syncthreads();
  }
  st = base + (unsigned)(rl - r0 + 1);
  if (GAP) gap->fold_run();
  return true;
}

// GAP: the first sweep of a check chunk, which also computes the gap of the
// state it reads (opyx_rof_gap_iterate) and runs the stop test on it.
template <int C, int TW = kPipeTW, int P = kSweepP, int DP = 1, bool GAP = false>
__global__ void __launch_bounds__(TW / P, GAP && C >= 3 ? 2 : sweep_min_blocks(TW, P))
k_sweep(Geo<float> g, Args<float> a, int RB, double ssd_shift) {
  extern __shared__ float4 smem4[];
  __shared__ __align__(8) uint64_t mbar[kSweepMaxBars];
  float* sm = reinterpret_cast<float*>(smem4);
  const int64_t q_beg = blockIdx.x * (int64_t)TW;
  const bool lead = threadIdx.x == 0;
  if (lead) {
    for (int i = 0; i < kSweepMaxBars; ++i) mbar_init(&mbar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // launched chained: the previous kernel may still be draining until here
  chain_wait();
  if (stopped(a)) return;
  __syncthreads();
  unsigned st = 0;   // stages issued so far; stage s uses mbar[s % (DP+1)]
  if constexpr (!GAP) {
    for (int64_t r0 = blockIdx.y * (int64_t)RB; r0 < g.rows; r0 += (int64_t)gridDim.y * RB) {
      const int64_t r1 = r0 + RB < g.rows ? r0 + RB : g.rows;
      if (!sweep_rows<C, TW, P, DP>(g, a, q_beg, g.nl, r0, r1, mbar, st, sm)) return;
    }
    if (lead) bulk_wait_all();   // the stores have left shared memory and landed
  } else {
    SweepGap<C, P> acc;
    bool ok = true;
    for (int64_t r0 = blockIdx.y * (int64_t)RB; ok && r0 < g.rows; r0 += (int64_t)gridDim.y * RB) {
      const int64_t r1 = r0 + RB < g.rows ? r0 + RB : g.rows;
      ok = sweep_rows<C, TW, P, DP, true>(g, a, q_beg, g.nl, r0, r1, mbar, st, sm, &acc);
    }
    if (ok && lead) bulk_wait_all();
    // every CTA takes part (also one whose copies timed out: the fault flag
    // is then set and the record is not used), so the ticket completes;
    // the infeasibility max(|y| - lbd) is taken with 0 as k_gap_p does
    block_reduce_df_and_finish<4>(acc.sum, fmaxf(acc.pinf, 0.f), a.partials, a.ticket,
                                  [&](double* tot) { write_info(g, a, tot, ssd_shift); });
  }
}

}  // namespace rof
}  // namespace opyx
