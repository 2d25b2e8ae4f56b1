// One PDHG iteration of the 3-D fused ROF path (one channel) in a single
// sweep over HBM.
//
// The 2-D sweep (rof_sweep.cuh) streams rows and keeps xbar of two rows on
// chip.  In 3-D, pass B at (z, y) needs xbar one plane further, so the unit
// of the stream is a plane tile instead of a row: a CTA owns TY rows y0 ..
// y0+TY-1 of full x-lines (the x extent is the whole row, TW = nl) and a
// range of planes [z0, z1), and at plane step z it runs
//   pass A on plane z, rows y0 .. y0+TY (the last one a halo row whose
//          x_{k+1} is not stored: pass B needs its xbar), and
//   pass B on plane z-1, rows y0 .. y0+TY-1,
// with xbar of planes z-1 and z in shared memory.  Pass A of plane z1 (the
// first plane of the next range) is recomputed as a halo plane.  As in 2-D,
// the sweep reads (x, y) and writes (x2, y2), so no CTA reads a value that
// another CTA rewrites in the same launch; an iteration moves about
// 4*N*(3C + 2K) bytes (256^3: 604 MB instead of 940 MB for two passes), plus
// re-reads of the halo rows and planes, mostly from L2.
//
// The rows of a plane tile are consecutive in memory, so each plane step is
// three 1-D bulk copies (y rows y0-1 .. y0+TY, x and f rows y0 .. y0+TY)
// issued by one thread, completing on an mbarrier (bounded waits; a timeout
// sets info->fault), and two bulk stores (x_{k+1} and y_{k+1} of the owned
// rows).  Threads: TY+1 row groups of TW/P threads, P pixels each; a warp
// never straddles two rows, so x-neighbours come by warp shuffles.  The
// arithmetic of every voxel is that of k_passA_p / k_passB_p (D = 3), so the
// results equal the two passes bit for bit.
#pragma once

#include "rof_sweep.cuh"

namespace opyx {
namespace rof {

template <int TW, int TY>
struct Sweep3Smem {
  static constexpr int M = 3;                      // one channel, three directions
  static constexpr int YS = (TY + 2) * TW * M;     // y rows y0-1 .. y0+TY
  static constexpr int XS = (TY + 1) * TW;         // x, f, xbar rows y0 .. y0+TY
  static constexpr int bytes = 4 * (3 * YS + 2 * XS + 2 * XS + 2 * XS);
};

// Rows [lo, hi) of plane z that exist, clipped to the volume.
OPYX_D unsigned plane_rows(const Geo<float>& g, int64_t z, int64_t lo, int64_t hi, int64_t* r_first,
                           int* skip) {
  const int64_t Yr = g.n[1];
  const int64_t a = lo > 0 ? lo : 0, b = hi < Yr ? hi : Yr;
  if (z < 0 || z >= g.n[0] || b <= a) return 0u;
  *r_first = z * Yr + a;
  *skip = (int)(a - lo);
  return (unsigned)(b - a);
}

template <int TW, int TY>
OPYX_D void issue_plane(const Geo<float>& g, const Args<float>& a, int64_t y0, uint64_t* m,
                        float* ys_prev, int64_t zprev, float* ysl, float* xsl, float* fsl, int64_t z) {
  constexpr int M = 3;
  int64_t ryp = 0, ry = 0, rx = 0;
  int kp = 0, ky = 0, kx = 0;
  const unsigned np = ys_prev ? plane_rows(g, zprev, y0 - 1, y0 + TY + 1, &ryp, &kp) : 0u;
  const unsigned ny = plane_rows(g, z, y0 - 1, y0 + TY + 1, &ry, &ky);
  const unsigned nx = plane_rows(g, z, y0, y0 + TY + 1, &rx, &kx);
  const unsigned by = ny * TW * M * 4, bx = nx * TW * 4;
  const unsigned bp = np * TW * M * 4;
  mbar_arrive_expect(m, bp + by + 2 * bx);
  if (bp) bulk_load(ys_prev + kp * TW * M, a.y + ryp * TW * M, bp, m);
  if (by) bulk_load(ysl + ky * TW * M, a.y + ry * TW * M, by, m);
  if (bx) {
    bulk_load(xsl + kx * TW, a.x + rx * TW, bx, m);
    bulk_load(fsl + kx * TW, a.f + rx * TW, bx, m);
  }
}

// Thread 0: store `nrows` rows of E floats per pixel from a slot to plane z
// starting at row y.
template <int E, int TW>
OPYX_D void store_rows(float* arr, const float* slot, const Geo<float>& g, int64_t z, int64_t y,
                       int64_t nrows) {
  if (nrows <= 0) return;
  fence_proxy_async();
  bulk_store(arr + (z * g.n[1] + y) * TW * E, slot, (unsigned)(nrows * TW * E * 4));
  bulk_commit();
}

template <int TW, int TY, int P>
__global__ void __launch_bounds__((TY + 1) * (TW / P))
k_sweep3(Geo<float> g, Args<float> a, int ZC, int nyt) {
  using S = Sweep3Smem<TW, TY>;
  constexpr int M = 3, NTR = TW / P, NB = 2;
  extern __shared__ float4 smem4[];
  __shared__ __align__(8) uint64_t mbar[NB];
  float* sm = reinterpret_cast<float*>(smem4);
  float* ys = sm;                    // 3 x YS: plane z in slot (z - z0 + 1) % 3
  float* xs = ys + 3 * S::YS;        // 2 x XS: plane z in slot (z - z0) % 2
  float* fs = xs + 2 * S::XS;        // 2 x XS
  float* bs = fs + 2 * S::XS;        // 2 x XS: xbar of plane z in slot (z - z0) & 1
  const int grp = threadIdx.x / NTR;             // row of the tile (TY: the halo row)
  const int lp0 = (threadIdx.x % NTR) * P;
  const int lane = threadIdx.x & 31;
  const bool lead = threadIdx.x == 0;
  const bool pre = g.steps == OPYX_STEPS_PRECOND;
  const PrimalCoefs<float, 1> pc(g, (float)a.tau);
  const float sig_c = (float)a.sigma;
  const float hub_c = 1.f / (1.f + sig_c * g.hub_ratio);
  const int64_t Z = g.n[0], Yr = g.n[1], nl = g.nl;
  if (lead) {
    for (int i = 0; i < NB; ++i) mbar_init(&mbar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // launched chained: the previous kernel may still be draining until here
  chain_wait();
  if (stopped(a)) return;
  __syncthreads();
  unsigned st = 0;
  const int64_t nzc = (Z + ZC - 1) / ZC;
  for (int64_t item = blockIdx.x; item < nzc * nyt; item += gridDim.x) {
    const int64_t y0 = (item % nyt) * TY;
    const int64_t z0 = (item / nyt) * ZC;
    const int64_t z1 = z0 + ZC < Z ? z0 + ZC : Z;
    const int64_t zl = z1 < Z ? z1 : Z - 1;     // last plane whose pass A runs here
    const int64_t own = y0 + TY < Yr ? TY : Yr - y0;   // owned rows that exist
    const int64_t y = y0 + grp;                 // this thread's row (pass A)
    const bool row_ok = y < Yr;
    const unsigned base = st;
    if (lead) {
      bulk_wait_read_all();
      fence_proxy_async();
      issue_plane<TW, TY>(g, a, y0, &mbar[base % NB], ys, z0 - 1, ys + S::YS, xs, fs, z0);
    }
    for (int64_t z = z0; z <= z1; ++z) {
      const int s = (int)(z - z0);
      const bool run_a = z <= zl;
      if (z + 1 <= zl && lead) {
        bulk_wait_read_all();   // stores still reading the slots about to be refilled
        fence_proxy_async();
        issue_plane<TW, TY>(g, a, y0, &mbar[(base + s + 1) % NB], nullptr, 0,
                            ys + ((s + 2) % 3) * S::YS, xs + ((s + 1) & 1) * S::XS,
                            fs + ((s + 1) & 1) * S::XS, z + 1);
      }
      const unsigned cur = base + (unsigned)s;
      bool ok = true;
      if (run_a) ok = mbar_wait(&mbar[cur % NB], (cur / NB) & 1u);
      if (__syncthreads_or(!ok)) {
        if (lead) {
          a.info->fault = 1.0;
          a.info->done = 1.0;
          for (int64_t q = z; q <= zl && q <= z + 1; ++q) {
            const unsigned sq = base + (unsigned)(q - z0);
            mbar_wait(&mbar[sq % NB], (sq / NB) & 1u);
          }
          bulk_wait_all();
        }
        return;
      }
      float* yz = ys + ((s + 1) % 3) * S::YS;          // y_k, plane z (rows y0-1 ..)
      float* yp = ys + (s % 3) * S::YS;                // plane z-1 (y_k; pass B updates it)
      float* xv = xs + (s & 1) * S::XS;
      const float* fv = fs + (s & 1) * S::XS;
      float* bz = bs + (s & 1) * S::XS;                // xbar, plane z
      const float* bp = bs + ((s + 1) & 1) * S::XS;    // xbar, plane z-1
      // ---- pass A, plane z, rows y0 .. y0+TY
      if (run_a && row_ok) {
        const bool has_up = y > 0, has_dn = y < Yr - 1;
        const bool has_zb = z > 0, has_zf = z < Z - 1;
        float qy[P * M], qu[P * M], qz[P * M], qx[P], qf[P], qb[P];
        const float* yc = yz + (grp + 1) * TW * M;
        lds(qy, yc + lp0 * M);
        lds(qu, yz + grp * TW * M + lp0 * M);
        lds(qz, yp + (grp + 1) * TW * M + lp0 * M);
        lds(qx, xv + grp * TW + lp0);
        lds(qf, fv + grp * TW + lp0);
        const float up = __shfl_up_sync(0xffffffffu, qy[(P - 1) * M + 2], 1);
        const float yl = lane ? up : (lp0 > 0 ? yc[(lp0 - 1) * M + 2] : 0.f);
#pragma unroll
        for (int p = 0; p < P; ++p) {
          const int64_t q = lp0 + p;
          const int cb = (int)((q < nl - 1) + (q > 0)) + 3 * (int)(has_dn + has_up) +
                         9 * (int)(has_zf + has_zb);
          float sum = 0.f;
          const float ihl = g.invh[2];
          if (q < nl - 1) sum -= qy[p * M + 2] * ihl;
          if (q > 0) sum += (p > 0 ? qy[(p - 1) * M + 2] : yl) * ihl;
          const float ihr = g.invh[1];
          if (has_dn) sum -= qy[p * M + 1] * ihr;
          if (has_up) sum += qu[p * M + 1] * ihr;
          const float ihz = g.invh[0];
          if (has_zf) sum -= qy[p * M] * ihz;
          if (has_zb) sum += qz[p * M] * ihz;
          const float dv = g.w[0] * sum;
          const float tau = pre ? g.tau_tab[cb][0] : pc.tau;
          const float xo = qx[p];
          float v = xo - tau * dv;
          v = (pre ? g.a_tab[cb][0] : pc.a[0]) * (v + (pre ? g.tv_tab[cb][0] : pc.tv[0]) * qf[p]);
          qx[p] = v;
          qb[p] = g.theta1 * v - g.theta * xo;
        }
        sts(xv + grp * TW + lp0, qx);
        sts(bz + grp * TW + lp0, qb);
      }
      __syncthreads();
      if (lead && run_a && z < z1) store_rows<1, TW>(a.x2, xv, g, z, y0, own);
      // ---- pass B, plane z-1, rows y0 .. y0+TY-1 (in place in its y slot)
      if (z > z0 && grp < TY && row_ok) {
        const bool has_next = y < Yr - 1;
        const bool has_z = z - 1 < Z - 1;
        float qx[P], qn[P], qzn[P], qy[P * M];
        lds(qx, bp + grp * TW + lp0);
        lds(qn, bp + (grp + 1) * TW + lp0);
        lds(qzn, bz + grp * TW + lp0);
        float* yv = yp + (grp + 1) * TW * M + lp0 * M;
        lds(qy, yv);
        const float dn = __shfl_down_sync(0xffffffffu, qx[0], 1);
        const float xr = lane < 31 ? dn : (lp0 + P < TW ? bp[grp * TW + lp0 + P] : 0.f);
#pragma unroll
        for (int p = 0; p < P; ++p) {
          const int64_t q = lp0 + p;
          const bool inx = q < nl - 1;
          float hf[M];
          const float xk = qx[p];
          const float nb = p < P - 1 ? qx[p + 1] : xr;
          const float gl = inx ? g.coef[2][0] * (nb - xk) : 0.f;
          qy[p * M + 2] += (pre ? (inx ? g.sig_pre[2][0] : 0.f) : sig_c) * gl;
          hf[2] = pre ? (inx ? g.hub_pre[2][0] : 1.f) : hub_c;
          const float gr = has_next ? g.coef[1][0] * (qn[p] - xk) : 0.f;
          qy[p * M + 1] += (pre ? (has_next ? g.sig_pre[1][0] : 0.f) : sig_c) * gr;
          hf[1] = pre ? (has_next ? g.hub_pre[1][0] : 1.f) : hub_c;
          const float gz = has_z ? g.coef[0][0] * (qzn[p] - xk) : 0.f;
          qy[p * M] += (pre ? (has_z ? g.sig_pre[0][0] : 0.f) : sig_c) * gz;
          hf[0] = pre ? (has_z ? g.hub_pre[0][0] : 1.f) : hub_c;
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
        sts(yv, qy);
      }
      __syncthreads();
      if (lead && z > z0) store_rows<M, TW>(a.y2, yp + TW * M, g, z - 1, y0, own);
    }
    st = base + (unsigned)(zl - z0 + 1);
  }
  if (lead) bulk_wait_all();
}

}  // namespace rof
}  // namespace opyx
