// Projection onto epigraphs of piecewise-linear convex conjugates, and the
// values of EpigraphInd / EpigraphSupp (opymize/operators/proj.py:388-480,
// proj.cu:222-831; opymize/functionals/epigraph.py:7-127).
//
// Instance (j, i) -- region j, function i -- owns the n+1 values x[j, i, :]
// (n = ndim) and the constraints
//
//     <v[l], y[:n]> - y[n] <= b[i, l]   for l = J[j, k] with I[i, l] set,
//
// i.e. rows a_l = (v[l], -1).  The projection is a tiny strictly convex QP; it
// is solved per thread with the primal active-set method (Nocedal & Wright,
// Numerical Optimization, 2nd ed., Algorithm 16.3), as the reference does.
// The equality-constrained subproblems and the Lagrange multipliers come from
// an orthonormal basis of the working set's normals (|W| <= n+1 <= 4), for
// every n alike (ActiveBasis below).
#include "common.cuh"
#include "epi1_dev.cuh"

namespace opyx {
namespace epi {

constexpr int kThreads = 128;
constexpr int kEvalBlocks = 1024;
constexpr int kCached = 8;

// The constraints of one instance.  NS > 0 (nsub <= NS): read once into
// registers by cache() -- the method scans them several times, and the rows
// b[i, :] and I[i, :] of neighbouring threads lie a row apart, so every scan
// from memory costs a warp one access per thread.  Slots past nsub are off.
// NS = 0: read from memory at every scan.
template <typename T, int ND, int NS>
struct Inst {
  const T* v;          // (npoints, ND)
  const T* brow;       // b[i, :]
  const uint8_t* irow; // I[i, :]
  const int64_t* jrow; // J[j, :]
  int nsub;
  static constexpr int NC = NS > 0 ? NS : 1;
  T cv[NC][ND];
  T cb[NC];
  int cid[NC];
  bool con[NC];

  OPYX_D void cache() {
    if constexpr (NS > 0) {
#pragma unroll
      for (int k = 0; k < NC; ++k) {
        const bool used = k < nsub;
        const int64_t l = used ? jrow[k] : 0;
        cid[k] = (int)l;
        con[k] = used && irow[l];
#pragma unroll
        for (int q = 0; q < ND; ++q) cv[k][q] = used ? v[l * ND + q] : T(0);
        cb[k] = used ? brow[l] : T(0);
      }
    }
  }
  OPYX_D int count() const { return NS > 0 ? NS : nsub; }
  OPYX_D int id(int k) const { return NS > 0 ? cid[k] : (int)jrow[k]; }
  OPYX_D bool on(int k, int l) const { return NS > 0 ? con[k] : irow[l] != 0; }
  OPYX_D const T* row(int k, int l) const { return NS > 0 ? cv[k] : v + (int64_t)l * ND; }
  OPYX_D T b(int k, int l) const { return NS > 0 ? cb[k] : brow[l]; }
};

// a_l . y with a_l = (v[l], -1)
template <typename T, int ND>
OPYX_D T adot(const T* vl, const T* y) {
  T s = -y[ND];
#pragma unroll
  for (int k = 0; k < ND; ++k) s += vl[k] * y[k];
  return s;
}

// Orthonormal basis q_0..q_{m-1} of span{a_w : w in W}, built by modified
// Gram-Schmidt (two passes) from e_0 = a_{W0} and the differences
// e_i = a_{Wi} - a_{W0} = (v_{Wi} - v_{W0}, 0).  Neighbouring constraints
// have nearly parallel normals; their difference vectors keep the basis well
// conditioned where the Gram matrix A_W A_W^T would square the condition
// number (which FP32 iterates cannot afford).  e_i = sum_{k<=i} R[k][i] q_k.
template <typename T, int ND>
struct ActiveBasis {
  static constexpr int N1 = ND + 1;
  T q[N1][N1];
  T R[N1][N1];
  int m;

  OPYX_D bool build(const T (&aw)[N1][ND], int m_) {
    m = m_;
    const T tiny = sizeof(T) == 4 ? T(1e-5) : T(1e-12);
#pragma unroll
    for (int i = 0; i < N1; ++i) {
      if (i >= m) break;
      T e[N1];
#pragma unroll
      for (int k = 0; k < ND; ++k) e[k] = i == 0 ? aw[0][k] : aw[i][k] - aw[0][k];
      e[ND] = i == 0 ? T(-1) : T(0);
      T en = T(0);
#pragma unroll
      for (int k = 0; k < N1; ++k) en += e[k] * e[k];
      en = sqrt(en);
#pragma unroll
      for (int c = 0; c < N1; ++c) R[c][i] = T(0);
#pragma unroll
      for (int pass = 0; pass < 2; ++pass) {
#pragma unroll
        for (int c = 0; c < N1; ++c) {
          if (c >= i) break;
          T dot = T(0);
#pragma unroll
          for (int k = 0; k < N1; ++k) dot += q[c][k] * e[k];
          R[c][i] += dot;
#pragma unroll
          for (int k = 0; k < N1; ++k) e[k] -= dot * q[c][k];
        }
      }
      T nn = T(0);
#pragma unroll
      for (int k = 0; k < N1; ++k) nn += e[k] * e[k];
      nn = sqrt(nn);
      if (!(nn > tiny * en)) return false;   // dependent constraint
      R[i][i] = nn;
      const T inv = T(1) / nn;
#pragma unroll
      for (int k = 0; k < N1; ++k) q[i][k] = e[k] * inv;
    }
    return true;
  }

  // p = d - Q Q^T d: the part of d orthogonal to the active normals
  OPYX_D void project_out(const T* d, T* p) const {
#pragma unroll
    for (int k = 0; k < N1; ++k) p[k] = d[k];
#pragma unroll
    for (int c = 0; c < N1; ++c) {
      if (c >= m) break;
      T dot = T(0);
#pragma unroll
      for (int k = 0; k < N1; ++k) dot += q[c][k] * p[k];
#pragma unroll
      for (int k = 0; k < N1; ++k) p[k] -= dot * q[c][k];
    }
  }

  // lambda with A_W^T lambda = r in the least-squares sense: R mu = Q^T r,
  // then lambda_i = mu_i (i >= 1), lambda_0 = mu_0 - sum_{i>=1} mu_i,
  // since A_W^T lambda = (sum_i lambda_i) e_0 + sum_{i>=1} lambda_i e_i.
  OPYX_D void multipliers(const T* r, T (&lam)[N1]) const {
    T mu[N1];
#pragma unroll
    for (int c = 0; c < N1; ++c) {
      T dot = T(0);
#pragma unroll
      for (int k = 0; k < N1; ++k) dot += q[c][k] * r[k];
      mu[c] = c < m ? dot : T(0);
    }
#pragma unroll
    for (int c = N1 - 1; c >= 0; --c) {
      if (c >= m) continue;
      T sum = mu[c];
#pragma unroll
      for (int k = c + 1; k < N1; ++k)
        if (k < m) sum -= R[c][k] * mu[k];
      mu[c] = sum / R[c][c];
    }
    T rest = T(0);
#pragma unroll
    for (int c = 1; c < N1; ++c) {
      lam[c] = c < m ? mu[c] : T(0);
      rest += lam[c];
    }
    lam[0] = mu[0] - rest;
  }
};

// Largest violation max_l (a_l . y - b_l) over the instance's constraints,
// the constraint attaining it (-1 if none) and its v_l (in wv, if given).
template <typename T, int ND, int NS>
OPYX_D T max_violation(const Inst<T, ND, NS>& in, const T* y, int* arg, T* wv = nullptr) {
  T worst = -INFINITY;
  *arg = -1;
#pragma unroll(NS > 0 ? NS : 1)
  for (int k = 0; k < in.count(); ++k) {
    const int l = in.id(k);
    if (!in.on(k, l)) continue;
    const T* vl = in.row(k, l);
    const T r = adot<T, ND>(vl, y) - in.b(k, l);
    if (r > worst) {
      worst = r;
      *arg = l;
      if (wv) {
#pragma unroll
        for (int q = 0; q < ND; ++q) wv[q] = vl[q];
      }
    }
  }
  return worst;
}

// Projection of one instance.  Returns false when the method did not finish
// within maxiter steps (the last iterate is kept, as the reference does).
//
// Tolerances: `tol` (the reference's 1e-9) bounds the ratio test and the
// descent test in FP64.  FP32 iterates use precision-scaled bounds instead:
// at degenerate vertices (several constraints through one point, as where a
// piecewise-linear function is flat) the ratio of a tight constraint rounds
// to about -1e-8, which an absolute 1e-9 would wrongly read as "behind the
// step" and step through it.  A claimed KKT point is accepted only if it is
// feasible to the same precision; otherwise the instance is reported as
// not converged.
template <typename T, int ND, int NS>
OPYX_D bool project(const Inst<T, ND, NS>& in, const T* x, T* y, int maxiter, T tol) {
  constexpr int N1 = ND + 1, NA = ND + 1;
  constexpr T eps = sizeof(T) == 4 ? T(1.1920929e-7) : T(2.220446049250313e-16);
  const T tol_s = fmax(tol, T(64) * eps);           // step-fraction tolerance
  T xs = T(1);
#pragma unroll
  for (int k = 0; k < N1; ++k) xs = fmax(xs, fabs(x[k]));
  const T tol_feas = T(64) * eps * xs;              // feasibility, absolute
  const T tol_tight = T(8) * eps * xs;              // a constraint counts as tight
  // feasible start: raise the last coordinate by the largest violation
  int first;
  T fv[ND];
  const T viol = max_violation(in, x, &first, fv);
#pragma unroll
  for (int k = 0; k < N1; ++k) y[k] = x[k];
  if (first < 0 || !(viol > T(0))) return true;  // feasible points are fixed
  y[ND] += viol;
  int W[NA];
  T aw[NA][ND];
  int m = 1;
  W[0] = first;
#pragma unroll
  for (int k = 0; k < ND; ++k) aw[0][k] = fv[k];
  // the constraint dropped last: its negative multiplier says the next step
  // leaves it, so it does not take part in that step's ratio test (in FP32
  // a short step's direction is noisy enough to read as "into" it)
  int dropped = -1;
  for (int it = 0; it < maxiter; ++it) {
    // step: the part of x - y orthogonal to the active normals
    T d[N1], p[N1], z[NA];
#pragma unroll
    for (int k = 0; k < N1; ++k) d[k] = x[k] - y[k];
    ActiveBasis<T, ND> basis;
    if (!basis.build(aw, m)) return false;
    basis.project_out(d, p);
    T pn = T(0), dn = T(0);
#pragma unroll
    for (int k = 0; k < N1; ++k) { pn += fabs(p[k]); dn += fabs(d[k]); }
    int blocking = -1;
    T bv[ND];
    bool null_step = false;
    // a step at the rounding level of its own computation (|p| against
    // |x - y|) or below the tightness tolerance is noise: the multipliers
    // decide without it (else, at a degenerate vertex that FP32 places 1e-7
    // off, noise steps are blocked by the vertex's other constraints and
    // the working set cycles through them)
    if (m < NA && pn > fmax(tol_tight, T(64) * eps * dn)) {
      // the nearest constraint outside W that the step would cross.
      // Constraints tight to within tol_tight block at once (s = 0): at a
      // degenerate vertex their ratio (slack / a.p) is rounding noise over
      // a small a.p.  Among the constraints blocking at the smallest step
      // (tight at the step's end point), the one most opposed to the step
      // (largest a.p) is taken, which leaves such a vertex in one exchange.
      const T tol_ap = fmax(tol, T(4) * eps * pn);
      T smin = T(1);
      for (int pass = 0; pass < 2; ++pass) {
        T apb = T(0);
#pragma unroll(NS > 0 ? NS : 1)
        for (int k = 0; k < in.count(); ++k) {
          const int l = in.id(k);
          if (!in.on(k, l)) continue;
          bool act = (int)l == dropped;
#pragma unroll
          for (int a = 0; a < NA; ++a) act |= (a < m && W[a] == (int)l);
          if (act) continue;
          const T* vl = in.row(k, l);
          const T ap = adot<T, ND>(vl, p);
          if (!(ap > tol_ap)) continue;
          const T slack = in.b(k, l) - adot<T, ND>(vl, y);
          const T s = slack > tol_tight ? slack / ap : T(0);
          if (!(s > -tol_s)) continue;
          if (pass == 0) {
            smin = fmin(smin, s);
          } else if (smin < T(1) && slack - smin * ap <= tol_tight && ap > apb) {
            // tight at the step's end point (the ratios themselves carry
            // errors of eps*|b|/slack, far above eps near a degenerate vertex)
            apb = ap;
            blocking = (int)l;
#pragma unroll
            for (int q = 0; q < ND; ++q) bv[q] = vl[q];
          }
        }
      }
      if (smin != T(0)) {
#pragma unroll
        for (int k = 0; k < N1; ++k) y[k] += smin * p[k];
      }
      null_step = smin == T(0);
    }
    dropped = -1;
    if (blocking >= 0) {
      W[m] = blocking;
#pragma unroll
      for (int k = 0; k < ND; ++k) aw[m][k] = bv[k];
      ++m;
      if (m < NA) continue;
    }
    // no blocking constraint (or a full working set): multipliers of
    // x - y = A_W^T lambda decide optimality
#pragma unroll
    for (int k = 0; k < N1; ++k) d[k] = x[k] - y[k];
    if (m > basis.m && !basis.build(aw, m)) return false;   // a constraint was added
    basis.multipliers(d, z);
    // a multiplier counts as negative only beyond the rounding of the
    // multipliers' scale: a zero multiplier at a degenerate vertex that
    // rounds to -1e-9 would otherwise be dropped and re-added forever
    T lscale = T(0);
#pragma unroll
    for (int a = 0; a < NA; ++a)
      if (a < m) lscale = fmax(lscale, fabs(z[a]));
    int amin = -1;
    T lmin = -T(64) * eps * lscale;
#pragma unroll
    for (int a = 0; a < NA; ++a)
      if (a < m && z[a] < lmin) { lmin = z[a]; amin = a; }
    // a constraint that a zero-length step added and the multipliers drop
    // again leaves y where it is: y is optimal to working precision
    if (amin < 0 || (null_step && blocking >= 0 && W[amin] == blocking)) {
      // a KKT point of the working set; it solves the full problem if it is
      // feasible (else a step crossed a constraint: reported, not hidden)
      int lv;
      return !(max_violation(in, y, &lv) > tol_feas);
    }
    // drop the most negative multiplier
    dropped = W[amin];
    --m;
    W[amin] = W[m];
#pragma unroll
    for (int k = 0; k < ND; ++k) aw[amin][k] = aw[m][k];
  }
  return false;
}

template <typename T, int ND, int NS>
__global__ void __launch_bounds__(kThreads)
k_proj(opyx_epigraph e, const T* __restrict__ x, T* y, int maxiter, double tol,
       unsigned* nonconv) {
  constexpr int N1 = ND + 1;
  const int64_t total = e.nregions * e.nfuns;
  unsigned bad = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = t / e.nfuns, i = t - j * e.nfuns;
    Inst<T, ND, NS> in;
    in.v = (const T*)e.v;
    in.brow = (const T*)e.b + i * e.npoints;
    in.irow = e.I + i * e.npoints;
    in.jrow = e.J + j * e.nsubpoints;
    in.nsub = e.nsubpoints;
    in.cache();
    T xi[N1], yi[N1];
#pragma unroll
    for (int k = 0; k < N1; ++k) xi[k] = x[t * N1 + k];
    if (!project<T, ND>(in, xi, yi, maxiter, (T)tol)) ++bad;
#pragma unroll
    for (int k = 0; k < N1; ++k) y[t * N1 + k] = yi[k];
  }
  if (nonconv && bad) atomicAdd(nonconv, bad);
}

// ndim = 1 with at most kDirect constraints per instance: the exact
// projection in one pass, no iterations (project1, epi1_dev.cuh).  The
// result is the QP's solution up to rounding, so instances never count as
// not converged.  Optional transposed copies bt (npoints, nfuns) of b and
// It of I make the reads of neighbouring instances (consecutive i)
// coalesced.
constexpr int kDirect = 16;

template <typename T, int NS>
__global__ void __launch_bounds__(kThreads)
k_proj1(opyx_epigraph e, const T* __restrict__ x, T* y) {
  const int64_t total = e.nregions * e.nfuns;
  const T* v = (const T*)e.v;
  const T* b = (const T*)e.b;
  const T* bt = (const T*)e.bt;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = t / e.nfuns, i = t - j * e.nfuns;
    T cv[NS], cb[NS];
    bool on[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const bool used = k < e.nsubpoints;
      const int64_t l = used ? e.J[j * e.nsubpoints + k] : 0;
      on[k] = used && (e.It ? e.It[l * e.nfuns + i] : e.I[i * e.npoints + l]) != 0;
      cv[k] = on[k] ? v[l] : T(0);
      cb[k] = on[k] ? (bt ? bt[l * e.nfuns + i] : b[i * e.npoints + l]) : T(0);
    }
    T ys, yt;
    project1<T, NS>(cv, cb, on, x[2 * t], x[2 * t + 1], ys, yt);
    y[2 * t] = ys;
    y[2 * t + 1] = yt;
  }
}

// which = 0: EpigraphInd (val 0, infeas = max(0, max_l a_l.x - b_l));
// which = 1: EpigraphSupp (val = sum xt * max_f <eq_f, (x[:n]/xt, 1)>, xt =
// max(eps, |x[n]|); infeas = max(0, -checks[j] x)) (epigraph.py:40-46, :101-112).
template <typename T, int ND>
__global__ void __launch_bounds__(kThreads)
k_eval(opyx_epigraph e, int which, const T* __restrict__ x, double* out, double* partials,
       unsigned* ticket) {
  constexpr int N1 = ND + 1;
  const int64_t total = e.nregions * e.nfuns;
  double val = 0.0, inf = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = t / e.nfuns, i = t - j * e.nfuns;
    double xi[N1];
#pragma unroll
    for (int k = 0; k < N1; ++k) xi[k] = (double)x[t * N1 + k];
    if (which == 0) {
      const T* v = (const T*)e.v;
      const T* b = (const T*)e.b;
      for (int k = 0; k < e.nsubpoints; ++k) {
        const int64_t l = e.J[j * e.nsubpoints + k];
        if (!e.I[i * e.npoints + l]) continue;
        double s = -xi[ND];
#pragma unroll
        for (int q = 0; q < ND; ++q) s += (double)v[l * ND + q] * xi[q];
        inf = fmax(inf, s - (double)b[i * e.npoints + l]);
      }
    } else {
      const double* ch = e.checks + j * N1 * N1;
#pragma unroll
      for (int r = 0; r < N1; ++r) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < N1; ++q) s += ch[r * N1 + q] * xi[q];
        inf = fmax(inf, -s);
      }
      const double xt = fmax(2.220446049250313e-16, fabs(xi[ND]));
      if (e.eq_off) {
        double best = -INFINITY;
        for (int64_t f = e.eq_off[t]; f < e.eq_off[t + 1]; ++f) {
          const double* eq = e.eqns + f * N1;
          double s = eq[ND];
#pragma unroll
          for (int q = 0; q < ND; ++q) s += eq[q] * (xi[q] / xt);
          best = fmax(best, s);
        }
        if (e.eq_off[t + 1] > e.eq_off[t]) val += xt * best;
      } else if (ND == 1) {
        // no faces given (1-D only): the convex envelope g of the points
        // (v_l, b_il), l in J[j], at p = x[0]/xt -- the smallest chord over
        // the point pairs bracketing p; outside the points' range the end
        // edges of the lower hull are extended, which is what the max over
        // the hull's faces gives there
        const T* v = (const T*)e.v;
        const T* b = (const T*)e.b;
        const int64_t* jr = e.J + j * e.nsubpoints;
        const uint8_t* ir = e.I + i * e.npoints;
        const T* bi = b + i * e.npoints;
        double lo = INFINITY, hi = -INFINITY, blo = 0.0, bhi = 0.0;
        for (int k = 0; k < e.nsubpoints; ++k) {
          if (!ir[jr[k]]) continue;
          const double vk = (double)v[jr[k]], bk = (double)bi[jr[k]];
          if (vk < lo || (vk == lo && bk < blo)) { lo = vk; blo = bk; }
          if (vk > hi || (vk == hi && bk < bhi)) { hi = vk; bhi = bk; }
        }
        const double p = xi[0] / xt;
        double best = INFINITY;
        if (lo == hi) {
          best = blo;
        } else if (p < lo || p > hi) {
          // first edge: least chord slope out of the leftmost point; last
          // edge: largest chord slope into the rightmost point
          double s = p < lo ? INFINITY : -INFINITY;
          for (int k = 0; k < e.nsubpoints; ++k) {
            if (!ir[jr[k]]) continue;
            const double vk = (double)v[jr[k]], bk = (double)bi[jr[k]];
            if (p < lo && vk > lo) s = fmin(s, (bk - blo) / (vk - lo));
            if (p > hi && vk < hi) s = fmax(s, (bhi - bk) / (hi - vk));
          }
          best = p < lo ? blo + s * (p - lo) : bhi + s * (p - hi);
        } else {
          for (int a = 0; a < e.nsubpoints; ++a) {
            const int64_t la = jr[a];
            if (!ir[la]) continue;
            const double va = (double)v[la], ba = (double)bi[la];
            if (va == p) { best = fmin(best, ba); continue; }
            if (va > p) continue;
            for (int c = 0; c < e.nsubpoints; ++c) {
              const int64_t lc = jr[c];
              if (!ir[lc]) continue;
              const double vc = (double)v[lc];
              if (!(vc > p)) continue;
              const double bc = (double)bi[lc];
              best = fmin(best, (ba * (vc - p) + bc * (p - va)) / (vc - va));
            }
          }
        }
        if (best < INFINITY) val += xt * best;
      }
    }
  }
  double vals[2] = {val, inf};
  const int ops[2] = {RED_SUM, RED_MAX};
  block_reduce_and_finish<2>(vals, ops, partials, ticket, [&](double* tot) {
    out[0] = which == 0 ? 0.0 : tot[0];
    out[1] = fmax(0.0, tot[1]);
  });
}

static int check(const opyx_epigraph* e) {
  if (!e || e->ndim < 1 || e->ndim > 3) return OPYX_ERR_UNSUPPORTED;
  if (e->nfuns < 0 || e->nregions < 0 || e->npoints < 1 || e->nsubpoints < 1)
    return OPYX_ERR_ARG;
  if (!e->I || !e->J || !e->v || !e->b) return OPYX_ERR_ARG;
  return OPYX_OK;
}

}  // namespace epi
}  // namespace opyx

using namespace opyx;
using namespace opyx::epi;

extern "C" {

int opyx_epigraph_proj(const opyx_epigraph* e, int dtype, const void* x, void* y, int maxiter,
                       double tol, unsigned* nonconv, void* stream) {
  int st = check(e);
  if (st) return st;
  const int64_t total = e->nregions * e->nfuns;
  if (total == 0) return OPYX_OK;
  if (!x || !y || maxiter < 1 || !(tol >= 0)) return OPYX_ERR_ARG;
  const unsigned g = grid_for(total, kThreads, 16);
  cudaStream_t s = (cudaStream_t)stream;
  // up to kCached constraints per instance are held in registers
#define OPYX_EPI_LAUNCH(TT, ND)                                                          \
  (e->nsubpoints <= kCached                                                              \
       ? k_proj<TT, ND, kCached><<<g, kThreads, 0, s>>>(*e, (const TT*)x, (TT*)y, maxiter, \
                                                        tol, nonconv)                     \
       : k_proj<TT, ND, 0><<<g, kThreads, 0, s>>>(*e, (const TT*)x, (TT*)y, maxiter, tol,  \
                                                  nonconv))
  if (e->ndim == 1 && e->nsubpoints <= kDirect && (dtype == OPYX_F32 || dtype == OPYX_F64)) {
    // the direct projection (exact, no iterations)
    if (dtype == OPYX_F32) {
      if (e->nsubpoints <= 8) k_proj1<float, 8><<<g, kThreads, 0, s>>>(*e, (const float*)x, (float*)y);
      else k_proj1<float, kDirect><<<g, kThreads, 0, s>>>(*e, (const float*)x, (float*)y);
    } else {
      if (e->nsubpoints <= 8) k_proj1<double, 8><<<g, kThreads, 0, s>>>(*e, (const double*)x, (double*)y);
      else k_proj1<double, kDirect><<<g, kThreads, 0, s>>>(*e, (const double*)x, (double*)y);
    }
    return check_launch();
  }
  if (dtype == OPYX_F32) {
    if (e->ndim == 1) OPYX_EPI_LAUNCH(float, 1);
    else if (e->ndim == 2) OPYX_EPI_LAUNCH(float, 2);
    else OPYX_EPI_LAUNCH(float, 3);
  } else if (dtype == OPYX_F64) {
    if (e->ndim == 1) OPYX_EPI_LAUNCH(double, 1);
    else if (e->ndim == 2) OPYX_EPI_LAUNCH(double, 2);
    else OPYX_EPI_LAUNCH(double, 3);
  } else {
    return OPYX_ERR_ARG;
  }
#undef OPYX_EPI_LAUNCH
  return check_launch();
}

int opyx_epigraph_eval(const opyx_epigraph* e, int dtype, int which, const void* x,
                       double* out, void* ws, void* stream) {
  int st = check(e);
  if (st) return st;
  if (which != 0 && which != 1) return OPYX_ERR_ARG;
  if (which == 1 && !e->checks) return OPYX_ERR_ARG;
  if (which == 1 && !e->eq_off && e->ndim != 1) return OPYX_ERR_UNSUPPORTED;
  if (which == 1 && e->eq_off && !e->eqns) return OPYX_ERR_ARG;
  if (!out || !ws || ((uintptr_t)ws & 7)) return OPYX_ERR_WORKSPACE;
  const int64_t total = e->nregions * e->nfuns;
  if (total > 0 && !x) return OPYX_ERR_ARG;
  double* partials = (double*)ws;
  unsigned* ticket = (unsigned*)((char*)ws + (size_t)kEvalBlocks * 8 * sizeof(double));
  unsigned g = grid_for(total > 0 ? total : 1, kThreads, 4);
  if (g > (unsigned)kEvalBlocks) g = kEvalBlocks;
  cudaStream_t s = (cudaStream_t)stream;
#define OPYX_EPI_EVAL(TT, ND)                                                          \
  k_eval<TT, ND><<<g, kThreads, 0, s>>>(*e, which, (const TT*)x, out, partials, ticket)
  if (dtype == OPYX_F32) {
    if (e->ndim == 1) OPYX_EPI_EVAL(float, 1);
    else if (e->ndim == 2) OPYX_EPI_EVAL(float, 2);
    else OPYX_EPI_EVAL(float, 3);
  } else if (dtype == OPYX_F64) {
    if (e->ndim == 1) OPYX_EPI_EVAL(double, 1);
    else if (e->ndim == 2) OPYX_EPI_EVAL(double, 2);
    else OPYX_EPI_EVAL(double, 3);
  } else {
    return OPYX_ERR_ARG;
  }
#undef OPYX_EPI_EVAL
  return check_launch();
}

}  // extern "C"
