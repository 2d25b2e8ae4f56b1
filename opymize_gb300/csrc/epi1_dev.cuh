// Exact projection onto a one-dimensional piecewise-linear epigraph
// (EpigraphProj with ndim = 1, opymize/operators/proj.py:388-480), shared by
// the epigraph projection kernel (epigraph.cu) and the fused sublabel
// passes (sublabel.cu).
#pragma once

#include "common.cuh"

namespace opyx {
namespace epi {

// The point (s0, t0) projected onto {(s, t) : t >= v_k s - b_k for every k
// with on[k]} (k < NS), into (ys, yt).
//
// The constraints bound the epigraph of g(s) = max_k (v_k s - b_k), a convex
// piecewise-linear function of one variable.  With the lines sorted by slope
// (then by offset), line k is the graph of g on [lo_k, hi_k],
//   lo_k = max over m < k of (b_k - b_m) / (v_k - v_m),
//   hi_k = min over m > k of (b_k - b_m) / (v_k - v_m)
// (no piece if lo_k > hi_k or an earlier line has the same slope), and the
// pieces follow each other left to right.  The projection p of a point x
// below the graph is the point where x - p lies in the normal cone, found by
// a left-to-right scan with first-order tests only:
//  * inside piece k:  x violates line k and the orthogonal projection onto
//    the line, s = (s0 + v_k (t0 + b_k)) / (1 + v_k^2), is in [lo_k, hi_k];
//  * at the vertex V between pieces L and R:  (V - x).(1, v_L) <= 0 <=
//    (V - x).(1, v_R) (x - V between the two outward normals).
// Comparing squared distances instead resolves p only to sqrt(eps) of the
// distance (in FP32 errors up to 1e-4 on the sublabel model's iterates).
// If rounding leaves no test true, the nearest candidate is taken.  Points
// with no positive violation are kept, as by the active-set method.  The
// arrays are reordered in place; SORTED: they already come in increasing
// slope with distinct slopes among the lines that are on (the sort is
// skipped).  inv (SORTED only, or NULL): per position pair m < k the
// reciprocal 1 / (v_k - v_m) at inv[pair_index(m, k)] and per position k
// 1 / (1 + v_k^2) at inv[NS (NS - 1) / 2 + k], precomputed where the slopes
// are shared by many instances: multiplications then replace the
// divisions.
template <int NS>
OPYX_D constexpr int pair_index(int m, int k) { return m * (2 * NS - m - 1) / 2 + (k - m - 1); }

template <typename T, int NS, bool SORTED = false>
OPYX_D void project1(T (&cv)[NS], T (&cb)[NS], bool (&on)[NS], T s0, T t0, T& ys, T& yt,
                     const T* inv = nullptr) {
  T viol = T(0);
  bool any = false;
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    if (on[k]) {
      const T r = cv[k] * s0 - t0 - cb[k];
      if (!any || r > viol) viol = r;
      any = true;
    }
  }
  ys = s0;
  yt = t0;
  if (!any || !(viol > T(0))) return;
  // sort by (off last, slope, offset): odd-even transposition, static indices
#pragma unroll
  for (int pass = 0; pass < (SORTED ? 0 : NS); ++pass) {
#pragma unroll
    for (int k = pass & 1; k + 1 < NS; k += 2) {
      const bool sw = (!on[k] && on[k + 1]) ||
                      (on[k] && on[k + 1] &&
                       (cv[k + 1] < cv[k] || (cv[k + 1] == cv[k] && cb[k + 1] < cb[k])));
      if (sw) {
        const T tv = cv[k], tb = cb[k];
        const bool to = on[k];
        cv[k] = cv[k + 1]; cb[k] = cb[k + 1]; on[k] = on[k + 1];
        cv[k + 1] = tv; cb[k + 1] = tb; on[k + 1] = to;
      }
    }
  }
  bool found = false, have_prev = false;
  T pv = T(0);                       // slope of the previous piece
  T best = T(INFINITY), fs = s0, ft = t0;
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    if (!on[k]) continue;
    T lo = -T(INFINITY), hi = T(INFINITY);
    bool live = true;
#pragma unroll
    for (int m = 0; m < NS; ++m) {
      if (m == k || !on[m]) continue;
      if (SORTED && inv) {
        // increasing, distinct slopes: m < k has v_m < v_k
        if (m < k) lo = fmax(lo, (cb[k] - cb[m]) * inv[pair_index<NS>(m, k)]);
        else hi = fmin(hi, (cb[m] - cb[k]) * inv[pair_index<NS>(k, m)]);
        continue;
      }
      const T dv = cv[k] - cv[m];
      if (m < k) {
        if (dv > T(0)) lo = fmax(lo, (cb[k] - cb[m]) / dv);
        else live = false;           // an earlier line of the same slope lies above
      } else if (dv < T(0)) {
        hi = fmin(hi, (cb[k] - cb[m]) / dv);
      }
    }
    if (!live || lo > hi) continue;
    // the vertex shared with the previous piece
    if (have_prev && !found) {
      const T vs = lo, vt = cv[k] * lo - cb[k];
      const T dl = (vs - s0) + pv * (vt - t0), dr = (vs - s0) + cv[k] * (vt - t0);
      if (dl <= T(0) && dr >= T(0)) { found = true; ys = vs; yt = vt; }
      const T d = (vs - s0) * (vs - s0) + (vt - t0) * (vt - t0);
      if (d < best) { best = d; fs = vs; ft = vt; }
    }
    // the inside of piece k
    if (!found) {
      const T sk = SORTED && inv ? (s0 + cv[k] * (t0 + cb[k])) * inv[NS * (NS - 1) / 2 + k]
                                 : (s0 + cv[k] * (t0 + cb[k])) / (T(1) + cv[k] * cv[k]);
      const T r = cv[k] * s0 - t0 - cb[k];
      if (r > T(0) && sk >= lo && sk <= hi) {
        found = true;
        ys = sk;
        yt = cv[k] * sk - cb[k];
      } else {
        const T sc = fmin(fmax(sk, lo), hi), tc = cv[k] * sc - cb[k];
        const T d = (sc - s0) * (sc - s0) + (tc - t0) * (tc - t0);
        if (d < best) { best = d; fs = sc; ft = tc; }
      }
    }
    pv = cv[k];
    have_prev = true;
  }
  if (!found) { ys = fs; yt = ft; }
}

// Bit k of the result: line k (of lines sorted by increasing, distinct
// slope) carries a piece of the envelope g -- the liveness test of project1
// alone.  It depends only on the lines, so where they stay fixed over many
// projections it is computed once (project1_live then skips it).
template <typename T, int NS>
OPYX_D unsigned live_mask1(const T (&cv)[NS], const T (&cb)[NS], const bool (&on)[NS]) {
  unsigned mask = 0;
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    if (!on[k]) continue;
    T lo = -T(INFINITY), hi = T(INFINITY);
#pragma unroll
    for (int m = 0; m < NS; ++m) {
      if (m == k || !on[m]) continue;
      const T sl = (cb[k] - cb[m]) / (cv[k] - cv[m]);
      if (m < k) lo = fmax(lo, sl);
      else hi = fmin(hi, sl);
    }
    if (!(lo > hi)) mask |= 1u << k;
  }
  return mask;
}

// project1 for lines sorted by increasing, distinct slope whose envelope's
// pieces are known (bit k of `live`: line k carries one): the scan visits
// the live lines only, each vertex is the intersection of two consecutive
// live lines (one division), and the violation is the largest over the live
// lines (the others lie below the envelope).  Same tests, same order.
template <typename T, int NS>
OPYX_D void project1_live(const T (&cv)[NS], const T (&cb)[NS], unsigned live, T s0, T t0, T& ys,
                          T& yt) {
  ys = s0;
  yt = t0;
  T viol = -T(INFINITY);
#pragma unroll
  for (int k = 0; k < NS; ++k)
    if ((live >> k) & 1u) viol = fmax(viol, cv[k] * s0 - t0 - cb[k]);
  if (!(viol > T(0))) return;
  bool found = false, have = false;
  T pv = T(0), pb = T(0), plo = -T(INFINITY);
  T best = T(INFINITY), fs = s0, ft = t0;
  // the inside of the piece of line (v, b) over [lo, hi]
  auto inside = [&](T v, T b, T lo, T hi) {
    const T sk = (s0 + v * (t0 + b)) / (T(1) + v * v);
    const T r = v * s0 - t0 - b;
    if (r > T(0) && sk >= lo && sk <= hi) {
      found = true;
      ys = sk;
      yt = v * sk - b;
    } else {
      const T sc = fmin(fmax(sk, lo), hi), tc = v * sc - b;
      const T d = (sc - s0) * (sc - s0) + (tc - t0) * (tc - t0);
      if (d < best) { best = d; fs = sc; ft = tc; }
    }
  };
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    if (!((live >> k) & 1u)) continue;
    if (have) {
      const T V = (cb[k] - pb) / (cv[k] - pv);   // vertex: hi of the previous piece, lo of this one
      if (!found) inside(pv, pb, plo, V);
      if (!found) {
        const T vt = cv[k] * V - cb[k];
        const T dl = (V - s0) + pv * (vt - t0), dr = (V - s0) + cv[k] * (vt - t0);
        if (dl <= T(0) && dr >= T(0)) { found = true; ys = V; yt = vt; }
        const T d = (V - s0) * (V - s0) + (vt - t0) * (vt - t0);
        if (d < best) { best = d; fs = V; ft = vt; }
      }
      plo = V;
    }
    pv = cv[k];
    pb = cb[k];
    have = true;
  }
  if (!found && have) inside(pv, pb, plo, T(INFINITY));
  if (!found) { ys = fs; yt = ft; }
}

}  // namespace epi
}  // namespace opyx
