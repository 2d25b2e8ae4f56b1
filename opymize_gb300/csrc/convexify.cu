// Piecewise convexification of sampled functions (host code, no device work):
// for every function i and region j, the lower convex hull of the graph
// points (v_k, vals[i, k]) over the region's sample points k = regions[j, :]
// -- the base points that span it and its faces -- as the reference computes
// with piecewise_convexify (opymize/quickhull/__init__.pyx:8-140, hull code
// convexhull.cpp).  The reference's 2-D and 3-D paths wrap QuickHull and
// Qhull, which are un-vendored submodules; here the 1-D hull is the
// reference's own gift-wrapping rule and the 2-D and 3-D hulls a direct
// enumeration of supporting planes and hyperplanes, all in double precision.
//
// Semantics kept from the reference (they decide the base masks):
//  * 1-D: from the leftmost point, the next hull point is the one with the
//    smallest slope, slopes rounded to a grid of 1e-9 and ties going to the
//    farthest point, so points on a straight piece are not base points
//    (convexhull.cpp:192-216; double here where the reference rounds in long
//    double).
//  * 2-D: the first three points of a region are its triangle's corners and
//    always base points; another point is a base point when its graph point
//    lies more than 1e-9 below the plane through the corners' graph points
//    (unit normal) and is a vertex of the lower hull; a face is kept when its
//    three points are base points, other than the corner triangle; a region
//    without such faces keeps the corner triangle; a function constant on a
//    region gives the corner triangle (convexhull.cpp:118-183,
//    __init__.pyx:117-135).  3-D: the same with the tetrahedron's four
//    corners, hyperplanes and tetrahedral faces.
//  * base[i, :] is assigned region by region, in region order.
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "opyx.h"

namespace opyx {
namespace cvx {

constexpr double kTol = 1e-9;

struct V3 {
  double x, y, z;
};

inline V3 sub(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 cross(const V3& a, const V3& b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Downward unit normal of the plane through a, b, c (left unscaled when its
// squared length is below the tolerance, as the reference's normalize).
inline V3 lower_normal(const V3& a, const V3& b, const V3& c) {
  V3 n = cross(sub(b, a), sub(c, a));
  if (n.z > 0) n = {-n.x, -n.y, -n.z};
  const double l2 = dot(n, n);
  if (l2 >= kTol) {
    const double s = 1.0 / std::sqrt(l2);
    n = {n.x * s, n.y * s, n.z * s};
  }
  return n;
}

struct Problem {
  int ndim;
  int64_t npoints, nfuns, nregions;
  int nsub, max_faces;
  const double* points;
  const double* vals;
  const int64_t* regions;
  uint8_t* base;
  int32_t* faces;
  int32_t* nfaces;
  std::vector<int> order;   // 1-D: each region's positions sorted by abscissa
};

// ---------------------------------------------------------------- 1-D
static void region_1d(const Problem& P, int64_t i, int64_t j, double* x, double* z,
                      uint8_t* keep) {
  const int n = P.nsub;
  const int* ord = P.order.data() + j * n;
  const int64_t* reg = P.regions + j * n;
  for (int k = 0; k < n; ++k) {
    const int64_t l = reg[ord[k]];
    x[k] = P.points[l];
    z[k] = P.vals[i * P.npoints + l];
    keep[k] = 1;
  }
  int a = 0;
  while (a < n - 1) {
    double best = INFINITY;
    int next = a + 1;
    for (int m = a + 1; m < n; ++m) {
      double s = (z[m] - z[a]) / (x[m] - x[a]);
      s = kTol * std::round(s / kTol);
      if (s <= best) {
        best = s;
        next = m;
      }
    }
    for (int m = a + 1; m < next; ++m) keep[m] = 0;
    a = next;
  }
  uint8_t* brow = P.base + i * P.npoints;
  for (int k = 0; k < n; ++k) brow[reg[ord[k]]] = keep[k];
  int32_t* f = P.faces + ((i * P.nregions + j) * P.max_faces) * 2;
  int nf = 0, prev = -1;
  for (int k = 0; k < n; ++k) {
    if (!keep[k]) continue;
    if (prev >= 0) {
      f[2 * nf] = ord[prev];
      f[2 * nf + 1] = ord[k];
      ++nf;
    }
    prev = k;
  }
  P.nfaces[i * P.nregions + j] = nf;
}

// ---------------------------------------------------------------- 2-D
// 2-D convex hull of the xy positions of `idx` (counter-clockwise, points on
// edges dropped; monotone chain, A. M. Andrew, Inf. Proc. Letters 9, 1979).
static void hull_xy(const std::vector<V3>& p, std::vector<int>& idx, std::vector<int>& out) {
  std::sort(idx.begin(), idx.end(), [&](int a, int b) {
    return p[a].x < p[b].x || (p[a].x == p[b].x && p[a].y < p[b].y);
  });
  out.assign(2 * idx.size(), -1);
  auto turn = [&](int o, int a, int b) {
    return (p[a].x - p[o].x) * (p[b].y - p[o].y) - (p[a].y - p[o].y) * (p[b].x - p[o].x);
  };
  int k = 0;
  for (size_t t = 0; t < idx.size(); ++t) {
    while (k >= 2 && turn(out[k - 2], out[k - 1], idx[t]) <= 0) --k;
    out[k++] = idx[t];
  }
  for (int t = (int)idx.size() - 2, lo = k + 1; t >= 0; --t) {
    while (k >= lo && turn(out[k - 2], out[k - 1], idx[t]) <= 0) --k;
    out[k++] = idx[t];
  }
  out.resize(k > 1 ? k - 1 : k);
}

struct Scratch2 {
  std::vector<V3> p;
  std::vector<uint8_t> eligible, vertex, done_group;
  std::vector<int> group, poly;
  std::vector<int> tri;   // accepted faces, 3 positions each
};

static int region_2d(const Problem& P, int64_t i, int64_t j, Scratch2& S) {
  const int n = P.nsub;
  const int64_t* reg = P.regions + j * n;
  S.p.resize(n);
  bool constant = true;
  for (int k = 0; k < n; ++k) {
    const int64_t l = reg[k];
    S.p[k] = {P.points[2 * l], P.points[2 * l + 1], P.vals[i * P.npoints + l]};
    constant &= S.p[k].z == S.p[0].z;
  }
  uint8_t* brow = P.base + i * P.npoints;
  int32_t* f = P.faces + ((i * P.nregions + j) * P.max_faces) * 3;
  int32_t* nf = P.nfaces + i * P.nregions + j;
  if (constant) {
    for (int k = 0; k < 3; ++k) brow[reg[k]] = 1;
    f[0] = 0, f[1] = 1, f[2] = 2;
    *nf = 1;
    return OPYX_OK;
  }
  // base eligibility: corners, and points below the corners' plane
  const V3 nc = lower_normal(S.p[0], S.p[1], S.p[2]);
  const double cc = dot(S.p[0], nc) + kTol;
  S.eligible.assign(n, 0);
  S.vertex.assign(n, 0);
  for (int k = 0; k < n; ++k) S.eligible[k] = k < 3 || dot(S.p[k], nc) > cc;
  // lower hull: planes through three points with no point below them; a
  // plane holding more than three points is triangulated once, as a fan over
  // the xy hull of its points, when its first three points (in position
  // order, not collinear in xy) come up
  S.tri.clear();
  for (int a = 0; a < n; ++a)
    for (int b = a + 1; b < n; ++b)
      for (int c = b + 1; c < n; ++c) {
        V3 m = cross(sub(S.p[b], S.p[a]), sub(S.p[c], S.p[a]));
        const double ml = std::sqrt(dot(m, m));
        if (!(ml > 0) || !(std::fabs(m.z) > kTol * ml)) continue;   // vertical or degenerate
        if (m.z > 0) m = {-m.x, -m.y, -m.z};
        m = {m.x / ml, m.y / ml, m.z / ml};
        bool support = true;
        int ncop = 0;
        for (int q = 0; q < n && support; ++q) {
          const double h = dot(sub(S.p[q], S.p[a]), m);   // > 0: below the plane
          if (h > kTol) support = false;
          else if (h >= -kTol) ++ncop;
        }
        if (!support) continue;
        if (ncop == 3) {
          S.tri.insert(S.tri.end(), {a, b, c});
          continue;
        }
        S.group.clear();
        for (int q = 0; q < n; ++q)
          if (std::fabs(dot(sub(S.p[q], S.p[a]), m)) <= kTol) S.group.push_back(q);
        // the group's first three members not collinear in xy
        int g0 = S.group[0], g1 = S.group[1], g2 = -1;
        for (size_t t = 2; t < S.group.size() && g2 < 0; ++t) {
          const int q = S.group[t];
          const double ar = (S.p[g1].x - S.p[g0].x) * (S.p[q].y - S.p[g0].y) -
                            (S.p[g1].y - S.p[g0].y) * (S.p[q].x - S.p[g0].x);
          if (std::fabs(ar) > kTol * kTol) g2 = q;
        }
        if (g0 != a || g1 != b || g2 != c) continue;
        hull_xy(S.p, S.group, S.poly);
        for (size_t t = 1; t + 1 < S.poly.size(); ++t) {
          int v[3] = {S.poly[0], S.poly[t], S.poly[t + 1]};
          std::sort(v, v + 3);
          S.tri.insert(S.tri.end(), {v[0], v[1], v[2]});
        }
      }
  // faces on base points only, without the corner triangle
  int cnt = 0;
  for (size_t t = 0; t < S.tri.size(); t += 3) {
    const int a = S.tri[t], b = S.tri[t + 1], c = S.tri[t + 2];
    for (int v : {a, b, c})
      if (S.eligible[v]) S.vertex[v] = 1;
    if (!(S.eligible[a] && S.eligible[b] && S.eligible[c])) continue;
    if (a == 0 && b == 1 && c == 2) continue;
    if (!(lower_normal(S.p[a], S.p[b], S.p[c]).z < -kTol)) continue;
    if (cnt >= P.max_faces) return OPYX_ERR_WORKSPACE;
    f[3 * cnt] = a, f[3 * cnt + 1] = b, f[3 * cnt + 2] = c;
    ++cnt;
  }
  if (cnt == 0) {
    f[0] = 0, f[1] = 1, f[2] = 2;
    cnt = 1;
  }
  *nf = cnt;
  for (int k = 0; k < n; ++k) brow[reg[k]] = k < 3 ? 1 : S.vertex[k];
  return OPYX_OK;
}

// ---------------------------------------------------------------- 3-D
// Graph points live in R^4 (x, y, z, f).  The lower hull's facets are
// tetrahedra; a hyperplane holding more than four points is split once into
// tetrahedra: a star from the first vertex of the points' xyz hull over the
// triangles of that hull's boundary (whose planar faces are fans over their
// 2-D hulls).
struct V4 {
  double v[4];
};

inline V4 sub4(const V4& a, const V4& b) {
  return {{a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2], a.v[3] - b.v[3]}};
}
inline double dot4(const V4& a, const V4& b) {
  return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2] + a.v[3] * b.v[3];
}
inline double det3(double a11, double a12, double a13, double a21, double a22, double a23,
                   double a31, double a32, double a33) {
  return a11 * (a22 * a33 - a23 * a32) - a12 * (a21 * a33 - a23 * a31) +
         a13 * (a21 * a32 - a22 * a31);
}
// A vector orthogonal to a, b and c (cofactors of the 3 x 4 matrix).
inline V4 cross4(const V4& a, const V4& b, const V4& c) {
  V4 n;
  for (int i = 0; i < 4; ++i) {
    int k[3], t = 0;
    for (int q = 0; q < 4; ++q)
      if (q != i) k[t++] = q;
    const double d = det3(a.v[k[0]], a.v[k[1]], a.v[k[2]], b.v[k[0]], b.v[k[1]], b.v[k[2]],
                          c.v[k[0]], c.v[k[1]], c.v[k[2]]);
    n.v[i] = (i & 1) ? -d : d;
  }
  return n;
}
// Downward unit normal of the hyperplane through a, b, c, d (left unscaled
// below the tolerance, as lower_normal).
inline V4 lower_normal4(const V4& a, const V4& b, const V4& c, const V4& d) {
  V4 n = cross4(sub4(b, a), sub4(c, a), sub4(d, a));
  if (n.v[3] > 0)
    for (double& t : n.v) t = -t;
  const double l2 = dot4(n, n);
  if (l2 >= kTol) {
    const double s = 1.0 / std::sqrt(l2);
    for (double& t : n.v) t *= s;
  }
  return n;
}

struct Scratch3 {
  std::vector<V4> p;
  std::vector<uint8_t> eligible, vertex;
  std::vector<int> group, face, poly, tri, tet;
  std::vector<V3> q3;       // xyz of the group's points (indexed like p)
  std::vector<int> tmp;
};

// Boundary triangles of the convex hull of the xyz points `idx` (indices into
// q), planar faces as fans over their 2-D hulls; appended to `tri`.
static void hull3_boundary(const std::vector<V3>& q, const std::vector<int>& idx, Scratch3& S) {
  const int m = (int)idx.size();
  for (int ia = 0; ia < m; ++ia)
    for (int ib = ia + 1; ib < m; ++ib)
      for (int ic = ib + 1; ic < m; ++ic) {
        const int a = idx[ia], b = idx[ib], c = idx[ic];
        V3 nrm = cross(sub(q[b], q[a]), sub(q[c], q[a]));
        const double nl = std::sqrt(dot(nrm, nrm));
        if (!(nl > kTol)) continue;   // collinear
        nrm = {nrm.x / nl, nrm.y / nl, nrm.z / nl};
        double lo = 0, hi = 0;
        int nface = 0;
        for (int t = 0; t < m; ++t) {
          const double h = dot(sub(q[idx[t]], q[a]), nrm);
          lo = std::min(lo, h);
          hi = std::max(hi, h);
          if (std::fabs(h) <= kTol) ++nface;
        }
        if (lo < -kTol && hi > kTol) continue;   // points on both sides
        if (nface == 3) {
          S.tri.insert(S.tri.end(), {a, b, c});
          continue;
        }
        S.face.clear();
        for (int t = 0; t < m; ++t)
          if (std::fabs(dot(sub(q[idx[t]], q[a]), nrm)) <= kTol) S.face.push_back(idx[t]);
        // once per planar face: its first three members not collinear
        int f2 = -1;
        const int f0 = S.face[0], f1 = S.face[1];
        for (size_t t = 2; t < S.face.size() && f2 < 0; ++t) {
          const V3 cr = cross(sub(q[f1], q[f0]), sub(q[S.face[t]], q[f0]));
          if (std::sqrt(dot(cr, cr)) > kTol) f2 = S.face[t];
        }
        if (f0 != a || f1 != b || f2 != c) continue;
        // 2-D hull in the face's plane, then a fan
        const V3 e = sub(q[b], q[a]);
        const double el = std::sqrt(dot(e, e));
        const V3 u = {e.x / el, e.y / el, e.z / el};
        const V3 w = cross(nrm, u);
        std::vector<V3> pl(q.size());
        for (int t : S.face) {
          const V3 d = sub(q[t], q[a]);
          pl[t] = {dot(d, u), dot(d, w), 0.0};
        }
        S.tmp = S.face;
        hull_xy(pl, S.tmp, S.poly);
        for (size_t t = 1; t + 1 < S.poly.size(); ++t)
          S.tri.insert(S.tri.end(), {S.poly[0], S.poly[t], S.poly[t + 1]});
      }
}

static int region_3d(const Problem& P, int64_t i, int64_t j, Scratch3& S) {
  const int n = P.nsub;
  const int64_t* reg = P.regions + j * n;
  S.p.resize(n);
  S.q3.resize(n);
  bool constant = true;
  for (int k = 0; k < n; ++k) {
    const int64_t l = reg[k];
    S.p[k] = {{P.points[3 * l], P.points[3 * l + 1], P.points[3 * l + 2], P.vals[i * P.npoints + l]}};
    S.q3[k] = {S.p[k].v[0], S.p[k].v[1], S.p[k].v[2]};
    constant &= S.p[k].v[3] == S.p[0].v[3];
  }
  uint8_t* brow = P.base + i * P.npoints;
  int32_t* f = P.faces + ((i * P.nregions + j) * P.max_faces) * 4;
  int32_t* nf = P.nfaces + i * P.nregions + j;
  if (constant) {
    for (int k = 0; k < 4; ++k) brow[reg[k]] = 1;
    for (int k = 0; k < 4; ++k) f[k] = k;
    *nf = 1;
    return OPYX_OK;
  }
  const V4 nc = lower_normal4(S.p[0], S.p[1], S.p[2], S.p[3]);
  const double cc = dot4(S.p[0], nc) + kTol;
  S.eligible.assign(n, 0);
  S.vertex.assign(n, 0);
  for (int k = 0; k < n; ++k) S.eligible[k] = k < 4 || dot4(S.p[k], nc) > cc;
  S.tet.clear();
  for (int a = 0; a < n; ++a)
    for (int b = a + 1; b < n; ++b)
      for (int c = b + 1; c < n; ++c)
        for (int d = c + 1; d < n; ++d) {
          V4 m = cross4(sub4(S.p[b], S.p[a]), sub4(S.p[c], S.p[a]), sub4(S.p[d], S.p[a]));
          const double ml = std::sqrt(dot4(m, m));
          if (!(ml > 0) || !(std::fabs(m.v[3]) > kTol * ml)) continue;   // vertical or degenerate
          const double s = (m.v[3] > 0 ? -1.0 : 1.0) / ml;
          for (double& t : m.v) t *= s;
          bool support = true;
          int ncop = 0;
          for (int q = 0; q < n && support; ++q) {
            const double h = dot4(sub4(S.p[q], S.p[a]), m);
            if (h > kTol) support = false;
            else if (h >= -kTol) ++ncop;
          }
          if (!support) continue;
          if (ncop == 4) {
            S.tet.insert(S.tet.end(), {a, b, c, d});
            continue;
          }
          S.group.clear();
          for (int q = 0; q < n; ++q)
            if (std::fabs(dot4(sub4(S.p[q], S.p[a]), m)) <= kTol) S.group.push_back(q);
          // once per hyperplane: its first four members affinely independent in xyz
          const int g0 = S.group[0];
          int g1 = -1, g2 = -1, g3 = -1;
          for (size_t t = 1; t < S.group.size() && g3 < 0; ++t) {
            const int q = S.group[t];
            const V3 e1 = sub(S.q3[q], S.q3[g0]);
            if (g1 < 0) {
              if (std::sqrt(dot(e1, e1)) > kTol) g1 = q;
            } else if (g2 < 0) {
              const V3 cr = cross(sub(S.q3[g1], S.q3[g0]), e1);
              if (std::sqrt(dot(cr, cr)) > kTol) g2 = q;
            } else {
              const V3 cr = cross(sub(S.q3[g1], S.q3[g0]), sub(S.q3[g2], S.q3[g0]));
              if (std::fabs(dot(cr, e1)) > kTol) g3 = q;
            }
          }
          if (g0 != a || g1 != b || g2 != c || g3 != d) continue;
          S.tri.clear();
          hull3_boundary(S.q3, S.group, S);
          int apex = n;
          for (int t : S.tri) apex = std::min(apex, t);
          for (size_t t = 0; t < S.tri.size(); t += 3) {
            if (S.tri[t] == apex || S.tri[t + 1] == apex || S.tri[t + 2] == apex) continue;
            int v[4] = {apex, S.tri[t], S.tri[t + 1], S.tri[t + 2]};
            std::sort(v, v + 4);
            S.tet.insert(S.tet.end(), {v[0], v[1], v[2], v[3]});
          }
        }
  int cnt = 0;
  for (size_t t = 0; t < S.tet.size(); t += 4) {
    const int* v = &S.tet[t];
    bool ok = true;
    for (int k = 0; k < 4; ++k) {
      if (S.eligible[v[k]]) S.vertex[v[k]] = 1;
      ok &= S.eligible[v[k]] != 0;
    }
    if (!ok) continue;
    if (v[0] == 0 && v[1] == 1 && v[2] == 2 && v[3] == 3) continue;
    if (!(lower_normal4(S.p[v[0]], S.p[v[1]], S.p[v[2]], S.p[v[3]]).v[3] < -kTol)) continue;
    if (cnt >= P.max_faces) return OPYX_ERR_WORKSPACE;
    for (int k = 0; k < 4; ++k) f[4 * cnt + k] = v[k];
    ++cnt;
  }
  if (cnt == 0) {
    for (int k = 0; k < 4; ++k) f[k] = k;
    cnt = 1;
  }
  *nf = cnt;
  for (int k = 0; k < n; ++k) brow[reg[k]] = k < 4 ? 1 : S.vertex[k];
  return OPYX_OK;
}

// functions [i0, i1), every region; returns the first failure
static int run_range(const Problem& P, int64_t i0, int64_t i1) {
  const int n = P.nsub;
  if (P.ndim == 1) {
    std::vector<double> x(n), z(n);
    std::vector<uint8_t> keep(n);
    for (int64_t i = i0; i < i1; ++i)
      for (int64_t j = 0; j < P.nregions; ++j) region_1d(P, i, j, x.data(), z.data(), keep.data());
    return OPYX_OK;
  }
  if (P.ndim == 2) {
    Scratch2 S;
    for (int64_t i = i0; i < i1; ++i)
      for (int64_t j = 0; j < P.nregions; ++j) {
        const int st = region_2d(P, i, j, S);
        if (st) return st;
      }
    return OPYX_OK;
  }
  Scratch3 S;
  for (int64_t i = i0; i < i1; ++i)
    for (int64_t j = 0; j < P.nregions; ++j) {
      const int st = region_3d(P, i, j, S);
      if (st) return st;
    }
  return OPYX_OK;
}

}  // namespace cvx
}  // namespace opyx

using namespace opyx::cvx;

extern "C" {

int opyx_convexify_max_faces(int ndim, int nsub) {
  if (ndim < 1 || ndim > 3 || nsub < ndim + 1) return 0;
  if (nsub == ndim + 1) return 1;
  if (ndim == 1) return nsub - 1;
  if (ndim == 2) return 2 * nsub;
  // a triangulation of n points in space has fewer than n (n - 3) / 2 + 1 tetrahedra
  return nsub * (nsub - 3) / 2 + 1;
}

int opyx_convexify(int ndim, int64_t npoints, const double* points, int64_t nfuns,
                   const double* vals, int64_t nregions, int nsub, const int64_t* regions,
                   uint8_t* base, int32_t* faces, int32_t* nfaces, int max_faces, int nthreads) {
  if (ndim < 1 || ndim > 3 || npoints < 1 || nfuns < 0 || nregions < 0 || nsub < ndim + 1)
    return OPYX_ERR_ARG;
  if (!points || !vals || !regions || !base || !faces || !nfaces) return OPYX_ERR_ARG;
  if (max_faces < opyx_convexify_max_faces(ndim, nsub)) return OPYX_ERR_WORKSPACE;
  for (int64_t t = 0; t < nregions * nsub; ++t)
    if (regions[t] < 0 || regions[t] >= npoints) return OPYX_ERR_ARG;
  std::fill(base, base + nfuns * npoints, (uint8_t)0);
  const int D1 = ndim + 1;
  if (nsub == D1) {   // every region a bare simplex (__init__.pyx:29-32)
    std::fill(base, base + nfuns * npoints, (uint8_t)1);
    for (int64_t t = 0; t < nfuns * nregions; ++t) {
      nfaces[t] = 1;
      for (int k = 0; k < D1; ++k) faces[t * max_faces * D1 + k] = k;
    }
    return OPYX_OK;
  }
  Problem P;
  P.ndim = ndim;
  P.npoints = npoints;
  P.nfuns = nfuns;
  P.nregions = nregions;
  P.nsub = nsub;
  P.max_faces = max_faces;
  P.points = points;
  P.vals = vals;
  P.regions = regions;
  P.base = base;
  P.faces = faces;
  P.nfaces = nfaces;
  std::fill(faces, faces + nfuns * nregions * max_faces * D1, -1);
  if (ndim == 1) {
    P.order.resize(nregions * nsub);
    for (int64_t j = 0; j < nregions; ++j) {
      int* o = P.order.data() + j * nsub;
      for (int k = 0; k < nsub; ++k) o[k] = k;
      const int64_t* reg = regions + j * nsub;
      std::stable_sort(o, o + nsub, [&](int a, int b) { return points[reg[a]] < points[reg[b]]; });
    }
  }
  int64_t nt = nthreads > 0 ? nthreads : (int64_t)std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  const int64_t per = 64;   // functions per thread at least
  if (nt > (nfuns + per - 1) / per) nt = (nfuns + per - 1) / per;
  if (nt <= 1) return run_range(P, 0, nfuns);
  std::vector<int> status(nt, OPYX_OK);
  std::vector<std::thread> pool;
  for (int64_t t = 0; t < nt; ++t) {
    const int64_t i0 = nfuns * t / nt, i1 = nfuns * (t + 1) / nt;
    pool.emplace_back([&, t, i0, i1] { status[t] = run_range(P, i0, i1); });
  }
  for (auto& th : pool) th.join();
  for (int s : status)
    if (s) return s;
  return OPYX_OK;
}

}  // extern "C"
