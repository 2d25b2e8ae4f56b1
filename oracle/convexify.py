"""CPU oracle of the reference's piecewise convexification -- TEST
INFRASTRUCTURE ONLY, like the rest of ``oracle/``.

Restates opymize/quickhull/__init__.pyx:8-140 with its hull code
(opymize/quickhull/convexhull.cpp):

* 1-D (`piecewise_convexify_1d`, __init__.pyx:42-83; getConvexHull1D,
  convexhull.cpp:192-216): per region the points sorted by abscissa, per
  function a gift wrap from the leftmost point that steps to the point of
  smallest slope (slopes rounded to a 1e-9 grid, ties to the farthest point).
* 2-D and 3-D (`piecewise_convexify_nd`, __init__.pyx:85-140;
  getConvexHullND, convexhull.cpp:118-183): the convex hull of the region's
  graph points plus an apex above their centroid -- computed here with
  scipy's Qhull (option Qt, triangulated facets), which the reference calls
  for 3-D points and where it calls QuickHull for 2-D -- and the
  reference's face filter: a face counts when its sorted vertices are not the
  corner simplex, every vertex is a corner or lies more than 1e-9 below the
  corners' hyperplane (tested lazily, in face order, as is_base_face does)
  and its unit lower normal points down by more than 1e-9.

Pinned to the known answers of the reference's tests/convexhull.py (restated
in tests/test_convexify.py).  The 2-D and 3-D face sets depend on the hull
library's triangulation of coplanar facets; on points in general position
they are unique.
"""

import numpy as np

TOL = 1e-9


def hull_1d(x, z):
    n = len(x)
    base = np.ones(n, dtype=bool)
    i = 0
    while i < n - 1:
        best, best_m = np.inf, i + 1
        for m in range(i + 1, n):
            s = (z[m] - z[i]) / (x[m] - x[i])
            s = TOL * np.round(s / TOL)
            if s <= best:
                best_m, best = m, s
        base[i + 1:best_m] = False
        i = best_m
    return base


def convexify_1d(points, vals, regions):
    nfuns, npoints = vals.shape
    base = np.zeros((nfuns, npoints), dtype=bool)
    faces = [[] for _ in range(nfuns)]
    for reg in regions:
        ordered = np.argsort(points[reg, 0], kind="stable")
        x = points[reg[ordered], 0]
        for i in range(nfuns):
            b = hull_1d(x, vals[i, reg[ordered]])
            base[i, reg[ordered]] = b
            idx = ordered[b]
            faces[i].append(np.array([idx[k:k + 2] for k in range(len(idx) - 1)], dtype=np.int64))
    return base, faces


def _lower_normal(v):
    """Downward normal of the hyperplane through the rows of v (DIM x DIM),
    by cofactors (hodge_3d / hodge_4d, convexhull.cpp:30-60), normalised
    unless its squared length is below TOL."""
    dim = v.shape[1]
    d = v[1:] - v[0]
    n = np.array([(-1) ** k * np.linalg.det(np.delete(d, k, axis=1)) for k in range(dim)])
    if n[-1] > 0:
        n = -n
    nn = np.dot(n, n)
    if nn >= TOL:
        n = n / np.sqrt(nn)
    return n


def convexify_nd(points, vals, regions):
    """2-D and 3-D points: __init__.pyx:85-140 with convexhull.cpp:118-183."""
    from scipy.spatial import ConvexHull
    nfuns, npoints = vals.shape
    ndim = points.shape[1]
    dim = ndim + 1
    nsub = regions.shape[1]
    base = np.zeros((nfuns, npoints), dtype=bool)
    faces = [[] for _ in range(nfuns)]
    for reg in regions:
        g = np.zeros((nsub + 1, dim))
        g[:nsub, :ndim] = points[reg]
        g[nsub, :ndim] = g[:nsub, :ndim].sum(axis=0) / nsub
        for i in range(nfuns):
            g[:nsub, ndim] = vals[i, reg]
            if np.all(g[:nsub, ndim] == g[0, ndim]):
                faces[i].append(np.arange(dim)[None])
                base[i, reg[:dim]] = True
                continue
            g[nsub, ndim] = g[:nsub, ndim].max() + 0.1
            simplices = ConvexHull(g, qhull_options="Qt").simplices
            n_c = _lower_normal(g[:dim])
            c = np.dot(g[0], n_c) + TOL
            b = np.array([1] * dim + [2] * (nsub + 1 - dim))      # 2 = not tested yet
            keep = []
            for f in simplices:
                f = np.sort(f)
                if list(f) == list(range(dim)):
                    continue
                ok = True
                for v in f:
                    if b[v] == 2:
                        b[v] = 1 if np.dot(g[v], n_c) > c else 0
                    if b[v] == 0:
                        ok = False
                        break
                if ok and _lower_normal(g[f])[-1] < -TOL:
                    keep.append(f)
            faces[i].append(np.array(keep, dtype=np.int64).reshape(-1, dim) if keep
                            else np.arange(dim)[None])
            base[i, reg] = b[:nsub] == 1
    return base, faces


def piecewise_convexify(points, vals, regions):
    points = np.asarray(points, dtype=np.float64)
    ndim = points.shape[1]
    nfuns = vals.shape[0]
    nregions, nsub = regions.shape
    if nsub == ndim + 1:
        return (np.ones((nfuns, points.shape[0]), dtype=bool),
                [[np.arange(ndim + 1)[None]] * nregions for _ in range(nfuns)])
    if ndim == 1:
        return convexify_1d(points, vals, regions)
    return convexify_nd(points, vals, regions)
