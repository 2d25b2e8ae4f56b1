"""Piecewise convexification of sampled functions: the base points and
faces that `EpigraphInd` / `EpigraphSupp` take as ``I`` and ``If``
(opymize/quickhull/__init__.pyx:8-140).

The hulls are computed by libopyx's host code (`opyx_convexify`, every host
thread): this is set-up work on the host in the reference too (Cython over
C++), not part of the GPU iteration.  Points of 1, 2 or 3 dimensions, as in
the reference.
"""

import ctypes as C

import numpy as np

from opymize_gb300 import _lib


def convexify_arrays(points, vals, regions, nthreads=0):
    """Array form of `piecewise_convexify`: base (nfuns, npoints) bool,
    faces (nfuns, nregions, max_faces, ndim+1) int32 positions in the rows
    of `regions` (-1 past the count) and nfaces (nfuns, nregions)."""
    points = np.ascontiguousarray(points, dtype=np.float64)
    if points.ndim == 1:
        points = points[:, None]
    vals = np.ascontiguousarray(np.atleast_2d(vals), dtype=np.float64)
    regions = np.ascontiguousarray(np.atleast_2d(regions), dtype=np.int64)
    npoints, ndim = points.shape
    nfuns = vals.shape[0]
    nregions, nsub = regions.shape
    if vals.shape[1] != npoints:
        raise ValueError("vals must be (nfuns, npoints)")
    lib = _lib.load()
    mf = lib.opyx_convexify_max_faces(ndim, nsub)
    if mf < 1:
        raise ValueError("regions need at least ndim+1 points, ndim 1, 2 or 3")
    base = np.empty((nfuns, npoints), dtype=np.uint8)
    faces = np.empty((nfuns, nregions, mf, ndim + 1), dtype=np.int32)
    nfaces = np.empty((nfuns, nregions), dtype=np.int32)
    _lib.call("opyx_convexify", ndim, npoints, points.ctypes.data, nfuns, vals.ctypes.data,
              nregions, nsub, regions.ctypes.data, base.ctypes.data, faces.ctypes.data,
              nfaces.ctypes.data, mf, int(nthreads))
    return base.astype(bool), faces, nfaces


def piecewise_convexify(points, vals, regions):
    """Convexify piecewise affine functions on given subsimplices
    (opymize/quickhull/__init__.pyx:8-40).

    points (npoints, ndim), vals (nfuns, npoints), regions (nregions,
    nsubpoints) indices of the points in each simplex, its ndim+1 vertices
    first.  Returns base (nfuns, npoints) bool -- the points spanning the
    piecewise convex hull -- and faces: nfuns lists of nregions arrays
    (nfaces, ndim+1) of positions in regions[j].
    """
    points = np.asarray(points, dtype=np.float64)
    if points.ndim == 1:
        points = points[:, None]
    ndim = points.shape[1]
    vals = np.atleast_2d(vals)
    regions = np.atleast_2d(regions)
    nfuns, nregions, nsub = vals.shape[0], regions.shape[0], regions.shape[1]
    if nsub == ndim + 1:
        base = np.ones((nfuns, points.shape[0]), dtype=bool)
        return base, [[np.arange(ndim + 1, dtype=np.int64)[None]] * nregions
                      for _ in range(nfuns)]
    base, faces, nfaces = convexify_arrays(points, vals, regions)
    out = [[faces[i, j, :nfaces[i, j]].astype(np.int64) for j in range(nregions)]
           for i in range(nfuns)]
    return base, out
