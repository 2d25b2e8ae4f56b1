"""Piecewise convexification (host code of libopyx, `opyx_convexify`) on the
CPU: the known answers and the invariances of the reference's
tests/convexhull.py, the Qhull-based oracle on random regions, and the faces
that the sublabel model's EpigraphSupp takes."""

import itertools

import numpy as np
import pytest

from oracle import convexify as ocvx
from opymize_gb300.tools.convexify import piecewise_convexify, convexify_arrays
from opymize_gb300.quickhull import piecewise_convexify as piecewise_convexify_ref_path


def barygrid(ndim, nse):
    """Barycentric grid with nse points per edge (boundary included)."""
    grid = []
    for coord in itertools.product(range(nse), repeat=ndim):
        s = sum(coord)
        if s < nse:
            grid.append(coord + (nse - 1 - s,))
    return np.array(grid, dtype=np.float64) / (nse - 1)


def rotation(rng, ndim):
    if ndim == 1:
        return np.ones((1, 1))
    phi = rng.random()
    if ndim == 2:
        return np.array([[np.cos(phi), -np.sin(phi)], [np.sin(phi), np.cos(phi)]])
    u = rng.random(3)
    u /= np.linalg.norm(u)
    K = np.array([[0, -u[2], u[1]], [u[2], 0, -u[0]], [-u[1], u[0], 0]])
    return np.eye(3) + np.sin(phi) * K + (1 - np.cos(phi)) * K @ K      # Rodrigues' formula


def check_invariant(points, vals, regions, result, seed=0):
    """The base mask is `result`, also after shifting, rotating and
    stretching the domain and adding affine functions to the values (the
    reference's test_convexify, tests/convexhull.py:31-57)."""
    rng = np.random.default_rng(seed)
    ndim, nfuns = points.shape[1], vals.shape[0]
    assert np.array_equal(piecewise_convexify(points, vals, regions)[0], result)
    evals = vals.copy()
    for _ in range(100):
        shift = -6 + 12 * rng.random((1, ndim))
        R = (0.2 + 2 * rng.random((1, ndim))) * rotation(rng, ndim)
        epoints = points.dot(R.T) + shift
        evals += points.dot(-5 + 10 * rng.random((ndim, nfuns))).T + (-4 + 8 * rng.random((nfuns, 1)))
        assert np.array_equal(piecewise_convexify(epoints, evals, regions)[0], result)


def test_handcrafted_1d():
    # tests/convexhull.py:66-80: point 3 belongs to no region
    points = np.array([[0.0], [1.0], [0.1], [0.2], [0.4], [0.7]])
    vals = np.array([[0.0, 0.0, 1.0, -0.3, -0.3, 2.0]])
    regions = np.array([[0, 1, 5, 2, 4]])
    result = np.array([[True, True, False, False, True, False]])
    check_invariant(points, vals, regions, result)
    np.testing.assert_array_equal(ocvx.piecewise_convexify(points, vals, regions)[0], result)
    _, faces = piecewise_convexify(points, vals, regions)
    np.testing.assert_array_equal(faces[0][0], [[0, 4], [4, 1]])


def test_handcrafted_2d():
    # tests/convexhull.py:82-101: point 4 belongs to no region
    points = np.array([[0.0, 0.0], [0.0, 1.0], [1.0, 1.0], [0.5, 0.5], [0.0, 0.2], [0.0, 0.5],
                       [0.5, 1.0], [0.3, 0.7]])
    vals = np.array([[0.0, 0.0, 0.0, 1.0, 2.0, 0.3, -0.3, -0.3]])
    regions = np.array([[0, 1, 2, 5, 6, 7, 3]])
    result = np.array([[True, True, True, False, False, False, True, True]])
    check_invariant(points, vals, regions, result)
    np.testing.assert_array_equal(ocvx.piecewise_convexify(points, vals, regions)[0], result)
    _, faces = piecewise_convexify(points, vals, regions)
    assert {tuple(f) for f in faces[0][0]} == {(0, 1, 5), (0, 2, 5), (1, 4, 5), (2, 4, 5)}


@pytest.mark.parametrize("ndim", [1, 2, 3])
@pytest.mark.parametrize("fun", ["zero", "square"])
def test_convex_functions(ndim, fun):
    """tests/convexhull.py:59-64: on a barycentric grid of the simplex a
    strictly convex function keeps every point, the zero function only the
    vertices."""
    bary = barygrid(ndim, 5)
    bary = bary[np.all(bary != 1, axis=1)]
    bary = np.concatenate((np.eye(ndim + 1), bary), axis=0)
    points = np.ascontiguousarray(bary[:, :-1])
    f = (lambda p: 0.0) if fun == "zero" else (lambda p: float((p ** 2).sum()))
    vals = np.array([[f(p) for p in points]])
    regions = np.arange(points.shape[0])[None]
    result = np.ones((1, points.shape[0]), dtype=bool)
    if fun == "zero":
        result[0, ndim + 1:] = False
    check_invariant(points, vals, regions, result)


def _random_regions_2d(rng, nregions, npts):
    """Triangles of a strip with interior points, sharing their corners."""
    corners = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0], [2.0, 0.0], [2.0, 1.0]])
    tris = [(0, 1, 2), (1, 3, 2), (1, 4, 3), (4, 5, 3)][:nregions]
    points, regions = [corners], []
    off = len(corners)
    for t in tris:
        w = rng.dirichlet(np.ones(3), size=npts)
        points.append(w @ corners[list(t)])
        regions.append(list(t) + list(range(off, off + npts)))
        off += npts
    return np.concatenate(points), np.array(regions, dtype=np.int64)


@pytest.mark.parametrize("seed", range(6))
def test_2d_matches_qhull_oracle(seed):
    rng = np.random.default_rng(seed)
    points, regions = _random_regions_2d(rng, 4, int(rng.integers(2, 12)))
    nfuns = 7
    vals = rng.standard_normal((nfuns, points.shape[0]))
    vals[::2] += 3.0 * (points ** 2).sum(axis=1)          # mostly convex functions
    vals[3] = 0.25                                          # constant: the corner triangles
    b1, f1 = ocvx.piecewise_convexify(points, vals, regions)
    b2, f2 = piecewise_convexify(points, vals, regions)
    np.testing.assert_array_equal(b1, b2)
    for i in range(nfuns):
        for j in range(regions.shape[0]):
            assert ({tuple(sorted(f)) for f in f1[i][j]} == {tuple(sorted(f)) for f in f2[i][j]})


@pytest.mark.parametrize("seed", range(4))
def test_3d_matches_qhull_oracle(seed):
    """3-D points: two tetrahedra sharing a face, interior points; the
    oracle is the reference's own procedure with Qhull, which the reference
    itself uses for 3-D points."""
    rng = np.random.default_rng(100 + seed)
    corners = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0],
                        [1.0, 1.0, 1.0]])
    tets = [(0, 1, 2, 3), (1, 2, 3, 4)]
    npts = int(rng.integers(2, 9))
    points, regions, off = [corners], [], len(corners)
    for t in tets:
        points.append(rng.dirichlet(np.ones(4), size=npts) @ corners[list(t)])
        regions.append(list(t) + list(range(off, off + npts)))
        off += npts
    points, regions = np.concatenate(points), np.array(regions, dtype=np.int64)
    vals = rng.standard_normal((5, points.shape[0]))
    vals[::2] += 3.0 * (points ** 2).sum(axis=1)
    vals[3] = -1.5
    b1, f1 = ocvx.piecewise_convexify(points, vals, regions)
    b2, f2 = piecewise_convexify(points, vals, regions)
    np.testing.assert_array_equal(b1, b2)
    for i in range(vals.shape[0]):
        for j in range(2):
            assert ({tuple(sorted(f)) for f in f1[i][j]} == {tuple(sorted(f)) for f in f2[i][j]})


@pytest.mark.parametrize("seed", range(4))
def test_1d_matches_oracle(seed):
    rng = np.random.default_rng(seed)
    L, S = 6, int(rng.integers(3, 9))
    npoints = (L - 1) * (S - 1) + 1
    points = np.sort(rng.uniform(0, 1, npoints))[:, None]
    points[0], points[-1] = 0.0, 1.0
    regions = np.empty((L - 1, S), dtype=np.int64)
    for j in range(L - 1):
        a = j * (S - 1)
        regions[j, :2] = a, a + S - 1                       # the interval's ends first
        regions[j, 2:] = rng.permutation(np.arange(a + 1, a + S - 1))
    vals = rng.standard_normal((9, npoints))
    vals[1] = 2.0 * points[:, 0] - 1.0                      # affine: only the ends
    vals[2] = (points[:, 0] - 0.4) ** 2
    b1, f1 = ocvx.piecewise_convexify(points, vals, regions)
    b2, f2 = piecewise_convexify(points, vals, regions)
    np.testing.assert_array_equal(b1, b2)
    for i in range(vals.shape[0]):
        for j in range(L - 1):
            np.testing.assert_array_equal(f1[i][j], f2[i][j])


def test_threads_agree_and_simplex_regions():
    rng = np.random.default_rng(9)
    points, regions = _random_regions_2d(rng, 3, 6)
    vals = rng.standard_normal((300, points.shape[0]))
    one = convexify_arrays(points, vals, regions, nthreads=1)
    many = convexify_arrays(points, vals, regions, nthreads=0)
    for a, b in zip(one, many):
        np.testing.assert_array_equal(a, b)
    base, faces = piecewise_convexify(points, vals, regions[:, :3])
    assert base.all() and all(np.array_equal(f, [[0, 1, 2]]) for fi in faces for f in fi)
    base, faces = piecewise_convexify(rng.random((4, 3)), rng.random((2, 4)), np.array([[0, 1, 2, 3]]))
    assert base.all() and all(np.array_equal(f, [[0, 1, 2, 3]]) for fi in faces for f in fi)


def test_errors():
    from opymize_gb300 import _lib
    lib = _lib.load()
    pts = np.ascontiguousarray([[0.0], [1.0], [0.5]])
    vals = np.zeros((1, 3))
    reg = np.array([[0, 1, 2]], dtype=np.int64)
    out = (np.zeros(3, np.uint8), np.zeros(8, np.int32), np.zeros(1, np.int32))
    args = lambda r, mf: (1, 3, pts.ctypes.data, 1, vals.ctypes.data, 1, 3, r.ctypes.data,
                          out[0].ctypes.data, out[1].ctypes.data, out[2].ctypes.data, mf, 1)
    assert lib.opyx_convexify(*args(reg, 1)) == _lib.OPYX_ERR_WORKSPACE     # needs nsub-1 = 2
    bad = np.array([[0, 1, 7]], dtype=np.int64)
    assert lib.opyx_convexify(*args(bad, 2)) == _lib.OPYX_ERR_ARG           # index out of range
    assert lib.opyx_convexify(*args(reg, 2)) == _lib.OPYX_OK


def test_sublabel_faces_match_lifting():
    """The sublabel model's intervals: convexify gives exactly the faces of
    the monotone-chain lower hull (tools.lifting.lower_hull_faces) that the
    model's EpigraphSupp takes as ``If``."""
    from opymize_gb300.tools import lifting
    for seed, (L, S) in enumerate(((6, 5), (16, 8), (4, 3))):
        f = np.random.default_rng(seed).uniform(0, 1, 60)
        d = lifting.sublabel_data(f, L=L, samples=S, trunc=0.04)
        base, faces = piecewise_convexify(d["v"], d["b"], d["J"])
        assert base.shape == d["b"].shape
        for i in range(f.size):
            for j in range(L - 1):
                ref = lifting.lower_hull_faces(d, i, j)
                assert faces[i][j].dtype == ref.dtype and np.array_equal(faces[i][j], ref), (i, j)


def test_degenerate_inputs():
    """Collinear corners, repeated points and non-finite values neither fail
    nor leave the documented output ranges."""
    pts = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0], [0.5, 0.0], [1.5, 0.0]])   # on a line
    vals = np.array([[0.0, 1.0, 0.0, -1.0, 2.0], [np.nan, 0.0, 1.0, 0.0, np.inf]])
    base, faces = piecewise_convexify(pts, vals, np.array([[0, 1, 2, 3, 4]]))
    assert base[:, :3].all()
    for fi in faces:
        assert all(f.shape[1] == 3 and f.min() >= 0 and f.max() < 5 for f in fi)
    pts = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [0.2, 0.2], [0.2, 0.2], [0.2, 0.2]])
    vals = np.array([[0.0, 0.0, 0.0, -1.0, -1.0, -1.0], [0.0, 0.0, 0.0, -1.0, -2.0, -1.0]])
    base, faces = piecewise_convexify(pts, vals, np.array([[0, 1, 2, 3, 4, 5]]))
    assert base[:, :3].all() and base[1, 4]
    for fi in faces:
        f = fi[0]
        assert f.shape[1] == 3 and f.min() >= 0 and f.max() < 6
    x = np.array([[0.0], [1.0], [0.5], [0.5]])                                      # repeated abscissa
    base, faces = piecewise_convexify(x, np.array([[0.0, 0.0, -1.0, -2.0]]), np.array([[0, 1, 2, 3]]))
    assert base[0, 0] and base[0, 1] and base[0, 3]


def test_reference_module_path():
    assert piecewise_convexify_ref_path is piecewise_convexify


def test_1d_three_point_intervals():
    """1-D regions of three points take the gift-wrap path, as in the
    reference, whose only shortcut for them is the bare-simplex case
    nsub == ndim + 1 (quickhull/__init__.pyx:30); its nd-path test
    nsubpoints == 3 (:116) is never reached for ndim 1.  Expected masks
    follow getConvexHull1D (quickhull/convexhull.cpp:190-217): from each hull
    point the next one is the smallest rounded slope, ties to the farthest."""
    points = np.array([[0.0], [0.5], [1.0], [1.5], [2.0], [7.0]])   # point 5 in no region
    regions = np.array([[0, 2, 1], [2, 4, 3]], dtype=np.int64)       # endpoints first
    vals = np.array([[0.0, 1.0, 0.0, -1.0, 0.0, 3.0],    # middle above its chord: dropped;
                                                          # below: kept
                     [0.0, 0.5, 1.0, 1.5, 2.0, 3.0]])     # collinear: ties to the farthest
    want = np.array([[1, 0, 1, 1, 1, 0],
                     [1, 0, 1, 0, 1, 0]], dtype=bool)
    for fn in (piecewise_convexify, ocvx.piecewise_convexify):
        base, faces = fn(points, vals, regions)
        np.testing.assert_array_equal(base, want)
    _, faces = piecewise_convexify(points, vals, regions)
    assert sorted(map(tuple, faces[0][0])) == [(0, 1)]            # positions in regions[0]
    assert sorted(map(tuple, faces[0][1])) == [(0, 2), (2, 1)]
    assert sorted(map(tuple, faces[1][1])) == [(0, 1)]
