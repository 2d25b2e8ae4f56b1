"""Generate tests/golden/epigraph.npz from the reference itself.

    python oracle/build_ref.py              # host build of proj.cu's QP
    python tests/golden/make_epigraph_golden.py

Projections come from the reference's own `epigraphproj` / `solve_qp`
(opymize/operators/proj.cu:222-831) compiled for the host by
oracle/build_ref.py (the reference's CPU path needs cvxpy + MOSEK, absent
here).  Functional values come from the reference's EpigraphInd /
EpigraphSupp (opymize/functionals/epigraph.py) imported with an identity
``numba.jit`` and a ``cvxpy`` stand-in that only lets EpigraphProj's
constructor run (its CPU projection is never called).  Geometry of the
known-answer cases follows tests/epigraph.py:11-59 (points on, inside and
outside the boundary) and the 1-D support test of tests/epigraph.py:61-104.
"""

import ctypes as C
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("OPYMIZE_REF", "/root/reference")

_numba = types.ModuleType("numba")
_numba.jit = lambda *a, **k: (a[0] if a and callable(a[0]) else (lambda f: f))
sys.modules.setdefault("numba", _numba)


class _CvxStub(types.ModuleType):
    """Enough of cvxpy for EpigraphProj.__init__ (proj.py:424-430)."""

    class _Expr(object):
        def __init__(self, *a, **k):
            pass

        def __sub__(self, o):
            return self

        __rmul__ = __mul__ = __le__ = __sub__

    Parameter = Variable = Constant = Minimize = Problem = _Expr

    @staticmethod
    def sum_squares(e):
        return e


sys.modules.setdefault("cvxpy", _CvxStub("cvxpy"))
sys.path.insert(0, REF)
sys.path.insert(0, REPO)

from opymize.functionals.epigraph import EpigraphInd, EpigraphSupp   # noqa: E402
from opymize.operators.proj import epigraph_Ab                        # noqa: E402
from oracle import build_ref                                          # noqa: E402


def ref_lib(nd):
    path = build_ref.lib_path(nd)
    if not os.path.exists(path):
        build_ref.build()
    lib = C.CDLL(path)
    lib.ref_epigraph_proj.argtypes = [C.c_void_p] * 5 + [C.c_int] * 4
    return lib


def ref_proj(I, J, v, b, x):
    nd = v.shape[1]
    y = np.ascontiguousarray(x, dtype=np.float64).copy()
    Ib = np.ascontiguousarray(I, dtype=np.uint8)
    Jb = np.ascontiguousarray(J, dtype=np.int64)
    vb = np.ascontiguousarray(v, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    ref_lib(nd).ref_epigraph_proj(y.ctypes.data, Ib.ctypes.data, Jb.ctypes.data,
                                  vb.ctypes.data, bb.ctypes.data, I.shape[0], J.shape[0],
                                  I.shape[1], J.shape[1])
    return y


def ref_ind(I, J, v, b):
    """The reference's EpigraphInd.  Its conjugate is passed in holding only
    the constraint system (epigraph_Ab, proj.py:376-386): the value and the
    projection need nothing else, and EpigraphSupp's face equations
    (epigraph.py:86-97) call np.linalg.solve with a (nfaces, ndim) right-hand
    side, which numpy 2 reads as a matrix."""
    conj = types.SimpleNamespace()
    conj.A, conj.b = epigraph_Ab(I, J, v, b)
    return EpigraphInd(I, None, J, v, b, conj=conj)


def ref_supp(I, If, J, v, b, with_conj=False):
    """The reference's EpigraphSupp (with its conjugate EpigraphInd when
    `with_conj`).  Its face equations (epigraph.py:86-97) pass a stack of
    right-hand-side vectors to np.linalg.solve, which numpy >= 2 reads as a
    matrix; the numpy 1 meaning is restored for the constructor only."""
    orig = np.linalg.solve

    def solve_stacked_vectors(a, rhs):
        a, rhs = np.asarray(a), np.asarray(rhs)
        if rhs.ndim == a.ndim - 1:
            return orig(a, rhs[..., None])[..., 0]
        return orig(a, rhs)

    np.linalg.solve = solve_stacked_vectors
    try:
        if with_conj:
            return EpigraphSupp(I, If, J, v, b)
        return EpigraphSupp(I, If, J, v, b, conj=types.SimpleNamespace())
    finally:
        np.linalg.solve = orig


def random_case(rng, nd, nfuns, nregions, npoints, nsub, density=0.8, scale=5.0):
    J = np.stack([rng.choice(npoints, nsub, replace=False) for _ in range(nregions)])
    I = rng.random((nfuns, npoints)) < density
    v = rng.uniform(-2, 2, (npoints, nd))
    b = rng.uniform(-2, 2, (nfuns, npoints))
    x = rng.uniform(-scale, scale, (nregions, nfuns, nd + 1))
    return I, J.astype(np.int64), v, b, x


def known_case(rng, nd):
    """tests/epigraph.py:11-59: x_in on the boundary; x inside (maps to
    itself) and x outside along the active normal (maps back to x_in)."""
    npoints, nfuns = 3, 2
    I = np.array([[True, False, False], [False, True, True]])
    J = np.arange(npoints, dtype=np.int64)[None, :]
    v = -2.0 + 4 * rng.random((npoints, nd))
    b = -2.0 + 4 * rng.random((nfuns, npoints))
    x_in = np.zeros((1, nfuns, nd + 1))
    x_in[0, 0] = -5.0 + 10 * rng.random(nd + 1)
    x_in[0, 0, -1] = -b[0, 0] + v[0].dot(x_in[0, 0, :-1])
    x_in[0, 1] = -5.0 + 10 * rng.random(nd + 1)
    vals = [-bk + vk.dot(x_in[0, 1, :-1]) for bk, vk in zip(b[1, 1:], v[1:])]
    ak = int(np.argmax(vals))
    x_in[0, 1, -1] = vals[ak]
    inside = x_in.copy()
    inside[0, :, -1] += 4 * rng.random(nfuns)
    outside = x_in.copy()
    sh = rng.random(2)
    outside[0, 0, :-1] += sh[0] * v[0]
    outside[0, 0, -1] -= sh[0]
    outside[0, 1, :-1] += sh[1] * v[1 + ak]
    outside[0, 1, -1] -= sh[1]
    return I, J, v, b, x_in, inside, outside


def support_case(rng, nsub, nfuns=5, nregions=2):
    """tests/epigraph.py:61-104 (1-D quadratics sampled on nsub points per
    region, faces between neighbours, x chosen inside every region)."""
    nd = 1
    npoints = nregions * nsub
    fct = lambda x, a_, b_, c_: a_ * (x - b_) ** 2 + c_
    x0 = 5 * (-1 + 2 * rng.random(nregions))
    x1 = x0 + 0.1 + 2 * rng.random(nregions)
    a_arr = 0.1 + 4 * rng.random(nfuns)
    b_arr = x0[0] + (-1.5 + 4 * rng.random(nfuns)) * (x1[0] - x0[0])
    c_arr = 5 * (-1 + 2 * rng.random(nfuns))
    I = np.ones((nfuns, npoints), dtype=bool)
    J = np.arange(npoints, dtype=np.int64).reshape(nregions, nsub)
    v = np.zeros((nregions, nsub, nd))
    for j in range(nregions):
        v[j, :] = np.linspace(x0[j], x1[j], nsub)[:, None]
        tmp = J[j, -1]
        J[j, 2:] = J[j, 1:-1].copy()
        J[j, 1] = tmp
    v = v.reshape(npoints, nd)
    b = np.zeros((nfuns, npoints))
    for i in range(nfuns):
        b[i, :] = fct(v, a_arr[i], b_arr[i], c_arr[i]).ravel()
    faces = np.array([(0, 2), (nsub - 1, 1)] + [(k, k + 1) for k in range(2, nsub - 1)])
    x = np.zeros((nregions, nfuns, nd + 1))
    for j in range(nregions):
        x[j, :, -1] = -rng.random()
        x[j, :, 0] = -x[j, :, -1] * (x0[j] + rng.random(nfuns) * (x1[j] - x0[j]))
    exact = 0.0
    for i in range(nfuns):
        for j in range(nregions):
            xx, xt = x[j, i, :-1], x[j, i, -1]
            exact += -xt * fct(-xx / xt, a_arr[i], b_arr[i], c_arr[i])[0]
    return I, J, v, b, x, faces, exact


def main():
    rng = np.random.default_rng(20240611)
    out = {}
    # random projections (ndim 1..3), EpigraphInd values before and after
    specs = [(1, 7, 4, 9, 5), (2, 9, 3, 12, 7), (3, 6, 3, 12, 8), (2, 40, 2, 6, 6),
             (3, 25, 2, 8, 8), (1, 64, 5, 16, 4)]
    for c, (nd, nfuns, nregions, npoints, nsub) in enumerate(specs):
        I, J, v, b, x = random_case(rng, nd, nfuns, nregions, npoints, nsub)
        y = ref_proj(I, J, v, b, x)
        ind = ref_ind(I, J, v, b)
        out.update({"rand%d_%s" % (c, k): a for k, a in
                    dict(I=I, J=J, v=v, b=b, x=x, y=y, ind_x=np.array(ind(x.ravel())),
                         ind_y=np.array(ind(y.ravel()))).items()})
    out["nrand"] = np.array(len(specs))
    # known answers
    for c, nd in enumerate([2, 3, 2, 3, 1]):
        I, J, v, b, x_in, inside, outside = known_case(rng, nd)
        out.update({"known%d_%s" % (c, k): a for k, a in
                    dict(I=I, J=J, v=v, b=b, x_in=x_in, inside=inside, outside=outside,
                         y_inside=ref_proj(I, J, v, b, inside),
                         y_outside=ref_proj(I, J, v, b, outside)).items()})
    out["nknown"] = np.array(5)
    # EpigraphSupp values (1-D quadratic support test)
    for c, nsub in enumerate([5, 50, 500]):
        I, J, v, b, x, faces, exact = support_case(rng, nsub)
        If = [[faces.copy() for _ in range(J.shape[0])] for _ in range(I.shape[0])]
        sig = ref_supp(I, If, J, v, b)
        out.update({"supp%d_%s" % (c, k): a for k, a in
                    dict(I=I, J=J, v=v, b=b, x=x, faces=faces, exact=np.array(exact),
                         val=np.array(sig(x.ravel()))).items()})
    out["nsupp"] = np.array(3)
    path = os.path.join(HERE, "epigraph.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, len(out), "arrays")


if __name__ == "__main__":
    main()
