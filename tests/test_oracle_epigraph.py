"""The epigraph oracle (oracle/epigraph.py) pinned against the reference:
fixtures made by the reference's own QP kernel built for the host and by its
EpigraphInd / EpigraphSupp (tests/golden/make_epigraph_golden.py), the
known answers of the reference's tests/epigraph.py, and KKT certificates."""

import os

import numpy as np
import pytest

from oracle import epigraph as E
from tests.conftest import GOLDEN

FIX = np.load(os.path.join(GOLDEN, "epigraph.npz"))


def case(prefix, c):
    p = "%s%d_" % (prefix, c)
    return {k[len(p):]: FIX[k] for k in FIX.files if k.startswith(p)}


@pytest.mark.parametrize("c", range(int(FIX["nrand"])))
def test_oracle_matches_reference_qp(c):
    d = case("rand", c)
    y, bad = E.epigraph_proj(d["I"], d["J"], d["v"], d["b"], d["x"])
    assert bad == 0
    assert np.abs(y - d["y"]).max() <= 1e-10
    assert E.epigraph_ind(d["I"], d["J"], d["v"], d["b"], d["x"])[1] == \
        pytest.approx(float(d["ind_x"][1]), rel=1e-12, abs=1e-14)
    assert E.epigraph_ind(d["I"], d["J"], d["v"], d["b"], y)[1] <= 1e-12
    assert float(d["ind_y"][1]) <= 1e-12


@pytest.mark.parametrize("c", range(int(FIX["nknown"])))
def test_known_answers(c):
    """tests/epigraph.py:42-56: inside points are fixed, points moved out
    along the active normal come back to the boundary point."""
    d = case("known", c)
    yi, _ = E.epigraph_proj(d["I"], d["J"], d["v"], d["b"], d["inside"])
    yo, _ = E.epigraph_proj(d["I"], d["J"], d["v"], d["b"], d["outside"])
    assert np.linalg.norm(yi - d["inside"]) ** 2 < 1e-10
    assert np.linalg.norm(yo - d["x_in"]) ** 2 < 1e-10
    assert np.linalg.norm(d["y_inside"] - d["inside"]) ** 2 < 1e-10
    assert np.linalg.norm(d["y_outside"] - d["x_in"]) ** 2 < 1e-10


@pytest.mark.parametrize("c", range(int(FIX["nsupp"])))
def test_support_values(c):
    d = case("supp", c)
    If = [[d["faces"] for _ in range(d["J"].shape[0])] for _ in range(d["I"].shape[0])]
    off, eqns, chk = E.supp_pieces(d["I"], If, d["J"], d["v"], d["b"])
    val, inf = E.epigraph_supp(off, eqns, chk, d["x"])
    assert val == pytest.approx(float(d["val"][0]), rel=1e-12)
    assert inf == pytest.approx(float(d["val"][1]), abs=1e-12)


def test_support_approaches_quadratic():
    """tests/epigraph.py:107-110: the sampled support converges to the exact
    perspective as the sampling refines."""
    errs = [abs(float(case("supp", c)["val"][0]) - float(case("supp", c)["exact"]))
            / abs(float(case("supp", c)["exact"])) for c in range(int(FIX["nsupp"]))]
    assert errs[-1] < errs[0] and errs[-1] < 1e-5


def kkt_residual(x, y, A, bb, tol=1e-9):
    from scipy.optimize import nnls
    feas = max(0.0, float((A @ y - bb).max())) if bb.size else 0.0
    act = np.abs(A @ y - bb) <= tol * max(1.0, np.abs(bb).max() if bb.size else 1.0) * 10
    if not act.any():
        return feas, float(np.linalg.norm(x - y))
    lam, res = nnls(A[act].T, x - y)
    return feas, res


def test_random_projections_satisfy_kkt():
    rng = np.random.default_rng(5)
    for nd in (1, 2, 3):
        for _ in range(40):
            npoints = int(rng.integers(nd + 1, 10))
            nsub = int(rng.integers(nd + 1, npoints + 1))
            J = rng.choice(npoints, nsub, replace=False)[None, :].astype(np.int64)
            I = np.ones((1, npoints), bool)
            v = rng.uniform(-2, 2, (npoints, nd))
            b = rng.uniform(-2, 2, (1, npoints))
            x = rng.uniform(-5, 5, (1, 1, nd + 1))
            A, bb, _ = E.instance_constraints(I, J, v, b, 0, 0)
            y, ok = E.project_polyhedron(x[0, 0], A, bb, nd * nsub)
            assert ok
            feas, res = kkt_residual(x[0, 0], y, A, bb)
            assert feas <= 1e-10 and res <= 1e-8, (nd, feas, res)


def test_oracle_matches_reference_library_random():
    """Direct cross-check against the host build of the reference's QP
    (present only where the reference sources were compiled)."""
    import ctypes as C
    from oracle import build_ref
    rng = np.random.default_rng(11)
    for nd in (1, 2, 3):
        path = build_ref.lib_path(nd)
        if not os.path.exists(path):
            pytest.skip("oracle/_ref not built (reference sources absent)")
        lib = C.CDLL(path)
        lib.ref_epigraph_proj.argtypes = [C.c_void_p] * 5 + [C.c_int] * 4
        for _ in range(25):
            npoints = int(rng.integers(nd + 1, 12))
            nfuns, nreg = int(rng.integers(1, 5)), int(rng.integers(1, 4))
            nsub = int(rng.integers(nd + 1, npoints + 1))
            J = np.stack([rng.choice(npoints, nsub, replace=False) for _ in range(nreg)])
            J = J.astype(np.int64)
            I = (rng.random((nfuns, npoints)) < 0.8).astype(np.uint8)
            v = rng.uniform(-2, 2, (npoints, nd))
            b = rng.uniform(-2, 2, (nfuns, npoints))
            x = rng.uniform(-5, 5, (nreg, nfuns, nd + 1))
            yr = x.copy()
            lib.ref_epigraph_proj(yr.ctypes.data, I.ctypes.data, J.ctypes.data, v.ctypes.data,
                                  b.ctypes.data, nfuns, nreg, npoints, nsub)
            yo, _ = E.epigraph_proj(I.astype(bool), J, v, b, x)
            assert np.abs(yo - yr).max() <= 1e-10
