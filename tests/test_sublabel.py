"""The sublabel lifting workload (opymize_gb300/tools/lifting.py) on the CPU
oracle against the reference's own PDHG run of the same model
(tests/golden/sublabel_*.npz, tests/golden/make_sublabel_golden.py), plus
host-side checks of the model data."""

import os

import numpy as np
import pytest

import oracle
from oracle.functionals import EpigraphSupp
from opymize_gb300.tools import lifting
from tests.conftest import GOLDEN

CASES = ["sublabel_small_precond", "sublabel_small_adaptive"]


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def fixture_faces(z, L, N):
    """If[i][j] from the flattened faces of a fixture."""
    flat, nf = z["faces"], z["nfaces"]
    If, pos = [], 0
    for i in range(N):
        row = []
        for j in range(L - 1):
            row.append(flat[pos:pos + nf[i, j]])
            pos += nf[i, j]
        If.append(row)
    return If


def oracle_model(z, with_faces=True):
    img = z["img"]
    L, lbd = int(z["L"]), float(z["lbd"])
    dims = img.shape
    N, D = int(np.prod(dims)), len(dims)
    d = lifting.sublabel_data(img.ravel(), L, int(z["samples"]), float(z["trunc"]))
    If = fixture_faces(z, L, N) if with_faces else None
    nmu = (L - 1) * N * 2
    g = oracle.SplitSum([oracle.PositivityFct(N * L), oracle.ZeroFct(N), oracle.ZeroFct(nmu)])
    f = oracle.SplitSum([oracle.IndicatorFct(N * L), oracle.IndicatorFct(N),
                         oracle.L1Norms(N, (1, D), lbd), oracle.IndicatorFct(N, c1=1.0),
                         EpigraphSupp(d["I"], If, d["J"], d["v"], d["b"])])
    Z = oracle.ZeroOp
    A = oracle.BlockOp([
        [oracle.IdentityOp(N * L), Z(N * L, N), oracle.IndexedMultAdj(L, N, d["P"], d["Bc"])],
        [oracle.MatrixMultR(N, d["t"][:, None]), oracle.ScaleOp(N, -1.0), Z(N, nmu)],
        [Z(N * D, N * L), oracle.Gradient(dims, 1, "forward"), Z(N * D, nmu)],
        [oracle.MatrixMultR(N, np.ones((L, 1))), Z(N, N), Z(N, nmu)],
        [Z(nmu, N * L), Z(nmu, N), oracle.IdentityOp(nmu)]])
    return g, f, A, d


def test_model_data():
    d = lifting.sublabel_data(np.array([0.0, 0.33, 1.0]), L=4, samples=5, trunc=0.04)
    assert d["v"].shape == (13, 1) and d["J"].shape == (3, 5)
    # the first two points of every region are its endpoints (simplex vertices)
    assert np.allclose(d["v"][d["J"][:, 0], 0], d["t"][:-1])
    assert np.allclose(d["v"][d["J"][:, 1], 0], d["t"][1:])
    # B q = (slope, t_j*slope - q_j) per interval: check on q = 3 t + 1
    q = 3 * d["t"] + 1
    Bq = np.einsum("jml,jl->jm", d["Bc"], q[d["P"]])
    assert np.allclose(Bq[:, 0], 3.0) and np.allclose(Bq[:, 1], -1.0)
    # hull faces cover the interval and the envelope lies below the samples
    for i in range(3):
        for j in range(3):
            fc = lifting.lower_hull_faces(d, i, j)
            xs = d["v"][d["J"][j], 0]
            assert xs[fc[0, 0]] == xs.min() and xs[fc[-1, 1]] == xs.max()


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    z = load(name)
    g, f, A, _ = oracle_model(z)
    solver = oracle.PDHG(g, f, A)
    rec = {}

    def cb(state, info):
        rec[info["iter"]] = (state[0].copy(), state[1].copy(), dict(info))

    np.random.seed(0)
    solver.solve(steps=str(z["steps"]), precision="double", term_pd_gap=1e-300,
                 term_maxiter=int(z["iters"]), granularity=int(z["gran"]), cbfun=cb)
    for k, it in enumerate(z["dump_iters"]):
        x, y, info = rec[int(it)]
        for a, b in ((x, z["x"][k]), (y, z["y"][k])):
            assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(b), (name, it)
        ref = z["info"][k]
        assert info["objp"] == pytest.approx(ref[1], rel=1e-9, abs=1e-9)
        assert info["objd"] == pytest.approx(ref[2], rel=1e-9, abs=1e-9)


def test_envelope_value_equals_faces_value():
    z = load(CASES[0])
    _, f, _, d = oracle_model(z)
    supp = f.fcts[-1]
    nof = EpigraphSupp(d["I"], None, d["J"], d["v"], d["b"])
    rng = np.random.default_rng(1)
    x = np.zeros(supp.shape)
    x[..., 1] = -rng.random(x.shape[:2]) - 0.1
    for j in range(x.shape[0]):
        x[j, :, 0] = -x[j, :, 1] * (d["t"][j] + rng.random(x.shape[1]) * d["h"])
    a, b = supp(x.ravel()), nof(x.ravel())
    assert a[0] == pytest.approx(b[0], rel=1e-12) and a[1] == b[1] == 0
    # also outside the regions (infeasible points): the hull's end edges
    for _ in range(3):
        x = rng.normal(0, 1, supp.shape)
        a, b = supp(x.ravel()), nof(x.ravel())
        assert a[0] == pytest.approx(b[0], rel=1e-12) and a[1] == pytest.approx(b[1])
