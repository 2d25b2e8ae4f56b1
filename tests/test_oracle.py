"""Pin the CPU oracle against the reference's golden vectors.

The fixtures in tests/golden/ come from running the reference's own Python
code (tests/golden/make_golden.py); the gradient values in
``REF_TEST_DV`` are the golden arrays of the reference's tests/sparse.py:59-93.
"""

import os

import numpy as np
import pytest

import oracle
from oracle import linops, prox, functionals as fn
from tests.conftest import GOLDEN

OPS = np.load(os.path.join(GOLDEN, "ops.npz"))

# reference tests/sparse.py:59-93 (centered scheme, 4x5 grid, y[t, r, c])
REF_TEST_V = np.array([[0., 0., 0., 0., 0.],
                       [0., 1., 0., 0., 0.],
                       [0., 0., 0., 0., 1.],
                       [0., 0., 0., 0., 0.]])
REF_TEST_DV = np.array([[[0.5, 0.5, 0., 0., 0.],
                         [-0.5, -0.5, 0., 0.5, 0.],
                         [0., 0., 0., -0.5, 0.],
                         [0., 0., 0., 0., 0.]],
                        [[0.5, -0.5, 0., 0., 0.],
                         [0.5, -0.5, 0., 0.5, 0.],
                         [0., 0., 0., 0.5, 0.],
                         [0., 0., 0., 0., 0.]]])


@pytest.mark.parametrize("C", [1, 2, 3])
def test_gradient_reference_golden(C):
    """reference tests/sparse.py:95-104 (test_gradop, centered)."""
    cc = min(1, C - 1)
    rng = np.random.default_rng(C)
    w = rng.standard_normal(C * REF_TEST_V.size)
    w.reshape(-1, C)[:, cc] = REF_TEST_V.ravel()
    op = linops.Gradient(REF_TEST_V.shape, C, scheme="centered")
    Dw = op.spmat.dot(w)
    expect = REF_TEST_DV.transpose(1, 2, 0).ravel()
    assert np.linalg.norm(Dw.reshape(-1, C)[:, cc] - expect, ord=np.inf) == 0.0


def _linop_keys(prefix):
    return sorted({k.split("/")[0] for k in OPS.files if k.startswith(prefix)})


def _check_linop(key, op):
    x, y = OPS[key + "/x"], OPS[key + "/y"]
    Ax = np.zeros(op.y_size)
    ATy = np.zeros(op.x_size)
    op(x, Ax)
    op.adjoint(y, ATy)
    np.testing.assert_allclose(Ax, OPS[key + "/Ax"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(ATy, OPS[key + "/ATy"], rtol=0, atol=1e-12)
    for p in (1, 2):
        r = np.zeros(op.y_size)
        op.rowwise_lp(r, p=p)
        np.testing.assert_allclose(r, OPS[key + "/rowlp%d" % p], rtol=1e-13, atol=1e-13)
        if key + "/collp%d" % p in OPS.files:
            r = np.zeros(op.x_size)
            op.adjoint.rowwise_lp(r, p=p)
            np.testing.assert_allclose(r, OPS[key + "/collp%d" % p], rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("key", _linop_keys("grad_"))
def test_gradient_ops(key):
    scheme = "forward" if "_fwd_" in key else "centered"
    op = linops.Gradient(tuple(OPS[key + "/dims"]), int(OPS[key + "/C"]), scheme,
                         OPS[key + "/h"], OPS[key + "/w"])
    _check_linop(key, op)


@pytest.mark.parametrize("key", _linop_keys("lapl_"))
def test_laplacian_ops(key):
    bc = key.split("_")[1]
    op = linops.Laplacian(tuple(OPS[key + "/dims"]), int(OPS[key + "/C"]),
                          OPS[key + "/h"], bc)
    _check_linop(key, op)


N_EINSUM = 37


@pytest.mark.parametrize("key", ["mm_n", "mm_t", "mmr_n", "mmr_t", "mmrb_n", "mmrb_t",
                                 "tmmr_n", "tmmr_t", "dmmr", "idx"])
def test_einsum_indexed_ops(key):
    A = OPS[key + "/A"] if key != "idx" else None
    trans = key.endswith("_t")
    if key.startswith("mmrb"):
        op = linops.MatrixMultRBatched(N_EINSUM, A, trans)
    elif key.startswith("mmr"):
        op = linops.MatrixMultR(N_EINSUM, A, trans)
    elif key.startswith("mm"):
        op = linops.MatrixMult(N_EINSUM, A, trans)
    elif key.startswith("tmmr"):
        op = linops.TangledMatrixMultR(N_EINSUM, A, trans)
    elif key == "dmmr":
        op = linops.DiagMatrixMultR(N_EINSUM, A)
    else:
        op = linops.IndexedMult(int(OPS["idx/K"]), N_EINSUM, OPS["idx/B"], OPS["idx/P"])
    _check_linop(key, op)


@pytest.mark.parametrize("key", sorted({k.split("/")[0] for k in OPS.files
                                        if k.startswith("l1proj_")}))
def test_l1_projection(key):
    norm, shp = key.split("_")[1:]
    M = tuple(int(v) for v in shp.split("x"))
    x = OPS[key + "/x"].copy()
    N = x.size // (M[0] * M[1])
    prox.l1_projection(x, N, M, float(OPS[key + "/lbd"]), norm)
    np.testing.assert_allclose(x, OPS[key + "/y"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("variant", ["abc", "shift", "trunc", "plain"])
def test_quadepi_projection(variant):
    key = "quadepi_" + variant
    x = OPS[key + "/x"].copy()
    shift = OPS[key + "/shift"]
    N = 40
    prox.quadepi_projection(x, N, 2, float(OPS[key + "/alph"]),
                            shift=None if shift.size == 0 else shift,
                            lbd=float(OPS[key + "/lbd"]))
    np.testing.assert_allclose(x, OPS[key + "/y"], rtol=1e-11, atol=1e-11)


def test_cubic_and_truncate():
    x = prox.solve_reduced_monic_cubic(OPS["cubic/a"], OPS["cubic/b"])
    np.testing.assert_allclose(x, OPS["cubic/x"], rtol=1e-13, atol=1e-13)
    y = np.array([prox.truncate(v, 3) for v in OPS["truncate/x"]])
    np.testing.assert_array_equal(y, OPS["truncate/y"])


def test_functional_values():
    G = fn.SSD(OPS["ssd/f"], vol=OPS["ssd/vol"], mask=OPS["ssd/mask"])
    x = OPS["ssd/x"]
    assert abs(G(x)[0] - OPS["ssd/val"]) < 1e-12
    assert abs(G.conj(x)[0] - OPS["ssd/conjval"]) < 1e-12
    px = x.copy()
    G.prox(OPS["ssd/tau"])(px)
    np.testing.assert_allclose(px, OPS["ssd/prox"], rtol=0, atol=1e-13)

    y = OPS["l1/x"]
    F = fn.L1Norms(30, (3, 2), 0.3)
    assert abs(F(y)[0] - OPS["l1/val"]) < 1e-12
    assert abs(F.conj(y)[1] - OPS["l1conj/infeas"]) < 1e-13
    Fn = fn.L1Norms(30, (2, 3), 0.3, matrixnorm="nuclear")
    assert abs(Fn(y)[0] - OPS["l1nuc/val"]) < 1e-12
    assert abs(Fn.conj(y)[1] - OPS["l1spec/infeas"]) < 1e-12

    hx = OPS["huberpersp/x"]
    Hb = fn.HuberPerspective(30, 2, lbd=0.7, alph=0.4)
    assert abs(Hb(hx)[0] - OPS["huberpersp/val"]) < 1e-12
    assert abs(Hb(hx)[1] - OPS["huberpersp/infeas"]) < 1e-12
    assert abs(Hb.conj(hx)[1] - OPS["truncquad/infeas"]) < 1e-12
    Qi = fn.QuadEpiInd(30, 2, a=1.5, b=OPS["quadepi_ind/b"], c=OPS["quadepi_ind/c"])
    assert abs(Qi(hx)[1] - OPS["quadepi_ind/infeas"]) < 1e-12
    assert abs(Qi.conj(hx)[0] - OPS["quadepi_supp/val"]) < 1e-10
    assert abs(Qi.conj(hx)[1] - OPS["quadepi_supp/infeas"]) < 1e-12


def test_normest_seeded():
    op = linops.Gradient((12, 9), 2, scheme="forward")
    np.random.seed(5)
    e, itn = linops.normest(op)
    assert itn == int(OPS["normest/itn"])
    assert abs(e - float(OPS["normest/e"])) < 1e-12


SOLVER_CASES = sorted(f[:-4] for f in os.listdir(GOLDEN)
                      if f.endswith(".npz") and f not in ("ops.npz", "epigraph.npz")
                      and not f.startswith("sublabel") and f != "ssn.npz")


def build_problem(d):
    """The oracle problem of a solver fixture."""
    dims = tuple(int(v) for v in d["imagedims"])
    f = d["f"]
    C = f.shape[-1]
    N = int(np.prod(dims))
    D = len(dims)
    G = fn.SSD(f.reshape(N, C), vol=d["vol"], mask=d["mask"])
    if float(d["huber"]) > 0:
        F = fn.HuberL1Norms(N, (C, D), float(d["lbd"]), float(d["huber"]))
    else:
        F = fn.L1Norms(N, (C, D), float(d["lbd"]))
    A = linops.Gradient(dims, C, str(d["scheme"]), d["imageh"], d["weights"])
    return G, F, A


def run_oracle_case(d, iters=None, precision="double"):
    G, F, A = build_problem(d)
    solver = oracle.PDHG(G, F, A)
    rec = {}

    def cb(state, info):
        rec[info["iter"]] = (state[0].copy(), state[1].copy(), dict(info),
                             solver.itervars.get("tauk", np.nan))

    np.random.seed(0)
    solver.solve(steps=str(d["steps"]), precision=precision, term_pd_gap=1e-300,
                 term_maxiter=int(d["iters_total"]) if iters is None else iters,
                 granularity=int(d["gran"]), cbfun=cb)
    return rec


@pytest.mark.parametrize("case", [c for c in SOLVER_CASES if c != "rof_gray256_adaptive"])
def test_oracle_solver_matches_reference(case):
    d = np.load(os.path.join(GOLDEN, case + ".npz"))
    rec = run_oracle_case(d)
    for j, it in enumerate(d["dump_iters"]):
        x, y, info, tau = rec[int(it)]
        assert np.linalg.norm(x - d["x"][j]) <= 1e-12 * max(1.0, np.linalg.norm(d["x"][j]))
        assert np.linalg.norm(y - d["y"][j]) <= 1e-12 * max(1.0, np.linalg.norm(d["y"][j]))
    for j, it in enumerate(d["info_iters"]):
        info = rec[int(it)][2]
        for k in ["objp", "objd", "gap"]:
            ref = d["info_" + k][j]
            assert abs(info[k] - ref) <= 1e-10 * max(1.0, abs(ref)), (k, it)
        if str(d["steps"]) == "adaptive":
            assert rec[int(it)][3] == d["info_tau"][j]


@pytest.mark.slow
def test_oracle_rof256_adaptive():
    d = np.load(os.path.join(GOLDEN, "rof_gray256_adaptive.npz"))
    rec = run_oracle_case(d)
    x, y, info, tau = rec[1000]
    assert np.linalg.norm(x - d["x"][0]) <= 1e-12 * np.linalg.norm(d["x"][0])
    assert np.linalg.norm(y - d["y"][0]) <= 1e-12 * np.linalg.norm(d["y"][0])
    for j, it in enumerate(d["info_iters"]):
        assert abs(rec[int(it)][2]["relgap"] - d["info_relgap"][j]) < 1e-9
        assert rec[int(it)][3] == d["info_tau"][j]
