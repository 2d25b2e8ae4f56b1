"""GPU parity of every operator, prox map and functional against the CPU
oracle, on the inputs of the golden fixtures (the reference's
test_gpu_op / compare_vars bootstrap, opymize/tools/tests.py:69-95).

Tolerances: FP64 1e-12 (absolute on O(1) data, relative 1e-12 on reductions);
FP32 relative L2 error 1e-5."""

import os

import numpy as np
import pytest

import oracle
from oracle import linops as olin, prox as oprox, functionals as ofn
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu

OPS = np.load(os.path.join(GOLDEN, "ops.npz"))
DTYPES = [np.float64, np.float32]


def tol_ok(got, ref, dtype):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    if dtype == np.float64:
        return np.max(np.abs(got - ref), initial=0.0) <= 1e-12 * max(1.0, np.max(np.abs(ref), initial=0.0))
    return np.linalg.norm(got - ref) <= 1e-5 * max(1e-30, np.linalg.norm(ref)) + 1e-6 * np.sqrt(ref.size) * 1e-1


@pytest.fixture(scope="module")
def gpu():
    import opymize_gb300.gpuarray as ga
    ga.torch()
    return ga


def _linop_check(gpu, key, op, dtype):
    x, y = OPS[key + "/x"], OPS[key + "/y"]
    xd = gpu.to_gpu(x, dtype)
    yd = gpu.to_gpu(y, dtype)
    Ax = gpu.DeviceArray.zeros((op.y.size,), dtype)
    ATy = gpu.DeviceArray.zeros((op.x.size,), dtype)
    op(xd, Ax)
    op.adjoint(yd, ATy)
    assert tol_ok(Ax.get(), OPS[key + "/Ax"], dtype), key
    assert tol_ok(ATy.get(), OPS[key + "/ATy"], dtype), key
    # add=True accumulates
    op(xd, Ax, add=True)
    assert tol_ok(Ax.get(), 2 * OPS[key + "/Ax"], dtype), key
    for p in (1, 2):
        r = gpu.DeviceArray.zeros((op.y.size,), dtype)
        op.rowwise_lp(r, p=p)
        assert tol_ok(r.get(), OPS[key + "/rowlp%d" % p], dtype), (key, p)
        if key + "/collp%d" % p in OPS.files:
            r = gpu.DeviceArray.zeros((op.x.size,), dtype)
            op.adjoint.rowwise_lp(r, p=p)
            assert tol_ok(r.get(), OPS[key + "/collp%d" % p], dtype), (key, "col", p)


GRAD_KEYS = sorted({k.split("/")[0] for k in OPS.files if k.startswith("grad_")})


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("key", GRAD_KEYS)
def test_gradient_divergence(gpu, key, dtype):
    from opymize_gb300.linear import GradientOp
    scheme = "forward" if "_fwd_" in key else "centered"
    op = GradientOp(tuple(OPS[key + "/dims"]), int(OPS[key + "/C"]), scheme=scheme,
                    imageh=OPS[key + "/h"], weights=OPS[key + "/w"])
    _linop_check(gpu, key, op, dtype)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("dims", [(6, 5, 4), (3, 4, 3, 2)])
def test_centered_gradient_high_dim(gpu, dims, dtype):
    """Centered scheme for D >= 3 follows the reference's GPU kernel
    (2^(D-1)-point average, diff.cu:53-63), restated in the oracle."""
    from opymize_gb300.linear import GradientOp
    C = 2
    op = GradientOp(dims, C, scheme="centered", imageh=np.linspace(0.5, 1.5, len(dims)),
                    weights=np.array([1.0, 0.5]))
    ref = olin.Gradient(dims, C, "centered", np.linspace(0.5, 1.5, len(dims)), np.array([1.0, 0.5]))
    rng = np.random.default_rng(0)
    x, y = rng.standard_normal(op.x.size), rng.standard_normal(op.y.size)
    Ax, ATy = gpu.DeviceArray.zeros((op.y.size,), dtype), gpu.DeviceArray.zeros((op.x.size,), dtype)
    op(gpu.to_gpu(x, dtype), Ax)
    op.adjoint(gpu.to_gpu(y, dtype), ATy)
    assert tol_ok(Ax.get(), ref.spmat.dot(x), dtype)
    assert tol_ok(ATy.get(), ref.spmat.T.dot(y), dtype)
    # unit slope along axis 0 averages to 1 in the interior
    xs = np.indices(dims)[0].astype(float)
    xs = np.repeat(xs.reshape(-1, 1), C, axis=1).ravel()
    op(gpu.to_gpu(xs, dtype), Ax)
    g = Ax.get().reshape(dims + (len(dims), C))
    assert abs(g[(0,) * len(dims)][0, 0] - 1.0 / 0.5) < 1e-5


LAPL_KEYS = sorted({k.split("/")[0] for k in OPS.files if k.startswith("lapl_")})


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("key", LAPL_KEYS)
def test_laplacian(gpu, key, dtype):
    from opymize_gb300.linear import LaplacianOp
    bc = key.split("_")[1]
    op = LaplacianOp(tuple(OPS[key + "/dims"]), int(OPS[key + "/C"]), imageh=OPS[key + "/h"],
                     boundary=bc)
    _linop_check(gpu, key, op, dtype)


N_EINSUM = 37


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("key", ["mm_n", "mm_t", "mmr_n", "mmr_t", "mmrb_n", "mmrb_t",
                                 "tmmr_n", "tmmr_t", "dmmr", "idx"])
def test_einsum_and_indexed(gpu, key, dtype):
    from opymize_gb300 import linear as L
    A = OPS[key + "/A"] if key != "idx" else None
    trans = key.endswith("_t")
    if key.startswith("mmrb"):
        op = L.MatrixMultRBatched(N_EINSUM, A, trans)
    elif key.startswith("mmr"):
        op = L.MatrixMultR(N_EINSUM, A, trans)
    elif key.startswith("mm"):
        op = L.MatrixMult(N_EINSUM, A, trans)
    elif key.startswith("tmmr"):
        op = L.TangledMatrixMultR(N_EINSUM, A, trans)
    elif key == "dmmr":
        op = L.DiagMatrixMultR(N_EINSUM, A)
    else:
        op = L.IndexedMult(int(OPS["idx/K"]), N_EINSUM, OPS["idx/B"], OPS["idx/P"])
    _linop_check(gpu, key, op, dtype)


def test_nonsquare_matrixmult_and_duplicate_labels(gpu):
    """Non-square MatrixMult (which the reference cannot build) and label
    indices with duplicates, against the oracle."""
    from opymize_gb300 import linear as L
    rng = np.random.default_rng(2)
    A = rng.standard_normal((4, 7))
    for trans in (False, True):
        op, ref = L.MatrixMult(11, A, trans), olin.MatrixMult(11, A, trans)
        x = rng.standard_normal(op.x.size)
        y = gpu.DeviceArray.zeros((op.y.size,))
        op(gpu.to_gpu(x), y)
        assert tol_ok(y.get(), ref.spmat.dot(x), np.float64)
    B = rng.standard_normal((3, 2, 4))
    P = np.array([[0, 0, 1, 2], [3, 3, 3, 0], [1, 2, 1, 2]])
    op, ref = L.IndexedMult(4, 9, B, P), olin.IndexedMult(4, 9, B, P)
    for p in (1, 2):
        r = gpu.DeviceArray.zeros((op.y.size,))
        op.rowwise_lp(r, p=p)
        rr = np.zeros(op.y.size)
        ref.rowwise_lp(rr, p=p)
        assert tol_ok(r.get(), rr, np.float64)
        r = gpu.DeviceArray.zeros((op.x.size,))
        op.adjoint.rowwise_lp(r, p=p)
        rr = np.zeros(op.x.size)
        ref.adjoint.rowwise_lp(rr, p=p)
        assert tol_ok(r.get(), rr, np.float64)
    y = rng.standard_normal(op.y.size)
    out = gpu.DeviceArray.zeros((op.x.size,))
    op.adjoint(gpu.to_gpu(y), out)
    assert tol_ok(out.get(), ref.spmat.T.dot(y), np.float64)


# Sizes with many CTAs (grid-stride loops), divisors that are not powers of
# two, and tables too large for the per-CTA shared-memory copy (the per-use
# FP64 path).
EINSUM_MANY = [("mm", (5, 7), 50021), ("mm", (100, 100), 3001), ("mmr", (16, 1), 70001),
               ("mmr", (1, 16), 70001), ("mmr", (3, 5), 40009), ("mmrb", (4, 3, 5), 9001),
               ("tmmr", (3, 2, 4, 5), 7001), ("dmmr", (7,), 30011),
               ("mmr", (3, 5), 400009), ("mmr", (50, 3), 20011), ("mmr", (100, 100), 3001)]


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("case", range(len(EINSUM_MANY)))
def test_einsum_many_ctas(gpu, case, dtype):
    from opymize_gb300 import linear as L
    kind, shape, N = EINSUM_MANY[case]
    rng = np.random.default_rng(case)
    A = rng.standard_normal(shape)
    for trans in ((False,) if kind == "dmmr" else (False, True)):
        if kind == "dmmr":
            op, ref = L.DiagMatrixMultR(N, A), olin.DiagMatrixMultR(N, A)
        else:
            cls = {"mm": "MatrixMult", "mmr": "MatrixMultR", "mmrb": "MatrixMultRBatched",
                   "tmmr": "TangledMatrixMultR"}[kind]
            op, ref = getattr(L, cls)(N, A, trans), getattr(olin, cls)(N, A, trans)
        x = rng.standard_normal(op.x.size)
        y = rng.standard_normal(op.y.size)
        Ax, ATy = np.zeros(op.y.size), np.zeros(op.x.size)
        ref(x, Ax)
        ref.adjoint(y, ATy)
        got = gpu.DeviceArray.zeros((op.y.size,), dtype)
        op(gpu.to_gpu(x, dtype), got)
        assert tol_ok(got.get(), Ax, dtype), (kind, shape, trans)
        got = gpu.DeviceArray.zeros((op.x.size,), dtype)
        op.adjoint(gpu.to_gpu(y, dtype), got)
        assert tol_ok(got.get(), ATy, dtype), (kind, shape, trans, "adjoint")


# (K, N, J, M, L, P): the sublabel layout (P[j] = (j, j+1)); random labels with
# duplicates; more labels than threads per CTA; more (j, l) pairs than the
# per-CTA label lists take (the unlisted scatter); more pixel tiles than CTAs
def _indexed_cases():
    r = np.random.default_rng(11)
    return [(16, 70001, 15, 2, 2, np.stack([np.arange(15), np.arange(1, 16)], 1)),
            (9, 20011, 6, 3, 4, r.integers(0, 9, (6, 4))),
            (300, 2001, 200, 1, 2, r.integers(0, 300, (200, 2))),
            (5, 301, 2100, 1, 2, r.integers(0, 5, (2100, 2))),
            (4, 400009, 3, 2, 2, r.integers(0, 4, (3, 2)))]


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("case", range(5))
def test_indexed_many_ctas(gpu, case, dtype):
    from opymize_gb300 import linear as L
    K, N, J, M, Ln, P = _indexed_cases()[case]
    rng = np.random.default_rng(case)
    B = rng.standard_normal((J, M, Ln))
    op, ref = L.IndexedMult(K, N, B, P), olin.IndexedMult(K, N, B, P)
    x = rng.standard_normal(op.x.size)
    y = rng.standard_normal(op.y.size)
    got = gpu.DeviceArray.zeros((op.y.size,), dtype)
    op(gpu.to_gpu(x, dtype), got)
    assert tol_ok(got.get(), ref.spmat.dot(x), dtype)
    got = gpu.DeviceArray.zeros((op.x.size,), dtype)
    op.adjoint(gpu.to_gpu(y, dtype), got)
    assert tol_ok(got.get(), ref.spmat.T.dot(y), dtype)
    # add=True accumulates onto the output
    op.adjoint(gpu.to_gpu(y, dtype), got, add=True)
    assert tol_ok(got.get(), 2 * ref.spmat.T.dot(y), dtype)


L1_KEYS = sorted({k.split("/")[0] for k in OPS.files if k.startswith("l1proj_")})


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("key", L1_KEYS)
def test_l1_projection(gpu, key, dtype):
    from opymize_gb300.operators import L1NormsProj
    norm, shp = key.split("_")[1:]
    M = tuple(int(v) for v in shp.split("x"))
    x = OPS[key + "/x"]
    N = x.size // (M[0] * M[1])
    lbd = float(OPS[key + "/lbd"])
    if norm == "spectral" and M[0] != M[1] and 1 not in M:
        # the GPU layout reads a group as the (M[1], M[0]) matrix, which is what
        # the reference's CPU path reads for M' = (M[1], M[0])
        other = "l1proj_spectral_%dx%d" % (M[1], M[0])
        x, ref = OPS[other + "/x"], OPS[other + "/y"]
    else:
        ref = OPS[key + "/y"]
    xd = gpu.to_gpu(x, dtype)
    L1NormsProj(N, M, lbd, norm)(xd)
    assert tol_ok(xd.get(), ref, dtype), key


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("variant", ["abc", "shift", "trunc", "plain"])
def test_quadepi_projection(gpu, variant, dtype):
    from opymize_gb300.operators import QuadEpiProj
    key = "quadepi_" + variant
    shift = OPS[key + "/shift"]
    op = QuadEpiProj(40, 2, alph=float(OPS[key + "/alph"]),
                     shift=None if shift.size == 0 else shift, lbd=float(OPS[key + "/lbd"]))
    xd = gpu.to_gpu(OPS[key + "/x"], dtype)
    op(xd)
    ref = OPS[key + "/y"]
    if dtype == np.float64:
        assert np.max(np.abs(xd.get() - ref)) < 1e-10
    else:
        assert np.linalg.norm(xd.get() - ref) <= 1e-5 * np.linalg.norm(ref)


@pytest.mark.parametrize("dtype", DTYPES)
def test_quadepi_known_answers(gpu, dtype):
    """Geometry of the reference's tests/quadepi.py:21-82: inside points are
    fixed, outside points land on the paraboloid, truncated points on the
    rim."""
    from opymize_gb300.operators import QuadEpiProj
    rng = np.random.default_rng(11)
    tol = 1e-10 if dtype == np.float64 else 2e-4
    for _ in range(5):
        N, M = 50, int(rng.integers(1, 5))
        a = 0.5 + 10 * rng.random()
        f = lambda v: 0.5 * a * (v ** 2).sum(axis=1)
        x = np.zeros((N, M + 1))
        d = rng.standard_normal((N, M))
        x[:, :-1] = 3 * d / np.linalg.norm(d, axis=1)[:, None] * rng.random((N, 1))
        x[:, -1] = f(x[:, :-1]) + rng.random(N)
        xd = gpu.to_gpu(x.ravel(), dtype)
        QuadEpiProj(N, M, alph=a)(xd)
        assert np.max(np.abs(xd.get() - x.ravel())) < tol * 10
        x[:, -1] = f(x[:, :-1]) - 3 * rng.random(N)
        xd = gpu.to_gpu(x.ravel(), dtype)
        QuadEpiProj(N, M, alph=a)(xd)
        y = xd.get().reshape(N, M + 1).astype(np.float64)
        assert np.max(np.abs(f(y[:, :-1]) - y[:, -1])) < tol * max(1.0, a) * 10


@pytest.mark.parametrize("dtype", DTYPES)
def test_prox_maps(gpu, dtype):
    from opymize_gb300.functionals import SSD, PositivityFct, NegativityFct, HuberL1Norms
    from opymize_gb300.operators import ConstrainOp, ShiftScaleOp
    rng = np.random.default_rng(5)
    f, vol, msk = OPS["ssd/f"], OPS["ssd/vol"], OPS["ssd/mask"]
    G = SSD(f, vol=vol, mask=msk)
    xd = gpu.to_gpu(OPS["ssd/x"], dtype)
    tau = gpu.to_gpu(OPS["ssd/tau"], dtype)
    G.prox(tau)(xd)
    assert tol_ok(xd.get(), OPS["ssd/prox"], dtype)
    x = rng.standard_normal(40)
    for F, ref in ((PositivityFct(40), np.fmax(0, x)), (NegativityFct(40), np.fmin(0, x))):
        xd = gpu.to_gpu(x, dtype)
        F.prox(1.0)(xd)
        assert tol_ok(xd.get(), ref, dtype)
    c = rng.standard_normal((10, 4))
    m = rng.random(10) < 0.5
    xd = gpu.to_gpu(x, dtype)
    ConstrainOp(m, c)(xd)
    ref = x.reshape(10, 4).copy()
    ref[m] = c[m]
    assert tol_ok(xd.get(), ref.ravel(), dtype)
    a, b, s = rng.random(40), rng.random(40), rng.random(40)
    yd = gpu.DeviceArray.zeros((40,), dtype)
    ShiftScaleOp(40, s, a, b)(gpu.to_gpu(x, dtype), yd)
    assert tol_ok(yd.get(), a * (x + b * s), dtype)
    # Huber conjugate prox
    Fh = HuberL1Norms(20, (3, 2), 0.3, 0.05)
    y = rng.standard_normal(120)
    sig = 0.1 + rng.random(120)
    yd = gpu.to_gpu(y, dtype)
    Fh.conj.prox(gpu.to_gpu(sig, dtype))(yd)
    ref = y.copy()
    oprox.huber_conj_prox(ref, 20, (3, 2), 0.3, 0.05, sig)
    assert tol_ok(yd.get(), ref, dtype)


@pytest.mark.parametrize("dtype", DTYPES)
def test_functional_values(gpu, dtype):
    from opymize_gb300 import functionals as F
    rtol = 1e-12 if dtype == np.float64 else 1e-5
    G = F.SSD(OPS["ssd/f"], vol=OPS["ssd/vol"], mask=OPS["ssd/mask"])
    x = gpu.to_gpu(OPS["ssd/x"], dtype)
    assert abs(G(x)[0] - OPS["ssd/val"]) <= rtol * abs(OPS["ssd/val"])
    assert abs(G.conj(x)[0] - OPS["ssd/conjval"]) <= rtol * abs(OPS["ssd/conjval"]) * 10
    y = gpu.to_gpu(OPS["l1/x"], dtype)
    L1 = F.L1Norms(30, (3, 2), 0.3)
    assert abs(L1(y)[0] - OPS["l1/val"]) <= rtol * abs(OPS["l1/val"])
    assert abs(L1.conj(y)[1] - OPS["l1conj/infeas"]) <= rtol * 10
    hx = gpu.to_gpu(OPS["huberpersp/x"], dtype)
    Hb = F.HuberPerspective(30, 2, lbd=0.7, alph=0.4)
    assert abs(Hb(hx)[0] - OPS["huberpersp/val"]) <= rtol * abs(OPS["huberpersp/val"]) * 10
    assert abs(Hb.conj(hx)[1] - OPS["truncquad/infeas"]) <= rtol * 10
    Qi = F.QuadEpiInd(30, 2, a=1.5, b=OPS["quadepi_ind/b"], c=OPS["quadepi_ind/c"])
    assert abs(Qi(hx)[1] - OPS["quadepi_ind/infeas"]) <= rtol * 10 * max(1, OPS["quadepi_ind/infeas"])
    assert abs(Qi.conj(hx)[0] - OPS["quadepi_supp/val"]) <= rtol * 100 * abs(OPS["quadepi_supp/val"])
    # Huber pair against the oracle
    rng = np.random.default_rng(9)
    z = rng.standard_normal(60) * 0.2
    H, Ho = F.HuberL1Norms(10, (3, 2), 0.3, 0.1), ofn.HuberL1Norms(10, (3, 2), 0.3, 0.1)
    zd = gpu.to_gpu(z, dtype)
    assert abs(H(zd)[0] - Ho(z)[0]) <= rtol * abs(Ho(z)[0]) * 10
    assert abs(H.conj(zd)[0] - Ho.conj(z)[0]) <= rtol * abs(Ho.conj(z)[0]) * 10
    assert abs(H.conj(zd)[1] - Ho.conj(z)[1]) <= rtol * 10


def test_normest_seeded(gpu):
    from opymize_gb300.linear import GradientOp, normest
    op = GradientOp((12, 9), 2, scheme="forward")
    np.random.seed(5)
    e, itn = normest(op)
    assert itn == int(OPS["normest/itn"])
    assert abs(e - float(OPS["normest/e"])) < 1e-12


def test_invalid_arguments_are_errors(gpu):
    """Bad sizes and enums come back as status codes, never as faults."""
    from opymize_gb300 import _lib
    from opymize_gb300.linear import GradientOp
    op = GradientOp((4, 5), 1, scheme="forward")
    with pytest.raises(ValueError):
        op(gpu.DeviceArray.zeros((19,)), gpu.DeviceArray.zeros((40,)))
    g = _lib.opyx_grid()
    g.ndim = 0
    with pytest.raises(_lib.OpyxError):
        _lib.call("opyx_gradient", g, 0, None, 1, 1, 1, 0, None)
    p = _lib.opyx_rof_problem()
    b = _lib.opyx_rof_buffers()
    p.ndim = 5
    with pytest.raises(_lib.OpyxError):
        _lib.call("opyx_rof_iterate", p, b, 1, None)
