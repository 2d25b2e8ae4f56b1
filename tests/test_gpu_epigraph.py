"""EpigraphProj / EpigraphInd / EpigraphSupp on the GPU against the
reference's own QP and functionals (tests/golden/epigraph.npz) and the
oracle.  Bars: FP64 projections within 1e-10 (absolute, inputs of size ~5)
of the reference's QP, values within 1e-12 relative; FP32 projections within
2e-5 relative to the input scale."""

import os

import numpy as np
import pytest

from oracle import epigraph as E
from tests.conftest import GOLDEN
from tests.test_oracle_epigraph import FIX, case

pytestmark = pytest.mark.gpu


def proj_gpu(d, x, dtype=np.float64, inplace=False):
    from opymize_gb300 import DeviceArray
    from opymize_gb300.operators import EpigraphProj
    op = EpigraphProj(d["I"], d["J"], d["v"], d["b"])
    xd = DeviceArray.to_gpu(np.ascontiguousarray(x).ravel(), dtype)
    if inplace:
        op(xd)
        out = xd
    else:
        out = DeviceArray.zeros((x.size,), dtype)
        op(xd, out)
        np.testing.assert_array_equal(xd.get(), np.asarray(x, dtype).ravel())
    return out.get().reshape(x.shape), op.nonconverged


@pytest.mark.parametrize("inplace", [False, True])
@pytest.mark.parametrize("c", range(int(FIX["nrand"])))
def test_fp64_matches_reference_qp(c, inplace):
    d = case("rand", c)
    y, bad = proj_gpu(d, d["x"], inplace=inplace)
    assert bad == 0
    assert np.abs(y - d["y"]).max() <= 1e-10


@pytest.mark.parametrize("c", range(int(FIX["nrand"])))
def test_fp32_matches_oracle(c):
    d = case("rand", c)
    y, bad = proj_gpu(d, d["x"], np.float32)
    assert bad == 0
    assert np.abs(y - d["y"]).max() <= 2e-5 * np.abs(d["x"]).max()


@pytest.mark.parametrize("c", range(int(FIX["nknown"])))
def test_known_answers(c):
    d = case("known", c)
    yi, _ = proj_gpu(d, d["inside"])
    yo, _ = proj_gpu(d, d["outside"])
    assert np.linalg.norm(yi - d["inside"]) ** 2 < 1e-10
    assert np.linalg.norm(yo - d["x_in"]) ** 2 < 1e-10


@pytest.mark.parametrize("c", range(int(FIX["nrand"])))
def test_indicator_values(c):
    from opymize_gb300 import DeviceArray
    from opymize_gb300.functionals import EpigraphInd
    d = case("rand", c)
    F = EpigraphInd(d["I"], None, d["J"], d["v"], d["b"])
    for key, arr in (("ind_x", d["x"]), ("ind_y", d["y"])):
        val, inf = F(DeviceArray.to_gpu(arr.ravel()))
        assert val == 0.0
        assert inf == pytest.approx(float(d[key][1]), rel=1e-12, abs=1e-12)
    assert F.prox(0.5) is F.prox(2.0)


@pytest.mark.parametrize("precision", ["double", "float"])
@pytest.mark.parametrize("c", range(int(FIX["nsupp"])))
def test_support_values(c, precision):
    from opymize_gb300 import DeviceArray
    from opymize_gb300.functionals import EpigraphSupp
    d = case("supp", c)
    If = [[d["faces"] for _ in range(d["J"].shape[0])] for _ in range(d["I"].shape[0])]
    F = EpigraphSupp(d["I"], If, d["J"], d["v"], d["b"])
    dt = np.float64 if precision == "double" else np.float32
    val, inf = F(DeviceArray.to_gpu(d["x"].ravel(), dt))
    tol = 1e-12 if precision == "double" else 1e-5
    assert val == pytest.approx(float(d["val"][0]), rel=tol)
    assert inf <= tol
    assert isinstance(F.conj, __import__("opymize_gb300").functionals.EpigraphInd)


def lifted_instances(rng, nfuns, L, nd=1):
    """Sublabel-style instances: nregions = L-1 intervals of L labels on
    [0, 1], nfuns pixels, b = per-pixel data term at the labels."""
    J = np.stack([np.arange(j, j + 2) for j in range(L - 1)]).astype(np.int64)
    v = np.linspace(0, 1, L)[:, None]
    f = rng.random(nfuns)
    b = np.minimum((v[:, 0][None, :] - f[:, None]) ** 2, 0.04)
    I = np.ones((nfuns, L), bool)
    x = rng.normal(0, 1, (L - 1, nfuns, nd + 1))
    return I, J, v, b, x


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_large_lifted_problem(dtype):
    """512 x 512 pixels x 15 regions (the sublabel layout): a random subset
    of instances against the oracle, idempotence on all of them."""
    from opymize_gb300 import DeviceArray
    from opymize_gb300.operators import EpigraphProj
    rng = np.random.default_rng(3)
    I, J, v, b, x = lifted_instances(rng, 512 * 512, 16)
    op = EpigraphProj(I, J, v, b)
    xd = DeviceArray.to_gpu(x.ravel(), dtype)
    yd = DeviceArray.zeros((x.size,), dtype)
    op(xd, yd)
    y = yd.get().reshape(x.shape)
    zd = DeviceArray.zeros((x.size,), dtype)
    op(yd, zd)
    tol = 1e-12 if dtype == np.float64 else 1e-5
    assert np.abs(zd.get() - yd.get()).max() <= tol * max(1.0, np.abs(y).max())
    assert op.nonconverged == 0
    pick = rng.choice(x.shape[1], 300, replace=False)
    for i in pick:
        for j in range(x.shape[0]):
            A, bb, _ = E.instance_constraints(I, J, v, b, j, i)
            yo, ok = E.project_polyhedron(x[j, i], A, bb, 2)
            assert ok
            assert np.abs(y[j, i] - yo).max() <= (1e-10 if dtype == np.float64 else 1e-5)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("samples", [5, 8, 12])
def test_sublabel_instances_both_constraint_paths(dtype, samples):
    """Sublabel-model instances with 5, 8 and 12 points per interval: up to 8
    constraints per instance are held in registers, more are read from
    memory at every scan; both against the oracle's projection."""
    from opymize_gb300 import DeviceArray
    from opymize_gb300.operators import EpigraphProj
    from opymize_gb300.tools import lifting
    rng = np.random.default_rng(samples)
    nfuns = 3000
    d = lifting.sublabel_data(rng.uniform(0, 1, nfuns), L=6, samples=samples, trunc=0.04)
    I, J, v, b = d["I"], d["J"], d["v"], d["b"]
    x = rng.normal(0, 0.5, (J.shape[0], nfuns, 2))
    op = EpigraphProj(I, J, v, b)
    yd = DeviceArray.zeros((x.size,), dtype)
    op(DeviceArray.to_gpu(x.ravel(), dtype), yd)
    y = yd.get().reshape(x.shape)
    assert op.nonconverged == 0
    for i in rng.choice(nfuns, 150, replace=False):
        for j in range(J.shape[0]):
            A, bb, _ = E.instance_constraints(I, J, v, b, j, i)
            yo, ok = E.project_polyhedron(x[j, i], A, bb)
            assert ok
            assert np.abs(y[j, i] - yo).max() <= (1e-10 if dtype == np.float64
                                                   else 2e-5 * max(1.0, np.abs(x).max()))
