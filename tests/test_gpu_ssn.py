"""Semismooth Newton on the device (opymize_gb300.solvers.SemismoothNewton)
and the Jacobian of the Frobenius-ball projection (L12ProjJacobian) against
the reference's own CPU solver (tests/golden/ssn.npz, written by
tests/golden/make_ssn_golden.py) and the CPU oracle (oracle/ssn.py): Newton
iterates after 1-3 steps from a PDHG start and from zero, FP64."""

import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def load():
    return np.load(os.path.join(GOLDEN, "ssn.npz"))


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name,C,lbd", [("jac1", 1, 0.1), ("jac3", 3, 0.08)])
def test_projection_jacobian_matches_reference(name, C, lbd):
    from opymize_gb300.gpuarray import DeviceArray
    from opymize_gb300.operators.proj import L1NormsProj, L12ProjJacobian
    d = load()
    x = d[name + "_jac_x"]
    N = x.shape[0]
    proj = L1NormsProj(N, (C, 2), lbd, "frobenius")
    xd = DeviceArray.to_gpu(x.ravel(), np.float64)
    J = proj(xd, jacobian=True)
    assert isinstance(J, L12ProjJacobian) and J.adjoint is J
    np.testing.assert_allclose(xd.get(), d[name + "_jac_proj"], rtol=1e-14, atol=1e-16)
    vd = DeviceArray.to_gpu(d[name + "_jac_v"].ravel(), np.float64)
    out = DeviceArray.zeros((vd.size,), np.float64)
    J(vd, out)
    np.testing.assert_allclose(out.get(), d[name + "_jac_Jv"], rtol=1e-13, atol=1e-15)
    # add= accumulates; a plain projection leaves the Jacobian's state alone
    J(vd, out, add=True)
    np.testing.assert_allclose(out.get(), 2 * d[name + "_jac_Jv"], rtol=1e-13, atol=1e-15)
    proj(DeviceArray.to_gpu(np.zeros(x.size), np.float64))
    out2 = DeviceArray.zeros((vd.size,), np.float64)
    J(vd, out2)
    np.testing.assert_allclose(out2.get(), d[name + "_jac_Jv"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("name", ["gray", "zero", "gray2"])
def test_ssn_matches_reference_and_oracle(name):
    import oracle
    from oracle.ssn import SemismoothNewton as OracleSSN
    from opymize_gb300.functionals import SSD, L1Norms
    from opymize_gb300.linear import GradientOp
    from opymize_gb300.solvers import SemismoothNewton
    d = load()
    f = d[name + "_f"]
    dims = f.shape[:2]
    N = int(np.prod(dims))
    lbd = float(d[name + "_lbd"])
    for k in (1, 2, 3):
        np.random.seed(1)
        s = SemismoothNewton(SSD(f.reshape(N, 1)), L1Norms(N, (1, 2), lbd), GradientOp(dims, 1))
        info = s.solve(continue_at=d[name + "_start"].copy(), granularity=1, term_relgap=1e-300,
                       term_maxiter=k)
        xy = np.concatenate([v.ravel() for v in s.state])
        ref = d["%s_xy%d" % (name, k)]
        assert rel(xy, ref) < 1e-8, (name, k, rel(xy, ref))
        assert s.lbd == pytest.approx(float(d["%s_lbd%d" % (name, k)]), rel=1e-12)
        ri = d["%s_info%d" % (name, k)]
        for j, key in enumerate(("objp", "objd")):
            assert info[key] == pytest.approx(ri[j], rel=1e-9, abs=1e-12)
        assert abs(info["relgap"] - ri[4]) <= 1e-7 * max(1.0, abs(ri[4]))
        o = OracleSSN(f, lbd, oracle.Gradient(dims, 1, "centered"), 2)
        assert rel(xy, o.solve(d[name + "_start"], k)) < 1e-8


def test_ssn_reaches_a_tight_gap_from_pdhg():
    """From a PDHG start the Newton iterations keep the relative gap at or
    below the PDHG level and end with every iterate finite (a small 2-D
    case, the reference example's use, examples/rof.py:79-85)."""
    from opymize_gb300.functionals import SSD, L1Norms
    from opymize_gb300.linear import GradientOp
    from opymize_gb300.solvers import PDHG, SemismoothNewton
    from opymize_gb300.tools.synthetic import piecewise_constant
    dims = (48, 40)
    N = int(np.prod(dims))
    f = piecewise_constant(dims, 1, sigma=0.1, seed=3).reshape(N, 1)
    p = PDHG(SSD(f), L1Norms(N, (1, 2), 0.1), GradientOp(dims, 1))
    p.solve(steps="precond", precision="double", term_pd_gap=1e-300, term_maxiter=500,
            granularity=500)
    s = SemismoothNewton(SSD(f), L1Norms(N, (1, 2), 0.1), GradientOp(dims, 1))
    np.random.seed(0)
    info = s.solve(continue_at=p.state, granularity=5, term_relgap=1e-300, term_maxiter=5)
    assert all(np.isfinite(v).all() for v in s.state)
    assert abs(info["relgap"]) <= 1.01 * abs(p.info["relgap"]) + 1e-12


def test_ssn_ten_steps_follow_the_oracle():
    """Ten Newton steps from a PDHG start (48 x 40 gray, lambda 0.1), device
    against the oracle's restatement of the reference's solver, and the
    progress both make.  The reference's method barely moves from a PDHG
    point: its CG stops once |r|^2 falls below the current residual
    0.5 |R|^2 (semismooth_newton.py:77-117), so its steps are inexact, and
    0.5 |R|^2 drops by well under 5 % in 10 steps (the oracle shows the same
    over 40 steps).  The device solver matches that trajectory rather than
    improving on it."""
    import oracle
    from oracle.ssn import SemismoothNewton as OracleSSN
    from opymize_gb300.functionals import SSD, L1Norms
    from opymize_gb300.linear import GradientOp
    from opymize_gb300.solvers import PDHG, SemismoothNewton
    from opymize_gb300.tools.synthetic import piecewise_constant
    dims = (48, 40)
    N = int(np.prod(dims))
    f = piecewise_constant(dims, 1, sigma=0.1, seed=3).reshape(N, 1)
    p = PDHG(SSD(f), L1Norms(N, (1, 2), 0.1), GradientOp(dims, 1))
    p.solve(steps="precond", precision="double", term_pd_gap=1e-300, term_maxiter=500,
            granularity=500)
    start = np.concatenate([v.ravel() for v in p.state])
    np.random.seed(1)
    s = SemismoothNewton(SSD(f), L1Norms(N, (1, 2), 0.1), GradientOp(dims, 1))
    s.solve(continue_at=start.copy(), granularity=10, term_relgap=1e-300, term_maxiter=10)
    xy = np.concatenate([v.ravel() for v in s.state])
    o = OracleSSN(f, 0.1, oracle.Gradient(dims, 1, "centered"), 2)
    ref = o.solve(start, 10)
    assert rel(xy, ref) < 1e-6, rel(xy, ref)
    res = np.zeros_like(start)
    r0, r10 = o._res(start, res), o._res(xy, res)
    assert r10 < r0                       # it descends ...
    assert r10 > 0.95 * r0                # ... by little, as the reference does
