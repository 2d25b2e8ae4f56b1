"""The semismooth Newton oracle (oracle/ssn.py) against the reference's own
solver (tests/golden/ssn.npz, written by tests/golden/make_ssn_golden.py):
Newton iterates after 1-3 steps from a PDHG start and from zero, and the
Jacobian of the Frobenius-ball projection."""

import os

import numpy as np
import pytest

from tests.conftest import GOLDEN


def load():
    return np.load(os.path.join(GOLDEN, "ssn.npz"))


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", ["gray", "zero", "gray2"])
def test_ssn_oracle_matches_reference(name):
    import oracle
    from oracle.ssn import SemismoothNewton
    d = load()
    f = d[name + "_f"]
    dims = f.shape[:2]
    A = oracle.Gradient(dims, 1, "centered")   # the reference default (examples/rof.py:73)
    for k in (1, 2, 3):
        s = SemismoothNewton(f, float(d[name + "_lbd"]), A, 2)
        xy = s.solve(d[name + "_start"], k)
        assert rel(xy, d["%s_xy%d" % (name, k)]) < 1e-9, (name, k)
        assert s.lam == pytest.approx(float(d["%s_lbd%d" % (name, k)]), rel=1e-12)
        assert s.tau == pytest.approx(float(d["%s_steps%d" % (name, k)][0]), rel=1e-12)


@pytest.mark.parametrize("name,C", [("jac1", 1), ("jac3", 3)])
def test_projection_jacobian_oracle(name, C):
    from oracle.ssn import FrobeniusProjJacobian, project_with_jacobian
    d = load()
    x = d[name + "_jac_x"].copy()
    N, M = x.shape
    J = FrobeniusProjJacobian(N, M)
    lbd = 0.1 if C == 1 else 0.08
    xp = x.ravel().copy()
    project_with_jacobian(xp, N, M, lbd, J)
    np.testing.assert_allclose(xp, d[name + "_jac_proj"], rtol=1e-14, atol=1e-16)
    np.testing.assert_allclose(J.apply(d[name + "_jac_v"]), d[name + "_jac_Jv"], rtol=1e-13, atol=1e-15)
