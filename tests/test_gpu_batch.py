"""Batched solves (BatchROF, opyx_rof_batch_*): every image of a batch must
follow its own single-image fused solve -- the same single-sweep arithmetic
per pixel, so identical iterates after the same iteration count -- and be
retired at its own stop test."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(64, 64), (100, 132), (200, 516), (37, 1028), (300, 256), (8, 4)]


def images(C, seed=0):
    from opymize_gb300.tools.synthetic import piecewise_constant
    return [piecewise_constant(s, C, sigma=0.1, seed=seed + k) for k, s in enumerate(SHAPES)]


def single(img, lbd, huber, tol, maxiter, gran):
    from opymize_gb300.functionals import SSD, L1Norms, HuberL1Norms
    from opymize_gb300.linear import GradientOp
    from opymize_gb300.solvers import PDHG
    H, W, C = img.shape
    N = H * W
    F = HuberL1Norms(N, (C, 2), lbd, huber) if huber > 0 else L1Norms(N, (C, 2), lbd)
    s = PDHG(SSD(img.reshape(N, C)), F, GradientOp((H, W), C, scheme="forward"))
    s.solve(steps="precond", precision="float", term_pd_gap=tol, term_maxiter=maxiter,
            granularity=gran)
    return s


@pytest.mark.parametrize("C,huber", [(1, 0.0), (3, 0.02)])
def test_fixed_iterations_match_single_solves(C, huber):
    from opymize_gb300.solvers import BatchROF
    imgs = images(C)
    lbds = [0.05, 0.1, 0.2, 0.08, 0.3, 0.1]
    b = BatchROF(imgs, lbds, huber=huber, tol=1e-300, granularity=10, rows_per_item=16)
    info = b.solve(maxiter=20)
    for i, img in enumerate(imgs):
        s = single(img, lbds[i], huber, 1e-300, 20, 10)
        assert info[i]["iter"] == 20
        x = b.state(i).ravel()
        assert np.array_equal(x, s.state[0].ravel().astype(np.float32)), i
        assert info[i]["relgap"] == pytest.approx(s.info["relgap"], rel=1e-5, abs=1e-7)


def test_images_retire_at_their_own_stop_test():
    from opymize_gb300.solvers import BatchROF
    imgs = images(1, seed=7)
    lbds = [0.02, 0.3, 0.1, 0.05, 0.2, 0.1]
    b = BatchROF(imgs, lbds, tol=1e-3, granularity=6)
    info = b.solve(maxiter=4000)
    assert b.rows_per_item in BatchROF.ROWS_CANDIDATES
    for i, img in enumerate(imgs):
        assert info[i]["converged"]
        s = single(img, lbds[i], 0.0, 1e-3, 4000, 6)
        if info[i]["iter"] != s.info["iter"]:
            # a stop decision on a near-tie of the two gap summations
            assert abs(abs(s.info["relgap"]) - 1e-3) < 1e-6
        else:
            assert np.array_equal(b.state(i).ravel(), s.state[0].ravel().astype(np.float32))
        assert abs(info[i]["relgap"]) < 1e-3


def test_batch_rejects_unsupported_images():
    from opymize_gb300.solvers import BatchROF
    with pytest.raises(ValueError):
        BatchROF([np.zeros((8, 6))], 0.1)              # last axis not a multiple of 4
    with pytest.raises(ValueError):
        BatchROF([np.zeros((8, 8)), np.zeros((8, 8, 3))], 0.1)   # mixed channels


def test_persistent_and_graph_paths_agree():
    """One-channel batches run as one persistent launch by default; the
    captured-graph path of per-iteration launches gives the same bits, the
    same stop iterations and the same gaps."""
    from opymize_gb300.solvers import BatchROF
    imgs = images(1, seed=3)
    lbds = [0.05, 0.1, 0.2, 0.08, 0.3, 0.1]
    out = []
    for persistent in (True, False):
        b = BatchROF(imgs, lbds, tol=2e-3, granularity=8, rows_per_item=16,
                     persistent=persistent)
        assert b.persistent == persistent
        info = b.solve(maxiter=600)
        out.append((b, info))
    (bp, ip), (bg, ig) = out
    assert bp.launches <= 4
    for i in range(len(imgs)):
        assert ip[i]["iter"] == ig[i]["iter"] and ip[i]["converged"] == ig[i]["converged"]
        assert np.array_equal(bp.state(i), bg.state(i)), i
        assert np.array_equal(bp.dual(i), bg.dual(i)), i
        assert ip[i]["relgap"] == pytest.approx(ig[i]["relgap"], rel=1e-6, abs=1e-9)


def test_persistent_batch_matches_oracle():
    """Four mixed-size one-channel instances (a narrow strip, a ragged tile,
    a multi-strip image, a tall one), 40 preconditioned iterations in the
    persistent launch, against the FP64 oracle of the reference's CPU solver
    (opymize/solvers/pdhg.py:229-315): relative L2 error of x and y <= 1e-5,
    the gap to 1e-6."""
    import oracle
    from opymize_gb300.solvers import BatchROF
    from opymize_gb300.tools.synthetic import piecewise_constant
    shapes = [(48, 20), (70, 132), (33, 300), (257, 64)]
    lbds = [0.07, 0.15, 0.05, 0.2]
    imgs = [piecewise_constant(s, 1, sigma=0.1, seed=40 + k) for k, s in enumerate(shapes)]
    b = BatchROF(imgs, lbds, tol=1e-300, granularity=10, rows_per_item=8, persistent=True)
    info = b.solve(maxiter=40)
    for i, (img, lbd) in enumerate(zip(imgs, lbds)):
        H, W = shapes[i]
        N = H * W
        so = oracle.PDHG(oracle.SSD(img.reshape(N, 1)), oracle.L1Norms(N, (1, 2), lbd),
                         oracle.Gradient((H, W), 1, "forward"))
        so.solve(steps="precond", term_pd_gap=1e-300, term_maxiter=40, granularity=10)
        x, y = so.state
        ex = np.linalg.norm(b.state(i).ravel() - x) / np.linalg.norm(x)
        ey = np.linalg.norm(b.dual(i).ravel() - y) / np.linalg.norm(y)
        assert ex <= 1e-5 and ey <= 1e-5, (i, ex, ey)
        assert info[i]["iter"] == 40
        assert abs(info[i]["relgap"] - so.info["relgap"]) <= 1e-6, i


def test_persistent_batch_maxiter_and_retirement():
    """Instances that reach the tolerance retire at their own check; the
    others stop at maxiter with converged False; the control record counts
    the instances still active at the last check."""
    from opymize_gb300.solvers import BatchROF
    imgs = images(1, seed=11)
    lbds = [0.02, 0.3, 0.1, 0.05, 0.2, 0.1]
    b = BatchROF(imgs, lbds, tol=5e-4, granularity=10, rows_per_item=32, persistent=True)
    info = b.solve(maxiter=300)
    for d in info:
        if d["converged"]:
            assert d["iter"] <= 300 and d["iter"] % 10 == 0 and abs(d["relgap"]) < 5e-4
        else:
            assert d["iter"] == 300 and abs(d["relgap"]) >= 5e-4
    assert b.persist_ctl["active"] == sum(not d["converged"] for d in info)
