"""The sublabel lifting workload on the GPU -- the generic PDHG path (BlockOp /
SplitSum of IdentityOp, IndexedMultAdj, MatrixMultR, ScaleOp, GradientOp,
PositivityFct, IndicatorFct, L1Norms, EpigraphSupp) and the two fused passes
that replace its iteration for this model (fused=None) -- against the
reference's own PDHG run of the same model (tests/golden/sublabel_*.npz).
Bars: FP64 relative L2 <= 1e-10 of x and y after each dumped iteration
(measured ~1e-14); FP32 <= 1e-5 (measured <= 4e-6 after 200 iterations)."""

import numpy as np
import pytest

from tests.test_sublabel import CASES, load, fixture_faces

pytestmark = pytest.mark.gpu


def gpu_solver(z, faces=True):
    from opymize_gb300.solvers import PDHG
    from opymize_gb300.tools import lifting
    img = z["img"]
    g, f, A, d = lifting.sublabel_problem(img, L=int(z["L"]), lbd=float(z["lbd"]),
                                          samples=int(z["samples"]), trunc=float(z["trunc"]),
                                          with_faces=False)
    if faces:
        supp = f.fcts[-1]
        supp.If = fixture_faces(z, int(z["L"]), img.size)
    return PDHG(g, f, A)


def run(z, precision, faces=True, fused=None):
    s = gpu_solver(z, faces)
    rec = {}

    def cb(state, info):
        rec[info["iter"]] = (state[0].copy(), state[1].copy(), dict(info))

    np.random.seed(0)
    s.solve(steps=str(z["steps"]), precision=precision, term_pd_gap=1e-300,
            term_maxiter=int(z["iters"]), granularity=int(z["gran"]), cbfun=cb, fused=fused)
    # adaptive steps stay on the generic path; precond runs the fused passes
    want = "sublabel" if fused is not False and str(z["steps"]) != "adaptive" else "generic"
    assert s.path == want, (s.path, want)
    return s, rec


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / max(1e-300, np.linalg.norm(b))


@pytest.mark.parametrize("fused", [None, False])
@pytest.mark.parametrize("name", CASES)
def test_fp64_matches_reference(name, fused):
    z = load(name)
    s, rec = run(z, "double", fused=fused)
    for k, it in enumerate(z["dump_iters"]):
        x, y, info = rec[int(it)]
        assert rel(x, z["x"][k]) <= 1e-10, (name, it, rel(x, z["x"][k]))
        assert rel(y, z["y"][k]) <= 1e-10, (name, it, rel(y, z["y"][k]))
        ref = z["info"][k]
        assert info["objp"] == pytest.approx(ref[1], rel=1e-9, abs=1e-9)
        assert info["objd"] == pytest.approx(ref[2], rel=1e-9, abs=1e-9)
        assert info["infeasp"] == pytest.approx(ref[4], rel=1e-6, abs=1e-9)
        assert info["infeasd"] == pytest.approx(ref[5], rel=1e-6, abs=1e-9)
    assert s.f.fcts[-1].conj.prox(1.0).nonconverged == 0


@pytest.mark.parametrize("fused", [None, False])
@pytest.mark.parametrize("name", CASES)
def test_fp32_matches_reference(name, fused):
    z = load(name)
    _, rec = run(z, "float", fused=fused)
    for k, it in enumerate(z["dump_iters"]):
        x, y, _ = rec[int(it)]
        assert rel(x, z["x"][k]) <= 1e-5 and rel(y, z["y"][k]) <= 1e-5, (name, it)


def test_envelope_gap_equals_faces_gap():
    z = load(CASES[0])
    _, ra = run(z, "double", faces=True)
    _, rb = run(z, "double", faces=False)
    for it in ra:
        assert ra[it][2]["objp"] == pytest.approx(rb[it][2]["objp"], rel=1e-12, abs=1e-12)


def test_full_size_iterates():
    """512 x 512, 16 labels, FP32: the workload's shape runs, the QP always
    converges, and the state stays finite and feasible in its cones."""
    from opymize_gb300.solvers import PDHG
    from opymize_gb300.tools import lifting
    from opymize_gb300.tools.synthetic import piecewise_constant
    img = np.clip(piecewise_constant((512, 512), 1, sigma=0.05, seed=1,
                                     salt_pepper=0.1)[..., 0], 0, 1)
    g, f, A, d = lifting.sublabel_problem(img, L=16, lbd=0.1, samples=8)
    s = PDHG(g, f, A)
    s.solve(steps="precond", precision="float", term_pd_gap=1e-300, term_maxiter=100,
            granularity=50)
    x, y = s.state
    assert np.isfinite(x).all() and np.isfinite(y).all()
    assert f.fcts[-1].conj.prox(1.0).nonconverged == 0
    assert np.isfinite(s.info["objp"]) and np.isfinite(s.info["objd"])
    u = x[:512 * 512 * 16].reshape(-1, 16)
    assert u.min() >= 0


def test_full_size_fused_matches_generic():
    """512 x 512, 16 labels (the sublabel configuration): the fused passes
    against the generic operator chain after 100 preconditioned iterations,
    FP32 (relative L2 <= 1e-5 of x and y, the same gap to 1e-6) and FP64
    (<= 1e-10) -- the generic path itself is pinned to the reference on the
    fixtures above."""
    from opymize_gb300.solvers import PDHG
    from opymize_gb300.tools import lifting
    from opymize_gb300.tools.synthetic import piecewise_constant
    img = np.clip(piecewise_constant((512, 512), 1, sigma=0.05, seed=1,
                                     salt_pepper=0.1)[..., 0], 0, 1)
    for precision, bar, iters in (("float", 1e-5, 100), ("double", 1e-10, 40)):
        out = []
        for fused in (None, False):
            g, f, A, d = lifting.sublabel_problem(img, L=16, lbd=0.1, samples=8)
            s = PDHG(g, f, A)
            s.solve(steps="precond", precision=precision, term_pd_gap=1e-300,
                    term_maxiter=iters, granularity=iters, fused=fused)
            assert s.path == ("sublabel" if fused is None else "generic")
            out.append((s.state, s.info))
        (xs, ys), ia = out[0]
        (xg, yg), ib = out[1]
        assert rel(xs, xg) <= bar and rel(ys, yg) <= bar, (precision, rel(xs, xg), rel(ys, yg))
        assert abs(ia["relgap"] - ib["relgap"]) <= 1e-6 * max(1.0, abs(ib["relgap"]))
