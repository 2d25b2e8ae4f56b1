"""Generate the golden fixtures in this folder from the reference itself.

Run in a container where the reference package is mounted (default path
``/root/reference``; override with ``OPYMIZE_REF``)::

    python tests/golden/make_golden.py

It imports the reference's pure-Python CPU path (``use_gpu=False``) with an
identity ``numba.jit`` stand-in (``numba`` is only used as a decorator on
``spectral_projection_2d``, opymize/operators/proj.py:114, and as an unused
import in opymize/linear/indexed.py:5), runs operators, functionals and the
PDHG solver on seeded inputs, and writes ``.npz`` files that the tests compare
against.  Nothing in the test suite reads the reference at run time; only
these fixtures travel.

The colour workload's Huber-smoothed total variation has no functional in
the reference, so ``RefHuberL1Norms`` / ``RefHuberL1NormsConj`` below define
it on top of the reference's own ``Functional`` base class and run inside the
reference's own ``PDHG``.
"""

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
sys.path.insert(0, REF)
sys.path.insert(0, REPO)

from opymize import Functional, Variable                       # noqa: E402
from opymize.solvers import PDHG                                # noqa: E402
from opymize.functionals import (SSD, L1Norms, L1NormsConj,      # noqa: E402
                                 QuadEpiInd, QuadEpiSupp,
                                 HuberPerspective, TruncQuadEpiInd)
from opymize.linear import normest                              # noqa: E402
from opymize.linear.diff import GradientOp, LaplacianOp         # noqa: E402
from opymize.linear.einsum import (MatrixMult, MatrixMultR,     # noqa: E402
                                   MatrixMultRBatched, TangledMatrixMultR,
                                   DiagMatrixMultR)
from opymize.linear.indexed import IndexedMult, IndexedMultAdj  # noqa: E402
from opymize.operators.proj import L1NormsProj, QuadEpiProj     # noqa: E402
from opymize.operators.proj import norm_projection              # noqa: E402
from opymize.tools import truncate, solve_reduced_monic_cubic   # noqa: E402

from opymize_gb300.tools.synthetic import piecewise_constant    # noqa: E402
import opymize.linear.sparse as _ref_sparse                     # noqa: E402


def fresh_einsum_dims():
    """The reference's ``einsumop`` takes ``dims={}`` as a mutable default
    and updates it in place (opymize/linear/sparse.py:303, :336-340), so letter
    sizes leak from one call to the next within a process.  Every operator
    built here starts from an empty dict, as a fresh process would."""
    _ref_sparse.einsumop.__defaults__[-1].clear()


# ---------------------------------------------------------------------------
# Huber-smoothed L1 norms, written against the reference's Functional API
# ---------------------------------------------------------------------------

class _RefHuberProj(object):
    """y <- proj_{|.|_F <= lbd}(y / (1 + sigma*alph/lbd)), per group."""

    def __init__(self, N, M, lbd, alph, sigma):
        self.N, self.M, self.lbd, self.alph = N, M, lbd, alph
        self.sigma = sigma
        self.x = Variable((N,) + M)
        self.y = self.x
        self._xnorms = np.zeros((N,))

    def __call__(self, x, y=None, add=False, jacobian=False):
        assert not add and not jacobian
        if y is None:
            y = x
        else:
            y[:] = x
        y /= (1.0 + self.sigma * self.alph / self.lbd)
        yv = self.y.vars(y)[0]
        norm_projection(yv, self._xnorms, self.lbd, matrixnorm="frobenius")


class RefHuberL1Norms(Functional):
    """F(x) = lbd * sum_i h_alph(|x_i|_F), h(r) = r^2/(2 alph) if r <= alph
    else r - alph/2."""

    def __init__(self, N, M, lbd, alph, conj=None):
        Functional.__init__(self)
        self.x = Variable((N,) + M)
        self.lbd, self.alph = lbd, alph
        self.conj = RefHuberL1NormsConj(N, M, lbd, alph, conj=self) \
            if conj is None else conj

    def __call__(self, x, grad=False):
        x = self.x.vars(x)[0]
        r = np.sqrt(np.einsum('ilm,ilm->i', x, x))
        h = np.where(r <= self.alph, 0.5 * r**2 / self.alph, r - 0.5 * self.alph)
        return (self.lbd * h.sum(), 0)


class RefHuberL1NormsConj(Functional):
    """F*(y) = sum_i alph/(2 lbd) |y_i|^2 + delta_{|y_i|_F <= lbd}."""

    def __init__(self, N, M, lbd, alph, conj=None):
        Functional.__init__(self)
        self.x = Variable((N,) + M)
        self.N, self.M, self.lbd, self.alph = N, M, lbd, alph
        self.conj = RefHuberL1Norms(N, M, lbd, alph, conj=self) \
            if conj is None else conj

    def __call__(self, x, grad=False):
        x = self.x.vars(x)[0]
        r2 = np.einsum('ilm,ilm->i', x, x)
        val = 0.5 * self.alph / self.lbd * r2.sum()
        infeas = np.linalg.norm(np.fmax(0, np.sqrt(r2) - self.lbd), ord=np.inf)
        return (val, infeas)

    def prox(self, tau):
        return _RefHuberProj(self.N, self.M, self.lbd, self.alph, tau)


# ---------------------------------------------------------------------------
# solver fixtures
# ---------------------------------------------------------------------------

INFO_KEYS = ["objp", "objd", "infeasp", "infeasd", "gap", "relgap"]


def run_solver(name, f, imagedims, lbd, steps, iters, gran=50, scheme="forward",
               imageh=None, weights=None, vol=None, mask=None, huber=None,
               seed=0, dump_all=True, dumps=None, step_bound=None):
    fresh_einsum_dims()
    C = f.shape[-1]
    D = len(imagedims)
    N = int(np.prod(imagedims))
    G = SSD(f.reshape(N, C), vol=vol, mask=mask)
    if huber is None:
        F = L1Norms(N, (C, D), lbd=lbd)
    else:
        F = RefHuberL1Norms(N, (C, D), lbd=lbd, alph=huber)
    A = GradientOp(imagedims, C, scheme=scheme, imageh=imageh, weights=weights)
    solver = PDHG(G, F, A)
    rec = {"iters": [], "tau": [], "sigma": []}
    for k in INFO_KEYS:
        rec[k] = []
    xs, ys = [], []

    def cb(state, info):
        it = info["iter"]
        rec["iters"].append(it)
        for k in INFO_KEYS:
            rec[k].append(float(info[k]))
        i = solver.itervars
        rec["tau"].append(float(i.get("tauk", np.nan)))
        rec["sigma"].append(float(i.get("sigmak", np.nan)))
        if dump_all or (dumps is not None and it in dumps):
            xs.append((it, state[0].copy()))
            ys.append((it, state[1].copy()))

    np.random.seed(seed)
    solver.solve(steps=steps, precision="double", use_gpu=False,
                 term_pd_gap=1e-300, term_maxiter=iters, granularity=gran,
                 cbfun=cb, step_bound=step_bound)
    c = solver.constvars
    out = {
        "f": f, "imagedims": np.array(imagedims), "lbd": lbd,
        "steps": steps, "scheme": scheme, "iters_total": iters, "gran": gran,
        "imageh": np.ones(D) if imageh is None else np.asarray(imageh),
        "weights": np.ones(C) if weights is None else np.asarray(weights),
        "vol": np.ones(C) if vol is None else np.asarray(vol),
        "mask": np.ones(N, dtype=bool) if mask is None else np.asarray(mask),
        "huber": -1.0 if huber is None else huber,
        "const_tau": float(c.get("tau", np.nan)),
        "const_sigma": float(c.get("sigma", np.nan)),
        "dump_iters": np.array([it for it, _ in xs], dtype=np.int64),
        "x": np.array([v for _, v in xs]), "y": np.array([v for _, v in ys]),
    }
    for k, v in rec.items():
        out["info_" + k] = np.array(v)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path) // 1024, "KiB")


def solver_fixtures():
    # 256x256 gray ROF, adaptive, 1000 iterations, gap every 50 iterations
    f = piecewise_constant((256, 256), 1, sigma=0.1, seed=0)
    run_solver("rof_gray256_adaptive", f, (256, 256), 0.1, "adaptive", 1000,
               dump_all=False, dumps=(1000,))

    g = piecewise_constant((32, 24), 1, sigma=0.1, seed=1)
    run_solver("g2d_const_fwd", g, (32, 24), 0.1, "const", 200)
    run_solver("g2d_adaptive_fwd", g, (32, 24), 0.1, "adaptive", 200)
    run_solver("g2d_precond_fwd", g, (32, 24), 0.1, "precond", 200)
    run_solver("g2d_adaptive_centered", g, (32, 24), 0.1, "adaptive", 200,
               scheme="centered")
    run_solver("g2d_const_imageh", g, (32, 24), 0.1, "const", 200,
               imageh=np.array([0.5, 0.7]), weights=np.array([2.0]))
    run_solver("g1d_precond_fwd", g.reshape(-1, 1)[:97], (97,), 0.2,
               "precond", 200)

    c = piecewise_constant((24, 20), 3, sigma=0.1, seed=2)
    run_solver("c2d_precond_fwd", c, (24, 20), 0.05, "precond", 200)
    run_solver("c2d_huber_precond", c, (24, 20), 0.05, "precond", 200,
               huber=0.05)
    run_solver("c2d_huber_adaptive", c, (24, 20), 0.05, "adaptive", 200,
               huber=0.01)
    msk = np.random.default_rng(3).random(24 * 20) < 0.8
    run_solver("c2d_volmask_const", c, (24, 20), 0.05, "const", 200,
               vol=np.array([1.0, 2.0, 0.5]), mask=msk,
               imageh=np.array([1.0, 0.8]))

    v = piecewise_constant((10, 9, 8), 1, sigma=0.1, seed=4)
    run_solver("v3d_precond_fwd", v, (10, 9, 8), 0.08, "precond", 200)
    run_solver("v3d_adaptive_fwd", v, (10, 9, 8), 0.08, "adaptive", 200)


# ---------------------------------------------------------------------------
# operator and functional fixtures
# ---------------------------------------------------------------------------

def op_fixtures():
    rng = np.random.default_rng(1234)
    out = {}

    def linop_case(key, mk):
        fresh_einsum_dims()
        op = mk()
        x = rng.standard_normal(op.x.size)
        y = rng.standard_normal(op.y.size)
        Ax = np.zeros(op.y.size)
        ATy = np.zeros(op.x.size)
        op(x, Ax)
        op.adjoint(y, ATy)
        out[key + "/x"], out[key + "/y"] = x, y
        out[key + "/Ax"], out[key + "/ATy"] = Ax, ATy
        for p in (1, 2):
            r = np.zeros(op.y.size)
            op.rowwise_lp(r, p=p)
            out[key + "/rowlp%d" % p] = r
            try:
                r = np.zeros(op.x.size)
                op.adjoint.rowwise_lp(r, p=p)
                out[key + "/collp%d" % p] = r
            except Exception:
                pass

    # finite differences.  For D >= 3 the reference's CPU matrix of the
    # centered scheme (avgopn, opymize/linear/sparse.py:223-250) sums the
    # per-axis averages instead of composing them (a unit slope gives 1.5),
    # while its GPU kernel averages 2^(D-1) differences (diff.cu:53-63); the
    # centered cases here stop at D = 2, where both agree.
    cases = [
        ("grad_fwd_2d_c1", (4, 5), 1, "forward", None, None),
        ("grad_cen_2d_c1", (4, 5), 1, "centered", None, None),
        ("grad_fwd_2d_c3", (7, 6), 3, "forward", [0.3, 0.4], [1.0, 2.0, 0.5]),
        ("grad_cen_2d_c3", (7, 6), 3, "centered", [0.3, 0.4], [1.0, 2.0, 0.5]),
        ("grad_fwd_3d_c2", (5, 4, 3), 2, "forward", [1.0, 0.5, 2.0], None),
        ("grad_fwd_1d_c1", (9,), 1, "forward", None, None),
        ("grad_cen_1d_c2", (9,), 2, "centered", None, None),
        ("grad_fwd_4d_c1", (3, 4, 2, 5), 1, "forward", None, None),
    ]
    for key, dims, C, scheme, h, w in cases:
        linop_case(key, lambda: GradientOp(
            dims, C, scheme=scheme,
            imageh=None if h is None else np.array(h),
            weights=None if w is None else np.array(w)))
        out[key + "/dims"] = np.array(dims)
        out[key + "/C"] = C
        out[key + "/h"] = np.ones(len(dims)) if h is None else np.array(h)
        out[key + "/w"] = np.ones(C) if w is None else np.array(w)

    for bc in ["neumann", "curvature", "second-order"]:
        for dims, C, h in [((7, 6), 2, [0.3, 0.4]), ((5, 4, 3), 1, [1.0, 0.5, 2.0])]:
            key = "lapl_%s_%dd" % (bc, len(dims))
            linop_case(key, lambda: LaplacianOp(dims, C, imageh=np.array(h),
                                                boundary=bc))
            out[key + "/dims"] = np.array(dims)
            out[key + "/C"] = C
            out[key + "/h"] = np.array(h)

    # einsum-type operators
    N = 37
    # MatrixMult builds x as (A.shape[0], N) but contracts over A.shape[1]
    # (opymize/linear/einsum.py:23-30), so the reference only constructs it
    # for square A
    Asq = rng.standard_normal((5, 5))
    A = rng.standard_normal((4, 6))
    for trans in (False, True):
        k = "mm_%s" % ("t" if trans else "n")
        linop_case(k, lambda: MatrixMult(N, Asq, trans=trans))
        out[k + "/A"] = Asq
        k = "mmr_%s" % ("t" if trans else "n")
        linop_case(k, lambda: MatrixMultR(N, A, trans=trans))
        out[k + "/A"] = A
    A3 = rng.standard_normal((5, 3, 4))
    for trans in (False, True):
        k = "mmrb_%s" % ("t" if trans else "n")
        linop_case(k, lambda: MatrixMultRBatched(N, A3, trans=trans))
        out[k + "/A"] = A3
    A4 = rng.standard_normal((3, 2, 4, 5))
    for trans in (False, True):
        k = "tmmr_%s" % ("t" if trans else "n")
        linop_case(k, lambda: TangledMatrixMultR(N, A4, trans=trans))
        out[k + "/A"] = A4
    dA = rng.standard_normal(6)
    linop_case("dmmr", lambda: DiagMatrixMultR(N, dA))
    out["dmmr/A"] = dA

    # indexed operators
    K, J, M, L = 7, 5, 3, 4
    B = rng.standard_normal((J, M, L))
    P = rng.integers(0, K, size=(J, L))
    linop_case("idx", lambda: IndexedMult(K, N, B, P))
    out["idx/B"], out["idx/P"], out["idx/K"] = B, P, K

    # projections
    for Mshape, norm in [((1, 2), "frobenius"), ((3, 2), "frobenius"),
                         ((2, 3), "spectral"), ((3, 2), "spectral"),
                         ((2, 2), "spectral"), ((1, 3), "spectral")]:
        Np = 50
        op = L1NormsProj(Np, Mshape, 0.7, norm)
        x = 0.6 * rng.standard_normal(op.x.size)
        if Mshape == (2, 2):
            x.reshape(Np, 2, 2)[:5, 0, 1] = 0.0  # C12 == 0 branch
            x.reshape(Np, 2, 2)[:5, 1, 0] = 0.0
        y = x.copy()
        op(y)
        key = "l1proj_%s_%dx%d" % (norm, Mshape[0], Mshape[1])
        out[key + "/x"], out[key + "/y"], out[key + "/lbd"] = x, y, 0.7

    for variant in ["abc", "shift", "trunc", "plain"]:
        Nq, Mq = 40, 2
        alph = 0.3 + 5 * rng.random()
        kw = {}
        if variant == "abc":
            kw = dict(b=rng.uniform(-5, 5, (Nq, Mq)), c=rng.uniform(-5, 5, Nq))
        elif variant == "shift":
            kw = dict(shift=rng.uniform(-5, 5, (Nq, Mq + 1)))
        elif variant == "trunc":
            kw = dict(lbd=0.2 + 3 * rng.random())
        op = QuadEpiProj(Nq, Mq, alph=alph, **kw)
        x = 4 * rng.standard_normal((Nq, Mq + 1))
        x[:3, :-1] = 0.0
        x = x.ravel()
        y = x.copy()
        op(y)
        key = "quadepi_%s" % variant
        out[key + "/x"], out[key + "/y"], out[key + "/alph"] = x, y, alph
        out[key + "/shift"] = np.zeros(0) if op.shift is None else op.shift
        out[key + "/lbd"] = op.lbd

    # cubic solver and truncate
    a = rng.uniform(-5, 5, 200)
    b = rng.uniform(-5, 5, 200)
    a[:5] = 0.0
    out["cubic/a"], out["cubic/b"] = a, b
    out["cubic/x"] = solve_reduced_monic_cubic(a, b)
    vals = np.concatenate([rng.uniform(1e-4, 1e3, 50),
                           [0.126, 0.125, 1 / 7.99, 123.456, 0.0061425]])
    out["truncate/x"] = vals
    out["truncate/y"] = np.array([truncate(v, 3) for v in vals])

    # functional values
    Nf, C = 30, 3
    fdat = rng.standard_normal((Nf, C))
    vol = np.array([1.0, 2.0, 0.5])
    msk = rng.random(Nf) < 0.7
    G = SSD(fdat, vol=vol, mask=msk)
    xx = rng.standard_normal(Nf * C)
    out["ssd/f"], out["ssd/vol"], out["ssd/mask"], out["ssd/x"] = fdat, vol, msk, xx
    out["ssd/val"] = G(xx)[0]
    out["ssd/conjval"] = G.conj(xx)[0]
    tau = rng.uniform(0.1, 2.0, Nf * C)
    px = xx.copy()
    G.prox(tau)(px)
    out["ssd/tau"], out["ssd/prox"] = tau, px

    F = L1Norms(Nf, (C, 2), lbd=0.3)
    yy = 0.3 * rng.standard_normal(Nf * C * 2)
    out["l1/x"] = yy
    out["l1/val"], out["l1/infeas"] = F(yy)
    out["l1conj/val"], out["l1conj/infeas"] = F.conj(yy)
    Fn = L1Norms(Nf, (2, 3), lbd=0.3, matrixnorm="nuclear")
    out["l1nuc/val"] = Fn(yy)[0]
    out["l1spec/infeas"] = Fn.conj(yy)[1]

    Hb = HuberPerspective(Nf, 2, lbd=0.7, alph=0.4)
    hx = rng.standard_normal((Nf, 3))
    hx[:, -1] = -np.abs(hx[:, -1]) - 0.1
    out["huberpersp/x"] = hx.ravel()
    out["huberpersp/val"], out["huberpersp/infeas"] = Hb(hx.ravel())
    out["truncquad/val"], out["truncquad/infeas"] = Hb.conj(hx.ravel())
    Qi = QuadEpiInd(Nf, 2, a=1.5, b=rng.standard_normal((Nf, 2)),
                    c=rng.standard_normal(Nf))
    out["quadepi_ind/b"], out["quadepi_ind/c"] = Qi.b, Qi.c
    out["quadepi_ind/val"], out["quadepi_ind/infeas"] = Qi(hx.ravel())
    out["quadepi_supp/val"], out["quadepi_supp/infeas"] = Qi.conj(hx.ravel())

    # power iteration (seeded)
    fresh_einsum_dims()
    op = GradientOp((12, 9), 2, scheme="forward")
    np.random.seed(5)
    e, itn = normest(op)
    out["normest/e"], out["normest/itn"] = e, itn

    path = os.path.join(HERE, "ops.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path) // 1024, "KiB")


if __name__ == "__main__":
    op_fixtures()
    solver_fixtures()
