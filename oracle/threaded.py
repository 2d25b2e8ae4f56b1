"""Oracle PDHG over every host thread -- TEST INFRASTRUCTURE ONLY.

The reference's CPU solver (opymize/solvers/pdhg.py:124-187 for one
iteration, :229-315 for the driver, :23-44 for the gap) for the ROF family
the fused GPU path serves: G = SSD (opymize/functionals/quad.py:7-55),
F = L1Norms (opymize/functionals/l1norms.py:34-92) or the Huber-smoothed
norms of ``oracle.HuberL1Norms``, A = forward-difference gradient
(opymize/linear/diff.py:67-144), diagonally preconditioned steps
(pdhg.py:189-203).

Every array operation of an iteration is the oracle's own numpy / scipy call
(``oracle.pdhg.PDHG``), applied to pixel ranges on a thread pool: numpy's
element-wise loops and scipy's CSR matrix-vector product release the GIL, so
the ranges run on separate cores.  A row range of a CSR product and an
element-wise formula on a sub-range give the same bits as on the whole array,
so iterates equal those of ``oracle.PDHG`` exactly; the gap's sums are
accumulated per range and then added, which moves the last bits of the
objectives only.

bench.py uses it as the CPU baseline (a reference CPU solve given all the host
cores); tests compare it with ``oracle.PDHG``.
"""

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from oracle.functionals import SSD, L1Norms, HuberL1Norms
from oracle.linops import Gradient


class ThreadedROF(object):
    """min_x 0.5*|x - f|^2 + lbd*sum_i |grad x_i| (Huber-smoothed when
    ``huber`` > 0) with preconditioned PDHG, the work of each step split into
    ``threads`` pixel ranges.  ``f`` is (N, C) with N = prod(dims)."""

    def __init__(self, f, dims, lbd, huber=0.0, threads=None):
        self.dims = tuple(dims)
        self.f = np.asarray(f, dtype=np.float64).reshape(-1, f.shape[-1])
        N, C = self.f.shape
        D = len(self.dims)
        assert N == int(np.prod(self.dims))
        self.N, self.C, self.D, self.K = N, C, D, C * D
        self.lbd, self.huber = lbd, huber
        self.threads = int(threads or os.cpu_count() or 1)
        op = Gradient(self.dims, C, "forward")
        nt = max(1, min(self.threads, N))
        px = np.linspace(0, N, nt + 1).astype(np.int64)
        self.ranges = [(int(px[k]), int(px[k + 1])) for k in range(nt)]
        K = self.K
        # row blocks of A (rows of y) and of A^T (rows of x) per pixel range
        self.A = [op.spmat[p0 * K:p1 * K] for (p0, p1) in self.ranges]
        self.AT = [op.adjoint.spmat[p0 * C:p1 * C] for (p0, p1) in self.ranges]
        self.G, self.F = [], []
        for (p0, p1) in self.ranges:
            self.G.append(SSD(self.f[p0:p1]))
            n = p1 - p0
            self.F.append(HuberL1Norms(n, (C, D), lbd, huber) if huber > 0
                          else L1Norms(n, (C, D), lbd))
        self.pool = ThreadPoolExecutor(nt)
        self.info = {}

    # --- helpers
    def _xs(self, k, a):
        p0, p1 = self.ranges[k]
        return a[p0 * self.C:p1 * self.C]

    def _ys(self, k, a):
        p0, p1 = self.ranges[k]
        return a[p0 * self.K:p1 * self.K]

    def _each(self, fn):
        return list(self.pool.map(fn, range(len(self.ranges))))

    def close(self):
        self.pool.shutdown(wait=True)

    # --- set-up (pdhg.py:236-275): zero start, A x0, A^T y0, precond tables
    def _setup(self):
        N, C, K = self.N, self.C, self.K
        v = self.v = {}
        for s in ("xk", "xkp1", "xgradk", "xgradkp1", "xtau"):
            v[s] = np.zeros(N * C)
        for s in ("yk", "ykp1", "ygradk", "ygradkp1", "ygradbk", "ysigma"):
            v[s] = np.zeros(N * K)
        eps = np.spacing(1)

        def setup(k):
            self._ys(k, v["ygradk"])[:] = self.A[k].dot(v["xk"])
            self._xs(k, v["xgradk"])[:] = self.AT[k].dot(v["yk"])
            # rowwise_lp with p = 1 (opymize/__init__.py:122-142), inverted above eps
            ys = self._ys(k, v["ysigma"])
            ys[:] = np.asarray(abs(self.A[k]).sum(axis=1)).ravel()
            ys[ys > eps] = 1.0 / ys[ys > eps]
            xt = self._xs(k, v["xtau"])
            xt[:] = np.asarray(abs(self.AT[k]).sum(axis=1)).ravel()
            xt[xt > eps] = 1.0 / xt[xt > eps]
            return (self.G[k].prox(xt), self.F[k].conj.prox(ys))
        proxes = self._each(setup)
        self.gprox = [p[0] for p in proxes]
        self.fprox = [p[1] for p in proxes]

    # --- one iteration (pdhg.py:124-187), theta = 1, precond steps
    def _iterate(self):
        v = self.v
        theta = 1.0

        def primal(k):
            xkp1 = self._xs(k, v["xkp1"])
            xkp1[:] = self._xs(k, v["xk"]) - self._xs(k, v["xtau"]) * self._xs(k, v["xgradk"])
            self.gprox[k](xkp1)

        def dual(k):
            ygkp1 = self._ys(k, v["ygradkp1"])
            ygkp1[:] = self.A[k].dot(v["xkp1"])
            ygb = self._ys(k, v["ygradbk"])
            ygb[:] = (1 + theta) * ygkp1 - theta * self._ys(k, v["ygradk"])
            ykp1 = self._ys(k, v["ykp1"])
            ykp1[:] = self._ys(k, v["yk"]) + self._ys(k, v["ysigma"]) * ygb
            self.fprox[k](ykp1)

        def adjoint(k):
            self._xs(k, v["xgradkp1"])[:] = self.AT[k].dot(v["ykp1"])
            # advance (pdhg.py:184-187): copies, as the reference makes them
            self._xs(k, v["xk"])[:] = self._xs(k, v["xkp1"])
            self._xs(k, v["xgradk"])[:] = self._xs(k, v["xgradkp1"])
            self._ys(k, v["yk"])[:] = self._ys(k, v["ykp1"])
            self._ys(k, v["ygradk"])[:] = self._ys(k, v["ygradkp1"])

        self._each(primal)
        self._each(dual)
        self._each(adjoint)

    # --- duality gap (pdhg.py:23-44), sums per range
    def pd_gap(self):
        v = self.v

        def part(k):
            xk, xg = self._xs(k, v["xk"]), self._xs(k, v["xgradk"])
            yk, yg = self._ys(k, v["yk"]), self._ys(k, v["ygradk"])
            gp, _ = self.G[k](xk)
            fp, _ = self.F[k](yg)
            gd, _ = self.G[k].conj(-xg)
            fd, infd = self.F[k].conj(yk)
            return gp, fp, gd, fd, infd
        parts = self._each(part)
        objp = sum(p[0] for p in parts) + sum(p[1] for p in parts)
        objd = -sum(p[2] for p in parts) - sum(p[3] for p in parts)
        infeasd = max(p[4] for p in parts)
        return {"objp": objp, "objd": objd, "infeasp": 0.0, "infeasd": infeasd,
                "gap": objp - objd,
                "relgap": (objp - objd) / max(np.spacing(1), abs(objd))}

    # --- driver (pdhg.py:229-315) with steps="precond"
    def solve(self, term_pd_gap=1e-4, term_maxiter=50000, granularity=10):
        """Iterate from zero until |relgap| < tol and the infeasibilities are
        below tol, testing every ``granularity`` iterations."""
        self._setup()
        it = 0
        self.info = {}
        while it < term_maxiter:
            it += 1
            self._iterate()
            if it % granularity == 0:
                self.info["iter"] = it
                self.info.update(self.pd_gap())
                if abs(self.info["relgap"]) < term_pd_gap and \
                        max(self.info["infeasp"], self.info["infeasd"]) < term_pd_gap:
                    break
        return self.info

    def iterate(self, n):
        """``n`` iterations with no set-up and no gap (for timing samples);
        call after ``solve`` or ``_setup``."""
        for _ in range(n):
            self._iterate()

    @property
    def state(self):
        return (self.v["xk"], self.v["yk"])
