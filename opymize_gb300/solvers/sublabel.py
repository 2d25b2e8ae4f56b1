"""Fused iterations of the sublabel-lifted scalar model on the generic path.

`tools.lifting.sublabel_problem` assembles the model from the reference's
operator vocabulary (BlockOp of IdentityOp, IndexedMultAdj, MatrixMultR,
ScaleOp, GradientOp; SplitSum of PositivityFct, ZeroFct, IndicatorFct,
L1Norms, EpigraphSupp) and tags its operator with the model's data.  For such
an operator `PDHG.solve` replaces the generic iteration's ~22 launches
(pdhg.py:124-187 over the operator tree) by two fused passes of libopyx
(`opyx_sublabel_pass`): pass A computes x_{k+1} and xbar from A^T y_k, pass B
computes y_{k+1} from A xbar with the prox maps of F* (the Frobenius ball of
the TV term and the direct epigraph projection) applied in place.  The gap at
checks, the set-up (steps, initial A x0) and everything else stay on the
generic path.
"""

import numpy as np

from opymize_gb300 import _lib
from opymize_gb300.gpuarray import DeviceArray, stream_ptr


class SublabelPasses(object):
    """The two fused passes for one solve, or None from `make` when the
    operator is not a tagged sublabel model or its steps do not have the
    per-label structure the kernels take."""

    MAX_LABELS = 32

    @classmethod
    def make(cls, solver, dtype, steps, tau, sigma, theta):
        model = getattr(solver.linop, "sublabel", None)
        if model is None or steps not in ("precond", "const"):
            return None
        L = int(model["L"])
        dims = tuple(model["dims"])
        epi = model["epi"]
        if not 2 <= L <= cls.MAX_LABELS or len(dims) != 2 or epi.data.ndim != 1 or \
                epi.data.nsubpoints > 16:
            return None
        H, W = dims
        N = H * W
        if solver.g.x.size != N * (L + 1) + (L - 1) * N * 2 or \
                solver.f.x.size != N * (3 * L + 2):
            return None
        return cls(model, dtype, steps, tau, sigma, theta, N, H, W, L)

    def __init__(self, model, dtype, steps, tau, sigma, theta, N, H, W, L):
        d = _lib.opyx_sublabel()
        d.dtype = _lib.OPYX_F32 if np.dtype(dtype) == np.float32 else _lib.OPYX_F64
        d.L, d.H, d.W = L, H, W
        data = model["data"]
        t = np.asarray(data["t"], dtype=np.float64)
        Bc = np.asarray(data["Bc"], dtype=np.float64)        # (L - 1, 2, 2): B[j, m, k]
        for l in range(L):
            d.t[l] = t[l]
        for j in range(L - 1):
            for m in range(2):
                for k in range(2):
                    d.B[(j * 2 + m) * 2 + k] = Bc[j, m, k]
        d.lbd = float(model["lbd"])
        d.theta = float(theta)
        esize = np.dtype(dtype).itemsize
        if steps == "precond":
            th, sh = tau.get(), sigma.get()
            tu = th[:N * L].reshape(N, L)
            tm = th[N * L + N:].reshape(L - 1, N, 2)
            sq = sh[:N * L].reshape(N, L)
            se = sh[N * L:N * L + N]
            ss = sh[N * L + 3 * N:N * L + 4 * N]
            sz = sh[N * L + 4 * N:].reshape(L - 1, N, 2)
            # the preconditioner of this A is the same for every pixel in
            # these parts; anything else stays on the generic path
            uniform = (tu == tu[:1]).all() and (tm == tm[:, :1]).all() and \
                (sq == sq[:1]).all() and (se == se[0]).all() and (ss == ss[0]).all() and \
                (sz == sz[:, :1]).all()
            if not uniform:
                raise ValueError("preconditioner not uniform over pixels")
            for l in range(L):
                d.tau_u[l], d.sig_q[l] = tu[0, l], sq[0, l]
            for j in range(L - 1):
                for m in range(2):
                    d.tau_mu[j * 2 + m], d.sig_z[j * 2 + m] = tm[j, 0, m], sz[j, 0, m]
            d.sig_e, d.sig_s = se[0], ss[0]
            d.tau_g = tau.ptr + N * L * esize
            d.sig_p = sigma.ptr + (N * L + N) * esize
            self._keep = (tau, sigma)
        else:
            tv, sv = float(tau), float(sigma)
            for l in range(L):
                d.tau_u[l], d.sig_q[l] = tv, sv
            for k in range(2 * (L - 1)):
                d.tau_mu[k], d.sig_z[k] = tv, sv
            d.sig_e = d.sig_s = sv
            d.tau_g, d.sig_p = None, None
            d.tau_g0, d.sig_p0 = tv, sv
        e = model["epi"].data.struct(dtype)
        d.nsub = int(e.nsubpoints)
        # each interval's points in increasing slope (the same for every
        # pixel): the projection then skips its per-instance sort
        ed = model["epi"].data
        vj = np.asarray(ed.v)[:, 0][np.asarray(ed.J)]          # (L - 1, nsub)
        order = np.argsort(vj, axis=1, kind="stable")
        srt = np.take_along_axis(vj, order, axis=1)
        if (np.diff(srt, axis=1) > 0).all():
            d.sorted = 1
            for j in range(L - 1):
                for k in range(d.nsub):
                    d.perm[j * 16 + k] = int(order[j, k])
                    d.vsorted[j * 16 + k] = float(srt[j, k])
        d.v, d.bt, d.J = e.v, e.bt, e.J
        d.It = None if bool(np.asarray(model["epi"].data.I).all()) else e.It
        self._epi = e
        self.d = d
        self.xbar = DeviceArray.empty((N * (L + 1) + (L - 1) * N * 2,), dtype)
        d.xbar = self.xbar.ptr
        if d.sorted:
            # which lines carry the envelope of every instance: fixed by the
            # data term, so found once; the projections then scan only those
            self.hull = DeviceArray.empty(((L - 1) * N,), np.uint8)
            d.hull = self.hull.ptr
            _lib.call("opyx_sublabel_pass", d, 2, stream_ptr())

    def iterate(self, v):
        """One iteration: x_{k+1} into v['xkp1'], y_{k+1} into v['ykp1']."""
        d = self.d
        d.xk, d.xkp1, d.yk, d.ykp1 = v['xk'].ptr, v['xkp1'].ptr, v['yk'].ptr, v['ykp1'].ptr
        s = stream_ptr()
        _lib.call("opyx_sublabel_pass", d, 0, s)
        _lib.call("opyx_sublabel_pass", d, 1, s)
