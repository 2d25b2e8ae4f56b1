"""Epigraph functionals of quadratics and the Huber perspective
(opymize/functionals/epigraph.py:129-274)."""

import numpy as np

from opymize_gb300 import Variable, Functional
from opymize_gb300.functionals._eval import fct, evaluate, devcopy
from opymize_gb300.operators.proj import QuadEpiProj


def quad_dual_coefficients(a, b, c):
    """f(x) = 0.5a|x|^2 + <b,x> + c  ->  f* coefficients (epigraph.py:129-133)."""
    return (1.0 / a, -b / a, 0.5 / a * (b ** 2).sum(axis=-1) - c)


class QuadEpiSupp(Functional):
    """sum_i -x[i,-1]*f_i(-x[i,:-1]/x[i,-1]) if x[i,-1] < 0, else inf
    (opymize/functionals/epigraph.py:135-167)."""

    def __init__(self, N, M, a=1.0, b=None, c=None, conj=None):
        Functional.__init__(self)
        assert a > 0
        self.N, self.M = int(N), int(M)
        self.x = Variable((self.N, self.M + 1))
        self.a = a
        self.b = np.zeros((N, M)) if b is None else b
        self.c = np.zeros((N,)) if c is None else c
        if conj is None:
            da, db, dc = quad_dual_coefficients(self.a, self.b, self.c)
            self.conj = QuadEpiInd(N, M, a=da, b=db, c=dc, conj=self)
        else:
            self.conj = conj

    def _eval_gpu(self, x):
        f = fct("quadepi_supp", self.N, self.M + 1, a=float(self.a),
                v0=devcopy(self, "b", self.b, x.dtype).ptr,
                v1=devcopy(self, "c", self.c, x.dtype).ptr)
        return evaluate(f, x)


QuadSupport = QuadEpiSupp


class QuadEpiInd(Functional):
    """sum_i indicator(f_i(x[i,:-1]) <= x[i,-1]), f_i = 0.5a|x|^2 + <b_i,x> + c_i
    (opymize/functionals/epigraph.py:169-201); prox = QuadEpiProj."""

    def __init__(self, N, M, a=1.0, b=None, c=None, conj=None):
        Functional.__init__(self)
        assert a > 0
        self.N, self.M = int(N), int(M)
        self.x = Variable((self.N, self.M + 1))
        self.a = a
        self.b = np.zeros((N, M)) if b is None else b
        self.c = np.zeros((N,)) if c is None else c
        if conj is None:
            da, db, dc = quad_dual_coefficients(self.a, self.b, self.c)
            self.conj = QuadEpiSupp(N, M, a=da, b=db, c=dc, conj=self)
        else:
            self.conj = conj
        self._prox = QuadEpiProj(N, M, alph=a, b=self.b, c=self.c)

    def _eval_gpu(self, x):
        f = fct("quadepi_ind", self.N, self.M + 1, a=float(self.a),
                v0=devcopy(self, "b", self.b, x.dtype).ptr,
                v1=devcopy(self, "c", self.c, x.dtype).ptr)
        return evaluate(f, x)

    def prox(self, tau):
        return self._prox


class HuberPerspective(Functional):
    """Perspective of the Huber function (opymize/functionals/epigraph.py:203-236)."""

    def __init__(self, N, M, lbd=1.0, alph=1.0, conj=None):
        Functional.__init__(self)
        assert lbd > 0 and alph > 0
        self.N, self.M = int(N), int(M)
        self.x = Variable((self.N, self.M + 1))
        self.lbd, self.alph = lbd, alph
        if conj is None:
            self.conj = TruncQuadEpiInd(N, M, lbd=self.lbd, alph=self.alph / self.lbd, conj=self)
        else:
            self.conj = conj

    def _eval_gpu(self, x):
        f = fct("huber_persp", self.N, self.M + 1, lbd=float(self.lbd), alpha=float(self.alph))
        return evaluate(f, x)


class TruncQuadEpiInd(Functional):
    """indicator(|x| <= lbd) + indicator(0.5 alph |x|^2 <= x[-1])
    (opymize/functionals/epigraph.py:238-274); prox = truncated QuadEpiProj."""

    def __init__(self, N, M, lbd=1.0, alph=1.0, conj=None):
        Functional.__init__(self)
        assert lbd > 0 and alph > 0
        self.N, self.M = int(N), int(M)
        self.x = Variable((self.N, self.M + 1))
        self.lbd, self.alph = lbd, alph
        if conj is None:
            self.conj = HuberPerspective(N, M, lbd=self.lbd, alph=self.alph * self.lbd, conj=self)
        else:
            self.conj = conj
        self._prox = QuadEpiProj(N, M, lbd=self.lbd, alph=self.alph)

    def _eval_gpu(self, x):
        f = fct("truncquad_ind", self.N, self.M + 1, lbd=float(self.lbd), alpha=float(self.alph))
        return evaluate(f, x)

    def prox(self, tau):
        return self._prox


def _epigraph_eval(data, which, x, supp=None):
    from opymize_gb300 import _lib
    from opymize_gb300.gpuarray import DeviceArray, Workspace, stream_ptr
    assert x.size == data.nregions * data.nfuns * (data.ndim + 1)
    ws = Workspace.get(_lib.load().opyx_reduce_workspace_size())
    out = DeviceArray.zeros((2,), np.float64)
    _lib.call("opyx_epigraph_eval", data.struct(x.dtype, supp), x.dcode, int(which), x.ptr,
              out.ptr, ws.ptr, stream_ptr())
    h = out.get()
    return float(h[0]), float(h[1])


class EpigraphInd(Functional):
    """F(x) = 0 if <v[k], x[j,i,:-1]> - b[i,k] <= x[j,i,-1] for every i, j and
    k in J[j] with I[i,k], else inf (opymize/functionals/epigraph.py:7-54).
    The value is (0, infeasibility) reduced on the device; prox = EpigraphProj
    (independent of tau)."""

    def __init__(self, I, If, J, v, b, conj=None):
        from opymize_gb300.operators.proj import EpigraphProj
        Functional.__init__(self)
        self._prox = EpigraphProj(I, J, v, b)
        d = self._prox.data
        self.I, self.If, self.J, self.v, self.b = d.I, If, d.J, d.v, d.b
        self.x = Variable((d.nregions, d.nfuns, d.ndim + 1))
        self.conj = EpigraphSupp(I, If, J, v, b, conj=self) if conj is None else conj

    @property
    def A(self):
        return self._prox.Ab[0]

    def _eval_gpu(self, x):
        return _epigraph_eval(self._prox.data, 0, x)

    def prox(self, tau):
        return self._prox


EpigraphFct = EpigraphInd


class EpigraphSupp(Functional):
    """F(x) = max sum_ji <y, x[j,i]> over y[j,i] in epi(f[i]_j*): the support
    function of the epigraphs (opymize/functionals/epigraph.py:56-112).
    f[i]_j is given by its affine faces If[i][j] (rows of ndim+1 indices
    into J[j]); the face equations and the region checks are computed once on
    the host, the value is reduced on the device."""

    def __init__(self, I, If, J, v, b, conj=None):
        from opymize_gb300.operators.proj import _EpigraphData
        Functional.__init__(self)
        self.data = _EpigraphData(I, J, v, b)
        d = self.data
        self.I, self.If, self.J, self.v, self.b = d.I, If, d.J, d.v, d.b
        self.x = Variable((d.nregions, d.nfuns, d.ndim + 1))
        self._pieces = None
        self._supp_dev = None
        self.conj = EpigraphInd(I, If, J, v, b, conj=self) if conj is None else conj

    def checks(self):
        """Per region the inverse transpose of the rows (v[J[j,k]], -1),
        k <= ndim: the region's simplex test (epigraph.py:98-100)."""
        d = self.data
        n1 = d.ndim + 1
        chk = -np.ones((d.nregions, n1, n1))
        chk[:, :, :-1] = d.v[d.J[:, :n1]]
        return np.ascontiguousarray(np.linalg.inv(chk).transpose(0, 2, 1))

    def pieces(self):
        """(eq_off, eqns): per instance (j, i) the affine functions c.p + d
        through the values on each face If[i][j] (epigraph.py:84-97)."""
        if self._pieces is None:
            d = self.data
            if self.If is None:
                raise ValueError("EpigraphSupp needs the faces If")
            n1 = d.ndim + 1
            rows, off = [], [0]
            for j in range(d.nregions):
                pts = d.v[d.J[j]]
                for i in range(d.nfuns):
                    faces = np.asarray(self.If[i][j], dtype=np.int64).reshape(-1, n1)
                    P = pts[faces]                                 # (nf, n1, ndim)
                    vals = d.b[i, d.J[j]][faces]                   # (nf, n1)
                    M = P[:, 1:] - P[:, :1]
                    c = np.linalg.solve(M, (vals[:, 1:] - vals[:, :1])[..., None])[..., 0]
                    eq = np.empty((faces.shape[0], n1))
                    eq[:, :-1] = c
                    eq[:, -1] = vals[:, 0] - (c * P[:, 0]).sum(axis=-1)
                    rows.append(eq)
                    off.append(off[-1] + eq.shape[0])
            self._pieces = (np.asarray(off, np.int64), np.concatenate(rows, axis=0))
        return self._pieces

    def _eval_gpu(self, x):
        """Faces given: max over their affine functions, as the reference.
        If = None (ndim 1): the convex envelope of each instance's points,
        evaluated on the device (the same value when the faces are the lower
        convex hull, without a host loop over every instance)."""
        from opymize_gb300.gpuarray import DeviceArray
        if self._supp_dev is None:
            chk = DeviceArray.to_gpu(self.checks())
            if self.If is None:
                if self.data.ndim != 1:
                    raise ValueError("EpigraphSupp without faces needs ndim 1")
                self._supp_dev = (None, None, chk)
            else:
                off, eqns = self.pieces()
                self._supp_dev = (DeviceArray.to_gpu(off), DeviceArray.to_gpu(eqns), chk)
        return _epigraph_eval(self.data, 1, x, self._supp_dev)


EpigraphSupportFct = EpigraphSupp
