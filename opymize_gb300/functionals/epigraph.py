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
