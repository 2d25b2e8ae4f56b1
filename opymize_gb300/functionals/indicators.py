"""Indicator, affine and constraint functionals (opymize/functionals/indicators.py,
opymize/functionals/affine.py)."""

import numpy as np

from opymize_gb300 import Variable, Functional
from opymize_gb300.functionals._eval import fct, evaluate, devcopy
from opymize_gb300.operators import ConstOp, ConstrainOp, PosProj, NegProj
from opymize_gb300.operators.affine import AffineProxOp


class AffineFct(Functional):
    """F(x) = b + sum_i c_i*x_i (opymize/functionals/affine.py:9-44)."""

    def __init__(self, N, b=0, c=1, conj=None):
        Functional.__init__(self)
        self.b, self.c = b, c
        self.x = Variable(N)
        self.conj = IndicatorFct(N, c1=c, c2=b, conj=self) if conj is None else conj

    def _eval_gpu(self, x):
        kw = dict(scalar0=float(self.b))
        if isinstance(self.c, np.ndarray):
            kw["v0"] = devcopy(self, "c", self.c, x.dtype).ptr
        else:
            kw["scalar1"] = float(self.c)
        return evaluate(fct("affine", self.x.size, 1, **kw), x)

    def prox(self, tau):
        """x - tau*c (affine.py:38-42) for any kind of step."""
        return AffineProxOp(self.x.size, 1.0, self.c, tau)


class ConstFct(AffineFct):
    """F(x) = const (opymize/functionals/affine.py:46-49)."""

    def __init__(self, N, const=0, conj=None):
        AffineFct.__init__(self, N, b=const, c=0)


class ZeroFct(ConstFct):
    """F(x) = 0 (opymize/functionals/affine.py:51-57)."""

    def __init__(self, N, conj=None):
        ConstFct.__init__(self, N, const=0)

    def prox(self, tau):
        from opymize_gb300.linear.scale import IdentityOp
        return IdentityOp(self.x.size)


class MaskedAffineFct(Functional):
    """F(x) = sum(c[mask]*x[mask]) + indicator(x[~mask] == 0)
    (opymize/functionals/affine.py:59-90)."""

    def __init__(self, mask, c, conj=None):
        Functional.__init__(self)
        self.x = Variable(c.shape)
        self.mask = np.asarray(mask).astype(bool)
        self.c = c
        self.conj = ConstrainFct(mask, c, conj=self) if conj is None else conj
        scale = np.zeros(c.shape)
        scale[self.mask, :] = 1.0
        self._scale = scale.ravel()

    def _eval_gpu(self, x):
        N, M = self.c.shape
        return evaluate(fct("masked_affine", N, M, v0=devcopy(self, "c", self.c, x.dtype).ptr,
                            mask=devcopy(self, "m", self.mask.astype(np.uint8), np.uint8).ptr), x)

    def prox(self, tau):
        """mask*(x - tau*c) (affine.py:86-90) for any kind of step."""
        return AffineProxOp(self.x.size, self._scale, self.c.ravel(), tau)


class IndicatorFct(Functional):
    """F(x) = c2 if x == c1 else inf (opymize/functionals/indicators.py:8-29)."""

    def __init__(self, N, c1=0, c2=0, conj=None):
        Functional.__init__(self)
        self.c1, self.c2 = c1, c2
        self.x = Variable(N)
        self.conj = AffineFct(N, b=-c2, c=c1, conj=self) if conj is None else conj
        self._prox = ConstOp(N, self.x.new() + c1)

    def _eval_gpu(self, x):
        kw = dict(scalar0=float(self.c2))
        if isinstance(self.c1, np.ndarray):
            kw["v0"] = devcopy(self, "c1", self.c1, x.dtype).ptr
        else:
            kw["scalar1"] = float(self.c1)
        return evaluate(fct("indicator", self.x.size, 1, **kw), x)

    def prox(self, tau):
        return self._prox


class ConstrainFct(Functional):
    """F(x) = 0 if x[mask,:] == c[mask,:] else inf
    (opymize/functionals/indicators.py:31-58)."""

    def __init__(self, mask, c, conj=None):
        Functional.__init__(self)
        self.x = Variable(c.shape)
        self.mask = np.asarray(mask).astype(bool)
        self.c = c
        self.conj = MaskedAffineFct(mask, c, conj=self) if conj is None else conj
        self._prox = ConstrainOp(self.mask, c)

    def _eval_gpu(self, x):
        N, M = self.c.shape
        return evaluate(fct("constrain", N, M, v0=devcopy(self, "c", self.c, x.dtype).ptr,
                            mask=devcopy(self, "m", self.mask.astype(np.uint8), np.uint8).ptr), x)

    def prox(self, tau):
        return self._prox


class PositivityFct(Functional):
    """F(x) = 0 if x >= 0 else inf (opymize/functionals/indicators.py:60-80)."""

    def __init__(self, N, conj=None):
        Functional.__init__(self)
        self.x = Variable(N)
        self.conj = NegativityFct(N, conj=self) if conj is None else conj
        self._prox = PosProj(N)

    def _eval_gpu(self, x):
        return evaluate(fct("positivity", self.x.size, 1), x)

    def prox(self, tau):
        return self._prox


class NegativityFct(Functional):
    """F(x) = 0 if x <= 0 else inf (opymize/functionals/indicators.py:82-98)."""

    def __init__(self, N, conj=None):
        Functional.__init__(self)
        self.x = Variable(N)
        self.conj = PositivityFct(N, conj=self) if conj is None else conj
        self._prox = NegProj(N)

    def _eval_gpu(self, x):
        return evaluate(fct("negativity", self.x.size, 1), x)

    def prox(self, tau):
        return self._prox
