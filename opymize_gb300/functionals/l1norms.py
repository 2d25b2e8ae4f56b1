"""L1 norms of per-pixel matrices and their Huber smoothing
(opymize/functionals/l1norms.py)."""

import numpy as np

from opymize_gb300 import Variable, Functional, _lib
from opymize_gb300.functionals._eval import fct, evaluate
from opymize_gb300.operators.proj import L1NormsProj, HuberConjProj


class L1Norms(Functional):
    """F(x) = lbd * sum_i |x[i,:,:]|, Frobenius or nuclear norm
    (opymize/functionals/l1norms.py:34-63)."""

    def __init__(self, N, M, lbd, matrixnorm="frobenius", conj=None):
        Functional.__init__(self)
        assert matrixnorm in ['frobenius', 'nuclear']
        self.N, self.M = int(N), tuple(M)
        self.x = Variable((self.N,) + self.M)
        self.lbd = lbd
        self.matrixnorm = matrixnorm
        conjnorm = 'spectral' if matrixnorm == 'nuclear' else 'frobenius'
        self.conj = L1NormsConj(N, M, lbd, conjnorm, conj=self) if conj is None else conj

    def _eval_gpu(self, x):
        f = fct("l1norms", self.N, self.M[0], self.M[1], lbd=float(self.lbd),
                matrixnorm=_lib.NORM["spectral" if self.matrixnorm == "nuclear" else "frobenius"])
        return evaluate(f, x)


class L1NormsConj(Functional):
    """F(x) = sum_i indicator(|x[i,:,:]| <= lbd), Frobenius or spectral norm
    (opymize/functionals/l1norms.py:65-92); prox does not depend on tau."""

    def __init__(self, N, M, lbd, matrixnorm="frobenius", conj=None):
        Functional.__init__(self)
        assert matrixnorm in ['frobenius', 'spectral']
        self.N, self.M = int(N), tuple(M)
        self.x = Variable((self.N,) + self.M)
        self.lbd = lbd
        self.matrixnorm = matrixnorm
        conjnorm = 'nuclear' if matrixnorm == 'spectral' else 'frobenius'
        self.conj = L1Norms(N, M, lbd, conjnorm, conj=self) if conj is None else conj
        self._prox = L1NormsProj(N, M, self.lbd, matrixnorm)

    def _eval_gpu(self, x):
        f = fct("l1norms_conj", self.N, self.M[0], self.M[1], lbd=float(self.lbd),
                matrixnorm=_lib.NORM[self.matrixnorm])
        return evaluate(f, x)

    def prox(self, tau):
        return self._prox


class HuberL1Norms(Functional):
    """F(x) = lbd * sum_i h_alph(|x_i|_F) with the Huber function
    h(r) = r^2/(2 alph) for r <= alph and r - alph/2 beyond: Huber-smoothed
    (colour) total variation.  As alph -> 0 it becomes L1Norms."""

    def __init__(self, N, M, lbd, alph, conj=None):
        Functional.__init__(self)
        assert lbd > 0 and alph > 0
        self.N, self.M = int(N), tuple(M)
        self.x = Variable((self.N,) + self.M)
        self.lbd, self.alph = lbd, alph
        self.conj = HuberL1NormsConj(N, M, lbd, alph, conj=self) if conj is None else conj

    def _eval_gpu(self, x):
        f = fct("huber", self.N, self.M[0], self.M[1], lbd=float(self.lbd),
                alpha=float(self.alph))
        return evaluate(f, x)


class HuberL1NormsConj(Functional):
    """F*(y) = sum_i alph/(2 lbd) |y_i|^2 + indicator(|y_i|_F <= lbd); its prox
    is y_i <- proj_{|.| <= lbd}(y_i / (1 + sigma*alph/lbd))."""

    def __init__(self, N, M, lbd, alph, conj=None):
        Functional.__init__(self)
        self.N, self.M = int(N), tuple(M)
        self.x = Variable((self.N,) + self.M)
        self.lbd, self.alph = lbd, alph
        self.conj = HuberL1Norms(N, M, lbd, alph, conj=self) if conj is None else conj

    def _eval_gpu(self, x):
        f = fct("huber_conj", self.N, self.M[0], self.M[1], lbd=float(self.lbd),
                alpha=float(self.alph))
        return evaluate(f, x)

    def prox(self, tau):
        return HuberConjProj(self.N, self.M, self.lbd, self.alph, tau)
