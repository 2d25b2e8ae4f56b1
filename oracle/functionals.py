"""Oracle functionals: value / infeasibility (for the duality gap) and prox
maps, restating opymize/functionals/* and the prox operators they return
(opymize/operators/*).  ``prox(tau)`` returns a callable that maps an array
in place; ``tau`` is a scalar or an array of the functional's size."""

import numpy as np
from numpy.linalg import norm

from oracle.prox import (l1_projection, huber_conj_prox, quadepi_projection)


class Functional(object):
    size = None
    conj = None

    def __call__(self, x):
        raise NotImplementedError

    def prox(self, tau):
        raise NotImplementedError


class SSD(Functional):
    """0.5*sum_{mask} vol_k (x - f)^2 + shift (opymize/functionals/quad.py:7-55)."""

    def __init__(self, data, vol=None, shift=0.0, mask=None, conj=None):
        self.f = np.atleast_2d(data)
        N, C = self.f.shape
        self.size = N * C
        self.shift = shift
        self.vol = np.ones(C) if vol is None else np.asarray(vol, float)
        self.mask = np.ones(N, dtype=bool) if mask is None else np.asarray(mask, bool)
        if conj is None:
            cj_vol = 1.0 / self.vol
            cj_data = np.zeros_like(self.f)
            cj_data[self.mask, :] = self.f[self.mask, :] * (-self.vol)
            cj_shift = -0.5 * np.einsum('ik,k->', cj_data ** 2, cj_vol) - self.shift
            self.conj = SSD(cj_data, vol=cj_vol, shift=cj_shift, mask=self.mask, conj=self)
        else:
            self.conj = conj

    def __call__(self, x):
        x = x.reshape(self.f.shape)
        val = 0.5 * np.einsum('ik,k->', (x - self.f)[self.mask, :] ** 2, self.vol)
        return val + self.shift, 0

    def prox(self, tau):
        tauvol = np.zeros_like(self.f)
        tv = (tau * np.ones(self.f.size)).reshape(self.f.shape)[self.mask, :]
        tauvol[self.mask, :] = tv * self.vol
        a = 1.0 / (1.0 + tauvol.ravel())
        b = tauvol.ravel()
        shift = np.zeros_like(self.f)
        shift[self.mask, :] = self.f[self.mask, :]
        shift = shift.ravel()

        def op(x):
            x[:] = a * (x + b * shift)
        return op


def _norms(x, matrixnorm):
    """Per-group norms (opymize/functionals/l1norms.py:8-32)."""
    N, M1, M2 = x.shape
    if M1 == 1 or M2 == 1 or matrixnorm == "frobenius":
        return np.sqrt(np.einsum('ilm,ilm->i', x, x))
    ordv = 'nuc' if matrixnorm == 'nuclear' else 2
    return norm(x, ord=ordv, axis=(1, 2))


class L1Norms(Functional):
    """lbd * sum_i |x_i| (opymize/functionals/l1norms.py:34-63)."""

    def __init__(self, N, M, lbd, matrixnorm="frobenius", conj=None):
        self.N, self.M, self.lbd, self.matrixnorm = N, tuple(M), lbd, matrixnorm
        self.size = N * M[0] * M[1]
        conjnorm = 'spectral' if matrixnorm == 'nuclear' else 'frobenius'
        self.conj = L1NormsConj(N, M, lbd, conjnorm, conj=self) if conj is None else conj

    def __call__(self, x):
        n = _norms(x.reshape((self.N,) + self.M), self.matrixnorm)
        return self.lbd * n.sum(), 0


class L1NormsConj(Functional):
    """Indicator of |x_i| <= lbd (opymize/functionals/l1norms.py:65-92);
    prox is the projection and does not depend on tau."""

    def __init__(self, N, M, lbd, matrixnorm="frobenius", conj=None):
        self.N, self.M, self.lbd, self.matrixnorm = N, tuple(M), lbd, matrixnorm
        self.size = N * M[0] * M[1]
        conjnorm = 'nuclear' if matrixnorm == 'spectral' else 'frobenius'
        self.conj = L1Norms(N, M, lbd, conjnorm, conj=self) if conj is None else conj

    def __call__(self, x):
        n = _norms(x.reshape((self.N,) + self.M), self.matrixnorm)
        return 0, norm(np.fmax(0, n - self.lbd), ord=np.inf)

    def prox(self, tau):
        def op(x):
            l1_projection(x, self.N, self.M, self.lbd, self.matrixnorm)
        return op


class HuberL1Norms(Functional):
    """lbd * sum_i h_alph(|x_i|_F), h(r) = r^2/(2 alph) for r <= alph and
    r - alph/2 otherwise (Huber-smoothed total variation; no reference
    counterpart)."""

    def __init__(self, N, M, lbd, alph, conj=None):
        self.N, self.M, self.lbd, self.alph = N, tuple(M), lbd, alph
        self.size = N * M[0] * M[1]
        self.conj = HuberL1NormsConj(N, M, lbd, alph, conj=self) if conj is None else conj

    def __call__(self, x):
        r = _norms(x.reshape((self.N,) + self.M), "frobenius")
        h = np.where(r <= self.alph, 0.5 * r ** 2 / self.alph, r - 0.5 * self.alph)
        return self.lbd * h.sum(), 0


class HuberL1NormsConj(Functional):
    """sum_i alph/(2 lbd) |y_i|^2 + indicator(|y_i|_F <= lbd)."""

    def __init__(self, N, M, lbd, alph, conj=None):
        self.N, self.M, self.lbd, self.alph = N, tuple(M), lbd, alph
        self.size = N * M[0] * M[1]
        self.conj = HuberL1Norms(N, M, lbd, alph, conj=self) if conj is None else conj

    def __call__(self, x):
        xv = x.reshape((self.N,) + self.M)
        r2 = np.einsum('ilm,ilm->i', xv, xv)
        val = 0.5 * self.alph / self.lbd * r2.sum()
        return val, norm(np.fmax(0, np.sqrt(r2) - self.lbd), ord=np.inf)

    def prox(self, tau):
        def op(x):
            huber_conj_prox(x, self.N, self.M, self.lbd, self.alph, tau)
        return op


def quad_dual_coefficients(a, b, c):
    """(opymize/functionals/epigraph.py:129-133)"""
    return (1.0 / a, -b / a, 0.5 / a * (b ** 2).sum(axis=-1) - c)


class QuadEpiSupp(Functional):
    """(opymize/functionals/epigraph.py:135-167)"""

    def __init__(self, N, M, a=1.0, b=None, c=None, conj=None):
        self.N, self.M, self.a = N, M, a
        self.size = N * (M + 1)
        self.b = np.zeros((N, M)) if b is None else b
        self.c = np.zeros((N,)) if c is None else c
        if conj is None:
            da, db, dc = quad_dual_coefficients(self.a, self.b, self.c)
            self.conj = QuadEpiInd(N, M, a=da, b=db, c=dc, conj=self)
        else:
            self.conj = conj

    def __call__(self, x):
        a, b, c = self.a, self.b, self.c
        x = x.reshape(self.N, self.M + 1)
        msk = x[:, -1] < -1e-8
        x1, x2 = x[msk, :-1], -x[msk, -1]
        val = ((0.5 * a * x1 ** 2 / x2[:, None] + b[msk] * x1).sum(axis=1)
               + x2 * c[msk]).sum()
        infeas = 0 if np.all(msk) else norm(x[~msk, -1], ord=np.inf)
        return val, infeas


class QuadEpiInd(Functional):
    """(opymize/functionals/epigraph.py:169-201)"""

    def __init__(self, N, M, a=1.0, b=None, c=None, conj=None):
        self.N, self.M, self.a = N, M, a
        self.size = N * (M + 1)
        self.b = np.zeros((N, M)) if b is None else b
        self.c = np.zeros((N,)) if c is None else c
        if conj is None:
            da, db, dc = quad_dual_coefficients(self.a, self.b, self.c)
            self.conj = QuadEpiSupp(N, M, a=da, b=db, c=dc, conj=self)
        else:
            self.conj = conj
        shift = np.zeros((N, M + 1))
        shift[:, :-1] = -self.b / self.a
        shift[:, -1] = -(0.5 / self.a * (self.b ** 2).sum(axis=-1) - self.c)
        self.shift = shift

    def __call__(self, x):
        x = x.reshape(self.N, self.M + 1)
        fx = (0.5 * self.a * x[:, :-1] ** 2 + self.b * x[:, :-1]).sum(axis=1) + self.c
        return 0, norm(np.fmax(0, fx - x[:, -1]), ord=np.inf)

    def prox(self, tau):
        def op(x):
            quadepi_projection(x, self.N, self.M, self.a, shift=self.shift)
        return op


class HuberPerspective(Functional):
    """(opymize/functionals/epigraph.py:203-236)"""

    def __init__(self, N, M, lbd=1.0, alph=1.0, conj=None):
        self.N, self.M, self.lbd, self.alph = N, M, lbd, alph
        self.size = N * (M + 1)
        self.conj = TruncQuadEpiInd(N, M, lbd=lbd, alph=alph / lbd, conj=self) \
            if conj is None else conj

    def __call__(self, x):
        x = x.reshape(self.N, self.M + 1)
        lbd, alph = self.lbd, self.alph
        x1, x2 = x[:, :-1], -x[:, -1]
        x1norm = np.linalg.norm(x1, axis=-1)
        qmsk = (x1norm < alph * x2)
        lmsk = (~qmsk) & (x2 > -1e-4)
        val = 0.5 / alph * (x1norm[qmsk] ** 2 / x2[qmsk]).sum()
        val += (x1norm[lmsk] - x2[lmsk] * alph / 2).sum()
        val *= lbd
        return val, norm(np.fmin(0, x2), ord=np.inf)


class TruncQuadEpiInd(Functional):
    """(opymize/functionals/epigraph.py:238-274)"""

    def __init__(self, N, M, lbd=1.0, alph=1.0, conj=None):
        self.N, self.M, self.lbd, self.alph = N, M, lbd, alph
        self.size = N * (M + 1)
        self.conj = HuberPerspective(N, M, lbd=lbd, alph=alph * lbd, conj=self) \
            if conj is None else conj

    def __call__(self, x):
        x = x.reshape(self.N, self.M + 1)
        x1norm = np.linalg.norm(x[:, :-1], axis=-1)
        infeas = norm(np.fmax(0, x1norm - self.lbd), ord=np.inf)
        fx = 0.5 * self.alph * np.fmin(self.lbd, x1norm) ** 2
        infeas += norm(np.fmax(0, fx - x[:, -1]), ord=np.inf)
        return 0, infeas

    def prox(self, tau):
        def op(x):
            quadepi_projection(x, self.N, self.M, self.alph, lbd=self.lbd)
        return op


class SplitSum(Functional):
    """F(x1, x2, ...) = sum_i F_i(x_i) (opymize/functionals/__init__.py:10-39)."""

    def __init__(self, fcts, conj=None):
        self.fcts = fcts
        self.size = sum(F.size for F in fcts)
        self.conj = SplitSum([F.conj for F in fcts], conj=self) if conj is None else conj

    def _split(self, x):
        out, off = [], 0
        for F in self.fcts:
            out.append(x[off:off + F.size])
            off += F.size
        return out

    def __call__(self, x):
        res = [F(xi) for F, xi in zip(self.fcts, self._split(x))]
        return sum(r[0] for r in res), max(r[1] for r in res)

    def prox(self, tau):
        if isinstance(tau, np.ndarray):
            ops = [F.prox(t) for F, t in zip(self.fcts, self._split(tau))]
        else:
            ops = [F.prox(tau) for F in self.fcts]

        def op(x):
            for o, xi in zip(ops, self._split(x)):
                o(xi)
        return op


class PositivityFct(Functional):
    """(opymize/functionals/indicators.py:74-98)"""

    def __init__(self, N, conj=None):
        self.size = N
        self.conj = NegativityFct(N, conj=self) if conj is None else conj

    def __call__(self, x):
        return 0, norm(np.fmin(0, x), ord=np.inf)

    def prox(self, tau):
        def op(x):
            np.fmax(0, x, out=x)
        return op


class NegativityFct(Functional):
    def __init__(self, N, conj=None):
        self.size = N
        self.conj = PositivityFct(N, conj=self) if conj is None else conj

    def __call__(self, x):
        return 0, norm(np.fmax(0, x), ord=np.inf)

    def prox(self, tau):
        def op(x):
            np.fmin(0, x, out=x)
        return op


class AffineFct(Functional):
    """b + <c, x> (opymize/functionals/affine.py:9-44); prox x - tau*c."""

    def __init__(self, N, b=0.0, c=1.0, conj=None):
        self.size, self.b, self.c = N, b, c
        self.conj = IndicatorFct(N, c1=c, c2=b, conj=self) if conj is None else conj

    def __call__(self, x):
        val = self.b
        if isinstance(self.c, np.ndarray):
            val += np.einsum('i,i->', x, self.c)
        elif self.c != 0:
            val += self.c * np.einsum('i->', x)
        return val, 0

    def prox(self, tau):
        c = self.c

        def op(x):
            x[:] = 1 * (x + (-tau) * c)
        return op


class ZeroFct(AffineFct):
    def __init__(self, N, conj=None):
        AffineFct.__init__(self, N, b=0, c=0)

    def prox(self, tau):
        return lambda x: None


class IndicatorFct(Functional):
    """c2 if x == c1 else inf (opymize/functionals/indicators.py:8-29)."""

    def __init__(self, N, c1=0.0, c2=0.0, conj=None):
        self.size, self.c1, self.c2 = N, c1, c2
        self.conj = AffineFct(N, b=-c2, c=c1, conj=self) if conj is None else conj

    def __call__(self, x):
        return self.c2, norm(x - self.c1, ord=np.inf)

    def prox(self, tau):
        c1 = self.c1

        def op(x):
            x[:] = np.zeros(self.size) + c1
        return op


class ConstrainFct(Functional):
    """0 if x[mask,:] == c[mask,:] else inf (opymize/functionals/indicators.py:31-58)."""

    def __init__(self, mask, c, conj=None):
        self.mask, self.c = np.asarray(mask, bool), c
        self.size = c.size
        self.conj = MaskedAffineFct(mask, c, conj=self) if conj is None else conj

    def __call__(self, x):
        x = x.reshape(self.c.shape)
        return 0, norm((x[self.mask, :] - self.c[self.mask, :]).ravel(), ord=np.inf)

    def prox(self, tau):
        def op(x):
            xv = x.reshape(self.c.shape)
            xv[self.mask, :] = self.c[self.mask, :]
        return op


class MaskedAffineFct(Functional):
    """sum(c[mask]*x[mask]) + indicator(x[~mask] == 0)
    (opymize/functionals/affine.py:59-90)."""

    def __init__(self, mask, c, conj=None):
        self.mask, self.c = np.asarray(mask, bool), c
        self.size = c.size
        self.conj = ConstrainFct(mask, c, conj=self) if conj is None else conj

    def __call__(self, x):
        x = x.reshape(self.c.shape)
        val = np.einsum('ik,ik->', x[self.mask, :], self.c[self.mask, :])
        infeas = 0.0 if np.all(self.mask) else norm(x[~self.mask, :].ravel(), ord=np.inf)
        return val, infeas

    def prox(self, tau):
        scale = np.zeros(self.c.shape)
        scale[self.mask, :] = 1.0
        scale, c = scale.ravel(), self.c.ravel()

        def op(x):
            x[:] = scale * (x + (-tau) * c)
        return op


class EpigraphInd(Functional):
    """0 if every instance lies in its epigraph, else inf
    (opymize/functionals/epigraph.py:7-54); prox = EpigraphProj."""

    def __init__(self, I, If, J, v, b, conj=None):
        from oracle import epigraph as E
        self.E = E
        self.I, self.If, self.J, self.v, self.b = np.asarray(I, bool), If, J, v, b
        self.shape = (J.shape[0], I.shape[0], v.shape[1] + 1)
        self.size = int(np.prod(self.shape))
        self.conj = EpigraphSupp(I, If, J, v, b, conj=self) if conj is None else conj

    def __call__(self, x):
        return self.E.epigraph_ind(self.I, self.J, self.v, self.b, x.reshape(self.shape))

    def prox(self, tau):
        def op(x):
            y, _ = self.E.epigraph_proj(self.I, self.J, self.v, self.b, x.reshape(self.shape))
            x[:] = y.ravel()
        return op


class EpigraphSupp(Functional):
    """Support function of the epigraphs (opymize/functionals/epigraph.py:56-112);
    with If = None (ndim 1) its value is the convex envelope of each
    instance's points, computed directly."""

    def __init__(self, I, If, J, v, b, conj=None):
        from oracle import epigraph as E
        self.E = E
        self.I, self.If, self.J, self.v, self.b = np.asarray(I, bool), If, J, v, b
        self.shape = (J.shape[0], I.shape[0], v.shape[1] + 1)
        self.size = int(np.prod(self.shape))
        self.conj = EpigraphInd(I, If, J, v, b, conj=self) if conj is None else conj

    def __call__(self, x):
        x = x.reshape(self.shape)
        if self.If is not None:
            off, eqns, chk = self.E.supp_pieces(self.I, self.If, self.J, self.v, self.b)
            return self.E.epigraph_supp(off, eqns, chk, x)
        return self.E.epigraph_supp_envelope(self.I, self.J, self.v, self.b, x)
