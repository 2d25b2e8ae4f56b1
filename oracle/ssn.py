"""CPU oracle of the reference's semismooth Newton solver for ROF-type
problems (SSD data term, Frobenius L1 norms, a linear operator with a
sparse matrix) -- TEST INFRASTRUCTURE ONLY, like the rest of ``oracle/``.

Restates opymize/solvers/semismooth_newton.py (armijo :14-47, SymRegOp
:49-75, CG_solve :77-117, SemismoothNewtonSystem and its adjoint :184-248,
SemismoothNewton :250-427) and the Jacobians of the two prox maps it
differentiates: the SSD prox is the affine map a*(x + b*f) with Jacobian
diag(a) (opymize/functionals/quad.py:45-55, opymize/operators/affine.py:
85-146), and the projection onto the Frobenius lbd-balls has the Jacobian of
``L12ProjJacobian`` (opymize/operators/proj.py:228-276): the identity on
groups inside the ball, lbd/|x| (I - n n^T), n = x/|x|, outside.  Pinned to
``tests/golden/ssn.npz`` (tests/golden/make_ssn_golden.py runs the
reference's own solver).
"""

import numpy as np

from oracle.linops import normest
from oracle.prox import truncate


def armijo(fun, xk, xkp1, p, p_gradf, fun_xk, eta=0.5, nu=0.9):
    """Backtracking: the first alpha = eta^j with f(xk + alpha p) <=
    f(xk) + alpha nu <p, Df> (semismooth_newton.py:14-47)."""
    if p_gradf >= 0:
        raise RuntimeError("Armijo: not a descent direction")
    alpha = 1.0
    while True:
        xkp1[:] = xk + alpha * p
        f_new = fun(xkp1)
        if f_new <= fun_xk + alpha * nu * p_gradf:
            return f_new, alpha
        alpha *= eta
        if alpha < 1e-10:
            raise RuntimeError("Armijo: not a descent direction")


class FrobeniusProjJacobian(object):
    """Jacobian of the projection onto the lbd-balls at the last projected
    point (proj.py:228-276): y = s_i (x_i - <n_i, x_i> n_i) with n_i = 0, s_i = 1
    inside the ball."""

    def __init__(self, N, M):
        self.N, self.M = N, M
        self.n = np.zeros((N, M))
        self.s = np.ones(N)

    def apply(self, x):
        x = x.reshape(self.N, self.M)
        d = np.einsum('ik,ik->i', self.n, x)
        return ((self.n * (-d)[:, None] + x) * self.s[:, None]).ravel()


def project_with_jacobian(x, N, M, lbd, jac=None):
    """Project groups of M values onto the Frobenius lbd-ball in place
    (proj.py:87-108); with ``jac``, record its Jacobian data."""
    xv = x.reshape(N, M)
    nrm = np.sqrt(np.einsum('ik,ik->i', xv, xv))
    ext = nrm > lbd
    rec = np.where(ext, 1.0 / np.where(ext, nrm, 1.0), 0.0)
    if jac is not None:
        jac.n[:] = 0.0
        jac.n[ext] = xv[ext] * rec[ext, None]
        jac.s[:] = 1.0
        jac.s[ext] = lbd * rec[ext]
    xv[ext] *= rec[ext, None]
    xv[ext] *= lbd


class SemismoothNewton(object):
    """min_x 0.5 |x - f|^2 + lbd sum_i |(A x)_i|_F as the root of the
    prox-residual map R(x, y) = (x - prox_tau G(x - tau A^T y),
    y - prox_sigma F*(y + sigma A x)), solved by Newton steps on the
    Levenberg-Marquardt-regularised normal equations with CG and Armijo
    backtracking (semismooth_newton.py:250-427)."""

    def __init__(self, f, lbd, A, M):
        self.f = np.asarray(f, float).ravel()
        self.lbd_f = lbd
        self.A = A
        self.nx = A.x_size
        self.ny = A.y_size
        self.N = self.ny // M
        self.M = M
        self.jac = FrobeniusProjJacobian(self.N, M)

    # -- the prox maps and their Jacobians
    def _gprox(self, x):
        x[:] = self.a * (x + self.tau * self.f)

    def _res(self, xy, out, subdiff=False):
        x, y = xy[:self.nx], xy[self.nx:]
        xg, yg = out[:self.nx], out[self.nx:]
        Aty = np.zeros(self.nx)
        self.A.adjoint(y, Aty)
        xg[:] = x - self.tau * Aty
        self._gprox(xg)
        xg[:] = x - xg
        Ax = np.zeros(self.ny)
        self.A(x, Ax)
        yg[:] = y + self.sigma * Ax
        project_with_jacobian(yg, self.N, self.M, self.lbd_f, self.jac if subdiff else None)
        yg[:] = y - yg
        return 0.5 * np.dot(out, out)

    # -- the Newton system [[I - K, tau K A^T], [-sigma H A, I - H]] and its adjoint
    def _K(self, v):
        return self.a * v

    def _H(self, v):
        return self.jac.apply(v)

    def _M(self, v):
        x1, x2 = v[:self.nx], v[self.nx:]
        out = np.zeros_like(v)
        t = np.zeros(self.nx)
        self.A.adjoint(x2, t)
        y1 = x1 + self.tau * self._K(t)
        out[:self.nx] = y1 - self._K(x1)
        t2 = np.zeros(self.ny)
        self.A(x1, t2)
        y2 = x2 - self.sigma * self._H(t2)
        out[self.nx:] = y2 - self._H(x2)
        return out

    def _MT(self, v):
        x1, x2 = v[:self.nx], v[self.nx:]
        out = np.zeros_like(v)
        t = np.zeros(self.nx)
        self.A.adjoint(self._H(x2), t)
        out[:self.nx] = x1 - self.sigma * t - self._K(x1)
        t2 = np.zeros(self.ny)
        self.A(self._K(x1), t2)
        out[self.nx:] = x2 + self.tau * t2 - self._H(x2)
        return out

    def _cg(self, b, xk, lam, tol, maxiter=1000):
        """(M^T M + lam I) x = -M^T b by CG (semismooth_newton.py:77-117)."""
        op = lambda v: self._MT(self._M(v)) + lam * v
        rk = -(op(xk) + self._MT(b))
        dk = rk.copy()
        for k in range(maxiter + 1):
            z = op(dk)
            alpha = np.dot(rk, rk) / np.dot(dk, z)
            xk += alpha * dk
            rkp1 = rk - alpha * z
            beta = np.dot(rkp1, rkp1) / np.dot(rk, rk)
            dk = rkp1 + beta * dk
            rk = rkp1
            if k % 2 == 0 and np.dot(rkp1, rkp1) < tol:
                break

    def solve(self, xy0, maxiter, seed=1):
        np.random.seed(seed)
        op_norm, _ = normest(self.A)
        bnd = truncate(1.0 / op_norm ** 2, 3) * 1.25
        self.sigma = np.sqrt(bnd)
        self.tau = bnd / self.sigma
        self.a = 1.0 / (1.0 + self.tau)
        lam, drop, boost = 1.0, 0.1, 5.0
        xy = np.array(xy0, dtype=float)
        res = np.zeros_like(xy)
        dk = xy.copy()            # CG starts from the start point, then from its last solution
        xyn = np.zeros_like(xy)
        for _ in range(maxiter):
            r2 = self._res(xy, res, subdiff=True)
            self._cg(res, dk, lam, r2)
            Md = self._M(dk)
            p_gradf = np.dot(res, Md)
            new, alpha = armijo(lambda v: self._res(v, res), xy, xyn, dk, p_gradf, r2)
            Md2 = 0.5 * np.dot(Md, Md)
            rho = (new - r2) / (alpha * p_gradf + alpha ** 2 * Md2)
            if rho > 0.75:
                lam *= drop
            elif rho < 0.25:
                lam *= boost
            xy[:] = xyn
        self.lam = lam
        return xy
