"""Semismooth Newton solver (opymize/solvers/semismooth_newton.py) on the
device.

The saddle point of min_x G(x) + F(Ax) is the root of the prox residual

    R(x, y) = (x - prox_tau G(x - tau A^T y), y - prox_sigma F*(y + sigma A x)).

Each Newton step linearises R with the Jacobians K of prox_tau G and H of
prox_sigma F* (the operators' ``jacobian=True`` calls: a ScaleOp for the SSD
prox, ``L12ProjJacobian`` for the Frobenius-ball projection), solves the
Levenberg-Marquardt-regularised normal equations (M^T M + lbd I) d = -M^T R
with M = [[I - K, tau K A^T], [-sigma H A, I - H]] by conjugate gradients,
and takes an Armijo-backtracked step; lbd shrinks or grows with the ratio of
actual to predicted decrease (semismooth_newton.py:293-331).  The reference
runs it on the CPU with numpy; here every vector lives in device memory and
every operation is a libopyx kernel (operators, Jacobians, axpby, FP64 dot
products).  The scipy-based variants of the reference (``scipy_solve`` with
lsqr/bicgstab, ``SemismoothQuasinewton`` with ``scipy.optimize.broyden1``)
are host algorithms and are not provided.
"""

import logging
import time

import numpy as np

from opymize_gb300 import Variable, LinOp, _lib
from opymize_gb300.gpuarray import DeviceArray, dot, stream_ptr
from opymize_gb300.linear import normest
from opymize_gb300.tools import truncate
from opymize_gb300.tools.util import GracefulInterruptHandler


def _axpby(a, x, b, y):
    """y = a*x + b*y (device)."""
    _lib.call("opyx_axpby", y.dcode, y.size, float(a), x.ptr, float(b), y.ptr, stream_ptr())


def armijo(fun, xk, xkp1, p, p_gradf, fun_xk, eta=0.5, nu=0.9):
    """Backtracking line search (semismooth_newton.py:14-47): the first
    alpha = eta^j with fun(xk + alpha p) <= fun_xk + alpha nu p_gradf; sets
    xkp1 = xk + alpha p and returns (fun(xkp1), alpha)."""
    if p_gradf >= 0:
        raise Exception("Armijo: Not a descent direction!")
    alpha = 1.0
    while True:
        xkp1.assign(xk)
        xkp1.axpy(alpha, p)
        f_xkp1 = fun(xkp1)
        if f_xkp1 <= fun_xk + alpha * nu * p_gradf:
            break
        alpha *= eta
        if alpha < 1e-10:
            raise Exception("Armijo: Not a descent direction!")
    return f_xkp1, alpha


class SymRegOp(LinOp):
    """M^T M + lbd I for the given M (semismooth_newton.py:49-75)."""

    def __init__(self, M, lbd=1.0, tmp=None):
        LinOp.__init__(self)
        self.M, self.lbd = M, lbd
        self.x = self.y = M.x
        self.tmp = tmp
        self.adjoint = self

    def _call_gpu(self, x, y=None, add=False):
        assert y is not None
        self.M(x, self.tmp)
        self.M.adjoint(self.tmp, y, add=add)
        if self.lbd != 0:
            y.axpy(self.lbd, x)


def CG_solve(A, b, xk, lbd=0, tmpvars=None, maxiter=int(1e3), tol=1e-5):
    """Solve A x + b = 0 as (A^T A + lbd I) x = -A^T b by conjugate gradients,
    starting from and writing to xk (semismooth_newton.py:77-117); every
    inner product is an FP64 device reduction."""
    if tmpvars is not None:
        rk, rkp1, z, dk = tmpvars
    else:
        rk, rkp1, z, dk = [xk.copy() for _ in range(4)]
    ATb = z
    modA = SymRegOp(A, lbd=lbd, tmp=rkp1)
    A.adjoint(b, ATb)
    modA(xk, rk)
    rk.axpy(1.0, ATb)
    rk *= -1.0
    dk.assign(rk)
    rr = dot(rk, rk)
    for k in range(maxiter + 1):
        modA(dk, z)
        alpha = rr / dot(dk, z)
        xk.axpy(alpha, dk)
        rkp1.assign(rk)
        rkp1.axpy(-alpha, z)
        rr1 = dot(rkp1, rkp1)
        beta = rr1 / rr
        _axpby(1.0, rkp1, beta, dk)
        rk.assign(rkp1)
        rr = rr1
        if k % 2 == 0:
            logging.debug("CG #{:03d}: {: 9.6g}".format(k, rr1))
            if rr1 < tol:
                break
    return k + 1


class SemismoothNewtonSystem(LinOp):
    """[[I - K, tau K A^T], [-sigma H A, I - H]] (semismooth_newton.py:184-219)."""

    def __init__(self, A, tau, sigma, dtype=np.float64):
        LinOp.__init__(self)
        self.A, self.tau, self.sigma = A, tau, sigma
        self.x = Variable((A.x.size,), (A.y.size,))
        self.y = self.x
        self.xtmp = DeviceArray.empty((self.x.size,), dtype)
        self.K = self.H = None
        self.adjoint = SemismoothNewtonSystemAdjoint(self)

    def _call_gpu(self, x, y=None, add=False):
        assert y is not None and not add
        x1tmp, x2tmp = self.x.vars(self.xtmp)
        x1, x2 = self.x.vars(x)
        y1, y2 = self.y.vars(y)
        self.A.adjoint(x2, x1tmp)
        self.K(x1tmp, y1)
        _axpby(1.0, x1, self.tau, y1)        # y1 = x1 + tau K A^T x2
        self.K(x1, x1tmp)
        y1.axpy(-1.0, x1tmp)
        self.A(x1, x2tmp)
        self.H(x2tmp, y2)
        _axpby(1.0, x2, -self.sigma, y2)     # y2 = x2 - sigma H A x1
        self.H(x2, x2tmp)
        y2.axpy(-1.0, x2tmp)


class SemismoothNewtonSystemAdjoint(LinOp):
    """Adjoint of a SemismoothNewtonSystem (semismooth_newton.py:221-248)."""

    def __init__(self, M):
        LinOp.__init__(self)
        self.M = M
        self.x, self.y = M.y, M.x
        self.adjoint = M

    def _call_gpu(self, x, y=None, add=False):
        assert y is not None and not add
        M = self.M
        x1tmp, x2tmp = self.x.vars(M.xtmp)
        x1, x2 = self.x.vars(x)
        y1, y2 = self.y.vars(y)
        M.H.adjoint(x2, x2tmp)
        M.A.adjoint(x2tmp, y1)
        _axpby(1.0, x1, -M.sigma, y1)        # y1 = x1 - sigma A^T H^T x2
        M.K.adjoint(x1, x1tmp)
        y1.axpy(-1.0, x1tmp)
        M.K.adjoint(x1, x1tmp)
        M.A(x1tmp, y2)
        _axpby(1.0, x2, M.tau, y2)           # y2 = x2 + tau A K^T x1
        M.H.adjoint(x2, x2tmp)
        y2.axpy(-1.0, x2tmp)


class SemismoothNewton(object):
    """SemismoothNewton(g, f, A).solve(continue_at, granularity, term_relgap,
    term_infeas, term_maxiter) as the reference (semismooth_newton.py:
    250-427), FP64 on the device.  ``continue_at``: the concatenated (x, y)
    or a pair; ``state``: (x, y) on the host."""

    def __init__(self, g, f, A):
        self.g, self.f, self.linop = g, f, A
        self.xy = Variable((g.x.size,), (f.x.size,))
        self.itervars = {'xyk': self.xy.new()}
        self.constvars = {'tau': 1.0, 'sigma': 1.0}
        self.info = {}
        self.cg_iters = []

    def obj_primal(self, x, Ax):
        obj, infeas = self.g(x)
        obj2, infeas2 = self.f(Ax)
        return obj + obj2, infeas + infeas2

    def obj_dual(self, ATy, y):
        neg = ATy.copy()
        neg *= -1.0
        obj, infeas = self.g.conj(neg)
        obj2, infeas2 = self.f.conj(y)
        return -obj - obj2, infeas + infeas2

    def res(self, xy, xyres, subdiff=False, norm=True):
        c = self.constvars
        x, y = self.xy.vars(xy)
        xgrad, ygrad = self.xy.vars(xyres)
        # xgrad = x - prox[tau g](x - tau A^T y)
        self.linop.adjoint(y, xgrad)
        _axpby(1.0, x, -c['tau'], xgrad)
        K = self.gprox(xgrad, jacobian=subdiff)
        _axpby(1.0, x, -1.0, xgrad)
        # ygrad = y - prox[sigma f*](y + sigma A x)
        self.linop(x, ygrad)
        _axpby(1.0, y, c['sigma'], ygrad)
        H = self.fconjprox(ygrad, jacobian=subdiff)
        _axpby(1.0, y, -1.0, ygrad)
        if subdiff:
            self.M.K, self.M.H = K, H
        if norm:
            return 0.5 * dot(xyres, xyres)

    def iteration_step(self, _iter):
        v = self.v
        res_normsq = self.res(v['xyk'], v['xyres'], subdiff=True)
        cg = CG_solve(self.M, v['xyres'], v['dk'], lbd=self.lbd,
                      tmpvars=(v['cg_rk'], v['cg_rkp1'], v['xytmp'], v['cg_dk']), tol=res_normsq)
        self.cg_iters.append(cg)
        self.M(v['dk'], v['xytmp'])
        p_gradf = dot(v['xyres'], v['xytmp'])
        fun = lambda xy: self.res(xy, v['xyres'], subdiff=False)
        new_normsq, alpha = armijo(fun, v['xyk'], v['xykp1'], v['dk'], p_gradf, res_normsq)
        # lbd update of "Distributed Newton Methods for Deep Neural Networks"
        # (C.-C. Wang et al., arXiv:1802.00130), as semismooth_newton.py:318-328
        Md_normsq = 0.5 * dot(v['xytmp'], v['xytmp'])
        rho = (new_normsq - res_normsq) / (alpha * p_gradf + alpha ** 2 * Md_normsq)
        if rho > 0.75:
            self.lbd *= self.lbd_drop
        elif rho < 0.25:
            self.lbd *= self.lbd_boost
        logging.debug("#{:6d}: alpha = {: 9.6g}, rho = {: 9.6g}, lbd = {: 9.6g}, normsq = {: 9.6g}"
                      .format(_iter, alpha, rho, self.lbd, res_normsq))
        v['xyk'].assign(v['xykp1'])

    def prepare_stepsizes(self, step_factor=1.0):
        c = self.constvars
        logging.info("Estimating optimal step bound...")
        op_norm, itn = normest(self.linop)
        bnd = truncate(1.0 / op_norm ** 2, 3) * 1.25    # < 1/|K|^2, boosted
        c['sigma'] = np.sqrt(bnd / step_factor)
        c['tau'] = bnd / c['sigma']
        self.gprox = self.g.prox(c['tau'])
        self.fconjprox = self.f.conj.prox(c['sigma'])
        self.M = SemismoothNewtonSystem(self.linop, c['tau'], c['sigma'])
        self.lbd = 1.0
        self.lbd_drop = 0.1
        self.lbd_boost = 5.0

    def solve(self, continue_at=None, granularity=50, term_relgap=1e-5, term_infeas=None,
              term_maxiter=int(5e2), use_gpu=True, precision="double"):
        if not use_gpu:
            raise NotImplementedError("this build has no CPU path")
        if precision != "double":
            raise ValueError("the semismooth Newton solver runs in double precision")
        i = self.itervars
        if continue_at is not None:
            if isinstance(continue_at, (tuple, list)):
                continue_at = np.concatenate([np.asarray(a, dtype=np.float64).ravel()
                                              for a in continue_at])
            i['xyk'][:] = np.asarray(continue_at, dtype=np.float64).ravel()
        v = {'xyk': DeviceArray.to_gpu(i['xyk'], np.float64)}
        for k in ('xykp1', 'xyres', 'dk', 'xytmp', 'cg_dk', 'cg_rk', 'cg_rkp1'):
            v[k] = v['xyk'].copy()
        self.v = v
        xk, yk = self.xy.vars(v['xyk'])
        xkp1, ykp1 = self.xy.vars(v['xykp1'])
        self.prepare_stepsizes()
        if term_infeas is None:
            term_infeas = term_relgap
        obj_p = obj_d = infeas_p = infeas_d = relgap = 0.
        logging.info("Solving (steps<%d)..." % term_maxiter)
        t0 = time.perf_counter()
        with GracefulInterruptHandler() as hdl:
            _iter = 0
            while _iter < term_maxiter:
                self.iteration_step(_iter)
                _iter += 1
                if hdl.interrupted or _iter % granularity == 0:
                    if hdl.interrupted:
                        print("Interrupt (SIGINT) at iter=%d" % _iter)
                    self.linop(xk, ykp1)
                    self.linop.adjoint(yk, xkp1)
                    obj_p, infeas_p = self.obj_primal(xk, ykp1)
                    obj_d, infeas_d = self.obj_dual(xkp1, yk)
                    relgap = (obj_p - obj_d) / max(np.spacing(1), obj_d)
                    logging.info("#{:6d}: objp = {: 9.6g} ({: 9.6g}), objd = {: 9.6g} ({: 9.6g}), "
                                 "gap = {: 9.6g}, relgap = {: 9.6g} ".format(
                                     _iter, obj_p, infeas_p, obj_d, infeas_d, obj_p - obj_d, relgap))
                    if np.abs(relgap) < term_relgap and max(infeas_p, infeas_d) < term_infeas:
                        break
                    if hdl.interrupted:
                        break
        i['xyk'] = v['xyk'].get()
        self.info = {'objp': obj_p, 'objd': obj_d, 'infeasp': infeas_p, 'infeasd': infeas_d,
                     'relgap': relgap, 'iter': _iter, 'time_s': time.perf_counter() - t0}
        return self.info

    @property
    def state(self):
        return self.xy.vars(self.itervars['xyk'])
