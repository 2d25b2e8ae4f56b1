"""Oracle PDHG solver: numpy restatement of the reference's CPU path
(opymize/solvers/pdhg.py, ``use_gpu=False``)."""

import numpy as np
from numpy.linalg import norm

from oracle.linops import normest
from oracle.prox import truncate


class PDHG(object):
    """Chambolle-Pock iteration for min_x G(x) + F(Ax)
    (opymize/solvers/pdhg.py:11-21)."""

    def __init__(self, g, f, A):
        assert A.x_size == g.size
        assert A.y_size == f.size
        self.g, self.f, self.linop = g, f, A
        self.itervars, self.constvars, self.info = {}, {}, {}

    # --- duality gap (pdhg.py:23-44)
    def pd_gap(self):
        i = self.itervars
        obj, inf1 = self.g(i['xk'])
        obj2, inf2 = self.f(i['ygradk'])
        objp, infeasp = obj + obj2, inf1 + inf2
        obj, inf1 = self.g.conj(-i['xgradk'])
        obj2, inf2 = self.f.conj(i['yk'])
        objd, infeasd = -obj - obj2, inf1 + inf2
        return {'objp': objp, 'objd': objd, 'infeasp': infeasp, 'infeasd': infeasd,
                'gap': objp - objd,
                'relgap': (objp - objd) / max(np.spacing(1), abs(objd))}

    @staticmethod
    def residual(a, zk, zkp1, b, zgk, c, zgkp1):
        """(pdhg.py:108-113)"""
        return norm((zk - zkp1) / a - b * zgk + c * zgkp1, ord=2)

    # --- one iteration (pdhg.py:124-187)
    def iteration_step(self):
        v, c = self.itervars, self.constvars
        xk, xkp1, xgradk, xgradkp1 = v['xk'], v['xkp1'], v['xgradk'], v['xgradkp1']
        yk, ykp1, ygradk, ygradkp1 = v['yk'], v['ykp1'], v['ygradk'], v['ygradkp1']
        ygradbk = v['ygradbk']
        theta = c['theta']
        if 'precond' in c:
            tau, sigma = c['xtau'], c['ysigma']
        elif 'adaptive' in c:
            tau, sigma = v['tauk'], v['sigmak']
        else:
            tau, sigma = c['tau'], c['sigma']

        xkp1[:] = xk - tau * xgradk
        self.gprox(xkp1)
        self.linop(xkp1, ygradkp1)
        ygradbk[:] = (1 + theta) * ygradkp1 - theta * ygradk
        ykp1[:] = yk + sigma * ygradbk
        self.fconjprox(ykp1)
        self.linop.adjoint(ykp1, xgradkp1)

        if 'adaptive' in c:
            resp = self.residual(tau, xk, xkp1, 1, xgradk, 1, xgradkp1)
            resd = self.residual(sigma, yk, ykp1, theta, ygradk, theta, ygradkp1)
            gnorm_pk = self.residual(tau, xk, xkp1, 1, xgradk, 0, xgradkp1)
            gnorm_dk = self.residual(sigma, yk, ykp1, theta, ygradk, theta + 1, ygradkp1)
            self.info['resp'], self.info['resd'] = resp, resd
            eps_absp, eps_relp, eps_absd, eps_reld = self.info['epspd']
            epsp = np.sqrt(xk.size) * eps_absp + eps_relp * gnorm_pk
            epsd = np.sqrt(yk.size) * eps_absd + eps_reld * gnorm_dk
            self.info['epsp'], self.info['epsd'] = epsp, epsd
            scale = epsp / epsd
            if resp > scale * resd * c['Delta']:
                v['tauk'] /= 1.0 - v['alphak']
                v['sigmak'] *= 1.0 - v['alphak']
                v['alphak'] *= c['eta']
                self.gprox = self.g.prox(v['tauk'])
                self.fconjprox = self.f.conj.prox(v['sigmak'])
            if resp < scale * resd / c['Delta']:
                v['tauk'] *= 1.0 - v['alphak']
                v['sigmak'] /= 1.0 - v['alphak']
                v['alphak'] *= c['eta']
                self.gprox = self.g.prox(v['tauk'])
                self.fconjprox = self.f.conj.prox(v['sigmak'])

        xk[:], xgradk[:] = xkp1, xgradkp1
        yk[:], ygradk[:] = ykp1, ygradkp1

    # --- step sizes (pdhg.py:189-227)
    def prepare_stepsizes(self, step_bound, step_factor, steps):
        i, c = self.itervars, self.constvars
        if steps == "precond":
            c['precond'] = True
            c['xtau'] = i['xk'].copy()
            c['ysigma'] = i['yk'].copy()
            self.linop.rowwise_lp(c['ysigma'])
            self.linop.adjoint.rowwise_lp(c['xtau'])
            eps = np.spacing(1)
            c['ysigma'][c['ysigma'] > eps] = 1.0 / c['ysigma'][c['ysigma'] > eps]
            c['xtau'][c['xtau'] > eps] = 1.0 / c['xtau'][c['xtau'] > eps]
            self.gprox = self.g.prox(c['xtau'])
            self.fconjprox = self.f.conj.prox(c['ysigma'])
        else:
            bnd = step_bound
            if step_bound is None:
                op_norm, itn = normest(self.linop)
                bnd = truncate(1.0 / op_norm ** 2, 3)
            self.step_bound = bnd
            if steps == "adaptive":
                c['adaptive'] = True
                c['eta'] = 0.95
                c['Delta'] = 1.50
                i['alphak'] = 0.5
                i['sigmak'] = i['tauk'] = np.sqrt(bnd)
                self.gprox = self.g.prox(i['tauk'])
                self.fconjprox = self.f.conj.prox(i['sigmak'])
            else:
                c['sigma'] = np.sqrt(bnd / step_factor)
                c['tau'] = bnd / c['sigma']
                self.gprox = self.g.prox(c['tau'])
                self.fconjprox = self.f.conj.prox(c['sigma'])

    # --- driver (pdhg.py:229-315)
    def solve(self, continue_at=None, precision="double", steps="const",
              step_bound=None, step_factor=1.0, term_pd_gap=1e-5,
              term_pd_res=None, term_maxiter=int(5e4), granularity=5000,
              cbfun=None):
        i, c = self.itervars, self.constvars
        dtype = np.float64 if precision == "double" else np.float32
        i['xk'] = np.zeros(self.g.size, dtype=dtype)
        i['yk'] = np.zeros(self.f.size, dtype=dtype)
        if continue_at is not None:
            i['xk'][:], i['yk'][:] = continue_at
        if term_maxiter == 0:
            self.info['iter'] = 0
            return self.info
        for s in ['xkp1', 'xgradk', 'xgradkp1']:
            i[s] = i['xk'].copy()
        for s in ['ykp1', 'ygradk', 'ygradkp1', 'ygradbk']:
            i[s] = i['yk'].copy()
        self.linop(i['xk'], i['ygradk'])
        self.linop.adjoint(i['yk'], i['xgradk'])

        pd_res_mode = term_pd_res is not None
        if pd_res_mode:
            steps = "adaptive"
            if type(term_pd_res) is not tuple:
                term_pd_res = (term_pd_res,) * 4
            self.info['epspd'] = term_pd_res
        else:
            if type(term_pd_gap) is not tuple:
                term_pd_gap = (term_pd_gap, term_pd_gap)
            if steps == "adaptive":
                self.info['epspd'] = (term_pd_gap[0],) * 4

        c['theta'] = 1.0
        self.prepare_stepsizes(step_bound, step_factor, steps)

        _iter = 0
        while _iter < term_maxiter:
            _iter += 1
            check_step = (_iter % granularity == 0)
            self.iteration_step()
            if check_step:
                self.info['iter'] = _iter
                if pd_res_mode:
                    test_term = (self.info['resp'] < self.info['epsp']
                                 and self.info['resd'] < self.info['epsd'])
                else:
                    self.info.update(self.pd_gap())
                    test_err = np.abs(self.info['relgap']) < term_pd_gap[0]
                    test_infeas = max(self.info['infeasp'], self.info['infeasd']) \
                        < term_pd_gap[1]
                    test_term = test_err and test_infeas
                if cbfun is not None:
                    cbfun(self.state, self.info)
                if test_term:
                    break
        return self.info

    @property
    def state(self):
        return (self.itervars['xk'], self.itervars['yk'])
