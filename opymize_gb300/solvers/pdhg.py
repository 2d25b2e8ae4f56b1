"""PDHG (Chambolle-Pock) solver on the GPU (opymize/solvers/pdhg.py).

``PDHG(g, f, A).solve(...)`` keeps the reference's keyword set and ``info``
dictionary.  Two device paths:

* fused -- G = SSD, F = L1Norms (Frobenius) or HuberL1Norms, A = forward
  GradientOp with D <= 3 and C <= 4: every iteration is two fused passes
  (three with adaptive steps) from libopyx, ``granularity`` iterations plus the
  FP64 gap are captured into one CUDA graph and replayed, and the host reads a
  104-byte info record once per check;
* generic -- any composition of GPU operators and functionals: the
  reference's iteration with the step kernels of libopyx, adaptive steps
  updated on the device, the gap from FP64 device reductions; the
  sublabel-lifted model of tools.lifting runs there as two fused passes per
  iteration (``path == "sublabel"``, solvers/sublabel.py).

``use_gpu=False`` is refused: this package has no CPU path.
"""

import logging
import time

import numpy as np

from opymize_gb300 import _lib
from opymize_gb300.gpuarray import DeviceArray, get_all, stream_ptr, torch
from opymize_gb300.steps import DeviceScalar, step_struct
from opymize_gb300.linear import normest
from opymize_gb300.linear.diff import GradientOp
from opymize_gb300.functionals.quad import SSD
from opymize_gb300.functionals.l1norms import L1Norms, HuberL1Norms
from opymize_gb300.tools import truncate
from opymize_gb300.solvers.sublabel import SublabelPasses
from opymize_gb300.tools.util import GracefulInterruptHandler

INFO_KEYS = ("objp", "objd", "infeasp", "infeasd", "gap", "relgap")


class PDHG(object):
    def __init__(self, g, f, A):
        assert A.x.size == g.x.size
        assert A.y.size == f.x.size
        self.g = g
        self.f = f
        self.linop = A
        self.itervars = {}
        self.constvars = {}
        self.use_gpu = True
        self.info = {}
        self.path = None
        self.graph_replays = 0      # generic path: CUDA graph launches of the last solve

    # ------------------------------------------------------------------ API
    def solve(self, continue_at=None, precision="double", steps="const", step_bound=None,
              step_factor=1.0, term_pd_gap=1e-5, term_pd_res=None, term_maxiter=int(5e4),
              granularity=5000, use_gpu=True, cbfun=None, fused=None, graph=True):
        """Solve to the termination criteria of the reference
        (opymize/solvers/pdhg.py:229-315) on the GPU.

        Extra keywords: ``fused`` (None = automatic, False forces the generic
        path) and ``graph`` (capture chunks of iterations in CUDA graphs, on
        both paths).
        """
        if not use_gpu:
            raise NotImplementedError("opymize_gb300 has no CPU path: use_gpu must be True")
        if steps == "constant":
            steps = "const"
        if steps not in ("const", "adaptive", "precond"):
            raise ValueError("unknown steps rule: %s" % steps)
        dtype = np.float64 if precision == "double" else np.float32
        i, c = self.itervars, self.constvars
        i.clear()
        c.clear()
        self.info = {}
        i['xk'] = self.g.x.new(dtype=dtype)
        i['yk'] = self.f.x.new(dtype=dtype)
        self._zero_start = continue_at is None
        if continue_at is not None:
            i['xk'][:], i['yk'][:] = continue_at
        if term_maxiter == 0:
            self.info['iter'] = 0
            return self.info

        pd_res_mode = term_pd_res is not None
        if pd_res_mode:
            steps = "adaptive"
            if type(term_pd_res) is not tuple:
                term_pd_res = (term_pd_res,) * 4
            else:
                assert len(term_pd_res) == 4
            self.info['epspd'] = term_pd_res
        else:
            if type(term_pd_gap) is not tuple:
                term_pd_gap = (term_pd_gap, term_pd_gap)
            if steps == "adaptive":
                self.info['epspd'] = (term_pd_gap[0],) * 4
        c['theta'] = 1.0

        bnd = None
        if steps != "precond":
            bnd = step_bound
            if step_bound is None:
                logging.info("Estimating optimal step bound...")
                op_norm, itn = normest(self.linop)
                bnd = truncate(1.0 / op_norm ** 2, 3)
        self.step_bound = bnd
        if steps == "adaptive":
            c['adaptive'] = True
            c['eta'], c['Delta'] = 0.95, 1.50
            i['alphak'] = 0.5
            i['sigmak'] = i['tauk'] = np.sqrt(bnd)
        elif steps == "const":
            c['sigma'] = np.sqrt(bnd / step_factor)
            c['tau'] = bnd / c['sigma']
        else:
            c['precond'] = True

        use_fused = self._fusable() if fused is None else (fused and self._fusable())
        self.path = "fused" if use_fused else "generic"
        args = (dtype, steps, term_pd_gap, term_pd_res, pd_res_mode, term_maxiter,
                granularity, cbfun)
        if use_fused:
            self._solve_fused(*args, graph=graph)
        else:
            self._solve_generic(*args, graph=graph, sublabel=fused is not False)
        return self.info

    @property
    def state(self):
        return (self.itervars['xk'], self.itervars['yk'])

    # ------------------------------------------------------------ helpers
    def _fusable(self):
        g, f, A = self.g, self.f, self.linop
        if type(g) is not SSD or type(A) is not GradientOp or A.scheme != "forward":
            return False
        D, C = len(A.imagedims), A.nchannels
        if D > 3 or C > _lib.ROF_MAX_C:
            return False
        if type(f) is L1Norms:
            if f.matrixnorm != "frobenius" and min(f.M) > 1:
                return False
        elif type(f) is not HuberL1Norms:
            return False
        return f.N == int(np.prod(A.imagedims)) and f.M[0] * f.M[1] == D * C

    def _check(self, pd_res_mode, term_pd_gap):
        if pd_res_mode:
            return self.info['resp'] < self.info['epsp'] and self.info['resd'] < self.info['epsd']
        test_err = np.abs(self.info['relgap']) < term_pd_gap[0]
        test_infeas = max(self.info['infeasp'], self.info['infeasd']) < term_pd_gap[1]
        return test_err and test_infeas

    # ------------------------------------------------------------ fused
    def _rof_problem(self, dtype, steps):
        g, f, A = self.g, self.f, self.linop
        c, i = self.constvars, self.itervars
        p = _lib.opyx_rof_problem()
        p.dtype = _lib.OPYX_F32 if dtype == np.float32 else _lib.OPYX_F64
        D, C = len(A.imagedims), A.nchannels
        p.ndim, p.nchannels, p.steps = D, C, _lib.STEPS[steps]
        for t in range(D):
            p.dims[t] = A.imagedims[t]
            p.h[t] = float(A.imageh[t])
        for k in range(C):
            p.weights[k] = float(A.weights[k])
            p.vol[k] = float(g.vol[k])
        p.ssd_shift = float(g.shift)
        p.lbd = float(f.lbd)
        p.huber_alpha = float(f.alph) if isinstance(f, HuberL1Norms) else 0.0
        p.theta = float(c['theta'])
        if steps == "const":
            p.tau, p.sigma = float(c['tau']), float(c['sigma'])
        elif steps == "adaptive":
            p.tau, p.sigma = float(i['tauk']), float(i['sigmak'])
            p.alpha0, p.eta, p.Delta = float(i['alphak']), float(c['eta']), float(c['Delta'])
            for j in range(4):
                p.eps[j] = float(self.info['epspd'][j])
        return p

    def _solve_fused(self, dtype, steps, term_pd_gap, term_pd_res, pd_res_mode, term_maxiter,
                     granularity, cbfun, graph=True):
        lib = _lib.load()
        i = self.itervars
        A = self.linop
        N, C, D = int(np.prod(A.imagedims)), A.nchannels, len(A.imagedims)
        x, y = self._start(dtype)
        xbar = DeviceArray.empty((N * C,), dtype)
        fdev = self.g.f_dev(dtype)
        mask = self.g.mask_dev()
        adaptive = steps == "adaptive"
        xgrad = DeviceArray.empty((N * C,), dtype) if adaptive else None
        gp = DeviceArray.empty((N * C,), dtype) if adaptive else None
        wsb = lib.opyx_rof_workspace_size()
        ws = DeviceArray.zeros(((wsb + 7) // 8,), np.float64)
        # second dual buffer: FP32 iterations then run as one sweep over HBM
        # each (2-D; 3-D with one channel) -- the library falls back to two
        # passes where it cannot
        y2 = DeviceArray.empty((y.size,), dtype) \
            if dtype == np.float32 and (D == 2 or (D == 3 and C == 1)) and not adaptive else None
        p = self._rof_problem(dtype, steps)
        b = _lib.opyx_rof_buffers()
        b.x, b.xbar, b.y, b.f = x.ptr, xbar.ptr, y.ptr, fdev.ptr
        b.mask = None if mask is None else mask.ptr
        b.xgrad = None if xgrad is None else xgrad.ptr
        b.gp = None if gp is None else gp.ptr
        b.ws = ws.ptr
        b.y2 = None if y2 is None else y2.ptr
        self._fused = dict(x=x, y=y, xbar=xbar, f=fdev, mask=mask, xgrad=xgrad, gp=gp, ws=ws,
                           y2=y2, problem=p, buffers=b)
        if pd_res_mode:
            p.term_mode = 2
        else:
            p.term_mode = 1
            p.term_relgap, p.term_infeas = float(term_pd_gap[0]), float(term_pd_gap[1])
        _lib.call("opyx_rof_init", p, b, stream_ptr())
        loop = _FusedLoop(p, b, ws, granularity, graph=graph)
        self._fused['loop'] = loop
        t0 = time.perf_counter()

        def on_check(rec, it):
            self._record_info(rec, it, t0)
            if cbfun is not None:
                self._download(x, y)
                cbfun(self.state, self.info)

        # a callback sees the state of its own check, so it waits for each
        depth = 0 if cbfun is not None else _FusedLoop.DEPTH
        with GracefulInterruptHandler() as hdl:
            it, _ = loop.run(term_maxiter, depth, on_check, lambda: hdl.interrupted)
        self._download(x, y)
        self.info['iter'] = it

    def _record_info(self, rec, it, t0):
        d = dict(zip(_lib.ROF_INFO_FIELDS, (float(v) for v in rec)))
        for k in INFO_KEYS:
            self.info[k] = d[k]
        if 'adaptive' in self.constvars:
            self.itervars['tauk'], self.itervars['sigmak'] = d['tau'], d['sigma']
            self.itervars['alphak'] = d['alpha']
            for k in ("resp", "resd", "epsp", "epsd"):
                self.info[k] = d[k]
        self.info['iter'] = it
        el = time.perf_counter() - t0
        self.info['time_s'] = el
        self.info['it_per_s'] = it / el if el > 0 else float('inf')

    def _start(self, dtype):
        """Device copies of the start point (zeros are filled on the device)."""
        i = self.itervars
        if self._zero_start:
            return (DeviceArray.zeros((i['xk'].size,), dtype),
                    DeviceArray.zeros((i['yk'].size,), dtype))
        return DeviceArray.to_gpu(i['xk'], dtype), DeviceArray.to_gpu(i['yk'], dtype)

    def _download(self, x, y):
        xh, yh = get_all([x, y])
        self.itervars['xk'] = xh.reshape(self.itervars['xk'].shape)
        self.itervars['yk'] = yh.reshape(self.itervars['yk'].shape)

    # ------------------------------------------------------------ generic
    def _solve_generic(self, dtype, steps, term_pd_gap, term_pd_res, pd_res_mode,
                       term_maxiter, granularity, cbfun, graph=True, sublabel=True):
        i, c = self.itervars, self.constvars
        v = {}
        v['xk'], v['yk'] = self._start(dtype)
        for s_ in ('xkp1', 'xgradk', 'xgradkp1'):
            v[s_] = DeviceArray.empty((self.g.x.size,), dtype)
        for s_ in ('ykp1', 'ygradk', 'ygradkp1'):
            v[s_] = DeviceArray.empty((self.f.x.size,), dtype)
        self.linop(v['xk'], v['ygradk'])
        self.linop.adjoint(v['yk'], v['xgradk'])
        self.gpu_itervars = v
        st = None
        if steps == "precond":
            c['xtau'] = DeviceArray.empty((self.g.x.size,), dtype)
            c['ysigma'] = DeviceArray.empty((self.f.x.size,), dtype)
            self.linop.rowwise_lp(c['ysigma'])
            self.linop.adjoint.rowwise_lp(c['xtau'])
            _invert_positive(c['ysigma'])
            _invert_positive(c['xtau'])
            tau, sigma = c['xtau'], c['ysigma']
        elif steps == "adaptive":
            st = _AdaptiveState(i['tauk'], i['sigmak'], i['alphak'], c['eta'], c['Delta'],
                                c['theta'], self.info['epspd'], self.g.x.size, self.f.x.size)
            tau, sigma = st.tau, st.sigma
            self._adaptive = st
        else:
            tau, sigma = c['tau'], c['sigma']
        gprox = self.g.prox(tau)
        fconjprox = self.f.conj.prox(sigma)
        ws = DeviceArray.zeros(((_lib.load().opyx_reduce_workspace_size() + 7) // 8,),
                               np.float64)
        theta = c['theta']
        # the sublabel-lifted model (tools.lifting) iterates as two fused passes
        fsub = None
        if sublabel and st is None and not pd_res_mode:
            try:
                fsub = SublabelPasses.make(self, dtype, steps, tau, sigma, theta)
            except ValueError as err:
                logging.info("sublabel model stays on the generic path: %s", err)
        if fsub is not None:
            self.path = "sublabel"
        self._sublabel = fsub

        def iterate():
            """Launch one iteration (pdhg.py:124-187) and swap the roles of
            the k and k+1 buffers."""
            if fsub is not None:
                fsub.iterate(v)
                swap(1)
                return
            s = stream_ptr()
            _lib.call("opyx_take_step", v['xk'].dcode, v['xk'].size, v['xkp1'].ptr,
                      v['xk'].ptr, -1, step_struct(tau, dtype), v['xgradk'].ptr, s)
            gprox(v['xkp1'])
            self.linop(v['xkp1'], v['ygradkp1'])
            _lib.call("opyx_dual_step", v['yk'].dcode, v['yk'].size, v['ykp1'].ptr,
                      v['yk'].ptr, step_struct(sigma, dtype), theta, v['ygradkp1'].ptr,
                      v['ygradk'].ptr, s)
            fconjprox(v['ykp1'])
            self.linop.adjoint(v['ykp1'], v['xgradkp1'])
            if st is not None:
                _lib.call("opyx_residual_pair", v['xk'].dcode, v['xk'].size,
                          step_struct(st.tau), v['xk'].ptr, v['xkp1'].ptr, 1.0,
                          v['xgradk'].ptr, 1.0, 0.0, v['xgradkp1'].ptr, st.sums_ptr(0),
                          ws.ptr, s)
                _lib.call("opyx_residual_pair", v['yk'].dcode, v['yk'].size,
                          step_struct(st.sigma), v['yk'].ptr, v['ykp1'].ptr, theta,
                          v['ygradk'].ptr, theta, theta + 1.0, v['ygradkp1'].ptr,
                          st.sums_ptr(2), ws.ptr, s)
                _lib.call("opyx_adaptive_update", st.ptr, s)
            swap(1)

        def swap(n):
            if n % 2:
                for a_, b_ in (('xk', 'xkp1'), ('xgradk', 'xgradkp1'), ('yk', 'ykp1'),
                               ('ygradk', 'ygradkp1')):
                    v[a_], v[b_] = v[b_], v[a_]

        # Between checks, iterations run as CUDA graphs of _GENERIC_CHUNK
        # iterations (one of a single iteration for odd remainders), captured
        # on first use for the buffer roles they start from (the parity of
        # the iterations done) and replayed back to back: a replay is one
        # launch where an iteration is a few dozen host calls.  Capturing runs
        # the host code of every iteration it records, so short graphs keep a
        # solve's capture cost at a few iterations.  The first iteration runs
        # eagerly (it creates the operators' lazily uploaded tables); a capture
        # that fails (an operator that reads device data on the host) leaves
        # the solve eager.
        graphs = {}
        capture = bool(graph)
        parity = 0

        def run(n):
            nonlocal parity, capture
            while n > 0:
                m = min(n, _SUBLABEL_CHUNK if fsub is not None else _GENERIC_CHUNK)
                g = graphs.get((m, parity)) if capture else None
                if g is None and capture:
                    saved = dict(v)
                    try:
                        g = graphs[(m, parity)] = _GenericGraph(iterate, m)
                    except Exception as err:          # noqa: BLE001
                        logging.info("generic PDHG path stays eager: %s", err)
                        capture, g = False, None
                    v.update(saved)
                if g is None:
                    iterate()
                    m = 1
                else:
                    g.launch()
                    swap(m)
                    self.graph_replays += 1
                parity ^= m & 1
                n -= m

        self.graph_replays = 0
        t0 = time.perf_counter()
        _iter = 0
        with GracefulInterruptHandler() as hdl:
            while _iter < term_maxiter:
                if _iter == 0:
                    iterate()               # eager: the operators' first calls upload their tables
                    parity, n = 1, 1
                else:
                    nxt = min((_iter // granularity + 1) * granularity, term_maxiter)
                    n = nxt - _iter
                    run(n)
                _iter += n
                check = (_iter % granularity == 0)
                if hdl.interrupted or check:
                    self.info['iter'] = _iter
                    if st is not None:
                        h = st.read()
                        i['tauk'], i['sigmak'], i['alphak'] = h.tau, h.sigma, h.alpha
                        self.info.update(resp=h.resp, resd=h.resd, epsp=h.epsp, epsd=h.epsd)
                    if not pd_res_mode:
                        if fsub is not None:
                            # the fused passes keep no A x_k, A^T y_k: the gap's
                            # operator values come from the generic operators
                            self.linop(v['xk'], v['ygradk'])
                            self.linop.adjoint(v['yk'], v['xgradk'])
                        self.info.update(self.pd_gap())
                    el = time.perf_counter() - t0
                    self.info['time_s'], self.info['it_per_s'] = el, _iter / el
                    if cbfun is not None:
                        self._download(v['xk'], v['yk'])
                        cbfun(self.state, self.info)
                    if self._check(pd_res_mode, term_pd_gap) or hdl.interrupted:
                        break
        self._download(v['xk'], v['yk'])
        self.info['iter'] = _iter

    def pd_gap(self):
        """Primal-dual gap of the current device iterate (pdhg.py:23-44),
        every functional reduced in FP64 on the device."""
        v = self.gpu_itervars
        obj, inf1 = self.g(v['xk'])
        obj2, inf2 = self.f(v['ygradk'])
        objp, infeasp = obj + obj2, inf1 + inf2
        neg = v['xgradk'].copy()
        neg *= -1.0
        obj, inf1 = self.g.conj(neg)
        obj2, inf2 = self.f.conj(v['yk'])
        objd, infeasd = -obj - obj2, inf1 + inf2
        return {'objp': objp, 'objd': objd, 'infeasp': infeasp, 'infeasd': infeasd,
                'gap': objp - objd,
                'relgap': (objp - objd) / max(np.spacing(1), abs(objd))}


def _invert_positive(a):
    """a_i <- 1/a_i where a_i > eps, else unchanged (pdhg.py:197-198)."""
    _lib.call("opyx_recip_positive", a.dcode, a.size, a.ptr, float(np.spacing(1)), stream_ptr())


class _AdaptiveState(object):
    """Device record of the adaptive rule (opyx_adaptive_state)."""

    def __init__(self, tau, sigma, alpha, eta, Delta, theta, eps, xsize, ysize):
        h = _lib.opyx_adaptive_state()
        h.tau, h.sigma, h.alpha, h.eta, h.Delta, h.theta = tau, sigma, alpha, eta, Delta, theta
        for j in range(4):
            h.eps[j] = eps[j]
        h.xsize, h.ysize = float(xsize), float(ysize)
        raw = np.frombuffer(bytes(h), dtype=np.float64).copy()
        self.dev = DeviceArray.to_gpu(raw)
        self.ptr = self.dev.ptr
        self.tau = DeviceScalar(self.ptr + _lib.opyx_adaptive_state.tau.offset, self.dev, tau)
        self.sigma = DeviceScalar(self.ptr + _lib.opyx_adaptive_state.sigma.offset, self.dev,
                                  sigma)

    def sums_ptr(self, j):
        return self.ptr + _lib.opyx_adaptive_state.sums.offset + 8 * j

    def read(self):
        raw = self.dev.get()
        h = _lib.opyx_adaptive_state.from_buffer_copy(raw.tobytes())
        self.tau.host_value, self.sigma.host_value = h.tau, h.sigma
        return h


class _FusedLoop(object):
    """Fused iterations queued ahead of their checks.

    A check is the gap kernel after `granularity` iterations, then an
    asynchronous copy of the info record into a pinned host slot and an event.
    The host reads a record only when `depth` newer ones are queued behind it,
    so the GPU does not idle on the host round trip.  The device-side stop test
    (term_mode of the problem) makes every kernel queued after the passing
    check return at once, so state, info and iteration count equal those of a
    loop that waits at every check, as the reference's does
    (opymize/solvers/pdhg.py:285-313).  With single sweeps and no per-check
    callback, a check is queued with the next chunk's iterations
    (opyx_rof_gap_iterate: the first sweep computes it from the rows it loads)
    and its record copied after that chunk; the record then arrives one chunk
    later, so one fewer newer record is waited for.  Chunks of a kind queued
    more than EAGER_USES times are replayed as CUDA graphs (one per kind and
    length).  `run` must follow opyx_rof_init, which clears the check counter.
    """
    DEPTH = 2
    # a chunk kind is queued by direct launches this many times before it is
    # captured: a capture costs ~0.25 ms on the host and a replay saves
    # ~7-9 us of GPU time per 10-iteration chunk against direct (chained)
    # launches; a kind met once per solve (the first chunk) is captured from
    # the third solve on a reused loop.  (16 direct uses measured slower on a
    # reused loop: 2.26 against 2.18 ms for the 30-iteration 2048x2048x3 solve,
    # whose first chunk then stayed direct and started behind the host.)
    EAGER_USES = 2

    def __init__(self, p, b, ws, granularity, graph=True):
        self.p, self.b, self.gran, self.use_graph = p, b, int(granularity), graph
        off = _lib.load().opyx_rof_info_offset() // 8
        self.info_dev = ws.t[off:off + len(_lib.ROF_INFO_FIELDS)]
        self.graphs = {}
        self.uses = {}         # chunks queued per kind
        self.host = None
        self.launches = 0      # kernel launches queued so far
        self.sweeps = bool(_lib.load().opyx_rof_uses_sweep(p, b))
        # 2-D sweeps compute a check in their first sweep (3-D: the gap kernel)
        self.fused_gap = self.sweeps and p.ndim == 2

    def chunk(self, n, check, first=False):
        """n iterations; `check`: the gap after them; `first`: the gap of the
        state before them, fused into their first sweep (n >= 2)."""
        key = (n, check, first)
        uses = self.uses.get(key, 0)
        self.uses[key] = uses + 1
        if n and self.use_graph and uses >= self.EAGER_USES:
            g = self.graphs.get(key)
            if g is None:
                g = self.graphs[key] = _RofGraph(self.p, self.b, n, check, first)
            g.launch()
        else:
            _RofGraph.queue(self.p, self.b, n, check, first, stream_ptr())
        p = self.p
        if self.sweeps:
            kernels = (n // 2) * 2 + (n % 2) * 2       # sweeps; an odd count ends two-pass
        else:
            kernels = n * (3 if p.steps == _lib.STEPS["adaptive"] else 2)
        self.launches += kernels + (1 if check else 0)

    def run(self, maxiter, depth=DEPTH, on_check=None, interrupted=None):
        """Iterate until the stop test passes at a check, `maxiter` iterations
        are done or `interrupted()` is true (then the current chunk ends with a
        check, as the reference's interrupt does).  Calls on_check(record,
        iteration) for every check that ran, in order; returns (iterations
        done, last record read)."""
        t = torch()
        nrec = len(_lib.ROF_INFO_FIELDS)
        if self.host is None or self.host.shape[0] < depth + 1:
            self.host = t.empty((depth + 1, nrec), dtype=t.float64, pin_memory=True)
        fuse = self.fused_gap and depth > 0
        wait_depth = depth - 1 if fuse else depth
        names = _lib.ROF_INFO_FIELDS
        i_checks, i_done, i_fault = names.index("checks"), names.index("done"), names.index("fault")
        pending = []          # (event, slot) of queued checks, oldest first
        check_iters = []      # iteration count at each queued check
        state = {"rec": None, "checks": 0}

        def read_oldest():
            ev, slot = pending.pop(0)
            ev.synchronize()
            rec = self.host[slot].numpy().copy()
            if rec[i_fault] != 0.0:
                raise _lib.OpyxError("fused PDHG iteration", _lib.OPYX_ERR_LAUNCH,
                                     "a kernel gave up waiting for its own copies")
            c = int(rec[i_checks])
            if c > state["checks"]:      # checks after the stop returned at once
                state["checks"], state["rec"] = c, rec
                if on_check is not None:
                    on_check(rec, check_iters[c - 1])
            return rec[i_done] != 0.0

        def queue_record(at):
            slot = len(check_iters) % (depth + 1)
            check_iters.append(at)
            self.host[slot].copy_(self.info_dev, non_blocking=True)
            ev = t.cuda.Event()
            ev.record()
            pending.append((ev, slot))
            return read_oldest() if len(pending) > wait_depth else False

        it, done = 0, False
        owed = None           # iteration of a check not queued yet (fused mode)
        while it < maxiter and not done:
            n = min(self.gran - (it % self.gran), maxiter - it)
            first = owed is not None and n >= 2
            if owed is not None and not first:
                self.chunk(0, True)
                done = queue_record(owed)
                owed = None
                if done:
                    break
            it += n
            stop = interrupted is not None and bool(interrupted())
            check = it % self.gran == 0 or stop
            self.chunk(n, check and not fuse, first)
            if first:
                done = queue_record(owed) or done
                owed = None
            if check:
                if fuse:
                    owed = it
                else:
                    done = queue_record(it) or done
            if stop:
                break
        if owed is not None and not done:
            self.chunk(0, True)
            queue_record(owed)
        while pending:
            done = read_oldest() or done
        rec = state["rec"]
        if rec is not None and rec[i_done] != 0.0:
            it = check_iters[state["checks"] - 1]
        else:
            t.cuda.current_stream().synchronize()
        return it, rec


# iterations per CUDA graph of the generic path (even: a replay keeps the
# buffer roles)
_GENERIC_CHUNK = 2
_SUBLABEL_CHUNK = 16    # two launches per fused sublabel iteration: longer graphs are cheap


class _GenericGraph(object):
    """`n` generic iterations captured once into a CUDA graph on a private
    capture stream (no host synchronisation may happen inside: the
    iteration's launches only) and replayed on the current stream."""

    def __init__(self, iterate, n):
        t = torch()
        self.stream = t.cuda.Stream()
        self.graph = t.cuda.CUDAGraph()
        self.stream.wait_stream(t.cuda.current_stream())
        with t.cuda.graph(self.graph, stream=self.stream):
            for _ in range(n):
                iterate()
        t.cuda.current_stream().wait_stream(self.stream)

    def launch(self):
        self.graph.replay()


class _RofGraph(object):
    """A chunk of fused iterations with its checks -- `first`: the gap of the
    state before them fused into their first sweep; `check`: the gap kernel
    after them -- captured once into a CUDA graph (on a private capture
    stream) and replayed on the current stream."""

    def __init__(self, p, b, n, check=True, first=False):
        t = torch()
        self.stream = t.cuda.Stream()
        self.graph = t.cuda.CUDAGraph()
        self.stream.wait_stream(t.cuda.current_stream())
        with t.cuda.graph(self.graph, stream=self.stream):
            self.queue(p, b, n, check, first, t.cuda.current_stream().cuda_stream)

    @staticmethod
    def queue(p, b, n, check, first, s):
        if first:
            _lib.call("opyx_rof_gap_iterate", p, b, n, s)
        elif n:
            _lib.call("opyx_rof_iterate", p, b, n, s)
        if check:
            _lib.call("opyx_rof_gap", p, b, s)

    def launch(self):
        self.graph.replay()
