"""Host logic of the fused solve's check loop (solvers.pdhg._FusedLoop) on
the CPU: the device is simulated by a record of iterations, checks and the
stop flag with the semantics of the C ABI (opyx_rof_iterate, opyx_rof_gap,
opyx_rof_gap_iterate: every launch after a passing check returns at once).
The loop must stop at the first check of the reference's schedule that
passes (opymize/solvers/pdhg.py:285-313: a check after every `granularity`
iterations, and one at an interrupt), return that iteration, leave the state
at it, and report each check in order -- whether checks run as the gap
kernel after a chunk or inside the next chunk's first sweep."""

import types

import numpy as np
import pytest
import torch as T

from opymize_gb300 import _lib
from opymize_gb300.solvers import pdhg

FIELDS = _lib.ROF_INFO_FIELDS
NREC = len(FIELDS)


class Device(object):
    """relgap(it) = 1 / (1 + it): the stop test passes once it >= 1/tol."""

    def __init__(self, tol):
        self.tol, self.it, self.done, self.checks = tol, 0, False, 0
        self.info = T.zeros(NREC, dtype=T.float64)
        self.ops = []

    def gap(self):
        self.ops.append(("gap", self.it))
        if self.done:
            return
        self.checks += 1
        relgap = 1.0 / (1.0 + self.it)
        self.info[FIELDS.index("checks")] = float(self.checks)
        self.info[FIELDS.index("relgap")] = relgap
        if relgap < self.tol:
            self.done = True
            self.info[FIELDS.index("done")] = 1.0

    def iterate(self, n):
        if not self.done:
            self.it += n


def fake_env(monkeypatch, dev, sweeps):
    class Graph(object):
        made = []

        def __init__(self, p, b, n, check=True, first=False):
            self.args = (p, b, n, check, first)
            Graph.made.append((n, check, first))

        @staticmethod
        def queue(p, b, n, check, first, s):
            if first:
                dev.gap()
                dev.iterate(n)
            elif n:
                dev.iterate(n)
            if check:
                dev.gap()

        def launch(self):
            self.queue(*self.args, 0)

    class Event(object):
        def record(self):
            pass

        def synchronize(self):
            pass

    cuda = types.SimpleNamespace(
        Event=Event, current_stream=lambda: types.SimpleNamespace(synchronize=lambda: None))
    fake_torch = types.SimpleNamespace(
        float64=T.float64, cuda=cuda,
        empty=lambda shape, dtype, pin_memory=False: T.empty(shape, dtype=dtype))
    lib = types.SimpleNamespace(opyx_rof_info_offset=lambda: 0,
                                opyx_rof_uses_sweep=lambda p, b: int(sweeps))
    fake_lib = types.SimpleNamespace(load=lambda: lib, ROF_INFO_FIELDS=FIELDS, STEPS=_lib.STEPS,
                                     OpyxError=_lib.OpyxError, OPYX_ERR_LAUNCH=_lib.OPYX_ERR_LAUNCH)
    monkeypatch.setattr(pdhg, "torch", lambda: fake_torch)
    monkeypatch.setattr(pdhg, "stream_ptr", lambda: 0)
    monkeypatch.setattr(pdhg, "_RofGraph", Graph)
    monkeypatch.setattr(pdhg, "_lib", fake_lib)
    return Graph


def expected(maxiter, gran, tol, stop_after=None):
    """(returned iteration, iterations of the checks that ran) of a loop that
    waits at every check; `stop_after`: the interrupt is seen after that many
    chunks."""
    it, checks, chunks = 0, [], 0
    while it < maxiter:
        n = min(gran - it % gran, maxiter - it)
        it += n
        chunks += 1
        stop = stop_after is not None and chunks >= stop_after
        if it % gran == 0 or stop:
            checks.append(it)
            if 1.0 / (1.0 + it) < tol:
                return it, checks
        if stop:
            break
    return it, checks


def run(monkeypatch, maxiter, gran, tol, depth, sweeps=True, ndim=2, graph=True, stop_after=None):
    dev = Device(tol)
    Graph = fake_env(monkeypatch, dev, sweeps)
    p = types.SimpleNamespace(ndim=ndim, steps=_lib.STEPS["precond"])
    ws = types.SimpleNamespace(t=dev.info)
    loop = pdhg._FusedLoop(p, None, ws, gran, graph=graph)
    seen = []
    calls = {"n": 0}

    def interrupted():
        calls["n"] += 1
        return stop_after is not None and calls["n"] >= stop_after

    it, rec = loop.run(maxiter, depth, lambda r, i: seen.append(i), interrupted)
    return dev, loop, Graph, it, rec, seen


CASES = [(300, 10, 1 / 75.0), (300, 10, 1 / 80.0), (300, 10, 1e-9), (47, 10, 1e-9),
         (47, 10, 1 / 40.0), (60, 6, 1 / 31.0), (61, 7, 1 / 50.0), (9, 10, 1e-9), (30, 1, 1 / 12.0),
         (40, 3, 1 / 20.0), (100, 2, 1 / 33.0)]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("depth,sweeps,ndim", [(2, True, 2), (0, True, 2), (2, False, 2),
                                               (2, True, 3), (1, True, 2)])
@pytest.mark.parametrize("graph", [True, False])
def test_stop_iteration_and_state(monkeypatch, case, depth, sweeps, ndim, graph):
    maxiter, gran, tol = case
    dev, loop, Graph, it, rec, seen = run(monkeypatch, maxiter, gran, tol, depth, sweeps, ndim,
                                          graph)
    want_it, want_checks = expected(maxiter, gran, tol)
    assert it == want_it
    assert dev.it == want_it                      # the state is the checked one
    assert seen == want_checks                    # every check reported once, in order
    if rec is not None:
        assert int(rec[FIELDS.index("checks")]) == len(want_checks)
    fused = sweeps and ndim == 2 and depth > 0
    if fused and gran >= 2:
        # checks ran inside the next chunk's first sweep, except the last one
        assert ("gap", 0) not in dev.ops
        assert not any(k[1] for k in Graph.made)   # no chunk ends with a gap kernel


@pytest.mark.parametrize("depth,sweeps", [(2, True), (0, True), (2, False)])
@pytest.mark.parametrize("stop_after", [1, 3, 4])
def test_interrupt_checks_and_stops(monkeypatch, depth, sweeps, stop_after):
    dev, loop, Graph, it, rec, seen = run(monkeypatch, 200, 7, 1e-9, depth, sweeps,
                                          stop_after=stop_after)
    want_it, want_checks = expected(200, 7, 1e-9, stop_after)
    assert it == want_it == dev.it
    assert seen == want_checks and seen[-1] == want_it


def test_graphs_captured_on_third_use(monkeypatch):
    dev, loop, Graph, it, rec, seen = run(monkeypatch, 200, 10, 1e-9, 2)
    # kinds: the first chunk (no check before it) and the later chunks (the
    # previous chunk's check in their first sweep)
    assert loop.uses[(10, False, False)] == 1 and loop.uses[(10, False, True)] == 19
    assert Graph.made == [(10, False, True)]
    assert it == dev.it == 200 and len(seen) == 20
