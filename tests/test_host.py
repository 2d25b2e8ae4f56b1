"""CPU tests of host-side logic: Variable views, step-bound truncation,
synthetic inputs, SIGINT handling and the solver's path selection."""

import os
import signal

import numpy as np
import pytest

import oracle
from opymize_gb300 import Variable
from opymize_gb300.tools import truncate
from opymize_gb300.tools.synthetic import piecewise_constant
from opymize_gb300.tools.util import GracefulInterruptHandler
from tests.conftest import GOLDEN


def test_variable_views():
    v = Variable((3, 2), (4,))
    assert v.size == 10
    data = np.arange(10.0)
    a, b = v.vars(data)
    assert a.shape == (3, 2) and b.shape == (4,)
    assert b[0] == 6
    assert v[1]['offset'] == 6
    named = Variable(('x', (2, 2)), ('y', 3))
    d = named.vars(np.arange(7.0), named=True)
    assert d['y'].tolist() == [4.0, 5.0, 6.0]


def test_truncate_matches_oracle_and_reference_values():
    ops = np.load(os.path.join(GOLDEN, "ops.npz"))
    for x, y in zip(ops["truncate/x"], ops["truncate/y"]):
        assert truncate(x, 3) == y == oracle.truncate(x, 3)


def test_synthetic_generator_is_seeded():
    a = piecewise_constant((64, 48), 3, seed=7)
    b = piecewise_constant((64, 48), 3, seed=7)
    c = piecewise_constant((64, 48), 3, seed=8)
    assert a.shape == (64, 48, 3)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    v = piecewise_constant((16, 12, 10), 1, seed=1)
    assert v.shape == (16, 12, 10, 1)
    # the fixtures were generated by this generator
    d = np.load(os.path.join(GOLDEN, "g2d_const_fwd.npz"))
    assert np.array_equal(d["f"], piecewise_constant((32, 24), 1, sigma=0.1, seed=1))


def test_salt_and_pepper():
    img = piecewise_constant((100, 100), 1, sigma=0.0, seed=3, salt_pepper=0.1)
    frac = np.mean((img == 0.0) | (img == 1.0))
    assert 0.05 < frac < 0.5


def test_graceful_interrupt():
    with GracefulInterruptHandler() as h:
        os.kill(os.getpid(), signal.SIGINT)
        assert h.interrupted
    assert signal.getsignal(signal.SIGINT) is not None


def test_fused_path_selection():
    from opymize_gb300.solvers import PDHG
    from opymize_gb300.functionals import SSD, L1Norms, HuberL1Norms, QuadEpiInd
    from opymize_gb300.linear import GradientOp, LaplacianOp
    f = np.zeros((20, 1))
    fwd = GradientOp((4, 5), 1, scheme="forward")
    cen = GradientOp((4, 5), 1, scheme="centered")
    assert PDHG(SSD(f), L1Norms(20, (1, 2), 0.1), fwd)._fusable()
    assert PDHG(SSD(f), HuberL1Norms(20, (1, 2), 0.1, 0.01), fwd)._fusable()
    assert not PDHG(SSD(f), L1Norms(20, (1, 2), 0.1), cen)._fusable()
    lap = LaplacianOp((4, 5), 1)
    assert not PDHG(SSD(f), SSD(np.zeros((20, 1))), lap)._fusable()
    assert not PDHG(SSD(f), QuadEpiInd(20, 1), GradientOp((4, 5), 1, "forward"))._fusable()


def test_batch_check_interval():
    """The batch autotuner's interval between stop tests: sqrt(2 n t_gap /
    t_iter) for n = 1000 assumed iterations, even, within [10, 100]."""
    from opymize_gb300.solvers.batch import BatchROF
    assert BatchROF.check_interval(1.0, 1.0) == 46           # sqrt(2000) = 44.7 -> 45 -> 46
    assert BatchROF.check_interval(0.5, 1.0) == 32           # sqrt(1000) = 31.6 -> 32
    assert BatchROF.check_interval(1e-6, 1.0) == 10
    assert BatchROF.check_interval(50.0, 1.0) == 100
    assert BatchROF.check_interval(1.0, 0.0) == 100          # no division by zero
    for t_gap in np.geomspace(1e-3, 10.0, 40):
        g = BatchROF.check_interval(t_gap, 0.37)
        assert g % 2 == 0 and 10 <= g <= 100


def test_interrupt_handler_first_sigint_recorded_second_raises():
    """A solve's first Ctrl-C is recorded (the loop stops at its next check);
    the handler installed before is back at once, so a second one raises."""
    import os
    import signal
    import time
    from opymize_gb300.tools.util import GracefulInterruptHandler
    before = signal.getsignal(signal.SIGINT)
    with GracefulInterruptHandler() as h:
        assert not h.interrupted
        os.kill(os.getpid(), signal.SIGINT)
        time.sleep(0.01)
        assert h.interrupted
        assert signal.getsignal(signal.SIGINT) is before
        with pytest.raises(KeyboardInterrupt):
            os.kill(os.getpid(), signal.SIGINT)
            time.sleep(0.01)
    assert signal.getsignal(signal.SIGINT) is before


def test_split_op_parts_and_jacobian():
    """SplitOp (opymize/operators/__init__.py:6-27): each part acts on its
    own sub-vector (in place when y is None), and with jacobian=True the
    result is the block-diagonal BlockOp of the parts' Jacobians."""
    from opymize_gb300 import Variable
    from opymize_gb300.linear import ZeroOp
    from opymize_gb300.operators import SplitOp

    class Part(object):
        def __init__(self, n, tag):
            self.x, self.y, self.tag, self.calls = Variable(n), Variable(n), tag, []
            self.adjoint = self

        def __call__(self, x, y=None, add=False, jacobian=False):
            self.calls.append((x.copy(), None if y is None else y.shape, add, jacobian))
            return self if jacobian else None

    a, b = Part(3, "a"), Part(5, "b")
    op = SplitOp([a, b])
    assert (op.x.size, op.y.size) == (8, 8)
    x = np.arange(8.0)
    assert op._call_gpu(x, np.zeros(8), add=True) is None
    np.testing.assert_array_equal(a.calls[0][0], x[:3])
    np.testing.assert_array_equal(b.calls[0][0], x[3:])
    assert a.calls[0][1:] == ((3,), True, False) and b.calls[0][1:] == ((5,), True, False)
    op._call_gpu(x)                                     # in place
    assert a.calls[1][1] is None and b.calls[1][1] is None
    J = op._call_gpu(x, jacobian=True)
    assert J.blocks[0][0] is a and J.blocks[1][1] is b
    assert isinstance(J.blocks[0][1], ZeroOp) and isinstance(J.blocks[1][0], ZeroOp)
    assert (J.blocks[0][1].y.size, J.blocks[0][1].x.size) == (3, 5)
