"""SIGINT handling for solver loops (the role of opymize/tools/util.py:4-39:
Ctrl-C ends a solve at its next check with the current state instead of
raising inside it)."""

import signal
import threading


class GracefulInterruptHandler(object):
    """While the context is active, the first SIGINT only sets
    ``interrupted``: the solver stops at its next check and returns its
    state.  The handler that was installed before is put back at that moment,
    so a second SIGINT acts as it would without this context, and again on
    exit.  Signal handlers can only be set from the main thread; in any other
    thread the context does nothing and ``interrupted`` stays False."""

    def __init__(self, sig=signal.SIGINT):
        self.sig = sig
        self.interrupted = False
        self._installed = False
        self._previous = None

    def __enter__(self):
        self.interrupted = False
        if threading.current_thread() is threading.main_thread():
            self._previous = signal.getsignal(self.sig)
            signal.signal(self.sig, self._on_signal)
            self._installed = True
        return self

    def _on_signal(self, signum, frame):
        self.interrupted = True
        self._restore()

    def _restore(self):
        if self._installed:
            self._installed = False
            previous = self._previous if self._previous is not None else signal.SIG_DFL
            signal.signal(self.sig, previous)

    def __exit__(self, exc_type, exc, tb):
        self._restore()
        return False
