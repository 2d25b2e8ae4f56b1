"""SIGINT handling for solver loops (opymize/tools/util.py:4-39)."""

import signal
import threading


class GracefulInterruptHandler(object):
    """Context manager that records SIGINT instead of raising, so that a
    solver can stop at the next check and return its current state.  Outside
    the main thread (where handlers cannot be installed) it is a no-op."""

    def __init__(self, sig=signal.SIGINT):
        self.sig = sig

    def __enter__(self):
        self.interrupted = False
        self.released = False
        self.active = threading.current_thread() is threading.main_thread()
        if self.active:
            self.original_handler = signal.getsignal(self.sig)
            signal.signal(self.sig, self.handle)
        return self

    def __exit__(self, type, value, tb):
        self.release()

    def handle(self, signum, frame):
        self.release()
        self.interrupted = True

    def release(self):
        if self.released:
            return False
        if self.active:
            signal.signal(self.sig, self.original_handler)
        self.released = True
        return True
