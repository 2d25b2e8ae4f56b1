"""Solvers (opymize/solvers) on libopyx kernels."""

from opymize_gb300.solvers.pdhg import PDHG   # noqa: F401
from opymize_gb300.solvers.batch import BatchROF   # noqa: F401
from opymize_gb300.solvers.semismooth_newton import SemismoothNewton   # noqa: F401
