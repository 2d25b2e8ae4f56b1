"""Solvers (opymize/solvers)."""

from opymize_gb300.solvers.pdhg import PDHG   # noqa: F401
