"""The reference's module path for piecewise convexification
(opymize/quickhull/__init__.pyx): ``from opymize_gb300.quickhull import
piecewise_convexify`` works as ``from opymize.quickhull import
piecewise_convexify`` does."""

from opymize_gb300.tools.convexify import piecewise_convexify, convexify_arrays  # noqa: F401

__all__ = ["piecewise_convexify", "convexify_arrays"]
