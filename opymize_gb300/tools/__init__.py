"""Numeric helpers (opymize/tools/__init__.py)."""

import numpy as np


def truncate(x, n):
    """Floor |x| to n significant digits (opymize/tools/__init__.py:4-12);
    used to round the step bound 1/|A|^2."""
    k = -int(np.floor(np.log10(abs(x))))
    k += n - 1
    if k > 0:
        x_str = str(abs(x))[:(k + 2)]
    else:
        x_str = str(abs(x))[:n] + "0" * (-k)
    return np.sign(x) * float(x_str)
