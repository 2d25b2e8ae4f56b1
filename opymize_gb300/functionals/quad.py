"""Sum of squared differences (opymize/functionals/quad.py)."""

import numpy as np

from opymize_gb300 import Variable, Functional
from opymize_gb300.functionals._eval import fct, evaluate, devcopy
from opymize_gb300.operators.affine import SSDProxOp


class SSD(Functional):
    """0.5*<x - f, x - f>_b + shift with volume element b per channel and an
    optional pixel mask (opymize/functionals/quad.py:7-55)."""

    def __init__(self, data, vol=None, shift=0, mask=None, conj=None):
        Functional.__init__(self)
        self.x = Variable(data.shape)
        self.f = np.atleast_2d(data)
        self.shift = shift
        self.vol = np.ones(data.shape[1]) if vol is None else np.asarray(vol, dtype=np.float64)
        self.mask = np.ones(data.shape[0], dtype=bool) if mask is None else np.asarray(mask, bool)
        if conj is None:
            cj_vol = 1.0 / self.vol
            cj_data = np.zeros_like(self.f)
            cj_data[self.mask, :] = np.einsum('ik,k->ik', self.f[self.mask, :], -self.vol)
            cj_shift = -0.5 * np.einsum('ik,k->', cj_data ** 2, cj_vol)
            cj_shift -= self.shift
            self.conj = SSD(cj_data, shift=cj_shift, vol=cj_vol, mask=mask, conj=self)
        else:
            self.conj = conj

    # device copies of the constant data
    def f_dev(self, dtype):
        return devcopy(self, "f", self.f, dtype)

    def vol_dev(self):
        return devcopy(self, "vol", self.vol, np.float64)

    def mask_dev(self):
        if np.all(self.mask):
            return None
        return devcopy(self, "mask", self.mask.astype(np.uint8), np.uint8)

    def _eval_gpu(self, x):
        m = self.mask_dev()
        f = fct("ssd", self.f.shape[0], self.f.shape[1], v0=self.f_dev(x.dtype).ptr,
                vol=self.vol_dev().ptr, mask=None if m is None else m.ptr,
                scalar0=float(self.shift))
        return evaluate(f, x)

    def prox(self, tau):
        """prox of tau*G; tau a scalar, a per-element DeviceArray or a
        DeviceScalar (adaptive steps)."""
        return SSDProxOp(self, tau)
