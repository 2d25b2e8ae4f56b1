"""Seeded synthetic inputs for ROF-type problems.

The reference's example denoises ``skimage.data.astronaut`` (examples/rof.py:36-38);
that dataset is not shipped here, so every workload uses this generator instead:
piecewise-constant images painted from random axis-aligned rectangles and discs
(2-D) or ellipsoids (3-D), plus Gaussian noise, all drawn from
``numpy.random.default_rng(seed)``.

Shape parameters (fixed here so that every run is reproducible):

* ``nshapes`` shapes are painted in order onto a zero background;
* in 2-D each is a box or a disc with probability 1/2; in 3-D every shape is
  an axis-aligned ellipsoid;
* centres are uniform over the domain;
* radii / half-widths are uniform in ``[0.02, 0.25] * min(shape)`` (one per
  axis for boxes and ellipsoids, one for discs);
* intensities are uniform in ``[0, 1]``, one per channel;
* finally ``N(0, sigma^2)`` noise is added to every value.
"""

import numpy as np

RADIUS_RANGE = (0.02, 0.25)


def _paint(img, rng, nshapes, channels):
    shape = img.shape[:-1]
    ndim = len(shape)
    smin = min(shape)
    lo, hi = RADIUS_RANGE
    for _ in range(nshapes):
        # volumes are painted with ellipsoids only
        is_box = (rng.random() < 0.5) and ndim != 3
        centre = rng.random(ndim) * np.asarray(shape, dtype=np.float64)
        if is_box or ndim == 3:
            radii = (lo + (hi - lo) * rng.random(ndim)) * smin
        else:
            radii = np.full(ndim, (lo + (hi - lo) * rng.random()) * smin)
        value = rng.random(channels)
        # bounding box of the shape, clipped to the domain
        sl = []
        for t in range(ndim):
            a = int(max(0, np.floor(centre[t] - radii[t])))
            b = int(min(shape[t], np.ceil(centre[t] + radii[t]) + 1))
            sl.append(slice(a, max(a, b)))
        if is_box:
            coords = [np.arange(s.start, s.stop) + 0.5 for s in sl]
            inside = np.ones([s.stop - s.start for s in sl], dtype=bool)
            for t, c in enumerate(coords):
                m = np.abs(c - centre[t]) <= radii[t]
                inside &= m.reshape([-1 if u == t else 1 for u in range(ndim)])
        else:
            grids = np.ogrid[tuple(sl)]
            r2 = 0.0
            for t, g in enumerate(grids):
                r2 = r2 + ((g + 0.5 - centre[t]) / radii[t]) ** 2
            inside = r2 <= 1.0
        if inside.size == 0:
            continue
        view = img[tuple(sl)]
        view[inside] = value


def piecewise_constant(shape, channels=1, nshapes=20, sigma=0.1, seed=0,
                       dtype=np.float64, salt_pepper=0.0):
    """Noisy piecewise-constant image of ``shape + (channels,)``.

    ``salt_pepper`` replaces that fraction of pixels by 0 or 1 (after the
    Gaussian noise), as used by the sublabel-lifted denoising workload.
    Returns a C-contiguous array of ``dtype``.
    """
    shape = tuple(int(s) for s in shape)
    rng = np.random.default_rng(seed)
    img = np.zeros(shape + (channels,), dtype=np.float64)
    _paint(img, rng, nshapes, channels)
    img += sigma * rng.standard_normal(img.shape)
    if salt_pepper > 0:
        npx = int(np.prod(shape))
        flat = img.reshape(npx, channels)
        hit = rng.random(npx) < salt_pepper
        flat[hit] = (rng.random(int(hit.sum())) < 0.5)[:, None].astype(np.float64)
    return np.ascontiguousarray(img, dtype=dtype)
