"""Sublabel-accurate lifting of scalar denoising with a nonconvex data term.

    min_gamma  sum_x rho_x(gamma(x)) + lbd * TV(gamma),
    rho_x(s) = min((s - f(x))^2, trunc),  gamma(x) in [0, 1]

The range [0, 1] carries L labels t_k = k/(L-1) and L-1 intervals.  Each
pixel's gamma is lifted to barycentric coordinates u(x) in the unit simplex of
R^L, gamma = <t, u>.  The data term is convexified per interval from samples
of rho (S points per interval, endpoints included), so that it is exactly the
piecewise-linear setting of the reference's EpigraphInd / EpigraphSupp
(opymize/functionals/epigraph.py:7-127) with ndim = 1: for interval j and
pixel i the dual pair mu[j, i] = (slope, offset) must lie in the epigraph of
the conjugate of rho_i restricted to the interval.

The reference ships these operators but assembles no such model; this module
does so with nothing but the reference's own operator vocabulary, as a user
of the reference would:

    primal  x = (u [N, L], gamma [N], mu [L-1, N, 2])
    g(x)    = PositivityFct(u) + 0(gamma) + 0(mu)
    dual    y = (q [N, L], e [N], p [N, D], s [N], z [L-1, N, 2])
    A x     = (u - B^T mu,            IdentityOp + IndexedMultAdj
               <t, u> - gamma,        MatrixMultR + ScaleOp(-1)
               grad gamma,            GradientOp
               <1, u>,                MatrixMultR
               mu)                    IdentityOp
    f(Ax)   = 0 iff q-part = 0, e-part = 0; lbd*L1Norms(p); 0 iff s-part = 1;
              EpigraphSupp(z)

B maps the lifted dual q [L] to the interval pairs: (Bq)_j = ((q_{j+1} -
q_j)/h, t_j (q_{j+1} - q_j)/h - q_j), h = 1/(L-1); IndexedMultAdj with
P[j] = (j, j+1) and coefficients Bc[j, m, l] applies -B^T.  The saddle point
is the biconjugate of the lifted data term (the supremum over q with Bq in
the epigraphs) plus the total variation of <t, u>.
"""

import numpy as np


def labels(L):
    return np.linspace(0.0, 1.0, L)


def sublabel_data(f, L=16, samples=8, trunc=0.04):
    """Constant data of the model for pixel values f (N,) in [0, 1].

    Returns a dict with t (L,), h, v (npoints, 1) sample points, J
    (L-1, samples) the points of every interval (the two endpoints first, the
    region's simplex vertices), I (N, npoints) all set, b (N, npoints) =
    rho_i(v), P (L-1, 2) and Bc (L-1, 2, 2) of IndexedMultAdj.
    """
    f = np.asarray(f, dtype=np.float64).ravel()
    assert L >= 2 and samples >= 2
    t = labels(L)
    h = 1.0 / (L - 1)
    S = samples
    npoints = (L - 1) * (S - 1) + 1
    v = np.linspace(0.0, 1.0, npoints)[:, None]
    J = np.empty((L - 1, S), dtype=np.int64)
    for j in range(L - 1):
        a = j * (S - 1)
        J[j, 0], J[j, 1] = a, a + S - 1
        J[j, 2:] = np.arange(a + 1, a + S - 1)
    b = np.minimum((v[:, 0][None, :] - f[:, None]) ** 2, trunc)
    I = np.ones((f.size, npoints), dtype=bool)
    P = np.stack([np.arange(L - 1), np.arange(1, L)], axis=1).astype(np.int64)
    Bc = np.empty((L - 1, 2, 2))
    Bc[:, 0, 0], Bc[:, 0, 1] = -1.0 / h, 1.0 / h
    Bc[:, 1, 0], Bc[:, 1, 1] = -t[:-1] / h - 1.0, t[:-1] / h
    return dict(t=t, h=h, v=v, J=J, I=I, b=b, P=P, Bc=Bc, L=L, samples=S, trunc=trunc)


def lower_hull_faces(d, i, j):
    """Faces (pairs of positions in J[j]) of the lower convex hull of pixel
    i's samples on interval j -- the convex pieces EpigraphSupp takes as If
    (monotone chain over the points sorted by v)."""
    pos = np.argsort(d["v"][d["J"][j], 0], kind="stable")
    xs = d["v"][d["J"][j][pos], 0]
    ys = d["b"][i, d["J"][j][pos]]
    hull = []
    for k in range(len(pos)):
        while len(hull) >= 2:
            a, c = hull[-2], hull[-1]
            cross = (xs[c] - xs[a]) * (ys[k] - ys[a]) - (ys[c] - ys[a]) * (xs[k] - xs[a])
            if cross <= 0:
                hull.pop()
            else:
                break
        hull.append(k)
    return np.array([[pos[hull[m]], pos[hull[m + 1]]] for m in range(len(hull) - 1)],
                    dtype=np.int64)


def faces(d):
    """If[i][j] for every pixel and interval: the lower hulls of
    `piecewise_convexify` (libopyx host code, every host thread), which are
    those of `lower_hull_faces`."""
    from opymize_gb300.tools.convexify import piecewise_convexify
    return piecewise_convexify(d["v"], d["b"], d["J"])[1]


def sublabel_problem(f_img, L=16, lbd=0.1, samples=8, trunc=0.04, with_faces=False):
    """(g, f, A, data) of the model on the GPU operators of this package for
    an image f_img (imagedims) with values in [0, 1]."""
    from opymize_gb300.functionals import (SplitSum, PositivityFct, ZeroFct, IndicatorFct,
                                           L1Norms, EpigraphSupp)
    from opymize_gb300.linear import BlockOp
    from opymize_gb300.linear.diff import GradientOp
    from opymize_gb300.linear.einsum import MatrixMultR
    from opymize_gb300.linear.indexed import IndexedMultAdj
    from opymize_gb300.linear.scale import IdentityOp, ScaleOp
    dims = tuple(int(s) for s in np.shape(f_img))
    N, D = int(np.prod(dims)), len(dims)
    d = sublabel_data(np.asarray(f_img).ravel(), L, samples, trunc)
    If = faces(d) if with_faces else None
    nmu = (L - 1) * N * 2
    g = SplitSum([PositivityFct(N * L), ZeroFct(N), ZeroFct(nmu)])
    f = SplitSum([IndicatorFct(N * L), IndicatorFct(N), L1Norms(N, (1, D), lbd),
                  IndicatorFct(N, c1=1.0), EpigraphSupp(d["I"], If, d["J"], d["v"], d["b"])])
    A = BlockOp([
        [IdentityOp(N * L), 0, IndexedMultAdj(L, N, d["P"], d["Bc"])],
        [MatrixMultR(N, d["t"][:, None]), ScaleOp(N, -1.0), 0],
        [0, GradientOp(dims, 1, scheme="forward"), 0],
        [MatrixMultR(N, np.ones((L, 1))), 0, 0],
        [0, 0, IdentityOp(nmu)]])
    # the model's data, for PDHG.solve's fused passes (solvers/sublabel.py)
    A.sublabel = dict(L=L, lbd=lbd, dims=dims, data=d, epi=f.fcts[-1])
    return g, f, A, d
