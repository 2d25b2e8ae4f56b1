"""CPU restatement of the epigraph projection and functionals (TEST
INFRASTRUCTURE ONLY: the product never imports this module).

EpigraphProj (opymize/operators/proj.py:388-480) projects every instance
x[j, i] (region j, function i) onto

    {y : <v[l], y[:n]> - y[n] <= b[i, l]  for l = J[j, k] with I[i, l]},

which the reference's GPU kernel solves with an active-set QP (`solve_qp`,
opymize/operators/proj.cu:660-790; its CPU path needs cvxpy + MOSEK, absent
here).  The projection is unique, so this module solves the same QP with the
same method (Nocedal & Wright, Numerical Optimization, 2nd ed., Algorithm
16.3) in plain numpy least-squares steps.  It is pinned against the known
answers of the reference's tests/epigraph.py:11-59 and against the
reference's own `solve_qp` built for the host (oracle/_ref, recipe
oracle/build_ref.py; fixtures tests/golden/epigraph.npz).
"""

import numpy as np


def instance_constraints(I, J, v, b, j, i):
    """Rows a_l = (v[l], -1) and bounds b[i, l] of instance (j, i), in the
    order of J[j] (proj.cu:819-826)."""
    ls = [int(l) for l in J[j] if I[i, l]]
    A = np.empty((len(ls), v.shape[1] + 1))
    A[:, :-1] = v[ls]
    A[:, -1] = -1.0
    return A, np.asarray(b[i, ls], dtype=np.float64), ls


def project_polyhedron(x, A, bb, maxiter=None, tol=1e-9):
    """Projection of x onto {y : A y <= bb} for rows A[k] = (v_k, -1).

    Returns (y, converged).  Start: x with its last coordinate raised by the
    largest violation (feasible, with that constraint active).  Each step
    moves towards x inside the working set's hyperplanes until a new
    constraint blocks; without a blocking constraint (or with n+1 active),
    the multipliers of x - y = A_W^T lambda decide: all >= 0 is optimal, else
    the most negative one leaves the working set.
    """
    x = np.asarray(x, dtype=np.float64)
    n1 = x.size
    m = A.shape[0]
    if maxiter is None:
        maxiter = (n1 - 1) * max(1, m)
    y = x.copy()
    if m == 0:
        return y, True
    viol = A @ x - bb
    k0 = int(np.argmax(viol))
    if not viol[k0] > 0:
        return y, True
    y[-1] += viol[k0]
    W = [k0]
    for _ in range(maxiter):
        d = x - y
        AW = A[W]
        if W:
            z = np.linalg.solve(AW @ AW.T, AW @ d)
            p = d - AW.T @ z
        else:
            p = d
        blocking = -1
        if len(W) < n1 and np.abs(p).sum() > 0:
            smin = 1.0
            for k in range(m):
                if k in W:
                    continue
                ap = A[k] @ p
                if ap > tol:
                    s = (bb[k] - A[k] @ y) / ap
                    if -tol < s < smin:
                        smin, blocking = s, k
            if smin != 0:
                y = y + smin * p
        if blocking >= 0:
            W.append(blocking)
            if len(W) < n1:
                continue
        AW = A[W]
        lam = np.linalg.solve(AW @ AW.T, AW @ (x - y)) if W else np.zeros(0)
        if lam.size == 0 or lam.min() >= 0:
            return y, True
        W.pop(int(np.argmin(lam)))
    return y, False


def epigraph_proj(I, J, v, b, x, maxiter=None, tol=1e-9):
    """EpigraphProj applied to x (nregions, nfuns, ndim+1); returns (y,
    number of instances that did not converge)."""
    nregions, nfuns = x.shape[:2]
    y = np.empty_like(x, dtype=np.float64)
    bad = 0
    nsub = J.shape[1]
    ndim = v.shape[1]
    for j in range(nregions):
        for i in range(nfuns):
            A, bb, _ = instance_constraints(I, J, v, b, j, i)
            it = ndim * nsub if maxiter is None else maxiter
            y[j, i], ok = project_polyhedron(x[j, i], A, bb, it, tol)
            bad += not ok
    return y, bad


def epigraph_ind(I, J, v, b, x):
    """(0, infeas) of EpigraphInd (functionals/epigraph.py:40-46)."""
    inf = 0.0
    for j in range(x.shape[0]):
        for i in range(x.shape[1]):
            A, bb, _ = instance_constraints(I, J, v, b, j, i)
            if bb.size:
                inf = max(inf, float((A @ x[j, i] - bb).max()))
    return 0.0, max(0.0, inf)


def supp_pieces(I, If, J, v, b):
    """Affine pieces (eq_off, eqns) of every instance and the region checks
    of EpigraphSupp (functionals/epigraph.py:84-100): a face of ndim+1 points
    carries the affine function c.p + d through its values; checks[j] is the
    inverse transpose of the rows (v[J[j, k]], -1), k <= ndim."""
    nfuns = I.shape[0]
    nregions = J.shape[0]
    ndim = v.shape[1]
    rows, off = [], [0]
    for j in range(nregions):
        for i in range(nfuns):
            faces = np.asarray(If[i][j])
            P = v[J[j]][faces]                       # (nfaces, ndim+1, ndim)
            vals = b[i, J[j]][faces]                 # (nfaces, ndim+1)
            eq = np.zeros((faces.shape[0], ndim + 1))
            for f in range(faces.shape[0]):
                M = P[f, 1:] - P[f, :1]
                c = np.linalg.solve(M, vals[f, 1:] - vals[f, 0])
                eq[f, :-1] = c
                eq[f, -1] = vals[f, 0] - c @ P[f, 0]
            rows.append(eq)
            off.append(off[-1] + eq.shape[0])
    chk = -np.ones((nregions, ndim + 1, ndim + 1))
    chk[:, :, :-1] = v[J[:, :ndim + 1]]
    chk = np.linalg.inv(chk).transpose(0, 2, 1)
    return np.asarray(off, np.int64), np.concatenate(rows, axis=0), chk


def epigraph_supp(eq_off, eqns, checks, x):
    """(val, infeas) of EpigraphSupp (functionals/epigraph.py:101-112)."""
    nregions, nfuns, n1 = x.shape
    val, inf = 0.0, 0.0
    for j in range(nregions):
        for i in range(nfuns):
            xi = x[j, i].astype(np.float64)
            inf = max(inf, float(np.max(np.fmax(0.0, -(checks[j] @ xi)))))
            xt = max(np.spacing(1), abs(xi[-1]))
            xh = np.append(xi[:-1] / xt, 1.0)
            t = j * nfuns + i
            val += xt * float((eqns[eq_off[t]:eq_off[t + 1]] @ xh).max())
    return val, inf


def region_checks(J, v):
    """checks[j] = inverse transpose of the rows (v[J[j,k]], -1), k <= ndim."""
    ndim = v.shape[1]
    chk = -np.ones((J.shape[0], ndim + 1, ndim + 1))
    chk[:, :, :-1] = v[J[:, :ndim + 1]]
    return np.linalg.inv(chk).transpose(0, 2, 1)


def epigraph_supp_envelope(I, J, v, b, x):
    """EpigraphSupp value for ndim 1 without faces: xt * g(p), p = x[0]/xt,
    g the convex envelope of each instance's points (the smallest chord over
    the pairs bracketing p; beyond the points' range the lower hull's end
    edges extended, as the max over the hull's faces gives there)."""
    assert v.shape[1] == 1
    chk = region_checks(J, v)
    nregions, nfuns, _ = x.shape
    val, inf = 0.0, 0.0
    for j in range(nregions):
        for i in range(nfuns):
            xi = x[j, i].astype(np.float64)
            inf = max(inf, float(np.max(np.fmax(0.0, -(chk[j] @ xi)))))
            xt = max(np.spacing(1), abs(xi[-1]))
            ls = [int(l) for l in J[j] if I[i, l]]
            vs, bs = v[ls, 0].astype(np.float64), b[i, ls].astype(np.float64)
            lo, hi = vs.min(), vs.max()
            blo, bhi = bs[vs == lo].min(), bs[vs == hi].min()
            p = xi[0] / xt
            if lo == hi:
                best = blo
            elif p < lo:
                best = blo + min((bs[vs > lo] - blo) / (vs[vs > lo] - lo)) * (p - lo)
            elif p > hi:
                best = bhi + max((bhi - bs[vs < hi]) / (hi - vs[vs < hi])) * (p - hi)
            else:
                best = np.inf
                for a in range(len(ls)):
                    if vs[a] == p:
                        best = min(best, bs[a])
                        continue
                    if vs[a] > p:
                        continue
                    for c in range(len(ls)):
                        if vs[c] > p:
                            best = min(best, (bs[a] * (vs[c] - p) + bs[c] * (p - vs[a]))
                                       / (vs[c] - vs[a]))
            val += xt * best
    return val, inf
