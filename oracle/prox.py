"""Oracle prox / projection maps (numpy restatements)."""

import numpy as np


def truncate(x, n):
    """Floor |x| to n significant digits via its decimal string
    (opymize/tools/__init__.py:4-12)."""
    k = -int(np.floor(np.log10(abs(x))))
    k += n - 1
    if k > 0:
        x_str = str(abs(x))[:(k + 2)]
    else:
        x_str = str(abs(x))[:n] + "0" * (-k)
    return np.sign(x) * float(x_str)


def solve_reduced_monic_cubic(a, b):
    """Real root of x^3 + a x + b = 0 (opymize/tools/__init__.py:14-58):
    cbrt(-b) if a == 0, trigonometric form if Q^3 + R^2 <= 0, else Cardano."""
    a, b = np.asarray(a, dtype=np.float64).ravel(), np.asarray(b, dtype=np.float64).ravel()
    x = np.zeros_like(a)
    m0 = (a == 0)
    x[m0] = np.cbrt(-b[m0])
    m = ~m0
    Q, R = a / 3.0, -b / 2.0
    Q3 = Q ** 3
    D = Q3 + R ** 2
    m2 = m & (D <= 0)
    with np.errstate(invalid="ignore", divide="ignore"):
        theta = np.arccos(R[m2] / np.sqrt(-Q3[m2]))
        x[m2] = 2 * np.sqrt(-Q[m2]) * np.cos(theta / 3.0)
        m3 = m & (D > 0)
        AD = np.cbrt(np.abs(R[m3]) + np.sqrt(D[m3])) * np.sign(R[m3])
        BD = np.where(AD != 0, -Q[m3] / np.where(AD != 0, AD, 1.0), 0.0)
        x[m3] = AD + BD
    return x


def l1_projection(x, N, M, lbd, matrixnorm="frobenius"):
    """Project each x_i (an M[0] x M[1] matrix) onto the lbd-ball, in place
    (opymize/operators/proj.py:87-168)."""
    xv = x.reshape(N, M[0], M[1])
    if M[0] == 1 or M[1] == 1 or matrixnorm == "frobenius":
        nrm = np.sqrt(np.einsum('ilm,ilm->i', xv, xv))
        ext = nrm > lbd
        xv[ext] *= (1.0 / nrm[ext])[:, None, None]
        xv[ext] *= lbd
        return
    # spectral-norm ball for 2 x M or M x 2 (proj.py:114-168)
    for i in range(N):
        A = xv[i] if M[1] == 2 else xv[i].T
        Cm = A.T.dot(A)
        trace = Cm[0, 0] + Cm[1, 1]
        d = Cm[0, 0] * Cm[1, 1] - Cm[0, 1] * Cm[0, 1]
        d = np.sqrt(max(0.0, 0.25 * trace ** 2 - d))
        lmin, lmax = max(0.0, 0.5 * trace - d), max(0.0, 0.5 * trace + d)
        smin, smax = np.sqrt(lmin), np.sqrt(lmax)
        if smax > lbd:
            V = np.zeros((2, 2))
            if Cm[0, 1] == 0.0:
                if Cm[0, 0] >= Cm[1, 1]:
                    V[0, 0] = V[1, 1] = 1.0
                else:
                    V[0, 1] = V[1, 0] = 1.0
            else:
                V[0, 0] = V[0, 1] = Cm[0, 1]
                V[1, 0] = lmax - Cm[0, 0]
                V[1, 1] = lmin - Cm[0, 0]
                V[:, 0] /= np.sqrt(V[0, 0] ** 2 + V[1, 0] ** 2)
                V[:, 1] /= np.sqrt(V[0, 1] ** 2 + V[1, 1] ** 2)
            S = np.diag([min(smax, lbd) / smax,
                         min(smin, lbd) / smin if smin > 0.0 else 0.0])
            A[:] = A.dot(V.dot(S).dot(V.T))


def huber_conj_prox(y, N, M, lbd, alph, sigma):
    """prox of sigma*F* for F = lbd*sum_i huber_alph(|x_i|_F):
    y <- proj_{|.|_F <= lbd}(y / (1 + sigma*alph/lbd)) (elementwise sigma)."""
    y /= (1.0 + np.asarray(sigma) * alph / lbd)
    l1_projection(y, N, M, lbd, "frobenius")


def quadepi_projection(x, N, M, alph, shift=None, lbd=np.inf):
    """Projection onto epi(0.5 alph |x1 - shift1|^2 + shift2), optionally
    truncated at |x1 - shift1| <= lbd, in place
    (opymize/operators/proj.py:338-374)."""
    y = x.reshape(N, M + 1)
    if shift is not None:
        y -= shift
    xnorms = np.linalg.norm(y[:, :-1], axis=-1)
    msk_c0 = (xnorms == 0)
    if lbd < np.inf:
        with np.errstate(divide="ignore", invalid="ignore"):
            msk_c1 = -xnorms / (lbd * alph) + 0.5 * alph * lbd ** 2 + 1 / alph > y[:, -1]
            msk_c2 = 0.5 * alph * lbd ** 2 > y[:, -1]
            msk = (xnorms > lbd) & (~msk_c2)
            y[msk, :-1] *= lbd / xnorms[msk, None]
            msk = msk_c2 & (~msk_c1)
            y[msk, :-1] *= lbd / xnorms[msk, None]
            y[msk, -1] = 0.5 * alph * lbd ** 2
    else:
        msk_c1 = np.ones(y.shape[:-1], dtype=bool)
    msk = msk_c1 & (~msk_c0) & (0.5 * alph * xnorms ** 2 > y[:, -1])
    a_2 = 2.0 / alph ** 2
    a = a_2 * (1 - y[msk, -1] * alph)
    b = -a_2 * xnorms[msk]
    ynorms = solve_reduced_monic_cubic(a, b)
    y[msk, :-1] *= (ynorms / xnorms[msk])[:, None]
    y[msk, -1] = 0.5 * alph * ynorms ** 2
    y[msk_c0 & (y[:, -1] < 0), -1] = 0.0
    if shift is not None:
        y += shift


def shift_scale(x, a, b, shift):
    """T(x) = a*(x + b*shift) (opymize/operators/affine.py:85-146)."""
    return a * (x + b * shift)
