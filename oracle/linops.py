"""Oracle linear operators (numpy / scipy.sparse restatements).

Each operator is stored as a scipy CSR matrix ``spmat`` and applied with
``spmat.dot`` exactly as the reference's ``LinOp._call_cpu`` does
(opymize/__init__.py:95-108), so the CPU cost profile of the oracle solver is
that of the reference.  Matrices are built directly from index arithmetic
rather than through the reference's general ``einsumop`` machinery.
"""

import numpy as np
import scipy.sparse as sp


def imagedim_skips(dims):
    """Row-major strides of the image grid (opymize/linear/diff.py:15-21)."""
    skips = np.ones(len(dims), dtype=np.int64)
    for t in range(len(dims) - 2, -1, -1):
        skips[t] = skips[t + 1] * dims[t + 1]
    return skips


def _coords(dims):
    return np.indices(dims, dtype=np.int64).reshape(len(dims), -1)


class LinOp(object):
    """y = A x with ``add`` accumulation (opymize/__init__.py:86-142)."""

    spmat = None
    adjoint = None

    def __call__(self, x, y, add=False):
        x, y = x.ravel(), y.ravel()
        if add:
            y += self.spmat.dot(x)
        else:
            y[:] = self.spmat.dot(x)

    def rowwise_lp(self, y, p=1, add=False):
        """y_i = sum_j |A_ij|^p (opymize/__init__.py:122-142)."""
        if not add:
            y.fill(0.0)
        y += sp.linalg.norm(self.spmat, ord=p, axis=1) if p != 1 else \
            np.asarray(abs(self.spmat).sum(axis=1)).ravel()


def _transposed(op, spmat_t, x_size, y_size):
    adj = LinOp()
    adj.spmat = spmat_t
    adj.x_size, adj.y_size = x_size, y_size
    adj.adjoint = op
    return adj


# ---------------------------------------------------------------------------
# finite differences
# ---------------------------------------------------------------------------

def gradient_matrix(dims, C, scheme="centered", h=None, w=None):
    """Sparse gradient y[i,t,k] (row (i*D+t)*C+k) of x[j,k] (col j*C+k).

    forward  : y = w_k/h_t (x[i+s_t] - x[i]) if c_t < n_t-1 else 0
               (sparse.py:64-99, :101-144; diff.cu:64-71)
    centered : y = w_k/(h_t 2^(D-1)) sum_a (x[b_a+s_t] - x[b_a]) with
               b_a = i + avgskip_a, zero if i lies on any far boundary
               (diff.cu:53-63, diff.py:23-42).  For D <= 2 this equals the
               reference's sparse avgopn*diffopn (sparse.py:83-86).
    """
    dims = tuple(int(d) for d in dims)
    D = len(dims)
    N = int(np.prod(dims))
    h = np.ones(D) if h is None else np.asarray(h, dtype=np.float64)
    w = np.ones(C) if w is None else np.asarray(w, dtype=np.float64)
    skips = imagedim_skips(dims)
    coords = _coords(dims)
    idx = np.arange(N, dtype=np.int64)
    rows, cols, vals = [], [], []
    for t in range(D):
        if scheme == "forward" or D == 1:
            valid = coords[t] < dims[t] - 1
            offs = [0]
            fac = 1.0 / h[t]
        elif scheme == "centered":
            valid = np.all(coords < (np.array(dims)[:, None] - 1), axis=0)
            others = [u for u in range(D) if u != t]
            offs = []
            for m in range(1 << (D - 1)):
                offs.append(sum(((m >> b) & 1) * skips[u]
                                for b, u in enumerate(others)))
            fac = 1.0 / (h[t] * len(offs))
        else:
            raise ValueError("unsupported scheme: %s" % scheme)
        i = idx[valid]
        for off in offs:
            base = i + off
            for k in range(C):
                r = (i * D + t) * C + k
                rows += [r, r]
                cols += [base * C + k, (base + skips[t]) * C + k]
                vals += [np.full(i.size, -w[k] * fac), np.full(i.size, w[k] * fac)]
    if rows:
        rows = np.concatenate(rows)
        cols = np.concatenate(cols)
        vals = np.concatenate(vals)
    return sp.csr_matrix((vals, (rows, cols)), shape=(N * D * C, N * C))


class Gradient(LinOp):
    """GradientOp (opymize/linear/diff.py:67-144); adjoint = Divergence."""

    def __init__(self, dims, C, scheme="centered", imageh=None, weights=None):
        self.dims, self.C, self.scheme = tuple(dims), C, scheme
        D, N = len(dims), int(np.prod(dims))
        self.x_size, self.y_size = N * C, N * D * C
        self.imageh = np.ones(D) if imageh is None else np.asarray(imageh, float)
        self.weights = np.ones(C) if weights is None else np.asarray(weights, float)
        self.spmat = gradient_matrix(dims, C, scheme, self.imageh, self.weights)
        self.adjoint = _transposed(self, self.spmat.T.tocsr(), self.y_size, self.x_size)


def Divergence(dims, C, scheme="centered", imageh=None, weights=None):
    """DivergenceOp (opymize/linear/diff.py:146-183) = GradientOp^T."""
    return Gradient(dims, C, scheme, imageh, weights).adjoint


def laplacian_matrix(dims, C, h=None, boundary="neumann"):
    """Sparse Laplacian (opymize/linear/sparse.py:11-62)."""
    dims = tuple(int(d) for d in dims)
    D = len(dims)
    h = np.ones(D) if h is None else np.asarray(h, dtype=np.float64)

    def dd(n):
        main = -2.0 * np.ones(n)
        lo = np.ones(n - 1)
        up = np.ones(n - 1)
        if boundary == "neumann":
            main[0] = main[-1] = -1.0
        elif boundary in ("curvature", "second-order"):
            main[0] = main[-1] = 0.0
            up[0] = 0.0
            lo[-1] = 0.0
        else:
            raise ValueError("unsupported boundary: %s" % boundary)
        return sp.diags([lo, main, up], [-1, 0, 1], shape=(n, n))

    Delta = sp.csr_matrix((int(np.prod(dims)),) * 2)
    for t, n in enumerate(dims):
        before = int(np.prod(dims[:t]))
        after = int(np.prod(dims[t + 1:]))
        part = sp.kron(sp.kron(sp.eye(before), dd(n) / h[t] ** 2), sp.eye(after))
        Delta = Delta + part
    if boundary == "curvature":
        keep = np.all((_coords(dims) > 0)
                      & (_coords(dims) < np.array(dims)[:, None] - 1), axis=0)
        Delta = sp.diags(keep.astype(np.float64)).dot(Delta)
    return sp.kron(Delta, sp.eye(C)).tocsr()


class Laplacian(LinOp):
    """LaplacianOp (opymize/linear/diff.py:185-249): boundary in neumann,
    curvature(_adj), second-order(_adj); neumann is self-adjoint."""

    def __init__(self, dims, C, imageh=None, boundary="neumann"):
        N = int(np.prod(dims))
        self.x_size = self.y_size = N * C
        base = boundary[:-4] if boundary.endswith("_adj") else boundary
        M = laplacian_matrix(dims, C, imageh, base)
        self.spmat = M.T.tocsr() if boundary.endswith("_adj") else M
        if boundary == "neumann":
            self.adjoint = self
        else:
            self.adjoint = _transposed(self, self.spmat.T.tocsr(), N * C, N * C)


# ---------------------------------------------------------------------------
# per-pixel small matrix products (opymize/linear/einsum.py)
# ---------------------------------------------------------------------------

def _dense_op(subscripts, A, x_shape, y_shape):
    """Sparse matrix of x -> einsum(subscripts, A, x) by probing columns of a
    block structure.  Used only at oracle sizes."""
    nx = int(np.prod(x_shape))
    rows, cols, vals = [], [], []
    eye = np.zeros(x_shape).ravel()
    for j in range(nx):
        eye[:] = 0.0
        eye[j] = 1.0
        col = np.einsum(subscripts, A, eye.reshape(x_shape)).ravel()
        nz = np.nonzero(col)[0]
        rows.append(nz)
        cols.append(np.full(nz.size, j))
        vals.append(col[nz])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows),
                                                 np.concatenate(cols))),
                         shape=(int(np.prod(y_shape)), nx))


class _EinsumOp(LinOp):
    def _setup(self, subscripts, A, x_shape, y_shape, adj_subscripts):
        self.A = A
        self.x_shape, self.y_shape = tuple(x_shape), tuple(y_shape)
        self.x_size, self.y_size = int(np.prod(x_shape)), int(np.prod(y_shape))
        self.subscripts = subscripts
        self.adj_subscripts = adj_subscripts
        self._spmat = None

    @property
    def spmat(self):
        if self._spmat is None:
            self._spmat = _dense_op(self.subscripts, self.A, self.x_shape, self.y_shape)
        return self._spmat

    def __call__(self, x, y, add=False):
        r = np.einsum(self.subscripts, self.A, x.reshape(self.x_shape)).ravel()
        if add:
            y.ravel()[:] += r
        else:
            y.ravel()[:] = r

    @property
    def adjoint(self):
        adj = _EinsumOp()
        adj._setup(self.adj_subscripts, self.A, self.y_shape, self.x_shape,
                   self.subscripts)
        return adj


class MatrixMult(_EinsumOp):
    """y_ji = sum_k A_jk x_ki (opymize/linear/einsum.py:17-56).  x is (K, N)
    with K = A.shape[1] (trans: A.shape[0]); the reference only builds this
    for square A."""

    def __init__(self, N, A, trans=False):
        if trans:
            self._setup('kj,ki->ji', A, (A.shape[0], N), (A.shape[1], N), 'jk,ki->ji')
        else:
            self._setup('jk,ki->ji', A, (A.shape[1], N), (A.shape[0], N), 'kj,ki->ji')


class MatrixMultR(_EinsumOp):
    """y_ij = sum_k x_ik A_kj (opymize/linear/einsum.py:58-97)."""

    def __init__(self, N, A, trans=False):
        if trans:
            self._setup('jk,ik->ij', A, (N, A.shape[1]), (N, A.shape[0]), 'kj,ik->ij')
        else:
            self._setup('kj,ik->ij', A, (N, A.shape[0]), (N, A.shape[1]), 'jk,ik->ij')


class MatrixMultRBatched(_EinsumOp):
    """y_jlk = sum_m x_jlm A_jmk (opymize/linear/einsum.py:175-214)."""

    def __init__(self, N, A, trans=False):
        J, M, K = A.shape
        if trans:
            self._setup('jkm,jlm->jlk', A, (J, N, K), (J, N, M), 'jmk,jlm->jlk')
        else:
            self._setup('jmk,jlm->jlk', A, (J, N, M), (J, N, K), 'jkm,jlm->jlk')


class TangledMatrixMultR(_EinsumOp):
    """y_mik = sum_jl x_jil A_jlmk (opymize/linear/einsum.py:130-173)."""

    def __init__(self, N, A, trans=False):
        J, L, M, K = A.shape
        if trans:
            self._setup('mkjl,jil->mik', A, (M, N, K), (J, N, L), 'jlmk,jil->mik')
        else:
            self._setup('jlmk,jil->mik', A, (J, N, L), (M, N, K), 'mkjl,jil->mik')


class DiagMatrixMultR(_EinsumOp):
    """y_ik = x_ik A_k (opymize/linear/einsum.py:104-128); self-adjoint."""

    def __init__(self, N, A):
        self._setup('k,ik->ik', A, (N, A.size), (N, A.size), 'k,ik->ik')


class IndexedMult(LinOp):
    """(Ax)[j,i,m] = -sum_l B[j,m,l] x[i,P[j,l]] (opymize/linear/indexed.py:63-94)."""

    def __init__(self, K, N, B, P):
        J, M, L = B.shape
        self.B, self.P, self.K, self.N = B, P, K, N
        self.x_size, self.y_size = N * K, J * N * M
        j, i, m, l = np.meshgrid(np.arange(J), np.arange(N), np.arange(M),
                                 np.arange(L), indexing="ij")
        rows = (j * N + i) * M + m
        cols = i * K + P[j, l]
        vals = -B[j, m, l]
        self.spmat = sp.csr_matrix((vals.ravel(), (rows.ravel(), cols.ravel())),
                                   shape=(self.y_size, self.x_size))
        self.adjoint = _transposed(self, self.spmat.T.tocsr(), self.y_size, self.x_size)


def IndexedMultAdj(K, N, P, B):
    """(Ax)[i,P[j,l]] -= sum_m B[j,m,l] x[j,i,m] (opymize/linear/indexed.py:34-61)."""
    return IndexedMult(K, N, B, P).adjoint


# ---------------------------------------------------------------------------
# trivial operators and block composition (opymize/linear/scale.py,
# opymize/linear/__init__.py)
# ---------------------------------------------------------------------------

class ZeroOp(LinOp):
    def __init__(self, M, N=None):
        N = M if N is None else N
        self.x_size, self.y_size = N, M
        self.spmat = sp.csr_matrix((M, N))

    @property
    def adjoint(self):
        return ZeroOp(self.x_size, self.y_size)


class ScaleOp(LinOp):
    def __init__(self, N, fact):
        self.x_size = self.y_size = N
        self.spmat = sp.diags(np.broadcast_to(np.asarray(fact, float), (N,))).tocsr()
        self.adjoint = self


class IdentityOp(ScaleOp):
    def __init__(self, N):
        ScaleOp.__init__(self, N, 1.0)


class BlockOp(LinOp):
    """A = [[A11, A12, ...], ...] (opymize/linear/__init__.py:48-111)."""

    def __init__(self, blocks):
        self.blocks = blocks
        self.spmat = sp.bmat([[b.spmat for b in row] for row in blocks]).tocsr()
        self.y_size, self.x_size = self.spmat.shape
        self.adjoint = _transposed(self, self.spmat.T.tocsr(), self.y_size, self.x_size)

    def rowwise_lp(self, y, p=1, add=False):
        """Sum of the blocks' row norms (opymize/linear/__init__.py:104-111)."""
        if not add:
            y.fill(0.0)
        off = 0
        for row in self.blocks:
            n = row[0].y_size
            for b in row:
                b.rowwise_lp(y[off:off + n], p=p, add=True)
            off += n


def normest(op, tol=1.0e-4, maxits=500):
    """Power iteration for |A| (opymize/linear/__init__.py:11-46), drawing
    from the global ``np.random`` state exactly like the reference."""
    from numpy.linalg import norm
    m, n = op.y_size, op.x_size
    itn = 0
    x, y = np.empty(n), np.empty(m)
    y[:] = 1.0
    y[np.random.randn(m) < 0] = -1
    op.adjoint(y, x)
    x[:] = np.abs(x)
    e = norm(x)
    if e < 1e-13:
        return e, itn
    x *= 1.0 / e
    e0 = 0
    while abs(e - e0) > tol * e:
        e0 = e
        op(x, y)
        normy = norm(y)
        if normy < 1e-13:
            y[:] = np.random.rand(m)
            normy = norm(y)
        op.adjoint(y, x)
        normx = norm(x)
        e = normx / normy
        x *= 1.0 / normx
        itn += 1
        if itn > maxits:
            break
    return e, itn
