"""Spin operators and density matrices, API-compatible with
``muspinsim/spinop.py``.

Host-side algebra on small matrices (scipy CSR by default, like the
reference).  The two numerical kernels of this module -- diagonalisation
(``Hermitian.diag``) and the change of basis -- run on the GPU through
``libmspgpu``.
"""

from copy import deepcopy
from numbers import Number

import numpy as np
from scipy import sparse

from muspinsim_gb300 import kernels


def _mvals(I):
    """m = +I ... -I (muspinsim/spinop.py:14-15)."""
    return np.linspace(I, -I, int(2 * I + 1))


def _Sp(mvals):
    """Raising operator: <m+1|S+|m> = sqrt(I(I+1) - m(m+1)), written via the
    cumulative sum of 2m (muspinsim/spinop.py:18-19)."""
    return 2 * np.diag(0.5 * (np.cumsum(2 * mvals)[:-1] ** 0.5), k=1) + 0.0j


def _Sm(mvals):
    return _Sp(mvals).T


def _Sx(mvals):
    o = _Sp(mvals)
    return 0.5 * (o + o.T)


def _Sy(mvals):
    o = _Sp(mvals)
    return 0.5j * (o.T - o)


def _Sz(mvals):
    return np.diag(mvals) + 0.0j


def _S0(mvals):
    return np.eye(len(mvals)) + 0.0j


_AXES = {"x": _Sx, "y": _Sy, "z": _Sz, "+": _Sp, "-": _Sm, "0": _S0}


def _dense(m):
    return m.toarray() if sparse.issparse(m) else np.asarray(m)


class Clonable:
    """``clone()`` = deep copy (muspinsim/utils.py:13-22)."""

    def clone(self):
        cls = self.__class__
        copy = cls.__new__(cls)
        copy.__dict__ = deepcopy(self.__dict__)
        return copy


class Hermitian:
    """Mixin marking operators that must be Hermitian (the reference's
    Hermitian, muspinsim/spinop.py:44-82): construction checks it, and the
    eigendecomposition runs on the GPU."""

    _must_be_hermitian = True

    def diag(self):
        """Eigenvalues (ascending) and eigenvector matrix (columns), as
        numpy.linalg.eigh returns them, computed by the GPU Jacobi solver in
        FP64.  The result is cached while the matrix is unchanged."""
        M = _dense(self.matrix)
        cached = getattr(self, "_eigh_cache", None)
        if cached is not None and cached[0].shape == M.shape and np.array_equal(cached[0], M):
            return cached[1]
        evals, evecs, status = kernels.eigh(M[None])
        if int(status[0].item()) != 0:
            raise RuntimeError("Hermitian.diag: the Jacobi eigensolver did not converge")
        eigh = (evals[0].cpu().numpy(), evecs[0].cpu().numpy())
        self._eigh_cache = (M.copy(), eigh)
        return eigh


def _as_storage(M, want_sparse):
    """M as a CSR matrix or a dense ndarray."""
    if want_sparse:
        return M.tocsr() if sparse.issparse(M) else sparse.csr_matrix(M)
    return M.toarray() if sparse.issparse(M) else np.array(M)


# The binary matrix operations behind the operator algebra, with the
# reference's message for operands on different spaces.
_MATRIX_OPS = {
    "+": (lambda a, b: a + b, "Can not add to Operators with different dimensions"),
    "-": (lambda a, b: a - b, "Can not subtract to Operators with different dimensions"),
    "@": (lambda a, b: a @ b, "Can not multiply to Operators with different dimensions"),
}


class Operator(Clonable):
    """A matrix on a tensor-product spin space (the reference's Operator,
    muspinsim/spinop.py:85-355).

    State: the matrix in CSR or dense storage (``matrix``), the dimension of
    each factor space (``dimension``) and the Hermiticity tolerance.  All
    arithmetic goes through one path: the other operand is turned into a
    matrix of the same space (a Number c stands for c times the identity
    under + and -, for a plain scale under * and /), checked for the same
    factor dimensions, and combined by one of _MATRIX_OPS into a copy of
    this operator.
    """

    def __init__(self, matrix, dim=None, herm_tol=1e-6, use_sparse=True):
        rows, cols = np.shape(matrix)[:2] if np.ndim(matrix) == 2 else (0, -1)
        if rows != cols:
            raise ValueError("Matrix passed to Operator must be square")
        factors = (rows,) if dim is None else tuple(dim)
        if np.prod(factors) != rows:
            raise ValueError("Dimensions are not compatible with matrix")
        self._mat = _as_storage(matrix, use_sparse)
        self._factors = factors
        self._tol = herm_tol
        # set by the Hermitian mixin, wherever it sits in the class's bases
        if getattr(self, "_must_be_hermitian", False) and not self.is_hermitian:
            raise ValueError("Operator must be hermitian")

    # -- state
    @property
    def matrix(self):
        return self._mat

    @property
    def dimension(self):
        return self._factors

    @property
    def Is(self):
        return tuple((d - 1) / 2.0 for d in self._factors)

    @property
    def N(self):
        return np.prod(self._factors)

    @property
    def is_sparse(self):
        return sparse.issparse(self._mat)

    @property
    def is_hermitian(self):
        return np.abs(self._mat - self._mat.conjugate().T).max() < self._tol

    def _with_matrix(self, M):
        """A copy of this operator (same class and space) holding M."""
        out = self.clone()
        out._mat = _as_storage(M, self.is_sparse)
        return out

    # -- algebra
    def _operand(self, x, op):
        """The matrix x stands for in `op` with self, or None."""
        if isinstance(x, Number):
            if op not in "+-":
                return None
            n = self._mat.shape[0]
            return x * (sparse.identity(n, format="csr") if self.is_sparse else np.eye(n))
        if isinstance(x, Operator) and self._accepts(x):
            if x.dimension != self.dimension:
                raise ArithmeticError(_MATRIX_OPS[op][1])
            return x.matrix
        return None

    def _accepts(self, x):
        """Whether an operator of x's type combines with this one."""
        return True

    _unsupported = "Unsupported operation for Operator"

    def _binary(self, x, op):
        M = self._operand(x, op)
        if M is None:
            raise TypeError(self._unsupported)
        return self._with_matrix(_MATRIX_OPS[op][0](self._mat, M))

    def _scaled(self, c):
        return self._with_matrix(self._mat * c)

    def __add__(self, x):
        return self._binary(x, "+")

    def __sub__(self, x):
        return self._binary(x, "-")

    def __mul__(self, x):
        if isinstance(x, Number):
            return self._scaled(x)
        return self._binary(x, "@")

    def __rmul__(self, x):
        if isinstance(x, Number):
            return self._scaled(x)
        if isinstance(x, Operator):
            return x.__mul__(self)
        raise TypeError("Unsupported operation for Operator")

    def __truediv__(self, x):
        if not isinstance(x, Number):
            raise TypeError("Unsupported operation for Operator")
        return self._scaled(1.0 / x)

    def __eq__(self, x):
        return (isinstance(x, Operator) and self.dimension == x.dimension
                and bool(np.array_equal(_dense(self._mat), _dense(x.matrix))))

    __hash__ = None

    def dagger(self):
        """The adjoint (conjugate transpose), same class and space."""
        return self._with_matrix(self._mat.conjugate().T)

    def kron(self, x):
        """Tensor product (muspinsim/spinop.py:266-295): the factor spaces
        of self followed by those of x."""
        if not isinstance(x, Operator):
            raise ValueError("Can only perform Kronecker product with another Operator")
        out = self._with_matrix(
            sparse.kron(self._mat, x.matrix, format="csr") if self.is_sparse
            else np.kron(_dense(self._mat), _dense(x.matrix)))
        out._factors = self._factors + x.dimension
        return out

    def hilbert_schmidt(self, x):
        """tr(A^dag B) (muspinsim/spinop.py:297-328)."""
        if not isinstance(x, Operator):
            raise ValueError("Can only perform Hilbert-Schmidt product with another Operator")
        if x.dimension != self.dimension:
            raise ValueError(
                "Operators must have the same dimension to perform Hilbert-Schmidt product"
            )
        # tr(A^dag B) = sum_ij conj(A_ij) B_ij
        return complex(np.sum(np.conj(_dense(self._mat)) * _dense(x.matrix)))

    def basis_change(self, basis, use_sparse=False):
        """basis^dag M basis, computed on the GPU (muspinsim/spinop.py:330-355)."""
        M = _dense(self._mat).astype(complex)
        out = kernels.basis_change(np.asarray(basis, dtype=complex), M)[0].cpu().numpy()
        ans = self.clone()
        ans._mat = _as_storage(out, use_sparse)
        return ans


class SpinOperator(Operator):
    @classmethod
    def from_axes(cls, Is=0.5, axes="x", use_sparse=True):
        """Kronecker product of single-spin operators (muspinsim/spinop.py:358-411)."""
        if isinstance(Is, Number):
            Is = [Is]
        if len(Is) != len(axes) or len(Is) == 0:
            raise ValueError("Arrays of moments and axes must have same length > 0")
        dim = tuple(int(2 * I + 1) for I in Is)
        matrices = []
        for I, axis in zip(Is, axes):
            if I % 0.5 or I < 0.5:
                raise ValueError(f"{I} is not a valid spin value")
            if axis not in "xyz+-0":
                raise ValueError(f"{axis} is not a valid spin axis")
            matrices.append(_AXES[axis](_mvals(I)))
        M = matrices[0]
        for m in matrices[1:]:
            M = np.kron(M, m)
        return cls(M, dim=dim, use_sparse=use_sparse)


class DensityOperator(Operator):
    """Trace-one Hermitian operator (muspinsim/spinop.py:414-600): the
    matrix is normalised to unit trace on construction."""

    def __init__(self, matrix, dim=None, use_sparse=True):
        super(DensityOperator, self).__init__(matrix, dim, use_sparse=use_sparse)
        if self.trace == 0:
            raise ValueError("Can not define a DensityOperator with zero trace")
        self.normalize()
        if not self.is_hermitian:
            raise ValueError("DensityOperator must be hermitian!")

    @classmethod
    def from_vectors(cls, Is=0.5, vectors=[0, 0, 1], gammas=0, use_sparse=True):
        """Product state of spins polarised along `vectors`, off-diagonal
        elements scaled by 1 - gamma (muspinsim/spinop.py:455-530)."""
        if isinstance(Is, Number):
            Is = [Is]
        if len(np.array(vectors).shape) == 1:
            vectors = [vectors]
        if isinstance(gammas, Number):
            gammas = [gammas]
        if len(Is) != len(vectors) or len(Is) != len(gammas) or len(Is) == 0:
            raise ValueError("Arrays of moments, axes and gammas must have same length > 0")
        dim = tuple(int(2 * I + 1) for I in Is)
        matrices = []
        for I, vec, gamma in zip(Is, vectors, gammas):
            if I % 0.5 or I < 0.5:
                raise ValueError(f"{I} is not a valid spin value")
            if not len(vec) == 3:
                raise ValueError(f"{vec} is not a valid 3D vector")
            if gamma < 0 or gamma > 1:
                raise ValueError(f"{gamma} is not a valid gamma value")
            m = _pure_state(I, vec)
            m *= (1 - gamma) * np.ones(m.shape) + gamma * np.eye(m.shape[0])
            matrices.append(m)
        M = matrices[0]
        for m in matrices[1:]:
            M = np.kron(M, m)
        return cls(M, dim=dim, use_sparse=use_sparse)

    @property
    def trace(self):
        return self._mat.trace()

    def clone_sparse(self):
        """Copy with CSR storage (what basis_change(..., use_sparse=True)
        returns in the reference)."""
        ans = self.clone()
        ans._mat = _as_storage(ans._mat, True)
        return ans

    def normalize(self):
        """Rescale to unit trace in place."""
        self._mat = _as_storage(self._mat * (1 / self.trace), self.is_sparse)

    def partial_trace(self, trace_dim=None):
        """Trace out the listed subsystems (muspinsim/spinop.py:543-572)."""
        if trace_dim is None:
            trace_dim = []
        dim = list(self._factors)
        tdim = list(sorted(trace_dim))
        m = _dense(self._mat).reshape(dim + dim)
        while len(tdim) > 0:
            td = tdim.pop(-1)
            m = np.trace(m, axis1=td, axis2=td + len(dim))
            dim.pop(td)
        return DensityOperator(m, dim, use_sparse=self.is_sparse)

    def expectation(self, operator):
        """tr(rho O) (muspinsim/spinop.py:574-600)."""
        if not isinstance(operator, SpinOperator):
            raise TypeError("Argument must be a SpinOperator")
        if not operator.dimension == self.dimension:
            raise ValueError("SpinOperator and DensityOperator do not have compatible dimensions")
        O = operator.matrix
        R = self.matrix
        if sparse.issparse(O):
            return O.multiply(R.T).sum()
        return np.sum(np.asarray(O) * _dense(R).T)


class SuperOperator(Operator):
    """Linear map on operators, as a matrix acting on row-major vec(rho)
    (muspinsim/spinop.py:603-764).  Host algebra: the propagation it feeds
    runs on the GPU (muspinsim_gb300.lindbladian)."""

    def __init__(self, matrix, dim=None):
        n = matrix.shape[0] ** 0.5
        if int(n) != n:
            raise ValueError("Matrix rank should be a perfect square")
        if dim is None:
            dim = (int(n), int(n))
        super(SuperOperator, self).__init__(matrix, dim)

    @classmethod
    def left_multiplier(cls, operator):
        """L rho = O rho: O (x) 1."""
        m = operator.matrix
        return cls(sparse.kron(m, sparse.eye(m.shape[0])), operator.dimension + operator.dimension)

    @classmethod
    def right_multiplier(cls, operator):
        """L rho = rho O: 1 (x) O^T."""
        m = operator.matrix
        return cls(sparse.kron(sparse.eye(m.shape[0]), m.T), operator.dimension + operator.dimension)

    @classmethod
    def commutator(cls, operator):
        return cls.left_multiplier(operator) - cls.right_multiplier(operator)

    @classmethod
    def anticommutator(cls, operator):
        return cls.left_multiplier(operator) + cls.right_multiplier(operator)

    @classmethod
    def bracket(cls, operator):
        """L rho = O rho O^dag: O (x) conj(O)."""
        m = operator.matrix
        return cls(sparse.kron(m, m.conjugate()), operator.dimension + operator.dimension)

    # algebra: + and - only with other superoperators (or numbers); a
    # product with a plain Operator applies the map to it
    def _accepts(self, x):
        return isinstance(x, SuperOperator)

    def _binary(self, x, op):
        if op in "+-" and not isinstance(x, (SuperOperator, Number)):
            raise TypeError("Unsupported operation for SuperOperator")
        return super(SuperOperator, self)._binary(x, op)

    def __mul__(self, x):
        if isinstance(x, Operator) and not isinstance(x, SuperOperator):
            rho = _dense(x.matrix)
            return Operator(self.matrix.dot(rho.reshape(-1)).reshape(rho.shape), x.dimension)
        return super(SuperOperator, self).__mul__(x)

    def __rmul__(self, x):
        if isinstance(x, Operator) and not isinstance(x, SuperOperator):
            raise TypeError("Unsupported operation for Operator")
        return super(SuperOperator, self).__rmul__(x)


def spin_projectors(I, axis):
    """Spectral projectors of n . S for a single spin I along unit(axis).

    n . S has eigenvalues m = +I ... -I; its projectors follow exactly from
    Lagrange interpolation, P_m = prod_{m' != m} (n . S - m') / (m - m'),
    so no eigensolver is needed.  A zero axis is taken as z (the state the
    reference's eigh of a zero matrix selects).  Returns [(m, P_m)]."""
    v = np.asarray(axis, dtype=float)
    nrm = np.linalg.norm(v)
    v = np.array([0.0, 0.0, 1.0]) if nrm == 0 else v / nrm
    mv = _mvals(I)
    nS = v[0] * _Sx(mv) + v[1] * _Sy(mv) + v[2] * _Sz(mv)
    eye = np.eye(len(mv))
    out = []
    for m in mv:
        P = eye + 0.0j
        for m2 in mv:
            if m2 != m:
                P = P @ (nS - m2 * eye) / (m - m2)
        out.append((m, P))
    return out


def _pure_state(I, vec):
    """|psi><psi| for the +I eigenstate of vec . S, the state the reference
    picks as the top eigenvector (muspinsim/spinop.py:513-521)."""
    return spin_projectors(I, vec)[0][1]
