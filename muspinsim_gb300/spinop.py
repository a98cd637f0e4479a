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
    """Mixin for Hermitian operators (muspinsim/spinop.py:44-82)."""

    def __init__(self):
        if not self.is_hermitian:
            raise ValueError("Operator must be hermitian")

    def diag(self):
        """Eigenvalues (ascending) and eigenvector matrix (columns), as
        numpy.linalg.eigh returns them, computed by the GPU Jacobi solver in
        FP64.  The result is cached while the matrix is unchanged."""
        M = _dense(self._matrix)
        dd = getattr(self, "_diagdata", None)
        if dd is not None and dd["matrix"].shape == M.shape and np.array_equal(dd["matrix"], M):
            return dd["eigh"]
        evals, evecs, status = kernels.eigh(M[None])
        if int(status[0].item()) != 0:
            raise RuntimeError("Hermitian.diag: the Jacobi eigensolver did not converge")
        eigh = (evals[0].cpu().numpy(), evecs[0].cpu().numpy())
        self._diagdata = {"matrix": M.copy(), "eigh": eigh}
        return eigh


class Operator(Clonable):
    """A spin-space operator (muspinsim/spinop.py:85-355)."""

    def __init__(self, matrix, dim=None, herm_tol=1e-6, use_sparse=True):
        self._sparse = use_sparse
        if self._sparse:
            self._matrix = sparse.csr_matrix(matrix)
        else:
            self._matrix = np.array(matrix)
        if not matrix.shape[0] == matrix.shape[1]:
            raise ValueError("Matrix passed to Operator must be square")
        if dim is None:
            dim = (matrix.shape[0],)
        elif np.prod(dim) != matrix.shape[0]:
            raise ValueError("Dimensions are not compatible with matrix")
        self._dim = tuple(dim)
        self._htol = herm_tol
        super(Operator, self).__init__()

    @property
    def Is(self):
        return tuple((d - 1) / 2.0 for d in self._dim)

    @property
    def dimension(self):
        return self._dim

    @property
    def N(self):
        return np.prod(self._dim)

    @property
    def matrix(self):
        return self._matrix

    @property
    def is_hermitian(self):
        x = self._matrix.conjugate().T
        y = self._matrix
        return np.abs(y - x).max() < self._htol

    @property
    def is_sparse(self):
        return self._sparse

    def dagger(self):
        cls = self.__class__
        ans = cls.__new__(cls)
        ans._dim = tuple(self._dim)
        ans._matrix = self.matrix.conjugate().T
        ans._sparse = self._sparse
        ans._htol = getattr(self, "_htol", 1e-6)
        return ans

    def __add__(self, x):
        if isinstance(x, Operator):
            if self.dimension != x.dimension:
                raise ArithmeticError("Can not add to Operators with different dimensions")
            ans = self.clone()
            ans._matrix = ans._matrix + x._matrix
            return ans
        elif isinstance(x, Number):
            ans = self.clone()
            if self._sparse:
                ans._matrix = ans._matrix + sparse.eye(ans._matrix.shape[0]) * x
            else:
                ans._matrix = ans._matrix + np.eye(ans._matrix.shape[0]) * x
            return ans
        raise TypeError("Unsupported operation for Operator")

    def __sub__(self, x):
        if isinstance(x, Operator):
            if self.dimension != x.dimension:
                raise ArithmeticError("Can not subtract to Operators with different dimensions")
            ans = self.clone()
            ans._matrix = ans._matrix - x._matrix
            return ans
        elif isinstance(x, Number):
            return self + (-x)
        raise TypeError("Unsupported operation for Operator")

    def __mul__(self, x):
        if isinstance(x, Operator):
            if self.dimension != x.dimension:
                raise ArithmeticError("Can not multiply to Operators with different dimensions")
            ans = self.clone()
            if self._sparse:
                ans._matrix = ans._matrix.dot(x._matrix)
            else:
                ans._matrix = ans._matrix @ x._matrix
            return ans
        elif isinstance(x, Number):
            ans = self.clone()
            if self._sparse:
                ans._matrix = ans._matrix.multiply(x).tocsr()
            else:
                ans._matrix = ans._matrix * x
            return ans
        raise TypeError("Unsupported operation for Operator")

    def __rmul__(self, x):
        if isinstance(x, Number):
            return self.__mul__(x)
        elif isinstance(x, Operator):
            return x * self
        raise TypeError("Unsupported operation for Operator")

    def __truediv__(self, x):
        if isinstance(x, Number):
            return self * (1.0 / x)
        raise TypeError("Unsupported operation for Operator")

    def __eq__(self, x):
        if not isinstance(x, Operator):
            return False
        if self.dimension != x.dimension:
            return False
        return bool(np.array_equal(_dense(self._matrix), _dense(x._matrix)))

    __hash__ = None

    def kron(self, x):
        """Tensor product (muspinsim/spinop.py:266-295)."""
        if not isinstance(x, Operator):
            raise ValueError("Can only perform Kronecker product with another Operator")
        ans = self.__class__.__new__(self.__class__)
        ans._dim = self._dim + x._dim
        ans._sparse = self._sparse
        ans._htol = getattr(self, "_htol", 1e-6)
        if self._sparse:
            ans._matrix = sparse.kron(self._matrix, x._matrix, format="csr")
        else:
            ans._matrix = np.kron(self._matrix, x._matrix)
        return ans

    def hilbert_schmidt(self, x):
        """tr(A^dag B) (muspinsim/spinop.py:297-328)."""
        if not isinstance(x, Operator):
            raise ValueError("Can only perform Hilbert-Schmidt product with another Operator")
        if not x.dimension == self.dimension:
            raise ValueError(
                "Operators must have the same dimension to perform Hilbert-Schmidt product"
            )
        A = self.matrix
        B = x.matrix
        return A.conjugate().T.dot(B).trace().item()

    def basis_change(self, basis, use_sparse=False):
        """basis^dag M basis, computed on the GPU (muspinsim/spinop.py:330-355)."""
        ans = self.clone()
        M = _dense(ans._matrix)
        out = kernels.basis_change(np.asarray(basis, dtype=complex), M.astype(complex))[0]
        ans._matrix = out.cpu().numpy()
        if use_sparse:
            ans._matrix = sparse.csr_matrix(ans._matrix)
        ans._sparse = use_sparse
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
    """Trace-one Hermitian operator (muspinsim/spinop.py:414-600)."""

    def __init__(self, matrix, dim=None, use_sparse=True):
        super(DensityOperator, self).__init__(matrix, dim, use_sparse=use_sparse)
        tr = self._matrix.trace()
        if tr == 0:
            raise ValueError("Can not define a DensityOperator with zero trace")
        else:
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
        return self._matrix.trace()

    def clone_sparse(self):
        """Copy with CSR storage (what basis_change(..., use_sparse=True)
        returns in the reference)."""
        ans = self.clone()
        ans._matrix = sparse.csr_matrix(_dense(ans._matrix))
        ans._sparse = True
        return ans

    def normalize(self):
        if self._sparse:
            self._matrix = self._matrix.multiply(1 / self.trace).tocsr()
        else:
            self._matrix = np.multiply(self._matrix, 1 / self.trace)

    def partial_trace(self, trace_dim=None):
        """Trace out the listed subsystems (muspinsim/spinop.py:543-572)."""
        if trace_dim is None:
            trace_dim = []
        dim = list(self._dim)
        tdim = list(sorted(trace_dim))
        m = _dense(self._matrix).reshape(dim + dim)
        while len(tdim) > 0:
            td = tdim.pop(-1)
            m = np.trace(m, axis1=td, axis2=td + len(dim))
            dim.pop(td)
        return DensityOperator(m, dim, use_sparse=self._sparse)

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

    def __add__(self, x):
        if isinstance(x, (SuperOperator, Number)):
            return super(SuperOperator, self).__add__(x)
        raise TypeError("Unsupported operation for SuperOperator")

    def __sub__(self, x):
        if isinstance(x, (SuperOperator, Number)):
            return super(SuperOperator, self).__sub__(x)
        raise TypeError("Unsupported operation for SuperOperator")

    def __mul__(self, x):
        if isinstance(x, (SuperOperator, Number)):
            return super(SuperOperator, self).__mul__(x)
        elif isinstance(x, Operator):
            m = _dense(x.matrix)
            v = self.matrix.dot(m.reshape((-1,))).reshape(m.shape)
            return Operator(v, x.dimension)
        raise TypeError("Unsupported operation for Operator")

    def __rmul__(self, x):
        if isinstance(x, Number):
            return self.__mul__(x)
        elif isinstance(x, SuperOperator):
            return x * self
        raise TypeError("Unsupported operation for Operator")

    def __truediv__(self, x):
        if isinstance(x, Number):
            return self * (1.0 / x)
        raise TypeError("Unsupported operation for Operator")


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
