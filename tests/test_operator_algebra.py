"""Operator algebra of muspinsim_gb300.spinop on the host: the behaviour of
the reference's Operator / DensityOperator / SuperOperator
(muspinsim/spinop.py:85-355, 414-600, 603-764): results, storage, classes
and the exceptions of the contract."""

import numpy as np
import pytest
from scipy import sparse

from muspinsim_gb300.spinop import DensityOperator, Operator, SpinOperator, SuperOperator


def _rand(n, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))


@pytest.mark.parametrize("use_sparse", [True, False])
def test_arithmetic(use_sparse):
    A, B = _rand(4, 1), _rand(4, 2)
    a = Operator(A, (2, 2), use_sparse=use_sparse)
    b = Operator(B, (2, 2), use_sparse=use_sparse)
    dense = lambda o: o.matrix.toarray() if sparse.issparse(o.matrix) else o.matrix
    assert np.allclose(dense(a + b), A + B)
    assert np.allclose(dense(a - b), A - B)
    assert np.allclose(dense(a * b), A @ B)
    assert np.allclose(dense(a * 2.5), 2.5 * A) and np.allclose(dense(2.5 * a), 2.5 * A)
    assert np.allclose(dense(a / 4), A / 4)
    assert np.allclose(dense(a + 3), A + 3 * np.eye(4))
    assert np.allclose(dense(a - 3), A - 3 * np.eye(4))
    assert np.allclose(dense(a.dagger()), A.conj().T)
    assert (a + b).is_sparse == use_sparse and (a + b).dimension == (2, 2)
    assert a == Operator(A, (2, 2)) and not a == b and not a == A
    assert np.isclose(a.hilbert_schmidt(b), np.trace(A.conj().T @ B))
    k = a.kron(Operator(B[:2, :2]))
    assert k.dimension == (2, 2, 2) and np.allclose(dense(k), np.kron(A, B[:2, :2]))


def test_errors():
    with pytest.raises(ValueError, match="square"):
        Operator(np.zeros((2, 3)))
    with pytest.raises(ValueError, match="compatible"):
        Operator(np.eye(4), (3,))
    a, c = Operator(np.eye(4), (2, 2)), Operator(np.eye(4), (4,))
    for op, word in ((lambda: a + c, "add"), (lambda: a - c, "subtract"),
                     (lambda: a * c, "multiply")):
        with pytest.raises(ArithmeticError, match=word):
            op()
    for op in (lambda: a + "x", lambda: a * "x", lambda: a / a, lambda: "x" * a):
        with pytest.raises(TypeError):
            op()
    with pytest.raises(ValueError, match="Kronecker"):
        a.kron(np.eye(2))
    with pytest.raises(ValueError, match="zero trace"):
        DensityOperator(np.zeros((2, 2)))
    with pytest.raises(ValueError, match="hermitian"):
        DensityOperator(np.array([[1.0, 1.0], [0.0, 1.0]]))


def test_density_operator_and_subclass_results():
    rho = DensityOperator(np.diag([3.0, 1.0]))
    assert np.isclose(rho.trace, 1.0) and np.allclose(rho.matrix.toarray(), np.diag([0.75, 0.25]))
    s = SpinOperator.from_axes([0.5], "z")
    assert isinstance(s * 2.0, SpinOperator) and isinstance(rho + rho, DensityOperator)
    assert np.isclose(rho.expectation(s), 0.25)
    assert (s * 2.0).is_sparse
    pt = DensityOperator.from_vectors([0.5, 0.5], [[0, 0, 1], [1, 0, 0]], [0, 0]).partial_trace([1])
    assert pt.dimension == (2,) and np.allclose(pt.matrix.toarray(), np.diag([1.0, 0.0]))


def test_superoperator_algebra():
    H = SpinOperator.from_axes([0.5], "x")
    rho = DensityOperator.from_vectors([0.5], [[0, 0, 1]])
    L = SuperOperator.commutator(H)
    v = (L * rho).matrix.toarray()
    R, M = rho.matrix.toarray(), H.matrix.toarray()
    assert np.allclose(v, M @ R - R @ M)
    assert isinstance(L + L, SuperOperator) and isinstance(2 * L, SuperOperator)
    assert np.allclose((L - L).matrix.toarray(), 0)
    with pytest.raises(TypeError, match="SuperOperator"):
        L + H
    with pytest.raises(ArithmeticError):  # Operator * SuperOperator: different spaces
        H * L
    with pytest.raises(ValueError, match="perfect square"):
        SuperOperator(np.eye(3))
