"""Lindbladian superoperator with GPU propagation, API-compatible with
``muspinsim/lindbladian.py``.

``from_hamiltonian`` and ``add_dissipative_term`` build
L = -i [H, .] + sum_k g_k (A_k . A_k^dag - 1/2 {A_k^dag A_k, .}) on the host
(a small sparse superoperator, as in the reference); ``evolve`` and
``integrate_decaying`` run in ``libmspgpu`` (``msp_superop_evolve`` /
``msp_superop_integrate``, FP64): exp(2 pi L t) by scaling and squaring
and a pivoted LU solve of (1/tau - 2 pi L), where the reference uses a
dense non-Hermitian eigendecomposition -- the same quantities up to
rounding.
"""

import numpy as np

from muspinsim_gb300 import kernels
from muspinsim_gb300.hamiltonian import Hamiltonian
from muspinsim_gb300.spinop import DensityOperator, SpinOperator, SuperOperator, _dense
from muspinsim_gb300.validation import (
    validate_evolve_params,
    validate_integrate_decaying_params,
)


class Lindbladian(SuperOperator):
    @classmethod
    def from_hamiltonian(cls, H, dissipators=[]):
        """L from a Hamiltonian and (operator, rate) pairs
        (muspinsim/lindbladian.py:17-31)."""
        if not isinstance(H, Hamiltonian):
            raise ValueError("Must use Hamiltonian to create Lindbladian")
        L = -1.0j * SuperOperator.commutator(H)
        L = cls(L.matrix, L.dimension)
        for A, gamma in dissipators:
            L.add_dissipative_term(A, gamma)
        return L

    def add_dissipative_term(self, A, gamma=1.0):
        """(muspinsim/lindbladian.py:33-41)"""
        AA = A.dagger() * A
        Ld = gamma * (SuperOperator.bracket(A) - 0.5 * SuperOperator.anticommutator(AA))
        if Ld.dimension != self.dimension:
            raise ValueError("Invalid dissipation operator for this Lindbladian")
        self._mat = self._mat + Ld.matrix

    def _checked(self, rho0, operators):
        dim = rho0.dimension
        if self.dimension != dim * 2:
            raise ValueError("Incompatible rho0 dimension")
        if any([self.dimension != o.dimension * 2 for o in operators]):
            raise ValueError("Incompatible measure operator dimension")
        n = int(np.prod(dim))
        L = np.asarray(_dense(self.matrix), dtype=complex)
        rho = np.asarray(_dense(rho0.matrix), dtype=complex)
        ops = (np.array([_dense(o.matrix) for o in operators], dtype=complex)
               if operators else np.zeros((0, n, n), dtype=complex))
        return n, L, rho, ops

    def evolve(self, rho0, times, operators=[]):
        """Expectation values as a complex (T, n_ops) array, or the evolved
        DensityOperators when no operator is given
        (muspinsim/lindbladian.py:43-111).  Times in microseconds."""
        times = np.array(times)
        if isinstance(operators, SpinOperator):
            operators = [operators]
        validate_evolve_params(rho0, times, operators)
        n, L, rho, ops = self._checked(rho0, operators)
        out = kernels.superop_evolve(L, n, rho, ops, times.astype(np.float64)).cpu().numpy()
        if len(operators) > 0:
            return out
        return [DensityOperator(out[k].reshape(n, n), rho0.dimension) for k in range(len(times))]

    def integrate_decaying(self, rho0, tau, operators):
        """integral_0^inf <O>(t) exp(-t/tau) dt for each operator
        (muspinsim/lindbladian.py:113-173)."""
        if isinstance(operators, SpinOperator):
            operators = [operators]
        validate_integrate_decaying_params(rho0, tau, operators)
        n, L, rho, ops = self._checked(rho0, operators)
        return kernels.superop_integrate(L, n, rho, ops, float(tau)).cpu().numpy()
