"""Spin Hamiltonian with GPU time evolution, API-compatible with
``muspinsim/hamiltonian.py``.

``evolve``, ``integrate_decaying`` and ``fast_evolve`` keep the reference's
signatures, return types and exceptions; the diagonalisation, the changes of
basis and the sums over eigenvalue pairs run in ``libmspgpu`` (FP64).
"""

import numpy as np

from muspinsim_gb300 import kernels
from muspinsim_gb300.spinop import DensityOperator, Hermitian, Operator, SpinOperator, _dense
from muspinsim_gb300.validation import (
    validate_evolve_params,
    validate_integrate_decaying_params,
    validate_times,
)


class Hamiltonian(Operator, Hermitian):
    def __init__(self, matrix, dim=None, use_sparse=True):
        """Hermitian matrix in MHz; ValueError if not square or not
        Hermitian within 1e-6 (muspinsim/hamiltonian.py:20-34)."""
        super(Hamiltonian, self).__init__(matrix, dim, use_sparse=use_sparse)

    @classmethod
    def from_spin_operator(cls, spinop):
        return cls(spinop.matrix, spinop.dimension)

    def _eigenbasis(self, rho0, operators):
        evals, evecs = self.diag()
        U = np.asarray(evecs)
        mats = [_dense(rho0.matrix)] + [_dense(o.matrix) for o in operators]
        rot = kernels.basis_change(U, np.asarray(mats, dtype=complex))
        return evals, U, rot[0], rot[1:]

    def evolve(self, rho0, times, operators=None):
        """Expectation values <O>(t) as a complex (T, n_ops) array, or the list
        of evolved DensityOperators when no operator is given
        (muspinsim/hamiltonian.py:40-117).  Times in microseconds."""
        if operators is None:
            operators = []
        times = np.array(times)
        if isinstance(operators, SpinOperator):
            operators = [operators]
        validate_evolve_params(rho0, times, operators)
        dim = rho0.dimension
        evals, U, rho_e, ops_e = self._eigenbasis(rho0, operators)
        if len(operators) > 0:
            out = kernels.evolve_expect(evals, rho_e, ops_e, times.astype(np.float64))
            return out.cpu().numpy()
        # density matrices: U (exp(-i w t) o rho') U^dag for every time
        ph = kernels.evolve_phases(evals, rho_e, times.astype(np.float64))
        back = kernels.basis_change(U, ph, adjoint=True).cpu().numpy()
        return [DensityOperator(back[i], dim).clone_sparse() for i in range(len(times))]

    def integrate_decaying(self, rho0, tau, operators):
        """integral_0^inf <O>(t) exp(-t/tau) dt for each operator, complex
        array (muspinsim/hamiltonian.py:119-164)."""
        if isinstance(operators, SpinOperator):
            operators = [operators]
        validate_integrate_decaying_params(rho0, tau, operators)
        evals, U, rho_e, ops_e = self._eigenbasis(rho0, operators)
        return kernels.integrate_decaying(evals, rho_e, ops_e, tau).cpu().numpy()

    def fast_evolve(self, sigma_mu, times, other_dimension):
        """Muon polarisation for a muon-first system at T = inf:
        0.5 (1/d) [1/2 sum_j A_jj + sum_{k<j} A_jk cos(W_jk t)] with
        A = |U^dag (sigma (x) 1_d) U|^2 (muspinsim/hamiltonian.py:166-217)."""
        times = np.array(times)
        validate_times(times)
        evals, evecs = self.diag()
        sig = np.asarray(_dense(sigma_mu), dtype=complex)
        A, W = kernels.fast_amplitudes(evals, evecs, sig, int(other_dimension))
        res = kernels.fast_cos_sum(times.astype(np.float64), int(other_dimension), A, W)
        return res.cpu().numpy() * 0.5

