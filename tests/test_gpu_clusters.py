"""Mixed-precision refinement on clustered spectra: near-degenerate levels
(level anticrossings) and exactly degenerate multiplets of three to ten
levels, at n <= 64 (Jacobi kernels) and n > 64 (Householder + QL kernels).

The mixed form's gate is max|dP| <= 1e-6 against the oracle; eigenvalues
to 1e-11 of max|lambda|.  The reference has no such mode: it calls LAPACK
(np.linalg.eigh, muspinsim/spinop.py:69) in FP64 throughout.
"""

import numpy as np
import pytest

from oracle import port

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6


@pytest.fixture(scope="module")
def K():
    from muspinsim_gb300 import kernels

    kernels.device()
    return kernels


def clustered_hermitian(n, clusters, seed, scale=300.0):
    """A random-basis Hermitian matrix whose spectrum holds, at random
    places, the given clusters: (levels, relative spacing) each."""
    rng = np.random.default_rng(seed)
    lam = np.sort(rng.uniform(-scale, scale, n))
    pos = 0
    for k, gap in clusters:
        for t in range(k):
            lam[pos + t] = lam[pos] + t * gap * scale
        pos += k + 2
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    V, _ = np.linalg.qr(A)
    H = (V * lam) @ V.conj().T
    return 0.5 * (H + H.conj().T)


CASES = [
    (8, [(3, 1e-6)]),
    (24, [(3, 1e-6), (2, 1e-8)]),
    (32, [(4, 0.0), (3, 3e-5)]),
    (64, [(10, 1e-7), (3, 1e-5)]),
    (96, [(10, 1e-9), (3, 1e-6)]),
    (128, [(10, 0.0), (5, 1e-6), (3, 3e-5)]),
]


@pytest.mark.parametrize("n,clusters", [c for c in CASES if c[0] <= 64])
def test_eigh_mixed_clustered(K, n, clusters):
    """Batched mixed eigensolve: FP64-level eigenvalues and FP32-level
    eigenpairs on spectra with near-degenerate and degenerate clusters."""
    from muspinsim_gb300 import _lib

    H = np.stack([clustered_hermitian(n, clusters, seed) for seed in range(4)])
    ev, U, st = K.eigh(H, precision=_lib.PREC_MIXED)
    ev, U, st = ev.cpu().numpy(), U.cpu().numpy(), st.cpu().numpy()
    assert np.all(st == 0)
    for b in range(H.shape[0]):
        ref = np.linalg.eigvalsh(H[b])
        scale = np.abs(ref).max()
        assert np.abs(ev[b] - ref).max() <= 1e-11 * scale
        assert np.abs(U[b].conj().T @ U[b] - np.eye(n)).max() <= 2e-6
        res = H[b] @ U[b] - U[b] * ev[b][None, :]
        assert np.abs(res).max() <= 2e-6 * scale


def _fast_reference(H, pols, times):
    d = H.shape[0] // 2
    out = np.zeros(len(times))
    for p in pols:
        out += port.fast_evolve(H, port.sigma_mu(p), times, d) / len(pols)
    return out


def _powder(K, H, pols, times, precision, max_refine=0):
    from muspinsim_gb300 import _lib

    n = H.shape[0]
    S = len(pols)
    out, st = K.powder_run(n, H, np.zeros((3, n, n), complex), np.zeros((S, 3)), pols,
                           np.full(S, 1.0 / S), np.zeros(S, np.int32), 1, times,
                           precision=precision, max_refine=max_refine)
    return out.cpu().numpy()[0], st.cpu().numpy()


@pytest.mark.parametrize("n,clusters", CASES)
def test_powder_mixed_clustered(K, n, clusters):
    """Fast-path powder average of a clustered Hamiltonian in both
    precisions against the oracle, and no refinement-limit flag."""
    from muspinsim_gb300 import _lib

    rng = np.random.default_rng(n)
    pols = rng.standard_normal((6, 3))
    pols /= np.linalg.norm(pols, axis=1, keepdims=True)
    times = np.linspace(0.0, 20.0, 300)
    H = clustered_hermitian(n, clusters, seed=n + 1)
    ref = _fast_reference(H, pols, times)
    got, st = _powder(K, H, pols, times, _lib.PREC_FP64)
    assert np.all(st == 0)
    assert np.abs(got - ref).max() <= 1e-10
    got, st = _powder(K, H, pols, times, _lib.PREC_MIXED)
    assert np.all(st == 0)
    assert np.abs(got - ref).max() <= MIXED_TOL


@pytest.mark.parametrize("n", [24, 128])
def test_refinement_limit_flag(K, n):
    """A refinement capped at one step on a spectrum whose FP32 eigenvectors
    mix near-degenerate levels by large angles reports
    MSP_ITEM_REFINE_LIMIT; with the default cap it does not."""
    from muspinsim_gb300 import _lib

    H = clustered_hermitian(n, [(3, 1e-7), (4, 1e-8)], seed=5)
    pols = np.array([[0.0, 0.0, 1.0], [1.0, 0.0, 0.0]])
    times = np.linspace(0.0, 10.0, 64)
    _, st1 = _powder(K, H, pols, times, _lib.PREC_MIXED, max_refine=1)
    assert np.all(st1 & _lib.MSP_ITEM_REFINE_LIMIT)
    assert not np.any(st1 & _lib.MSP_ITEM_NOT_CONVERGED)
    _, st = _powder(K, H, pols, times, _lib.PREC_MIXED)
    assert np.all(st == 0)
