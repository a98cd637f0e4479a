"""The gradient checker (oracle/port.py fast_snapshot_grad / fast_powder_grad)
pinned against central finite differences of the oracle's fast path, and the
torch term matrices against the numpy SpinSystem.  CPU only."""

import numpy as np
import pytest
import torch

from oracle import port
from tests.helpers import oracle_system, random_hermitian


def _herm(rng, n):
    return random_hermitian(rng, n)


def _loss(H, sig, d, t, g, w):
    return float(g @ (w * port.fast_evolve(H, sig, t, d)))


def richardson(f, h):
    """Central difference of f at 0 extrapolated from steps h and h / 2
    (truncation error O(h^4))."""
    c1 = (f(h) - f(-h)) / (2 * h)
    c2 = (f(h / 2) - f(-h / 2)) / h
    return (4 * c2 - c1) / 3


@pytest.mark.parametrize("degenerate", [False, True])
def test_snapshot_grad_matches_finite_differences(degenerate):
    rng = np.random.default_rng(7 + degenerate)
    n, d = 8, 4
    if degenerate:
        lam = np.array([-3.0, -3.0, -1.0, 0.5, 0.5, 0.5, 2.0, 4.0])
        Q, _ = np.linalg.qr(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
        H = Q @ np.diag(lam) @ Q.conj().T
    else:
        H = _herm(rng, n)
    p = rng.normal(size=3)
    sig = port.sigma_mu(p / np.linalg.norm(p))
    t = np.linspace(0, 2.0, 150)
    g = rng.normal(size=t.size)
    w = 0.7
    G = port.fast_snapshot_grad(H, sig, d, t, g, w)
    for k in range(3):
        D = _herm(rng, n)
        fd = richardson(lambda h: _loss(H + h * D, sig, d, t, g, w), 1e-5)
        an = np.real(np.sum(np.conj(G) * D))
        assert abs(fd - an) <= 1e-7 * max(1.0, abs(fd))


def test_powder_grad_field_matches_finite_differences():
    from muspinsim_gb300 import workloads

    wl = workloads.config5(n_orient=5, n_times=120)
    sy = oracle_system(wl.spins, wl.couplings)
    B = np.array([0.002, -0.001, 0.004])
    p = np.array([0.0, 0.0, 1.0])
    rng = np.random.default_rng(3)
    g = rng.normal(size=wl.times.size)
    GH, GB = port.fast_powder_grad(sy, wl.orientations, B, p, wl.times, g)
    # dL/dB (crystal frame) = sum_s R_s^T dL/dB_lab,s
    R = np.stack([np.column_stack([port.quat_rotate(port.orientation_quat(o)[0], e)
                                   for e in np.eye(3)]) for o in wl.orientations])
    an = np.einsum("sab,sa->b", R, GB)
    for a in range(3):
        e = np.eye(3)[a]
        fd = richardson(lambda h: g @ port.powder_average(sy, wl.orientations, B + h * e, p,
                                                          np.inf, wl.times), 1e-6)
        assert abs(fd - an[a]) <= 1e-7 * max(1.0, abs(fd))


def test_torch_terms_match_spin_system():
    from muspinsim_gb300 import workloads
    from muspinsim_gb300.adjoint import TorchSpinHamiltonian

    for wl in (workloads.config5(n_orient=2, n_times=4), workloads.config2(n_orient=2, n_times=4)):
        ref = wl.system().hamiltonian_matrix()
        th = TorchSpinHamiltonian(wl.spins, device=torch.device("cpu"))
        H = torch.zeros((th.n, th.n), dtype=torch.complex128)
        for kind, idx, val in wl.couplings:  # 1-based indices, electron = spin 2
            i, j = idx["i"] - 1, idx.get("j", 2) - 1
            if kind == "dipolar":
                H = H + th.dipolar(i, j, val)
            elif kind == "hyperfine":
                H = H + th.hyperfine(i, j, val)
            elif kind == "quadrupolar":
                H = H + th.quadrupolar(i, val)
        assert np.abs(H.numpy() - ref).max() <= 1e-12 * np.abs(ref).max()
        Z = wl.system().zeeman_operators()
        assert np.abs(th.Z.numpy() - Z).max() == 0.0
