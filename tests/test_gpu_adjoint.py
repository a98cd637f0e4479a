"""CUDA adjoint of the fast-path powder average (msp_adjoint_fast) against
the gradient checker (oracle/port.py, itself pinned by finite differences),
autograd through TorchSpinHamiltonian against finite differences of the
oracle, and a gradient-based fit of config-5-shaped data."""

import numpy as np
import pytest
import torch

from oracle import port
from tests.helpers import oracle_system

pytestmark = pytest.mark.gpu


def _geometry(wl, B):
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300.orientations import orientation_rows_to_quats

    qs, ws = orientation_rows_to_quats(wl.orientations)
    N = len(qs)
    w = ws * (N / ws.sum()) / N
    p = wl.polarization / np.linalg.norm(wl.polarization)
    return Q.rotate(qs, B), Q.rotate(qs, p), w


@pytest.mark.parametrize("B", [(0.0, 0.0, 0.0), (0.002, -0.001, 0.004)])
@pytest.mark.parametrize("uniform", [True, False])
def test_adjoint_matches_checker(B, uniform):
    from muspinsim_gb300 import kernels, workloads

    wl = workloads.config5(n_orient=40, n_times=400)
    times = wl.times if uniform else np.sort(np.random.default_rng(2).uniform(0, 20, 400))
    sy = wl.system()
    Hs, Z = sy.hamiltonian_matrix(), sy.zeeman_operators()
    B = np.asarray(B, dtype=float)
    Bl, pl, w = _geometry(wl, B)
    g = np.random.default_rng(11).normal(size=times.size)
    gH, gF, st = kernels.adjoint_fast(Hs.shape[0], Hs, Z, Bl, pl, w, np.zeros(len(w), np.int32), 1,
                                      times, g)
    assert int(st.max()) == 0
    GH, GB = port.fast_powder_grad(oracle_system(wl.spins, wl.couplings), wl.orientations, B,
                                   wl.polarization, times, g)
    gH, gF = gH.cpu().numpy(), gF.cpu().numpy()
    assert np.abs(gH - GH).max() <= 1e-9 * np.abs(GH).max()
    # at B = 0 the field gradient vanishes by symmetry (P is even in B): scale
    # the tolerance by |dL/dH| |Z|, the size a field gradient would have
    scale = max(np.abs(GB).max(), np.abs(GH).max() * np.abs(Z).max())
    assert np.abs(gF - GB).max() <= 1e-9 * scale


def _dipolar_model(th, dirs, fixed):
    """Hsys of mu-F-F with mu-F distances as parameters (directions fixed)."""
    def model(params):
        d1, d2 = params
        H = th.dipolar(0, 1, d1 * dirs[0]) + th.dipolar(0, 2, d2 * dirs[1]) + fixed
        return H, torch.zeros(3, dtype=torch.float64, device=th.device)
    return model


def _oracle_loss(wl, r1, r2, r3, data):
    coup = [("dipolar", {"i": 1, "j": 2}, r1), ("dipolar", {"i": 1, "j": 3}, r2),
            ("dipolar", {"i": 2, "j": 3}, r3)]
    sy = oracle_system(wl.spins, coup)
    P = port.powder_average(sy, wl.orientations, np.zeros(3), wl.polarization, np.inf, wl.times)
    return float(((P - data) ** 2).sum())


def test_autograd_distances_vs_finite_differences():
    from muspinsim_gb300 import workloads
    from muspinsim_gb300.adjoint import GradientFitter, TorchSpinHamiltonian

    wl = workloads.config5(n_orient=30, n_times=300)
    r = [np.asarray(v, dtype=float) for _, _, v in wl.couplings]
    dirs = [r[0] / np.linalg.norm(r[0]), r[1] / np.linalg.norm(r[1])]
    th = TorchSpinHamiltonian(wl.spins)
    fixed = th.dipolar(1, 2, r[2])
    data = np.random.default_rng(4).normal(scale=0.05, size=wl.times.size) + 0.3
    fit = GradientFitter(_dipolar_model(th, [torch.as_tensor(x, device=th.device) for x in dirs],
                                        fixed), th.Z, wl.orientations, wl.times, data,
                         wl.polarization)
    d0 = [float(np.linalg.norm(r[0])) * 1.01, float(np.linalg.norm(r[1])) * 0.99]
    ps = [torch.tensor(v, dtype=torch.float64, device=th.device, requires_grad=True) for v in d0]
    L, grads = fit.loss_and_grad(ps)
    L_or = _oracle_loss(wl, d0[0] * dirs[0], d0[1] * dirs[1], r[2], data)
    assert abs(float(L) - L_or) <= 1e-10 * max(1.0, abs(L_or))
    for k in range(2):
        def f(h):
            d = list(d0)
            d[k] += h
            return _oracle_loss(wl, d[0] * dirs[0], d[1] * dirs[1], r[2], data)
        h = 1e-5
        fd = (4 * (f(h / 2) - f(-h / 2)) / h - (f(h) - f(-h)) / (2 * h)) / 3
        assert abs(float(grads[k]) - fd) <= 1e-6 * max(1.0, abs(fd))


def test_gradient_fit_recovers_distances():
    from muspinsim_gb300 import workloads
    from muspinsim_gb300.adjoint import GradientFitter, TorchSpinHamiltonian

    wl = workloads.config5(n_orient=200, n_times=400)
    r = [np.asarray(v, dtype=float) for _, _, v in wl.couplings]
    true = [float(np.linalg.norm(r[0])), float(np.linalg.norm(r[1]))]
    dirs = [torch.as_tensor(r[k] / true[k]) for k in range(2)]
    th = TorchSpinHamiltonian(wl.spins)
    fixed = th.dipolar(1, 2, r[2])
    data = port.powder_average(oracle_system(wl.spins, wl.couplings), wl.orientations, np.zeros(3),
                               wl.polarization, np.inf, wl.times)
    fit = GradientFitter(_dipolar_model(th, [x.to(th.device) for x in dirs], fixed), th.Z,
                         wl.orientations, wl.times, data, wl.polarization)
    res = fit.fit([np.array(true[0] * 1.03), np.array(true[1] * 0.97)],
                  options={"maxiter": 200, "gtol": 1e-12})
    got = [float(p) for p in res.params]
    print("fit:", got, "true:", true, "evaluations:", fit.evaluations)
    assert abs(got[0] - true[0]) <= 1e-5 and abs(got[1] - true[1]) <= 1e-5
