"""GPU parity of the CUDA kernels against the CPU oracle (oracle/port.py).

Tolerances: FP64 path max|dP| <= 1e-10 and eigenvalues <= 1e-12 relative
to max|lambda|; mixed path max|dP| <= 1e-6 on powder averages.
"""

import numpy as np
import pytest

from oracle import port
from tests.helpers import oracle_powder, oracle_system, random_hermitian

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-6


@pytest.fixture(scope="module")
def K():
    from muspinsim_gb300 import kernels

    kernels.device()
    return kernels


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 12, 16, 24, 31, 32, 48, 64])
def test_eigh_fp64_random(K, n):
    rng = np.random.default_rng(100 + n)
    H = np.stack([random_hermitian(rng, n) for _ in range(6)])
    ev, U, st = K.eigh(H)
    ev, U, st = ev.cpu().numpy(), U.cpu().numpy(), st.cpu().numpy()
    assert np.all(st == 0)
    for b in range(H.shape[0]):
        ref = np.linalg.eigvalsh(H[b])
        scale = np.abs(ref).max()
        assert np.abs(ev[b] - ref).max() <= 1e-12 * scale
        assert np.all(np.diff(ev[b]) >= 0)
        rec = (U[b] * ev[b][None, :]) @ U[b].conj().T
        assert np.abs(rec - H[b]).max() <= 1e-12 * scale
        assert np.abs(U[b].conj().T @ U[b] - np.eye(n)).max() <= 1e-12


@pytest.mark.parametrize("n", [4, 8, 24, 32, 64])
def test_eigh_mixed_random(K, n):
    from muspinsim_gb300 import _lib

    rng = np.random.default_rng(200 + n)
    H = np.stack([random_hermitian(rng, n) for _ in range(6)])
    ev, U, st = K.eigh(H, precision=_lib.PREC_MIXED)
    ev, U, st = ev.cpu().numpy(), U.cpu().numpy(), st.cpu().numpy()
    assert np.all(st == 0)
    for b in range(H.shape[0]):
        ref = np.linalg.eigvalsh(H[b])
        scale = np.abs(ref).max()
        # refined eigenvalues: FP64-level; eigenvectors stored in FP32
        assert np.abs(ev[b] - ref).max() <= 1e-11 * scale
        assert np.abs(U[b].conj().T @ U[b] - np.eye(n)).max() <= 2e-6


def test_eigh_degenerate_and_trivial(K):
    rng = np.random.default_rng(7)
    n = 24
    Qm, _ = np.linalg.qr(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    lam = np.repeat([-3.0, 0.5, 0.5 + 1e-9, 2.0], 6)
    H = np.stack([(Qm * lam) @ Qm.conj().T, np.zeros((n, n)), np.eye(n) * 5.0,
                  np.diag(np.arange(n, dtype=float))])
    ev, U, st = K.eigh(H)
    ev, U = ev.cpu().numpy(), U.cpu().numpy()
    assert np.all(st.cpu().numpy() == 0)
    for b in range(H.shape[0]):
        ref = np.linalg.eigvalsh(H[b])
        assert np.abs(ev[b] - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1.0)
        rec = (U[b] * ev[b][None, :]) @ U[b].conj().T
        assert np.abs(rec - H[b]).max() <= 1e-12 * max(np.abs(ref).max(), 1.0)


def test_fast_cos_sum_matches_oracle(K):
    rng = np.random.default_rng(3)
    n = 24
    H = random_hermitian(rng, n)
    A, W, _ = port.fast_amplitudes(H, port.sigma_mu([0, 0, 1.0]), n // 2)
    t = np.linspace(0, 20, 777)
    ref = port.fast_cos_sum(t, n // 2, A, W)
    got = K.fast_cos_sum(t, n // 2, A, W).cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-13


def _workload2(n_orient=24, n_times=640):
    from muspinsim_gb300 import workloads

    return workloads.config2(n_orient=n_orient, n_times=n_times)


def _gpu_powder(wl, precision="fp64", **kw):
    from muspinsim_gb300.powder import powder_average

    sy = wl.system()
    args = dict(orientations=wl.orientations, field=wl.fields[0], polarization=wl.polarization,
                times=wl.times, temperature=wl.temperature, y_axis=wl.y_axis)
    args.update(kw)
    return powder_average(sy, precision=precision, **args)


def test_powder_fast_fp64_vs_oracle():
    wl = _workload2()
    ref = oracle_powder(wl)
    got = _gpu_powder(wl)
    assert np.abs(got - ref).max() <= FP64_TOL


def test_powder_fast_mixed_vs_oracle():
    wl = _workload2()
    ref = oracle_powder(wl)
    got = _gpu_powder(wl, "mixed")
    assert np.abs(got - ref).max() <= MIXED_TOL


def test_powder_fast_nonuniform_times():
    wl = _workload2(n_orient=8, n_times=300)
    rng = np.random.default_rng(11)
    t = np.sort(rng.uniform(0, 20, 300))
    ref = oracle_powder(wl, times=t)
    got = _gpu_powder(wl, times=t)
    assert np.abs(got - ref).max() <= FP64_TOL
    got_m = _gpu_powder(wl, "mixed", times=t)
    assert np.abs(got_m - ref).max() <= MIXED_TOL


def test_powder_multi_tile_times():
    # more than one 4096-sample tile, with a ragged last tile
    wl = _workload2(n_orient=4, n_times=9000)
    ref = oracle_powder(wl)
    got = _gpu_powder(wl)
    assert np.abs(got - ref).max() <= FP64_TOL


def test_powder_evolve_finite_temperature():
    wl = _workload2(n_orient=10, n_times=400)
    ref = oracle_powder(wl, temperature=5.0)
    got = _gpu_powder(wl, temperature=5.0)
    assert np.abs(got - ref).max() <= FP64_TOL
    got_m = _gpu_powder(wl, "mixed", temperature=5.0)
    assert np.abs(got_m - ref).max() <= MIXED_TOL


def test_powder_evolve_muon_not_first():
    from muspinsim_gb300.spinsys import MuonSpinSystem
    from muspinsim_gb300.powder import powder_average

    rng = np.random.default_rng(21)
    spins = ["e", "mu", "H"]
    A1 = rng.normal(0, 50, (3, 3))
    A1 = A1 + A1.T
    A2 = rng.normal(0, 5, (3, 3))
    A2 = A2 + A2.T
    coup = [("hyperfine", {"i": 2, "j": 1}, A1), ("hyperfine", {"i": 3, "j": 1}, A2)]
    sy = MuonSpinSystem(spins)
    sy.add_hyperfine_term(1, A1, 0)
    sy.add_hyperfine_term(2, A2, 0)
    orients = [(0.1, 0.2, 0.3), (1.0, 2.0, 0.5, 2.0), (0.7, 1.1)]
    t = np.linspace(0, 5, 333)
    B = np.array([0.0, 0.01, 0.02])
    p = np.array([1.0, 0.0, 0.0])
    ref = port.powder_average(oracle_system(spins, coup), orients, B, p, np.inf, t)
    got = powder_average(sy, orients, B, p, t)
    assert np.abs(got - ref).max() <= FP64_TOL


def test_powder_integral_vs_oracle():
    from muspinsim_gb300 import workloads

    wl = workloads.config3(n_fields=4, n_orient=6)
    e64, emx = [], []
    for B in wl.fields:
        ref = oracle_powder(wl, field=B)
        e64.append(abs(_gpu_powder(wl, field=B) - ref))
        emx.append(abs(_gpu_powder(wl, "mixed", field=B) - ref))
    print("integral |dP| fp64:", e64, "mixed:", emx)
    assert max(e64) <= FP64_TOL
    assert max(emx) <= MIXED_TOL


def test_mixed_single_orientations():
    """Mixed precision per crystallite (no powder averaging to hide errors)."""
    from muspinsim_gb300 import workloads

    wl = workloads.config2(n_orient=12, n_times=1024)
    errs = []
    for o in wl.orientations:
        ref = oracle_powder(wl, orientations=[o])
        got = _gpu_powder(wl, "mixed", orientations=[o])
        errs.append(np.abs(got - ref).max())
    print("mixed per-orientation max|dP|:", max(errs))
    assert max(errs) <= 5e-7


# Snapshots of a dense ALC scan (dim 32, fields linspace(0, 1, 500) T along
# z, 24 ZCW-style orientations) whose Hamiltonians have level pairs within
# a few FP32 resolutions of |H| (gap / max|lambda| ~ 2e-7 .. 6e-7): FP32
# Jacobi leaves them mixed by angles up to ~0.5.  (field index, orientation)
NEAR_DEGENERATE = [(352, 21), (447, 20), (199, 12), (107, 17)]


def _alc_scan():
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300 import workloads
    from muspinsim_gb300.orientations import orientation_rows_to_quats

    wl = workloads.config3(n_fields=500, n_orient=24)
    qs, ws = orientation_rows_to_quats(wl.orientations)
    return wl, qs, ws, Q


def test_eigh_mixed_near_degenerate(K):
    from muspinsim_gb300 import _lib

    wl, qs, _, Q = _alc_scan()
    sy = wl.system()
    Hs, Z = sy.hamiltonian_matrix(), sy.zeeman_operators()
    H = np.stack([Hs + np.einsum("a,aij->ij", Q.rotate(qs[o:o + 1], wl.fields[f])[0], Z)
                  for f, o in NEAR_DEGENERATE])
    ev, U, st = K.eigh(H, precision=_lib.PREC_MIXED)
    ev, U, st = ev.cpu().numpy(), U.cpu().numpy(), st.cpu().numpy()
    assert np.all(st == 0)
    n = H.shape[1]
    for b in range(H.shape[0]):
        ref = np.linalg.eigvalsh(H[b])
        scale = np.abs(ref).max()
        assert np.diff(ref).min() < 1e-6 * scale  # the case is what it claims to be
        assert np.abs(ev[b] - ref).max() <= 1e-12 * scale
        assert np.abs(U[b].conj().T @ U[b] - np.eye(n)).max() <= 1e-6
        assert np.abs(H[b] @ U[b] - U[b] * ev[b][None, :]).max() <= 1e-6 * scale


def test_alc_integral_mixed_near_degenerate():
    """Orientation-averaged ALC integrals at the fields of the near-degenerate
    snapshots: mixed against FP64 and against the oracle."""
    from muspinsim_gb300 import _lib, constants, kernels

    wl, qs, ws, Q = _alc_scan()
    sy = wl.system()
    Hs, Z = sy.hamiltonian_matrix(), sy.zeeman_operators()
    fields = sorted({f for f, _ in NEAR_DEGENERATE})
    N = len(qs)
    w = ws * (N / ws.sum()) / N
    B = np.concatenate([Q.rotate(qs, wl.fields[f]) for f in fields])
    P = np.tile(Q.rotate(qs, wl.polarization), (len(fields), 1))
    W = np.tile(w, len(fields))
    slot = np.repeat(np.arange(len(fields)), N).astype(np.int32)
    out = {}
    for prec in (_lib.PREC_MIXED, _lib.PREC_FP64):
        out[prec], st = kernels.powder_run(
            Hs.shape[0], Hs, Z, B, P, W, slot, len(fields), None, mode=_lib.MODE_INTEGRAL,
            precision=prec, dims=list(sy.dimension), mu_index=sy.muon_index, gammas=sy.gammas,
            tau=constants.MU_TAU)
        assert int(st.max()) == 0
    mixed = out[_lib.PREC_MIXED].cpu().numpy()
    fp64 = out[_lib.PREC_FP64].cpu().numpy()
    ref = np.array([oracle_powder(wl, field=wl.fields[f]) for f in fields])
    print("near-degenerate ALC |mixed - fp64|:", np.abs(mixed - fp64))
    assert np.abs(fp64 - ref).max() <= FP64_TOL
    assert np.abs(mixed - ref).max() <= MIXED_TOL


@pytest.mark.parametrize("n", [65, 96, 128, 192])
def test_eigh_large_random(K, n):
    """n > 64: Householder + QL (FP64) for both precisions."""
    from muspinsim_gb300 import _lib

    rng = np.random.default_rng(300 + n)
    H = np.stack([random_hermitian(rng, n) for _ in range(3)])
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):
        ev, U, st = K.eigh(H, precision=prec)
        ev, U, st = ev.cpu().numpy(), U.cpu().numpy(), st.cpu().numpy()
        assert np.all(st == 0)
        for b in range(H.shape[0]):
            ref = np.linalg.eigvalsh(H[b])
            scale = np.abs(ref).max()
            assert np.abs(ev[b] - ref).max() <= 1e-12 * scale
            rec = (U[b] * ev[b][None, :]) @ U[b].conj().T
            assert np.abs(rec - H[b]).max() <= 1e-12 * scale
            assert np.abs(U[b].conj().T @ U[b] - np.eye(n)).max() <= 1e-12


def test_eigh_large_degenerate(K):
    """Exactly repeated eigenvalues (clusters up to 40 levels)."""
    rng = np.random.default_rng(77)
    n = 96
    lam = np.concatenate([np.full(40, -2.0), np.full(20, 0.5), rng.normal(size=36)])
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    H = Q @ np.diag(lam) @ Q.conj().T
    H = 0.5 * (H + H.conj().T)
    ev, U, st = K.eigh(H[None])
    ev, U = ev[0].cpu().numpy(), U[0].cpu().numpy()
    assert int(st.max()) == 0
    assert np.abs(ev - np.sort(lam)).max() <= 1e-12 * np.abs(lam).max()
    assert np.abs(U.conj().T @ U - np.eye(n)).max() <= 1e-12
    assert np.abs((U * ev) @ U.conj().T - H).max() <= 1e-12 * np.abs(lam).max()


def _large_workload(n_orient=4, n_times=256):
    """mu, e, 3 x 1H, 14N: dim 96, random anisotropic hyperfine, 14N EFG."""
    from muspinsim_gb300 import workloads

    rng = np.random.default_rng(96)
    coup = [("hyperfine", {"i": 1}, workloads.random_hyperfine(rng))]
    for i in (3, 4, 5, 6):
        coup.append(("hyperfine", {"i": i}, workloads.random_hyperfine(rng)))
    V = rng.normal(size=(3, 3))
    V = 0.5 * (V + V.T)
    coup.append(("quadrupolar", {"i": 6}, V - np.trace(V) / 3 * np.eye(3)))
    return workloads.Workload(
        name="mu_e_3H_N_dim96", spins=["mu", "e", "H", "H", "H", "N"], couplings=coup,
        orientations=workloads.zcw_gen(n_orient),
        fields=np.array([[0.0, 0.0, 0.01]]), polarization=np.array([0.0, 0.0, 1.0]),
        times=np.linspace(0, 10, n_times))


def test_powder_fast_large_vs_oracle():
    wl = _large_workload()
    assert int(np.prod(wl.system().dimension)) == 96
    ref = oracle_powder(wl)
    got = _gpu_powder(wl)
    assert np.abs(got - ref).max() <= FP64_TOL
    got = _gpu_powder(wl, "mixed")
    assert np.abs(got - ref).max() <= MIXED_TOL


def _ragged_large_workload(field, n_orient=3, n_times=200, seed=162):
    """mu + 4 x 14N: dim 162 (a row count that is not a multiple of 4),
    muon-nitrogen point dipoles and 14N EFGs.  The total spin is
    half-integer, so at zero field every level is an exact Kramers doublet;
    1e-5 T splits the doublets by ~1e-4 of the spectral width."""
    from muspinsim_gb300 import workloads

    rng = np.random.default_rng(seed)
    coup = []
    for i in range(2, 6):
        coup.append(("dipolar", {"i": 1, "j": i}, workloads.random_vector(rng, 0.3, 0.5)))
        coup.append(("quadrupolar", {"i": i}, workloads.random_efg(rng)))
    return workloads.Workload(
        name="mu_4N_dim162", spins=["mu", "N", "N", "N", "N"], couplings=coup,
        orientations=workloads.zcw_gen(n_orient), fields=np.array([[0.0, 0.0, field]]),
        polarization=np.array([1.0, 0.0, 0.0]), times=np.linspace(0, 10, n_times))


@pytest.mark.parametrize("field", [0.0, 1e-5, 0.01])
def test_powder_fast_large_mixed_degenerate_and_ragged(field):
    """The n > 64 mixed solver (FP32 Householder + QL, double-word
    refinement) on exact and near doublets at n = 162."""
    wl = _ragged_large_workload(field)
    assert int(np.prod(wl.system().dimension)) == 162
    ref = oracle_powder(wl)
    assert np.abs(_gpu_powder(wl) - ref).max() <= FP64_TOL
    assert np.abs(_gpu_powder(wl, "mixed") - ref).max() <= MIXED_TOL


def test_powder_fast_large_mixed_dim192():
    """A 192-dimensional system of the heterogeneous batch (mu, e, 14N and
    protons; hyperfine, dipoles, EFG) in both precisions."""
    from muspinsim_gb300 import workloads

    rng = np.random.default_rng(1004)
    wl = workloads.random_system_workload(rng, 192, workloads.zcw_gen(3),
                                          np.linspace(0.0, 20.0, 300))
    ref = oracle_powder(wl)
    assert np.abs(_gpu_powder(wl) - ref).max() <= FP64_TOL
    assert np.abs(_gpu_powder(wl, "mixed") - ref).max() <= MIXED_TOL


@pytest.mark.parametrize("n_times,t_end", [(4096, 20.0), (1500, 10.0), (9000, 30.0),
                                           (256, 60.0)])
def test_phase_tensor_cores_match_simt_and_oracle(monkeypatch, n_times, t_end):
    """Mixed precision on a uniform grid: the tcgen05 (3xTF32) phase sum
    against the FP32 SIMT kernel (same inputs, FP32-rounding agreement) and
    the oracle (1e-6).  4096 times use 128 x 32 tiles, 1500 one 128 x 16
    tile, 9000 three 128 x 32 tiles; 256 times over 60 us make the phase
    steps psi = omega dt hundreds of radians (the double-word reduction
    modulo 2 pi in the snapshot kernel)."""
    from muspinsim_gb300 import workloads

    wl = workloads.config2(n_orient=40, n_times=n_times)
    wl.times = np.linspace(0.0, t_end, n_times)
    tc = _gpu_powder(wl, "mixed")
    monkeypatch.setenv("MSP_PHASE_SIMT", "1")
    simt = _gpu_powder(wl, "mixed")
    monkeypatch.delenv("MSP_PHASE_SIMT")
    ref = oracle_powder(wl)
    assert np.abs(tc - simt).max() <= 3e-7
    assert np.abs(tc - ref).max() <= MIXED_TOL
    assert np.abs(simt - ref).max() <= MIXED_TOL


@pytest.mark.parametrize("cols,mode", [(2, "zyz"), (3, "zyz"), (3, "zxz"), (4, "zyz"), (4, "zxz")])
def test_orient_snapshots_match_host(K, cols, mode):
    """Device rotation of B and p by the stored conjugate quaternions (and
    the weight normalisation) against the host quaternion code."""
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300.orientations import orientation_rows_to_quats

    rng = np.random.default_rng(9 + cols)
    N = 57
    rows = rng.uniform(0.0, 2.0 * np.pi, (N, cols))
    if cols == 4:
        rows[:, 3] = rng.uniform(0.1, 2.0, N)
    B = np.array([0.1, -0.2, 0.3])
    p = np.array([0.3, 0.4, 0.5])
    p /= np.linalg.norm(p)
    intr = np.array([0.01, 0.0, -0.02])
    F, Pl, W = K.orient_snapshots(rows, B, p, intr, mode)
    qs, ws = orientation_rows_to_quats(rows, mode)
    ws = ws * (N / ws.sum())
    assert np.abs(F.cpu().numpy() - (Q.rotate(qs, B) + intr)).max() <= 1e-15
    assert np.abs(Pl.cpu().numpy() - Q.rotate(qs, p)).max() <= 1e-15
    assert np.abs(W.cpu().numpy() - ws / N).max() <= 1e-15


def test_mixed_degenerate_and_single_crystallites_vs_oracle():
    """Mixed path (FP32 Jacobi + double-word refinement) against the oracle:
    powder average, single crystallites and a degenerate zero-field
    spectrum (isotropic couplings, clusters of equal levels)."""
    from muspinsim_gb300 import workloads

    wl = workloads.config2(n_orient=60, n_times=1024)
    assert np.abs(_gpu_powder(wl, "mixed") - oracle_powder(wl)).max() <= MIXED_TOL
    for o in wl.orientations[:6]:
        ref = oracle_powder(wl, orientations=[o])
        assert np.abs(_gpu_powder(wl, "mixed", orientations=[o]) - ref).max() <= 5e-7
    iso = workloads.Workload(
        name="iso", spins=["mu", "e", "H", "H"],
        couplings=[("hyperfine", {"i": 1}, 400.0 * np.eye(3)),
                   ("hyperfine", {"i": 3}, 50.0 * np.eye(3)),
                   ("hyperfine", {"i": 4}, 50.0 * np.eye(3))],
        orientations=workloads.zcw_gen(8), fields=np.zeros((1, 3)),
        polarization=np.array([0.0, 0.0, 1.0]), times=np.linspace(0.0, 5.0, 512))
    assert np.abs(_gpu_powder(iso, "mixed") - oracle_powder(iso)).max() <= MIXED_TOL
    assert np.abs(_gpu_powder(iso, "fp64") - oracle_powder(iso)).max() <= FP64_TOL


def test_assemble_rotated_vs_host_and_field_rotation(K):
    """msp_assemble_rotated against SpinSystem.rotate on the host, and the
    equivalence with the driver's formulation: rotating every coupling by R
    gives the spectrum of the unrotated system in the field R^T B."""
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300 import workloads

    sy = workloads.config2(n_orient=4, n_times=8).system()
    rng = np.random.default_rng(11)
    qs = Q.from_euler(*rng.uniform(0, 2 * np.pi, (3, 12)), "zyz")
    Rs = Q.rotation_matrix(qs)
    H = K.assemble_rotated(sy, Rs).cpu().numpy()
    Hsys, Z = sy.hamiltonian_matrix(), sy.zeeman_operators()
    B = np.array([0.003, -0.004, 0.01])
    scale = np.abs(Hsys).max()
    for s in range(len(Rs)):
        ref = sy.rotate(Rs[s]).hamiltonian_matrix()
        assert np.abs(H[s] - ref).max() <= 1e-12 * scale
        lam_rot = np.linalg.eigvalsh(H[s] + np.einsum("a,aij->ij", B, Z))
        lam_fld = np.linalg.eigvalsh(Hsys + np.einsum("a,aij->ij", Rs[s].T @ B, Z))
        assert np.abs(lam_rot - lam_fld).max() <= 1e-10 * np.abs(lam_fld).max()


def test_powder_general_path_large():
    """The n > 64 general path (finite temperature, muon not first, decay
    integrals) at n = 96 in both precisions against the oracle."""
    from muspinsim_gb300 import workloads

    wl = _large_workload(n_orient=3, n_times=200)
    ref = oracle_powder(wl, temperature=5.0)
    assert np.abs(_gpu_powder(wl, temperature=5.0) - ref).max() <= FP64_TOL
    assert np.abs(_gpu_powder(wl, "mixed", temperature=5.0) - ref).max() <= MIXED_TOL
    # electron first, muon second: the general path at T = inf
    rng = np.random.default_rng(97)
    coup = [("hyperfine", {"i": 2, "j": 1}, workloads.random_hyperfine(rng))]
    for i in (3, 4, 5):
        coup.append(("dipolar", {"i": 2, "j": i}, workloads.random_vector(rng, 1.0, 2.0)))
    coup.append(("quadrupolar", {"i": 6}, workloads.random_efg(rng)))
    wl2 = workloads.Workload(
        name="e_mu_3H_N_dim96", spins=["e", "mu", "H", "H", "H", "N"], couplings=coup,
        orientations=workloads.zcw_gen(3), fields=np.array([[0.0, 0.0, 0.005]]),
        polarization=np.array([1.0, 0.0, 0.0]), times=np.linspace(0, 5, 150))
    ref2 = oracle_powder(wl2)
    assert np.abs(_gpu_powder(wl2) - ref2).max() <= FP64_TOL
    assert np.abs(_gpu_powder(wl2, "mixed") - ref2).max() <= MIXED_TOL
    # decay integrals over a field scan
    for B in ([0.0, 0.0, 0.02], [0.0, 0.0, 0.3]):
        refi = oracle_powder(wl, field=np.array(B), y_axis="integral")
        got = _gpu_powder(wl, field=np.array(B), y_axis="integral")
        assert abs(got - refi) <= FP64_TOL
        got_m = _gpu_powder(wl, "mixed", field=np.array(B), y_axis="integral")
        assert abs(got_m - refi) <= MIXED_TOL


def test_powder_fast_large_dim512():
    """mu, e and seven protons (n = 512): the large-n kernels well above the
    heterogeneous batch's sizes (32 tridiagonalisation panels and
    reflector blocks, 16 x 32 refinement tiles), both precisions."""
    from muspinsim_gb300 import workloads

    rng = np.random.default_rng(512)
    spins = ["mu", "e"] + ["H"] * 7
    coup = [("hyperfine", {"i": 1}, workloads.random_hyperfine(rng))]
    for i in range(3, 10):
        coup.append(("hyperfine", {"i": i}, workloads.random_hyperfine(rng) * 0.05))
        coup.append(("dipolar", {"i": 1, "j": i}, workloads.random_vector(rng, 1.0, 3.0)))
    wl = workloads.Workload(
        name="mu_e_7H_dim512", spins=spins, couplings=coup, orientations=workloads.zcw_gen(2),
        fields=np.array([[0.0, 0.0, 0.01]]), polarization=np.array([0.0, 0.0, 1.0]),
        times=np.linspace(0.0, 10.0, 60))
    assert int(np.prod(wl.system().dimension)) == 512
    ref = oracle_powder(wl)
    assert np.abs(_gpu_powder(wl) - ref).max() <= FP64_TOL
    assert np.abs(_gpu_powder(wl, "mixed") - ref).max() <= MIXED_TOL


@pytest.mark.parametrize("field", [0.0, 0.02])
def test_powder_fast_large_degenerate_extremes(field):
    """mu, e and five protons (n = 128) with no couplings: at zero field H
    is exactly zero (one 128-fold level: no reflections, zero residual
    anchors); in a field the lab-frame Zeeman H has exactly degenerate
    multiplets up to 10-fold, which the mixed refinement resolves as
    clusters.  Both precisions against the oracle."""
    from muspinsim_gb300 import workloads

    wl = workloads.Workload(
        name="mu_e_5H_free", spins=["mu", "e"] + ["H"] * 5, couplings=[],
        orientations=workloads.zcw_gen(2), fields=np.array([[0.0, 0.0, field]]),
        polarization=np.array([1.0, 0.0, 0.0]), times=np.linspace(0.0, 5.0, 80))
    assert int(np.prod(wl.system().dimension)) == 128
    ref = oracle_powder(wl)
    assert np.abs(_gpu_powder(wl) - ref).max() <= FP64_TOL
    assert np.abs(_gpu_powder(wl, "mixed") - ref).max() <= MIXED_TOL


@pytest.mark.parametrize("spins", [["mu", "e", "H", "H", "H"], ["mu", "e", "H"],
                                   ["mu"] + ["H"] * 5])
def test_powder_mixed_free_spins_degenerate_multiplets(spins):
    """mu, (e) and equivalent protons with no couplings in a field (n = 32,
    8 and 64): the lab-frame Zeeman Hamiltonian has exactly degenerate
    multiplets (3-fold; 10-fold for mu + 5 H), whose eigenvalue gaps are
    rounding noise.  The mixed refinement must treat them as degenerate
    (any orthonormal basis of the multiplet is exact)."""
    from muspinsim_gb300 import workloads

    wl = workloads.Workload(
        name="mu_e_H_free", spins=spins, couplings=[],
        orientations=workloads.zcw_gen(3), fields=np.array([[0.0, 0.0, 0.02]]),
        polarization=np.array([1.0, 0.0, 0.0]), times=np.linspace(0.0, 5.0, 80))
    ref = oracle_powder(wl)
    assert np.abs(_gpu_powder(wl) - ref).max() <= FP64_TOL
    assert np.abs(_gpu_powder(wl, "mixed") - ref).max() <= MIXED_TOL
