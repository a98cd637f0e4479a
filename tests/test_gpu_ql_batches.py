"""GPU parity of the batched Householder + QL first stage of the mixed
snapshot pipeline (msp_ql_warp.cu), which launches of 4,096 snapshots or
more take (smaller batches run the warp Jacobi).  Mixed results against the
FP64 pipeline, itself checked against the oracle in test_gpu_kernels.py:
max|dP| <= 1e-6 and every snapshot status 0.  The batches are 4,201
snapshots long, so the last group of four matrices a warp takes is ragged.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6
BATCH = 4201


def _euler_rows(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(0, 2 * np.pi, n), rng.uniform(0, np.pi, n),
                     rng.uniform(0, 2 * np.pi, n)], axis=1)


def _mixed_and_fp64(sy, B, P, W, slot, nslots, times, mode, tau=1.0):
    from muspinsim_gb300 import _lib, kernels

    kernels.device()
    Hs, Z = sy.hamiltonian_matrix(), sy.zeeman_operators()
    out = {}
    for prec in (_lib.PREC_MIXED, _lib.PREC_FP64):
        o, st = kernels.powder_run(Hs.shape[0], Hs, Z, B, P, W, slot, nslots, times, mode=mode,
                                   precision=prec, dims=list(sy.dimension),
                                   mu_index=sy.muon_index, gammas=sy.gammas, tau=tau)
        assert len(st) == len(B) and int(st.max()) == 0
        out[prec] = o.cpu().numpy()
    return out[_lib.PREC_MIXED], out[_lib.PREC_FP64]


def _powder(sy, field, pol, times, seed):
    from muspinsim_gb300 import _lib
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300.orientations import orientation_rows_to_quats

    qs, _ = orientation_rows_to_quats(_euler_rows(BATCH, seed))
    B = Q.rotate(qs, np.asarray(field, dtype=float))
    P = Q.rotate(qs, np.asarray(pol, dtype=float))
    W = np.full(BATCH, 1.0 / BATCH)
    slot = np.zeros(BATCH, dtype=np.int32)
    return _mixed_and_fp64(sy, B, P, W, slot, 1, times, _lib.MODE_FAST)


def _system(spins, couplings):
    from muspinsim_gb300 import workloads

    return workloads.Workload(name="ql_batch", spins=spins, couplings=couplings,
                              orientations=np.zeros((1, 2)), fields=np.zeros((1, 3)),
                              polarization=np.array([0.0, 0.0, 1.0]),
                              times=np.zeros(1)).system()


def _coupled(kind, seed):
    from muspinsim_gb300 import workloads

    rng = np.random.default_rng(seed)
    hf = lambda i: ("hyperfine", {"i": i}, workloads.random_hyperfine(rng))  # noqa: E731
    dip = lambda i, j: ("dipolar", {"i": i, "j": j}, workloads.random_vector(rng, 1.0, 3.0))  # noqa: E731
    quad = lambda i: ("quadrupolar", {"i": i}, workloads.random_efg(rng))  # noqa: E731
    table = {
        2: (["mu"], []),
        4: (["mu", "e"], [hf(1)]),
        6: (["mu", "N"], [dip(1, 2), quad(2)]),
        8: (["mu", "e", "H"], [hf(1), hf(3), dip(1, 3)]),
        12: (["mu", "e", "N"], [hf(1), hf(3), quad(3)]),
        18: (["mu", "N", "N"], [dip(1, 2), dip(1, 3), quad(2), quad(3)]),
    }
    if kind == 24:
        return workloads.config2(n_orient=1, n_times=1).system()
    if kind == 32:
        return workloads.config3(n_fields=1, n_orient=1).system()
    spins, coup = table[kind]
    return _system(spins, coup)


@pytest.mark.parametrize("n", [2, 4, 6, 8, 12, 18, 24, 32])
def test_ql_batch_coupled_systems(n):
    sy = _coupled(n, 100 + n)
    assert int(np.prod(sy.dimension)) == n
    times = np.linspace(0.0, 10.0, 64)
    mixed, fp64 = _powder(sy, [0.0, 0.0, 0.01], [0.0, 0.0, 1.0], times, seed=n)
    err = np.abs(mixed - fp64).max()
    print(f"n = {n}: QL batch max|dP| mixed vs FP64 = {err:.2e}")
    assert err <= MIXED_TOL


@pytest.mark.parametrize("spins", [["mu", "e", "H"], ["mu", "e", "H", "H", "H"]])
@pytest.mark.parametrize("field", [0.0, 0.02])
def test_ql_batch_exact_degeneracies(spins, field):
    """Uncoupled spins: the Hamiltonian is a sum of single-spin Zeeman terms
    (zero at zero field), so its levels come in exact multiplets and the
    tridiagonal form splits into decoupled blocks."""
    sy = _system(spins, [])
    times = np.linspace(0.0, 5.0, 80)
    mixed, fp64 = _powder(sy, [0.0, 0.0, field], [1.0, 0.0, 0.0], times, seed=7)
    assert np.abs(mixed - fp64).max() <= MIXED_TOL


# (field index, orientation) snapshots of a dense ALC scan (dim 32, fields
# linspace(0, 1, 500) T along z, 24 ZCW-style orientations) with level pairs
# within a few FP32 resolutions of |H|
NEAR_DEGENERATE = [(352, 21), (447, 20), (199, 12), (107, 17)]


def test_ql_batch_alc_near_degenerate():
    """The near-degenerate ALC snapshots, each repeated into a slot of its
    own, integral mode: every slot is one snapshot's integral."""
    from muspinsim_gb300 import _lib, constants, workloads
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300.orientations import orientation_rows_to_quats

    wl = workloads.config3(n_fields=500, n_orient=24)
    sy = wl.system()
    qs, _ = orientation_rows_to_quats(wl.orientations)
    reps = -(-BATCH // len(NEAR_DEGENERATE))
    B = np.concatenate([np.repeat(Q.rotate(qs[o:o + 1], wl.fields[f]), reps, axis=0)
                        for f, o in NEAR_DEGENERATE])
    P = np.concatenate([np.repeat(Q.rotate(qs[o:o + 1], wl.polarization), reps, axis=0)
                        for _, o in NEAR_DEGENERATE])
    W = np.full(len(B), 1.0 / reps)
    slot = np.repeat(np.arange(len(NEAR_DEGENERATE), dtype=np.int32), reps)
    mixed, fp64 = _mixed_and_fp64(sy, B, P, W, slot, len(NEAR_DEGENERATE), None,
                                  _lib.MODE_INTEGRAL, tau=constants.MU_TAU)
    print("near-degenerate ALC slots |mixed - fp64|:", np.abs(mixed - fp64))
    assert np.abs(mixed - fp64).max() <= MIXED_TOL
