"""Host-side logic on the CPU: constants, spin operators, spin systems,
orientation conventions, configuration expansion and the C ABI surface.

Known answers restate the reference's own tests
(muspinsim/tests/test_constants.py, test_spinop.py, test_spinsys.py,
test_config.py:214-285, test_utils.py, test_validation.py)."""

import ctypes
import os
import re

import numpy as np
import pytest
from scipy import sparse

from muspinsim_gb300 import constants
from muspinsim_gb300 import quaternion as Q
from muspinsim_gb300.orientations import (eulrange_gen, orientation_rows_to_quats,
                                          quat_from_polar, zcw_gen)
from muspinsim_gb300.spinop import DensityOperator, Operator, SpinOperator, spin_projectors
from muspinsim_gb300.spinsys import DoubleTerm, InteractionTerm, MuonSpinSystem, SingleTerm, SpinSystem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# ---------------------------------------------------------------- constants
def test_constants_values():
    assert constants.ELEC_GAMMA == pytest.approx(-28024.9514242)
    assert constants.MU_GAMMA == pytest.approx(135.53880943285955)
    assert constants.MU_TAU == pytest.approx(2.19703)
    assert constants.EFG_2_MHZ == pytest.approx(0.23496477815245767)
    assert constants.gyromagnetic_ratio("e") == constants.ELEC_GAMMA
    assert constants.gyromagnetic_ratio("mu") == constants.MU_GAMMA
    assert round(constants.gyromagnetic_ratio("H") - 42.577478518, 3) == 0
    assert constants.quadrupole_moment("e") == 0
    assert constants.quadrupole_moment("H") == 0
    assert round(constants.quadrupole_moment("H", 2) - 2.859, 2) == 0
    assert constants.spin("mu") == 0.5 and constants.spin("e") == 0.5
    assert constants.spin("H") == 0.5 and constants.spin("H", 2) == 1.0
    with pytest.raises(ValueError, match="Invalid isotope 4 for element H"):
        constants.gyromagnetic_ratio("H", 4)
    with pytest.raises(ValueError, match="Invalid isotope 4 for element H"):
        constants.spin("H", 4)
    with pytest.raises(ValueError, match="Invalid multiplicity 0.5 for electron"):
        constants.spin("e", 0.5)


# ---------------------------------------------------------------- operators
def test_spin_half_and_one_matrices():
    sx = SpinOperator.from_axes(0.5, "x").matrix.toarray()
    sy = SpinOperator.from_axes(0.5, "y").matrix.toarray()
    sz = SpinOperator.from_axes(0.5, "z").matrix.toarray()
    assert np.allclose(sx, [[0, 0.5], [0.5, 0]])
    assert np.allclose(sy, [[0, -0.5j], [0.5j, 0]])
    assert np.allclose(sz, [[0.5, 0], [0, -0.5]])
    s1 = [SpinOperator.from_axes(1.0, a).matrix.toarray() for a in "xyz"]
    assert np.allclose(s1[2], np.diag([1, 0, -1]))
    assert np.allclose(s1[0], np.array([[0, 1, 0], [1, 0, 1], [0, 1, 0]]) / 2**0.5)
    # commutation [Sx, Sy] = i Sz
    assert np.allclose(s1[0] @ s1[1] - s1[1] @ s1[0], 1j * s1[2])
    with pytest.raises(ValueError):
        SpinOperator.from_axes(0.3, "x")
    with pytest.raises(ValueError):
        SpinOperator.from_axes(0.5, "w")


def test_operator_algebra_and_errors():
    a = SpinOperator.from_axes([0.5, 0.5], "xz")
    b = SpinOperator.from_axes([0.5, 0.5], "zx")
    assert (a + b).dimension == (2, 2)
    assert np.allclose((a * 2).matrix.toarray(), 2 * a.matrix.toarray())
    assert np.allclose((a * b).matrix.toarray(), a.matrix.toarray() @ b.matrix.toarray())
    assert a.kron(SpinOperator.from_axes(0.5, "y")).dimension == (2, 2, 2)
    assert a.hilbert_schmidt(a) == pytest.approx(0.25)  # tr(Sx^2) tr(Sz^2)
    with pytest.raises(ValueError):
        Operator(np.zeros((2, 3)))
    with pytest.raises(ValueError):
        Operator(np.eye(4), dim=(3,))
    with pytest.raises(ArithmeticError):
        a + SpinOperator.from_axes(0.5, "x")


def test_density_from_vectors():
    rho = DensityOperator.from_vectors(0.5, [1, 0, 0])
    assert np.allclose(rho.matrix.toarray(), [[0.5, 0.5], [0.5, 0.5]])
    rho = DensityOperator.from_vectors(0.5, [0, 0, 1], 0.5)
    assert np.allclose(rho.matrix.toarray(), [[1, 0], [0, 0]])
    rho = DensityOperator.from_vectors(0.5, [1, 0, 0], 1.0)  # fully decohered
    assert np.allclose(rho.matrix.toarray(), [[0.5, 0], [0, 0.5]])
    rho = DensityOperator.from_vectors([0.5, 1.0], [[0, 0, 1], [0, 0, 1]], [0, 0])
    assert np.allclose(np.diag(rho.matrix.toarray()), [1, 0, 0, 0, 0, 0])
    assert rho.expectation(SpinOperator.from_axes([0.5, 1.0], "z0")) == pytest.approx(0.5)
    pt = rho.partial_trace([1])
    assert np.allclose(pt.matrix.toarray(), [[1, 0], [0, 0]])
    with pytest.raises(ValueError):
        DensityOperator(np.zeros((2, 2)))


@pytest.mark.parametrize("I", [0.5, 1.0, 1.5, 2.5])
def test_spin_projectors_are_the_eigenprojectors(I):
    rng = np.random.default_rng(int(10 * I))
    v = rng.normal(size=3)
    proj = spin_projectors(I, v)
    n = v / np.linalg.norm(v)
    mv = np.linspace(I, -I, int(2 * I + 1))
    nS = sum(n[a] * SpinOperator.from_axes(I, ax).matrix.toarray() for a, ax in enumerate("xyz"))
    tot = np.zeros_like(nS)
    for m, P in proj:
        assert np.allclose(nS @ P, m * P, atol=1e-12)
        assert np.allclose(P @ P, P, atol=1e-12)
        tot += P
    assert np.allclose(tot, np.eye(len(mv)))


# ---------------------------------------------------------------- spin systems
def test_terms_and_hamiltonian():
    ssys = SpinSystem(["mu", "e"])
    assert ssys.gamma(0) == constants.MU_GAMMA and ssys.gamma(1) == constants.ELEC_GAMMA
    assert len(ssys) == 2 and ssys.dimension == (2, 2)
    term = SingleTerm(ssys, 0, [0, 0, 1])
    assert np.allclose(term.operator.matrix.toarray(), ssys.operator({0: "z"}).matrix.toarray())
    term = DoubleTerm(ssys, 0, 1, np.diag([1, 1, 2]))
    ref = (ssys.operator({0: "x", 1: "x"}) + ssys.operator({0: "y", 1: "y"})
           + 2 * ssys.operator({0: "z", 1: "z"}))
    assert np.allclose(term.matrix.toarray(), ref.matrix.toarray())
    R = np.array([[1, 0, 0], [0, 0, 1], [0, -1, 0]])
    rot = term.rotate(R)
    ref = (ssys.operator({0: "x", 1: "x"}) + 2 * ssys.operator({0: "y", 1: "y"})
           + ssys.operator({0: "z", 1: "z"}))
    assert np.allclose(rot.matrix.toarray(), ref.matrix.toarray())
    scal = InteractionTerm(ssys, [], 2.0)
    assert np.allclose(scal.matrix.toarray(), 2 * np.eye(4))
    ssys.add_linear_term(0, [1, 0, 1])
    ssys.add_bilinear_term(0, 1, np.eye(3))
    H = ssys.hamiltonian.matrix.toarray()
    assert np.allclose(H, [[0.75, 0, 0.5, 0.0], [0, 0.25, 0.5, 0.5], [0.5, 0.5, -0.75, 0],
                           [0.0, 0.5, 0, -0.25]])
    ssys.clear_terms()
    assert np.allclose(ssys.hamiltonian.matrix.toarray(), 0)
    with pytest.raises(ValueError):
        ssys.add_linear_term(3, [0, 0, 1])


def test_muon_system_terms():
    m = MuonSpinSystem(["e", "mu"])
    assert m.elec_indices == {0} and m.muon_index == 1
    gmu, ge = constants.MU_GAMMA, constants.ELEC_GAMMA
    m.add_zeeman_term(0, 1.0)
    m.add_zeeman_term(1, 1.0)
    h01 = m.add_hyperfine_term(1, np.eye(3) * 100)
    H = m.hamiltonian.matrix.toarray()
    assert np.allclose(np.diag(H), [0.5 * (ge + gmu) + 25, 0.5 * (ge - gmu) - 25,
                                    0.5 * (-ge + gmu) - 25, 0.5 * (-ge - gmu) + 25])
    m.remove_term(h01)
    assert h01.label == "Hyperfine"
    m2 = MuonSpinSystem(["e", "e", "mu"])
    with pytest.raises(ValueError):
        m2.add_hyperfine_term(2, np.eye(3))
    with pytest.raises(ValueError):
        MuonSpinSystem(["e", "H"])
    with pytest.raises(ValueError):
        MuonSpinSystem(["mu", "H"]).add_quadrupolar_term(1, np.eye(3))
    with pytest.raises(ValueError):
        MuonSpinSystem(["mu", "e"]).add_dipolar_term(0, 0, [1, 0, 0])


def test_muon_operators():
    m = MuonSpinSystem(["mu", "e"])
    op = m.muon_operator([1, 1, 1]).matrix.toarray()
    assert np.array_equal(op, [[0.5, 0, 0.5 - 0.5j, 0], [0, 0.5, 0, 0.5 - 0.5j],
                               [0.5 + 0.5j, 0, -0.5, 0], [0, 0.5 + 0.5j, 0, -0.5]])
    sm = m.sigma_mu([1, 1, 1])
    assert sm.shape == (2, 2)
    assert np.array_equal(sm.toarray(), [[1, 1 - 1j], [1 + 1j, -1]])


def test_zeeman_operators_consistent_with_terms():
    m = MuonSpinSystem(["mu", "e", "H"])
    B = np.array([0.01, -0.02, 0.03])
    Z = m.zeeman_operators()
    m2 = MuonSpinSystem(["mu", "e", "H"])
    for i in range(3):
        m2.add_zeeman_term(i, B)
    assert np.allclose(np.einsum("a,aij->ij", B, Z), m2.hamiltonian_matrix())


# ---------------------------------------------------------------- orientations
def test_quaternion_conventions():
    q1 = quat_from_polar(np.pi / 4.0, 0)
    assert np.allclose(q1.rotate([0, 0, 1]), [2 ** (-0.5), 0, 2 ** (-0.5)])
    th, ph = 0.6 * np.pi, 0.4 * np.pi
    q2 = quat_from_polar(th, ph)
    st, ct, cp, sp = np.sin(th), np.cos(th), np.cos(ph), np.sin(ph)
    assert np.allclose(q2.rotate([0, 0, 1]), [st * cp, st * sp, ct])
    assert np.allclose(q2.conjugate().rotate([0, 0, 1]), [-st * cp, st * sp, ct])
    # stored orientation = conj(q_z(c) q_y(b) q_z(a)) (muspinsim/tests/test_config.py:233-285)
    qs, ws = orientation_rows_to_quats([(0.5 * np.pi, 0, 0, 2.0)])
    assert np.allclose(qs[0], [2 ** (-0.5), 0, 0, -(2 ** (-0.5))]) and ws[0] == 2.0
    rng = np.linspace(0, np.pi, 4)
    angles = np.array(np.meshgrid(rng, rng, rng)).reshape((3, -1)).T
    for mode, bax in (("zyz", [0, 1, 0]), ("zxz", [1, 0, 0])):
        qs, _ = orientation_rows_to_quats(angles, mode)
        for (a, b, c), q in zip(angles, qs):
            q2 = Q.Quaternion.from_axis_angle([0, 0, 1], c)
            q2 = q2 * Q.Quaternion.from_axis_angle(bax, b)
            q2 = q2 * Q.Quaternion.from_axis_angle([0, 0, 1], a)
            assert np.allclose(q, q2.conjugate().q)
    R = Q.Quaternion.from_euler_angles(0.3, 0.7, 1.1).rotation_matrix()
    v = np.array([0.2, -0.5, 0.9])
    assert np.allclose(R @ v, Q.Quaternion.from_euler_angles(0.3, 0.7, 1.1).rotate(v))


def test_powder_grids():
    o = zcw_gen(1000)
    assert o.shape == (1000, 2)
    assert abs(np.average(3.0 * np.cos(o[:, 0]) ** 2 - 1.0)) < 1e-5
    ow = eulrange_gen(10)
    A = np.array([[1, 2, 3], [2, 4, 4], [3, 4, -3]])
    Asum = np.zeros((3, 3))
    for a, b, c, w in ow:
        R = Q.Quaternion.from_euler_angles(a, b, c).rotation_matrix()
        Asum += (R @ A @ R.T) * w
    Asum /= np.sum(ow[:, -1])
    assert np.sum(np.abs(Asum - np.eye(3) * np.trace(A) / 3)) < 1.0


# ---------------------------------------------------------------- validation
def test_validation_errors():
    from muspinsim_gb300.validation import (validate_evolve_params,
                                            validate_integrate_decaying_params, validate_times)

    with pytest.raises(TypeError):
        validate_times([0, 1])
    with pytest.raises(ValueError):
        validate_times(np.zeros((2, 2)))
    rho = DensityOperator.from_vectors()
    with pytest.raises(TypeError):
        validate_evolve_params(np.eye(2), np.zeros(2), [])
    with pytest.raises(ValueError):
        validate_evolve_params(rho, np.zeros(2), [np.eye(2)])
    with pytest.raises(ValueError):
        validate_integrate_decaying_params(rho, -1.0, [SpinOperator.from_axes()])
    with pytest.raises(ValueError):
        validate_integrate_decaying_params(rho, 1.0, [])


def test_hamiltonian_rejects_non_hermitian():
    from muspinsim_gb300.hamiltonian import Hamiltonian

    assert Hamiltonian(np.array([[1, 0], [0, -1]])).dimension == (2,)
    with pytest.raises(ValueError):
        Hamiltonian(np.array([[1, 1], [0, 1]]))


# ---------------------------------------------------------------- configuration
def test_config_expansion_and_weights():
    from muspinsim_gb300.simconfig import MuSpinConfig, make_params

    p = make_params(spins=["e", "mu"], orientation=[(0, 0, 0, 1.0), (0.5 * np.pi, 0, 0, 2.0)],
                    field=[(0.0,), (10.0,)], temperature=[np.inf, 0.0],
                    time=np.linspace(0, 10, 100))
    cfg = MuSpinConfig(p)
    assert cfg.results.shape == (2, 2, 100)
    assert len(cfg) == 2 * 2 * 2 and cfg.avg_N == 2
    orange = cfg.avg_ranges["orient"]
    assert sum(w for q, w in orange) == pytest.approx(2.0)
    assert np.allclose(orange[1][0].q, [2 ** (-0.5), 0, 0, -(2 ** (-0.5))])
    snap = cfg[0]
    assert snap.y == "asymmetry" and len(snap.t) == 100


def test_results_function_hook():
    from muspinsim_gb300.simconfig import CallableResults

    r = CallableResults(lambda x, y: 2 * y)
    assert np.allclose(r.evaluate(x=np.arange(3), y=np.ones(3)), 2)


# ---------------------------------------------------------------- C ABI
def test_capi_library_exports_header():
    """libmspgpu.so loads without a GPU and exports every function that
    include/mspgpu.h declares (no compute call is made)."""
    from muspinsim_gb300 import _lib

    with open(os.path.join(ROOT, "include", "mspgpu.h")) as f:
        header = f.read()
    declared = set(re.findall(r"^int\s+(msp_\w+)\s*\(", header, flags=re.M))
    assert {"msp_powder_run", "msp_eigh_batched", "msp_fast_cos_sum"} <= declared
    lib = _lib.load()
    for name in declared:
        assert hasattr(lib, name), name
    assert set(_lib.EXPORTED) >= declared
    assert lib.msp_version() >= 10000
    # argument validation needs no device
    a = _lib.PowderArgs()
    a.n = 2000
    nbytes = ctypes.c_size_t(0)
    assert lib.msp_powder_workspace(ctypes.byref(a), ctypes.byref(nbytes)) == _lib.MSP_ERR_UNSUPPORTED
    assert "exceeds" in _lib.last_error()
    # n > 64 takes every mode: the size passes, the next check (no output
    # rows) fails
    a.n = 200
    a.mode = _lib.MODE_EVOLVE
    assert lib.msp_powder_workspace(ctypes.byref(a), ctypes.byref(nbytes)) == _lib.MSP_ERR_ARG
    assert "num_slots" in _lib.last_error()
    assert ctypes.sizeof(_lib.PowderArgs) > 0


def test_rotation_basis_reproduces_rotated_hamiltonians():
    """The operator basis of the tensor-rotation assembly, contracted with
    rotated tensors on the host, equals the Hamiltonian of
    SpinSystem.rotate (muspinsim/spinsys.py:594-626)."""
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300 import workloads

    sy = workloads.config2(n_orient=4, n_times=8).system()
    sy.add_zeeman_term(2, [0.0, 0.1, 0.2])
    tensors, vectors, B = sy.rotation_basis()
    assert B.shape == (9 * len(tensors) + 3 * len(vectors), 24, 24)
    rng = np.random.default_rng(3)
    for q in Q.from_euler(*rng.uniform(0, 2 * np.pi, (3, 3)), "zyz"):
        R = Q.rotation_matrix(q)
        coef = np.concatenate([np.einsum("ac,tcd,bd->tab", R, tensors, R).reshape(-1),
                               np.einsum("ab,ub->ua", R, vectors).reshape(-1)])
        H = np.einsum("k,kij->ij", coef, B)
        ref = sy.rotate(R).hamiltonian_matrix()
        assert np.abs(H - ref).max() <= 1e-12 * np.abs(ref).max()


def test_capi_large_n_workspace_sizes():
    """Workspace sizing of msp_powder_run for 64 < n through the C ABI (no
    device needed: the occupancy query falls back to one CTA per SM): the
    fast path's FP64 and mixed working sets, and the general path's (two
    more n x n complex matrices per CTA) for EVOLVE and INTEGRAL."""
    from muspinsim_gb300 import _lib

    lib = _lib.load()
    n = 96
    a = _lib.PowderArgs()
    a.n = n
    a.num_spins = 6
    a.mu_index = 0
    for k, d in enumerate((2, 2, 2, 2, 2, 3)):
        a.dims[k] = d
    a.num_snap = 10
    a.num_slots = 1
    a.num_times = 8
    a.uniform = 1
    a.dt = 0.1
    a.tau = 2.19703

    def size(mode, prec):
        a.mode, a.precision = mode, prec
        nbytes = ctypes.c_size_t(0)
        assert lib.msp_powder_workspace(ctypes.byref(a), ctypes.byref(nbytes)) == _lib.MSP_OK, \
            _lib.last_error()
        return nbytes.value

    fast64 = size(_lib.MODE_FAST, _lib.PREC_FP64)
    fastmx = size(_lib.MODE_FAST, _lib.PREC_MIXED)
    evolve = size(_lib.MODE_EVOLVE, _lib.PREC_FP64)
    integ = size(_lib.MODE_INTEGRAL, _lib.PREC_FP64)
    per_fp64 = 5 * n * n * 8  # A, U (complex) and Zt per CTA
    assert fast64 >= 10 * per_fp64
    assert fastmx >= 10 * 56 * n * n  # double-word H and Y, X, X2, SR per CTA
    # the general path adds two complex n x n matrices per CTA
    assert evolve >= fast64 + 10 * 4 * n * n * 8 - 10 * 4096
    assert integ >= 10 * (9 * n * n * 8)
