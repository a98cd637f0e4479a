"""CPU oracle for the polarisation path -- TEST INFRASTRUCTURE ONLY.

A plain numpy restatement of the reference's algorithm, used by ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg as the checker.
Nothing in ``muspinsim_gb300`` imports it; the product path runs on the GPU
and fails loudly without its CUDA library.

Every function cites the reference lines it restates.  The oracle is pinned
against golden vectors produced by running the reference itself
(``tests/golden/make_golden.py``) and against the analytic known-answer tests
of the reference suite (``muspinsim/tests/test_hamiltonian.py``,
``test_experiment.py``, ``test_spinsys.py``).  Matrices are dense complex128;
the reference keeps them in scipy CSR, which changes storage, not values.
"""

import ctypes
import os

import numpy as np
import scipy.constants as cnst

HERE = os.path.dirname(os.path.abspath(__file__))

ELEC_GAMMA = -28024.9514242  # muspinsim/constants.py:12
MU_GAMMA = -(ELEC_GAMMA / 206.7669883)  # muspinsim/constants.py:13
MU_TAU = 2.19703  # muspinsim/constants.py:14
EFG_2_MHZ = (  # muspinsim/constants.py:20-25
    cnst.physical_constants["atomic unit of electric field gradient"][0] * cnst.e * 1e-37 / cnst.h
)


# ---------------------------------------------------------------- spin matrices
def mvals(I):
    """m = +I ... -I (muspinsim/spinop.py:14-15)."""
    return np.linspace(I, -I, int(2 * I + 1))


def spin_matrix(I, axis):
    """Single-spin operator for axis in 'xyz+-0' (muspinsim/spinop.py:18-41)."""
    m = mvals(I)
    sp = 2 * np.diag(0.5 * (np.cumsum(2 * m)[:-1] ** 0.5), k=1) + 0.0j
    if axis == "+":
        return sp
    if axis == "-":
        return sp.T
    if axis == "x":
        return 0.5 * (sp + sp.T)
    if axis == "y":
        return 0.5j * (sp.T - sp)
    if axis == "z":
        return np.diag(m) + 0.0j
    if axis == "0":
        return np.eye(len(m)) + 0.0j
    raise ValueError(axis)


def embed(Is, ops):
    """Kronecker embedding of per-spin operators, identity elsewhere; spin 0
    is the slowest index (muspinsim/spinsys.py:545-592).  ``ops`` maps a spin
    index to an axis letter or a list of letters (multiplied in order)."""
    M = None
    for i, I in enumerate(Is):
        o = ops.get(i, "0")
        if isinstance(o, (list, tuple)):
            m = spin_matrix(I, o[0])
            for a in o[1:]:
                m = m @ spin_matrix(I, a)
        else:
            m = spin_matrix(I, o)
        M = m if M is None else np.kron(M, m)
    return M


# ---------------------------------------------------------------- spin systems
class System:
    """Spins plus interaction terms (muspinsim/spinsys.py:161-216, 640-705).

    ``terms`` holds ``(indices, tensor)`` with tensors already in MHz, as the
    reference's ``InteractionTerm`` stores them."""

    def __init__(self, spins, gammas, Is, Qs):
        self.spins = list(spins)
        self.gammas = np.array(gammas, dtype=float)
        self.Is = np.array(Is, dtype=float)
        self.Qs = np.array(Qs, dtype=float)
        self.dims = tuple(int(2 * I + 1) for I in self.Is)
        self.terms = []
        self.mu_i = self.spins.index("mu") if "mu" in self.spins else None

    @property
    def n(self):
        return int(np.prod(self.dims))

    def add_term(self, indices, tensor):
        self.terms.append((tuple(indices), np.array(tensor, dtype=float)))

    def add_zeeman(self, i, B):
        """(muspinsim/spinsys.py:354-375)"""
        if np.isscalar(B):
            B = [0, 0, B]
        self.add_term([i], np.array(B, dtype=float) * self.gammas[i])

    def add_hyperfine(self, i, A, j):
        """(muspinsim/spinsys.py:664-705); j is the electron index."""
        self.add_term([i, j], A)

    def add_dipolar(self, i, j, r):
        """(muspinsim/spinsys.py:377-413), r in Angstrom."""
        r = np.array(r, dtype=float)
        rnorm = np.linalg.norm(r)
        D = -(np.eye(3) - 3.0 / rnorm**2.0 * r[:, None] * r[None, :])
        dij = -(cnst.mu_0 * cnst.hbar * (self.gammas[i] * self.gammas[j] * 1e6)) / (
            2 * (rnorm * 1e-10) ** 3
        )
        self.add_term([i, j], D * dij)

    def add_quadrupolar(self, i, EFG):
        """(muspinsim/spinsys.py:415-442)"""
        I = self.Is[i]
        Qtens = EFG_2_MHZ * self.Qs[i] / (2 * I * (2 * I - 1)) * np.array(EFG, dtype=float)
        self.add_term([i, i], Qtens)

    def term_matrix(self, indices, tensor):
        """sum over tensor index tuples of T_ab S^a_i S^b_j; a same-spin pair
        uses the matrix product S^a_i S^b_i (muspinsim/spinsys.py:34-69)."""
        n = self.n
        total = np.zeros((n, n), dtype=complex)
        if len(indices) == 0:
            return total + tensor * np.eye(n)
        for ii in np.ndindex(*tensor.shape):
            if len(indices) == 2 and indices[0] == indices[1]:
                ops = {indices[0]: ["xyz"[ii[0]], "xyz"[ii[1]]]}
            else:
                ops = {ind: "xyz"[ii[k]] for k, ind in enumerate(indices)}
            total += embed(self.Is, ops) * tensor[ii]
        return total

    def hamiltonian(self):
        """Hsys = sum of the term matrices (muspinsim/spinsys.py:613-626)."""
        H = np.zeros((self.n, self.n), dtype=complex)
        for ind, T in self.terms:
            H += self.term_matrix(ind, T)
        return H

    def zeeman_operators(self):
        """Z_a = sum_i gamma_i S^a_i, so that Hz(B) = sum_a B_a Z_a
        (muspinsim/experiment.py:105-111, 239-250)."""
        Z = np.zeros((3, self.n, self.n), dtype=complex)
        for i, g in enumerate(self.gammas):
            for a, ax in enumerate("xyz"):
                Z[a] += g * embed(self.Is, {i: ax})
        return Z

    def muon_operator(self, v):
        """O = sum_a v_a S^a_mu (muspinsim/spinsys.py:707-732)."""
        return sum(v[a] * embed(self.Is, {self.mu_i: ax}) for a, ax in enumerate("xyz"))


def sigma_mu(v):
    """sum_a v_a sigma_a, 2x2 Pauli combination (muspinsim/spinsys.py:734-760)."""
    sx = np.array([[0, 1], [1, 0]], dtype=complex)
    sy = np.array([[0, -1j], [1j, 0]], dtype=complex)
    sz = np.array([[1, 0], [0, -1]], dtype=complex)
    return v[0] * sx + v[1] * sy + v[2] * sz


# ---------------------------------------------------------------- orientations
def quat_mul(a, b):
    w1, x1, y1, z1 = a
    w2, x2, y2, z2 = b
    return np.array(
        [
            w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2,
            w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
            w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2,
            w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2,
        ]
    )


def quat_axis(axis, angle):
    axis = np.asarray(axis, dtype=float)
    return np.concatenate([[np.cos(angle / 2)], np.sin(angle / 2) * axis])


def orientation_quat(row, mode="zyz"):
    """Stored (conjugated) orientation quaternion and weight for an input row:
    (theta, phi) polar, (a, b, c) or (a, b, c, w) Euler
    (muspinsim/simconfig.py:596-613; muspinsim/utils.py:53-68; Euler
    composition q_c q_b q_a pinned by muspinsim/tests/test_config.py:233-285)."""
    row = list(row)
    w = 1.0
    if len(row) == 2:
        theta, phi = row
        a, b, c, mode = phi, theta, phi, "zyz"
    else:
        a, b, c = row[:3]
        if len(row) == 4:
            w = row[3]
    bax = [0, 1, 0] if mode == "zyz" else [1, 0, 0]
    q = quat_mul(quat_mul(quat_axis([0, 0, 1], c), quat_axis(bax, b)), quat_axis([0, 0, 1], a))
    return q * np.array([1.0, -1, -1, -1]), w


def quat_rotate(q, v):
    """q v q* (muspinsim/experiment.py:405-406)."""
    qv = np.concatenate([[0.0], np.asarray(v, dtype=float)])
    return quat_mul(quat_mul(q, qv), q * np.array([1.0, -1, -1, -1]))[1:]


# ---------------------------------------------------------------- states
def density_from_vector(I, vec):
    """Pure state along vec (muspinsim/spinop.py:455-530, gamma = 0)."""
    S = [spin_matrix(I, a) for a in "xyz"]
    o = sum(S[i] * vec[i] for i in range(3))
    evals, evecs = np.linalg.eigh(o)
    psi = evecs[:, np.argmax(evals)]
    m = psi[:, None] * psi[None, :].conj()
    return m / np.trace(m)


def rho0(system, B, p, T):
    """Initial state: muon along p, other spins thermal in their own Zeeman
    field, uniform at T = inf (muspinsim/experiment.py:170-236)."""
    rhos = []
    for i, I in enumerate(system.Is):
        if i == system.mu_i:
            r = density_from_vector(I, p)
        else:
            Hz = sum(B[j] * spin_matrix(I, e) for j, e in enumerate("xyz"))
            evals, evecs = np.linalg.eigh(Hz)
            E = evals * 1e6 * system.gammas[i]
            if T > 0:
                Z = np.exp(-cnst.h * E / (cnst.k * T))
            else:
                Z = np.where(E == np.amin(E), 1.0, 0.0)
            if np.sum(Z) > 0:
                Z /= np.sum(Z)
            else:
                Z = np.ones(len(E)) / len(E)
            r = np.sum(evecs[:, None, :] * evecs[None, :, :].conj() * Z[None, None, :], axis=-1)
            r = r / np.trace(r)
        rhos.append(r)
    M = rhos[0]
    for r in rhos[1:]:
        M = np.kron(M, r)
    return M


# ---------------------------------------------------------------- propagation
def evolve(H, rho, times, operators):
    """<O>(t) = sum_ij rho'_ij O'_ji exp(-2 pi i (l_i - l_j) t) in the
    eigenbasis; complex [T, n_ops] (muspinsim/hamiltonian.py:40-117)."""
    evals, evecs = np.linalg.eigh(H)
    U = evecs
    rp = U.conj().T @ rho @ U
    ll = -2.0j * np.pi * (evals[:, None] - evals[None, :])
    times = np.asarray(times, dtype=float)
    out = np.empty((len(times), len(operators)), dtype=complex)
    for k, O in enumerate(operators):
        Op = U.conj().T @ O @ U
        c = (rp * Op.T).reshape(-1)
        ph = np.exp(ll.reshape(-1)[None, :] * times[:, None])
        out[:, k] = ph @ c
    return out


def evolve_per_time(H, rho, times, operators):
    """The same <O>(t) computed the way the reference's Hamiltonian.evolve
    does it, for CPU-baseline timing (muspinsim/hamiltonian.py:76-107): per
    time, the n x n phase matrix exp(ll t) times rho', an elementwise
    product-sum with each O'^T, and the row appended to the result with
    np.concatenate (quadratic in the number of times, as there)."""
    evals, evecs = np.linalg.eigh(H)
    U = evecs
    rp = U.conj().T @ rho @ U
    opsT = np.array([(U.conj().T @ O @ U).T for O in operators])
    ll = -2.0j * np.pi * (evals[:, None] - evals[None, :])
    times = np.asarray(times, dtype=float)
    result = None
    for i in range(times.shape[0]):
        r = np.exp(ll[None, :, :] * times[i, None, None]) * rp[None, :, :]
        single = np.sum(r[0, None, :, :] * opsT[None, :, :, :], axis=(2, 3))
        result = single if result is None else np.concatenate(([result, single]), axis=0)
    return result


def integrate_decaying(H, rho, tau, operators):
    """int_0^inf <O>(t) exp(-t/tau) dt = sum_ij rho'_ij [-O'/(2 pi i (l_i -
    l_j) - 1/tau)]^T_ij (muspinsim/hamiltonian.py:119-164)."""
    evals, evecs = np.linalg.eigh(H)
    U = evecs
    rp = U.conj().T @ rho @ U
    ll = 2.0j * np.pi * (evals[:, None] - evals[None, :])
    res = []
    for O in operators:
        Op = U.conj().T @ O @ U
        intop = (-Op / (ll - 1.0 / tau)).T
        res.append(np.sum(rp * intop))
    return np.array(res)


# ---------------------------------------------------------------- Lindblad
def lindblad_matrix(H, dissipators=()):
    """L = -i (H (x) 1 - 1 (x) H^T) + sum_k g_k [A_k (x) conj(A_k)
    - 1/2 (A_k^H A_k (x) 1 + 1 (x) (A_k^H A_k)^T)], row-major vec
    (muspinsim/lindbladian.py:17-41; superoperators muspinsim/spinop.py:
    622-714)."""
    n = H.shape[0]
    one = np.eye(n)
    L = -1.0j * (np.kron(H, one) - np.kron(one, H.T))
    for A, g in dissipators:
        M = A.conj().T @ A
        L = L + g * (np.kron(A, A.conj()) - 0.5 * (np.kron(M, one) + np.kron(one, M.T)))
    return L


def lindblad_evolve(L, rho, times, operators):
    """<O>(t) from the eigendecomposition of L: complex [T, n_ops]
    (muspinsim/lindbladian.py:43-111)."""
    evals, revecs = np.linalg.eig(L)
    r0 = np.linalg.solve(revecs, rho.reshape(-1))
    opsT = np.array([O.T.reshape(-1) @ revecs for O in operators])
    times = np.asarray(times, dtype=float)
    r = np.exp(2.0 * np.pi * evals[None, :] * times[:, None]) * r0[None, :]
    return np.sum(opsT[None, :, :] * r[:, None, :], axis=-1)


def lindblad_states(L, rho, times):
    """Density matrices of lindblad_evolve without operators
    (muspinsim/lindbladian.py:104-109)."""
    n = rho.shape[0]
    evals, revecs = np.linalg.eig(L)
    r0 = np.linalg.solve(revecs, rho.reshape(-1))
    times = np.asarray(times, dtype=float)
    r = np.exp(2.0 * np.pi * evals[None, :] * times[:, None]) * r0[None, :]
    return np.array([(revecs @ x).reshape(n, n) for x in r])


def lindblad_integrate(L, rho, tau, operators):
    """int_0^inf <O>(t) exp(-t/tau) dt (muspinsim/lindbladian.py:113-173)."""
    evals, revecs = np.linalg.eig(L)
    r0 = np.linalg.solve(revecs, rho.reshape(-1))
    intops = np.array([(O.T.reshape(-1) @ revecs) / (1.0 / tau - 2.0 * np.pi * evals)
                       for O in operators])
    return np.sum(r0[None, :] * intops, axis=1)


def get_xy(z):
    """Two axes orthogonal to z (muspinsim/utils.py:71-93)."""
    z = np.asarray(z, dtype=float)
    z = z / np.linalg.norm(z)
    if z[0] == 0 and z[1] == 0:
        return np.array([1.0, 0, 0]), np.array([0, z[2], 0])
    x = np.array([z[1], -z[0], 0.0]) / (z[0] ** 2 + z[1] ** 2) ** 0.5
    y = np.array([z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2],
                  z[0] * x[1] - z[1] * x[0]])
    return x, y


def dissipation_operators(system, B, T, dterms):
    """(A, rate) pairs of the driver: per dissipative spin i with rate a,
    S_+ and S_- about the field direction with rates a Zu / (pi (1 + Zu))
    and a / (pi (1 + Zu)), Zu = exp(-h gamma_i |B| 1e6 / (k T))
    (muspinsim/experiment.py:272-325)."""
    Bn = np.linalg.norm(B)
    g = system.gammas
    if T > 0:
        Zu = np.exp(-cnst.h * g * Bn * 1e6 / (cnst.k * T))
    else:
        Zu = g * 0.0
    if Bn == 0:
        x, y = np.array([1.0, 0, 0]), np.array([0, 1.0, 0])
    else:
        x, y = get_xy(np.asarray(B, dtype=float) / Bn)
    ops = []
    for i, a in dterms.items():
        S = [embed(system.Is, {i: ax}) for ax in "xyz"]
        ox = sum(S[k] * x[k] for k in range(3))
        oy = sum(S[k] * y[k] for k in range(3))
        ops.append((ox + 1.0j * oy, 1 / np.pi * a * Zu[i] / (1 + Zu[i])))
        ops.append((ox - 1.0j * oy, 1 / np.pi * a / (1 + Zu[i])))
    return ops


_LIB = None


def _oracle_lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            import importlib.util

            spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            path = mod.build_port()
        lib = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        lib.oracle_fast_cos_sum.argtypes = [dp, ctypes.c_long, ctypes.c_long, dp, dp,
                                            ctypes.c_long, dp, ctypes.c_int]
        lib.oracle_fast_cos_powder.argtypes = [dp, ctypes.c_long, ctypes.c_long, dp, dp,
                                               ctypes.c_long, ctypes.c_long, dp, dp, ctypes.c_int]
        _LIB = lib
    return _LIB


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def fast_cos_sum(times, d, A, W, nthreads=0):
    """The reference's cosine phase sum (muspinsim/cython/parallel.pyx:16-69),
    through the C restatement in oracle/fast_cos_sum.c."""
    times = np.ascontiguousarray(times, dtype=np.float64)
    A = np.ascontiguousarray(A, dtype=np.float64)
    W = np.ascontiguousarray(W, dtype=np.float64)
    out = np.zeros(len(times))
    _oracle_lib().oracle_fast_cos_sum(_dp(times), len(times), int(d), _dp(A), _dp(W),
                                      A.shape[0], _dp(out), int(nthreads))
    return out


def fast_amplitudes(H, sig, d):
    """A = |U^dag (sigma (x) 1_d) U|^2 and W = 2 pi (l_j - l_k)
    (muspinsim/hamiltonian.py:196-211)."""
    evals, U = np.linalg.eigh(H)
    S = np.kron(sig, np.eye(d))
    A = np.abs(U.conj().T @ S @ U) ** 2
    W = 2 * np.pi * np.subtract.outer(evals, evals)
    return A, W, evals


def fast_evolve(H, sig, times, d, nthreads=0):
    """Muon-first, T = inf shortcut, x 0.5 (muspinsim/hamiltonian.py:166-217)."""
    A, W, _ = fast_amplitudes(H, sig, d)
    return fast_cos_sum(times, d, A, W, nthreads) * 0.5


# ---------------------------------------------------------------- driver
def t_inf_speedup(B, T, mu_i):
    """Fast-path selection rule (muspinsim/experiment.py:413-430)."""
    Bn = np.linalg.norm(B)
    check = (cnst.e * (cnst.hbar**2) * Bn) / (2 * cnst.m_p * cnst.k * T)
    return bool(check == 0) and mu_i == 0


def snapshot(system, Hsys, Z, q, w, B, p, T, intrinsic_B, times, y="asymmetry", nthreads=0,
             dissipation=None, celio=(0, 0), phases=None):
    """One configuration: rotate B and p by q, add the intrinsic field, pick
    the path, return real(data) * w (muspinsim/experiment.py:384-498).
    ``dissipation``: {spin index: rate}; when given, the Lindbladian path
    (muspinsim/experiment.py:332-341).  ``celio``: (k, averages) of Celio's
    method, with ``phases`` [averages, d] for its random initial states
    (muspinsim/experiment.py:451-471)."""
    Bl = quat_rotate(q, B) + np.asarray(intrinsic_B, dtype=float)
    pl = quat_rotate(q, p)
    if celio[0]:
        if y == "integral":
            raise NotImplementedError("integrate_decaying is not implemented for Celio's method")
        k, avg = celio
        times = np.asarray(times, dtype=float)
        factors = celio_snapshot_factors(system, Bl, times[1] - times[0], k)
        if avg:
            if T != np.inf:
                raise ValueError("The fast version of Celio's method requires T -> inf.")
            if system.mu_i != 0:
                raise ValueError("Muon must be the first spin in the system")
            data = celio_fast_evolve(factors, list(system.dims), sigma_mu(pl), times, k, phases)
        else:
            data = celio_evolve(factors, list(system.dims), rho0(system, Bl, pl, T), times,
                                [system.muon_operator(pl)], k)[:, 0]
        return np.real(data) * w
    H = Hsys + np.einsum("a,aij->ij", Bl, Z)
    if dissipation:
        L = lindblad_matrix(H, dissipation_operators(system, Bl, T, dissipation))
        rho = rho0(system, Bl, pl, T)
        O = system.muon_operator(pl)
        if y == "integral":
            data = lindblad_integrate(L, rho, MU_TAU, [O])[0] / MU_TAU
        else:
            data = lindblad_evolve(L, rho, times, [O])[:, 0]
        return np.real(data) * w
    if y == "integral":
        rho = rho0(system, Bl, pl, T)
        O = system.muon_operator(pl)
        data = integrate_decaying(H, rho, MU_TAU, [O])[0] / MU_TAU
    elif t_inf_speedup(Bl, T, system.mu_i):
        d = system.n // system.dims[system.mu_i]
        data = fast_evolve(H, sigma_mu(pl), times, d, nthreads)
    else:
        rho = rho0(system, Bl, pl, T)
        O = system.muon_operator(pl)
        data = evolve(H, rho, times, [O])[:, 0]
    return np.real(data) * w


def powder_average(system, orientations, B, p, T, times, intrinsic_B=(0, 0, 0),
                   y="asymmetry", nthreads=0, dissipation=None, celio=(0, 0), phases=None):
    """Orientation average: weights normalised to sum to N, result = sum_k
    w_k P_k / N (muspinsim/simconfig.py:152-159, 347-368).  ``phases``:
    [orientations, averages, d] for Celio's method with averages."""
    Hsys = system.hamiltonian()
    Z = system.zeeman_operators()
    qs = [orientation_quat(o) for o in orientations]
    N = len(qs)
    if N > 1:
        norm = N / np.sum([w for _, w in qs])
        qs = [(q, w * norm) for q, w in qs]
    else:
        qs = [(q, 1.0) for q, _ in qs]
    acc = None
    for s_i, (q, w) in enumerate(qs):
        r = snapshot(system, Hsys, Z, q, w, B, p, T, intrinsic_B, times, y, nthreads,
                     dissipation, celio, None if phases is None else phases[s_i])
        acc = r / N if acc is None else acc + r / N
    return acc


# ---------------------------------------------------------------- gradient checker
def fast_snapshot_grad(H, sig, d, times, g, w):
    """dL/dH of L = sum_t g(t) * w * fast_evolve(H, sig, times, d)(t).

    The reference has no gradient (its fits difference the simulation
    numerically, muspinsim/fitting.py:67-179); this restates the derivative
    of the fast-path formula (muspinsim/hamiltonian.py:166-217) written as
    P(t) = kappa Tr(S V S V^H), V = exp(2 pi i H t), kappa = w / (4 d), via
    the Frechet derivative of the exponential in the eigenbasis (divided
    differences of exp(2 pi i l t); their derivative for equal levels).  It
    is the checker of the CUDA adjoint and is itself pinned against central
    finite differences of fast_evolve in the CPU tests.  Returns G with
    dL = Re sum conj(G) dH."""
    n = H.shape[0]
    lam, U = np.linalg.eigh(H)
    S = np.kron(sig, np.eye(d))
    M = U.conj().T @ S @ U
    t = np.asarray(times, dtype=float)
    nu = np.subtract.outer(lam, lam).T                      # nu[a, b] = l_b - l_a
    E = np.exp(2j * np.pi * nu[:, :, None] * t[None, None, :])
    Gh = E @ g
    Gd = (E * (2j * np.pi * t)[None, None, :]) @ g
    tmax = np.abs(t).max()
    gap = np.subtract.outer(lam, lam)                       # gap[b, c] = l_b - l_c
    dd = np.abs(2 * np.pi * tmax * gap) > 1e-5
    inv = np.where(dd, 1.0 / np.where(dd, gap, 1.0), 0.0)
    # D[a, b, c]
    D = np.where(dd[None], (Gh[:, :, None] - Gh[:, None, :]) * inv[None],
                 0.5 * (Gd[:, :, None] + Gd[:, None, :]))
    K = np.einsum("ca,ab,abc->bc", M, M, D)
    kappa = w / (4.0 * d)
    Gp = kappa * (np.conj(K) + K.T)
    return U @ Gp @ U.conj().T


def fast_powder_grad(system, orientations, B, p, times, g):
    """dL/dHsys and dL/dB_lab (per orientation) of L = sum_t g(t) P(t) for
    the fast-path powder_average (muon first, T = inf)."""
    Hsys = system.hamiltonian()
    Z = system.zeeman_operators()
    qs = [orientation_quat(o) for o in orientations]
    N = len(qs)
    if N > 1:
        norm = N / np.sum([w for _, w in qs])
        qs = [(q, w * norm) for q, w in qs]
    else:
        qs = [(q, 1.0) for q, _ in qs]
    d = system.n // system.dims[system.mu_i]
    GH = np.zeros_like(Hsys)
    GB = []
    for q, w in qs:
        Bl = quat_rotate(q, B)
        pl = quat_rotate(q, p)
        H = Hsys + np.einsum("a,aij->ij", Bl, Z)
        G = fast_snapshot_grad(H, sigma_mu(pl), d, times, g, w / N)
        GH += G
        GB.append([np.real(np.sum(np.conj(G) * Z[a])) for a in range(3)])
    return GH, np.array(GB)


# ---------------------------------------------------------------- Celio's method
def celio_term_matrix(system, indices, tensor):
    """A term's operator over its own spins only, in ascending spin order
    (``include_only_given``: muspinsim/spinsys.py:34-69, 545-592).  A
    same-spin pair (quadrupole) multiplies S^a_i S^b_i."""
    involved = sorted(set(int(i) for i in indices))
    loc = {s: k for k, s in enumerate(involved)}
    Is = [system.Is[s] for s in involved]
    total = None
    for ii in np.ndindex(*tensor.shape):
        if len(indices) == 2 and indices[0] == indices[1]:
            ops = {loc[indices[0]]: ["xyz"[ii[0]], "xyz"[ii[1]]]}
        else:
            ops = {loc[int(ind)]: "xyz"[ii[k]] for k, ind in enumerate(indices)}
        m = embed(Is, ops) * tensor[ii]
        total = m if total is None else total + m
    return total


def celio_terms(system, B=None):
    """(indices, small matrix) for every term of the system, followed by the
    field's Zeeman terms gamma_i B.S_i when B is not zero
    (muspinsim/experiment.py:239-269: appended after the system's terms)."""
    out = [(tuple(int(i) for i in ind), celio_term_matrix(system, ind, T))
           for ind, T in system.terms]
    if B is not None and not np.array_equal(np.asarray(B, dtype=float), [0, 0, 0]):
        for i in range(len(system.spins)):
            v = np.asarray(B, dtype=float) * system.gammas[i]
            out.append(((i,), celio_term_matrix(system, (i,), v)))
    return out


def celio_contribs(dims, terms):
    """Hamiltonian contributions H_c (muspinsim/celio.py:73-143): per spin i
    in order, the terms whose first index is i, split into runs of equal
    index tuples (itertools.groupby, so only consecutive terms merge), each
    run summed.  Returns (matrix, other_dim, spin_order, spin_dims) with
    spin_order = the run's indices (a repeated index once) followed by the
    uninvolved spins in ascending order."""
    import itertools

    L = len(dims)
    out = []
    for i in range(L):
        spin_ints = [t for t in terms if t[0][0] == i]
        other = [s for s in range(L) if s != i]
        for ind, grp in itertools.groupby(spin_ints, key=lambda t: t[0]):
            grp = list(grp)
            H = sum(m for _, m in grp)
            unin = list(other)
            for t in grp:
                for j in t[0]:
                    if j in unin:
                        unin.remove(j)
            other_dim = int(np.prod([dims[j] for j in unin])) if unin else 1
            ind = list(ind)
            if len(ind) == 2 and ind[0] == ind[1]:
                ind.pop()
            order = ind + unin
            out.append((H, other_dim, order, [dims[s] for s in order]))
    return out


def celio_factors(contribs, dt, k):
    """U_c = expm(-2 pi i H_c dt / k) (muspinsim/celio.py:145-208)."""
    from scipy.linalg import expm

    return [(expm(-2j * np.pi * H * dt / k), od, order, sd) for H, od, order, sd in contribs]


def celio_index_map(dims, order):
    """Flat index, in the system's ordering, of each element of the
    permuted ordering (muspinsim/celio.py:171-177)."""
    N = int(np.prod(dims))
    return np.transpose(np.arange(N).reshape(dims), axes=order).flatten()


def celio_apply(psi, U, idx):
    """(U (x) 1_d) acting through the index map, in place
    (muspinsim/cpp/parallel.cpp:236-262)."""
    D = U.shape[0]
    ix = idx.reshape(D, -1)
    psi[ix] = U @ psi[ix]


def celio_measure_h(psi, M, d):
    """Re <psi|(M (x) 1_d)|psi> for Hermitian M, using the upper triangle
    twice (muspinsim/cpp/parallel.cpp:126-160)."""
    D = M.shape[0]
    V = psi.reshape(D, d)
    total = 0.0
    for i in range(D):
        term = M[i, i] * V[i]
        for j in range(i + 1, D):
            term = term + M[i, j] * V[j] * 2.0
        total += np.sum(np.real(np.conj(V[i]) * term))
    return total


def celio_mu_psi(sig):
    """The muon state of eigenvalue +1 of sigma_mu (muspinsim/celio.py:361-363)."""
    evals, evecs = np.linalg.eig(np.asarray(sig) + np.eye(2))
    return evecs[:, 1] if np.real(evals[1]) > 0.1 else evecs[:, 0]


def celio_fast_evolve(factors, dims, sig, times, k, phases):
    """Averaged random-state evolution (muspinsim/celio.py:318-476,
    muspinsim/cpp/celio.cpp:23-64): psi = mu_psi (x) exp(2 pi i r) /
    sqrt(d), then per time: measure, then k passes of every factor in
    order.  ``phases``: [averages, d] uniform numbers r (the reference draws
    them with np.random.rand(d) per average).  Returns 0.5 * mean."""
    N = int(np.prod(dims))
    half = N // 2
    sig = np.asarray(sig, dtype=complex)
    mu_psi = celio_mu_psi(sig)
    maps = [celio_index_map(dims, order) for _, _, order, _ in factors]
    res = np.zeros(len(times))
    for r in np.atleast_2d(phases):
        psi = np.kron(mu_psi, np.exp(2j * np.pi * r)) * (1.0 / np.sqrt(half))
        for i in range(len(times)):
            res[i] += celio_measure_h(psi, sig, half)
            for _ in range(k):
                for (U, _, _, _), idx in zip(factors, maps):
                    celio_apply(psi, U, idx)
    return res * (1.0 / len(np.atleast_2d(phases))) * 0.5


def celio_full_factor(U, dims, order):
    """The factor on the whole space: (U (x) 1) in the permuted ordering,
    permuted back to the system's ordering (muspinsim/celio.py:180-206)."""
    N = int(np.prod(dims))
    D = U.shape[0]
    F = np.kron(U, np.eye(N // D))
    sd = [dims[s] for s in order]
    L = len(dims)
    perm = list(np.argsort(order))
    F = F.reshape(sd + sd).transpose(perm + [L + p for p in perm]).reshape(N, N)
    return F


def celio_evolve(factors, dims, rho0, times, operators, k):
    """Density-matrix variant (muspinsim/celio.py:210-293): E = (prod_c
    F_c)^k with the factors multiplied left to right; per time t_i,
    rho = T^dag rho0 T with T = E^i, result_j = sum(rho * O_j^T)."""
    N = int(np.prod(dims))
    E = np.eye(N, dtype=complex)
    for U, _, order, _ in factors:
        E = E @ celio_full_factor(U, dims, order)
    E = np.linalg.matrix_power(E, k)
    T = np.eye(N, dtype=complex)
    out = np.zeros((len(times), len(operators)), dtype=complex)
    for i in range(len(times)):
        rho = T.conj().T @ (rho0 @ T)
        for j, O in enumerate(operators):
            out[i, j] = np.sum(rho * np.asarray(O).T)
        T = T @ E
    return out


def celio_snapshot_factors(system, B, dt, k):
    """Trotter factors of one snapshot: the system's terms plus the field's
    Zeeman terms (muspinsim/experiment.py:239-269, 332-334)."""
    dims = list(system.dims)
    return celio_factors(celio_contribs(dims, celio_terms(system, B)), dt, k)


def celio_fast_evolve_c(factors, dims, sig, times, k, phases, nthreads=0):
    """celio_fast_evolve through the C restatement (oracle/celio.c), with
    OpenMP inside every factor application as the reference's native
    module does."""
    lib = _oracle_lib()
    if not getattr(lib, "_celio_bound", False):
        vp = ctypes.c_void_p
        lib.oracle_celio_evolve.argtypes = [ctypes.c_int, vp, vp, ctypes.c_long, ctypes.c_int,
                                            ctypes.c_int, vp, vp, vp, vp, ctypes.c_long, vp,
                                            ctypes.c_int]
        lib._celio_bound = True
    N = int(np.prod(dims))
    half = N // 2
    sig = np.ascontiguousarray(sig, dtype=complex)
    mu_psi = celio_mu_psi(sig)
    mats = np.ascontiguousarray(np.concatenate([U.reshape(-1) for U, _, _, _ in factors]),
                                dtype=complex)
    dims_f = np.array([U.shape[0] for U, _, _, _ in factors], dtype=np.int64)
    other_f = np.array([N // U.shape[0] for U, _, _, _ in factors], dtype=np.int64)
    idx = np.ascontiguousarray(np.concatenate(
        [celio_index_map(dims, order) for _, _, order, _ in factors]).astype(np.uint64))
    times = np.asarray(times, dtype=float)
    res = np.zeros(len(times))
    ph = np.atleast_2d(phases)
    for r in ph:
        psi = np.ascontiguousarray(np.kron(mu_psi, np.exp(2j * np.pi * r)) * (1.0 / np.sqrt(half)))
        lib.oracle_celio_evolve(len(times), psi.ctypes.data, sig.ctypes.data, half, int(k),
                                len(factors), mats.ctypes.data, dims_f.ctypes.data,
                                other_f.ctypes.data, idx.ctypes.data, N, res.ctypes.data,
                                int(nthreads))
    return res * (1.0 / len(ph)) * 0.5
