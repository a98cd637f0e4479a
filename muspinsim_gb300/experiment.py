"""ExperimentRunner, API-compatible with ``muspinsim/experiment.py``.

``run()`` does not loop over snapshots: every (file, average, x) snapshot's
field, polarisation, temperature, orientation and weight is gathered into
arrays at once, the evolution path of each snapshot is chosen with the
reference's rule, and the whole set is diagonalised, evolved and reduced
into the results array by one GPU pipeline per path (``powder.py``).  The
single-snapshot methods (``load_config``, ``run_single``, ``rho0``, ``Hz``,
``Htot``, ``p_operator``) are kept for callers that drive snapshots one by
one, and run on the GPU through the Hamiltonian methods.
"""

import numpy as np
import scipy.constants as cnst

from muspinsim_gb300 import kernels
from muspinsim_gb300 import quaternion as Q
from muspinsim_gb300.constants import MU_TAU
from muspinsim_gb300.hamiltonian import Hamiltonian
from muspinsim_gb300 import celio
from muspinsim_gb300.celio import CelioHamiltonian
from muspinsim_gb300.lindbladian import Lindbladian
from muspinsim_gb300.powder import run_snapshots, t_inf_speedup
from muspinsim_gb300.simconfig import MuSpinConfig
from muspinsim_gb300.spinop import DensityOperator, SpinOperator, spin_projectors


def get_xy(z):
    """Two axes x, y orthogonal to z, right-handed with it
    (muspinsim/utils.py:71-93)."""
    zn = np.linalg.norm(z)
    if zn == 0:
        raise ValueError("Can not find X and Y for null Z vector")
    z = np.array(z) / zn
    if z[0] == 0 and z[1] == 0:
        return np.array([1.0, 0, 0]), np.array([0, z[2], 0])
    x = np.array([z[1], -z[0], 0.0]) / (z[0] ** 2 + z[1] ** 2) ** 0.5
    y = np.array([z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2],
                  z[0] * x[1] - z[1] * x[0]])
    return x, y


def thermal_state(I, gamma, B, T):
    """Single-spin state in its own Zeeman field gamma B at temperature T:
    uniform at T = inf, ground state at T <= 0 (muspinsim/experiment.py:
    201-228), written with exact spectral projectors of B.S."""
    proj = spin_projectors(I, B)
    Bn = np.linalg.norm(B)
    E = np.array([m * Bn for m, _ in proj]) * 1e6 * gamma
    if T > 0:
        x = -cnst.h * E / (cnst.k * T)
        Z = np.exp(x - x.max())
    else:
        Z = np.where(E == np.amin(E), 1.0, 0.0)
    Z = Z / np.sum(Z) if np.sum(Z) > 0 else np.ones(len(E)) / len(E)
    rho = sum(z * P for z, (_, P) in zip(Z, proj))
    return rho / np.trace(rho)


class ExperimentRunner:
    """Runs every snapshot of a MuSpinConfig (muspinsim/experiment.py:22-498).

    ``in_file``: an object with ``evaluate(**variables)`` returning the
    evaluated parameters (a MuSpinInput, or ``simconfig.ParamsInput``), or the
    parameter dictionary itself.  ``precision``: 'fp64' (default, matches the
    reference to 1e-10) or 'mixed'."""

    def __init__(self, in_file, variables=None, use_experimental_x_axis=True, precision="fp64"):
        if variables is None:
            variables = {}
        self._variables = variables
        params = in_file if isinstance(in_file, dict) else in_file.evaluate(**variables)
        self._config = MuSpinConfig(params, use_experimental_x_axis=use_experimental_x_axis)
        self._system = self._config.system
        self.precision = precision
        self._B = np.zeros(3)
        self._p = np.array([1.0, 0, 0])
        self._T = np.inf
        self._Hsys = self._system.hamiltonian
        self._rho0 = None
        self._Hz = None
        self._T_inf_speedup = None

    # -------------------------------------------------------------- state
    @property
    def config(self):
        return self._config

    @property
    def system(self):
        return self._system

    @property
    def B(self):
        return self._B

    @B.setter
    def B(self, x):
        x = np.array(x, dtype=float)
        if (x != self._B).any():
            self._B = x
            self._rho0 = None
            self._Hz = None

    @property
    def p(self):
        return self._p

    @p.setter
    def p(self, x):
        x = np.array(x, dtype=float)
        if (x != self._p).any():
            self._p = x
            self._rho0 = None

    @property
    def T(self):
        return self._T

    @T.setter
    def T(self, x):
        if x != self._T:
            self._T = x
            self._rho0 = None

    @property
    def rho0(self):
        """Initial density matrix (muspinsim/experiment.py:170-236)."""
        if self._rho0 is None:
            sy = self._system
            mats = []
            for i in range(len(sy.spins)):
                I = sy.I(i)
                if i == sy.muon_index:
                    mats.append(spin_projectors(I, self._p)[0][1])
                else:
                    mats.append(thermal_state(I, sy.gamma(i), self._B, self._T))
            M = mats[0]
            for m in mats[1:]:
                M = np.kron(M, m)
            self._rho0 = DensityOperator(M, sy.dimension)
        return self._rho0

    @property
    def Hz(self):
        """Zeeman Hamiltonian sum_i gamma_i B.S_i (muspinsim/experiment.py:239-269);
        with Celio's method, a CelioHamiltonian of one Zeeman term per spin
        (none in zero field)."""
        if self._Hz is None and self._config.celio_k:
            from muspinsim_gb300.celio import CelioHamiltonian
            from muspinsim_gb300.spinsys import SingleTerm

            extra = []
            if not np.array_equal(self._B, [0, 0, 0]):
                extra = [SingleTerm(self._system, i, self._B * self._system.gammas[i],
                                    label="Zeeman") for i in range(len(self._system.spins))]
            self._Hz = CelioHamiltonian(extra, self._config.celio_k, self._system)
        if self._Hz is None:
            Z = self._system.zeeman_operators()
            self._Hz = Hamiltonian(np.einsum("a,aij->ij", self._B, Z), dim=self._system.dimension)
        return self._Hz

    @property
    def Hsys(self):
        return self._Hsys

    @property
    def dissipation_operators(self):
        """(operator, rate) pairs of the dissipative spins: S+ and S- about
        the field direction with rates a Zu / (pi (1 + Zu)) and
        a / (pi (1 + Zu)), Zu = exp(-h gamma |B| 1e6 / (k T))
        (muspinsim/experiment.py:272-325)."""
        if self._config.celio_k:
            raise NotImplementedError("Dissipation is not supported when using Celio's method")
        B = np.linalg.norm(self._B)
        g = np.array(self._system.gammas, dtype=float)
        T = self._T
        Zu = np.exp(-cnst.h * g * B * 1e6 / (cnst.k * T)) if T > 0 else g * 0.0
        if B == 0:
            x, y = np.array([1.0, 0, 0]), np.array([0, 1.0, 0])
        else:
            x, y = get_xy(self._B / B)
        dops = []
        for i, a in self._config.dissipation_terms.items():
            S = [self._system.operator({i: ax}).matrix for ax in "xyz"]
            op_x = sum(S[k] * x[k] for k in range(3))
            op_y = sum(S[k] * y[k] for k in range(3))
            dim = self._system.dimension
            dops.append((SpinOperator(op_x + 1.0j * op_y, dim=dim), 1 / np.pi * a * Zu[i] / (1 + Zu[i])))
            dops.append((SpinOperator(op_x - 1.0j * op_y, dim=dim), 1 / np.pi * a / (1 + Zu[i])))
        return dops

    @property
    def Htot(self):
        """Hsys + Hz, or its Lindbladian when the configuration has
        dissipation terms (muspinsim/experiment.py:332-341)."""
        H = self.Hsys + self.Hz
        if len(self._config.dissipation_terms) > 0:
            H = Lindbladian.from_hamiltonian(H, self.dissipation_operators)
        return H

    @property
    def p_operator(self):
        return self._system.muon_operator(self.p)

    def apply_results_function(self, results, variables):
        return np.array(
            self._config.results_function.evaluate(**variables, x=self._config.x_axis_values,
                                                   y=results)
        ).reshape(results.shape)

    # -------------------------------------------------------------- one snapshot
    def load_config(self, cfg_snap):
        """Rotate B and p into the crystal frame, add the intrinsic field,
        pick the path; returns the orientation weight
        (muspinsim/experiment.py:384-432)."""
        q, w = cfg_snap.orient
        self.B = q.rotate(cfg_snap.B)
        self.p = q.rotate(cfg_snap.mupol)
        self.T = cfg_snap.T
        self.B = self._B + cfg_snap.intrinsic_B
        self._T_inf_speedup = bool(t_inf_speedup(self._B, self._T, self._system.muon_index)[0]) \
            and len(self._config.dissipation_terms) == 0
        return w

    def run_single(self, cfg_snap):
        """One snapshot on the GPU (muspinsim/experiment.py:434-498)."""
        w = self.load_config(cfg_snap)
        H = self.Htot
        if cfg_snap.y == "asymmetry":
            if isinstance(H, CelioHamiltonian) and self._config.celio_averages:
                if self.T != np.inf:
                    raise ValueError(
                        "The fast version of Celio's method requires T -> inf. Either remove "
                        "the number of averages or don't use celio.")
                data = H.fast_evolve(self._system.sigma_mu(self.p), cfg_snap.t,
                                     self._config.celio_averages, True)
            elif self._T_inf_speedup and not isinstance(H, (Lindbladian, CelioHamiltonian)):
                other = int(np.prod(self._system.dimension)) // 2
                data = H.fast_evolve(self._system.sigma_mu(self.p), cfg_snap.t, other)
            else:
                data = H.evolve(self.rho0, cfg_snap.t, operators=[self.p_operator])[:, 0]
        elif cfg_snap.y == "integral":
            data = H.integrate_decaying(self.rho0, MU_TAU, operators=[self.p_operator])[0] / MU_TAU
        return np.real(data) * w

    # -------------------------------------------------------------- all snapshots
    def _snapshot_arrays(self):
        """Per-snapshot parameter arrays in configuration order, and the
        result-array layout (time axis, row index of each snapshot)."""
        cfg = self._config
        groups = [cfg.file_ranges, cfg.avg_ranges, cfg.x_range]
        dims, keys = [], []
        for g in groups:
            for k, v in g.items():
                dims.append(1 if k == "t" else len(v))
                keys.append(k)
        S = int(np.prod(dims)) if dims else 1
        idx = np.unravel_index(np.arange(S), dims) if dims else ()
        consts = cfg.constants

        def gather(key):
            if key in keys:
                pos = keys.index(key)
                rng = [g for g in groups if key in g][0][key]
                return [rng[i] for i in idx[pos]] if key != "t" else None
            return None

        def vec3(key):
            got = gather(key)
            if got is None:
                return np.broadcast_to(np.asarray(consts[key], dtype=float), (S, 3))
            return np.asarray(got, dtype=float)

        B = vec3("B")
        intr = vec3("intrinsic_B")
        mupol = vec3("mupol")
        Tg = gather("T")
        T = np.full(S, float(consts["T"])) if Tg is None else np.asarray(Tg, dtype=float)
        og = gather("orient")
        orients = [consts["orient"]] * S if og is None else og
        qs = np.array([q.q for q, w in orients])
        ws = np.array([w for q, w in orients], dtype=float)

        # result layout: file dims then x dims; the time axis (x or file) is
        # computed in full by every snapshot
        res_dims, res_pos, t_axis = [], [], None
        for gi, g in enumerate([cfg.file_ranges, cfg.x_range]):
            for k, v in g.items():
                if k == "t":
                    t_axis = len(res_dims)
                    res_dims.append(len(v))
                    res_pos.append(None)
                else:
                    res_dims.append(len(v))
                    res_pos.append(keys.index(k))
        row_dims = [d for d, p in zip(res_dims, res_pos) if p is not None]
        row_idx = [idx[p] for p in res_pos if p is not None]
        rows = np.ravel_multi_index(row_idx, row_dims) if row_idx else np.zeros(S, dtype=np.int64)
        nrows = int(np.prod(row_dims)) if row_dims else 1
        return B, intr, mupol, T, qs, ws, rows, nrows, res_dims, t_axis

    def _run_lindblad(self, B_lab, p_lab, T, wscale, rows, nrows, times):
        """Dissipative snapshots on the GPU (msp_lindblad_run): every
        snapshot's Lindbladian is built and propagated on the device, results
        reduced into the output rows; the 'mixed' precision propagates in
        double-word FP32 where that form applies (uniform time grid,
        n^2 <= 64), FP64 otherwise."""
        from muspinsim_gb300 import _lib
        from muspinsim_gb300.powder import _rows_sorted

        sy = self._system
        order = _rows_sorted(np.asarray(rows))
        n = int(np.prod(sy.dimension))
        S_ops = np.array([[sy.operator({i: ax}).matrix.toarray() for ax in "xyz"]
                          for i in range(len(sy.spins))], dtype=complex)
        mode = _lib.MODE_INTEGRAL if self._config.y_axis == "integral" else _lib.MODE_EVOLVE
        out, st = kernels.lindblad_run(
            n, sy.hamiltonian_matrix(), sy.zeeman_operators(), S_ops, list(sy.dimension),
            sy.muon_index, sy.gammas, self._config.dissipation_terms, B_lab[order], p_lab[order],
            np.asarray(wscale)[order], np.asarray(rows)[order].astype(np.int32), nrows, times,
            temperature=np.asarray(T, dtype=float)[order], mode=mode, tau=MU_TAU,
            precision=_lib.PREC_MIXED if self.precision == "mixed" else _lib.PREC_FP64)
        status = np.zeros(len(order), dtype=np.int32)
        status[order] = st.cpu().numpy()
        return out, status

    def run(self):
        """All snapshots, gathered into the results array; the results
        function is applied unless running with fitting variables
        (muspinsim/experiment.py:358-382)."""
        cfg = self._config
        B, intr, mupol, T, qs, ws, rows, nrows, res_dims, t_axis = self._snapshot_arrays()
        B_lab = Q.rotate(qs, B) + intr
        p_lab = Q.rotate(qs, mupol)
        if cfg.y_axis == "integral":
            times = np.array([np.inf])
        else:
            tval = cfg.x_range.get("t") or cfg.file_ranges.get("t") or cfg.avg_ranges.get("t")
            if tval is None:
                tval = cfg.constants["t"]
                if np.ndim(tval) == 0:
                    # the reference's evolve rejects a scalar time (validate_times)
                    raise ValueError("times must be an array of values in microseconds")
            times = np.asarray(tval, dtype=float).reshape(-1)
        if cfg.celio_k:
            if len(cfg.dissipation_terms) > 0:
                raise NotImplementedError("Dissipation is not supported when using Celio's method")
            if cfg.y_axis == "integral":
                raise NotImplementedError(
                    "integrate_decaying is not implemented for Celio's method")
            out = celio.run_snapshots(self._system, cfg.celio_k, cfg.celio_averages, B_lab, p_lab,
                                      T, ws / cfg.avg_N, rows, nrows, times, self.precision)
            status = np.zeros(len(B_lab), dtype=np.int32)
        elif len(cfg.dissipation_terms) > 0:
            out, status = self._run_lindblad(B_lab, p_lab, T, ws / cfg.avg_N, rows, nrows, times)
        else:
            out, status = run_snapshots(self._system, B_lab, p_lab, T, ws / cfg.avg_N, rows,
                                        nrows, times, cfg.y_axis, self.precision)
        if np.any(status & 1):
            raise RuntimeError("Jacobi eigensolver did not converge for some snapshots")
        out = out.cpu().numpy()
        if cfg.y_axis == "integral":
            res = out.reshape([d for i, d in enumerate(res_dims) if i != t_axis])
        elif t_axis is not None:
            other = [d for i, d in enumerate(res_dims) if i != t_axis]
            res = np.moveaxis(out.reshape(other + [len(times)]), -1, t_axis)
        else:
            if not cfg.time_is_averaged:
                raise ValueError("times must be an array of values in microseconds")
            res = out.mean(axis=1).reshape(res_dims)
        self._T_inf_speedup = bool(t_inf_speedup(B_lab[-1], T[-1], self._system.muon_index)[0])
        if not self._variables:
            res = self.apply_results_function(res, {})
        cfg.results = res
        return cfg.results
