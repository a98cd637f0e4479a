"""Fitting simulations to data, API-compatible with ``muspinsim/fitting.py``,
with analytic gradients where the simulation allows them.

The reference minimises over its input variables with scipy, re-running
``ExperimentRunner`` for every objective evaluation and, for L-BFGS-B,
differencing the objective numerically (muspinsim/fitting.py:67-179).  This
``FittingRunner`` keeps its constructor, ``run()`` (a scipy
``OptimizeResult``), its objectives (mean absolute deviation for
``minimize``, residuals for ``least_squares``), the ``single_simulation``
cache and the ``results_function`` chaining
(muspinsim/experiment.py:347-356).  For the L-BFGS-B method on the
muon-first, T = inf time-domain path it supplies the gradient itself:

    dL/dx_k = Re sum conj(G_H) dHsys/dx_k + sum_s G_B,s . dB_lab,s/dx_k
              + (dL/dy) (dy/dx_k at fixed signal),

where G_H = dL/dHsys and G_B = dL/dB_lab come from one adjoint launch
(msp_adjoint_fast) for the upstream dL/dP(t), and dHsys/dx_k, dB_lab/dx_k
are central differences of the host-side Hamiltonian and field set-up (no
eigensolve; exact for couplings linear in the variables, up to rounding
otherwise).  One objective + gradient evaluation therefore costs one forward
powder average and one adjoint, where the reference's difference quotients
cost 1 + n_variables forward simulations.

Inputs: an object like the reference's ``MuSpinInput`` with
``fitting_info`` (``fit``, ``data`` (N, 2), ``method`` in nelder-mead /
lbfgs / least-squares, ``rtol``, ``single_simulation``), ``variables``
(name -> ``FittingVariable``) and ``evaluate(**variables)`` returning the
evaluated parameters; :class:`FitInput` builds one from a Python function.
"""

import numpy as np
from scipy.optimize import least_squares, minimize

from muspinsim_gb300 import kernels
from muspinsim_gb300.experiment import ExperimentRunner


class FittingVariable:
    """A fitting variable with a starting value and bounds
    (muspinsim/input/variables.py:4-50)."""

    def __init__(self, name, value=0.0, min_value=-np.inf, max_value=np.inf):
        self._name = name
        self._value = float(value)
        self._min = float(min_value)
        self._max = float(max_value)
        problems = []
        if self._max <= self._min:
            problems.append(f"Variable {name} has invalid range: (max value {self._max} cannot "
                            f"be less than or equal to min value {self._min})")
        if self._value > self._max:
            problems.append(f"Variable {name} has invalid starting value: (starting value "
                            f"{self._value} cannot be greater than max value {self._max})")
        if self._value < self._min:
            problems.append(f"Variable {name} has invalid starting value: (starting value "
                            f"{self._value} cannot be less than min value {self._min})")
        if problems:
            raise ValueError("\n".join(problems))

    name = property(lambda self: self._name)
    value = property(lambda self: self._value)
    bounds = property(lambda self: (self._min, self._max))


class FitInput:
    """The fitting side of a MuSpinInput built from Python: ``build(**x)``
    returns the evaluated parameter dictionary (``simconfig.make_params``)
    for variable values x; ``data`` is the (N, 2) target (x, y)."""

    def __init__(self, build, variables, data, method="lbfgs", rtol=1e-8,
                 single_simulation=False):
        self._build = build
        self._variables = {v.name: v for v in variables}
        self._fitting_info = {"fit": True, "data": np.asarray(data, dtype=float),
                              "method": method, "rtol": rtol, "function": None,
                              "single_simulation": bool(single_simulation),
                              "evaluate_x_axis": False}

    @property
    def variables(self):
        return dict(self._variables)

    @property
    def fitting_info(self):
        return dict(self._fitting_info)

    def evaluate(self, **variables):
        p = dict(self._build(**variables))
        p["fitting_info"] = dict(self._fitting_info)
        return p


_METHODS = {"nelder-mead": "nelder-mead", "lbfgs": "L-BFGS-B"}


class FittingRunner:
    """Fit the input's variables to its data (muspinsim/fitting.py:15-179).

    ``precision``: the simulations' precision ('fp64', the reference's
    results to 1e-10, or 'mixed').  ``gradient``: supply analytic gradients
    to L-BFGS-B where the simulation runs on the fast path (set False for the
    reference's numerical differences).
    """

    def __init__(self, inpfile, precision="fp64", gradient=True):
        self._input = inpfile
        self._runner = None
        self._fitinfo = inpfile.fitting_info
        self._ytarg = np.asarray(self._fitinfo["data"])[:, 1]
        variables = inpfile.variables
        if len(variables) == 0:
            raise ValueError("MuSpinInput passed to FittingRunner has no variables to fit")
        self._xnames = tuple(sorted(variables.keys()))  # the order scipy sees
        self._x = np.array([variables[k].value for k in self._xnames])
        self._xbounds = np.array([variables[k].bounds for k in self._xnames])
        self._constrained = bool(np.any(self._xbounds[:, 0] != -np.inf)
                                 or np.any(self._xbounds[:, 1] != np.inf))
        self._sol = None
        self._cached_results = None
        self.precision = precision
        self.gradient = gradient
        self.simulations = 0          # forward simulations run
        self.adjoint_evaluations = 0  # analytic gradients computed

    # ---------------------------------------------------------------- run
    def run(self):
        method = self._fitinfo["method"]
        if method == "least-squares":
            # curve_fit's choice: Levenberg-Marquardt unless constrained
            self._sol = least_squares(self._targfun_residuals, self._x,
                                      method="trf" if self._constrained else "lm",
                                      gtol=self._fitinfo["rtol"],
                                      bounds=(self._xbounds[:, 0], self._xbounds[:, 1]))
        else:
            jac = method == "lbfgs" and self.gradient and self._adjoint_applies()
            fun = self._targfun_with_gradient if jac else self._targfun_minimise
            self._sol = minimize(fun, self._x, method=_METHODS[method],
                                 tol=self._fitinfo["rtol"], bounds=self._xbounds,
                                 jac=True if jac else None)
        best = dict(zip(self._xnames, self._sol["x"]))
        # the simulation at the optimum, then the results function on it
        self._compute_result(self._sol["x"])
        self._runner.config.results = self._runner.apply_results_function(
            self._runner.config.results, best)
        return self._sol

    @property
    def runner(self):
        return self._runner

    # ---------------------------------------------------------------- objective
    def _obtain_results(self, vardict):
        if self._fitinfo["single_simulation"]:
            if self._cached_results is None:
                self._runner = self._experiment(vardict)
                self._cached_results = self._runner.run()
            return self._cached_results
        self._runner = self._experiment(vardict)
        return self._runner.run()

    def _experiment(self, vardict):
        self.simulations += 1
        return ExperimentRunner(self._input, variables=vardict, precision=self.precision)

    def _compute_result(self, x):
        self._x = np.asarray(x, dtype=float)
        vardict = dict(zip(self._xnames, self._x))
        y = self._obtain_results(vardict)
        return self._runner.apply_results_function(y, vardict)

    def _targfun_residuals(self, x):
        return self._compute_result(x) - self._ytarg

    def _targfun_minimise(self, x):
        return float(np.average(np.abs(self._compute_result(x) - self._ytarg)))

    # ---------------------------------------------------------------- gradient
    def _adjoint_applies(self):
        """Whether the simulation at the starting point is one fast-path
        powder average over orientations on a time axis: muon first, T = inf,
        no Celio or dissipation, nothing but orientations averaged."""
        runner = ExperimentRunner(self._input, variables=dict(zip(self._xnames, self._x)),
                                  precision=self.precision)
        cfg = runner.config
        if cfg.x_axis != "t" or cfg.y_axis != "asymmetry" or cfg.celio_k:
            return False
        if cfg.dissipation_terms or cfg.file_ranges:
            return False
        if set(cfg.avg_ranges) - {"orient"}:
            return False
        if runner.system.muon_index != 0:
            return False
        return np.isinf(cfg.constants.get("T", np.inf))

    def _snapshot_inputs(self, vardict):
        """Host-side set-up of the simulation at vardict: Hsys, Z, lab-frame
        fields and polarisations, weights and times (no GPU work)."""
        from muspinsim_gb300 import quaternion as Q

        runner = ExperimentRunner(self._input, variables=vardict, precision=self.precision)
        B, intr, mupol, T, qs, ws, rows, nrows, res_dims, t_axis = runner._snapshot_arrays()
        cfg = runner.config
        sy = runner.system
        times = np.asarray(cfg.x_axis_values, dtype=float).reshape(-1)
        return (sy.hamiltonian_matrix(), sy.zeeman_operators(), Q.rotate(qs, B) + intr,
                Q.rotate(qs, mupol), ws / cfg.avg_N, times)

    def _targfun_with_gradient(self, x):
        x = np.asarray(x, dtype=float)
        vardict = dict(zip(self._xnames, x))
        P = np.asarray(self._obtain_results(vardict), dtype=float)
        runner = self._runner
        y = runner.apply_results_function(P, vardict)
        r = y - self._ytarg
        f = float(np.average(np.abs(r)))
        dLdy = np.sign(r) / r.size
        dLdP, dydx_direct = self._results_function_terms(runner, P, vardict, dLdy)
        grad = np.array(dydx_direct, dtype=float)
        if dLdP is None:
            # the results function is not elementwise in the signal: central
            # differences of the whole objective, as scipy would take them
            return f, self._fd_gradient(x)
        if not self._fitinfo["single_simulation"]:
            Hsys, Z, B_lab, p_lab, wscale, times = self._snapshot_inputs(vardict)
            dH, dB = [], []
            for k in range(len(x)):
                h = 1e-6 * max(1.0, abs(x[k]))
                up, dn = x.copy(), x.copy()
                up[k] += h
                dn[k] -= h
                Hu, _, Bu, _, _, _ = self._snapshot_inputs(dict(zip(self._xnames, up)))
                Hd, _, Bd, _, _, _ = self._snapshot_inputs(dict(zip(self._xnames, dn)))
                dH.append((Hu - Hd) / (2 * h))
                dB.append((Bu - Bd) / (2 * h))
            if any(np.any(d != 0) for d in dH) or any(np.any(d != 0) for d in dB):
                S = B_lab.shape[0]
                gH, gF, st = kernels.adjoint_fast(
                    Hsys.shape[0], Hsys, Z, B_lab, p_lab, wscale, np.zeros(S, np.int32), 1,
                    times, np.ascontiguousarray(dLdP.reshape(1, -1)))
                self.adjoint_evaluations += 1
                gH = gH.cpu().numpy()
                gF = gF.cpu().numpy() if gF is not None else np.zeros_like(B_lab)
                for k in range(len(x)):
                    grad[k] += float(np.real(np.sum(np.conj(gH) * dH[k])))
                    grad[k] += float(np.sum(gF * dB[k]))
        return f, grad

    def _results_function_terms(self, runner, P, vardict, dLdy):
        """dL/dP through the results function, when that function acts on
        the signal elementwise (checked with a second, random probe), and
        dL/dx_k of its direct dependence on the variables."""
        x_names = self._xnames
        h = 1e-6 * max(1.0, float(np.max(np.abs(P))))

        def g(Pv, vd):
            return np.asarray(runner.apply_results_function(Pv, vd), dtype=float)

        ones = np.ones_like(P)
        diag = (g(P + h * ones, vardict) - g(P - h * ones, vardict)) / (2 * h)
        probe = np.random.default_rng(7).uniform(0.5, 1.5, P.shape)
        jr = (g(P + h * probe, vardict) - g(P - h * probe, vardict)) / (2 * h)
        scale = max(1.0, float(np.max(np.abs(jr))))
        dLdP = dLdy * diag if np.max(np.abs(jr - diag * probe)) <= 1e-6 * scale else None
        direct = np.zeros(len(x_names))
        for k, name in enumerate(x_names):
            hv = 1e-6 * max(1.0, abs(vardict[name]))
            up, dn = dict(vardict), dict(vardict)
            up[name] += hv
            dn[name] -= hv
            direct[k] = float(np.sum(dLdy * (g(P, up) - g(P, dn)) / (2 * hv)))
        return dLdP, direct

    def _fd_gradient(self, x):
        grad = np.zeros(len(x))
        for k in range(len(x)):
            h = 1e-6 * max(1.0, abs(x[k]))
            up, dn = x.copy(), x.copy()
            up[k] += h
            dn[k] -= h
            grad[k] = (self._targfun_minimise(up) - self._targfun_minimise(dn)) / (2 * h)
        self._compute_result(x)
        return grad
