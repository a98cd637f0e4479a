"""Simulation configuration: evaluated input parameters expanded into
snapshots, API-compatible with ``muspinsim/simconfig.py``.

Each input keyword holds one value or a range.  A range is the x axis, an
averaged axis or a file range (``muspinsim/simconfig.py:112-171``);
snapshots are the Cartesian product file x average x x-axis
(``:299-321``); a snapshot's result is added to
results[file idx + x idx] divided by the number of averaged configurations
(``store_time_slice``, ``:347-368``).  Orientation weights are normalised to
sum to N when orientations are averaged, else ignored (``:152-159``).

The text input language (a lark grammar in the reference) is not part of
this library: parameters come as the dictionary ``MuSpinInput.evaluate``
returns, which ``make_params`` builds from Python values.
"""

import datetime
import logging
import os
import re
from collections import OrderedDict, namedtuple
from collections.abc import Iterable
from itertools import product

import numpy as np

from muspinsim_gb300.orientations import orientation_rows_to_quats
from muspinsim_gb300.quaternion import Quaternion
from muspinsim_gb300.spinsys import MuonSpinSystem

__version__ = "2.3.1"  # reference version whose output format is written

_CDICT = {
    "polarization": "mupol",
    "field": "B",
    "intrinsic_field": "intrinsic_B",
    "time": "t",
    "orientation": "orient",
    "temperature": "T",
}
# Coupling kinds: the shape of the value and how a term enters the spin
# system (i, j 0-based; j may be None).  Dissipation terms are collected
# per spin instead, for the runner's Lindbladian.
_COUPLINGS = {
    "zeeman": ((3,), lambda sy, i, j, v: sy.add_zeeman_term(i, v)),
    "dipolar": ((3,), lambda sy, i, j, v: sy.add_dipolar_term(i, j, v)),
    "hyperfine": ((3, 3), lambda sy, i, j, v: sy.add_hyperfine_term(i, v, j)),
    "quadrupolar": ((3, 3), lambda sy, i, j, v: sy.add_quadrupolar_term(i, v)),
    "dissipation": ((1,), None),
}


def _index_grid(ranges):
    """Every index combination of an ordered set of ranges (a time range is
    kept whole: its index is slice(None)), first range slowest."""
    return list(product(*[[slice(None)] if k == "t" else range(len(v))
                          for k, v in ranges.items()]))


def _exposed(attr, view=None):
    """Read-only property returning attribute `attr` (through `view`, which
    returns a copy where callers must not alias the state)."""
    if view is None:
        return property(lambda self: getattr(self, attr))
    return property(lambda self: view(getattr(self, attr)))

ConfigSnapshot = namedtuple("ConfigSnapshot", ["id", "y"] + list(_CDICT.values()))
MuSpinInputValue = namedtuple("MuSpinInputValue", ["name", "args", "value"])


class MuSpinConfigError(Exception):
    pass


class _Identity:
    def evaluate(self, **kw):
        return kw["y"]


class CallableResults:
    """Wraps f(x, y, **variables) as a results_function."""

    def __init__(self, fn):
        self.fn = fn

    def evaluate(self, **kw):
        return self.fn(**kw)


def make_params(spins=("mu", "e"), couplings=(), time=None, orientation=((0.0, 0.0, 0.0),),
                field=(0.0,), intrinsic_field=(0.0,), polarization=((1.0, 0.0, 0.0),),
                temperature=(np.inf,), y_axis="asymmetry", x_axis="time",
                average_axes=("orientation",), name="muspinsim", orientation_mode="zyz",
                results_function=None, celio=(0, 0)):
    """The evaluated-parameter dictionary for MuSpinConfig / ExperimentRunner.

    Every axis keyword takes a list of rows (one value: a constant; several:
    a range), with the reference's defaults (``muspinsim/input/keyword.py:
    364-485``): time = linspace(0, 10, 101), polarization transverse (x),
    orientation (0, 0, 0), temperature inf, field 0.  ``couplings`` is a list
    of ``(kind, {"i": 1-based, ["j": 1-based]}, value)``.
    """
    if time is None:
        time = np.linspace(0, 10, 101)

    def rows(v):
        return np.array([np.atleast_1d(np.asarray(r, dtype=float)) for r in v], dtype=float)

    p = {
        "name": MuSpinInputValue("name", {}, np.array([[name]])),
        "spins": MuSpinInputValue("spins", {}, np.array([list(spins)], dtype=object)),
        "celio": MuSpinInputValue("celio", {}, np.array([[str(c) for c in celio]])),
        "y_axis": MuSpinInputValue("y_axis", {}, np.array([[y_axis]])),
        "x_axis": MuSpinInputValue("x_axis", {}, np.array([[x_axis]])),
        "average_axes": MuSpinInputValue("average_axes", {}, np.array([list(average_axes)])),
        "polarization": MuSpinInputValue("polarization", {}, rows(polarization)),
        "field": MuSpinInputValue("field", {}, rows(field)),
        "intrinsic_field": MuSpinInputValue("intrinsic_field", {}, rows(intrinsic_field)),
        "time": MuSpinInputValue("time", {}, np.asarray(time, dtype=float).reshape(-1, 1)),
        "orientation": MuSpinInputValue("orientation", {"mode": orientation_mode},
                                        np.array([np.asarray(o, float) for o in orientation],
                                                 dtype=object if len({len(o) for o in orientation}) > 1 else float)),
        "temperature": MuSpinInputValue("temperature", {},
                                        np.asarray(temperature, dtype=float).reshape(-1, 1)),
        "results_function": results_function if results_function is not None else _Identity(),
        "fitting_info": {"fit": False},
        "couplings": {},
    }
    for k, (kind, args, value) in enumerate(couplings):
        p["couplings"][f"{kind}_{k}"] = MuSpinInputValue(kind, dict(args),
                                                          [np.asarray(value, dtype=float)])
    return p


class ParamsInput:
    """Minimal stand-in for MuSpinInput: ``evaluate()`` returns the params."""

    def __init__(self, params):
        self._params = params

    def evaluate(self, **variables):
        return dict(self._params)


class MuSpinConfig:
    """Ranges, snapshots and result accumulation of one simulation
    (muspinsim/simconfig.py:78-647).

    Every axis keyword is validated into a list of values and then takes
    one role: a constant (one value), the x axis, an averaged axis or a
    file range (several values; _axis_role).  The snapshots are the index
    grid file x averaged x x, and results[file, x] accumulates the averaged
    snapshots' signal.
    """

    def __init__(self, params={}, use_experimental_x_axis=True):
        self._constants = {}
        self._file_ranges = OrderedDict()
        self._avg_ranges = OrderedDict()
        self._x_range = OrderedDict()
        if len(params) == 0:
            return
        self._name = self.validate("name", params["name"].value)[0]
        self._spins = self.validate("spins", params["spins"].value[0])
        self._celio = self._validate_celio(params["celio"].value[0])
        self._y_axis = self.validate("y", params["y_axis"].value[0])[0]
        self._results_function = params["results_function"]
        x_axis, averaged = self._declared_axes(params)
        self._time_isavg = "t" in averaged
        self._time_N = 0
        avg_values = OrderedDict((a, None) for a in averaged)
        x_values = None
        for iname, cname in _CDICT.items():
            if iname not in params:
                raise MuSpinConfigError(
                    f"Invalid params object passed to MuSpinConfig: missing {iname}")
            values = self._axis_values(cname, params[iname], averaged)
            role = self._axis_role(cname, len(values), x_axis, averaged)
            if role == "const":
                self._constants[cname] = values[0]
            elif role == "x":
                x_values = values
            elif role == "avg":
                avg_values[cname] = values
            else:
                self._file_ranges[cname] = values
        if self._y_axis == "integral" and x_axis == "t":
            raise MuSpinConfigError("Can not use time as X axis when evaluating integral of signal")
        finfo = params["fitting_info"]
        if finfo.get("fit"):
            x_values = self._fit_x_axis(finfo, x_axis, x_values, use_experimental_x_axis)
        if x_values is None:
            raise MuSpinConfigError("Specified x axis is not a range")
        self._x_range[x_axis] = x_values
        # averaged axes in the order they were declared, ranges only
        self._avg_ranges = OrderedDict((k, v) for k, v in avg_values.items() if v is not None)
        self._system, self._dissip_terms = self._build_system(params["couplings"])
        self._results = np.zeros([len(v) for v in self._file_ranges.values()]
                                 + [len(x_values)])
        grids = [_index_grid(r) for r in (self._file_ranges, self._avg_ranges, self._x_range)]
        self._configurations = list(product(*grids))
        self._avg_N = len(grids[1])

    @staticmethod
    def _declared_axes(params):
        """The x axis and the averaged axes (declaration order), as config
        keys."""
        try:
            x_axis = _CDICT[params["x_axis"].value[0][0]]
        except KeyError as exc:
            raise MuSpinConfigError("Invalid x axis name in input file") from exc
        averaged = []
        for a in np.asarray(params["average_axes"].value).reshape((-1,)):
            if str(a).lower() == "none":
                continue
            if a not in _CDICT:
                raise MuSpinConfigError("Invalid average axis name in input file")
            if _CDICT[a] not in averaged:
                averaged.append(_CDICT[a])
        return x_axis, averaged

    def _axis_values(self, cname, pvalue, averaged):
        """Validated values of one axis keyword.  Time: a single infinite
        time when the y axis is the integral.  Orientations: weights scaled
        to sum to the count when averaged, else all 1."""
        values = self.validate(cname, pvalue.value, pvalue.args)
        if cname == "t":
            if self._y_axis == "integral":
                logging.warning("Ignoring time axis since Y = integral")
                values = [np.inf]
            self._time_N = len(values)
        elif cname == "orient":
            if cname in averaged:
                scale = len(values) / np.sum([w for (_, w) in values])
                values = [(q, w * scale) for (q, w) in values]
            else:
                values = [(q, 1.0) for (q, _) in values]
        return values

    def _fit_x_axis(self, finfo, x_axis, x_values, use_experimental):
        """Fitting (muspinsim/simconfig.py:180-233): no file ranges; the x axis
        becomes the experimental data's first column (fields along z) when
        asked, or when the x keyword holds a single value; the declared x
        axis is then only used for the output file."""
        if len(self._file_ranges) > 0:
            raise MuSpinConfigError("Can not have file ranges when fitting")
        self._constants.pop(x_axis, None)
        if x_values is None:
            use_experimental = True
            finfo["evaluate_x_axis"] = False
        if not use_experimental:
            return x_values
        data_x = np.asarray(finfo["data"])[:, 0]
        if x_axis in ("B", "intrinsic_B"):
            exp_x = np.array([[0.0, 0.0, v] for v in data_x])
        else:
            exp_x = data_x
        if finfo.get("evaluate_x_axis") and x_values is not None:
            logging.info("Fitting will be performed on experimental data-points, specified "
                         "'x_axis' will only be used to generate final .dat file")
            xv = np.asarray(x_values, dtype=float)
            lo, hi = xv < exp_x[0], xv > exp_x[-1]
            if np.all(hi) or np.all(lo):
                logging.warning("All points on specified 'x_axis' are outside the experimental "
                                "range, fitted parameters may not be appropriate for "
                                "extrapolation")
            elif np.any(hi) or np.any(lo):
                logging.info("Some points on specified 'x_axis' are outside the experimental "
                             "range, fitted parameters may not be appropriate for "
                             "extrapolation")
        if x_axis == "t":
            self._time_N = len(exp_x)
        return list(exp_x)

    @staticmethod
    def _axis_role(cname, count, x_axis, averaged):
        if count <= 1:
            return "const"
        if cname == x_axis:
            return "x"
        return "avg" if cname in averaged else "file"

    def _build_system(self, couplings):
        """The MuonSpinSystem of the coupling terms, and the dissipation
        rates by spin."""
        system = MuonSpinSystem(self._spins, self.celio_k)
        dissipation = {}
        nspins = len(self._spins)
        for term in couplings.values():
            if term.name not in _COUPLINGS:
                raise MuSpinConfigError(
                    f"Invalid params object passed to MuSpinConfig: unknown {term.name} coupling")
            shape, add = _COUPLINGS[term.name]
            indices = [v for v in term.args.values() if v is not None]
            if any(k < 1 or k > nspins for k in indices):
                raise MuSpinConfigError("Out of range indices for coupling")
            value = np.asarray(term.value[0], dtype=float)
            if value.shape != shape:
                raise MuSpinConfigError(f"Invalid shape for {term.name} coupling term")
            i, j = (None if k is None else k - 1 for k in (term.args.get("i"), term.args.get("j")))
            if add is None:
                dissipation[i] = value[0]
            else:
                add(system, i, j, value)
        return system, dissipation

    # -------------------------------------------------------------- validators
    def validate(self, name, value, args=None):
        args = {} if args is None else args
        fn = getattr(self, f"_validate_{name}", None)
        if fn is not None:
            value = [fn(v, **args) for v in value]
        return value

    def _validate_name(self, v):
        if len(v) > 1:
            raise MuSpinConfigError("Name must be a word without spaces")
        return v[0]

    def _validate_spins(self, v):
        m = re.compile("([0-9]+)([A-Z][a-z]*|e)").match(v)
        if m is None:
            return v
        A, el = m.groups()
        return (el, int(A))

    def _validate_celio(self, v):
        try:
            k = int(v[0])
        except ValueError as exc:
            raise MuSpinConfigError("Value of k for Celio's method must be an integer") from exc
        if k < 0:
            raise MuSpinConfigError("Value of k for Celio's method must a postive integer or 0")
        avg = int(v[1]) if len(v) == 2 else 0
        if avg < 0:
            raise MuSpinConfigError(
                "Value of averages for Celio's method must a postive integer or 0")
        return (k, avg)

    def _validate_t(self, v):
        if len(v) != 1:
            raise MuSpinConfigError("Invalid line in time range")
        return v[0]

    def _validate_B(self, v):
        v = np.atleast_1d(np.asarray(v, dtype=float))
        if len(v) == 1:
            return np.array([0, 0, v[0]])
        if len(v) != 3:
            raise MuSpinConfigError("Invalid magnetic field value")
        return v

    def _validate_intrinsic_B(self, v):
        v = np.atleast_1d(np.asarray(v, dtype=float))
        if len(v) == 1:
            return np.array([0, 0, v[0]])
        if len(v) != 3:
            raise MuSpinConfigError("Invalid intrinsic magnetic field value")
        return v

    def _validate_mupol(self, v):
        v = np.array(v, dtype=float)
        if len(v) != 3:
            raise MuSpinConfigError("Invalid muon polarization direction")
        return v / np.linalg.norm(v)

    def _validate_orient(self, v, mode="zyz"):
        qs, ws = orientation_rows_to_quats([np.asarray(v, dtype=float)], mode)
        return (Quaternion(qs[0]), float(ws[0]))

    def _validate_T(self, v):
        return np.atleast_1d(v)[0]

    # -------------------------------------------------------------- results
    def store_time_slice(self, config_id, tslice):
        if isinstance(tslice, Iterable) and len(tslice) != self._time_N:
            raise ValueError("Time slice has invalid length")
        if self._time_isavg:
            tslice = np.average(tslice)
        ii = tuple(list(config_id[0]) + list(config_id[2]))
        self._results[ii] += tslice / self._avg_N

    def save_output(self, name=None, path=".", extension=".dat"):
        """Write one two-column .dat file per file-range combination
        (muspinsim/simconfig.py:370-429)."""
        if name is None:
            name = self.name
        header = ("MUSPINSIM v.{version}\nOutput file written on {date}\nParameters used:\n"
                  .format(version=__version__, date=datetime.datetime.now().ctime()))
        for fn in self._file_ranges:
            header += "\t{0:<20} = {{{0}}}\n".format(fn)
        x = self.x_axis_values
        if "B" in self._x_range or "intrinsic_B" in self._x_range:
            x = np.linalg.norm(x, axis=-1)
        for inds in product(*[range(len(r)) for r in self._file_ranges.values()]):
            fid = "".join(f"_{i}" for i in inds)
            vdict = {}
            for i, (key, val) in enumerate(self._file_ranges.items()):
                v = val[inds[i]]
                pf = getattr(self, f"_print_{key}", None)
                vdict[key] = pf(v) if pf else v
            data = np.zeros((len(x), 2))
            data[:, 0] = x
            data[:, 1] = self._results[inds]
            np.savetxt(os.path.join(path, f"{name}{fid}{extension}"), data,
                       header=header.format(**vdict))

    def _print_B(self, v):
        return "{0} T".format(v)

    def _print_orient(self, v):
        o, w = v
        abc = o.euler_angles("zyz") * 180 / np.pi
        return "[ZYZ] a = {0:.1f} deg, b = {1:.1f} deg, c = {2:.1f} deg, weight = {3}".format(*abc, w)

    # -------------------------------------------------------------- properties
    name = _exposed("_name")
    spins = _exposed("_spins", list)
    celio_k = property(lambda self: self._celio[0])
    celio_averages = property(lambda self: self._celio[1])
    system = _exposed("_system", lambda sy: sy.clone())
    constants = _exposed("_constants", dict)
    dissipation_terms = _exposed("_dissip_terms", dict)
    x_axis = property(lambda self: next(iter(self._x_range)))
    x_axis_values = property(lambda self: np.array(next(iter(self._x_range.values()))))
    y_axis = _exposed("_y_axis")
    results_function = _exposed("_results_function")
    file_ranges = _exposed("_file_ranges", OrderedDict)
    avg_ranges = _exposed("_avg_ranges", OrderedDict)
    x_range = _exposed("_x_range", OrderedDict)
    avg_N = _exposed("_avg_N")
    time_N = _exposed("_time_N")
    time_is_averaged = _exposed("_time_isavg")

    @property
    def results(self):
        return np.array(self._results)

    @results.setter
    def results(self, r):
        r = np.array(r)
        if r.shape != self._results.shape:
            raise ValueError("Trying to set an invalid results array")
        self._results = r

    @property
    def configurations(self):
        return list(self._configurations)

    def __len__(self):
        return len(self._configurations)

    def __getitem__(self, i):
        isint = isinstance(i, int)
        if isint:
            i = slice(i, i + 1)
        elif not isinstance(i, slice):
            raise TypeError(f"Indices must be integer or slices, not {type(i)}")

        def pick(inds, od):
            return {k: v[inds[n]] for n, (k, v) in enumerate(od.items())}

        ans = []
        for fc, ac, xc in self._configurations[i]:
            ans.append(ConfigSnapshot(id=(fc, ac, xc), y=self._y_axis, **self._constants,
                                      **pick(fc, self._file_ranges), **pick(ac, self._avg_ranges),
                                      **pick(xc, self._x_range)))
        return ans[0] if isint else ans
