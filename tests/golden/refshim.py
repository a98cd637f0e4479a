"""Import the reference implementation in this container, for golden vectors.

Used only by ``tests/golden/make_golden.py`` on a machine that holds the
reference tree; nothing on the product path or in the GPU tests imports it.

The reference depends on five packages that are not installed here (ase,
soprano, qutip, lark, mpi4py).  Its polarisation path touches only a sliver
of each, so this module registers small stand-ins in ``sys.modules`` before
importing it:

* ``ase.quaternions.Quaternion`` -- [w, x, y, z] quaternions with the Hamilton
  product; ``from_euler_angles(a, b, c, mode)`` = q_c * q_b * q_a about z,y|x,z;
  ``rotate(v)`` = q v q*.  The reference's own tests pin this convention
  (``muspinsim/tests/test_config.py:233-285``,
  ``muspinsim/tests/test_utils.py:43-65``).
* ``soprano.nmr.utils._get_isotope_data`` -- backed by the same isotope table
  the product and the oracle use (``muspinsim_gb300/isotopes.py``).
* ``soprano.calculate.powder.ZCW`` -- never called: orientations are passed
  explicitly.
* ``qutip`` Pauli matrices with ``.data_as("csr_matrix")``
  (``muspinsim/spinsys.py:754-757``).
* ``lark`` -- import-only placeholders; the text input language is not used.
* ``muspinsim.cpp`` (Celio's method) -- the reference's own pybind11 module
  compiled from its sources by ``oracle/build.py`` where pybind11 is
  installed, else an import-only placeholder.
* ``numpy.product`` -- removed in numpy 2; the reference's Celio code calls
  it, so it is aliased to ``numpy.prod`` (the same function in numpy 1.x).
* ``muspinsim.celio.np.sum`` -- the density-matrix branch of
  ``CelioHamiltonian.evolve`` stores a 1x1 ``np.matrix`` into a complex
  array element (``muspinsim/celio.py:286-288``), which numpy 1.26 (the
  reference's pin) accepted and numpy 2 rejects.  The reference's ``celio``
  module sees numpy through a proxy whose ``sum`` unwraps a size-1 matrix
  to its scalar; every other name is numpy's own.
* ``muspinsim.cython`` -- the reference's own Cython kernel compiled from its
  sources by ``oracle/build.py``.
"""

import importlib.util
import os
import sys
import types

import numpy as np
from scipy import sparse

REFERENCE_ROOT = "/root/reference"
REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


class _Quaternion:
    def __init__(self, qin=(1.0, 0.0, 0.0, 0.0)):
        self.q = np.array(qin, dtype=float)

    def __mul__(self, other):
        w1, x1, y1, z1 = self.q
        w2, x2, y2, z2 = other.q
        return _Quaternion(
            [
                w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2,
                w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2,
                w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2,
            ]
        )

    def conjugate(self):
        return _Quaternion(self.q * np.array([1.0, -1.0, -1.0, -1.0]))

    def rotate(self, vector):
        v = _Quaternion(np.concatenate([[0.0], np.asarray(vector, dtype=float)]))
        return (self * v * self.conjugate()).q[1:]

    def rotation_matrix(self):
        return np.array([self.rotate(e) for e in np.eye(3)]).T

    @staticmethod
    def from_axis_angle(axis, angle):
        axis = np.asarray(axis, dtype=float)
        axis = axis / np.linalg.norm(axis)
        return _Quaternion(np.concatenate([[np.cos(angle / 2)], np.sin(angle / 2) * axis]))

    @staticmethod
    def from_euler_angles(a, b, c, mode="zyz"):
        qa = _Quaternion.from_axis_angle([0, 0, 1], a)
        if mode == "zyz":
            qb = _Quaternion.from_axis_angle([0, 1, 0], b)
        elif mode == "zxz":
            qb = _Quaternion.from_axis_angle([1, 0, 0], b)
        else:
            raise ValueError(mode)
        qc = _Quaternion.from_axis_angle([0, 0, 1], c)
        return qc * qb * qa


def _get_isotope_data(elems, prop, isotope_list=None):
    from muspinsim_gb300.isotopes import isotope_data

    if isotope_list is None:
        isotope_list = [None] * len(elems)
    return np.array([isotope_data(e, prop, i) for e, i in zip(elems, isotope_list)])


class _Qobj:
    """Operator container: ``data_as('csr_matrix')`` and, for Celio's
    method, ``permute(order)`` -- new subsystem i is old subsystem order[i]
    (muspinsim/celio.py:193-204)."""

    def __init__(self, m=None, arg=None, dims=None):
        m = arg if m is None else m
        if m is not None and sparse.issparse(m):
            m = m.toarray()
        self._m = sparse.csr_matrix(np.asarray(m, dtype=complex)) if m is not None else None
        self._dims = dims

    def permute(self, order):
        sd = list(self._dims[0])
        L = len(sd)
        order = [int(o) for o in order]
        n = self._m.shape[0]
        T = self._m.toarray().reshape(sd + sd).transpose(order + [L + o for o in order])
        new = [sd[o] for o in order]
        return _Qobj(T.reshape(n, n), dims=[new, new])

    def data_as(self, fmt):
        return self._m


class _NumpyCompat(types.ModuleType):
    """numpy with ``sum`` returning the scalar of a size-1 np.matrix, as
    numpy 1.x's scalar assignment did implicitly."""

    def __init__(self):
        super().__init__("numpy")

    def __getattr__(self, name):
        return getattr(np, name)

    @staticmethod
    def sum(*args, **kwargs):
        r = np.sum(*args, **kwargs)
        if isinstance(r, np.matrix) and r.size == 1:
            return r.item()
        return r


def _module(name, **attrs):
    mod = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(mod, k, v)
    sys.modules[name] = mod
    return mod


def install():
    """Register the stand-ins and the compiled kernel; return the reference
    package ``muspinsim`` with its hot-path submodules imported."""
    if "muspinsim.hamiltonian" in sys.modules:
        return sys.modules["muspinsim"]
    if REPO not in sys.path:
        sys.path.insert(0, REPO)

    _module("ase")
    _module("ase.io")
    _module("ase.quaternions", Quaternion=_Quaternion)
    _module("soprano")
    _module("soprano.nmr")
    _module("soprano.nmr.utils", _get_isotope_data=_get_isotope_data)
    _module("soprano.calculate")

    class ZCW:  # orientations are always passed explicitly
        def __init__(self, *a, **k):
            raise NotImplementedError("ZCW grids are generated by the caller")

    _module("soprano.calculate.powder", ZCW=ZCW)
    _module("qutip", Qobj=_Qobj)
    _module("qutip.core")
    _module(
        "qutip.core.operators",
        sigmax=lambda: _Qobj([[0, 1], [1, 0]]),
        sigmay=lambda: _Qobj([[0, -1j], [1j, 0]]),
        sigmaz=lambda: _Qobj([[1, 0], [0, -1]]),
    )

    class _Lark:  # built at import time by the reference; never parses here
        def __init__(self, *a, **k):
            pass

        def parse(self, *a, **k):
            raise NotImplementedError("the input language is not available")

    _module("lark", Lark=_Lark, Transformer=object, Tree=object, Token=str)
    _module("lark.exceptions", UnexpectedToken=Exception, UnexpectedInput=Exception)

    sys.path.insert(0, REFERENCE_ROOT)
    if not hasattr(np, "product"):
        np.product = np.prod

    # the reference's native modules, compiled from its own sources
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import build as oracle_build  # oracle/build.py

    cpp_path = oracle_build.build_ref_cpp()
    if cpp_path is not None:
        spec = importlib.util.spec_from_file_location("cpp", cpp_path)
        cpp = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(cpp)
        sys.modules["muspinsim.cpp"] = cpp
    else:
        _module("muspinsim.cpp", Celio_EvolveContrib=None, celio_evolve=None)

    path = oracle_build.build_ref()
    spec = importlib.util.spec_from_file_location(oracle_build.REF_MODULE, path)
    cy = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(cy)
    sys.modules["muspinsim.cython"] = cy

    import muspinsim.hamiltonian  # noqa: F401
    import muspinsim.spinsys  # noqa: F401
    import muspinsim.experiment  # noqa: F401
    import muspinsim.celio

    muspinsim.celio.np = _NumpyCompat()

    return sys.modules["muspinsim"]


def input_value(name, value, args=None):
    """A stand-in for one evaluated input keyword (``muspinsim/input/input.py:26``)."""
    from muspinsim.input.input import MuSpinInputValue

    return MuSpinInputValue(name, args or {}, value)


class _Results:
    def evaluate(self, **kw):
        return kw["y"]


class ParamsInput:
    """Object with ``evaluate(**variables)`` returning an evaluated-params dict,
    which is all ``ExperimentRunner`` needs from a ``MuSpinInput``
    (``muspinsim/experiment.py:65-68``)."""

    def __init__(self, params):
        self._params = params

    def evaluate(self, **variables):
        return dict(self._params)


def make_params(
    spins,
    couplings,
    times,
    orientations,
    field=((0.0, 0.0, 0.0),),
    intrinsic_field=((0.0, 0.0, 0.0),),
    polarization=(1.0, 0.0, 0.0),
    temperature=(np.inf,),
    y_axis="asymmetry",
    x_axis="time",
    average_axes=("orientation",),
    dissipation=None,
    celio=(0, 0),
):
    """Build the evaluated-params dict for ``MuSpinConfig``.

    ``couplings`` is a list of ``(kind, args, value)`` with kind in
    zeeman/hyperfine/dipolar/quadrupolar and 1-based ``i``/``j`` args, exactly
    as the input file would give them.  ``orientations`` rows are
    ``(a, b, c[, w])`` ZYZ Euler angles or ``(theta, phi)`` polar angles.
    """
    install()
    p = {
        "name": input_value("name", np.array([["test"]])),
        "spins": input_value("spins", np.array([list(spins)], dtype=object)),
        "celio": input_value("celio", np.array([[str(c) for c in celio]])),
        "y_axis": input_value("y_axis", np.array([[y_axis]])),
        "x_axis": input_value("x_axis", np.array([[x_axis]])),
        "average_axes": input_value("average_axes", np.array([list(average_axes)])),
        "polarization": input_value("polarization", np.array([polarization], dtype=float)),
        "field": input_value("field", np.array([np.atleast_1d(f) for f in field], dtype=float)),
        "intrinsic_field": input_value(
            "intrinsic_field", np.array([np.atleast_1d(f) for f in intrinsic_field], dtype=float)
        ),
        "time": input_value("time", np.array(times, dtype=float)[:, None]),
        "orientation": input_value(
            "orientation", np.array(orientations, dtype=float), {"mode": "zyz"}
        ),
        "temperature": input_value("temperature", np.array(temperature, dtype=float)[:, None]),
        "results_function": _Results(),
        "fitting_info": {"fit": False},
        "couplings": {},
    }
    for n, (kind, args, value) in enumerate(couplings):
        p["couplings"][f"{kind}_{n}"] = input_value(kind, [np.array(value, dtype=float)], args)
    for i, rate in (dissipation or {}).items():  # 1-based spin index -> rate (MHz)
        p["couplings"][f"dissipation_{i}"] = input_value(
            "dissipation", [np.array([rate], dtype=float)], {"i": int(i)})
    return p
