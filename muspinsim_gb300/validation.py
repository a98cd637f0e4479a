"""Argument checks with the reference's exception types and messages
(muspinsim/validation.py:8-101)."""

from numbers import Number

import numpy as np


def validate_times(times):
    """times must be a 1-D numpy array (muspinsim/validation.py:8-21)."""
    if not isinstance(times, np.ndarray):
        raise TypeError("times must be an array of values in microseconds")
    if len(times.shape) != 1:
        raise ValueError("times must be an array of values in microseconds")


def validate_evolve_params(rho0, times, operators):
    """(muspinsim/validation.py:24-45)"""
    from muspinsim_gb300.spinop import DensityOperator, SpinOperator

    if not isinstance(rho0, DensityOperator):
        raise TypeError("rho0 must be a valid DensityOperator")
    validate_times(times)
    if not all([isinstance(o, SpinOperator) for o in operators]):
        raise ValueError("operators must be a SpinOperator or a list of SpinOperator objects")


def validate_integrate_decaying_params(rho0, tau, operators):
    """(muspinsim/validation.py:74-101)"""
    from muspinsim_gb300.spinop import DensityOperator, SpinOperator

    if not isinstance(rho0, DensityOperator):
        raise TypeError("'rho0' must be a valid DensityOperator")
    if not (isinstance(tau, Number) and np.isreal(tau) and tau > 0):
        raise ValueError("'tau' must be a real number > 0")
    if not operators:
        raise ValueError("At least one SpinOperator must be present in 'operators'")
    if not all([isinstance(o, SpinOperator) for o in operators]):
        raise ValueError("'operators' must be a SpinOperator or a list of SpinOperator objects")


def validate_celio_params(terms, times):
    """Celio's method needs interaction terms and a uniform time grid that
    starts at 0 (muspinsim/validation.py:48-71)."""
    if len(terms) == 0:
        raise ValueError("No interaction terms to evolve")
    if times[0] != 0:
        raise ValueError("Cannot use Celio's method with a non-zero start time")
    differences = np.diff(times)
    if not np.isclose(differences, differences[0]).all():
        raise ValueError("Cannot use Celio's method with uneven spacing between times")
